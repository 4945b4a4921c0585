"""The dense-ordered ("NQt") vector path of the drop-in boundary.

The reference dispatches ``HVec`` / ``HDiag`` on ``dmrg.ifQt``
(``mpo_dmrg_kernel.py:45-48, 121-124``): with ``ifQt = False`` the Davidson
vector lists the allowed elements of the dense (ldim, 4, 4, rdim) tensor in the
order of ``prjmap`` (``HVecNQt`` 138-181).  CPU: the oracle's dense kernels and
its block-sparse kernels agree through the index maps (the reference's own
Qt-vs-dense consistency).  GPU: the product with ``ifQt = False`` against the
oracle's dense ``HVecNQt`` / ``HDiagNQt`` (FP64 path <= 1e-10, split <= 1e-8
relative).
"""
import numpy
import pytest

from tests.problems import (random_problem, oracle_dense_side, nqt_prjmap, packed_to_nqt,
                            oracle_sigma, oracle_hdiag, oracle_sigma_nqt)

CASES = [dict(K=4, nelec=4, D=8, isite=1, seed=5),
         dict(K=6, nelec=6, D=16, isite=2, seed=1)]


def rel(a, b):
    return numpy.linalg.norm(a - b) / max(numpy.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("case", CASES)
def test_oracle_dense_path_equals_block_path(case):
    from oracle import kernel as ok
    P = random_problem(device=False, **case)
    md = oracle_dense_side(P)
    prj = nqt_prjmap(P)
    assert prj.size == P.ndim0
    pos = packed_to_nqt(P, prj)
    assert sorted(pos.tolist()) == list(range(P.ndim0))
    x = numpy.random.default_rng(3).standard_normal(P.ndim0)
    y_nqt = ok.HVecNQt(x, [md, P.isite, 2, md.flst, 'L', True], prj.size, prj)
    y_qt = oracle_sigma(P, x[pos])
    assert rel(y_nqt[pos], y_qt) < 1e-12
    d_nqt = ok.HDiagNQt([md, P.isite, 2, md.flst, 'L', True], prj.size, prj)
    assert rel(d_nqt[pos], oracle_hdiag(P)) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("split", 1e-8)])
def test_product_dense_order_path(gpu, case, precision, tol):
    from oracle import kernel as ok
    from zmpo_dmrg_gb300.mpo_dmrg_kernel import HVec, HDiag
    P = random_problem(**case)
    md = oracle_dense_side(P)
    prj = nqt_prjmap(P)
    x = numpy.random.default_rng(4).standard_normal(prj.size)
    ref = oracle_sigma_nqt(P, x, md)
    m = P.p
    m.precision = precision
    m.ifQt = False
    try:
        y = HVec(x, [m, P.isite, 2, m.flst, 'L', True], prj.size, prj)
        m.device_vectors = False
        d = HDiag([m, P.isite, 2, m.flst, 'L', True], prj.size, prj)
    finally:
        m.ifQt = True
        m.device_vectors = True
    assert isinstance(y, numpy.ndarray) and isinstance(d, numpy.ndarray)
    assert rel(y, ref) < tol
    d_ref = ok.HDiagNQt([md, P.isite, 2, md.flst, 'L', True], prj.size, prj)
    assert rel(d, d_ref) < 1e-12


def test_perturbation_path_is_refused():
    """``dmrg.ifpt`` (H0 - E0, ``mpo_dmrg_kernel.py:126-135``) is not served:
    an explicit error instead of a wrong vector."""
    from zmpo_dmrg_gb300.mpo_dmrg_kernel import HVec
    from zmpo_dmrg_gb300.mpo_dmrg_class import mpo_dmrg
    m = mpo_dmrg(seed=0)
    m.ifpt = True
    with pytest.raises(NotImplementedError):
        HVec(numpy.zeros(4), [m, 0, 2, None, 'L', True], 4, None)
