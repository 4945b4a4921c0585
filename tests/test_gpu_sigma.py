"""Sigma vector, diagonal and renormalisation on the GPU against the CPU
oracle (restated HVecQt / HDiagQt / renormQt_H00 of the reference) on seeded
random block-sparse problems.  Tolerances: FP64 path <= 1e-10 relative,
split path <= 1e-8 relative (norm of the difference over the norm)."""
import numpy
import pytest

from tests.problems import (random_problem, oracle_sigma, product_sigma, oracle_hdiag,
                            product_hdiag, oracle_renorm, product_renorm, oracle_prdm,
                            product_prdm, b_resident_tiles)

pytestmark = pytest.mark.gpu

CASES = [dict(K=4, nelec=4, D=8, isite=1, seed=5),
         dict(K=6, nelec=6, D=16, isite=2, seed=1),
         dict(K=6, nelec=6, D=24, isite=0, seed=2),
         dict(K=6, nelec=6, D=24, isite=4, seed=3),
         dict(K=8, nelec=8, D=32, isite=3, seed=4)]

_cache = {}


def prob(c):
    key = tuple(sorted(c.items()))
    if key not in _cache:
        _cache[key] = random_problem(**c)
    return _cache[key]


def rel(a, b):
    return numpy.linalg.norm(a - b) / max(numpy.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("case", CASES)
def test_sigma_fp64(gpu, case):
    P = prob(case)
    x = numpy.random.default_rng(7).standard_normal(P.ndim0)
    assert rel(product_sigma(P, x, "fp64"), oracle_sigma(P, x)) < 1e-10


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("precision,tol", [("split", 1e-8), ("emu64", 1e-10)])
def test_sigma_split(gpu, case, precision, tol):
    P = prob(case)
    x = numpy.random.default_rng(8).standard_normal(P.ndim0)
    assert rel(product_sigma(P, x, precision), oracle_sigma(P, x)) < tol


# large enough that whole groups span several 64-row tiles: the B-resident
# kernel (k_step_tcb, four independent parts) carries most of T1 and T3
BRES_CASE = dict(K=10, nelec=10, D=128, isite=4, seed=7)


def test_sigma_b_resident_kernel(gpu):
    P = prob(BRES_CASE)
    assert b_resident_tiles(P) > 100
    x = numpy.random.default_rng(12).standard_normal(P.ndim0)
    ref = oracle_sigma(P, x)
    assert rel(product_sigma(P, x, "fp64"), ref) < 1e-10
    assert rel(product_sigma(P, x, "split"), ref) < 1e-8
    assert rel(product_sigma(P, x, "emu64"), ref) < 1e-10


@pytest.mark.parametrize("case", CASES)
def test_hdiag(gpu, case):
    P = prob(case)
    assert rel(product_hdiag(P), oracle_hdiag(P)) < 1e-12


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("status", ["L", "R"])
def test_renorm(gpu, case, status):
    P = prob(case)
    a = product_renorm(P, status)
    b = oracle_renorm(P, status)
    assert len(a) == len(b)
    for x, y in zip(a, b):
        assert x.shape == y.shape
        if y.size:
            assert numpy.abs(x - y).max() <= 1e-12 * max(1.0, numpy.abs(y).max())


@pytest.mark.parametrize("case", CASES[1:])
@pytest.mark.parametrize("status", ["L", "R"])
@pytest.mark.parametrize("precision,tol", [("emu64", 1e-12), ("split", 1e-8)])
def test_renorm_tensor_core_paths(gpu, case, status, precision, tol):
    """The renormalisation in the 56-bit emulation and the split precision
    (relative to the largest element of each new environment)."""
    P = prob(case)
    a = product_renorm(P, status, precision)
    b = oracle_renorm(P, status)
    P.p.precision_renorm = "fp64"
    assert len(a) == len(b)
    for x, y in zip(a, b):
        assert x.shape == y.shape
        if y.size:
            assert numpy.abs(x - y).max() <= tol * max(1.0, numpy.abs(y).max())


def test_sigma_deterministic(gpu):
    P = prob(CASES[1])
    x = numpy.random.default_rng(9).standard_normal(P.ndim0)
    a = product_sigma(P, x, "fp64")
    b = product_sigma(P, x, "fp64")
    assert numpy.array_equal(a, b)


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_sigma_graph_replay(gpu, precision):
    """The site's launches recorded in a CUDA graph give the eager result."""
    P = prob(CASES[1])
    x = numpy.random.default_rng(10).standard_normal(P.ndim0)
    eager = product_sigma(P, x, precision)
    P.p.use_graph = True
    try:
        a = product_sigma(P, x, precision)
        b = product_sigma(P, 2.0 * x, precision)
    finally:
        P.p.use_graph = False
    assert numpy.array_equal(a, eager)
    assert numpy.allclose(b, 2.0 * eager, rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("case", CASES[1:4])
@pytest.mark.parametrize("status", ["L", "R"])
def test_perturbed_rdm(gpu, case, status):
    """Noise density matrix of the decimation (pRDMQt) on the GPU."""
    P = prob(case)
    a = product_prdm(P, status)
    b = oracle_prdm(P, status)
    assert a.shape == b.shape
    assert numpy.abs(a - b).max() <= 1e-12 * max(1.0, numpy.abs(b).max())
    noise_part = oracle_prdm(P, status, noise=1.0) - oracle_prdm(P, status, noise=0.0)
    assert numpy.abs(noise_part).max() > 1e-6   # the noise term is exercised


@pytest.mark.parametrize("case", CASES[1:4])
@pytest.mark.parametrize("status", ["L", "R"])
def test_perturbed_rdm_one_site(gpu, case, status):
    """Noise density matrix of a one-site dot (the reference's first sweep
    from the occupation-number state uses one-site dots with noise):
    'L' at the dot's first site, 'R' at its second."""
    from oracle import dmrg as od
    from zmpo_dmrg_gb300 import prdm
    from zmpo_dmrg_gb300.mpo_dmrg_class import dense_sector
    from tests.problems import QPHYS
    P = prob(case)
    i = P.isite if status == 'L' else P.isite + 1
    qlst = [numpy.asarray(P.qnuml[i], dtype=float), QPHYS, numpy.asarray(P.qnumr[i + 1], dtype=float)]
    dims = [len(q) for q in qlst]
    civec = numpy.zeros(int(numpy.prod(dims)))
    sel = dense_sector(qlst, P.key)
    civec[sel] = numpy.random.default_rng(5).standard_normal(sel.size)
    civec = civec.reshape(1, *dims)
    o, m = P.o, P.p
    o.noise, o.inoise = 1e-4, 0
    m.noise, m.inoise = 1e-4, 0
    saved = m.qlst
    m.qlst, m.qkey = qlst, numpy.array(P.key)
    b = od.pRDM(civec, [o, i, 1, o.flst, status, True])
    try:
        a = prdm.pRDM(civec, [m, i, 1, m.flst, status, True])
    finally:
        m.qlst = saved
    assert a.shape == b.shape
    assert numpy.abs(a - b).max() <= 1e-12 * max(1.0, numpy.abs(b).max())
    # the noise term is exercised
    o.noise = 1.0
    assert numpy.abs(od.pRDM(civec, [o, i, 1, o.flst, status, True]) - b).max() > 1e-6


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_sigma_term_batches(gpu, precision):
    """With a workspace budget the terms run in batches (summed on the
    device); sigma and diag(H) agree with the single-plan result."""
    from zmpo_dmrg_gb300.mpo_dmrg_kernel import HVec, HDiag
    P = prob(CASES[4])
    m = P.p
    x = numpy.random.default_rng(12).standard_normal(P.ndim0)
    info = [m, P.isite, 2, m.flst, 'L', True]
    m.precision = precision
    m._sigma_plan = None
    y1 = HVec(x, info, P.ndim0, None)
    d1 = HDiag(info, P.ndim0, None).cpu().numpy()
    ws1 = m._sigma_plan[1].workspace.numel() * 8
    m._sigma_plan[1].release()
    m._sigma_plan = None
    m.workspace_budget = ws1 // 3
    try:
        y2 = HVec(x, info, P.ndim0, None)
        d2 = HDiag(info, P.ndim0, None).cpu().numpy()
        assert len(m._sigma_plan[1].pids) >= 3
    finally:
        m._sigma_plan[1].release()
        m._sigma_plan = None
        m.workspace_budget = None
        m.precision = "fp64"
    tol = 1e-12 if precision == "fp64" else 1e-8
    assert rel(y2, y1) < tol
    assert rel(d2, d1) < 1e-12


def test_sigma_reuses_kept_records_only_while_operands_are_unchanged(gpu):
    """Within a Davidson solve the environments and the MPO stay fixed: the
    second split H.psi of a plan reuses the digit planes cut from them on the
    first call and gives the identical vector.  An in-place change of an
    environment makes the next call cut them again (the result equals that
    of a fresh plan on the changed environments)."""
    import torch
    from zmpo_dmrg_gb300.mpo_dmrg_kernel import _sigma_plan
    P = random_problem(**BRES_CASE)
    m = P.p
    info = [m, P.isite, 2, m.flst, 'L', True]
    plan = _sigma_plan(info)
    x = torch.from_numpy(numpy.random.default_rng(21).standard_normal(P.ndim0)).cuda()
    y1, y2, y3 = (torch.empty_like(x) for _ in range(3))
    plan.run(m, x, y1, "split")
    assert plan._kept_token is not None
    plan.run(m, x, y2, "split")
    assert torch.equal(y1, y2)
    fL = m.flst[0][0]
    fL.buf.mul_(0.5)                      # in place: the version counter moves
    plan.run(m, x, y3, "split")
    plan.rebind(fL, m.flst[0][1])         # forgets the kept records
    y4 = torch.empty_like(x)
    plan.run(m, x, y4, "split")
    assert torch.equal(y3, y4)
    assert not torch.equal(y3, y1)
    ref = oracle_sigma(P, x.cpu().numpy())  # the oracle side was not scaled
    assert rel(2.0 * y3.cpu().numpy(), ref) < 1e-8
    fL.buf.mul_(2.0)
