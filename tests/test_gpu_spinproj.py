"""Spin-projected (SP-MPS) kernels on the GPU against the CPU oracle: H psi
with the N-only relabelling and projection back on (N, Sz), diag(H), the
overlap S psi = sum_g w_g P_g psi and its diagonal, and the renormalised H_p
and P_g environments (restated HVecQt / HDiagQt / SVecQt / SDiagQt /
renormQt_H00 / renormQt_S00 of the reference).  Tolerances: FP64 <= 1e-10
relative, split <= 1e-8 relative."""
import numpy
import pytest

from tests.problems import (random_problem, oracle_sigma, product_sigma, oracle_hdiag,
                            product_hdiag, oracle_renorm, product_renorm, oracle_svec,
                            product_svec, oracle_sdiag, product_sdiag, oracle_prdm, product_prdm)

pytestmark = pytest.mark.gpu

CASES = [dict(K=4, nelec=4, D=8, isite=1, seed=5, npts=4, sval=0.0),
         dict(K=6, nelec=6, D=16, isite=2, seed=1, npts=5, sval=0.0),
         dict(K=6, nelec=5, D=16, isite=0, seed=2, npts=4, sval=0.5, sz=0.5),
         dict(K=6, nelec=6, D=24, isite=4, seed=3, npts=6, sval=1.0),
         dict(K=8, nelec=8, D=32, isite=3, seed=4, npts=4, sval=0.0)]

_cache = {}


def prob(c):
    key = tuple(sorted(c.items()))
    if key not in _cache:
        _cache[key] = random_problem(**c)
    return _cache[key]


def rel(a, b):
    return numpy.linalg.norm(a - b) / max(numpy.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("split", 1e-8)])
def test_sigma_sp(gpu, case, precision, tol):
    P = prob(case)
    x = numpy.random.default_rng(7).standard_normal(P.ndim0)
    assert rel(product_sigma(P, x, precision), oracle_sigma(P, x)) < tol


@pytest.mark.parametrize("case", CASES)
def test_svec(gpu, case):
    P = prob(case)
    x = numpy.random.default_rng(8).standard_normal(P.ndim0)
    assert rel(product_svec(P, x), oracle_svec(P, x)) < 1e-10


@pytest.mark.parametrize("case", CASES)
def test_diagonals_sp(gpu, case):
    P = prob(case)
    assert rel(product_hdiag(P), oracle_hdiag(P)) < 1e-10
    assert rel(product_sdiag(P), oracle_sdiag(P)) < 1e-10


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("status", ["L", "R"])
@pytest.mark.parametrize("which", [0, 1])
def test_renorm_sp(gpu, case, status, which):
    P = prob(case)
    got = product_renorm(P, status, which=which)
    ref = oracle_renorm(P, status, which=which)
    assert len(got) == len(ref)
    for g, r in zip(got, ref):
        assert g.shape == r.shape
        if r.size:
            assert rel(g, r) < 1e-10


@pytest.mark.parametrize("case", CASES[1:4])
@pytest.mark.parametrize("status", ["L", "R"])
def test_perturbed_rdm_sp(gpu, case, status):
    """Noise density matrix with N-labelled terms (pRDMQt, spin-projected)."""
    P = prob(case)
    got = product_prdm(P, status)
    ref = oracle_prdm(P, status)
    assert numpy.abs(got - ref).max() <= 1e-12 * numpy.abs(ref).max()
    clean = oracle_prdm(P, status, noise=0.0)
    assert numpy.abs(got - clean).max() > 1e-8 * numpy.abs(ref).max()


def _run_sp(int1e, int2e, K, nelec, sz, sval, npts, occ, maxM, precision="fp64", seed=1):
    from zmpo_dmrg_gb300.mpo_dmrg_class import mpo_dmrg
    from zmpo_dmrg_gb300.mpo_dmrg_schedule import schedule
    m = mpo_dmrg(seed=seed)
    m.nsite, m.sbas, m.isym = K, 2 * K, 2
    m.ifs2proj, m.npts = True, npts
    m.s2quad(sval, sz)
    m.build()
    m.occun = occ
    m.qsectors = {str([float(nelec), float(sz)]): 1}
    m.precision = precision
    m.partition()
    m.loadInts((int1e, int2e))
    m.dumpMPO()
    sc = schedule(maxM=maxM, tol=1e-9, maxiter=10)
    sc.startNoise = 0.0
    sc.normal(2)
    m.default(sc)
    return m


@pytest.mark.parametrize("sval,occ,npts", [
    (0.0, [1., 1.] * 3 + [0., 0.] * 3, 4),
    (1.0, [1., 1.] * 2 + [1., 0.] + [0., 1.] + [0., 0.] * 2, 5)])
def test_spin_projected_sweep_reaches_spin_fci(gpu, sval, occ, npts):
    """Spin-projected two-site DMRG (generalised Davidson with H P and P) at an
    exact bond dimension lands on the lowest FCI eigenvalue with
    S^2 = S(S+1) in the Sz = 0 sector: the singlet ground state, and the
    triplet that an unprojected Sz = 0 run cannot reach.  The split path
    agrees within 1e-8 Eh."""
    from oracle import integrals as oint
    K = 6
    h, eri, _ = oint.synthetic(K, 21, 1.0)
    i1, i2, g = oint.to_spin_orbital(h, eri)
    eref = oint.fci_spin_energy(i1, g, 6, 0.0, sval)[0]
    occ = numpy.array(occ)
    m = _run_sp(i1, i2, K, 6, 0.0, sval, npts, occ, 64)
    assert abs(m.Energy - eref) < 1e-8
    e, esum, ovlp, psum = m.checkMPS()
    assert abs(e - eref) < 1e-7
    ms = _run_sp(i1, i2, K, 6, 0.0, sval, npts, occ, 64, precision="split")
    assert abs(ms.Energy - m.Energy) < 1e-8
