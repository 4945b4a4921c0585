"""Energy gradient at a converged MPS through the adjoint of the H.psi
contraction: dE/dh1e and dE/d(pq|rs) against (1) central differences of the
fixed-MPS energy, (2) the one- and two-particle density matrices of the FCI
ground state (the reference's property routines compute these RDMs), and
(3) central differences (step 1e-5) of the FCI energy, which a converged
exact-bond-dimension MPS reproduces (Hellmann-Feynman)."""
import numpy
import pytest

from oracle import integrals as oint

pytestmark = pytest.mark.gpu


def _fci_rdms(int1e, gphys, nelec, sz):
    """Spin-summed 1-RDM g[p,q] = <E_pq> and 2-RDM G[p,q,r,s] =
    sum_{st} <a+_ps a+_rt a_rt... > in the chemists' order of (pq|rs)."""
    sbas = int1e.shape[0]
    K = sbas // 2
    H = oint.fci_hamiltonian(int1e, gphys)
    idx = oint.sector_indices(sbas, nelec, sz)
    w, v = numpy.linalg.eigh(H[idx][:, idx].toarray())
    psi = numpy.zeros(2 ** sbas)
    psi[idx] = v[:, 0]
    a = oint._jw_ops(sbas)
    one = numpy.zeros((K, K))
    ap = [a[k] @ psi for k in range(sbas)]
    for p in range(K):
        for q in range(K):
            one[p, q] = sum(ap[2 * p + s] @ ap[2 * q + s] for s in (0, 1))
    pair = {}
    for x in range(sbas):
        for y in range(sbas):
            pair[x, y] = a[y] @ ap[x]          # a_y a_x psi
    two = numpy.zeros((K, K, K, K))
    for p in range(K):
        for q in range(K):
            for r in range(K):
                for s in range(K):
                    t = 0.0
                    for sg in (0, 1):
                        for tg in (0, 1):
                            t += pair[2 * p + sg, 2 * r + tg] @ pair[2 * q + sg, 2 * s + tg]
                    two[p, q, r, s] = t
    return w[0], one, two


@pytest.fixture(scope="module")
def converged():
    import torch
    from zmpo_dmrg_gb300.mpo_dmrg_class import mpo_dmrg
    from zmpo_dmrg_gb300.mpo_dmrg_schedule import schedule
    from zmpo_dmrg_gb300 import adjoint
    K = 6
    h, eri, _ = oint.synthetic(K, 21, 1.0)
    i1, i2, gphys = oint.to_spin_orbital(h, eri)
    m = mpo_dmrg(seed=1)
    m.nsite, m.sbas, m.isym = K, 2 * K, 2
    m.build()
    m.occun = numpy.array([1., 1.] * 3 + [0., 0.] * 3)
    m.qsectors = {str([6.0, 0.0]): 1}
    m.partition()
    m.loadInts((i1, i2))
    m.dumpMPO()
    sc = schedule(maxM=64, tol=1e-10, maxiter=10)
    sc.startNoise = 0.0
    sc.normal(2)
    m.default(sc)
    ht = torch.tensor(h, requires_grad=True)
    gt = torch.tensor(eri, requires_grad=True)
    E = adjoint.energy(ht, gt, m)
    E.backward()
    return dict(m=m, h=h, eri=eri, i1=i1, gphys=gphys, E=float(E), dh=ht.grad.numpy(),
                dg=gt.grad.numpy(), K=K)


def test_energy_matches_sweep(converged):
    assert abs(converged["E"] - converged["m"].Energy) < 1e-9


def test_gradient_matches_rdms(converged):
    e0, one, two = _fci_rdms(converged["i1"], converged["gphys"], 6, 0.0)
    assert abs(converged["E"] - e0) < 1e-9
    assert numpy.abs(converged["dh"] - one).max() < 1e-8
    assert numpy.abs(converged["dg"] - 0.5 * two).max() < 1e-8


def test_gradient_matches_fixed_mps_differences(converged):
    """E at fixed MPS is linear in the integrals: central differences along
    random symmetric directions equal the adjoint's directional derivative."""
    import torch
    from zmpo_dmrg_gb300 import adjoint
    m, h, eri, K = converged["m"], converged["h"], converged["eri"], converged["K"]
    rng = numpy.random.default_rng(4)
    dh = rng.standard_normal((K, K))
    dh = dh + dh.T
    dg = rng.standard_normal((K, K, K, K))
    dg = adjoint.symmetrize_eri_gradient(dg)
    eps = 1e-5
    ep = float(adjoint.energy(torch.tensor(h + eps * dh), torch.tensor(eri + eps * dg), m))
    em = float(adjoint.energy(torch.tensor(h - eps * dh), torch.tensor(eri - eps * dg), m))
    fd = (ep - em) / (2 * eps)
    an = float((converged["dh"] * dh).sum() + (converged["dg"] * dg).sum())
    assert abs(fd - an) < 1e-7 * max(1.0, abs(an))
    # restore the MPO of the unperturbed integrals
    adjoint.energy(torch.tensor(h), torch.tensor(eri), m)


def test_gradient_matches_fci_energy_differences(converged):
    """Hellmann-Feynman at the converged exact-D MPS: central differences
    (step 1e-5) of the FCI energy along symmetric directions, tol 1e-7."""
    from zmpo_dmrg_gb300 import adjoint
    h, eri, K = converged["h"], converged["eri"], converged["K"]
    rng = numpy.random.default_rng(6)
    dh = rng.standard_normal((K, K))
    dh = dh + dh.T
    dg = adjoint.symmetrize_eri_gradient(rng.standard_normal((K, K, K, K)))
    eps = 1e-5

    def efci(hh, gg):
        i1, _, gp = oint.to_spin_orbital(hh, gg)
        return oint.fci_energy(i1, gp, 6, 0.0)[0]
    fd = (efci(h + eps * dh, eri + eps * dg) - efci(h - eps * dh, eri - eps * dg)) / (2 * eps)
    an = float((converged["dh"] * dh).sum() + (converged["dg"] * dg).sum())
    assert abs(fd - an) < 1e-7 * max(1.0, abs(an))


def test_rdm12_properties(converged):
    """The property routine returns the FCI state's 1- and 2-particle
    densities (the reference's eval_rdm1BF / genMPO_Apqrs quantities)."""
    from zmpo_dmrg_gb300 import properties, adjoint
    import torch
    m, h, eri = converged["m"], converged["h"], converged["eri"]
    adjoint.energy(torch.tensor(h), torch.tensor(eri), m)   # MPO of these integrals
    g1, g2 = properties.rdm12(m, h, eri)
    _, one, two = _fci_rdms(converged["i1"], converged["gphys"], 6, 0.0)
    assert abs(g1.trace() - 6.0) < 1e-9
    assert numpy.abs(g1 - one).max() < 1e-8
    assert numpy.abs(g2 - two).max() < 1e-8


def test_rdm1_matches_reference_brute_force(converged):
    """The product's 1-RDM (site gradients of the H MPO through the adjoint
    contractions) against the restatement of the reference's brute-force
    eval_rdm1BF (an E_pq MPO per element, properties/mpo_dmrg_propsItrf.py:
    204-263) on the same left-canonical MPS, element by element."""
    from oracle.properties import eval_rdm1BF
    from zmpo_dmrg_gb300 import properties
    m, K = converged["m"], converged["K"]
    sites = []
    for i in range(K):
        t = m.flmps['site%d' % i]
        sites.append(t.toDenseTensor(t.idlst) if hasattr(t, "toDenseTensor") else numpy.asarray(t))
    ref_t, _ = eval_rdm1BF(sites)
    got = properties.rdm1(m, converged["h"], converged["eri"])
    assert numpy.abs(got - ref_t).max() < 1e-10


def test_recomputed_environments_give_the_same_gradients(converged):
    """Site gradients with the left environments kept only at checkpoints and
    recomputed segment by segment, and one right environment carried along
    (about 2 sqrt(nsite) environments held), equal those with every
    environment of the MPS stored: the same renormalisations on the same
    inputs."""
    from zmpo_dmrg_gb300 import adjoint
    m = converged["m"]
    g1, e1, n1 = adjoint.site_gradients(m)
    g2, e2, n2 = adjoint.site_gradients(m, recompute_envs=True)
    assert e1 == e2 and n1 == n2
    nterms = 0
    for a, b in zip(g1, g2):
        for x, y in zip(a, b):
            assert (x is None) == (y is None)
            if x is not None:
                nterms += 1
                assert numpy.array_equal(x, y)
    assert nterms > 0
