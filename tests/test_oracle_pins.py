"""Pins of the CPU oracle against the reference: its own C block rule, the
exact Hamiltonian, its Qt-vs-dense MPO self-test, its HVec/HDiag debug check,
its Davidson self-test and the BLOCK energy recorded for the K=6 FCIDUMP."""
import ctypes
import os

import numpy
import pytest

from oracle import integrals, mpo, qtensor as oq, qtensor_opers as oqo, dmrg as od, kernel as ok

GOLD = os.path.join(os.path.dirname(__file__), "golden")
REF_LIB = os.path.join(os.path.dirname(os.path.dirname(__file__)), "oracle", "_ref", "libqsym.so")


def _golden_qsym():
    z = numpy.load(os.path.join(GOLD, "qsym_reference.npz"))
    for c in range(int(z["ncase"])):
        nsyms = z["c%d_nsyms" % c]
        yield (nsyms, z["c%d_status" % c], int(z["c%d_nq" % c]),
               [z["c%d_q%d" % (c, i)] for i in range(len(nsyms))], z["c%d_allowed" % c])


def test_blks_allowed_vs_reference_golden():
    """Restated rule == outputs of the reference's compiled symAllowed."""
    for nsyms, status, nq, qs, allowed in _golden_qsym():
        nb = int(numpy.prod(nsyms))
        got = oq.blks_allowed(nb, len(nsyms), nq, nsyms, status.astype(bool), qs)
        assert numpy.array_equal(got, allowed)
        got0 = oq.blks_allowed0(nb, len(nsyms), nq, nsyms, status.astype(bool), qs)
        assert numpy.array_equal(got0, allowed)


@pytest.mark.skipif(not os.path.exists(REF_LIB), reason="reference qsym.c not built here")
def test_blks_allowed_vs_reference_live():
    lib = ctypes.CDLL(REF_LIB)
    rng = numpy.random.default_rng(7)
    for _ in range(50):
        rank = int(rng.integers(2, 8))
        nq = 2
        nsyms = rng.integers(1, 5, size=rank).astype(numpy.int32)
        status = rng.integers(0, 2, size=rank).astype(numpy.int32)
        qs = [numpy.ascontiguousarray(rng.integers(-2, 3, size=(n, nq)) * 0.5) for n in nsyms]
        nb = int(numpy.prod(nsyms))
        ref = numpy.zeros(nb, dtype=numpy.int32)
        args = [q.ctypes.data_as(ctypes.c_void_p) for q in qs] + [ctypes.c_void_p()] * (8 - rank)
        lib.symAllowed(rank, nq, nsyms.ctypes.data_as(ctypes.c_void_p), status.ctypes.data_as(ctypes.c_void_p),
                       ref.ctypes.data_as(ctypes.c_void_p), *args)
        assert numpy.array_equal(oq.blks_allowed(nb, rank, nq, nsyms, status.astype(bool), qs), ref)


def _mpo_chain(K, p, int1e, int2e):
    T = mpo.genHfacSpatial(p, 2 * K, 0, int1e[p], int2e[p])[0].transpose(1, 2, 0)
    for i in range(1, K):
        W = mpo.genHfacSpatial(p, 2 * K, i, int1e[p], int2e[p])
        T = numpy.tensordot(T, W, axes=([-1], [0])).transpose(0, 3, 1, 4, 2)
        s = T.shape
        T = T.reshape(s[0] * s[1], s[2] * s[3], s[4])
    return T[:, :, 0]


@pytest.mark.parametrize("K", [2, 3])
def test_mpo_sum_equals_exact_hamiltonian(K):
    h, eri, _ = integrals.synthetic(K, 11)
    i1, i2, g = integrals.to_spin_orbital(h, eri)
    H = sum(_mpo_chain(K, p, i1, i2) for p in range(2 * K))
    Hf = integrals.fci_hamiltonian(i1, g).toarray()
    assert numpy.linalg.norm(H - Hf) < 1e-12 * numpy.linalg.norm(Hf)


def test_qt_mpo_matches_dense():
    """qtensor_opers.testHRfacSpatial (qtensor_opers.py:907-960): Qt == dense."""
    K = 4
    h, eri, _ = integrals.synthetic(K, 2)
    i1, i2, _ = integrals.to_spin_orbital(h, eri)
    pdic = {q: q for q in range(2 * K)}
    for p in range(2 * K):
        for i in range(K):
            qt = oqo.genHRfacSpatialQt([p, None], 2 * K, i, i1, i2, None, pdic)
            dense = mpo.genHRfacSpatial([p, None], 2 * K, i, i1, i2, None, pdic)
            ql, qr = oqo.bond_qnums(p, 2 * K, i)
            il = oqo.sortQnums(ql)
            ir = oqo.sortQnums(qr)
            assert numpy.abs(qt.toDenseTensor(qt.idlst) - dense[numpy.ix_(il, ir)]).max() < 1e-14


def test_hvec_hermitian_and_diag():
    """checkDiagQt (mpo_dmrg_kernelQt.py:129-150) on a seeded problem."""
    from tests.problems import random_problem, oracle_sigma, oracle_hdiag
    P = random_problem(K=4, nelec=4, D=6, isite=1, seed=3, device=False)
    n = P.ndim0
    H = numpy.array([oracle_sigma(P, e) for e in numpy.identity(n)]).T
    assert numpy.linalg.norm(H - H.T) < 1e-10 * numpy.linalg.norm(H)
    assert numpy.linalg.norm(numpy.diag(H) - oracle_hdiag(P)) < 1e-10


def test_davidson_vs_eigh():
    """tools/pdvdson.py:396-429 self-test (random 100x100, seed 0)."""
    numpy.random.seed(0)
    mat = numpy.random.uniform(-1, 1, size=(100, 100))
    mat = 0.5 * (mat + mat.T)
    efull = numpy.linalg.eigvalsh(mat)
    s = od.eigenSolver(numpy.random.default_rng(0))
    s.crit_vec = 1.e-7
    s.maxcycle = 200
    s.ndim = 100
    s.neig = 2
    s.diag = numpy.diag(mat).copy()
    s.HVec = mat.dot
    eigs, vecs, _ = s.solve_iter(iop=4)
    assert numpy.abs(eigs - efull[:2]).max() < 1e-8


def _fcidump():
    z = numpy.load(os.path.join(GOLD, "h6p_doublet_fcidump.npz"))
    return z


def test_fcidump_fci_matches_block():
    z = _fcidump()
    i1, i2, g = integrals.to_spin_orbital(z["h1e"], z["eri"])
    e = integrals.fci_energy(i1, g, int(z["nelec"]), 0.5 * int(z["ms2"]))[0] + float(z["ecore"])
    assert abs(e - float(z["e_block"])) < 5e-9


def test_oracle_dmrg_reaches_fci_on_fcidump():
    z = _fcidump()
    K = z["h1e"].shape[0]
    i1, i2, g = integrals.to_spin_orbital(z["h1e"], z["eri"])
    efci = integrals.fci_energy(i1, g, int(z["nelec"]), 0.0)[0]
    m = od.mpo_dmrg(seed=1)
    m.nsite, m.sbas, m.isym = K, 2 * K, 2
    m.build()
    m.occun = numpy.array([1., 1.] * 3 + [0., 0.] * 3)
    m.qsectors = {str([6.0, 0.0]): 1}
    m.partition()
    m.loadInts(i1, i2)
    m.dumpMPO()
    sc = od.schedule(maxM=64, tol=1e-9, maxiter=8)
    sc.normal(2)
    m.default(sc)
    assert abs(m.Energy - efci) < 1e-9
    assert abs(m.Energy + float(z["ecore"]) - float(z["e_block"])) < 5e-9


def _dense_spin_ops(K, npts, sval, sz):
    """Exact Fock-space P = sum_g w_g exp(-i beta_g S_y) from the JW operators."""
    import scipy.linalg
    from oracle import spinproj as osp
    a = integrals._jw_ops(2 * K)
    sp = sum((a[2 * i].T @ a[2 * i + 1]) for i in range(K)).toarray()
    gen = sp - sp.T

    class Q:
        pass
    q = Q()
    q.npts = npts
    osp.s2quad(q, sval, sz)
    P = sum(w * scipy.linalg.expm(-0.5 * b * gen) for b, w in zip(q.qpts, q.qwts))
    return P, gen


def test_spin_projection_exact_projector():
    """The restated quadrature (smalld + s2quad) gives the exact spin projector
    on the M = 0 sector of a K=4 Fock space: idempotent, and S^2 = S(S+1) on it."""
    K, npts = 4, 4
    P, gen = _dense_spin_ops(K, npts, 0, 0)
    idx = integrals.sector_indices(2 * K, 4, 0.0)
    Pm = P[numpy.ix_(idx, idx)]
    assert numpy.abs(Pm @ Pm - Pm).max() < 1e-12
    a = integrals._jw_ops(2 * K)
    sp = sum((a[2 * i].T @ a[2 * i + 1]) for i in range(K)).toarray()
    nup = sum((a[2 * i].T @ a[2 * i]) for i in range(K)).toarray()
    ndn = sum((a[2 * i + 1].T @ a[2 * i + 1]) for i in range(K)).toarray()
    szm = 0.5 * (nup - ndn)
    s2 = sp.T @ sp + szm @ szm + szm
    assert numpy.abs((s2 @ P)[numpy.ix_(idx, idx)]).max() < 1e-12
    assert numpy.trace(Pm) > 0.5


def test_spin_projected_kernels_equal_dense_operators():
    """Oracle HVecQt / SVecQt / SDiagQt of a spin-projected two-site dot equal
    U^T H P U x, U^T P U x and diag(U^T P U), with U the MPS basis of the dot
    (K=4, N=4, S=0, 4 Gauss-Legendre points): pins the N-only relabelling,
    the projection back on (N, Sz), the R(beta) site tensors and the P
    environments built by renormQt_S00."""
    import sys
    sys.path.insert(0, os.path.dirname(__file__))
    import problems
    from oracle import spinproj as osp
    K, nelec = 4, 4
    P = problems.random_problem(K=K, nelec=nelec, D=16, isite=1, seed=5, device=False, npts=4)
    m = P.o
    h1e, eri, _ = integrals.synthetic(K, P.seed, 1.0)
    _, _, gphys = integrals.to_spin_orbital(h1e, eri)
    H = integrals.fci_hamiltonian(P.int1e, gphys).toarray()
    Pd, _ = _dense_spin_ops(K, 4, 0, 0)
    A0 = P.lsites[0][0]            # (4, ldim)
    B3 = P.rsites[3][:, :, 0]      # (rdim, 4)

    def up(x):
        m.qtmp.value = numpy.asarray(x, dtype=float).copy()
        psi = m.qtmp.toDenseTensor(m.idlstCI)
        return numpy.einsum('al,lcdr,rb->acdb', A0, psi, B3).reshape(-1)

    def down(f):
        psi = numpy.einsum('al,acdb,rb->lcdr', A0, f.reshape(4, 4, 4, 4), B3)
        t = oq.qtensor(m.qtmp.status)
        t.fromQsyms(m.qtmp.rank, m.qtmp.qsyms, m.qtmp.ndims)
        t.fromDense(psi, m.idlstCI)
        return t.value

    rng = numpy.random.default_rng(11)
    x = rng.standard_normal(P.ndim0)
    hx = ok.HVecQt(x, [m, 1, 2, m.flst, 'L', True], P.ndim0, None)
    sx = osp.SVecQt(x, [m, 1, 2, m.flst, 'L', True], P.ndim0, None)
    hx_ref = down(H @ (Pd @ up(x)))
    sx_ref = down(Pd @ up(x))
    assert numpy.abs(hx - hx_ref).max() < 1e-10 * numpy.abs(hx_ref).max()
    assert numpy.abs(sx - sx_ref).max() < 1e-10 * numpy.abs(sx_ref).max()
    sd = problems.oracle_sdiag(P)
    eye = numpy.eye(P.ndim0)
    sd_ref = numpy.array([down(Pd @ up(eye[i]))[i] for i in range(P.ndim0)])
    assert numpy.abs(sd - sd_ref).max() < 1e-10


def test_rdm1_brute_force_restatement_equals_fock_space():
    """The restated eval_rdm1BF (reference properties/mpo_dmrg_propsItrf.py:
    204-263) on a random left-canonical MPS equals <psi|a+_p a_q|psi> from the
    Jordan-Wigner operators of the Fock space."""
    from oracle import properties as op
    rng = numpy.random.default_rng(8)
    K, D = 4, 6
    dims = [1] + [min(4 ** i, 4 ** (K - i), D) for i in range(1, K)] + [1]
    sites = []
    for i in range(K):
        a = rng.standard_normal((dims[i] * 4, dims[i + 1]))
        q, _ = numpy.linalg.qr(a)
        sites.append(q.reshape(dims[i], 4, dims[i + 1]))
    psi = op.mps_to_fock(sites)
    assert abs(psi @ psi - 1.0) < 1e-12
    a = integrals._jw_ops(2 * K)
    ref_t = numpy.zeros((K, K))
    ref_s = numpy.zeros((K, K))
    for p in range(K):
        for q in range(K):
            al = psi @ (a[2 * p].T @ (a[2 * q] @ psi))
            be = psi @ (a[2 * p + 1].T @ (a[2 * q + 1] @ psi))
            ref_t[p, q] = al + be
            ref_s[p, q] = 0.5 * (al - be)
    got_t, got_s = op.eval_rdm1BF(sites)
    assert numpy.abs(got_t - ref_t).max() < 1e-12
    assert numpy.abs(got_s - ref_s).max() < 1e-12
