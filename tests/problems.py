"""Seeded two-site problems shared by the parity tests, ``smoke()`` and the
benchmark: random block-sparse MPS sites with (N, Sz) bond sectors of a given
bond dimension, their left / right environments for every operator term,
and the wavefunction layout of the dot.  The same dense data feed the CPU
oracle (``oracle/``) and the GPU engine (``zmpo_dmrg_gb300``).
"""
import numpy

QPHYS = numpy.array([[0., 0.], [1., -0.5], [1., 0.5], [2., 0.]])


def _feasible_left(N, Sz, nelec, sz, nrest):
    ne = nelec - N
    na = 0.5 * ne + (sz - Sz)
    nb = 0.5 * ne - (sz - Sz)
    return 0 <= ne <= 2 * nrest and -1e-9 <= na <= nrest + 1e-9 and -1e-9 <= nb <= nrest + 1e-9 \
        and abs(na - round(na)) < 1e-9


def _pick(cands, D, center, rng, spread):
    """Sector dimensions of a truncated bond: keep sectors closest to the
    expected filling, each no larger than its multiplicity."""
    keys = sorted(cands)
    w = numpy.array([-((k[0] - center) ** 2) / spread - abs(k[1]) + 0.01 * rng.random() for k in keys])
    order = numpy.argsort(-w, kind="stable")
    dims = {}
    left = D
    # share proportional to exp(w), bounded by multiplicity, at least 1
    pw = numpy.exp(w - w.max())
    share = pw / pw.sum()
    for i in order:
        if left <= 0:
            break
        k = keys[i]
        d = int(min(cands[k], max(1, round(share[i] * D * 1.2)), left))
        if d > 0:
            dims[k] = d
            left -= d
    out = []
    for k in sorted(dims):
        out += [list(k)] * dims[k]
    return numpy.array(out, dtype=float)


def bond_structure(K, nelec, sz, D, rng):
    qnuml = [numpy.array([[0., 0.]])]
    for i in range(K):
        cands = {}
        for ql in map(tuple, qnuml[i]):
            for qn in map(tuple, QPHYS):
                k = (ql[0] + qn[0], ql[1] + qn[1])
                if _feasible_left(k[0], k[1], nelec, sz, K - i - 1):
                    cands[k] = cands.get(k, 0) + 1
        qnuml.append(_pick(cands, D, nelec * (i + 1) / K, rng, 2.0 + 0.25 * min(i + 1, K - i - 1)))
    qnumr = [None] * (K + 1)
    qnumr[K] = numpy.array([[0., 0.]])
    for i in range(K - 1, -1, -1):
        cands = {}
        for qn in map(tuple, QPHYS):
            for qr in map(tuple, qnumr[i + 1]):
                k = (qn[0] + qr[0], qn[1] + qr[1])
                if _feasible_left(k[0], k[1], nelec, sz, i):
                    cands[k] = cands.get(k, 0) + 1
        qnumr[i] = _pick(cands, D, nelec * (K - i) / K, rng, 2.0 + 0.25 * min(i, K - i))
    return qnuml, qnumr


def random_left_site(ql, qr, rng):
    """Left-canonical A[l, n, r] with q_l + q_n = q_r (QR per r sector)."""
    A = numpy.zeros((len(ql), 4, len(qr)))
    qln = (ql[:, None, :] + QPHYS[None, :, :]).reshape(-1, 2)
    for key in {tuple(x) for x in qr}:
        cols = numpy.flatnonzero(numpy.all(qr == key, axis=1))
        rows = numpy.flatnonzero(numpy.all(numpy.abs(qln - key) < 1e-12, axis=1))
        if rows.size == 0:
            continue
        M = rng.standard_normal((rows.size, cols.size))
        Q, _ = numpy.linalg.qr(M) if rows.size >= cols.size else (M / numpy.sqrt(rows.size), None)
        A.reshape(-1, len(qr))[numpy.ix_(rows, cols)] = Q[:, :cols.size]
    return A


def random_right_site(ql, qr, rng):
    """Right-canonical B[l, n, r] with q_l = q_n + q_r (QR per l sector)."""
    B = numpy.zeros((len(ql), 4, len(qr)))
    qnr = (QPHYS[:, None, :] + qr[None, :, :]).reshape(-1, 2)
    for key in {tuple(x) for x in ql}:
        rows = numpy.flatnonzero(numpy.all(ql == key, axis=1))
        cols = numpy.flatnonzero(numpy.all(numpy.abs(qnr - key) < 1e-12, axis=1))
        if cols.size == 0:
            continue
        M = rng.standard_normal((cols.size, rows.size))
        Q, _ = numpy.linalg.qr(M) if cols.size >= rows.size else (M / numpy.sqrt(cols.size), None)
        B.reshape(len(ql), -1)[numpy.ix_(rows, cols)] = Q[:, :rows.size].T
    return B


class Problem:
    pass


def random_problem(K=6, nelec=6, D=16, isite=2, seed=0, hop=1.0, sz=0.0, device=True,
                   with_oracle=True, npts=None, sval=0.0):
    """Two-site dot at (isite, isite+1) with environments of every H_p.
    With ``npts`` the problem is spin-projected: terms [p, g] over ``npts``
    Gauss-Legendre points for <S^2> = sval(sval+1), N-labelled environments
    and the P_g environments."""
    from oracle import integrals as oint
    rng = numpy.random.default_rng(seed)
    h1e, eri, _ = oint.synthetic(K, seed, hop)
    int1e, int2e, _ = oint.to_spin_orbital(h1e, eri)
    qnuml, qnumr = bond_structure(K, nelec, sz, D, rng)
    lsites = [random_left_site(qnuml[i], qnuml[i + 1], rng) for i in range(isite + 1)]
    rsites = {i: random_right_site(qnumr[i], qnumr[i + 1], rng) for i in range(isite + 2, K)}
    P = Problem()
    P.K, P.nelec, P.D, P.isite, P.seed = K, nelec, D, isite, seed
    P.int1e, P.int2e = int1e, int2e
    P.qnuml, P.qnumr, P.lsites, P.rsites = qnuml, qnumr, lsites, rsites
    P.key = [float(nelec), float(sz)]
    P.npts, P.sval, P.sz = npts, sval, sz
    if with_oracle:
        P.o = _oracle_side(P)
        P.ndim0 = P.o.qtmp.size_allowed
    if device:
        P.p = _product_side(P)
        P.ndim0 = P.p.qtmp.size_allowed
    return P


def _oracle_side(P):
    from oracle import dmrg as od, kernel as ok
    from oracle.qtensor import qtensor
    from oracle import spinproj as osp
    m = od.mpo_dmrg(seed=P.seed)
    m.nsite, m.sbas, m.isym, m.ifQt = P.K, 2 * P.K, 2, True
    sp = P.npts is not None
    if sp:
        m.ifs2proj, m.npts = True, P.npts
        osp.s2quad(m, P.sval, P.sz)
    m.build()
    m.partition()
    m.loadInts(P.int1e, P.int2e)
    m.dumpMPO()
    if sp:
        osp.dumpMPO_R(m)
    m.qnuml = list(P.qnuml)
    m.qnumr = list(P.qnumr)
    fL = m._boundary('lop', -1)
    fLp = osp.boundary_pops(m) if sp else None
    for i in range(P.isite):
        t = qtensor([False, False, True])
        t.fromDenseTensor(P.lsites[i], [P.qnuml[i], QPHYS, P.qnuml[i + 1]])
        fN = {}
        ok.renorm(m, i, 1, [[fL, None]], [[fN]], t, 'L')
        fL = fN
        if sp:
            fNp = {}
            osp.renormQt_S00(m, i, 1, [[None, None, fLp, None]], [[None, fNp]], t, 'L')
            fLp = fNp
    fR = m._boundary('rop', P.K)
    fRp = osp.boundary_pops(m) if sp else None
    for i in range(P.K - 1, P.isite + 1, -1):
        t = qtensor([True, False, False])
        t.fromDenseTensor(P.rsites[i], [P.qnumr[i], QPHYS, P.qnumr[i + 1]])
        fN = {}
        ok.renorm(m, i, 1, [[None, fR]], [[fN]], t, 'R')
        fR = fN
        if sp:
            fNp = {}
            osp.renormQt_S00(m, i, 1, [[None, None, None, fRp]], [[None, fNp]], t, 'R')
            fRp = fNp
    m.flst = [[fL, fR, fLp, fRp]] if sp else [[fL, fR]]
    m.dims = (len(P.qnuml[P.isite]), 16, len(P.qnumr[P.isite + 2]), 0)
    m.qlst = [P.qnuml[P.isite], QPHYS, QPHYS, P.qnumr[P.isite + 2]]
    m.setupQtmpCI(2, P.key)
    m._hvec_templates = None
    return m


def _product_side(P):
    from zmpo_dmrg_gb300.mpo_dmrg_class import mpo_dmrg
    from zmpo_dmrg_gb300.mpo_dmrg_kernel import renorm
    from zmpo_dmrg_gb300.qtensor import qtensor
    from zmpo_dmrg_gb300 import spinproj
    m = mpo_dmrg(seed=P.seed)
    m.nsite, m.sbas, m.isym = P.K, 2 * P.K, 2
    sp = P.npts is not None
    if sp:
        m.ifs2proj, m.npts = True, P.npts
        m.s2quad(P.sval, P.sz)
    m.build()
    m.partition()
    m.loadInts((P.int1e, P.int2e))
    m.dumpMPO()
    fL = m.boundary_env()
    fLp = spinproj.boundary_pops(m) if sp else None
    for i in range(P.isite):
        t = qtensor([False, False, True])
        t.fromDenseTensor(P.lsites[i], [P.qnuml[i], QPHYS, P.qnuml[i + 1]])
        fN = [[None, None]]
        renorm(m, i, 1, [[fL, None, fLp, None]], fN, t, 'L')
        fL, fLp = fN[0][0], fN[0][1]
    fR = m.boundary_env()
    fRp = spinproj.boundary_pops(m) if sp else None
    for i in range(P.K - 1, P.isite + 1, -1):
        t = qtensor([True, False, False])
        t.fromDenseTensor(P.rsites[i], [P.qnumr[i], QPHYS, P.qnumr[i + 1]])
        fN = [[None, None]]
        renorm(m, i, 1, [[None, fR, None, fRp]], fN, t, 'R')
        fR, fRp = fN[0][0], fN[0][1]
    m.flst = [[fL, fR, fLp, fRp]] if sp else [[fL, fR]]
    m.qnuml, m.qnumr = list(P.qnuml), list(P.qnumr)
    m.qlst = [P.qnuml[P.isite], QPHYS, QPHYS, P.qnumr[P.isite + 2]]
    m.setupQtmpCI(2, P.key)
    return m


def oracle_dense_side(P):
    """The oracle in its dense ("NQt") mode on the same dot: dense MPO sites,
    dense environments renormalised from the same random sites, ``dims`` as the
    reference's ``ci_solver`` sets them (normal problems only)."""
    from oracle import dmrg as od, kernel as ok
    assert P.npts is None
    m = od.mpo_dmrg(seed=P.seed)
    m.nsite, m.sbas, m.isym, m.ifQt = P.K, 2 * P.K, 2, False
    m.build()
    m.partition()
    m.loadInts(P.int1e, P.int2e)
    m.dumpMPO()
    fL = m._boundary('lop', -1)
    for i in range(P.isite):
        fN = {}
        ok.renorm(m, i, 1, [[fL, None]], [[fN]], P.lsites[i], 'L')
        fL = fN
    fR = m._boundary('rop', P.K)
    for i in range(P.K - 1, P.isite + 1, -1):
        fN = {}
        ok.renorm(m, i, 1, [[None, fR]], [[fN]], P.rsites[i], 'R')
        fR = fN
    m.flst = [[fL, fR]]
    ldim, rdim = len(P.qnuml[P.isite]), len(P.qnumr[P.isite + 2])
    m.dims = (ldim, 16, rdim, ldim * 16 * rdim)
    return m


def nqt_prjmap(P):
    """Dense indices of the (ldim, 4, 4, rdim) elements carrying the target
    label, ascending: the reference's NQt basis of the dot
    (``mpo_dmrg_dotutil.dptSymmetry``, 102-145)."""
    ql = numpy.asarray(P.qnuml[P.isite], dtype=float)
    qr = numpy.asarray(P.qnumr[P.isite + 2], dtype=float)
    qp = numpy.asarray(QPHYS, dtype=float)
    qt = (ql[:, None, None, None, :] + qp[None, :, None, None, :] + qp[None, None, :, None, :] +
          qr[None, None, None, :, :]).reshape(-1, ql.shape[1])
    key = numpy.asarray(P.key, dtype=float)
    return numpy.nonzero(numpy.abs(qt - key).sum(axis=1) < 1e-10)[0]


def packed_to_nqt(P, prj):
    """pos[i] = position in the NQt vector of packed element i."""
    m = P.o if getattr(P, "o", None) is not None else P.p
    dense_of_packed = numpy.asarray(m.qtmp.prjmap(m.idlstCI))
    inv = numpy.full(int(prj.max()) + 1, -1)
    inv[prj] = numpy.arange(prj.size)
    return inv[dense_of_packed]


def oracle_sigma_nqt(P, x, m=None):
    from oracle import kernel as ok
    m = m or oracle_dense_side(P)
    prj = nqt_prjmap(P)
    return ok.HVecNQt(numpy.asarray(x, dtype=float), [m, P.isite, 2, m.flst, 'L', True], prj.size, prj)


def oracle_sigma(P, x):
    from oracle import kernel as ok
    m = P.o
    return ok.HVecQt(numpy.asarray(x, dtype=float), [m, P.isite, 2, m.flst, 'L', True], P.ndim0, None)


def oracle_hdiag(P):
    from oracle import kernel as ok
    m = P.o
    prj = m.qtmp.prjmap(m.idlstCI)
    ldim, rdim = len(P.qnuml[P.isite]), len(P.qnumr[P.isite + 2])
    m.dims = (ldim, 16, rdim, ldim * 16 * rdim)
    return ok.HDiagQt([m, P.isite, 2, m.flst, 'L', True], P.ndim0, prj)


def product_sigma(P, x, precision="fp64"):
    from zmpo_dmrg_gb300.mpo_dmrg_kernel import HVec
    m = P.p
    m.precision = precision
    return HVec(numpy.asarray(x, dtype=float), [m, P.isite, 2, m.flst, 'L', True], P.ndim0, None)


def product_hdiag(P):
    from zmpo_dmrg_gb300.mpo_dmrg_kernel import HDiag
    m = P.p
    return HDiag([m, P.isite, 2, m.flst, 'L', True], P.ndim0, None).cpu().numpy()


def _renorm_site(P):
    """A left site at the dot (status 'L') or a right site (status 'R')."""
    rng = numpy.random.default_rng(P.seed + 101)
    i = P.isite
    return (P.lsites[i],
            random_right_site(P.qnumr[i + 1], P.qnumr[i + 2], rng))


def oracle_renorm(P, status, which=0):
    """New environments of the H_p terms (which=0) or, for a spin-projected
    problem, of the P_g points (which=1)."""
    from oracle import kernel as ok
    from oracle import spinproj as osp
    from oracle.qtensor import qtensor
    m = P.o
    A, B = _renorm_site(P)
    fN = {}
    fNp = {}
    if status == 'L':
        t = qtensor([False, False, True])
        t.fromDenseTensor(A, [P.qnuml[P.isite], QPHYS, P.qnuml[P.isite + 1]])
        ok.renorm(m, P.isite, 1, m.flst, [[fN]], t, 'L')
        if which == 1:
            osp.renormQt_S00(m, P.isite, 1, m.flst, [[fN, fNp]], t, 'L')
    else:
        t = qtensor([True, False, False])
        t.fromDenseTensor(B, [P.qnumr[P.isite + 1], QPHYS, P.qnumr[P.isite + 2]])
        ok.renorm(m, P.isite, 2, m.flst, [[fN]], t, 'R')
        if which == 1:
            osp.renormQt_S00(m, P.isite, 2, m.flst, [[fN, fNp]], t, 'R')
    f = fNp if which == 1 else fN
    out = []
    for iop in range(m.npts if which == 1 else m.nops):
        v = f['opers%d' % iop]
        out.append(numpy.zeros(0) if v is None else v.value)
    return out


def product_renorm(P, status, precision="fp64", which=0):
    from zmpo_dmrg_gb300.mpo_dmrg_kernel import renorm
    from zmpo_dmrg_gb300.qtensor import qtensor
    m = P.p
    m.precision_renorm = precision
    A, B = _renorm_site(P)
    fN = [[None]]
    if status == 'L':
        t = qtensor([False, False, True])
        t.fromDenseTensor(A, [P.qnuml[P.isite], QPHYS, P.qnuml[P.isite + 1]])
        renorm(m, P.isite, 1, m.flst, fN, t, 'L')
    else:
        t = qtensor([True, False, False])
        t.fromDenseTensor(B, [P.qnumr[P.isite + 1], QPHYS, P.qnumr[P.isite + 2]])
        renorm(m, P.isite, 2, m.flst, fN, t, 'R')
    E = fN[0][which]
    buf = E.buf.cpu().numpy()
    out = []
    for iop in range(m.npts if which == 1 else m.nops):
        if E.off[iop] < 0:
            out.append(numpy.zeros(0))
        else:
            n = E.tensors[iop].size_allowed
            out.append(buf[E.off[iop]:E.off[iop] + n])
    return out


def _random_civec(P, seed):
    m = P.o
    rng = numpy.random.default_rng(seed)
    m.qtmp.value = rng.standard_normal(m.qtmp.size_allowed)
    dense = m.qtmp.toDenseTensor(m.idlstCI)          # (ldim, 4, 4, rdim)
    return dense / numpy.linalg.norm(dense)


def prdm_inputs(P, status, seed=0):
    c = _random_civec(P, seed)
    ldim, rdim = c.shape[0], c.shape[3]
    if status == 'L':
        return c.reshape(1, ldim, 4, 4 * rdim)
    return c.reshape(1, ldim * 4, 4, rdim)


def oracle_prdm(P, status, noise=1e-4, seed=0):
    from oracle import dmrg as od
    m = P.o
    m.noise, m.inoise = noise, 0
    return od.pRDM(prdm_inputs(P, status, seed), [m, P.isite, 2, m.flst, status, True])


def product_prdm(P, status, noise=1e-4, seed=0):
    from zmpo_dmrg_gb300 import prdm
    m = P.p
    m.noise, m.inoise = noise, 0
    m.qkey = numpy.array(P.key)
    return prdm.pRDM(prdm_inputs(P, status, seed), [m, P.isite, 2, m.flst, status, True])


def oracle_svec(P, x):
    from oracle import spinproj as osp
    m = P.o
    return osp.SVecQt(numpy.asarray(x, dtype=float), [m, P.isite, 2, m.flst, 'L', True], P.ndim0, None)


def product_svec(P, x):
    from zmpo_dmrg_gb300.mpo_dmrg_kernel import SVec
    m = P.p
    return SVec(numpy.asarray(x, dtype=float), [m, P.isite, 2, m.flst, 'L', True], P.ndim0, None)


def oracle_sdiag(P):
    from oracle import spinproj as osp
    m = P.o
    prj = m.qtmp.prjmap(m.idlstCI)
    ldim, rdim = len(P.qnuml[P.isite]), len(P.qnumr[P.isite + 2])
    m.dims = (ldim, 16, rdim, ldim * 16 * rdim)
    return osp.SDiagQt([m, P.isite, 2, m.flst, 'L', True], P.ndim0, prj)


def product_sdiag(P):
    from zmpo_dmrg_gb300.mpo_dmrg_kernel import SDiag
    m = P.p
    return SDiag([m, P.isite, 2, m.flst, 'L', True], P.ndim0, None).cpu().numpy()


def b_resident_tiles(P):
    """Column tiles of the problem's sigma plan that the planner gives to the
    B-resident kernel (its rule: 64-column tiles over two or more 64-row
    tiles, or 32-column tiles over two or more 128-row tiles, K <= 256 in at
    most 32 segments).  Reads the task lists before the plan's first run."""
    from zmpo_dmrg_gb300 import engine as E
    from zmpo_dmrg_gb300.mpo_dmrg_kernel import _sigma_plan
    m = P.p
    plan = _sigma_plan([m, P.isite, 2, m.flst, 'L', True])
    eng = E.get()
    n = 0
    for pid in plan.pids:
        for st in range(plan.nlaunch):
            G, Sg = eng.step_tasks(pid, st)[:2]
            cs = numpy.concatenate([[0], numpy.cumsum(Sg['K'].astype(numpy.int64))])
            kt = cs[G['seg0'] + G['nseg']] - cs[G['seg0']]
            for M, N, k, ns in zip(G['M'], G['N'], kt, G['nseg']):
                wmax = 32 if k <= 32 else 64
                n0 = 0
                while n0 < N:
                    rem = N - n0
                    tn = wmax if rem >= wmax else (8 if rem <= 8 else 16 if rem <= 16 else 32 if rem <= 32 else 64)
                    hmax = 64 if tn == 64 else 128
                    if tn in (32, 64) and ns <= 32 and k <= 256 and M // hmax >= 2:
                        n += 1
                    n0 += tn
    return n


# ------------------------------------------- parity over a subset of terms
# At the benchmark sizes (K=24 D=512, K=20 D=512 with 8 quadrature points)
# the oracle cannot build the environments in reasonable time, so the check
# runs on the environments the engine built: the oracle's HVecQt over a subset
# of operator terms, fed the same environment values (copied from the device),
# against the engine's sigma over the same terms.

def class_covering_terms(P, per_class=1):
    """Operator terms of the dot with both environments, ``per_class`` of
    each operator class the dot meets (``qtensor_opers.case``, the unit the
    reference builds its task-list templates for, mpo_dmrg_kernelQt.py:196-236),
    evenly spaced within the class (for a spin-projected problem this varies
    the rotation angle from class to class), in term order."""
    from oracle import qtensor_opers
    m = P.p
    fL, fR = m.flst[0][0:2]
    by_class = {}
    for iop in range(m.nops):
        if fL.present(iop) and fR.present(iop):
            by_class.setdefault(qtensor_opers.case(m.opers[iop][0], P.isite, 2), []).append(iop)
    chosen = []
    for c, lst in by_class.items():
        n = min(per_class, len(lst))
        chosen += [lst[int((j + 0.5) * len(lst) / n)] for j in range(n)]
    return sorted(chosen), sorted(by_class)


def _oracle_qt_from_device(env, iop, host_buf):
    from oracle.qtensor import qtensor
    t = env.tensors[iop]
    q = qtensor(t.status)
    q.fromQsyms(3, t.qsyms, t.ndims)
    q.value = host_buf[env.off[iop]:env.off[iop] + q.size_allowed].copy()
    return q


def oracle_subset_driver(P, terms):
    """Oracle driver whose operator list is ``terms`` of the engine's driver,
    environments copied from the engine's EnvSets, MPO sites from the
    oracle's own builder."""
    from oracle import dmrg as od, qtensor_opers
    from oracle import spinproj as osp
    pm = P.p
    m = od.mpo_dmrg(seed=0)
    m.nsite, m.sbas, m.isym, m.ifQt = P.K, 2 * P.K, 2, True
    if P.npts is not None:
        m.ifs2proj, m.npts = True, P.npts
        osp.s2quad(m, P.sval, P.sz)
    m.build()
    m.partition()
    m.loadInts(P.int1e, P.int2e)
    fL, fR = pm.flst[0][0:2]
    Lb = fL.buf.cpu().numpy()
    Rb = fR.buf.cpu().numpy()
    opers = [m.opers[i] for i in terms]
    hpwts = numpy.array([m.hpwts[i] for i in terms])
    m.opers = opers
    m.hpwts = hpwts
    m.fhop = {'nops': len(terms)}
    fLo, fRo = {}, {}
    for k, iop in enumerate(terms):
        fLo['opers%d' % k] = _oracle_qt_from_device(fL, iop, Lb)
        fRo['opers%d' % k] = _oracle_qt_from_device(fR, iop, Rb)
        for s in (P.isite, P.isite + 1):
            m.fhop['site%d/op%d' % (s, k)] = qtensor_opers.genHRfacSpatialQt(
                opers[k], m.sbas, s, m.int1e, m.int2e, m.qpts, m.pdic)
    m.flst = [[fLo, fRo]]
    m.qlst = [P.qnuml[P.isite], QPHYS, QPHYS, P.qnumr[P.isite + 2]]
    m.setupQtmpCI(2, P.key)
    m._hvec_templates = None
    return m


def oracle_sigma_subset(P, terms, x, m=None):
    from oracle import kernel as ok
    m = m or oracle_subset_driver(P, terms)
    return ok.HVecQt(numpy.asarray(x, dtype=float), [m, P.isite, 2, m.flst, 'L', True],
                     m.qtmp.size_allowed, None)


def product_sigma_subset(P, terms, x, precision="fp64"):
    """The engine's HVec over ``terms`` only: views of the environment sets
    in which every other term is absent (a plan over exactly those terms)."""
    from zmpo_dmrg_gb300.mpo_dmrg_kernel import HVec, EnvSet
    m = P.p
    keep = numpy.zeros(m.nops, dtype=bool)
    keep[list(terms)] = True
    views = []
    for env in m.flst[0][0:2]:
        off = numpy.where(keep, env.off, -1)
        views.append(EnvSet(env.buf, off, env.layouts, env.tensors))
    flst = [views + list(m.flst[0][2:])]
    m.precision = precision
    return HVec(numpy.asarray(x, dtype=float), [m, P.isite, 2, flst, 'L', True], P.ndim0, None)


# ------------------------------------------ host model of a plan's tasks
def run_tasks_on_host(eng, pid, nsteps, bufs, gemm=None, written=None, part_gemm=None):
    """Execute a plan's task records with NumPy (test-only model of the
    kernels' semantics, incl. column-block groups and split-K sums); returns
    the buffers.  ``gemm(A, B)``, when given, computes each group's product
    from its segments joined along K (A scaled by the segment weights) -- a
    model of a kernel's arithmetic; it may return None to keep the FP64 sum.
    ``part_gemm`` (default ``gemm``) does the same for the split-K parts of
    groups longer than the split-K length, whose results the split-K sums add
    in order.  ``written``, when given, collects (buffer, flat indices,
    values) of the groups (and sums of parts) whose product came from the
    model."""
    PART = 6  # scratch buffer of the split-K parts
    for st in range(nsteps):
        groups, segs, cbl, segb, reds = eng.step_tasks(pid, st)
        if len(reds):
            bufs = list(bufs)
            bufs[PART] = numpy.zeros(int(max(r["part_off"] + r["nparts"] * r["M"] * r["N"] for r in reds)))
        part_modelled = {}
        for g in groups:
            M, N = int(g["M"]), int(g["N"])
            is_part = int(g["cbuf"]) == PART
            acc = numpy.zeros((M, N))
            mi = numpy.arange(M)
            As, Bs = [], []
            for si in range(int(g["nseg"])):
                s = segs[g["seg0"] + si]
                K = int(s["K"])
                ki = numpy.arange(K)
                A = bufs[int(s["abuf"])][s["a_off"] + mi[:, None] * s["sam"] + ki[None, :] * s["sak"]]
                if g["ncb"] == 0:
                    ni = numpy.arange(N)
                    B = bufs[int(s["bbuf"])][s["b_off"] + ki[:, None] * s["sbk"] + ni[None, :] * s["sbn"]]
                else:
                    B = numpy.zeros((K, N))
                    for j in range(int(g["ncb"])):
                        cb = cbl[g["cb0"] + j]
                        sb = segb[g["sb0"] + si * g["ncb"] + j]
                        if sb["b_off"] < 0:
                            continue
                        ni = numpy.arange(int(cb["n"]))
                        B[:, cb["n0"]:cb["n0"] + cb["n"]] = bufs[int(s["bbuf"])][
                            sb["b_off"] + ki[:, None] * sb["sbk"] + ni[None, :] * sb["sbn"]]
                acc += s["alpha"] * (A @ B)
                if gemm is not None:
                    As.append(A * s["alpha"] if s["alpha"] != 1.0 else A)
                    Bs.append(B)
            modelled = False
            f = (part_gemm or gemm) if is_part else gemm
            if f is not None and As:
                got = f(numpy.concatenate(As, axis=1), numpy.concatenate(Bs, axis=0))
                if got is not None:
                    acc = got
                    modelled = True
            out = bufs[int(g["cbuf"])]
            if g["ncb"] == 0:
                ni = numpy.arange(N)
                idx = g["c_off"] + mi[:, None] * g["scm"] + ni[None, :] * g["scn"]
                out[idx] = acc
                if is_part:
                    part_modelled[int(g["c_off"])] = modelled
                elif modelled and written is not None:
                    written.append((int(g["cbuf"]), idx.ravel(), acc.ravel()))
            else:
                for j in range(int(g["ncb"])):
                    cb = cbl[g["cb0"] + j]
                    ni = numpy.arange(int(cb["n"]))
                    idx = cb["c_off"] + mi[:, None] * cb["scm"] + ni[None, :] * cb["scn"]
                    part = acc[:, cb["n0"]:cb["n0"] + cb["n"]]
                    out[idx] = part
                    if modelled and written is not None:
                        written.append((int(g["cbuf"]), idx.ravel(), part.ravel()))
        for r in reds:
            # the split-K sum: parts added in order (as k_reduce does)
            M, N, mn = int(r["M"]), int(r["N"]), int(r["M"]) * int(r["N"])
            acc = numpy.zeros(mn)
            for t in range(int(r["nparts"])):
                acc = acc + bufs[PART][int(r["part_off"]) + t * mn:int(r["part_off"]) + (t + 1) * mn]
            mi, ni = numpy.divmod(numpy.arange(mn), N)
            idx = r["c_off"] + mi * r["scm"] + ni * r["scn"]
            bufs[int(r["cbuf"])][idx] = acc
            if written is not None and all(part_modelled.get(int(r["part_off"]) + t * mn, False)
                                           for t in range(int(r["nparts"]))):
                written.append((int(r["cbuf"]), idx, acc))
    return bufs


def host_sigma_terms(P, terms, x, gemm=None, fill=0.0):
    """The engine's sigma plan over the operator terms ``terms`` of the
    oracle side of ``P`` (its environments and MPO sites as the operands),
    built by the engine's planner and executed on the host from the task
    records (NumPy model of the kernels); returns (sigma, groups per step).
    ``fill`` is the initial value of the output and of the workspace (NaN:
    an output element no task writes, or a read of an intermediate no task
    wrote, shows up as NaN).  Needs no GPU."""
    from zmpo_dmrg_gb300 import engine as E, mpo as pm
    m = P.o
    eng = E.get()
    fL, fR = m.flst[0]

    def lay(t):
        return eng.layout(t.qsyms, t.ndims, t.status)

    Lv, Rv, Wv = [], [], []
    offL, offR, offWi, offWj, wts = [], [], [], [], []
    classes, op_cls, lL, lWi, lWj, lRf = {}, [], [], [], [], []
    pos = {"L": 0, "R": 0, "W": 0}
    for iop in terms:
        Lt, Rt = fL['opers%d' % iop], fR['opers%d' % iop]
        if Lt is None or Rt is None:
            continue
        Wi = m.fhop['site%d/op%d' % (P.isite, iop)]
        Wj = m.fhop['site%d/op%d' % (P.isite + 1, iop)]
        offL.append(pos["L"]); Lv.append(Lt.value); pos["L"] += Lt.value.size
        offR.append(pos["R"]); Rv.append(Rt.value); pos["R"] += Rt.value.size
        offWi.append(pos["W"]); Wv.append(Wi.value); pos["W"] += Wi.value.size
        offWj.append(pos["W"]); Wv.append(Wj.value); pos["W"] += Wj.value.size
        wts.append(m.hpwts[iop])
        c0 = pm.op_class(m.opers[iop][0], P.isite, 2)
        if c0 not in classes:
            classes[c0] = len(classes)
            lL.append(lay(Lt)); lWi.append(lay(Wi)); lWj.append(lay(Wj))
            lRf.append(eng.derive(lay(Rt), [-Rt.qsyms[0], m.qkey - Rt.qsyms[1], m.qkey - Rt.qsyms[2]],
                                  Rt.status))
        op_cls.append(classes[c0])
    if not op_cls:
        return numpy.zeros(P.ndim0), []
    pid, ws = eng.sigma_plan(2, op_cls, lL, lWi, lWj, lRf, lay(m.qtmp), offL, offR, offWi, offWj, wts)
    bufs = [numpy.concatenate(Lv), numpy.concatenate(Rv), numpy.concatenate(Wv), numpy.asarray(x, dtype=float),
            numpy.full(P.ndim0, fill), numpy.full(max(ws // 8, 1), fill), numpy.zeros(1), numpy.zeros(1)]
    _, _, nl = eng.plan_stats(pid)
    groups_all = [eng.step_tasks(pid, st)[0] for st in range(nl)]
    y = run_tasks_on_host(eng, pid, nl, bufs, gemm)[4]
    eng.destroy_plan(pid)
    return y, groups_all


def host_renorm(P, status, fill=0.0):
    """The engine's renormalisation plan for the oracle side of ``P`` (status
    'L': the left environments extended by the dot's left site; 'R': the
    right ones by the site right of the dot), built by the engine's planner
    and executed on the host from the task records (NumPy model of the
    kernels).  Returns the new environment of every term (empty where absent)
    and the plan's groups per step.  ``fill`` is the initial value of the
    output and of the workspace (as in ``host_sigma_terms``).  Needs no GPU."""
    from zmpo_dmrg_gb300 import engine as E, mpo as pm
    from oracle.qtensor import qtensor
    m = P.o
    eng = E.get()

    def lay(t):
        return eng.layout(t.qsyms, t.ndims, t.status)

    A, B = _renorm_site(P)
    if status == 'L':
        t = qtensor([False, False, True])
        t.fromDenseTensor(A, [P.qnuml[P.isite], QPHYS, P.qnuml[P.isite + 1]])
        fE, jsite = m.flst[0][0], P.isite
    else:
        t = qtensor([True, False, False])
        t.fromDenseTensor(B, [P.qnumr[P.isite + 1], QPHYS, P.qnumr[P.isite + 2]])
        fE, jsite = m.flst[0][1], P.isite + 1
    ops, Ev, Wv, off_env, off_W = [], [], [], [], []
    classes, op_cls, lay_env, lay_W = {}, [], [], []
    pos = {"E": 0, "W": 0}
    for iop in range(m.nops):
        Et = fE['opers%d' % iop]
        if Et is None:
            continue
        Wt = m.fhop['site%d/op%d' % (jsite, iop)]
        ops.append(iop)
        off_env.append(pos["E"]); Ev.append(Et.value); pos["E"] += Et.value.size
        off_W.append(pos["W"]); Wv.append(Wt.value); pos["W"] += Wt.value.size
        c0 = pm.op_class(m.opers[iop][0], jsite)
        if c0 not in classes:
            classes[c0] = len(classes)
            lay_env.append(lay(Et))
            if status == 'L':
                lay_W.append(lay(Wt))
            else:
                st = numpy.array(Wt.status).copy()
                st[0], st[1] = not st[0], not st[1]
                lay_W.append(eng.derive(lay(Wt), [-Wt.qsyms[0], -Wt.qsyms[1], Wt.qsyms[2], Wt.qsyms[3]], st))
        op_cls.append(classes[c0])
    pid, lay_out, off_out, total, ws = eng.renorm_plan(status, op_cls, lay_env, lay_W, lay(t), off_env, off_W)
    bufs = [numpy.concatenate(Ev), numpy.zeros(1), numpy.concatenate(Wv), t.value.copy(), numpy.full(max(total, 1), fill),
            numpy.full(max(ws // 8, 1), fill), numpy.zeros(1), numpy.zeros(1)]
    groups_all = [eng.step_tasks(pid, st)[0] for st in range(3)]
    out = run_tasks_on_host(eng, pid, 3, bufs)[4]
    envs = [numpy.zeros(0) for _ in range(m.nops)]
    for k, iop in enumerate(ops):
        c = op_cls[k]
        if lay_out[c] < 0 or off_out[k] < 0:
            continue
        size = eng.layout_blocks(int(lay_out[c]))[0]
        envs[iop] = out[off_out[k]:off_out[k] + size]
    eng.destroy_plan(pid)
    return envs, groups_all
