"""Host-side logic of the product on the CPU (no GPU calls): the C ABI
library loads and exports every declared symbol, its block rule, layouts and
task lists agree with the oracle, and the product's MPO / integrals /
schedule / decimation agree with the oracle's restatement."""
import ctypes
import os
import re

import numpy
import pytest

from oracle import integrals as oint, mpo as omp, qtensor as oq, qtensor_opers as oqo, dmrg as od
from zmpo_dmrg_gb300 import _lib, engine as E, mpo as pm, integrals as pint
from zmpo_dmrg_gb300.mpo_dmrg_schedule import schedule as pschedule
from zmpo_dmrg_gb300.mpo_dmrg_class import rdm_blkdiag as p_rdm_blkdiag
from zmpo_dmrg_gb300.qtensor import qtensor as pq
from tests.problems import run_tasks_on_host as _run_tasks_on_host

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "zmpo_gb300.h")


@pytest.fixture(scope="module", autouse=True)
def built():
    from zmpo_dmrg_gb300 import build
    build.build()


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*int\s+(\w+)\s*\(", text, flags=re.M)))


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(_lib.LIBPATH)
    names = declared_symbols()
    assert "zmpo_sigma" in names and "symAllowed" in names
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) <= set(_lib.EXPORTS)
    assert _lib.lib().zmpo_version() == 1


def test_symallowed_export_matches_reference_golden():
    z = numpy.load(os.path.join(ROOT, "tests", "golden", "qsym_reference.npz"))
    lib = _lib.lib()
    for c in range(int(z["ncase"])):
        nsyms = z["c%d_nsyms" % c].astype(numpy.int32)
        status = z["c%d_status" % c].astype(numpy.int32)
        nq = int(z["c%d_nq" % c])
        qs = [numpy.ascontiguousarray(z["c%d_q%d" % (c, i)]) for i in range(len(nsyms))]
        out = numpy.zeros(int(numpy.prod(nsyms)), dtype=numpy.int32)
        args = [q.ctypes.data_as(ctypes.c_void_p) for q in qs] + [None] * (8 - len(qs))
        assert lib.symAllowed(len(nsyms), nq, _lib.iptr(nsyms), _lib.iptr(status), _lib.iptr(out), *args) == 0
        assert numpy.array_equal(out, z["c%d_allowed" % c])


def test_error_convention():
    eng = E.get()
    with pytest.raises(RuntimeError, match="unknown"):
        eng.layout_blocks(10 ** 6)
    assert "unknown layout" in _lib.last_error()


def test_integrals_match_oracle(tmp_path):
    for K, seed, hop in [(4, 1, 1.0), (6, 9, 0.7)]:
        a = pint.synthetic(K, seed, hop)
        b = oint.synthetic(K, seed, hop)
        assert numpy.array_equal(a[0], b[0]) and numpy.allclose(a[1], b[1], atol=1e-15, rtol=0)
        p1, p2 = pint.spin_orbital(a[0], a[1])
        o1, o2, _ = oint.to_spin_orbital(b[0], b[1])
        assert numpy.array_equal(p1, o1) and numpy.allclose(p2, o2, atol=1e-15, rtol=0)
    fd = os.path.join(ROOT, "tests", "golden", "h6p_doublet_fcidump.npz")
    z = numpy.load(fd)
    # round trip through the FCIDUMP text format
    path = str(tmp_path / "rt.FCIDUMP")
    n = z["h1e"].shape[0]
    with open(path, "w") as f:
        f.write(" &FCI NORB=%d,NELEC=%d,MS2=%d,\n  ORBSYM=%s\n  ISYM=1,\n &END\n"
                % (n, int(z["nelec"]), int(z["ms2"]), "1," * n))
        for i in range(n):
            for j in range(i + 1):
                for k in range(n):
                    for l in range(k + 1):
                        if i * (i + 1) // 2 + j >= k * (k + 1) // 2 + l and z["eri"][i, j, k, l] != 0:
                            f.write("%.16e %d %d %d %d\n" % (z["eri"][i, j, k, l], i + 1, j + 1, k + 1, l + 1))
        for i in range(n):
            for j in range(i + 1):
                f.write("%.16e %d %d 0 0\n" % (z["h1e"][i, j], i + 1, j + 1))
        f.write("%.16e 0 0 0 0\n" % float(z["ecore"]))
    a = pint.read_fcidump(path)
    b = oint.read_fcidump(path)
    assert numpy.array_equal(a["eri"], b["eri"]) and numpy.array_equal(a["h1e"], b["h1e"])
    assert a["ecore"] == b["ecore"] and a["norb"] == b["norb"] == n
    assert numpy.allclose(a["eri"], z["eri"], atol=1e-15)


def test_mpo_matches_oracle():
    K = 5
    h, eri, _ = oint.synthetic(K, 4)
    i1, i2, _ = oint.to_spin_orbital(h, eri)
    pdic = {q: q for q in range(2 * K)}
    for p in range(2 * K):
        for i in range(K):
            a = omp.genHRfacSpatial([p, None], 2 * K, i, i1, i2, None, pdic)
            b = pm.hp_spatial_site([p, None], 2 * K, i, i1, i2)
            assert numpy.array_equal(a, b)
            qa = oqo.genHRfacSpatialQt([p, None], 2 * K, i, i1, i2, None, pdic)
            qb = pm.hp_spatial_qt([p, None], 2 * K, i, i1, i2)
            assert numpy.array_equal(qa.value, qb.value)
            assert all(numpy.array_equal(x, y) for x, y in zip(qa.qsyms, qb.qsyms))
            assert oqo.case(p, i, 2) == pm.op_class(p, i, 2) and oqo.case(p, i) == pm.op_class(p, i)


def test_spin_projected_mpo_matches_oracle():
    K = 3
    h, eri, _ = oint.synthetic(K, 8)
    i1, i2, _ = oint.to_spin_orbital(h, eri)
    qpts = [0.3, 1.7]
    pdic = {q: q for q in range(2 * K)}
    for p in range(2 * K):
        for ip in range(2):
            for i in range(K):
                qa = oqo.genHRfacSpatialQt([p, ip], 2 * K, i, i1, i2, qpts, pdic)
                qb = pm.hp_spatial_qt([p, ip], 2 * K, i, i1, i2, qpts, pdic)
                assert numpy.allclose(qa.value, qb.value, atol=1e-15, rtol=0)


def test_layouts_and_task_lists_match_oracle():
    """Engine packing == oracle fromQsyms; engine sigma task lists give the
    oracle's F_ref (sum of 2mnk over its tensordotSYM tasks)."""
    from tests.problems import random_problem, oracle_sigma
    P = random_problem(K=6, nelec=6, D=16, isite=2, seed=1, device=False)
    m = P.o
    eng = E.get()
    fL, fR = m.flst[0]

    def lay(t):
        return eng.layout(t.qsyms, t.ndims, t.status)

    for iop in range(m.nops):
        for t in (fL['opers%d' % iop], fR['opers%d' % iop]):
            size, flat, off = eng.layout_blocks(lay(t))
            assert size == t.size_allowed
            assert numpy.array_equal(flat, t.idx_allowed)
            assert numpy.array_equal(off, t.ioff_allowed[t.idx_allowed])
    classes, op_cls, lL, lWi, lWj, lRf = {}, [], [], [], [], []
    for iop in range(m.nops):
        c0 = pm.op_class(m.opers[iop][0], P.isite, 2)
        if c0 not in classes:
            classes[c0] = len(classes)
            R = fR['opers%d' % iop]
            lL.append(lay(fL['opers%d' % iop]))
            lWi.append(lay(m.fhop['site%d/op%d' % (P.isite, iop)]))
            lWj.append(lay(m.fhop['site%d/op%d' % (P.isite + 1, iop)]))
            lRf.append(eng.derive(lay(R), [-R.qsyms[0], m.qkey - R.qsyms[1], m.qkey - R.qsyms[2]], R.status))
        op_cls.append(classes[c0])
    n = m.nops
    pid, ws = eng.sigma_plan(2, op_cls, lL, lWi, lWj, lRf, lay(m.qtmp), [0] * n, [0] * n, [0] * n, [0] * n,
                             [1.0] * n)
    oq.reset_flops()
    oracle_sigma(P, numpy.ones(P.ndim0))
    flops, ntasks, nl = eng.plan_stats(pid)
    assert flops == oq.FLOPS["count"] and nl == 4 and ws > 0


def test_product_qtensor_dense_roundtrip_and_prjmap():
    rng = numpy.random.default_rng(3)
    ql = numpy.array([[0, 0], [1, .5], [1, -.5], [1, .5], [2, 0]], dtype=float)
    qp = numpy.array([[0., 0.], [1., -0.5], [1., 0.5], [2., 0.]])
    qr = numpy.array([[1, .5], [2, 0], [2, 0], [3, .5]], dtype=float)
    A = rng.standard_normal((5, 4, 4))
    a = pq([False, False, True])
    a.fromDenseTensor(A, [ql, qp, qr])
    b = oq.qtensor([False, False, True])
    b.fromDenseTensor(A, [ql, qp, qr])
    assert numpy.array_equal(a.value, b.value)
    assert numpy.array_equal(a.prjmap(a.idlst), b.prjmap(b.idlst))
    assert numpy.array_equal(a.toDenseTensor(a.idlst), b.toDenseTensor(b.idlst))


def test_schedule_matches_oracle():
    for maxM, tol in [(64, 1e-9), (512, 1e-8), (1000, 1e-7)]:
        a = pschedule(maxM=maxM, tol=tol)
        a.normal()
        b = od.schedule(maxM=maxM, tol=tol)
        b.normal()
        assert (a.MaxMs, a.Tols, a.Noises, a.change) == (b.MaxMs, b.Tols, b.Noises, b.change)


def test_rdm_blkdiag_matches_oracle():
    rng = numpy.random.default_rng(5)
    classes = [[0., 0.], [1., .5], [1., -.5], [2., 0.]] * 6
    X = rng.standard_normal((24, 30))
    rho = X @ X.T
    for cut in (5, 12, -1):
        a = p_rdm_blkdiag(rho, classes, -1e-14, cut)
        b = od.rdm_blkdiag(rho, classes, -1e-14, cut)
        assert abs(a[0] - b[0]) < 1e-13
        assert numpy.array_equal(numpy.array(a[1]), numpy.array(b[1]))
        assert numpy.allclose(numpy.abs(a[2]), numpy.abs(b[2]), atol=1e-10)


def test_generalised_davidson_matches_eigh():
    """The generalised Davidson (pgdvdson restated, basis as torch tensors; CPU
    here) reaches scipy's eigh(H, S) with restarts, S-normalised vectors."""
    import scipy.linalg
    import torch
    from zmpo_dmrg_gb300 import pgdvdson
    rng = numpy.random.default_rng(3)
    n = 200
    A = rng.standard_normal((n, n))
    H = (A + A.T) / 2 + numpy.diag(numpy.arange(n) * 0.5)
    B = rng.standard_normal((n, n)) * 0.05
    S = numpy.eye(n) + B @ B.T
    e_ref = scipy.linalg.eigh(H, S, eigvals_only=True)[:2]
    Ht, St = torch.tensor(H), torch.tensor(S)
    sol = pgdvdson.eigenSolver(numpy.random.default_rng(0))
    sol.HVec = lambda v: Ht @ v
    sol.SVec = lambda v: St @ v
    sol.ndim, sol.neig = n, 2
    sol.diag = torch.diag(Ht).clone()
    sol.maxcycle = 200
    sol.crit_e, sol.crit_vec = 1e-12, 1e-9
    e, x, nmvp = sol.solve_iter()
    assert sol.ifconv and nmvp > 2 * sol.nfac * sol.neig   # restarted at least once
    assert numpy.abs(e - e_ref).max() < 1e-9
    assert float(((x @ St) @ x.T - torch.eye(2, dtype=torch.float64)).abs().max()) < 1e-12


def test_n_only_relabel_matches_oracle():
    """Product N-only scatter / gather maps == the oracle's reduceQsymsToN and
    projectionNMs on a spin-projected dot (bit-exact), and the quadrature
    points and weights agree."""
    import torch
    from tests.problems import random_problem
    from zmpo_dmrg_gb300 import spinproj
    from zmpo_dmrg_gb300.qtensor import qtensor as pqt, fromQnums
    from oracle import spinproj as osp
    P = random_problem(K=6, nelec=5, D=16, isite=2, seed=2, device=False, npts=4, sval=0.5, sz=0.5)
    m = P.o
    qn = [m.qlst[0], m.qlst[1], m.qlst[2], m.qkey - m.qlst[3]]
    t = pqt([False, False, False, True])
    rank, qsyms, ndims, _ = fromQnums(qn)
    t.fromQsyms(rank, qsyms, ndims, ifallocate=False)
    qN, idx = spinproj.n_only_map(t)
    x = numpy.random.default_rng(1).standard_normal(m.qtmp.size_allowed)
    m.qtmp.value = x.copy()
    red = m.qtmp.reduceQsymsToN()
    assert qN.size_allowed == red.size_allowed
    xN = numpy.zeros(qN.size_allowed)
    xN[idx] = x
    assert numpy.array_equal(xN, red.value)
    y = numpy.random.default_rng(2).standard_normal(qN.size_allowed)
    red.value = y.copy()
    assert numpy.array_equal(y[idx], red.projectionNMs(m.qtmp.qsyms).value)

    class Q:
        npts = 6
    a, b = Q(), Q()
    spinproj.s2quad(a, 1.5, 0.5)
    osp.s2quad(b, 1.5, 0.5)
    assert numpy.abs(a.qpts - b.qpts).max() < 1e-14
    assert numpy.abs(a.qwts - b.qwts).max() < 1e-13


def _host_sigma(P, gemm=None):
    """The engine's sigma plan for the oracle side of ``P`` executed on the
    host from its task records; returns (sigma, oracle sigma, groups)."""
    from tests.problems import oracle_sigma, host_sigma_terms
    x = numpy.random.default_rng(3).standard_normal(P.ndim0)
    y, groups_all = host_sigma_terms(P, range(P.o.nops), x, gemm)
    return y, oracle_sigma(P, x), groups_all


def test_sigma_task_lists_compute_the_oracle_sigma():
    """The engine's sigma plan (O = Wi.Wj, T1 = L.psi, T3 = T1.O, sigma = T3.R
    with column-block groups) executed from its task records by a NumPy model
    of the kernels equals the oracle's HVecQt (FP64, 1e-12): checks the
    planner's addressing on the CPU, before any kernel runs."""
    from tests.problems import random_problem
    P = random_problem(K=6, nelec=6, D=16, isite=2, seed=1, device=False)
    y, ref, groups_all = _host_sigma(P)
    assert any((g["ncb"] > 0).any() for g in groups_all)      # column-block groups are in use
    assert numpy.linalg.norm(y - ref) <= 1e-12 * numpy.linalg.norm(ref)


@pytest.mark.parametrize("case", [dict(K=8, nelec=8, D=32, isite=3, seed=4),
                                  dict(K=10, nelec=10, D=64, isite=4, seed=7)])
def test_sigma_one_pass_split_model_error(case):
    """Sigma with every group whose K fits one pass (K <= 256) multiplied by
    the exact model of the one-pass split arithmetic (whole-K row and column
    exponents, tests/split_model.py): within the split path's 1e-8 of the
    oracle's FP64 sigma."""
    from tests.problems import random_problem
    from tests.split_model import one_pass_gemm
    P = random_problem(device=False, **case)
    used = []

    def gemm(A, B):
        if A.shape[1] > 256:
            return None
        used.append(A.shape)
        return one_pass_gemm(A, B)

    y, ref, _ = _host_sigma(P, gemm)
    assert len(used) > 100
    err = numpy.linalg.norm(y - ref) / numpy.linalg.norm(ref)
    assert err < 1e-8, err


def test_sigma_plan_key_is_structural():
    """Sigma plans are reused across sweeps by a content key: equal for
    environments of the same block structure and offsets (new buffers),
    different when any structure, offset or the wavefunction layout differs."""
    from types import SimpleNamespace
    from zmpo_dmrg_gb300.mpo_dmrg_kernel import EnvSet, _sigma_key
    qa = numpy.array([[0, 0], [1, .5], [1, -.5]], dtype=float)
    qb = numpy.array([[0, 0], [1, .5]], dtype=float)

    def tens(q, d):
        t = pq([True, False, True])
        t.fromQsyms(3, [q, q, q], [d, d, d], ifallocate=False)
        return t

    def env(d, off1=7):
        t = tens(qa, d)
        return EnvSet(None, [0, off1, -1], [t.layout] * 3, [t, t, None])

    psi = tens(qb, [2, 3])
    dmrg = SimpleNamespace(mpo_store=SimpleNamespace(uid=1), ifs2proj=False, nops=3, qkey=[2.0, 0.0],
                           hpwts=numpy.ones(3), qtmp=psi)
    k0 = _sigma_key(dmrg, 1, 2, env([1, 2, 2]), env([3, 1, 1]))
    assert k0 == _sigma_key(dmrg, 1, 2, env([1, 2, 2]), env([3, 1, 1]))      # new EnvSets, same structure
    assert k0 != _sigma_key(dmrg, 1, 2, env([1, 2, 3]), env([3, 1, 1]))      # a sector dimension
    assert k0 != _sigma_key(dmrg, 1, 2, env([1, 2, 2], 8), env([3, 1, 1]))   # an offset
    assert k0 != _sigma_key(dmrg, 2, 2, env([1, 2, 2]), env([3, 1, 1]))      # the dot
    dmrg.qtmp = tens(qb, [2, 4])
    assert k0 != _sigma_key(dmrg, 1, 2, env([1, 2, 2]), env([3, 1, 1]))      # the wavefunction layout


def test_transposed_builder_equals_autograd_of_the_builder():
    """The energy gradient's chain rule (adjoint.integral_gradients: the
    transposed MPO builder, the site tensors being linear in the integrals)
    equals torch autograd through the builder, and the exact change of the
    linear functional sum_j,p <G_p(j), W_p(j)(h, g)> along a random direction."""
    import torch
    from zmpo_dmrg_gb300.mpo_dmrg_class import mpo_dmrg
    from zmpo_dmrg_gb300 import adjoint
    K = 5
    m = mpo_dmrg(seed=1)
    m.nsite, m.sbas, m.isym = K, 2 * K, 2
    m.build()
    m.partition()
    h, eri, _ = pint.synthetic(K, 3)
    i1, i2 = pint.spin_orbital(h, eri)
    rng = numpy.random.default_rng(0)
    grads = [[None] * m.nops for _ in range(K)]
    for j in range(K):
        for iop in range(m.nops):
            if rng.random() < 0.8:
                W = pm.hp_spatial_site(m.opers[iop], m.sbas, j, i1[m.pidx], i2[m.pidx], None, m.pdic)
                grads[j][iop] = rng.standard_normal(W.shape)
    a1, a2 = adjoint.integral_gradients(m, h, eri, grads)
    hh = torch.tensor(h, requires_grad=True)
    gg = torch.tensor(eri, requires_grad=True)
    t1, t2 = adjoint.spin_orbital_torch(hh, gg)
    t1, t2 = t1[m.pidx], t2[m.pidx]
    tot = torch.zeros((), dtype=torch.float64)
    for j in range(K):
        for iop in range(m.nops):
            if grads[j][iop] is not None:
                W = pm.hp_spatial_site(m.opers[iop], m.sbas, j, t1, t2, None, m.pdic)
                tot = tot + (W * torch.from_numpy(grads[j][iop])).sum()
    tot.backward()
    assert numpy.allclose(a1, hh.grad.numpy(), rtol=1e-13, atol=1e-13)
    assert numpy.allclose(a2, gg.grad.numpy(), rtol=1e-13, atol=1e-13)

    def energy(hv, ev):
        j1, j2 = pint.spin_orbital(hv, ev)
        return sum(float((pm.hp_spatial_site(m.opers[iop], m.sbas, j, j1[m.pidx], j2[m.pidx], None, m.pdic)
                          * grads[j][iop]).sum())
                   for j in range(K) for iop in range(m.nops) if grads[j][iop] is not None)
    dh = rng.standard_normal(h.shape)
    dh = dh + dh.T
    de = rng.standard_normal(eri.shape)
    de = de + de.transpose(1, 0, 2, 3)
    de = de + de.transpose(0, 1, 3, 2)
    de = de + de.transpose(2, 3, 0, 1)
    change = energy(h + dh, eri + de) - energy(h, eri)
    assert abs(change - float((a1 * dh).sum() + (a2 * de).sum())) <= 1e-12 * abs(change)


def test_plan_caches_are_released_with_their_driver():
    """Cached sigma / renorm plans hold device task lists: they are released
    when the driver that owns the cache is collected."""
    import gc
    from zmpo_dmrg_gb300.mpo_dmrg_kernel import _plan_cache

    class Driver:
        pass

    class Plan:
        released = 0

        def release(self):
            Plan.released += 1

    d = Driver()
    cache = _plan_cache(d, "_sigma_cache")
    assert _plan_cache(d, "_sigma_cache") is cache
    cache["a"] = Plan()
    cache["b"] = Plan()
    del d
    gc.collect()
    assert Plan.released == 2 and not cache


@pytest.mark.parametrize("status", ["L", "R"])
@pytest.mark.parametrize("case", [dict(K=6, nelec=6, D=16, isite=2, seed=1),
                                  dict(K=8, nelec=8, D=32, isite=3, seed=4)])
def test_renorm_task_lists_compute_the_oracle_environments(status, case):
    """The engine's renormalisation plan (site . env, W . T1, T2 . site per
    term, the reference's chain of renormQt_H00) executed from its task
    records by the NumPy model of the kernels equals the oracle's new
    environments (FP64, 1e-12 of each term's largest element): checks the
    planner's addressing of every step on the CPU."""
    from tests.problems import random_problem, host_renorm, oracle_renorm
    P = random_problem(device=False, **case)
    got, groups = host_renorm(P, status)
    ref = oracle_renorm(P, status)
    n = 0
    for g, r in zip(got, ref):
        assert g.size == r.size
        if r.size:
            n += 1
            assert numpy.abs(g - r).max() <= 1e-12 * max(numpy.abs(r).max(), 1.0)
    assert n > 10


@pytest.mark.parametrize("isite", [0, 3, 6])
def test_sigma_task_records_cover_every_output_and_read_only_written_blocks(isite):
    """Sigma plans of the left-boundary, a middle and the right-boundary dot
    (K=8, D=32) executed from their task records with the output and the
    workspace filled with NaN: every element of H.psi is written, no step
    reads an intermediate block that no task wrote, and the result equals
    the oracle's HVecQt."""
    from tests.problems import random_problem, host_sigma_terms, oracle_sigma
    P = random_problem(K=8, nelec=8, D=32, isite=isite, seed=3, device=False)
    x = numpy.random.default_rng(1).standard_normal(P.ndim0)
    y, _ = host_sigma_terms(P, range(P.o.nops), x, fill=numpy.nan)
    assert not numpy.isnan(y).any()
    ref = oracle_sigma(P, x)
    assert numpy.linalg.norm(y - ref) <= 1e-12 * numpy.linalg.norm(ref)


@pytest.mark.parametrize("status,isite", [("L", 0), ("L", 3), ("R", 3), ("R", 6)])
def test_renorm_task_records_cover_every_output_and_read_only_written_blocks(status, isite):
    """Renormalisation plans next to both chain ends and in the middle (K=8,
    D=32) with the output and the workspace filled with NaN: every element of
    every new environment is written and no intermediate block is read
    unwritten; the environments equal the oracle's."""
    from tests.problems import random_problem, host_renorm, oracle_renorm
    P = random_problem(K=8, nelec=8, D=32, isite=isite, seed=3, device=False)
    got, _ = host_renorm(P, status, fill=numpy.nan)
    ref = oracle_renorm(P, status)
    n = 0
    for g, r in zip(got, ref):
        assert g.size == r.size and not numpy.isnan(g).any()
        if r.size:
            n += 1
            assert numpy.abs(g - r).max() <= 1e-12 * max(numpy.abs(r).max(), 1.0)
    assert n > 10


def test_threaded_planner_is_deterministic():
    """The planner builds class chains, steps and step parts on host threads:
    two builds of the same sigma plan and of the same renormalisation plan
    give identical task records, step by step."""
    from tests.problems import random_problem, host_sigma_terms, host_renorm
    P = random_problem(K=10, nelec=10, D=64, isite=4, seed=7, device=False)
    x = numpy.random.default_rng(2).standard_normal(P.ndim0)
    y1, g1 = host_sigma_terms(P, range(P.o.nops), x)
    y2, g2 = host_sigma_terms(P, range(P.o.nops), x)
    assert len(g1) == len(g2) and all(numpy.array_equal(a, b) for a, b in zip(g1, g2))
    assert numpy.array_equal(y1, y2)
    e1, r1 = host_renorm(P, "L")
    e2, r2 = host_renorm(P, "L")
    assert all(numpy.array_equal(a, b) for a, b in zip(r1, r2))
    assert all(numpy.array_equal(a, b) for a, b in zip(e1, e2))


def test_adjoint_left_environment_schedule():
    """Recompute mode of the energy gradient: taking the sites from right to
    left, every site finds its left environment held (a checkpoint or
    recomputed in the segment above the nearest checkpoint), at most about
    2 sqrt(nsite) environments are held at once, and each left environment
    is recomputed at most once."""
    from zmpo_dmrg_gb300.adjoint import left_env_schedule, checkpoint_stride
    for nsite in range(1, 49):
        stride = checkpoint_stride(nsite)
        assert stride * stride >= nsite and (stride - 1) ** 2 < nsite
        checkpoints = {-1} | set(range(stride - 1, nsite, stride))
        sched = left_env_schedule(nsite, stride)
        assert len(sched) == nsite
        recomputed = []
        for (seg, held), j in zip(sched, range(nsite - 1, -1, -1)):
            assert j - 1 in held
            if seg is not None:
                assert seg - 1 in checkpoints and seg - 1 in held
                recomputed += list(range(seg, j))
            assert set(held) <= checkpoints | set(recomputed)
            assert len(held) <= 2 * stride + 1
        assert len(recomputed) == len(set(recomputed)) and len(recomputed) < nsite


def test_bench_section_records_a_failure():
    """A benchmark section that raises is recorded in the result line as an
    error entry instead of stopping the run."""
    import bench

    def boom():
        raise RuntimeError("Davidson: subspace H not symmetric")

    assert bench.section("ok", lambda: {"s": 1.0}) == {"s": 1.0}
    rec = bench.section("sweep", boom)
    assert rec == {"error": "RuntimeError: Davidson: subspace H not symmetric"}


def test_buffer_check_names_the_changed_buffer():
    """The driver's debug integrity check (dmrg.check_buffers) records the
    checksums of the MPO buffer and of every stored environment set, accepts
    them unchanged and new sets as they appear, and names the buffer that
    changed."""
    import torch
    from types import SimpleNamespace
    from zmpo_dmrg_gb300.mpo_dmrg_class import check_buffers
    from zmpo_dmrg_gb300.mpo_dmrg_kernel import EnvSet
    rng = numpy.random.default_rng(0)

    def env(n):
        return EnvSet(torch.from_numpy(rng.standard_normal(n)), numpy.zeros(1, dtype=numpy.int64),
                      numpy.zeros(1, dtype=numpy.int64), [None])

    d = SimpleNamespace(mpo_store=SimpleNamespace(buf=torch.from_numpy(rng.standard_normal(50))),
                        envs={('lop', 0): env(10), ('rop', 5): env(1)})
    check_buffers(d, "at the start")
    check_buffers(d, "unchanged")
    d.envs[('lop', 1)] = env(7)          # a new set is recorded, not an error
    check_buffers(d, "after a renormalisation")
    d.envs[('rop', 5)].buf[0] += 1.0
    with pytest.raises(RuntimeError, match="environment rop 5 changed before dot 3"):
        check_buffers(d, "before dot 3")
    d2 = SimpleNamespace(mpo_store=SimpleNamespace(buf=torch.ones(4, dtype=torch.float64)), envs={})
    check_buffers(d2, "first")
    d2.mpo_store.buf[3] = 2.0
    with pytest.raises(RuntimeError, match="MPO buffer changed"):
        check_buffers(d2, "second")


def test_adjoint_recompute_choice_follows_memory():
    """Without an explicit choice the energy gradient recomputes its
    environments when one more full set (the size of the sets the driver
    holds) would take more than half of the free device memory."""
    from types import SimpleNamespace
    import torch
    from zmpo_dmrg_gb300.adjoint import needs_recompute, _held_env_bytes
    assert not needs_recompute(10 * 2 ** 30, 200 * 2 ** 30)
    assert needs_recompute(120 * 2 ** 30, 200 * 2 ** 30)
    d = SimpleNamespace(envs={('lop', 0): SimpleNamespace(buf=torch.zeros(1000, dtype=torch.float64)),
                              ('rop', 3): SimpleNamespace(buf=torch.zeros(24, dtype=torch.float64)),
                              ('lop', 1): None})
    assert _held_env_bytes(d) == 8 * 1024
