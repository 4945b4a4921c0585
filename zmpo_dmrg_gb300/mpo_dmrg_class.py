"""DMRG driver object with the reference's API, running the hot path on the GPU.

Interface of ``source/mpo_dmrg_class.py`` (``mpo_dmrg``: attributes 47-192,
``partition`` 206, ``loadInts`` 249, ``dumpMPO`` 254, ``build`` 279,
``initStates`` 299, ``default`` 329, ``checkMPS`` 470) together with the sweep
of ``mpo_dmrg_opt.py`` (``sweep`` 31, ``checkOpers`` 153, ``updateSite`` 313,
``updateBoundary`` 347), the local solver of ``mpo_dmrg_dot.ci_solver`` 24 and
the decimation / guess of ``mpo_dmrg_dotutil.py`` (288-559).

GB300 design: the MPO, every environment L_p / R_p of every operator term and
the Davidson basis live in device memory (no files, no MPI); H.psi, diag(H) and
the renormalisation are engine launches over all terms at once; the density
matrix decimation and the guess run on the host (they are O(D^3) once per
site).  Storage is always block-sparse (the reference's "Qt" form).
Engine options on the object: ``precision`` ('fp64', 'split' or 'emu64') for
the sigma vector, ``precision_renorm`` for the environments.
"""
import copy
import time

import numpy

from . import mpo as _mpo
from . import parallel
from . import pdvdson
from . import pgdvdson
from . import prdm
from . import spinproj
from .mpo_dmrg_kernel import EnvSet, MPOStore, HVec, HDiag, SVec, renorm, _sigma_plan
from .qtensor import qtensor, fromQnums


def _torch():
    import torch
    return torch


def vacuum(isym=2):
    return [[0.]] if isym == 1 else [[0., 0.]]


def dpt(q1, q2):
    """Labels of a direct product, first index slowest (mpo_dmrg_qphys.dpt)."""
    a = numpy.asarray(q1, dtype=float)
    b = numpy.asarray(q2, dtype=float)
    return (a[:, None, :] + b[None, :, :]).reshape(-1, a.shape[1])


def init_spatial_orb(norb, isym=2):
    q = numpy.array([[0., 0.], [1., -0.5], [1., 0.5], [2., 0.]])
    if isym == 1:
        q = q[:, :1]
    return [q.copy() for _ in range(norb)]


def dense_sector(qlst, key):
    """Ascending dense indices of the elements of the tensor with legs
    ``qlst`` whose labels add up to ``key``."""
    qs = [numpy.asarray(q, dtype=float) for q in qlst]
    nq = qs[0].shape[1]
    tot = numpy.zeros([len(q) for q in qs] + [nq])
    for i, q in enumerate(qs):
        shape = [1] * len(qs) + [nq]
        shape[i] = len(q)
        tot = tot + q.reshape(shape)
    tot = tot.reshape(-1, nq)
    k = numpy.asarray(key, dtype=float).reshape(-1)[:nq]
    return numpy.flatnonzero(numpy.abs(tot - k).sum(axis=1) < 1e-10)


def check_buffers(dmrg, where):
    """Integrity check for debugging (``dmrg.check_buffers = True``, off by
    default): the MPO buffer and every stored environment set must keep the
    checksums (sum and sum of squares) they had when first seen; an
    environment set replaced by a new one is checked from then on.  Raises
    RuntimeError naming the first buffer that changed and ``where``.  Each
    check reads every stored environment once (a device reduction)."""
    torch = _torch()
    seen = dmrg.__dict__.setdefault("_buffer_sums", {})

    def sums(t):
        t = t.reshape(-1)
        return (float(t.sum()), float(torch.dot(t, t)))

    items = [("MPO buffer", "mpo", dmrg.mpo_store.buf)]
    for key in sorted(dmrg.envs, key=lambda k: (k[0], k[1])):
        env = dmrg.envs[key]
        if env is not None:
            items.append(("environment %s %d" % key, ("env", env.uid), env.buf))
    live = set()
    for name, tag, buf in items:
        live.add(tag)
        cur = sums(buf)
        old = seen.get(tag)
        if old is None:
            seen[tag] = cur
        elif old != cur:
            raise RuntimeError("buffer check: %s changed %s (sum %r -> %r, squares %r -> %r)"
                               % (name, where, old[0], cur[0], old[1], cur[1]))
    for tag in [t for t in seen if t not in live]:
        del seen[tag]


def rdm_blkdiag(rho0, classes, thresh, Dcut=-1):
    """Block eigen-decomposition of the reduced density matrix by sector and
    truncation (mpo_dmrg_qparser.rdm_blkdiag, mpo_dmrg_qparser.py:106-183)."""
    import scipy.linalg
    cls = numpy.asarray(classes, dtype=float)
    keys, first, inv = numpy.unique(cls, axis=0, return_index=True, return_inverse=True)
    inv = inv.reshape(-1)
    order = numpy.argsort(first, kind="stable")
    nrows = rho0.shape[0]
    qsymL, cols, sigs = [], [], []
    for k in order:
        rows = numpy.flatnonzero(inv == k)
        s2, u = scipy.linalg.eigh(rho0[numpy.ix_(rows, rows)])
        s2 = numpy.abs(s2)
        ucol = numpy.zeros((nrows, len(rows)))
        ucol[rows, :] = u
        cols.append(ucol)
        sigs.append(s2)
        qsymL += [list(keys[k])] * len(rows)
    rotL = numpy.hstack(cols)
    sigs = numpy.hstack(sigs)
    sigs = sigs / numpy.sum(sigs)
    indx = numpy.argsort(sigs, kind="stable")[::-1]
    nres = len(sigs)
    ts = sigs[indx]
    below = numpy.flatnonzero(ts < thresh * 1.01)
    if below.size:
        nres = int(below[0])
    nres = max(nres, 1)
    if Dcut > 0:
        nres = min(nres, Dcut)
    indx = indx[:nres]
    sigs = sigs[indx]
    dwts = 1.0 - numpy.sum(sigs)
    qsymL = [qsymL[i] for i in indx]
    rotL = rotL[:, indx]
    o = sorted(range(nres), key=lambda x: qsymL[x])
    return dwts, numpy.array([qsymL[i] for i in o]), rotL[:, o].copy(), sigs[o].copy()


class mpo_dmrg:
    def __init__(self, seed=0):
        self.iprt = 0
        self.nsite = None
        self.sbas = None
        self.occun = None
        self.crit_vec = 1.e-8
        self.thresh = -1.e-14
        self.ifdvdnz = True
        self.Dcut = None
        self.Dmax = None
        self.crit_e = 1.e-10
        self.noise = 1.e-4
        self.inoise = 0
        self.ifprecond = True
        self.ifguess = True
        self.psi0 = None
        self.ncsite = None
        self.status = None
        self.isym = 2
        self.qphys = None
        self.dphys = None
        self.qnuml = None
        self.qnumr = None
        self.nelec = 0.0
        self.sz = 0.0
        self.neig = None
        self.wts = None
        self.qsectors = None
        self.const = 0.0
        self.ifs2proj = False
        self.npts = None
        self.qwts = None
        self.qpts = None
        self.opers = []
        self.nops = None
        self.ifQt = True
        # first MPS from occun when default() gets none (mpo_dmrg_class.py:113-115)
        self.initNsweep = 0
        self.initNcsite = 1
        # this driver keeps Davidson vectors and diagonals on the device
        self.device_vectors = True
        self.qkey = None
        self.qlst = None
        self.qtmp = None
        self.idlstCI = None
        self.maxslc = 1
        self.int1e = None
        self.int2e = None
        self.hpwts = None
        # engine options: precision of H.psi inside Davidson, of the final
        # Rayleigh quotient of each converged vector, and of the renormalisation
        self.precision = "fp64"
        self.precision_final = "emu64"
        self.precision_renorm = "fp64"
        # replay each site's H.psi launches from a CUDA graph
        self.use_graph = False
        self.rng = numpy.random.default_rng(seed)
        # operator-term partition over ranks (partition())
        self.rank, self.size, self.group = 0, 1, None
        # device state
        self.mpo_store = None
        self.pop_store = None
        self.exppop = None
        self.envs = {}
        self.flmps = {}
        self.frmps = {}
        self.nmvp = []
        self.eav = []
        self.dwt = []
        self.esweeps = []
        self.timings = []
        # seconds per phase of the sweep, summed over dots, when set to a
        # dict (each phase boundary then synchronises the device)
        self.phase_times = None
        self._phase_t0 = 0.0

    def tick(self, name):
        """Adds the seconds since the previous tick to phase ``name`` of
        ``phase_times`` (no-op unless ``phase_times`` is a dict)."""
        pt = self.phase_times
        if pt is None:
            return
        _torch().cuda.synchronize()
        t = time.perf_counter()
        if name is not None:
            pt[name] = pt.get(name, 0.0) + t - self._phase_t0
        self._phase_t0 = t

    # ------------------------------------------------------------ set-up
    def build(self):
        if self.nsite < 2:
            raise ValueError('mps is not supported for nsite < 2')
        assert self.isym in (1, 2)
        self.qphys = init_spatial_orb(self.nsite, self.isym)
        self.dphys = [len(x) for x in self.qphys]
        self.qnuml = [None] * (self.nsite + 1)
        self.qnuml[0] = numpy.array(vacuum(self.isym))
        self.qnumr = [None] * (self.nsite + 1)
        self.qnumr[-1] = numpy.array(vacuum(self.isym))
        return 0

    def s2quad(self, sval=0, sz=0):
        from .spinproj import s2quad
        s2quad(self, sval, sz)
        return 0

    def partition(self, rank=None, size=None, group=None):
        """This rank's operator terms H_p (mpo_dmrg_class.partition, 206-246;
        tools/parallel_util.partitionSites): a contiguous block of the 2K
        terms (npts * 2K with spin projection) per rank.  ``rank`` / ``size``
        default to the torch.distributed process group (one rank without it).
        With several ranks every sum over terms (H.psi, its diagonal, the
        noise density matrix, the energy of an MPS) is summed over the ranks;
        the Davidson subspace and the decimation are replicated."""
        if self.sbas is None:
            raise ValueError('sbas is not defined')
        if rank is None or size is None:
            rank, size = parallel.world(group)
        self.rank, self.size, self.group = rank, size, group
        self.opers = parallel.partition_ops(self.sbas, size, rank, self.npts)
        if self.npts is None:
            self.hpwts = numpy.ones(len(self.opers))
        else:
            self.hpwts = numpy.array([self.qwts[x[1]] for x in self.opers])
        self.nops = len(self.opers)
        self.pidx = sorted(set(x[0] for x in self.opers))
        self.pdic = dict((p, i) for i, p in enumerate(self.pidx))
        return 0

    def loadInts(self, mol):
        """``mol`` carries spin-orbital ``int1e`` [p,q] and ``int2e`` [p,q,r,s]
        = V_pqrs (the arrays the reference reads from mole.h5), or is the pair."""
        if isinstance(mol, (tuple, list)):
            int1e, int2e = mol
        else:
            int1e, int2e = mol.int1e, mol.int2e
        self.int1e = numpy.asarray(int1e)[self.pidx]
        self.int2e = numpy.asarray(int2e)[self.pidx]
        return 0

    def dumpMPO(self):
        """Build every W_p(i) in block-sparse form and upload them at once."""
        torch = _torch()
        tens = [[None] * self.nops for _ in range(self.nsite)]
        off = numpy.zeros((self.nsite, self.nops), dtype=numpy.int64)
        vals = []
        pos = 0
        for isite in range(self.nsite):
            for iop in range(self.nops):
                t = _mpo.hp_spatial_qt(self.opers[iop], self.sbas, isite, self.int1e, self.int2e,
                                       self.qpts, self.pdic)
                tens[isite][iop] = t
                off[isite, iop] = pos
                vals.append(t.value)
                pos += t.size_allowed
        buf = torch.from_numpy(numpy.concatenate(vals)).cuda()
        self.mpo_store = MPOStore(buf, off, tens)
        if self.ifs2proj:
            spinproj.dumpMPO_R(self)
        return 0

    def initStates(self):
        if self.qsectors is None:
            if self.neig is None:
                raise ValueError('no state is specified')
            key = str([self.nelec]) if self.isym == 1 else str([self.nelec, self.sz])
            self.qsectors = {key: self.neig}
        self.neig = sum(self.qsectors.values())
        if self.wts is None:
            self.wts = numpy.ones(self.neig) / float(self.neig)
        return 0

    # ------------------------------------------------------- environments
    def boundary_env(self):
        """Environment of the empty block: 1 for every term
        (mpo_dmrg_initQt.genBopsQt, mpo_dmrg_initQt.py:49-85)."""
        torch = _torch()
        q = [[0.]] if (self.isym == 1 or self.ifs2proj) else [[0., 0.]]
        t = qtensor([True, False, True])
        t.fromQsyms(3, [q, q, q], [[1], [1], [1]], ifallocate=False)
        buf = torch.ones(self.nops, dtype=torch.float64, device="cuda")
        return EnvSet(buf, numpy.arange(self.nops, dtype=numpy.int64),
                      numpy.full(self.nops, t.layout, dtype=numpy.int64), [t] * self.nops)

    def site_qt(self, isite, dense, qnums, status):
        t = qtensor(status)
        t.fromDenseTensor(dense, qnums)
        return t

    def product_mps(self):
        """Left-canonical product state from ``occun`` (mpo_dmrg_util.mps0occun,
        mpo_dmrg_util.py:118-155) in block-sparse form."""
        nsite = self.nsite
        fmps = {'nsite': nsite}
        qn = [numpy.array([[0., 0.]])]
        ne, ms = 0.0, 0.0
        for i in range(nsite):
            na, nb = self.occun[2 * i], self.occun[2 * i + 1]
            idx = int(round(na)) * 2 + int(round(nb))
            ne += round(na) + round(nb)
            ms += 0.5 * (round(na) - round(nb))
            site = numpy.zeros((1, 4, 1))
            site[0, idx, 0] = 1.0
            qn.append(numpy.array([[ne, ms]]))
            fmps['site%d' % i] = self.site_qt(i, site, [qn[i], self.qphys[i], qn[i + 1]],
                                              [False, False, True])
        for i in range(nsite + 1):
            fmps['qnum%d' % i] = qn[i]
        return fmps

    def product_mps_right(self):
        """The same occupation-number product state as right-canonical sites
        [l, n, r] (status [T, F, F]) with the reference's right labels
        qnumr[i] = (N - N_left(i), Sz - Sz_left(i)) (mps0occun, 118-155)."""
        left = self.product_mps()
        qn = [numpy.asarray(left['qnum%d' % i], dtype=float) for i in range(self.nsite + 1)]
        tot = qn[-1]
        qr = [tot - q for q in qn]
        fmps = {'nsite': self.nsite}
        for i in range(self.nsite):
            d = numpy.asarray(left['site%d' % i].toDenseTensor(left['site%d' % i].idlst))
            fmps['site%d' % i] = self.site_qt(i, d, [qr[i], self.qphys[i], qr[i + 1]], [True, False, False])
        return qn, qr, fmps

    def initMPS(self):
        """Initial MPS when no MPS is given (mpo_dmrg_util.initMPS, 158-190):
        the occupation-number product state, its right environments, then one
        left sweep of ``initNcsite``-site dots under the first schedule entry
        (the perturbed density matrix grows the bond dimension), plus
        ``initNsweep`` further sweep pairs."""
        qn, qr, fmps0 = self.product_mps_right()
        self.qnuml = [q.copy() for q in qn]
        self.qnumr = [q.copy() for q in qr]
        self.envs[('lop', -1)] = self.boundary_env()
        if self.ifs2proj:
            self.envs[('lpop', -1)] = spinproj.boundary_pops(self)
        self.genHops(fmps0, 'rop')
        sitelst = list(range(self.nsite))
        self.sweep(sitelst, self.initNcsite, 'L')
        for _ in range(self.initNsweep):
            self.sweep(sitelst, self.initNcsite, 'R')
            self.sweep(sitelst, self.initNcsite, 'L')
        return 0

    def _flst(self, lsite, rsite):
        """Environments of a dot: [L, R] or, spin-projected, [L, R, L_P, R_P]."""
        f = [self.envs.get(('lop', lsite)), self.envs.get(('rop', rsite))]
        if self.ifs2proj:
            f += [self.envs.get(('lpop', lsite)), self.envs.get(('rpop', rsite))]
        return [f]

    def _store_envs(self, kind, isite, fN):
        self.envs[(kind, isite)] = fN[0][0]
        if self.ifs2proj:
            self.envs[(kind[0] + 'pop', isite)] = fN[0][1]

    @staticmethod
    def _scalars(env, n):
        vals = env.buf.cpu().numpy()
        out = numpy.zeros(n)
        for iop in range(n):
            if env.off[iop] >= 0:
                out[iop] = vals[env.off[iop]]
        return out

    def genHops(self, fmps, kind='lop'):
        """All left (or right) environments of an MPS and <H_p> at the end
        (with spin projection also the P_g environments and <P_g>)."""
        nsite = self.nsite
        if kind == 'lop':
            bnd, order = -1, range(nsite)
        else:
            bnd, order = nsite, range(nsite - 1, -1, -1)
        self.envs[(kind, bnd)] = self.boundary_env()
        if self.ifs2proj:
            self.envs[(kind[0] + 'pop', bnd)] = spinproj.boundary_pops(self)
        for isite in order:
            site = fmps['site%d' % isite]
            if kind == 'lop':
                flst = self._flst(isite - 1, None)
            else:
                flst = self._flst(None, isite + 1)
            fN = [[None, None]]
            renorm(self, isite, 1, flst, fN, site, 'L' if kind == 'lop' else 'R')
            self._store_envs(kind, isite, fN)
        iend = nsite - 1 if kind == 'lop' else 0
        exphop = self._scalars(self.envs[(kind, iend)], self.nops)
        self.exppop = None
        if self.ifs2proj:
            self.exppop = self._scalars(self.envs[(kind[0] + 'pop', iend)], self.npts)
        return exphop

    def initOps(self, fmps):
        self.envs[('rop', self.nsite)] = self.boundary_env()
        if self.ifs2proj:
            self.envs[('rpop', self.nsite)] = spinproj.boundary_pops(self)
        self.genHops(fmps, 'lop')
        return 0

    def checkMPS(self, fbra=None):
        """Energy sum_p w_p <H_p> (over sum_g w_g <P_g> with spin projection)
        of the left-canonical MPS (checkMPS 470-558): (energy, <H(P)>, ovlp, <P>)."""
        fmps = self.flmps if fbra is None else fbra
        exphop = self.genHops(fmps, 'lop')
        esum = float(numpy.dot(self.hpwts, exphop))
        if getattr(self, "size", 1) > 1:
            t = _torch().tensor([esum], dtype=_torch().float64)
            esum = float(parallel.allreduce_(t, self.group)[0])
        if self.ifs2proj:
            psum = float(numpy.dot(self.qwts, self.exppop))
            return esum / psum, esum, 1.0, psum
        return esum, esum, 1.0, None

    # ----------------------------------------------------------- local solver
    def _qlst(self, isite, ncsite):
        q = [numpy.asarray(self.qnuml[isite]), self.qphys[isite]]
        if ncsite == 2:
            q.append(self.qphys[isite + 1])
        q.append(numpy.asarray(self.qnumr[isite + ncsite]))
        return q

    def setupQtmpCI(self, ncsite, key):
        self.qkey = numpy.array(key, dtype=float)
        qn = list(self.qlst[:-1]) + [self.qkey - self.qlst[-1]]
        self.qtmp = qtensor([False] * (len(qn) - 1) + [True])
        rank, qsyms, ndims, idlst = fromQnums(qn)
        self.qtmp.fromQsyms(rank, qsyms, ndims, ifallocate=False)
        self.idlstCI = idlst
        self.qtmp_psi_layout = self.qtmp.layout
        return 0

    def ci_solver(self, isite, ncsite, actlst, flst, status, ifsym=True):
        torch = _torch()
        cdim = self.dphys[isite] * (self.dphys[isite + 1] if ncsite == 2 else 1)
        ldim = len(self.qnuml[isite])
        rdim = len(self.qnumr[isite + ncsite])
        ndim = ldim * cdim * rdim
        self.dims = (ldim, cdim, rdim, ndim)
        self.qlst = self._qlst(isite, ncsite)
        info = [self, isite, ncsite, flst, status, ifsym]
        ioff = 0
        eigs, civecs = [], []
        nmvps = 0
        for qkey in self.qsectors:
            neig = self.qsectors[qkey]
            key = [float(x) for x in eval(qkey)]
            self.setupQtmpCI(ncsite, key)
            if self.ifQt:
                prjmap = self.qtmp.prjmap(self.idlstCI)
                ndim0 = self.qtmp.size_allowed
            else:
                # the reference's dense ("NQt") basis of the sector: every
                # element of the (ldim, c, rdim) tensor with the target label,
                # ascending (mpo_dmrg_dotutil.dptSymmetry, 102-145); vectors in
                # this order, the engine gathers them into its block order
                prjmap = dense_sector(self.qlst, self.qkey)
                ndim0 = prjmap.size
            if ndim0 == 0:
                raise RuntimeError('no basis in symmetry sector %s' % qkey)
            self.tick("setup")
            if self.phase_times is not None:
                _sigma_plan(info)
                self.tick("sigma_plan")
            if self.ifprecond:
                diag = HDiag(info, ndim0, prjmap)
                if getattr(self, "size", 1) > 1:
                    parallel.allreduce_(diag, self.group)
            else:
                diag = torch.ones(ndim0, dtype=torch.float64, device="cuda")
            # H.psi over this rank's terms, summed over the ranks
            hvec = parallel.DistributedHVec(HVec, self.group) if getattr(self, "size", 1) > 1 else HVec
            if not self.ifs2proj:
                solver = pdvdson.eigenSolver(self.rng)
                solver.HVec = pdvdson.mask([info, ndim0, prjmap], hvec).matvec
            else:
                solver = pgdvdson.eigenSolver(self.rng)
                solver.HVec = pgdvdson.mask([info, ndim0, prjmap], hvec).matvec
                solver.SVec = pgdvdson.mask([info, ndim0, prjmap], SVec).matvec
            solver.crit_e = self.crit_e
            solver.crit_vec = self.crit_vec
            solver.ndim = ndim0
            solver.neig = neig
            solver.diag = diag
            solver.noise = self.ifdvdnz and (self.noise > 1.e-10)
            solver.hvec_eps = {"fp64": 0.0, "emu64": 1e-14, "split": 1e-8}[self.precision]
            self.tick("hdiag")
            v0 = None
            if self.psi0 is not None:
                idx = torch.as_tensor(numpy.asarray(prjmap, dtype=numpy.int64), device=self.psi0.device)
                v0 = self.psi0[ioff:ioff + neig].index_select(1, idx)
            eig, vec, nmvp = solver.solve_iter(v0=v0, iop=4)
            self.tick("davidson")
            if self.precision == "split":
                # energy error is second order in the vector error: one
                # Rayleigh quotient per vector with the 56-bit product
                saved = self.precision
                self.precision = self.precision_final
                for i in range(neig):
                    v = vec[i].contiguous()
                    hv = hvec(v, info, ndim0, prjmap)
                    sv = SVec(v, info, ndim0, prjmap) if self.ifs2proj else v
                    eig[i] = float(torch.dot(v, hv) / torch.dot(v, sv))
                self.precision = saved
                self.tick("rayleigh")
            civec = torch.zeros((neig, ndim), dtype=torch.float64, device="cuda")
            civec[:, torch.as_tensor(numpy.asarray(prjmap, dtype=numpy.int64), device="cuda")] = vec
            civecs.append(civec)
            eigs += list(eig)
            nmvps += nmvp
            ioff += neig
        civecs = torch.cat(civecs, dim=0)
        eigs = numpy.array(eigs)
        self.tick("setup")
        sigs, dwts, qred, site, srotR = self.decimation(civecs, info)
        self.tick("decimation")
        if self.ifguess:
            self.genGuess(isite, ncsite, actlst, civecs, srotR, status)
            self.tick("guess")
        return nmvps, eigs, sigs, dwts, qred, site, srotR

    def decimation(self, civecs, info):
        """Reduced density matrix (with the perturbation noise), its block
        eigen-decomposition and truncation, the new site and the rotated
        wavefunction (mpo_dmrg_dotutil.decimation, 259-345).  ``civecs``
        (neig, ndim) live on the device; the dense products (rho = C C^T and
        the rotation of C) run there, the block eigen-decomposition of rho on
        the host (it decides which states are kept, with LAPACK as in the
        reference)."""
        torch = _torch()
        dmrg, isite, ncsite, flst, status, ifsym = info
        ldim, cdim, rdim, ndim = self.dims
        neig = civecs.shape[0]
        if status == 'L':
            dim = self.dphys[isite]
            cdimc = cdim // dim
            lcdim, crdim = ldim * dim, cdimc * rdim
        else:
            jsite = isite + ncsite - 1
            dim = self.dphys[jsite]
            cdimc = cdim // dim
            lcdim, crdim = ldim * cdimc, dim * rdim
        if self.noise >= 1.e-10 and self.inoise == 1:
            nz = self.rng.uniform(-1, 1, size=tuple(civecs.shape)) * 10.0 * self.noise
            civecs = civecs + torch.as_tensor(nz, device=civecs.device)
        mats = civecs.reshape(neig, lcdim, crdim)
        if status == 'L':
            shaped = civecs.reshape(neig, ldim, dim, crdim)
        else:
            shaped = civecs.reshape(neig, lcdim, dim, rdim)
        rdm1 = prdm.pRDM(shaped, info)
        tr = float(torch.trace(rdm1))
        if tr < -1e-12:
            raise RuntimeError('RDM should be positive definite')
        if tr < 1e-12:
            rdm1 = rdm1 + torch.eye(rdm1.shape[0], dtype=rdm1.dtype, device=rdm1.device) / rdm1.shape[0]
        else:
            rdm1 = rdm1 / tr
        rdm1 = rdm1.cpu().numpy()
        Dcut = self.Dmax
        if ncsite == 1 and ((status == 'L' and isite == self.nsite - 1) or (status == 'R' and isite == 0)):
            Dcut = 1
        if status == 'L':
            if self.Dcut is not None:
                Dcut = self.Dcut[isite + 1]
            classes = dpt(self.qnuml[isite], self.qphys[isite])
            dwts, qred, rotL, sigs = rdm_blkdiag(rdm1, classes, self.thresh, Dcut)
            nres = len(qred)
            site = rotL.reshape(ldim, dim, nres).copy()
            rot = torch.from_numpy(numpy.ascontiguousarray(rotL)).cuda()
            srotR = torch.matmul(rot.T, mats).reshape(neig, nres, cdimc, rdim)
        else:
            jsite = isite + ncsite - 1
            if self.Dcut is not None:
                Dcut = self.Dcut[jsite]
            classes = dpt(self.qphys[jsite], self.qnumr[jsite + 1])
            dwts, qred, rotL, sigs = rdm_blkdiag(rdm1, classes, self.thresh, Dcut)
            nres = len(qred)
            site = rotL.reshape(dim, rdim, nres).transpose(2, 0, 1).copy()
            rot = torch.from_numpy(numpy.ascontiguousarray(rotL)).cuda()
            srotR = torch.matmul(mats, rot).reshape(neig, ldim, cdimc, nres)
        return sigs, dwts, qred, site, srotR

    def genGuess(self, isite, ncsite, actlst, civecs, srotR, status):
        """Guess for the next dot (mpo_dmrg_dotutil.guess, 498-559): the
        rotated wavefunction times the neighbouring site, on the device."""
        torch = _torch()
        if isite == actlst[-1]:
            self.psi0 = civecs.clone()
            return 0
        if status == 'R':
            t = self.flmps.get('site%d' % (isite - 1))
            if t is not None:
                d = torch.from_numpy(t.toDenseTensor(t.idlst)).cuda()
                self.psi0 = torch.stack([torch.tensordot(d, srotR[e], dims=([2], [0])).reshape(-1)
                                         for e in range(self.neig)])
        else:
            t = self.frmps.get('site%d' % (isite + ncsite))
            if t is not None:
                d = torch.from_numpy(t.toDenseTensor(t.idlst)).cuda()
                self.psi0 = torch.stack([torch.tensordot(srotR[e], d, dims=([2], [0])).reshape(-1)
                                         for e in range(self.neig)])
        return 0

    # ----------------------------------------------------------------- sweep
    def checkOpers(self, sitelst, ncsite, status):
        if status == 'L':
            return [i - ncsite for i in range(sitelst[0] + ncsite, min(self.nsite, sitelst[-1] + ncsite) + 1)]
        lst = list(range(max(-1, sitelst[0] - ncsite), sitelst[-1] - ncsite + 1))
        return [i + 1 for i in lst[::-1]]

    def updateSite(self, isite, ncsite, qred, site, status):
        if status == 'L':
            self.qnuml[isite + 1] = qred.copy()
            t = self.site_qt(isite, site, [self.qlst[0], self.qlst[1], qred], [False, False, True])
            self.flmps['qnum%d' % (isite + 1)] = qred.copy()
            self.flmps['site%d' % isite] = t
        else:
            jsite = isite + ncsite - 1
            self.qnumr[jsite] = qred.copy()
            t = self.site_qt(jsite, site, [qred, self.qlst[-2], self.qlst[-1]], [True, False, False])
            self.frmps['qnum%d' % jsite] = qred.copy()
            self.frmps['site%d' % jsite] = t
        return t

    def updateBoundary(self, ncsite, sitelst, qred, srotR, status):
        if ncsite != 2:
            return 0
        key = numpy.array([float(x) for x in eval(next(iter(self.qsectors)))])
        s0 = srotR[0].cpu().numpy() if hasattr(srotR, "cpu") else srotR[0]
        smat = s0 / numpy.linalg.norm(s0)
        if status == 'L' and sitelst[-1] == self.nsite - 1:
            self.flmps['qnum%d' % self.nsite] = key[None, :]
            self.flmps['site%d' % (self.nsite - 1)] = self.site_qt(
                self.nsite - 1, smat, [qred, self.qphys[self.nsite - 1], key[None, :]], [False, False, True])
        elif status == 'R' and sitelst[0] == 0:
            self.frmps['qnum0'] = key[None, :]
            self.frmps['site0'] = self.site_qt(0, smat, [key[None, :], self.qphys[0], qred],
                                               [True, False, False])
        return 0

    def sweep(self, sitelst, ncsite, status, ifsym=True):
        torch = _torch()
        actlst = self.checkOpers(sitelst, ncsite, status)
        elst, dlst = [], []
        nmvp = 0
        for isite in actlst:
            if getattr(self, "check_buffers", False):
                check_buffers(self, "before the %s-sweep dot at site %d" % (status, isite))
            t0 = time.perf_counter()
            self.tick(None)
            flst = self._flst(isite - 1, isite + ncsite)
            nmvps, eigs, sigs, dwts, qred, site, srotR = self.ci_solver(isite, ncsite, actlst, flst, status, ifsym)
            t1 = time.perf_counter()
            nmvp += nmvps
            elst.append(eigs)
            dlst.append(dwts)
            self.tick(None)
            siteN = self.updateSite(isite, ncsite, qred, site, status)
            self.tick("site_update")
            fN = [[None, None]]
            renorm(self, isite, ncsite, flst, fN, siteN, status)
            self.tick("renorm")
            if status == 'L':
                self._store_envs('lop', isite, fN)
            else:
                self._store_envs('rop', isite + ncsite - 1, fN)
            self.tick("store_envs")
            # no device synchronisation here: the renormalisation runs on the
            # GPU while the host sets up the next dot and builds its plans
            self.timings.append((status, isite, t1 - t0, time.perf_counter() - t1, nmvps))
        self.updateBoundary(ncsite, sitelst, qred, srotR, status)
        eavs = numpy.array(elst).dot(self.wts)
        indx = int(numpy.argmin(eavs))
        return nmvp, indx, eavs[indx], dlst[indx], elst, dlst

    def default(self, sc, fmps=None):
        """Standard DMRG following the schedule (mpo_dmrg_class.py:329-434)."""
        self.schedule = sc
        self.crit_tol = sc.tol
        self.initStates()
        self.flmps = {'nsite': self.nsite, 'qnum0': self.qnuml[0]}
        self.frmps = {'nsite': self.nsite, 'qnum%d' % self.nsite: self.qnumr[-1]}
        if fmps is None:
            # the reference builds the first MPS by a sweep under the first
            # schedule entry (mpo_dmrg_class.py:359-367)
            self.status = 'init'
            self.Dmax = sc.MaxMs[0]
            self.crit_e = sc.Tols[0]
            self.noise = sc.Noises[0]
            self.initMPS()
        else:
            self.qnuml = [numpy.asarray(fmps['qnum%d' % i]) for i in range(self.nsite + 1)]
            self.flmps.update(fmps)
            self.initOps(fmps)
        self.psi0 = None
        sitelst = list(range(self.nsite))
        eold, deltaE, ifconv, isweep = 1.e3, 1.e3, False, -1
        for isweep in range(sc.maxiter):
            self.isweep = isweep
            sc.getParameters(self, isweep)
            r1 = self.sweep(sitelst, self.ncsite, 'R')
            r2 = self.sweep(sitelst, self.ncsite, 'L')
            self.nmvp.append(r1[0] + r2[0])
            self.esweeps += r1[4] + r2[4]
            eav, dwt = (r1[2], r1[3]) if r1[2] < r2[2] else (r2[2], r2[3])
            self.eav.append(eav)
            self.dwt.append(dwt)
            self.Energy = eav
            deltaE = eav - eold
            ifconv = sc.checkConv(self, isweep, deltaE)
            eold = eav
            if ifconv:
                break
        self.ifconv = ifconv
        self.nsweep = isweep + 1
        self.deltaE = deltaE
        return 0
