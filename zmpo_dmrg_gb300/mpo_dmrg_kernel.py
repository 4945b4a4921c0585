"""Drop-in replacements for the reference's hot-path kernels, on the GPU.

Same call signatures as ``source/mpo_dmrg_kernel.py``:
  ``HVec(vec0, info, ndim0, prjmap)``   (117-136; Qt body HVecQt,
                                         mpo_dmrg_kernelQt.py:153-319)
  ``HDiag(info, ndim0, prjmap)``         (41-51; HDiagQt 30-127)
  ``renorm(dmrg, isite, ncsite, flst, flstN, site, status)`` (347-377;
                                         renormQt_H00 633-768)
with ``info = [dmrg, isite, ncsite, flst, status, ifsym]``.  ``flst[0][0:2]``
are the left / right environment sets (``EnvSet``: one device buffer holding
L_p or R_p for every operator term, in the reference's packed block order),
``dmrg.qtmp`` is the wavefunction layout and ``dmrg.qkey`` its target label.
Vectors may be NumPy (copied to and from the device) or float64 CUDA tensors
(kept on the device).  Every product runs in the engine; there is no host
fallback.

Vector order follows ``dmrg.ifQt`` as in the reference (``HVec`` 121-124,
``HDiag`` 45-48): with ``ifQt`` (the default) a vector is the packed block
order of ``dmrg.qtmp``; with ``ifQt = False`` it is the caller's dense order,
element j at dense index ``prjmap[j]`` of the (ldim, 4, 4, rdim) tensor
(``HVecNQt`` 138-181).  The environments stay block-sparse either way: the
dense-ordered vector is gathered into the packed order on the device and the
result scattered back.  ``HDiag`` returns NumPy (as the reference's
``genHDiag`` expects) unless the driver keeps its vectors on the device
(``dmrg.device_vectors``).  The perturbation-theory variant of the
reference's ``HVec`` (``dmrg.ifpt``: H0 - E0 through ``fdopXfhop``, 118-135)
is not part of this path and raises ``NotImplementedError``.
"""
import collections
import hashlib
import itertools
import weakref

import numpy

from . import engine as _engine
from .qtensor import qtensor

_serial = itertools.count()


class EnvSet:
    """Environments of all operator terms at one bond (replaces the reference's
    per-site HDF5 file ``lop_site_i`` / ``rop_site_i`` with datasets ``opers{p}``)."""

    def __init__(self, buf, off, layouts, tensors):
        self.uid = next(_serial)  # plan caches key on this, never on id()
        self.buf = buf            # torch float64 CUDA tensor
        self.off = off            # [nop] element offsets (-1: absent)
        self.layouts = layouts    # [nop] engine layout ids (-1: absent)
        self.tensors = tensors    # [nop] host qtensor structure (value unset)

    def present(self, iop):
        return self.off[iop] >= 0


class MPOStore:
    """All MPO site tensors on the device (replaces the reference's ``hop`` file)."""

    def __init__(self, buf, off, tensors):
        self.uid = next(_serial)
        self.buf = buf            # torch float64 CUDA tensor
        self.off = off            # off[isite][iop]
        self.tensors = tensors    # tensors[isite][iop] host qtensor


def _torch():
    import torch
    return torch


def _to_device(v):
    torch = _torch()
    if isinstance(v, numpy.ndarray):
        return torch.from_numpy(numpy.ascontiguousarray(v, dtype=numpy.float64)).cuda(), True
    return v.contiguous(), False


def _flip_layout(dmrg, t):
    """Right environment with the reference's label flip (kernelQt.py:301)."""
    qkey = numpy.asarray(dmrg.qkey, dtype=float)
    if dmrg.ifs2proj:
        qkey = qkey[:1]
    key = (t.layout, tuple(qkey.tolist()))
    cache = dmrg.__dict__.setdefault("_flip_cache", {})
    lid = cache.get(key)
    if lid is None:
        lid = _engine.get().derive(t.layout, [-t.qsyms[0], qkey - t.qsyms[1], qkey - t.qsyms[2]],
                                   t.status)
        cache[key] = lid
    return lid


def _shared_workspace(dmrg, nelem):
    """The sigma plans of one driver run one after the other on one stream:
    they share one workspace buffer, grown on demand (cached plans hold none)."""
    torch = _torch()
    buf = dmrg.__dict__.get("_sigma_ws")
    if buf is None or buf.numel() < nelem:
        dmrg._sigma_ws = None
        buf = torch.empty(nelem, dtype=torch.float64, device="cuda")
        dmrg._sigma_ws = buf
    return buf[:nelem]


class SigmaPlan:
    released = False

    def __init__(self, dmrg, isite, ncsite, fL, fR):
        from .mpo import op_class
        self._dmrg = weakref.ref(dmrg)  # the driver owns the shared workspace (no cycle)
        eng = _engine.get()
        mpo = dmrg.mpo_store
        ops = [iop for iop in range(dmrg.nops) if fL.present(iop) and fR.present(iop)]
        classes = {}
        op_cls, lay_L, lay_Wi, lay_Wj, lay_Rf = [], [], [], [], []
        off_L, off_R, off_Wi, off_Wj, wts = [], [], [], [], []
        for iop in ops:
            c0 = op_class(dmrg.opers[iop][0], isite, ncsite)
            if c0 not in classes:
                classes[c0] = len(classes)
                lay_L.append(fL.layouts[iop])
                lay_Wi.append(mpo.tensors[isite][iop].layout)
                lay_Wj.append(mpo.tensors[isite + 1][iop].layout if ncsite == 2 else -1)
                lay_Rf.append(_flip_layout(dmrg, fR.tensors[iop]))
            c = classes[c0]
            op_cls.append(c)
            off_L.append(fL.off[iop])
            off_R.append(fR.off[iop])
            off_Wi.append(mpo.off[isite][iop])
            off_Wj.append(mpo.off[isite + 1][iop] if ncsite == 2 else 0)
            wts.append(dmrg.hpwts[iop])
        self.nops = len(ops)
        if self.nops == 0:
            self.pid = None
            self.pids = []
            return
        torch = _torch()
        lay_psi = dmrg.qtmp_psi_layout
        self.nmap = None
        if dmrg.ifs2proj:
            # psi relabelled by N (reduceQsymsToN): same sectors, more allowed
            # blocks; the result is read back on the (N, Sz) blocks only
            from .spinproj import n_only_map
            qN, idx = n_only_map(dmrg.qtmp)
            lay_psi = qN.layout
            self.nmap = (torch.as_tensor(idx, device="cuda"), qN.size_allowed)
        # the terms' intermediates live in one workspace; with a budget
        # (dmrg.workspace_budget, bytes) the terms are cut into consecutive
        # batches whose workspace fits, run one after the other
        budget = getattr(dmrg, "workspace_budget", None)
        nb = 1
        while True:
            cuts = numpy.linspace(0, self.nops, nb + 1).round().astype(int)
            pids, wss = [], []
            for b in range(nb):
                sl = slice(cuts[b], cuts[b + 1])
                if sl.start == sl.stop:
                    continue
                used = sorted(set(op_cls[sl]))
                remap = {c: i for i, c in enumerate(used)}
                pid, ws = eng.sigma_plan(ncsite, [remap[c] for c in op_cls[sl]], [lay_L[c] for c in used],
                                         [lay_Wi[c] for c in used],
                                         [lay_Wj[c] for c in used] if ncsite == 2 else None,
                                         [lay_Rf[c] for c in used], lay_psi, off_L[sl], off_R[sl],
                                         off_Wi[sl], off_Wj[sl] if ncsite == 2 else None, wts[sl])
                pids.append(pid)
                wss.append(ws)
            if budget is None or max(wss) <= budget or nb >= self.nops:
                break
            for pid in pids:
                eng.destroy_plan(pid)
            nb *= 2
        self.pids = pids
        self.pid = pids[0]
        self.ws_elems = max(max(wss) // 8, 1)
        stats = [eng.plan_stats(pid) for pid in pids]
        self.flops = sum(x[0] for x in stats)
        self.ntasks = sum(x[1] for x in stats)
        self.nlaunch = stats[0][2]
        self.fL, self.fR = fL, fR
        self.graphs = {}
        self._kept_token = None

    @property
    def workspace(self):
        return _shared_workspace(self._dmrg(), self.ws_elems)

    def rebind(self, fL, fR):
        """Reuse for environments of the same structure (new device buffers)."""
        self.fL, self.fR = fL, fR
        self.graphs = {}
        self._kept_token = None

    def _fixed_token(self, W):
        """Identity and in-place-write counters of the operands that stay
        fixed during a Davidson solve (environments, MPO) and the workspace:
        equal tokens on two calls mean the engine may reuse the digit planes
        it cut from them on the first call."""
        ts = (self.fL.buf, self.fR.buf, W)
        return tuple((id(t), t.data_ptr(), t._version) for t in ts) + (self.workspace.data_ptr(),)

    def run(self, dmrg, x, y, precision, use_graph=False):
        """y = H x.  With ``use_graph`` the launches of this plan are recorded
        once into a CUDA graph (per precision) over staging vectors and
        replayed on every later call of the site."""
        eng = _engine.get()
        W = dmrg.mpo_store.buf
        if self.nmap is not None:
            torch = _torch()
            idx, nN = self.nmap
            xN = torch.zeros(nN, dtype=torch.float64, device=x.device)
            xN[idx] = x
            yN = torch.empty_like(xN)
            self._run(eng, W, xN, yN, precision, use_graph)
            torch.index_select(yN, 0, idx, out=y)
            return
        self._run(eng, W, x, y, precision, use_graph)

    def _run(self, eng, W, x, y, precision, use_graph):
        if len(self.pids) > 1:
            tmp = _torch().empty_like(y)
            eng.sigma(self.pids[0], self.fL.buf, self.fR.buf, W, x, y, self.workspace, precision)
            for pid in self.pids[1:]:
                eng.sigma(pid, self.fL.buf, self.fR.buf, W, x, tmp, self.workspace, precision)
                y += tmp
            return
        if not use_graph:
            tok = None
            if precision == "split":
                tok = self._fixed_token(W)
                eng.sigma_reuse_kept(self.pid, tok == self._kept_token)
                self._kept_token = None
            eng.sigma(self.pid, self.fL.buf, self.fR.buf, W, x, y, self.workspace, precision)
            if tok is not None:
                self._kept_token = tok
            return
        torch = _torch()
        rec = self.graphs.get(precision)
        if rec is not None and rec[3] != self.workspace.data_ptr():
            rec = None  # the shared workspace was reallocated since the recording
        if rec is None:
            xs = torch.empty_like(x)
            ys = torch.empty_like(y)
            xs.copy_(x)
            # warm-up outside capture: builds the device task lists
            eng.sigma(self.pid, self.fL.buf, self.fR.buf, W, xs, ys, self.workspace, precision)
            torch.cuda.synchronize()
            graph = torch.cuda.CUDAGraph()
            with torch.cuda.graph(graph):
                eng.sigma(self.pid, self.fL.buf, self.fR.buf, W, xs, ys, self.workspace, precision)
            rec = (graph, xs, ys, self.workspace.data_ptr())
            self.graphs[precision] = rec
        graph, xs, ys, _ = rec
        xs.copy_(x)
        graph.replay()
        y.copy_(ys)

    def hdiag(self, dmrg, d):
        eng = _engine.get()
        W = dmrg.mpo_store.buf
        eng.hdiag(self.pids[0], self.fL.buf, self.fR.buf, W, d)
        if len(self.pids) > 1:
            tmp = _torch().empty_like(d)
            for pid in self.pids[1:]:
                eng.hdiag(pid, self.fL.buf, self.fR.buf, W, tmp)
                d += tmp

    def release(self):
        self.released = True
        self.graphs = {}
        if self.pid is not None:
            for pid in self.pids:
                _engine.get().destroy_plan(pid)
            self.pid = None
            self.pids = []


def _qt_signature(h, t):
    h.update(numpy.asarray(t.status, dtype=numpy.int8).tobytes())
    for q, d in zip(t.qsyms, t.ndims):
        q = numpy.ascontiguousarray(q, dtype=numpy.float64)
        d = numpy.ascontiguousarray(d, dtype=numpy.int64)
        h.update(numpy.int64(q.size).tobytes())
        h.update(q.tobytes())
        h.update(numpy.int64(d.size).tobytes())
        h.update(d.tobytes())


def _sigma_key(dmrg, isite, ncsite, fL, fR):
    """Content key of a sigma plan: everything its task lists depend on (the
    dot, the MPO and its term weights, the target label, the wavefunction
    block structure, the block structures and offsets of every environment).
    Equal keys give identical plans, so a later sweep that meets the same
    structures at a dot reuses the plan with the new environment buffers."""
    h = hashlib.blake2b(digest_size=24)
    h.update(repr((isite, ncsite, dmrg.mpo_store.uid, bool(dmrg.ifs2proj), dmrg.nops,
                   getattr(dmrg, "workspace_budget", None))).encode())
    h.update(numpy.ascontiguousarray(dmrg.qkey, dtype=numpy.float64).tobytes())
    h.update(numpy.ascontiguousarray(dmrg.hpwts, dtype=numpy.float64).tobytes())
    _qt_signature(h, dmrg.qtmp)
    for env in (fL, fR):
        off = numpy.asarray(env.off, dtype=numpy.int64)
        h.update(off.tobytes())
        for iop in numpy.nonzero(off >= 0)[0]:
            _qt_signature(h, env.tensors[iop])
    return h.digest()


# cached sigma plans per driver: at most this many block tasks in total
# (the plans' device task lists; their workspace is shared)
_SIGMA_CACHE_TASKS = 60_000_000


def _release_all(cache):
    for plan in list(cache.values()):
        try:
            plan.release()
        except Exception:  # the engine may already be gone at interpreter exit
            pass
    cache.clear()


def _plan_cache(dmrg, name):
    """The driver's plan cache ``name``; its plans (device task lists) are
    released when the driver is collected."""
    cache = dmrg.__dict__.get(name)
    if cache is None:
        cache = collections.OrderedDict()
        dmrg.__dict__[name] = cache
        weakref.finalize(dmrg, _release_all, cache)
    return cache


def _sigma_plan(info):
    dmrg, isite, ncsite, flst, status, ifsym = info
    fL, fR = flst[0][0:2]
    fast = (fL.uid, fR.uid, isite, ncsite, dmrg.qtmp_psi_layout, dmrg.mpo_store.uid,
            getattr(dmrg, "workspace_budget", None))
    cur = getattr(dmrg, "_sigma_plan", None)
    if cur is not None and cur[0] == fast and not cur[1].released:
        return cur[1]
    key = _sigma_key(dmrg, isite, ncsite, fL, fR)
    cache = _plan_cache(dmrg, "_sigma_cache")
    plan = cache.pop(key, None)
    counts = dmrg.__dict__.setdefault("plan_counts", collections.Counter())
    if plan is None or plan.released:
        plan = SigmaPlan(dmrg, isite, ncsite, fL, fR)
        counts["sigma_built"] += 1
    else:
        plan.rebind(fL, fR)
        counts["sigma_reused"] += 1
    cache[key] = plan
    total = sum(getattr(p, "ntasks", 0) for p in cache.values())
    while total > _SIGMA_CACHE_TASKS and len(cache) > 1:
        _, old = cache.popitem(last=False)
        total -= getattr(old, "ntasks", 0)
        old.release()
    dmrg._sigma_plan = (fast, plan)
    return plan


def _check_path(dmrg):
    if getattr(dmrg, "ifpt", False):
        raise NotImplementedError("the perturbation-theory H0 - E0 form of HVec (dmrg.ifpt) is not part "
                                  "of this engine's sigma-vector path")


def _nqt_positions(info, ndim0, prjmap):
    """For ``dmrg.ifQt = False``: position in the caller's dense-ordered
    vector of every packed block element, as a device index tensor (None in
    the packed-order case).  ``prjmap`` lists the dense indices of the
    caller's elements (the reference's ``dptSymmetry`` dictionary entry,
    ``mpo_dmrg_dotutil.py:102-145``); the target label is read from it, the
    packed layout set up for that label, and the map cached per driver."""
    dmrg, isite, ncsite = info[0], info[1], info[2]
    if getattr(dmrg, "ifQt", True):
        return None
    if prjmap is None:
        raise ValueError("HVec/HDiag with dmrg.ifQt = False need prjmap (dense index of each element)")
    torch = _torch()
    prj = numpy.asarray(prjmap, dtype=numpy.int64).reshape(-1)
    if prj.size != ndim0:
        raise ValueError("prjmap has %d entries, ndim0 is %d" % (prj.size, ndim0))
    qlst = [numpy.asarray(q, dtype=float) for q in dmrg.qlst]
    dims = [len(q) for q in qlst]
    ndim = int(numpy.prod(dims))
    if prj.size == 0 or prj.min() < 0 or prj.max() >= ndim:
        raise ValueError("prjmap entries outside the dense (%s) tensor" % ",".join(map(str, dims)))
    h = hashlib.blake2b(prj.tobytes(), digest_size=16)
    for q in qlst:
        h.update(q.tobytes())
    key = (isite, ncsite, h.digest())
    cache = dmrg.__dict__.setdefault("_nqt_pos_cache", {})
    hit = cache.get(key)
    if hit is not None:
        if dmrg.qtmp_psi_layout != hit[1]:
            dmrg.setupQtmpCI(ncsite, list(hit[2]))
        return hit[0]
    # total label of the caller's elements, from the first one
    idx0 = numpy.unravel_index(int(prj[0]), dims)
    qkey = sum(qlst[i][idx0[i]] for i in range(len(qlst)))
    dmrg.setupQtmpCI(ncsite, [float(v) for v in numpy.atleast_1d(qkey)])
    dense_of_packed = numpy.asarray(dmrg.qtmp.prjmap(dmrg.idlstCI), dtype=numpy.int64)
    inv = numpy.full(ndim, -1, dtype=numpy.int64)
    inv[prj] = numpy.arange(prj.size)
    pos = inv[dense_of_packed]
    if dense_of_packed.size != prj.size or (pos < 0).any():
        raise ValueError("prjmap does not span the symmetry sector of its first element")
    if len(cache) > 64:
        cache.clear()
    pos_d = torch.as_tensor(pos, device="cuda")
    cache[key] = (pos_d, dmrg.qtmp_psi_layout, tuple(float(v) for v in numpy.atleast_1d(qkey)))
    return pos_d


def HVec(vec0, info, ndim0, prjmap):
    """y = H x over every operator term of the dot, on the GPU."""
    dmrg = info[0]
    _check_path(dmrg)
    torch = _torch()
    pos = _nqt_positions(info, ndim0, prjmap)
    plan = _sigma_plan(info)
    x, was_host = _to_device(vec0)
    if pos is not None:
        x = x.index_select(0, pos)
    y = torch.empty(ndim0, dtype=torch.float64, device=x.device)
    if plan.pid is None:
        y.zero_()
    else:
        plan.run(dmrg, x, y, getattr(dmrg, "precision", "fp64"), getattr(dmrg, "use_graph", False))
    if pos is not None:
        yd = torch.empty_like(y)
        yd[pos] = y
        y = yd
    return y.cpu().numpy() if was_host else y


def _diag_out(dmrg, d, pos):
    if pos is not None:
        dd = _torch().empty_like(d)
        dd[pos] = d
        d = dd
    return d if getattr(dmrg, "device_vectors", False) else d.cpu().numpy()


def HDiag(info, ndim0, prjmap):
    """diag(H) (Davidson preconditioner) in the caller's vector order."""
    dmrg = info[0]
    _check_path(dmrg)
    torch = _torch()
    pos = _nqt_positions(info, ndim0, prjmap)
    plan = _sigma_plan(info)
    d = torch.zeros(ndim0, dtype=torch.float64, device="cuda")
    if plan.pid is None:
        return _diag_out(dmrg, d, pos)
    if plan.nmap is not None:
        idx, nN = plan.nmap
        dN = torch.zeros(nN, dtype=torch.float64, device="cuda")
        plan.hdiag(dmrg, dN)
        torch.index_select(dN, 0, idx, out=d)
        return _diag_out(dmrg, d, pos)
    plan.hdiag(dmrg, d)
    return _diag_out(dmrg, d, pos)


def renorm(dmrg, isite, ncsite, flst, flstN, site, status):
    """New environments of every operator term after the site update; the
    result EnvSet is stored in ``flstN[0][0]`` (a one-element list)."""
    eng = _engine.get()
    torch = _torch()
    mpo = dmrg.mpo_store
    qsite = site
    if dmrg.ifs2proj:
        from .spinproj import reduce_site
        qsite = reduce_site(site)
    if status == 'L':
        fE = flst[0][0]
        jsite = isite
    else:
        fE = flst[0][1]
        jsite = isite + ncsite - 1
    ops = [iop for iop in range(dmrg.nops) if fE.present(iop)]
    nop = dmrg.nops
    if not ops:
        buf = torch.zeros(1, dtype=torch.float64, device="cuda")
        flstN[0][0] = EnvSet(buf, numpy.full(nop, -1, dtype=numpy.int64), numpy.full(nop, -1, dtype=numpy.int64),
                             [None] * nop)
    else:
        rp = _renorm_plan(dmrg, status, jsite, fE, qsite, ops)
        tick = getattr(dmrg, "tick", None)
        if tick is not None:
            tick("renorm_plan")
        buf = torch.empty(max(rp.total, 1), dtype=torch.float64, device="cuda")
        work = torch.empty(max(rp.ws // 8, 1), dtype=torch.float64, device="cuda")
        sval, _ = _to_device(qsite.value)
        eng.renorm(rp.pid, fE.buf, mpo.buf, sval, buf, work, getattr(dmrg, "precision_renorm", "fp64"))
        flstN[0][0] = EnvSet(buf, rp.off.copy(), rp.lays.copy(), list(rp.tens))
    if dmrg.ifs2proj:
        from .spinproj import renorm_S00
        renorm_S00(dmrg, isite, ncsite, flst, flstN, site, status)
    return 0


class RenormPlan:
    """A renormalisation plan and the host structure of its outputs (block
    structure and offset of every term's new environment)."""
    released = False

    def __init__(self, dmrg, status, jsite, fE, qsite, ops):
        from .mpo import op_class
        eng = _engine.get()
        mpo = dmrg.mpo_store
        classes = {}
        op_cls, lay_env, lay_W, off_env, off_W = [], [], [], [], []
        for iop in ops:
            c0 = op_class(dmrg.opers[iop][0], jsite)
            if c0 not in classes:
                classes[c0] = len(classes)
                lay_env.append(fE.layouts[iop])
                wt = mpo.tensors[jsite][iop]
                if status == 'L':
                    lay_W.append(wt.layout)
                else:
                    st = wt.status.copy()
                    st[0], st[1] = not st[0], not st[1]
                    lay_W.append(eng.derive(wt.layout, [-wt.qsyms[0], -wt.qsyms[1], wt.qsyms[2],
                                                        wt.qsyms[3]], st))
            op_cls.append(classes[c0])
            off_env.append(fE.off[iop])
            off_W.append(mpo.off[jsite][iop])
        nop = dmrg.nops
        self.off = numpy.full(nop, -1, dtype=numpy.int64)
        self.lays = numpy.full(nop, -1, dtype=numpy.int64)
        self.tens = [None] * nop
        self.pid, lay_out, off_out, self.total, self.ws = eng.renorm_plan(status, op_cls, lay_env, lay_W,
                                                                          qsite.layout, off_env, off_W)
        self.ntasks = eng.plan_stats(self.pid)[1]
        # host structure of each output (layout id per class)
        struct = {}
        for k, iop in enumerate(ops):
            c = op_cls[k]
            if lay_out[c] < 0 or off_out[k] < 0:
                continue
            if c not in struct:
                struct[c] = _env_structure(dmrg, status, qsite, mpo.tensors[jsite][iop], fE.tensors[iop],
                                           int(lay_out[c]))
            self.off[iop] = off_out[k]
            self.lays[iop] = struct[c].layout
            self.tens[iop] = struct[c]

    def release(self):
        if not self.released:
            self.released = True
            _engine.get().destroy_plan(self.pid)


def _renorm_plan(dmrg, status, jsite, fE, qsite, ops):
    """Renormalisation plan for this site update, reused when a later sweep
    meets the same structures (key: the side, the site, the MPO, the site
    tensor's block structure and the block structures and offsets of the
    environments it extends)."""
    h = hashlib.blake2b(digest_size=24)
    h.update(repr((status, jsite, dmrg.mpo_store.uid, bool(dmrg.ifs2proj), dmrg.nops)).encode())
    _qt_signature(h, qsite)
    off = numpy.asarray(fE.off, dtype=numpy.int64)
    h.update(off.tobytes())
    for iop in ops:
        _qt_signature(h, fE.tensors[iop])
    key = h.digest()
    cache = _plan_cache(dmrg, "_renorm_cache")
    rp = cache.pop(key, None)
    counts = dmrg.__dict__.setdefault("plan_counts", collections.Counter())
    if rp is None or rp.released:
        rp = RenormPlan(dmrg, status, jsite, fE, qsite, ops)
        counts["renorm_built"] += 1
    else:
        counts["renorm_reused"] += 1
    cache[key] = rp
    total = sum(p.ntasks for p in cache.values())
    while total > _SIGMA_CACHE_TASKS and len(cache) > 1:
        _, old = cache.popitem(last=False)
        total -= old.ntasks
        old.release()
    return rp


def SVec(vec0, info, ndim0, prjmap):
    """S psi for the spin-projected problem (``mpo_dmrg_kernel.SVec``, 226-231)."""
    from .spinproj import SVec as _svec
    pos = _nqt_positions(info, ndim0, prjmap)
    if pos is None:
        return _svec(vec0, info, ndim0, prjmap)
    x, was_host = _to_device(vec0)
    y = _svec(x.index_select(0, pos), info, ndim0, prjmap)
    yd = _torch().empty_like(y)
    yd[pos] = y
    return yd.cpu().numpy() if was_host else yd


def SDiag(info, ndim0, prjmap):
    """diag(S) in the caller's vector order (``SDiag``, 185-224)."""
    from .spinproj import SDiag as _sdiag
    pos = _nqt_positions(info, ndim0, prjmap)
    return _diag_out(info[0], _sdiag(info, ndim0, prjmap), pos)


def _env_structure(dmrg, status, qsite, wt, env, lay_out):
    """Host qtensor describing a renormalised environment block structure:
    legs [b, bra, ket] with the reference's labels (status [T, F, T])."""
    t = qtensor([True, False, True])
    if status == 'L':
        q = [wt.qsyms[1], qsite.qsyms[2], qsite.qsyms[2]]
        d = [wt.ndims[1], qsite.ndims[2], qsite.ndims[2]]
    else:
        q = [-wt.qsyms[0], qsite.qsyms[0], qsite.qsyms[0]]
        d = [wt.ndims[0], qsite.ndims[0], qsite.ndims[0]]
    t.fromQsyms(3, q, d, ifallocate=False)
    size, flat, _ = _engine.get().layout_blocks(lay_out)
    if size != t.size_allowed or not numpy.array_equal(flat, t.blk_flat):
        raise RuntimeError("renormalised environment layout mismatch")
    return t
