"""Python handle on the GB300 engine: layouts, plans and device launches.

Device memory is owned by torch tensors; the engine receives raw pointers and
the current CUDA stream.  Only block structure (layouts, task lists) lives in
the engine.
"""
import ctypes

import numpy

from . import _lib
from ._lib import check, as_i32, as_i64, as_f64, iptr, lptr, dptr

_ENGINES = {}


def _torch():
    import torch
    return torch


def device_ptr(t):
    """Raw device pointer of a contiguous float64 torch tensor."""
    if t is None:
        return None
    if not t.is_cuda:
        raise RuntimeError("engine buffers must be CUDA tensors")
    if t.dtype != _torch().float64 or not t.is_contiguous():
        raise RuntimeError("engine buffers must be contiguous float64")
    return ctypes.c_void_p(t.data_ptr())


ZMPO_E_NOMEM = -5


def checked_call(call, what):
    """Run an engine call; when it fails for want of device memory, return
    the blocks PyTorch's caching allocator holds unused to the device and try
    once more (the engine allocates with cudaMalloc, which cannot use them)."""
    rc = call()
    if rc == ZMPO_E_NOMEM:
        _torch().cuda.empty_cache()
        rc = call()
    return check(rc, what)


def current_stream():
    torch = _torch()
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


class Engine:
    def __init__(self, device=0):
        self.device = device
        h = ctypes.c_void_p()
        check(_lib.lib().zmpo_engine_create(ctypes.byref(h), device), "engine_create")
        self.h = h
        self._layout_cache = {}

    def __del__(self):
        try:
            if self.h:
                _lib.lib().zmpo_engine_destroy(self.h)
        except Exception:
            pass

    # ----------------------------------------------------------- layouts
    def layout(self, qsyms, ndims, status):
        """Layout id of a block-sparse tensor (cached on its structure)."""
        rank = len(qsyms)
        nq = int(numpy.asarray(qsyms[0]).reshape(len(ndims[0]), -1).shape[1]) if rank else 1
        q = [as_f64(numpy.asarray(x, dtype=float).reshape(len(d), nq)) for x, d in zip(qsyms, ndims)]
        key = (tuple(x.tobytes() for x in q), tuple(tuple(int(v) for v in d) for d in ndims),
               tuple(int(bool(s)) for s in status))
        lid = self._layout_cache.get(key)
        if lid is not None:
            return lid
        nsec = as_i32([len(d) for d in ndims])
        qcat = as_f64(numpy.concatenate([x.reshape(-1) for x in q]) if rank else numpy.zeros(1))
        dcat = as_i64(numpy.concatenate([numpy.asarray(d, dtype=numpy.int64) for d in ndims])
                      if rank else numpy.zeros(1))
        st = as_i32([1 if s else 0 for s in status] or [0])
        out = ctypes.c_int()
        check(_lib.lib().zmpo_layout_create(self.h, rank, nq, iptr(nsec), dptr(qcat), lptr(dcat),
                                            iptr(st), ctypes.byref(out)), "layout_create")
        self._layout_cache[key] = out.value
        return out.value

    def derive(self, src, qsyms, status):
        q = as_f64(numpy.concatenate([numpy.asarray(x, dtype=float).reshape(-1) for x in qsyms]))
        st = as_i32([1 if s else 0 for s in status])
        out = ctypes.c_int()
        check(_lib.lib().zmpo_layout_derive(self.h, src, dptr(q), iptr(st), ctypes.byref(out)),
              "layout_derive")
        return out.value

    def layout_blocks(self, lid):
        size = ctypes.c_int64()
        nb = ctypes.c_int64()
        rank = ctypes.c_int()
        check(_lib.lib().zmpo_layout_info(self.h, lid, ctypes.byref(size), ctypes.byref(nb),
                                          ctypes.byref(rank)), "layout_info")
        flat = numpy.zeros(max(nb.value, 1), dtype=numpy.int64)
        off = numpy.zeros(max(nb.value, 1), dtype=numpy.int64)
        check(_lib.lib().zmpo_layout_blocks(self.h, lid, lptr(flat), lptr(off)), "layout_blocks")
        return int(size.value), flat[:nb.value], off[:nb.value]

    # ---------------------------------------------------------- contraction
    def contract_plan(self, lay_a, lay_b, axes):
        ax1 = as_i32(list(axes[0]) or [0])
        ax2 = as_i32(list(axes[1]) or [0])
        lo = ctypes.c_int()
        pid = ctypes.c_int()
        check(_lib.lib().zmpo_contract_plan(self.h, lay_a, lay_b, len(axes[0]), iptr(ax1), iptr(ax2),
                                            ctypes.byref(lo), ctypes.byref(pid)), "contract_plan")
        return lo.value, pid.value

    def contract_exec(self, pid, a, b, out, precision="fp64"):
        checked_call(lambda: _lib.lib().zmpo_contract_exec(self.h, pid, device_ptr(a), device_ptr(b),
                                                           device_ptr(out), _lib.PREC[precision],
                                                           current_stream()), "contract_exec")

    def plan_stats(self, pid):
        fl = ctypes.c_double()
        nt = ctypes.c_int64()
        nl = ctypes.c_int()
        check(_lib.lib().zmpo_plan_stats(self.h, pid, ctypes.byref(fl), ctypes.byref(nt),
                                         ctypes.byref(nl)), "plan_stats")
        return fl.value, nt.value, nl.value

    # task records of csrc/engine.h (C layout)
    GROUP = numpy.dtype([("c_off", "i8"), ("scm", "i8"), ("scn", "i8"), ("M", "i4"), ("N", "i4"),
                         ("seg0", "i4"), ("nseg", "i4"), ("cbuf", "i4"), ("ncb", "i4"), ("cb0", "i4"),
                         ("sb0", "i4")], align=True)
    SEG = numpy.dtype([("a_off", "i8"), ("b_off", "i8"), ("sam", "i8"), ("sak", "i8"), ("sbk", "i8"),
                       ("sbn", "i8"), ("alpha", "f8"), ("K", "i4"), ("abuf", "i1"), ("bbuf", "i1"),
                       ("pad0", "i1"), ("pad1", "i1")], align=True)
    COLBLOCK = numpy.dtype([("c_off", "i8"), ("scm", "i8"), ("scn", "i8"), ("n0", "i4"), ("n", "i4")],
                           align=True)
    SEGB = numpy.dtype([("b_off", "i8"), ("sbk", "i8"), ("sbn", "i8")], align=True)
    REDUCTION = numpy.dtype([("c_off", "i8"), ("scm", "i8"), ("scn", "i8"), ("part_off", "i8"), ("M", "i4"),
                             ("N", "i4"), ("nparts", "i4"), ("cbuf", "i4"), ("elem0", "i8")], align=True)

    def step_tasks(self, pid, step):
        """Host copy of a step's task records (before its first execution):
        groups, segments, column blocks, B parts, split-K sums."""
        cnt = numpy.zeros(5, dtype=numpy.int64)
        check(_lib.lib().zmpo_plan_step_tasks(self.h, pid, step, lptr(cnt), None, None, None, None, None),
              "plan_step_tasks")
        arrs = [numpy.zeros(int(n), dtype=d) for n, d in zip(cnt, (self.GROUP, self.SEG, self.COLBLOCK,
                                                                   self.SEGB, self.REDUCTION))]
        check(_lib.lib().zmpo_plan_step_tasks(self.h, pid, step, lptr(cnt), *[a.ctypes.data_as(ctypes.c_void_p)
                                                                               for a in arrs]),
              "plan_step_tasks")
        return arrs

    def kernel_count(self, pid, precision="split"):
        """Kernel launches one execution of the plan issues at ``precision``."""
        n = ctypes.c_int()
        check(_lib.lib().zmpo_plan_kernel_count(self.h, pid, _lib.PREC[precision], ctypes.byref(n)),
              "plan_kernel_count")
        return n.value

    def mma_macs(self, pid, precision="split", nmax=8):
        """Multiply-adds the tiles of each step issue at ``precision``."""
        macs = numpy.zeros(nmax)
        check(_lib.lib().zmpo_plan_mma_macs(self.h, pid, _lib.PREC[precision], nmax, dptr(macs)), "plan_mma_macs")
        return macs

    def profile(self, on=True):
        check(_lib.lib().zmpo_profile(self.h, 1 if on else 0), "profile")

    def launch_times(self, pid, nmax=8):
        ms = numpy.zeros(nmax)
        by = numpy.zeros(nmax)
        nc = numpy.zeros(nmax, dtype=numpy.int64)
        check(_lib.lib().zmpo_plan_launch_times(self.h, pid, nmax, dptr(ms), dptr(by), lptr(nc)),
              "launch_times")
        return ms, by, nc

    def plan_groups(self, pid, step):
        n = ctypes.c_int64()
        check(_lib.lib().zmpo_plan_groups(self.h, pid, step, ctypes.byref(n), None, None, None, None),
              "plan_groups")
        M = numpy.zeros(max(n.value, 1), dtype=numpy.int32)
        N = numpy.zeros_like(M)
        S = numpy.zeros_like(M)
        Kt = numpy.zeros(max(n.value, 1), dtype=numpy.int64)
        check(_lib.lib().zmpo_plan_groups(self.h, pid, step, ctypes.byref(n), iptr(M), iptr(N), iptr(S),
                                          lptr(Kt)), "plan_groups")
        k = n.value
        return M[:k], N[:k], S[:k], Kt[:k]

    def device_status(self, reset=False):
        """Error word of the device kernels (0: none); see zmpo_device_status."""
        code = ctypes.c_int()
        check(_lib.lib().zmpo_device_status(self.h, ctypes.byref(code), 1 if reset else 0), "device_status")
        return code.value

    def destroy_plan(self, pid):
        check(_lib.lib().zmpo_plan_destroy(self.h, pid), "plan_destroy")

    # --------------------------------------------------------------- sigma
    def sigma_plan(self, ncsite, op_class, lay_L, lay_Wi, lay_Wj, lay_Rf, lay_psi, off_L, off_R,
                   off_Wi, off_Wj, wts):
        keep = dict(op_class=as_i32(op_class), lay_L=as_i32(lay_L), lay_Wi=as_i32(lay_Wi),
                    lay_Wj=as_i32(lay_Wj if lay_Wj is not None else lay_Wi), lay_Rf=as_i32(lay_Rf),
                    off_L=as_i64(off_L), off_R=as_i64(off_R), off_Wi=as_i64(off_Wi),
                    off_Wj=as_i64(off_Wj if off_Wj is not None else off_Wi), wts=as_f64(wts))
        d = _lib.SigmaDesc(ncsite, len(op_class), len(lay_L), iptr(keep["op_class"]),
                           iptr(keep["lay_L"]), iptr(keep["lay_Wi"]), iptr(keep["lay_Wj"]),
                           iptr(keep["lay_Rf"]), lay_psi, lptr(keep["off_L"]), lptr(keep["off_R"]),
                           lptr(keep["off_Wi"]), lptr(keep["off_Wj"]), dptr(keep["wts"]))
        pid = ctypes.c_int()
        check(_lib.lib().zmpo_sigma_plan(self.h, ctypes.byref(d), ctypes.byref(pid)), "sigma_plan")
        ws = ctypes.c_int64()
        check(_lib.lib().zmpo_sigma_workspace(self.h, pid.value, ctypes.byref(ws)), "sigma_workspace")
        return pid.value, ws.value

    def sigma(self, pid, L, R, W, x, y, workspace, precision="fp64"):
        ws = device_ptr(workspace) if workspace is not None else None
        checked_call(lambda: _lib.lib().zmpo_sigma(self.h, pid, device_ptr(L), device_ptr(R), device_ptr(W),
                                                   device_ptr(x), device_ptr(y), ws, _lib.PREC[precision],
                                                   current_stream()), "sigma")

    def sigma_reuse_kept(self, pid, reuse):
        """The next sigma call of plan ``pid`` may reuse the digit planes of
        its fixed operands (environments, MPO) from its previous call."""
        check(_lib.lib().zmpo_sigma_reuse_kept(self.h, pid, 1 if reuse else 0), "sigma_reuse_kept")

    def hdiag(self, pid, L, R, W, diag):
        checked_call(lambda: _lib.lib().zmpo_hdiag(self.h, pid, device_ptr(L), device_ptr(R), device_ptr(W),
                                                   device_ptr(diag), current_stream()), "hdiag")

    # -------------------------------------------------------------- renorm
    def renorm_plan(self, status, op_class, lay_env, lay_W, lay_site, off_env, off_W):
        keep = dict(op_class=as_i32(op_class), lay_env=as_i32(lay_env), lay_W=as_i32(lay_W),
                    off_env=as_i64(off_env), off_W=as_i64(off_W))
        d = _lib.RenormDesc(0 if status == 'L' else 1, len(op_class), len(lay_env),
                            iptr(keep["op_class"]), iptr(keep["lay_env"]), iptr(keep["lay_W"]),
                            lay_site, lptr(keep["off_env"]), lptr(keep["off_W"]))
        pid = ctypes.c_int()
        check(_lib.lib().zmpo_renorm_plan(self.h, ctypes.byref(d), ctypes.byref(pid)), "renorm_plan")
        lay_out = numpy.zeros(len(lay_env), dtype=numpy.int32)
        off_out = numpy.zeros(len(op_class), dtype=numpy.int64)
        tot = ctypes.c_int64()
        check(_lib.lib().zmpo_renorm_outputs(self.h, pid.value, iptr(lay_out), lptr(off_out),
                                             ctypes.byref(tot)), "renorm_outputs")
        ws = ctypes.c_int64()
        check(_lib.lib().zmpo_renorm_workspace(self.h, pid.value, ctypes.byref(ws)), "renorm_ws")
        return pid.value, lay_out, off_out, tot.value, ws.value

    def renorm(self, pid, env, W, site, out, workspace, precision="fp64"):
        ws = device_ptr(workspace) if workspace is not None else None
        checked_call(lambda: _lib.lib().zmpo_renorm(self.h, pid, device_ptr(env), device_ptr(W), device_ptr(site),
                                                    device_ptr(out), ws, _lib.PREC[precision],
                                                    current_stream()), "renorm")


def get(device=0):
    """Process-wide engine for ``device``."""
    eng = _ENGINES.get(device)
    if eng is None:
        eng = Engine(device)
        _ENGINES[device] = eng
    return eng
