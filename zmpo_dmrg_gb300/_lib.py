"""ctypes binding of ``libzmpo_gb300.so`` (declared in include/zmpo_gb300.h).

The library is built in-tree by ``zmpo_dmrg_gb300.build``.  Loading fails
loudly when it is missing: there is no CPU fallback for the engine.
"""
import ctypes
import os

import numpy

HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(HERE, "libzmpo_gb300.so")

PREC = {"fp64": 0, "split": 1, "emu64": 2}

c_int_p = ctypes.POINTER(ctypes.c_int)
c_i64_p = ctypes.POINTER(ctypes.c_int64)
c_dbl_p = ctypes.POINTER(ctypes.c_double)
c_void_p = ctypes.c_void_p


class SigmaDesc(ctypes.Structure):
    _fields_ = [("ncsite", ctypes.c_int), ("nop", ctypes.c_int), ("nclass", ctypes.c_int),
                ("op_class", c_int_p), ("lay_L", c_int_p), ("lay_Wi", c_int_p),
                ("lay_Wj", c_int_p), ("lay_Rf", c_int_p), ("lay_psi", ctypes.c_int),
                ("off_L", c_i64_p), ("off_R", c_i64_p), ("off_Wi", c_i64_p),
                ("off_Wj", c_i64_p), ("wts", c_dbl_p)]


class RenormDesc(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("nop", ctypes.c_int), ("nclass", ctypes.c_int),
                ("op_class", c_int_p), ("lay_env", c_int_p), ("lay_W", c_int_p),
                ("lay_site", ctypes.c_int), ("off_env", c_i64_p), ("off_W", c_i64_p)]


EXPORTS = {
    "zmpo_last_error": ([ctypes.c_char_p, ctypes.c_size_t], ctypes.c_int),
    "zmpo_version": ([], ctypes.c_int),
    "symAllowed": ([ctypes.c_int, ctypes.c_int, c_int_p, c_int_p, c_int_p] + [c_void_p] * 8,
                   ctypes.c_int),
    "zmpo_engine_create": ([ctypes.POINTER(c_void_p), ctypes.c_int], ctypes.c_int),
    "zmpo_engine_destroy": ([c_void_p], ctypes.c_int),
    "zmpo_layout_create": ([c_void_p, ctypes.c_int, ctypes.c_int, c_int_p, c_dbl_p, c_i64_p,
                            c_int_p, c_int_p], ctypes.c_int),
    "zmpo_layout_derive": ([c_void_p, ctypes.c_int, c_dbl_p, c_int_p, c_int_p], ctypes.c_int),
    "zmpo_layout_info": ([c_void_p, ctypes.c_int, c_i64_p, c_i64_p, c_int_p], ctypes.c_int),
    "zmpo_layout_blocks": ([c_void_p, ctypes.c_int, c_i64_p, c_i64_p], ctypes.c_int),
    "zmpo_contract_plan": ([c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, c_int_p, c_int_p,
                            c_int_p, c_int_p], ctypes.c_int),
    "zmpo_contract_exec": ([c_void_p, ctypes.c_int, c_void_p, c_void_p, c_void_p, ctypes.c_int,
                            c_void_p], ctypes.c_int),
    "zmpo_contract_exec_noalloc": ([c_void_p, ctypes.c_int, c_void_p, c_void_p, c_void_p, ctypes.c_int,
                                    c_void_p], ctypes.c_int),
    "zmpo_sigma_plan": ([c_void_p, ctypes.POINTER(SigmaDesc), c_int_p], ctypes.c_int),
    "zmpo_sigma_workspace": ([c_void_p, ctypes.c_int, c_i64_p], ctypes.c_int),
    "zmpo_plan_stats": ([c_void_p, ctypes.c_int, c_dbl_p, c_i64_p, c_int_p], ctypes.c_int),
    "zmpo_plan_kernel_count": ([c_void_p, ctypes.c_int, ctypes.c_int, c_int_p], ctypes.c_int),
    "zmpo_plan_mma_macs": ([c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, c_dbl_p], ctypes.c_int),
    "zmpo_plan_step_tasks": ([c_void_p, ctypes.c_int, ctypes.c_int, c_i64_p, c_void_p, c_void_p, c_void_p,
                              c_void_p, c_void_p], ctypes.c_int),
    "zmpo_sigma_reuse_kept": ([c_void_p, ctypes.c_int, ctypes.c_int], ctypes.c_int),
    "zmpo_sigma": ([c_void_p, ctypes.c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                    c_void_p, ctypes.c_int, c_void_p], ctypes.c_int),
    "zmpo_hdiag": ([c_void_p, ctypes.c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p],
                   ctypes.c_int),
    "zmpo_renorm_plan": ([c_void_p, ctypes.POINTER(RenormDesc), c_int_p], ctypes.c_int),
    "zmpo_renorm_outputs": ([c_void_p, ctypes.c_int, c_int_p, c_i64_p, c_i64_p], ctypes.c_int),
    "zmpo_renorm_workspace": ([c_void_p, ctypes.c_int, c_i64_p], ctypes.c_int),
    "zmpo_renorm": ([c_void_p, ctypes.c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                     ctypes.c_int, c_void_p], ctypes.c_int),
    "zmpo_profile": ([c_void_p, ctypes.c_int], ctypes.c_int),
    "zmpo_plan_launch_times": ([c_void_p, ctypes.c_int, ctypes.c_int, c_dbl_p, c_dbl_p, c_i64_p],
                               ctypes.c_int),
    "zmpo_plan_groups": ([c_void_p, ctypes.c_int, ctypes.c_int, c_i64_p, c_int_p, c_int_p, c_int_p,
                          c_i64_p], ctypes.c_int),
    "zmpo_device_status": ([c_void_p, c_int_p, ctypes.c_int], ctypes.c_int),
    "zmpo_plan_destroy": ([c_void_p, ctypes.c_int], ctypes.c_int),
}

_lib = None


def lib():
    """Load the engine library (once); raise if it was not built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIBPATH):
            raise RuntimeError("libzmpo_gb300.so is not built; run `python -m zmpo_dmrg_gb300.build`"
                               " (or __graft_entry__.build()) first")
        L = ctypes.CDLL(LIBPATH)
        for name, (argtypes, restype) in EXPORTS.items():
            fn = getattr(L, name)
            fn.argtypes = argtypes
            fn.restype = restype
        _lib = L
    return _lib


def last_error():
    buf = ctypes.create_string_buffer(4096)
    lib().zmpo_last_error(buf, 4096)
    return buf.value.decode(errors="replace")


def check(rc, what=""):
    if rc != 0:
        raise RuntimeError("zmpo engine error %d in %s: %s" % (rc, what, last_error()))
    return rc


def iptr(a):
    return a.ctypes.data_as(c_int_p)


def lptr(a):
    return a.ctypes.data_as(c_i64_p)


def dptr(a):
    return a.ctypes.data_as(c_dbl_p)


def as_i32(x):
    return numpy.ascontiguousarray(x, dtype=numpy.int32)


def as_i64(x):
    return numpy.ascontiguousarray(x, dtype=numpy.int64)


def as_f64(x):
    return numpy.ascontiguousarray(x, dtype=numpy.float64)
