"""Build ``libzmpo_gb300.so`` (the engine's C ABI) in-tree with nvcc for sm_103a.

Run as ``python -m zmpo_dmrg_gb300.build``; ``__graft_entry__.build()`` calls
``build()``.  Three translation units are compiled in parallel and linked
against the shared CUDA runtime.  Rebuilds only when a source is newer than
the library.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libzmpo_gb300.so")
SOURCES = ["planner.cpp", "kernels.cu", "kernels_umma.cu"]
HEADERS = [os.path.join(CSRC, "engine.h"), os.path.join(CSRC, "device_common.cuh"),
           os.path.join(os.path.dirname(HERE), "include", "zmpo_gb300.h")]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


def nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False):
    os.makedirs(BUILD, exist_ok=True)
    objs = []
    jobs = []
    for src in SOURCES:
        path = os.path.join(CSRC, src)
        obj = os.path.join(BUILD, src + ".o")
        objs.append(obj)
        if force or _stale(obj, [path] + HEADERS):
            cmd = [nvcc(), "-c", path, "-o", obj] + ARCH + FLAGS
            if src.endswith(".cpp"):
                cmd = [nvcc(), "-x", "cu", "-c", path, "-o", obj] + ARCH + FLAGS
            jobs.append(cmd)

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
        return r.stderr

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        for out in ex.map(run, jobs):
            if verbose and out:
                print(out)
    if force or jobs or _stale(LIB, objs):
        run([nvcc(), "-shared", "-o", LIB] + objs + ARCH + ["-cudart", "shared"])
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
