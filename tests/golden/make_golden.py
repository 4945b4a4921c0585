"""Generate the golden fixtures from the reference checkout (run here, not on
the GPU machine): the K=6 FCIDUMP of ``samps/example_conversion/5.h6+_doublet``
with the BLOCK M=1000 sweep energy recorded in its ``dmrg.out``, and the
reference's own block rule (``ctypes/qsym.c``, built by ``oracle/Makefile``)
evaluated on seeded random leg labels.

    python tests/golden/make_golden.py [/path/to/reference]
"""
import ctypes
import os
import re
import sys

import numpy

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def main(ref=os.environ.get("ZMPO_REFERENCE", "/root/reference")):
    from oracle import integrals
    case = os.path.join(ref, "source", "samps", "example_conversion", "5.h6+_doublet")
    d = integrals.read_fcidump(os.path.join(case, "FCIDUMP"))
    text = open(os.path.join(case, "dmrg.out")).read()
    m = re.findall(r"Sweep Energy = ([-0-9.]+)", text)
    e_block = float(m[-1])
    numpy.savez_compressed(os.path.join(HERE, "h6p_doublet_fcidump.npz"), h1e=d["h1e"], eri=d["eri"],
                           ecore=d["ecore"], nelec=d["nelec"], ms2=d["ms2"], e_block=e_block)
    # reference symAllowed on random labels
    lib = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libqsym.so"))
    rng = numpy.random.default_rng(12345)
    cases = {}
    for c in range(24):
        rank = int(rng.integers(2, 8))
        nq = int(rng.integers(1, 3))
        nsyms = rng.integers(1, 5, size=rank).astype(numpy.int32)
        status = rng.integers(0, 2, size=rank).astype(numpy.int32)
        qs = [numpy.ascontiguousarray(rng.integers(-2, 3, size=(n, nq)) * 0.5, dtype=numpy.float64)
              for n in nsyms]
        nb = int(numpy.prod(nsyms))
        allowed = numpy.zeros(nb, dtype=numpy.int32)
        args = [q.ctypes.data_as(ctypes.c_void_p) for q in qs] + [ctypes.c_void_p()] * (8 - rank)
        lib.symAllowed(ctypes.c_int(rank), ctypes.c_int(nq), nsyms.ctypes.data_as(ctypes.c_void_p),
                       status.ctypes.data_as(ctypes.c_void_p), allowed.ctypes.data_as(ctypes.c_void_p), *args)
        cases["c%d_nsyms" % c] = nsyms
        cases["c%d_status" % c] = status
        cases["c%d_nq" % c] = numpy.array(nq)
        for i, q in enumerate(qs):
            cases["c%d_q%d" % (c, i)] = q
        cases["c%d_allowed" % c] = allowed
    numpy.savez_compressed(os.path.join(HERE, "qsym_reference.npz"), ncase=24, **cases)
    print("e_block", e_block)


if __name__ == "__main__":
    main(*sys.argv[1:])
