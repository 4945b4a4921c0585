"""CPU oracle for the DMRG sigma-vector / renormalisation path.

TEST INFRASTRUCTURE ONLY.  This package is a Python-3 + NumPy restatement of the
reference code's own algorithm (zhendongli2008/zmpo_dmrg, Python 2, FP64), used
as the checker for the GPU engine in ``zmpo_dmrg_gb300``.  Only ``tests/``,
``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl reference`` legs
of ``bench.py`` may import it.  The product package never imports it.

Pinning (how the restatement is tied to the reference):
  * ``qtensor.py`` block-selection rule == the reference's own C ``symAllowed``
    (``ctypes/qsym.c``), compiled from the reference sources into
    ``oracle/_ref/libqsym.so`` by ``oracle/Makefile`` (tests skip when absent);
  * sum_p MPO_p contracted over the chain == exact Jordan-Wigner H
    (``integrals.py``);
  * Qt MPO blocks == dense MPO (reference self-test ``testHRfacSpatial``);
  * H built column-by-column from HVec is symmetric and its diagonal equals
    HDiag (reference debug switch ``checkDiagNQt`` / ``checkDiagQt``);
  * two-site DMRG on the reference's ``5.h6+_doublet/FCIDUMP`` reaches the BLOCK
    M=1000 energy -3.236066277269 recorded in the reference's ``dmrg.out``.

Mechanical edits relative to the reference: Python 3 syntax, h5py files replaced
by in-memory dicts, MPI communicator of size 1 (no Reduce/Bcast), seeded
``numpy.random.Generator`` for the Davidson/decimation noise, MPO slicing fixed
at ``maxslc = 1`` (the reference default, ``mpo_dmrg_class.py:147``).
"""
