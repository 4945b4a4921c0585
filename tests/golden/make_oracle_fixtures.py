"""Generate the oracle fixtures the GPU parity tests compare against (run on
a CPU host; the oracle needs a few minutes).

``sweep_k10_d64.npz``: the first benchmark configuration -- K=10 spatial
orbitals, 10 electrons, Sz=0, seeded synthetic integrals (seed 2024), bond
dimension 64, the default two-site schedule (M ramp from 25, perturbed
density-matrix noise 1e-4 in the first four sweeps, Davidson tolerance
1e-4 down to 1e-9), 12 sweeps, driver seed 1 -- run by the oracle's
restatement of the reference's driver (``mpo_dmrg_class.default``,
``mpo_dmrg_opt.sweep``).  Stores the energy of every sweep (the lower of its
two half sweeps), of every dot in sweep order, and the final energy.  Runs
with other noise seeds reach the same energies to 1e-10 from the sixth sweep
on (the first sweeps depend on the random noise draws).

    python tests/golden/make_oracle_fixtures.py
"""
import os
import sys
import time

import numpy

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

SWEEP_K10 = dict(K=10, nelec=10, D=64, seed=2024, driver_seed=1, tol=1e-9, maxiter=12)


def sweep_k10():
    from oracle import dmrg as od, integrals as oint
    c = SWEEP_K10
    K = c["K"]
    h, eri, _ = oint.synthetic(K, c["seed"])
    i1, i2, _ = oint.to_spin_orbital(h, eri)
    occ = numpy.array([1., 1.] * (c["nelec"] // 2) + [0., 0.] * (K - c["nelec"] // 2))
    o = od.mpo_dmrg(seed=c["driver_seed"])
    o.nsite, o.sbas, o.isym = K, 2 * K, 2
    o.build()
    o.occun = occ
    o.qsectors = {str([float(c["nelec"]), 0.0]): 1}
    o.partition()
    o.loadInts(i1, i2)
    o.dumpMPO()
    sc = od.schedule(maxM=c["D"], tol=c["tol"], maxiter=c["maxiter"])
    sc.normal(2)
    t0 = time.time()
    o.default(sc)
    dots = numpy.array([float(numpy.asarray(e).ravel()[0]) for e in o.esweeps])
    numpy.savez_compressed(os.path.join(HERE, "sweep_k10_d64.npz"), dot_energies=dots,
                           sweep_energies=numpy.array(o.eav, dtype=float),
                           energy=float(o.Energy), nsweep=int(o.nsweep),
                           **{k: v for k, v in c.items()})
    print("sweep_k10_d64: E = %.12f after %d sweeps (%.0f s)" % (o.Energy, o.nsweep, time.time() - t0))


if __name__ == "__main__":
    sweep_k10()
