"""GPU-vs-oracle parity at the benchmark configurations themselves.

* K=24, 24 electrons, D=512, middle two-site dot (the sigma-vector benchmark):
  the engine's H.psi over a subset of operator terms that covers every
  operator class the dot meets, against the oracle's HVecQt
  (``mpo_dmrg_kernelQt.py:153-319``) over the same terms fed the same
  environment values.  FP64 path <= 1e-10, split <= 1e-8, 56-bit emulation
  <= 1e-10 relative (norm of the difference over the norm).
* K=20, 20 electrons, D=512, singlet projection with 8 quadrature points:
  the same check on the spin-projected H.psi (N-only relabelled terms).
* K=10, 10 electrons, D=64, the reference's default two-site schedule from
  the occupation-number state (its initial one-site sweep included), 12
  sweeps: the energies of the converged sweeps and the final energy of the
  GPU driver against the oracle driver's (frozen in
  ``tests/golden/sweep_k10_d64.npz`` by
  ``tests/golden/make_oracle_fixtures.py``), within 1e-8 Eh.  The schedule
  adds density-matrix noise in the first four sweeps and tightens the
  Davidson tolerance from 1e-4 to 1e-9 over the next four (sweeps 3-7), so
  until then a sweep's energy is only as sharp as its tolerance and depends
  on the noise draws and on the rounding of the products (the GPU driver
  differs from the oracle by up to 6e-7 at the 1e-7 sweep); the sweeps from
  the ninth on (tolerance 1e-9 after a sweep at 1e-9) and the final energy
  are compared.  The reference builds a first MPS only in its
  dense-vector mode, so the driver runs with ``ifQt = False``: Davidson
  vectors (and their random start noise) in the reference's dense order, the
  engine's block-sparse products underneath.
"""
import os

import numpy
import pytest

from tests.problems import (random_problem, class_covering_terms, oracle_subset_driver,
                            oracle_sigma_subset, product_sigma_subset)

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")

SIGMA_K24 = dict(K=24, nelec=24, D=512, isite=11, seed=2024)
SIGMA_SP_K20 = dict(K=20, nelec=20, D=512, isite=9, seed=2024, npts=8, sval=0.0)
TOL = {"fp64": 1e-10, "split": 1e-8, "emu64": 1e-10}


def rel(a, b):
    return numpy.linalg.norm(a - b) / max(numpy.linalg.norm(b), 1e-300)


def _subset_parity(cfg, per_class, seed):
    P = random_problem(with_oracle=False, **cfg)
    terms, classes = class_covering_terms(P, per_class)
    assert len(classes) >= 4
    m = oracle_subset_driver(P, terms)
    x = numpy.random.default_rng(seed).standard_normal(P.ndim0)
    ref = oracle_sigma_subset(P, terms, x, m)
    assert numpy.linalg.norm(ref) > 0
    errs = {prec: rel(product_sigma_subset(P, terms, x, prec), ref) for prec in TOL}
    return errs, terms, classes


def test_sigma_k24_d512_term_subset(gpu):
    errs, terms, classes = _subset_parity(SIGMA_K24, 1, 31)
    for prec, tol in TOL.items():
        assert errs[prec] < tol, (prec, errs[prec], terms)


def test_sigma_spin_projected_k20_d512_term_subset(gpu):
    errs, terms, classes = _subset_parity(SIGMA_SP_K20, 1, 32)
    # the middle term of each class: the rotation angle varies over the subset
    for prec, tol in TOL.items():
        assert errs[prec] < tol, (prec, errs[prec], terms)


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_sweep_k10_d64_matches_oracle_driver(gpu, precision):
    from oracle import integrals as oint
    from zmpo_dmrg_gb300.mpo_dmrg_class import mpo_dmrg
    from zmpo_dmrg_gb300.mpo_dmrg_schedule import schedule
    z = numpy.load(os.path.join(GOLD, "sweep_k10_d64.npz"))
    K, nelec, D = int(z["K"]), int(z["nelec"]), int(z["D"])
    h, eri, _ = oint.synthetic(K, int(z["seed"]))
    i1, i2, _ = oint.to_spin_orbital(h, eri)
    m = mpo_dmrg(seed=int(z["driver_seed"]))
    m.nsite, m.sbas, m.isym = K, 2 * K, 2
    m.build()
    m.occun = numpy.array([1., 1.] * (nelec // 2) + [0., 0.] * (K - nelec // 2))
    m.qsectors = {str([float(nelec), 0.0]): 1}
    m.precision = precision
    m.ifQt = False
    m.partition()
    m.loadInts((i1, i2))
    m.dumpMPO()
    sc = schedule(maxM=D, tol=float(z["tol"]), maxiter=int(z["maxiter"]))
    sc.normal(2)
    m.default(sc)
    assert m.nsweep == int(z["nsweep"])
    got = numpy.array([float(e) for e in m.eav])
    ref = z["sweep_energies"]
    assert got.shape == ref.shape
    assert numpy.abs(got[8:] - ref[8:]).max() < 1e-8, (got - ref)
    assert abs(float(m.Energy) - float(z["energy"])) < 1e-8
