"""Full two-site DMRG sweeps with the hot path on the GPU (driver with the
reference's API): the reference's K=6 FCIDUMP must reach the FCI energy and
the BLOCK M=1000 energy recorded in the reference's dmrg.out; the split
(BF16 tensor-core) path must reach the FP64 path's energy within 1e-8 Eh;
seeded synthetic K=6 problems must reach their FCI energies."""
import os

import numpy
import pytest

from oracle import integrals as oint

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _run(int1e, int2e, K, nelec, occ, maxM, tol, maxiter, precision="fp64", seed=1, noise=0.0):
    from zmpo_dmrg_gb300.mpo_dmrg_class import mpo_dmrg
    from zmpo_dmrg_gb300.mpo_dmrg_schedule import schedule
    m = mpo_dmrg(seed=seed)
    m.nsite, m.sbas, m.isym = K, 2 * K, 2
    m.build()
    m.occun = occ
    m.qsectors = {str([float(nelec), 0.0]): 1}
    m.precision = precision
    m.partition()
    m.loadInts((int1e, int2e))
    m.dumpMPO()
    sc = schedule(maxM=maxM, tol=tol, maxiter=maxiter)
    sc.startNoise = noise
    sc.normal(2)
    m.default(sc)
    return m


def test_fcidump_energy(gpu):
    z = numpy.load(os.path.join(GOLD, "h6p_doublet_fcidump.npz"))
    i1, i2, g = oint.to_spin_orbital(z["h1e"], z["eri"])
    efci = oint.fci_energy(i1, g, 6, 0.0)[0]
    occ = numpy.array([1., 1.] * 3 + [0., 0.] * 3)
    m = _run(i1, i2, 6, 6, occ, 64, 1e-9, 10)
    assert abs(m.Energy - efci) < 1e-9
    assert abs(m.Energy + float(z["ecore"]) - float(z["e_block"])) < 5e-9
    ms = _run(i1, i2, 6, 6, occ, 64, 1e-9, 10, precision="split")
    assert abs(ms.Energy - m.Energy) < 1e-8


@pytest.mark.parametrize("hop,seed", [(1.0, 21), (0.7, 5)])
def test_synthetic_k6_reaches_fci(gpu, hop, seed):
    """Seeded synthetic integrals of the benchmark generator; D = 64 is exact
    for K = 6, so every implementation must land on the FCI energy."""
    K = 6
    h, eri, _ = oint.synthetic(K, seed, hop)
    i1, i2, g = oint.to_spin_orbital(h, eri)
    efci = oint.fci_energy(i1, g, 6, 0.0)[0]
    occ = numpy.array([1., 1.] * 3 + [0., 0.] * 3)
    m = _run(i1, i2, K, 6, occ, 64, 1e-9, 10)
    assert abs(m.Energy - efci) < 1e-9
    ms = _run(i1, i2, K, 6, occ, 64, 1e-9, 10, precision="split")
    assert abs(ms.Energy - efci) < 1e-8


def test_default_noise_schedule_k8(gpu):
    """The reference's default schedule (perturbed density-matrix noise 1e-4 in
    the first sweeps) with truncation: FP64 and split runs reach the same
    energy, and the oracle with the same schedule agrees."""
    from oracle import dmrg as od
    K = 8
    h, eri, _ = oint.synthetic(K, 21)
    i1, i2, _ = oint.to_spin_orbital(h, eri)
    occ = numpy.array([1., 1.] * 4 + [0., 0.] * 4)
    m = _run(i1, i2, K, 8, occ, 48, 1e-9, 10, noise=1e-4)
    ms = _run(i1, i2, K, 8, occ, 48, 1e-9, 10, precision="split", noise=1e-4)
    assert abs(ms.Energy - m.Energy) < 1e-8
    o = od.mpo_dmrg(seed=1)
    o.nsite, o.sbas, o.isym = K, 2 * K, 2
    o.build()
    o.occun = occ
    o.qsectors = {str([8.0, 0.0]): 1}
    o.partition()
    o.loadInts(i1, i2)
    o.dumpMPO()
    sc = od.schedule(maxM=48, tol=1e-9, maxiter=10)
    sc.normal(2)
    o.default(sc)
    assert abs(o.Energy - m.Energy) < 1e-7


def _rank_sweep(rank, size, port, out):
    """One rank of a partitioned sweep: this process holds the operator terms
    of its block (the reference's partitionSites rule); H.psi, its diagonal,
    the noise density matrix and MPS energies are summed over the ranks
    through gloo on the host."""
    import os as _os
    import torch
    import torch.distributed as dist
    _os.environ["MASTER_ADDR"] = "127.0.0.1"
    _os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=size)
    torch.cuda.set_device(0)
    K = 6
    h, eri, _ = oint.synthetic(K, 21, 1.0)
    i1, i2, _ = oint.to_spin_orbital(h, eri)
    occ = numpy.array([1., 1.] * 3 + [0., 0.] * 3)
    m = _run(i1, i2, K, 6, occ, 64, 1e-9, 10, noise=1e-4)
    out[rank] = (float(m.Energy), len(m.opers), m.nsweep)
    dist.barrier()
    dist.destroy_process_group()


def test_partitioned_sweep_two_ranks(gpu):
    """Two processes on one GPU, each with half of the 12 operator terms
    (their kernels independent; the only coupling is the gloo all-reduce of
    the partial vectors on the host): the default noisy schedule at the
    exact D = 64 reaches the FCI energy on both ranks, equal to the
    one-process run."""
    import socket
    import torch.multiprocessing as mp
    K = 6
    h, eri, _ = oint.synthetic(K, 21, 1.0)
    i1, i2, g = oint.to_spin_orbital(h, eri)
    efci = oint.fci_energy(i1, g, 6, 0.0)[0]
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    procs = [ctx.Process(target=_rank_sweep, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=600)
    for p in procs:
        assert p.exitcode == 0
    (e0, n0, s0), (e1, n1, s1) = out[0], out[1]
    assert n0 + n1 == 2 * K and n0 == n1 == K
    assert abs(e0 - e1) < 1e-12
    assert abs(e0 - efci) < 1e-8
