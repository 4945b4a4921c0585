"""Operator partition and the per-product sum over ranks, on two gloo ranks
(CPU processes): the rank-local partial products over each rank's operator
terms must add up to the full product."""
import os
import socket

import numpy

from zmpo_dmrg_gb300.parallel import partition_sites, partition_ops


def test_partition_matches_reference_rule():
    # parallel_util.py:4-36: size 2 splits at n//size; larger sizes spread the
    # remainder over the first ranks
    assert partition_sites(10, 1, 0) == list(range(10))
    assert partition_sites(10, 2, 0) == [0, 1, 2, 3, 4] and partition_sites(10, 2, 1) == [5, 6, 7, 8, 9]
    got = [partition_sites(10, 4, r) for r in range(4)]
    assert got == [[0, 1, 2], [3, 4, 5], [6, 7], [8, 9]]
    got0 = [partition_sites(10, 4, r, iop=0) for r in range(4)]
    assert sorted(sum(got0, [])) == list(range(10))
    for n in (7, 48, 96):
        for size in (2, 3, 4, 8):
            allops = sum((partition_sites(n, size, r) for r in range(size)), [])
            assert allops == list(range(n))
    assert partition_ops(4, 2, 1, npts=2) == [[2, 0], [2, 1], [3, 0], [3, 1]]


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, size, port, ops_mats, x, out):
    import torch
    import torch.distributed as dist
    from zmpo_dmrg_gb300.parallel import DistributedHVec, partition_sites
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=size)
    mine = partition_sites(len(ops_mats), size, rank)

    def local(v):
        return sum(torch.as_tensor(ops_mats[p]) @ v for p in mine)

    hv = DistributedHVec(local)
    y = hv(torch.as_tensor(x))
    out[rank] = y.numpy().copy()
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_sum_equals_full_product():
    import torch.multiprocessing as mp
    rng = numpy.random.default_rng(0)
    mats = [rng.standard_normal((12, 12)) for _ in range(7)]
    x = rng.standard_normal(12)
    full = sum(m @ x for m in mats)
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, mats, x, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    for r in range(2):
        assert numpy.allclose(out[r], full, atol=1e-12)


def _oracle_worker(rank, size, port, case, x, out):
    """Rank-local sigma of the oracle (the reference's HVecQt restated) over
    this rank's contiguous range of operator terms, summed over ranks."""
    import copy
    import torch
    import torch.distributed as dist
    from oracle import kernel as ok
    from tests.problems import random_problem
    from zmpo_dmrg_gb300.parallel import DistributedHVec, partition_sites
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=size)
    P = random_problem(device=False, **case)
    m = P.o
    mine = partition_sites(m.nops, size, rank)
    view = copy.copy(m)     # this rank's terms, renumbered 0..len(mine)-1
    view.fhop = {"nsite": m.fhop["nsite"], "nops": len(mine), "wts": numpy.asarray(m.hpwts)[mine]}
    for i in range(m.nsite):
        for k, iop in enumerate(mine):
            view.fhop["site%d/op%d" % (i, k)] = m.fhop["site%d/op%d" % (i, iop)]
    view.opers = [m.opers[iop] for iop in mine]
    view.hpwts = numpy.asarray(m.hpwts)[mine]
    view.nops = len(mine)
    view._hvec_templates = None
    fL = {"opers%d" % k: m.flst[0][0]["opers%d" % iop] for k, iop in enumerate(mine)}
    fR = {"opers%d" % k: m.flst[0][1]["opers%d" % iop] for k, iop in enumerate(mine)}

    def local(v):
        return torch.as_tensor(ok.HVecQt(v.numpy(), [view, P.isite, 2, [[fL, fR]], "L", True], P.ndim0, None))

    y = DistributedHVec(local)(torch.as_tensor(x))
    out[rank] = y.numpy().copy()
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_oracle_sigma_equals_full_sigma():
    """The operator partition of a real two-site dot: each rank's oracle sigma
    over its terms, all-reduced, equals the oracle sigma over all terms."""
    import torch.multiprocessing as mp
    from tests.problems import random_problem, oracle_sigma
    case = dict(K=4, nelec=4, D=8, isite=1, seed=5)
    P = random_problem(device=False, **case)
    x = numpy.random.default_rng(4).standard_normal(P.ndim0)
    full = oracle_sigma(P, x)
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_oracle_worker, args=(r, 2, port, case, x, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(300)
        assert p.exitcode == 0
    for r in range(2):
        assert numpy.allclose(out[r], full, rtol=1e-12, atol=1e-12)


def _product_plan_worker(rank, size, port, case, x, out):
    """One CPU rank: the engine's own sigma plan over this rank's operator
    terms (``partition_ops``, the reference's partitionSites rule), executed
    on the host by the NumPy model of the kernels, then summed over ranks."""
    import torch
    import torch.distributed as dist
    from zmpo_dmrg_gb300.parallel import DistributedHVec, partition_ops
    from tests.problems import random_problem, host_sigma_terms
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=size)
    P = random_problem(device=False, **case)
    mine = [o[0] for o in partition_ops(P.o.sbas, size, rank)]
    hv = DistributedHVec(lambda v: torch.as_tensor(host_sigma_terms(P, mine, v.numpy())[0]))
    out[rank] = hv(torch.as_tensor(x)).numpy().copy()
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_product_plans_sum_to_the_oracle_sigma():
    """Each rank plans and runs (on the host) the engine's sigma over its
    range of operator terms; the all-reduced result equals the oracle's
    sigma over every term of the dot."""
    import torch.multiprocessing as mp
    from tests.problems import random_problem, oracle_sigma
    case = dict(K=6, nelec=6, D=16, isite=2, seed=1)
    P = random_problem(device=False, **case)
    x = numpy.random.default_rng(11).standard_normal(P.ndim0)
    ref = oracle_sigma(P, x)
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_product_plan_worker, args=(2, _free_port(), case, x, out), nprocs=2, join=True)
    for r in range(2):
        assert numpy.linalg.norm(out[r] - ref) <= 1e-12 * numpy.linalg.norm(ref)


def test_driver_partition_covers_every_term_once():
    """mpo_dmrg.partition(rank, size): the ranks' operator terms are disjoint
    contiguous blocks that together give every term (with and without spin
    projection), with the matching weights."""
    from zmpo_dmrg_gb300.mpo_dmrg_class import mpo_dmrg
    for npts, sbas, size in [(None, 12, 2), (None, 20, 3), (None, 48, 8), (4, 12, 3)]:
        seen = []
        for rank in range(size):
            m = mpo_dmrg()
            m.nsite, m.sbas, m.isym = sbas // 2, sbas, 2
            if npts:
                m.npts = npts
                m.qwts = numpy.arange(1.0, npts + 1.0)
            m.partition(rank, size)
            assert (m.rank, m.size) == (rank, size)
            assert len(m.hpwts) == len(m.opers) == m.nops
            if npts:
                assert all(w == m.qwts[o[1]] for w, o in zip(m.hpwts, m.opers))
            flat = [o[0] * (npts or 1) + (o[1] or 0) for o in m.opers]
            assert flat == list(range(flat[0], flat[0] + len(flat))) if flat else True
            seen += flat
        assert sorted(seen) == list(range(sbas * (npts or 1)))
