"""Operator-level data parallelism (the reference's only parallel strategy).

The 2K (or npts * 2K) terms H_p are block-partitioned over ranks
(``tools/parallel_util.partitionSites``, parallel_util.py:4-36, and ``unrank``
39-42, as used by ``mpo_dmrg_class.partition`` 206-246).  Each rank keeps only
its own environments and computes a partial H.psi over its terms; one sum over
ranks per product (the reference's ``comm.Reduce``, tools/pdvdson.py:75) gives
the full vector on every rank, so the Davidson subspace work is replicated
instead of broadcast.  Renormalisation needs no communication.  On GPUs the sum
is an NCCL all-reduce of the float64 vector; with the gloo backend (CPU ranks,
or ranks sharing a device) the vector goes through host memory.
"""


def partition_sites(nsites, size, rank, iop=1):
    """Contiguous block of ``range(nsites)`` owned by ``rank``."""
    block = nsites // size
    sites = list(range(nsites))
    if size == 1:
        return sites
    if size == 2:
        return sites[:block] if rank == 0 else sites[block:]
    nres = nsites % size
    parts = [block] * size
    if nres:
        if iop == 0:
            nl = nres // 2
            res = [1] * nl + [0] * (size - nres) + [1] * (nres - nl)
        else:
            res = [1] * nres + [0] * (size - nres)
        parts = [p + r for p, r in zip(parts, res)]
    if rank == 0:
        return sites[:parts[0]]
    if rank == size - 1:
        return sites[nsites - parts[-1]:]
    off = sum(parts[:rank])
    return sites[off:off + parts[rank]]


def partition_ops(sbas, size, rank, npts=None):
    """Operator terms [p, ipt] of ``rank`` (ipt None without spin projection)."""
    if npts is None:
        return [[x, None] for x in partition_sites(sbas, size, rank)]
    return [[x // npts, x % npts] for x in partition_sites(npts * sbas, size, rank)]


class DistributedHVec:
    """Wrap a rank-local product (sum over the rank's terms) into the full
    product: one all-reduce (sum) per call over ``group``."""

    def __init__(self, local_mvp, group=None):
        self.local = local_mvp
        self.group = group

    def __call__(self, vec, *info):
        import torch
        y = self.local(vec, *info)
        was_numpy = not isinstance(y, torch.Tensor)
        t = torch.as_tensor(y) if was_numpy else y
        allreduce_(t, self.group)
        return t.numpy() if was_numpy else t


def world(group=None):
    """(rank, size) of this process in ``group`` (0, 1 without torch.distributed)."""
    try:
        import torch.distributed as dist
    except ImportError:
        return 0, 1
    if not (dist.is_available() and dist.is_initialized()):
        return 0, 1
    return dist.get_rank(group), dist.get_world_size(group)


def allreduce_(t, group=None):
    """Sum ``t`` (a torch tensor or a NumPy array) over the ranks of
    ``group``, in place; a no-op on one rank.  Under the gloo backend a
    device tensor is summed through a host copy."""
    import torch
    import torch.distributed as dist
    rank, size = world(group)
    if size <= 1:
        return t
    if not isinstance(t, torch.Tensor):
        dist.all_reduce(torch.from_numpy(t), op=dist.ReduceOp.SUM, group=group)
        return t
    if t.is_cuda and dist.get_backend(group) == "gloo":
        h = t.cpu()
        dist.all_reduce(h, op=dist.ReduceOp.SUM, group=group)
        t.copy_(h)
    else:
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return t
