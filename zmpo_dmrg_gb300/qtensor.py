"""Block-sparse (Abelian quantum-number) tensor, host side.

Mirrors the reference ``qtensor`` API (source/qtensor/qtensor.py: ``fromQsyms``
272, ``fromDenseTensor`` 355, ``toDenseTensor`` 381, ``toDenseDiag`` 400,
``prjmap`` 442, ``reduceQsymsToN`` 528, ``projectionNMs`` 546,
``tensordotSYM`` 563, ``tensordotCAL`` 642) with the same packed ``value``
layout.  The block rule, packing and contraction task lists are computed by
the engine (``libzmpo_gb300.so``); ``tensordotCAL`` runs on the GPU.
``value`` is a NumPy array on the host or a float64 CUDA tensor.
"""
import numpy

from . import engine as _engine


def classification(qnums, collect=1):
    """Sectors of a list of quantum numbers in order of first appearance
    (qtensor_util.classification, qtensor_util.py:34-51)."""
    q = numpy.asarray(qnums, dtype=numpy.float64)
    if q.ndim == 1:
        q = q.reshape(-1, 1)
    if not collect:
        return q.copy(), numpy.ones(len(q), dtype=numpy.int64), [[i] for i in range(len(q))]
    _, first, inv = numpy.unique(q, axis=0, return_index=True, return_inverse=True)
    inv = inv.reshape(-1)
    order = numpy.argsort(first, kind="stable")
    rank_of = numpy.empty_like(order)
    rank_of[order] = numpy.arange(len(order))
    lab = rank_of[inv]
    idlst = [[] for _ in range(len(order))]
    for i, s in enumerate(lab):
        idlst[s].append(i)
    qsyms = q[first[order]]
    ndims = numpy.array([len(x) for x in idlst], dtype=numpy.int64)
    return qsyms, ndims, idlst


def fromQnums(qnums, ifcollect=None):
    rank = len(qnums)
    ifclt = [1] * rank if ifcollect is None else ifcollect
    cls = [classification(x, c) for x, c in zip(qnums, ifclt)]
    return rank, [c[0] for c in cls], [c[1] for c in cls], [c[2] for c in cls]


class qtensor:
    def __init__(self, status=None):
        self.status = None if status is None else numpy.array(status, dtype=bool)
        self.rank = None
        self.qsyms = None
        self.ndims = None
        self.idlst = None
        self.layout = None
        self.size_allowed = 0
        self.blk_flat = None
        self.blk_off = None
        self.value = None
        self._plan = None

    # ------------------------------------------------------------ structure
    @property
    def nsyms(self):
        return numpy.array([len(d) for d in self.ndims], dtype=numpy.int64)

    @property
    def shape(self):
        return numpy.array([int(numpy.sum(d)) for d in self.ndims], dtype=numpy.int64)

    @property
    def nqnum(self):
        return self.qsyms[0].shape[1]

    def fromQsyms(self, rank, qsyms, ndims, ifallocate=True, idlst=None):
        self.rank = rank
        self.qsyms = [numpy.asarray(q, dtype=numpy.float64).reshape(len(d), -1)
                      for q, d in zip(qsyms, ndims)]
        self.ndims = [numpy.asarray(d, dtype=numpy.int64) for d in ndims]
        if idlst is not None:
            self.idlst = [list(map(list, x)) for x in idlst]
        eng = _engine.get()
        self.layout = eng.layout(self.qsyms, self.ndims, self.status)
        self.size_allowed, self.blk_flat, self.blk_off = eng.layout_blocks(self.layout)
        self.value = numpy.zeros(self.size_allowed) if ifallocate else None
        return 0

    def blocks(self):
        """Yield (sector multi-index, block dims, offset) of allowed blocks."""
        nsyms = tuple(int(x) for x in self.nsyms)
        flat = numpy.asarray(self.blk_flat, dtype=numpy.int64)
        if self.rank == 0:
            for off in self.blk_off:
                yield (), (), int(off)
            return
        secs = numpy.unravel_index(flat, nsyms)        # all blocks at once
        dims = [numpy.asarray(self.ndims[i])[secs[i]] for i in range(self.rank)]
        secs = numpy.stack(secs, axis=1).tolist()
        dims = numpy.stack(dims, axis=1).tolist()
        for b, off in enumerate(self.blk_off):
            yield tuple(secs[b]), tuple(dims[b]), int(off)

    def fromDenseTensor(self, val, qnums, ifcollect=None):
        rank, qsyms, ndims, idlst = fromQnums(qnums, ifcollect)
        self.fromQsyms(rank, qsyms, ndims)
        self.fromDense(val, idlst)
        self.idlst = idlst
        return 0

    def fromDense(self, val, idlst):
        val = numpy.asarray(val)
        if val.shape == tuple(int(x) for x in self.shape):
            # one gather through the packed -> dense index map
            self.value = val.reshape(-1)[self.prjmap(idlst)].astype(numpy.float64, copy=False)
            return 0
        out = numpy.zeros(self.size_allowed)
        for sec, dims, off in self.blocks():
            ix = numpy.ix_(*[idlst[i][sec[i]] for i in range(self.rank)])
            out[off:off + int(numpy.prod(dims))] = val[ix].reshape(-1)
        self.value = out
        return 0

    def _host_value(self):
        v = self.value
        if v is None:
            return None
        if not isinstance(v, numpy.ndarray):
            v = v.detach().cpu().numpy()
        return v

    def toDenseTensor(self, idlst):
        v = self._host_value()
        val = numpy.zeros(tuple(int(x) for x in self.shape))
        val.reshape(-1)[self.prjmap(idlst)] = v   # one scatter through the index map
        return val

    def toDenseDiag(self, idlst):
        v = self._host_value()
        val = numpy.zeros(tuple(int(x) for x in self.shape[:-1]))
        for sec, dims, off in self.blocks():
            if sec[-1] != sec[-2]:
                continue
            ix = numpy.ix_(*[idlst[i][sec[i]] for i in range(self.rank - 1)])
            blk = v[off:off + int(numpy.prod(dims))].reshape(dims)
            val[ix] = numpy.einsum('...ii->...i', blk)
        return val

    def prjmap(self, idlst):
        """Dense (row-major, full shape) index of every packed element: per
        block the outer sum of each leg's indices times its dense stride."""
        shape = tuple(int(x) for x in self.shape)
        strides = [1] * self.rank
        for i in range(self.rank - 2, -1, -1):
            strides[i] = strides[i + 1] * shape[i + 1]
        scaled = [[numpy.asarray(ix, dtype=numpy.int64) * strides[i] for ix in idlst[i]]
                  for i in range(self.rank)]
        out = []
        for sec, dims, off in self.blocks():
            acc = numpy.zeros((), dtype=numpy.int64)
            for i in range(self.rank):
                acc = numpy.add.outer(acc, scaled[i][sec[i]])
            out.append(acc.reshape(-1))
        return numpy.concatenate(out) if out else numpy.zeros(0, dtype=numpy.int64)

    def copy_structure(self, other, qsyms=None, status=None):
        """Same packing as ``other`` with replaced quantum numbers / status
        (the reference's in-place flips of ``qsyms``)."""
        self.rank = other.rank
        self.ndims = other.ndims
        self.qsyms = other.qsyms if qsyms is None else [numpy.asarray(q, dtype=float).reshape(len(d), -1)
                                                         for q, d in zip(qsyms, other.ndims)]
        self.status = other.status if status is None else numpy.array(status, dtype=bool)
        self.size_allowed = other.size_allowed
        self.blk_flat = other.blk_flat
        self.blk_off = other.blk_off
        self.idlst = other.idlst
        self.value = other.value
        if qsyms is None and status is None:
            self.layout = other.layout
        else:
            self.layout = _engine.get().derive(other.layout, self.qsyms, self.status)
        return self

    # ------------------------------------------------ N-only relabelling (SP)
    def reduceQsymsToN(self):
        """(N,Sz) -> N labels without moving data (qtensor.py:528-543); the
        packing is unchanged only when each N sector keeps its blocks, which the
        caller must ensure (it holds for the layouts this engine builds)."""
        qt = qtensor(self.status)
        qt.fromQsyms(self.rank, [q[:, :1] for q in self.qsyms], self.ndims, ifallocate=False,
                     idlst=self.idlst)
        src = {tuple(int(s) for s in sec): off for sec, dims, off in self.blocks()}
        v = self._host_value()
        out = numpy.zeros(qt.size_allowed)
        for sec, dims, off in qt.blocks():
            o = src.get(tuple(int(s) for s in sec))
            if o is not None:
                n = int(numpy.prod(dims))
                out[off:off + n] = v[o:o + n]
        qt.value = out
        return qt

    # ----------------------------------------------------------- contraction
    def tensordotSYM(self, qt1, qt2, axes):
        """Output structure + GPU task list of tensordot(qt1, qt2, axes)."""
        i1, i2 = list(axes[0]), list(axes[1])
        e1 = [j for j in range(qt1.rank) if j not in i1]
        e2 = [j for j in range(qt2.rank) if j not in i2]
        s2 = [bool(qt2.status[j]) for j in e2]
        if i1 and bool(qt1.status[i1[0]]) == bool(qt2.status[i2[0]]):
            s2 = [not s for s in s2]
        self.status = numpy.array([bool(qt1.status[j]) for j in e1] + s2, dtype=bool)
        lay_out, pid = _engine.get().contract_plan(qt1.layout, qt2.layout, (i1, i2))
        self.fromQsyms(len(e1) + len(e2), [qt1.qsyms[j] for j in e1] + [qt2.qsyms[j] for j in e2],
                       [qt1.ndims[j] for j in e1] + [qt2.ndims[j] for j in e2], ifallocate=False)
        self._plan = pid
        return len(self.blk_flat)

    def tensordotCAL(self, qt1, qt2, ifc1=False, ifc2=False, precision="fp64"):
        """Numeric contraction on the GPU over the cached task list (real
        tensors: ``ifc1`` / ``ifc2`` are no-ops)."""
        import torch
        a = qt1.value if not isinstance(qt1.value, numpy.ndarray) else torch.from_numpy(qt1.value).cuda()
        b = qt2.value if not isinstance(qt2.value, numpy.ndarray) else torch.from_numpy(qt2.value).cuda()
        out = torch.empty(self.size_allowed, dtype=torch.float64, device=a.device)
        _engine.get().contract_exec(self._plan, a.contiguous(), b.contiguous(), out, precision)
        self.value = out
        return 0
