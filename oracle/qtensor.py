"""Abelian block-sparse tensor (oracle restatement of the reference ``qtensor``).

Follows ``source/qtensor/qtensor.py`` (class ``qtensor``: ``fromQsyms`` 272-346,
``fromDense`` 361-378, ``toDenseTensor`` 381-397, ``toDenseDiag`` 400-410,
``prjmap`` 442-453, ``reduceQsymsToN`` 528-543, ``projectionNMs`` 546-560,
``tensordotSYM`` 563-637, ``tensordotCAL`` 642-659) and
``source/qtensor/qtensor_util.py`` (``classification`` 34-51, ``fromQnums``
20-31, ``blks_allowed0`` 53-67, ``cartesian_prod`` 128-168).

Packed layout: allowed blocks in row-major order of their sector multi-index,
each block row-major.  ``tensordotCAL`` counts 2*m*n*k per task into the
module-level ``FLOPS`` counter (the algorithmic work unit F_ref).
"""
import copy
import numpy

FLOPS = {"count": 0}


def reset_flops():
    FLOPS["count"] = 0


def cartesian_prod(arrays):
    """qtensor_util.py:128-168 (row-major cartesian product, shape (M, n))."""
    arrays = [numpy.asarray(x) for x in arrays]
    if len(arrays) == 0:
        return numpy.zeros((1, 0), dtype=numpy.int64)
    grids = numpy.meshgrid(*arrays, indexing="ij")
    return numpy.stack([g.reshape(-1) for g in grids], axis=1)


def classification(qnums, ifclt=1):
    """Group equal quantum numbers into sectors in order of first appearance
    (qtensor_util.py:34-51)."""
    if ifclt:
        keys = []
        groups = {}
        for idx, val in enumerate(qnums):
            key = tuple(float(x) for x in val)
            if key not in groups:
                groups[key] = []
                keys.append(key)
            groups[key].append(idx)
        # sorted by min index == order of first appearance
        qsyms = numpy.array([list(k) for k in keys], dtype=numpy.float64)
        idlst = [groups[k] for k in keys]
        ndims = numpy.array([len(x) for x in idlst])
    else:
        qsyms = numpy.array(qnums, dtype=numpy.float64)
        idlst = [[i] for i in range(len(qnums))]
        ndims = numpy.array([1] * len(qnums))
    return qsyms, ndims, idlst


def fromQnums(qnums, ifcollect=None):
    """qtensor_util.py:20-31."""
    rank = len(qnums)
    ifclt = [1] * rank if ifcollect is None else ifcollect
    classes = [classification(x, y) for x, y in zip(qnums, ifclt)]
    return (rank, [c[0] for c in classes], [c[1] for c in classes],
            [c[2] for c in classes])


def blks_allowed0(nblks, rank, nqnum, nsyms, status, qsyms):
    """Pure-Python allowed-block rule (qtensor_util.py:53-67)."""
    allowed = numpy.zeros(nblks, dtype=numpy.int32)
    for idx in range(nblks):
        isyms = numpy.unravel_index(idx, nsyms)
        okey = numpy.zeros(nqnum)
        ikey = numpy.zeros(nqnum)
        for i in range(rank):
            if status[i]:
                okey += qsyms[i][isyms[i]]
            else:
                ikey += qsyms[i][isyms[i]]
        if numpy.amax(abs(okey - ikey)) < 1.e-10:
            allowed[idx] = 1
    return allowed


def blks_allowed(nblks, rank, nqnum, nsyms, status, qsyms):
    """Vectorised form of the C rule ``symAllowed`` (ctypes/qsym.c:5-480):
    block allowed iff sum_k |sum_{in} q_k - sum_{out} q_k| < 1e-10."""
    diff = numpy.zeros(tuple(nsyms) + (nqnum,))
    for i in range(rank):
        shp = [1] * rank + [nqnum]
        shp[i] = nsyms[i]
        q = numpy.asarray(qsyms[i], dtype=numpy.float64).reshape(shp)
        if status[i]:
            diff = diff - q
        else:
            diff = diff + q
    dtot = numpy.sum(numpy.abs(diff), axis=-1)
    return (dtot < 1.e-10).astype(numpy.int32).reshape(nblks)


class qtensor:
    def __init__(self, status=None):
        self.rank = None
        self.qsyms = None
        self.ndims = None
        self.nqnum = None
        self.nsyms = None
        self.shape = None
        self.size = None
        self.nblks = None
        self.nblks_allowed = None
        self.iblks_allowed = None
        self.dims_allowed = None
        self.idx_allowed = None
        self.ndim_allowed = None
        self.ioff_allowed = None
        self.size_allowed = None
        self.value = None
        self.status = None if status is None else numpy.array(status)
        self.axes = None
        self.clst = None
        self.idlst = None

    def copy(self, other):
        """qtensor.py:154-184 (structure + value, not clst/idlst)."""
        self.rank = other.rank
        self.nqnum = other.nqnum
        self.size = other.size
        self.nblks = other.nblks
        self.nblks_allowed = other.nblks_allowed
        self.size_allowed = other.size_allowed
        self.qsyms = [q.copy() for q in other.qsyms]
        self.ndims = [n.copy() for n in other.ndims]
        self.nsyms = numpy.array(other.nsyms).copy()
        self.shape = numpy.array(other.shape).copy()
        self.iblks_allowed = other.iblks_allowed.copy()
        self.dims_allowed = other.dims_allowed.copy()
        self.idx_allowed = other.idx_allowed.copy()
        self.ndim_allowed = other.ndim_allowed.copy()
        self.ioff_allowed = other.ioff_allowed.copy()
        self.value = None if other.value is None else other.value.copy()
        self.status = None if other.status is None else other.status.copy()
        self.axes = None
        self.clst = None
        self.idlst = None

    def fromQsyms(self, rank, qsyms, ndims, ifallocate=True, idlst=None):
        """qtensor.py:272-346."""
        self.rank = rank
        self.qsyms = copy.deepcopy([numpy.asarray(q, dtype=numpy.float64) for q in qsyms])
        self.ndims = copy.deepcopy([numpy.asarray(n) for n in ndims])
        if idlst is not None:
            self.idlst = copy.deepcopy(idlst)
        self.nqnum = self.qsyms[0].shape[1]
        self.shape = numpy.array([int(sum(d)) for d in self.ndims])
        self.size = int(numpy.prod(self.shape))
        self.nsyms = numpy.array([q.shape[0] for q in self.qsyms], dtype=numpy.int32)
        self.nblks = int(numpy.prod(self.nsyms))
        assert self.status is not None
        allowed = blks_allowed(self.nblks, self.rank, self.nqnum, self.nsyms,
                               self.status, self.qsyms)
        self.nblks_allowed = int(numpy.sum(allowed))
        self.idx_allowed = numpy.flatnonzero(allowed)
        allowed[self.idx_allowed] = self.idx_allowed + 1
        self.iblks_allowed = allowed.reshape(self.nsyms).copy()
        self.dims_allowed = numpy.array(cartesian_prod(self.ndims), dtype=numpy.int64)
        self.ndim_allowed = numpy.prod(self.dims_allowed, axis=1).astype(numpy.int64)
        self.ioff_allowed = numpy.zeros(self.nblks, dtype=numpy.int64)
        ioff = 0
        for idx in self.idx_allowed:
            self.ioff_allowed[idx] = ioff
            ioff += self.ndim_allowed[idx]
        self.size_allowed = int(ioff)
        self.value = numpy.zeros(self.size_allowed) if ifallocate else None
        return 0

    def fromDenseTensor(self, val, qnums, ifcollect=None):
        """qtensor.py:355-359."""
        rank, qsyms, ndims, idlst = fromQnums(qnums, ifcollect)
        self.fromQsyms(rank, qsyms, ndims)
        self.fromDense(val, idlst)
        self.idlst = copy.deepcopy(idlst)
        return 0

    def fromDense(self, val, idlst):
        for idx in self.idx_allowed:
            ioff = self.ioff_allowed[idx]
            ndim = self.ndim_allowed[idx]
            isyms = numpy.unravel_index(idx, self.nsyms)
            ind = numpy.ix_(*[idlst[i][isyms[i]] for i in range(self.rank)])
            self.value[ioff:ioff + ndim] = val[ind].reshape(ndim)
        return 0

    def toDenseTensor(self, idlst):
        val = numpy.zeros(self.shape)
        for idx in self.idx_allowed:
            ioff = self.ioff_allowed[idx]
            dims = self.dims_allowed[idx]
            ndim = self.ndim_allowed[idx]
            isyms = numpy.unravel_index(idx, self.nsyms)
            ind = numpy.ix_(*[idlst[i][isyms[i]] for i in range(self.rank)])
            val[ind] = self.value[ioff:ioff + ndim].reshape(dims)
        return val

    def toDenseDiag(self, idlst):
        """Diagonal of the last two legs (qtensor.py:400-410)."""
        val = numpy.zeros(self.shape[:-1])
        for idx in self.idx_allowed:
            ioff = self.ioff_allowed[idx]
            dims = self.dims_allowed[idx]
            ndim = self.ndim_allowed[idx]
            isyms = numpy.unravel_index(idx, self.nsyms)
            if isyms[-1] != isyms[-2]:
                continue
            ind = numpy.ix_(*[idlst[i][isyms[i]] for i in range(self.rank - 1)])
            val[ind] = numpy.einsum('...ii->...i',
                                    self.value[ioff:ioff + ndim].reshape(dims))
        return val

    def prjmap(self, idlst):
        """Packed position -> dense flat index (qtensor.py:442-453)."""
        out = []
        for idx in self.idx_allowed:
            isyms = numpy.unravel_index(idx, self.nsyms)
            indices = [idlst[i][isyms[i]] for i in range(self.rank)]
            ntuple = cartesian_prod(indices)
            out.append(numpy.ravel_multi_index(tuple(ntuple.T), self.shape))
        if not out:
            return numpy.zeros(0, dtype=numpy.int64)
        return numpy.concatenate(out)

    def reduceQsymsToN(self):
        """(N,Sz) -> N relabelling without moving data (qtensor.py:528-543)."""
        qt = qtensor(self.status)
        qsyms = [q[:, 0:1] for q in self.qsyms]
        qt.fromQsyms(self.rank, qsyms, self.ndims, idlst=self.idlst)
        for idx in self.idx_allowed:
            ioff = self.ioff_allowed[idx]
            ndim = self.ndim_allowed[idx]
            isyms = numpy.unravel_index(idx, self.nsyms)
            idx_new = qt.iblks_allowed[isyms] - 1
            ioff_new = qt.ioff_allowed[idx_new]
            assert ndim == qt.ndim_allowed[idx_new]
            qt.value[ioff_new:ioff_new + ndim] = self.value[ioff:ioff + ndim]
        return qt

    def projectionNMs(self, qsyms0):
        """Inverse of reduceQsymsToN onto target (N,Sz) blocks (qtensor.py:546-560)."""
        qt = qtensor(self.status)
        qt.fromQsyms(self.rank, qsyms0, self.ndims)
        for idx in qt.idx_allowed:
            ioff = qt.ioff_allowed[idx]
            ndim = qt.ndim_allowed[idx]
            isyms = numpy.unravel_index(idx, qt.nsyms)
            idx_old = self.iblks_allowed[isyms] - 1
            ioff_old = self.ioff_allowed[idx_old]
            assert ndim == self.ndim_allowed[idx_old]
            qt.value[ioff:ioff + ndim] = self.value[ioff_old:ioff_old + ndim]
        return qt

    def tensordotSYM(self, qt1, qt2, axes):
        """Symbolic contraction: output structure + task list (qtensor.py:563-637)."""
        r1 = range(qt1.rank)
        r2 = range(qt2.rank)
        i1, i2 = list(axes[0]), list(axes[1])
        e1 = sorted(set(r1) - set(i1))
        e2 = sorted(set(r2) - set(i2))
        ne1 = len(e1)
        nii = len(i1)
        for a, b in zip(i1, i2):
            assert numpy.array_equal(qt1.qsyms[a], qt2.qsyms[b])
        extqsyms12 = [qt1.qsyms[i] for i in e1] + [qt2.qsyms[i] for i in e2]
        extndims12 = [qt1.ndims[i] for i in e1] + [qt2.ndims[i] for i in e2]
        ints1 = [qt1.status[i] for i in i1]
        ints2 = [qt2.status[i] for i in i2]
        exts1 = [qt1.status[i] for i in e1]
        exts2 = [qt2.status[i] for i in e2]
        if nii != 0:
            if ints1[0] == ints2[0]:
                ints2 = [not x for x in ints2]
                exts2 = [not x for x in exts2]
            for is1, is2 in zip(ints1, ints2):
                assert is1 != is2
        self.status = numpy.array(exts1 + exts2)
        self.fromQsyms(ne1 + len(e2), extqsyms12, extndims12, ifallocate=False)
        self.axes = (i1, i2)
        self.clst = []
        iblks1 = qt1.iblks_allowed.transpose(e1 + i1).copy()
        iblks2 = qt2.iblks_allowed.transpose(e2 + i2).copy()
        for idx in self.idx_allowed:
            ioff = self.ioff_allowed[idx]
            dims = self.dims_allowed[idx]
            ndim = self.ndim_allowed[idx]
            isyms = numpy.unravel_index(idx, self.nsyms)
            nzpt1 = iblks1[isyms[:ne1]]
            nzpt2 = iblks2[isyms[ne1:]]
            nzpt12 = numpy.nonzero(numpy.logical_and(nzpt1, nzpt2))
            for inzpt in zip(*nzpt12):
                idx1 = nzpt1[inzpt] - 1
                idx2 = nzpt2[inzpt] - 1
                self.clst.append([ioff, qt1.ioff_allowed[idx1], qt2.ioff_allowed[idx2],
                                  ndim, qt1.ndim_allowed[idx1], qt2.ndim_allowed[idx2],
                                  dims, qt1.dims_allowed[idx1], qt2.dims_allowed[idx2]])
        return len(self.idx_allowed)

    def tensordotCAL(self, qt1, qt2, ifc1=False, ifc2=False, thresh=1.e-20, tsize=10000):
        """Numeric contraction over the cached task list (qtensor.py:642-659)."""
        self.value = numpy.zeros(self.size_allowed)
        i1 = self.axes[0]
        for item in self.clst:
            ioff, ioff1, ioff2, ndim, ndim1, ndim2, dims, dims1, dims2 = item
            t1 = qt1.value[ioff1:ioff1 + ndim1].reshape(dims1)
            t2 = qt2.value[ioff2:ioff2 + ndim2].reshape(dims2)
            k = int(numpy.prod([dims1[a] for a in i1])) if i1 else 1
            FLOPS["count"] += 2 * (int(ndim1) // k) * (int(ndim2) // k) * k
            if ndim1 > tsize and numpy.max(numpy.abs(t1)) < thresh:
                continue
            if ndim2 > tsize and numpy.max(numpy.abs(t2)) < thresh:
                continue
            self.value[ioff:ioff + ndim] += numpy.tensordot(t1, t2, self.axes).reshape(ndim)
        return 0
