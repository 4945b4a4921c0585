"""Qt (block-sparse) form of the MPO site tensors (oracle restatement).

Follows ``source/qtensor/qtensor_opers.py``: ``case`` 72-90, ``genQphys`` 95-109,
``genElemQnums`` 113-142, ``genWfacSpinQnumsRight`` 161-172, ``genWfacQnums``
175-193, ``genHRfacSpatialQt`` 358-408 (with ``maxslc = 1``),
``genExpISyPhiQt`` 457-469.

Deliberate deviation: ``sortQnums`` (qtensor_opers.py:56-58) orders the MPO
bond quantum numbers by the *string* form of a NumPy row, whose format depends
on the NumPy version.  Here the bond is sorted numerically.  The order only
permutes the MPO bond index (hence the packing of environment blocks); sigma
vectors and energies do not depend on it.
"""
import numpy
from . import mpo
from .qtensor import qtensor


def case(porb, isite, ncsite=1):
    """Operator class of a_p^+ V_p relative to the dot (qtensor_opers.py:72-90)."""
    if porb // 2 < isite:
        icase = 1 if porb % 2 == 1 else 0
    elif porb // 2 == isite:
        icase = 3 if porb % 2 == 1 else 2
    else:
        if ncsite == 1:
            icase = 5 if porb % 2 == 1 else 4
        else:
            if porb // 2 == isite + 1:
                icase = 5 if porb % 2 == 1 else 4
            else:
                icase = 7 if porb % 2 == 1 else 6
    return icase


def genQphys(isym, isite=None):
    """qtensor_opers.py:95-109."""
    if isym == 1:
        if isite % 2 == 0:
            qu = [[0., 0.], [1., 0.5]]
        else:
            qu = [[0., 0.], [1., -0.5]]
        qd = list(qu)
    else:
        qu = [[0., 0.], [1., -0.5], [1., 0.5], [2., 0.]]
        qd = list(qu)
    return numpy.array(qu), numpy.array(qd)


def genElemQnums(p, isite, iop, status='L'):
    """qtensor_opers.py:113-142."""
    spin = 0.5 if p % 2 == 0 else -0.5
    sgn = 1.0 if iop == 1 else -1.0
    nchange = sgn
    schange = sgn * spin
    if isite < p:
        ql = [[0., 0.]]
        qr = [[0., 0.]]
    elif isite == p:
        ql = [[0., 0.]]
        qr = [[nchange, schange]]
    else:
        ql = [[nchange, schange]]
        qr = [[nchange, schange]]
    if status == 'R':
        ql = [[nchange - q[0], schange - q[1]] for q in ql]
        qr = [[nchange - q[0], schange - q[1]] for q in qr]
    return numpy.array(ql), numpy.array(qr)


def genWfacSpinQnumsRight(nsite, isite, sz):
    """qtensor_opers.py:161-172."""
    spins = [0.5, -0.5]
    q0 = [[0., 0.]]
    q1 = [[-2., -sz - spins[i % 2]] for i in range(isite + 1, nsite)]
    q2 = [[0., -sz + spins[i % 2]] for i in range(isite + 1, nsite)]
    q3 = [[-1., -spins[i % 2]] for i in range(isite + 1)]
    q4 = [[1., spins[i % 2]] for i in range(isite + 1)]
    q5 = [[-1., -sz]]
    qnums = q0 + q1 + q2 + q3 + q4 + q5
    assert len(qnums) == 2 * (nsite + 1)
    return numpy.array(qnums)


def genWfacQnums(nsite, isite, isz, status='L'):
    """qtensor_opers.py:175-193."""
    spins = [0.5, -0.5]
    sz = spins[isz]
    if isite == 0:
        ql = [[0., 0.]]
        qr = genWfacSpinQnumsRight(nsite, isite, sz)
    elif isite == nsite - 1:
        ql = genWfacSpinQnumsRight(nsite, isite - 1, sz)
        qr = [[-1., -sz]]
    else:
        ql = genWfacSpinQnumsRight(nsite, isite - 1, sz)
        qr = genWfacSpinQnumsRight(nsite, isite, sz)
    if status == 'R':
        ql = [[-1. - q[0], -sz - q[1]] for q in ql]
        qr = [[-1. - q[0], -sz - q[1]] for q in qr]
    return numpy.array(ql), numpy.array(qr)


def sortQnums(qnums):
    """Numeric order of the bond quantum numbers (see module docstring)."""
    return numpy.array(sorted(range(len(qnums)), key=lambda k: tuple(qnums[k])))


def bond_qnums(p, nsite, isite):
    """Left/right MPO bond quantum numbers of H_p at spatial site ``isite``
    (the qnum part of qtensor_opers.py:358-379)."""
    iop = 1
    isz = p % 2
    ql1e, _ = genElemQnums(p, 2 * isite, iop, 'L')
    _, qr2e = genElemQnums(p, 2 * isite + 1, iop, 'L')
    ql1w, _ = genWfacQnums(nsite, 2 * isite, isz, 'L')
    _, qr2w = genWfacQnums(nsite, 2 * isite + 1, isz, 'L')
    ql = [q1 + q2 for q1 in ql1e for q2 in ql1w]
    qr = [q1 + q2 for q1 in qr2e for q2 in qr2w]
    return ql, qr


def genHRfacSpatialQt(pindx, nsite, isite, int1e, int2e, qpts, pdic):
    """Qt site tensor of H_p [R(theta)] with bond sectors collected and the
    physical legs uncollected (qtensor_opers.py:358-408, maxslc = 1)."""
    p, ip = pindx
    site = mpo.genHRfacSpatial(pindx, nsite, isite, int1e, int2e, qpts, pdic)
    qu, qd = genQphys(2, isite)
    ql, qr = bond_qnums(p, nsite, isite)
    if ip is not None:
        ql = [q[:1] for q in ql]
        qr = [q[:1] for q in qr]
        qu = qu[:, :1]
        qd = qd[:, :1]
    idxl = sortQnums(ql)
    idxr = sortQnums(qr)
    ql = numpy.array(ql)[idxl]
    qr = numpy.array(qr)[idxr]
    site = site[numpy.ix_(idxl, idxr)].copy()
    qt = qtensor([False, True, False, True])
    qt.fromDenseTensor(site, [ql, qr, qu, qd], ifcollect=[1, 1, 0, 0])
    return qt


def genExpISyPhiQt(phi):
    """qtensor_opers.py:457-469."""
    site = mpo.genExpISyPhiMat(phi).reshape(1, 1, 4, 4)
    qt = qtensor([False, True, False, True])
    qu = [[0.], [1.], [1.], [2.]]
    qt.fromDenseTensor(site, [[[0.]], [[0.]], qu, qu], ifcollect=[0, 0, 0, 0])
    return qt
