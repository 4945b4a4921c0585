"""Sigma vector, diagonal and renormalisation kernels (oracle restatement).

Dense ("NQt") forms follow ``source/mpo_dmrg_kernel.py``: ``HDiagNQt`` 53-83,
``linkDiag`` 108-114, ``HVecNQt`` 138-181, ``renormNQt_H00`` 380-409.
Block-sparse ("Qt") forms follow ``source/mpo_dmrg_kernelQt.py``: ``HDiagQt``
30-127, ``HVecQt`` 153-319, ``renormQt_H00`` 633-768 (``maxslc = 1``).

Storage: ``flst[0] = [fL, fR]`` where ``fL['opers%d' % iop]`` is the left
environment of operator ``iop`` (ndarray [a, bra, ket] or ``qtensor``, or None
when the reference would have stored an empty slice); ``dmrg.fhop`` maps
``'site%d/op%d'`` to the MPO site tensor.
"""
import numpy
from .qtensor import qtensor
from . import qtensor_opers


# ----------------------------------------------------------------- dense (NQt)
def linkDiag(cdiag, wdiag):
    cdiag = numpy.tensordot(cdiag, wdiag, axes=([1], [0]))
    cdiag = cdiag.transpose(0, 2, 1, 3)
    s = cdiag.shape
    return cdiag.reshape(s[0], s[1], s[2] * s[3])


def HDiagNQt(info, ndim0, prjmap):
    dmrg, isite, ncsite, flst, status, ifsym = info
    fL, fR = flst[0][0:2]
    ldim, cdim, rdim, ndim = dmrg.dims
    diag = numpy.zeros((ldim, cdim, rdim))
    for iop in range(dmrg.fhop['nops']):
        cop = dmrg.fhop['site%d/op%d' % (isite, iop)]
        cdiag = numpy.einsum('abii->abi', cop)
        if ncsite == 2:
            wop = dmrg.fhop['site%d/op%d' % (isite + 1, iop)]
            cdiag = linkDiag(cdiag, numpy.einsum('bcjj->bcj', wop))
        lop = fL['opers%d' % iop]
        rop = fR['opers%d' % iop]
        ldiag = lop[:, range(ldim), range(ldim)]
        rdiag = rop[:, range(rdim), range(rdim)]
        tmp = numpy.tensordot(ldiag, cdiag, axes=([0], [0]))
        tmp = numpy.tensordot(tmp, rdiag, axes=([1], [0]))
        diag += dmrg.hpwts[iop] * tmp
    return diag.reshape(ndim)[prjmap].real.copy()


def HVecNQt(vec0, info, ndim0, prjmap):
    dmrg, isite, ncsite, flst, status, ifsym = info
    fL, fR = flst[0][0:2]
    ldim, cdim, rdim, ndim = dmrg.dims
    vtensor = numpy.zeros(ndim)
    vtensor[prjmap] = vec0
    nop = dmrg.fhop['nops']
    if ncsite == 1:
        vtensor = vtensor.reshape(ldim, cdim, rdim)
        hvec = numpy.zeros(vtensor.shape)
        for iop in range(nop):
            cop = dmrg.fhop['site%d/op%d' % (isite, iop)]
            lop = fL['opers%d' % iop]
            rop = fR['opers%d' % iop]
            tmp = numpy.tensordot(lop, vtensor, axes=([2], [0]))
            tmp = numpy.tensordot(tmp, cop, axes=([0, 2], [0, 3]))
            tmp = numpy.tensordot(tmp, rop, axes=([1, 2], [2, 0]))
            hvec += dmrg.hpwts[iop] * tmp
    else:
        assert cdim == 16
        vtensor = vtensor.reshape(ldim, 4, 4, rdim)
        hvec = numpy.zeros(vtensor.shape)
        for iop in range(nop):
            cop = dmrg.fhop['site%d/op%d' % (isite, iop)]
            wop = dmrg.fhop['site%d/op%d' % (isite + 1, iop)]
            lop = fL['opers%d' % iop]
            rop = fR['opers%d' % iop]
            tmp = numpy.tensordot(lop, vtensor, axes=([2], [0]))
            tmp = numpy.tensordot(tmp, cop, axes=([0, 2], [0, 3]))
            tmp = numpy.tensordot(tmp, wop, axes=([1, 3], [3, 0]))
            tmp = numpy.tensordot(tmp, rop, axes=([1, 3], [2, 0]))
            hvec += dmrg.hpwts[iop] * tmp
    return hvec.reshape(ndim)[prjmap]


def renormNQt_H00(dmrg, isite, ncsite, flst, flstN, site, status):
    nop = dmrg.fhop['nops']
    fN = flstN[0][0]
    if status == 'L':
        fL = flst[0][0]
        for iop in range(nop):
            cop = dmrg.fhop['site%d/op%d' % (isite, iop)]
            lop = fL['opers%d' % iop]
            tmp = numpy.tensordot(site.conj(), lop, axes=([0], [1]))
            tmp = numpy.tensordot(cop, tmp, axes=([0, 2], [2, 0]))
            tmp = numpy.tensordot(tmp, site, axes=([1, 3], [1, 0]))
            fN['opers%d' % iop] = tmp
    else:
        jsite = isite + ncsite - 1
        fR = flst[0][1]
        for iop in range(nop):
            cop = dmrg.fhop['site%d/op%d' % (jsite, iop)]
            rop = fR['opers%d' % iop]
            tmp = numpy.tensordot(site.conj(), rop, axes=([2], [1]))
            tmp = numpy.tensordot(cop, tmp, axes=([1, 2], [2, 1]))
            tmp = numpy.tensordot(tmp, site, axes=([1, 3], [1, 2]))
            fN['opers%d' % iop] = tmp
    return 0


# ------------------------------------------------------------ block-sparse (Qt)
def _flipped(qt, qsyms):
    """Shallow view of ``qt`` with replaced quantum numbers (the reference
    reassigns ``rop.qsyms`` on a freshly loaded object, mpo_dmrg_kernelQt.py:301)."""
    out = qtensor(qt.status)
    out.__dict__.update(qt.__dict__)
    out.qsyms = qsyms
    return out


def HDiagQt(info, ndim0, prjmap):
    dmrg, isite, ncsite, flst, status, ifsym = info
    fL, fR = flst[0][0:2]
    ldim, cdim, rdim, ndim = dmrg.dims
    diag = numpy.zeros(ndim)
    nop = dmrg.fhop['nops']
    for iop in range(nop):
        lop = fL['opers%d' % iop]
        rop = fR['opers%d' % iop]
        cop = dmrg.fhop['site%d/op%d' % (isite, iop)]
        if lop is None or rop is None:
            continue
        ldiag = lop.toDenseDiag(lop.idlst)
        rdiag = rop.toDenseDiag(rop.idlst)
        cdiag = cop.toDenseDiag(cop.idlst)
        if ncsite == 1:
            tmp = numpy.tensordot(ldiag, cdiag, axes=([0], [0]))
            tmp = numpy.tensordot(tmp, rdiag, axes=([1], [0]))
        else:
            wop = dmrg.fhop['site%d/op%d' % (isite + 1, iop)]
            wdiag = wop.toDenseDiag(wop.idlst)
            tmp = numpy.tensordot(ldiag, cdiag, axes=([0], [0]))
            tmp = numpy.tensordot(tmp, wdiag, axes=([1], [0]))
            tmp = numpy.tensordot(tmp, rdiag, axes=([2], [0]))
        diag += dmrg.hpwts[iop] * tmp.reshape(ndim)
    return diag[prjmap].real.copy()


def HVecQt(vec0, info, ndim0, prjmap):
    dmrg, isite, ncsite, flst, status, ifsym = info
    fL, fR = flst[0][0:2]
    dmrg.qtmp.value = vec0.copy()
    qvec = dmrg.qtmp if not dmrg.ifs2proj else dmrg.qtmp.reduceQsymsToN()
    qkey = dmrg.qkey[:1] if dmrg.ifs2proj else dmrg.qkey
    hvec = numpy.zeros(ndim0)
    tmpl = getattr(dmrg, '_hvec_templates', None)
    key_site = (isite, ncsite, id(dmrg.qtmp))
    if tmpl is None or tmpl[0] != key_site:
        tmpl = (key_site, {})
        dmrg._hvec_templates = tmpl
    tops = tmpl[1]
    nop = dmrg.fhop['nops']
    for iop in range(nop):
        lop = fL['opers%d' % iop]
        rop = fR['opers%d' % iop]
        if lop is None or rop is None:
            continue
        cop = dmrg.fhop['site%d/op%d' % (isite, iop)]
        icase0 = qtensor_opers.case(dmrg.opers[iop][0], isite, ncsite)
        if icase0 not in tops:
            t1 = qtensor()
            ilen1 = t1.tensordotSYM(lop, qvec, axes=([2], [0]))
            t2 = qtensor()
            ilen2 = t2.tensordotSYM(t1, cop, axes=([0, 2], [0, 3])) if ilen1 > 0 else 0
            flip = [-rop.qsyms[0], qkey - rop.qsyms[1], qkey - rop.qsyms[2]]
            if ncsite == 1:
                t3 = qtensor()
                ilen3 = t3.tensordotSYM(t2, _flipped(rop, flip), axes=([1, 2], [2, 0])) \
                    if ilen2 > 0 else 0
                tops[icase0] = (ilen1, ilen2, ilen3, t1, t2, t3, None)
            else:
                wop = dmrg.fhop['site%d/op%d' % (isite + 1, iop)]
                t3 = qtensor()
                t4 = qtensor()
                ilen3 = 0
                if ilen2 > 0:
                    t3.tensordotSYM(t2, wop, axes=([1, 3], [3, 0]))
                    ilen3 = t4.tensordotSYM(t3, _flipped(rop, flip), axes=([1, 3], [2, 0]))
                tops[icase0] = (ilen1, ilen2, ilen3, t1, t2, t3, t4)
        ilen1, ilen2, ilen3, t1, t2, t3, t4 = tops[icase0]
        if ilen1 <= 0 or ilen2 <= 0 or ilen3 <= 0:
            continue
        t1.tensordotCAL(lop, qvec)
        t2.tensordotCAL(t1, cop)
        if ncsite == 1:
            t3.tensordotCAL(t2, rop)
            last = t3
        else:
            wop = dmrg.fhop['site%d/op%d' % (isite + 1, iop)]
            t3.tensordotCAL(t2, wop)
            t4.tensordotCAL(t3, rop)
            last = t4
        if dmrg.ifs2proj:
            hvec += dmrg.hpwts[iop] * last.projectionNMs(dmrg.qtmp.qsyms).value
        else:
            hvec += dmrg.hpwts[iop] * last.value
    return hvec


def renormQt_H00(dmrg, isite, ncsite, flst, flstN, site, status):
    qsite = site if not dmrg.ifs2proj else site.reduceQsymsToN()
    nop = dmrg.fhop['nops']
    fN = flstN[0][0]
    tops = {}
    if status == 'L':
        fL = flst[0][0]
        for iop in range(nop):
            lop = fL['opers%d' % iop]
            cop = dmrg.fhop['site%d/op%d' % (isite, iop)]
            fN['opers%d' % iop] = None
            if lop is None:
                continue
            icase = qtensor_opers.case(dmrg.opers[iop][0], isite)
            if icase not in tops:
                t1, t2, t3 = qtensor(), qtensor(), qtensor()
                t1.tensordotSYM(qsite, lop, axes=([0], [1]))
                t2.tensordotSYM(cop, t1, axes=([0, 2], [2, 0]))
                ilen3 = t3.tensordotSYM(t2, qsite, axes=([1, 3], [1, 0]))
                tops[icase] = (ilen3, t1, t2, t3)
            ilen3, t1, t2, t3 = tops[icase]
            if ilen3 <= 0:
                continue
            t1.tensordotCAL(qsite, lop, ifc1=True)
            t2.tensordotCAL(cop, t1)
            t3.tensordotCAL(t2, qsite)
            out = qtensor()
            out.copy(t3)
            out.idlst = [cop.idlst[1], qsite.idlst[2], qsite.idlst[2]]
            fN['opers%d' % iop] = out
    else:
        jsite = isite + ncsite - 1
        fR = flst[0][1]
        for iop in range(nop):
            rop = fR['opers%d' % iop]
            cop = dmrg.fhop['site%d/op%d' % (jsite, iop)]
            fN['opers%d' % iop] = None
            if rop is None:
                continue
            icase = qtensor_opers.case(dmrg.opers[iop][0], jsite)
            if icase not in tops:
                fcop = _flipped(cop, [-cop.qsyms[0], -cop.qsyms[1],
                                      cop.qsyms[2], cop.qsyms[3]])
                st = cop.status.copy()
                st[0] = not st[0]
                st[1] = not st[1]
                fcop.status = st
                t1, t2, t3 = qtensor(), qtensor(), qtensor()
                t1.tensordotSYM(qsite, rop, axes=([2], [1]))
                t2.tensordotSYM(fcop, t1, axes=([1, 2], [2, 1]))
                ilen3 = t3.tensordotSYM(t2, qsite, axes=([1, 3], [1, 2]))
                tops[icase] = (ilen3, t1, t2, t3)
            ilen3, t1, t2, t3 = tops[icase]
            if ilen3 <= 0:
                continue
            t1.tensordotCAL(qsite, rop, ifc1=True)
            t2.tensordotCAL(cop, t1)
            t3.tensordotCAL(t2, qsite)
            out = qtensor()
            out.copy(t3)
            out.idlst = [cop.idlst[0], qsite.idlst[0], qsite.idlst[0]]
            fN['opers%d' % iop] = out
    return 0


# ------------------------------------------------------------- dispatchers
def HVec(vec0, info, ndim0, prjmap):
    """mpo_dmrg_kernel.py:117-136 (no PT shift)."""
    if info[0].ifQt:
        return HVecQt(vec0, info, ndim0, prjmap)
    return HVecNQt(vec0, info, ndim0, prjmap)


def HDiag(info, ndim0, prjmap):
    """mpo_dmrg_kernel.py:41-51."""
    if info[0].ifQt:
        return HDiagQt(info, ndim0, prjmap)
    return HDiagNQt(info, ndim0, prjmap)


def renorm(dmrg, isite, ncsite, flst, flstN, site, status):
    """mpo_dmrg_kernel.py:347-377 (Hamiltonian environments only)."""
    if dmrg.ifQt:
        renormQt_H00(dmrg, isite, ncsite, flst, flstN, site, status)
    else:
        renormNQt_H00(dmrg, isite, ncsite, flst, flstN, site, status)
    return 0
