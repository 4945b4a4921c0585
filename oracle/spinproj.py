"""Spin-projection pieces of the oracle (test infrastructure only).

Restates the reference:
  * ``tools/smalld.py:8-40`` (Wigner small-d) and ``mpo_dmrg_util.s2quad``
    (mpo_dmrg_util.py:35-89, Gauss-Legendre branch);
  * ``mpo_dmrg_kernelQt.SVecQt`` (373-450) and ``SDiagQt`` (322-370): the
    overlap S psi = sum_g w_g P_g psi with the bond-1 R(theta) MPO;
  * ``mpo_dmrg_kernelQt.renormQt_S00`` (770-855) and
    ``mpo_dmrg_initQt.genPopsQt`` (347-450): environments of P_g.
Storage: ``flst[0][2:4]`` are the P environments (dict 'opers%d' per point g);
``dmrg.fpop['op%d' % g]`` the R(theta_g) site tensor (same for every site).
"""
import math

import numpy
import scipy.special

from .qtensor import qtensor
from . import qtensor_opers
from .kernel import _flipped


def smalld(j, mp, ms, beta0):
    """Wigner small-d d^j_{mp,ms}(beta) (tools/smalld.py:8-40)."""
    r1, r2, r3 = j - math.floor(j), mp - math.floor(mp), ms - math.floor(ms)
    if abs(r1 - r2) > 1e-10 or abs(r2 - r3) > 1e-10 or abs(r1 - r3) > 1e-10:
        return 0.0
    beta = float(beta0)
    g = scipy.special.gamma
    f1234 = math.sqrt(g(j + mp + 1) * g(j - mp + 1) * g(j + ms + 1) * g(j - ms + 1))
    cb, sb = math.cos(beta / 2.0), math.sin(beta / 2.0)
    val = 0.0
    for s in numpy.arange(0.0, 2 * j + 0.1):
        if j + ms - s > -0.1 and mp - ms + s > -0.1 and j - mp - s > -0.1:
            sgn = math.pow(-1.0, mp - ms + s)
            a = 1.0 / (g(j + ms - s + 1) * g(s + 1) * g(mp - ms + s + 1) * g(j - mp - s + 1))
            val += sgn * a * math.pow(cb, 2 * j + ms - mp - 2 * s) * math.pow(sb, mp - ms + 2 * s)
    return f1234 * val


def s2quad(dmrg, sval=0, sz=0):
    """Gauss-Legendre points beta = acos(x) and weights (2S+1)/2 d^S_{MM} w."""
    assert sval + 1.e-4 > abs(sz)
    xts, wts = numpy.polynomial.legendre.leggauss(dmrg.npts)
    xts = [math.acos(x) for x in xts]
    fac = numpy.array([smalld(sval, sz, sz, x) for x in xts])
    wts = (2. * sval + 1.) / 2.0 * fac * wts
    dmrg.qpts = numpy.array(xts)
    dmrg.qwts = wts
    return xts, wts


def dumpMPO_R(dmrg):
    """R(theta_g) site tensors (mpo_dmrg_io.py:209-229, Qt branch)."""
    dmrg.fpop = {'nops': dmrg.npts, 'wts': dmrg.qwts}
    for g in range(dmrg.npts):
        dmrg.fpop['op%d' % g] = qtensor_opers.genExpISyPhiQt(dmrg.qpts[g])
    return 0


def SVecQt(vec0, info, ndim0, prjmap):
    dmrg, isite, ncsite, flst, status, ifsym = info
    fLp, fRp = flst[0][2:4]
    svec = numpy.zeros(ndim0)
    dmrg.qtmp.value = vec0.copy()
    qvec = dmrg.qtmp.reduceQsymsToN()
    qkey = dmrg.qkey[:1]
    tops = None
    for iop in range(dmrg.npts):
        cop = dmrg.fpop['op%d' % iop]
        lop = fLp['opers%d' % iop]
        rop = fRp['opers%d' % iop]
        flip = _flipped(rop, [-rop.qsyms[0], qkey - rop.qsyms[1], qkey - rop.qsyms[2]])
        if tops is None:
            t1, t2, t3, t4 = qtensor(), qtensor(), qtensor(), qtensor()
            t1.tensordotSYM(lop, qvec, axes=([2], [0]))
            t2.tensordotSYM(t1, cop, axes=([0, 2], [0, 3]))
            if ncsite == 1:
                t3.tensordotSYM(t2, flip, axes=([1, 2], [2, 0]))
            else:
                t3.tensordotSYM(t2, cop, axes=([1, 3], [3, 0]))
                t4.tensordotSYM(t3, flip, axes=([1, 3], [2, 0]))
            tops = (t1, t2, t3, t4)
        t1, t2, t3, t4 = tops
        t1.tensordotCAL(lop, qvec)
        t2.tensordotCAL(t1, cop)
        if ncsite == 1:
            t3.tensordotCAL(t2, rop)
            last = t3
        else:
            t3.tensordotCAL(t2, cop)
            t4.tensordotCAL(t3, rop)
            last = t4
        svec += dmrg.qwts[iop] * last.projectionNMs(dmrg.qtmp.qsyms).value
    return svec


def SDiagQt(info, ndim0, prjmap):
    """diag(S) from the dense diagonals of the P environments and R(theta)
    (mpo_dmrg_kernelQt.py:322-370)."""
    dmrg, isite, ncsite, flst, status, ifsym = info
    fLp, fRp = flst[0][2:4]
    ldim, cdim, rdim, ndim = dmrg.dims
    diag = numpy.zeros(ndim)
    for iop in range(dmrg.npts):
        cop = dmrg.fpop['op%d' % iop]
        lop = fLp['opers%d' % iop]
        rop = fRp['opers%d' % iop]
        cdiag = cop.toDenseDiag(cop.idlst)
        ldiag = lop.toDenseDiag(lop.idlst)
        rdiag = rop.toDenseDiag(rop.idlst)
        tmp = numpy.tensordot(ldiag, cdiag, axes=([0], [0]))
        if ncsite == 1:
            tmp = numpy.tensordot(tmp, rdiag, axes=([1], [0]))
        else:
            tmp = numpy.tensordot(tmp, cdiag, axes=([1], [0]))
            tmp = numpy.tensordot(tmp, rdiag, axes=([2], [0]))
        diag += dmrg.qwts[iop] * tmp.reshape(ndim)
    return diag[prjmap].real.copy()


def renormQt_S00(dmrg, isite, ncsite, flst, flstN, site, status):
    """New P environments for every quadrature point."""
    qsite = site.reduceQsymsToN()
    fN = flstN[0][1]
    tops = None
    if status == 'L':
        fLp = flst[0][2]
        for iop in range(dmrg.npts):
            cop = dmrg.fpop['op%d' % iop]
            top = fLp['opers%d' % iop]
            if tops is None:
                t1, t2, t3 = qtensor(), qtensor(), qtensor()
                t1.tensordotSYM(qsite, top, axes=([0], [1]))
                t2.tensordotSYM(cop, t1, axes=([0, 2], [2, 0]))
                t3.tensordotSYM(t2, qsite, axes=([1, 3], [1, 0]))
                tops = (t1, t2, t3)
            t1, t2, t3 = tops
            t1.tensordotCAL(qsite, top, ifc1=True)
            t2.tensordotCAL(cop, t1)
            t3.tensordotCAL(t2, qsite)
            out = qtensor()
            out.copy(t3)
            out.idlst = [cop.idlst[1], qsite.idlst[2], qsite.idlst[2]]
            fN['opers%d' % iop] = out
    else:
        fRp = flst[0][3]
        for iop in range(dmrg.npts):
            cop = dmrg.fpop['op%d' % iop]
            top = fRp['opers%d' % iop]
            if tops is None:
                fcop = _flipped(cop, [-cop.qsyms[0], -cop.qsyms[1], cop.qsyms[2], cop.qsyms[3]])
                st = cop.status.copy()
                st[0], st[1] = not st[0], not st[1]
                fcop.status = st
                t1, t2, t3 = qtensor(), qtensor(), qtensor()
                t1.tensordotSYM(qsite, top, axes=([2], [1]))
                t2.tensordotSYM(fcop, t1, axes=([1, 2], [2, 1]))
                t3.tensordotSYM(t2, qsite, axes=([1, 3], [1, 2]))
                tops = (t1, t2, t3)
            t1, t2, t3 = tops
            t1.tensordotCAL(qsite, top, ifc1=True)
            t2.tensordotCAL(cop, t1)
            t3.tensordotCAL(t2, qsite)
            out = qtensor()
            out.copy(t3)
            out.idlst = [cop.idlst[0], qsite.idlst[0], qsite.idlst[0]]
            fN['opers%d' % iop] = out
    return 0


def boundary_pops(dmrg):
    """P environment of the empty block: 1 for every point (genBopsQt, N-only)."""
    f = {}
    for iop in range(dmrg.npts):
        t = qtensor([True, False, True])
        t.fromDenseTensor(numpy.ones((1, 1, 1)), [[[0.]], [[0.]], [[0.]]])
        f['opers%d' % iop] = t
    return f
