"""Dense MPO site tensors W_p(i) for H = sum_p a_p^+ V_p (oracle restatement).

Follows the reference ``source/mpo_dmrg_const.py:12-20`` (2x2 local matrices)
and ``source/mpo_dmrg_opers.py`` (``linkTwoOpers`` 43-49, ``genElemSpinMat``
56-66, ``genElemSpatialMat`` 68-72, ``genWfacSpin`` 91-194, ``genHfacSpin``
197-203, ``genHfacSpatial`` 216-219, ``genExpISyPhiMat`` 228-238,
``genHRfacSpatial`` 253-260).  Layout W[a_left, b_right, n_out, n_in].
"""
import math
import numpy

# mpo_dmrg_const.py:12-20 -- spin-orbital local operators, basis [|0>, |1>]
sgn = numpy.array([[1., 0.], [0., -1.]])
idn = numpy.array([[1., 0.], [0., 1.]])
idnt = numpy.array([[1., 0.], [0., -1.]])
cre = numpy.array([[0., 0.], [1., 0.]])
cret = numpy.array([[0., 0.], [1., 0.]])
ann = numpy.array([[0., 1.], [0., 0.]])
annt = numpy.array([[0., -1.], [0., 0.]])
nii = numpy.array([[0., 0.], [0., 1.]])
niit = numpy.array([[0., 0.], [0., -1.]])


def linkTwoOpers(op1, op2):
    """abij,bckl->ac(ik)(jl)  (mpo_dmrg_opers.py:43-49)."""
    op12 = numpy.tensordot(op1, op2, axes=([1], [0]))
    op12 = op12.transpose(0, 3, 1, 4, 2, 5)
    s = op12.shape
    return op12.reshape((s[0], s[1], s[2] * s[3], s[4] * s[5]))


def genElemSpinMat(p, isite, iop=1):
    """mpo_dmrg_opers.py:56-66: JW string left of p, cre/ann at p, identity right."""
    if isite < p:
        return sgn
    if isite == p:
        return cre if iop == 1 else ann
    return idn


def genElemSpatialMat(p, isite, iop):
    """mpo_dmrg_opers.py:68-72."""
    return numpy.kron(genElemSpinMat(p, 2 * isite, iop),
                      genElemSpinMat(p, 2 * isite + 1, iop))


def genWfacSpin(nsite, isite, hq, vqrs):
    """V_p MPO on spin-orbital site ``isite`` (mpo_dmrg_opers.py:91-194).

    ``nsite`` = number of spin orbitals, ``hq[q]`` = h_pq, ``vqrs[q,r,s]`` = V_pqrs.
    """
    ndim1 = 2 * (nsite + 1)
    ndim2 = 2 * (nsite + 1)
    if isite == 0:
        ndim1 = 1
    if isite == nsite - 1:
        ndim2 = 1
    wop = numpy.zeros((ndim1, ndim2, 2, 2))
    diml = isite
    dimr = nsite - isite - 1
    if isite == 0:
        wop[0, 0] = idnt
        off = 1 + dimr
        for rindx, rsite in enumerate(range(isite + 1, nsite)):
            wop[0, off + rindx] = vqrs[isite, isite, rsite] * niit
        off = 1 + 2 * dimr + diml
        wop[0, off] = -ann
        off = 2 + 2 * dimr + 2 * diml
        wop[0, off] = cre
        wop[0, ndim2 - 1] = hq[isite] * ann
    elif isite == nsite - 1:
        wop[0, 0] = hq[isite] * ann
        wop[1, 0] = cre
        wop[2, 0] = ann
        for jsite in range(isite):
            wop[3 + jsite, 0] = vqrs[isite, jsite, isite] * nii
        wop[ndim1 - 1, 0] = idn
    else:
        # row 1
        wop[0, 0] = idnt
        off = 1 + dimr
        for rindx, rsite in enumerate(range(isite + 1, nsite)):
            wop[0, off + rindx] = vqrs[isite, isite, rsite] * niit
        off = 1 + 2 * dimr + diml
        wop[0, off] = -ann
        off = 2 + 2 * dimr + 2 * diml
        wop[0, off] = cre
        wop[0, ndim2 - 1] = hq[isite] * ann
        # row 2
        wop[1, ndim2 - 1] = cre
        # row 3
        for rindx, rsite in enumerate(range(isite + 1, nsite)):
            wop[2 + rindx, 1 + rindx] = idnt
        # row 4
        wop[2 + dimr, ndim2 - 1] = ann
        # row 5
        offl = 3 + dimr
        offr = 1 + dimr
        for rindx, rsite in enumerate(range(isite + 1, nsite)):
            wop[offl + rindx, offr + rindx] = idnt
        # row 6
        offl = 3 + 2 * dimr
        for lsite in range(isite):
            for rindx, rsite in enumerate(range(isite + 1, nsite)):
                wop[offl + lsite, 1 + rindx] = -vqrs[rsite, lsite, isite] * annt
        offr = 1 + dimr
        for lsite in range(isite):
            for rindx, rsite in enumerate(range(isite + 1, nsite)):
                wop[offl + lsite, offr + rindx] = vqrs[isite, lsite, rsite] * cret
        offr = 1 + 2 * dimr
        for lsite in range(isite):
            wop[offl + lsite, offr + lsite] = idn
        for lsite in range(isite):
            wop[offl + lsite, ndim2 - 1] = vqrs[isite, lsite, isite] * nii
        # row 7
        offl = 3 + 2 * dimr + diml
        offr = 1 + dimr
        for lsite in range(isite):
            for rindx, rsite in enumerate(range(isite + 1, nsite)):
                wop[offl + lsite, offr + rindx] = vqrs[lsite, isite, rsite] * annt
        offr = 2 + 2 * dimr + diml
        for lsite in range(isite):
            wop[offl + lsite, offr + lsite] = idn
        # row 8
        wop[ndim1 - 1, ndim2 - 1] = idn
    return wop


def genHfacSpin(p, nsite, isite, hq, vqrs):
    """H_p = a_p^+ V_p on one spin-orbital site (mpo_dmrg_opers.py:197-203)."""
    wfac = genWfacSpin(nsite, isite, hq, vqrs)
    elem = genElemSpinMat(p, isite)
    hfac = numpy.tensordot(wfac, elem, axes=([2], [1]))
    return hfac.transpose(0, 1, 3, 2).copy()


def genHfacSpatial(p, nsite, isite, hq, vqrs):
    """Spatial site = spin sites (2i, 2i+1) linked (mpo_dmrg_opers.py:216-219)."""
    op1 = genHfacSpin(p, nsite, 2 * isite, hq, vqrs)
    op2 = genHfacSpin(p, nsite, 2 * isite + 1, hq, vqrs)
    return linkTwoOpers(op1, op2)


def genExpISyPhiMat(phi):
    """exp(-i phi S_y) on the spatial basis [0, b, a, ab] (mpo_dmrg_opers.py:228-238)."""
    expm = numpy.zeros((4, 4))
    expm[0, 0] = 1.0
    c = math.cos(0.5 * phi)
    s = math.sin(0.5 * phi)
    expm[1, 1] = c
    expm[1, 2] = s
    expm[2, 1] = -s
    expm[2, 2] = c
    expm[3, 3] = 1.0
    return expm


def genHRfacSpatial(pindx, nsite, isite, int1e, int2e, qpts, pdic):
    """H_p (times R(theta) for spin projection) (mpo_dmrg_opers.py:253-260)."""
    porb, ipop = pindx
    idx = pdic[porb]
    wop = genHfacSpatial(porb, nsite, isite, int1e[idx], int2e[idx])
    if ipop is not None:
        pop = genExpISyPhiMat(qpts[ipop])
        wop = numpy.tensordot(wop, pop, axes=([3], [0]))
    return wop
