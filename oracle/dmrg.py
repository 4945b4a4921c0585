"""Two-site / one-site DMRG sweep driver (oracle restatement, single process).

Follows the reference:
  * ``mpo_dmrg_class.py``: ``mpo_dmrg.__init__`` 47-192, ``partition`` 206-246,
    ``build`` 279-297, ``initStates`` 299-326, ``default`` 329-434,
    ``checkMPS`` 470-558;
  * ``mpo_dmrg_schedule.py``: ``getParameters`` 37-84, ``checkConv`` 87-97,
    ``fixed`` 100-125, ``normal`` 129-168;
  * ``mpo_dmrg_opt.py``: ``sweep`` 31-95, ``checkOpers`` 153-193,
    ``sweep_updateSite`` 313-344, ``sweep_updateBoundary`` 347-377;
  * ``mpo_dmrg_dot.py``: ``ci_solver`` 24-112;
  * ``mpo_dmrg_dotutil.py``: ``genDimensions`` 54-80, ``setupQlst`` 83-97,
    ``dptSymmetry`` 105-145, ``symmetrySpaceInfo`` 148-189, ``setupQtmpCI``
    192-203, ``genHDiag`` 206-231, ``finalizeDot`` 259-285, ``decimation``
    288-495, ``genGuess`` 498-559;
  * ``mpo_dmrg_qparser.py``: ``rdm_blkdiag`` 106-183;
  * ``mpo_dmrg_kernel.py``: ``pRDMNQt`` 285-344 (used for both storage forms:
    block-sparse environments are expanded to dense, which gives the same
    matrix as ``pRDMQt``, mpo_dmrg_kernelQt.py:453-626);
  * ``mpo_dmrg_init.py`` / ``mpo_dmrg_initQt.py``: ``genBops`` / ``genHops``;
  * ``mpo_dmrg_util.py``: ``mps0occun`` 118-155, ``initMPS`` 158-190,
    ``initOps`` 193-275;
  * ``mpo_dmrg_qphys.py``: ``vacuum``, ``initSpatialOrb``, ``dpt``;
  * ``tools/pdvdson.py``: ``eigenSolver.solve_iter`` 90-330, ``genOrthoBas``
    335-347, ``dvdson_ortho`` 350-390.
HDF5 files become dicts; MPI is a single process; random noise comes from a
seeded ``numpy.random.Generator`` held on the driver object.
"""
import copy
import math
import numpy
import scipy.linalg

from . import mpo as mpo_opers
from . import qtensor_opers
from . import kernel
from .qtensor import qtensor, fromQnums


# ------------------------------------------------------------- quantum numbers
def vacuum(isym=2):
    return [[0.]] if isym == 1 else [[0., 0.]]


def dpt(q1, q2):
    return [[qi[k] + qj[k] for k in range(len(qi))] for qi in q1 for qj in q2]


def initSpatialOrb(norb, isym=2):
    """mpo_dmrg_qphys.py:127-151: [0, b, a, ab] per spatial orbital."""
    spin = [[[0., 0.], [1., 0.5]], [[0., 0.], [1., -0.5]]]
    out = []
    for _ in range(norb):
        q = dpt(spin[0], spin[1])
        if isym == 1:
            q = [[x[0]] for x in q]
        out.append(q)
    return out


# ---------------------------------------------------------------- schedule
class schedule:
    def __init__(self, maxM=1000, tol=1.e-7, maxiter=40):
        self.maxM = maxM
        self.tol = tol
        self.maxiter = maxiter
        self.startM = None
        self.startTol = 1.e-4
        self.startNoise = 1.e-4
        self.coff = 2
        self.change = None
        self.Tag = None
        self.Sweeps = []
        self.MaxMs = []
        self.Tols = []
        self.Noises = []

    def getParameters(self, dmrg, isweep):
        if self.Tag == 'Normal0':
            if isweep < self.change:
                idx = min(len(self.MaxMs) - 1, isweep)
                dmrg.ncsite = 2
                dmrg.Dmax, dmrg.crit_e, dmrg.noise = self.MaxMs[idx], self.Tols[idx], self.Noises[idx]
            else:
                dmrg.ncsite = 1
                dmrg.Dmax, dmrg.crit_e, dmrg.noise = self.MaxMs[-1], self.Tols[-1], self.Noises[-1]
                if isweep == self.change:
                    dmrg.psi0 = None
        elif self.Tag in ('Normal1', 'Normal2'):
            dmrg.ncsite = 1 if self.Tag == 'Normal1' else 2
            idx = min(len(self.MaxMs) - 1, isweep)
            dmrg.Dmax, dmrg.crit_e, dmrg.noise = self.MaxMs[idx], self.Tols[idx], self.Noises[idx]
        elif self.Tag in ('Fixed1', 'Fixed2'):
            dmrg.ncsite = 1 if self.Tag == 'Fixed1' else 2
            dmrg.Dmax, dmrg.crit_e, dmrg.noise = self.MaxMs[-1], self.Tols[-1], self.Noises[-1]
        else:
            raise ValueError('no such Tag: %r' % self.Tag)
        return 0

    def checkConv(self, dmrg, isweep, deltaE):
        if self.Tag in ('Normal0', 'Normal1', 'Normal2'):
            return isweep > self.change and abs(deltaE) < self.tol
        return abs(deltaE) < self.tol

    def fixed(self, ncsite=2, maxM=None, tol=None, maxiter=None, noise=1.e-4):
        self.Tag = 'Fixed1' if ncsite == 1 else 'Fixed2'
        self.Sweeps = [0]
        if maxM is not None:
            self.maxM = maxM
        self.MaxMs = [self.maxM]
        if tol is not None:
            self.tol = tol
        self.Tols = [self.tol]
        if maxiter is not None:
            self.maxiter = maxiter
        self.Noises = [noise]
        self.change = 0
        return 0

    def normal(self, iop=0):
        self.Sweeps, self.MaxMs, self.Tols, self.Noises = [], [], [], []
        self.Tag = ['Normal0', 'Normal1', 'Normal2'][iop]
        if self.startM is None:
            self.startM = min(max(int(1.5 * math.sqrt(self.maxM)), 25), self.maxM)
        startM = min(self.startM, self.maxM)
        nsweep = 0
        Tol = self.startTol
        Noise = self.startNoise
        while startM < self.maxM:
            self.Sweeps.append(nsweep)
            self.MaxMs.append(startM)
            self.Tols.append(Tol)
            self.Noises.append(Noise)
            nsweep += 1
            startM *= 2
        iNoise = 0
        while Tol >= self.tol:
            self.Sweeps.append(nsweep)
            self.MaxMs.append(self.maxM)
            self.Tols.append(Tol)
            self.Noises.append(Noise)
            nsweep += 1
            Tol /= 10.0
            iNoise += 1
            if iNoise == 1:
                Noise = 0.0
        self.change = nsweep + self.coff
        return 0


# ------------------------------------------------------------------ Davidson
def dvdson_ortho(vbas, rbas, crit_indp):
    nres = rbas.shape[0]
    nindp = 0
    vbas2 = numpy.zeros(rbas.shape)
    rbas = rbas.copy()
    for _ in range(5):
        rbas = rbas - rbas.dot(vbas.T).dot(vbas)
    for i in range(nres):
        rvec = rbas[i, :].copy()
        rii = numpy.linalg.norm(rvec)
        if rii <= crit_indp:
            continue
        rvec = rvec / rii
        rvec = rvec / numpy.linalg.norm(rvec)
        vbas2[nindp] = rvec
        nindp += 1
        for _ in range(5):
            rbas[i:, :] -= rbas[i:, :].dot(vbas.T).dot(vbas)
            rbas[i:, :] -= rbas[i:, :].dot(vbas2[:nindp, :].T).dot(vbas2[:nindp, :])
    return nindp, vbas2[:nindp].copy()


def genOrthoBas(vbas, crit_indp):
    vbas[0] = vbas[0] / numpy.linalg.norm(vbas[0])
    nbas = vbas.shape[0]
    if nbas != 1:
        nindp, vbas2 = dvdson_ortho(vbas[0:1], vbas[1:], crit_indp)
        if nindp + 1 != nbas:
            raise RuntimeError('insufficient orthonormal basis')
        vbas[1:] = vbas2
    return 0


class eigenSolver:
    def __init__(self, rng=None):
        self.maxcycle = 20
        self.crit_e = 1.e-8
        self.crit_vec = 1.e-8
        self.crit_indp = 1.e-12
        self.crit_demo = 1.e-10
        self.ndim = 0
        self.neig = 0
        self.diag = None
        self.HVec = None
        self.noise = True
        self.nmvp = 0
        self.lshift = 1.e-4
        self.nz = 1.e-5
        self.ifall = True
        self.nfac = 10
        self.rng = rng if rng is not None else numpy.random.default_rng(0)

    def HVecs(self, vbas):
        self.nmvp += vbas.shape[0]
        return numpy.array([self.HVec(v) for v in vbas])

    def genV0(self, neig):
        diag = self.diag + 1.e-12 * numpy.arange(1, 1 + self.ndim) / float(self.ndim)
        index = numpy.argsort(diag)[:neig]
        v0 = numpy.zeros((neig, self.ndim))
        v0[range(neig), index] = 1.0
        return v0

    def solve_iter(self, v0=None, iop=4):
        if self.neig > self.ndim:
            raise RuntimeError('neig > ndim')
        self.nmvp = 0
        vbas = self.genV0(self.neig) if v0 is None else v0.copy()
        if self.noise:
            vbas = vbas + self.nz * self.rng.uniform(-1, 1, size=(self.neig, self.ndim))
        genOrthoBas(vbas, self.crit_indp)
        wbas = self.HVecs(vbas)
        neig = self.neig
        eigs = numpy.zeros(neig) + 1.e3
        ndim = neig
        ifconv = False
        for niter in range(1, self.maxcycle):
            iden = vbas.dot(vbas.T)
            if numpy.linalg.norm(iden - numpy.identity(ndim)) > 1.e-10:
                raise RuntimeError('basis not orthonormal')
            tmpH = vbas.dot(wbas.T)
            if numpy.linalg.norm(tmpH - tmpH.T) > 1.e-10:
                raise RuntimeError('subspace H not symmetric')
            tmpH = 0.5 * (tmpH + tmpH.T)
            eig, vr = scipy.linalg.eigh(tmpH)
            vr = vr[:, :neig].T.copy()
            teig = eig[:neig]
            econv = [abs(teig[i] - eigs[i]) <= self.crit_e for i in range(neig)]
            eigs = teig.copy()
            rbas = vr.dot(vbas)
            rbas = vr.dot(wbas) - numpy.diag(eigs).dot(rbas)
            rindx = []
            rconv = [None] * neig
            for i in range(neig):
                tmp = numpy.linalg.norm(rbas[i, :])
                rconv[i] = (tmp <= self.crit_vec, tmp)
                if not rconv[i][0] and not econv[i]:
                    rindx.append(i)
            ifconv = len(rindx) == 0
            if ifconv or niter == self.maxcycle - 1:
                rbas = vr.dot(vbas)
                break
            if (not self.ifall) or (self.ifall and ndim > self.nfac * self.neig):
                pr = numpy.identity(ndim)[:neig, :] - vr
                nindp, vr2 = dvdson_ortho(vr, pr[rindx, :], self.crit_indp)
                if nindp != 0:
                    vr = numpy.vstack((vr, vr2))
                vbas = vr.dot(vbas)
                wbas = vr.dot(wbas)
            for i in range(neig):
                if rconv[i][0]:
                    continue
                if iop == 4:
                    rbas[i, :] = rbas[i, :] / (abs(self.diag - eigs[i]) + self.lshift)
                elif iop == 1:
                    tmp = self.diag - eigs[i]
                    tmp[abs(tmp) < self.crit_demo] = self.crit_demo
                    rbas[i, :] = rbas[i, :] / tmp
            nindp, vbas2 = dvdson_ortho(vbas, rbas[rindx, :], self.crit_indp)
            if nindp == 0:
                raise RuntimeError('Davidson: unable to generate new direction')
            wbas2 = self.HVecs(vbas2)
            vbas = numpy.vstack((vbas, vbas2))
            wbas = numpy.vstack((wbas, wbas2))
            ndim = vbas.shape[0]
        self.ifconv = ifconv
        return eigs, rbas, self.nmvp


# ---------------------------------------------------------------- decimation
def rdm_blkdiag(rho0, classes, thresh, Dcut=-1):
    dic = {}
    keys = []
    for idx, val in enumerate(classes):
        key = tuple(val)
        if key not in dic:
            dic[key] = []
            keys.append(key)
        dic[key].append(idx)
    nrows = rho0.shape[0]
    qsymL, rotL, sigs = [], [], []
    for key in keys:
        rows = dic[key]
        sig2, u = scipy.linalg.eigh(rho0[numpy.ix_(rows, rows)])
        sig2 = numpy.abs(sig2)
        ndim = len(sig2)
        qsymL += [list(key)] * ndim
        ucol = numpy.zeros((nrows, ndim))
        ucol[rows, :] = u
        rotL.append(ucol)
        sigs.append(sig2)
    rotL = numpy.hstack(rotL)
    sigs = numpy.hstack(sigs)
    sigs = sigs / numpy.sum(sigs)
    indx = numpy.argsort(sigs, kind='stable')[::-1]
    nres = len(sigs)
    tsig = sigs[indx]
    for i in range(nres):
        if tsig[i] < thresh * 1.01:
            nres = i
            break
    if nres == 0:
        nres = 1
    if Dcut > 0:
        nres = min(nres, Dcut)
    indx = indx[:nres]
    sigs = sigs[indx].copy()
    dwts = 1.0 - numpy.sum(sigs)
    qsymL = [qsymL[i] for i in indx]
    rotL = rotL[:, indx]
    order = sorted(range(nres), key=lambda x: qsymL[x])
    qsymL = [qsymL[i] for i in order]
    return dwts, qsymL, rotL[:, order].copy(), sigs[order].copy()


def _dense(t):
    return t.toDenseTensor(t.idlst) if isinstance(t, qtensor) else t


def pRDM(cimat, info):
    """Noise-perturbed reduced density matrix (mpo_dmrg_kernel.py:285-344)."""
    dmrg, isite, ncsite, flst, status, ifsym = info
    fL, fR = flst[0][0:2]
    neig, diml, dimc, dimr = cimat.shape
    addnoise = dmrg.inoise == 0 and dmrg.noise >= 1.e-10
    if status == 'L':
        rdm1 = numpy.zeros((diml * dimc, diml * dimc))
        if addnoise:
            for iop in range(dmrg.nops):
                lop = fL['opers%d' % iop]
                if lop is None:
                    continue
                cop = _dense(dmrg.fhop['site%d/op%d' % (isite, iop)])
                lop = _dense(lop)
                for ieig in range(neig):
                    tmp = numpy.tensordot(lop, cimat[ieig], axes=([2], [0]))
                    tmp = numpy.tensordot(tmp, cop, axes=([0, 2], [0, 3]))
                    tmp = tmp.transpose(0, 3, 1, 2)
                    s = tmp.shape
                    tmp = tmp.reshape(s[0] * s[1], s[2] * s[3])
                    rdm1 += tmp.dot(tmp.T) * dmrg.noise
        s = cimat[0].shape
        for ieig in range(neig):
            tmp = cimat[ieig].reshape(s[0] * s[1], s[2])
            rdm1 += tmp.dot(tmp.T)
    else:
        rdm1 = numpy.zeros((dimc * dimr, dimc * dimr))
        jsite = isite + ncsite - 1
        if addnoise:
            for iop in range(dmrg.nops):
                rop = fR['opers%d' % iop]
                if rop is None:
                    continue
                cop = _dense(dmrg.fhop['site%d/op%d' % (jsite, iop)])
                rop = _dense(rop)
                for ieig in range(neig):
                    tmp = numpy.tensordot(cimat[ieig], rop, axes=([2], [2]))
                    tmp = numpy.tensordot(cop, tmp, axes=([1, 3], [2, 1]))
                    tmp = tmp.transpose(0, 2, 1, 3)
                    s = tmp.shape
                    tmp = tmp.reshape(s[0] * s[1], s[2] * s[3])
                    rdm1 += tmp.T.dot(tmp) * dmrg.noise
        s = cimat[0].shape
        for ieig in range(neig):
            tmp = cimat[ieig].reshape(s[0], s[1] * s[2])
            rdm1 += tmp.T.dot(tmp)
    return rdm1


# --------------------------------------------------------------- the driver
class mpo_dmrg:
    """Attribute names follow mpo_dmrg_class.py:47-192."""

    def __init__(self, seed=0):
        self.nsite = None
        self.sbas = None
        self.occun = None
        self.crit_vec = 1.e-8
        self.thresh = -1.e-14
        self.ifdvdnz = True
        self.Dcut = None
        self.Dmax = None
        self.crit_e = 1.e-10
        self.noise = 1.e-4
        self.inoise = 0
        self.ifprecond = True
        self.schedule = None
        self.ifguess = True
        self.psi0 = None
        self.ncsite = None
        self.isym = 2
        self.qphys = None
        self.dphys = None
        self.qnuml = None
        self.qnumr = None
        self.nelec = 0.0
        self.sz = 0.0
        self.neig = None
        self.wts = None
        self.qsectors = None
        self.initNsweep = 0
        self.initNcsite = 1
        self.const = 0.0
        self.ifs2proj = False
        self.npts = None
        self.qwts = None
        self.qpts = None
        self.opers = []
        self.nops = None
        self.dims = None
        self.ifQt = False
        self.qkey = None
        self.qlst = None
        self.qtmp = None
        self.idlstCI = None
        self.fhop = None
        self.int1e = None
        self.int2e = None
        self.rng = numpy.random.default_rng(seed)
        self.ops = {}          # ('lop'|'rop', site) -> {'opers%d': tensor}
        self.flmps = {}
        self.frmps = {}
        self.nmvp = []
        self.eav = []
        self.dwt = []
        self.esweeps = []
        self.hpwts = None
        self.sweep_log = []

    # mpo_dmrg_class.py:279-297
    def build(self):
        assert self.nsite >= 2 and self.isym in [1, 2]
        self.qphys = initSpatialOrb(self.nsite, self.isym)
        self.dphys = [len(x) for x in self.qphys]
        self.qnuml = [None] * (self.nsite + 1)
        self.qnuml[0] = numpy.array(vacuum(self.isym))
        self.qnumr = [None] * (self.nsite + 1)
        self.qnumr[-1] = numpy.array(vacuum(self.isym))
        return 0

    # mpo_dmrg_class.py:206-246 (one rank)
    def partition(self):
        if self.npts is None:
            self.opers = [[x, None] for x in range(self.sbas)]
        else:
            self.opers = [[x // self.npts, x % self.npts] for x in range(self.npts * self.sbas)]
        self.nops = len(self.opers)
        self.pidx = sorted(set(x[0] for x in self.opers))
        self.pdic = dict((p, i) for i, p in enumerate(self.pidx))
        if self.npts is None:
            self.hpwts = numpy.ones(self.nops)
        else:
            self.hpwts = numpy.array([self.qwts[x[1]] for x in self.opers])
        return 0

    def loadInts(self, int1e, int2e):
        """Spin-orbital integrals int1e[p,q], int2e[p,q,r,s] = V_pqrs
        (mpo_dmrg_io.py:388-440 reads the same arrays from mole.h5)."""
        self.int1e = int1e[self.pidx]
        self.int2e = int2e[self.pidx]
        return 0

    # mpo_dmrg_io.py:168-206
    def dumpMPO(self):
        self.fhop = {'nsite': self.nsite, 'nops': self.nops, 'wts': self.hpwts}
        for isite in range(self.nsite):
            for iop in range(self.nops):
                pindx = self.opers[iop]
                if self.ifQt:
                    cop = qtensor_opers.genHRfacSpatialQt(pindx, self.sbas, isite, self.int1e,
                                                          self.int2e, self.qpts, self.pdic)
                else:
                    cop = mpo_opers.genHRfacSpatial(pindx, self.sbas, isite, self.int1e,
                                                    self.int2e, self.qpts, self.pdic)
                self.fhop['site%d/op%d' % (isite, iop)] = cop
        return 0

    def initStates(self):
        if self.qsectors is None:
            self.qsectors = {str([self.nelec, self.sz]): self.neig}
        self.neig = sum(self.qsectors.values())
        if self.wts is None:
            self.wts = numpy.ones(self.neig) / float(self.neig)
        return 0

    # ------------------------------------------------------- environments
    def _boundary(self, kind, isite):
        """genBopsNQt / genBopsQt (mpo_dmrg_init.py:52-78, mpo_dmrg_initQt.py:49-85)."""
        f = {}
        for iop in range(self.nops):
            if self.ifQt:
                q = [[0.]] if (self.isym == 1 or self.ifs2proj) else [[0., 0.]]
                t = qtensor([True, False, True])
                t.fromDenseTensor(numpy.ones((1, 1, 1)), [q, q, q])
            else:
                t = numpy.ones((1, 1, 1))
            f['opers%d' % iop] = t
        self.ops[(kind, isite)] = f
        return f

    def genHops(self, fmps, kind):
        """Full L ('lop', status 'L') or R sweep of environments
        (mpo_dmrg_init.py:90-176 / mpo_dmrg_initQt.py:88-275); returns <H_p>."""
        nsite = self.nsite
        exphop = numpy.zeros(self.nops)
        if kind == 'lop':
            self._boundary('lop', -1)
            for isite in range(nsite):
                site = fmps['site%d' % isite]
                flst = [[self.ops[('lop', isite - 1)], None]]
                fN = {}
                kernel.renorm(self, isite, 1, flst, [[fN]], site, 'L')
                self.ops[('lop', isite)] = fN
            last = self.ops[('lop', nsite - 1)]
        else:
            self._boundary('rop', nsite)
            for isite in range(nsite - 1, -1, -1):
                site = fmps['site%d' % isite]
                flst = [[None, self.ops[('rop', isite + 1)]]]
                fN = {}
                kernel.renorm(self, isite, 1, flst, [[fN]], site, 'R')
                self.ops[('rop', isite)] = fN
            last = self.ops[('rop', 0)]
        for iop in range(self.nops):
            t = last['opers%d' % iop]
            if t is None:
                continue
            exphop[iop] = (t.value[0] if isinstance(t, qtensor) else t[0, 0, 0])
        return exphop

    # mpo_dmrg_util.py:118-155
    def mps0occun(self):
        nsite = self.nsite
        sites = [None] * nsite
        qnuml = [None] * (nsite + 1)
        qnuml[0] = [[0., 0.]]
        nelec = 0.
        mspin = 0.
        for isite in range(nsite):
            na, nb = self.occun[2 * isite], self.occun[2 * isite + 1]
            tmp = numpy.zeros(self.dphys[isite])
            if abs(na) < 1e-4 and abs(nb) < 1e-4:
                tmp[0] = 1.0
            elif abs(na) < 1e-4 and abs(nb - 1) < 1e-4:
                nelec += 1
                mspin -= 0.5
                tmp[1] = 1.0
            elif abs(na - 1) < 1e-4 and abs(nb) < 1e-4:
                nelec += 1
                mspin += 0.5
                tmp[2] = 1.0
            else:
                nelec += 2
                tmp[3] = 1.0
            sites[isite] = tmp.reshape(1, self.dphys[isite], 1)
            qnuml[isite + 1] = [[nelec, mspin]]
        qnumr = [[[nelec - qnuml[i][0][0], mspin - qnuml[i][0][1]]] for i in range(nsite + 1)]
        return qnuml, qnumr, sites

    def product_mps(self):
        """Left-canonical product-state MPS from ``occun`` in the storage form
        selected by ``ifQt`` (the reference reaches the same object through
        initMPS + its MPS file conversion)."""
        qnuml, qnumr, sites = self.mps0occun()
        fmps = {'nsite': self.nsite}
        for i in range(self.nsite + 1):
            fmps['qnum%d' % i] = numpy.array(qnuml[i])
        for i in range(self.nsite):
            if self.ifQt:
                t = qtensor([False, False, True])
                t.fromDenseTensor(sites[i], [qnuml[i], self.qphys[i], qnuml[i + 1]])
                fmps['site%d' % i] = t
            else:
                fmps['site%d' % i] = sites[i]
        return fmps

    # mpo_dmrg_util.py:158-190 (no-MPS start, dense storage only)
    def initMPS(self):
        qnuml, qnumr, mps0 = self.mps0occun()
        self.qnuml = [numpy.array(q) for q in qnuml]
        self.qnumr = [numpy.array(q) for q in qnumr]
        fmps0 = {'nsite': self.nsite}
        for i in range(self.nsite):
            fmps0['site%d' % i] = mps0[i]
        self._boundary('lop', -1)
        self.genHops(fmps0, 'rop')
        self.sweep(list(range(self.nsite)), self.initNcsite, 'L', ifsym=True)
        return 0

    # mpo_dmrg_util.py:193-275 (Hamiltonian environments)
    def initOps(self, fmps):
        self._boundary('rop', self.nsite)
        self.genHops(fmps, 'lop')
        return 0

    # --------------------------------------------------------- local solver
    def _qlst(self, isite, ncsite):
        if ncsite == 1:
            return [numpy.array(self.qnuml[isite]), numpy.array(self.qphys[isite]),
                    numpy.array(self.qnumr[isite + 1])]
        return [numpy.array(self.qnuml[isite]), numpy.array(self.qphys[isite]),
                numpy.array(self.qphys[isite + 1]), numpy.array(self.qnumr[isite + 2])]

    def ci_solver(self, isite, ncsite, actlst, flst, status, ifsym):
        fL, fR = flst[0][0:2]
        cdim = self.dphys[isite] * (self.dphys[isite + 1] if ncsite == 2 else 1)
        ldim = len(self.qnuml[isite])
        rdim = len(self.qnumr[isite + ncsite])
        ndim = ldim * cdim * rdim
        self.dims = (ldim, cdim, rdim, ndim)
        self.qlst = self._qlst(isite, ncsite)
        info = [self, isite, ncsite, flst, status, ifsym]
        self._hvec_templates = None
        ioff = 0
        eigs = []
        civecs = []
        nmvps = 0
        for qkey in self.qsectors:
            neig = self.qsectors[qkey]
            key = [float(x) for x in eval(qkey)]
            if self.ifQt:
                self.setupQtmpCI(ncsite, key)
                prjmap = self.qtmp.prjmap(self.idlstCI)
                ndim0 = self.qtmp.size_allowed
            else:
                qsymt = self.qlst[0].tolist()
                for q in self.qlst[1:]:
                    qsymt = dpt(qsymt, q.tolist())
                prjmap = numpy.array([i for i, q in enumerate(qsymt)
                                      if max(abs(a - b) for a, b in zip(q, key)) < 1e-10],
                                     dtype=numpy.int64)
                ndim0 = len(prjmap)
            if ndim0 == 0:
                raise RuntimeError('no basis in symmetry sector %s' % qkey)
            diag = kernel.HDiag(info, ndim0, prjmap) if self.ifprecond else numpy.ones(ndim0)
            solver = eigenSolver(self.rng)
            solver.HVec = lambda v: kernel.HVec(v, info, ndim0, prjmap)
            solver.crit_e = self.crit_e
            solver.crit_vec = self.crit_vec
            solver.ndim = ndim0
            solver.neig = neig
            solver.diag = diag
            solver.noise = self.ifdvdnz and (self.noise > 1.e-10)
            v0guess = None
            if self.psi0 is not None:
                v0guess = self.psi0[ioff:ioff + neig, prjmap].copy()
            eig, vec, nmvp = solver.solve_iter(v0=v0guess, iop=4)
            civec = numpy.zeros((neig, ndim))
            civec[:, prjmap] = vec
            civecs.append(civec)
            eigs += list(eig)
            nmvps += nmvp
            ioff += neig
        civecs = numpy.vstack(civecs)
        eigs = numpy.array(eigs)
        sigs, dwts, qred, site, srotR = self.decimation(civecs, info)
        if self.ifguess:
            self.genGuess(isite, ncsite, actlst, civecs, srotR, status)
        return nmvps, eigs, sigs, dwts, qred, site, srotR

    def setupQtmpCI(self, ncsite, key):
        """mpo_dmrg_dotutil.py:192-203."""
        self.qkey = numpy.array(key)
        if ncsite == 1:
            qnums = [self.qlst[0], self.qlst[1], self.qkey - self.qlst[2]]
            self.qtmp = qtensor([False, False, True])
        else:
            qnums = [self.qlst[0], self.qlst[1], self.qlst[2], self.qkey - self.qlst[3]]
            self.qtmp = qtensor([False, False, False, True])
        rank, qsyms, ndims, idlst = fromQnums(qnums)
        self.qtmp.fromQsyms(rank, qsyms, ndims)
        self.idlstCI = copy.deepcopy(idlst)
        return 0

    def decimation(self, civecs, info):
        dmrg, isite, ncsite, flst, status, ifsym = info
        ldim, cdim, rdim, ndim = self.dims
        neig = civecs.shape[0]
        if status == 'L':
            dim = self.dphys[isite]
            cdimc = cdim // dim
            lcdim = ldim * dim
            crdim = cdimc * rdim
            civecs = civecs.reshape(neig, ldim, dim, crdim)
        else:
            jsite = isite + ncsite - 1
            dim = self.dphys[jsite]
            cdimc = cdim // dim
            lcdim = ldim * cdimc
            crdim = dim * rdim
            civecs = civecs.reshape(neig, lcdim, dim, rdim)
        if self.inoise == 1 and self.noise >= 1.e-10:
            civecs = civecs + self.rng.uniform(-1, 1, size=civecs.shape) * 10.0 * self.noise
        rdm1 = pRDM(civecs, info)
        trRDM = numpy.trace(rdm1)
        if trRDM < -1e-12:
            raise RuntimeError('RDM should be positive definite')
        elif trRDM < 1e-12:
            rdm1 = rdm1 + numpy.identity(rdm1.shape[0]) / float(rdm1.shape[0])
        else:
            rdm1 = rdm1 / trRDM
        Dcut = self.Dmax
        if ncsite == 1:
            if (status == 'L' and isite == self.nsite - 1) or (status == 'R' and isite == 0):
                Dcut = 1
        if status == 'L':
            if self.Dcut is not None:
                Dcut = self.Dcut[isite + 1]
            classes = dpt(numpy.array(self.qnuml[isite]).tolist(), self.qphys[isite])
            dwts, qred, rotL, sigs = rdm_blkdiag(rdm1, classes, self.thresh, Dcut)
            nres = len(qred)
            site = rotL.reshape(ldim, dim, nres).copy()
            srotR = numpy.empty((neig, nres, cdimc, rdim))
            for ieig in range(neig):
                cimat = civecs[ieig].reshape(lcdim, crdim)
                srotR[ieig] = rotL.T.dot(cimat).reshape(nres, cdimc, rdim)
        else:
            jsite = isite + ncsite - 1
            if self.Dcut is not None:
                Dcut = self.Dcut[jsite]
            classes = dpt(self.qphys[jsite], numpy.array(self.qnumr[jsite + 1]).tolist())
            dwts, qred, rotL, sigs = rdm_blkdiag(rdm1, classes, self.thresh, Dcut)
            nres = len(qred)
            site = rotL.reshape(dim, rdim, nres).transpose(2, 0, 1).copy()
            srotR = numpy.empty((neig, ldim, cdimc, nres))
            for ieig in range(neig):
                cimat = civecs[ieig].reshape(lcdim, crdim)
                srotR[ieig] = cimat.dot(rotL).reshape(ldim, cdimc, nres)
        return sigs, dwts, numpy.array(qred), site, srotR

    def _load_dense(self, fmps, isite):
        t = fmps['site%d' % isite]
        return t.toDenseTensor(t.idlst) if isinstance(t, qtensor) else t

    def genGuess(self, isite, ncsite, actlst, civecs, srotR, status):
        """mpo_dmrg_dotutil.py:498-559."""
        if status == 'R':
            if isite == actlst[-1]:
                self.psi0 = civecs.copy()
            elif 'site%d' % (isite - 1) in self.flmps:
                tmp0 = self._load_dense(self.flmps, isite - 1)
                rows = []
                for ieig in range(self.neig):
                    rows.append(numpy.tensordot(tmp0, srotR[ieig], axes=([2], [0])).reshape(-1))
                self.psi0 = numpy.array(rows)
        else:
            nxt = isite + ncsite
            if isite == actlst[-1]:
                self.psi0 = civecs.copy()
            elif 'site%d' % nxt in self.frmps:
                tmp0 = self._load_dense(self.frmps, nxt)
                rows = []
                for ieig in range(self.neig):
                    rows.append(numpy.tensordot(srotR[ieig], tmp0, axes=([2], [0])).reshape(-1))
                self.psi0 = numpy.array(rows)
        return 0

    # ---------------------------------------------------------------- sweep
    def checkOpers(self, sitelst, ncsite, status):
        nsite = self.nsite
        if status == 'L':
            oplstR = range(sitelst[0] + ncsite, min(nsite, sitelst[-1] + ncsite) + 1)
            return [i - ncsite for i in oplstR]
        oplstL = list(range(max(-1, sitelst[0] - ncsite), sitelst[-1] - ncsite + 1))
        return [i + 1 for i in oplstL[::-1]]

    def updateSite(self, isite, ncsite, qred, site, status):
        if status == 'L':
            self.qnuml[isite + 1] = qred.copy()
            if self.ifQt:
                t = qtensor([False, False, True])
                t.fromDenseTensor(site, [self.qlst[0], self.qlst[1], qred])
                site = t
            self.flmps['qnum%d' % (isite + 1)] = qred.copy()
            self.flmps['site%d' % isite] = site
        else:
            jsite = isite + ncsite - 1
            self.qnumr[jsite] = qred.copy()
            if self.ifQt:
                t = qtensor([True, False, False])
                t.fromDenseTensor(site, [qred, self.qlst[-2], self.qlst[-1]])
                site = t
            self.frmps['qnum%d' % jsite] = qred.copy()
            self.frmps['site%d' % jsite] = site
        return site

    def updateBoundary(self, ncsite, sitelst, qred, srotR, status):
        if ncsite != 2:
            return 0
        key = [float(x) for x in eval(next(iter(self.qsectors)))]
        if status == 'L' and sitelst[-1] == self.nsite - 1:
            smat = srotR[0] / numpy.linalg.norm(srotR[0])
            if self.ifQt:
                t = qtensor([False, False, True])
                t.fromDenseTensor(smat, [qred, self.qphys[self.nsite - 1], [key]])
                smat = t
            self.flmps['qnum%d' % self.nsite] = numpy.array([key])
            self.flmps['site%d' % (self.nsite - 1)] = smat
        elif status == 'R' and sitelst[0] == 0:
            smat = srotR[0] / numpy.linalg.norm(srotR[0])
            if self.ifQt:
                t = qtensor([True, False, False])
                t.fromDenseTensor(smat, [[key], self.qphys[0], qred])
                smat = t
            self.frmps['qnum0'] = numpy.array([key])
            self.frmps['site0'] = smat
        return 0

    def sweep(self, sitelst, ncsite, status, ifsym=True):
        actlst = self.checkOpers(sitelst, ncsite, status)
        elst, dlst = [], []
        nmvp = 0
        for isite in actlst:
            flst = [[self.ops[('lop', isite - 1)], self.ops[('rop', isite + ncsite)]]]
            nmvps, eigs, sigs, dwts, qred, site, srotR = self.ci_solver(
                isite, ncsite, actlst, flst, status, ifsym)
            nmvp += nmvps
            elst.append(eigs)
            dlst.append(dwts)
            siteN = self.updateSite(isite, ncsite, qred, site, status)
            fN = {}
            kernel.renorm(self, isite, ncsite, flst, [[fN]], siteN, status)
            if status == 'L':
                self.ops[('lop', isite)] = fN
            else:
                self.ops[('rop', isite + ncsite - 1)] = fN
            self.sweep_log.append((status, isite, float(eigs[0]), float(dwts)))
        self.updateBoundary(ncsite, sitelst, qred, srotR, status)
        eavs = numpy.array(elst).dot(self.wts)
        indx = int(numpy.argmin(eavs))
        return nmvp, indx, eavs[indx], dlst[indx], elst, dlst

    # mpo_dmrg_class.py:329-434
    def default(self, sc, fmps=None):
        self.schedule = sc
        self.crit_tol = sc.tol
        self.initStates()
        self.flmps = {'nsite': self.nsite, 'qnum0': self.qnuml[0]}
        self.frmps = {'nsite': self.nsite, 'qnum%d' % self.nsite: self.qnumr[-1]}
        if fmps is None:
            assert not self.ifQt
            self.Dmax = sc.MaxMs[0]
            self.crit_e = sc.Tols[0]
            self.noise = sc.Noises[0]
            self.initMPS()
        else:
            self.qnuml = [numpy.array(fmps['qnum%d' % i]) for i in range(self.nsite + 1)]
            for k, v in fmps.items():
                self.flmps[k] = v
            self.initOps(fmps)
        self.psi0 = None
        sitelst = list(range(self.nsite))
        eold = 1.e3
        deltaE = 1.e3
        ifconv = False
        isweep = -1
        for isweep in range(sc.maxiter):
            self.isweep = isweep
            sc.getParameters(self, isweep)
            r1 = self.sweep(sitelst, self.ncsite, 'R')
            r2 = self.sweep(sitelst, self.ncsite, 'L')
            self.nmvp.append(r1[0] + r2[0])
            self.esweeps += r1[4] + r2[4]
            if r1[2] < r2[2]:
                eav, dwt = r1[2], r1[3]
            else:
                eav, dwt = r2[2], r2[3]
            self.eav.append(eav)
            self.dwt.append(dwt)
            self.Energy = eav
            deltaE = eav - eold
            ifconv = sc.checkConv(self, isweep, deltaE)
            eold = eav
            if ifconv:
                break
        self.ifconv = ifconv
        self.nsweep = isweep + 1
        self.deltaE = deltaE
        return 0
