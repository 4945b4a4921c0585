"""Spin projection (SP-MPS) on the GPU engine.

Same quantities as the reference:
  * quadrature: ``mpo_dmrg_util.s2quad`` (mpo_dmrg_util.py:35-89,
    Gauss-Legendre: beta_g = acos(x_g), w_g = (2S+1)/2 d^S_{MM}(beta_g) v_g)
    with the Wigner small-d of ``tools/smalld.py``;
  * operator terms [p, g] with weights w_g and H_p R(beta_g) site tensors
    labelled by N only (``mpo_dmrg_class.partition`` 217-240,
    ``qtensor_opers.genHRfacSpatialQt`` 380-384);
  * H psi with the wavefunction relabelled by N (``qtensor.reduceQsymsToN``) and
    the result projected back on the (N, Sz) blocks (``projectionNMs``):
    ``mpo_dmrg_kernelQt.HVecQt`` 157-160, 309-312;
  * the overlap S psi = sum_g w_g P_g psi with the bond-1 R(beta_g) MPO
    (``SVecQt`` 373-450) and its environments (``renormQt_S00`` 770-855).
All contractions are engine launches; relabelling is a device gather.
"""
import math

import numpy

from . import engine as _engine
from .qtensor import qtensor
from .mpo import ry_matrix


def _torch():
    import torch
    return torch


def wigner_small_d(j, m1, m2, beta):
    """d^j_{m1 m2}(beta) from the explicit sum over k (Wigner's formula)."""
    def fact(x):
        return math.gamma(x + 1.0)
    pref = math.sqrt(fact(j + m1) * fact(j - m1) * fact(j + m2) * fact(j - m2))
    c, s = math.cos(beta / 2.0), math.sin(beta / 2.0)
    kmin = max(0, int(round(m2 - m1)))
    kmax = min(int(round(j + m2)), int(round(j - m1)))
    tot = 0.0
    for k in range(kmin, kmax + 1):
        den = fact(j + m2 - k) * fact(k) * fact(m1 - m2 + k) * fact(j - m1 - k)
        tot += (-1.0) ** (m1 - m2 + k) / den * c ** (2 * j + m2 - m1 - 2 * k) * s ** (m1 - m2 + 2 * k)
    return pref * tot


def s2quad(dmrg, sval=0, sz=0):
    if sval + 1.e-4 <= abs(sz):
        raise ValueError("|Sz| must not exceed S")
    x, v = numpy.polynomial.legendre.leggauss(dmrg.npts)
    beta = numpy.arccos(x)
    w = numpy.array([wigner_small_d(sval, sz, sz, b) for b in beta]) * v * (2.0 * sval + 1.0) / 2.0
    dmrg.qpts = beta
    dmrg.qwts = w
    return beta, w


class PopStore:
    """R(beta_g) site tensors (one per quadrature point) on the device."""

    def __init__(self, qpts):
        torch = _torch()
        self.tensors = []
        vals = []
        self.off = []
        pos = 0
        qn = numpy.array([[0.], [1.], [1.], [2.]])
        for phi in qpts:
            t = qtensor([False, True, False, True])
            t.fromDenseTensor(ry_matrix(phi).reshape(1, 1, 4, 4), [[[0.]], [[0.]], qn, qn],
                              ifcollect=[0, 0, 0, 0])
            self.tensors.append(t)
            self.off.append(pos)
            vals.append(t.value)
            pos += t.size_allowed
        self.buf = torch.from_numpy(numpy.concatenate(vals)).cuda()
        self.uid = id(self)


def dumpMPO_R(dmrg):
    """Device copies of R(beta_g) (the reference's ``pop`` file, mpo_dmrg_io.py:209)."""
    dmrg.pop_store = PopStore(dmrg.qpts)
    return 0


def n_only_map(qt):
    """Structure of ``qt`` relabelled by N and, for every element of qt's
    packing, its position in the N-labelled packing."""
    qn = qtensor(qt.status)
    qn.fromQsyms(qt.rank, [q[:, :1] for q in qt.qsyms], qt.ndims, ifallocate=False)
    where = {tuple(int(s) for s in sec): off for sec, dims, off in qn.blocks()}
    idx = numpy.empty(qt.size_allowed, dtype=numpy.int64)
    for sec, dims, off in qt.blocks():
        n = int(numpy.prod(dims))
        o = where[tuple(int(s) for s in sec)]
        idx[off:off + n] = numpy.arange(o, o + n)
    return qn, idx


def reduce_site(site):
    """Site tensor relabelled by N with its values moved to the new packing."""
    qn, idx = n_only_map(site)
    v = site.value
    if not isinstance(v, numpy.ndarray):
        v = v.detach().cpu().numpy()
    out = numpy.zeros(qn.size_allowed)
    out[idx] = v
    qn.value = out
    qn.idlst = site.idlst
    return qn


def boundary_pops(dmrg):
    from .mpo_dmrg_kernel import EnvSet
    torch = _torch()
    t = qtensor([True, False, True])
    t.fromQsyms(3, [[[0.]], [[0.]], [[0.]]], [[1], [1], [1]], ifallocate=False)
    buf = torch.ones(dmrg.npts, dtype=torch.float64, device="cuda")
    return EnvSet(buf, numpy.arange(dmrg.npts, dtype=numpy.int64),
                  numpy.full(dmrg.npts, t.layout, dtype=numpy.int64), [t] * dmrg.npts)


def _svec_plan(info):
    dmrg, isite, ncsite, flst, status, ifsym = info
    torch = _torch()
    eng = _engine.get()
    fLp, fRp = flst[0][2:4]
    key = (fLp.uid, fRp.uid, isite, ncsite, dmrg.qtmp.layout, 'S')
    cur = getattr(dmrg, "_svec_plan", None)
    if cur is None or cur[0] != key:
        if cur is not None:
            eng.destroy_plan(cur[1])
        from .mpo_dmrg_kernel import _flip_layout
        ps = dmrg.pop_store
        lay_rf = _flip_layout(dmrg, fRp.tensors[0])
        npts = dmrg.npts
        qN, idx = n_only_map(dmrg.qtmp)
        pid, ws = eng.sigma_plan(ncsite, [0] * npts, [fLp.layouts[0]], [ps.tensors[0].layout],
                                 [ps.tensors[0].layout] if ncsite == 2 else None, [lay_rf], qN.layout,
                                 fLp.off, fRp.off, ps.off, ps.off if ncsite == 2 else None, dmrg.qwts)
        work = torch.empty(max(ws // 8, 1), dtype=torch.float64, device="cuda")
        cur = (key, pid, work, torch.as_tensor(idx, device="cuda"), qN.size_allowed)
        dmrg._svec_plan = cur
    return cur


def SVec(vec0, info, ndim0, prjmap):
    """S psi = sum_g w_g P_g psi (``SVecQt``; flst[0][2:4] hold the P environments)."""
    dmrg = info[0]
    torch = _torch()
    eng = _engine.get()
    fLp, fRp = info[3][0][2:4]
    _, pid, work, idx, nN = _svec_plan(info)
    was_host = isinstance(vec0, numpy.ndarray)
    x = torch.as_tensor(numpy.asarray(vec0), dtype=torch.float64).cuda() if was_host else vec0
    xN = torch.zeros(nN, dtype=torch.float64, device="cuda")
    xN[idx] = x
    yN = torch.empty(nN, dtype=torch.float64, device="cuda")
    # the overlap is a bond-1 chain, negligible next to H psi: always FP64
    eng.sigma(pid, fLp.buf, fRp.buf, dmrg.pop_store.buf, xN, yN, work, "fp64")
    y = yN[idx]
    return y.cpu().numpy() if was_host else y


def SDiag(info, ndim0, prjmap):
    """diag(S) on the (N, Sz) packing (``SDiagQt``, mpo_dmrg_kernelQt.py:322-370)."""
    dmrg = info[0]
    torch = _torch()
    _svec_plan(info)
    _, pid, work, idx, nN = dmrg._svec_plan
    fLp, fRp = info[3][0][2:4]
    dN = torch.zeros(nN, dtype=torch.float64, device="cuda")
    _engine.get().hdiag(pid, fLp.buf, fRp.buf, dmrg.pop_store.buf, dN)
    return dN[idx]


def renorm_S00(dmrg, isite, ncsite, flst, flstN, site, status):
    """P environments after the site update for every quadrature point
    (``renormQt_S00``, mpo_dmrg_kernelQt.py:770-855); the EnvSet is stored
    in ``flstN[0][1]``."""
    from .mpo_dmrg_kernel import EnvSet, _env_structure
    torch = _torch()
    eng = _engine.get()
    ps = dmrg.pop_store
    qsite = reduce_site(site)
    fE = flst[0][2] if status == 'L' else flst[0][3]
    wt = ps.tensors[0]
    if status == 'L':
        lay_w = wt.layout
    else:
        st = wt.status.copy()
        st[0], st[1] = not st[0], not st[1]
        lay_w = eng.derive(wt.layout, [-wt.qsyms[0], -wt.qsyms[1], wt.qsyms[2], wt.qsyms[3]], st)
    npts = dmrg.npts
    pid, lay_out, off_out, total, ws = eng.renorm_plan(status, [0] * npts, [fE.layouts[0]], [lay_w],
                                                       qsite.layout, fE.off, ps.off)
    buf = torch.empty(max(total, 1), dtype=torch.float64, device="cuda")
    work = torch.empty(max(ws // 8, 1), dtype=torch.float64, device="cuda")
    sval = torch.from_numpy(numpy.ascontiguousarray(qsite.value)).cuda()
    eng.renorm(pid, fE.buf, ps.buf, sval, buf, work, getattr(dmrg, "precision_renorm", "fp64"))
    eng.destroy_plan(pid)
    t = _env_structure(dmrg, status, qsite, wt, None, int(lay_out[0]))
    while len(flstN[0]) < 2:
        flstN[0].append(None)
    flstN[0][1] = EnvSet(buf, numpy.asarray(off_out, dtype=numpy.int64),
                         numpy.full(npts, t.layout, dtype=numpy.int64), [t] * npts)
    return 0
