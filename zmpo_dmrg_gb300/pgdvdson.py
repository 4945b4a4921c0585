"""Generalised Davidson solver for H c = E S c with the basis on the GPU.

Same algorithm and settings as ``source/tools/pgdvdson.py`` (``solve_iter``
90-330), used by the spin-projected solver: an orthonormal (not S-orthogonal)
basis V with W = H V and Z = S V kept in device memory; the subspace pair
(V W^T, V Z^T) is symmetrised and solved on the host with
``scipy.linalg.eigh(a, b)``; residuals r = x W - e x Z; convergence by the
eigenvalue change ``<= crit_e`` or ``|r| <= crit_vec``; preconditioner
``r / (|diag - e| + 1e-4)`` (iop = 4); ``maxcycle = 10``; restart to the Ritz
vectors and their corrections once the basis exceeds ``nfac * neig``.  The
returned vectors are S-normalised (x S x^T = 1), as in the reference.
"""
import numpy
import scipy.linalg

from .pdvdson import mask, dvdson_ortho  # noqa: F401  (same mask as pdvdson)


def _torch():
    import torch
    return torch


def gen_ortho_bas(vbas, crit_indp):
    """Orthonormal rows spanning ``vbas`` (the reference's genOrthoBas)."""
    vbas = vbas.clone()
    torch = _torch()
    first = torch.linalg.norm(vbas[0])
    vbas[0] = vbas[0] / first
    if vbas.shape[0] == 1:
        return vbas
    n, v2 = dvdson_ortho(vbas[:1], vbas[1:], crit_indp)
    # dependent rows are dropped, as genOrthoBas does
    return vbas[:1] if n == 0 else torch.cat([vbas[:1], v2])


class eigenSolver:
    def __init__(self, rng=None):
        self.maxcycle = 10
        self.crit_e = 1.e-8
        self.crit_vec = 1.e-8
        self.crit_indp = 1.e-12
        self.ndim = 0
        self.neig = 0
        self.diag = None
        self.HVec = None
        self.SVec = None
        self.noise = True
        self.nmvp = 0
        self.lshift = 1.e-4
        self.nz = 1.e-5
        self.ifall = True
        self.nfac = 10
        self.ifconv = False
        self.hvec_eps = 0.0
        self.rng = rng if rng is not None else numpy.random.default_rng(0)

    def HSVecs(self, vbas):
        torch = _torch()
        self.nmvp += vbas.shape[0]
        w = torch.stack([self.HVec(v) for v in vbas])
        s = torch.stack([self.SVec(v) for v in vbas])
        return w, s

    def genV0(self, neig):
        torch = _torch()
        d = self.diag.detach().cpu().numpy() + 1.e-12 * numpy.arange(1, 1 + self.ndim) / float(self.ndim)
        index = numpy.argsort(d, kind="stable")[:neig]
        v0 = torch.zeros((neig, self.ndim), dtype=torch.float64, device=self.diag.device)
        v0[torch.arange(neig), torch.as_tensor(index, device=self.diag.device)] = 1.0
        return v0

    def solve_iter(self, v0=None, iop=4):
        torch = _torch()
        if self.neig > self.ndim:
            raise RuntimeError("generalised Davidson: neig > ndim")
        self.nmvp = 0
        dev = self.diag.device
        if v0 is None:
            vbas = self.genV0(self.neig)
        else:
            vbas = (v0 if torch.is_tensor(v0) else torch.as_tensor(numpy.asarray(v0))).to(
                device=dev, dtype=torch.float64).clone()
        if self.noise:
            nz = self.rng.uniform(-1, 1, size=(self.neig, self.ndim))
            vbas = vbas + self.nz * torch.as_tensor(nz, device=dev)
        vbas = gen_ortho_bas(vbas, self.crit_indp)
        if vbas.shape[0] != self.neig:
            raise RuntimeError("generalised Davidson: insufficient orthonormal basis")
        wbas, sbas = self.HSVecs(vbas)
        neig = self.neig
        eigs = numpy.zeros(neig) + 1.e3
        ndim = neig
        xbas = None
        for niter in range(1, self.maxcycle):
            iden = (vbas @ vbas.T).cpu().numpy()
            if numpy.linalg.norm(iden - numpy.identity(ndim)) > 1.e-10:
                raise RuntimeError("generalised Davidson: basis lost orthonormality")
            tmpH = (vbas @ wbas.T).cpu().numpy()
            tmpS = (vbas @ sbas.T).cpu().numpy()
            tol_h = max(1.e-10, 100.0 * self.hvec_eps * numpy.linalg.norm(tmpH))
            if numpy.linalg.norm(tmpH - tmpH.T) > tol_h or numpy.linalg.norm(tmpS - tmpS.T) > 1.e-10:
                raise RuntimeError("generalised Davidson: subspace H or S not symmetric")
            tmpH = 0.5 * (tmpH + tmpH.T)
            tmpS = 0.5 * (tmpS + tmpS.T)
            try:
                eig, vr = scipy.linalg.eigh(tmpH, tmpS)
            except numpy.linalg.LinAlgError:
                raise RuntimeError("generalised Davidson: subspace S is not positive definite")
            vr = vr[:, :neig].T.copy()
            over = vr @ tmpS @ vr.T
            if numpy.linalg.norm(over - numpy.identity(neig)) > 1.e-10:
                raise RuntimeError("generalised Davidson: Ritz vectors not S-orthonormal")
            teig = eig[:neig]
            econv = [abs(teig[i] - eigs[i]) <= self.crit_e for i in range(neig)]
            eigs = teig.copy()
            vr_d = torch.as_tensor(vr, device=dev)
            xbas = vr_d @ vbas
            rbas = vr_d @ wbas - torch.as_tensor(eigs, device=dev)[:, None] * (vr_d @ sbas)
            rn = torch.linalg.norm(rbas, dim=1).cpu().numpy()
            crit = max(self.crit_vec, 10.0 * self.hvec_eps * max(1.0, float(numpy.abs(eigs).max())))
            rconv = [rn[i] <= crit for i in range(neig)]
            rindx = [i for i in range(neig) if not rconv[i] and not econv[i]]
            self.rnorm = rn
            if not rindx or niter == self.maxcycle - 1:
                self.ifconv = not rindx
                return eigs, xbas, self.nmvp
            if (not self.ifall) or ndim > self.nfac * neig:
                pr = numpy.identity(ndim)[:neig, :] - vr
                vr2 = numpy.vstack((vr, pr[rindx, :]))
                vr2 = gen_ortho_bas(torch.as_tensor(vr2, device=dev), self.crit_indp)
                vbas = vr2 @ vbas
                wbas = vr2 @ wbas
                sbas = vr2 @ sbas
            for i in range(neig):
                if rconv[i]:
                    continue
                if iop == 4:
                    rbas[i] = rbas[i] / (torch.abs(self.diag - eigs[i]) + self.lshift)
                elif iop == 1:
                    t = self.diag - eigs[i]
                    t = torch.where(torch.abs(t) < 1.e-10, torch.full_like(t, 1.e-10), t)
                    rbas[i] = rbas[i] / t
            n, vbas2 = dvdson_ortho(vbas, rbas[rindx], self.crit_indp)
            if n == 0:
                raise RuntimeError("generalised Davidson: unable to generate new direction")
            wbas2, sbas2 = self.HSVecs(vbas2)
            vbas = torch.cat([vbas, vbas2])
            wbas = torch.cat([wbas, wbas2])
            sbas = torch.cat([sbas, sbas2])
            ndim = vbas.shape[0]
        self.ifconv = False
        return eigs, xbas, self.nmvp
