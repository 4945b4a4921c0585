"""Davidson eigensolver with the basis on the GPU (FP64).

Same algorithm and settings as ``source/tools/pdvdson.py`` (``solve_iter``
90-330): start from the lowest diagonal entries or a guess plus 1e-5 uniform
noise, subspace matrix V W^T symmetrised and diagonalised, residual test
``|r| <= crit_vec`` or eigenvalue change ``<= crit_e``, preconditioner
``r / (|diag - e| + 1e-4)`` (iop = 4), modified Gram-Schmidt with five
projection passes (``dvdson_ortho`` 350-390), restart to the Ritz vectors and
their corrections once the basis exceeds ``nfac * neig``.  The basis V, the
images W = H V and all projections stay in device memory; only the small
subspace matrix goes to the host for ``eigh``.  The sum over operator terms
(the reference's MPI Reduce, pdvdson.py:75) happens inside the engine.
"""
import numpy


class mask:
    def __init__(self, info, mvp):
        self.info = info
        self.mvp = mvp

    def matvec(self, vec):
        return self.mvp(vec, *self.info)


def _torch():
    import torch
    return torch


def dvdson_ortho(vbas, rbas, crit_indp):
    """Orthonormalise the rows of ``rbas`` against ``vbas`` and each other."""
    torch = _torch()
    rbas = rbas.clone()
    for _ in range(5):
        rbas = rbas - (rbas @ vbas.T) @ vbas
    out = []
    for i in range(rbas.shape[0]):
        rvec = rbas[i].clone()
        rii = float(torch.linalg.norm(rvec))
        if rii <= crit_indp:
            continue
        rvec = rvec / rii
        rvec = rvec / torch.linalg.norm(rvec)
        out.append(rvec)
        v2 = torch.stack(out)
        tail = rbas[i:]
        for _ in range(5):
            tail = tail - (tail @ vbas.T) @ vbas
            tail = tail - (tail @ v2.T) @ v2
        rbas[i:] = tail
    if not out:
        return 0, None
    return len(out), torch.stack(out)


class eigenSolver:
    def __init__(self, rng=None):
        self.maxcycle = 20
        self.crit_e = 1.e-8
        self.crit_vec = 1.e-8
        self.crit_indp = 1.e-12
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
        self.ifconv = False
        # relative accuracy of H.v (0 for FP64); bounds the symmetry check and
        # the reachable residual of a split-precision product
        self.hvec_eps = 0.0
        self.rng = rng if rng is not None else numpy.random.default_rng(0)

    def HVecs(self, vbas):
        torch = _torch()
        self.nmvp += vbas.shape[0]
        return torch.stack([self.HVec(v) for v in vbas])

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
            raise RuntimeError("Davidson: neig > ndim")
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
        vbas[0] = vbas[0] / torch.linalg.norm(vbas[0])
        if self.neig > 1:
            n, v2 = dvdson_ortho(vbas[:1], vbas[1:], self.crit_indp)
            if n + 1 != self.neig:
                raise RuntimeError("Davidson: insufficient orthonormal basis")
            vbas = torch.cat([vbas[:1], v2])
        wbas = self.HVecs(vbas)
        neig = self.neig
        eigs = numpy.zeros(neig) + 1.e3
        ndim = neig
        for niter in range(1, self.maxcycle):
            iden = (vbas @ vbas.T).cpu().numpy()
            if numpy.linalg.norm(iden - numpy.identity(ndim)) > 1.e-10:
                raise RuntimeError("Davidson: basis lost orthonormality")
            tmpH = (vbas @ wbas.T).cpu().numpy()
            tol_sym = max(1.e-10, 100.0 * self.hvec_eps * numpy.linalg.norm(tmpH))
            if numpy.linalg.norm(tmpH - tmpH.T) > tol_sym:
                raise RuntimeError("Davidson: subspace H not symmetric")
            tmpH = 0.5 * (tmpH + tmpH.T)
            eig, vr = numpy.linalg.eigh(tmpH)
            vr = vr[:, :neig].T.copy()
            teig = eig[:neig]
            econv = [abs(teig[i] - eigs[i]) <= self.crit_e for i in range(neig)]
            eigs = teig.copy()
            vr_d = torch.as_tensor(vr, device=dev)
            xbas = vr_d @ vbas
            rbas = vr_d @ wbas - torch.as_tensor(eigs, device=dev)[:, None] * xbas
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
                n, vr2 = dvdson_ortho(vr_d, torch.as_tensor(pr[rindx, :], device=dev), self.crit_indp)
                if n:
                    vr_d = torch.cat([vr_d, vr2])
                vbas = vr_d @ vbas
                wbas = vr_d @ wbas
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
                raise RuntimeError("Davidson: unable to generate new direction")
            wbas2 = self.HVecs(vbas2)
            vbas = torch.cat([vbas, vbas2])
            wbas = torch.cat([wbas, wbas2])
            ndim = vbas.shape[0]
        self.ifconv = False
        return eigs, vr_d @ vbas, self.nmvp
