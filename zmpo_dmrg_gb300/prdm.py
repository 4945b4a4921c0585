"""Perturbed reduced density matrix for the decimation, on the GPU.

Same matrix as ``mpo_dmrg_kernelQt.pRDMQt`` (mpo_dmrg_kernelQt.py:453-626) /
``pRDMNQt`` (mpo_dmrg_kernel.py:285-344): rho = sum_e C_e C_e^T plus, when
``dmrg.noise >= 1e-10`` and ``dmrg.inoise == 0``, noise * sum_p T_p T_p^T with
T_p = L_p . psi . W_p(isite) for a left step and W_p(jsite) . psi . R_p for a
right step.  The wavefunction is packed with the right (left) two legs merged
(``mpo_dmrg_dotutil.setupQtmpPRDM``, mpo_dmrg_dotutil.py:562-589); the three
contractions per term run as engine block contractions and the per-term
results are summed on the device before one conversion to a dense matrix.
"""
import numpy

from . import engine as _engine
from .qtensor import qtensor, fromQnums


def _torch():
    import torch
    return torch


def _dpt(a, b):
    a = numpy.asarray(a, dtype=float)
    b = numpy.asarray(b, dtype=float)
    return (a[:, None, :] + b[None, :, :]).reshape(-1, a.shape[1])


class _Chain:
    """Three contraction plans of one operator class."""

    def __init__(self, eng, lay_env, lay_w, lay_psi, status):
        if status == 'L':
            lo1, self.p1 = eng.contract_plan(lay_env, lay_psi, ([2], [0]))
            lo2, self.p2 = eng.contract_plan(lo1, lay_w, ([0, 2], [0, 3]))
            lo3, self.p3 = eng.contract_plan(lo2, lo2, ([1, 2], [1, 2]))
        else:
            lo1, self.p1 = eng.contract_plan(lay_psi, lay_env, ([2], [2]))
            lo2, self.p2 = eng.contract_plan(lay_w, lo1, ([1, 3], [2, 1]))
            lo3, self.p3 = eng.contract_plan(lo2, lo2, ([0, 2], [0, 2]))
        self.sizes = [eng.layout_blocks(x)[0] for x in (lo1, lo2, lo3)]
        self.plans = (self.p1, self.p2, self.p3)

    def release(self, eng):
        for p in self.plans:
            eng.destroy_plan(p)


def pRDM(civecs, info):
    """civecs: (neig, diml, dimc, dimr) as reshaped by the decimation, a NumPy
    array or a float64 CUDA tensor; the result is of the same kind."""
    dmrg, isite, ncsite, flst, status, ifsym = info
    torch = _torch()
    on_device = torch.is_tensor(civecs)
    cv = civecs if on_device else torch.from_numpy(numpy.ascontiguousarray(civecs, dtype=numpy.float64)).cuda()
    neig, diml, dimc, dimr = cv.shape
    # sum_e C_e C_e^T as one dense product on the device (the states side by side)
    if status == 'L':
        cat = cv.reshape(neig, diml * dimc, dimr).permute(1, 0, 2).reshape(diml * dimc, neig * dimr)
        rho = cat @ cat.T
    else:
        mats = cv.reshape(neig * diml, dimc * dimr)
        rho = mats.T @ mats
    if not (dmrg.inoise == 0 and dmrg.noise >= 1.e-10):
        return rho if on_device else rho.cpu().numpy()
    eng = _engine.get()
    qkey = numpy.asarray(dmrg.qkey, dtype=float)
    # the dot as three legs [l, n, r] around the site being decimated: a
    # two-site dot merges the other site into its outer leg, a one-site dot
    # is already in that form (pRDMNQt, mpo_dmrg_kernel.py:290-340)
    if ncsite == 2:
        ql, qc1, qc2, qr = dmrg.qlst
        ql3, qc3, qr3 = (ql, qc1, _dpt(qc2, qr)) if status == 'L' else (_dpt(ql, qc1), qc2, qr)
    else:
        ql3, qc3, qr3 = dmrg.qlst
    qn = [ql3, qc3, qkey - numpy.asarray(qr3, dtype=float)]
    if status == 'L':
        qn2 = [qn[0], qn[1], qn[0], qn[1]]
        env = flst[0][0]
        jsite = isite
    else:
        qn2 = [qn[1], qn[2], qn[1], qn[2]]
        env = flst[0][1]
        jsite = isite + ncsite - 1
    psi = qtensor([False, False, True])
    rank, qsyms, ndims, idlst = fromQnums(qn)
    psi.fromQsyms(rank, qsyms, ndims, ifallocate=False)
    lay_psi, nmap = psi.layout, None
    if dmrg.ifs2proj:
        # spin projection: the terms carry N-only labels (reduceQsymsToN)
        from .spinproj import n_only_map
        psiN, idx = n_only_map(psi)
        lay_psi, nmap = psiN.layout, (idx, psiN.size_allowed)
    mpo = dmrg.mpo_store
    from .mpo import op_class
    # the packed wavefunction of every state: a device gather of the dense
    # vector through the packing's index map
    dense_idx = torch.as_tensor(numpy.asarray(psi.prjmap(idlst), dtype=numpy.int64), device="cuda")
    flat = cv.reshape(neig, -1)
    xs = []
    for e in range(neig):
        xv = flat[e].index_select(0, dense_idx)
        if nmap is not None:
            xN = torch.zeros(nmap[1], dtype=torch.float64, device="cuda")
            xN[torch.as_tensor(nmap[0], device="cuda")] = xv
            xv = xN
        xs.append(xv.contiguous())
    chains = {}
    acc = None
    for iop in range(dmrg.nops):
        if not env.present(iop):
            continue
        c0 = op_class(dmrg.opers[iop][0], jsite)
        if c0 not in chains:
            et = env.tensors[iop]
            wt = mpo.tensors[jsite][iop]
            if status == 'L':
                lay_env = et.layout
            else:
                q0 = qkey[:et.qsyms[1].shape[1]]
                st = et.status.copy()
                st[1] = not st[1]
                lay_env = eng.derive(et.layout, [-et.qsyms[0], et.qsyms[1] - q0, q0 - et.qsyms[2]], st)
            chains[c0] = _Chain(eng, lay_env, wt.layout, lay_psi, status)
        ch = chains[c0]
        if acc is None:
            acc = torch.zeros(ch.sizes[2], dtype=torch.float64, device="cuda")
            buf3 = torch.empty_like(acc)
        n_env = env.tensors[iop].size_allowed
        e_view = env.buf.narrow(0, int(env.off[iop]), n_env)
        w_view = mpo.buf.narrow(0, int(mpo.off[jsite][iop]), mpo.tensors[jsite][iop].size_allowed)
        t1 = torch.empty(max(ch.sizes[0], 1), dtype=torch.float64, device="cuda")
        t2 = torch.empty(max(ch.sizes[1], 1), dtype=torch.float64, device="cuda")
        for x in xs:
            if status == 'L':
                eng.contract_exec(ch.p1, e_view, x, t1)
                eng.contract_exec(ch.p2, t1, w_view, t2)
            else:
                eng.contract_exec(ch.p1, x, e_view, t1)
                eng.contract_exec(ch.p2, w_view, t1, t2)
            eng.contract_exec(ch.p3, t2, t2, buf3)
            acc += buf3
    for ch in chains.values():
        ch.release(eng)
    n = int(numpy.prod([len(x) for x in qn2[:2]]))
    noise_dense = torch.zeros(n * n, dtype=torch.float64, device="cuda")
    if acc is not None:
        # block structure of the summed T T^T (legs of the last contraction)
        et = next(env.tensors[i] for i in range(dmrg.nops) if env.present(i))
        qp = mpo.tensors[jsite][0].qsyms[2]
        dp = mpo.tensors[jsite][0].ndims[2]
        if status == 'L':
            legs_q = [et.qsyms[1], qp, et.qsyms[1], qp]
            legs_d = [et.ndims[1], dp, et.ndims[1], dp]
        else:
            qb = et.qsyms[1] - qkey[:et.qsyms[1].shape[1]]
            legs_q = [qp, qb, qp, qb]
            legs_d = [dp, et.ndims[1], dp, et.ndims[1]]
        out = qtensor([False, False, True, True])
        out.fromQsyms(4, legs_q, legs_d, ifallocate=False)
        _, _, _, idlst2 = fromQnums(qn2)
        if out.size_allowed != acc.numel():
            raise RuntimeError("perturbed RDM layout mismatch")
        # scatter the summed blocks into the dense (n, n) matrix on the device
        didx = torch.as_tensor(numpy.asarray(out.prjmap(idlst2), dtype=numpy.int64), device="cuda")
        noise_dense[didx] = acc
    if getattr(dmrg, "size", 1) > 1:
        # the noise term sums over the operator terms of every rank (a rank
        # may hold no term at this site: its share is zero)
        from .parallel import allreduce_
        allreduce_(noise_dense, dmrg.group)
    elif acc is None:
        return rho if on_device else rho.cpu().numpy()
    rho = rho + dmrg.noise * noise_dense.reshape(n, n)
    return rho if on_device else rho.cpu().numpy()
