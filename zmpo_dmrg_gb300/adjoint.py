"""Energy gradient with respect to the integrals at a converged MPS.

E(h1e, eri) = sum_p w_p <psi| H_p(h1e, eri) |psi> / <psi|psi> at a fixed MPS
psi (at a converged state the Hellmann-Feynman gradient).  E is linear in
every MPO site tensor W_p(j), so

    dE/dW_p(j)[a,b,n',n] = sum L_p(j-1)[a,l,l'] A_j[l,n',r] A_j[l',n,r'] R_p(j+1)[b,r,r']

with L and R the environments of the same MPS (exact for any gauge: the
left-canonical sites of the last sweep serve for both sides).  These site
gradients are engine contractions (three per term and site, block-sparse,
FP64 on the GPU); the chain rule through the MPO construction is the
transposed builder (``mpo.hp_spatial_site_adjoint``: every site tensor is
linear in the integrals) and through the spin-orbital expansion of the
integrals torch autograd.  ``EnergyGradient`` is
the ``torch.autograd.Function`` wrapping it: forward returns E, backward
dE/dh1e (K x K) and dE/d(pq|rs) (K^4).

For the reference, dE/dh1e is the spin-summed one-particle density matrix
(``properties/mpo_dmrg_propsItrf.eval_rdm1BF``, propsItrf.py:204-263) and
dE/d(pq|rs) half the two-particle one (``genMPO_Apqrs`` with ``evalProps``,
propsMPO.py:73-113).
"""
import numpy

from . import engine as _engine
from . import mpo as _mpo
from .mpo import op_class
from .qtensor import qtensor


def _torch():
    import torch
    return torch


def spin_orbital_torch(h1e, eri):
    """Differentiable copy of ``integrals.spin_orbital`` (torch tensors)."""
    torch = _torch()
    K = h1e.shape[0]
    n = 2 * K
    int1e = torch.zeros((n, n), dtype=h1e.dtype, device=h1e.device)
    int1e[0::2, 0::2] = h1e
    int1e[1::2, 1::2] = h1e
    chem = torch.zeros((n, n, n, n), dtype=eri.dtype, device=eri.device)
    for s in (0, 1):
        for t in (0, 1):
            chem[s::2, s::2, t::2, t::2] = eri
    g = chem.permute(0, 2, 1, 3)
    int2e = -0.5 * (g - g.permute(0, 1, 3, 2))
    return int1e, int2e


def _right_convention(site, qkey):
    """A left-canonical site [l, n, r] (status F,F,T) relabelled as a site of
    the right block (status T,F,F; labels qkey - q on both bonds): the same
    allowed blocks and packing, so the values carry over unchanged."""
    t = qtensor([True, False, False])
    q = [qkey - site.qsyms[0], site.qsyms[1], qkey - site.qsyms[2]]
    t.fromQsyms(3, q, site.ndims, ifallocate=False)
    if t.size_allowed != site.size_allowed or not numpy.array_equal(t.blk_flat, site.blk_flat):
        raise RuntimeError("site relabelling changed the block structure")
    t.value = site.value
    t.idlst = site.idlst
    return t


class _GradChain:
    """Three contractions of one operator class at one site:
    t1 = A . L over the bra left bond, u = t1 . A over the ket left bond,
    G = u . Rf over both right bonds -> G[n', a, n, b]."""

    def __init__(self, eng, lay_site, lay_L, lay_Rf):
        lo1, self.p1 = eng.contract_plan(lay_site, lay_L, ([0], [1]))
        lo2, self.p2 = eng.contract_plan(lo1, lay_site, ([3], [0]))
        self.lay_out, self.p3 = eng.contract_plan(lo2, lay_Rf, ([1, 4], [1, 2]))
        self.sizes = [eng.layout_blocks(x)[0] for x in (lo1, lo2, self.lay_out)]

    def release(self, eng):
        for p in (self.p1, self.p2, self.p3):
            eng.destroy_plan(p)


def right_environments(dmrg, fmps):
    """R_p(j) for j = nsite-1 .. 0 from the left-canonical sites."""
    from .mpo_dmrg_kernel import renorm
    nsite = dmrg.nsite
    qkey = numpy.asarray(fmps['qnum%d' % nsite], dtype=float)[0]
    envs = {nsite: dmrg.boundary_env()}
    for j in range(nsite - 1, -1, -1):
        site = _right_convention(fmps['site%d' % j], qkey)
        fN = [[None, None]]
        renorm(dmrg, j, 1, [[None, envs[j + 1]]], fN, site, 'R')
        envs[j] = fN[0][0]
    return envs, qkey


def _left_step(dmrg, j, fL, site):
    """L(j) from L(j-1) and the left-canonical site j (one renormalisation)."""
    from .mpo_dmrg_kernel import renorm
    fN = [[None, None]]
    renorm(dmrg, j, 1, [[fL, None]], fN, site, 'L')
    return fN[0][0]


def _right_step(dmrg, j, fR, site, qkey):
    """R(j) from R(j+1) and site j in the right block's labels."""
    from .mpo_dmrg_kernel import renorm
    fN = [[None, None]]
    renorm(dmrg, j, 1, [[None, fR]], fN, _right_convention(site, qkey), 'R')
    return fN[0][0]


def checkpoint_stride(nsite):
    """Sites between kept left environments when they are recomputed:
    ceil(sqrt(nsite)), so about 2 sqrt(nsite) environments are held at once."""
    return max(1, int(numpy.ceil(numpy.sqrt(nsite))))


def left_env_schedule(nsite, stride):
    """The left environments the recompute mode holds.  The forward pass
    keeps the checkpoints L(c), c = -1 and c = stride-1, 2 stride-1, ...;
    then the sites are taken from j = nsite-1 down to 0, site j needing
    L(j-1): when that is not held, the segment L(c+1) .. L(j-1) is
    recomputed from the nearest checkpoint c below it, and after site j
    every L(x) with x >= j-1 is dropped (no later site needs it).  Returns,
    per site j in that order, (the segment's first index, or None when
    nothing is recomputed; the indices held while site j is taken)."""
    checkpoints = {-1} | set(range(stride - 1, nsite, stride))
    held = set(checkpoints)
    out = []
    for j in range(nsite - 1, -1, -1):
        need = j - 1
        seg = None
        if need not in held:
            c = max(x for x in held if x < need)
            seg = c + 1
            held |= set(range(seg, need + 1))
        out.append((seg, sorted(held)))
        held = {x for x in held if x < need}
    return out


def _site_gradient(dmrg, eng, j, site, fL, fR, qkey, norm2, grads):
    """dE/dW_p(j) of every term present in both environments."""
    torch = _torch()
    mpo = dmrg.mpo_store
    sval = torch.from_numpy(numpy.ascontiguousarray(site.value)).cuda()
    chains = {}
    for iop in range(dmrg.nops):
        if not (fL.present(iop) and fR.present(iop)):
            continue
        c0 = op_class(dmrg.opers[iop][0], j)
        if c0 not in chains:
            rt = fR.tensors[iop]
            lay_rf = eng.derive(rt.layout, [-rt.qsyms[0], qkey - rt.qsyms[1], qkey - rt.qsyms[2]],
                                rt.status)
            chains[c0] = _GradChain(eng, site.layout, fL.layouts[iop], lay_rf)
        ch = chains[c0]
        lv = fL.buf.narrow(0, int(fL.off[iop]), fL.tensors[iop].size_allowed)
        rv = fR.buf.narrow(0, int(fR.off[iop]), fR.tensors[iop].size_allowed)
        t1 = torch.empty(max(ch.sizes[0], 1), dtype=torch.float64, device="cuda")
        t2 = torch.empty(max(ch.sizes[1], 1), dtype=torch.float64, device="cuda")
        g = torch.empty(max(ch.sizes[2], 1), dtype=torch.float64, device="cuda")
        eng.contract_exec(ch.p1, sval, lv, t1)
        eng.contract_exec(ch.p2, t1, sval, t2)
        eng.contract_exec(ch.p3, t2, rv, g)
        wt = mpo.tensors[j][iop]
        # legs [n', a, n, b]: directions follow the contraction (bra
        # site against the bra leg of L, ket legs against ket legs)
        out = qtensor([False, False, True, True])
        out.fromQsyms(4, [site.qsyms[1], wt.qsyms[0], site.qsyms[1], wt.qsyms[1]],
                      [site.ndims[1], wt.ndims[0], site.ndims[1], wt.ndims[1]], ifallocate=False)
        size, flat, _ = eng.layout_blocks(ch.lay_out)
        if size != out.size_allowed or not numpy.array_equal(flat, out.blk_flat):
            raise RuntimeError("site gradient layout mismatch")
        out.value = g[:size].cpu().numpy()
        dense = out.toDenseTensor([site.idlst[1], wt.idlst[0], site.idlst[1], wt.idlst[1]])
        gq = dense.transpose(1, 3, 0, 2)            # [a, b, n', n] in sorted bond order
        il, ir = _mpo.bond_order(dmrg.opers[iop], dmrg.sbas, j)
        gb = numpy.zeros_like(gq)
        gb[numpy.ix_(il, ir)] = gq
        grads[j][iop] = dmrg.hpwts[iop] * gb / norm2
    for ch in chains.values():
        ch.release(eng)


def needs_recompute(env_bytes, free_bytes, margin=0.5):
    """Whether the energy gradient should recompute its environments: the
    stored mode makes one more full set of environments next to the ones the
    driver holds (``env_bytes``, estimated by their size); it is used while
    that stays below ``margin`` of the free device memory."""
    return env_bytes > margin * free_bytes


def _held_env_bytes(dmrg):
    """Bytes of the environment sets the driver holds (every bond, both sides)."""
    return sum(int(env.buf.numel()) * 8 for env in dmrg.envs.values() if env is not None)


def site_gradients(dmrg, fmps=None, recompute_envs=None):
    """dE/dW_p(j) for every site j and term p as dense [Dw_l, Dw_r, 4, 4]
    arrays in the builder's bond order, and <H> and <psi|psi> of the MPS.

    By default every left and right environment of the MPS is made once and
    kept (2 nsite environment sets on the device).  With ``recompute_envs``
    (default ``dmrg.adjoint_recompute_envs``, False) they are recomputed
    where memory requires it: the sites are taken from right to left with
    one right environment carried along, and the left environments are kept
    only at checkpoints every ``checkpoint_stride(nsite)`` sites, the ones
    between recomputed from the nearest checkpoint when they are needed
    (``left_env_schedule``): about 2 sqrt(nsite) environment sets held and
    one more left renormalisation per site.  The same renormalisations run
    on the same inputs, so both modes give the same gradients.  When neither
    the argument nor the attribute chooses, the mode follows the memory:
    recompute when another full set of environments would not fit
    (``needs_recompute``)."""
    if dmrg.ifs2proj:
        raise NotImplementedError("energy gradient of the spin-projected energy")
    if recompute_envs is None:
        recompute_envs = getattr(dmrg, "adjoint_recompute_envs", None)
    if recompute_envs is None:
        free, _ = _torch().cuda.mem_get_info()
        recompute_envs = needs_recompute(_held_env_bytes(dmrg), free)
    fmps = dmrg.flmps if fmps is None else fmps
    eng = _engine.get()
    nsite = dmrg.nsite
    last = fmps['site%d' % (nsite - 1)]
    norm2 = float(numpy.dot(last.value, last.value))
    grads = [[None] * dmrg.nops for _ in range(nsite)]
    if not recompute_envs:
        exphop = dmrg.genHops(fmps, 'lop')
        esum = float(numpy.dot(dmrg.hpwts, exphop))
        Lenv = {j: dmrg.envs[('lop', j)] for j in range(-1, nsite)}
        Renv, qkey = right_environments(dmrg, fmps)
        for j in range(nsite):
            _site_gradient(dmrg, eng, j, fmps['site%d' % j], Lenv[j - 1], Renv[j + 1], qkey, norm2, grads)
        return grads, esum / norm2, norm2
    stride = checkpoint_stride(nsite)
    schedule = left_env_schedule(nsite, stride)
    checkpoints = {-1} | set(range(stride - 1, nsite, stride))
    # forward pass: left environments, kept at the checkpoints only
    L = {-1: dmrg.boundary_env()}
    fL = L[-1]
    for j in range(nsite):
        fL = _left_step(dmrg, j, fL, fmps['site%d' % j])
        if j in checkpoints:
            L[j] = fL
    esum = float(numpy.dot(dmrg.hpwts, dmrg._scalars(fL, dmrg.nops)))
    del fL
    qkey = numpy.asarray(fmps['qnum%d' % nsite], dtype=float)[0]
    fR = dmrg.boundary_env()
    for (seg, held), j in zip(schedule, range(nsite - 1, -1, -1)):
        if seg is not None:
            fL = L[seg - 1]
            for i in range(seg, j):
                fL = _left_step(dmrg, i, fL, fmps['site%d' % i])
                L[i] = fL
            del fL
        if sorted(L) != held:
            raise RuntimeError("left environment schedule out of step")
        site = fmps['site%d' % j]
        _site_gradient(dmrg, eng, j, site, L[j - 1], fR, qkey, norm2, grads)
        for x in [x for x in L if x >= j - 1]:
            del L[x]
        if j > 0:
            fR = _right_step(dmrg, j, fR, site, qkey)
    return grads, esum / norm2, norm2


def integral_gradients(dmrg, h1e, eri, grads):
    """Chain rule from the site gradients to dE/dh1e and dE/d(pq|rs)
    (spatial orbitals).  Every W_p(j) is linear in the spin-orbital rows
    int1e[p], int2e[p], so their gradients are the transposed builder applied
    to the site gradients (``mpo.hp_spatial_site_adjoint``, NumPy); the small
    spin-orbital expansion of the spatial integrals is differentiated by
    torch autograd."""
    torch = _torch()
    from .integrals import spin_orbital
    i1, i2 = spin_orbital(numpy.asarray(h1e, dtype=float), numpy.asarray(eri, dtype=float))
    i1, i2 = i1[dmrg.pidx], i2[dmrg.pidx]
    d1 = numpy.zeros_like(i1)
    d2 = numpy.zeros_like(i2)
    for j in range(dmrg.nsite):
        for iop in range(dmrg.nops):
            G = grads[j][iop]
            if G is None:
                continue
            idx, dh, dv = _mpo.hp_spatial_site_adjoint(dmrg.opers[iop], dmrg.sbas, j, i1, i2, G, dmrg.pdic)
            d1[idx] += dh
            d2[idx] += dv
    with torch.enable_grad():   # also when called from a Function's backward
        h = torch.tensor(numpy.asarray(h1e, dtype=float), requires_grad=True)
        g = torch.tensor(numpy.asarray(eri, dtype=float), requires_grad=True)
        int1e, int2e = spin_orbital_torch(h, g)
        total = (int1e[dmrg.pidx] * torch.from_numpy(d1)).sum() + (int2e[dmrg.pidx] * torch.from_numpy(d2)).sum()
        total.backward()
    return h.grad.numpy().copy(), g.grad.numpy().copy()


def symmetrize_eri_gradient(d):
    """Average over the eight index permutations that leave (pq|rs) invariant."""
    perms = [(0, 1, 2, 3), (1, 0, 2, 3), (0, 1, 3, 2), (1, 0, 3, 2),
             (2, 3, 0, 1), (3, 2, 0, 1), (2, 3, 1, 0), (3, 2, 1, 0)]
    return sum(d.transpose(p) for p in perms) / 8.0


def _make_function():
    torch = _torch()

    class EnergyGradient(torch.autograd.Function):
        """E(h1e, eri) at the MPS held by ``dmrg``; backward is the adjoint of
        the H.psi contraction (site gradients) chained through the builder."""

        @staticmethod
        def forward(ctx, h1e, eri, dmrg):
            from .integrals import spin_orbital
            int1e, int2e = spin_orbital(h1e.detach().cpu().numpy(), eri.detach().cpu().numpy())
            dmrg.loadInts((int1e, int2e))
            dmrg.dumpMPO()
            grads, energy, _ = site_gradients(dmrg)
            ctx.saved = (dmrg, h1e.detach().cpu().numpy(), eri.detach().cpu().numpy(), grads)
            return torch.tensor(energy, dtype=torch.float64)

        @staticmethod
        def backward(ctx, gout):
            dmrg, h1e, eri, grads = ctx.saved
            dh, dg = integral_gradients(dmrg, h1e, eri, grads)
            s = float(gout)
            return torch.from_numpy(dh * s), torch.from_numpy(dg * s), None

    return EnergyGradient


_FN = None


def energy(h1e, eri, dmrg):
    """E at the MPS of ``dmrg`` as a differentiable function of the spatial
    integrals (torch float64 tensors)."""
    global _FN
    if _FN is None:
        _FN = _make_function()
    return _FN.apply(h1e, eri, dmrg)
