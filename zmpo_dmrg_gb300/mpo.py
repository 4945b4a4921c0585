"""MPO site tensors of H = sum_p a_p^+ V_p for the engine.

The bond-index layout is the reference's MPO format (it fixes the structure
of every environment, so it has to be the same): spin-orbital site ``k`` of
``nsite`` spin orbitals carries a bond of dimension 2(nsite+1) ordered as
``mpo_dmrg_opers.genWfacSpin`` (source/mpo_dmrg_opers.py:91-194) orders it;
H_p = a_p^+ V_p (``genHfacSpin`` 197-203); a spatial site joins spin sites
(2i, 2i+1) (``linkTwoOpers`` 43-49); spin projection multiplies the ket leg by
exp(-i theta S_y) (``genHRfacSpatial`` 253-260).  The block-sparse form sorts
the bond quantum numbers and collects equal ones into sectors, with physical
legs uncollected (``qtensor_opers.genHRfacSpatialQt`` 358-408); the bond
order inside a sector is ascending in the (N, Sz) label.
"""
import math

import numpy

from .qtensor import qtensor

# local 2x2 operators on [|0>, |1>] of one spin orbital
_I = numpy.eye(2)
_Z = numpy.diag([1.0, -1.0])      # Jordan-Wigner sign (also the "idnt" string)
_C = numpy.array([[0.0, 0.0], [1.0, 0.0]])   # creation
_A = numpy.array([[0.0, 1.0], [0.0, 0.0]])   # annihilation
_N = numpy.array([[0.0, 0.0], [0.0, 1.0]])   # number


class _Backend:
    """Array operations for the builder: NumPy (the site tensors the engine
    uploads) or torch (the same tensors as a differentiable function of the
    integrals, for the energy gradient)."""

    def __init__(self, like):
        self.torch = not isinstance(like, numpy.ndarray)
        if self.torch:
            import torch
            self.t = torch
            kw = dict(dtype=like.dtype, device=like.device)
            self.kw = kw
            self.I, self.Z, self.C, self.A, self.N = (torch.as_tensor(x, **kw) for x in (_I, _Z, _C, _A, _N))
        else:
            self.I, self.Z, self.C, self.A, self.N = _I, _Z, _C, _A, _N

    def zeros(self, shape):
        return self.t.zeros(shape, **self.kw) if self.torch else numpy.zeros(shape)

    def arange(self, a, b=None):
        if b is None:
            a, b = 0, a
        if self.torch:
            return self.t.arange(a, b, device=self.kw["device"])
        return numpy.arange(a, b)

    def matmul(self, a, b):
        return self.t.matmul(a, b) if self.torch else numpy.matmul(a, b)


def spin_site(nsite, k, h, v):
    """V_p MPO on spin orbital ``k``: ``h[q]`` = h_pq, ``v[q,r,s]`` = V_pqrs
    (NumPy arrays, or float64 torch tensors for a differentiable build)."""
    B = _Backend(h)
    nl = 1 if k == 0 else 2 * (nsite + 1)
    nr = 1 if k == nsite - 1 else 2 * (nsite + 1)
    W = B.zeros((nl, nr, 2, 2))
    L = k                 # spin orbitals left of k
    R = nsite - k - 1     # spin orbitals right of k
    right = B.arange(k + 1, nsite)
    left = B.arange(k)
    rr = B.arange(R)
    last = nr - 1
    if k == nsite - 1:
        W[0, 0] = h[k] * B.A
        W[1, 0] = B.C
        W[2, 0] = B.A
        W[3 + left, 0] = v[k, left, k][:, None, None] * B.N
        W[nl - 1, 0] = B.I
        return W
    # first row: string, V(k,k,r) n_k, -a_k, a+_k, h_k a_k
    W[0, 0] = B.Z
    W[0, 1 + R + rr] = v[k, k, right][:, None, None] * (-B.N)
    W[0, 1 + 2 * R + L] = -B.A
    W[0, 2 + 2 * R + 2 * L] = B.C
    W[0, last] = h[k] * B.A
    if k == 0:
        return W
    W[1, last] = B.C
    W[2 + rr, 1 + rr] = B.Z
    W[2 + R, last] = B.A
    W[3 + R + rr, 1 + R + rr] = B.Z
    o6 = 3 + 2 * R
    for li in range(L):
        W[o6 + li, 1 + rr] = -v[right, li, k][:, None, None] * (-B.A)
        W[o6 + li, 1 + R + rr] = v[k, li, right][:, None, None] * B.C
        W[o6 + li, 1 + 2 * R + li] = B.I
        W[o6 + li, last] = v[k, li, k] * B.N
    o7 = 3 + 2 * R + L
    for li in range(L):
        W[o7 + li, 1 + R + rr] = v[li, k, right][:, None, None] * (-B.A)
        W[o7 + li, 2 + 2 * R + L + li] = B.I
    W[nl - 1, last] = B.I
    return W


def spin_site_adjoint(nsite, k, G):
    """Gradient of <G, spin_site(nsite, k, h, v)> with respect to h and v
    (spin_site is linear in them): the transpose of its assignments, as
    NumPy arrays dh [nsite], dv [nsite, nsite, nsite]."""
    dh = numpy.zeros(nsite)
    dv = numpy.zeros((nsite, nsite, nsite))
    nr = 1 if k == nsite - 1 else 2 * (nsite + 1)
    L, R = k, nsite - k - 1
    right = numpy.arange(k + 1, nsite)
    left = numpy.arange(k)
    rr = numpy.arange(R)
    last = nr - 1

    def ip(X, M):  # <X[..., i, j], M[i, j]>
        return numpy.tensordot(X, M, axes=([-2, -1], [0, 1]))

    if k == nsite - 1:
        dh[k] += ip(G[0, 0], _A)
        dv[k, left, k] += ip(G[3 + left, 0], _N)
        return dh, dv
    dv[k, k, right] += ip(G[0, 1 + R + rr], -_N)
    dh[k] += ip(G[0, last], _A)
    if k == 0:
        return dh, dv
    o6 = 3 + 2 * R
    for li in range(L):
        dv[right, li, k] += ip(G[o6 + li, 1 + rr], _A)       # -v * (-A)
        dv[k, li, right] += ip(G[o6 + li, 1 + R + rr], _C)
        dv[k, li, k] += ip(G[o6 + li, last], _N)
    o7 = 3 + 2 * R + L
    for li in range(L):
        dv[li, k, right] += ip(G[o7 + li, 1 + R + rr], -_A)
    return dh, dv


def hp_spatial_site_adjoint(pindx, nspin, isite, int1e, int2e, G, pdic=None):
    """Gradient of <G, hp_spatial_site(...)> with respect to the spin-orbital
    rows int1e[idx] and int2e[idx] of term p (the site is linear in them):
    G [Dw_l, Dw_r, 4, 4] in the builder's bond order.  Returns (idx, dh, dv)."""
    p, ipt = pindx
    if ipt is not None:
        raise NotImplementedError("adjoint of the spin-projected site")
    idx = p if pdic is None else pdic[p]
    h, v = int1e[idx], int2e[idx]
    k0, k1 = 2 * isite, 2 * isite + 1
    e0, e1 = _elem(p, k0), _elem(p, k1)
    W1 = numpy.matmul(e0, spin_site(nspin, k0, h, v))
    W2 = numpy.matmul(e1, spin_site(nspin, k1, h, v))
    # link: W[a, c, (i k), (j l)] = sum_b W1[a, b, i, j] W2[b, c, k, l]
    G6 = G.reshape(G.shape[0], G.shape[1], 2, 2, 2, 2)        # [a, c, i, k, j, l]
    dW1 = numpy.einsum('acikjl,bckl->abij', G6, W2, optimize=True)
    dW2 = numpy.einsum('acikjl,abij->bckl', G6, W1, optimize=True)
    # hp_spin_site: e @ W over the row index of the local operator
    dh0, dv0 = spin_site_adjoint(nspin, k0, numpy.matmul(e0.T, dW1))
    dh1, dv1 = spin_site_adjoint(nspin, k1, numpy.matmul(e1.T, dW2))
    return idx, dh0 + dh1, dv0 + dv1


def _elem(p, k):
    if k < p:
        return _Z
    return _C if k == p else _I


def hp_spin_site(p, nsite, k, h, v):
    """a_p^+ V_p on spin orbital k: the local a_p^+ factor acts after V_p."""
    W = spin_site(nsite, k, h, v)
    B = _Backend(h)
    e = _elem(p, k)
    if B.torch:
        e = B.t.as_tensor(e, **B.kw)
    return B.matmul(e, W)


def link(W1, W2):
    """Join two sites: [a,b,i,j] x [b,c,k,l] -> [a,c,(ik),(jl)] (one GEMM over b)."""
    if not isinstance(W1, numpy.ndarray):
        import torch
        t = torch.tensordot(W1, W2, dims=([1], [0])).permute(0, 3, 1, 4, 2, 5)
        s = t.shape
        return t.reshape(s[0], s[1], s[2] * s[3], s[4] * s[5])
    t = numpy.tensordot(W1, W2, axes=([1], [0]))        # a,i,j,c,k,l
    t = t.transpose(0, 3, 1, 4, 2, 5)
    s = t.shape
    return numpy.ascontiguousarray(t).reshape(s[0], s[1], s[2] * s[3], s[4] * s[5])


def ry_matrix(phi):
    """exp(-i phi S_y) on the spatial basis [0, b, a, ab]."""
    m = numpy.eye(4)
    c, s = math.cos(0.5 * phi), math.sin(0.5 * phi)
    m[1, 1], m[1, 2], m[2, 1], m[2, 2] = c, s, -s, c
    return m


def hp_spatial_site(pindx, nspin, isite, int1e, int2e, qpts=None, pdic=None):
    p, ipt = pindx
    idx = p if pdic is None else pdic[p]
    W = link(hp_spin_site(p, nspin, 2 * isite, int1e[idx], int2e[idx]),
             hp_spin_site(p, nspin, 2 * isite + 1, int1e[idx], int2e[idx]))
    if ipt is not None:
        W = numpy.einsum('abij,jk->abik', W, ry_matrix(qpts[ipt]))
    return W


# --------------------------------------------------------- quantum numbers
_SPIN = (0.5, -0.5)


def _bond_right(nsite, k, sz):
    """(N, Sz) labels of the right bond of spin orbital k for V_p with
    Sz(p) = sz (qtensor_opers.genWfacSpinQnumsRight, qtensor_opers.py:161)."""
    q = [[0.0, 0.0]]
    q += [[-2.0, -sz - _SPIN[i % 2]] for i in range(k + 1, nsite)]
    q += [[0.0, -sz + _SPIN[i % 2]] for i in range(k + 1, nsite)]
    q += [[-1.0, -_SPIN[i % 2]] for i in range(k + 1)]
    q += [[1.0, _SPIN[i % 2]] for i in range(k + 1)]
    q += [[-1.0, -sz]]
    return numpy.array(q)


def _elem_q(p, k):
    """Label change of the a_p^+ factor across spin orbital k."""
    d = numpy.array([1.0, _SPIN[p % 2]])
    left = d if k > p else numpy.zeros(2)
    right = d if k >= p else numpy.zeros(2)
    return left, right


def spatial_bond_qnums(p, nspin, isite):
    """Left / right bond labels of H_p at spatial site ``isite``."""
    sz = _SPIN[p % 2]
    k0, k1 = 2 * isite, 2 * isite + 1
    ql = numpy.zeros((1, 2)) if k0 == 0 else _bond_right(nspin, k0 - 1, sz)
    qr = numpy.array([[-1.0, -sz]]) if k1 == nspin - 1 else _bond_right(nspin, k1, sz)
    el, _ = _elem_q(p, k0)
    _, er = _elem_q(p, k1)
    return ql + el, qr + er


def _bond_labels(pindx, nspin, isite):
    ql, qr = spatial_bond_qnums(pindx[0], nspin, isite)
    if pindx[1] is not None:
        ql, qr = ql[:, :1], qr[:, :1]
    return ql, qr


def bond_order(pindx, nspin, isite):
    """Permutations (left, right) from the builder's bond order to the
    block-sparse tensor's order (ascending label, stable)."""
    ql, qr = _bond_labels(pindx, nspin, isite)
    return numpy.lexsort(ql.T[::-1]), numpy.lexsort(qr.T[::-1])


def hp_spatial_qt(pindx, nspin, isite, int1e, int2e, qpts=None, pdic=None):
    """Block-sparse site tensor of H_p with bond sectors collected."""
    W = hp_spatial_site(pindx, nspin, isite, int1e, int2e, qpts, pdic)
    ql, qr = _bond_labels(pindx, nspin, isite)
    qphys = numpy.array([[0.0, 0.0], [1.0, -0.5], [1.0, 0.5], [2.0, 0.0]])
    if pindx[1] is not None:
        qphys = qphys[:, :1]
    il, ir = bond_order(pindx, nspin, isite)
    W = W[numpy.ix_(il, ir)]
    qt = qtensor([False, True, False, True])
    qt.fromDenseTensor(W, [ql[il], qr[ir], qphys, qphys], ifcollect=[1, 1, 0, 0])
    return qt


def op_class(p, isite, ncsite=1):
    """Layout class of H_p relative to the dot (qtensor_opers.case, qtensor_opers.py:72)."""
    i = p // 2
    odd = p % 2
    if i < isite:
        return odd
    if i == isite:
        return 2 + odd
    if ncsite == 1 or i == isite + 1:
        return 4 + odd
    return 6 + odd
