"""Integral input and an exact (FCI) reference for the oracle.

* ``read_fcidump`` restates ``source/itools/fromFCIDUMP/tools_io.py:19-52``
  (8-fold symmetric chemist (ij|kl), 1-based indices, core energy on 0 0 0 0).
* ``to_spin_orbital`` restates ``source/itools/fromFCIDUMP/tools_itrf.py:20-35``:
  alpha/beta interleaved, <ij|kl> = (ik|jl), V_pqrs = -1/2 (<pq|rs> - <pq|sr>).
* ``synthetic`` is the seeded generator the benchmark configurations name:
  symmetric h1e with diag ~ N(-1, 0.1), nearest-neighbour hopping ``-hop``,
  other entries N(0, 0.05); (pq|rs) = sum_L B[L,pq] B[L,rs], B ~ N(0, 0.3/sqrt K)
  of shape (3K, K(K+1)/2) over symmetric pairs; nuclear repulsion 0.
* ``fci_hamiltonian`` builds the exact Jordan-Wigner H in the MPS product basis
  (spatial site basis [0, b, a, ab], index 2 n_a + n_b, site 0 most significant).
"""
import itertools
import numpy
import scipy.sparse
import scipy.sparse.linalg


def read_fcidump(path):
    with open(path) as f:
        lines = f.read().splitlines()
    header = []
    body = 0
    for i, line in enumerate(lines):
        header.append(line)
        if '&END' in line.upper() or line.strip() == '/':
            body = i + 1
            break
    htxt = ' '.join(header).replace(',', ' ')
    tok = htxt.split()

    def _get(name):
        for j, t in enumerate(tok):
            if t.upper().startswith(name + '='):
                v = t.split('=')[1]
                return int(v) if v else int(tok[j + 1])
        raise KeyError(name)

    norb = _get('NORB')
    nelec = _get('NELEC')
    ms2 = _get('MS2')
    h1e = numpy.zeros((norb, norb))
    eri = numpy.zeros((norb, norb, norb, norb))
    ecore = 0.0
    for line in lines[body:]:
        data = line.split()
        if len(data) < 5:
            continue
        val = float(data[0])
        i, j, k, l = [int(x) - 1 for x in data[1:5]]
        if k == -1 and l == -1:
            if i == -1 and j == -1:
                ecore = val
            else:
                h1e[i, j] = h1e[j, i] = val
        else:
            for a, b, c, d in ((i, j, k, l), (j, i, k, l), (i, j, l, k), (j, i, l, k),
                               (k, l, i, j), (l, k, i, j), (k, l, j, i), (l, k, j, i)):
                eri[a, b, c, d] = val
    return dict(norb=norb, nelec=nelec, ms2=ms2, h1e=h1e, eri=eri, ecore=ecore)


def synthetic(K, seed, hop=1.0):
    rng = numpy.random.default_rng(seed)
    h1e = rng.normal(0.0, 0.05, size=(K, K))
    h1e = numpy.triu(h1e, 1)
    for i in range(K - 1):
        h1e[i, i + 1] = -hop
    h1e = h1e + h1e.T
    h1e[numpy.diag_indices(K)] = rng.normal(-1.0, 0.1, size=K)
    npair = K * (K + 1) // 2
    B = rng.normal(0.0, 0.3 / numpy.sqrt(K), size=(3 * K, npair))
    Bf = numpy.zeros((3 * K, K, K))
    iu = numpy.triu_indices(K)
    Bf[:, iu[0], iu[1]] = B
    Bf[:, iu[1], iu[0]] = B
    eri = numpy.einsum('Lpq,Lrs->pqrs', Bf, Bf)
    return h1e, eri, 0.0


def to_spin_orbital(h1e, eri):
    """Returns (int1e, int2e) in the reference's MPO convention plus the
    physicist-notation spin-orbital <pq|rs> used by the exact Hamiltonian."""
    nbas = h1e.shape[0]
    sbas = 2 * nbas
    int1e = numpy.zeros((sbas, sbas))
    int1e[0::2, 0::2] = h1e
    int1e[1::2, 1::2] = h1e
    h2e = numpy.zeros((sbas, sbas, sbas, sbas))
    h2e[0::2, 0::2, 0::2, 0::2] = eri
    h2e[1::2, 1::2, 1::2, 1::2] = eri
    h2e[0::2, 0::2, 1::2, 1::2] = eri
    h2e[1::2, 1::2, 0::2, 0::2] = eri
    gphys = h2e.transpose(0, 2, 1, 3).copy()
    int2e = -0.5 * (gphys - gphys.transpose(0, 1, 3, 2))
    return int1e, int2e, gphys


def _jw_ops(sbas):
    sgn = scipy.sparse.csr_matrix(numpy.diag([1., -1.]))
    idn = scipy.sparse.identity(2, format='csr')
    ann = scipy.sparse.csr_matrix(numpy.array([[0., 1.], [0., 0.]]))
    ops = []
    for p in range(sbas):
        mats = [sgn] * p + [ann] + [idn] * (sbas - p - 1)
        op = mats[0]
        for m in mats[1:]:
            op = scipy.sparse.kron(op, m, format='csr')
        ops.append(op)
    return ops


def fci_hamiltonian(int1e, gphys):
    """H = sum h_pq a+_p a_q + 1/2 sum <pq|rs> a+_p a+_q a_s a_r (sparse)."""
    sbas = int1e.shape[0]
    a = _jw_ops(sbas)
    ad = [x.T.tocsr() for x in a]
    dim = 2 ** sbas
    H = scipy.sparse.csr_matrix((dim, dim))
    for p, q in itertools.product(range(sbas), repeat=2):
        if int1e[p, q] != 0.0:
            H = H + int1e[p, q] * (ad[p] @ a[q])
    pairs_c = {}
    for p, q in itertools.product(range(sbas), repeat=2):
        if p != q:
            pairs_c[(p, q)] = ad[p] @ ad[q]
    pairs_a = {}
    for s, r in itertools.product(range(sbas), repeat=2):
        if s != r:
            pairs_a[(s, r)] = a[s] @ a[r]
    for (p, q), cc in pairs_c.items():
        acc = None
        for (s, r), aa in pairs_a.items():
            v = gphys[p, q, r, s]
            if v == 0.0:
                continue
            term = v * aa
            acc = term if acc is None else acc + term
        if acc is not None:
            H = H + 0.5 * (cc @ acc)
    return H.tocsr()


def sector_indices(sbas, nelec, sz):
    """Product-basis states with N = nelec and Sz = sz (alpha = even spin orbital)."""
    out = []
    for idx in range(2 ** sbas):
        bits = [(idx >> (sbas - 1 - p)) & 1 for p in range(sbas)]
        n = sum(bits)
        s = 0.5 * (sum(bits[0::2]) - sum(bits[1::2]))
        if n == nelec and abs(s - sz) < 1e-12:
            out.append(idx)
    return numpy.array(out)


def fci_energy(int1e, gphys, nelec, sz, nroots=1):
    H = fci_hamiltonian(int1e, gphys)
    idx = sector_indices(int1e.shape[0], nelec, sz)
    Hs = H[idx][:, idx].toarray()
    e = numpy.linalg.eigvalsh(Hs)
    return e[:nroots]


def spin_ops(sbas):
    """S+ and S_z (sparse) with alpha = even spin orbital."""
    a = _jw_ops(sbas)
    K = sbas // 2
    sp = a[0].T @ a[1]
    for i in range(1, K):
        sp = sp + a[2 * i].T @ a[2 * i + 1]
    nup = a[0].T @ a[0]
    ndn = a[1].T @ a[1]
    for i in range(1, K):
        nup = nup + a[2 * i].T @ a[2 * i]
        ndn = ndn + a[2 * i + 1].T @ a[2 * i + 1]
    return sp.tocsr(), (0.5 * (nup - ndn)).tocsr()


def fci_spin_energy(int1e, gphys, nelec, sz, sval, nroots=1):
    """Lowest eigenvalues of H restricted to S^2 = sval(sval+1) in the
    (nelec, sz) sector (H and S^2 are diagonalised jointly)."""
    sbas = int1e.shape[0]
    H = fci_hamiltonian(int1e, gphys)
    sp, szm = spin_ops(sbas)
    s2 = (sp.T @ sp + szm @ szm + szm).tocsr()
    idx = sector_indices(sbas, nelec, sz)
    Hs = H[idx][:, idx].toarray()
    S2 = s2[idx][:, idx].toarray()
    w, v = numpy.linalg.eigh(S2)
    sel = numpy.abs(w - sval * (sval + 1.0)) < 1e-8
    if not numpy.any(sel):
        return numpy.zeros(0)
    u = v[:, sel]
    e = numpy.linalg.eigvalsh(u.T @ Hs @ u)
    return e[:nroots]
