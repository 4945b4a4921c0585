"""Integral input for the driver.

* ``read_fcidump``: FCIDUMP text (8-fold symmetric chemist (ij|kl), 1-based,
  core energy on the 0 0 0 0 line), as ``itools/fromFCIDUMP/tools_io.py:19-52``
  consumes it.
* ``spin_orbital``: the reference's MPO integral convention
  (``itools/fromFCIDUMP/tools_itrf.py:20-35``): alpha/beta interleaved
  spin orbitals, <ij|kl> = (ik|jl), int2e = V_pqrs = -1/2 (<pq|rs> - <pq|sr>).
* ``synthetic``: the seeded generator of the benchmark workloads: symmetric
  h1e with diagonal ~ N(-1, 0.1), nearest-neighbour hopping -hop, other
  entries N(0, 0.05); (pq|rs) = sum_L B[L,pq] B[L,rs] with B ~ N(0, 0.3/sqrt K)
  of shape (3K, K(K+1)/2) over symmetric pairs (8-fold symmetric, positive
  semidefinite); nuclear repulsion 0.  One ``numpy.random.default_rng(seed)``
  stream drives h1e (upper triangle, then the diagonal) and then B.
"""
import numpy


def read_fcidump(path):
    with open(path) as f:
        text = f.read()
    head, _, body = text.partition('&END') if '&END' in text else text.partition('/')
    fields = head.replace(',', ' ').replace('&FCI', ' ').split()
    kv = {}
    for i, tok in enumerate(fields):
        if '=' in tok:
            k, v = tok.split('=', 1)
            kv[k.upper()] = v if v else (fields[i + 1] if i + 1 < len(fields) else '')
    norb = int(kv['NORB'])
    out = dict(norb=norb, nelec=int(kv.get('NELEC', 0)), ms2=int(kv.get('MS2', 0)),
               h1e=numpy.zeros((norb, norb)), eri=numpy.zeros((norb,) * 4), ecore=0.0)
    data = numpy.array([row.split() for row in body.splitlines() if len(row.split()) == 5],
                       dtype=float).reshape(-1, 5)
    idx = data[:, 1:].astype(int) - 1
    for v, (i, j, k, l) in zip(data[:, 0], idx):
        if k < 0 and l < 0:
            if i < 0 and j < 0:
                out['ecore'] = v
            else:
                out['h1e'][i, j] = out['h1e'][j, i] = v
        else:
            e = out['eri']
            e[i, j, k, l] = e[j, i, k, l] = e[i, j, l, k] = e[j, i, l, k] = v
            e[k, l, i, j] = e[l, k, i, j] = e[k, l, j, i] = e[l, k, j, i] = v
    return out


def synthetic(K, seed, hop=1.0):
    rng = numpy.random.default_rng(seed)
    off = numpy.triu(rng.normal(0.0, 0.05, size=(K, K)), 1)
    off[numpy.arange(K - 1), numpy.arange(1, K)] = -hop
    h1e = off + off.T
    h1e[numpy.diag_indices(K)] = rng.normal(-1.0, 0.1, size=K)
    iu = numpy.triu_indices(K)
    B = rng.normal(0.0, 0.3 / numpy.sqrt(K), size=(3 * K, iu[0].size))
    Bf = numpy.zeros((3 * K, K, K))
    Bf[:, iu[0], iu[1]] = B
    Bf[:, iu[1], iu[0]] = B
    X = Bf.reshape(3 * K, K * K)
    eri = (X.T @ X).reshape(K, K, K, K)
    return h1e, eri, 0.0


def spin_orbital(h1e, eri):
    """Returns (int1e, int2e) for the MPO (V = -1/2 <pq||rs>)."""
    K = h1e.shape[0]
    n = 2 * K
    int1e = numpy.zeros((n, n))
    int1e[0::2, 0::2] = h1e
    int1e[1::2, 1::2] = h1e
    chem = numpy.zeros((n, n, n, n))
    for s in (0, 1):
        for t in (0, 1):
            chem[s::2, s::2, t::2, t::2] = eri
    g = chem.transpose(0, 2, 1, 3)
    int2e = -0.5 * (g - g.transpose(0, 1, 3, 2))
    return int1e, int2e


def closed_shell_occun(K, nelec, sz=0.0):
    """Aufbau spin-orbital occupation (alpha on even, beta on odd orbitals)."""
    na = int(round(nelec / 2.0 + sz))
    nb = int(round(nelec / 2.0 - sz))
    occ = numpy.zeros(2 * K)
    occ[0:2 * na:2] = 1.0
    occ[1:2 * nb:2] = 1.0
    return occ
