"""The tcgen05 kernels (csrc/kernels_umma.cu) against their exact model
(tests/split_model.py): every group whose whole K fits one exact pass (1 <= K
<= 256) and that has at least 64 rows runs on the tensor cores with
whole-K row and column exponents; longer groups (and the split-K parts of
groups longer than 2048 slots) run in exact passes of 256 slots summed in
FP64; the output must equal the model bit for bit.
Dense products over the edge shapes (K = 1 and 256, ragged rows and columns,
one to several column tiles and row-tile runs) and block-sparse contractions
of a DMRG dot (column-block groups, strided operands).  The kernel's error
word must stay clear."""
import numpy
import pytest

from tests.problems import random_problem, run_tasks_on_host
from tests.split_model import one_pass_gemm, long_gemm

pytestmark = pytest.mark.gpu

UMMA_MAX_K, UMMA_MIN_M = 256, 64


def routed(A, B):
    return A.shape[1] <= UMMA_MAX_K and A.shape[1] >= 1 and A.shape[0] >= UMMA_MIN_M


def model(A, B):
    """The tcgen05 routes' result for a group of the task model, None for a
    group the chunked kernels run (K <= 256 with fewer than 64 rows)."""
    K = A.shape[1]
    if K == 0:
        return None
    if K > UMMA_MAX_K:
        return long_gemm(A, B)
    return one_pass_gemm(A, B) if routed(A, B) else None


def _dense(eng, M, K, N, rng, spread):
    import torch
    q = numpy.zeros((1, 2))
    la = eng.layout([q, q], [[M], [K]], [False, True])
    lb = eng.layout([q, q], [[K], [N]], [False, True])
    lo, pid = eng.contract_plan(la, lb, ([1], [0]))
    A = rng.standard_normal((M, K)) * numpy.exp(rng.uniform(-spread, spread, (M, K)))
    B = rng.standard_normal((K, N)) * numpy.exp(rng.uniform(-spread, spread, (K, N)))
    A[rng.random((M, K)) < 0.05] = 0.0     # zeros, and a whole zero row
    A[min(3, M - 1), :] = 0.0
    a = torch.from_numpy(A.ravel().copy()).cuda()
    b = torch.from_numpy(B.ravel().copy()).cuda()
    out = torch.full((M * N,), numpy.nan, dtype=torch.float64, device="cuda")
    return pid, A, B, a, b, out


@pytest.mark.parametrize("M,K,N", [(64, 1, 16), (128, 16, 64), (130, 7, 3), (300, 33, 50), (257, 256, 64),
                                   (1000, 100, 130), (2100, 200, 407), (96, 255, 17), (128, 32, 33)])
def test_dense_one_pass_bit_exact(gpu, M, K, N):
    from zmpo_dmrg_gb300 import engine as E
    eng = E.get()
    rng = numpy.random.default_rng(M * 7 + K * 3 + N)
    for spread in (0.0, 6.0):
        pid, A, B, a, b, out = _dense(eng, M, K, N, rng, spread)
        eng.contract_exec(pid, a, b, out, "split")
        got = out.cpu().numpy().reshape(M, N)
        ref = one_pass_gemm(A, B)
        assert numpy.array_equal(got, ref), (spread, numpy.abs(got - ref).max())
        # and close to the FP64 product: per product a.b the digits drop at
        # most 2^-31 P of each operand (P = 2^(E-1022) <= 2 max|row| or
        # 2 max|column|) and the levels 4-6 at most 3.05 2^-32 Pa Pb, so
        # |error| <= 1.76 2^-30 Pa Pb <= 2^-27 K max|A_i.| max|B_.j|
        exact = A @ B
        scale = K * numpy.abs(A).max(axis=1)[:, None] * numpy.abs(B).max(axis=0)[None, :]
        assert (numpy.abs(got - exact) <= 2.0 ** -27 * scale + 1e-300).all()
        eng.destroy_plan(pid)
    assert eng.device_status() == 0


@pytest.mark.parametrize("M,K,N", [(200, 257, 40), (24, 300, 17), (100, 1000, 64), (130, 2048, 70),
                                   (64, 2049, 33), (7, 5000, 130), (300, 700, 16)])
def test_dense_long_k_bit_exact(gpu, M, K, N):
    """K > 256: exact passes of 256 slots summed in FP64 (and parts of 2048
    slots summed by the split-K reduction beyond that), any row count."""
    from zmpo_dmrg_gb300 import engine as E
    eng = E.get()
    rng = numpy.random.default_rng(M + 3 * K + 7 * N)
    for spread in (0.0, 6.0):
        pid, A, B, a, b, out = _dense(eng, M, K, N, rng, spread)
        eng.contract_exec(pid, a, b, out, "split")
        got = out.cpu().numpy().reshape(M, N)
        ref = long_gemm(A, B)
        assert numpy.array_equal(got, ref), (spread, numpy.abs(got - ref).max())
        exact = A @ B
        scale = K * numpy.abs(A).max(axis=1)[:, None] * numpy.abs(B).max(axis=0)[None, :]
        assert (numpy.abs(got - exact) <= 2.0 ** -27 * scale + 1e-300).all()
        eng.destroy_plan(pid)
    assert eng.device_status() == 0


def _dot_contraction(P, which):
    """T1 = L_p . psi (which = 1) or T3 = T1 . O (which = 2) for one term of the
    dot as a stand-alone contraction plan; returns the plan, its operands on
    the host and on the device."""
    import torch
    from zmpo_dmrg_gb300 import engine as E
    eng = E.get()
    m = P.p
    fL = m.flst[0][0]
    iop = next(i for i in range(m.nops) if fL.present(i) and fL.tensors[i].size_allowed > 2000)
    Lt = fL.tensors[iop]
    L = fL.buf[fL.off[iop]:fL.off[iop] + Lt.size_allowed].clone()
    x = torch.from_numpy(numpy.random.default_rng(2).standard_normal(P.ndim0)).cuda()
    lo1, pid1 = eng.contract_plan(Lt.layout, m.qtmp.layout, ([2], [0]))
    size1 = eng.layout_blocks(lo1)[0]
    if which == 1:
        return eng, pid1, [L, x]
    T1 = torch.empty(size1, dtype=torch.float64, device="cuda")
    eng.contract_exec(pid1, L, x, T1, "fp64")
    W = m.mpo_store
    wi = W.tensors[P.isite][iop]
    wj = W.tensors[P.isite + 1][iop]
    lO, pO = eng.contract_plan(wi.layout, wj.layout, ([1], [0]))
    O = torch.empty(eng.layout_blocks(lO)[0], dtype=torch.float64, device="cuda")
    Wi = W.buf[W.off[P.isite][iop]:W.off[P.isite][iop] + wi.size_allowed].clone()
    Wj = W.buf[W.off[P.isite + 1][iop]:W.off[P.isite + 1][iop] + wj.size_allowed].clone()
    eng.contract_exec(pO, Wi, Wj, O, "fp64")
    lo2, pid2 = eng.contract_plan(lo1, lO, ([0, 2, 3], [0, 2, 5]))
    return eng, pid2, [T1, O]


@pytest.mark.parametrize("which", [1, 2])
def test_dot_contractions_bit_exact_on_routed_groups(gpu, which):
    import torch
    P = random_problem(K=10, nelec=10, D=128, isite=4, seed=7)
    eng, pid, (a, b) = _dot_contraction(P, which)
    groups, _, cbl, _, reds = eng.step_tasks(pid, 0)
    written = []
    # buffers of a contraction plan: 0 = A, 1 = B, 4 = output (6: split-K
    # parts); the output size from the furthest element the groups and the
    # split-K sums write
    host_bufs = [a.cpu().numpy(), b.cpu().numpy(), None, None, None, None, numpy.zeros(1), numpy.zeros(1)]
    outn = 0
    for r in reds:
        outn = max(outn, int(r["c_off"] + (r["M"] - 1) * r["scm"] + (r["N"] - 1) * r["scn"]) + 1)
    for g in groups:
        if g["cbuf"] == 6:
            continue
        if g["ncb"] == 0:
            outn = max(outn, int(g["c_off"] + (g["M"] - 1) * g["scm"] + (g["N"] - 1) * g["scn"]) + 1)
        for j in range(int(g["ncb"])):
            cb = cbl[g["cb0"] + j]
            outn = max(outn, int(cb["c_off"] + (g["M"] - 1) * cb["scm"] + (cb["n"] - 1) * cb["scn"]) + 1)
    host_bufs[4] = numpy.full(outn, numpy.nan)
    run_tasks_on_host(eng, pid, 1, host_bufs, model, written, part_gemm=long_gemm)
    assert len(written) > 10
    out = torch.full((outn,), numpy.nan, dtype=torch.float64, device="cuda")
    eng.contract_exec(pid, a, b, out, "split")
    got = out.cpu().numpy()
    for buf, idx, vals in written:
        assert buf == 4
        assert numpy.array_equal(got[idx], vals)
    ref = host_bufs[4]
    mask = ~numpy.isnan(ref)                 # every element some group writes
    assert not numpy.isnan(got[mask]).any()
    assert numpy.linalg.norm(got[mask] - ref[mask]) <= 1e-8 * numpy.linalg.norm(ref[mask])
    assert eng.device_status() == 0
