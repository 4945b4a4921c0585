"""Exact NumPy model of the split path's arithmetic (test infrastructure).

Split precision multiplies FP64 matrices on the BF16 tensor cores with exact
digit products:

* every element x of a row i of A (column j of B) is written relative to the
  row's (column's) largest biased exponent E over the whole K of the product:
  X = |x| / 2^(E - 1053) rounded to the nearest integer (halves up) <= 2^31,
  and X = d0 2^24 + d1 2^16 + d2 2^8 + d3
  with d1..d3 in [-128, 127], d0 in [0, 128] (the bytes of X + 0x808080); the
  element's sign goes on every digit (``balanced_digits``);
* the levels L_l = sum_{s+t=l} Da_s Db_t^T, l = 0..3, are integers below 2^24
  for K <= 256 (a digit product is at most 2^14, at most four per level and
  slot), so FP32 accumulation on the tensor cores is exact;
* the result is S = L0 2^24 + L1 2^16 + L2 2^8 + L3 (an integer below 2^48,
  exact in FP64) times 2^(Ea_i + Eb_j - 2082).

``one_pass_gemm`` computes that result exactly (int64 products); the
tensor-core kernel that runs a group in one pass must reproduce it bit for
bit.  Results below the normal FP64 range are flushed to zero in both.

``long_gemm``: a group with a longer K runs in passes of 256 slots (each
exact as above, with its own exponents) whose results are added in FP64 in
pass order, starting from zero; a group longer than 2048 slots is first cut
into parts of 2048 (the last one shorter) whose results are added in FP64 in
part order, starting from zero (the split-K sum).
"""
import numpy

BIAS = 2082


def dexp(x):
    """Biased exponent of each float64 (0 for zero and subnormals)."""
    return ((numpy.ascontiguousarray(x, dtype=numpy.float64).view(numpy.uint64) >> 52) & 0x7ff).astype(numpy.int64)


def aligned31(x, E):
    """|x| / 2^(E - 1053) rounded to the nearest integer, halves up, from the
    53-bit significand m: (m + 2^(s-1)) >> s with s = E - e + 22 capped at 63,
    as the kernel computes it (E >= the element's exponent e; 0 for zero and
    subnormals)."""
    b = numpy.ascontiguousarray(x, dtype=numpy.float64).view(numpy.uint64)
    e = ((b >> numpy.uint64(52)) & numpy.uint64(0x7ff)).astype(numpy.int64)
    mant = (b & numpy.uint64((1 << 52) - 1)) | numpy.uint64(1 << 52)
    sh = numpy.minimum(numpy.asarray(E, dtype=numpy.int64) - e + 22, 63)
    sh, mant = numpy.broadcast_arrays(sh, mant)
    X = (mant + (numpy.uint64(1) << (sh - 1).astype(numpy.uint64))) >> sh.astype(numpy.uint64)
    return numpy.where(e > 0, X.astype(numpy.int64), 0)


def balanced_digits(x, E):
    """Four signed digits (int64 arrays, most significant first)."""
    X = aligned31(x, E)
    Y = X + 0x808080
    d = [(Y >> 24) & 0xff, ((Y >> 16) & 0xff) - 128, ((Y >> 8) & 0xff) - 128, (Y & 0xff) - 128]
    s = numpy.where(numpy.signbit(numpy.asarray(x, dtype=numpy.float64)), -1, 1)
    return [s * v for v in d]


def one_pass_gemm(A, B):
    """Exact result of the one-pass split product of A (M x K) and B (K x N),
    K <= 256, as float64."""
    A = numpy.asarray(A, dtype=numpy.float64)
    B = numpy.asarray(B, dtype=numpy.float64)
    M, K = A.shape
    N = B.shape[1]
    assert K <= 256
    if K == 0:
        return numpy.zeros((M, N))
    Ea = dexp(A).max(axis=1)
    Eb = dexp(B).max(axis=0)
    da = balanced_digits(A, Ea[:, None])
    db = balanced_digits(B, Eb[None, :])
    L = [numpy.zeros((M, N), dtype=numpy.int64) for _ in range(4)]
    for s in range(4):
        for t in range(4 - s):
            L[s + t] += da[s] @ db[t]
    for lv in L:
        assert numpy.abs(lv).max(initial=0) < 2 ** 24
    S = (L[0] << 24) + (L[1] << 16) + (L[2] << 8) + L[3]
    e = Ea[:, None] + Eb[None, :] - BIAS
    out = numpy.ldexp(S.astype(numpy.float64), e)   # exact: |S| < 2^53
    # below the normal range the kernel flushes to zero
    tiny = (S != 0) & (numpy.abs(out) < numpy.ldexp(1.0, -1022))
    out[tiny] = 0.0
    out[(Ea[:, None] == 0) | (Eb[None, :] == 0)] = 0.0
    return out


PASS, PART = 256, 2048


def passes_gemm(A, B):
    """FP64 sum, in pass order from zero, of the one-pass products of the
    256-slot passes of A (M x K) and B (K x N)."""
    A = numpy.asarray(A, dtype=numpy.float64)
    B = numpy.asarray(B, dtype=numpy.float64)
    acc = numpy.zeros((A.shape[0], B.shape[1]))
    for k0 in range(0, A.shape[1], PASS):
        acc = acc + one_pass_gemm(A[:, k0:k0 + PASS], B[k0:k0 + PASS])
    return acc


def long_gemm(A, B):
    """The long tcgen05 route: parts of 2048 slots, each a pass sum; the parts
    added in order from zero when there is more than one."""
    A = numpy.asarray(A, dtype=numpy.float64)
    B = numpy.asarray(B, dtype=numpy.float64)
    K = A.shape[1]
    if K <= PART:
        return passes_gemm(A, B)
    acc = numpy.zeros((A.shape[0], B.shape[1]))
    for k0 in range(0, K, PART):
        acc = acc + passes_gemm(A[:, k0:k0 + PART], B[k0:k0 + PART])
    return acc
