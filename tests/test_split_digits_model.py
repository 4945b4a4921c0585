"""Model of the split path's digit arithmetic (csrc/kernels.cu: aligned32,
balanced31, digits4_pair, mma_fold), checked on the CPU.

S = 4: the 31 most significant significand bits X of |x|, aligned to the
chunk exponent E, are written X = d0 2^24 + d1 2^16 + d2 2^8 + d3 with
d1..d3 in [-128, 127] and d0 in [0, 128] (the bytes of X + 0x808080).  A level
(at most four digit products per slot) then stays below 2^24 for 256 slots,
so the BF16 tensor-core sums are exact; the chunk's levels are folded into a
two-float accumulator with the scale 2^(Ea + Eb - 2058 - 8 l).
"""
import struct

import numpy


def _bits(x):
    return struct.unpack('<Q', struct.pack('<d', x))[0]


def dexp(x):
    return (_bits(x) >> 52) & 0x7ff


def aligned32(x, E):
    b = _bits(x)
    hi, lo = b >> 32, b & 0xffffffff
    e = (hi >> 20) & 0x7ff
    top = ((((hi & 0xfffff) | 0x100000) << 11) | (lo >> 21)) & 0xffffffff if e else 0
    sh = E - e
    return top >> sh if sh < 32 else 0


def digits(x, E):
    Y = (aligned32(x, E) >> 1) + 0x808080
    d = [(Y >> 24) & 0xff, ((Y >> 16) & 0xff) - 128, ((Y >> 8) & 0xff) - 128, (Y & 0xff) - 128]
    s = -1 if x < 0 else 1
    return [s * v for v in d]


def f32(x):
    return numpy.float32(x)


def two_sum(a, b):
    s = f32(a + b)
    z = f32(s - a)
    return s, f32(f32(a - f32(s - z)) + f32(b - z))


def split_dot(a, b, TK=64):
    hi, lo = f32(0), f32(0)
    for c0 in range(0, len(a), TK):
        ac, bc = a[c0:c0 + TK], b[c0:c0 + TK]
        Ea, Eb = max(dexp(x) for x in ac), max(dexp(x) for x in bc)
        if Ea == 0 or Eb == 0:
            continue
        da, db = [digits(x, Ea) for x in ac], [digits(x, Eb) for x in bc]
        acc = [0, 0, 0, 0]
        for k in range(len(ac)):
            for sa in range(4):
                for sb in range(4 - sa):
                    acc[sa + sb] += da[k][sa] * db[k][sb]
        assert all(abs(v) < 2 ** 24 for v in acc)
        acc = [f32(v) for v in acc]
        h, e = two_sum(acc[0], f32(acc[1] * f32(2 ** -8)))
        e = f32(acc[2] * f32(2 ** -16) + e)
        e = f32(acc[3] * f32(2 ** -24) + e)
        sc = f32(2.0 ** (Ea + Eb - 2044 - 14))
        s2, e2 = two_sum(hi, f32(h * sc))
        hi, lo = s2, f32(lo + f32(e2 + f32(e * sc)))
    return float(hi) + float(lo)


def test_balanced_digits_reconstruct_the_aligned_bits():
    rng = numpy.random.default_rng(1)
    xs = list(rng.standard_normal(200) * 10.0 ** rng.uniform(-5, 5, 200))
    xs += [0.0, 1.0, -1.0, 2.0, numpy.nextafter(2.0, 0.0), -numpy.nextafter(1.0, 0.0), 1e-300, 5e-324]
    for x in xs:
        for dE in (0, 1, 7, 31):
            E = max(dexp(x), 1) + dE
            d = digits(x, E)
            assert all(-128 <= v <= 128 for v in d)
            X31 = aligned32(x, E) >> 1
            s = -1 if x < 0 else 1   # the element's sign is on every digit
            assert d[0] * 2 ** 24 + d[1] * 2 ** 16 + d[2] * 2 ** 8 + d[3] == s * X31


def test_levels_stay_exact_for_256_slots():
    x = numpy.nextafter(2.0, 0.0)   # every digit at its extreme
    E = dexp(x)
    worst = 0
    for a in (x, -x):
        da = digits(a, E)
        db = digits(x, E)
        for lvl in range(4):
            per_slot = sum(abs(da[s] * db[lvl - s]) for s in range(lvl + 1))
            worst = max(worst, per_slot)
    assert worst <= 2 ** 16
    assert 256 * worst <= 2 ** 24


def test_split_dot_error_bound():
    rng = numpy.random.default_rng(7)
    worst = 0.0
    for trial in range(40):
        n = int(rng.integers(1, 300))
        a = rng.standard_normal(n) * numpy.exp(rng.uniform(-8, 8, n) * (trial % 2))
        b = rng.standard_normal(n) * 10.0 ** rng.uniform(-3, 3)
        ref = float(numpy.dot(a.astype(numpy.longdouble), b.astype(numpy.longdouble)))
        got = split_dot(list(a), list(b))
        worst = max(worst, abs(got - ref) / float(numpy.dot(numpy.abs(a), numpy.abs(b))))
    assert worst < 1e-8


# ------------------------------------------------ one-pass (whole-K) scheme
def test_one_pass_model_matches_slot_model():
    """The vectorised one-pass model (tests/split_model.py) equals the scalar
    digit model above with a single chunk covering all of K."""
    from tests.split_model import one_pass_gemm
    rng = numpy.random.default_rng(3)
    for n in (1, 5, 64, 200, 256):
        a = rng.standard_normal(n) * numpy.exp(rng.uniform(-6, 6, n))
        b = rng.standard_normal(n)
        got = one_pass_gemm(a[None, :], b[:, None])[0, 0]
        ref = split_dot(list(a), list(b), TK=256)
        assert abs(got - ref) <= 2e-7 * abs(ref) + 1e-300   # the scalar model folds in two floats


def test_one_pass_model_error_bound():
    """Error of the one-pass product: below 2^-29 K max_k|a_ik| max_k|b_kj|
    per element (every digit cut is relative to its row's or column's largest
    element), also for rows and columns with a wide dynamic range."""
    from tests.split_model import one_pass_gemm
    rng = numpy.random.default_rng(11)
    for trial in range(6):
        M, K, N = 37, int(rng.integers(1, 257)), 23
        A = rng.standard_normal((M, K)) * numpy.exp(rng.uniform(-10, 10, (M, K)) * (trial % 2))
        B = rng.standard_normal((K, N)) * numpy.exp(rng.uniform(-4, 4, (K, N)))
        got = one_pass_gemm(A, B)
        ref = (A.astype(numpy.longdouble) @ B.astype(numpy.longdouble)).astype(numpy.float64)
        scale = K * numpy.abs(A).max(axis=1)[:, None] * numpy.abs(B).max(axis=0)[None, :]
        assert (numpy.abs(got - ref) <= 2.0 ** -29 * scale + 1e-300).all()
