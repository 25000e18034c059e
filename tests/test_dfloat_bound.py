"""The double-float arithmetic of the recheck (csrc/dfloat.cuh), restated
with exact rational arithmetic and correctly rounded float32 operations, and
checked against the error bound the host uses (abi.cu: 2^-43 per operation
over the float32 bound's operation count).

Every float32 operation of the kernel (__fadd_rn, __fsub_rn, __fmul_rn,
__fmaf_rn) is one round-to-nearest-even of the exact result, so the
restatement is exact; operands are non-negative, as every tensor entry of
the decoder is.
"""
from fractions import Fraction as Fr

import numpy as np


def round_f32(x: Fr) -> Fr:
    """Nearest float32 (ties to even) of an exact rational in the normal range."""
    if x == 0:
        return Fr(0)
    sign = -1 if x < 0 else 1
    a = abs(x)
    e = a.numerator.bit_length() - a.denominator.bit_length()
    if Fr(2) ** e > a:
        e -= 1
    elif Fr(2) ** (e + 1) <= a:
        e += 1
    assert -126 <= e <= 127, "outside the normal float32 range"
    scaled = a * Fr(2) ** (23 - e)
    q = scaled.numerator // scaled.denominator
    rem = scaled - q
    if rem > Fr(1, 2) or (rem == Fr(1, 2) and q % 2 == 1):
        q += 1
    return sign * Fr(q) * Fr(2) ** (e - 23)


def fadd(a, b):
    return round_f32(a + b)


def fsub(a, b):
    return round_f32(a - b)


def fmul(a, b):
    return round_f32(a * b)


def fma(a, b, c):
    return round_f32(a * b + c)


def fast_two_sum(a, b):
    s = fadd(a, b)
    return s, fsub(b, fsub(s, a))


def two_sum(a, b):
    s = fadd(a, b)
    bb = fsub(s, a)
    return s, fadd(fsub(a, fsub(s, bb)), fsub(b, bb))


def df_fma(a, b, c):
    """c + a*b, dfloat.cuh:fma."""
    p = fmul(a[0], b[0])
    e = fma(a[0], b[0], -p)
    t = fma(a[0], b[1], fma(a[1], b[0], e))
    s_hi, s_lo = two_sum(c[0], p)
    return fast_two_sum(s_hi, fadd(s_lo, fadd(c[1], t)))


def to_df(x: float):
    hi = round_f32(Fr(x))
    return hi, round_f32(Fr(x) - hi)


def value(d):
    return d[0] + d[1]


def test_round_f32_matches_numpy():
    rng = np.random.default_rng(1)
    for x in rng.random(200) * 10.0 ** rng.integers(-20, 20, 200):
        assert float(round_f32(Fr(float(x)))) == float(np.float32(x))


def test_double_float_fma_error_below_2_pow_minus_44():
    """One multiply-add: |result - (c + a*b)| <= 15 * 2^-48 * (c + a*b)."""
    rng = np.random.default_rng(7)
    worst = 0.0
    for _ in range(1500):
        a, b, c = (to_df(float(x) * 10.0 ** int(k)) for x, k in zip(rng.random(3), rng.integers(-6, 6, 3)))
        got = value(df_fma(a, b, c))
        exact = value(c) + value(a) * value(b)
        worst = max(worst, float(abs(got - exact) / exact))
    assert worst <= 15 * 2.0 ** -48 < 2.0 ** -44


def test_double_float_dot_products_within_the_host_bound():
    """Sums of K products accumulated by repeated fma stay within
    (K + 1) * 2^-43 relative: the host's per-step operation count times its
    per-operation bound."""
    rng = np.random.default_rng(11)
    for K in (1, 2, 8, 16, 64):
        for _ in range(12):
            a = [to_df(float(x)) for x in rng.random(K)]
            b = [to_df(float(x) * 10.0 ** int(k)) for x, k in zip(rng.random(K), rng.integers(-4, 4, K))]
            acc = (Fr(0), Fr(0))
            for ak, bk in zip(a, b):
                acc = df_fma(ak, bk, acc)
            exact = sum(value(ak) * value(bk) for ak, bk in zip(a, b))
            if exact == 0:
                continue
            assert abs(value(acc) - exact) / exact <= (K + 1) * Fr(2) ** -43


def test_power_of_two_scaling_is_exact():
    """The normalisers scale both halves by a power of two (dfloat.cuh:scale)."""
    rng = np.random.default_rng(3)
    for x in rng.random(50):
        hi, lo = to_df(float(x) * 1e-5)
        for e in (-40, -7, 0, 9, 60):
            s = Fr(2) ** e
            assert fmul(hi, s) + fmul(lo, s) == (hi + lo) * s
