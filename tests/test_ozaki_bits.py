"""CPU checks (numpy, exact integer arithmetic) of the bit-level identities the
Ozaki slicing kernels rely on (zq_ozaki.cu: k_oz_exp, k_oz_slice, oz_fixed,
oz_digit_pair; zq_common.cuh: absmax_bits).

* A slice digit d in [0, 127] with sign s is stored as bf16 without a
  conversion instruction: the bit pattern 0x4300 | d is the bf16 value 128 + d,
  and one bf16 FMA s (128 + d) + (-128 s) gives s d exactly (+0 for d = 0), the
  same bits as converting the integer s d.
* For non-negative doubles the unsigned order of the bit patterns is the order
  of the values, so running maxima of |x| may be taken on integers.
* The frexp exponent is monotone in the value, so the exponent of a row's
  maximum is the largest exponent of its parts (several warps per row combined
  by atomicMax).
* The digits of V = floor(|v| 2^(7S - e)), 2^e > max |v|, rebuild V exactly,
  and |v| - V 2^(e - 7S) < 2^(e - 7S).
"""
import math
import struct
from fractions import Fraction

import numpy as np


def _bf16_bits_to_float(b: int) -> float:
    return struct.unpack("<f", struct.pack("<I", (b & 0xFFFF) << 16))[0]


def _float_to_bf16_bits_exact(x: float) -> int:
    """bf16 bits of x, which must be exactly representable in bf16."""
    u = struct.unpack("<I", struct.pack("<f", x))[0]
    assert u & 0xFFFF == 0, x
    assert _bf16_bits_to_float(u >> 16) == x
    return u >> 16


def test_bf16_digit_from_bit_pattern_and_one_fma():
    for d in range(128):
        assert _bf16_bits_to_float(0x4300 | d) == 128.0 + d
        for s in (1.0, -1.0):
            # the FMA's exact result; it is representable in bf16 (|s d| <= 127
            # has at most 7 significant bits), so the bf16 rounding keeps it
            exact = s * (128.0 + d) + (-128.0 * s)
            assert exact == s * d
            got = _float_to_bf16_bits_exact(exact)  # d = 0: x + (-x) = +0 in round-to-nearest
            want = _float_to_bf16_bits_exact(float(int(s) * d))  # conversion of the integer s d
            assert got == want, (d, s, hex(got), hex(want))
    # the packed sign factors: +1 0x3F80, -1 0xBF80, -128 0xC300, +128 0x4300
    assert _bf16_bits_to_float(0x3F80) == 1.0 and _bf16_bits_to_float(0xBF80) == -1.0
    assert _bf16_bits_to_float(0xC300) == -128.0 and _bf16_bits_to_float(0x4300) == 128.0


def _special_doubles(rng, n):
    x = np.concatenate([
        rng.standard_normal(n) * 10.0 ** rng.integers(-300, 300, n),
        np.array([0.0, -0.0, 5e-324, -5e-324, 2.2250738585072014e-308, 1.7976931348623157e308, np.inf, -np.inf]),
        rng.standard_normal(n) * 1e-310,  # subnormals
    ])
    return x


def test_bit_pattern_order_is_value_order_for_magnitudes():
    rng = np.random.default_rng(11)
    x = np.abs(_special_doubles(rng, 4000))
    bits = x.view(np.uint64) & np.uint64(0x7FFFFFFFFFFFFFFF)
    order_v = np.argsort(x, kind="stable")
    sorted_bits = bits[order_v]
    assert np.all(sorted_bits[1:] >= sorted_bits[:-1])
    # pairwise: a < b  <=>  bits(a) < bits(b)
    a, b = x[:2000], x[2000:4000]
    ba, bb = bits[:2000], bits[2000:4000]
    assert np.array_equal(a < b, ba < bb)
    assert np.array_equal(a == b, ba == bb)
    # the maximum by bits is the maximum by value
    assert bits.max().view(np.float64) == x.max()


def test_sign_flip_on_bits_equals_negation():
    rng = np.random.default_rng(12)
    x = _special_doubles(rng, 1000)
    flipped = (x.view(np.uint64) ^ np.uint64(1 << 63)).view(np.float64)
    assert np.array_equal(flipped.view(np.uint64), (-x).view(np.uint64))
    assert np.array_equal(flipped.view(np.uint64), (x * -1.0).view(np.uint64))


def test_largest_part_exponent_is_exponent_of_maximum():
    rng = np.random.default_rng(13)
    for _ in range(200):
        v = np.abs(rng.standard_normal(rng.integers(1, 50)) * 10.0 ** rng.integers(-30, 30))
        s2 = rng.choice([1.0, -1.0, 0.75, 3.0])
        parts = np.array_split(v, rng.integers(1, 9))
        part_exps = [math.frexp(float(p.max()))[1] for p in parts if p.size and p.max() > 0]
        # the second segment's entries scaled by |s2|: exponent of max(m1, |s2| m2)
        m1, m2 = float(v[: len(v) // 2 + 1].max()), float(v[len(v) // 2 + 1:].max(initial=0.0))
        combined = max(math.frexp(m1)[1], math.frexp(abs(s2) * m2)[1] if m2 > 0 else -1100)
        assert combined == math.frexp(max(m1, abs(s2) * m2))[1]
        assert max(part_exps) == math.frexp(float(v.max()))[1]


def _fixed(v: float, e: int, F: int) -> int:
    """floor(|v| 2^(F - e)) with exact rational arithmetic."""
    m, ex = math.frexp(abs(v))  # |v| = m 2^ex
    mant = int(m * (1 << 53))  # exact: m has 53 significant bits
    sh = ex - 53 - e + F
    return mant << sh if sh >= 0 else mant >> (-sh)


def test_digits_rebuild_the_fixed_point_value_and_bound_the_truncation():
    rng = np.random.default_rng(14)
    for S in (3, 4, 5, 7, 8):
        F = 7 * S
        for _ in range(300):
            row = rng.standard_normal(16) * 10.0 ** rng.integers(-20, 20)
            e = math.frexp(float(np.abs(row).max()))[1]  # 2^e > max |v|
            for v in row:
                V = _fixed(float(v), e, F)
                assert 0 <= V < (1 << F)
                digits = [(V >> (F - 7 * (q + 1))) & 127 for q in range(S)]
                assert sum(d << (7 * (S - 1 - q)) for q, d in enumerate(digits)) == V
                # truncation: |v| - V 2^(e - F) in [0, 2^(e - F)), checked exactly
                rem = Fraction(abs(float(v))) - Fraction(V) * Fraction(2) ** (e - F)
                assert 0 <= rem < Fraction(2) ** (e - F)
