"""Exact integer models of the two digit schemes the FP64 paths use, checked
on the CPU.  They pin the arithmetic claims the kernels rest on:

* Ozaki DGEMM (gemm_ozaki.cu): s balanced base-256 digits of
  N = +-trunc(|x| 2^(8s-1-e)) reconstruct N exactly, every digit is in
  [-128, 127] (the leading one in [-128, 128]), so a digit product is at most
  2^14 and a 1024-long chunk of them sums to at most 2^24 (exact in FP32);
  127 chunk sums fit an int32.
* FP64 skinny (skinny_oz.cu): F = trunc(|x| 2^(48-e)) from the fast mantissa
  shift (rs = 1027 + e - E, shifts of 64 or more give 0, the implicit bit of
  zeros / subnormals shifted out) equals the exact value whenever e >= -974;
  the 18 / 18 / 12-bit pieces and their base-64 digits reconstruct F; a level
  sum over a 256-long chunk is below 2^24 and the combination
  T = sum_L S_L 2^(6(9-L)) of one chunk is below 2^63 in magnitude."""
import math
import random
import struct
from fractions import Fraction

import pytest


def _bits(x):
    return struct.unpack("<Q", struct.pack("<d", x))[0]


def _exp_of_max(xs):
    """The line exponent: smallest e with max |x| < 2^e (0 for all zeros)."""
    mb = max(_bits(abs(x)) for x in xs)
    if mb == 0:
        return 0
    E = (mb >> 52) & 0x7FF
    if E == 0:
        return mb.bit_length() - 1074
    return E - 1022


def _trunc_scaled(x, shift):
    """trunc(|x| * 2^shift) exactly."""
    f = abs(Fraction(x)) * Fraction(2) ** shift
    return f.numerator // f.denominator


def _balanced_digits(N, s):
    out = []
    for _ in range(s - 1):
        d = ((N + 128) & 255) - 128
        out.append(d)
        N = (N - d) >> 8
    out.append(N)          # the leading digit takes what is left
    return out[::-1]       # most significant first


def _random_line(rng, n, spread):
    return [rng.uniform(-1, 1) * 2.0 ** rng.randint(-spread, spread) for _ in range(n)]


@pytest.mark.parametrize("s", [2, 4, 7, 9])
def test_ozaki_balanced_digits(s):
    rng = random.Random(s)
    for _ in range(300):
        line = _random_line(rng, 16, 30)
        e = _exp_of_max(line)
        for x in line:
            F = _trunc_scaled(x, 8 * s - 1 - e)
            assert F < 2 ** (8 * s - 1)
            N = -F if x < 0 else F
            d = _balanced_digits(N, s)
            assert sum(dt * 256 ** (s - 1 - i) for i, dt in enumerate(d)) == N
            assert all(-128 <= dt <= 127 for dt in d[1:]) and -128 <= d[0] <= 128
            # x ~= 2^(e+1) sum_t d_t 2^-8t, truncation below 2^(e+1-8s)
            approx = Fraction(2) ** (e + 1) * sum(Fraction(dt, 256 ** (i + 1)) for i, dt in enumerate(d))
            assert abs(Fraction(x) - approx) < Fraction(2) ** (e + 1 - 8 * s)


def test_ozaki_chunk_bounds():
    assert 1024 * 128 * 128 == 2 ** 24          # largest |chunk sum| of digit products: exact in FP32
    assert 127 * 2 ** 24 < 2 ** 31             # 127 chunk sums in an int32 (per diagonal)


def _skinny_F_fast(x, e):
    b = _bits(x)
    hi, lo = b >> 32, b & 0xFFFFFFFF
    rs = (1027 + e - ((hi >> 20) & 0x7FF)) & 0xFFFFFFFF
    m = (((hi & 0xFFFFF) | 0x100000) << 32) | lo
    return 0 if rs >= 64 else m >> rs


@pytest.mark.parametrize("spread", [0, 20, 60])
def test_skinny_fast_mantissa_and_digits(spread):
    rng = random.Random(100 + spread)
    for _ in range(300):
        line = _random_line(rng, 32, spread) + [0.0, -0.0, 5e-324, -2.5e-310]
        e = _exp_of_max(line)
        assert e >= -974
        for x in line:
            F = _trunc_scaled(x, 48 - e)
            assert F < 2 ** 48
            assert _skinny_F_fast(x, e) == F
            fh, fl = F >> 32, F & 0xFFFFFFFF
            p0 = ((fh << 2) | (fl >> 30)) & 0xFFFFFFFF       # bits 30..47 (fh < 2^16)
            p1 = (fl >> 12) & 0x3FFFF
            p2 = fl & 0xFFF
            digits = [p0 >> 12, (p0 >> 6) & 63, p0 & 63, p1 >> 12, (p1 >> 6) & 63, p1 & 63, p2 >> 6, p2 & 63]
            assert all(0 <= d < 64 for d in digits)
            assert sum(d << (48 - 6 * (t + 1)) for t, d in enumerate(digits)) == F


def test_skinny_level_and_combination_bounds():
    chunk = 256
    levels = {L: (L - 1) * chunk * 63 * 63 for L in range(2, 10)}   # pairs t + u = L, t, u in 1..8
    assert max(levels.values()) < 2 ** 24
    T = sum(v * 2 ** (6 * (9 - L)) for L, v in levels.items())
    assert T < 2 ** 63
    assert math.log2(T) < 62.2
