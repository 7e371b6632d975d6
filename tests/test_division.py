"""The GPU path replaces some FP64 divisions by multiplications with a
reciprocal plus fma corrections (Markstein, IBM J. Res. Dev. 34(1), 1990):
`div3` for the centroid's /3 in the clip and `div_rcp` for divisions by a
value whose reciprocal is formed once (rho c2 dt^2, the mass, the cell size).
The meshes, operators and right-hand sides they feed are compared bit for bit
with the oracle by the GPU tests; this test checks the two sequences
themselves on the CPU against IEEE division, with fma evaluated exactly
(rational arithmetic, then one correct rounding)."""
import math
import random
import struct
from fractions import Fraction

import pytest


def fma(a, b, c):
    """Correctly rounded a*b + c (Python's float(Fraction) rounds to nearest even)."""
    return float(Fraction(a) * Fraction(b) + Fraction(c))


def exponent(a):
    return (struct.unpack("<Q", struct.pack("<d", a))[0] >> 52) & 0x7FF


def div3(a):
    # the guard and sequence of div3 (lv_mesh.cu)
    if (exponent(a) - 123) & 0xFFFFFFFF < 1900:
        y = float.fromhex("0x1.5555555555555p-2")
        q = a * y
        r = fma(-3.0, q, a)
        return fma(r, y, q)
    return a / 3.0


def div_rcp(a, b, y):
    # the guard and sequence of div_rcp (lv_internal.cuh)
    if (exponent(a) - 123) & 0xFFFFFFFF < 1800 and (exponent(b) - 923) & 0xFFFFFFFF < 200:
        q = a * y
        r = fma(-b, q, a)
        q = fma(r, y, q)
        r = fma(-b, q, a)
        return fma(r, y, q)
    return a / b


def random_double(rng, emin, emax, hard=0):
    e = rng.randrange(emin, emax)
    if hard == 1:
        m = (1 << 52) - 1 - rng.randrange(16)  # significand near 2
    elif hard == 2:
        m = rng.randrange(256)  # near a power of two
    else:
        m = rng.getrandbits(52)
    bits = (rng.getrandbits(1) << 63) | (e << 52) | m
    return struct.unpack("<d", struct.pack("<Q", bits))[0]


def same(x, y):
    return struct.pack("<d", x) == struct.pack("<d", y) or (math.isnan(x) and math.isnan(y))


def test_div3_is_correctly_rounded():
    assert float.fromhex("0x1.5555555555555p-2") == 1.0 / 3.0
    rng = random.Random(20240601)
    for k in range(20000):
        a = random_double(rng, 100, 2000, hard=k % 3)
        assert same(div3(a), a / 3.0), a.hex()
    for m in range(1, 3000):
        for a in (float(m), float(3 * m + 1) * 2.0**20, -float(m) * 2.0**-500):
            assert same(div3(a), a / 3.0), a.hex()
    for a in (0.0, -0.0, math.inf, -math.inf, math.nan, 2.0**-1000, 5e-324, 1.7976931348623157e308):
        assert same(div3(a), a / 3.0)


def test_div_rcp_is_correctly_rounded():
    rng = random.Random(777)
    for k in range(20000):
        a = random_double(rng, 100, 1950, hard=k % 3)
        b = random_double(rng, 900, 1150, hard=(k // 3) % 3)
        assert same(div_rcp(a, b, 1.0 / b), a / b), (a.hex(), b.hex())
    # equal significands, integers, the divisors this build uses
    for k in range(2000):
        b = random_double(rng, 1000, 1050)
        a = b * float(1 + k % 7)
        assert same(div_rcp(a, b, 1.0 / b), a / b)
    for a in (0.0, -0.0, math.inf, -math.inf, math.nan, 1.0, -3.5):
        for b in (0.0, -0.0, math.inf, -math.inf, math.nan, 1.0, -3.5):
            q = a / b if b != 0.0 else None
            if q is None:
                continue  # Python raises on division by zero; the device path takes the IEEE division there
            assert same(div_rcp(a, b, 1.0 / b if b not in (0.0,) else math.inf), q)
