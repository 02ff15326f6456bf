"""Division by a small integer in three FP64 operations (photon_gb300/csrc/
fdiv.cuh: Markstein's correction with RN(1/d)) gives the IEEE quotient x / d.

The CPU test emulates the method exactly: each FMA is computed in rationals and
rounded once to double, and the result must equal Python's correctly rounded
x / d bit for bit. The GPU test (test_gpu_div_small.py) compares the device
function itself with the device's own division."""
import math
import random
import struct
from fractions import Fraction

import numpy as np

RECIP = {1: 1.0, 2: 0.5, 3: float.fromhex("0x1.5555555555555p-2"), 4: 0.25,
         5: float.fromhex("0x1.999999999999ap-3"), 6: float.fromhex("0x1.5555555555555p-3"),
         7: float.fromhex("0x1.2492492492492p-3")}


def rn(fr):
    """a rational rounded to the nearest double (ties to even)"""
    return float(fr)


def div_small(x, d):
    hi = struct.unpack("<Q", struct.pack("<d", x))[0] >> 32
    ex = (hi >> 20) & 0x7FF
    if ex < 63 or ex == 0x7FF:
        return x / d
    y = RECIP[d]
    q = x * y                                           # RN(x y)
    e = rn(Fraction(x) - d * Fraction(q))               # fma(-q, d, x)
    assert Fraction(e) == Fraction(x) - d * Fraction(q)   # the remainder is exact
    return rn(Fraction(e) * Fraction(y) + Fraction(q))  # fma(e, y, q)


def bits(v):
    return struct.unpack("<Q", struct.pack("<d", v))[0]


def inputs(n_random, seed):
    rng = random.Random(seed)
    xs = []
    for _ in range(n_random):   # random significands over the normal exponents the method handles
        m = rng.getrandbits(52)
        e = rng.randrange(63, 2047)
        s = rng.getrandbits(1)
        xs.append(struct.unpack("<d", struct.pack("<Q", (s << 63) | (e << 52) | m))[0])
    for k in range(2000):       # significands at both ends of a binade
        for e in (0, -17, 40):
            xs.append(math.ldexp(1.0 + k * 2.0 ** -52, e))
            xs.append(math.ldexp(2.0 - (k + 1) * 2.0 ** -52, e))
    for d in range(3, 8):       # quotients next to a midpoint between two doubles
        for _ in range(1500):
            q = 1.0 + rng.getrandbits(52) * 2.0 ** -52
            mid = Fraction(q) + Fraction(1, 2 ** 53)
            for off in (-2, -1, 0, 1, 2):
                xs.append(rn(d * mid + off * Fraction(1, 2 ** 60)))
    xs += [0.0, -0.0, 5e-324, -5e-324, 2.0 ** -1000, 2.0 ** -960, math.inf, -math.inf, 1.7976931348623157e308]
    xs += [float(3 * j) for j in range(1, 3000)] + [float(7 * j) / 4 for j in range(1, 3000)]
    return xs


def test_method_matches_ieee_quotient():
    for x in inputs(4000, 1):
        for d in range(1, 8):
            a, b = div_small(x, d), x / d
            assert bits(a) == bits(b), (x.hex(), d, a.hex(), b.hex())


def test_reciprocals_are_rounded_to_nearest():
    for d, y in RECIP.items():
        assert y == float(Fraction(1, d))
        assert abs(Fraction(y) * d - 1) <= Fraction(1, 2 ** 54)   # within 2^-54 relative: q within one ulp


def test_nan_takes_the_division():
    assert math.isnan(div_small(math.nan, 3))
    assert np.isfinite(div_small(1.0, 7))
