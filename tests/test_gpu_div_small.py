"""The FP64 path's division of a coded cell's smoothing numerator by its
integer diagonal (photon_gb300/csrc/fdiv.cuh) equals the device's IEEE
quotient x / d bit for bit, for d = 1..7, on 4 M random doubles over the whole
exponent range and constructed inputs (binade edges, quotients next to a
rounding midpoint, zeros, subnormals, infinities). The harness
(tests/cuda/div_small.cu) is compiled with the FP64 unit's flags."""
import ctypes
import os
import subprocess
from fractions import Fraction

import numpy as np
import pytest

from photon_gb300 import build

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cuda", "div_small.cu")
LIB = os.path.join(ROOT, "photon_gb300", "_build", "div_small.so")


def harness():
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    cmd = [build.NVCC] + build.ARCH + ["-O3", "-std=c++17", "--fmad=false", "-shared", "-Xcompiler", "-fPIC", SRC, "-o", LIB]
    subprocess.run(cmd, check=True)
    lib = ctypes.CDLL(LIB)
    lib.div_small_check.restype = ctypes.c_int
    lib.div_small_check.argtypes = [ctypes.c_void_p, ctypes.c_longlong, ctypes.c_void_p, ctypes.c_void_p]
    return lib


def inputs():
    rng = np.random.default_rng(7)
    n = 4_000_000
    sign = rng.integers(0, 2, n, dtype=np.uint64) << np.uint64(63)
    expo = rng.integers(0, 2047, n, dtype=np.uint64) << np.uint64(52)    # subnormal to the largest finite
    mant = rng.integers(0, 1 << 52, n, dtype=np.uint64)
    parts = [(sign | expo | mant).view(np.float64)]
    k = np.arange(20000, dtype=np.float64)
    for e in (-300, -17, 0, 40, 900):
        parts.append(np.ldexp(1.0 + k * 2.0 ** -52, e))
        parts.append(np.ldexp(2.0 - (k + 1) * 2.0 ** -52, e))
    mids = []
    q = 1.0 + rng.integers(0, 1 << 52, 2000) * 2.0 ** -52
    for d in range(3, 8):
        for qv in q:
            mid = Fraction(float(qv)) + Fraction(1, 2 ** 53)
            for off in (-2, -1, 0, 1, 2):
                mids.append(float(d * mid + off * Fraction(1, 2 ** 60)))
    parts.append(np.array(mids))
    parts.append(np.array([0.0, -0.0, 5e-324, -5e-324, 2.0 ** -1000, 2.0 ** -960, np.inf, -np.inf,
                           1.7976931348623157e308, -1.7976931348623157e308]))
    parts.append(np.arange(1, 100000, dtype=np.float64) * 3.0)
    return np.ascontiguousarray(np.concatenate(parts))


def test_div_small_equals_ieee_quotient():
    lib = harness()
    x = inputs()
    fast = np.empty(x.size * 7)
    ref = np.empty(x.size * 7)
    rc = lib.div_small_check(x.ctypes.data, x.size, fast.ctypes.data, ref.ctypes.data)
    assert rc == 0, rc
    fb, rb = fast.view(np.uint64), ref.view(np.uint64)
    bad = np.nonzero(fb != rb)[0]
    # NaN inputs (random patterns with the top exponent) give NaN both ways
    nan_both = np.isnan(fast[bad]) & np.isnan(ref[bad])
    bad = bad[~nan_both]
    assert bad.size == 0, [(float(x[i // 7]).hex(), i % 7 + 1, float(fast[i]).hex(), float(ref[i]).hex())
                           for i in bad[:5]]
    # the reference is the IEEE quotient: check a sample against Python's
    idx = np.random.default_rng(1).integers(0, x.size, 2000)
    for j in idx:
        for d in range(1, 8):
            v = float(x[j]) / d
            if not np.isnan(v):
                assert np.float64(v).view(np.uint64) == rb[7 * j + d - 1]
