// FP64 division by a small positive integer, correctly rounded: the same
// result as x / d, in three FP64 operations instead of a full division.
//
// The level-0 smoothing sweeps of the FP64 path divide by each cell's diagonal,
// which for a coded cell (level0.cuh) is the integer d = 1..7. GB300 issues
// FP64 arithmetic at a small fraction of its FP32 rate, and a general division
// costs several times the operations of a multiply.
//
// Method: Markstein's correction (P. Markstein, "Computation of elementary
// functions on the IBM RISC System/6000 processor", IBM J. Res. Dev. 34(1),
// 1990). If y is within half an ulp of 1/d and q within one ulp of x/d, then
// e = x - d q is exactly representable (one FMA computes it exactly), and
// RN(q + e y) = RN(x / d). Here y = RN(1/d) (the constants below), and q =
// RN(x y): for d = 1, 2, 4 it is exact; for d = 3, 5, 6, 7, RN(1/d) is within
// 2^-54 relative of 1/d, so |q - x/d| < 0.5 ulp + 2^53 * 2^-54 ulp = 1 ulp.
// The theorem assumes no underflow or overflow: zeros (whose sign the FMAs
// would not keep), values below 2^-960, infinities and NaNs take the plain
// division. A GPU test compares the two forms bit for bit over random and
// constructed inputs for every d.
#pragma once

namespace phx {

static_assert(1.0 / 3.0 == 0x1.5555555555555p-2 && 1.0 / 5.0 == 0x1.999999999999ap-3 &&
                  1.0 / 6.0 == 0x1.5555555555555p-3 && 1.0 / 7.0 == 0x1.2492492492492p-3,
              "reciprocals rounded to nearest");

// RN(1/d) for d = 1..7 (selects, no table in memory)
__device__ __forceinline__ double recipSmall(int d) {
    return d == 1 ? 1.0 : d == 2 ? 0.5 : d == 3 ? 0x1.5555555555555p-2 : d == 4 ? 0.25
         : d == 5 ? 0x1.999999999999ap-3 : d == 6 ? 0x1.5555555555555p-3 : 0x1.2492492492492p-3;
}

// x / d for d = 1..7, bit-identical to the IEEE quotient
__device__ __forceinline__ double divSmall(double x, int d) {
    const unsigned ex = ((unsigned)__double2hiint(x) >> 20) & 0x7ffu;
    if (ex < 63u || ex == 0x7ffu) return x / (double)d;
    const double y = recipSmall(d);
    const double q = x * y;
    const double e = fma(-q, (double)d, x);
    return fma(e, y, q);
}

}  // namespace phx
