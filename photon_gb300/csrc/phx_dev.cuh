// Device-side data layout and helpers of the GB300 gas-phase step.
//
// One scenario's state lives in HBM as structure-of-arrays in the reference's
// index order (src/sim/solver.h:216-220), so a field downloads into a
// photon::Solver vector with one copy. A scenario is described to the kernels
// by a Scn record in device memory; a launch covers one "domain" (cells,
// faces of one axis, one multigrid level, ...) of every scenario of a batch,
// with CTA b of the launch mapped to (scenario, tile) by a prefix table.
#pragma once
#include <cstdint>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

namespace phx {

// model constants: src/sim/solver.h:159-181, src/sim/gasphase.cpp:25-32,
// src/sim/solver.cpp:15-20, all as the FP64 values of the reference's literals
constexpr double K_T0 = 293.15;
constexpr double K_P0 = 101325.0;
constexpr double K_RS = 287.0;
constexpr double K_CP = 1100.0;
constexpr double K_G = 9.81;
constexpr double K_YO2_AMB = 0.232;
constexpr double K_DHC_FUEL = 25.0e6;
constexpr double K_S_O2 = 1.95;
constexpr double K_Y_H2O = 0.761;
constexpr double K_C_FRAC = 0.597;
constexpr double K_CO_YIELD = 0.02;
constexpr double K_YCO2_AMB = 0.0006;
constexpr double K_YH2O_AMB = 0.0073;
constexpr double K_CHI_R = 0.35;
constexpr double K_T_CRIT = 1600.0;
constexpr double K_T_AUTO = 800.0;
constexpr double K_TAU_MIX = 0.1;
constexpr double K_PR_T = 0.5;
constexpr double K_SC_T = 0.5;
constexpr double K_C_NU = 0.1;
constexpr double K_D_MAX = 50.0;
constexpr double K_VMAX = 40.0;
constexpr double K_T_MIN = 200.0;
constexpr double K_T_MAX = 2300.0;
constexpr double K_BURNER_SOOT = 0.01;
constexpr double K_GAMMA = K_CP / (K_CP - K_RS);

constexpr int NSC = 10;          // transported scalars: T Yo Yf Ys Ya Yp Yc Yw Yco Yai

// Temperature storage. The FP64 path stores the temperature itself. The mixed
// path stores its offset from the ambient T0 (theta = T - 293.15 K, converted
// in FP64 at the host boundary): ambient cells hold exactly 0 and a cell a
// fraction of a kelvin above ambient keeps FP32's relative precision on that
// fraction. With T itself in FP32 (ulp about 3e-5 K near 293 K), the rounding
// of near-ambient cells drives buoyancy and baroclinic noise that the
// projection turns into pressure errors of up to 3e-5 relative in a
// quiescent house (the reference's own float build shows the same).
// Differences of temperatures are differences of offsets; the absolute
// temperature (densities, viscosity, conductivity, ignition, radiation)
// is tAbs(stored).
template <class R>
__host__ __device__ __forceinline__ constexpr bool tempIsOffset() { return sizeof(R) == 4; }
template <class R>
__host__ __device__ __forceinline__ R tAbs(R stored) {
    if constexpr (sizeof(R) == 4) return R(K_T0) + stored;
    else return stored;
}
// the stored value of the ambient temperature
template <class R>
__host__ __device__ __forceinline__ constexpr R tAmbient() { return sizeof(R) == 4 ? R(0) : R(K_T0); }
// conversions between a temperature in K and the stored value, in FP64
template <class R>
__host__ __device__ __forceinline__ constexpr double tStoredFromKd(double t) { return sizeof(R) == 4 ? t - K_T0 : t; }
template <class R>
__host__ __device__ __forceinline__ constexpr double tKFromStoredd(double s) { return sizeof(R) == 4 ? K_T0 + s : s; }
// per-face transport record: upwind density, the 10 limited face values, and
// the diffusion terms of the 9 species for the momentum-free and the mass form
constexpr int ADV_RUP = 0, ADV_FACE = 1, ADV_DQ = ADV_FACE + NSC, ADV_MQ = ADV_DQ + NSC - 1,
              ADV_REC = ADV_MQ + NSC - 1;
constexpr int MAX_SRC = 16;      // burners + ignitions per scenario
constexpr int MAX_LEVELS = 12;   // multigrid levels (the reference's cap)
constexpr int TPB = 256;         // threads per CTA of the cell/face kernels
constexpr int MAX_BATCH = 1024;  // scenarios per batch (the persistent kernels keep their table in shared memory)

// scalar slots of a scenario (double each)
enum Slot {
    SV_DTMAX_ARG = 0, SV_DT, SV_TIME, SV_MAXVEL, SV_MAXNU, SV_MAXDIV,
    SV_RZ, SV_ALPHA, SV_BETA, SV_RMAX, SV_BMAX, SV_IT, SV_DONE, SV_DQ,
    SV_PITERS, SV_PRES, SV_PREL, SV_HRR, SV_MAXGAST, SV_BURNING, SV_FUELIN, SV_FUELBURNED, SV_FUELINDOMAIN,
    SV_INV, SV_ACTIVE,
    // mixed path: FP64 refinement loop around the FP32 inner CG
    SV_R64MAX, SV_R0MAX, SV_OUTER, SV_ODONE, SV_ITTOT, SV_REPL,
    SV_HAVEPREV,                 // mixed path: p64prev holds the previous step's pressure
    SV_SRC_MF = 32,              // MAX_SRC injection amounts of this step (-1 = inactive)
    SV_BREAK = SV_SRC_MF + MAX_SRC,   // mixed path: 1 after a CG breakdown (next update skipped), 2 restart pending
    SV_COUNT = 64
};

// reduction partial slots (each holds one double per CTA of the cell domain)
enum PartSlot { PS_DQ = 0, PS_RZ, PS_HRR, PS_FUEL, PS_COUNT };

// a burner or ignition source: the gas cells it feeds are the unblocked cells
// of the box [i0,i1] x [j0,j1] x {k} (Solver::addBurner, src/sim/gasphase.cpp:72-90)
struct Src {
    int kind;                    // 0 ignition, 1 burner
    int i0, i1, j0, j1, k;
    int ncells;                  // b.cells.size() at addBurner time
    double peakW, rampS, start, duration;   // burner
    double power;                // ignition power (W)
};

// division by a grid dimension d as a multiply-high: q = floor(x m / 2^64)
// with m = ceil(2^64 / d) is exact for every 32-bit x (the error x (m - 2^64 / d)
// / 2^64 stays below 1 / d)
struct DivU {
    unsigned long long m;
    unsigned d;
};
inline DivU makeDivU(unsigned d) {
    DivU v;
    v.d = d;
    v.m = d <= 1 ? 0ull : (~0ull / d) + 1ull;
    return v;
}
__device__ __forceinline__ unsigned divU(unsigned x, const DivU& v) {
    return v.d <= 1 ? x : (unsigned)__umul64hi((unsigned long long)x, v.m);
}

template <class R>
struct Level {
    int n;                       // unknowns
    const int *rowStart, *col;   // couplings (off-diagonal, positive), coarse levels
    const R* val;
    const R* diag;
    const int* agg;              // unknown -> unknown of the next coarser level (nullptr at the coarsest)
    const int *childStart, *child;   // next coarser unknown -> its unknowns here, ascending
    R *x, *y, *b;                // iterate, Jacobi scratch, right-hand side
    const R* dense;              // coarsest only: n x n operator of the reference's coarse solve
};

template <class R>
struct Scn {
    int nx, ny, nz, N, NX, NY, NZ;
    // index recovery of the three layouts (kind 0: cells and z-faces, 1: x-faces, 2: y-faces):
    // row length dvA, plane size dvB, rows per plane dY
    DivU dvA[3], dvB[3];
    int dY[3];
    DivU dvL0[2];                // 2x2x2 blocks of the mixed path's level-0 kernels: blocks per row, per plane
    double dx, ox, oy, oz;
    double cfl, dtMaxP, tol, relTol;
    const double* dtMaxArg;      // this step's dtMax argument (one slot per scenario of the batch)
    int maxIters;
    int radiationOn;
    double windSpeed, windSin, windCos, windExp;   // sin/cos of the wind direction taken on the host
    int nsrc;
    Src src[MAX_SRC];
    // geometry
    R rdx, rdx2;                 // 1 / dx and 1 / (dx dx), each one division in R
    const uint8_t* blocked;
    const R *fx, *fy, *fz;       // face open fractions
    const R *ax, *ay, *az;       // pressure-matrix coefficients (ax_, ay_, az_)
    const R *a0x, *a0y, *a0z;    // the same with wind-inflow boundary faces closed (multigrid level 0)
    const uint8_t *lx, *ly, *lz; // crack faces (null when there are none)
    const R* diag;               // level-0 diagonal
    const unsigned char* code0;  // mixed path: level-0 coefficient code per cell (level0.cuh)
    const int* zone;
    const uint8_t* zoneOpen;
    int nZones, nClosed;
    const int* closedZone;       // closed zone ids
    const int *closedStart, *closedCells;   // per closed zone: its cells, ascending
    double* zoneP;               // Pa per zone
    double* zoneVol;
    double* zoneDP;
    double* zoneShift;
    double* zoneMean;
    // crack faces (the leakage network, src/sim/gasphase.cpp:410-499)
    int nLeak;                   // leak faces (0: none)
    const int4* leak;            // per face: axis, face index, cell a (-1 outside), cell b
    const int *leakZStart, *leakZList;   // per zone: its leak faces to other zones, ascending
    double* leakQ;               // m3/s through each leak face this step (a -> b)
    double* zonePnew;            // the implicit end-of-step pressure of each closed zone
    double* zoneDInt;            // the zone integral of S
    // state
    R *u, *v, *w, *u2, *v2, *w2;
    R* sc[NSC];                  // current scalars
    R* sc2[NSC];                 // next scalars (swapped after transport)
    R *p, *S, *nu, *Pb, *Q, *Qr, *hrr, *massSrc;
    uint8_t *lit, *lit2, *pilot;
    R* tmp[9];                   // turbulence: cell-centre velocities and filter passes
    double* adv;                 // FP64 path: per-face transport records (ADV_REC arrays over the
                                 // NX + NY + NZ faces, x faces first), k_adv_faces -> k_advect
    // pressure solve
    R *b, *r, *z, *d, *q;
    double* p64;                 // mixed path: FP64 pressure; the FP32 iterate p holds the part not yet folded in
    int mixed;                   // mixed path: FP32 CG with FP64 residual replacement
    int replaceEvery;            // mixed path: iterations between FP64 residual replacements
    int extrap;                  // mixed path: start the solve from 2 p(n) - p(n-1) (PHX_NO_EXTRAP=1: from p(n))
    double* p64prev;             // mixed path: the previous step's pressure (FP64)
    int fp16Scratch;             // mixed path: Jacobi scratch rounded to FP16 (an accuracy study; off by default)
    int fp16Z0;                  // mixed path: level-0 smoother output z rounded to FP16 (an accuracy study; off by default)
    int nLevels;
    int smooth1;                 // mixed path: one damped Jacobi sweep per coarse level on each leg
                                 // of the V-cycle (the reference: two, src/sim/pressure_mg.cpp:281-297)
    Level<R> lv[MAX_LEVELS];
    // row-block tiles of the level-0 pressure kernels: tj rows x RB_KZ planes, njb blocks along y
    int tj, njb;
    unsigned* errWord;           // the context's error word (a bounded wait that ran out sets bit 0)
    // scalars and reductions
    double* sv;
    double* part;                // PS_COUNT x partStride
    int partStride;
    unsigned* cnt;               // last-CTA counters, one per reduction kind
};

// CTA -> (scenario, tile) over a domain
struct Dom {
    const int* start;            // [nscn + 1] prefix of CTAs per scenario
    int nscn;
    int total;                   // CTAs of the launch
    const unsigned* owner;       // [total] scenario << 20 | tile of each CTA (null: search the prefix)
};

// the same over the scenarios still active in a solve: the prefix and the
// total live in device memory and are rebuilt between iterations, so a
// persistent grid loops over the tiles of unfinished scenarios only
struct ADom {
    const int* start;            // [nscn + 1], zero-width for finished scenarios
    const int* total;
    int nscn;
};

// binary search in a shared-memory copy of an active prefix
__device__ __forceinline__ void locateShared(const int* st, int nscn, int b, int& s, int& tile) {
    int lo = 0, hi = nscn - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (st[mid] <= b) lo = mid; else hi = mid - 1;
    }
    s = lo;
    tile = b - st[lo];
}

__device__ __forceinline__ void locate(const ADom& d, int b, int& s, int& tile) {
    int lo = 0, hi = d.nscn - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (d.start[mid] <= b) lo = mid; else hi = mid - 1;
    }
    s = lo;
    tile = b - d.start[lo];
}

__device__ __forceinline__ void locate(const Dom& d, int b, int& s, int& tile) {
    if (d.owner) {   // one load instead of a search through the prefix
        const unsigned v = __ldg(d.owner + b);
        s = (int)(v >> 20);
        tile = (int)(v & 0xFFFFFu);
        return;
    }
    int lo = 0, hi = d.nscn - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (__ldg(d.start + mid) <= b) lo = mid; else hi = mid - 1;
    }
    s = lo;
    tile = b - __ldg(d.start + lo);
}

// libstdc++'s std::min / std::max / std::clamp
__device__ __forceinline__ double mn(double a, double b) { return (b < a) ? b : a; }
__device__ __forceinline__ double mx(double a, double b) { return (a < b) ? b : a; }
__device__ __forceinline__ double clampd(double v, double lo, double hi) { return (v < lo) ? lo : (hi < v) ? hi : v; }
__device__ __forceinline__ float mn(float a, float b) { return (b < a) ? b : a; }
__device__ __forceinline__ float mx(float a, float b) { return (a < b) ? b : a; }
__device__ __forceinline__ float clampd(float v, float lo, float hi) { return (v < lo) ? lo : (hi < v) ? hi : v; }

// max of non-negative doubles through their bit patterns (order independent)
__device__ __forceinline__ void atomicMaxPos(double* a, double v) {
    if (!(v > 0)) return;
    atomicMax(reinterpret_cast<unsigned long long*>(a), (unsigned long long)__double_as_longlong(v));
}

__device__ __forceinline__ double warpMax(double v) {
    for (int o = 16; o > 0; o >>= 1) v = mx(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ double warpSum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ float warpSum(float v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ float warpMax(float v) {
    for (int o = 16; o > 0; o >>= 1) v = mx(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// CTA-wide max of non-negative values into *dst: warp maxima, then one warp
// over them and one atomic per CTA (an atomic per warp put thousands of
// same-address atomics per scenario into each launch). Every thread of the CTA
// must call it (it has barriers); V is the arithmetic type of the values.
template <class V>
__device__ __forceinline__ void blockMaxTo(double* dst, V v) {
    __shared__ V shMax[32];
    v = warpMax(v);
    const int w = (int)(threadIdx.x >> 5), l = (int)(threadIdx.x & 31), nw = (int)((blockDim.x + 31) >> 5);
    __syncthreads();   // a previous call's last warp may still read the buffer
    if (l == 0) shMax[w] = v;
    __syncthreads();
    if (w == 0) {
        V x = l < nw ? shMax[l] : V(0);
        x = warpMax(x);
        if (l == 0) atomicMaxPos(dst, (double)x);
    }
}

// Sums of the FP32 path: an unevaluated pair hi + lo of floats (about 48
// significant bits) formed and added with FP32 instructions only -- the exact
// product of Dekker (an FMA yields the rounding error of a*b) and Knuth's
// TwoSum, i.e. the double-float arithmetic of Hida, Li & Bailey's QD library.
// GB300 issues FP64 at a small fraction of its FP32 rate, so the dot products
// of the FP32 CG keep FP64-grade accuracy at FP32 cost. The _rn intrinsics
// keep the compiler from contracting the error terms.
struct F2 {
    float hi, lo;
};
__device__ __forceinline__ F2 f2prod(float a, float b) {
    const float p = __fmul_rn(a, b);
    return F2{p, __fmaf_rn(a, b, -p)};
}
__device__ __forceinline__ F2 f2add(F2 a, F2 b) {
    const float s = __fadd_rn(a.hi, b.hi);
    const float v = __fsub_rn(s, a.hi);
    const float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, v)), __fsub_rn(b.hi, v));
    const float t = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
    const float hi = __fadd_rn(s, t);
    return F2{hi, __fsub_rn(t, __fsub_rn(hi, s))};
}
__device__ __forceinline__ double f2value(F2 v) { return (double)v.hi + (double)v.lo; }

// one term of a dot product in the accumulator of the arithmetic type
__device__ __forceinline__ double dotTerm(double a, double b) { return a * b; }
__device__ __forceinline__ F2 dotTerm(float a, float b) { return f2prod(a, b); }
__device__ __forceinline__ double accAdd(double a, double b) { return a + b; }
__device__ __forceinline__ F2 accAdd(F2 a, F2 b) { return f2add(a, b); }

__device__ __forceinline__ F2 warpSum(F2 v) {
    for (int o = 16; o > 0; o >>= 1) {
        const F2 w{__shfl_down_sync(0xffffffffu, v.hi, o), __shfl_down_sync(0xffffffffu, v.lo, o)};
        v = f2add(v, w);
    }
    return v;
}

// fixed-order CTA sum (the order depends only on the CTA size)
__device__ __forceinline__ double blockSum(double v, double* sh) {
    v = warpSum(v);
    int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
    __syncthreads();
    if (l == 0) sh[w] = v;
    __syncthreads();
    double t = 0;
    if (w == 0) {
        t = l < nw ? sh[l] : 0.0;
        t = warpSum(t);
    }
    return t;   // valid in thread 0
}
// the same for double-float terms; the CTA total is rounded to double once
__device__ __forceinline__ double blockSum(F2 v, double* sh) {
    static_assert(sizeof(F2) == sizeof(double), "F2 shares the double scratch");
    F2* shf = reinterpret_cast<F2*>(sh);
    v = warpSum(v);
    int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
    __syncthreads();
    if (l == 0) shf[w] = v;
    __syncthreads();
    F2 t{0.f, 0.f};
    if (w == 0) {
        if (l < nw) t = shf[l];
        t = warpSum(t);
    }
    return f2value(t);   // valid in thread 0
}

// Solver::windAt (src/sim/gasphase.cpp:52-61); NaN = no inflow on this face
template <class R>
__device__ __forceinline__ double windAt(const Scn<R>& s, int axis, int side, double z) {
    if (s.windSpeed <= 0 || axis == 2) return __longlong_as_double(0x7ff8000000000000LL);
    double U = s.windSpeed * pow(mx(z, 0.05) / 10.0, s.windExp);
    double comp = axis == 0 ? -s.windSin * U : -s.windCos * U;
    if (side == 0 && comp > 0) return comp;
    if (side == 1 && comp < 0) return comp;
    return __longlong_as_double(0x7ff8000000000000LL);
}

template <class R>
__device__ __forceinline__ bool bndOpen(const Scn<R>& s, int axis, int side, double z) {
    return isnan(windAt(s, axis, side, z));
}

}  // namespace phx
