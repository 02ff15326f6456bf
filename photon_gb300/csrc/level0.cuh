// Level-0 pressure kernels: the 7-point structured grid of the multigrid
// V-cycle and of q = A d, with the matrix coefficients coded in one byte per
// cell. Both precisions run them (R = double: the FP64 path; R = float: the
// mixed path).
//
// Coefficient codes. On the grids Photon discretizes, the level-0 matrix
// coefficients (a0x, a0y, a0z: open fractions of a cell's six faces) are 0 or
// 1 nearly everywhere, and the diagonal is their sum. A cell's code holds, in
// bits 0-5, which of its interior faces (x-, x+, y-, y+, z-, z+) couple it to
// its neighbour with a coefficient of exactly 1, and in bit 7 one open
// domain-boundary face (it adds 1 to the diagonal and has no neighbour). Its
// diagonal is then the number of those bits. A cell with any other
// coefficient, more than one open boundary face, or a diagonal that is not
// that count gets bit 6 ("general") and its coefficients are read from the
// arrays as before. The host builds and checks every code. Multiplying by a
// coefficient of 1 is exact and adding a zero term changes nothing, so a
// coded cell computes what the array form computes, in the same order (the
// FP64 path's sums keep the reference's order and rounding). A pass then
// streams 1 byte per cell of matrix data instead of four coefficient arrays.
//
// Blocks of 2x2x2 cells. A thread owns one 2x2x2 block (the blocks level 1
// aggregates) and computes its eight cells: it loads the block's values once,
// takes three of each cell's six stencil neighbours from its own registers and
// loads the other three from the neighbouring blocks (cache hits: the
// neighbouring threads load them as their own). No thread waits for another
// and every load of a thread is independent of the others, so the loads of
// many blocks are in flight at once; the level-1 restriction of a block is
// the sum of one thread's registers in ascending cell order. Red cells
// (i + j + k even) are cells 0, 3, 5 and 6 of every block (cell u = di + 2 dj
// + 4 dk), so a sweep loads only the neighbours of the colour it reads.
#pragma once
#include <type_traits>

#include "fdiv.cuh"
#include "rowblock.cuh"

namespace phx {

// bits 0-5: interior faces x-, x+, y-, y+, z-, z+ with coefficient 1; bit 7:
// one open boundary face; bit 6: read the arrays
constexpr unsigned char CODE_GENERAL = 64;
constexpr unsigned char CODE_BOUNDARY = 128;

constexpr int L0_THREADS = 128;

// passes of k_l0; q = A d reads the d that k_l0_dupdate formed
enum { L0_APPLY = 0, L0_PRE, L0_RES, L0_BLACK, L0_RED, L0_MODES };

// 2x2x2 blocks per thread: one for the sweeps, the residual and q = A d;
// four for the red sweep of a batch that fills the GPU several times over,
// whose per-tile r.z reduction they amortise (a small grid keeps one, so
// that its few tiles spread over more CTAs)
constexpr int L0_RED_WIDE = 4;
__host__ __device__ constexpr int l0Bpt(int mode) { return mode == L0_RED ? L0_RED_WIDE : 1; }

// tiles of a scenario: L0_THREADS x bpt 2x2x2 blocks each
__host__ __device__ inline int l0Tiles(int nx, int ny, int nz, int bpt) {
    const long long nb = (long long)((nx + 1) >> 1) * ((ny + 1) >> 1) * ((nz + 1) >> 1);
    const long long per = (long long)L0_THREADS * bpt;
    return (int)((nb + per - 1) / per);
}

// diagonal of a coded cell
template <class T>
__device__ __forceinline__ T codeDiag(unsigned cd) { return (T)(__popc(cd & 63u) + (cd >> 7)); }

// a smoothing sweep's division by the diagonal: for a coded cell of the FP64
// path by the integer diagonal in three FP64 operations (fdiv.cuh, the same
// quotient), otherwise as the row-block kernels divide
template <class T>
__device__ __forceinline__ T l0Div(T a, unsigned cd, T dg) {
    if constexpr (sizeof(T) == 8) {
        if (!(cd & CODE_GENERAL)) return divSmall(a, (int)(__popc(cd & 63u) + (cd >> 7)));
    }
    return gsDiv(a, dg);
}

// the general-cell form of the stencil: coefficients and diagonal from the arrays
template <class R>
struct L0Coef {
    R dg, xm, xp, ym, yp, zm, zp;
};
template <class R>
__device__ __forceinline__ L0Coef<R> l0General(const Scn<R>& g, int i, int j, int k) {
    const int nx = g.nx, ny = g.ny;
    const long long c = (long long)k * nx * ny + (long long)j * nx + i;
    const long long fx = i + (long long)(nx + 1) * (j + (long long)ny * k);
    const long long fy = i + (long long)nx * (j + (long long)(ny + 1) * k);
    L0Coef<R> o;
    o.dg = g.diag[c];
    o.xm = g.a0x[fx];
    o.xp = g.a0x[fx + 1];
    o.ym = g.a0y[fy];
    o.yp = g.a0y[fy + nx];
    o.zm = g.a0z[c];
    o.zp = g.a0z[c + (long long)nx * ny];
    return o;
}

// neighbour values of one cell in the reference's term order
template <class R>
struct L0Nb {
    R xm, xp, ym, yp, zm, zp;
};

// sacc plus (SIGN > 0) or minus (SIGN < 0) the neighbour terms in the order
// x-, x+, y-, y+, z-, z+: for a coded cell every set bit adds its neighbour
// (coefficient 1); a general cell multiplies by the arrays' coefficients its
// interior neighbours
template <int SIGN, class R>
__device__ __forceinline__ R l0Sum(R sacc, unsigned cd, const L0Coef<R>& a, const L0Nb<R>& n, int i, int j, int k,
                                   int nx, int ny, int nz) {
    if (!(cd & CODE_GENERAL)) {
        if (cd & 1u) sacc = SIGN > 0 ? sacc + n.xm : sacc - n.xm;
        if (cd & 2u) sacc = SIGN > 0 ? sacc + n.xp : sacc - n.xp;
        if (cd & 4u) sacc = SIGN > 0 ? sacc + n.ym : sacc - n.ym;
        if (cd & 8u) sacc = SIGN > 0 ? sacc + n.yp : sacc - n.yp;
        if (cd & 16u) sacc = SIGN > 0 ? sacc + n.zm : sacc - n.zm;
        if (cd & 32u) sacc = SIGN > 0 ? sacc + n.zp : sacc - n.zp;
        return sacc;
    }
    if (SIGN > 0) {
        if (i > 0) sacc += a.xm * n.xm;
        if (i < nx - 1) sacc += a.xp * n.xp;
        if (j > 0) sacc += a.ym * n.ym;
        if (j < ny - 1) sacc += a.yp * n.yp;
        if (k > 0) sacc += a.zm * n.zm;
        if (k < nz - 1) sacc += a.zp * n.zp;
    } else {
        if (i > 0) sacc -= a.xm * n.xm;
        if (i < nx - 1) sacc -= a.xp * n.xp;
        if (j > 0) sacc -= a.ym * n.ym;
        if (j < ny - 1) sacc -= a.yp * n.yp;
        if (k > 0) sacc -= a.zm * n.zm;
        if (k < nz - 1) sacc -= a.zp * n.zp;
    }
    return sacc;
}

// the level-0 smoother's output as stored: as computed, or (mixed path)
// rounded to FP16 when the context studies FP16 storage of the smoother
// scratch (PHX_FP16_Z0)
template <class R>
__device__ __forceinline__ R z0Store(const Scn<R>& g, R v) {
    if constexpr (sizeof(R) == 4) {
        if (g.fp16Z0) return __half2float(__float2half_rn(v));
    }
    return v;
}

// whether a cell reads its neighbour across face f (0..5): a set bit of a
// coded cell, an interior face of a general cell
__device__ __forceinline__ bool l0Reads(unsigned cd, int f, bool interior) {
    return (cd & CODE_GENERAL) ? interior : ((cd >> f) & 1u) != 0;
}

// CTAs per SM the compiler budgets registers for (FP32): the most that keep
// each pass free of spills or nearly so -- eight for the pre-smoothing pair
// and the black sweep (64 registers), six for q = A d and the red sweep (80),
// five for the residual with its restriction (96). The FP64 passes keep the
// compiler's own choice.
template <class R, int MODE>
struct L0MinCtas {
    static constexpr int value = sizeof(R) == 8 ? 1
                                 : (MODE == L0_PRE || MODE == L0_BLACK) ? 8
                                 : (MODE == L0_APPLY || MODE == L0_RED) ? 6
                                 : 5;
};

// One pass over the active tiles of a batch; a thread computes BPT 2x2x2
// blocks. MODE selects the pass:
//   L0_APPLY  q = A d (src/sim/gasphase.cpp:551-570) of the d that
//             k_l0_dupdate formed, d.q (:606-608); alpha in the last CTA of a
//             scenario
//   L0_PRE    pre-smoothing pair from x = 0 (gsColor, pressure_mg.cpp:195-216):
//             red = r / diag, black from its red neighbours; writes z
//   L0_RES    residual (residualGrid, :217-235) restricted to level 1
//             (:285-286): each aggregate's cells summed in ascending order;
//             then level 1's first Jacobi sweep from x = 0
//   L0_BLACK  black sweep after the prolongation (:290-297); red neighbours
//             are z + x1[agg]; writes the black cells of z
//   L0_RED    red sweep with r.z (dotRZ, gasphase.cpp:582-588); the last CTA
//             of a scenario closes the CG iteration (phase 2: a bare V-cycle)
template <class R, int MODE, int BPT>
__global__ void __launch_bounds__(L0_THREADS, (L0MinCtas<R, MODE>::value)) k_l0(const Scn<R>* __restrict__ S, ADom dom,
                                                                                 R* const* dbuf, int phase) {
    using T = R;
    using Acc = decltype(dotTerm(T(0), T(0)));
    __shared__ int sst_[MAX_BATCH + 1];
    __shared__ double shd[32];
    __shared__ int amLastS;
    for (int i = threadIdx.x; i <= dom.nscn; i += blockDim.x) sst_[i] = dom.start[i];
    __syncthreads();
    const int tot = sst_[dom.nscn];
    for (int b = blockIdx.x; b < tot; b += gridDim.x) {
        int s, tile;
        locateShared(sst_, dom.nscn, b, s, tile);
        const Scn<R>& g = S[s];
        const int nx = g.nx, ny = g.ny, nz = g.nz, sxy = nx * ny;
        const int hx = g.dvL0[0].d, hxy = g.dvL0[1].d;
        const int nblk = hxy * ((nz + 1) >> 1);
        Acc dot{};
#pragma unroll 1
        for (int ub = 0; ub < BPT; ++ub) {
        const int q = (tile * BPT + ub) * L0_THREADS + (int)threadIdx.x;
        const bool live = q < nblk;
        const int bz = live ? (int)divU((unsigned)q, g.dvL0[1]) : 0;
        const int rem = q - bz * hxy;
        const int by = live ? (int)divU((unsigned)rem, g.dvL0[0]) : 0;
        const int bx = rem - by * hx;
        const int i0 = 2 * bx, j0 = 2 * by, k0 = 2 * bz;
        const int it = (int)g.sv[SV_IT];
        const T* __restrict__ zf = g.z;
        const T* __restrict__ rf = g.r;
        const unsigned char* __restrict__ cf = g.code0;
        const int* __restrict__ af = g.lv[0].agg;
        const T* __restrict__ dcur = MODE == L0_APPLY ? dbuf[2 * s + ((it + 1) & 1)] : nullptr;
        const T* __restrict__ xc = MODE == L0_BLACK ? g.lv[1].x : nullptr;
        // the stencil value of cell c (red: i + j + k even)
        auto value = [&](int c, bool red) -> T {
            if constexpr (MODE == L0_APPLY) {
                return dcur[c];                                       // d, formed by k_l0_dupdate
            } else if constexpr (MODE == L0_PRE) {
                const T rv = rf[c];
                if (!red) return rv;                                  // black: its right-hand side
                const unsigned cd = cf[c];
                const T dg = (cd & CODE_GENERAL) ? g.diag[c] : codeDiag<T>(cd);
                return dg <= T(0) ? T(0) : l0Div(rv, cd, dg);         // red: after the first half sweep
            } else if constexpr (MODE == L0_BLACK) {
                if (!red) return rf[c];
                const int a = af[c];
                const T zv = zf[c];
                return a >= 0 ? (T)(zv + xc[a]) : zv;                 // red: z plus the prolongated correction
            } else if constexpr (MODE == L0_RED) {
                return red ? rf[c] : zf[c];                           // black: its new z
            } else {
                return zf[c];
            }
        };
        // the block's cells u = di + 2 dj + 4 dk; cells past the grid's end are off
        const int st[3] = {1, nx, sxy};
        const int dimv[3] = {nx, ny, nz};
        const int org[3] = {i0, j0, k0};
        bool on[8];
        int cc[8];
        unsigned cd[8];
        T X[8], Rv[8], NB[8][3];
        int A[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int di = u & 1, dj = (u >> 1) & 1, dk = u >> 2;
            on[u] = live && i0 + di < nx && j0 + dj < ny && k0 + dk < nz;
            cc[u] = (i0 + di) + nx * (j0 + dj) + sxy * (k0 + dk);
            const bool red = ((di + dj + dk) & 1) == 0;
            cd[u] = 0;
            X[u] = T(0);
            Rv[u] = T(0);
            A[u] = -1;
            if (!on[u]) continue;
            cd[u] = cf[cc[u]];
            X[u] = value(cc[u], red);
            if constexpr (MODE == L0_RED) { if (!red) Rv[u] = rf[cc[u]]; }
            if constexpr (MODE == L0_RES) { Rv[u] = rf[cc[u]]; A[u] = af[cc[u]]; }
        }
        // each cell's neighbour outside the block along each axis, where the cell
        // reads it (the sweeps read only the other colour's neighbours of the
        // colour they update)
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const bool red = (((u & 1) + ((u >> 1) & 1) + (u >> 2)) & 1) == 0;
            const bool reads = MODE == L0_APPLY || MODE == L0_RES ||
                               (MODE == L0_RED ? red : !red);   // the colour this pass updates
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                NB[u][a] = T(0);
                const int bit = (u >> a) & 1;                    // 0: the outside neighbour is below, 1: above
                const int f = 2 * a + bit;
                const bool interior = bit ? org[a] + 2 < dimv[a] : org[a] > 0;
                if (on[u] && reads && l0Reads(cd[u], f, interior))
                    NB[u][a] = value(bit ? cc[u] + st[a] : cc[u] - st[a], !red);
            }
        }
        T resv[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            resv[u] = T(0);
            if (!on[u]) continue;
            const int di = u & 1, dj = (u >> 1) & 1, dk = u >> 2;
            const int i = i0 + di, j = j0 + dj, k = k0 + dk;
            const int c = cc[u];
            const bool red = ((di + dj + dk) & 1) == 0;
            const unsigned code = cd[u];
            L0Coef<T> gen{};
            if (code & CODE_GENERAL) gen = l0General(g, i, j, k);
            const T dg = (code & CODE_GENERAL) ? gen.dg : codeDiag<T>(code);
            L0Nb<T> n;
            n.xm = di ? X[u - 1] : NB[u][0];
            n.xp = di ? NB[u][0] : X[u + 1];
            n.ym = dj ? X[u - 2] : NB[u][1];
            n.yp = dj ? NB[u][1] : X[u + 2];
            n.zm = dk ? X[u - 4] : NB[u][2];
            n.zp = dk ? NB[u][2] : X[u + 4];
            if constexpr (MODE == L0_APPLY) {
                if (dg <= T(0)) { g.q[c] = T(0); continue; }
                const T sacc = l0Sum<-1>(dg * X[u], code, gen, n, i, j, k, nx, ny, nz);
                g.q[c] = sacc;
                dot = accAdd(dot, dotTerm(sacc, X[u]));
            } else if constexpr (MODE == L0_PRE) {
                if (red) { g.z[c] = z0Store(g, X[u]); continue; }
                T zc = T(0);
                if (dg > T(0)) zc = z0Store(g, l0Div(l0Sum<1>(X[u], code, gen, n, i, j, k, nx, ny, nz), code, dg));
                g.z[c] = zc;
            } else if constexpr (MODE == L0_BLACK) {
                if (red) continue;
                T zc = T(0);
                if (dg > T(0)) zc = z0Store(g, l0Div(l0Sum<1>(X[u], code, gen, n, i, j, k, nx, ny, nz), code, dg));
                g.z[c] = zc;
            } else if constexpr (MODE == L0_RED) {
                if (red) {
                    T zc = T(0);
                    if (dg > T(0)) zc = z0Store(g, l0Div(l0Sum<1>(X[u], code, gen, n, i, j, k, nx, ny, nz), code, dg));
                    g.z[c] = zc;
                    dot = accAdd(dot, dotTerm(X[u], zc));
                } else {
                    dot = accAdd(dot, dotTerm(Rv[u], X[u]));
                }
            } else {   // L0_RES
                if (A[u] >= 0) resv[u] = l0Sum<1>(Rv[u] - dg * X[u], code, gen, n, i, j, k, nx, ny, nz);
            }
        }
        if constexpr (MODE == L0_RES) {
            // each level-1 aggregate lies in one 2x2x2 block: its cells are summed in
            // ascending cell order (i, then j, then k), the order of the reference's scatter
            if (live) {
                T* const cb = g.lv[1].b;
                T* const y1 = g.nLevels > 2 ? g.lv[1].y : nullptr;
                const T* const d1 = g.lv[1].diag;
#pragma unroll
                for (int m = 0; m < 8; ++m) {
                    const int a = on[m] ? A[m] : -1;
                    bool first = a >= 0;
#pragma unroll
                    for (int p = 0; p < m; ++p) first = first && !(on[p] && A[p] == a);
                    if (!first) continue;
                    T acc = T(0);
#pragma unroll
                    for (int p = m; p < 8; ++p)
                        if (on[p] && A[p] == a) acc = acc + resv[p];
                    cb[a] = acc;
                    // level 1's first damped Jacobi sweep from x = 0 (jacobi,
                    // pressure_mg.cpp:237-247), unless level 1 is the coarsest
                    if (y1) {
                        const T dc = d1[a];
                        const T om = T(OMEGA);
                        y1[a] = dc <= T(0) ? T(0) : scratchRound(g, (T(1) - om) * T(0) + om * acc / dc);
                    }
                }
            }
        }
        }   // blocks of the thread
        if constexpr (MODE == L0_APPLY || MODE == L0_RED) {
            if (MODE == L0_RED && phase == 2) continue;
            const int nt = sst_[s + 1] - sst_[s];
            // fixed-order CTA sum, then the last CTA of the scenario sums the CTA partials
            const double v = blockSum(dot, shd);
            constexpr int slot = MODE == L0_RED ? PS_RZ : PS_DQ;
            double* part = g.part + (size_t)slot * g.partStride;
            unsigned* cnt = g.cnt + slot;
            if (threadIdx.x == 0) {
                part[tile] = v;
                __threadfence();
                const unsigned tk = atomicAdd(cnt, 1u);
                amLastS = (tk == (unsigned)nt - 1u);
            }
            __syncthreads();
            if (amLastS) {
                __threadfence();
                double acc = 0;
                for (int i = threadIdx.x; i < nt; i += L0_THREADS) acc += __ldcg(part + i);
                const double total = blockSum(acc, shd);
                if (threadIdx.x == 0) {
                    *cnt = 0;
                    if constexpr (MODE == L0_APPLY) {
                        g.sv[SV_DQ] = total;
                        if (g.sv[SV_BREAK] == 1) {   // the iteration after a breakdown: no update, then a restart
                            g.sv[SV_ALPHA] = 0;
                            g.sv[SV_BREAK] = 2;
                        } else if (total <= 0) {
                            g.sv[SV_DONE] = 1;
                        } else {
                            g.sv[SV_ALPHA] = g.sv[SV_RZ] / total;
                        }
                    } else {
                        closeCgIteration(g, phase, total);
                    }
                }
            }
        }
    }
}

// d = z + beta d (src/sim/gasphase.cpp:620-622; d = z on the first iteration)
// ahead of q = A d, four cells per thread over the tiles of k_cg_update (1024
// cells: every tile starts on a 16-byte boundary of a float array and a
// 32-byte boundary of a double array)
template <class R>
__global__ void __launch_bounds__(256) k_l0_dupdate(const Scn<R>* __restrict__ S, ADom dom, R* const* dbuf) {
    __shared__ int sst_[MAX_BATCH + 1];
    for (int i = threadIdx.x; i <= dom.nscn; i += blockDim.x) sst_[i] = dom.start[i];
    __syncthreads();
    const int tot = sst_[dom.nscn];
    for (int b = blockIdx.x; b < tot; b += gridDim.x) {
        int s, tile;
        locateShared(sst_, dom.nscn, b, s, tile);
        const Scn<R>& g = S[s];
        const int it = (int)g.sv[SV_IT];
        const R beta = (R)g.sv[SV_BETA];
        const R* __restrict__ dp = it > 0 ? dbuf[2 * s + (it & 1)] : nullptr;
        R* __restrict__ dn = dbuf[2 * s + ((it + 1) & 1)];
        const R* __restrict__ z = g.z;
        const int c0 = (tile * 256 + (int)threadIdx.x) * 4;
        if (c0 + 4 <= g.N) {
            // d = z where there is no previous d; one 16-byte access per array and
            // thread (float), two (double)
            constexpr int NV = sizeof(R) == 4 ? 1 : 2;
            using V = typename std::conditional<sizeof(R) == 4, float4, double2>::type;
            constexpr int W = 4 / NV;   // cells per vector
#pragma unroll
            for (int h = 0; h < NV; ++h) {
                V zv = *reinterpret_cast<const V*>(z + c0 + W * h);
                if (dp) {
                    const V pv = *reinterpret_cast<const V*>(dp + c0 + W * h);
                    zv.x = zv.x + beta * pv.x;
                    zv.y = zv.y + beta * pv.y;
                    if constexpr (W == 4) {
                        zv.z = zv.z + beta * pv.z;
                        zv.w = zv.w + beta * pv.w;
                    }
                }
                *reinterpret_cast<V*>(dn + c0 + W * h) = zv;
            }
        } else {
            for (int c = c0; c < g.N; ++c) dn[c] = dp ? (R)(z[c] + beta * dp[c]) : z[c];
        }
    }
}

}  // namespace phx
