// CUDA kernels of the pressure projection: the multigrid V-cycle
// (src/sim/pressure_mg.cpp:193-300) and the preconditioned CG loop
// (src/sim/gasphase.cpp:551-626).
//
// Level 0, the structured 7-point grid, runs on row-block tiles staged in
// shared memory (rowblock.cuh: q = A d, the red-black half sweeps, the
// residual with its restriction). This file holds the CG update, the coarse
// levels and the active-tile tables.
// Coarse levels are CSR rows: damped Jacobi (omega 0.7) and a gather of the
// children's residuals in ascending order. The coarsest level's 20 forward +
// backward Gauss-Seidel sweeps from x = 0 are a fixed linear map of b; it is
// applied as a dense operator built on the host from those sweeps.
//
// The CG scalars live in device memory per scenario: the last CTA of each
// reduction computes alpha, beta and the stop test, so no host round trip is
// needed between iterations, and a converged scenario's CTAs return at once.
#pragma once
#include "step_kernels.cuh"

namespace phx {

// Persistent loop over the active tiles of a domain: the body runs once per
// (scenario, tile); `break` ends the current tile.
#define PHX_TILES_BEGIN(ad)                                              \
    __shared__ int sst_[MAX_BATCH + 1];                                  \
    for (int i_ = threadIdx.x; i_ <= (ad).nscn; i_ += blockDim.x)        \
        sst_[i_] = (ad).start[i_];                                       \
    __syncthreads();                                                     \
    const int tot_ = sst_[(ad).nscn];                                    \
    for (int b_ = blockIdx.x; b_ < tot_; b_ += gridDim.x) {              \
        int s_, tile_;                                                   \
        locateShared(sst_, (ad).nscn, b_, s_, tile_);                    \
        const Scn<R>& g = S[s_];                                         \
        if (g.sv[SV_DONE] != 0) continue;                                \
        do {
#define PHX_TILES_END \
        } while (0);  \
    }

constexpr double OMEGA = 0.7;

// the Jacobi sweeps' scratch value (y, between the two sweeps of a level),
// rounded to FP16 when the context studies FP16 scratch storage
template <class R>
__device__ __forceinline__ R scratchRound(const Scn<R>& g, R v) {
    if constexpr (sizeof(R) == 4) {
        if (g.fp16Scratch) return __half2float(__float2half_rn(v));
    }
    return v;
}

// The solve kernels compute in the arithmetic type T = R of the path (FP64 or
// FP32); dot products accumulate in Acc (double, or a double-float pair on
// the FP32 path) and reach the per-scenario scalars as doubles.

// ---- coarse levels ------------------------------------------------------------------
// Each coarse-level pass is a per-tile device function run by a persistent
// kernel over the active tiles; a tile function returns early where the tile
// ends. (Two ways of saving the passes' launches were measured slower: all
// coarse passes as phases of one cooperative kernel with grid barriers, and a
// scenario's small levels on one thread-block cluster per scenario with
// cluster barriers between the passes. A launch over the whole GPU hides the
// dependent loads of a pass's rows better than either.)

// damped Jacobi sweep on a coarse level (jacobi, pressure_mg.cpp:237-247).
// mode 0: from x = 0, into y; mode 1: y -> x; mode 2: x plus the coarser
// level's x prolongated (:290-297), into y; mode 3 (the mixed path's one-sweep
// schedule): y plus the coarser level's x prolongated, into x.
template <class R>
__device__ __forceinline__ void jacobiRow(const Scn<R>& g, int I, int l, int mode) {
    using T = R;
    const Level<R>& L = g.lv[l];
    if (I >= L.n) return;
    const bool toX = mode == 1 || mode == 3, prolong = mode == 2 || mode == 3;
    R* out = toX ? L.x : L.y;
    const T dg = L.diag[I];
    if (dg <= 0) { out[I] = 0; return; }
    const T om = T(OMEGA);
    if (mode == 0) {
        T s = L.b[I];
        out[I] = scratchRound(g, (T(1) - om) * T(0) + om * s / dg);
        return;
    }
    const R* in = toX ? L.y : L.x;
    const R* xc = prolong ? g.lv[l + 1].x : nullptr;
    const int* agg = L.agg;
    auto X = [&](int n) -> T {
        T v = in[n];
        if (prolong) v = v + xc[agg[n]];
        return v;
    };
    T s = L.b[I];
    for (int q = L.rowStart[I]; q < L.rowStart[I + 1]; ++q) s += L.val[q] * X(L.col[q]);
    const T v = (T(1) - om) * X(I) + om * s / dg;
    out[I] = toX ? v : scratchRound(g, v);
}
template <class R>
__device__ __forceinline__ void jacobiTile(const Scn<R>& g, int tile, int l, int mode) {
    jacobiRow(g, tile * TPB + (int)threadIdx.x, l, mode);
}

// residual of level l fused with its restriction to level l+1 and the first
// (from-zero) Jacobi sweep of level l+1 (pressure_mg.cpp:248-257, 285-286,
// 237-247). Eight lanes serve one unknown J of level l+1: they compute the
// residuals of J's children eight at a time (children in ascending order),
// and the group's first lane sums them in that order -- the order of the
// reference's scatter -- then sets y_J = omega b_J / diag_J unless level l+1
// is the coarsest. Every thread of the tile takes part (warp shuffles).
constexpr int RRJ_LANES = 8;
template <class R>
__device__ __forceinline__ void resRestrictJac0Group(const Scn<R>& g, int jBase, int l) {
    using T = R;
    const Level<R>& L = g.lv[l];
    const Level<R>& C = g.lv[l + 1];
    const int J = jBase + (threadIdx.x / RRJ_LANES);
    const int c = threadIdx.x % RRJ_LANES;
    const int groupLane0 = threadIdx.x & 31 & ~(RRJ_LANES - 1);
    int nch = 0, e0 = 0;
    if (J < C.n) {
        e0 = L.childStart[J];
        nch = L.childStart[J + 1] - e0;
    }
    const int chunks = __reduce_max_sync(0xffffffffu, (nch + RRJ_LANES - 1) / RRJ_LANES);
    T acc = 0;
    for (int ch = 0; ch < chunks; ++ch) {
        const int idx = ch * RRJ_LANES + c;
        T r = 0;
        if (idx < nch) {
            const int I = L.child[e0 + idx];
            const T dg = L.diag[I];
            if (dg > 0) {
                const R* it = g.smooth1 ? L.y : L.x;   // the level's iterate after its down-leg sweeps
                T s = L.b[I] - dg * it[I];
                for (int q = L.rowStart[I]; q < L.rowStart[I + 1]; ++q) s += L.val[q] * it[L.col[q]];
                r = s;
            }
        }
        for (int q = 0; q < RRJ_LANES; ++q) {
            const T rq = __shfl_sync(0xffffffffu, r, groupLane0 + q);
            if (ch * RRJ_LANES + q < nch) acc = acc + rq;
        }
    }
    if (J < C.n && c == 0) {
        C.b[J] = acc;
        if (l + 1 < g.nLevels - 1) {
            const T dc = C.diag[J];
            const T om = T(OMEGA);
            C.y[J] = dc <= 0 ? T(0) : scratchRound(g, (T(1) - om) * T(0) + om * acc / dc);
        }
    }
}
template <class R>
__device__ __forceinline__ void resRestrictJac0Tile(const Scn<R>& g, int tile, int l) {
    resRestrictJac0Group(g, tile * (TPB / RRJ_LANES), l);
}

// coarsest level: x = M b with the dense operator of the reference's 20
// forward + backward Gauss-Seidel sweeps (pressure_mg.cpp:258-266, 279).
// One warp per row.
template <class R>
__device__ __forceinline__ void coarseDenseRows(const Scn<R>& g, int rowBase) {
    using T = R;
    const Level<R>& L = g.lv[g.nLevels - 1];
    const int row = rowBase + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (row >= L.n) return;
    const R* M = L.dense + (size_t)row * L.n;
    T acc = 0;
    for (int j = lane; j < L.n; j += 32) acc += M[j] * L.b[j];
    acc = warpSum(acc);
    if (lane == 0) L.x[row] = acc;
}
template <class R>
__device__ __forceinline__ void coarseDenseTile(const Scn<R>& g, int tile) {
    coarseDenseRows(g, tile * (TPB / 32));
}

// coarsest level solved as the reference does it: 20 forward + backward
// sweeps, serially in one thread (used when the level is too large for a dense
// operator)
template <class R>
__device__ __forceinline__ void coarseSerialTile(const Scn<R>& g) {
    using T = R;
    if (threadIdx.x != 0) return;
    const Level<R>& L = g.lv[g.nLevels - 1];
    for (int I = 0; I < L.n; ++I) L.x[I] = 0;
    for (int it = 0; it < 20; ++it)
        for (int dir = 0; dir < 2; ++dir)
            for (int t = 0; t < L.n; ++t) {
                int I = dir == 0 ? t : L.n - 1 - t;
                T dg = L.diag[I];
                if (dg <= 0) { L.x[I] = 0; continue; }
                T s = L.b[I];
                for (int q = L.rowStart[I]; q < L.rowStart[I + 1]; ++q) s += L.val[q] * L.x[L.col[q]];
                L.x[I] = s / dg;
            }
}

template <class R>
__global__ void k_jacobi(const Scn<R>* __restrict__ S, ADom dom, int l, int mode) {
    PHX_TILES_BEGIN(dom)
    jacobiTile(g, tile_, l, mode);
    PHX_TILES_END
}
template <class R>
__global__ void k_res_restrict_jac0(const Scn<R>* __restrict__ S, ADom dom, int l) {
    PHX_TILES_BEGIN(dom)
    resRestrictJac0Tile(g, tile_, l);
    PHX_TILES_END
}
template <class R>
__global__ void k_coarse_dense(const Scn<R>* __restrict__ S, ADom dom) {
    PHX_TILES_BEGIN(dom)
    coarseDenseTile(g, tile_);
    PHX_TILES_END
}
template <class R>
__global__ void k_coarse_serial(const Scn<R>* __restrict__ S, ADom dom) {
    PHX_TILES_BEGIN(dom)
    coarseSerialTile(g);
    PHX_TILES_END
}

// CG stop test of the reference (src/sim/gasphase.cpp:605) plus the optional
// relative test max|r| <= relTol max|b|
template <class R>
__device__ __forceinline__ bool cgContinue(const Scn<R>& g, double res, double rmax, int it, double rz) {
    double relStop = g.relTol > 0 ? g.relTol * g.sv[SV_BMAX] : -1.0;
    return res > g.tol && it < g.maxIters && rz > 0 && !(rmax <= relStop);
}

// closes a CG iteration in the last CTA of a scenario once r.z = tot is known:
// beta, the iteration count and the stop test (src/sim/gasphase.cpp:589-605).
// phase 0: first preconditioning before the loop; 1: inside the loop.
template <class R>
__device__ void closeCgIteration(const Scn<R>& g, int phase, double tot) {
    double* sv = g.sv;
    int it = (int)sv[SV_IT];
    if (phase == 0) {
        sv[SV_RZ] = tot;
        it = 0;
    } else {
        sv[SV_BETA] = tot / sv[SV_RZ];
        sv[SV_RZ] = tot;
        it += 1;
    }
    sv[SV_IT] = it;
    if (!g.mixed) {
        const double rmax = sv[SV_RMAX];
        const double res = rmax / sv[SV_INV];
        sv[SV_PRES] = res;
        sv[SV_PREL] = sv[SV_BMAX] > 0 ? rmax / sv[SV_BMAX] : 0.0;
        sv[SV_RMAX] = 0;
        if (!cgContinue(g, res, rmax, it, sv[SV_RZ])) sv[SV_DONE] = 1;
    } else {
        // mixed: the stop test uses the FP64 residual, known where it was
        // just replaced; the FP32 recursive residual schedules the next
        // replacement (every replaceEvery iterations, or once it claims
        // convergence)
        const bool replaced = phase == 0 || sv[SV_REPL] != 0;
        bool converged = false;
        if (replaced) {
            const double r64 = sv[SV_R64MAX];
            const double res = r64 / sv[SV_INV];
            const double rel = sv[SV_BMAX] > 0 ? r64 / sv[SV_BMAX] : 0.0;
            sv[SV_PRES] = res;
            sv[SV_PREL] = rel;
            converged = !(res > g.tol) || (g.relTol > 0 && rel <= g.relTol) || !(r64 > 0);
            sv[SV_R64MAX] = 0;
            // restart the FP32 CG from the replaced residual (d = z) where it is no
            // longer conjugate to the search direction: closed zones (their
            // operators are singular), and any scenario whose FP32 recursion had
            // drifted below the true residual (a strong preconditioner takes the
            // recursion to FP32's rounding floor within a few iterations; the old
            // direction then carries only rounding noise)
            const double rrec = sv[SV_RMAX];
            if (phase != 0 && (g.nClosed > 0 || r64 > 4.0 * rrec)) sv[SV_BETA] = 0;
        }
        // the first iteration after a breakdown's replacement restarts the FP32 CG (d = z)
        if (phase != 0 && sv[SV_BREAK] == 2) {
            sv[SV_BETA] = 0;
            sv[SV_BREAK] = 0;
        }
        // a breakdown (r.z <= 0) of the FP32 recursion short of the FP64 bar: the recursive
        // residual has reached FP32's rounding floor, not the solution. Replace it by the FP64
        // residual on the next iteration (whose update is skipped: alpha = 0) and restart from it.
        const bool breakdown = !(sv[SV_RZ] > 0);
        const bool recover = breakdown && !replaced && phase != 0 && !converged && it < g.maxIters;
        if (recover) {
            sv[SV_BREAK] = 1;
            sv[SV_RZ] = 1.0;   // any positive value: the skipped update does not use it
            sv[SV_BETA] = 0;
        }
        const bool stop = converged || it >= g.maxIters || (breakdown && !recover);
        const double rrec = sv[SV_RMAX];
        const bool claims = phase != 0 && ((g.relTol > 0 && rrec <= 2.0 * g.relTol * sv[SV_BMAX]) ||
                                           rrec / sv[SV_INV] <= 0.5 * g.tol);
        sv[SV_REPL] = (!stop && phase != 0 && ((it % g.replaceEvery) == 0 || claims || recover)) ? 1.0 : 0.0;
        sv[SV_RMAX] = 0;
        if (stop) sv[SV_DONE] = 1;
    }
}

// p += alpha d; r -= alpha q (src/sim/gasphase.cpp:609-615) and max|r| for
// the stop test (:592-602). Four consecutive cells per thread (a tile is 1024
// cells, so a thread's quad starts on a 16-byte boundary on the FP32 path and
// is moved with vector loads and stores).
constexpr int CG_QUAD = 4;
template <class R>
__device__ __forceinline__ void cgUpdateCell(R* p, R* r, const R* d, const R* q, const R* diag, R alpha, int c, R& rm) {
    const R dg = diag[c];
    R rv = r[c];
    if (dg > 0) {
        p[c] = p[c] + alpha * d[c];
        rv = rv - alpha * q[c];
        r[c] = rv;
    }
    rm = mx(rm, (R)fabs(rv));
}

// In the step graph (setCond != 0) the kernel also sets the condition of the
// loop body's conditional node that runs the mixed path's residual
// replacement: on while any scenario replaces its residual this iteration
// (its active-tile total replTotal, built at the end of the previous
// iteration, is not zero), counting the runs in *replRuns.
template <class R>
__global__ void k_cg_update(const Scn<R>* __restrict__ S, ADom dom, R* const* dbuf, cudaGraphConditionalHandle repl,
                            const int* replTotal, int* replRuns, int setCond) {
    using T = R;
    if (setCond && blockIdx.x == 0 && threadIdx.x == 0) {
        const bool run = *replTotal > 0;
        if (run) ++*replRuns;
        cudaGraphSetConditional(repl, run ? 1u : 0u);
    }
    PHX_TILES_BEGIN(dom)
    const int c0 = (tile_ * TPB + threadIdx.x) * CG_QUAD;
    T rm = 0;
    if (c0 < g.N) {
        const int it = (int)g.sv[SV_IT];
        const R* d = dbuf[2 * s_ + ((it + 1) & 1)];
        const T alpha = (T)g.sv[SV_ALPHA];
        if constexpr (sizeof(R) == 4) {
            if (c0 + CG_QUAD <= g.N) {
                const float4 dg = *reinterpret_cast<const float4*>(g.diag + c0);
                const float4 dv = *reinterpret_cast<const float4*>(d + c0);
                const float4 qv = *reinterpret_cast<const float4*>(g.q + c0);
                float4 pv = *reinterpret_cast<const float4*>(g.p + c0);
                float4 rv = *reinterpret_cast<const float4*>(g.r + c0);
                const float* dgs = &dg.x;
                const float* ds = &dv.x;
                const float* qs = &qv.x;
                float* ps = &pv.x;
                float* rs = &rv.x;
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    if (dgs[u] > 0) {
                        ps[u] = ps[u] + alpha * ds[u];
                        rs[u] = rs[u] - alpha * qs[u];
                    }
                    rm = mx(rm, (T)fabsf(rs[u]));
                }
                *reinterpret_cast<float4*>(g.p + c0) = pv;
                *reinterpret_cast<float4*>(g.r + c0) = rv;
            } else {
                for (int c = c0; c < g.N; ++c) cgUpdateCell<R>(g.p, g.r, d, g.q, g.diag, alpha, c, rm);
            }
        } else {
            const int c1 = min(c0 + CG_QUAD, g.N);
            for (int c = c0; c < c1; ++c) cgUpdateCell<R>(g.p, g.r, d, g.q, g.diag, alpha, c, rm);
        }
    }
    blockMaxTo(g.sv + SV_RMAX, rm);
    PHX_TILES_END
}

// Active-tile tables of the solve: for every domain, the prefix of the tiles
// of the scenarios still solving (kind 0) and of those replacing their
// residual this iteration (kind 1, mixed path).
struct ActiveTables {
    const int* tiles;            // [ndom][cap] tiles of each scenario
    int* astart;                 // [2][ndom][cap + 1]
    int* atotal;                 // [2][ndom]
    int nscn, cap, ndom;
    int nlist;                   // the (kind, domain) prefixes the solve's persistent kernels use
    short list[32];              // kind * ndom + domain
};

// One warp per listed (kind, domain): the scenarios' flags are read once into
// shared memory, then each warp scans its domain's tile counts 32 scenarios at
// a time (warp shuffles), so the rebuild costs a few microseconds for any batch.
// Every thread of the block must call it.
template <class R>
__device__ void buildActive(const Scn<R>* __restrict__ S, const ActiveTables& t) {
    __shared__ unsigned char on[2][MAX_BATCH];
    for (int s = threadIdx.x; s < t.nscn; s += blockDim.x) {
        const double* sv = S[s].sv;
        const bool solving = sv[SV_DONE] == 0;
        on[0][s] = solving;
        on[1][s] = solving && sv[SV_REPL] != 0;
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int li = threadIdx.x >> 5; li < t.nlist; li += nw) {
        const int kd = t.list[li];
        const int kind = kd / t.ndom, d = kd % t.ndom;
        int* as = t.astart + (size_t)kd * (t.cap + 1);
        const int* tl = t.tiles + (size_t)d * t.cap;
        int base = 0;
        if (lane == 0) as[0] = 0;
        for (int s0 = 0; s0 < t.nscn; s0 += 32) {
            const int s = s0 + lane;
            int v = (s < t.nscn && on[kind][s]) ? tl[s] : 0;
            for (int o = 1; o < 32; o <<= 1) {
                const int u = __shfl_up_sync(0xffffffffu, v, o);
                if (lane >= o) v += u;
            }
            if (s < t.nscn) as[s + 1] = base + v;
            base += __shfl_sync(0xffffffffu, v, 31);
        }
        if (lane == 0) t.atotal[kd] = base;
    }
}

template <class R>
__global__ void k_active(const Scn<R>* __restrict__ S, ActiveTables t) {
    buildActive(S, t);
}

// Condition of the CG while-loop of the captured step graph: continue while
// any scenario of the launch has not stopped. The loop counter bounds the
// loop whatever the scenarios' flags say, so the graph always terminates.
// Also rebuilds the active-tile tables for the next iteration.
template <class R>
__global__ void k_cg_cond(const Scn<R>* __restrict__ S, int nscn, cudaGraphConditionalHandle handle, int* loopCount,
                          int cap, ActiveTables t, int setCond) {
    bool active = false;
    for (int s = threadIdx.x; s < nscn; s += blockDim.x) active |= S[s].sv[SV_DONE] == 0;
    int any = __syncthreads_or(active);
    buildActive(S, t);
    if (threadIdx.x == 0 && setCond) {
        int lc = ++(*loopCount);
        cudaGraphSetConditional(handle, (any && lc <= cap) ? 1u : 0u);
    }
}

#undef PHX_TILES_BEGIN
#undef PHX_TILES_END
}  // namespace phx
