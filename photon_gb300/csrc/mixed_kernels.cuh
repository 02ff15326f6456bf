// Kernels of the mixed-precision pressure solve: an FP64 iterative-refinement
// loop around the FP32 multigrid-preconditioned CG of pressure_kernels.cuh.
//
// The pressure is accumulated in FP64 (p64). Each refinement pass computes the
// residual r = b - A p64 in FP64 from the FP32 right-hand side and the FP32
// matrix coefficients (both exact in FP64), hands it to the FP32 inner CG as
// its right-hand side (iterate e = 0), and adds the inner solution to p64. The
// passes stop when max|r| <= relTol * max|b| in FP64, so the converged pressure
// meets the same relative residual as the FP64 path.
#pragma once
#include "pressure_kernels.cuh"

namespace phx {

// In-loop replacement kernels run for a scenario only when its last iteration
// scheduled a replacement (SV_REPL) and it has not stopped; at the start of the
// solve (inLoop 0) they always run.
template <class R>
__device__ __forceinline__ bool replaceActive(const Scn<R>& g, int inLoop) {
    return inLoop == 0 || (g.sv[SV_REPL] != 0 && g.sv[SV_DONE] == 0);
}

// r = b - A p64 in FP64 -> r (FP32); the FP32 iterate e (kept in p) restarts at 0
template <class R>
__global__ void k_mx_res64(const Scn<R>* __restrict__ S, ADom dom, int inLoop) {
    __shared__ int sst_[MAX_BATCH + 1];
    for (int i_ = threadIdx.x; i_ <= dom.nscn; i_ += blockDim.x) sst_[i_] = dom.start[i_];
    __syncthreads();
    const int tot_ = sst_[dom.nscn];
    for (int b_ = blockIdx.x; b_ < tot_; b_ += gridDim.x) {
        int s_, tile_;
        locateShared(sst_, dom.nscn, b_, s_, tile_);
        const Scn<R>& g = S[s_];
        if (!replaceActive(g, inLoop)) continue;
        do {
    const int nx = g.nx, ny = g.ny, nz = g.nz, sxy = nx * ny;
    const int c = tile_ * TPB + threadIdx.x;
    double rm = 0;
    if (c < g.N) {
        // a coded cell (level0.cuh) has coefficients of exactly 0 or 1 and
        // needs no FP64 multiply per neighbour; the others read the arrays
        const unsigned cd = g.code0 ? g.code0[c] : 64u;
        const bool coded = !(cd & 64u);
        const double dg = coded ? (double)(__popc(cd & 63u) + (cd >> 7)) : (double)g.diag[c];
        double r = 0;
        if (dg > 0) {
            int i, j, k;
            ijkOf(g, 0, c, i, j, k);
            const double* x = g.p64;
            double s = dg * x[c];
            if (coded) {
                if (cd & 1u) s -= x[c - 1];
                if (cd & 2u) s -= x[c + 1];
                if (cd & 4u) s -= x[c - nx];
                if (cd & 8u) s -= x[c + nx];
                if (cd & 16u) s -= x[c - sxy];
                if (cd & 32u) s -= x[c + sxy];
            } else {
                const int fx0 = i + (nx + 1) * (j + ny * k), fy0 = i + nx * (j + (ny + 1) * k);
                if (i > 0) s -= (double)g.a0x[fx0] * x[c - 1];
                if (i < nx - 1) s -= (double)g.a0x[fx0 + 1] * x[c + 1];
                if (j > 0) s -= (double)g.a0y[fy0] * x[c - nx];
                if (j < ny - 1) s -= (double)g.a0y[fy0 + nx] * x[c + nx];
                if (k > 0) s -= (double)g.a0z[c] * x[c - sxy];
                if (k < nz - 1) s -= (double)g.a0z[c + sxy] * x[c + sxy];
            }
            r = (double)g.b[c] - s;
        }
        g.r[c] = (R)r;
        g.p[c] = 0;
        // cells of closed zones get their max after the zone-mean projection
        const int z = g.nClosed > 0 ? g.zone[c] : -1;
        if (!(z >= 0 && !g.zoneOpen[z])) rm = fabs(r);
    }
    blockMaxTo(g.sv + SV_R64MAX, rm);
        } while (0);
    }
}

// Closed zones make A singular (constants are its null space): the residual
// must have zero mean over each closed zone. In FP64 the step's b is
// consistent to rounding; its FP32 copy is not, so the mean of the residual
// over each closed zone is removed (one CTA per closed zone; FP64 sums).
template <class R>
__global__ void k_mx_zone_proj(const Scn<R>* __restrict__ S, ADom dom, int inLoop) {
    __shared__ int sst_[MAX_BATCH + 1];
    for (int i_ = threadIdx.x; i_ <= dom.nscn; i_ += blockDim.x) sst_[i_] = dom.start[i_];
    __syncthreads();
    const int tot_ = sst_[dom.nscn];
    for (int b_ = blockIdx.x; b_ < tot_; b_ += gridDim.x) {
        int s_, tile_;
        locateShared(sst_, dom.nscn, b_, s_, tile_);
        const Scn<R>& g = S[s_];
        if (!replaceActive(g, inLoop)) continue;
        do {
    __shared__ double sh[32];
    __shared__ double meanSh;
    const int zi = tile_;
    const int e0 = g.closedStart[zi], e1 = g.closedStart[zi + 1];
    double acc = 0;
    for (int e = e0 + threadIdx.x; e < e1; e += blockDim.x) acc += (double)g.r[g.closedCells[e]];
    double sum = blockSum(acc, sh);
    if (threadIdx.x == 0) meanSh = e1 > e0 ? sum / (double)(e1 - e0) : 0.0;
    __syncthreads();
    const double mean = meanSh;
    double rm = 0;
    for (int e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
        const int c = g.closedCells[e];
        if (g.diag[c] > 0) {
            const R v = (R)((double)g.r[c] - mean);
            g.r[c] = v;
            rm = fmax(rm, fabs((double)v));
        }
    }
    blockMaxTo(g.sv + SV_R64MAX, rm);
        } while (0);
    }
}

// Closed zones, every CG iteration (mixed path): the FP32 matrix's diagonal is
// not exactly the sum of its off-diagonals, so the recursive residual r and
// the preconditioned residual z pick up a constant per closed zone (the null
// space of the zone's operator) that the FP32 iteration cannot remove. Their
// mean over each closed zone is subtracted (which 0: r after its update,
// 1: z after the V-cycle; FP64 sums, one CTA per closed zone).
template <class R>
__global__ void k_mx_zone_center(const Scn<R>* __restrict__ S, ADom dom, int which) {
    __shared__ int sst_[MAX_BATCH + 1];
    for (int i_ = threadIdx.x; i_ <= dom.nscn; i_ += blockDim.x) sst_[i_] = dom.start[i_];
    __syncthreads();
    const int tot_ = sst_[dom.nscn];
    for (int b_ = blockIdx.x; b_ < tot_; b_ += gridDim.x) {
        int s_, tile_;
        locateShared(sst_, dom.nscn, b_, s_, tile_);
        const Scn<R>& g = S[s_];
        __shared__ double sh[32];
        __shared__ double meanSh;
        R* const a = which == 0 ? g.r : g.z;
        const int e0 = g.closedStart[tile_], e1 = g.closedStart[tile_ + 1];
        double acc = 0;
        for (int e = e0 + threadIdx.x; e < e1; e += blockDim.x) acc += (double)a[g.closedCells[e]];
        const double sum = blockSum(acc, sh);
        if (threadIdx.x == 0) meanSh = e1 > e0 ? sum / (double)(e1 - e0) : 0.0;
        __syncthreads();
        const double mean = meanSh;
        for (int e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
            const int c = g.closedCells[e];
            if (g.diag[c] > 0) a[c] = (R)((double)a[c] - mean);
        }
        __syncthreads();
    }
}

// start of a mixed solve: the initial guess 2 p(n) - p(n-1) when the previous
// step's pressure is known (a linear extrapolation in time), and p(n) kept
// as the next step's p(n-1). The solve stops on the same residual test, so
// only the iteration count depends on the guess.
template <class R>
__global__ void k_mx_extrap(const Scn<R>* __restrict__ S, Dom dom) {
    int s_, tile_;
    locate(dom, blockIdx.x, s_, tile_);
    const Scn<R>& g = S[s_];
    const int c = tile_ * TPB + threadIdx.x;
    if (c >= g.N || !g.p64prev) return;
    const double cur = g.p64[c];
    if (g.extrap && g.sv[SV_HAVEPREV] != 0 && g.diag[c] > 0) g.p64[c] = 2.0 * cur - g.p64prev[c];
    g.p64prev[c] = cur;
}

// p64 += e: fold the FP32 iterate into the FP64 pressure
template <class R>
__global__ void k_mx_update(const Scn<R>* __restrict__ S, ADom dom, int inLoop) {
    __shared__ int sst_[MAX_BATCH + 1];
    for (int i_ = threadIdx.x; i_ <= dom.nscn; i_ += blockDim.x) sst_[i_] = dom.start[i_];
    __syncthreads();
    const int tot_ = sst_[dom.nscn];
    for (int b_ = blockIdx.x; b_ < tot_; b_ += gridDim.x) {
        int s_, tile_;
        locateShared(sst_, dom.nscn, b_, s_, tile_);
        const Scn<R>& g = S[s_];
        if (!replaceActive(g, inLoop)) continue;
        do {
    const int c = tile_ * TPB + threadIdx.x;
    if (c < g.N && g.diag[c] > 0) g.p64[c] += (double)g.p[c];
        } while (0);
    }
}

// end of the solve: p64 += e; p (FP32, read by momentum and the velocity
// correction) = p64
template <class R>
__global__ void k_mx_final(const Scn<R>* __restrict__ S, Dom dom) {
    int s_, tile_;
    locate(dom, blockIdx.x, s_, tile_);
    const Scn<R>& g = S[s_];
    const int c = tile_ * TPB + threadIdx.x;
    if (c >= g.N) return;
    double v = g.p64[c];
    if (g.diag[c] > 0) v += (double)g.p[c];
    g.p64[c] = v;
    g.p[c] = (R)v;
    if (c == 0) g.sv[SV_HAVEPREV] = 1;
}

// simulated time of every scenario into one array (one read-back per batch)
template <class R>
__global__ void k_read_times(const Scn<R>* __restrict__ S, int n, double* out) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < n) out[s] = S[s].sv[SV_TIME];
}

// per-scenario resets of the solve's scalar slots (one thread per scenario):
// which 0: the CG of either path; 2: a bare V-cycle
template <class R>
__global__ void k_reset(const Scn<R>* __restrict__ S, Dom dom, int which) {
    int s_, tile_;
    locate(dom, blockIdx.x, s_, tile_);
    if (threadIdx.x != 0) return;
    double* sv = S[s_].sv;
    sv[SV_DONE] = 0;
    if (which == 2) return;
    sv[SV_IT] = 0;
    sv[SV_RMAX] = 0;
    sv[SV_BMAX] = 0;
    sv[SV_R64MAX] = 0;
    sv[SV_REPL] = 0;
    sv[SV_BREAK] = 0;
}

}  // namespace phx
