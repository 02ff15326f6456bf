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

// r = b - A p64 in FP64; r (FP32) = r, inner iterate e = 0 (kept in p)
template <class R>
__global__ void k_mx_res64(const Scn<R>* __restrict__ S, Dom dom) {
    int s_, tile_;
    locate(dom, blockIdx.x, s_, tile_);
    const Scn<R>& g = S[s_];
    if (g.sv[SV_ODONE] != 0) return;
    const int nx = g.nx, ny = g.ny, nz = g.nz, sxy = nx * ny;
    const int c = tile_ * TPB + threadIdx.x;
    double rm = 0;
    if (c < g.N) {
        const double dg = g.diag[c];
        double r = 0;
        if (dg > 0) {
            const int i = c % nx, j = (c / nx) % ny, k = c / sxy;
            const int fx0 = i + (nx + 1) * (j + ny * k), fy0 = i + nx * (j + (ny + 1) * k);
            const double* x = g.p64;
            double s = dg * x[c];
            if (i > 0) s -= (double)g.a0x[fx0] * x[c - 1];
            if (i < nx - 1) s -= (double)g.a0x[fx0 + 1] * x[c + 1];
            if (j > 0) s -= (double)g.a0y[fy0] * x[c - nx];
            if (j < ny - 1) s -= (double)g.a0y[fy0 + nx] * x[c + nx];
            if (k > 0) s -= (double)g.a0z[c] * x[c - sxy];
            if (k < nz - 1) s -= (double)g.a0z[c + sxy] * x[c + sxy];
            r = (double)g.b[c] - s;
        }
        g.r[c] = (R)r;
        g.p[c] = 0;
        // cells of closed zones get their max after the zone-mean projection
        const int z = g.nClosed > 0 ? g.zone[c] : -1;
        if (!(z >= 0 && !g.zoneOpen[z])) rm = fabs(r);
    }
    blockMaxTo(g.sv + SV_R64MAX, rm);
}

// Closed zones make A singular (constants are its null space): the right-hand
// side of the inner solve must have zero mean over each closed zone. In FP64
// the step's b is consistent to rounding; its FP32 copy is not, so the mean of
// the residual over each closed zone is removed before the inner solve (one
// CTA per closed zone; FP64 sums).
template <class R>
__global__ void k_mx_zone_proj(const Scn<R>* __restrict__ S, Dom dom) {
    int s_, tile_;
    locate(dom, blockIdx.x, s_, tile_);
    const Scn<R>& g = S[s_];
    if (g.sv[SV_ODONE] != 0) return;
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
}

// p64 += e after an inner solve
template <class R>
__global__ void k_mx_update(const Scn<R>* __restrict__ S, Dom dom) {
    int s_, tile_;
    locate(dom, blockIdx.x, s_, tile_);
    const Scn<R>& g = S[s_];
    if (g.sv[SV_ODONE] != 0) return;
    const int c = tile_ * TPB + threadIdx.x;
    if (c < g.N && g.diag[c] > 0) g.p64[c] += (double)g.p[c];
}

// p (FP32, read by momentum and the velocity correction) = p64
template <class R>
__global__ void k_mx_final(const Scn<R>* __restrict__ S, Dom dom) {
    int s_, tile_;
    locate(dom, blockIdx.x, s_, tile_);
    const Scn<R>& g = S[s_];
    const int c = tile_ * TPB + threadIdx.x;
    if (c < g.N) g.p[c] = (R)g.p64[c];
}

// refinement stop test per scenario, then the condition of the refinement
// loop; also readies the inner CG (its stop flag and reference residual).
// The pass counter bounds the loop whatever the flags say.
template <class R>
__global__ void k_mx_outer(const Scn<R>* __restrict__ S, int nscn, cudaGraphConditionalHandle handle, int* loopCount,
                           int cap, int setCond) {
    bool active = false;
    for (int s = threadIdx.x; s < nscn; s += blockDim.x) {
        const Scn<R>& g = S[s];
        double* sv = g.sv;
        if (sv[SV_ODONE] == 0) {
            const double rmax = sv[SV_R64MAX];
            const double rel = sv[SV_BMAX] > 0 ? rmax / sv[SV_BMAX] : 0.0;
            const double res = rmax / sv[SV_INV];
            sv[SV_PREL] = rel;
            sv[SV_PRES] = res;
            sv[SV_ITTOT] += sv[SV_IT];
            sv[SV_OUTER] += 1;
            bool more = rel > g.relTol && res > g.tol && sv[SV_OUTER] <= g.outerMax && rmax > 0;
            if (!more) sv[SV_ODONE] = 1;
            sv[SV_R0MAX] = rmax;
            sv[SV_R64MAX] = 0;
        }
        sv[SV_DONE] = sv[SV_ODONE];   // the inner CG runs for the scenarios still refining
        sv[SV_IT] = 0;
        sv[SV_RMAX] = sv[SV_ODONE] != 0 ? 0.0 : sv[SV_R0MAX];   // max|r| at the inner start
        active |= sv[SV_ODONE] == 0;
    }
    int any = __syncthreads_or(active);
    if (threadIdx.x == 0 && setCond) {
        int lc = ++(*loopCount);
        cudaGraphSetConditional(handle, (any && lc <= cap) ? 1u : 0u);
    }
}

// per-scenario resets of the solve's scalar slots (one thread per scenario):
// which 0: FP64 CG; 1: mixed refinement; 2: a bare V-cycle
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
    if (which == 1) {
        sv[SV_ODONE] = 0;
        sv[SV_OUTER] = 0;
        sv[SV_ITTOT] = 0;
        sv[SV_R64MAX] = 0;
    }
}

}  // namespace phx
