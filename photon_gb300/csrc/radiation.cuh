// Radiation trace of Photon's room-scale radiation model
// (Solver::traceRadiation, src/sim/radiation.cpp:181-319) over the gas fields
// resident on the device.
//
// Four wavelength bands, 32 golden-spiral directions, an Amanatides-Woo march
// from every radiating surface element through the cells until the ray leaves
// the domain, meets a wall or a blocked cell, runs 8 m, or becomes opaque in
// every band. Everything is relative to ambient, as in the reference.
//
// GB300 mapping:
// * a warp per element (lane = direction: the reference's 32 directions are
//   one warp) computes the element's emission and weights and lists the
//   directions it emits into; a persistent march kernel then hands rays to
//   lanes as they free up, so lanes neither idle on directions an element
//   does not emit into nor wait for the longest ray of their warp; each
//   element's absorbed power is its rays' results summed in direction order,
//   as the reference sums them;
// * per-cell absorption coefficient and source function of the four bands are
//   computed once per trace into one interleaved record per cell (32 B FP32,
//   64 B FP64), so a ray step gathers one record;
// * the band powers a ray ends on (an intact wall seen from either side, a
//   blocked cell's solid temperature) are tabulated before the march, so a
//   ray's end costs a table read instead of the Planck series;
// * gas cells gain their rays' contributions by atomic adds in the trace's
//   precision.
// The FP64 instantiation evaluates every expression in the reference's order
// (the FP64 engine is compiled without fused multiply-add).
#pragma once
#include "phx_dev.cuh"

namespace phx {

constexpr int RAD_NB = 4, RAD_DIRS = 32, RAD_WARPS = 8;

// the reference's PI is the literal 3.14159265 (src/sim/radiation.cpp:44)
template <class R> struct RadPi;
template <> struct RadPi<double> { static constexpr double v = 3.14159265; };
template <> struct RadPi<float> { static constexpr float v = 3.14159265f; };

template <class R>
struct RadConst {
    R dir[RAD_DIRS][3];
    R f0[RAD_NB];       // band fractions of ambient
    R fFlame[RAD_NB];   // band fractions of the sub-grid flame (T_FLAME_RAD 1400 K)
    R dW;               // solid angle per direction
};

template <class R>
struct __align__(sizeof(R) * 8) RadCell {
    R kap[RAD_NB];   // 1/m; blocked cells: unused
    R src[RAD_NB];   // W/m2/sr; blocked cells: the band intensity a ray ending there sees
};

__device__ __forceinline__ double radExp(double x) { return exp(x); }
__device__ __forceinline__ float radExp(float x) { return expf(x); }
__device__ __forceinline__ double radSqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float radSqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double radFloor(double x) { return floor(x); }
__device__ __forceinline__ float radFloor(float x) { return floorf(x); }

// fraction of blackbody emission below lambda*T (um K): Chang & Rhee series
// (src/sim/radiation.cpp:54-63)
template <class R>
__device__ R radPlanckBelow(R lambdaT) {
    if (lambdaT <= 0) return 0;
    if (lambdaT > (R)1e8) return 1;
    const R PI = RadPi<R>::v;
    R x = (R)14388.0 / lambdaT, s = 0;
#pragma unroll 1
    for (int n = 1; n <= 12; ++n) {
        R xn = x * n, dn = (R)n;
        s += radExp(-xn) / n * (x * x * x + 3 * x * x / n + 6 * x / (dn * n) + 6 / (dn * n * n));
    }
    R v = (R)1.0 - (R)15.0 / (PI * PI * PI * PI) * s;
    return v < 0 ? (R)0 : v > 1 ? (R)1 : v;
}

template <class R>
__device__ __forceinline__ R radEdge(int b) {   // band edges, um (:46)
    return b == 1 ? (R)2.7 : b == 2 ? (R)8.0 : (R)14.0;
}

// band fractions (:64-71)
template <class R>
__device__ void radBandFractions(R T, R f[RAD_NB]) {
    R prev = 0;
#pragma unroll
    for (int b = 0; b < RAD_NB; ++b) {
        R up = b == RAD_NB - 1 ? (R)1 : radPlanckBelow<R>(radEdge<R>(b + 1) * T);
        f[b] = up - prev;
        prev = up;
    }
}

// band emissive power relative to ambient, W/m2 (:73-81), from the band fractions f
template <class R>
__device__ __forceinline__ R radPower(const RadConst<R>& k, const R f[RAD_NB], R T, int b) {
    const R a = T * T, a0 = (R)K_T0 * (R)K_T0;
    return (R)5.670374e-8 * (f[b] * a * a - k.f0[b] * a0 * a0);
}

// directions and band tables (:84-96, 185-192); one warp
template <class R>
__global__ void k_rad_setup(RadConst<R>* k) {
    const int i = threadIdx.x;
    const R PI = RadPi<R>::v;
    if (i < RAD_DIRS) {
        const R ga = PI * ((R)3.0 - radSqrt((R)5.0));
        R z = (R)1.0 - (R)2.0 * (i + (R)0.5) / RAD_DIRS;
        R r = radSqrt(mx((R)0, 1 - z * z));
        R ang = ga * i;
        k->dir[i][0] = r * (R)cos((double)ang);
        k->dir[i][1] = r * (R)sin((double)ang);
        k->dir[i][2] = z;
    }
    if (i == 0) {
        radBandFractions<R>((R)K_T0, k->f0);
        radBandFractions<R>((R)1400.0, k->fFlame);
        k->dW = (R)4.0 * PI / RAD_DIRS;
    }
}

// end-of-ray band intensities of every wall, seen from below (0-3) and above (4-7)
template <class R>
__global__ void k_rad_walls(const phx_rad_wall* __restrict__ wl, int nW, int NX, int NY, int* __restrict__ wallOf,
                            R* __restrict__ wallI, const RadConst<R>* __restrict__ kc) {
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= nW) return;
    const phx_rad_wall x = wl[w];
    wallOf[(x.axis == 0 ? 0 : x.axis == 1 ? NX : NX + NY) + x.face] = w;
    const R PI = RadPi<R>::v;
    R f[RAD_NB];
#pragma unroll
    for (int side = 0; side < 2; ++side) {
        const R T = (R)(side == 0 ? x.t_lower : x.t_upper);
        radBandFractions<R>(T, f);
#pragma unroll
        for (int q = 0; q < RAD_NB; ++q) wallI[8 * w + 4 * side + q] = radPower<R>(*kc, f, T, q) * ((R)0.9 / PI);
    }
}

// per-cell absorption and source of the four bands (:193-222); flags bit 0
// blocked, bit 1 flame cell
template <class R>
__global__ void k_rad_cells(const Scn<R>* __restrict__ S, int s, const double* __restrict__ solidT,
                            RadCell<R>* __restrict__ cells, uint8_t* __restrict__ flags,
                            const RadConst<R>* __restrict__ kc) {
    const Scn<R>& g = S[s];
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.N) return;
    const R PI = RadPi<R>::v;
    R f[RAD_NB];
    RadCell<R> o;
    if (g.blocked[c]) {
        const R T = solidT ? (R)solidT[c] : (R)K_T0;
        radBandFractions<R>(T, f);
#pragma unroll
        for (int q = 0; q < RAD_NB; ++q) { o.kap[q] = 0; o.src[q] = radPower<R>(*kc, f, T, q) * ((R)0.9 / PI); }
        cells[c] = o;
        flags[c] = 1;
        return;
    }
    const R T = tAbs(g.sc[0][c]), Ys = g.sc[3][c], Yc = g.sc[6][c], Yw = g.sc[7][c], Pb = g.Pb[c], hrr = g.hrr[c];
    const R rho = Pb / ((R)K_RS * T);
    const R fv = rho * Ys / (R)1800.0;
    const R pg = (Yw * (R)28.96 / (R)18.02 + Yc * (R)28.96 / (R)44.01) * Pb / (R)K_P0;
    radBandFractions<R>(T, f);
    const R jfTot = hrr > 0 ? (R)K_CHI_R * hrr / ((R)4.0 * PI) : (R)0;
    const R lam[RAD_NB] = {(R)1.5, (R)4.5, (R)11.0, (R)25.0};
    const R kg[RAD_NB] = {(R)0.05, (R)3.0, (R)0.1, (R)6.0};
    R k[RAD_NB], Eb[RAD_NB], jTot = 0;
#pragma unroll
    for (int q = 0; q < RAD_NB; ++q) {
        Eb[q] = radPower<R>(*kc, f, T, q);
        k[q] = (R)5.5 * fv / (lam[q] * (R)1e-6) + kg[q] * pg + (R)1e-4;
        jTot += k[q] * Eb[q] / PI;
    }
    const bool fl = jfTot > jTot;
#pragma unroll
    for (int q = 0; q < RAD_NB; ++q) {
        const R j = fl ? jfTot * kc->fFlame[q] : k[q] * Eb[q] / PI;
        o.kap[q] = k[q];
        o.src[q] = j / k[q];
    }
    cells[c] = o;
    flags[c] = fl ? 2 : 0;
}

// Per element (one warp, lane = direction; :225-248): the element's own
// emission in each band, the hemisphere normalisation summed in direction
// order, and each direction's weight w (0 for a direction the element does
// not emit into or an origin outside the grid). The directions with w > 0
// are appended to the ray list (slot = 32 e + d); every slot's result is
// cleared.
template <class R>
__global__ void __launch_bounds__(RAD_WARPS * 32)
k_rad_elems(const Scn<R>* __restrict__ S, int s, const phx_rad_elem* __restrict__ els, int nE,
            const RadConst<R>* __restrict__ kc, R* __restrict__ elemIs, R* __restrict__ rayW,
            R* __restrict__ rayVal, int* __restrict__ rays, int* __restrict__ counters) {
    const int lane = threadIdx.x & 31;
    const int e = blockIdx.x * RAD_WARPS + (threadIdx.x >> 5);
    if (e >= nE) return;   // warp-uniform
    const Scn<R>& g = S[s];
    const R PI = RadPi<R>::v;
    const phx_rad_elem& el = els[e];
    const R eps = (R)el.emissivity, temp = (R)el.temperature, area = (R)el.area;
    const bool sphere = el.sphere != 0;
    const R n0 = (R)el.n[0], n1 = (R)el.n[1], n2 = (R)el.n[2];
    const R dW = kc->dW;
    // own emission, relative to ambient: lanes 0-2 evaluate the band edges
    R up = 0;
    if (lane < 3) up = radPlanckBelow<R>(radEdge<R>(lane + 1) * temp);
    const R u0 = __shfl_sync(0xffffffffu, up, 0), u1 = __shfl_sync(0xffffffffu, up, 1),
            u2 = __shfl_sync(0xffffffffu, up, 2);
    if (lane < RAD_NB) {
        const R f[RAD_NB] = {u0 - (R)0, u1 - u0, u2 - u1, (R)1 - u2};
        R Is = radPower<R>(*kc, f, temp, lane);
        Is *= eps / PI;
        elemIs[(size_t)e * RAD_NB + lane] = Is;
    }
    // hemisphere weights normalised so that sum(cos dW) = pi, in direction order
    R wsum = 0;
    if (!sphere) {
#pragma unroll 4
        for (int d = 0; d < RAD_DIRS; ++d) {
            const R cs = kc->dir[d][0] * n0 + kc->dir[d][1] * n1 + kc->dir[d][2] * n2;
            if (cs > 0) wsum += cs * dW;
        }
    }
    const R norm = sphere ? (R)1 : (wsum > 0 ? PI / wsum : (R)0);
    const R dvx = kc->dir[lane][0], dvy = kc->dir[lane][1], dvz = kc->dir[lane][2];
    bool active = true;
    R w = 0;
    if (sphere) w = dW * (R)0.25 * area;
    else {
        const R cs = dvx * n0 + dvy * n1 + dvz * n2;
        if (cs <= 0) active = false;
        else w = cs * dW * norm * area;
    }
    const R px = ((R)el.o[0] - (R)g.ox) / (R)g.dx, py = ((R)el.o[1] - (R)g.oy) / (R)g.dx,
            pz = ((R)el.o[2] - (R)g.oz) / (R)g.dx;
    const int ci = (int)radFloor(px), cj = (int)radFloor(py), ck = (int)radFloor(pz);
    if (ci < 0 || cj < 0 || ck < 0 || ci >= g.nx || cj >= g.ny || ck >= g.nz) active = false;
    const size_t slot = (size_t)e * RAD_DIRS + lane;
    rayW[slot] = active ? w : (R)0;
    rayVal[slot] = 0;
    const unsigned mask = __ballot_sync(0xffffffffu, active);
    int base = 0;
    if (lane == 0 && mask) base = atomicAdd(counters, __popc(mask));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (active) rays[base + __popc(mask & ((1u << lane) - 1u))] = (int)slot;
}

// The march (:249-306), persistent: every lane takes the next ray of the list
// as soon as its own ray ends (a warp-aggregated atomic hands out rays), so
// lanes do not idle behind the longest ray of their warp. A ray's result
// eps w It lands in its slot; gas cells gain by atomic adds.
template <class R>
__global__ void __launch_bounds__(256)
k_rad_march(const Scn<R>* __restrict__ S, int s, const phx_rad_elem* __restrict__ els,
            const RadCell<R>* __restrict__ cells, const uint8_t* __restrict__ flags, const int* __restrict__ wallOf,
            const R* __restrict__ wallI, const RadConst<R>* __restrict__ kc, const R* __restrict__ elemIs,
            const R* __restrict__ rayW, R* __restrict__ rayVal, const int* __restrict__ rays,
            int* __restrict__ counters, R* __restrict__ radGas) {
    const int lane = threadIdx.x & 31;
    const Scn<R>& g = S[s];
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const int NX = g.NX, NY = g.NY;
    const R dx = (R)g.dx;
    const int nRays = counters[0];
    const R tEnd = (R)8.0 / dx;
    int slot = -1;        // ray in flight; -1 none, -2 the list is exhausted
    int ci = 0, cj = 0, ck = 0, c = 0, skip = -1, sx = 0, sy = 0, sz = 0;
    R tMx = 0, tMy = 0, tMz = 0, tDx = 0, tDy = 0, tDz = 0, t = 0, w = 0, eps = 0;
    R tau[RAD_NB], I[RAD_NB], Is[RAD_NB];
    for (;;) {
        const bool need = slot == -1;
        const unsigned mNeed = __ballot_sync(0xffffffffu, need);
        if (mNeed) {
            const int leader = __ffs(mNeed) - 1;
            int base = 0;
            if (lane == leader) base = atomicAdd(counters + 1, __popc(mNeed));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (need) {
                const int k = base + __popc(mNeed & ((1u << lane) - 1u));
                if (k >= nRays) slot = -2;
                else {
                    slot = rays[k];
                    const int e = slot >> 5, d = slot & 31;
                    const phx_rad_elem& el = els[e];
                    eps = (R)el.emissivity;
                    w = rayW[slot];
#pragma unroll
                    for (int q = 0; q < RAD_NB; ++q) { Is[q] = elemIs[(size_t)e * RAD_NB + q]; tau[q] = 1; I[q] = 0; }
                    const R dvx = kc->dir[d][0], dvy = kc->dir[d][1], dvz = kc->dir[d][2];
                    const R px = ((R)el.o[0] - (R)g.ox) / dx, py = ((R)el.o[1] - (R)g.oy) / dx,
                            pz = ((R)el.o[2] - (R)g.oz) / dx;
                    ci = (int)radFloor(px); cj = (int)radFloor(py); ck = (int)radFloor(pz);
                    if (dvx > (R)1e-9) { sx = 1; tMx = (ci + 1 - px) / dvx; tDx = 1 / dvx; }
                    else if (dvx < (R)-1e-9) { sx = -1; tMx = (px - ci) / -dvx; tDx = -1 / dvx; }
                    else { sx = 0; tMx = (R)1e30; tDx = (R)1e30; }
                    if (dvy > (R)1e-9) { sy = 1; tMy = (cj + 1 - py) / dvy; tDy = 1 / dvy; }
                    else if (dvy < (R)-1e-9) { sy = -1; tMy = (py - cj) / -dvy; tDy = -1 / dvy; }
                    else { sy = 0; tMy = (R)1e30; tDy = (R)1e30; }
                    if (dvz > (R)1e-9) { sz = 1; tMz = (ck + 1 - pz) / dvz; tDz = 1 / dvz; }
                    else if (dvz < (R)-1e-9) { sz = -1; tMz = (pz - ck) / -dvz; tDz = -1 / dvz; }
                    else { sz = 0; tMz = (R)1e30; tDz = (R)1e30; }
                    t = 0;
                    c = ci + nx * (cj + ny * ck);
                    skip = el.skip_own_cell ? c : -1;
                }
            }
        }
        if (__ballot_sync(0xffffffffu, slot >= 0) == 0) break;   // every lane exhausted
        if (slot < 0) continue;
        // advance this lane's ray by up to 16 cells
        bool ended = false;
        R Iend[RAD_NB] = {0, 0, 0, 0};
        for (int it = 0; it < 16; ++it) {
            const int a = tMx < tMy ? (tMx < tMz ? 0 : 2) : (tMy < tMz ? 1 : 2);
            const R tMa = a == 0 ? tMx : a == 1 ? tMy : tMz;
            const R tn = tEnd < tMa ? tEnd : tMa;
            const R ds = (tn - t) * dx;
            const uint8_t fl = flags[c];
            if (ds > 0 && !(fl & 1) && c != skip) {
                const RadCell<R> cell = cells[c];
                const bool flame = (fl & 2) != 0;
                R gsum = 0;
#pragma unroll
                for (int q = 0; q < RAD_NB; ++q) {
                    const R x = cell.kap[q] * ds;
                    const R att = x < (R)1e-3 ? x * (1 - (R)0.5 * x) : (R)1.0 - radExp(-x);
                    const R fromCell = tau[q] * cell.src[q] * att;
                    I[q] += fromCell;
                    gsum += Is[q] * tau[q] * att - (flame ? (R)0 : eps * fromCell);
                    tau[q] *= (R)1.0 - att;
                }
                atomicAdd(radGas + c, w * gsum);
            }
            t = tn;
            if (t >= tEnd || (tau[0] < (R)1e-3 && tau[1] < (R)1e-3 && tau[2] < (R)1e-3 && tau[3] < (R)1e-3)) {
                ended = true;
                break;
            }
            // the face crossed next: an intact wall ends the ray with its surface seen from c
            const int st = a == 0 ? sx : a == 1 ? sy : sz;
            const int upf = st > 0 ? 1 : 0;
            const int f = a == 0 ? (ci + upf) + (nx + 1) * (cj + ny * ck)
                        : a == 1 ? NX + ci + nx * ((cj + upf) + (ny + 1) * ck)
                                 : NX + NY + ci + nx * (cj + ny * (ck + upf));
            const int wi = wallOf[f];
            if (wi >= 0) {
#pragma unroll
                for (int q = 0; q < RAD_NB; ++q) Iend[q] = wallI[8 * wi + (upf ? 0 : 4) + q];
                ended = true;
                break;
            }
            bool out;
            if (a == 0) { ci += sx; out = ci < 0 || ci >= nx; }
            else if (a == 1) { cj += sy; out = cj < 0 || cj >= ny; }
            else { ck += sz; out = ck < 0 || ck >= nz; }
            if (out) { ended = true; break; }
            const int nb = ci + nx * (cj + ny * ck);
            if (flags[nb] & 1) {
                const RadCell<R> cell = cells[nb];
#pragma unroll
                for (int q = 0; q < RAD_NB; ++q) Iend[q] = cell.src[q];
                ended = true;
                break;
            }
            c = nb;
            if (a == 0) tMx += tDx; else if (a == 1) tMy += tDy; else tMz += tDz;
        }
        if (ended) {
            R It = 0;
#pragma unroll
            for (int q = 0; q < RAD_NB; ++q) It += I[q] + tau[q] * Iend[q];
            rayVal[slot] = eps * w * It;
            slot = -1;
        }
    }
}

// absorbed power of each element: its directions' results summed in direction
// order (:305, directions it does not emit into hold 0)
template <class R>
__global__ void k_rad_absorbed(const R* __restrict__ rayVal, int nE, double* __restrict__ radAbs) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nE) return;
    const R* v = rayVal + (size_t)e * RAD_DIRS;
    R acc = 0;
#pragma unroll
    for (int d = 0; d < RAD_DIRS; ++d) acc += v[d];
    radAbs[e] = (double)acc;
}

}  // namespace phx
