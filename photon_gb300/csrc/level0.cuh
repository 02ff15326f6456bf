// Level-0 pressure kernels of the mixed path: the 7-point structured grid of
// the multigrid V-cycle and of q = A d, with the matrix coefficients coded in
// one byte per cell.
//
// Coefficient codes. On the grids Photon discretizes, the level-0 matrix
// coefficients (a0x, a0y, a0z: open fractions of a cell's six faces) are 0 or
// 1 nearly everywhere, and the diagonal is their sum. A cell's code holds, in
// bits 0-5, which of its faces (x-, x+, y-, y+, z-, z+) have a coefficient of
// exactly 1; its diagonal is then the number of those bits. An interior face
// couples the cell to its neighbour; an open domain-boundary face adds to the
// diagonal only. A cell with any other coefficient, or a diagonal that is not
// that count, gets bit 6 ("general") and its coefficients are read from the
// arrays as before. The host builds and
// checks every code. Multiplying by a coefficient of 1 is exact and adding a
// zero term changes nothing, so a coded cell computes exactly what the array
// form computes, in the same order. A pass then streams 1 byte per cell of
// matrix data instead of 16 (four FP32 arrays).
//
// Tiles. A CTA takes a row-block tile (tj whole rows by RB_KZ planes, the
// tiles of the row-block kernels of the FP64 path) and marches up its planes.
// For plane k+1 every thread stages, into a 4-plane ring in shared memory,
// the value the stencil needs at each cell of the tile's rows and their two
// halo rows (d = z + beta d for q = A d; the red value r / diag for the
// pre-smoothing; z plus the prolongated coarse correction for the black
// sweep; z for the residual and the red sweep) together with the cell's code;
// one barrier later it computes plane k from the ring. Each value is formed
// once per cell and read by up to seven stencils; each array is read from HBM
// once per pass. Plain coalesced loads with many CTAs per SM keep enough bytes
// in flight; no thread waits on another except at the one barrier per plane.
#pragma once
#include "rowblock.cuh"

namespace phx {

constexpr int L0_THREADS = 256;
constexpr unsigned char CODE_GENERAL = 64;

// x-, x+, y-, y+, z-, z+ faces of a cell with coefficient 1; bit 6: read the arrays
__device__ __forceinline__ int codeDiagCount(unsigned code) { return __popc(code & 63u); }

// shared-memory layout of a level-0 launch over a batch: the ring planes hold
// (tj + 2) rows of the widest plane of the batch
struct L0Shape {
    int plane;      // elements per ring plane (max over the batch of (tj + 2) nx)
    int own;        // elements of the tile's own rows in one plane (max tj nx)
};
// staged elements of a plane per thread (the registers of the prefetch):
// planes of up to L0_PF * L0_THREADS elements
constexpr int L0_PF = 6;
constexpr int L0_MAX_PLANE = L0_PF * 256;

enum { L0_APPLY = 0, L0_PRE, L0_RES, L0_BLACK, L0_RED };

// rings of a pass: V (the staged values) and C (the codes) always; W (r) for
// the residual and the red sweep; G (aggregates) for the residual, which also
// keeps the residuals and aggregates of two planes for the restriction
__host__ __device__ inline size_t l0Smem(const L0Shape& sh, int mode) {
    const size_t f = (size_t)roundUp(sh.plane * 4, 16), cbytes = (size_t)roundUp(sh.plane, 16);
    size_t b = 4 * f + 4 * cbytes;
    if (mode == 2 || mode == 4) b += 4 * f;                                      // W
    if (mode == 2) b += 4 * f + 4 * (size_t)roundUp(sh.own * 4, 16);            // G, RA RB GA GB
    return b;
}


// the general-cell form of the stencil: coefficients and diagonal from the arrays
struct L0Coef {
    float dg, xm, xp, ym, yp, zm, zp;
};
__device__ __forceinline__ L0Coef l0General(const Scn<float>& g, int i, int j, int k) {
    const int nx = g.nx, ny = g.ny;
    const long long c = (long long)k * nx * ny + (long long)j * nx + i;
    const long long fx = i + (long long)(nx + 1) * (j + (long long)ny * k);
    const long long fy = i + (long long)nx * (j + (long long)(ny + 1) * k);
    L0Coef o;
    o.dg = g.diag[c];
    o.xm = g.a0x[fx];
    o.xp = g.a0x[fx + 1];
    o.ym = g.a0y[fy];
    o.yp = g.a0y[fy + nx];
    o.zm = g.a0z[c];
    o.zp = g.a0z[c + (long long)nx * ny];
    return o;
}

// sacc + the six neighbour terms in the order x-, x+, y-, y+, z-, z+ (sign
// s = +1 for the sweeps and the residual, -1 for q = A d). X0 is the ring
// plane of the cell at index e, Xm / Xp the planes below and above.
template <int SIGN>
__device__ __forceinline__ float l0Terms(float sacc, unsigned code, const L0Coef* gen, const float* X0, const float* Xm,
                                         const float* Xp, int e, int nx, int i, int j, int ny, bool hasM, bool hasP) {
    if (!(code & CODE_GENERAL)) {
        if ((code & 1u) && i > 0) sacc = SIGN > 0 ? sacc + X0[e - 1] : sacc - X0[e - 1];
        if ((code & 2u) && i < nx - 1) sacc = SIGN > 0 ? sacc + X0[e + 1] : sacc - X0[e + 1];
        if ((code & 4u) && j > 0) sacc = SIGN > 0 ? sacc + X0[e - nx] : sacc - X0[e - nx];
        if ((code & 8u) && j < ny - 1) sacc = SIGN > 0 ? sacc + X0[e + nx] : sacc - X0[e + nx];
        if ((code & 16u) && hasM) sacc = SIGN > 0 ? sacc + Xm[e] : sacc - Xm[e];
        if ((code & 32u) && hasP) sacc = SIGN > 0 ? sacc + Xp[e] : sacc - Xp[e];
        return sacc;
    }
    const L0Coef& a = *gen;
    if (SIGN > 0) {
        if (i > 0) sacc += a.xm * X0[e - 1];
        if (i < nx - 1) sacc += a.xp * X0[e + 1];
        if (j > 0) sacc += a.ym * X0[e - nx];
        if (j < ny - 1) sacc += a.yp * X0[e + nx];
        if (hasM) sacc += a.zm * Xm[e];
        if (hasP) sacc += a.zp * Xp[e];
    } else {
        if (i > 0) sacc -= a.xm * X0[e - 1];
        if (i < nx - 1) sacc -= a.xp * X0[e + 1];
        if (j > 0) sacc -= a.ym * X0[e - nx];
        if (j < ny - 1) sacc -= a.yp * X0[e + nx];
        if (hasM) sacc -= a.zm * Xm[e];
        if (hasP) sacc -= a.zp * Xp[e];
    }
    return sacc;
}

// diagonal of a cell: the count of its coupling bits, or the array's value
__device__ __forceinline__ float l0Diag(const Scn<float>& g, unsigned code, long long c) {
    return (code & CODE_GENERAL) ? g.diag[c] : (float)codeDiagCount(code);
}

// One pass over the active row-block tiles of a batch. MODE selects the pass:
//   L0_APPLY  q = A d with d = z + beta d (src/sim/gasphase.cpp:551-570,
//             620-622), d.q (:606-608); alpha in the last CTA of a scenario
//   L0_PRE    pre-smoothing pair from x = 0 (gsColor, pressure_mg.cpp:195-216):
//             red = r / diag, black from its red neighbours; writes z
//   L0_RES    residual (residualGrid, :217-235) restricted to level 1
//             (:285-286): each aggregate's cells summed in ascending order;
//             then level 1's first Jacobi sweep from x = 0
//   L0_BLACK  black sweep after the prolongation (:290-297); red neighbours
//             are z + x1[agg]; writes the black cells of z
//   L0_RED    red sweep with r.z (dotRZ, gasphase.cpp:582-588); the last CTA
//             of a scenario closes the CG iteration (phase 2: a bare V-cycle)
template <int MODE>
__global__ void __launch_bounds__(L0_THREADS, 4) k_l0(const Scn<float>* __restrict__ S, ADom dom, float* const* dbuf,
                                                   L0Shape shape, int phase) {
    using T = float;
    constexpr bool kW = MODE == L0_RES || MODE == L0_RED;
    constexpr bool kG = MODE == L0_RES;
    extern __shared__ __align__(16) unsigned char l0sm[];
    __shared__ int sst_[MAX_BATCH + 1];
    __shared__ double shd[32];
    __shared__ int amLastS;
    const int pl4 = roundUp(shape.plane * 4, 16) / 4, plC = roundUp(shape.plane, 16);
    float* const ringV = reinterpret_cast<float*>(l0sm);
    float* const ringW = ringV + 4 * (size_t)pl4;                                       // kW only
    int* const ringG = reinterpret_cast<int*>(ringW + (kW ? 4 * (size_t)pl4 : 0));       // kG only
    unsigned char* const ringC = reinterpret_cast<unsigned char*>(ringG + (kG ? 4 * (size_t)pl4 : 0));
    const int ownW = roundUp(shape.own * 4, 16) / 4;
    float* const RA = reinterpret_cast<float*>(ringC + 4 * (size_t)plC);   // residuals of the even plane
    float* const RB = RA + ownW;                                           // and of the odd plane
    int* const GA = reinterpret_cast<int*>(RB + ownW);                     // aggregates of the even plane
    int* const GB = GA + ownW;                                             // and of the odd plane
    for (int i = threadIdx.x; i <= dom.nscn; i += blockDim.x) sst_[i] = dom.start[i];
    __syncthreads();
    const int tot = sst_[dom.nscn];
    for (int b = blockIdx.x; b < tot; b += gridDim.x) {
        int s, tile;
        locateShared(sst_, dom.nscn, b, s, tile);
        const Scn<float>& g = S[s];
        const RbTile t = rbTile(g, tile, 1);
        const int nx = t.nx, ny = t.ny, nz = t.nz, j0 = t.j0, j1 = t.j1;
        const long long sxy = t.sxy;
        const int ringRa = max(j0 - 1, 0), ringRe = min(j1 + 1, ny);
        const int nStage = (ringRe - ringRa) * nx;          // staged elements of a plane
        const int stOff = (ringRa - (j0 - 1)) * nx;         // ring index of row ringRa (row j0 - 1 is index 0)
        const int rows = j1 - j0, ncell = rows * nx;
        const unsigned magic = divMagic(nx);
        const int it = (int)g.sv[SV_IT];
        const T beta = (T)g.sv[SV_BETA];
        const float* dprev = (MODE == L0_APPLY && it > 0) ? dbuf[2 * s + (it & 1)] : nullptr;
        float* const dnew = MODE == L0_APPLY ? dbuf[2 * s + ((it + 1) & 1)] : nullptr;
        const float* const xc = MODE == L0_BLACK ? g.lv[1].x : nullptr;
        const int* const agg = g.lv[0].agg;
        const unsigned char* const code = g.code0;
        // one plane's staged inputs, held in registers from their loads until
        // the plane enters the ring one iteration later
        float pa[L0_PF], pw[L0_PF];
        int pg[L0_PF];
        unsigned char pc[L0_PF];
        auto load = [&](int k) {
            const long long base = (long long)k * sxy + (long long)ringRa * nx;
#pragma unroll
            for (int u = 0; u < L0_PF; ++u) {
                const int e = threadIdx.x + u * L0_THREADS;
                if (e >= nStage) break;
                const long long c = base + e;
                pc[u] = code[c];
                if constexpr (MODE == L0_APPLY) {
                    pa[u] = g.z[c];
                    if (dprev) pw[u] = dprev[c];
                } else if constexpr (MODE == L0_PRE) {
                    pa[u] = g.r[c];
                } else if constexpr (MODE == L0_BLACK) {
                    const int jr = divBy(e, nx, magic);
                    const int i = e - jr * nx;
                    if (((i + ringRa + jr + k) & 1) == 0) {   // red: z and its aggregate
                        pa[u] = g.z[c];
                        pg[u] = agg[c];
                    } else {                                  // black: r
                        pa[u] = g.r[c];
                        pg[u] = -1;
                    }
                } else {
                    pa[u] = g.z[c];
                    if constexpr (kW) pw[u] = g.r[c];
                    if constexpr (kG) pg[u] = agg[c];
                }
            }
        };
        auto commit = [&](int k) {
            const int sl = k & 3;
            float* V = ringV + (size_t)sl * pl4 + stOff;
            unsigned char* C = ringC + (size_t)sl * plC + stOff;
            const long long base = (long long)k * sxy + (long long)ringRa * nx;
            const bool own = k >= t.k0 && k < t.k1;
#pragma unroll
            for (int u = 0; u < L0_PF; ++u) {
                const int e = threadIdx.x + u * L0_THREADS;
                if (e >= nStage) break;
                const unsigned cd = pc[u];
                C[e] = (unsigned char)cd;
                float v = pa[u];
                if constexpr (MODE == L0_APPLY) {
                    if (dprev) v = v + beta * pw[u];
                    if (own) {
                        const int jr = ringRa + divBy(e, nx, magic);
                        if (jr >= j0 && jr < j1) dnew[base + e] = v;
                    }
                } else if constexpr (MODE == L0_PRE) {
                    const int jr = divBy(e, nx, magic);
                    const int i = e - jr * nx;
                    if (((i + ringRa + jr + k) & 1) == 0) {   // red: its value after the first half sweep
                        const float dg = l0Diag(g, cd, base + e);
                        v = dg <= 0.f ? 0.f : gsDiv(v, dg);
                    }
                } else if constexpr (MODE == L0_BLACK) {
                    if (pg[u] >= 0) v = (float)(v + xc[pg[u]]);   // red: z plus the prolongated correction
                }
                V[e] = v;
                if constexpr (kW) ringW[(size_t)sl * pl4 + stOff + e] = pw[u];
                if constexpr (kG) ringG[(size_t)sl * pl4 + stOff + e] = pg[u];
            }
        };
        using Acc = F2;
        Acc dot{0.f, 0.f};
        __syncthreads();   // the ring of the previous tile is no longer read
        load(t.kLo);
        commit(t.kLo);
        if (t.kLo < t.k0) {
            load(t.k0);
            commit(t.k0);
        }
        bool pending = false;
        if (t.k0 + 1 <= t.kHi) {
            load(t.k0 + 1);
            pending = true;
        }
        for (int kk = t.k0; kk < t.k1; ++kk) {
            if (pending) commit(kk + 1);
            pending = false;
            if (kk + 2 <= t.kHi) {   // in flight during the barrier and this plane's stencils
                load(kk + 2);
                pending = true;
            }
            __syncthreads();
            const int sl = kk & 3;
            const float* X0 = ringV + (size_t)sl * pl4 + nx;                 // row j0 of plane kk
            const float* Xm = ringV + (size_t)((kk + 3) & 3) * pl4 + nx;
            const float* Xp = ringV + (size_t)((kk + 1) & 3) * pl4 + nx;
            const float* W0 = ringW + (size_t)sl * pl4 + nx;
            const int* G0 = ringG + (size_t)sl * pl4 + nx;
            const unsigned char* C0 = ringC + (size_t)sl * plC + nx;
            const bool hasM = kk > 0, hasP = kk < nz - 1;
            const long long cbase = (long long)kk * sxy + (long long)j0 * nx;
            const bool odd = (kk & 1) != 0;
            for (int e = threadIdx.x; e < ncell; e += L0_THREADS) {
                const int jj = divBy(e, nx, magic);
                const int i = e - jj * nx, j = j0 + jj;
                const long long c = cbase + e;
                const unsigned cd = C0[e];
                L0Coef gen;
                if (cd & CODE_GENERAL) gen = l0General(g, i, j, kk);
                const float dg = (cd & CODE_GENERAL) ? gen.dg : (float)codeDiagCount(cd);
                if constexpr (MODE == L0_APPLY) {
                    const float dc = X0[e];
                    if (dg <= 0.f) { g.q[c] = 0.f; continue; }
                    const float sacc = l0Terms<-1>(dg * dc, cd, &gen, X0, Xm, Xp, e, nx, i, j, ny, hasM, hasP);
                    g.q[c] = sacc;
                    dot = accAdd(dot, dotTerm(sacc, dc));
                } else if constexpr (MODE == L0_PRE) {
                    if (((i + j + kk) & 1) == 0) { g.z[c] = X0[e]; continue; }
                    float zc = 0.f;
                    if (dg > 0.f) zc = gsDiv(l0Terms<1>(X0[e], cd, &gen, X0, Xm, Xp, e, nx, i, j, ny, hasM, hasP), dg);
                    g.z[c] = zc;
                } else if constexpr (MODE == L0_BLACK) {
                    if (((i + j + kk) & 1) == 0) continue;
                    float zc = 0.f;
                    if (dg > 0.f) zc = gsDiv(l0Terms<1>(X0[e], cd, &gen, X0, Xm, Xp, e, nx, i, j, ny, hasM, hasP), dg);
                    g.z[c] = zc;
                } else if constexpr (MODE == L0_RED) {
                    const float r = W0[e];
                    if (((i + j + kk) & 1) == 0) {
                        float zc = 0.f;
                        if (dg > 0.f) zc = gsDiv(l0Terms<1>(r, cd, &gen, X0, Xm, Xp, e, nx, i, j, ny, hasM, hasP), dg);
                        g.z[c] = zc;
                        dot = accAdd(dot, dotTerm(r, zc));
                    } else {
                        dot = accAdd(dot, dotTerm(r, X0[e]));
                    }
                } else {   // L0_RES
                    const int A = G0[e];
                    float rv = 0.f;
                    if (A >= 0) rv = l0Terms<1>(W0[e] - dg * X0[e], cd, &gen, X0, Xm, Xp, e, nx, i, j, ny, hasM, hasP);
                    (odd ? RB : RA)[e] = rv;
                    (odd ? GB : GA)[e] = A;
                }
            }
            if constexpr (MODE == L0_RES) {
                // 2x2x2 blocks close on odd planes, and on the grid's last plane when nz is odd:
                // each level-1 aggregate lies in one block; its cells are summed in ascending
                // cell order, the order of the reference's scatter
                if (odd || kk == nz - 1) {
                    __syncthreads();
                    float* const cb = g.lv[1].b;
                    float* const y1 = g.nLevels > 2 ? g.lv[1].y : nullptr;
                    const float* const d1 = g.lv[1].diag;
                    const int hx = (nx + 1) >> 1, hy = (rows + 1) >> 1, nblk = hx * hy;
                    const unsigned magicHx = divMagic(hx);
                    for (int q = threadIdx.x; q < nblk; q += L0_THREADS) {
                        const int by = divBy(q, hx, magicHx), bx = q - by * hx;
                        int ag[8];
                        float rv[8];
#pragma unroll
                        for (int m = 0; m < 8; ++m) {
                            const int di = m & 1, dj = (m >> 1) & 1, dk = m >> 2;
                            const int i = 2 * bx + di, jj = 2 * by + dj;
                            const bool in = i < nx && jj < rows && (odd || dk == 0);
                            const int e = jj * nx + i;
                            const bool even = !odd || dk == 0;   // the even plane (or a lone last plane)
                            ag[m] = in ? (even ? GA[e] : GB[e]) : -1;
                            rv[m] = in ? (even ? RA[e] : RB[e]) : 0.f;
                        }
#pragma unroll
                        for (int m = 0; m < 8; ++m) {
                            const int a = ag[m];
                            bool first = a >= 0;
#pragma unroll
                            for (int p = 0; p < m; ++p) first = first && ag[p] != a;
                            if (!first) continue;
                            float acc = 0.f;
#pragma unroll
                            for (int p = m; p < 8; ++p)
                                if (ag[p] == a) acc = acc + rv[p];
                            cb[a] = acc;
                            // level 1's first damped Jacobi sweep from x = 0 (jacobi,
                            // pressure_mg.cpp:237-247), unless level 1 is the coarsest
                            if (y1) {
                                const float dc = d1[a];
                                const float om = (float)OMEGA;
                                y1[a] = dc <= 0.f ? 0.f : scratchRound(g, (1.f - om) * 0.f + om * acc / dc);
                            }
                        }
                    }
                    // RA/GA are rewritten two planes later, after this tile's next barrier
                }
            }
        }
        if constexpr (MODE == L0_APPLY || MODE == L0_RED) {
            if (MODE == L0_RED && phase == 2) continue;
            const int nt = sst_[s + 1] - sst_[s];
            // fixed-order CTA sum, then the last CTA of the scenario sums the CTA partials
            const double v = blockSum(dot, shd);
            double* part = g.part + (size_t)(MODE == L0_APPLY ? PS_DQ : PS_RZ) * g.partStride;
            unsigned* cnt = g.cnt + (MODE == L0_APPLY ? PS_DQ : PS_RZ);
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
                        if (total <= 0) g.sv[SV_DONE] = 1;
                        else g.sv[SV_ALPHA] = g.sv[SV_RZ] / total;
                    } else {
                        closeCgIteration(g, phase, total);
                    }
                }
            }
        }
    }
}

}  // namespace phx
