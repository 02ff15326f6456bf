// Row-block tiles of the level-0 pressure kernels, staged in shared memory by
// the Tensor Memory Accelerator.
//
// A tile is TJ whole rows (all of x) of a scenario's grid times RB_KZ planes
// along z. A CTA marches through the tile's planes from bottom to top. Every
// plane of every array the stencil reads is one contiguous run of HBM (whole
// rows), so it is fetched by a single bulk copy (cp.async.bulk) into a slot of
// a ring of RB_STAGES plane slots and signalled by that slot's mbarrier; the
// copies of the next planes are in flight while the current plane is
// computed. No thread waits on global loads, so the stream rate does not
// depend on occupancy. A bulk copy needs 16-byte aligned ends: the run is
// widened to 16-byte boundaries (the arena pads every array) and the consumer
// indexes a slot relative to the aligned start of the plane's first row.
//
// Every wait on an mbarrier is bounded: past the limit the CTA records an
// error in the context's error word, waits (bounded again) for the copies it
// still has in flight and returns; the host reports the error.
#pragma once
#include <type_traits>

#include "pressure_kernels.cuh"

namespace phx {

constexpr int RB_KZ = 16;          // planes per tile along z
constexpr long long RB_WAIT_CYCLES = 2000000000LL;   // about one second at the GB300 clock

// rows per tile for a grid of nx cells per row: about 1024 cells per plane of
// a tile on the FP32 path and 512 on the FP64 path (twice the bytes), even
// (2x2x2 restriction blocks never straddle tiles), at least 2, at most ny
// rounded up to even
template <class R>
__host__ __device__ inline int rowBlockRows(int nx, int ny) {
    const int cells = sizeof(R) == 8 ? 512 : 1024;
    int tj = (cells / (nx > 0 ? nx : 1)) & ~1;
    if (tj < 2) tj = 2;
    const int cap = ny + (ny & 1);
    return tj < cap ? tj : cap;
}

// ---- PTX wrappers: mbarrier and the bulk global -> shared copy -------------------
__device__ __forceinline__ unsigned smemAddr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbarInit(uint64_t* b, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smemAddr(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void fenceBarrierInit() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void mbarArriveExpectTx(uint64_t* b, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smemAddr(b)), "r"(bytes) : "memory");
}
// try_wait suspends the thread until the phase completes or the hint (ns)
// runs out, so a waiting warp takes no issue slots from the working ones
__device__ __forceinline__ bool mbarTryWait(uint64_t* b, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smemAddr(b)), "r"(parity), "r"(20000u)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ void bulkLoad(void* dst, const void* src, unsigned bytes, uint64_t* b) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smemAddr(dst)),
                 "l"(src), "r"(bytes), "r"(smemAddr(b))
                 : "memory");
}

// bounded wait for the phase of the given parity; false on time-out. Between
// polls the warp sleeps for backoffNs so that a waiting warp (the producer is
// usually ahead of the consumers) does not take issue slots from working ones.
__device__ __forceinline__ bool mbarWaitBounded(uint64_t* b, unsigned parity, unsigned backoffNs = 0) {
    if (mbarTryWait(b, parity)) return true;
    const long long t0 = clock64();
    while (!mbarTryWait(b, parity)) {
        if (clock64() - t0 > RB_WAIT_CYCLES) return false;
        if (backoffNs) __nanosleep(backoffNs);
    }
    return true;
}


// One staged array of a plane slot: rows [rowLo, rowLo + rows) of plane k of
// an array with `pitch` elements per row and `plane` elements per plane, at
// element offset `off` of the slot. The slot holds element gidx at index
// off + gidx - G0(k), G0(k) = the 16-byte aligned start of row rowLo.
struct StageDesc {
    const char* src;
    long long plane;             // elements per plane
    int pitch;                   // elements per row
    int rowLo, rows;             // nominal rows of the slot (rowLo may be negative at the grid's edge)
    int rowMin, rowMax;          // rows that exist: [rowMin, rowMax)
    int off;                     // element offset of the array in the slot
};

__host__ __device__ inline long long floorTo(long long v, int m) { return v >= 0 ? v / m * m : -((-v + m - 1) / m) * m; }
__host__ __device__ inline long long ceilTo(long long v, int m) { return floorTo(v + m - 1, m); }
__host__ __device__ inline int roundUp(int v, int m) { return (v + m - 1) / m * m; }

// slot capacity (elements) of `rows` rows of `pitch` elements, with the
// alignment slack of both ends
template <class R>
__host__ __device__ inline int stageCapacity(int rows, int pitch) {
    constexpr int EPV = 16 / (int)sizeof(R);
    return roundUp(rows * pitch + 2 * EPV, EPV);
}

// slot index of element (row, i) of plane k of a staged array
template <class R>
__device__ __forceinline__ int stageAt(const StageDesc& d, int k, int row, int i) {
    constexpr int EPV = 16 / (int)sizeof(R);
    const long long v = (long long)k * d.plane + (long long)d.rowLo * d.pitch;
    return d.off + (int)(v & (EPV - 1)) + (row - d.rowLo) * d.pitch + i;
}

// total bytes of plane k over the descriptors, then the copies (thread 0)
template <class R>
__device__ __noinline__ void stagePlane(const StageDesc* ds, int n, int k, R* slot, uint64_t* bar) {
    constexpr int EPV = 16 / (int)sizeof(R);
    unsigned total = 0;
    for (int q = 0; q < n; ++q) {
        const StageDesc& d = ds[q];
        const int a = max(d.rowLo, d.rowMin), e = min(d.rowLo + d.rows, d.rowMax);
        if (a >= e || !d.src) continue;
        const long long ga = floorTo((long long)k * d.plane + (long long)a * d.pitch, EPV);
        const long long gb = ceilTo((long long)k * d.plane + (long long)e * d.pitch, EPV);
        total += (unsigned)((gb - ga) * sizeof(R));
    }
    mbarArriveExpectTx(bar, total);
    for (int q = 0; q < n; ++q) {
        const StageDesc& d = ds[q];
        const int a = max(d.rowLo, d.rowMin), e = min(d.rowLo + d.rows, d.rowMax);
        if (a >= e || !d.src) continue;
        const long long g0 = floorTo((long long)k * d.plane + (long long)d.rowLo * d.pitch, EPV);
        const long long ga = floorTo((long long)k * d.plane + (long long)a * d.pitch, EPV);
        const long long gb = ceilTo((long long)k * d.plane + (long long)e * d.pitch, EPV);
        bulkLoad(slot + d.off + (ga - g0), d.src + ga * (long long)sizeof(R), (unsigned)((gb - ga) * sizeof(R)), bar);
    }
}

// shared-memory shape of a launch: one slot stride for every tile of the
// batch (the largest slot of its scenarios), so that planes of consecutive
// tiles of different scenarios never overlap in the ring
struct RbShape {
    int slot;                    // elements per plane slot
    int ring;                    // elements per plane of the d ring (FP64 path)
};

// ---- warp-specialised pipeline -------------------------------------------------
// A CTA of a row-block kernel is RB_CONSUMERS consumer warps plus one producer
// warp. The producer walks the CTA's tiles plane by plane: it waits until the
// slot it refills has been released by every consumer warp (the slot's
// "empty" mbarrier), then its lanes issue the bulk copies of the plane's
// arrays, signalled on the slot's "full" mbarrier. The consumers wait on
// "full", compute, and release a plane once no later step reads it. Consumer
// warps synchronise among themselves with named barrier 1 only, never with
// the producer.
constexpr int RB_CONSUMERS = 8;
constexpr int RB_THREADS = (RB_CONSUMERS + 1) * 32;
constexpr int RB_CTHREADS = RB_CONSUMERS * 32;

__device__ __forceinline__ void mbarArrive(uint64_t* b) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smemAddr(b)) : "memory");
}
__device__ __forceinline__ void consumerSync() { asm volatile("bar.sync 1, %0;" ::"n"(RB_CTHREADS) : "memory"); }
// named barrier of the consumer warps with an OR of a predicate
__device__ __forceinline__ bool consumerSyncOr(bool p) {
    unsigned r;
    asm volatile(
        "{\n\t.reg .pred q, o;\n\t"
        "setp.ne.u32 q, %1, 0;\n\t"
        "bar.red.or.pred o, 1, %2, q;\n\t"
        "selp.u32 %0, 1, 0, o;\n\t}"
        : "=r"(r)
        : "r"((unsigned)p), "n"(RB_CTHREADS)
        : "memory");
    return r != 0;
}

// fixed-order sum over the consumer threads (valid in thread 0)
template <class V>
__device__ __forceinline__ double consumerSum(V v, double* sh) {
    v = warpSum(v);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) reinterpret_cast<V*>(sh)[w] = v;
    consumerSync();
    double t = 0;
    if (w == 0) {
        V x{};
        if (l < RB_CONSUMERS) x = reinterpret_cast<V*>(sh)[l];
        x = warpSum(x);
        if constexpr (sizeof(V) == sizeof(double) && !std::is_same<V, double>::value) t = f2value(x);
        else t = (double)x;
    }
    consumerSync();   // sh is free again
    return t;
}

// lastCtaSum among the consumer threads of a row-block CTA
template <class R, class V>
__device__ bool lastCtaSumC(const Scn<R>& g, int slot, int tile, int ntiles, V vThread, double* total, double* sh,
                            int* amLast) {
    const double v = consumerSum(vThread, sh);
    double* part = g.part + (size_t)slot * g.partStride;
    if (threadIdx.x == 0) {
        part[tile] = v;
        __threadfence();
        const unsigned t = atomicAdd(g.cnt + slot, 1u);
        *amLast = (t == (unsigned)ntiles - 1u);
    }
    consumerSync();
    if (!*amLast) return false;
    __threadfence();
    double acc = 0;
    for (int i = threadIdx.x; i < ntiles; i += RB_CTHREADS) acc += __ldcg(part + i);
    const double tot = consumerSum(acc, sh);
    if (threadIdx.x == 0) {
        *total = tot;
        g.cnt[slot] = 0;
    }
    return true;
}

// geometry of a row-block tile
struct RbTile {
    int nx, ny, nz, j0, j1, k0, k1, kLo, kHi, nPl;
    long long sxy;
};
template <class R>
__device__ __forceinline__ RbTile rbTile(const Scn<R>& g, int tile) {
    RbTile t;
    t.nx = g.nx; t.ny = g.ny; t.nz = g.nz;
    const int jb = tile % g.njb, kb = tile / g.njb;
    t.j0 = jb * g.tj; t.j1 = min(t.j0 + g.tj, t.ny);
    t.k0 = kb * RB_KZ; t.k1 = min(t.k0 + RB_KZ, t.nz);
    t.kLo = max(t.k0 - 1, 0); t.kHi = min(t.k1, t.nz - 1);
    t.nPl = t.kHi - t.kLo + 1;
    t.sxy = (long long)t.nx * t.ny;
    return t;
}

// Producer warp: stage the planes of every tile of the CTA. Lane q < nd holds
// descriptor q of the current tile, made by desc(lane, g, tile, t, d).
template <class R, int ST, class DescFn>
__device__ void rbProducer(const Scn<R>* __restrict__ S, const int* sst, int nscn, R* sm, int slotStride,
                           uint64_t* full, uint64_t* empty, volatile int* abortFlag, DescFn desc) {
    constexpr int EPV = 16 / (int)sizeof(R);
    const int lane = threadIdx.x & 31;
    const int tot = sst[nscn];
    unsigned seq = 0;
    for (int b = blockIdx.x; b < tot; b += gridDim.x) {
        int s, tile;
        locateShared(sst, nscn, b, s, tile);
        const Scn<R>& g = S[s];
        const RbTile t = rbTile(g, tile);
        StageDesc d{};
        const bool has = desc(lane, s, g, t, d);
        for (int idx = 0; idx < t.nPl; ++idx) {
            const unsigned q = seq + idx;
            const int slot = q % ST;
            bool ok = true;
            if (lane == 0) {
                if (*abortFlag) ok = false;
                else if (q >= (unsigned)ST && !mbarWaitBounded(&empty[slot], ((q / ST) - 1) & 1, 256)) {
                    ok = false;
                    *abortFlag = 1;
                    atomicOr(g.errWord, 2u);
                }
            }
            if (!__shfl_sync(0xffffffffu, ok, 0)) goto drain;
            {
                const int k = t.kLo + idx;
                long long ga = 0, gb = 0, g0 = 0;
                const int a = max(d.rowLo, d.rowMin), e = min(d.rowLo + d.rows, d.rowMax);
                const bool live = has && d.src && a < e;
                if (live) {
                    g0 = floorTo((long long)k * d.plane + (long long)d.rowLo * d.pitch, EPV);
                    ga = floorTo((long long)k * d.plane + (long long)a * d.pitch, EPV);
                    gb = ceilTo((long long)k * d.plane + (long long)e * d.pitch, EPV);
                }
                unsigned bytes = live ? (unsigned)((gb - ga) * sizeof(R)) : 0u;
                unsigned total = bytes;
                for (int o = 16; o > 0; o >>= 1) total += __shfl_xor_sync(0xffffffffu, total, o);
                if (lane == 0) mbarArriveExpectTx(&full[slot], total);
                __syncwarp();
                if (live) bulkLoad(sm + (size_t)slot * slotStride + d.off + (ga - g0), d.src + ga * (long long)sizeof(R), bytes,
                                   &full[slot]);
            }
        }
        seq += t.nPl;
    }
drain:
    // no copy may be in flight when the CTA ends: wait for the last use of every slot
    if (lane == 0)
        for (unsigned q = seq > (unsigned)ST ? seq - ST : 0; q < seq; ++q) mbarWaitBounded(&full[q % ST], (q / ST) & 1);
}

// ---------------------------------------------------------------------------------
// q = A d with d = z + beta d (src/sim/gasphase.cpp:551-570, 620-622) and the
// d.q partial sums (:606-608) on row-block tiles: the same arithmetic as
// k_cg_apply. d is computed once per cell into a 4-plane ring in shared
// memory (rows j0-1 .. j1), then the 7-point stencil reads the ring.
//
// Slot layout: {z, d_prev, diag, a0z, a0x, a0y}; z and d over rows j0-1 .. j1.
template <class R>
struct ApplyLayout {
    static constexpr int ST = 3;
    int cz, cc, cx, cy, slot, ring;
    __host__ __device__ ApplyLayout(int nx, int tj) {
        cz = stageCapacity<R>(tj + 2, nx);
        cc = stageCapacity<R>(tj, nx);
        cx = stageCapacity<R>(tj, nx + 1);
        cy = stageCapacity<R>(tj + 1, nx);
        slot = 2 * cz + 2 * cc + cx + cy;
        ring = roundUp((tj + 2) * nx, 4);
    }
};

template <class R>
inline size_t rbApplySmem(const RbShape& sh) {
    return ((size_t)ApplyLayout<R>::ST * sh.slot + 4 * (size_t)sh.ring) * sizeof(R);
}
template <class R>
inline size_t rbApplySmem(int nx, int ny) {
    const ApplyLayout<R> L(nx, rowBlockRows<R>(nx, ny));
    return rbApplySmem<R>(RbShape{L.slot, L.ring});
}

enum { SA_Z = 0, SA_D, SA_DIAG, SA_AZ, SA_AX, SA_AY, SA_COUNT };

template <class R>
__global__ void __launch_bounds__(RB_THREADS, 2) k_cg_apply_rb(const Scn<R>* __restrict__ S, ADom dom, R* const* dbuf,
                                                               RbShape shape) {
    using T = R;
    using Acc = decltype(dotTerm(T(0), T(0)));
    using LY = ApplyLayout<R>;
    constexpr int ST = LY::ST;
    constexpr int EPV = 16 / (int)sizeof(R);
    extern __shared__ __align__(128) unsigned char smraw[];
    __shared__ uint64_t full[ST], empty[ST];
    __shared__ int sst_[MAX_BATCH + 1];
    __shared__ volatile int abortFlag;
    __shared__ int amLast;
    __shared__ double sh[RB_CONSUMERS];
    for (int i = threadIdx.x; i <= dom.nscn; i += blockDim.x) sst_[i] = dom.start[i];
    if (threadIdx.x == 0) {
        for (int q = 0; q < ST; ++q) {
            mbarInit(&full[q], 1);
            mbarInit(&empty[q], RB_CONSUMERS);
        }
        fenceBarrierInit();
        abortFlag = 0;
    }
    __syncthreads();
    R* const sm = reinterpret_cast<R*>(smraw);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (warp == RB_CONSUMERS) {
        rbProducer<R, ST>(S, sst_, dom.nscn, sm, shape.slot, full, empty, &abortFlag,
                          [&](int ln, int s, const Scn<R>& g, const RbTile& t, StageDesc& d) {
                              const LY L(t.nx, g.tj);
                              const int it = (int)g.sv[SV_IT];
                              const int nx = t.nx, ny = t.ny, j0 = t.j0, tj = g.tj;
                              switch (ln) {
                              case SA_Z: d = StageDesc{(const char*)g.z, t.sxy, nx, j0 - 1, tj + 2, 0, ny, 0}; return true;
                              case SA_D:
                                  d = StageDesc{it > 0 ? (const char*)dbuf[2 * s + (it & 1)] : nullptr, t.sxy, nx, j0 - 1,
                                                tj + 2, 0, ny, L.cz};
                                  return true;
                              case SA_DIAG: d = StageDesc{(const char*)g.diag, t.sxy, nx, j0, tj, 0, ny, 2 * L.cz}; return true;
                              case SA_AZ: d = StageDesc{(const char*)g.a0z, t.sxy, nx, j0, tj, 0, ny, 2 * L.cz + L.cc}; return true;
                              case SA_AX:
                                  d = StageDesc{(const char*)g.a0x, (long long)(nx + 1) * ny, nx + 1, j0, tj, 0, ny,
                                                2 * L.cz + 2 * L.cc};
                                  return true;
                              case SA_AY:
                                  d = StageDesc{(const char*)g.a0y, (long long)nx * (ny + 1), nx, j0, tj + 1, 0, ny + 1,
                                                2 * L.cz + 2 * L.cc + L.cx};
                                  return true;
                              default: return false;
                              }
                          });
        return;
    }
    // ---- consumers --------------------------------------------------------------
    const int tot = sst_[dom.nscn];
    R* const ring = sm + (size_t)ST * shape.slot;
    unsigned seq = 0;
    for (int b = blockIdx.x; b < tot; b += gridDim.x) {
        int s, tile;
        locateShared(sst_, dom.nscn, b, s, tile);
        const Scn<R>& g = S[s];
        const RbTile t = rbTile(g, tile);
        const int nx = t.nx, ny = t.ny, nz = t.nz, j0 = t.j0, kLo = t.kLo, kHi = t.kHi;
        const LY L(nx, g.tj);
        const int it = (int)g.sv[SV_IT];
        const bool useD = it > 0;
        const T beta = (T)g.sv[SV_BETA];
        R* const dnew = dbuf[2 * s + ((it + 1) & 1)];
        R* const q = g.q;
        const int ncell = (t.j1 - j0) * nx;
        // e / nx as umulhi(e, ceil(2^32 / nx)): exact for e, nx < 65536 (nx = 1 apart)
        const unsigned magic = nx == 1 ? 0u : (unsigned)((0x100000000ULL + nx - 1) / nx);
        const int ringRa = max(j0 - 1, 0), ringRe = min(t.j1 + 1, ny);
        // alignment offsets (mod EPV) of the first staged row of plane k: k * plane + row * pitch
        const int mC = (int)(t.sxy & (EPV - 1)), mX = (int)(((long long)(nx + 1) * ny) & (EPV - 1));
        const int mY = (int)(((long long)nx * (ny + 1)) & (EPV - 1));
        const auto offMod = [](int k, int m, int rowTerm) { return ((k & (EPV - 1)) * m + rowTerm) & (EPV - 1); };
        const int rC = (j0 * nx) & (EPV - 1), rCm = ((j0 - 1) * nx) & (EPV - 1);
        const int rX = (j0 * (nx + 1)) & (EPV - 1), rY = rC;
        Acc dot{};
        int waited = 0, released = 0;
        for (int kk = t.k0; kk < t.k1; ++kk) {
            const int ic = kk - kLo;
            for (const int need = min(ic + 2, t.nPl); waited < need; ++waited) {
                if (abortFlag) break;
                const unsigned qn = seq + waited;
                if (!mbarWaitBounded(&full[qn % ST], (qn / ST) & 1, 32)) {
                    abortFlag = 1;
                    atomicOr(g.errWord, 1u);
                }
            }
            // d of the planes entering the ring (rows j0-1 .. j1)
            if (!abortFlag) {
                for (int k = kk == t.k0 ? kLo : kk + 1; k <= min(kk + 1, kHi); ++k) {
                    const R* base = sm + (size_t)((seq + (k - kLo)) % ST) * shape.slot;
                    const int n = (ringRe - ringRa) * nx;
                    const int oz = offMod(k, mC, rCm) + (ringRa - (j0 - 1)) * nx;
                    const R* zs = base + oz;
                    const R* ds = base + L.cz + oz;
                    R* out = ring + (size_t)(k & 3) * shape.ring + (ringRa - (j0 - 1)) * nx;
                    if (useD)
                        for (int e = threadIdx.x; e < n; e += RB_CTHREADS) out[e] = (T)(zs[e] + beta * ds[e]);
                    else
                        for (int e = threadIdx.x; e < n; e += RB_CTHREADS) out[e] = zs[e];
                }
            }
            consumerSync();
            if (!abortFlag) {
                const R* cur = sm + (size_t)((seq + ic) % ST) * shape.slot;
                const R* nxt = kk + 1 <= kHi ? sm + (size_t)((seq + ic + 1) % ST) * shape.slot : cur;
                const int oC = offMod(kk, mC, rC);
                const R* dgp = cur + 2 * L.cz + oC;
                const R* azp = cur + 2 * L.cz + L.cc + oC;
                const R* azn = nxt + 2 * L.cz + L.cc + offMod(kk + 1, mC, rC);
                const R* axp = cur + 2 * L.cz + 2 * L.cc + offMod(kk, mX, rX);
                const R* ayp = cur + 2 * L.cz + 2 * L.cc + L.cx + offMod(kk, mY, rY);
                const R* D0 = ring + (size_t)(kk & 3) * shape.ring + nx;
                const R* Dm = ring + (size_t)((kk + 3) & 3) * shape.ring + nx;
                const R* Dp = ring + (size_t)((kk + 1) & 3) * shape.ring + nx;
                const long long cbase = (long long)kk * t.sxy + (long long)j0 * nx;
                R* const dnp = dnew + cbase;
                R* const qp = q + cbase;
                const bool hasM = kk > 0, hasP = kk < nz - 1;
                for (int e = threadIdx.x; e < ncell; e += RB_CTHREADS) {
                    const int jj = nx == 1 ? e : (int)__umulhi((unsigned)e, magic);
                    const int i = e - jj * nx, j = j0 + jj;
                    const T dc = D0[e];
                    dnp[e] = dc;
                    const T dg = dgp[e];
                    if (dg <= 0) { qp[e] = 0; continue; }
                    const R* ax = axp + e + jj;   // a0x index jj * (nx + 1) + i
                    T sacc = dg * dc;
                    if (i > 0) sacc -= ax[0] * D0[e - 1];
                    if (i < nx - 1) sacc -= ax[1] * D0[e + 1];
                    if (j > 0) sacc -= ayp[e] * D0[e - nx];
                    if (j < ny - 1) sacc -= ayp[e + nx] * D0[e + nx];
                    if (hasM) sacc -= azp[e] * Dm[e];
                    if (hasP) sacc -= azn[e] * Dp[e];
                    qp[e] = sacc;
                    dot = accAdd(dot, dotTerm(sacc, dc));
                }
            }
            // planes up to kk are read by no later step
            __syncwarp();
            if (lane == 0)
                for (; released <= ic; ++released) mbarArrive(&empty[(seq + released) % ST]);
        }
        __syncwarp();
        if (lane == 0)
            for (; released < t.nPl; ++released) mbarArrive(&empty[(seq + released) % ST]);
        seq += t.nPl;
        if (consumerSyncOr(abortFlag)) return;
        double total;
        if (lastCtaSumC(g, PS_DQ, tile, sst_[s + 1] - sst_[s], dot, &total, sh, &amLast) && threadIdx.x == 0) {
            g.sv[SV_DQ] = total;
            if (total <= 0) g.sv[SV_DONE] = 1;
            else g.sv[SV_ALPHA] = g.sv[SV_RZ] / total;
        }
    }
}

}  // namespace phx
