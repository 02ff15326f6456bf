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

// rows per tile for a grid of nx cells per row: about 768 cells per plane of
// a tile on the FP32 path and 384 on the FP64 path (twice the bytes), even
// (2x2x2 restriction blocks never straddle tiles), at least 2, at most ny
// rounded up to even. 768 is the measured best of 512 / 768 / 1024 on the
// 64-scenario batch: the wider planes favour q = A d and the sweeps with a
// ring, the narrower ones let the residual and the prolongated sweep (the
// largest slots) run two CTAs per SM.
template <class R>
__host__ __device__ inline int rowBlockRows(int nx, int ny) {
    const int cells = sizeof(R) == 8 ? 384 : 768;
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

// Self-test of the failure path of a bounded wait: one thread waits, with a
// limit of `limitCycles`, on an mbarrier that nothing arrives on. The wait
// runs out, the kernel records bit 4 in the context's error word and
// returns; no copy is in flight and nothing else waits on it. R is the
// engine's precision (one instance per engine).
template <class R>
__global__ void k_selftest_wait(unsigned* errWord, long long limitCycles) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x != 0) return;
    mbarInit(&bar, 1);
    fenceBarrierInit();
    const long long t0 = clock64();
    bool arrived = false;
    while (!(arrived = mbarTryWait(&bar, 0))) {
        if (clock64() - t0 > limitCycles) break;
        __nanosleep(1000);
    }
    if (!arrived) atomicOr(errWord, 4u);
}

// One staged array of a plane slot: rows [rowLo, rowLo + rows) of plane k of
// an array with `pitch` elements of `esz` bytes per row and `plane` elements
// per plane, at byte `off` of the slot. The slot holds element gidx at byte
// off + (gidx - G0(k)) * esz, G0(k) = the 16-byte aligned start of row rowLo.
struct StageDesc {
    const char* src;
    long long plane;             // elements per plane
    int pitch;                   // elements per row
    int rowLo, rows;             // nominal rows of the slot (rowLo may be negative at the grid's edge)
    int rowMin, rowMax;          // rows that exist: [rowMin, rowMax)
    int off;                     // byte offset of the array in the slot
    int esz;                     // bytes per element (4 or 8)
};

__host__ __device__ inline long long floorTo(long long v, int m) { return v >= 0 ? v / m * m : -((-v + m - 1) / m) * m; }
__host__ __device__ inline long long ceilTo(long long v, int m) { return floorTo(v + m - 1, m); }
__host__ __device__ inline int roundUp(int v, int m) { return (v + m - 1) / m * m; }

// slot bytes of `rows` rows of `pitch` elements of esz bytes, with the
// alignment slack of both ends (a multiple of 16)
__host__ __device__ inline int stageBytes(int rows, int pitch, int esz) { return roundUp(rows * pitch * esz + 32, 16); }

// element offset, within the slot array, of element 0 of row rowLo of plane k:
// (k * plane + rowLo * pitch) mod (16 / esz), from small residues
__device__ __forceinline__ int stageMod(int k, int planeMod, int rowTerm, int epv) {
    return ((k & (epv - 1)) * planeMod + rowTerm) & (epv - 1);
}

// shared-memory shape of a launch: one slot stride for every tile of the
// batch (the largest slot of its scenarios), so that planes of consecutive
// tiles of different scenarios never overlap in the ring
struct RbShape {
    int slot;                    // bytes per plane slot
    int ring;                    // bytes per plane of the consumers' ring
    int st;                      // slots of the staging ring (chosen per launch from the shared-memory budget)
};
constexpr int RB_MAX_ST = 8;

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
        if constexpr (std::is_same<V, F2>::value) t = f2value(x);
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

// geometry of a row-block tile; the staged planes are [kLo, kHi] (the tile's
// planes plus `halo` planes on each side, clipped to the grid)
struct RbTile {
    int nx, ny, nz, j0, j1, k0, k1, kLo, kHi, nPl;
    long long sxy;
};
template <class R>
__device__ __forceinline__ RbTile rbTile(const Scn<R>& g, int tile, int halo = 1) {
    RbTile t;
    t.nx = g.nx; t.ny = g.ny; t.nz = g.nz;
    const int jb = tile % g.njb, kb = tile / g.njb;
    t.j0 = jb * g.tj; t.j1 = min(t.j0 + g.tj, t.ny);
    t.k0 = kb * RB_KZ; t.k1 = min(t.k0 + RB_KZ, t.nz);
    t.kLo = max(t.k0 - halo, 0); t.kHi = min(t.k1 - 1 + halo, t.nz - 1);
    t.nPl = t.kHi - t.kLo + 1;
    t.sxy = (long long)t.nx * t.ny;
    return t;
}

// Producer warp: stage the planes of every tile of the CTA. Lane q holds
// descriptor q of the current tile (desc returns false for unused lanes).
template <class R, class DescFn>
__device__ void rbProducer(const Scn<R>* __restrict__ S, const int* sst, int nscn, char* sm, int slotStride, int ST,
                           int halo, uint64_t* full, uint64_t* empty, volatile int* abortFlag, DescFn desc) {
    const int lane = threadIdx.x & 31;
    const int tot = sst[nscn];
    unsigned seq = 0;
    for (int b = blockIdx.x; b < tot; b += gridDim.x) {
        int s, tile;
        locateShared(sst, nscn, b, s, tile);
        const Scn<R>& g = S[s];
        const RbTile t = rbTile(g, tile, halo);
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
                const int epv = 16 / (d.esz > 0 ? d.esz : 16);
                long long ga = 0, gb = 0, g0 = 0;
                const int a = max(d.rowLo, d.rowMin), e = min(d.rowLo + d.rows, d.rowMax);
                const bool live = has && d.src && a < e;
                if (live) {
                    g0 = floorTo((long long)k * d.plane + (long long)d.rowLo * d.pitch, epv);
                    ga = floorTo((long long)k * d.plane + (long long)a * d.pitch, epv);
                    gb = ceilTo((long long)k * d.plane + (long long)e * d.pitch, epv);
                }
                const unsigned bytes = live ? (unsigned)((gb - ga) * d.esz) : 0u;
                unsigned total = bytes;
                for (int o = 16; o > 0; o >>= 1) total += __shfl_xor_sync(0xffffffffu, total, o);
                if (lane == 0) mbarArriveExpectTx(&full[slot], total);
                __syncwarp();
                if (live)
                    bulkLoad(sm + (size_t)slot * slotStride + d.off + (ga - g0) * d.esz, d.src + ga * d.esz, bytes,
                             &full[slot]);
            }
        }
        seq += t.nPl;
    }
drain:
    // no copy may be in flight when the CTA ends: wait for the last use of every slot
    if (lane == 0)
        for (unsigned q = seq > (unsigned)ST ? seq - ST : 0; q < seq; ++q) mbarWaitBounded(&full[q % ST], (q / ST) & 1, 64);
}

// Consumer side of the slot ring for one tile: planes are waited in order and
// released in order (one arrival per consumer warp).
struct RbPipe {
    uint64_t* full;
    uint64_t* empty;
    volatile int* abortFlag;
    unsigned seq;                // planes of the CTA's earlier tiles
    int nPl, waited, released;
    unsigned ST;                 // slots of the ring
    // wait for planes [waited, idx] (idx clipped to the tile's planes)
    __device__ __forceinline__ void waitThrough(int idx, unsigned* errWord) {
        idx = min(idx, nPl - 1);
        for (; waited <= idx; ++waited) {
            if (*abortFlag) return;
            const unsigned q = seq + waited;
            if (!mbarWaitBounded(&full[q % ST], (q / ST) & 1, 32)) {
                *abortFlag = 1;
                atomicOr(errWord, 1u);
            }
        }
    }
    // release planes [released, idx]
    __device__ __forceinline__ void releaseThrough(int idx) {
        idx = min(idx, nPl - 1);
        __syncwarp();
        if ((threadIdx.x & 31) == 0)
            for (int q = released; q <= idx; ++q) mbarArrive(&empty[(seq + q) % ST]);
        released = max(released, idx + 1);
    }
    __device__ __forceinline__ int slotOf(int idx) const { return (int)((seq + idx) % ST); }
};

// common prologue of a row-block kernel: the active prefix and the barriers
#define PHX_RB_PROLOGUE()                                                     \
    extern __shared__ __align__(128) unsigned char smraw[];                   \
    __shared__ uint64_t full[RB_MAX_ST], empty[RB_MAX_ST];                    \
    __shared__ int sst_[MAX_BATCH + 1];                                       \
    __shared__ volatile int abortFlag;                                        \
    __shared__ int amLast;                                                    \
    __shared__ double sh[RB_CONSUMERS];                                       \
    for (int i_ = threadIdx.x; i_ <= dom.nscn; i_ += blockDim.x)              \
        sst_[i_] = dom.start[i_];                                             \
    if (threadIdx.x == 0) {                                                   \
        for (int q_ = 0; q_ < RB_MAX_ST; ++q_) {                              \
            mbarInit(&full[q_], 1);                                           \
            mbarInit(&empty[q_], RB_CONSUMERS);                               \
        }                                                                     \
        fenceBarrierInit();                                                   \
        abortFlag = 0;                                                        \
    }                                                                         \
    __syncthreads();                                                          \
    char* const sm = reinterpret_cast<char*>(smraw);                          \
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;               \
    (void)amLast; (void)sh; (void)lane;

// e / nx as umulhi(e, ceil(2^32 / nx)): exact for e, nx < 65536 (nx = 1 apart)
__device__ __forceinline__ unsigned divMagic(int nx) { return nx == 1 ? 0u : (unsigned)((0x100000000ULL + nx - 1) / nx); }
__device__ __forceinline__ int divBy(int e, int nx, unsigned magic) { return nx == 1 ? e : (int)__umulhi((unsigned)e, magic); }

// ---------------------------------------------------------------------------------
// q = A d with d = z + beta d (src/sim/gasphase.cpp:551-570, 620-622) and the
// d.q partial sums (:606-608) on row-block tiles: the same arithmetic as
// the reference. d is computed once per cell into a 4-plane ring in shared
// memory (rows j0-1 .. j1), then the 7-point stencil reads the ring.
//
// Slot layout: {z, d_prev, diag, a0z, a0x, a0y}; z and d over rows j0-1 .. j1.
template <class R>
struct ApplyLayout {
    static constexpr int MIN_ST = 3;
    int bz, bc, bx, by, slot, ring;
    __host__ __device__ ApplyLayout(int nx, int tj) {
        bz = stageBytes(tj + 2, nx, sizeof(R));
        bc = stageBytes(tj, nx, sizeof(R));
        bx = stageBytes(tj, nx + 1, sizeof(R));
        by = stageBytes(tj + 1, nx, sizeof(R));
        slot = 2 * bz + 2 * bc + bx + by;
        ring = roundUp((tj + 2) * nx * (int)sizeof(R), 16);
    }
};

// dynamic shared memory of a row-block launch: the staging ring, the
// consumers' 4-plane ring and a kernel's own tail
inline size_t rbSmem(const RbShape& sh, int tail = 0) { return (size_t)sh.st * sh.slot + 4 * (size_t)sh.ring + (size_t)tail; }

enum { SA_Z = 0, SA_D, SA_DIAG, SA_AZ, SA_AX, SA_AY, SA_COUNT };

template <class R>
__global__ void __launch_bounds__(RB_THREADS, 2) k_cg_apply_rb(const Scn<R>* __restrict__ S, ADom dom, R* const* dbuf,
                                                               RbShape shape) {
    using T = R;
    using Acc = decltype(dotTerm(T(0), T(0)));
    using LY = ApplyLayout<R>;
    const int ST = shape.st;
    constexpr int EPV = 16 / (int)sizeof(R);
    constexpr int ES = (int)sizeof(R);
    PHX_RB_PROLOGUE()
    if (warp == RB_CONSUMERS) {
        rbProducer<R>(S, sst_, dom.nscn, sm, shape.slot, ST, 1, full, empty, &abortFlag,
                          [&](int ln, int s, const Scn<R>& g, const RbTile& t, StageDesc& d) {
                              const LY L(t.nx, g.tj);
                              const int it = (int)g.sv[SV_IT];
                              const int nx = t.nx, ny = t.ny, j0 = t.j0, tj = g.tj;
                              switch (ln) {
                              case SA_Z: d = StageDesc{(const char*)g.z, t.sxy, nx, j0 - 1, tj + 2, 0, ny, 0, ES}; return true;
                              case SA_D:
                                  d = StageDesc{it > 0 ? (const char*)dbuf[2 * s + (it & 1)] : nullptr, t.sxy, nx, j0 - 1,
                                                tj + 2, 0, ny, L.bz, ES};
                                  return true;
                              case SA_DIAG: d = StageDesc{(const char*)g.diag, t.sxy, nx, j0, tj, 0, ny, 2 * L.bz, ES}; return true;
                              case SA_AZ:
                                  d = StageDesc{(const char*)g.a0z, t.sxy, nx, j0, tj, 0, ny, 2 * L.bz + L.bc, ES};
                                  return true;
                              case SA_AX:
                                  d = StageDesc{(const char*)g.a0x, (long long)(nx + 1) * ny, nx + 1, j0, tj, 0, ny,
                                                2 * L.bz + 2 * L.bc, ES};
                                  return true;
                              case SA_AY:
                                  d = StageDesc{(const char*)g.a0y, (long long)nx * (ny + 1), nx, j0, tj + 1, 0, ny + 1,
                                                2 * L.bz + 2 * L.bc + L.bx, ES};
                                  return true;
                              default: return false;
                              }
                          });
        return;
    }
    // ---- consumers --------------------------------------------------------------
    const int tot = sst_[dom.nscn];
    char* const ringB = sm + (size_t)ST * shape.slot;
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
        const unsigned magic = divMagic(nx);
        const int ringRa = max(j0 - 1, 0), ringRe = min(t.j1 + 1, ny);
        const int mC = (int)(t.sxy & (EPV - 1)), mX = (int)(((long long)(nx + 1) * ny) & (EPV - 1));
        const int mY = (int)(((long long)nx * (ny + 1)) & (EPV - 1));
        const int rC = (j0 * nx) & (EPV - 1), rCm = ((j0 - 1) * nx) & (EPV - 1);
        const int rX = (j0 * (nx + 1)) & (EPV - 1), rY = rC;
        RbPipe pipe{full, empty, &abortFlag, seq, t.nPl, 0, 0, (unsigned)ST};
        Acc dot{};
        for (int kk = t.k0; kk < t.k1; ++kk) {
            const int ic = kk - kLo;
            pipe.waitThrough(ic + 1, g.errWord);
            // d of the planes entering the ring (rows j0-1 .. j1)
            if (!abortFlag) {
                for (int k = kk == t.k0 ? kLo : kk + 1; k <= min(kk + 1, kHi); ++k) {
                    const char* base = sm + (size_t)pipe.slotOf(k - kLo) * shape.slot;
                    const int n = (ringRe - ringRa) * nx;
                    const int oz = stageMod(k, mC, rCm, EPV) + (ringRa - (j0 - 1)) * nx;
                    const R* zs = reinterpret_cast<const R*>(base) + oz;
                    const R* ds = reinterpret_cast<const R*>(base + L.bz) + oz;
                    R* out = reinterpret_cast<R*>(ringB + (size_t)(k & 3) * shape.ring) + (ringRa - (j0 - 1)) * nx;
                    if (useD)
                        for (int e = threadIdx.x; e < n; e += RB_CTHREADS) out[e] = (T)(zs[e] + beta * ds[e]);
                    else
                        for (int e = threadIdx.x; e < n; e += RB_CTHREADS) out[e] = zs[e];
                }
            }
            consumerSync();
            if (!abortFlag) {
                const char* cur = sm + (size_t)pipe.slotOf(ic) * shape.slot;
                const char* nxt = kk + 1 <= kHi ? sm + (size_t)pipe.slotOf(ic + 1) * shape.slot : cur;
                const int oC = stageMod(kk, mC, rC, EPV);
                const R* dgp = reinterpret_cast<const R*>(cur + 2 * L.bz) + oC;
                const R* azp = reinterpret_cast<const R*>(cur + 2 * L.bz + L.bc) + oC;
                const R* azn = reinterpret_cast<const R*>(nxt + 2 * L.bz + L.bc) + stageMod(kk + 1, mC, rC, EPV);
                const R* axp = reinterpret_cast<const R*>(cur + 2 * L.bz + 2 * L.bc) + stageMod(kk, mX, rX, EPV);
                const R* ayp = reinterpret_cast<const R*>(cur + 2 * L.bz + 2 * L.bc + L.bx) + stageMod(kk, mY, rY, EPV);
                const R* D0 = reinterpret_cast<const R*>(ringB + (size_t)(kk & 3) * shape.ring) + nx;
                const R* Dm = reinterpret_cast<const R*>(ringB + (size_t)((kk + 3) & 3) * shape.ring) + nx;
                const R* Dp = reinterpret_cast<const R*>(ringB + (size_t)((kk + 1) & 3) * shape.ring) + nx;
                const long long cbase = (long long)kk * t.sxy + (long long)j0 * nx;
                R* const dnp = dnew + cbase;
                R* const qp = q + cbase;
                const bool hasM = kk > 0, hasP = kk < nz - 1;
                for (int e = threadIdx.x; e < ncell; e += RB_CTHREADS) {
                    const int jj = divBy(e, nx, magic);
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
            pipe.releaseThrough(ic);   // planes up to kk are read by no later step
        }
        pipe.releaseThrough(t.nPl - 1);
        seq += t.nPl;
        if (consumerSyncOr(abortFlag)) return;
        double total;
        if (lastCtaSumC(g, PS_DQ, tile, sst_[s + 1] - sst_[s], dot, &total, sh, &amLast) && threadIdx.x == 0) {
            g.sv[SV_DQ] = total;
            if (g.sv[SV_BREAK] == 1) {   // the iteration after a breakdown: no update, then a restart
                g.sv[SV_ALPHA] = 0;
                g.sv[SV_BREAK] = 2;
            } else if (total <= 0) {
                g.sv[SV_DONE] = 1;
            } else {
                g.sv[SV_ALPHA] = g.sv[SV_RZ] / total;
            }
        }
    }
}

}  // namespace phx

namespace phx {

// ---------------------------------------------------------------------------------
// Level-0 Gauss-Seidel half sweeps of the V-cycle (gsColor, pressure_mg.cpp:195-216)
// on row-block tiles; red cells have i + j + k even.
//
// GS_PRE   the pre-smoothing pair from x = 0: red = r / diag, then black from
//          its red neighbours. The red values of the tile and its halo go to a
//          4-plane ring, so each is divided once. Writes z on every cell.
// GS_BLACK the post-smoothing black sweep after the prolongation
//          (pressure_mg.cpp:290-297): the red neighbours are z + x_c[agg]; the
//          ring holds them. Writes the black cells of z.
// GS_RED   the last (red) half sweep fused with r.z (dotRZ,
//          src/sim/gasphase.cpp:582-588); the last CTA of a scenario closes the
//          CG iteration (closeCgIteration). Writes the red cells of z.
enum { GS_PRE = 0, GS_BLACK = 1, GS_RED = 2 };

template <class R, int MODE>
struct GsLayout {
    static constexpr int MIN_ST = MODE == GS_RED ? 4 : 3;
    static constexpr int ES = (int)sizeof(R);
    int oZ, oAG, oR, oDG, oAZ, oAX, oAY, slot, ring;
    __host__ __device__ GsLayout(int nx, int tj) {
        const int hr = MODE == GS_PRE ? tj + 2 : tj;   // rows of r and diag
        int o = 0;
        oZ = o;  o += MODE == GS_PRE ? 0 : stageBytes(tj + 2, nx, ES);
        oAG = o; o += MODE == GS_BLACK ? stageBytes(tj + 2, nx, 4) : 0;
        oR = o;  o += stageBytes(hr, nx, ES);
        oDG = o; o += stageBytes(hr, nx, ES);
        oAZ = o; o += stageBytes(tj, nx, ES);
        oAX = o; o += stageBytes(tj, nx + 1, ES);
        oAY = o; o += stageBytes(tj + 1, nx, ES);
        slot = o;
        ring = MODE == GS_RED ? 0 : roundUp((tj + 2) * nx * ES, 16);
    }
};


enum { SG_Z = 0, SG_AG, SG_R, SG_DG, SG_AZ, SG_AX, SG_AY, SG_COUNT };

// the sweeps' division by the diagonal: IEEE on the FP64 path (the
// reference's operation), the fast reciprocal-based division on the FP32
// path (a preconditioner; diagonals are far from the range where it loses
// accuracy)
__device__ __forceinline__ double gsDiv(double a, double b) { return a / b; }
__device__ __forceinline__ float gsDiv(float a, float b) { return __fdividef(a, b); }

template <class R, int MODE>
__global__ void __launch_bounds__(RB_THREADS, 2) k_gs_rb(const Scn<R>* __restrict__ S, ADom dom, RbShape shape, int phase) {
    using T = R;
    using Acc = decltype(dotTerm(T(0), T(0)));
    using LY = GsLayout<R, MODE>;
    const int ST = shape.st;
    constexpr int EPV = 16 / (int)sizeof(R);
    constexpr int ES = (int)sizeof(R);
    PHX_RB_PROLOGUE()
    if (warp == RB_CONSUMERS) {
        rbProducer<R>(S, sst_, dom.nscn, sm, shape.slot, ST, 1, full, empty, &abortFlag,
                          [&](int ln, int, const Scn<R>& g, const RbTile& t, StageDesc& d) {
                              const LY L(t.nx, g.tj);
                              const int nx = t.nx, ny = t.ny, j0 = t.j0, tj = g.tj;
                              const int hlo = MODE == GS_PRE ? j0 - 1 : j0, hr = MODE == GS_PRE ? tj + 2 : tj;
                              switch (ln) {
                              case SG_Z:
                                  if (MODE == GS_PRE) return false;
                                  d = StageDesc{(const char*)g.z, t.sxy, nx, j0 - 1, tj + 2, 0, ny, L.oZ, ES};
                                  return true;
                              case SG_AG:
                                  if (MODE != GS_BLACK) return false;
                                  d = StageDesc{(const char*)g.lv[0].agg, t.sxy, nx, j0 - 1, tj + 2, 0, ny, L.oAG, 4};
                                  return true;
                              case SG_R: d = StageDesc{(const char*)g.r, t.sxy, nx, hlo, hr, 0, ny, L.oR, ES}; return true;
                              case SG_DG: d = StageDesc{(const char*)g.diag, t.sxy, nx, hlo, hr, 0, ny, L.oDG, ES}; return true;
                              case SG_AZ: d = StageDesc{(const char*)g.a0z, t.sxy, nx, j0, tj, 0, ny, L.oAZ, ES}; return true;
                              case SG_AX:
                                  d = StageDesc{(const char*)g.a0x, (long long)(nx + 1) * ny, nx + 1, j0, tj, 0, ny, L.oAX, ES};
                                  return true;
                              case SG_AY:
                                  d = StageDesc{(const char*)g.a0y, (long long)nx * (ny + 1), nx, j0, tj + 1, 0, ny + 1, L.oAY, ES};
                                  return true;
                              default: return false;
                              }
                          });
        return;
    }
    // ---- consumers --------------------------------------------------------------
    const int tot = sst_[dom.nscn];
    char* const ringB = sm + (size_t)ST * shape.slot;
    unsigned seq = 0;
    for (int b = blockIdx.x; b < tot; b += gridDim.x) {
        int s, tile;
        locateShared(sst_, dom.nscn, b, s, tile);
        const Scn<R>& g = S[s];
        const RbTile t = rbTile(g, tile);
        const int nx = t.nx, ny = t.ny, nz = t.nz, j0 = t.j0, kLo = t.kLo, kHi = t.kHi;
        const LY L(nx, g.tj);
        R* const z = g.z;
        const R* const xc = g.lv[1].x;
        const int ncell = (t.j1 - j0) * nx;
        const unsigned magic = divMagic(nx);
        const int ringRa = max(j0 - 1, 0), ringRe = min(t.j1 + 1, ny);
        const int mC = (int)(t.sxy & (EPV - 1)), mX = (int)(((long long)(nx + 1) * ny) & (EPV - 1));
        const int mY = (int)(((long long)nx * (ny + 1)) & (EPV - 1)), mC4 = (int)(t.sxy & 3);
        const int rC = (j0 * nx) & (EPV - 1), rCm = ((j0 - 1) * nx) & (EPV - 1), rCm4 = ((j0 - 1) * nx) & 3;
        const int rX = (j0 * (nx + 1)) & (EPV - 1), rY = rC;
        const int hx = (nx + 1) >> 1;                       // pairs of cells per row
        const unsigned magicHx = divMagic(hx);
        const int rH = MODE == GS_PRE ? rCm : rC;           // residue of the first row of r and diag
        const int hOff = MODE == GS_PRE ? nx : 0;           // row j0 within the r and diag arrays
        RbPipe pipe{full, empty, &abortFlag, seq, t.nPl, 0, 0, (unsigned)ST};
        Acc dot{};
        for (int kk = t.k0; kk < t.k1; ++kk) {
            const int ic = kk - kLo;
            pipe.waitThrough(ic + 1, g.errWord);
            if constexpr (MODE != GS_RED) {
                // red values of the planes entering the ring (rows j0-1 .. j1), one
                // per pair of cells (2m, 2m+1) of a row
                if (!abortFlag) {
                    for (int k = kk == t.k0 ? kLo : kk + 1; k <= min(kk + 1, kHi); ++k) {
                        const char* base = sm + (size_t)pipe.slotOf(k - kLo) * shape.slot;
                        const int np = (ringRe - ringRa) * hx;
                        const int row0 = (ringRa - (j0 - 1)) * nx;   // ring index of row ringRa
                        R* out = reinterpret_cast<R*>(ringB + (size_t)(k & 3) * shape.ring) + row0;
                        if constexpr (MODE == GS_PRE) {
                            const int o = stageMod(k, mC, rCm, EPV) + row0;
                            const R* rs = reinterpret_cast<const R*>(base + L.oR) + o;
                            const R* ds = reinterpret_cast<const R*>(base + L.oDG) + o;
                            for (int p = threadIdx.x; p < np; p += RB_CTHREADS) {
                                const int jr = divBy(p, hx, magicHx), m = p - jr * hx;
                                const int i = 2 * m + ((ringRa + jr + k) & 1);
                                if (i >= nx) continue;
                                const int e = jr * nx + i;
                                const T dg = ds[e];
                                out[e] = dg <= 0 ? T(0) : gsDiv(rs[e], dg);
                            }
                        } else {
                            const R* zs = reinterpret_cast<const R*>(base + L.oZ) + stageMod(k, mC, rCm, EPV) + row0;
                            const int* as = reinterpret_cast<const int*>(base + L.oAG) + stageMod(k, mC4, rCm4, 4) + row0;
                            // four pairs per thread at a time, so that their gathers of
                            // the coarse correction are in flight together
                            for (int p0 = threadIdx.x; p0 < np; p0 += 4 * RB_CTHREADS) {
                                T v[4], xv[4];
                                int a[4], ee[4];
#pragma unroll
                                for (int u = 0; u < 4; ++u) {
                                    const int p = p0 + u * RB_CTHREADS;
                                    ee[u] = -1;
                                    a[u] = -1;
                                    v[u] = T(0);
                                    if (p < np) {
                                        const int jr = divBy(p, hx, magicHx), m = p - jr * hx;
                                        const int i = 2 * m + ((ringRa + jr + k) & 1);
                                        if (i < nx) {
                                            ee[u] = jr * nx + i;
                                            v[u] = zs[ee[u]];
                                            a[u] = as[ee[u]];
                                        }
                                    }
                                }
#pragma unroll
                                for (int u = 0; u < 4; ++u) xv[u] = a[u] >= 0 ? (T)xc[a[u]] : T(0);
#pragma unroll
                                for (int u = 0; u < 4; ++u)
                                    if (ee[u] >= 0) out[ee[u]] = a[u] >= 0 ? (T)(v[u] + xv[u]) : v[u];
                            }
                        }
                    }
                }
                consumerSync();
            }
            if (!abortFlag) {
                const char* cur = sm + (size_t)pipe.slotOf(ic) * shape.slot;
                const char* nxt = kk + 1 <= kHi ? sm + (size_t)pipe.slotOf(ic + 1) * shape.slot : cur;
                const char* prv = kk - 1 >= kLo ? sm + (size_t)pipe.slotOf(ic - 1) * shape.slot : cur;
                const int oC = stageMod(kk, mC, rC, EPV);
                const R* rp = reinterpret_cast<const R*>(cur + L.oR) + stageMod(kk, mC, rH, EPV) + hOff;
                const R* dgp = reinterpret_cast<const R*>(cur + L.oDG) + stageMod(kk, mC, rH, EPV) + hOff;
                const R* azp = reinterpret_cast<const R*>(cur + L.oAZ) + oC;
                const R* azn = reinterpret_cast<const R*>(nxt + L.oAZ) + stageMod(kk + 1, mC, rC, EPV);
                const R* axp = reinterpret_cast<const R*>(cur + L.oAX) + stageMod(kk, mX, rX, EPV);
                const R* ayp = reinterpret_cast<const R*>(cur + L.oAY) + stageMod(kk, mY, rY, EPV);
                // neighbour values: the ring (red values) or the staged z (GS_RED), at row j0
                const R *X0, *Xm, *Xp;
                if constexpr (MODE == GS_RED) {
                    X0 = reinterpret_cast<const R*>(cur + L.oZ) + stageMod(kk, mC, rCm, EPV) + nx;
                    Xm = reinterpret_cast<const R*>(prv + L.oZ) + stageMod(kk - 1, mC, rCm, EPV) + nx;
                    Xp = reinterpret_cast<const R*>(nxt + L.oZ) + stageMod(kk + 1, mC, rCm, EPV) + nx;
                } else {
                    X0 = reinterpret_cast<const R*>(ringB + (size_t)(kk & 3) * shape.ring) + nx;
                    Xm = reinterpret_cast<const R*>(ringB + (size_t)((kk + 3) & 3) * shape.ring) + nx;
                    Xp = reinterpret_cast<const R*>(ringB + (size_t)((kk + 1) & 3) * shape.ring) + nx;
                }
                R* const zp = z + (long long)kk * t.sxy + (long long)j0 * nx;
                const bool hasM = kk > 0, hasP = kk < nz - 1;
                // the colour this sweep updates: black (odd) for GS_PRE and GS_BLACK, red for GS_RED
                const int upd = MODE == GS_RED ? 0 : 1;
                const int np = (t.j1 - j0) * hx;
                // one pair of cells (2m, 2m+1) of a row per thread: one is updated,
                // the other (GS_PRE: its red value; GS_RED: its r.z term) is passed on
                for (int p = threadIdx.x; p < np; p += RB_CTHREADS) {
                    const int jj = divBy(p, hx, magicHx), m = p - jj * hx;
                    const int j = j0 + jj;
                    const int iu = 2 * m + ((j + kk + upd) & 1), io = 4 * m + 1 - iu;
                    if (iu < nx) {
                        const int e = jj * nx + iu;
                        const T dg = dgp[e];
                        T zc = 0;
                        if (dg > 0) {
                            const R* ax = axp + e + jj;   // a0x index jj * (nx + 1) + i
                            T sacc = rp[e];
                            if (iu > 0) sacc += ax[0] * X0[e - 1];
                            if (iu < nx - 1) sacc += ax[1] * X0[e + 1];
                            if (j > 0) sacc += ayp[e] * X0[e - nx];
                            if (j < ny - 1) sacc += ayp[e + nx] * X0[e + nx];
                            if (hasM) sacc += azp[e] * Xm[e];
                            if (hasP) sacc += azn[e] * Xp[e];
                            zc = gsDiv(sacc, dg);
                        }
                        zp[e] = zc;
                        if constexpr (MODE == GS_RED) dot = accAdd(dot, dotTerm((T)rp[e], zc));
                    }
                    if (io < nx) {
                        const int e = jj * nx + io;
                        if constexpr (MODE == GS_PRE) zp[e] = X0[e];                       // the red value of the ring
                        if constexpr (MODE == GS_RED) dot = accAdd(dot, dotTerm((T)rp[e], (T)X0[e]));   // staged black
                    }
                }
            }
            pipe.releaseThrough(MODE == GS_RED ? ic - 1 : ic);
        }
        pipe.releaseThrough(t.nPl - 1);
        seq += t.nPl;
        if (consumerSyncOr(abortFlag)) return;
        if constexpr (MODE == GS_RED) {
            if (phase == 2) continue;
            double tot2;
            if (lastCtaSumC(g, PS_RZ, tile, sst_[s + 1] - sst_[s], dot, &tot2, sh, &amLast) && threadIdx.x == 0)
                closeCgIteration(g, phase, tot2);
        }
    }
}

}  // namespace phx

namespace phx {

// ---------------------------------------------------------------------------------
// Level-0 residual (residualGrid, pressure_mg.cpp:217-235) and its restriction
// to level 1 (:285-286) on row-block tiles. z of the tile and its halo rows
// goes to a 4-plane ring; the residuals of an even plane wait in shared memory
// (with their aggregate ids) until the odd plane above it is done, then one
// thread per 2x2x2 block sums each level-1 aggregate's cells in ascending
// cell order -- the order of the reference's scatter (an aggregate lies in one
// block; tiles start on even rows and even planes).
template <class R>
struct ResLayout {
    static constexpr int MIN_ST = 3;
    static constexpr int ES = (int)sizeof(R);
    int oZ, oAG, oR, oDG, oAZ, oAX, oAY, slot, ring, oRA, oRB, oGA, bytes;
    __host__ __device__ ResLayout(int nx, int tj) {
        int o = 0;
        oZ = o;  o += stageBytes(tj + 2, nx, ES);
        oAG = o; o += stageBytes(tj, nx, 4);
        oR = o;  o += stageBytes(tj, nx, ES);
        oDG = o; o += stageBytes(tj, nx, ES);
        oAZ = o; o += stageBytes(tj, nx, ES);
        oAX = o; o += stageBytes(tj, nx + 1, ES);
        oAY = o; o += stageBytes(tj + 1, nx, ES);
        slot = o;
        ring = roundUp((tj + 2) * nx * ES, 16);
        // after the ring: residuals of the even and odd plane, aggregate ids of the even plane
        oRA = 0;
        oRB = roundUp(tj * nx * ES, 16);
        oGA = 2 * oRB;
        bytes = oGA + roundUp(tj * nx * 4, 16);
    }
};


template <class R>
__global__ void __launch_bounds__(RB_THREADS, 1) k_res_rb(const Scn<R>* __restrict__ S, ADom dom, RbShape shape) {
    using T = R;
    using LY = ResLayout<R>;
    const int ST = shape.st;
    constexpr int EPV = 16 / (int)sizeof(R);
    constexpr int ES = (int)sizeof(R);
    PHX_RB_PROLOGUE()
    if (warp == RB_CONSUMERS) {
        rbProducer<R>(S, sst_, dom.nscn, sm, shape.slot, ST, 1, full, empty, &abortFlag,
                          [&](int ln, int, const Scn<R>& g, const RbTile& t, StageDesc& d) {
                              const LY L(t.nx, g.tj);
                              const int nx = t.nx, ny = t.ny, j0 = t.j0, tj = g.tj;
                              switch (ln) {
                              case SG_Z: d = StageDesc{(const char*)g.z, t.sxy, nx, j0 - 1, tj + 2, 0, ny, L.oZ, ES}; return true;
                              case SG_AG: d = StageDesc{(const char*)g.lv[0].agg, t.sxy, nx, j0, tj, 0, ny, L.oAG, 4}; return true;
                              case SG_R: d = StageDesc{(const char*)g.r, t.sxy, nx, j0, tj, 0, ny, L.oR, ES}; return true;
                              case SG_DG: d = StageDesc{(const char*)g.diag, t.sxy, nx, j0, tj, 0, ny, L.oDG, ES}; return true;
                              case SG_AZ: d = StageDesc{(const char*)g.a0z, t.sxy, nx, j0, tj, 0, ny, L.oAZ, ES}; return true;
                              case SG_AX:
                                  d = StageDesc{(const char*)g.a0x, (long long)(nx + 1) * ny, nx + 1, j0, tj, 0, ny, L.oAX, ES};
                                  return true;
                              case SG_AY:
                                  d = StageDesc{(const char*)g.a0y, (long long)nx * (ny + 1), nx, j0, tj + 1, 0, ny + 1, L.oAY, ES};
                                  return true;
                              default: return false;
                              }
                          });
        return;
    }
    // ---- consumers --------------------------------------------------------------
    const int tot = sst_[dom.nscn];
    char* const ringB = sm + (size_t)ST * shape.slot;
    char* const tail = ringB + 4 * (size_t)shape.ring;
    unsigned seq = 0;
    for (int b = blockIdx.x; b < tot; b += gridDim.x) {
        int s, tile;
        locateShared(sst_, dom.nscn, b, s, tile);
        const Scn<R>& g = S[s];
        const RbTile t = rbTile(g, tile);
        const int nx = t.nx, ny = t.ny, nz = t.nz, j0 = t.j0, kLo = t.kLo, kHi = t.kHi;
        const LY L(nx, g.tj);
        R* const cb = g.lv[1].b;
        const int rows = t.j1 - j0, ncell = rows * nx;
        const unsigned magic = divMagic(nx);
        const int ringRa = max(j0 - 1, 0), ringRe = min(t.j1 + 1, ny);
        const int mC = (int)(t.sxy & (EPV - 1)), mX = (int)(((long long)(nx + 1) * ny) & (EPV - 1));
        const int mY = (int)(((long long)nx * (ny + 1)) & (EPV - 1)), mC4 = (int)(t.sxy & 3);
        const int rC = (j0 * nx) & (EPV - 1), rCm = ((j0 - 1) * nx) & (EPV - 1), rC4 = (j0 * nx) & 3;
        const int rX = (j0 * (nx + 1)) & (EPV - 1), rY = rC;
        T* const RA = reinterpret_cast<T*>(tail + L.oRA);
        T* const RB = reinterpret_cast<T*>(tail + L.oRB);
        int* const GA = reinterpret_cast<int*>(tail + L.oGA);
        const int hx = (nx + 1) >> 1, hy = (rows + 1) >> 1, nblk = hx * hy;
        const unsigned magicHx = divMagic(hx);
        RbPipe pipe{full, empty, &abortFlag, seq, t.nPl, 0, 0, (unsigned)ST};
        for (int kk = t.k0; kk < t.k1; ++kk) {
            const int ic = kk - kLo;
            pipe.waitThrough(ic + 1, g.errWord);
            if (!abortFlag) {
                for (int k = kk == t.k0 ? kLo : kk + 1; k <= min(kk + 1, kHi); ++k) {
                    const char* base = sm + (size_t)pipe.slotOf(k - kLo) * shape.slot;
                    const int n = (ringRe - ringRa) * nx;
                    const int row0 = (ringRa - (j0 - 1)) * nx;
                    const R* zs = reinterpret_cast<const R*>(base + L.oZ) + stageMod(k, mC, rCm, EPV) + row0;
                    R* out = reinterpret_cast<R*>(ringB + (size_t)(k & 3) * shape.ring) + row0;
                    for (int e = threadIdx.x; e < n; e += RB_CTHREADS) out[e] = zs[e];
                }
            }
            consumerSync();
            const bool odd = (kk & 1) != 0;
            if (!abortFlag) {
                const char* cur = sm + (size_t)pipe.slotOf(ic) * shape.slot;
                const char* nxt = kk + 1 <= kHi ? sm + (size_t)pipe.slotOf(ic + 1) * shape.slot : cur;
                const int oC = stageMod(kk, mC, rC, EPV);
                const R* rp = reinterpret_cast<const R*>(cur + L.oR) + oC;
                const R* dgp = reinterpret_cast<const R*>(cur + L.oDG) + oC;
                const int* agp = reinterpret_cast<const int*>(cur + L.oAG) + stageMod(kk, mC4, rC4, 4);
                const R* azp = reinterpret_cast<const R*>(cur + L.oAZ) + oC;
                const R* azn = reinterpret_cast<const R*>(nxt + L.oAZ) + stageMod(kk + 1, mC, rC, EPV);
                const R* axp = reinterpret_cast<const R*>(cur + L.oAX) + stageMod(kk, mX, rX, EPV);
                const R* ayp = reinterpret_cast<const R*>(cur + L.oAY) + stageMod(kk, mY, rY, EPV);
                const R* X0 = reinterpret_cast<const R*>(ringB + (size_t)(kk & 3) * shape.ring) + nx;
                const R* Xm = reinterpret_cast<const R*>(ringB + (size_t)((kk + 3) & 3) * shape.ring) + nx;
                const R* Xp = reinterpret_cast<const R*>(ringB + (size_t)((kk + 1) & 3) * shape.ring) + nx;
                T* const RR = odd ? RB : RA;
                const bool hasM = kk > 0, hasP = kk < nz - 1;
                for (int e = threadIdx.x; e < ncell; e += RB_CTHREADS) {
                    const int jj = divBy(e, nx, magic);
                    const int i = e - jj * nx, j = j0 + jj;
                    const int A = agp[e];
                    T rv = 0;
                    if (A >= 0) {
                        const R* ax = axp + e + jj;
                        T sacc = rp[e] - dgp[e] * X0[e];
                        if (i > 0) sacc += ax[0] * X0[e - 1];
                        if (i < nx - 1) sacc += ax[1] * X0[e + 1];
                        if (j > 0) sacc += ayp[e] * X0[e - nx];
                        if (j < ny - 1) sacc += ayp[e + nx] * X0[e + nx];
                        if (hasM) sacc += azp[e] * Xm[e];
                        if (hasP) sacc += azn[e] * Xp[e];
                        rv = sacc;
                    }
                    RR[e] = rv;
                    if (!odd) GA[e] = A;
                }
            }
            // blocks close on odd planes, and on the grid's last plane when nz is odd
            const bool close = odd || kk == nz - 1;
            if (close) {
                consumerSync();
                if (!abortFlag) {
                    const char* cur = sm + (size_t)pipe.slotOf(ic) * shape.slot;
                    const int* agOdd = reinterpret_cast<const int*>(cur + L.oAG) + stageMod(kk, mC4, rC4, 4);
                    for (int q = threadIdx.x; q < nblk; q += RB_CTHREADS) {
                        const int by = divBy(q, hx, magicHx), bx = q - by * hx;
                        int ag[8];
                        T rv[8];
#pragma unroll
                        for (int m = 0; m < 8; ++m) {
                            const int di = m & 1, dj = (m >> 1) & 1, dk = m >> 2;
                            const int i = 2 * bx + di, jj = 2 * by + dj;
                            const bool in = i < nx && jj < rows && (odd || dk == 0);
                            const int e = jj * nx + i;
                            // dk = 0: the even plane (or the lone last plane); dk = 1: the odd plane
                            const bool useEven = !odd || dk == 0;
                            ag[m] = in ? (useEven ? GA[e] : agOdd[e]) : -1;
                            rv[m] = in ? (useEven ? RA[e] : RB[e]) : T(0);
                        }
#pragma unroll
                        for (int m = 0; m < 8; ++m) {
                            const int a = ag[m];
                            bool first = a >= 0;
#pragma unroll
                            for (int p = 0; p < m; ++p) first = first && ag[p] != a;
                            if (!first) continue;
                            T acc = 0;
#pragma unroll
                            for (int p = m; p < 8; ++p)
                                if (ag[p] == a) acc = acc + rv[p];
                            cb[a] = acc;
                        }
                    }
                }
            }
            pipe.releaseThrough(ic);
            // RA / GA of an even plane are read at the next (odd) step: no barrier needed
            // before they are rewritten, which happens two steps later after a consumerSync
        }
        pipe.releaseThrough(t.nPl - 1);
        seq += t.nPl;
        if (consumerSyncOr(abortFlag)) return;
    }
}

}  // namespace phx

namespace phx {

// host side: the shared-memory shapes of the row-block kernels over a batch
// (the largest slot and ring of its grids), and the number of staging slots
// of each kernel. The slot count is chosen from the shared memory of an SM:
// for one or two CTAs per SM, as many slots as fit (up to RB_MAX_ST), keeping
// the configuration with the most bytes in flight per SM (slots beyond the
// ones the stencil holds resident, times CTAs per SM).
constexpr size_t RB_SM_SMEM = 228 * 1024;      // shared memory of a GB300 SM
constexpr size_t RB_STATIC_SMEM = 6 * 1024;    // the kernels' static shared memory, rounded up
template <class R>
struct RbShapes {
    RbShape apply{0, 0, 0}, gs[3] = {RbShape{0, 0, 0}, RbShape{0, 0, 0}, RbShape{0, 0, 0}}, res{0, 0, 0};
    int resTail = 0;
    static void grow(RbShape& a, int slot, int ring) {
        a.slot = a.slot > slot ? a.slot : slot;
        a.ring = a.ring > ring ? a.ring : ring;
    }
    void add(int nx, int ny) {
        const int tj = rowBlockRows<R>(nx, ny);
        const ApplyLayout<R> a(nx, tj);
        grow(apply, a.slot, a.ring);
        const GsLayout<R, GS_PRE> g0(nx, tj);
        grow(gs[0], g0.slot, g0.ring);
        const GsLayout<R, GS_BLACK> g1(nx, tj);
        grow(gs[1], g1.slot, g1.ring);
        const GsLayout<R, GS_RED> g2(nx, tj);
        grow(gs[2], g2.slot, g2.ring);
        const ResLayout<R> rl(nx, tj);
        grow(res, rl.slot, rl.ring);
        resTail = resTail > rl.bytes ? resTail : rl.bytes;
    }
    // slots for one kernel (0 if even one CTA per SM cannot hold minSt slots)
    static int pickSlots(const RbShape& sh, int tail, int minSt) {
        int best = 0;
        size_t bestFlight = 0;
        for (int ctas = 2; ctas >= 1; --ctas) {
            const size_t per = RB_SM_SMEM / ctas - RB_STATIC_SMEM;
            const size_t fixed = 4 * (size_t)sh.ring + (size_t)tail;
            if (sh.slot <= 0 || per <= fixed) continue;
            int st = (int)((per - fixed) / (size_t)sh.slot);
            if (st > RB_MAX_ST) st = RB_MAX_ST;
            if (st < minSt) continue;
            const size_t flight = (size_t)ctas * (size_t)(st - minSt + 1) * (size_t)sh.slot;
            if (flight > bestFlight) { bestFlight = flight; best = st; }
        }
        return best;
    }
    // fills the slot counts; false if a kernel does not fit
    bool finish() {
        apply.st = pickSlots(apply, 0, ApplyLayout<R>::MIN_ST);
        gs[0].st = pickSlots(gs[0], 0, GsLayout<R, GS_PRE>::MIN_ST);
        gs[1].st = pickSlots(gs[1], 0, GsLayout<R, GS_BLACK>::MIN_ST);
        gs[2].st = pickSlots(gs[2], 0, GsLayout<R, GS_RED>::MIN_ST);
        res.st = pickSlots(res, resTail, ResLayout<R>::MIN_ST);
        return apply.st && gs[0].st && gs[1].st && gs[2].st && res.st;
    }
    size_t smemApply() const { return rbSmem(apply); }
    size_t smemGs(int m) const { return rbSmem(gs[m]); }
    size_t smemRes() const { return rbSmem(res, resTail); }
};

}  // namespace phx
