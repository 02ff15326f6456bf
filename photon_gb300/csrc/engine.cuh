// The GPU engine: a batch of scenarios stepped together, their device state,
// the domain tables of the launches and the launch sequence of the gas-phase
// step (src/sim/solver.cpp:226-269). A single-scenario context is a batch of
// one. Every kernel launch covers one domain (cells, faces of one axis, one
// multigrid level, ...) of every scenario; the whole step is captured once as
// a CUDA graph whose pressure-solve loops are device-side while nodes.
// Instantiated per precision by engine_fp64.cu and engine_mixed.cu.
#pragma once
#include <array>
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include "engine.h"
#include "host_setup.h"
#include "mixed_kernels.cuh"
#include "radiation.cuh"
#include "volume.cuh"
#include "rowblock.cuh"
#include "level0.cuh"

namespace phx {

#define PHX_CK(x)                                                                        \
    do {                                                                                 \
        cudaError_t e_ = (x);                                                            \
        if (e_ != cudaSuccess) {                                                         \
            err = std::string(#x) + ": " + cudaGetErrorString(e_);                      \
            return PHX_ERR_CUDA;                                                         \
        }                                                                                \
    } while (0)
#define PHX_TRY(x) do { int r_ = (x); if (r_) return r_; } while (0)

// dense coarse operators up to this many unknowns (n^2 reals)
constexpr int DENSE_MAX = 4096;

enum DomId {
    D_ONE = 0, D_CELLS, D_FX, D_FY, D_FZ, D_BX, D_BY, D_BZ, D_CZ, D_CC, D_CO_DENSE, D_CO_SERIAL, D_RB, D_QUAD, D_LEAK,
    D_L0,                        // level-0 tiles of the mixed path: 2x2x2 blocks (level0.cuh)
    D_L0R,                       // the same, several blocks per thread (the passes with a dot product)
    D_LV0,                       // D_LV0 + l: rows of level l when l is not the coarsest (1 <= l < 12)
    D_RS0 = D_LV0 + MAX_LEVELS,  // D_RS0 + l: rows of level l+1 for restriction from level l >= 1
    D_COUNT = D_RS0 + MAX_LEVELS
};

template <class T>
static T* carve(char*& base, size_t& off, size_t n) {
    off = (off + 255) & ~(size_t)255;
    T* p = base ? (T*)(base + off) : nullptr;
    off += n * sizeof(T);
    return p;
}

// One scenario: host set-up results, its device arena and its descriptor.
// mixed path: CG iterations between replacements of the FP32 recursive
// residual by the FP64 residual b - A p64
constexpr int REPLACE_EVERY = 10;

// V-cycle schedules of the mixed path, per bucket of scenario size: bucket b
// holds scenarios of [20000 * 2^b, 20000 * 2^(b+1)) cells (bucket 0 also the
// smaller ones, the last one the larger ones). A bucket's entry is the
// multigrid coarsening stop the autotuner chose (0: not tuned, the
// reference's 2000). Process-wide, so scenarios admitted later (serving,
// batch_add) are built with the tuned schedule of their size.
constexpr int VC_BUCKETS = 8;
inline int vcycleBucket(long long cells) {
    int b = 0;
    long long e = 40000;
    while (cells >= e && b < VC_BUCKETS - 1) { e *= 2; ++b; }
    return b;
}
inline std::mutex& vcycleMutex() { static std::mutex m; return m; }
inline int* vcycleTable() { static int t[VC_BUCKETS] = {0}; return t; }
// the mixed path's smoothing on the coarse levels: Jacobi sweeps per level on
// each leg of the V-cycle (2, the reference's schedule, until tuned; 1 after a
// tuning that found it faster at the solve's relative residual)
inline int& vcycleSweeps() { static int v = 2; return v; }
inline int vcycleStopFor(long long cells) {
    std::lock_guard<std::mutex> lock(vcycleMutex());
    const int v = vcycleTable()[vcycleBucket(cells)];
    return v > 0 ? v : MG_COARSE_STOP_REF;
}

template <class R>
struct Scenario {
    static constexpr bool kMixed = std::is_same<R, float>::value;
    GridGeom geo;
    double cfl = 0.5, dtMaxP = 0.02, tol = 0.002, relTol = 0;
    int maxIters = 400, radiationOn = 1;
    int coarseStop = MG_COARSE_STOP_REF;   // multigrid coarsening stop (the V-cycle schedule)
    Zones Z;
    Multigrid MG;
    std::vector<double> Pb0;
    std::vector<Src> ignitions, burners;
    char* arena = nullptr;       // fields, geometry, solve vectors, scalars
    char* mgArena = nullptr;     // the multigrid levels (replaced when the V-cycle schedule changes)
    size_t arenaBytes = 0;       // both arenas
    size_t mainBytes = 0, mgBytes = 0;
    Scn<R> h{};                  // host copy of the device descriptor
    R* dbuf[2] = {nullptr, nullptr};
    std::string err;

    ~Scenario() {
        if (arena) cudaFree(arena);
        if (mgArena) cudaFree(mgArena);
    }

    int setup(const phx_grid* g) {
        if (!g || g->nx <= 0 || g->ny <= 0 || g->nz <= 0 || !(g->dx > 0)) { err = "invalid grid dimensions"; return PHX_ERR_INVALID; }
        long long N = (long long)g->nx * g->ny * g->nz;
        if (N > 20000000LL) { err = "grid size out of range (the reference caps N at 20,000,000)"; return PHX_ERR_INVALID; }
        if (!g->blocked || !g->fx || !g->fy || !g->fz || !g->ax || !g->ay || !g->az) { err = "missing geometry array"; return PHX_ERR_INVALID; }
        if (g->radiation_on && !g->adiabatic_surfaces) {
            err = "radiation with non-adiabatic surfaces (the ray-traced radiation stage) is not part of the GPU step";
            return PHX_ERR_UNSUPPORTED;
        }
        geo.nx = g->nx; geo.ny = g->ny; geo.nz = g->nz;
        geo.dx = g->dx; geo.ox = g->ox; geo.oy = g->oy; geo.oz = g->oz;
        geo.windSpeed = g->wind_speed; geo.windFromDeg = g->wind_from_deg; geo.windExp = g->wind_exponent;
        const int NN = geo.N(), NX = geo.NX(), NY = geo.NY(), NZ = geo.NZ();
        geo.blocked.assign(g->blocked, g->blocked + NN);
        geo.fx.assign(g->fx, g->fx + NX); geo.fy.assign(g->fy, g->fy + NY); geo.fz.assign(g->fz, g->fz + NZ);
        geo.ax.assign(g->ax, g->ax + NX); geo.ay.assign(g->ay, g->ay + NY); geo.az.assign(g->az, g->az + NZ);
        geo.lx.assign(NX, 0); geo.ly.assign(NY, 0); geo.lz.assign(NZ, 0);
        if (g->lx) geo.lx.assign(g->lx, g->lx + NX);
        if (g->ly) geo.ly.assign(g->ly, g->ly + NY);
        if (g->lz) geo.lz.assign(g->lz, g->lz + NZ);
        geo.anyLeak = false;
        for (auto v : geo.lx) geo.anyLeak |= v != 0;
        for (auto v : geo.ly) geo.anyLeak |= v != 0;
        for (auto v : geo.lz) geo.anyLeak |= v != 0;
        RbShapes<R> one;
        one.add(g->nx, g->ny);
        if (!one.finish()) {
            err = "grid rows too long for the shared-memory tiles of the pressure kernels (nx = " + std::to_string(g->nx) + ")";
            return PHX_ERR_UNSUPPORTED;
        }
        cfl = g->cfl; dtMaxP = g->dt_max; tol = g->tol; relTol = g->rel_tol; maxIters = g->max_iters;
        radiationOn = g->radiation_on;
        // set-up on the host: zones, multigrid
        Pb0.assign(NN, 101325.0);
        Z = computeZones(geo, Pb0);
        if (kMixed) coarseStop = vcycleStopFor(NN);   // the tuned schedule of the scenario's size, if any
        MG = buildMultigrid(geo, DENSE_MAX, coarseStop, coarseSolveFor());
        buildLeakFaces();
        return PHX_OK;
    }

    // leak faces in the reference's order (axis, then face index) that touch no
    // blocked cell, and per zone its faces to other zones (src/sim/gasphase.cpp:410-445)
    std::vector<int> leak;       // 4 per face: axis, f, a, b
    std::vector<int> leakZStart, leakZList;
    void buildLeakFaces() {
        leak.clear();
        const int nx = geo.nx, ny = geo.ny, nz = geo.nz;
        for (int axis = 0; axis < 3 && geo.anyLeak; ++axis) {
            const std::vector<uint8_t>& lk = axis == 0 ? geo.lx : axis == 1 ? geo.ly : geo.lz;
            const int dX = nx + (axis == 0), dY = ny + (axis == 1);
            const int ncell = axis == 0 ? nx : axis == 1 ? ny : nz;
            for (int f = 0; f < (int)lk.size(); ++f) {
                if (!lk[f]) continue;
                const int i = f % dX, j = (f / dX) % dY, k = f / (dX * dY);
                int id[3] = {i, j, k}, a[3] = {i, j, k};
                a[axis] -= 1;
                const int ca = a[axis] >= 0 ? geo.cell(a[0], a[1], a[2]) : -1;
                const int cb = id[axis] < ncell ? geo.cell(i, j, k) : -1;
                if ((ca >= 0 && geo.blocked[ca]) || (cb >= 0 && geo.blocked[cb])) continue;
                leak.insert(leak.end(), {axis, f, ca, cb});
            }
        }
        const int nZ = (int)Z.zoneP.size(), nf = (int)leak.size() / 4;
        leakZStart.assign(nZ + 1, 0);
        auto zoneOf = [&](int c) { return c >= 0 ? Z.zone[c] : -1; };
        for (int q = 0; q < nf; ++q) {
            const int za = zoneOf(leak[4 * q + 2]), zb = zoneOf(leak[4 * q + 3]);
            if (za == zb) continue;
            if (za >= 0) leakZStart[za + 1]++;
            if (zb >= 0) leakZStart[zb + 1]++;
        }
        for (int z = 0; z < nZ; ++z) leakZStart[z + 1] += leakZStart[z];
        leakZList.assign(leakZStart[nZ], 0);
        std::vector<int> fill(nZ, 0);
        for (int q = 0; q < nf; ++q) {
            const int za = zoneOf(leak[4 * q + 2]), zb = zoneOf(leak[4 * q + 3]);
            if (za == zb) continue;
            if (za >= 0) leakZList[leakZStart[za] + fill[za]++] = q;
            if (zb >= 0) leakZList[leakZStart[zb] + fill[zb]++] = q;
        }
    }

    // device bytes the scenario will take (both arenas' layouts without memory)
    size_t layout(char* base) {
        if (base) return layoutMain(base) + layoutLevels(mgArena);
        return layoutMain(nullptr) + layoutLevels(nullptr);
    }

    size_t layoutMain(char* base) {
        const int N = geo.N(), NX = geo.NX(), NY = geo.NY(), NZ = geo.NZ();
        const int nl = (int)MG.lv.size();
        // one reduction partial per CTA of the widest reduction domain (cells,
        // row-block tiles, level-0 tiles)
        int tl[D_COUNT];
        tiles(tl);
        const int partStride = std::max(tl[D_CELLS], std::max(tl[D_RB], tl[D_L0])) + 1;
        size_t off = 0;
        Scn<R>& s = h;
        s.blocked = carve<uint8_t>(base, off, N);
        s.fx = carve<R>(base, off, NX); s.fy = carve<R>(base, off, NY); s.fz = carve<R>(base, off, NZ);
        s.ax = carve<R>(base, off, NX); s.ay = carve<R>(base, off, NY); s.az = carve<R>(base, off, NZ);
        s.a0x = carve<R>(base, off, NX); s.a0y = carve<R>(base, off, NY); s.a0z = carve<R>(base, off, NZ);
        s.lx = geo.anyLeak ? carve<uint8_t>(base, off, NX) : nullptr;
        s.ly = geo.anyLeak ? carve<uint8_t>(base, off, NY) : nullptr;
        s.lz = geo.anyLeak ? carve<uint8_t>(base, off, NZ) : nullptr;
        s.diag = carve<R>(base, off, N);
        s.code0 = carve<unsigned char>(base, off, N);
        s.zone = carve<int>(base, off, N);
        const int nZ = (int)Z.zoneP.size(), nC = (int)Z.closed.size();
        s.zoneOpen = carve<uint8_t>(base, off, nZ + 1);
        s.closedZone = carve<int>(base, off, nC + 1);
        s.closedStart = carve<int>(base, off, nC + 1);
        s.closedCells = carve<int>(base, off, Z.closedCells.size() + 1);
        s.zoneP = carve<double>(base, off, nZ + 1);
        s.zoneVol = carve<double>(base, off, nZ + 1);
        s.zoneDP = carve<double>(base, off, nZ + 1);
        s.zoneShift = carve<double>(base, off, nZ + 1);
        s.zoneMean = carve<double>(base, off, nZ + 1);
        s.nLeak = (int)leak.size() / 4;
        s.leak = carve<int4>(base, off, s.nLeak + 1);
        s.leakZStart = carve<int>(base, off, leakZStart.size() + 1);
        s.leakZList = carve<int>(base, off, leakZList.size() + 1);
        s.leakQ = carve<double>(base, off, s.nLeak + 1);
        s.zonePnew = carve<double>(base, off, nZ + 1);
        s.zoneDInt = carve<double>(base, off, nZ + 1);
        s.u = carve<R>(base, off, NX); s.v = carve<R>(base, off, NY); s.w = carve<R>(base, off, NZ);
        s.u2 = carve<R>(base, off, NX); s.v2 = carve<R>(base, off, NY); s.w2 = carve<R>(base, off, NZ);
        for (int q = 0; q < NSC; ++q) { s.sc[q] = carve<R>(base, off, N); s.sc2[q] = carve<R>(base, off, N); }
        s.p = carve<R>(base, off, N); s.S = carve<R>(base, off, N); s.nu = carve<R>(base, off, N);
        s.Pb = carve<R>(base, off, N); s.Q = carve<R>(base, off, N); s.Qr = carve<R>(base, off, N);
        s.hrr = carve<R>(base, off, N); s.massSrc = carve<R>(base, off, N);
        s.lit = carve<uint8_t>(base, off, N); s.lit2 = carve<uint8_t>(base, off, N); s.pilot = carve<uint8_t>(base, off, N);
        for (int q = 0; q < 9; ++q) s.tmp[q] = carve<R>(base, off, N);
        s.adv = kMixed ? nullptr : carve<double>(base, off, (size_t)ADV_REC * (NX + NY + NZ));
        s.b = carve<R>(base, off, N); s.r = carve<R>(base, off, N); s.z = carve<R>(base, off, N);
        dbuf[0] = carve<R>(base, off, N); dbuf[1] = carve<R>(base, off, N);
        s.d = dbuf[0];
        s.q = carve<R>(base, off, N);
        s.p64 = kMixed ? carve<double>(base, off, N) : nullptr;
        s.p64prev = kMixed ? carve<double>(base, off, N) : nullptr;
        Level<R>& L0 = s.lv[0];
        L0.diag = s.diag;
        L0.x = s.z; L0.y = nullptr; L0.b = s.r;
        L0.rowStart = nullptr; L0.col = nullptr; L0.val = nullptr;
        L0.childStart = nullptr; L0.child = nullptr;
        s.sv = carve<double>(base, off, SV_COUNT);
        s.part = carve<double>(base, off, (size_t)PS_COUNT * partStride);
        s.partStride = partStride;
        s.cnt = carve<unsigned>(base, off, PS_COUNT + 4);
        return off + 256;
    }

    // the coarsest solve: the reference's 20 Gauss-Seidel sweep pairs on the FP64
    // path; on the mixed path the exact inverse of the coarsest matrix
    // (PHX_COARSE_EXACT=0: the reference's sweeps)
    static CoarseSolve coarseSolveFor() {
        CoarseSolve cs;
        if (kMixed) {
            static const bool exact = [] {
                const char* e = std::getenv("PHX_COARSE_EXACT");
                return !(e && std::atoi(e) == 0);
            }();
            cs.exact = exact;
        }
        return cs;
    }

    // the levels' arrays in their own arena: level 0's aggregation map, and per
    // coarser level its CSR rows, diagonal, iterate and scratch, child lists and,
    // at the coarsest level, the dense operator
    size_t layoutLevels(char* base) {
        const int nl = (int)MG.lv.size();
        size_t off = 0;
        Scn<R>& s = h;
        s.nLevels = nl;
        for (int l = 0; l < nl; ++l) {
            const MgLevel& L = MG.lv[l];
            Level<R>& D = s.lv[l];
            D.n = L.n;
            if (l > 0) {
                D.rowStart = carve<int>(base, off, L.rowStart.size());
                D.col = carve<int>(base, off, L.col.size() + 1);
                D.val = carve<R>(base, off, L.val.size() + 1);
                D.diag = carve<R>(base, off, L.n + 1);
                D.x = carve<R>(base, off, L.n + 1); D.y = carve<R>(base, off, L.n + 1); D.b = carve<R>(base, off, L.n + 1);
            }
            D.agg = L.agg.empty() ? nullptr : carve<int>(base, off, L.agg.size());
            D.childStart = (l == 0 || L.childStart.empty()) ? nullptr : carve<int>(base, off, L.childStart.size());
            D.child = (l == 0 || L.child.empty()) ? nullptr : carve<int>(base, off, L.child.size() + 1);
            D.dense = L.dense.empty() ? nullptr : carve<R>(base, off, L.dense.size());
        }
        return off + 256;
    }

    int allocate() {
        mainBytes = layoutMain(nullptr);
        mgBytes = layoutLevels(nullptr);
        arenaBytes = mainBytes + mgBytes;
        cudaError_t e = cudaMalloc(&arena, mainBytes);
        if (e == cudaSuccess) e = cudaMalloc(&mgArena, mgBytes);
        if (e != cudaSuccess) {
            cudaGetLastError();
            if (arena) cudaFree(arena);
            arena = nullptr;
            mgArena = nullptr;
            err = std::string("device allocation of ") + std::to_string(arenaBytes) + " bytes failed: " + cudaGetErrorString(e);
            return PHX_ERR_OOM;
        }
        layoutMain(arena);
        layoutLevels(mgArena);
        return PHX_OK;
    }

    // Replace the multigrid hierarchy by one built with another coarsening stop
    // (the V-cycle schedule): a new levels arena, uploaded; the fields and the
    // solve's state in the main arena are untouched. The caller rebuilds the
    // batch tables (the level domains change).
    int rebuildLevels(cudaStream_t st, int stop) {
        if (stop == coarseStop && mgArena) return PHX_OK;
        Multigrid M = buildMultigrid(geo, DENSE_MAX, stop, coarseSolveFor());
        PHX_CK(cudaStreamSynchronize(st));
        char* old = mgArena;
        MG = std::move(M);
        coarseStop = stop;
        mgBytes = layoutLevels(nullptr);
        char* fresh = nullptr;
        if (cudaMalloc(&fresh, mgBytes) != cudaSuccess) {
            cudaGetLastError();
            err = "device allocation of the multigrid levels failed";
            return PHX_ERR_OOM;
        }
        mgArena = fresh;
        arenaBytes = mainBytes + mgBytes;
        layoutLevels(mgArena);
        PHX_TRY(uploadLevels(st));
        if (old) cudaFree(old);
        return PHX_OK;
    }

    template <class T>
    int put(cudaStream_t st, const T* dstc, const std::vector<double>& src) {
        using U = typename std::remove_const<T>::type;
        U* dst = const_cast<U*>(dstc);
        std::vector<U> tmp(src.begin(), src.end());
        if (!tmp.empty()) PHX_CK(cudaMemcpyAsync(dst, tmp.data(), tmp.size() * sizeof(U), cudaMemcpyHostToDevice, st));
        PHX_CK(cudaStreamSynchronize(st));
        return PHX_OK;
    }
    template <class T, class V>
    int putRaw(cudaStream_t st, const T* dstc, const V* src, size_t n) {
        static_assert(sizeof(T) == sizeof(V), "element size");
        void* dst = const_cast<void*>((const void*)dstc);
        if (n) PHX_CK(cudaMemcpyAsync(dst, src, n * sizeof(T), cudaMemcpyHostToDevice, st));
        PHX_CK(cudaStreamSynchronize(st));
        return PHX_OK;
    }

    int upload(cudaStream_t st) {
        const int N = geo.N();
        Scn<R>& s = h;
        PHX_CK(cudaMemsetAsync(arena, 0, mainBytes, st));
        s.nx = geo.nx; s.ny = geo.ny; s.nz = geo.nz; s.N = N; s.NX = geo.NX(); s.NY = geo.NY(); s.NZ = geo.NZ();
        s.dvA[0] = makeDivU(geo.nx); s.dvB[0] = makeDivU(geo.nx * geo.ny); s.dY[0] = geo.ny;
        s.dvA[1] = makeDivU(geo.nx + 1); s.dvB[1] = makeDivU((geo.nx + 1) * geo.ny); s.dY[1] = geo.ny;
        s.dvA[2] = makeDivU(geo.nx); s.dvB[2] = makeDivU(geo.nx * (geo.ny + 1)); s.dY[2] = geo.ny + 1;
        s.dvL0[0] = makeDivU((geo.nx + 1) >> 1); s.dvL0[1] = makeDivU(((geo.nx + 1) >> 1) * ((geo.ny + 1) >> 1));
        s.dx = geo.dx; s.ox = geo.ox; s.oy = geo.oy; s.oz = geo.oz;
        {   // IEEE divisions in R: the values of the kernels' R(1) / dx
            const R dxr = (R)geo.dx;
            s.rdx = R(1) / dxr;
            s.rdx2 = R(1) / (dxr * dxr);
        }
        s.cfl = cfl; s.dtMaxP = dtMaxP; s.tol = tol; s.relTol = relTol; s.maxIters = maxIters; s.radiationOn = radiationOn;
        double th = geo.windFromDeg * 3.14159265 / 180.0;
        s.windSpeed = geo.windSpeed; s.windSin = std::sin(th); s.windCos = std::cos(th); s.windExp = geo.windExp;
        s.nZones = (int)Z.zoneP.size();
        s.nClosed = (int)Z.closed.size();
        s.mixed = kMixed ? 1 : 0;
        {   // PHX_REPLACE_EVERY=n: another interval, for measurements
            static const int every = [] {
                const char* e = std::getenv("PHX_REPLACE_EVERY");
                const int v = e ? std::atoi(e) : 0;
                return v >= 2 && v <= 100 ? v : REPLACE_EVERY;
            }();
            s.replaceEvery = every;
        }
        s.extrap = std::getenv("PHX_NO_EXTRAP") == nullptr;   // mixed path: extrapolated initial guess
        s.fp16Scratch = kMixed && std::getenv("PHX_FP16_SCRATCH") != nullptr;
        s.fp16Z0 = kMixed && std::getenv("PHX_FP16_Z0") != nullptr;
        s.tj = rowBlockRows<R>(geo.nx, geo.ny);
        s.njb = (geo.ny + s.tj - 1) / s.tj;
        PHX_TRY(putRaw(st, s.blocked, geo.blocked.data(), N));
        PHX_TRY(put(st, s.fx, geo.fx)); PHX_TRY(put(st, s.fy, geo.fy)); PHX_TRY(put(st, s.fz, geo.fz));
        PHX_TRY(put(st, s.ax, geo.ax)); PHX_TRY(put(st, s.ay, geo.ay)); PHX_TRY(put(st, s.az, geo.az));
        PHX_TRY(put(st, s.a0x, MG.a0x)); PHX_TRY(put(st, s.a0y, MG.a0y)); PHX_TRY(put(st, s.a0z, MG.a0z));
        PHX_TRY(put(st, s.diag, MG.lv[0].diag));
        {
            const std::vector<unsigned char> cd = levelZeroCodes();
            PHX_TRY(putRaw(st, s.code0, cd.data(), cd.size()));
        }
        PHX_TRY(putRaw(st, s.zone, Z.zone.data(), N));
        PHX_TRY(putRaw(st, s.zoneOpen, Z.zoneOpen.data(), Z.zoneOpen.size()));
        PHX_TRY(putRaw(st, s.closedZone, Z.closed.data(), Z.closed.size()));
        PHX_TRY(putRaw(st, s.closedStart, Z.closedStart.data(), Z.closedStart.size()));
        PHX_TRY(putRaw(st, s.closedCells, Z.closedCells.data(), Z.closedCells.size()));
        PHX_TRY(putRaw(st, s.zoneP, Z.zoneP.data(), Z.zoneP.size()));
        PHX_TRY(putRaw(st, s.zoneVol, Z.zoneVol.data(), Z.zoneVol.size()));
        if (geo.anyLeak) {
            PHX_TRY(putRaw(st, s.lx, geo.lx.data(), geo.lx.size()));
            PHX_TRY(putRaw(st, s.ly, geo.ly.data(), geo.ly.size()));
            PHX_TRY(putRaw(st, s.lz, geo.lz.data(), geo.lz.size()));
        }
        if (!leak.empty()) PHX_TRY(putRaw(st, s.leak, reinterpret_cast<const int4*>(leak.data()), leak.size() / 4));
        PHX_TRY(putRaw(st, s.leakZStart, leakZStart.data(), leakZStart.size()));
        PHX_TRY(putRaw(st, s.leakZList, leakZList.data(), leakZList.size()));
        // initial state (src/sim/discretize.cpp:28-31)
        const double amb[NSC] = {tStoredFromKd<R>(K_T0), K_YO2_AMB, 0, 0, 0, 0, K_YCO2_AMB, K_YH2O_AMB, 0, 0};
        for (int q = 0; q < NSC; ++q) {
            PHX_TRY(put(st, s.sc[q], std::vector<double>(N, amb[q])));
            PHX_TRY(put(st, s.sc2[q], std::vector<double>(N, amb[q])));
        }
        PHX_TRY(put(st, s.Pb, Pb0));
        return uploadLevels(st);
    }

    int uploadLevels(cudaStream_t st) {
        Scn<R>& s = h;
        PHX_CK(cudaMemsetAsync(mgArena, 0, mgBytes, st));
        for (int l = 1; l < (int)MG.lv.size(); ++l) {
            const MgLevel& L = MG.lv[l];
            Level<R>& D = s.lv[l];
            PHX_TRY(putRaw(st, D.rowStart, L.rowStart.data(), L.rowStart.size()));
            PHX_TRY(putRaw(st, D.col, L.col.data(), L.col.size()));
            PHX_TRY(put(st, D.val, L.val));
            PHX_TRY(put(st, D.diag, L.diag));
        }
        for (int l = 0; l < (int)MG.lv.size(); ++l) {
            const MgLevel& L = MG.lv[l];
            Level<R>& D = s.lv[l];
            if (D.agg) PHX_TRY(putRaw(st, D.agg, L.agg.data(), L.agg.size()));
            if (D.childStart) PHX_TRY(putRaw(st, D.childStart, L.childStart.data(), L.childStart.size()));
            if (D.child) PHX_TRY(putRaw(st, D.child, L.child.data(), L.child.size()));
            if (D.dense) PHX_TRY(put(st, D.dense, L.dense));
        }
        return PHX_OK;
    }

    // The level-0 coefficient code of every cell (level0.cuh): bits 0-5 for the
    // interior x-, x+, y-, y+, z-, z+ faces whose coefficient is exactly 1 (they
    // couple the cell to its neighbour), bit 7 for one open domain-boundary
    // face with coefficient 1 (it adds to the diagonal only), bit 6 when the
    // cell needs the arrays (a coefficient other than 0 or 1, two or more open
    // boundary faces, or a diagonal other than the count of its bits).
    std::vector<unsigned char> levelZeroCodes() const {
        const int nx = geo.nx, ny = geo.ny, nz = geo.nz;
        std::vector<unsigned char> cd(geo.N(), 0);
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i) {
                    const int c = geo.cell(i, j, k);
                    const double a[6] = {MG.a0x[geo.xface(i, j, k)], MG.a0x[geo.xface(i + 1, j, k)],
                                         MG.a0y[geo.yface(i, j, k)], MG.a0y[geo.yface(i, j + 1, k)],
                                         MG.a0z[geo.zface(i, j, k)], MG.a0z[geo.zface(i, j, k + 1)]};
                    const bool inner[6] = {i > 0, i < nx - 1, j > 0, j < ny - 1, k > 0, k < nz - 1};
                    unsigned bits = 0;
                    int boundary = 0;
                    bool general = false;
                    for (int f = 0; f < 6; ++f) {
                        if (a[f] == 1.0) {
                            if (inner[f]) bits |= 1u << f;
                            else ++boundary;
                        } else if (a[f] != 0.0) {
                            general = true;   // a fraction
                        }
                    }
                    if (boundary > 1) general = true;
                    int cnt = boundary;
                    for (int f = 0; f < 6; ++f) cnt += (bits >> f) & 1u;
                    if (MG.lv[0].diag[c] != (double)cnt) general = true;
                    cd[c] = general ? CODE_GENERAL : (unsigned char)(bits | (boundary ? CODE_BOUNDARY : 0u));
                }
        return cd;
    }

    // CTAs of each domain of this scenario
    void tiles(int* t) const {
        const int N = geo.N(), nx = geo.nx, ny = geo.ny, nz = geo.nz;
        auto cdiv = [](long long a, long long b) { return (int)((a + b - 1) / b); };
        for (int d = 0; d < D_COUNT; ++d) t[d] = 0;
        t[D_ONE] = 1;
        t[D_CELLS] = cdiv(N, TPB);
        t[D_RB] = cdiv(ny, rowBlockRows<R>(nx, ny)) * cdiv(nz, RB_KZ);      // row blocks x plane blocks
        t[D_L0] = l0Tiles(nx, ny, nz, 1);
        t[D_L0R] = l0Tiles(nx, ny, nz, l0Bpt(L0_RED));
        t[D_QUAD] = cdiv(N, TPB * CG_QUAD);                                 // 4 cells per thread
        t[D_LEAK] = cdiv((long long)leak.size() / 4, TPB);
        t[D_FX] = cdiv(geo.NX(), TPB);
        t[D_FY] = cdiv(geo.NY(), TPB);
        t[D_FZ] = cdiv(geo.NZ(), TPB);
        t[D_BX] = cdiv((long long)ny * nz * 2, TPB);
        t[D_BY] = cdiv((long long)nx * nz * 2, TPB);
        t[D_BZ] = cdiv((long long)nx * ny, TPB);
        t[D_CZ] = (int)Z.closed.size();
        t[D_CC] = cdiv((long long)Z.closedCells.size(), TPB);
        const int nl = (int)MG.lv.size();
        const MgLevel& Lc = MG.lv[nl - 1];
        t[D_CO_DENSE] = Lc.dense.empty() ? 0 : cdiv(Lc.n, TPB / 32);
        t[D_CO_SERIAL] = Lc.dense.empty() ? 1 : 0;
        for (int l = 1; l < MAX_LEVELS; ++l) {
            t[D_LV0 + l] = (l < nl - 1) ? cdiv(MG.lv[l].n, TPB) : 0;
            t[D_RS0 + l] = (l + 1 <= nl - 1) ? cdiv(MG.lv[l + 1].n, TPB / RRJ_LANES) : 0;   // 8 lanes per unknown
        }
    }
};

template <class R>
class Ctx : public CtxBase {
public:
    // the float instantiation is the mixed path: FP32 fields and stencils, FP64
    // refinement of the pressure solve, FP64 dots and global sums
    static constexpr bool kMixed = std::is_same<R, float>::value;

    std::vector<std::unique_ptr<Scenario<R>>> sc;
    cudaStream_t st = nullptr;
    // batch-wide device tables
    int cap = 0;                 // scenario capacity of the tables
    char* tab = nullptr;
    Scn<R>* dS = nullptr;        // descriptors
    R** dD = nullptr;            // CG direction buffers, 2 per scenario
    int* dDomStart = nullptr;    // D_COUNT x (cap + 1)
    double* dDtMax = nullptr;    // per-scenario dtMax of the step
    int* dLoop = nullptr;        // [0] iterations of the graph's CG while node, [1] runs of its replacement node
    int* dTiles = nullptr;       // [D_COUNT][cap] tiles of each scenario per domain
    int* dAStart = nullptr;      // [2][D_COUNT][cap + 1] active-tile prefixes (solving / replacing)
    int* dATotal = nullptr;      // [2][D_COUNT]
    unsigned* dErr = nullptr;    // error word of the device side (bounded waits that ran out)
    unsigned* ownTab = nullptr;  // CTA -> (scenario, tile) of every domain (Dom::owner)
    size_t ownCap = 0;
    double* dTimes = nullptr;    // simulated time of each scenario (read-back staging)
    int* dAllTotal = nullptr;    // the row-block tile total of the batch (every tile active), for tuning runs
    // launch shape of a row-block kernel: dynamic shared memory, persistent grid, slot strides
    struct RbCfg {
        size_t smem = 0;
        int grid = 0;
        RbShape shape{0, 0, 0};
    };
    RbCfg cfgApply, cfgGs[3], cfgRes;
    // the coded-coefficient level-0 kernels (level0.cuh) and their launch shape;
    // PHX_L0_ROWBLOCK=1 runs level 0 on the row-block kernels instead
    const bool l0Requested = std::getenv("PHX_L0_ROWBLOCK") == nullptr;
    bool useL0 = false;
    bool smoothOne = false;            // mixed path: one Jacobi sweep per coarse level and leg (vcycleSweeps)
    bool l0RedWide = false;            // the red sweep with L0_RED_WIDE blocks per thread
    int l0grid[L0_MODES + 1] = {};     // per pass; [L0_MODES]: the wide red sweep
    ADom adom[2][D_COUNT];
    double* hPin = nullptr;      // pinned scratch for read-backs
    Dom dom[D_COUNT];
    int maxLevels = 0;
    bool anyClosed = false;
    bool anyLeak = false;
    bool tablesDirty = true;
    int launches = 0;
    cudaEvent_t ev[4] = {};

    // radiation trace work space, grown on demand (traces are seconds of
    // simulated time apart)
    struct RadWork {
        enum { EL, WL, WALLI, ABS, WALLOF, CELLS, FLAGS, SOLIDT, GAS, KC, ELEMIS, RAYW, RAYVAL, RAYS, CNT, NBUF };
        int marchCtas = 0;
        void* buf[NBUF] = {};
        size_t cap[NBUF] = {};
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        double lastMs = 0;
        void release() {
            for (void* p : buf) if (p) cudaFree(p);
            if (e0) cudaEventDestroy(e0);
            if (e1) cudaEventDestroy(e1);
        }
    } rad;

    ~Ctx() override {
        if (st) cudaStreamSynchronize(st);
        rad.release();
        volw.release();
        destroyGraph();
        sc.clear();
        if (tab) cudaFree(tab);
        if (ownTab) cudaFree(ownTab);
        if (hPin) cudaFreeHost(hPin);
        if (flushBuf) cudaFree(flushBuf);
        for (auto e : evPool) cudaEventDestroy(e);
        for (auto& e : ev) if (e) cudaEventDestroy(e);
        if (st) cudaStreamDestroy(st);
    }

    int nscn() const { return (int)sc.size(); }

    int initStream() {
        if (st) return PHX_OK;
        PHX_CK(cudaGetDevice(&device));
        PHX_CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        PHX_CK(cudaMallocHost(&hPin, 8192 * sizeof(double)));
        for (auto& e : ev) PHX_CK(cudaEventCreate(&e));
        return PHX_OK;
    }

    // ---- membership ---------------------------------------------------------------
    int addScenario(const phx_grid* g, int* id) override {
        if (nscn() >= MAX_BATCH) { err = "batch is full (1024 scenarios)"; return PHX_ERR_BUDGET; }
        size_t bytes = 0;
        // validation and host set-up first: no device needed to reject bad input
        void* p = prepare(g, &bytes, err);
        if (!p) return lastPrepareStatus;
        return admit(p, id);
    }

    int lastPrepareStatus = PHX_OK;
    void* prepare(const phx_grid* g, size_t* bytes, std::string& e) override {
        auto s = std::make_unique<Scenario<R>>();
        const int r = s->setup(g);
        lastPrepareStatus = r;
        if (r != PHX_OK) { e = s->err; return nullptr; }
        if (bytes) *bytes = s->layout(nullptr);
        return s.release();
    }
    int admit(void* prepared, int* id) override {
        std::unique_ptr<Scenario<R>> s(static_cast<Scenario<R>*>(prepared));
        if (nscn() >= MAX_BATCH) { err = "batch is full (1024 scenarios)"; return PHX_ERR_BUDGET; }
        PHX_TRY(initStream());
        int r = s->allocate();
        if (r == PHX_OK) r = s->upload(st);
        if (r != PHX_OK) { err = s->err.empty() ? err : s->err; return r; }
        sc.push_back(std::move(s));
        if (id) *id = nscn() - 1;
        tablesDirty = true;
        return PHX_OK;
    }
    void discard(void* prepared) override { delete static_cast<Scenario<R>*>(prepared); }
    // Solver::traceRadiation (src/sim/radiation.cpp:181-319) for scenario s
    int radTrace(int s, const phx_rad_elem* el, int nE, const phx_rad_wall* wl, int nW, const double* solidT,
                 double* radAbs, double* radGas) override {
        PHX_TRY(checkScn(s));
        if (nE < 0 || nW < 0 || (nE > 0 && (!el || !radAbs)) || (nW > 0 && !wl)) {
            err = "invalid radiation trace arguments";
            return PHX_ERR_INVALID;
        }
        const Scenario<R>& S = *sc[s];
        const int nx = S.geo.nx, ny = S.geo.ny, nz = S.geo.nz;
        const size_t N = (size_t)nx * ny * nz;
        const size_t NF[3] = {(size_t)(nx + 1) * ny * nz, (size_t)nx * (ny + 1) * nz, (size_t)nx * ny * (nz + 1)};
        {   // at most one wall per face, every face in range
            std::vector<size_t> key(nW);
            for (int w = 0; w < nW; ++w) {
                if (wl[w].axis < 0 || wl[w].axis > 2 || wl[w].face < 0 || (size_t)wl[w].face >= NF[wl[w].axis]) {
                    err = "radiation wall " + std::to_string(w) + ": axis or face out of range";
                    return PHX_ERR_INVALID;
                }
                key[w] = (wl[w].axis == 0 ? 0 : wl[w].axis == 1 ? NF[0] : NF[0] + NF[1]) + (size_t)wl[w].face;
            }
            std::sort(key.begin(), key.end());
            for (int w = 1; w < nW; ++w)
                if (key[w] == key[w - 1]) { err = "two radiation walls on one face"; return PHX_ERR_INVALID; }
        }
        PHX_TRY(ensureTables());
        PHX_TRY(initStream());
        // buffer b holds at least `bytes` (device memory is allocated here only)
        auto grow = [&](int b, size_t bytes) -> int {
            bytes = std::max<size_t>(bytes, 16);
            if (rad.buf[b] && rad.cap[b] >= bytes) return PHX_OK;
            if (rad.buf[b]) { PHX_CK(cudaStreamSynchronize(st)); cudaFree(rad.buf[b]); rad.buf[b] = nullptr; rad.cap[b] = 0; }
            if (cudaMalloc(&rad.buf[b], bytes) != cudaSuccess) {
                cudaGetLastError();
                rad.buf[b] = nullptr;
                err = "out of device memory for the radiation trace";
                return PHX_ERR_OOM;
            }
            rad.cap[b] = bytes;
            return PHX_OK;
        };
        const size_t nF = NF[0] + NF[1] + NF[2];
        PHX_TRY(grow(RadWork::EL, nE * sizeof(phx_rad_elem)));
        PHX_TRY(grow(RadWork::ABS, nE * sizeof(double)));
        PHX_TRY(grow(RadWork::WL, nW * sizeof(phx_rad_wall)));
        PHX_TRY(grow(RadWork::WALLI, nW * 8 * sizeof(R)));
        PHX_TRY(grow(RadWork::WALLOF, nF * sizeof(int)));
        PHX_TRY(grow(RadWork::CELLS, N * sizeof(RadCell<R>)));
        PHX_TRY(grow(RadWork::FLAGS, N));
        PHX_TRY(grow(RadWork::SOLIDT, N * sizeof(double)));
        PHX_TRY(grow(RadWork::GAS, N * sizeof(R)));
        PHX_TRY(grow(RadWork::KC, sizeof(RadConst<R>)));
        PHX_TRY(grow(RadWork::ELEMIS, (size_t)nE * RAD_NB * sizeof(R)));
        PHX_TRY(grow(RadWork::RAYW, (size_t)nE * RAD_DIRS * sizeof(R)));
        PHX_TRY(grow(RadWork::RAYVAL, (size_t)nE * RAD_DIRS * sizeof(R)));
        PHX_TRY(grow(RadWork::RAYS, (size_t)nE * RAD_DIRS * sizeof(int)));
        PHX_TRY(grow(RadWork::CNT, 2 * sizeof(int)));
        if (!rad.marchCtas) {
            int dev = 0, sms = 0, per = 0;
            PHX_CK(cudaGetDevice(&dev));
            PHX_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
            PHX_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_rad_march<R>, 256, 0));
            rad.marchCtas = std::max(1, sms * std::max(1, per));
        }
        if (!rad.e0) {
            PHX_CK(cudaEventCreate(&rad.e0));
            PHX_CK(cudaEventCreate(&rad.e1));
        }
        phx_rad_elem* dEl = static_cast<phx_rad_elem*>(rad.buf[RadWork::EL]);
        phx_rad_wall* dWl = static_cast<phx_rad_wall*>(rad.buf[RadWork::WL]);
        R* dWallI = static_cast<R*>(rad.buf[RadWork::WALLI]);
        double* dAbs = static_cast<double*>(rad.buf[RadWork::ABS]);
        int* dWallOf = static_cast<int*>(rad.buf[RadWork::WALLOF]);
        RadCell<R>* dCells = static_cast<RadCell<R>*>(rad.buf[RadWork::CELLS]);
        uint8_t* dFlags = static_cast<uint8_t*>(rad.buf[RadWork::FLAGS]);
        double* dSolid = static_cast<double*>(rad.buf[RadWork::SOLIDT]);
        R* dGas = static_cast<R*>(rad.buf[RadWork::GAS]);
        RadConst<R>* dKc = static_cast<RadConst<R>*>(rad.buf[RadWork::KC]);
        R* dElemIs = static_cast<R*>(rad.buf[RadWork::ELEMIS]);
        R* dRayW = static_cast<R*>(rad.buf[RadWork::RAYW]);
        R* dRayVal = static_cast<R*>(rad.buf[RadWork::RAYVAL]);
        int* dRays = static_cast<int*>(rad.buf[RadWork::RAYS]);
        int* dCnt = static_cast<int*>(rad.buf[RadWork::CNT]);
        if (nE) PHX_CK(cudaMemcpyAsync(dEl, el, nE * sizeof(phx_rad_elem), cudaMemcpyHostToDevice, st));
        if (nW) PHX_CK(cudaMemcpyAsync(dWl, wl, nW * sizeof(phx_rad_wall), cudaMemcpyHostToDevice, st));
        if (solidT) PHX_CK(cudaMemcpyAsync(dSolid, solidT, N * sizeof(double), cudaMemcpyHostToDevice, st));
        PHX_CK(cudaMemsetAsync(dWallOf, 0xff, nF * sizeof(int), st));
        PHX_CK(cudaMemsetAsync(dGas, 0, N * sizeof(R), st));
        PHX_CK(cudaMemsetAsync(dCnt, 0, 2 * sizeof(int), st));
        PHX_CK(cudaEventRecord(rad.e0, st));
        k_rad_setup<R><<<1, 32, 0, st>>>(dKc);
        if (nW) k_rad_walls<R><<<(nW + 127) / 128, 128, 0, st>>>(dWl, nW, (int)NF[0], (int)NF[1], dWallOf, dWallI, dKc);
        k_rad_cells<R><<<(unsigned)((N + 255) / 256), 256, 0, st>>>(dS, s, solidT ? dSolid : nullptr, dCells, dFlags,
                                                                    dKc);
        if (nE) {
            k_rad_elems<R><<<(nE + RAD_WARPS - 1) / RAD_WARPS, RAD_WARPS * 32, 0, st>>>(
                dS, s, dEl, nE, dKc, dElemIs, dRayW, dRayVal, dRays, dCnt);
            k_rad_march<R><<<rad.marchCtas, 256, 0, st>>>(dS, s, dEl, dCells, dFlags, dWallOf, dWallI, dKc, dElemIs,
                                                          dRayW, dRayVal, dRays, dCnt, dGas);
            k_rad_absorbed<R><<<(nE + 255) / 256, 256, 0, st>>>(dRayVal, nE, dAbs);
        }
        PHX_CK(cudaGetLastError());
        PHX_CK(cudaEventRecord(rad.e1, st));
        if (nE) PHX_CK(cudaMemcpyAsync(radAbs, dAbs, nE * sizeof(double), cudaMemcpyDeviceToHost, st));
        std::vector<R> gasHost;
        if (radGas) {
            if (std::is_same<R, double>::value)
                PHX_CK(cudaMemcpyAsync(radGas, dGas, N * sizeof(double), cudaMemcpyDeviceToHost, st));
            else {
                gasHost.resize(N);
                PHX_CK(cudaMemcpyAsync(gasHost.data(), dGas, N * sizeof(R), cudaMemcpyDeviceToHost, st));
            }
        }
        PHX_CK(cudaStreamSynchronize(st));
        if (!gasHost.empty()) for (size_t c = 0; c < N; ++c) radGas[c] = (double)gasHost[c];
        float ms = 0;
        PHX_CK(cudaEventElapsedTime(&ms, rad.e0, rad.e1));
        rad.lastMs = ms;
        return checkDeviceError();
    }
    double radLastMs() const override { return rad.lastMs; }

    // one bounded wait that nothing satisfies: the failure path a timed-out
    // copy takes (error word, host report, context still usable)
    // ---- V-cycle schedule autotuner ----------------------------------------------
    // For each size bucket present in the batch (largest total first), every
    // candidate coarsening stop is applied to the bucket's scenarios and the
    // whole batch is stepped from the same saved state: one untimed step (the
    // step graph is rebuilt), then `steps` steps timed with CUDA events. Every
    // candidate solves to the same relative residual, so the fastest one
    // delivers the most cell-updates per second at equal residual; it is kept
    // and recorded in the process-wide table. The batch's state is restored at
    // the end. The FP64 path keeps the reference's schedule (its parity with
    // the reference needs the reference's V-cycle).
    int tuneVcycle(int steps, double dtMax, int* out, int cap) override {
        if (steps < 1 || steps > 50 || !(dtMax > 0)) { err = "invalid tuning arguments"; return PHX_ERR_INVALID; }
        auto report = [&]() {
            std::lock_guard<std::mutex> lock(vcycleMutex());
            for (int b = 0; b < cap && b < VC_BUCKETS && out; ++b) {
                const int v = vcycleTable()[b];
                out[b] = v > 0 ? v : MG_COARSE_STOP_REF;
            }
            if (out && cap > VC_BUCKETS) out[VC_BUCKETS] = kMixed ? vcycleSweeps() : 2;
        };
        if (!kMixed || nscn() == 0) { report(); return PHX_OK; }
        PHX_TRY(ensureTables());
        PHX_CK(cudaStreamSynchronize(st));
        // the batch's state: every scenario's main arena (fields, solve vectors, scalars)
        size_t snapBytes = 0;
        for (auto& S : sc) snapBytes += S->mainBytes;
        char* snap = nullptr;
        if (cudaMalloc(&snap, snapBytes) != cudaSuccess) {
            cudaGetLastError();
            err = "device allocation of the tuner's state copy failed";
            return PHX_ERR_OOM;
        }
        auto copyState = [&](bool save) -> int {
            size_t o = 0;
            for (auto& S : sc) {
                if (save) PHX_CK(cudaMemcpyAsync(snap + o, S->arena, S->mainBytes, cudaMemcpyDeviceToDevice, st));
                else PHX_CK(cudaMemcpyAsync(S->arena, snap + o, S->mainBytes, cudaMemcpyDeviceToDevice, st));
                o += S->mainBytes;
            }
            return PHX_OK;
        };
        // host descriptors: the swap state of the double buffers is part of the state
        std::vector<Scn<R>> hostSaved;
        for (auto& S : sc) hostSaved.push_back(S->h);
        auto restoreHost = [&]() {
            for (int i = 0; i < nscn(); ++i) {
                Scn<R>& h = sc[i]->h;
                const Scn<R>& o = hostSaved[i];
                h.u = o.u; h.v = o.v; h.w = o.w; h.u2 = o.u2; h.v2 = o.v2; h.w2 = o.w2;
                h.lit = o.lit; h.lit2 = o.lit2;
                for (int q = 0; q < NSC; ++q) { h.sc[q] = o.sc[q]; h.sc2[q] = o.sc2[q]; }
            }
        };
        int r = copyState(true);
        std::vector<long long> bucketCells(VC_BUCKETS, 0);
        for (auto& S : sc) bucketCells[vcycleBucket(S->geo.N())] += S->geo.N();
        std::vector<int> order;
        for (int b = 0; b < VC_BUCKETS; ++b) if (bucketCells[b] > 0) order.push_back(b);
        std::sort(order.begin(), order.end(), [&](int a, int b) { return bucketCells[a] > bucketCells[b]; });
        const int cands[] = {MG_COARSE_STOP_REF, 1000, 500};
        auto trial = [&](double* ms) -> int {
            PHX_TRY(copyState(false));
            restoreHost();
            tablesDirty = true;
            PHX_TRY(step(1, dtMax, nullptr, nullptr));
            double t = 0;
            int nl = 0;
            PHX_TRY(timeSteps(steps, dtMax, 0, &t, &nl));
            *ms = t;
            return PHX_OK;
        };
        // the coarse levels' smoothing first, one schedule for the batch (two Jacobi
        // sweeps per level and leg, the reference's, or one; PHX_COARSE_SWEEPS=1|2
        // fixes it), then the coarsening stop per size bucket
        auto setSweeps = [&](int v) {
            std::lock_guard<std::mutex> lock(vcycleMutex());
            vcycleSweeps() = v;
        };
        if (r == PHX_OK) {
            const char* fixed = std::getenv("PHX_COARSE_SWEEPS");
            if (fixed && (std::atoi(fixed) == 1 || std::atoi(fixed) == 2)) {
                setSweeps(std::atoi(fixed));
            } else {
                double ms2 = 0, ms1 = 0;
                setSweeps(2);
                r = trial(&ms2);
                if (r == PHX_OK) {
                    setSweeps(1);
                    r = trial(&ms1);
                }
                setSweeps(r == PHX_OK && ms1 < ms2 ? 1 : 2);
            }
        }
        for (int b : order) {
            if (r != PHX_OK) break;
            int best = MG_COARSE_STOP_REF;
            double bestMs = 1e300;
            for (int c : cands) {
                for (auto& S : sc)
                    if (vcycleBucket(S->geo.N()) == b && (r = S->rebuildLevels(st, c)) != PHX_OK) { err = S->err; break; }
                if (r != PHX_OK) break;
                double ms = 0;
                if ((r = trial(&ms)) != PHX_OK) break;
                if (ms < bestMs) { bestMs = ms; best = c; }
            }
            if (r != PHX_OK) break;
            for (auto& S : sc)
                if (vcycleBucket(S->geo.N()) == b && (r = S->rebuildLevels(st, best)) != PHX_OK) { err = S->err; break; }
            std::lock_guard<std::mutex> lock(vcycleMutex());
            vcycleTable()[b] = best;
        }
        if (r == PHX_OK) r = copyState(false);
        restoreHost();
        tablesDirty = true;
        cudaStreamSynchronize(st);
        cudaFree(snap);
        if (r != PHX_OK) return r;
        report();
        return checkDeviceError();
    }

    int selftestWait(double limitMs) override {
        if (!(limitMs > 0) || limitMs > 1000) { err = "self-test limit must be in (0, 1000] ms"; return PHX_ERR_INVALID; }
        PHX_TRY(ensureTables());
        PHX_TRY(initStream());
        int dev = 0, khz = 0;
        PHX_CK(cudaGetDevice(&dev));
        PHX_CK(cudaDeviceGetAttribute(&khz, cudaDevAttrClockRate, dev));
        const long long cycles = (long long)(limitMs * (double)std::max(khz, 1000000));
        k_selftest_wait<R><<<1, 32, 0, st>>>(dErr, cycles);
        PHX_CK(cudaGetLastError());
        PHX_CK(cudaStreamSynchronize(st));
        return checkDeviceError();
    }

    // the viewer's volume ray march for scenario s (src/render/renderer.cpp:119-283)
    struct VolWork {
        float4* vol = nullptr;
        size_t capVol = 0;
        float* depth = nullptr;
        float* rgb = nullptr;
        size_t capPix = 0;
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        double lastMs = 0;
        void release() {
            if (vol) cudaFree(vol);
            if (depth) cudaFree(depth);
            if (rgb) cudaFree(rgb);
            if (e0) cudaEventDestroy(e0);
            if (e1) cudaEventDestroy(e1);
        }
    } volw;

    int volRender(int s, const phx_vol_params* p, const float* depth, float* rgb) override {
        PHX_TRY(checkScn(s));
        if (!p || !rgb || p->width <= 0 || p->height <= 0 || (size_t)p->width * p->height > (size_t)1 << 26 ||
            p->n_lights < 0 || p->n_lights > 8 || !(p->step > 0)) {
            err = "invalid volume render parameters";
            return PHX_ERR_INVALID;
        }
        const Scenario<R>& S = *sc[s];
        const size_t N = (size_t)S.geo.nx * S.geo.ny * S.geo.nz, npx = (size_t)p->width * p->height;
        PHX_TRY(ensureTables());
        PHX_TRY(initStream());
        auto alloc = [&](auto*& ptr, size_t& cap, size_t n, size_t esz) -> int {
            if (ptr && cap >= n) return PHX_OK;
            if (ptr) { PHX_CK(cudaStreamSynchronize(st)); cudaFree(ptr); ptr = nullptr; cap = 0; }
            void* q = nullptr;
            if (cudaMalloc(&q, n * esz) != cudaSuccess) {
                cudaGetLastError();
                err = "out of device memory for the volume render";
                return PHX_ERR_OOM;
            }
            ptr = static_cast<std::remove_reference_t<decltype(ptr)>>(q);
            cap = n;
            return PHX_OK;
        };
        PHX_TRY(alloc(volw.vol, volw.capVol, N, sizeof(float4)));
        if (volw.capPix < npx || !volw.rgb) {
            size_t c1 = volw.capPix, c2 = volw.capPix;
            PHX_TRY(alloc(volw.rgb, c1, npx, 3 * sizeof(float)));
            PHX_TRY(alloc(volw.depth, c2, npx, sizeof(float)));
            volw.capPix = npx;
        }
        if (!volw.e0) { PHX_CK(cudaEventCreate(&volw.e0)); PHX_CK(cudaEventCreate(&volw.e1)); }
        if (depth) PHX_CK(cudaMemcpyAsync(volw.depth, depth, npx * sizeof(float), cudaMemcpyHostToDevice, st));
        VolGrid G;
        G.vol = volw.vol;
        G.nx = S.geo.nx; G.ny = S.geo.ny; G.nz = S.geo.nz;
        const float dxf = (float)S.geo.dx;
        G.bmin = v3((float)S.geo.ox, (float)S.geo.oy, (float)S.geo.oz);
        G.bmax = v3((float)S.geo.ox + G.nx * dxf, (float)S.geo.oy + G.ny * dxf, (float)S.geo.oz + G.nz * dxf);
        PHX_CK(cudaEventRecord(volw.e0, st));
        k_vol_pack<R><<<(unsigned)((N + 255) / 256), 256, 0, st>>>(dS, s, volw.vol);
        dim3 grid((p->width + 15) / 16, (p->height + 7) / 8);
        k_vol_render<R><<<grid, 128, 0, st>>>(G, *p, depth ? volw.depth : nullptr, volw.rgb);
        PHX_CK(cudaGetLastError());
        PHX_CK(cudaEventRecord(volw.e1, st));
        PHX_CK(cudaMemcpyAsync(rgb, volw.rgb, npx * 3 * sizeof(float), cudaMemcpyDeviceToHost, st));
        PHX_CK(cudaStreamSynchronize(st));
        float ms = 0;
        PHX_CK(cudaEventElapsedTime(&ms, volw.e0, volw.e1));
        volw.lastMs = ms;
        return checkDeviceError();
    }
    double volLastMs() const override { return volw.lastMs; }

    int readTimes(double* out) override {
        const int n = nscn();
        if (n == 0) return PHX_OK;
        PHX_TRY(ensureTables());
        k_read_times<R><<<(n + 127) / 128, 128, 0, st>>>(dS, n, dTimes);
        ++launches;
        PHX_CK(cudaMemcpyAsync(out, dTimes, n * sizeof(double), cudaMemcpyDeviceToHost, st));
        PHX_CK(cudaStreamSynchronize(st));
        return checkDeviceError();
    }

    int removeScenario(int s) override {
        if (s < 0 || s >= nscn()) { err = "no such scenario"; return PHX_ERR_INVALID; }
        PHX_CK(cudaStreamSynchronize(st));
        sc.erase(sc.begin() + s);
        tablesDirty = true;
        return PHX_OK;
    }

    int scenarioCount() const override { return nscn(); }
    size_t scenarioBytes(int s) const override { return s >= 0 && s < nscn() ? sc[s]->arenaBytes : 0; }

    // batch tables: descriptors, domain prefixes, CG buffers; invalidates the graph
    int rebuildTables() {
        destroyGraph();
        const int n = nscn();
        if (n > cap || !tab) {
            if (tab) { PHX_CK(cudaStreamSynchronize(st)); cudaFree(tab); tab = nullptr; }
            cap = std::max(n, std::max(1, cap * 2));
            char* base = nullptr;
            for (int pass = 0; pass < 2; ++pass) {
                size_t off = 0;
                dS = carve<Scn<R>>(base, off, cap);
                dD = carve<R*>(base, off, 2 * cap);
                dDomStart = carve<int>(base, off, (size_t)D_COUNT * (cap + 1));
                dDtMax = carve<double>(base, off, cap);
                dLoop = carve<int>(base, off, 4);
                dTiles = carve<int>(base, off, (size_t)D_COUNT * cap);
                dAStart = carve<int>(base, off, (size_t)2 * D_COUNT * (cap + 1));
                dATotal = carve<int>(base, off, 2 * D_COUNT);
                dErr = carve<unsigned>(base, off, 4);
                dTimes = carve<double>(base, off, cap);
                dAllTotal = carve<int>(base, off, 4);
                if (pass == 0) {
                    cudaError_t e = cudaMalloc(&tab, off + 256);
                    if (e != cudaSuccess) { tab = nullptr; err = "device allocation of the batch tables failed"; return PHX_ERR_OOM; }
                    PHX_CK(cudaMemsetAsync(tab, 0, off + 256, st));
                    base = tab;
                }
            }
        }
        std::vector<int> starts((size_t)D_COUNT * (n + 1), 0);
        std::vector<int> tilesAll((size_t)D_COUNT * cap, 0);
        std::vector<R*> dd(2 * std::max(n, 1), nullptr);
        maxLevels = 0;
        anyClosed = false;
        anyLeak = false;
        {
            std::lock_guard<std::mutex> lock(vcycleMutex());
            smoothOne = kMixed && vcycleSweeps() == 1;
        }
        RbShapes<R> shp;
        int t[D_COUNT];
        for (int s = 0; s < n; ++s) {
            Scenario<R>& S = *sc[s];
            S.tiles(t);
            for (int d = 0; d < D_COUNT; ++d) {
                starts[(size_t)d * (n + 1) + s + 1] = starts[(size_t)d * (n + 1) + s] + t[d];
                tilesAll[(size_t)d * cap + s] = t[d];
            }
            dd[2 * s] = S.dbuf[0];
            dd[2 * s + 1] = S.dbuf[1];
            maxLevels = std::max(maxLevels, (int)S.MG.lv.size());
            anyClosed |= !S.Z.closed.empty();
            anyLeak |= !S.leak.empty();
            S.h.dtMaxArg = dDtMax + s;
            S.h.errWord = dErr;
            S.h.smooth1 = smoothOne ? 1 : 0;
            shp.add(S.geo.nx, S.geo.ny);
        }
        // per domain, the scenario and tile of every CTA (packed 11 + 20 bits)
        size_t ownTotal = 0;
        bool packable = true;
        for (int d = 0; d < D_COUNT; ++d) {
            ownTotal += (size_t)starts[(size_t)d * (n + 1) + n];
            for (int s = 0; s < n; ++s) packable &= tilesAll[(size_t)d * cap + s] < (1 << 20);
        }
        std::vector<unsigned> own;
        if (packable && n <= 2048) {
            own.reserve(ownTotal);
            for (int d = 0; d < D_COUNT; ++d)
                for (int s = 0; s < n; ++s)
                    for (int t = 0; t < tilesAll[(size_t)d * cap + s]; ++t) own.push_back(((unsigned)s << 20) | (unsigned)t);
            if (own.size() > ownCap) {
                if (ownTab) { PHX_CK(cudaStreamSynchronize(st)); cudaFree(ownTab); ownTab = nullptr; ownCap = 0; }
                if (cudaMalloc(&ownTab, own.size() * sizeof(unsigned)) != cudaSuccess) {
                    ownTab = nullptr;
                    err = "device allocation of the CTA owner tables failed";
                    return PHX_ERR_OOM;
                }
                ownCap = own.size();
            }
            if (!own.empty())
                PHX_CK(cudaMemcpyAsync(ownTab, own.data(), own.size() * sizeof(unsigned), cudaMemcpyHostToDevice, st));
        }
        size_t ownOff = 0;
        for (int d = 0; d < D_COUNT; ++d) {
            dom[d].start = dDomStart + (size_t)d * (n + 1);
            dom[d].nscn = n;
            dom[d].total = starts[(size_t)d * (n + 1) + n];
            dom[d].owner = own.empty() ? nullptr : ownTab + ownOff;
            ownOff += (size_t)dom[d].total;
        }
        for (int k = 0; k < 2; ++k)
            for (int d = 0; d < D_COUNT; ++d) {
                adom[k][d].start = dAStart + (size_t)(k * D_COUNT + d) * (cap + 1);
                adom[k][d].total = dATotal + k * D_COUNT + d;
                adom[k][d].nscn = n;
            }
        persistCtas = PERSIST_CTAS;
        if (const char* cap = std::getenv("PHX_PERSIST_CTAS")) persistCtas = std::max(1, std::min(persistCtas, std::atoi(cap)));
        if (n > 0) {
            if (!shp.finish()) {
                err = "the batch's widest grids need more shared memory than a CTA has";
                return PHX_ERR_UNSUPPORTED;
            }
        }
        PHX_CK(cudaMemcpyAsync(dDomStart, starts.data(), starts.size() * sizeof(int), cudaMemcpyHostToDevice, st));
        PHX_CK(cudaMemcpyAsync(dTiles, tilesAll.data(), tilesAll.size() * sizeof(int), cudaMemcpyHostToDevice, st));
        if (n > 0) PHX_CK(cudaMemcpyAsync(dD, dd.data(), 2 * n * sizeof(R*), cudaMemcpyHostToDevice, st));
        tablesDirty = false;
        for (int s = 0; s < n; ++s) PHX_TRY(pushDescriptor(s, false));
        const int allTotal = dom[D_RB].total;
        PHX_CK(cudaMemcpyAsync(dAllTotal, &allTotal, sizeof(int), cudaMemcpyHostToDevice, st));
        PHX_CK(cudaStreamSynchronize(st));
        if (n > 0) PHX_TRY(tuneRowBlocks(shp));
        useL0 = false;
        if (n > 0 && l0Requested) PHX_TRY(setupL0());
        return PHX_OK;
    }

    // launch shape of the level-0 kernels: a persistent grid of as many CTAs
    // as fit on the SMs
    int setupL0() {
        int dev = 0, sms = 0;
        PHX_CK(cudaGetDevice(&dev));
        PHX_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        // Grid per pass: k times the resident CTAs, or (k = 0) one CTA per tile.
        // q = A d and the red sweep end every tile with a reduction of d.q or
        // r.z; one CTA per tile lets the SM overlap those of different tiles,
        // which a persistent CTA runs one after the other (mixed batch of 64:
        // 443 to 452 M cell-updates/s). The smoothing passes have no reduction
        // and run one persistent wave. PHX_L0_WAVES="k0,k1,k2,k3,k4" (in pass
        // order; one value sets all five) overrides this for measurements.
        static const std::array<int, L0_MODES> waves = [] {
            std::array<int, L0_MODES> w = {0, 1, 1, 1, 0};
            if (const char* e = std::getenv("PHX_L0_WAVES")) {
                int v[L0_MODES], n = 0;
                for (const char* c = e; *c && n < L0_MODES;) {
                    v[n++] = std::max(0, std::atoi(c));
                    while (*c && *c != ',') ++c;
                    if (*c == ',') ++c;
                }
                if (n > 0) for (int m = 0; m < L0_MODES; ++m) w[m] = v[n == 1 ? 0 : std::min(m, n - 1)];
            }
            return w;
        }();
        int residentWide = 0;   // CTAs of the four-block red sweep resident on the GPU at once
        auto one = [&](auto kern, int mode) -> int {
            int occ = 0;
            PHX_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, L0_THREADS, 0));
            const int k = waves[std::min(mode, L0_MODES - 1)];
            const int cap = persistCtas * TPB / L0_THREADS;   // PHX_PERSIST_CTAS caps every shape
            const int resident = std::min(sms * std::max(occ, 1), cap);
            if (mode == L0_MODES) residentWide = resident;
            l0grid[mode] = k == 0 ? (persistCtas < PERSIST_CTAS ? cap : (1 << 30)) : resident * k;
            return PHX_OK;
        };
        PHX_TRY(one(k_l0<R, L0_APPLY, 1>, L0_APPLY));
        PHX_TRY(one(k_l0<R, L0_PRE, 1>, L0_PRE));
        PHX_TRY(one(k_l0<R, L0_RES, 1>, L0_RES));
        PHX_TRY(one(k_l0<R, L0_BLACK, 1>, L0_BLACK));
        PHX_TRY(one(k_l0<R, L0_RED, 1>, L0_RED));
        PHX_TRY(one(k_l0<R, L0_RED, L0_RED_WIDE>, L0_MODES));
        // several blocks per thread only where the batch's wide tiles still fill
        // every CTA slot of the GPU twice (PHX_L0_RED_WIDE=0|1 forces it)
        static const int redWide = [] {
            const char* e = std::getenv("PHX_L0_RED_WIDE");
            return e ? std::atoi(e) : -1;
        }();
        l0RedWide = redWide >= 0 ? redWide == 1 : (long long)dom[D_L0R].total >= 2LL * residentWide;
        useL0 = true;
        return PHX_OK;
    }

    // a level-0 pass over the active level-0 tiles
    template <int MODE>
    void launchL0(const char* name, int phase) {
        if constexpr (MODE == L0_RED) {
            if (l0RedWide) {
                launchL0k<MODE, L0_RED_WIDE>(name, phase, D_L0R, l0grid[L0_MODES]);
                return;
            }
        }
        launchL0k<MODE, 1>(name, phase, D_L0, l0grid[MODE]);
    }
    template <int MODE, int BPT>
    void launchL0k(const char* name, int phase, int d, int gridCap) {
        {
            if (dom[d].total <= 0) return;
            const int grid = std::min(dom[d].total, gridCap);
            const Scn<R>* S = dS;
            R* const* D = (R* const*)dD;
            if (prof) {
                if (evNext + 2 > (int)evPool.size()) {
                    for (int i = 0; i < 64; ++i) { cudaEvent_t e; cudaEventCreate(&e); evPool.push_back(e); }
                }
                cudaEventRecord(evPool[evNext], st);
                k_l0<R, MODE, BPT><<<grid, L0_THREADS, 0, st>>>(S, adom[0][d], D, phase);
                cudaEventRecord(evPool[evNext + 1], st);
                evUse.push_back({name, evNext});
                evNext += 2;
            } else {
                k_l0<R, MODE, BPT><<<grid, L0_THREADS, 0, st>>>(S, adom[0][d], D, phase);
            }
            ++launches;
        }
    }

    // ---- launch shapes of the row-block kernels -----------------------------------------
    // The slot count of each kernel's staging ring (and with it how many CTAs
    // share an SM) is tuned on the batch itself: every candidate that fits an
    // SM's shared memory is timed on all tiles of the batch (the kernels only
    // write scratch that the next projection recomputes), and the fastest is
    // kept, cached per kernel and slot shape. The results do not depend on the
    // choice. PHX_NO_AUTOTUNE=1 takes the first candidate that fits two CTAs
    // per SM instead.
    std::map<std::string, int> tuneCache;
    int tuneRowBlocks(const RbShapes<R>& shp) {
        const Scn<R>* S = dS;
        const ADom all{dom[D_RB].start, dAllTotal, nscn()};
        PHX_TRY(tuneRB("apply", cfgApply, k_cg_apply_rb<R>, shp.apply, 0, ApplyLayout<R>::MIN_ST,
                       [&](const RbShape& sh, size_t smem, int grid) {
                           k_cg_apply_rb<R><<<grid, RB_THREADS, smem, st>>>(S, all, (R* const*)dD, sh);
                       }));
        PHX_TRY(tuneRB("gs_pre", cfgGs[GS_PRE], k_gs_rb<R, GS_PRE>, shp.gs[GS_PRE], 0, GsLayout<R, GS_PRE>::MIN_ST,
                       [&](const RbShape& sh, size_t smem, int grid) {
                           k_gs_rb<R, GS_PRE><<<grid, RB_THREADS, smem, st>>>(S, all, sh, 2);
                       }));
        PHX_TRY(tuneRB("gs_black", cfgGs[GS_BLACK], k_gs_rb<R, GS_BLACK>, shp.gs[GS_BLACK], 0,
                       GsLayout<R, GS_BLACK>::MIN_ST, [&](const RbShape& sh, size_t smem, int grid) {
                           k_gs_rb<R, GS_BLACK><<<grid, RB_THREADS, smem, st>>>(S, all, sh, 2);
                       }));
        PHX_TRY(tuneRB("gs_red", cfgGs[GS_RED], k_gs_rb<R, GS_RED>, shp.gs[GS_RED], 0, GsLayout<R, GS_RED>::MIN_ST,
                       [&](const RbShape& sh, size_t smem, int grid) {
                           k_gs_rb<R, GS_RED><<<grid, RB_THREADS, smem, st>>>(S, all, sh, 2);
                       }));
        PHX_TRY(tuneRB("res", cfgRes, k_res_rb<R>, shp.res, shp.resTail, ResLayout<R>::MIN_ST,
                       [&](const RbShape& sh, size_t smem, int grid) {
                           k_res_rb<R><<<grid, RB_THREADS, smem, st>>>(S, all, sh);
                       }));
        return PHX_OK;
    }

    template <class K, class Launch>
    int tuneRB(const char* name, RbCfg& c, K kern, RbShape shape, int tail, int minSt, Launch launchFn) {
        int dev = 0, sms = 0;
        PHX_CK(cudaGetDevice(&dev));
        PHX_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        const size_t maxSmem = RB_SM_SMEM - RB_STATIC_SMEM;
        PHX_CK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)maxSmem));
        std::vector<int> cands;
        for (int k = minSt; k <= RB_MAX_ST; ++k) {
            RbShape sh = shape;
            sh.st = k;
            if (rbSmem(sh, tail) <= maxSmem) cands.push_back(k);
        }
        if (cands.empty()) {
            err = std::string("the batch's widest grids need more shared memory than an SM has (") + name + ")";
            return PHX_ERR_UNSUPPORTED;
        }
        auto gridFor = [&](size_t smem, int* grid) -> int {
            int occ = 0;
            PHX_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, RB_THREADS, smem));
            *grid = std::min(sms * std::max(occ, 1), persistCtas);
            return PHX_OK;
        };
        // default: the deepest ring that still lets two CTAs share an SM, else one more slot than the minimum
        int best = cands.front() + (cands.size() > 1 ? 1 : 0);
        for (int k : cands) {
            RbShape sh = shape;
            sh.st = k;
            if (rbSmem(sh, tail) <= RB_SM_SMEM / 2 - RB_STATIC_SMEM) best = k;
        }
        const std::string key = std::string(name) + ":" + std::to_string(shape.slot) + ":" + std::to_string(shape.ring) +
                                ":" + std::to_string(tail);
        auto hit = tuneCache.find(key);
        if (hit != tuneCache.end()) {
            best = hit->second;
        } else if (std::getenv("PHX_NO_AUTOTUNE") == nullptr && dom[D_RB].total > 0 && cands.size() > 1) {
            float bestMs = 1e30f;
            for (int k : cands) {
                RbShape sh = shape;
                sh.st = k;
                const size_t smem = rbSmem(sh, tail);
                int grid = 0;
                PHX_TRY(gridFor(smem, &grid));
                grid = std::min(grid, dom[D_RB].total);
                launchFn(sh, smem, grid);
                PHX_CK(cudaEventRecord(ev[2], st));
                launchFn(sh, smem, grid);
                launchFn(sh, smem, grid);
                PHX_CK(cudaEventRecord(ev[3], st));
                PHX_CK(cudaEventSynchronize(ev[3]));
                float ms = 0;
                PHX_CK(cudaEventElapsedTime(&ms, ev[2], ev[3]));
                if (ms < bestMs) { bestMs = ms; best = k; }
            }
            PHX_TRY(checkLaunch());
            PHX_TRY(checkDeviceError());
            tuneCache[key] = best;
        }
        shape.st = best;
        c.shape = shape;
        c.smem = rbSmem(shape, tail);
        PHX_TRY(gridFor(c.smem, &c.grid));
        return PHX_OK;
    }

    int ensureTables() { return tablesDirty ? rebuildTables() : PHX_OK; }

    int pushDescriptor(int s, bool sync = true) {
        Scenario<R>& S = *sc[s];
        S.h.nsrc = (int)(S.ignitions.size() + S.burners.size());
        int q = 0;
        for (auto& x : S.ignitions) S.h.src[q++] = x;
        for (auto& x : S.burners) S.h.src[q++] = x;
        if (tablesDirty) return PHX_OK;   // uploaded with the tables
        PHX_CK(cudaMemcpyAsync(dS + s, &S.h, sizeof(Scn<R>), cudaMemcpyHostToDevice, st));
        if (sync) PHX_CK(cudaStreamSynchronize(st));
        return PHX_OK;
    }

    int checkScn(int s) {
        if (s < 0 || s >= nscn()) { err = "no such scenario"; return PHX_ERR_INVALID; }
        return PHX_OK;
    }

    // ---- sources ------------------------------------------------------------------
    int addBurner(int s, double x0, double y0, double x1, double y1, double z, double peakW, double rampS,
                  double start, double duration, int* index) override {
        if (index) *index = -1;
        PHX_TRY(checkScn(s));
        Scenario<R>& S = *sc[s];
        std::vector<int> cells = burnerCells(S.geo, x0, y0, x1, y1, z);
        if (cells.empty()) { err = "burner covers no gas cell"; return PHX_ERR_INVALID; }
        if ((int)(S.ignitions.size() + S.burners.size()) >= MAX_SRC) { err = "too many burners and ignitions (16)"; return PHX_ERR_INVALID; }
        Src b{};
        b.kind = 1;
        b.i0 = b.j0 = 1 << 30; b.i1 = b.j1 = -1; b.k = -1;
        for (int c : cells) {
            int i = c % S.geo.nx, j = (c / S.geo.nx) % S.geo.ny, k = c / (S.geo.nx * S.geo.ny);
            b.i0 = std::min(b.i0, i); b.i1 = std::max(b.i1, i); b.j0 = std::min(b.j0, j); b.j1 = std::max(b.j1, j);
            if (b.k >= 0 && b.k != k) { err = "burner cells span several layers"; return PHX_ERR_UNSUPPORTED; }
            b.k = k;
        }
        // the device selects the unblocked cells of the box: check that this is the same set
        size_t inBox = 0;
        for (int j = b.j0; j <= b.j1; ++j)
            for (int i = b.i0; i <= b.i1; ++i) inBox += !S.geo.blocked[S.geo.cell(i, j, b.k)];
        if (inBox != cells.size()) { err = "burner cells do not form a box of gas cells"; return PHX_ERR_UNSUPPORTED; }
        b.ncells = (int)cells.size();
        b.peakW = peakW; b.rampS = rampS; b.start = start; b.duration = duration;
        S.burners.push_back(b);
        if (index) *index = (int)S.burners.size() - 1;
        return pushDescriptor(s);
    }

    int addIgnition(int s, int cell, double power, double duration) override {
        PHX_TRY(checkScn(s));
        Scenario<R>& S = *sc[s];
        if (cell < 0 || cell >= S.geo.N()) return PHX_OK;   // the reference ignores it
        if ((int)(S.ignitions.size() + S.burners.size()) >= MAX_SRC) { err = "too many burners and ignitions (16)"; return PHX_ERR_INVALID; }
        PHX_CK(cudaMemcpyAsync(hPin, S.h.sv + SV_TIME, sizeof(double), cudaMemcpyDeviceToHost, st));
        PHX_CK(cudaStreamSynchronize(st));
        Src x{};
        x.kind = 0;
        x.i0 = x.i1 = cell % S.geo.nx; x.j0 = x.j1 = (cell / S.geo.nx) % S.geo.ny; x.k = cell / (S.geo.nx * S.geo.ny);
        x.ncells = 1;
        x.power = power; x.start = hPin[0]; x.duration = duration;
        S.ignitions.push_back(x);
        return pushDescriptor(s);
    }

    // ---- launch helpers -------------------------------------------------------------
    bool prof = false;
    std::vector<cudaEvent_t> evPool;
    std::vector<std::pair<const char*, int>> evUse;   // (kernel name, first event index)
    int evNext = 0;
    struct KStat { std::string name; int launches = 0; double ms = 0; };
    std::vector<KStat> kstats;
    void* flushBuf = nullptr;
    size_t flushBytes = 0;

    template <class K, class... A>
    void launch(const char* name, int d, int threads, K kern, A... args) {
        if (dom[d].total <= 0) return;
        if (prof) {
            if (evNext + 2 > (int)evPool.size()) {
                for (int i = 0; i < 64; ++i) { cudaEvent_t e; cudaEventCreate(&e); evPool.push_back(e); }
            }
            cudaEventRecord(evPool[evNext], st);
            kern<<<dom[d].total, threads, 0, st>>>(args...);
            cudaEventRecord(evPool[evNext + 1], st);
            evUse.push_back({name, evNext});
            evNext += 2;
        } else {
            kern<<<dom[d].total, threads, 0, st>>>(args...);
        }
        ++launches;
    }

    // persistent grid over the active tiles of domain d (solve kernels): 16 CTAs of 256
    // threads per SM of GB300 measured best on the 64-scenario batch (8: 274.5, 12: 278.5,
    // 16: 279.0, 32: 278.2 M cell-updates/s; a CTA per tile: 268.7)
    static constexpr int PERSIST_CTAS = 152 * 16;
    int persistCtas = PERSIST_CTAS;   // PHX_PERSIST_CTAS caps it (tests: many tiles per CTA)
    template <class K, class... A>
    void launchA(const char* name, int d, int threads, K kern, A... args) {
        if (dom[d].total <= 0) return;
        const int grid = std::min(dom[d].total, persistCtas);
        if (prof) {
            if (evNext + 2 > (int)evPool.size()) {
                for (int i = 0; i < 64; ++i) { cudaEvent_t e; cudaEventCreate(&e); evPool.push_back(e); }
            }
            cudaEventRecord(evPool[evNext], st);
            kern<<<grid, threads, 0, st>>>(args...);
            cudaEventRecord(evPool[evNext + 1], st);
            evUse.push_back({name, evNext});
            evNext += 2;
        } else {
            kern<<<grid, threads, 0, st>>>(args...);
        }
        ++launches;
    }

    // persistent grid over the active row-block tiles, with the staging ring in dynamic shared memory
    template <class K, class... A>
    void launchRB(const char* name, const RbCfg& c, K kern, A... args) {
        if (dom[D_RB].total <= 0) return;
        const int grid = std::min(dom[D_RB].total, c.grid);
        const size_t rbSmem = c.smem;
        if (prof) {
            if (evNext + 2 > (int)evPool.size()) {
                for (int i = 0; i < 64; ++i) { cudaEvent_t e; cudaEventCreate(&e); evPool.push_back(e); }
            }
            cudaEventRecord(evPool[evNext], st);
            kern<<<grid, RB_THREADS, rbSmem, st>>>(args...);
            cudaEventRecord(evPool[evNext + 1], st);
            evUse.push_back({name, evNext});
            evNext += 2;
        } else {
            kern<<<grid, RB_THREADS, rbSmem, st>>>(args...);
        }
        ++launches;
    }

    // the device error word: a bounded wait inside a kernel that ran out
    int checkDeviceError() {
        if (!dErr) return PHX_OK;
        unsigned w = 0;
        PHX_CK(cudaMemcpyAsync(&w, dErr, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
        PHX_CK(cudaStreamSynchronize(st));
        if (w) {
            // report once and clear, so that the context stays usable
            PHX_CK(cudaMemsetAsync(dErr, 0, sizeof(unsigned), st));
            PHX_CK(cudaStreamSynchronize(st));
            err = (w & 3u) ? "a staged shared-memory copy did not arrive within its time limit; the step's results are "
                             "not valid (device error word " + std::to_string(w) + ")"
                           : "a bounded device wait ran out (self-test, device error word " + std::to_string(w) + ")";
            return PHX_ERR_TIMEOUT;
        }
        return PHX_OK;
    }

    ActiveTables activeTables() const {
        ActiveTables t;
        t.tiles = dTiles;
        t.astart = dAStart;
        t.atotal = dATotal;
        t.nscn = nscn();
        t.cap = cap;
        t.ndom = D_COUNT;
        // the domains of the solve's persistent kernels (kind 0: solving, kind 1: replacing)
        int n = 0;
        auto add = [&](int kind, int d) { if (n < 32) t.list[n++] = (short)(kind * D_COUNT + d); };
        add(0, D_CELLS); add(0, D_CZ); add(0, D_RB); add(0, D_L0); add(0, D_L0R); add(0, D_QUAD); add(0, D_CO_DENSE); add(0, D_CO_SERIAL);
        for (int l = 1; l < maxLevels - 1 && l < MAX_LEVELS; ++l) { add(0, D_LV0 + l); add(0, D_RS0 + l); }
        add(1, D_CELLS); add(1, D_CZ);
        t.nlist = n;
        return t;
    }    void rebuildActive() {
        k_active<R><<<1, 256, 0, st>>>(dS, activeTables());
        ++launches;
    }

    int collectProfile() {
        PHX_CK(cudaStreamSynchronize(st));
        for (auto& u : evUse) {
            float ms = 0;
            cudaEventElapsedTime(&ms, evPool[u.second], evPool[u.second + 1]);
            KStat* k = nullptr;
            for (auto& x : kstats) if (x.name == u.first) k = &x;
            if (!k) { kstats.push_back(KStat{u.first, 0, 0}); k = &kstats.back(); }
            k->launches++;
            k->ms += ms;
        }
        evUse.clear();
        evNext = 0;
        return PHX_OK;
    }

    void swapHost(int what) {
        for (auto& S : sc) {
            Scn<R>& h = S->h;
            if (what & 1) std::swap(h.lit, h.lit2);
            if (what & 2) { std::swap(h.u, h.u2); std::swap(h.v, h.v2); std::swap(h.w, h.w2); }
            if (what & 4) for (int q = 0; q < NSC; ++q) std::swap(h.sc[q], h.sc2[q]);
        }
    }
    void swapBoth(int what) {
        launch("k_swap", D_ONE, 32, k_swap<R>, dS, dom[D_ONE], what);
        swapHost(what);
    }

    int setDtMax(double dtMax, const double* per) {
        std::vector<double> v(nscn(), dtMax);
        if (per) for (int s = 0; s < nscn(); ++s) v[s] = per[s];
        // pageable source: staged at the call, safe to reuse at once
        if (!v.empty()) PHX_CK(cudaMemcpyAsync(dDtMax, v.data(), v.size() * sizeof(double), cudaMemcpyHostToDevice, st));
        return PHX_OK;
    }

    // ---- stages ---------------------------------------------------------------------
    void stBegin(bool computeDt, double dt) {
        launch("k_begin", D_ONE, 32, k_begin<R>, (const Scn<R>*)dS, dom[D_ONE], computeDt ? 1 : 0, dt);
    }
    void stCombustion() {
        launch("k_combust", D_CELLS, TPB, k_combust<R>, (const Scn<R>*)dS, dom[D_CELLS]);
        swapBoth(1);
    }
    void stTurbulence() {
        const Scn<R>* S = dS;
        launch("k_turb_center", D_CELLS, TPB, k_turb_center<R>, S, dom[D_CELLS]);
        launch("k_turb_filter", D_CELLS, TPB, k_turb_filter<R, 0>, S, dom[D_CELLS]);
        launch("k_turb_filter", D_CELLS, TPB, k_turb_filter<R, 1>, S, dom[D_CELLS]);
        launch("k_turb_filter", D_CELLS, TPB, k_turb_filter<R, 2>, S, dom[D_CELLS]);
        launch("k_turb_nu", D_CELLS, TPB, k_turb_nu<R>, S, dom[D_CELLS]);
    }
    void stHeat() {
        if (!kMixed) {   // FP64: each interior face's conductive flux once
            launch("k_heat_faces", D_FX, TPB, k_heat_faces<R>, (const Scn<R>*)dS, dom[D_FX], 0);
            launch("k_heat_faces", D_FY, TPB, k_heat_faces<R>, (const Scn<R>*)dS, dom[D_FY], 1);
            launch("k_heat_faces", D_FZ, TPB, k_heat_faces<R>, (const Scn<R>*)dS, dom[D_FZ], 2);
        }
        launch("k_heat", D_CELLS, TPB, k_heat<R>, (const Scn<R>*)dS, dom[D_CELLS]);
    }
    void stEnergy() { launch("k_energy", D_CELLS, TPB, k_energy<R>, (const Scn<R>*)dS, dom[D_CELLS]); }
    void stMomentum() {
        const Scn<R>* S = dS;
        launch("k_momentum", D_FX, TPB, k_momentum<R, 0>, S, dom[D_FX]);
        launch("k_momentum", D_FY, TPB, k_momentum<R, 1>, S, dom[D_FY]);
        launch("k_momentum", D_FZ, TPB, k_momentum<R, 2>, S, dom[D_FZ]);
        launch("k_mom_bnd", D_BX, TPB, k_mom_bnd<R>, S, dom[D_BX], 0);
        launch("k_mom_bnd", D_BY, TPB, k_mom_bnd<R>, S, dom[D_BY], 1);
        launch("k_mom_bnd", D_BZ, TPB, k_mom_bnd<R>, S, dom[D_BZ], 2);
        swapBoth(2);
    }
    void stLeakage() {
        launch("k_zone_integral", D_CZ, TPB, k_zone_integral<R>, (const Scn<R>*)dS, dom[D_CZ]);
        if (anyLeak) {
            launch("k_leak_faces", D_LEAK, TPB, k_leak_faces<R>, (const Scn<R>*)dS, dom[D_LEAK]);
            launch("k_leak_finish", D_CZ, TPB, k_leak_finish<R>, (const Scn<R>*)dS, dom[D_CZ]);
        }
    }
    // one V-cycle z = M r (src/sim/pressure_mg.cpp:270-300) closed by the
    // last red half sweep with r.z; phase 0: before the CG loop, 1: inside
    // it, 2: a bare V-cycle
    void vcycle(int phase) {
        const Scn<R>* S = dS;
        if (useL0) {
            launchL0<L0_PRE>("k_gs_pre", phase);
            launchL0<L0_RES>("k_res_restrict", phase);
        } else {
            launchRB("k_gs_pre", cfgGs[GS_PRE], k_gs_rb<R, GS_PRE>, S, adom[0][D_RB], cfgGs[GS_PRE].shape, phase);
            launchRB("k_res_restrict", cfgRes, k_res_rb<R>, S, adom[0][D_RB], cfgRes.shape);
        }
        // down: level 1's first Jacobi sweep; then per level its second sweep (not
        // in the one-sweep schedule) and its residual restricted to level l+1 with
        // l+1's first sweep; up: per level the prolongating sweep and (two-sweep
        // schedule) a plain one
        if (!useL0) launchA("k_jacobi", D_LV0 + 1, TPB, k_jacobi<R>, S, adom[0][D_LV0 + 1], 1, 0);
        for (int l = 1; l < maxLevels - 1; ++l) {
            if (!smoothOne) launchA("k_jacobi", D_LV0 + l, TPB, k_jacobi<R>, S, adom[0][D_LV0 + l], l, 1);
            launchA("k_res_restrict_jac0", D_RS0 + l, TPB, k_res_restrict_jac0<R>, S, adom[0][D_RS0 + l], l);
        }
        launchA("k_coarse_dense", D_CO_DENSE, TPB, k_coarse_dense<R>, S, adom[0][D_CO_DENSE]);
        launchA("k_coarse_serial", D_CO_SERIAL, 32, k_coarse_serial<R>, S, adom[0][D_CO_SERIAL]);
        for (int l = maxLevels - 2; l >= 1; --l) {
            if (smoothOne) {
                launchA("k_jacobi", D_LV0 + l, TPB, k_jacobi<R>, S, adom[0][D_LV0 + l], l, 3);
            } else {
                launchA("k_jacobi", D_LV0 + l, TPB, k_jacobi<R>, S, adom[0][D_LV0 + l], l, 2);
                launchA("k_jacobi", D_LV0 + l, TPB, k_jacobi<R>, S, adom[0][D_LV0 + l], l, 1);
            }
        }
        if (useL0) {
            launchL0<L0_BLACK>("k_gs_black", phase);
            launchL0<L0_RED>("k_gs_red_dot", phase);
        } else {
            launchRB("k_gs_black", cfgGs[GS_BLACK], k_gs_rb<R, GS_BLACK>, S, adom[0][D_RB], cfgGs[GS_BLACK].shape, phase);
            launchRB("k_gs_red_dot", cfgGs[GS_RED], k_gs_rb<R, GS_RED>, S, adom[0][D_RB], cfgGs[GS_RED].shape, phase);
        }
    }
    // all scenarios' flag in slot `slot` set?
    int readAll(int slot, bool& all) {
        const int n = nscn();
        for (int s = 0; s < n; ++s)
            PHX_CK(cudaMemcpyAsync(hPin + 16 + s % 4000, sc[s]->h.sv + slot, sizeof(double), cudaMemcpyDeviceToHost, st));
        PHX_CK(cudaStreamSynchronize(st));
        all = true;
        for (int s = 0; s < n; ++s) all &= hPin[16 + s % 4000] != 0;
        return PHX_OK;
    }
    // Solver::project: right-hand side, first V-cycle and CG set-up
    void projectPrelude() {
        const Scn<R>* S = dS;
        launch("k_reset", D_ONE, 32, k_reset<R>, S, dom[D_ONE], 0);
        rebuildActive();
        launch("k_rhs", D_CELLS, TPB, k_rhs<R>, S, dom[D_CELLS]);
        vcycle(0);
    }
    // one CG iteration (src/sim/gasphase.cpp:605-625). The mixed path can
    // replace the recursive residual by the FP64 one before preconditioning,
    // so its first red half sweep runs after that.
    // The CG iteration in three parts: q = A d and the update; the mixed path's
    // residual replacement (in the step graph, a conditional node that runs it
    // only on iterations where some scenario replaces); the preconditioner.
    void cgIterUpdate(cudaGraphConditionalHandle repl, int setCond) {
        const Scn<R>* S = dS;
        if (useL0) {
            launchA("k_l0_dupdate", D_QUAD, TPB, k_l0_dupdate<R>, S, adom[0][D_QUAD], (R* const*)dD);
            launchL0<L0_APPLY>("k_cg_apply", 1);
        } else launchRB("k_cg_apply", cfgApply, k_cg_apply_rb<R>, S, adom[0][D_RB], (R* const*)dD, cfgApply.shape);
        launchA("k_cg_update", D_QUAD, TPB, k_cg_update<R>, S, adom[0][D_QUAD], (R* const*)dD, repl,
                (const int*)adom[1][D_CELLS].total, dLoop + 1, setCond);
        if (kMixed && anyClosed) launchA("k_mx_zone_center", D_CZ, TPB, k_mx_zone_center<R>, S, adom[0][D_CZ], 0);
    }
    void cgIterReplace() {
        const Scn<R>* S = dS;
        launchA("k_mx_update", D_CELLS, TPB, k_mx_update<R>, S, adom[1][D_CELLS], 1);
        launchA("k_mx_res64", D_CELLS, TPB, k_mx_res64<R>, S, adom[1][D_CELLS], 1);
        launchA("k_mx_zone_proj", D_CZ, TPB, k_mx_zone_proj<R>, S, adom[1][D_CZ], 1);
    }
    void cgIterPrecondition() {
        const Scn<R>* S = dS;
        vcycle(1);
        if (kMixed && anyClosed) launchA("k_mx_zone_center", D_CZ, TPB, k_mx_zone_center<R>, S, adom[0][D_CZ], 1);
    }
    // one CG iteration (src/sim/gasphase.cpp:605-625), launched kernel by kernel
    void cgIteration() {
        cgIterUpdate(cudaGraphConditionalHandle{}, 0);
        if (kMixed) cgIterReplace();
        cgIterPrecondition();
    }
    // zone mean removal and velocity correction (:629-676)
    void projectEpilogue() {
        const Scn<R>* S = dS;
        launch("k_zone_mean", D_CZ, TPB, k_zone_mean<R>, S, dom[D_CZ]);
        launch("k_zone_mean_sub", D_CC, TPB, k_zone_mean_sub<R>, S, dom[D_CC]);
        launch("k_velcorr", D_FX, TPB, k_velcorr<R>, S, dom[D_FX], 0);
        launch("k_velcorr", D_FY, TPB, k_velcorr<R>, S, dom[D_FY], 1);
        launch("k_velcorr", D_FZ, TPB, k_velcorr<R>, S, dom[D_FZ], 2);
    }
    // ---- mixed path: the FP32 CG starts from the FP64 residual b - A p64 ---------------
    void mixedPrelude() {
        const Scn<R>* S = dS;
        launch("k_reset", D_ONE, 32, k_reset<R>, S, dom[D_ONE], 0);
        rebuildActive();
        launch("k_mx_extrap", D_CELLS, TPB, k_mx_extrap<R>, S, dom[D_CELLS]);
        launch("k_rhs", D_CELLS, TPB, k_rhs<R>, S, dom[D_CELLS]);
        launchA("k_mx_res64", D_CELLS, TPB, k_mx_res64<R>, S, adom[0][D_CELLS], 0);
        launchA("k_mx_zone_proj", D_CZ, TPB, k_mx_zone_proj<R>, S, adom[0][D_CZ], 0);
        vcycle(0);
        if (anyClosed) launchA("k_mx_zone_center", D_CZ, TPB, k_mx_zone_center<R>, S, adom[0][D_CZ], 1);
    }
    void mixedEpilogue() {
        launch("k_mx_final", D_CELLS, TPB, k_mx_final<R>, dS, dom[D_CELLS]);
    }

    int maxItersAll() const {
        int m = 0;
        for (auto& S : sc) m = std::max(m, S->maxIters);
        return m;
    }

    // host-driven CG loop: the stop test is read back after every iteration
    int stProject() {
        if (kMixed) mixedPrelude();
        else projectPrelude();
        const int maxIt = maxItersAll();
        bool done = false;
        PHX_TRY(readAll(SV_DONE, done));
        for (int it = 0; !done && it <= maxIt + 1; ++it) {
            rebuildActive();
            cgIteration();
            PHX_TRY(readAll(SV_DONE, done));
        }
        if (kMixed) mixedEpilogue();
        projectEpilogue();
        return PHX_OK;
    }
    void stAdvect() {
        if (!kMixed) {
            launch("k_adv_faces", D_FX, TPB, k_adv_faces<R>, (const Scn<R>*)dS, dom[D_FX], 0);
            launch("k_adv_faces", D_FY, TPB, k_adv_faces<R>, (const Scn<R>*)dS, dom[D_FY], 1);
            launch("k_adv_faces", D_FZ, TPB, k_adv_faces<R>, (const Scn<R>*)dS, dom[D_FZ], 2);
        }
        launch("k_advect", D_CELLS, TPB, kMixed ? k_advect<R> : k_advect_2cta<R>, (const Scn<R>*)dS, dom[D_CELLS]);
        swapBoth(4);
    }
    void stEnd() {
        const Scn<R>* S = dS;
        launch("k_zone_pressure", D_ONE, 32, k_zone_pressure<R>, S, dom[D_ONE]);
        launch("k_zone_pb", D_CC, TPB, k_zone_pb<R>, S, dom[D_CC]);
        launch("k_stats", D_CELLS, TPB, k_stats<R>, S, dom[D_CELLS]);
    }

    int checkLaunch() {
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) { err = std::string("kernel launch: ") + cudaGetErrorString(e); return PHX_ERR_CUDA; }
        return PHX_OK;
    }

    // ---- captured step graph: the CG loops are device-side while nodes ---------------
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    cudaGraphConditionalHandle cgHandle{};
    int outerKernels = 0, bodyKernels = 0, replKernels = 0;
    // the step runs as one CUDA graph; PHX_NO_GRAPH=1 launches the same kernels
    // one by one (kernels inside conditional graphs cannot be profiled by ncu)
    bool useGraph = std::getenv("PHX_NO_GRAPH") == nullptr;

    void destroyGraph() {
        if (gexec) cudaGraphExecDestroy(gexec);
        if (graph) cudaGraphDestroy(graph);
        gexec = nullptr;
        graph = nullptr;
    }

    // add a conditional node (while or if) after the current capture position of
    // st (which captures into graph g); capture continues after it
    int addConditional(cudaGraph_t g, cudaGraphConditionalHandle handle, cudaGraphConditionalNodeType type,
                       cudaGraph_t* body) {
        cudaStreamCaptureStatus cs;
        const cudaGraphNode_t* deps = nullptr;
        size_t ndeps = 0;
        PHX_CK(cudaStreamGetCaptureInfo(st, &cs, nullptr, nullptr, &deps, nullptr, &ndeps));
        cudaGraphNodeParams cp = {};
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = handle;
        cp.conditional.type = type;
        cp.conditional.size = 1;
        cudaGraphNode_t cond;
        PHX_CK(cudaGraphAddNode(&cond, g, deps, nullptr, ndeps, &cp));
        *body = cp.conditional.phGraph_out[0];
        PHX_CK(cudaStreamUpdateCaptureDependencies(st, &cond, nullptr, 1, cudaStreamSetCaptureDependencies));
        return PHX_OK;
    }

    int buildGraph() {
        destroyGraph();
        std::vector<Scn<R>> saved;
        for (auto& S : sc) saved.push_back(S->h);
        const int n = nscn();
        PHX_CK(cudaGraphCreate(&graph, 0));
        // conditional handles are created before the capture of the graph that holds their node
        PHX_CK(cudaGraphConditionalHandleCreate(&cgHandle, graph, 0, 0));
        PHX_CK(cudaStreamBeginCaptureToGraph(st, graph, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
        launches = 0;
        stBegin(true, 0.0);
        stCombustion();
        stTurbulence();
        stHeat();
        stEnergy();
        stMomentum();
        stLeakage();
        if (kMixed) mixedPrelude();
        else projectPrelude();
        cudaMemsetAsync(dLoop, 0, 2 * sizeof(int), st);
        const int capIt = maxItersAll() + 2;
        k_cg_cond<R><<<1, 256, 0, st>>>(dS, n, cgHandle, dLoop, capIt, activeTables(), 1);
        ++launches;
        cudaGraph_t body = nullptr;
        PHX_TRY(addConditional(graph, cgHandle, cudaGraphCondTypeWhile, &body));
        if (kMixed) mixedEpilogue();
        projectEpilogue();
        stAdvect();
        stEnd();
        cudaGraph_t outGraph = nullptr;
        PHX_CK(cudaStreamEndCapture(st, &outGraph));
        outerKernels = launches;
        // the loop body; the mixed path's residual replacement is a conditional
        // node of it, set by k_cg_update on each iteration
        cudaGraphConditionalHandle replHandle{};
        cudaGraph_t replBody = nullptr;
        if (kMixed) PHX_CK(cudaGraphConditionalHandleCreate(&replHandle, body, 0, 0));
        PHX_CK(cudaStreamBeginCaptureToGraph(st, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
        launches = 0;
        cgIterUpdate(replHandle, kMixed ? 1 : 0);
        if (kMixed) PHX_TRY(addConditional(body, replHandle, cudaGraphCondTypeIf, &replBody));
        cgIterPrecondition();
        k_cg_cond<R><<<1, 256, 0, st>>>(dS, n, cgHandle, dLoop, capIt, activeTables(), 1);
        ++launches;
        PHX_CK(cudaStreamEndCapture(st, &body));
        bodyKernels = launches;
        replKernels = 0;
        if (kMixed) {
            PHX_CK(cudaStreamBeginCaptureToGraph(st, replBody, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
            launches = 0;
            cgIterReplace();
            PHX_CK(cudaStreamEndCapture(st, &replBody));
            replKernels = launches;
        }
        for (int s = 0; s < n; ++s) sc[s]->h = saved[s];
        PHX_CK(cudaGraphInstantiate(&gexec, graph, 0));
        return checkLaunch();
    }

    int graphStep(double dtMax, const double* per) {
        if (!gexec) PHX_TRY(buildGraph());
        PHX_TRY(setDtMax(dtMax, per));
        PHX_CK(cudaGraphLaunch(gexec, st));
        swapHost(1 | 2 | 4);
        return PHX_OK;
    }

    // kernels the last graph step ran: the outer nodes plus the loop body per iteration
    int graphLaunchCount(int* out) {
        int lc[2] = {0, 0};
        PHX_CK(cudaMemcpyAsync(lc, dLoop, 2 * sizeof(int), cudaMemcpyDeviceToHost, st));
        PHX_CK(cudaStreamSynchronize(st));
        *out = outerKernels + bodyKernels * std::max(0, lc[0] - 1) + replKernels * lc[1];
        return PHX_OK;
    }

    int oneStep(double dtMax, const double* per = nullptr) {
        PHX_TRY(ensureTables());
        if (nscn() == 0) return PHX_OK;
        if (useGraph && !prof) return graphStep(dtMax, per);
        PHX_TRY(setDtMax(dtMax, per));
        stBegin(true, 0.0);
        stCombustion();
        stTurbulence();
        stHeat();
        stEnergy();
        stMomentum();
        stLeakage();
        PHX_TRY(stProject());
        stAdvect();
        stEnd();
        return checkLaunch();
    }

    int step(int n, double dtMax, const double* per, double* dtOut) override {
        for (int i = 0; i < n; ++i) {
            launches = 0;
            PHX_TRY(oneStep(dtMax, per));
            if (dtOut) {
                const int m = nscn();
                for (int s = 0; s < m; ++s)
                    PHX_CK(cudaMemcpyAsync(hPin + 16 + s % 4000, sc[s]->h.sv + SV_DT, sizeof(double), cudaMemcpyDeviceToHost, st));
                PHX_CK(cudaStreamSynchronize(st));
                if (per) for (int s = 0; s < m; ++s) dtOut[(size_t)i * m + s] = hPin[16 + s % 4000];
                else dtOut[i] = hPin[16];
                PHX_TRY(checkDeviceError());
            }
        }
        return PHX_OK;
    }

    int stage(int which, double arg) override {
        PHX_TRY(ensureTables());
        switch (which) {
        case PHX_STAGE_BEGIN: PHX_TRY(setDtMax(arg, nullptr)); stBegin(true, 0.0); break;
        case PHX_STAGE_COMBUSTION: stBegin(false, arg); stCombustion(); break;
        case PHX_STAGE_TURBULENCE: stTurbulence(); break;
        case PHX_STAGE_HEAT: stBegin(false, arg); stHeat(); break;
        case PHX_STAGE_ENERGY: stBegin(false, arg); stEnergy(); break;
        case PHX_STAGE_MOMENTUM: stBegin(false, arg); stMomentum(); break;
        case PHX_STAGE_LEAKAGE: stBegin(false, arg); stLeakage(); break;
        case PHX_STAGE_PROJECT: stBegin(false, arg); PHX_TRY(stProject()); break;
        case PHX_STAGE_ADVECT: stBegin(false, arg); stAdvect(); break;
        case PHX_STAGE_END: stBegin(false, arg); stEnd(); break;
        default: err = "unknown stage"; return PHX_ERR_INVALID;
        }
        PHX_TRY(checkLaunch());
        PHX_CK(cudaStreamSynchronize(st));
        return PHX_OK;
    }

    // z = M^-1 r with one V-cycle of the multigrid (single-scenario contexts)
    int precondition(const double* r, double* z) override {
        PHX_TRY(ensureTables());
        if (nscn() != 1) { err = "precondition needs a single-scenario context"; return PHX_ERR_STATE; }
        Scenario<R>& S = *sc[0];
        const int N = S.geo.N();
        PHX_TRY(S.put(st, S.h.r, std::vector<double>(r, r + N)));
        launch("k_reset", D_ONE, 32, k_reset<R>, (const Scn<R>*)dS, dom[D_ONE], 2);
        rebuildActive();
        vcycle(2);
        PHX_TRY(checkLaunch());
        return getReal(S.h.z, N, z);
    }

    // ---- fields -----------------------------------------------------------------------
    int getReal(const R* src, size_t n, double* out) {
        if (std::is_same<R, double>::value) {
            PHX_CK(cudaMemcpyAsync(out, src, n * sizeof(double), cudaMemcpyDeviceToHost, st));
            PHX_CK(cudaStreamSynchronize(st));
            return PHX_OK;
        }
        std::vector<R> tmp(n);
        PHX_CK(cudaMemcpyAsync(tmp.data(), src, n * sizeof(R), cudaMemcpyDeviceToHost, st));
        PHX_CK(cudaStreamSynchronize(st));
        for (size_t i = 0; i < n; ++i) out[i] = (double)tmp[i];
        return PHX_OK;
    }

    bool fieldPtr(int s, int f, void** p, size_t* n, int* type) const {
        if (s < 0 || s >= nscn()) return false;
        const Scenario<R>& S = *sc[s];
        const Scn<R>& h = S.h;
        const size_t N = S.geo.N(), NX = S.geo.NX(), NY = S.geo.NY(), NZ = S.geo.NZ();
        *type = 0;
        switch (f) {
        case PHX_FIELD_U: *p = h.u; *n = NX; return true;
        case PHX_FIELD_V: *p = h.v; *n = NY; return true;
        case PHX_FIELD_W: *p = h.w; *n = NZ; return true;
        case PHX_FIELD_P: *p = h.p; *n = N; return true;
        case PHX_FIELD_S: *p = h.S; *n = N; return true;
        case PHX_FIELD_NU: *p = h.nu; *n = N; return true;
        case PHX_FIELD_PB: *p = h.Pb; *n = N; return true;
        case PHX_FIELD_Q: *p = h.Q; *n = N; return true;
        case PHX_FIELD_QR: *p = h.Qr; *n = N; return true;
        case PHX_FIELD_HRR: *p = h.hrr; *n = N; return true;
        case PHX_FIELD_MASSSRC: *p = h.massSrc; *n = N; return true;
        case PHX_FIELD_RHS: *p = h.b; *n = N; return true;
        case PHX_FIELD_CGR: *p = h.r; *n = N; return true;
        case PHX_FIELD_CGZ: *p = h.z; *n = N; return true;
        case PHX_FIELD_LIT: *p = h.lit; *n = N; *type = 1; return true;
        case PHX_FIELD_ZONE: *p = (void*)h.zone; *n = N; *type = 2; return true;
        case PHX_FIELD_ZONEP: *p = (void*)h.zoneP; *n = S.Z.zoneP.size(); *type = 3; return true;
        default:
            if (f >= PHX_FIELD_T && f <= PHX_FIELD_YAI) { *p = h.sc[f - PHX_FIELD_T]; *n = N; return true; }
            return false;
        }
    }

    size_t fieldCount(int s, int f) const override {
        void* p;
        size_t n;
        int t;
        return fieldPtr(s, f, &p, &n, &t) ? n : 0;
    }

    int getField(int s, int f, void* host, size_t bytes) override {
        void* p;
        size_t n;
        int t;
        if (!fieldPtr(s, f, &p, &n, &t)) { err = "unknown field or scenario"; return PHX_ERR_INVALID; }
        size_t want = n * (t == 0 || t == 3 ? sizeof(double) : t == 1 ? 1 : 4);
        if (bytes != want) { err = "field size mismatch: expected " + std::to_string(want) + " bytes"; return PHX_ERR_INVALID; }
        if (kMixed && f == PHX_FIELD_P) {   // the FP64 pressure of the refinement loop
            PHX_CK(cudaMemcpyAsync(host, sc[s]->h.p64, bytes, cudaMemcpyDeviceToHost, st));
            PHX_CK(cudaStreamSynchronize(st));
            return PHX_OK;
        }
        if (t == 0) {
            PHX_TRY(getReal((const R*)p, n, (double*)host));
            if (tempIsOffset<R>() && f == PHX_FIELD_T)   // the stored offset back to kelvin, in FP64
                for (size_t i = 0; i < n; ++i) ((double*)host)[i] = tKFromStoredd<R>(((double*)host)[i]);
            return PHX_OK;
        }
        PHX_CK(cudaMemcpyAsync(host, p, bytes, cudaMemcpyDeviceToHost, st));
        PHX_CK(cudaStreamSynchronize(st));
        return PHX_OK;
    }

    int setField(int s, int f, const void* host, size_t bytes) override {
        void* p;
        size_t n;
        int t;
        if (!fieldPtr(s, f, &p, &n, &t) || f == PHX_FIELD_ZONE) { err = "unknown or read-only field"; return PHX_ERR_INVALID; }
        size_t want = n * (t == 0 || t == 3 ? sizeof(double) : t == 1 ? 1 : 4);
        if (bytes != want) { err = "field size mismatch: expected " + std::to_string(want) + " bytes"; return PHX_ERR_INVALID; }
        Scenario<R>& S = *sc[s];
        if (t == 0) {
            const double* d = (const double*)host;
            if (kMixed && f == PHX_FIELD_P) {
                PHX_TRY(S.putRaw(st, S.h.p64, d, n));
                const double zero = 0;   // the previous step's pressure no longer applies
                PHX_CK(cudaMemcpyAsync(S.h.sv + SV_HAVEPREV, &zero, sizeof(double), cudaMemcpyHostToDevice, st));
                PHX_CK(cudaStreamSynchronize(st));
            }
            std::vector<double> v(d, d + n);
            if (tempIsOffset<R>() && f == PHX_FIELD_T)   // kelvin to the stored offset, in FP64
                for (auto& x : v) x = tStoredFromKd<R>(x);
            return S.put(st, (R*)p, v);
        }
        PHX_CK(cudaMemcpyAsync(p, host, bytes, cudaMemcpyHostToDevice, st));
        PHX_CK(cudaStreamSynchronize(st));
        return PHX_OK;
    }

    int getStats(int s, phx_stats* o) override {
        PHX_TRY(checkScn(s));
        PHX_CK(cudaMemcpyAsync(hPin + 4096, sc[s]->h.sv, SV_COUNT * sizeof(double), cudaMemcpyDeviceToHost, st));
        PHX_CK(cudaStreamSynchronize(st));
        const double* sv = hPin + 4096;
        o->time = sv[SV_TIME]; o->dt = sv[SV_DT];
        o->max_vel = sv[SV_MAXVEL]; o->max_nu = sv[SV_MAXNU]; o->max_div = sv[SV_MAXDIV];
        o->pressure_iters = (int)sv[SV_IT];
        o->pressure_residual = sv[SV_PRES]; o->pressure_rel_residual = sv[SV_PREL];
        o->hrr = sv[SV_HRR]; o->max_gas_t = sv[SV_MAXGAST]; o->burning_cells = (int)sv[SV_BURNING];
        o->fuel_in = sv[SV_FUELIN]; o->fuel_burned = sv[SV_FUELBURNED]; o->fuel_in_domain = sv[SV_FUELINDOMAIN];
        o->zones = (int)sc[s]->Z.zoneP.size(); o->leak_faces = (int)sc[s]->leak.size() / 4;
        return PHX_OK;
    }

    int setScalars(int s, double time, double maxVel, double maxNu, double maxDiv) override {
        PHX_TRY(checkScn(s));
        double v[4] = {time, maxVel, maxNu, maxDiv};
        double* sv = sc[s]->h.sv;
        PHX_CK(cudaMemcpyAsync(sv + SV_TIME, &v[0], sizeof(double), cudaMemcpyHostToDevice, st));
        PHX_CK(cudaMemcpyAsync(sv + SV_MAXVEL, &v[1], sizeof(double), cudaMemcpyHostToDevice, st));
        PHX_CK(cudaMemcpyAsync(sv + SV_MAXNU, &v[2], sizeof(double), cudaMemcpyHostToDevice, st));
        PHX_CK(cudaMemcpyAsync(sv + SV_MAXDIV, &v[3], sizeof(double), cudaMemcpyHostToDevice, st));
        PHX_CK(cudaStreamSynchronize(st));
        return PHX_OK;
    }

    // the scalar slots a checkpoint restores (src/sim/state.cpp:144-145,186)
    int setStats(int s, const phx_stats* in) override {
        PHX_TRY(checkScn(s));
        const int slot[10] = {SV_TIME, SV_MAXVEL, SV_MAXNU, SV_MAXDIV, SV_HRR, SV_MAXGAST, SV_BURNING,
                              SV_FUELIN, SV_FUELBURNED, SV_FUELINDOMAIN};
        const double v[10] = {in->time, in->max_vel, in->max_nu, in->max_div, in->hrr, in->max_gas_t,
                              (double)in->burning_cells, in->fuel_in, in->fuel_burned, in->fuel_in_domain};
        double* sv = sc[s]->h.sv;
        for (int q = 0; q < 10; ++q)
            PHX_CK(cudaMemcpyAsync(sv + slot[q], &v[q], sizeof(double), cudaMemcpyHostToDevice, st));
        PHX_CK(cudaStreamSynchronize(st));
        return PHX_OK;
    }

    size_t deviceBytes() const override {
        size_t b = 0;
        for (auto& S : sc) b += S->arenaBytes;
        return b;
    }
    int sync() override {
        if (st) PHX_CK(cudaStreamSynchronize(st));
        return checkDeviceError();
    }
    int deviceView(int s, const void** descriptor, int* cells, void** stream) override {
        PHX_TRY(checkScn(s));
        if (tablesDirty || !dS) {
            // building the tables would allocate: the caller steps (or syncs) the context first
            err = "the context's device tables are not built yet: step the context once after adding scenarios";
            return PHX_ERR_STATE;
        }
        *descriptor = dS + s;
        *cells = sc[s]->geo.N();
        *stream = (void*)st;
        return PHX_OK;
    }
    int mgInfo(int s, int* levels, int* rows, int cap) override {
        PHX_TRY(checkScn(s));
        const Multigrid& M = sc[s]->MG;
        if (levels) *levels = (int)M.lv.size();
        for (int l = 0; rows && l < cap && l < (int)M.lv.size(); ++l) rows[l] = M.lv[l].n;
        return PHX_OK;
    }
    int mgNnz(int s, int* nnz, int cap) override {
        PHX_TRY(checkScn(s));
        const Multigrid& M = sc[s]->MG;
        for (int l = 0; nnz && l < cap && l < (int)M.lv.size(); ++l)
            nnz[l] = M.lv[l].rowStart.empty() ? 0 : M.lv[l].rowStart.back();
        return PHX_OK;
    }
    int lastLaunches() const override {
        if (useGraph && gexec) {
            int k = 0;
            if (const_cast<Ctx*>(this)->graphLaunchCount(&k) == PHX_OK) return k;
        }
        return launches;
    }

    // n steps timed with CUDA events on the context's stream; with flushL2 a
    // buffer larger than L2 is written (untimed) before each step
    int timeSteps(int n, double dtMax, int flushL2, double* totalMs, int* launchesOut) override {
        PHX_TRY(ensureTables());
        if (flushL2 && !flushBuf) {
            flushBytes = (size_t)512 << 20;
            PHX_CK(cudaMalloc(&flushBuf, flushBytes));
        }
        PHX_CK(cudaStreamSynchronize(st));
        double total = 0;
        int nl = 0;
        for (int i = 0; i < n; ++i) {
            if (flushL2) PHX_CK(cudaMemsetAsync(flushBuf, i & 0xff, flushBytes, st));
            PHX_CK(cudaEventRecord(ev[0], st));
            launches = 0;
            PHX_TRY(oneStep(dtMax));
            PHX_CK(cudaEventRecord(ev[1], st));
            PHX_CK(cudaEventSynchronize(ev[1]));
            float ms = 0;
            PHX_CK(cudaEventElapsedTime(&ms, ev[0], ev[1]));
            total += ms;
            if (useGraph) {
                int k = 0;
                PHX_TRY(graphLaunchCount(&k));
                nl += k;
            } else {
                nl += launches;
            }
        }
        if (totalMs) *totalMs = total;
        if (launchesOut) *launchesOut = nl;
        return checkDeviceError();
    }

    // one step with an event pair around every launch; per-kernel totals
    int profileStep(double dtMax, int flushL2, phx_kernel_time* out, int cap_, int* count) override {
        PHX_TRY(ensureTables());
        if (flushL2) {
            if (!flushBuf) { flushBytes = (size_t)512 << 20; PHX_CK(cudaMalloc(&flushBuf, flushBytes)); }
            PHX_CK(cudaMemsetAsync(flushBuf, 0x5a, flushBytes, st));
        }
        kstats.clear();
        prof = true;
        launches = 0;
        int r = oneStep(dtMax);
        prof = false;
        PHX_TRY(r);
        PHX_TRY(collectProfile());
        int n = 0;
        for (auto& k : kstats) {
            if (n < cap_ && out) {
                std::memset(&out[n], 0, sizeof(phx_kernel_time));
                std::strncpy(out[n].name, k.name.c_str(), sizeof(out[n].name) - 1);
                out[n].launches = k.launches;
                out[n].ms = k.ms;
            }
            ++n;
        }
        if (count) *count = n;
        return PHX_OK;
    }
};

#undef PHX_TRY
}  // namespace phx
