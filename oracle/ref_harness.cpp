// Harness over the reference's own photon::Solver, compiled together with a
// build copy of the reference sources (see make_ref.py). Test infrastructure
// only: it is never linked into the product library.
//
// The reference sources are compiled with a prelude that maps `private` to
// `public` (so single stages such as Solver::momentum can be called) and, for
// the FP64 oracle build, `float` to `double`. This file is compiled under the
// same prelude, so `float` below is the solver's real type in either build.
//
// Grid set-up without a scene mirrors the field allocation list of
// Solver::build (src/sim/discretize.cpp:24-62); geometry (blocked mask, face
// fractions, pressure-matrix coefficients, leak flags) is then supplied by the
// caller, exactly as the discretizer would leave it.
#include "scene/materials.h"
#include "scene/scene.h"
#include "sim/devices.h"
#include "sim/solver.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>

using namespace photon;

namespace {
struct Ctx {
    Solver* s = nullptr;
    MaterialLibrary lib;
    Scene scene;
};

template <class V>
void assignN(V& vec, size_t n, typename V::value_type val) { vec.assign(n, val); }

// typed view of one named field
struct FieldRef {
    int type = -1;   // 0 real, 1 uint8, 2 int32
    void* vec = nullptr;
};

FieldRef lookup(Solver& s, const std::string& n) {
    FieldRef r;
    auto R = [&](std::vector<float>& v) { r.type = 0; r.vec = &v; };
    auto B = [&](std::vector<uint8_t>& v) { r.type = 1; r.vec = &v; };
    auto I = [&](std::vector<int>& v) { r.type = 2; r.vec = &v; };
    if (n == "u") R(s.u); else if (n == "v") R(s.v); else if (n == "w") R(s.w);
    else if (n == "fx") R(s.fx); else if (n == "fy") R(s.fy); else if (n == "fz") R(s.fz);
    else if (n == "ax") R(s.ax_); else if (n == "ay") R(s.ay_); else if (n == "az") R(s.az_);
    else if (n == "lx") B(s.lx_); else if (n == "ly") B(s.ly_); else if (n == "lz") B(s.lz_);
    else if (n == "p") R(s.p); else if (n == "S") R(s.S); else if (n == "T") R(s.T);
    else if (n == "Yo") R(s.Yo); else if (n == "Yf") R(s.Yf); else if (n == "Ys") R(s.Ys);
    else if (n == "Ya") R(s.Ya); else if (n == "Yp") R(s.Yp); else if (n == "Yc") R(s.Yc);
    else if (n == "Yw") R(s.Yw); else if (n == "Yco") R(s.Yco); else if (n == "Yai") R(s.Yai);
    else if (n == "nu") R(s.nu); else if (n == "Pb") R(s.Pb); else if (n == "Q") R(s.Q);
    else if (n == "Qr") R(s.Qr); else if (n == "hrr") R(s.hrr); else if (n == "massSrc") R(s.massSrc);
    else if (n == "lit") B(s.lit); else if (n == "pilot") B(s.pilot); else if (n == "blocked") B(s.blocked);
    else if (n == "zone") I(s.zone); else if (n == "zoneOpen") B(s.zoneOpen); else if (n == "zoneP") R(s.zoneP);
    else if (n == "rhs") R(s.rhs_); else if (n == "diag") R(s.tmp_[9]);
    else if (n == "cgR") R(s.cgR_); else if (n == "cgZ") R(s.cgZ_); else if (n == "cgP") R(s.cgP_); else if (n == "cgQ") R(s.cgQ_);
    else if (n == "zoneDP") R(s.zoneDP_);
    return r;
}
} // namespace

extern "C" {

int ref_real_bytes() { return (int)sizeof(float); }

// The reference JobPool's workers read its generation counter only once they
// start running (src/core/jobs.h:79-80); a parallelFor issued before a worker
// has started is never seen by that worker and the caller waits forever. Give
// the workers time to start before the solver is used.
void* ref_new(int threads) {
    Ctx* c = new Ctx;
    c->s = threads > 0 ? new Solver(threads) : new Solver();
    std::this_thread::sleep_for(std::chrono::milliseconds(200));
    return c;
}

void ref_free(void* h) {
    Ctx* c = (Ctx*)h;
    delete c->s;
    delete c;
}

// Allocate every field for an nx*ny*nz grid as Solver::build does, with the
// domain's faces fully open and no geometry; zones and the multigrid are rebuilt
// on the next step.
int ref_init_grid(void* h, int nx, int ny, int nz, double dx, double ox, double oy, double oz) {
    Solver& s = *((Ctx*)h)->s;
    s.dx = (float)dx; s.ox = (float)ox; s.oy = (float)oy; s.oz = (float)oz;
    s.nx = nx; s.ny = ny; s.nz = nz; s.N = nx * ny * nz;
    const int N = s.N;
    if (N <= 0 || N > 20000000) return -1;
    size_t NX = (size_t)(nx + 1) * ny * nz, NY = (size_t)nx * (ny + 1) * nz, NZ = (size_t)nx * ny * (nz + 1);
    assignN(s.u, NX, 0.f); assignN(s.v, NY, 0.f); assignN(s.w, NZ, 0.f);
    assignN(s.fx, NX, 1.f); assignN(s.fy, NY, 1.f); assignN(s.fz, NZ, 1.f);
    assignN(s.bx, NX, -1); assignN(s.by, NY, -1); assignN(s.bz, NZ, -1);
    assignN(s.p, N, 0.f); assignN(s.S, N, 0.f); assignN(s.T, N, Solver::T0); assignN(s.Yo, N, Solver::YO2_AMB);
    assignN(s.Yf, N, 0.f); assignN(s.Ys, N, 0.f); assignN(s.Ya, N, 0.f); assignN(s.Yp, N, 0.f);
    assignN(s.Yc, N, Solver::YCO2_AMB); assignN(s.Yw, N, Solver::YH2O_AMB); assignN(s.Yco, N, 0.f);
    assignN(s.nu, N, 0.f); assignN(s.Yai, N, 0.f);
    s.matAIT.clear();
    assignN(s.Pb, N, Solver::P0); assignN(s.zone, N, -1); assignN(s.massSrc, N, 0.f);
    s.zoneP.clear(); s.zoneOpen.clear(); s.burners.clear();
    assignN(s.ax_, NX, 0.f); assignN(s.ay_, NY, 0.f); assignN(s.az_, NZ, 0.f);
    assignN(s.lx_, NX, (uint8_t)0); assignN(s.ly_, NY, (uint8_t)0); assignN(s.lz_, NZ, (uint8_t)0);
    assignN(s.cgR_, N, 0.f); assignN(s.cgZ_, N, 0.f); assignN(s.cgP_, N, 0.f); assignN(s.cgQ_, N, 0.f);
    s.zonesDirty_ = true;
    s.mgDirty_ = true;
    s.maxVel = s.maxNu = 0;
    s.maxDiv = 0;
    assignN(s.Q, N, 0.f); assignN(s.Qr, N, 0.f); assignN(s.hrr, N, 0.f);
    assignN(s.lit, N, (uint8_t)0); assignN(s.pilot, N, (uint8_t)0);
    assignN(s.blocked, N, (uint8_t)0); assignN(s.porous, N, (uint8_t)0);
    assignN(s.fuelMat, N, (int16_t)-1); assignN(s.itemOf, N, (int16_t)-1);
    assignN(s.fuelMass, N, 0.f); assignN(s.fuelMass0, N, 0.f); assignN(s.charMass, N, 0.f);
    assignN(s.fuelT, N, Solver::T0); assignN(s.fuelArea, N, 0.f); assignN(s.radQ, N, 0.f);
    assignN(s.condQ, N, 0.f); assignN(s.burnFrac, N, 0.f); assignN(s.ignE, N, 0.f);
    assignN(s.slab, (size_t)N * Solver::SLAB_NODES, Solver::T0); assignN(s.slabF, (size_t)N * Solver::SLAB_NODES, 1.f);
    assignN(s.coverMat, N, (int16_t)-1); assignN(s.coverLeft, N, 0.f);
    for (auto& t : s.tmp_) t.assign(N, 0.f);
    s.u2_.assign(NX, 0.f); s.v2_.assign(NY, 0.f); s.w2_.assign(NZ, 0.f); s.rhs_.assign(N, 0.f);
    s.barriers.clear(); s.ignitions.clear(); s.events.clear(); s.eventKeys_.clear(); s.solidCells.clear();
    s.time = 0;
    s.stats = SimStats{};
    s.mg_.clear();
    s.zoneDP_.clear();
    return 0;
}

// Load the material library from dataDir and build from a scene file, as the
// reference's own tests do (src/tests/test_main.cpp:44-55, 420-433).
int ref_load_scene(void* h, const char* dataDir, const char* scenePath, int referenceProfile, int radiationOn,
                   int adiabatic, int noLeak, char* err, int errLen) {
    Ctx* c = (Ctx*)h;
    std::string e, d = dataDir;
    bool ok = c->lib.loadGases(d + "/gases.txt", e) && c->lib.loadMaterials(d + "/materials.txt", e) &&
              c->lib.loadAssemblies(d + "/assemblies.txt", e) && c->lib.loadComponents(d + "/components.txt", e) &&
              c->lib.loadAssets(d + "/assets.txt", e) && c->scene.load(scenePath, c->lib, e);
    if (ok) {
        if (referenceProfile) c->s->profile = FidelityProfile::reference();
        c->s->radiationOn = radiationOn != 0;
        c->s->adiabaticSurfaces = adiabatic != 0;
        ok = c->s->build(c->scene, c->lib, e);
        if (ok && noLeak) c->s->clearLeakage();
    }
    if (!ok && err && errLen > 0) { std::strncpy(err, e.c_str(), errLen - 1); err[errLen - 1] = 0; }
    return ok ? 0 : -1;
}

// Door open/close or window break by scene opening name; returns the new state or -1.
int ref_toggle_opening(void* h, const char* name) {
    Ctx* c = (Ctx*)h;
    for (size_t o = 0; o < c->scene.openings.size(); ++o)
        if (c->scene.openings[o].name == name) return c->s->toggleOpening((int)o) ? 1 : 0;
    return -1;
}

void ref_grid_info(void* h, int* dims, double* geo) {
    Solver& s = *((Ctx*)h)->s;
    dims[0] = s.nx; dims[1] = s.ny; dims[2] = s.nz; dims[3] = s.N;
    geo[0] = s.dx; geo[1] = s.ox; geo[2] = s.oy; geo[3] = s.oz;
}

void ref_set_profile(void* h, double cfl, double dtMax, int maxIters, double tol) {
    Solver& s = *((Ctx*)h)->s;
    s.profile.cfl = (float)cfl; s.profile.dtMax = (float)dtMax;
    s.profile.pressureMaxIters = maxIters; s.profile.pressureTol = (float)tol;
}

// the CG stop of the next steps: Solver::profile.pressureTol, 1/s (the
// reference's only stop test, src/sim/gasphase.cpp:604-605)
void ref_set_pressure_tol(void* h, double tol) {
    ((Ctx*)h)->s->profile.pressureTol = (float)tol;
}

// max |b| of the last projection's right-hand side (src/sim/gasphase.cpp:528-549),
// in the solver's units: 1/s times dx^2 / dt
double ref_rhs_max_abs(void* h) {
    const Solver& s = *((Ctx*)h)->s;
    float m = 0;
    for (float v : s.rhs_) m = std::max(m, std::fabs(v));
    return m;
}

void ref_set_switches(void* h, int radiationOn, int adiabatic) {
    Solver& s = *((Ctx*)h)->s;
    s.radiationOn = radiationOn != 0;
    s.adiabaticSurfaces = adiabatic != 0;
}

void ref_set_wind(void* h, double speed, double fromDeg, double exponent) {
    Solver& s = *((Ctx*)h)->s;
    s.wind.speed = (float)speed; s.wind.fromDeg = (float)fromDeg; s.wind.exponent = (float)exponent;
}

// geometry changed through ref_field: zones and multigrid are rebuilt on the next step
void ref_mark_geometry_dirty(void* h) {
    Solver& s = *((Ctx*)h)->s;
    s.zonesDirty_ = true;
    s.mgDirty_ = true;
}

int ref_add_burner(void* h, double x0, double y0, double x1, double y1, double z, double peakW, double rampS,
                   double start, double duration) {
    Burner b;
    b.x0 = (float)x0; b.y0 = (float)y0; b.x1 = (float)x1; b.y1 = (float)y1; b.z = (float)z;
    b.peakW = (float)peakW; b.rampS = (float)rampS; b.start = (float)start; b.duration = (float)duration;
    b.label = "burner";
    return ((Ctx*)h)->s->addBurner(b);
}

int ref_burner_cells(void* h, int b, int* out, int cap) {
    Solver& s = *((Ctx*)h)->s;
    if (b < 0 || b >= (int)s.burners.size()) return -1;
    int n = (int)s.burners[b].cells.size();
    for (int i = 0; i < n && i < cap; ++i) out[i] = s.burners[b].cells[i];
    return n;
}

void ref_add_ignition(void* h, int cell, double power, double duration) {
    ((Ctx*)h)->s->addIgnition(cell, (float)power, (float)duration, "ignition");
}

double ref_step(void* h, double dtMax) { return ((Ctx*)h)->s->step((float)dtMax); }

// One stage of the gas-phase step, for per-stage parity tests. "zones" and
// "mg" run the set-up passes.
int ref_stage(void* h, const char* stage, double dt) {
    Solver& s = *((Ctx*)h)->s;
    std::string n = stage;
    float d = (float)dt;
    if (n == "zones") s.computeZones();
    else if (n == "mg") s.buildPressureLevels();
    else if (n == "burners") s.injectBurners(d);
    else if (n == "combustion") s.combustion(d);
    else if (n == "turbulence") s.turbulence();
    else if (n == "heat") s.heatDiffusion(d);
    else if (n == "energy") s.energyAndExpansion(d);
    else if (n == "momentum") s.momentum(d);
    else if (n == "leakage") s.leakage(d);
    else if (n == "project") s.project(d);
    else if (n == "advect") s.advectScalars(d);
    else if (n == "stats") s.gatherStats(d);
    else if (n == "clear") {
        for (int c = 0; c < s.N; ++c) { s.Q[c] = 0; s.Qr[c] = 0; s.pilot[c] = 0; s.massSrc[c] = 0; }
    } else if (n == "zonep") {
        for (size_t z = 0; z < s.zoneP.size(); ++z)
            if (!s.zoneOpen[z]) s.zoneP[z] = std::clamp(s.zoneP[z] + d * s.zoneDP_[z], Solver::P0 - 20000.0f, Solver::P0 + 50000.0f);
        for (int c = 0; c < s.N; ++c) if (s.zone[c] >= 0) s.Pb[c] = s.zoneP[s.zone[c]];
    } else return -1;
    return 0;
}

double ref_stable_dt(void* h, double dtMax) { return ((Ctx*)h)->s->stableDt((float)dtMax); }

// Precondition r -> z with one V-cycle (pressure_mg.cpp:270-300).
void ref_precondition(void* h, const double* r, double* z) {
    Solver& s = *((Ctx*)h)->s;
    std::vector<float> rv(s.N), zv(s.N);
    for (int c = 0; c < s.N; ++c) rv[c] = (float)r[c];
    s.pressurePrecondition(rv, zv);
    for (int c = 0; c < s.N; ++c) z[c] = zv[c];
}

long ref_field_len(void* h, const char* name) {
    Solver& s = *((Ctx*)h)->s;
    FieldRef f = lookup(s, name);
    if (f.type == 0) return (long)((std::vector<float>*)f.vec)->size();
    if (f.type == 1) return (long)((std::vector<uint8_t>*)f.vec)->size();
    if (f.type == 2) return (long)((std::vector<int>*)f.vec)->size();
    return -1;
}

// dir 0: copy the field out; dir 1: copy it in. Real fields travel as double,
// uint8 fields as uint8, int fields as int32. Returns the field type or -1.
int ref_field(void* h, const char* name, int dir, void* buf, long n) {
    Solver& s = *((Ctx*)h)->s;
    FieldRef f = lookup(s, name);
    if (f.type == 0) {
        auto& v = *(std::vector<float>*)f.vec;
        if (dir == 1) v.resize(n);
        if ((long)v.size() != n) return -1;
        double* d = (double*)buf;
        for (long i = 0; i < n; ++i) { if (dir == 0) d[i] = v[i]; else v[i] = (float)d[i]; }
    } else if (f.type == 1) {
        auto& v = *(std::vector<uint8_t>*)f.vec;
        if (dir == 1) v.resize(n);
        if ((long)v.size() != n) return -1;
        if (dir == 0) std::memcpy(buf, v.data(), n); else std::memcpy(v.data(), buf, n);
    } else if (f.type == 2) {
        auto& v = *(std::vector<int>*)f.vec;
        if (dir == 1) v.resize(n);
        if ((long)v.size() != n) return -1;
        if (dir == 0) std::memcpy(buf, v.data(), n * 4); else std::memcpy(v.data(), buf, n * 4);
    } else return -1;
    return f.type;
}

// time, maxVel, maxNu, maxDiv, pressureIters, pressureResidual, hrr, maxGasT,
// burningCells, fuelIn, fuelBurned, fuelInDomain, leakFaces, nZones
void ref_scalars(void* h, double* o) {
    Solver& s = *((Ctx*)h)->s;
    o[0] = s.time; o[1] = s.maxVel; o[2] = s.maxNu; o[3] = s.maxDiv;
    o[4] = s.pressureIters; o[5] = s.pressureResidual; o[6] = s.stats.hrr; o[7] = s.stats.maxGasT;
    o[8] = s.stats.burningCells; o[9] = s.stats.fuelIn; o[10] = s.stats.fuelBurned; o[11] = s.stats.fuelInDomain;
    o[12] = s.leakFaces; o[13] = (double)s.zoneP.size();
}

void ref_set_scalars(void* h, double time, double maxVel, double maxNu, double maxDiv) {
    Solver& s = *((Ctx*)h)->s;
    s.time = (float)time; s.maxVel = (float)maxVel; s.maxNu = (float)maxNu; s.maxDiv = (float)maxDiv;
}

// multigrid hierarchy export: level count, and per level n, nnz and arrays
int ref_mg_levels(void* h) { return (int)((Ctx*)h)->s->mg_.size(); }

void ref_mg_info(void* h, int l, int* info) {
    const PressureLevel& L = ((Ctx*)h)->s->mg_[l];
    info[0] = L.n; info[1] = (int)L.col.size(); info[2] = (int)L.agg.size();
}

// agg (int n or empty), rowStart (int n+1), col (int nnz), val (double nnz), diag (double n)
void ref_mg_get(void* h, int l, int* agg, int* rowStart, int* col, double* val, double* diag) {
    const PressureLevel& L = ((Ctx*)h)->s->mg_[l];
    for (size_t i = 0; i < L.agg.size(); ++i) agg[i] = L.agg[i];
    for (size_t i = 0; i < L.rowStart.size(); ++i) rowStart[i] = L.rowStart[i];
    for (size_t i = 0; i < L.col.size(); ++i) { col[i] = L.col[i]; val[i] = L.val[i]; }
    for (int i = 0; i < L.n; ++i) diag[i] = L.diag[i];
}

double ref_phase_ms(void* h, int i) { return ((Ctx*)h)->s->phaseMs[i]; }

// the order of ref_scalars' first four, then hrr, maxGasT, burningCells,
// fuelIn, fuelBurned, fuelInDomain
void ref_set_stats(void* h, const double* v) {
    Solver& s = *((Ctx*)h)->s;
    s.time = (float)v[0]; s.maxVel = (float)v[1]; s.maxNu = (float)v[2]; s.maxDiv = (float)v[3];
    s.stats.hrr = (float)v[4]; s.stats.maxGasT = (float)v[5]; s.stats.burningCells = (int)v[6];
    s.stats.fuelIn = v[7]; s.stats.fuelBurned = v[8]; s.stats.fuelInDomain = v[9];
}

// the zone tables Solver::step builds on its first call (src/sim/gasphase.cpp:111-158)
void ref_compute_zones(void* h) { ((Ctx*)h)->s->computeZones(); }

// Radiation trace inputs in the flat form the GPU trace takes
// (src/sim/radiation.cpp:104-193): the elements buildRadElements makes, with
// their emissivity and temperature; every intact barrier as a wall with the
// surface temperature seen from its lower and its upper cell; the solid
// temperature of every cell. counts = {elements, walls}.
void ref_rad_counts(void* h, int* counts) {
    Solver& s = *((Ctx*)h)->s;
    s.buildRadElements();
    int nw = 0;
    for (int b = 0; b < (int)s.barriers.size(); ++b) nw += s.barrierIntact(b) ? 1 : 0;
    counts[0] = (int)s.radElems_.size();
    counts[1] = nw;
}
// elem: 11 per element (o[3], n[3], area, eps, temp, sphere, skip own cell);
// wall: 4 per wall (axis, face, T seen from the lower cell, from the upper);
// solidT: N
void ref_rad_export(void* h, double* elem, double* wall, double* solidT) {
    Solver& s = *((Ctx*)h)->s;
    s.buildRadElements();
    for (size_t e = 0; e < s.radElems_.size(); ++e) {
        const RadElem& r = s.radElems_[e];
        double* o = elem + 11 * e;
        for (int q = 0; q < 3; ++q) { o[q] = r.o[q]; o[3 + q] = r.n[q]; }
        o[6] = r.area; o[7] = s.elemEmissivity(r); o[8] = s.elemTemp(r); o[9] = r.sphere ? 1 : 0;
        o[10] = r.kind == 2 ? 1 : 0;
    }
    int w = 0;
    for (int b = 0; b < (int)s.barriers.size(); ++b) {
        if (!s.barrierIntact(b)) continue;
        const Barrier& br = s.barriers[b];
        double* o = wall + 4 * w++;
        o[0] = br.axis; o[1] = br.face;
        o[2] = br.T[br.cellOn(0) == br.cellA ? 0 : 1];
        o[3] = br.T[br.cellOn(0) == br.cellB ? 0 : 1];
    }
    for (int c = 0; c < s.N; ++c) solidT[c] = s.fuelT[c];
}
// Solver::traceRadiation (src/sim/radiation.cpp:181-319): radAbs per element (W), radGas per cell (W)
void ref_rad_trace(void* h, double* radAbs, double* radGas) {
    Solver& s = *((Ctx*)h)->s;
    s.traceRadiation();
    for (size_t e = 0; e < s.radAbs_.size(); ++e) radAbs[e] = s.radAbs_[e];
    for (int c = 0; c < s.N; ++c) radGas[c] = s.radGas_[c];
}

// photon::sampleDevice (src/sim/devices.h:61-96) of the harness's solver:
// kind is the DeviceKind's position in its enum
double ref_sample_device(void* h, int kind, double x, double y, double z, double z0, double z1) {
    Device d;
    d.kind = (DeviceKind)kind;
    d.x = (float)x; d.y = (float)y; d.z = (float)z; d.z0 = (float)z0; d.z1 = (float)z1;
    return sampleDevice(*((Ctx*)h)->s, d);
}

// Solver::saveState / Solver::loadState (src/sim/state.cpp:62-195); 0 on success
int ref_save_state(void* h, const char* path, char* err, int errLen) {
    std::string e;
    if (((Ctx*)h)->s->saveState(path, e)) return 0;
    std::snprintf(err, errLen, "%s", e.c_str());
    return -1;
}
int ref_load_state(void* h, const char* path, char* err, int errLen) {
    std::string e;
    if (((Ctx*)h)->s->loadState(path, e)) return 0;
    std::snprintf(err, errLen, "%s", e.c_str());
    return -1;
}

} // extern "C"
