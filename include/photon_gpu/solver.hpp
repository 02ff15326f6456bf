// photon_gpu::Solver -- C++ adapter with photon::Solver's step API over the
// GB300 C ABI (include/phx.h).
//
// It mirrors the surface Photon's callers use after Solver::build
// (src/sim/solver.h:156-347): the grid and geometry members, step(dtMax) -> dt,
// addBurner / addIgnition, the public field vectors, stats, maxVel and the
// pressure-solve counters. Fields live on the GPU; the host vectors are filled
// on demand (sync()) so device probes, CSV writers and checkpoints
// (src/sim/devices.h, src/app/cli_case.cpp, src/sim/state.cpp) can read them
// as before. Header only; link with libphx.so.
#pragma once
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "../phx.h"

namespace photon_gpu {

// FidelityProfile (src/sim/solver.h:82-104) plus the relative stop of the
// pressure solve (0 = the reference's absolute test only)
struct FidelityProfile {
    float cfl = 0.8f, dtMax = 0.05f;
    int pressureMaxIters = 80;
    float pressureTol = 0.02f;
    double pressureRelTol = 0;
    static FidelityProfile realtime() { return FidelityProfile(); }
    static FidelityProfile reference() {
        FidelityProfile p;
        p.cfl = 0.5f; p.dtMax = 0.02f; p.pressureMaxIters = 400; p.pressureTol = 0.002f;
        return p;
    }
};

struct Wind {
    float speed = 0, fromDeg = 0, exponent = 0.25f;
};

// Burner (src/sim/solver.h:115-127)
struct Burner {
    float x0 = 0, y0 = 0, x1 = 0, y1 = 0, z = 0;
    float peakW = 0, rampS = 0, start = 0, duration = 1e9f;
    std::string label;
};

struct SimStats {
    float hrr = 0, maxGasT = 293.15f;
    int burningCells = 0;
    float stepMs = 0;
    double fuelIn = 0, fuelBurned = 0, fuelInDomain = 0;
};

class Solver {
public:
    enum class Precision { FP64 = PHX_PREC_FP64, Mixed = PHX_PREC_MIXED };

    FidelityProfile profile;
    Wind wind;
    bool radiationOn = true;
    bool adiabaticSurfaces = false;
    Precision precision = Precision::FP64;

    // grid (src/sim/solver.h:211-220)
    int nx = 0, ny = 0, nz = 0, N = 0;
    float dx = 0.2f, ox = 0, oy = 0, oz = 0;
    int cell(int i, int j, int k) const { return i + nx * (j + ny * k); }
    int xface(int i, int j, int k) const { return i + (nx + 1) * (j + ny * k); }
    int yface(int i, int j, int k) const { return i + nx * (j + (ny + 1) * k); }
    int zface(int i, int j, int k) const { return i + nx * (j + ny * k); }

    // geometry as the discretizer leaves it (set before build)
    std::vector<uint8_t> blocked;
    std::vector<float> fx, fy, fz, ax, ay, az;
    std::vector<uint8_t> lx, ly, lz;

    // state, filled from the device by sync()
    float time = 0;
    std::vector<float> u, v, w, p, S, T, Yo, Yf, Ys, Ya, Yp, Yc, Yw, Yco, Yai, nu, Pb, Q, Qr, hrr, massSrc;
    std::vector<uint8_t> lit;
    std::vector<int> zone;
    std::vector<float> zoneP;
    SimStats stats;
    float maxVel = 0, maxNu = 0, maxDiv = 0;
    int pressureIters = 0;
    float pressureResidual = 0;

    Solver() = default;
    Solver(const Solver&) = delete;
    Solver& operator=(const Solver&) = delete;
    ~Solver() { if (ctx_) phx_destroy(ctx_); }

    // Size the grid and open every face (Solver::build's allocation, without a scene)
    void setGrid(int nx_, int ny_, int nz_, float dx_, float ox_ = 0, float oy_ = 0, float oz_ = 0) {
        nx = nx_; ny = ny_; nz = nz_; N = nx * ny * nz; dx = dx_; ox = ox_; oy = oy_; oz = oz_;
        size_t NX = (size_t)(nx + 1) * ny * nz, NY = (size_t)nx * (ny + 1) * nz, NZ = (size_t)nx * ny * (nz + 1);
        blocked.assign(N, 0);
        fx.assign(NX, 1.f); fy.assign(NY, 1.f); fz.assign(NZ, 1.f);
        ax.assign(NX, 1.f); ay.assign(NY, 1.f); az.assign(NZ, 1.f);
        lx.assign(NX, 0); ly.assign(NY, 0); lz.assign(NZ, 0);
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) { fz[zface(i, j, 0)] = 0; az[zface(i, j, 0)] = 0; }   // the ground
    }

    // Create the device context from the geometry; false with a message on failure
    bool build(std::string& err) {
        if (ctx_) { phx_destroy(ctx_); ctx_ = nullptr; }
        std::vector<double> dfx(fx.begin(), fx.end()), dfy(fy.begin(), fy.end()), dfz(fz.begin(), fz.end());
        std::vector<double> dax(ax.begin(), ax.end()), day(ay.begin(), ay.end()), daz(az.begin(), az.end());
        phx_grid g{};
        g.nx = nx; g.ny = ny; g.nz = nz; g.dx = dx; g.ox = ox; g.oy = oy; g.oz = oz;
        g.cfl = profile.cfl; g.dt_max = profile.dtMax; g.max_iters = profile.pressureMaxIters;
        g.tol = profile.pressureTol; g.rel_tol = profile.pressureRelTol;
        g.radiation_on = radiationOn; g.adiabatic_surfaces = adiabaticSurfaces;
        g.wind_speed = wind.speed; g.wind_from_deg = wind.fromDeg; g.wind_exponent = wind.exponent;
        g.blocked = blocked.data();
        g.fx = dfx.data(); g.fy = dfy.data(); g.fz = dfz.data();
        g.ax = dax.data(); g.ay = day.data(); g.az = daz.data();
        g.lx = lx.empty() ? nullptr : lx.data();
        g.ly = ly.empty() ? nullptr : ly.data();
        g.lz = lz.empty() ? nullptr : lz.data();
        if (phx_create(&g, (int)precision, &ctx_) != PHX_OK) {
            err = phx_last_global_error();
            return false;
        }
        sync();
        return true;
    }

    // Solver::addBurner: index, or -1 if it covers no gas cell
    int addBurner(const Burner& b) {
        int idx = -1;
        if (phx_add_burner(ctx_, b.x0, b.y0, b.x1, b.y1, b.z, b.peakW, b.rampS, b.start, b.duration, &idx) != PHX_OK)
            return -1;
        return idx;
    }
    void addIgnition(int cell, float power, float duration, const std::string& = std::string()) {
        check(phx_add_ignition(ctx_, cell, power, duration));
    }

    // Solver::step: one gas-phase step on the GPU, returns dt. Host fields are
    // refreshed only when autoSync is set (or on sync()).
    bool autoSync = false;
    float step(float dtMax) {
        double dt = 0;
        check(phx_step(ctx_, dtMax, &dt));
        readScalars();
        if (autoSync) sync();
        return (float)dt;
    }

    // device -> host copy of every field
    void sync() {
        get(PHX_FIELD_U, u); get(PHX_FIELD_V, v); get(PHX_FIELD_W, w);
        get(PHX_FIELD_P, p); get(PHX_FIELD_S, S);
        get(PHX_FIELD_T, T); get(PHX_FIELD_YO, Yo); get(PHX_FIELD_YF, Yf); get(PHX_FIELD_YS, Ys);
        get(PHX_FIELD_YA, Ya); get(PHX_FIELD_YP, Yp); get(PHX_FIELD_YC, Yc); get(PHX_FIELD_YW, Yw);
        get(PHX_FIELD_YCO, Yco); get(PHX_FIELD_YAI, Yai); get(PHX_FIELD_NU, nu); get(PHX_FIELD_PB, Pb);
        get(PHX_FIELD_Q, Q); get(PHX_FIELD_QR, Qr); get(PHX_FIELD_HRR, hrr); get(PHX_FIELD_MASSSRC, massSrc);
        get(PHX_FIELD_ZONEP, zoneP);
        zone.resize(phx_field_count(ctx_, PHX_FIELD_ZONE));
        check(phx_get_field(ctx_, PHX_FIELD_ZONE, zone.data(), zone.size() * sizeof(int)));
        lit.resize(phx_field_count(ctx_, PHX_FIELD_LIT));
        check(phx_get_field(ctx_, PHX_FIELD_LIT, lit.data(), lit.size()));
        readScalars();
    }

    // host -> device copy of the state fields (after the caller edited them)
    void push() {
        put(PHX_FIELD_U, u); put(PHX_FIELD_V, v); put(PHX_FIELD_W, w); put(PHX_FIELD_P, p);
        put(PHX_FIELD_T, T); put(PHX_FIELD_YO, Yo); put(PHX_FIELD_YF, Yf); put(PHX_FIELD_YS, Ys);
        put(PHX_FIELD_YA, Ya); put(PHX_FIELD_YP, Yp); put(PHX_FIELD_YC, Yc); put(PHX_FIELD_YW, Yw);
        put(PHX_FIELD_YCO, Yco); put(PHX_FIELD_YAI, Yai);
    }

    // Checkpoint interop. A checkpoint is written and read by the host
    // photon::Solver (saveState / loadState, src/sim/state.cpp:62-195); these
    // two move the gas-phase part of that state between the GPU and any host
    // object with photon::Solver's public members (u v w p S T Yo Yf Ys Ya Yp
    // Yc Yw Yco Yai nu Pb hrr lit zone zoneP, time, maxVel, maxNu, maxDiv,
    // stats). The host's zone tables must exist (they do after its first step
    // or a loadState): zones depend on the geometry only, and the host's
    // numbering is the GPU's.
    template <class Host>
    void exportTo(Host& h) {
        sync();
        auto cp = [](auto& dst, const auto& src) { dst.assign(src.begin(), src.end()); };
        cp(h.u, u); cp(h.v, v); cp(h.w, w); cp(h.p, p); cp(h.S, S);
        cp(h.T, T); cp(h.Yo, Yo); cp(h.Yf, Yf); cp(h.Ys, Ys); cp(h.Ya, Ya); cp(h.Yp, Yp);
        cp(h.Yc, Yc); cp(h.Yw, Yw); cp(h.Yco, Yco); cp(h.Yai, Yai); cp(h.nu, nu); cp(h.Pb, Pb);
        cp(h.hrr, hrr); cp(h.lit, lit); cp(h.zoneP, zoneP);
        h.time = time; h.maxVel = maxVel; h.maxNu = maxNu; h.maxDiv = maxDiv;
        h.stats.hrr = stats.hrr; h.stats.maxGasT = stats.maxGasT; h.stats.burningCells = stats.burningCells;
        h.stats.fuelIn = stats.fuelIn; h.stats.fuelBurned = stats.fuelBurned; h.stats.fuelInDomain = stats.fuelInDomain;
    }
    // The reverse, after the host loaded a checkpoint; false with a message when
    // the host's grid or zone count is not this solver's.
    template <class Host>
    bool importFrom(const Host& h, std::string& err) {
        if (h.nx != nx || h.ny != ny || h.nz != nz || h.dx != dx) { err = "state grid does not match this solver's grid"; return false; }
        if (h.zoneP.size() != phx_field_count(ctx_, PHX_FIELD_ZONEP)) { err = "state zone count does not match"; return false; }
        auto cp = [](auto& dst, const auto& src) { dst.assign(src.begin(), src.end()); };
        cp(u, h.u); cp(v, h.v); cp(w, h.w); cp(p, h.p); cp(S, h.S);
        cp(T, h.T); cp(Yo, h.Yo); cp(Yf, h.Yf); cp(Ys, h.Ys); cp(Ya, h.Ya); cp(Yp, h.Yp);
        cp(Yc, h.Yc); cp(Yw, h.Yw); cp(Yco, h.Yco); cp(Yai, h.Yai); cp(nu, h.nu); cp(Pb, h.Pb);
        cp(hrr, h.hrr); cp(lit, h.lit); cp(zoneP, h.zoneP);
        push();
        put(PHX_FIELD_S, S); put(PHX_FIELD_NU, nu); put(PHX_FIELD_PB, Pb); put(PHX_FIELD_HRR, hrr);
        put(PHX_FIELD_ZONEP, zoneP);
        if (!lit.empty()) check(phx_set_field(ctx_, PHX_FIELD_LIT, lit.data(), lit.size()));
        phx_stats s{};
        s.time = h.time; s.max_vel = h.maxVel; s.max_nu = h.maxNu; s.max_div = h.maxDiv;
        s.hrr = h.stats.hrr; s.max_gas_t = h.stats.maxGasT; s.burning_cells = h.stats.burningCells;
        s.fuel_in = h.stats.fuelIn; s.fuel_burned = h.stats.fuelBurned; s.fuel_in_domain = h.stats.fuelInDomain;
        check(phx_set_stats(ctx_, &s));
        readScalars();
        return true;
    }

    phx_ctx* handle() const { return ctx_; }

private:
    phx_ctx* ctx_ = nullptr;
    std::vector<double> buf_;

    void check(int r) {
        if (r != PHX_OK) throw std::runtime_error(std::string("phx: ") + phx_last_error(ctx_));
    }
    void get(int f, std::vector<float>& out) {
        size_t n = phx_field_count(ctx_, f);
        buf_.resize(n);
        check(phx_get_field(ctx_, f, buf_.data(), n * sizeof(double)));
        out.assign(buf_.begin(), buf_.end());
    }
    void put(int f, const std::vector<float>& in) {
        if (in.empty()) return;
        buf_.assign(in.begin(), in.end());
        check(phx_set_field(ctx_, f, buf_.data(), buf_.size() * sizeof(double)));
    }
    void readScalars() {
        phx_stats s{};
        check(phx_get_stats(ctx_, &s));
        time = (float)s.time;
        maxVel = (float)s.max_vel; maxNu = (float)s.max_nu; maxDiv = (float)s.max_div;
        pressureIters = s.pressure_iters; pressureResidual = (float)s.pressure_residual;
        stats.hrr = (float)s.hrr; stats.maxGasT = (float)s.max_gas_t; stats.burningCells = s.burning_cells;
        stats.fuelIn = s.fuel_in; stats.fuelBurned = s.fuel_burned; stats.fuelInDomain = s.fuel_in_domain;
    }
};

}  // namespace photon_gpu
