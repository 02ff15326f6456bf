// A Photon-style caller of photon_gpu::Solver: the ISO 9705 size room of the
// reference's gas-phase tests (src/tests/test_main.cpp:420-433) as a closed box
// at 20 cm with an open doorway, a 100 kW burner, 40 steps; prints one line of
// results for the test to check.
//
// With a second argument "checkpoint" it then moves the state through a host
// object with photon::Solver's public state members (what saveState writes,
// src/sim/state.cpp:62-121) into a second GPU solver, checks that the fields
// arrive unchanged, steps both solvers 10 more steps and prints the largest
// relative difference of their temperature and velocity fields.
//
// With "dump <prefix>" as the second and third arguments it writes, after the
// 40 steps, the adapter's host vectors (float, as photon::Solver holds them)
// to <prefix>_<field>.f32 and the same fields read through the C ABI in
// double to <prefix>_<field>.f64, for a comparison with the oracle.
//
// With "case <prefix>" it runs photon_gpu::runCase for 2 s with rows every
// 0.5 s and a checkpoint every 1 s (the host's saveState writes the time and
// the temperature field), and prints the row times.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "photon_gpu/case_loop.hpp"
#include "photon_gpu/solver.hpp"

// the members of photon::Solver a checkpoint's gas phase consists of
struct HostState {
    int nx = 0, ny = 0, nz = 0;
    float dx = 0;
    float time = 0, maxVel = 0, maxNu = 0, maxDiv = 0;
    std::vector<float> u, v, w, p, S, T, Yo, Yf, Ys, Ya, Yp, Yc, Yw, Yco, Yai, nu, Pb, hrr, zoneP;
    std::vector<uint8_t> lit;
    struct {
        float hrr = 0, maxGasT = 0;
        int burningCells = 0;
        double fuelIn = 0, fuelBurned = 0, fuelInDomain = 0;
    } stats;
    // a stand-in for Solver::saveState: the time and the temperature field
    bool saveState(const std::string& path, std::string& err) const {
        FILE* f = std::fopen(path.c_str(), "wb");
        if (!f) { err = "cannot open " + path; return false; }
        std::fwrite(&time, sizeof(time), 1, f);
        std::fwrite(T.data(), sizeof(float), T.size(), f);
        std::fclose(f);
        return true;
    }
};

static bool setupRoom(photon_gpu::Solver& s, bool mixed) {
    s.profile = photon_gpu::FidelityProfile::realtime();
    s.radiationOn = false;
    s.adiabaticSurfaces = true;
    if (mixed) s.precision = photon_gpu::Solver::Precision::Mixed;
    const int nx = 18, ny = 12, nz = 12;
    s.setGrid(nx, ny, nz, 0.2f);
    // closed walls and ceiling, one doorway in the x = 0 wall (j 4..7, k 0..9)
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j) {
            bool door = j >= 4 && j < 8 && k < 10;
            s.fx[s.xface(0, j, k)] = s.ax[s.xface(0, j, k)] = door ? 1.f : 0.f;
            s.fx[s.xface(nx, j, k)] = s.ax[s.xface(nx, j, k)] = 0.f;
        }
    for (int k = 0; k < nz; ++k)
        for (int i = 0; i < nx; ++i) {
            s.fy[s.yface(i, 0, k)] = s.ay[s.yface(i, 0, k)] = 0.f;
            s.fy[s.yface(i, ny, k)] = s.ay[s.yface(i, ny, k)] = 0.f;
        }
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) s.fz[s.zface(i, j, nz)] = s.az[s.zface(i, j, nz)] = 0.f;
    std::string err;
    if (!s.build(err)) { std::printf("build failed: %s\n", err.c_str()); return false; }
    photon_gpu::Burner b;
    b.x0 = 2.4f; b.y0 = 1.0f; b.x1 = 2.8f; b.y1 = 1.4f; b.z = 0; b.peakW = 100e3f;
    if (s.addBurner(b) < 0) { std::printf("burner rejected\n"); return false; }
    return true;
}

static double maxRel(const std::vector<float>& a, const std::vector<float>& b) {
    double num = 0, den = 0;
    for (size_t i = 0; i < a.size(); ++i) {
        num = std::max(num, (double)std::fabs(a[i] - b[i]));
        den = std::max(den, (double)std::fabs(b[i]));
    }
    return den > 0 ? num / den : num;
}

template <class T>
static bool writeRaw(const std::string& path, const std::vector<T>& v) {
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) return false;
    const size_t n = std::fwrite(v.data(), sizeof(T), v.size(), f);
    std::fclose(f);
    return n == v.size();
}

// the fields of the comparison: adapter vector, C-ABI field id, name
static bool dumpFields(photon_gpu::Solver& s, const std::string& prefix) {
    s.sync();
    struct F { const std::vector<float>* v; int id; const char* name; };
    const F fs[] = {{&s.u, PHX_FIELD_U, "u"}, {&s.v, PHX_FIELD_V, "v"}, {&s.w, PHX_FIELD_W, "w"},
                    {&s.p, PHX_FIELD_P, "p"}, {&s.T, PHX_FIELD_T, "T"}, {&s.Yo, PHX_FIELD_YO, "Yo"},
                    {&s.Yf, PHX_FIELD_YF, "Yf"}, {&s.Ys, PHX_FIELD_YS, "Ys"}, {&s.nu, PHX_FIELD_NU, "nu"}};
    for (const F& f : fs) {
        std::vector<double> d(phx_field_count(s.handle(), f.id));
        if (phx_get_field(s.handle(), f.id, d.data(), d.size() * sizeof(double)) != PHX_OK) return false;
        if (!writeRaw(prefix + "_" + f.name + ".f32", *f.v) || !writeRaw(prefix + "_" + f.name + ".f64", d)) return false;
    }
    return true;
}

int main(int argc, char** argv) {
    const bool mixed = argc > 1 && std::string(argv[1]) == "mixed";
    const bool ckpt = argc > 2 && std::string(argv[2]) == "checkpoint";
    const bool dump = argc > 3 && std::string(argv[2]) == "dump";
    const bool caseRun = argc > 3 && std::string(argv[2]) == "case";
    if (caseRun) {
        photon_gpu::Solver c;
        if (!setupRoom(c, mixed)) return 1;
        HostState h;
        h.nx = c.nx; h.ny = c.ny; h.nz = c.nz; h.dx = c.dx;
        photon_gpu::CaseSchedule sc;
        sc.duration = 2.0f;
        sc.outputInterval = 0.5f;
        sc.checkpoint = 1.0f;
        sc.prefix = argv[3];
        const long steps = photon_gpu::runCase(c, h, sc, false, [&](HostState& host) {
            std::printf("row %.7f\n", (double)host.time);
        });
        std::printf("steps %ld\n", steps);
        return 0;
    }
    photon_gpu::Solver s;
    if (!setupRoom(s, mixed)) return 1;
    float t = 0;
    for (int i = 0; i < 40; ++i) t += s.step(0.05f);
    s.sync();
    float maxT = 0;
    for (float v : s.T) maxT = std::fmax(maxT, v);
    std::printf("time %.6f hrr %.3f maxT %.3f iters %d fuelIn %.9f maxVel %.6f cells %zu", t, s.stats.hrr, maxT,
                s.pressureIters, s.stats.fuelIn, s.maxVel, s.T.size());
    if (dump && !dumpFields(s, argv[3])) { std::printf("\ndump failed\n"); return 1; }
    if (ckpt) {
        HostState h;
        h.nx = s.nx; h.ny = s.ny; h.nz = s.nz; h.dx = s.dx;
        s.exportTo(h);
        photon_gpu::Solver r;
        if (!setupRoom(r, mixed)) return 1;
        std::string err;
        if (!r.importFrom(h, err)) { std::printf("\nimport failed: %s\n", err.c_str()); return 1; }
        r.sync();
        const bool same = r.u == h.u && r.v == h.v && r.w == h.w && r.p == h.p && r.T == h.T && r.Yf == h.Yf &&
                          r.zoneP == h.zoneP && r.lit == h.lit && r.time == h.time && r.stats.fuelIn == h.stats.fuelIn;
        for (int i = 0; i < 10; ++i) { s.step(0.05f); r.step(0.05f); }
        s.sync(); r.sync();
        const double d = std::max({maxRel(r.T, s.T), maxRel(r.u, s.u), maxRel(r.v, s.v), maxRel(r.w, s.w)});
        std::printf(" ckpt_same %d ckpt_maxrel %.3e ckpt_dtime %.3e", same ? 1 : 0, d, (double)std::fabs(r.time - s.time));
    }
    std::printf("\n");
    return 0;
}
