// A Photon-style caller of photon_gpu::Solver: the ISO 9705 size room of the
// reference's gas-phase tests (src/tests/test_main.cpp:420-433) as a closed box
// at 20 cm with an open doorway, a 100 kW burner, 40 steps; prints one line of
// results for the test to check.
#include <cmath>
#include <cstdio>
#include <string>

#include "photon_gpu/solver.hpp"

int main(int argc, char** argv) {
    photon_gpu::Solver s;
    s.profile = photon_gpu::FidelityProfile::realtime();
    s.radiationOn = false;
    s.adiabaticSurfaces = true;
    if (argc > 1 && std::string(argv[1]) == "mixed") s.precision = photon_gpu::Solver::Precision::Mixed;
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
    if (!s.build(err)) { std::printf("build failed: %s\n", err.c_str()); return 1; }
    photon_gpu::Burner b;
    b.x0 = 2.4f; b.y0 = 1.0f; b.x1 = 2.8f; b.y1 = 1.4f; b.z = 0; b.peakW = 100e3f;
    if (s.addBurner(b) < 0) { std::printf("burner rejected\n"); return 1; }
    float t = 0;
    for (int i = 0; i < 40; ++i) t += s.step(0.05f);
    s.sync();
    float maxT = 0;
    for (float v : s.T) maxT = std::fmax(maxT, v);
    std::printf("time %.6f hrr %.3f maxT %.3f iters %d fuelIn %.9f maxVel %.6f cells %zu\n", t, s.stats.hrr, maxT,
                s.pressureIters, s.stats.fuelIn, s.maxVel, s.T.size());
    return 0;
}
