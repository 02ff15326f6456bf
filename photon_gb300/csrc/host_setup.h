// Host-side set-up of one scenario: pressure zones, the multigrid hierarchy
// and its coarse operator, and burner cells. These run once per geometry on the
// host (as in the reference) and are uploaded; the step itself runs on the GPU.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace phx {

struct GridGeom {
    int nx = 0, ny = 0, nz = 0;
    double dx = 0, ox = 0, oy = 0, oz = 0;
    double windSpeed = 0, windFromDeg = 0, windExp = 0.25;
    std::vector<uint8_t> blocked;
    std::vector<double> fx, fy, fz, ax, ay, az;
    std::vector<uint8_t> lx, ly, lz;
    bool anyLeak = false;
    int N() const { return nx * ny * nz; }
    int NX() const { return (nx + 1) * ny * nz; }
    int NY() const { return nx * (ny + 1) * nz; }
    int NZ() const { return nx * ny * (nz + 1); }
    int cell(int i, int j, int k) const { return i + nx * (j + ny * k); }
    int xface(int i, int j, int k) const { return i + (nx + 1) * (j + ny * k); }
    int yface(int i, int j, int k) const { return i + nx * (j + (ny + 1) * k); }
    int zface(int i, int j, int k) const { return i + nx * (j + ny * k); }
    // Solver::windAt (src/sim/gasphase.cpp:52-61)
    double windAt(int axis, int side, double z) const;
    bool bndOpen(int axis, int side, double z) const;
};

struct Zones {
    std::vector<int> zone;            // per cell, -1 solid
    std::vector<double> zoneP;        // Pa
    std::vector<uint8_t> zoneOpen;
    std::vector<double> zoneVol;      // m3
    std::vector<int> closed;          // closed zone ids
    std::vector<int> closedStart, closedCells;   // cells of each closed zone, ascending
};

// Solver::computeZones (src/sim/gasphase.cpp:111-158); Pb is updated in place
// from the zone pressures (closed zones keep the mean of their old Pb).
Zones computeZones(const GridGeom& g, std::vector<double>& Pb);

struct MgLevel {
    int n = 0;
    std::vector<int> rowStart, col;   // coarse levels
    std::vector<double> val;
    std::vector<int> bi, bj, bk;
    std::vector<int> agg;             // empty at the coarsest level
    std::vector<double> diag;
    std::vector<int> childStart, child;   // per unknown of the next level: its children here, ascending
    std::vector<double> dense;        // coarsest level: n x n operator of the coarse solve (row-major)
};

struct Multigrid {
    std::vector<double> a0x, a0y, a0z;   // level 0 coefficients, wind-inflow boundary faces closed
    std::vector<MgLevel> lv;             // lv[0]: diag and agg of the structured grid
};

// Solver::buildPressureLevels (src/sim/pressure_mg.cpp:28-191), plus the
// children lists of each aggregation and, when the coarsest level has at most
// denseMax unknowns, the dense operator of its 20 forward + backward
// Gauss-Seidel sweeps from x = 0 (pressure_mg.cpp:258-266, 279). Levels are
// added while the last one has more than coarseStop unknowns: 2000 is the
// reference's schedule (:141); a smaller stop gives a deeper hierarchy.
constexpr int MG_COARSE_STOP_REF = 2000;
// forward + backward Gauss-Seidel sweep pairs of the coarsest solve (src/sim/pressure_mg.cpp:258-266)
constexpr int MG_COARSE_SWEEPS_REF = 20;
// the coarsest solve's dense operator: the reference's sweeps from x = 0, or,
// with exact, the inverse of the coarsest matrix (dense Cholesky; the sweeps
// where the matrix is singular, as with closed zones). The FP64 path keeps the
// reference's.
struct CoarseSolve {
    int sweeps = MG_COARSE_SWEEPS_REF;
    bool exact = false;
};
Multigrid buildMultigrid(const GridGeom& g, int denseMax, int coarseStop = MG_COARSE_STOP_REF,
                         const CoarseSolve& cs = CoarseSolve());
// inverse of a level's matrix (diag - off-diagonal couplings) by dense
// Cholesky, row-major into inv; false (inv untouched) if the matrix is not
// positive definite to working precision. Rows with diag <= 0 (which the
// sweeps leave at 0) get 0 rows and columns.
bool coarseInverse(const MgLevel& L, std::vector<double>& inv);

// Solver::addBurner cell selection (src/sim/gasphase.cpp:72-90): the gas cells
// whose centres lie in the rectangle at height z + dx/2, or the centre cell.
std::vector<int> burnerCells(const GridGeom& g, double x0, double y0, double x1, double y1, double z);

}  // namespace phx
