// Host-side set-up of one scenario (see host_setup.h).
#include "host_setup.h"

#include <algorithm>
#include <cmath>
#include <limits>
#include <numeric>
#include <thread>

namespace phx {

double GridGeom::windAt(int axis, int side, double z) const {
    const double nan = std::numeric_limits<double>::quiet_NaN();
    if (windSpeed <= 0 || axis == 2) return nan;
    double th = windFromDeg * 3.14159265 / 180.0;
    double U = windSpeed * std::pow(std::max(z, 0.05) / 10.0, windExp);
    double comp = axis == 0 ? -std::sin(th) * U : -std::cos(th) * U;
    if (side == 0 && comp > 0) return comp;
    if (side == 1 && comp < 0) return comp;
    return nan;
}

bool GridGeom::bndOpen(int axis, int side, double z) const { return std::isnan(windAt(axis, side, z)); }

Zones computeZones(const GridGeom& g, std::vector<double>& Pb) {
    const int N = g.N(), nx = g.nx, ny = g.ny, nz = g.nz, sxy = nx * ny;
    const double P0 = 101325.0;
    std::vector<double> oldPb = Pb;
    Zones Z;
    Z.zone.assign(N, -1);
    std::vector<double> pSum, vSum;
    std::vector<int> stack;
    for (int seed = 0; seed < N; ++seed) {
        if (g.blocked[seed] || Z.zone[seed] >= 0) continue;
        int z = (int)Z.zoneP.size();
        Z.zoneP.push_back(P0);
        Z.zoneOpen.push_back(0);
        pSum.push_back(0);
        vSum.push_back(0);
        stack.clear();
        stack.push_back(seed);
        Z.zone[seed] = z;
        while (!stack.empty()) {
            int c = stack.back();
            stack.pop_back();
            pSum[z] += oldPb.empty() ? P0 : oldPb[c];
            vSum[z] += 1;
            int i = c % nx, j = (c / nx) % ny, k = c / sxy;
            double a[6] = {g.ax[g.xface(i, j, k)], g.ax[g.xface(i + 1, j, k)], g.ay[g.yface(i, j, k)],
                           g.ay[g.yface(i, j + 1, k)], g.az[g.zface(i, j, k)], g.az[g.zface(i, j, k + 1)]};
            int nb[6] = {i > 0 ? c - 1 : -1, i < nx - 1 ? c + 1 : -1, j > 0 ? c - nx : -1, j < ny - 1 ? c + nx : -1,
                         k > 0 ? c - sxy : -1, k < nz - 1 ? c + sxy : -1};
            for (int d = 0; d < 6; ++d) {
                if (a[d] <= 0) continue;
                if (nb[d] < 0) { if (d != 4) Z.zoneOpen[z] = 1; continue; }
                if (g.blocked[nb[d]] || Z.zone[nb[d]] >= 0) continue;
                Z.zone[nb[d]] = z;
                stack.push_back(nb[d]);
            }
        }
    }
    const int nZ = (int)Z.zoneP.size();
    for (int z = 0; z < nZ; ++z) Z.zoneP[z] = Z.zoneOpen[z] ? P0 : pSum[z] / std::max(1.0, vSum[z]);
    for (int c = 0; c < N; ++c) Pb[c] = Z.zone[c] >= 0 ? Z.zoneP[Z.zone[c]] : P0;
    Z.zoneVol.assign(nZ, 0.0);
    for (int z = 0; z < nZ; ++z) Z.zoneVol[z] = vSum[z] * g.dx * g.dx * g.dx;
    // closed zones and their cells in ascending order
    std::vector<int> slot(nZ, -1);
    for (int z = 0; z < nZ; ++z)
        if (!Z.zoneOpen[z]) { slot[z] = (int)Z.closed.size(); Z.closed.push_back(z); }
    Z.closedStart.assign(Z.closed.size() + 1, 0);
    for (int c = 0; c < N; ++c)
        if (Z.zone[c] >= 0 && slot[Z.zone[c]] >= 0) Z.closedStart[slot[Z.zone[c]] + 1]++;
    for (size_t q = 0; q < Z.closed.size(); ++q) Z.closedStart[q + 1] += Z.closedStart[q];
    Z.closedCells.assign(Z.closedStart.back(), 0);
    std::vector<int> fill(Z.closed.size(), 0);
    for (int c = 0; c < N; ++c)
        if (Z.zone[c] >= 0 && slot[Z.zone[c]] >= 0) {
            int q = slot[Z.zone[c]];
            Z.closedCells[Z.closedStart[q] + fill[q]++] = c;
        }
    return Z;
}

namespace {
struct UnionFind {
    std::vector<int> p;
    explicit UnionFind(int n) : p(n) { std::iota(p.begin(), p.end(), 0); }
    int find(int a) {
        while (p[a] != a) a = p[a] = p[p[a]];
        return a;
    }
    void join(int a, int b) {
        a = find(a);
        b = find(b);
        if (a != b) p[std::max(a, b)] = std::min(a, b);
    }
};

// coupling rows kept in first-insertion order, as the reference's vectors of pairs
struct Rows {
    std::vector<std::vector<std::pair<int, double>>> r;
    explicit Rows(int n) : r(n) {}
    void add(int row, int col, double w) {
        for (auto& e : r[row])
            if (e.first == col) { e.second += w; return; }
        r[row].push_back({col, w});
    }
};

void toCsr(MgLevel& C, const Rows& rows, const std::vector<double>& dg) {
    C.diag.resize(C.n);
    C.rowStart.assign(C.n + 1, 0);
    for (int I = 0; I < C.n; ++I) {
        C.diag[I] = std::max(dg[I], 0.0);
        C.rowStart[I + 1] = C.rowStart[I] + (int)rows.r[I].size();
    }
    C.col.reserve(C.rowStart[C.n]);
    C.val.reserve(C.rowStart[C.n]);
    for (int I = 0; I < C.n; ++I)
        for (auto& e : rows.r[I]) { C.col.push_back(e.first); C.val.push_back(e.second); }
}

void childrenOf(MgLevel& F, int nCoarse) {
    F.childStart.assign(nCoarse + 1, 0);
    for (int I = 0; I < F.n; ++I)
        if (F.agg[I] >= 0) F.childStart[F.agg[I] + 1]++;
    for (int J = 0; J < nCoarse; ++J) F.childStart[J + 1] += F.childStart[J];
    F.child.assign(F.childStart[nCoarse], 0);
    std::vector<int> fill(nCoarse, 0);
    for (int I = 0; I < F.n; ++I)
        if (F.agg[I] >= 0) F.child[F.childStart[F.agg[I]] + fill[F.agg[I]]++] = I;
}

// one Gauss-Seidel sweep of the coarsest level (gsSparseSweep)
void gsSweep(const MgLevel& L, const double* b, double* x, bool forward) {
    for (int t = 0; t < L.n; ++t) {
        int I = forward ? t : L.n - 1 - t;
        if (L.diag[I] <= 0) { x[I] = 0; continue; }
        double s = b[I];
        for (int q = L.rowStart[I]; q < L.rowStart[I + 1]; ++q) s += L.val[q] * x[L.col[q]];
        x[I] = s / L.diag[I];
    }
}
}  // namespace

namespace {
// the host's worker threads for a loop over [0, n) in contiguous chunks
template <class F>
void parallelFor(int n, long long work, F f) {
    int nt = (int)std::min<unsigned>(16, std::max(1u, std::thread::hardware_concurrency()));
    if (work < 200000) nt = 1;
    nt = std::max(1, std::min(nt, n));
    if (nt == 1) { f(0, n); return; }
    std::vector<std::thread> pool;
    for (int t = 0; t < nt; ++t) pool.emplace_back(f, (int)((long long)n * t / nt), (int)((long long)n * (t + 1) / nt));
    for (auto& th : pool) th.join();
}
}  // namespace

bool coarseInverse(const MgLevel& L, std::vector<double>& inv) {
    const int n = L.n;
    const size_t nn = (size_t)n * n;
    // the matrix, lower triangle used: diag on the diagonal, minus the couplings off it;
    // rows without a positive diagonal become identity rows (their output is zeroed below)
    std::vector<double> A(nn, 0.0);
    std::vector<char> dead(n, 0);
    for (int I = 0; I < n; ++I) {
        if (L.diag[I] <= 0) { dead[I] = 1; A[(size_t)I * n + I] = 1.0; continue; }
        A[(size_t)I * n + I] = L.diag[I];
    }
    for (int I = 0; I < n; ++I) {
        if (dead[I]) continue;
        for (int q = L.rowStart[I]; q < L.rowStart[I + 1]; ++q)
            if (!dead[L.col[q]]) A[(size_t)I * n + L.col[q]] -= L.val[q];
    }
    std::vector<double> d0(n);
    for (int I = 0; I < n; ++I) d0[I] = A[(size_t)I * n + I];
    // right-looking blocked Cholesky A = L L^T in the lower triangle; the trailing
    // update of each block step is split over rows
    constexpr int B = 64;
    for (int k0 = 0; k0 < n; k0 += B) {
        const int k1 = std::min(n, k0 + B);
        for (int j = k0; j < k1; ++j) {   // the diagonal block
            double* rj = &A[(size_t)j * n];
            double dj = rj[j];
            for (int k = k0; k < j; ++k) dj -= rj[k] * rj[k];
            if (!(dj > 1e-10 * d0[j])) return false;   // not positive definite: a singular (closed) zone
            dj = std::sqrt(dj);
            rj[j] = dj;
            for (int i = j + 1; i < k1; ++i) {
                double* ri = &A[(size_t)i * n];
                double v = ri[j];
                for (int k = k0; k < j; ++k) v -= ri[k] * rj[k];
                ri[j] = v / dj;
            }
        }
        // the panel below the block (rows independent), then the trailing matrix,
        // which reads other rows' panel entries: two passes, each split over rows
        parallelFor(n - k1, (long long)(n - k1) * (k1 - k0) * (k1 - k0), [&](int a, int b) {
            for (int i = k1 + a; i < k1 + b; ++i) {
                double* ri = &A[(size_t)i * n];
                for (int j = k0; j < k1; ++j) {
                    const double* rj = &A[(size_t)j * n];
                    double v = ri[j];
                    for (int k = k0; k < j; ++k) v -= ri[k] * rj[k];
                    ri[j] = v / rj[j];
                }
            }
        });
        parallelFor(n - k1, (long long)(n - k1) * (n - k1) * (k1 - k0) / 2, [&](int a, int b) {
            for (int i = k1 + a; i < k1 + b; ++i) {
                double* ri = &A[(size_t)i * n];
                for (int j = k1; j <= i; ++j) {
                    const double* rj = &A[(size_t)j * n];
                    double v = 0;
                    for (int k = k0; k < k1; ++k) v += ri[k] * rj[k];
                    ri[j] -= v;
                }
            }
        });
    }
    // columns of the inverse: L y = e_j, then L^T x = y (L^T read from a transposed copy)
    std::vector<double> U(nn, 0.0);
    for (int i = 0; i < n; ++i)
        for (int k = 0; k <= i; ++k) U[(size_t)k * n + i] = A[(size_t)i * n + k];
    inv.assign(nn, 0.0);
    parallelFor(n, (long long)n * n * n / 2, [&](int a, int b) {
        std::vector<double> y(n);
        for (int j = a; j < b; ++j) {
            std::fill(y.begin(), y.end(), 0.0);
            for (int i = j; i < n; ++i) {
                const double* ri = &A[(size_t)i * n];
                double v = i == j ? 1.0 : 0.0;
                for (int k = j; k < i; ++k) v -= ri[k] * y[k];
                y[i] = v / ri[i];
            }
            for (int i = n - 1; i >= 0; --i) {
                const double* ui = &U[(size_t)i * n];
                double v = y[i];
                for (int k = i + 1; k < n; ++k) v -= ui[k] * y[k];
                y[i] = v / ui[i];
            }
            for (int i = 0; i < n; ++i) inv[(size_t)i * n + j] = (dead[i] || dead[j]) ? 0.0 : y[i];
        }
    });
    return true;
}

Multigrid buildMultigrid(const GridGeom& g, int denseMax, int coarseStop, const CoarseSolve& cs) {
    Multigrid M;
    const int nx = g.nx, ny = g.ny, nz = g.nz, n0 = g.N(), sxy = nx * ny;
    M.a0x = g.ax;
    M.a0y = g.ay;
    M.a0z = g.az;
    for (int k = 0; k < nz; ++k) {
        double z = g.oz + (k + 0.5) * g.dx;
        for (int j = 0; j < ny; ++j) {
            if (!g.bndOpen(0, 0, z)) M.a0x[g.xface(0, j, k)] = 0;
            if (!g.bndOpen(0, 1, z)) M.a0x[g.xface(nx, j, k)] = 0;
        }
        for (int i = 0; i < nx; ++i) {
            if (!g.bndOpen(1, 0, z)) M.a0y[g.yface(i, 0, k)] = 0;
            if (!g.bndOpen(1, 1, z)) M.a0y[g.yface(i, ny, k)] = 0;
        }
    }
    M.lv.emplace_back();
    MgLevel& L0 = M.lv[0];
    L0.n = n0;
    L0.diag.assign(n0, 0.0);
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                int c = g.cell(i, j, k);
                if (g.blocked[c]) continue;
                L0.diag[c] = M.a0x[g.xface(i, j, k)] + M.a0x[g.xface(i + 1, j, k)] + M.a0y[g.yface(i, j, k)] +
                             M.a0y[g.yface(i, j + 1, k)] + M.a0z[g.zface(i, j, k)] + M.a0z[g.zface(i, j, k + 1)];
            }
    // level 1: connected pieces of 2x2x2 blocks, joined through open faces
    {
        UnionFind uf(n0);
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i) {
                    int c = g.cell(i, j, k);
                    if (L0.diag[c] <= 0) continue;
                    if (i + 1 < nx && (i >> 1) == ((i + 1) >> 1) && M.a0x[g.xface(i + 1, j, k)] > 0 && L0.diag[c + 1] > 0) uf.join(c, c + 1);
                    if (j + 1 < ny && (j >> 1) == ((j + 1) >> 1) && M.a0y[g.yface(i, j + 1, k)] > 0 && L0.diag[c + nx] > 0) uf.join(c, c + nx);
                    if (k + 1 < nz && (k >> 1) == ((k + 1) >> 1) && M.a0z[g.zface(i, j, k + 1)] > 0 && L0.diag[c + sxy] > 0) uf.join(c, c + sxy);
                }
        L0.agg.assign(n0, -1);
        std::vector<int> rootId(n0, -1);
        MgLevel C;
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i) {
                    int c = g.cell(i, j, k);
                    if (L0.diag[c] <= 0) continue;
                    int r = uf.find(c);
                    if (rootId[r] < 0) {
                        rootId[r] = C.n++;
                        C.bi.push_back(i >> 1); C.bj.push_back(j >> 1); C.bk.push_back(k >> 1);
                    }
                    L0.agg[c] = rootId[r];
                }
        // Galerkin product: couplings between aggregates, diagonal = fine
        // coefficients leaving the aggregate
        Rows rows(C.n);
        std::vector<double> dg(C.n, 0.0);
        auto couple = [&](int a, int b, double w) {
            if (w <= 0) return;
            int A = L0.agg[a], B = L0.agg[b];
            if (A < 0 || B < 0 || A == B) return;
            rows.add(A, B, w);
            rows.add(B, A, w);
        };
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i) {
                    int c = g.cell(i, j, k);
                    if (L0.diag[c] <= 0) continue;
                    if (i + 1 < nx) couple(c, c + 1, M.a0x[g.xface(i + 1, j, k)]);
                    if (j + 1 < ny) couple(c, c + nx, M.a0y[g.yface(i, j + 1, k)]);
                    if (k + 1 < nz) couple(c, c + sxy, M.a0z[g.zface(i, j, k + 1)]);
                }
        for (int c = 0; c < n0; ++c) if (L0.agg[c] >= 0) dg[L0.agg[c]] += L0.diag[c];
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i) {
                    int c = g.cell(i, j, k);
                    if (L0.diag[c] <= 0) continue;
                    auto inner = [&](int n2, double w) { if (w > 0 && L0.agg[n2] == L0.agg[c]) dg[L0.agg[c]] -= 2.0 * w; };
                    if (i + 1 < nx && L0.diag[c + 1] > 0) inner(c + 1, M.a0x[g.xface(i + 1, j, k)]);
                    if (j + 1 < ny && L0.diag[c + nx] > 0) inner(c + nx, M.a0y[g.yface(i, j + 1, k)]);
                    if (k + 1 < nz && L0.diag[c + sxy] > 0) inner(c + sxy, M.a0z[g.zface(i, j, k + 1)]);
                }
        toCsr(C, rows, dg);
        childrenOf(M.lv[0], C.n);
        M.lv.push_back(std::move(C));
    }
    // coarser levels: connected pieces of 2x2x2 groups of block coordinates
    while (M.lv.back().n > coarseStop && M.lv.size() < 12) {
        MgLevel& F = M.lv.back();
        UnionFind uf(F.n);
        for (int I = 0; I < F.n; ++I)
            for (int e = F.rowStart[I]; e < F.rowStart[I + 1]; ++e) {
                int J = F.col[e];
                if (J > I && (F.bi[I] >> 1) == (F.bi[J] >> 1) && (F.bj[I] >> 1) == (F.bj[J] >> 1) && (F.bk[I] >> 1) == (F.bk[J] >> 1))
                    uf.join(I, J);
            }
        F.agg.assign(F.n, -1);
        std::vector<int> rootId(F.n, -1);
        MgLevel C;
        for (int I = 0; I < F.n; ++I) {
            int r = uf.find(I);
            if (rootId[r] < 0) {
                rootId[r] = C.n++;
                C.bi.push_back(F.bi[I] >> 1); C.bj.push_back(F.bj[I] >> 1); C.bk.push_back(F.bk[I] >> 1);
            }
            F.agg[I] = rootId[r];
        }
        if (C.n > 0.8 * F.n) { F.agg.clear(); break; }
        Rows rows(C.n);
        std::vector<double> dg(C.n, 0.0);
        for (int I = 0; I < F.n; ++I) dg[F.agg[I]] += F.diag[I];
        for (int I = 0; I < F.n; ++I)
            for (int e = F.rowStart[I]; e < F.rowStart[I + 1]; ++e) {
                int A = F.agg[I], B = F.agg[F.col[e]];
                if (A == B) { dg[A] -= F.val[e]; continue; }
                rows.add(A, B, F.val[e]);
            }
        toCsr(C, rows, dg);
        childrenOf(F, C.n);
        M.lv.push_back(std::move(C));
    }
    // dense operator of the coarsest solve: the exact inverse where asked for and
    // the matrix is definite; else column j = the sweeps applied to e_j
    MgLevel& Lc = M.lv.back();
    if (Lc.n <= denseMax && !(cs.exact && coarseInverse(Lc, Lc.dense))) {
        const int n = Lc.n;
        Lc.dense.assign((size_t)n * n, 0.0);
        // columns are independent: split them over the host's threads
        auto cols = [&](int j0, int j1) {
            std::vector<double> b(n, 0.0), x(n, 0.0);
            for (int jcol = j0; jcol < j1; ++jcol) {
                std::fill(b.begin(), b.end(), 0.0);
                std::fill(x.begin(), x.end(), 0.0);
                b[jcol] = 1.0;
                for (int it = 0; it < cs.sweeps; ++it) {
                    gsSweep(Lc, b.data(), x.data(), true);
                    gsSweep(Lc, b.data(), x.data(), false);
                }
                for (int i = 0; i < n; ++i) Lc.dense[(size_t)i * n + jcol] = x[i];
            }
        };
        int nt = (int)std::min<unsigned>(16, std::max(1u, std::thread::hardware_concurrency()));
        if ((long long)n * n < 200000) nt = 1;
        std::vector<std::thread> pool;
        for (int t = 0; t < nt; ++t) pool.emplace_back(cols, (int)((long long)n * t / nt), (int)((long long)n * (t + 1) / nt));
        for (auto& th : pool) th.join();
    }
    return M;
}

std::vector<int> burnerCells(const GridGeom& g, double x0, double y0, double x1, double y1, double z) {
    std::vector<int> cells;
    auto cellAt = [&](double x, double y, double zz) -> int {
        int i = (int)std::floor((x - g.ox) / g.dx), j = (int)std::floor((y - g.oy) / g.dx), k = (int)std::floor((zz - g.oz) / g.dx);
        if (i < 0 || j < 0 || k < 0 || i >= g.nx || j >= g.ny || k >= g.nz) return -1;
        return g.cell(i, j, k);
    };
    for (int j = 0; j < g.ny; ++j)
        for (int i = 0; i < g.nx; ++i) {
            double x = g.ox + (i + 0.5) * g.dx, y = g.oy + (j + 0.5) * g.dx;
            if (x < x0 || x > x1 || y < y0 || y > y1) continue;
            int c = cellAt(x, y, z + 0.5 * g.dx);
            if (c >= 0 && !g.blocked[c]) cells.push_back(c);
        }
    if (cells.empty()) {
        int c = cellAt(0.5 * (x0 + x1), 0.5 * (y0 + y1), z + 0.5 * g.dx);
        if (c >= 0 && !g.blocked[c]) cells.push_back(c);
    }
    return cells;
}

}  // namespace phx
