// Checks phx::coarseInverse, the mixed path's exact coarsest solve
// (photon_gb300/csrc/host_setup.cpp): on random sparse symmetric positive
// definite levels of 1 to 1700 unknowns, with a row that has no positive
// diagonal, A inv = I on the live rows and columns (within 1e-12), inv is
// symmetric, and the dead row and column are zero; on a singular level (a
// chain whose rows sum to zero, like a closed zone) it reports failure.
// Prints "ok" and exits 0 when every check holds.
#include <cmath>
#include <cstdio>
#include <random>

#include "host_setup.h"

using phx::MgLevel;

static MgLevel randomLevel(int n, unsigned seed) {
    MgLevel L;
    L.n = n;
    std::mt19937 rng(seed);
    std::uniform_real_distribution<double> U(0.1, 2.0);
    std::vector<std::vector<std::pair<int, double>>> rows(n);
    for (int i = 0; i < n; ++i)
        for (int k = 0; k < 3; ++k) {
            const int j = (int)(rng() % (unsigned)n);
            if (j == i) continue;
            const double w = U(rng);
            rows[i].push_back({j, w});
            rows[j].push_back({i, w});
        }
    L.diag.assign(n, 0.0);
    L.rowStart.assign(n + 1, 0);
    for (int i = 0; i < n; ++i) {
        double s = 0;
        for (auto& e : rows[i]) s += e.second;
        L.diag[i] = s + (i % 7 == 0 ? 0.5 : 0.01);   // diagonally dominant: definite
    }
    if (n > 10) L.diag[3] = 0;                      // a row without a positive diagonal
    for (int i = 0; i < n; ++i) {
        L.rowStart[i + 1] = L.rowStart[i] + (int)rows[i].size();
        for (auto& e : rows[i]) { L.col.push_back(e.first); L.val.push_back(e.second); }
    }
    return L;
}

int main() {
    bool good = true;
    for (int n : {1, 5, 63, 64, 65, 200, 900, 1700}) {
        const MgLevel L = randomLevel(n, (unsigned)n);
        std::vector<double> inv;
        if (!phx::coarseInverse(L, inv)) { std::printf("n=%d: reported singular\n", n); good = false; continue; }
        auto dead = [&](int i) { return L.diag[i] <= 0; };
        double err = 0, asym = 0, deadMax = 0;
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) {
                asym = std::max(asym, std::fabs(inv[(size_t)i * n + j] - inv[(size_t)j * n + i]));
                if (dead(i) || dead(j)) { deadMax = std::max(deadMax, std::fabs(inv[(size_t)i * n + j])); continue; }
                double s = L.diag[i] * inv[(size_t)i * n + j];
                for (int q = L.rowStart[i]; q < L.rowStart[i + 1]; ++q)
                    if (!dead(L.col[q])) s -= L.val[q] * inv[(size_t)L.col[q] * n + j];
                err = std::max(err, std::fabs(s - (i == j ? 1.0 : 0.0)));
            }
        std::printf("n=%d max|A inv - I|=%.3e asym=%.3e dead=%.1e\n", n, err, asym, deadMax);
        good = good && err <= 1e-12 && asym <= 1e-12 && deadMax == 0.0;
    }
    {   // a chain with zero row sums: singular, as a closed zone's level
        const int n = 50;
        MgLevel L;
        L.n = n;
        L.diag.assign(n, 0.0);
        L.rowStart.assign(n + 1, 0);
        for (int i = 0; i < n; ++i) {
            if (i > 0) { L.col.push_back(i - 1); L.val.push_back(1.0); L.diag[i] += 1; }
            if (i < n - 1) { L.col.push_back(i + 1); L.val.push_back(1.0); L.diag[i] += 1; }
            L.rowStart[i + 1] = (int)L.col.size();
        }
        std::vector<double> inv;
        const bool ok = phx::coarseInverse(L, inv);
        std::printf("singular chain reported %s\n", ok ? "definite" : "singular");
        good = good && !ok;
    }
    std::printf("%s\n", good ? "ok" : "FAILED");
    return good ? 0 : 1;
}
