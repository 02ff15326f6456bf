/* FP64 CPU restatement of Photon's gas-phase step -- TEST INFRASTRUCTURE ONLY.
 *
 * The oracle for the CUDA path (see phx_oracle.h). Only tests/, the smoke test
 * and the CPU-baseline leg of bench.py load it; the product never does.
 *
 * Every real is double. Expressions keep the reference's evaluation order
 * (left to right, as written), reductions keep its order (z-slice partials
 * summed in slice order), and std::min / std::max / std::clamp are restated as
 * the comparisons libstdc++ performs, so results match the reference source
 * compiled at FP64 bit for bit. The one addition is a relative residual test
 * for the pressure solve (relTol), off by default.
 *
 * Scope: the gas-only step used by the synthetic workloads -- no solid fuel
 * cells and no barriers, with radiation either off or adiabatic surfaces on
 * (then the radiative fraction is a local sink). Crack faces (lx/ly/lz) and
 * closed zones are handled as in the reference.
 */
#include "phx_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* constants of the model: src/sim/solver.h:159-181, src/sim/gasphase.cpp:25-32,
 * src/sim/solver.cpp:15-20 */
#define T0 293.15
#define P0 101325.0
#define RS 287.0
#define CP 1100.0
#define GRAV 9.81
#define YO2_AMB 0.232
#define DHC_FUEL 25.0e6
#define S_O2 1.95
#define Y_H2O 0.761
#define C_FRAC 0.597
#define CO_YIELD 0.02
#define YCO2_AMB 0.0006
#define YH2O_AMB 0.0073
#define CHI_R 0.35
#define T_CRIT 1600.0
#define T_AUTO 800.0
#define TAU_MIX 0.1
#define PR_T 0.5
#define SC_T 0.5
#define C_NU 0.1
#define CD_LEAK 1.0
#define LEAK_VMAX 40.0
#define D_MAX 50.0
#define VMAX 40.0
#define T_MIN 200.0
#define T_MAX 2300.0
#define BURNER_SOOT 0.01
static const double GAMMA = CP / (CP - RS);

/* libstdc++'s std::min, std::max and std::clamp */
static inline double mn(double a, double b) { return (b < a) ? b : a; }
static inline double mx(double a, double b) { return (a < b) ? b : a; }
static inline double clampd(double v, double lo, double hi) { return (v < lo) ? lo : (hi < v) ? hi : v; }

typedef struct {
    int n, nx, ny, nz;
    double *ax, *ay, *az;           /* level 0 */
    int *rowStart, *col, nnz;       /* coarse levels */
    double* val;
    int *bi, *bj, *bk;
    int* agg;                       /* NULL when this level is the coarsest */
    double *diag, *x, *b, *r, *t;
} Level;

typedef struct {
    double x0, y0, x1, y1, z, peakW, rampS, start, duration;
    int* cells;
    int ncells;
} OBurner;

typedef struct {
    int cell;
    double power, start, duration;
} OIgnition;

typedef struct {
    int axis, f, a, b;
} LeakFace;

struct Orc {
    int nx, ny, nz, N, NX, NY, NZ;
    double dx, ox, oy, oz;
    double cfl, dtMaxP, tol, relTol;
    int maxIters;
    int radiationOn, adiabatic;
    double windSpeed, windFrom, windExp;
    double *u, *v, *w, *fx, *fy, *fz, *ax, *ay, *az;
    uint8_t *lx, *ly, *lz;
    double *p, *S, *T, *Yo, *Yf, *Ys, *Ya, *Yp, *Yc, *Yw, *Yco, *Yai, *nu, *Pb, *Q, *Qr, *hrr, *massSrc;
    uint8_t *lit, *pilot, *blocked;
    int* zone;
    int nZones;
    double *zoneP, *zoneVol, *zoneDP;
    uint8_t* zoneOpen;
    double* tmp[12];
    double *u2, *v2, *w2, *rhs, *cgR, *cgZ, *cgP, *cgQ;
    int nLevels;
    Level lv[12];
    int mgDirty, zonesDirty;
    OBurner* burners;
    int nBurners;
    OIgnition* ign;
    int nIgn;
    int coarseMode;
    double time, maxVel, maxNu, maxDiv, pressureResidual;
    int pressureIters, leakFaces;
    double st_hrr, st_maxGasT, st_fuelIn, st_fuelBurned, st_fuelInDomain;
    int st_burning;
};

static double* dalloc(size_t n, double v) {
    double* a = (double*)malloc((n ? n : 1) * sizeof(double));
    for (size_t i = 0; i < n; ++i) a[i] = v;
    return a;
}
static uint8_t* balloc(size_t n) { return (uint8_t*)calloc(n ? n : 1, 1); }

static inline int cellI(const Orc* o, int i, int j, int k) { return i + o->nx * (j + o->ny * k); }
static inline int xfaceI(const Orc* o, int i, int j, int k) { return i + (o->nx + 1) * (j + o->ny * k); }
static inline int yfaceI(const Orc* o, int i, int j, int k) { return i + o->nx * (j + (o->ny + 1) * k); }
static inline int zfaceI(const Orc* o, int i, int j, int k) { return i + o->nx * (j + o->ny * k); }
static inline double gasDensity(const Orc* o, int c) { return o->Pb[c] / (RS * o->T[c]); }

/* allocation mirrors Solver::build, src/sim/discretize.cpp:24-62 */
Orc* orc_new(int nx, int ny, int nz, double dx, double ox, double oy, double oz) {
    Orc* o = (Orc*)calloc(1, sizeof(Orc));
    o->nx = nx; o->ny = ny; o->nz = nz; o->N = nx * ny * nz;
    o->NX = (nx + 1) * ny * nz; o->NY = nx * (ny + 1) * nz; o->NZ = nx * ny * (nz + 1);
    o->dx = dx; o->ox = ox; o->oy = oy; o->oz = oz;
    o->cfl = 0.5; o->dtMaxP = 0.02; o->maxIters = 400; o->tol = 0.002; o->relTol = 0;
    o->radiationOn = 1; o->adiabatic = 1; o->windExp = 0.25;
    int N = o->N;
    o->u = dalloc(o->NX, 0); o->v = dalloc(o->NY, 0); o->w = dalloc(o->NZ, 0);
    o->fx = dalloc(o->NX, 1); o->fy = dalloc(o->NY, 1); o->fz = dalloc(o->NZ, 1);
    o->ax = dalloc(o->NX, 0); o->ay = dalloc(o->NY, 0); o->az = dalloc(o->NZ, 0);
    o->lx = balloc(o->NX); o->ly = balloc(o->NY); o->lz = balloc(o->NZ);
    o->p = dalloc(N, 0); o->S = dalloc(N, 0); o->T = dalloc(N, T0); o->Yo = dalloc(N, YO2_AMB);
    o->Yf = dalloc(N, 0); o->Ys = dalloc(N, 0); o->Ya = dalloc(N, 0); o->Yp = dalloc(N, 0);
    o->Yc = dalloc(N, YCO2_AMB); o->Yw = dalloc(N, YH2O_AMB); o->Yco = dalloc(N, 0); o->Yai = dalloc(N, 0);
    o->nu = dalloc(N, 0); o->Pb = dalloc(N, P0); o->Q = dalloc(N, 0); o->Qr = dalloc(N, 0);
    o->hrr = dalloc(N, 0); o->massSrc = dalloc(N, 0);
    o->lit = balloc(N); o->pilot = balloc(N); o->blocked = balloc(N);
    o->zone = (int*)malloc(N * sizeof(int));
    for (int c = 0; c < N; ++c) o->zone[c] = -1;
    for (int q = 0; q < 12; ++q) o->tmp[q] = dalloc(N, 0);
    o->u2 = dalloc(o->NX, 0); o->v2 = dalloc(o->NY, 0); o->w2 = dalloc(o->NZ, 0);
    o->rhs = dalloc(N, 0); o->cgR = dalloc(N, 0); o->cgZ = dalloc(N, 0); o->cgP = dalloc(N, 0); o->cgQ = dalloc(N, 0);
    o->mgDirty = 1; o->zonesDirty = 1;
    return o;
}

static void free_levels(Orc* o) {
    for (int l = 0; l < o->nLevels; ++l) {
        Level* L = &o->lv[l];
        free(L->ax); free(L->ay); free(L->az); free(L->rowStart); free(L->col); free(L->val);
        free(L->bi); free(L->bj); free(L->bk); free(L->agg);
        free(L->diag); free(L->x); free(L->b); free(L->r); free(L->t);
        memset(L, 0, sizeof(Level));
    }
    o->nLevels = 0;
}

void orc_free(Orc* o) {
    if (!o) return;
    free_levels(o);
    double* ds[] = {o->u, o->v, o->w, o->fx, o->fy, o->fz, o->ax, o->ay, o->az, o->p, o->S, o->T, o->Yo, o->Yf,
                    o->Ys, o->Ya, o->Yp, o->Yc, o->Yw, o->Yco, o->Yai, o->nu, o->Pb, o->Q, o->Qr, o->hrr, o->massSrc,
                    o->u2, o->v2, o->w2, o->rhs, o->cgR, o->cgZ, o->cgP, o->cgQ, o->zoneP, o->zoneVol, o->zoneDP};
    for (size_t i = 0; i < sizeof(ds) / sizeof(ds[0]); ++i) free(ds[i]);
    for (int q = 0; q < 12; ++q) free(o->tmp[q]);
    free(o->lx); free(o->ly); free(o->lz); free(o->lit); free(o->pilot); free(o->blocked);
    free(o->zone); free(o->zoneOpen);
    for (int b = 0; b < o->nBurners; ++b) free(o->burners[b].cells);
    free(o->burners); free(o->ign);
    free(o);
}

void orc_set_profile(Orc* o, double cfl, double dtMax, int maxIters, double tol, double relTol) {
    o->cfl = cfl; o->dtMaxP = dtMax; o->maxIters = maxIters; o->tol = tol; o->relTol = relTol;
}
void orc_set_switches(Orc* o, int radiationOn, int adiabatic) { o->radiationOn = radiationOn; o->adiabatic = adiabatic; }
void orc_set_wind(Orc* o, double speed, double fromDeg, double exponent) {
    o->windSpeed = speed; o->windFrom = fromDeg; o->windExp = exponent;
}
void orc_mark_geometry_dirty(Orc* o) { o->zonesDirty = 1; o->mgDirty = 1; }
void orc_set_coarse_mode(Orc* o, int mode) { o->coarseMode = mode; }

/* Solver::cellAt, src/sim/solver.cpp:44-48 */
static int cellAt(const Orc* o, double x, double y, double z) {
    int i = (int)floor((x - o->ox) / o->dx), j = (int)floor((y - o->oy) / o->dx), k = (int)floor((z - o->oz) / o->dx);
    if (i < 0 || j < 0 || k < 0 || i >= o->nx || j >= o->ny || k >= o->nz) return -1;
    return cellI(o, i, j, k);
}

/* Solver::windAt, src/sim/gasphase.cpp:52-61 */
static double windAt(const Orc* o, int axis, int side, double z) {
    if (o->windSpeed <= 0 || axis == 2) return NAN;
    double th = o->windFrom * 3.14159265 / 180.0;
    double U = o->windSpeed * pow(mx(z, 0.05) / 10.0, o->windExp);
    double comp = axis == 0 ? -sin(th) * U : -cos(th) * U;
    if (side == 0 && comp > 0) return comp;
    if (side == 1 && comp < 0) return comp;
    return NAN;
}
static inline int bndOpen(const Orc* o, int axis, int side, double z) { return isnan(windAt(o, axis, side, z)); }

/* Solver::stableDt, src/sim/gasphase.cpp:63-70 */
double orc_stable_dt(Orc* o, double dtMax) {
    double dt = mn(dtMax, o->dtMaxP);
    dt = mn(dt, o->cfl * o->dx / mx(o->maxVel, 0.1));
    double alpha = o->maxNu * (1.0 + 1.0 / PR_T);
    if (alpha > 0) dt = mn(dt, 0.9 * o->dx * o->dx / (6.0 * alpha));
    if (o->maxDiv > 0) dt = mn(dt, 0.25 / o->maxDiv);
    return mx(dt, 1e-3);
}

/* Solver::addBurner, src/sim/gasphase.cpp:72-90 */
int orc_add_burner(Orc* o, double x0, double y0, double x1, double y1, double z, double peakW, double rampS,
                   double start, double duration) {
    OBurner b;
    b.x0 = x0; b.y0 = y0; b.x1 = x1; b.y1 = y1; b.z = z; b.peakW = peakW; b.rampS = rampS;
    b.start = start; b.duration = duration;
    b.cells = (int*)malloc((size_t)o->nx * o->ny * sizeof(int) + sizeof(int));
    b.ncells = 0;
    for (int j = 0; j < o->ny; ++j)
        for (int i = 0; i < o->nx; ++i) {
            double x = o->ox + (i + 0.5) * o->dx, y = o->oy + (j + 0.5) * o->dx;
            if (x < b.x0 || x > b.x1 || y < b.y0 || y > b.y1) continue;
            int c = cellAt(o, x, y, b.z + 0.5 * o->dx);
            if (c >= 0 && !o->blocked[c]) b.cells[b.ncells++] = c;
        }
    if (b.ncells == 0) {
        int c = cellAt(o, 0.5 * (b.x0 + b.x1), 0.5 * (b.y0 + b.y1), b.z + 0.5 * o->dx);
        if (c < 0 || o->blocked[c]) { free(b.cells); return -1; }
        b.cells[b.ncells++] = c;
    }
    o->burners = (OBurner*)realloc(o->burners, (o->nBurners + 1) * sizeof(OBurner));
    o->burners[o->nBurners] = b;
    return o->nBurners++;
}

int orc_burner_cells(Orc* o, int b, int* out, int cap) {
    if (b < 0 || b >= o->nBurners) return -1;
    for (int i = 0; i < o->burners[b].ncells && i < cap; ++i) out[i] = o->burners[b].cells[i];
    return o->burners[b].ncells;
}

/* Solver::addIgnition, src/sim/solver.cpp:122-134 (the event text is not restated) */
void orc_add_ignition(Orc* o, int cell, double power, double duration) {
    if (cell < 0 || cell >= o->N) return;
    o->ign = (OIgnition*)realloc(o->ign, (o->nIgn + 1) * sizeof(OIgnition));
    OIgnition g = {cell, power, o->time, duration};
    o->ign[o->nIgn++] = g;
}

/* Burner::powerAt, src/sim/solver.h:122-126 */
static double powerAt(const OBurner* b, double t) {
    if (t < b->start || t > b->start + b->duration) return 0;
    double r = b->rampS > 0 ? mn(1.0, (t - b->start) / b->rampS) : 1.0;
    return b->peakW * r * r;
}

/* Solver::addGasSpecies, src/sim/solver.cpp:212-223 */
static void addGasSpecies(Orc* o, int c, double fuelGen, double aerosol, double sootPot, double ait) {
    double m = gasDensity(o, c) * o->dx * o->dx * o->dx;
    double madd = fuelGen + aerosol;
    if (madd <= 0) return;
    double mt = m + madd, sc = m / mt;
    o->Yo[c] *= sc; o->Ys[c] *= sc; o->Yc[c] *= sc; o->Yw[c] *= sc; o->Yco[c] *= sc;
    o->Yai[c] = o->Yai[c] * sc + fuelGen * ait / mt;
    o->Yf[c] = o->Yf[c] * sc + fuelGen / mt;
    o->Ya[c] = o->Ya[c] * sc + aerosol / mt;
    o->Yp[c] = o->Yp[c] * sc + sootPot / mt;
    o->massSrc[c] += madd;
}

/* Solver::injectIgnitions, src/sim/solver.cpp:271-280 */
static void injectIgnitions(Orc* o, double dt) {
    for (int g = 0; g < o->nIgn; ++g) {
        OIgnition* ig = &o->ign[g];
        if (o->time < ig->start || o->time > ig->start + ig->duration) continue;
        if (o->blocked[ig->cell]) continue;
        double mf = ig->power * dt / DHC_FUEL;
        addGasSpecies(o, ig->cell, mf, 0, mf * BURNER_SOOT, T_AUTO);
        o->st_fuelIn += mf;
        o->pilot[ig->cell] = 1;
    }
}

/* Solver::injectBurners, src/sim/gasphase.cpp:92-105 */
static void injectBurners(Orc* o, double dt) {
    for (int bi = 0; bi < o->nBurners; ++bi) {
        OBurner* b = &o->burners[bi];
        double P = powerAt(b, o->time);
        if (P <= 0) continue;
        double mf = P * dt / DHC_FUEL / b->ncells;
        for (int q = 0; q < b->ncells; ++q) {
            int c = b->cells[q];
            if (o->blocked[c]) continue;
            addGasSpecies(o, c, mf, 0, mf * BURNER_SOOT, T_AUTO);
            o->st_fuelIn += mf;
            o->pilot[c] = 1;
        }
    }
}

/* Solver::combustion, src/sim/solver.cpp:284-344 */
static void combustion(Orc* o, double dt) {
    const double V = o->dx * o->dx * o->dx;
    const double s = S_O2;
    const double frac = 1.0 - exp(-dt / TAU_MIX);
    const double chiR = o->radiationOn ? CHI_R : 0.0;
    const int nx = o->nx, ny = o->ny, nz = o->nz, sx = 1, sy = nx, sz = nx * ny;
    double* litNew = o->tmp[0];
    for (int c = 0; c < o->N; ++c) {
        litNew[c] = 0;
        o->hrr[c] = 0;
        if (o->blocked[c]) continue;
        double yf = o->Yf[c];
        if (yf < 1e-6) continue;
        double Tc = o->T[c];
        double ait = yf > 1e-9 ? o->Yai[c] / yf : T_AUTO;
        int ign = o->pilot[c] || Tc > ait;
        if (!ign) {
            int i = c % nx, j = (c / nx) % ny, k = c / sz;
            ign = (i > 0 && o->lit[c - sx]) || (i < nx - 1 && o->lit[c + sx]) || (j > 0 && o->lit[c - sy]) ||
                  (j < ny - 1 && o->lit[c + sy]) || (k > 0 && o->lit[c - sz]) || (k < nz - 1 && o->lit[c + sz]);
        }
        if (!ign) continue;
        double burnable = mn(yf, o->Yo[c] / s);
        if (burnable <= 1e-7) continue;
        double tAd = Tc + DHC_FUEL / (CP * (1.0 + S_O2 / mx(o->Yo[c], 1e-4)));
        if (!o->pilot[c] && tAd < T_CRIT) continue;
        double m = gasDensity(o, c) * V;
        double dmf = burnable * m * frac;
        double q = dmf * DHC_FUEL;
        double sootMade = yf > 0 ? o->Yp[c] * (dmf / m) / yf : 0;
        double coMade = CO_YIELD * dmf / m;
        double co2Made = mx(0.0, (C_FRAC * dmf / m - sootMade - (12.0 / 28.0) * coMade) * (44.0 / 12.0));
        double o2Used = s * dmf / m - (32.0 / 12.0) * sootMade - (16.0 / 28.0) * coMade;
        o->Yf[c] = mx(0.0, yf - dmf / m);
        o->Yai[c] = o->Yf[c] * ait;
        o->Yo[c] = mx(0.0, o->Yo[c] - o2Used);
        o->Yp[c] = mx(0.0, o->Yp[c] - sootMade);
        o->Ys[c] += sootMade;
        o->Yco[c] += coMade;
        o->Yc[c] += co2Made;
        o->Yw[c] += Y_H2O * dmf / m;
        o->Ya[c] *= (1.0 - frac);
        o->Q[c] += q * (1.0 - chiR);
        o->Qr[c] = q * chiR;
        o->hrr[c] = q / (dt * V);
        litNew[c] = q > 1e-3 ? 1.0 : 0.0;
    }
    (void)ny; (void)nz;
    for (int c = 0; c < o->N; ++c) o->lit[c] = litNew[c] > 0.5;
}

/* Solver::computeZones, src/sim/gasphase.cpp:111-158 */
static void computeZones(Orc* o) {
    o->zonesDirty = 0;
    o->mgDirty = 1;
    const int N = o->N, nx = o->nx, ny = o->ny, nz = o->nz, sxy = nx * ny;
    double* oldPb = (double*)malloc(N * sizeof(double));
    memcpy(oldPb, o->Pb, N * sizeof(double));
    for (int c = 0; c < N; ++c) o->zone[c] = -1;
    int cap = 16, nZ = 0;
    double* zoneP = (double*)malloc(cap * sizeof(double));
    uint8_t* zoneOpen = (uint8_t*)malloc(cap);
    double* pSum = (double*)malloc(cap * sizeof(double));
    double* vSum = (double*)malloc(cap * sizeof(double));
    int* stack = (int*)malloc((N + 1) * sizeof(int));
    for (int seed = 0; seed < N; ++seed) {
        if (o->blocked[seed] || o->zone[seed] >= 0) continue;
        if (nZ == cap) {
            cap *= 2;
            zoneP = (double*)realloc(zoneP, cap * sizeof(double));
            zoneOpen = (uint8_t*)realloc(zoneOpen, cap);
            pSum = (double*)realloc(pSum, cap * sizeof(double));
            vSum = (double*)realloc(vSum, cap * sizeof(double));
        }
        int z = nZ++;
        zoneP[z] = P0; zoneOpen[z] = 0; pSum[z] = 0; vSum[z] = 0;
        int sp = 0;
        stack[sp++] = seed;
        o->zone[seed] = z;
        while (sp > 0) {
            int c = stack[--sp];
            pSum[z] += oldPb[c];
            vSum[z] += 1;
            int i = c % nx, j = (c / nx) % ny, k = c / sxy;
            double a[6] = {o->ax[xfaceI(o, i, j, k)], o->ax[xfaceI(o, i + 1, j, k)], o->ay[yfaceI(o, i, j, k)],
                           o->ay[yfaceI(o, i, j + 1, k)], o->az[zfaceI(o, i, j, k)], o->az[zfaceI(o, i, j, k + 1)]};
            int nb[6] = {i > 0 ? c - 1 : -1, i < nx - 1 ? c + 1 : -1, j > 0 ? c - nx : -1, j < ny - 1 ? c + nx : -1,
                         k > 0 ? c - sxy : -1, k < nz - 1 ? c + sxy : -1};
            for (int d = 0; d < 6; ++d) {
                if (a[d] <= 0) continue;
                if (nb[d] < 0) { if (d != 4) zoneOpen[z] = 1; continue; }
                if (o->blocked[nb[d]] || o->zone[nb[d]] >= 0) continue;
                o->zone[nb[d]] = z;
                stack[sp++] = nb[d];
            }
        }
    }
    for (int z = 0; z < nZ; ++z) zoneP[z] = zoneOpen[z] ? P0 : (double)(pSum[z] / mx(1.0, vSum[z]));
    for (int c = 0; c < N; ++c) o->Pb[c] = o->zone[c] >= 0 ? zoneP[o->zone[c]] : P0;
    free(o->zoneP); free(o->zoneOpen); free(o->zoneVol); free(o->zoneDP);
    o->zoneP = zoneP; o->zoneOpen = zoneOpen; o->nZones = nZ;
    o->zoneVol = (double*)malloc((nZ ? nZ : 1) * sizeof(double));
    for (int z = 0; z < nZ; ++z) o->zoneVol[z] = vSum[z] * o->dx * o->dx * o->dx;
    o->zoneDP = NULL;   /* sized by leakage(), as zoneDP_ in the reference */
    free(pSum); free(vSum); free(stack); free(oldPb);
}

/* Solver::turbulence, src/sim/gasphase.cpp:163-218 */
static void turbulence(Orc* o) {
    const int nx = o->nx, ny = o->ny, nz = o->nz;
    double *uc = o->tmp[0], *vc = o->tmp[1], *wc = o->tmp[2];
    double* f[3] = {o->tmp[3], o->tmp[4], o->tmp[5]};
    double* g[3] = {o->tmp[6], o->tmp[7], o->tmp[8]};
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                int c = cellI(o, i, j, k);
                if (o->blocked[c]) { uc[c] = vc[c] = wc[c] = 0; continue; }
                uc[c] = 0.5 * (o->u[xfaceI(o, i, j, k)] + o->u[xfaceI(o, i + 1, j, k)]);
                vc[c] = 0.5 * (o->v[yfaceI(o, i, j, k)] + o->v[yfaceI(o, i, j + 1, k)]);
                wc[c] = 0.5 * (o->w[zfaceI(o, i, j, k)] + o->w[zfaceI(o, i, j, k + 1)]);
            }
    double* src[3] = {uc, vc, wc};
    const int str[3] = {1, nx, nx * ny};
    for (int q = 0; q < 3; ++q)
        for (int axis = 0; axis < 3; ++axis) {
            const double* in = axis == 0 ? src[q] : axis == 1 ? f[q] : g[q];
            double* out = axis == 1 ? g[q] : f[q];
            for (int k = 0; k < nz; ++k)
                for (int j = 0; j < ny; ++j)
                    for (int i = 0; i < nx; ++i) {
                        int c = cellI(o, i, j, k);
                        if (o->blocked[c]) { out[c] = 0; continue; }
                        int id = axis == 0 ? i : axis == 1 ? j : k, n = axis == 0 ? nx : axis == 1 ? ny : nz;
                        double lo = id > 0 && !o->blocked[c - str[axis]] ? in[c - str[axis]] : in[c];
                        double hi = id < n - 1 && !o->blocked[c + str[axis]] ? in[c + str[axis]] : in[c];
                        out[c] = 0.25 * lo + 0.5 * in[c] + 0.25 * hi;
                    }
        }
    double maxNu = 0;
    for (int k = 0; k < nz; ++k) {
        double m = 0;
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                int c = cellI(o, i, j, k);
                if (o->blocked[c]) { o->nu[c] = 0; continue; }
                double du = uc[c] - f[0][c], dv = vc[c] - f[1][c], dw = wc[c] - f[2][c];
                double ks = 0.5 * (du * du + dv * dv + dw * dw);
                o->nu[c] = mn(1.0, C_NU * o->dx * sqrt(ks) + 1.5e-5 * pow(o->T[c] / 293.15, 1.7));
                m = mx(m, o->nu[c]);
            }
        maxNu = k == 0 ? m : mx(maxNu, m);
    }
    o->maxNu = maxNu;
}

static inline double kMol(double T) { return 0.0258 * pow(T / 293.15, 0.8); }

/* Solver::heatDiffusion, src/sim/gasphase.cpp:221-248 */
static void heatDiffusion(Orc* o, double dt) {
    const int nx = o->nx, ny = o->ny, nz = o->nz, sxy = nx * ny;
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                int c = cellI(o, i, j, k);
                if (o->blocked[c]) continue;
                double fo[6] = {o->fx[xfaceI(o, i, j, k)], o->fx[xfaceI(o, i + 1, j, k)], o->fy[yfaceI(o, i, j, k)],
                                o->fy[yfaceI(o, i, j + 1, k)], o->fz[zfaceI(o, i, j, k)], o->fz[zfaceI(o, i, j, k + 1)]};
                int nb[6] = {i > 0 ? c - 1 : -1, i < nx - 1 ? c + 1 : -1, j > 0 ? c - nx : -1, j < ny - 1 ? c + nx : -1,
                             k > 0 ? c - sxy : -1, k < nz - 1 ? c + sxy : -1};
                double rc = gasDensity(o, c), q = 0;
                for (int d = 0; d < 6; ++d) {
                    if (fo[d] <= 0) continue;
                    int n = nb[d];
                    if (n >= 0 && o->blocked[n]) continue;
                    double Tn = n >= 0 ? o->T[n] : T0;
                    double nun = n >= 0 ? o->nu[n] : o->nu[c];
                    double rn = n >= 0 ? gasDensity(o, n) : P0 / (RS * T0);
                    double Tf = 0.5 * (o->T[c] + Tn);
                    double kf = 0.5 * (rc + rn) * CP * 0.5 * (o->nu[c] + nun) / PR_T + kMol(Tf);
                    q += fo[d] * kf * o->dx * (Tn - o->T[c]);
                }
                o->Q[c] += q * dt;
            }
}

/* Solver::energyAndExpansion, src/sim/gasphase.cpp:251-271 */
static void energyAndExpansion(Orc* o, double dt) {
    const double V = o->dx * o->dx * o->dx;
    double md = 0;
    for (int c = 0; c < o->N; ++c) {
        if (o->blocked[c]) { o->S[c] = 0; continue; }
        double rho = gasDensity(o, c);
        double m = rho * V;
        double Tn = clampd(o->T[c] + o->Q[c] / (m * CP), T_MIN, T_MAX);
        double rhoN = o->Pb[c] / (RS * Tn);
        double D = o->Q[c] / (m * CP * o->T[c] * dt) + o->massSrc[c] / (rhoN * V * dt);
        o->T[c] = Tn;
        o->S[c] = clampd(D, -D_MAX, D_MAX);
        md = mx(md, fabs(o->S[c]));
    }
    o->maxDiv = md;
}

static inline double vanLeer(double a, double b) { return a * b > 0 ? 2 * a * b / (a + b) : 0.0; }

/* Solver::momentum, src/sim/gasphase.cpp:275-399 */
static void momentum(Orc* o, double dt) {
    const int nx = o->nx, ny = o->ny, nz = o->nz;
    const double idx = 1.0 / o->dx, idx2 = 1.0 / (o->dx * o->dx);
    const int ncell[3] = {nx, ny, nz};
    for (int comp = 0; comp < 3; ++comp) {
        const double* vel = comp == 0 ? o->u : comp == 1 ? o->v : o->w;
        const double* fo = comp == 0 ? o->fx : comp == 1 ? o->fy : o->fz;
        const uint8_t* lk = comp == 0 ? o->lx : comp == 1 ? o->ly : o->lz;
        double* out = comp == 0 ? o->u2 : comp == 1 ? o->v2 : o->w2;
        const int dX = nx + (comp == 0), dY = ny + (comp == 1), dZ = nz + (comp == 2);
        const int st[3] = {1, dX, dX * dY};
        const int dim[3] = {dX, dY, dZ};
        for (int k = 0; k < dZ; ++k)
            for (int j = 0; j < dY; ++j)
                for (int i = 0; i < dX; ++i) {
                    int f = i + dX * (j + dY * k);
                    if (fo[f] <= 0) { out[f] = 0; continue; }
                    if (lk[f]) { out[f] = vel[f]; continue; }
                    int id[3] = {i, j, k};
                    int lo = id[comp] - 1;
                    int bnd = lo < 0 || id[comp] >= ncell[comp];
                    int ca = -1, cb = -1;
                    {
                        int a[3] = {i, j, k};
                        a[comp] -= 1;
                        if (a[comp] >= 0) ca = cellI(o, a[0], a[1], a[2]);
                        if (id[comp] < ncell[comp]) cb = cellI(o, i, j, k);
                    }
                    double zc = o->oz + (comp == 2 ? (double)k : k + 0.5) * o->dx;
                    if (bnd) {
                        double wv = windAt(o, comp, lo < 0 ? 0 : 1, zc);
                        if (!isnan(wv)) { out[f] = wv; continue; }
                        out[f] = vel[f];
                        continue;
                    }
                    double v0 = vel[f];
                    double adv[3];
                    adv[comp] = v0;
                    for (int a = 0; a < 3; ++a) {
                        if (a == comp) continue;
                        const double* va = a == 0 ? o->u : a == 1 ? o->v : o->w;
                        int aX = nx + (a == 0), aY = ny + (a == 1);
                        double s = 0;
                        for (int q = 0; q < 4; ++q) {
                            int p[3] = {i, j, k};
                            if (q & 1) p[a] += 1;
                            if (q & 2) p[comp] -= 1;
                            p[a] = p[a] < ncell[a] ? p[a] : ncell[a];
                            p[comp] = p[comp] > 0 ? p[comp] : 0;
                            s += va[p[0] + aX * (p[1] + aY * p[2])];
                        }
                        adv[a] = 0.25 * s;
                    }
                    double acc = 0, lap = 0;
                    for (int a = 0; a < 3; ++a) {
                        double m1, p1, m2, p2;
                        /* nbv: neighbour along a, free slip across closed faces */
                        {
                            int ni = id[a] - 1;
                            int g = f - st[a];
                            m1 = (ni < 0 || ni >= dim[a]) ? v0 : (fo[g] > 0 && !lk[g] ? vel[g] : v0);
                            ni = id[a] + 1;
                            g = f + st[a];
                            p1 = (ni < 0 || ni >= dim[a]) ? v0 : (fo[g] > 0 && !lk[g] ? vel[g] : v0);
                        }
                        /* nb2: second neighbour, only through two open faces */
                        {
                            int ni = id[a] - 2;
                            if (ni < 0 || ni >= dim[a]) m2 = m1;
                            else {
                                int g = f - 2 * st[a], g1 = f - st[a];
                                m2 = fo[g] > 0 && fo[g1] > 0 && !lk[g] && !lk[g1] ? vel[g] : m1;
                            }
                            ni = id[a] + 2;
                            if (ni < 0 || ni >= dim[a]) p2 = p1;
                            else {
                                int g = f + 2 * st[a], g1 = f + st[a];
                                p2 = fo[g] > 0 && fo[g1] > 0 && !lk[g] && !lk[g1] ? vel[g] : p1;
                            }
                        }
                        double fp, fm;
                        if (adv[a] >= 0) {
                            fp = v0 + 0.5 * vanLeer(v0 - m1, p1 - v0);
                            fm = m1 + 0.5 * vanLeer(m1 - m2, v0 - m1);
                        } else {
                            fp = p1 - 0.5 * vanLeer(p1 - v0, p2 - p1);
                            fm = v0 - 0.5 * vanLeer(v0 - m1, p1 - v0);
                        }
                        acc -= adv[a] * (fp - fm) * idx;
                        lap += (m1 - 2 * v0 + p1) * idx2;
                    }
                    double ra = gasDensity(o, ca), rb = gasDensity(o, cb);
                    double rf = 0.5 * (ra + rb);
                    double nuf = 0.5 * (o->nu[ca] + o->nu[cb]);
                    acc += nuf * lap;
                    if (comp == 2) {
                        double r0 = 0.5 * (o->Pb[ca] + o->Pb[cb]) / (RS * T0);
                        acc += GRAV * (r0 - rf) / rf;
                    }
                    double pt = rf * 0.5 * (o->p[ca] + o->p[cb]);
                    acc += pt * (1.0 / rb - 1.0 / ra) * idx;
                    out[f] = clampd(v0 + dt * acc, -VMAX, VMAX);
                }
        /* open boundary faces without wind inflow: zero gradient from the new
         * value one cell inside, src/sim/gasphase.cpp:376-393 */
        int nAx = ncell[comp];
        int nA = dim[(comp + 1) % 3], nB = dim[(comp + 2) % 3];
        for (int b2 = 0; b2 < nB; ++b2)
            for (int a2 = 0; a2 < nA; ++a2)
                for (int side = (comp == 2 ? 1 : 0); side < 2; ++side) {
                    int id[3];
                    id[comp] = side == 0 ? 0 : nAx;
                    id[(comp + 1) % 3] = a2;
                    id[(comp + 2) % 3] = b2;
                    int f = id[0] + dX * (id[1] + dY * id[2]);
                    if (fo[f] <= 0 || lk[f]) continue;
                    double zc = o->oz + (comp == 2 ? (double)id[2] : id[2] + 0.5) * o->dx;
                    if (!isnan(windAt(o, comp, side, zc))) continue;
                    int g = f + (side == 0 ? 1 : -1) * st[comp];
                    out[f] = fo[g] > 0 && !lk[g] ? out[g] : 0.0;
                }
    }
    double* t;
    t = o->u; o->u = o->u2; o->u2 = t;
    t = o->v; o->v = o->v2; o->v2 = t;
    t = o->w; o->w = o->w2; o->w2 = t;
}

/* Solver::leakage, src/sim/gasphase.cpp:403-499 */
static double zPof(const Orc* o, int c, const double* P) { return c >= 0 && o->zone[c] >= 0 ? P[o->zone[c]] : P0; }
static double flowOf(double dp, double rhoUp) {
    double s = dp >= 0 ? 1.0 : -1.0;
    return s * mn(LEAK_VMAX, CD_LEAK * sqrt(2.0 * fabs(dp) / mx(rhoUp, 0.05)));
}
static double openFracOf(const Orc* o, const LeakFace* lf) {
    return (lf->axis == 0 ? o->fx : lf->axis == 1 ? o->fy : o->fz)[lf->f];
}

static void leakage(Orc* o, double dt) {
    const int nZ = o->nZones, nx = o->nx, ny = o->ny, nz = o->nz;
    const double V = o->dx * o->dx * o->dx;
    double* dInt = (double*)calloc(nZ ? nZ : 1, sizeof(double));
    for (int c = 0; c < o->N; ++c)
        if (o->zone[c] >= 0) dInt[o->zone[c]] += o->S[c] * V;
    int nf = 0, capf = 64;
    LeakFace* faces = (LeakFace*)malloc(capf * sizeof(LeakFace));
    for (int axis = 0; axis < 3; ++axis) {
        const uint8_t* lk = axis == 0 ? o->lx : axis == 1 ? o->ly : o->lz;
        const int dX = nx + (axis == 0), dY = ny + (axis == 1);
        const int len = axis == 0 ? o->NX : axis == 1 ? o->NY : o->NZ;
        const int ncell = axis == 0 ? nx : axis == 1 ? ny : nz;
        for (int f = 0; f < len; ++f) {
            if (!lk[f]) continue;
            int i = f % dX, j = (f / dX) % dY, k = f / (dX * dY);
            int id[3] = {i, j, k}, a[3] = {i, j, k};
            a[axis] -= 1;
            int ca = a[axis] >= 0 ? cellI(o, a[0], a[1], a[2]) : -1;
            int cb = id[axis] < ncell ? cellI(o, i, j, k) : -1;
            if ((ca >= 0 && o->blocked[ca]) || (cb >= 0 && o->blocked[cb])) continue;
            if (nf == capf) { capf *= 2; faces = (LeakFace*)realloc(faces, capf * sizeof(LeakFace)); }
            LeakFace lf = {axis, f, ca, cb};
            faces[nf++] = lf;
        }
    }
    o->leakFaces = nf;
    const double A = o->dx * o->dx;
    double* Pnew = (double*)malloc((nZ ? nZ : 1) * sizeof(double));
    memcpy(Pnew, o->zoneP, nZ * sizeof(double));
    /* per-zone face lists in face order */
    int* zcount = (int*)calloc(nZ + 1, sizeof(int));
    for (int q = 0; q < nf; ++q) {
        int za = faces[q].a >= 0 ? o->zone[faces[q].a] : -1, zb = faces[q].b >= 0 ? o->zone[faces[q].b] : -1;
        if (za == zb) continue;
        if (za >= 0) zcount[za + 1]++;
        if (zb >= 0) zcount[zb + 1]++;
    }
    for (int z = 0; z < nZ; ++z) zcount[z + 1] += zcount[z];
    int* zlist = (int*)malloc((zcount[nZ] + 1) * sizeof(int));
    int* zfill = (int*)calloc(nZ + 1, sizeof(int));
    for (int q = 0; q < nf; ++q) {
        int za = faces[q].a >= 0 ? o->zone[faces[q].a] : -1, zb = faces[q].b >= 0 ? o->zone[faces[q].b] : -1;
        if (za == zb) continue;
        if (za >= 0) zlist[zcount[za] + zfill[za]++] = q;
        if (zb >= 0) zlist[zcount[zb] + zfill[zb]++] = q;
    }
    for (int z = 0; z < nZ; ++z) {
        if (o->zoneOpen[z]) continue;
        double P = o->zoneP[z];
        double Vz = o->zoneVol[z];
        double lo = P - 20000.0, hi = P + 20000.0;
        double rlo, rhi;
        for (int side = 0; side < 2; ++side) {
            double Pt = side == 0 ? lo : hi, out = 0;
            for (int e = zcount[z]; e < zcount[z + 1]; ++e) {
                const LeakFace* lf = &faces[zlist[e]];
                int zIsA = lf->a >= 0 && o->zone[lf->a] == z;
                int other = zIsA ? lf->b : lf->a;
                double Po = zPof(o, other, o->zoneP);
                double dp = Pt - Po;
                int up = dp >= 0 ? (zIsA ? lf->a : lf->b) : other;
                double rho = up >= 0 ? gasDensity(o, up) : P0 / (RS * T0);
                out += openFracOf(o, lf) * A * fabs(flowOf(dp, rho)) * (dp >= 0 ? 1 : -1);
            }
            double r = Pt - P - dt * GAMMA * P / Vz * (double)(dInt[z] - out);
            if (side == 0) rlo = r; else rhi = r;
        }
        if (rlo > 0 || rhi < 0) { Pnew[z] = P; continue; }
        for (int it = 0; it < 40; ++it) {
            double mid = 0.5 * (lo + hi), out = 0;
            for (int e = zcount[z]; e < zcount[z + 1]; ++e) {
                const LeakFace* lf = &faces[zlist[e]];
                int zIsA = lf->a >= 0 && o->zone[lf->a] == z;
                int other = zIsA ? lf->b : lf->a;
                double Po = zPof(o, other, o->zoneP);
                double dp = mid - Po;
                int up = dp >= 0 ? (zIsA ? lf->a : lf->b) : other;
                double rho = up >= 0 ? gasDensity(o, up) : P0 / (RS * T0);
                out += openFracOf(o, lf) * A * fabs(flowOf(dp, rho)) * (dp >= 0 ? 1 : -1);
            }
            double r = mid - P - dt * GAMMA * P / Vz * (double)(dInt[z] - out);
            if (r > 0) hi = mid; else lo = mid;
        }
        Pnew[z] = 0.5 * (lo + hi);
    }
    double* outz = (double*)calloc(nZ ? nZ : 1, sizeof(double));
    for (int q = 0; q < nf; ++q) {
        const LeakFace* lf = &faces[q];
        double pa = zPof(o, lf->a, Pnew), pb = zPof(o, lf->b, Pnew);
        double ra = lf->a >= 0 ? gasDensity(o, lf->a) : P0 / (RS * T0);
        double rb = lf->b >= 0 ? gasDensity(o, lf->b) : P0 / (RS * T0);
        double Ha = lf->a >= 0 ? o->p[lf->a] : 0, Hb = lf->b >= 0 ? o->p[lf->b] : 0;
        double dp = (pa - pb) + 0.5 * (ra + rb) * (Ha - Hb);
        double un = flowOf(dp, dp >= 0 ? ra : rb);
        double* vel = lf->axis == 0 ? o->u : lf->axis == 1 ? o->v : o->w;
        vel[lf->f] = 0.5 * (vel[lf->f] + un);
        double qf = openFracOf(o, lf) * A * vel[lf->f];
        if (lf->a >= 0 && o->zone[lf->a] >= 0) outz[o->zone[lf->a]] += qf;
        if (lf->b >= 0 && o->zone[lf->b] >= 0) outz[o->zone[lf->b]] -= qf;
    }
    free(o->zoneDP);
    o->zoneDP = (double*)calloc(nZ ? nZ : 1, sizeof(double));
    double* shift = (double*)calloc(nZ ? nZ : 1, sizeof(double));
    for (int z = 0; z < nZ; ++z) {
        if (o->zoneOpen[z]) continue;
        double Vz = o->zoneVol[z];
        o->zoneDP[z] = GAMMA * o->zoneP[z] * (double)(dInt[z] - outz[z]) / Vz;
        shift[z] = (double)(dInt[z] - outz[z]) / Vz;
    }
    for (int c = 0; c < o->N; ++c)
        if (o->zone[c] >= 0 && !o->zoneOpen[o->zone[c]]) o->S[c] -= shift[o->zone[c]];
    free(dInt); free(faces); free(Pnew); free(zcount); free(zlist); free(zfill); free(outz); free(shift);
}

/* ---------------------------------------------------------------------------
 * Multigrid preconditioner: Solver::buildPressureLevels and
 * Solver::pressurePrecondition, src/sim/pressure_mg.cpp:28-300 */
static int uf_find(int* p, int a) {
    while (p[a] != a) a = p[a] = p[p[a]];
    return a;
}
static void uf_join(int* p, int a, int b) {
    a = uf_find(p, a);
    b = uf_find(p, b);
    if (a != b) { if (a > b) p[a] = b; else p[b] = a; }
}

/* growable rows of (col, val) pairs kept in insertion order */
typedef struct { int n, cap; int* col; double* val; } Row;
static void row_add(Row* r, int col, double w) {
    for (int e = 0; e < r->n; ++e)
        if (r->col[e] == col) { r->val[e] += w; return; }
    if (r->n == r->cap) {
        r->cap = r->cap ? 2 * r->cap : 8;
        r->col = (int*)realloc(r->col, r->cap * sizeof(int));
        r->val = (double*)realloc(r->val, r->cap * sizeof(double));
    }
    r->col[r->n] = col;
    r->val[r->n] = w;
    r->n++;
}

static void rows_to_csr(Level* C, Row* rows, const double* dg) {
    C->diag = (double*)malloc((C->n ? C->n : 1) * sizeof(double));
    C->rowStart = (int*)malloc((C->n + 1) * sizeof(int));
    C->rowStart[0] = 0;
    for (int I = 0; I < C->n; ++I) {
        C->diag[I] = (double)mx(dg[I], 0.0);
        C->rowStart[I + 1] = C->rowStart[I] + rows[I].n;
    }
    C->nnz = C->rowStart[C->n];
    C->col = (int*)malloc((C->nnz ? C->nnz : 1) * sizeof(int));
    C->val = (double*)malloc((C->nnz ? C->nnz : 1) * sizeof(double));
    for (int I = 0; I < C->n; ++I) {
        memcpy(C->col + C->rowStart[I], rows[I].col, rows[I].n * sizeof(int));
        memcpy(C->val + C->rowStart[I], rows[I].val, rows[I].n * sizeof(double));
        free(rows[I].col);
        free(rows[I].val);
    }
}

static void buildPressureLevels(Orc* o) {
    o->mgDirty = 0;
    free_levels(o);
    const int nx = o->nx, ny = o->ny, nz = o->nz, n0 = o->N, sxy = nx * ny;
    /* level 0: structured grid, boundary faces with wind inflow closed (:33-57) */
    Level* L0 = &o->lv[0];
    L0->nx = nx; L0->ny = ny; L0->nz = nz; L0->n = n0;
    L0->ax = (double*)malloc(o->NX * sizeof(double)); memcpy(L0->ax, o->ax, o->NX * sizeof(double));
    L0->ay = (double*)malloc(o->NY * sizeof(double)); memcpy(L0->ay, o->ay, o->NY * sizeof(double));
    L0->az = (double*)malloc(o->NZ * sizeof(double)); memcpy(L0->az, o->az, o->NZ * sizeof(double));
    for (int k = 0; k < nz; ++k) {
        double z = o->oz + (k + 0.5) * o->dx;
        for (int j = 0; j < ny; ++j) {
            if (!bndOpen(o, 0, 0, z)) L0->ax[xfaceI(o, 0, j, k)] = 0;
            if (!bndOpen(o, 0, 1, z)) L0->ax[xfaceI(o, nx, j, k)] = 0;
        }
        for (int i = 0; i < nx; ++i) {
            if (!bndOpen(o, 1, 0, z)) L0->ay[yfaceI(o, i, 0, k)] = 0;
            if (!bndOpen(o, 1, 1, z)) L0->ay[yfaceI(o, i, ny, k)] = 0;
        }
    }
    L0->diag = dalloc(n0, 0);
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                int c = cellI(o, i, j, k);
                if (o->blocked[c]) continue;
                L0->diag[c] = L0->ax[xfaceI(o, i, j, k)] + L0->ax[xfaceI(o, i + 1, j, k)] + L0->ay[yfaceI(o, i, j, k)] +
                              L0->ay[yfaceI(o, i, j + 1, k)] + L0->az[zfaceI(o, i, j, k)] + L0->az[zfaceI(o, i, j, k + 1)];
            }
    o->nLevels = 1;
    /* level 1: connected pieces of 2x2x2 blocks (:59-139) */
    {
        int* uf = (int*)malloc(n0 * sizeof(int));
        for (int c = 0; c < n0; ++c) uf[c] = c;
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i) {
                    int c = cellI(o, i, j, k);
                    if (L0->diag[c] <= 0) continue;
                    if (i + 1 < nx && (i >> 1) == ((i + 1) >> 1) && L0->ax[xfaceI(o, i + 1, j, k)] > 0 && L0->diag[c + 1] > 0) uf_join(uf, c, c + 1);
                    if (j + 1 < ny && (j >> 1) == ((j + 1) >> 1) && L0->ay[yfaceI(o, i, j + 1, k)] > 0 && L0->diag[c + nx] > 0) uf_join(uf, c, c + nx);
                    if (k + 1 < nz && (k >> 1) == ((k + 1) >> 1) && L0->az[zfaceI(o, i, j, k + 1)] > 0 && L0->diag[c + sxy] > 0) uf_join(uf, c, c + sxy);
                }
        L0->agg = (int*)malloc(n0 * sizeof(int));
        int* rootId = (int*)malloc(n0 * sizeof(int));
        for (int c = 0; c < n0; ++c) { L0->agg[c] = -1; rootId[c] = -1; }
        Level* C = &o->lv[1];
        C->n = 0;
        int capb = 1024;
        C->bi = (int*)malloc(capb * sizeof(int)); C->bj = (int*)malloc(capb * sizeof(int)); C->bk = (int*)malloc(capb * sizeof(int));
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i) {
                    int c = cellI(o, i, j, k);
                    if (L0->diag[c] <= 0) continue;
                    int r = uf_find(uf, c);
                    if (rootId[r] < 0) {
                        if (C->n == capb) {
                            capb *= 2;
                            C->bi = (int*)realloc(C->bi, capb * sizeof(int)); C->bj = (int*)realloc(C->bj, capb * sizeof(int));
                            C->bk = (int*)realloc(C->bk, capb * sizeof(int));
                        }
                        rootId[r] = C->n;
                        C->bi[C->n] = i >> 1; C->bj[C->n] = j >> 1; C->bk[C->n] = k >> 1;
                        C->n++;
                    }
                    L0->agg[c] = rootId[r];
                }
        Row* rows = (Row*)calloc(C->n ? C->n : 1, sizeof(Row));
        double* dg = (double*)calloc(C->n ? C->n : 1, sizeof(double));
#define COUPLE(a_, b_, w_)                                               \
    do {                                                                 \
        double w__ = (w_);                                               \
        if (w__ > 0) {                                                   \
            int A__ = L0->agg[a_], B__ = L0->agg[b_];                    \
            if (A__ >= 0 && B__ >= 0 && A__ != B__) {                    \
                row_add(&rows[A__], B__, w__);                           \
                row_add(&rows[B__], A__, w__);                           \
            }                                                            \
        }                                                                \
    } while (0)
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i) {
                    int c = cellI(o, i, j, k);
                    if (L0->diag[c] <= 0) continue;
                    if (i + 1 < nx) COUPLE(c, c + 1, L0->ax[xfaceI(o, i + 1, j, k)]);
                    if (j + 1 < ny) COUPLE(c, c + nx, L0->ay[yfaceI(o, i, j + 1, k)]);
                    if (k + 1 < nz) COUPLE(c, c + sxy, L0->az[zfaceI(o, i, j, k + 1)]);
                }
#undef COUPLE
        for (int c = 0; c < n0; ++c) if (L0->agg[c] >= 0) dg[L0->agg[c]] += L0->diag[c];
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i) {
                    int c = cellI(o, i, j, k);
                    if (L0->diag[c] <= 0) continue;
                    double w;
                    if (i + 1 < nx && L0->diag[c + 1] > 0) {
                        w = L0->ax[xfaceI(o, i + 1, j, k)];
                        if (w > 0 && L0->agg[c + 1] == L0->agg[c]) dg[L0->agg[c]] -= 2.0 * w;
                    }
                    if (j + 1 < ny && L0->diag[c + nx] > 0) {
                        w = L0->ay[yfaceI(o, i, j + 1, k)];
                        if (w > 0 && L0->agg[c + nx] == L0->agg[c]) dg[L0->agg[c]] -= 2.0 * w;
                    }
                    if (k + 1 < nz && L0->diag[c + sxy] > 0) {
                        w = L0->az[zfaceI(o, i, j, k + 1)];
                        if (w > 0 && L0->agg[c + sxy] == L0->agg[c]) dg[L0->agg[c]] -= 2.0 * w;
                    }
                }
        rows_to_csr(C, rows, dg);
        free(rows); free(dg); free(uf); free(rootId);
        o->nLevels = 2;
    }
    /* coarser levels: connected pieces of 2x2x2 groups of block coordinates (:141-184) */
    while (o->lv[o->nLevels - 1].n > 2000 && o->nLevels < 12) {
        Level* F = &o->lv[o->nLevels - 1];
        int* uf = (int*)malloc((F->n ? F->n : 1) * sizeof(int));
        for (int I = 0; I < F->n; ++I) uf[I] = I;
        for (int I = 0; I < F->n; ++I)
            for (int e = F->rowStart[I]; e < F->rowStart[I + 1]; ++e) {
                int J = F->col[e];
                if (J > I && (F->bi[I] >> 1) == (F->bi[J] >> 1) && (F->bj[I] >> 1) == (F->bj[J] >> 1) &&
                    (F->bk[I] >> 1) == (F->bk[J] >> 1))
                    uf_join(uf, I, J);
            }
        F->agg = (int*)malloc(F->n * sizeof(int));
        int* rootId = (int*)malloc(F->n * sizeof(int));
        for (int I = 0; I < F->n; ++I) rootId[I] = -1;
        Level* C = &o->lv[o->nLevels];
        memset(C, 0, sizeof(Level));
        C->bi = (int*)malloc(F->n * sizeof(int)); C->bj = (int*)malloc(F->n * sizeof(int)); C->bk = (int*)malloc(F->n * sizeof(int));
        for (int I = 0; I < F->n; ++I) {
            int r = uf_find(uf, I);
            if (rootId[r] < 0) {
                rootId[r] = C->n;
                C->bi[C->n] = F->bi[I] >> 1; C->bj[C->n] = F->bj[I] >> 1; C->bk[C->n] = F->bk[I] >> 1;
                C->n++;
            }
            F->agg[I] = rootId[r];
        }
        free(uf); free(rootId);
        if (C->n > 0.8 * F->n) {   /* not coarsening any more */
            free(F->agg); F->agg = NULL;
            free(C->bi); free(C->bj); free(C->bk);
            memset(C, 0, sizeof(Level));
            break;
        }
        Row* rows = (Row*)calloc(C->n ? C->n : 1, sizeof(Row));
        double* dg = (double*)calloc(C->n ? C->n : 1, sizeof(double));
        for (int I = 0; I < F->n; ++I) dg[F->agg[I]] += F->diag[I];
        for (int I = 0; I < F->n; ++I)
            for (int e = F->rowStart[I]; e < F->rowStart[I + 1]; ++e) {
                int J = F->col[e];
                int A = F->agg[I], B = F->agg[J];
                if (A == B) { dg[A] -= F->val[e]; continue; }
                /* first-found accumulate, else append */
                Row* r = &rows[A];
                int found = 0;
                for (int x = 0; x < r->n; ++x)
                    if (r->col[x] == B) { r->val[x] += F->val[e]; found = 1; break; }
                if (!found) row_add(r, B, F->val[e]);
            }
        rows_to_csr(C, rows, dg);
        free(rows); free(dg);
        o->nLevels++;
    }
    for (int l = 0; l < o->nLevels; ++l) {
        Level* L = &o->lv[l];
        L->x = dalloc(L->n, 0); L->b = dalloc(L->n, 0); L->r = dalloc(L->n, 0); L->t = dalloc(L->n, 0);
    }
}

/* gsColor, src/sim/pressure_mg.cpp:195-216 */
static void gsColor(Level* L, int color) {
    const int sx = L->nx, sxy = L->nx * L->ny;
    for (int r = 0; r < L->ny * L->nz; ++r) {
        int j = r % L->ny, k = r / L->ny;
        int i0 = (j + k + color) & 1;
        for (int i = i0; i < L->nx; i += 2) {
            int c = i + sx * (j + L->ny * k);
            double dg = L->diag[c];
            if (dg <= 0) { L->x[c] = 0; continue; }
            double s = L->b[c];
            if (i > 0) s += L->ax[i + (L->nx + 1) * (j + L->ny * k)] * L->x[c - 1];
            if (i < L->nx - 1) s += L->ax[i + 1 + (L->nx + 1) * (j + L->ny * k)] * L->x[c + 1];
            if (j > 0) s += L->ay[i + L->nx * (j + (L->ny + 1) * k)] * L->x[c - sx];
            if (j < L->ny - 1) s += L->ay[i + L->nx * (j + 1 + (L->ny + 1) * k)] * L->x[c + sx];
            if (k > 0) s += L->az[i + L->nx * (j + L->ny * k)] * L->x[c - sxy];
            if (k < L->nz - 1) s += L->az[i + L->nx * (j + L->ny * (k + 1))] * L->x[c + sxy];
            L->x[c] = s / dg;
        }
    }
}

/* residualGrid, src/sim/pressure_mg.cpp:217-235 */
static void residualGrid(Level* L) {
    const int sx = L->nx, sxy = L->nx * L->ny;
    for (int k = 0; k < L->nz; ++k)
        for (int j = 0; j < L->ny; ++j)
            for (int i = 0; i < L->nx; ++i) {
                int c = i + sx * (j + L->ny * k);
                if (L->diag[c] <= 0) { L->r[c] = 0; continue; }
                double s = L->b[c] - L->diag[c] * L->x[c];
                if (i > 0) s += L->ax[i + (L->nx + 1) * (j + L->ny * k)] * L->x[c - 1];
                if (i < L->nx - 1) s += L->ax[i + 1 + (L->nx + 1) * (j + L->ny * k)] * L->x[c + 1];
                if (j > 0) s += L->ay[i + L->nx * (j + (L->ny + 1) * k)] * L->x[c - sx];
                if (j < L->ny - 1) s += L->ay[i + L->nx * (j + 1 + (L->ny + 1) * k)] * L->x[c + sx];
                if (k > 0) s += L->az[i + L->nx * (j + L->ny * k)] * L->x[c - sxy];
                if (k < L->nz - 1) s += L->az[i + L->nx * (j + L->ny * (k + 1))] * L->x[c + sxy];
                L->r[c] = s;
            }
}

/* jacobi, src/sim/pressure_mg.cpp:237-247 */
static void jacobi(Level* L, double omega) {
    for (int I = 0; I < L->n; ++I) {
        if (L->diag[I] <= 0) { L->t[I] = 0; continue; }
        double s = L->b[I];
        for (int q = L->rowStart[I]; q < L->rowStart[I + 1]; ++q) s += L->val[q] * L->x[L->col[q]];
        L->t[I] = (1 - omega) * L->x[I] + omega * s / L->diag[I];
    }
    double* t = L->x; L->x = L->t; L->t = t;
}

/* residualSparse, src/sim/pressure_mg.cpp:248-257 */
static void residualSparse(Level* L) {
    for (int I = 0; I < L->n; ++I) {
        if (L->diag[I] <= 0) { L->r[I] = 0; continue; }
        double s = L->b[I] - L->diag[I] * L->x[I];
        for (int q = L->rowStart[I]; q < L->rowStart[I + 1]; ++q) s += L->val[q] * L->x[L->col[q]];
        L->r[I] = s;
    }
}

/* gsSparseSweep, src/sim/pressure_mg.cpp:258-266 */
static void gsSparseSweep(Level* L, int forward) {
    for (int t = 0; t < L->n; ++t) {
        int I = forward ? t : L->n - 1 - t;
        if (L->diag[I] <= 0) { L->x[I] = 0; continue; }
        double s = L->b[I];
        for (int q = L->rowStart[I]; q < L->rowStart[I + 1]; ++q) s += L->val[q] * L->x[L->col[q]];
        L->x[I] = s / L->diag[I];
    }
}

/* Solver::pressurePrecondition, src/sim/pressure_mg.cpp:270-300 */
static void precondition(Orc* o, const double* r, double* z) {
    if (o->mgDirty || o->nLevels == 0) buildPressureLevels(o);
    const int nl = o->nLevels;
    memcpy(o->lv[0].b, r, o->N * sizeof(double));
    for (int l = 0; l < nl; ++l) {
        Level* L = &o->lv[l];
        for (int i = 0; i < L->n; ++i) L->x[i] = 0;
        int coarsest = l == nl - 1 || L->agg == NULL;
        if (coarsest) {
            for (int it = 0; it < 20; ++it) { gsSparseSweep(L, 1); gsSparseSweep(L, 0); }
            break;
        }
        if (l == 0) { gsColor(L, 0); gsColor(L, 1); residualGrid(L); }
        else { jacobi(L, 0.7); jacobi(L, 0.7); residualSparse(L); }
        Level* C = &o->lv[l + 1];
        for (int i = 0; i < C->n; ++i) C->b[i] = 0;
        for (int i = 0; i < L->n; ++i) if (L->agg[i] >= 0) C->b[L->agg[i]] += L->r[i];
    }
    int last = 0;
    while (last + 1 < nl && o->lv[last].agg != NULL) ++last;
    for (int l = last - 1; l >= 0; --l) {
        Level* L = &o->lv[l];
        const Level* C = &o->lv[l + 1];
        for (int i = 0; i < L->n; ++i) if (L->agg[i] >= 0) L->x[i] += C->x[L->agg[i]];
        if (l == 0) { gsColor(L, 1); gsColor(L, 0); }
        else { jacobi(L, 0.7); jacobi(L, 0.7); }
    }
    memcpy(z, o->lv[0].x, o->N * sizeof(double));
}

void orc_precondition(Orc* o, const double* r, double* z) { precondition(o, r, z); }

/* Solver::project, src/sim/gasphase.cpp:505-677 */
static inline double hOut(double vel, int inflow) { return inflow ? -0.5 * vel * vel : 0.0; }

static void coefs(const Orc* o, int i, int j, int k, double a[6]) {
    a[0] = o->ax[xfaceI(o, i, j, k)]; a[1] = o->ax[xfaceI(o, i + 1, j, k)];
    a[2] = o->ay[yfaceI(o, i, j, k)]; a[3] = o->ay[yfaceI(o, i, j + 1, k)];
    a[4] = o->az[zfaceI(o, i, j, k)]; a[5] = o->az[zfaceI(o, i, j, k + 1)];
    double z = o->oz + (k + 0.5) * o->dx;
    if (i == 0 && !bndOpen(o, 0, 0, z)) a[0] = 0;
    if (i == o->nx - 1 && !bndOpen(o, 0, 1, z)) a[1] = 0;
    if (j == 0 && !bndOpen(o, 1, 0, z)) a[2] = 0;
    if (j == o->ny - 1 && !bndOpen(o, 1, 1, z)) a[3] = 0;
}

static double applySlice(const Orc* o, const double* diag, const double* x, double* y, int k) {
    const int nx = o->nx, ny = o->ny, nz = o->nz, sxy = nx * ny;
    double dot = 0;
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            int c = cellI(o, i, j, k);
            if (diag[c] <= 0) { y[c] = 0; continue; }
            double a[6];
            coefs(o, i, j, k, a);
            double s = diag[c] * x[c];
            if (i > 0) s -= a[0] * x[c - 1];
            if (i < nx - 1) s -= a[1] * x[c + 1];
            if (j > 0) s -= a[2] * x[c - nx];
            if (j < ny - 1) s -= a[3] * x[c + nx];
            if (k > 0) s -= a[4] * x[c - sxy];
            if (k < nz - 1) s -= a[5] * x[c + sxy];
            y[c] = s;
            dot += (double)s * x[c];
        }
    return dot;
}

static double maxAbsOf(const Orc* o, const double* r) {
    const int sxy = o->nx * o->ny;
    double m = 0;
    for (int k = 0; k < o->nz; ++k) {
        double mk = 0;
        for (int c = k * sxy; c < (k + 1) * sxy; ++c) mk = mx(mk, fabs(r[c]));
        m = k == 0 ? mk : mx(m, mk);
    }
    return m;
}

static double dotRZ(const Orc* o, const double* r, const double* z) {
    const int sxy = o->nx * o->ny;
    double tot = 0;
    for (int k = 0; k < o->nz; ++k) {
        double s = 0;
        for (int c = k * sxy; c < (k + 1) * sxy; ++c) s += (double)r[c] * z[c];
        tot += s;
    }
    return tot;
}

static void project(Orc* o, double dt) {
    const int nx = o->nx, ny = o->ny, nz = o->nz, sxy = nx * ny, N = o->N;
    const double inv = o->dx * o->dx / dt;
    double* diag = o->tmp[9];
    double* b = o->rhs;
    double bmax = 0;
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                int c = cellI(o, i, j, k);
                if (o->blocked[c]) { b[c] = 0; diag[c] = 0; o->p[c] = 0; continue; }
                int a0 = xfaceI(o, i, j, k), a1 = a0 + 1, b0 = yfaceI(o, i, j, k), b1 = yfaceI(o, i, j + 1, k),
                    c0 = zfaceI(o, i, j, k), c1 = zfaceI(o, i, j, k + 1);
                double div = (o->fx[a1] * o->u[a1] - o->fx[a0] * o->u[a0] + o->fy[b1] * o->v[b1] - o->fy[b0] * o->v[b0] +
                              o->fz[c1] * o->w[c1] - o->fz[c0] * o->w[c0]) / o->dx;
                b[c] = (o->S[c] - div) * inv;
                double a[6];
                coefs(o, i, j, k, a);
                if (i == 0 && a[0] > 0) b[c] += a[0] * hOut(o->u[a0], o->u[a0] > 0);
                if (i == nx - 1 && a[1] > 0) b[c] += a[1] * hOut(o->u[a1], o->u[a1] < 0);
                if (j == 0 && a[2] > 0) b[c] += a[2] * hOut(o->v[b0], o->v[b0] > 0);
                if (j == ny - 1 && a[3] > 0) b[c] += a[3] * hOut(o->v[b1], o->v[b1] < 0);
                if (k == nz - 1 && a[5] > 0) b[c] += a[5] * hOut(o->w[c1], o->w[c1] < 0);
                diag[c] = a[0] + a[1] + a[2] + a[3] + a[4] + a[5];
                if (diag[c] > 0) bmax = mx(bmax, fabs(b[c]));
            }
    double *r = o->cgR, *z = o->cgZ, *d = o->cgP, *q = o->cgQ;
    for (int k = 0; k < nz; ++k) {
        applySlice(o, diag, o->p, q, k);
        for (int c = k * sxy; c < (k + 1) * sxy; ++c) r[c] = diag[c] > 0 ? b[c] - q[c] : 0.0;
    }
    precondition(o, r, z);
    memcpy(d, z, N * sizeof(double));
    double rz = dotRZ(o, r, z);
    int it = 0;
    double rmax = maxAbsOf(o, r);
    double res = rmax / inv;
    /* the relative test (an addition to the reference): max|r| <= relTol max|b| */
    double relStop = o->relTol > 0 ? o->relTol * bmax : -1.0;
    while (res > o->tol && it < o->maxIters && rz > 0 && !(rmax <= relStop)) {
        double dq = 0;
        for (int k = 0; k < nz; ++k) dq += applySlice(o, diag, d, q, k);
        if (dq <= 0) break;
        double alpha = rz / dq;
        for (int c = 0; c < N; ++c) {
            if (diag[c] <= 0) continue;
            o->p[c] += (double)(alpha * d[c]);
            r[c] -= (double)(alpha * q[c]);
        }
        precondition(o, r, z);
        double rzNew = dotRZ(o, r, z);
        double beta = rzNew / rz;
        rz = rzNew;
        for (int c = 0; c < N; ++c) d[c] = z[c] + (double)(beta * d[c]);
        ++it;
        rmax = maxAbsOf(o, r);
        res = rmax / inv;
    }
    o->pressureIters = it;
    o->pressureResidual = maxAbsOf(o, r) / inv;
    /* closed zones: keep the zone mean of H at zero (:629-639) */
    {
        int nZ = o->nZones;
        double* sum = (double*)calloc(nZ ? nZ : 1, sizeof(double));
        double* cnt = (double*)calloc(nZ ? nZ : 1, sizeof(double));
        for (int c = 0; c < N; ++c)
            if (o->zone[c] >= 0 && !o->zoneOpen[o->zone[c]]) { sum[o->zone[c]] += o->p[c]; cnt[o->zone[c]] += 1; }
        int any = 0;
        for (int zz = 0; zz < nZ; ++zz) if (cnt[zz] > 0) { sum[zz] /= cnt[zz]; any = 1; }
        if (any)
            for (int c = 0; c < N; ++c)
                if (o->zone[c] >= 0 && !o->zoneOpen[o->zone[c]]) o->p[c] -= (double)sum[o->zone[c]];
        free(sum); free(cnt);
    }
    /* velocity correction u -= dt grad H on matrix faces (:641-676) */
    const double s = dt / o->dx;
    double maxVel = 0;
#define PP(i_, j_, k_) o->p[cellI(o, i_, j_, k_)]
    for (int k = 0; k < nz; ++k) {
        double vm = 0;
        double zc = o->oz + (k + 0.5) * o->dx;
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i <= nx; ++i) {
                int f = xfaceI(o, i, j, k);
                if (o->fx[f] <= 0) { o->u[f] = 0; continue; }
                if (o->ax[f] > 0 && !((i == 0 || i == nx) && !bndOpen(o, 0, i == 0 ? 0 : 1, zc)))
                    o->u[f] = clampd(o->u[f] - s * ((i < nx ? PP(i, j, k) : hOut(o->u[f], o->u[f] < 0)) -
                                                    (i > 0 ? PP(i - 1, j, k) : hOut(o->u[f], o->u[f] > 0))), -VMAX, VMAX);
                vm = mx(vm, fabs(o->u[f]) * o->fx[f]);
            }
        for (int j = 0; j <= ny; ++j)
            for (int i = 0; i < nx; ++i) {
                int f = yfaceI(o, i, j, k);
                if (o->fy[f] <= 0) { o->v[f] = 0; continue; }
                if (o->ay[f] > 0 && !((j == 0 || j == ny) && !bndOpen(o, 1, j == 0 ? 0 : 1, zc)))
                    o->v[f] = clampd(o->v[f] - s * ((j < ny ? PP(i, j, k) : hOut(o->v[f], o->v[f] < 0)) -
                                                    (j > 0 ? PP(i, j - 1, k) : hOut(o->v[f], o->v[f] > 0))), -VMAX, VMAX);
                vm = mx(vm, fabs(o->v[f]) * o->fy[f]);
            }
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                int f = zfaceI(o, i, j, k + 1);
                if (o->fz[f] <= 0) { o->w[f] = 0; continue; }
                if (o->az[f] > 0)
                    o->w[f] = clampd(o->w[f] - s * ((k + 1 < nz ? PP(i, j, k + 1) : hOut(o->w[f], o->w[f] < 0)) - PP(i, j, k)),
                                     -VMAX, VMAX);
                vm = mx(vm, fabs(o->w[f]) * o->fz[f]);
            }
        maxVel = k == 0 ? vm : mx(maxVel, vm);
    }
#undef PP
    o->maxVel = maxVel;
}

/* Solver::advectScalars, src/sim/gasphase.cpp:685-784 */
static inline double superbee(double r) {
    double m = 0.0, a = mn(2 * r, 1.0), b = mn(r, 2.0);
    if (m < a) m = a;
    if (m < b) m = b;
    return m;
}

static void advectScalars(Orc* o, double dt) {
    enum { NF = 10 };
    double* fields[NF] = {o->T, o->Yo, o->Yf, o->Ys, o->Ya, o->Yp, o->Yc, o->Yw, o->Yco, o->Yai};
    const double amb[NF] = {T0, YO2_AMB, 0, 0, 0, 0, YCO2_AMB, YH2O_AMB, 0, 0};
    const double s = dt / o->dx;
    const int nx = o->nx, ny = o->ny, nz = o->nz, sxy = nx * ny;
    const double* T = o->T;
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                int c = cellI(o, i, j, k);
                if (o->blocked[c]) {
                    for (int q = 0; q < NF; ++q) o->tmp[q][c] = fields[q][c];
                    continue;
                }
                int fa0 = xfaceI(o, i, j, k), fa1 = fa0 + 1, fb0 = yfaceI(o, i, j, k), fb1 = yfaceI(o, i, j + 1, k),
                    fc0 = zfaceI(o, i, j, k), fc1 = zfaceI(o, i, j, k + 1);
                double un[6] = {-o->fx[fa0] * o->u[fa0], o->fx[fa1] * o->u[fa1], -o->fy[fb0] * o->v[fb0],
                                o->fy[fb1] * o->v[fb1], -o->fz[fc0] * o->w[fc0], o->fz[fc1] * o->w[fc1]};
                double fo[6] = {o->fx[fa0], o->fx[fa1], o->fy[fb0], o->fy[fb1], o->fz[fc0], o->fz[fc1]};
                int id[3] = {i, j, k};
                const int dim[3] = {nx, ny, nz}, st[3] = {1, nx, sxy};
                int nb[6], nb2[6], opp[6];
                for (int d = 0; d < 6; ++d) {
                    int a = d >> 1, sg = (d & 1) ? 1 : -1;
                    int n1 = id[a] + sg, n2 = id[a] + 2 * sg, o1 = id[a] - sg;
                    nb[d] = (n1 >= 0 && n1 < dim[a]) ? c + sg * st[a] : -1;
                    nb2[d] = (n2 >= 0 && n2 < dim[a]) ? c + 2 * sg * st[a] : -1;
                    opp[d] = (o1 >= 0 && o1 < dim[a]) ? c - sg * st[a] : -1;
                    if (nb[d] >= 0 && o->blocked[nb[d]]) nb[d] = -2;
                    if (nb2[d] >= 0 && o->blocked[nb2[d]]) nb2[d] = -2;
                    if (opp[d] >= 0 && o->blocked[opp[d]]) opp[d] = -2;
                }
                double nuc = o->nu[c];
                double rc = gasDensity(o, c), rUp[6], mden = rc;
                for (int d = 0; d < 6; ++d) {
                    rUp[d] = 0;
                    if (fo[d] <= 0 || nb[d] == -2) continue;
                    double tn = nb[d] >= 0 ? T[nb[d]] : T0, tc = T[c], tf;
                    if (un[d] > 0) {
                        double tu2 = opp[d] >= 0 ? T[opp[d]] : (opp[d] == -1 ? T0 : tc);
                        double den = tn - tc;
                        tf = tc + (fabs(den) > 1e-6 ? 0.5 * superbee((tc - tu2) / den) * den : 0.0);
                    } else {
                        double tu2 = nb2[d] >= 0 ? T[nb2[d]] : (nb2[d] == -1 ? T0 : tn);
                        double den = tc - tn;
                        tf = tn + (fabs(den) > 1e-6 ? 0.5 * superbee((tn - tu2) / den) * den : 0.0);
                    }
                    double pu = un[d] > 0 ? o->Pb[c] : (nb[d] >= 0 ? o->Pb[nb[d]] : P0);
                    rUp[d] = pu / (RS * mx(tf, T_MIN));
                    mden -= s * rUp[d] * un[d];
                }
                int conservative = mden > 0.25 * rc;
                for (int q = 0; q < NF; ++q) {
                    const double* F = fields[q];
                    double fc = F[c];
                    double lo = fc, hi = fc, acc = 0, macc = 0;
                    for (int d = 0; d < 6; ++d) {
                        if (fo[d] <= 0 || nb[d] == -2) continue;
                        double fn = nb[d] >= 0 ? F[nb[d]] : amb[q];
                        lo = mn(lo, fn);
                        hi = mx(hi, fn);
                        double flux = un[d];
                        double face = fc;
                        if (flux > 0) {
                            double fu2 = opp[d] >= 0 ? F[opp[d]] : (opp[d] == -1 ? amb[q] : fc);
                            double den = fn - fc;
                            if (fabs(den) > 1e-12) face += 0.5 * superbee((fc - fu2) / den) * den;
                        } else if (flux < 0) {
                            double fu2 = nb2[d] >= 0 ? F[nb2[d]] : (nb2[d] == -1 ? amb[q] : fn);
                            double den = fc - fn;
                            face = fn;
                            if (fabs(den) > 1e-12) face += 0.5 * superbee((fn - fu2) / den) * den;
                        }
                        acc -= flux * (face - fc);
                        macc -= rUp[d] * flux * face;
                        if (q > 0) {
                            double nun = nb[d] >= 0 ? o->nu[nb[d]] : nuc;
                            double D = 0.5 * (nuc + nun) / SC_T + 2.0e-5;
                            double rf = nb[d] >= 0 ? 0.5 * (rc + gasDensity(o, nb[d])) : rc;
                            acc += fo[d] * D * (fn - fc) / o->dx;
                            macc += fo[d] * rf * D * (fn - fc) / o->dx;
                        }
                    }
                    double val = conservative ? (rc * fc + s * macc) / mden : fc + s * acc;
                    o->tmp[q][c] = clampd(val, lo, hi);
                }
            }
    double** fp[NF] = {&o->T, &o->Yo, &o->Yf, &o->Ys, &o->Ya, &o->Yp, &o->Yc, &o->Yw, &o->Yco, &o->Yai};
    for (int q = 0; q < NF; ++q) {
        double* t = *fp[q];
        *fp[q] = o->tmp[q];
        o->tmp[q] = t;
    }
}

/* Solver::gatherStats, src/sim/solver.cpp:884-915 (gas part) */
static void gatherStats(Orc* o, double dt) {
    const double V = o->dx * o->dx * o->dx;
    double h = 0, mt = T0, fd = 0;
    int nb = 0;
    for (int c = 0; c < o->N; ++c) {
        if (o->blocked[c]) continue;
        fd += (double)o->Yf[c] * gasDensity(o, c) * V;
        h += o->hrr[c] * V;
        if (o->T[c] > mt) mt = o->T[c];
        if (o->hrr[c] > 0) ++nb;
    }
    o->st_hrr = h;
    o->st_fuelBurned += (double)h * dt / DHC_FUEL;
    o->st_fuelInDomain = fd;
    o->st_maxGasT = mt;
    o->st_burning = nb;
}

static void clearStep(Orc* o) {
    for (int c = 0; c < o->N; ++c) { o->Q[c] = 0; o->Qr[c] = 0; o->pilot[c] = 0; o->massSrc[c] = 0; }
}

static void zonePressureUpdate(Orc* o, double dt) {
    for (int z = 0; z < o->nZones; ++z)
        if (!o->zoneOpen[z]) o->zoneP[z] = clampd(o->zoneP[z] + dt * o->zoneDP[z], P0 - 20000.0, P0 + 50000.0);
    for (int c = 0; c < o->N; ++c) if (o->zone[c] >= 0) o->Pb[c] = o->zoneP[o->zone[c]];
}

/* Solver::step, src/sim/solver.cpp:226-269 (gas-only stages) */
double orc_step(Orc* o, double dtMax) {
    double dt = orc_stable_dt(o, dtMax);
    if (o->zonesDirty) computeZones(o);
    clearStep(o);
    injectIgnitions(o, dt);
    injectBurners(o, dt);
    combustion(o, dt);
    /* radiationStep returns at once when radiation is off or surfaces are adiabatic
     * (src/sim/radiation.cpp:322); solidsStep and barriersStep loop over solid cells
     * and barriers, of which the gas-only cases have none */
    turbulence(o);
    heatDiffusion(o, dt);
    energyAndExpansion(o, dt);
    momentum(o, dt);
    leakage(o, dt);
    project(o, dt);
    advectScalars(o, dt);
    zonePressureUpdate(o, dt);
    gatherStats(o, dt);
    o->time += dt;
    return dt;
}

int orc_stage(Orc* o, const char* n, double dt) {
    if (!strcmp(n, "zones")) computeZones(o);
    else if (!strcmp(n, "mg")) buildPressureLevels(o);
    else if (!strcmp(n, "clear")) clearStep(o);
    else if (!strcmp(n, "burners")) { injectIgnitions(o, dt); injectBurners(o, dt); }
    else if (!strcmp(n, "combustion")) combustion(o, dt);
    else if (!strcmp(n, "turbulence")) turbulence(o);
    else if (!strcmp(n, "heat")) heatDiffusion(o, dt);
    else if (!strcmp(n, "energy")) energyAndExpansion(o, dt);
    else if (!strcmp(n, "momentum")) momentum(o, dt);
    else if (!strcmp(n, "leakage")) leakage(o, dt);
    else if (!strcmp(n, "project")) project(o, dt);
    else if (!strcmp(n, "advect")) advectScalars(o, dt);
    else if (!strcmp(n, "zonep")) zonePressureUpdate(o, dt);
    else if (!strcmp(n, "stats")) gatherStats(o, dt);
    else return -1;
    return 0;
}

/* ---- field access ------------------------------------------------------- */
static int lookup(Orc* o, const char* n, void** ptr, long* len) {
    int N = o->N;
#define RF(name_, arr_, n_) if (!strcmp(n, name_)) { *ptr = (void*)(arr_); *len = (n_); return 0; }
#define BF(name_, arr_, n_) if (!strcmp(n, name_)) { *ptr = (void*)(arr_); *len = (n_); return 1; }
    RF("u", o->u, o->NX) RF("v", o->v, o->NY) RF("w", o->w, o->NZ)
    RF("fx", o->fx, o->NX) RF("fy", o->fy, o->NY) RF("fz", o->fz, o->NZ)
    RF("ax", o->ax, o->NX) RF("ay", o->ay, o->NY) RF("az", o->az, o->NZ)
    BF("lx", o->lx, o->NX) BF("ly", o->ly, o->NY) BF("lz", o->lz, o->NZ)
    RF("p", o->p, N) RF("S", o->S, N) RF("T", o->T, N) RF("Yo", o->Yo, N) RF("Yf", o->Yf, N) RF("Ys", o->Ys, N)
    RF("Ya", o->Ya, N) RF("Yp", o->Yp, N) RF("Yc", o->Yc, N) RF("Yw", o->Yw, N) RF("Yco", o->Yco, N)
    RF("Yai", o->Yai, N) RF("nu", o->nu, N) RF("Pb", o->Pb, N) RF("Q", o->Q, N) RF("Qr", o->Qr, N)
    RF("hrr", o->hrr, N) RF("massSrc", o->massSrc, N)
    BF("lit", o->lit, N) BF("pilot", o->pilot, N) BF("blocked", o->blocked, N)
    RF("rhs", o->rhs, N) RF("diag", o->tmp[9], N) RF("cgR", o->cgR, N) RF("cgZ", o->cgZ, N) RF("cgP", o->cgP, N)
    RF("cgQ", o->cgQ, N)
    RF("zoneP", o->zoneP, o->nZones) BF("zoneOpen", o->zoneOpen, o->nZones)
    RF("zoneDP", o->zoneDP, o->zoneDP ? o->nZones : 0)
    if (!strcmp(n, "zone")) { *ptr = (void*)o->zone; *len = N; return 2; }
#undef RF
#undef BF
    return -1;
}

long orc_field_len(Orc* o, const char* name) {
    void* p;
    long n;
    return lookup(o, name, &p, &n) < 0 ? -1 : n;
}

int orc_field(Orc* o, const char* name, int dir, void* buf, long n) {
    void* p;
    long len;
    int t = lookup(o, name, &p, &len);
    if (t < 0 || len != n) return -1;
    size_t bytes = (size_t)n * (t == 0 ? 8 : t == 1 ? 1 : 4);
    if (dir == 0) memcpy(buf, p, bytes); else memcpy(p, buf, bytes);
    return t;
}

void orc_scalars(Orc* o, double* out) {
    out[0] = o->time; out[1] = o->maxVel; out[2] = o->maxNu; out[3] = o->maxDiv;
    out[4] = o->pressureIters; out[5] = o->pressureResidual; out[6] = o->st_hrr; out[7] = o->st_maxGasT;
    out[8] = o->st_burning; out[9] = o->st_fuelIn; out[10] = o->st_fuelBurned; out[11] = o->st_fuelInDomain;
    out[12] = o->leakFaces; out[13] = o->nZones;
}

void orc_set_scalars(Orc* o, double time, double maxVel, double maxNu, double maxDiv) {
    o->time = time; o->maxVel = maxVel; o->maxNu = maxNu; o->maxDiv = maxDiv;
}

int orc_mg_levels(Orc* o) { return o->nLevels; }

void orc_mg_info(Orc* o, int l, int* info) {
    Level* L = &o->lv[l];
    info[0] = L->n; info[1] = l == 0 ? 0 : L->nnz; info[2] = L->agg ? L->n : 0;
}

void orc_mg_get(Orc* o, int l, int* agg, int* rowStart, int* col, double* val, double* diag) {
    Level* L = &o->lv[l];
    if (L->agg) memcpy(agg, L->agg, L->n * sizeof(int));
    if (l > 0) {
        memcpy(rowStart, L->rowStart, (L->n + 1) * sizeof(int));
        memcpy(col, L->col, L->nnz * sizeof(int));
        memcpy(val, L->val, L->nnz * sizeof(double));
    }
    memcpy(diag, L->diag, L->n * sizeof(double));
}

/* ------------------------------------------------------------------------
 * Radiation trace (src/sim/radiation.cpp). Constants of :41-51; the
 * reference's PI is the literal 3.14159265 (:44), not M_PI.
 * ------------------------------------------------------------------------ */
#define RAD_NB 4
#define RAD_DIRS 32
#define RAD_BLOCKS 24
static const double RAD_PI = 3.14159265;
static const double RAD_MAXLEN = 8.0, RAD_SIGMA = 5.670374e-8, RAD_T0 = 293.15;
static const double RAD_EDGE[RAD_NB + 1] = {0.0, 2.7, 8.0, 14.0, 1e9};
static const double RAD_LAMBDA[RAD_NB] = {1.5, 4.5, 11.0, 25.0};
static const double RAD_GAS[RAD_NB] = {0.05, 3.0, 0.1, 6.0};
static const double RAD_SOOT_C = 5.5, RAD_SOOT_DENSITY = 1800.0, RAD_T_FLAME = 1400.0, RAD_CHI_R = 0.35;

/* fraction of blackbody emission below lambda*T (um K): Chang & Rhee series (:54-63) */
static double rad_planck_below(double lambdaT) {
    if (lambdaT <= 0) return 0;
    if (lambdaT > 1e8) return 1;
    double x = 14388.0 / lambdaT, s = 0;
    for (int n = 1; n <= 12; ++n) {
        double xn = x * n, dn = (double)n;
        s += exp(-xn) / n * (x * x * x + 3 * x * x / n + 6 * x / (dn * n) + 6 / (dn * n * n));
    }
    double v = 1.0 - 15.0 / (RAD_PI * RAD_PI * RAD_PI * RAD_PI) * s;
    return v < 0.0 ? 0.0 : v > 1.0 ? 1.0 : v;
}
static void rad_band_fractions(double T, double f[RAD_NB]) {   /* :64-71 */
    double prev = 0;
    for (int b = 0; b < RAD_NB; ++b) {
        double up = b == RAD_NB - 1 ? 1.0 : rad_planck_below(RAD_EDGE[b + 1] * T);
        f[b] = up - prev;
        prev = up;
    }
}
/* band emissive power relative to ambient, W/m2 (:73-81) */
static void rad_band_power(double T, double out[RAD_NB]) {
    double f0[RAD_NB], f[RAD_NB];
    rad_band_fractions(RAD_T0, f0);
    rad_band_fractions(T, f);
    double a = T * T, a0 = RAD_T0 * RAD_T0;
    for (int b = 0; b < RAD_NB; ++b) out[b] = RAD_SIGMA * (f[b] * a * a - f0[b] * a0 * a0);
}

void orc_rad_trace(int nx, int ny, int nz, double dx, double ox, double oy, double oz, const uint8_t* blocked,
                   const double* T, const double* Ys, const double* Yw, const double* Yc, const double* Pb,
                   const double* hrr, int nElem, const double* elem, int nWall, const double* wall,
                   const double* solidT, double* radAbs, double* radGas) {
    const long N = (long)nx * ny * nz;
    const long NF[3] = {(long)(nx + 1) * ny * nz, (long)nx * (ny + 1) * nz, (long)nx * ny * (nz + 1)};
    /* directions: golden-spiral points on the sphere (:84-96) */
    double dir[RAD_DIRS][3];
    const double ga = RAD_PI * (3.0 - sqrt(5.0));
    for (int i = 0; i < RAD_DIRS; ++i) {
        double z = 1.0 - 2.0 * (i + 0.5) / RAD_DIRS;
        double r = sqrt(fmax(0.0, 1 - z * z));
        dir[i][0] = r * cos(ga * i); dir[i][1] = r * sin(ga * i); dir[i][2] = z;
    }
    const double dW = 4.0 * RAD_PI / RAD_DIRS;
    /* per-cell absorption coefficient and source function per band (:193-222) */
    double* kap = calloc((size_t)N * RAD_NB, sizeof(double));
    double* src = calloc((size_t)N * RAD_NB, sizeof(double));
    uint8_t* flame = calloc((size_t)N, 1);
    double fFlame[RAD_NB];
    rad_band_fractions(RAD_T_FLAME, fFlame);
    for (long c = 0; c < N; ++c) {
        if (blocked[c]) continue;
        double rho = Pb[c] / (287.0 * T[c]);
        double fv = rho * Ys[c] / RAD_SOOT_DENSITY;
        double pg = (Yw[c] * 28.96 / 18.02 + Yc[c] * 28.96 / 44.01) * Pb[c] / 101325.0;
        double Eb[RAD_NB], k[RAD_NB];
        rad_band_power(T[c], Eb);
        double jfTot = hrr[c] > 0 ? RAD_CHI_R * hrr[c] / (4.0 * RAD_PI) : 0.0;
        double jTot = 0;
        for (int q = 0; q < RAD_NB; ++q) {
            k[q] = RAD_SOOT_C * fv / (RAD_LAMBDA[q] * 1e-6) + RAD_GAS[q] * pg + 1e-4;
            jTot += k[q] * Eb[q] / RAD_PI;
        }
        int fl = jfTot > jTot;
        flame[c] = (uint8_t)fl;
        for (int q = 0; q < RAD_NB; ++q) {
            double j = fl ? jfTot * fFlame[q] : k[q] * Eb[q] / RAD_PI;
            kap[c * RAD_NB + q] = k[q];
            src[c * RAD_NB + q] = j / k[q];
        }
    }
    /* wall per face (Solver::barrierOn + barrierIntact, src/sim/solver.cpp:51-62) */
    int* wallOf[3];
    for (int a = 0; a < 3; ++a) {
        wallOf[a] = malloc((size_t)NF[a] * sizeof(int));
        for (long f = 0; f < NF[a]; ++f) wallOf[a][f] = -1;
    }
    for (int w = 0; w < nWall; ++w) wallOf[(int)wall[4 * w]][(long)wall[4 * w + 1]] = w;

    double* gb = malloc((size_t)N * sizeof(double));
    for (long c = 0; c < N; ++c) radGas[c] = 0;
    const int dim[3] = {nx, ny, nz};
    for (int blk = 0; blk < RAD_BLOCKS; ++blk) {   /* :223-306 */
        for (long c = 0; c < N; ++c) gb[c] = 0;
        int e0 = (int)((long)nElem * blk / RAD_BLOCKS), e1 = (int)((long)nElem * (blk + 1) / RAD_BLOCKS);
        for (int ei = e0; ei < e1; ++ei) {
            const double* el = elem + 11 * ei;
            const double* n = el + 3;
            const double area = el[6], eps = el[7], temp = el[8];
            const int sphere = el[9] != 0, skipOwn = el[10] != 0;
            double Is[RAD_NB];
            rad_band_power(temp, Is);
            for (int q = 0; q < RAD_NB; ++q) Is[q] *= eps / RAD_PI;
            double wsum = 0;
            if (!sphere)
                for (int d = 0; d < RAD_DIRS; ++d) {
                    double cs = dir[d][0] * n[0] + dir[d][1] * n[1] + dir[d][2] * n[2];
                    if (cs > 0) wsum += cs * dW;
                }
            double norm = sphere ? 1.0 : (wsum > 0 ? RAD_PI / wsum : 0.0);
            double absorbed = 0;
            for (int d = 0; d < RAD_DIRS; ++d) {
                double w;
                if (sphere) w = dW * 0.25 * area;
                else {
                    double cs = dir[d][0] * n[0] + dir[d][1] * n[1] + dir[d][2] * n[2];
                    if (cs <= 0) continue;
                    w = cs * dW * norm * area;
                }
                /* Amanatides-Woo march from the element origin */
                double p[3] = {(el[0] - ox) / dx, (el[1] - oy) / dx, (el[2] - oz) / dx};
                int ci[3] = {(int)floor(p[0]), (int)floor(p[1]), (int)floor(p[2])};
                if (ci[0] < 0 || ci[1] < 0 || ci[2] < 0 || ci[0] >= nx || ci[1] >= ny || ci[2] >= nz) continue;
                int stp[3];
                double tMax[3], tDel[3];
                for (int a = 0; a < 3; ++a) {
                    double dv = dir[d][a];
                    if (dv > 1e-9) { stp[a] = 1; tMax[a] = (ci[a] + 1 - p[a]) / dv; tDel[a] = 1 / dv; }
                    else if (dv < -1e-9) { stp[a] = -1; tMax[a] = (p[a] - ci[a]) / -dv; tDel[a] = -1 / dv; }
                    else { stp[a] = 0; tMax[a] = 1e30; tDel[a] = 1e30; }
                }
                double t = 0, tau[RAD_NB] = {1, 1, 1, 1}, I[RAD_NB] = {0, 0, 0, 0}, Iend[RAD_NB] = {0, 0, 0, 0};
                const double tEnd = RAD_MAXLEN / dx;
                long c = ci[0] + (long)nx * (ci[1] + (long)ny * ci[2]);
                const long skip = skipOwn ? c : -1;
                for (;;) {
                    int a = tMax[0] < tMax[1] ? (tMax[0] < tMax[2] ? 0 : 2) : (tMax[1] < tMax[2] ? 1 : 2);
                    double tn = tEnd < tMax[a] ? tEnd : tMax[a];
                    double ds = (tn - t) * dx;
                    if (ds > 0 && !blocked[c] && c != skip) {
                        double g = 0;
                        for (int q = 0; q < RAD_NB; ++q) {
                            double x = kap[c * RAD_NB + q] * ds;
                            double att = x < 1e-3 ? x * (1 - 0.5 * x) : 1.0 - exp(-x);
                            double fromCell = tau[q] * src[c * RAD_NB + q] * att;
                            I[q] += fromCell;
                            g += Is[q] * tau[q] * att - (flame[c] ? 0.0 : eps * fromCell);
                            tau[q] *= 1.0 - att;
                        }
                        gb[c] += w * g;
                    }
                    t = tn;
                    if (t >= tEnd || (tau[0] < 1e-3 && tau[1] < 1e-3 && tau[2] < 1e-3 && tau[3] < 1e-3)) break;
                    /* the face crossed: the upper face of c along a when stepping up */
                    int up = stp[a] > 0;
                    int fi[3] = {ci[0], ci[1], ci[2]};
                    fi[a] += up;
                    long f = a == 0 ? fi[0] + (long)(nx + 1) * (fi[1] + (long)ny * fi[2])
                           : a == 1 ? fi[0] + (long)nx * (fi[1] + (long)(ny + 1) * fi[2])
                                    : fi[0] + (long)nx * (fi[1] + (long)ny * fi[2]);
                    int wi = wallOf[a][f];
                    if (wi >= 0) {
                        /* c is the lower cell of its upper face, the upper cell of its lower face */
                        rad_band_power(wall[4 * wi + (up ? 2 : 3)], Iend);
                        for (int q = 0; q < RAD_NB; ++q) Iend[q] *= 0.9 / RAD_PI;
                        break;
                    }
                    ci[a] += stp[a];
                    if (ci[a] < 0 || ci[a] >= dim[a]) break;
                    long nb = ci[0] + (long)nx * (ci[1] + (long)ny * ci[2]);
                    if (blocked[nb]) {
                        rad_band_power(solidT[nb], Iend);
                        for (int q = 0; q < RAD_NB; ++q) Iend[q] *= 0.9 / RAD_PI;
                        break;
                    }
                    c = nb;
                    tMax[a] += tDel[a];
                }
                double It = 0;
                for (int q = 0; q < RAD_NB; ++q) It += I[q] + tau[q] * Iend[q];
                absorbed += eps * w * It;
            }
            radAbs[ei] = absorbed;
        }
        for (long c = 0; c < N; ++c) radGas[c] += gb[c];
    }
    free(gb); free(kap); free(src); free(flame);
    for (int a = 0; a < 3; ++a) free(wallOf[a]);
}

/* ------------------------------------------------------------------------
 * Volume ray march of the viewer (src/render/renderer.cpp:119-283) in FP32.
 * GLSL built-ins follow the GLSL 3.30 definitions (mix = x(1-a) + ya,
 * smoothstep, fract = x - floor x); the 3D texture is sampled with linear
 * filtering and clamp-to-edge addressing (src/render/renderer.cpp:406-413).
 * ------------------------------------------------------------------------ */
typedef struct { float x, y, z; } ov3;
static ov3 o3(float a, float b, float c) { ov3 r = {a, b, c}; return r; }
static ov3 oadd(ov3 a, ov3 b) { return o3(a.x + b.x, a.y + b.y, a.z + b.z); }
static ov3 osub(ov3 a, ov3 b) { return o3(a.x - b.x, a.y - b.y, a.z - b.z); }
static ov3 omul(ov3 a, float s) { return o3(a.x * s, a.y * s, a.z * s); }
static ov3 omulv(ov3 a, ov3 b) { return o3(a.x * b.x, a.y * b.y, a.z * b.z); }
static float odot(ov3 a, ov3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static float ofract(float x) { return x - floorf(x); }
static float oclamp(float x, float a, float b) { return fminf(fmaxf(x, a), b); }
static float omix(float a, float b, float t) { return a * (1.0f - t) + b * t; }
static ov3 omix3(ov3 a, ov3 b, float t) { return oadd(omul(a, 1.0f - t), omul(b, t)); }
static float osmooth(float e0, float e1, float x) {
    float t = oclamp((x - e0) / (e1 - e0), 0.0f, 1.0f);
    return t * t * (3.0f - 2.0f * t);
}
static ov3 oheatmap(float t) {
    t = oclamp(t, 0.0f, 1.0f);
    ov3 c0 = o3(0.10f, 0.15f, 0.55f), c1 = o3(0.10f, 0.65f, 0.85f), c2 = o3(0.95f, 0.90f, 0.20f),
        c3 = o3(0.95f, 0.35f, 0.05f), c4 = o3(0.85f, 0.05f, 0.05f);
    if (t < 0.25f) return omix3(c0, c1, t / 0.25f);
    if (t < 0.5f) return omix3(c1, c2, (t - 0.25f) / 0.25f);
    if (t < 0.75f) return omix3(c2, c3, (t - 0.5f) / 0.25f);
    return omix3(c3, c4, (t - 0.75f) / 0.25f);
}
static ov3 oglow(float T) {
    float t = oclamp((T - 700.0f) / 1000.0f, 0.0f, 1.0f);
    return omul(omul(o3(1.0f, 0.22f + 0.6f * t, 0.04f + 0.45f * t * t), t), t);
}
static float ohash2(float px, float py) { return ofract(sinf(px * 12.9898f + py * 78.233f) * 43758.5453f); }
static float ohash3(ov3 p) {
    p = o3(ofract(p.x * 0.3183099f + 0.1f), ofract(p.y * 0.3183099f + 0.1f), ofract(p.z * 0.3183099f + 0.1f));
    p = omul(p, 17.0f);
    return ofract(p.x * p.y * p.z * (p.x + p.y + p.z));
}
static float onoise(ov3 x) {
    ov3 i = o3(floorf(x.x), floorf(x.y), floorf(x.z));
    ov3 f = o3(ofract(x.x), ofract(x.y), ofract(x.z));
    f = o3(f.x * f.x * (3.0f - 2.0f * f.x), f.y * f.y * (3.0f - 2.0f * f.y), f.z * f.z * (3.0f - 2.0f * f.z));
    float a = omix(omix(ohash3(i), ohash3(oadd(i, o3(1, 0, 0))), f.x),
                   omix(ohash3(oadd(i, o3(0, 1, 0))), ohash3(oadd(i, o3(1, 1, 0))), f.x), f.y);
    float b = omix(omix(ohash3(oadd(i, o3(0, 0, 1))), ohash3(oadd(i, o3(1, 0, 1))), f.x),
                   omix(ohash3(oadd(i, o3(0, 1, 1))), ohash3(oadd(i, o3(1, 1, 1))), f.x), f.y);
    return omix(a, b, f.z);
}
static float oflame_noise(ov3 p, float time) {
    ov3 q = osub(omulv(p, o3(5.0f, 5.0f, 2.6f)), o3(0.0f, 0.0f, time * 3.2f));
    return 0.55f * onoise(q) + 0.30f * onoise(oadd(omul(q, 2.1f), o3(0.0f, 0.0f, -time * 2.0f))) +
           0.15f * onoise(omul(q, 4.3f));
}
static float osmoke_noise(ov3 p, float time) {
    ov3 q = osub(omul(p, 1.6f), o3(0.0f, 0.0f, time * 0.35f));
    ov3 w = o3(onoise(oadd(q, o3(5.2f, 1.3f, 0.0f))), onoise(oadd(q, o3(1.7f, 9.2f, 3.1f))),
               onoise(oadd(q, o3(8.3f, 2.8f, 4.7f))));
    q = oadd(q, osub(omul(w, 0.6f), o3(0.3f, 0.3f, 0.3f)));
    float n = 0.5f * onoise(q) + 0.3f * onoise(oadd(omul(q, 2.03f), o3(1.7f, 1.7f, 1.7f))) +
              0.2f * onoise(oadd(omul(q, 4.1f), o3(3.3f, 3.3f, 3.3f)));
    return osmooth(0.2f, 0.8f, n);
}
static ov3 oflame_color(float k) {
    return omix3(omix3(o3(0.9f, 0.18f, 0.02f), o3(1.0f, 0.5f, 0.08f), osmooth(0.0f, 0.4f, k)), o3(1.0f, 0.9f, 0.55f),
                 osmooth(0.45f, 1.0f, k));
}
typedef struct { const float* vol; int nx, ny, nz; ov3 bmin, bmax; } OVol;
static void osample(const OVol* G, ov3 p, float out[4]) {
    ov3 u = o3((p.x - G->bmin.x) / (G->bmax.x - G->bmin.x), (p.y - G->bmin.y) / (G->bmax.y - G->bmin.y),
               (p.z - G->bmin.z) / (G->bmax.z - G->bmin.z));
    float x = u.x * G->nx - 0.5f, y = u.y * G->ny - 0.5f, z = u.z * G->nz - 0.5f;
    float fx = floorf(x), fy = floorf(y), fz = floorf(z);
    float ax = x - fx, ay = y - fy, az = z - fz;
    int i0 = (int)fmaxf(fminf(fx, (float)(G->nx - 1)), 0.0f), i1 = (int)fmaxf(fminf(fx + 1.0f, (float)(G->nx - 1)), 0.0f);
    int j0 = (int)fmaxf(fminf(fy, (float)(G->ny - 1)), 0.0f), j1 = (int)fmaxf(fminf(fy + 1.0f, (float)(G->ny - 1)), 0.0f);
    int k0 = (int)fmaxf(fminf(fz, (float)(G->nz - 1)), 0.0f), k1 = (int)fmaxf(fminf(fz + 1.0f, (float)(G->nz - 1)), 0.0f);
#define OAT(i, j, k) (G->vol + 4 * ((size_t)(i) + (size_t)G->nx * ((size_t)(j) + (size_t)G->ny * (size_t)(k))))
    for (int q = 0; q < 4; ++q) {
        float c00 = OAT(i0, j0, k0)[q] * (1.0f - ax) + OAT(i1, j0, k0)[q] * ax;
        float c10 = OAT(i0, j1, k0)[q] * (1.0f - ax) + OAT(i1, j1, k0)[q] * ax;
        float c01 = OAT(i0, j0, k1)[q] * (1.0f - ax) + OAT(i1, j0, k1)[q] * ax;
        float c11 = OAT(i0, j1, k1)[q] * (1.0f - ax) + OAT(i1, j1, k1)[q] * ax;
        float a = c00 * (1.0f - ay) + c10 * ay, b = c01 * (1.0f - ay) + c11 * ay;
        out[q] = a * (1.0f - az) + b * az;
    }
#undef OAT
}

/* the temperature slice where the ray crosses uSliceZ */
static void oslice(const OVol* G, const orc_vol_params* P, ov3 ro, ov3 rd, float tS, ov3* col, float* tr) {
    float sv[4];
    osample(G, oadd(ro, omul(rd, tS)), sv);
    if (sv[2] > 150.0f) {
        float tn = (sv[2] - P->t_min) / (P->t_max - P->t_min);
        float sa = omix(0.12f, 0.88f, osmooth(0.0f, 0.2f, tn));
        *col = oadd(*col, omul(oheatmap(tn), *tr * sa));
        *tr *= 1.0f - sa;
    }
}

void orc_vol_render(int nx, int ny, int nz, float dx, float ox, float oy, float oz, const float* vol,
                    const orc_vol_params* P, const float* depth, float* rgb, int row0, int row1) {
    OVol G = {vol, nx, ny, nz, o3(ox, oy, oz), o3(ox + nx * dx, oy + ny * dx, oz + nz * dx)};
    const float* M = P->inv_vp;
    for (int py = row0; py < row1; ++py)
        for (int px = 0; px < P->width; ++px) {
            float uvx = (px + 0.5f) / P->width, uvy = (py + 0.5f) / P->height;
            float wa = uvx * 2.0f - 1.0f, wb = uvy * 2.0f - 1.0f;
#define OWORLD(dd, out)                                                                   \
    do {                                                                                  \
        float c_ = (dd) * 2.0f - 1.0f;                                                    \
        float X_ = M[0] * wa + M[4] * wb + M[8] * c_ + M[12], Y_ = M[1] * wa + M[5] * wb + M[9] * c_ + M[13]; \
        float Z_ = M[2] * wa + M[6] * wb + M[10] * c_ + M[14], W_ = M[3] * wa + M[7] * wb + M[11] * c_ + M[15]; \
        out = o3(X_ / W_, Y_ / W_, Z_ / W_);                                              \
    } while (0)
            ov3 base = o3(P->background[0], P->background[1], P->background[2]);
            float d = depth ? depth[(size_t)py * P->width + px] : 1.0f;
            ov3 ro = o3(P->eye[0], P->eye[1], P->eye[2]), far_, wd;
            OWORLD(1.0f, far_);
            ov3 rd = osub(far_, ro);
            rd = omul(rd, 1.0f / sqrtf(odot(rd, rd)));
            float tScene = 1e9f;
            if (d < 1.0f) { OWORLD(d, wd); ov3 e = osub(wd, ro); tScene = sqrtf(odot(e, e)); }
#undef OWORLD
            ov3 bmax = o3(G.bmax.x, G.bmax.y, fminf(G.bmax.z, P->clip_z));
            ov3 inv = o3(1.0f / rd.x, 1.0f / rd.y, 1.0f / rd.z);
            ov3 ta = omulv(osub(G.bmin, ro), inv), tb = omulv(osub(bmax, ro), inv);
            ov3 tmn = o3(fminf(ta.x, tb.x), fminf(ta.y, tb.y), fminf(ta.z, tb.z));
            ov3 tmx = o3(fmaxf(ta.x, tb.x), fmaxf(ta.y, tb.y), fmaxf(ta.z, tb.z));
            float t0 = fmaxf(fmaxf(fmaxf(tmn.x, tmn.y), tmn.z), 0.0f);
            float t1 = fminf(fminf(tmx.x, tmx.y), tmx.z);
            float tEnd = fminf(t1, tScene);
            ov3 col = o3(0, 0, 0);
            float tr = 1.0f;
            float tS = (P->slice_z - ro.z) / rd.z;
            int sliceHit = P->slice == 1 && tS > t0 && tS < tEnd && P->slice_z < bmax.z;
            ov3 sun = o3(P->sun_dir[0], P->sun_dir[1], P->sun_dir[2]);
            int sliceDone = !sliceHit;
            if (t0 < tEnd) {
                float ds = P->step;
                float jit = ohash2(px + 0.5f, py + 0.5f);
                int n = (int)fminf(600.0f, (tEnd - t0) / ds + 1.0f);
                for (int i = 0; i < n; ++i) {
                    float t = t0 + ((float)i + jit) * ds;
                    if (t > tEnd) break;
                    if (!sliceDone && t >= tS) {
                        oslice(&G, P, ro, rd, tS, &col, &tr);
                        sliceDone = 1;
                    }
                    if (P->smoke == 0 && P->fire == 0) continue;
                    ov3 p = oadd(ro, omul(rd, t));
                    float v[4];
                    osample(&G, p, v);
                    float soot = fmaxf(v[0], 0.0f), aero = fmaxf(v[1], 0.0f);
                    float sigma0 = (8700.0f * soot + 3000.0f * aero) * P->smoke_scale;
                    float sigma = sigma0, a = 0.0f;
                    float lightFrac = aero / (soot * 3.0f + aero + 1e-12f);
                    ov3 scat = o3(0, 0, 0);
                    if (P->smoke == 1 && sigma0 > 0.02f) {
                        float bill = osmoke_noise(p, P->time);
                        sigma = sigma0 * omix(0.25f, 1.75f, bill);
                        a = 1.0f - expf(-sigma * ds);
                        float od = 0.0f;
                        for (int sh = 1; sh <= 4; ++sh) {
                            float sv2[4];
                            osample(&G, oadd(p, omul(sun, 0.35f * (float)sh)), sv2);
                            od += (8700.0f * fmaxf(sv2[0], 0.0f) + 3000.0f * fmaxf(sv2[1], 0.0f)) * P->smoke_scale * 0.35f;
                        }
                        float sunT = expf(-od);
                        float g = 0.35f, ct = odot(rd, sun);
                        float hg = (1.0f - g * g) / powf(1.0f + g * g - 2.0f * g * ct, 1.5f) * 0.25f;
                        ov3 albedo = omix3(o3(0.10f, 0.095f, 0.09f), o3(0.86f, 0.84f, 0.78f), lightFrac);
                        float amb = 0.45f + 0.25f * oclamp((p.z - G.bmin.z) * 0.15f, 0.0f, 1.0f);
                        scat = omul(albedo, amb * omix(0.55f, 1.0f, sunT) + 1.6f * hg * sunT);
                        scat = omul(scat, omix(0.85f, 1.1f, bill));
                    }
                    if (P->fire == 1) {
                        float alb = omix(0.45f, 0.95f, lightFrac);
                        float fl = 0.0f;
                        for (int li = 0; li < P->n_lights; ++li) {
                            ov3 dl = osub(o3(P->lights[li][0], P->lights[li][1], P->lights[li][2]), p);
                            fl += P->lights[li][3] / (0.6f + odot(dl, dl));
                        }
                        scat = oadd(scat, omul(omul(omul(o3(1.0f, 0.45f, 0.15f), fl), alb), 0.9f));
                    }
                    ov3 emit = o3(0, 0, 0);
                    if (P->fire == 1) {
                        float q = v[3] / 1.0e6f;
                        float hot = osmooth(1000.0f, 1600.0f, v[2]);
                        float drive = oclamp(q * 0.9f, 0.0f, 3.0f) + hot * 0.9f;
                        if (drive > 0.01f) {
                            float nn = oflame_noise(p, P->time);
                            float shape = osmooth(0.62f - 0.25f * oclamp(drive, 0.0f, 1.5f), 0.85f, nn + 0.15f * fminf(drive, 1.5f));
                            float k = oclamp(0.25f * drive + 0.6f * nn * shape, 0.0f, 1.0f);
                            emit = omul(omul(omul(oflame_color(k), shape), drive), 6.0f);
                        }
                        emit = oadd(emit, omul(omul(oglow(v[2]), oclamp(sigma * 0.6f, 0.0f, 1.0f)), 4.0f));
                    }
                    col = oadd(col, omul(oadd(omul(scat, a), omul(emit, ds)), tr));
                    tr *= 1.0f - a;
                    if (tr < 0.004f) break;
                }
                if (!sliceDone) oslice(&G, P, ro, rd, tS, &col, &tr);
            }
            float* o = rgb + 3 * ((size_t)py * P->width + px);
            o[0] = base.x * tr + (1.0f - expf(-col.x * 1.1f));
            o[1] = base.y * tr + (1.0f - expf(-col.y * 1.1f));
            o[2] = base.z * tr + (1.0f - expf(-col.z * 1.1f));
        }
}
