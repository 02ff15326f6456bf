// CUDA kernels of the gas-phase step (all stages except the pressure solve).
//
// Each kernel is one pass of the reference's step over one domain of every
// scenario in a launch; the arithmetic of every cell or face restates the
// reference expression in its own evaluation order (the FP64 build is compiled
// with --fmad=false so no multiply-add is fused), which keeps the FP64 path
// within rounding of the reference's own FP64 step. Reductions that the
// reference sums in a fixed order are summed here in a fixed order as well:
// per-CTA partials, then the last CTA of a scenario sums the partials in CTA
// order, so results do not depend on scheduling.
#pragma once
#include "phx_dev.cuh"

namespace phx {

#define PHX_PROLOGUE(dom)                 \
    int s_, tile_;                        \
    locate(dom, blockIdx.x, s_, tile_);   \
    const Scn<R>& g = S[s_];

// (i, j, k) of element f of a layout: kind 0 cells and z-faces, 1 x-faces, 2 y-faces
template <class R>
__device__ __forceinline__ void ijkOf(const Scn<R>& g, int kind, int f, int& i, int& j, int& k) {
    const unsigned q = divU((unsigned)f, g.dvA[kind]);
    k = (int)divU((unsigned)f, g.dvB[kind]);
    i = f - (int)(q * g.dvA[kind].d);
    j = (int)q - k * g.dY[kind];
}
// the layout kind of the faces normal to axis a
__device__ __forceinline__ int faceKind(int a) { return a == 0 ? 1 : a == 1 ? 2 : 0; }

// ambient value of transported scalar q (the value outside the domain):
// T (stored), O2, CO2 and H2O; zero for the others
template <class T>
__device__ __forceinline__ T ambOf(int q) {
    return q == 0 ? tAmbient<T>() : q == 1 ? T(K_YO2_AMB) : q == 6 ? T(K_YCO2_AMB) : q == 7 ? T(K_YH2O_AMB) : T(0);
}

template <class R>
__device__ __forceinline__ double gasDensity(const Scn<R>& g, int c) {
    const double t = tempIsOffset<R>() ? K_T0 + (double)g.sc[0][c] : (double)g.sc[0][c];
    return (double)g.Pb[c] / (K_RS * t);
}

// ---------------------------------------------------------------------------
// Last-CTA reduction: every CTA of a scenario sums its threads' values (fixed
// order) and stores the partial; the CTA that finishes last sums the partials
// in CTA order. Every thread of the CTA must call it. Returns true in every
// thread of the last CTA, with the total in *total (thread 0).
template <class R, class V>
__device__ bool lastCtaSum(const Scn<R>& g, int slot, int tile, int ntiles, V vThread, double* total) {
    __shared__ double sh[32];
    __shared__ int amLast;
    double v = blockSum(vThread, sh);
    double* part = g.part + (size_t)slot * g.partStride;
    if (threadIdx.x == 0) {
        part[tile] = v;
        __threadfence();
        unsigned t = atomicAdd(g.cnt + slot, 1u);
        amLast = (t == (unsigned)ntiles - 1u);
    }
    __syncthreads();
    if (!amLast) return false;
    __threadfence();
    double acc = 0;
    for (int i = threadIdx.x; i < ntiles; i += blockDim.x) acc += __ldcg(part + i);
    double tot = blockSum(acc, sh);
    if (threadIdx.x == 0) {
        *total = tot;
        g.cnt[slot] = 0;
    }
    return true;
}

__device__ __forceinline__ int ntilesOf(const Dom& d, int s) { return __ldg(d.start + s + 1) - __ldg(d.start + s); }
__device__ __forceinline__ int ntilesOf(const ADom& d, int s) { return d.start[s + 1] - d.start[s]; }

// ---------------------------------------------------------------------------
// Solver::stableDt (src/sim/gasphase.cpp:63-70) and the injection amounts of
// injectIgnitions / injectBurners (src/sim/solver.cpp:271-280,
// src/sim/gasphase.cpp:92-105, Burner::powerAt src/sim/solver.h:122-126).
// One thread per scenario.
template <class R>
__global__ void k_begin(const Scn<R>* __restrict__ S, Dom dom, int computeDt, double dtGiven) {
    PHX_PROLOGUE(dom);
    if (threadIdx.x != 0) return;
    double* sv = g.sv;
    double dt;
    if (computeDt) {
        double dtMax = *g.dtMaxArg;
        dt = mn(dtMax, g.dtMaxP);
        dt = mn(dt, g.cfl * g.dx / mx(sv[SV_MAXVEL], 0.1));
        double alpha = sv[SV_MAXNU] * (1.0 + 1.0 / K_PR_T);
        if (alpha > 0) dt = mn(dt, 0.9 * g.dx * g.dx / (6.0 * alpha));
        if (sv[SV_MAXDIV] > 0) dt = mn(dt, 0.25 / sv[SV_MAXDIV]);
        dt = mx(dt, 1e-3);
    } else {
        dt = dtGiven;
    }
    sv[SV_DT] = dt;
    sv[SV_INV] = g.dx * g.dx / dt;
    double time = sv[SV_TIME];
    double fuelIn = sv[SV_FUELIN];
    for (int q = 0; q < g.nsrc; ++q) {
        const Src& src = g.src[q];
        double mf = -1.0;
        if (src.kind == 0) {
            int c = src.i0 + g.nx * (src.j0 + g.ny * src.k);
            if (!(time < src.start || time > src.start + src.duration) && !g.blocked[c]) {
                mf = src.power * dt / K_DHC_FUEL;
                fuelIn += mf;
            }
        } else {
            double P = 0;
            if (!(time < src.start || time > src.start + src.duration)) {
                double r = src.rampS > 0 ? mn(1.0, (time - src.start) / src.rampS) : 1.0;
                P = src.peakW * r * r;
            }
            if (P > 0) {
                mf = P * dt / K_DHC_FUEL / src.ncells;
                for (int n = 0; n < src.ncells; ++n) fuelIn += mf;
            }
        }
        sv[SV_SRC_MF + q] = mf;
    }
    sv[SV_FUELIN] = fuelIn;
    // reductions of this step start from their neutral values
    sv[SV_MAXNU] = 0;
    sv[SV_MAXDIV] = 0;
    sv[SV_MAXVEL] = 0;
    sv[SV_RMAX] = 0;
    sv[SV_BMAX] = 0;
    sv[SV_MAXGAST] = K_T0;
    sv[SV_BURNING] = 0;
}

// ---------------------------------------------------------------------------
// The stage kernels below compute in their storage type T = R: double for the
// FP64 path (the expressions keep the reference's evaluation order), float for
// the mixed path. Literals are written T(...) so the float path stays in FP32.

// gas density P / (R T) of a cell in the arithmetic type
template <class R>
__device__ __forceinline__ R rhoOf(const Scn<R>& g, int c) {
    return g.Pb[c] / (R(K_RS) * tAbs(g.sc[0][c]));
}

// Per-step clears (src/sim/solver.cpp:231-233), injectIgnitions + injectBurners
// through addGasSpecies (src/sim/solver.cpp:212-223), and combustion
// (src/sim/solver.cpp:284-344). lit is double-buffered: neighbours read the
// previous step's flags from lit, the new flags go to lit2.
template <class R>
__global__ void k_combust(const Scn<R>* __restrict__ S, Dom dom) {
    using T = R;
    PHX_PROLOGUE(dom);
    int c = tile_ * TPB + threadIdx.x;
    if (c >= g.N) return;
    const double* sv = g.sv;
    const T dt = (T)sv[SV_DT];
    const T dx = (T)g.dx;
    const int nx = g.nx, ny = g.ny, nz = g.nz, sz = nx * ny;
    T Qc = 0, Qrc = 0, hrrc = 0, ms = 0;
    uint8_t pil = 0, litn = 0;
    if (!g.blocked[c]) {
        int i, j, k;
        ijkOf(g, 0, c, i, j, k);
        R* const* Y = g.sc;
        T Tc = tAbs(Y[0][c]);
        T yf = Y[2][c];
        bool member = false;
        for (int q = 0; q < g.nsrc; ++q) {
            const Src& sr = g.src[q];
            if (sv[SV_SRC_MF + q] >= 0 && k == sr.k && i >= sr.i0 && i <= sr.i1 && j >= sr.j0 && j <= sr.j1) member = true;
        }
        if (member || yf >= T(1e-6)) {
            T Yo = Y[1][c], Ys = Y[3][c], Ya = Y[4][c], Yp = Y[5][c], Yc = Y[6][c], Yw = Y[7][c], Yco = Y[8][c],
              Yai = Y[9][c];
            bool modified = false;
            if (member) {
                const T m = rhoOf(g, c) * dx * dx * dx;
                for (int q = 0; q < g.nsrc; ++q) {
                    const Src& sr = g.src[q];
                    const double mfd = sv[SV_SRC_MF + q];
                    if (!(mfd >= 0 && k == sr.k && i >= sr.i0 && i <= sr.i1 && j >= sr.j0 && j <= sr.j1)) continue;
                    const T mf = (T)mfd;
                    const T fuelGen = mf, aerosol = T(0), sootPot = mf * T(K_BURNER_SOOT);
                    const T madd = fuelGen + aerosol;
                    if (madd <= T(0)) continue;
                    const T mt = m + madd, scl = m / mt;
                    Yo *= scl; Ys *= scl; Yc *= scl; Yw *= scl; Yco *= scl;
                    Yai = Yai * scl + fuelGen * T(K_T_AUTO) / mt;
                    yf = yf * scl + fuelGen / mt;
                    Ya = Ya * scl + aerosol / mt;
                    Yp = Yp * scl + sootPot / mt;
                    ms += madd;
                    pil = 1;
                    modified = true;
                }
            }
            if (yf >= T(1e-6)) {
                const T V = dx * dx * dx;
                const T frac = T(1) - exp(-dt / T(K_TAU_MIX));
                const T chiR = g.radiationOn ? T(K_CHI_R) : T(0);
                T ait = yf > T(1e-9) ? Yai / yf : T(K_T_AUTO);
                bool ign = pil || Tc > ait;
                if (!ign) {
                    const uint8_t* lit = g.lit;
                    ign = (i > 0 && lit[c - 1]) || (i < nx - 1 && lit[c + 1]) || (j > 0 && lit[c - nx]) ||
                          (j < ny - 1 && lit[c + nx]) || (k > 0 && lit[c - sz]) || (k < nz - 1 && lit[c + sz]);
                }
                if (ign) {
                    T burnable = mn(yf, Yo / T(K_S_O2));
                    if (burnable > T(1e-7)) {
                        T tAd = Tc + T(K_DHC_FUEL) / (T(K_CP) * (T(1) + T(K_S_O2) / mx(Yo, T(1e-4))));
                        if (pil || !(tAd < T(K_T_CRIT))) {
                            T m = rhoOf(g, c) * V;
                            T dmf = burnable * m * frac;
                            T q = dmf * T(K_DHC_FUEL);
                            T sootMade = yf > T(0) ? Yp * (dmf / m) / yf : T(0);
                            T coMade = T(K_CO_YIELD) * dmf / m;
                            T co2Made = mx(T(0), (T(K_C_FRAC) * dmf / m - sootMade - T(12.0 / 28.0) * coMade) * T(44.0 / 12.0));
                            T o2Used = T(K_S_O2) * dmf / m - T(32.0 / 12.0) * sootMade - T(16.0 / 28.0) * coMade;
                            yf = mx(T(0), yf - dmf / m);
                            Yai = yf * ait;
                            Yo = mx(T(0), Yo - o2Used);
                            Yp = mx(T(0), Yp - sootMade);
                            Ys += sootMade;
                            Yco += coMade;
                            Yc += co2Made;
                            Yw += T(K_Y_H2O) * dmf / m;
                            Ya *= (T(1) - frac);
                            Qc = q * (T(1) - chiR);
                            Qrc = q * chiR;
                            hrrc = q / (dt * V);
                            litn = q > T(1e-3) ? 1 : 0;
                            modified = true;
                        }
                    }
                }
            }
            if (modified) {
                Y[1][c] = Yo; Y[2][c] = yf; Y[3][c] = Ys; Y[4][c] = Ya; Y[5][c] = Yp;
                Y[6][c] = Yc; Y[7][c] = Yw; Y[8][c] = Yco; Y[9][c] = Yai;
            }
        }
    }
    g.Q[c] = Qc;
    g.Qr[c] = Qrc;
    g.hrr[c] = hrrc;
    g.massSrc[c] = ms;
    g.pilot[c] = pil;
    g.lit2[c] = litn;
}

// ---------------------------------------------------------------------------
// Solver::turbulence (src/sim/gasphase.cpp:163-218): cell-centre velocities,
// the blocked-aware 1-2-1 test filter x -> y -> z per component, and the
// Deardorff viscosity.
template <class R>
__global__ void k_turb_center(const Scn<R>* __restrict__ S, Dom dom) {
    using T = R;
    PHX_PROLOGUE(dom);
    int c = tile_ * TPB + threadIdx.x;
    if (c >= g.N) return;
    R *uc = g.tmp[0], *vc = g.tmp[1], *wc = g.tmp[2];
    if (g.blocked[c]) { uc[c] = vc[c] = wc[c] = 0; return; }
    const int nx = g.nx, ny = g.ny;
    int i, j, k;
    ijkOf(g, 0, c, i, j, k);
    int fx0 = i + (nx + 1) * (j + ny * k);
    int fy0 = i + nx * (j + (ny + 1) * k);
    uc[c] = T(0.5) * (g.u[fx0] + g.u[fx0 + 1]);
    vc[c] = T(0.5) * (g.v[fy0] + g.v[fy0 + nx]);
    wc[c] = T(0.5) * (g.w[c] + g.w[c + nx * ny]);
}

// one pass of the test filter along AXIS for the three velocity components
// (the reference filters each component x -> y -> z; the components are
// independent, so one launch per axis covers all three)
template <class R, int AXIS>
__global__ void k_turb_filter(const Scn<R>* __restrict__ S, Dom dom) {
    using T = R;
    PHX_PROLOGUE(dom);
    int c = tile_ * TPB + threadIdx.x;
    if (c >= g.N) return;
    if (g.blocked[c]) {
#pragma unroll
        for (int q = 0; q < 3; ++q) (AXIS == 1 ? g.tmp[6 + q] : g.tmp[3 + q])[c] = 0;
        return;
    }
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    int i, j, k;
    ijkOf(g, 0, c, i, j, k);
    const int id = AXIS == 0 ? i : AXIS == 1 ? j : k, n = AXIS == 0 ? nx : AXIS == 1 ? ny : nz;
    const int st = AXIS == 0 ? 1 : AXIS == 1 ? nx : nx * ny;
    // neighbours at clamped indices, loaded together with their solid flags and
    // used through selects
    const int cLo = id > 0 ? c - st : c, cHi = id < n - 1 ? c + st : c;
    const bool hasLo = id > 0 && !g.blocked[cLo], hasHi = id < n - 1 && !g.blocked[cHi];
    T self[3], lov[3], hiv[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        const R* in = AXIS == 0 ? g.tmp[q] : AXIS == 1 ? g.tmp[3 + q] : g.tmp[6 + q];
        self[q] = in[c];
        lov[q] = in[cLo];
        hiv[q] = in[cHi];
    }
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        R* out = AXIS == 1 ? g.tmp[6 + q] : g.tmp[3 + q];
        const T lo = hasLo ? lov[q] : self[q];
        const T hi = hasHi ? hiv[q] : self[q];
        out[c] = T(0.25) * lo + T(0.5) * self[q] + T(0.25) * hi;
    }
}

template <class R>
__global__ void k_turb_nu(const Scn<R>* __restrict__ S, Dom dom) {
    using T = R;
    PHX_PROLOGUE(dom);
    int c = tile_ * TPB + threadIdx.x;
    T m = 0;   // the max is taken in the arithmetic type: no FP64 instruction per cell on the mixed path
    if (c < g.N) {
        if (g.blocked[c]) g.nu[c] = 0;
        else {
            T du = g.tmp[0][c] - g.tmp[3][c];
            T dv = g.tmp[1][c] - g.tmp[4][c];
            T dw = g.tmp[2][c] - g.tmp[5][c];
            T ks = T(0.5) * (du * du + dv * dv + dw * dw);
            T nu = mn(T(1), T(K_C_NU) * (T)g.dx * sqrt(ks) + T(1.5e-5) * pow(tAbs(g.sc[0][c]) / T(293.15), T(1.7)));
            g.nu[c] = nu;
            m = nu;
        }
    }
    blockMaxTo(g.sv + SV_MAXNU, m);
}

// ---------------------------------------------------------------------------
// Solver::heatDiffusion (src/sim/gasphase.cpp:221-248)
// FP64 path: the conductive flux of every interior face between two gas cells,
// fo kf dx (T_upper - T_lower), once per face into the transport's record
// scratch (free at this point of the step). kf is symmetric in the two cells
// (the sums commute in IEEE arithmetic), and the lower cell's term is the
// exact negation of the upper cell's, so k_heat's sums are unchanged.
template <class R>
__global__ void k_heat_faces(const Scn<R>* __restrict__ S, Dom dom, int axis) {
    using T = R;
    PHX_PROLOGUE(dom);
    const int f = tile_ * TPB + threadIdx.x;
    const int nx = g.nx, ny = g.ny, nz = g.nz, sxy = nx * ny;
    const int nfa = axis == 0 ? g.NX : axis == 1 ? g.NY : g.NZ;
    if (!g.adv || f >= nfa) return;
    int i, j, k, id, dim, st;
    ijkOf(g, faceKind(axis), f, i, j, k);
    if (axis == 0) { id = i; dim = nx; st = 1; }
    else if (axis == 1) { id = j; dim = ny; st = nx; }
    else { id = k; dim = nz; st = sxy; }
    if (id < 1 || id > dim - 1) return;
    const int U = i + nx * (j + ny * k), L = U - st;
    const T fo = axis == 0 ? g.fx[f] : axis == 1 ? g.fy[f] : g.fz[f];
    if (fo <= T(0) || g.blocked[L] || g.blocked[U]) return;
    const R* Tf = g.sc[0];
    const T dx = (T)g.dx;
    // from the lower cell's side, as k_heat evaluates it (src/sim/gasphase.cpp:230-243)
    const T Tc = Tf[L], Tn = Tf[U], nuc = g.nu[L], nun = g.nu[U];
    const T rc = rhoOf(g, L), rn = rhoOf(g, U);
    const T Tface = T(0.5) * (Tc + Tn);
    const T kf = T(0.5) * (rc + rn) * T(K_CP) * T(0.5) * (nuc + nun) / T(K_PR_T) + T(0.0258) * pow(Tface / T(293.15), T(0.8));
    g.adv[(axis == 0 ? 0 : axis == 1 ? g.NX : g.NX + g.NY) + f] = (double)(fo * kf * dx * (Tn - Tc));
}

template <class R>
__global__ void k_heat(const Scn<R>* __restrict__ S, Dom dom) {
    using T = R;
    PHX_PROLOGUE(dom);
    int c = tile_ * TPB + threadIdx.x;
    if (c >= g.N || g.blocked[c]) return;
    const int nx = g.nx, ny = g.ny, nz = g.nz, sxy = nx * ny;
    int i, j, k;
    ijkOf(g, 0, c, i, j, k);
    const int fx0 = i + (nx + 1) * (j + ny * k), fy0 = i + nx * (j + (ny + 1) * k);
    const T fo[6] = {g.fx[fx0], g.fx[fx0 + 1], g.fy[fy0], g.fy[fy0 + nx], g.fz[c], g.fz[c + sxy]};
    const int nb[6] = {i > 0 ? c - 1 : -1, i < nx - 1 ? c + 1 : -1, j > 0 ? c - nx : -1, j < ny - 1 ? c + nx : -1,
                       k > 0 ? c - sxy : -1, k < nz - 1 ? c + sxy : -1};
    const R* Tf = g.sc[0];
    const T dx = (T)g.dx;
    const T Tc = Tf[c], nuc = g.nu[c];
    T rc = rhoOf(g, c), q = 0;
    const double* hf = std::is_same<T, float>::value ? nullptr : g.adv;   // FP64: fluxes from k_heat_faces
    const int fgl[6] = {fx0, fx0 + 1, g.NX + fy0, g.NX + fy0 + nx, g.NX + g.NY + c, g.NX + g.NY + c + sxy};
    for (int d = 0; d < 6; ++d) {
        if (fo[d] <= T(0)) continue;
        int n = nb[d];
        if (n >= 0 && g.blocked[n]) continue;
        if (hf && n >= 0) {
            const T F = (T)hf[fgl[d]];
            q += (d & 1) ? F : -F;   // the cell is the face's lower cell for d odd
            continue;
        }
        T Tn = n >= 0 ? Tf[n] : tAmbient<T>();
        T nun = n >= 0 ? g.nu[n] : nuc;
        T rn = n >= 0 ? rhoOf(g, n) : T(K_P0) / (T(K_RS) * T(K_T0));
        T Tface = tAbs(T(0.5) * (Tc + Tn));
        T kf = T(0.5) * (rc + rn) * T(K_CP) * T(0.5) * (nuc + nun) / T(K_PR_T) + T(0.0258) * pow(Tface / T(293.15), T(0.8));
        q += fo[d] * kf * dx * (Tn - Tc);
    }
    g.Q[c] = g.Q[c] + q * (T)g.sv[SV_DT];
}

// Solver::energyAndExpansion (src/sim/gasphase.cpp:251-271)
template <class R>
__global__ void k_energy(const Scn<R>* __restrict__ S, Dom dom) {
    using T = R;
    PHX_PROLOGUE(dom);
    int c = tile_ * TPB + threadIdx.x;
    T md = 0;
    if (c < g.N) {
        if (g.blocked[c]) g.S[c] = 0;
        else {
            const T dt = (T)g.sv[SV_DT];
            const T dx = (T)g.dx;
            const T V = dx * dx * dx;
            const T Ts = g.sc[0][c], Q = g.Q[c], Pb = g.Pb[c];
            const T Tc = tAbs(Ts);
            T rho = Pb / (T(K_RS) * Tc);
            T m = rho * V;
            // the clamp to [T_MIN, T_MAX] on the stored value (the offset on the mixed path)
            T Tns = clampd(Ts + Q / (m * T(K_CP)), T(tStoredFromKd<T>(K_T_MIN)), T(tStoredFromKd<T>(K_T_MAX)));
            T rhoN = Pb / (T(K_RS) * tAbs(Tns));
            T D = Q / (m * T(K_CP) * Tc * dt) + g.massSrc[c] / (rhoN * V * dt);
            g.sc[0][c] = Tns;
            T Sv = clampd(D, -T(K_D_MAX), T(K_D_MAX));
            g.S[c] = Sv;
            md = fabs(Sv);
        }
    }
    blockMaxTo(g.sv + SV_MAXDIV, md);
}

// ---------------------------------------------------------------------------
// Solver::momentum (src/sim/gasphase.cpp:275-372): one component on its faces,
// written to the second velocity buffer.
template <class T>
__device__ __forceinline__ T vanLeer(T a, T b) { return a * b > T(0) ? T(2) * a * b / (a + b) : T(0); }

template <class R, int COMP>
__global__ void k_momentum(const Scn<R>* __restrict__ S, Dom dom) {
    using T = R;
    constexpr int comp = COMP;   // the face component: compile-time, so the per-axis arrays stay in registers
    PHX_PROLOGUE(dom);
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const int dX = nx + (comp == 0), dY = ny + (comp == 1), dZ = nz + (comp == 2);
    const int nf = dX * dY * dZ;
    int f = tile_ * TPB + threadIdx.x;
    if (f >= nf) return;
    const R* vel = comp == 0 ? g.u : comp == 1 ? g.v : g.w;
    const R* fo = comp == 0 ? g.fx : comp == 1 ? g.fy : g.fz;
    const uint8_t* lk = comp == 0 ? g.lx : comp == 1 ? g.ly : g.lz;   // null: no crack faces
    R* out = comp == 0 ? g.u2 : comp == 1 ? g.v2 : g.w2;
    if (fo[f] <= T(0)) { out[f] = 0; return; }
    if (lk && lk[f]) { out[f] = vel[f]; return; }   // set by leakage()
    int i, j, k;
    ijkOf(g, faceKind(comp), f, i, j, k);
    const int id[3] = {i, j, k};
    const int ncell[3] = {nx, ny, nz};
    const int st[3] = {1, dX, dX * dY};
    const int dim[3] = {dX, dY, dZ};
    const int lo = id[comp] - 1;
    const bool bnd = lo < 0 || id[comp] >= ncell[comp];
    if (bnd) {
        const double zc = g.oz + (comp == 2 ? (double)k : k + 0.5) * g.dx;
        double wv = windAt(g, comp, lo < 0 ? 0 : 1, zc);
        out[f] = isnan(wv) ? vel[f] : (R)wv;
        return;
    }
    int a3[3] = {i, j, k};
    a3[comp] -= 1;
    const int ca = a3[0] + nx * (a3[1] + ny * a3[2]);
    const int cb = i + nx * (j + ny * k);
    const T v0 = vel[f];
    T adv[3];
    adv[comp] = v0;
    for (int a = 0; a < 3; ++a) {
        if (a == comp) continue;
        const R* va = a == 0 ? g.u : a == 1 ? g.v : g.w;
        const int aX = nx + (a == 0), aY = ny + (a == 1);
        T s = 0;
        for (int q = 0; q < 4; ++q) {
            int p[3] = {i, j, k};
            if (q & 1) p[a] += 1;
            if (q & 2) p[comp] -= 1;
            p[a] = p[a] < ncell[a] ? p[a] : ncell[a];
            p[comp] = p[comp] > 0 ? p[comp] : 0;
            s += va[p[0] + aX * (p[1] + aY * p[2])];
        }
        adv[a] = T(0.25) * s;
    }
    const T idx = g.rdx, idx2 = g.rdx2;   // 1 / dx and 1 / (dx dx) in R, from the host
    T acc = 0, lap = 0;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        // free slip across closed faces: neighbour along a, then the second
        // neighbour only through two open faces. Every load is issued up front
        // (indices clamped into the face grid, used only through the selects
        // below), so a face's loads are in flight together.
        const bool hm1 = id[a] >= 1, hp1 = id[a] + 1 < dim[a], hm2 = id[a] >= 2, hp2 = id[a] + 2 < dim[a];
        const int im1 = hm1 ? f - st[a] : f, ip1 = hp1 ? f + st[a] : f;
        const int im2 = hm2 ? f - 2 * st[a] : f, ip2 = hp2 ? f + 2 * st[a] : f;
        const T om1 = fo[im1], op1 = fo[ip1], om2 = fo[im2], op2 = fo[ip2];
        const T vm1 = vel[im1], vp1 = vel[ip1], vm2 = vel[im2], vp2 = vel[ip2];
        bool cm1 = false, cp1 = false, cm2 = false, cp2 = false;   // crack faces
        if (lk) {
            cm1 = lk[im1] != 0;
            cp1 = lk[ip1] != 0;
            cm2 = lk[im2] != 0;
            cp2 = lk[ip2] != 0;
        }
        const T m1 = hm1 && om1 > T(0) && !cm1 ? vm1 : v0;
        const T p1 = hp1 && op1 > T(0) && !cp1 ? vp1 : v0;
        const T m2 = hm2 && om2 > T(0) && om1 > T(0) && !(cm2 || cm1) ? vm2 : m1;
        const T p2 = hp2 && op2 > T(0) && op1 > T(0) && !(cp2 || cp1) ? vp2 : p1;
        // the upwind-biased face values, the limiter arguments chosen by the
        // sign of the advecting velocity (two van Leer evaluations, no branch)
        const bool pos = adv[a] >= T(0);
        const T vlA = vanLeer(v0 - m1, p1 - v0);
        const T vlB = vanLeer(pos ? m1 - m2 : p1 - v0, pos ? v0 - m1 : p2 - p1);
        const T fp = pos ? v0 + T(0.5) * vlA : p1 - T(0.5) * vlB;
        const T fm = pos ? m1 + T(0.5) * vlB : v0 - T(0.5) * vlA;
        acc -= adv[a] * (fp - fm) * idx;
        lap += (m1 - T(2) * v0 + p1) * idx2;
    }
    T ra = rhoOf(g, ca), rb = rhoOf(g, cb);
    T rf = T(0.5) * (ra + rb);
    T nuf = T(0.5) * (g.nu[ca] + g.nu[cb]);
    acc += nuf * lap;
    T pt;
    if constexpr (tempIsOffset<T>()) {
        // The same terms from the temperature offsets th = T - T0, free of the
        // cancellation of two near-equal FP32 densities:
        //   r0 - rf = 0.5 (Pa / (R T0) - ra + Pb / (R T0) - rb) = 0.5 (ra th_a + rb th_b) / T0
        //   1 / rb - 1 / ra = R (Tb / Pb - Ta / Pa) = R (T0 (1 / Pb - 1 / Pa) + th_b / Pb - th_a / Pa)
        const T tha = g.sc[0][ca], thb = g.sc[0][cb];
        if (comp == 2) acc += T(K_G) * (T(0.5) * (ra * tha + rb * thb) / T(K_T0)) / rf;
        pt = rf * T(0.5) * (g.p[ca] + g.p[cb]);
        const T ipa = T(1) / g.Pb[ca], ipb = T(1) / g.Pb[cb];
        acc += pt * (T(K_RS) * (T(K_T0) * (ipb - ipa) + (thb * ipb - tha * ipa))) * idx;
    } else {
        if (comp == 2) {
            T r0 = T(0.5) * (g.Pb[ca] + g.Pb[cb]) / (T(K_RS) * T(K_T0));
            acc += T(K_G) * (r0 - rf) / rf;
        }
        pt = rf * T(0.5) * (g.p[ca] + g.p[cb]);
        acc += pt * (T(1) / rb - T(1) / ra) * idx;
    }
    out[f] = clampd(v0 + (T)g.sv[SV_DT] * acc, -T(K_VMAX), T(K_VMAX));
}

// open boundary faces without wind inflow take the new value of the face one
// cell inside (src/sim/gasphase.cpp:374-393). One thread per boundary face.
template <class R>
__global__ void k_mom_bnd(const Scn<R>* __restrict__ S, Dom dom, int comp) {
    PHX_PROLOGUE(dom);
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const int dX = nx + (comp == 0), dY = ny + (comp == 1), dZ = nz + (comp == 2);
    const int dim[3] = {dX, dY, dZ};
    const int st[3] = {1, dX, dX * dY};
    const int nAx = comp == 0 ? nx : comp == 1 ? ny : nz;
    const int nA = dim[(comp + 1) % 3], nB = dim[(comp + 2) % 3];
    const int sides = comp == 2 ? 1 : 2;
    int t = tile_ * TPB + threadIdx.x;
    if (t >= nA * nB * sides) return;
    int side = comp == 2 ? 1 : t % 2;
    int ab = comp == 2 ? t : t / 2;
    int a2 = ab % nA, b2 = ab / nA;
    int id[3];
    id[comp] = side == 0 ? 0 : nAx;
    id[(comp + 1) % 3] = a2;
    id[(comp + 2) % 3] = b2;
    int f = id[0] + dX * (id[1] + dY * id[2]);
    const R* fo = comp == 0 ? g.fx : comp == 1 ? g.fy : g.fz;
    const uint8_t* lk = comp == 0 ? g.lx : comp == 1 ? g.ly : g.lz;
    R* out = comp == 0 ? g.u2 : comp == 1 ? g.v2 : g.w2;
    if (fo[f] <= R(0) || (lk && lk[f])) return;
    double zc = g.oz + (comp == 2 ? (double)id[2] : id[2] + 0.5) * g.dx;
    if (!isnan(windAt(g, comp, side, zc))) return;
    int gg = f + (side == 0 ? 1 : -1) * st[comp];
    out[f] = fo[gg] > R(0) && !(lk && lk[gg]) ? out[gg] : (R)0;
}

// ---------------------------------------------------------------------------
// Solver::leakage (src/sim/gasphase.cpp:403-499). k_zone_integral: per closed
// zone (one CTA each) the integral of S and, with crack faces, the implicit
// end-of-step zone pressure by the reference's 40-step bisection of the
// zone's mass balance against the orifice flow through its leak faces (each
// evaluation sums the zone's faces with a fixed-order CTA reduction).
// k_leak_faces: the relaxed orifice velocity of every leak face and its volume
// flow. k_leak_finish: per closed zone the pressure-rise rate and the
// divergence shift. FP64 arithmetic in either path (a few hundred faces).
constexpr double K_CD_LEAK = 1.0, K_LEAK_VMAX = 40.0;

__device__ __forceinline__ double leakFlow(double dp, double rhoUp) {   // m/s, positive a -> b
    const double sgn = dp >= 0 ? 1.0 : -1.0;
    return sgn * mn(K_LEAK_VMAX, K_CD_LEAK * sqrt(2.0 * fabs(dp) / mx(rhoUp, 0.05)));
}
template <class R>
__device__ __forceinline__ double leakOpenFrac(const Scn<R>& g, const int4& lf) {
    return (double)(lf.x == 0 ? g.fx : lf.x == 1 ? g.fy : g.fz)[lf.y];
}

template <class R>
__global__ void k_zone_integral(const Scn<R>* __restrict__ S, Dom dom) {
    PHX_PROLOGUE(dom);
    __shared__ double sh[32];
    __shared__ double bcast;
    const int zi = tile_;
    const int z = g.closedZone[zi];
    const double V = g.dx * g.dx * g.dx;
    double acc = 0;
    for (int e = g.closedStart[zi] + threadIdx.x; e < g.closedStart[zi + 1]; e += blockDim.x) {
        int c = g.closedCells[e];
        acc += (double)g.S[c] * V;
    }
    double dInt = blockSum(acc, sh);
    if (threadIdx.x == 0) bcast = dInt;
    __syncthreads();
    dInt = bcast;
    const double Vz = g.zoneVol[z];
    if (g.nLeak == 0) {
        if (threadIdx.x == 0) {
            double out = 0.0;
            g.zoneDP[z] = K_GAMMA * g.zoneP[z] * (double)(dInt - out) / Vz;
            g.zoneShift[z] = (double)(dInt - out) / Vz;
        }
        return;
    }
    const double P = g.zoneP[z], dt = g.sv[SV_DT], A = g.dx * g.dx;
    const int e0 = g.leakZStart[z], e1 = g.leakZStart[z + 1];
    // residual of the zone's mass balance at trial pressure Pt (every thread)
    auto resid = [&](double Pt) {
        double acc2 = 0;
        for (int e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
            const int4 lf = g.leak[g.leakZList[e]];
            const bool zIsA = lf.z >= 0 && g.zone[lf.z] == z;
            const int other = zIsA ? lf.w : lf.z;
            const double Po = other >= 0 && g.zone[other] >= 0 ? g.zoneP[g.zone[other]] : K_P0;
            const double dp = Pt - Po;
            const int up = dp >= 0 ? (zIsA ? lf.z : lf.w) : other;
            const double rho = up >= 0 ? gasDensity(g, up) : K_P0 / (K_RS * K_T0);
            acc2 += leakOpenFrac(g, lf) * A * fabs(leakFlow(dp, rho)) * (dp >= 0 ? 1 : -1);
        }
        const double out = blockSum(acc2, sh);
        __syncthreads();
        if (threadIdx.x == 0) bcast = out;
        __syncthreads();
        return Pt - P - dt * K_GAMMA * P / Vz * (double)(dInt - bcast);
    };
    double lo = P - 20000.0, hi = P + 20000.0, Pnew;
    const double rlo = resid(lo), rhi = resid(hi);
    if (rlo > 0 || rhi < 0) {
        Pnew = P;
    } else {
        for (int it = 0; it < 40; ++it) {
            const double mid = 0.5 * (lo + hi);
            if (resid(mid) > 0) hi = mid; else lo = mid;
        }
        Pnew = 0.5 * (lo + hi);
    }
    if (threadIdx.x == 0) {
        g.zonePnew[z] = Pnew;
        g.zoneDInt[z] = dInt;
    }
}

// one thread per leak face (src/sim/gasphase.cpp:475-486)
template <class R>
__global__ void k_leak_faces(const Scn<R>* __restrict__ S, Dom dom) {
    PHX_PROLOGUE(dom);
    const int q = tile_ * TPB + threadIdx.x;
    if (q >= g.nLeak) return;
    const int4 lf = g.leak[q];
    auto Pz = [&](int c) -> double {
        if (c < 0 || g.zone[c] < 0) return K_P0;
        const int zc = g.zone[c];
        return g.zoneOpen[zc] ? g.zoneP[zc] : g.zonePnew[zc];
    };
    const double rho0 = K_P0 / (K_RS * K_T0);
    const double pa = Pz(lf.z), pb = Pz(lf.w);
    const double ra = lf.z >= 0 ? gasDensity(g, lf.z) : rho0, rb = lf.w >= 0 ? gasDensity(g, lf.w) : rho0;
    const double Ha = lf.z >= 0 ? (double)g.p[lf.z] : 0, Hb = lf.w >= 0 ? (double)g.p[lf.w] : 0;
    const double dp = (pa - pb) + 0.5 * (ra + rb) * (Ha - Hb);
    const double un = leakFlow(dp, dp >= 0 ? ra : rb);
    R* vel = lf.x == 0 ? g.u : lf.x == 1 ? g.v : g.w;
    vel[lf.y] = (R)(0.5 * ((double)vel[lf.y] + un));
    g.leakQ[q] = leakOpenFrac(g, lf) * (g.dx * g.dx) * (double)vel[lf.y];
}

// per closed zone: the net flow out through its leak faces, the zone's
// pressure-rise rate and the divergence shift (src/sim/gasphase.cpp:484-498)
template <class R>
__global__ void k_leak_finish(const Scn<R>* __restrict__ S, Dom dom) {
    PHX_PROLOGUE(dom);
    __shared__ double sh[32];
    const int z = g.closedZone[tile_];
    double acc = 0;
    for (int e = g.leakZStart[z] + threadIdx.x; e < g.leakZStart[z + 1]; e += blockDim.x) {
        const int q = g.leakZList[e];
        const int4 lf = g.leak[q];
        const bool zIsA = lf.z >= 0 && g.zone[lf.z] == z;
        acc += zIsA ? g.leakQ[q] : -g.leakQ[q];
    }
    const double out = blockSum(acc, sh);
    if (threadIdx.x == 0) {
        const double Vz = g.zoneVol[z], dInt = g.zoneDInt[z];
        g.zoneDP[z] = K_GAMMA * g.zoneP[z] * (double)(dInt - out) / Vz;
        g.zoneShift[z] = (double)(dInt - out) / Vz;
    }
}

// ---------------------------------------------------------------------------
// Solver::project, right-hand side and warm-start residual
// (src/sim/gasphase.cpp:528-549, 576-581), with the closed-zone divergence
// shift of leakage (:495-498) applied to S first. The right-hand side is
// stored in the arithmetic type (FP32 on the mixed path: the system the
// refinement loop solves to 1e-8 is the one with this b).
template <class R>
__global__ void k_rhs(const Scn<R>* __restrict__ S, Dom dom) {
    using T = R;
    PHX_PROLOGUE(dom);
    int c = tile_ * TPB + threadIdx.x;
    T bm = 0, rm = 0;
    if (c < g.N) {
        if (g.blocked[c]) {
            g.b[c] = 0;
            g.p[c] = 0;
            g.r[c] = 0;
        } else {
            const int nx = g.nx, ny = g.ny, nz = g.nz, sxy = nx * ny;
            int i, j, k;
            ijkOf(g, 0, c, i, j, k);
            const T dt = (T)g.sv[SV_DT];
            const T dx = (T)g.dx;
            const T inv = dx * dx / dt;
            T Sc = g.S[c];
            if (g.nClosed > 0) {
                int z = g.zone[c];
                if (z >= 0 && !g.zoneOpen[z]) {
                    Sc -= (T)g.zoneShift[z];
                    g.S[c] = Sc;
                }
            }
            const int a0 = i + (nx + 1) * (j + ny * k), a1 = a0 + 1;
            const int b0 = i + nx * (j + (ny + 1) * k), b1 = b0 + nx;
            const int c0 = c, c1 = c + sxy;
            const T u0 = g.u[a0], u1 = g.u[a1], v0 = g.v[b0], v1 = g.v[b1], w0 = g.w[c0], w1 = g.w[c1];
            T div = (g.fx[a1] * u1 - g.fx[a0] * u0 + g.fy[b1] * v1 - g.fy[b0] * v0 + g.fz[c1] * w1 - g.fz[c0] * w0) / dx;
            T b = (Sc - div) * inv;
            const T A0 = g.a0x[a0], A1 = g.a0x[a1], A2 = g.a0y[b0], A3 = g.a0y[b1], A4 = g.a0z[c0], A5 = g.a0z[c1];
            if (i == 0 && A0 > T(0)) b += A0 * (u0 > T(0) ? T(-0.5) * u0 * u0 : T(0));
            if (i == nx - 1 && A1 > T(0)) b += A1 * (u1 < T(0) ? T(-0.5) * u1 * u1 : T(0));
            if (j == 0 && A2 > T(0)) b += A2 * (v0 > T(0) ? T(-0.5) * v0 * v0 : T(0));
            if (j == ny - 1 && A3 > T(0)) b += A3 * (v1 < T(0) ? T(-0.5) * v1 * v1 : T(0));
            if (k == nz - 1 && A5 > T(0)) b += A5 * (w1 < T(0) ? T(-0.5) * w1 * w1 : T(0));
            g.b[c] = b;
            const T dg = g.diag[c];
            T r = 0;
            if (dg > T(0)) {
                const R* x = g.p;
                T s = dg * x[c];
                if (i > 0) s -= A0 * x[c - 1];
                if (i < nx - 1) s -= A1 * x[c + 1];
                if (j > 0) s -= A2 * x[c - nx];
                if (j < ny - 1) s -= A3 * x[c + nx];
                if (k > 0) s -= A4 * x[c - sxy];
                if (k < nz - 1) s -= A5 * x[c + sxy];
                r = b - s;
                bm = fabs(b);
            }
            g.r[c] = r;
            rm = fabs(r);
        }
    }
    blockMaxTo(g.sv + SV_BMAX, bm);
    blockMaxTo(g.sv + SV_RMAX, rm);
}

// closed zones: H is defined up to a constant; its zone mean is removed
// (src/sim/gasphase.cpp:629-639). One CTA per closed zone, then a pass over
// the closed cells.
template <class R>
__global__ void k_zone_mean(const Scn<R>* __restrict__ S, Dom dom) {
    PHX_PROLOGUE(dom);
    __shared__ double sh[32];
    const int zi = tile_;
    double acc = 0;
    for (int e = g.closedStart[zi] + threadIdx.x; e < g.closedStart[zi + 1]; e += blockDim.x) {
        const int c = g.closedCells[e];
        acc += g.p64 ? g.p64[c] : (double)g.p[c];   // mixed path: the FP64 pressure
    }
    double sum = blockSum(acc, sh);
    if (threadIdx.x == 0) {
        double cnt = (double)(g.closedStart[zi + 1] - g.closedStart[zi]);
        g.zoneMean[g.closedZone[zi]] = cnt > 0 ? sum / cnt : 0.0;
    }
}

template <class R>
__global__ void k_zone_mean_sub(const Scn<R>* __restrict__ S, Dom dom) {
    PHX_PROLOGUE(dom);
    int e = tile_ * TPB + threadIdx.x;
    int n = g.closedStart[g.nClosed];
    if (e >= n) return;
    int c = g.closedCells[e];
    const double mean = g.zoneMean[g.zone[c]];
    if (g.p64) {   // mixed path: the FP64 pressure is the solution; p follows it
        g.p64[c] -= mean;
        g.p[c] = (R)g.p64[c];
    } else {
        g.p[c] = (R)((double)g.p[c] - mean);
    }
}

// velocity correction u -= dt/dx grad H on matrix faces, clamp, maxVel
// (src/sim/gasphase.cpp:641-676). One thread per face of one axis.
template <class R>
__global__ void k_velcorr(const Scn<R>* __restrict__ S, Dom dom, int comp) {
    using T = R;
    PHX_PROLOGUE(dom);
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const int dX = nx + (comp == 0), dY = ny + (comp == 1), dZ = nz + (comp == 2);
    int f = tile_ * TPB + threadIdx.x;
    T vm = 0;
    if (f < dX * dY * dZ) {
        int i, j, k;
        ijkOf(g, faceKind(comp), f, i, j, k);
        R* vel = comp == 0 ? g.u : comp == 1 ? g.v : g.w;
        const R* fo = comp == 0 ? g.fx : comp == 1 ? g.fy : g.fz;
        const R* am = comp == 0 ? g.ax : comp == 1 ? g.ay : g.az;
        const T s = (T)g.sv[SV_DT] / (T)g.dx;
        const R* P = g.p;
        // every load of the face up front (cell indices clamped into the grid,
        // used only where the face has that cell)
        const int ca = comp == 0 ? i : comp == 1 ? j : k;   // index of the face along its axis
        const int na = comp == 0 ? nx : comp == 1 ? ny : nz;
        const int stc = comp == 0 ? 1 : comp == 1 ? nx : nx * ny;
        const int cHi = ca < na ? i + nx * (j + ny * k) : 0;
        const int cLo = ca > 0 ? i + nx * (j + ny * k) - stc : 0;
        const T fof = fo[f];
        T un = vel[f];
        const T amf = am[f];
        const T pHi = P[cHi], pLo = P[cLo];
        if (comp == 2 && k == 0) {
            // the ground faces are not visited by the reference's loop
            vm = 0;
        } else if (fof <= T(0)) {
            vel[f] = 0;
        } else {
            // open boundary faces of x and y take part where the wind profile leaves them open
            const bool side = comp != 2 && (ca == 0 || ca == na);
            if (amf > T(0) && !(side && !bndOpen(g, comp, ca == 0 ? 0 : 1, g.oz + (k + 0.5) * g.dx))) {
                const T hi = ca < na ? pHi : (un < T(0) ? T(-0.5) * un * un : T(0));
                const T lo = ca > 0 ? pLo : (un > T(0) ? T(-0.5) * un * un : T(0));
                un = clampd(un - s * (hi - lo), -T(K_VMAX), T(K_VMAX));
                vel[f] = un;
            }
            vm = fabs(un) * fof;   // in the arithmetic type, as the reference's float build
        }
    }
    blockMaxTo(g.sv + SV_MAXVEL, vm);
}

// ---------------------------------------------------------------------------
// Solver::advectScalars (src/sim/gasphase.cpp:685-784): Superbee-limited
// transport of the ten scalars, written to the second scalar buffers.
template <class T>
__device__ __forceinline__ T superbee(T r) {
    T m = T(0), a = mn(T(2) * r, T(1)), b = mn(r, T(2));
    if (m < a) m = a;
    if (m < b) m = b;
    return m;
}

// superbee(num / den) * den without the division (FP32 path): for den > 0
// max(0, min(2 num, den), min(num, 2 den)); a negative den swaps min and max
__device__ __forceinline__ float superbeeTimes(float num, float den) {
    if (den > 0.f) return fmaxf(0.f, fmaxf(fminf(2.f * num, den), fminf(num, 2.f * den)));
    return fminf(0.f, fminf(fmaxf(2.f * num, den), fmaxf(num, 2.f * den)));
}

// FP64 path: the quantities of one interior face between two gas cells that
// both cells' transport reads -- the upwind density, each scalar's
// Superbee-limited face value and the species' diffusion terms -- evaluated
// once per face, from the lower cell's side, with the cell kernel's
// expressions. The upper cell's diffusion terms are their exact negations
// ((a - b) = -(b - a) in IEEE arithmetic; products and quotients keep the
// sign), its face values the same upwind expressions, its Dd and rfd the same
// sums in the other order (IEEE addition commutes). At zero flux the cells
// use their own values (multiplied by zero). Halves the FP64 divisions of the
// transport.
template <class R>
__global__ void k_adv_faces(const Scn<R>* __restrict__ S, Dom dom, int axis) {
    using T = R;
    PHX_PROLOGUE(dom);
    const int f = tile_ * TPB + threadIdx.x;
    const int nx = g.nx, ny = g.ny, nz = g.nz, sxy = nx * ny;
    const int nfa = axis == 0 ? g.NX : axis == 1 ? g.NY : g.NZ;
    if (!g.adv || f >= nfa) return;
    int i, j, k, id, dim, st;
    ijkOf(g, faceKind(axis), f, i, j, k);
    if (axis == 0) { id = i; dim = nx; st = 1; }
    else if (axis == 1) { id = j; dim = ny; st = nx; }
    else { id = k; dim = nz; st = sxy; }
    if (id < 1 || id > dim - 1) return;   // domain faces: one cell, evaluated inline
    const int U = i + nx * (j + ny * k), L = U - st;
    const T fo = axis == 0 ? g.fx[f] : axis == 1 ? g.fy[f] : g.fz[f];
    if (!(fo > T(0)) || g.blocked[L] || g.blocked[U]) return;
    const T un = fo * (axis == 0 ? g.u[f] : axis == 1 ? g.v[f] : g.w[f]);
    int opp = id - 2 >= 0 ? L - st : -1, nb2 = id + 1 < dim ? U + st : -1;
    if (opp >= 0 && g.blocked[opp]) opp = -2;
    if (nb2 >= 0 && g.blocked[nb2]) nb2 = -2;
    const int NF = g.NX + g.NY + g.NZ;
    const int fg = (axis == 0 ? 0 : axis == 1 ? g.NX : g.NX + g.NY) + f;
    double* rec = g.adv + fg;
    const T dx = (T)g.dx;
    // upwind density (the temperature part of :700-717)
    {
        const R* Tf = g.sc[0];
        const T tn = Tf[U], tc = Tf[L];
        T tface;
        if (un > T(0)) {
            T tu2 = opp >= 0 ? Tf[opp] : (opp == -1 ? T(K_T0) : tc);
            T den = tn - tc;
            tface = tc + (fabs(den) > T(1e-6) ? T(0.5) * superbee((tc - tu2) / den) * den : T(0));
        } else {
            T tu2 = nb2 >= 0 ? Tf[nb2] : (nb2 == -1 ? T(K_T0) : tn);
            T den = tc - tn;
            tface = tn + (fabs(den) > T(1e-6) ? T(0.5) * superbee((tn - tu2) / den) * den : T(0));
        }
        T pu = un > T(0) ? g.Pb[L] : g.Pb[U];
        rec[(size_t)ADV_RUP * NF] = (double)(pu / (T(K_RS) * mx(tface, T(K_T_MIN))));
    }
    const T Dd = T(0.5) * (g.nu[L] + g.nu[U]) / T(K_SC_T) + T(2.0e-5);
    const T rfd = T(0.5) * (rhoOf(g, L) + rhoOf(g, U));
    for (int q = 0; q < NSC; ++q) {
        const R* F = g.sc[q];
        const T fc = F[L], fn = F[U];
        T face = fc;
        if (un > T(0)) {
            T fu2 = opp >= 0 ? F[opp] : (opp == -1 ? ambOf<T>(q) : fc);
            T den = fn - fc;
            if (fabs(den) > T(1e-12)) face += T(0.5) * superbee((fc - fu2) / den) * den;
        } else if (un < T(0)) {
            T fu2 = nb2 >= 0 ? F[nb2] : (nb2 == -1 ? ambOf<T>(q) : fn);
            T den = fc - fn;
            face = fn;
            if (fabs(den) > T(1e-12)) face += T(0.5) * superbee((fn - fu2) / den) * den;
        }
        rec[(size_t)(ADV_FACE + q) * NF] = (double)face;
        if (q > 0) {
            rec[(size_t)(ADV_DQ + q - 1) * NF] = (double)(fo * Dd * (fn - fc) / dx);
            rec[(size_t)(ADV_MQ + q - 1) * NF] = (double)(fo * rfd * Dd * (fn - fc) / dx);
        }
    }
}

template <class R>
__device__ __forceinline__ void advectCells(const Scn<R>* __restrict__ S, const Dom& dom) {
    using T = R;
    PHX_PROLOGUE(dom);
    int c = tile_ * TPB + threadIdx.x;
    if (c >= g.N) return;
    if (g.blocked[c]) {
        for (int q = 0; q < NSC; ++q) g.sc2[q][c] = g.sc[q][c];
        return;
    }
    // The FP32 path (mixed precision) uses division-free forms of the same
    // expressions: the limiter as superbeeTimes, 1/dx and 1/mden multiplied.
    // The FP64 path keeps the reference's operations one for one.
    constexpr bool kF32 = std::is_same<T, float>::value;
    const int nx = g.nx, ny = g.ny, nz = g.nz, sxy = nx * ny;
    int i, j, k;
    ijkOf(g, 0, c, i, j, k);
    const T dx = (T)g.dx;
    const T invDx = T(1) / dx;
    const T dt = (T)g.sv[SV_DT];
    const T s = dt / dx;
    const int fa0 = i + (nx + 1) * (j + ny * k), fa1 = fa0 + 1;
    const int fb0 = i + nx * (j + (ny + 1) * k), fb1 = fb0 + nx;
    const int fc0 = c, fc1 = c + sxy;
    T fo[6] = {g.fx[fa0], g.fx[fa1], g.fy[fb0], g.fy[fb1], g.fz[fc0], g.fz[fc1]};
    T un[6] = {-fo[0] * g.u[fa0], fo[1] * g.u[fa1], -fo[2] * g.v[fb0], fo[3] * g.v[fb1], -fo[4] * g.w[fc0],
               fo[5] * g.w[fc1]};
    const int id[3] = {i, j, k};
    const int dim[3] = {nx, ny, nz}, st[3] = {1, nx, sxy};
    int nb[6], nb2[6], opp[6];
    for (int d = 0; d < 6; ++d) {
        int a = d >> 1, sg = (d & 1) ? 1 : -1;
        int n1 = id[a] + sg, n2 = id[a] + 2 * sg, o1 = id[a] - sg;
        nb[d] = (n1 >= 0 && n1 < dim[a]) ? c + sg * st[a] : -1;
        nb2[d] = (n2 >= 0 && n2 < dim[a]) ? c + 2 * sg * st[a] : -1;
        opp[d] = (o1 >= 0 && o1 < dim[a]) ? c - sg * st[a] : -1;
        if (nb[d] >= 0 && g.blocked[nb[d]]) nb[d] = -2;
        if (nb2[d] >= 0 && g.blocked[nb2[d]]) nb2[d] = -2;
        if (opp[d] >= 0 && g.blocked[opp[d]]) opp[d] = -2;
    }
    const R* Tf = g.sc[0];
    const T nuc = g.nu[c];
    const T rc = rhoOf(g, c);
    // FP64 path: interior faces between gas cells come from k_adv_faces
    const double* adv = kF32 ? nullptr : g.adv;
    const int NF = g.NX + g.NY + g.NZ;
    const int fgl[6] = {fa0, fa1, g.NX + fb0, g.NX + fb1, g.NX + g.NY + fc0, g.NX + g.NY + fc1};
    T rUp[6], Dd[6], rfd[6], mden = rc;
    for (int d = 0; d < 6; ++d) {
        rUp[d] = 0;
        Dd[d] = 0;
        rfd[d] = 0;
        if (fo[d] <= T(0) || nb[d] == -2) continue;
        if (adv && nb[d] >= 0) {
            rUp[d] = (T)adv[(size_t)ADV_RUP * NF + fgl[d]];
            mden -= s * rUp[d] * un[d];
            continue;
        }
        T tn = nb[d] >= 0 ? Tf[nb[d]] : tAmbient<T>(), tc = Tf[c], tface;
        if (un[d] > T(0)) {
            T tu2 = opp[d] >= 0 ? Tf[opp[d]] : (opp[d] == -1 ? tAmbient<T>() : tc);
            T den = tn - tc;
            if constexpr (kF32) tface = tc + (fabs(den) > T(1e-6) ? T(0.5) * superbeeTimes(tc - tu2, den) : T(0));
            else tface = tc + (fabs(den) > T(1e-6) ? T(0.5) * superbee((tc - tu2) / den) * den : T(0));
        } else {
            T tu2 = nb2[d] >= 0 ? Tf[nb2[d]] : (nb2[d] == -1 ? tAmbient<T>() : tn);
            T den = tc - tn;
            if constexpr (kF32) tface = tn + (fabs(den) > T(1e-6) ? T(0.5) * superbeeTimes(tn - tu2, den) : T(0));
            else tface = tn + (fabs(den) > T(1e-6) ? T(0.5) * superbee((tn - tu2) / den) * den : T(0));
        }
        T pu = un[d] > T(0) ? g.Pb[c] : (nb[d] >= 0 ? g.Pb[nb[d]] : T(K_P0));
        rUp[d] = pu / (T(K_RS) * mx(tAbs(tface), T(K_T_MIN)));
        mden -= s * rUp[d] * un[d];
        // species diffusion coefficient and face density: the same for every species
        T nun = nb[d] >= 0 ? g.nu[nb[d]] : nuc;
        Dd[d] = T(0.5) * (nuc + nun) / T(K_SC_T) + T(2.0e-5);
        rfd[d] = nb[d] >= 0 ? T(0.5) * (rc + rhoOf(g, nb[d])) : rc;
    }
    const bool conservative = mden > T(0.25) * rc;
    // FP32 path: the per-face diffusion factors of the species
    T kd[6], km[6];
    if constexpr (kF32)
        for (int d = 0; d < 6; ++d) {
            kd[d] = fo[d] * Dd[d] * invDx;
            km[d] = fo[d] * rfd[d] * Dd[d] * invDx;
        }
    const T invMden = T(1) / mden;
    for (int q = 0; q < NSC; ++q) {
        const R* F = g.sc[q];
        const T fc = F[c];
        T lo = fc, hi = fc, acc = 0, macc = 0;
        for (int d = 0; d < 6; ++d) {
            if (fo[d] <= T(0) || nb[d] == -2) continue;
            T fn = nb[d] >= 0 ? F[nb[d]] : ambOf<T>(q);
            lo = mn(lo, fn);
            hi = mx(hi, fn);
            T flux = un[d];
            if (adv && nb[d] >= 0) {
                const T face = flux != T(0) ? (T)adv[(size_t)(ADV_FACE + q) * NF + fgl[d]] : fc;
                acc -= flux * (face - fc);
                macc -= rUp[d] * flux * face;
                if (q > 0) {
                    T dq = (T)adv[(size_t)(ADV_DQ + q - 1) * NF + fgl[d]];
                    T mq = (T)adv[(size_t)(ADV_MQ + q - 1) * NF + fgl[d]];
                    if (!(d & 1)) { dq = -dq; mq = -mq; }   // the cell is the face's upper cell
                    acc += dq;
                    macc += mq;
                }
                continue;
            }
            T face = fc;
            if (flux > T(0)) {
                T fu2 = opp[d] >= 0 ? F[opp[d]] : (opp[d] == -1 ? ambOf<T>(q) : fc);
                T den = fn - fc;
                if constexpr (kF32) {
                    if (fabs(den) > T(1e-12)) face += T(0.5) * superbeeTimes(fc - fu2, den);
                } else {
                    if (fabs(den) > T(1e-12)) face += T(0.5) * superbee((fc - fu2) / den) * den;
                }
            } else if (flux < T(0)) {
                T fu2 = nb2[d] >= 0 ? F[nb2[d]] : (nb2[d] == -1 ? ambOf<T>(q) : fn);
                T den = fc - fn;
                face = fn;
                if constexpr (kF32) {
                    if (fabs(den) > T(1e-12)) face += T(0.5) * superbeeTimes(fn - fu2, den);
                } else {
                    if (fabs(den) > T(1e-12)) face += T(0.5) * superbee((fn - fu2) / den) * den;
                }
            }
            acc -= flux * (face - fc);
            macc -= rUp[d] * flux * face;
            if (q > 0) {
                if constexpr (kF32) {
                    acc += kd[d] * (fn - fc);
                    macc += km[d] * (fn - fc);
                } else {
                    acc += fo[d] * Dd[d] * (fn - fc) / dx;
                    macc += fo[d] * rfd[d] * Dd[d] * (fn - fc) / dx;
                }
            }
        }
        T val;
        if constexpr (kF32) val = conservative ? (rc * fc + s * macc) * invMden : fc + s * acc;
        else val = conservative ? (rc * fc + s * macc) / mden : fc + s * acc;
        g.sc2[q][c] = clampd(val, lo, hi);
    }
}

// superbeeTimes without a branch on the sign of den: with sg = sign(den),
// superbee(num / den) den = sg superbee(sg num / (sg den)) (sg den), and the
// sign flips are exact, so the value is superbeeTimes' value.
__device__ __forceinline__ float superbeeTimesSigned(float num, float den) {
    const float sg = den > 0.f ? 1.f : -1.f;
    const float n = sg * num, d = sg * den;
    return sg * fmaxf(0.f, fmaxf(fminf(2.f * n, d), fminf(n, 2.f * d)));
}

// FP32 transport of one gas cell (the mixed path) with the cell kernel's
// expressions, laid out so that a warp's lanes follow one instruction stream:
// what a face needs from the cell's side (its flux, the upwind density times
// the flux, the species' diffusion factors, where the upwind cell's upwind
// neighbour lies) is worked out once per cell, and each scalar's face is then
// the same straight-line sequence whatever the direction of the flow. The
// upwind cell is chosen by selects (fu, fd), the Superbee limiter is
// superbeeTimesSigned, so a warp whose cells see flows of both signs no longer
// runs both branches ten times. The values are those of the branching form
// (src/sim/gasphase.cpp:685-784 in its float build, with the division-free
// limiter).
__device__ __forceinline__ void advectCellF32(const Scn<float>& g, int c) {
    using T = float;
    const int nx = g.nx, ny = g.ny, nz = g.nz, sxy = nx * ny;
    int i, j, k;
    ijkOf(g, 0, c, i, j, k);
    const T dx = (T)g.dx;
    const T invDx = T(1) / dx;
    const T dt = (T)g.sv[SV_DT];
    const T s = dt / dx;
    const int fa0 = i + (nx + 1) * (j + ny * k);
    const int fb0 = i + nx * (j + (ny + 1) * k);
    const T fo[6] = {g.fx[fa0], g.fx[fa0 + 1], g.fy[fb0], g.fy[fb0 + nx], g.fz[c], g.fz[c + sxy]};
    const T un[6] = {-fo[0] * g.u[fa0], fo[1] * g.u[fa0 + 1], -fo[2] * g.v[fb0], fo[3] * g.v[fb0 + nx],
                     -fo[4] * g.w[c], fo[5] * g.w[c + sxy]};
    const int id[3] = {i, j, k};
    const int dim[3] = {nx, ny, nz}, st[3] = {1, nx, sxy};
    const T* Tf = g.sc[0];
    const T nuc = g.nu[c];
    const T rc = rhoOf(g, c);
    const T tc = Tf[c];
    // per face d (axis d / 2, side -1 / +1): open (fo > 0, neighbour not solid);
    // the neighbour's offset from c (0 outside the domain, where the value is
    // ambient); and the upwind cell's upwind neighbour: behind this cell for an
    // outflow, beyond the neighbour for an inflow -- its offset from c, with a
    // solid cell there standing for the upwind cell itself (offset 0 or the
    // neighbour's offset) and a cell outside the domain for ambient
    unsigned openM = 0, nbAmbM = 0, uuAmbM = 0;
    int nbOff[6], uuOff[6];
    T ruf[6], kd[6], km[6], mden = rc;
#pragma unroll
    for (int d = 0; d < 6; ++d) {
        const int a = d >> 1, sg = (d & 1) ? 1 : -1;
        const int n1 = id[a] + sg, n2 = id[a] + 2 * sg, o1 = id[a] - sg;
        const bool in1 = n1 >= 0 && n1 < dim[a], in2 = n2 >= 0 && n2 < dim[a], ino = o1 >= 0 && o1 < dim[a];
        const int so = sg * st[a];
        nbOff[d] = 0;
        uuOff[d] = 0;
        ruf[d] = T(0);
        kd[d] = T(0);
        km[d] = T(0);
        if (fo[d] <= T(0) || (in1 && g.blocked[c + so])) continue;
        openM |= 1u << d;
        if (in1) nbOff[d] = so;
        else nbAmbM |= 1u << d;
        const bool up = un[d] > T(0);
        const bool uuIn = up ? ino : in2;
        const int uuCell = up ? -so : 2 * so;
        if (!uuIn) uuAmbM |= 1u << d;
        else uuOff[d] = g.blocked[c + uuCell] ? (up ? 0 : so) : uuCell;
        // temperature face, upwind density, species diffusion (as the cell kernel)
        const T tn = in1 ? Tf[c + so] : tAmbient<T>();
        const T tuu = uuIn ? Tf[c + uuOff[d]] : tAmbient<T>();
        const T tu = up ? tc : tn, td = up ? tn : tc;
        const T tden = td - tu;
        const T tface = tu + (fabs(tden) > T(1e-6) ? T(0.5) * superbeeTimesSigned(tu - tuu, tden) : T(0));
        const T pu = up ? g.Pb[c] : (in1 ? g.Pb[c + so] : T(K_P0));
        const T rUp = pu / (T(K_RS) * mx(tAbs(tface), T(K_T_MIN)));
        mden -= s * rUp * un[d];
        ruf[d] = rUp * un[d];
        const T nun = in1 ? g.nu[c + so] : nuc;
        const T Dd = T(0.5) * (nuc + nun) / T(K_SC_T) + T(2.0e-5);
        const T rfd = in1 ? T(0.5) * (rc + rhoOf(g, c + so)) : rc;
        kd[d] = fo[d] * Dd * invDx;
        km[d] = fo[d] * rfd * Dd * invDx;
    }
    const bool conservative = mden > T(0.25) * rc;
    const T invMden = T(1) / mden;
    // Each scalar: per open face, the limited face value of the upwind cell.
    // A face without flow adds nothing (flux and upwind density times flux
    // are 0), whatever value the limiter gives it, so the face value needs no
    // zero-flux case.
#pragma unroll 1
    for (int q = 0; q < NSC; ++q) {
        const T* __restrict__ Fc = g.sc[q] + c;
        const T fc = Fc[0];
        const T amb = ambOf<T>(q);
        T lo = fc, hi = fc, acc = 0, macc = 0;
#pragma unroll
        for (int d = 0; d < 6; ++d) {
            if (!((openM >> d) & 1u)) continue;
            const T fnv = Fc[nbOff[d]], fuuv = Fc[uuOff[d]];
            const T fn = ((nbAmbM >> d) & 1u) ? amb : fnv;
            const T fuu = ((uuAmbM >> d) & 1u) ? amb : fuuv;
            lo = mn(lo, fn);
            hi = mx(hi, fn);
            const T flux = un[d];
            const bool up = flux > T(0);
            const T fu = up ? fc : fn, fd = up ? fn : fc;
            const T den = fd - fu;
            const T face = fabs(den) > T(1e-12) ? fu + T(0.5) * superbeeTimesSigned(fu - fuu, den) : fu;
            acc -= flux * (face - fc);
            macc -= ruf[d] * face;
            if (q > 0) {
                acc += kd[d] * (fn - fc);
                macc += km[d] * (fn - fc);
            }
        }
        const T val = conservative ? (rc * fc + s * macc) * invMden : fc + s * acc;
        g.sc2[q][c] = clampd(val, lo, hi);
    }
}

// The FP32 transport kernel is bounded to three CTAs per SM (80 registers, a
// few spilled in the per-cell set-up): 1.71 ms per batch-of-64 step against
// 2.36 ms with the compiler's own 95 registers (two CTAs). The FP64 body at
// 128 registers wants two CTAs per SM guaranteed.
template <class R>
__device__ __forceinline__ void advectBody(const Scn<R>* __restrict__ S, const Dom& dom) {
    if constexpr (sizeof(R) == 4) {
        PHX_PROLOGUE(dom);
        const int c = tile_ * TPB + threadIdx.x;
        if (c >= g.N) return;
        if (g.blocked[c]) {
            for (int q = 0; q < NSC; ++q) g.sc2[q][c] = g.sc[q][c];
            return;
        }
        advectCellF32(g, c);
    } else {
        advectCells<R>(S, dom);
    }
}
template <class R>
__global__ void __launch_bounds__(TPB, 3) k_advect(const Scn<R>* __restrict__ S, Dom dom) {
    advectBody<R>(S, dom);
}
template <class R>
__global__ void __launch_bounds__(TPB, 2) k_advect_2cta(const Scn<R>* __restrict__ S, Dom dom) {
    advectCells<R>(S, dom);
}

// ---------------------------------------------------------------------------
// End of step (src/sim/solver.cpp:258-268): closed-zone background pressure,
// Pb of closed-zone cells, gatherStats (:884-915), time += dt.
template <class R>
__global__ void k_zone_pressure(const Scn<R>* __restrict__ S, Dom dom) {
    PHX_PROLOGUE(dom);
    if (threadIdx.x != 0) return;
    const double dt = g.sv[SV_DT];
    for (int zi = 0; zi < g.nClosed; ++zi) {
        int z = g.closedZone[zi];
        g.zoneP[z] = clampd(g.zoneP[z] + dt * g.zoneDP[z], K_P0 - 20000.0, K_P0 + 50000.0);
    }
}

template <class R>
__global__ void k_zone_pb(const Scn<R>* __restrict__ S, Dom dom) {
    PHX_PROLOGUE(dom);
    int e = tile_ * TPB + threadIdx.x;
    if (e >= g.closedStart[g.nClosed]) return;
    int c = g.closedCells[e];
    g.Pb[c] = (R)g.zoneP[g.zone[c]];
}

// gatherStats' terms of cell c (src/sim/solver.cpp:889-894): heat release
// hrr V, fuel mass Yf rho V, temperature, burning flag; zero for blocked cells
// and c >= N. FP64 path: in FP64. Mixed path: the FP32 terms of the
// reference's float build (its gasDensity and hrr V are float), carried as
// double-float pairs into the sums, so that no FP64 instruction runs per cell.
template <class R>
struct StatsTerms {
    decltype(dotTerm(R(0), R(0))) h{}, fd{};   // double, or F2 on the mixed path
    R t = 0;
    int burning = 0;
};
template <class R>
__device__ __forceinline__ StatsTerms<R> statsTerms(const Scn<R>& g, int c) {
    StatsTerms<R> o;
    if (c >= g.N || g.blocked[c]) return o;
    const R hr = g.hrr[c];
    if constexpr (sizeof(R) == 4) {
        const float dxf = (float)g.dx, V = dxf * dxf * dxf;
        const float rho = g.Pb[c] / ((float)K_RS * tAbs(g.sc[0][c]));
        o.h = F2{hr * V, 0.f};
        o.fd = F2{g.sc[2][c] * rho * V, 0.f};
    } else {
        const double V = g.dx * g.dx * g.dx;
        o.fd = g.sc[2][c] * gasDensity(g, c) * V;
        o.h = hr * V;
    }
    o.t = tAbs(g.sc[0][c]);
    o.burning = hr > 0;
    return o;
}

template <class R>
__global__ void k_stats(const Scn<R>* __restrict__ S, Dom dom) {
    PHX_PROLOGUE(dom);
    __shared__ double shA[32];
    const StatsTerms<R> st = statsTerms(g, tile_ * TPB + threadIdx.x);
    const auto h = st.h;
    blockMaxTo(g.sv + SV_MAXGAST, st.t);
    const int nbs = __syncthreads_count(st.burning);
    if (threadIdx.x == 0 && nbs > 0) atomicAdd(g.sv + SV_BURNING, (double)nbs);
    double fs = blockSum(st.fd, shA);
    int nt = ntilesOf(dom, s_);
    double tot;
    // two partial slots; the last CTA of the first closes both
    if (threadIdx.x == 0) {
        g.part[(size_t)PS_FUEL * g.partStride + tile_] = fs;
    }
    if (lastCtaSum(g, PS_HRR, tile_, nt, h, &tot)) {
        double acc = 0;
        for (int t = threadIdx.x; t < nt; t += blockDim.x) acc += __ldcg(g.part + (size_t)PS_FUEL * g.partStride + t);
        double fdTot = blockSum(acc, shA);
        if (threadIdx.x == 0) {
            const double dt = g.sv[SV_DT];
            g.sv[SV_HRR] = tot;
            g.sv[SV_FUELBURNED] += (double)tot * dt / K_DHC_FUEL;
            g.sv[SV_FUELINDOMAIN] = fdTot;
            g.sv[SV_TIME] += dt;
        }
    }
}

// pointer swaps of the double-buffered fields, one thread per scenario
template <class R>
__global__ void k_swap(Scn<R>* S, Dom dom, int what) {
    int s_, tile_;
    locate(dom, blockIdx.x, s_, tile_);
    if (threadIdx.x != 0) return;
    Scn<R>& g = S[s_];
    if (what & 1) { uint8_t* t = g.lit; g.lit = g.lit2; g.lit2 = t; }
    if (what & 2) {
        R* t;
        t = g.u; g.u = g.u2; g.u2 = t;
        t = g.v; g.v = g.v2; g.v2 = t;
        t = g.w; g.w = g.w2; g.w2 = t;
    }
    if (what & 4)
        for (int q = 0; q < NSC; ++q) { R* t = g.sc[q]; g.sc[q] = g.sc2[q]; g.sc2[q] = t; }
}

#undef PHX_PROLOGUE
}  // namespace phx
