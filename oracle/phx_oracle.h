/* FP64 CPU restatement of Photon's gas-phase step (test infrastructure only).
 *
 * This is the oracle the CUDA path is checked against. It restates, in plain C
 * with every real in double precision, the reference's gas-phase step
 * (src/sim/solver.cpp:226-269 and the stages in src/sim/gasphase.cpp and
 * src/sim/pressure_mg.cpp). Each function cites the reference lines it follows.
 * Operation order, reduction order (per-z-slice double partials summed in
 * order, src/sim/gasphase.cpp:39-49) and branch thresholds follow the
 * reference, so this oracle agrees with the reference's own source compiled
 * at FP64 (oracle/make_ref.py) to the last bit on the same inputs; the tests
 * in tests/test_oracle_pin.py check that.
 *
 * It is never linked into the product library.
 */
#ifndef PHX_ORACLE_H
#define PHX_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct Orc Orc;

Orc* orc_new(int nx, int ny, int nz, double dx, double ox, double oy, double oz);
void orc_free(Orc* o);
/* profile: cfl, dtMax, maxIters, tol (1/s), relTol (max|r| <= relTol max|b|, 0 = off) */
void orc_set_profile(Orc* o, double cfl, double dtMax, int maxIters, double tol, double relTol);
void orc_set_switches(Orc* o, int radiationOn, int adiabatic);
void orc_set_wind(Orc* o, double speed, double fromDeg, double exponent);
void orc_mark_geometry_dirty(Orc* o);
int orc_add_burner(Orc* o, double x0, double y0, double x1, double y1, double z, double peakW, double rampS,
                   double start, double duration);
int orc_burner_cells(Orc* o, int b, int* out, int cap);
void orc_add_ignition(Orc* o, int cell, double power, double duration);
/* coarsest-level solve: 0 = 20 forward+backward Gauss-Seidel sweeps (the reference), */
void orc_set_coarse_mode(Orc* o, int mode);
double orc_step(Orc* o, double dtMax);
int orc_stage(Orc* o, const char* stage, double dt);
double orc_stable_dt(Orc* o, double dtMax);
void orc_precondition(Orc* o, const double* r, double* z);
long orc_field_len(Orc* o, const char* name);
int orc_field(Orc* o, const char* name, int dir, void* buf, long n);
void orc_scalars(Orc* o, double* out);
void orc_set_scalars(Orc* o, double time, double maxVel, double maxNu, double maxDiv);
int orc_mg_levels(Orc* o);
void orc_mg_info(Orc* o, int l, int* info);
void orc_mg_get(Orc* o, int l, int* agg, int* rowStart, int* col, double* val, double* diag);

/* Radiation trace, Solver::traceRadiation (src/sim/radiation.cpp:181-319),
 * over flat inputs: the gas fields it reads (N each); nElem elements of 11
 * doubles (origin[3], normal[3], area, emissivity, temperature, sphere flag,
 * skip-own-cell flag: porous fuel); nWall intact barriers of 4 doubles (axis,
 * face, surface temperature seen from the lower cell, from the upper cell);
 * solidT (N): the temperature a ray sees where it enters a blocked cell.
 * Outputs: radAbs (nElem, W absorbed by each element), radGas (N, W gained by
 * each gas cell). Elements run in the reference's 24 blocks, each with its own
 * gas buffer, the buffers summed in block order. */
void orc_rad_trace(int nx, int ny, int nz, double dx, double ox, double oy, double oz, const uint8_t* blocked,
                   const double* T, const double* Ys, const double* Yw, const double* Yc, const double* Pb,
                   const double* hrr, int nElem, const double* elem, int nWall, const double* wall,
                   const double* solidT, double* radAbs, double* radGas);

/* The viewer's smoke and flame volume ray march (the VOL_FS fragment shader,
 * src/render/renderer.cpp:119-283), restated in C with FP32 arithmetic: vol
 * holds 4 floats per cell (soot density, aerosol density, T, heat release, as
 * src/app/viewer.cpp:941-949 packs them); the parameters mirror the shader's
 * uniforms (same layout as phx_vol_params); rgb gets width*height*3 floats,
 * rows from the bottom. depth may be NULL (no scene). */
typedef struct orc_vol_params {
    int width, height;
    float inv_vp[16];
    float eye[3];
    float step, clip_z, slice_z, t_min, t_max;
    int smoke, slice, fire;
    float time, smoke_scale;
    float sun_dir[3];
    int n_lights;
    float lights[8][4];
    float background[3];
} orc_vol_params;
void orc_vol_render(int nx, int ny, int nz, float dx, float ox, float oy, float oz, const float* vol,
                    const orc_vol_params* p, const float* depth, float* rgb, int row0, int row1);

#ifdef __cplusplus
}
#endif
#endif
