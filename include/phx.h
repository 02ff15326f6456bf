/* phx.h -- C ABI of the GB300 gas-phase step for Photon's src/sim solver.
 *
 * Drop-in boundary. Photon's callers hold a photon::Solver and call
 * `float Solver::step(float dtMax)` (src/sim/solver.h:195), then read its public
 * field vectors (src/sim/solver.h:231-284) and stats (src/sim/solver.h:141-154,
 * 273-278). The reference has no FFI layer; this header is the C boundary a
 * host (the C++ adapter in include/photon_gpu/solver.hpp, a ctypes binding, a
 * cgo/JNI stub) binds instead of linking photon::Solver's gas phase.
 *
 * Conventions: every call returns an int status (PHX_OK = 0) and never throws;
 * the message of the last failure is phx_last_error(ctx) (or
 * phx_last_global_error() when no context exists). All buffers passed in are
 * owned by the caller and are copied before the call returns. Grid indexing is
 * the reference's (src/sim/solver.h:216-220): cell i + nx (j + ny k), x-face
 * i + (nx+1)(j + ny k), y-face i + nx (j + (ny+1) k), z-face i + nx (j + ny k).
 * One context is driven by one host thread at a time (as photon::Solver).
 */
#ifndef PHX_H
#define PHX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PHX_ABI_VERSION 1

/* status codes */
enum {
    PHX_OK = 0,
    PHX_ERR_INVALID = 1,      /* bad argument or size */
    PHX_ERR_UNSUPPORTED = 2,  /* input outside what the GPU step implements */
    PHX_ERR_OOM = 3,          /* device allocation failed */
    PHX_ERR_CUDA = 4,         /* CUDA runtime error (message has the detail) */
    PHX_ERR_TIMEOUT = 5,      /* a bounded device wait gave up */
    PHX_ERR_BUDGET = 6,       /* admission refused by the memory budget */
    PHX_ERR_STATE = 7         /* call not valid in the current state */
};

/* precision of a context */
enum {
    PHX_PREC_FP64 = 0,   /* every field and every operation in FP64 */
    PHX_PREC_MIXED = 1   /* FP32 fields, stencils and smoother scratch; FP64 dots, residual
                            refinement, closed-zone mean removal and global sums */
};

/* Grid and settings of one scenario. Mirrors what Solver::build leaves in the
 * solver (src/sim/discretize.cpp:10-62, FidelityProfile src/sim/solver.h:82-104,
 * Wind :107-111, switches :187-188). Geometry arrays are host pointers with the
 * reference's sizes: blocked N, fx/ax/lx (nx+1) ny nz, fy/ay/ly nx (ny+1) nz,
 * fz/az/lz nx ny (nz+1). lx/ly/lz may be NULL (no crack faces). */
typedef struct phx_grid {
    int nx, ny, nz;
    double dx, ox, oy, oz;
    double cfl, dt_max;          /* profile.cfl, profile.dtMax */
    int max_iters;               /* profile.pressureMaxIters */
    double tol;                  /* profile.pressureTol: largest divergence error, 1/s */
    double rel_tol;              /* extra stop: max|r| <= rel_tol * max|b| (0 = off) */
    int radiation_on;            /* Solver::radiationOn */
    int adiabatic_surfaces;      /* Solver::adiabaticSurfaces */
    double wind_speed, wind_from_deg, wind_exponent;
    const uint8_t* blocked;
    const double *fx, *fy, *fz;  /* face open fractions */
    const double *ax, *ay, *az;  /* pressure-matrix coefficients (open, not leak) */
    const uint8_t *lx, *ly, *lz; /* crack faces (orifice flow) */
} phx_grid;

/* fields readable/writable with phx_get_field / phx_set_field. Real fields
 * travel as double (converted in the mixed context), flags as uint8, zone as
 * int32. */
enum {
    PHX_FIELD_U = 0, PHX_FIELD_V, PHX_FIELD_W,
    PHX_FIELD_P, PHX_FIELD_S,
    PHX_FIELD_T, PHX_FIELD_YO, PHX_FIELD_YF, PHX_FIELD_YS, PHX_FIELD_YA, PHX_FIELD_YP,
    PHX_FIELD_YC, PHX_FIELD_YW, PHX_FIELD_YCO, PHX_FIELD_YAI,
    PHX_FIELD_NU, PHX_FIELD_PB, PHX_FIELD_Q, PHX_FIELD_QR, PHX_FIELD_HRR, PHX_FIELD_MASSSRC,
    PHX_FIELD_LIT,      /* uint8 */
    PHX_FIELD_ZONE,     /* int32, read only */
    PHX_FIELD_RHS, PHX_FIELD_CGR, PHX_FIELD_CGZ,
    PHX_FIELD_ZONEP,    /* double per zone: background pressure (Solver::zoneP, src/sim/solver.h:262) */
    PHX_FIELD_COUNT
};

/* stages for per-stage parity runs (phx_stage); the names follow the
 * reference's Solver methods. */
enum {
    PHX_STAGE_BEGIN = 0,     /* dt = stableDt(dtMax) and burner/ignition injection amounts */
    PHX_STAGE_COMBUSTION,    /* clears + injectIgnitions + injectBurners + combustion */
    PHX_STAGE_TURBULENCE,
    PHX_STAGE_HEAT,
    PHX_STAGE_ENERGY,
    PHX_STAGE_MOMENTUM,
    PHX_STAGE_LEAKAGE,
    PHX_STAGE_PROJECT,
    PHX_STAGE_ADVECT,
    PHX_STAGE_END,           /* zone pressure, Pb, gatherStats, time += dt */
    PHX_STAGE_COUNT
};

/* Solver scalars after a step (src/sim/solver.h:141-154, 273-278) */
typedef struct phx_stats {
    double time, dt;
    double max_vel, max_nu, max_div;
    int pressure_iters;
    double pressure_residual;    /* 1/s, largest divergence error left */
    double pressure_rel_residual;/* max|r| / max|b| of the last solve */
    double hrr, max_gas_t;
    int burning_cells;
    double fuel_in, fuel_burned, fuel_in_domain;
    int zones, leak_faces;
} phx_stats;

/* Create a context for one scenario and upload its geometry.
 * Replaces Solver::build (src/sim/discretize.cpp:10) for a discretized grid;
 * zones (src/sim/gasphase.cpp:111-158) and the multigrid hierarchy
 * (src/sim/pressure_mg.cpp:28-191) are built on the host here. */
int phx_create(const phx_grid* grid, int precision, struct phx_ctx** out);
void phx_destroy(struct phx_ctx* ctx);
const char* phx_last_error(const struct phx_ctx* ctx);
const char* phx_last_global_error(void);
int phx_abi_version(void);

/* Solver::addBurner (src/sim/gasphase.cpp:72-90): index_out gets the burner
 * index, or -1 with PHX_ERR_INVALID if it covers no gas cell. */
int phx_add_burner(struct phx_ctx* ctx, double x0, double y0, double x1, double y1, double z, double peak_w,
                   double ramp_s, double start, double duration, int* index_out);
/* Solver::addIgnition (src/sim/solver.cpp:122-134) */
int phx_add_ignition(struct phx_ctx* ctx, int cell, double power, double duration);

/* Solver::step (src/sim/solver.cpp:226-269), gas-only stages. dt_out may be NULL. */
int phx_step(struct phx_ctx* ctx, double dt_max, double* dt_out);
/* n steps back to back; dt_out (n entries) may be NULL */
int phx_run(struct phx_ctx* ctx, int n, double dt_max, double* dt_out);

/* one stage of the step, for per-stage parity runs; dt is used by the stages
 * that take it (the BEGIN stage ignores it and takes dt_max from the argument) */
int phx_stage(struct phx_ctx* ctx, int stage, double dt_or_dtmax);
/* z = M^-1 r with one V-cycle of the pressure multigrid (src/sim/pressure_mg.cpp:270-300) */
int phx_precondition(struct phx_ctx* ctx, const double* r, double* z);

int phx_get_field(struct phx_ctx* ctx, int field, void* host, size_t bytes);
int phx_set_field(struct phx_ctx* ctx, int field, const void* host, size_t bytes);
size_t phx_field_count(const struct phx_ctx* ctx, int field);
int phx_get_stats(struct phx_ctx* ctx, phx_stats* out);
/* time, maxVel, maxNu, maxDiv as read by the next stableDt */
int phx_set_scalars(struct phx_ctx* ctx, double time, double max_vel, double max_nu, double max_div);
/* Restore what a checkpoint holds besides the fields (Solver::loadState,
 * src/sim/state.cpp:144-145,186: time, maxVel, maxNu and the SimStats): time,
 * max_vel, max_nu, max_div, hrr, max_gas_t, burning_cells and the cumulative
 * fuel_in, fuel_burned, fuel_in_domain. The other members of *in are ignored. */
int phx_set_stats(struct phx_ctx* ctx, const phx_stats* in);
/* device bytes this context holds */
size_t phx_device_bytes(const struct phx_ctx* ctx);
/* wait for the context's stream */
int phx_sync(struct phx_ctx* ctx);

/* --- measurement helpers (the GPU analog of Solver::phaseMs, src/sim/solver.h:280-284)
 * Run n steps with everything resident in HBM; total_ms is the device time of
 * the steps measured with CUDA events on the context's stream. flush_l2 != 0
 * writes a buffer larger than L2 (untimed) before each step. launches gets the
 * number of kernel launches of the n steps. */
int phx_time_steps(struct phx_ctx* ctx, int n, double dt_max, int flush_l2, double* total_ms, int* launches);

typedef struct phx_kernel_time {
    char name[48];
    int launches;
    double ms;
} phx_kernel_time;
/* one step with CUDA events around every kernel launch; out[0..cap) gets the
 * per-kernel launch counts and summed times, *count the number of kernels */
int phx_profile_step(struct phx_ctx* ctx, double dt_max, int flush_l2, phx_kernel_time* out, int cap, int* count);
/* kernel launches of the last step */
int phx_last_step_launches(const struct phx_ctx* ctx);

/* ---- serving: continuous batching under an HBM budget -------------------------
 * No counterpart in the reference (one Solver per process there). A server
 * owns one batch context. Requests (a grid, its burners, a simulated duration
 * and a dtMax) may be submitted from any host thread at any time; the
 * submitting thread does the request's host set-up. phx_server_step, called
 * by one stepping thread, admits queued requests in arrival order while their
 * device bytes fit the budget and the batch has room, steps every running
 * request once (all in the same kernel launches), and retires the requests
 * whose simulated time reached their duration: their final fields are copied
 * to host memory and their device memory is freed. */
typedef struct phx_server phx_server;
enum { PHX_REQ_QUEUED = 0, PHX_REQ_RUNNING = 1, PHX_REQ_DONE = 2, PHX_REQ_REJECTED = 3 };
typedef struct phx_request_info {
    int state;                   /* PHX_REQ_* */
    int steps;                   /* steps run */
    double sim_time, duration;   /* simulated seconds run / requested */
    double t_submit, t_admit, t_done;   /* host steady-clock seconds */
    size_t device_bytes;
    long long cells;
    phx_stats stats;             /* final stats (finished requests) */
} phx_request_info;

int phx_server_create(int precision, size_t hbm_budget_bytes, int max_scenarios, phx_server** out);
void phx_server_destroy(phx_server* server);
const char* phx_server_last_error(const phx_server* server);
/* burners: n_burners x 9 doubles (x0 y0 x1 y1 z peak_w ramp_s start duration, as phx_add_burner) */
int phx_server_submit(phx_server* server, const phx_grid* grid, const double* burners, int n_burners,
                      double duration, double dt_max, int* request_id);
int phx_server_step(phx_server* server, int* admitted, int* finished, int* running);
int phx_server_poll(phx_server* server, int request_id, phx_request_info* out);
/* fields of a running request (from the device) or of a finished one (u v w p T, the 9 species,
 * nu, hrr, kept on the host); real fields as double */
int phx_server_get_field(phx_server* server, int request_id, int field, void* host, size_t bytes);
int phx_server_release(phx_server* server, int request_id);
int phx_server_counts(phx_server* server, int* queued, int* running, size_t* used_bytes, long long* cell_updates);

/* The statistics gatherStats reports (heat-release rate, fuel mass in the
 * domain, hottest gas temperature, burning cells) of one scenario's current
 * fields, recomputed without allocating device memory. No counterpart in the
 * reference (its stats live in host memory). For callers that must not
 * allocate at the time of the call: a serving process whose device memory is
 * committed to admitted scenarios under an HBM budget (an allocation could
 * fail or overrun the budget), or a real-time stepping loop where an
 * allocation's implicit device synchronisation would stall the stepping
 * stream. Fills hrr, fuel_in_domain, max_gas_t and burning_cells (the values
 * phx_batch_get_stats reports after the step's gatherStats, when the fields
 * have not changed since) and zeroes the other members; the context's own
 * stats are not modified. Limits and rules:
 *  - the scenario has at most 4,194,304 cells (PHX_ERR_INVALID beyond);
 *  - the context has been stepped since its last membership change
 *    (PHX_ERR_STATE otherwise: building its tables would allocate);
 *  - like every call on a context, it must not overlap another call on the
 *    same context (one host thread at a time): it reads the context's
 *    tables and enqueues work on the context's stream. While that stream is
 *    being captured into a graph it returns PHX_ERR_STATE;
 *  - it runs on the context's device, whichever device the calling thread
 *    has selected, and restores the caller's device before returning;
 *  - the first call on a device does a one-time set-up (it looks up the
 *    address of the function's device scratch); make it before any stream
 *    capture begins;
 *  - the device scratch is one array per device shared by all contexts: calls
 *    that overlap in time (from several host threads, or on different
 *    streams) race on it and give wrong results; serialise them.
 * Runs on the context's stream and returns when the result is on the host. */
int phx_gather_stats_noalloc(struct phx_ctx* ctx, int scenario, phx_stats* out);

/* --- batches ---------------------------------------------------------------
 * A context can hold several scenarios of different grids; every kernel of a
 * step covers all of them (one launch per pass, one CUDA graph per step). The
 * single-scenario calls above act on scenario 0. Scenario indices are
 * positions in the batch: removing a scenario moves the later ones down. */
int phx_create_batch(const phx_grid* grids, int n, int precision, struct phx_ctx** out);
int phx_batch_add(struct phx_ctx* ctx, const phx_grid* grid, int* scenario_out);
int phx_batch_remove(struct phx_ctx* ctx, int scenario);
int phx_batch_size(const struct phx_ctx* ctx);
size_t phx_batch_scenario_bytes(const struct phx_ctx* ctx, int scenario);
int phx_batch_add_burner(struct phx_ctx* ctx, int scenario, double x0, double y0, double x1, double y1, double z,
                         double peak_w, double ramp_s, double start, double duration, int* index_out);
/* one step of every scenario: dt_max per scenario (or NULL: dt_max_all for all);
 * dt_out (may be NULL) gets each scenario's dt */
int phx_batch_step(struct phx_ctx* ctx, const double* dt_max, double dt_max_all, double* dt_out);
int phx_batch_get_field(struct phx_ctx* ctx, int scenario, int field, void* host, size_t bytes);
int phx_batch_set_field(struct phx_ctx* ctx, int scenario, int field, const void* host, size_t bytes);
size_t phx_batch_field_count(const struct phx_ctx* ctx, int scenario, int field);
int phx_batch_get_stats(struct phx_ctx* ctx, int scenario, phx_stats* out);
int phx_batch_set_stats(struct phx_ctx* ctx, int scenario, const phx_stats* in);
/* The pressure multigrid hierarchy Solver::buildPressureLevels built for a
 * scenario (src/sim/pressure_mg.cpp:28-191): *levels gets the number of
 * levels and rows[0..cap) the unknowns of the first cap levels (level 0 is
 * the grid's cells). For tests and tuning; rows may be NULL. */
int phx_batch_mg_info(struct phx_ctx* ctx, int scenario, int* levels, int* rows, int cap);
/* Stored off-diagonal entries of each level's CSR rows in the same hierarchy
 * (the reference's PressureLevel rowStart/col/val arrays,
 * src/sim/pressure_mg.cpp:100-184): nnz[0..cap) for the first cap levels;
 * level 0, the structured grid, has no CSR rows and gets 0. For the
 * benchmark's byte model of the coarse-level kernels. */
int phx_batch_mg_nnz(struct phx_ctx* ctx, int scenario, int* nnz, int cap);
/* V-cycle schedule autotuner of the mixed path. No counterpart in the
 * reference, whose schedule is fixed (levels are added while the coarsest has
 * more than 2000 unknowns, src/sim/pressure_mg.cpp:141). Scenarios fall in
 * size buckets: bucket b holds scenarios of [20000 * 2^b, 20000 * 2^(b+1))
 * cells (bucket 0 also the smaller ones, bucket 7 also the larger ones).
 * First the coarse levels' smoothing is chosen for the whole batch: two
 * damped Jacobi sweeps per level on each leg of the V-cycle (the reference's,
 * src/sim/pressure_mg.cpp:281-297) or one (the environment variable
 * PHX_COARSE_SWEEPS=1 or 2 fixes it instead). Then, for each bucket present in
 * the batch, each candidate coarsening stop (2000, 1000, 500 unknowns) is
 * applied to the bucket's scenarios. Each candidate is timed by stepping the
 * batch `steps` times (1-50, CUDA events, after one untimed step) from the
 * same saved state at dt_max; every candidate solves to the same relative
 * residual, and the fastest is kept. The choices are recorded process-wide,
 * so scenarios and batches created later use them; the batch's state is
 * restored when the call returns. stops_out[0..min(cap, 8)) gets the chosen
 * stop of every bucket (2000 where none was tuned), stops_out[8] (cap > 8)
 * the sweeps per level and leg. On an FP64 context the call changes nothing
 * (the FP64 path keeps the reference's schedule). */
int phx_batch_tune_vcycle(struct phx_ctx* ctx, int steps, double dt_max, int* stops_out, int cap);

/* --- radiation trace -------------------------------------------------------
 * Replaces Solver::traceRadiation (src/sim/radiation.cpp:181-319): rays from
 * every radiating surface element over the gas fields resident on the device,
 * in the reference's four bands and 32 directions. The radiating elements and
 * the wall and solid temperatures come from the host (they belong to the
 * solid phase, src/sim/radiation.cpp:104-164 builds them); the gas fields
 * (T, soot, H2O, CO2, background pressure, heat release, blocked cells) are
 * the scenario's own. The FP64 context traces in FP64, the mixed context in
 * FP32 (the reference's own precision). */
typedef struct phx_rad_elem {
    double o[3];          /* ray origin, m (RadElem::o) */
    double n[3];          /* outward unit normal; unused for porous fuel */
    double area;          /* m2 */
    double emissivity;    /* Solver::elemEmissivity */
    double temperature;   /* K, Solver::elemTemp */
    int sphere;           /* porous fuel: rays over the full sphere */
    int skip_own_cell;    /* porous fuel: the ray does not absorb in its own start cell */
} phx_rad_elem;
typedef struct phx_rad_wall {  /* an intact barrier (Solver::barrierOn + barrierIntact) */
    int axis;             /* 0 x-face, 1 y-face, 2 z-face */
    int face;             /* index into that axis' face arrays */
    double t_lower;       /* K, surface seen from the cell below the face along the axis */
    double t_upper;       /* K, surface seen from the cell above it */
} phx_rad_wall;
/* rad_abs (n_elems, W absorbed by each element) and rad_gas (cells, W gained
 * by each gas cell; may be NULL) are host arrays. solid_t (cells, K; NULL =
 * ambient everywhere) is the temperature a ray sees where it enters a blocked
 * cell. At most one wall per face. Results do not depend on the order of the
 * walls; rad_gas sums its rays' contributions in an unspecified order. */
int phx_rad_trace(struct phx_ctx* ctx, const phx_rad_elem* elems, int n_elems, const phx_rad_wall* walls,
                  int n_walls, const double* solid_t, double* rad_abs, double* rad_gas);
int phx_batch_rad_trace(struct phx_ctx* ctx, int scenario, const phx_rad_elem* elems, int n_elems,
                        const phx_rad_wall* walls, int n_walls, const double* solid_t, double* rad_abs,
                        double* rad_gas);
/* device time (ms, CUDA events) of the last trace's kernels on this context */
double phx_rad_last_ms(const struct phx_ctx* ctx);

/* --- smoke and flame volume render --------------------------------------------
 * The viewer's volume ray march (the VOL_FS shader, src/render/renderer.cpp:
 * 119-283, over the volume Viewer::uploadVolume packs, src/app/viewer.cpp:
 * 941-949) into a host RGB image, without a window or GL. The members mirror
 * the shader's uniforms; the volume box is the scenario's grid. */
typedef struct phx_vol_params {
    int width, height;        /* pixels */
    float inv_vp[16];         /* inverse view-projection matrix, column-major (uInvVP) */
    float eye[3];             /* camera position, m (uEye) */
    float step;               /* march step, m (uStep; the viewer uses 0.3 dx) */
    float clip_z;             /* cut-away height, m (uClipZ) */
    float slice_z;            /* temperature slice plane height, m (uSliceZ) */
    float t_min, t_max;       /* slice colour range, K (uTMin, uTMax) */
    int smoke, slice, fire;   /* switches (uSmoke, uSlice, uFire) */
    float time;               /* s, animates the display-only noise (uTime) */
    float smoke_scale;        /* uSmokeScale */
    float sun_dir[3];         /* unit vector towards the sun (uSunDir) */
    int n_lights;             /* fire lights in use, 0-8 (uNumLights) */
    float lights[8][4];       /* x, y, z, intensity (uLights) */
    float background[3];      /* colour of the scene behind the volume (uColor) */
} phx_vol_params;
/* rgb: width*height*3 floats, rows from the bottom (GL window order). depth:
 * width*height scene depths in [0, 1] (uDepth), or NULL for no scene. */
int phx_vol_render(struct phx_ctx* ctx, const phx_vol_params* params, const float* depth, float* rgb);
int phx_batch_vol_render(struct phx_ctx* ctx, int scenario, const phx_vol_params* params, const float* depth,
                         float* rgb);
/* device time (ms, CUDA events) of the last render's kernels on this context */
double phx_vol_last_ms(const struct phx_ctx* ctx);

/* --- failure-path self-test ------------------------------------------------
 * Every wait inside a kernel of this library is bounded; when one runs out the
 * kernel records it in the context's device error word and returns, and the
 * next synchronising call reports PHX_ERR_TIMEOUT and clears the word. This
 * call exercises that path on purpose: one thread waits, for limit_ms (at most
 * 1000), on an mbarrier that nothing arrives on. It returns PHX_ERR_TIMEOUT
 * with a message; the context stays usable. No counterpart in the reference. */
int phx_selftest_wait_timeout(struct phx_ctx* ctx, double limit_ms);

/* --- process-level helpers ------------------------------------------------
 * select the CUDA device later contexts of this thread are created on */
int phx_select_device(int device);
/* page-locked host buffers for callers that stream fields every step */
void* phx_alloc_host(size_t bytes);
void phx_free_host(void* p);

#ifdef __cplusplus
}
#endif
#endif /* PHX_H */
