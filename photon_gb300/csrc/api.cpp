// C ABI of the GB300 gas-phase step (include/phx.h). No exception crosses it;
// every entry point returns a status and keeps the message for phx_last_error.
#include <cstring>
#include <memory>
#include <new>
#include <string>

#include <cuda_runtime.h>

#include "engine.h"

struct phx_ctx {
    phx::CtxBase* impl = nullptr;
    int precision = 0;
    std::string err;
};

namespace {
thread_local std::string g_err;

int fail(phx_ctx* c, int code, const std::string& msg) {
    if (c) c->err = msg; else g_err = msg;
    return code;
}

template <class F>
int guarded(phx_ctx* c, F f) {
    if (!c || !c->impl) return fail(c, PHX_ERR_INVALID, "null context");
    try {
        int r = f(c->impl);
        if (r != PHX_OK) c->err = c->impl->err;
        return r;
    } catch (const std::bad_alloc&) {
        return fail(c, PHX_ERR_OOM, "host allocation failed");
    } catch (const std::exception& e) {
        return fail(c, PHX_ERR_CUDA, e.what());
    } catch (...) {
        return fail(c, PHX_ERR_CUDA, "unknown error");
    }
}

phx::CtxBase* makeEngine(int precision) {
    return precision == PHX_PREC_FP64 ? phx::makeCtxFp64() : phx::makeCtxMixed();
}
}  // namespace

extern "C" {

int phx_abi_version(void) { return PHX_ABI_VERSION; }
const char* phx_last_global_error(void) { return g_err.c_str(); }
const char* phx_last_error(const phx_ctx* c) { return c ? c->err.c_str() : g_err.c_str(); }

int phx_create_batch(const phx_grid* grids, int n, int precision, phx_ctx** out) {
    if (!out) return fail(nullptr, PHX_ERR_INVALID, "out is null");
    *out = nullptr;
    if (n < 0 || (n > 0 && !grids)) return fail(nullptr, PHX_ERR_INVALID, "grids is null");
    if (precision != PHX_PREC_FP64 && precision != PHX_PREC_MIXED) return fail(nullptr, PHX_ERR_INVALID, "unknown precision");
    try {
        std::unique_ptr<phx::CtxBase> impl(makeEngine(precision));
        for (int i = 0; i < n; ++i) {
            int r = impl->addScenario(&grids[i], nullptr);
            if (r != PHX_OK) return fail(nullptr, r, "scenario " + std::to_string(i) + ": " + impl->err);
        }
        phx_ctx* c = new phx_ctx;
        c->impl = impl.release();
        c->precision = precision;
        *out = c;
        return PHX_OK;
    } catch (const std::bad_alloc&) {
        return fail(nullptr, PHX_ERR_OOM, "host allocation failed");
    } catch (const std::exception& e) {
        return fail(nullptr, PHX_ERR_CUDA, e.what());
    }
}

int phx_create(const phx_grid* grid, int precision, phx_ctx** out) {
    if (!grid) {
        if (out) *out = nullptr;
        return fail(nullptr, PHX_ERR_INVALID, "grid is null");
    }
    return phx_create_batch(grid, 1, precision, out);
}

void phx_destroy(phx_ctx* c) {
    if (!c) return;
    delete c->impl;
    delete c;
}

int phx_batch_add(phx_ctx* c, const phx_grid* grid, int* scenario_out) {
    if (!grid) return fail(c, PHX_ERR_INVALID, "grid is null");
    return guarded(c, [&](phx::CtxBase* x) { return x->addScenario(grid, scenario_out); });
}

int phx_batch_remove(phx_ctx* c, int scenario) {
    return guarded(c, [&](phx::CtxBase* x) { return x->removeScenario(scenario); });
}

int phx_batch_size(const phx_ctx* c) { return c && c->impl ? c->impl->scenarioCount() : 0; }

size_t phx_batch_scenario_bytes(const phx_ctx* c, int scenario) {
    return c && c->impl ? c->impl->scenarioBytes(scenario) : 0;
}

int phx_batch_add_burner(phx_ctx* c, int s, double x0, double y0, double x1, double y1, double z, double peak_w,
                         double ramp_s, double start, double duration, int* index_out) {
    return guarded(c, [&](phx::CtxBase* x) {
        return x->addBurner(s, x0, y0, x1, y1, z, peak_w, ramp_s, start, duration, index_out);
    });
}

int phx_add_burner(phx_ctx* c, double x0, double y0, double x1, double y1, double z, double peak_w, double ramp_s,
                   double start, double duration, int* index_out) {
    return phx_batch_add_burner(c, 0, x0, y0, x1, y1, z, peak_w, ramp_s, start, duration, index_out);
}

int phx_add_ignition(phx_ctx* c, int cell, double power, double duration) {
    return guarded(c, [&](phx::CtxBase* x) { return x->addIgnition(0, cell, power, duration); });
}

int phx_step(phx_ctx* c, double dt_max, double* dt_out) {
    return guarded(c, [&](phx::CtxBase* x) { return x->step(1, dt_max, nullptr, dt_out); });
}

int phx_run(phx_ctx* c, int n, double dt_max, double* dt_out) {
    if (n < 0) return fail(c, PHX_ERR_INVALID, "negative step count");
    return guarded(c, [&](phx::CtxBase* x) { return x->step(n, dt_max, nullptr, dt_out); });
}

int phx_batch_step(phx_ctx* c, const double* dt_max, double dt_max_all, double* dt_out) {
    return guarded(c, [&](phx::CtxBase* x) {
        if (dt_max || dt_out) {
            // per-scenario dtMax and/or dt read-back
            const int n = x->scenarioCount();
            std::unique_ptr<double[]> tmp;
            const double* per = dt_max;
            if (!per) {
                tmp.reset(new double[n > 0 ? n : 1]);
                for (int i = 0; i < n; ++i) tmp[i] = dt_max_all;
                per = tmp.get();
            }
            return x->step(1, dt_max_all, per, dt_out);
        }
        return x->step(1, dt_max_all, nullptr, nullptr);
    });
}

int phx_stage(phx_ctx* c, int stage, double arg) {
    return guarded(c, [&](phx::CtxBase* x) { return x->stage(stage, arg); });
}

int phx_precondition(phx_ctx* c, const double* r, double* z) {
    if (!r || !z) return fail(c, PHX_ERR_INVALID, "null buffer");
    return guarded(c, [&](phx::CtxBase* x) { return x->precondition(r, z); });
}

int phx_batch_get_field(phx_ctx* c, int s, int field, void* host, size_t bytes) {
    if (!host) return fail(c, PHX_ERR_INVALID, "null buffer");
    return guarded(c, [&](phx::CtxBase* x) { return x->getField(s, field, host, bytes); });
}

int phx_batch_set_field(phx_ctx* c, int s, int field, const void* host, size_t bytes) {
    if (!host) return fail(c, PHX_ERR_INVALID, "null buffer");
    return guarded(c, [&](phx::CtxBase* x) { return x->setField(s, field, host, bytes); });
}

size_t phx_batch_field_count(const phx_ctx* c, int s, int field) {
    return c && c->impl ? c->impl->fieldCount(s, field) : 0;
}

int phx_batch_get_stats(phx_ctx* c, int s, phx_stats* out) {
    if (!out) return fail(c, PHX_ERR_INVALID, "null stats");
    return guarded(c, [&](phx::CtxBase* x) { return x->getStats(s, out); });
}

int phx_batch_set_stats(phx_ctx* c, int s, const phx_stats* in) {
    if (!in) return fail(c, PHX_ERR_INVALID, "null stats");
    return guarded(c, [&](phx::CtxBase* x) { return x->setStats(s, in); });
}
int phx_set_stats(phx_ctx* c, const phx_stats* in) { return phx_batch_set_stats(c, 0, in); }

int phx_batch_tune_vcycle(phx_ctx* c, int steps, double dt_max, int* stops_out, int cap) {
    if (cap < 0) return fail(c, PHX_ERR_INVALID, "negative capacity");
    return guarded(c, [&](phx::CtxBase* x) { return x->tuneVcycle(steps, dt_max, stops_out, cap); });
}

int phx_batch_mg_info(phx_ctx* c, int s, int* levels, int* rows, int cap) {
    if (cap < 0) return fail(c, PHX_ERR_INVALID, "negative capacity");
    return guarded(c, [&](phx::CtxBase* x) { return x->mgInfo(s, levels, rows, cap); });
}

int phx_batch_mg_nnz(phx_ctx* c, int s, int* nnz, int cap) {
    if (cap < 0) return fail(c, PHX_ERR_INVALID, "negative capacity");
    return guarded(c, [&](phx::CtxBase* x) { return x->mgNnz(s, nnz, cap); });
}

int phx_get_field(phx_ctx* c, int field, void* host, size_t bytes) { return phx_batch_get_field(c, 0, field, host, bytes); }
int phx_set_field(phx_ctx* c, int field, const void* host, size_t bytes) { return phx_batch_set_field(c, 0, field, host, bytes); }
size_t phx_field_count(const phx_ctx* c, int field) { return phx_batch_field_count(c, 0, field); }
int phx_get_stats(phx_ctx* c, phx_stats* out) { return phx_batch_get_stats(c, 0, out); }

int phx_set_scalars(phx_ctx* c, double time, double max_vel, double max_nu, double max_div) {
    return guarded(c, [&](phx::CtxBase* x) { return x->setScalars(0, time, max_vel, max_nu, max_div); });
}

size_t phx_device_bytes(const phx_ctx* c) { return c && c->impl ? c->impl->deviceBytes() : 0; }

int phx_sync(phx_ctx* c) {
    return guarded(c, [&](phx::CtxBase* x) { return x->sync(); });
}

int phx_time_steps(phx_ctx* c, int n, double dt_max, int flush_l2, double* total_ms, int* launches) {
    if (n < 0) return fail(c, PHX_ERR_INVALID, "negative step count");
    return guarded(c, [&](phx::CtxBase* x) { return x->timeSteps(n, dt_max, flush_l2, total_ms, launches); });
}

int phx_profile_step(phx_ctx* c, double dt_max, int flush_l2, phx_kernel_time* out, int cap, int* count) {
    return guarded(c, [&](phx::CtxBase* x) { return x->profileStep(dt_max, flush_l2, out, cap, count); });
}

int phx_last_step_launches(const phx_ctx* c) { return c && c->impl ? c->impl->lastLaunches() : 0; }

int phx_batch_rad_trace(phx_ctx* c, int s, const phx_rad_elem* elems, int n_elems, const phx_rad_wall* walls,
                        int n_walls, const double* solid_t, double* rad_abs, double* rad_gas) {
    return guarded(c, [&](phx::CtxBase* x) {
        return x->radTrace(s, elems, n_elems, walls, n_walls, solid_t, rad_abs, rad_gas);
    });
}
int phx_rad_trace(phx_ctx* c, const phx_rad_elem* elems, int n_elems, const phx_rad_wall* walls, int n_walls,
                  const double* solid_t, double* rad_abs, double* rad_gas) {
    return phx_batch_rad_trace(c, 0, elems, n_elems, walls, n_walls, solid_t, rad_abs, rad_gas);
}
double phx_rad_last_ms(const phx_ctx* c) { return c && c->impl ? c->impl->radLastMs() : 0.0; }

int phx_batch_vol_render(phx_ctx* c, int s, const phx_vol_params* params, const float* depth, float* rgb) {
    return guarded(c, [&](phx::CtxBase* x) { return x->volRender(s, params, depth, rgb); });
}
int phx_vol_render(phx_ctx* c, const phx_vol_params* params, const float* depth, float* rgb) {
    return phx_batch_vol_render(c, 0, params, depth, rgb);
}
double phx_vol_last_ms(const phx_ctx* c) { return c && c->impl ? c->impl->volLastMs() : 0.0; }

int phx_selftest_wait_timeout(phx_ctx* c, double limit_ms) {
    return guarded(c, [&](phx::CtxBase* x) { return x->selftestWait(limit_ms); });
}

int phx_gather_stats_noalloc(phx_ctx* c, int scenario, phx_stats* out) {
    if (!out) return fail(c, PHX_ERR_INVALID, "null stats");
    return guarded(c, [&](phx::CtxBase* x) { return phx::gatherStatsNoAlloc(x, c->precision, scenario, out, x->err); });
}

int phx_select_device(int device) {
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return fail(nullptr, PHX_ERR_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
    return PHX_OK;
}

void* phx_alloc_host(size_t bytes) {
    void* p = nullptr;
    if (cudaMallocHost(&p, bytes) != cudaSuccess) {
        g_err = "cudaMallocHost failed";
        return nullptr;
    }
    return p;
}

void phx_free_host(void* p) {
    if (p) cudaFreeHost(p);
}

}  // extern "C"
