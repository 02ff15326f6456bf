// C ABI of the GB300 gas-phase step (include/phx.h). No exception crosses it;
// every entry point returns a status and keeps the message for phx_last_error.
#include <cstring>

#include <cuda_runtime.h>
#include <new>
#include <string>

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
}  // namespace

extern "C" {

int phx_abi_version(void) { return PHX_ABI_VERSION; }
const char* phx_last_global_error(void) { return g_err.c_str(); }
const char* phx_last_error(const phx_ctx* c) { return c ? c->err.c_str() : g_err.c_str(); }

int phx_create(const phx_grid* grid, int precision, phx_ctx** out) {
    if (!out) return fail(nullptr, PHX_ERR_INVALID, "out is null");
    *out = nullptr;
    if (!grid) return fail(nullptr, PHX_ERR_INVALID, "grid is null");
    if (precision != PHX_PREC_FP64 && precision != PHX_PREC_MIXED) return fail(nullptr, PHX_ERR_INVALID, "unknown precision");
    try {
        std::string err;
        phx::CtxBase* impl = precision == PHX_PREC_FP64 ? phx::makeCtxFp64(grid, err) : phx::makeCtxMixed(grid, err);
        if (!impl) {
            int code = err.find("not implemented") != std::string::npos || err.find("not part of") != std::string::npos
                           ? PHX_ERR_UNSUPPORTED
                       : err.find("allocation") != std::string::npos ? PHX_ERR_OOM
                       : err.find("cuda") != std::string::npos || err.find("CUDA") != std::string::npos ? PHX_ERR_CUDA
                                                                                                          : PHX_ERR_INVALID;
            return fail(nullptr, code, err);
        }
        phx_ctx* c = new phx_ctx;
        c->impl = impl;
        c->precision = precision;
        *out = c;
        return PHX_OK;
    } catch (const std::bad_alloc&) {
        return fail(nullptr, PHX_ERR_OOM, "host allocation failed");
    } catch (const std::exception& e) {
        return fail(nullptr, PHX_ERR_CUDA, e.what());
    }
}

void phx_destroy(phx_ctx* c) {
    if (!c) return;
    delete c->impl;
    delete c;
}

int phx_add_burner(phx_ctx* c, double x0, double y0, double x1, double y1, double z, double peak_w, double ramp_s,
                   double start, double duration, int* index_out) {
    return guarded(c, [&](phx::CtxBase* x) { return x->addBurner(x0, y0, x1, y1, z, peak_w, ramp_s, start, duration, index_out); });
}

int phx_add_ignition(phx_ctx* c, int cell, double power, double duration) {
    return guarded(c, [&](phx::CtxBase* x) { return x->addIgnition(cell, power, duration); });
}

int phx_step(phx_ctx* c, double dt_max, double* dt_out) {
    return guarded(c, [&](phx::CtxBase* x) { return x->step(1, dt_max, dt_out); });
}

int phx_run(phx_ctx* c, int n, double dt_max, double* dt_out) {
    if (n < 0) return fail(c, PHX_ERR_INVALID, "negative step count");
    return guarded(c, [&](phx::CtxBase* x) { return x->step(n, dt_max, dt_out); });
}

int phx_stage(phx_ctx* c, int stage, double arg) {
    return guarded(c, [&](phx::CtxBase* x) { return x->stage(stage, arg); });
}

int phx_precondition(phx_ctx* c, const double* r, double* z) {
    if (!r || !z) return fail(c, PHX_ERR_INVALID, "null buffer");
    return guarded(c, [&](phx::CtxBase* x) { return x->precondition(r, z); });
}

int phx_get_field(phx_ctx* c, int field, void* host, size_t bytes) {
    if (!host) return fail(c, PHX_ERR_INVALID, "null buffer");
    return guarded(c, [&](phx::CtxBase* x) { return x->getField(field, host, bytes); });
}

int phx_set_field(phx_ctx* c, int field, const void* host, size_t bytes) {
    if (!host) return fail(c, PHX_ERR_INVALID, "null buffer");
    return guarded(c, [&](phx::CtxBase* x) { return x->setField(field, host, bytes); });
}

size_t phx_field_count(const phx_ctx* c, int field) { return c && c->impl ? c->impl->fieldCount(field) : 0; }

int phx_get_stats(phx_ctx* c, phx_stats* out) {
    if (!out) return fail(c, PHX_ERR_INVALID, "null stats");
    return guarded(c, [&](phx::CtxBase* x) { return x->getStats(out); });
}

int phx_set_scalars(phx_ctx* c, double time, double max_vel, double max_nu, double max_div) {
    return guarded(c, [&](phx::CtxBase* x) { return x->setScalars(time, max_vel, max_nu, max_div); });
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
