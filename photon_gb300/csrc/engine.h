// Host-facing interface of an engine (a batch of scenarios), independent of
// its precision. A single-scenario context is a batch of one.
#pragma once
#include <cstddef>
#include <string>
#include <vector>

#include "../../include/phx.h"

namespace phx {

class CtxBase {
public:
    virtual ~CtxBase() = default;
    virtual int addScenario(const phx_grid* g, int* id) = 0;
    virtual int removeScenario(int s) = 0;
    virtual int scenarioCount() const = 0;
    virtual size_t scenarioBytes(int s) const = 0;
    virtual int addBurner(int s, double x0, double y0, double x1, double y1, double z, double peakW, double rampS,
                          double start, double duration, int* index) = 0;
    virtual int addIgnition(int s, int cell, double power, double duration) = 0;
    // n steps of every scenario; per (optional) holds one dtMax per scenario;
    // dtOut gets one dt per step (per == null) or per step and scenario
    virtual int step(int n, double dtMax, const double* per, double* dtOut) = 0;
    virtual int stage(int stage, double arg) = 0;
    virtual int precondition(const double* r, double* z) = 0;
    virtual int getField(int s, int field, void* host, size_t bytes) = 0;
    virtual int setField(int s, int field, const void* host, size_t bytes) = 0;
    virtual size_t fieldCount(int s, int field) const = 0;
    virtual int getStats(int s, phx_stats* out) = 0;
    virtual int setStats(int s, const phx_stats* in) = 0;
    virtual int setScalars(int s, double time, double maxVel, double maxNu, double maxDiv) = 0;
    virtual size_t deviceBytes() const = 0;
    virtual int sync() = 0;
    virtual int timeSteps(int n, double dtMax, int flushL2, double* totalMs, int* launches) = 0;
    virtual int profileStep(double dtMax, int flushL2, phx_kernel_time* out, int cap, int* count) = 0;
    virtual int lastLaunches() const = 0;
    // device view of scenario s for kernels outside the engine: its descriptor
    // in device memory, its cell count and the context's stream (as void*)
    virtual int deviceView(int s, const void** descriptor, int* cells, void** stream) = 0;
    // the CUDA device the context's stream and memory live on (-1 before the first scenario)
    int device = -1;
    // multigrid hierarchy of scenario s: the number of levels, and the unknowns
    // of levels 0..min(levels, cap)-1 into rows
    virtual int mgInfo(int s, int* levels, int* rows, int cap) = 0;
    // stored off-diagonal entries of each level's CSR rows (0 for level 0)
    virtual int mgNnz(int s, int* nnz, int cap) = 0;
    // two-phase admission for the serving loop: host set-up of a scenario
    // (validation, zones, multigrid; no device work) with its device bytes,
    // then its allocation and upload into the batch. prepare() may run on
    // another host thread while the batch steps; a prepared scenario that is
    // never admitted is released with discard().
    virtual void* prepare(const phx_grid* g, size_t* bytes, std::string& err) = 0;
    virtual int admit(void* prepared, int* id) = 0;
    virtual void discard(void* prepared) = 0;
    // simulated time of every scenario, one read-back for the batch
    virtual int readTimes(double* out) = 0;
    virtual int radTrace(int s, const phx_rad_elem* el, int nE, const phx_rad_wall* wl, int nW, const double* solidT,
                         double* radAbs, double* radGas) = 0;
    virtual double radLastMs() const = 0;
    virtual int volRender(int s, const phx_vol_params* p, const float* depth, float* rgb) = 0;
    virtual int selftestWait(double limitMs) = 0;
    // V-cycle schedule autotuner (mixed path): per scenario-size bucket, the
    // multigrid coarsening stop that steps the batch fastest at the solve's
    // relative residual; out[b] gets bucket b's stop
    virtual int tuneVcycle(int steps, double dtMax, int* out, int cap) = 0;
    virtual double volLastMs() const = 0;
    std::string err;
};

// empty engines (one translation unit per precision)
CtxBase* makeCtxFp64();
CtxBase* makeCtxMixed();

// gatherStats sums of one scenario without any device allocation (noalloc.cu)
int gatherStatsNoAlloc(CtxBase* ctx, int precision, int scenario, phx_stats* out, std::string& err);

}  // namespace phx
