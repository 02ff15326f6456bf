// Host-facing interface of a scenario context, independent of its precision.
#pragma once
#include <cstddef>
#include <string>
#include <vector>

#include "../../include/phx.h"

namespace phx {

class CtxBase {
public:
    virtual ~CtxBase() = default;
    virtual int addBurner(double x0, double y0, double x1, double y1, double z, double peakW, double rampS, double start,
                          double duration, int* index) = 0;
    virtual int addIgnition(int cell, double power, double duration) = 0;
    virtual int step(int n, double dtMax, double* dtOut) = 0;
    virtual int stage(int stage, double arg) = 0;
    virtual int precondition(const double* r, double* z) = 0;
    virtual int getField(int field, void* host, size_t bytes) = 0;
    virtual int setField(int field, const void* host, size_t bytes) = 0;
    virtual size_t fieldCount(int field) const = 0;
    virtual int getStats(phx_stats* out) = 0;
    virtual int setScalars(double time, double maxVel, double maxNu, double maxDiv) = 0;
    virtual size_t deviceBytes() const = 0;
    virtual int sync() = 0;
    virtual int timeSteps(int n, double dtMax, int flushL2, double* totalMs, int* launches) = 0;
    virtual int profileStep(double dtMax, int flushL2, phx_kernel_time* out, int cap, int* count) = 0;
    virtual int lastLaunches() const = 0;
    std::string err;
};

// factories (one translation unit per precision)
CtxBase* makeCtxFp64(const phx_grid* g, std::string& err);
CtxBase* makeCtxMixed(const phx_grid* g, std::string& err);

}  // namespace phx
