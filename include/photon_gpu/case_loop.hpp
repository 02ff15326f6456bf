// photon_gpu::runCase -- the stepping loop of `photon_cli --case` with the GPU
// solver stepping and the host photon::Solver sampling devices and writing
// checkpoints.
//
// The reference's case runner (src/app/cli_case.cpp:205-248) steps a
// photon::Solver to a duration, landing steps exactly on output and checkpoint
// times so that a resumed run samples the same instants. runCase keeps that
// loop and its float arithmetic; at every output time it moves the gas-phase
// state into the host solver (Solver::exportTo) and calls onRow(host), where
// the caller samples its devices (photon::sampleDevice, src/sim/devices.h:65-96)
// and writes its CSV rows; at every checkpoint time it moves the state and
// calls host.saveState (src/sim/state.cpp:62-121). To resume, the caller runs
// host.loadState and gpu.importFrom(host) first and passes resumed = true.
// Header only; needs include/photon_gpu/solver.hpp.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <string>

#include "solver.hpp"

namespace photon_gpu {

struct CaseSchedule {
    float duration = 60.0f;        // s simulated
    float outputInterval = 1.0f;   // s between rows
    float checkpoint = 0.0f;       // s between checkpoints (0: none)
    std::string prefix = "case";   // checkpoints: <prefix>_<t>s.state
};

// Host: anything with photon::Solver's public gas-phase members (for exportTo)
// and bool saveState(const std::string&, std::string&). RowFn: void(Host&).
// Returns the number of steps; a failed checkpoint is reported on stderr and
// the run continues, as the reference does.
template <class Host, class RowFn>
long runCase(Solver& gpu, Host& host, const CaseSchedule& sc, bool resumed, RowFn onRow) {
    const float outDt = sc.outputInterval, duration = sc.duration, ck = sc.checkpoint;
    float nextOut = resumed ? std::floor(gpu.time / outDt + 0.5f) * outDt + outDt : 0.0f;
    float nextCk = ck > 0 ? std::floor(gpu.time / ck + 0.5f) * ck + ck : 1e30f;
    auto row = [&] {
        gpu.exportTo(host);
        onRow(host);
    };
    long steps = 0;
    if (!resumed) {
        row();
        nextOut = outDt;
    }
    while (gpu.time < duration - 1e-5f) {
        // land exactly on output and checkpoint times so resumed runs sample the same instants
        const float target = std::min({nextOut, duration, nextCk});
        gpu.step(std::max(1e-4f, target - gpu.time));
        ++steps;
        if (gpu.time >= nextOut - 1e-5f) {
            row();
            nextOut += outDt;
        }
        if (gpu.time >= nextCk - 1e-5f) {
            gpu.exportTo(host);
            const std::string path = sc.prefix + "_" + std::to_string((int)std::lround(gpu.time)) + "s.state";
            std::string err;
            if (!host.saveState(path, err)) std::fprintf(stderr, "checkpoint: %s\n", err.c_str());
            nextCk += ck;
        }
    }
    return steps;
}

}  // namespace photon_gpu
