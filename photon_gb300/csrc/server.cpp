// Serving form of the GB300 gas-phase step: continuous batching of fire
// scenario requests under an HBM budget (include/phx.h, phx_server_*).
//
// Requests arrive at any time (phx_server_submit, from any host thread): the
// submitting thread does the request's host set-up (validation, zones,
// multigrid) and learns its device footprint. Between steps, phx_server_step
// admits queued requests in arrival order while they fit the budget and the
// batch has room, steps every running request together (one launch sequence,
// each request with its own dtMax), and retires requests whose simulated time
// reached their duration: their final fields are copied to host memory and
// their device memory is freed at once, so later arrivals can take it.
#include <chrono>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "engine.h"

namespace {

double nowSeconds() {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

// fields kept for a finished request (copied before its device memory is freed)
const int kResultFields[] = {PHX_FIELD_U, PHX_FIELD_V, PHX_FIELD_W, PHX_FIELD_P, PHX_FIELD_T, PHX_FIELD_YO,
                             PHX_FIELD_YF, PHX_FIELD_YS, PHX_FIELD_YA, PHX_FIELD_YP, PHX_FIELD_YC, PHX_FIELD_YW,
                             PHX_FIELD_YCO, PHX_FIELD_YAI, PHX_FIELD_NU, PHX_FIELD_HRR};

struct Request {
    int id = 0;
    int state = PHX_REQ_QUEUED;
    void* prepared = nullptr;    // host set-up done, not yet on the device
    size_t bytes = 0;
    std::vector<double> burners; // n x 9: x0 y0 x1 y1 z peakW rampS start duration
    double duration = 0, dtMax = 0;
    int steps = 0;
    double simTime = 0;
    double tSubmit = 0, tAdmit = 0, tDone = 0;
    long long cells = 0;
    std::map<int, std::vector<double>> results;
    phx_stats stats{};
};

}  // namespace

struct phx_server {
    std::unique_ptr<phx::CtxBase> ctx;
    int precision = 0;
    size_t budget = 0, used = 0;
    int maxScenarios = 0;
    std::mutex mu;               // guards the request table and the queue
    std::map<int, Request> reqs;
    std::deque<int> queue;
    std::vector<int> running;    // request id of each scenario of the batch, in scenario order
    int nextId = 1;
    std::string err;
    long long cellUpdates = 0;
};

namespace {

int failS(phx_server* sv, int code, const std::string& msg) {
    if (sv) sv->err = msg;
    return code;
}

// admit queued requests in arrival order while they fit (lock held)
int admitQueued(phx_server* sv, int* admitted) {
    while (!sv->queue.empty()) {
        Request& r = sv->reqs[sv->queue.front()];
        if (sv->used + r.bytes > sv->budget || (int)sv->running.size() >= sv->maxScenarios) break;
        int sid = -1;
        void* p = r.prepared;
        r.prepared = nullptr;
        int rc = sv->ctx->admit(p, &sid);   // takes ownership of the prepared scenario
        if (rc == PHX_ERR_OOM) {
            // the device is fuller than the budget says (other users): retry after a retirement
            r.state = PHX_REQ_REJECTED;
            sv->queue.pop_front();
            r.tDone = nowSeconds();
            sv->err = "request " + std::to_string(r.id) + ": " + sv->ctx->err;
            continue;
        }
        if (rc != PHX_OK) return failS(sv, rc, "admitting request " + std::to_string(r.id) + ": " + sv->ctx->err);
        for (size_t b = 0; b + 9 <= r.burners.size(); b += 9) {
            const double* q = &r.burners[b];
            int idx = -1;
            rc = sv->ctx->addBurner(sid, q[0], q[1], q[2], q[3], q[4], q[5], q[6], q[7], q[8], &idx);
            if (rc != PHX_OK) return failS(sv, rc, "request " + std::to_string(r.id) + " burner: " + sv->ctx->err);
        }
        sv->used += r.bytes;
        sv->running.push_back(r.id);
        r.state = PHX_REQ_RUNNING;
        r.tAdmit = nowSeconds();
        sv->queue.pop_front();
        ++*admitted;
    }
    return PHX_OK;
}

// copy the results of scenario s, then free it (lock held)
int retire(phx_server* sv, int s) {
    Request& r = sv->reqs[sv->running[s]];
    for (int f : kResultFields) {
        const size_t n = sv->ctx->fieldCount(s, f);
        std::vector<double>& v = r.results[f];
        v.resize(n);
        int rc = sv->ctx->getField(s, f, v.data(), n * sizeof(double));
        if (rc != PHX_OK) return failS(sv, rc, sv->ctx->err);
    }
    int rc = sv->ctx->getStats(s, &r.stats);
    if (rc != PHX_OK) return failS(sv, rc, sv->ctx->err);
    rc = sv->ctx->removeScenario(s);
    if (rc != PHX_OK) return failS(sv, rc, sv->ctx->err);
    sv->used -= r.bytes;
    sv->running.erase(sv->running.begin() + s);
    r.state = PHX_REQ_DONE;
    r.tDone = nowSeconds();
    return PHX_OK;
}

}  // namespace

extern "C" {

int phx_server_create(int precision, size_t hbm_budget_bytes, int max_scenarios, phx_server** out) {
    if (!out) return PHX_ERR_INVALID;
    *out = nullptr;
    if (precision != PHX_PREC_FP64 && precision != PHX_PREC_MIXED) return PHX_ERR_INVALID;
    if (hbm_budget_bytes == 0 || max_scenarios <= 0) return PHX_ERR_INVALID;
    std::unique_ptr<phx_server> sv(new phx_server);
    sv->ctx.reset(precision == PHX_PREC_FP64 ? phx::makeCtxFp64() : phx::makeCtxMixed());
    sv->precision = precision;
    sv->budget = hbm_budget_bytes;
    sv->maxScenarios = max_scenarios < 1024 ? max_scenarios : 1024;
    *out = sv.release();
    return PHX_OK;
}

void phx_server_destroy(phx_server* sv) {
    if (!sv) return;
    for (auto& kv : sv->reqs)
        if (kv.second.prepared) sv->ctx->discard(kv.second.prepared);
    delete sv;
}

const char* phx_server_last_error(const phx_server* sv) { return sv ? sv->err.c_str() : ""; }

int phx_server_submit(phx_server* sv, const phx_grid* grid, const double* burners, int n_burners, double duration,
                      double dt_max, int* request_id) {
    if (!sv || !grid || (n_burners > 0 && !burners) || n_burners < 0) return failS(sv, PHX_ERR_INVALID, "bad argument");
    if (!(duration > 0) || !(dt_max > 0)) return failS(sv, PHX_ERR_INVALID, "duration and dt_max must be positive");
    Request r;
    std::string e;
    try {
        r.prepared = sv->ctx->prepare(grid, &r.bytes, e);   // host set-up in the caller's thread
    } catch (const std::exception& x) {
        return failS(sv, PHX_ERR_OOM, std::string("host set-up: ") + x.what());
    }
    if (!r.prepared) return failS(sv, PHX_ERR_INVALID, e);
    if (r.bytes > sv->budget) {
        sv->ctx->discard(r.prepared);
        return failS(sv, PHX_ERR_BUDGET, "request needs " + std::to_string(r.bytes) + " device bytes, more than the budget");
    }
    r.burners.assign(burners, burners + 9 * (size_t)n_burners);
    r.duration = duration;
    r.dtMax = dt_max;
    r.cells = (long long)grid->nx * grid->ny * grid->nz;
    r.tSubmit = nowSeconds();
    std::lock_guard<std::mutex> lock(sv->mu);
    r.id = sv->nextId++;
    if (request_id) *request_id = r.id;
    sv->queue.push_back(r.id);
    sv->reqs.emplace(r.id, std::move(r));
    return PHX_OK;
}

int phx_server_step(phx_server* sv, int* admitted, int* finished, int* running) {
    if (!sv) return PHX_ERR_INVALID;
    std::lock_guard<std::mutex> lock(sv->mu);
    int nAdm = 0, nFin = 0;
    try {
        int rc = admitQueued(sv, &nAdm);
        if (rc != PHX_OK) return rc;
        const int n = (int)sv->running.size();
        if (n > 0) {
            std::vector<double> per(n), times(n);
            for (int s = 0; s < n; ++s) per[s] = sv->reqs[sv->running[s]].dtMax;
            rc = sv->ctx->step(1, 0.0, per.data(), nullptr);
            if (rc != PHX_OK) return failS(sv, rc, sv->ctx->err);
            rc = sv->ctx->readTimes(times.data());
            if (rc != PHX_OK) return failS(sv, rc, sv->ctx->err);
            for (int s = 0; s < n; ++s) {
                Request& r = sv->reqs[sv->running[s]];
                r.steps += 1;
                r.simTime = times[s];
                sv->cellUpdates += r.cells;
            }
            for (int s = n - 1; s >= 0; --s) {
                Request& r = sv->reqs[sv->running[s]];
                if (r.simTime >= r.duration) {
                    rc = retire(sv, s);
                    if (rc != PHX_OK) return rc;
                    ++nFin;
                }
            }
        }
    } catch (const std::exception& x) {
        return failS(sv, PHX_ERR_CUDA, x.what());
    }
    if (admitted) *admitted = nAdm;
    if (finished) *finished = nFin;
    if (running) *running = (int)sv->running.size();
    return PHX_OK;
}

int phx_server_poll(phx_server* sv, int request_id, phx_request_info* out) {
    if (!sv || !out) return PHX_ERR_INVALID;
    std::lock_guard<std::mutex> lock(sv->mu);
    auto it = sv->reqs.find(request_id);
    if (it == sv->reqs.end()) return failS(sv, PHX_ERR_INVALID, "no such request");
    const Request& r = it->second;
    std::memset(out, 0, sizeof(*out));
    out->state = r.state;
    out->steps = r.steps;
    out->sim_time = r.simTime;
    out->duration = r.duration;
    out->t_submit = r.tSubmit;
    out->t_admit = r.tAdmit;
    out->t_done = r.tDone;
    out->device_bytes = r.bytes;
    out->cells = r.cells;
    out->stats = r.stats;
    return PHX_OK;
}

int phx_server_get_field(phx_server* sv, int request_id, int field, void* host, size_t bytes) {
    if (!sv || !host) return PHX_ERR_INVALID;
    std::lock_guard<std::mutex> lock(sv->mu);
    auto it = sv->reqs.find(request_id);
    if (it == sv->reqs.end()) return failS(sv, PHX_ERR_INVALID, "no such request");
    const Request& r = it->second;
    if (r.state == PHX_REQ_RUNNING) {
        for (size_t s = 0; s < sv->running.size(); ++s)
            if (sv->running[s] == request_id) {
                int rc = sv->ctx->getField((int)s, field, host, bytes);
                return rc == PHX_OK ? rc : failS(sv, rc, sv->ctx->err);
            }
    }
    if (r.state != PHX_REQ_DONE) return failS(sv, PHX_ERR_STATE, "request has no fields yet");
    auto f = r.results.find(field);
    if (f == r.results.end()) return failS(sv, PHX_ERR_INVALID, "field not kept for finished requests");
    if (bytes != f->second.size() * sizeof(double)) return failS(sv, PHX_ERR_INVALID, "size mismatch");
    std::memcpy(host, f->second.data(), bytes);
    return PHX_OK;
}

int phx_server_release(phx_server* sv, int request_id) {
    if (!sv) return PHX_ERR_INVALID;
    std::lock_guard<std::mutex> lock(sv->mu);
    auto it = sv->reqs.find(request_id);
    if (it == sv->reqs.end()) return failS(sv, PHX_ERR_INVALID, "no such request");
    if (it->second.state == PHX_REQ_RUNNING || it->second.state == PHX_REQ_QUEUED)
        return failS(sv, PHX_ERR_STATE, "request still queued or running");
    sv->reqs.erase(it);
    return PHX_OK;
}

int phx_server_counts(phx_server* sv, int* queued, int* running, size_t* used_bytes, long long* cell_updates) {
    if (!sv) return PHX_ERR_INVALID;
    std::lock_guard<std::mutex> lock(sv->mu);
    if (queued) *queued = (int)sv->queue.size();
    if (running) *running = (int)sv->running.size();
    if (used_bytes) *used_bytes = sv->used;
    if (cell_updates) *cell_updates = sv->cellUpdates;
    return PHX_OK;
}

}  // extern "C"
