// gatherStats sums of one scenario recomputed with no device allocation.
//
// phx_gather_stats_noalloc (include/phx.h) serves callers that must not
// allocate device memory at the time of the call: a watchdog or monitoring
// thread sampling a running batch whose device memory is committed to
// admitted scenarios under an HBM budget (an allocation could fail or
// overrun the budget), and real-time stepping loops where cudaMalloc's
// implicit device synchronisation would stall the stepping stream. Its
// reduction scratch is the file-scope device array below, so a call
// allocates nothing; the cost is that one scratch array serves every call
// on a device, so calls must not overlap (see phx.h).
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <string>

#include "engine.h"
#include "step_kernels.cuh"

namespace phx {
namespace {

constexpr int NA_TPB = 256;                       // threads per CTA (one tile of cells each, as k_stats)
constexpr int NA_MAX_TILES = 16384;               // largest scenario: 16384 * 256 = 4,194,304 cells
constexpr int NA_MAX_DEVICES = 64;
// scratch words: [0] HRR total, [1] fuel total, [2] max T (bits, atomic max),
// [3] burning cells, [4] last-CTA counter (as unsigned), [5..7] unused,
// then the per-CTA partials of HRR and of the fuel mass
enum { NA_HRR = 0, NA_FUEL, NA_MAXT, NA_BURN, NA_CNT, NA_HEAD = 8 };
constexpr int NA_WORDS = NA_HEAD + 2 * NA_MAX_TILES;   // 262,208 bytes

// Must be zero at the start of a call: words [2], [3] and [4] (the entry
// point clears the head with cudaMemsetAsync before each launch; the last CTA
// also returns the counter to zero). The partials need no initial value.
static __device__ __align__(256) double g_naScratch[NA_WORDS];

std::mutex g_naMutex;
double* g_naPtr[NA_MAX_DEVICES] = {};

// address of the scratch on device dev (the current device), taken once per device
int scratchOnDevice(int dev, double** out, std::string& err) {
    if (dev < 0 || dev >= NA_MAX_DEVICES) { err = "device index out of range for the no-allocation scratch"; return PHX_ERR_CUDA; }
    std::lock_guard<std::mutex> lock(g_naMutex);
    if (!g_naPtr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_naScratch);
        if (e != cudaSuccess || !p) {
            err = std::string("cudaGetSymbolAddress of the no-allocation scratch: ") + cudaGetErrorString(e);
            return PHX_ERR_CUDA;
        }
        g_naPtr[dev] = static_cast<double*>(p);
    }
    *out = g_naPtr[dev];
    return PHX_OK;
}

// makes the context's device current for the duration of a call and restores
// the caller's device afterwards
struct DeviceGuard {
    int prev = -1;
    bool switched = false;
    int enter(int dev, std::string& err) {
        cudaError_t e = cudaGetDevice(&prev);
        if (e != cudaSuccess) { err = std::string("cudaGetDevice: ") + cudaGetErrorString(e); return PHX_ERR_CUDA; }
        if (prev != dev) {
            e = cudaSetDevice(dev);
            if (e != cudaSuccess) { err = std::string("cudaSetDevice: ") + cudaGetErrorString(e); return PHX_ERR_CUDA; }
            switched = true;
        }
        return PHX_OK;
    }
    ~DeviceGuard() {
        if (switched) cudaSetDevice(prev);
    }
};

// k_stats' sums over one scenario, with the same
// CTA tiling and the same fixed-order reductions, into the scratch w
template <class R>
__global__ void k_stats_noalloc(const Scn<R>* __restrict__ gp, double* __restrict__ w) {
    const Scn<R>& g = *gp;
    __shared__ double sh[32];
    __shared__ int amLast;
    const int tile = blockIdx.x, ntiles = gridDim.x;
    const StatsTerms<R> st = statsTerms(g, tile * NA_TPB + threadIdx.x);
    blockMaxTo(w + NA_MAXT, st.t);
    const int nbs = __syncthreads_count(st.burning);
    if (threadIdx.x == 0 && nbs > 0) atomicAdd(w + NA_BURN, (double)nbs);
    const double fs = blockSum(st.fd, sh);
    const double hs = blockSum(st.h, sh);
    if (threadIdx.x == 0) {
        w[NA_HEAD + tile] = hs;
        w[NA_HEAD + NA_MAX_TILES + tile] = fs;
        __threadfence();
        const unsigned t = atomicAdd(reinterpret_cast<unsigned*>(w + NA_CNT), 1u);
        amLast = (t == (unsigned)ntiles - 1u);
    }
    __syncthreads();
    if (!amLast) return;
    __threadfence();
    double a = 0, b = 0;
    for (int t = threadIdx.x; t < ntiles; t += blockDim.x) {
        a += __ldcg(w + NA_HEAD + t);
        b += __ldcg(w + NA_HEAD + NA_MAX_TILES + t);
    }
    const double ht = blockSum(a, sh);
    const double ft = blockSum(b, sh);
    if (threadIdx.x == 0) {
        w[NA_HRR] = ht;
        w[NA_FUEL] = ft;
        *reinterpret_cast<unsigned*>(w + NA_CNT) = 0u;
    }
}

}  // namespace

int gatherStatsNoAlloc(CtxBase* ctx, int precision, int scenario, phx_stats* out, std::string& err) {
    const void* desc = nullptr;
    void* streamV = nullptr;
    int cells = 0;
    int r = ctx->deviceView(scenario, &desc, &cells, &streamV);
    if (r != PHX_OK) { err = ctx->err; return r; }
    if (cells > NA_MAX_TILES * NA_TPB) {
        err = "scenario has " + std::to_string(cells) + " cells; phx_gather_stats_noalloc handles at most " +
              std::to_string(NA_MAX_TILES * NA_TPB) + " (its scratch holds " + std::to_string(NA_MAX_TILES) +
              " partial sums)";
        return PHX_ERR_INVALID;
    }
    std::memset(out, 0, sizeof(*out));
    if (cells <= 0) {   // nothing to sum: gatherStats' initial values
        out->max_gas_t = K_T0;
        return PHX_OK;
    }
    cudaStream_t st = static_cast<cudaStream_t>(streamV);
    // work enqueued here while another thread captures the context's stream
    // would land in (or break) that capture: refuse instead
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaError_t e = cudaStreamIsCapturing(st, &cs);
    if (e != cudaSuccess) { err = std::string("cudaStreamIsCapturing: ") + cudaGetErrorString(e); return PHX_ERR_CUDA; }
    if (cs != cudaStreamCaptureStatusNone) {
        err = "the context's stream is being captured into a graph; call phx_gather_stats_noalloc between other "
              "calls on this context, not during one";
        return PHX_ERR_STATE;
    }
    DeviceGuard guard;
    r = guard.enter(ctx->device, err);
    if (r != PHX_OK) return r;
    double* w = nullptr;
    r = scratchOnDevice(ctx->device, &w, err);
    if (r != PHX_OK) return r;
    e = cudaMemsetAsync(w, 0, NA_HEAD * sizeof(double), st);
    if (e != cudaSuccess) { err = std::string("cudaMemsetAsync: ") + cudaGetErrorString(e); return PHX_ERR_CUDA; }
    const int ntiles = (cells + NA_TPB - 1) / NA_TPB;
    if (precision == PHX_PREC_FP64)
        k_stats_noalloc<double><<<ntiles, NA_TPB, 0, st>>>(static_cast<const Scn<double>*>(desc), w);
    else
        k_stats_noalloc<float><<<ntiles, NA_TPB, 0, st>>>(static_cast<const Scn<float>*>(desc), w);
    e = cudaGetLastError();
    if (e != cudaSuccess) { err = std::string("kernel launch: ") + cudaGetErrorString(e); return PHX_ERR_CUDA; }
    double head[NA_HEAD];
    e = cudaMemcpyAsync(head, w, sizeof(head), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) { err = std::string("reading the no-allocation scratch: ") + cudaGetErrorString(e); return PHX_ERR_CUDA; }
    out->hrr = head[NA_HRR];
    out->fuel_in_domain = head[NA_FUEL];
    out->max_gas_t = head[NA_MAXT] > K_T0 ? head[NA_MAXT] : K_T0;   // gatherStats starts its max at T0
    out->burning_cells = (int)head[NA_BURN];
    return PHX_OK;
}

}  // namespace phx
