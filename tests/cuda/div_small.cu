// Test harness: divSmall (photon_gb300/csrc/fdiv.cuh) against the IEEE
// quotient x / d on the GPU, for every d = 1..7 and every input given.
// Built by tests/test_gpu_div_small.py with the FP64 unit's flags.
#include <cuda_runtime.h>

#include "../../photon_gb300/csrc/fdiv.cuh"

__global__ void k_div_small(const double* __restrict__ x, long long n, double* __restrict__ fast,
                            double* __restrict__ ref) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n * 7) return;
    const long long j = i / 7;
    const int d = (int)(i % 7) + 1;
    fast[i] = phx::divSmall(x[j], d);
    ref[i] = x[j] / (double)d;
}

// fast[7 j + d - 1] = divSmall(x[j], d), ref[...] = x[j] / d; 0 on success,
// else the CUDA error code
extern "C" int div_small_check(const double* hx, long long n, double* hfast, double* href) {
    double *x = nullptr, *fast = nullptr, *ref = nullptr;
    const size_t bx = (size_t)n * sizeof(double), bo = bx * 7;
    cudaError_t e = cudaMalloc(&x, bx);
    if (e == cudaSuccess) e = cudaMalloc(&fast, bo);
    if (e == cudaSuccess) e = cudaMalloc(&ref, bo);
    if (e == cudaSuccess) e = cudaMemcpy(x, hx, bx, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && n > 0) {
        const long long total = n * 7;
        k_div_small<<<(unsigned)((total + 255) / 256), 256>>>(x, n, fast, ref);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(hfast, fast, bo, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(href, ref, bo, cudaMemcpyDeviceToHost);
    cudaFree(x);
    cudaFree(fast);
    cudaFree(ref);
    return (int)e;
}
