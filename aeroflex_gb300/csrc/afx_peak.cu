// FP64 arithmetic peak of this GPU, measured (no counterpart in the
// reference).  The FP64 residual path is bound by the FP64 pipe rather than
// by HBM, so its roofline denominator is the FP64 rate this kernel reaches:
// every thread runs CHAINS independent fused multiply-add chains, long enough
// that issue, not latency, limits the rate; the grid fills every SM several
// times over.  A fused multiply-add counts as 2 flops.  The chains' results
// are written out so nothing is eliminated.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

namespace afx {
namespace {

constexpr int CHAINS = 8;

__global__ void __launch_bounds__(256) k_fp64_fma_chains(int iters, double b, double c, double* out) {
    double a[CHAINS];
#pragma unroll
    for (int k = 0; k < CHAINS; ++k) a[k] = 1.0 + 1e-3 * (threadIdx.x + k);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < CHAINS; ++k) a[k] = __fma_rn(a[k], b, c);
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < CHAINS; ++k) s += a[k];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

// Runs the kernel `reps` times after one warm-up and returns the best rate
// in TFLOP/s, or a negative value on a CUDA error.
double fp64_fma_peak(int reps) {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return -1.0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return -1.0;
    const int threads = 256, blocks = sms * 16, iters = 4096;
    double* out = nullptr;
    if (cudaMalloc(&out, sizeof(double) * threads * blocks) != cudaSuccess) return -1.0;
    cudaStream_t s;
    cudaEvent_t e0, e1;
    cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    double best = 0.0;
    for (int r = 0; r <= reps; ++r) {
        cudaEventRecord(e0, s);
        k_fp64_fma_chains<<<blocks, threads, 0, s>>>(iters, 0.999999, 1e-7, out);
        cudaEventRecord(e1, s);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        const double flops = 2.0 * CHAINS * (double)iters * threads * blocks;
        if (r > 0 && ms > 0.f) best = std::max(best, flops / (ms * 1e-3) / 1e12);
    }
    const cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(s);
    cudaFree(out);
    return err == cudaSuccess ? best : -1.0;
}

}  // namespace afx
