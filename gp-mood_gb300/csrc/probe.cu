// probe.cu -- FP64 FMA throughput microbenchmark (roofline denominator), and
// the fast mode's reciprocal on caller arrays (for its accuracy test).
//
// Every thread runs 8 independent FMA chains; the grid covers every SM several
// times over, so the FP64 pipe, not latency, bounds the kernel.
#include <cuda_runtime.h>

#include "fast_rcp.cuh"

namespace {

__global__ void k_dfma(double* out, int iters, double b, double c) {
    double a0 = 1.0 + threadIdx.x * 1e-9, a1 = a0 + 1e-3, a2 = a0 + 2e-3, a3 = a0 + 3e-3;
    double a4 = a0 + 4e-3, a5 = a0 + 5e-3, a6 = a0 + 6e-3, a7 = a0 + 7e-3;
    for (int i = 0; i < iters; i++) {
        a0 = fma(a0, b, c); a1 = fma(a1, b, c); a2 = fma(a2, b, c); a3 = fma(a3, b, c);
        a4 = fma(a4, b, c); a5 = fma(a5, b, c); a6 = fma(a6, b, c); a7 = fma(a7, b, c);
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}

__global__ void k_fast_rcp(const double* x, double* y, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = gpm_fast_rcp(x[i]);
}

}  // namespace

// y[i] = the fast mode's 1/x[i] for device arrays of n doubles; 0 or -1.
int gpm_fast_rcp_dev(const double* x, double* y, int n) {
    if (n <= 0) return 0;
    k_fast_rcp<<<(n + 255) / 256, 256>>>(x, y, n);
    return cudaDeviceSynchronize() == cudaSuccess ? 0 : -1;
}

// Returns GFLOP/s (FMA = 2 flops) of the best of three runs, or a negative value on error.
double gpm_probe_fp64() {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return -1.0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return -1.0;
    const int blocks = sms * 8, threads = 256, iters = 2000;
    double* out = nullptr;
    if (cudaMalloc(&out, sizeof(double) * blocks * threads) != cudaSuccess) return -1.0;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    for (int rep = 0; rep < 4; rep++) {
        cudaEventRecord(e0);
        k_dfma<<<blocks, threads>>>(out, iters, 0.999999, 1e-12);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best) best = ms;
    }
    const cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (err != cudaSuccess) return -1.0;
    const double flops = 2.0 * 8.0 * (double)blocks * threads * iters;
    return flops / (best * 1e-3) / 1e9;
}
