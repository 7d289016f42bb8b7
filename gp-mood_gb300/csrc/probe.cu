// probe.cu -- FP64 FMA throughput microbenchmark (roofline denominator), a
// probe of whether FP64 mma.sync adds to it, and the fast mode's reciprocal
// and square root on caller arrays (for their accuracy tests).
//
// Every thread runs 8 independent FMA chains (or four independent 8x8x4 FP64
// products); the grid covers every SM several times over, so the FP64 pipe,
// not latency, bounds the kernels.
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

__device__ __forceinline__ void dmma_8x8x4(double& d0, double& d1, double a, double b) {
    asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
                 : "+d"(d0), "+d"(d1) : "d"(a), "d"(b));
}

// Per warp and iteration: DFMA 8 chains x 32 lanes x 2 = 512 flops; DMMA four
// independent 8x8x4 products = 2048 flops.  kind 0: DFMA in every warp; 1: DMMA
// in every warp; 2: DMMA in even warps and DFMA in odd ones, equal flops each.
__global__ void k_pipes(double* out, int kind, int iters_f, int iters_m, double b, double c) {
    const bool mma = kind == 1 || (kind == 2 && ((threadIdx.x >> 5) & 1) == 0);
    double r;
    if (!mma) {
        double a0 = 1.0 + threadIdx.x * 1e-9, a1 = a0 + 1e-3, a2 = a0 + 2e-3, a3 = a0 + 3e-3;
        double a4 = a0 + 4e-3, a5 = a0 + 5e-3, a6 = a0 + 6e-3, a7 = a0 + 7e-3;
        for (int i = 0; i < iters_f; i++) {
            a0 = fma(a0, b, c); a1 = fma(a1, b, c); a2 = fma(a2, b, c); a3 = fma(a3, b, c);
            a4 = fma(a4, b, c); a5 = fma(a5, b, c); a6 = fma(a6, b, c); a7 = fma(a7, b, c);
        }
        r = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
    } else {
        double x0 = c, x1 = c, y0 = c, y1 = c, z0 = c, z1 = c, w0 = c, w1 = c;
        const double a = 1e-9 * threadIdx.x;
        for (int i = 0; i < iters_m; i++) {
            dmma_8x8x4(x0, x1, a, b); dmma_8x8x4(y0, y1, a, b);
            dmma_8x8x4(z0, z1, a, b); dmma_8x8x4(w0, w1, a, b);
        }
        r = x0 + x1 + y0 + y1 + z0 + z1 + w0 + w1;
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = r;
}

__global__ void k_fast_rcp(const double* x, double* y, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = gpm_fast_rcp(x[i]);
}

__global__ void k_fast_sqrt(const double* x, double* y, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = gpm_fast_sqrt(x[i]);
}

}  // namespace

// y[i] = the fast mode's 1/x[i] for device arrays of n doubles; 0 or -1.
int gpm_fast_rcp_dev(const double* x, double* y, int n) {
    if (n <= 0) return 0;
    k_fast_rcp<<<(n + 255) / 256, 256>>>(x, y, n);
    return cudaDeviceSynchronize() == cudaSuccess ? 0 : -1;
}

// y[i] = the fast mode's sqrt(x[i]) for device arrays of n doubles; 0 or -1.
int gpm_fast_sqrt_dev(const double* x, double* y, int n) {
    if (n <= 0) return 0;
    k_fast_sqrt<<<(n + 255) / 256, 256>>>(x, y, n);
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

// Whether FP64 mma.sync (DMMA) adds to the DFMA pipe: gflops[0..2] = GFLOP/s of
// DFMA alone, DMMA alone, and half the warps on each (equal flops per half),
// best of three after a warm-up, 8 CTAs of 256 threads per SM (as the FMA probe).  A mixed rate
// near the single ones means the two share the FP64 hardware.  0 or -1.
int gpm_probe_fp64_pipes(double* gflops) {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return -1;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return -1;
    const int blocks = sms * 8, threads = 256, iters_m = 500, iters_f = 2000;
    double* out = nullptr;
    if (cudaMalloc(&out, sizeof(double) * blocks * threads) != cudaSuccess) return -1;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const double warps = (double)blocks * threads / 32;
    for (int kind = 0; kind < 3; kind++) {
        float best = 1e30f;
        for (int rep = 0; rep < 4; rep++) {
            cudaEventRecord(e0);
            k_pipes<<<blocks, threads>>>(out, kind, iters_f, iters_m, 0.999999, 1e-12);
            cudaEventRecord(e1);
            cudaEventSynchronize(e1);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (rep > 0 && ms < best) best = ms;
        }
        const double flops = kind == 0 ? warps * iters_f * 512.0
                           : kind == 1 ? warps * iters_m * 2048.0
                                       : warps / 2 * iters_f * 512.0 + warps / 2 * iters_m * 2048.0;
        gflops[kind] = flops / (best * 1e-3) / 1e9;
    }
    const cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    return err == cudaSuccess ? 0 : -1;
}
