// nn_gate.cu -- a-priori MLP gate: features, BF16 tensor-core inference
// (tcgen05, k_gate below), training sample harvest, and BF16 tensor-core
// forward/backward + Adam.
//
// The training products run as mma.sync.m16n8k16 with BF16 operands and FP32
// accumulation; a CTA handles 128 rows (samples), 16 per warp.
// Fragment layouts (PTX ISA, m16n8k16 .bf16): with g = lane/4, t = lane%4,
//   A (16x16, row): a0 = A[g][2t..2t+1], a1 = A[g+8][2t..], a2 = A[g][2t+8..], a3 = A[g+8][2t+8..]
//   B (16x8, col) : b0 = B[2t..2t+1][g], b1 = B[2t+8..2t+9][g]
//   C (16x8)      : c0 = C[g][2t], c1 = C[g][2t+1], c2 = C[g+8][2t], c3 = C[g+8][2t+1]
// so the accumulator tiles of one layer are the A fragments of the next.
#include <cuda_bf16.h>
#include <math.h>

#include <new>

#include "nn_gate.h"

namespace {

constexpr int ROWS = 128;          // rows per CTA
constexpr int THREADS = 2 * ROWS;  // 8 warps x 16 rows
constexpr int K0 = 48;             // layer-0 inputs padded to 3 k-tiles
constexpr int XS = K0 + 8;         // smem row stride (bf16) of X and W0
constexpr int HS = 64 + 8;         // smem row stride of W1 / W1^T
constexpr int TS = ROWS + 8;       // smem row stride of transposed activations

// Offsets of the parameter vector (PyTorch flatten order).
constexpr int P_W0 = 0;
constexpr int P_B0 = P_W0 + 64 * 36;
constexpr int P_W1 = P_B0 + 64;
constexpr int P_B1 = P_W1 + 64 * 64;
constexpr int P_W2 = P_B1 + 64;
constexpr int P_B2 = P_W2 + 64;
static_assert(P_B2 + 1 == NN_GATE_NPARAMS, "parameter layout");

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&v);
}
__device__ __forceinline__ float bf16r(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

__device__ __forceinline__ void mma16816(float* c, const uint32_t* a, uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t ld32(const __nv_bfloat16* p) { return *reinterpret_cast<const uint32_t*>(p); }

// 9-point radius-2 cross: (0,0), (-1,0), (1,0), (0,-1), (0,1), (-2,0), (2,0), (0,-2), (0,2).
__device__ __forceinline__ int cx_(int j) { return j == 1 ? -1 : j == 2 ? 1 : j == 5 ? -2 : j == 6 ? 2 : 0; }
__device__ __forceinline__ int cy_(int j) { return j == 3 ? -1 : j == 4 ? 1 : j == 7 ? -2 : j == 8 ? 2 : 0; }

// Features of interior cell (l, n); returns true when every variable is
// constant over the stencil (max - min < 1e-10 in FP32, mod_append_NN_dataset.f90:101).
__device__ bool cell_features(const GridGeom& g, const double* __restrict__ u, int l, int n, float* x) {
    float q[4][9];
#pragma unroll
    for (int j = 0; j < 9; j++) {
        const size_t c = (size_t)(n + cy_(j) + 3) * g.nx + (size_t)(l + cx_(j) + 3);
        const double2 a = __ldg(reinterpret_cast<const double2*>(u + 4 * c));
        const double2 b = __ldg(reinterpret_cast<const double2*>(u + 4 * c) + 1);
        q[0][j] = (float)a.x; q[1][j] = (float)a.y; q[2][j] = (float)b.x; q[3][j] = (float)b.y;
    }
    bool cst = true;
#pragma unroll
    for (int v = 0; v < 4; v++) {
        float mx = -INFINITY, mn = INFINITY, am = 0.f;
#pragma unroll
        for (int j = 0; j < 9; j++) {
            mx = fmaxf(mx, q[v][j]);
            mn = fminf(mn, q[v][j]);
            am = fmaxf(am, fabsf(q[v][j]));
        }
        if (!(mx - mn < 1e-10f)) cst = false;
        const float s = am > 0.f ? 1.f / am : 0.f;
#pragma unroll
        for (int j = 0; j < 9; j++) x[v * 9 + j] = q[v][j] * s;
    }
    return cst;
}

// Shared memory of a CTA: BF16 weights and the CTA's input rows.
struct SmemFwd {
    __nv_bfloat16 w0[64][XS];
    __nv_bfloat16 w1[64][HS];
    __nv_bfloat16 x[ROWS][XS];
    float b0[64], b1[64], w2[64];
};

__device__ void load_weights(SmemFwd& s, const float* __restrict__ p) {
    for (int i = threadIdx.x; i < 64 * K0; i += blockDim.x) {
        const int o = i / K0, k = i % K0;
        s.w0[o][k] = __float2bfloat16_rn(k < 36 ? p[P_W0 + o * 36 + k] : 0.f);
    }
    for (int i = threadIdx.x; i < 64 * 64; i += blockDim.x) s.w1[i / 64][i % 64] = __float2bfloat16_rn(p[P_W1 + i]);
    for (int i = threadIdx.x; i < 64; i += blockDim.x) {
        s.b0[i] = p[P_B0 + i];
        s.b1[i] = p[P_B1 + i];
        s.w2[i] = bf16r(p[P_W2 + i]);
    }
}

// Forward pass of one warp's 16 rows (r0..r0+15 of s.x).  Leaves the
// layer activations in registers: pre-activations a1, a2 (FP32) and the
// BF16 A fragments of h1; returns the logits of rows g and g+8.
struct WarpFwd {
    float a1[8][4], a2[8][4];
    uint32_t h1f[4][4];
    float logit_lo, logit_hi;
};

__device__ __forceinline__ void warp_forward(const SmemFwd& s, int r0, float b2, WarpFwd& f) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int j = 0; j < 8; j++) f.a1[j][0] = f.a1[j][1] = f.a1[j][2] = f.a1[j][3] = 0.f;
#pragma unroll
    for (int kk = 0; kk < 3; kk++) {
        uint32_t a[4];
        a[0] = ld32(&s.x[r0 + g][16 * kk + 2 * t]);
        a[1] = ld32(&s.x[r0 + g + 8][16 * kk + 2 * t]);
        a[2] = ld32(&s.x[r0 + g][16 * kk + 8 + 2 * t]);
        a[3] = ld32(&s.x[r0 + g + 8][16 * kk + 8 + 2 * t]);
#pragma unroll
        for (int j = 0; j < 8; j++)
            mma16816(f.a1[j], a, ld32(&s.w0[8 * j + g][16 * kk + 2 * t]), ld32(&s.w0[8 * j + g][16 * kk + 8 + 2 * t]));
    }
    float h1[8][4];
#pragma unroll
    for (int j = 0; j < 8; j++) {
        const float bl = s.b0[8 * j + 2 * t], bh = s.b0[8 * j + 2 * t + 1];
        f.a1[j][0] += bl; f.a1[j][1] += bh; f.a1[j][2] += bl; f.a1[j][3] += bh;
#pragma unroll
        for (int e = 0; e < 4; e++) h1[j][e] = fmaxf(f.a1[j][e], 0.f);
    }
#pragma unroll
    for (int kk = 0; kk < 4; kk++) {
        f.h1f[kk][0] = pack_bf16(h1[2 * kk][0], h1[2 * kk][1]);
        f.h1f[kk][1] = pack_bf16(h1[2 * kk][2], h1[2 * kk][3]);
        f.h1f[kk][2] = pack_bf16(h1[2 * kk + 1][0], h1[2 * kk + 1][1]);
        f.h1f[kk][3] = pack_bf16(h1[2 * kk + 1][2], h1[2 * kk + 1][3]);
    }
#pragma unroll
    for (int j = 0; j < 8; j++) f.a2[j][0] = f.a2[j][1] = f.a2[j][2] = f.a2[j][3] = 0.f;
#pragma unroll
    for (int kk = 0; kk < 4; kk++)
#pragma unroll
        for (int j = 0; j < 8; j++)
            mma16816(f.a2[j], f.h1f[kk], ld32(&s.w1[8 * j + g][16 * kk + 2 * t]),
                     ld32(&s.w1[8 * j + g][16 * kk + 8 + 2 * t]));
    float lo = 0.f, hi = 0.f;
#pragma unroll
    for (int j = 0; j < 8; j++) {
        const int c0 = 8 * j + 2 * t, c1 = c0 + 1;
        const float bl = s.b1[c0], bh = s.b1[c1];
        f.a2[j][0] += bl; f.a2[j][1] += bh; f.a2[j][2] += bl; f.a2[j][3] += bh;
        lo += bf16r(fmaxf(f.a2[j][0], 0.f)) * s.w2[c0] + bf16r(fmaxf(f.a2[j][1], 0.f)) * s.w2[c1];
        hi += bf16r(fmaxf(f.a2[j][2], 0.f)) * s.w2[c0] + bf16r(fmaxf(f.a2[j][3], 0.f)) * s.w2[c1];
    }
    lo += __shfl_xor_sync(0xffffffffu, lo, 1);
    lo += __shfl_xor_sync(0xffffffffu, lo, 2);
    hi += __shfl_xor_sync(0xffffffffu, hi, 1);
    hi += __shfl_xor_sync(0xffffffffu, hi, 2);
    f.logit_lo = lo + b2;
    f.logit_hi = hi + b2;
}

// ---------------------------------------------------------------------------
// The gate on the 5th-generation tensor cores (tcgen05).  A persistent CTA of
// 4 warps walks tiles of 128 interior cells; thread r owns row r of a tile
// (TMEM lane r).  Per tile:
//   X[128 x 48]  (BF16 features, zero-padded from 36) -> shared memory
//   D1 = X . W0^T      3 MMAs  M128 N64 K16 -> TMEM columns 0..63 (FP32)
//   H  = BF16(ReLU(D1 + b0))                    -> shared memory (tcgen05.ld, per row)
//   D2 = H . W1^T      4 MMAs                  -> TMEM columns 64..127
//   logit = sum_j BF16(ReLU(D2 + b1))_j * BF16(w2)_j + b2   (per row, FP32)
// Operands sit in shared memory in the K-major, no-swizzle canonical layout:
// 8x8 BF16 core matrices of 128 contiguous bytes (row r of a core matrix at
// 16 r), K-adjacent core matrices 128 B apart (the descriptor's leading byte
// offset) and 8-row groups KC*128 B apart (stride byte offset).  One thread
// issues the MMAs and commits them to an mbarrier; every wait is bounded and a
// timeout sets GPM_STATUS_TENSOR, frees the TMEM and leaves the kernel.
constexpr int TC_THREADS = 128;
constexpr int TC_COLS = 128;         // TMEM columns held by a CTA (D1: 0..63, D2: 64..127)
constexpr int TC_SMEM = 56 * 1024;   // dynamic shared memory requested: at most 4 CTAs (512 TMEM columns) per SM
constexpr uint32_t TC_IDESC =        // kind::f16: D F32, A and B BF16, both K-major, N = 64, M = 128
    (1u << 4) | (1u << 7) | (1u << 10) | ((64u >> 3) << 17) | ((128u >> 4) << 24);

struct __align__(1024) SmemTc {
    unsigned char w0[64 * 48 * 2];    // B of layer 0: 8 row groups x 6 k-chunks
    unsigned char w1[64 * 64 * 2];    // B of layer 1: 8 x 8
    unsigned char x[128 * 48 * 2];    // A of layer 0: 16 x 6
    unsigned char h[128 * 64 * 2];    // A of layer 1: 16 x 8
    float b0[64], b1[64], w2[64];
    unsigned long long mbar;
    uint32_t tmem;
};
static_assert(sizeof(SmemTc) <= TC_SMEM, "gate shared memory");

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Byte offset of element (r, k) of a K-major tile with kc 8-wide k-chunks.
__device__ __forceinline__ uint32_t core_off(int r, int k, int kc) {
    return (uint32_t)((r >> 3) * (kc * 128) + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// Shared-memory matrix descriptor: start, leading and stride byte offsets
// (16-byte units), descriptor version 1 (bits 46-48), no swizzle.
__device__ __forceinline__ uint64_t tc_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46);
}

__device__ __forceinline__ void tc_mma(uint32_t d, uint64_t a, uint64_t b, uint32_t accumulate) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
        "l"(a), "l"(b), "r"(TC_IDESC), "r"(accumulate));
}

__device__ __forceinline__ void tc_commit(unsigned long long* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

// Bounded wait for the mbarrier phase `parity` (~1 s at most).
__device__ __forceinline__ bool tc_wait(unsigned long long* bar, uint32_t parity) {
    for (int it = 0; it < (1 << 20); it++) {
        uint32_t done;
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(smem_u32(bar)), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// The wait of the gate's MMAs: with limit > 0 (a test hook) at most `limit`
// non-blocking polls; when that runs out, the MMAs still in flight are waited
// for with the default bound before the caller frees the TMEM they write.
__device__ __forceinline__ bool tc_wait_limited(unsigned long long* bar, uint32_t parity, int limit) {
    if (limit <= 0) return tc_wait(bar, parity);
    for (int it = 0; it < limit; it++) {
        uint32_t done;
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(smem_u32(bar)), "r"(parity)
            : "memory");
        if (done) return true;
    }
    tc_wait(bar, parity);
    return false;
}

// 32 consecutive FP32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tc_ld32(uint32_t taddr, float* v) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
        "tcgen05.wait::ld.sync.aligned;\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int j = 0; j < 32; j++) v[j] = __uint_as_float(r[j]);
}

__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__global__ void __launch_bounds__(TC_THREADS) k_gate(GridGeom g, const double* __restrict__ u,
                                                  const float* __restrict__ p, float thr, int8_t* __restrict__ order,
                                                  unsigned long long* __restrict__ count, int* __restrict__ list,
                                                  int* __restrict__ list_count, float* __restrict__ logits,
                                                  int* __restrict__ status, int wait_limit) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    SmemTc& s = *reinterpret_cast<SmemTc*>(smem_raw);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // weights, BF16, in the K-major core-matrix layout
    for (int i = tid; i < 64 * 48; i += TC_THREADS) {
        const int o = i / 48, k = i % 48;
        *reinterpret_cast<__nv_bfloat16*>(s.w0 + core_off(o, k, 6)) =
            __float2bfloat16_rn(k < 36 ? p[P_W0 + o * 36 + k] : 0.f);
    }
    for (int i = tid; i < 64 * 64; i += TC_THREADS)
        *reinterpret_cast<__nv_bfloat16*>(s.w1 + core_off(i / 64, i % 64, 8)) = __float2bfloat16_rn(p[P_W1 + i]);
    for (int i = tid; i < 64; i += TC_THREADS) {
        s.b0[i] = p[P_B0 + i];
        s.b1[i] = p[P_B1 + i];
        s.w2[i] = bf16r(p[P_W2 + i]);
    }
    const float b2 = p[P_B2];
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&s.tmem)),
                     "r"(TC_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&s.mbar)));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    fence_async_smem();
    tc_before_sync();
    __syncthreads();
    tc_after_sync();
    const uint32_t tmem = s.tmem;
    const uint32_t lane_base = (uint32_t)(32 * warp) << 16;
    const uint32_t sx = smem_u32(s.x), sh = smem_u32(s.h), sw0 = smem_u32(s.w0), sw1 = smem_u32(s.w1);
    uint32_t phase = 0;
    bool timed_out = false;
    const long long ncells = (long long)g.lf * g.nf;
    const long long ntiles = (ncells + TC_THREADS - 1) / TC_THREADS;
    for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const long long row = tile * TC_THREADS + tid;
        bool c = true;
        {
            float x[36];
            if (row < ncells) {
                const int l = 1 + (int)(row % g.lf), n = 1 + (int)(row / g.lf);
                c = cell_features(g, u, l, n, x);
            } else {
#pragma unroll
                for (int k = 0; k < 36; k++) x[k] = 0.f;
            }
#pragma unroll
            for (int kc = 0; kc < 6; kc++) {  // one 16-byte row of a core matrix per k-chunk
                uint32_t w[4];
#pragma unroll
                for (int e = 0; e < 4; e++) {
                    const int k = 8 * kc + 2 * e;
                    w[e] = pack_bf16(k < 36 ? x[k] : 0.f, k + 1 < 36 ? x[k + 1] : 0.f);
                }
                *reinterpret_cast<uint4*>(s.x + core_off(tid, 8 * kc, 6)) = make_uint4(w[0], w[1], w[2], w[3]);
            }
        }
        fence_async_smem();
        if (__syncthreads_and(c)) {  // every stencil constant: nothing to gate
            if (logits && row < ncells) logits[row] = 0.f;
            continue;
        }
        // layer 0
        if (tid == 0) {
            tc_after_sync();
#pragma unroll
            for (int k = 0; k < 3; k++) tc_mma(tmem, tc_desc(sx + 256 * k, 128, 768), tc_desc(sw0 + 256 * k, 128, 768), k > 0);
            tc_commit(&s.mbar);
        }
        bool ok = tc_wait_limited(&s.mbar, phase, wait_limit);
        phase ^= 1;
        if (__syncthreads_or(!ok)) {
            timed_out = true;
            break;
        }
        tc_after_sync();
#pragma unroll
        for (int half = 0; half < 2; half++) {
            float d[32];
            tc_ld32(tmem + lane_base + 32 * half, d);
#pragma unroll
            for (int kc = 0; kc < 4; kc++) {
                uint32_t w[4];
#pragma unroll
                for (int e = 0; e < 4; e++) {
                    const int j = 8 * kc + 2 * e, o = 32 * half + j;
                    w[e] = pack_bf16(fmaxf(d[j] + s.b0[o], 0.f), fmaxf(d[j + 1] + s.b0[o + 1], 0.f));
                }
                *reinterpret_cast<uint4*>(s.h + core_off(tid, 32 * half + 8 * kc, 8)) = make_uint4(w[0], w[1], w[2], w[3]);
            }
        }
        fence_async_smem();
        tc_before_sync();
        __syncthreads();
        // layer 1
        if (tid == 0) {
            tc_after_sync();
#pragma unroll
            for (int k = 0; k < 4; k++)
                tc_mma(tmem + 64, tc_desc(sh + 256 * k, 128, 1024), tc_desc(sw1 + 256 * k, 128, 1024), k > 0);
            tc_commit(&s.mbar);
        }
        ok = tc_wait_limited(&s.mbar, phase, wait_limit);
        phase ^= 1;
        if (__syncthreads_or(!ok)) {
            timed_out = true;
            break;
        }
        tc_after_sync();
        float z = 0.f;
#pragma unroll
        for (int half = 0; half < 2; half++) {
            float d[32];
            tc_ld32(tmem + lane_base + 64 + 32 * half, d);
#pragma unroll
            for (int j = 0; j < 32; j++) {
                const int o = 32 * half + j;
                z += bf16r(fmaxf(d[j] + s.b1[o], 0.f)) * s.w2[o];
            }
        }
        z += b2;
        bool fire = false;
        int cidx = 0;
        if (row < ncells) {
            if (logits) logits[row] = c ? 0.f : z;
            if (!c && z > thr) {
                const int l = 1 + (int)(row % g.lf), n = 1 + (int)(row / g.lf);
                cidx = (n + 3) * g.nx + (l + 3);
                order[cidx] = (int8_t)(g.mord - 2);
                fire = true;
            }
        }
        const unsigned m = __ballot_sync(0xffffffffu, fire);
        if (m) {  // warp-aggregated append to the gated-cell list
            int base = 0;
            if (lane == 0) {
                atomicAdd(count, (unsigned long long)__popc(m));
                base = atomicAdd(list_count, __popc(m));
            }
            base = __shfl_sync(0xffffffffu, base, 0);
            if (fire) list[base + __popc(m & ((1u << lane) - 1))] = cidx;
        }
        tc_before_sync();
        __syncthreads();  // X, H and the TMEM columns are rewritten by the next tile
    }
    if (timed_out && tid == 0) atomicOr(status, GPM_STATUS_TENSOR);
    tc_before_sync();
    __syncthreads();
    tc_after_sync();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_COLS));
}

__global__ void k_features(GridGeom g, const double* __restrict__ u, float* __restrict__ x, int8_t* __restrict__ cst) {
    const long long ncells = (long long)g.lf * g.nf;
    const long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= ncells) return;
    const int l = 1 + (int)(row % g.lf), n = 1 + (int)(row / g.lf);
    float f[36];
    const bool c = cell_features(g, u, l, n, f);
    for (int k = 0; k < 36; k++) x[row * 36 + k] = f[k];
    if (cst) cst[row] = c ? 1 : 0;
}

__device__ __forceinline__ unsigned hash3(unsigned a, unsigned b) {
    unsigned h = a * 0x9E3779B1u ^ (b + 0x7F4A7C15u + (a << 6) + (a >> 2));
    h ^= h >> 16; h *= 0x85EBCA6Bu; h ^= h >> 13; h *= 0xC2B2AE35u; h ^= h >> 16;
    return h;
}

__global__ void k_harvest(GridGeom g, const double* __restrict__ u, const int8_t* __restrict__ order, float* __restrict__ x,
                          float* __restrict__ y, int capacity, int* __restrict__ count, float keep_neg, unsigned seed) {
    const long long ncells = (long long)g.lf * g.nf;
    const long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= ncells) return;
    const int l = 1 + (int)(row % g.lf), n = 1 + (int)(row / g.lf);
    float f[36];
    if (cell_features(g, u, l, n, f)) return;  // constant stencils are never gated
    const int lab = order[(size_t)(n + 3) * g.nx + (size_t)(l + 3)] < g.mord ? 1 : 0;
    if (!lab) {
        const float r = (hash3((unsigned)row, seed) >> 8) * (1.0f / 16777216.0f);
        if (r >= keep_neg) return;
    }
    const int i = atomicAdd(count, 1);
    if (i >= capacity) return;
    for (int k = 0; k < 36; k++) x[(size_t)i * 36 + k] = f[k];
    y[i] = (float)lab;
}

// ---------------------------------------------------------------------------
// Training: forward + backward of 128 samples per CTA; gradients and loss
// accumulated with FP32 atomics into grad[] and *loss.

struct SmemTrain {
    SmemFwd f;
    __nv_bfloat16 w1t[64][HS];      // W1^T for dh1 = dh2 W1
    __nv_bfloat16 xt[K0][TS];       // x^T
    __nv_bfloat16 h1t[64][TS];      // h1^T
    __nv_bfloat16 dh1t[64][TS];     // dh1^T
    __nv_bfloat16 dh2t[64][TS];     // dh2^T
    float gw2[64], gb1[64], gb0[64];
    float gb2, loss;
};

__global__ void __launch_bounds__(THREADS) k_train(const float* __restrict__ p, const float* __restrict__ xin,
                                                const float* __restrict__ yin, int n, float pos_weight, float inv_n,
                                                float* __restrict__ grad, float* __restrict__ loss_out, int fwd_only,
                                                float* __restrict__ logits_out) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SmemTrain& s = *reinterpret_cast<SmemTrain*>(smem_raw);
    load_weights(s.f, p);
    for (int i = threadIdx.x; i < 64 * 64; i += blockDim.x) {
        const int o = i / 64, k = i % 64;
        s.w1t[k][o] = __float2bfloat16_rn(p[P_W1 + i]);
    }
    for (int i = threadIdx.x; i < 64; i += blockDim.x) s.gw2[i] = s.gb1[i] = s.gb0[i] = 0.f;
    if (threadIdx.x == 0) s.gb2 = s.loss = 0.f;
    const long long row = (long long)blockIdx.x * ROWS + threadIdx.x;
    const bool valid = row < n;
    if (threadIdx.x < ROWS) {
#pragma unroll
        for (int k = 0; k < K0; k += 2) {
            const float v0 = (valid && k < 36) ? xin[row * 36 + k] : 0.f;
            const float v1 = (valid && k + 1 < 36) ? xin[row * 36 + k + 1] : 0.f;
            *reinterpret_cast<uint32_t*>(&s.f.x[threadIdx.x][k]) = pack_bf16(v0, v1);
            s.xt[k][threadIdx.x] = __float2bfloat16_rn(v0);
            s.xt[k + 1][threadIdx.x] = __float2bfloat16_rn(v1);
        }
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int r0 = 16 * warp;
    WarpFwd f;
    warp_forward(s.f, r0, p[P_B2], f);
    // rows of this thread: r0+g (lo) and r0+g+8 (hi)
    const long long rlo = (long long)blockIdx.x * ROWS + r0 + g, rhi = rlo + 8;
    if (fwd_only) {  // no labels, gradients or loss in this mode (yin, grad, loss_out are null)
        if (t == 0) {
            if (rlo < n) logits_out[rlo] = f.logit_lo;
            if (rhi < n) logits_out[rhi] = f.logit_hi;
        }
        return;
    }
    float dz[2] = {0.f, 0.f};
    float lsum = 0.f;
    const float zz[2] = {f.logit_lo, f.logit_hi};
    const long long rr[2] = {rlo, rhi};
#pragma unroll
    for (int h = 0; h < 2; h++) {
        if (rr[h] < n) {
            const float z = zz[h], yv = yin[rr[h]];
            const float pz = 1.f / (1.f + expf(-z));
            // softplus(z) = max(z,0) + log1p(exp(-|z|)); BCE = pw*y*softplus(-z) + (1-y)*softplus(z)
            const float sp = fmaxf(z, 0.f) + log1pf(expf(-fabsf(z)));
            const float spn = sp - z;
            lsum += pos_weight * yv * spn + (1.f - yv) * sp;
            dz[h] = (pos_weight * yv * (pz - 1.f) + (1.f - yv) * pz) * inv_n;
        }
    }
    if (t == 0) atomicAdd(&s.loss, lsum);
    // Layer 3: grad w2, b2; dh2 = dz * w2 * relu'(a2).
    float gw2l[8][2], dh2[8][4];
#pragma unroll
    for (int j = 0; j < 8; j++) {
        const int c0 = 8 * j + 2 * t, c1 = c0 + 1;
        gw2l[j][0] = dz[0] * bf16r(fmaxf(f.a2[j][0], 0.f)) + dz[1] * bf16r(fmaxf(f.a2[j][2], 0.f));
        gw2l[j][1] = dz[0] * bf16r(fmaxf(f.a2[j][1], 0.f)) + dz[1] * bf16r(fmaxf(f.a2[j][3], 0.f));
        dh2[j][0] = f.a2[j][0] > 0.f ? dz[0] * s.f.w2[c0] : 0.f;
        dh2[j][1] = f.a2[j][1] > 0.f ? dz[0] * s.f.w2[c1] : 0.f;
        dh2[j][2] = f.a2[j][2] > 0.f ? dz[1] * s.f.w2[c0] : 0.f;
        dh2[j][3] = f.a2[j][3] > 0.f ? dz[1] * s.f.w2[c1] : 0.f;
    }
    // reduce gw2 and gb1 over the 8 row-groups of the warp (lanes with equal t)
#pragma unroll
    for (int j = 0; j < 8; j++) {
        float a = gw2l[j][0], b = gw2l[j][1];
        float c = dh2[j][0] + dh2[j][2], d = dh2[j][1] + dh2[j][3];
#pragma unroll
        for (int o = 4; o < 32; o <<= 1) {
            a += __shfl_xor_sync(0xffffffffu, a, o);
            b += __shfl_xor_sync(0xffffffffu, b, o);
            c += __shfl_xor_sync(0xffffffffu, c, o);
            d += __shfl_xor_sync(0xffffffffu, d, o);
        }
        if (g == 0) {
            atomicAdd(&s.gw2[8 * j + 2 * t], a);
            atomicAdd(&s.gw2[8 * j + 2 * t + 1], b);
            atomicAdd(&s.gb1[8 * j + 2 * t], c);
            atomicAdd(&s.gb1[8 * j + 2 * t + 1], d);
        }
    }
    {
        float b2s = dz[0] + dz[1];
#pragma unroll
        for (int o = 4; o < 32; o <<= 1) b2s += __shfl_xor_sync(0xffffffffu, b2s, o);
        if (lane == 0) atomicAdd(&s.gb2, b2s);
    }
    // dh2 as A fragments; dh1 = (dh2 W1) * relu'(a1)
    uint32_t dh2f[4][4];
#pragma unroll
    for (int kk = 0; kk < 4; kk++) {
        dh2f[kk][0] = pack_bf16(dh2[2 * kk][0], dh2[2 * kk][1]);
        dh2f[kk][1] = pack_bf16(dh2[2 * kk][2], dh2[2 * kk][3]);
        dh2f[kk][2] = pack_bf16(dh2[2 * kk + 1][0], dh2[2 * kk + 1][1]);
        dh2f[kk][3] = pack_bf16(dh2[2 * kk + 1][2], dh2[2 * kk + 1][3]);
    }
    float dh1[8][4];
#pragma unroll
    for (int j = 0; j < 8; j++) dh1[j][0] = dh1[j][1] = dh1[j][2] = dh1[j][3] = 0.f;
#pragma unroll
    for (int kk = 0; kk < 4; kk++)
#pragma unroll
        for (int j = 0; j < 8; j++)
            mma16816(dh1[j], dh2f[kk], ld32(&s.w1t[8 * j + g][16 * kk + 2 * t]),
                     ld32(&s.w1t[8 * j + g][16 * kk + 8 + 2 * t]));
#pragma unroll
    for (int j = 0; j < 8; j++) {
        const int c0 = 8 * j + 2 * t, c1 = c0 + 1;
        dh1[j][0] = f.a1[j][0] > 0.f ? dh1[j][0] : 0.f;
        dh1[j][1] = f.a1[j][1] > 0.f ? dh1[j][1] : 0.f;
        dh1[j][2] = f.a1[j][2] > 0.f ? dh1[j][2] : 0.f;
        dh1[j][3] = f.a1[j][3] > 0.f ? dh1[j][3] : 0.f;
        float c = dh1[j][0] + dh1[j][2], d = dh1[j][1] + dh1[j][3];
#pragma unroll
        for (int o = 4; o < 32; o <<= 1) {
            c += __shfl_xor_sync(0xffffffffu, c, o);
            d += __shfl_xor_sync(0xffffffffu, d, o);
        }
        if (g == 0) {
            atomicAdd(&s.gb0[c0], c);
            atomicAdd(&s.gb0[c1], d);
        }
        // transposed BF16 copies for the weight-gradient products
        const int rl = r0 + g, rh = rl + 8;
        s.dh2t[c0][rl] = __float2bfloat16_rn(dh2[j][0]);
        s.dh2t[c1][rl] = __float2bfloat16_rn(dh2[j][1]);
        s.dh2t[c0][rh] = __float2bfloat16_rn(dh2[j][2]);
        s.dh2t[c1][rh] = __float2bfloat16_rn(dh2[j][3]);
        s.dh1t[c0][rl] = __float2bfloat16_rn(dh1[j][0]);
        s.dh1t[c1][rl] = __float2bfloat16_rn(dh1[j][1]);
        s.dh1t[c0][rh] = __float2bfloat16_rn(dh1[j][2]);
        s.dh1t[c1][rh] = __float2bfloat16_rn(dh1[j][3]);
        s.h1t[c0][rl] = __float2bfloat16_rn(fmaxf(f.a1[j][0], 0.f));
        s.h1t[c1][rl] = __float2bfloat16_rn(fmaxf(f.a1[j][1], 0.f));
        s.h1t[c0][rh] = __float2bfloat16_rn(fmaxf(f.a1[j][2], 0.f));
        s.h1t[c1][rh] = __float2bfloat16_rn(fmaxf(f.a1[j][3], 0.f));
    }
    __syncthreads();
    // dW1[o][i] = sum_rows dh2[row][o] h1[row][i]: 4 x 8 tiles of 16x8, K = 128 rows.
    // dW0[o][f] = sum_rows dh1[row][o] x[row][f]:  4 x 6 tiles (f padded to 48).
    // 56 tiles spread over the CTA's 8 warps: warp w takes tiles w, w+8, ...
    for (int tile = warp; tile < 32 + 24; tile += THREADS / 32) {
        const bool w1t = tile < 32;
        const int mt = w1t ? tile / 8 : (tile - 32) / 6;
        const int nt = w1t ? tile % 8 : (tile - 32) % 6;
        const __nv_bfloat16(*A)[TS] = w1t ? s.dh2t : s.dh1t;
        const __nv_bfloat16(*B)[TS] = w1t ? s.h1t : s.xt;
        float acc[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int ks = 0; ks < ROWS / 16; ks++) {
            uint32_t a[4];
            a[0] = ld32(&A[16 * mt + g][16 * ks + 2 * t]);
            a[1] = ld32(&A[16 * mt + g + 8][16 * ks + 2 * t]);
            a[2] = ld32(&A[16 * mt + g][16 * ks + 8 + 2 * t]);
            a[3] = ld32(&A[16 * mt + g + 8][16 * ks + 8 + 2 * t]);
            mma16816(acc, a, ld32(&B[8 * nt + g][16 * ks + 2 * t]), ld32(&B[8 * nt + g][16 * ks + 8 + 2 * t]));
        }
        const int o0 = 16 * mt + g, o1 = o0 + 8, c0 = 8 * nt + 2 * t, c1 = c0 + 1;
        if (w1t) {
            atomicAdd(&grad[P_W1 + o0 * 64 + c0], acc[0]);
            atomicAdd(&grad[P_W1 + o0 * 64 + c1], acc[1]);
            atomicAdd(&grad[P_W1 + o1 * 64 + c0], acc[2]);
            atomicAdd(&grad[P_W1 + o1 * 64 + c1], acc[3]);
        } else {
            if (c0 < 36) {
                atomicAdd(&grad[P_W0 + o0 * 36 + c0], acc[0]);
                atomicAdd(&grad[P_W0 + o1 * 36 + c0], acc[2]);
            }
            if (c1 < 36) {
                atomicAdd(&grad[P_W0 + o0 * 36 + c1], acc[1]);
                atomicAdd(&grad[P_W0 + o1 * 36 + c1], acc[3]);
            }
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 64; i += blockDim.x) {
        atomicAdd(&grad[P_W2 + i], s.gw2[i]);
        atomicAdd(&grad[P_B1 + i], s.gb1[i]);
        atomicAdd(&grad[P_B0 + i], s.gb0[i]);
    }
    if (threadIdx.x == 0) {
        atomicAdd(&grad[P_B2], s.gb2);
        atomicAdd(loss_out, s.loss * inv_n);
    }
}

__global__ void k_adam(float* __restrict__ p, const float* __restrict__ gr, float* __restrict__ m, float* __restrict__ v,
                       float lr_t, float beta1, float beta2, float eps) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= NN_GATE_NPARAMS) return;
    const float gi = gr[i];
    const float mi = beta1 * m[i] + (1.f - beta1) * gi;
    const float vi = beta2 * v[i] + (1.f - beta2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr_t * mi / (sqrtf(vi) + eps);
}

}  // namespace

struct NnGate {
    float* params;
    float thr;
    bool loaded;
    int wait_limit;  // polls of the MMA waits before a timeout (0: ~1 s); a test hook
};

NnGate* nn_gate_create(const GridGeom&) {
    NnGate* n = new (std::nothrow) NnGate();
    if (!n) return nullptr;
    if (cudaMalloc(&n->params, sizeof(float) * NN_GATE_NPARAMS) != cudaSuccess) {
        delete n;
        return nullptr;
    }
    n->thr = 0.f;
    n->loaded = false;
    return n;
}

void nn_gate_destroy(NnGate* n) {
    if (!n) return;
    cudaFree(n->params);
    delete n;
}

int nn_gate_set(NnGate* n, const float* params, cudaStream_t s) {
    if (cudaMemcpyAsync(n->params, params, sizeof(float) * NN_GATE_NPARAMS, cudaMemcpyHostToDevice, s) != cudaSuccess)
        return -1;
    n->loaded = true;
    return 0;
}

void nn_gate_set_threshold(NnGate* n, float thr) { n->thr = thr; }
void nn_gate_set_wait_limit(NnGate* n, int polls) { n->wait_limit = polls; }

bool nn_gate_loaded(const NnGate* n) { return n && n->loaded; }

int nn_gate_orders(NnGate* n, const GridGeom& g, const double* uin, int8_t* order, unsigned long long* count,
                   int* list, int* list_count, float* logits, int* status, cudaStream_t s) {
    if (!n->loaded || g.mord < 3) return 0;
    const long long cells = (long long)g.lf * g.nf;
    const long long tiles = (cells + TC_THREADS - 1) / TC_THREADS;
    static std::atomic<int> nsms[GPM_MAX_DEVICES];
    const int dev = gpm_device();
    int nsm = nsms[dev].load(std::memory_order_relaxed);
    if (!nsm) {
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        if (nsm <= 0) nsm = 1;
        cudaFuncSetAttribute(k_gate, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM);
        nsms[dev].store(nsm, std::memory_order_relaxed);
    }
    // persistent: 4 CTAs per SM, each holding 128 of the SM's 512 TMEM columns
    const int blocks = (int)(tiles < 4LL * nsm ? tiles : 4LL * nsm);
    k_gate<<<blocks, TC_THREADS, TC_SMEM, s>>>(g, uin, n->params, n->thr, order, count, list, list_count, logits,
                                               status, n->wait_limit);
    return cudaGetLastError() == cudaSuccess ? 1 : -1;
}

int nn_features(const GridGeom& g, const double* uin, float* x, int8_t* is_const, cudaStream_t s) {
    const long long cells = (long long)g.lf * g.nf;
    k_features<<<(int)((cells + 255) / 256), 256, 0, s>>>(g, uin, x, is_const);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int nn_harvest(const GridGeom& g, const double* uin, const int8_t* order, float* x, float* y, int capacity, int* count,
               float keep_negative, unsigned seed, cudaStream_t s) {
    const long long cells = (long long)g.lf * g.nf;
    k_harvest<<<(int)((cells + 255) / 256), 256, 0, s>>>(g, uin, order, x, y, capacity, count, keep_negative, seed);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

static int train_launch(const float* p, const float* x, const float* y, int n, float pw, float* grad, float* loss,
                        int fwd_only, float* logits, cudaStream_t s) {
    if (n <= 0) return -1;
    const size_t sm = sizeof(SmemTrain);
    static std::atomic<bool> attr[GPM_MAX_DEVICES];
    const int dev = gpm_device();
    if (!attr[dev].load(std::memory_order_relaxed)) {
        cudaFuncSetAttribute(k_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        attr[dev].store(true, std::memory_order_relaxed);
    }
    k_train<<<(n + ROWS - 1) / ROWS, THREADS, sm, s>>>(p, x, y, n, pw, 1.0f / (float)n, grad, loss, fwd_only, logits);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int nn_forward(const float* params, const float* x, int n, float* logits, cudaStream_t s) {
    return train_launch(params, x, nullptr, n, 1.f, nullptr, nullptr, 1, logits, s);
}

int nn_loss_grad(const float* params, const float* x, const float* y, int n, float pos_weight, float* grad, float* loss,
                 cudaStream_t s) {
    if (cudaMemsetAsync(grad, 0, sizeof(float) * NN_GATE_NPARAMS, s) != cudaSuccess) return -1;
    if (cudaMemsetAsync(loss, 0, sizeof(float), s) != cudaSuccess) return -1;
    return train_launch(params, x, y, n, pos_weight, grad, loss, 0, nullptr, s);
}

int nn_adam(float* params, const float* grad, float* m, float* v, int step, float lr, float beta1, float beta2,
            float eps, cudaStream_t s) {
    const float lr_t = lr * sqrtf(1.f - powf(beta2, (float)step)) / (1.f - powf(beta1, (float)step));
    k_adam<<<(NN_GATE_NPARAMS + 255) / 256, 256, 0, s>>>(params, grad, m, v, lr_t, beta1, beta2, eps);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}
