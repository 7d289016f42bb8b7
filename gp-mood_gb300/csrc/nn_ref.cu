// nn_ref.cu -- the reference's own a-priori network (method NN_GP_MOOD with
// gpmood_params.nn_reference = 1): compute_CellGPO_with_NN, format_input and
// forward of gp-mood-code/mod_NN.f90:14-58,168-183 and
// mod_append_NN_dataset.f90:81-125.
//
// Per interior cell: the conserved variables of the R+1 stencil
// (ixiy_sp1(Mord+2, :), GP_init.f90:270-355: 13 points for Mord 3, 25 for
// Mord 5) rounded to FP32, variable fastest (L = 4 * points inputs, raw, no
// scaling).  A stencil whose every variable spans less than 1e-10 is
// constant: CellGPO = 3.  Otherwise x0 = sigmoid(W0 x + b0),
// x1 = sigmoid(W1 x0 + b1), r = W2 x1 + b2 in FP32 (sigmoid 1/(1+exp(-x)) in
// FP32, constants.f90:65); r(1) > r(2) sets CellGPO = 1 and counts an
// a-priori detection, else CellGPO = 3.  Sums run in index order without FMA
// contraction.  With the convex-combination method (NN_GP_MOOD_CC) the
// outputs pass through softmax first (forward, mod_NN.f90:181) and the
// decision compares the softmaxed pair; every row n also leaves the pair of
// its last cell (l = lf; (0, 1) for a constant stencil) in ccw[2n..2n+1]:
// the reference stores each cell's pair in values_NN(L, n, :), L the input
// count (mod_NN.f90:41,44), so the last write of the row stays.
#include <cuda_runtime.h>

#include <new>

#include "nn_ref.h"

namespace {

constexpr int THREADS = 128;

// ixiy_sp1 offsets (dx, dy) of points 1..25, GP_init.f90:274-353.
__constant__ int kOx[25] = {0, -1, 0, 1, 0, -1, -1, 1, 1, 0, -2, 0, 2, -3, -2, -1, 0, 1, 2, 3, 2, 1, 0, -1, -2};
__constant__ int kOy[25] = {0, 0, 1, 0, -1, -1, 1, 1, -1, -2, 0, 2, 0, 0, 1, 2, 3, 2, 1, 0, -1, -2, -3, -2, -1};

__device__ __forceinline__ float sigmoid_ref(float x) {
    return __fdiv_rn(1.0f, __fadd_rn(1.0f, expf(-x)));
}

// Weights in shared memory: W0[len][L], b0[len], W1[len][len], b1[len], W2[2][len], b2[2].
__global__ void __launch_bounds__(THREADS) k_nn_ref(GridGeom g, const double* __restrict__ u,
                                                    const float* __restrict__ p, int len, int npts,
                                                    int8_t* __restrict__ order, unsigned long long* __restrict__ count,
                                                    float* __restrict__ logits, float* __restrict__ ccw) {
    extern __shared__ float w[];
    const int L = 4 * npts;
    const int nparam = len * L + len + len * len + len + 2 * len + 2;
    for (int i = threadIdx.x; i < nparam; i += blockDim.x) w[i] = p[i];
    __syncthreads();
    const float* W0 = w;
    const float* b0 = W0 + len * L;
    const float* W1 = b0 + len;
    const float* b1 = W1 + len * len;
    const float* W2 = b1 + len;
    const float* b2 = W2 + 2 * len;
    const long long ncells = (long long)g.lf * g.nf;
    for (long long cell = (long long)blockIdx.x * blockDim.x + threadIdx.x; cell < ncells;
         cell += (long long)gridDim.x * blockDim.x) {
        const int l = 1 + (int)(cell % g.lf), n = 1 + (int)(cell / g.lf);
        float x[100];
        bool cst = true;
        float mx[4], mn[4];
        for (int j = 0; j < npts; j++) {
            const size_t c = (size_t)(n + kOy[j] + 3) * g.nx + (size_t)(l + kOx[j] + 3);
            for (int k = 0; k < 4; k++) {
                const float v = (float)u[4 * c + k];
                x[4 * j + k] = v;
                if (j == 0) {
                    mx[k] = v;
                    mn[k] = v;
                } else {
                    mx[k] = fmaxf(mx[k], v);
                    mn[k] = fminf(mn[k], v);
                }
            }
        }
        for (int k = 0; k < 4; k++)
            if (!((double)__fsub_rn(mx[k], mn[k]) < 1e-10)) cst = false;
        const size_t ci = (size_t)(n + 3) * g.nx + (size_t)(l + 3);
        if (cst) {
            order[ci] = 3;
            if (logits) {
                logits[2 * cell] = 0.0f;
                logits[2 * cell + 1] = ccw ? 1.0f : 0.0f;
            }
            if (ccw && l == g.lf) {
                ccw[2 * n] = 0.0f;
                ccw[2 * n + 1] = 1.0f;
            }
            continue;
        }
        float h0[128], r0 = b2[0], r1 = b2[1];
        for (int i = 0; i < len; i++) {
            float s = 0.0f;
            for (int j = 0; j < L; j++) s = __fadd_rn(s, __fmul_rn(W0[i * L + j], x[j]));
            h0[i] = sigmoid_ref(__fadd_rn(s, b0[i]));
        }
        float s0 = 0.0f, s1 = 0.0f;
        for (int i = 0; i < len; i++) {
            float s = 0.0f;
            for (int j = 0; j < len; j++) s = __fadd_rn(s, __fmul_rn(W1[i * len + j], h0[j]));
            const float h1 = sigmoid_ref(__fadd_rn(s, b1[i]));
            s0 = __fadd_rn(s0, __fmul_rn(W2[i], h1));
            s1 = __fadd_rn(s1, __fmul_rn(W2[len + i], h1));
        }
        r0 = __fadd_rn(s0, r0);
        r1 = __fadd_rn(s1, r1);
        if (ccw) {  // softmax, mod_NN.f90:132-145
            const float e0 = expf(r0), e1 = expf(r1), d = __fadd_rn(e0, e1);
            r0 = __fdiv_rn(e0, d);
            r1 = __fdiv_rn(e1, d);
            if (l == g.lf) {
                ccw[2 * n] = r0;
                ccw[2 * n + 1] = r1;
            }
        }
        if (logits) {
            logits[2 * cell] = r0;
            logits[2 * cell + 1] = r1;
        }
        if (r0 > r1) {
            order[ci] = 1;
            atomicAdd(count, 1ull);
        } else {
            order[ci] = 3;
        }
    }
}

}  // namespace

struct NnRef {
    float* params = nullptr;
    int len = 0, npts = 0;
};

NnRef* nn_ref_create() { return new (std::nothrow) NnRef(); }

void nn_ref_destroy(NnRef* r) {
    if (!r) return;
    cudaFree(r->params);
    delete r;
}

int nn_ref_inputs(int mord) { return mord == 3 ? 4 * 13 : (mord == 5 ? 4 * 25 : 0); }

int nn_ref_hidden(int n, int L) {
    // n = len*L + len + len*len + len + 2*len + 2 = len^2 + (L+4)*len + 2
    for (int len = 1; len <= 128; len++)
        if (len * len + (L + 4) * len + 2 == n) return len;
    return 0;
}

int nn_ref_set(NnRef* r, const float* params, int n, int mord, cudaStream_t s) {
    const int L = nn_ref_inputs(mord);
    const int len = L ? nn_ref_hidden(n, L) : 0;
    if (!len) return -1;
    cudaFree(r->params);
    r->params = nullptr;
    if (cudaMalloc(&r->params, sizeof(float) * n) != cudaSuccess) return -2;
    if (cudaMemcpyAsync(r->params, params, sizeof(float) * n, cudaMemcpyHostToDevice, s) != cudaSuccess) return -2;
    r->len = len;
    r->npts = L / 4;
    return 0;
}

bool nn_ref_loaded(const NnRef* r) { return r && r->params && r->len > 0; }

int nn_ref_orders(NnRef* r, const GridGeom& g, const double* uin, int8_t* order, unsigned long long* count,
                  float* logits, float* ccw, cudaStream_t s) {
    if (!nn_ref_loaded(r)) return -1;
    const int L = 4 * r->npts;
    const size_t sm = sizeof(float) * ((size_t)r->len * L + r->len * r->len + 4 * r->len + 2);
    static size_t attr = 0;
    if (sm > attr) {
        cudaFuncSetAttribute(k_nn_ref, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        attr = sm;
    }
    const long long cells = (long long)g.lf * g.nf;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long want = (cells + THREADS - 1) / THREADS;
    const int blocks = (int)(want < 4LL * sms ? want : 4LL * sms);
    k_nn_ref<<<blocks, THREADS, sm, s>>>(g, uin, r->params, r->len, r->npts, order, count, logits, ccw);
    return cudaGetLastError() == cudaSuccess ? 1 : -1;
}
