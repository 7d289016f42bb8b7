// nn_gate.h -- the a-priori MLP troubled-cell gate (method NN_GP_MOOD) and its
// training kernels.
//
// 36 features per interior cell: rho, rho*u, rho*v, E on the 9-point radius-2
// cross ((0,0), (-1,0), (1,0), (0,-1), (0,1), (-2,0), (2,0), (0,-2), (0,2)),
// each variable divided by its max-abs over the stencil, feature index
// v*9 + j.  MLP 36 -> 64 -> 64 -> 1 with ReLU hidden layers and a sigmoid
// output; BF16 operands with FP32 accumulation on the tensor cores
// (inference: tcgen05.mma with TMEM accumulators; training: mma.sync
// m16n8k16).  A positive prediction (logit > threshold) starts the cell at
// reduced order (mord - 2) before the first MOOD pass; the
// a-posteriori DETECTION stays on unchanged.  Cells whose stencil is constant
// in every variable are never gated, as in the reference's format_input
// (gp-mood-code/mod_append_NN_dataset.f90:96-114).  The gate's role is that of
// compute_CellGPO_with_NN (gp-mood-code/mod_NN.f90:14-58).
//
// Parameter vector (FP32, PyTorch flatten order): W0[64][36], b0[64],
// W1[64][64], b1[64], w2[64], b2.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "gpm_common.h"

#define NN_GATE_IN 36
#define NN_GATE_HID 64
#define NN_GATE_NPARAMS (NN_GATE_HID * NN_GATE_IN + NN_GATE_HID + NN_GATE_HID * NN_GATE_HID + NN_GATE_HID + NN_GATE_HID + 1)

struct NnGate;

NnGate* nn_gate_create(const GridGeom& g);
void nn_gate_destroy(NnGate* n);
// Upload FP32 parameters and pack the BF16 weight copies used by the kernels.
int nn_gate_set(NnGate* n, const float* params, cudaStream_t s);
void nn_gate_set_threshold(NnGate* n, float logit_threshold);
// Test hook: the gate's MMA waits give up after `polls` polls (0: ~1 s).
void nn_gate_set_wait_limit(NnGate* n, int polls);
bool nn_gate_loaded(const NnGate* n);
// Overwrite order[] of gated interior cells with mord-2; adds the number of
// gated cells to *count and appends their padded indices to list (running
// length *list_count); logits[lf*nf] (may be NULL) receives every interior
// cell's logit (0 for constant stencils).  The MLP runs on the tcgen05 tensor
// cores; a tensor-core wait that times out sets GPM_STATUS_TENSOR in *status.
// Returns the number of kernels launched, or -1.
int nn_gate_orders(NnGate* n, const GridGeom& g, const double* uin, int8_t* order, unsigned long long* count,
                   int* list, int* list_count, float* logits, int* status, cudaStream_t s);

// Features (FP32, [n][36]) and constant-stencil flags of every interior cell
// (x fastest), for callers that evaluate or train the network themselves.
int nn_features(const GridGeom& g, const double* uin, float* x, int8_t* is_const, cudaStream_t s);

// Append stage-1 training samples: features of every non-constant interior
// cell with label 1 if its final order is below mord; negatives are kept with
// probability keep_negative (hash of cell, seed).  *count is the running
// sample count on the device; samples beyond capacity are dropped.
int nn_harvest(const GridGeom& g, const double* uin, const int8_t* order, float* x, float* y, int capacity,
               int* count, float keep_negative, unsigned seed, cudaStream_t s);

// Forward pass of the network on features x[n][36] -> logits[n].
int nn_forward(const float* params, const float* x, int n, float* logits, cudaStream_t s);
// Mean binary cross-entropy with logits (positives weighted by pos_weight)
// and its gradient with respect to every parameter (grad[NN_GATE_NPARAMS]).
int nn_loss_grad(const float* params, const float* x, const float* y, int n, float pos_weight, float* grad,
                 float* loss, cudaStream_t s);
// One Adam step (bias-corrected) on params with moments m, v.
int nn_adam(float* params, const float* grad, float* m, float* v, int step, float lr, float beta1, float beta2,
            float eps, cudaStream_t s);
