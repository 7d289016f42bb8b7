// nn_gate.h -- the a-priori MLP troubled-cell gate (method NN_GP_MOOD).
//
// 36 features per interior cell (rho, rho*u, rho*v, E on the 9-point radius-2
// cross, each variable scaled by its stencil max-abs), a 36-64-64-1 MLP with
// ReLU hidden layers and a sigmoid output, BF16 operands with FP32
// accumulation on the tensor cores.  A positive prediction starts the cell at
// reduced order (5 -> 3) before the first MOOD pass; the a-posteriori
// DETECTION stays on unchanged.  The gate's role matches compute_CellGPO_with_NN
// (gp-mood-code/mod_NN.f90:14-58), with the feature set and network of the
// GB300 design instead of the reference's 52-input sigmoid MLP.
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
// Upload FP32 parameters (w0[64][36], b0[64], w1[64][64], b1[64], w2[64], b2).
int nn_gate_set(NnGate* n, const float* params, cudaStream_t s);
// Overwrite the interior of order[] with mord-2 where the gate fires; adds the
// number of gated cells to *count.  Returns nonzero on a launch error.
int nn_gate_orders(NnGate* n, const GridGeom& g, const double* uin, int8_t* order, unsigned long long* count,
                   cudaStream_t s);
