// nn_ref.h -- the reference's own a-priori network (mod_NN.f90:14-58), used
// by method NN_GP_MOOD when gpmood_params.nn_reference = 1 (nn_ref.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "gpm_common.h"

struct NnRef;

NnRef* nn_ref_create();
void nn_ref_destroy(NnRef* r);
// Inputs of the network for a maximal order: 4 x the R+1 stencil (Mord 3: 52,
// Mord 5: 100); 0 if the reference has no network for that order.
int nn_ref_inputs(int mord);
// Hidden width of a parameter vector of n values for L inputs, or 0.
int nn_ref_hidden(int n, int L);
// Upload W0[len][L], b0[len], W1[len][len], b1[len], W2[2][len], b2[2]
// (the reference's text-file order); 0, -1 bad size, -2 CUDA error.
int nn_ref_set(NnRef* r, const float* params, int n, int mord, cudaStream_t s);
bool nn_ref_loaded(const NnRef* r);
// CellGPO of every interior cell (1 or 3) from the network on uin; adds the
// cells set to 1 to *count; logits[2*cell] = r(1), r(2) if logits != NULL.
// ccw != NULL selects NN_GP_MOOD_CC: r passes through softmax (logits hold
// values_NN, (0, 1) for constant stencils) and ccw[2n..2n+1], n = 1..nf,
// receives the pair of the row's last cell.  Returns the number of kernels
// launched, or -1.
int nn_ref_orders(NnRef* r, const GridGeom& g, const double* uin, int8_t* order, unsigned long long* count,
                  float* logits, float* ccw, cudaStream_t s);
