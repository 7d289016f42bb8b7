// nn_gate.cu -- a-priori MLP gate (see nn_gate.h).
#include "nn_gate.h"

struct NnGate {
    int unused;
};

NnGate* nn_gate_create(const GridGeom&) { return nullptr; }
void nn_gate_destroy(NnGate* n) { delete n; }
int nn_gate_set(NnGate*, const float*, cudaStream_t) { return -1; }
int nn_gate_orders(NnGate*, const GridGeom&, const double*, int8_t*, unsigned long long*, cudaStream_t) { return -1; }
