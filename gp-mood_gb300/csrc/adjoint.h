// adjoint.h -- vector-Jacobian product of one GP-MOOD RK stage with its order
// mask frozen (adjoint.cu), and the transpose of Boundary_C.
#pragma once
#include "gpm_common.h"

struct AdjArgs {
    GridGeom g;
    const double* u_in;     // stage input, ghosts filled by Boundary_C (padded layout)
    const int8_t* order;    // frozen CellGPO of the stage (padded)
    const double* lam_out;  // adjoint of the stage output (interior cells; ghosts zero)
    double* lam_in;         // adjoint of the stage input: interior written, ghosts untouched
    double* face_adj;       // scratch, 2 * ncell * 8 * GPM_MAXGP doubles
    double* mu_pad;         // scratch, ncell * 4 doubles
    double qx, qy;          // dt/dx, dt/dy of the step
};

// lam_in = lam_out + BC^T (dF/du_in)^T lam_out for periodic, Neumann and
// reflective boundaries.  Returns 0, or -1 if a launch failed.
int gpm_adj_stage(const AdjArgs& a, const GpWeights& w, cudaStream_t s);

// out(interior) = base(interior) + BC^T mu, where mu is a padded array that is
// overwritten (its interior rows receive the ghost rows' values).
int gpm_adj_fold(const GridGeom& g, double* mu, const double* base, double* out, cudaStream_t s);
