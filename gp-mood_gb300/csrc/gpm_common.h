// gpm_common.h -- types shared by the GP-MOOD kernels and the C-ABI host code.
//
// Device layout (identical to the reference's U(4, lb:le, nb:ne)): one cell is
// four consecutive doubles (rho, rho*u, rho*v, E); cells run x-fastest over the
// padded grid of (lf+8) x (nf+8) cells, ngc = 4 ghost layers on every side.
// Cell (l, n) with l in [-3, lf+4] sits at linear index (n+3)*nx + (l+3).
//
// Face fluxes are stored per cell index of the face's low side:
//   Fx[ci(l,n)] = x-face between (l,n) and (l+1,n), l in [0,lf], n in [1,nf]
//   Fy[ci(l,n)] = y-face between (l,n) and (l,n+1), l in [1,lf], n in [0,nf]
// (the L_Flux_x / L_Flux_y of gp-mood-code/mod_FE.f90:30-31).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>

// Kernel attributes and occupancy-derived grid sizes belong to a device, so
// the launchers keep them per device index (at most GPM_MAX_DEVICES).
#define GPM_MAX_DEVICES 64
inline int gpm_device() {
    int d = 0;
    cudaGetDevice(&d);
    return d >= 0 && d < GPM_MAX_DEVICES ? d : 0;
}

#define GPM_NGC 4
#define GPM_MAXGP 5
#define GPM_MAXST 5  // RK stages of the longest integrator (SSP-RK4: 5 Forward_Euler calls)

// Mirror-symmetric split of the diamond stencil for ngp = 3.  The Gauss
// points of an x face (iL, iR) lie along y and those of a y face along x; the
// outer two are mirror images across the face's normal axis and the middle one
// is on it.  Stencil points on that axis are their own mirror images; the
// others form mirror pairs (m, m').  With S = q_m + q_m', D = q_m - q_m':
//   u_0 = A_0 + sum al*S + sum be*D,  u_2 = A_0 + sum al*S - sum be*D,
//   u_1 = A_1 + sum ga*S
// (A_g = sum of the axis points' weights times values), 32 FP64 operations
// per variable instead of 39.  Lists: [dir][k] (dir 0: x faces, 1: y faces),
// first the 13-point order, whose first entries are the 5-point order's.
__host__ __device__ constexpr int gpm_sym_axis(int dir, int k) {
    return dir == 0 ? (k == 0 ? 0 : k == 1 ? 1 : k == 2 ? 3 : k == 3 ? 10 : 12)
                    : (k == 0 ? 0 : k == 1 ? 2 : k == 2 ? 4 : k == 3 ? 9 : 11);
}
__host__ __device__ constexpr int gpm_sym_pair(int dir, int k, int side) {
    return dir == 0 ? (k == 0 ? (side ? 4 : 2) : k == 1 ? (side ? 5 : 6) : k == 2 ? (side ? 8 : 7) : (side ? 9 : 11))
                    : (k == 0 ? (side ? 3 : 1) : k == 1 ? (side ? 8 : 5) : k == 2 ? (side ? 7 : 6) : (side ? 12 : 10));
}
// Weights of a whole cell's face states on the symmetry components of its
// 13-point stencil (ngp = 3, order 5; fast first pass).  Under the mirrors
// x -> -x and y -> -y the stencil splits into orbits whose values combine
// into components Q: Q0 = q(0,0); Q1p/Q1m = q(-1,0) +/- q(1,0);
// Q2p/Q2m = q(-2,0) +/- q(2,0); Q3p/Q3m = q(0,-1) +/- q(0,1);
// Q4p/Q4m = q(0,-2) +/- q(0,2); for the corners a=(-1,-1), b=(1,-1),
// c=(-1,1), d=(1,1): Q5pp = a+b+c+d, Q5mp = (a-b)+(c-d), Q5pm = (a+b)-(c+d),
// Q5mm = (a-b)-(c-d).  x0 weighs them for the left face at Gauss point 0 in
// the order [Q0 Q1p Q2p Q3p Q4p Q5pp | Q1m Q2m Q5mp | Q3m Q4m Q5pm | Q5mm];
// the right face and Gauss point 2 follow by sign changes of the groups.  x1
// (Gauss point 1, on the face's axis) has [Q0 Q1p Q2p Q3p Q4p Q5pp | Q1m Q2m
// Q5mp].  y0/y1 do the same for the bottom face, with y1's second group
// [Q3m Q4m Q5pm].
struct GpOrbit {
    double x0[13], x1[9], y0[13], y1[9];
};

struct GpSym {
    double a0[5], a1[5];         // axis weights of Gauss points 0 and 1
    double al[4], be[4], ga[4];  // per pair: (z0_m + z0_m')/2, (z0_m - z0_m')/2, z1_m
};

// GP weights of GP_presim_sphere (gp-mood-code/GP_init.f90:254-268), passed to
// kernels by value so that they sit in the constant parameter bank.
struct GpWeights {
    double zt[3][4][GPM_MAXGP][13];  // [ord 1,3,5][face iL,iT,iR,iB][gauss pt][stencil pt]
    double gw[GPM_MAXGP];            // gauss_weight(ngp, :)
    double d2x[5], d2y[5];           // GP_d2x_sp(3,:), GP_d2y_sp(3,:)
    GpSym sym[3][4];                 // ngp = 3 split of zt (fast mode); zero otherwise
    GpOrbit orb;                     // ngp = 3 order-5 cell-wise split (fast mode); zero otherwise
};

struct GridGeom {
    int lf, nf, nx, ny;  // interior sizes and padded sizes (nx = lf + 8)
    double dx, dy;
    int bc_type, ngp, mord, method;
    int dmp, u2, u2_tol;
    int u2_fd;           // POL_MOOD: the U2 test's second derivatives are the 3-point differences
                         // D2O2/dx^2 (mod_subroutine_MOOD.f90:81-84) instead of the GP weights
    int num_flux;        // 100 HLLC, 101 LLF, 102 HLL, 103 unsplit
    int mood_solo;       // device MOOD loop: lists of at most this many cells run in one CTA
    int flux_tma;        // fast first pass: halo tiles staged by a TMA bulk tensor copy (1) or loads (0)
    int solo_split;      // one-CTA MOOD passes: DETECTION split over warp roles (1) or per cell (0)
    int cc_col;          // NN_GP_MOOD_CC: the column l whose order-3 states are blended (-1: none)
};

// Default of GridGeom::mood_solo; the environment variable GPMOOD_MOOD_SOLO
// overrides it (tuning only: results do not depend on it).
int gpm_mood_solo_default();

// Default of GridGeom::flux_tma (1); the environment variable GPMOOD_FLUX_TMA=0
// selects the plain-load staging (A/B timing only: the staged tile, and so
// every result, is the same either way).  Read at context creation.
int gpm_flux_tma_default();

// Default of GridGeom::solo_split (1); GPMOOD_SOLO_SPLIT=0 keeps DETECTION on
// one thread per cross cell (A/B timing only: the decisions are the same).
int gpm_solo_split_default();

// Scalars that stay on the device across a step.
struct DevScalars {
    double t, dt, qx, qy;             // time, step, dt/dx, dt/dy
    double tmax, cfl;
    unsigned long long dtmin_bits;    // Setdt reduction slot (bits of a positive double)
    int ntrb[2];                      // troubled-cell counts, double-buffered lists
    int status;                       // GPMOOD status bits
    int passes_stage[GPM_MAXST];      // MOOD passes of each RK stage of the last step (device loop)
    unsigned stamp_epoch;             // first unused pass stamp of the device MOOD loop
    unsigned long long detected_step; // count_detected_cell of the current step
    unsigned long long apriori_step;
    double bcd[4][4];                 // Dirichlet BC (19): the right ghost columns' states, from the host
};

enum { GPM_STATUS_NAN = 1, GPM_STATUS_MOODCAP = 2, GPM_STATUS_DT = 4, GPM_STATUS_BARRIER = 8,
       GPM_STATUS_TENSOR = 16,  // a tensor-core (tcgen05) wait timed out
       GPM_STATUS_TMA = 32 };   // a TMA tile copy's mbarrier wait timed out

// Grid barrier state of the cooperative MOOD-loop kernel (zeroed device memory).
struct GridBar {
    unsigned count, gen;
    int err;
    int limit;  // polls a waiting CTA makes before it gives up; 0: the default, ~1 s (test hook)
};

// Launch-time arguments of one RK stage.
struct StageArgs {
    GridGeom g;
    const double* uin;     // stage input (BC applied)
    double* uout;          // stage output
    double* fx;            // face flux stores (4 doubles per face)
    double* fy;
    int8_t* order;         // CellGPO per padded cell
    unsigned* stamp;       // per-cell pass stamps (dedup of the dirty set)
    int* tlist[2];         // troubled-cell lists (padded linear indices)
    DevScalars* sc;
    int uniform_order;     // 1: every cell starts at mord (plain GP-MOOD)
    int stage;             // 0, 1, 2 -> t_rk = t, t+dt, t+dt/2
    const float* ccw;      // NN_GP_MOOD_CC: (v1, v2) of column g.cc_col per row n (2 floats per row
                           // 0..nf+1); NULL: no blend (every other method, and warm-up steps)
};

// Host-side launchers implemented once per floating-point variant
// (stage_kernels.cu compiled with and without FMA contraction).
struct KernelTable {
    void (*bc)(const GridGeom& g, double* u, const DevScalars* sc, int stage, cudaStream_t s);
    int (*flux_all)(const StageArgs& a, const GpWeights& w, cudaStream_t s);  // returns the launches made
    void (*update_detect)(const StageArgs& a, const GpWeights& w, int cur, cudaStream_t s);
    // the faces of the listed cells tlist[cur] at their current orders (the gate's fix-up)
    void (*mood_faces)(const StageArgs& a, const GpWeights& w, int cur, int max_trb, cudaStream_t s);
    void (*combine)(const GridGeom& g, const double* x, double* y, double a, double b, int with_cfl,
                    DevScalars* sc, cudaStream_t s);
    void (*cfl)(const GridGeom& g, const double* u, DevScalars* sc, cudaStream_t s);
    void (*dt_finalize)(const GridGeom& g, DevScalars* sc, double dtfinal, cudaStream_t s);
    void (*advance_t)(DevScalars* sc, cudaStream_t s);
    // MOOD passes 2, 3, ... of RK stage `stage` in one cooperative launch; the
    // pass count goes to sc->passes_stage[stage]; returns -1 if the launch failed
    int (*mood_loop)(const StageArgs& a, const GpWeights& w, GridBar* bar, int max_pass, int stage,
                     cudaStream_t s);
    // y = sum c[i]*x[i], i < n <= 5, left to right; optionally the Setdt reduction of y
    void (*lincomb)(const GridGeom& g, double* y, int n, const double* const* x, const double* c, int with_cfl,
                    DevScalars* sc, cudaStream_t s);
    // the gate's extras repair on the gated list tlist[1] (at most max_items cells)
    void (*gate_repair)(const StageArgs& a, const GpWeights& w, int max_items, cudaStream_t s);
};

namespace gpm_exact { extern const KernelTable table; }
namespace gpm_fast { extern const KernelTable table; }

// Store a message in the calling thread's error buffer (gpmood_last_error(NULL, ...)).
void gpm_set_thread_error(const char* msg);

// real(L_16/n, PR): the cell size rounded once from binary128 (global_variables.f90:86-88).
double gpm_cell_size(double length, int n);

// Host GP precompute (gp_weights.cpp).  Returns 0 or -1 on bad knobs.
extern "C" int gpm_gp_presim(double ell_o_dx, double lx, double ly, int lf, int nf, int mord, int ngp,
                             GpWeights* out, double inv_err[3]);
