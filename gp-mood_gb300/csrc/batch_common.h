// batch_common.h -- many independent GP-MOOD problems of uneven size stepped
// together: one persistent launch per phase of an RK stage covers every
// problem, and a whole step is captured in one CUDA graph.
//
// All problems' padded grids are concatenated in one arena (cells in the
// layout of gpm_common.h, each problem at its own cell offset); face stores,
// order masks and stamps use the same offsets.  Troubled-cell lists hold
// (problem, padded cell index) pairs of every problem at once.
#pragma once
#include "gpm_common.h"

struct BProb {
    long long off;     // first cell of the problem's padded grid in the arena
    int lf, nf, nx, ny;
    double dx, dy;
    int wc, pad;       // index of the problem's GP weights in BatchArgs::wtab
};

// Per-problem scalars (one problem's DevScalars).
struct BScal {
    double t, dt, qx, qy, tmax, cfl;
    unsigned long long dtmin_bits;
    int status, pad;
};

// Work items.  Face tiles: (problem, direction, first face l, first face n);
// cell blocks: (problem, first interior cell in x-fastest order); padded-cell
// blocks: (problem, first padded cell).
struct BatchArgs {
    const BProb* prob;
    const GpWeights* wtab;  // one weight set per distinct grid size (device memory)
    BScal* sc;
    int nprob;
    int bc_type, ngp, mord, method, dmp, u2, u2_tol, num_flux;
    const double* uin;
    double* uout;
    double* fx;
    double* fy;
    int8_t* order;
    unsigned* stamp;
    int2* tlist[2];
    int* ntrb;            // [0..1] list counts, [2] pass epoch, [3] cap flag, [4] detected, [5] passes,
                          // [6] NaN or inadmissible state left in an order-1 cell (sticky)
    const int4* ftiles;
    int nftiles;
    const int4* etiles;   // edge items of the two-direction cell tiles
    int netiles;
    const int2* cblocks;
    int ncblocks;
    const int2* pblocks;
    int npblocks;
    int stage;            // 0, 1, 2 -> t_rk = t, t+dt, t+dt/2
    int tile;             // face-tile shape index chosen by the autotuner
    int mood_solo;        // as GridGeom::mood_solo
};

// Face-tile shapes (TX x TY faces per CTA) the autotuner chooses from.  The
// last one is the fast mode's two-direction cell tile (order 5, ngp = 3
// only): items (problem, 2, l0, n0) over the interior cells, with edge items
// (problem, 3, k0, 0) in BatchArgs::etiles for the faces whose low cell is a
// ghost.
#define GPM_NTILES 5
#define GPM_TILE_XY 4
static const int kTileTX[GPM_NTILES] = {32, 32, 16, 64, 32};
static const int kTileTY[GPM_NTILES] = {8, 4, 16, 4, 8};

struct BatchTable {
    void (*bc)(const BatchArgs& a, double* u, cudaStream_t s);
    void (*flux)(const BatchArgs& a, cudaStream_t s);
    void (*update)(const BatchArgs& a, cudaStream_t s);
    // one MOOD pass that reads the list count on the device and returns at
    // once when it is zero (so a fixed number of passes can be captured)
    void (*mood_pass)(const BatchArgs& a, int cur, cudaStream_t s);
    void (*leftover)(const BatchArgs& a, int cur, cudaStream_t s);
    void (*combine)(const BatchArgs& a, const double* x, double* y, double ca, double cb, int with_cfl,
                    cudaStream_t s);
    void (*cfl)(const BatchArgs& a, const double* u, cudaStream_t s);
    void (*dt_finalize)(const BatchArgs& a, cudaStream_t s);
    void (*advance_t)(const BatchArgs& a, cudaStream_t s);
    // the whole MOOD loop in one cooperative launch; -1 if the launch failed
    int (*mood_loop)(const BatchArgs& a, GridBar* bar, int max_pass, cudaStream_t s);
};

namespace gpm_exact { extern const BatchTable batch_table; void batch_set_max_nx(int nx); }
namespace gpm_fast { extern const BatchTable batch_table; void batch_set_max_nx(int nx); }
