// sor_blocks.cuh -- persistent red-black SOR over 2-D blocks with deep halos
// (internal).
#pragma once

#include "solver.cuh"

namespace pcd {

// Threads of a block CTA: 16 warps, one CTA per SM.
constexpr int kBlocksThreads = 512;
// Columns of a block's region (owned columns plus the halo on both sides):
// one column pair per lane.
constexpr int kBlocksRegionCols = 64;

struct BlocksArgs {
    int W, H, ld;         // grid (phi, b, r64 have leading dimension ld)
    int TY, TX, G;        // block rows x block columns = CTAs
    int K;                // sweeps per halo exchange (h = 2K halo cells)
    int RTmax;            // most region rows of any block (owned + 2h)
    int xs;               // row stride of the exchange grids (even, >= W)
    const double *b;      // right-hand side (FP64 form)
    double *phi;          // solution, in/out
    double *r64;          // mixed: FP64 residual b - L phi, refreshed in place
    void *xb;             // exchange grids: 2 x H x xs elements of the sweep type
    float *r32x;          // mixed: FP32 right-hand side of every cell (H x xs)
    unsigned *flags;      // G epoch flags, then the grid barrier counter
    double *part;         // check partials: 2 x G x 3
    Ctl *ctl;
    int stop, max_iter, check_every, cycle_cap;
    double tol, drop;     // drop: mixed cycle ends once its FP32 estimate fell by this
    double omega;
    double w64[5];
    float w32[5];
    long long spin_limit;
    int withhold;         // failure test: CTA 0 never raises its epoch flag
};

// The block layout of a W x H grid with K sweeps per exchange: PCD_BAD_ARG
// when no layout fits (blocks narrower or shorter than the halo, or the
// shared planes beyond the opt-in limit).
struct BlocksPlan {
    int TY = 0, TX = 0, K = 0, RTmax = 0;
    size_t smem = 0;
};
int blocks_plan(int dev, int W, int H, int K, bool mixed, BlocksPlan *plan);
int launch_blocks(BlocksArgs &a, bool mixed, size_t smem, cudaStream_t s);

}  // namespace pcd
