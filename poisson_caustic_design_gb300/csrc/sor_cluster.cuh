// sor_cluster.cuh -- FP32 red-black SOR on one thread-block cluster (internal).
#pragma once

#include "solver.cuh"

namespace pcd {

constexpr int kClusterThreads = 1024;

struct ClusterArgs {
    int W, H, ld;
    int khp;             // shared-memory row stride of a colour plane (multiple of 4)
    float *e;            // FP32 correction (global, ld-strided), in/out
    const float *r32;    // FP32 right-hand side
    Ctl *ctl;            // reads bnorm / rnorm / sweeps, writes sweeps / halt
    int check_every;     // sweeps between FP32 residual estimates
    int cycle_cap;       // sweeps per cycle at most
    int max_iter;        // total sweep cap
    double tol;          // relative stop tolerance
    double drop;         // end the cycle when the estimate fell by this factor
    float w32[5];        // omega / cnt
    float one_minus_omega;
    int depth;           // sweeps between halo exchanges (1, 2 or 4; 0: one exchange per half sweep)
};

// How one grid runs on one cluster: C CTAs (16 or 8), dynamic shared memory,
// the shared-memory plane stride, the sweeps per halo exchange (0: one
// exchange per half sweep) and, for the register-resident form, the rows per
// warp and quads per lane (rr_l = 0: the shared-memory forms).
struct ClusterPlan {
    int C;
    size_t smem;
    int khp;
    int depth;
    int rr_l;
    int rr_nq;
};

// The plan for a W x H grid; PCD_BAD_ARG when the grid does not fit in one
// cluster.  max_depth caps the sweeps per exchange (0: the per-half-sweep
// exchange; the register-resident form needs at least 2).
int cluster_plan(int dev, int W, int H, int max_depth, ClusterPlan *plan);
int launch_cluster(ClusterArgs &a, const ClusterPlan &p, cudaStream_t s);

// Register-resident tile passes for grids in HBM (FP32 correction sweeps,
// ping-pong buffers): K sweeps per pass, tiles of 16 L rows and 256 NQ
// columns (halo included), ncol x nrow tiles on `grid` persistent CTAs.
struct TilePlan {
    int K = 0, L = 0, NQ = 0;
    int ncol = 0, nrow = 0, grid = 0;
    size_t smem = 0;
};

// One grid of a batched tile pass (the 64 x 256-cell tile form, 4 sweeps per
// pass at most).
struct TileJob {
    float *ea, *eb;      // FP32 correction buffers (ping-pong)
    const float *r32;    // FP32 right-hand side
    Ctl *ctl;            // the grid's control block
    int W, H, ld;        // W a multiple of 8, ld of 4
    int ncol, nrow;      // tiles (tile_counts)
    int tile0;           // first global tile index of the grid
    int max_iter;
    float w32[5];        // omega / cnt
};
static_assert(sizeof(TileJob) % 8 == 0, "job table copied to shared memory in words");

// Tiles of a W x H grid in the batched form.
void tile_counts(int W, int H, int *ncol, int *nrow);
// Most grids in one batched pass (the job table sits in shared memory).
constexpr int kTileBatchJobsMax = 1024;
// Dynamic shared memory of the batched pass for njobs grids and its
// persistent grid.
int tile_batch_config(int dev, int njobs, size_t *smem, int *grid);
// One batched pass of nsw <= 4 sweeps over ntiles tiles of njobs grids
// (d_jobs on the device, tile0 ascending); parity par reads ea (0) or eb.
// counter: a device word that is zero between passes.
int launch_tile_batch(const TileJob *d_jobs, int njobs, int ntiles, int nsw, int par, int grid, size_t smem,
                      unsigned *counter, cudaStream_t s);

// The plan for a W x H grid with leading dimension ld (W a multiple of 8, ld
// of 4); depth = sweeps per pass (2 or 4; 0: 4).  PCD_BAD_ARG when no form
// applies.
int tile_plan(int dev, int W, int H, int ld, int depth, TilePlan *plan);
// One pass of nsw <= K sweeps from ein into eout (fewer at the sweep cap);
// track: the pass reports the largest |update| of its last sweep.
int launch_tile(const TilePlan &p, const float *ein, float *eout, const float *r32, Ctl *ctl, const SolveArgs &a,
                int nsw, int out_idx, bool track, cudaStream_t s);

}  // namespace pcd
