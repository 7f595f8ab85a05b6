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
    int depth;           // sweeps between halo exchanges (1 or 2; 0: one exchange per half sweep)
};

// Cluster size (16 or 8 CTAs), sweeps per halo exchange and dynamic shared
// memory for a W x H grid; PCD_BAD_ARG when the grid does not fit in one
// cluster.  max_depth caps the sweeps per exchange (0: the per-half-sweep
// exchange).
int cluster_plan(int dev, int W, int H, int max_depth, int *C_out, size_t *smem_out, int *khp_out, int *depth_out);
int launch_cluster(ClusterArgs &a, int C, size_t smem, cudaStream_t s);

}  // namespace pcd
