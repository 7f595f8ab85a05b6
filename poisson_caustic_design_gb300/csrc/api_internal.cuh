// api_internal.cuh -- the context object behind pcd_ctx* (internal).
#pragma once

#include <mutex>
#include <set>

#include "common.cuh"
#include "grid.cuh"
#include "solver.cuh"
#include "sor_batch.cuh"

struct pcd_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    pcd::SolverWorkspace solver;
    pcd::GridScratch grid;
    pcd::BatchWorkspace batch;
    // device staging of the host-array entry points
    double *d_b = nullptr;
    double *d_phi = nullptr;
    size_t host_cells = 0;
    std::mutex mu;
    // designs created on this context; destroyed with it
    std::set<pcd_design *> designs;
};

namespace pcd {
int ctx_stage(pcd_ctx *ctx, size_t cells);
int ctx_activate(pcd_ctx *ctx);
}  // namespace pcd
