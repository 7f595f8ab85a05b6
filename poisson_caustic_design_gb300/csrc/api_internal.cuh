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
    // ordering between a caller's stream and `stream` (StreamJoin)
    cudaEvent_t join_in = nullptr, join_out = nullptr;
    // network of the learned warm start (not owned)
    pcd_unet *net = nullptr;
    // networks created on this context; their device state is released with it
    std::set<pcd_unet *> nets;
};

namespace pcd {
// Runs library work on the context's stream, ordered after everything the
// caller enqueued on `user` before the call and before everything it
// enqueues after it (user NULL = the CUDA default stream).
struct StreamJoin {
    pcd_ctx *ctx;
    cudaStream_t user, work;
    StreamJoin(pcd_ctx *c, void *stream) : ctx(c), user((cudaStream_t)stream), work(c->stream) {}
    int begin();
    int end();
};
int ctx_stage(pcd_ctx *ctx, size_t cells);
int ctx_activate(pcd_ctx *ctx);
int solve_with_warm_start(pcd_ctx *ctx, const double *b, double *phi, int W, int H, int ld, pcd_solve_opts o,
                          pcd_solve_stats *stats, cudaStream_t s);
}  // namespace pcd
