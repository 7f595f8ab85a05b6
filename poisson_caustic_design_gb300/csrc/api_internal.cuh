// api_internal.cuh -- the context object behind pcd_ctx* (internal).
#pragma once

#include <map>
#include <mutex>
#include <set>
#include <vector>

#include "common.cuh"
#include "grid.cuh"
#include "solver.cuh"
#include "sor_batch.cuh"

namespace pcd {
// Settings the autotuner picked for one solve shape / batch signature.
struct TunedSolve {
    int check_every = 0, refine_every = 0, schedule = PCD_SCHED_AUTO;
    double refine_drop = 0.0;
};
struct TunedBatch {
    int cluster = 16, check_every = 0;
    double refine_drop = 0.0;
};
struct Autotuner {
    int enabled = 0;
    long long trials = 0;
    std::map<std::vector<long long>, TunedSolve> solves;
    std::map<std::vector<long long>, TunedBatch> batches;
    double *save = nullptr;  // phi snapshot between trials
    size_t save_cells = 0;
    void release();
};
}  // namespace pcd

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
    pcd::Autotuner tuner;
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
// solve_device through the context's autotuner (autotune.cu)
int solve_autotuned(pcd_ctx *ctx, const double *b, double *phi, int W, int H, int ld, const pcd_solve_opts &o,
                    pcd_solve_stats *stats, cudaStream_t s);
int batch_autotuned(pcd_ctx *ctx, const pcd_instance *inst, int count, const pcd_solve_opts &o,
                    pcd_instance_stats *stats, pcd_batch_stats *bstats, cudaStream_t s);
}  // namespace pcd
