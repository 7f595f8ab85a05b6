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
    int block_sweeps = 0;
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

namespace pcd {
// Result of the learned warm start's judge: whether the prediction was kept
// and the two smoothed relative residuals.
struct JudgeOut {
    int keep;
    int pad_;
    double rel_pred, rel_zero;
};

// The learned warm start and its judge (prediction, kLearnedSmooth Gauss-
// Seidel sweeps on it and on a zero guess -- FP32 sweeps on one cluster with
// the residuals in FP64 where the grid fits one cluster, FP64 half-sweep
// launches otherwise -- and both FP64 residuals) as one CUDA graph per grid
// shape and network, on buffers of its own: the caller's b is
// copied in before the replay and the chosen start copied out after it, so a
// solve with the learned warm start has no host round trip before the solver.
struct JudgeGraph {
    int W = 0, H = 0, ld = 0;
    const void *net = nullptr, *arena = nullptr;
    cudaGraphExec_t exec = nullptr;
    unsigned long long launches = 0;  // kernels per replay
    size_t cells = 0;
    double *b = nullptr, *pred = nullptr, *zero = nullptr, *partials = nullptr, *partials_z = nullptr;
    uint8_t *mask = nullptr, *mask_z = nullptr;
    float *e32 = nullptr, *r32 = nullptr;  // [2 * cells]: the mixed smoothing's correction and RHS per branch
    bool mixed = false;                   // the graph smooths in the mixed form (one cluster, FP32 sweeps)
    cudaStream_t side = nullptr;    // the zero guess's branch of the capture
    cudaEvent_t fork = nullptr, join = nullptr;
    Ctl *ctl = nullptr;             // [2]: zero guess, prediction
    JudgeOut *out = nullptr;        // device
    JudgeOut *out_host = nullptr;   // pinned
    cudaEvent_t done = nullptr;
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
    pcd::JudgeGraph judge;
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
