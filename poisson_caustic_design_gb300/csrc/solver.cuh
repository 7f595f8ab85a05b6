// solver.cuh -- red-black SOR Poisson solver of libpcd_gb300 (internal).
//
// Solves  sum_nbr phi - cnt*phi = b  (the Neumann graph Laplacian of the
// reference, src/solver.cpp:29-47) on a W x H grid with leading dimension ld.
// A neighbour counts when it lies inside the grid and its b is not NaN.
#pragma once

#include <cuda_runtime.h>
#include <map>
#include <tuple>
#include <vector>

#include "common.cuh"

namespace pcd {

// Device-resident control block of one solve.  Flags are written only by the
// last block of a kernel (after every block of that kernel has finished) and
// read by later kernels, so no kernel races with its own writes.
struct Ctl {
    int halt;                    // no further sweeps
    int done;                    // solve finished (mixed: last correction folded in)
    int converged;               // stop test passed
    int sweeps;                  // full red+black sweeps done
    unsigned int blocks_done;    // last-block counter of the sweep kernels
    unsigned int blocks_done_r;  // last-block counter of the residual kernels
    int checks;                  // residual evaluations
    int nan_cells;               // NaN entries of b
    int error;                   // PCD_TIMEOUT when a bounded device wait gave up
    int stream_out;              // ping-pong buffer holding the latest FP32 correction
    unsigned long long maxbits;  // running max |delta| of the current sweep
    double last_max;             // max |delta| of the last full sweep
    double rnorm, bnorm, rmax, rel;
};

struct SolveArgs {
    int W, H, ld;
    int stop;         // pcd_stop
    int max_iter;
    double tol;
    double omega;
    double w64[5];   // omega / cnt for cnt = 0..4, divided once on the host
    float w32[5];    // the same in FP32 ((float)omega / cnt)
};

// End-of-sweep bookkeeping, run by the last block of the black half sweep
// (n sweeps done by a kernel that runs several).
__device__ __forceinline__ void end_of_sweep(Ctl *ctl, const SolveArgs &a, int n = 1)
{
    volatile Ctl *c = ctl;
    unsigned long long bits = atomicExch(&ctl->maxbits, 0ull);
    double mx = __longlong_as_double((long long)bits);
    c->last_max = mx;
    int s = c->sweeps + n;
    c->sweeps = s;
    if (a.stop == PCD_STOP_MAX_UPDATE && mx < a.tol) {
        c->converged = 1;
        c->halt = 1;
    }
    if (s >= a.max_iter) c->halt = 1;
    c->blocks_done = 0;
    __threadfence();
}

// omega > 0: used as given; omega == 0: the reference's 2/(1+pi/width)
// (solver.cpp:71); omega < 0: 2/(1+sin t) with cos t = (1+cos(pi/n))/2,
// n = max(width, height), the optimum for the Neumann operator (its slowest
// mode varies along one axis only, so the reference's value is too small).
double resolve_omega(double omega, int W, int H);

// Per-context workspace of the solver; grows on demand.
// A mixed-precision FP32 cycle hands over to the FP64 stop test once its
// FP32 residual estimate is below this fraction of the stop tolerance (the
// estimate's rounding error, ~1e-7 of the cycle's starting residual, is far
// below the margin; a cycle that ends just short runs one more check).
constexpr double kFp32StopFrac = 0.9;

struct SolverWorkspace {
    int dev = 0;
    size_t cells = 0;           // capacity in elements of the per-cell buffers
    uint8_t *mask = nullptr;    // neighbour-validity bits per cell
    float *e32 = nullptr;       // FP32 correction (mixed precision)
    float *e32b = nullptr;      // second FP32 correction buffer (ping-pong stream sweeps)
    float *r32 = nullptr;       // FP32 right-hand side of the correction equation
    double *partials = nullptr; // per-block reduction partials
    int max_partials = 0;
    Ctl *ctl = nullptr;         // device control block
    Ctl *ctl_host = nullptr;    // pinned copies, 2 slots
    cudaEvent_t ev[2] = {nullptr, nullptr};
    cudaEvent_t t0 = nullptr, t1 = nullptr, k0 = nullptr, k1 = nullptr;
    // persistent-kernel state
    double *r64 = nullptr;      // FP64 residual (mixed form)
    double *xbuf = nullptr;     // exchange rows
    size_t xbuf_elems = 0;
    unsigned *flags = nullptr;  // epoch flags + barrier counter
    int max_ctas = 0;
    int stripe_resident = 0;    // resident stripe blocks (SMs x blocks per SM)
    double *part = nullptr;     // check partials
    // bounded waits of the persistent schedule: polls before a flag wait gives
    // up (0: 2^24), and the failure test's withheld flag (pcd_ctx_set_wait_limit)
    long long wait_limit = 0;
    int withhold_flag = 0;
    // the block schedule's exchange grids (and the mixed form's FP32 rhs grid)
    void *bx = nullptr;
    size_t bx_bytes = 0;

    struct GraphEntry {
        cudaGraphExec_t exec;
        int nodes;
    };
    std::map<std::vector<long long>, GraphEntry> graphs;

    int reserve(size_t n);
    void release();
};

// Workspace of the batched tile solve (every grid of a batch in one tile
// pass per launch); grows on demand.
struct TileBatchWorkspace {
    float *arena = nullptr;     // [all e][all e'][all r32], each grid H x ld
    size_t arena_floats = 0;
    Ctl *ctl = nullptr;         // one control block per grid
    Ctl *ctl_host = nullptr;    // pinned, 2 slots of cap blocks
    double *partials = nullptr; // residual partials per grid
    void *jobs = nullptr;       // TileJob[cap] (device)
    void *rjobs = nullptr;      // refine descriptors [cap] (device)
    unsigned *counter = nullptr; // last-CTA counter of the batched pass
    int cap = 0;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    std::map<std::vector<long long>, cudaGraphExec_t> graphs;
    int reserve(size_t floats, int count);
    void release();
};

// Mixed-precision batch solve (relative-residual stop) on batched tile
// passes: every grid's width a multiple of 8 and ld of 4.  PCD_BAD_ARG
// without device work when a grid does not qualify.
int batch_tiles_solve(TileBatchWorkspace &ws, int dev, const pcd_instance *inst, int count, const pcd_solve_opts &o,
                      pcd_instance_stats *stats, pcd_batch_stats *bstats, cudaStream_t s);
bool batch_tiles_apply(const pcd_instance *inst, int count);

// ||b - L phi|| / ||b|| (FP64) of a given phi
int residual_rel(SolverWorkspace &ws, const double *b, const double *phi, int W, int H, int ld, cudaStream_t s,
                 double *rel);
int zero_grid(double *phi, int W, int H, int ld, cudaStream_t s);
// `sweeps` red-black sweeps with relaxation factor omega (FP64, NaN cells
// excluded as in the solver) on phi, then ||b - L phi|| / ||b||.
int smooth_residual(SolverWorkspace &ws, const double *b, double *phi, int W, int H, int ld, int sweeps, double omega,
                    cudaStream_t s, double *rel);
// The same without the host read: enqueues the sweeps and the residual on
// caller-owned buffers (mask: H * ld bytes, ctl: one block whose rel field
// receives the result, partials: residual_partials_bytes()); capturable.
int enqueue_smooth(const double *b, double *phi, uint8_t *mask, Ctl *ctl, double *partials, int W, int H, int ld,
                   int sweeps, double omega, cudaStream_t s);
size_t residual_partials_bytes();
// The same smoothing (Gauss-Seidel, omega = 1) in the mixed form: r = b - L
// phi in FP64, `sweeps` FP32 sweeps of L e = r on one thread-block cluster,
// then ||b - L (phi + e)|| / ||b|| in FP64 into ctl->rel and phi += e; for
// grids that fit one cluster (smooth_mixed_applies) and have no NaN cells
// (a NaN in b makes rel NaN).  e32, r32: H * ld floats.  Capturable.
int enqueue_smooth_mixed(const double *b, double *phi, float *e32, float *r32, Ctl *ctl, double *partials, int W,
                         int H, int ld, int sweeps, int dev, cudaStream_t s);
bool smooth_mixed_applies(int dev, int W, int H);

int solve_device(SolverWorkspace &ws, const double *b, double *phi, int W, int H, int ld,
                 const pcd_solve_opts &o, pcd_solve_stats *stats, cudaStream_t s);

}  // namespace pcd
