/*
 * pcd.h -- C ABI of the GB300 (sm_103a) Poisson caustic-design library
 * (libpcd_gb300.so).
 *
 * Plain C types only: pointers, sizes, enums and small POD structs.  Every
 * entry point returns a pcd_status; none exits the process or falls back to a
 * CPU path.  Grids are row-major doubles g[y*ld + x] (the reference's
 * vector<vector<double>> g[y][x]); mesh points are n x 3 doubles (x, y, z).
 *
 * The interfaces replaced, by reference file:line (dylanmsu/poisson_caustic_design):
 *   pcd_poisson_solver           <- poisson_solver()            src/solver.h:8, src/solver.cpp:70-148
 *   pcd_poisson_solve(_device)   <- same, with explicit options/statistics (new surface)
 *   pcd_subtract_average_device  <- subtractAverage()           src/utils.h:13, src/utils.cpp:60-86
 *   pcd_gradient_device          <- calculate_gradient()        src/utils.h:18, src/utils.cpp:3-20
 *   pcd_divergence_device        <- calculate_divergence()      src/utils.h:19, src/utils.cpp:22-39
 *   pcd_design_*                 <- class Caustic_design        src/caustic_design.h:7-66
 *       pcd_design_create            set_mesh_resolution / set_domain_resolution /
 *                                    set_mesh_size / set_lens_focal_length /
 *                                    set_lens_thickness     caustic_design.h:53-58
 *       pcd_design_initialize        initialize_solvers()   caustic_design.cpp:334-364
 *       pcd_design_transport_iteration perform_transport_iteration() caustic_design.cpp:190-266
 *       pcd_design_height_iteration  perform_height_map_iteration() caustic_design.cpp:269-332
 *       pcd_design_get_grid / _get_vertices  the public members phi, h, raster,
 *                                    divergence, norm_x, norm_y, errors, target_areas,
 *                                    mesh->target_points / source_points (caustic_design.h:16-30,
 *                                    mesh.h:51-52)
 */
#ifndef PCD_H
#define PCD_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    PCD_OK = 0,
    PCD_NOT_CONVERGED = 1,   /* stopped at max_iterations (the reference stops silently) */
    PCD_BAD_ARG = 2,
    PCD_DEVICE_ERROR = 3,    /* a CUDA call failed; pcd_last_error() has the text */
    PCD_TIMEOUT = 4,         /* a bounded device-side wait gave up */
    PCD_RASTER_MISS = 5,     /* a grid sample fell in no triangle (the reference calls exit(0)) */
    PCD_NO_DEVICE = 6,
    PCD_FALLBACK_USED = 7,   /* learned warm start rejected; solved from a zero guess */
    PCD_MESH_SMOOTHED = 8    /* transport iteration: a raster miss was handled by Laplacian smoothing
                                of the target mesh (raster_miss_policy 1); step is NaN */
} pcd_status;

typedef enum {
    /* max |delta| of one sweep below tol: the reference's test (solver.cpp:142) */
    PCD_STOP_MAX_UPDATE = 0,
    /* ||b - L phi||_2 / ||b||_2 <= tol, evaluated in FP64 */
    PCD_STOP_REL_RESIDUAL = 1
} pcd_stop;

typedef enum {
    PCD_PREC_FP64 = 0,       /* FP64 red-black SOR sweeps */
    PCD_PREC_MIXED = 1       /* FP32 sweeps on the error equation, FP64 residual/update */
} pcd_precision;

typedef struct {
    int max_iterations;      /* sweep cap (reference callers pass 100000) */
    double tol;              /* threshold of `stop` */
    int stop;                /* pcd_stop */
    int precision;           /* pcd_precision */
    double omega;            /* relaxation factor: > 0 as given; 0 the reference's 2/(1+pi/width)
                                (solver.cpp:71); < 0 the optimum for the Neumann operator,
                                2/(1+sin t) with cos t = (1+cos(pi/max(width,height)))/2 */
    int check_every;         /* sweeps between stop tests; 0 = auto.  The launch schedule tests
                                max |delta| after every sweep; the persistent one every
                                check_every sweeps (default 8 FP64 / 16 mixed), so it may run
                                up to check_every-1 sweeps past the first passing sweep */
    int refine_every;        /* FP32 sweeps between FP64 residual replacements (mixed); 0 = auto */
    int warm_start;          /* pcd_warm_start: 1 phi holds the initial guess (reference
                                behaviour); 0 start at 0; 2 the learned prediction */
    int schedule;            /* pcd_schedule */
    double refine_drop;      /* mixed precision, cluster and batch schedules: an FP32 cycle ends
                                once its residual estimate fell by this factor (then the FP64
                                residual is refreshed); 0 = auto (3e-2) */
    int block_sweeps;        /* block schedule: sweeps between halo exchanges, 1..8 (halo of
                                2 x that many cells); 0 = auto (FP64 4, FP32 8) */
} pcd_solve_opts;

typedef enum {
    PCD_WARM_ZERO = 0,
    PCD_WARM_GIVEN = 1,
    /* the context's network (pcd_ctx_set_warm_start_net) predicts phi from b;
     * after 8 Gauss-Seidel sweeps the prediction is kept if its residual is
     * below that of a zero guess after the same sweeps, otherwise the solve
     * starts from zero (stats->warm_used = 3) */
    PCD_WARM_LEARNED = 2
} pcd_warm_start;

typedef enum {
    PCD_SCHED_AUTO = 0,        /* FP32 sweeps: cluster, else tiles (grids of at least 64 x 64
                                  cells), else persistent, else stream; FP64: persistent, else
                                  stripes; else launches, as the grid allows */
    PCD_SCHED_LAUNCHES = 1,    /* one kernel per half sweep, CUDA-graph chunks (any grid) */
    PCD_SCHED_PERSISTENT = 2,  /* one cooperative launch per solve, bands in shared memory
                                  (no NaN cells, band fits on chip) */
    PCD_SCHED_CLUSTER = 3,     /* mixed precision with the relative-residual stop: FP32 sweeps
                                  on one 16-CTA cluster (grid fits in its shared memory),
                                  FP64 defect correction on all SMs between cycles */
    PCD_SCHED_STRIPES = 4,     /* grids in HBM without NaN cells: one fused red+black pass per
                                  sweep (row stripes walked top-down, in place), CUDA-graph
                                  chunks; AUTO picks it for FP64 sweeps when the on-chip
                                  schedules do not fit */
    PCD_SCHED_STREAM = 5,      /* mixed precision, grids in HBM without NaN cells, ld a multiple
                                  of 4, W <= 4096: passes of one or two sweeps from one FP32
                                  correction buffer into another (row window in registers,
                                  stripe edges recomputed, no boundary pass); AUTO picks it for
                                  FP32 sweeps when neither the on-chip schedules nor the tile
                                  passes apply */
    PCD_SCHED_TILES = 6,       /* mixed precision, grids in HBM without NaN cells, width a multiple
                                  of 8, ld of 4: passes of up to 4 FP32 sweeps from one correction
                                  buffer into another, each tile of the grid held in registers
                                  for the whole pass (halo recomputed); check_every = sweeps per
                                  pass, i.e. between stop tests (1..4, 0 = 4), so the max |delta|
                                  stop may come up to 3 sweeps after the first passing sweep;
                                  AUTO picks it for FP32 sweeps when the cluster schedule does
                                  not apply */
    PCD_SCHED_BLOCKS = 7       /* grids without NaN cells: one cooperative launch per solve on
                                  2-D blocks (one per SM), each kept in shared memory with a
                                  halo of 2K cells, K red-black sweeps between exchanges of
                                  the halo rings through L2 (K = 2 FP64, 8 FP32); mixed
                                  precision folds the FP32 correction into phi in FP64 inside
                                  the launch.  Grids up to about a million cells */
} pcd_schedule;

typedef struct {
    int sweeps;              /* full red+black sweeps run */
    int converged;           /* 1 if the stop test passed */
    double rel_residual;     /* ||b - L phi|| / ||b|| at exit (FP64, non-NaN cells) */
    double max_residual;     /* max |b - L phi| at exit */
    double last_max_update;  /* max |delta| of the last sweep (when tracked) */
    double device_ms;        /* device time of the solve (CUDA events) */
    int residual_checks;     /* FP64 residual evaluations */
    double sweep_ms;         /* device time of the sweep kernel(s) alone (CUDA events) */
    int schedule_used;       /* pcd_schedule that ran */
    int warm_used;           /* 0 zero, 1 given, 2 learned, 3 learned prediction rejected (zero) */
    double warm_rel_residual;/* warm_start 2: ||b - L phi|| / ||b|| of the learned prediction after
                                8 Gauss-Seidel sweeps (red-black, omega = 1) */
    int tuned;               /* 1: the context's autotuner chose the knobs below for this shape */
    int check_every_used;    /* check_every the solve ran with (0 = the schedule's default) */
    int refine_every_used;   /* refine_every the solve ran with (0 = default) */
    double refine_drop_used; /* refine_drop the solve ran with (0 = default) */
    double warm_zero_rel_residual; /* warm_start 2: the same for a zero guess after the same sweeps;
                                      the prediction is kept when warm_rel_residual is smaller */
} pcd_solve_stats;

typedef struct pcd_ctx pcd_ctx;
typedef struct pcd_design pcd_design;

/* ---- context ---------------------------------------------------------- */
int pcd_ctx_create(int device, pcd_ctx **out);
int pcd_ctx_destroy(pcd_ctx *ctx);
/* Stream the context launches on (a cudaStream_t). */
void *pcd_ctx_stream(pcd_ctx *ctx);
const char *pcd_last_error(void);
const char *pcd_status_string(int status);
int pcd_solve_opts_default(pcd_solve_opts *opts);
/* Number of kernels this library launched in this process (monotonic). */
unsigned long long pcd_kernel_launches(void);
/* Bounded device waits (no counterpart in the reference, whose solver has no
 * device waits).  The persistent schedule's CTAs wait for their neighbours'
 * epoch flags and for a grid barrier; each wait gives up after `polls` polls
 * (0 = the default 2^24, about half a second), records PCD_TIMEOUT and every
 * CTA returns, leaving the context usable; the solve returns PCD_TIMEOUT.
 * withhold_first_flag = 1 is the failure test's switch: the first CTA never
 * raises its epoch flag, a flag that nothing else sets, so a neighbour's wait
 * runs out on purpose.  Both stay in force for later solves on the context
 * until changed. */
int pcd_ctx_set_wait_limit(pcd_ctx *ctx, long long polls, int withhold_first_flag);

/* ---- Poisson solve ------------------------------------------------------ */
/* Drop-in for poisson_solver(D, phi, width, height, max_iterations,
 * convergence_threshold, max_threads), solver.cpp:70: solves
 * sum_nbr phi - cnt*phi = D in place on phi (host arrays, width*height,
 * row-major), phi is the warm start, stops when one sweep's max |delta| falls
 * below convergence_threshold or after max_iterations sweeps.  Neighbours
 * outside the grid or whose D is NaN are excluded (Neumann).  max_threads is
 * accepted and ignored.  Uses a process-wide context on the current device. */
int pcd_poisson_solver(const double *D, double *phi, int width, int height, int max_iterations,
                       double convergence_threshold, int max_threads);

/* Host arrays, explicit options and statistics. */
int pcd_poisson_solve(pcd_ctx *ctx, const double *b, double *phi, int width, int height,
                      const pcd_solve_opts *opts, pcd_solve_stats *stats);

/* Device arrays with leading dimension ld (elements, >= width).  `stream` is
 * the caller's stream (NULL = the CUDA default stream): the library works on
 * the context's own stream, ordered after everything already enqueued on
 * `stream` and before anything enqueued on it after the call.  The same
 * holds for every entry point below that takes a stream.  b is read, phi
 * updated in place. */
int pcd_poisson_solve_device(pcd_ctx *ctx, const double *b, double *phi, int width, int height,
                             int ld, const pcd_solve_opts *opts, pcd_solve_stats *stats,
                             void *stream);

/* ---- batched solve (no counterpart in the reference: it solves one grid per
 * call; this runs many independent grids of uneven sizes in one persistent
 * launch, captured in a CUDA graph) ------------------------------------- */
typedef struct {
    int width, height, ld;   /* ld >= width.  Batched tile form: width a multiple of 8, ld of 4,
                                any height.  Cluster form: width <= 4096, height >= 2 x the
                                cluster size (32 with 16-CTA clusters) */
    const double *b;         /* device, right-hand side */
    double *phi;             /* device, solution (warm start when opts->warm_start) */
} pcd_instance;

typedef struct {
    int sweeps;
    int converged;
    double rel_residual;     /* FP64 ||b - L phi|| / ||b|| at exit */
    int cycles;              /* FP64 defect-correction cycles */
} pcd_instance_stats;

typedef struct {
    double device_ms;        /* the graph launch, CUDA events */
    int clusters;            /* co-resident clusters used */
    int cluster_size;        /* CTAs per cluster (one per SM) */
    long long smem_bytes;    /* dynamic shared memory per CTA */
    long long cell_sweeps;   /* sum over instances of width*height*sweeps */
    int check_every;         /* FP32 sweeps between residual estimates used */
    double refine_drop;      /* cycle drop factor used */
    int tuned;               /* 1: the context's autotuner chose cluster size, check_every, refine_drop */
} pcd_batch_stats;

/* Mixed precision (FP32 sweeps, FP64 defect correction) with the relative-
 * residual stop; opts->omega as in pcd_solve_opts, per instance.  When every
 * width is a multiple of 8 and every ld of 4 (and at most 1024 instances),
 * each launch runs up to 4 sweeps over the tiles of every instance that has
 * not converged, with a batched FP64 refresh every refine_every sweeps (0:
 * 32 to 128 by the largest side; batch_stats->check_every reports it,
 * clusters = 0); otherwise, or with opts->schedule = PCD_SCHED_CLUSTER, each
 * 16-CTA cluster takes instances from a work queue (largest first) and solves
 * them whole.  stats has `count` entries in the caller's order. */
int pcd_batch_solve_device(pcd_ctx *ctx, const pcd_instance *inst, int count, const pcd_solve_opts *opts,
                           pcd_instance_stats *stats, pcd_batch_stats *batch_stats, void *stream);

/* ---- image ingest (main.cpp:13-109) ----------------------------------------
 * image_to_grid: decode a PNG file (any colour type and bit depth, Adam7)
 * with the reference's libpng transforms (16-bit -> high byte, palette ->
 * RGB, gray < 8 bit -> 8 bit, tRNS -> alpha) and convert each pixel to
 * 0.299 r + 0.587 g + 0.114 b on samples / 255 (main.cpp:91-99); gray images
 * take r = g = b (the reference mis-reads their 2-byte rows as 4-byte).  Host
 * code.  gray NULL: only width / height.  gray: height x width doubles. */
int pcd_image_to_grid(const char *filename, int *width, int *height, double *gray);
/* The decoder alone: rgba NULL queries the size; else width*height*4 bytes. */
int pcd_png_decode(const unsigned char *data, size_t size, int *width, int *height, unsigned char *rgba);
/* resize_image (main.cpp:13-27): host arrays (through the process-wide
 * context of device 0, like pcd_poisson_solver) or device grids. */
int pcd_resize_image(const double *in, int old_width, int old_height, double *out, int new_width, int new_height);
int pcd_resize_image_device(pcd_ctx *ctx, const double *in, int old_width, int old_height, int in_ld, double *out,
                            int new_width, int new_height, int out_ld, void *stream);

/* Fold handling (no counterpart: the reference exits on a raster miss).
 * Mesh::laplacian_smoothing (mesh.cpp:534-606) of the target mesh on the
 * device; the number of triangles of the structured mesh whose signed area
 * is not positive; replacing the target points (n x 3 host array, z ignored),
 * e.g. to resume from a saved mesh. */
int pcd_design_smooth_target_mesh(pcd_design *d, double smoothing_factor);
int pcd_design_count_folds(pcd_design *d, long long *folds);
int pcd_design_set_target_points(pcd_design *d, const double *points);

/* ---- output files (caustic_design.cpp:55-61, mesh.cpp:608-610,411-414,
 * utils.cpp:198-307, main.cpp:111-135) ------------------------------------
 * Host functions: the reference's text, byte for byte, from host arrays
 * (points: mesh_res_x * mesh_res_y x 3, row-major like Mesh::target_points).
 * No device work; PCD_BAD_ARG if the file cannot be written. */
int pcd_write_solid_obj(const double *front_points, const double *back_points, int mesh_res_x, int mesh_res_y,
                        double thickness, double width, double height, const char *filename);  /* save_solid_obj */
int pcd_write_grid_svg(const double *points, int mesh_res_x, int mesh_res_y, double width, double height,
                       const char *filename, double stroke_width);                             /* export_grid_to_svg */
int pcd_write_heightmap_json(const double *h, int width, int height, const char *filename);   /* save_heightmap_as_json */
/* From a design's device state: which = 0 save_solid_obj_source, 1 _target. */
int pcd_design_save_solid_obj(pcd_design *d, int which, const char *filename);
int pcd_design_export_parameterization_svg(pcd_design *d, const char *filename, double stroke_width);
int pcd_design_export_inverted_transport_map_svg(pcd_design *d, const char *filename, double stroke_width);
int pcd_design_save_heightmap_json(pcd_design *d, const char *filename);

/* ---- autotuner (no counterpart in the reference) ---------------------------
 * With autotuning on, the first solve of each (width, height, precision, stop)
 * with schedule PCD_SCHED_AUTO and check_every, refine_every, refine_drop all
 * 0, and the first batch of each size signature, time a small set of
 * candidate settings on the caller's own problem (phi is restored between
 * trials; the result is that of the winner, solved again from the caller's
 * phi), keep the fastest that converged and reuse it for later calls of that
 * shape.  Single solves: check_every, refine_drop, refine_every and the
 * schedule; batches: cluster size (16 or 8 CTAs), check_every, refine_drop.
 * Off by default; the trial solves are extra work on the first call only. */
int pcd_ctx_set_autotune(pcd_ctx *ctx, int enable);
/* entries: shapes tuned so far; trials: trial solves (or batches) run */
int pcd_ctx_autotune_info(pcd_ctx *ctx, int *entries, long long *trials);

/* ---- learned warm start (no counterpart in the reference) ------------------
 * A 4-level BF16 U-Net (1->32->64->128->256 channels, 3x3 convolutions, FP32
 * accumulation on the tensor cores) that maps a normalised right-hand side
 * x = (b - mean b) / std(b) on a resolution x resolution grid to
 * phi_hat = phi / (std(b) * resolution^2) with the mean removed.  Training and
 * inference run the library's own kernels.  x, target, out: device FP32,
 * batch x resolution x resolution. */
typedef struct pcd_unet pcd_unet;
int pcd_unet_create(pcd_ctx *ctx, int resolution, int max_batch, unsigned long long seed, pcd_unet **out);
int pcd_unet_destroy(pcd_unet *net);
long long pcd_unet_num_params(pcd_unet *net);
int pcd_unet_resolution(pcd_unet *net);
int pcd_unet_get_params(pcd_unet *net, float *host);
int pcd_unet_set_params(pcd_unet *net, const float *host);
/* one AdamW step on the mean squared error of the mean-removed prediction */
int pcd_unet_train_step(pcd_unet *net, const float *x, const float *target, int batch, float lr,
                        float weight_decay, float *loss, void *stream);
int pcd_unet_predict(pcd_unet *net, const float *x, int batch, float *out, void *stream);
/* gradients of the last training step (FP32, pcd_unet_num_params values) */
int pcd_unet_get_grads(pcd_unet *net, float *host);
/* The tensor-core GEMM the network is built on: C[M x N] (FP32, row stride
 * ldc) = A[M x K] * B[N x K]^T with A, B BF16 row-major, K a multiple of 32,
 * lda/ldb multiples of 8; ksplit > 1 needs ksplit*M*N floats of partials. */
int pcd_gemm_bf16(const void *A, int lda, const void *B, int ldb, float *C, int ldc, int M, int N, int K,
                  int ksplit, float *partials, void *stream);
/* The same GEMM on a chosen path: 0 automatic, 1 mma.sync (warp-level
 * tensor-core fragments through ldmatrix), 2 tcgen05 (TMA loads with the
 * 128-byte swizzle, tcgen05.mma into tensor-memory accumulators; one
 * or two persistent CTAs per SM with a TMA warp, an MMA warp and four
 * epilogue warps, two accumulators so that a tile's epilogue overlaps the
 * next tile; A and B 16-byte aligned).  The tcgen05 kernel's bounded waits
 * report through a
 * device error word that pcd_gemm_bf16_status reads (after synchronising the
 * device; PCD_TIMEOUT if a wait gave up since the last call) and clears.  No
 * counterpart in the reference. */
int pcd_gemm_bf16_path(const void *A, int lda, const void *B, int ldb, float *C, int ldc, int M, int N, int K,
                       int ksplit, float *partials, int path, void *stream);
int pcd_gemm_bf16_status(void);
/* The tcgen05 GEMM with operand layouts: a_mn = 1 gives A as K rows of M
 * (A^T stored row-major, [K][M] with row stride lda), b_mn = 1 gives B as
 * [K][N] (row stride ldb), trans_c = 1 stores C transposed (C[n][m] at
 * n * ldc + m).  MN-major extents of at least 64 (32 for B with N <= 32),
 * K >= 64 and any K; the U-Net's weight gradient dW^T = col^T dY is this
 * form.  No counterpart in the reference. */
int pcd_gemm_bf16_layout(const void *A, int lda, int a_mn, const void *B, int ldb, int b_mn, float *C, int ldc,
                         int trans_c, int M, int N, int K, int ksplit, float *partials, void *stream);
/* The U-Net's 3x3, pad-1 convolution as an implicit GEMM on the tcgen05
 * kernel (no im2col matrix: 4-D TMA boxes of the input, zero-filled outside
 * the image).  x: BF16 NHWC, B images of H x W, C >= 32 channels (a multiple
 * of 8) at pixel stride ldx; the images must tile into 128-pixel boxes (64
 * for the weight gradient), e.g. powers of two.
 * pcd_conv3x3_bf16: out[p][n] (FP32, row stride ldo) = sum over taps t and
 * channels c of x[p shifted by t][c] * w[n][t * C + c] (w BF16, row stride
 * ldw, N output channels).
 * pcd_conv3x3_wgrad_bf16: dw[n][t * C + c] (FP32, row stride ldw) = sum_p
 * x[p shifted by t][c] * dy[p][n] (dy BF16 dense [P][N]); ksplit > 1 needs
 * ksplit * N * 9C floats of partials.  No counterpart in the reference. */
int pcd_conv3x3_bf16(const void *x, int B, int H, int W, int C, int ldx, const void *w, int ldw, int N, float *out,
                     int ldo, void *stream);
int pcd_conv3x3_wgrad_bf16(const void *x, int B, int H, int W, int C, int ldx, const void *dy, int N, float *dw,
                           int ldw, int ksplit, float *partials, void *stream);
/* What path 0 (automatic) means for every GEMM of the process, the U-Net's
 * included: 0 (default) tcgen05 wherever it applies (16-byte aligned
 * operands, K >= 64), else mma.sync; 1 mma.sync always. */
int pcd_gemm_set_default_path(int path);
/* network used by warm_start = PCD_WARM_LEARNED (not owned; NULL clears) */
int pcd_ctx_set_warm_start_net(pcd_ctx *ctx, pcd_unet *net);

/* ---- grid utilities on device arrays (dense, ld == width) -------------- */
int pcd_subtract_average_device(pcd_ctx *ctx, double *g, int width, int height, void *stream);
int pcd_gradient_device(pcd_ctx *ctx, const double *g, double *gx, double *gy, int width,
                        int height, void *stream);
int pcd_divergence_device(pcd_ctx *ctx, const double *nx, const double *ny, double *div,
                          int width, int height, void *stream);

/* Mean removal that allocates no device memory (no counterpart in the
 * reference; it is an extra entry point of this library).  For callers that
 * cannot let a library call cudaMalloc -- a host application that gives its
 * whole device-memory budget to its own pool, or a latency-critical path where
 * an allocation would synchronise the device.  Same result as
 * pcd_subtract_average_device on g (device array, width*height, dense), on the
 * CURRENT device, enqueued on `stream` (NULL = legacy default stream).  Its
 * scratch is a static device array of 2*16384+2 doubles held by every GPU
 * that loads the library until exit, so height must be <= 16384 (else
 * PCD_BAD_ARG).  A call on a stream that is not capturing looks that array's
 * device address up afresh; a call on a capturing stream reuses the address
 * of the last such lookup on the device, so make one call on each device
 * before any stream capture, and again after a cudaDeviceReset.  All calls
 * share the array: calls that overlap on the GPU race and must be serialised
 * by the caller. */
int pcd_subtract_average_noalloc(double *g, int width, int height, void *stream);

/* ---- Caustic_design ----------------------------------------------------- */
typedef enum {
    PCD_GRID_PHI = 0, PCD_GRID_H = 1, PCD_GRID_RASTER = 2, PCD_GRID_DIVERGENCE = 3,
    PCD_GRID_NORM_X = 4, PCD_GRID_NORM_Y = 5,
    PCD_GRID_PIXELS = 6,       /* the target image scaled to [0, 1] (caustic_design.cpp:335) */
    PCD_GRID_GRADIENT_X = 7,   /* calculate_gradient(phi) (utils.cpp:3-20, caustic_design.cpp:225), */
    PCD_GRID_GRADIENT_Y = 8    /* computed from the current phi on request */
} pcd_grid;

typedef enum {
    PCD_VERT_TARGET_POINTS = 10, PCD_VERT_SOURCE_POINTS = 11, PCD_VERT_TARGET_AREAS = 12,
    PCD_VERT_ERRORS = 13, PCD_VERT_NORMALS_X = 14, PCD_VERT_NORMALS_Y = 15,
    PCD_VERT_GRADIENT_X = 16, PCD_VERT_GRADIENT_Y = 17,
    PCD_VERT_INVERTED_MAP = 18,  /* n x 3: the inverted transport map of the current target mesh
                                    (mesh.cpp:348-409), computed on request; z = 0 */
    PCD_VERT_CELL_POINTS = 19    /* n x 3: the target mesh the dual cells of the last transport
                                    iteration (or of the initialisation) were built from: the
                                    reference's target_cells (caustic_design.cpp:195-196,343-344)
                                    are its barycentric dual cells; z = 0 */
} pcd_vertex_field;

typedef struct {
    int mesh_res_x, mesh_res_y;  /* set_mesh_resolution */
    int res_x, res_y;            /* set_domain_resolution (Poisson grid) */
    double width, height;        /* set_mesh_size */
    double focal_l;              /* set_lens_focal_length */
    double thickness;            /* set_lens_thickness */
    pcd_solve_opts transport;    /* solve options of the transport iterations */
    pcd_solve_opts height_solve; /* solve options of the height iterations */
    int raster_miss_policy;      /* 0: a raster miss returns PCD_RASTER_MISS (the reference exits,
                                    mesh.cpp:277-279); 1: smooth the target mesh (factor 0.1, the
                                    reference's unreached caustic_design.cpp:214-217) and return
                                    PCD_MESH_SMOOTHED */
} pcd_design_params;

/* Defaults: the reference's solves (max |delta| < 1e-7 transport,
 * < 1e-8 height, 100000 sweeps, FP64). */
int pcd_design_params_default(pcd_design_params *p);
int pcd_design_create(pcd_ctx *ctx, const pcd_design_params *p, pcd_design **out);
int pcd_design_destroy(pcd_design *d);
/* image: res_y x res_x gray grid (host), as passed to initialize_solvers. */
int pcd_design_initialize(pcd_design *d, const double *image);
/* *step_out = max vertex displacement / width (caustic_design.cpp:253-265). */
int pcd_design_transport_iteration(pcd_design *d, double *step_out, pcd_solve_stats *stats);
/* *update_out = sum of squared height changes (mesh.cpp:735-741). */
int pcd_design_height_iteration(pcd_design *d, int itr, double *update_out, pcd_solve_stats *stats);
/* Copy a grid (res_y x res_x) or vertex field (n or n x 3) to host memory. */
int pcd_design_get_grid(pcd_design *d, int which, double *host_out);
int pcd_design_get_vertices(pcd_design *d, int which, double *host_out);

/* Batched designs (no counterpart in the reference, which runs one
 * Caustic_design per process): the same call on n designs (1..1024, no
 * design twice) at once.  Two forms:
 *   lock-step -- every design on one context, and the step's solve options
 *     (transport / height_solve) the same for all and of the mixed-precision
 *     relative-residual form: the designs' steps before the solve, then ONE
 *     batched solve of all their grids (pcd_batch_solve_device: every grid's
 *     tiles in each launch, so grids too small to fill the GPU alone share
 *     it), then the steps after the solve.  Each grid reaches the tolerance;
 *     the iterates differ from single calls' within it.
 *   concurrent -- otherwise: each design on a host thread of its own, its
 *     work on its context's stream, so designs on distinct contexts overlap
 *     on the GPU; results are those of the single calls, bit for bit.
 * steps / updates / statuses / stats / images have n entries (stats and
 * statuses may be NULL); the return value is PCD_OK or the first failing
 * design's status, whose text pcd_last_error() gives on the calling thread
 * (PCD_MESH_SMOOTHED, as for the single call, is a result). */
int pcd_design_initialize_batch(pcd_design *const *designs, int n, const double *const *images, int *statuses);
int pcd_design_transport_iteration_batch(pcd_design *const *designs, int n, double *steps, pcd_solve_stats *stats,
                                         int *statuses);
int pcd_design_height_iteration_batch(pcd_design *const *designs, int n, int itr, double *updates,
                                      pcd_solve_stats *stats, int *statuses);

#ifdef __cplusplus
}
#endif
#endif /* PCD_H */
