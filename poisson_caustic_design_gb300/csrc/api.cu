// api.cu -- C ABI of libpcd_gb300: context, Poisson solve, grid utilities.
//
// Declarations and the reference interfaces they replace: include/pcd.h.
#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>

#include "api_internal.cuh"
#include "design.cuh"
#include "unet.cuh"

namespace pcd {

// Gauss-Seidel sweeps applied to a learned prediction before it is judged.
constexpr int kLearnedSmooth = 8;

namespace {
thread_local std::string g_last_error;
std::atomic<unsigned long long> g_launches{0};
}  // namespace

void set_error(const std::string &msg) { g_last_error = msg; }
void count_launches(unsigned long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

namespace {

// Keeps the smoothed prediction when its residual is below the smoothed zero
// guess's (a NaN residual never is), else a zero start; records the verdict.
__global__ void k_judge_pick(const Ctl *cz, const Ctl *cp, const double *__restrict__ pred, double *__restrict__ phi,
                             int W, int H, int ld, JudgeOut *out)
{
    const double rz = cz->rel, rp = cp->rel;
    const bool keep = rp < rz;
    const long n = (long)W * H;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const long y = i / W, j = y * ld + (i - y * W);
        phi[j] = keep ? pred[j] : 0.0;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        out->keep = keep ? 1 : 0;
        out->rel_pred = rp;
        out->rel_zero = rz;
    }
}

// (Re)builds the judge graph for this shape and network: buffers sized for
// H * ld cells, then the prediction, the zero guess and both smoothings
// captured from the context's stream.
int judge_prepare(pcd_ctx *ctx, int W, int H, int ld, cudaStream_t s)
{
    JudgeGraph &J = ctx->judge;
    UNet &net = ctx->net->net;
    if (J.exec && J.W == W && J.H == H && J.ld == ld && J.net == (const void *)ctx->net && J.arena == net.arena)
        return PCD_OK;
    if (J.exec) {
        cudaGraphExecDestroy(J.exec);
        J.exec = nullptr;
    }
    const size_t cells = (size_t)H * ld;
    if (cells > J.cells) {
        PCD_CUDA(cudaStreamSynchronize(s));
        if (J.b) cudaFree(J.b);
        if (J.pred) cudaFree(J.pred);
        if (J.zero) cudaFree(J.zero);
        if (J.mask) cudaFree(J.mask);
        if (J.mask_z) cudaFree(J.mask_z);
        if (J.e32) cudaFree(J.e32);
        if (J.r32) cudaFree(J.r32);
        J.b = J.pred = J.zero = nullptr;
        J.mask = J.mask_z = nullptr;
        J.e32 = J.r32 = nullptr;
        J.cells = 0;
        PCD_CUDA(cudaMalloc(&J.b, cells * sizeof(double)));
        PCD_CUDA(cudaMalloc(&J.pred, cells * sizeof(double)));
        PCD_CUDA(cudaMalloc(&J.zero, cells * sizeof(double)));
        PCD_CUDA(cudaMalloc(&J.mask, cells));
        PCD_CUDA(cudaMalloc(&J.mask_z, cells));
        PCD_CUDA(cudaMalloc(&J.e32, 2 * cells * sizeof(float)));
        PCD_CUDA(cudaMalloc(&J.r32, 2 * cells * sizeof(float)));
        J.cells = cells;
    }
    if (!J.ctl) {
        PCD_CUDA(cudaMalloc(&J.ctl, 2 * sizeof(Ctl)));
        PCD_CUDA(cudaMalloc(&J.partials, residual_partials_bytes()));
        PCD_CUDA(cudaMalloc(&J.partials_z, residual_partials_bytes()));
        PCD_CUDA(cudaMalloc(&J.out, sizeof(JudgeOut)));
        PCD_CUDA(cudaMallocHost(&J.out_host, sizeof(JudgeOut)));
        PCD_CUDA(cudaEventCreateWithFlags(&J.done, cudaEventDisableTiming));
        PCD_CUDA(cudaEventCreateWithFlags(&J.fork, cudaEventDisableTiming));
        PCD_CUDA(cudaEventCreateWithFlags(&J.join, cudaEventDisableTiming));
        PCD_CUDA(cudaStreamCreateWithFlags(&J.side, cudaStreamNonBlocking));
    }
    // grids that fit one cluster smooth in the mixed form (FP64 residuals,
    // FP32 sweeps on the cluster), others with FP64 half-sweep launches
    J.mixed = smooth_mixed_applies(ctx->device, W, H);
    auto smooth = [&](double *phi, uint8_t *mask, Ctl *ctl, double *partials, int branch, cudaStream_t st) {
        if (J.mixed)
            return enqueue_smooth_mixed(J.b, phi, J.e32 + (size_t)branch * cells, J.r32 + (size_t)branch * cells, ctl,
                                        partials, W, H, ld, kLearnedSmooth, ctx->device, st);
        return enqueue_smooth(J.b, phi, mask, ctl, partials, W, H, ld, kLearnedSmooth, 1.0, st);
    };
    const unsigned long long n0 = g_launches.load();
    cudaGraph_t g;
    PCD_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    // the zero guess's smoothing on a side branch (it needs only b), the
    // prediction and its smoothing on the main one, joined before the end
    int st = cudaEventRecord(J.fork, s) == cudaSuccess && cudaStreamWaitEvent(J.side, J.fork, 0) == cudaSuccess
                 ? PCD_OK
                 : PCD_DEVICE_ERROR;
    if (st == PCD_OK) st = zero_grid(J.zero, W, H, ld, J.side);
    if (st == PCD_OK) st = smooth(J.zero, J.mask_z, J.ctl, J.partials_z, 0, J.side);
    if (st == PCD_OK && cudaEventRecord(J.join, J.side) != cudaSuccess) st = PCD_DEVICE_ERROR;
    if (st == PCD_OK) st = net.warm_start(J.b, W, H, ld, J.pred, s);
    if (st == PCD_OK) st = smooth(J.pred, J.mask, J.ctl + 1, J.partials, 1, s);
    if (st == PCD_OK && cudaStreamWaitEvent(s, J.join, 0) != cudaSuccess) st = PCD_DEVICE_ERROR;
    if (st == PCD_DEVICE_ERROR) set_error("judge graph: fork / join of the capture failed");
    const cudaError_t ce = cudaStreamEndCapture(s, &g);
    // nothing ran during the capture: count the kernels at each replay instead
    J.launches = g_launches.load() - n0;
    g_launches.fetch_sub(J.launches, std::memory_order_relaxed);
    if (st != PCD_OK) {
        if (ce == cudaSuccess) cudaGraphDestroy(g);
        return st;
    }
    if (ce != cudaSuccess) {
        set_error(std::string("judge graph capture: ") + cudaGetErrorString(ce));
        return PCD_DEVICE_ERROR;
    }
    const cudaError_t ie = cudaGraphInstantiate(&J.exec, g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) {
        J.exec = nullptr;
        set_error(std::string("judge graph instantiate: ") + cudaGetErrorString(ie));
        return PCD_DEVICE_ERROR;
    }
    J.W = W;
    J.H = H;
    J.ld = ld;
    J.net = ctx->net;
    J.arena = net.arena;
    return PCD_OK;
}

}  // namespace

void JudgeGraph::release()
{
    if (exec) cudaGraphExecDestroy(exec);
    if (b) cudaFree(b);
    if (pred) cudaFree(pred);
    if (zero) cudaFree(zero);
    if (mask) cudaFree(mask);
    if (mask_z) cudaFree(mask_z);
    if (e32) cudaFree(e32);
    if (r32) cudaFree(r32);
    if (ctl) cudaFree(ctl);
    if (partials) cudaFree(partials);
    if (partials_z) cudaFree(partials_z);
    if (side) cudaStreamDestroy(side);
    if (fork) cudaEventDestroy(fork);
    if (join) cudaEventDestroy(join);
    if (out) cudaFree(out);
    if (out_host) cudaFreeHost(out_host);
    if (done) cudaEventDestroy(done);
    *this = JudgeGraph();
}

int ctx_stage(pcd_ctx *ctx, size_t cells)
{
    if (cells > ctx->host_cells) {
        if (ctx->d_b) cudaFree(ctx->d_b);
        if (ctx->d_phi) cudaFree(ctx->d_phi);
        ctx->d_b = nullptr;
        ctx->d_phi = nullptr;
        ctx->host_cells = 0;
        PCD_CUDA(cudaMalloc(&ctx->d_b, cells * sizeof(double)));
        PCD_CUDA(cudaMalloc(&ctx->d_phi, cells * sizeof(double)));
        ctx->host_cells = cells;
    }
    return PCD_OK;
}

int StreamJoin::begin()
{
    if (user == work) return PCD_OK;
    PCD_CUDA(cudaEventRecord(ctx->join_in, user));
    PCD_CUDA(cudaStreamWaitEvent(work, ctx->join_in, 0));
    return PCD_OK;
}

int StreamJoin::end()
{
    if (user == work) return PCD_OK;
    PCD_CUDA(cudaEventRecord(ctx->join_out, work));
    PCD_CUDA(cudaStreamWaitEvent(user, ctx->join_out, 0));
    return PCD_OK;
}

int ctx_activate(pcd_ctx *ctx)
{
    PCD_CUDA(cudaSetDevice(ctx->device));
    return PCD_OK;
}

// Solve with the warm-start policy of o: the learned prediction is kept only
// when its smoothed FP64 residual is below that of a smoothed zero guess.
int solve_with_warm_start(pcd_ctx *ctx, const double *b, double *phi, int W, int H, int ld, pcd_solve_opts o,
                          pcd_solve_stats *stats, cudaStream_t s)
{
    int used = o.warm_start == PCD_WARM_GIVEN ? 1 : 0;
    double rel0 = -1.0, relz = -1.0;
    int pre_sweeps = 0;
    bool judged = false;
    if (o.warm_start == PCD_WARM_LEARNED) {
        if (!ctx->net) {
            set_error("warm_start = PCD_WARM_LEARNED needs a network (pcd_ctx_set_warm_start_net)");
            return PCD_BAD_ARG;
        }
        // Judge the prediction after kLearnedSmooth Gauss-Seidel sweeps (red-
        // black, omega = 1) against a zero guess after the same sweeps: the
        // sweeps remove the cell-scale error that the prediction's
        // interpolation and BF16 arithmetic leave (it would dominate the raw
        // residual), and the zero guess's residual also moves under them.
        // The smoothed prediction is kept when its residual is the smaller.
        // All on the device: b in, one graph replay, the pick, the verdict
        // read back after the solve.
        JudgeGraph &J = ctx->judge;
        PCD_TRY(judge_prepare(ctx, W, H, ld, s));
        PCD_CUDA(cudaMemcpy2DAsync(J.b, (size_t)ld * sizeof(double), b, (size_t)ld * sizeof(double),
                                   (size_t)W * sizeof(double), H, cudaMemcpyDeviceToDevice, s));
        PCD_CUDA(cudaGraphLaunch(J.exec, s));
        count_launches(J.launches);
        const int pblocks = (int)std::min<long>(1216, ((long)W * H + 255) / 256);
        k_judge_pick<<<pblocks, 256, 0, s>>>(J.ctl, J.ctl + 1, J.pred, phi, W, H, ld, J.out);
        PCD_LAUNCHED(1);
        PCD_CUDA(cudaMemcpyAsync(J.out_host, J.out, sizeof(JudgeOut), cudaMemcpyDeviceToHost, s));
        PCD_CUDA(cudaEventRecord(J.done, s));
        judged = true;
        o.warm_start = PCD_WARM_GIVEN;
    } else if (o.warm_start != PCD_WARM_ZERO && o.warm_start != PCD_WARM_GIVEN) {
        set_error("pcd solve: unknown warm_start");
        return PCD_BAD_ARG;
    }
    int st = solve_autotuned(ctx, b, phi, W, H, ld, o, stats, s);
    if (judged) {
        PCD_CUDA(cudaEventSynchronize(ctx->judge.done));
        const JudgeOut &v = *ctx->judge.out_host;
        used = v.keep ? 2 : 3;
        pre_sweeps = v.keep ? kLearnedSmooth : 0;
        rel0 = v.rel_pred;
        relz = v.rel_zero;
    }
    if (stats) {
        stats->warm_used = used;
        stats->warm_rel_residual = rel0;
        stats->warm_zero_rel_residual = relz;
        stats->sweeps += pre_sweeps;
    }
    return st;
}

}  // namespace pcd

using namespace pcd;

extern "C" {

const char *pcd_last_error(void) { return g_last_error.c_str(); }

unsigned long long pcd_kernel_launches(void) { return g_launches.load(); }

const char *pcd_status_string(int status)
{
    switch (status) {
    case PCD_OK: return "ok";
    case PCD_NOT_CONVERGED: return "not converged";
    case PCD_BAD_ARG: return "bad argument";
    case PCD_DEVICE_ERROR: return "device error";
    case PCD_TIMEOUT: return "timeout";
    case PCD_RASTER_MISS: return "raster miss";
    case PCD_NO_DEVICE: return "no CUDA device";
    case PCD_FALLBACK_USED: return "fallback used";
    case PCD_MESH_SMOOTHED: return "raster miss: target mesh smoothed";
    }
    return "unknown status";
}

int pcd_solve_opts_default(pcd_solve_opts *o)
{
    if (!o) return PCD_BAD_ARG;
    std::memset(o, 0, sizeof(*o));
    o->max_iterations = 100000;   // caustic_design.cpp:222,311
    o->tol = 1e-7;                // caustic_design.cpp:222
    o->stop = PCD_STOP_MAX_UPDATE;
    o->precision = PCD_PREC_FP64;
    o->omega = 0.0;
    o->check_every = 0;
    o->refine_every = 0;
    o->warm_start = 1;
    o->schedule = PCD_SCHED_AUTO;
    return PCD_OK;
}

int pcd_ctx_create(int device, pcd_ctx **out)
{
    if (!out) return PCD_BAD_ARG;
    *out = nullptr;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
        set_error(std::string("no CUDA device: ") + cudaGetErrorString(e));
        return PCD_NO_DEVICE;
    }
    if (device < 0) PCD_CUDA(cudaGetDevice(&device));
    if (device >= n) {
        set_error("pcd_ctx_create: device index out of range");
        return PCD_BAD_ARG;
    }
    PCD_CUDA(cudaSetDevice(device));
    auto *c = new pcd_ctx();
    c->device = device;
    c->solver.dev = device;
    cudaError_t ce = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&c->join_in, cudaEventDisableTiming);
    if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&c->join_out, cudaEventDisableTiming);
    if (ce != cudaSuccess) {
        delete c;
        set_error(std::string("cudaStreamCreate: ") + cudaGetErrorString(ce));
        return PCD_DEVICE_ERROR;
    }
    *out = c;
    return PCD_OK;
}

int pcd_ctx_destroy(pcd_ctx *ctx)
{
    if (!ctx) return PCD_OK;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    design_detach_all(ctx);
    unet_detach_all(ctx);
    ctx->solver.release();
    ctx->grid.release();
    ctx->batch.release();
    ctx->tuner.release();
    ctx->judge.release();
    if (ctx->d_b) cudaFree(ctx->d_b);
    if (ctx->d_phi) cudaFree(ctx->d_phi);
    if (ctx->join_in) cudaEventDestroy(ctx->join_in);
    if (ctx->join_out) cudaEventDestroy(ctx->join_out);
    cudaStreamDestroy(ctx->stream);
    delete ctx;
    return PCD_OK;
}

void *pcd_ctx_stream(pcd_ctx *ctx) { return ctx ? (void *)ctx->stream : nullptr; }

int pcd_ctx_set_wait_limit(pcd_ctx *ctx, long long polls, int withhold_first_flag)
{
    if (!ctx || polls < 0) {
        set_error("pcd_ctx_set_wait_limit: null context or negative poll count");
        return PCD_BAD_ARG;
    }
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->solver.wait_limit = polls;
    ctx->solver.withhold_flag = withhold_first_flag ? 1 : 0;
    return PCD_OK;
}

int pcd_poisson_solve_device(pcd_ctx *ctx, const double *b, double *phi, int width, int height, int ld,
                             const pcd_solve_opts *opts, pcd_solve_stats *stats, void *stream)
{
    if (!ctx) return PCD_BAD_ARG;
    std::lock_guard<std::mutex> lk(ctx->mu);
    PCD_TRY(ctx_activate(ctx));
    pcd_solve_opts o;
    if (opts) o = *opts; else pcd_solve_opts_default(&o);
    StreamJoin j(ctx, stream);
    PCD_TRY(j.begin());
    const int st = solve_with_warm_start(ctx, b, phi, width, height, ld, o, stats, j.work);
    PCD_TRY(j.end());
    return st;
}

int pcd_poisson_solve(pcd_ctx *ctx, const double *b, double *phi, int width, int height,
                      const pcd_solve_opts *opts, pcd_solve_stats *stats)
{
    if (!ctx || !b || !phi || width < 1 || height < 1) {
        set_error("pcd_poisson_solve: bad arguments");
        return PCD_BAD_ARG;
    }
    std::lock_guard<std::mutex> lk(ctx->mu);
    PCD_TRY(ctx_activate(ctx));
    pcd_solve_opts o;
    if (opts) o = *opts; else pcd_solve_opts_default(&o);
    const size_t n = (size_t)width * height;
    PCD_TRY(ctx_stage(ctx, n));
    cudaStream_t s = ctx->stream;
    PCD_CUDA(cudaMemcpyAsync(ctx->d_b, b, n * sizeof(double), cudaMemcpyHostToDevice, s));
    if (o.warm_start == PCD_WARM_GIVEN)
        PCD_CUDA(cudaMemcpyAsync(ctx->d_phi, phi, n * sizeof(double), cudaMemcpyHostToDevice, s));
    int st = solve_with_warm_start(ctx, ctx->d_b, ctx->d_phi, width, height, width, o, stats, s);
    if (st != PCD_OK && st != PCD_NOT_CONVERGED) return st;
    PCD_CUDA(cudaMemcpyAsync(phi, ctx->d_phi, n * sizeof(double), cudaMemcpyDeviceToHost, s));
    PCD_CUDA(cudaStreamSynchronize(s));
    return st;
}

// Process-wide contexts for the reference-shaped entry point, one per device.
static std::mutex g_default_mu;
static std::map<int, pcd_ctx *> g_default;

static int default_ctx(pcd_ctx **out)
{
    int dev = 0;
    PCD_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(g_default_mu);
    auto it = g_default.find(dev);
    if (it != g_default.end()) {
        *out = it->second;
        return PCD_OK;
    }
    pcd_ctx *c = nullptr;
    PCD_TRY(pcd_ctx_create(dev, &c));
    g_default[dev] = c;
    *out = c;
    return PCD_OK;
}

int pcd_poisson_solver(const double *D, double *phi, int width, int height, int max_iterations,
                       double convergence_threshold, int max_threads)
{
    (void)max_threads;  // the reference splits each sweep over threads; one GPU here
    pcd_ctx *ctx = nullptr;
    PCD_TRY(default_ctx(&ctx));
    pcd_solve_opts o;
    pcd_solve_opts_default(&o);
    o.max_iterations = max_iterations;
    o.tol = convergence_threshold;
    o.stop = PCD_STOP_MAX_UPDATE;
    o.precision = PCD_PREC_FP64;
    o.warm_start = 1;
    return pcd_poisson_solve(ctx, D, phi, width, height, &o, nullptr);
}

int pcd_resize_image(const double *in, int old_width, int old_height, double *out, int new_width, int new_height)
{
    if (!in || !out || old_width < 1 || old_height < 1 || new_width < 1 || new_height < 1) return PCD_BAD_ARG;
    pcd_ctx *ctx = nullptr;
    PCD_TRY(default_ctx(&ctx));
    std::lock_guard<std::mutex> lk(ctx->mu);
    PCD_TRY(ctx_activate(ctx));
    const size_t ni = (size_t)old_width * old_height, no = (size_t)new_width * new_height;
    PCD_TRY(ctx_stage(ctx, std::max(ni, no)));
    cudaStream_t s = ctx->stream;
    PCD_CUDA(cudaMemcpyAsync(ctx->d_b, in, ni * sizeof(double), cudaMemcpyHostToDevice, s));
    PCD_TRY(resize_nearest(ctx->d_b, old_width, old_height, old_width, ctx->d_phi, new_width, new_height, new_width,
                           s));
    PCD_CUDA(cudaMemcpyAsync(out, ctx->d_phi, no * sizeof(double), cudaMemcpyDeviceToHost, s));
    PCD_CUDA(cudaStreamSynchronize(s));
    return PCD_OK;
}

int pcd_batch_solve_device(pcd_ctx *ctx, const pcd_instance *inst, int count, const pcd_solve_opts *opts,
                           pcd_instance_stats *stats, pcd_batch_stats *batch_stats, void *stream)
{
    if (!ctx) return PCD_BAD_ARG;
    std::lock_guard<std::mutex> lk(ctx->mu);
    PCD_TRY(ctx_activate(ctx));
    pcd_solve_opts o;
    if (opts) o = *opts;
    else {
        pcd_solve_opts_default(&o);
        o.stop = PCD_STOP_REL_RESIDUAL;
        o.tol = 1e-6;
    }
    StreamJoin j(ctx, stream);
    PCD_TRY(j.begin());
    const int st = batch_autotuned(ctx, inst, count, o, stats, batch_stats, j.work);
    PCD_TRY(j.end());
    return st;
}

int pcd_subtract_average_device(pcd_ctx *ctx, double *g, int width, int height, void *stream)
{
    if (!ctx || !g || width < 1 || height < 1) return PCD_BAD_ARG;
    std::lock_guard<std::mutex> lk(ctx->mu);
    PCD_TRY(ctx_activate(ctx));
    StreamJoin j(ctx, stream);
    PCD_TRY(j.begin());
    PCD_TRY(subtract_average(ctx->grid, g, (long)width * height, j.work));
    return j.end();
}

int pcd_gradient_device(pcd_ctx *ctx, const double *g, double *gx, double *gy, int width, int height,
                        void *stream)
{
    if (!ctx || !g || !gx || !gy || width < 1 || height < 1) return PCD_BAD_ARG;
    std::lock_guard<std::mutex> lk(ctx->mu);
    PCD_TRY(ctx_activate(ctx));
    StreamJoin j(ctx, stream);
    PCD_TRY(j.begin());
    PCD_TRY(gradient(g, gx, gy, width, height, j.work));
    return j.end();
}

int pcd_resize_image_device(pcd_ctx *ctx, const double *in, int old_width, int old_height, int in_ld, double *out,
                            int new_width, int new_height, int out_ld, void *stream)
{
    if (!ctx || !in || !out || old_width < 1 || old_height < 1 || new_width < 1 || new_height < 1 ||
        in_ld < old_width || out_ld < new_width)
        return PCD_BAD_ARG;
    std::lock_guard<std::mutex> lk(ctx->mu);
    PCD_TRY(ctx_activate(ctx));
    StreamJoin j(ctx, stream);
    PCD_TRY(j.begin());
    PCD_TRY(resize_nearest(in, old_width, old_height, in_ld, out, new_width, new_height, out_ld, j.work));
    return j.end();
}

int pcd_divergence_device(pcd_ctx *ctx, const double *nx, const double *ny, double *div, int width, int height,
                          void *stream)
{
    if (!ctx || !nx || !ny || !div || width < 1 || height < 1) return PCD_BAD_ARG;
    std::lock_guard<std::mutex> lk(ctx->mu);
    PCD_TRY(ctx_activate(ctx));
    StreamJoin j(ctx, stream);
    PCD_TRY(j.begin());
    PCD_TRY(divergence(nx, ny, div, width, height, j.work));
    return j.end();
}

}  // extern "C"
