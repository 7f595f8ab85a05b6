// design_api.cu -- C ABI of the Caustic_design replacement (declared in include/pcd.h).
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "api_internal.cuh"
#include "design.cuh"

using namespace pcd;

namespace pcd {
void design_detach_all(pcd_ctx *ctx)
{
    for (pcd_design *d : ctx->designs) {
        d->d.release();
        d->d.ctx = nullptr;
    }
    ctx->designs.clear();
}
}  // namespace pcd

static int live(pcd_design *d)
{
    if (!d || !d->d.ctx) {
        set_error("design handle is null or its context was destroyed");
        return PCD_BAD_ARG;
    }
    return PCD_OK;
}

// Runs fn(i) for the n designs of a batch, each on a host thread of its own
// (a design's work stays on its context's stream, so designs of distinct
// contexts overlap on the GPU).  statuses[i] receives each status; the
// return value is PCD_OK, or the first failing design's status with its
// error text moved to the calling thread (errors are per thread).
// PCD_MESH_SMOOTHED is a result, not a failure, as for the single call.
template <typename F>
static int run_batch(pcd_design *const *ds, int n, int *statuses, F fn)
{
    if (!ds || n < 1 || n > 1024) {
        set_error("design batch: 1 to 1024 designs");
        return PCD_BAD_ARG;
    }
    for (int i = 0; i < n; i++) PCD_TRY(live(ds[i]));
    std::vector<int> st((size_t)n, PCD_OK);
    std::vector<std::string> err((size_t)n);
    std::vector<std::thread> th;
    th.reserve((size_t)n);
    for (int i = 0; i < n; i++)
        th.emplace_back([&, i] {
            st[(size_t)i] = fn(i);
            if (st[(size_t)i] != PCD_OK) err[(size_t)i] = pcd_last_error();
        });
    for (auto &t : th) t.join();
    int first = PCD_OK;
    for (int i = 0; i < n; i++) {
        if (statuses) statuses[i] = st[(size_t)i];
        if (first == PCD_OK && st[(size_t)i] != PCD_OK && st[(size_t)i] != PCD_MESH_SMOOTHED) {
            first = st[(size_t)i];
            set_error("design " + std::to_string(i) + " of the batch: " + err[(size_t)i]);
        }
    }
    return first;
}

extern "C" {

int pcd_design_params_default(pcd_design_params *p)
{
    if (!p) return PCD_BAD_ARG;
    std::memset(p, 0, sizeof(*p));
    pcd_solve_opts_default(&p->transport);
    pcd_solve_opts_default(&p->height_solve);
    p->transport.tol = 1e-7;      // caustic_design.cpp:222
    p->height_solve.tol = 1e-8;   // caustic_design.cpp:311
    return PCD_OK;
}

int pcd_design_create(pcd_ctx *ctx, const pcd_design_params *p, pcd_design **out)
{
    if (!ctx || !p || !out) return PCD_BAD_ARG;
    *out = nullptr;
    if (p->mesh_res_x < 2 || p->mesh_res_y < 2 || p->res_x < 2 || p->res_y < 2 || !(p->width > 0) ||
        !(p->height > 0)) {
        set_error("pcd_design_create: mesh and grid resolutions must be >= 2 and sizes > 0");
        return PCD_BAD_ARG;
    }
    std::lock_guard<std::mutex> lk(ctx->mu);
    PCD_TRY(ctx_activate(ctx));
    auto *d = new pcd_design();
    d->d.ctx = ctx;
    d->d.p = *p;
    int st = d->d.alloc();
    if (st != PCD_OK) {
        d->d.release();
        delete d;
        return st;
    }
    ctx->designs.insert(d);
    *out = d;
    return PCD_OK;
}

int pcd_design_destroy(pcd_design *d)
{
    if (!d) return PCD_OK;
    if (pcd_ctx *ctx = d->d.ctx) {
        std::lock_guard<std::mutex> lk(ctx->mu);
        ctx_activate(ctx);
        cudaStreamSynchronize(ctx->stream);
        d->d.release();
        ctx->designs.erase(d);
    }
    delete d;
    return PCD_OK;
}

int pcd_design_initialize(pcd_design *d, const double *image)
{
    if (!d || !image) return PCD_BAD_ARG;
    PCD_TRY(live(d));
    std::lock_guard<std::mutex> lk(d->d.ctx->mu);
    PCD_TRY(ctx_activate(d->d.ctx));
    return d->d.initialize(image);
}

int pcd_design_transport_iteration(pcd_design *d, double *step_out, pcd_solve_stats *stats)
{
    if (!d) return PCD_BAD_ARG;
    PCD_TRY(live(d));
    std::lock_guard<std::mutex> lk(d->d.ctx->mu);
    PCD_TRY(ctx_activate(d->d.ctx));
    return d->d.transport_iteration(step_out, stats);
}

int pcd_design_height_iteration(pcd_design *d, int itr, double *update_out, pcd_solve_stats *stats)
{
    if (!d) return PCD_BAD_ARG;
    PCD_TRY(live(d));
    std::lock_guard<std::mutex> lk(d->d.ctx->mu);
    PCD_TRY(ctx_activate(d->d.ctx));
    return d->d.height_iteration(itr, update_out, stats);
}

int pcd_design_transport_iteration_batch(pcd_design *const *designs, int n, double *steps, pcd_solve_stats *stats,
                                         int *statuses)
{
    if (!steps) return PCD_BAD_ARG;
    return run_batch(designs, n, statuses, [&](int i) {
        return pcd_design_transport_iteration(designs[i], steps + i, stats ? stats + i : nullptr);
    });
}

int pcd_design_height_iteration_batch(pcd_design *const *designs, int n, int itr, double *updates,
                                      pcd_solve_stats *stats, int *statuses)
{
    if (!updates) return PCD_BAD_ARG;
    return run_batch(designs, n, statuses, [&](int i) {
        return pcd_design_height_iteration(designs[i], itr, updates + i, stats ? stats + i : nullptr);
    });
}

int pcd_design_initialize_batch(pcd_design *const *designs, int n, const double *const *images, int *statuses)
{
    if (!images) return PCD_BAD_ARG;
    return run_batch(designs, n, statuses, [&](int i) { return pcd_design_initialize(designs[i], images[i]); });
}

int pcd_design_get_grid(pcd_design *d, int which, double *host_out)
{
    if (!d || !host_out) return PCD_BAD_ARG;
    PCD_TRY(live(d));
    std::lock_guard<std::mutex> lk(d->d.ctx->mu);
    PCD_TRY(ctx_activate(d->d.ctx));
    return d->d.get_grid(which, host_out);
}

int pcd_design_get_vertices(pcd_design *d, int which, double *host_out)
{
    if (!d || !host_out) return PCD_BAD_ARG;
    PCD_TRY(live(d));
    std::lock_guard<std::mutex> lk(d->d.ctx->mu);
    PCD_TRY(ctx_activate(d->d.ctx));
    return d->d.get_vertices(which, host_out);
}

int pcd_design_smooth_target_mesh(pcd_design *d, double smoothing_factor)
{
    if (!d) return PCD_BAD_ARG;
    PCD_TRY(live(d));
    std::lock_guard<std::mutex> lk(d->d.ctx->mu);
    PCD_TRY(ctx_activate(d->d.ctx));
    if (!d->d.initialized) return PCD_BAD_ARG;
    return d->d.smooth_target(smoothing_factor);
}

int pcd_design_count_folds(pcd_design *d, long long *folds)
{
    if (!d || !folds) return PCD_BAD_ARG;
    PCD_TRY(live(d));
    std::lock_guard<std::mutex> lk(d->d.ctx->mu);
    PCD_TRY(ctx_activate(d->d.ctx));
    if (!d->d.initialized) return PCD_BAD_ARG;
    return d->d.count_folds(folds);
}

int pcd_design_set_target_points(pcd_design *d, const double *points)
{
    if (!d || !points) return PCD_BAD_ARG;
    PCD_TRY(live(d));
    std::lock_guard<std::mutex> lk(d->d.ctx->mu);
    PCD_TRY(ctx_activate(d->d.ctx));
    if (!d->d.initialized) return PCD_BAD_ARG;
    return d->d.set_target_points(points);
}

}  // extern "C"
