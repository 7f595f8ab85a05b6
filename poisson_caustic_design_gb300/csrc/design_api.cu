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
    for (int i = 0; i < n; i++) {
        PCD_TRY(live(ds[i]));
        for (int j = 0; j < i; j++)
            if (ds[j] == ds[i]) {
                set_error("design batch: design " + std::to_string(i) + " appears twice");
                return PCD_BAD_ARG;
            }
    }
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

// Lock-step batches: every design on one context, and the solve options of
// the step (transport or height) identical across the designs and of the
// mixed-precision relative-residual form.  Then the designs' steps before the
// solve run one after the other on the context's stream, all their grids go
// to one batched solve (pcd_batch_solve_device: every grid's tiles in each
// launch, so grids too small to fill the GPU alone share it), and the steps
// after the solve follow.
static bool lockstep(pcd_design *const *ds, int n, bool height)
{
    if (n < 2) return false;
    pcd_ctx *c = ds[0]->d.ctx;
    const pcd_solve_opts &o0 = height ? ds[0]->d.p.height_solve : ds[0]->d.p.transport;
    if (o0.precision != PCD_PREC_MIXED || o0.stop != PCD_STOP_REL_RESIDUAL || !(o0.tol > 0.0) ||
        o0.warm_start == PCD_WARM_LEARNED)
        return false;
    for (int i = 1; i < n; i++) {
        const pcd_solve_opts &o = height ? ds[i]->d.p.height_solve : ds[i]->d.p.transport;
        if (ds[i]->d.ctx != c || std::memcmp(&o, &o0, sizeof(o)) != 0) return false;
    }
    return true;
}

// pre(i) for every design, one batched solve of the grids of those that are
// ready (solve_of(i) gives b and phi), post(i) for them; per-design statuses
// as run_batch.
template <typename Pre, typename SolveOf, typename Post>
static int run_lockstep(pcd_design *const *ds, int n, bool height, int *statuses, pcd_solve_stats *stats, Pre pre,
                        SolveOf solve_of, Post post)
{
    pcd_ctx *c = ds[0]->d.ctx;
    std::lock_guard<std::mutex> lk(c->mu);
    PCD_TRY(ctx_activate(c));
    std::vector<int> st((size_t)n, PCD_OK);
    std::vector<std::string> err((size_t)n);
    std::vector<pcd_instance> inst;
    std::vector<int> idx;
    for (int i = 0; i < n; i++) {
        st[(size_t)i] = pre(i);
        if (st[(size_t)i] == PCD_OK) {
            const Design &d = ds[i]->d;
            pcd_instance q{};
            q.width = d.p.res_x;
            q.height = d.p.res_y;
            q.ld = d.p.res_x;
            solve_of(i, &q.b, &q.phi);
            inst.push_back(q);
            idx.push_back(i);
        } else if (st[(size_t)i] != PCD_MESH_SMOOTHED) {
            err[(size_t)i] = pcd_last_error();
        }
    }
    if (!inst.empty()) {
        const pcd_solve_opts o = height ? ds[0]->d.p.height_solve : ds[0]->d.p.transport;
        std::vector<pcd_instance_stats> is(inst.size());
        pcd_batch_stats bs{};
        const int sst = batch_autotuned(c, inst.data(), (int)inst.size(), o, is.data(), &bs, c->stream);
        if (sst != PCD_OK && sst != PCD_NOT_CONVERGED) return sst;
        for (size_t k = 0; k < idx.size(); k++) {
            const int i = idx[k];
            if (stats) {
                pcd_solve_stats &s = stats[i];
                std::memset(&s, 0, sizeof(s));
                s.sweeps = is[k].sweeps;
                s.converged = is[k].converged;
                s.rel_residual = is[k].rel_residual;
                s.device_ms = bs.device_ms;
                s.residual_checks = is[k].cycles;
                s.schedule_used = bs.clusters == 0 ? PCD_SCHED_TILES : PCD_SCHED_CLUSTER;
                s.warm_used = o.warm_start ? 1 : 0;
            }
            st[(size_t)i] = post(i);
            if (st[(size_t)i] != PCD_OK) err[(size_t)i] = pcd_last_error();
        }
    }
    int first = PCD_OK;
    for (int i = 0; i < n; i++) {
        if (statuses) statuses[i] = st[(size_t)i];
        if (first == PCD_OK && st[(size_t)i] != PCD_OK && st[(size_t)i] != PCD_MESH_SMOOTHED) {
            first = st[(size_t)i];
            set_error("design " + std::to_string(i) + " of the batch: " + err[(size_t)i]);
        }
    }
    (void)height;
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
    // validation (null, destroyed or repeated designs) first
    const int ok = run_batch(designs, n, statuses, [&](int) { return PCD_OK; });
    if (ok != PCD_OK) return ok;
    if (lockstep(designs, n, false))
        return run_lockstep(
            designs, n, false, statuses, stats, [&](int i) { return designs[i]->d.transport_pre(steps + i); },
            [&](int i, const double **b, double **phi) {
                *b = designs[i]->d.raster;
                *phi = designs[i]->d.phi;
            },
            [&](int i) { return designs[i]->d.transport_post(steps + i); });
    return run_batch(designs, n, statuses, [&](int i) {
        return pcd_design_transport_iteration(designs[i], steps + i, stats ? stats + i : nullptr);
    });
}

int pcd_design_height_iteration_batch(pcd_design *const *designs, int n, int itr, double *updates,
                                      pcd_solve_stats *stats, int *statuses)
{
    if (!updates) return PCD_BAD_ARG;
    const int ok = run_batch(designs, n, statuses, [&](int) { return PCD_OK; });
    if (ok != PCD_OK) return ok;
    (void)itr;
    if (lockstep(designs, n, true))
        return run_lockstep(
            designs, n, true, statuses, stats, [&](int i) { return designs[i]->d.height_pre(); },
            [&](int i, const double **b, double **phi) {
                *b = designs[i]->d.div;
                *phi = designs[i]->d.h;
            },
            [&](int i) { return designs[i]->d.height_post(updates + i); });
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
