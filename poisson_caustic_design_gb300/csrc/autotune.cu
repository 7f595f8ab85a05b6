// autotune.cu -- per-context autotuner of the solve and batch settings.
//
// The first AUTO-schedule solve of a (width, height, precision, stop) shape,
// and the first batch of a size signature, run a small candidate set on the
// caller's own data: phi is snapshotted, each candidate solves from the
// snapshot, the fastest that converged (device time, CUDA events) is kept,
// and the call returns the winner solved again from the snapshot.  Later
// calls of the shape reuse the kept settings.  Every candidate is an exact
// configuration of the same red-black iteration, so the choice only moves
// time, not the fixed point.
#include <algorithm>
#include <cstring>
#include <vector>

#include "api_internal.cuh"

namespace pcd {

void Autotuner::release()
{
    if (save) cudaFree(save);
    save = nullptr;
    save_cells = 0;
    solves.clear();
    batches.clear();
}

namespace {

int ensure_save(Autotuner &T, size_t cells)
{
    if (cells <= T.save_cells) return PCD_OK;
    if (T.save) cudaFree(T.save);
    T.save = nullptr;
    T.save_cells = 0;
    PCD_CUDA(cudaMalloc(&T.save, cells * sizeof(double)));
    T.save_cells = cells;
    return PCD_OK;
}

long long bits(double d)
{
    long long b;
    std::memcpy(&b, &d, 8);
    return b;
}

std::vector<TunedSolve> solve_candidates(const pcd_solve_opts &o)
{
    std::vector<TunedSolve> c;
    auto add = [&](int ce, double drop, int re, int sched, int ks = 0) {
        TunedSolve t;
        t.check_every = ce;
        t.refine_drop = drop;
        t.refine_every = re;
        t.schedule = sched;
        t.block_sweeps = ks;
        c.push_back(t);
    };
    if (o.precision == PCD_PREC_MIXED && o.stop == PCD_STOP_REL_RESIDUAL) {
        // cluster (when the grid fits): residual-estimate spacing and cycle drop
        for (int ce : {8, 16, 32, 64}) add(ce, 3e-2, 0, PCD_SCHED_AUTO);
        add(32, 1e-1, 0, PCD_SCHED_AUTO);
        // grids beyond one cluster: the persistent, tile and stream schedules
        // with the FP32 sweeps between FP64 refreshes
        add(32, 0.0, 0, PCD_SCHED_PERSISTENT);
        for (int re : {128, 512}) add(4, 0.0, re, PCD_SCHED_TILES);
        for (int re : {128, 512}) add(0, 0.0, re, PCD_SCHED_STREAM);
    } else if (o.precision == PCD_PREC_MIXED) {
        for (int re : {32, 64, 128}) add(0, 0.0, re, PCD_SCHED_AUTO);
        add(0, 0.0, 0, PCD_SCHED_PERSISTENT);
    } else {
        // the block schedule with 2 or 4 sweeps per halo exchange (grids that
        // fit on chip), the persistent bands, stripes and launches
        for (int ks : {4, 2})
            for (int ce : {16, 32}) add(ce, 0.0, 0, PCD_SCHED_BLOCKS, ks);
        add(32, 0.0, 0, PCD_SCHED_PERSISTENT);
        add(32, 0.0, 0, PCD_SCHED_STRIPES);
        add(32, 0.0, 0, PCD_SCHED_LAUNCHES);
    }
    return c;
}

pcd_solve_opts apply(pcd_solve_opts o, const TunedSolve &t)
{
    o.check_every = t.check_every;
    o.refine_every = t.refine_every;
    o.refine_drop = t.refine_drop;
    o.schedule = t.schedule;
    o.block_sweeps = t.block_sweeps;
    return o;
}

void note(pcd_solve_stats *stats, const TunedSolve &t, int tuned)
{
    if (!stats) return;
    stats->tuned = tuned;
    stats->check_every_used = t.check_every;
    stats->refine_every_used = t.refine_every;
    stats->refine_drop_used = t.refine_drop;
}

int copy_grid(double *dst, int dld, const double *src, int sld, int W, int H, cudaStream_t s)
{
    PCD_CUDA(cudaMemcpy2DAsync(dst, (size_t)dld * sizeof(double), src, (size_t)sld * sizeof(double),
                               (size_t)W * sizeof(double), H, cudaMemcpyDeviceToDevice, s));
    return PCD_OK;
}

}  // namespace

int solve_autotuned(pcd_ctx *ctx, const double *b, double *phi, int W, int H, int ld, const pcd_solve_opts &o,
                    pcd_solve_stats *stats, cudaStream_t s)
{
    Autotuner &T = ctx->tuner;
    const bool pinned = o.schedule != PCD_SCHED_AUTO || o.check_every != 0 || o.refine_every != 0 ||
                        o.refine_drop != 0.0 || o.block_sweeps != 0;
    if (!T.enabled || pinned) {
        TunedSolve given;
        given.check_every = o.check_every;
        given.refine_every = o.refine_every;
        given.refine_drop = o.refine_drop;
        given.schedule = o.schedule;
        given.block_sweeps = o.block_sweeps;
        const int st = solve_device(ctx->solver, b, phi, W, H, ld, o, stats, s);
        note(stats, given, 0);
        return st;
    }
    const std::vector<long long> key = {W, H, o.precision, o.stop};
    auto it = T.solves.find(key);
    if (it != T.solves.end()) {
        const int st = solve_device(ctx->solver, b, phi, W, H, ld, apply(o, it->second), stats, s);
        note(stats, it->second, 1);
        return st;
    }
    // snapshot phi (the warm start, or whatever the caller left for a zero start)
    PCD_TRY(ensure_save(T, (size_t)W * H));
    PCD_TRY(copy_grid(T.save, W, phi, ld, W, H, s));
    const std::vector<TunedSolve> cand = solve_candidates(o);
    int best = -1;
    double best_ms = 0.0;
    bool best_conv = false;
    for (size_t i = 0; i < cand.size(); i++) {
        PCD_TRY(copy_grid(phi, ld, T.save, W, W, H, s));
        pcd_solve_stats st{};
        const int rc = solve_device(ctx->solver, b, phi, W, H, ld, apply(o, cand[i]), &st, s);
        T.trials++;
        if (rc != PCD_OK && rc != PCD_NOT_CONVERGED) {
            if (rc == PCD_BAD_ARG) continue;  // candidate does not apply to this grid
            return rc;
        }
        const bool conv = st.converged != 0;
        if (best < 0 || (conv && !best_conv) || (conv == best_conv && st.device_ms < best_ms)) {
            best = (int)i;
            best_ms = st.device_ms;
            best_conv = conv;
        }
    }
    if (best < 0) {
        set_error("autotuner: no candidate setting ran");
        return PCD_BAD_ARG;
    }
    T.solves[key] = cand[best];
    PCD_TRY(copy_grid(phi, ld, T.save, W, W, H, s));
    const int st = solve_device(ctx->solver, b, phi, W, H, ld, apply(o, cand[best]), stats, s);
    note(stats, cand[best], 1);
    return st;
}

int batch_autotuned(pcd_ctx *ctx, const pcd_instance *inst, int count, const pcd_solve_opts &o,
                    pcd_instance_stats *stats, pcd_batch_stats *bstats, cudaStream_t s)
{
    Autotuner &T = ctx->tuner;
    const bool pinned = o.check_every != 0 || o.refine_drop != 0.0;
    if (!T.enabled || pinned || count < 1 || !inst) {
        const int st = batch_solve_device(ctx->batch, ctx->device, inst, count, o, stats, bstats, s);
        return st;
    }
    std::vector<long long> key = {o.precision, bits(o.tol), o.max_iterations, o.warm_start ? 1 : 0};
    {
        std::vector<long long> sizes;
        for (int i = 0; i < count; i++) sizes.push_back(((long long)inst[i].width << 32) | inst[i].height);
        std::sort(sizes.begin(), sizes.end());
        key.insert(key.end(), sizes.begin(), sizes.end());
    }
    auto run = [&](const TunedBatch &t, pcd_instance_stats *st, pcd_batch_stats *bs) {
        pcd_solve_opts q = o;
        q.check_every = t.check_every;
        q.refine_drop = t.refine_drop;
        return batch_solve_device(ctx->batch, ctx->device, inst, count, q, st, bs, s, t.cluster);
    };
    auto it = T.batches.find(key);
    if (it != T.batches.end()) {
        const int st = run(it->second, stats, bstats);
        if (bstats) bstats->tuned = 1;
        return st;
    }
    // warm starts: snapshot every instance's phi to restore it between trials
    size_t total = 0;
    if (o.warm_start) {
        for (int i = 0; i < count; i++) total += (size_t)inst[i].width * inst[i].height;
        PCD_TRY(ensure_save(T, total));
        size_t off = 0;
        for (int i = 0; i < count; i++) {
            PCD_TRY(copy_grid(T.save + off, inst[i].width, inst[i].phi, inst[i].ld, inst[i].width, inst[i].height, s));
            off += (size_t)inst[i].width * inst[i].height;
        }
    }
    auto restore = [&]() {
        if (!o.warm_start) return (int)PCD_OK;
        size_t off = 0;
        for (int i = 0; i < count; i++) {
            PCD_TRY(copy_grid(inst[i].phi, inst[i].ld, T.save + off, inst[i].width, inst[i].width, inst[i].height, s));
            off += (size_t)inst[i].width * inst[i].height;
        }
        return (int)PCD_OK;
    };
    std::vector<TunedBatch> cand;
    for (int cl : {16, 8})
        for (int ce : {16, 32}) {
            TunedBatch t;
            t.cluster = cl;
            t.check_every = ce;
            t.refine_drop = 3e-2;
            cand.push_back(t);
        }
    if (batch_tiles_apply(inst, count)) {
        // the batched tile passes (cluster 0 with the default schedule)
        TunedBatch t;
        t.cluster = 0;
        t.check_every = 0;
        t.refine_drop = 0.0;
        cand.push_back(t);
    }
    std::vector<pcd_instance_stats> tmp((size_t)count);
    int best = -1;
    double best_ms = 0.0;
    bool best_conv = false;
    for (size_t i = 0; i < cand.size(); i++) {
        PCD_TRY(restore());
        pcd_batch_stats bs{};
        const int rc = run(cand[i], tmp.data(), &bs);
        T.trials++;
        if (rc != PCD_OK && rc != PCD_NOT_CONVERGED) {
            if (rc == PCD_BAD_ARG) continue;
            return rc;
        }
        bool conv = true;
        for (int k = 0; k < count; k++) conv = conv && tmp[(size_t)k].converged;
        if (best < 0 || (conv && !best_conv) || (conv == best_conv && bs.device_ms < best_ms)) {
            best = (int)i;
            best_ms = bs.device_ms;
            best_conv = conv;
        }
    }
    if (best < 0) {
        set_error("autotuner: no candidate batch setting ran");
        return PCD_BAD_ARG;
    }
    T.batches[key] = cand[best];
    PCD_TRY(restore());
    const int st = run(cand[best], stats, bstats);
    if (bstats) bstats->tuned = 1;
    return st;
}

}  // namespace pcd

using namespace pcd;

extern "C" {

int pcd_ctx_set_autotune(pcd_ctx *ctx, int enable)
{
    if (!ctx) return PCD_BAD_ARG;
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->tuner.enabled = enable ? 1 : 0;
    return PCD_OK;
}

int pcd_ctx_autotune_info(pcd_ctx *ctx, int *entries, long long *trials)
{
    if (!ctx) return PCD_BAD_ARG;
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (entries) *entries = (int)(ctx->tuner.solves.size() + ctx->tuner.batches.size());
    if (trials) *trials = ctx->tuner.trials;
    return PCD_OK;
}

}  // extern "C"
