// sor_batch.cu -- many independent Poisson solves of uneven sizes in one
// persistent launch (sm_103a).
//
// The grid is a set of 16-CTA thread-block clusters (as many as are
// co-resident).  Each cluster takes the next instance from an atomic work
// counter -- instances are sorted by estimated cost, largest first, so the
// queue is a longest-processing-time-first schedule -- and runs the whole
// mixed-precision solve of that instance by itself:
//   1. FP64 residual r = b - L phi over its 16 SMs (phi = 0 or the warm start),
//      ||b||, r32 = (float) r into the colour planes;
//   2. cycles of FP32 red-black sweeps on the colour planes (sor_planes.cuh),
//      ended by the FP32 residual estimate (a 3e-2 drop, or half the
//      tolerance);
//   3. FP64 defect correction r = b - L(phi + e), phi += e, e = 0, stop test
//      ||r|| / ||b|| <= tol; back to 2 until it passes or max_iterations.
// The planes live in shared memory when the instance fits (<= ~512^2 with 16
// CTAs), otherwise in an L2-resident global scratch region of the cluster.
// Every exit decision of a cluster is computed by all its CTAs from the same
// partial sums in the same order, so all CTAs pass the same cluster barriers;
// there is no inter-cluster synchronisation at all.
#include <algorithm>
#include <cstring>
#include <numeric>

#include "sor_batch.cuh"
#include "sor_planes.cuh"

namespace pcd {

namespace {

using namespace planes;

constexpr int kBatchThreads = 1024;

__device__ void zero_own_rows(const Planes &P, int n)
{
    const long m = (long)(n + 2) * P.KHp;
    for (long t = threadIdx.x; t < m; t += blockDim.x) {
        P.e0[t] = 0.f;
        P.e1[t] = 0.f;
    }
}

// FP64 defect correction of the band: r = b - L(phi + e) (e ignored when
// init), r32 planes = (float) r; returns the cluster-wide sums of r^2 and
// (init) b^2.  Unless init, then phi += e and e = 0.  Ends with every CTA's
// phi update visible to the cluster.
__device__ void refine(cg::cluster_group &cl, const Planes &P, const BatchInst &I, const Grid &G, int g, int C,
                       int n, int r0, bool init, double *s_red, double *s_part2, double &r2, double &b2)
{
    const int W = G.W, H = G.H, ld = I.ld, KHp = P.KHp;
    if (!init) {
        fetch_halo_plane(cl, P, 0, g, C, n, H);
        fetch_halo_plane(cl, P, 1, g, C, n, H);
        __syncthreads();
    }
    const double *ph = I.phi;
    double ar = 0.0, ab = 0.0;
    for (int t = threadIdx.x; t < n * W; t += blockDim.x) {
        const int row = t / W, x = t - row * W, y = r0 + row;
        const size_t gi = (size_t)y * ld + x;
        const int c = (x + y) & 1, kk = x >> 1;
        const size_t ro = (size_t)(row + 1) * KHp;
        const float *oth = P.e(c ^ 1);
        const int q = 1 - ((y & 1) ^ c);
        double sum = 0.0, cnt = 0.0;
        if (x > 0) { sum += __ldcg(ph + gi - 1) + (init ? 0.0 : (double)oth[ro + kk - q]); cnt += 1.0; }
        if (x < W - 1) { sum += __ldcg(ph + gi + 1) + (init ? 0.0 : (double)oth[ro + kk - q + 1]); cnt += 1.0; }
        if (y > 0) { sum += __ldcg(ph + gi - ld) + (init ? 0.0 : (double)oth[ro - KHp + kk]); cnt += 1.0; }
        if (y < H - 1) { sum += __ldcg(ph + gi + ld) + (init ? 0.0 : (double)oth[ro + KHp + kk]); cnt += 1.0; }
        const double xi = __ldcg(ph + gi) + (init ? 0.0 : (double)P.e(c)[ro + kk]);
        const double bi = I.b[gi];
        const double r = bi - (sum - cnt * xi);
        P.r(c)[ro - KHp + kk] = (float)r;
        ar += r * r;
        if (init) ab += bi * bi;
    }
    ar = block_sum(ar, s_red);
    ab = block_sum(ab, s_red);
    if (threadIdx.x == 0) {
        s_part2[0] = ar;
        s_part2[1] = ab;
    }
    double tr, tb;
    // ends with a cluster barrier: partials read, and every CTA is done
    // reading its neighbours' phi
    cluster_sum2(cl, s_part2, s_red, C, tr, tb);
    r2 = tr;
    b2 = tb;
    if (!init) {
        double *phw = I.phi;
        for (int t = threadIdx.x; t < n * W; t += blockDim.x) {
            const int row = t / W, x = t - row * W, y = r0 + row;
            const int c = (x + y) & 1;
            float *ep = P.e(c) + (size_t)(row + 1) * KHp + (x >> 1);
            phw[(size_t)y * ld + x] += (double)(*ep);
            *ep = 0.f;
        }
        cl.sync();
    }
}

__global__ void __launch_bounds__(kBatchThreads, 1) k_sor_batch(BatchArgs a)
{
    cg::cluster_group cl = cg::this_cluster();
    extern __shared__ __align__(16) float smem_f[];
    __shared__ double s_red[32];
    __shared__ double s_part[1];
    __shared__ double s_part2[2];
    __shared__ int s_job;
    const int C = (int)cl.num_blocks(), g = (int)cl.block_rank();
    const int cluster_id = blockIdx.x / C;

    for (;;) {
        if (g == 0 && threadIdx.x == 0) s_job = (int)atomicAdd(a.counter, 1u);
        cl.sync();
        const int job = *cl.map_shared_rank(&s_job, 0);
        cl.sync();
        if (job >= a.count) break;
        BatchInst &I = a.inst[job];
        Grid G;
        G.W = I.W;
        G.H = I.H;
        G.w0 = I.w32[0]; G.w1 = I.w32[1]; G.w2 = I.w32[2]; G.w3 = I.w32[3]; G.w4 = I.w32[4];
        int r0, n;
        band_of(g, C, G.H, r0, n);
        const int nmax = (G.H + C - 1) / C;
        Planes P;
        P.KHp = I.khp;
        P.in_smem = I.in_smem;
        P.cta_stride = planes_floats(nmax, P.KHp);
        float *base = I.in_smem ? smem_f
                                : a.gscratch + (size_t)cluster_id * a.gscratch_per_cluster + (size_t)g * P.cta_stride;
        carve(P, base, nmax);
        const int KH4 = P.KHp >> 2;
        const int RP = blockDim.x / KH4;
        const int k = 4 * (threadIdx.x % KH4), rg = threadIdx.x / KH4;

        zero_own_rows(P, n);
        if (!a.warm_start)
            for (int t = threadIdx.x; t < n * G.W; t += blockDim.x) {
                const int row = t / G.W, x = t - row * G.W;
                I.phi[(size_t)(r0 + row) * I.ld + x] = 0.0;
            }
        __syncthreads();
        cl.sync();

        double r2, b2;
        refine(cl, P, I, G, g, C, n, r0, true, s_red, s_part2, r2, b2);
        const double bnorm = sqrt(b2);
        double rel = bnorm > 0.0 ? sqrt(r2) / bnorm : sqrt(r2);
        bool converged = rel <= I.tol;
        int sweeps = 0, cycles = 0;
        while (!converged && sweeps < I.max_iter) {
            const double stop_abs = kFp32StopFrac * I.tol * bnorm;
            const double drop_abs = a.drop * sqrt(r2);
            int cyc = 0;
            for (;;) {
                for (int c = 0; c < 2; c++) {
                    fetch_halo_plane(cl, P, c ^ 1, g, C, n, G.H);
                    __syncthreads();
                    relax_quad(P, c, n, r0, G, k, rg, RP);
                    cl.sync();
                }
                ++cyc;
                ++sweeps;
                const bool cap = cyc >= a.cycle_cap || sweeps >= I.max_iter;
                if (cyc % a.check_every == 0 || cap) {
                    fetch_halo_plane(cl, P, 0, g, C, n, G.H);
                    fetch_halo_plane(cl, P, 1, g, C, n, G.H);
                    __syncthreads();
                    const double v = block_sum((double)residual_rows_quad(P.e0, P.e1, P.r0, P.r1, -(long)P.KHp, 1,
                                                                          n + 1, r0 - 1, G, P.KHp, k, rg, RP),
                                               s_red);
                    if (threadIdx.x == 0) s_part[0] = v;
                    const double est = sqrt(cluster_sum(cl, s_part, s_red, C));
                    if (cap || est <= stop_abs || est <= drop_abs) break;
                }
            }
            refine(cl, P, I, G, g, C, n, r0, false, s_red, s_part2, r2, b2);
            ++cycles;
            rel = bnorm > 0.0 ? sqrt(r2) / bnorm : sqrt(r2);
            converged = rel <= I.tol;
        }
        if (g == 0 && threadIdx.x == 0) {
            I.sweeps = sweeps;
            I.converged = converged ? 1 : 0;
            I.cycles = cycles;
            I.rel = rel;
        }
    }
}

}  // namespace

int BatchWorkspace::reserve_inst(int count)
{
    if (count > cap) {
        // cached graphs hold the old descriptor addresses: drop them with them
        for (auto &kv : graphs) cudaGraphExecDestroy(kv.second);
        graphs.clear();
        if (d_inst) cudaFree(d_inst);
        if (h_inst) cudaFreeHost(h_inst);
        d_inst = nullptr;
        h_inst = nullptr;
        cap = 0;
        PCD_CUDA(cudaMalloc(&d_inst, sizeof(BatchInst) * count));
        PCD_CUDA(cudaMallocHost(&h_inst, sizeof(BatchInst) * count));
        cap = count;
    }
    if (!counter) PCD_CUDA(cudaMalloc(&counter, sizeof(unsigned)));
    if (!t0) {
        PCD_CUDA(cudaEventCreate(&t0));
        PCD_CUDA(cudaEventCreate(&t1));
    }
    return PCD_OK;
}

void BatchWorkspace::release()
{
    tiles.release();
    for (auto &kv : graphs) cudaGraphExecDestroy(kv.second);
    graphs.clear();
    if (d_inst) cudaFree(d_inst);
    if (h_inst) cudaFreeHost(h_inst);
    if (gscratch) cudaFree(gscratch);
    if (counter) cudaFree(counter);
    if (t0) cudaEventDestroy(t0);
    if (t1) cudaEventDestroy(t1);
    d_inst = nullptr;
    h_inst = nullptr;
    gscratch = nullptr;
    counter = nullptr;
    t0 = t1 = nullptr;
    cap = 0;
    gscratch_floats = 0;
}

int batch_solve_device(BatchWorkspace &ws, int dev, const pcd_instance *inst, int count, const pcd_solve_opts &o,
                       pcd_instance_stats *stats, pcd_batch_stats *bstats, cudaStream_t s, int cluster)
{
    if (!inst || count < 1) {
        set_error("pcd_batch_solve_device: empty batch");
        return PCD_BAD_ARG;
    }
    if (o.stop != PCD_STOP_REL_RESIDUAL || !(o.tol > 0.0) || o.max_iterations < 1) {
        set_error("pcd_batch_solve_device: the batch solve takes the relative-residual stop with tol > 0");
        return PCD_BAD_ARG;
    }
    if (cluster != 0 && cluster != 8 && cluster != 16) {
        set_error("pcd_batch_solve_device: cluster size must be 8 or 16");
        return PCD_BAD_ARG;
    }
    // the batched tile passes take any height and width (widths multiples of
    // 8); the cluster form's limits below apply only to batches it solves
    if (cluster == 0 && o.schedule != PCD_SCHED_CLUSTER && batch_tiles_apply(inst, count))
        return batch_tiles_solve(ws.tiles, dev, inst, count, o, stats, bstats, s);
    const int C = cluster ? cluster : 16;
    for (int i = 0; i < count; i++) {
        const pcd_instance &q = inst[i];
        if (!q.b || !q.phi || q.width < 2 || q.height < 2 * C || q.ld < q.width ||
            plane_stride(q.width) / 2 > kBatchThreads) {
            set_error("pcd_batch_solve_device: instance " + std::to_string(i) +
                      " needs 2 <= width <= 4096, height >= 2 x cluster size, ld >= width and device arrays "
                      "(the cluster form; the tile form takes widths that are multiples of 8 and ld of 4)");
            return PCD_BAD_ARG;
        }
    }
    PCD_TRY(ws.reserve_inst(count));

    // largest first (cost ~ cells x sweeps ~ W*H*max(W,H))
    std::vector<int> order(count);
    std::iota(order.begin(), order.end(), 0);
    auto cost = [&](int i) {
        const double w = inst[i].width, h = inst[i].height;
        return w * h * std::max(w, h);
    };
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return cost(x) > cost(y); });

    int max_smem = 0;
    PCD_CUDA(cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    const size_t smem_cap = (size_t)max_smem - 4096;
    size_t smem = 0, gper = 0;
    for (int j = 0; j < count; j++) {
        const pcd_instance &q = inst[order[j]];
        const int nmax = (q.height + C - 1) / C;
        const size_t bytes = (size_t)planes_floats(nmax, plane_stride(q.width)) * sizeof(float);
        if (bytes <= smem_cap) smem = std::max(smem, bytes);
        else gper = std::max(gper, (size_t)C * planes_floats(nmax, plane_stride(q.width)));
    }
    PCD_CUDA(cudaFuncSetAttribute((const void *)k_sor_batch, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    PCD_CUDA(cudaFuncSetAttribute((const void *)k_sor_batch, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)std::max<size_t>(smem, 16)));
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.blockDim = dim3(kBatchThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cfg.gridDim = dim3(C);
    int ncl = 0;
    PCD_CUDA(cudaOccupancyMaxActiveClusters(&ncl, (const void *)k_sor_batch, &cfg));
    if (ncl < 1) {
        set_error("pcd_batch_solve_device: no " + std::to_string(C) + "-CTA cluster fits on this device");
        return PCD_BAD_ARG;
    }
    ncl = std::min(ncl, count);
    if (gper * ncl > ws.gscratch_floats) {
        // cached graphs hold the old scratch address: drop them with it
        for (auto &kv : ws.graphs) cudaGraphExecDestroy(kv.second);
        ws.graphs.clear();
        if (ws.gscratch) cudaFree(ws.gscratch);
        ws.gscratch = nullptr;
        ws.gscratch_floats = 0;
        PCD_CUDA(cudaMalloc(&ws.gscratch, gper * ncl * sizeof(float)));
        ws.gscratch_floats = gper * ncl;
    }

    for (int j = 0; j < count; j++) {
        const pcd_instance &q = inst[order[j]];
        BatchInst &d = ws.h_inst[j];
        std::memset(&d, 0, sizeof(d));
        d.W = q.width;
        d.H = q.height;
        d.ld = q.ld;
        d.khp = plane_stride(q.width);
        d.b = q.b;
        d.phi = q.phi;
        const double om = resolve_omega(o.omega, q.width, q.height);
        for (int c = 0; c < 5; c++) d.w32[c] = (float)om / (float)c;
        d.tol = o.tol;
        d.max_iter = o.max_iterations;
        const int nmax = (q.height + C - 1) / C;
        d.in_smem = (size_t)planes_floats(nmax, d.khp) * sizeof(float) <= smem_cap ? 1 : 0;
    }

    BatchArgs ba{};
    ba.inst = ws.d_inst;
    ba.count = count;
    ba.counter = ws.counter;
    ba.gscratch = ws.gscratch;
    ba.gscratch_per_cluster = gper;
    ba.check_every = o.check_every > 0 ? o.check_every : 16;
    ba.cycle_cap = o.refine_every > 0 ? o.refine_every : 4096;
    ba.drop = o.refine_drop > 0.0 ? o.refine_drop : 3e-2;
    ba.warm_start = o.warm_start ? 1 : 0;
    cfg.gridDim = dim3(ncl * C);
    cfg.stream = s;

    // one CUDA graph per batch signature: upload descriptors, reset the work
    // counter, the persistent launch, read the descriptors (statistics) back
    long long drop_bits;
    std::memcpy(&drop_bits, &ba.drop, 8);
    std::vector<long long> key = {count, C, ncl, (long long)smem, ba.check_every, ba.cycle_cap, ba.warm_start,
                                  drop_bits};
    for (int j = 0; j < count; j++) {
        const BatchInst &d = ws.h_inst[j];
        long long tb;
        std::memcpy(&tb, &d.tol, 8);
        key.insert(key.end(), {(long long)d.W, (long long)d.H, (long long)d.ld, (long long)(uintptr_t)d.b,
                               (long long)(uintptr_t)d.phi, tb, (long long)d.max_iter, (long long)d.in_smem,
                               (long long)(d.w32[1] * 1e7)});
    }
    cudaGraphExec_t exec = nullptr;
    auto it = ws.graphs.find(key);
    if (it != ws.graphs.end()) {
        exec = it->second;
    } else {
        cudaGraph_t gph;
        PCD_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        cudaMemcpyAsync(ws.d_inst, ws.h_inst, sizeof(BatchInst) * count, cudaMemcpyHostToDevice, s);
        cudaMemsetAsync(ws.counter, 0, sizeof(unsigned), s);
        cudaError_t le = cudaLaunchKernelEx(&cfg, k_sor_batch, ba);
        cudaMemcpyAsync(ws.h_inst, ws.d_inst, sizeof(BatchInst) * count, cudaMemcpyDeviceToHost, s);
        cudaError_t ce = cudaStreamEndCapture(s, &gph);
        if (le != cudaSuccess || ce != cudaSuccess) {
            if (ce == cudaSuccess) cudaGraphDestroy(gph);
            set_error(std::string("batch graph capture: ") + cudaGetErrorString(le != cudaSuccess ? le : ce));
            return PCD_DEVICE_ERROR;
        }
        ce = cudaGraphInstantiate(&exec, gph, 0);
        cudaGraphDestroy(gph);
        if (ce != cudaSuccess) {
            set_error(std::string("batch graph instantiate: ") + cudaGetErrorString(ce));
            return PCD_DEVICE_ERROR;
        }
        if (ws.graphs.size() > 16) {
            for (auto &kv : ws.graphs) cudaGraphExecDestroy(kv.second);
            ws.graphs.clear();
        }
        ws.graphs[key] = exec;
    }
    PCD_CUDA(cudaEventRecord(ws.t0, s));
    PCD_CUDA(cudaGraphLaunch(exec, s));
    count_launches(1);
    PCD_CUDA(cudaEventRecord(ws.t1, s));
    PCD_CUDA(cudaStreamSynchronize(s));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ws.t0, ws.t1);

    int all = 1;
    long long cell_sweeps = 0;
    for (int j = 0; j < count; j++) {
        const BatchInst &d = ws.h_inst[j];
        const int i = order[j];
        if (stats) {
            stats[i].sweeps = d.sweeps;
            stats[i].converged = d.converged;
            stats[i].rel_residual = d.rel;
            stats[i].cycles = d.cycles;
        }
        all &= d.converged;
        cell_sweeps += (long long)d.W * d.H * d.sweeps;
    }
    if (bstats) {
        bstats->device_ms = ms;
        bstats->clusters = ncl;
        bstats->cluster_size = C;
        bstats->smem_bytes = (long long)smem;
        bstats->cell_sweeps = cell_sweeps;
        bstats->check_every = ba.check_every;
        bstats->refine_drop = ba.drop;
        bstats->tuned = 0;
    }
    return all ? PCD_OK : PCD_NOT_CONVERGED;
}

}  // namespace pcd
