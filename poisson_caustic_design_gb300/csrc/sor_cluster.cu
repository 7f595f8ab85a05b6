// sor_cluster.cu -- FP32 red-black SOR on one thread-block cluster (sm_103a).
//
// The mixed-precision solve alternates two kernels:
//   k_sor_cluster   FP32 sweeps on the correction equation L e = r32, the
//                   whole grid resident in the distributed shared memory of
//                   one cluster of up to 16 CTAs (one per SM);
//   k_refine_*      (solver.cu) the FP64 defect correction on every SM:
//                   r = b - L(phi + e), phi += e, e = 0, r32 = (float) r.
//
// Inside the cluster CTA g owns the rows [r0, r0+n) of e and r32.  A half
// sweep reads the facing boundary row of each neighbouring CTA straight from
// that CTA's shared memory (DSMEM) into a local halo row, relaxes its own
// cells of one colour, and ends with the hardware cluster barrier
// (barrier.cluster arrive.release / wait.acquire).  Reading the neighbour's
// row while it relaxes the other colour is race free: a cell of colour c only
// needs neighbours of colour 1-c, which were final at the previous barrier.
//
// Every `check_every` sweeps the cluster evaluates the FP32 residual
// ||r32 - L e|| (FP64 accumulation); all CTAs read the same per-CTA partials
// after a barrier and take the same exit decision, so they execute the same
// sequence of barriers.  A cycle ends when that estimate has dropped by
// `drop` (the FP32 iteration cannot resolve much more than two digits of the
// correction) or is below half the stop tolerance, or at the sweep caps; the
// FP64 residual then decides convergence.
#include <cooperative_groups.h>

#include "sor_cluster.cuh"

namespace cg = cooperative_groups;

namespace pcd {

namespace {

__device__ __forceinline__ void band_of(int g, int G, int H, int &r0, int &n)
{
    const int base = H / G, extra = H % G;
    n = base + (g < extra ? 1 : 0);
    r0 = g * base + (g < extra ? g : extra);
}

__device__ __forceinline__ float w_of(const ClusterArgs &a, int cnt)
{
    return cnt == 4 ? a.w32[4] : cnt == 3 ? a.w32[3] : cnt == 2 ? a.w32[2] : cnt == 1 ? a.w32[1] : a.w32[0];
}

// Copy the neighbours' facing rows into halo rows 0 and n+1 of se.
__device__ __forceinline__ void fetch_halos(cg::cluster_group &cl, float *se, int g, int C, int n, int H, int W)
{
    if (g > 0) {
        int pr0, pn;
        band_of(g - 1, C, H, pr0, pn);
        const float *src = cl.map_shared_rank(se, g - 1) + (size_t)pn * W;  // its last own row
        for (int c = threadIdx.x; c < W; c += blockDim.x) se[c] = src[c];
    }
    if (g < C - 1) {
        const float *src = cl.map_shared_rank(se, g + 1) + (size_t)W;       // its first own row
        for (int c = threadIdx.x; c < W; c += blockDim.x) se[(size_t)(n + 1) * W + c] = src[c];
    }
}

__device__ __forceinline__ void relax(float *se, const float *sr, int n, int r0, const ClusterArgs &a, int color)
{
    const int W = a.W, H = a.H, half = (W + 1) >> 1;
    int row = 0, k = threadIdx.x;
    while (k >= half && row < n) { k -= half; row++; }
    while (row < n) {
        const int y = r0 + row;
        const int x = 2 * k + ((y + color) & 1);
        if (x < W) {
            float *c = se + (size_t)(row + 1) * W + x;
            float sum = 0.f;
            int cnt = 0;
            if (x > 0) { sum += c[-1]; cnt++; }
            if (y > 0) { sum += c[-W]; cnt++; }
            if (x < W - 1) { sum += c[1]; cnt++; }
            if (y < H - 1) { sum += c[W]; cnt++; }
            const float v = *c;
            *c = v + w_of(a, cnt) * (sum - (float)cnt * v - sr[(size_t)row * W + x]);
        }
        k += blockDim.x;
        while (k >= half) { k -= half; row++; }
    }
}

// sum over own cells of (r32 - L e)^2 in FP64 accumulation
__device__ __forceinline__ double residual_sq(const float *se, const float *sr, int n, int r0, const ClusterArgs &a)
{
    const int W = a.W, H = a.H;
    double acc = 0.0;
    for (int t = threadIdx.x; t < n * W; t += blockDim.x) {
        const int row = t / W, x = t - row * W, y = r0 + row;
        const float *c = se + (size_t)(row + 1) * W + x;
        float sum = 0.f;
        int cnt = 0;
        if (x > 0) { sum += c[-1]; cnt++; }
        if (y > 0) { sum += c[-W]; cnt++; }
        if (x < W - 1) { sum += c[1]; cnt++; }
        if (y < H - 1) { sum += c[W]; cnt++; }
        const float r = sr[t] - (sum - (float)cnt * (*c));
        acc += (double)r * (double)r;
    }
    return acc;
}

__global__ void __launch_bounds__(kClusterThreads, 1) k_sor_cluster(ClusterArgs a)
{
    cg::cluster_group cl = cg::this_cluster();
    extern __shared__ __align__(16) float smem_f[];
    __shared__ double s_part[1];
    __shared__ double s_red[32];
    const int C = (int)cl.num_blocks(), g = (int)cl.block_rank(), W = a.W;
    int r0, n;
    band_of(g, C, a.H, r0, n);
    const int nmax = (a.H + C - 1) / C;
    float *se = smem_f;                          // (nmax+2) x W: halo, own rows, halo
    float *sr = smem_f + (size_t)(nmax + 2) * W; // nmax x W

    const Ctl *ctl = a.ctl;
    if (*(volatile const int *)&ctl->done) return;  // speculative launch after convergence: all CTAs agree
    for (int t = threadIdx.x; t < n * W; t += blockDim.x) {
        const int row = t / W, x = t - row * W;
        const size_t gi = (size_t)(r0 + row) * a.ld + x;
        se[(size_t)(row + 1) * W + x] = a.e[gi];
        sr[t] = a.r32[gi];
    }
    const int done_before = *(volatile const int *)&ctl->sweeps;
    const double bnorm = *(volatile const double *)&ctl->bnorm;
    const double rstart = *(volatile const double *)&ctl->rnorm;
    const double stop_abs = 0.5 * a.tol * bnorm;       // verify in FP64 below this
    const double drop_abs = a.drop * rstart;
    cl.sync();

    int sweeps = 0;
    double est = rstart;
    for (;;) {
        for (int color = 0; color < 2; color++) {
            fetch_halos(cl, se, g, C, n, a.H, W);
            __syncthreads();
            relax(se, sr, n, r0, a, color);
            cl.sync();
        }
        ++sweeps;
        const bool cap = sweeps >= a.cycle_cap || done_before + sweeps >= a.max_iter;
        if (sweeps % a.check_every == 0 || cap) {
            fetch_halos(cl, se, g, C, n, a.H, W);
            __syncthreads();
            double v = residual_sq(se, sr, n, r0, a);
            v = warp_sum(v);
            if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = v;
            __syncthreads();
            if (threadIdx.x == 0) {
                double t = 0.0;
                for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += s_red[w];
                s_part[0] = t;
            }
            cl.sync();
            // every CTA sums the same partials in the same order
            double tot = 0.0;
            for (int q = 0; q < C; q++) tot += *cl.map_shared_rank(s_part, q);
            est = sqrt(tot);
            cl.sync();
            if (cap || est <= stop_abs || est <= drop_abs) break;
        }
    }
    for (int t = threadIdx.x; t < n * W; t += blockDim.x) {
        const int row = t / W, x = t - row * W;
        a.e[(size_t)(r0 + row) * a.ld + x] = se[(size_t)(row + 1) * W + x];
    }
    if (g == 0 && threadIdx.x == 0) {
        volatile Ctl *c = a.ctl;
        c->sweeps = done_before + sweeps;
        if (done_before + sweeps >= a.max_iter) c->halt = 1;
    }
    cl.sync();
}

}  // namespace

int cluster_plan(int dev, int W, int H, int *C_out, size_t *smem_out)
{
    int max_smem = 0, cluster_ok = 0;
    PCD_CUDA(cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    PCD_CUDA(cudaDeviceGetAttribute(&cluster_ok, cudaDevAttrClusterLaunch, dev));
    if (!cluster_ok) return PCD_BAD_ARG;
    for (int C : {16, 8}) {
        if (H < 2 * C) continue;
        const int nmax = (H + C - 1) / C;
        const size_t smem = (size_t)(2 * nmax + 2) * W * sizeof(float);
        if (smem + 2048 > (size_t)max_smem) continue;
        PCD_CUDA(cudaFuncSetAttribute((const void *)k_sor_cluster, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
        PCD_CUDA(cudaFuncSetAttribute((const void *)k_sor_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(C);
        cfg.blockDim = dim3(kClusterThreads);
        cfg.dynamicSmemBytes = smem;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = C;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        int nclusters = 0;
        if (cudaOccupancyMaxActiveClusters(&nclusters, (const void *)k_sor_cluster, &cfg) != cudaSuccess) {
            cudaGetLastError();
            continue;
        }
        if (nclusters < 1) continue;
        *C_out = C;
        *smem_out = smem;
        return PCD_OK;
    }
    return PCD_BAD_ARG;
}

int launch_cluster(ClusterArgs &a, int C, size_t smem, cudaStream_t s)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(C);
    cfg.blockDim = dim3(kClusterThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    PCD_CUDA(cudaLaunchKernelEx(&cfg, k_sor_cluster, a));
    count_launches(1);
    return PCD_OK;
}

}  // namespace pcd
