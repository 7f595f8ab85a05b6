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

// Shared-memory layout of one CTA (all FP32, row stride KHp = even >= ceil(W/2)):
//   plane[0] = red  cells ((x+y) even) of e, rows 0..n+1 (0 and n+1: halos)
//   plane[1] = black cells of e, same shape
//   rhs[0], rhs[1] = red / black cells of r32, rows 0..n-1
// Cell (x, y) of colour c = (x+y)&1 lives at plane[c][(y - r0 + 1)*KHp + (x >> 1)].
// In row y (p = y&1) the cell of colour c at slot k sits at x = 2k + (p^c); its
// left and right neighbours (other colour) sit at slots k - q and k - q + 1
// with q = 1 - (p^c); its up and down neighbours at slot k of rows y-1, y+1.
struct Planes {
    float *e0, *e1;  // red, black planes of e
    float *r0, *r1;  // red, black planes of r32
    int KHp;
    __device__ __forceinline__ float *e(int c) const { return c ? e1 : e0; }
    __device__ __forceinline__ float *r(int c) const { return c ? r1 : r0; }
};

// Copy the neighbours' facing rows of plane `c` into its halo rows.
__device__ __forceinline__ void fetch_halo_plane(cg::cluster_group &cl, const Planes &P, int c, int g, int C, int n,
                                                 int H)
{
    float *pl = P.e(c);
    const int KHp = P.KHp, K4 = KHp >> 2;  // KHp is a multiple of 4
    if (g > 0) {
        int pr0, pn;
        band_of(g - 1, C, H, pr0, pn);
        const float4 *src = reinterpret_cast<const float4 *>(cl.map_shared_rank(pl, g - 1) + (size_t)pn * KHp);
        float4 *dst = reinterpret_cast<float4 *>(pl);
        for (int i = threadIdx.x; i < K4; i += blockDim.x) dst[i] = src[i];
    }
    if (g < C - 1) {
        const float4 *src = reinterpret_cast<const float4 *>(cl.map_shared_rank(pl, g + 1) + (size_t)KHp);
        float4 *dst = reinterpret_cast<float4 *>(pl + (size_t)(n + 1) * KHp);
        for (int i = threadIdx.x; i < K4; i += blockDim.x) dst[i] = src[i];
    }
}

// One half sweep of colour c over the band: each thread owns slot pair
// (k, k+1) of rows lr = 1 + rg, 1 + rg + RP, ...
__device__ __forceinline__ void relax_pair(const Planes &P, int c, int n, int r0, const ClusterArgs &a, int k, int rg,
                                          int RP)
{
    const int W = a.W, H = a.H, KHp = P.KHp;
    float *own = P.e(c);
    const float *oth = P.e(c ^ 1);
    const float *rhs = P.r(c);
    const float w1 = a.w32[1], w2 = a.w32[2], w3 = a.w32[3], w4 = a.w32[4];
    for (int lr = 1 + rg; lr <= n; lr += RP) {
        const int y = r0 + lr - 1;
        const int s = (y & 1) ^ c;     // x = 2k + s
        const int q = 1 - s;           // left neighbour slot = k - q
        const size_t ro = (size_t)lr * KHp;
        float2 v = *reinterpret_cast<float2 *>(own + ro + k);
        const float2 rh = *reinterpret_cast<const float2 *>(rhs + ro - KHp + k);
        const float2 up = *reinterpret_cast<const float2 *>(oth + ro - KHp + k);
        const float2 dn = *reinterpret_cast<const float2 *>(oth + ro + KHp + k);
        const float2 mid = *reinterpret_cast<const float2 *>(oth + ro + k);
        const float extra = oth[ro + (q ? k - 1 : k + 2)];
        const float l0 = q ? extra : mid.x, r0v = q ? mid.x : mid.y;
        const float l1 = q ? mid.x : mid.y, r1v = q ? mid.y : extra;
        const int x0 = 2 * k + s, x1 = x0 + 2;
        const bool hu = y > 0, hd = y < H - 1;
        const float vert0 = (hu ? up.x : 0.f) + (hd ? dn.x : 0.f);
        const float vert1 = (hu ? up.y : 0.f) + (hd ? dn.y : 0.f);
        const int cv = (int)hu + (int)hd;
        if (x0 < W) {
            const bool hl = x0 > 0, hr = x0 + 1 < W;
            const float sum = vert0 + (hl ? l0 : 0.f) + (hr ? r0v : 0.f);
            const int cnt = cv + (int)hl + (int)hr;
            const float w = cnt == 4 ? w4 : cnt == 3 ? w3 : cnt == 2 ? w2 : cnt == 1 ? w1 : a.w32[0];
            v.x = v.x + w * (sum - (float)cnt * v.x - rh.x);
        }
        if (x1 < W) {
            const bool hr = x1 + 1 < W;  // x1 >= 2 always has a left neighbour
            const float sum = vert1 + l1 + (hr ? r1v : 0.f);
            const int cnt = cv + 1 + (int)hr;
            const float w = cnt == 4 ? w4 : cnt == 3 ? w3 : cnt == 2 ? w2 : w1;
            v.y = v.y + w * (sum - (float)cnt * v.y - rh.y);
        }
        *reinterpret_cast<float2 *>(own + ro + k) = v;
    }
}

// sum over own cells of (r32 - L e)^2, both colours, FP64 accumulation
__device__ __forceinline__ double residual_sq(const Planes &P, int n, int r0, const ClusterArgs &a)
{
    const int W = a.W, H = a.H, KHp = P.KHp;
    double acc = 0.0;
    for (int t = threadIdx.x; t < n * W; t += blockDim.x) {
        const int row = t / W, x = t - row * W, y = r0 + row;
        const int c = (x + y) & 1, kk = x >> 1;
        const size_t ro = (size_t)(row + 1) * KHp;
        const float *oth = P.e(c ^ 1);
        const int s = (y & 1) ^ c, q = 1 - s;
        float sum = 0.f;
        int cnt = 0;
        if (x > 0) { sum += oth[ro + kk - q]; cnt++; }
        if (x < W - 1) { sum += oth[ro + kk - q + 1]; cnt++; }
        if (y > 0) { sum += oth[ro - KHp + kk]; cnt++; }
        if (y < H - 1) { sum += oth[ro + KHp + kk]; cnt++; }
        const float e = P.e(c)[ro + kk];
        const float r = P.r(c)[ro - KHp + kk] - (sum - (float)cnt * e);
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
    Planes P;
    P.KHp = a.khp;
    const size_t plane = (size_t)(nmax + 2) * P.KHp, rplane = (size_t)nmax * P.KHp;
    P.e0 = smem_f;
    P.e1 = smem_f + plane;
    P.r0 = smem_f + 2 * plane;
    P.r1 = smem_f + 2 * plane + rplane;

    const Ctl *ctl = a.ctl;
    if (*(volatile const int *)&ctl->done) return;  // speculative launch after convergence: all CTAs agree
    for (int t = threadIdx.x; t < n * W; t += blockDim.x) {
        const int row = t / W, x = t - row * W, y = r0 + row;
        const int c = (x + y) & 1;
        const size_t gi = (size_t)y * a.ld + x;
        P.e(c)[(size_t)(row + 1) * P.KHp + (x >> 1)] = a.e[gi];
        P.r(c)[(size_t)row * P.KHp + (x >> 1)] = a.r32[gi];
    }
    const int done_before = *(volatile const int *)&ctl->sweeps;
    const double bnorm = *(volatile const double *)&ctl->bnorm;
    const double rstart = *(volatile const double *)&ctl->rnorm;
    const double stop_abs = 0.5 * a.tol * bnorm;       // verify in FP64 below this
    const double drop_abs = a.drop * rstart;
    // thread -> (slot pair, row group)
    const int KH2 = P.KHp >> 1;
    const int RP = blockDim.x / KH2;
    const int k = 2 * (threadIdx.x % KH2), rg = threadIdx.x / KH2;
    const bool active = rg < RP;
    cl.sync();

    int sweeps = 0;
    for (;;) {
        for (int c = 0; c < 2; c++) {
            fetch_halo_plane(cl, P, c ^ 1, g, C, n, a.H);
            __syncthreads();
            if (active) relax_pair(P, c, n, r0, a, k, rg, RP);
            cl.sync();
        }
        ++sweeps;
        const bool cap = sweeps >= a.cycle_cap || done_before + sweeps >= a.max_iter;
        if (sweeps % a.check_every == 0 || cap) {
            fetch_halo_plane(cl, P, 0, g, C, n, a.H);
            fetch_halo_plane(cl, P, 1, g, C, n, a.H);
            __syncthreads();
            double v = residual_sq(P, n, r0, a);
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
            for (int qq = 0; qq < C; qq++) tot += *cl.map_shared_rank(s_part, qq);
            const double est = sqrt(tot);
            cl.sync();
            if (cap || est <= stop_abs || est <= drop_abs) break;
        }
    }
    for (int t = threadIdx.x; t < n * W; t += blockDim.x) {
        const int row = t / W, x = t - row * W, y = r0 + row;
        a.e[(size_t)y * a.ld + x] = P.e((x + y) & 1)[(size_t)(row + 1) * P.KHp + (x >> 1)];
    }
    if (g == 0 && threadIdx.x == 0) {
        volatile Ctl *cc = a.ctl;
        cc->sweeps = done_before + sweeps;
        if (done_before + sweeps >= a.max_iter) cc->halt = 1;
    }
    cl.sync();
}

}  // namespace

int cluster_plan(int dev, int W, int H, int *C_out, size_t *smem_out, int *khp_out)
{
    int max_smem = 0, cluster_ok = 0;
    PCD_CUDA(cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    PCD_CUDA(cudaDeviceGetAttribute(&cluster_ok, cudaDevAttrClusterLaunch, dev));
    if (!cluster_ok) return PCD_BAD_ARG;
    for (int C : {16, 8}) {
        if (H < 2 * C) continue;
        const int nmax = (H + C - 1) / C;
        const int khp = ((W + 1) / 2 + 3) / 4 * 4;
        if (khp / 2 > kClusterThreads) continue;
        const size_t smem = (size_t)(2 * (nmax + 2) + 2 * nmax) * khp * sizeof(float);
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
        *khp_out = khp;
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
