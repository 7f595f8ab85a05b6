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
#include "sor_planes.cuh"

namespace cg = cooperative_groups;

namespace pcd {

namespace {

using namespace planes;

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
    P.in_smem = 1;
    P.cta_stride = 0;
    carve(P, smem_f, nmax);
    Grid G;
    G.W = a.W; G.H = a.H;
    G.w0 = a.w32[0]; G.w1 = a.w32[1]; G.w2 = a.w32[2]; G.w3 = a.w32[3]; G.w4 = a.w32[4];

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
    // thread -> (slot quad, row group)
    const int KH4 = P.KHp >> 2;
    const int RP = blockDim.x / KH4;
    const int k = 4 * (threadIdx.x % KH4), rg = threadIdx.x / KH4;
    const bool active = rg < RP;
    cl.sync();

    int sweeps = 0;
    for (;;) {
        for (int c = 0; c < 2; c++) {
            fetch_halo_plane(cl, P, c ^ 1, g, C, n, a.H);
            __syncthreads();
            if (active) relax_quad(P, c, n, r0, G, k, rg, RP);
            cl.sync();
        }
        ++sweeps;
        const bool cap = sweeps >= a.cycle_cap || done_before + sweeps >= a.max_iter;
        if (sweeps % a.check_every == 0 || cap) {
            fetch_halo_plane(cl, P, 0, g, C, n, a.H);
            fetch_halo_plane(cl, P, 1, g, C, n, a.H);
            __syncthreads();
            double v = residual_sq(P, n, r0, G);
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
