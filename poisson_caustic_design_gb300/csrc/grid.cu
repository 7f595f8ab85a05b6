// grid.cu -- per-cell grid kernels of the caustic-design iterations (sm_103a).
//
//   subtract_average  utils.cpp:60-86   NaN-skipping mean removal (FP64 sums)
//   gradient          utils.cpp:3-20    central differences, clamped edges, /2
//   divergence        utils.cpp:22-39   d(Nx)/dx + d(Ny)/dy, zero on the ring
//
// All grids are dense row-major doubles (ld == width).  The mean uses a
// two-level reduction with a fixed block count and a fixed summation order,
// so repeated runs give identical bits.
#include "grid.cuh"

namespace pcd {

namespace {
constexpr int kT = 256;
constexpr int kBlocks = 1216;

__device__ __forceinline__ bool is_last_block(unsigned int *counter)
{
    __shared__ bool last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        last = atomicAdd(counter, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (last) __threadfence();
    return last;
}

// NaN by its bit pattern (integer instructions: the FP64 pipe of this part
// runs at 1/56 of the FP32 rate, and a per-cell FP64 compare would make the
// mean removal FP64-bound instead of HBM-bound).
__device__ __forceinline__ bool is_nan_bits(double x)
{
    return (__double_as_longlong(x) & 0x7fffffffffffffffll) > 0x7ff0000000000000ll;
}

// Pass 1: per-block NaN-skipping (sum, count); the last block folds them into
// the mean (scratch[0]) and resets the counter.  Per cell one FP64 addition;
// the count is an integer until the block reduction.
__global__ void __launch_bounds__(kT) k_mean(const double *__restrict__ g, long n, double *scratch,
                                             unsigned int *counter)
{
    double v[2] = {0.0, 0.0};
    long cnt = 0;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const double x = g[i];
        if (!is_nan_bits(x)) { v[0] += x; cnt++; }
    }
    v[1] = (double)cnt;
    block_reduce<2, 0u>(v);
    if (threadIdx.x == 0) {
        scratch[2 + 2 * blockIdx.x] = v[0];
        scratch[3 + 2 * blockIdx.x] = v[1];
    }
    if (is_last_block(counter)) {
        double w[2] = {0.0, 0.0};
        for (int k = threadIdx.x; k < (int)gridDim.x; k += blockDim.x) {
            w[0] += scratch[2 + 2 * k];
            w[1] += scratch[3 + 2 * k];
        }
        block_reduce<2, 0u>(w);
        if (threadIdx.x == 0) {
            scratch[0] = w[0] / w[1];
            scratch[1] = w[1];
            *counter = 0;
            __threadfence();
        }
    }
}

__global__ void __launch_bounds__(kT) k_sub_mean(double *__restrict__ g, long n, const double *scratch)
{
    const double avg = scratch[0];
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const double x = g[i];
        if (!is_nan_bits(x)) g[i] = x - avg;
    }
}

__global__ void __launch_bounds__(kT) k_gradient(const double *__restrict__ g, double *__restrict__ gx,
                                                 double *__restrict__ gy, int W, int H)
{
    const long n = (long)W * H;
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
        const int y = (int)(t / W), x = (int)(t - (long)y * W);
        const int xp = min(x + 1, W - 1), xm = max(x - 1, 0);
        const int yp = min(y + 1, H - 1), ym = max(y - 1, 0);
        gx[t] = (g[(long)y * W + xp] - g[(long)y * W + xm]) / 2.0;
        gy[t] = (g[(long)yp * W + x] - g[(long)ym * W + x]) / 2.0;
    }
}

__global__ void __launch_bounds__(kT) k_divergence(const double *__restrict__ nx, const double *__restrict__ ny,
                                                   double *__restrict__ div, int W, int H)
{
    const long n = (long)W * H;
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
        const int y = (int)(t / W), x = (int)(t - (long)y * W);
        if (x == 0 || x == W - 1 || y == 0 || y == H - 1) {
            div[t] = 0.0;
        } else {
            const double dx = (nx[t + 1] - nx[t - 1]) / 2.0;
            const double dy = (ny[t + W] - ny[t - W]) / 2.0;
            div[t] = dx + dy;
        }
    }
}

// resize_image, main.cpp:13-27: nearest sample at integer source indices
// x * old_width / new_width, y * old_height / new_height.
__global__ void __launch_bounds__(kT) k_resize_nearest(const double *__restrict__ in, int ow, int oh, int ild,
                                                       double *__restrict__ out, int nw, int nh, int old)
{
    const long n = (long)nw * nh;
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
        const int y = (int)(t / nw), x = (int)(t - (long)y * nw);
        const int sx = (int)((long)x * ow / nw), sy = (int)((long)y * oh / nh);
        out[(long)y * old + x] = in[(long)sy * ild + sx];
    }
}

inline int blocks_for(long n) { return (int)std::min<long>(kBlocks, (n + kT - 1) / kT); }

}  // namespace

int GridScratch::reserve()
{
    if (!buf) {
        PCD_CUDA(cudaMalloc(&buf, sizeof(double) * (2 + 2 * kBlocks)));
        PCD_CUDA(cudaMalloc(&counter, sizeof(unsigned int)));
        PCD_CUDA(cudaMemset(counter, 0, sizeof(unsigned int)));
    }
    return PCD_OK;
}

void GridScratch::release()
{
    if (buf) cudaFree(buf);
    if (counter) cudaFree(counter);
    buf = nullptr;
    counter = nullptr;
}

int subtract_average(GridScratch &sc, double *g, long n, cudaStream_t s)
{
    if (n <= 0) return PCD_OK;
    PCD_TRY(sc.reserve());
    const int nb = blocks_for(n);
    k_mean<<<nb, kT, 0, s>>>(g, n, sc.buf, sc.counter);
    PCD_LAUNCHED(1);
    k_sub_mean<<<nb, kT, 0, s>>>(g, n, sc.buf);
    PCD_LAUNCHED(1);
    return PCD_OK;
}

int gradient(const double *g, double *gx, double *gy, int W, int H, cudaStream_t s)
{
    k_gradient<<<blocks_for((long)W * H), kT, 0, s>>>(g, gx, gy, W, H);
    PCD_LAUNCHED(1);
    return PCD_OK;
}

int resize_nearest(const double *in, int ow, int oh, int ild, double *out, int nw, int nh, int old, cudaStream_t s)
{
    k_resize_nearest<<<blocks_for((long)nw * nh), kT, 0, s>>>(in, ow, oh, ild, out, nw, nh, old);
    PCD_LAUNCHED(1);
    return PCD_OK;
}

int divergence(const double *nx, const double *ny, double *div, int W, int H, cudaStream_t s)
{
    k_divergence<<<blocks_for((long)W * H), kT, 0, s>>>(nx, ny, div, W, H);
    PCD_LAUNCHED(1);
    return PCD_OK;
}

}  // namespace pcd
