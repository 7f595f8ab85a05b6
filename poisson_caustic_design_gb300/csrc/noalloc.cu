// noalloc.cu -- mean removal (subtractAverage, utils.cpp:60-86) for callers
// that cannot allocate device memory.
//
// pcd_subtract_average_device() takes a context whose reduction scratch is
// created with cudaMalloc on first use.  Some callers cannot allow that: a host
// application that hands its whole device-memory budget to its own pool at
// start-up and forbids any other allocation, or code on a latency-critical
// path where cudaMalloc/cudaFree would synchronise the device and stall every
// other stream.  pcd_subtract_average_noalloc() serves them: it allocates
// nothing and keeps its scratch in the file-scope array below, which every
// GPU that loads this library holds until the process exits.
//
// Scratch layout: one (sum, count) pair per grid row, so the array bounds the
// grid height: at most kNoallocMaxRows = 16384 rows (256 KiB + the mean).
// Larger grids are rejected with PCD_BAD_ARG.  Three kernels run in order:
//   1. one block per row writes that row's NaN-skipping (sum, count),
//   2. one block folds the row pairs in a fixed order and writes the mean,
//   3. every non-NaN cell has the mean subtracted.
// Each kernel writes the scratch it later reads, so nothing has to start at
// zero and a call never sees values a previous call left behind.  All calls
// share the one array: calls that overlap on the GPU (different streams, or
// different host threads, on the same device) race on it and must be
// serialised by the caller.
//
// The host side never dereferences the array's name: in host code that name
// is only a stand-in for the device variable.  Its device address comes from
// cudaGetSymbolAddress with the device current.  A call on a stream that is
// not capturing looks it up again every time (a host lookup, no device work),
// so a cudaDeviceReset or a released primary context, after which the module
// is loaded again and the array may sit elsewhere, leaves no stale address
// behind.  A call made while its stream is capturing reuses the address that
// the last non-capturing call on that device found (looking a symbol up can
// load the module, which a capture does not allow): make one call on the
// device before any stream capture, and again after a device reset.
#include <mutex>

#include "common.cuh"

namespace pcd {
namespace {

constexpr int kNoallocMaxRows = 16384;
constexpr int kNoallocThreads = 256;
constexpr int kMaxDevices = 64;

// [0] mean, [1] count, then (sum, count) for row y at [2 + 2y], [3 + 2y]
static __device__ __align__(256) double g_noalloc_scratch[2 + 2 * kNoallocMaxRows];

std::mutex g_setup_mu;
double *g_scratch_addr[kMaxDevices] = {};

__global__ void __launch_bounds__(kNoallocThreads) k_row_sums(const double *__restrict__ g, int W, double *scratch)
{
    const int y = blockIdx.x;
    double v[2] = {0.0, 0.0};
    for (int x = threadIdx.x; x < W; x += blockDim.x) {
        const double a = g[(size_t)y * W + x];
        if (!isnan(a)) { v[0] += a; v[1] += 1.0; }
    }
    block_reduce<2, 0u>(v);
    if (threadIdx.x == 0) {
        scratch[2 + 2 * y] = v[0];
        scratch[3 + 2 * y] = v[1];
    }
}

__global__ void __launch_bounds__(kNoallocThreads) k_fold_rows(int H, double *scratch)
{
    double v[2] = {0.0, 0.0};
    for (int y = threadIdx.x; y < H; y += blockDim.x) {
        v[0] += scratch[2 + 2 * y];
        v[1] += scratch[3 + 2 * y];
    }
    block_reduce<2, 0u>(v);
    if (threadIdx.x == 0) {
        scratch[0] = v[0] / v[1];
        scratch[1] = v[1];
    }
}

__global__ void __launch_bounds__(kNoallocThreads) k_subtract(double *__restrict__ g, long n, const double *scratch)
{
    const double avg = scratch[0];
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const double a = g[i];
        if (!isnan(a)) g[i] = a - avg;
    }
}

// Device address of g_noalloc_scratch on the current device: looked up again
// unless `s` is capturing, then the address of the last lookup on the device.
int scratch_address(cudaStream_t s, double **out)
{
    int dev = 0;
    PCD_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) {
        set_error("pcd_subtract_average_noalloc: device index out of range");
        return PCD_BAD_ARG;
    }
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    PCD_CUDA(cudaStreamIsCapturing(s, &cs));
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (cs == cudaStreamCaptureStatusNone) {
        void *p = nullptr;
        PCD_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        g_scratch_addr[dev] = static_cast<double *>(p);
    } else if (!g_scratch_addr[dev]) {
        set_error("pcd_subtract_average_noalloc: the first call on a device must come before any stream capture");
        return PCD_BAD_ARG;
    }
    *out = g_scratch_addr[dev];
    return PCD_OK;
}

}  // namespace
}  // namespace pcd

using namespace pcd;

extern "C" int pcd_subtract_average_noalloc(double *g, int width, int height, void *stream)
{
    if (!g || width < 1 || height < 1) {
        set_error("pcd_subtract_average_noalloc: null grid or empty size");
        return PCD_BAD_ARG;
    }
    if (height > kNoallocMaxRows) {
        set_error("pcd_subtract_average_noalloc: height " + std::to_string(height) + " exceeds the " +
                  std::to_string(kNoallocMaxRows) + "-row scratch of this entry point; use "
                  "pcd_subtract_average_device");
        return PCD_BAD_ARG;
    }
    double *scratch = nullptr;
    cudaStream_t s = (cudaStream_t)stream;
    PCD_TRY(scratch_address(s, &scratch));
    const long n = (long)width * height;
    k_row_sums<<<height, kNoallocThreads, 0, s>>>(g, width, scratch);
    PCD_LAUNCHED(1);
    k_fold_rows<<<1, kNoallocThreads, 0, s>>>(height, scratch);
    PCD_LAUNCHED(1);
    const int blocks = (int)std::min<long>(1216, (n + kNoallocThreads - 1) / kNoallocThreads);
    k_subtract<<<blocks, kNoallocThreads, 0, s>>>(g, n, scratch);
    PCD_LAUNCHED(1);
    return PCD_OK;
}
