// common.cuh -- shared helpers of libpcd_gb300 (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string>

#include "../../include/pcd.h"

namespace pcd {

// Records the text of the last failure for pcd_last_error().
void set_error(const std::string &msg);
// Counts kernel launches issued by the library (direct launches + graph nodes).
void count_launches(unsigned long long n);

#define PCD_CUDA(call)                                                                     \
    do {                                                                                   \
        cudaError_t e_ = (call);                                                           \
        if (e_ != cudaSuccess) {                                                           \
            ::pcd::set_error(std::string(#call) + ": " + cudaGetErrorString(e_) + " (" +    \
                             __FILE__ + ":" + std::to_string(__LINE__) + ")");             \
            return PCD_DEVICE_ERROR;                                                       \
        }                                                                                  \
    } while (0)

#define PCD_TRY(expr)                                                                      \
    do {                                                                                   \
        int s_ = (expr);                                                                   \
        if (s_ != PCD_OK) return s_;                                                       \
    } while (0)

// Checks the launch that just happened on the stream.
#define PCD_LAUNCHED(n)                                                                    \
    do {                                                                                   \
        PCD_CUDA(cudaGetLastError());                                                      \
        ::pcd::count_launches(n);                                                          \
    } while (0)

__device__ __forceinline__ float warp_sum_f(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Max that ignores NaN on the left operand's side the way the reference's
// `if (abs_delta > max_update)` does (solver.cpp:51-53).
__device__ __forceinline__ double nan_skip_max(double m, double v) { return v > m ? v : m; }

__device__ __forceinline__ double warp_max(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = nan_skip_max(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

__device__ __forceinline__ double warp_min(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Block-wide reduction of up to 4 doubles (sum/max selectable per slot via
// OPS bits: bit k set = max for slot k).  Result valid in thread 0.
template <int N, unsigned OPS>
__device__ __forceinline__ void block_reduce(double (&v)[N])
{
    __shared__ double sm[32][N];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int k = 0; k < N; k++) v[k] = ((OPS >> k) & 1u) ? warp_max(v[k]) : warp_sum(v[k]);
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < N; k++) sm[wid][k] = v[k];
    __syncthreads();
    if (wid == 0) {
#pragma unroll
        for (int k = 0; k < N; k++) {
            // lanes past the last warp hold each slot's identity: 0 for a sum,
            // -inf for a max (so signed maxima come out right as well)
            double x = lane < nw ? sm[lane][k] : (((OPS >> k) & 1u) ? -__longlong_as_double(0x7ff0000000000000ll) : 0.0);
            v[k] = ((OPS >> k) & 1u) ? warp_max(x) : warp_sum(x);
        }
    }
    __syncthreads();
}

inline int ceil_div(long a, long b) { return (int)((a + b - 1) / b); }

}  // namespace pcd
