// solver.cu -- red-black SOR for the reference's Poisson problem on sm_103a.
//
// Reference: poisson_solver / patial_relax, src/solver.cpp:12-148.  The
// reference relaxes lexicographically (Gauss-Seidel order) with
// omega = 2/(1+pi/width) and stops when one sweep's max |delta| drops below a
// threshold.  Here every sweep is two half sweeps over the red ((x+y) even)
// and black cells, which have no neighbours of their own colour, so each half
// sweep is one fully parallel kernel.  Red-black SOR with the same omega has
// the same asymptotic rate as the lexicographic ordering (both are consistent
// orderings); intermediate iterates differ, the fixed point is the same.
//
// Two stop tests: the reference's max |delta| (checked after every sweep by
// the last block of the black half sweep) and a relative FP64 residual
// ||b - L phi|| / ||b|| checked every `check_every` sweeps.
//
// Two precisions: FP64 sweeps on phi, or FP32 sweeps on the error equation
// L e = r with the residual r = b - L(phi + e) and the update phi += e done in
// FP64 every `refine_every` sweeps (defect correction).  SOR is a stationary
// iteration, so restarting it on the refreshed residual from e = 0 changes
// nothing in exact arithmetic; FP32 only limits how far e may be pushed
// between refreshes.
//
// Sweeps are issued as CUDA-graph chunks; the stop flags live in device memory
// and make the remaining kernels of a chunk return at once, so the host reads
// the control block once per chunk and launches the next chunk speculatively.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "solver.cuh"
#include "sor_persist.cuh"
#include "sor_cluster.cuh"
#include "sor_blocks.cuh"

namespace pcd {

namespace {

constexpr int kThreads = 256;
constexpr int kResidualBlocksMax = 1216;  // 152 SMs x 8

__device__ __forceinline__ int vol_load(const int *p) { return *(volatile const int *)p; }

// ---------------------------------------------------------------------------
// Neighbour-validity mask: bit0 left, bit1 up, bit2 right, bit3 down (inside
// the grid and b not NaN, solver.cpp:29-44); bit4 set when b itself is NaN.
// ---------------------------------------------------------------------------
__global__ void k_mask(const double *__restrict__ b, uint8_t *__restrict__ mask, int W, int H, int ld,
                       Ctl *ctl)
{
    long n = (long)W * H;
    int nan_local = 0;
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
        int y = (int)(t / W), x = (int)(t - (long)y * W);
        long i = (long)y * ld + x;
        uint8_t m = 0;
        if (x > 0 && !isnan(b[i - 1])) m |= 1;
        if (y > 0 && !isnan(b[i - ld])) m |= 2;
        if (x < W - 1 && !isnan(b[i + 1])) m |= 4;
        if (y < H - 1 && !isnan(b[i + ld])) m |= 8;
        if (isnan(b[i])) { m |= 16; nan_local++; }
        mask[i] = m;
    }
    if (nan_local) atomicAdd(&ctl->nan_cells, nan_local);
}

template <typename T, bool MASKED>
__device__ __forceinline__ void gather(const T *__restrict__ phi, const uint8_t *__restrict__ mask, long i, int x,
                                       int y, int W, int H, int ld, T &sum, T &cnt)
{
    sum = T(0);
    cnt = T(0);
    if (MASKED) {
        const uint8_t m = mask[i];
        if (m & 1) { cnt += T(1); sum += phi[i - 1]; }
        if (m & 2) { cnt += T(1); sum += phi[i - ld]; }
        if (m & 4) { cnt += T(1); sum += phi[i + 1]; }
        if (m & 8) { cnt += T(1); sum += phi[i + ld]; }
    } else {
        if (x > 0) { cnt += T(1); sum += phi[i - 1]; }
        if (y > 0) { cnt += T(1); sum += phi[i - ld]; }
        if (x < W - 1) { cnt += T(1); sum += phi[i + 1]; }
        if (y < H - 1) { cnt += T(1); sum += phi[i + ld]; }
    }
}

// omega/cnt from the host-divided table, selected without dynamic indexing
// (which would place the argument struct in local memory).
template <typename T>
__device__ __forceinline__ T omega_over_cnt(const SolveArgs &a, int cnt)
{
    if (sizeof(T) == 8)
        return (T)(cnt == 4 ? a.w64[4] : cnt == 3 ? a.w64[3] : cnt == 2 ? a.w64[2] : cnt == 1 ? a.w64[1] : a.w64[0]);
    return (T)(cnt == 4 ? a.w32[4] : cnt == 3 ? a.w32[3] : cnt == 2 ? a.w32[2] : cnt == 1 ? a.w32[1] : a.w32[0]);
}

// One half sweep over the cells of `color`: delta = omega/cnt*(sum - cnt*v - b)
// (solver.cpp:47), phi += delta.  TRACK keeps the sweep's max |delta|.
template <typename T, bool MASKED, bool TRACK>
__global__ void __launch_bounds__(kThreads)
    k_rb_half(T *__restrict__ phi, const T *__restrict__ rhs, const uint8_t *__restrict__ mask, Ctl *ctl,
              SolveArgs a, int color, int last_half)
{
    if (vol_load(&ctl->halt)) return;
    const int half = (a.W + 1) >> 1;
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    double m = 0.0;
    if (idx < (long)a.H * half) {
        const int y = (int)(idx / half);
        const int x = 2 * (int)(idx - (long)y * half) + ((y + color) & 1);
        if (x < a.W) {
            const long i = (long)y * a.ld + x;
            T sum, cnt;
            gather<T, MASKED>(phi, mask, i, x, y, a.W, a.H, a.ld, sum, cnt);
            const T v = phi[i];
            const T w = omega_over_cnt<T>(a, (int)cnt);
            const T delta = w * (sum - cnt * v - rhs[i]);
            phi[i] = v + delta;
            if (TRACK) {
                double ad = fabs((double)delta);
                m = ad > 0.0 ? ad : 0.0;  // NaN deltas never raise the max (solver.cpp:51)
            }
        }
    }
    if (!TRACK && !last_half) return;
    if (TRACK) {
        double v[1] = {m};
        block_reduce<1, 1u>(v);
        m = v[0];
    }
    if (threadIdx.x == 0) {
        if (TRACK && m > 0.0) atomicMax(&ctl->maxbits, (unsigned long long)__double_as_longlong(m));
        if (last_half) {
            __threadfence();
            unsigned t = atomicAdd(&ctl->blocks_done, 1u);
            if (t == gridDim.x - 1) {
                __threadfence();
                end_of_sweep(ctl, a);
            }
        }
    }
}

// Last-block finalisation of a residual reduction: sums the per-block
// partials in a fixed order (deterministic), stores the norms and applies the
// relative-residual stop test when `test` is set.
__device__ void finalize_residual(Ctl *ctl, const double *partials, int nblk, const SolveArgs &a, int test,
                                  int with_b)
{
    double v[3] = {0.0, 0.0, 0.0};
    for (int k = threadIdx.x; k < nblk; k += blockDim.x) {
        v[0] += partials[3 * k];
        v[1] += partials[3 * k + 1];
        v[2] = fmax(v[2], partials[3 * k + 2]);
    }
    block_reduce<3, 4u>(v);
    if (threadIdx.x == 0) {
        volatile Ctl *c = ctl;
        double rn = sqrt(v[0]);
        if (with_b) c->bnorm = sqrt(v[1]);
        double bn = c->bnorm;
        c->rnorm = rn;
        c->rmax = v[2];
        double rel = bn > 0.0 ? rn / bn : rn;
        c->rel = rel;
        c->checks = c->checks + 1;
        if (test && a.stop == PCD_STOP_REL_RESIDUAL && rel <= a.tol) {
            c->converged = 1;
            c->halt = 1;
        }
        c->blocks_done_r = 0;
        __threadfence();
    }
}

__device__ __forceinline__ bool last_block(Ctl *ctl)
{
    __shared__ bool is_last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        unsigned t = atomicAdd(&ctl->blocks_done_r, 1u);
        is_last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (is_last) __threadfence();
    return is_last;
}

// FP64 residual r = b - L phi over non-NaN cells; partial sums of r^2, b^2
// and max |r|.  `test`: apply the stop test (loop checks); `skip_halted`:
// return at once when the solve already halted.
template <bool MASKED>
__global__ void __launch_bounds__(kThreads)
    k_residual64(const double *__restrict__ phi, const double *__restrict__ b, const uint8_t *__restrict__ mask,
                 Ctl *ctl, double *partials, SolveArgs a, int test, int with_b, int skip_halted,
                 double *__restrict__ rout = nullptr)
{
    if (skip_halted && vol_load(&ctl->halt)) return;
    const long n = (long)a.W * a.H;
    double v[3] = {0.0, 0.0, 0.0};
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
        const int y = (int)(t / a.W), x = (int)(t - (long)y * a.W);
        const long i = (long)y * a.ld + x;
        const double bi = b[i];
        if (isnan(bi)) continue;
        double sum, cnt;
        gather<double, MASKED>(phi, mask, i, x, y, a.W, a.H, a.ld, sum, cnt);
        const double r = bi - (sum - cnt * phi[i]);
        if (rout) rout[i] = r;
        v[0] += r * r;
        v[1] += bi * bi;
        v[2] = nan_skip_max(v[2], fabs(r));
    }
    block_reduce<3, 4u>(v);
    if (threadIdx.x == 0) {
        partials[3 * blockIdx.x] = v[0];
        partials[3 * blockIdx.x + 1] = v[1];
        partials[3 * blockIdx.x + 2] = v[2];
    }
    if (last_block(ctl)) finalize_residual(ctl, partials, gridDim.x, a, test, with_b);
}

// Mixed precision: r = b - L(phi + e) in FP64 (e widened exactly), written to
// r32 as the next right-hand side of the FP32 correction sweeps.
template <bool MASKED>
__global__ void __launch_bounds__(kThreads)
    k_refine_residual(const double *__restrict__ phi, const float *__restrict__ e, const double *__restrict__ b,
                      const uint8_t *__restrict__ mask, float *__restrict__ r32, Ctl *ctl, double *partials,
                      SolveArgs a, int with_b)
{
    if (vol_load(&ctl->done)) return;
    const long n = (long)a.W * a.H;
    double v[3] = {0.0, 0.0, 0.0};
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
        const int y = (int)(t / a.W), x = (int)(t - (long)y * a.W);
        const long i = (long)y * a.ld + x;
        const double bi = b[i];
        double sum = 0.0, cnt = 0.0;
        if (MASKED) {
            const uint8_t m = mask[i];
            if (m & 1) { cnt += 1.0; sum += phi[i - 1] + (double)e[i - 1]; }
            if (m & 2) { cnt += 1.0; sum += phi[i - a.ld] + (double)e[i - a.ld]; }
            if (m & 4) { cnt += 1.0; sum += phi[i + 1] + (double)e[i + 1]; }
            if (m & 8) { cnt += 1.0; sum += phi[i + a.ld] + (double)e[i + a.ld]; }
        } else {
            if (x > 0) { cnt += 1.0; sum += phi[i - 1] + (double)e[i - 1]; }
            if (y > 0) { cnt += 1.0; sum += phi[i - a.ld] + (double)e[i - a.ld]; }
            if (x < a.W - 1) { cnt += 1.0; sum += phi[i + 1] + (double)e[i + 1]; }
            if (y < a.H - 1) { cnt += 1.0; sum += phi[i + a.ld] + (double)e[i + a.ld]; }
        }
        const double xi = phi[i] + (double)e[i];
        const double r = bi - (sum - cnt * xi);
        r32[i] = (float)r;
        if (isnan(bi)) continue;
        v[0] += r * r;
        v[1] += bi * bi;
        v[2] = nan_skip_max(v[2], fabs(r));
    }
    block_reduce<3, 4u>(v);
    if (threadIdx.x == 0) {
        partials[3 * blockIdx.x] = v[0];
        partials[3 * blockIdx.x + 1] = v[1];
        partials[3 * blockIdx.x + 2] = v[2];
    }
    if (last_block(ctl)) finalize_residual(ctl, partials, gridDim.x, a, 1, with_b);
}

// Mixed precision: phi += e, e = 0.  The last block marks the solve done once
// the sweeps have halted (the correction that halted them is now in phi).
__global__ void __launch_bounds__(kThreads)
    k_refine_update(double *__restrict__ phi, float *__restrict__ e, Ctl *ctl, SolveArgs a)
{
    if (vol_load(&ctl->done)) return;
    const long n = (long)a.W * a.H;
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
        const int y = (int)(t / a.W), x = (int)(t - (long)y * a.W);
        const long i = (long)y * a.ld + x;
        phi[i] += (double)e[i];
        e[i] = 0.0f;
    }
    if (last_block(ctl)) {
        if (threadIdx.x == 0) {
            volatile Ctl *c = ctl;
            if (c->halt) c->done = 1;
            c->blocks_done_r = 0;
            __threadfence();
        }
    }
}


// ---------------------------------------------------------------------------
// Fused red+black sweep for grids that live in HBM (no NaN cells).
//
// Block s walks down its stripe of rows [y0, y1): at step j it relaxes the red
// cells of row y0+j and then the black cells of row y0+j-1.  A red cell needs
// the black rows y-1, y, y+1 as they were before the sweep, and a black cell
// needs the new red rows y-1, y, y+1; walking down the stripe gives exactly
// that order, with one block barrier per step.  The black cells of the first
// and last row of every stripe depend on a neighbouring stripe's red row, so a
// second kernel relaxes those after all stripes finished.  The result is
// exactly one red-black SOR sweep, and phi and b cross HBM once per sweep
// (24 B per cell in FP64, 12 B in FP32) instead of twice.
constexpr int kStripeThreads = 512;

__device__ __forceinline__ void prefetch_l2(const void *p)
{
    asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

// One colour of row y.  All loads of a thread's cells are issued before any
// store: a cell's neighbours have the other colour, so no cell of this row
// reads what another cell of it writes, and batching lets the DRAM latency of
// the cells overlap instead of serialising behind each store.
constexpr int kRowCellsMax = 8;  // cells per thread per row: W <= 2 * 8 * kStripeThreads

template <typename T, bool TRACK, int CELLS>
__device__ __forceinline__ double relax_row(T *__restrict__ phi, const T *__restrict__ rhs, const SolveArgs &a,
                                            int y, int color)
{
    const int W = a.W, H = a.H, ld = a.ld;
    const int off = (y + color) & 1;
    const long rowi = (long)y * ld;
    T sum[CELLS], v[CELLS], r[CELLS];
    int cnt[CELLS];
#pragma unroll
    for (int j = 0; j < CELLS; j++) {
        const int x = 2 * (threadIdx.x + j * (int)blockDim.x) + off;
        sum[j] = T(0);
        cnt[j] = 0;
        v[j] = T(0);
        r[j] = T(0);
        if (x < W) {
            const long i = rowi + x;
            if (x > 0) { sum[j] += phi[i - 1]; cnt[j]++; }
            if (y > 0) { sum[j] += phi[i - ld]; cnt[j]++; }
            if (x < W - 1) { sum[j] += phi[i + 1]; cnt[j]++; }
            if (y < H - 1) { sum[j] += phi[i + ld]; cnt[j]++; }
            v[j] = phi[i];
            r[j] = rhs[i];
        }
    }
    double m = 0.0;
#pragma unroll
    for (int j = 0; j < CELLS; j++) {
        const int x = 2 * (threadIdx.x + j * (int)blockDim.x) + off;
        if (x < W) {
            const T delta = omega_over_cnt<T>(a, cnt[j]) * (sum[j] - (T)cnt[j] * v[j] - r[j]);
            phi[rowi + x] = v[j] + delta;
            if (TRACK) {
                const double ad = fabs((double)delta);
                m = ad > m ? ad : m;
            }
        }
    }
    return m;
}

template <typename T, bool TRACK, int CELLS>
__global__ void __launch_bounds__(kStripeThreads, 2)
    k_stripe_a(T *__restrict__ phi, const T *__restrict__ rhs, Ctl *ctl, SolveArgs a, int R)
{
    if (vol_load(&ctl->halt)) return;
    const int y0 = blockIdx.x * R, y1 = min(y0 + R, a.H);
    double m = 0.0;
    // lines of one row (128 B each); threads [0, L) prefetch the next step's
    // new phi row, threads [L, 2L) its right-hand-side row
    const int L = (int)((a.W * sizeof(T) + 127) / 128);
    for (int j = 0; j <= y1 - y0; j++) {
        const int yr = y0 + j;
        const int t = threadIdx.x;
        if (yr + 2 < a.H && t < L) prefetch_l2(phi + (long)(yr + 2) * a.ld + t * (128 / sizeof(T)));
        else if (yr + 1 < y1 && t >= L && t < 2 * L)
            prefetch_l2(rhs + (long)(yr + 1) * a.ld + (t - L) * (128 / sizeof(T)));
        if (yr < y1) m = fmax(m, relax_row<T, TRACK, CELLS>(phi, rhs, a, yr, 0));
        __syncthreads();
        const int yb = yr - 1;
        if (yb >= y0 + 1 && yb <= y1 - 2) m = fmax(m, relax_row<T, TRACK, CELLS>(phi, rhs, a, yb, 1));
    }
    if (TRACK) {
        double v[1] = {m};
        block_reduce<1, 1u>(v);
        if (threadIdx.x == 0 && v[0] > 0.0) atomicMax(&ctl->maxbits, (unsigned long long)__double_as_longlong(v[0]));
    }
}

// Black cells of the first and last row of every stripe; the last block
// closes the sweep (end_of_sweep).  blockIdx.y = 2*stripe + {0: first, 1: last}.
template <typename T, bool TRACK, int CELLS>
__global__ void __launch_bounds__(kStripeThreads, 2)
    k_stripe_b(T *__restrict__ phi, const T *__restrict__ rhs, Ctl *ctl, SolveArgs a, int R)
{
    if (vol_load(&ctl->halt)) return;
    const int st = blockIdx.y >> 1, which = blockIdx.y & 1;
    const int y0 = st * R, y1 = min(y0 + R, a.H);
    const int y = which ? y1 - 1 : y0;
    double m = 0.0;
    if (!(which && y == y0)) m = relax_row<T, TRACK, CELLS>(phi, rhs, a, y, 1);
    if (TRACK) {
        double v[1] = {m};
        block_reduce<1, 1u>(v);
        m = v[0];
    }
    if (threadIdx.x == 0) {
        if (TRACK && m > 0.0) atomicMax(&ctl->maxbits, (unsigned long long)__double_as_longlong(m));
        __threadfence();
        const unsigned t = atomicAdd(&ctl->blocks_done, 1u);
        if (t == gridDim.x * gridDim.y - 1) {
            __threadfence();
            end_of_sweep(ctl, a);
        }
    }
}

// Rows per stripe such that all stripes are resident at once (one wave):
// stripes = resident blocks per SM x SMs.
inline int stripe_rows(int H, int resident)
{
    const int target = resident > 0 ? resident : 304;
    int R = (H + target - 1) / target;
    return R < 3 ? 3 : R;
}

#include "sor_stream.cuh"
#include "sor_stream2.cuh"

// Launch shape of the ping-pong stream sweep: G 4-cell groups per thread,
// T threads (one row of the grid per block), ns stripes of R rows; rows
// staged by bulk copies (tma, rows of wpad floats, smem bytes of dynamic
// shared memory) or loaded into registers.
struct StreamPlan {
    int G = 0, T = 0, R = 0, ns = 0;
    int tma = 0, wpad = 0;
    size_t smem = 0;
    int two = 0;          // two sweeps per pass (k_sweep2_tma) available
    size_t smem2 = 0;
    TilePlan tile;        // register-resident tile passes (schedule TILES)
    int tile_sweeps = 0;  // sweeps per tile pass (between stop tests)
};

int stream_plan(int dev, int W, int H, int ld, bool allow_tma, StreamPlan *p)
{
    const int groups = (W + 3) / 4;
    // two groups per thread at most: four would not fit in 128 registers
    if (H < 3 || ld % 4 != 0 || groups > 2 * kStreamThreadsMax) return PCD_BAD_ARG;
    const int G = groups <= kStreamThreadsMax ? 1 : 2;
    const int T = 32 * ceil_div(ceil_div(groups, G), 32);
    int sms = 0, bps = 0, max_smem = 0;
    PCD_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    PCD_CUDA(cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    const int wpad = 4 * groups;
    const size_t smem = tma_smem_bytes(wpad);
    const bool tma = allow_tma && smem <= (size_t)max_smem;
    if (tma) {
        const void *fns[2] = {G == 1 ? (const void *)k_sweep_tma<1, false> : (const void *)k_sweep_tma<2, false>,
                              G == 1 ? (const void *)k_sweep_tma<1, true> : (const void *)k_sweep_tma<2, true>};
        for (const void *fn : fns) PCD_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        int bps_t = 0;
        PCD_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, fns[0], T, smem));
        PCD_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps_t, fns[1], T, smem));
        bps = std::min(bps, bps_t);
    } else if (G == 1) {
        PCD_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_sweep_stream<1, false>, T, 0));
    } else {
        PCD_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_sweep_stream<2, false>, T, 0));
    }
    if (bps < 1) return PCD_BAD_ARG;
    int ns = std::min(bps * sms, ceil_div(H, kStreamRowsMin));
    if (ns < 1) ns = 1;
    // even stripe heights: every stripe starts on an even row (the two-sweep
    // pass relies on it for its compile-time cell parities)
    const int R = 2 * ceil_div(ceil_div(H, ns), 2);
    p->G = G;
    p->T = T;
    p->R = R;
    p->ns = ceil_div(H, R);
    p->tma = tma ? 1 : 0;
    p->wpad = wpad;
    p->smem = tma ? smem : 0;
    // the two-sweep pass: whole 4G-cell groups (W a multiple of 4G, one
    // group column per thread), one block per SM, stripes of >= 8 rows
    const size_t smem2 = tma2_smem_bytes(wpad, T);
    p->two = 0;
    p->smem2 = 0;
    if (tma && W % (4 * G) == 0 && T * 4 * G == W && smem2 + 1024 <= (size_t)max_smem && p->R >= 8 &&
        p->R % 2 == 0) {
        const void *fns2[2] = {G == 1 ? (const void *)k_sweep2_tma<1, false> : (const void *)k_sweep2_tma<2, false>,
                               G == 1 ? (const void *)k_sweep2_tma<1, true> : (const void *)k_sweep2_tma<2, true>};
        int ok2 = 1;
        for (const void *fn : fns2) {
            PCD_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem2));
            int b2 = 0;
            PCD_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b2, fn, T, smem2));
            if (b2 < 1) ok2 = 0;
        }
        if (ok2) {
            p->two = 1;
            p->smem2 = smem2;
        }
    }
    return PCD_OK;
}

constexpr long kTmaSpinLimit = 1l << 22;

// Two sweeps from ein into eout (one when a single sweep is left before
// max_iter).
template <bool TRACK>
void launch_stream2_t(const StreamPlan &p, const float *ein, float *eout, const float *r, Ctl *ctl,
                      const SolveArgs &a, int out_idx, cudaStream_t s)
{
    if (p.G == 1)
        k_sweep2_tma<1, TRACK><<<p.ns, p.T, p.smem2, s>>>(ein, eout, r, ctl, a, p.R, out_idx, p.wpad, kTmaSpinLimit);
    else
        k_sweep2_tma<2, TRACK><<<p.ns, p.T, p.smem2, s>>>(ein, eout, r, ctl, a, p.R, out_idx, p.wpad, kTmaSpinLimit);
}

template <bool TRACK>
void launch_stream_t(const StreamPlan &p, const float *ein, float *eout, const float *r, Ctl *ctl, const SolveArgs &a,
                     int out_idx, cudaStream_t s)
{
    if (p.tma) {
        if (p.G == 1)
            k_sweep_tma<1, TRACK><<<p.ns, p.T, p.smem, s>>>(ein, eout, r, ctl, a, p.R, out_idx, p.wpad, kTmaSpinLimit);
        else
            k_sweep_tma<2, TRACK><<<p.ns, p.T, p.smem, s>>>(ein, eout, r, ctl, a, p.R, out_idx, p.wpad, kTmaSpinLimit);
    } else if (p.G == 1) {
        k_sweep_stream<1, TRACK><<<p.ns, p.T, 0, s>>>(ein, eout, r, ctl, a, p.R, out_idx);
    } else {
        k_sweep_stream<2, TRACK><<<p.ns, p.T, 0, s>>>(ein, eout, r, ctl, a, p.R, out_idx);
    }
}


__global__ void k_fill(double *p, int W, int H, int ld, double v)
{
    const long n = (long)W * H;
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
        const int y = (int)(t / W), x = (int)(t - (long)y * W);
        p[(long)y * ld + x] = v;
    }
}

inline int grid_blocks(long n) { return (int)std::min<long>(kResidualBlocksMax, (n + kThreads - 1) / kThreads); }

}  // namespace

double resolve_omega(double omega, int W, int H)
{
    if (omega > 0.0) return omega;
    if (omega == 0.0) return 2.0 / (1.0 + 3.14159265 / W);  // solver.cpp:71
    const int n = W > H ? W : H;
    if (n < 2) return 1.0;
    const double mu = 0.5 * (1.0 + std::cos(M_PI / n));
    return 2.0 / (1.0 + std::sqrt(1.0 - mu * mu));
}

int SolverWorkspace::reserve(size_t n)
{
    if (!ctl) {
        PCD_CUDA(cudaMalloc(&ctl, sizeof(Ctl)));
        PCD_CUDA(cudaMallocHost(&ctl_host, 2 * sizeof(Ctl)));
        PCD_CUDA(cudaMalloc(&partials, 3 * sizeof(double) * kResidualBlocksMax));
        max_partials = kResidualBlocksMax;
        for (int k = 0; k < 2; k++) PCD_CUDA(cudaEventCreateWithFlags(&ev[k], cudaEventDisableTiming));
        PCD_CUDA(cudaEventCreate(&t0));
        PCD_CUDA(cudaEventCreate(&t1));
        PCD_CUDA(cudaEventCreate(&k0));
        PCD_CUDA(cudaEventCreate(&k1));
    }
    if (n > cells) {
        if (mask) cudaFree(mask);
        if (e32) cudaFree(e32);
        if (e32b) cudaFree(e32b);
        if (r32) cudaFree(r32);
        if (r64) cudaFree(r64);
        mask = nullptr; e32 = nullptr; e32b = nullptr; r32 = nullptr; r64 = nullptr;
        for (auto &kv : graphs) cudaGraphExecDestroy(kv.second.exec);
        graphs.clear();
        PCD_CUDA(cudaMalloc(&mask, n));
        PCD_CUDA(cudaMalloc(&e32, n * sizeof(float)));
        PCD_CUDA(cudaMalloc(&e32b, n * sizeof(float)));
        PCD_CUDA(cudaMalloc(&r32, n * sizeof(float)));
        PCD_CUDA(cudaMalloc(&r64, n * sizeof(double)));
        cells = n;
    }
    return PCD_OK;
}

void SolverWorkspace::release()
{
    for (auto &kv : graphs) cudaGraphExecDestroy(kv.second.exec);
    graphs.clear();
    if (mask) cudaFree(mask);
    if (e32) cudaFree(e32);
    if (e32b) cudaFree(e32b);
    if (r32) cudaFree(r32);
    if (r64) cudaFree(r64);
    if (xbuf) cudaFree(xbuf);
    if (flags) cudaFree(flags);
    if (part) cudaFree(part);
    if (bx) cudaFree(bx);
    r64 = nullptr; xbuf = nullptr; flags = nullptr; part = nullptr; bx = nullptr;
    xbuf_elems = 0; max_ctas = 0; bx_bytes = 0;
    if (partials) cudaFree(partials);
    if (ctl) cudaFree(ctl);
    if (ctl_host) cudaFreeHost(ctl_host);
    for (int k = 0; k < 2; k++)
        if (ev[k]) cudaEventDestroy(ev[k]);
    if (t0) cudaEventDestroy(t0);
    if (t1) cudaEventDestroy(t1);
    if (k0) cudaEventDestroy(k0);
    if (k1) cudaEventDestroy(k1);
    mask = nullptr; e32 = nullptr; e32b = nullptr; r32 = nullptr; partials = nullptr; ctl = nullptr;
    ctl_host = nullptr;
    cells = 0;
}

namespace {

template <typename T, bool TRACK, int CELLS>
void launch_stripes_c(T *phi, const T *rhs, Ctl *ctl, const SolveArgs &a, int R, int ns, dim3 gb, cudaStream_t s)
{
    k_stripe_a<T, TRACK, CELLS><<<ns, kStripeThreads, 0, s>>>(phi, rhs, ctl, a, R);
    k_stripe_b<T, TRACK, CELLS><<<gb, kStripeThreads, 0, s>>>(phi, rhs, ctl, a, R);
}

template <typename T, bool TRACK>
int launch_stripes(T *phi, const T *rhs, Ctl *ctl, const SolveArgs &a, int R, int ns, dim3 gb, int cells,
                   cudaStream_t s)
{
    if (cells <= 1) launch_stripes_c<T, TRACK, 1>(phi, rhs, ctl, a, R, ns, gb, s);
    else if (cells <= 2) launch_stripes_c<T, TRACK, 2>(phi, rhs, ctl, a, R, ns, gb, s);
    else if (cells <= 4) launch_stripes_c<T, TRACK, 4>(phi, rhs, ctl, a, R, ns, gb, s);
    else launch_stripes_c<T, TRACK, kRowCellsMax>(phi, rhs, ctl, a, R, ns, gb, s);
    return PCD_OK;
}

// Enqueues one chunk of `sweeps` sweeps (plus the checks that follow them) on s.
template <bool MASKED>
int enqueue_chunk(SolverWorkspace &ws, const double *b, double *phi, const SolveArgs &a, int precision,
                  int sweeps, cudaStream_t s, int *nodes, int sched, const StreamPlan &sp)
{
    const bool stripes = sched == PCD_SCHED_STRIPES;
    const int half = (a.W + 1) >> 1;
    const int blocks = ceil_div((long)a.H * half, kThreads);
    const int rblocks = grid_blocks((long)a.W * a.H);
    const bool track = (a.stop == PCD_STOP_MAX_UPDATE);
    int n = 0;
    if (!MASKED && stripes) {
        const int R = stripe_rows(a.H, ws.stripe_resident);
        const int ns = (a.H + R - 1) / R;
        const dim3 gb(1, 2 * ns);  // one block per boundary row (relax_row strides over the row)
        const int cells = ceil_div(half, kStripeThreads);
        for (int k = 0; k < sweeps; k++) {
            if (precision == PCD_PREC_MIXED) {
                if (track) PCD_TRY((launch_stripes<float, true>(ws.e32, ws.r32, ws.ctl, a, R, ns, gb, cells, s)));
                else PCD_TRY((launch_stripes<float, false>(ws.e32, ws.r32, ws.ctl, a, R, ns, gb, cells, s)));
            } else {
                if (track) PCD_TRY((launch_stripes<double, true>(phi, b, ws.ctl, a, R, ns, gb, cells, s)));
                else PCD_TRY((launch_stripes<double, false>(phi, b, ws.ctl, a, R, ns, gb, cells, s)));
            }
            n += 2;
        }
        sweeps = 0;
    }
    if (!MASKED && sched == PCD_SCHED_TILES) {
        // as the stream passes: pass k reads buffer k&1 and writes the other
        int k = 0;
        for (int done = 0; done < sweeps; k++) {
            const float *ein = (k & 1) ? ws.e32b : ws.e32;
            float *eout = (k & 1) ? ws.e32 : ws.e32b;
            const int nsw = std::min(sp.tile_sweeps, sweeps - done);
            PCD_TRY(launch_tile(sp.tile, ein, eout, ws.r32, ws.ctl, a, nsw, (k & 1) ? 0 : 1, track, s));
            done += nsw;
            n++;
        }
        k_stream_settle<<<rblocks, kThreads, 0, s>>>(ws.e32, ws.e32b, ws.ctl, a);
        n++;
        sweeps = 0;
    }
    if (!MASKED && sched == PCD_SCHED_STREAM) {
        // launch k reads buffer k&1 and writes the other (two sweeps per
        // launch where the plan allows, a single sweep for an odd rest); the
        // settle kernel moves the latest correction into e32 for the refinement
        int k = 0;
        for (int done = 0; done < sweeps; k++) {
            const float *ein = (k & 1) ? ws.e32b : ws.e32;
            float *eout = (k & 1) ? ws.e32 : ws.e32b;
            const int out = (k & 1) ? 0 : 1;
            if (sp.two && sweeps - done >= 2) {
                if (track) launch_stream2_t<true>(sp, ein, eout, ws.r32, ws.ctl, a, out, s);
                else launch_stream2_t<false>(sp, ein, eout, ws.r32, ws.ctl, a, out, s);
                done += 2;
            } else {
                if (track) launch_stream_t<true>(sp, ein, eout, ws.r32, ws.ctl, a, out, s);
                else launch_stream_t<false>(sp, ein, eout, ws.r32, ws.ctl, a, out, s);
                done += 1;
            }
            n++;
        }
        k_stream_settle<<<rblocks, kThreads, 0, s>>>(ws.e32, ws.e32b, ws.ctl, a);
        n++;
        sweeps = 0;
    }
    for (int k = 0; k < sweeps; k++) {
        for (int color = 0; color < 2; color++) {
            const int last = color == 1;
            if (precision == PCD_PREC_MIXED) {
                if (track)
                    k_rb_half<float, MASKED, true><<<blocks, kThreads, 0, s>>>(ws.e32, ws.r32, ws.mask, ws.ctl, a, color, last);
                else
                    k_rb_half<float, MASKED, false><<<blocks, kThreads, 0, s>>>(ws.e32, ws.r32, ws.mask, ws.ctl, a, color, last);
            } else {
                if (track)
                    k_rb_half<double, MASKED, true><<<blocks, kThreads, 0, s>>>(phi, b, ws.mask, ws.ctl, a, color, last);
                else
                    k_rb_half<double, MASKED, false><<<blocks, kThreads, 0, s>>>(phi, b, ws.mask, ws.ctl, a, color, last);
            }
            n++;
        }
    }
    if (precision == PCD_PREC_MIXED) {
        k_refine_residual<MASKED><<<rblocks, kThreads, 0, s>>>(phi, ws.e32, b, ws.mask, ws.r32, ws.ctl, ws.partials, a, 0);
        k_refine_update<<<rblocks, kThreads, 0, s>>>(phi, ws.e32, ws.ctl, a);
        n += 2;
    } else if (a.stop == PCD_STOP_REL_RESIDUAL) {
        k_residual64<MASKED><<<rblocks, kThreads, 0, s>>>(phi, b, ws.mask, ws.ctl, ws.partials, a, 1, 0, 1);
        n++;
    }
    PCD_CUDA(cudaGetLastError());
    *nodes = n;
    return PCD_OK;
}

// Smallest grid (cells) that AUTO hands to the tile passes rather than the
// persistent schedule (the smallest size measured: 64^2, where the tile
// passes took 1.0 ms against 2.2 ms to the reference's stop at 1e-7).
constexpr long kTileMinCells = 64L * 64L;

int get_chunk_graph(SolverWorkspace &ws, const double *b, double *phi, const SolveArgs &a, int precision,
                    int masked, int sweeps, cudaStream_t s, SolverWorkspace::GraphEntry **out, int sched,
                    const StreamPlan &sp)
{
    std::vector<long long> key = {(long long)(uintptr_t)b, (long long)(uintptr_t)phi, a.W, a.H, a.ld, a.stop,
                                  a.max_iter, precision, masked, sweeps, sched, sp.G, sp.T, sp.R, sp.tma, sp.two,
                                  sp.tile.K, sp.tile.L, sp.tile.NQ, sp.tile_sweeps};
    long long tb, ob;
    std::memcpy(&tb, &a.tol, 8);
    std::memcpy(&ob, &a.omega, 8);
    key.push_back(tb);
    key.push_back(ob);
    auto it = ws.graphs.find(key);
    if (it != ws.graphs.end()) {
        *out = &it->second;
        return PCD_OK;
    }
    cudaGraph_t g;
    int nodes = 0;
    PCD_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    int st = masked ? enqueue_chunk<true>(ws, b, phi, a, precision, sweeps, s, &nodes, PCD_SCHED_LAUNCHES, sp)
                    : enqueue_chunk<false>(ws, b, phi, a, precision, sweeps, s, &nodes, sched, sp);
    cudaError_t ce = cudaStreamEndCapture(s, &g);
    if (st != PCD_OK) {
        if (ce == cudaSuccess) cudaGraphDestroy(g);
        return st;
    }
    if (ce != cudaSuccess) {
        set_error(std::string("cudaStreamEndCapture: ") + cudaGetErrorString(ce));
        return PCD_DEVICE_ERROR;
    }
    cudaGraphExec_t exec;
    ce = cudaGraphInstantiate(&exec, g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) {
        set_error(std::string("cudaGraphInstantiate: ") + cudaGetErrorString(ce));
        return PCD_DEVICE_ERROR;
    }
    if (ws.graphs.size() > 64) {
        for (auto &kv : ws.graphs) cudaGraphExecDestroy(kv.second.exec);
        ws.graphs.clear();
    }
    auto &e = ws.graphs[key];
    e.exec = exec;
    e.nodes = nodes;
    *out = &e;
    return PCD_OK;
}

}  // namespace

namespace {

// One cooperative launch per solve (sor_persist.cu), bracketed by the FP64
// residual kernels that supply ||b|| / r64 before and the exact statistics after.
int solve_persistent(SolverWorkspace &ws, const double *b, double *phi, const SolveArgs &a, int precision,
                     const pcd_solve_opts &o, int G, size_t smem, pcd_solve_stats *stats, cudaStream_t s)
{
    const bool mixed = precision == PCD_PREC_MIXED;
    const size_t xe = (size_t)G * 4 * a.W;
    if (xe > ws.xbuf_elems) {
        if (ws.xbuf) cudaFree(ws.xbuf);
        ws.xbuf = nullptr;
        ws.xbuf_elems = 0;
        PCD_CUDA(cudaMalloc(&ws.xbuf, xe * sizeof(double)));
        ws.xbuf_elems = xe;
    }
    if (G > ws.max_ctas) {
        if (ws.flags) cudaFree(ws.flags);
        if (ws.part) cudaFree(ws.part);
        ws.flags = nullptr;
        ws.part = nullptr;
        ws.max_ctas = 0;
        PCD_CUDA(cudaMalloc(&ws.flags, (G + 1) * sizeof(unsigned)));
        PCD_CUDA(cudaMalloc(&ws.part, 2 * 3 * G * sizeof(double)));
        ws.max_ctas = G;
    }
    PCD_CUDA(cudaMemsetAsync(ws.flags, 0, (G + 1) * sizeof(unsigned), s));

    PersistArgs pa{};
    pa.W = a.W; pa.H = a.H; pa.ld = a.ld; pa.G = G;
    pa.b = b; pa.phi = phi; pa.r64 = ws.r64;
    pa.xbuf = ws.xbuf; pa.flags = ws.flags; pa.bar = ws.flags + G; pa.part = ws.part; pa.ctl = ws.ctl;
    pa.stop = a.stop; pa.max_iter = a.max_iter; pa.tol = a.tol;
    if (o.check_every > 0) pa.check_every = o.check_every;
    else if (a.stop == PCD_STOP_MAX_UPDATE) pa.check_every = mixed ? 16 : 8;
    else pa.check_every = 32;
    if (mixed && o.refine_every > 0 && o.refine_every < pa.check_every) pa.check_every = o.refine_every;
    for (int c = 0; c < 5; c++) { pa.w64[c] = a.w64[c]; pa.w32[c] = a.w32[c]; }
    pa.spin_limit = ws.wait_limit > 0 ? ws.wait_limit : 1ll << 24;
    pa.withhold = ws.withhold_flag;
    PCD_CUDA(cudaEventRecord(ws.k0, s));
    PCD_TRY(launch_persist(pa, mixed, smem, s));
    PCD_CUDA(cudaEventRecord(ws.k1, s));

    // exact FP64 statistics of the returned phi
    const int rblocks = grid_blocks((long)a.W * a.H);
    k_residual64<false><<<rblocks, kThreads, 0, s>>>(phi, b, ws.mask, ws.ctl, ws.partials, a, 0, 1, 0);
    PCD_LAUNCHED(1);
    PCD_CUDA(cudaEventRecord(ws.t1, s));
    PCD_CUDA(cudaMemcpyAsync(&ws.ctl_host[0], ws.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s));
    PCD_CUDA(cudaStreamSynchronize(s));
    const Ctl &c = ws.ctl_host[0];
    if (c.error) {
        set_error("persistent SOR: a bounded device wait gave up (status " + std::to_string(c.error) + ")");
        return c.error;
    }
    int converged = c.converged;
    if (a.stop == PCD_STOP_REL_RESIDUAL) converged = c.rel <= a.tol;
    if (stats) {
        stats->sweeps = c.sweeps;
        stats->converged = converged;
        stats->rel_residual = c.rel;
        stats->max_residual = c.rmax;
        stats->last_max_update = c.last_max;
        stats->residual_checks = c.checks + 2;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ws.t0, ws.t1);
        stats->device_ms = ms;
        cudaEventElapsedTime(&ms, ws.k0, ws.k1);
        stats->sweep_ms = ms;
        stats->schedule_used = PCD_SCHED_PERSISTENT;
    }
    return converged ? PCD_OK : PCD_NOT_CONVERGED;
}

// The CTA-count dependent buffers of the persistent schedules: G epoch flags
// plus a barrier counter, and 2 x G x 3 check partials.
int reserve_ctas(SolverWorkspace &ws, int G)
{
    if (G > ws.max_ctas) {
        if (ws.flags) cudaFree(ws.flags);
        if (ws.part) cudaFree(ws.part);
        ws.flags = nullptr;
        ws.part = nullptr;
        ws.max_ctas = 0;
        PCD_CUDA(cudaMalloc(&ws.flags, (G + 1) * sizeof(unsigned)));
        PCD_CUDA(cudaMalloc(&ws.part, 2 * 3 * G * sizeof(double)));
        ws.max_ctas = G;
    }
    return PCD_OK;
}

// One cooperative launch per solve on 2-D blocks with deep halos
// (sor_blocks.cu), then the exact FP64 statistics of the returned phi.
int solve_blocks(SolverWorkspace &ws, const double *b, double *phi, const SolveArgs &a, int precision,
                 const pcd_solve_opts &o, const BlocksPlan &bp, pcd_solve_stats *stats, cudaStream_t s)
{
    const bool mixed = precision == PCD_PREC_MIXED;
    const int G = bp.TY * bp.TX;
    const int xs = (a.W + 3) & ~3;
    const size_t elt = mixed ? sizeof(float) : sizeof(double);
    const size_t need = 2 * (size_t)a.H * xs * elt + (mixed ? (size_t)a.H * xs * sizeof(float) : 0);
    if (need > ws.bx_bytes) {
        if (ws.bx) cudaFree(ws.bx);
        ws.bx = nullptr;
        ws.bx_bytes = 0;
        PCD_CUDA(cudaMalloc(&ws.bx, need));
        ws.bx_bytes = need;
    }
    PCD_TRY(reserve_ctas(ws, G));
    PCD_CUDA(cudaMemsetAsync(ws.flags, 0, (G + 1) * sizeof(unsigned), s));

    BlocksArgs ba{};
    ba.W = a.W; ba.H = a.H; ba.ld = a.ld;
    ba.TY = bp.TY; ba.TX = bp.TX; ba.G = G; ba.K = bp.K; ba.RTmax = bp.RTmax; ba.xs = xs;
    ba.b = b; ba.phi = phi; ba.r64 = ws.r64;
    ba.xb = ws.bx;
    ba.r32x = mixed ? reinterpret_cast<float *>(static_cast<char *>(ws.bx) + 2 * (size_t)a.H * xs * elt) : nullptr;
    ba.flags = ws.flags; ba.part = ws.part; ba.ctl = ws.ctl;
    ba.stop = a.stop; ba.max_iter = a.max_iter; ba.tol = a.tol; ba.omega = a.omega;
    // a stop test costs a grid barrier (a few L2 round trips): every 16
    // sweeps for the max-update stop, 32 for the relative residual
    int ce = o.check_every > 0 ? o.check_every : (a.stop == PCD_STOP_MAX_UPDATE ? 16 : 32);
    ce = std::max(bp.K, (ce + bp.K - 1) / bp.K * bp.K);  // a multiple of the sweeps per exchange
    ba.check_every = ce;
    ba.cycle_cap = o.refine_every > 0 ? o.refine_every : 2048;
    ba.drop = o.refine_drop > 0.0 ? o.refine_drop : 3e-2;
    for (int c = 0; c < 5; c++) { ba.w64[c] = a.w64[c]; ba.w32[c] = a.w32[c]; }
    ba.spin_limit = ws.wait_limit > 0 ? ws.wait_limit : 1ll << 24;
    ba.withhold = ws.withhold_flag;
    PCD_CUDA(cudaEventRecord(ws.k0, s));
    PCD_TRY(launch_blocks(ba, mixed, bp.smem, s));
    PCD_CUDA(cudaEventRecord(ws.k1, s));

    // exact FP64 statistics of the returned phi
    const int rblocks = grid_blocks((long)a.W * a.H);
    k_residual64<false><<<rblocks, kThreads, 0, s>>>(phi, b, ws.mask, ws.ctl, ws.partials, a, 0, 1, 0);
    PCD_LAUNCHED(1);
    PCD_CUDA(cudaEventRecord(ws.t1, s));
    PCD_CUDA(cudaMemcpyAsync(&ws.ctl_host[0], ws.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s));
    PCD_CUDA(cudaStreamSynchronize(s));
    const Ctl &c = ws.ctl_host[0];
    if (c.error) {
        set_error("block SOR: a bounded device wait gave up (status " + std::to_string(c.error) + ")");
        return c.error;
    }
    int converged = c.converged;
    if (a.stop == PCD_STOP_REL_RESIDUAL) converged = c.rel <= a.tol;
    if (stats) {
        stats->sweeps = c.sweeps;
        stats->converged = converged;
        stats->rel_residual = c.rel;
        stats->max_residual = c.rmax;
        stats->last_max_update = c.last_max;
        stats->residual_checks = c.checks + 2;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ws.t0, ws.t1);
        stats->device_ms = ms;
        cudaEventElapsedTime(&ms, ws.k0, ws.k1);
        stats->sweep_ms = ms;
        stats->schedule_used = PCD_SCHED_BLOCKS;
        stats->check_every_used = ce;
    }
    return converged ? PCD_OK : PCD_NOT_CONVERGED;
}

}  // namespace

namespace {

// Mixed precision on one cluster: cycles of [FP32 cluster sweeps, FP64
// residual refresh, phi += e] until the FP64 relative residual passes.  The
// next cycle is launched before the previous one's control block is read; a
// cycle launched after convergence returns at once.
int solve_cluster(SolverWorkspace &ws, const double *b, double *phi, const SolveArgs &a, const pcd_solve_opts &o,
                  const ClusterPlan &plan, pcd_solve_stats *stats, cudaStream_t s)
{
    const int rblocks = grid_blocks((long)a.W * a.H);
    PCD_CUDA(cudaMemsetAsync(ws.e32, 0, sizeof(float) * (size_t)a.H * a.ld, s));
    // r32 = b - L phi0; ||b||; stop test on the initial guess
    k_refine_residual<false><<<rblocks, kThreads, 0, s>>>(phi, ws.e32, b, ws.mask, ws.r32, ws.ctl, ws.partials, a, 1);
    PCD_LAUNCHED(1);
    k_refine_update<<<rblocks, kThreads, 0, s>>>(phi, ws.e32, ws.ctl, a);
    PCD_LAUNCHED(1);

    ClusterArgs ca{};
    ca.W = a.W; ca.H = a.H; ca.ld = a.ld; ca.khp = plan.khp;
    ca.e = ws.e32; ca.r32 = ws.r32; ca.ctl = ws.ctl;
    ca.check_every = o.check_every > 0 ? o.check_every : 16;
    ca.cycle_cap = o.refine_every > 0 ? o.refine_every : 2048;
    ca.max_iter = a.max_iter;
    ca.tol = a.tol;
    ca.drop = o.refine_drop > 0.0 ? o.refine_drop : 3e-2;
    for (int c = 0; c < 5; c++) ca.w32[c] = a.w32[c];
    ca.one_minus_omega = (float)(1.0 - a.omega);
    ca.depth = plan.depth;

    PCD_CUDA(cudaEventRecord(ws.k0, s));
    long launched = 0;
    const long max_cycles = (long)a.max_iter + 4;
    bool finished = false;
    while (!finished) {
        if (launched >= max_cycles) {
            set_error("cluster SOR: cycle budget exceeded without a done flag");
            return PCD_TIMEOUT;
        }
        PCD_TRY(launch_cluster(ca, plan, s));
        k_refine_residual<false><<<rblocks, kThreads, 0, s>>>(phi, ws.e32, b, ws.mask, ws.r32, ws.ctl, ws.partials, a, 0);
        PCD_LAUNCHED(1);
        k_refine_update<<<rblocks, kThreads, 0, s>>>(phi, ws.e32, ws.ctl, a);
        PCD_LAUNCHED(1);
        const int slot = (int)(launched & 1);
        PCD_CUDA(cudaMemcpyAsync(&ws.ctl_host[slot], ws.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s));
        PCD_CUDA(cudaEventRecord(ws.ev[slot], s));
        launched++;
        if (launched >= 2) {
            const int prev = (int)((launched - 2) & 1);
            PCD_CUDA(cudaEventSynchronize(ws.ev[prev]));
            if (ws.ctl_host[prev].done) finished = true;
        }
    }
    PCD_CUDA(cudaEventRecord(ws.k1, s));
    PCD_CUDA(cudaEventRecord(ws.t1, s));
    PCD_CUDA(cudaMemcpyAsync(&ws.ctl_host[0], ws.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s));
    PCD_CUDA(cudaStreamSynchronize(s));
    const Ctl &c = ws.ctl_host[0];
    if (stats) {
        stats->sweeps = c.sweeps;
        stats->converged = c.converged;
        stats->rel_residual = c.rel;
        stats->max_residual = c.rmax;
        stats->last_max_update = 0.0;
        stats->residual_checks = c.checks;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ws.t0, ws.t1);
        stats->device_ms = ms;
        cudaEventElapsedTime(&ms, ws.k0, ws.k1);
        stats->sweep_ms = ms;
        stats->schedule_used = PCD_SCHED_CLUSTER;
    }
    return c.converged ? PCD_OK : PCD_NOT_CONVERGED;
}

}  // namespace

int residual_rel(SolverWorkspace &ws, const double *b, const double *phi, int W, int H, int ld, cudaStream_t s,
                 double *rel)
{
    PCD_TRY(ws.reserve((size_t)H * ld));
    SolveArgs a{};
    a.W = W; a.H = H; a.ld = ld;
    a.stop = PCD_STOP_REL_RESIDUAL;
    PCD_CUDA(cudaMemsetAsync(ws.ctl, 0, sizeof(Ctl), s));
    const int rblocks = grid_blocks((long)W * H);
    k_mask<<<rblocks, kThreads, 0, s>>>(b, ws.mask, W, H, ld, ws.ctl);
    PCD_LAUNCHED(1);
    k_residual64<true><<<rblocks, kThreads, 0, s>>>(phi, b, ws.mask, ws.ctl, ws.partials, a, 0, 1, 0);
    PCD_LAUNCHED(1);
    PCD_CUDA(cudaMemcpyAsync(ws.ctl_host, ws.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s));
    PCD_CUDA(cudaStreamSynchronize(s));
    *rel = ws.ctl_host[0].rel;
    return PCD_OK;
}

int enqueue_smooth(const double *b, double *phi, uint8_t *mask, Ctl *ctl, double *partials, int W, int H, int ld,
                   int sweeps, double omega, cudaStream_t s)
{
    SolveArgs a{};
    a.W = W; a.H = H; a.ld = ld;
    a.stop = PCD_STOP_REL_RESIDUAL;
    a.max_iter = sweeps;
    a.tol = 0.0;
    a.omega = omega;
    for (int c = 0; c < 5; c++) {
        a.w64[c] = omega / (double)c;
        a.w32[c] = (float)omega / (float)c;
    }
    PCD_CUDA(cudaMemsetAsync(ctl, 0, sizeof(Ctl), s));
    const int rblocks = grid_blocks((long)W * H);
    k_mask<<<rblocks, kThreads, 0, s>>>(b, mask, W, H, ld, ctl);
    PCD_LAUNCHED(1);
    const int half = (W + 1) >> 1;
    const int blocks = ceil_div((long)H * half, kThreads);
    for (int k = 0; k < sweeps; k++)
        for (int color = 0; color < 2; color++) {
            k_rb_half<double, true, false><<<blocks, kThreads, 0, s>>>(phi, b, mask, ctl, a, color, color);
            PCD_LAUNCHED(1);
        }
    k_residual64<true><<<rblocks, kThreads, 0, s>>>(phi, b, mask, ctl, partials, a, 0, 1, 0);
    PCD_LAUNCHED(1);
    return PCD_OK;
}

int enqueue_smooth_mixed(const double *b, double *phi, float *e32, float *r32, Ctl *ctl, double *partials, int W,
                         int H, int ld, int sweeps, int dev, cudaStream_t s)
{
    ClusterPlan plan{};
    if (cluster_plan(dev, W, H, 4, &plan) != PCD_OK) {
        set_error("mixed smoothing: the grid does not fit one cluster");
        return PCD_BAD_ARG;
    }
    SolveArgs a{};
    a.W = W; a.H = H; a.ld = ld;
    a.stop = PCD_STOP_REL_RESIDUAL;
    a.max_iter = sweeps;
    a.tol = 0.0;
    a.omega = 1.0;
    for (int c = 0; c < 5; c++) {
        a.w64[c] = 1.0 / (double)c;
        a.w32[c] = 1.0f / (float)c;
    }
    PCD_CUDA(cudaMemsetAsync(ctl, 0, sizeof(Ctl), s));
    PCD_CUDA(cudaMemsetAsync(e32, 0, sizeof(float) * (size_t)H * ld, s));
    const int rblocks = grid_blocks((long)W * H);
    // r32 = b - L phi and ||b|| (FP64)
    k_refine_residual<false><<<rblocks, kThreads, 0, s>>>(phi, e32, b, nullptr, r32, ctl, partials, a, 1);
    PCD_LAUNCHED(1);
    // `sweeps` FP32 Gauss-Seidel sweeps of L e = r32 on one cluster (no
    // estimates, no early end: tolerance 0, drop 0, one cycle of `sweeps`)
    ClusterArgs ca{};
    ca.W = W; ca.H = H; ca.ld = ld; ca.khp = plan.khp;
    ca.e = e32; ca.r32 = r32; ca.ctl = ctl;
    ca.check_every = sweeps + 1;
    ca.cycle_cap = sweeps;
    ca.max_iter = sweeps;
    ca.tol = 0.0;
    ca.drop = 0.0;
    for (int c = 0; c < 5; c++) ca.w32[c] = a.w32[c];
    ca.one_minus_omega = 0.0f;
    ca.depth = plan.depth;
    PCD_TRY(launch_cluster(ca, plan, s));
    // ||b - L (phi + e)|| / ||b|| in FP64 into ctl->rel, then phi += e
    k_refine_residual<false><<<rblocks, kThreads, 0, s>>>(phi, e32, b, nullptr, r32, ctl, partials, a, 0);
    PCD_LAUNCHED(1);
    k_refine_update<<<rblocks, kThreads, 0, s>>>(phi, e32, ctl, a);
    PCD_LAUNCHED(1);
    return PCD_OK;
}

bool smooth_mixed_applies(int dev, int W, int H)
{
    ClusterPlan plan{};
    return cluster_plan(dev, W, H, 4, &plan) == PCD_OK;
}

size_t residual_partials_bytes() { return sizeof(double) * 3 * kResidualBlocksMax; }

int smooth_residual(SolverWorkspace &ws, const double *b, double *phi, int W, int H, int ld, int sweeps, double omega,
                    cudaStream_t s, double *rel)
{
    PCD_TRY(ws.reserve((size_t)H * ld));
    PCD_TRY(enqueue_smooth(b, phi, ws.mask, ws.ctl, ws.partials, W, H, ld, sweeps, omega, s));
    PCD_CUDA(cudaMemcpyAsync(ws.ctl_host, ws.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s));
    PCD_CUDA(cudaStreamSynchronize(s));
    *rel = ws.ctl_host[0].rel;
    return PCD_OK;
}

int zero_grid(double *phi, int W, int H, int ld, cudaStream_t s)
{
    k_fill<<<grid_blocks((long)W * H), kThreads, 0, s>>>(phi, W, H, ld, 0.0);
    PCD_LAUNCHED(1);
    return PCD_OK;
}

int solve_device(SolverWorkspace &ws, const double *b, double *phi, int W, int H, int ld, const pcd_solve_opts &o,
                 pcd_solve_stats *stats, cudaStream_t s)
{
    if (W < 1 || H < 1 || ld < W || !b || !phi) {
        set_error("pcd solve: bad grid arguments");
        return PCD_BAD_ARG;
    }
    if (o.max_iterations < 0 || o.stop < 0 || o.stop > 1 || o.precision < 0 || o.precision > 1) {
        set_error("pcd solve: bad options");
        return PCD_BAD_ARG;
    }
    PCD_TRY(ws.reserve((size_t)H * ld));

    SolveArgs a;
    a.W = W; a.H = H; a.ld = ld;
    a.stop = o.stop;
    a.max_iter = o.max_iterations;
    a.tol = o.tol;
    a.omega = resolve_omega(o.omega, W, H);
    for (int c = 0; c < 5; c++) {
        a.w64[c] = a.omega / (double)c;             // solver.cpp:47 divides omega by cnt
        a.w32[c] = (float)a.omega / (float)c;
    }
    const int precision = o.precision;

    PCD_CUDA(cudaEventRecord(ws.t0, s));
    PCD_CUDA(cudaMemsetAsync(ws.ctl, 0, sizeof(Ctl), s));
    const int rblocks = grid_blocks((long)W * H);
    k_mask<<<rblocks, kThreads, 0, s>>>(b, ws.mask, W, H, ld, ws.ctl);
    PCD_LAUNCHED(1);
    if (!o.warm_start) {
        k_fill<<<rblocks, kThreads, 0, s>>>(phi, W, H, ld, 0.0);
        PCD_LAUNCHED(1);
    }
    // Initial FP64 residual (masked form: valid with or without NaN cells);
    // it also yields ||b|| and, for the mixed form, the FP64 residual r64.
    k_residual64<true><<<rblocks, kThreads, 0, s>>>(phi, b, ws.mask, ws.ctl, ws.partials, a,
                                                   a.stop == PCD_STOP_REL_RESIDUAL, 1, 0,
                                                   precision == PCD_PREC_MIXED ? ws.r64 : nullptr);
    PCD_LAUNCHED(1);
    PCD_CUDA(cudaMemcpyAsync(ws.ctl_host, ws.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s));
    PCD_CUDA(cudaStreamSynchronize(s));
    const int masked = ws.ctl_host[0].nan_cells > 0 ? 1 : 0;
    const bool done_already = ws.ctl_host[0].converged != 0 || a.max_iter == 0;

    // FP64 sweeps: the block schedule (on chip, 2-D blocks, one L2 exchange per
    // K sweeps) before the persistent bands (one per half sweep): 6.4 against
    // 16.0 us per 512^2 sweep, 17 against 28 us (stripes) at 1024^2
    const bool auto_blocks = o.schedule == PCD_SCHED_AUTO && precision == PCD_PREC_FP64 &&
                             (long)W * H >= kTileMinCells;
    if (!done_already && !masked && (o.schedule == PCD_SCHED_BLOCKS || auto_blocks)) {
        BlocksPlan bp{};
        const bool mixed = precision == PCD_PREC_MIXED;
        int st = PCD_BAD_ARG;
        if (o.block_sweeps < 0 || o.block_sweeps > 8) {
            set_error("pcd solve: block_sweeps must be 0 (auto) or 1..8");
            return PCD_BAD_ARG;
        }
        if (o.block_sweeps > 0) st = blocks_plan(ws.dev, W, H, o.block_sweeps, mixed, &bp);
        else
            for (int K : {mixed ? 8 : 4, 4, 2, 1})
                if ((st = blocks_plan(ws.dev, W, H, K, mixed, &bp)) == PCD_OK) break;
        if (st == PCD_OK) return solve_blocks(ws, b, phi, a, precision, o, bp, stats, s);
    }
    if (!done_already && !masked && precision == PCD_PREC_MIXED && a.stop == PCD_STOP_REL_RESIDUAL &&
        (o.schedule == PCD_SCHED_AUTO || o.schedule == PCD_SCHED_CLUSTER)) {
        ClusterPlan plan{};
        if (cluster_plan(ws.dev, W, H, 4, &plan) == PCD_OK) return solve_cluster(ws, b, phi, a, o, plan, stats, s);
    }
    // FP32 sweeps beyond one cluster: the tile passes before the persistent
    // schedule (measured 2-3.5x faster from 64^2 to 1024^2)
    TilePlan tp_probe;
    const bool prefer_tiles = precision == PCD_PREC_MIXED && o.schedule != PCD_SCHED_PERSISTENT &&
                              (long)W * H >= kTileMinCells && tile_plan(ws.dev, W, H, ld, 4, &tp_probe) == PCD_OK;
    if (!done_already && !masked && !prefer_tiles &&
        (o.schedule == PCD_SCHED_AUTO || o.schedule == PCD_SCHED_PERSISTENT || o.schedule == PCD_SCHED_CLUSTER)) {
        int G = 0;
        size_t smem = 0;
        if (persist_grid(ws.dev, W, H, precision == PCD_PREC_MIXED, &G, &smem) == PCD_OK)
            return solve_persistent(ws, b, phi, a, precision, o, G, smem, stats, s);
    }

    if (done_already) {
        int one = 1;
        PCD_CUDA(cudaMemcpyAsync(&ws.ctl->halt, &one, sizeof(int), cudaMemcpyHostToDevice, s));
        PCD_CUDA(cudaMemcpyAsync(&ws.ctl->done, &one, sizeof(int), cudaMemcpyHostToDevice, s));
    } else if (precision == PCD_PREC_MIXED) {
        // first right-hand side of the FP32 correction sweeps
        PCD_CUDA(cudaMemsetAsync(ws.e32, 0, sizeof(float) * (size_t)H * ld, s));
        if (masked)
            k_refine_residual<true><<<rblocks, kThreads, 0, s>>>(phi, ws.e32, b, ws.mask, ws.r32, ws.ctl, ws.partials, a, 1);
        else
            k_refine_residual<false><<<rblocks, kThreads, 0, s>>>(phi, ws.e32, b, ws.mask, ws.r32, ws.ctl, ws.partials, a, 1);
        PCD_LAUNCHED(1);
    }

    // HBM grids without NaN cells: ping-pong tile passes or stream sweeps
    // (FP32), else fused in-place stripe sweeps (grids with at least 3 rows)
    int sched = PCD_SCHED_LAUNCHES;
    StreamPlan sp;
    if (!masked && precision == PCD_PREC_MIXED && o.schedule != PCD_SCHED_STREAM &&
        o.schedule != PCD_SCHED_LAUNCHES && o.schedule != PCD_SCHED_STRIPES) {
        // register-resident tile passes (4096^2 FP32 sweep: 26 us against the
        // stream pass's 40 us); check_every: sweeps per pass (stop tests
        // after every pass), 4 at most
        sp.tile_sweeps = o.check_every > 0 ? std::min(o.check_every, 4) : 4;
        if (tile_plan(ws.dev, W, H, ld, sp.tile_sweeps <= 2 ? 2 : 4, &sp.tile) == PCD_OK) sched = PCD_SCHED_TILES;
    }
    if (sched == PCD_SCHED_TILES) {
        // chosen above
    } else if (!masked && precision == PCD_PREC_MIXED &&
               (o.schedule == PCD_SCHED_AUTO || o.schedule == PCD_SCHED_STREAM ||
                o.schedule == PCD_SCHED_PERSISTENT || o.schedule == PCD_SCHED_CLUSTER ||
                o.schedule == PCD_SCHED_TILES) &&
               stream_plan(ws.dev, W, H, ld, true, &sp) == PCD_OK) {
        sched = PCD_SCHED_STREAM;
    } else if (!masked && H >= 3 && W <= 2 * kRowCellsMax * kStripeThreads && o.schedule != PCD_SCHED_LAUNCHES) {
        sched = PCD_SCHED_STRIPES;
    }
    const bool stripes = sched == PCD_SCHED_STRIPES;
    if (stripes && ws.stripe_resident == 0) {
        int sms = 0, bps = 0;
        PCD_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ws.dev));
        PCD_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_stripe_a<double, false, 4>, kStripeThreads, 0));
        ws.stripe_resident = std::max(1, bps) * sms;
    }
    int chunk;
    if (a.stop == PCD_STOP_MAX_UPDATE)
        // mixed: FP32 sweeps between FP64 refreshes (the stop test runs after
        // every sweep either way)
        chunk = precision == PCD_PREC_MIXED
                    ? (o.refine_every > 0 ? o.refine_every : std::max(32, std::min(128, std::max(W, H) / 32)))
                    : 32;
    else if (precision == PCD_PREC_MIXED)
        // the FP64 refresh costs several FP32 sweeps; FP32 can carry ~2 digits
        // of the correction, i.e. hundreds of sweeps on large grids
        chunk = o.refine_every > 0 ? o.refine_every
                                   : (o.check_every > 0 ? o.check_every
                                                        : std::max(32, std::min(256, std::max(W, H) / 16)));
    else
        chunk = o.check_every > 0 ? o.check_every : 32;
    if (chunk > a.max_iter && a.max_iter > 0) chunk = a.max_iter;

    SolverWorkspace::GraphEntry *ge = nullptr;
    if (!done_already) PCD_TRY(get_chunk_graph(ws, b, phi, a, precision, masked, chunk, s, &ge, sched, sp));

    PCD_CUDA(cudaEventRecord(ws.k0, s));
    // Chunk loop: launch chunk i+1 before inspecting chunk i's control block.
    const long max_chunks = a.max_iter > 0 ? (long)a.max_iter / chunk + 3 : 0;
    long launched = 0;
    int finished = done_already;
    auto flag_done = [&](const Ctl &c) { return precision == PCD_PREC_MIXED ? c.done : c.halt; };
    while (!finished) {
        if (launched >= max_chunks) {
            set_error("pcd solve: chunk budget exceeded without a halt flag");
            return PCD_TIMEOUT;
        }
        PCD_CUDA(cudaGraphLaunch(ge->exec, s));
        count_launches(ge->nodes);
        const int slot = (int)(launched & 1);
        PCD_CUDA(cudaMemcpyAsync(&ws.ctl_host[slot], ws.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s));
        PCD_CUDA(cudaEventRecord(ws.ev[slot], s));
        launched++;
        if (launched >= 2) {
            const int prev = (int)((launched - 2) & 1);
            PCD_CUDA(cudaEventSynchronize(ws.ev[prev]));
            if (flag_done(ws.ctl_host[prev])) finished = 1;
        }
    }
    PCD_CUDA(cudaEventRecord(ws.k1, s));
    // Final statistics (FP64 residual of the returned phi).
    if (precision != PCD_PREC_MIXED) {
        if (masked)
            k_residual64<true><<<rblocks, kThreads, 0, s>>>(phi, b, ws.mask, ws.ctl, ws.partials, a, 0, 1, 0);
        else
            k_residual64<false><<<rblocks, kThreads, 0, s>>>(phi, b, ws.mask, ws.ctl, ws.partials, a, 0, 1, 0);
        PCD_LAUNCHED(1);
    }
    PCD_CUDA(cudaEventRecord(ws.t1, s));
    PCD_CUDA(cudaMemcpyAsync(&ws.ctl_host[0], ws.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s));
    PCD_CUDA(cudaStreamSynchronize(s));
    const Ctl &c = ws.ctl_host[0];
    if (c.error) {
        set_error("stream SOR: a bounded wait for a row copy gave up (status " + std::to_string(c.error) + ")");
        return c.error;
    }
    if (stats) {
        stats->sweeps = c.sweeps;
        stats->converged = c.converged;
        stats->rel_residual = c.rel;
        stats->max_residual = c.rmax;
        stats->last_max_update = c.last_max;
        stats->residual_checks = c.checks;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ws.t0, ws.t1);
        stats->device_ms = ms;
        cudaEventElapsedTime(&ms, ws.k0, ws.k1);
        stats->sweep_ms = ms;
        stats->schedule_used = sched;
    }
    return c.converged ? PCD_OK : PCD_NOT_CONVERGED;
}


// ---------------------------------------------------------------------------
// Batched tile solve: the grids of a batch share one tile pass per launch
// (k_sor_tile_batch) and one FP64 refresh pair per chunk of passes, each
// grid with its own control block, so a grid that has converged drops out
// while the others go on.
namespace {

// One grid of the batched FP64 refresh: blocks [blk0, blk0 + nblk) of the
// launch work on it.
struct RefineJob {
    const double *b;
    double *phi;
    float *e, *eb;       // the correction buffers (eb holds the latest when stream_out is set)
    float *r32;
    Ctl *ctl;
    double *partials;    // 3 per block
    int W, H, ld;
    int blk0, nblk;
};

// Blocks per grid of the batched FP64 refresh: about 4 cells per thread, so
// that the large grids' FP64 work spreads over every SM.
constexpr int kBatchRefineBlocks = 1024;
constexpr int kBatchRefineCellsPerBlock = 4 * kThreads;

__device__ __forceinline__ int refine_job(const RefineJob *jobs, int njobs, int blk)
{
    int lo = 0, hi = njobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(&jobs[mid].blk0) <= blk) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ bool last_block_of(Ctl *ctl, int nblk)
{
    __shared__ bool is_last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned t = atomicAdd(&ctl->blocks_done_r, 1u);
        is_last = (t == (unsigned)nblk - 1u);
    }
    __syncthreads();
    if (is_last) __threadfence();
    return is_last;
}

// r = b - L(phi + e) in FP64 per grid (the latest correction buffer), r32 =
// (float) r, norms and the relative-residual test by each grid's last block.
__global__ void __launch_bounds__(kThreads)
    k_batch_refine_residual(const RefineJob *__restrict__ jobs, int njobs, double tol, int with_b)
{
    const RefineJob &J = jobs[refine_job(jobs, njobs, blockIdx.x)];
    Ctl *ctl = J.ctl;
    if (vol_load(&ctl->done)) return;
    const float *__restrict__ e = vol_load(&ctl->stream_out) ? J.eb : J.e;
    const int lb = (int)blockIdx.x - J.blk0, W = J.W, H = J.H, ld = J.ld;
    const long n = (long)W * H;
    double v[3] = {0.0, 0.0, 0.0};
    for (long t = (long)lb * blockDim.x + threadIdx.x; t < n; t += (long)J.nblk * blockDim.x) {
        const int y = (int)(t / W), x = (int)(t - (long)y * W);
        const long i = (long)y * ld + x;
        const double bi = J.b[i];
        // the neighbour sum in k_refine_residual's order; the count as an integer
        double sum = 0.0;
        int cnt = 0;
        if (x > 0) { cnt++; sum += J.phi[i - 1] + (double)e[i - 1]; }
        if (y > 0) { cnt++; sum += J.phi[i - ld] + (double)e[i - ld]; }
        if (x < W - 1) { cnt++; sum += J.phi[i + 1] + (double)e[i + 1]; }
        if (y < H - 1) { cnt++; sum += J.phi[i + ld] + (double)e[i + ld]; }
        const double xi = J.phi[i] + (double)e[i];
        const double r = bi - (sum - (double)cnt * xi);
        J.r32[i] = (float)r;
        if (isnan(bi)) continue;
        v[0] += r * r;
        v[1] += bi * bi;
        v[2] = nan_skip_max(v[2], fabs(r));
    }
    block_reduce<3, 4u>(v);
    if (threadIdx.x == 0) {
        J.partials[3 * lb] = v[0];
        J.partials[3 * lb + 1] = v[1];
        J.partials[3 * lb + 2] = v[2];
    }
    if (last_block_of(ctl, J.nblk)) {
        SolveArgs a{};
        a.stop = PCD_STOP_REL_RESIDUAL;
        a.tol = tol;
        finalize_residual(ctl, J.partials, J.nblk, a, 1, with_b);
    }
}

// phi += latest correction, e = 0 per grid; a halted grid is done.
__global__ void __launch_bounds__(kThreads) k_batch_refine_update(const RefineJob *__restrict__ jobs, int njobs)
{
    const RefineJob &J = jobs[refine_job(jobs, njobs, blockIdx.x)];
    Ctl *ctl = J.ctl;
    if (vol_load(&ctl->done)) return;
    const float *el = vol_load(&ctl->stream_out) ? J.eb : J.e;
    const int lb = (int)blockIdx.x - J.blk0, W = J.W, ld = J.ld;
    const long n = (long)W * J.H;
    for (long t = (long)lb * blockDim.x + threadIdx.x; t < n; t += (long)J.nblk * blockDim.x) {
        const int y = (int)(t / W), x = (int)(t - (long)y * W);
        const long i = (long)y * ld + x;
        J.phi[i] += (double)el[i];
        J.e[i] = 0.0f;
    }
    if (last_block_of(ctl, J.nblk)) {
        if (threadIdx.x == 0) {
            volatile Ctl *c = ctl;
            if (c->halt) c->done = 1;
            c->stream_out = 0;
            c->blocks_done_r = 0;
            __threadfence();
        }
    }
}

}  // namespace

int TileBatchWorkspace::reserve(size_t floats, int count)
{
    if (floats > arena_floats) {
        for (auto &kv : graphs) cudaGraphExecDestroy(kv.second);
        graphs.clear();
        if (arena) cudaFree(arena);
        arena = nullptr;
        arena_floats = 0;
        PCD_CUDA(cudaMalloc(&arena, floats * sizeof(float)));
        arena_floats = floats;
    }
    if (count > cap) {
        for (auto &kv : graphs) cudaGraphExecDestroy(kv.second);
        graphs.clear();
        if (ctl) cudaFree(ctl);
        if (ctl_host) cudaFreeHost(ctl_host);
        if (partials) cudaFree(partials);
        if (jobs) cudaFree(jobs);
        if (rjobs) cudaFree(rjobs);
        ctl = nullptr; ctl_host = nullptr; partials = nullptr; jobs = nullptr; rjobs = nullptr;
        cap = 0;
        PCD_CUDA(cudaMalloc(&ctl, sizeof(Ctl) * count));
        PCD_CUDA(cudaMallocHost(&ctl_host, 2 * sizeof(Ctl) * count));
        PCD_CUDA(cudaMalloc(&partials, sizeof(double) * 3 * kBatchRefineBlocks * count));
        PCD_CUDA(cudaMalloc(&jobs, sizeof(TileJob) * count));
        PCD_CUDA(cudaMalloc(&rjobs, sizeof(RefineJob) * count));
        cap = count;
    }
    if (!t0) {
        PCD_CUDA(cudaEventCreate(&t0));
        PCD_CUDA(cudaEventCreate(&t1));
        PCD_CUDA(cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming));
        PCD_CUDA(cudaEventCreateWithFlags(&ev[1], cudaEventDisableTiming));
        PCD_CUDA(cudaMalloc(&counter, sizeof(unsigned)));
    }
    return PCD_OK;
}

void TileBatchWorkspace::release()
{
    for (auto &kv : graphs) cudaGraphExecDestroy(kv.second);
    graphs.clear();
    if (arena) cudaFree(arena);
    if (ctl) cudaFree(ctl);
    if (ctl_host) cudaFreeHost(ctl_host);
    if (partials) cudaFree(partials);
    if (jobs) cudaFree(jobs);
    if (rjobs) cudaFree(rjobs);
    if (counter) cudaFree(counter);
    for (cudaEvent_t *e : {&t0, &t1, &ev[0], &ev[1]})
        if (*e) cudaEventDestroy(*e);
    *this = TileBatchWorkspace();
}

bool batch_tiles_apply(const pcd_instance *inst, int count)
{
    if (!inst || count < 1 || count > kTileBatchJobsMax) return false;
    for (int i = 0; i < count; i++) {
        const pcd_instance &q = inst[i];
        if (!q.b || !q.phi || q.width < 8 || q.height < 1 || q.width % 8 != 0 || q.ld < q.width || q.ld % 4 != 0)
            return false;
    }
    return true;
}

int batch_tiles_solve(TileBatchWorkspace &ws, int dev, const pcd_instance *inst, int count, const pcd_solve_opts &o,
                      pcd_instance_stats *stats, pcd_batch_stats *bstats, cudaStream_t s)
{
    if (!batch_tiles_apply(inst, count)) {
        set_error("batched tile solve: every grid needs a width that is a multiple of 8 and ld a multiple of 4, "
                  "and at most " + std::to_string(kTileBatchJobsMax) + " grids");
        return PCD_BAD_ARG;
    }
    if (o.stop != PCD_STOP_REL_RESIDUAL || !(o.tol > 0.0) || o.max_iterations < 1) {
        set_error("pcd_batch_solve_device: the batch solve takes the relative-residual stop with tol > 0");
        return PCD_BAD_ARG;
    }
    size_t smem = 0;
    int grid = 0;
    PCD_TRY(tile_batch_config(dev, count, &smem, &grid));
    size_t per = 0;
    for (int i = 0; i < count; i++) per += (size_t)inst[i].height * inst[i].ld;
    PCD_TRY(ws.reserve(3 * per, count));

    // largest grids first: their refresh blocks are dispatched first
    std::vector<int> order(count);
    for (int i = 0; i < count; i++) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
        return (long)inst[x].width * inst[x].height > (long)inst[y].width * inst[y].height;
    });
    std::vector<TileJob> tj((size_t)count);
    std::vector<RefineJob> rj((size_t)count);
    size_t off = 0;
    int tiles = 0, blocks = 0, maxdim = 0;
    for (int k = 0; k < count; k++) {
        const int i = order[k];
        const pcd_instance &q = inst[i];
        maxdim = std::max(maxdim, std::max(q.width, q.height));
        TileJob &t = tj[k];
        RefineJob &r = rj[k];
        t.ea = ws.arena + off;
        t.eb = ws.arena + per + off;
        t.r32 = ws.arena + 2 * per + off;
        t.ctl = ws.ctl + k;
        t.W = q.width;
        t.H = q.height;
        t.ld = q.ld;
        tile_counts(q.width, q.height, &t.ncol, &t.nrow);
        t.tile0 = tiles;
        t.max_iter = o.max_iterations;
        const double om = resolve_omega(o.omega, q.width, q.height);
        for (int c = 0; c < 5; c++) t.w32[c] = (float)om / (float)c;
        tiles += t.ncol * t.nrow;
        r.b = q.b;
        r.phi = q.phi;
        r.e = t.ea;
        r.eb = t.eb;
        r.r32 = ws.arena + 2 * per + off;
        r.ctl = t.ctl;
        r.partials = ws.partials + (size_t)3 * kBatchRefineBlocks * k;
        r.W = q.width;
        r.H = q.height;
        r.ld = q.ld;
        r.blk0 = blocks;
        r.nblk = (int)std::min<long>(kBatchRefineBlocks,
                                     ((long)q.width * q.height + kBatchRefineCellsPerBlock - 1) /
                                         kBatchRefineCellsPerBlock);
        blocks += r.nblk;
        off += (size_t)q.height * q.ld;
    }
    const TileJob *d_jobs = static_cast<const TileJob *>(ws.jobs);
    const RefineJob *d_rjobs = static_cast<const RefineJob *>(ws.rjobs);
    // sweeps between FP64 refreshes (passes of 4, the last one shorter):
    // refine_every, else 128 when the largest side is 1024 or more, down to
    // 32 when it is 256 or less
    const int chunk = o.refine_every > 0 ? o.refine_every : 4 * std::max(8, std::min(32, maxdim / 32));
    const int passes = (chunk + 3) / 4;

    PCD_CUDA(cudaEventRecord(ws.t0, s));
    PCD_CUDA(cudaMemcpyAsync(ws.jobs, tj.data(), sizeof(TileJob) * count, cudaMemcpyHostToDevice, s));
    PCD_CUDA(cudaMemcpyAsync(ws.rjobs, rj.data(), sizeof(RefineJob) * count, cudaMemcpyHostToDevice, s));
    PCD_CUDA(cudaMemsetAsync(ws.ctl, 0, sizeof(Ctl) * count, s));
    PCD_CUDA(cudaMemsetAsync(ws.counter, 0, sizeof(unsigned), s));
    PCD_CUDA(cudaMemsetAsync(ws.arena, 0, sizeof(float) * per, s));
    if (!o.warm_start)
        for (int i = 0; i < count; i++)
            PCD_CUDA(cudaMemset2DAsync(inst[i].phi, sizeof(double) * inst[i].ld, 0, sizeof(double) * inst[i].width,
                                       inst[i].height, s));
    // first right-hand side, ||b|| and the stop test of the starting phi
    k_batch_refine_residual<<<blocks, kThreads, 0, s>>>(d_rjobs, count, o.tol, 1);
    k_batch_refine_update<<<blocks, kThreads, 0, s>>>(d_rjobs, count);
    PCD_LAUNCHED(2);

    // one CUDA graph per batch signature: the chunk's passes and the refresh
    std::vector<long long> key = {count, tiles, blocks, chunk, grid, (long long)smem,
                                  (long long)(uintptr_t)ws.jobs, (long long)(uintptr_t)ws.rjobs};
    {
        long long tb;
        std::memcpy(&tb, &o.tol, 8);
        key.push_back(tb);
    }
    cudaGraphExec_t exec = nullptr;
    auto it = ws.graphs.find(key);
    if (it != ws.graphs.end()) {
        exec = it->second;
    } else {
        cudaGraph_t g;
        PCD_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        int st = PCD_OK;
        for (int k = 0; k < passes && st == PCD_OK; k++)
            st = launch_tile_batch(d_jobs, count, tiles, std::min(4, chunk - 4 * k), k & 1, grid, smem, ws.counter,
                                   s);
        k_batch_refine_residual<<<blocks, kThreads, 0, s>>>(d_rjobs, count, o.tol, 0);
        k_batch_refine_update<<<blocks, kThreads, 0, s>>>(d_rjobs, count);
        cudaError_t ce = cudaStreamEndCapture(s, &g);
        if (st != PCD_OK) {
            if (ce == cudaSuccess) cudaGraphDestroy(g);
            return st;
        }
        if (ce != cudaSuccess) {
            set_error(std::string("batched tile graph capture: ") + cudaGetErrorString(ce));
            return PCD_DEVICE_ERROR;
        }
        ce = cudaGraphInstantiate(&exec, g, 0);
        cudaGraphDestroy(g);
        if (ce != cudaSuccess) {
            set_error(std::string("batched tile graph instantiate: ") + cudaGetErrorString(ce));
            return PCD_DEVICE_ERROR;
        }
        if (ws.graphs.size() > 16) {
            for (auto &kv : ws.graphs) cudaGraphExecDestroy(kv.second);
            ws.graphs.clear();
        }
        ws.graphs[key] = exec;
    }

    // chunk i+1 is launched before chunk i's control blocks are inspected
    const long max_chunks = (long)o.max_iterations / chunk + 3;
    long launched = 0;
    bool finished = false;
    auto all_done = [&](const Ctl *c) {
        for (int i = 0; i < count; i++)
            if (!c[i].done) return false;
        return true;
    };
    while (!finished) {
        if (launched >= max_chunks) {
            set_error("batched tile solve: chunk budget exceeded without every grid done");
            return PCD_TIMEOUT;
        }
        PCD_CUDA(cudaGraphLaunch(exec, s));
        count_launches(passes + 2);
        const int slot = (int)(launched & 1);
        PCD_CUDA(cudaMemcpyAsync(ws.ctl_host + (size_t)slot * count, ws.ctl, sizeof(Ctl) * count,
                                 cudaMemcpyDeviceToHost, s));
        PCD_CUDA(cudaEventRecord(ws.ev[slot], s));
        launched++;
        if (launched >= 2) {
            const int prev = (int)((launched - 2) & 1);
            PCD_CUDA(cudaEventSynchronize(ws.ev[prev]));
            if (all_done(ws.ctl_host + (size_t)prev * count)) finished = true;
        }
    }
    PCD_CUDA(cudaEventRecord(ws.t1, s));
    PCD_CUDA(cudaMemcpyAsync(ws.ctl_host, ws.ctl, sizeof(Ctl) * count, cudaMemcpyDeviceToHost, s));
    PCD_CUDA(cudaStreamSynchronize(s));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ws.t0, ws.t1);
    int all = 1;
    long long cell_sweeps = 0;
    for (int k = 0; k < count; k++) {
        const int i = order[k];
        const Ctl &c = ws.ctl_host[k];
        if (stats) {
            stats[i].sweeps = c.sweeps;
            stats[i].converged = c.converged;
            stats[i].rel_residual = c.rel;
            stats[i].cycles = c.checks;
        }
        all &= c.converged;
        cell_sweeps += (long long)inst[i].width * inst[i].height * c.sweeps;
    }
    if (bstats) {
        bstats->device_ms = ms;
        bstats->clusters = 0;
        bstats->cluster_size = 0;
        bstats->smem_bytes = (long long)smem;
        bstats->cell_sweeps = cell_sweeps;
        bstats->check_every = chunk;
        bstats->refine_drop = 0.0;
        bstats->tuned = 0;
    }
    return all ? PCD_OK : PCD_NOT_CONVERGED;
}

}  // namespace pcd
