// sor_blocks.cu -- persistent red-black SOR over 2-D blocks with deep halos
// (sm_103a): one cooperative launch per solve, the whole chip on one grid.
//
// The grid is cut into TY x TX blocks, one CTA each.  A CTA keeps the region
// of its block -- the owned cells plus a halo of h = 2K cells on every side --
// in shared memory and runs K red-black sweeps on it between exchanges.  The
// dependency cone of K sweeps (2K half sweeps, one cell per half sweep) ends
// inside the halo, so after the K sweeps the owned cells are exactly what K
// sweeps over the whole grid would give; the halo values are recomputed
// copies, thrown away.  Then each CTA writes its owned cells to an exchange
// grid (double-buffered by pass parity), raises its epoch flag (st.release),
// waits for its eight neighbours' flags (ld.acquire, bounded) and reloads the
// halo ring from their owned cells.  Against the persistent band schedule
// (sor_persist.cu), which trades boundary rows through L2 after every half
// sweep, this pays one L2 round trip per K sweeps and spreads a 512^2 grid
// over ~144 SMs instead of bands of 3-4 rows.
//
// Region layout: 64 columns, lane k holding the column pair (ox + 2k,
// ox + 2k + 1) with ox even, so that colour planes are conflict-free: plane c
// row r index k is the cell of colour c (colour = (x + y) & 1) of lane k's
// pair.  A cell's vertical neighbours are the other plane's index k in the
// rows above and below, its horizontal neighbours the other plane's index k
// and the neighbouring lane's index (a shuffle).  Cells outside the grid, and
// the region's columns beyond the halo ring, hold 0 and are never relaxed;
// guard rows above and below the region hold 0.
//
// Update: with w = omega / cnt (cnt the in-grid neighbours) the reference's
// phi += w (sum - cnt phi - b) (solver.cpp:47) is phi' = (1 - omega) phi +
// w (sum - b), since w cnt = omega; with w b kept per cell that is two FMAs
// after the neighbour sum (5 FP64 operations per cell).  Missing neighbours
// read 0, so the sum runs over the in-grid neighbours as in solver.cpp:29-44.
//
// Forms:
//   FP64 (plain): phi and b in FP64; stop tests every check_every sweeps
//     (the FP64 residual of the owned cells, or the last sweep's max |delta|)
//     with a grid barrier and partials summed in a fixed order.
//   MIXED: FP32 correction e on the FP32 right-hand side r32 = (float) r; an
//     FP32 residual estimate every check_every sweeps ends a cycle once it
//     fell by `drop` (or below 0.9 tol); the cycle's end folds e into phi in
//     FP64 inside the launch: r -= L e (FP64, e widened exactly), phi += e,
//     r32 = (float) r, e = 0, the FP64 norm of r as the stop test.
//
// Every wait is bounded: a flag or barrier wait gives up after spin_limit
// polls, records PCD_TIMEOUT in the control block and every CTA returns.
#include <algorithm>
#include <type_traits>

#include "sor_blocks.cuh"

namespace pcd {

namespace {

__device__ __forceinline__ unsigned bl_ld_acquire(const unsigned *p)
{
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void bl_st_release(unsigned *p, unsigned v)
{
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ int bl_error(const BlocksArgs &a) { return *(volatile const int *)&a.ctl->error; }

// Polls *p until it reaches target, the error word is set or the poll budget
// runs out (then PCD_TIMEOUT is recorded).  Returns 1 on success.  No sleep
// between polls: each poll is an L2 round trip already, and a sleep's wake-up
// delay would add to every exchange.
__device__ __forceinline__ int bl_poll(const unsigned *p, unsigned target, const BlocksArgs &a)
{
    long long it = 0;
    while (bl_ld_acquire(p) < target) {
        if (bl_error(a)) return 0;
        if (++it > a.spin_limit) {
            atomicCAS(&a.ctl->error, 0, PCD_TIMEOUT);
            return 0;
        }
    }
    return 1;
}

// Grid barrier number k (1-based) on the counter after the G epoch flags.
__device__ bool bl_grid_barrier(const BlocksArgs &a, unsigned k, int *s_ok)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(a.flags + a.G, 1u);
        s_ok[0] = bl_poll(a.flags + a.G, k * (unsigned)a.G, a);
    }
    __syncthreads();
    const bool ok = s_ok[0] != 0;
    __syncthreads();
    return ok;
}

// Threads 0..7 wait for the eight neighbouring blocks to reach epoch ep.
__device__ bool bl_wait_neighbours(const BlocksArgs &a, int ty, int tx, unsigned ep, int *s_ok)
{
    if (threadIdx.x < 8) {
        const int d = threadIdx.x < 4 ? (int)threadIdx.x : (int)threadIdx.x + 1;  // skip the centre
        const int ny = ty + d / 3 - 1, nx = tx + d % 3 - 1;
        int ok = 1;
        if (ny >= 0 && ny < a.TY && nx >= 0 && nx < a.TX) ok = bl_poll(a.flags + ny * a.TX + nx, ep, a);
        s_ok[threadIdx.x] = ok;
    }
    __syncthreads();
    bool ok = true;
#pragma unroll
    for (int t = 0; t < 8; t++) ok = ok && s_ok[t] != 0;
    __syncthreads();
    return ok;
}

template <typename T>
__device__ __forceinline__ T bl_fma(T a, T b, T c)
{
    return fma(a, b, c);
}
template <>
__device__ __forceinline__ float bl_fma<float>(float a, float b, float c)
{
    return fmaf(a, b, c);
}

// Per-CTA geometry and per-lane column state.
template <typename T>
struct BlockState {
    int ty, tx, y0, y1, x0, x1, oy, ox, R, RT, h;
    int k, warp;
    // lane's two cells q = 0, 1 (columns ox + 2k + q)
    bool act0, act1, own0, own1;
    int cx0, cx1;
    T wi0, wi1, we0, we1;  // weight omega / cnt: interior rows (2 row neighbours), edge rows (1)
    T *X, *BS, *BU;        // planes: state, w * rhs, rhs
    int ps;                // one colour's plane: (RTmax + 2) x 32 elements

    __device__ T *xrow(int c, int r) const { return X + (size_t)c * ps + (size_t)(r + 1) * 32; }
    __device__ T *bsrow(int c, int r) const { return BS + (size_t)c * ps + (size_t)(r + 1) * 32; }
    __device__ T *burow(int c, int r) const { return BU + (size_t)c * ps + (size_t)(r + 1) * 32; }
};

template <typename T>
__device__ __forceinline__ T weight_of(const BlocksArgs &a, int cnt)
{
    if (sizeof(T) == 8) return (T)a.w64[cnt];
    return (T)a.w32[cnt];
}

template <typename T>
__device__ void block_setup(BlockState<T> &s, const BlocksArgs &a, unsigned char *smem)
{
    const int g = blockIdx.x;
    s.ty = g / a.TX;
    s.tx = g - s.ty * a.TX;
    s.h = 2 * a.K;
    s.y0 = (int)((long long)s.ty * a.H / a.TY);
    s.y1 = (int)((long long)(s.ty + 1) * a.H / a.TY);
    const int WP = (a.W + 1) >> 1;
    s.x0 = 2 * (int)((long long)s.tx * WP / a.TX);
    s.x1 = min(a.W, 2 * (int)((long long)(s.tx + 1) * WP / a.TX));
    s.oy = s.y0 - s.h;
    s.ox = s.x0 - s.h;  // x0 and h even: colour of (ox + j, y) is (j + y) & 1
    s.R = s.y1 - s.y0;
    s.RT = s.R + 2 * s.h;
    s.k = threadIdx.x & 31;
    s.warp = threadIdx.x >> 5;
    s.ps = (a.RTmax + 2) * 32;
    s.X = reinterpret_cast<T *>(smem);
    s.BS = s.X + 2 * s.ps;
    s.BU = s.BS + 2 * s.ps;
    const int gx0 = s.ox + 2 * s.k, gx1 = gx0 + 1;
    const int bl = s.x0 - s.h, br = s.x1 + s.h;
    s.act0 = gx0 >= 0 && gx0 < a.W && gx0 >= bl && gx0 < br;
    s.act1 = gx1 >= 0 && gx1 < a.W && gx1 >= bl && gx1 < br;
    s.own0 = gx0 >= s.x0 && gx0 < s.x1;
    s.own1 = gx1 >= s.x0 && gx1 < s.x1;
    s.cx0 = (gx0 > 0) + (gx0 < a.W - 1);
    s.cx1 = (gx1 > 0) + (gx1 < a.W - 1);
    s.wi0 = weight_of<T>(a, min(4, s.cx0 + 2));
    s.wi1 = weight_of<T>(a, min(4, s.cx1 + 2));
    s.we0 = weight_of<T>(a, s.cx0 + 1);
    s.we1 = weight_of<T>(a, s.cx1 + 1);
}

// Row neighbours in the grid of row gy (2 inside, 1 on the first / last row).
__device__ __forceinline__ int row_cnt(int gy, int H) { return (gy > 0) + (gy < H - 1); }

// The cell weight of lane's cell q in a row with cy row neighbours.
template <typename T>
__device__ __forceinline__ T cell_weight(const BlockState<T> &s, int q, int cy)
{
    return q ? (cy == 2 ? s.wi1 : s.we1) : (cy == 2 ? s.wi0 : s.we0);
}

// One half sweep of colour c over region rows [lo, hi) (rows interleaved by
// warp, unrolled so that several rows' loads are in flight).  TRACK: mx takes
// max |update| over the owned cells.  FP64: phi' = (1 - omega) phi + w sum -
// w b (two FMAs); FP32: the reference's form v + w (sum - cnt v - rhs), whose
// rounding stays at the size of the update (the two-FMA form rounds at the
// size of phi twice, which at omega ~ 2 costs FP32 correction sweeps).
template <typename T, bool TRACK>
__device__ __forceinline__ void relax_half(const BlockState<T> &s, const BlocksArgs &a, int c, int lo, int hi, T omc,
                                           T &mx)
{
    lo = max(lo, -s.oy);  // grid rows only: the others hold 0 and stay 0
    hi = min(hi, a.H - s.oy);
#pragma unroll 4
    for (int r = lo + s.warp; r < hi; r += kBlocksThreads / 32) {
        const int gy = s.oy + r;
        const int q = (c + gy) & 1;
        const int cy = row_cnt(gy, a.H);
        const T w = cell_weight(s, q, cy);
        const T *O = s.xrow(1 - c, r) + s.k;
        const T up = O[-32], mid = O[0], dn = O[32];
        T nb = q ? __shfl_down_sync(0xffffffffu, mid, 1) : __shfl_up_sync(0xffffffffu, mid, 1);
        if (q ? s.k == 31 : s.k == 0) nb = T(0);
        T *V = s.xrow(c, r) + s.k;
        const T v = *V;
        const T sum = (up + dn) + (mid + nb);
        T vn;
        if (sizeof(T) == 8) {
            vn = bl_fma<T>(w, sum, bl_fma<T>(omc, v, -s.bsrow(c, r)[s.k]));
        } else {
            const T cnt = (T)((q ? s.cx1 : s.cx0) + cy);
            vn = bl_fma<T>(w, bl_fma<T>(-cnt, v, sum) - s.burow(c, r)[s.k], v);
        }
        const bool act = q ? s.act1 : s.act0;
        if (act) *V = vn;
        if (TRACK) {
            const bool own = (q ? s.own1 : s.own0) && r >= s.h && r < s.h + s.R;
            const T d = vn > v ? vn - v : v - vn;
            if (own && d > mx) mx = d;
        }
    }
}

// The residual of the lane's owned cells of region row r (both colours):
// acc += res^2, mx = max |res| with res = rhs - (sum - cnt x) in the sweep
// precision T (FP64 for the plain form's stop test; FP32 for the mixed form's
// cycle estimate, which keeps the FP64 pipe out of the FP32 kernel).
template <typename T>
__device__ __forceinline__ void residual_row(const BlockState<T> &s, const BlocksArgs &a, int r, T &acc, T &mx)
{
    const int gy = s.oy + r, cy = row_cnt(gy, a.H);
#pragma unroll
    for (int q = 0; q < 2; q++) {
        const int c = (q + gy) & 1;
        const T *O = s.xrow(1 - c, r) + s.k;
        const T mid = O[0];
        T nb = q ? __shfl_down_sync(0xffffffffu, mid, 1) : __shfl_up_sync(0xffffffffu, mid, 1);
        if (q ? s.k == 31 : s.k == 0) nb = T(0);
        const T sum = (O[-32] + O[32]) + (mid + nb);
        const T cnt = (T)((q ? s.cx1 : s.cx0) + cy);
        const T x = s.xrow(c, r)[s.k];
        const T res = s.burow(c, r)[s.k] - (sum - cnt * x);
        if (q ? s.own1 : s.own0) {
            acc += res * res;
            const T ar = res < T(0) ? -res : res;
            mx = ar > mx ? ar : mx;
        }
    }
}

// Loads the halo ring (every active, not owned cell of the region) from the
// exchange grid src (row stride xs) into the state planes, or -- rhs -- into
// the rhs planes (rhs and w * rhs).
template <typename T, bool RHS>
__device__ void load_ring(const BlockState<T> &s, const BlocksArgs &a, const T *src)
{
    for (int r = s.warp; r < s.RT; r += kBlocksThreads / 32) {
        const int gy = s.oy + r;
        if (gy < 0 || gy >= a.H) continue;
        const bool orow = r >= s.h && r < s.h + s.R;
        const int cy = row_cnt(gy, a.H);
#pragma unroll
        for (int q = 0; q < 2; q++) {
            const bool act = q ? s.act1 : s.act0, own = q ? s.own1 : s.own0;
            if (!act || (orow && own)) continue;
            const int gx = s.ox + 2 * s.k + q, c = (q + gy) & 1;
            const T v = __ldcg(src + (size_t)gy * a.xs + gx);
            if (RHS) {
                s.burow(c, r)[s.k] = v;
                s.bsrow(c, r)[s.k] = cell_weight(s, q, cy) * v;
            } else {
                s.xrow(c, r)[s.k] = v;
            }
        }
    }
}

// Owned cells of the state planes to the exchange grid dst.
template <typename T>
__device__ void publish_own(const BlockState<T> &s, const BlocksArgs &a, T *dst)
{
    for (int r = s.h + s.warp; r < s.h + s.R; r += kBlocksThreads / 32) {
        const int gy = s.oy + r;
#pragma unroll
        for (int q = 0; q < 2; q++) {
            if (!(q ? s.own1 : s.own0)) continue;
            const int gx = s.ox + 2 * s.k + q, c = (q + gy) & 1;
            dst[(size_t)gy * a.xs + gx] = s.xrow(c, r)[s.k];
        }
    }
}

template <bool MIXED>
__global__ void __launch_bounds__(kBlocksThreads, 1) k_sor_blocks(BlocksArgs a)
{
    using T = typename std::conditional<MIXED, float, double>::type;
    extern __shared__ __align__(16) unsigned char smem_b[];
    __shared__ int s_ok[8];
    __shared__ double s_dec[3];
    BlockState<T> s;
    block_setup<T>(s, a, smem_b);
    const int g = blockIdx.x;
    T *xb0 = reinterpret_cast<T *>(a.xb);
    T *xb1 = xb0 + (size_t)a.H * a.xs;

    // ---- load the region: planes zeroed, then the grid's cells
    for (int i = threadIdx.x; i < 6 * s.ps; i += blockDim.x) s.X[i] = T(0);
    __syncthreads();
    for (int r = s.warp; r < s.RT; r += kBlocksThreads / 32) {
        const int gy = s.oy + r;
        if (gy < 0 || gy >= a.H) continue;
        const int cy = row_cnt(gy, a.H);
#pragma unroll
        for (int q = 0; q < 2; q++) {
            if (!(q ? s.act1 : s.act0)) continue;
            const int gx = s.ox + 2 * s.k + q, c = (q + gy) & 1;
            const size_t i = (size_t)gy * a.ld + gx;
            T rhs;
            if (MIXED) {
                rhs = (T)a.r64[i];
            } else {
                rhs = (T)a.b[i];
                s.xrow(c, r)[s.k] = (T)a.phi[i];
            }
            s.burow(c, r)[s.k] = rhs;
            s.bsrow(c, r)[s.k] = cell_weight(s, q, cy) * rhs;
        }
    }
    __syncthreads();

    const T omc = (T)(1.0 - a.omega);
    const double bnorm = *(volatile const double *)&a.ctl->bnorm;
    const bool track = a.stop == PCD_STOP_MAX_UPDATE;
    unsigned ep = 0, checks = 0;
    int sweeps = 0, converged = 0, cyc_sweeps = 0;
    double rel = -1.0, rmax = 0.0, last_max = 0.0;
    double cyc0 = *(volatile const double *)&a.ctl->rnorm;  // FP64 residual norm at the cycle start
    T mx = T(0);
    bool ok = true;

    for (;;) {
        // ---- here the owned cells and the halo ring hold epoch ep
        const bool check = sweeps > 0 && (sweeps % a.check_every == 0 || sweeps >= a.max_iter);
        if (check) {
            double v[3] = {0.0, 0.0, 0.0};
            if (!MIXED && track) {
                v[2] = (double)mx;
            } else if (MIXED && track) {
                v[2] = (double)mx;
            } else {
                T acc = T(0), m = T(0);
                for (int r = s.h + s.warp; r < s.h + s.R; r += kBlocksThreads / 32) residual_row(s, a, r, acc, m);
                v[0] = (double)acc;
                v[2] = (double)m;
            }
            block_reduce<3, 4u>(v);
            double *part = a.part + (size_t)(checks & 1) * 3 * a.G;
            if (threadIdx.x == 0) {
                part[3 * g] = v[0];
                part[3 * g + 2] = v[2];
            }
            ++checks;
            if (!bl_grid_barrier(a, checks, s_ok)) { ok = false; break; }
            double w[3] = {0.0, 0.0, 0.0};
            // every CTA folds the partials in the same order: the same decision everywhere
            if (threadIdx.x < 32) {
                for (int t = threadIdx.x; t < a.G; t += 32) {
                    w[0] += __ldcg(part + 3 * t);
                    w[2] = fmax(w[2], __ldcg(part + 3 * t + 2));
                }
                w[0] = warp_sum(w[0]);
                w[2] = warp_max(w[2]);
                if (threadIdx.x == 0) {
                    s_dec[0] = w[0];
                    s_dec[2] = w[2];
                }
            }
            __syncthreads();
            const double ssum = s_dec[0], smax = s_dec[2];
            __syncthreads();
            bool end_cycle;
            if (!MIXED) {
                if (track) {
                    last_max = smax;
                    converged = last_max < a.tol;
                } else {
                    rel = bnorm > 0.0 ? sqrt(ssum) / bnorm : sqrt(ssum);
                    rmax = smax;
                    converged = rel <= a.tol;
                }
                if (converged || sweeps >= a.max_iter) break;
                end_cycle = false;
            } else {
                if (track) {
                    last_max = smax;
                    end_cycle = last_max < a.tol;
                } else {
                    const double est = sqrt(ssum);
                    end_cycle = est <= a.drop * cyc0 || est <= 0.9 * a.tol * (bnorm > 0.0 ? bnorm : 1.0);
                }
                end_cycle = end_cycle || sweeps >= a.max_iter || sweeps - cyc_sweeps >= a.cycle_cap;
            }
            if (MIXED && end_cycle) {
                // ---- fold e into phi in FP64: r -= L e, phi += e, r32 = (float) r
                double acc = 0.0, m = 0.0;
                for (int r = s.h + s.warp; r < s.h + s.R; r += kBlocksThreads / 32) {
                    const int gy = s.oy + r, cy = row_cnt(gy, a.H);
#pragma unroll
                    for (int q = 0; q < 2; q++) {
                        const int c = (q + gy) & 1;
                        const T *O = s.xrow(1 - c, r) + s.k;
                        const T mid = O[0];
                        T nb = q ? __shfl_down_sync(0xffffffffu, mid, 1) : __shfl_up_sync(0xffffffffu, mid, 1);
                        if (q ? s.k == 31 : s.k == 0) nb = T(0);
                        if (!(q ? s.own1 : s.own0)) continue;
                        const double sum = ((double)O[-32] + (double)O[32]) + ((double)mid + (double)nb);
                        const int cnt = (q ? s.cx1 : s.cx0) + cy;
                        const double e = (double)s.xrow(c, r)[s.k];
                        const int gx = s.ox + 2 * s.k + q;
                        const size_t i = (size_t)gy * a.ld + gx;
                        const double rn = a.r64[i] - (sum - (double)cnt * e);
                        a.r64[i] = rn;
                        a.phi[i] += e;
                        acc += rn * rn;
                        m = fmax(m, fabs(rn));
                        const T r32 = (T)rn;
                        s.burow(c, r)[s.k] = r32;
                        s.bsrow(c, r)[s.k] = cell_weight(s, q, cy) * r32;
                        a.r32x[(size_t)gy * a.xs + gx] = (float)r32;
                    }
                }
                double v2[3] = {acc, 0.0, m};
                block_reduce<3, 4u>(v2);
                double *part2 = a.part + (size_t)(checks & 1) * 3 * a.G;
                if (threadIdx.x == 0) {
                    part2[3 * g] = v2[0];
                    part2[3 * g + 2] = v2[2];
                }
                ++checks;
                if (!bl_grid_barrier(a, checks, s_ok)) { ok = false; break; }
                if (threadIdx.x < 32) {
                    double u0 = 0.0, u2 = 0.0;
                    for (int t = threadIdx.x; t < a.G; t += 32) {
                        u0 += __ldcg(part2 + 3 * t);
                        u2 = fmax(u2, __ldcg(part2 + 3 * t + 2));
                    }
                    u0 = warp_sum(u0);
                    u2 = warp_max(u2);
                    if (threadIdx.x == 0) {
                        s_dec[0] = u0;
                        s_dec[2] = u2;
                    }
                }
                __syncthreads();
                const double rn = sqrt(s_dec[0]);
                rmax = s_dec[2];
                __syncthreads();
                rel = bnorm > 0.0 ? rn / bnorm : rn;
                cyc0 = rn;
                cyc_sweeps = sweeps;
                converged = track ? (last_max < a.tol) : (rel <= a.tol);
                if (converged || sweeps >= a.max_iter) break;
                // the neighbours' new r32 (written before the barrier) and e = 0 everywhere
                load_ring<T, true>(s, a, reinterpret_cast<const T *>(a.r32x));
                for (int i = threadIdx.x; i < 2 * s.ps; i += blockDim.x) s.X[i] = T(0);
                __syncthreads();
            }
        }

        // ---- one pass: nsw sweeps, the relaxed rows shrinking with the
        // dependency cone of the owned rows
        const int nsw = min(a.K, a.max_iter - sweeps);
        mx = T(0);
        for (int t = 0; t < nsw; t++) {
            const int d = 2 * (nsw - t) - 1;
            const bool last = track && t == nsw - 1;
            if (last) relax_half<T, true>(s, a, 0, s.h - d, s.h + s.R + d, omc, mx);
            else relax_half<T, false>(s, a, 0, s.h - d, s.h + s.R + d, omc, mx);
            __syncthreads();
            if (last) relax_half<T, true>(s, a, 1, s.h - d + 1, s.h + s.R + d - 1, omc, mx);
            else relax_half<T, false>(s, a, 1, s.h - d + 1, s.h + s.R + d - 1, omc, mx);
            __syncthreads();
        }
        sweeps += nsw;

        // ---- exchange: owned cells out, epoch flag up, halo ring in
        T *dst = ((ep + 1) & 1) ? xb1 : xb0;
        publish_own(s, a, dst);
        __syncthreads();
        if (threadIdx.x == 0 && !(a.withhold && g == 0)) {
            __threadfence();
            bl_st_release(a.flags + g, ep + 1);
        }
        ++ep;
        if (!bl_wait_neighbours(a, s.ty, s.tx, ep, s_ok)) { ok = false; break; }
        load_ring<T, false>(s, a, (ep & 1) ? xb1 : xb0);
        __syncthreads();
    }

    // ---- results: the FP64 form writes its owned cells back (the mixed form
    // updated phi at every cycle's end)
    if (!MIXED) {
        for (int r = s.h + s.warp; r < s.h + s.R; r += kBlocksThreads / 32) {
            const int gy = s.oy + r;
#pragma unroll
            for (int q = 0; q < 2; q++) {
                if (!(q ? s.own1 : s.own0)) continue;
                const int gx = s.ox + 2 * s.k + q, c = (q + gy) & 1;
                a.phi[(size_t)gy * a.ld + gx] = (double)s.xrow(c, r)[s.k];
            }
        }
    }
    if (g == 0 && threadIdx.x == 0 && ok) {
        volatile Ctl *c = a.ctl;
        c->sweeps = sweeps;
        c->converged = converged;
        c->rel = rel;
        c->rmax = rmax;
        c->last_max = last_max;
        c->checks = (int)checks;
        c->halt = 1;
        c->done = 1;
    }
}

}  // namespace

int blocks_plan(int dev, int W, int H, int K, bool mixed, BlocksPlan *plan)
{
    if (K < 1 || K > 8 || W < 8 || H < 8) return PCD_BAD_ARG;
    int sms = 0, max_smem = 0, coop = 0;
    PCD_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    PCD_CUDA(cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    PCD_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
    if (!coop) return PCD_BAD_ARG;
    const int h = 2 * K;
    const int pairs_max = kBlocksRegionCols / 2 - h;  // owned column pairs of a block
    if (pairs_max < 1) return PCD_BAD_ARG;
    const int WP = (W + 1) / 2;
    const int TX = (WP + pairs_max - 1) / pairs_max;
    // blocks at least h wide and tall, so the eight neighbours cover the halo
    if (TX > 1 && (2 * (WP / TX) - 1) < h) return PCD_BAD_ARG;
    int TY = std::min(sms / TX, H / std::max(h, 1));
    if (TY < 1) return PCD_BAD_ARG;
    if (TY > 1 && H / TY < h) return PCD_BAD_ARG;
    if (TX * TY < 2) return PCD_BAD_ARG;
    const int RTmax = (H + TY - 1) / TY + 2 * h;
    const size_t elt = mixed ? sizeof(float) : sizeof(double);
    const size_t smem = (size_t)6 * (RTmax + 2) * 32 * elt;
    if (smem > (size_t)max_smem - 2048) return PCD_BAD_ARG;
    plan->TY = TY;
    plan->TX = TX;
    plan->K = K;
    plan->RTmax = RTmax;
    plan->smem = smem;
    return PCD_OK;
}

int launch_blocks(BlocksArgs &a, bool mixed, size_t smem, cudaStream_t s)
{
    void *fn = mixed ? (void *)k_sor_blocks<true> : (void *)k_sor_blocks<false>;
    PCD_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    void *params[] = {&a};
    PCD_CUDA(cudaLaunchCooperativeKernel(fn, dim3(a.G), dim3(kBlocksThreads), params, smem, s));
    count_launches(1);
    return PCD_OK;
}

}  // namespace pcd
