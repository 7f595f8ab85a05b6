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
// correction) or is below 0.9 of the stop tolerance, or at the sweep caps; the
// FP64 residual then decides convergence.
#include <algorithm>
#include <cooperative_groups.h>
#include <string>

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
    const double stop_abs = kFp32StopFrac * a.tol * bnorm;  // verify in FP64 below this
    const double drop_abs = a.drop * rstart;
    // thread -> (slot quad, row group)
    const int KH4 = P.KHp >> 2;
    const int RP = blockDim.x / KH4;
    const int k = 4 * (threadIdx.x % KH4), rg = threadIdx.x / KH4;
    cl.sync();

    int sweeps = 0;
    for (;;) {
        for (int c = 0; c < 2; c++) {
            fetch_halo_plane(cl, P, c ^ 1, g, C, n, a.H);
            __syncthreads();
            relax_quad(P, c, n, r0, G, k, rg, RP);
            cl.sync();
        }
        ++sweeps;
        const bool cap = sweeps >= a.cycle_cap || done_before + sweeps >= a.max_iter;
        if (sweeps % a.check_every == 0 || cap) {
            fetch_halo_plane(cl, P, 0, g, C, n, a.H);
            fetch_halo_plane(cl, P, 1, g, C, n, a.H);
            __syncthreads();
            double v = (double)residual_rows_quad(P.e0, P.e1, P.r0, P.r1, -(long)P.KHp, 1, n + 1, r0 - 1, G, P.KHp,
                                                  k, rg, RP);
            v = warp_sum(v);
            if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = v;
            __syncthreads();
            if (threadIdx.x == 0) {
                double t = 0.0;
                for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += s_red[w];
                s_part[0] = t;
            }
            // every CTA sums the same partials in the same order
            const double est = sqrt(cluster_sum(cl, s_part, s_red, C));
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

// ---------------------------------------------------------------------------
// Temporally blocked variant: K sweeps per halo exchange.  CTA g keeps its n
// own rows at plane rows [HK, HK + n) and HK = 2K halo rows on each side, of
// both colours of e and of r32.  Sweep t of a round relaxes red on the rows
// within d = 2(K - t) - 1 of the band and black within d - 1, recomputing the
// halo rows the neighbours own; the values are bit-identical to the owners'
// (same inputs, same arithmetic), so after K sweeps the own rows equal K
// red-black sweeps of the whole grid.  The own boundary rows are then copied
// to an export buffer of the round's parity; after one cluster barrier each
// CTA copies its neighbours' exports into its halo rows.  A CTA rewrites an
// export buffer only two rounds later, after the barrier that follows its
// neighbours' reads, so one barrier per round suffices.
template <int K>
struct TBPlanes {
    static constexpr int HK = 2 * K;
    float *e[2];    // colour planes of e, rows [0, n + 2 HK)
    float *r[2];    // colour planes of r32, same rows
    float *ex;      // exports: [parity][side: 0 top, 1 bottom][colour][HK rows][KHp]
    int KHp;
    __device__ __forceinline__ float *exp_row(int par, int side, int c, int i) const
    {
        return ex + ((size_t)(((par * 2 + side) * 2 + c) * HK + i)) * KHp;
    }
};

template <int K>
__host__ __device__ inline size_t tb_floats(int nmax, int KHp)
{
    constexpr int HK = 2 * K;
    return (size_t)4 * (nmax + 2 * HK) * KHp + (size_t)8 * HK * KHp;
}

__device__ __forceinline__ float4 lds4(unsigned a)
{
    float4 v;
    asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];" : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "r"(a));
    return v;
}
__device__ __forceinline__ float lds1(unsigned a)
{
    float v;
    asm volatile("ld.shared.f32 %0, [%1];" : "=f"(v) : "r"(a));
    return v;
}
__device__ __forceinline__ void sts4(unsigned a, const float4 &v)
{
    asm volatile("st.shared.v4.f32 [%0], {%1, %2, %3, %4};" ::"r"(a), "f"(v.x), "f"(v.y), "f"(v.z), "f"(v.w)
                 : "memory");
}

// The first / last quad of an interior row after the interior form: the
// cell at x = 0 lacks its left neighbour, the one at x = W-1 its right one
// (three neighbours, both when W = 1), cells past the last column keep v.
__device__ __forceinline__ float4 quad_edge_fix(float4 nv, const float4 &v, const float4 &rh, const float4 &up,
                                               const float4 &dn, const float4 &mid, float extra, int q, int x0,
                                               int W, float w2, float w3)
{
    const float ls[4] = {q ? extra : mid.x, q ? mid.x : mid.y, q ? mid.y : mid.z, q ? mid.z : mid.w};
    const float rs[4] = {q ? mid.x : mid.y, q ? mid.y : mid.z, q ? mid.z : mid.w, q ? mid.w : extra};
    const float us[4] = {up.x, up.y, up.z, up.w}, ds[4] = {dn.x, dn.y, dn.z, dn.w};
    const float rr[4] = {rh.x, rh.y, rh.z, rh.w}, vv[4] = {v.x, v.y, v.z, v.w};
    float out[4] = {nv.x, nv.y, nv.z, nv.w};
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const int x = x0 + 2 * j;
        if (x >= W) {
            out[j] = vv[j];
        } else if (x == 0 || x == W - 1) {
            const bool hl = x > 0, hr = x + 1 < W;
            const float sum = (us[j] + ds[j]) + ((hl ? ls[j] : 0.f) + (hr ? rs[j] : 0.f));
            const int cnt = 2 + (int)hl + (int)hr;
            out[j] = vv[j] + (cnt == 3 ? w3 : w2) * (sum - (float)cnt * vv[j] - rr[j]);
        }
    }
    return make_float4(out[0], out[1], out[2], out[3]);
}

// Colour c on plane rows [lo, hi) intersected with the thread's row block
// [rb0, rb1), walked top-down: the other colour's rows lr-1, lr, lr+1 stay in
// registers from one row to the next (one new 16-byte load of them per row),
// the neighbour one slot beyond the quad is a 4-byte load.  Any width; the
// first and last quads of a row take the edge fix-up, the grid's first and
// last rows the general form.
__device__ __forceinline__ void tb_relax_block(float *own_p, const float *oth_p, const float *rhs_p, int c, int lo,
                                               int hi, int rb0, int rb1, int ybase, const Grid &G, int KHp, int k)
{
    const int W = G.W, H = G.H;
    const float w4 = G.w4, w3 = G.w3, w2 = G.w2;
    const int l0 = max(lo, rb0), l1 = min(hi, rb1);
    // 32-bit shared-memory addresses of slot k of row 0 of each plane
    const unsigned row_bytes = 4u * (unsigned)KHp;
    const unsigned own = (unsigned)__cvta_generic_to_shared(own_p) + 4u * k;
    const unsigned oth = (unsigned)__cvta_generic_to_shared(oth_p) + 4u * k;
    const unsigned rhs = (unsigned)__cvta_generic_to_shared(rhs_p) + 4u * k;
    float4 up = make_float4(0.f, 0.f, 0.f, 0.f), mid = up, dn = up;
    if (l0 < l1) {
        up = lds4(oth + (unsigned)(l0 - 1) * row_bytes);
        mid = lds4(oth + (unsigned)l0 * row_bytes);
    }
    // parity of the first cell's column: s = (y & 1) ^ c, flips every row
    int s = ((ybase + l0) & 1) ^ c;
#pragma unroll 1
    for (int lr = l0; lr < l1; lr++, s ^= 1) {
        const unsigned ro = (unsigned)lr * row_bytes;
        dn = lds4(oth + ro + row_bytes);
        const int y = ybase + lr;
        const int q = 1 - s;
        const float extra = lds1(oth + ro + (q ? -4 : 16));
        if (y >= 0 && y < H) {
            const float4 v = lds4(own + ro);
            const float4 rh = lds4(rhs + ro);
            const int x0 = 2 * k + s;
            float4 nv;
            if (y > 0 && y < H - 1) {
                nv = quad_interior(v, rh, up, dn, mid, extra, q, w4);
                if (x0 == 0 || x0 + 7 >= W) nv = quad_edge_fix(nv, v, rh, up, dn, mid, extra, q, x0, W, w2, w3);
            } else {
                nv = quad_general(v, rh, up, dn, mid, extra, q, x0, y, W, H, G.w0, G.w1, G.w2, G.w3, w4);
            }
            sts4(own + ro, nv);
        }
        up = mid;
        mid = dn;
    }
}

// Widths that are a multiple of 8 (KHp = W / 2, no padding slots): the quad
// of cells x0, x0+2, x0+4, x0+6 with x0 = 2k + 1 - Q.  A cell without some
// neighbour (x = 0 in the first quad of a Q = 1 row, x = W-1 in the last quad
// of a Q = 0 row, every cell of the grid's first / last row) takes its own
// value in that neighbour's place, so the four-term sum minus 4v is the
// Neumann sum minus cnt v, and is scaled by omega / cnt (we for the edge
// slot, wa for the others).  Interior cells get exactly the interior form.
template <int Q>
__device__ __forceinline__ float4 quad_ghost(float4 v, const float4 &rh, const float4 &u, const float4 &d,
                                            const float4 &m, float ex, float wa, float we)
{
    const float l0 = Q ? ex : m.x, r0v = Q ? m.x : m.y;
    const float l1 = Q ? m.x : m.y, r1v = Q ? m.y : m.z;
    const float l2 = Q ? m.y : m.z, r2v = Q ? m.z : m.w;
    const float l3 = Q ? m.z : m.w, r3v = Q ? m.w : ex;
    v.x = fmaf(Q ? we : wa, fmaf(-4.f, v.x, (l0 + r0v) + (u.x + d.x)) - rh.x, v.x);
    v.y = fmaf(wa, fmaf(-4.f, v.y, (l1 + r1v) + (u.y + d.y)) - rh.y, v.y);
    v.z = fmaf(wa, fmaf(-4.f, v.z, (l2 + r2v) + (u.z + d.z)) - rh.z, v.z);
    v.w = fmaf(Q ? wa : we, fmaf(-4.f, v.w, (l3 + r3v) + (u.w + d.w)) - rh.w, v.w);
    return v;
}

struct QuadIn {
    float4 v, rh;
    float ex;
};

// Loads of one row: the own quad, its r32 and the neighbour one slot beyond
// the quad (slot k-1 for Q = 1, k+4 for Q = 0; at the row ends these fall in
// the previous / next plane row and are replaced by the ghost).
template <int Q>
__device__ __forceinline__ QuadIn quad_load(unsigned own, unsigned oth, unsigned rhs, unsigned ro)
{
    QuadIn in;
    in.ex = lds1(Q ? oth + ro - 4u : oth + ro + 16u);
    in.v = lds4(own + ro);
    in.rh = lds4(rhs + ro);
    return in;
}

template <int Q>
__device__ __forceinline__ void quad_store(unsigned own, unsigned ro, QuadIn in, const float4 &up, const float4 &mid,
                                           const float4 &dn, int y, int H, bool edge, float we4, const Grid &G)
{
    if (y < 0 || y >= H) return;  // halo rows beyond the grid
    if (edge) in.ex = Q ? in.v.x : in.v.w;
    float4 nv;
    if (y > 0 && y < H - 1) {
        nv = quad_ghost<Q>(in.v, in.rh, up, dn, mid, in.ex, G.w4, we4);
    } else {
        const bool two = H > 1;  // vertical neighbours: one, or none when H = 1
        const float wa = two ? G.w3 : G.w2, we = edge ? (two ? G.w2 : G.w1) : wa;
        nv = quad_ghost<Q>(in.v, in.rh, y > 0 ? up : in.v, y < H - 1 ? dn : in.v, mid, in.ex, wa, we);
    }
    sts4(own + ro, nv);
}

// tb_relax_block for widths that are a multiple of 8: rows in pairs (a
// Q = 1 row then a Q = 0 row, parity known at compile time), both rows'
// loads issued before either store.
__device__ __forceinline__ void tb_relax_fast(float *own_p, const float *oth_p, const float *rhs_p, int c, int lo,
                                              int hi, int rb0, int rb1, int ybase, const Grid &G, int KHp, int k)
{
    const int H = G.H;
    int lr = max(lo, rb0);
    const int l1 = min(hi, rb1);
    if (lr >= l1) return;
    const unsigned rb = 4u * (unsigned)KHp;
    const unsigned own = (unsigned)__cvta_generic_to_shared(own_p) + 4u * k;
    const unsigned oth = (unsigned)__cvta_generic_to_shared(oth_p) + 4u * k;
    const unsigned rhs = (unsigned)__cvta_generic_to_shared(rhs_p) + 4u * k;
    const bool eL = k == 0, eR = k == KHp - 4;
    const float wL = eL ? G.w3 : G.w4, wR = eR ? G.w3 : G.w4;
    float4 up = lds4(oth + (unsigned)(lr - 1) * rb), mid = lds4(oth + (unsigned)lr * rb);
    // Q = 1 - ((y & 1) ^ c)
    if (((ybase + lr) & 1) ^ c) {
        const unsigned ro = (unsigned)lr * rb;
        const float4 dn = lds4(oth + ro + rb);
        const QuadIn a = quad_load<0>(own, oth, rhs, ro);
        quad_store<0>(own, ro, a, up, mid, dn, ybase + lr, H, eR, wR, G);
        up = mid;
        mid = dn;
        lr++;
    }
#pragma unroll 1
    for (; lr + 1 < l1; lr += 2) {
        const unsigned ro = (unsigned)lr * rb;
        const float4 dn = lds4(oth + ro + rb);
        const float4 dn2 = lds4(oth + ro + 2 * rb);
        const QuadIn a = quad_load<1>(own, oth, rhs, ro);
        const QuadIn b = quad_load<0>(own, oth, rhs, ro + rb);
        quad_store<1>(own, ro, a, up, mid, dn, ybase + lr, H, eL, wL, G);
        quad_store<0>(own, ro + rb, b, mid, dn, dn2, ybase + lr + 1, H, eR, wR, G);
        up = dn;
        mid = dn2;
    }
    if (lr < l1) {
        const unsigned ro = (unsigned)lr * rb;
        const float4 dn = lds4(oth + ro + rb);
        const QuadIn a = quad_load<1>(own, oth, rhs, ro);
        quad_store<1>(own, ro, a, up, mid, dn, ybase + lr, H, eL, wL, G);
    }
}

template <int K>
__global__ void __launch_bounds__(kClusterThreads, 1) k_sor_cluster_tb(ClusterArgs a)
{
    constexpr int HK = 2 * K;
    cg::cluster_group cl = cg::this_cluster();
    extern __shared__ __align__(16) float smem_f[];
    __shared__ double s_part[1];
    __shared__ double s_red[32];
    const int C = (int)cl.num_blocks(), g = (int)cl.block_rank(), W = a.W, H = a.H;
    int r0, n;
    band_of(g, C, H, r0, n);
    const int nmax = (H + C - 1) / C;
    const int KHp = a.khp;
    const int rows = nmax + 2 * HK;
    TBPlanes<K> P;
    P.KHp = KHp;
    P.e[0] = smem_f;
    P.e[1] = smem_f + (size_t)rows * KHp;
    P.r[0] = smem_f + (size_t)2 * rows * KHp;
    P.r[1] = smem_f + (size_t)3 * rows * KHp;
    P.ex = smem_f + (size_t)4 * rows * KHp;
    Grid G;
    G.W = W; G.H = H;
    G.w0 = a.w32[0]; G.w1 = a.w32[1]; G.w2 = a.w32[2]; G.w3 = a.w32[3]; G.w4 = a.w32[4];

    const Ctl *ctl = a.ctl;
    if (*(volatile const int *)&ctl->done) return;  // speculative launch after convergence: all CTAs agree
    const int ybase = r0 - HK;  // grid row of plane row 0
    // own and halo rows of e and r32 from global memory (zero outside the grid)
    for (int t = threadIdx.x; t < (n + 2 * HK) * KHp * 2; t += blockDim.x) {
        const int lr = t / (2 * KHp), x = t - lr * 2 * KHp, y = ybase + lr;
        const int c = (x + y) & 1;
        float ev = 0.f, rv = 0.f;
        if (y >= 0 && y < H && x < W) {
            const size_t gi = (size_t)y * a.ld + x;
            ev = a.e[gi];
            rv = a.r32[gi];
        }
        (c ? P.e[1] : P.e[0])[(size_t)lr * KHp + (x >> 1)] = ev;
        (c ? P.r[1] : P.r[0])[(size_t)lr * KHp + (x >> 1)] = rv;
    }
    const int done_before = *(volatile const int *)&ctl->sweeps;
    const double bnorm = *(volatile const double *)&ctl->bnorm;
    const double rstart = *(volatile const double *)&ctl->rnorm;
    const double stop_abs = kFp32StopFrac * a.tol * bnorm;
    const double drop_abs = a.drop * rstart;
    const int KH4 = KHp >> 2;
    const int RP = blockDim.x / KH4;
    const int k = 4 * (threadIdx.x % KH4), rg = threadIdx.x / KH4;
    const int K4 = KHp >> 2;
    // contiguous row blocks over the relaxed span [1, n + 2 HK - 1); warps
    // within one row group when a row group is a whole number of warps
    const int span = n + 2 * HK - 2, L = (span + RP - 1) / RP;
    const int rb0 = rg < RP ? 1 + rg * L : 0, rb1 = rg < RP ? min(rb0 + L, n + 2 * HK - 1) : 0;
    const bool fast = (W & 7) == 0;  // KHp = W / 2: the ghost-cell row form
    __syncthreads();

    int sweeps = 0, par = 0, next_check = a.check_every;
    for (;;) {
        // kr <= K sweeps on the band and its halo (fewer at the sweep caps)
        const int kr = min(K, min(a.cycle_cap - sweeps, a.max_iter - done_before - sweeps));
        for (int t = 0; t < kr; t++) {
            const int d = 2 * (kr - t) - 1;
            if (fast) {
                tb_relax_fast(P.e[0], P.e[1], P.r[0], 0, HK - d, HK + n + d, rb0, rb1, ybase, G, KHp, k);
                __syncthreads();
                tb_relax_fast(P.e[1], P.e[0], P.r[1], 1, HK - d + 1, HK + n + d - 1, rb0, rb1, ybase, G, KHp, k);
            } else {
                tb_relax_block(P.e[0], P.e[1], P.r[0], 0, HK - d, HK + n + d, rb0, rb1, ybase, G, KHp, k);
                __syncthreads();
                tb_relax_block(P.e[1], P.e[0], P.r[1], 1, HK - d + 1, HK + n + d - 1, rb0, rb1, ybase, G, KHp, k);
            }
            __syncthreads();
        }
        sweeps += kr;
        // export the own boundary rows, one barrier, import the neighbours'
        for (int i = threadIdx.x; i < 2 * 2 * HK * K4; i += blockDim.x) {
            const int q4 = i % K4, rest = i / K4, row = rest % HK, cs = rest / HK, c = cs & 1, side = cs >> 1;
            const int lr = side == 0 ? HK + row : n + row;
            reinterpret_cast<float4 *>(P.exp_row(par, side, c, row))[q4] =
                reinterpret_cast<const float4 *>((c ? P.e[1] : P.e[0]) + (size_t)lr * KHp)[q4];
        }
        cl.sync();
        for (int i = threadIdx.x; i < 2 * 2 * HK * K4; i += blockDim.x) {
            const int q4 = i % K4, rest = i / K4, row = rest % HK, cs = rest / HK, c = cs & 1, side = cs >> 1;
            // side 0: my top halo <- upper neighbour's bottom export; side 1: my bottom halo <- lower neighbour's top
            const int nb = side == 0 ? g - 1 : g + 1;
            if (nb < 0 || nb >= C) continue;
            const float *src = cl.map_shared_rank(P.exp_row(par, side ^ 1, c, row), nb);
            const int lr = side == 0 ? row : HK + n + row;
            reinterpret_cast<float4 *>((c ? P.e[1] : P.e[0]) + (size_t)lr * KHp)[q4] =
                reinterpret_cast<const float4 *>(src)[q4];
        }
        par ^= 1;
        __syncthreads();
        const bool cap = sweeps >= a.cycle_cap || done_before + sweeps >= a.max_iter;
        if (sweeps >= next_check || cap) {
            next_check = sweeps + a.check_every;
            double v = (double)residual_rows_quad(P.e[0], P.e[1], P.r[0], P.r[1], 0, HK, HK + n, ybase, G, KHp, k,
                                                  rg, RP);
            v = warp_sum(v);
            if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = v;
            __syncthreads();
            if (threadIdx.x == 0) {
                double tt = 0.0;
                for (int w = 0; w < (int)(blockDim.x >> 5); w++) tt += s_red[w];
                s_part[0] = tt;
            }
            const double est = sqrt(cluster_sum(cl, s_part, s_red, C));
            if (cap || est <= stop_abs || est <= drop_abs) break;
        }
    }
    for (int t = threadIdx.x; t < n * W; t += blockDim.x) {
        const int row = t / W, x = t - row * W, y = r0 + row;
        a.e[(size_t)y * a.ld + x] = (((x + y) & 1) ? P.e[1] : P.e[0])[(size_t)(row + HK) * KHp + (x >> 1)];
    }
    if (g == 0 && threadIdx.x == 0) {
        volatile Ctl *cc = a.ctl;
        cc->sweeps = done_before + sweeps;
        if (done_before + sweeps >= a.max_iter) cc->halt = 1;
    }
    cl.sync();
}

#include "sor_cluster_rr.cuh"
#include "sor_tile_rr.cuh"

template <int K, bool TRACK>
const void *tile_kernel_k(int L, int NQ)
{
    if (L == 3 && NQ == 2) return (const void *)k_sor_tile_rr<K, 3, 2, TRACK>;
    if (L == 4 && NQ == 1) return (const void *)k_sor_tile_rr<K, 4, 1, TRACK>;
    return nullptr;
}

// The tile pass for K sweeps, L rows per warp and NQ quads per lane (nullptr
// outside the compiled set).
const void *tile_kernel(int K, int L, int NQ, bool track)
{
    if (K == 4) return track ? tile_kernel_k<4, true>(L, NQ) : tile_kernel_k<4, false>(L, NQ);
    if (K == 2) return track ? tile_kernel_k<2, true>(L, NQ) : tile_kernel_k<2, false>(L, NQ);
    return nullptr;
}

}  // namespace

namespace {

bool cluster_fits(const void *fn, int C, int threads, size_t smem)
{
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess ||
        cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(C);
    cfg.blockDim = dim3(threads);
    cfg.dynamicSmemBytes = smem;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int nclusters = 0;
    if (cudaOccupancyMaxActiveClusters(&nclusters, fn, &cfg) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return nclusters >= 1;
}

// Register-resident form: W a multiple of 8 up to 512, the band at least HK
// rows, L = ceil((nmax + 2 HK) / 16) rows per warp in 2..4.
bool rr_plan(int W, int H, int max_depth, int max_smem, ClusterPlan &p)
{
    if (W % 8 != 0 || W > 512 || max_depth < 2) return false;
    const int KQ = W / 8, NQ = KQ <= 32 ? 1 : 2;
    for (int C : {16, 8}) {
        if (H < 2 * C) continue;
        const int nmax = (H + C - 1) / C, nmin = H / C;
        for (int K : {4, 2}) {
            if (K > max_depth) continue;
            const int HK = 2 * K, R = nmax + 2 * HK;
            if (nmin < HK) continue;
            const int L = std::max(2, (R + kRRWarps - 1) / kRRWarps);
            const void *fn = rr_kernel(K, L, NQ);
            if (!fn) continue;
            const size_t smem = rr_floats(K, NQ, R) * sizeof(float);
            if (smem + 2048 > (size_t)max_smem) continue;
            if (!cluster_fits(fn, C, kRRThreads, smem)) continue;
            p.C = C;
            p.smem = smem;
            p.khp = ((W + 1) / 2 + 3) / 4 * 4;
            p.depth = K;
            p.rr_l = L;
            p.rr_nq = NQ;
            return true;
        }
    }
    return false;
}

}  // namespace

int cluster_plan(int dev, int W, int H, int max_depth, ClusterPlan *plan)
{
    int max_smem = 0, cluster_ok = 0;
    PCD_CUDA(cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    PCD_CUDA(cudaDeviceGetAttribute(&cluster_ok, cudaDevAttrClusterLaunch, dev));
    if (!cluster_ok) return PCD_BAD_ARG;
    ClusterPlan p{};
    if (rr_plan(W, H, max_depth, max_smem, p)) {
        *plan = p;
        return PCD_OK;
    }
    const int khp = ((W + 1) / 2 + 3) / 4 * 4;
    if (khp / 2 > kClusterThreads) return PCD_BAD_ARG;
    for (int C : {16, 8}) {
        if (H < 2 * C) continue;
        const int nmax = (H + C - 1) / C, nmin = H / C;
        // deepest blocking that fits, then the per-half-sweep exchange
        for (int depth = std::min(max_depth, 2); depth >= 0; depth--) {
            size_t smem;
            const void *fn;
            if (depth == 0) {
                smem = (size_t)(2 * (nmax + 2) + 2 * nmax) * khp * sizeof(float);
                fn = (const void *)k_sor_cluster;
            } else {
                if (nmin < 2 * depth) continue;
                smem = (depth == 2 ? tb_floats<2>(nmax, khp) : tb_floats<1>(nmax, khp)) * sizeof(float);
                fn = depth == 2 ? (const void *)k_sor_cluster_tb<2> : (const void *)k_sor_cluster_tb<1>;
            }
            if (smem + 2048 > (size_t)max_smem) continue;
            if (!cluster_fits(fn, C, kClusterThreads, smem)) continue;
            p.C = C;
            p.smem = smem;
            p.khp = khp;
            p.depth = depth;
            *plan = p;
            return PCD_OK;
        }
    }
    return PCD_BAD_ARG;
}

int tile_plan(int dev, int W, int H, int ld, int depth, TilePlan *plan)
{
    if (W < 8 || H < 1 || W % 8 != 0 || ld % 4 != 0) return PCD_BAD_ARG;
    if (depth != 0 && depth != 2 && depth != 4) return PCD_BAD_ARG;
    const int K = depth ? depth : 4;
    int sms = 0, max_smem = 0;
    PCD_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    PCD_CUDA(cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    const int WQ = W / 8;
    TilePlan best{};
    long best_cost = 0;
    // tiles of 16 L rows and 256 NQ columns; a tile costs about L NQ quad
    // updates per thread and half sweep whatever its interior
    const int forms[2][2] = {{3, 2}, {4, 1}};
    for (const auto &f : forms) {
        const int L = f[0], NQ = f[1];
        const int N = kRRWarps * L - 4 * K;
        if (N < 1) continue;
        const int ncol = ceil_div(WQ, 32 * NQ - 2), nrow = ceil_div(H, N);
        const long cost = (long)ncol * nrow * L * NQ;
        if (best.K && cost >= best_cost) continue;
        const size_t smem = tile_floats(L, NQ) * sizeof(float);
        if (smem + 2048 > (size_t)max_smem) continue;
        int bps = 1;
        for (int tr = 0; tr < 2; tr++) {
            const void *fn = tile_kernel(K, L, NQ, tr != 0);
            if (!fn) {
                bps = 0;
                break;
            }
            int b = 0;
            PCD_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            PCD_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, fn, kRRThreads, smem));
            bps = std::min(bps, b);
        }
        if (bps < 1) continue;
        best.K = K;
        best.L = L;
        best.NQ = NQ;
        best.ncol = ncol;
        best.nrow = nrow;
        best.grid = (int)std::min<long>((long)ncol * nrow, (long)sms * bps);
        best.smem = smem;
        best_cost = cost;
    }
    if (!best.K) return PCD_BAD_ARG;
    *plan = best;
    return PCD_OK;
}

int launch_tile(const TilePlan &p, const float *ein, float *eout, const float *r32, Ctl *ctl, const SolveArgs &a,
                int nsw, int out_idx, bool track, cudaStream_t s)
{
    const void *fn = tile_kernel(p.K, p.L, p.NQ, track);
    if (!fn || nsw < 1 || nsw > p.K) {
        set_error("tile SOR: no kernel for this plan");
        return PCD_BAD_ARG;
    }
    using Fn = void (*)(const float *, float *, const float *, Ctl *, SolveArgs, int, int, int, int);
    reinterpret_cast<Fn>(const_cast<void *>(fn))<<<p.grid, kRRThreads, p.smem, s>>>(ein, eout, r32, ctl, a, p.ncol,
                                                                                    p.nrow, nsw, out_idx);
    return PCD_OK;
}

void tile_counts(int W, int H, int *ncol, int *nrow)
{
    constexpr int L = 4, NQ = 1, K = 4;
    *ncol = ceil_div(W / 8, 32 * NQ - 2);
    *nrow = ceil_div(H, kRRWarps * L - 4 * K);
}

int tile_batch_config(int dev, int njobs, size_t *smem, int *grid)
{
    if (njobs < 1 || njobs > kTileBatchJobsMax) {
        set_error("batched tile pass: 1 to " + std::to_string(kTileBatchJobsMax) + " grids");
        return PCD_BAD_ARG;
    }
    const void *fn = (const void *)k_sor_tile_batch<4, 4, 1>;
    const size_t base = tile_floats(4, 1) * sizeof(float), per_job = sizeof(TileJob) + sizeof(int);
    const size_t most = base + kTileBatchJobsMax * per_job, bytes = base + (size_t)njobs * per_job;
    int sms = 0, bps = 0;
    PCD_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    PCD_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)most));
    PCD_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, fn, kRRThreads, bytes));
    if (bps < 1) {
        set_error("batched tile pass: the kernel does not fit on an SM");
        return PCD_BAD_ARG;
    }
    *smem = bytes;
    *grid = sms * bps;
    return PCD_OK;
}

int launch_tile_batch(const TileJob *d_jobs, int njobs, int ntiles, int nsw, int par, int grid, size_t smem,
                      unsigned *counter, cudaStream_t s)
{
    if (njobs < 1 || njobs > kTileBatchJobsMax || ntiles < 1 || nsw < 1 || nsw > 4) {
        set_error("batched tile pass: bad arguments");
        return PCD_BAD_ARG;
    }
    k_sor_tile_batch<4, 4, 1>
        <<<std::min(grid, ntiles), kRRThreads, smem, s>>>(d_jobs, njobs, ntiles, nsw, par, counter);
    return PCD_OK;
}

int launch_cluster(ClusterArgs &a, const ClusterPlan &p, cudaStream_t s)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(p.C);
    cfg.blockDim = dim3(p.rr_l ? kRRThreads : kClusterThreads);
    cfg.dynamicSmemBytes = p.smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = p.C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    a.depth = p.depth;
    if (p.rr_l) {
        const void *fn = rr_kernel(p.depth, p.rr_l, p.rr_nq);
        if (!fn) {
            set_error("cluster SOR: no register-resident kernel for this plan");
            return PCD_BAD_ARG;
        }
        PCD_CUDA(cudaLaunchKernelEx(&cfg, reinterpret_cast<void (*)(ClusterArgs)>(const_cast<void *>(fn)), a));
    } else if (p.depth == 2) {
        PCD_CUDA(cudaLaunchKernelEx(&cfg, k_sor_cluster_tb<2>, a));
    } else if (p.depth == 1) {
        PCD_CUDA(cudaLaunchKernelEx(&cfg, k_sor_cluster_tb<1>, a));
    } else {
        PCD_CUDA(cudaLaunchKernelEx(&cfg, k_sor_cluster, a));
    }
    count_launches(1);
    return PCD_OK;
}

}  // namespace pcd
