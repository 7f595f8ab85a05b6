// sor_planes.cuh -- FP32 red-black SOR on colour planes split across the
// CTAs of one thread-block cluster (internal; used by sor_cluster.cu and
// sor_batch.cu).
//
// CTA g of a C-CTA cluster owns grid rows [r0, r0+n) (band_of).  Its state is
// four FP32 planes with row stride KHp (even, >= ceil(W/2), multiple of 4):
//   e0 / e1 : red / black cells of the correction e, rows 0..n+1 (0 and n+1
//             are halo copies of the neighbouring CTAs' facing rows)
//   r0 / r1 : red / black cells of the right-hand side r32, rows 0..n-1
// Cell (x, y) of colour c = (x+y)&1 lives at e_c[(y - r0 + 1)*KHp + (x >> 1)].
// In row y (p = y&1) the cell of colour c at slot k sits at x = 2k + (p^c); its
// left / right neighbours (other colour) sit at slots k - q and k - q + 1 with
// q = 1 - (p^c); its up / down neighbours at slot k of rows y-1, y+1.
//
// The planes live either in the CTA's shared memory (neighbours reached
// through DSMEM) or in an L2-resident global scratch region laid out the same
// way per CTA (neighbours read with ld.global.cg, ordered by the cluster
// barrier's release/acquire).
#pragma once

#include <cooperative_groups.h>

#include "common.cuh"

namespace pcd {
namespace planes {

namespace cg = cooperative_groups;

__device__ __forceinline__ void band_of(int g, int G, int H, int &r0, int &n)
{
    const int base = H / G, extra = H % G;
    n = base + (g < extra ? 1 : 0);
    r0 = g * base + (g < extra ? g : extra);
}

// Relaxation factors and grid size of one solve.
struct Grid {
    int W, H;
    float w0, w1, w2, w3, w4;  // omega / cnt
};

struct Planes {
    float *e0, *e1;  // red, black planes of e
    float *r0, *r1;  // red, black planes of r32
    int KHp;
    int in_smem;     // 1: shared memory; 0: global scratch
    long cta_stride; // global scratch: floats between consecutive CTAs' regions
    __device__ __forceinline__ float *e(int c) const { return c ? e1 : e0; }
    __device__ __forceinline__ float *r(int c) const { return c ? r1 : r0; }
};

__host__ __device__ inline int plane_stride(int W) { return ((W + 1) / 2 + 3) / 4 * 4; }

// floats of one CTA's four planes for bands of at most nmax rows
__host__ __device__ inline long planes_floats(int nmax, int KHp) { return (long)(2 * (nmax + 2) + 2 * nmax) * KHp; }

__device__ __forceinline__ void carve(Planes &P, float *base, int nmax)
{
    const long plane = (long)(nmax + 2) * P.KHp, rplane = (long)nmax * P.KHp;
    P.e0 = base;
    P.e1 = base + plane;
    P.r0 = base + 2 * plane;
    P.r1 = base + 2 * plane + rplane;
}

// Copy the neighbours' facing rows of plane c into its halo rows.
__device__ __forceinline__ void fetch_halo_plane(cg::cluster_group &cl, const Planes &P, int c, int g, int C, int n,
                                                 int H)
{
    float *pl = P.e(c);
    const int KHp = P.KHp, K4 = KHp >> 2;
    if (g > 0) {
        int pr0, pn;
        band_of(g - 1, C, H, pr0, pn);
        const float *nb = P.in_smem ? cl.map_shared_rank(pl, g - 1) : pl - P.cta_stride;
        const float4 *src = reinterpret_cast<const float4 *>(nb + (size_t)pn * KHp);
        float4 *dst = reinterpret_cast<float4 *>(pl);
        if (P.in_smem)
            for (int i = threadIdx.x; i < K4; i += blockDim.x) dst[i] = src[i];
        else
            for (int i = threadIdx.x; i < K4; i += blockDim.x) dst[i] = __ldcg(src + i);
    }
    if (g < C - 1) {
        const float *nb = P.in_smem ? cl.map_shared_rank(pl, g + 1) : pl + P.cta_stride;
        const float4 *src = reinterpret_cast<const float4 *>(nb + (size_t)KHp);
        float4 *dst = reinterpret_cast<float4 *>(pl + (size_t)(n + 1) * KHp);
        if (P.in_smem)
            for (int i = threadIdx.x; i < K4; i += blockDim.x) dst[i] = src[i];
        else
            for (int i = threadIdx.x; i < K4; i += blockDim.x) dst[i] = __ldcg(src + i);
    }
}

// One half sweep of colour c over the band: each thread owns slot pair
// (k, k+1) of rows lr = 1 + rg, 1 + rg + RP, ...
__device__ __forceinline__ void relax_pair(const Planes &P, int c, int n, int r0, const Grid &G, int k, int rg, int RP)
{
    const int W = G.W, H = G.H, KHp = P.KHp;
    float *__restrict__ own = P.e(c);
    const float *__restrict__ oth = P.e(c ^ 1);
    const float *__restrict__ rhs = P.r(c);
    const float w1 = G.w1, w2 = G.w2, w3 = G.w3, w4 = G.w4;
#pragma unroll 2
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
        const int x0 = 2 * k + s, x1 = x0 + 2;
        if (y > 0 && y < H - 1 && x0 > 0 && x1 + 1 < W) {
            // interior pair: four neighbours each; the reference's form
            // v + w (sum - 4 v - r) forms the small correction first, which
            // keeps FP32 rounding at the level of the change
            float s0, s1;
            if (q) { s0 = extra + mid.x; s1 = mid.x + mid.y; }
            else { s0 = mid.x + mid.y; s1 = mid.y + extra; }
            s0 += up.x + dn.x;
            s1 += up.y + dn.y;
            v.x = fmaf(w4, fmaf(-4.f, v.x, s0) - rh.x, v.x);
            v.y = fmaf(w4, fmaf(-4.f, v.y, s1) - rh.y, v.y);
        } else {
            const float l0 = q ? extra : mid.x, r0v = q ? mid.x : mid.y;
            const float l1 = q ? mid.x : mid.y, r1v = q ? mid.y : extra;
            const bool hu = y > 0, hd = y < H - 1;
            const float vert0 = (hu ? up.x : 0.f) + (hd ? dn.x : 0.f);
            const float vert1 = (hu ? up.y : 0.f) + (hd ? dn.y : 0.f);
            const int cv = (int)hu + (int)hd;
            if (x0 < W) {
                const bool hl = x0 > 0, hr = x0 + 1 < W;
                const float sum = vert0 + (hl ? l0 : 0.f) + (hr ? r0v : 0.f);
                const int cnt = cv + (int)hl + (int)hr;
                const float w = cnt == 4 ? w4 : cnt == 3 ? w3 : cnt == 2 ? w2 : cnt == 1 ? w1 : G.w0;
                v.x = v.x + w * (sum - (float)cnt * v.x - rh.x);
            }
            if (x1 < W) {
                const bool hr = x1 + 1 < W;  // x1 >= 2 always has a left neighbour
                const float sum = vert1 + l1 + (hr ? r1v : 0.f);
                const int cnt = cv + 1 + (int)hr;
                const float w = cnt == 4 ? w4 : cnt == 3 ? w3 : cnt == 2 ? w2 : w1;
                v.y = v.y + w * (sum - (float)cnt * v.y - rh.y);
            }
        }
        *reinterpret_cast<float2 *>(own + ro + k) = v;
    }
}

// Four cells of colour c at slots k..k+3 of one plane row (x0 = 2k + s is
// the column of the first).  `extra` is the neighbour one slot beyond the
// quad: left of its first cell when q = 1, right of its last when q = 0.
// Interior form: every cell has four neighbours.
__device__ __forceinline__ float4 quad_interior(float4 v, const float4 &rh, const float4 &up, const float4 &dn,
                                               const float4 &mid, float extra, int q, float w4)
{
    const float l0 = q ? extra : mid.x, r0v = q ? mid.x : mid.y;
    const float l1 = q ? mid.x : mid.y, r1v = q ? mid.y : mid.z;
    const float l2 = q ? mid.y : mid.z, r2v = q ? mid.z : mid.w;
    const float l3 = q ? mid.z : mid.w, r3v = q ? mid.w : extra;
    v.x = fmaf(w4, fmaf(-4.f, v.x, (l0 + r0v) + (up.x + dn.x)) - rh.x, v.x);
    v.y = fmaf(w4, fmaf(-4.f, v.y, (l1 + r1v) + (up.y + dn.y)) - rh.y, v.y);
    v.z = fmaf(w4, fmaf(-4.f, v.z, (l2 + r2v) + (up.z + dn.z)) - rh.z, v.z);
    v.w = fmaf(w4, fmaf(-4.f, v.w, (l3 + r3v) + (up.w + dn.w)) - rh.w, v.w);
    return v;
}

// General form (cells without some neighbour, cells past the last column
// left unchanged): v + omega/cnt * (sum over existing neighbours - cnt v - r).
static __device__ __noinline__ float4 quad_general(float4 v, float4 rh, float4 up, float4 dn, float4 mid, float extra, int q,
                                            int x0, int y, int W, int H, float w0, float w1, float w2, float w3,
                                            float w4)
{
    const float ls[4] = {q ? extra : mid.x, q ? mid.x : mid.y, q ? mid.y : mid.z, q ? mid.z : mid.w};
    const float rs[4] = {q ? mid.x : mid.y, q ? mid.y : mid.z, q ? mid.z : mid.w, q ? mid.w : extra};
    const float us[4] = {up.x, up.y, up.z, up.w}, ds[4] = {dn.x, dn.y, dn.z, dn.w};
    const float rr[4] = {rh.x, rh.y, rh.z, rh.w};
    float vv[4] = {v.x, v.y, v.z, v.w};
    const bool hu = y > 0, hd = y < H - 1;
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const int x = x0 + 2 * j;
        if (x >= W) continue;
        const bool hl = x > 0, hr = x + 1 < W;
        const float sum = ((hu ? us[j] : 0.f) + (hd ? ds[j] : 0.f)) + ((hl ? ls[j] : 0.f) + (hr ? rs[j] : 0.f));
        const int cnt = (int)hu + (int)hd + (int)hl + (int)hr;
        const float w = cnt == 4 ? w4 : cnt == 3 ? w3 : cnt == 2 ? w2 : cnt == 1 ? w1 : w0;
        vv[j] = vv[j] + w * (sum - (float)cnt * vv[j] - rr[j]);
    }
    return make_float4(vv[0], vv[1], vv[2], vv[3]);
}

// Four cells of an interior row (up and down neighbours exist) in the first
// or last quad of the row: a cell at x = 0 has no left neighbour, one at
// x = W-1 no right neighbour, cells at x >= W stay unchanged.
__device__ __forceinline__ float4 quad_row_edge(float4 v, const float4 &rh, const float4 &up, const float4 &dn,
                                               const float4 &mid, float extra, int q, int x0, int W, float w2,
                                               float w3, float w4)
{
    const float ls[4] = {q ? extra : mid.x, q ? mid.x : mid.y, q ? mid.y : mid.z, q ? mid.z : mid.w};
    const float rs[4] = {q ? mid.x : mid.y, q ? mid.y : mid.z, q ? mid.z : mid.w, q ? mid.w : extra};
    const float us[4] = {up.x, up.y, up.z, up.w}, ds[4] = {dn.x, dn.y, dn.z, dn.w};
    const float rr[4] = {rh.x, rh.y, rh.z, rh.w};
    float vv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const int x = x0 + 2 * j;
        const bool hl = x > 0, hr = x + 1 < W;
        const float sum = (us[j] + ds[j]) + ((hl ? ls[j] : 0.f) + (hr ? rs[j] : 0.f));
        const int cnt = 2 + (int)hl + (int)hr;
        const float w = cnt == 4 ? w4 : (cnt == 3 ? w3 : w2);
        const float nv = vv[j] + w * (sum - (float)cnt * vv[j] - rr[j]);
        vv[j] = x < W ? nv : vv[j];
    }
    return make_float4(vv[0], vv[1], vv[2], vv[3]);
}

// One half sweep of colour c over plane rows [lo, hi) with four slots per
// thread: slots k..k+3 (k a multiple of 4); row group rg walks the rows
// [lo + rg L, lo + rg L + L) top-down (grid row y = ybase + lr; rows outside
// the grid are skipped; threads with rg >= RP idle), keeping the other
// colour's rows lr-1, lr, lr+1 in registers from one row to the next (one
// new 16-byte load of them per row), which matters where the planes live in
// L2.  rhs row lr sits at rhs + lr * KHp + roff.  In rows other than the
// grid's first and last only the first quad (x0 = 0) and the last quad
// (x0 + 7 >= W) have cells without four neighbours: they take the short edge
// form, the first and last grid rows the general form.  Reads of slot k-1
// at k = 0 and of slot KHp at k = KHp-4 fall in the previous / next plane
// row (both exist) and are used only for cells without that neighbour.
__device__ __forceinline__ void relax_block_quad(float *__restrict__ own, const float *__restrict__ oth,
                                                 const float *__restrict__ rhs, long roff, int c, int lo, int hi,
                                                 int ybase, const Grid &G, int KHp, int k, int rg, int RP)
{
    const int W = G.W, H = G.H;
    const float w4 = G.w4;
    if (rg >= RP) return;
    const int L = (hi - lo + RP - 1) / RP;
    const int b0 = lo + rg * L, b1 = min(b0 + L, hi);
    if (b0 >= b1) return;
    float4 up = *reinterpret_cast<const float4 *>(oth + (size_t)(b0 - 1) * KHp + k);
    float4 mid = *reinterpret_cast<const float4 *>(oth + (size_t)b0 * KHp + k);
#pragma unroll 1
    for (int lr = b0; lr < b1; lr++) {
        const size_t ro = (size_t)lr * KHp;
        const float4 dn = *reinterpret_cast<const float4 *>(oth + ro + KHp + k);
        const int y = ybase + lr;
        if (y >= 0 && y < H) {
            const int s = (y & 1) ^ c;
            const int q = 1 - s;
            const int x0 = 2 * k + s;
            const float4 v = *reinterpret_cast<const float4 *>(own + ro + k);
            const float4 rh = *reinterpret_cast<const float4 *>(rhs + ro + roff + k);
            const float extra = oth[ro + (q ? k - 1 : k + 4)];
            float4 nv;
            if (y > 0 && y < H - 1) {
                if (x0 > 0 && x0 + 7 < W) nv = quad_interior(v, rh, up, dn, mid, extra, q, w4);
                else nv = quad_row_edge(v, rh, up, dn, mid, extra, q, x0, W, G.w2, G.w3, w4);
            } else {
                nv = quad_general(v, rh, up, dn, mid, extra, q, x0, y, W, H, G.w0, G.w1, G.w2, G.w3, w4);
            }
            *reinterpret_cast<float4 *>(own + ro + k) = nv;
        }
        up = mid;
        mid = dn;
    }
}

// Sum of squares of r - L e over the four cells of a quad (cells past the
// last column excluded), branch free.
__device__ __forceinline__ float quad_residual_sq(const float4 &v, const float4 &rh, const float4 &up,
                                                  const float4 &dn, const float4 &mid, float extra, int q, int x0,
                                                  int y, int W, int H)
{
    const float ls[4] = {q ? extra : mid.x, q ? mid.x : mid.y, q ? mid.y : mid.z, q ? mid.z : mid.w};
    const float rs[4] = {q ? mid.x : mid.y, q ? mid.y : mid.z, q ? mid.z : mid.w, q ? mid.w : extra};
    const float us[4] = {up.x, up.y, up.z, up.w}, ds[4] = {dn.x, dn.y, dn.z, dn.w};
    const float rr[4] = {rh.x, rh.y, rh.z, rh.w}, vv[4] = {v.x, v.y, v.z, v.w};
    const bool hu = y > 0, hd = y < H - 1;
    float acc = 0.f;
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const int x = x0 + 2 * j;
        const bool hl = x > 0, hr = x + 1 < W;
        const float sum = ((hu ? us[j] : 0.f) + (hd ? ds[j] : 0.f)) + ((hl ? ls[j] : 0.f) + (hr ? rs[j] : 0.f));
        const int cnt = (int)hu + (int)hd + (int)hl + (int)hr;
        const float r = rr[j] - (sum - (float)cnt * vv[j]);
        acc = x < W ? fmaf(r, r, acc) : acc;
    }
    return acc;
}

// Sum over plane rows [lo, hi) (grid row ybase + lr), both colours, of
// (r - L e)^2 in FP32 per thread; the same slot mapping as relax_block_quad
// with the rows taken round-robin over the row groups.
__device__ __forceinline__ float residual_rows_quad(const float *__restrict__ e0, const float *__restrict__ e1,
                                                   const float *__restrict__ r0p, const float *__restrict__ r1p,
                                                   long roff, int lo, int hi, int ybase, const Grid &G, int KHp,
                                                   int k, int rg, int RP)
{
    float acc = 0.f;
    if (rg >= RP) return acc;
    for (int lr = lo + rg; lr < hi; lr += RP) {
        const int y = ybase + lr;
        if (y < 0 || y >= G.H) continue;
        const size_t ro = (size_t)lr * KHp;
#pragma unroll
        for (int c = 0; c < 2; c++) {
            const float *own = c ? e1 : e0, *oth = c ? e0 : e1, *rhs = c ? r1p : r0p;
            const int s = (y & 1) ^ c, q = 1 - s;
            const float4 v = *reinterpret_cast<const float4 *>(own + ro + k);
            const float4 rh = *reinterpret_cast<const float4 *>(rhs + ro + roff + k);
            const float4 up = *reinterpret_cast<const float4 *>(oth + ro - KHp + k);
            const float4 dn = *reinterpret_cast<const float4 *>(oth + ro + KHp + k);
            const float4 mid = *reinterpret_cast<const float4 *>(oth + ro + k);
            const float extra = oth[ro + (q ? k - 1 : k + 4)];
            acc += quad_residual_sq(v, rh, up, dn, mid, extra, q, 2 * k + s, y, G.W, G.H);
        }
    }
    return acc;
}

// Cluster-wide sum of one value per CTA (s_part[0], written before the call
// by each CTA), identical in every CTA: lanes 0..C-1 of warp 0 read the C
// partials in parallel and reduce them in a fixed order.  Ends with a
// cluster barrier, after which s_part may be rewritten.
__device__ __forceinline__ double cluster_sum(cg::cluster_group &cl, double *s_part, double *s_bcast, int C)
{
    cl.sync();
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        double x = lane < C ? *cl.map_shared_rank(s_part, lane) : 0.0;
        x = warp_sum(x);
        if (lane == 0) *s_bcast = x;
    }
    __syncthreads();
    const double tot = *s_bcast;
    cl.sync();
    return tot;
}

// Two values per CTA (s_part[0..1]) summed over the cluster the same way.
__device__ __forceinline__ void cluster_sum2(cg::cluster_group &cl, double *s_part, double *s_bcast, int C,
                                             double &t0, double &t1)
{
    cl.sync();
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        double x = 0.0, z = 0.0;
        if (lane < C) {
            const double *pp = cl.map_shared_rank(s_part, lane);
            x = pp[0];
            z = pp[1];
        }
        x = warp_sum(x);
        z = warp_sum(z);
        if (lane == 0) {
            s_bcast[0] = x;
            s_bcast[1] = z;
        }
    }
    __syncthreads();
    t0 = s_bcast[0];
    t1 = s_bcast[1];
    cl.sync();
}

// One half sweep of colour c over the band (plane rows 1..n, rhs rows 0..n-1).
__device__ __forceinline__ void relax_quad(const Planes &P, int c, int n, int r0, const Grid &G, int k, int rg, int RP)
{
    relax_block_quad(P.e(c), P.e(c ^ 1), P.r(c), -(long)P.KHp, c, 1, n + 1, r0 - 1, G, P.KHp, k, rg, RP);
}

// Block-wide sum into thread 0 (blockDim a multiple of 32).
__device__ __forceinline__ double block_sum(double v, double *s_red)
{
    v = warp_sum(v);
    if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += s_red[w];
    __syncthreads();
    return t;
}

}  // namespace planes
}  // namespace pcd
