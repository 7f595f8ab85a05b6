// sor_stream.cuh -- one exact red-black SOR sweep of the FP32 correction
// equation for grids that live in HBM, reading the old correction from one
// buffer and writing the new one to another (ping-pong).  Included by
// solver.cu inside its internal namespace (it uses the sweep bookkeeping
// defined there: Ctl, SolveArgs, end_of_sweep, last_block, vol_load).
//
// Block s owns the rows [y0, y1) of its stripe and walks down them keeping a
// window of four rows in registers: at step y it relaxes the red cells of row
// y (neighbours: old black values) and then the black cells of row y-1
// (neighbours: the new red values of rows y-2, y-1, y), after which row y-1
// is final and is stored.  The window is fed by loads issued three steps
// ahead.  The red rows y0-1 and y1 that the first and last black rows need
// belong to the neighbouring stripes; they are recomputed here from the old
// buffer, which gives bit-identical values, so the stripes need no ordering
// among themselves and no boundary pass.  A cell's update is the reference's
// delta = omega/cnt * (sum - cnt*v - b) (solver.cpp:47), summed in its order
// (left, up, right, down).
//
// Thread t owns the G consecutive 4-cell groups starting at column 4*G*t and
// loads each row of them with 16-byte loads (rows start 16-byte aligned: the
// row stride is a multiple of 4 floats).  Horizontal neighbours across groups
// come from registers, across lanes by shuffles and across warps through a
// small double-buffered shared-memory array (one block barrier per step).
#pragma once

constexpr int kStreamThreadsMax = 512;
constexpr int kStreamRowsMin = 16;

__device__ __forceinline__ float f4get(const float4 &v, int i)
{
    return i == 0 ? v.x : (i == 1 ? v.y : (i == 2 ? v.z : v.w));
}

__device__ __forceinline__ void f4put(float4 &v, int i, float f)
{
    if (i == 0) v.x = f;
    else if (i == 1) v.y = f;
    else if (i == 2) v.z = f;
    else v.w = f;
}

// Row `row` of the group at column `col`; zeros outside the grid and past the
// last row the stripe needs (`last`).
__device__ __forceinline__ float4 load_row(const float *__restrict__ p, int row, int last, int ld, int H, int col,
                                           int W)
{
    if (row < 0 || row >= H || row > last || col >= W) return make_float4(0.f, 0.f, 0.f, 0.f);
    return __ldg(reinterpret_cast<const float4 *>(p + (long)row * ld + col));
}

// Relaxes the cells of group `cur` whose column parity is `par` (cells par and
// par + 2 of the group).  lft / rgt: the cells left of the group's first and
// right of its last cell.
template <bool TRACK>
__device__ __forceinline__ void relax_group(float4 &cur, const float4 &up, const float4 &dn, const float4 &rhs,
                                            float lft, float rgt, int col, int y, int W, int H, int par,
                                            const float (&w)[5], float &m)
{
#pragma unroll
    for (int q = 0; q < 2; q++) {
        const int i = par + 2 * q;
        const int x = col + i;
        if (x >= W) continue;
        const float v = f4get(cur, i);
        const float l = i > 0 ? f4get(cur, i - 1) : lft;
        const float r = i < 3 ? f4get(cur, i + 1) : rgt;
        float s = 0.f;
        int c = 0;
        if (x > 0) { s += l; c++; }
        if (y > 0) { s += f4get(up, i); c++; }
        if (x < W - 1) { s += r; c++; }
        if (y < H - 1) { s += f4get(dn, i); c++; }
        const float wc = c == 4 ? w[4] : (c == 3 ? w[3] : (c == 2 ? w[2] : w[1]));
        const float d = wc * (s - (float)c * v - f4get(rhs, i));
        f4put(cur, i, v + d);
        if (TRACK) m = fmaxf(m, fabsf(d));
    }
}

// Edge groups (a cell without four neighbours) without max tracking, kept
// out of line: the sweep loops are unrolled and the rare path would
// otherwise crowd the instruction cache.  Arguments and result by value so
// that the call keeps them in registers.
__device__ __noinline__ float4 relax_group_edge(float4 cur, float4 up, float4 dn, float4 rhs, float lft, float rgt,
                                                int col, int y, int W, int H, int par, float w1, float w2, float w3,
                                                float w4)
{
    const float w[5] = {0.f, w1, w2, w3, w4};
    float m = 0.f;
    relax_group<false>(cur, up, dn, rhs, lft, rgt, col, y, W, H, par, w, m);
    return cur;
}

// Relaxes the cells of parity `par` in the G groups of one row.  `lft` / `rgt`:
// the cells left of the thread's first and right of its last group.  Groups
// whose cells all have four neighbours take the short form
// v + w4 * ((l + r + u + d) - 4 v - b).
template <int G, bool TRACK>
__device__ __forceinline__ void relax_row_groups(float4 (&cur)[G], const float4 (&up)[G], const float4 (&dn)[G],
                                                 const float4 (&rhs)[G], float lft, float rgt, int col0, int y,
                                                 int W, int H, int par, const float (&w)[5], float &m)
{
    const bool rows_in = y > 0 && y < H - 1;
#pragma unroll
    for (int k = 0; k < G; k++) {
        const int col = col0 + 4 * k;
        const float l = k > 0 ? cur[k - 1].w : lft;
        const float r = k + 1 < G ? cur[k + 1].x : rgt;
        if (rows_in && col > 0 && col + 4 < W) {
            float4 &c = cur[k];
            if (par == 0) {
                const float s0 = (l + c.y) + (up[k].x + dn[k].x);
                const float s2 = (c.y + c.w) + (up[k].z + dn[k].z);
                const float n0 = fmaf(w[4], fmaf(-4.f, c.x, s0) - rhs[k].x, c.x);
                const float n2 = fmaf(w[4], fmaf(-4.f, c.z, s2) - rhs[k].z, c.z);
                if (TRACK) m = fmaxf(m, fmaxf(fabsf(n0 - c.x), fabsf(n2 - c.z)));
                c.x = n0;
                c.z = n2;
            } else {
                const float s1 = (c.x + c.z) + (up[k].y + dn[k].y);
                const float s3 = (c.z + r) + (up[k].w + dn[k].w);
                const float n1 = fmaf(w[4], fmaf(-4.f, c.y, s1) - rhs[k].y, c.y);
                const float n3 = fmaf(w[4], fmaf(-4.f, c.w, s3) - rhs[k].w, c.w);
                if (TRACK) m = fmaxf(m, fmaxf(fabsf(n1 - c.y), fabsf(n3 - c.w)));
                c.y = n1;
                c.w = n3;
            }
        } else if (TRACK) {
            relax_group<TRACK>(cur[k], up[k], dn[k], rhs[k], l, r, col, y, W, H, par, w, m);
        } else {
            cur[k] = relax_group_edge(cur[k], up[k], dn[k], rhs[k], l, r, col, y, W, H, par, w[1], w[2], w[3], w[4]);
        }
    }
}

// Ring slots of the row window: E holds rows y-2 .. y+3 and Rr rows y-1 ..
// y+4 of step j at slot (row - ys) mod 6, so with the row loop unrolled six
// times every slot index is a compile-time constant and no register is ever
// copied (a copy of a register whose load is in flight would wait for it).
template <int G, bool TRACK, int P>
__device__ __forceinline__ bool stream_step(float4 (&E)[6][G], float4 (&Rr)[6][G], const float *__restrict__ ein,
                                            float *__restrict__ eout, const float *__restrict__ rhs, int j, int ys,
                                            int y0, int y1, int W, int H, int ld, int col0, int lane, int warp,
                                            int nwarps, float (&edge)[2][2][2][kStreamThreadsMax / 32],
                                            const float (&w)[5], float &m)
{
    constexpr int sA = (P + 4) % 6, sB = (P + 5) % 6, sC = P % 6, sD = (P + 1) % 6;
    const int y = ys + j;
    if (y > y1) return true;
    const int par = y & 1;  // red cells of row y and black cells of row y-1 sit at columns of parity y
    // horizontal neighbours at the thread's edges: rows C (old) and B (red new)
    const float cF = E[sC][0].x, cL = E[sC][G - 1].w, bF = E[sB][0].x, bL = E[sB][G - 1].w;
    float cLft = __shfl_up_sync(0xffffffffu, cL, 1), bLft = __shfl_up_sync(0xffffffffu, bL, 1);
    float cRgt = __shfl_down_sync(0xffffffffu, cF, 1), bRgt = __shfl_down_sync(0xffffffffu, bF, 1);
    if (lane == 0) { edge[par][0][0][warp] = cF; edge[par][0][1][warp] = bF; }
    if (lane == 31) { edge[par][1][0][warp] = cL; edge[par][1][1][warp] = bL; }
    __syncthreads();
    if (lane == 0 && warp > 0) { cLft = edge[par][1][0][warp - 1]; bLft = edge[par][1][1][warp - 1]; }
    if (lane == 31 && warp + 1 < nwarps) { cRgt = edge[par][0][0][warp + 1]; bRgt = edge[par][0][1][warp + 1]; }

    // red cells of row y
    if (y >= 0 && y < H)
        relax_row_groups<G, TRACK>(E[sC], E[sB], E[sD], Rr[sC], cLft, cRgt, col0, y, W, H, par, w, m);
    // black cells of row y-1, then row y-1 is final
    const int yb = y - 1;
    if (yb >= y0 && yb < y1) {
        relax_row_groups<G, TRACK>(E[sB], E[sA], E[sC], Rr[sB], bLft, bRgt, col0, yb, W, H, par, w, m);
#pragma unroll
        for (int k = 0; k < G; k++) {
            const int col = col0 + 4 * k;
            float *dst = eout + (long)yb * ld + col;
            if (col + 3 < W) {
                *reinterpret_cast<float4 *>(dst) = E[sB][k];
            } else if (col < W) {
                for (int i = 0; i < W - col; i++) dst[i] = f4get(E[sB][k], i);
            }
        }
    }
    // the slots of rows y-2 (E) and y-1 (Rr) are free: load rows y+4 and y+5
#pragma unroll
    for (int k = 0; k < G; k++) {
        const int col = col0 + 4 * k;
        E[sA][k] = load_row(ein, y + 4, y1 + 1, ld, H, col, W);
        Rr[sB][k] = load_row(rhs, y + 5, y1, ld, H, col, W);
    }
    return false;
}

template <int G, bool TRACK>
__global__ void __launch_bounds__(kStreamThreadsMax, 1)
    k_sweep_stream(const float *__restrict__ ein, float *__restrict__ eout, const float *__restrict__ rhs, Ctl *ctl,
                   SolveArgs a, int R, int out_idx)
{
    if (vol_load(&ctl->halt)) return;
    // [parity][0: first cell of the warp's first group, 1: last cell of its
    // last group][row C, row B][warp]
    __shared__ float edge[2][2][2][kStreamThreadsMax / 32];

    const int W = a.W, H = a.H, ld = a.ld;
    const int y0 = blockIdx.x * R, y1 = min(y0 + R, H);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const int col0 = 4 * G * threadIdx.x;
    float w[5];
#pragma unroll
    for (int c = 0; c < 5; c++) w[c] = a.w32[c];

    const int ys = y0 - 1;  // first step: the red row above the stripe
    float4 E[6][G], Rr[6][G];
#pragma unroll
    for (int k = 0; k < G; k++) {
        const int col = col0 + 4 * k;
#pragma unroll
        for (int q = 0; q < 6; q++) {
            // E slot q: row ys + q for q <= 3, rows ys - 2 (A, unused) and ys - 1 (B) at slots 4, 5
            const int er = q <= 3 ? ys + q : ys + q - 6;
            E[q][k] = q == 4 ? make_float4(0.f, 0.f, 0.f, 0.f) : load_row(ein, er, y1 + 1, ld, H, col, W);
            // Rr slot q: row ys + q for q <= 4; slot 5 is row ys - 1 (rB of the first step, unused)
            Rr[q][k] = q <= 4 ? load_row(rhs, ys + q, y1, ld, H, col, W) : make_float4(0.f, 0.f, 0.f, 0.f);
        }
    }
    float m = 0.f;
    for (int j = 0;; j += 6) {
        if (stream_step<G, TRACK, 0>(E, Rr, ein, eout, rhs, j, ys, y0, y1, W, H, ld, col0, lane, warp, nwarps, edge, w, m)) break;
        if (stream_step<G, TRACK, 1>(E, Rr, ein, eout, rhs, j + 1, ys, y0, y1, W, H, ld, col0, lane, warp, nwarps, edge, w, m)) break;
        if (stream_step<G, TRACK, 2>(E, Rr, ein, eout, rhs, j + 2, ys, y0, y1, W, H, ld, col0, lane, warp, nwarps, edge, w, m)) break;
        if (stream_step<G, TRACK, 3>(E, Rr, ein, eout, rhs, j + 3, ys, y0, y1, W, H, ld, col0, lane, warp, nwarps, edge, w, m)) break;
        if (stream_step<G, TRACK, 4>(E, Rr, ein, eout, rhs, j + 4, ys, y0, y1, W, H, ld, col0, lane, warp, nwarps, edge, w, m)) break;
        if (stream_step<G, TRACK, 5>(E, Rr, ein, eout, rhs, j + 5, ys, y0, y1, W, H, ld, col0, lane, warp, nwarps, edge, w, m)) break;
    }
    if (TRACK) {
        double v[1] = {(double)m};
        block_reduce<1, 1u>(v);
        if (threadIdx.x == 0 && v[0] > 0.0) atomicMax(&ctl->maxbits, (unsigned long long)__double_as_longlong(v[0]));
    }
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned t = atomicAdd(&ctl->blocks_done, 1u);
        if (t == gridDim.x - 1) {
            __threadfence();
            ((volatile Ctl *)ctl)->stream_out = out_idx;
            end_of_sweep(ctl, a);
        }
    }
}

// Brings the latest correction into buffer 0 when the last sweep that ran
// wrote buffer 1 (odd chunk, or sweeps halted mid-chunk).
__global__ void __launch_bounds__(256)
    k_stream_settle(float *__restrict__ e0, const float *__restrict__ e1, Ctl *ctl, SolveArgs a)
{
    if (vol_load(&ctl->done) || vol_load(&ctl->stream_out) == 0) return;
    const long n = (long)a.W * a.H;
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
        const int y = (int)(t / a.W), x = (int)(t - (long)y * a.W);
        const long i = (long)y * a.ld + x;
        e0[i] = e1[i];
    }
    if (last_block(ctl)) {
        if (threadIdx.x == 0) {
            ((volatile Ctl *)ctl)->stream_out = 0;
            ctl->blocks_done_r = 0;
            __threadfence();
        }
    }
}

// ---------------------------------------------------------------------------
// The same sweep with its rows staged in shared memory by the bulk-copy
// engine (cp.async.bulk, one copy per row, completion on an mbarrier per
// slot).  Ring of kTmaE rows of the old correction and kTmaR rows of the
// right-hand side per block; thread 0 refills a slot right after the block
// barrier that ends its last use, so the copies run kTmaE-3 / kTmaR rows
// ahead of the rows being relaxed.  The register window holds rows y-2..y+1
// of the thread's groups.  A red-updated row is written back to its slot;
// horizontal neighbours at a thread's edges are read from the slot (old
// black values for the red cells of row y, new red values for the black
// cells of row y-1), so no lane or warp exchange is needed.  Slot lifetimes
// (e row r): copy issued after barrier S_{r-kTmaE+2}, read at step r-1 (as
// D), red-updated and written back at step r, edge-read at step r+1, free
// after barrier S_{r+2}.  r rows: read at step r, free after S_r.
// Every wait on an mbarrier is bounded; on timeout the block records
// PCD_TIMEOUT in the control block and stops waiting (the sweep result is
// then invalid and the host reports the error).
constexpr int kTmaE = 8;  // ring sizes: powers of two (slot = ring index & (size - 1))
constexpr int kTmaR = 4;

__device__ __forceinline__ unsigned smem_u32(const void *p)
{
    return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Thread 0: announce `bytes` and start the copy of one row into a slot.
__device__ __forceinline__ void tma_row(float *dst, const float *src, unsigned bytes, unsigned long long *bar)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

// Bounded wait for phase `parity` of an mbarrier; false on timeout.
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, unsigned parity, long limit)
{
    const unsigned a = smem_u32(bar);
    for (long i = 0; i < limit; i++) {
        unsigned ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok)
            : "r"(a), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}

// One step of the staged sweep (row y = ys + j, j = 8 i + P).  Ring slots:
// e row y+d sits at slot (j + 1 + d) & 7 (e ring index t = row - (y0 - 2)),
// r row y at slot j & 3 (r ring index t = row - (y0 - 1)); the register
// window W4[(j + c) & 3] holds e rows y-2+c (c = 0..3) and rr[j & 1] / rr[(j+1)
// & 1] the r rows y-1 / y.  With P a template argument every slot, register
// and mbarrier parity below is a compile-time constant up to the bit i & 1.
template <int G, bool TRACK, int P>
__device__ __forceinline__ bool tma_step(float4 (&W4)[4][G], float4 (&rr)[2][G], float *es, float *rs,
                                         unsigned long long *ebar, unsigned long long *rbar,
                                         const float *__restrict__ ein, float *__restrict__ eout,
                                         const float *__restrict__ rhs, int i, int ys, int y0, int y1, int W, int H,
                                         int ld, int wpad, unsigned bytes, int e_last, int r_last, int col0,
                                         bool lft_ok, bool rgt_ok, const float (&w)[5], long spin_limit, bool &ok,
                                         float &m)
{
    constexpr int cA = (P + 0) & 3, cB = (P + 1) & 3, cC = (P + 2) & 3, cD = (P + 3) & 3;
    // e ring index of row y + d is j + 1 + d: A (y-2) j-1, B j, C j+1, D j+2
    constexpr int sB = P & 7, sC = (P + 1) & 7, sD = (P + 2) & 7, sFree = (P + 7) & 7;
    constexpr int rS = P & 3;
    const int j = 8 * i + P;
    const int y = ys + j;
    if (y > y1) return true;
    // e row y+1 into the window
    const int yd = y + 1;
    if (yd >= 0 && yd <= e_last) {
        const unsigned par = (unsigned)(((j + 2) >> 3) & 1);
        if (ok && !mbar_wait(ebar + sD, par, spin_limit)) ok = false;
        const float *src = es + (size_t)sD * wpad;
#pragma unroll
        for (int k = 0; k < G; k++) {
            const int col = col0 + 4 * k;
            W4[cD][k] = col < W ? *reinterpret_cast<const float4 *>(src + col) : make_float4(0.f, 0.f, 0.f, 0.f);
        }
    } else {
#pragma unroll
        for (int k = 0; k < G; k++) W4[cD][k] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    // r row y (ring index j)
    float4 (&rC)[G] = rr[P & 1];
    const float4 (&rB)[G] = rr[(P + 1) & 1];
    if (y >= 0 && y <= r_last) {
        const unsigned par = (unsigned)((j >> 2) & 1);
        if (ok && !mbar_wait(rbar + rS, par, spin_limit)) ok = false;
        const float *src = rs + (size_t)rS * wpad;
#pragma unroll
        for (int k = 0; k < G; k++) {
            const int col = col0 + 4 * k;
            rC[k] = col < W ? *reinterpret_cast<const float4 *>(src + col) : make_float4(0.f, 0.f, 0.f, 0.f);
        }
    }
    __syncthreads();  // S_y
    if (threadIdx.x == 0) {
        // refill the slots freed by S_y: e row y+6 (slot of row y-2) and r row y+4
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        const int en = y + 6, rn = y + 4;
        if (j >= 1 && en <= e_last) tma_row(es + (size_t)sFree * wpad, ein + (long)en * ld, bytes, ebar + sFree);
        if (rn <= r_last) tma_row(rs + (size_t)rS * wpad, rhs + (long)rn * ld, bytes, rbar + rS);
    }
    const int par = y & 1;
    // red cells of row y: edges are old black values in the slot of row y
    if (y >= 0 && y < H) {
        float *sl = es + (size_t)sC * wpad;
        const float lft = lft_ok ? sl[col0 - 1] : 0.f;
        const float rgt = rgt_ok ? sl[col0 + 4 * G] : 0.f;
        relax_row_groups<G, TRACK>(W4[cC], W4[cB], W4[cD], rC, lft, rgt, col0, y, W, H, par, w, m);
#pragma unroll
        for (int k = 0; k < G; k++) {
            const int col = col0 + 4 * k;
            if (col < W) *reinterpret_cast<float4 *>(sl + col) = W4[cC][k];
        }
    }
    // black cells of row y-1: edges are the new red values written back at step y-1
    const int yb = y - 1;
    if (yb >= y0 && yb < y1) {
        const float *sl = es + (size_t)sB * wpad;
        const float lft = lft_ok ? sl[col0 - 1] : 0.f;
        const float rgt = rgt_ok ? sl[col0 + 4 * G] : 0.f;
        relax_row_groups<G, TRACK>(W4[cB], W4[cA], W4[cC], rB, lft, rgt, col0, yb, W, H, par, w, m);
#pragma unroll
        for (int k = 0; k < G; k++) {
            const int col = col0 + 4 * k;
            float *dst = eout + (long)yb * ld + col;
            if (col + 3 < W) *reinterpret_cast<float4 *>(dst) = W4[cB][k];
            else if (col < W)
                for (int q = 0; q < W - col; q++) dst[q] = f4get(W4[cB][k], q);
        }
    }
    return false;
}

template <int G, bool TRACK>
__global__ void __launch_bounds__(kStreamThreadsMax, 1)
    k_sweep_tma(const float *__restrict__ ein, float *__restrict__ eout, const float *__restrict__ rhs, Ctl *ctl,
                SolveArgs a, int R, int out_idx, int wpad, long spin_limit)
{
    if (vol_load(&ctl->halt)) return;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    float *es = reinterpret_cast<float *>(smem_raw);
    float *rs = es + (size_t)kTmaE * wpad;
    unsigned long long *bar = reinterpret_cast<unsigned long long *>(rs + (size_t)kTmaR * wpad);
    unsigned long long *ebar = bar, *rbar = bar + kTmaE;

    const int W = a.W, H = a.H, ld = a.ld;
    const int y0 = blockIdx.x * R, y1 = min(y0 + R, H);
    const int e_last = min(y1 + 1, H - 1), r_last = min(y1, H - 1);  // last rows the stripe needs
    const int ys = y0 - 1;
    const unsigned bytes = (unsigned)wpad * 4u;
    const int col0 = 4 * G * threadIdx.x;
    const bool lft_ok = col0 > 0, rgt_ok = col0 + 4 * G < W;
    float w[5];
#pragma unroll
    for (int c = 0; c < 5; c++) w[c] = a.w32[c];

    if (threadIdx.x == 0) {
        for (int q = 0; q < kTmaE + kTmaR; q++) mbar_init(bar + q, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        // first use of every slot; rows above the grid complete their phase
        // with a plain arrive so that slot parities follow the ring index
        for (int t = 0; t < kTmaE; t++) {
            const int row = y0 - 2 + t;
            if (row < 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(ebar + t)) : "memory");
            else if (row <= e_last) tma_row(es + (size_t)t * wpad, ein + (long)row * ld, bytes, ebar + t);
        }
        for (int t = 0; t < kTmaR; t++) {
            const int row = ys + t;
            if (row < 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(rbar + t)) : "memory");
            else if (row <= r_last) tma_row(rs + (size_t)t * wpad, rhs + (long)row * ld, bytes, rbar + t);
        }
    }
    __syncthreads();

    bool ok = true;
    float m = 0.f;
    float4 W4[4][G], rr[2][G];
    // window before step 0: rows y0-3 (unused), y0-2, y0-1 at W4[0..2]
#pragma unroll
    for (int c = 0; c < 3; c++) {
        const int row = y0 - 3 + c;  // ring index c - 1
#pragma unroll
        for (int k = 0; k < G; k++) W4[c][k] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (c >= 1 && row >= 0 && row <= e_last) {
            if (ok && !mbar_wait(ebar + (c - 1), 0u, spin_limit)) ok = false;
            const float *src = es + (size_t)(c - 1) * wpad;
#pragma unroll
            for (int k = 0; k < G; k++) {
                const int col = col0 + 4 * k;
                if (col < W) W4[c][k] = *reinterpret_cast<const float4 *>(src + col);
            }
        }
    }
#pragma unroll
    for (int k = 0; k < G; k++) {
        rr[0][k] = make_float4(0.f, 0.f, 0.f, 0.f);
        rr[1][k] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    for (int i = 0;; i++) {
#define PCD_TMA_STEP(PP)                                                                                           \
    if (tma_step<G, TRACK, PP>(W4, rr, es, rs, ebar, rbar, ein, eout, rhs, i, ys, y0, y1, W, H, ld, wpad, bytes,   \
                               e_last, r_last, col0, lft_ok, rgt_ok, w, spin_limit, ok, m))                    \
        break;
        PCD_TMA_STEP(0) PCD_TMA_STEP(1) PCD_TMA_STEP(2) PCD_TMA_STEP(3)
        PCD_TMA_STEP(4) PCD_TMA_STEP(5) PCD_TMA_STEP(6) PCD_TMA_STEP(7)
#undef PCD_TMA_STEP
    }
    if (!ok) atomicExch(&ctl->error, (int)PCD_TIMEOUT);
    if (TRACK) {
        double v[1] = {(double)m};
        block_reduce<1, 1u>(v);
        if (threadIdx.x == 0 && v[0] > 0.0) atomicMax(&ctl->maxbits, (unsigned long long)__double_as_longlong(v[0]));
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned t = atomicAdd(&ctl->blocks_done, 1u);
        if (t == gridDim.x - 1) {
            __threadfence();
            ((volatile Ctl *)ctl)->stream_out = out_idx;
            end_of_sweep(ctl, a);
        }
    }
}

// Dynamic shared memory of k_sweep_tma for rows of wpad floats.
inline size_t tma_smem_bytes(int wpad)
{
    return (size_t)(kTmaE + kTmaR) * wpad * sizeof(float) + (kTmaE + kTmaR) * sizeof(unsigned long long);
}
