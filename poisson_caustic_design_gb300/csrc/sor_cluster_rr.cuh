// sor_cluster_rr.cuh -- register-resident form of the cluster FP32 SOR
// (included by sor_cluster.cu inside its anonymous namespace, after the
// shared-memory helpers lds4 / sts4).
//
// Widths W = 8 KQ up to 512, K = 4 or 2 sweeps per halo exchange, L = 2..4
// rows per warp, NQ = 1 or 2 quads per lane.  A CTA of 16 warps; warp w
// holds the plane rows [w L, w L + L) of the CTA's band plus halo, lane l the
// quads qi = l + 32 i (i < NQ) of both colours of each of its rows in
// registers: quad qi of colour c in row y covers the cells
// x = 8 qi + 2 t + ((y & 1) ^ c), t < 4.
// Horizontal neighbours come from the adjacent lane by shuffle, vertical ones
// from the warp's own registers except across warp boundaries, where each
// warp publishes its first and last row of the colour it just relaxed in
// shared memory (double-buffered by colour, so one block barrier per half
// sweep).  The right-hand side stays in shared memory, negated (one 16-byte
// load per quad and half sweep); the update runs in packed FP32 pairs.
//
// Temporal blocking as in k_sor_cluster_tb: K sweeps per halo exchange on the
// band and HK = 2K halo rows on each side, the halo recomputed with the same
// arithmetic as its owner.  After a round the warps holding the band's first
// and last HK rows store them straight into the neighbouring CTAs' inboxes
// (distributed shared memory, double-buffered by round parity); one cluster
// barrier later the warps holding halo rows read their inbox.  A CTA writes
// an inbox buffer again two rounds later, after the barrier that follows the
// reader's reads.
//
// Cells without some neighbour (x = 0, x = W-1, y = 0, y = H-1) take their own
// value in that neighbour's place and the weight omega / cnt of their true
// neighbour count, which is the Neumann update of the reference operator.
// Quads past the last column keep weight 0 and stay zero.

constexpr int kRRThreads = 512;
constexpr int kRRWarps = kRRThreads / 32;

// Shared floats: edge rows [2 colours][16 warps][2 sides], inbox
// [2 parities][2 sides][2 colours][HK rows], -r32 planes [2 colours][R rows],
// each row KS = 128 NQ slots.
__host__ __device__ inline size_t rr_floats(int K, int NQ, int R)
{
    const size_t KS = (size_t)128 * NQ;
    return ((size_t)4 * kRRWarps + (size_t)16 * K + (size_t)2 * R) * KS;
}

// The update of quad_ghost with the parity q as an argument (folded to a
// constant where the caller's q is one), in packed FP32 pairs: cells (x, y)
// and (z, w) of the quad share one instruction per step.  nrh is -r32.  The
// steps and their rounding are those of the scalar form
// v + w ((l + r) + (u + d) - 4 v - r32).
__device__ __forceinline__ float4 quad_ghost_q(int q, const float4 &v, const float4 &nrh, const float4 &u,
                                              const float4 &d, const float4 &m, float ex, float2 wA, float2 wB)
{
    const float h0 = q ? ex + m.x : m.x + m.y;
    const float h1 = q ? m.x + m.y : m.y + m.z;
    const float h2 = q ? m.y + m.z : m.z + m.w;
    const float h3 = q ? m.z + m.w : m.w + ex;
    const float2 vA = make_float2(v.x, v.y), vB = make_float2(v.z, v.w);
    const float2 m4 = make_float2(-4.f, -4.f);
    float2 tA = __fadd2_rn(make_float2(h0, h1), __fadd2_rn(make_float2(u.x, u.y), make_float2(d.x, d.y)));
    float2 tB = __fadd2_rn(make_float2(h2, h3), __fadd2_rn(make_float2(u.z, u.w), make_float2(d.z, d.w)));
    tA = __fadd2_rn(__ffma2_rn(m4, vA, tA), make_float2(nrh.x, nrh.y));
    tB = __fadd2_rn(__ffma2_rn(m4, vB, tB), make_float2(nrh.z, nrh.w));
    const float2 nA = __ffma2_rn(wA, tA, vA), nB = __ffma2_rn(wB, tB, vB);
    return make_float4(nA.x, nA.y, nB.x, nB.y);
}

// Largest |nv - v| over the quad (a NaN change does not raise it).
__device__ __forceinline__ float quad_max_change(const float4 &v, const float4 &nv)
{
    return fmaxf(fmaxf(fabsf(nv.x - v.x), fabsf(nv.y - v.y)), fmaxf(fabsf(nv.z - v.z), fabsf(nv.w - v.w)));
}

// Sum of squares of r32 - L v over the quad (ghost neighbours as above; nrh
// is -r32).
__device__ __forceinline__ float quad_ghost_res2(int q, const float4 &v, const float4 &nrh, const float4 &u,
                                                const float4 &d, const float4 &m, float ex)
{
    const float l0 = q ? ex : m.x, r0v = q ? m.x : m.y;
    const float l1 = q ? m.x : m.y, r1v = q ? m.y : m.z;
    const float l2 = q ? m.y : m.z, r2v = q ? m.z : m.w;
    const float l3 = q ? m.z : m.w, r3v = q ? m.w : ex;
    const float a0 = nrh.x + fmaf(-4.f, v.x, (l0 + r0v) + (u.x + d.x));
    const float a1 = nrh.y + fmaf(-4.f, v.y, (l1 + r1v) + (u.y + d.y));
    const float a2 = nrh.z + fmaf(-4.f, v.z, (l2 + r2v) + (u.z + d.z));
    const float a3 = nrh.w + fmaf(-4.f, v.w, (l3 + r3v) + (u.w + d.w));
    return fmaf(a0, a0, fmaf(a1, a1, fmaf(a2, a2, a3 * a3)));
}

template <int K, int L, int NQ>
struct RRState {
    static constexpr int HK = 2 * K, KS = 128 * NQ;
    float4 e[2][L][NQ];      // both colours of the warp's rows
    float2 waa[NQ], wla[NQ], war[NQ];  // weight pairs: (wa, wa), (wl, wa), (wa, wr)
    bool act[NQ], eL[NQ], eR[NQ];
    bool own[NQ];            // tile passes: quad in the tile's interior columns
    float w4, w3, w2, w1;
    int lane, w, H, ybase, R;
    unsigned edge_s, r_s;    // shared addresses of slot 4 * lane of edge row 0 / -r32 row 0

    __device__ __forceinline__ unsigned edge_addr(int c, int ww, int side) const
    {
        return edge_s + 4u * (unsigned)(((c * kRRWarps + ww) * 2 + side) * KS);
    }

    template <int CC>
    __device__ __forceinline__ void put_edges() const
    {
#pragma unroll
        for (int i = 0; i < NQ; i++) {
            sts4(edge_addr(CC, w, 0) + 512u * i, e[CC][0][i]);
            sts4(edge_addr(CC, w, 1) + 512u * i, e[CC][L - 1][i]);
        }
    }

    // The other colour's value one slot beyond quad i of a row (slot 4 qi - 1
    // when q = 1, 4 qi + 4 when q = 0): the adjacent lane's quad, or across the
    // lane wrap the neighbouring quad column.
    __device__ __forceinline__ float beyond(int q, const float4 (&m)[NQ], int i) const
    {
        if (q) {
            const float snd = (lane == 31 && i > 0) ? m[i > 0 ? i - 1 : 0].w : m[i].w;
            return __shfl_sync(0xffffffffu, snd, (lane + 31) & 31);
        }
        const float snd = (lane == 0 && i + 1 < NQ) ? m[i + 1 < NQ ? i + 1 : i].x : m[i].x;
        return __shfl_sync(0xffffffffu, snd, (lane + 1) & 31);
    }

    // Half sweep of colour CC over plane rows [lo, hi); P = parity of the
    // grid row of the warp's first row.  TR: mx takes the largest |update| of
    // the cells of plane rows [olo, ohi) in quads marked own.
    template <int CC, int P, bool TR = false>
    __device__ __forceinline__ void half(int lo, int hi, float *mx = nullptr, int olo = 0, int ohi = 0)
    {
        constexpr int OC = 1 - CC;
        float4 eu[NQ], ed[NQ];
#pragma unroll
        for (int i = 0; i < NQ; i++) {
            eu[i] = make_float4(0.f, 0.f, 0.f, 0.f);
            ed[i] = eu[i];
        }
        if (w > 0) {
#pragma unroll
            for (int i = 0; i < NQ; i++) eu[i] = lds4(edge_addr(OC, w - 1, 1) + 512u * i);
        }
        if (w < kRRWarps - 1) {
#pragma unroll
            for (int i = 0; i < NQ; i++) ed[i] = lds4(edge_addr(OC, w + 1, 0) + 512u * i);
        }
        const int lr0 = w * L, y0 = ybase + lr0;
        if (lr0 >= hi || lr0 + L <= lo) {
            // no row of the warp in range
        } else if (y0 > 0 && y0 + L < H) {
            // every row of the warp is an interior grid row: no branches, so
            // the quads of all rows interleave.  Rows of the warp outside
            // [lo, hi) are relaxed too: they lie in the halo outside the
            // dependency cone of the band (a row in [lo, hi) reads only rows
            // of the previous half sweep's range), and the halo is
            // overwritten at the next exchange; rows past the CTA's plane
            // stay bounded and are never read by a band row.
#pragma unroll
            for (int j = 0; j < L; j++) {
                const int q = 1 - ((P ^ j ^ CC) & 1);
                // rows past the plane (16 L > R) read its last row, and are dropped
                const unsigned rrow = r_s + 4u * (unsigned)((CC * R + min(lr0 + j, R - 1)) * KS);
#pragma unroll
                for (int i = 0; i < NQ; i++) {
                    const float4 v = e[CC][j][i];
                    const float4 rh = lds4(rrow + 512u * i);
                    float ex = beyond(q, e[OC][j], i);
                    if (q ? eL[i] : eR[i]) ex = q ? v.x : v.w;
                    const float4 u = j > 0 ? e[OC][j > 0 ? j - 1 : 0][i] : eu[i];
                    const float4 d = j + 1 < L ? e[OC][j + 1 < L ? j + 1 : j][i] : ed[i];
                    const float4 nv =
                        quad_ghost_q(q, v, rh, u, d, e[OC][j][i], ex, q ? wla[i] : waa[i], q ? waa[i] : war[i]);
                    if (TR && own[i] && lr0 + j >= olo && lr0 + j < ohi) *mx = fmaxf(*mx, quad_max_change(v, nv));
                    e[CC][j][i] = nv;
                }
            }
        } else {
            // a warp holding the grid's first or last row (or rows beyond
            // it): branch free as well, rows outside the grid with weight 0,
            // the first / last row with its missing neighbour's ghost and
            // weight omega / (cnt)
            const bool two = H > 1;
#pragma unroll
            for (int j = 0; j < L; j++) {
                const int lr = lr0 + j, y = ybase + lr;
                const bool on = lr >= lo && lr < hi && y >= 0 && y < H;
                const bool top = y == 0, bot = y == H - 1, brd = top || bot;
                const int q = 1 - ((P ^ j ^ CC) & 1);
                const unsigned rrow = r_s + 4u * (unsigned)((CC * R + min(lr, R - 1)) * KS);
#pragma unroll
                for (int i = 0; i < NQ; i++) {
                    const float4 v = e[CC][j][i];
                    const float4 rh = lds4(rrow + 512u * i);
                    float ex = beyond(q, e[OC][j], i);
                    const bool edge = q ? eL[i] : eR[i];
                    if (edge) ex = q ? v.x : v.w;
                    float4 u = j > 0 ? e[OC][j > 0 ? j - 1 : 0][i] : eu[i];
                    float4 d = j + 1 < L ? e[OC][j + 1 < L ? j + 1 : j][i] : ed[i];
                    if (top) u = v;
                    if (bot) d = v;
                    const float a = !on || !act[i] ? 0.f : brd ? (two ? w3 : w2) : w4;
                    const float we = !on ? 0.f : edge ? (brd ? (two ? w2 : w1) : w3) : a;
                    const float2 wA = make_float2(q ? we : a, a), wB = make_float2(a, q ? a : we);
                    const float4 nv = quad_ghost_q(q, v, rh, u, d, e[OC][j][i], ex, wA, wB);
                    if (TR && on && own[i] && lr >= olo && lr < ohi) *mx = fmaxf(*mx, quad_max_change(v, nv));
                    e[CC][j][i] = nv;
                }
            }
        }
        put_edges<CC>();
    }

    // Sum over the band's rows [HK, HK + n) of (r32 - L e)^2, both colours.
    template <int P>
    __device__ __forceinline__ float residual(int n) const
    {
        float acc = 0.f;
#pragma unroll
        for (int CC = 0; CC < 2; CC++) {
            const int OC = 1 - CC;
            float4 eu[NQ], ed[NQ];
#pragma unroll
            for (int i = 0; i < NQ; i++) {
                eu[i] = w > 0 ? lds4(edge_addr(OC, w > 0 ? w - 1 : 0, 1) + 512u * i) : make_float4(0.f, 0.f, 0.f, 0.f);
                ed[i] = w < kRRWarps - 1 ? lds4(edge_addr(OC, w < kRRWarps - 1 ? w + 1 : w, 0) + 512u * i)
                                         : make_float4(0.f, 0.f, 0.f, 0.f);
            }
#pragma unroll
            for (int j = 0; j < L; j++) {
                const int lr = w * L + j, y = ybase + lr;
                // rows outside the band (and outside the grid) computed and dropped
                const bool on = lr >= HK && lr < HK + n;
                const unsigned rr = (unsigned)min(lr, R - 1);
                const int q = 1 - ((P ^ j ^ CC) & 1);
                const unsigned rrow = r_s + 4u * ((unsigned)CC * (unsigned)R + rr) * (unsigned)KS;
#pragma unroll
                for (int i = 0; i < NQ; i++) {
                    const float4 v = e[CC][j][i];
                    const float4 rh = lds4(rrow + 512u * i);
                    float ex = beyond(q, e[OC][j], i);
                    if (q ? eL[i] : eR[i]) ex = q ? v.x : v.w;
                    float4 u = j > 0 ? e[OC][j > 0 ? j - 1 : 0][i] : eu[i];
                    float4 d = j + 1 < L ? e[OC][j + 1 < L ? j + 1 : j][i] : ed[i];
                    if (y == 0) u = v;
                    if (y == H - 1) d = v;
                    const float s2 = quad_ghost_res2(q, v, rh, u, d, e[OC][j][i], ex);
                    acc += (on && act[i]) ? s2 : 0.f;
                }
            }
        }
        return acc;
    }
};

template <int K, int L, int NQ>
__global__ void __launch_bounds__(kRRThreads, 1) k_sor_cluster_rr(ClusterArgs a)
{
    using S = RRState<K, L, NQ>;
    constexpr int HK = S::HK, KS = S::KS;
    cg::cluster_group cl = cg::this_cluster();
    extern __shared__ __align__(16) float smem_f[];
    __shared__ float s_part[2];
    __shared__ float s_tot;
    __shared__ float s_red[kRRWarps];
    const int C = (int)cl.num_blocks(), g = (int)cl.block_rank(), W = a.W, H = a.H;
    int r0, n;
    band_of(g, C, H, r0, n);
    const int nmax = (H + C - 1) / C;
    const int R = nmax + 2 * HK;
    float *edge = smem_f;
    float *inbox = edge + (size_t)4 * kRRWarps * KS;
    float *rp = inbox + (size_t)16 * K * KS;

    const Ctl *ctl = a.ctl;
    if (*(volatile const int *)&ctl->done) return;  // speculative launch after convergence: all CTAs agree

    S st;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    st.lane = lane;
    st.w = w;
    st.H = H;
    st.ybase = r0 - HK;
    st.R = R;
    st.edge_s = (unsigned)__cvta_generic_to_shared(edge) + 16u * lane;
    st.r_s = (unsigned)__cvta_generic_to_shared(rp) + 16u * lane;
    st.w4 = a.w32[4];
    st.w3 = a.w32[3];
    st.w2 = a.w32[2];
    st.w1 = a.w32[1];
    const int KQ = W >> 3;
#pragma unroll
    for (int i = 0; i < NQ; i++) {
        const int qi = lane + 32 * i;
        st.act[i] = qi < KQ;
        st.eL[i] = qi == 0;
        st.eR[i] = qi == KQ - 1;
        const float wa = st.act[i] ? a.w32[4] : 0.f;
        st.waa[i] = make_float2(wa, wa);
        st.wla[i] = make_float2(st.eL[i] ? a.w32[3] : wa, wa);
        st.war[i] = make_float2(wa, st.eR[i] ? a.w32[3] : wa);
    }
    // own and halo rows of e (registers) and r32 (shared) from global memory
    const int Rn = n + 2 * HK;
#pragma unroll
    for (int j = 0; j < L; j++) {
        const int lr = w * L + j, y = st.ybase + lr;
        const bool in = lr < Rn && y >= 0 && y < H;
#pragma unroll
        for (int c = 0; c < 2; c++) {
            const int sc = (y & 1) ^ c;
#pragma unroll
            for (int i = 0; i < NQ; i++) {
                const int qi = lane + 32 * i;
                float4 ev = make_float4(0.f, 0.f, 0.f, 0.f), rv = ev;
                if (in && qi < KQ) {
                    const size_t b0 = (size_t)y * a.ld + 8 * qi + sc;
                    ev = make_float4(a.e[b0], a.e[b0 + 2], a.e[b0 + 4], a.e[b0 + 6]);
                    rv = make_float4(-a.r32[b0], -a.r32[b0 + 2], -a.r32[b0 + 4], -a.r32[b0 + 6]);
                }
                st.e[c][j][i] = ev;
                if (lr < R) reinterpret_cast<float4 *>(rp + (size_t)(c * R + lr) * KS)[qi] = rv;
            }
        }
    }
    st.template put_edges<0>();
    st.template put_edges<1>();
    const int done_before = *(volatile const int *)&ctl->sweeps;
    const double bnorm = *(volatile const double *)&ctl->bnorm;
    const double rstart = *(volatile const double *)&ctl->rnorm;
    const double stop_abs = kFp32StopFrac * a.tol * bnorm;
    const double drop_abs = a.drop * rstart;
    const double stop2 = stop_abs * stop_abs, drop2 = drop_abs * drop_abs;
    const int P = (st.ybase + w * L) & 1;
    __syncthreads();

    // A residual estimate taken after round m is summed over the cluster at
    // round m + 1's barrier (the warps' partials wait in s_red, the CTA's in
    // s_part[cpar]), so it costs no barrier of its own; the cycle then ends
    // after round m + 1.  s_part is double-buffered: a CTA rewrites one
    // buffer only after the next barrier, which every reader passes after
    // its read.
    int sweeps = 0, par = 0, cpar = 0, next_check = a.check_every;
    bool pending = false;
    for (;;) {
        // kr <= K sweeps on the band and its halo (fewer at the sweep caps)
        const int kr = min(K, min(a.cycle_cap - sweeps, a.max_iter - done_before - sweeps));
        for (int t = 0; t < kr; t++) {
            const int d = 2 * (kr - t) - 1;
            if (P) st.template half<0, 1>(HK - d, HK + n + d);
            else st.template half<0, 0>(HK - d, HK + n + d);
            __syncthreads();
            if (P) st.template half<1, 1>(HK - d + 1, HK + n + d - 1);
            else st.template half<1, 0>(HK - d + 1, HK + n + d - 1);
            __syncthreads();
        }
        sweeps += kr;
        if (pending && w == 0) {
            float t = lane < kRRWarps ? s_red[lane] : 0.f;
            t = warp_sum_f(t);
            if (lane == 0) s_part[cpar] = t;
        }
        // the band's first HK rows to the upper neighbour's bottom inbox, its
        // last HK rows to the lower neighbour's top inbox
#pragma unroll
        for (int j = 0; j < L; j++) {
            const int lr = w * L + j;
            // (a row can go both ways when the band has fewer than 2 HK rows)
#pragma unroll
            for (int side = 0; side < 2; side++) {
                float *dst = nullptr;
                if (side == 0 && g > 0 && lr >= HK && lr < 2 * HK)
                    dst = cl.map_shared_rank(inbox + (size_t)(((par * 2 + 1) * 2) * HK + (lr - HK)) * KS, g - 1);
                if (side == 1 && g < C - 1 && lr >= n && lr < n + HK)
                    dst = cl.map_shared_rank(inbox + (size_t)(((par * 2 + 0) * 2) * HK + (lr - n)) * KS, g + 1);
                if (dst) {
#pragma unroll
                    for (int c = 0; c < 2; c++)
#pragma unroll
                        for (int i = 0; i < NQ; i++)
                            reinterpret_cast<float4 *>(dst + (size_t)c * HK * KS)[lane + 32 * i] = st.e[c][j][i];
                }
            }
        }
        cl.sync();
        if (pending && w == 0) {
            // every CTA sums the same partials in the same order
            float x = lane < C ? *cl.map_shared_rank(&s_part[cpar], lane) : 0.f;
            x = warp_sum_f(x);
            if (lane == 0) s_tot = x;
        }
#pragma unroll
        for (int j = 0; j < L; j++) {
            const int lr = w * L + j;
            const float *src = nullptr;
            if (g > 0 && lr < HK) src = inbox + (size_t)(((par * 2 + 0) * 2) * HK + lr) * KS;
            else if (g < C - 1 && lr >= n + HK && lr < n + 2 * HK)
                src = inbox + (size_t)(((par * 2 + 1) * 2) * HK + (lr - n - HK)) * KS;
            if (src) {
#pragma unroll
                for (int c = 0; c < 2; c++)
#pragma unroll
                    for (int i = 0; i < NQ; i++)
                        st.e[c][j][i] = reinterpret_cast<const float4 *>(src + (size_t)c * HK * KS)[lane + 32 * i];
            }
        }
        par ^= 1;
        const bool cap = sweeps >= a.cycle_cap || done_before + sweeps >= a.max_iter;
        const bool check = !cap && sweeps >= next_check;
        st.template put_edges<1>();
        if (check) st.template put_edges<0>();
        __syncthreads();
        if (cap) break;
        if (pending) {
            pending = false;
            cpar ^= 1;
            const double est2 = (double)s_tot;
            if (est2 <= stop2 || est2 <= drop2) break;
        }
        if (check) {
            next_check = sweeps + a.check_every;
            float v = P ? st.template residual<1>(n) : st.template residual<0>(n);
            v = warp_sum_f(v);
            if (lane == 0) s_red[w] = v;
            pending = true;
        }
    }
#pragma unroll
    for (int j = 0; j < L; j++) {
        const int lr = w * L + j, y = st.ybase + lr;
        if (lr < HK || lr >= HK + n) continue;
#pragma unroll
        for (int c = 0; c < 2; c++) {
            const int sc = (y & 1) ^ c;
#pragma unroll
            for (int i = 0; i < NQ; i++) {
                const int qi = lane + 32 * i;
                if (qi >= KQ) continue;
                const size_t b0 = (size_t)y * a.ld + 8 * qi + sc;
                const float4 v = st.e[c][j][i];
                a.e[b0] = v.x;
                a.e[b0 + 2] = v.y;
                a.e[b0 + 4] = v.z;
                a.e[b0 + 6] = v.w;
            }
        }
    }
    if (g == 0 && threadIdx.x == 0) {
        volatile Ctl *cc = a.ctl;
        cc->sweeps = done_before + sweeps;
        if (done_before + sweeps >= a.max_iter) cc->halt = 1;
    }
    cl.sync();
}

template <int K, int NQ>
const void *rr_kernel_l(int L)
{
    switch (L) {
    case 2: return (const void *)k_sor_cluster_rr<K, 2, NQ>;
    case 3: return (const void *)k_sor_cluster_rr<K, 3, NQ>;
    case 4: return (const void *)k_sor_cluster_rr<K, 4, NQ>;
    default: return nullptr;
    }
}

// The register-resident kernel for K sweeps per exchange, L rows per warp and
// NQ quads per lane (nullptr outside the compiled set).
const void *rr_kernel(int K, int L, int NQ)
{
    if (K == 4) return NQ == 1 ? rr_kernel_l<4, 1>(L) : rr_kernel_l<4, 2>(L);
    if (K == 2) return NQ == 1 ? rr_kernel_l<2, 1>(L) : rr_kernel_l<2, 2>(L);
    return nullptr;
}
