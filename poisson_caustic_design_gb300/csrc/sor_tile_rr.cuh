// sor_tile_rr.cuh -- register-resident FP32 red-black SOR passes over grids
// that live in HBM (included by sor_cluster.cu inside its anonymous
// namespace, after sor_cluster_rr.cuh, whose RRState holds one tile).
//
// One launch runs kr <= K sweeps of the correction equation L e = r32 over
// the whole grid, reading e from one buffer and writing the other
// (ping-pong, as the stream passes do).  The grid is cut into tiles of
// R = 16 L rows and 256 NQ columns, halo included: tile (ty, tx) holds the
// rows [ty N - HK, ty N + N + HK) with N = R - 2 HK, and the columns
// [b_tx - 8, b_tx - 8 + 256 NQ) with b_t = 8 floor(t WQ / ncol), WQ = W / 8;
// it writes the rows [ty N, ty N + N) and the columns [b_tx, b_tx+1), so
// the tiles' written parts partition the grid.
//
// Rows: as in the cluster kernel, rows outside the grid have weight 0 and
// the relaxation ranges shrink with the dependency cone of the written rows
// (HK = 2 K halo rows on each side).  Columns: every quad is relaxed in
// every half sweep.  A tile's outermost quads take the lane wrap's value in
// place of their missing neighbour; that wrong value spreads by one cell per
// half sweep, 2 kr <= 8 cells per pass, so it stays in the 8-column halo.
// Quads outside the grid keep weight 0, and the grid's first and last
// columns take their own value as the missing neighbour with weight
// omega / 3 (the Neumann ghost of the cluster kernel).
//
// The kernel is persistent, one CTA per SM, taking the tiles in row-major
// order strided by the grid size; while a CTA relaxes a tile it asks L2 for
// the rows of its next tile (bulk prefetches), so that tile's loads hit L2.
// The CTA that finishes last closes the pass (end_of_sweep with kr sweeps);
// with TRACK the pass reports the largest |update| of its last sweep.
//
// k_sor_tile_batch runs the same tiles for many grids at once: the grids'
// tiles are numbered one after the other (TileJob::tile0) and the persistent
// CTAs stride over all of them, skipping the grids whose solves have halted.

// Shared floats of one tile: edge rows [2 colours][16 warps][2 sides] and the
// -r32 planes [2 colours][R rows], each row KS = 128 NQ slots.
__host__ __device__ inline size_t tile_floats(int L, int NQ)
{
    const size_t KS = (size_t)128 * NQ;
    return ((size_t)4 * kRRWarps + (size_t)2 * kRRWarps * L) * KS;
}

__device__ __forceinline__ float4 ldg4(const float *p) { return __ldg(reinterpret_cast<const float4 *>(p)); }

__device__ __forceinline__ void prefetch_bulk_l2(const void *p, unsigned bytes)
{
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

// Where tile `tile` of a grid with ncol tile columns lies: its first loaded
// row and column and its written columns [b0, b1).
struct TileGeom {
    int ybase, x0, b0, b1;
};

__device__ __forceinline__ TileGeom tile_geom(int tile, int ncol, int W, int N, int HK)
{
    const int ty = tile / ncol, tx = tile - ty * ncol, WQ = W >> 3;
    TileGeom g;
    g.b0 = 8 * ((tx * WQ) / ncol);
    g.b1 = 8 * (((tx + 1) * WQ) / ncol);
    g.x0 = g.b0 - 8;
    g.ybase = ty * N - HK;
    return g;
}

// Per-tile lane state: the quads' grid columns, ghost flags and weights.
template <int K, int L, int NQ>
__device__ __forceinline__ void tile_setup(RRState<K, L, NQ> &st, const TileGeom &g, int W, int H, const float *w32)
{
    st.ybase = g.ybase;
    st.H = H;
    st.w4 = w32[4];
    st.w3 = w32[3];
    st.w2 = w32[2];
    st.w1 = w32[1];
#pragma unroll
    for (int i = 0; i < NQ; i++) {
        const int x = g.x0 + 8 * (st.lane + 32 * i);
        st.act[i] = x >= 0 && x < W;
        st.eL[i] = x == 0;
        st.eR[i] = x + 8 == W;
        st.own[i] = x >= g.b0 && x < g.b1;
        const float wa = st.act[i] ? st.w4 : 0.f;
        st.waa[i] = make_float2(wa, wa);
        st.wla[i] = make_float2(st.eL[i] ? st.w3 : wa, wa);
        st.war[i] = make_float2(wa, st.eR[i] ? st.w3 : wa);
    }
}

// e of the tile's rows into registers and -r32 into the shared planes (zero
// outside the grid), then the warps' edge rows.
template <int K, int L, int NQ>
__device__ __forceinline__ void tile_load(RRState<K, L, NQ> &st, float *rp, const TileGeom &g,
                                          const float *__restrict__ ein, const float *__restrict__ r32, int H,
                                          int ld)
{
    constexpr int KS = RRState<K, L, NQ>::KS, R = kRRWarps * L;
#pragma unroll
    for (int j = 0; j < L; j++) {
        const int lr = st.w * L + j, y = st.ybase + lr, par = y & 1;
#pragma unroll
        for (int i = 0; i < NQ; i++) {
            const int qi = st.lane + 32 * i;
            float4 A = make_float4(0.f, 0.f, 0.f, 0.f), B = A, RA = A, RB = A;
            if (y >= 0 && y < H && st.act[i]) {
                const size_t p = (size_t)y * ld + g.x0 + 8 * qi;
                A = ldg4(ein + p);
                B = ldg4(ein + p + 4);
                RA = ldg4(r32 + p);
                RB = ldg4(r32 + p + 4);
            }
            // colour c holds the cells at offsets ((y & 1) ^ c) + 2 t
            const float4 ev = make_float4(A.x, A.z, B.x, B.z), od = make_float4(A.y, A.w, B.y, B.w);
            const float4 rev = make_float4(-RA.x, -RA.z, -RB.x, -RB.z);
            const float4 rod = make_float4(-RA.y, -RA.w, -RB.y, -RB.w);
            st.e[0][j][i] = par ? od : ev;
            st.e[1][j][i] = par ? ev : od;
            reinterpret_cast<float4 *>(rp + (size_t)lr * KS)[qi] = par ? rod : rev;
            reinterpret_cast<float4 *>(rp + (size_t)(R + lr) * KS)[qi] = par ? rev : rod;
        }
    }
    st.template put_edges<0>();
    st.template put_edges<1>();
}

// Threads [0, 2R): one bulk L2 prefetch per row of e and r32 of a tile.
template <int L, int NQ>
__device__ __forceinline__ void tile_prefetch(const TileGeom &g, const float *ein, const float *r32, int W, int H,
                                              int ld)
{
    constexpr int R = kRRWarps * L, TW = 256 * NQ;
    if ((int)threadIdx.x >= 2 * R) return;
    const int y = g.ybase + ((int)threadIdx.x % R);
    const int xs = max(g.x0, 0), xe = min(g.x0 + TW, W);
    if (y >= 0 && y < H && xe > xs) {
        const float *src = ((int)threadIdx.x < R ? ein : r32) + (size_t)y * ld + xs;
        prefetch_bulk_l2(src, (unsigned)(xe - xs) * 4u);
    }
}

// kr sweeps on the loaded tile (a block barrier after every half sweep);
// TRACK: mx takes the largest update of the last sweep over the written cells.
template <int K, int L, int NQ, bool TRACK>
__device__ __forceinline__ void tile_sweeps(RRState<K, L, NQ> &st, int kr, float &mx)
{
    constexpr int HK = 2 * K, N = kRRWarps * L - 2 * HK;
    const int P = (st.ybase + st.w * L) & 1;
    for (int t = 0; t < kr; t++) {
        const int d = 2 * (kr - t) - 1;
        if (TRACK && t == kr - 1) {
            if (P) st.template half<0, 1, true>(HK - d, HK + N + d, &mx, HK, HK + N);
            else st.template half<0, 0, true>(HK - d, HK + N + d, &mx, HK, HK + N);
            __syncthreads();
            if (P) st.template half<1, 1, true>(HK - d + 1, HK + N + d - 1, &mx, HK, HK + N);
            else st.template half<1, 0, true>(HK - d + 1, HK + N + d - 1, &mx, HK, HK + N);
        } else {
            if (P) st.template half<0, 1>(HK - d, HK + N + d);
            else st.template half<0, 0>(HK - d, HK + N + d);
            __syncthreads();
            if (P) st.template half<1, 1>(HK - d + 1, HK + N + d - 1);
            else st.template half<1, 0>(HK - d + 1, HK + N + d - 1);
        }
        __syncthreads();
    }
}

// The tile's written rows and columns to eout.
template <int K, int L, int NQ>
__device__ __forceinline__ void tile_store(const RRState<K, L, NQ> &st, const TileGeom &g, float *__restrict__ eout,
                                           int H, int ld)
{
    constexpr int HK = 2 * K, N = kRRWarps * L - 2 * HK;
#pragma unroll
    for (int j = 0; j < L; j++) {
        const int lr = st.w * L + j, y = st.ybase + lr, par = y & 1;
        if (lr < HK || lr >= HK + N || y >= H) continue;
#pragma unroll
        for (int i = 0; i < NQ; i++) {
            if (!st.own[i]) continue;
            const float4 c0 = st.e[0][j][i], c1 = st.e[1][j][i];
            const float4 ev = par ? c1 : c0, od = par ? c0 : c1;
            const size_t p = (size_t)y * ld + g.x0 + 8 * (st.lane + 32 * i);
            *reinterpret_cast<float4 *>(eout + p) = make_float4(ev.x, od.x, ev.y, od.y);
            *reinterpret_cast<float4 *>(eout + p + 4) = make_float4(ev.z, od.z, ev.w, od.w);
        }
    }
}

template <int K, int L, int NQ>
__device__ __forceinline__ void tile_state_init(RRState<K, L, NQ> &st, const float *edge, const float *rp)
{
    st.lane = threadIdx.x & 31;
    st.w = threadIdx.x >> 5;
    st.R = kRRWarps * L;
    st.edge_s = (unsigned)__cvta_generic_to_shared(edge) + 16u * st.lane;
    st.r_s = (unsigned)__cvta_generic_to_shared(rp) + 16u * st.lane;
}

template <int K, int L, int NQ, bool TRACK>
__global__ void __launch_bounds__(kRRThreads, 1)
    k_sor_tile_rr(const float *__restrict__ ein, float *__restrict__ eout, const float *__restrict__ r32, Ctl *ctl,
                  SolveArgs a, int ncol, int nrow, int nsw, int out_idx)
{
    using S = RRState<K, L, NQ>;
    constexpr int HK = S::HK, KS = S::KS, N = kRRWarps * L - 2 * HK;
    static_assert(N > 0, "tile without interior rows");
    if (*(volatile const int *)&ctl->halt) return;
    const int kr = min(nsw, a.max_iter - *(volatile const int *)&ctl->sweeps);
    if (kr < 1) return;  // every CTA reads the same count
    extern __shared__ __align__(16) float smem_f[];
    float *edge = smem_f;
    float *rp = edge + (size_t)4 * kRRWarps * KS;
    const int W = a.W, H = a.H, ld = a.ld;

    S st;
    tile_state_init(st, edge, rp);
    float mx = 0.f;
    const int ntiles = ncol * nrow;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const TileGeom g = tile_geom(tile, ncol, W, N, HK);
        tile_setup(st, g, W, H, a.w32);
        __syncthreads();  // the previous tile's half sweeps are done with the edge rows and planes
        tile_load(st, rp, g, ein, r32, H, ld);
        if (tile + (int)gridDim.x < ntiles)
            tile_prefetch<L, NQ>(tile_geom(tile + (int)gridDim.x, ncol, W, N, HK), ein, r32, W, H, ld);
        __syncthreads();
        tile_sweeps<K, L, NQ, TRACK>(st, kr, mx);
        tile_store(st, g, eout, H, ld);
    }
    if (TRACK) {
        double v[1] = {(double)mx};
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
            end_of_sweep(ctl, a, kr);
        }
    }
}

// The job owning global tile `t` (tile0 ascending from 0).
__device__ __forceinline__ int tile_job(const TileJob *jobs, int njobs, int t)
{
    int lo = 0, hi = njobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (jobs[mid].tile0 <= t) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// One pass of up to nsw sweeps over the tiles of every job (grid) of a batch
// whose solve has not halted: pass parity `par` reads buffer ea (par 0) or
// eb and writes the other.  Each CTA copies the job table into shared memory
// and takes every job's sweeps for this pass from its control block at the
// start (the blocks change only at the end of the pass); the CTA that
// finishes last closes the pass of every job that ran (sweep count, sweep
// cap, ping-pong side) and resets `counter`.
template <int K, int L, int NQ>
__global__ void __launch_bounds__(kRRThreads, 1)
    k_sor_tile_batch(const TileJob *__restrict__ jobs_g, int njobs, int ntiles, int nsw, int par, unsigned *counter)
{
    using S = RRState<K, L, NQ>;
    constexpr int HK = S::HK, KS = S::KS, N = kRRWarps * L - 2 * HK;
    extern __shared__ __align__(16) float smem_f[];
    __shared__ bool s_last;
    float *edge = smem_f;
    float *rp = edge + (size_t)4 * kRRWarps * KS;
    TileJob *jobs = reinterpret_cast<TileJob *>(rp + (size_t)2 * kRRWarps * L * KS);
    int *s_kr = reinterpret_cast<int *>(jobs + njobs);
    {
        const int words = njobs * (int)(sizeof(TileJob) / 4);
        const int *src = reinterpret_cast<const int *>(jobs_g);
        int *dst = reinterpret_cast<int *>(jobs);
        for (int k = threadIdx.x; k < words; k += blockDim.x) dst[k] = __ldg(src + k);
        for (int j = threadIdx.x; j < njobs; j += blockDim.x) {
            const TileJob &J = jobs_g[j];
            const volatile Ctl *c = J.ctl;
            s_kr[j] = c->halt ? 0 : max(0, min(nsw, J.max_iter - c->sweeps));
        }
    }
    __syncthreads();
    S st;
    tile_state_init(st, edge, rp);
    float mx = 0.f;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int j = tile_job(jobs, njobs, tile);
        const int kr = s_kr[j];
        if (kr < 1) continue;
        const TileJob &J = jobs[j];
        const float *ein = par ? J.eb : J.ea;
        float *eout = par ? J.ea : J.eb;
        const TileGeom g = tile_geom(tile - J.tile0, J.ncol, J.W, N, HK);
        tile_setup(st, g, J.W, J.H, J.w32);
        __syncthreads();
        tile_load(st, rp, g, ein, J.r32, J.H, J.ld);
        const int nt = tile + (int)gridDim.x;
        if (nt < ntiles) {
            const TileJob &Jn = jobs[tile_job(jobs, njobs, nt)];
            tile_prefetch<L, NQ>(tile_geom(nt - Jn.tile0, Jn.ncol, Jn.W, N, HK), par ? Jn.eb : Jn.ea, Jn.r32, Jn.W,
                                 Jn.H, Jn.ld);
        }
        __syncthreads();
        tile_sweeps<K, L, NQ, false>(st, kr, mx);
        tile_store(st, g, eout, J.H, J.ld);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        s_last = atomicAdd(counter, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (s_last) {
        __threadfence();
        for (int j = threadIdx.x; j < njobs; j += blockDim.x) {
            if (s_kr[j] < 1) continue;
            volatile Ctl *c = jobs[j].ctl;
            c->stream_out = par ? 0 : 1;
            const int sw = c->sweeps + s_kr[j];
            c->sweeps = sw;
            if (sw >= jobs[j].max_iter) c->halt = 1;
        }
        if (threadIdx.x == 0) *counter = 0u;
        __threadfence();
    }
}
