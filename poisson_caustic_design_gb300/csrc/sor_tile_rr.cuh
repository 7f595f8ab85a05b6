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

template <int K, int L, int NQ, bool TRACK>
__global__ void __launch_bounds__(kRRThreads, 1)
    k_sor_tile_rr(const float *__restrict__ ein, float *__restrict__ eout, const float *__restrict__ r32, Ctl *ctl,
                  SolveArgs a, int ncol, int nrow, int nsw, int out_idx)
{
    using S = RRState<K, L, NQ>;
    constexpr int HK = S::HK, KS = S::KS, R = kRRWarps * L, N = R - 2 * HK, TW = 256 * NQ;
    static_assert(N > 0, "tile without interior rows");
    if (*(volatile const int *)&ctl->halt) return;
    const int kr = min(nsw, a.max_iter - *(volatile const int *)&ctl->sweeps);
    if (kr < 1) return;  // every CTA reads the same count
    extern __shared__ __align__(16) float smem_f[];
    float *edge = smem_f;
    float *rp = edge + (size_t)4 * kRRWarps * KS;
    const int W = a.W, H = a.H, ld = a.ld, WQ = W >> 3;

    S st;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    st.lane = lane;
    st.w = w;
    st.H = H;
    st.R = R;
    st.edge_s = (unsigned)__cvta_generic_to_shared(edge) + 16u * lane;
    st.r_s = (unsigned)__cvta_generic_to_shared(rp) + 16u * lane;
    st.w4 = a.w32[4];
    st.w3 = a.w32[3];
    st.w2 = a.w32[2];
    st.w1 = a.w32[1];
    float mx = 0.f;
    const int ntiles = ncol * nrow;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int ty = tile / ncol, tx = tile - ty * ncol;
        const int b0 = 8 * ((tx * WQ) / ncol), b1 = 8 * (((tx + 1) * WQ) / ncol), x0 = b0 - 8;
        st.ybase = ty * N - HK;
#pragma unroll
        for (int i = 0; i < NQ; i++) {
            const int x = x0 + 8 * (lane + 32 * i);
            st.act[i] = x >= 0 && x < W;
            st.eL[i] = x == 0;
            st.eR[i] = x + 8 == W;
            st.own[i] = x >= b0 && x < b1;
            const float wa = st.act[i] ? st.w4 : 0.f;
            st.waa[i] = make_float2(wa, wa);
            st.wla[i] = make_float2(st.eL[i] ? st.w3 : wa, wa);
            st.war[i] = make_float2(wa, st.eR[i] ? st.w3 : wa);
        }
        __syncthreads();  // the previous tile's half sweeps are done with the edge rows and planes
        // e (registers) and -r32 (shared) of the tile's rows; zero outside the grid
#pragma unroll
        for (int j = 0; j < L; j++) {
            const int lr = w * L + j, y = st.ybase + lr, par = y & 1;
#pragma unroll
            for (int i = 0; i < NQ; i++) {
                const int qi = lane + 32 * i;
                float4 A = make_float4(0.f, 0.f, 0.f, 0.f), B = A, RA = A, RB = A;
                if (y >= 0 && y < H && st.act[i]) {
                    const size_t p = (size_t)y * ld + x0 + 8 * qi;
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
        // the next tile's rows of e and r32 into L2 (one bulk prefetch per row and array)
        const int nt = tile + (int)gridDim.x;
        if (nt < ntiles && (int)threadIdx.x < 2 * R) {
            const int nty = nt / ncol, ntx = nt - nty * ncol;
            const int nb0 = 8 * ((ntx * WQ) / ncol);
            const int y = nty * N - HK + ((int)threadIdx.x % R);
            const int xs = max(nb0 - 8, 0), xe = min(nb0 - 8 + TW, W);
            if (y >= 0 && y < H && xe > xs) {
                const float *src = ((int)threadIdx.x < R ? ein : r32) + (size_t)y * ld + xs;
                prefetch_bulk_l2(src, (unsigned)(xe - xs) * 4u);
            }
        }
        st.template put_edges<0>();
        st.template put_edges<1>();
        __syncthreads();
        const int P = (st.ybase + w * L) & 1;
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
        // the tile's own rows and columns to the other buffer
#pragma unroll
        for (int j = 0; j < L; j++) {
            const int lr = w * L + j, y = st.ybase + lr, par = y & 1;
            if (lr < HK || lr >= HK + N || y >= H) continue;
#pragma unroll
            for (int i = 0; i < NQ; i++) {
                if (!st.own[i]) continue;
                const float4 c0 = st.e[0][j][i], c1 = st.e[1][j][i];
                const float4 ev = par ? c1 : c0, od = par ? c0 : c1;
                const size_t p = (size_t)y * ld + x0 + 8 * (lane + 32 * i);
                *reinterpret_cast<float4 *>(eout + p) = make_float4(ev.x, od.x, ev.y, od.y);
                *reinterpret_cast<float4 *>(eout + p + 4) = make_float4(ev.z, od.z, ev.w, od.w);
            }
        }
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
