// sor_stream2.cuh -- two exact red-black sweeps of the FP32 correction
// equation per pass over an HBM grid: the bulk-copy stream sweep of
// sor_stream.cuh, temporally blocked.  Included by solver.cu after
// sor_stream.cuh, inside its internal namespace.
//
// Block s owns the rows [y0, y1) of its stripe and streams down rows
// y0-4 .. y1+3 of the input buffer.  At step j (y = y0 - 3 + j) it updates
//   the red cells of row y      (first sweep: neighbours are input values),
//   the black cells of row y-1  (first sweep: first-sweep red neighbours),
//   the red cells of row y-2    (second sweep: first-sweep black neighbours),
//   the black cells of row y-3  (second sweep), and stores row y-3.
// The first sweep runs on rows [y0-3, y1+3) and the second on [y0-1, y1+1):
// the dependency cone of the stripe's rows, recomputed from the input with the
// owners' arithmetic, so the values are bit-identical to theirs and the
// stripes need no ordering among themselves.  The result equals two
// launches of k_sweep_tma.
//
// Per thread: G 4-cell groups (columns 4 G t ..), a register window of six
// rows (y-4 .. y+1), the input row's outer neighbours for the first red
// update, and the right-hand side rows y-3 .. y read from their ring slots.
// Horizontal neighbours of updated cells across threads go through a small
// shared array of each thread's first and last cell per updated row
// (double-buffered by step), so one block barrier per step suffices; those
// of the input row come from the adjacent lanes.  Stripes start on even rows,
// which makes every cell parity a compile-time constant of the step.
// Rows arrive by cp.async.bulk into two rings with one mbarrier per slot:
// the input ring (4 rows, filled 2 steps ahead) and the right-hand side ring
// (8 rows: a row is read in 4 consecutive steps, filled 4 steps ahead).
// Every wait is bounded; on timeout the block records PCD_TIMEOUT.
//
// With one sweep left before max_iter (read from the control block at entry,
// the same value in every block) the kernel runs the first sweep only and
// stores rows as their black update completes.  With TRACK the largest
// update of the pass's last sweep is kept (the max-update stop rule is then
// tested every second sweep).
constexpr int kE2 = 4;  // input ring rows
constexpr int kR2 = 8;  // right-hand side ring rows

// Dynamic shared memory of k_sweep2_tma for rows of wpad floats and T threads.
inline size_t tma2_smem_bytes(int wpad, int T)
{
    return (size_t)(kE2 + kR2) * wpad * sizeof(float) + (size_t)2 * 3 * T * 2 * sizeof(float) +
           (kE2 + kR2) * sizeof(unsigned long long);
}

// One step of the two-sweep pass (j = 6 i + P; window index of row y + d is
// (P + 1 + d) mod 6, the outer-neighbour buffer of the row loaded at step j
// is (P + 1) & 1).
template <int G, bool TRACK, int P>
__device__ __forceinline__ bool tma2_step(float4 (&Wn)[6][G], float (&edg)[2][2], float *es, float *rs, float *xb,
                                          unsigned long long *ebar, unsigned long long *rbar,
                                          const float *__restrict__ ein, float *__restrict__ eout,
                                          const float *__restrict__ rhs, int i, int nsteps, int y0, int y1, int W,
                                          int H, int ld, int wpad, int T, unsigned bytes, int e_last, int r_last,
                                          int col0, bool two, const float (&w)[5], long spin_limit, bool &ok, float &m)
{
    constexpr int wB1 = (P + 2) % 6, w0 = (P + 1) % 6, wA1 = P % 6, wA2 = (P + 5) % 6, wA3 = (P + 4) % 6,
                  wA4 = (P + 3) % 6;
    const int j = 6 * i + P;
    if (j >= nsteps) return true;
    const int y = y0 - 3 + j;
    const int tid = threadIdx.x;
    // input row y+1 (ring index j+2) into the window, with its outer neighbours
    {
        const int row = y + 1;
        float4 (&dst)[G] = Wn[wB1];
        float &lft = edg[(P + 1) & 1][0], &rgt = edg[(P + 1) & 1][1];
        if (row >= 0 && row <= e_last) {
            const int t = j + 2;
            if (ok && !mbar_wait(ebar + (t & (kE2 - 1)), (unsigned)((t / kE2) & 1), spin_limit)) ok = false;
            const float *src = es + (size_t)(t & (kE2 - 1)) * wpad;
#pragma unroll
            for (int k = 0; k < G; k++) dst[k] = *reinterpret_cast<const float4 *>(src + col0 + 4 * k);
            // outer neighbours from the adjacent lanes; the warp's end lanes
            // read theirs from the slot
            const int lane = tid & 31;
            lft = __shfl_up_sync(0xffffffffu, dst[G - 1].w, 1);
            rgt = __shfl_down_sync(0xffffffffu, dst[0].x, 1);
            if (lane == 0) lft = col0 > 0 ? src[col0 - 1] : 0.f;
            if (lane == 31) rgt = col0 + 4 * G < W ? src[col0 + 4 * G] : 0.f;
        } else {
#pragma unroll
            for (int k = 0; k < G; k++) dst[k] = make_float4(0.f, 0.f, 0.f, 0.f);
            lft = 0.f;
            rgt = 0.f;
        }
    }
    // first use of right-hand side row y (ring index j)
    if (y >= 0 && y <= r_last && ok && !mbar_wait(rbar + (j & (kR2 - 1)), (unsigned)((j / kR2) & 1), spin_limit))
        ok = false;
    __syncthreads();  // S_j
    if (tid == 0) {
        // refill: input ring index j+4 (slot of index j, read at step j-2) and
        // right-hand side ring index j+4 (slot of index j-4, last read at step j-1)
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        const int er = y0 + j, rr = y0 + 1 + j;
        if (er <= e_last) tma_row(es + (size_t)((j + 4) & (kE2 - 1)) * wpad, ein + (long)er * ld, bytes,
                                  ebar + ((j + 4) & (kE2 - 1)));
        if (rr <= r_last) tma_row(rs + (size_t)((j + 4) & (kR2 - 1)) * wpad, rhs + (long)rr * ld, bytes,
                                  rbar + ((j + 4) & (kR2 - 1)));
    }
    // column parity of the red cells of y, y-2 and the black cells of y-1,
    // y-3: y0 is even (the plan gives even stripe heights), so y & 1 =
    // (P + 1) & 1
    constexpr int par = (P + 1) & 1;
    // boundary cells [buffer][kind][first / last][thread]
    float *xw = xb + (size_t)(P & 1) * 3 * 2 * T;              // written at this step
    const float *xr = xb + (size_t)((P + 1) & 1) * 3 * 2 * T;  // written at step j-1
    const bool lo_ok = tid > 0, hi_ok = tid + 1 < T;
    auto rhs_row = [&](int jr, float4 (&r)[G]) {
        const float *src = rs + (size_t)(jr & (kR2 - 1)) * wpad;
#pragma unroll
        for (int k = 0; k < G; k++) r[k] = *reinterpret_cast<const float4 *>(src + col0 + 4 * k);
    };
    auto publish = [&](int kind, const float4 (&c)[G]) {
        xw[(size_t)(2 * kind) * T + tid] = c[0].x;
        xw[(size_t)(2 * kind + 1) * T + tid] = c[G - 1].w;
    };
    auto store = [&](int row, const float4 (&c)[G]) {
#pragma unroll
        for (int k = 0; k < G; k++) *reinterpret_cast<float4 *>(eout + (long)row * ld + col0 + 4 * k) = c[k];
    };
    float tm = 0.f;
    // 1. red cells of row y (first sweep)
    if (y >= max(y0 - 3, 0) && y <= min(y1 + 2, H - 1)) {
        float4 r[G];
        rhs_row(j, r);
        if (TRACK && !two && y >= y0 && y < y1)
            relax_row_groups<G, true>(Wn[w0], Wn[wA1], Wn[wB1], r, edg[P & 1][0], edg[P & 1][1], col0, y, W, H, par,
                                      w, m);
        else
            relax_row_groups<G, false>(Wn[w0], Wn[wA1], Wn[wB1], r, edg[P & 1][0], edg[P & 1][1], col0, y, W, H, par,
                                       w, tm);
        publish(0, Wn[w0]);
    }
    // 2. black cells of row y-1 (first sweep)
    const int y1b = y - 1;
    if (y1b >= max(y0 - 2, 0) && y1b <= min(y1 + 1, H - 1)) {
        float4 r[G];
        rhs_row(j - 1, r);
        const float lft = lo_ok ? xr[(size_t)1 * T + tid - 1] : 0.f;
        const float rgt = hi_ok ? xr[(size_t)0 * T + tid + 1] : 0.f;
        if (TRACK && !two && y1b >= y0 && y1b < y1)
            relax_row_groups<G, true>(Wn[wA1], Wn[wA2], Wn[w0], r, lft, rgt, col0, y1b, W, H, par, w, m);
        else
            relax_row_groups<G, false>(Wn[wA1], Wn[wA2], Wn[w0], r, lft, rgt, col0, y1b, W, H, par, w, tm);
        publish(1, Wn[wA1]);
        if (!two && y1b >= y0 && y1b < y1) store(y1b, Wn[wA1]);
    }
    if (!two) return false;
    // 3. red cells of row y-2 (second sweep)
    const int y2r = y - 2;
    if (y2r >= max(y0 - 1, 0) && y2r <= min(y1, H - 1)) {
        float4 r[G];
        rhs_row(j - 2, r);
        const float lft = lo_ok ? xr[(size_t)3 * T + tid - 1] : 0.f;
        const float rgt = hi_ok ? xr[(size_t)2 * T + tid + 1] : 0.f;
        if (TRACK && y2r >= y0 && y2r < y1)
            relax_row_groups<G, true>(Wn[wA2], Wn[wA3], Wn[wA1], r, lft, rgt, col0, y2r, W, H, par, w, m);
        else
            relax_row_groups<G, false>(Wn[wA2], Wn[wA3], Wn[wA1], r, lft, rgt, col0, y2r, W, H, par, w, tm);
        publish(2, Wn[wA2]);
    }
    // 4. black cells of row y-3 (second sweep); row y-3 is final
    const int y2b = y - 3;
    if (y2b >= max(y0, 0) && y2b <= min(y1 - 1, H - 1)) {
        float4 r[G];
        rhs_row(j - 3, r);
        const float lft = lo_ok ? xr[(size_t)5 * T + tid - 1] : 0.f;
        const float rgt = hi_ok ? xr[(size_t)4 * T + tid + 1] : 0.f;
        relax_row_groups<G, TRACK>(Wn[wA3], Wn[wA4], Wn[wA2], r, lft, rgt, col0, y2b, W, H, par, w, m);
        store(y2b, Wn[wA3]);
    }
    return false;
}

template <int G, bool TRACK>
__global__ void __launch_bounds__(kStreamThreadsMax, 1)
    k_sweep2_tma(const float *__restrict__ ein, float *__restrict__ eout, const float *__restrict__ rhs, Ctl *ctl,
                 SolveArgs a, int R, int out_idx, int wpad, long spin_limit)
{
    if (vol_load(&ctl->halt)) return;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    float *es = reinterpret_cast<float *>(smem_raw);
    float *rs = es + (size_t)kE2 * wpad;
    const int T = blockDim.x;
    float *xb = rs + (size_t)kR2 * wpad;
    unsigned long long *bar = reinterpret_cast<unsigned long long *>(xb + (size_t)2 * 3 * T * 2);
    unsigned long long *ebar = bar, *rbar = bar + kE2;

    const int W = a.W, H = a.H, ld = a.ld;
    const bool two = a.max_iter - *(volatile const int *)&ctl->sweeps >= 2;
    const int y0 = blockIdx.x * R, y1 = min(y0 + R, H);
    const int e_last = min(y1 + 3, H - 1), r_last = min(y1 + 2, H - 1);  // last rows the stripe reads
    const int nsteps = (y1 + 3) - (y0 - 3);                              // steps y = y0-3 .. y1+2
    const unsigned bytes = (unsigned)wpad * 4u;
    const int col0 = 4 * G * threadIdx.x;
    float w[5];
#pragma unroll
    for (int c = 0; c < 5; c++) w[c] = a.w32[c];

    if (threadIdx.x == 0) {
        for (int q = 0; q < kE2 + kR2; q++) mbar_init(bar + q, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        // first use of every slot; rows above the grid complete their phase
        // with a plain arrive so that slot parities follow the ring index
        for (int t = 0; t < kE2; t++) {
            const int row = y0 - 4 + t;
            if (row < 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(ebar + t)) : "memory");
            else if (row <= e_last) tma_row(es + (size_t)t * wpad, ein + (long)row * ld, bytes, ebar + t);
        }
        for (int t = 0; t < kE2; t++) {  // right-hand side ring indices 0..3 (rows y0-3 .. y0)
            const int row = y0 - 3 + t;
            if (row < 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(rbar + t)) : "memory");
            else if (row <= r_last) tma_row(rs + (size_t)t * wpad, rhs + (long)row * ld, bytes, rbar + t);
        }
    }
    __syncthreads();

    bool ok = true;
    float m = 0.f;
    float4 Wn[6][G];
    float edg[2][2];
    // window before step 0: rows y0-4 (index 0) and y0-3 (index 1) with the
    // outer neighbours of row y0-3 (for the red update at step 0)
#pragma unroll
    for (int c = 0; c < 6; c++)
#pragma unroll
        for (int k = 0; k < G; k++) Wn[c][k] = make_float4(0.f, 0.f, 0.f, 0.f);
    edg[0][0] = edg[0][1] = edg[1][0] = edg[1][1] = 0.f;
#pragma unroll
    for (int t = 0; t < 2; t++) {
        const int row = y0 - 4 + t;
        if (row >= 0 && row <= e_last) {
            if (ok && !mbar_wait(ebar + t, 0u, spin_limit)) ok = false;
            const float *src = es + (size_t)t * wpad;
#pragma unroll
            for (int k = 0; k < G; k++) Wn[t][k] = *reinterpret_cast<const float4 *>(src + col0 + 4 * k);
            if (t == 1) {
                edg[0][0] = col0 > 0 ? src[col0 - 1] : 0.f;
                edg[0][1] = col0 + 4 * G < W ? src[col0 + 4 * G] : 0.f;
            }
        }
    }
    for (int i = 0;; i++) {
#define PCD_TMA2_STEP(PP)                                                                                            \
    if (tma2_step<G, TRACK, PP>(Wn, edg, es, rs, xb, ebar, rbar, ein, eout, rhs, i, nsteps, y0, y1, W, H, ld, wpad,  \
                                T, bytes, e_last, r_last, col0, two, w, spin_limit, ok, m))                         \
        break;
        PCD_TMA2_STEP(0) PCD_TMA2_STEP(1) PCD_TMA2_STEP(2) PCD_TMA2_STEP(3) PCD_TMA2_STEP(4) PCD_TMA2_STEP(5)
#undef PCD_TMA2_STEP
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
            end_of_sweep(ctl, a, two ? 2 : 1);
        }
    }
}
