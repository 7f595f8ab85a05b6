// nn_tc.cu -- the U-Net's BF16 GEMM on the 5th-generation tensor cores
// (tcgen05, sm_103a).
//
// C[M x N] = A[M x K] * B[N x K]^T, FP32 accumulation in tensor memory.  The
// operands come in by TMA (cp.async.bulk.tensor) with the 128-byte swizzle
// (64-byte for 32-wide tiles), as
//   * K-major 2-D tiles (A, B row-major with K contiguous: "TN", the layout of
//     nn::gemm),
//   * MN-major 2-D tiles (an operand stored K rows x M or N contiguous: the
//     weight gradient reads the activations and dY where they lie),
//   * implicit 3x3 convolution tiles: 4-D boxes (channels x columns x rows x
//     images) of the NHWC input at each tap's shift, the coordinates outside
//     the image zero-filled by TMA, which is the convolution's padding -- the
//     im2col matrix is never formed (forward and data gradient as K-major A,
//     weight gradient as MN-major A);
// and one elected thread issues tcgen05.mma.cta_group::1.kind::f16 (M = 128,
// N = BN, K = 16 per instruction) on shared memory descriptors.  The kernel
// (k_gemm_tcp, described above it) is persistent and warp-specialised: a TMA
// warp, an MMA warp and four epilogue warps, two accumulators in tensor
// memory so that a tile's epilogue overlaps the next tile's loads and MMAs.
// The epilogue reads the accumulator with tcgen05.ld.32x32b and applies
// nn::gemm's (bias, ReLU, BF16 or FP32 store, FP32 split-K partials, or a
// transposed store).  Every mbarrier wait is bounded: a wait that runs out
// records PCD_TIMEOUT in an error word, the CTA stops issuing, waits
// (bounded) for what it has in flight and frees its tensor memory.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <mutex>

#include "nn.cuh"

namespace pcd {
namespace nn {

namespace {

constexpr int kTcBM = 128, kTcBK = 64;
constexpr long long kTcSpin = 1ll << 24;

__device__ __forceinline__ unsigned tc_smem(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

// Bounded wait for phase `parity` of the barrier: true once it completed,
// false when the poll budget ran out.
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity)
{
    for (long long it = 0; it < kTcSpin; it++) {
        unsigned done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void tma_load_2d(unsigned dst, const CUtensorMap *map, unsigned bar, int x, int y)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];"
        ::"r"(dst), "l"(map), "r"(bar), "r"(x), "r"(y)
        : "memory");
}

__device__ __forceinline__ void tma_load_4d(unsigned dst, const CUtensorMap *map, unsigned bar, int c0, int c1, int c2,
                                            int c3)
{
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5, %6}], "
        "[%2];" ::"r"(dst),
        "l"(map), "r"(bar), "r"(c0), "r"(c1), "r"(c2), "r"(c3)
        : "memory");
}

// Shared memory descriptor: start address >> 4 (bits 0-13), leading byte
// offset >> 4 (bits 16-29), stride byte offset >> 4 (bits 32-45), descriptor
// version 1 (bits 46-47), swizzle mode (bits 61-63: 2 = 128-byte, 4 = 64-byte).
__device__ __forceinline__ unsigned long long smem_desc(unsigned addr, unsigned lbo, unsigned sbo, unsigned mode)
{
    return (unsigned long long)((addr & 0x3FFFFu) >> 4) | ((unsigned long long)((lbo >> 4) & 0x3FFFu) << 16) |
           ((unsigned long long)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46) | ((unsigned long long)mode << 61);
}

// Operand tiles as TMA lays them down with the 128-byte swizzle (and, for a
// 32-wide MN-major tile, the 64-byte swizzle), and the descriptor of the
// 16-deep K slice kk:
//   K-major: rows of 64 K values (128 bytes), 8-row atoms 1024 bytes apart
//     (stride offset); the leading offset is unused for this layout (encoded
//     1); slice kk starts 32 bytes further inside the atom;
//   MN-major: rows of 64 M (or N) values, one row per K index; 8-row atoms
//     along K 1024 bytes apart (stride offset), 64-wide MN blocks of 64 rows
//     8192 bytes apart (leading offset); slice kk starts 16 rows (2048 bytes)
//     further.  32-wide (64-byte swizzle): 512-byte atoms, 1024 bytes a slice.
__device__ __forceinline__ unsigned long long desc_kmajor(unsigned tile, int kk)
{
    return smem_desc(tile + 32u * kk, 16u, 1024u, 2u);
}

// K-major with the 64-byte swizzle (32 K values a row): 512-byte atoms
__device__ __forceinline__ unsigned long long desc_kmajor_sw64(unsigned tile, int kk)
{
    return smem_desc(tile + 32u * kk, 16u, 512u, 4u);
}

__device__ __forceinline__ unsigned long long desc_mnmajor(unsigned tile, int kk, int width)
{
    return width == 32 ? smem_desc(tile + 1024u * kk, 4096u, 512u, 4u) : smem_desc(tile + 2048u * kk, 8192u, 1024u, 2u);
}

// Instruction descriptor of kind::f16: D FP32 (bits 4-5 = 1), A and B BF16
// (bits 7-9 = 1, 10-12 = 1), A and B major-ness (bits 15, 16: 0 K-major,
// 1 MN-major), N >> 3 in bits 17-22, M >> 4 in bits 24-28.
__host__ __device__ constexpr unsigned idesc_bf16_f32(int M, int N, int a_mn = 0, int b_mn = 0)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((unsigned)a_mn << 15) | ((unsigned)b_mn << 16) |
           ((unsigned)(N >> 3) << 17) | ((unsigned)(M >> 4) << 24);
}

// First pixel p0 of a tile -> (image, row, column)
__device__ __forceinline__ void pixel_of(const GemmArgs &g, int p0, int &b0, int &y0, int &x0)
{
    const int hw = g.xh * g.xw;
    b0 = p0 / hw;
    const int r = p0 - b0 * hw;
    y0 = r / g.xw;
    x0 = r - y0 * g.xw;
}

// One stage's loads: A (128 rows of M) and B (BN rows of N) for K tile kt.
// A K-major operand is one box of 64 K columns; an MN-major operand is one
// box of 64 K rows per 64 (or 32) columns of M / N, 8192 bytes apart.  An
// implicit convolution operand is one 4-D box of the input (channels x
// columns x rows x images) at the tile's pixels shifted by the tap, the
// coordinates outside the image reading zeros (the convolution's padding):
// conv = 1, 128 pixels x cwid channels for (tap, chunk) = K tile kt, and the
// weights' cwid columns of that tap and chunk; conv = 2, for each cwid-wide M
// block of the tile (one tap and chunk) 64 pixels (K tile kt) x cwid channels.
template <int BN>
__device__ __forceinline__ void load_stage(unsigned st, unsigned stB, const CUtensorMap *mA, const CUtensorMap *mB,
                                           unsigned bar, const GemmArgs &g, int kt, int bm, int bn)
{
    const int k0 = kt * kTcBK;
    if (g.conv == 1) {
        const int t = kt / g.nch, j = kt - t * g.nch;
        int b0, y0, x0;
        pixel_of(g, bm, b0, y0, x0);
        tma_load_4d(st, mA, bar, j * g.cwid, x0 + t % 3 - 1, y0 + t / 3 - 1, b0);
        tma_load_2d(stB, mB, bar, t * g.xc + j * g.cwid, bn);
        return;
    }
    if (g.conv == 2) {
        int b0, y0, x0;
        pixel_of(g, k0, b0, y0, x0);
        for (int i = 0; i < kTcBM / g.cwid; i++) {
            const int mb = bm / g.cwid + i, t = mb / g.nch, j = mb - t * g.nch;
            tma_load_4d(st + (unsigned)(i * 64 * g.cwid * 2), mA, bar, j * g.cwid, x0 + t % 3 - 1, y0 + t / 3 - 1, b0);
        }
    } else if (g.a_mn) {
        tma_load_2d(st, mA, bar, bm, k0);
        tma_load_2d(st + 8192u, mA, bar, bm + 64, k0);
    } else {
        tma_load_2d(st, mA, bar, k0, bm);
    }
    if (g.b_mn) {
#pragma unroll
        for (int c = 0; c < (BN < 64 ? 1 : BN / 64); c++) tma_load_2d(stB + 8192u * c, mB, bar, bn + 64 * c, k0);
    } else {
        tma_load_2d(stB, mB, bar, k0, bn);
    }
}

__device__ __forceinline__ void mma_bf16_tc(unsigned tmem_d, unsigned long long a, unsigned long long b, unsigned idesc,
                                            unsigned accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(tmem_d), "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void mma_commit(unsigned bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

// Row of a transposed C for accumulator row m: m itself, or for the weight
// gradient (conv = 2) tap * xc + c of the M block's tap and channel; false
// for rows past M and for the padding channels of a partial chunk.
__device__ __forceinline__ bool out_row(const GemmArgs &g, int m, int &row)
{
    if (g.conv != 2) {
        row = m;
        return m < g.M;
    }
    const int mb = m / g.cwid, t = mb / g.nch, j = mb - t * g.nch, c = j * g.cwid + (m - mb * g.cwid);
    row = t * g.xc + c;
    return m < g.M && t < 9 && c < g.xc;
}

// ---------------------------------------------------------------------------
// The persistent form: one CTA per SM (two for N tiles up to 64) walks the
// output tiles (units of 128 x BN x one K share, M fastest so that CTAs
// running together share B), with three roles so that nothing waits for a
// tile's end:
//   warp 0 (one lane): TMA producer over a ring of nst stages, running ahead
//     across unit boundaries (waits: the stage's empty barrier);
//   warp 1 (one lane): MMA issuer into one of two tensor-memory accumulators
//     (2 x BN columns), alternating per unit; commits free each stage and,
//     after a unit's last K tile, signal its accumulator full (waits: the
//     stage's full barrier, the accumulator's empty barrier);
//   warps 2-5: epilogue; warp w reads accumulator lanes 32 (w % 4) + [0, 32)
//     (the quarter its warp slot may access), stores the rows (or, for a
//     transposed C, the columns) and releases the accumulator (one arrive
//     per warp; the barrier counts 4).
// The epilogue of one unit overlaps the loads and MMAs of the next.  Every
// wait is bounded: the first to run out records PCD_TIMEOUT and raises a
// shared abort flag that the other roles' loops test; before freeing tensor
// memory the CTA waits (bounded) for its MMAs and its last loads.
constexpr int kTpThreads = 192, kTpMaxStages = 12;
constexpr unsigned kTpStageBytes = 4u * 32u * 33u * 4u;  // epilogue: a [32][33] float tile per warp

// CTAs per SM: two for N tiles up to 64 (their units are short; two CTAs
// hide each other's unit boundaries), else one; and the stage ring's share
// of shared memory (227 KB per SM less the epilogue tiles and slack).
__host__ __device__ constexpr int tp_ctas_per_sm(int BN) { return BN <= 64 ? 2 : 1; }
__host__ __device__ constexpr unsigned tp_ring_budget(int BN)
{
    return (227u * 1024u) / (unsigned)tp_ctas_per_sm(BN) - kTpStageBytes - 2048u;
}

__host__ __device__ inline unsigned tp_stage_a(const GemmArgs &g)
{
    return (g.conv == 1 && g.cwid == 32) ? kTcBM * 32 * 2 : kTcBM * kTcBK * 2;
}

__host__ __device__ inline unsigned tp_stage_b(const GemmArgs &g, int BN)
{
    return (unsigned)BN * ((g.conv == 1 && g.cwid == 32) ? 32u : (unsigned)kTcBK) * 2u;
}

__host__ __device__ inline unsigned tp_stride(const GemmArgs &g, int BN)
{
    return (tp_stage_a(g) + tp_stage_b(g, BN) + 1023u) & ~1023u;
}

__device__ __forceinline__ void mbar_arrive(unsigned bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

template <int BN>
__global__ void __launch_bounds__(kTpThreads, tp_ctas_per_sm(BN))
    k_gemm_tcp(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB, GemmArgs g, int nst,
               int *err)
{
    static_assert(BN == 32 || BN == 64 || BN == 128 || BN == 256, "N tile");
    constexpr int kCols = 2 * BN;  // two accumulators (a power of 2, >= 64)
    extern __shared__ __align__(1024) unsigned char tc_buf[];
    __shared__ __align__(8) unsigned long long bars[2 * kTpMaxStages + 5];
    __shared__ unsigned tmem_base;
    __shared__ volatile int s_abort;
    __shared__ int s_fills[kTpMaxStages];  // loads issued per stage (producer)

    const unsigned raw = tc_smem(tc_buf);
    const unsigned ring = (raw + 1023u) & ~1023u;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const bool k32 = g.conv == 1 && g.cwid == 32;
    const unsigned aBytes = tp_stage_a(g), tx = aBytes + tp_stage_b(g, BN), sstride = tp_stride(g, BN);
    const int MT = (g.M + kTcBM - 1) / kTcBM, NT = (g.N + BN - 1) / BN;
    const int units = MT * NT * g.ksplit;
    const int KT = g.conv == 1 ? 9 * g.nch : (g.K + kTcBK - 1) / kTcBK;
    const int per = (KT + g.ksplit - 1) / g.ksplit;
    const unsigned bar0 = tc_smem(&bars[0]);
    auto full = [&](int s) { return bar0 + 8u * s; };
    auto empty = [&](int s) { return bar0 + 8u * (kTpMaxStages + s); };
    auto tfull = [&](int a) { return bar0 + 8u * (2 * kTpMaxStages + a); };
    auto tempty = [&](int a) { return bar0 + 8u * (2 * kTpMaxStages + 2 + a); };
    const unsigned drain = bar0 + 8u * (2 * kTpMaxStages + 4);
    auto fail = [&]() {
        atomicCAS(err, 0, PCD_TIMEOUT);
        s_abort = 1;
    };

    if (threadIdx.x == 0) {
        s_abort = 0;
        for (int s = 0; s < nst; s++) {
            s_fills[s] = 0;
            mbar_init(full(s), 1);
            mbar_init(empty(s), 1);
        }
        for (int a = 0; a < 2; a++) {
            mbar_init(tfull(a), 1);
            mbar_init(tempty(a), 4);
        }
        mbar_init(drain, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"(&mapA) : "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"(&mapB) : "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc_smem(&tmem_base)),
                     "r"(kCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const unsigned tmem = tmem_base;

    if (warp == 0) {
        if (lane == 0) {
            int it = 0;
            for (int u = blockIdx.x; u < units && !s_abort; u += gridDim.x) {
                const int mt = u % MT, r = u / MT, nt = r % NT, z = r / NT;
                const int k0 = z * per, nk = max(0, min(KT, k0 + per) - k0);
                for (int i = 0; i < nk; i++, it++) {
                    const int s = it % nst, round = it / nst;
                    if (round > 0 && !mbar_wait(empty(s), (unsigned)((round - 1) & 1))) {
                        fail();
                        break;
                    }
                    if (s_abort) break;
                    const unsigned st = ring + (unsigned)s * sstride;
                    mbar_expect_tx(full(s), tx);
                    load_stage<BN>(st, st + aBytes, &mapA, &mapB, full(s), g, k0 + i, mt * kTcBM, nt * BN);
                    s_fills[s]++;
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            const unsigned idesc = idesc_bf16_f32(kTcBM, BN, g.a_mn, g.b_mn);
            int it = 0, lu = 0;
            for (int u = blockIdx.x; u < units && !s_abort; u += gridDim.x, lu++) {
                const int r = u / MT, z = r / NT;
                const int k0 = z * per, nk = max(0, min(KT, k0 + per) - k0);
                const int a = lu & 1, use = lu >> 1;
                if (use > 0 && !mbar_wait(tempty(a), (unsigned)((use - 1) & 1))) {
                    fail();
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const unsigned acc = tmem + (unsigned)(a * BN);
                for (int i = 0; i < nk && !s_abort; i++, it++) {
                    const int s = it % nst, round = it / nst;
                    if (!mbar_wait(full(s), (unsigned)(round & 1))) {
                        fail();
                        break;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const unsigned sa = ring + (unsigned)s * sstride, sb = sa + aBytes;
#pragma unroll
                    for (int kk = 0; kk < kTcBK / 16; kk++) {
                        if (k32 && kk >= 2) break;
                        const unsigned long long da = k32         ? desc_kmajor_sw64(sa, kk)
                                                      : g.conv == 2 ? desc_mnmajor(sa, kk, g.cwid)
                                                      : g.a_mn      ? desc_mnmajor(sa, kk, 64)
                                                                    : desc_kmajor(sa, kk);
                        const unsigned long long db = k32    ? desc_kmajor_sw64(sb, kk)
                                                      : g.b_mn ? desc_mnmajor(sb, kk, BN < 64 ? BN : 64)
                                                               : desc_kmajor(sb, kk);
                        mma_bf16_tc(acc, da, db, idesc, (i > 0 || kk > 0) ? 1u : 0u);
                    }
                    mma_commit(empty(s));
                }
                if (s_abort) break;
                mma_commit(tfull(a));  // arrives once this unit's MMAs are done (at once when it had none)
            }
        }
    } else {
        const int q = warp & 3;  // the accumulator lane quarter this warp may read
        float *tile = reinterpret_cast<float *>(tc_buf + (ring - raw) + (size_t)nst * sstride) + (warp - 2) * 32 * 33;
        int lu = 0;
        for (int u = blockIdx.x; u < units; u += gridDim.x, lu++) {
            const int mt = u % MT, r = u / MT, nt = r % NT, z = r / NT;
            const int k0 = z * per, nk = max(0, min(KT, k0 + per) - k0);
            const int a = lu & 1, use = lu >> 1;
            const bool ok = __all_sync(0xffffffffu, s_abort == 0 && mbar_wait(tfull(a), (unsigned)(use & 1)));
            if (!ok) {
                if (lane == 0) fail();
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const int m = mt * kTcBM + q * 32 + lane;
            for (int c0 = 0; c0 < BN; c0 += 32) {
                unsigned v[32];
                if (nk > 0) {
                    const unsigned addr = tmem + ((unsigned)(q * 32) << 16) + (unsigned)(a * BN + c0);
                    asm volatile(
                        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,"
                        "%15}, [%16];"
                        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
                          "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
                          "=r"(v[14]), "=r"(v[15])
                        : "r"(addr));
                    asm volatile(
                        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,"
                        "%15}, [%16];"
                        : "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]),
                          "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]),
                          "=r"(v[30]), "=r"(v[31])
                        : "r"(addr + 16u));
                    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                } else {
#pragma unroll
                    for (int j = 0; j < 32; j++) v[j] = 0u;  // an empty K share: zero partials
                }
                const int n0 = nt * BN + c0;
                if (g.trans_c) {
                    int row = 0;
                    if (out_row(g, m, row)) {
                        float *base = g.Cf + (g.ksplit > 1 ? (size_t)z * g.N * g.ldc : 0);
#pragma unroll
                        for (int j = 0; j < 32; j++)
                            if (n0 + j < g.N) base[(size_t)(n0 + j) * g.ldc + row] = __uint_as_float(v[j]);
                    }
                    continue;
                }
                // through the warp's shared tile: lane l then stores column
                // n0 + l of the warp's 32 rows, a row per instruction
#pragma unroll
                for (int jj = 0; jj < 32; jj++) tile[lane * 33 + jj] = __uint_as_float(v[jj]);
                __syncwarp();
                const int n = n0 + lane;
                if (n < g.N) {
                    const float bias = (g.ksplit == 1 && g.bias) ? g.bias[n] : 0.f;
                    for (int rr = 0; rr < 32; rr++) {
                        const int row = mt * kTcBM + q * 32 + rr;
                        if (row >= g.M) break;
                        float x = tile[rr * 33 + lane];
                        if (g.ksplit > 1) {
                            g.Cf[((size_t)z * g.M + row) * g.ldc + n] = x;
                            continue;
                        }
                        x += bias;
                        if (g.relu) x = fmaxf(x, 0.f);
                        if (g.Cb) g.Cb[(size_t)row * g.ldc + n] = __float2bfloat16(x);
                        else g.Cf[(size_t)row * g.ldc + n] = x;
                    }
                }
                __syncwarp();
            }
            // release the accumulator: every lane's loads have completed
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(tempty(a));
        }
    }

    __syncthreads();
    if (s_abort) {
        // let what is in flight land before the tensor memory and the shared
        // memory go away: every MMA issued (a last commit), every stage's
        // latest load (bounded waits)
        if (warp == 1 && lane == 0) {
            mma_commit(drain);
            (void)mbar_wait(drain, 0u);
        }
        if (warp == 0 && lane == 0)
            for (int s = 0; s < nst; s++)
                if (s_fills[s] > 0) (void)mbar_wait(full(s), (unsigned)((s_fills[s] - 1) & 1));
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kCols) : "memory");
    }
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against the driver library).
PFN_cuTensorMapEncodeTiled_v12000 encode_fn()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}

// A 2-D tensor map of a rows x cols BF16 matrix (row stride ld elements) with
// a box of box_rows x box_cols (box_cols of 64: the 128-byte swizzle; of 32:
// the 64-byte swizzle).
int make_map(CUtensorMap *map, const void *base, int rows, int cols, int ld, int box_rows, int box_cols = kTcBK)
{
    auto fn = encode_fn();
    if (!fn) {
        set_error("tcgen05 gemm: cuTensorMapEncodeTiled is not available");
        return PCD_DEVICE_ERROR;
    }
    const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
    const cuuint32_t box[2] = {(cuuint32_t)box_cols, (cuuint32_t)box_rows};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), dims, strides, box, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE,
                          box_cols == 32 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_128B,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error("tcgen05 gemm: cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
        return PCD_DEVICE_ERROR;
    }
    return PCD_OK;
}

// The box of T consecutive pixels of an H x W image batch: (columns, rows,
// images) = (T, 1, 1) for W a multiple of T, (W, T / W, 1) for W < T with T
// rows of W dividing H, (W, H, T / (W H)) for whole images; false when the
// sizes tile no other way (powers of two always do).
bool conv_box(int W, int H, int T, int box[3])
{
    if (W <= 0 || H <= 0) return false;
    if (W >= T) {
        if (W % T) return false;
        box[0] = T, box[1] = 1, box[2] = 1;
        return true;
    }
    if (T % W) return false;
    const int rows = T / W;
    if (H >= rows) {
        if (H % rows) return false;
        box[0] = W, box[1] = rows, box[2] = 1;
    } else {
        if (rows % H) return false;
        box[0] = W, box[1] = H, box[2] = rows / H;
    }
    return true;
}

// A 4-D tensor map of an NHWC BF16 activation (C channels at pixel stride ldx
// elements; B images of H x W) with a box of cwid channels x the T-pixel box
// of conv_box (the 128-byte swizzle for 64 channels, the 64-byte for 32).
int make_map4(CUtensorMap *map, const void *base, int C, int W, int H, int B, int ldx, int cwid, int T)
{
    auto fn = encode_fn();
    if (!fn) {
        set_error("tcgen05 conv: cuTensorMapEncodeTiled is not available");
        return PCD_DEVICE_ERROR;
    }
    int bx[3];
    if (!conv_box(W, H, T, bx)) {
        set_error("tcgen05 conv: the image size does not tile into boxes of " + std::to_string(T) + " pixels");
        return PCD_BAD_ARG;
    }
    const cuuint64_t dims[4] = {(cuuint64_t)C, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)B};
    const cuuint64_t strides[3] = {(cuuint64_t)ldx * 2, (cuuint64_t)ldx * 2 * W, (cuuint64_t)ldx * 2 * W * H};
    const cuuint32_t box[4] = {(cuuint32_t)cwid, (cuuint32_t)bx[0], (cuuint32_t)bx[1], (cuuint32_t)bx[2]};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    const CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void *>(base), dims, strides, box, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE,
                          cwid == 32 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_128B,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error("tcgen05 conv: cuTensorMapEncodeTiled (4-D) failed (" + std::to_string((int)r) + ")");
        return PCD_DEVICE_ERROR;
    }
    return PCD_OK;
}

// One error word per device: a kernel that gives up a bounded wait writes a
// nonzero code there.
int *err_word()
{
    constexpr int kMaxDev = 64;
    static int *w[kMaxDev] = {};
    static std::mutex mu;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDev) return nullptr;
    std::lock_guard<std::mutex> lk(mu);
    if (!w[dev] && cudaMalloc(&w[dev], sizeof(int)) == cudaSuccess) cudaMemset(w[dev], 0, sizeof(int));
    return w[dev];
}

template <int BN>
int tcp_attr()
{
    static std::mutex mu;
    static unsigned long long done_mask = 0;
    int dev = 0;
    PCD_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(mu);
    if (dev < 64 && (done_mask >> dev & 1ull)) return PCD_OK;
    PCD_CUDA(cudaFuncSetAttribute(k_gemm_tcp<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)(tp_ring_budget(BN) + kTpStageBytes + 1024u)));
    if (dev < 64) done_mask |= 1ull << dev;
    return PCD_OK;
}

template <int BN>
int launch_tcp(const CUtensorMap &ma, const CUtensorMap &mb, const GemmArgs &g, cudaStream_t s, int *err)
{
    PCD_TRY(tcp_attr<BN>());
    const unsigned stride = tp_stride(g, BN);
    const int nst = (int)std::min<unsigned>(kTpMaxStages, tp_ring_budget(BN) / stride);
    const size_t smem = (size_t)nst * stride + kTpStageBytes + 1024;
    const long units = (long)((g.M + kTcBM - 1) / kTcBM) * ((g.N + BN - 1) / BN) * g.ksplit;
    const int grid = (int)std::max<long>(1, std::min<long>(units, (long)tp_ctas_per_sm(BN) * sm_count()));
    k_gemm_tcp<BN><<<grid, kTpThreads, smem, s>>>(ma, mb, g, nst, err);
    PCD_LAUNCHED(1);
    return PCD_OK;
}

}  // namespace

bool conv_tc_applies(const void *x, int B, int H, int W, int C, int ldx, int T)
{
    // every box dimension within the tensor's (a box of more images than the
    // batch holds is not formed)
    int box[3];
    return x && ((uintptr_t)x % 16) == 0 && B >= 1 && C >= 32 && C % 8 == 0 && ldx >= C && ldx % 8 == 0 &&
           conv_box(W, H, T, box) && box[2] <= B;
}

bool gemm_tc_applies(const GemmArgs &g)
{
    if (g.conv == 1 || g.conv == 2) {
        const int cw = g.xc == 32 ? 32 : 64;
        const long P = (long)g.xb * g.xh * g.xw;
        if (g.cwid != cw || g.nch != (g.xc + cw - 1) / cw || P > (1L << 30) ||
            !conv_tc_applies(g.A, g.xb, g.xh, g.xw, g.xc, g.lda, g.conv == 1 ? kTcBM : kTcBK))
            return false;
        if (g.conv == 1)
            return g.M == P && g.K == 9 * g.xc && !g.a_mn && !g.b_mn && ((uintptr_t)g.B % 16) == 0 && g.ldb % 8 == 0;
        return g.M == 9 * g.nch * g.cwid && g.K == P && g.trans_c && g.b_mn && ((uintptr_t)g.B % 16) == 0 &&
               g.N >= (g.N <= 32 ? 32 : 64);
    }
    if (g.conv != 0) return false;
    // TMA: 16-byte aligned bases and row strides (ld multiples of 8, checked
    // by gemm); at least one 64-wide K tile; an MN-major operand at least as
    // wide as its box (64 columns; 32 for a 32-wide B)
    if (g.a_mn && g.M < 64) return false;
    if (g.b_mn && g.N < (g.N <= 32 ? 32 : 64)) return false;
    return ((uintptr_t)g.A % 16) == 0 && ((uintptr_t)g.B % 16) == 0 && g.K >= kTcBK;
}

static int tc_bn(int N) { return N <= 32 ? 32 : (N <= 64 ? 64 : (N <= 128 ? 128 : 256)); }

bool gemm_tc_fills_chip(const GemmArgs &g)
{
    // Below one output tile per SM a plain GEMM gains nothing from the
    // persistent form's overlap and pays its set-up (tensor-memory
    // allocation, barrier initialisation, the tensor maps' fetch); such
    // GEMMs stay on the mma.sync kernel unless the caller asks for tcgen05.
    static int sms = 0;
    if (!sms) {
        int dev = 0, n = 0;
        if (cudaGetDevice(&dev) == cudaSuccess &&
            cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && n > 0)
            sms = n;
        else
            return false;
    }
    const long tiles = (long)((g.M + kTcBM - 1) / kTcBM) * ((g.N + tc_bn(g.N) - 1) / tc_bn(g.N)) * g.ksplit;
    return tiles >= sms;
}

int gemm_tc(const GemmArgs &g, cudaStream_t s)
{
    CUtensorMap ma, mb;
    const int BN = tc_bn(g.N);
    if (g.conv == 1) {
        PCD_TRY(make_map4(&ma, g.A, g.xc, g.xw, g.xh, g.xb, g.lda, g.cwid, kTcBM));
        PCD_TRY(make_map(&mb, g.B, g.N, g.K, g.ldb, BN, g.cwid));
    } else {
        if (g.conv == 2) PCD_TRY(make_map4(&ma, g.A, g.xc, g.xw, g.xh, g.xb, g.lda, g.cwid, kTcBK));
        else if (g.a_mn) PCD_TRY(make_map(&ma, g.A, g.K, g.M, g.lda, kTcBK, 64));
        else PCD_TRY(make_map(&ma, g.A, g.M, g.K, g.lda, kTcBM));
        if (g.b_mn) PCD_TRY(make_map(&mb, g.B, g.K, g.N, g.ldb, kTcBK, BN < 64 ? BN : 64));
        else PCD_TRY(make_map(&mb, g.B, g.N, g.K, g.ldb, BN));
    }
    int *err = err_word();
    if (!err) {
        set_error("tcgen05 gemm: no error word");
        return PCD_DEVICE_ERROR;
    }
    if (BN == 32) return launch_tcp<32>(ma, mb, g, s, err);
    if (BN == 64) return launch_tcp<64>(ma, mb, g, s, err);
    if (BN == 128) return launch_tcp<128>(ma, mb, g, s, err);
    return launch_tcp<256>(ma, mb, g, s, err);
}

int gemm_tc_prepare()
{
    if (!err_word()) {
        set_error("tcgen05 gemm: no error word");
        return PCD_DEVICE_ERROR;
    }
    PCD_TRY(tcp_attr<32>());
    PCD_TRY(tcp_attr<64>());
    PCD_TRY(tcp_attr<128>());
    PCD_TRY(tcp_attr<256>());
    if (!encode_fn()) {
        set_error("tcgen05 gemm: cuTensorMapEncodeTiled is not available");
        return PCD_DEVICE_ERROR;
    }
    return PCD_OK;
}

int gemm_tc_check(cudaStream_t s)
{
    int *w = err_word();
    if (!w) {
        set_error("tcgen05 gemm: no error word");
        return PCD_DEVICE_ERROR;
    }
    int v = 0;
    PCD_CUDA(cudaMemcpyAsync(&v, w, sizeof(int), cudaMemcpyDeviceToHost, s));
    PCD_CUDA(cudaStreamSynchronize(s));
    if (v != 0) {
        PCD_CUDA(cudaMemsetAsync(w, 0, sizeof(int), s));
        PCD_CUDA(cudaStreamSynchronize(s));
        set_error("tcgen05 gemm: a pipeline wait gave up (code " + std::to_string(v) + ")");
        return PCD_DEVICE_ERROR;
    }
    return PCD_OK;
}

int gemm_tc_error(int *out, bool reset)
{
    int *w = err_word();
    if (!w) return PCD_DEVICE_ERROR;
    PCD_CUDA(cudaDeviceSynchronize());
    PCD_CUDA(cudaMemcpy(out, w, sizeof(int), cudaMemcpyDeviceToHost));
    if (reset) PCD_CUDA(cudaMemset(w, 0, sizeof(int)));
    return PCD_OK;
}

}  // namespace nn
}  // namespace pcd
