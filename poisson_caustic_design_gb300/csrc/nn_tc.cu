// nn_tc.cu -- the U-Net's BF16 GEMM on the 5th-generation tensor cores
// (tcgen05, sm_103a).
//
// C[M x N] = A[M x K] * B[N x K]^T with A and B BF16 row-major, K contiguous
// ("TN", the layout of nn::gemm), FP32 accumulation in tensor memory.  One CTA
// computes a 128 x BN tile of C over its share of K:
//
//   * TMA (cp.async.bulk.tensor.2d) loads 128 x 64 tiles of A and BN x 64
//     tiles of B into shared memory with the 128-byte swizzle, through a ring
//     of kStages stages (full / empty mbarriers; the transfer size is the
//     whole box, zero-filled where the box leaves the matrix);
//   * one thread issues tcgen05.mma.cta_group::1.kind::f16 (M = 128, N = BN,
//     K = 16 per instruction, both operands K-major, described by shared
//     memory descriptors whose start address steps 32 bytes per K slice
//     inside the 128-byte swizzle atom) into a 128-lane x BN-column FP32
//     accumulator in tensor memory, and tcgen05.commit signals the stage free
//     once the MMAs that read it are done;
//   * after the last MMA, warps 0-3 read their 32 lanes (rows) of the
//     accumulator with tcgen05.ld.32x32b and apply the epilogue of nn::gemm
//     (bias, ReLU, BF16 or FP32 store, or FP32 split-K partials).
//
// The same thread produces and consumes the ring: it refills the stage the
// previous K tile used once that tile's MMAs have completed, while the MMAs
// of the current tile run.  Every mbarrier wait is bounded: a wait that runs
// out records PCD_TIMEOUT in *err, the CTA stops issuing, waits (bounded) for
// what it has in flight and frees its tensor memory.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <mutex>

#include "nn.cuh"

namespace pcd {
namespace nn {

namespace {

constexpr int kTcBM = 128, kTcBK = 64, kTcStages = 4, kTcThreads = 128;
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

template <int BN>
__global__ void __launch_bounds__(kTcThreads, 1)
    k_gemm_tc(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB, GemmArgs g, int *err)
{
    static_assert(BN == 32 || BN == 64 || BN == 128 || BN == 256, "N tile");
    static_assert(kTcBM * 33 * 4 <= kTcStages * (kTcBM * kTcBK * 2), "epilogue tile fits in the ring");
    constexpr unsigned kStageA = kTcBM * kTcBK * 2, kStageB = BN * kTcBK * 2, kStage = kStageA + kStageB;
    constexpr int kCols = BN < 32 ? 32 : BN;  // tensor memory columns (a power of 2, >= 32)
    extern __shared__ __align__(1024) unsigned char tc_buf[];
    __shared__ __align__(8) unsigned long long bars[2 * kTcStages + 1];
    __shared__ unsigned tmem_base;
    __shared__ int s_fail;
    __shared__ int s_fills[kTcStages];  // loads issued per stage (thread 0)

    // the ring must start on a 1024-byte boundary (the swizzle atom)
    const unsigned raw = tc_smem(tc_buf);
    const unsigned ring = (raw + 1023u) & ~1023u;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int bm = blockIdx.y * kTcBM, bn = blockIdx.x * BN;
    const int KT = g.conv == 1 ? 9 * g.nch : (g.K + kTcBK - 1) / kTcBK;
    const int per = (KT + g.ksplit - 1) / g.ksplit;
    // bytes a stage's loads deliver (a 32-channel convolution tile fills half the stage)
    const unsigned tx = g.conv == 1 ? (unsigned)(kTcBM + BN) * (unsigned)g.cwid * 2u : kStage;
    const int kt0 = blockIdx.z * per, kt1 = min(KT, kt0 + per);
    const int nk = max(0, kt1 - kt0);
    const unsigned full0 = tc_smem(&bars[0]), empty0 = tc_smem(&bars[kTcStages]), done = tc_smem(&bars[2 * kTcStages]);

    if (threadIdx.x == 0) {
        s_fail = 0;
        for (int s = 0; s < kTcStages; s++) {
            s_fills[s] = 0;
            mbar_init(full0 + 8 * s, 1);
            mbar_init(empty0 + 8 * s, 1);
        }
        mbar_init(done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"(&mapA) : "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"(&mapB) : "memory");
    }
    if (warp == 0) {
        // one warp allocates the accumulator's columns (and frees them at the end)
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc_smem(&tmem_base)),
                     "r"(kCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const unsigned tmem = tmem_base;

    // ---- producer + MMA issuer: thread 0
    if (threadIdx.x == 0 && nk > 0) {
        const unsigned idesc = idesc_bf16_f32(kTcBM, BN, g.a_mn, g.b_mn);
        bool ok = true;
        const int pre = min(nk, kTcStages);
        for (int i = 0; i < pre; i++) {
            const unsigned st = ring + (unsigned)i * kStage;
            mbar_expect_tx(full0 + 8 * i, tx);
            load_stage<BN>(st, st + kStageA, &mapA, &mapB, full0 + 8 * i, g, kt0 + i, bm, bn);
            s_fills[i]++;
        }
        int issued = pre;
        for (int i = 0; i < nk && ok; i++) {
            const int s = i % kTcStages;
            const unsigned phase = (unsigned)((i / kTcStages) & 1);
            if (!mbar_wait(full0 + 8 * s, phase)) { ok = false; break; }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const unsigned a = ring + (unsigned)s * kStage, b = a + kStageA;
            const bool k32 = g.conv == 1 && g.cwid == 32;  // a 32-deep K tile (64-byte swizzle)
#pragma unroll
            for (int kk = 0; kk < kTcBK / 16; kk++) {
                if (k32 && kk >= 2) break;
                const unsigned long long da = k32         ? desc_kmajor_sw64(a, kk)
                                              : g.conv == 2 ? desc_mnmajor(a, kk, g.cwid)
                                              : g.a_mn      ? desc_mnmajor(a, kk, 64)
                                                            : desc_kmajor(a, kk);
                const unsigned long long db = k32    ? desc_kmajor_sw64(b, kk)
                                              : g.b_mn ? desc_mnmajor(b, kk, BN < 64 ? BN : 64)
                                                       : desc_kmajor(b, kk);
                mma_bf16_tc(tmem, da, db, idesc, (i > 0 || kk > 0) ? 1u : 0u);
            }
            mma_commit(empty0 + 8 * s);
            // refill the stage of the previous K tile once its MMAs are done
            if (i > 0 && issued < nk) {
                const int ps = (i - 1) % kTcStages;
                const unsigned pphase = (unsigned)(((i - 1) / kTcStages) & 1);
                if (!mbar_wait(empty0 + 8 * ps, pphase)) { ok = false; break; }
                const unsigned st = ring + (unsigned)ps * kStage;
                mbar_expect_tx(full0 + 8 * ps, tx);
                load_stage<BN>(st, st + kStageA, &mapA, &mapB, full0 + 8 * ps, g, kt0 + issued, bm, bn);
                s_fills[ps]++;
                issued++;
            }
        }
        if (ok) {
            mma_commit(done);  // arrives when every MMA issued above has completed
        } else {
            atomicCAS(err, 0, PCD_TIMEOUT);
            s_fail = 1;
        }
    }
    __syncthreads();

    // ---- epilogue: 32 columns at a time, warp w reading accumulator lanes
    // [32w, 32w + 32) (tile rows) with tcgen05.ld, through a shared tile in
    // the (now idle) ring so that the stores of C run along its rows
    const bool fail = s_fail != 0 || nk == 0;  // the same for every thread (read after a barrier)
    bool lost = false;                         // the done wait ran out somewhere in the block
    if (!fail) {
        // one decision for the whole block: every thread takes the same path
        // through the barriers below
        const bool ok = __syncthreads_and(mbar_wait(done, 0u)) != 0;
        lost = !ok;
        if (!ok && threadIdx.x == 0) atomicCAS(err, 0, PCD_TIMEOUT);
        if (ok) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            float *tile = reinterpret_cast<float *>(tc_buf + (ring - raw));  // [128][33]
            for (int c0 = 0; c0 < BN; c0 += 32) {
                unsigned r[32];
                const unsigned addr = tmem + ((unsigned)(warp * 32) << 16) + (unsigned)c0;
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
                    "[%16];"
                    : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                      "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                      "=r"(r[15])
                    : "r"(addr));
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
                    "[%16];"
                    : "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]),
                      "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]),
                      "=r"(r[30]), "=r"(r[31])
                    : "r"(addr + 16u));
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                if (g.trans_c) {
                    // C[n][m]: a warp's 32 lanes are 32 consecutive m, so each
                    // column n is one 128-byte store (split-K partials as
                    // [split][N][M], ldc = M)
                    int m = 0;
                    if (out_row(g, bm + warp * 32 + lane, m)) {
                        float *base = g.Cf + (g.ksplit > 1 ? (size_t)blockIdx.z * g.N * g.ldc : 0);
#pragma unroll
                        for (int j = 0; j < 32; j++) {
                            const int n = bn + c0 + j;
                            if (n < g.N) base[(size_t)n * g.ldc + m] = __uint_as_float(r[j]);
                        }
                    }
                    continue;
                }
                float *mine = tile + (warp * 32 + lane) * 33;
#pragma unroll
                for (int j = 0; j < 32; j++) mine[j] = __uint_as_float(r[j]);
                __syncthreads();
                const int n = bn + c0 + lane;
                const float bias = (g.ksplit == 1 && g.bias && n < g.N) ? g.bias[n] : 0.f;
                for (int rr = warp; rr < kTcBM; rr += kTcThreads / 32) {
                    const int row = bm + rr;
                    if (row >= g.M || n >= g.N) continue;
                    float v = tile[rr * 33 + lane];
                    if (g.ksplit > 1) {
                        g.Cf[((size_t)blockIdx.z * g.M + row) * g.ldc + n] = v;
                        continue;
                    }
                    v += bias;
                    if (g.relu) v = fmaxf(v, 0.f);
                    if (g.Cb) g.Cb[(size_t)row * g.ldc + n] = __float2bfloat16(v);
                    else g.Cf[(size_t)row * g.ldc + n] = v;
                }
                __syncthreads();
            }
        }
    } else if (nk == 0 && g.ksplit > 1) {
        // an empty K share still writes zero partials
        const int row = bm + warp * 32 + lane;
        int m = 0;
        if (g.trans_c && out_row(g, row, m))
            for (int n = bn; n < min(g.N, bn + BN); n++) g.Cf[((size_t)blockIdx.z * g.N + n) * g.ldc + m] = 0.f;
        else if (!g.trans_c && row < g.M)
            for (int n = bn; n < min(g.N, bn + BN); n++) g.Cf[((size_t)blockIdx.z * g.M + row) * g.ldc + n] = 0.f;
    }
    if ((s_fail != 0 || lost) && threadIdx.x == 0) {
        // let what is still in flight land before the shared memory and the
        // tensor memory go away: every MMA issued (one more commit), and each
        // stage's latest load (bounded waits)
        mma_commit(done);
        (void)mbar_wait(done, 0u);
        for (int s = 0; s < kTcStages; s++)
            if (s_fills[s] > 0) (void)mbar_wait(full0 + 8 * s, (unsigned)((s_fills[s] - 1) & 1));
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
constexpr size_t tc_smem_bytes()
{
    return (size_t)kTcStages * (kTcBM * kTcBK * 2 + BN * kTcBK * 2) + 1024;
}

// The kernel's shared-memory attribute, set on the current device the first
// time (the setting belongs to the function on that device).
template <int BN>
int tc_attr()
{
    static std::mutex mu;
    static unsigned long long done_mask = 0;
    int dev = 0;
    PCD_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(mu);
    if (dev < 64 && (done_mask >> dev & 1ull)) return PCD_OK;
    PCD_CUDA(cudaFuncSetAttribute(k_gemm_tc<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tc_smem_bytes<BN>()));
    if (dev < 64) done_mask |= 1ull << dev;
    return PCD_OK;
}

template <int BN>
int launch_tc(const CUtensorMap &ma, const CUtensorMap &mb, const GemmArgs &g, cudaStream_t s, int *err)
{
    const size_t smem = tc_smem_bytes<BN>();
    PCD_TRY(tc_attr<BN>());
    const dim3 grid((g.N + BN - 1) / BN, (g.M + kTcBM - 1) / kTcBM, g.ksplit);
    k_gemm_tc<BN><<<grid, kTcThreads, smem, s>>>(ma, mb, g, err);
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
    // Below one CTA per SM the per-CTA set-up (tensor-memory allocation,
    // barrier initialisation, the tensor maps' fetch) and the single issuing
    // thread's latency are not hidden: at 64^2 pixels and batch 1 the U-Net's
    // GEMMs (32 tiles and fewer) run faster on the mma.sync kernel.
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
    if (BN == 32) return launch_tc<32>(ma, mb, g, s, err);
    if (BN == 64) return launch_tc<64>(ma, mb, g, s, err);
    if (BN == 128) return launch_tc<128>(ma, mb, g, s, err);
    return launch_tc<256>(ma, mb, g, s, err);
}

int gemm_tc_prepare()
{
    if (!err_word()) {
        set_error("tcgen05 gemm: no error word");
        return PCD_DEVICE_ERROR;
    }
    PCD_TRY(tc_attr<32>());
    PCD_TRY(tc_attr<64>());
    PCD_TRY(tc_attr<128>());
    PCD_TRY(tc_attr<256>());
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
