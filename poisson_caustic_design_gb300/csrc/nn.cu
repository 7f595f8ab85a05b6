// nn.cu -- the building blocks of the learned warm start (sm_103a).
//
// A 3x3 convolution is an implicit GEMM: im2col turns an NHWC activation
// (BF16) into a P x Kp matrix (P pixels, Kp = 9*C rounded up to 32, tap-major
// then channel), and one BF16 tensor-core GEMM with FP32 accumulation
// multiplies it by the weights W[Cout][Kp].  Backward-data is the same
// convolution of the output gradient with the flipped, channel-transposed
// weights; backward-weight is a GEMM over the pixel dimension (split-K).
//
// GEMM: C[M x N] = A[M x K] * B[N x K]^T, A and B row-major with K
// contiguous ("TN"), K a multiple of 32, leading dimensions multiples of 8.
// 128 x BN x 32 block tile, 8 warps, mma.sync.m16n8k16 BF16 -> FP32,
// ldmatrix fragment loads from a padded (80-byte rows, conflict-free) shared
// tile, 3-stage cp.async pipeline with zero-filled M/N tails.  Epilogue:
// + bias, ReLU, BF16 or FP32 store, or FP32 split-K partials reduced by a
// second kernel in a fixed order.
#include <cuda_bf16.h>

#include <atomic>

#include "nn.cuh"

namespace pcd {
namespace nn {

namespace {

constexpr int GBM = 128, GBK = 32, GST = 3, GTHREADS = 256;
// automatic path for a plain GEMM: the tcgen05 form (nn_tc.cu) when it takes
// it and its output tiles fill the chip, else mma.sync; 1 pins everything,
// the U-Net's implicit convolutions included, to mma.sync (the convolutions
// choose the tcgen05 form themselves, with split-K on small grids)
std::atomic<int> g_default_path{0};
constexpr int SROW = GBK + 8;  // padded shared row: 40 bf16 = 80 bytes

__device__ __forceinline__ unsigned smem_u32(const void *p)
{
    return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void cp_async16(void *dst, const void *src, bool valid)
{
    const unsigned d = smem_u32(dst);
    const int n = valid ? 16 : 0;  // zero-fill when out of range
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(d), "l"(src), "r"(n) : "memory");
}

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }

template <int N>
__device__ __forceinline__ void cp_async_wait()
{
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

__device__ __forceinline__ void ldmatrix_x4(unsigned (&r)[4], const void *p)
{
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(smem_u32(p)));
}

__device__ __forceinline__ void mma_bf16(float (&c)[4], const unsigned (&a)[4], unsigned b0, unsigned b1)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// BN = 128: warps 2 (M) x 4 (N), warp tile 64 x 32
// BN =  64: warps 4 x 2, warp tile 32 x 32
// BN =  32: warps 8 x 1, warp tile 16 x 32
template <int BN>
__global__ void __launch_bounds__(GTHREADS) k_gemm(GemmArgs g)
{
    constexpr int WN = BN / 32, WM = 8 / WN, MI = (GBM / WM) / 16;
    extern __shared__ __align__(16) __nv_bfloat16 gsm[];
    __nv_bfloat16 *sA = gsm;                        // GST x GBM x SROW
    __nv_bfloat16 *sB = gsm + GST * GBM * SROW;     // GST x BN x SROW
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int wm = warp / WN, wn = warp % WN;
    const int bm = blockIdx.y * GBM, bn = blockIdx.x * BN;
    const int KT = g.K / GBK;
    const int per = (KT + g.ksplit - 1) / g.ksplit;
    const int kt0 = blockIdx.z * per, kt1 = min(KT, kt0 + per);

    float acc[MI][4][4];
#pragma unroll
    for (int i = 0; i < MI; i++)
#pragma unroll
        for (int j = 0; j < 4; j++)
#pragma unroll
            for (int r = 0; r < 4; r++) acc[i][j][r] = 0.f;

    auto load_tile = [&](int stage, int kt) {
        __nv_bfloat16 *a = sA + stage * GBM * SROW;
        __nv_bfloat16 *b = sB + stage * BN * SROW;
        const int k0 = kt * GBK;
        for (int idx = tid; idx < GBM * 4; idx += GTHREADS) {
            const int row = idx >> 2, ch = idx & 3;
            const int gm = bm + row;
            const bool ok = gm < g.M;
            const __nv_bfloat16 *src = g.A + (size_t)(ok ? gm : 0) * g.lda + k0 + ch * 8;
            cp_async16(a + row * SROW + ch * 8, src, ok);
        }
        for (int idx = tid; idx < BN * 4; idx += GTHREADS) {
            const int row = idx >> 2, ch = idx & 3;
            const int gn = bn + row;
            const bool ok = gn < g.N;
            const __nv_bfloat16 *src = g.B + (size_t)(ok ? gn : 0) * g.ldb + k0 + ch * 8;
            cp_async16(b + row * SROW + ch * 8, src, ok);
        }
    };

    const int nk = kt1 - kt0;
#pragma unroll
    for (int s = 0; s < GST - 1; s++) {
        if (s < nk) load_tile(s, kt0 + s);
        cp_async_commit();
    }
    for (int it = 0; it < nk; it++) {
        cp_async_wait<GST - 2>();
        __syncthreads();
        const int pf = it + GST - 1;
        if (pf < nk) load_tile(pf % GST, kt0 + pf);
        cp_async_commit();
        const __nv_bfloat16 *a = sA + (it % GST) * GBM * SROW;
        const __nv_bfloat16 *b = sB + (it % GST) * BN * SROW;
#pragma unroll
        for (int kk = 0; kk < GBK; kk += 16) {
            unsigned af[MI][4], bf[4][2];
#pragma unroll
            for (int mi = 0; mi < MI; mi++) {
                const int row = wm * (GBM / WM) + mi * 16 + (lane & 15);
                ldmatrix_x4(af[mi], a + row * SROW + kk + (lane >> 4) * 8);
            }
#pragma unroll
            for (int nj = 0; nj < 2; nj++) {
                unsigned r[4];
                const int row = wn * 32 + nj * 16 + (lane & 7) + ((lane >> 4) << 3);
                ldmatrix_x4(r, b + row * SROW + kk + ((lane >> 3) & 1) * 8);
                bf[2 * nj][0] = r[0];
                bf[2 * nj][1] = r[1];
                bf[2 * nj + 1][0] = r[2];
                bf[2 * nj + 1][1] = r[3];
            }
#pragma unroll
            for (int mi = 0; mi < MI; mi++)
#pragma unroll
                for (int ni = 0; ni < 4; ni++) mma_bf16(acc[mi][ni], af[mi], bf[ni][0], bf[ni][1]);
        }
    }
    cp_async_wait<0>();

    // epilogue
#pragma unroll
    for (int mi = 0; mi < MI; mi++)
#pragma unroll
        for (int ni = 0; ni < 4; ni++)
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const int gm = bm + wm * (GBM / WM) + mi * 16 + (lane >> 2) + h * 8;
                const int gn = bn + wn * 32 + ni * 8 + (lane & 3) * 2;
                if (gm >= g.M) continue;
#pragma unroll
                for (int e = 0; e < 2; e++) {
                    const int n = gn + e;
                    if (n >= g.N) continue;
                    float v = acc[mi][ni][2 * h + e];
                    if (g.ksplit > 1) {
                        g.Cf[((size_t)blockIdx.z * g.M + gm) * g.ldc + n] = v;
                        continue;
                    }
                    if (g.bias) v += g.bias[n];
                    if (g.relu) v = fmaxf(v, 0.f);
                    if (g.Cb) g.Cb[(size_t)gm * g.ldc + n] = __float2bfloat16(v);
                    else g.Cf[(size_t)gm * g.ldc + n] = v;
                }
            }
}

// sum of split-K partials in a fixed order, + bias, ReLU, store
// C = sum over the K splits of part[z][m][n] (+ bias, ReLU), one thread per
// output (few splits, many outputs)
__global__ void k_splitk_reduce(const float *part, int splits, int M, int N, int ldc, const float *bias, int relu,
                                __nv_bfloat16 *Cb, float *Cf, int ldo)
{
    const long total = (long)M * N;
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
        const int m = (int)(t / N), n = (int)(t - (long)m * N);
        float v = 0.f;
        for (int z = 0; z < splits; z++) v += part[((size_t)z * M + m) * ldc + n];
        if (bias) v += bias[n];
        if (relu) v = fmaxf(v, 0.f);
        if (Cb) Cb[(size_t)m * ldo + n] = __float2bfloat16(v);
        else Cf[(size_t)m * ldo + n] = v;
    }
}

// The same for many splits over few outputs (the weight gradients): a block
// of 32 x 8 threads takes 32 consecutive outputs, thread (x, y) adds splits
// y, y + 8, ..., and column x's eight sums fold in a fixed order.
constexpr int kReduceLanes = 8, kReduceLanesFrom = 16;
__global__ void k_splitk_reduce_lanes(const float *part, int splits, int M, int N, int ldc, const float *bias, int relu,
                                __nv_bfloat16 *Cb, float *Cf, int ldo)
{
    __shared__ float red[kReduceLanes][33];
    const long total = (long)M * N;
    for (long t0 = (long)blockIdx.x * 32; t0 < total; t0 += (long)gridDim.x * 32) {
        const long t = t0 + threadIdx.x;
        const int m = (int)(t / N), n = (int)(t - (long)m * N);
        float v = 0.f;
        if (t < total)
            for (int z = threadIdx.y; z < splits; z += kReduceLanes) v += part[((size_t)z * M + m) * ldc + n];
        red[threadIdx.y][threadIdx.x] = v;
        __syncthreads();
        if (threadIdx.y == 0 && t < total) {
            for (int y = 1; y < kReduceLanes; y++) v += red[y][threadIdx.x];
            if (bias) v += bias[n];
            if (relu) v = fmaxf(v, 0.f);
            if (Cb) Cb[(size_t)m * ldo + n] = __float2bfloat16(v);
            else Cf[(size_t)m * ldo + n] = v;
        }
        __syncthreads();
    }
}

inline int reduce_blocks(long outputs) { return (int)std::max<long>(1, std::min<long>(16384, (outputs + 31) / 32)); }

inline int grid1d(long n, int t = 256);

// out = the split-K partials' sum: the per-output form for few splits, the
// 8-lane form from kReduceLanesFrom splits on
void splitk_reduce(const float *part, int splits, int M, int N, int ldc, const float *bias, int relu,
                   __nv_bfloat16 *Cb, float *Cf, int ldo, cudaStream_t s)
{
    if (splits >= kReduceLanesFrom)
        k_splitk_reduce_lanes<<<reduce_blocks((long)M * N), dim3(32, kReduceLanes), 0, s>>>(part, splits, M, N, ldc,
                                                                                           bias, relu, Cb, Cf, ldo);
    else
        k_splitk_reduce<<<grid1d((long)M * N), 256, 0, s>>>(part, splits, M, N, ldc, bias, relu, Cb, Cf, ldo);
}

inline int grid1d(long n, int t) { return (int)std::max<long>(1, std::min<long>(8192, (n + t - 1) / t)); }

// im2col of an NHWC activation slice: out[p][tap*C + c] (zeros outside the
// image and for k >= 9C up to Kp)
__global__ void k_im2col(const __nv_bfloat16 *in, int B, int H, int W, int C, int ldcin, __nv_bfloat16 *out, int Kp)
{
    const long P = (long)B * H * W;
    const long total = P * Kp;
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
        const long p = t / Kp;
        const int k = (int)(t - p * Kp);
        __nv_bfloat16 v = __float2bfloat16(0.f);
        if (k < 9 * C) {
            const int tap = k / C, c = k - tap * C;
            const int ky = tap / 3, kx = tap - ky * 3;
            const int n = (int)(p / ((long)H * W));
            const int rem = (int)(p - (long)n * H * W);
            const int y = rem / W + ky - 1, x = rem % W + kx - 1;
            if (y >= 0 && y < H && x >= 0 && x < W) v = in[(((size_t)n * H + y) * W + x) * ldcin + c];
        }
        out[t] = v;
    }
}

// vectorised variant for C % 8 == 0: 8 channels (16 bytes) per thread
__global__ void k_im2col8(const __nv_bfloat16 *in, int B, int H, int W, int C, int ldcin, __nv_bfloat16 *out, int Kp)
{
    const long P = (long)B * H * W;
    const int K8 = Kp / 8;
    const long total = P * K8;
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
        const long p = t / K8;
        const int k = (int)(t - p * K8) * 8;
        uint4 v = make_uint4(0, 0, 0, 0);
        if (k < 9 * C) {
            const int tap = k / C, c = k - tap * C;
            const int ky = tap / 3, kx = tap - ky * 3;
            const int n = (int)(p / ((long)H * W));
            const int rem = (int)(p - (long)n * H * W);
            const int y = rem / W + ky - 1, x = rem % W + kx - 1;
            if (y >= 0 && y < H && x >= 0 && x < W)
                v = *reinterpret_cast<const uint4 *>(in + (((size_t)n * H + y) * W + x) * ldcin + c);
        }
        *reinterpret_cast<uint4 *>(out + (size_t)p * Kp + k) = v;
    }
}

// out[c][r] = in[r][c] (bf16), 32 x 32 tiles through shared memory
__global__ void k_transpose(const __nv_bfloat16 *in, int rows, int cols, int ldin, __nv_bfloat16 *out, int ldout)
{
    __shared__ __nv_bfloat16 tile[32][33];
    const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
    for (int j = threadIdx.y; j < 32; j += blockDim.y) {
        const int r = by + j, c = bx + threadIdx.x;
        tile[j][threadIdx.x] = (r < rows && c < cols) ? in[(size_t)r * ldin + c] : __float2bfloat16(0.f);
    }
    __syncthreads();
    for (int j = threadIdx.y; j < 32; j += blockDim.y) {
        const int c = bx + j, r = by + threadIdx.x;
        if (c < cols && r < rows) out[(size_t)c * ldout + r] = tile[threadIdx.x][j];
    }
}

// W'[ci][tap'*Cout + co] = W[co][(8 - tap')*Cin + ci] (flipped taps, channels swapped)
__global__ void k_flip(const __nv_bfloat16 *Wt, int Cout, int Cin, int Kp, __nv_bfloat16 *Wf, int Kpf)
{
    const long total = (long)Cin * Kpf;
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
        const int ci = (int)(t / Kpf), k = (int)(t - (long)ci * Kpf);
        __nv_bfloat16 v = __float2bfloat16(0.f);
        if (k < 9 * Cout) {
            const int tp = k / Cout, co = k - tp * Cout;
            v = Wt[(size_t)co * Kp + (8 - tp) * Cin + ci];
        }
        Wf[t] = v;
    }
}

// dYm = dY * (Y > 0) as bf16 (dense P x C), and (optionally) FP32 column sums
__global__ void k_relu_bwd(const float *dY, int lddy, const __nv_bfloat16 *Y, int ldy, long P, int C, int relu,
                           __nv_bfloat16 *dYm)
{
    const long total = P * C;
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
        const long p = t / C;
        const int c = (int)(t - p * C);
        float d = dY[p * lddy + c];
        if (relu && !(__bfloat162float(Y[p * ldy + c]) > 0.f)) d = 0.f;
        dYm[t] = __float2bfloat16(d);
    }
}

// The same masking fused with the bias gradient's first pass: block b takes
// one contiguous range of pixels, thread t channel t % C of every
// (blockDim / C)-th pixel in it, and part[b][c] = the block's sum of the
// BF16 values it stored (lanes folded in a fixed order); C divides blockDim.
__global__ void k_relu_bwd_colsum(const float *dY, int lddy, const __nv_bfloat16 *Y, int ldy, long P, int C, int relu,
                                  __nv_bfloat16 *dYm, float *part, int chunks)
{
    __shared__ float red[256];
    const int c = threadIdx.x % C, lane = threadIdx.x / C, lanes = blockDim.x / C;
    const long per = (P + chunks - 1) / chunks;
    const long p0 = (long)blockIdx.x * per, p1 = min(P, p0 + per);
    float s = 0.f;
#pragma unroll 4
    for (long p = p0 + lane; p < p1; p += lanes) {
        float d = dY[p * lddy + c];
        if (relu && !(__bfloat162float(Y[p * ldy + c]) > 0.f)) d = 0.f;
        const __nv_bfloat16 q = __float2bfloat16(d);
        dYm[p * C + c] = q;
        s += __bfloat162float(q);
    }
    red[threadIdx.x] = s;
    __syncthreads();
    if (lane == 0) {
        for (int l = 1; l < lanes; l++) s += red[l * C + c];
        part[(size_t)blockIdx.x * C + c] = s;
    }
}

// db[c] = sum_p dYm[p][c]: per-block partials over pixel chunks, fixed order
__global__ void k_colsum(const __nv_bfloat16 *X, long P, int C, float *part, int chunks)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= C) return;
    const long per = (P + chunks - 1) / chunks;
    const long p0 = blockIdx.y * per, p1 = min(P, p0 + per);
    float s = 0.f;
    for (long p = p0; p < p1; p++) s += __bfloat162float(X[p * C + c]);
    part[(size_t)blockIdx.y * C + c] = s;
}

// out[c] = sum_k part[k][c] with one warp per column: lane l adds rows l,
// l + 32, ... and the lanes fold by shuffles (a fixed order)
__global__ void k_colsum_fold_warp(const float *part, int chunks, int C, float *out)
{
    const int c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (c >= C) return;
    float s = 0.f;
#pragma unroll 4
    for (int k = lane; k < chunks; k += 32) s += part[(size_t)k * C + c];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) out[c] = s;
}

// 2x2 average pool of a channel slice (in stride ldin) into dense out (stride C)
__global__ void k_pool(const __nv_bfloat16 *in, int B, int H, int W, int C, int ldin, __nv_bfloat16 *out)
{
    const int Ho = H / 2, Wo = W / 2;
    const long total = (long)B * Ho * Wo * C;
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
        const int c = (int)(t % C);
        const long q = t / C;
        const int xo = (int)(q % Wo), yo = (int)((q / Wo) % Ho), n = (int)(q / ((long)Wo * Ho));
        const size_t base = (((size_t)n * H + 2 * yo) * W + 2 * xo) * ldin + c;
        const float s = __bfloat162float(in[base]) + __bfloat162float(in[base + ldin]) +
                        __bfloat162float(in[base + (size_t)W * ldin]) + __bfloat162float(in[base + (size_t)W * ldin + ldin]);
        out[t] = __float2bfloat16(0.25f * s);
    }
}

// gradient of the pool: dIn[2y+dy][2x+dx] += 0.25 dOut[y][x] (dIn FP32, slice stride lddin)
__global__ void k_pool_bwd(const float *dOut, int B, int H, int W, int C, float *dIn, int lddin)
{
    const long total = (long)B * H * W * C;
    const int Ho = H / 2, Wo = W / 2;
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
        const int c = (int)(t % C);
        const long q = t / C;
        const int x = (int)(q % W), y = (int)((q / W) % H), n = (int)(q / ((long)W * H));
        dIn[q * lddin + c] += 0.25f * dOut[(((size_t)n * Ho + y / 2) * Wo + x / 2) * C + c];
    }
}

// nearest 2x upsample of dense in (stride C) into a channel slice of out (stride ldout)
__global__ void k_up(const __nv_bfloat16 *in, int B, int H, int W, int C, __nv_bfloat16 *out, int ldout)
{
    const int Ho = 2 * H, Wo = 2 * W;
    const long total = (long)B * Ho * Wo * C;
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
        const int c = (int)(t % C);
        const long q = t / C;
        const int x = (int)(q % Wo), y = (int)((q / Wo) % Ho), n = (int)(q / ((long)Wo * Ho));
        out[q * ldout + c] = in[(((size_t)n * H + y / 2) * W + x / 2) * C + c];
    }
}

// gradient of the upsample: dIn[y][x] = sum of the four dOut children (slice stride lddout)
__global__ void k_up_bwd(const float *dOut, int lddout, int B, int H, int W, int C, float *dIn)
{
    const long total = (long)B * H * W * C;
    const int Wo = 2 * W, Ho = 2 * H;
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
        const int c = (int)(t % C);
        const long q = t / C;
        const int x = (int)(q % W), y = (int)((q / W) % H), n = (int)(q / ((long)W * H));
        const size_t b0 = (((size_t)n * Ho + 2 * y) * Wo + 2 * x) * lddout + c;
        dIn[t] = dOut[b0] + dOut[b0 + lddout] + dOut[b0 + (size_t)Wo * lddout] + dOut[b0 + (size_t)Wo * lddout + lddout];
    }
}

// 1x1 convolution with one output channel: out[p] = sum_c x[p][c] w[c] + bias
__global__ void k_head(const __nv_bfloat16 *X, long P, int C, const float *w, const float *bias, float *out)
{
    for (long p = (long)blockIdx.x * blockDim.x + threadIdx.x; p < P; p += (long)gridDim.x * blockDim.x) {
        float s = bias[0];
        for (int c = 0; c < C; c++) s += __bfloat162float(X[p * C + c]) * w[c];
        out[p] = s;
    }
}

// head gradients: dX[p][c] = d[p] w[c]; per-block partial sums of d[p] x[p][c] and d[p]
__global__ void k_head_bwd(const float *d, const __nv_bfloat16 *X, long P, int C, const float *w, float *dX,
                           float *part)
{
    extern __shared__ float hs[];  // C + 1 accumulators per warp... kept simple: per thread
    float acc[33];
    for (int c = 0; c <= C; c++) acc[c] = 0.f;
    for (long p = (long)blockIdx.x * blockDim.x + threadIdx.x; p < P; p += (long)gridDim.x * blockDim.x) {
        const float dp = d[p];
        for (int c = 0; c < C; c++) {
            const float xv = __bfloat162float(X[p * C + c]);
            dX[p * C + c] = dp * w[c];
            acc[c] += dp * xv;
        }
        acc[C] += dp;
    }
    for (int c = 0; c <= C; c++) {
        float v = warp_sum_f(acc[c]);
        if ((threadIdx.x & 31) == 0) hs[(threadIdx.x >> 5) * (C + 1) + c] = v;
    }
    __syncthreads();
    if (threadIdx.x <= C) {
        float s = 0.f;
        for (int wgi = 0; wgi < (int)(blockDim.x >> 5); wgi++) s += hs[wgi * (C + 1) + threadIdx.x];
        part[(size_t)blockIdx.x * (C + 1) + threadIdx.x] = s;
    }
}

// per-sample means of pred and target (one block per sample)
__global__ void k_sample_means(const float *pred, const float *tgt, long P1, float *means)
{
    double sp = 0.0, st = 0.0;
    const float *p = pred + (size_t)blockIdx.x * P1, *t = tgt + (size_t)blockIdx.x * P1;
    for (long i = threadIdx.x; i < P1; i += blockDim.x) {
        sp += p[i];
        st += t[i];
    }
    double v[2] = {sp, st};
    block_reduce<2, 0u>(v);
    if (threadIdx.x == 0) {
        means[2 * blockIdx.x] = (float)(v[0] / P1);
        means[2 * blockIdx.x + 1] = (float)(v[1] / P1);
    }
}

// loss = mean over all pixels of (pred - mean_pred - (tgt - mean_tgt))^2;
// d = 2 (diff - mean diff) / total; per-block loss partials
__global__ void k_mse(const float *pred, const float *tgt, long P1, int B, const float *means, float *d,
                      float *loss_part)
{
    const long total = P1 * B;
    double acc = 0.0;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
        const int s = (int)(i / P1);
        const float diff = (pred[i] - means[2 * s]) - (tgt[i] - means[2 * s + 1]);
        d[i] = 2.f * diff / (float)total;
        acc += (double)diff * diff;
    }
    double v[1] = {acc};
    block_reduce<1, 0u>(v);
    if (threadIdx.x == 0) loss_part[blockIdx.x] = (float)(v[0] / total);
}

// AdamW on FP32 master weights; also writes the BF16 copy (rows of `cols`
// values placed at stride ld, padding untouched)
__global__ void k_adamw(float *w, const float *grad, float *m, float *v, long n, int cols, int ld, float lr,
                        float beta1, float beta2, float eps, float wd, float bc1, float bc2, __nv_bfloat16 *wb)
{
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const float g = grad[i];
        const float mi = beta1 * m[i] + (1.f - beta1) * g;
        const float vi = beta2 * v[i] + (1.f - beta2) * g * g;
        m[i] = mi;
        v[i] = vi;
        float wi = w[i] * (1.f - lr * wd);
        wi -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
        w[i] = wi;
        if (wb) {
            const long r = i / cols, c = i - r * cols;
            wb[r * ld + c] = __float2bfloat16(wi);
        }
    }
}

__global__ void k_f32_to_bf16(const float *x, long n, __nv_bfloat16 *y)
{
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        y[i] = __float2bfloat16(x[i]);
}

__global__ void k_bf16_to_f32(const __nv_bfloat16 *x, long n, float *y, int ldx, int cols)
{
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const long r = i / cols, c = i - r * cols;
        y[i] = __bfloat162float(x[r * ldx + c]);
    }
}

__global__ void k_fill_f32(float *x, long n, float v)
{
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) x[i] = v;
}

// dense FP32 [P x C] into a channel slice of an FP32 buffer: out[p*ld + c] (+)= in[p*C + c]
__global__ void k_slice_add(const float *in, long P, int C, float *out, int ld, int accumulate)
{
    const long total = P * C;
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
        const long p = t / C;
        const int c = (int)(t - p * C);
        if (accumulate) out[p * ld + c] += in[t];
        else out[p * ld + c] = in[t];
    }
}

}  // namespace

// ---------------------------------------------------------------------------
int set_default_path(int path)
{
    if (path != 0 && path != 1) {
        set_error("gemm default path must be 0 (tcgen05 where it applies) or 1 (mma.sync)");
        return PCD_BAD_ARG;
    }
    g_default_path.store(path);
    return PCD_OK;
}

int default_path() { return g_default_path.load(); }

int sm_count()
{
    int dev = 0, n = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return 1;
    return n > 0 ? n : 1;
}

static GemmArgs conv_args(const __nv_bfloat16 *x, int B, int H, int W, int C, int ldx)
{
    GemmArgs g{};
    g.A = x;
    g.lda = ldx;
    g.xb = B;
    g.xh = H;
    g.xw = W;
    g.xc = C;
    g.cwid = C == 32 ? 32 : 64;
    g.nch = (C + g.cwid - 1) / g.cwid;
    g.path = 2;
    return g;
}

int conv3x3_tc(const __nv_bfloat16 *x, int B, int H, int W, int C, int ldx, const __nv_bfloat16 *w, int ldw, int N,
               const float *bias, int relu, __nv_bfloat16 *Cb, float *Cf, int ldc, int ksplit, float *partials,
               cudaStream_t s)
{
    GemmArgs g = conv_args(x, B, H, W, C, ldx);
    g.conv = 1;
    g.B = w;
    g.ldb = ldw;
    g.M = B * H * W;
    g.N = N;
    g.K = 9 * C;
    g.ksplit = ksplit;
    g.bias = bias;
    g.relu = relu;
    g.Cb = Cb;
    g.Cf = Cf;
    g.ldc = ldc;
    return gemm(g, s, ksplit > 1 ? partials : nullptr);
}

int conv3x3_wgrad_tc(const __nv_bfloat16 *x, int B, int H, int W, int C, int ldx, const __nv_bfloat16 *dy, int N,
                     float *dw, int ldw, int ksplit, float *partials, cudaStream_t s)
{
    GemmArgs g = conv_args(x, B, H, W, C, ldx);
    g.conv = 2;
    g.a_mn = 1;
    g.B = dy;
    g.ldb = N;
    g.b_mn = 1;
    g.trans_c = 1;
    g.M = 9 * g.nch * g.cwid;
    g.N = N;
    g.K = B * H * W;
    g.ksplit = ksplit;
    g.Cf = dw;
    g.ldc = ldw;
    return gemm(g, s, ksplit > 1 ? partials : nullptr);
}

size_t gemm_smem(int BN) { return (size_t)GST * (GBM + BN) * SROW * sizeof(__nv_bfloat16); }

int gemm(const GemmArgs &g0, cudaStream_t s, float *partials)
{
    GemmArgs g = g0;
    const bool layout_tc = g.a_mn || g.b_mn || g.trans_c || g.conv;  // forms only the tcgen05 kernel has
    if (layout_tc) {
        if (g.path == 1 || !gemm_tc_applies(g) || g.lda % 8 || g.ldb % 8 || g.M < 1 || g.N < 1 ||
            (g.trans_c && (g.Cb || g.bias || g.relu || !g.Cf))) {
            set_error("nn gemm: MN-major operands, implicit convolutions and a transposed C need the tcgen05 path "
                      "(aligned operands, K >= 64, MN-major extents >= 64, FP32 C without bias or ReLU, images "
                      "that tile into 128-pixel boxes)");
            return PCD_BAD_ARG;
        }
        g.path = 2;
    }
    // rows of a transposed C: M, or for the weight gradient 9 taps x channels
    const int Mo = g.conv == 2 ? 9 * g.xc : g.M;
    if ((!layout_tc && g.K % GBK != 0) || g.lda % 8 || g.ldb % 8 || g.M < 1 || g.N < 1) {
        set_error("nn gemm: K must be a multiple of 32 and leading dimensions multiples of 8");
        return PCD_BAD_ARG;
    }
    if (g.ksplit < 1) g.ksplit = 1;
    const int KT = g.K / GBK;
    if (g.ksplit > KT) g.ksplit = KT;
    float *outF = g.Cf;
    __nv_bfloat16 *outB = g.Cb;
    const int ldo = g.ldc;
    if (g.ksplit > 1) {
        if (!partials) {
            set_error("nn gemm: split-K needs a partial buffer");
            return PCD_BAD_ARG;
        }
        g.Cf = partials;
        g.Cb = nullptr;
        g.ldc = g.trans_c ? Mo : g.N;  // partials as [split][M][N], or [split][N][Mo] for a transposed C
    }
    const bool tc = g.path == 2 || (g.path == 0 && g_default_path.load() == 0 && gemm_tc_applies(g) &&
                                    gemm_tc_fills_chip(g));
    const int BN = g.N <= 32 ? 32 : (g.N <= 64 ? 64 : 128);
    const dim3 grid((g.N + BN - 1) / BN, (g.M + GBM - 1) / GBM, g.ksplit);
    const size_t smem = gemm_smem(BN);
    if (tc) {
        if (((uintptr_t)g.A % 16) || ((uintptr_t)g.B % 16)) {
            set_error("nn gemm: the tcgen05 path needs 16-byte aligned operands");
            return PCD_BAD_ARG;
        }
        PCD_TRY(gemm_tc(g, s));
    } else if (BN == 32) {
        PCD_CUDA(cudaFuncSetAttribute(k_gemm<32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_gemm<32><<<grid, GTHREADS, smem, s>>>(g);
    } else if (BN == 64) {
        PCD_CUDA(cudaFuncSetAttribute(k_gemm<64>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_gemm<64><<<grid, GTHREADS, smem, s>>>(g);
    } else {
        PCD_CUDA(cudaFuncSetAttribute(k_gemm<128>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_gemm<128><<<grid, GTHREADS, smem, s>>>(g);
    }
    if (!tc) PCD_LAUNCHED(1);
    if (g.ksplit > 1 && g.trans_c) {
        // the transposed partials reduce as an N x M matrix into C[n][m]
        splitk_reduce(partials, g.ksplit, g.N, Mo, Mo, nullptr, 0, nullptr, outF, ldo, s);
        PCD_LAUNCHED(1);
    } else if (g.ksplit > 1) {
        splitk_reduce(partials, g.ksplit, g.M, g.N, g.N, g.bias, g.relu, outB, outF, ldo, s);
        PCD_LAUNCHED(1);
    }
    return PCD_OK;
}

int im2col(const __nv_bfloat16 *in, int B, int H, int W, int C, int ldcin, __nv_bfloat16 *out, int Kp, cudaStream_t s)
{
    const long P = (long)B * H * W;
    if (C % 8 == 0 && ldcin % 8 == 0 && ((uintptr_t)in % 16) == 0) {
        k_im2col8<<<grid1d(P * (Kp / 8)), 256, 0, s>>>(in, B, H, W, C, ldcin, out, Kp);
    } else {
        k_im2col<<<grid1d(P * Kp), 256, 0, s>>>(in, B, H, W, C, ldcin, out, Kp);
    }
    PCD_LAUNCHED(1);
    return PCD_OK;
}

int transpose(const __nv_bfloat16 *in, int rows, int cols, int ldin, __nv_bfloat16 *out, int ldout, cudaStream_t s)
{
    const dim3 grid((cols + 31) / 32, (rows + 31) / 32);
    k_transpose<<<grid, dim3(32, 8), 0, s>>>(in, rows, cols, ldin, out, ldout);
    PCD_LAUNCHED(1);
    return PCD_OK;
}

int flip(const __nv_bfloat16 *Wt, int Cout, int Cin, int Kp, __nv_bfloat16 *Wf, int Kpf, cudaStream_t s)
{
    k_flip<<<grid1d((long)Cin * Kpf), 256, 0, s>>>(Wt, Cout, Cin, Kp, Wf, Kpf);
    PCD_LAUNCHED(1);
    return PCD_OK;
}

int relu_bwd(const float *dY, int lddy, const __nv_bfloat16 *Y, int ldy, long P, int C, int relu, __nv_bfloat16 *dYm,
             cudaStream_t s)
{
    k_relu_bwd<<<grid1d(P * C), 256, 0, s>>>(dY, lddy, Y, ldy, P, C, relu, dYm);
    PCD_LAUNCHED(1);
    return PCD_OK;
}

int relu_bwd_colsum(const float *dY, int lddy, const __nv_bfloat16 *Y, int ldy, long P, int C, int relu,
                    __nv_bfloat16 *dYm, float *part, long part_cap, float *db, cudaStream_t s)
{
    constexpr int kThreads = 256;
    if (C > kThreads || kThreads % C != 0) {
        PCD_TRY(relu_bwd(dY, lddy, Y, ldy, P, C, relu, dYm, s));
        return colsum(dYm, P, C, part, db, s);
    }
    // about 4096 values (16 a thread) per block, at most 1024 blocks (and what part holds)
    const int chunks = (int)std::max<long>(1, std::min<long>(std::min<long>((P * C + 4095) / 4096, 1024), part_cap / C));
    k_relu_bwd_colsum<<<chunks, kThreads, 0, s>>>(dY, lddy, Y, ldy, P, C, relu, dYm, part, chunks);
    PCD_LAUNCHED(1);
    k_colsum_fold_warp<<<(C + 7) / 8, 256, 0, s>>>(part, chunks, C, db);
    PCD_LAUNCHED(1);
    return PCD_OK;
}

int colsum(const __nv_bfloat16 *X, long P, int C, float *part, float *out, cudaStream_t s)
{
    const int chunks = 256;
    k_colsum<<<dim3((C + 63) / 64, chunks), 64, 0, s>>>(X, P, C, part, chunks);
    PCD_LAUNCHED(1);
    k_colsum_fold_warp<<<(C + 7) / 8, 256, 0, s>>>(part, chunks, C, out);
    PCD_LAUNCHED(1);
    return PCD_OK;
}

int colsum_f32(const float *part, int rows, int C, float *out, cudaStream_t s)
{
    k_colsum_fold_warp<<<(C + 7) / 8, 256, 0, s>>>(part, rows, C, out);
    PCD_LAUNCHED(1);
    return PCD_OK;
}

int pool(const __nv_bfloat16 *in, int B, int H, int W, int C, int ldin, __nv_bfloat16 *out, cudaStream_t s)
{
    k_pool<<<grid1d((long)B * (H / 2) * (W / 2) * C), 256, 0, s>>>(in, B, H, W, C, ldin, out);
    PCD_LAUNCHED(1);
    return PCD_OK;
}

int pool_bwd(const float *dOut, int B, int H, int W, int C, float *dIn, int lddin, cudaStream_t s)
{
    k_pool_bwd<<<grid1d((long)B * H * W * C), 256, 0, s>>>(dOut, B, H, W, C, dIn, lddin);
    PCD_LAUNCHED(1);
    return PCD_OK;
}

int up(const __nv_bfloat16 *in, int B, int H, int W, int C, __nv_bfloat16 *out, int ldout, cudaStream_t s)
{
    k_up<<<grid1d((long)B * 4 * H * W * C), 256, 0, s>>>(in, B, H, W, C, out, ldout);
    PCD_LAUNCHED(1);
    return PCD_OK;
}

int up_bwd(const float *dOut, int lddout, int B, int H, int W, int C, float *dIn, cudaStream_t s)
{
    k_up_bwd<<<grid1d((long)B * H * W * C), 256, 0, s>>>(dOut, lddout, B, H, W, C, dIn);
    PCD_LAUNCHED(1);
    return PCD_OK;
}

int head(const __nv_bfloat16 *X, long P, int C, const float *w, const float *bias, float *out, cudaStream_t s)
{
    k_head<<<grid1d(P), 256, 0, s>>>(X, P, C, w, bias, out);
    PCD_LAUNCHED(1);
    return PCD_OK;
}

int head_bwd(const float *d, const __nv_bfloat16 *X, long P, int C, const float *w, float *dX, float *part,
             int *nparts, cudaStream_t s)
{
    if (C > 32) {
        set_error("nn head: at most 32 channels");
        return PCD_BAD_ARG;
    }
    const int blocks = 512;
    k_head_bwd<<<blocks, 256, (256 / 32) * (C + 1) * sizeof(float), s>>>(d, X, P, C, w, dX, part);
    PCD_LAUNCHED(1);
    *nparts = blocks;
    return PCD_OK;
}

int mse(const float *pred, const float *tgt, long P1, int B, float *means, float *d, float *loss_part, int *nparts,
        cudaStream_t s)
{
    k_sample_means<<<B, 256, 0, s>>>(pred, tgt, P1, means);
    PCD_LAUNCHED(1);
    const int blocks = 512;
    k_mse<<<blocks, 256, 0, s>>>(pred, tgt, P1, B, means, d, loss_part);
    PCD_LAUNCHED(1);
    *nparts = blocks;
    return PCD_OK;
}

int adamw(float *w, const float *grad, float *m, float *v, long n, int cols, int ld, const AdamParams &p, int step,
          __nv_bfloat16 *wb, cudaStream_t s)
{
    const float bc1 = 1.f - powf(p.beta1, (float)step), bc2 = 1.f - powf(p.beta2, (float)step);
    k_adamw<<<grid1d(n), 256, 0, s>>>(w, grad, m, v, n, cols, ld, p.lr, p.beta1, p.beta2, p.eps, p.wd, bc1, bc2, wb);
    PCD_LAUNCHED(1);
    return PCD_OK;
}

int f32_to_bf16(const float *x, long n, __nv_bfloat16 *y, cudaStream_t s)
{
    k_f32_to_bf16<<<grid1d(n), 256, 0, s>>>(x, n, y);
    PCD_LAUNCHED(1);
    return PCD_OK;
}

int bf16_to_f32(const __nv_bfloat16 *x, long n, float *y, int ldx, int cols, cudaStream_t s)
{
    k_bf16_to_f32<<<grid1d(n), 256, 0, s>>>(x, n, y, ldx, cols);
    PCD_LAUNCHED(1);
    return PCD_OK;
}

int fill(float *x, long n, float v, cudaStream_t s)
{
    k_fill_f32<<<grid1d(n), 256, 0, s>>>(x, n, v);
    PCD_LAUNCHED(1);
    return PCD_OK;
}

int slice_add(const float *in, long P, int C, float *out, int ld, int accumulate, cudaStream_t s)
{
    k_slice_add<<<grid1d(P * C), 256, 0, s>>>(in, P, C, out, ld, accumulate);
    PCD_LAUNCHED(1);
    return PCD_OK;
}

}  // namespace nn
}  // namespace pcd
