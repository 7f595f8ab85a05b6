// nn.cuh -- kernels of the learned warm start (internal).
#pragma once

#include <cuda_bf16.h>

#include "common.cuh"

namespace pcd {
namespace nn {

struct GemmArgs {
    const __nv_bfloat16 *A;  // M x K, row stride lda
    int lda;
    const __nv_bfloat16 *B;  // N x K, row stride ldb
    int ldb;
    int M, N, K;             // K multiple of 32
    int ksplit;              // K splits (partials reduced in a fixed order)
    const float *bias;       // [N] or null
    int relu;
    __nv_bfloat16 *Cb;       // BF16 output (row stride ldc), or
    float *Cf;               // FP32 output
    int ldc;
    int path = 0;            // 0 automatic, 1 mma.sync, 2 tcgen05 (persistent, warp-specialised)
    // tcgen05 only: an operand stored K-rows x M (or N) contiguous ("MN-major",
    // e.g. A given as [K][M] with row stride lda), and C stored transposed
    // (C[n][m] at n * ldc + m; FP32 only, no bias or ReLU)
    int a_mn = 0, b_mn = 0, trans_c = 0;
    // tcgen05 only: A as the implicit im2col of a 3x3, pad-1 convolution's
    // input X (NHWC: xb images of xh x xw pixels, xc channels, pixel stride
    // lda; A points at X).  conv = 1: A[p][k] with k = (tap, chunk of cwid
    // channels), K tiles tap-major, B the weights [N][9 * xc] (k = tap * xc +
    // c); conv = 2: the transpose as an MN-major operand for the weight
    // gradient (M = 9 taps x nch chunks of cwid channels, K = pixels, C stored
    // transposed at row tap * xc + c).  cwid = 32 for xc = 32, else 64.
    int conv = 0, xb = 0, xh = 0, xw = 0, xc = 0, cwid = 64, nch = 1;
};

struct AdamParams {
    float lr, beta1, beta2, eps, wd;
};

size_t gemm_smem(int BN);
// partials: ksplit * M * N floats when ksplit > 1
int gemm(const GemmArgs &g, cudaStream_t s, float *partials);
// The tcgen05 form (nn_tc.cu): whether it takes g (16-byte aligned operands,
// K >= 64), whether its output tiles fill the chip (at least one per SM; the
// automatic choice takes it only then), the launch (split-K partials to
// g.Cf), and the error word its bounded waits set (PCD_TIMEOUT).
bool gemm_tc_applies(const GemmArgs &g);
bool gemm_tc_fills_chip(const GemmArgs &g);
int gemm_tc(const GemmArgs &g, cudaStream_t s);
int gemm_tc_error(int *out, bool reset);
// Everything the tcgen05 form sets up on first use (its error word, the
// kernels' shared-memory attributes on the current device), done ahead so
// that no allocation falls inside a stream capture; the error word itself.
int gemm_tc_prepare();
// Reads the current device's error word on stream s (synchronising it); a
// nonzero word (a wait gave up, its tile left unwritten) is reset and
// reported as PCD_DEVICE_ERROR.
int gemm_tc_check(cudaStream_t s);
// What path 0 means for the whole process: 0 tcgen05 where it applies, else
// mma.sync; 1 mma.sync always.
int set_default_path(int path);
int default_path();
int sm_count();  // of the current device
// The 3x3, pad-1 convolution on the tcgen05 kernel without an im2col matrix
// (4-D TMA boxes of the NHWC input, zero-filled outside the image).
// conv_tc_applies: whether x (B images of H x W, C >= 32 channels at pixel
// stride ldx) takes it with T-pixel boxes (T = 128: conv3x3_tc; T = 64:
// conv3x3_wgrad_tc).  conv3x3_tc: out[p][n] = sum_{tap, c} x[p + tap][c]
// w[n][tap * C + c] (+ bias, ReLU), BF16 or FP32; conv3x3_wgrad_tc:
// dw[n][tap * C + c] = sum_p x[p + tap][c] dy[p][n] (dy dense [P][N]).
bool conv_tc_applies(const void *x, int B, int H, int W, int C, int ldx, int T);
int conv3x3_tc(const __nv_bfloat16 *x, int B, int H, int W, int C, int ldx, const __nv_bfloat16 *w, int ldw, int N,
               const float *bias, int relu, __nv_bfloat16 *Cb, float *Cf, int ldc, int ksplit, float *partials,
               cudaStream_t s);
int conv3x3_wgrad_tc(const __nv_bfloat16 *x, int B, int H, int W, int C, int ldx, const __nv_bfloat16 *dy, int N,
                     float *dw, int ldw, int ksplit, float *partials, cudaStream_t s);
int im2col(const __nv_bfloat16 *in, int B, int H, int W, int C, int ldcin, __nv_bfloat16 *out, int Kp, cudaStream_t s);
int transpose(const __nv_bfloat16 *in, int rows, int cols, int ldin, __nv_bfloat16 *out, int ldout, cudaStream_t s);
int flip(const __nv_bfloat16 *Wt, int Cout, int Cin, int Kp, __nv_bfloat16 *Wf, int Kpf, cudaStream_t s);
int relu_bwd(const float *dY, int lddy, const __nv_bfloat16 *Y, int ldy, long P, int C, int relu, __nv_bfloat16 *dYm,
             cudaStream_t s);
// relu_bwd and the bias gradient db[c] = sum_p dYm[p][c] in one pass over
// dY (part: scratch of part_cap floats for the per-block sums)
int relu_bwd_colsum(const float *dY, int lddy, const __nv_bfloat16 *Y, int ldy, long P, int C, int relu,
                    __nv_bfloat16 *dYm, float *part, long part_cap, float *db, cudaStream_t s);
int colsum(const __nv_bfloat16 *X, long P, int C, float *part, float *out, cudaStream_t s);
// out[c] = sum over rows of part[r][c] (FP32, fixed order)
int colsum_f32(const float *part, int rows, int C, float *out, cudaStream_t s);
int pool(const __nv_bfloat16 *in, int B, int H, int W, int C, int ldin, __nv_bfloat16 *out, cudaStream_t s);
int pool_bwd(const float *dOut, int B, int H, int W, int C, float *dIn, int lddin, cudaStream_t s);
int up(const __nv_bfloat16 *in, int B, int H, int W, int C, __nv_bfloat16 *out, int ldout, cudaStream_t s);
int up_bwd(const float *dOut, int lddout, int B, int H, int W, int C, float *dIn, cudaStream_t s);
int head(const __nv_bfloat16 *X, long P, int C, const float *w, const float *bias, float *out, cudaStream_t s);
int head_bwd(const float *d, const __nv_bfloat16 *X, long P, int C, const float *w, float *dX, float *part,
             int *nparts, cudaStream_t s);
int mse(const float *pred, const float *tgt, long P1, int B, float *means, float *d, float *loss_part, int *nparts,
        cudaStream_t s);
int adamw(float *w, const float *grad, float *m, float *v, long n, int cols, int ld, const AdamParams &p, int step,
          __nv_bfloat16 *wb, cudaStream_t s);
int f32_to_bf16(const float *x, long n, __nv_bfloat16 *y, cudaStream_t s);
int bf16_to_f32(const __nv_bfloat16 *x, long n, float *y, int ldx, int cols, cudaStream_t s);
int fill(float *x, long n, float v, cudaStream_t s);
int slice_add(const float *in, long P, int C, float *out, int ld, int accumulate, cudaStream_t s);

}  // namespace nn
}  // namespace pcd
