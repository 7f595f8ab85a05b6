// unet.cu -- the learned warm start: a 4-level BF16 U-Net on tensor cores.
//
// Topology (3x3 convolutions with ReLU, NHWC, S = training resolution):
//   e1a 1->32, e1b 32->32 @S      -> skip1     pool
//   e2a 32->64, e2b 64->64 @S/2   -> skip2     pool
//   e3a 64->128, e3b 128->128 @S/4 -> skip3    pool
//   bta 128->256, btb 256->256 @S/8
//   up, [up | skip3] = 384 -> d3a 128, d3b 128 @S/4
//   up, [up | skip2] = 192 -> d2a 64,  d2b 64  @S/2
//   up, [up | skip1] =  96 -> d1a 32,  d1b 32  @S
//   head: 1x1, 32 -> 1 (FP32, no activation)
// Pooling is a 2x2 average, upsampling nearest; the concatenations are
// zero-copy: the encoder's second convolution of each level writes straight
// into the channel slice of the decoder's input buffer.
//
// Every convolution runs im2col + the tensor-core GEMM of nn.cu (BF16 inputs,
// FP32 accumulation); training keeps FP32 master weights, FP32 gradients and
// AdamW state.  The network maps a normalised density residual x = b / std(b)
// to phi_hat = phi / (std(b) * S^2) with the mean removed (the Neumann
// solution is defined up to a constant); the loss is the mean squared error
// of the mean-removed prediction.
#include <cmath>
#include <cstring>
#include <random>
#include <algorithm>
#include <vector>

#include "api_internal.cuh"
#include "nn.cuh"
#include "unet.cuh"

namespace pcd {

namespace {

inline int round32(int k) { return (k + 31) / 32 * 32; }

// binomial filter passes on a prediction before it is interpolated to the grid
constexpr int kPredFilter = 4;
inline int grid1d(long n) { return (int)std::max<long>(1, std::min<long>(8192, (n + 255) / 256)); }

// b (FP64, W x H, ld) -> x (FP32, S x S): area-average / nearest resample
__global__ void k_resample_in(const double *b, int W, int H, int ld, float *x, int S)
{
    const long total = (long)S * S;
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
        const int yo = (int)(t / S), xo = (int)(t - (long)yo * S);
        const int y0 = (int)((long)yo * H / S), y1 = max(y0 + 1, (int)((long)(yo + 1) * H / S));
        const int x0 = (int)((long)xo * W / S), x1 = max(x0 + 1, (int)((long)(xo + 1) * W / S));
        double s = 0.0;
        for (int y = y0; y < y1; y++)
            for (int xx = x0; xx < x1; xx++) s += b[(size_t)y * ld + xx];
        x[t] = (float)(s / ((y1 - y0) * (x1 - x0)));
    }
}

// per-sample mean and inverse std of x (S*S values), one block per sample
__global__ void k_norm_stats(const float *x, long n, float *stats)
{
    const float *p = x + (size_t)blockIdx.x * n;
    double v[2] = {0.0, 0.0};
    for (long i = threadIdx.x; i < n; i += blockDim.x) {
        v[0] += p[i];
        v[1] += (double)p[i] * p[i];
    }
    block_reduce<2, 0u>(v);
    if (threadIdx.x == 0) {
        const double mean = v[0] / n, var = fmax(v[1] / n - mean * mean, 1e-30);
        stats[2 * blockIdx.x] = (float)mean;
        stats[2 * blockIdx.x + 1] = (float)(1.0 / sqrt(var));
    }
}

// x -> bf16 (x - mean) * inv_std
__global__ void k_normalize(const float *x, long n, int B, const float *stats, __nv_bfloat16 *out)
{
    const long total = n * B;
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
        const int s = (int)(t / n);
        out[t] = __float2bfloat16((x[t] - stats[2 * s]) * stats[2 * s + 1]);
    }
}

// phi0 (FP64, W x H, ld) = wh * std(x) * bilinear(phi_hat (S x S)), std from
// stats[1] = 1 / std of the network input
__global__ void k_resample_out(const float *ph, int S, const float *stats, double wh, double *phi, int W, int H,
                               int ld)
{
    const double scale = wh / (double)stats[1];
    const long total = (long)W * H;
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
        const int y = (int)(t / W), x = (int)(t - (long)y * W);
        // cell-centred coordinates
        const float fy = fminf(fmaxf((y + 0.5f) * S / H - 0.5f, 0.f), (float)(S - 1));
        const float fx = fminf(fmaxf((x + 0.5f) * S / W - 0.5f, 0.f), (float)(S - 1));
        const int y0 = (int)fy, x0 = (int)fx, y1 = min(y0 + 1, S - 1), x1 = min(x0 + 1, S - 1);
        const float ty = fy - y0, tx = fx - x0;
        const float v = (1 - ty) * ((1 - tx) * ph[y0 * S + x0] + tx * ph[y0 * S + x1]) +
                        ty * ((1 - tx) * ph[y1 * S + x0] + tx * ph[y1 * S + x1]);
        phi[(size_t)y * ld + x] = scale * (double)v;
    }
}

// One pass of the 3x3 binomial filter [1 2 1]^T [1 2 1] / 16 on an S x S
// field (edge cells reuse the nearest cell).
__global__ void k_binomial(const float *__restrict__ in, float *__restrict__ out, int S)
{
    const long total = (long)S * S;
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
        const int y = (int)(t / S), x = (int)(t - (long)y * S);
        const int ym = max(y - 1, 0), yp = min(y + 1, S - 1), xm = max(x - 1, 0), xp = min(x + 1, S - 1);
        const float r0 = in[ym * S + xm] + 2.f * in[ym * S + x] + in[ym * S + xp];
        const float r1 = in[y * S + xm] + 2.f * in[y * S + x] + in[y * S + xp];
        const float r2 = in[yp * S + xm] + 2.f * in[yp * S + x] + in[yp * S + xp];
        out[t] = (r0 + 2.f * r1 + r2) * (1.f / 16.f);
    }
}

}  // namespace

// ---------------------------------------------------------------------------
struct UNet::Conv {
    int Cin, Cout, Kp, Kpf, relu;
    int S;                  // spatial side at this layer
    size_t off_w, off_b;    // parameter offsets (floats) in the flat FP32 arrays
    __nv_bfloat16 *wb = nullptr;  // [Cout][Kp]
    __nv_bfloat16 *wf = nullptr;  // [Cin][Kpf]
    __nv_bfloat16 *col = nullptr; // [P][Kp]
    bool col_valid = false;       // col holds the last forward pass's im2col
    const __nv_bfloat16 *in = nullptr;
    int ldin = 0;
    __nv_bfloat16 *out = nullptr;
    int ldout = 0;
};

UNet::~UNet() { release(); }

void UNet::release()
{
    if (arena) cudaFree(arena);
    arena = nullptr;
    if (params_f) cudaFree(params_f);
    params_f = nullptr;
    convs.clear();
}

int UNet::build(int S_, int maxB_)
{
    S = S_;
    maxB = maxB_;
    if (S < 16 || S % 8 != 0 || maxB < 1) {
        set_error("pcd_unet_create: the resolution must be a multiple of 8 (>= 16) and the batch >= 1");
        return PCD_BAD_ARG;
    }
    // layers: (Cin, Cout, level)
    struct L { int cin, cout, lvl; };
    const std::vector<L> spec = {
        {1, 32, 0}, {32, 32, 0},   {32, 64, 1},  {64, 64, 1},   {64, 128, 2}, {128, 128, 2},
        {128, 256, 3}, {256, 256, 3}, {384, 128, 2}, {128, 128, 2}, {192, 64, 1}, {64, 64, 1},
        {96, 32, 0},  {32, 32, 0}};
    convs.clear();
    size_t np = 0;
    for (auto &l : spec) {
        Conv c;
        c.Cin = l.cin;
        c.Cout = l.cout;
        c.Kp = round32(9 * l.cin);
        c.Kpf = round32(9 * l.cout);
        c.relu = 1;
        c.S = S >> l.lvl;
        c.off_w = np;
        np += (size_t)c.Cout * c.Kp;
        c.off_b = np;
        np += c.Cout;
        convs.push_back(c);
    }
    head_w = np;
    np += 32;
    head_b = np;
    np += 1;
    nparams = np;
    // FP32 master, grad, adam m, v: 4 * np floats
    PCD_CUDA(cudaMalloc(&params_f, 4 * np * sizeof(float)));
    PCD_CUDA(cudaMemset(params_f, 0, 4 * np * sizeof(float)));

    // arena layout (bytes), sized for maxB
    const long P0 = (long)maxB * S * S, P1 = P0 / 4, P2 = P0 / 16, P3 = P0 / 64;
    auto bf = [](long n) { return (size_t)((n * 2 + 255) / 256 * 256); };
    auto f4 = [](long n) { return (size_t)((n * 4 + 255) / 256 * 256); };
    std::vector<std::pair<void **, size_t>> plan;
    plan.push_back({(void **)&x_in, bf(P0)});
    plan.push_back({(void **)&t1, bf(P0 * 32)});
    plan.push_back({(void **)&cat1, bf(P0 * 96)});
    plan.push_back({(void **)&p1, bf(P1 * 32)});
    plan.push_back({(void **)&t2, bf(P1 * 64)});
    plan.push_back({(void **)&cat2, bf(P1 * 192)});
    plan.push_back({(void **)&p2, bf(P2 * 64)});
    plan.push_back({(void **)&t3, bf(P2 * 128)});
    plan.push_back({(void **)&cat3, bf(P2 * 384)});
    plan.push_back({(void **)&p3, bf(P3 * 128)});
    plan.push_back({(void **)&t4, bf(P3 * 256)});
    plan.push_back({(void **)&u4, bf(P3 * 256)});
    plan.push_back({(void **)&t5, bf(P2 * 128)});
    plan.push_back({(void **)&u3, bf(P2 * 128)});
    plan.push_back({(void **)&t6, bf(P1 * 64)});
    plan.push_back({(void **)&u2, bf(P1 * 64)});
    plan.push_back({(void **)&t7, bf(P0 * 32)});
    plan.push_back({(void **)&u1, bf(P0 * 32)});
    plan.push_back({(void **)&pred, f4(P0)});
    // im2col per layer
    for (auto &c : convs) plan.push_back({(void **)&c.col, bf((long)maxB * c.S * c.S * c.Kp)});
    // backward scratch: largest P*C (fp32 gradients), transposes, dX im2col
    long maxPK = 0, maxPC = 0, maxPKf = 0;
    for (auto &c : convs) {
        const long P = (long)maxB * c.S * c.S;
        maxPK = std::max(maxPK, P * c.Kp);
        maxPKf = std::max(maxPKf, P * c.Kpf);
        maxPC = std::max(maxPC, P * std::max(c.Cin, c.Cout));
    }
    maxPC = std::max(maxPC, P0 * 96);
    plan.push_back({(void **)&g_a, f4(maxPC)});     // gradient ping
    plan.push_back({(void **)&g_b, f4(maxPC)});     // gradient pong
    plan.push_back({(void **)&g_cat, f4(P0 * 96)}); // concat gradients (per level, reused)
    plan.push_back({(void **)&g_cat2, f4(P1 * 192)});
    plan.push_back({(void **)&g_cat3, f4(P2 * 384)});
    plan.push_back({(void **)&dym, bf(maxPC)});
    plan.push_back({(void **)&tr_a, bf(maxPC)});
    plan.push_back({(void **)&tr_b, bf(maxPK)});
    plan.push_back({(void **)&colD, bf(maxPKf)});
    plan.push_back({(void **)&wflip, bf(256 * round32(9 * 384))});
    partials_cap = 32L * 256 * round32(9 * 384);
    plan.push_back({(void **)&partials, f4((long)partials_cap)});
    plan.push_back({(void **)&colpart, f4(kColpartCap)});
    plan.push_back({(void **)&small, f4(512L * 33)});
    plan.push_back({(void **)&lossbuf, f4(4096)});
    plan.push_back({(void **)&xin_f, f4(P0)});
    plan.push_back({(void **)&stats, f4(2L * maxB)});
    plan.push_back({(void **)&dpred, f4(P0)});
    for (auto &c : convs) {
        plan.push_back({(void **)&c.wb, bf((long)c.Cout * c.Kp)});
    }
    size_t total = 0;
    for (auto &pe : plan) total += pe.second;
    PCD_CUDA(cudaMalloc(&arena, total));
    PCD_CUDA(cudaMemset(arena, 0, total));
    size_t o = 0;
    for (auto &pe : plan) {
        *pe.first = (unsigned char *)arena + o;
        o += pe.second;
    }
    // wiring (ld = channel stride of the buffer a layer reads / writes)
    Conv *c = convs.data();
    c[0].in = x_in;  c[0].ldin = 1;   c[0].out = t1;         c[0].ldout = 32;
    c[1].in = t1;    c[1].ldin = 32;  c[1].out = cat1 + 64;  c[1].ldout = 96;
    c[2].in = p1;    c[2].ldin = 32;  c[2].out = t2;         c[2].ldout = 64;
    c[3].in = t2;    c[3].ldin = 64;  c[3].out = cat2 + 128; c[3].ldout = 192;
    c[4].in = p2;    c[4].ldin = 64;  c[4].out = t3;         c[4].ldout = 128;
    c[5].in = t3;    c[5].ldin = 128; c[5].out = cat3 + 256; c[5].ldout = 384;
    c[6].in = p3;    c[6].ldin = 128; c[6].out = t4;         c[6].ldout = 256;
    c[7].in = t4;    c[7].ldin = 256; c[7].out = u4;         c[7].ldout = 256;
    c[8].in = cat3;  c[8].ldin = 384; c[8].out = t5;         c[8].ldout = 128;
    c[9].in = t5;    c[9].ldin = 128; c[9].out = u3;         c[9].ldout = 128;
    c[10].in = cat2; c[10].ldin = 192; c[10].out = t6;       c[10].ldout = 64;
    c[11].in = t6;   c[11].ldin = 64; c[11].out = u2;        c[11].ldout = 64;
    c[12].in = cat1; c[12].ldin = 96; c[12].out = t7;        c[12].ldout = 32;
    c[13].in = t7;   c[13].ldin = 32; c[13].out = u1;        c[13].ldout = 32;
    step = 0;
    return PCD_OK;
}

int UNet::init_random(unsigned long long seed)
{
    std::vector<float> h(nparams, 0.f);
    std::mt19937_64 rng(seed);
    for (auto &c : convs) {
        std::normal_distribution<float> nd(0.f, std::sqrt(2.f / (9.f * c.Cin)));  // He initialisation
        for (int co = 0; co < c.Cout; co++)
            for (int k = 0; k < 9 * c.Cin; k++) h[c.off_w + (size_t)co * c.Kp + k] = nd(rng);
    }
    std::normal_distribution<float> nh(0.f, std::sqrt(1.f / 32.f));
    for (int k = 0; k < 32; k++) h[head_w + k] = nh(rng);
    return set_params(h.data());
}

int UNet::set_params(const float *host)
{
    PCD_CUDA(cudaMemcpy(params_f, host, nparams * sizeof(float), cudaMemcpyHostToDevice));
    PCD_CUDA(cudaMemset(params_f + 2 * nparams, 0, 2 * nparams * sizeof(float)));
    step = 0;
    PCD_TRY(sync_bf16(nullptr));
    PCD_CUDA(cudaDeviceSynchronize());
    return PCD_OK;
}

int UNet::get_params(float *host)
{
    PCD_CUDA(cudaMemcpy(host, params_f, nparams * sizeof(float), cudaMemcpyDeviceToHost));
    return PCD_OK;
}

int UNet::sync_bf16(cudaStream_t s)
{
    for (auto &c : convs) PCD_TRY(nn::f32_to_bf16(params_f + c.off_w, (long)c.Cout * c.Kp, c.wb, s));
    return PCD_OK;
}

// output tiles of a [P x N] result on the tcgen05 kernel
static long tc_tiles(long P, int N)
{
    const int bn = N <= 32 ? 32 : (N <= 64 ? 64 : (N <= 128 ? 128 : 256));
    return ((P + 127) / 128) * ((N + bn - 1) / bn);
}

// K splits for an implicit convolution on the tcgen05 kernel whose output
// tiles do not fill the chip: enough for about one unit per SM, at most the
// K tiles (taps x channel chunks) and what the partial buffer holds
int UNet::conv_splits(long P, int N, int Cin) const
{
    const long tiles = tc_tiles(P, N), sms = nn::sm_count();
    if (tiles >= sms) return 1;
    const int kt = 9 * (Cin == 32 ? 1 : (Cin + 63) / 64);
    int ks = (int)std::min<long>(std::min<long>((sms + tiles - 1) / tiles, kt), 16);
    while (ks > 1 && (size_t)ks * P * N > partials_cap) ks /= 2;
    return std::max(1, ks);
}

int UNet::conv_fwd(Conv &c, int B, cudaStream_t s)
{
    // an implicit GEMM on the tcgen05 kernel (no im2col matrix; split-K where
    // its tiles do not fill the chip); otherwise im2col and the GEMM
    const long P = (long)B * c.S * c.S;
    c.col_valid = false;
    if (nn::default_path() == 0 && c.Kp == 9 * c.Cin && nn::conv_tc_applies(c.in, B, c.S, c.S, c.Cin, c.ldin, 128)) {
        const int ks = conv_splits(P, c.Cout, c.Cin);
        return nn::conv3x3_tc(c.in, B, c.S, c.S, c.Cin, c.ldin, c.wb, c.Kp, c.Cout, params_f + c.off_b, c.relu, c.out,
                              nullptr, c.ldout, ks, partials, s);
    }
    PCD_TRY(nn::im2col(c.in, B, c.S, c.S, c.Cin, c.ldin, c.col, c.Kp, s));
    c.col_valid = true;
    nn::GemmArgs g{};
    g.A = c.col;
    g.lda = c.Kp;
    g.B = c.wb;
    g.ldb = c.Kp;
    g.M = B * c.S * c.S;
    g.N = c.Cout;
    g.K = c.Kp;
    g.bias = params_f + c.off_b;
    g.relu = c.relu;
    g.Cb = c.out;
    g.ldc = c.ldout;
    // Small grids (the 64² warm start: 2 to 32 output tiles on the coarse
    // levels): split K so that about 128 CTAs share the reduction, each with
    // at least two 32-wide k-tiles, partials summed in a fixed order by
    // nn::gemm (the training forward pass at full batch keeps one split).
    const int bn = g.N <= 32 ? 32 : (g.N <= 64 ? 64 : 128);
    const long tiles = (long)((g.N + bn - 1) / bn) * ((g.M + 127) / 128);
    const int kt = g.K / 32;
    g.ksplit = 1;
    if (tiles < 64 && kt >= 4) {
        const long want = (128 + tiles - 1) / tiles;
        g.ksplit = (int)std::min<long>(std::min<long>(want, kt / 2), 32);
        // the split-K partials must fit the shared partial buffer
        while (g.ksplit > 1 && (size_t)g.ksplit * g.M * g.N > partials_cap) g.ksplit /= 2;
    }
    return nn::gemm(g, s, g.ksplit > 1 ? partials : nullptr);
}

int UNet::forward(int B, cudaStream_t s)
{
    Conv *c = convs.data();
    const int S0 = S, S1 = S / 2, S2 = S / 4, S3 = S / 8;
    PCD_TRY(conv_fwd(c[0], B, s));
    PCD_TRY(conv_fwd(c[1], B, s));
    PCD_TRY(nn::pool(cat1 + 64, B, S0, S0, 32, 96, p1, s));
    PCD_TRY(conv_fwd(c[2], B, s));
    PCD_TRY(conv_fwd(c[3], B, s));
    PCD_TRY(nn::pool(cat2 + 128, B, S1, S1, 64, 192, p2, s));
    PCD_TRY(conv_fwd(c[4], B, s));
    PCD_TRY(conv_fwd(c[5], B, s));
    PCD_TRY(nn::pool(cat3 + 256, B, S2, S2, 128, 384, p3, s));
    PCD_TRY(conv_fwd(c[6], B, s));
    PCD_TRY(conv_fwd(c[7], B, s));
    PCD_TRY(nn::up(u4, B, S3, S3, 256, cat3, 384, s));
    PCD_TRY(conv_fwd(c[8], B, s));
    PCD_TRY(conv_fwd(c[9], B, s));
    PCD_TRY(nn::up(u3, B, S2, S2, 128, cat2, 192, s));
    PCD_TRY(conv_fwd(c[10], B, s));
    PCD_TRY(conv_fwd(c[11], B, s));
    PCD_TRY(nn::up(u2, B, S1, S1, 64, cat1, 96, s));
    PCD_TRY(conv_fwd(c[12], B, s));
    PCD_TRY(conv_fwd(c[13], B, s));
    PCD_TRY(nn::head(u1, (long)B * S0 * S0, 32, params_f + head_w, params_f + head_b, pred, s));
    return PCD_OK;
}

// dY: FP32 gradient of c.out (channel stride lddy); writes dX (dense FP32
// [P][Cin]) unless dX is null; accumulates the weight and bias gradients.
int UNet::conv_bwd(Conv &c, int B, const float *dY, int lddy, float *dX, cudaStream_t s)
{
    const long P = (long)B * c.S * c.S;
    float *gw = params_f + nparams + c.off_w, *gb = params_f + nparams + c.off_b;
    PCD_TRY(nn::relu_bwd_colsum(dY, lddy, c.out, c.ldout, P, c.Cout, c.relu, dym, colpart, kColpartCap, gb, s));
    const int sms = nn::sm_count();
    if (nn::default_path() == 0 && c.Kp == 9 * c.Cin && nn::conv_tc_applies(c.in, B, c.S, c.S, c.Cin, c.ldin, 64)) {
        // dW[Cout][(tap, c)] = sum_p x[p + tap][c] dYm[p][Cout]: the implicit
        // transposed im2col of the input (MN-major 4-D boxes) against dYm,
        // K = P split so that about two CTAs per SM share it
        const int cw = c.Cin == 32 ? 32 : 64;
        const long Mpad = 9L * ((c.Cin + cw - 1) / cw) * cw;
        const long tiles = tc_tiles(Mpad, c.Cout);
        const long kt = (P + 63) / 64;
        int ks = (int)std::max<long>(1, std::min<long>(std::min<long>((2L * sms + tiles - 1) / tiles, kt), 128));
        while (ks > 1 && (size_t)ks * c.Kp * c.Cout > partials_cap) ks /= 2;
        PCD_TRY(nn::conv3x3_wgrad_tc(c.in, B, c.S, c.S, c.Cin, c.ldin, dym, c.Cout, gw, c.Kp, ks, partials, s));
    } else {
        if (!c.col_valid) {
            PCD_TRY(nn::im2col(c.in, B, c.S, c.S, c.Cin, c.ldin, c.col, c.Kp, s));
            c.col_valid = true;
        }
        nn::GemmArgs g{};
        // dW^T[Kp][Cout] = col^T (Kp x P) * dYm (P x Cout) on the tcgen05 kernel,
        // both operands read where they lie (MN-major: col is [P][Kp], dYm
        // [P][Cout]) and the result stored transposed into dW[Cout][Kp]; K = P
        // split so that about two CTAs per SM share it
        nn::GemmArgs mn{};
        mn.A = c.col;
        mn.lda = c.Kp;
        mn.a_mn = 1;
        mn.B = dym;
        mn.ldb = c.Cout;
        mn.b_mn = 1;
        mn.M = c.Kp;
        mn.N = c.Cout;
        mn.K = (int)P;
        mn.trans_c = 1;
        if (nn::default_path() == 0 && nn::gemm_tc_applies(mn)) {
            g = mn;
            const int bn = c.Cout <= 32 ? 32 : (c.Cout <= 64 ? 64 : (c.Cout <= 128 ? 128 : 256));
            const long tiles = (long)((c.Kp + 127) / 128) * ((c.Cout + bn - 1) / bn);
            const long kt = (P + 63) / 64;
            g.ksplit = (int)std::max<long>(1, std::min<long>(std::min<long>((2L * sms + tiles - 1) / tiles, kt), 128));
            while (g.ksplit > 1 && (size_t)g.ksplit * g.M * g.N > partials_cap) g.ksplit /= 2;
        } else {
            // dW[Cout][Kp] = dYm^T (Cout x P) * col (P x Kp): both operands
            // transposed to K = P contiguous for the mma.sync kernel
            PCD_TRY(nn::transpose(dym, (int)P, c.Cout, c.Cout, tr_a, (int)P, s));
            PCD_TRY(nn::transpose(c.col, (int)P, c.Kp, c.Kp, tr_b, (int)P, s));
            g.A = tr_a;
            g.lda = (int)P;
            g.B = tr_b;
            g.ldb = (int)P;
            g.M = c.Cout;
            g.N = c.Kp;
            g.K = (int)P;
            const int tiles = ((c.Kp + 127) / 128) * ((c.Cout + 127) / 128);
            g.ksplit = std::max(1, std::min(32, 1216 / tiles));
        }
        g.Cf = gw;
        g.ldc = c.Kp;
        PCD_TRY(nn::gemm(g, s, partials));
    }
    if (dX) {
        // dX = conv(dYm, flipped weights): implicit on the tcgen05 kernel,
        // else through im2col
        PCD_TRY(nn::flip(c.wb, c.Cout, c.Cin, c.Kp, wflip, c.Kpf, s));
        if (nn::default_path() == 0 && c.Kpf == 9 * c.Cout && nn::conv_tc_applies(dym, B, c.S, c.S, c.Cout, c.Cout, 128))
            return nn::conv3x3_tc(dym, B, c.S, c.S, c.Cout, c.Cout, wflip, c.Kpf, c.Cin, nullptr, 0, nullptr, dX, c.Cin,
                                  conv_splits(P, c.Cin, c.Cout), partials, s);
        PCD_TRY(nn::im2col(dym, B, c.S, c.S, c.Cout, c.Cout, colD, c.Kpf, s));
        nn::GemmArgs d{};
        d.A = colD;
        d.lda = c.Kpf;
        d.B = wflip;
        d.ldb = c.Kpf;
        d.M = (int)P;
        d.N = c.Cin;
        d.K = c.Kpf;
        d.ksplit = 1;
        d.Cf = dX;
        d.ldc = c.Cin;
        PCD_TRY(nn::gemm(d, s, nullptr));
    }
    return PCD_OK;
}

int UNet::backward(int B, cudaStream_t s)
{
    Conv *c = convs.data();
    const int S0 = S, S1 = S / 2, S2 = S / 4, S3 = S / 8;
    const long P0 = (long)B * S0 * S0, P1 = P0 / 4, P2 = P0 / 16, P3 = P0 / 64;
    float *gp = params_f + nparams;
    // head: d(pred) -> d(u1) [P0 x 32], head weight/bias gradients
    int np = 0;
    PCD_TRY(nn::head_bwd(dpred, u1, P0, 32, params_f + head_w, g_a, small, &np, s));
    PCD_TRY(nn::colsum_f32(small, np, 33, gp + head_w, s));
    // level 1 decoder
    PCD_TRY(conv_bwd(c[13], B, g_a, 32, g_b, s));        // d(t7)
    PCD_TRY(conv_bwd(c[12], B, g_b, 32, g_cat, s));      // d(cat1) [P0 x 96]
    PCD_TRY(nn::up_bwd(g_cat, 96, B, S1, S1, 64, g_a, s));  // d(u2) [P1 x 64]
    PCD_TRY(conv_bwd(c[11], B, g_a, 64, g_b, s));        // d(t6)
    PCD_TRY(conv_bwd(c[10], B, g_b, 64, g_cat2, s));     // d(cat2) [P1 x 192]
    PCD_TRY(nn::up_bwd(g_cat2, 192, B, S2, S2, 128, g_a, s));  // d(u3) [P2 x 128]
    PCD_TRY(conv_bwd(c[9], B, g_a, 128, g_b, s));        // d(t5)
    PCD_TRY(conv_bwd(c[8], B, g_b, 128, g_cat3, s));     // d(cat3) [P2 x 384]
    PCD_TRY(nn::up_bwd(g_cat3, 384, B, S3, S3, 256, g_a, s));  // d(u4) [P3 x 256]
    PCD_TRY(conv_bwd(c[7], B, g_a, 256, g_b, s));        // d(t4)
    PCD_TRY(conv_bwd(c[6], B, g_b, 256, g_a, s));        // d(p3) [P3 x 128]
    // level 3 encoder: skip3 gradient = decoder slice + pool gradient
    PCD_TRY(nn::pool_bwd(g_a, B, S2, S2, 128, g_cat3 + 256, 384, s));
    PCD_TRY(conv_bwd(c[5], B, g_cat3 + 256, 384, g_b, s));  // d(t3)
    PCD_TRY(conv_bwd(c[4], B, g_b, 128, g_a, s));            // d(p2) [P2 x 64]
    PCD_TRY(nn::pool_bwd(g_a, B, S1, S1, 64, g_cat2 + 128, 192, s));
    PCD_TRY(conv_bwd(c[3], B, g_cat2 + 128, 192, g_b, s));  // d(t2)
    PCD_TRY(conv_bwd(c[2], B, g_b, 64, g_a, s));             // d(p1) [P1 x 32]
    PCD_TRY(nn::pool_bwd(g_a, B, S0, S0, 32, g_cat + 64, 96, s));
    PCD_TRY(conv_bwd(c[1], B, g_cat + 64, 96, g_b, s));     // d(t1)
    PCD_TRY(conv_bwd(c[0], B, g_b, 32, nullptr, s));         // input gradient not needed
    (void)P1; (void)P2; (void)P3;
    return PCD_OK;
}

int UNet::load_input(const float *x, int B, cudaStream_t s)
{
    const long n = (long)S * S;
    k_norm_stats<<<B, 256, 0, s>>>(x, n, stats);
    PCD_LAUNCHED(1);
    k_normalize<<<grid1d(n * B), 256, 0, s>>>(x, n, B, stats, x_in);
    PCD_LAUNCHED(1);
    return PCD_OK;
}

int UNet::train_step(const float *x, const float *target, int B, const nn::AdamParams &ap, float *loss,
                     cudaStream_t s)
{
    if (B < 1 || B > maxB) {
        set_error("pcd_unet_train_step: batch out of range");
        return PCD_BAD_ARG;
    }
    PCD_TRY(load_input(x, B, s));
    PCD_TRY(forward(B, s));
    int np = 0;
    const long P1 = (long)S * S;
    PCD_TRY(nn::mse(pred, target, P1, B, lossbuf, dpred, lossbuf + 64, &np, s));
    // zero gradients, backward, AdamW
    PCD_CUDA(cudaMemsetAsync(params_f + nparams, 0, nparams * sizeof(float), s));
    PCD_CUDA(cudaMemsetAsync(g_cat, 0, (size_t)B * S * S * 96 * sizeof(float), s));
    PCD_CUDA(cudaMemsetAsync(g_cat2, 0, (size_t)B * S * S / 4 * 192 * sizeof(float), s));
    PCD_CUDA(cudaMemsetAsync(g_cat3, 0, (size_t)B * S * S / 16 * 384 * sizeof(float), s));
    PCD_TRY(backward(B, s));
    ++step;
    float *w = params_f, *gr = params_f + nparams, *m = params_f + 2 * nparams, *v = params_f + 3 * nparams;
    // one AdamW pass over the flat parameter array; then refresh the BF16 copies
    PCD_TRY(nn::adamw(w, gr, m, v, (long)nparams, (int)nparams, (int)nparams, ap, step, nullptr, s));
    PCD_TRY(sync_bf16(s));
    if (loss) {
        std::vector<float> lp(np);
        PCD_CUDA(cudaMemcpyAsync(lp.data(), lossbuf + 64, np * sizeof(float), cudaMemcpyDeviceToHost, s));
        PCD_CUDA(cudaStreamSynchronize(s));
        // the step already waits for the loss: the tensor-core GEMMs' wait
        // status costs one more 4-byte copy here
        PCD_TRY(nn::gemm_tc_check(s));
        double t = 0.0;
        for (float f : lp) t += f;
        *loss = (float)t;
    }
    return PCD_OK;
}

int UNet::predict(const float *x, int B, float *out, cudaStream_t s)
{
    if (B < 1 || B > maxB) {
        set_error("pcd_unet_predict: batch out of range");
        return PCD_BAD_ARG;
    }
    PCD_TRY(load_input(x, B, s));
    PCD_TRY(forward(B, s));
    PCD_CUDA(cudaMemcpyAsync(out, pred, (size_t)B * S * S * sizeof(float), cudaMemcpyDeviceToDevice, s));
    return PCD_OK;
}

// phi0 on the W x H grid from the network's prediction for b
int UNet::warm_start(const double *b, int W, int H, int ld, double *phi, cudaStream_t s)
{
    k_resample_in<<<grid1d((long)S * S), 256, 0, s>>>(b, W, H, ld, xin_f, S);
    PCD_LAUNCHED(1);
    PCD_TRY(load_input(xin_f, 1, s));
    PCD_TRY(forward(1, s));
    // phi ~ phi_hat * std(b_resampled) * W * H; std from stats[1] = 1/std on the device
    // kPredFilter binomial passes on the network grid: the prediction's error
    // is largest at the scale of the network's cells, where the fine-grid
    // Laplacian amplifies it most; the filter leaves the large scales that
    // shorten the solve (ping-pong between pred and dpred, ending in pred)
    static_assert(kPredFilter % 2 == 0, "the filter passes end in pred");
    for (int k = 0; k < kPredFilter; k++) {
        k_binomial<<<grid1d((long)S * S), 256, 0, s>>>(k % 2 ? dpred : pred, k % 2 ? pred : dpred, S);
        PCD_LAUNCHED(1);
    }
    k_resample_out<<<grid1d((long)W * H), 256, 0, s>>>(pred, S, stats, (double)W * (double)H, phi, W, H, ld);
    PCD_LAUNCHED(1);
    return PCD_OK;
}

}  // namespace pcd

// ---------------------------------------------------------------------------
using namespace pcd;

extern "C" {

int pcd_unet_create(pcd_ctx *ctx, int resolution, int max_batch, unsigned long long seed, pcd_unet **out)
{
    if (!ctx || !out) return PCD_BAD_ARG;
    *out = nullptr;
    std::lock_guard<std::mutex> lk(ctx->mu);
    PCD_TRY(ctx_activate(ctx));
    auto *u = new pcd_unet();
    u->ctx = ctx;
    int st = u->net.build(resolution, max_batch);
    if (st == PCD_OK) st = u->net.init_random(seed);
    // the tensor-core GEMM's set-up before any use of the network inside a
    // stream capture (the learned warm start's judge graph)
    if (st == PCD_OK) st = nn::gemm_tc_prepare();
    if (st != PCD_OK) {
        delete u;
        return st;
    }
    ctx->nets.insert(u);
    *out = u;
    return PCD_OK;
}

int pcd_unet_destroy(pcd_unet *u)
{
    if (!u) return PCD_OK;
    if (pcd_ctx *ctx = u->ctx) {
        std::lock_guard<std::mutex> lk(ctx->mu);
        ctx_activate(ctx);
        cudaStreamSynchronize(ctx->stream);
        if (ctx->net == u) ctx->net = nullptr;
        ctx->nets.erase(u);
        u->net.release();
    }
    delete u;
    return PCD_OK;
}

long long pcd_unet_num_params(pcd_unet *u) { return u ? (long long)u->net.nparams : -1; }

}  // extern "C"

namespace pcd {
void unet_detach_all(pcd_ctx *ctx)
{
    for (pcd_unet *u : ctx->nets) {
        u->net.release();
        u->ctx = nullptr;
    }
    ctx->nets.clear();
    ctx->net = nullptr;
}
}  // namespace pcd

extern "C" {

int pcd_unet_resolution(pcd_unet *u) { return u ? u->net.S : -1; }

int pcd_unet_get_params(pcd_unet *u, float *host)
{
    if (!u || !host) return PCD_BAD_ARG;
    if (!u->ctx) {
        set_error("network's context was destroyed");
        return PCD_BAD_ARG;
    }
    std::lock_guard<std::mutex> lk(u->ctx->mu);
    PCD_TRY(ctx_activate(u->ctx));
    PCD_CUDA(cudaStreamSynchronize(u->ctx->stream));
    return u->net.get_params(host);
}

int pcd_unet_set_params(pcd_unet *u, const float *host)
{
    if (!u || !host) return PCD_BAD_ARG;
    if (!u->ctx) {
        set_error("network's context was destroyed");
        return PCD_BAD_ARG;
    }
    std::lock_guard<std::mutex> lk(u->ctx->mu);
    PCD_TRY(ctx_activate(u->ctx));
    PCD_CUDA(cudaStreamSynchronize(u->ctx->stream));
    return u->net.set_params(host);
}

int pcd_unet_train_step(pcd_unet *u, const float *x, const float *target, int batch, float lr, float weight_decay,
                        float *loss, void *stream)
{
    if (!u || !x || !target) return PCD_BAD_ARG;
    if (!u->ctx) {
        set_error("network's context was destroyed");
        return PCD_BAD_ARG;
    }
    std::lock_guard<std::mutex> lk(u->ctx->mu);
    PCD_TRY(ctx_activate(u->ctx));
    nn::AdamParams ap{lr, 0.9f, 0.999f, 1e-8f, weight_decay};
    StreamJoin j(u->ctx, stream);
    PCD_TRY(j.begin());
    PCD_TRY(u->net.train_step(x, target, batch, ap, loss, j.work));
    return j.end();
}

int pcd_unet_predict(pcd_unet *u, const float *x, int batch, float *out, void *stream)
{
    if (!u || !x || !out) return PCD_BAD_ARG;
    if (!u->ctx) {
        set_error("network's context was destroyed");
        return PCD_BAD_ARG;
    }
    std::lock_guard<std::mutex> lk(u->ctx->mu);
    PCD_TRY(ctx_activate(u->ctx));
    StreamJoin j(u->ctx, stream);
    PCD_TRY(j.begin());
    PCD_TRY(u->net.predict(x, batch, out, j.work));
    return j.end();
}

int pcd_unet_get_grads(pcd_unet *u, float *host)
{
    if (!u || !host) return PCD_BAD_ARG;
    if (!u->ctx) {
        set_error("network's context was destroyed");
        return PCD_BAD_ARG;
    }
    std::lock_guard<std::mutex> lk(u->ctx->mu);
    PCD_TRY(ctx_activate(u->ctx));
    PCD_CUDA(cudaStreamSynchronize(u->ctx->stream));
    PCD_CUDA(cudaMemcpy(host, u->net.params_f + u->net.nparams, u->net.nparams * sizeof(float),
                        cudaMemcpyDeviceToHost));
    return PCD_OK;
}

int pcd_gemm_bf16(const void *A, int lda, const void *B, int ldb, float *C, int ldc, int M, int N, int K, int ksplit,
                  float *partials, void *stream)
{
    nn::GemmArgs g{};
    g.A = (const __nv_bfloat16 *)A;
    g.lda = lda;
    g.B = (const __nv_bfloat16 *)B;
    g.ldb = ldb;
    g.M = M;
    g.N = N;
    g.K = K;
    g.ksplit = ksplit;
    g.Cf = C;
    g.ldc = ldc;
    return nn::gemm(g, (cudaStream_t)stream, partials);
}

int pcd_gemm_bf16_path(const void *A, int lda, const void *B, int ldb, float *C, int ldc, int M, int N, int K,
                       int ksplit, float *partials, int path, void *stream)
{
    if (path < 0 || path > 2) {
        set_error("pcd_gemm_bf16_path: path must be 0, 1 or 2");
        return PCD_BAD_ARG;
    }
    nn::GemmArgs g{};
    g.A = (const __nv_bfloat16 *)A;
    g.lda = lda;
    g.B = (const __nv_bfloat16 *)B;
    g.ldb = ldb;
    g.M = M;
    g.N = N;
    g.K = K;
    g.ksplit = ksplit;
    g.Cf = C;
    g.ldc = ldc;
    g.path = path;
    return nn::gemm(g, (cudaStream_t)stream, partials);
}

int pcd_gemm_bf16_layout(const void *A, int lda, int a_mn, const void *B, int ldb, int b_mn, float *C, int ldc,
                         int trans_c, int M, int N, int K, int ksplit, float *partials, void *stream)
{
    nn::GemmArgs g{};
    g.A = (const __nv_bfloat16 *)A;
    g.lda = lda;
    g.B = (const __nv_bfloat16 *)B;
    g.ldb = ldb;
    g.M = M;
    g.N = N;
    g.K = K;
    g.ksplit = ksplit;
    g.Cf = C;
    g.ldc = ldc;
    g.path = 2;
    g.a_mn = a_mn != 0;
    g.b_mn = b_mn != 0;
    g.trans_c = trans_c != 0;
    return nn::gemm(g, (cudaStream_t)stream, partials);
}

int pcd_conv3x3_bf16(const void *x, int B, int H, int W, int C, int ldx, const void *w, int ldw, int N, float *out,
                     int ldo, void *stream)
{
    if (!out || N < 1 || ldo < N || !nn::conv_tc_applies(x, B, H, W, C, ldx, 128)) {
        set_error("pcd_conv3x3_bf16: unsupported arguments (C >= 32 a multiple of 8, ldx a multiple of 8, aligned x, "
                  "images tiling into 128-pixel boxes)");
        return PCD_BAD_ARG;
    }
    return nn::conv3x3_tc((const __nv_bfloat16 *)x, B, H, W, C, ldx, (const __nv_bfloat16 *)w, ldw, N, nullptr, 0,
                          nullptr, out, ldo, 1, nullptr, (cudaStream_t)stream);
}

int pcd_conv3x3_wgrad_bf16(const void *x, int B, int H, int W, int C, int ldx, const void *dy, int N, float *dw,
                           int ldw, int ksplit, float *partials, void *stream)
{
    if (!dw || N < 32 || ldw < 9 * C || !nn::conv_tc_applies(x, B, H, W, C, ldx, 64)) {
        set_error("pcd_conv3x3_wgrad_bf16: unsupported arguments (N >= 32, C >= 32 a multiple of 8, aligned x, images "
                  "tiling into 64-pixel boxes)");
        return PCD_BAD_ARG;
    }
    return nn::conv3x3_wgrad_tc((const __nv_bfloat16 *)x, B, H, W, C, ldx, (const __nv_bfloat16 *)dy, N, dw, ldw,
                                ksplit, partials, (cudaStream_t)stream);
}

int pcd_gemm_set_default_path(int path) { return nn::set_default_path(path); }

int pcd_gemm_bf16_status(void)
{
    int e = 0;
    PCD_TRY(nn::gemm_tc_error(&e, true));
    if (e) {
        set_error("a bounded wait of the tcgen05 GEMM gave up");
        return e;
    }
    return PCD_OK;
}

int pcd_ctx_set_warm_start_net(pcd_ctx *ctx, pcd_unet *u)
{
    if (!ctx) return PCD_BAD_ARG;
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->net = u;
    return PCD_OK;
}

}  // extern "C"
