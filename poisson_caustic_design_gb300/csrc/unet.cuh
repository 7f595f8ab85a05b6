// unet.cuh -- the learned warm start (internal).
#pragma once

#include <vector>

#include "nn.cuh"

namespace pcd {

struct UNet {
    struct Conv;
    int S = 0, maxB = 0;
    size_t nparams = 0, head_w = 0, head_b = 0;
    int step = 0;
    float *params_f = nullptr;  // [4][nparams]: weights, gradients, Adam m, Adam v (FP32)
    void *arena = nullptr;
    std::vector<Conv> convs;
    // activations (BF16, NHWC)
    __nv_bfloat16 *x_in, *t1, *cat1, *p1, *t2, *cat2, *p2, *t3, *cat3, *p3, *t4, *u4, *t5, *u3, *t6, *u2, *t7, *u1;
    float *pred, *dpred, *xin_f, *stats;
    // backward scratch
    float *g_a, *g_b, *g_cat, *g_cat2, *g_cat3, *partials, *colpart, *small, *lossbuf;
    static constexpr long kColpartCap = 1024L * 384;  // floats of colpart (per-block column sums)
    size_t partials_cap = 0;  // floats in partials (split-K of the GEMMs)
    __nv_bfloat16 *dym, *tr_a, *tr_b, *colD, *wflip;

    ~UNet();
    int build(int S, int maxB);
    void release();
    int init_random(unsigned long long seed);
    int set_params(const float *host);
    int get_params(float *host);
    int train_step(const float *x, const float *target, int B, const nn::AdamParams &ap, float *loss, cudaStream_t s);
    int predict(const float *x, int B, float *out, cudaStream_t s);
    int warm_start(const double *b, int W, int H, int ld, double *phi, cudaStream_t s);

   private:
    int sync_bf16(cudaStream_t s);
    int load_input(const float *x, int B, cudaStream_t s);
    int forward(int B, cudaStream_t s);
    int backward(int B, cudaStream_t s);
    int conv_splits(long P, int N, int Cin) const;
    int conv_fwd(Conv &c, int B, cudaStream_t s);
    int conv_bwd(Conv &c, int B, const float *dY, int lddy, float *dX, cudaStream_t s);
};

}  // namespace pcd

struct pcd_ctx;
namespace pcd {
// Releases the device state of every network of ctx and detaches them.
void unet_detach_all(pcd_ctx *ctx);
}  // namespace pcd
struct pcd_unet {
    pcd_ctx *ctx = nullptr;
    pcd::UNet net;
};
