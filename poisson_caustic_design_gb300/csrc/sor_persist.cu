// sor_persist.cu -- persistent, shared-memory-resident red-black SOR (sm_103a).
//
// One cooperative launch runs a whole solve.  CTA g owns a band of grid rows
// [r0, r1) and keeps them in shared memory for the entire solve; the grid in
// HBM/L2 is touched only at the start and the end.  Between half sweeps a CTA
// needs the boundary rows of its two neighbouring bands, so each CTA publishes
// its first and last row into a double-buffered exchange slot in global memory
// and raises a per-CTA epoch flag (st.release); its neighbours wait for that
// flag (ld.acquire) before reading.  No grid-wide barrier is taken per sweep:
// a band is never more than one half sweep ahead of its neighbours.  A
// grid-wide barrier is taken only every `check_every` sweeps, where all CTAs
// reduce the residual (or the sweep's max |delta|) in a fixed order and so take
// the same stop decision.
//
// Every wait is bounded: after `spin_limit` polls a CTA records PCD_TIMEOUT in
// the control block and returns; the others see the error word and return too.
//
// Two state types:
//   FP64  (plain form)  phi and b in FP64, the reference's update
//                       phi += omega/cnt*(sum - cnt*phi - b)  (solver.cpp:47)
//   MIXED               FP32 correction e with FP32 right-hand side r32 in the
//                       sweeps; at each check the FP64 residual is refreshed
//                       r = r_prev - L e (FP64, e widened exactly), phi += e
//                       in FP64, e = 0, r32 = (float) r.
//
// Neighbour counts come from the grid edges only; grids with NaN cells in b use
// the launch-per-half-sweep kernels of solver.cu.
#include <cooperative_groups.h>

#include "sor_persist.cuh"

namespace pcd {

namespace {

__device__ __forceinline__ unsigned ld_acquire(const unsigned *p)
{
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release(unsigned *p, unsigned v)
{
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ int ld_error(const PersistArgs &a) { return *(volatile const int *)&a.ctl->error; }

// Thread 0 polls until *p >= target (or the error word is set); the block then
// agrees on the outcome.  Returns false on timeout/error.
__device__ bool block_wait(const unsigned *p, unsigned target, const PersistArgs &a, int *s_ok)
{
    if (threadIdx.x == 0) {
        int ok = 1;
        long long it = 0;
        while (ld_acquire(p) < target) {
            if (ld_error(a)) { ok = 0; break; }
            if (++it > a.spin_limit) {
                atomicCAS(&a.ctl->error, 0, PCD_TIMEOUT);
                ok = 0;
                break;
            }
            __nanosleep(32);
        }
        *s_ok = ok;
    }
    __syncthreads();
    const bool ok = *s_ok != 0;
    __syncthreads();
    return ok;
}

// Grid-wide barrier number `k` (1-based): arrive on a monotonic counter and
// wait for all G arrivals.
__device__ bool grid_barrier(const PersistArgs &a, unsigned k, int *s_ok)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(a.bar, 1u);
    }
    return block_wait(a.bar, k * (unsigned)a.G, a, s_ok);
}

__device__ __forceinline__ void band_of(int g, int G, int H, int &r0, int &n)
{
    const int base = H / G, extra = H % G;
    n = base + (g < extra ? 1 : 0);
    r0 = g * base + (g < extra ? g : extra);
}

// Publish rows 1 and n of the (n+2)-row shared array `s` (element type T) to
// slot `slot` of this CTA's exchange area, then raise the epoch flag to `ep`.
template <typename T>
__device__ void publish(const PersistArgs &a, const T *s, int n, int slot, unsigned ep)
{
    T *x = reinterpret_cast<T *>(a.xbuf + (size_t)blockIdx.x * 4 * a.W);
    T *dst0 = x + (size_t)(2 * slot) * a.W;
    T *dst1 = dst0 + a.W;
    for (int c = threadIdx.x; c < a.W; c += blockDim.x) {
        dst0[c] = s[(size_t)1 * a.W + c];
        dst1[c] = s[(size_t)n * a.W + c];
    }
    __syncthreads();
    if (threadIdx.x == 0 && !(a.withhold && blockIdx.x == 0)) {
        __threadfence();
        st_release(&a.flags[blockIdx.x], ep);
    }
}

// Wait for both neighbours to reach epoch `ep` and copy their facing rows
// (published in slot `slot`) into halo rows 0 and n+1 of `s`.
template <typename T>
__device__ bool load_halo(const PersistArgs &a, T *s, int n, int slot, unsigned ep, int *s_ok)
{
    const int g = blockIdx.x;
    if (g > 0 && !block_wait(&a.flags[g - 1], ep, a, s_ok)) return false;
    if (g < a.G - 1 && !block_wait(&a.flags[g + 1], ep, a, s_ok)) return false;
    if (g > 0) {
        const T *src = reinterpret_cast<const T *>(a.xbuf + (size_t)(g - 1) * 4 * a.W) + (size_t)(2 * slot + 1) * a.W;
        for (int c = threadIdx.x; c < a.W; c += blockDim.x) s[c] = __ldcg(src + c);
    }
    if (g < a.G - 1) {
        const T *src = reinterpret_cast<const T *>(a.xbuf + (size_t)(g + 1) * 4 * a.W) + (size_t)(2 * slot) * a.W;
        for (int c = threadIdx.x; c < a.W; c += blockDim.x) s[(size_t)(n + 1) * a.W + c] = __ldcg(src + c);
    }
    __syncthreads();
    return true;
}

// Red-black update of colour `color` on the band held in s (rows 1..n, halo
// rows 0 and n+1); rhs holds rows 0..n-1.  Returns this thread's max |delta|.
template <typename T>
__device__ __forceinline__ double relax_band(T *s, const T *rhs, int n, int r0, const PersistArgs &a, int color,
                                             bool track)
{
    const int W = a.W, H = a.H, half = (W + 1) >> 1;
    double m = 0.0;
    int row = 0, k = threadIdx.x;
    while (k >= half && row < n) { k -= half; row++; }
    for (; row < n;) {
        const int y = r0 + row;
        const int x = 2 * k + ((y + color) & 1);
        if (x < W) {
            T *c = s + (size_t)(row + 1) * W + x;
            T sum = T(0);
            int cnt = 0;
            if (x > 0) { sum += c[-1]; cnt++; }
            if (y > 0) { sum += c[-W]; cnt++; }
            if (x < W - 1) { sum += c[1]; cnt++; }
            if (y < H - 1) { sum += c[W]; cnt++; }
            const T v = *c;
            const T w = sizeof(T) == 8 ? (T)a.w64[cnt] : (T)a.w32[cnt];
            const T delta = w * (sum - (T)cnt * v - rhs[(size_t)row * W + x]);
            *c = v + delta;
            if (track) {
                const double ad = fabs((double)delta);
                m = ad > m ? ad : m;
            }
        }
        k += blockDim.x;
        while (k >= half) { k -= half; row++; }
    }
    return m;
}

// FP64 residual r = b - L phi over the band (rows 1..n of s), partial sums.
__device__ void band_residual64(const double *s, const double *b, int n, int r0, const PersistArgs &a, double v[3])
{
    const int W = a.W, H = a.H;
    for (int t = threadIdx.x; t < n * W; t += blockDim.x) {
        const int row = t / W, x = t - row * W, y = r0 + row;
        const double *c = s + (size_t)(row + 1) * W + x;
        double sum = 0.0, cnt = 0.0;
        if (x > 0) { sum += c[-1]; cnt += 1.0; }
        if (y > 0) { sum += c[-W]; cnt += 1.0; }
        if (x < W - 1) { sum += c[1]; cnt += 1.0; }
        if (y < H - 1) { sum += c[W]; cnt += 1.0; }
        const double bi = b[(size_t)row * W + x];
        const double r = bi - (sum - cnt * (*c));
        v[0] += r * r;
        v[1] += bi * bi;
        v[2] = nan_skip_max(v[2], fabs(r));
    }
}

// Mixed refresh over the band: r = r_prev - L e (FP64), phi += e, e = 0,
// r32 = (float) r.  Halo rows of e must hold the neighbours' current e.
__device__ void band_refine(float *se, float *sr32, double *srl, double *sphi, int n, int r0, const PersistArgs &a,
                            double v[3])
{
    const int W = a.W, H = a.H;
    for (int t = threadIdx.x; t < n * W; t += blockDim.x) {
        const int row = t / W, x = t - row * W, y = r0 + row;
        const float *c = se + (size_t)(row + 1) * W + x;
        double sum = 0.0, cnt = 0.0;
        if (x > 0) { sum += (double)c[-1]; cnt += 1.0; }
        if (y > 0) { sum += (double)c[-W]; cnt += 1.0; }
        if (x < W - 1) { sum += (double)c[1]; cnt += 1.0; }
        if (y < H - 1) { sum += (double)c[W]; cnt += 1.0; }
        const double e = (double)(*c);
        const size_t i = (size_t)row * W + x;
        const double r = srl[i] - (sum - cnt * e);
        v[0] += r * r;
        v[2] = nan_skip_max(v[2], fabs(r));
        srl[i] = r;
        sr32[i] = (float)r;
        sphi[i] += e;
    }
}

template <bool MIXED>
__global__ void __launch_bounds__(kPersistThreads, 1) k_sor_persist(PersistArgs a)
{
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int s_ok;
    const int g = blockIdx.x, W = a.W;
    int r0, n;
    band_of(g, a.G, a.H, r0, n);

    // shared layout
    double *s_phi;   // FP64: (n+2) x W with halos; MIXED: n x W
    double *s_b = nullptr, *s_rl = nullptr;
    float *s_e = nullptr, *s_r32 = nullptr;
    if (!MIXED) {
        s_phi = reinterpret_cast<double *>(smem);
        s_b = s_phi + (size_t)(n + 2) * W;
    } else {
        s_phi = reinterpret_cast<double *>(smem);
        s_rl = s_phi + (size_t)n * W;
        s_e = reinterpret_cast<float *>(s_rl + (size_t)n * W);
        s_r32 = s_e + (size_t)(n + 2) * W;
    }

    // load the band
    for (int t = threadIdx.x; t < n * W; t += blockDim.x) {
        const int row = t / W, x = t - row * W;
        const size_t gi = (size_t)(r0 + row) * a.ld + x;
        if (!MIXED) {
            s_phi[(size_t)(row + 1) * W + x] = a.phi[gi];
            s_b[t] = a.b[gi];
        } else {
            s_phi[t] = a.phi[gi];
            const double r = a.r64[gi];
            s_rl[t] = r;
            s_r32[t] = (float)r;
        }
    }
    if (MIXED)
        for (int t = threadIdx.x; t < (n + 2) * W; t += blockDim.x) s_e[t] = 0.0f;
    __syncthreads();

    const double bnorm = *(volatile const double *)&a.ctl->bnorm;
    unsigned ep = 0;          // phases completed by this CTA
    unsigned checks = 0;      // grid barriers passed
    int sweeps = 0;
    double last_max = 0.0, rel = -1.0, rmax = 0.0;
    int converged = 0;
    bool ok = true;

    // phase 0: publish the initial boundary rows
    if (!MIXED) publish<double>(a, s_phi, n, 0, ++ep);
    else publish<float>(a, s_e, n, 0, ++ep);

    const bool track = a.stop == PCD_STOP_MAX_UPDATE;
    double sweep_max = 0.0;
    for (;;) {
        // ---- start of a sweep: halos hold the neighbours' state after the last phase
        const int slot_in = (int)((ep - 1) & 1);
        if (!MIXED) ok = load_halo<double>(a, s_phi, n, slot_in, ep, &s_ok);
        else ok = load_halo<float>(a, s_e, n, slot_in, ep, &s_ok);
        if (!ok) break;

        const bool check = sweeps > 0 && (sweeps % a.check_every == 0 || sweeps >= a.max_iter);
        if (check) {
            double v[3] = {0.0, 0.0, 0.0};
            if (!MIXED) {
                if (track) v[2] = sweep_max;
                else band_residual64(s_phi, s_b, n, r0, a, v);
            } else {
                band_refine(s_e, s_r32, s_rl, s_phi, n, r0, a, v);
                if (track) v[2] = sweep_max;
            }
            block_reduce<3, 4u>(v);
            double *part = a.part + (size_t)(checks & 1) * 3 * a.G;
            if (threadIdx.x == 0) {
                part[3 * g] = v[0];
                part[3 * g + 1] = v[1];
                part[3 * g + 2] = v[2];
            }
            ++checks;
            if (!grid_barrier(a, checks, &s_ok)) { ok = false; break; }
            double w[3] = {0.0, 0.0, 0.0};
            for (int k = threadIdx.x; k < a.G; k += blockDim.x) {
                w[0] += __ldcg(part + 3 * k);
                w[2] = fmax(w[2], __ldcg(part + 3 * k + 2));
            }
            block_reduce<3, 4u>(w);
            __shared__ double s_dec[3];
            if (threadIdx.x == 0) { s_dec[0] = w[0]; s_dec[2] = w[2]; }
            __syncthreads();
            const double rn = sqrt(s_dec[0]);
            if (track) {
                last_max = s_dec[2];
                converged = last_max < a.tol;
                if (!MIXED) rel = -1.0;
                else { rel = bnorm > 0 ? rn / bnorm : rn; }
            } else {
                rel = bnorm > 0 ? rn / bnorm : rn;
                rmax = s_dec[2];
                converged = rel <= a.tol;
            }
            if (MIXED) {
                // e was folded into phi; the neighbours' e halos are zero too
                for (int t = threadIdx.x; t < (n + 2) * W; t += blockDim.x) s_e[t] = 0.0f;
                __syncthreads();
            }
            if (converged || sweeps >= a.max_iter) break;
        }
        sweep_max = 0.0;
        // ---- red half sweep
        double m;
        if (!MIXED) m = relax_band<double>(s_phi, s_b, n, r0, a, 0, track);
        else m = relax_band<float>(s_e, s_r32, n, r0, a, 0, track);
        sweep_max = fmax(sweep_max, m);
        __syncthreads();
        if (!MIXED) publish<double>(a, s_phi, n, (int)(ep & 1), ep + 1);
        else publish<float>(a, s_e, n, (int)(ep & 1), ep + 1);
        ++ep;
        // ---- black half sweep
        if (!MIXED) ok = load_halo<double>(a, s_phi, n, (int)((ep - 1) & 1), ep, &s_ok);
        else ok = load_halo<float>(a, s_e, n, (int)((ep - 1) & 1), ep, &s_ok);
        if (!ok) break;
        if (!MIXED) m = relax_band<double>(s_phi, s_b, n, r0, a, 1, track);
        else m = relax_band<float>(s_e, s_r32, n, r0, a, 1, track);
        sweep_max = fmax(sweep_max, m);
        __syncthreads();
        if (!MIXED) publish<double>(a, s_phi, n, (int)(ep & 1), ep + 1);
        else publish<float>(a, s_e, n, (int)(ep & 1), ep + 1);
        ++ep;
        ++sweeps;
    }

    // write the band back
    if (ok) {
        for (int t = threadIdx.x; t < n * W; t += blockDim.x) {
            const int row = t / W, x = t - row * W;
            const size_t gi = (size_t)(r0 + row) * a.ld + x;
            a.phi[gi] = MIXED ? s_phi[t] : s_phi[(size_t)(row + 1) * W + x];
        }
    }
    if (g == 0 && threadIdx.x == 0) {
        volatile Ctl *c = a.ctl;
        c->sweeps = sweeps;
        c->converged = ok && converged;
        c->last_max = last_max;
        if (rel >= 0.0) c->rel = rel;
        c->rmax = rmax;
        c->checks = (int)checks;
    }
}

}  // namespace

size_t persist_smem_bytes(int W, int H, int G, bool mixed)
{
    const int n = (H + G - 1) / G;
    if (!mixed) return (size_t)(2 * n + 2) * W * sizeof(double);
    return (size_t)n * W * 2 * sizeof(double) + (size_t)(2 * n + 2) * W * sizeof(float);
}

int persist_grid(int dev, int W, int H, bool mixed, int *G_out, size_t *smem_out)
{
    int sms = 0, max_smem = 0;
    PCD_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    PCD_CUDA(cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    int coop = 0;
    PCD_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
    if (!coop) return PCD_BAD_ARG;
    // one CTA per SM, at least two rows per band
    int G = sms;
    if (G > H / 2) G = H / 2;
    if (G < 2) return PCD_BAD_ARG;
    const size_t smem = persist_smem_bytes(W, H, G, mixed) + 64;
    if (smem > (size_t)max_smem - 1024) return PCD_BAD_ARG;
    *G_out = G;
    *smem_out = smem;
    return PCD_OK;
}

int launch_persist(PersistArgs &a, bool mixed, size_t smem, cudaStream_t s)
{
    void *fn = mixed ? (void *)k_sor_persist<true> : (void *)k_sor_persist<false>;
    PCD_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    void *params[] = {&a};
    PCD_CUDA(cudaLaunchCooperativeKernel(fn, dim3(a.G), dim3(kPersistThreads), params, smem, s));
    count_launches(1);
    return PCD_OK;
}

}  // namespace pcd
