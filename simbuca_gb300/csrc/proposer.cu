// proposer.cu -- the learned step-size proposer: per-cloud features, an MLP
// 16 -> 64 -> 64 -> 1 with SiLU activations, BF16 weights and FP32 accumulation, its
// training kernels (forward + backward + Adam), and the step-history log it learns from.
//
// After every Dormand-Prince attempt the proposer kernel (one warp per cloud):
//   * on an accepted step, appends (features of the step start, h of the previous
//     step, h and error norm of this step) to the cloud's log and recomputes the
//     features from the new state;
//   * when the proposer is on, replaces the controller's next step size h_c by
//     safety * h * exp(MLP(features)), clamped to [0.2, 10] x h and to [1/2, 2] x h_c:
//     the reference's controller stays the fallback, so features outside the training
//     range (a tiny error norm after tiny steps, say) cannot drive h down step after step.
// Rejected attempts keep the reference's reject rule (bin/ode.cpp:451-455): every step
// is still accepted or rejected by the embedded Dormand-Prince error estimate.
//
// Features (all O(1)):  0-2 centroid / L;  3-5 RMS spread / L - 1;  6-8 RMS velocity
// / v0 - 1 (L, v0: frame scale and RMS velocity at upload);  9 log10(h_last) + 8;
// 10 log10(err_last) (>= -8);  11 rejects of the last step;  12-13 cos/sin of the
// active drive's phase;  14 +1 quadrupole / -1 dipole / 0 none;  15 log10(h_last/h_prev).
// The target of a logged step is log(h_k err_k^-0.2 / h_{k-1}): the ratio to the
// previous step of the step size that would have met the tolerance exactly.
#include <cuda_bf16.h>

#include "sg_internal.cuh"

namespace {

__device__ __forceinline__ float silu(float z) { return z / (1.0f + __expf(-z)); }
__device__ __forceinline__ float silu_grad(float z) {
    const float s = 1.0f / (1.0f + __expf(-z));
    return s * (1.0f + z * (1.0f - s));
}

// MLP forward of one feature vector by one warp; returns the output on every lane.
__device__ float mlp_warp(const __nv_bfloat16* __restrict__ w, const float* x) {
    const int lane = threadIdx.x & 31;
    const __nv_bfloat16* W1 = w + SG_MLP_W1;
    const __nv_bfloat16* B1 = w + SG_MLP_B1;
    const __nv_bfloat16* W2 = w + SG_MLP_W2;
    const __nv_bfloat16* B2 = w + SG_MLP_B2;
    const __nv_bfloat16* W3 = w + SG_MLP_W3;
    float h1[2], h2[2];
#pragma unroll
    for (int r = 0; r < 2; r++) {
        const int u = lane + 32 * r;
        float z = __bfloat162float(B1[u]);
#pragma unroll
        for (int k = 0; k < SG_MLP_IN; k++) z = fmaf(__bfloat162float(W1[u * SG_MLP_IN + k]), x[k], z);
        h1[r] = silu(z);
    }
#pragma unroll
    for (int r = 0; r < 2; r++) {
        const int u = lane + 32 * r;
        float z = __bfloat162float(B2[u]);
        for (int m = 0; m < SG_MLP_H; m++) {
            const float hm = __shfl_sync(0xffffffffu, h1[m >> 5], m & 31);
            z = fmaf(__bfloat162float(W2[u * SG_MLP_H + m]), hm, z);
        }
        h2[r] = silu(z);
    }
    float o = __bfloat162float(W3[lane]) * h2[0] + __bfloat162float(W3[lane + 32]) * h2[1];
    for (int off = 16; off > 0; off >>= 1) o += __shfl_xor_sync(0xffffffffu, o, off);
    return o + __bfloat162float(w[SG_MLP_B3]);
}

// Per-cloud features from the row-block moment partials of moments_kernel.
__device__ void cloud_features(const SgCloud& cl, const SgCtrl& cs, const double* mom,
                               const SgProposerState& ps, float* f) {
    double s[11];
    for (int q = 0; q < 11; q++) s[q] = 0.0;
    for (int b = 0; b < cl.nrb; b++)
        for (int q = 0; q < 11; q++) s[q] += mom[(size_t)(cl.rb0 + b) * 11 + q];
    const double n = cl.n;
    const double L = cl.L, v0 = cl.vref > 0.0 ? cl.vref : 1.0;
    for (int c = 0; c < 3; c++) {
        const double m = s[c] / n;
        const double var = s[3 + c] / n - m * m;
        f[c] = (float)((m - (c == 0 ? cl.cx : c == 1 ? cl.cy : cl.cz)) / L);
        f[3 + c] = (float)((var > 0 ? sqrt(var) : 0.0) / L - 1.0);
        f[6 + c] = (float)(sqrt(s[6 + c] / n) / v0 - 1.0);
    }
    const double hl = cs.h_last > 0 ? cs.h_last : cs.h;
    f[9] = (float)(log10(hl) + 8.0);
    f[10] = (float)fmax(log10(fmax(cs.err, 1e-30)), -8.0);
    f[11] = (float)ps.rejects_in_step;
    const sg_field_params& fp = cl.fp;
    const double t = cs.t;
    double ph = 0.0, kind = 0.0;
    if ((fp.flags & SG_F_QUAD) && t >= fp.tq_on && t < fp.tq_off) {
        ph = 2.0 * SG_PI * fp.nu_q * t + fp.phi_q;
        kind = 1.0;
    } else if ((fp.flags & SG_F_DIPOLE) && t >= fp.td_on && t < fp.td_off) {
        ph = 2.0 * SG_PI * fp.nu_d * t + fp.phi_d;
        kind = -1.0;
    }
    f[12] = kind != 0.0 ? (float)cos(ph) : 0.f;
    f[13] = kind != 0.0 ? (float)sin(ph) : 0.f;
    f[14] = (float)kind;
    f[15] = ps.h_prev > 0 ? (float)log10(hl / ps.h_prev) : 0.f;
}

// One warp per cloud, after the commit of an attempt.
__global__ void proposer_kernel(const SgCloud* __restrict__ clouds, SgCtrl* __restrict__ ctrl,
                                const double* __restrict__ mom, SgProposerState* __restrict__ pst,
                                const __nv_bfloat16* __restrict__ w, float* __restrict__ log_feat,
                                double* __restrict__ log_num, int log_cap, int use_mlp,
                                double safety, int n_clouds) {
    sg_griddep_wait();
    const int c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (c >= n_clouds) return;
    SgCtrl cs = ctrl[c];
    SgProposerState ps = pst[c];
    const SgCloud& cl = clouds[c];
    // a fresh upload marks the state with init == 0: features of the first step
    if (!ps.init) {
        float f[SG_MLP_IN];
        cloud_features(cl, cs, mom, ps, f);
        if (lane == 0) {
            for (int k = 0; k < SG_MLP_IN; k++) pst[c].feat[k] = f[k];
            pst[c].init = 1;
        }
        return;
    }
    if (cs.status != SG_OK) return;
    if (!cs.accepted) {
        // a rejected attempt: remember it for the features; the reject rule stands
        if (lane == 0 && !cs.done && !cs.hold) pst[c].rejects_in_step = ps.rejects_in_step + 1;
        return;
    }
    // accepted: log (features at the step start, h_prev, h, err)
    if (lane == 0 && log_cap > 0 && ps.logged < log_cap) {
        const long long r = (long long)c * log_cap + ps.logged;
        for (int k = 0; k < SG_MLP_IN; k++) log_feat[r * SG_MLP_IN + k] = ps.feat[k];
        log_num[r * 4 + 0] = ps.h_prev;
        log_num[r * 4 + 1] = cs.h_last;
        log_num[r * 4 + 2] = cs.err;
        log_num[r * 4 + 3] = cs.t;
    }
    SgProposerState nps = ps;
    nps.logged = (log_cap > 0 && ps.logged < log_cap) ? ps.logged + 1 : ps.logged;
    nps.h_prev = cs.h_last;
    nps.rejects_in_step = 0;
    float f[SG_MLP_IN];
    cloud_features(cl, cs, mom, ps, f);
    if (use_mlp == 2 && !cs.done) {
        // the controller's rule with another safety factor (the ablation of the MLP)
        if (lane == 0) ctrl[c].h = safety * cs.h;
    } else if (use_mlp && !cs.done) {
        const float o = mlp_warp(w, f);
        const double lo = log(0.2), hi = log(10.0);
        const double r = fmin(fmax((double)o, lo), hi);
        const double h_ctrl = cs.h;  // the controller's next step (bin/ode.cpp:443-446)
        const double h_mlp = safety * cs.h_last * exp(r);
        if (lane == 0) ctrl[c].h = fmin(fmax(h_mlp, 0.5 * h_ctrl), 2.0 * h_ctrl);
    }
    if (lane == 0) {
        for (int k = 0; k < SG_MLP_IN; k++) nps.feat[k] = f[k];
        pst[c] = nps;
    }
}

// ---- training ----------------------------------------------------------------
// Forward + backward of a batch; block b takes samples [b*per, (b+1)*per) (of the
// index list idx) and writes its gradient partial to gpart[b][SG_MLP_NP] and its
// squared-error sum to lpart[b].  MSE loss L = (1/B) sum (o - y)^2.
constexpr int kTrainThreads = 128;

__global__ void __launch_bounds__(kTrainThreads) mlp_grad_kernel(
    const __nv_bfloat16* __restrict__ w, const float* __restrict__ X, const float* __restrict__ Y,
    const int* __restrict__ idx, int B, int per, float* __restrict__ gpart,
    float* __restrict__ lpart) {
    sg_griddep_wait();
    __shared__ float g[SG_MLP_NP];
    __shared__ float lsum[kTrainThreads / 32];
    for (int k = threadIdx.x; k < SG_MLP_NP; k += blockDim.x) g[k] = 0.f;
    __syncthreads();
    float lerr = 0.f;
    const int s0 = blockIdx.x * per;
    for (int si = s0 + threadIdx.x; si < min(B, s0 + per); si += blockDim.x) {
        const int sidx = idx ? idx[si] : si;
        const float* x = X + (size_t)sidx * SG_MLP_IN;
        float xv[SG_MLP_IN];
#pragma unroll
        for (int k = 0; k < SG_MLP_IN; k++) xv[k] = x[k];
        float z1[SG_MLP_H], h1[SG_MLP_H], z2[SG_MLP_H], h2[SG_MLP_H];
        for (int u = 0; u < SG_MLP_H; u++) {
            float z = __bfloat162float(w[SG_MLP_B1 + u]);
#pragma unroll
            for (int k = 0; k < SG_MLP_IN; k++)
                z = fmaf(__bfloat162float(w[SG_MLP_W1 + u * SG_MLP_IN + k]), xv[k], z);
            z1[u] = z;
            h1[u] = silu(z);
        }
        for (int u = 0; u < SG_MLP_H; u++) {
            float z = __bfloat162float(w[SG_MLP_B2 + u]);
            for (int m = 0; m < SG_MLP_H; m++)
                z = fmaf(__bfloat162float(w[SG_MLP_W2 + u * SG_MLP_H + m]), h1[m], z);
            z2[u] = z;
            h2[u] = silu(z);
        }
        float o = __bfloat162float(w[SG_MLP_B3]);
        for (int u = 0; u < SG_MLP_H; u++) o = fmaf(__bfloat162float(w[SG_MLP_W3 + u]), h2[u], o);
        const float d = o - Y[sidx];
        lerr += d * d;
        const float go = 2.0f * d / (float)B;
        atomicAdd(&g[SG_MLP_B3], go);
        float gz2[SG_MLP_H];
        for (int u = 0; u < SG_MLP_H; u++) {
            atomicAdd(&g[SG_MLP_W3 + u], go * h2[u]);
            gz2[u] = go * __bfloat162float(w[SG_MLP_W3 + u]) * silu_grad(z2[u]);
            atomicAdd(&g[SG_MLP_B2 + u], gz2[u]);
        }
        for (int m = 0; m < SG_MLP_H; m++) {
            float gh = 0.f;
            for (int u = 0; u < SG_MLP_H; u++) {
                atomicAdd(&g[SG_MLP_W2 + u * SG_MLP_H + m], gz2[u] * h1[m]);
                gh = fmaf(__bfloat162float(w[SG_MLP_W2 + u * SG_MLP_H + m]), gz2[u], gh);
            }
            const float gz1 = gh * silu_grad(z1[m]);
            atomicAdd(&g[SG_MLP_B1 + m], gz1);
#pragma unroll
            for (int k = 0; k < SG_MLP_IN; k++) atomicAdd(&g[SG_MLP_W1 + m * SG_MLP_IN + k], gz1 * xv[k]);
        }
    }
    for (int o = 16; o > 0; o >>= 1) lerr += __shfl_down_sync(0xffffffffu, lerr, o);
    if ((threadIdx.x & 31) == 0) lsum[threadIdx.x >> 5] = lerr;
    __syncthreads();
    for (int k = threadIdx.x; k < SG_MLP_NP; k += blockDim.x)
        gpart[(size_t)blockIdx.x * SG_MLP_NP + k] = g[k];
    if (threadIdx.x == 0) {
        float s = 0.f;
        for (int q = 0; q < kTrainThreads / 32; q++) s += lsum[q];
        lpart[blockIdx.x] = s;
    }
}

// grad[k] = sum_b gpart[b][k] (fixed order); loss = sum_b lpart[b] / B.
__global__ void mlp_reduce_kernel(const float* __restrict__ gpart, const float* __restrict__ lpart,
                                  int nb, int B, float* __restrict__ grad, float* __restrict__ loss) {
    sg_griddep_wait();
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < SG_MLP_NP) {
        float s = 0.f;
        for (int b = 0; b < nb; b++) s += gpart[(size_t)b * SG_MLP_NP + k];
        grad[k] = s;
    }
    if (k == 0) {
        float s = 0.f;
        for (int b = 0; b < nb; b++) s += lpart[b];
        *loss = s / (float)B;
    }
}

// Adam on the FP32 master weights, then the BF16 copy used by the forward pass.
__global__ void mlp_adam_kernel(float* __restrict__ wm, __nv_bfloat16* __restrict__ wb,
                                float* __restrict__ m1, float* __restrict__ m2,
                                const float* __restrict__ grad, float lr, float b1, float b2,
                                float eps, int step) {
    sg_griddep_wait();
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= SG_MLP_NP) return;
    const float g = grad[k];
    const float a = b1 * m1[k] + (1.f - b1) * g;
    const float v = b2 * m2[k] + (1.f - b2) * g * g;
    m1[k] = a;
    m2[k] = v;
    const float ah = a / (1.f - powf(b1, (float)step));
    const float vh = v / (1.f - powf(b2, (float)step));
    const float nw = wm[k] - lr * ah / (sqrtf(vh) + eps);
    wm[k] = nw;
    wb[k] = __float2bfloat16_rn(nw);
}

__global__ void mlp_to_bf16_kernel(const float* __restrict__ wm, __nv_bfloat16* __restrict__ wb) {
    sg_griddep_wait();
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < SG_MLP_NP) wb[k] = __float2bfloat16_rn(wm[k]);
}

// Inference of a batch: one warp per sample.
__global__ void mlp_forward_kernel(const __nv_bfloat16* __restrict__ w, const float* __restrict__ X,
                                   int n, float* __restrict__ out) {
    sg_griddep_wait();
    const int s = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (s >= n) return;
    float x[SG_MLP_IN];
#pragma unroll
    for (int k = 0; k < SG_MLP_IN; k++) x[k] = X[(size_t)s * SG_MLP_IN + k];
    const float o = mlp_warp(w, x);
    if ((threadIdx.x & 31) == 0) out[s] = o;
}

}  // namespace

cudaError_t sg_proposer_launch(const SgCloud* clouds, SgCtrl* ctrl, const double* mom,
                               SgProposerState* pst, const void* wbf, float* log_feat,
                               double* log_num, int log_cap, int use_mlp, double safety,
                               int n_clouds, cudaStream_t st) {
    const int warps = 4;
    sg_launch(proposer_kernel, (n_clouds + warps - 1) / warps, 32 * warps, 0, st, 
        clouds, ctrl, mom, pst, static_cast<const __nv_bfloat16*>(wbf), log_feat, log_num, log_cap,
        use_mlp, safety, n_clouds);
    return cudaGetLastError();
}

cudaError_t sg_mlp_grad_launch(const void* wbf, const float* X, const float* Y, const int* idx,
                               int B, float* gpart, float* lpart, int nb, float* grad, float* loss,
                               cudaStream_t st) {
    const int per = (B + nb - 1) / nb;
    sg_launch(mlp_grad_kernel, nb, kTrainThreads, 0, st, static_cast<const __nv_bfloat16*>(wbf), X, Y, idx,
                                                  B, per, gpart, lpart);
    sg_launch(mlp_reduce_kernel, (SG_MLP_NP + 255) / 256, 256, 0, st, gpart, lpart, nb, B, grad, loss);
    return cudaGetLastError();
}

cudaError_t sg_mlp_adam_launch(float* wm, void* wbf, float* m1, float* m2, const float* grad,
                               float lr, int step, cudaStream_t st) {
    sg_launch(mlp_adam_kernel, (SG_MLP_NP + 255) / 256, 256, 0, st, 
        wm, static_cast<__nv_bfloat16*>(wbf), m1, m2, grad, lr, 0.9f, 0.999f, 1e-8f, step);
    return cudaGetLastError();
}

cudaError_t sg_mlp_to_bf16_launch(const float* wm, void* wbf, cudaStream_t st) {
    sg_launch(mlp_to_bf16_kernel, (SG_MLP_NP + 255) / 256, 256, 0, st, wm, static_cast<__nv_bfloat16*>(wbf));
    return cudaGetLastError();
}

cudaError_t sg_mlp_forward_launch(const void* wbf, const float* X, int n, float* out,
                                  cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    sg_launch(mlp_forward_kernel, (n + 3) / 4, 128, 0, st, static_cast<const __nv_bfloat16*>(wbf), X, n, out);
    return cudaGetLastError();
}
