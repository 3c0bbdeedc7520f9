// aux_kernels.cu -- the CUNBODY-compatible force kernel and the issue-rate probes.
#include "sg_internal.cuh"

namespace {

__device__ __forceinline__ float rsqrt_approx_f(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
// Same refinement as the FP64 Coulomb kernel: SFU seed + third-order binomial step.
__device__ __forceinline__ double rsqrt_fp64_aux(double r2) {
    const double y0 = (double)rsqrt_approx_f(__double2float_rn(r2));
    const double e = fma(-r2 * y0, y0, 1.0);
    const double p = fma(e, 0.375, 0.5);
    return fma(y0 * e, p, y0);
}

// ai[i] = sum_j mj[j] (xj[j] - xi[i]) / (|xj[j]-xi[i]|^2 + eps2)^{3/2}
// (the CUNBODY contract, bin/cunbody.h:11-33), FP64, j-tiles through shared memory.
__global__ void __launch_bounds__(128) cunbody_kernel(const double* __restrict__ xj,
                                                      const double* __restrict__ mj,
                                                      const double* __restrict__ xi, double eps2,
                                                      double* __restrict__ ai, int ni, int nj) {
    sg_griddep_wait();
    __shared__ double t[4][128];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool act = i < ni;
    const double x = act ? xi[3 * (size_t)i] : 0.0, y = act ? xi[3 * (size_t)i + 1] : 0.0,
                 z = act ? xi[3 * (size_t)i + 2] : 0.0;
    double ax = 0.0, ay = 0.0, az = 0.0;
    for (int j0 = 0; j0 < nj; j0 += 128) {
        const int len = min(128, nj - j0);
        __syncthreads();
        if ((int)threadIdx.x < len) {
            const size_t j = (size_t)(j0 + threadIdx.x);
            t[0][threadIdx.x] = xj[3 * j];
            t[1][threadIdx.x] = xj[3 * j + 1];
            t[2][threadIdx.x] = xj[3 * j + 2];
            t[3][threadIdx.x] = mj[j];
        }
        __syncthreads();
        for (int jj = 0; jj < len; jj++) {
            const double dx = t[0][jj] - x, dy = t[1][jj] - y, dz = t[2][jj] - z;
            const double r2 = dx * dx + dy * dy + dz * dz + eps2;
            // a coincident pair without softening contributes nothing (0 * inf avoided)
            double w = 0.0;
            if (r2 > 0.0) {
                const double yv = rsqrt_fp64_aux(r2);
                w = t[3][jj] * (yv * yv * yv);
            }
            ax = fma(w, dx, ax);
            ay = fma(w, dy, ay);
            az = fma(w, dz, az);
        }
    }
    if (act) {
        ai[3 * (size_t)i] = ax;
        ai[3 * (size_t)i + 1] = ay;
        ai[3 * (size_t)i + 2] = az;
    }
}

// Issue-rate probes: every thread runs 8 independent FMA chains (4 packed pairs) of
// `iters` steps; the result is stored so the chains are not eliminated.
constexpr int kProbeIters = 4096;

__global__ void probe_ffma(float* sink, float a, float b) {
    sg_griddep_wait();
    float v[8];
#pragma unroll
    for (int q = 0; q < 8; q++) v[q] = threadIdx.x * 1e-3f + q;
#pragma unroll 16
    for (int it = 0; it < kProbeIters; it++)
#pragma unroll
        for (int q = 0; q < 8; q++) v[q] = __fmaf_rn(v[q], a, b);
    float s = 0.f;
#pragma unroll
    for (int q = 0; q < 8; q++) s += v[q];
    if (s == 1.2345f) sink[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void probe_ffma2(float* sink, float a, float b) {
    sg_griddep_wait();
    unsigned long long v[4], A, B;
    asm("mov.b64 %0, {%1, %1};" : "=l"(A) : "f"(a));
    asm("mov.b64 %0, {%1, %1};" : "=l"(B) : "f"(b));
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const float lo = threadIdx.x * 1e-3f + q, hi = lo + 0.5f;
        asm("mov.b64 %0, {%1, %2};" : "=l"(v[q]) : "f"(lo), "f"(hi));
    }
#pragma unroll 16
    for (int it = 0; it < kProbeIters; it++)
#pragma unroll
        for (int q = 0; q < 4; q++)
            asm volatile("fma.rn.f32x2 %0, %0, %1, %2;" : "+l"(v[q]) : "l"(A), "l"(B));
    float s = 0.f;
#pragma unroll
    for (int q = 0; q < 4; q++) {
        float lo, hi;
        asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v[q]));
        s += lo + hi;
    }
    if (s == 1.2345f) sink[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void probe_dfma(float* sink, double a, double b) {
    sg_griddep_wait();
    double v[8];
#pragma unroll
    for (int q = 0; q < 8; q++) v[q] = threadIdx.x * 1e-3 + q;
    // FP64 issue is far slower: fewer steps keep the probe short
#pragma unroll 8
    for (int it = 0; it < kProbeIters / 16; it++)
#pragma unroll
        for (int q = 0; q < 8; q++) v[q] = fma(v[q], a, b);
    double s = 0.0;
#pragma unroll
    for (int q = 0; q < 8; q++) s += v[q];
    if (s == 1.2345) sink[blockIdx.x * blockDim.x + threadIdx.x] = (float)s;
}

}  // namespace

cudaError_t sg_cunbody_launch(const double* xj, const double* mj, const double* xi, double eps2,
                              double* ai, int ni, int nj, cudaStream_t st) {
    if (ni <= 0) return cudaSuccess;
    sg_launch(cunbody_kernel, (ni + 127) / 128, 128, 0, st, xj, mj, xi, eps2, ai, ni, nj);
    return cudaGetLastError();
}

// which: 0 FFMA, 1 FFMA2 (packed), 2 DFMA.  Returns flops per launch via the caller:
// 2 * 8 * iters * blocks * threads (FP32 / FP32x2), iters/16 for FP64.
cudaError_t sg_probe_launch(int which, int blocks, int threads, float* sink, cudaStream_t st) {
    switch (which) {
        case 0: sg_launch(probe_ffma, blocks, threads, 0, st, sink, 0.999f, 1e-4f); break;
        case 1: sg_launch(probe_ffma2, blocks, threads, 0, st, sink, 0.999f, 1e-4f); break;
        case 2: sg_launch(probe_dfma, blocks, threads, 0, st, sink, 0.999, 1e-4); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

int sg_probe_iters(int which) { return which == 2 ? kProbeIters / 16 : kProbeIters; }
