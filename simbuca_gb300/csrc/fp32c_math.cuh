// fp32c_math.cuh -- value-only arithmetic of the FP32-compensated Coulomb form, shared
// by the tiled kernels (coulomb.cu) and the fused small-cloud kernel (fused.cu) so that
// both take their pair terms, compensated sums and FP64 re-evaluations with the same
// operations: the SFU reciprocal square root, packed FP32x2 arithmetic, the float-float
// pair term, Kahan summation, and the refined FP64 reciprocal square root.
#pragma once

#include <cuda_runtime.h>

namespace {

__device__ __forceinline__ float rsqrt_approx(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// packed FP32x2 (two floats in one 64-bit register pair)
typedef unsigned long long f2;
__device__ __forceinline__ f2 pk(float a, float b) {
    f2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void upk(f2 v, float& a, float& b) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
}
__device__ __forceinline__ f2 add2(f2 a, f2 b) {
    f2 d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2 sub2(f2 a, f2 b) {
    f2 d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2 mul2(f2 a, f2 b) {
    f2 d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2 fma2(f2 a, f2 b, f2 c) {
    f2 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}

// Softening added to r^2 in frame units (u ~ 1): below the rounding of any real
// pair distance, it keeps the self pair (dx = 0) finite: 1/r^3 = 1e36 < FLT_MAX.
constexpr float kTiny = 1e-24f;

// One FP32c pair term, scalar form.  Written with explicit rounding intrinsics so the
// close-pair re-evaluation reproduces it bit for bit.
struct PairF {
    float dx, dy, dz, y3;
};
__device__ __forceinline__ PairF pair_f32(float xjh, float yjh, float zjh, float xjl, float yjl,
                                          float zjl, float xih, float yih, float zih, float xil,
                                          float yil, float zil) {
    PairF p;
    p.dx = __fadd_rn(__fsub_rn(xjh, xih), __fsub_rn(xjl, xil));
    p.dy = __fadd_rn(__fsub_rn(yjh, yih), __fsub_rn(yjl, yil));
    p.dz = __fadd_rn(__fsub_rn(zjh, zih), __fsub_rn(zjl, zil));
    float r2 = __fmaf_rn(p.dx, p.dx, kTiny);
    r2 = __fmaf_rn(p.dy, p.dy, r2);
    r2 = __fmaf_rn(p.dz, p.dz, r2);
    const float y = rsqrt_approx(r2);
    p.y3 = __fmul_rn(__fmul_rn(y, y), y);
    return p;
}

__device__ __forceinline__ void kahan_add(float& s, float& c, float x) {
    const float y = __fsub_rn(x, c);
    const float t = __fadd_rn(s, y);
    c = __fsub_rn(__fsub_rn(t, s), y);
    s = t;
}


__device__ __forceinline__ double rsqrt_fp64(double r2) {
    // FP32 SFU seed, then y = y0 (1 + e/2 + 3 e^2/8), e = 1 - r2 y0^2 (binomial series of
    // (1-e)^(-1/2)); the truncation error is ~(5/16) e^3 with |e| < 2^-22.
    const double y0 = (double)rsqrt_approx(__double2float_rn(r2));
    const double e = fma(-r2 * y0, y0, 1.0);
    const double p = fma(e, 0.375, 0.5);
    return fma(y0 * e, p, y0);
}

// The conditioning estimate of an ion: the sum of squares of its FP32 partial sums, or,
// if larger, the squared magnitude of its strongest single pair term, |f|^2 = (1/r^3)^(4/3)
// in frame units for a unit charge (y3max, self pair excluded; in tiles with a close
// pair, the pairs below the cap and the capped terms, capped_term_y3).  A dominant pair
// whose partial sum is cancelled by other terms of the same block must still flag the ion
// for the FP64 re-evaluation of its row.  A threshold test: FP32 suffices (an overflow to
// infinity only flags the ion).
// A close pair (y3 > wc) enters the main loop's sums with its 1/r^3 capped at wc: a term
// of magnitude wc r, whose rounding in the partial sum stays although the pair itself is
// re-evaluated exactly.  As a strongest-term candidate it counts as the y3 whose |f| is
// that magnitude: (wc r)^(3/2) = wc sqrt(wc / y3) (<= wc).
__device__ __forceinline__ float capped_term_y3(float y3, float wc) {
    return wc * sqrtf(wc / y3);
}

__device__ __forceinline__ float conditioning_s2(float s2, float y3max) {
    const float r1 = cbrtf(y3max);  // 1/r
    const float f = r1 * r1;        // |f| = 1/r^2
    return fmaxf(s2, f * f);
}

}  // namespace
