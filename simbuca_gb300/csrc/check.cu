// check.cu -- the in-run check of the FP32-compensated Coulomb sums.
//
// The FP32c form promises a per-ion relative force error of at most 1e-6 against the
// FP64 direct sum (bin/force.cpp:147-174).  Its one approximation beyond FP32 rounding
// is the far tile pairs of the k-d ordered shapes, summed from the high FP32 parts;
// ions whose net force is small next to their far terms (sqrt(s2f) > kfar |P|) get an
// exact first-order correction, and the threshold kfar must follow how large the
// hi-only error is, which grows with the ion density.  The check measures it while
// the cloud evolves: every few attempts (sg_batch_set_force_check) it takes, per
// cloud, eight probe ions of the last Coulomb sum of the attempt --
//   * the two unflagged ions with the largest far ratio rf = sqrt(s2f)/|P|,
//   * the two unflagged ions with the largest near ratio rn = sqrt(s2)/|P|,
//   * four ions drawn at random --
// evaluates their rows exactly in FP64 from the same SI coordinates, and records the
// relative errors.  From the far-ranked probes it takes c = err / rf, the constant of
// the hi-only error model err ~ c rf, keeps the largest c seen, and lowers the cloud's
// far fix-up threshold to kfar = 5e-7 / c (half the bound) when that is below the
// prior: the threshold in use is the measured one.  The record (largest error, probes,
// errors above 1e-6, c, kfar) is read by sg_batch_force_check.
//
// The sums checked are the stage-7 sums (stage 6 for Cash-Karp, the one sum for Gear)
// left in coulS with the coordinates they were taken at: no stage kernel rewrites the
// Coulomb inputs after the last sum of an attempt, and a cloud is checked only if that
// sum ran since its last check (`ran`, set by the reduction, cleared here and by every
// upload).
#include <math.h>

#include "sg_internal.cuh"

namespace {

constexpr int kCheckThreads = 256;
constexpr int kRanked = 4;                 // probes 0-1 far-ranked, 2-3 near-ranked
constexpr double kTarget = 5e-7;           // unflagged ions at half the bound
constexpr double kBound = 1e-6;            // the FP32c form's per-ion bound
constexpr double kFarRatioMin = 0.1;       // below this the far error is negligible
constexpr float kKfar2Min = 0.0025f;       // kfar >= 0.05

__device__ __forceinline__ uint32_t mix32(uint32_t x) {
    // integer finaliser (xor-shift-multiply), only to spread the random probes
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

// larger value wins; equal values: the lower ion index (a fixed result)
__device__ __forceinline__ bool better(float v, int i, float bv, int bi) {
    return bi < 0 || v > bv || (v == bv && i >= 0 && i < bi);
}

// One block per cloud: the probe ions.
__global__ void __launch_bounds__(kCheckThreads) check_select_kernel(
    const SgCloud* __restrict__ clouds, const int* __restrict__ ran, const float* __restrict__ risk,
    int n_total, SgCheck* __restrict__ chk) {
    const int c = blockIdx.x;
    if (!ran[c]) return;
    const SgCloud& cl = clouds[c];
    if (cl.n <= 0) return;
    __shared__ float wv[kCheckThreads / 32];
    __shared__ int wi[kCheckThreads / 32];
    __shared__ int picked[SG_CHECK_PROBES];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int k = 0; k < kRanked; k++) {
        const float* r = risk + (k < 2 ? 0 : (size_t)n_total);
        float best = 0.f;
        int bidx = -1;
        for (int i = cl.off + tid; i < cl.off + cl.n; i += kCheckThreads) {
            bool taken = false;
            for (int q = 0; q < k; q++) taken |= picked[q] == i;
            if (!taken && better(r[i], i, best, bidx)) {
                best = r[i];
                bidx = i;
            }
        }
        for (int o = 16; o > 0; o >>= 1) {
            const float ov = __shfl_down_sync(0xffffffffu, best, o);
            const int oi = __shfl_down_sync(0xffffffffu, bidx, o);
            if (oi >= 0 && better(ov, oi, best, bidx)) {
                best = ov;
                bidx = oi;
            }
        }
        if (lane == 0) {
            wv[warp] = best;
            wi[warp] = bidx;
        }
        __syncthreads();
        if (tid == 0) {
            float b = 0.f;
            int bi = -1;
            for (int w = 0; w < kCheckThreads / 32; w++)
                if (wi[w] >= 0 && better(wv[w], wi[w], b, bi)) {
                    b = wv[w];
                    bi = wi[w];
                }
            picked[k] = bi >= 0 ? bi : cl.off;
        }
        __syncthreads();
    }
    if (tid == 0) {
        SgCheck& h = chk[c];
        const uint32_t seed = (uint32_t)h.checks * 2654435761u + (uint32_t)c * 40503u;
        for (int k = kRanked; k < SG_CHECK_PROBES; k++)
            picked[k] = cl.off + (int)(mix32(seed + (uint32_t)k) % (uint32_t)cl.n);
        for (int k = 0; k < SG_CHECK_PROBES; k++) {
            const int i = picked[k];
            h.ion[k] = i;
            h.rf[k] = risk[i];
            h.rn[k] = risk[(size_t)n_total + i];
        }
    }
}

// Block (k, c): the FP64 row of probe k of cloud c, over the cloud's padded range (the
// padding ions carry no charge), and its relative error against the checked sum.
__global__ void __launch_bounds__(kCheckThreads) check_rows_kernel(
    const SgCloud* __restrict__ clouds, const int* __restrict__ ran, const double* __restrict__ c64,
    int npad_total, const double* __restrict__ out, int n_total, SgCheck* __restrict__ chk) {
    const int k = blockIdx.x, c = blockIdx.y;
    if (!ran[c]) return;
    const SgCloud& cl = clouds[c];
    if (cl.n <= 0) return;
    const int i = chk[c].ion[k];
    const int ig = cl.poff + (i - cl.off);
    const size_t NP = (size_t)npad_total;
    const double xi = c64[ig], yi = c64[NP + ig], zi = c64[2 * NP + ig];
    double ax = 0.0, ay = 0.0, az = 0.0;
    for (int j = threadIdx.x; j < cl.npad; j += kCheckThreads) {
        const int jg = cl.poff + j;
        if (jg == ig) continue;
        const double rx = xi - c64[jg], ry = yi - c64[NP + jg], rz = zi - c64[2 * NP + jg];
        const double inv = 1.0 / sqrt(rx * rx + ry * ry + rz * rz);
        const double w = c64[3 * NP + jg] * (inv * inv * inv);
        ax = fma(w, rx, ax);
        ay = fma(w, ry, ay);
        az = fma(w, rz, az);
    }
    __shared__ double s[3][kCheckThreads / 32];
    for (int o = 16; o > 0; o >>= 1) {
        ax += __shfl_down_sync(0xffffffffu, ax, o);
        ay += __shfl_down_sync(0xffffffffu, ay, o);
        az += __shfl_down_sync(0xffffffffu, az, o);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
        s[0][warp] = ax;
        s[1][warp] = ay;
        s[2][warp] = az;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double p[3] = {0.0, 0.0, 0.0};
        for (int w = 0; w < kCheckThreads / 32; w++)
            for (int q = 0; q < 3; q++) p[q] += s[q][w];
        const double dx = out[i] - p[0], dy = out[(size_t)n_total + i] - p[1],
                     dz = out[2 * (size_t)n_total + i] - p[2];
        const double d = sqrt(dx * dx + dy * dy + dz * dz);
        const double pn = sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
        double e = pn > 0.0 ? d / pn : (d > 0.0 ? INFINITY : 0.0);
        if (!(e == e)) e = INFINITY;  // a NaN sum is a breach
        chk[c].err[k] = e;
    }
}

// One thread per cloud: fold the probes into the record and the threshold.
__global__ void check_update_kernel(int* __restrict__ ran, SgCheck* __restrict__ chk,
                                    int n_clouds) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n_clouds || !ran[c]) return;
    ran[c] = 0;
    SgCheck h = chk[c];
    double last = 0.0;
    long long br = 0;
    for (int k = 0; k < SG_CHECK_PROBES; k++) {
        last = fmax(last, h.err[k]);
        br += h.err[k] > kBound ? 1 : 0;
        const int kind = k < 2 ? 0 : (k < kRanked ? 1 : 2);
        h.max_kind[kind] = fmax(h.max_kind[kind], h.err[k]);
        if (h.err[k] > h.worst_err) {
            h.worst_err = h.err[k];
            h.worst_rf = h.rf[k];
            h.worst_rn = h.rn[k];
            h.worst_ion = h.ion[k];
            h.worst_kind = kind;
        }
    }
    for (int k = 0; k < 2; k++)
        if (h.rf[k] > kFarRatioMin) h.c_far = fmax(h.c_far, h.err[k] / (double)h.rf[k]);
    if (h.c_far > 0.0) {
        const double kf = kTarget / h.c_far;
        h.kfar2 = fminf(h.kfar2, fmaxf((float)(kf * kf), kKfar2Min));
    }
    h.last_err = last;
    h.max_err = fmax(h.max_err, last);
    h.checks += 1;
    h.probes += SG_CHECK_PROBES;
    h.breaches += br;
    chk[c] = h;
}

}  // namespace

cudaError_t sg_force_check(const SgCloud* clouds, int n_clouds, int* ran, const float* risk,
                           const double* c64, int npad_total, const double* out, int n_total,
                           SgCheck* chk, cudaStream_t st) {
    if (n_clouds <= 0) return cudaSuccess;
    sg_launch(check_select_kernel, n_clouds, kCheckThreads, 0, st, clouds, (const int*)ran, risk,
              n_total, chk);
    sg_launch(check_rows_kernel, dim3(SG_CHECK_PROBES, n_clouds), kCheckThreads, 0, st, clouds,
              (const int*)ran, c64, npad_total, out, n_total, chk);
    sg_launch(check_update_kernel, (n_clouds + 127) / 128, 128, 0, st, ran, chk, n_clouds);
    return cudaGetLastError();
}
