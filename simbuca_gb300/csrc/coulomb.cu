// coulomb.cu -- direct-sum Coulomb kernels of libsimgb (sm_103a).
//
// Both kernels compute, for every i-ion of a work item and the j-range of the item,
//     P_i = sum_{j != i} q_j (x_i - x_j) / |x_i - x_j|^3          (SI units, m^-2)
// and store P_i in the item's partial-sum slot; the stage kernels multiply the sum of
// the slots by kq_i = coulomb_scale k_e e^2 q_i / m_i.  This is the CPU loop of the
// reference (bin/force.cpp:147-174) regrouped into tiles: same pair terms, no
// softening, self term excluded by index.
//
// FP32c (coulomb_fp32c_kernel): pair terms in FP32 on cloud-frame coordinates
// u = (x - c)/L held as float-float pairs (hi, lo).  The difference
// u_j - u_i = (hi_j - hi_i) + (lo_j - lo_i) keeps the pair distance accurate to an
// FP32 rounding even for ions far from the frame centre.  1/r is the SFU
// approximation (rsqrt.approx), 1/r^3 is capped at wc: the rare close pairs whose
// 1/r^3 exceeds wc are re-evaluated in FP64 once the tile is done, and the capped
// FP32 contribution is taken out again exactly.  Within a 128-ion j-tile the terms
// are summed in FP32; tile sums are added with Kahan compensation.  Arithmetic uses
// the packed FP32x2 instructions of sm_100+ (add/mul/fma.rn.f32x2) on pairs of
// consecutive j-ions.  j-tiles are fetched with TMA bulk copies (cp.async.bulk) into
// a 4-stage shared-memory ring guarded by mbarriers.
//
// FP64 (coulomb_fp64_kernel): the plain form, every operation in FP64; 1/sqrt(r^2)
// is an FP32 SFU seed refined by one third-order step of the binomial series
// 1/sqrt(1-e) = 1 + e/2 + 3e^2/8 (e = 1 - r^2 y0^2), accurate to ~1 ulp.
#include <stdio.h>

#include "fp32c_math.cuh"
#include "sg_internal.cuh"

namespace {

// ---- PTX helpers ---------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ uint64_t globaltimer() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
                 : "memory");
}
__device__ __forceinline__ void mbar_arrive_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait on an mbarrier phase: false once limit_ns have passed.
__device__ __forceinline__ bool mbar_wait_for(uint64_t* bar, uint32_t parity, uint64_t limit_ns) {
    if (mbar_try(bar, parity)) return true;
    const uint64_t t0 = globaltimer();
    for (;;) {
        if (mbar_try(bar, parity)) return true;
        if (globaltimer() - t0 > limit_ns) return false;
    }
}
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    return mbar_wait_for(bar, parity, SG_WAIT_NS);
}
// The wait test (flags[SG_FLAG_WAIT_TILE] = t + 1): after tile t has arrived, the block
// also waits on `never`, a barrier that nothing arrives at, until the test's limit runs
// out; the kernel then takes its timeout path, whose drain finds every issued copy landed.
__device__ __forceinline__ bool wait_test(uint64_t* never, const int* flags) {
    const uint64_t limit = 1000ull * (uint64_t)max(flags[SG_FLAG_WAIT_US], 1);
    return mbar_wait_for(never, 0, limit);
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes,
                                         uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
        ::"r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}
__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// Close pairs of one flagged ion against one shared-memory tile, evaluated by the
// whole warp (lanes stride over the tile): pairs whose FP32 1/r^3 exceeded wc get their
// exact FP64 term, minus the capped FP32 term the main loop already summed (a product
// of two floats, exact in FP64).  Returns the warp-reduced correction (all lanes) and,
// in ymx, the tile's strongest FP32 term as a y3 (pairs below the cap, capped terms:
// capped_term_y3), which the main loop's y3max cannot give for a tile with a close pair.
template <int TL>
__device__ __forceinline__ void close_pairs_warp(const float (*tl)[TL], int len, int j0,
                                                 int ig, float xih, float yih, float zih,
                                                 float xil, float yil, float zil, float wc,
                                                 double invL2, double qscale,
                                                 const double* __restrict__ c64,
                                                 int npad_total, double& ox, double& oy,
                                                 double& oz, float& ymx) {
    const int lane = threadIdx.x & 31;
    const double xi = c64[ig], yi = c64[npad_total + ig], zi = c64[2 * (size_t)npad_total + ig];
    double cx = 0.0, cy = 0.0, cz = 0.0;
    float ym = 0.f;
    for (int jj = lane; jj < len; jj += 32) {
        const PairF p = pair_f32(tl[0][jj], tl[1][jj], tl[2][jj], tl[4][jj], tl[5][jj],
                                 tl[6][jj], xih, yih, zih, xil, yil, zil);
        const int jg = j0 + jj;
        if (jg != ig && tl[3][jj] != 0.f)
            ym = fmaxf(ym, p.y3 > wc ? capped_term_y3(p.y3, wc) : p.y3);
        if (p.y3 > wc && jg != ig) {
            const float wf = __fmul_rn(tl[3][jj], wc);
            const double rx = xi - c64[jg];
            const double ry = yi - c64[npad_total + jg];
            const double rz = zi - c64[2 * (size_t)npad_total + jg];
            const double r2d = rx * rx + ry * ry + rz * rz;
            const double inv = rsqrt_fp64(r2d);
            const double wq = c64[3 * (size_t)npad_total + jg] * inv * inv * inv;
            const double wsc = invL2 * qscale * (double)wf;
            cx += wq * rx + wsc * (double)p.dx;
            cy += wq * ry + wsc * (double)p.dy;
            cz += wq * rz + wsc * (double)p.dz;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        cx += __shfl_xor_sync(0xffffffffu, cx, o);
        cy += __shfl_xor_sync(0xffffffffu, cy, o);
        cz += __shfl_xor_sync(0xffffffffu, cz, o);
    }
    ox = cx;
    oy = cy;
    oz = cz;
    // non-negative floats order as their bit patterns
    ymx = __uint_as_float(__reduce_max_sync(0xffffffffu, __float_as_uint(ym)));
}

// Main loop over one shared-memory j-tile for the IPT ions of a thread: packed FP32x2
// over consecutive j pairs.  DIAG: the tile contains the thread's own ions, whose self
// pair must not raise the close-pair flag.
template <int IPT, bool DIAG, bool NOQ = false, int NU = 2>
__device__ __forceinline__ void tile_pairs(const float* tx, const float* ty, const float* tz,
                                           const float* tq, const float* txl, const float* tyl,
                                           const float* tzl, int jb, int je, int j0,
                                           const int* ipad,
                                           const f2* xh, const f2* yh, const f2* zh,
                                           const f2* xl, const f2* yl, const f2* zl, f2 tiny2,
                                           float wc, f2* ax, f2* ay, f2* az, float* y3max) {
#pragma unroll NU
    for (int jj = jb; jj < je; jj += 2) {
        const f2 Xj = *reinterpret_cast<const f2*>(tx + jj);
        const f2 Yj = *reinterpret_cast<const f2*>(ty + jj);
        const f2 Zj = *reinterpret_cast<const f2*>(tz + jj);
        const f2 Qj = NOQ ? 0ull : *reinterpret_cast<const f2*>(tq + jj);
        const f2 XLj = *reinterpret_cast<const f2*>(txl + jj);
        const f2 YLj = *reinterpret_cast<const f2*>(tyl + jj);
        const f2 ZLj = *reinterpret_cast<const f2*>(tzl + jj);
#pragma unroll
        for (int k = 0; k < IPT; k++) {
            const f2 dx = add2(sub2(Xj, xh[k]), sub2(XLj, xl[k]));
            const f2 dy = add2(sub2(Yj, yh[k]), sub2(YLj, yl[k]));
            const f2 dz = add2(sub2(Zj, zh[k]), sub2(ZLj, zl[k]));
            f2 r2 = fma2(dx, dx, tiny2);
            r2 = fma2(dy, dy, r2);
            r2 = fma2(dz, dz, r2);
            float ra, rb;
            upk(r2, ra, rb);
            const f2 y = pk(rsqrt_approx(ra), rsqrt_approx(rb));
            const f2 y3 = mul2(mul2(y, y), y);
            float ua, ub;
            upk(y3, ua, ub);
            if (DIAG) {
                const float ma = (j0 + jj == ipad[k]) ? 0.f : ua;
                const float mb = (j0 + jj + 1 == ipad[k]) ? 0.f : ub;
                y3max[k] = fmaxf(y3max[k], fmaxf(ma, mb));
            } else {
                y3max[k] = fmaxf(y3max[k], fmaxf(ua, ub));
            }
            const f2 wy = pk(fminf(ua, wc), fminf(ub, wc));
            const f2 w = NOQ ? wy : mul2(Qj, wy);
            ax[k] = fma2(w, dx, ax[k]);
            ay[k] = fma2(w, dy, ay[k]);
            az[k] = fma2(w, dz, az[k]);
        }
    }
}


// Squared distance between two tile bounding boxes (frame units).
__device__ __forceinline__ float box_dist2(const float* a, const float* b) {
    float d2 = 0.f;
#pragma unroll
    for (int c = 0; c < 3; c++) {
        const float g = fmaxf(0.f, fmaxf(b[c] - a[3 + c], a[c] - b[3 + c]));
        d2 = fmaf(g, g, d2);
    }
    return d2;
}

// Far tiles: packed FP32x2 over j pairs, high parts only, no close pairs possible.
// FU: j pairs unrolled (0: 4 for one ion per thread, else 2).
template <int IPT, bool NOQ = false, int FU = 0>
__device__ __forceinline__ void tile_pairs_far(const float* tx, const float* ty, const float* tz,
                                               const float* tq, int jb, int je, const f2* xh,
                                               const f2* yh, const f2* zh, f2 tiny2, f2* ax,
                                               f2* ay, f2* az) {
    constexpr int kFarUnroll = FU > 0 ? FU : (IPT == 1 ? 4 : 2);  // more j pairs in flight
#pragma unroll kFarUnroll
    for (int jj = jb; jj < je; jj += 2) {
        const f2 Xj = *reinterpret_cast<const f2*>(tx + jj);
        const f2 Yj = *reinterpret_cast<const f2*>(ty + jj);
        const f2 Zj = *reinterpret_cast<const f2*>(tz + jj);
        const f2 Qj = NOQ ? 0ull : *reinterpret_cast<const f2*>(tq + jj);
#pragma unroll
        for (int k = 0; k < IPT; k++) {
            const f2 dx = sub2(Xj, xh[k]);
            const f2 dy = sub2(Yj, yh[k]);
            const f2 dz = sub2(Zj, zh[k]);
            f2 r2 = fma2(dx, dx, tiny2);
            r2 = fma2(dy, dy, r2);
            r2 = fma2(dz, dz, r2);
            float ra, rb;
            upk(r2, ra, rb);
            const f2 y = pk(rsqrt_approx(ra), rsqrt_approx(rb));
            const f2 y3 = mul2(mul2(y, y), y);
            const f2 w = NOQ ? y3 : mul2(Qj, y3);
            ax[k] = fma2(w, dx, ax[k]);
            ay[k] = fma2(w, dy, ay[k]);
            az[k] = fma2(w, dz, az[k]);
        }
    }
}

// ---------------------------------------------------------------------------
// FP32c kernel.  Global layout: c32 = 7 float arrays of npad_total entries
// (x, y, z, q, xl, yl, zl in frame units); shared tile = the same 7 arrays of SG_TILE.
// ---------------------------------------------------------------------------
template <int NT, int IPT>
__global__ void __launch_bounds__(NT) coulomb_fp32c_kernel(const float* __restrict__ c32,
                                                            const double* __restrict__ c64,
                                                            const SgWorkItem* __restrict__ items,
                                                            const SgCloud* __restrict__ clouds,
                                                            const SgCtrl* __restrict__ ctrl,
                                                            double* __restrict__ part,
                                                            int npad_total, int* errword) {
    sg_griddep_wait();
    constexpr int T = SG_TILE;
    __shared__ __align__(128) float tile[SG_STAGES][7][T];
    __shared__ __align__(8) uint64_t full[SG_STAGES];
    __shared__ __align__(8) uint64_t never;  // the wait test's barrier
    __shared__ double corr[3][NT * IPT];

    const SgWorkItem it = items[blockIdx.x];
    const int wtest = errword ? errword[SG_FLAG_WAIT_TILE] : 0;
    if (ctrl != nullptr && (ctrl[it.cloud].done || ctrl[it.cloud].hold || ctrl[it.cloud].status != SG_OK)) return;
    const SgCloud& cl = clouds[it.cloud];
    const float wc = cl.wc;
    const double invL2 = cl.invL * cl.invL;
    // uniform-charge clouds hold q_j / qscale (1 for ions, 0 for padding): tiles without
    // padding skip the charge product and the sums are scaled once at the end
    const double qscale = cl.qscale;
    const int j_real_end = cl.poff + cl.n;
    const int tid = threadIdx.x;
    const float* X = c32;
    const float* Y = c32 + npad_total;
    const float* Z = c32 + 2 * (size_t)npad_total;
    const float* XL = c32 + 4 * (size_t)npad_total;
    const float* YL = c32 + 5 * (size_t)npad_total;
    const float* ZL = c32 + 6 * (size_t)npad_total;

    // i-ions of this thread: it.i0 + tid + k*NT (clamped into the item for loads)
    int ipad[IPT];
    f2 xh[IPT], yh[IPT], zh[IPT], xl[IPT], yl[IPT], zl[IPT];
#pragma unroll
    for (int k = 0; k < IPT; k++) {
        int li = tid + k * NT;
        int ii = it.i0 + (li < it.ni ? li : 0);
        ipad[k] = li < it.ni ? ii : -1;
        float a = X[ii], b = Y[ii], c = Z[ii], d = XL[ii], e = YL[ii], f = ZL[ii];
        xh[k] = pk(a, a);
        yh[k] = pk(b, b);
        zh[k] = pk(c, c);
        xl[k] = pk(d, d);
        yl[k] = pk(e, e);
        zl[k] = pk(f, f);
        corr[0][li] = 0.0;
        corr[1][li] = 0.0;
        corr[2][li] = 0.0;
    }
    float ks[IPT][3], kc[IPT][3], s2[IPT], fmx[IPT];
#pragma unroll
    for (int k = 0; k < IPT; k++) {
        s2[k] = 0.f;
        fmx[k] = 0.f;
#pragma unroll
        for (int c = 0; c < 3; c++) ks[k][c] = kc[k][c] = 0.f;
    }

    const int ntiles = (it.nj + T - 1) / T;
    bool ok = true;
    if (tid == 0) {
        for (int s = 0; s < SG_STAGES; s++) mbar_init(&full[s], 1);
        mbar_init(&never, 1);
        fence_mbar_init();
    }
    __syncthreads();
    // prologue: fill the ring
    if (tid == 0) {
        for (int s = 0; s < SG_STAGES && s < ntiles; s++) {
            const int j0 = it.j0 + s * T;
            const int len = min(T, it.j0 + it.nj - j0);
            const uint32_t bytes = (uint32_t)len * 4u;
            mbar_arrive_tx(&full[s], 7u * bytes);
            for (int a = 0; a < 7; a++)
                bulk_g2s(&tile[s][a][0], c32 + (size_t)a * npad_total + j0, bytes, &full[s]);
        }
    }

    const f2 tiny2 = pk(kTiny, kTiny);
    // one ion per thread (the small-cloud shapes): four j pairs in flight per thread
    constexpr int kNU = IPT == 1 ? 4 : 2;
    // Small clouds fold partial sums every 16 j-ions so that the squared partial sums
    // still estimate sum_j |f_ij|^2 when the whole cloud is one or two tiles.
    const int flush_len = (cl.npad <= 2048) ? 16 : SG_TILE;
    for (int t = 0; t < ntiles; t++) {
        const int s = t % SG_STAGES;
        const uint32_t parity = (uint32_t)((t / SG_STAGES) & 1);
        const int j0 = it.j0 + t * T;
        const int len = min(T, it.j0 + it.nj - j0);
        bool arrived = mbar_wait(&full[s], parity);
        if (t + 1 == wtest) arrived = wait_test(&never, errword) && arrived;
        if (!__syncthreads_and(arrived)) {  // block-uniform decision
            ok = false;
            if (tid == 0) {
                atomicExch(errword, SG_TIMEOUT);
                // drain the copies still in flight (tiles t .. t+STAGES-1), bounded
                for (int u = t; u < ntiles && u < t + SG_STAGES; u++)
                    (void)mbar_wait(&full[u % SG_STAGES], (uint32_t)((u / SG_STAGES) & 1));
            }
            __syncthreads();
            break;
        }

        float y3max[IPT];
#pragma unroll
        for (int k = 0; k < IPT; k++) y3max[k] = 0.f;
        const float* tx = tile[s][0];
        const float* ty = tile[s][1];
        const float* tz = tile[s][2];
        const float* tq = tile[s][3];
        const float* txl = tile[s][4];
        const float* tyl = tile[s][5];
        const float* tzl = tile[s][6];
        // The tile holding this block's own ions takes the variant that keeps the self
        // pair (dx = 0, contributes nothing) out of the close-pair flag.
        const bool diag = (j0 < it.i0 + it.ni) && (j0 + len > it.i0);
        // no padding ions in this tile: their normalized charge 0 is the only one not 1
        const bool noq = cl.quniform && j0 + len <= j_real_end;
        for (int jb = 0; jb < len; jb += flush_len) {
            const int je = min(len, jb + flush_len);
            f2 ax[IPT], ay[IPT], az[IPT];
#pragma unroll
            for (int k = 0; k < IPT; k++) ax[k] = ay[k] = az[k] = 0ull;
            if (!diag && noq)
                tile_pairs<IPT, false, true, kNU>(tx, ty, tz, tq, txl, tyl, tzl, jb, je, j0, ipad, xh,
                                             yh, zh, xl, yl, zl, tiny2, wc, ax, ay, az, y3max);
            else if (!diag)
                tile_pairs<IPT, false, false, kNU>(tx, ty, tz, tq, txl, tyl, tzl, jb, je, j0, ipad, xh, yh, zh,
                                       xl, yl, zl, tiny2, wc, ax, ay, az, y3max);
            else
                tile_pairs<IPT, true, false, kNU>(tx, ty, tz, tq, txl, tyl, tzl, jb, je, j0, ipad, xh, yh, zh,
                                      xl, yl, zl, tiny2, wc, ax, ay, az, y3max);
            // fold the partial sums into the compensated accumulators
#pragma unroll
            for (int k = 0; k < IPT; k++) {
                float a, b;
                upk(ax[k], a, b);
                const float tx_ = __fadd_rn(a, b);
                upk(ay[k], a, b);
                const float ty_ = __fadd_rn(a, b);
                upk(az[k], a, b);
                const float tz_ = __fadd_rn(a, b);
                kahan_add(ks[k][0], kc[k][0], tx_);
                kahan_add(ks[k][1], kc[k][1], ty_);
                kahan_add(ks[k][2], kc[k][2], tz_);
                // sum of squared partial sums: estimates sum_j |f_ij|^2 (conditioning test)
                s2[k] = fmaf(tx_, tx_, fmaf(ty_, ty_, fmaf(tz_, tz_, s2[k])));
            }
        }
        // the strongest single FP32 term so far (conditioning estimate); a tile with a
        // close pair gives its strongest term below the cap from the close-pair pass
#pragma unroll
        for (int k = 0; k < IPT; k++)
            if (y3max[k] <= wc) fmx[k] = fmaxf(fmx[k], y3max[k]);
        // close pairs of this tile, one flagged ion at a time by the whole warp
#pragma unroll
        for (int k = 0; k < IPT; k++) {
            unsigned m = __ballot_sync(0xffffffffu, y3max[k] > wc && ipad[k] >= 0);
            while (m) {
                const int src = __ffs(m) - 1;
                m &= m - 1;
                float a, dummy;
                upk(xh[k], a, dummy);
                const float xih = __shfl_sync(0xffffffffu, a, src);
                upk(yh[k], a, dummy);
                const float yih = __shfl_sync(0xffffffffu, a, src);
                upk(zh[k], a, dummy);
                const float zih = __shfl_sync(0xffffffffu, a, src);
                upk(xl[k], a, dummy);
                const float xil = __shfl_sync(0xffffffffu, a, src);
                upk(yl[k], a, dummy);
                const float yil = __shfl_sync(0xffffffffu, a, src);
                upk(zl[k], a, dummy);
                const float zil = __shfl_sync(0xffffffffu, a, src);
                const int igs = __shfl_sync(0xffffffffu, ipad[k], src);
                double ox, oy, oz;
                float ymx;
                close_pairs_warp(tile[s], len, j0, igs, xih, yih, zih, xil, yil, zil, wc, invL2, qscale,
                                 c64, npad_total, ox, oy, oz, ymx);
                if ((tid & 31) == src) {
                    fmx[k] = fmaxf(fmx[k], ymx);
                    const int li = tid + k * NT;
                    corr[0][li] += ox;
                    corr[1][li] += oy;
                    corr[2][li] += oz;
                }
            }
        }
        __syncthreads();  // every thread is done with ring slot s
        if (tid == 0 && t + SG_STAGES < ntiles) {
            fence_proxy_async();
            const int jn = it.j0 + (t + SG_STAGES) * T;
            const int ln = min(T, it.j0 + it.nj - jn);
            const uint32_t bytes = (uint32_t)ln * 4u;
            mbar_arrive_tx(&full[s], 7u * bytes);
            for (int a = 0; a < 7; a++)
                bulk_g2s(&tile[s][a][0], c32 + (size_t)a * npad_total + jn, bytes, &full[s]);
        }
    }
    if (!ok) return;
    double* P = part + (size_t)it.slot * SG_PART_ARRAYS * npad_total;
#pragma unroll
    for (int k = 0; k < IPT; k++) {
        if (ipad[k] < 0) continue;
        const int li = tid + k * NT;
        const int ig = ipad[k];
        P[3 * (size_t)npad_total + ig] = (double)conditioning_s2(s2[k], fmx[k]) * (qscale * qscale);
        P[4 * (size_t)npad_total + ig] = 0.0;  // no far tiles in this form
        // P_i = sum q_j (x_i - x_j)/r^3 = -invL^2 qscale sum w (u_j - u_i) + close-pair
        // terms, w carrying the charges q_j / qscale
        const double sc = -invL2 * qscale;
        P[ig] = sc * ((double)ks[k][0] - (double)kc[k][0]) + corr[0][li];
        P[npad_total + ig] = sc * ((double)ks[k][1] - (double)kc[k][1]) + corr[1][li];
        P[2 * (size_t)npad_total + ig] = sc * ((double)ks[k][2] - (double)kc[k][2]) + corr[2][li];
    }
}

// Adds packed partial sums (two interleaved FP32 sums per ion and component) into the
// compensated accumulators, and their squares into the conditioning estimate of the
// near tiles (s2: the pairs the FP64 fix-up re-evaluates) or of the far tiles (s2f: the
// hi-only pair terms, whose error grows with it; in k-d order a far tile's 32-ion sums
// are coherent, so s2f is kept apart rather than flagging ions through s2).
template <int IPT, bool S2F = true>
__device__ __forceinline__ void fold_partials(const f2* ax, const f2* ay, const f2* az,
                                              float (*ks)[3], float (*kc)[3], float* s2,
                                              float* s2f, bool near) {
#pragma unroll
    for (int k = 0; k < IPT; k++) {
        float a, b;
        upk(ax[k], a, b);
        const float tx_ = __fadd_rn(a, b);
        upk(ay[k], a, b);
        const float ty_ = __fadd_rn(a, b);
        upk(az[k], a, b);
        const float tz_ = __fadd_rn(a, b);
        kahan_add(ks[k][0], kc[k][0], tx_);
        kahan_add(ks[k][1], kc[k][1], ty_);
        kahan_add(ks[k][2], kc[k][2], tz_);
        if (near)
            s2[k] = fmaf(tx_, tx_, fmaf(ty_, ty_, fmaf(tz_, tz_, s2[k])));
        else if (S2F)
            s2f[k] = fmaf(tx_, tx_, fmaf(ty_, ty_, fmaf(tz_, tz_, s2f[k])));
    }
}

template <int NT, int IPT, int MINB, int STAGES, int TJ = SG_TILE, int FU = 0, bool S2F = true>
__global__ void __launch_bounds__(NT, MINB) coulomb_fp32c_sorted_kernel(const float* __restrict__ c32,
                                                            const double* __restrict__ c64,
                                                            const SgWorkItem* __restrict__ items,
                                                            const SgCloud* __restrict__ clouds,
                                                            const SgCtrl* __restrict__ ctrl,
                                                            double* __restrict__ part,
                                                            int npad_total, int* errword,
                                                            const float* __restrict__ bbox) {
    sg_griddep_wait();
    constexpr int T = TJ;  // j-tile: a multiple of the 128-ion leaves
    __shared__ __align__(128) float tile[STAGES][7][T];
    __shared__ __align__(8) uint64_t full[STAGES];
    __shared__ __align__(8) uint64_t never;  // the wait test's barrier
    __shared__ double corr[3][NT * IPT];

    const SgWorkItem it = items[blockIdx.x];
    const int wtest = errword ? errword[SG_FLAG_WAIT_TILE] : 0;
    if (ctrl != nullptr && (ctrl[it.cloud].done || ctrl[it.cloud].hold || ctrl[it.cloud].status != SG_OK)) return;
    const SgCloud& cl = clouds[it.cloud];
    const float wc = cl.wc;
    const double invL2 = cl.invL * cl.invL;
    // uniform-charge clouds hold q_j / qscale (1 for ions, 0 for padding): tiles without
    // padding skip the charge product and the sums are scaled once at the end
    const double qscale = cl.qscale;
    const int j_real_end = cl.poff + cl.n;
    const int tid = threadIdx.x;
    const float* X = c32;
    const float* Y = c32 + npad_total;
    const float* Z = c32 + 2 * (size_t)npad_total;
    const float* XL = c32 + 4 * (size_t)npad_total;
    const float* YL = c32 + 5 * (size_t)npad_total;
    const float* ZL = c32 + 6 * (size_t)npad_total;

    // i-ions of this thread: it.i0 + tid + k*NT (clamped into the item for loads)
    int ipad[IPT];
    f2 xh[IPT], yh[IPT], zh[IPT], xl[IPT], yl[IPT], zl[IPT];
#pragma unroll
    for (int k = 0; k < IPT; k++) {
        int li = IPT * tid + k;  // contiguous: warp w holds the 128-ion tile w of the block
        int ii = it.i0 + (li < it.ni ? li : 0);
        ipad[k] = li < it.ni ? ii : -1;
        float a = X[ii], b = Y[ii], c = Z[ii], d = XL[ii], e = YL[ii], f = ZL[ii];
        xh[k] = pk(a, a);
        yh[k] = pk(b, b);
        zh[k] = pk(c, c);
        xl[k] = pk(d, d);
        yl[k] = pk(e, e);
        zl[k] = pk(f, f);
        corr[0][li] = 0.0;
        corr[1][li] = 0.0;
        corr[2][li] = 0.0;
    }
    float ks[IPT][3], kc[IPT][3], s2[IPT], s2f[IPT], fmx[IPT];
#pragma unroll
    for (int k = 0; k < IPT; k++) {
        s2[k] = 0.f;
        s2f[k] = 0.f;
        fmx[k] = 0.f;
#pragma unroll
        for (int c = 0; c < 3; c++) ks[k][c] = kc[k][c] = 0.f;
    }

    const int ntiles = (it.nj + T - 1) / T;
    bool ok = true;
    if (tid == 0) {
        for (int s = 0; s < STAGES; s++) mbar_init(&full[s], 1);
        mbar_init(&never, 1);
        fence_mbar_init();
    }
    __syncthreads();
    // prologue: fill the ring
    if (tid == 0) {
        for (int s = 0; s < STAGES && s < ntiles; s++) {
            const int j0 = it.j0 + s * T;
            const int len = min(T, it.j0 + it.nj - j0);
            const uint32_t bytes = (uint32_t)len * 4u;
            mbar_arrive_tx(&full[s], 7u * bytes);
            for (int a = 0; a < 7; a++)
                bulk_g2s(&tile[s][a][0], c32 + (size_t)a * npad_total + j0, bytes, &full[s]);
        }
    }

    const f2 tiny2 = pk(kTiny, kTiny);
    // bounds of this warp's 128 i-ions (a k-d tree leaf after sorting)
    float wbox[6];
    {
        // warps past the cloud's last ion read the last tile (their results are dropped)
        const int last = (cl.npad + 127) / 128 - 1;
        const int wt = cl.tile0 + min(last, (it.i0 - cl.poff) / 128 + (tid >> 5) * (32 * IPT) / 128);
        for (int q = 0; q < 6; q++) wbox[q] = bbox[8 * (size_t)wt + q];
    }
    const float dfar2 = cl.dfar * cl.dfar;
    // FP32 running sums restart every 32 j-ions (16 for small clouds): in k-d order the
    // terms of a tile point the same way, and a 128-term running sum would carry several
    // times the rounding error of the summands.
    const int flush_len = (cl.npad <= 2048) ? 16 : 32;
    for (int t = 0; t < ntiles; t++) {
        const int s = t % STAGES;
        const uint32_t parity = (uint32_t)((t / STAGES) & 1);
        const int j0 = it.j0 + t * T;
        const int len = min(T, it.j0 + it.nj - j0);
        bool arrived = mbar_wait(&full[s], parity);
        if (t + 1 == wtest) arrived = wait_test(&never, errword) && arrived;
        if (!__syncthreads_and(arrived)) {  // block-uniform decision
            ok = false;
            if (tid == 0) {
                atomicExch(errword, SG_TIMEOUT);
                // drain the copies still in flight (tiles t .. t+STAGES-1), bounded
                for (int u = t; u < ntiles && u < t + STAGES; u++)
                    (void)mbar_wait(&full[u % STAGES], (uint32_t)((u / STAGES) & 1));
            }
            __syncthreads();
            break;
        }

        float y3max[IPT];
#pragma unroll
        for (int k = 0; k < IPT; k++) y3max[k] = 0.f;
        const float* tx = tile[s][0];
        const float* ty = tile[s][1];
        const float* tz = tile[s][2];
        const float* tq = tile[s][3];
        const float* txl = tile[s][4];
        const float* tyl = tile[s][5];
        const float* tzl = tile[s][6];
        // Per 128-ion leaf of the tile: far from this block's leaf, or not.  The leaf holding
        // this block's own ions takes the variant that keeps the self pair (dx = 0,
        // contributes nothing) out of the close-pair flag.
        // no padding ions in this tile: their normalized charge 0 is the only one not 1
        const bool noq = cl.quniform && j0 + len <= j_real_end;
        for (int sub = 0; sub < len; sub += SG_TILE) {
            const int send = min(len, sub + SG_TILE);
            const int sj0 = j0 + sub;
            const bool diag = (sj0 < it.i0 + it.ni) && (j0 + send > it.i0);
            float jbox[6];
            const int jt = cl.tile0 + (sj0 - cl.poff) / 128;
            for (int q = 0; q < 6; q++) jbox[q] = bbox[8 * (size_t)jt + q];
            const bool far = !diag && box_dist2(wbox, jbox) > dfar2;  // uniform per warp
            // Each 32-ion FP32 partial goes straight into the compensated accumulators.
            // (Adding the partials of a tile first, in FP32, saved 3 % of the kernel time but
            // raised the worst ion's error on the 65,536-ion cloud from 5.7e-7 to 8.8e-7.)
            for (int jb = sub; jb < send; jb += flush_len) {
                const int je = min(send, jb + flush_len);
                f2 ax[IPT], ay[IPT], az[IPT];
#pragma unroll
                for (int k = 0; k < IPT; k++) ax[k] = ay[k] = az[k] = 0ull;
                if (far && noq)
                    tile_pairs_far<IPT, true, FU>(tx, ty, tz, tq, jb, je, xh, yh, zh, tiny2, ax, ay,
                                                  az);
                else if (far)
                    tile_pairs_far<IPT, false, FU>(tx, ty, tz, tq, jb, je, xh, yh, zh, tiny2, ax, ay,
                                                   az);
                else if (!diag && noq)
                    tile_pairs<IPT, false, true>(tx, ty, tz, tq, txl, tyl, tzl, jb, je, j0, ipad,
                                                 xh, yh, zh, xl, yl, zl, tiny2, wc, ax, ay, az,
                                                 y3max);
                else if (!diag)
                    tile_pairs<IPT, false>(tx, ty, tz, tq, txl, tyl, tzl, jb, je, j0, ipad, xh, yh,
                                           zh, xl, yl, zl, tiny2, wc, ax, ay, az, y3max);
                else
                    tile_pairs<IPT, true>(tx, ty, tz, tq, txl, tyl, tzl, jb, je, j0, ipad, xh, yh,
                                          zh, xl, yl, zl, tiny2, wc, ax, ay, az, y3max);
                fold_partials<IPT, S2F>(ax, ay, az, ks, kc, s2, s2f, !far);
            }
        }
        // the strongest single FP32 term so far (conditioning estimate); a tile with a
        // close pair gives its strongest term below the cap from the close-pair pass
#pragma unroll
        for (int k = 0; k < IPT; k++)
            if (y3max[k] <= wc) fmx[k] = fmaxf(fmx[k], y3max[k]);
        // close pairs of this tile, one flagged ion at a time by the whole warp
#pragma unroll
        for (int k = 0; k < IPT; k++) {
            unsigned m = __ballot_sync(0xffffffffu, y3max[k] > wc && ipad[k] >= 0);
            while (m) {
                const int src = __ffs(m) - 1;
                m &= m - 1;
                float a, dummy;
                upk(xh[k], a, dummy);
                const float xih = __shfl_sync(0xffffffffu, a, src);
                upk(yh[k], a, dummy);
                const float yih = __shfl_sync(0xffffffffu, a, src);
                upk(zh[k], a, dummy);
                const float zih = __shfl_sync(0xffffffffu, a, src);
                upk(xl[k], a, dummy);
                const float xil = __shfl_sync(0xffffffffu, a, src);
                upk(yl[k], a, dummy);
                const float yil = __shfl_sync(0xffffffffu, a, src);
                upk(zl[k], a, dummy);
                const float zil = __shfl_sync(0xffffffffu, a, src);
                const int igs = __shfl_sync(0xffffffffu, ipad[k], src);
                double ox, oy, oz;
                float ymx;
                close_pairs_warp(tile[s], len, j0, igs, xih, yih, zih, xil, yil, zil, wc, invL2, qscale,
                                 c64, npad_total, ox, oy, oz, ymx);
                if ((tid & 31) == src) {
                    fmx[k] = fmaxf(fmx[k], ymx);
                    const int li = IPT * tid + k;
                    corr[0][li] += ox;
                    corr[1][li] += oy;
                    corr[2][li] += oz;
                }
            }
        }
        __syncthreads();  // every thread is done with ring slot s
        if (tid == 0 && t + STAGES < ntiles) {
            fence_proxy_async();
            const int jn = it.j0 + (t + STAGES) * T;
            const int ln = min(T, it.j0 + it.nj - jn);
            const uint32_t bytes = (uint32_t)ln * 4u;
            mbar_arrive_tx(&full[s], 7u * bytes);
            for (int a = 0; a < 7; a++)
                bulk_g2s(&tile[s][a][0], c32 + (size_t)a * npad_total + jn, bytes, &full[s]);
        }
    }
    if (!ok) return;
    double* P = part + (size_t)it.slot * SG_PART_ARRAYS * npad_total;
#pragma unroll
    for (int k = 0; k < IPT; k++) {
        if (ipad[k] < 0) continue;
        const int li = IPT * tid + k;
        const int ig = ipad[k];
        P[3 * (size_t)npad_total + ig] = (double)conditioning_s2(s2[k], fmx[k]) * (qscale * qscale);
        if (S2F) P[4 * (size_t)npad_total + ig] = (double)s2f[k] * (qscale * qscale);
        // P_i = sum q_j (x_i - x_j)/r^3 = -invL^2 qscale sum w (u_j - u_i) + close-pair
        // terms, w carrying the charges q_j / qscale
        const double sc = -invL2 * qscale;
        P[ig] = sc * ((double)ks[k][0] - (double)kc[k][0]) + corr[0][li];
        P[npad_total + ig] = sc * ((double)ks[k][1] - (double)kc[k][1]) + corr[1][li];
        P[2 * (size_t)npad_total + ig] = sc * ((double)ks[k][2] - (double)kc[k][2]) + corr[2][li];
    }
}

// ---------------------------------------------------------------------------
// FP64 kernel (plain form).  c64 = 4 double arrays (x, y, z, q) in SI units.
// ---------------------------------------------------------------------------

template <int NT, int IPT>
__global__ void __launch_bounds__(NT) coulomb_fp64_kernel(const double* __restrict__ c64,
                                                           const SgWorkItem* __restrict__ items,
                                                           const SgCtrl* __restrict__ ctrl,
                                                           double* __restrict__ part,
                                                           int npad_total) {
    sg_griddep_wait();
    constexpr int T = NT;
    __shared__ double tile[4][T];
    const SgWorkItem it = items[blockIdx.x];
    if (ctrl != nullptr && (ctrl[it.cloud].done || ctrl[it.cloud].hold || ctrl[it.cloud].status != SG_OK)) return;
    const int tid = threadIdx.x;
    const double* X = c64;
    const double* Y = c64 + npad_total;
    const double* Z = c64 + 2 * (size_t)npad_total;
    const double* Q = c64 + 3 * (size_t)npad_total;
    int ipad[IPT];
    double xi[IPT], yi[IPT], zi[IPT], ax[IPT], ay[IPT], az[IPT];
#pragma unroll
    for (int k = 0; k < IPT; k++) {
        const int li = tid + k * NT;
        const int ii = it.i0 + (li < it.ni ? li : 0);
        ipad[k] = li < it.ni ? ii : -1;
        xi[k] = X[ii];
        yi[k] = Y[ii];
        zi[k] = Z[ii];
        ax[k] = ay[k] = az[k] = 0.0;
    }
    for (int j0 = it.j0; j0 < it.j0 + it.nj; j0 += T) {
        const int len = min(T, it.j0 + it.nj - j0);
        __syncthreads();
        if (tid < len) {
            tile[0][tid] = X[j0 + tid];
            tile[1][tid] = Y[j0 + tid];
            tile[2][tid] = Z[j0 + tid];
            tile[3][tid] = Q[j0 + tid];
        }
        __syncthreads();
        for (int jj = 0; jj < len; jj++) {
            const double xj = tile[0][jj], yj = tile[1][jj], zj = tile[2][jj], qj = tile[3][jj];
            const int jg = j0 + jj;
#pragma unroll
            for (int k = 0; k < IPT; k++) {
                const double rx = xi[k] - xj, ry = yi[k] - yj, rz = zi[k] - zj;
                const double r2 = rx * rx + ry * ry + rz * rz;
                const double y = rsqrt_fp64(r2);
                double w = qj * (y * y * y);
                w = (jg == ipad[k]) ? 0.0 : w;
                ax[k] = fma(w, rx, ax[k]);
                ay[k] = fma(w, ry, ay[k]);
                az[k] = fma(w, rz, az[k]);
            }
        }
    }
    double* P = part + (size_t)it.slot * SG_PART_ARRAYS * npad_total;
#pragma unroll
    for (int k = 0; k < IPT; k++) {
        if (ipad[k] < 0) continue;
        P[3 * (size_t)npad_total + ipad[k]] = 0.0;
        P[4 * (size_t)npad_total + ipad[k]] = 0.0;
        P[ipad[k]] = ax[k];
        P[npad_total + ipad[k]] = ay[k];
        P[2 * (size_t)npad_total + ipad[k]] = az[k];
    }
}


// ---------------------------------------------------------------------------
// Sum of the partial-sum slots of every ion into out[3][N] (SI, m^-2).
//
// FP32c only: the conditioning test.  sqrt(s2) estimates sqrt(sum_j |f_ij|^2) of the
// FP32 terms; the rounding of those terms is random, so the error of P_i is about
// 2.5e-7 * sqrt(s2).  An ion whose FP32 terms cancel strongly (sqrt(s2) > 1.5 |P_i|,
// e.g. near the centre of a cloud, or a single term above 1.5 |P_i|) gets its whole row
// re-evaluated in FP64 (fixup_row), spread over work units for a large cloud.
//
// k-d ordered shapes: the far tile pairs were summed from the high FP32 parts only, an
// error of ~1e-7 per pair that averages out unless the ion's net force is small next to
// its far terms (the centre of a uniform cloud).  Its size tracks sqrt(s2f), the far
// tiles' conditioning estimate: on the 1M-ion spheroid and the 65,536-ion Gaussian cloud
// (numpy model of the kernel's arithmetic) the relative error of P_i stayed below
// 1.3e-6 sqrt(s2f)/|P_i|, the constant growing with the ion density.  An ion with
// s2f > SgCloud::kfar2 |P_i|^2 gets the exact first-order correction of every far pair
// term (fixup_ion), which leaves it at the near tiles' FP32 accuracy.
// ---------------------------------------------------------------------------
constexpr double kKappa2 = 2.25;
// Clouds of up to kSmallRow padded ions flag at sqrt(s2) > |P| instead: their FP64 row
// is cheap, and with few terms per ion the error per unit of sqrt(s2)/|P| ran up to
// ~9e-7 (an unflagged ion at 1.37 measured 1.2e-6 in the 512-cloud scan's small clouds;
// 2.5e-7 at most on the 65,536-ion cloud).  Their flagged rows are one work unit each.
constexpr double kKappa2Small = 1.0;
constexpr int kSmallRow = 4096;
// kinds of fix-up of a flagged ion
constexpr int kFixNear = 1, kFixFar = 2;

// blocks of the fix-up kernel (each takes every kFixupBlocks-th work unit)
constexpr int kFixupBlocks = 512;
// work units of one listed ion in the fix-up kernel, and the listed ions that get them
constexpr int kFarChunks = SG_FIX_UNITS;
constexpr int kChunkedCap = SG_FIX_CHUNKED_CAP;
// batches up to this many ions fix their flagged ions inside the reduction's blocks
constexpr int kInBlockFixupMax = 8192;

// Error-free difference: a - b = s + err exactly, s = fl(a - b) (Knuth's two-sum).
__device__ __forceinline__ float two_diff_err(float a, float b, float s) {
    const float bv = __fsub_rn(s, a);
    const float av = __fsub_rn(s, bv);
    return __fadd_rn(__fsub_rn(a, av), __fsub_rn(-b, bv));
}

template <int NTH>
struct FixupShared {
    double wsum[NTH / 32][3];
};

struct Corr3 {
    double x, y, z;
};

// Block-wide sum of one value per thread and component; the result is thread 0's.
template <int NTH>
__device__ Corr3 block_sum3(double ax, double ay, double az, FixupShared<NTH>& sh) {
    const int li = threadIdx.x, warp = li >> 5, lane = li & 31;
    for (int o = 16; o > 0; o >>= 1) {
        ax += __shfl_down_sync(0xffffffffu, ax, o);
        ay += __shfl_down_sync(0xffffffffu, ay, o);
        az += __shfl_down_sync(0xffffffffu, az, o);
    }
    if (lane == 0) {
        sh.wsum[warp][0] = ax;
        sh.wsum[warp][1] = ay;
        sh.wsum[warp][2] = az;
    }
    __syncthreads();
    Corr3 r{0.0, 0.0, 0.0};
    if (li == 0)
        for (int w = 0; w < NTH / 32; w++) {
            r.x += sh.wsum[w][0];
            r.y += sh.wsum[w][1];
            r.z += sh.wsum[w][2];
        }
    __syncthreads();
    return r;
}

// Row of a flagged ion in FP64, chunk c of nch (contiguous j-ranges of the cloud's padded
// range; the padding ions carry no charge), by the whole block of NTH threads: the sum
// of q_j (x_i - x_j) / r^3 over the chunk, from the SI coordinates (thread 0's result).
// Re-evaluating only the dominant pairs is not enough: an ion whose FP32 terms cancel
// keeps the rounding of every addition made while a dominant term was in its partial sum
// (~1e-7 |f_max|), so the flagged ion's sum is replaced by its exact row.
template <int NTH>
__device__ Corr3 fixup_row(const SgCloud& cl, int i, const double* __restrict__ c64,
                           int npad_total, int c, int nch, FixupShared<NTH>& sh) {
    const size_t NP = (size_t)npad_total;
    const int igk = cl.poff + (i - cl.off);
    const double xi = c64[igk], yi = c64[NP + igk], zi = c64[2 * NP + igk];
    const int len = (cl.npad + nch - 1) / nch;
    const int j0 = c * len, j1 = min(cl.npad, j0 + len);
    double ax = 0.0, ay = 0.0, az = 0.0;
    // independent pairs in flight: each one's 1/r is a chain of dependent FP64 operations
#pragma unroll 4
    for (int j = j0 + (int)threadIdx.x; j < j1; j += NTH) {
        const int jg = cl.poff + j;
        if (jg == igk) continue;
        const double rx = xi - c64[jg], ry = yi - c64[NP + jg], rz = zi - c64[2 * NP + jg];
        const double inv = rsqrt_fp64(rx * rx + ry * ry + rz * rz);
        const double wq = c64[3 * NP + jg] * inv * inv * inv;
        ax = fma(wq, rx, ax);
        ay = fma(wq, ry, ay);
        az = fma(wq, rz, az);
    }
    return block_sum3<NTH>(ax, ay, az, sh);
}

// Far fix-up of ion i, chunk c of nch: the warps take the 128-ion tiles t = (c + m nch) W
// + w (W warps per block) that the Coulomb kernel treated as far from the ion's own
// tile, and each pair term f(u) = q u / |u|^3 of the hi-part difference u = fl(hi_j - hi_i)
// gets
//     delta = q y3 (D - 3 y^2 (u.D) u),   D = (lo_j - lo_i) + (hi_j - hi_i - u),
// the exact first-order change to the float-float difference (|D|/|u| ~ 1e-7, so the
// second order is far below FP32 rounding); y and y3 are formed as the kernel formed
// them.  Summed in FP32 per thread (the terms are small), in FP64 across the block;
// returns the correction of P_i (SI, thread 0).
template <int NTH>
__device__ Corr3 fixup_far(const SgCloud& cl, int i, const float* __restrict__ c32,
                           int npad_total, const float* __restrict__ bbox, int c, int nch,
                           FixupShared<NTH>& sh) {
    constexpr int W = NTH / 32;
    const int li = threadIdx.x;
    const int warp = li >> 5, lane = li & 31;
    const size_t NP = (size_t)npad_total;
    const int igk = cl.poff + (i - cl.off);
    const float xih = c32[igk], yih = c32[NP + igk], zih = c32[2 * NP + igk];
    const float xil = c32[4 * NP + igk], yil = c32[5 * NP + igk], zil = c32[6 * NP + igk];
    const int nt = (cl.npad + 127) / 128, itile = (igk - cl.poff) / 128;
    const float* ibox = bbox + 8 * (size_t)(cl.tile0 + itile);
    const float dfar2 = cl.dfar * cl.dfar;
    float fx = 0.f, fy = 0.f, fz = 0.f;
    for (int t = c * W + warp; t < nt; t += nch * W) {
        // the Coulomb kernel's far test for this (leaf, tile) pair, uniform per warp
        if (t == itile || !(box_dist2(ibox, bbox + 8 * (size_t)(cl.tile0 + t)) > dfar2)) continue;
        for (int jj = lane; jj < 128; jj += 32) {
            const int j = t * 128 + jj;
            if (j >= cl.npad) break;
            const int jg = cl.poff + j;
            const float xjh = c32[jg], yjh = c32[NP + jg], zjh = c32[2 * NP + jg];
            const float q = c32[3 * NP + jg];
            const float ux = __fsub_rn(xjh, xih), uy = __fsub_rn(yjh, yih), uz = __fsub_rn(zjh, zih);
            float r2 = __fmaf_rn(ux, ux, kTiny);
            r2 = __fmaf_rn(uy, uy, r2);
            r2 = __fmaf_rn(uz, uz, r2);
            const float y = rsqrt_approx(r2);
            const float y3 = __fmul_rn(__fmul_rn(y, y), y);
            const float dx = __fadd_rn(__fsub_rn(c32[4 * NP + jg], xil), two_diff_err(xjh, xih, ux));
            const float dy = __fadd_rn(__fsub_rn(c32[5 * NP + jg], yil), two_diff_err(yjh, yih, uy));
            const float dz = __fadd_rn(__fsub_rn(c32[6 * NP + jg], zil), two_diff_err(zjh, zih, uz));
            const float ud = fmaf(ux, dx, fmaf(uy, dy, uz * dz));
            const float s3 = 3.f * y * y * ud;
            const float qy3 = q * y3;
            fx = fmaf(qy3, fmaf(-s3, ux, dx), fx);
            fy = fmaf(qy3, fmaf(-s3, uy, dy), fy);
            fz = fmaf(qy3, fmaf(-s3, uz, dz), fz);
        }
    }
    Corr3 r = block_sum3<NTH>(fx, fy, fz, sh);
    // frame sums of q u / r^3 -> P (SI), as the kernel's epilogue scales them
    const double sc = -(cl.invL * cl.invL) * cl.qscale;
    r.x *= sc;
    r.y *= sc;
    r.z *= sc;
    return r;
}

// Whole fix-up of one flagged ion by one block: kFixNear replaces its sum by the exact
// FP64 row (which also covers its far terms); kFixFar alone adds the far correction
// (k-d ordered shapes).  Written to out by thread 0.  The j-ions are taken in a fixed
// order, so the result does not depend on which block runs it or when.
template <int NTH>
__device__ void fixup_ion(const SgCloud& cl, int i, int kind, const float* __restrict__ c32,
                          const double* __restrict__ c64, int npad_total,
                          double* __restrict__ out, int n_total, const float* __restrict__ bbox,
                          FixupShared<NTH>& sh) {
    if (kind & kFixNear) {
        const Corr3 r = fixup_row<NTH>(cl, i, c64, npad_total, 0, 1, sh);
        if (threadIdx.x == 0) {
            out[i] = r.x;
            out[(size_t)n_total + i] = r.y;
            out[2 * (size_t)n_total + i] = r.z;
        }
    } else if (bbox != nullptr) {
        const Corr3 r = fixup_far<NTH>(cl, i, c32, npad_total, bbox, 0, 1, sh);
        if (threadIdx.x == 0) {
            out[i] += r.x;
            out[(size_t)n_total + i] += r.y;
            out[2 * (size_t)n_total + i] += r.z;
        }
    }
    __syncthreads();
}

// Sums the j-chunk partials of each ion (x, y, z and the FP32c conditioning estimates
// s2, s2f) into out.  FP32c: an ion whose near terms cancel strongly (sqrt(s2) > 1.5 |P|,
// > |P| in clouds of up to kSmallRow ions) or whose far terms are large next to |P|
// (s2f > SgCloud::kfar2 |P|^2) is fixed up (fixup_ion): INBLOCK, by this block right away
// (small batches, where a second launch costs more than the work); otherwise it is put
// on a work list of coulomb_fixup_kernel (ion index; cloud | kind << 28): the ions whose
// row is re-evaluated in one list, the far-only ones in the other.
template <bool F32, bool INBLOCK>
__global__ void __launch_bounds__(SG_ROWS) coulomb_reduce_kernel(
    const SgRowBlock* __restrict__ rows, const SgCloud* __restrict__ clouds,
    const SgCtrl* __restrict__ ctrl, const double* __restrict__ part, int npad_total,
    double* __restrict__ out, int n_total, int* __restrict__ counters,
    int* __restrict__ fix_list, const float* __restrict__ c32,
    const double* __restrict__ c64, const float* __restrict__ bbox, float* __restrict__ risk,
    int* __restrict__ ran, const SgCheck* __restrict__ chk) {
    sg_griddep_wait();
    const SgRowBlock rb = rows[blockIdx.x];
    if (ctrl != nullptr &&
        (ctrl[rb.cloud].done || ctrl[rb.cloud].hold || ctrl[rb.cloud].status != SG_OK))
        return;
    const SgCloud& cl = clouds[rb.cloud];
    if (!(cl.fp.flags & SG_F_COULOMB)) return;
    const int li = threadIdx.x;
    const int i = rb.i0 + li;
    int kind = 0;
    double pf = 0.0;
    if (li < rb.n) {
        const int ig = cl.poff + (i - cl.off);
        const size_t NP = (size_t)npad_total;
        double px = 0.0, py = 0.0, pz = 0.0, s2 = 0.0, s2f = 0.0;
        for (int sl = 0; sl < cl.nslots; sl++) {
            const double* P = part + (size_t)sl * SG_PART_ARRAYS * NP;
            px += P[ig];
            py += P[NP + ig];
            pz += P[2 * NP + ig];
            if (F32) {
                s2 += P[3 * NP + ig];
                s2f += P[4 * NP + ig];
            }
        }
        out[i] = px;
        out[(size_t)n_total + i] = py;
        out[2 * (size_t)n_total + i] = pz;
        if (F32) {
            pf = sqrt(px * px + py * py + pz * pz) * (cl.L * cl.L);  // frame units
            // the far threshold: the prior of the frame set-up, or the measured one
            const double kf2 = chk ? fmin((double)cl.kfar2, (double)chk[rb.cloud].kfar2)
                                   : (double)cl.kfar2;
            const double kap2 = cl.npad <= kSmallRow ? kKappa2Small : kKappa2;
            kind = (s2 > kap2 * pf * pf ? kFixNear : 0) | (s2f > kf2 * pf * pf ? kFixFar : 0);
            if (risk != nullptr) {
                risk[i] = kind ? -1.f : (float)(sqrt(s2f) / pf);
                risk[(size_t)n_total + i] = kind ? -1.f : (float)(sqrt(s2) / pf);
            }
        }
    }
    if (F32 && ran != nullptr && li == 0) ran[rb.cloud] = 1;
    if (!F32) return;
    if (!INBLOCK) {
        if (kind) {
            // two lists: ions whose row is re-evaluated (kFixNear) from fix_list[2], the
            // far-only ones from fix_list[2 + 2N]
            const bool far = kind == kFixFar;
            const int at = atomicAdd(fix_list + (far ? 1 : 0), 1);
            const size_t base = far ? 2 + 2 * (size_t)n_total : 2;
            fix_list[base + 2 * at] = i;
            fix_list[base + 2 * at + 1] = rb.cloud | (kind << 28);
            if (counters != nullptr) atomicAdd(counters, 1);
        }
        return;
    }
    __shared__ FixupShared<SG_ROWS> sh;
    __shared__ int nflag;
    __shared__ int flist[SG_ROWS];
    __shared__ int fkind[SG_ROWS];
    if (li == 0) nflag = 0;
    __syncthreads();
    if (kind) {
        const int at = atomicAdd(&nflag, 1);
        flist[at] = i;
        fkind[at] = kind;
        if (counters != nullptr) atomicAdd(counters, 1);
    }
    __syncthreads();  // also orders this block's writes of out before the corrections
    const int nf = nflag;
    for (int k = 0; k < nf; k++)
        fixup_ion(cl, flist[k], fkind[k], c32, c64, npad_total, out, n_total, bbox, sh);
}

// The flagged ions of a whole batch, in two lists: the ions whose row is re-evaluated in
// FP64 (kFixNear) and the far-only ones (kFixFar).  Each of the first kChunkedCap ions of
// a list is kFarChunks work units, so that the scan of a large cloud is spread over
// blocks: each unit leaves its part in fix_part and the last unit of the ion (counted in
// fix_done) combines them in unit order -- writing the row, or adding the far correction
// -- so the result does not depend on the order the units ran in.  Units are numbered
// so that every ion's first units come first.  Ions past the caps are one unit each.
// Blocks of 256 threads, three per SM: the units of a 65,536-ion call run in one or two
// waves.
constexpr int kFixupThreads = 256;
__global__ void __launch_bounds__(kFixupThreads, 3) coulomb_fixup_kernel(
    const SgCloud* __restrict__ clouds, const float* __restrict__ c32,
    const double* __restrict__ c64, int npad_total, double* __restrict__ out, int n_total,
    const int* __restrict__ fix_list, const float* __restrict__ bbox,
    double* __restrict__ fix_part, int* __restrict__ fix_done) {
    sg_griddep_wait();
    __shared__ FixupShared<kFixupThreads> sh;
    __shared__ int last;
    constexpr int U = kFarChunks;
    const int cn = fix_list[0], cf = fix_list[1];
    const int* row_list = fix_list + 2;
    const int* far_list = fix_list + 2 + 2 * (size_t)n_total;
    const int cnc = min(cn, kChunkedCap), cfc = min(cf, kChunkedCap);
    const int u_rows = cnc * U + (cn - cnc);
    const int units = u_rows + cfc * U + (cf - cfc);
    for (int u = blockIdx.x; u < units; u += gridDim.x) {
        const bool row = u < u_rows;
        const int v = row ? u : u - u_rows;
        const int nc = row ? cnc : cfc;
        const int* list = row ? row_list : far_list;
        if (v >= nc * U) {  // past the cap: the whole ion in this unit
            const int k = nc + (v - nc * U);
            const int ck = list[2 * k + 1];
            fixup_ion<kFixupThreads>(clouds[ck & 0x0FFFFFFF], list[2 * k], ck >> 28, c32, c64,
                                     npad_total, out, n_total, bbox, sh);
            continue;
        }
        const int k = v % nc, c = v / nc;
        const int i = list[2 * k];
        const SgCloud& cl = clouds[list[2 * k + 1] & 0x0FFFFFFF];
        if (row && cl.npad <= kSmallRow) {  // a small cloud's row: unit 0 alone, whole
            if (c == 0)
                fixup_ion<kFixupThreads>(cl, i, kFixNear, c32, c64, npad_total, out, n_total,
                                         bbox, sh);
            continue;
        }
        Corr3 r{0.0, 0.0, 0.0};
        if (row)
            r = fixup_row<kFixupThreads>(cl, i, c64, npad_total, c, U, sh);
        else if (bbox != nullptr)
            r = fixup_far<kFixupThreads>(cl, i, c32, npad_total, bbox, c, U, sh);
        const size_t slot = (row ? 0 : (size_t)kChunkedCap) + (size_t)k;
        if (threadIdx.x == 0) {
            double* fp = fix_part + (slot * U + c) * 3;
            fp[0] = r.x;
            fp[1] = r.y;
            fp[2] = r.z;
            __threadfence();
            last = atomicAdd(&fix_done[slot], 1) == U - 1;
        }
        __syncthreads();
        if (last && threadIdx.x == 0) {
            __threadfence();
            const volatile double* vp = fix_part + slot * U * 3;
            double sx = 0.0, sy = 0.0, sz = 0.0;
            for (int q = 0; q < U; q++) {
                sx += vp[3 * q];
                sy += vp[3 * q + 1];
                sz += vp[3 * q + 2];
            }
            if (row) {
                out[i] = sx;
                out[(size_t)n_total + i] = sy;
                out[2 * (size_t)n_total + i] = sz;
            } else {
                out[i] += sx;
                out[(size_t)n_total + i] += sy;
                out[2 * (size_t)n_total + i] += sz;
            }
            fix_done[slot] = 0;  // ready for the next call
        }
        __syncthreads();
    }
}

}  // namespace

// Launch shapes of the FP32c kernel (threads per block, ions per thread); the work
// planner sizes i-blocks as threads x ions.  Variant 0 is the default.
static const int kC32Shapes[SG_C32_VARIANTS][2] = {{128, 4}, {128, 2}, {256, 2}, {64, 4},
                                                   {128, 4}, {64, 2}, {32, 4}, {32, 4},
                                                   {64, 2}, {128, 1}, {32, 2}, {32, 1},
                                                   {128, 1}, {64, 2}, {64, 2}, {32, 4},
                                                   {64, 2}};

int sg_coulomb_fp32c_ib(int variant) {
    if (variant < 0 || variant >= SG_C32_VARIANTS) variant = 0;
    return kC32Shapes[variant][0] * kC32Shapes[variant][1];
}

cudaError_t sg_launch_coulomb_fp32c(const SgCoulombArgs& a, cudaStream_t s) {
    if (a.n_items <= 0) return cudaSuccess;
    switch (a.variant) {
        case 1:
            sg_launch(coulomb_fp32c_kernel<128, 2>, a.n_items, 128, 0, s, 
                a.c32, a.c64, a.items, a.clouds, a.ctrl, a.part, a.npad_total, a.errword);
            break;
        case 2:
            sg_launch(coulomb_fp32c_kernel<256, 2>, a.n_items, 256, 0, s, 
                a.c32, a.c64, a.items, a.clouds, a.ctrl, a.part, a.npad_total, a.errword);
            break;
        case 3:
            sg_launch(coulomb_fp32c_kernel<64, 4>, a.n_items, 64, 0, s, 
                a.c32, a.c64, a.items, a.clouds, a.ctrl, a.part, a.npad_total, a.errword);
            break;
        case 5:
            sg_launch(coulomb_fp32c_kernel<64, 2>, a.n_items, 64, 0, s, 
                a.c32, a.c64, a.items, a.clouds, a.ctrl, a.part, a.npad_total, a.errword);
            break;
        case 6:
            sg_launch(coulomb_fp32c_kernel<32, 4>, a.n_items, 32, 0, s, 
                a.c32, a.c64, a.items, a.clouds, a.ctrl, a.part, a.npad_total, a.errword);
            break;
        case SG_C32_SORTED:
            sg_launch(coulomb_fp32c_sorted_kernel<128, 4, 4, SG_STAGES>, a.n_items, 128, 0, s, 
                a.c32, a.c64, a.items, a.clouds, a.ctrl, a.part, a.npad_total, a.errword, a.bbox);
            break;
        case SG_C32_SORTED_LEAF:
            // one k-d leaf per block: warps never wait for a slower (near) neighbour
            sg_launch(coulomb_fp32c_sorted_kernel<32, 4, 16, 3>, a.n_items, 32, 0, s, 
                a.c32, a.c64, a.items, a.clouds, a.ctrl, a.part, a.npad_total, a.errword, a.bbox);
            break;
        case 8:
            // one leaf per block split over two warps (same far/near decisions)
            sg_launch(coulomb_fp32c_sorted_kernel<64, 2, 12, 3>, a.n_items, 64, 0, s, 
                a.c32, a.c64, a.items, a.clouds, a.ctrl, a.part, a.npad_total, a.errword, a.bbox);
            break;
        case 9:
            if (a.far_estimate)
                sg_launch(coulomb_fp32c_sorted_kernel<128, 1, 8, 3>, a.n_items, 128, 0, s, 
                    a.c32, a.c64, a.items, a.clouds, a.ctrl, a.part, a.npad_total, a.errword, a.bbox);
            else
                sg_launch(coulomb_fp32c_sorted_kernel<128, 1, 8, 3, SG_TILE, 0, false>, a.n_items, 128, 0, s, 
                    a.c32, a.c64, a.items, a.clouds, a.ctrl, a.part, a.npad_total, a.errword, a.bbox);
            break;
        case 12:
            // as 9 with 256-ion j-tiles: half the ring waits and barriers per pair
            if (a.far_estimate)
                sg_launch(coulomb_fp32c_sorted_kernel<128, 1, 8, 3, 256>, a.n_items, 128, 0, s, 
                    a.c32, a.c64, a.items, a.clouds, a.ctrl, a.part, a.npad_total, a.errword, a.bbox);
            else
                sg_launch(coulomb_fp32c_sorted_kernel<128, 1, 8, 3, 256, 0, false>, a.n_items, 128, 0, s, 
                    a.c32, a.c64, a.items, a.clouds, a.ctrl, a.part, a.npad_total, a.errword, a.bbox);
            break;
        case 13:
            if (a.far_estimate)
                sg_launch(coulomb_fp32c_sorted_kernel<64, 2, 9, 3, 256>, a.n_items, 64, 0, s, 
                    a.c32, a.c64, a.items, a.clouds, a.ctrl, a.part, a.npad_total, a.errword, a.bbox);
            else
                sg_launch(coulomb_fp32c_sorted_kernel<64, 2, 9, 3, 256, 0, false>, a.n_items, 64, 0, s, 
                    a.c32, a.c64, a.items, a.clouds, a.ctrl, a.part, a.npad_total, a.errword, a.bbox);
            break;
        case 14:
            // as 13 with four j pairs in flight per ion on far tiles
            if (a.far_estimate)
                sg_launch(coulomb_fp32c_sorted_kernel<64, 2, 9, 3, 256, 4>, a.n_items, 64, 0, s, 
                    a.c32, a.c64, a.items, a.clouds, a.ctrl, a.part, a.npad_total, a.errword, a.bbox);
            else
                sg_launch(coulomb_fp32c_sorted_kernel<64, 2, 9, 3, 256, 4, false>, a.n_items, 64, 0, s, 
                    a.c32, a.c64, a.items, a.clouds, a.ctrl, a.part, a.npad_total, a.errword, a.bbox);
            break;
        case 15:
            // the leaf in one warp (4 ions per thread), 256-ion j-tiles
            sg_launch(coulomb_fp32c_sorted_kernel<32, 4, 16, 3, 256>, a.n_items, 32, 0, s, 
                a.c32, a.c64, a.items, a.clouds, a.ctrl, a.part, a.npad_total, a.errword, a.bbox);
            break;
        case 16:
            // as 13 with a 4-stage ring
            sg_launch(coulomb_fp32c_sorted_kernel<64, 2, 8, 4, 256>, a.n_items, 64, 0, s, 
                a.c32, a.c64, a.items, a.clouds, a.ctrl, a.part, a.npad_total, a.errword, a.bbox);
            break;
        case 10:
            sg_launch(coulomb_fp32c_kernel<32, 2>, a.n_items, 32, 0, s, 
                a.c32, a.c64, a.items, a.clouds, a.ctrl, a.part, a.npad_total, a.errword);
            break;
        case 11:
            sg_launch(coulomb_fp32c_kernel<32, 1>, a.n_items, 32, 0, s, 
                a.c32, a.c64, a.items, a.clouds, a.ctrl, a.part, a.npad_total, a.errword);
            break;
        default:
            sg_launch(coulomb_fp32c_kernel<128, 4>, a.n_items, 128, 0, s, 
                a.c32, a.c64, a.items, a.clouds, a.ctrl, a.part, a.npad_total, a.errword);
    }
    return cudaGetLastError();
}

cudaError_t sg_launch_coulomb_fp64(const SgCoulombArgs& a, cudaStream_t s) {
    if (a.n_items <= 0) return cudaSuccess;
    sg_launch(coulomb_fp64_kernel<SG_C64_THREADS, SG_C64_IPT>, a.n_items, SG_C64_THREADS, 0, s, 
        a.c64, a.items, a.ctrl, a.part, a.npad_total);
    return cudaGetLastError();
}

cudaError_t sg_launch_coulomb_reduce(const SgCoulombArgs& a, const SgRowBlock* rows, int n_rows,
                                     int fp32c, double* out, int n_total, int* counters,
                                     cudaStream_t s) {
    if (n_rows <= 0) return cudaSuccess;
    if (fp32c) {
        const float* bbox = sg_variant_sorted(a.variant) ? a.bbox : nullptr;
        if (n_total <= kInBlockFixupMax) {
            sg_launch(coulomb_reduce_kernel<true, true>, n_rows, SG_ROWS, 0, s, 
                rows, a.clouds, a.ctrl, a.part, a.npad_total, out, n_total, counters, nullptr,
                a.c32, a.c64, bbox, a.risk, a.ran, a.chk);
            return cudaGetLastError();
        }
        cudaError_t e = cudaMemsetAsync(a.fix_list, 0, 2 * sizeof(int), s);
        if (e != cudaSuccess) return e;
        coulomb_reduce_kernel<true, false><<<n_rows, SG_ROWS, 0, s>>>(
            rows, a.clouds, a.ctrl, a.part, a.npad_total, out, n_total, counters, a.fix_list,
            nullptr, nullptr, nullptr, a.risk, a.ran, a.chk);
        // a fixed grid that strides over however many work units there are (a batch of
        // small clouds can flag a few percent of its ions; unused blocks exit at once)
        const int grid = kFixupBlocks;
        sg_launch(coulomb_fixup_kernel, grid, kFixupThreads, 0, s, 
            a.clouds, a.c32, a.c64, a.npad_total, out, n_total, a.fix_list, bbox,
            a.fix_part, a.fix_done);
    } else {
        sg_launch(coulomb_reduce_kernel<false, false>, n_rows, SG_ROWS, 0, s, 
            rows, a.clouds, a.ctrl, a.part, a.npad_total, out, n_total, counters, nullptr,
            nullptr, nullptr, nullptr, nullptr, nullptr, nullptr);
    }
    return cudaGetLastError();
}
