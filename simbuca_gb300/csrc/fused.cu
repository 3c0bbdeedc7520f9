// fused.cu -- the small-cloud path: whole Dormand-Prince attempts of a cloud in one kernel.
//
// A cloud of a few thousand ions is latency-bound in every kernel of the tiled path: an
// attempt is 21 launches (stage 1, then for s = 2..7 the pair kernel, the reduction and
// stage s, then control and commit), each a few microseconds of dependent work on a
// handful of SMs, plus the launch gaps between them.  Here one thread-block cluster of
// up to 16 CTAs holds one cloud and runs its attempts back to back inside one launch,
// the phases separated by cluster barriers (hardware barriers of co-scheduled CTAs: no
// flag is spun on).  CTA r of the cluster owns the cloud's ions [r m, (r+1) m),
// m = ceil(n / R), in every phase:
//   * stage S (bin/ode.cpp:101-175): k_S from the field terms at t + c_S h and the
//     Coulomb sum, the next stage state y + h sum a_Sj k_j and its Coulomb inputs (SI and
//     FP32 frame coordinates), or for S = 7 the CTA's part of the error norm
//     (bin/ode.cpp:189-205);
//   * the Coulomb sum of stage S (bin/force.cpp:147-174): every CTA copies the cloud's
//     FP32 frame coordinates into shared memory and G threads sum each of its ions
//     against interleaved G-ths of the cloud, in the FP32-compensated form of the tiled kernel
//     (float-float differences, SFU 1/r, 1/r^3 capped with FP64 close pairs, partial sums
//     folded into Kahan accumulators every 16 j-ions); the G parts are added in FP64 in a
//     fixed order, and an ion whose terms cancel strongly (sqrt(s2) > 1.5 |P|) gets its
//     whole row in FP64 instead, as the tiled reduction does;
//   * control (CTA 0): error_succes and step() (sg_error_succes), then the commit
//     pos <- pos2, vel <- vel2 of accepted attempts (bin/ode.cpp:488-489).
// The cloud's coordinates, FP32 frame and SI, sit in shared memory during a Coulomb phase
// (close pairs and fix-ups read their SI coordinates there), which bounds the path to
// clouds of 2,048 ions.  Per-ion state stays in the batch's global arrays, so every other entry point (upload,
// download, moments, the tiled path itself) sees the same state.  Data a CTA wrote for
// its own ions it reads back itself; what other CTAs wrote (coordinates, the control
// block, error partials) is read with L2-only loads after the cluster barrier.
#include <cooperative_groups.h>
#include <math.h>

#include "dp_tableau.cuh"
#include "fp32c_math.cuh"
#include "sg_internal.cuh"

namespace cg = cooperative_groups;

namespace {

constexpr int kThreads = SG_FUSED_THREADS;
constexpr int kMaxIons = SG_FUSED_MAX_IONS;
constexpr int kFlush = 16;        // j-ions per FP32 partial sum before the Kahan fold
constexpr double kKappa2 = 2.25;  // FP64 row when s2 > 2.25 |P|^2 (the tiled reduction's for large clouds)

struct FusedShared {
    double part[kThreads][3];  // per thread: its part of P x, y, z (FP64)
    float s2[kThreads];        // per thread: its conditioning estimate
    int nflag;
    int flag_il[kThreads];     // flagged ions (local index) ...
    double flag_corr[kThreads][3];  // ... and their FP64 rows
};

__device__ __forceinline__ int ldcg_int(const int* p) { return __ldcg(p); }

// Stage S of the CTA's ions [lo, hi): k_S, then the state and Coulomb inputs of stage
// S+1, or (S = 7) the CTA's sum of squared scaled errors, returned on thread 0.
template <int S>
__device__ double stage_phase(const SgFusedArgs& f, const SgCloud& cl, const SgCtrl& cs, int lo,
                              int hi) {
    const size_t N = (size_t)f.n;
    const double h = cs.h;
    const bool frozen = (cl.fp.flags & SG_F_FROZEN_T) != 0;
    const double ts = frozen ? cs.t : cs.t + c_c[S] * h;
    const SgFieldCoef fk = sg_field_coef_block(cl.fp, ts);
    const int i = lo + (int)threadIdx.x;
    double acc2 = 0.0;
    if (i < hi) {
        const double* st = (S == 1) ? f.y : f.ys;
        const double px = st[i], py = st[N + i], pz = st[2 * N + i];
        const double vx = st[3 * N + i], vy = st[4 * N + i], vz = st[5 * N + i];
        double cx = 0.0, cy = 0.0, cz = 0.0;
        if (cl.fp.flags & SG_F_COULOMB) {
            const double* cs_ = (S == 1) ? f.coul1 : f.coulS;
            cx = cs_[i];
            cy = cs_[N + i];
            cz = cs_[2 * N + i];
            if (S == 7) {
                f.coul7[i] = cx;
                f.coul7[N + i] = cy;
                f.coul7[2 * N + i] = cz;
            }
        }
        double fx, fy, fz;
        sg_field_apply(cl.fp, fk, f.qm[i], px, py, pz, vx, vy, vz, fx, fy, fz);
        const double kqi = f.kq[i];
        double* kS = f.k + (size_t)(S - 1) * 6 * N;
        kS[i] = vx;
        kS[N + i] = vy;
        kS[2 * N + i] = vz;
        kS[3 * N + i] = fx + kqi * cx;
        kS[4 * N + i] = fy + kqi * cy;
        kS[5 * N + i] = fz + kqi * cz;
        if (S < 7) {
            double out[6];
#pragma unroll
            for (int c = 0; c < 6; c++) {
                double s = 0.0;
#pragma unroll
                for (int j = 1; j <= S; j++) s += c_a[S + 1][j - 1] * f.k[((size_t)(j - 1) * 6 + c) * N + i];
                out[c] = f.y[c * N + i] + h * s;
            }
#pragma unroll
            for (int c = 0; c < 6; c++) f.ys[c * N + i] = out[c];
            // Coulomb inputs of stage S+1 (SI and FP32 frame coordinates)
            const int ig = cl.poff + (i - cl.off);
            const size_t NP = (size_t)f.npad;
            f.c64[ig] = out[0];
            f.c64[NP + ig] = out[1];
            f.c64[2 * NP + ig] = out[2];
            const double u = (out[0] - cl.cx) * cl.invL, v = (out[1] - cl.cy) * cl.invL,
                         w = (out[2] - cl.cz) * cl.invL;
            const float uh = __double2float_rn(u), vh = __double2float_rn(v),
                        wh = __double2float_rn(w);
            f.c32[ig] = uh;
            f.c32[NP + ig] = vh;
            f.c32[2 * NP + ig] = wh;
            f.c32[4 * NP + ig] = __double2float_rn(u - (double)uh);
            f.c32[5 * NP + ig] = __double2float_rn(v - (double)vh);
            f.c32[6 * NP + ig] = __double2float_rn(w - (double)wh);
        } else {
            const double rtol = cs.rtol, atol = cs.atol;
#pragma unroll
            for (int c = 0; c < 6; c++) {
                double e = 0.0;
#pragma unroll
                for (int j = 1; j <= 7; j++)
                    if (j != 2) e += c_e[j] * f.k[((size_t)(j - 1) * 6 + c) * N + i];
                const double yerr = h * e;
                const double y0 = fabs(f.y[c * N + i]), y1 = fabs(f.ys[c * N + i]);
                const double sk = atol + rtol * ((y0 < y1) ? y1 : y0);
                const double r = yerr / sk;
                acc2 += r * r;
            }
        }
    }
    if constexpr (S == 7) {
        __shared__ double red[kThreads / 32];
        for (int o = 16; o > 0; o >>= 1) acc2 += __shfl_down_sync(0xffffffffu, acc2, o);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc2;
        __syncthreads();
        double s = 0.0;
        if (threadIdx.x == 0)
            for (int w = 0; w < kThreads / 32; w++) s += red[w];
        __syncthreads();
        return s;
    } else {
        return 0.0;
    }
}

// The Coulomb sums of the CTA's ions [lo, hi) at the current Coulomb inputs, into coulS
// (SI, m^-2), in the FP32-compensated form.  sc: the cloud's FP32 frame coordinates
// (7 x npad floats) and then its SI coordinates and charges (4 x npad doubles, 16-byte
// aligned) in shared memory.
__device__ void coulomb_phase(const SgFusedArgs& f, const SgCloud& cl, int lo, int hi, float* sc,
                              FusedShared& sh) {
    const int tid = threadIdx.x;
    const int npc = cl.npad;
    const size_t NP = (size_t)f.npad;
    double* sd = reinterpret_cast<double*>(sc + 7 * npc);  // 7 npc floats: a multiple of 16 B
    // the cloud's coordinates (written by every CTA of the cluster) through L2
    {
        const int nv = npc / 4;
        for (int q = tid; q < 7 * nv; q += kThreads) {
            const int a = q / nv, v = q - a * nv;
            const float4* src = reinterpret_cast<const float4*>(f.c32 + a * NP + cl.poff);
            reinterpret_cast<float4*>(sc + a * npc)[v] = __ldcg(src + v);
        }
        const int nd = npc / 2;
        for (int q = tid; q < 4 * nd; q += kThreads) {
            const int a = q / nd, v = q - a * nd;
            const double2* src = reinterpret_cast<const double2*>(f.c64 + a * NP + cl.poff);
            reinterpret_cast<double2*>(sd + a * npc)[v] = __ldcg(src + v);
        }
    }
    __syncthreads();
    const double* SX = sd;
    const double* SY = sd + npc;
    const double* SZ = sd + 2 * npc;
    const double* SQ = sd + 3 * npc;
    const float* X = sc;
    const float* Y = sc + npc;
    const float* Z = sc + 2 * npc;
    const float* Q = sc + 3 * npc;
    const float* XL = sc + 4 * npc;
    const float* YL = sc + 5 * npc;
    const float* ZL = sc + 6 * npc;
    const int m = hi - lo;
    // G threads per ion.  Thread q of an ion takes the packed j-pairs q, q + G, q + 2G, ...
    // (j = 2p, 2p + 1), so the G threads of an ion read consecutive 8-byte words of
    // shared memory (no bank conflicts; the ions of a warp read the same words); every 8
    // pairs (16 j-ions) its FP32 partial sums are folded into the Kahan accumulators.
    int G = 1;
    while (2 * G * m <= kThreads && 2 * G <= 32) G *= 2;
    const int il = tid / G, q = tid - (tid / G) * G;
    const int npair = npc / 2;
    const double invL2 = cl.invL * cl.invL;
    const double qscale = cl.qscale;
    const float wc = cl.wc;
    double px = 0.0, py = 0.0, pz = 0.0;
    float ps2 = 0.f;
    if (il < m) {
        const int i = lo + il;
        const int li = i - cl.off;  // index in the cloud's coordinate arrays
        const float xih = X[li], yih = Y[li], zih = Z[li];
        const float xil = XL[li], yil = YL[li], zil = ZL[li];
        const f2 xh = pk(xih, xih), yh = pk(yih, yih), zh = pk(zih, zih);
        const f2 xl = pk(xil, xil), yl = pk(yil, yil), zl = pk(zil, zil);
        const f2 tiny2 = pk(kTiny, kTiny);
        float ks[3] = {0.f, 0.f, 0.f}, kc[3] = {0.f, 0.f, 0.f}, s2 = 0.f, fmx = 0.f;
        double cx = 0.0, cy = 0.0, cz = 0.0;
        for (int p0 = q; p0 < npair; p0 += kFlush / 2 * G) {
            f2 ax = 0ull, ay = 0ull, az = 0ull;
            float y3max = 0.f;
#pragma unroll
            for (int u = 0; u < kFlush / 2; u++) {
                // past the cloud's last pair (ragged tail): pair 0 again, with no weight
                const bool ok = p0 + u * G < npair;
                const int jj = ok ? 2 * (p0 + u * G) : 0;
                const f2 Xj = *reinterpret_cast<const f2*>(X + jj);
                const f2 Yj = *reinterpret_cast<const f2*>(Y + jj);
                const f2 Zj = *reinterpret_cast<const f2*>(Z + jj);
                const f2 Qj = *reinterpret_cast<const f2*>(Q + jj);
                const f2 XLj = *reinterpret_cast<const f2*>(XL + jj);
                const f2 YLj = *reinterpret_cast<const f2*>(YL + jj);
                const f2 ZLj = *reinterpret_cast<const f2*>(ZL + jj);
                const f2 dx = add2(sub2(Xj, xh), sub2(XLj, xl));
                const f2 dy = add2(sub2(Yj, yh), sub2(YLj, yl));
                const f2 dz = add2(sub2(Zj, zh), sub2(ZLj, zl));
                f2 r2 = fma2(dx, dx, tiny2);
                r2 = fma2(dy, dy, r2);
                r2 = fma2(dz, dz, r2);
                float ra, rb;
                upk(r2, ra, rb);
                const f2 yv = pk(rsqrt_approx(ra), rsqrt_approx(rb));
                const f2 y3 = mul2(mul2(yv, yv), yv);
                float ua, ub;
                upk(y3, ua, ub);
                // the self pair (dx = 0, no contribution) stays out of the close-pair flag
                y3max = fmaxf(y3max, ok ? fmaxf(jj == li ? 0.f : ua, jj + 1 == li ? 0.f : ub) : 0.f);
                const f2 w = mul2(ok ? Qj : 0ull, pk(fminf(ua, wc), fminf(ub, wc)));
                ax = fma2(w, dx, ax);
                ay = fma2(w, dy, ay);
                az = fma2(w, dz, az);
            }
            float a, bb;
            upk(ax, a, bb);
            const float tx = __fadd_rn(a, bb);
            upk(ay, a, bb);
            const float ty = __fadd_rn(a, bb);
            upk(az, a, bb);
            const float tz = __fadd_rn(a, bb);
            kahan_add(ks[0], kc[0], tx);
            kahan_add(ks[1], kc[1], ty);
            kahan_add(ks[2], kc[2], tz);
            s2 = fmaf(tx, tx, fmaf(ty, ty, fmaf(tz, tz, s2)));
            if (y3max <= wc) fmx = fmaxf(fmx, y3max);  // blocks without a close pair
            if (y3max > wc) {
                // close pairs of this partial: the exact FP64 term, minus the capped FP32 term;
                // the block's strongest FP32 term (below the cap, or capped) for fmx
                const double xi = SX[li], yi = SY[li], zi = SZ[li];
                for (int u = 0; u < kFlush; u++) {
                    const int p = p0 + (u >> 1) * G;
                    if (p >= npair) break;
                    const int jj = 2 * p + (u & 1);
                    const PairF pr = pair_f32(X[jj], Y[jj], Z[jj], XL[jj], YL[jj], ZL[jj], xih,
                                              yih, zih, xil, yil, zil);
                    if (jj != li && Q[jj] != 0.f)
                        fmx = fmaxf(fmx, pr.y3 > wc ? capped_term_y3(pr.y3, wc) : pr.y3);
                    if (pr.y3 > wc && jj != li) {
                        const float wf = __fmul_rn(Q[jj], wc);
                        const double rx = xi - SX[jj];
                        const double ry = yi - SY[jj];
                        const double rz = zi - SZ[jj];
                        const double inv = rsqrt_fp64(rx * rx + ry * ry + rz * rz);
                        const double wq = SQ[jj] * inv * inv * inv;
                        const double wsc = invL2 * qscale * (double)wf;
                        cx += wq * rx + wsc * (double)pr.dx;
                        cy += wq * ry + wsc * (double)pr.dy;
                        cz += wq * rz + wsc * (double)pr.dz;
                    }
                }
            }
        }
        // P_i = -invL^2 qscale sum w (u_j - u_i) + close-pair terms (w carries q_j/qscale)
        const double s = -invL2 * qscale;
        px = s * ((double)ks[0] - (double)kc[0]) + cx;
        py = s * ((double)ks[1] - (double)kc[1]) + cy;
        pz = s * ((double)ks[2] - (double)kc[2]) + cz;
        ps2 = conditioning_s2(s2, fmx);
    }
    sh.part[tid][0] = px;
    sh.part[tid][1] = py;
    sh.part[tid][2] = pz;
    sh.s2[tid] = ps2;
    if (tid == 0) sh.nflag = 0;
    __syncthreads();
    // the G parts of each ion, in a fixed order; the conditioning test (in FP32, frame
    // units for a unit charge: a threshold test)
    double P[3] = {0.0, 0.0, 0.0};
    const int i = lo + tid;
    if (tid < m) {
        float s2 = 0.f;
        for (int g = 0; g < G; g++) {
            const double* pp = sh.part[tid * G + g];
            P[0] += pp[0];
            P[1] += pp[1];
            P[2] += pp[2];
            s2 += sh.s2[tid * G + g];
        }
        const float sc2 = (float)(cl.L * cl.L / qscale);  // SI sums -> frame units
        const float pf = sqrtf((float)(P[0] * P[0] + P[1] * P[1] + P[2] * P[2])) * sc2;
        const bool flagged = s2 > (float)kKappa2 * pf * pf;
        if (flagged) {
            const int at = atomicAdd(&sh.nflag, 1);
            sh.flag_il[at] = tid;
        }
        if (f.risk != nullptr) {
            f.risk[i] = flagged ? -1.f : 0.f;
            f.risk[(size_t)f.n + i] = flagged ? -1.f : sqrtf(s2) / pf;
        }
    }
    __syncthreads();
    // fix-up of the flagged ions, one warp per ion: the whole row in FP64 from the SI
    // coordinates, which replaces the ion's sum (re-evaluating only its dominant pairs
    // would keep the rounding of the FP32 additions made while they were in a partial sum)
    const int nf = sh.nflag;
    const int warp = tid >> 5, lane = tid & 31;
    for (int k = warp; k < nf; k += kThreads / 32) {
        const int li = lo + sh.flag_il[k] - cl.off;
        double ax = 0.0, ay = 0.0, az = 0.0;
        const double xi = SX[li], yi = SY[li], zi = SZ[li];
        for (int jj = lane; jj < npc; jj += 32) {
            if (jj == li) continue;
            const double rx = xi - SX[jj], ry = yi - SY[jj], rz = zi - SZ[jj];
            const double inv = rsqrt_fp64(rx * rx + ry * ry + rz * rz);
            const double wq = SQ[jj] * inv * inv * inv;
            ax = fma(wq, rx, ax);
            ay = fma(wq, ry, ay);
            az = fma(wq, rz, az);
        }
        for (int o = 16; o > 0; o >>= 1) {
            ax += __shfl_down_sync(0xffffffffu, ax, o);
            ay += __shfl_down_sync(0xffffffffu, ay, o);
            az += __shfl_down_sync(0xffffffffu, az, o);
        }
        if (lane == 0) {
            sh.flag_corr[k][0] = ax;
            sh.flag_corr[k][1] = ay;
            sh.flag_corr[k][2] = az;
        }
    }
    __syncthreads();
    for (int k = 0; k < nf; k++)
        if (sh.flag_il[k] == tid) {
            P[0] = sh.flag_corr[k][0];
            P[1] = sh.flag_corr[k][1];
            P[2] = sh.flag_corr[k][2];
        }
    if (tid < m) {
        const size_t N = (size_t)f.n;
        f.coulS[i] = P[0];
        f.coulS[N + i] = P[1];
        f.coulS[2 * N + i] = P[2];
    }
}

// One attempt's worth of control for cloud c (CTA 0, thread 0): error_succes, step()
// and the bookkeeping of dp_control_kernel for clouds without a recorder or operations.
__device__ void control_phase(const SgFusedArgs& f, const SgCloud& cl, int c, int nctas) {
    SgCtrl cs = f.ctrl[c];
    double s = 0.0;
    for (int r = 0; r < nctas; r++) s += __ldcg(f.errp + (size_t)c * SG_FUSED_MAX_CTAS + r);
    const double err = sqrt(s / (6 * cl.n));
    cs.err = err;
    cs.print_due = 0;
    cs.force_evals += 7;
    cs.coulomb_evals += (cl.fp.flags & SG_F_COULOMB) ? 6 : 0;
    int accepted;
    const int ew = ldcg_int(f.flags + SG_FLAG_ERR);
    if (ew != 0) {
        cs.status = ew;
        cs.done = 1;
        accepted = 0;
    } else {
        accepted = sg_error_succes(cs, err, f.y + cl.ion0);
    }
    if (accepted) {
        cs.h_last = cs.h;
        cs.t = cs.t + cs.h;
        cs.h = cs.hnext;
        cs.steps++;
        cs.rejects_here = 0;
        if (cs.t >= cs.t_end) cs.done = 1;
        if (f.flags[SG_FLAG_HOLD]) cs.hold |= 1;
    }
    cs.accepted = accepted;
    f.ctrl[c] = cs;
}

__global__ void __launch_bounds__(kThreads, 1) fused_attempts_kernel(SgFusedArgs f) {
    extern __shared__ __align__(16) float sc[];  // 7 x npad floats + 4 x npad doubles
    __shared__ FusedShared sh;
    cg::cluster_group cluster = cg::this_cluster();
    const int R = (int)cluster.num_blocks();
    const int r = (int)cluster.block_rank();
    const int c = blockIdx.x / R;
    if (c >= f.n_clouds) return;  // whole clusters only: uniform
    const SgCloud& cl = f.clouds[c];
    const int m = (cl.n + R - 1) / R;
    const int lo = cl.off + min(cl.n, r * m), hi = cl.off + min(cl.n, (r + 1) * m);
    const bool coul = (cl.fp.flags & SG_F_COULOMB) != 0;
    for (int att = 0; att < f.max_attempts; att++) {
        {
            // every CTA reads the control block after the previous cluster barrier
            const SgCtrl* cp = f.ctrl + c;
            if (ldcg_int(&cp->done) || ldcg_int(&cp->hold) || ldcg_int(&cp->status) != SG_OK ||
                ldcg_int(f.flags + SG_FLAG_ERR) != 0)
                break;
        }
        SgCtrl cs;
        cs.t = __ldcg(&f.ctrl[c].t);
        cs.h = __ldcg(&f.ctrl[c].h);
        cs.rtol = __ldcg(&f.ctrl[c].rtol);
        cs.atol = __ldcg(&f.ctrl[c].atol);
        stage_phase<1>(f, cl, cs, lo, hi);
        cluster.sync();
#define SG_FUSED_STAGE(S)                                      \
    if (coul) {                                                \
        coulomb_phase(f, cl, lo, hi, sc, sh);                  \
        cluster.sync();                                        \
    }                                                          \
    {                                                          \
        const double e = stage_phase<S>(f, cl, cs, lo, hi);    \
        if (S == 7 && threadIdx.x == 0)                        \
            f.errp[(size_t)c * SG_FUSED_MAX_CTAS + r] = e;     \
    }                                                          \
    cluster.sync();
        SG_FUSED_STAGE(2)
        SG_FUSED_STAGE(3)
        SG_FUSED_STAGE(4)
        SG_FUSED_STAGE(5)
        SG_FUSED_STAGE(6)
        SG_FUSED_STAGE(7)
#undef SG_FUSED_STAGE
        if (r == 0 && threadIdx.x == 0) control_phase(f, cl, c, R);
        cluster.sync();
        if (ldcg_int(&f.ctrl[c].accepted)) {
            // commit: pos <- pos2, vel <- vel2; the stage-7 sum is the next stage-1 sum
            const size_t N = (size_t)f.n;
            const int i = lo + (int)threadIdx.x;
            if (i < hi) {
#pragma unroll
                for (int q = 0; q < 6; q++) f.y[q * N + i] = f.ys[q * N + i];
#pragma unroll
                for (int q = 0; q < 3; q++) f.coul1[q * N + i] = f.coul7[q * N + i];
            }
        }
        if (f.ran != nullptr && coul && r == 0 && threadIdx.x == 0) f.ran[c] = 1;
        cluster.sync();
    }
}

}  // namespace

constexpr size_t smem_bytes(int npad) {
    return (7 * sizeof(float) + 4 * sizeof(double)) * (size_t)npad;
}

int sg_fused_cluster_size(int max_npad) {
    const size_t smem = smem_bytes(max_npad);
    if (cudaFuncSetAttribute(fused_attempts_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed,
                             1) != cudaSuccess)
        return 0;
    if (cudaFuncSetAttribute(fused_attempts_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem_bytes(kMaxIons)) != cudaSuccess)
        return 0;
    for (int R = SG_FUSED_MAX_CTAS; R >= 4; R /= 2) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(R);
        cfg.blockDim = dim3(kThreads);
        cfg.dynamicSmemBytes = smem;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = R;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        int n = 0;
        if (cudaOccupancyMaxActiveClusters(&n, fused_attempts_kernel, &cfg) == cudaSuccess && n > 0)
            return R;
    }
    cudaGetLastError();
    return 0;
}

cudaError_t sg_fused_attempts(const SgFusedArgs& f, int cluster, int max_npad, cudaStream_t st) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(f.n_clouds * cluster);
    cfg.blockDim = dim3(kThreads);
    cfg.dynamicSmemBytes = smem_bytes(max_npad);
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = cluster;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, fused_attempts_kernel, f);
}
