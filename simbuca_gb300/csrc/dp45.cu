// dp45.cu -- Dormand-Prince 5(4) stage, error-norm and step-control kernels of
// libsimgb (sm_103a), plus the O(N) helpers of the stand-alone force calls.
//
// Device layout (FP64, structure of arrays over all ions of all clouds, N ions):
//   y   [6][N]     state at the step start: x, y, z, vx, vy, vz  (IonCloud::pos/vel)
//   ys  [6][N]     stage state (IonCloud::pos2/vel2)
//   k   [7][6][N]  stage derivatives: stage velocity, stage acceleration (_ode_vars::k1..k7)
//   coul1, coul7 [3][N]  Coulomb sums P of stage 1 and stage 7
// The Coulomb inputs of the next stage are written by the stage kernel itself:
//   c64 [4][Npad] SI x, y, z, q;  c32 [7][Npad] frame hi x, y, z, q, lo x, y, z.
//
// One attempt = stage1, (coulomb, stage s) for s = 2..7, control, commit.  The stage-1
// Coulomb sum is never recomputed: after an accepted step the positions of stage 1
// are those of stage 7 (coul1 <- coul7), after a rejected one they are unchanged.
// The force count still follows the reference (7 per attempt, bin/ode.cpp:101-175).
#include <math.h>

#include "dp_tableau.cuh"
#include "sg_internal.cuh"

namespace {

typedef SgDpArgs DpArgs;

__device__ __forceinline__ void write_coords(const DpArgs& a, const SgCloud& cl, int ig,
                                             double x, double y, double z, float* hu = nullptr) {
    a.c64[ig] = x;
    a.c64[a.npad + ig] = y;
    a.c64[2 * (size_t)a.npad + ig] = z;
    if (a.fp32c) {
        const double u = (x - cl.cx) * cl.invL, v = (y - cl.cy) * cl.invL,
                     w = (z - cl.cz) * cl.invL;
        const float uh = __double2float_rn(u), vh = __double2float_rn(v),
                    wh = __double2float_rn(w);
        a.c32[ig] = uh;
        a.c32[a.npad + ig] = vh;
        a.c32[2 * (size_t)a.npad + ig] = wh;
        a.c32[4 * (size_t)a.npad + ig] = __double2float_rn(u - (double)uh);
        a.c32[5 * (size_t)a.npad + ig] = __double2float_rn(v - (double)vh);
        a.c32[6 * (size_t)a.npad + ig] = __double2float_rn(w - (double)wh);
        if (hu) {
            hu[0] = uh;
            hu[1] = vh;
            hu[2] = wh;
        }
    }
}


// Bounds of the 128-ion tiles covered by a row block (256 ions = 2 tiles of the cloud):
// min/max of the FP32 frame coordinates of the block's real ions.
__device__ __forceinline__ void tile_bounds(const DpArgs& a, const SgCloud& cl,
                                            const SgRowBlock& rb, bool active, float u,
                                            float v, float w) {
    __shared__ float sb[SG_ROWS / 32][6];
    float b[6] = {active ? u : INFINITY, active ? v : INFINITY, active ? w : INFINITY,
                  active ? u : -INFINITY, active ? v : -INFINITY, active ? w : -INFINITY};
    for (int o = 16; o > 0; o >>= 1)
        for (int q = 0; q < 6; q++) {
            const float x = __shfl_xor_sync(0xffffffffu, b[q], o);
            b[q] = q < 3 ? fminf(b[q], x) : fmaxf(b[q], x);
        }
    const int warp = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0)
        for (int q = 0; q < 6; q++) sb[warp][q] = b[q];
    __syncthreads();
    if (threadIdx.x < 2) {
        const int h = threadIdx.x;                 // tile 0 or 1 of this row block
        float r[6];
        for (int q = 0; q < 6; q++) r[q] = sb[4 * h][q];
        for (int wv = 4 * h + 1; wv < 4 * h + 4; wv++)
            for (int q = 0; q < 6; q++) r[q] = q < 3 ? fminf(r[q], sb[wv][q]) : fmaxf(r[q], sb[wv][q]);
        const int local = rb.i0 - cl.off;          // multiple of SG_ROWS
        const int tile = local / 128 + h;
        if (local + 128 * h < cl.n) {
            float* B = a.bbox + 8 * (size_t)(cl.tile0 + tile);
            for (int q = 0; q < 6; q++) B[q] = r[q];
        }
    }
}

// Stage S (1..7) evaluated: finish its force, store k_S, build stage S+1 (or, for
// S = 7, the embedded error of the attempt).
template <int S>
__global__ void __launch_bounds__(SG_ROWS) dp_stage_kernel(DpArgs a) {
    sg_griddep_wait();
    __shared__ double red[SG_ROWS / 32];
    const SgRowBlock rb = a.rows[blockIdx.x];
    const SgCtrl& cs = a.ctrl[rb.cloud];
    if (cs.done || cs.hold || cs.status != SG_OK) return;
    const SgCloud& cl = a.clouds[rb.cloud];
    const int li = threadIdx.x;
    const bool active = li < rb.n;
    const int i = rb.i0 + (active ? li : 0);
    const int ig = cl.poff + (i - cl.off);
    const size_t N = (size_t)a.n;
    const double h = cs.h;
    const bool frozen = (cl.fp.flags & SG_F_FROZEN_T) != 0;
    const double ts = frozen ? cs.t : cs.t + c_c[S] * h;
    const SgFieldCoef fk = sg_field_coef_block(cl.fp, ts);

    double acc2 = 0.0;
    float hu[3] = {0.f, 0.f, 0.f};
    if (active) {
        const double* st = (S == 1) ? a.y : a.ys;
        const double px = st[i], py = st[N + i], pz = st[2 * N + i];
        const double vx = st[3 * N + i], vy = st[4 * N + i], vz = st[5 * N + i];
        double cx = 0.0, cy = 0.0, cz = 0.0;
        if (cl.fp.flags & SG_F_COULOMB) {
            if (S == 1) {
                cx = a.coul1[i];
                cy = a.coul1[N + i];
                cz = a.coul1[2 * N + i];
            } else {
                cx = a.coulS[i];
                cy = a.coulS[N + i];
                cz = a.coulS[2 * N + i];
                if (S == 7) {
                    a.coul7[i] = cx;
                    a.coul7[N + i] = cy;
                    a.coul7[2 * N + i] = cz;
                }
            }
        }
        double fx, fy, fz;
        sg_field_apply(cl.fp, fk, a.qm[i], px, py, pz, vx, vy, vz, fx, fy, fz);
        const double kqi = a.kq[i];
        double* kS = a.k + (size_t)(S - 1) * 6 * N;
        kS[i] = vx;
        kS[N + i] = vy;
        kS[2 * N + i] = vz;
        kS[3 * N + i] = fx + kqi * cx;
        kS[4 * N + i] = fy + kqi * cy;
        kS[5 * N + i] = fz + kqi * cz;

        if (S < 7) {
            // stage S+1: y + h * sum_j a[S+1][j] k_j   (bin/ode.cpp:107-173)
            double out[6];
#pragma unroll
            for (int c = 0; c < 6; c++) {
                double s = 0.0;
#pragma unroll
                for (int j = 1; j <= S; j++) s += c_a[S + 1][j - 1] * a.k[((size_t)(j - 1) * 6 + c) * N + i];
                out[c] = a.y[c * N + i] + h * s;
            }
#pragma unroll
            for (int c = 0; c < 6; c++) a.ys[c * N + i] = out[c];
            write_coords(a, cl, ig, out[0], out[1], out[2], hu);
        } else {
            // embedded error of the attempt (bin/ode.cpp:189-205); y5 = stage-7 state
            const double rtol = cs.rtol, atol = cs.atol;
#pragma unroll
            for (int c = 0; c < 6; c++) {
                double e = 0.0;
#pragma unroll
                for (int j = 1; j <= 7; j++)
                    if (j != 2) e += c_e[j] * a.k[((size_t)(j - 1) * 6 + c) * N + i];
                const double yerr = h * e;
                const double y0 = fabs(a.y[c * N + i]), y1 = fabs(a.ys[c * N + i]);
                const double sk = atol + rtol * ((y0 < y1) ? y1 : y0);
                const double r = yerr / sk;
                acc2 += r * r;
            }
        }
    }
    if (S < 7 && a.fp32c && a.bbox) tile_bounds(a, cl, rb, active, hu[0], hu[1], hu[2]);
    if (S == 7) {
        // deterministic block reduction -> one partial per row block
        for (int o = 16; o > 0; o >>= 1) acc2 += __shfl_down_sync(0xffffffffu, acc2, o);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc2;
        __syncthreads();
        if (threadIdx.x == 0) {
            double s = 0.0;
            for (int w = 0; w < SG_ROWS / 32; w++) s += red[w];
            a.err_part[blockIdx.x] = s;
        }
    }
}


// ---- Cash-Karp 5(4), the reference's "RungaKutta4" (bin/ode.cpp:220-345) ----------
__constant__ double c_ck_a[7][6] = {
    {0, 0, 0, 0, 0, 0},
    {0, 0, 0, 0, 0, 0},
    {0.2, 0, 0, 0, 0, 0},
    {3.0 / 40.0, 9.0 / 40.0, 0, 0, 0, 0},
    {0.3, -0.9, 1.2, 0, 0, 0},
    {-11.0 / 54.0, 2.5, -70.0 / 27.0, 35.0 / 27.0, 0, 0},
    {1631.0 / 55296.0, 175.0 / 512.0, 575.0 / 13824.0, 44275.0 / 110592.0, 253.0 / 4096.0, 0}};
__constant__ double c_ck_c[7] = {0, 0.0, 0.2, 0.3, 0.6, 1.0, 0.875};
__constant__ double c_ck_b[7] = {0, 37.0 / 378.0, 0.0, 250.0 / 621.0, 125.0 / 594.0, 0.0,
                                 512.0 / 1771.0};
__constant__ double c_ck_e[7] = {0,
                                 37.0 / 378.0 - 2825.0 / 27648.0,
                                 0.0,
                                 250.0 / 621.0 - 18575.0 / 48384.0,
                                 125.0 / 594.0 - 13525.0 / 55296.0,
                                 -277.00 / 14336.0,
                                 512.0 / 1771.0 - 0.25};

// Stage S (1..6) of Cash-Karp: finish its force (the Coulomb sum of every stage comes
// from coulS: no stage coincides with the next step's start), store k_S, build stage
// S+1, or for S = 6 the 5th-order solution (into ys) and the embedded error.
template <int S>
__global__ void __launch_bounds__(SG_ROWS) ck_stage_kernel(DpArgs a) {
    sg_griddep_wait();
    __shared__ double red[SG_ROWS / 32];
    const SgRowBlock rb = a.rows[blockIdx.x];
    const SgCtrl& cs = a.ctrl[rb.cloud];
    if (cs.done || cs.hold || cs.status != SG_OK) return;
    const SgCloud& cl = a.clouds[rb.cloud];
    const int li = threadIdx.x;
    const bool active = li < rb.n;
    const int i = rb.i0 + (active ? li : 0);
    const int ig = cl.poff + (i - cl.off);
    const size_t N = (size_t)a.n;
    const double h = cs.h;
    const bool frozen = (cl.fp.flags & SG_F_FROZEN_T) != 0;
    const double ts = frozen ? cs.t : cs.t + c_ck_c[S] * h;
    const SgFieldCoef fk = sg_field_coef_block(cl.fp, ts);
    double acc2 = 0.0;
    float hu[3] = {0.f, 0.f, 0.f};
    if (active) {
        const double* st = (S == 1) ? a.y : a.ys;
        const double px = st[i], py = st[N + i], pz = st[2 * N + i];
        const double vx = st[3 * N + i], vy = st[4 * N + i], vz = st[5 * N + i];
        double cx = 0.0, cy = 0.0, cz = 0.0;
        if (cl.fp.flags & SG_F_COULOMB) {
            cx = a.coulS[i];
            cy = a.coulS[N + i];
            cz = a.coulS[2 * N + i];
        }
        double fx, fy, fz;
        sg_field_apply(cl.fp, fk, a.qm[i], px, py, pz, vx, vy, vz, fx, fy, fz);
        const double kqi = a.kq[i];
        double* kS = a.k + (size_t)(S - 1) * 6 * N;
        kS[i] = vx;
        kS[N + i] = vy;
        kS[2 * N + i] = vz;
        kS[3 * N + i] = fx + kqi * cx;
        kS[4 * N + i] = fy + kqi * cy;
        kS[5 * N + i] = fz + kqi * cz;
        if (S < 6) {
            double out[6];
#pragma unroll
            for (int c = 0; c < 6; c++) {
                double sum = 0.0;
#pragma unroll
                for (int j = 1; j <= S; j++) sum += c_ck_a[S + 1][j - 1] * a.k[((size_t)(j - 1) * 6 + c) * N + i];
                out[c] = a.y[c * N + i] + h * sum;
            }
#pragma unroll
            for (int c = 0; c < 6; c++) a.ys[c * N + i] = out[c];
            write_coords(a, cl, ig, out[0], out[1], out[2], hu);
        } else {
            const double rtol = cs.rtol, atol = cs.atol;
#pragma unroll
            for (int c = 0; c < 6; c++) {
                double b = 0.0, e = 0.0;
#pragma unroll
                for (int j = 1; j <= 6; j++) {
                    const double kj = a.k[((size_t)(j - 1) * 6 + c) * N + i];
                    b += c_ck_b[j] * kj;
                    e += c_ck_e[j] * kj;
                }
                const double y0 = a.y[c * N + i];
                const double y5 = y0 + h * b;
                a.ys[c * N + i] = y5;
                const double yerr = h * e;
                const double m0 = fabs(y0), m1 = fabs(y5);
                const double sk = atol + rtol * ((m0 < m1) ? m1 : m0);
                const double r = yerr / sk;
                acc2 += r * r;
            }
        }
    }
    if (S < 6 && a.fp32c && a.bbox) tile_bounds(a, cl, rb, active, hu[0], hu[1], hu[2]);
    if (S == 6) {
        for (int o = 16; o > 0; o >>= 1) acc2 += __shfl_down_sync(0xffffffffu, acc2, o);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc2;
        __syncthreads();
        if (threadIdx.x == 0) {
            double sum = 0.0;
            for (int w = 0; w < SG_ROWS / 32; w++) sum += red[w];
            a.err_part[blockIdx.x] = sum;
        }
    }
}


// ---- Gear predictor-corrector, the reference's GearMethod (bin/ode.cpp:347-424) ----
// Fifth-order Nordsieck form with one force evaluation per step and a fixed step.
// Gear state in k, by column: acceleration of the last force call [0..2], b [3..5],
// c [6..8], d [9..11].  The e terms of the reference are never read there; left out.
#define SG_GEA0 (3.0 / 20.0)
#define SG_GEA1 (251.0 / 360.0)
#define SG_GEA3 (11.0 / 18.0)
#define SG_GEA4 (1.0 / 6.0)
#define SG_GEA5 (1.0 / 60.0)

// InitAcceleraction (bin/ode.cpp:36-59): constant seeds for every ion of a cloud but the
// last in the caller's order (left as allocated there, zero here); b = c = d = 0.
__global__ void __launch_bounds__(SG_ROWS) gear_init_kernel(DpArgs a, const int* __restrict__ perm) {
    sg_griddep_wait();
    const SgRowBlock rb = a.rows[blockIdx.x];
    const SgCloud& cl = a.clouds[rb.cloud];
    const int li = threadIdx.x;
    if (li >= rb.n) return;
    const int i = rb.i0 + li;
    const size_t N = (size_t)a.n;
    const int caller = perm ? perm[i] : i;
    const bool last = caller == cl.off + cl.n - 1;
    a.k[i] = last ? 0.0 : 1.6e9;
    a.k[N + i] = last ? 0.0 : 1.1e9;
    a.k[2 * N + i] = last ? 0.0 : -5e8;
#pragma unroll
    for (int c = 3; c < 12; c++) a.k[c * N + i] = 0.0;
}

template <int PHASE>
__global__ void __launch_bounds__(SG_ROWS) gear_kernel(DpArgs a) {
    sg_griddep_wait();
    const SgRowBlock rb = a.rows[blockIdx.x];
    const SgCtrl& cs = a.ctrl[rb.cloud];
    if (cs.done || cs.hold || cs.status != SG_OK) return;
    const SgCloud& cl = a.clouds[rb.cloud];
    const int li = threadIdx.x;
    const bool active = li < rb.n;
    const int i = rb.i0 + (active ? li : 0);
    const int ig = cl.poff + (i - cl.off);
    const size_t N = (size_t)a.n;
    const double h = cs.h;
    const double h2f = cs.hf[0], h3f = cs.hf[1], h4f = cs.hf[2], h5f = cs.hf[3];
    float hu[3] = {0.f, 0.f, 0.f};
    int bad = 0;
    if (active) {
        if (PHASE == 0) {
            // predictor: Taylor series of the Nordsieck vector (bin/ode.cpp:367-375)
            double p2[3];
#pragma unroll
            for (int c = 0; c < 3; c++) {
                const double ac = a.k[c * N + i], b = a.k[(3 + c) * N + i];
                const double cc = a.k[(6 + c) * N + i], d = a.k[(9 + c) * N + i];
                const double x = a.y[c * N + i], v = a.y[(3 + c) * N + i];
                p2[c] = x + v * h + ac * h2f + b * h3f + cc * h4f + d * h5f;
                a.ys[c * N + i] = p2[c];
                a.ys[(3 + c) * N + i] = v + ac * h + b * h2f + cc * h3f + d * h4f;
            }
            write_coords(a, cl, ig, p2[0], p2[1], p2[2], hu);
        } else {
            // corrector (bin/ode.cpp:396-420) with the force at the predicted state
            const bool frozen = (cl.fp.flags & SG_F_FROZEN_T) != 0;
            const double ts = frozen ? cs.t : cs.t + h;
            double st[6];
#pragma unroll
            for (int c = 0; c < 6; c++) st[c] = a.ys[c * N + i];
            double f[3];
            sg_field_accel(cl.fp, ts, a.qm[i], st[0], st[1], st[2], st[3], st[4], st[5], f[0],
                           f[1], f[2]);
            if (cl.fp.flags & SG_F_COULOMB) {
                const double kqi = a.kq[i];
#pragma unroll
                for (int c = 0; c < 3; c++) f[c] += kqi * a.coulS[c * N + i];
            }
#pragma unroll
            for (int c = 0; c < 3; c++) {
                const double ac = a.k[c * N + i], b = a.k[(3 + c) * N + i];
                const double cc = a.k[(6 + c) * N + i], d = a.k[(9 + c) * N + i];
                const double sug = ac + b * h + cc * h2f + d * h3f;
                const double bn = b + cc * h + d * h2f;
                const double cn = cc + d * h;
                const double ad = h2f * (f[c] - sug);
                const double x = st[c] + SG_GEA0 * ad;
                const double v = st[3 + c] + SG_GEA1 * ad / h;
                a.ys[c * N + i] = x;
                a.ys[(3 + c) * N + i] = v;
                a.k[c * N + i] = f[c];
                a.k[(3 + c) * N + i] = bn + SG_GEA3 * ad / h3f;
                a.k[(6 + c) * N + i] = cn + SG_GEA4 * ad / h4f;
                a.k[(9 + c) * N + i] = d + SG_GEA5 * ad / h5f;
                bad |= !isfinite(x) || !isfinite(v);
            }
        }
    }
    if (PHASE == 0) {
        if (a.fp32c && a.bbox) tile_bounds(a, cl, rb, active, hu[0], hu[1], hu[2]);
    } else {
        // no error estimate: the partial is 0, or NaN when the step left finite numbers
        bad = __syncthreads_or(bad);
        if (threadIdx.x == 0) a.err_part[blockIdx.x] = bad ? __longlong_as_double(0x7ff8000000000000LL) : 0.0;
    }
}

// error_succes + step bookkeeping (bin/ode.cpp:426-494), one thread per cloud.
// With flags[SG_FLAG_HOLD] set, a cloud that accepts holds (skips further attempts) until
// the host clears the hold: used to take exactly one step per cloud.
__global__ void dp_control_kernel(SgCloud* __restrict__ clouds, SgCtrl* __restrict__ ctrl,
                                  const double* __restrict__ err_part, const double* __restrict__ y,
                                  int n_clouds, const int* __restrict__ flags,
                                  const SgOp* __restrict__ ops) {
    sg_griddep_wait();
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n_clouds) return;
    SgCtrl cs = ctrl[c];
    const SgCloud cl = clouds[c];
    if (cs.done || cs.hold || cs.status != SG_OK) {
        ctrl[c].accepted = 0;
        ctrl[c].print_due = 0;
        return;
    }
    cs.print_due = 0;
    double s = 0.0;
    // Cash-Karp: the reference adds to the previous norm, odev.err is never reset there
    if (cs.method == 4) s = cs.err;
    for (int b = 0; b < cl.nrb; b++) s += err_part[cl.rb0 + b];
    const double err = sqrt(s / (6 * cl.n));
    cs.err = err;
    cs.force_evals += (cs.method == 4) ? 6 : (cs.method == 1 ? 1 : 7);
    cs.coulomb_evals += (cl.fp.flags & SG_F_COULOMB) ? (cs.method == 1 ? 1 : 6) : 0;
    int accepted = 1;
    if (flags[SG_FLAG_ERR] != 0) {
        // a kernel of this attempt gave up a bounded wait: its sums are incomplete, so
        // the attempt is neither accepted nor used for step control
        cs.status = flags[SG_FLAG_ERR];
        cs.done = 1;
        accepted = 0;
    } else {
        // IonCloud::pos[0][0] (bin/ode.cpp:482): x of the caller's first ion
        accepted = sg_error_succes(cs, err, y + cl.ion0);
    }
    if (accepted) {
        cs.h_last = cs.h;
        cs.t = cs.t + cs.h;
        cs.h = cs.hnext;
        cs.steps++;
        cs.rejects_here = 0;
        int print_now = 0;
        if (cs.n_ops > 0) {
            cs.dis_due = 0;
            if (cs.t >= cs.t_end) {
                // the operation has ended: print after it, start the next one
                print_now = ops[cs.op_index].print_after;
                print_now |= sg_start_ops(cs, clouds[c].fp, ops, cs.op_index + 1);
            } else if (ops[cs.op_index].kind == SG_OP_TRAP_RAMP) {
                // Vrf/Vdc for the next step (bin/ion_fly.cpp:95-99)
                const SgOp& op = ops[cs.op_index];
                const double ramp = (cs.t - cs.t_op_start) / (cs.t_end - cs.t_op_start);
                clouds[c].fp.Vrf = cs.old_vrf * (1 - ramp) + op.new_vrf * ramp;
                clouds[c].fp.Vdc = cs.old_vdc * (1 - ramp) + op.new_vdc * ramp;
            }
        } else if (cs.t >= cs.t_end) {
            cs.done = 1;
        }
        if (flags[SG_FLAG_HOLD]) cs.hold |= 1;
        // the reference prints after a step once (t - start) > interval * prints so far
        // (bin/ion_fly.cpp:103-108); the record goes to the next ring slot, and a full
        // ring holds the cloud until the host has drained it
        const bool rule = cs.print_interval > 0.0 &&
                          (cs.t - cs.t_print0) > cs.print_interval * (double)cs.n_print;
        if (cs.rec_cap > 0 && (rule || print_now)) {
            if (rule) cs.n_print++;
            if (cs.rec_count - cs.rec_drained < cs.rec_cap) {
                cs.print_due = 1;
                cs.rec_slot = (int)(cs.rec_count % cs.rec_cap);
                cs.rec_count++;
            }
            if (cs.rec_count - cs.rec_drained >= cs.rec_cap) cs.hold |= 2;
        }
    }
    cs.accepted = accepted;
    ctrl[c] = cs;
}

__global__ void clear_hold_kernel(SgCtrl* ctrl, int n_clouds) {
    sg_griddep_wait();
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < n_clouds) ctrl[c].hold &= ~1;
}

// Commit an accepted attempt: pos <- pos2, vel <- vel2 (bin/ode.cpp:488-489) and the
// stage-7 Coulomb sum becomes the next stage-1 sum.
__global__ void __launch_bounds__(SG_ROWS) dp_commit_kernel(DpArgs a) {
    sg_griddep_wait();
    const SgRowBlock rb = a.rows[blockIdx.x];
    if (!a.ctrl[rb.cloud].accepted) return;
    const int li = threadIdx.x;
    if (li >= rb.n) return;
    const int i = rb.i0 + li;
    const size_t N = (size_t)a.n;
#pragma unroll
    for (int c = 0; c < 6; c++) a.y[c * N + i] = a.ys[c * N + i];
#pragma unroll
    for (int c = 0; c < 3; c++) a.coul1[c * N + i] = a.coul7[c * N + i];
}

// Coulomb inputs of the state y (set-up and stand-alone calls); ghosts get q = 0.
__global__ void __launch_bounds__(SG_ROWS) coords_from_state_kernel(DpArgs a,
                                                                    const double* __restrict__ q) {
    sg_griddep_wait();
    const SgRowBlock rb = a.rows[blockIdx.x];
    const SgCloud& cl = a.clouds[rb.cloud];
    const int li = threadIdx.x;
    const size_t N = (size_t)a.n;
    // this block also covers the ghost tail of its cloud when it holds the cloud's last row
    const bool last = (rb.i0 + rb.n == cl.off + cl.n);
    float hu[3] = {0.f, 0.f, 0.f};
    if (li < rb.n) {
        const int i = rb.i0 + li;
        const int ig = cl.poff + (i - cl.off);
        write_coords(a, cl, ig, a.y[i], a.y[N + i], a.y[2 * N + i], hu);
        a.c64[3 * (size_t)a.npad + ig] = q[i];
        if (a.fp32c) a.c32[3 * (size_t)a.npad + ig] = (float)(q[i] / cl.qscale);
    }
    if (a.fp32c && a.bbox) tile_bounds(a, cl, rb, li < rb.n, hu[0], hu[1], hu[2]);
    if (last) {
        for (int g = cl.n + li; g < cl.npad; g += blockDim.x) {
            const int ig = cl.poff + g;
            // far away, no charge: contributes exactly zero as a j-ion
            const double far = 1.0e3 + 1.0e-3 * g;
            a.c64[ig] = far;
            a.c64[a.npad + ig] = far;
            a.c64[2 * (size_t)a.npad + ig] = far;
            a.c64[3 * (size_t)a.npad + ig] = 0.0;
            if (a.fp32c) {
                const float ff = 1.0e4f + (float)g;
                a.c32[ig] = ff;
                a.c32[a.npad + ig] = ff;
                a.c32[2 * (size_t)a.npad + ig] = ff;
                a.c32[3 * (size_t)a.npad + ig] = 0.f;
                a.c32[4 * (size_t)a.npad + ig] = 0.f;
                a.c32[5 * (size_t)a.npad + ig] = 0.f;
                a.c32[6 * (size_t)a.npad + ig] = 0.f;
            }
        }
    }
}

// Stand-alone force: out[i][c] (AoS) = field(t) + kq_i * sum_slots P (if Coulomb).
__global__ void __launch_bounds__(SG_ROWS) force_finish_kernel(DpArgs a, double t,
                                                               int with_field,
                                                               const int* __restrict__ perm,
                                                               double* __restrict__ out) {
    sg_griddep_wait();
    const SgRowBlock rb = a.rows[blockIdx.x];
    const SgCloud& cl = a.clouds[rb.cloud];
    const int li = threadIdx.x;
    if (li >= rb.n) return;
    const int i = rb.i0 + li;
    const size_t N = (size_t)a.n;
    double cx = 0.0, cy = 0.0, cz = 0.0;
    if (cl.fp.flags & SG_F_COULOMB) {
        cx = a.coulS[i];
        cy = a.coulS[N + i];
        cz = a.coulS[2 * N + i];
    }
    double fx = 0.0, fy = 0.0, fz = 0.0;
    if (with_field)
        sg_field_accel(cl.fp, t, a.qm[i], a.y[i], a.y[N + i], a.y[2 * N + i], a.y[3 * N + i],
                       a.y[4 * N + i], a.y[5 * N + i], fx, fy, fz);
    const double kqi = a.kq[i];
    const size_t o = 3 * (size_t)(perm ? perm[i] : i);
    out[o + 0] = fx + kqi * cx;
    out[o + 1] = fy + kqi * cy;
    out[o + 2] = fz + kqi * cz;
}

// AoS host layout -> SoA state (positions and velocities).
// y[c][k] = pos[perm[k]][c]: the caller's order into the device (sorted) order.
__global__ void aos_to_soa_kernel(const double* __restrict__ pos, const double* __restrict__ vel,
                                  const int* __restrict__ perm, double* __restrict__ y, int n) {
    sg_griddep_wait();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const size_t N = (size_t)n;
    const size_t s = 3 * (size_t)(perm ? perm[i] : i);
    for (int c = 0; c < 3; c++) {
        y[c * N + i] = pos[s + c];
        y[(3 + c) * N + i] = vel ? vel[s + c] : 0.0;
    }
}

// pos[perm[k]][c] = y[c][k]: back to the caller's order.
__global__ void soa_to_aos_kernel(const double* __restrict__ y, const int* __restrict__ perm,
                                  double* __restrict__ pos, double* __restrict__ vel, int n) {
    sg_griddep_wait();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const size_t N = (size_t)n;
    const size_t d = 3 * (size_t)(perm ? perm[i] : i);
    for (int c = 0; c < 3; c++) {
        pos[d + c] = y[c * N + i];
        vel[d + c] = y[(3 + c) * N + i];
    }
}

__global__ void gather_kernel(const double* __restrict__ src, const int* __restrict__ perm,
                              double* __restrict__ dst, int n) {
    sg_griddep_wait();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = src[perm ? perm[i] : i];
}

// Per-row-block moment partials: sum x, x^2 per axis, v^2 per axis, m(vx^2+vy^2), m vz^2.
__global__ void __launch_bounds__(SG_ROWS) moments_kernel(DpArgs a, const double* __restrict__ mass,
                                                          double* __restrict__ out) {
    sg_griddep_wait();
    __shared__ double red[11][SG_ROWS / 32];
    const SgRowBlock rb = a.rows[blockIdx.x];
    const int li = threadIdx.x;
    const size_t N = (size_t)a.n;
    double v[11];
    for (int q = 0; q < 11; q++) v[q] = 0.0;
    if (li < rb.n) {
        const int i = rb.i0 + li;
        for (int c = 0; c < 3; c++) {
            const double x = a.y[c * N + i], u = a.y[(3 + c) * N + i];
            v[c] = x;
            v[3 + c] = x * x;
            v[6 + c] = u * u;
        }
        v[9] = mass[i] * (v[6] + v[7]);
        v[10] = mass[i] * v[8];
    }
    for (int q = 0; q < 11; q++) {
        double s = v[q];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if ((li & 31) == 0) red[q][li >> 5] = s;
    }
    __syncthreads();
    if (li < 11) {
        double s = 0.0;
        for (int w = 0; w < SG_ROWS / 32; w++) s += red[li][w];
        out[(size_t)blockIdx.x * 11 + li] = s;
    }
}

}  // namespace

// ---- host-side launchers (called from capi.cu) ------------------------------------

cudaError_t sg_dp_stage(const SgDpArgs& a, int stage, int n_rows, cudaStream_t st) {
    if (n_rows <= 0) return cudaSuccess;
    switch (stage) {
        case 1: sg_launch(dp_stage_kernel<1>, n_rows, SG_ROWS, 0, st, a); break;
        case 2: sg_launch(dp_stage_kernel<2>, n_rows, SG_ROWS, 0, st, a); break;
        case 3: sg_launch(dp_stage_kernel<3>, n_rows, SG_ROWS, 0, st, a); break;
        case 4: sg_launch(dp_stage_kernel<4>, n_rows, SG_ROWS, 0, st, a); break;
        case 5: sg_launch(dp_stage_kernel<5>, n_rows, SG_ROWS, 0, st, a); break;
        case 6: sg_launch(dp_stage_kernel<6>, n_rows, SG_ROWS, 0, st, a); break;
        case 7: sg_launch(dp_stage_kernel<7>, n_rows, SG_ROWS, 0, st, a); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t sg_ck_stage(const SgDpArgs& a, int stage, int n_rows, cudaStream_t st) {
    if (n_rows <= 0) return cudaSuccess;
    switch (stage) {
        case 1: sg_launch(ck_stage_kernel<1>, n_rows, SG_ROWS, 0, st, a); break;
        case 2: sg_launch(ck_stage_kernel<2>, n_rows, SG_ROWS, 0, st, a); break;
        case 3: sg_launch(ck_stage_kernel<3>, n_rows, SG_ROWS, 0, st, a); break;
        case 4: sg_launch(ck_stage_kernel<4>, n_rows, SG_ROWS, 0, st, a); break;
        case 5: sg_launch(ck_stage_kernel<5>, n_rows, SG_ROWS, 0, st, a); break;
        case 6: sg_launch(ck_stage_kernel<6>, n_rows, SG_ROWS, 0, st, a); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t sg_gear_stage(const SgDpArgs& a, int phase, int n_rows, cudaStream_t st) {
    if (n_rows <= 0) return cudaSuccess;
    if (phase == 0)
        sg_launch(gear_kernel<0>, n_rows, SG_ROWS, 0, st, a);
    else
        sg_launch(gear_kernel<1>, n_rows, SG_ROWS, 0, st, a);
    return cudaGetLastError();
}

cudaError_t sg_gear_init(const SgDpArgs& a, const int* perm, int n_rows, cudaStream_t st) {
    if (n_rows <= 0) return cudaSuccess;
    sg_launch(gear_init_kernel, n_rows, SG_ROWS, 0, st, a, perm);
    return cudaGetLastError();
}

cudaError_t sg_dp_control(SgCloud* clouds, SgCtrl* ctrl, const double* err_part,
                          const double* y, int n_clouds, const int* flags,
                          const SgOp* ops, cudaStream_t st) {
    sg_launch(dp_control_kernel, (n_clouds + 127) / 128, 128, 0, st, clouds, ctrl, err_part, y, n_clouds,
                                                              flags, ops);
    return cudaGetLastError();
}

cudaError_t sg_clear_hold(SgCtrl* ctrl, int n_clouds, cudaStream_t st) {
    sg_launch(clear_hold_kernel, (n_clouds + 127) / 128, 128, 0, st, ctrl, n_clouds);
    return cudaGetLastError();
}

cudaError_t sg_dp_commit(const SgDpArgs& a, int n_rows, cudaStream_t st) {
    sg_launch(dp_commit_kernel, n_rows, SG_ROWS, 0, st, a);
    return cudaGetLastError();
}

cudaError_t sg_coords_from_state(const SgDpArgs& a, const double* q, int n_rows, cudaStream_t st) {
    sg_launch(coords_from_state_kernel, n_rows, SG_ROWS, 0, st, a, q);
    return cudaGetLastError();
}

cudaError_t sg_force_finish(const SgDpArgs& a, double t, int with_field, const int* perm,
                            double* out, int n_rows, cudaStream_t st) {
    sg_launch(force_finish_kernel, n_rows, SG_ROWS, 0, st, a, t, with_field, perm, out);
    return cudaGetLastError();
}

cudaError_t sg_aos_to_soa(const double* pos, const double* vel, const int* perm, double* y, int n,
                          cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    sg_launch(aos_to_soa_kernel, (n + 255) / 256, 256, 0, st, pos, vel, perm, y, n);
    return cudaGetLastError();
}

cudaError_t sg_soa_to_aos(const double* y, const int* perm, double* pos, double* vel, int n,
                          cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    sg_launch(soa_to_aos_kernel, (n + 255) / 256, 256, 0, st, y, perm, pos, vel, n);
    return cudaGetLastError();
}

cudaError_t sg_gather(const double* src, const int* perm, double* dst, int n, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    sg_launch(gather_kernel, (n + 255) / 256, 256, 0, st, src, perm, dst, n);
    return cudaGetLastError();
}

cudaError_t sg_moments(const SgDpArgs& a, const double* mass, double* out, int n_rows,
                       cudaStream_t st) {
    sg_launch(moments_kernel, n_rows, SG_ROWS, 0, st, a, mass, out);
    return cudaGetLastError();
}

