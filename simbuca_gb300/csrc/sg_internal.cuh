// sg_internal.cuh -- shared device-side definitions of libsimgb (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <utility>

#include "../../include/simgb.h"

// ---- constants of the reference (bin/globals.h:4-16) -------------------------
#define SG_PI 3.14159265358979323
#define SG_EL_CHARGE 1.60217733e-19
#define SG_KE 8.987551787E9
#define SG_KB 1.3806504E-23

// ---- programmatic dependent launch -----------------------------------------------
// Kernels of the graph-captured attempt are launched with programmatic stream
// serialization: the next kernel's grid is set up while the previous one drains, and
// every kernel waits (griddepcontrol.wait) for its predecessor's completion and memory
// before its first global access -- a no-op when it was launched without the attribute.
// g_sg_pdl (capi.cu) is set only while the untimed attempt graph is captured (opt-in,
// SIMGB_PDL=1), whose only non-kernel node (the fix-up list reset) is followed by a
// plain launch.
extern int g_sg_pdl;

__device__ __forceinline__ void sg_griddep_wait() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    // the next kernel may be scheduled once every block of this one has started; its
    // blocks then wait above for this grid's completion
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

template <typename... KArgs, typename... Args>
inline cudaError_t sg_launch(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem,
                             cudaStream_t st, Args&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = g_sg_pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

// ---- launch geometry ---------------------------------------------------------
// FP32c Coulomb: 128 threads x 4 ions per thread = 512 i-ions per block; j-tiles of
// 128 ions (2 KB of float4 hi + 2 KB of float4 lo) streamed by TMA bulk copies.
#define SG_C32_THREADS 128
#define SG_C32_IPT 4
#define SG_C32_IB (SG_C32_THREADS * SG_C32_IPT)
#define SG_TILE 128
#define SG_STAGES 4
// FP64 Coulomb: 128 threads x 2 ions per thread.
#define SG_C64_THREADS 128
#define SG_C64_IPT 2
#define SG_C64_IB (SG_C64_THREADS * SG_C64_IPT)
// Per-cloud ion ranges are padded to a multiple of this (ghost ions carry q = 0).
#define SG_PAD 32
// O(N) kernels: ions per block.
#define SG_ROWS 256
// Arrays of a Coulomb partial-sum slot: x, y, z, and the FP32c conditioning estimates
// of the near tiles and of the far tiles (sums of squared 32-ion partial sums).
#define SG_PART_ARRAYS 5
// FP32c fix-up kernel: work units per listed ion, and the listed ions that get them
#define SG_FIX_UNITS 16
#define SG_FIX_CHUNKED_CAP 4096

// Bounded device waits: a wait gives up after this many nanoseconds of
// %globaltimer and raises SG_TIMEOUT in the context's error word.
#define SG_WAIT_NS 1000000000ull

// The context's device flag words (Problem::flags): the error word the kernels raise,
// the hold-on-accept word, the fix-up list count, and the wait test: with
// flags[SG_FLAG_WAIT_TILE] = t + 1, every block of the FP32c Coulomb kernels waits, at
// j-tile t, on a barrier that nothing arrives at until flags[SG_FLAG_WAIT_US]
// microseconds have passed, and takes the timeout path (sg_set_wait_test).
#define SG_FLAG_ERR 0
#define SG_FLAG_HOLD 1
#define SG_FLAG_WAIT_TILE 4
#define SG_FLAG_WAIT_US 5
#define SG_NFLAGS 8

// One unit of Coulomb work: i-ions [i0, i0+ni) (padded indices) of cloud `cloud`
// against j-ions [j0, j0+nj) of the same cloud; the partial sums go to slot `slot`.
struct SgWorkItem {
    int32_t cloud;
    int32_t i0, ni;
    int32_t j0, nj;
    int32_t slot;
    int32_t pad0, pad1;
};

// Rows of one cloud handled by one block of the O(N) kernels.
struct SgRowBlock {
    int32_t cloud;
    int32_t i0;     // first ion (unpadded global index)
    int32_t n;      // ions in this block (<= SG_ROWS)
    int32_t pad;
};

// Device description of a cloud.
struct SgCloud {
    int32_t off;     // first ion, unpadded global index
    int32_t n;       // ions
    int32_t poff;    // first ion, padded global index
    int32_t npad;    // padded ions (multiple of SG_PAD)
    int32_t nslots;  // Coulomb partial-sum slots (j-chunks) of this cloud
    int32_t rb0, nrb;  // row blocks [rb0, rb0+nrb)
    int32_t ion0;      // device index of the caller's first ion of the cloud (k-d order
                       // moves it; the step-size underflow test reads its x)
    double cx, cy, cz;   // centre of the FP32 frame (m)
    double L, invL;      // scale of the FP32 frame (m)
    double vref;         // RMS velocity per axis at upload (m/s), proposer features
    int32_t tile0;       // first entry of this cloud in the 128-ion tile bounding boxes
    float dfar;          // FP32c: tiles farther apart than this (frame units) use hi parts only
    float wc;            // FP32c close-pair threshold on 1/r^3 (frame units)
    float kfar2;         // FP32c: far fix-up when s2f > kfar2 |P|^2 (k-d ordered shapes)
    sg_field_params fp;
    long long rec_off;   // recorder: first double of this cloud's record ring
    int32_t nsel;        // recorder: ions kept per record (every stride-th in caller order)
    int32_t rec_len;     // recorder: doubles per record
    // FP32c charges: the FP32 coordinate array holds q / qscale; with all ions of the cloud
    // at one charge q, qscale = q (quniform = 1) and the normalized charges are 1
    double qscale;
    int32_t quniform, pad4;
};

// Per-cloud Dormand-Prince controller (the scalar part of _ode_vars, bin/ode.h:58-97).
struct SgCtrl {
    double t, h, hnext, errold, err, t_end, rtol, atol, h_last;
    // hold: bit 0 = one step per call taken, bit 1 = record ring full; either stops the
    // cloud's kernels until the host clears it
    int32_t reject, adaptive, max_rejects, status, done, accepted, rejects_here, hold;
    int32_t method, pad2;  // 5 Dormand-Prince, 4 Cash-Karp, 1 Gear
    double hf[4];          // Gear: h^2/2, h^3/6, h^4/24, h^5/120 of the initial step
    long long steps, rejects, force_evals, coulomb_evals;
    // recorder: the reference's print rule (bin/ion_fly.cpp:103-108), record due now
    // when (t - t_print0) > print_interval * n_print after an accepted step
    double print_interval, t_print0;
    long long n_print, rec_count, rec_drained;
    int32_t print_due, rec_slot, rec_cap, pad3;
    // operation sequence (sg_batch_set_operations): current operation, its start, the
    // ramp's starting Vrf/Vdc, the cloud's trap terms, dissociation to apply (index+1)
    int32_t op_index, n_ops, trap_bits, dis_due;
    double t_op_start, old_vrf, old_vdc;
    double beta;  // PI term of error_succes (0: the reference's I-controller)
};

// error_succes and the retry bookkeeping of step() (bin/ode.cpp:426-494) for one attempt
// of one cloud with error norm err: returns 1 if the attempt is accepted.  A non-finite
// norm stops the cloud (SG_NONFINITE); a reject shrinks h and checks the underflow
// |h| <= |pos[0][0]| eps against *x0 (the caller's first ion) and the reject budget.
// Gear (method 1) and fixed-step runs accept every attempt.  beta = 0 is the
// reference's I-controller: pow(errold, 0) = 1 exactly.
__device__ inline int sg_error_succes(SgCtrl& cs, double err, const double* x0) {
    if (!isfinite(err)) {
        cs.status = SG_NONFINITE;
        cs.done = 1;
        return 0;
    }
    if (!cs.adaptive || cs.method == 1) return 1;  // step() turns control off for Gear
    const double beta = cs.beta, alpha = 0.2 - beta * 0.75, safe = 0.9, minscale = 0.2,
                 maxscale = 10.0;
    if (err <= 1.0) {
        double scale;
        if (err == 0.0)
            scale = maxscale;
        else {
            scale = safe * pow(err, -alpha) * pow(cs.errold, beta);
            if (scale < minscale) scale = minscale;
            if (scale > maxscale) scale = maxscale;
        }
        cs.hnext = cs.reject ? cs.h * ((1.0 < scale) ? 1.0 : scale) : cs.h * scale;
        cs.errold = (err < 1.0e-4) ? 1.0e-4 : err;
        cs.reject = 0;
        return 1;
    }
    double scale = safe * pow(err, -alpha);
    scale = (scale < minscale) ? minscale : scale;
    cs.h *= scale;
    cs.reject = 1;
    cs.rejects++;
    cs.rejects_here++;
    if (fabs(cs.h) <= fabs(*x0) * 2.220446049250313e-16) {
        cs.status = SG_H_UNDERFLOW;
        cs.done = 1;
    } else if (cs.max_rejects > 0 && cs.rejects_here >= cs.max_rejects) {
        cs.status = SG_TOO_MANY_REJECTS;
        cs.done = 1;
    }
    return 0;
}

// One operation of the sequence (sg_operation plus the row of its dissociation table).
struct SgOp {
    int32_t kind, print_after;
    double duration, print_time, timestep, new_vrf, new_vdc, e_kick;
    int32_t dis_index, reactant, product, pad;
    double fraction, product_mass;
};

// Starts operation `from` of the sequence at the cloud's current time: the settings of
// operation::launch (bin/operation.cpp:33-77) and move_particles' end time; operations
// that take no time end at once (a dissociation applies its table).  Past the last
// operation the cloud is done.  Returns 1 if an ended operation asked for a print.
__host__ __device__ inline int sg_start_ops(SgCtrl& cs, sg_field_params& fp, const SgOp* ops,
                                            int from) {
    int print = 0;
    for (int k = from; k < cs.n_ops; k++) {
        const SgOp& op = ops[k];
        cs.op_index = k;
        if (op.kind == SG_OP_DISSOCIATION) {
            cs.dis_due = op.dis_index + 1;
            continue;
        }
        if (op.print_time > 0.0) cs.print_interval = op.print_time;
        if (op.timestep != 0.0) cs.h = cs.hnext = op.print_time;
        const bool trap = op.kind == SG_OP_NORMAL || op.kind == SG_OP_TRAP_RAMP;
        fp.flags = trap ? (fp.flags | cs.trap_bits) : (fp.flags & ~cs.trap_bits);
        if (op.kind == SG_OP_TOF) {
            fp.flags |= SG_F_TOF;
            fp.E_kick = op.e_kick;
        } else {
            fp.flags &= ~SG_F_TOF;
        }
        cs.old_vrf = fp.Vrf;
        cs.old_vdc = fp.Vdc;
        cs.t_op_start = cs.t;
        cs.t_end = cs.t + op.duration;
        if (cs.t < cs.t_end) return print;
        print |= op.print_after;
    }
    cs.op_index = cs.n_ops;
    cs.done = 1;
    return print;
}

// ---- learned step-size proposer (proposer.cu) -------------------------------------
#define SG_MLP_IN 16
#define SG_MLP_H 64
#define SG_MLP_W1 0
#define SG_MLP_B1 (SG_MLP_W1 + SG_MLP_H * SG_MLP_IN)
#define SG_MLP_W2 (SG_MLP_B1 + SG_MLP_H)
#define SG_MLP_B2 (SG_MLP_W2 + SG_MLP_H * SG_MLP_H)
#define SG_MLP_W3 (SG_MLP_B2 + SG_MLP_H)
#define SG_MLP_B3 (SG_MLP_W3 + SG_MLP_H)
#define SG_MLP_NP (SG_MLP_B3 + 1)

// Per-cloud proposer state: features of the current step start and step history.
struct SgProposerState {
    float feat[SG_MLP_IN];
    double h_prev;          // accepted step size before the last accepted step
    int32_t init;           // features computed since the last upload
    int32_t logged;         // log records written
    int32_t rejects_in_step;
    int32_t pad;
};

// ---- field terms ---------------------------------------------------------------
// Paul/TOF follow bin/force.cpp:40-44,70-80; the Penning trap, the RF excitations and
// friction follow the formulas of include/simgb.h.  The factors that depend only on
// the cloud and the time (divisions by trap dimensions, the drive cosines) are one
// SgFieldCoef, computed once per block by the stage kernels: GB300 runs FP64 at a small
// fraction of its FP32 rate, and a division plus a cosine per ion and stage made the
// O(N) kernels FP64-bound.  The per-ion arithmetic is unchanged.
struct SgFieldCoef {
    double paul_x, paul_y, paul_z;  // (kVdc/z0^2 -+ Vrf cos(w t)/r0^2), -2 kVdc/z0^2
    double kp;                      // V0 / (2 d0^2)
    double gq;                      // quadrupole factor at t (0 when off)
    double gd;                      // dipole field at t (0 when off)
};

// Products and sums below are rounded one operation at a time, in the order of the
// oracle's restatement (compiled without contraction), so that the FP64 path's field
// terms are the oracle's to the last bit; only the cosines may differ by an ulp.
__device__ __forceinline__ SgFieldCoef sg_field_coef(const sg_field_params& fp, double t) {
    SgFieldCoef k;
    const uint32_t f = fp.flags;
    k.paul_x = k.paul_y = k.paul_z = 0.0;
    k.kp = k.gq = k.gd = 0.0;
    if (f & SG_F_PAUL) {
        const double kVdc = fp.kappa * fp.Vdc;
        const double r02 = fp.r0 * fp.r0, z02 = fp.z0 * fp.z0;
        const double c = fp.Vrf * cos(fp.freq_rf * 2 * SG_PI * t) / r02;
        k.paul_x = kVdc / z02 - c;
        k.paul_y = kVdc / z02 + c;
        k.paul_z = -2.0 * kVdc / z02;
    }
    if (f & SG_F_PENNING) k.kp = fp.V0 / (2.0 * fp.d0 * fp.d0);
    if ((f & SG_F_QUAD) && t >= fp.tq_on && t < fp.tq_off)
        k.gq = __dmul_rn(2.0 * fp.Uq / (fp.r_el * fp.r_el),
                         cos(__dadd_rn(__dmul_rn(2.0 * SG_PI * fp.nu_q, t), fp.phi_q)));
    if ((f & SG_F_DIPOLE) && t >= fp.td_on && t < fp.td_off)
        k.gd = __dmul_rn(fp.Ud / fp.r_el,
                         cos(__dadd_rn(__dmul_rn(2.0 * SG_PI * fp.nu_d, t), fp.phi_d)));
    return k;
}

__device__ __forceinline__ void sg_field_apply(const sg_field_params& fp, const SgFieldCoef& k,
                                               double qm, double x, double y, double z,
                                               double vx, double vy, double vz, double& ax,
                                               double& ay, double& az) {
    const uint32_t f = fp.flags;
    ax = 0.0;
    ay = 0.0;
    az = 0.0;
    if (f & SG_F_PAUL) {
        ax = __dmul_rn(__dmul_rn(qm, k.paul_x), x);
        ay = __dmul_rn(__dmul_rn(qm, k.paul_y), y);
        az = __dmul_rn(__dmul_rn(qm, k.paul_z), z);
    }
    if (f & SG_F_TOF) ax = __dadd_rn(ax, __dmul_rn(qm, fp.E_kick));
    if (f & (SG_F_PENNING | SG_F_QUAD | SG_F_DIPOLE)) {
        double ex = 0.0, ey = 0.0, ez = 0.0;
        if (f & SG_F_PENNING) {
            ex = __dadd_rn(__dmul_rn(k.kp, x), __dmul_rn(fp.B, vy));
            ey = __dsub_rn(__dmul_rn(k.kp, y), __dmul_rn(fp.B, vx));
            ez = __dmul_rn(__dmul_rn(-2.0, k.kp), z);
        }
        ex = __dadd_rn(ex, __dadd_rn(__dmul_rn(k.gq, y), k.gd));
        ey = __dadd_rn(ey, __dmul_rn(k.gq, x));
        ax = __dadd_rn(ax, __dmul_rn(qm, ex));
        ay = __dadd_rn(ay, __dmul_rn(qm, ey));
        az = __dadd_rn(az, __dmul_rn(qm, ez));
    }
    if (f & SG_F_FRICTION) {
        ax = __dsub_rn(ax, __dmul_rn(fp.delta, vx));
        ay = __dsub_rn(ay, __dmul_rn(fp.delta, vy));
        az = __dsub_rn(az, __dmul_rn(fp.delta, vz));
    }
}

__device__ __forceinline__ void sg_field_accel(const sg_field_params& fp, double t, double qm,
                                               double x, double y, double z, double vx,
                                               double vy, double vz, double& ax, double& ay,
                                               double& az) {
    sg_field_apply(fp, sg_field_coef(fp, t), qm, x, y, z, vx, vy, vz, ax, ay, az);
}

// The block's field coefficients at time t, computed by thread 0 (every thread of the
// block must call this: it synchronises the block).
__device__ __forceinline__ SgFieldCoef sg_field_coef_block(const sg_field_params& fp, double t) {
    __shared__ SgFieldCoef sk;
    if (threadIdx.x == 0) sk = sg_field_coef(fp, t);
    __syncthreads();
    return sk;
}

// ---- Dormand-Prince 5(4) tableau (bin/ode.cpp:76-86) ------------------------------
#define DP_C2 (1.0 / 5.0)
#define DP_C3 (3.0 / 10.0)
#define DP_C4 (4.0 / 5.0)
#define DP_C5 (8.0 / 9.0)

// Arguments of the O(N) Dormand-Prince kernels (dp45.cu).
struct SgDpArgs {
    const SgRowBlock* rows;
    const SgCloud* clouds;
    SgCtrl* ctrl;
    double* y;            // [6][N]
    double* ys;           // [6][N]
    double* k;            // [7][6][N]
    const double* coulS;  // [3][N] Coulomb sum of the stage being finished
    double* coul1;        // [3][N]
    double* coul7;        // [3][N]
    const double* kq;     // [N]
    const double* qm;     // [N]
    double* c64;          // [4][Npad]
    float* c32;           // [7][Npad]
    double* err_part;     // [rows]
    float* bbox;          // [tiles][8] frame-unit bounds of each 128-ion tile (FP32c)
    int n;                // ions (unpadded)
    int npad;             // padded ions
    int fp32c;            // write the FP32 frame coordinates
};

// ---- fused small-cloud attempts (fused.cu) -----------------------------------------
// One thread-block cluster per cloud runs whole Dormand-Prince attempts (FP32c, no
// recorder, operations or proposer) for clouds of at most SG_FUSED_MAX_IONS ions, and
// at most SG_FUSED_THREADS ions per CTA of the cluster.
#define SG_FUSED_THREADS 512
#define SG_FUSED_MAX_CTAS 16
#define SG_FUSED_MAX_IONS 2048
// Clouds the fused path takes by default (sg_set_fused mode 1): measured on GB300 it
// needs ~180 us per attempt at 256 ions against ~245 us for the tiled kernels, breaks
// even near 1,000 ions and loses beyond; mode 2 takes it up to SG_FUSED_MAX_IONS.
#define SG_FUSED_AUTO_IONS 512
struct SgFusedArgs {
    const SgCloud* clouds;
    SgCtrl* ctrl;
    double *y, *ys, *k, *coul1, *coul7, *coulS;
    const double *kq, *qm;
    double* c64;
    float* c32;
    double* errp;    // [clouds][SG_FUSED_MAX_CTAS] error partials of an attempt
    int* flags;      // the context's flag words (error word, hold on accept)
    float* risk;     // in-run force check inputs (null: not written)
    int* ran;
    int n, npad, n_clouds;
    int max_attempts;  // attempts per launch at most
};
// The cluster size the fused kernel can be launched with on this device for clouds of
// up to max_npad padded ions (16, 8 or 4), or 0 if none.
int sg_fused_cluster_size(int max_npad);
cudaError_t sg_fused_attempts(const SgFusedArgs& f, int cluster, int max_npad, cudaStream_t st);

// ---- device-side observables (observe.cu) -------------------------------------------
// A record of a cloud: [0] t, then per species s < n_species the PrintCloud statistics
// (bin/ioncloud.cpp:148-183) x0 y0 z0 x1 y1 z1 (m) energy (eV) n_s n, then the state
// x y z vx vy vz, energy (eV) and species of every stride-th ion in the caller's order.
#define SG_MAX_SPECIES 8
#define SG_STAT_LEN 9
#define SG_ION_LEN 8
struct SgRecArgs {
    const SgRowBlock* rows;
    const SgCloud* clouds;
    const SgCtrl* ctrl;
    const double* y;     // [6][N]
    const double* mass;  // [N] print mass (kg), device order
    int* spec;           // [N] species, device order
    const int* dis_spec;     // dissociation tables [tables][N] in the caller's order
    const double* dis_mass;
    const int* perm;     // device position -> caller's ion index
    double* ring;
    int n, n_species, stride;
};
cudaError_t sg_record(const SgRecArgs& r, int n_rows, int n_clouds, cudaStream_t st);
// species and print masses of a dissociation that the control kernel applied
cudaError_t sg_dissociate(const SgRecArgs& r, double* mass, int* spec0, double* mass0, int n_rows,
                          cudaStream_t st);
cudaError_t sg_record_now(SgCtrl* ctrl, int n_clouds, cudaStream_t st);
cudaError_t sg_gather_int(const int* src, const int* perm, int* dst, int n, cudaStream_t st);

// ---- launchers implemented in the .cu files ------------------------------------
cudaError_t sg_dp_stage(const SgDpArgs& a, int stage, int n_rows, cudaStream_t st);
cudaError_t sg_ck_stage(const SgDpArgs& a, int stage, int n_rows, cudaStream_t st);
// Gear: phase 0 predicts, phase 1 corrects; sg_gear_init seeds the Gear state in k
cudaError_t sg_gear_stage(const SgDpArgs& a, int phase, int n_rows, cudaStream_t st);
cudaError_t sg_gear_init(const SgDpArgs& a, const int* perm, int n_rows, cudaStream_t st);
cudaError_t sg_dp_control(SgCloud* clouds, SgCtrl* ctrl, const double* err_part,
                          const double* y, int n_clouds, const int* flags,
                          const SgOp* ops, cudaStream_t st);
cudaError_t sg_clear_hold(SgCtrl* ctrl, int n_clouds, cudaStream_t st);
int sg_probe_iters(int which);
cudaError_t sg_dp_commit(const SgDpArgs& a, int n_rows, cudaStream_t st);
cudaError_t sg_coords_from_state(const SgDpArgs& a, const double* q, int n_rows, cudaStream_t st);
cudaError_t sg_force_finish(const SgDpArgs& a, double t, int with_field, const int* perm,
                            double* out, int n_rows, cudaStream_t st);
// layout changes with the ion order perm (sorted position -> caller's index)
cudaError_t sg_aos_to_soa(const double* pos, const double* vel, const int* perm, double* y, int n,
                          cudaStream_t st);
cudaError_t sg_soa_to_aos(const double* y, const int* perm, double* pos, double* vel, int n,
                          cudaStream_t st);
cudaError_t sg_gather(const double* src, const int* perm, double* dst, int n, cudaStream_t st);
cudaError_t sg_moments(const SgDpArgs& a, const double* mass, double* out, int n_rows,
                       cudaStream_t st);
cudaError_t sg_cunbody_launch(const double* xj, const double* mj, const double* xi, double eps2,
                              double* ai, int ni, int nj, cudaStream_t st);
cudaError_t sg_probe_launch(int which, int blocks, int threads, float* sink, cudaStream_t st);
cudaError_t sg_proposer_launch(const SgCloud* clouds, SgCtrl* ctrl, const double* mom,
                               SgProposerState* pst, const void* wbf, float* log_feat,
                               double* log_num, int log_cap, int use_mlp, double safety,
                               int n_clouds, cudaStream_t st);
cudaError_t sg_mlp_grad_launch(const void* wbf, const float* X, const float* Y, const int* idx,
                               int B, float* gpart, float* lpart, int nb, float* grad, float* loss,
                               cudaStream_t st);
cudaError_t sg_mlp_adam_launch(float* wm, void* wbf, float* m1, float* m2, const float* grad,
                               float lr, int step, cudaStream_t st);
cudaError_t sg_mlp_to_bf16_launch(const float* wm, void* wbf, cudaStream_t st);
cudaError_t sg_mlp_forward_launch(const void* wbf, const float* X, int n, float* out,
                                  cudaStream_t st);

struct SgCoulombArgs {
    const float* c32;        // [7][Npad] frame coords hi x,y,z, charge, lo x,y,z (FP32c)
    const double* c64;       // [4][Npad] SI coords x,y,z and charge (FP64, close pairs)
    const SgWorkItem* items;
    int n_items;
    const SgCloud* clouds;
    const SgCtrl* ctrl;      // may be null (stand-alone calls)
    double* part;            // [slots][SG_PART_ARRAYS][Npad]: x, y, z sums, FP32c s2, s2f
    int npad_total;
    int* errword;
    int variant;             // FP32c launch shape (sg_coulomb_fp32c_ib)
    const float* bbox;       // [tiles][8] tile bounds (sorted variant)
    // FP32c conditioning fix-up work list, filled by the reduction: [0] count, then
    // per flagged ion its global index and cloud (ints) and |P| in frame units
    int* fix_list;
    // per listed ion and work unit its correction, and the count of finished units
    double* fix_part;
    int* fix_done;
    // k-d ordered shapes: accumulate the far tiles' conditioning estimate s2f in this
    // call (it costs the kernel ~4 %); otherwise the slots keep the last call's values
    int far_estimate;
    // in-run force check (check.cu), FP32c sums of an attempt only: the reduction writes
    // each ion's far and near ratios sqrt(s2f)/|P|, sqrt(s2)/|P| (-1 when the ion is
    // fixed up) to risk[2][N] and marks its cloud in ran[]; chk holds each cloud's
    // measured far fix-up threshold
    float* risk = nullptr;
    int* ran = nullptr;
    const struct SgCheck* chk = nullptr;
};

// ---- in-run force check (check.cu) ---------------------------------------------
#define SG_CHECK_PROBES 8
struct SgCheck {
    double max_err;    // largest per-ion relative error over every check
    double last_err;   // largest of the last check
    double c_far;      // largest err / (sqrt(s2f)/|P|) of the far-ranked probes
    double max_kind[3];  // largest error of the far-ranked, near-ranked, random probes
    long long checks, probes, breaches;  // breaches: probes above 1e-6
    float kfar2;       // measured far fix-up threshold (kfar^2); +inf until measured
    int32_t pad;
    int32_t ion[SG_CHECK_PROBES];
    float rf[SG_CHECK_PROBES], rn[SG_CHECK_PROBES];
    double err[SG_CHECK_PROBES];
    // the probe with the largest error over every check: its error, its ratios (-1:
    // flagged, fixed up), its ion (device order) and kind (0 far, 1 near, 2 random)
    double worst_err;
    float worst_rf, worst_rn;
    int32_t worst_ion, worst_kind;
};
cudaError_t sg_force_check(const SgCloud* clouds, int n_clouds, int* ran, const float* risk,
                           const double* c64, int npad_total, const double* out, int n_total,
                           SgCheck* chk, cudaStream_t st);

#define SG_C32_VARIANTS 17
// variant 4: ions in k-d tree order, far tile pairs from the high parts only
#define SG_C32_SORTED 4
#define SG_C32_SORTED_LEAF 7
// launch shapes that keep ions in k-d tree order
__host__ __device__ inline bool sg_variant_sorted(int v) {
    return v == SG_C32_SORTED || (v >= SG_C32_SORTED_LEAF && v <= 9) || (v >= 12 && v <= 16);
}
int sg_coulomb_fp32c_ib(int variant);
cudaError_t sg_launch_coulomb_fp32c(const SgCoulombArgs& a, cudaStream_t s);
cudaError_t sg_launch_coulomb_fp64(const SgCoulombArgs& a, cudaStream_t s);
cudaError_t sg_launch_coulomb_reduce(const SgCoulombArgs& a, const SgRowBlock* rows, int n_rows,
                                     int fp32c, double* out, int n_total, int* counters,
                                     cudaStream_t s);
