/*
 * simgb.h -- C ABI of libsimgb, the GB300 (sm_103a) integration hot path of the
 * Simbuca ion-cloud simulator: direct-sum Coulomb interaction, per-ion trap field
 * terms, and the Dormand-Prince 5(4) stage / error-norm / step-control loop.
 *
 * Conventions
 *  - Every entry point returns an int status (SG_OK on success); nothing throws or
 *    calls exit() across this boundary.  sg_status_string() names a status.
 *  - Host buffers are owned by the caller.  Device buffers are owned by the
 *    context and freed by sg_destroy().
 *  - Host position/velocity buffers use the reference's layout: double[n][3]
 *    (array of structures, metres and metres/second), as IonCloud::pos/vel
 *    (bin/ioncloud.h:27-30).  Accelerations come back as double[n][3] in m/s^2,
 *    like _force_vars::derivs (bin/ode.h:45, bin/force.h:7).
 *  - One context per host thread; all work of a context is ordered on the
 *    context's CUDA stream.
 *
 * Physical constants are the reference's (bin/globals.h:4-16).
 */
#ifndef SIMGB_H
#define SIMGB_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------------- */
enum {
    SG_OK = 0,
    SG_BAD_ARG = 1,          /* invalid argument or size                               */
    SG_CUDA_ERR = 2,         /* a CUDA runtime call failed (see sg_last_cuda_error)    */
    SG_H_UNDERFLOW = 3,      /* step size underflow; the reference throws
                                "stepsize underflow created" (bin/ode.cpp:482-483)     */
    SG_NONFINITE = 4,        /* non-finite error norm or state                         */
    SG_TIMEOUT = 5,          /* a bounded device-side wait ran out                     */
    SG_NO_DEVICE = 6,        /* no usable CUDA device                                  */
    SG_TOO_MANY_REJECTS = 7, /* a step exceeded its reject budget                      */
    SG_NOT_READY = 8,        /* call order violated (e.g. step before upload)          */
    SG_TOO_LARGE = 9,        /* size beyond a fixed capacity                           */
    SG_IO_ERR = 10           /* a file could not be opened, read, written or parsed    */
};

/* ---- arithmetic of the Coulomb sum ----------------------------------------- */
enum {
    SG_PREC_FP64 = 0,   /* plain form: every operation in FP64                          */
    SG_PREC_FP32C = 1   /* FP32 pair terms on cloud-centre-relative float-float
                           coordinates, Kahan-compensated per-ion accumulation across
                           j-tiles, and FP64 evaluation of close pairs                  */
};

/* ---- field terms (bit flags of sg_field_params.flags) ---------------------- */
enum {
    SG_F_COULOMB  = 1u << 0,  /* ion-ion Coulomb sum (force.cpp:84-177)               */
    SG_F_PAUL     = 1u << 1,  /* ideal RF+DC quadrupole (force.cpp:70-75)             */
    SG_F_TOF      = 1u << 2,  /* constant x kick E_kick (force.cpp:77-80)             */
    SG_F_PENNING  = 1u << 3,  /* ideal Penning trap: quadrupole V0/d0 + B along z     */
    SG_F_QUAD     = 1u << 4,  /* azimuthal quadrupole RF excitation                   */
    SG_F_DIPOLE   = 1u << 5,  /* uniform dipole RF excitation along x                 */
    SG_F_FRICTION = 1u << 6,  /* buffer-gas friction a = -delta v                     */
    SG_F_FROZEN_T = 1u << 7   /* evaluate every stage at the step-start time, as the
                                 reference does (force.cpp:36 reads lifetime); without
                                 it stage s is evaluated at t + c_s h                 */
};

/* Per-cloud field description.  SI units.  Terms without a flag are ignored.
 *  Paul (reference _trap_param, bin/trapparameters.h:6-27):
 *    a_x += q e/m (kappa Vdc/z0^2 - Vrf cos(2 pi freq_rf t)/r0^2) x
 *    a_y += q e/m (kappa Vdc/z0^2 + Vrf cos(2 pi freq_rf t)/r0^2) y
 *    a_z += q e/m (-2 kappa Vdc/z0^2) z ;   TOF: a_x += q e/m E_kick
 *  Penning (no reference implementation; potential V0/(2 d0^2) (z^2 - (x^2+y^2)/2)):
 *    a += q e/m ( V0/(2 d0^2) x + B v_y,  V0/(2 d0^2) y - B v_x,  -V0/d0^2 z )
 *  Quadrupole excitation, on for tq_on <= t < tq_off:
 *    a_x += q e/m (2 Uq/r_el^2) cos(2 pi nu_q t + phi_q) y
 *    a_y += q e/m (2 Uq/r_el^2) cos(2 pi nu_q t + phi_q) x
 *  Dipole excitation, on for td_on <= t < td_off:
 *    a_x += q e/m (Ud/r_el) cos(2 pi nu_d t + phi_d)
 *  Friction: a -= delta v.
 *  Coulomb: a_i += coulomb_scale k_e e^2 q_i/m_i sum_{j!=i} q_j (x_i-x_j)/|x_i-x_j|^3.
 */
typedef struct sg_field_params {
    uint32_t flags;
    uint32_t pad0;
    double coulomb_scale;
    /* Paul trap and TOF kick */
    double Vrf, Vdc, kappa, r0, z0, freq_rf, E_kick;
    /* Penning trap */
    double B, V0, d0;
    /* RF excitations */
    double r_el;
    double Uq, nu_q, phi_q, tq_on, tq_off;
    double Ud, nu_d, phi_d, td_on, td_off;
    /* buffer gas */
    double delta;
} sg_field_params;

/* Dormand-Prince controller settings of one cloud (the reference's _ode_vars
 * fields rk_rtol, rk_atol, h, EPS; bin/ode.h:66-83, bin/ode.cpp:515-520). */
typedef struct sg_ode_params {
    double rtol, atol;   /* reference defaults 1e-7 / 1e-7 (ode.cpp:515-516)           */
    double h0;           /* first trial step                                            */
    double t0;           /* cloud lifetime at upload                                    */
    double t_end;        /* the cloud stops advancing once t >= t_end                    */
    int32_t adaptive;    /* 1: step-size control on (ode.cpp:478); 0: fixed step h0     */
    int32_t max_rejects; /* reject budget per step (0 = unlimited)                      */
    int32_t method;      /* Init_ode order (ode.cpp:556-583): 5 Dormand-Prince (0 = 5),
                            4 Cash-Karp, the reference's "RungaKutta4" (ode.cpp:220-345),
                            1 Gear predictor-corrector (ode.cpp:347-424): fixed step h0,
                            adaptive ignored, history restarted by upload and set_state.
                            All clouds of a batch use one method.                      */
    int32_t pad;
    double beta;         /* PI term of error_succes (bin/ode.cpp:431-439): on an accepted
                            step scale = 0.9 err^-(0.2 - 0.75 beta) errold^beta; the
                            reference's build has beta = 0 (the I-controller) and names
                            0.04-0.08 for PI control.  0 reproduces the reference.       */
} sg_ode_params;

/* State of one cloud after a call. */
typedef struct sg_step_info {
    double t;            /* cloud lifetime                                              */
    double h;            /* step size for the next attempt (the reference's odev.h)     */
    double h_last;       /* step size of the last accepted step                         */
    double err;          /* error norm of the last attempt                              */
    double errold;       /* controller memory (ode.cpp:447)                             */
    int64_t steps;       /* accepted steps                                              */
    int64_t rejects;     /* rejected attempts                                           */
    int64_t force_evals; /* force evaluations (7 per attempt, as the reference counts)  */
    int64_t coulomb_evals; /* Coulomb sums actually launched                            */
    int32_t status;      /* SG_OK, SG_H_UNDERFLOW, SG_NONFINITE, SG_TOO_MANY_REJECTS    */
    int32_t done;        /* 1 once t >= t_end                                           */
    int32_t reject;      /* controller flag (ode.cpp:443-454)                           */
    int32_t pad;
} sg_step_info;

typedef struct sg_ctx sg_ctx;

/* ---- context ----------------------------------------------------------------- */
int sg_create(int device, sg_ctx** out);
int sg_destroy(sg_ctx* ctx);
const char* sg_status_string(int status);
int sg_last_cuda_error(sg_ctx* ctx);          /* last cudaError_t seen (0 = none)     */
int sg_sync(sg_ctx* ctx);                     /* wait for the context stream          */
int sg_version(void);

/* ---- stand-alone force calls (host buffers, synchronous) --------------------- */

/* Coulomb accelerations only: acc[i] = kq[i] * sum_{j!=i} q[j] (x_i-x_j)/|x_i-x_j|^3.
 * With kq[i] = coulomb_scale k_e e^2 q_i/m_i this is the CPU sum of the reference
 * (bin/force.cpp:147-174) and the term the GPU backends return (force.cpp:84-105). */
int sg_coulomb_accel(sg_ctx* ctx, int precision, int n, const double* pos,
                     const double* q, const double* kq, double* acc);

/* Complete force() replacement (bin/force.cpp:34-178): field terms of `fp` at time t
 * (stage time; SG_F_FROZEN_T is irrelevant here) plus the Coulomb sum when
 * SG_F_COULOMB is set.  mass in kg, charge in units of e. */
int sg_force(sg_ctx* ctx, int precision, int n, const double* pos, const double* vel,
             const double* mass, const int* charge, double t,
             const sg_field_params* fp, double* acc);

/* Coulomb accelerations without any device allocation (no counterpart in the
 * reference).  For callers that must not call cudaMalloc -- applications that
 * allocate all device memory up front, or plug-ins that only receive device pointers
 * from a host framework's pool.  pos [n][3], q [n], kq [n] and acc [n][3] are DEVICE
 * buffers owned by the caller; the result is the FP64 form of sg_coulomb_accel.  Work
 * is queued on `stream` (a cudaStream_t, NULL = legacy default stream) of the current
 * device and the call returns without waiting.  Scratch lives in a fixed 1.8 MB device
 * array of the library: n <= 8192, else SG_TOO_LARGE.  The array has one address per
 * CUDA context: the first call made in a context looks it up and keeps it under that
 * context's unique id (make that first call before capturing any stream).  n = 0
 * returns SG_OK and queues nothing; a null pointer gives SG_BAD_ARG.  Calls share the
 * array: calls that overlap on the GPU race. */
int sg_coulomb_accel_noalloc(int n, const double* pos, const double* q, const double* kq,
                             double* acc, void* stream);

/* ---- resident clouds: Dormand-Prince integration on the device -------------- */

/* Describe n_clouds independent clouds with counts[c] ions each (ions of cloud c
 * follow those of cloud c-1 in every host array).  Allocates device state. */
int sg_batch_create(sg_ctx* ctx, int n_clouds, const int* counts,
                    const sg_field_params* fp, const sg_ode_params* op, int precision);
/* Upload state (host double[n_total][3] pos/vel, kg masses, integer charges) and
 * reset every cloud's controller to its sg_ode_params. */
int sg_batch_upload(sg_ctx* ctx, const double* pos, const double* vel,
                    const double* mass, const int* charge);
/* Upload positions and velocities only (controller state kept). */
int sg_batch_set_state(sg_ctx* ctx, const double* pos, const double* vel);
/* Download positions and velocities (host double[n_total][3]). */
int sg_batch_download(sg_ctx* ctx, double* pos, double* vel);
/* Enqueue n_attempts Dormand-Prince attempts for every cloud that is not done
 * (an accepted attempt commits the step, a rejected one shrinks h; ode.cpp:459-494).
 * Asynchronous: returns once the work is queued. */
int sg_batch_attempts(sg_ctx* ctx, int n_attempts);
/* One accepted step for every cloud that is not done: attempts until each cloud
 * has accepted (or failed).  Synchronous. */
int sg_dp45_step(sg_ctx* ctx, sg_step_info* info);
/* Advance every cloud to its t_end (or until max_attempts attempts); synchronous. */
int sg_batch_run(sg_ctx* ctx, int64_t max_attempts, sg_step_info* info);
/* Per-cloud controller state (host array of n_clouds). Synchronous. */
int sg_batch_info(sg_ctx* ctx, sg_step_info* info);
/* Change one cloud's field parameters (e.g. a trap ramp between steps). */
int sg_batch_set_field(sg_ctx* ctx, int cloud, const sg_field_params* fp);
/* Change one cloud's end time. */
int sg_batch_set_t_end(sg_ctx* ctx, int cloud, double t_end);
/* Record each Coulomb launch with CUDA events (1) or not (0); read back the total
 * kernel time and launch count since the last reset. */
int sg_set_kernel_timing(sg_ctx* ctx, int on);
int sg_kernel_timing(sg_ctx* ctx, double* coulomb_ms, int64_t* coulomb_launches,
                     double* coulomb_interactions);
/* The O(N) kernels of the attempts run with kernel timing on (stage combines, control,
 * commit; graph-replayed attempts only): summed milliseconds and launches. */
int sg_stage_timing(sg_ctx* ctx, double* ms, int64_t* launches);
/* FP32c conditioning fix-ups (flagged ions: their rows re-evaluated in FP64, or their
 * far terms corrected) since the last call; resets the count. */
int sg_fixup_count(sg_ctx* ctx, int64_t* count);
/* Launch shape of the FP32c Coulomb kernel for batches and calls created afterwards:
 * -1 = chosen from the cloud sizes (default), 0 = 128 threads x 4 ions,
 * 1 = 128 x 2, 2 = 256 x 2, 3 = 64 x 4, 4 = 128 x 4 with the ions kept in k-d tree
 * order and far tile pairs summed from the high parts of the coordinates, 5 = 64 x 2,
 * 6 = 32 x 4, 7 = the k-d ordered form with one 128-ion leaf per block (32 x 4), 8 = the
 * same with the leaf over two warps (64 x 2), 9 = over four warps (128 x 1), 10 = 32 x 2,
 * 11 = 32 x 1, 12 and 13 = 9 and 8 with 256-ion j-tiles, 14 = 13 with four j pairs in
 * flight on far tiles, 15 = 7 with 256-ion j-tiles, 16 = 13 with a 4-stage copy ring. */
int sg_set_coulomb_variant(sg_ctx* ctx, int variant);
/* Launch shape the resident batch was planned with (0..4; 0 for FP64 batches). */
int sg_batch_variant(sg_ctx* ctx, int* variant);
/* Capture the attempt sequence in a CUDA graph (1) or launch it directly (0). */
int sg_set_use_graph(sg_ctx* ctx, int on);
/* Host-side timer on the context stream (CUDA events). */
int sg_timer_start(sg_ctx* ctx);
int sg_timer_stop(sg_ctx* ctx, double* ms);

/* Per-cloud moments of the resident state (host double[n_clouds][12]):
 * centroid x,y,z; RMS size x,y,z; mean v^2 per axis x,y,z (m^2/s^2);
 * T_radial, T_axial in kelvin (the reference's Temperature(), bin/ioncloud.cpp:316-335,
 * with per-ion masses); number of ions. */
int sg_batch_moments(sg_ctx* ctx, double* out);

/* ---- learned step-size proposer ---------------------------------------------
 * An MLP 16 -> 64 -> 64 -> 1 (SiLU; BF16 weights, FP32 accumulation) proposes each
 * accepted step's successor from 16 features of the cloud (moments, last step size,
 * last error norm, excitation phase).  Weights are a flat float array of
 * sg_mlp_param_count() values: W1[64][16], b1[64], W2[64][64], b2[64], W3[64], b3.
 * Every attempt is still accepted or rejected by the Dormand-Prince error estimate. */
int sg_mlp_param_count(void);
/* out[i] = MLP(X[i]) for n feature rows X[n][16]. */
int sg_mlp_forward(sg_ctx* ctx, int n, const float* X, const float* w, float* out);
/* Gradient of the MSE loss (1/n) sum (MLP(X_i) - Y_i)^2 w.r.t. the weights. */
int sg_mlp_grad(sg_ctx* ctx, int n, const float* X, const float* Y, const float* w,
                float* grad, float* loss);
/* Adam (lr, beta 0.9/0.999) on minibatches of `batch` rows for `iters` iterations;
 * w is the initial FP32 master copy on input and the trained one on output. */
int sg_mlp_train(sg_ctx* ctx, int n, const float* X, const float* Y, int iters, int batch,
                 float lr, uint64_t seed, float* w, float* loss_hist);
/* Use the MLP (w != NULL) with step-size safety factor `safety` in (0, 1] for the
 * clouds of the batch, or the reference's controller (w == NULL). */
int sg_batch_set_proposer(sg_ctx* ctx, const float* w, double safety);
/* Small clouds (no counterpart in the reference): FP32c Dormand-Prince batches whose
 * clouds are small, in the plain ion order and without a recorder, operations,
 * dissociation, step log or proposer, run whole attempts in one launch, one thread-block
 * cluster of up to 16 CTAs per cloud.  sg_set_fused(ctx, mode): 1 (default) for clouds
 * of at most 512 ions, where it is faster than the tiled kernels; 2 for clouds of up to
 * 2,048 ions; 0 never.  sg_batch_fused gives the cluster size
 * the current batch runs with (0: the tiled kernels).  sg_fused_timing: CUDA-event time
 * of the fused launches while sg_set_kernel_timing is on. */
int sg_set_fused(sg_ctx* ctx, int on);
int sg_batch_fused(sg_ctx* ctx, int* cluster);
int sg_fused_timing(sg_ctx* ctx, double* ms, int64_t* launches);

/* In-run check of the FP32c Coulomb sums (no counterpart in the reference).  Every
 * `every_attempts` attempts (default 16; 0 = off) the last Coulomb sum of the attempt
 * is checked, per cloud, at eight probe ions -- the two ions without fix-up whose far
 * terms are largest next to their net force (sqrt(s2f)/|P|), the two whose near terms
 * are, and four drawn at random -- against their rows evaluated exactly in FP64.  From
 * the far-ranked probes the check measures c = err / (sqrt(s2f)/|P|) and lowers the
 * cloud's far fix-up threshold kfar (an ion with sqrt(s2f) > kfar |P| is corrected) to
 * 5e-7 / c when that is below the prior set from the cloud's density.  FP32c batches
 * only. */
typedef struct sg_check_info {
    double max_err;      /* largest per-ion relative error over every check               */
    double last_err;     /* largest of the last check                                     */
    double c_far;        /* largest measured err / (sqrt(s2f)/|P|), 0 before any          */
    double kfar;         /* far fix-up threshold in use                                   */
    double kfar_prior;   /* the prior from the cloud's density (or sg_batch_set_far_threshold) */
    int64_t checks;      /* checks made                                                   */
    int64_t probes;      /* probe ions evaluated                                          */
    int64_t breaches;    /* probes above 1e-6                                             */
    double max_err_far;    /* largest error of the far-ranked probes                      */
    double max_err_near;   /* ... of the near-ranked probes                               */
    double max_err_random; /* ... of the random probes                                    */
    /* the probe with the largest error over every check */
    double worst_err;      /* its relative error                                          */
    double worst_rf;       /* its far ratio sqrt(s2f)/|P| (-1: flagged and fixed up)       */
    double worst_rn;       /* its near ratio sqrt(s2)/|P| (-1: flagged and fixed up)       */
    int32_t worst_ion;     /* its index within the cloud, in the caller's order (-1: none) */
    int32_t worst_kind;    /* 0 far-ranked, 1 near-ranked, 2 random                       */
} sg_check_info;
int sg_batch_set_force_check(sg_ctx* ctx, int every_attempts);
int sg_batch_force_check(sg_ctx* ctx, sg_check_info* out);  /* out[n_clouds] */
/* Prior of the far fix-up threshold for every cloud of the batch (kfar > 0), or the
 * automatic prior from each cloud's density (kfar = 0); clears the measured record.
 * Takes effect at the next sg_batch_upload / sg_batch_set_state. */
int sg_batch_set_far_threshold(sg_ctx* ctx, double kfar);

/* Test of the bounded device waits (no counterpart in the reference).  With tile >= 0,
 * every block of the FP32c Coulomb kernels of the current batch, once its j-tile
 * `tile` has arrived, also waits on a barrier that nothing arrives at until limit_us
 * microseconds (1 .. 1e6) have passed, and then takes its timeout path: it raises
 * SG_TIMEOUT, waits (bounded) for the copies it has issued, and returns without writing
 * sums.  The attempt is then neither accepted nor used for step control: every cloud
 * stops with status SG_TIMEOUT and the call returns it.  tile < 0 turns the test off;
 * sg_batch_upload clears the error word.  No copy is left in flight and no device
 * state is lost: the context stays usable. */
int sg_set_wait_test(sg_ctx* ctx, int tile, int limit_us);
/* The reference's controller with the safety factor of its accepted-step rule
 * (0.9, bin/ode.cpp:431,439) replaced by `safety` in (0, 1]: the ablation that separates
 * the proposer's learning from a plain change of safety.  Replaces the proposer; the
 * reject rule is unchanged.  sg_batch_set_proposer(ctx, NULL, ...) restores the rule. */
int sg_batch_set_controller_safety(sg_ctx* ctx, double safety);
/* Record up to `capacity` accepted steps per cloud: features at the step start and
 * (h_prev, h, err, t_end_of_step). */
int sg_batch_set_log(sg_ctx* ctx, int capacity);
int sg_batch_read_log(sg_ctx* ctx, int cloud, float* feat, double* num, int cap, int* count);

/* ---- measurement probes ----------------------------------------------------- */
/* Issue-rate probes: FP32 FFMA, packed FP32x2 FFMA2 and FP64 DFMA throughput of the
 * device in GFLOP/s (2 flops per FMA lane), measured with CUDA events. */
int sg_probe_peaks(sg_ctx* ctx, double* fp32_gflops, double* fp32x2_gflops,
                   double* fp64_gflops);

/* ---- recorder: device-side observables ---------------------------------------
 * The reference prints after a step once (t - t_start) > print_interval * prints so
 * far (move_particles, bin/ion_fly.cpp:103-108): the state of every ion
 * (PrintParticles) and per species the centroid, spread and energy (PrintCloud,
 * bin/ioncloud.cpp:148-183).  The recorder applies the same rule on the device,
 * inside the attempt sequence (no host round trip): a record is
 *   [0] t (s),
 *   [1 + 9 s .. 9 s + 9] for species s: x0 y0 z0 x1 y1 z1 (m), energy (eV), ions of s,
 *                        ions of the cloud -- with the reference's arithmetic: centroid
 *                        and spread divide by the cloud's ion count, the energy sums
 *                        m (vx^2 + vy^2 + vz vy) / 2,
 *   then x y z vx vy vz of every stride-th ion of the cloud (caller's order).
 * Each cloud has a device ring of `capacity` records; the host drains the rings into
 * host memory whenever a call synchronises (sg_batch_run, sg_dp45_step, sg_batch_info,
 * ...), and a cloud whose ring is full waits until then.  The print clock starts at
 * the time of this call (at t0 before an upload) and restarts on upload.
 * print_interval 0 records only on sg_batch_record_now; capacity 0 turns it off.
 * species: per ion (caller order) in [0, n_species), NULL = all 0; n_species <= 8. */
int sg_batch_set_recorder(sg_ctx* ctx, double print_interval, int stride, int capacity,
                          const int* species, int n_species);
/* A record of every active cloud now (the reference's print after an operation). */
int sg_batch_record_now(sg_ctx* ctx);
/* Drained records held for `cloud`, doubles per record, ions kept per record. */
int sg_batch_records(sg_ctx* ctx, int cloud, int64_t* n_records, int* record_len,
                     int* n_kept);
/* Moves up to max_records drained records of `cloud` (oldest first) into out
 * [n][record_len]. */
int sg_batch_read_records(sg_ctx* ctx, int cloud, int64_t max_records, double* out,
                          int64_t* n_read);
/* The reference's text output of the drained records of `cloud`, appended to
 * <prefix>_pAll.txt (ID name t(ms) x y z (mm) vx vy vz (m/s) E(eV) per kept ion) and
 * <prefix>_cloud<s>.txt (s name N t(ms) x0 y0 z0 x1 y1 z1 (mm) E(eV)), with the
 * reference's header for new files; names[s] names species s.  Consumes the records. */
int sg_batch_write_text(sg_ctx* ctx, int cloud, const char* prefix, const char* const* names,
                        int n_names);

/* ---- operations: the reference's operation sequence, run on the device --------
 * operations::launch (bin/operation.cpp:33-77, 111-124) runs its operations one after
 * the other, each through move_particles (bin/ion_fly.cpp:17-116): steps are taken
 * while t < t_start + duration, the trap ramp sets Vrf/Vdc before every step
 * (bin/ion_fly.cpp:95-99).  Here the whole sequence advances inside the control kernel,
 * on the device, between two attempts, with no host round trip:
 *   NORMAL        trap terms on (the cloud's Paul and Penning terms), TOF off
 *   TOF           trap off, TOF kick E_kick on
 *   TRAP_RAMP     trap on, Vrf/Vdc = old (1 - r) + new r before each step,
 *                 r = (t - t_start) / duration, old = the values when it starts
 *   FREE          trap and TOF off (the reference's fall-through "free flight")
 *   DISSOCIATION  no time passes; ions of species `reactant` become species `product`
 *                 with print mass `product_mass` (kg) where the reference's MT19937
 *                 stream, seeded 0, draws below `fraction`, one draw per reactant ion
 *                 in order (bin/operation.cpp:59-70).  As in the reference the
 *                 dynamics keep the ions' masses: only records and text change.
 * print_time > 0 sets the recorder's print interval from that operation on;
 * timestep > 0 sets h = hnext = print_time, which is what the reference does with its
 * ode_timestep (bin/operation.cpp:36-39).  print_after records the state when the
 * operation ends (odev.print_after_operation).  The batch's t_end is replaced by the
 * end of the last operation.  Set after sg_batch_create (before or after an upload: an
 * upload restarts the sequence). */
enum {
    SG_OP_NORMAL = 0,
    SG_OP_TOF = 1,
    SG_OP_TRAP_RAMP = 2,
    SG_OP_FREE = 3,
    SG_OP_DISSOCIATION = 4
};
typedef struct sg_operation {
    int32_t kind;
    int32_t print_after;
    double duration;      /* s */
    double print_time;    /* s, 0 = unchanged */
    double timestep;      /* nonzero: h = hnext = print_time */
    double new_vrf, new_vdc;  /* TRAP_RAMP targets (V) */
    double e_kick;        /* TOF (V/m) */
    int32_t reactant, product;  /* DISSOCIATION species */
    double fraction, product_mass;
} sg_operation;
int sg_batch_set_operations(sg_ctx* ctx, const sg_operation* ops, int n_ops);
/* Index of each cloud's current operation (n_ops once the sequence has ended). */
int sg_batch_operation_index(sg_ctx* ctx, int* index);

/* ---- initial cloud ------------------------------------------------------------
 * InitCloud (bin/initialization.cpp:117-206), host side: n ions uniform in the
 * ellipsoid offset + semiaxis * (unit ball), drawn by rejection from the unit cube;
 * speed v = sqrt(-2 E e / m ln(1 - sqrt(u))) around the energy E (eV) of the
 * Maxwell-Boltzmann maximum, direction uniform on the sphere (theta = 2 pi u,
 * phi = acos(2u - 1)).  With n_ev = 2, ev_max[1] sets the speed of the axial component.
 * Random stream: MT19937 seeded with `seed`, doubles = 32-bit output * 2^-32, in the
 * reference's draw order, so the same seed gives the reference's cloud.  mass in kg;
 * pos (m) and vel (m/s) are written AoS [n][3]. */
int sg_init_cloud(int n, const double* ev_max, int n_ev, uint32_t seed, const double* semiaxis,
                  const double* offset, const double* mass, double* pos, double* vel);

/* ---- state files ----------------------------------------------------------------
 * Binary state file, for restarts: the 8 bytes "SGSTATE1", uint32 version (1), uint32 n,
 * double t, then pos [n][3], vel [n][3], mass [n] (f64), charge [n], species [n] (i32),
 * all little-endian.  species may be NULL (written as 0).  sg_state_info reads the
 * header; sg_state_load needs cap >= n (SG_TOO_LARGE otherwise).  SG_IO_ERR on a file
 * that cannot be opened, is truncated or is not a state file. */
int sg_state_save(const char* path, int n, double t, const double* pos, const double* vel,
                  const double* mass, const int* charge, const int* species);
int sg_state_info(const char* path, int* n, double* t);
int sg_state_load(const char* path, int cap, double* t, double* pos, double* vel, double* mass,
                  int* charge, int* species);

/* Restart from the reference's particle output (PrintParticles, bin/ioncloud.cpp:85-111:
 * per ion "ID name t[ms] x y z[mm] vx vy vz[m/s] E[eV]", one block of lines per print,
 * IDs ascending): the ions of the last print (a print starts where the time changes or
 * the IDs start over), in file order.  The reference's own importer
 * (ImportData, bin/parser.cpp:102) expects other columns and cannot read this output.
 * Names are looked up in names[0..n_names) for species, mass (kg) and charge.  *n is the
 * number of ions read (SG_TOO_LARGE if more than cap); SG_BAD_ARG for an unknown name,
 * SG_IO_ERR for an unreadable or malformed file. */
int sg_particles_text_last(const char* path, const char* const* names, const double* masses,
                           const int* charges, int n_names, int cap, int* n, double* t,
                           int* ids, double* pos, double* vel, double* mass, int* charge,
                           int* species);

/* ---- drop-in slot of the reference's CUNBODY backend ------------------------
 * Same symbols and argument meaning as the closed library (bin/cunbody.h:11-33):
 *   ai[i] = sum_j mj[j] (xj[j]-xi[i]) / (|xj[j]-xi[i]|^2 + eps2)^{3/2}
 * begin is asynchronous, end blocks and writes ai; cunbody1_force does both.
 * Evaluated in FP64 on the default device with a process-wide context. */
void cunbody1_force(double xj[][3], double mj[], double xi[][3], double eps2,
                    double ai[][3], int ni, int nj);
void cunbody1_force_begin(double xj[][3], double mj[], double xi[][3], double eps2,
                          double ai[][3], int ni, int nj);
void cunbody1_force_end(double xj[][3], double mj[], double xi[][3], double eps2,
                        double ai[][3], int ni, int nj);

#ifdef __cplusplus
}
#endif

#endif /* SIMGB_H */
