/*
 * oracle.h -- CPU restatement of the Simbuca integration hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for libsimgb: the
 * parity tests, __graft_entry__.smoke() and the CPU-baseline leg of bench.py call
 * it; the product never links, loads or calls it.
 *
 * It restates, in plain C and FP64, with the reference's operation order:
 *   - the CPU direct-sum Coulomb loop            bin/force.cpp:147-174
 *   - the trap and TOF field terms               bin/force.cpp:34-82
 *   - Dormand_Prince_5                           bin/ode.cpp:61-218
 *   - RungaKutta4 (Cash-Karp 5(4))               bin/ode.cpp:220-345
 *   - GearMethod (5th-order predictor-corrector) bin/ode.cpp:347-424
 *   - error_succes (step-size controller)        bin/ode.cpp:426-457
 *   - step (retry loop, underflow, commit)       bin/ode.cpp:459-494
 *   - IonCloud::Temperature                      bin/ioncloud.cpp:316-335
 * and adds the Penning-trap, RF-excitation and buffer-gas terms, which have no
 * reference implementation, written from the physics in simgb.h.
 *
 * Compile with -ffp-contract=off so that x86-64 and aarch64 builds round alike.
 * Parity of this restatement with the reference itself is pinned by
 * tests/test_oracle_golden.py against vectors generated by the compiled
 * reference (oracle/ref_harness.cpp).
 */
#ifndef SIMGB_ORACLE_H
#define SIMGB_ORACLE_H

#include "../include/simgb.h"

#ifdef __cplusplus
extern "C" {
#endif

/* reference constants, bin/globals.h:4-16 */
#define ORC_PI 3.14159265358979323
#define ORC_EL_CHARGE 1.60217733e-19
#define ORC_AMU 1.6605402E-27
#define ORC_KE 8.987551787E9
#define ORC_KB 1.3806504E-23

/* controller state of one cloud: the scalar members of _ode_vars (bin/ode.h:58-97)
 * plus the cloud lifetime and counters. */
typedef struct orc_ctrl {
    double rtol, atol;
    double h, hnext, errold, err;
    double t, t_end;
    int32_t reject, adaptive, max_rejects, status;
    int64_t steps, rejects, force_evals, attempts;
    double beta; /* PI term of error_succes; the reference's build has 0 */
} orc_ctrl;

void orc_set_threads(int n);
int orc_get_threads(void);

/* derivs[i] -= coulomb_scale ke e^2 q_i/m_i sum_{j!=i} q_j (x_j-x_i)/r^3 ... written
 * exactly as bin/force.cpp:149-174 (derivs is updated in place). */
void orc_coulomb_sub(int n, const double* pos, const double* mass, const int* charge,
                     double coulomb_scale, double* derivs);

/* acc[i] = kq[i] sum_{j!=i} q[j] (x_i-x_j)/r^3, same loop order as above. */
void orc_coulomb_kq(int n, const double* pos, const double* q, const double* kq,
                    double* acc);

/* Same as orc_coulomb_kq for rows [i0, i1) only (sampled rows for large n). */
void orc_coulomb_kq_rows(int n, const double* pos, const double* q, const double* kq,
                         int i0, int i1, double* acc_rows);

/* Field terms only (derivs overwritten): bin/force.cpp:58-82 + Penning/drives/friction. */
void orc_field(int n, const double* pos, const double* vel, const double* mass,
               const int* charge, double t, const sg_field_params* fp, double* derivs);

/* force(): field terms then the Coulomb sum when SG_F_COULOMB is set. */
void orc_force(int n, const double* pos, const double* vel, const double* mass,
               const int* charge, double t, const sg_field_params* fp, double* derivs);

/* One Dormand_Prince_5 attempt from (pos, vel) with ctrl->h; writes pos2/vel2 (y5)
 * and returns the RMS error norm.  k is scratch of 7*n*6 doubles, derivs n*3. */
double orc_dp45_attempt(int n, const double* pos, const double* vel, const double* mass,
                        const int* charge, const sg_field_params* fp, orc_ctrl* c,
                        double* pos2, double* vel2, double* k, double* derivs);

/* One Cash-Karp 5(4) attempt, the reference's "RungaKutta4" (bin/ode.cpp:220-345):
 * 6 stages, 5th-order solution into pos2/vel2.  As in the reference the error sum
 * starts from the previous error norm (odev.err is never reset there), carried in
 * c->err.  k is scratch of 6*n*6 doubles. */
double orc_ck45_attempt(int n, const double* pos, const double* vel, const double* mass,
                        const int* charge, const sg_field_params* fp, orc_ctrl* c,
                        double* pos2, double* vel2, double* k, double* derivs);

/* GearMethod (bin/ode.cpp:347-424), one fixed step from (pos, vel) into pos2/vel2.
 * g is the Gear state [4][n][3] (acceleration, b, c, d), updated in place; hf the
 * step powers h^2/2, h^3/6, h^4/24, h^5/120 of the initial step.  orc_gear_init seeds
 * g as InitAcceleraction does (bin/ode.cpp:36-59). */
void orc_gear_init(int n, double* g);
void orc_gear_step(int n, const double* pos, const double* vel, const double* mass,
                   const int* charge, const sg_field_params* fp, orc_ctrl* c, const double* hf,
                   double* pos2, double* vel2, double* g, double* derivs);

/* Step loop with the method of the reference's Init_ode order: 5 = Dormand-Prince,
 * 4 = Cash-Karp, 1 = Gear (fixed step, error control off).  Same contract as
 * orc_dp45_run. */
int64_t orc_rk_run(int method, int n, double* pos, double* vel, const double* mass,
                   const int* charge, const sg_field_params* fp, orc_ctrl* c,
                   int64_t max_steps, double* hist, int64_t hist_cap);

/* error_succes (bin/ode.cpp:426-457): 1 = accepted. */
int orc_error_succes(double err, orc_ctrl* c);

/* Run accepted steps until ctrl->t >= ctrl->t_end or max_steps accepted steps;
 * pos/vel are updated in place.  Each attempt appends (t_start, h, err, accepted)
 * to hist (capacity hist_cap attempts; pass NULL to skip).  Returns the number of
 * attempts recorded, or a negative SG_ status on failure. */
int64_t orc_dp45_run(int n, double* pos, double* vel, const double* mass,
                     const int* charge, const sg_field_params* fp, orc_ctrl* c,
                     int64_t max_steps, double* hist, int64_t hist_cap);

/* Fixed steps with a given schedule: step k starts at ts[k] with size hs[k] (no error
 * control), as the reference's step() does with change_stepsize false.  Used to
 * replay the step sequence another implementation accepted. */
int orc_dp45_replay(int n, double* pos, double* vel, const double* mass, const int* charge,
                    const sg_field_params* fp, const double* ts, const double* hs, int nsteps);
/* The same with method 5 (Dormand-Prince) or 4 (Cash-Karp). */
int orc_rk_replay(int method, int n, double* pos, double* vel, const double* mass,
                  const int* charge, const sg_field_params* fp, const double* ts,
                  const double* hs, int nsteps);

/* PrintCloud statistics (bin/ioncloud.cpp:148-183) per species: out[n_species][9] =
 * x0, y0, z0, x1, y1, z1 (m), energy (eV), ions of the species, ions of the cloud,
 * with the reference's arithmetic (divisions by the cloud's ion count, vz vy term). */
void orc_cloud_stats(int n, const double* pos, const double* vel, const double* mass,
                     const int* species, int n_species, double* out);

/* Moments of one cloud: out[12] as sg_batch_moments. */
void orc_moments(int n, const double* pos, const double* vel, const double* mass,
                 double* out);

#ifdef __cplusplus
}
#endif

#endif
