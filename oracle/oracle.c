/*
 * oracle.c -- CPU restatement of the Simbuca hot path (test infrastructure only;
 * see oracle.h).  Each function names the reference lines it restates.
 *
 * Threads: the Coulomb rows are split over POSIX threads.  Every row is still
 * summed by one thread in the reference's order, so results do not depend on the
 * thread count.
 */
#include "oracle.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

static int g_threads = 1;

void orc_set_threads(int n) { g_threads = n < 1 ? 1 : (n > 256 ? 256 : n); }
int orc_get_threads(void) { return g_threads; }

/* std::max / std::min of the reference (C++98 <algorithm>): max(a,b) = a<b ? b : a */
static inline double ref_max(double a, double b) { return (a < b) ? b : a; }
static inline double ref_min(double a, double b) { return (b < a) ? b : a; }

/* ---------------------------------------------------------------------------
 * Coulomb rows.  bin/force.cpp:147-174 (serial CPU path, no MPI):
 *   kTqiTqjDmj = coulomb_scale*ke*el_charge*charge[j]*el_charge/mass[j];
 *   for i != j: rx = pos2[i]-pos2[j] ...; distSqr = rx*rx+ry*ry+rz*rz;
 *     invDist = 1./sqrt(distSqr); invDistCube = invDist*invDist*invDist;
 *     fx += rx*invDistCube*kTqiTqjDmj*charge_i;
 *   derivs[j] -= fx
 * Here "self" is the reference's j_ and "other" its i_.
 * ------------------------------------------------------------------------- */
typedef struct {
    int n, r0, r1;
    const double* pos;
    const double* qd;     /* charge of the other ion as double              */
    const double* kq;     /* per-row coefficient kTqiTqjDmj, or NULL        */
    const double* mass;   /* used with charge when kq == NULL               */
    const int* charge;
    double coulomb_scale;
    double* out;          /* rows r0..r1 */
    int mode;             /* 0: out -= f (reference derivs); 1: out = -f (kq)  */
    int out_offset;       /* out row index = row - out_offset                */
} coul_job;

static void coul_rows(const coul_job* jb) {
    const double* pos = jb->pos;
    const int n = jb->n;
    for (int j = jb->r0; j < jb->r1; j++) {
        double fx = 0.0, fy = 0.0, fz = 0.0;
        double kT;
        if (jb->kq) {
            kT = jb->kq[j];
        } else {
            /* left-to-right as written at force.cpp:153 */
            kT = jb->coulomb_scale * ORC_KE * ORC_EL_CHARGE * jb->charge[j] * ORC_EL_CHARGE /
                 jb->mass[j];
        }
        const double bjx = pos[3 * j + 0], bjy = pos[3 * j + 1], bjz = pos[3 * j + 2];
        for (int i = 0; i < n; i++) {
            if (i != j) {
                double rx = pos[3 * i + 0] - bjx;
                double ry = pos[3 * i + 1] - bjy;
                double rz = pos[3 * i + 2] - bjz;
                double distSqr = rx * rx + ry * ry + rz * rz;
                double invDist = 1. / sqrt(distSqr);
                double invDistCube = (invDist * invDist * invDist);
                double qi = jb->charge ? (double)jb->charge[i] : jb->qd[i];
                fx += rx * invDistCube * kT * qi;
                fy += ry * invDistCube * kT * qi;
                fz += rz * invDistCube * kT * qi;
            }
        }
        double* o = jb->out + 3 * (size_t)(j - jb->out_offset);
        if (jb->mode == 0) {
            o[0] -= fx;
            o[1] -= fy;
            o[2] -= fz;
        } else {
            o[0] = 0.0 - fx;
            o[1] = 0.0 - fy;
            o[2] = 0.0 - fz;
        }
    }
}

static void* coul_thread(void* arg) {
    coul_rows((const coul_job*)arg);
    return NULL;
}

static void coul_parallel(coul_job base, int r0, int r1) {
    int nt = g_threads;
    int rows = r1 - r0;
    if (nt <= 1 || rows < 64) {
        base.r0 = r0;
        base.r1 = r1;
        coul_rows(&base);
        return;
    }
    if (nt > rows) nt = rows;
    pthread_t th[256];
    coul_job jobs[256];
    int started = 0;
    for (int t = 0; t < nt; t++) {
        jobs[t] = base;
        jobs[t].r0 = r0 + (int)((long long)rows * t / nt);
        jobs[t].r1 = r0 + (int)((long long)rows * (t + 1) / nt);
        if (t == 0) continue;
        if (pthread_create(&th[t], NULL, coul_thread, &jobs[t]) != 0) {
            coul_rows(&jobs[t]); /* no thread available: do it here */
            th[t] = 0;
        } else {
            started |= 0;
        }
    }
    coul_rows(&jobs[0]);
    for (int t = 1; t < nt; t++)
        if (th[t]) pthread_join(th[t], NULL);
    (void)started;
}

void orc_coulomb_sub(int n, const double* pos, const double* mass, const int* charge,
                     double coulomb_scale, double* derivs) {
    coul_job jb;
    memset(&jb, 0, sizeof jb);
    jb.n = n;
    jb.pos = pos;
    jb.mass = mass;
    jb.charge = charge;
    jb.coulomb_scale = coulomb_scale;
    jb.out = derivs;
    jb.mode = 0;
    coul_parallel(jb, 0, n);
}

void orc_coulomb_kq(int n, const double* pos, const double* q, const double* kq,
                    double* acc) {
    coul_job jb;
    memset(&jb, 0, sizeof jb);
    jb.n = n;
    jb.pos = pos;
    jb.qd = q;
    jb.kq = kq;
    jb.out = acc;
    jb.mode = 1;
    coul_parallel(jb, 0, n);
}

void orc_coulomb_kq_rows(int n, const double* pos, const double* q, const double* kq,
                         int i0, int i1, double* acc_rows) {
    coul_job jb;
    memset(&jb, 0, sizeof jb);
    jb.n = n;
    jb.pos = pos;
    jb.qd = q;
    jb.kq = kq;
    jb.out = acc_rows;
    jb.mode = 1;
    jb.out_offset = i0;
    coul_parallel(jb, i0, i1);
}

/* ---------------------------------------------------------------------------
 * Field terms.  Paul trap and TOF: bin/force.cpp:40-44 and 58-82, same operation
 * order.  Penning, excitations and friction: no reference code; formulas in simgb.h.
 * ------------------------------------------------------------------------- */
void orc_field(int n, const double* pos, const double* vel, const double* mass,
               const int* charge, double t, const sg_field_params* fp, double* derivs) {
    const double kVdc = fp->kappa * fp->Vdc;
    const double Vrf = fp->Vrf;
    const double r02 = fp->r0 * fp->r0;
    const double z02 = fp->z0 * fp->z0;
    const double omega_rf = fp->freq_rf * 2 * ORC_PI;
    const uint32_t f = fp->flags;

    /* Penning and drive coefficients (per unit q e/m) */
    const double kp = (f & SG_F_PENNING) ? fp->V0 / (2.0 * fp->d0 * fp->d0) : 0.0;
    double gq = 0.0, gd = 0.0;
    if ((f & SG_F_QUAD) && t >= fp->tq_on && t < fp->tq_off)
        gq = (2.0 * fp->Uq / (fp->r_el * fp->r_el)) * cos(2.0 * ORC_PI * fp->nu_q * t + fp->phi_q);
    if ((f & SG_F_DIPOLE) && t >= fp->td_on && t < fp->td_off)
        gd = (fp->Ud / fp->r_el) * cos(2.0 * ORC_PI * fp->nu_d * t + fp->phi_d);

    for (int j_ = 0; j_ < n; j_++) {
        double x = pos[3 * j_ + 0], y = pos[3 * j_ + 1], z = pos[3 * j_ + 2];
        double vx = vel[3 * j_ + 0], vy = vel[3 * j_ + 1], vz = vel[3 * j_ + 2];
        double* d = derivs + 3 * (size_t)j_;
        d[0] = 0;
        d[1] = 0;
        d[2] = 0;
        if (f & SG_F_PAUL) {
            double qDmassa = charge[j_] * ORC_EL_CHARGE / mass[j_];
            d[0] += qDmassa * (kVdc / z02 - Vrf * cos(omega_rf * t) / r02) * x;
            d[1] += qDmassa * (kVdc / z02 + Vrf * cos(omega_rf * t) / r02) * y;
            d[2] += qDmassa * (-2.0 * kVdc / z02) * z;
        }
        if (f & SG_F_TOF) {
            double qDmassa = charge[j_] * ORC_EL_CHARGE / mass[j_];
            d[0] += qDmassa * fp->E_kick;
        }
        if (f & (SG_F_PENNING | SG_F_QUAD | SG_F_DIPOLE)) {
            double qm = charge[j_] * ORC_EL_CHARGE / mass[j_];
            double ex = 0.0, ey = 0.0, ez = 0.0;
            if (f & SG_F_PENNING) {
                ex = kp * x + fp->B * vy;
                ey = kp * y - fp->B * vx;
                ez = -2.0 * kp * z;
            }
            ex += gq * y + gd;
            ey += gq * x;
            d[0] += qm * ex;
            d[1] += qm * ey;
            d[2] += qm * ez;
        }
        if (f & SG_F_FRICTION) {
            d[0] -= fp->delta * vx;
            d[1] -= fp->delta * vy;
            d[2] -= fp->delta * vz;
        }
        (void)vz;
    }
}

void orc_force(int n, const double* pos, const double* vel, const double* mass,
               const int* charge, double t, const sg_field_params* fp, double* derivs) {
    orc_field(n, pos, vel, mass, charge, t, fp, derivs);
    if (fp->flags & SG_F_COULOMB) orc_coulomb_sub(n, pos, mass, charge, fp->coulomb_scale, derivs);
}

/* ---------------------------------------------------------------------------
 * Dormand_Prince_5, bin/ode.cpp:61-218.  k[s][j][0..2] = stage velocity,
 * k[s][j][3..5] = stage acceleration.  Stage s of the reference reads the time
 * from the cloud lifetime (force.cpp:36), i.e. the step start for every stage;
 * without SG_F_FROZEN_T stage s is evaluated at t + c_s h.
 * ------------------------------------------------------------------------- */
static const double DPc2 = 1.0 / 5.0, DPc3 = 3.0 / 10.0, DPc4 = 4.0 / 5.0, DPc5 = 8.0 / 9.0,
                    DPc6 = 1.0, DPc7 = 1.0;
static const double DPa21 = 1.0 / 5.0, DPa31 = 3.0 / 40.0, DPa32 = 9.0 / 40.0,
                    DPa41 = 44.0 / 45.0, DPa42 = -56.0 / 15.0, DPa43 = 32.0 / 9.0,
                    DPa51 = 19372.0 / 6561.0, DPa52 = -25360.0 / 2187.0,
                    DPa53 = 64448.0 / 6561.0, DPa54 = -212.0 / 729.0,
                    DPa61 = 9017.0 / 3168.0, DPa62 = -355.0 / 33.0, DPa63 = 46732.0 / 5247.0,
                    DPa64 = 49.0 / 176.0, DPa65 = -5103.0 / 18656.0, DPa71 = 35.0 / 384.0,
                    DPa73 = 500.0 / 1113.0, DPa74 = 125.0 / 192.0, DPa75 = -2187.0 / 6784.0,
                    DPa76 = 11.0 / 84.0;
static const double DPb1 = 35.0 / 384.0, DPb3 = 500.0 / 1113.0, DPb4 = 125.0 / 192.0,
                    DPb5 = -2187.0 / 6784.0, DPb6 = 11.0 / 84.0;
static const double DPe1 = 71.0 / 57600.0, DPe3 = -71.0 / 16695.0, DPe4 = 71.0 / 1920.0,
                    DPe5 = -17253.0 / 339200.0, DPe6 = 22.0 / 525.0, DPe7 = -1.0 / 40.0;

#define KS(s, j, c) k[((size_t)(s) * n + (j)) * 6 + (c)]

double orc_dp45_attempt(int n, const double* pos, const double* vel, const double* mass,
                        const int* charge, const sg_field_params* fp, orc_ctrl* cs,
                        double* pos2, double* vel2, double* k, double* derivs) {
    const double h = cs->h;
    const int frozen = (fp->flags & SG_F_FROZEN_T) != 0;
    const double t0 = cs->t;
    double ts[7];
    const double cc[7] = {0.0, DPc2, DPc3, DPc4, DPc5, DPc6, DPc7};
    for (int s = 0; s < 7; s++) ts[s] = frozen ? t0 : t0 + cc[s] * h;

    double err = 0.0, sk;
    for (int j = 0; j < n; j++) {
        KS(0, j, 0) = vel[3 * j + 0];
        KS(0, j, 1) = vel[3 * j + 1];
        KS(0, j, 2) = vel[3 * j + 2];
    }
    memcpy(pos2, pos, sizeof(double) * 3 * (size_t)n);
    memcpy(vel2, vel, sizeof(double) * 3 * (size_t)n);

    /* stage 1 -> 2 */
    orc_force(n, pos2, vel2, mass, charge, ts[0], fp, derivs);
    for (int j = 0; j < n; j++) {
        for (int c = 0; c < 3; c++) KS(0, j, 3 + c) = derivs[3 * j + c];
        for (int c = 0; c < 3; c++) pos2[3 * j + c] = pos[3 * j + c] + h * (DPa21 * KS(0, j, c));
        for (int c = 0; c < 3; c++)
            KS(1, j, c) = vel2[3 * j + c] = vel[3 * j + c] + h * (DPa21 * KS(0, j, 3 + c));
    }
    /* stage 2 -> 3 */
    orc_force(n, pos2, vel2, mass, charge, ts[1], fp, derivs);
    for (int j = 0; j < n; j++) {
        for (int c = 0; c < 3; c++) KS(1, j, 3 + c) = derivs[3 * j + c];
        for (int c = 0; c < 3; c++)
            pos2[3 * j + c] = pos[3 * j + c] + h * (DPa31 * KS(0, j, c) + DPa32 * KS(1, j, c));
        for (int c = 0; c < 3; c++)
            KS(2, j, c) = vel2[3 * j + c] =
                vel[3 * j + c] + h * (DPa31 * KS(0, j, 3 + c) + DPa32 * KS(1, j, 3 + c));
    }
    /* stage 3 -> 4 */
    orc_force(n, pos2, vel2, mass, charge, ts[2], fp, derivs);
    for (int j = 0; j < n; j++) {
        for (int c = 0; c < 3; c++) KS(2, j, 3 + c) = derivs[3 * j + c];
        for (int c = 0; c < 3; c++)
            pos2[3 * j + c] = pos[3 * j + c] + h * (DPa41 * KS(0, j, c) + DPa42 * KS(1, j, c) +
                                                    DPa43 * KS(2, j, c));
        for (int c = 0; c < 3; c++)
            KS(3, j, c) = vel2[3 * j + c] =
                vel[3 * j + c] + h * (DPa41 * KS(0, j, 3 + c) + DPa42 * KS(1, j, 3 + c) +
                                      DPa43 * KS(2, j, 3 + c));
    }
    /* stage 4 -> 5 */
    orc_force(n, pos2, vel2, mass, charge, ts[3], fp, derivs);
    for (int j = 0; j < n; j++) {
        for (int c = 0; c < 3; c++) KS(3, j, 3 + c) = derivs[3 * j + c];
        for (int c = 0; c < 3; c++)
            pos2[3 * j + c] = pos[3 * j + c] + h * (DPa51 * KS(0, j, c) + DPa52 * KS(1, j, c) +
                                                    DPa53 * KS(2, j, c) + DPa54 * KS(3, j, c));
        for (int c = 0; c < 3; c++)
            KS(4, j, c) = vel2[3 * j + c] =
                vel[3 * j + c] + h * (DPa51 * KS(0, j, 3 + c) + DPa52 * KS(1, j, 3 + c) +
                                      DPa53 * KS(2, j, 3 + c) + DPa54 * KS(3, j, 3 + c));
    }
    /* stage 5 -> 6 */
    orc_force(n, pos2, vel2, mass, charge, ts[4], fp, derivs);
    for (int j = 0; j < n; j++) {
        for (int c = 0; c < 3; c++) KS(4, j, 3 + c) = derivs[3 * j + c];
        for (int c = 0; c < 3; c++)
            pos2[3 * j + c] =
                pos[3 * j + c] + h * (DPa61 * KS(0, j, c) + DPa62 * KS(1, j, c) +
                                      DPa63 * KS(2, j, c) + DPa64 * KS(3, j, c) +
                                      DPa65 * KS(4, j, c));
        for (int c = 0; c < 3; c++)
            KS(5, j, c) = vel2[3 * j + c] =
                vel[3 * j + c] + h * (DPa61 * KS(0, j, 3 + c) + DPa62 * KS(1, j, 3 + c) +
                                      DPa63 * KS(2, j, 3 + c) + DPa64 * KS(3, j, 3 + c) +
                                      DPa65 * KS(4, j, 3 + c));
    }
    /* stage 6 -> 7 */
    orc_force(n, pos2, vel2, mass, charge, ts[5], fp, derivs);
    for (int j = 0; j < n; j++) {
        for (int c = 0; c < 3; c++) KS(5, j, 3 + c) = derivs[3 * j + c];
        for (int c = 0; c < 3; c++)
            pos2[3 * j + c] =
                pos[3 * j + c] + h * (DPa71 * KS(0, j, c) + DPa73 * KS(2, j, c) +
                                      DPa74 * KS(3, j, c) + DPa75 * KS(4, j, c) +
                                      DPa76 * KS(5, j, c));
        for (int c = 0; c < 3; c++)
            KS(6, j, c) = vel2[3 * j + c] =
                vel[3 * j + c] + h * (DPa71 * KS(0, j, 3 + c) + DPa73 * KS(2, j, 3 + c) +
                                      DPa74 * KS(3, j, 3 + c) + DPa75 * KS(4, j, 3 + c) +
                                      DPa76 * KS(5, j, 3 + c));
    }
    /* stage 7 and the 5th-order solution (ode.cpp:175-187) */
    orc_force(n, pos2, vel2, mass, charge, ts[6], fp, derivs);
    for (int j = 0; j < n; j++) {
        for (int c = 0; c < 3; c++) KS(6, j, 3 + c) = derivs[3 * j + c];
        for (int c = 0; c < 3; c++)
            pos2[3 * j + c] =
                pos[3 * j + c] + h * (DPb1 * KS(0, j, c) + DPb3 * KS(2, j, c) +
                                      DPb4 * KS(3, j, c) + DPb5 * KS(4, j, c) +
                                      DPb6 * KS(5, j, c));
        for (int c = 0; c < 3; c++)
            vel2[3 * j + c] =
                vel[3 * j + c] + h * (DPb1 * KS(0, j, 3 + c) + DPb3 * KS(2, j, 3 + c) +
                                      DPb4 * KS(3, j, 3 + c) + DPb5 * KS(4, j, 3 + c) +
                                      DPb6 * KS(5, j, 3 + c));
    }
    /* embedded error, ode.cpp:189-215 */
    for (int j = 0; j < n; j++) {
        double yerr[6];
        for (int i = 0; i < 6; i++)
            yerr[i] = h * (DPe1 * KS(0, j, i) + DPe3 * KS(2, j, i) + DPe4 * KS(3, j, i) +
                           DPe5 * KS(4, j, i) + DPe6 * KS(5, j, i) + DPe7 * KS(6, j, i));
        for (int c = 0; c < 3; c++) {
            sk = cs->atol + cs->rtol * ref_max(fabs(pos[3 * j + c]), fabs(pos2[3 * j + c]));
            err = err + (yerr[c] / sk) * (yerr[c] / sk);
        }
        for (int c = 0; c < 3; c++) {
            sk = cs->atol + cs->rtol * ref_max(fabs(vel[3 * j + c]), fabs(vel2[3 * j + c]));
            err = err + (yerr[3 + c] / sk) * (yerr[3 + c] / sk);
        }
    }
    err = sqrt(err / (6 * n));
    cs->err = err;
    cs->force_evals += 7;
    return err;
}


/* ---------------------------------------------------------------------------
 * Cash-Karp 5(4), bin/ode.cpp:220-345 (the reference calls it RungaKutta4).
 * ------------------------------------------------------------------------- */
static const double RKb21 = 0.2, RKb31 = 3.0 / 40.0, RKb32 = 9.0 / 40.0, RKb41 = 0.3,
                    RKb42 = -0.9, RKb43 = 1.2, RKb51 = -11.0 / 54.0, RKb52 = 2.5,
                    RKb53 = -70.0 / 27.0, RKb54 = 35.0 / 27.0, RKb61 = 1631.0 / 55296.0,
                    RKb62 = 175.0 / 512.0, RKb63 = 575.0 / 13824.0, RKb64 = 44275.0 / 110592.0,
                    RKb65 = 253.0 / 4096.0, RKc1 = 37.0 / 378.0, RKc3 = 250.0 / 621.0,
                    RKc4 = 125.0 / 594.0, RKc6 = 512.0 / 1771.0;
#define RKdc5 (-277.00 / 14336.0)
#define RKdc1 (RKc1 - 2825.0 / 27648.0)
#define RKdc3 (RKc3 - 18575.0 / 48384.0)
#define RKdc4 (RKc4 - 13525.0 / 55296.0)
#define RKdc6 (RKc6 - 0.25)

double orc_ck45_attempt(int n, const double* pos, const double* vel, const double* mass,
                        const int* charge, const sg_field_params* fp, orc_ctrl* cs,
                        double* pos2, double* vel2, double* k, double* derivs) {
    const double h = cs->h;
    const int frozen = (fp->flags & SG_F_FROZEN_T) != 0;
    const double t0 = cs->t;
    /* stage times of the Cash-Karp nodes c = 0, 1/5, 3/10, 3/5, 1, 7/8 */
    const double cc[6] = {0.0, 0.2, 0.3, 0.6, 1.0, 0.875};
    double ts[6];
    for (int s = 0; s < 6; s++) ts[s] = frozen ? t0 : t0 + cc[s] * h;
    double err = cs->err;  /* not reset, as in the reference */
    double sk;
    for (int j = 0; j < n; j++) {
        KS(0, j, 0) = vel[3 * j + 0];
        KS(0, j, 1) = vel[3 * j + 1];
        KS(0, j, 2) = vel[3 * j + 2];
    }
    memcpy(pos2, pos, sizeof(double) * 3 * (size_t)n);
    memcpy(vel2, vel, sizeof(double) * 3 * (size_t)n);
    orc_force(n, pos2, vel2, mass, charge, ts[0], fp, derivs);
    for (int j = 0; j < n; j++) {
        for (int c = 0; c < 3; c++) KS(0, j, 3 + c) = derivs[3 * j + c];
        for (int c = 0; c < 3; c++) pos2[3 * j + c] = pos[3 * j + c] + h * (RKb21 * KS(0, j, c));
        for (int c = 0; c < 3; c++)
            KS(1, j, c) = vel2[3 * j + c] = vel[3 * j + c] + h * (RKb21 * KS(0, j, 3 + c));
    }
    orc_force(n, pos2, vel2, mass, charge, ts[1], fp, derivs);
    for (int j = 0; j < n; j++) {
        for (int c = 0; c < 3; c++) KS(1, j, 3 + c) = derivs[3 * j + c];
        for (int c = 0; c < 3; c++)
            pos2[3 * j + c] = pos[3 * j + c] + h * (RKb31 * KS(0, j, c) + RKb32 * KS(1, j, c));
        for (int c = 0; c < 3; c++)
            KS(2, j, c) = vel2[3 * j + c] =
                vel[3 * j + c] + h * (RKb31 * KS(0, j, 3 + c) + RKb32 * KS(1, j, 3 + c));
    }
    orc_force(n, pos2, vel2, mass, charge, ts[2], fp, derivs);
    for (int j = 0; j < n; j++) {
        for (int c = 0; c < 3; c++) KS(2, j, 3 + c) = derivs[3 * j + c];
        for (int c = 0; c < 3; c++)
            pos2[3 * j + c] = pos[3 * j + c] + h * (RKb41 * KS(0, j, c) + RKb42 * KS(1, j, c) +
                                                    RKb43 * KS(2, j, c));
        for (int c = 0; c < 3; c++)
            KS(3, j, c) = vel2[3 * j + c] =
                vel[3 * j + c] + h * (RKb41 * KS(0, j, 3 + c) + RKb42 * KS(1, j, 3 + c) +
                                      RKb43 * KS(2, j, 3 + c));
    }
    orc_force(n, pos2, vel2, mass, charge, ts[3], fp, derivs);
    for (int j = 0; j < n; j++) {
        for (int c = 0; c < 3; c++) KS(3, j, 3 + c) = derivs[3 * j + c];
        for (int c = 0; c < 3; c++)
            pos2[3 * j + c] = pos[3 * j + c] + h * (RKb51 * KS(0, j, c) + RKb52 * KS(1, j, c) +
                                                    RKb53 * KS(2, j, c) + RKb54 * KS(3, j, c));
        for (int c = 0; c < 3; c++)
            KS(4, j, c) = vel2[3 * j + c] =
                vel[3 * j + c] + h * (RKb51 * KS(0, j, 3 + c) + RKb52 * KS(1, j, 3 + c) +
                                      RKb53 * KS(2, j, 3 + c) + RKb54 * KS(3, j, 3 + c));
    }
    orc_force(n, pos2, vel2, mass, charge, ts[4], fp, derivs);
    for (int j = 0; j < n; j++) {
        for (int c = 0; c < 3; c++) KS(4, j, 3 + c) = derivs[3 * j + c];
        for (int c = 0; c < 3; c++)
            pos2[3 * j + c] =
                pos[3 * j + c] + h * (RKb61 * KS(0, j, c) + RKb62 * KS(1, j, c) +
                                      RKb63 * KS(2, j, c) + RKb64 * KS(3, j, c) +
                                      RKb65 * KS(4, j, c));
        for (int c = 0; c < 3; c++)
            KS(5, j, c) = vel2[3 * j + c] =
                vel[3 * j + c] + h * (RKb61 * KS(0, j, 3 + c) + RKb62 * KS(1, j, 3 + c) +
                                      RKb63 * KS(2, j, 3 + c) + RKb64 * KS(3, j, 3 + c) +
                                      RKb65 * KS(4, j, 3 + c));
    }
    orc_force(n, pos2, vel2, mass, charge, ts[5], fp, derivs);
    for (int j = 0; j < n; j++) {
        double yerr[6];
        for (int c = 0; c < 3; c++) KS(5, j, 3 + c) = derivs[3 * j + c];
        for (int c = 0; c < 3; c++)
            pos2[3 * j + c] = pos[3 * j + c] + h * (RKc1 * KS(0, j, c) + RKc3 * KS(2, j, c) +
                                                    RKc4 * KS(3, j, c) + RKc6 * KS(5, j, c));
        for (int c = 0; c < 3; c++)
            vel2[3 * j + c] = vel[3 * j + c] + h * (RKc1 * KS(0, j, 3 + c) + RKc3 * KS(2, j, 3 + c) +
                                                    RKc4 * KS(3, j, 3 + c) + RKc6 * KS(5, j, 3 + c));
        for (int i = 0; i < 6; i++)
            yerr[i] = h * (RKdc1 * KS(0, j, i) + RKdc3 * KS(2, j, i) + RKdc4 * KS(3, j, i) +
                           RKdc5 * KS(4, j, i) + RKdc6 * KS(5, j, i));
        for (int c = 0; c < 3; c++) {
            sk = cs->atol + cs->rtol * ref_max(fabs(pos[3 * j + c]), fabs(pos2[3 * j + c]));
            err = err + (yerr[c] / sk) * (yerr[c] / sk);
        }
        for (int c = 0; c < 3; c++) {
            sk = cs->atol + cs->rtol * ref_max(fabs(vel[3 * j + c]), fabs(vel2[3 * j + c]));
            err = err + (yerr[3 + c] / sk) * (yerr[3 + c] / sk);
        }
    }
    err = sqrt(err / (6 * n));
    cs->err = err;
    cs->force_evals += 6;
    return err;
}


/* GearMethod, bin/ode.cpp:347-424: fifth-order Gear predictor-corrector in Nordsieck
 * form, one force evaluation per step.  g holds [4][n][3]: the acceleration of the
 * last force call (odev.forcev.derivs), and b, c, d (odev.b/c/d).  hf = h^2/2, h^3/6,
 * h^4/24, h^5/120 as Init_ode computes them from the initial step (bin/ode.cpp:548-552).
 * The e terms of the reference are computed there but never read; they are left out. */
#define GEA0 (3.0 / 20.0)
#define GEA1 (251.0 / 360.0)
#define GEA3 (11.0 / 18.0)
#define GEA4 (1.0 / 6.0)
#define GEA5 (1.0 / 60.0)
#define GS(s, j, c) g[((size_t)(s) * n + (j)) * 3 + (c)]

void orc_gear_init(int n, double* g) {
    /* InitAcceleraction, bin/ode.cpp:36-59: constant seeds for every ion but the last,
     * whose entry the reference leaves as allocated; it is zero here.  b = c = d = 0
     * (std::vector value-initialised, bin/ode.cpp:599-630). */
    memset(g, 0, sizeof(double) * 12 * (size_t)n);
    for (int i = 0; i + 1 < n; i++) {
        GS(0, i, 0) = 1.6e9;
        GS(0, i, 1) = 1.1e9;
        GS(0, i, 2) = -5e8;
    }
}

void orc_gear_step(int n, const double* pos, const double* vel, const double* mass,
                   const int* charge, const sg_field_params* fp, orc_ctrl* cs, const double* hf,
                   double* pos2, double* vel2, double* g, double* derivs) {
    const double h = cs->h;
    const double h2f = hf[0], h3f = hf[1], h4f = hf[2], h5f = hf[3];
    const int frozen = (fp->flags & SG_F_FROZEN_T) != 0;
    for (int i = 0; i < n; i++)
        for (int c = 0; c < 3; c++) {
            pos2[3 * i + c] = pos[3 * i + c] + vel[3 * i + c] * h + GS(0, i, c) * h2f +
                              GS(1, i, c) * h3f + GS(2, i, c) * h4f + GS(3, i, c) * h5f;
            vel2[3 * i + c] = vel[3 * i + c] + GS(0, i, c) * h + GS(1, i, c) * h2f +
                              GS(2, i, c) * h3f + GS(3, i, c) * h4f;
        }
    orc_force(n, pos2, vel2, mass, charge, frozen ? cs->t : cs->t + h, fp, derivs);
    for (int i = 0; i < n; i++)
        for (int c = 0; c < 3; c++) {
            const double a = GS(0, i, c), b = GS(1, i, c), cc = GS(2, i, c), d = GS(3, i, c);
            const double sug = a + b * h + cc * h2f + d * h3f;
            const double bn = b + cc * h + d * h2f;
            const double cn = cc + d * h;
            const double ad = h2f * (derivs[3 * i + c] - sug);
            pos2[3 * i + c] += GEA0 * ad;
            vel2[3 * i + c] += GEA1 * ad / h;
            GS(0, i, c) = derivs[3 * i + c];
            GS(1, i, c) = bn + GEA3 * ad / h3f;
            GS(2, i, c) = cn + GEA4 * ad / h4f;
            GS(3, i, c) = d + GEA5 * ad / h5f;
        }
    cs->err = 0.0;
    cs->force_evals += 1;
}
#undef GS

/* error_succes, bin/ode.cpp:426-457 (alpha = 0.2 - 0.75 beta, safe = 0.9,
 * minscale = 0.2, maxscale = 10).  The reference compiles beta = 0 (the I-controller,
 * :431) and recommends 0.04-0.08 for PI control (:428, :433); beta comes from the
 * controller state here. */
int orc_error_succes(double err, orc_ctrl* c) {
    const double beta = c->beta, alpha = 0.2 - beta * 0.75, safe = 0.9, minscale = 0.2,
                 maxscale = 10.0;
    double scale;
    if (err <= 1.0) {
        if (err == 0.0)
            scale = maxscale;
        else {
            scale = safe * pow(err, -alpha) * pow(c->errold, beta);
            if (scale < minscale) scale = minscale;
            if (scale > maxscale) scale = maxscale;
        }
        if (c->reject)
            c->hnext = c->h * ref_min(scale, 1.0);
        else
            c->hnext = c->h * scale;
        c->errold = ref_max(err, 1.0e-4);
        c->reject = 0;
        return 1;
    } else {
        scale = ref_max(safe * pow(err, -alpha), minscale);
        c->h *= scale;
        c->reject = 1;
        return 0;
    }
}

/* step, bin/ode.cpp:459-494, driven as move_particles does (bin/ion_fly.cpp:83-101):
 * while lifetime < endtime: step().  A non-finite error norm stops with
 * SG_NONFINITE (the reference would keep shrinking h by NaN). */
int64_t orc_dp45_run(int n, double* pos, double* vel, const double* mass,
                     const int* charge, const sg_field_params* fp, orc_ctrl* c,
                     int64_t max_steps, double* hist, int64_t hist_cap) {
    return orc_rk_run(5, n, pos, vel, mass, charge, fp, c, max_steps, hist, hist_cap);
}

int64_t orc_rk_run(int method, int n, double* pos, double* vel, const double* mass,
                   const int* charge, const sg_field_params* fp, orc_ctrl* c,
                   int64_t max_steps, double* hist, int64_t hist_cap) {
    double* k = (double*)malloc(sizeof(double) * 7 * 6 * (size_t)n);
    double* pos2 = (double*)malloc(sizeof(double) * 3 * (size_t)n);
    double* vel2 = (double*)malloc(sizeof(double) * 3 * (size_t)n);
    double* derivs = (double*)malloc(sizeof(double) * 3 * (size_t)n);
    int64_t nh = 0;
    int64_t done_steps = 0;
    /* Gear: step powers fixed at the initial step (bin/ode.cpp:548-552).  The reference
     * is C++98 code, where pow(double, int) is std::pow's integer overload, evaluated by
     * repeated multiplication: h^3 = h^2 h, h^4 = h^2 h^2, h^5 = h^3 h^2. */
    const double h1 = c->h, h2 = h1 * h1, h3 = h2 * h1;
    const double hf[4] = {h1 * h1 / 2., h3 / 6., h2 * h2 / 24., h3 * h2 / 120.};
    c->status = SG_OK;
    if (!k || !pos2 || !vel2 || !derivs) {
        free(k); free(pos2); free(vel2); free(derivs);
        return -SG_BAD_ARG;
    }
    if (method == 1) orc_gear_init(n, k);
    while (done_steps < max_steps && c->t < c->t_end) {
        int rejects_here = 0;
        for (;;) {
            double tstart = c->t, hs = c->h;
            if (method == 1) {
                /* step() turns error control off for Gear (bin/ode.cpp:473-476) */
                orc_gear_step(n, pos, vel, mass, charge, fp, c, hf, pos2, vel2, k, derivs);
                c->attempts++;
                c->hnext = c->h;
                if (hist && nh < hist_cap) {
                    hist[4 * nh + 0] = tstart;
                    hist[4 * nh + 1] = hs;
                    hist[4 * nh + 2] = 0.0;
                    hist[4 * nh + 3] = 1.0;
                }
                nh++;
                break;
            }
            double err = method == 4
                             ? orc_ck45_attempt(n, pos, vel, mass, charge, fp, c, pos2, vel2, k, derivs)
                             : orc_dp45_attempt(n, pos, vel, mass, charge, fp, c, pos2, vel2, k, derivs);
            int acc = 1;
            if (!isfinite(err)) {
                c->status = SG_NONFINITE;
                acc = 0;
            } else if (c->adaptive) {
                c->attempts++;
                acc = orc_error_succes(err, c);
                if (!acc) {
                    c->rejects++;
                    rejects_here++;
                    if (fabs(c->h) <= fabs(pos[0]) * DBL_EPSILON) c->status = SG_H_UNDERFLOW;
                    else if (c->max_rejects > 0 && rejects_here >= c->max_rejects)
                        c->status = SG_TOO_MANY_REJECTS;
                }
            } else {
                c->attempts++;
            }
            if (hist && nh < hist_cap) {
                hist[4 * nh + 0] = tstart;
                hist[4 * nh + 1] = hs;
                hist[4 * nh + 2] = err;
                hist[4 * nh + 3] = acc;
            }
            nh++;
            if (c->status != SG_OK) goto out;
            if (acc) break;
        }
        memcpy(pos, pos2, sizeof(double) * 3 * (size_t)n);
        memcpy(vel, vel2, sizeof(double) * 3 * (size_t)n);
        c->t = c->t + c->h;
        c->h = c->hnext;
        c->steps++;
        done_steps++;
    }
out:
    free(k); free(pos2); free(vel2); free(derivs);
    if (c->status != SG_OK) return -(int64_t)c->status;
    return nh;
}

int orc_dp45_replay(int n, double* pos, double* vel, const double* mass, const int* charge,
                    const sg_field_params* fp, const double* ts, const double* hs, int nsteps) {
    return orc_rk_replay(5, n, pos, vel, mass, charge, fp, ts, hs, nsteps);
}

int orc_rk_replay(int method, int n, double* pos, double* vel, const double* mass,
                  const int* charge, const sg_field_params* fp, const double* ts,
                  const double* hs, int nsteps) {
    double* k = (double*)malloc(sizeof(double) * 7 * 6 * (size_t)n);
    double* pos2 = (double*)malloc(sizeof(double) * 3 * (size_t)n);
    double* vel2 = (double*)malloc(sizeof(double) * 3 * (size_t)n);
    double* derivs = (double*)malloc(sizeof(double) * 3 * (size_t)n);
    if (!k || !pos2 || !vel2 || !derivs) {
        free(k); free(pos2); free(vel2); free(derivs);
        return SG_BAD_ARG;
    }
    orc_ctrl c;
    memset(&c, 0, sizeof c);
    c.rtol = 1e-9;
    c.atol = 1e-15;
    for (int s = 0; s < nsteps; s++) {
        c.t = ts[s];
        c.h = hs[s];
        if (method == 4)
            orc_ck45_attempt(n, pos, vel, mass, charge, fp, &c, pos2, vel2, k, derivs);
        else
            orc_dp45_attempt(n, pos, vel, mass, charge, fp, &c, pos2, vel2, k, derivs);
        memcpy(pos, pos2, sizeof(double) * 3 * (size_t)n);
        memcpy(vel, vel2, sizeof(double) * 3 * (size_t)n);
    }
    free(k); free(pos2); free(vel2); free(derivs);
    return SG_OK;
}

/* Cloud moments.  Temperature restates IonCloud::Temperature (bin/ioncloud.cpp:316-335):
 * T_r = (0.5/N sum m (vx^2+vy^2)) * 2/(3 kb), T_z = (0.5/N sum m vz^2) * 2/(3 kb). */
void orc_moments(int n, const double* pos, const double* vel, const double* mass,
                 double* out) {
    double s[3] = {0, 0, 0}, s2[3] = {0, 0, 0}, v2[3] = {0, 0, 0};
    double er = 0.0, ez = 0.0;
    for (int i = 0; i < n; i++) {
        for (int c = 0; c < 3; c++) {
            double x = pos[3 * i + c], v = vel[3 * i + c];
            s[c] += x;
            s2[c] += x * x;
            v2[c] += v * v;
        }
        er += mass[i] * (vel[3 * i + 0] * vel[3 * i + 0] + vel[3 * i + 1] * vel[3 * i + 1]);
        ez += mass[i] * (vel[3 * i + 2] * vel[3 * i + 2]);
    }
    for (int c = 0; c < 3; c++) {
        double m = n ? s[c] / n : 0.0;
        out[c] = m;
        double var = n ? s2[c] / n - m * m : 0.0;
        out[3 + c] = var > 0 ? sqrt(var) : 0.0;
        out[6 + c] = n ? v2[c] / n : 0.0;
    }
    if (n) {
        er *= (0.5 / n);
        ez *= (0.5 / n);
    }
    out[9] = er * (2.0 / (3.0 * ORC_KB));
    out[10] = ez * (2.0 / (3.0 * ORC_KB));
    out[11] = n;
}

/* PrintCloud statistics (bin/ioncloud.cpp:148-183) per species s (ions with
 * species[i] == s): out[9 s + 0..8] = centroid x0, y0, z0 (m), spread x1, y1, z1 (m),
 * energy (eV), ions of the species, ions of the cloud.  The reference's arithmetic is
 * kept as it is: the centroid and the spread divide by the number of ions of the whole
 * cloud, and the energy sums m (vx^2 + vy^2 + vz vy) / 2. */
void orc_cloud_stats(int n, const double* pos, const double* vel, const double* mass,
                     const int* species, int n_species, double* out) {
    const double j_to_ev = 6.24150e18; /* bin/globals.h:9 */
    for (int s = 0; s < n_species; s++) {
        double x0 = 0, y0 = 0, z0 = 0, x1 = 0, y1 = 0, z1 = 0, energy = 0.0;
        int count = 0;
        for (int i = 0; i < n; i++)
            if (species[i] == s) {
                x0 += pos[3 * i];
                y0 += pos[3 * i + 1];
                z0 += pos[3 * i + 2];
                energy += 0.5 * j_to_ev * mass[i] *
                          (vel[3 * i] * vel[3 * i] + vel[3 * i + 1] * vel[3 * i + 1] +
                           vel[3 * i + 2] * vel[3 * i + 1]);
                count++;
            }
        x0 /= n;
        y0 /= n;
        z0 /= n;
        for (int i = 0; i < n; i++)
            if (species[i] == s) {
                x1 += (pos[3 * i] - x0) * (pos[3 * i] - x0);
                y1 += (pos[3 * i + 1] - y0) * (pos[3 * i + 1] - y0);
                z1 += (pos[3 * i + 2] - z0) * (pos[3 * i + 2] - z0);
            }
        double* o = out + 9 * s;
        o[0] = x0;
        o[1] = y0;
        o[2] = z0;
        o[3] = sqrt(x1 / n);
        o[4] = sqrt(y1 / n);
        o[5] = sqrt(z1 / n);
        o[6] = energy;
        o[7] = count;
        o[8] = n;
    }
}
