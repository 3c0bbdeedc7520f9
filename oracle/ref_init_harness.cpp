/*
 * ref_init_harness.cpp -- runs the reference's InitCloud (bin/initialization.cpp:117-206)
 * through a small extern "C" surface, for golden vectors of the initial-cloud
 * generator.  TEST INFRASTRUCTURE ONLY: built into oracle/_ref/ (make ref-init) from
 * the reference's own sources, never linked by the product.
 *
 * initialization.cpp loads the mass tables at static-initialisation time from
 * ../libraries/ relative to the working directory (bin/initialization.cpp:34-35), so
 * the library must be loaded from the reference's bin/ directory.
 */
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <unistd.h>
#include <vector>

#include "initialization.h"
#include "ion_fly.h"
#include "ioncloud.h"
#include "operation.h"
#include "trapparameters.h"

void InitCloud(int nparticles, std::vector<double> eV_max_boltz, int seed, double semiaxis[3],
               double offset[3], std::vector<Ion> Ions, IonCloud& _cloud,
               _trap_param& trap_param);

extern "C" int ref_init_cloud(int n, const double* ev, int n_ev, int seed, const double* semi,
                              const double* off, const double* mass, const int* charge,
                              double* pos, double* vel) {
    char tmpl[] = "/tmp/simgb_refinitXXXXXX";
    char* dir = mkdtemp(tmpl);
    std::string prefix = std::string(dir ? dir : "/tmp") + "/run";
    IonCloud* cl = new IonCloud;
    cl->Create(prefix.c_str());
    cl->use_particles_files(false);
    std::vector<Ion> ions(n);
    for (int i = 0; i < n; i++) {
        ions[i].mass = (long double)mass[i];
        ions[i].charge = charge[i];
        ions[i].SetName("ion");
    }
    std::vector<double> e(ev, ev + n_ev);
    double s[3] = {semi[0], semi[1], semi[2]}, o[3] = {off[0], off[1], off[2]};
    _trap_param tp;
    InitCloud(n, e, seed, s, o, ions, *cl, tp);
    cl->InitializePoolVectors();
    cl->CopyParticlesToVectors();
    memcpy(pos, cl->pos, sizeof(double) * 3 * (size_t)n);
    memcpy(vel, cl->vel, sizeof(double) * 3 * (size_t)n);
    std::string a = prefix + "_pAll.txt";
    unlink(a.c_str());
    if (dir) rmdir(dir);
    return cl->nrparticles;
}

/* The reference's operation sequence (operations::launch, bin/operation.cpp:111-124)
 * on a Paul-trap cloud with a fixed Runge-Kutta step (Init_ode order `order`):
 * ops kinds 0 normal, 1 tof, 2 trap_ramp, 3 free flight ("nop").  As its INI parser
 * does (bin/initialization.cpp:520-552), the trap-ramp targets and the TOF kick are
 * trap parameters set once, here from the last ramp/TOF operation.  Set-up follows
 * DoSimulation: InitIonFly, print interval, Coulomb switch, ions, trap parameters.
 * out: pos, vel (AoS), then lifetime, Vrf, Vdc.  Uses the reference's globals
 * (firstoperation, print_interval): one call per process. */
extern "C" int ref_ops_run(int n, const double* pos, const double* vel, const double* mass,
                           const int* charge, const double* trapp, int coulomb, double h0,
                           int order, int n_ops, const int* kinds, const double* durations,
                           const double* new_vrf, const double* new_vdc, const double* e_kick,
                           double* pos_out, double* vel_out, double* t_out) {
    char tmpl[] = "/tmp/simgb_refopsXXXXXX";
    char* dir = mkdtemp(tmpl);
    std::string prefix = std::string(dir ? dir : "/tmp") + "/run";
    IonCloud* cl = new IonCloud;
    _ode_vars* od = new _ode_vars;
    InitIonFly(prefix.c_str(), order, h0, false, *cl, *od);
    cl->use_particles_files(false);
    SetPrintInterval(1e9);
    SetCoulomb(coulomb != 0);
    UseScaledCoulomb(1.0);
    for (int i = 0; i < n; i++) {
        Ion ion;
        ion.mass = (long double)mass[i];
        ion.charge = charge[i];
        ion.SetName("ion");
        AddParticle(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], vel[3 * i], vel[3 * i + 1],
                    vel[3 * i + 2], ion, *cl);
    }
    _trap_param& tp = od->forcev.trap_param;
    tp.Vrf = trapp[0];
    tp.Vdc = trapp[1];
    tp.kappa = trapp[2];
    tp.r0 = trapp[3];
    tp.z0 = trapp[4];
    tp.freq_rf = trapp[5];
    tp.E_kick = trapp[6];
    operations ops;
    for (int k = 0; k < n_ops; k++) {
        static const char* names[4] = {"normal", "tof", "trap_ramp", "nop"};
        operation op(names[kinds[k]]);
        op.time = durations[k];
        op.print_time = 0.0;
        op.timestep = 0.0;
        if (kinds[k] == 1) tp.E_kick = e_kick[k];
        if (kinds[k] == 2) {
            tp.newVrf = new_vrf[k];
            tp.newVdc = new_vdc[k];
        }
        ops.add(op);
    }
    ops.launch(*cl, *od);
    memcpy(pos_out, cl->pos, sizeof(double) * 3 * (size_t)n);
    memcpy(vel_out, cl->vel, sizeof(double) * 3 * (size_t)n);
    t_out[0] = cl->lifetime;
    t_out[1] = tp.Vrf;
    t_out[2] = tp.Vdc;
    std::string a = prefix + "_pAll.txt";
    unlink(a.c_str());
    std::string b = prefix + "_cloud0.txt";
    unlink(b.c_str());
    if (dir) rmdir(dir);
    return 0;
}
