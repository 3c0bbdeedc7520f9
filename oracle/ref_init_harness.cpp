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
#include "ioncloud.h"
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
