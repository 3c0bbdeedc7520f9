/*
 * gb300_force_check.cpp -- TEST INFRASTRUCTURE ONLY.  Links the __GB300_ON__ backend
 * of force() (simbuca_gb300/host/gb300_force.cpp) with the reference's own objects
 * and libsimgb.so, so that the backend is compiled against the reference's headers
 * and cannot drift from them.  Run, it builds a small cloud, evaluates the Coulomb
 * term once through the reference's CPU loop (force() with the CPU backend) and once
 * through gb300_coulomb, and prints the largest per-ion relative difference; with no
 * usable GPU it prints the backend's error and exits with status 3.
 */
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <unistd.h>

#include "force.h"
#include "gb300_force.h"
#include "ioncloud.h"
#include "ode.h"

int main() {
    const int n = 64;
    char tmpl[] = "/tmp/simgb_gbfXXXXXX";
    char* dir = mkdtemp(tmpl);
    std::string prefix = std::string(dir ? dir : "/tmp") + "/run";
    IonCloud cloud;
    cloud.Create(prefix.c_str());
    cloud.use_particles_files(false);
    srand(7);
    for (int i = 0; i < n; i++) {
        Ion ion;
        ion.mass = (long double)(132.905 * amu);
        ion.charge = 1 + (i % 3 == 0);
        ion.SetName("ion");
        double r[3];
        for (int c = 0; c < 3; c++) r[c] = 1e-3 * ((double)rand() / RAND_MAX - 0.5);
        Particle p(r[0], r[1], r[2], 0.0, 0.0, 0.0);
        cloud.AddParticle(p, ion);
    }
    _ode_vars odev;
    odev.Init_ode(5, 1e-9, true);
    odev.Initpoolvectors(n);
    cloud.InitializePoolVectors();
    cloud.CopyParticlesToVectors();
    odev.forcev.trap = false;
    odev.forcev.tof = false;
    odev.forcev.coulomb_scale = 1.0;
    for (int i = 0; i < n; i++)
        for (int c = 0; c < 3; c++) {
            cloud.pos2[i][c] = cloud.pos[i][c];
            cloud.vel2[i][c] = cloud.vel[i][c];
        }
    odev.forcev.coulomb_interaction = true;
    force(cloud, odev);  // the reference's CPU Coulomb loop
    std::vector<double> ref(3 * n);
    for (int i = 0; i < n; i++)
        for (int c = 0; c < 3; c++) ref[3 * i + c] = odev.forcev.derivs[i][c];
    odev.forcev.coulomb_interaction = false;
    force(cloud, odev);  // field terms only (none here): derivs = 0
    try {
        gb300_coulomb(cloud, odev);
    } catch (const char* e) {
        std::printf("%s\n", e);
        return 3;
    }
    double worst = 0.0;
    for (int i = 0; i < n; i++) {
        double d2 = 0.0, r2 = 0.0;
        for (int c = 0; c < 3; c++) {
            const double d = odev.forcev.derivs[i][c] - ref[3 * i + c];
            d2 += d * d;
            r2 += ref[3 * i + c] * ref[3 * i + c];
        }
        const double e = std::sqrt(d2 / r2);
        if (e > worst) worst = e;
    }
    gb300_release();
    std::printf("max per-ion relative difference %.3e\n", worst);
    return worst <= 1e-6 ? 0 : 1;
}
