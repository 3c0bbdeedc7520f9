/*
 * ref_harness.cpp -- drives the reference Simbuca CPU path, compiled from its own
 * sources (oracle/Makefile), through a small extern "C" surface so that tests can
 * generate golden vectors with it.  TEST INFRASTRUCTURE ONLY: built into
 * oracle/_ref/, never linked by the product.
 *
 * Set-up follows what move_particles does on its first call
 * (bin/ion_fly.cpp:26-62): Init_ode, Initpoolvectors, InitializePoolVectors,
 * CopyParticlesToVectors, coulomb flags; ions are added with IonCloud::AddParticle
 * (bin/ion_fly.cpp:139-142) with their mass given in kg directly.
 */
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <unistd.h>

#include "force.h"
#include "ioncloud.h"
#include "ode.h"

/* defined at global scope in bin/ode.cpp:61 and :426 */
double Dormand_Prince_5(IonCloud& _cloud, _ode_vars& odev);
double RungaKutta4(IonCloud& _cloud, _ode_vars& odev);
void GearMethod(IonCloud& _cloud, _ode_vars& odev);
bool error_succes(const double err, _ode_vars& odev);

namespace {

struct RefRun {
    IonCloud cloud;
    _ode_vars odev;
    std::string prefix;
};

/* trap: Vrf, Vdc, kappa, r0, z0, freq_rf, E_kick */
void setup(RefRun& r, int n, const double* pos, const double* vel, const double* mass,
           const int* charge, int trap, int tof, int coulomb, double coulomb_scale,
           const double* trapp, double t0, double h0, int adaptive, double rtol,
           double atol, int method = 5) {
    char tmpl[] = "/tmp/simgb_refXXXXXX";
    char* dir = mkdtemp(tmpl);
    r.prefix = std::string(dir ? dir : "/tmp") + "/run";
    r.cloud.Create(r.prefix.c_str());
    r.cloud.use_particles_files(false);
    for (int i = 0; i < n; i++) {
        Ion ion;
        ion.mass = (long double)mass[i];
        ion.charge = charge[i];
        ion.SetName("ion");
        Particle p(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], vel[3 * i], vel[3 * i + 1],
                   vel[3 * i + 2]);
        r.cloud.AddParticle(p, ion);
    }
    r.odev.Init_ode(method, h0, adaptive != 0);
    r.odev.err = 0.0;  // the Cash-Karp error sum starts from the previous norm
    r.odev.rk_rtol = rtol;
    r.odev.rk_atol = atol;
    r.odev.Initpoolvectors(n);
    // InitAcceleraction leaves the last ion's initial acceleration as allocated; zero it
    // so that Gear runs are defined (the Runge-Kutta methods overwrite it before use)
    memset(r.odev.forcev.derivs, 0, sizeof(double) * 3 * (size_t)n);
    r.cloud.InitializePoolVectors();
    r.cloud.CopyParticlesToVectors();
    r.odev.forcev.coulomb_interaction = coulomb != 0;
    r.odev.forcev.coulomb_scale = coulomb_scale;
    r.odev.forcev.trap = trap != 0;
    r.odev.forcev.tof = tof != 0;
    r.odev.forcev.trap_param.Vrf = trapp[0];
    r.odev.forcev.trap_param.Vdc = trapp[1];
    r.odev.forcev.trap_param.kappa = trapp[2];
    r.odev.forcev.trap_param.r0 = trapp[3];
    r.odev.forcev.trap_param.z0 = trapp[4];
    r.odev.forcev.trap_param.freq_rf = trapp[5];
    r.odev.forcev.trap_param.E_kick = trapp[6];
    r.cloud.lifetime = t0;
    r.odev.time_start_op = t0;
}

void teardown(RefRun& r) {
    if (r.cloud.globalstream) {
        r.cloud.globalstream->close();
        delete r.cloud.globalstream;
        r.cloud.globalstream = NULL;
    }
    for (size_t k = 0; k < r.cloud.cloud_stream.size(); k++) {
        r.cloud.cloud_stream[k]->close();
        delete r.cloud.cloud_stream[k];
    }
    r.cloud.cloud_stream.clear();
    std::string a = r.prefix + "_pAll.txt", b = r.prefix + "_cloud0.txt";
    unlink(a.c_str());
    unlink(b.c_str());
    std::string d = r.prefix.substr(0, r.prefix.rfind('/'));
    rmdir(d.c_str());
    for (size_t k = 0; k < r.cloud.particles.size(); k++) delete r.cloud.particles[k];
    r.cloud.particles.clear();
    delete r.cloud.ions;
    r.cloud.ions = NULL;
}

}  // namespace

extern "C" {

/* force() on the given state: out = odev.forcev.derivs (bin/force.cpp:34-178). */
int ref_force(int n, const double* pos, const double* vel, const double* mass,
              const int* charge, double t, int trap, int tof, int coulomb,
              double coulomb_scale, const double* trapp, double* out) {
    RefRun* r = new RefRun;
    setup(*r, n, pos, vel, mass, charge, trap, tof, coulomb, coulomb_scale, trapp, t, 1e-9,
          1, 1e-7, 1e-7);
    force(r->cloud, r->odev);
    memcpy(out, r->odev.forcev.derivs, sizeof(double) * 3 * (size_t)n);
    teardown(*r);
    delete r;
    return 0;
}

/* Integrator run, method 5 = Dormand-Prince, 4 = Cash-Karp, 1 = Gear (Init_ode's order).
 * mode 0: call the reference step() (bin/ode.cpp:459-494)
 * until lifetime >= t_end or max_steps steps; mode 1: the same loop written out
 * with the reference's Dormand_Prince_5 and error_succes so each attempt can be
 * recorded as (t_start, h, err, accepted) in hist.  ctrl_out receives
 * (t, h, hnext, errold, reject, steps, attempts).  Returns attempts recorded, or
 * -3 when step() threw its underflow exception. */
long long ref_dp45_run(int n, double* pos, double* vel, const double* mass,
                       const int* charge, int trap, int tof, int coulomb,
                       double coulomb_scale, const double* trapp, double t0, double t_end,
                       double h0, int adaptive, double rtol, double atol, long long max_steps,
                       int mode, double* hist, long long hist_cap, double* ctrl_out,
                       int method) {
    RefRun* r = new RefRun;
    setup(*r, n, pos, vel, mass, charge, trap, tof, coulomb, coulomb_scale, trapp, t0, h0,
          adaptive, rtol, atol, method);
    IonCloud& cl = r->cloud;
    _ode_vars& od = r->odev;
    long long nh = 0, steps = 0;
    long long ret = 0;
    try {
        while (cl.lifetime < t_end && steps < max_steps) {
            if (mode == 0) {
                step(cl, od);
            } else {
                for (;;) {
                    double ts = cl.lifetime, hs = od.h;
                    double err = 0.0;
                    if (method == 1) {
                        GearMethod(cl, od);
                        od.change_stepsize = false;  // as step() does for Gear
                    } else {
                        err = method == 4 ? RungaKutta4(cl, od) : Dormand_Prince_5(cl, od);
                    }
                    bool acc = true;
                    if (od.change_stepsize) {
                        od.countstep++;
                        acc = error_succes(err, od);
                    }
                    if (hist && nh < hist_cap) {
                        hist[4 * nh + 0] = ts;
                        hist[4 * nh + 1] = hs;
                        hist[4 * nh + 2] = err;
                        hist[4 * nh + 3] = acc ? 1.0 : 0.0;
                    }
                    nh++;
                    if (acc) break;
                    if (fabs(od.h) <= fabs(cl.pos[0][0]) * od.EPS) throw("stepsize underflow created");
                }
                memcpy(cl.pos, cl.pos2, sizeof(double) * 3 * n);
                memcpy(cl.vel, cl.vel2, sizeof(double) * 3 * n);
                cl.lifetime = cl.lifetime + od.h;
                od.h = od.hnext;
            }
            steps++;
        }
        ret = nh;
    } catch (const char*) {
        ret = -3;
    }
    memcpy(pos, cl.pos, sizeof(double) * 3 * (size_t)n);
    memcpy(vel, cl.vel, sizeof(double) * 3 * (size_t)n);
    if (ctrl_out) {
        ctrl_out[0] = cl.lifetime;
        ctrl_out[1] = od.h;
        ctrl_out[2] = od.hnext;
        ctrl_out[3] = od.errold;
        ctrl_out[4] = od.reject ? 1.0 : 0.0;
        ctrl_out[5] = (double)steps;
        ctrl_out[6] = (double)od.countstep;
    }
    teardown(*r);
    delete r;
    return ret;
}

/* PrintParticles + PrintCloud (bin/ioncloud.cpp:85-183) of the given state at lifetime t,
 * ions named names[species[i]].  The text of <prefix>_pAll.txt followed by each
 * <prefix>_cloud<k>.txt is copied into out (capacity cap bytes, NUL-terminated),
 * files separated by a line "@@<file name suffix>".  Returns the length written. */
long long ref_print(int n, const double* pos, const double* vel, const double* mass,
                    const int* charge, const int* species, const char* const* names,
                    int n_names, double t, char* out, long long cap) {
    RefRun* r = new RefRun;
    const double trapp[7] = {0, 0, 0, 1, 1, 0, 0};
    setup(*r, 0, pos, vel, mass, charge, 0, 0, 0, 1.0, trapp, t, 1e-9, 1, 1e-7, 1e-7);
    for (int i = 0; i < n; i++) {
        Ion ion;
        ion.mass = (long double)mass[i];
        ion.charge = charge[i];
        ion.SetName(names[species[i]]);
        Particle p(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], vel[3 * i], vel[3 * i + 1],
                   vel[3 * i + 2]);
        r->cloud.AddParticle(p, ion);
    }
    r->cloud.InitializePoolVectors();
    r->cloud.CopyParticlesToVectors();
    r->cloud.lifetime = t;
    r->cloud.PrintParticles();
    r->cloud.PrintCloud();
    r->cloud.globalstream->flush();
    for (size_t k = 0; k < r->cloud.cloud_stream.size(); k++) r->cloud.cloud_stream[k]->flush();
    long long len = 0;
    std::string files[64];
    int nf = 0;
    files[nf++] = "_pAll.txt";
    for (size_t k = 0; k < r->cloud.cloud_stream.size() && nf < 64; k++) {
        char b[32];
        snprintf(b, sizeof b, "_cloud%d.txt", (int)k);
        files[nf++] = b;
    }
    for (int f = 0; f < nf; f++) {
        std::string name = r->prefix + files[f];
        std::string head = "@@" + files[f] + "\n";
        if (len + (long long)head.size() < cap) {
            memcpy(out + len, head.data(), head.size());
            len += head.size();
        }
        FILE* fp = fopen(name.c_str(), "r");
        if (!fp) continue;
        char buf[4096];
        size_t got;
        while ((got = fread(buf, 1, sizeof buf, fp)) > 0)
            for (size_t i = 0; i < got && len + 1 < cap; i++) out[len++] = buf[i];
        fclose(fp);
        if (f > 0) unlink(name.c_str());
    }
    if (cap > 0) out[len < cap ? len : cap - 1] = 0;
    teardown(*r);
    delete r;
    (void)n_names;
    return len;
}

}  // extern "C"
