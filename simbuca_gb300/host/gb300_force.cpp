/*
 * gb300_force.cpp -- the __GB300_ON__ Coulomb backend of force(): one call of
 * libsimgb's sg_coulomb_accel on the stage positions, added to the field terms that
 * force() has already written.  See gb300_force.h for how it is wired in.
 */
#include "gb300_force.h"

#include <cstdlib>
#include <cstring>
#include <vector>

#include "simgb.h"

namespace {

sg_ctx* g_ctx = 0;
int g_precision = SG_PREC_FP32C;
std::vector<double> g_q, g_kq, g_acc;

}  // namespace

void gb300_coulomb(const IonCloud& _cloud, _ode_vars& odev) {
    const int n = _cloud.nrparticles;
    if (n <= 0) return;
    if (!g_ctx) {
        if (sg_create(0, &g_ctx) != SG_OK || !g_ctx) {
            g_ctx = 0;
            throw("gb300_coulomb: no usable CUDA device");
        }
        const char* p = std::getenv("SIMGB_FORCE_PRECISION");
        g_precision = (p && (!std::strcmp(p, "fp64") || !std::strcmp(p, "FP64")))
                          ? SG_PREC_FP64
                          : SG_PREC_FP32C;
    }
    _force_vars& forcev = odev.forcev;
    g_q.resize(n);
    g_kq.resize(n);
    g_acc.resize(3 * (size_t)n);
    for (int j = 0; j < n; j++) {
        // q_j as the CPU loop reads it for the source ion, and q_i/m_i for the target
        // in the factor order of bin/force.cpp:153
        g_q[j] = (double)(*_cloud.ions)[j].Getcharge();
        g_kq[j] = forcev.coulomb_scale * ke * el_charge * _cloud.charge[j] * el_charge /
                  _cloud.mass[j];
    }
    if (sg_coulomb_accel(g_ctx, g_precision, n, &_cloud.pos2[0][0], &g_q[0], &g_kq[0],
                         &g_acc[0]) != SG_OK)
        throw("gb300_coulomb: sg_coulomb_accel failed");
    for (int j = 0; j < n; j++)
        for (int c = 0; c < 3; c++) forcev.derivs[j][c] += g_acc[3 * (size_t)j + c];
}

void gb300_release() {
    if (g_ctx) sg_destroy(g_ctx);
    g_ctx = 0;
}
