// Initial-cloud generator of the reference (InitCloud, bin/initialization.cpp:117-206):
// positions uniform in an ellipsoid by rejection from the unit cube, speeds from the
// reference's Maxwell-Boltzmann law around the energy of the distribution's maximum
// (after Petersson, ISCOOL), directions uniform on the sphere.
//
// The random stream is the 32-bit Mersenne Twister MT19937 (Matsumoto & Nishimura,
// ACM TOMACS 8(1), 1998), seeded by its published 32-bit initialisation; a double is
// the 32-bit output times 2^-32 in [0, 1), as the reference's MTRand (bin/mtrand.h:
// 102-104) returns it.  Rejection sampling consumes a data-dependent number of draws,
// so the stream is inherently sequential: this runs on the host, once per cloud, and
// writes AoS arrays ready for sg_batch_upload.
#include <cmath>
#include <cstdint>
#include <cstring>

#include "../../include/simgb.h"
#include "sg_mt19937.h"

namespace {

// bin/globals.h:4,11 (pi, eV_to_Joule)
constexpr double kPi = 3.14159265358979323;
constexpr double kEvToJoule = 1.60217646e-19;

}  // namespace

extern "C" int sg_init_cloud(int n, const double* ev_max, int n_ev, uint32_t seed,
                             const double* semiaxis, const double* offset, const double* mass,
                             double* pos, double* vel) {
    if (n < 0 || (n > 0 && (!ev_max || !semiaxis || !offset || !mass || !pos || !vel)))
        return SG_BAD_ARG;
    if (n_ev != 1 && n_ev != 2) return SG_BAD_ARG;
    SgMt19937 rng(seed);
    for (int i = 0; i < n; i++) {
        double u[3];
        for (;;) {
            for (int c = 0; c < 3; c++) u[c] = rng.uniform() * 2. - 1.;
            if (u[0] * u[0] + u[1] * u[1] + u[2] * u[2] <= 1) break;
        }
        for (int c = 0; c < 3; c++) pos[3 * (size_t)i + c] = offset[c] + semiaxis[c] * u[c];
        const double m = mass[i];
        const double theta = rng.uniform() * 2.0 * kPi;
        const double phi = std::acos(rng.uniform() * 2.0 - 1.0);
        // speed whose distribution peaks at ev_max (radial part; axial from ev_max[1])
        double v = std::sqrt(-2.0 * (ev_max[0] * kEvToJoule) / m * std::log(1 - std::sqrt(rng.uniform())));
        vel[3 * (size_t)i + 0] = v * std::cos(theta) * std::sin(phi);
        vel[3 * (size_t)i + 1] = v * std::sin(theta) * std::sin(phi);
        if (n_ev == 2)
            v = std::sqrt(-2.0 * (ev_max[1] * kEvToJoule) / m * std::log(1 - std::sqrt(rng.uniform())));
        vel[3 * (size_t)i + 2] = v * std::cos(phi);
    }
    return SG_OK;
}
