/*
 * gb300_force.h -- the __GB300_ON__ Coulomb backend of Simbuca's force()
 * (bin/force.cpp:34-178), for the reference's own C++ host.
 *
 * Compiled together with the reference's sources (it includes their ode.h, which
 * declares IonCloud and _ode_vars).  force() keeps its signature (bin/force.h:6); the
 * only edit to bin/force.cpp is one more branch of its backend ladder, beside the
 * CUNBODY and NBODY ones (bin/force.cpp:84-105), after the field loop:
 *
 *     #ifdef __GB300_ON__
 *         gb300_coulomb(_cloud, odev);
 *     #endif
 *
 * plus -D__GB300_ON__, this directory and include/ on the include path, this file's
 * .cpp among the objects, and libsimgb.so on the link line.
 */
#ifndef GB300_FORCE_H
#define GB300_FORCE_H

#include "ode.h"

/* Adds the Coulomb term of every ion to odev.forcev.derivs (accelerations, m/s^2):
 * coulomb_scale k_e e^2 q_i/m_i sum_{j!=i} q_j (x_i-x_j)/|x_i-x_j|^3 at _cloud.pos2,
 * the charge-aware, unsoftened sum of the CPU path (bin/force.cpp:147-174).  The GPU
 * context is created on the first call (device 0).  SIMGB_FORCE_PRECISION=fp64 in the
 * environment selects the plain FP64 form; the default is the FP32-compensated one.
 * Throws a const char* on failure, as the reference's own error paths do
 * (bin/ode.cpp:483). */
void gb300_coulomb(const IonCloud& _cloud, _ode_vars& odev);

/* Frees the GPU context (optional; the process exit frees it too). */
void gb300_release();

#endif
