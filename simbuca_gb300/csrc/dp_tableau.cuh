// dp_tableau.cuh -- the Dormand-Prince 5(4) tableau of the reference (bin/ode.cpp:76-86)
// in constant memory, shared by the tiled stage kernels (dp45.cu) and the fused
// small-cloud kernel (fused.cu): a, c and e = b - b* (the embedded error weights).
#pragma once

#include <cuda_runtime.h>

namespace {

// Tableau of bin/ode.cpp:76-86.
__constant__ double c_a[8][7] = {
    {0, 0, 0, 0, 0, 0, 0},
    {0, 0, 0, 0, 0, 0, 0},
    {1.0 / 5.0, 0, 0, 0, 0, 0, 0},
    {3.0 / 40.0, 9.0 / 40.0, 0, 0, 0, 0, 0},
    {44.0 / 45.0, -56.0 / 15.0, 32.0 / 9.0, 0, 0, 0, 0},
    {19372.0 / 6561.0, -25360.0 / 2187.0, 64448.0 / 6561.0, -212.0 / 729.0, 0, 0, 0},
    {9017.0 / 3168.0, -355.0 / 33.0, 46732.0 / 5247.0, 49.0 / 176.0, -5103.0 / 18656.0, 0, 0},
    {35.0 / 384.0, 0.0, 500.0 / 1113.0, 125.0 / 192.0, -2187.0 / 6784.0, 11.0 / 84.0, 0}};
__constant__ double c_c[8] = {0, 0.0, 1.0 / 5.0, 3.0 / 10.0, 4.0 / 5.0, 8.0 / 9.0, 1.0, 1.0};
// e = b - b* (bin/ode.cpp:85-86); index by stage 1..7
__constant__ double c_e[8] = {0,
                              71.0 / 57600.0,
                              0.0,
                              -71.0 / 16695.0,
                              71.0 / 1920.0,
                              -17253.0 / 339200.0,
                              22.0 / 525.0,
                              -1.0 / 40.0};

}  // namespace
