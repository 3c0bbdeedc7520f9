/*
 * ref_compat.h -- force-included (g++ -include) when compiling the reference's
 * own sources for the oracle/_ref build.
 *
 * IonCloud::DelParticle (bin/ioncloud.cpp:299-308) calls std::copy on
 * double(*)[3] ranges.  Modern libstdc++ implements std::copy by element
 * assignment, which C++ forbids for arrays, so the file no longer compiles.  This
 * non-template overload is preferred by overload resolution for exactly those
 * argument types and copies the rows with memmove, which is what the 2012-era
 * library did.  Nothing else in the reference is affected.
 */
#ifndef SIMGB_REF_COMPAT_H
#define SIMGB_REF_COMPAT_H
#include <algorithm>
#include <cstring>

namespace std {
inline double (*copy(double (*first)[3], double (*last)[3], double (*out)[3]))[3] {
    std::memmove(out, first, (size_t)(last - first) * sizeof(double[3]));
    return out + (last - first);
}
}  // namespace std

#endif
