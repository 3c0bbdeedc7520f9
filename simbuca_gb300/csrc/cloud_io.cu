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
#include <cstdio>
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

// ---- state files ------------------------------------------------------------------
// Binary restart file (layout in simgb.h).  The host is little-endian on both machines
// this library is built for (x86-64, aarch64); values are written as their bytes.
namespace {

const char kStateMagic[8] = {'S', 'G', 'S', 'T', 'A', 'T', 'E', '1'};

struct File {
    FILE* f;
    explicit File(FILE* p) : f(p) {}
    ~File() {
        if (f) fclose(f);
    }
};

bool put(FILE* f, const void* p, size_t bytes) { return bytes == 0 || fwrite(p, 1, bytes, f) == bytes; }
bool get(FILE* f, void* p, size_t bytes) { return bytes == 0 || fread(p, 1, bytes, f) == bytes; }

int read_header(FILE* f, uint32_t* n, double* t) {
    char magic[8];
    uint32_t version = 0;
    if (!get(f, magic, 8) || memcmp(magic, kStateMagic, 8) != 0) return SG_IO_ERR;
    if (!get(f, &version, 4) || version != 1) return SG_IO_ERR;
    if (!get(f, n, 4) || !get(f, t, 8)) return SG_IO_ERR;
    return SG_OK;
}

}  // namespace

extern "C" int sg_state_save(const char* path, int n, double t, const double* pos,
                             const double* vel, const double* mass, const int* charge,
                             const int* species) {
    if (!path || n < 0 || (n > 0 && (!pos || !vel || !mass || !charge))) return SG_BAD_ARG;
    File fl(fopen(path, "wb"));
    if (!fl.f) return SG_IO_ERR;
    const uint32_t version = 1, un = (uint32_t)n;
    bool ok = put(fl.f, kStateMagic, 8) && put(fl.f, &version, 4) && put(fl.f, &un, 4) &&
              put(fl.f, &t, 8) && put(fl.f, pos, 24 * (size_t)n) &&
              put(fl.f, vel, 24 * (size_t)n) && put(fl.f, mass, 8 * (size_t)n) &&
              put(fl.f, charge, 4 * (size_t)n);
    if (ok && species) {
        ok = put(fl.f, species, 4 * (size_t)n);
    } else if (ok) {
        const int32_t zero = 0;
        for (int i = 0; ok && i < n; i++) ok = put(fl.f, &zero, 4);
    }
    if (fflush(fl.f) != 0) ok = false;
    return ok ? SG_OK : SG_IO_ERR;
}

extern "C" int sg_state_info(const char* path, int* n, double* t) {
    if (!path || !n || !t) return SG_BAD_ARG;
    File fl(fopen(path, "rb"));
    if (!fl.f) return SG_IO_ERR;
    uint32_t un = 0;
    const int st = read_header(fl.f, &un, t);
    if (st != SG_OK) return st;
    if (un > 0x7fffffffu) return SG_IO_ERR;
    *n = (int)un;
    return SG_OK;
}

extern "C" int sg_state_load(const char* path, int cap, double* t, double* pos, double* vel,
                             double* mass, int* charge, int* species) {
    if (!path || !t || cap < 0) return SG_BAD_ARG;
    File fl(fopen(path, "rb"));
    if (!fl.f) return SG_IO_ERR;
    uint32_t un = 0;
    const int st = read_header(fl.f, &un, t);
    if (st != SG_OK) return st;
    if (un > (uint32_t)cap) return SG_TOO_LARGE;
    const size_t n = un;
    if (n > 0 && (!pos || !vel || !mass || !charge)) return SG_BAD_ARG;
    bool ok = get(fl.f, pos, 24 * n) && get(fl.f, vel, 24 * n) && get(fl.f, mass, 8 * n) &&
              get(fl.f, charge, 4 * n);
    if (ok && species) {
        ok = get(fl.f, species, 4 * n);
    } else if (ok) {
        int32_t skip = 0;
        for (size_t i = 0; ok && i < n; i++) ok = get(fl.f, &skip, 4);
    }
    return ok ? SG_OK : SG_IO_ERR;
}

// ---- the reference's particle text output -------------------------------------------
// One line per ion and print time: ID name t[ms] x y z[mm] vx vy vz[m/s] E[eV]
// (bin/ioncloud.cpp:85-111), the ions of a print in ID order.  A print starts where the
// time changes or the IDs start over; the last one is read.
namespace {

bool skip_line(const char* line) { return line[0] == '\n' || line[0] == '\0' || line[0] == '#'; }

int parse_particle(const char* line, int* id, char* name, double* tm, double* v) {
    return sscanf(line, "%d %255s %lf %lf %lf %lf %lf %lf %lf %lf", id, name, tm, &v[0], &v[1],
                  &v[2], &v[3], &v[4], &v[5], &v[6]) == 10
               ? SG_OK
               : SG_IO_ERR;
}

}  // namespace

extern "C" int sg_particles_text_last(const char* path, const char* const* names,
                                      const double* masses, const int* charges, int n_names,
                                      int cap, int* n, double* t, int* ids, double* pos,
                                      double* vel, double* mass, int* charge, int* species) {
    if (!path || !names || !masses || !charges || n_names < 1 || cap < 0 || !n || !t)
        return SG_BAD_ARG;
    File fl(fopen(path, "r"));
    if (!fl.f) return SG_IO_ERR;
    char line[1024], name[256];
    long block = -1;
    double t_block = 0.0, t_prev = 0.0;
    int id_prev = 0;
    for (;;) {
        const long off = ftell(fl.f);
        if (!fgets(line, sizeof line, fl.f)) break;
        if (skip_line(line)) continue;
        int id;
        double tm, v[7];
        if (parse_particle(line, &id, name, &tm, v) != SG_OK) return SG_IO_ERR;
        if (block < 0 || tm != t_prev || id <= id_prev) {
            block = off;
            t_block = tm;
        }
        t_prev = tm;
        id_prev = id;
    }
    if (block < 0 || fseek(fl.f, block, SEEK_SET) != 0) return SG_IO_ERR;
    int k = 0;
    while (fgets(line, sizeof line, fl.f)) {
        if (skip_line(line)) continue;
        int id;
        double tm, v[7];
        if (parse_particle(line, &id, name, &tm, v) != SG_OK) return SG_IO_ERR;
        int s = -1;
        for (int q = 0; q < n_names && s < 0; q++)
            if (names[q] && strcmp(names[q], name) == 0) s = q;
        if (s < 0) return SG_BAD_ARG;
        if (k >= cap) {
            k++;
            continue;  // count the ions for *n, report SG_TOO_LARGE below
        }
        if (ids) ids[k] = id;
        if (pos)
            for (int c = 0; c < 3; c++) pos[3 * (size_t)k + c] = v[c] / 1000.0;
        if (vel)
            for (int c = 0; c < 3; c++) vel[3 * (size_t)k + c] = v[3 + c];
        if (mass) mass[k] = masses[s];
        if (charge) charge[k] = charges[s];
        if (species) species[k] = s;
        k++;
    }
    *n = k;
    *t = t_block / 1000.0;
    return k > cap ? SG_TOO_LARGE : SG_OK;
}
