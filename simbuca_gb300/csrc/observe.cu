// Device-side observables of the reference's output path (IonCloud::PrintParticle /
// PrintCloud, bin/ioncloud.cpp:85-183, called from move_particles,
// bin/ion_fly.cpp:103-108), kept on the device: when a cloud's print is due the two
// kernels below write one record into that cloud's ring (statistics per species and
// the state of every stride-th ion) without a host round trip; the host drains the
// rings when it synchronises and formats the reference's text from them.
#include "sg_internal.cuh"

namespace {

constexpr double kJouleToEv = 6.24150e18;  // bin/globals.h:9

__device__ __forceinline__ double* record_of(const SgRecArgs& r, const SgCloud& cl,
                                             const SgCtrl& cs) {
    return r.ring + cl.rec_off + (long long)cs.rec_slot * cl.rec_len;
}

// The kept ions: device position i holds caller index perm[i]; every stride-th caller
// index of the cloud goes to slot (index - first) / stride.
__global__ void __launch_bounds__(SG_ROWS) record_ions_kernel(SgRecArgs r) {
    sg_griddep_wait();
    const SgRowBlock rb = r.rows[blockIdx.x];
    const SgCtrl& cs = r.ctrl[rb.cloud];
    if (!cs.print_due) return;
    const SgCloud& cl = r.clouds[rb.cloud];
    const int li = threadIdx.x;
    if (li >= rb.n) return;
    const int i = rb.i0 + li;
    const int loc = r.perm[i] - cl.off;
    if (loc % r.stride) return;
    double* out = record_of(r, cl, cs) + 1 + SG_STAT_LEN * r.n_species + SG_ION_LEN * (loc / r.stride);
    const size_t N = (size_t)r.n;
#pragma unroll
    for (int c = 0; c < 6; c++) out[c] = r.y[c * N + i];
    // PrintParticle's energy (bin/ioncloud.cpp:86)
    out[6] = r.mass[i] * (out[3] * out[3] + out[4] * out[4] + out[5] * out[5]) * 0.5 * kJouleToEv;
    out[7] = (double)r.spec[i];
}

// Species and print masses after a dissociation (tables in the caller's order).
__global__ void __launch_bounds__(SG_ROWS) dissociate_kernel(SgRecArgs r, double* __restrict__ mass,
                                                             int* __restrict__ spec0,
                                                             double* __restrict__ mass0) {
    sg_griddep_wait();
    const SgRowBlock rb = r.rows[blockIdx.x];
    const SgCtrl& cs = r.ctrl[rb.cloud];
    if (!cs.dis_due) return;
    const int li = threadIdx.x;
    if (li >= rb.n) return;
    const int i = rb.i0 + li;
    const size_t at = (size_t)(cs.dis_due - 1) * r.n + r.perm[i];
    r.spec[i] = r.dis_spec[at];
    mass[i] = r.dis_mass[at];
    spec0[r.perm[i]] = r.dis_spec[at];  // caller's order, for later state uploads
    mass0[r.perm[i]] = r.dis_mass[at];
}

// Block-wide sum of K values per thread into red (thread 0 reads the totals).
template <int K>
__device__ void block_sum(double (&v)[K], double* red) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < K; k++) {
        double x = v[k];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (lane == 0) red[w * K + k] = x;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 0; k < K; k++) {
            double x = 0.0;
            for (int ww = 0; ww < (int)(blockDim.x >> 5); ww++) x += red[ww * K + k];
            v[k] = x;
        }
    }
    __syncthreads();
}

// PrintCloud's statistics, one block per cloud, two passes over its ions (centroid,
// then spread about it).  As in the reference, both divide by the cloud's ion count and
// the energy sums m (vx^2 + vy^2 + vz vy) / 2.
__global__ void __launch_bounds__(256) record_stats_kernel(SgRecArgs r) {
    sg_griddep_wait();
    __shared__ double red[8 * 5 * SG_MAX_SPECIES];
    __shared__ double cen[3 * SG_MAX_SPECIES];
    const SgCtrl& cs = r.ctrl[blockIdx.x];
    if (!cs.print_due) return;
    const SgCloud& cl = r.clouds[blockIdx.x];
    const int S = r.n_species;
    const size_t N = (size_t)r.n;
    double acc[5 * SG_MAX_SPECIES];
#pragma unroll
    for (int k = 0; k < 5 * SG_MAX_SPECIES; k++) acc[k] = 0.0;
    for (int i = cl.off + threadIdx.x; i < cl.off + cl.n; i += blockDim.x) {
        const int s = r.spec[i];
        const double x = r.y[i], y = r.y[N + i], z = r.y[2 * N + i];
        const double vx = r.y[3 * N + i], vy = r.y[4 * N + i], vz = r.y[5 * N + i];
        const double e = 0.5 * kJouleToEv * r.mass[i] * (vx * vx + vy * vy + vz * vy);
#pragma unroll
        for (int q = 0; q < SG_MAX_SPECIES; q++)
            if (q == s) {
                acc[5 * q] += x;
                acc[5 * q + 1] += y;
                acc[5 * q + 2] += z;
                acc[5 * q + 3] += e;
                acc[5 * q + 4] += 1.0;
            }
    }
    block_sum(acc, red);
    double* out = record_of(r, cl, cs);
    const double n = (double)cl.n;
    if (threadIdx.x == 0) {
        out[0] = cs.t;
        for (int q = 0; q < S; q++) {
            cen[3 * q] = acc[5 * q] / n;
            cen[3 * q + 1] = acc[5 * q + 1] / n;
            cen[3 * q + 2] = acc[5 * q + 2] / n;
            double* o = out + 1 + SG_STAT_LEN * q;
            o[0] = cen[3 * q];
            o[1] = cen[3 * q + 1];
            o[2] = cen[3 * q + 2];
            o[6] = acc[5 * q + 3];
            o[7] = acc[5 * q + 4];
            o[8] = n;
        }
    }
    __syncthreads();
    double sp[3 * SG_MAX_SPECIES];
#pragma unroll
    for (int k = 0; k < 3 * SG_MAX_SPECIES; k++) sp[k] = 0.0;
    for (int i = cl.off + threadIdx.x; i < cl.off + cl.n; i += blockDim.x) {
        const int s = r.spec[i];
        const double x = r.y[i], y = r.y[N + i], z = r.y[2 * N + i];
#pragma unroll
        for (int q = 0; q < SG_MAX_SPECIES; q++)
            if (q == s) {
                const double dx = x - cen[3 * q], dy = y - cen[3 * q + 1], dz = z - cen[3 * q + 2];
                sp[3 * q] += dx * dx;
                sp[3 * q + 1] += dy * dy;
                sp[3 * q + 2] += dz * dz;
            }
    }
    block_sum(sp, red);
    if (threadIdx.x == 0)
        for (int q = 0; q < S; q++) {
            double* o = out + 1 + SG_STAT_LEN * q;
            o[3] = sqrt(sp[3 * q] / n);
            o[4] = sqrt(sp[3 * q + 1] / n);
            o[5] = sqrt(sp[3 * q + 2] / n);
        }
}

// A record of every cloud now (the reference's print after an operation): takes the
// next ring slot, or holds the cloud when its ring is full.
__global__ void record_now_kernel(SgCtrl* ctrl, int n_clouds) {
    sg_griddep_wait();
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n_clouds) return;
    SgCtrl& cs = ctrl[c];
    cs.print_due = 0;
    if (cs.rec_cap <= 0 || cs.status != SG_OK) return;
    if (cs.rec_count - cs.rec_drained >= cs.rec_cap) {
        cs.hold |= 2;
        return;
    }
    cs.print_due = 1;
    cs.rec_slot = (int)(cs.rec_count % cs.rec_cap);
    cs.rec_count++;
}

__global__ void gather_int_kernel(const int* __restrict__ src, const int* __restrict__ perm,
                                  int* __restrict__ dst, int n) {
    sg_griddep_wait();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = src[perm[i]];
}

}  // namespace

cudaError_t sg_gather_int(const int* src, const int* perm, int* dst, int n, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    sg_launch(gather_int_kernel, (n + 255) / 256, 256, 0, st, src, perm, dst, n);
    return cudaGetLastError();
}

cudaError_t sg_record(const SgRecArgs& r, int n_rows, int n_clouds, cudaStream_t st) {
    if (n_rows > 0) sg_launch(record_ions_kernel, n_rows, SG_ROWS, 0, st, r);
    if (n_clouds > 0) sg_launch(record_stats_kernel, n_clouds, 256, 0, st, r);
    return cudaGetLastError();
}

cudaError_t sg_dissociate(const SgRecArgs& r, double* mass, int* spec0, double* mass0, int n_rows,
                          cudaStream_t st) {
    if (n_rows > 0) sg_launch(dissociate_kernel, n_rows, SG_ROWS, 0, st, r, mass, spec0, mass0);
    return cudaGetLastError();
}

cudaError_t sg_record_now(SgCtrl* ctrl, int n_clouds, cudaStream_t st) {
    sg_launch(record_now_kernel, (n_clouds + 127) / 128, 128, 0, st, ctrl, n_clouds);
    return cudaGetLastError();
}
