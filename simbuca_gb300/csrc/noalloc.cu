// noalloc.cu -- sg_coulomb_accel_noalloc: the FP64 Coulomb sum for callers that must
// not allocate device memory.
//
// Some callers of this library cannot call cudaMalloc: a host application that does
// all its device allocation up front and forbids it afterwards (real-time or
// memory-budgeted loops), or a plug-in that runs inside another framework's device
// memory pool and is only handed device pointers.  This entry point takes the
// caller's device buffers for inputs and outputs and keeps its own scratch -- the
// work items, the structure-of-arrays copy of the positions and the per-j-chunk
// partial sums -- in one file-scope device array of fixed size, so it creates no
// context, allocates nothing and frees nothing.
//
// Capacity: at most kNaMaxIons ions per call (larger n returns SG_TOO_LARGE before
// any work is queued).  The array is 1.8 MB and every GPU that loads this library
// holds it until the process exits.  All calls on a device share it and it keeps
// the last call's contents: every scratch entry a call reads is written earlier in
// the same call, so nothing has to start at zero, but calls that overlap on the GPU
// (different streams, or host threads without ordering) race on the array.
#include <algorithm>
#include <mutex>

#include "sg_internal.cuh"

namespace {

constexpr int kNaMaxIons = 8192;
constexpr int kNaMaxSlots = 8;
constexpr int kNaThreads = 128;
constexpr int kNaIpt = 2;
constexpr int kNaIb = kNaThreads * kNaIpt;
constexpr int kNaMaxItems = (kNaMaxIons / kNaIb) * kNaMaxSlots;
constexpr int kNaMaxDevices = 64;

// byte offsets inside the scratch array (each a multiple of 256)
constexpr size_t kOffItems = 0;
constexpr size_t kOffC64 = 16384;  // >= kNaMaxItems * sizeof(SgWorkItem) = 8192
constexpr size_t kOffPart = kOffC64 + 4 * (size_t)kNaMaxIons * sizeof(double);
constexpr size_t kScratchBytes = kOffPart + (size_t)kNaMaxSlots * 3 * kNaMaxIons * sizeof(double);
static_assert(kNaMaxItems * sizeof(SgWorkItem) <= kOffC64, "work items overflow their region");
static_assert(kOffC64 % 256 == 0 && kOffPart % 256 == 0, "scratch regions must stay aligned");

static __device__ __align__(256) unsigned char g_na_scratch[kScratchBytes];

__device__ __forceinline__ SgWorkItem* na_items(unsigned char* scratch) {
    return reinterpret_cast<SgWorkItem*>(scratch + kOffItems);
}
__device__ __forceinline__ double* na_c64(unsigned char* scratch) {
    return reinterpret_cast<double*>(scratch + kOffC64);
}
__device__ __forceinline__ double* na_part(unsigned char* scratch) {
    return reinterpret_cast<double*>(scratch + kOffPart);
}

// positions [n][3] (caller's device buffer) -> SoA x, y, z, q in the scratch; the
// padding ions up to npad sit far away with no charge.
__global__ void na_coords_kernel(unsigned char* scratch, const double* __restrict__ pos,
                                 const double* __restrict__ q, int n, int npad) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npad) return;
    double* c = na_c64(scratch);
    if (i < n) {
        c[i] = pos[3 * (size_t)i];
        c[npad + i] = pos[3 * (size_t)i + 1];
        c[2 * npad + i] = pos[3 * (size_t)i + 2];
        c[3 * npad + i] = q[i];
    } else {
        const double far = 1.0e3 + 1.0e-3 * i;
        c[i] = far;
        c[npad + i] = far;
        c[2 * npad + i] = far;
        c[3 * npad + i] = 0.0;
    }
}

__device__ __forceinline__ double na_rsqrt(double r2) {
    float y0f;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y0f) : "f"(__double2float_rn(r2)));
    const double y0 = (double)y0f;
    const double e = fma(-r2 * y0, y0, 1.0);
    const double p = fma(e, 0.375, 0.5);
    return fma(y0 * e, p, y0);
}

// The FP64 tile kernel of coulomb.cu, reading its work items and coordinates from the
// scratch array and writing the partial sums of each j-chunk there.
__global__ void __launch_bounds__(kNaThreads) na_coulomb_kernel(unsigned char* scratch, int npad) {
    __shared__ double tile[4][kNaThreads];
    const SgWorkItem it = na_items(scratch)[blockIdx.x];
    const double* c = na_c64(scratch);
    const int tid = threadIdx.x;
    int ipad[kNaIpt];
    double xi[kNaIpt], yi[kNaIpt], zi[kNaIpt], ax[kNaIpt], ay[kNaIpt], az[kNaIpt];
#pragma unroll
    for (int k = 0; k < kNaIpt; k++) {
        const int li = tid + k * kNaThreads;
        const int ii = it.i0 + (li < it.ni ? li : 0);
        ipad[k] = li < it.ni ? ii : -1;
        xi[k] = c[ii];
        yi[k] = c[npad + ii];
        zi[k] = c[2 * npad + ii];
        ax[k] = ay[k] = az[k] = 0.0;
    }
    for (int j0 = it.j0; j0 < it.j0 + it.nj; j0 += kNaThreads) {
        const int len = min(kNaThreads, it.j0 + it.nj - j0);
        __syncthreads();
        if (tid < len) {
            tile[0][tid] = c[j0 + tid];
            tile[1][tid] = c[npad + j0 + tid];
            tile[2][tid] = c[2 * npad + j0 + tid];
            tile[3][tid] = c[3 * npad + j0 + tid];
        }
        __syncthreads();
        for (int jj = 0; jj < len; jj++) {
            const double xj = tile[0][jj], yj = tile[1][jj], zj = tile[2][jj], qj = tile[3][jj];
            const int jg = j0 + jj;
#pragma unroll
            for (int k = 0; k < kNaIpt; k++) {
                const double rx = xi[k] - xj, ry = yi[k] - yj, rz = zi[k] - zj;
                const double y = na_rsqrt(rx * rx + ry * ry + rz * rz);
                double w = qj * (y * y * y);
                w = (jg == ipad[k]) ? 0.0 : w;
                ax[k] = fma(w, rx, ax[k]);
                ay[k] = fma(w, ry, ay[k]);
                az[k] = fma(w, rz, az[k]);
            }
        }
    }
    double* P = na_part(scratch) + (size_t)it.slot * 3 * npad;
#pragma unroll
    for (int k = 0; k < kNaIpt; k++) {
        if (ipad[k] < 0) continue;
        P[ipad[k]] = ax[k];
        P[npad + ipad[k]] = ay[k];
        P[2 * (size_t)npad + ipad[k]] = az[k];
    }
}

// acc[i][c] = kq[i] * sum over the j-chunks of the partial sums (caller's buffers).
__global__ void na_finish_kernel(unsigned char* scratch, const double* __restrict__ kq,
                                 double* __restrict__ acc, int n, int npad, int nslots) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double* part = na_part(scratch);
    double s[3] = {0.0, 0.0, 0.0};
    for (int sl = 0; sl < nslots; sl++)
        for (int c = 0; c < 3; c++) s[c] += part[((size_t)sl * 3 + c) * npad + i];
    for (int c = 0; c < 3; c++) acc[3 * (size_t)i + c] = kq[i] * s[c];
}

std::mutex g_na_mu;
void* g_na_addr[kNaMaxDevices] = {nullptr};

}  // namespace

extern "C" int sg_coulomb_accel_noalloc(int n, const double* pos, const double* q,
                                        const double* kq, double* acc, void* stream) {
    if (n < 0) return SG_BAD_ARG;
    if (n == 0) return SG_OK;
    if (!pos || !q || !kq || !acc) return SG_BAD_ARG;
    if (n > kNaMaxIons) return SG_TOO_LARGE;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return SG_NO_DEVICE;
    if (dev < 0 || dev >= kNaMaxDevices) return SG_NO_DEVICE;
    void* base = nullptr;
    {
        // Set-up, once per device with that device current: the device address of the
        // scratch array.  In host code g_na_scratch names a host-side stand-in, so the
        // kernels and the copy below get this pointer, never the symbol itself.
        std::lock_guard<std::mutex> lk(g_na_mu);
        if (!g_na_addr[dev]) {
            void* p = nullptr;
            if (cudaGetSymbolAddress(&p, g_na_scratch) != cudaSuccess || !p) return SG_CUDA_ERR;
            g_na_addr[dev] = p;
        }
        base = g_na_addr[dev];
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int npad = (n + SG_PAD - 1) / SG_PAD * SG_PAD;
    // work items: i-blocks of kNaIb ions x up to kNaMaxSlots j-chunks (multiples of 128)
    const int nib = (n + kNaIb - 1) / kNaIb;
    int slots = std::max(1, std::min(kNaMaxSlots, npad / 512));
    const int jc = ((npad + slots - 1) / slots + 127) / 128 * 128;
    slots = (npad + jc - 1) / jc;
    SgWorkItem items[kNaMaxItems];
    int ni = 0;
    for (int s = 0; s < slots; s++)
        for (int b = 0; b < nib; b++) {
            SgWorkItem& it = items[ni++];
            it.cloud = 0;
            it.i0 = b * kNaIb;
            it.ni = std::min(kNaIb, n - b * kNaIb);
            it.j0 = s * jc;
            it.nj = std::min(jc, npad - s * jc);
            it.slot = s;
            it.pad0 = it.pad1 = 0;
        }
    if (cudaMemcpyAsync(static_cast<unsigned char*>(base) + kOffItems, items,
                        sizeof(SgWorkItem) * ni, cudaMemcpyHostToDevice, st) != cudaSuccess)
        return SG_CUDA_ERR;
    unsigned char* scratch = static_cast<unsigned char*>(base);
    na_coords_kernel<<<(npad + 255) / 256, 256, 0, st>>>(scratch, pos, q, n, npad);
    na_coulomb_kernel<<<ni, kNaThreads, 0, st>>>(scratch, npad);
    na_finish_kernel<<<(n + 255) / 256, 256, 0, st>>>(scratch, kq, acc, n, npad, slots);
    return cudaGetLastError() == cudaSuccess ? SG_OK : SG_CUDA_ERR;
}
