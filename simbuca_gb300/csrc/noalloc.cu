// noalloc.cu -- sg_coulomb_accel_noalloc: the FP64 Coulomb sum for callers that must
// not allocate device memory.
//
// Some callers of this library cannot call cudaMalloc: a host application that does
// all its device allocation up front and forbids it afterwards (real-time or
// memory-budgeted loops), or a plug-in that runs inside another framework's device
// memory pool and is only handed device pointers.  This entry point takes the
// caller's device buffers for inputs and outputs and keeps its own scratch -- the
// structure-of-arrays copy of the positions and the per-j-chunk partial sums -- in
// one file-scope device array of fixed size, so it creates no context, allocates
// nothing and frees nothing, and it copies nothing from host memory: each block
// derives its rows and its j-chunk from its block index.
//
// Capacity: at most kNaMaxIons ions per call (larger n returns SG_TOO_LARGE before
// any work is queued).  The array is 1.8 MB and every GPU that loads this library
// holds it until the process exits.  All calls on a device share it and it keeps
// the last call's contents: every scratch entry a call reads is written earlier in
// the same call, so nothing has to start at zero, but calls that overlap on the GPU
// (different streams, or host threads without ordering) race on the array.
//
// Set-up: a __device__ array has one address per CUDA context.  The first call made
// in a context looks that address up (cudaGetSymbolAddress, with the context
// current) and keeps it under the context's unique id, so a caller that switches
// between contexts on one device, or destroys and re-creates one, never gets an
// address from another context.  That first call should come before any stream
// capture.
#include <cuda.h>

#include <algorithm>
#include <mutex>

#include "sg_internal.cuh"

namespace {

constexpr int kNaMaxIons = 8192;
constexpr int kNaMaxSlots = 8;
constexpr int kNaThreads = 128;
constexpr int kNaIpt = 2;
constexpr int kNaIb = kNaThreads * kNaIpt;
constexpr int kNaMaxContexts = 64;

// byte offsets inside the scratch array (each a multiple of 256)
constexpr size_t kOffC64 = 0;
constexpr size_t kOffPart = kOffC64 + 4 * (size_t)kNaMaxIons * sizeof(double);
constexpr size_t kScratchBytes = kOffPart + (size_t)kNaMaxSlots * 3 * kNaMaxIons * sizeof(double);
static_assert(kOffPart % 256 == 0, "scratch regions must stay aligned");

static __device__ __align__(256) unsigned char g_na_scratch[kScratchBytes];

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

// The FP64 tile kernel of coulomb.cu.  Block b covers rows [ib*kNaIb, +kNaIb) of
// j-chunk s = b / nib, i.e. columns [s*jc, s*jc + jc) cut at npad, and writes that
// chunk's partial sums to slot s of the scratch.
__global__ void __launch_bounds__(kNaThreads) na_coulomb_kernel(unsigned char* scratch, int n,
                                                               int npad, int nib, int jc) {
    __shared__ double tile[4][kNaThreads];
    const int s = blockIdx.x / nib;
    const int i0 = (blockIdx.x - s * nib) * kNaIb;
    const int ni = min(kNaIb, n - i0);
    const int jb = s * jc;
    const int je = min(jb + jc, npad);
    const double* c = na_c64(scratch);
    const int tid = threadIdx.x;
    int ipad[kNaIpt];
    double xi[kNaIpt], yi[kNaIpt], zi[kNaIpt], ax[kNaIpt], ay[kNaIpt], az[kNaIpt];
#pragma unroll
    for (int k = 0; k < kNaIpt; k++) {
        const int li = tid + k * kNaThreads;
        const int ii = i0 + (li < ni ? li : 0);
        ipad[k] = li < ni ? ii : -1;
        xi[k] = c[ii];
        yi[k] = c[npad + ii];
        zi[k] = c[2 * npad + ii];
        ax[k] = ay[k] = az[k] = 0.0;
    }
    for (int j0 = jb; j0 < je; j0 += kNaThreads) {
        const int len = min(kNaThreads, je - j0);
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
    double* P = na_part(scratch) + (size_t)s * 3 * npad;
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

// The current context's unique id, through the driver entry points the runtime hands
// out (no link against the driver library).
using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

struct NaCtxEntry {
    unsigned long long id;
    void* addr;
};

std::mutex g_na_mu;
CtxGetCurrentFn g_get_current = nullptr;
CtxGetIdFn g_get_id = nullptr;
NaCtxEntry g_na_ctx[kNaMaxContexts];
int g_na_nctx = 0;

bool na_current_context_id(unsigned long long* id) {
    if (!g_get_current || !g_get_id) {
        void* f0 = nullptr;
        void* f1 = nullptr;
        cudaDriverEntryPointQueryResult q0, q1;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f0, 12000, cudaEnableDefault,
                                             &q0) != cudaSuccess ||
            q0 != cudaDriverEntryPointSuccess || !f0)
            return false;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f1, 12000, cudaEnableDefault,
                                             &q1) != cudaSuccess ||
            q1 != cudaDriverEntryPointSuccess || !f1)
            return false;
        g_get_current = reinterpret_cast<CtxGetCurrentFn>(f0);
        g_get_id = reinterpret_cast<CtxGetIdFn>(f1);
    }
    CUcontext ctx = nullptr;
    if (g_get_current(&ctx) != CUDA_SUCCESS || !ctx) return false;
    return g_get_id(ctx, id) == CUDA_SUCCESS;
}

// The scratch array's device address in the current context (set-up on first use in
// that context).  Returns null on failure.
void* na_scratch_address() {
    std::lock_guard<std::mutex> lk(g_na_mu);
    unsigned long long id = 0;
    const bool have_id = na_current_context_id(&id);
    if (have_id)
        for (int k = 0; k < g_na_nctx; k++)
            if (g_na_ctx[k].id == id) return g_na_ctx[k].addr;
    // In host code g_na_scratch names a host-side stand-in: the kernels get this
    // pointer, never the symbol itself.  With no context current, this runtime call
    // makes the current device's primary context current first.
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_na_scratch) != cudaSuccess || !p) return nullptr;
    if (!have_id && !na_current_context_id(&id)) return p;  // valid now, not kept
    if (g_na_nctx < kNaMaxContexts) {
        g_na_ctx[g_na_nctx++] = {id, p};
    } else {
        // more contexts than the table holds: replace the oldest entry
        std::rotate(g_na_ctx, g_na_ctx + 1, g_na_ctx + kNaMaxContexts);
        g_na_ctx[kNaMaxContexts - 1] = {id, p};
    }
    return p;
}

}  // namespace

extern "C" int sg_coulomb_accel_noalloc(int n, const double* pos, const double* q,
                                        const double* kq, double* acc, void* stream) {
    if (n < 0) return SG_BAD_ARG;
    if (n == 0) return SG_OK;
    if (!pos || !q || !kq || !acc) return SG_BAD_ARG;
    if (n > kNaMaxIons) return SG_TOO_LARGE;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return SG_NO_DEVICE;
    unsigned char* scratch = static_cast<unsigned char*>(na_scratch_address());
    if (!scratch) return SG_CUDA_ERR;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int npad = (n + SG_PAD - 1) / SG_PAD * SG_PAD;
    // blocks: i-blocks of kNaIb ions x up to kNaMaxSlots j-chunks (multiples of 128)
    const int nib = (n + kNaIb - 1) / kNaIb;
    int slots = std::max(1, std::min(kNaMaxSlots, npad / 512));
    const int jc = ((npad + slots - 1) / slots + 127) / 128 * 128;
    slots = (npad + jc - 1) / jc;
    // Each launch's own return value: an error an earlier call left in the runtime's
    // last-error slot neither fails this call nor gets cleared by it.
    cudaLaunchConfig_t cfg = {};
    cfg.stream = st;
    cfg.gridDim = dim3((npad + 255) / 256);
    cfg.blockDim = dim3(256);
    if (cudaLaunchKernelEx(&cfg, na_coords_kernel, scratch, pos, q, n, npad) != cudaSuccess)
        return SG_CUDA_ERR;
    cfg.gridDim = dim3(slots * nib);
    cfg.blockDim = dim3(kNaThreads);
    if (cudaLaunchKernelEx(&cfg, na_coulomb_kernel, scratch, n, npad, nib, jc) != cudaSuccess)
        return SG_CUDA_ERR;
    cfg.gridDim = dim3((n + 255) / 256);
    cfg.blockDim = dim3(256);
    if (cudaLaunchKernelEx(&cfg, na_finish_kernel, scratch, kq, acc, n, npad, slots) !=
        cudaSuccess)
        return SG_CUDA_ERR;
    return SG_OK;
}
