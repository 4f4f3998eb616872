// FP64 fluid-node norms without any allocation.
//
// Some callers cannot allocate device memory while they run the solver: a
// host framework that owns a fixed device arena and forbids cudaMalloc and
// cudaFree inside its step callback (allocation there synchronises the device
// and can fail mid-run), or code that must stay allocation-free for
// predictable memory use.  This entry point computes the same norms as
// lbm_macro_norms from device arrays the caller passes, and keeps its
// per-block partial sums in one file-scope device array instead of memory it
// would have to allocate.
//
// Limits and sharing:
//   * at most LBM_NOALLOC_MAX_NODES nodes per call (NOALLOC_MAX_BLOCKS blocks
//     of NOALLOC_NODES_PER_BLOCK nodes each); larger calls are rejected;
//   * the partials array (NOALLOC_MAX_BLOCKS * 5 doubles, 160 KiB) exists once
//     in every device context that loads the library and lives until the
//     process exits;
//   * every call shares it.  Each call writes every partial it reads before
//     reading it, so nothing has to start at zero, but two calls whose kernels
//     overlap on the GPU (different streams, or threads launching at once)
//     race on the partials and give wrong sums: serialise them;
//   * the first call on a device looks up the array's device address with
//     cudaGetSymbolAddress (with that device current) and caches it; make that
//     first call before any stream capture on the device.  The cached address
//     belongs to the device's context: cudaDeviceReset destroys that context
//     and the library's module with it, so a process that resets a device must
//     not call this entry point on that device afterwards (the cached address
//     would point at memory that no longer holds the array);
//   * errors: a CUDA error already pending when the call starts, or raised by
//     its launches, is returned as LBM_ERR_CUDA with a message in
//     lbm_noalloc_last_error().  The pending error is only peeked at, never
//     cleared, so the caller's own error checks still see it.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "lbm_types.h"

namespace lbm {
namespace {

constexpr int NOALLOC_THREADS = 256;
constexpr long long NOALLOC_NODES_PER_BLOCK = 256 * 64;
constexpr int NOALLOC_MAX_BLOCKS = 4096;
constexpr int NOALLOC_MAX_DEVICES = 64;

static __device__ __align__(256) double g_noalloc_partials[NOALLOC_MAX_BLOCKS * LBM_NORMS];

std::mutex g_noalloc_mutex;
double *g_noalloc_ptr[NOALLOC_MAX_DEVICES] = {nullptr};
thread_local std::string g_noalloc_error;

__device__ __forceinline__ double noalloc_warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// One block per NOALLOC_NODES_PER_BLOCK consecutive nodes, so the number of
// partials grows with the lattice and is bounded by the static array.
__global__ void __launch_bounds__(NOALLOC_THREADS)
noalloc_partial(const uint32_t *__restrict__ word, const float *__restrict__ rho,
                const float *__restrict__ ux, const float *__restrict__ uy,
                const float *__restrict__ uz, float *pux, float *puy, float *puz, long long n,
                double *partial) {
    const long long lo = (long long)blockIdx.x * NOALLOC_NODES_PER_BLOCK;
    const long long hi = lo + NOALLOC_NODES_PER_BLOCK < n ? lo + NOALLOC_NODES_PER_BLOCK : n;
    double acc[LBM_NORMS] = {0, 0, 0, 0, 0};
    for (long long i = lo + threadIdx.x; i < hi; i += NOALLOC_THREADS) {
        if (!(word[i] & W_FLUID)) continue;
        const double u = ux[i], v = uy[i], w = uz[i], r = rho[i];
        const double du = u - pux[i], dv = v - puy[i], dw = w - puz[i];
        acc[0] += du * du + dv * dv + dw * dw;
        acc[1] += u * u + v * v + w * w;
        acc[2] += r;
        acc[3] += 1.0;
        acc[4] += r * u;
        pux[i] = (float)u;
        puy[i] = (float)v;
        puz[i] = (float)w;
    }
    __shared__ double sm[NOALLOC_THREADS / 32][LBM_NORMS];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < LBM_NORMS; ++k) {
        const double s = noalloc_warp_sum(acc[k]);
        if (lane == 0) sm[warp][k] = s;
    }
    __syncthreads();
    if (threadIdx.x < LBM_NORMS) {
        double s = 0;
        for (int k = 0; k < NOALLOC_THREADS / 32; ++k) s += sm[k][threadIdx.x];
        partial[(long long)blockIdx.x * LBM_NORMS + threadIdx.x] = s;
    }
}

__global__ void noalloc_final(const double *partial, int nblocks, double *out) {
    if (threadIdx.x >= LBM_NORMS) return;
    double s = 0;
    for (int b = 0; b < nblocks; ++b) s += partial[(long long)b * LBM_NORMS + threadIdx.x];
    out[threadIdx.x] = s;
}

int noalloc_fail(int code, const std::string &msg) {
    g_noalloc_error = msg;
    return code;
}

}  // namespace
}  // namespace lbm

using namespace lbm;

extern "C" {

long long lbm_noalloc_max_nodes(void) { return (long long)NOALLOC_MAX_BLOCKS * NOALLOC_NODES_PER_BLOCK; }

const char *lbm_noalloc_last_error(void) { return g_noalloc_error.c_str(); }

int lbm_fluid_norms_noalloc(const uint32_t *word, const float *rho, const float *u, const float *v,
                            const float *w, float *u_prev, float *v_prev, float *w_prev, long long n,
                            double *out, void *stream) {
    if (!word || !rho || !u || !v || !w || !u_prev || !v_prev || !w_prev || !out)
        return noalloc_fail(LBM_ERR_INVALID, "lbm_fluid_norms_noalloc: null pointer");
    if (n <= 0) return noalloc_fail(LBM_ERR_INVALID, "lbm_fluid_norms_noalloc: n must be positive");
    if (n > lbm_noalloc_max_nodes())
        return noalloc_fail(LBM_ERR_INVALID,
                            "lbm_fluid_norms_noalloc: " + std::to_string(n) + " nodes exceed the maximum of " +
                                std::to_string(lbm_noalloc_max_nodes()) + " (static partials array)");
    cudaError_t e = cudaPeekAtLastError();
    if (e != cudaSuccess)
        return noalloc_fail(LBM_ERR_CUDA, std::string("lbm_fluid_norms_noalloc: an earlier CUDA error is pending: ") +
                                              cudaGetErrorString(e));
    int dev = 0;
    e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return noalloc_fail(LBM_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES)
        return noalloc_fail(LBM_ERR_INVALID, "lbm_fluid_norms_noalloc: device ordinal out of range");
    double *partials = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_noalloc_mutex);
        if (!g_noalloc_ptr[dev]) {
            void *p = nullptr;
            e = cudaGetSymbolAddress(&p, g_noalloc_partials);
            if (e != cudaSuccess || !p)
                return noalloc_fail(LBM_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            g_noalloc_ptr[dev] = (double *)p;
        }
        partials = g_noalloc_ptr[dev];
    }
    const int nblocks = (int)((n + NOALLOC_NODES_PER_BLOCK - 1) / NOALLOC_NODES_PER_BLOCK);
    cudaStream_t s = (cudaStream_t)stream;
    noalloc_partial<<<nblocks, NOALLOC_THREADS, 0, s>>>(word, rho, u, v, w, u_prev, v_prev, w_prev, n, partials);
    noalloc_final<<<1, 32, 0, s>>>(partials, nblocks, out);
    e = cudaPeekAtLastError();
    if (e != cudaSuccess) return noalloc_fail(LBM_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
    return LBM_OK;
}

}  // extern "C"
