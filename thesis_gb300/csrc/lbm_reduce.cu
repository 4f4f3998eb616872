// Deterministic FP64 reductions over fluid nodes: the steady-state velocity
// residual and the global mass and momentum sums.  The grid has a fixed size,
// each block writes one partial per quantity, and a single thread adds the
// partials in block order, so the result does not depend on scheduling.
// Replaces the reference's multi-pass float tree reductions with a host loop
// (GpuSum.cu:82-264) and its divergence flag (GpuSum.cu:10-23).
#include <cuda_runtime.h>

#include "lbm_types.h"

namespace lbm {

constexpr int NORM_BLOCKS = 304;  // 2 x 152 SMs
constexpr int NORM_THREADS = 256;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

__global__ void __launch_bounds__(NORM_THREADS)
norms_partial(const uint32_t *__restrict__ word, const float *__restrict__ rho,
              const float *__restrict__ ux, const float *__restrict__ uy,
              const float *__restrict__ uz, float *pux, float *puy, float *puz, long long n,
              double *partial) {
    double acc[LBM_NORMS] = {0, 0, 0, 0, 0};
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
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
    __shared__ double sm[NORM_THREADS / 32][LBM_NORMS];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < LBM_NORMS; ++k) {
        const double s = warp_sum(acc[k]);
        if (lane == 0) sm[warp][k] = s;
    }
    __syncthreads();
    if (threadIdx.x < LBM_NORMS) {
        double s = 0;
        for (int wI = 0; wI < NORM_THREADS / 32; ++wI) s += sm[wI][threadIdx.x];
        partial[blockIdx.x * LBM_NORMS + threadIdx.x] = s;
    }
}

__global__ void norms_final(const double *partial, int nblocks, double *out) {
    if (threadIdx.x >= LBM_NORMS) return;
    double s = 0;
    for (int b = 0; b < nblocks; ++b) s += partial[b * LBM_NORMS + threadIdx.x];
    out[threadIdx.x] = s;
}

int launch_norms(const uint32_t *word, const float *rho, const float *ux, const float *uy,
                 const float *uz, float *pux, float *puy, float *puz, long long n,
                 double *partial, double *out, cudaStream_t s) {
    norms_partial<<<NORM_BLOCKS, NORM_THREADS, 0, s>>>(word, rho, ux, uy, uz, pux, puy, puz, n,
                                                       partial);
    norms_final<<<1, 32, 0, s>>>(partial, NORM_BLOCKS, out);
    return 0;
}

int norm_partial_count() { return NORM_BLOCKS * LBM_NORMS; }

// The reference's MaxMacroDiff residual (Iterate3D.cu:696-735, gpu_abs_sub +
// gpu_max_h, GpuSum.cu:10-23, 241-264): max |x - x_prev| over all nodes for
// u, v, w, rho, then x_prev <- x.  out[4] counts non-finite differences (the
// reference's divergence flag).  Max is order-independent, so the result is
// deterministic.
__global__ void __launch_bounds__(NORM_THREADS)
macro_diff_partial(const float *__restrict__ ux, const float *__restrict__ uy, const float *__restrict__ uz,
                   const float *__restrict__ rho, float *pux, float *puy, float *puz, float *prho, long long n,
                   double *partial) {
    double acc[5] = {0, 0, 0, 0, 0};
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const float cur[4] = {ux[i], uy[i], uz[i], rho[i]};
        float *prev[4] = {pux, puy, puz, prho};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const double d = fabs((double)cur[k] - (double)prev[k][i]);
            if (!isfinite(d)) acc[4] += 1.0;
            else acc[k] = d > acc[k] ? d : acc[k];
            prev[k][i] = cur[k];
        }
    }
    __shared__ double sm[NORM_THREADS][5];
#pragma unroll
    for (int k = 0; k < 5; ++k) sm[threadIdx.x][k] = acc[k];
    __syncthreads();
    if (threadIdx.x < 5) {
        double r = 0;
        for (int t = 0; t < NORM_THREADS; ++t) {
            const double v = sm[t][threadIdx.x];
            r = threadIdx.x == 4 ? r + v : (v > r ? v : r);
        }
        partial[blockIdx.x * 5 + threadIdx.x] = r;
    }
}

__global__ void macro_diff_final(const double *partial, int nblocks, double *out) {
    if (threadIdx.x >= 5) return;
    double r = 0;
    for (int b = 0; b < nblocks; ++b) {
        const double v = partial[b * 5 + threadIdx.x];
        r = threadIdx.x == 4 ? r + v : (v > r ? v : r);
    }
    out[threadIdx.x] = r;
}

int launch_macro_diff(const float *ux, const float *uy, const float *uz, const float *rho, float *pux, float *puy,
                      float *puz, float *prho, long long n, double *partial, double *out, cudaStream_t s) {
    macro_diff_partial<<<NORM_BLOCKS, NORM_THREADS, 0, s>>>(ux, uy, uz, rho, pux, puy, puz, prho, n, partial);
    macro_diff_final<<<1, 32, 0, s>>>(partial, NORM_BLOCKS, out);
    return 0;
}

}  // namespace lbm
