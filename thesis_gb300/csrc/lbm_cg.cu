// Colour-gradient two-phase D2Q9 on a periodic lattice (the reference's
// multiphase 2D path: gpuCollBgkwGC2D / gpuCollEnhancedBgkwGC2D,
// GpuCollision.cu:552-707; gpuStreaming2DCG, GpuStream.cu:30-158;
// gpuUpdateMacro2DCG, GpuUpdateMacro.cu:43-135; Laplace-law sums,
// Iterate.cu:496-499).
//
// The collision of a node needs the colour field (rho_r - rho_b)/rho of its
// 8 (3x3 stencil) or 24 (5x5 stencil) neighbours after streaming, so a step is
// two launches over the lattice:
//   cg_density_kernel  pull both colours, write the colour field
//                      phi = (rho_r - rho_b)/rho and rho per node;
//   cg_collide_kernel  pull both colours again, take the neighbours' phi and
//                      rho for the gradients, collide, perturb, recolour,
//                      write both post-collision colours and rho_r, rho_b.
// State between steps: post-collision red and blue populations, SoA by
// direction, pull double buffer.  Both kernels are HBM-bound: 72 B of
// populations read by each, 72 B written by the second, 8 B of densities.
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <new>
#include <string>
#include <vector>

#include "lbm_cg3.cuh"
#include "lbm_device.cuh"
#include "thesis_lbm.h"

namespace lbm {
namespace {

struct CgArgs {
    const float *rin[9], *bin[9];
    float *rout[9], *bout[9];
    float *R, *B;            // colour densities (output)
    float *phi, *dn;         // colour field and density of the streamed state (gradients)
    float *rho, *ux, *uy;    // macroscopic output (when write_macro)
    int nx, ny;
    int write_macro;
    float r_alpha, b_alpha, r_visc, b_visc, beta, A, g_limit;
};

constexpr int CG_BLOCK = 128;
__constant__ float c_phi[9] = {0.f, 0.2f, 0.2f, 0.2f, 0.2f, 0.05f, 0.05f, 0.05f, 0.05f};
__constant__ float c_teta[9] = {1.f, -0.2f, -0.2f, -0.2f, -0.2f, -0.05f, -0.05f, -0.05f, -0.05f};

__device__ __forceinline__ int wrapi(int a, int n) { return a < 0 ? a + n : (a >= n ? a - n : a); }

// PULL: gather from the neighbours (a time step); otherwise read the node's
// own populations (the first collision from a given post-stream state).
template <bool PULL>
__device__ __forceinline__ void cg_gather(const CgArgs &a, int x, int y, float (&r)[9], float (&b)[9]) {
    using L = Lat<9>;
#pragma unroll
    for (int d = 0; d < 9; ++d) {
        const int sx = PULL ? wrapi(x - L::cx(d), a.nx) : x;
        const int sy = PULL ? wrapi(y - L::cy(d), a.ny) : y;
        const int s = sx + a.nx * sy;
        r[d] = __ldg(a.rin[d] + s);
        b[d] = __ldg(a.bin[d] + s);
    }
}

template <bool PULL>
__global__ void __launch_bounds__(CG_BLOCK) cg_density_kernel(const CgArgs a) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= a.nx) return;
    float r[9], b[9];
    cg_gather<PULL>(a, x, y, r, b);
    float rr = 0.f, bb = 0.f;
#pragma unroll
    for (int d = 0; d < 9; ++d) {
        rr += r[d];
        bb += b[d];
    }
    const int node = x + a.nx * y;
    const float rho = rr + bb;
    a.phi[node] = (rr - bb) / rho;
    a.dn[node] = rho;
}

template <bool PULL, bool HO, bool ENH>
__global__ void __launch_bounds__(CG_BLOCK) cg_collide_kernel(const CgArgs a) {
    using L = Lat<9>;
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= a.nx) return;
    const int node = x + a.nx * y;
    float r[9], b[9];
    cg_gather<PULL>(a, x, y, r, b);
    float f[9], r_r = 0.f, b_r = 0.f, jx = 0.f, jy = 0.f;
#pragma unroll
    for (int d = 0; d < 9; ++d) {
        f[d] = r[d] + b[d];
        r_r += r[d];
        b_r += b[d];
        if (L::cx(d)) jx += (float)L::cx(d) * f[d];
        if (L::cy(d)) jy += (float)L::cy(d) * f[d];
    }
    const float rho = r_r + b_r;
    const float u = jx / rho, v = jy / rho;
    a.R[node] = r_r;
    a.B[node] = b_r;
    if (a.write_macro) {
        a.rho[node] = rho;
        a.ux[node] = u;
        a.uy[node] = v;
    }
    // colour and density gradients from the neighbours (GpuCollision.cu:112-281)
    float cgx = 0.f, cgy = 0.f, grx = 0.f, gry = 0.f;
    if (HO) {
        constexpr int hx[24] = {1, 0, -1, 0, 1, -1, -1, 1, 0, 1, 2, 2, 2, 2, 2, 1, 0, -1, -2, -2, -2, -2, -2, -1};
        constexpr int hy[24] = {0, 1, 0, -1, 1, 1, -1, -1, 2, 2, 2, 1, 0, -1, -2, -2, -2, -2, -2, -1, 0, 1, 2, 2};
        constexpr double hw[24] = {960., 960., 960., 960., 448., 448., 448., 448., 84., 32., 1., 32.,
                                   84.,  32.,  1.,   32.,  84.,  32.,  1.,   32.,  84., 32., 1., 32.};
#pragma unroll
        for (int k = 0; k < 24; ++k) {
            const int j = wrapi(x + hx[k], a.nx) + a.nx * wrapi(y + hy[k], a.ny);
            const float w = (float)(hw[k] / 5040.0);
            const float a1 = w * __ldg(a.phi + j), a2 = ENH ? w * __ldg(a.dn + j) : 0.f;
            if (ENH) {
                grx += a2 * (float)hx[k];
                gry += a2 * (float)hy[k];
            }
            cgx += a1 * (float)hx[k];
            cgy += a1 * (float)hy[k];
        }
    } else {
#pragma unroll
        for (int k = 1; k < 9; ++k) {
            const int j = wrapi(x + L::cx(k), a.nx) + a.nx * wrapi(y + L::cy(k), a.ny);
            const float w = k <= 4 ? (float)(4.0 / 12.0) : (float)(1.0 / 12.0);
            const float a1 = w * __ldg(a.phi + j), a2 = ENH ? w * __ldg(a.dn + j) : 0.f;
            if (ENH) {
                grx += a2 * (float)L::cx(k);
                gry += a2 * (float)L::cy(k);
            }
            cgx += a1 * (float)L::cx(k);
            cgy += a1 * (float)L::cy(k);
        }
    }
    const float mean_nu = 1.f / (r_r / (rho * a.r_visc) + b_r / (rho * a.b_visc));
    const float omega_eff = 1.f / (3.f * mean_nu + 0.5f);
    const float mean_alpha = a.r_alpha * r_r / rho + a.b_alpha * b_r / rho;
    const float gnorm = sqrtf(cgx * cgx + cgy * cgy);
    const float k_r = r_r / rho, k_b = b_r / rho, k_k = a.beta * r_r * b_r / rho;
    const float cu1 = u * u + v * v;
    const float G1 = 2.f * u * grx, G2 = u * gry + v * grx, G4 = 2.f * v * gry;
    const float ugr = u * grx + v * gry;
    const bool interface = gnorm > a.g_limit;
    // one reciprocal per node instead of two divisions per direction
    const float inv_g = interface ? 1.f / gnorm : 0.f, inv_g2 = inv_g * inv_g;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        const float cxk = (float)L::cx(k), cyk = (float)L::cy(k);
        const float wk = k == 0 ? (float)(4. / 9.) : (k <= 4 ? (float)(1. / 9.) : (float)(1. / 36.));
        float pert = 0.f, cosin = 0.f;
        if (interface) {
            const float pcg = cxk * cgx + cyk * cgy;
            if (k != 0) cosin = pcg * inv_g * (k <= 4 ? 1.f : 0.70710678f);
            const float bk = k == 0 ? (float)(-4. / 27.) : (k <= 4 ? (float)(2. / 27.) : (float)(5. / 108.));
            pert = a.A * gnorm * (wk * (pcg * pcg) * inv_g2 - bk);
        }
        const float cu2 = u * cxk + v * cyk;
        const float rest = c_phi[k] + c_teta[k] * mean_alpha;
        float feq = rho * (rest + wk * (3.f * cu2 + 4.5f * cu2 * cu2 - 1.5f * cu1));
        if (ENH) {
            const float chi = k == 0 ? (float)(-8. / 3.) : (k <= 4 ? (float)(-1. / 6.) : (float)(1. / 12.));
            const float psi = k == 0 ? 0.f : (k <= 4 ? 0.5f : 0.125f);
            const float TC = G1 * (cxk * cxk) + 2.f * G2 * (cxk * cyk) + G4 * (cyk * cyk);
            feq += mean_nu * (chi * ugr + psi * TC);
        }
        const float fp = omega_eff * feq + (1.f - omega_eff) * f[k] + pert;
        a.rout[k][node] = k_r * fp + k_k * cosin * rest;
        a.bout[k][node] = k_b * fp - k_k * cosin * rest;
    }
}

// FP64 Laplace-law sums: sum rho_r and count where chi >= c, sum rho_b and
// count where chi <= -c, max |u| (Iterate.cu:496-499, GpuUpdateMacro.cu:122-133).
constexpr int LAP_BLOCKS = 304, LAP_THREADS = 256;
__global__ void __launch_bounds__(LAP_THREADS)
cg_laplace_partial(const float *R, const float *B, const float *ux, const float *uy, const float *uz, long long n,
                   float c, double *partial) {
    double acc[5] = {0, 0, 0, 0, 0};
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double r = R[i], b = B[i], chi = (r - b) / (r + b);
        if (chi >= c) {
            acc[0] += r;
            acc[1] += 1;
        } else if (chi <= -c) {
            acc[2] += b;
            acc[3] += 1;
        }
        const double wz = uz ? (double)uz[i] : 0.0;
        const double um = sqrt((double)ux[i] * ux[i] + (double)uy[i] * uy[i] + wz * wz);
        acc[4] = um > acc[4] ? um : acc[4];
    }
    __shared__ double sm[LAP_THREADS][5];
#pragma unroll
    for (int k = 0; k < 5; ++k) sm[threadIdx.x][k] = acc[k];
    __syncthreads();
    if (threadIdx.x < 5) {
        double s = 0;
        for (int t = 0; t < LAP_THREADS; ++t)
            s = threadIdx.x == 4 ? (sm[t][4] > s ? sm[t][4] : s) : s + sm[t][threadIdx.x];
        partial[blockIdx.x * 5 + threadIdx.x] = s;
    }
}

__global__ void cg_laplace_final(const double *partial, double *out) {
    if (threadIdx.x >= 5) return;
    double s = 0;
    for (int bI = 0; bI < LAP_BLOCKS; ++bI) {
        const double v = partial[bI * 5 + threadIdx.x];
        s = threadIdx.x == 4 ? (v > s ? v : s) : s + v;
    }
    out[threadIdx.x] = s;
}

thread_local std::string g_cg_error;
int cg_fail(int code, const std::string &m) {
    g_cg_error = m;
    return code;
}

}  // namespace
}  // namespace lbm

using namespace lbm;

struct lbm_cg_handle_s {
    int n = 0, m = 0, h = 1, q = 9;  // D2Q9 (h = 1) or D3Q19
    long long N = 0;
    lbm_cg_params P{};
    float *buf = nullptr;  // 2 buffers x 2 colours x q directions x N
    float *R = nullptr, *B = nullptr, *rho = nullptr, *ux = nullptr, *uy = nullptr, *uz = nullptr;
    float *phi = nullptr, *dn = nullptr;  // D3Q19: colour field and density for the gradients
    double *partial = nullptr, *sums = nullptr;
    int cur = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t stepped = nullptr;  // after the last lbm_cg_step, on its stream
};

static CgArgs cg_args(const lbm_cg_handle_s *H, int from, int write_macro) {
    CgArgs a;
    memset(&a, 0, sizeof(a));
    const size_t N = (size_t)H->N;
    float *src = H->buf + (size_t)from * 18 * N, *dst = H->buf + (size_t)(1 - from) * 18 * N;
    for (int d = 0; d < 9; ++d) {
        a.rin[d] = src + d * N;
        a.bin[d] = src + (9 + d) * N;
        a.rout[d] = dst + d * N;
        a.bout[d] = dst + (9 + d) * N;
    }
    a.R = H->R;
    a.B = H->B;
    a.phi = H->phi;
    a.dn = H->dn;
    a.rho = H->rho;
    a.ux = H->ux;
    a.uy = H->uy;
    a.nx = H->n;
    a.ny = H->m;
    a.write_macro = write_macro;
    a.r_alpha = (float)H->P.r_alpha;
    a.b_alpha = (float)H->P.b_alpha;
    a.r_visc = (float)H->P.r_viscosity;
    a.b_visc = (float)H->P.b_viscosity;
    a.beta = (float)H->P.beta;
    a.A = (float)H->P.A;
    a.g_limit = (float)H->P.g_limit;
    return a;
}

static Cg3Args cg3_args(const lbm_cg_handle_s *H, int from, int write_macro) {
    Cg3Args a;
    memset(&a, 0, sizeof(a));
    const size_t N = (size_t)H->N;
    a.in = H->buf + (size_t)from * 38 * N;
    a.out = H->buf + (size_t)(1 - from) * 38 * N;
    a.R = H->R;
    a.B = H->B;
    a.phi = H->phi;
    a.dn = H->dn;
    a.rho = H->rho;
    a.ux = H->ux;
    a.uy = H->uy;
    a.uz = H->uz;
    a.nx = H->n;
    a.ny = H->m;
    a.nz = H->h;
    a.N = H->N;
    a.write_macro = write_macro;
    a.r_alpha = (float)H->P.r_alpha;
    a.b_alpha = (float)H->P.b_alpha;
    a.r_visc = (float)H->P.r_viscosity;
    a.b_visc = (float)H->P.b_viscosity;
    a.beta = (float)H->P.beta;
    a.A = (float)H->P.A;
    a.g_limit = (float)H->P.g_limit;
    return a;
}

template <bool PULL>
static void cg3_launch(const lbm_cg_handle_s *H, int from, int write_macro, cudaStream_t s) {
    const Cg3Args a = cg3_args(H, from, write_macro);
    const dim3 grid((unsigned)((H->n + CG3_BLOCK - 1) / CG3_BLOCK), (unsigned)H->m, (unsigned)H->h);
    cg3_density_kernel<PULL><<<grid, CG3_BLOCK, 0, s>>>(a);
    if (H->P.high_order) {
        if (H->P.enhanced) cg3_collide_kernel<PULL, true, true><<<grid, CG3_BLOCK, 0, s>>>(a);
        else cg3_collide_kernel<PULL, true, false><<<grid, CG3_BLOCK, 0, s>>>(a);
    } else {
        if (H->P.enhanced) cg3_collide_kernel<PULL, false, true><<<grid, CG3_BLOCK, 0, s>>>(a);
        else cg3_collide_kernel<PULL, false, false><<<grid, CG3_BLOCK, 0, s>>>(a);
    }
}

template <bool PULL>
static void cg_launch(const lbm_cg_handle_s *H, const CgArgs &a, cudaStream_t s) {
    const dim3 grid((unsigned)((H->n + CG_BLOCK - 1) / CG_BLOCK), (unsigned)H->m);
    cg_density_kernel<PULL><<<grid, CG_BLOCK, 0, s>>>(a);
    if (H->P.high_order) {
        if (H->P.enhanced) cg_collide_kernel<PULL, true, true><<<grid, CG_BLOCK, 0, s>>>(a);
        else cg_collide_kernel<PULL, true, false><<<grid, CG_BLOCK, 0, s>>>(a);
    } else {
        if (H->P.enhanced) cg_collide_kernel<PULL, false, true><<<grid, CG_BLOCK, 0, s>>>(a);
        else cg_collide_kernel<PULL, false, false><<<grid, CG_BLOCK, 0, s>>>(a);
    }
}

extern "C" {

const char *lbm_cg_last_error(void) { return g_cg_error.c_str(); }

static int cg_create(int n, int m, int h, const lbm_cg_params *P, lbm_cg_handle *out) {
    if (!P || !out) return cg_fail(LBM_ERR_INVALID, "null argument");
    *out = nullptr;
    if (n < 5 || m < 5 || h < 1 || m > 65535 || h > 65535 || (h > 1 && h < 5))
        return cg_fail(LBM_ERR_INVALID, "lattice must be at least 5 nodes along each axis (m, h <= 65535)");
    if ((long long)n * m * h >= (1ll << 31)) return cg_fail(LBM_ERR_INVALID, "more than 2^31 nodes");
    if (P->storage != LBM_STORE_F32) return cg_fail(LBM_ERR_UNSUPPORTED, "colour-gradient storage is F32");
    if (!(P->r_viscosity > 0) || !(P->b_viscosity > 0)) return cg_fail(LBM_ERR_INVALID, "viscosities must be positive");
    lbm_cg_handle_s *H = new (std::nothrow) lbm_cg_handle_s();
    if (!H) return cg_fail(LBM_ERR_NOMEM, "out of host memory");
    H->n = n;
    H->m = m;
    H->h = h;
    H->q = h > 1 ? 19 : 9;
    H->N = (long long)n * m * h;
    H->P = *P;
    const size_t N = (size_t)H->N;
    cudaError_t e = cudaMalloc((void **)&H->buf, sizeof(float) * 4 * H->q * N);
    if (e == cudaSuccess) e = cudaMalloc((void **)&H->R, sizeof(float) * 8 * N);
    if (e == cudaSuccess) e = cudaMalloc((void **)&H->partial, sizeof(double) * (LAP_BLOCKS * 5 + 5));
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&H->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&H->stepped, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        lbm_cg_destroy(H);
        return cg_fail(LBM_ERR_NOMEM, std::string("allocation: ") + cudaGetErrorString(e));
    }
    H->B = H->R + N;
    H->rho = H->R + 2 * N;
    H->ux = H->R + 3 * N;
    H->uy = H->R + 4 * N;
    H->uz = H->R + 5 * N;
    H->phi = H->R + 6 * N;
    H->dn = H->R + 7 * N;
    H->sums = H->partial + LAP_BLOCKS * 5;
    cudaMemset(H->R, 0, sizeof(float) * 8 * N);
    *out = H;
    return LBM_OK;
}

int lbm_cg_create(int n, int m, const lbm_cg_params *P, lbm_cg_handle *out) { return cg_create(n, m, 1, P, out); }

int lbm_cg_create3d(int n, int m, int h, const lbm_cg_params *P, lbm_cg_handle *out) {
    if (h < 5) return cg_fail(LBM_ERR_INVALID, "lattice must be at least 5 nodes along each axis");
    return cg_create(n, m, h, P, out);
}

int lbm_cg_init(lbm_cg_handle H, const float *r_f, const float *b_f) {
    if (!H || !r_f || !b_f) return cg_fail(LBM_ERR_INVALID, "null argument");
    const size_t N = (size_t)H->N, Q = (size_t)H->q;
    // the given post-stream state goes to buffer 1; one collision without
    // streaming turns it into the post-collision state in buffer 0
    float *b1 = H->buf + 2 * Q * N;
    cudaError_t e = cudaMemcpyAsync(b1, r_f, sizeof(float) * Q * N, cudaMemcpyHostToDevice, H->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(b1 + Q * N, b_f, sizeof(float) * Q * N, cudaMemcpyHostToDevice, H->stream);
    if (e != cudaSuccess) return cg_fail(LBM_ERR_CUDA, std::string("upload: ") + cudaGetErrorString(e));
    if (H->q == 19)
        cg3_launch<false>(H, 1, 1, H->stream);
    else
        cg_launch<false>(H, cg_args(H, 1, 1), H->stream);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(H->stream);
    if (e != cudaSuccess) return cg_fail(LBM_ERR_CUDA, std::string("init: ") + cudaGetErrorString(e));
    H->cur = 0;
    return LBM_OK;
}

int lbm_cg_step(lbm_cg_handle H, int nsteps, int write_macro_last, void *stream) {
    if (!H || nsteps < 0) return cg_fail(LBM_ERR_INVALID, "invalid argument");
    cudaStream_t s = stream ? (cudaStream_t)stream : H->stream;
    for (int i = 0; i < nsteps; ++i) {
        const int wm = write_macro_last && i == nsteps - 1;
        if (H->q == 19)
            cg3_launch<true>(H, H->cur, wm, s);
        else
            cg_launch<true>(H, cg_args(H, H->cur, wm), s);
        H->cur ^= 1;
    }
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaEventRecord(H->stepped, s);
    if (e != cudaSuccess) return cg_fail(LBM_ERR_CUDA, std::string("step: ") + cudaGetErrorString(e));
    return LBM_OK;
}

int lbm_cg_get_macro(lbm_cg_handle H, float *r_rho, float *b_rho, float *u, float *v) {
    if (!H) return cg_fail(LBM_ERR_INVALID, "null handle");
    cudaError_t e = cudaDeviceSynchronize();
    const size_t b = sizeof(float) * (size_t)H->N;
    if (e == cudaSuccess && r_rho) e = cudaMemcpy(r_rho, H->R, b, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && b_rho) e = cudaMemcpy(b_rho, H->B, b, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && u) e = cudaMemcpy(u, H->ux, b, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && v) e = cudaMemcpy(v, H->uy, b, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cg_fail(LBM_ERR_CUDA, std::string("read-back: ") + cudaGetErrorString(e));
    return LBM_OK;
}

int lbm_cg_get_macro3d(lbm_cg_handle H, float *r_rho, float *b_rho, float *u, float *v, float *w) {
    int rc = lbm_cg_get_macro(H, r_rho, b_rho, u, v);
    if (rc || !w) return rc;
    cudaError_t e = cudaMemcpy(w, H->uz, sizeof(float) * (size_t)H->N, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cg_fail(LBM_ERR_CUDA, std::string("read-back: ") + cudaGetErrorString(e));
    return LBM_OK;
}

int lbm_cg_get_populations(lbm_cg_handle H, float *r, float *b) {
    if (!H || !r || !b) return cg_fail(LBM_ERR_INVALID, "null argument");
    const size_t N = (size_t)H->N, Q = (size_t)H->q;
    cudaError_t e = cudaDeviceSynchronize();
    const float *src = H->buf + (size_t)H->cur * 2 * Q * N;
    if (e == cudaSuccess) e = cudaMemcpy(r, src, sizeof(float) * Q * N, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(b, src + Q * N, sizeof(float) * Q * N, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cg_fail(LBM_ERR_CUDA, std::string("read-back: ") + cudaGetErrorString(e));
    return LBM_OK;
}

int lbm_cg_laplace(lbm_cg_handle H, double *out) {
    if (!H || !out) return cg_fail(LBM_ERR_INVALID, "null argument");
    if (H->stepped) cudaStreamWaitEvent(H->stream, H->stepped, 0);
    cg_laplace_partial<<<LAP_BLOCKS, LAP_THREADS, 0, H->stream>>>(H->R, H->B, H->ux, H->uy, H->q == 19 ? H->uz : nullptr,
                                                                   H->N, (float)H->P.control_param, H->partial);
    cg_laplace_final<<<1, 32, 0, H->stream>>>(H->partial, H->sums);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, H->sums, sizeof(double) * 5, cudaMemcpyDeviceToHost, H->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(H->stream);
    if (e != cudaSuccess) return cg_fail(LBM_ERR_CUDA, std::string("laplace: ") + cudaGetErrorString(e));
    for (int k = 0; k < 5; ++k)
        if (!isfinite(out[k])) return cg_fail(LBM_DIVERGED, "non-finite colour-gradient field");
    return LBM_OK;
}

long long lbm_cg_nodes(lbm_cg_handle H) { return H ? H->N : -1; }

int lbm_cg_q(lbm_cg_handle H) { return H ? H->q : -1; }

void lbm_cg_destroy(lbm_cg_handle H) {
    if (!H) return;
    if (H->stream) cudaStreamSynchronize(H->stream);
    if (H->buf) cudaFree(H->buf);
    if (H->R) cudaFree(H->R);
    if (H->partial) cudaFree(H->partial);
    if (H->stepped) cudaEventDestroy(H->stepped);
    if (H->stream) cudaStreamDestroy(H->stream);
    delete H;
}

}  // extern "C"
