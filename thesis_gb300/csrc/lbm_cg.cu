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
#include "lbm_cg_store.cuh"
#include "lbm_device.cuh"
#include "thesis_lbm.h"

namespace lbm {
namespace {

struct CgArgs {
    const void *in;          // slot c of direction d at (c*9 + d)*N (lbm_cg_store.cuh)
    void *out;
    float *R, *B;            // colour densities (output)
    void *phi, *dn;          // colour field and density of the streamed state (gradients), arithmetic type
    float *rho, *ux, *uy;    // macroscopic output (when write_macro)
    int nx, ny;
    long long N;
    int write_macro;
    double r_alpha, b_alpha, r_visc, b_visc, beta, A, g_limit;
    float scale, inv_scale;  // F16S: S and 1/S of the summed population
};

constexpr int CG_BLOCK = 128;
__constant__ float c_phi[9] = {0.f, 0.2f, 0.2f, 0.2f, 0.2f, 0.05f, 0.05f, 0.05f, 0.05f};
__constant__ float c_teta[9] = {1.f, -0.2f, -0.2f, -0.2f, -0.2f, -0.05f, -0.05f, -0.05f, -0.05f};
__constant__ double c_phi_d[9] = {0., 0.2, 0.2, 0.2, 0.2, 0.05, 0.05, 0.05, 0.05};
__constant__ double c_teta_d[9] = {1., -0.2, -0.2, -0.2, -0.2, -0.05, -0.05, -0.05, -0.05};

template <class R> __device__ __forceinline__ R cg_rest_phi(int k) {
    if constexpr (sizeof(R) == 8) return c_phi_d[k];
    else return c_phi[k];
}
template <class R> __device__ __forceinline__ R cg_rest_teta(int k) {
    if constexpr (sizeof(R) == 8) return c_teta_d[k];
    else return c_teta[k];
}

__device__ __forceinline__ int wrapi(int a, int n) { return a < 0 ? a + n : (a >= n ? a - n : a); }

// PULL: gather from the neighbours (a time step); otherwise read the node's
// own populations (the first collision from a given post-stream state).
template <int ST, bool PULL>
__device__ __forceinline__ void cg_gather(const CgArgs &a, int x, int y, typename CgStore<ST>::R (&r)[9],
                                          typename CgStore<ST>::R (&b)[9]) {
    using L = Lat<9>;
    using S = CgStore<ST>;
    using T = typename S::T;
    using R = typename S::R;
    const T *in = (const T *)a.in;
#pragma unroll
    for (int d = 0; d < 9; ++d) {
        const int sx = PULL ? wrapi(x - L::cx(d), a.nx) : x;
        const int sy = PULL ? wrapi(y - L::cy(d), a.ny) : y;
        const long long s = sx + (long long)a.nx * sy;
        S::load(in + d * a.N + s, in + (9 + d) * a.N + s, (R)L::w(d), (R)a.inv_scale, r[d], b[d]);
    }
}

template <int ST, bool PULL>
__global__ void __launch_bounds__(CG_BLOCK) cg_density_kernel(const CgArgs a) {
    using R = typename CgStore<ST>::R;
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= a.nx) return;
    R r[9], b[9];
    cg_gather<ST, PULL>(a, x, y, r, b);
    R rr = 0, bb = 0;
#pragma unroll
    for (int d = 0; d < 9; ++d) {
        rr += r[d];
        bb += b[d];
    }
    const int node = x + a.nx * y;
    const R rho = rr + bb;
    ((R *)a.phi)[node] = (rr - bb) / rho;
    ((R *)a.dn)[node] = rho;
}

template <int ST, bool PULL, bool HO, bool ENH>
__global__ void __launch_bounds__(CG_BLOCK) cg_collide_kernel(const CgArgs a) {
    using L = Lat<9>;
    using SP = CgStore<ST>;
    using T = typename SP::T;
    using R = typename SP::R;
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= a.nx) return;
    const int node = x + a.nx * y;
    const R *phi = (const R *)a.phi, *dn = (const R *)a.dn;
    R r[9], b[9];
    cg_gather<ST, PULL>(a, x, y, r, b);
    R f[9], r_r = 0, b_r = 0, jx = 0, jy = 0;
#pragma unroll
    for (int d = 0; d < 9; ++d) {
        f[d] = r[d] + b[d];
        r_r += r[d];
        b_r += b[d];
        if (L::cx(d)) jx += (R)L::cx(d) * f[d];
        if (L::cy(d)) jy += (R)L::cy(d) * f[d];
    }
    const R rho = r_r + b_r;
    const R u = jx / rho, v = jy / rho;
    a.R[node] = (float)r_r;
    a.B[node] = (float)b_r;
    if (a.write_macro) {
        a.rho[node] = (float)rho;
        a.ux[node] = (float)u;
        a.uy[node] = (float)v;
    }
    // colour and density gradients from the neighbours (GpuCollision.cu:112-281)
    R cgx = 0, cgy = 0, grx = 0, gry = 0;
    if (HO) {
        constexpr int hx[24] = {1, 0, -1, 0, 1, -1, -1, 1, 0, 1, 2, 2, 2, 2, 2, 1, 0, -1, -2, -2, -2, -2, -2, -1};
        constexpr int hy[24] = {0, 1, 0, -1, 1, 1, -1, -1, 2, 2, 2, 1, 0, -1, -2, -2, -2, -2, -2, -1, 0, 1, 2, 2};
        constexpr double hw[24] = {960., 960., 960., 960., 448., 448., 448., 448., 84., 32., 1., 32.,
                                   84.,  32.,  1.,   32.,  84.,  32.,  1.,   32.,  84., 32., 1., 32.};
#pragma unroll
        for (int k = 0; k < 24; ++k) {
            const int j = wrapi(x + hx[k], a.nx) + a.nx * wrapi(y + hy[k], a.ny);
            const R w = (R)(hw[k] / 5040.0);
            const R a1 = w * __ldg(phi + j), a2 = ENH ? w * __ldg(dn + j) : (R)0;
            if (ENH) {
                grx += a2 * (R)hx[k];
                gry += a2 * (R)hy[k];
            }
            cgx += a1 * (R)hx[k];
            cgy += a1 * (R)hy[k];
        }
    } else {
#pragma unroll
        for (int k = 1; k < 9; ++k) {
            const int j = wrapi(x + L::cx(k), a.nx) + a.nx * wrapi(y + L::cy(k), a.ny);
            const R w = k <= 4 ? (R)(4.0 / 12.0) : (R)(1.0 / 12.0);
            const R a1 = w * __ldg(phi + j), a2 = ENH ? w * __ldg(dn + j) : (R)0;
            if (ENH) {
                grx += a2 * (R)L::cx(k);
                gry += a2 * (R)L::cy(k);
            }
            cgx += a1 * (R)L::cx(k);
            cgy += a1 * (R)L::cy(k);
        }
    }
    const R r_visc = (R)a.r_visc, b_visc = (R)a.b_visc, beta = (R)a.beta, A = (R)a.A;
    const R mean_nu = (R)1 / (r_r / (rho * r_visc) + b_r / (rho * b_visc));
    const R omega_eff = (R)1 / ((R)3 * mean_nu + (R)0.5);
    const R mean_alpha = (R)a.r_alpha * r_r / rho + (R)a.b_alpha * b_r / rho;
    const R gnorm = sqrt(cgx * cgx + cgy * cgy);
    const R k_r = r_r / rho, k_b = b_r / rho, k_k = beta * r_r * b_r / rho;
    const R cu1 = u * u + v * v;
    const R G1 = (R)2 * u * grx, G2 = u * gry + v * grx, G4 = (R)2 * v * gry;
    const R ugr = u * grx + v * gry;
    const bool interface = gnorm > (R)a.g_limit;
    // one reciprocal per node instead of two divisions per direction
    const R inv_g = interface ? (R)1 / gnorm : (R)0, inv_g2 = inv_g * inv_g;
    T *out = (T *)a.out;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        const R cxk = (R)L::cx(k), cyk = (R)L::cy(k);
        const R wk = k == 0 ? (R)(4. / 9.) : (k <= 4 ? (R)(1. / 9.) : (R)(1. / 36.));
        R pert = 0, cosin = 0;
        if (interface) {
            const R pcg = cxk * cgx + cyk * cgy;
            if (k != 0) cosin = pcg * inv_g * (k <= 4 ? (R)1 : (R)0.70710678118654752);
            const R bk = k == 0 ? (R)(-4. / 27.) : (k <= 4 ? (R)(2. / 27.) : (R)(5. / 108.));
            pert = A * gnorm * (wk * (pcg * pcg) * inv_g2 - bk);
        }
        const R cu2 = u * cxk + v * cyk;
        const R rest = cg_rest_phi<R>(k) + cg_rest_teta<R>(k) * mean_alpha;
        R feq = rho * (rest + wk * ((R)3 * cu2 + (R)4.5 * cu2 * cu2 - (R)1.5 * cu1));
        if (ENH) {
            const R chi = k == 0 ? (R)(-8. / 3.) : (k <= 4 ? (R)(-1. / 6.) : (R)(1. / 12.));
            const R psi = k == 0 ? (R)0 : (k <= 4 ? (R)0.5 : (R)0.125);
            const R TC = G1 * (cxk * cxk) + (R)2 * G2 * (cxk * cyk) + G4 * (cyk * cyk);
            feq += mean_nu * (chi * ugr + psi * TC);
        }
        const R fp = omega_eff * feq + ((R)1 - omega_eff) * f[k] + pert;
        SP::store(out + k * a.N + node, out + (9 + k) * a.N + node, (R)L::w(k), (R)a.scale,
                  k_r * fp + k_k * cosin * rest, k_b * fp - k_k * cosin * rest);
    }
}

// Post-streaming red and blue populations (FP32, SoA) into storage slots.
template <int ST>
__global__ void cg_encode_kernel(const float *r, const float *b, void *out, int q, long long N, float scale) {
    using SP = CgStore<ST>;
    using T = typename SP::T;
    using R = typename SP::R;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)q * N) return;
    const int d = (int)(i / N);
    const R w = q == 9 ? (R)Lat<9>::w(d) : (R)Lat<19>::w(d);
    T *o = (T *)out;
    SP::store(o + i, o + (long long)q * N + i, w, (R)scale, (R)r[i], (R)b[i]);
}

// Storage slots back to red and blue populations (FP32, SoA).
template <int ST>
__global__ void cg_decode_kernel(const void *in, float *r, float *b, int q, long long N, float inv_scale) {
    using SP = CgStore<ST>;
    using T = typename SP::T;
    using R = typename SP::R;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)q * N) return;
    const int d = (int)(i / N);
    const R w = q == 9 ? (R)Lat<9>::w(d) : (R)Lat<19>::w(d);
    const T *s = (const T *)in;
    R rr, bb;
    SP::load(s + i, s + (long long)q * N + i, w, (R)inv_scale, rr, bb);
    r[i] = (float)rr;
    b[i] = (float)bb;
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
    int st = LBM_STORE_F32;          // population storage (lbm_cg_store.cuh)
    void *buf = nullptr;             // 2 buffers x 2 slots x q directions x N values
    float *R = nullptr, *B = nullptr, *rho = nullptr, *ux = nullptr, *uy = nullptr, *uz = nullptr;
    void *phi = nullptr, *dn = nullptr;  // colour field and density for the gradients (arithmetic type)
    double *partial = nullptr, *sums = nullptr;
    int cur = 0;
    float scale = 1024.f;            // F16S: scale of the summed population's deviation
    cudaStream_t stream = nullptr;
    cudaEvent_t stepped = nullptr;  // after the last lbm_cg_step, on its stream
    size_t slot_bytes() const { return (size_t)q * (size_t)N * cg_elem_bytes(st); }
    void *buffer(int c) const { return (char *)buf + (size_t)c * 2 * slot_bytes(); }
};

template <class A>
static void cg_fill_common(const lbm_cg_handle_s *H, int from, int write_macro, A &a) {
    a.in = H->buffer(from);
    a.out = H->buffer(1 - from);
    a.R = H->R;
    a.B = H->B;
    a.phi = H->phi;
    a.dn = H->dn;
    a.rho = H->rho;
    a.ux = H->ux;
    a.uy = H->uy;
    a.nx = H->n;
    a.ny = H->m;
    a.N = H->N;
    a.write_macro = write_macro;
    a.r_alpha = H->P.r_alpha;
    a.b_alpha = H->P.b_alpha;
    a.r_visc = H->P.r_viscosity;
    a.b_visc = H->P.b_viscosity;
    a.beta = H->P.beta;
    a.A = H->P.A;
    a.g_limit = H->P.g_limit;
    a.scale = H->scale;
    a.inv_scale = 1.0f / H->scale;
}

static CgArgs cg_args(const lbm_cg_handle_s *H, int from, int write_macro) {
    CgArgs a;
    memset(&a, 0, sizeof(a));
    cg_fill_common(H, from, write_macro, a);
    return a;
}

static Cg3Args cg3_args(const lbm_cg_handle_s *H, int from, int write_macro) {
    Cg3Args a;
    memset(&a, 0, sizeof(a));
    cg_fill_common(H, from, write_macro, a);
    a.uz = H->uz;
    a.nz = H->h;
    return a;
}

template <int ST, bool PULL>
static void cg3_launch_st(const lbm_cg_handle_s *H, int from, int write_macro, cudaStream_t s) {
    const Cg3Args a = cg3_args(H, from, write_macro);
    const dim3 grid((unsigned)((H->n + CG3_BLOCK - 1) / CG3_BLOCK), (unsigned)H->m, (unsigned)H->h);
    cg3_density_kernel<ST, PULL><<<grid, CG3_BLOCK, 0, s>>>(a);
    if (H->P.high_order) {
        if (H->P.enhanced) cg3_collide_kernel<ST, PULL, true, true><<<grid, CG3_BLOCK, 0, s>>>(a);
        else cg3_collide_kernel<ST, PULL, true, false><<<grid, CG3_BLOCK, 0, s>>>(a);
    } else {
        if (H->P.enhanced) cg3_collide_kernel<ST, PULL, false, true><<<grid, CG3_BLOCK, 0, s>>>(a);
        else cg3_collide_kernel<ST, PULL, false, false><<<grid, CG3_BLOCK, 0, s>>>(a);
    }
}

template <int ST, bool PULL>
static void cg_launch_st(const lbm_cg_handle_s *H, int from, int write_macro, cudaStream_t s) {
    const CgArgs a = cg_args(H, from, write_macro);
    const dim3 grid((unsigned)((H->n + CG_BLOCK - 1) / CG_BLOCK), (unsigned)H->m);
    cg_density_kernel<ST, PULL><<<grid, CG_BLOCK, 0, s>>>(a);
    if (H->P.high_order) {
        if (H->P.enhanced) cg_collide_kernel<ST, PULL, true, true><<<grid, CG_BLOCK, 0, s>>>(a);
        else cg_collide_kernel<ST, PULL, true, false><<<grid, CG_BLOCK, 0, s>>>(a);
    } else {
        if (H->P.enhanced) cg_collide_kernel<ST, PULL, false, true><<<grid, CG_BLOCK, 0, s>>>(a);
        else cg_collide_kernel<ST, PULL, false, false><<<grid, CG_BLOCK, 0, s>>>(a);
    }
}

// One step (PULL) or the first collision from a given post-stream state.
template <bool PULL>
static void cg_any_launch(const lbm_cg_handle_s *H, int from, int write_macro, cudaStream_t s) {
    if (H->q == 19) {
        if (H->st == LBM_STORE_F16S) cg3_launch_st<LBM_STORE_F16S, PULL>(H, from, write_macro, s);
        else if (H->st == LBM_STORE_F64) cg3_launch_st<LBM_STORE_F64, PULL>(H, from, write_macro, s);
        else cg3_launch_st<LBM_STORE_F32, PULL>(H, from, write_macro, s);
    } else {
        if (H->st == LBM_STORE_F16S) cg_launch_st<LBM_STORE_F16S, PULL>(H, from, write_macro, s);
        else if (H->st == LBM_STORE_F64) cg_launch_st<LBM_STORE_F64, PULL>(H, from, write_macro, s);
        else cg_launch_st<LBM_STORE_F32, PULL>(H, from, write_macro, s);
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
    if (P->storage != LBM_STORE_F32 && P->storage != LBM_STORE_F16S && P->storage != LBM_STORE_F64)
        return cg_fail(LBM_ERR_INVALID, "colour-gradient storage must be F32, F16S or F64");
    if (!(P->r_viscosity > 0) || !(P->b_viscosity > 0)) return cg_fail(LBM_ERR_INVALID, "viscosities must be positive");
    lbm_cg_handle_s *H = new (std::nothrow) lbm_cg_handle_s();
    if (!H) return cg_fail(LBM_ERR_NOMEM, "out of host memory");
    H->n = n;
    H->m = m;
    H->h = h;
    H->q = h > 1 ? 19 : 9;
    H->N = (long long)n * m * h;
    H->P = *P;
    H->st = P->storage;
    const size_t N = (size_t)H->N;
    const size_t rbytes = H->st == LBM_STORE_F64 ? sizeof(double) : sizeof(float);
    cudaError_t e = cudaMalloc((void **)&H->buf, 4 * H->slot_bytes());
    if (e == cudaSuccess) e = cudaMalloc((void **)&H->R, sizeof(float) * 6 * N);
    if (e == cudaSuccess) e = cudaMalloc((void **)&H->phi, rbytes * 2 * N);
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
    H->dn = (char *)H->phi + rbytes * N;
    H->sums = H->partial + LAP_BLOCKS * 5;
    cudaMemset(H->R, 0, sizeof(float) * 6 * N);
    cudaMemset(H->phi, 0, rbytes * 2 * N);
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
    // the given post-stream state goes to buffer 1 (through an FP32 staging
    // area in buffer 0, encoded into the storage); one collision without
    // streaming turns it into the post-collision state in buffer 0
    float *stage = (float *)H->buffer(0);
    const size_t fl = sizeof(float) * Q * N;
    float *stage_r = nullptr, *stage_b = nullptr;
    bool own = false;
    if (2 * fl <= 2 * H->slot_bytes()) {
        stage_r = stage;
        stage_b = stage + Q * N;
    } else {
        // F16S: buffer 0 holds fewer bytes than two FP32 colour sets
        cudaError_t e = cudaMalloc((void **)&stage_r, 2 * fl);
        if (e != cudaSuccess) return cg_fail(LBM_ERR_NOMEM, std::string("staging: ") + cudaGetErrorString(e));
        stage_b = stage_r + Q * N;
        own = true;
    }
    cudaError_t e = cudaMemcpyAsync(stage_r, r_f, fl, cudaMemcpyHostToDevice, H->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(stage_b, b_f, fl, cudaMemcpyHostToDevice, H->stream);
    if (e == cudaSuccess) {
        const unsigned blocks = (unsigned)((Q * N + 255) / 256);
        void *dst = H->buffer(1);
        if (H->st == LBM_STORE_F16S)
            cg_encode_kernel<LBM_STORE_F16S><<<blocks, 256, 0, H->stream>>>(stage_r, stage_b, dst, (int)Q, (long long)N, H->scale);
        else if (H->st == LBM_STORE_F64)
            cg_encode_kernel<LBM_STORE_F64><<<blocks, 256, 0, H->stream>>>(stage_r, stage_b, dst, (int)Q, (long long)N, H->scale);
        else
            cg_encode_kernel<LBM_STORE_F32><<<blocks, 256, 0, H->stream>>>(stage_r, stage_b, dst, (int)Q, (long long)N, H->scale);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(H->stream);
    if (own) cudaFree(stage_r);
    if (e != cudaSuccess) return cg_fail(LBM_ERR_CUDA, std::string("upload: ") + cudaGetErrorString(e));
    cg_any_launch<false>(H, 1, 1, H->stream);
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
        cg_any_launch<true>(H, H->cur, wm, s);
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
    if (e != cudaSuccess) return cg_fail(LBM_ERR_CUDA, std::string("read-back: ") + cudaGetErrorString(e));
    // decoded into the other buffer (free between steps) or a temporary
    const size_t fl = sizeof(float) * Q * N;
    float *tmp = nullptr;
    bool own = false;
    if (2 * fl <= 2 * H->slot_bytes()) {
        tmp = (float *)H->buffer(1 - H->cur);
    } else {
        e = cudaMalloc((void **)&tmp, 2 * fl);
        if (e != cudaSuccess) return cg_fail(LBM_ERR_NOMEM, std::string("read-back: ") + cudaGetErrorString(e));
        own = true;
    }
    const unsigned blocks = (unsigned)((Q * N + 255) / 256);
    const void *src = H->buffer(H->cur);
    const float inv = 1.0f / H->scale;
    if (H->st == LBM_STORE_F16S)
        cg_decode_kernel<LBM_STORE_F16S><<<blocks, 256, 0, H->stream>>>(src, tmp, tmp + Q * N, (int)Q, (long long)N, inv);
    else if (H->st == LBM_STORE_F64)
        cg_decode_kernel<LBM_STORE_F64><<<blocks, 256, 0, H->stream>>>(src, tmp, tmp + Q * N, (int)Q, (long long)N, inv);
    else
        cg_decode_kernel<LBM_STORE_F32><<<blocks, 256, 0, H->stream>>>(src, tmp, tmp + Q * N, (int)Q, (long long)N, inv);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(H->stream);
    if (e == cudaSuccess) e = cudaMemcpy(r, tmp, fl, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(b, tmp + Q * N, fl, cudaMemcpyDeviceToHost);
    if (own) cudaFree(tmp);
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
    if (H->phi) cudaFree(H->phi);
    if (H->partial) cudaFree(H->partial);
    if (H->stepped) cudaEventDestroy(H->stepped);
    if (H->stream) cudaStreamDestroy(H->stream);
    delete H;
}

}  // extern "C"
