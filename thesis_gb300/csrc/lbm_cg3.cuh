// Colour-gradient two-phase D3Q19 on a lattice periodic in all three axes
// (the reference's multiphase 3D collision gpuCollBgkwGC3D /
// gpuCollEnhancedBgkwGC3D, GpuCollision.cu:283-526, :709-880; two-colour
// streaming gpuStreaming3DCG, GpuStream.cu:196-250; densities and velocity
// of gpuUpdateMacro3DCG, GpuUpdateMacro.cu:215-360).
//
// The same two launches per step as the D2Q9 path (lbm_cg.cu):
//   cg3_density_kernel  pull both colours, write the colour field
//                       phi = (rho_r - rho_b)/rho and rho per node;
//   cg3_collide_kernel  pull both colours again, take the neighbours' phi and
//                       rho for the gradients, collide, perturb, recolour,
//                       write both colours and the node's rho_r, rho_b.
// State between steps: post-collision red and blue populations, SoA by
// direction (direction d of colour c at base + (c*19 + d) N), pull double
// buffer.  Per update the two kernels read 2 x 152 B of populations and
// write 152 B, plus 16 B of per-node fields written and the neighbours'
// phi and rho read through L1/L2.
#pragma once
#include "lbm_device.cuh"

namespace lbm {

struct Cg3Args {
    const float *in;   // red directions 0..18, then blue, N floats each
    float *out;
    float *R, *B;      // colour densities (output)
    float *phi, *dn;   // colour field and density of the streamed state (gradients)
    float *rho, *ux, *uy, *uz;
    int nx, ny, nz;
    long long N;
    int write_macro;
    float r_alpha, b_alpha, r_visc, b_visc, beta, A, g_limit;
};

constexpr int CG3_BLOCK = 128;
// minimum resident blocks per SM the collide kernel is compiled for (a
// register cap of 65536 / (128 * CG3_MINB) per thread)
#ifndef CG3_MINB
#define CG3_MINB 5
#endif

__device__ __forceinline__ int cg3_wrap(int a, int n) { return a < 0 ? a + n : (a >= n ? a - n : a); }

// Wrapped neighbour coordinates of node (x, y, z) as node-index parts:
// X[1 + t] + Y[1 + t'] + Z[1 + t''] is the node at offset (t, t', t''),
// t in {-1, 0, 1}.  Node indices fit in 32 bits (fewer than 2^31 nodes).
struct Cg3Nb {
    int X[3], Y[3], Z[3];
    __device__ __forceinline__ Cg3Nb(const Cg3Args &a, int x, int y, int z) {
        const int plane = a.nx * a.ny;
        X[0] = x == 0 ? a.nx - 1 : x - 1;
        X[1] = x;
        X[2] = x == a.nx - 1 ? 0 : x + 1;
        Y[0] = (y == 0 ? a.ny - 1 : y - 1) * a.nx;
        Y[1] = y * a.nx;
        Y[2] = (y == a.ny - 1 ? 0 : y + 1) * a.nx;
        Z[0] = (z == 0 ? a.nz - 1 : z - 1) * plane;
        Z[1] = z * plane;
        Z[2] = (z == a.nz - 1 ? 0 : z + 1) * plane;
    }
    __device__ __forceinline__ int at(int cx, int cy, int cz) const { return X[1 + cx] + Y[1 + cy] + Z[1 + cz]; }
};

// Both colours of the node after streaming (PULL: population d from the
// node at -c_d) or as stored.
template <bool PULL>
__device__ __forceinline__ void cg3_gather(const Cg3Args &a, const Cg3Nb &nb, float (&r)[19], float (&b)[19]) {
    using L = Lat<19>;
#pragma unroll
    for (int d = 0; d < 19; ++d) {
        const int s = PULL ? nb.at(-L::cx(d), -L::cy(d), -L::cz(d)) : nb.at(0, 0, 0);
        r[d] = __ldg(a.in + d * a.N + s);
        b[d] = __ldg(a.in + (19 + d) * a.N + s);
    }
}

template <bool PULL>
__global__ void __launch_bounds__(CG3_BLOCK) cg3_density_kernel(const Cg3Args a) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, z = blockIdx.z;
    if (x >= a.nx) return;
    float r[19], b[19];
    cg3_gather<PULL>(a, Cg3Nb(a, x, y, z), r, b);
    float rr = 0.f, bb = 0.f;
#pragma unroll
    for (int d = 0; d < 19; ++d) {
        rr += r[d];
        bb += b[d];
    }
    const int node = x + a.nx * (y + a.ny * z);
    const float rho = rr + bb;
    a.phi[node] = (rr - bb) / rho;
    a.dn[node] = rho;
}

// Per-direction constants of the 3D colour-gradient model (GpuInit.cu:
// 896-940): lattice weight, perturbation offset B_k, rest weights phi_k and
// theta_k, enhanced-equilibrium chi_k and psi_k, gradient weight.
__device__ __forceinline__ float cg3_w(int k) { return k == 0 ? 1.f / 3.f : (k <= 6 ? 1.f / 18.f : 1.f / 36.f); }
__device__ __forceinline__ float cg3_bpert(int k) { return k == 0 ? -2.f / 9.f : (k <= 6 ? 1.f / 54.f : 1.f / 27.f); }
__device__ __forceinline__ float cg3_phi(int k) { return k == 0 ? 0.f : (k <= 6 ? 1.f / 12.f : 1.f / 24.f); }
__device__ __forceinline__ float cg3_teta(int k) { return k == 0 ? 1.f : (k <= 6 ? -1.f / 12.f : -1.f / 24.f); }
__device__ __forceinline__ float cg3_chi(int k) { return k == 0 ? -2.5f : (k <= 6 ? -1.f / 6.f : 1.f / 24.f); }
__device__ __forceinline__ float cg3_psi(int k) { return k == 0 ? 0.f : (k <= 6 ? 0.25f : 0.125f); }

// Weight of the 104-point isotropic gradient stencil (Shan's eighth-order 3D
// set) for an offset of squared length s2: shells 1, 2, 3, 4, 5, 6 and 9.
__device__ __forceinline__ float cg3_ho_weight(int s2) {
    switch (s2) {
    case 1: return 4.f / 45.f;
    case 2: return 1.f / 21.f;
    case 3: return 2.f / 105.f;
    case 4: return 5.f / 504.f;
    case 5: return 1.f / 315.f;
    case 6: return 1.f / 630.f;
    case 9: return 1.f / 5040.f;
    default: return 0.f;
    }
}

// One node's colour-gradient step: moments of the streamed colours, the
// colour and density gradients from the neighbours' densities (18 lattice
// neighbours, weights 1/6 and 1/12, or the 104-point set when HO), then per
// direction the BGK relaxation with omega from the harmonic mean viscosity,
// the phase-dependent rest weights phi_k + theta_k alpha, the perturbation
// A |g| (w_k (c_k.g)^2/|g|^2 - B_k) and the recolouring
// +/- beta rho_r rho_b / rho cos(c_k, g) (phi_k + theta_k alpha); ENH adds the
// enhanced equilibrium's nu (chi_k u.grad rho + psi_k G:c_k c_k).  Below the
// gradient limit the perturbation and the recolouring vanish.
template <bool PULL, bool HO, bool ENH>
__global__ void __launch_bounds__(CG3_BLOCK, CG3_MINB) cg3_collide_kernel(const Cg3Args a) {
    using L = Lat<19>;
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, z = blockIdx.z;
    if (x >= a.nx) return;
    const int plane = a.nx * a.ny;
    const int node = x + a.nx * y + plane * z;
    const Cg3Nb nb(a, x, y, z);
    float f[19], r_r = 0.f, b_r = 0.f, jx = 0.f, jy = 0.f, jz = 0.f;
    {
        float r[19], b[19];
        cg3_gather<PULL>(a, nb, r, b);
#pragma unroll
        for (int d = 0; d < 19; ++d) {
            f[d] = r[d] + b[d];
            r_r += r[d];
            b_r += b[d];
            if (L::cx(d)) jx += (float)L::cx(d) * f[d];
            if (L::cy(d)) jy += (float)L::cy(d) * f[d];
            if (L::cz(d)) jz += (float)L::cz(d) * f[d];
        }
    }
    const float rho = r_r + b_r;
    const float u = jx / rho, v = jy / rho, w = jz / rho;
    a.R[node] = r_r;
    a.B[node] = b_r;
    if (a.write_macro) {
        a.rho[node] = rho;
        a.ux[node] = u;
        a.uy[node] = v;
        a.uz[node] = w;
    }
    float cgx = 0.f, cgy = 0.f, cgz = 0.f, grx = 0.f, gry = 0.f, grz = 0.f;
    auto add = [&](int j, float wt, int ox, int oy, int oz) {
        const float a1 = wt * __ldg(a.phi + j);
        if (ENH) {
            const float a2 = wt * __ldg(a.dn + j);
            grx += a2 * (float)ox;
            gry += a2 * (float)oy;
            grz += a2 * (float)oz;
        }
        cgx += a1 * (float)ox;
        cgy += a1 * (float)oy;
        cgz += a1 * (float)oz;
    };
    if (HO) {
        int xo[5], yo[5], zo[5];
#pragma unroll
        for (int t = 0; t < 5; ++t) {
            xo[t] = cg3_wrap(x + t - 2, a.nx);
            yo[t] = a.nx * cg3_wrap(y + t - 2, a.ny);
            zo[t] = plane * cg3_wrap(z + t - 2, a.nz);
        }
#pragma unroll
        for (int ox = -2; ox <= 2; ++ox)
#pragma unroll
            for (int oy = -2; oy <= 2; ++oy)
#pragma unroll
                for (int oz = -2; oz <= 2; ++oz) {
                    const float wt = cg3_ho_weight(ox * ox + oy * oy + oz * oz);
                    if (wt == 0.f) continue;
                    add(xo[ox + 2] + yo[oy + 2] + zo[oz + 2], wt, ox, oy, oz);
                }
    } else {
#pragma unroll
        for (int k = 1; k < 19; ++k)
            add(nb.at(L::cx(k), L::cy(k), L::cz(k)), k <= 6 ? 1.f / 6.f : 1.f / 12.f, L::cx(k), L::cy(k), L::cz(k));
    }
    const float mean_nu = 1.f / (r_r / (rho * a.r_visc) + b_r / (rho * a.b_visc));
    const float omega_eff = 1.f / (3.f * mean_nu + 0.5f);
    const float mean_alpha = a.r_alpha * r_r / rho + a.b_alpha * b_r / rho;
    const float gnorm = sqrtf(cgx * cgx + cgy * cgy + cgz * cgz);
    const float k_r = r_r / rho, k_b = b_r / rho, k_k = a.beta * r_r * b_r / rho;
    const float cu1 = u * u + v * v + w * w;
    const float G1 = 2.f * u * grx, G2 = u * gry + v * grx, G3 = u * grz + w * grx;
    const float G5 = 2.f * v * gry, G6 = v * grz + w * gry, G9 = 2.f * w * grz;
    const float ugr = u * grx + v * gry + w * grz;
    const bool interface = gnorm > a.g_limit;
    // one reciprocal per node instead of two divisions per direction
    const float inv_g = interface ? 1.f / gnorm : 0.f, inv_g2 = inv_g * inv_g;
    float *rout = a.out + node, *bout = a.out + 19 * a.N + node;
#pragma unroll
    for (int k = 0; k < 19; ++k) {
        const float cx = (float)L::cx(k), cy = (float)L::cy(k), cz = (float)L::cz(k);
        const float wk = cg3_w(k);
        float pert = 0.f, cosin = 0.f;
        if (interface) {
            const float pcg = cx * cgx + cy * cgy + cz * cgz;
            if (k != 0) cosin = pcg * inv_g * (k <= 6 ? 1.f : 0.70710678f);
            pert = a.A * gnorm * (wk * (pcg * pcg) * inv_g2 - cg3_bpert(k));
        }
        const float cu2 = u * cx + v * cy + w * cz;
        const float rest = cg3_phi(k) + cg3_teta(k) * mean_alpha;
        float feq = rho * (rest + wk * (3.f * cu2 + 4.5f * cu2 * cu2 - 1.5f * cu1));
        if (ENH) {
            const float TC = G1 * (cx * cx) + 2.f * G2 * (cx * cy) + 2.f * G3 * (cx * cz) + G5 * (cy * cy) +
                             2.f * G6 * (cy * cz) + G9 * (cz * cz);
            feq += mean_nu * (cg3_chi(k) * ugr + cg3_psi(k) * TC);
        }
        const float fp = omega_eff * feq + (1.f - omega_eff) * f[k] + pert;
        rout[k * a.N] = k_r * fp + k_k * cosin * rest;
        bout[k * a.N] = k_b * fp - k_k * cosin * rest;
    }
}

}  // namespace lbm
