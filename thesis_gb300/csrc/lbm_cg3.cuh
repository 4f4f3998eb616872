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
#include "lbm_cg_store.cuh"
#include "lbm_device.cuh"

namespace lbm {

struct Cg3Args {
    const void *in;    // slot c of direction d at (c*19 + d)*N (lbm_cg_store.cuh)
    void *out;
    float *R, *B;      // colour densities (output)
    void *phi, *dn;    // colour field and density of the streamed state (gradients), arithmetic type
    float *rho, *ux, *uy, *uz;
    int nx, ny, nz;
    long long N;
    int write_macro;
    double r_alpha, b_alpha, r_visc, b_visc, beta, A, g_limit;
    float scale, inv_scale;  // F16S: S and 1/S of the summed population
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
template <int ST, bool PULL>
__device__ __forceinline__ void cg3_gather(const Cg3Args &a, const Cg3Nb &nb, typename CgStore<ST>::R (&r)[19],
                                           typename CgStore<ST>::R (&b)[19]) {
    using L = Lat<19>;
    using SP = CgStore<ST>;
    using T = typename SP::T;
    using R = typename SP::R;
    const T *in = (const T *)a.in;
#pragma unroll
    for (int d = 0; d < 19; ++d) {
        const int s = PULL ? nb.at(-L::cx(d), -L::cy(d), -L::cz(d)) : nb.at(0, 0, 0);
        SP::load(in + d * a.N + s, in + (19 + d) * a.N + s, (R)L::w(d), (R)a.inv_scale, r[d], b[d]);
    }
}

template <int ST, bool PULL>
__global__ void __launch_bounds__(CG3_BLOCK) cg3_density_kernel(const Cg3Args a) {
    using R = typename CgStore<ST>::R;
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, z = blockIdx.z;
    if (x >= a.nx) return;
    R r[19], b[19];
    cg3_gather<ST, PULL>(a, Cg3Nb(a, x, y, z), r, b);
    R rr = 0, bb = 0;
#pragma unroll
    for (int d = 0; d < 19; ++d) {
        rr += r[d];
        bb += b[d];
    }
    const int node = x + a.nx * (y + a.ny * z);
    const R rho = rr + bb;
    ((R *)a.phi)[node] = (rr - bb) / rho;
    ((R *)a.dn)[node] = rho;
}

// Per-direction constants of the 3D colour-gradient model (GpuInit.cu:
// 896-940): lattice weight, perturbation offset B_k, rest weights phi_k and
// theta_k, enhanced-equilibrium chi_k and psi_k, gradient weight.
template <class R = float> __device__ __forceinline__ R cg3_w(int k) {
    return k == 0 ? (R)(1. / 3.) : (k <= 6 ? (R)(1. / 18.) : (R)(1. / 36.));
}
template <class R = float> __device__ __forceinline__ R cg3_bpert(int k) {
    return k == 0 ? (R)(-2. / 9.) : (k <= 6 ? (R)(1. / 54.) : (R)(1. / 27.));
}
template <class R = float> __device__ __forceinline__ R cg3_phi(int k) {
    return k == 0 ? (R)0 : (k <= 6 ? (R)(1. / 12.) : (R)(1. / 24.));
}
template <class R = float> __device__ __forceinline__ R cg3_teta(int k) {
    return k == 0 ? (R)1 : (k <= 6 ? (R)(-1. / 12.) : (R)(-1. / 24.));
}
template <class R = float> __device__ __forceinline__ R cg3_chi(int k) {
    return k == 0 ? (R)-2.5 : (k <= 6 ? (R)(-1. / 6.) : (R)(1. / 24.));
}
template <class R = float> __device__ __forceinline__ R cg3_psi(int k) {
    return k == 0 ? (R)0 : (k <= 6 ? (R)0.25 : (R)0.125);
}

// Weight of the 104-point isotropic gradient stencil (Shan's eighth-order 3D
// set) for an offset of squared length s2: shells 1, 2, 3, 4, 5, 6 and 9.
template <class R = float> __device__ __forceinline__ R cg3_ho_weight(int s2) {
    switch (s2) {
    case 1: return (R)(4. / 45.);
    case 2: return (R)(1. / 21.);
    case 3: return (R)(2. / 105.);
    case 4: return (R)(5. / 504.);
    case 5: return (R)(1. / 315.);
    case 6: return (R)(1. / 630.);
    case 9: return (R)(1. / 5040.);
    default: return (R)0;
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
template <int ST, bool PULL, bool HO, bool ENH>
__global__ void __launch_bounds__(CG3_BLOCK, CG3_MINB) cg3_collide_kernel(const Cg3Args a) {
    using L = Lat<19>;
    using SP = CgStore<ST>;
    using T = typename SP::T;
    using R = typename SP::R;
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, z = blockIdx.z;
    if (x >= a.nx) return;
    const int plane = a.nx * a.ny;
    const int node = x + a.nx * y + plane * z;
    const Cg3Nb nb(a, x, y, z);
    const R *phi = (const R *)a.phi, *dn = (const R *)a.dn;
    R f[19], r_r = 0, b_r = 0, jx = 0, jy = 0, jz = 0;
    {
        R r[19], b[19];
        cg3_gather<ST, PULL>(a, nb, r, b);
#pragma unroll
        for (int d = 0; d < 19; ++d) {
            f[d] = r[d] + b[d];
            r_r += r[d];
            b_r += b[d];
            if (L::cx(d)) jx += (R)L::cx(d) * f[d];
            if (L::cy(d)) jy += (R)L::cy(d) * f[d];
            if (L::cz(d)) jz += (R)L::cz(d) * f[d];
        }
    }
    const R rho = r_r + b_r;
    const R u = jx / rho, v = jy / rho, w = jz / rho;
    a.R[node] = (float)r_r;
    a.B[node] = (float)b_r;
    if (a.write_macro) {
        a.rho[node] = (float)rho;
        a.ux[node] = (float)u;
        a.uy[node] = (float)v;
        a.uz[node] = (float)w;
    }
    R cgx = 0, cgy = 0, cgz = 0, grx = 0, gry = 0, grz = 0;
    auto add = [&](int j, R wt, int ox, int oy, int oz) {
        const R a1 = wt * __ldg(phi + j);
        if (ENH) {
            const R a2 = wt * __ldg(dn + j);
            grx += a2 * (R)ox;
            gry += a2 * (R)oy;
            grz += a2 * (R)oz;
        }
        cgx += a1 * (R)ox;
        cgy += a1 * (R)oy;
        cgz += a1 * (R)oz;
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
                    const R wt = cg3_ho_weight<R>(ox * ox + oy * oy + oz * oz);
                    if (wt == (R)0) continue;
                    add(xo[ox + 2] + yo[oy + 2] + zo[oz + 2], wt, ox, oy, oz);
                }
    } else {
#pragma unroll
        for (int k = 1; k < 19; ++k)
            add(nb.at(L::cx(k), L::cy(k), L::cz(k)), k <= 6 ? (R)(1. / 6.) : (R)(1. / 12.), L::cx(k), L::cy(k),
                L::cz(k));
    }
    const R mean_nu = (R)1 / (r_r / (rho * (R)a.r_visc) + b_r / (rho * (R)a.b_visc));
    const R omega_eff = (R)1 / ((R)3 * mean_nu + (R)0.5);
    const R mean_alpha = (R)a.r_alpha * r_r / rho + (R)a.b_alpha * b_r / rho;
    const R gnorm = sqrt(cgx * cgx + cgy * cgy + cgz * cgz);
    const R k_r = r_r / rho, k_b = b_r / rho, k_k = (R)a.beta * r_r * b_r / rho;
    const R cu1 = u * u + v * v + w * w;
    const R G1 = (R)2 * u * grx, G2 = u * gry + v * grx, G3 = u * grz + w * grx;
    const R G5 = (R)2 * v * gry, G6 = v * grz + w * gry, G9 = (R)2 * w * grz;
    const R ugr = u * grx + v * gry + w * grz;
    const bool interface = gnorm > (R)a.g_limit;
    // one reciprocal per node instead of two divisions per direction
    const R inv_g = interface ? (R)1 / gnorm : (R)0, inv_g2 = inv_g * inv_g;
    const R A = (R)a.A;
    T *out = (T *)a.out;
#pragma unroll
    for (int k = 0; k < 19; ++k) {
        const R cx = (R)L::cx(k), cy = (R)L::cy(k), cz = (R)L::cz(k);
        const R wk = cg3_w<R>(k);
        R pert = 0, cosin = 0;
        if (interface) {
            const R pcg = cx * cgx + cy * cgy + cz * cgz;
            if (k != 0) cosin = pcg * inv_g * (k <= 6 ? (R)1 : (R)0.70710678118654752);
            pert = A * gnorm * (wk * (pcg * pcg) * inv_g2 - cg3_bpert<R>(k));
        }
        const R cu2 = u * cx + v * cy + w * cz;
        const R rest = cg3_phi<R>(k) + cg3_teta<R>(k) * mean_alpha;
        R feq = rho * (rest + wk * ((R)3 * cu2 + (R)4.5 * cu2 * cu2 - (R)1.5 * cu1));
        if (ENH) {
            const R TC = G1 * (cx * cx) + (R)2 * G2 * (cx * cy) + (R)2 * G3 * (cx * cz) + G5 * (cy * cy) +
                         (R)2 * G6 * (cy * cz) + G9 * (cz * cz);
            feq += mean_nu * (cg3_chi<R>(k) * ugr + cg3_psi<R>(k) * TC);
        }
        const R fp = omega_eff * feq + ((R)1 - omega_eff) * f[k] + pert;
        SP::store(out + k * a.N + node, out + (19 + k) * a.N + node, (R)L::w(k), (R)a.scale,
                  k_r * fp + k_k * cosin * rest, k_b * fp - k_k * cosin * rest);
    }
}

}  // namespace lbm
