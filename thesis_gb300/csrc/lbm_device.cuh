// Device-side building blocks of the fused lattice-Boltzmann step for sm_103a:
// lattice tables, population storage formats, collision operators and the
// node-local boundary conditions.  One thread owns one lattice node for a whole
// time step: pull-stream -> boundary -> macroscopic moments -> collision, with
// the populations kept in registers between the phases.
//
// Direction order, weights and pull offsets follow the reference solver
// (Source code/lbm-solver_final/GpuInit.cu:94-99 for D2Q9, :822-842 for
// D3Q19) so that populations can be exchanged with its SoA layout
// f[d*N + node], node = x + nx*(y + ny*z).
#pragma once
#include <cuda_fp16.h>
#include <stdint.h>

#include "lbm_types.h"

namespace lbm {

// ---------------------------------------------------------------------------
// Lattice tables as constexpr functions: inside fully unrolled loops every
// lookup folds to an immediate, so no constant-memory traffic remains.
// ---------------------------------------------------------------------------
template <int Q> struct Lat;

template <> struct Lat<9> {
    static constexpr int Q = 9;
    __host__ __device__ static constexpr int cx(int d) {
        return (d == 1 || d == 5 || d == 8) ? 1 : ((d == 3 || d == 6 || d == 7) ? -1 : 0);
    }
    __host__ __device__ static constexpr int cy(int d) {
        return (d == 2 || d == 5 || d == 6) ? 1 : ((d == 4 || d == 7 || d == 8) ? -1 : 0);
    }
    __host__ __device__ static constexpr int cz(int) { return 0; }
    __host__ __device__ static constexpr int opp(int d) {
        return d == 0 ? 0 : (d <= 4 ? ((d + 1) % 4) + 1 : ((d - 5 + 2) % 4) + 5);
    }
    __host__ __device__ static constexpr double w(int d) {
        return d == 0 ? 4.0 / 9.0 : (d <= 4 ? 1.0 / 9.0 : 1.0 / 36.0);
    }
};

template <> struct Lat<19> {
    static constexpr int Q = 19;
    __host__ __device__ static constexpr int cx(int d) {
        return (d == 1 || d == 7 || d == 9 || d == 11 || d == 13) ? 1
               : ((d == 2 || d == 8 || d == 10 || d == 12 || d == 14) ? -1 : 0);
    }
    __host__ __device__ static constexpr int cy(int d) {
        return (d == 3 || d == 7 || d == 8 || d == 15 || d == 17) ? 1
               : ((d == 4 || d == 9 || d == 10 || d == 16 || d == 18) ? -1 : 0);
    }
    __host__ __device__ static constexpr int cz(int d) {
        return (d == 5 || d == 11 || d == 12 || d == 15 || d == 16) ? 1
               : ((d == 6 || d == 13 || d == 14 || d == 17 || d == 18) ? -1 : 0);
    }
    __host__ __device__ static constexpr int opp(int d) {
        return d == 0 ? 0 : (d <= 6 ? (d % 2 ? d + 1 : d - 1) : (d <= 10 ? 17 - d : (d <= 14 ? 25 - d : 33 - d)));
    }
    __host__ __device__ static constexpr double w(int d) {
        return d == 0 ? 1.0 / 3.0 : (d <= 6 ? 1.0 / 18.0 : 1.0 / 36.0);
    }
};

// D2Q9 and D3Q19 moment bases of the reference MRT (CellFunctions.cu:31-40,
// :94-113).  Rows are orthogonal, so M^-1 = M^T diag(1/|row|^2).
__host__ __device__ constexpr int mrt2(int k, int i) {
    constexpr int M[81] = {1, 1, 1, 1, 1, 1, 1, 1, 1,   -4, -1, -1, -1, -1, 2, 2, 2, 2,
                           4, -2, -2, -2, -2, 1, 1, 1, 1, 0, 1, 0, -1, 0, 1, -1, -1, 1,
                           0, -2, 0, 2, 0, 1, -1, -1, 1, 0, 0, 1, 0, -1, 1, 1, -1, -1,
                           0, 0, -2, 0, 2, 1, 1, -1, -1, 0, 1, -1, 1, -1, 0, 0, 0, 0,
                           0, 0, 0, 0, 0, 1, -1, 1, -1};
    return M[k * 9 + i];
}
__host__ __device__ constexpr int mrt2_norm(int k) {
    constexpr int N[9] = {9, 36, 36, 6, 12, 6, 12, 4, 4};
    return N[k];
}
__host__ __device__ constexpr int mrt3(int k, int i) {
    constexpr int M[361] = {
        1,   1,   1,   1,   1,   1,   1,   1,  1,  1,  1,  1,  1,  1,  1,  1,  1,  1,  1,
        -30, -11, -11, -11, -11, -11, -11, 8,  8,  8,  8,  8,  8,  8,  8,  8,  8,  8,  8,
        12,  -4,  -4,  -4,  -4,  -4,  -4,  1,  1,  1,  1,  1,  1,  1,  1,  1,  1,  1,  1,
        0,   1,   -1,  0,   0,   0,   0,   1,  -1, 1,  -1, 1,  -1, 1,  -1, 0,  0,  0,  0,
        0,   -4,  4,   0,   0,   0,   0,   1,  -1, 1,  -1, 1,  -1, 1,  -1, 0,  0,  0,  0,
        0,   0,   0,   1,   -1,  0,   0,   1,  1,  -1, -1, 0,  0,  0,  0,  1,  -1, 1,  -1,
        0,   0,   0,   -4,  4,   0,   0,   1,  1,  -1, -1, 0,  0,  0,  0,  1,  -1, 1,  -1,
        0,   0,   0,   0,   0,   1,   -1,  0,  0,  0,  0,  1,  1,  -1, -1, 1,  1,  -1, -1,
        0,   0,   0,   0,   0,   -4,  4,   0,  0,  0,  0,  1,  1,  -1, -1, 1,  1,  -1, -1,
        0,   2,   2,   -1,  -1,  -1,  -1,  1,  1,  1,  1,  1,  1,  1,  1,  -2, -2, -2, -2,
        0,   -4,  -4,  2,   2,   2,   2,   1,  1,  1,  1,  1,  1,  1,  1,  -2, -2, -2, -2,
        0,   0,   0,   1,   1,   -1,  -1,  1,  1,  1,  1,  -1, -1, -1, -1, 0,  0,  0,  0,
        0,   0,   0,   -2,  -2,  2,   2,   1,  1,  1,  1,  -1, -1, -1, -1, 0,  0,  0,  0,
        0,   0,   0,   0,   0,   0,   0,   1,  -1, -1, 1,  0,  0,  0,  0,  0,  0,  0,  0,
        0,   0,   0,   0,   0,   0,   0,   0,  0,  0,  0,  0,  0,  0,  0,  1,  -1, -1, 1,
        0,   0,   0,   0,   0,   0,   0,   0,  0,  0,  0,  1,  -1, -1, 1,  0,  0,  0,  0,
        0,   0,   0,   0,   0,   0,   0,   1,  -1, 1,  -1, -1, 1,  -1, 1,  0,  0,  0,  0,
        0,   0,   0,   0,   0,   0,   0,   -1, -1, 1,  1,  0,  0,  0,  0,  1,  -1, 1,  -1,
        0,   0,   0,   0,   0,   0,   0,   0,  0,  0,  0,  1,  1,  -1, -1, -1, -1, 1,  1};
    return M[k * 19 + i];
}
__host__ __device__ constexpr int mrt3_norm(int k) {
    constexpr int N[19] = {19, 2394, 252, 10, 40, 10, 40, 10, 40, 36, 72, 12, 24, 4, 4, 4, 8, 8, 8};
    return N[k];
}

// ---------------------------------------------------------------------------
// Population storage.  F32 and F64 hold f itself; F16S holds the scaled
// deviation from the rest-state weight, h = (f - w_d) * scale, so the few
// significant digits of a slow flow land in FP16's normal range.
// ---------------------------------------------------------------------------
template <int ST> struct Store;
template <> struct Store<LBM_STORE_F32> {
    using T = float;   // element type in HBM
    using R = float;   // arithmetic type
    __device__ static __forceinline__ R load(const T *p, double, float) { return __ldg(p); }
    __device__ static __forceinline__ void store(T *p, R v, double, float) { *p = v; }
    __device__ static __forceinline__ T encode(R v, double, float) { return v; }
};
template <> struct Store<LBM_STORE_F16S> {
    using T = __half;
    using R = float;
    __device__ static __forceinline__ R load(const T *p, double w, float inv_scale) {
        return fmaf(__half2float(__ldg(p)), inv_scale, (float)w);
    }
    __device__ static __forceinline__ T encode(R v, double w, float scale) {
        return __float2half_rn((v - (float)w) * scale);
    }
    __device__ static __forceinline__ void store(T *p, R v, double w, float scale) {
        *p = encode(v, w, scale);
    }
};
template <> struct Store<LBM_STORE_F64> {
    using T = double;
    using R = double;
    __device__ static __forceinline__ R load(const T *p, double, float) { return __ldg(p); }
    __device__ static __forceinline__ void store(T *p, R v, double, float) { *p = v; }
    __device__ static __forceinline__ T encode(R v, double, float) { return v; }
};

// ---------------------------------------------------------------------------
// Equilibrium and collision operators (GpuCollision.cu:21-32, :528-550,
// :882-1170).  R is float for F32/F16S storage and double for F64.
// ---------------------------------------------------------------------------
template <int Q, class R>
__device__ __forceinline__ R feq(int d, R rho, R ux, R uy, R uz, R usq15) {
    using L = Lat<Q>;
    const R cu = (R)L::cx(d) * ux + (R)L::cy(d) * uy + (R)L::cz(d) * uz;
    return (R)L::w(d) * rho * ((R)1 + (R)3 * cu + (R)4.5 * cu * cu - usq15);
}

template <int Q, class R>
__device__ __forceinline__ void collide_bgk(R (&f)[Q], R rho, R ux, R uy, R uz, R omega) {
    const R usq15 = (R)1.5 * (ux * ux + uy * uy + uz * uz);
#pragma unroll
    for (int d = 0; d < Q; ++d) f[d] = f[d] - omega * (f[d] - feq<Q>(d, rho, ux, uy, uz, usq15));
}

// Two-relaxation-time: symmetric part relaxes with omega, antisymmetric with
// omega_minus = 8(2-omega)/(8-omega) (GpuInit.cu:103).
template <int Q, class R>
__device__ __forceinline__ void collide_trt(R (&f)[Q], R rho, R ux, R uy, R uz, R omega, R omega_m) {
    using L = Lat<Q>;
    const R usq15 = (R)1.5 * (ux * ux + uy * uy + uz * uz);
    R fe[Q];
#pragma unroll
    for (int d = 0; d < Q; ++d) fe[d] = feq<Q>(d, rho, ux, uy, uz, usq15);
    R out[Q];
#pragma unroll
    for (int d = 0; d < Q; ++d) {
        const int o = L::opp(d);
        const R sp = (R)0.5 * (f[d] + f[o] - fe[d] - fe[o]);
        const R sm = (R)0.5 * (f[d] - f[o] - fe[d] + fe[o]);
        out[d] = f[d] - omega * sp - omega_m * sm;
    }
#pragma unroll
    for (int d = 0; d < Q; ++d) f[d] = out[d];
}

// D2Q9 MRT with the reference relaxation rates s = (1, 1.4, 1.4, 1, 1.2, 1,
// 1.2, omega, omega) (CellFunctions.cu:47-55).  REF keeps the reference's
// energy equilibria rho(-2 + 3 rho |u|^2), rho(1 - 3 rho |u|^2)
// (GpuCollision.cu:987-988); otherwise -2 rho + 3 rho |u|^2 and
// rho - 3 rho |u|^2.
template <bool REF, class R>
__device__ __forceinline__ void collide_mrt9(R (&f)[9], R rho, R ux, R uy, R omega) {
    const R usq = ux * ux + uy * uy;
    const R ef = REF ? rho : (R)1;
    R meq[9];
    meq[0] = rho;
    meq[1] = rho * ((R)-2 + (R)3 * ef * usq);
    meq[2] = rho * ((R)1 - (R)3 * ef * usq);
    meq[3] = rho * ux;
    meq[4] = -rho * ux;
    meq[5] = rho * uy;
    meq[6] = -rho * uy;
    meq[7] = rho * (ux * ux - uy * uy);
    meq[8] = rho * ux * uy;
    const R s[9] = {(R)1, (R)1.4, (R)1.4, (R)1, (R)1.2, (R)1, (R)1.2, omega, omega};
    R dm[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        R m = 0;
#pragma unroll
        for (int i = 0; i < 9; ++i)
            if (mrt2(k, i) != 0) m += (R)mrt2(k, i) * f[i];
        dm[k] = s[k] * (m - meq[k]) * ((R)1 / (R)mrt2_norm(k));
    }
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        R c = 0;
#pragma unroll
        for (int k = 0; k < 9; ++k)
            if (mrt2(k, i) != 0) c += (R)mrt2(k, i) * dm[k];
        f[i] -= c;
    }
}

// D3Q19 MRT (d'Humieres basis, incompressible equilibria with rho0 = 1,
// GpuCollision.cu:1062-1083) with s = (0, 1.19, 1.4, 0, 1.2, 0, 1.2, 0, 1.2,
// omega, 1.4, omega, 1.4, omega, omega, omega, 1.98, 1.98, 1.98).  The
// conserved moments (s = 0) are skipped.  REF reproduces the reference's
// unwritten direction 18 (GpuCollision.cu:1161): its post-collision value is
// the zero the buffer was initialised with.
template <bool REF, class R>
__device__ __forceinline__ void collide_mrt19(R (&f)[19], R rho, R ux, R uy, R uz, R omega) {
    const R jx = rho * ux, jy = rho * uy, jz = rho * uz;
    const R jsq = jx * jx + jy * jy + jz * jz;
    R meq[19];
    meq[0] = rho;
    meq[1] = (R)-11 * rho + (R)19 * jsq;
    meq[2] = (R)(-475.0 / 63.0) * jsq;
    meq[3] = jx;
    meq[4] = (R)(-2.0 / 3.0) * jx;
    meq[5] = jy;
    meq[6] = (R)(-2.0 / 3.0) * jy;
    meq[7] = jz;
    meq[8] = (R)(-2.0 / 3.0) * jz;
    meq[9] = (R)2 * jx * jx - (jy * jy + jz * jz);
    meq[10] = 0;
    meq[11] = jy * jy - jz * jz;
    meq[12] = 0;
    meq[13] = jx * jy;
    meq[14] = jy * jz;
    meq[15] = jx * jz;
    meq[16] = 0;
    meq[17] = 0;
    meq[18] = 0;
    const R s[19] = {0,     (R)1.19, (R)1.4, 0,     (R)1.2, 0,     (R)1.2,  0,       (R)1.2, omega,
                     (R)1.4, omega,  (R)1.4, omega, omega,  omega, (R)1.98, (R)1.98, (R)1.98};
    R dm[19];
#pragma unroll
    for (int k = 0; k < 19; ++k) {
        if (k == 0 || k == 3 || k == 5 || k == 7) {
            dm[k] = 0;
            continue;
        }
        R m = 0;
#pragma unroll
        for (int i = 0; i < 19; ++i)
            if (mrt3(k, i) != 0) m += (R)mrt3(k, i) * f[i];
        dm[k] = s[k] * (m - meq[k]) * ((R)1 / (R)mrt3_norm(k));
    }
#pragma unroll
    for (int i = 0; i < 19; ++i) {
        R c = 0;
#pragma unroll
        for (int k = 0; k < 19; ++k)
            if (mrt3(k, i) != 0 && !(k == 0 || k == 3 || k == 5 || k == 7)) c += (R)mrt3(k, i) * dm[k];
        f[i] -= c;
    }
    if (REF) f[18] = 0;
}

}  // namespace lbm
