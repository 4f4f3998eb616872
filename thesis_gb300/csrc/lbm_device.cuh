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

// Rest-state populations of a collision model, the F16S storage shift.
__host__ __device__ constexpr double rest_shift(int q, int coll, int d);

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

// w_d for BGK/TRT and the D2Q9 MRT (whose rest state is w); for the D3Q19
// MRT, w_d minus the eps-moment part 3/252 * M_eps,d that its zero-density
// eps equilibrium removes (w -> 4/21, 13/126, 1/63).
__host__ __device__ constexpr double rest_shift(int q, int coll, int d) {
    return q == 9 ? Lat<9>::w(d)
                  : (coll == LBM_MRT ? Lat<19>::w(d) - 3.0 / 252.0 * mrt3(2, d) : Lat<19>::w(d));
}

// ---------------------------------------------------------------------------
// Population storage.  F32 and F64 hold f itself; F16S holds the scaled
// deviation from the collision model's rest state, h = (f - shift_d) * scale,
// so the few significant digits of a slow flow land in FP16's normal range.
// The shift is the lattice weights w_d, except for the D3Q19 MRT whose
// incompressible energy-square equilibrium (eps_eq = -475/63 j^2, no density
// term) puts its rest state at w_d - (3/252) M_eps,d (rest_shift below).
// ---------------------------------------------------------------------------
// F16C: a 16-bit float with 1 sign, 4 exponent and 11 mantissa bits,
// exponent bias 15: (1 + m/2^11) 2^(E-15) for E = 1..15 ([2^-14, 2)), m 2^-25
// for E = 0.  Rounding to nearest even from FP32; magnitudes from 2 up
// saturate to the largest value; a non-finite input becomes 0xFFFF, which
// decodes to NaN, so a diverging run still shows non-finite fields.
struct f16c_t {
    unsigned short bits;
};
__device__ __forceinline__ f16c_t f16c_from_float(float x) {
    const unsigned int b = __float_as_uint(x);
    const unsigned int sign = (b >> 16) & 0x8000u;
    const unsigned int a = b & 0x7FFFFFFFu;
    unsigned int out;
    if (a >= 0x7F800000u) {
        return f16c_t{0xFFFFu};
    } else if (a < 0x38800000u) {  // below 2^-14: subnormal, steps of 2^-25
        out = (unsigned int)__float2int_rn(__uint_as_float(a) * 33554432.0f);
    } else {
        const unsigned int r = a + 0x7FFu + ((a >> 12) & 1u);  // round the 12 dropped bits to nearest even
        out = (r >> 12) - (112u << 11);
        if (out > 0x7FFFu) out = 0x7FFFu;
    }
    if (sign && out == 0x7FFFu) out = 0x7FFEu;  // 0xFFFF is reserved for NaN
    return f16c_t{(unsigned short)(sign | out)};
}
__device__ __forceinline__ float f16c_to_float(f16c_t v) {
    const unsigned int u = v.bits;
    if (u == 0xFFFFu) return __uint_as_float(0x7FC00000u);
    const unsigned int a = u & 0x7FFFu;
    const float m = a < 0x800u ? (float)a * 2.98023223876953125e-8f  // 2^-25
                               : __uint_as_float((a << 12) + (112u << 23));
    return (u & 0x8000u) ? -m : m;
}
// Read-only population load.  HINT 1 asks L2 to fetch the whole 256-byte
// block around the address from DRAM (ld.global.nc.L2::256B), so the
// neighbouring warps that read the rest of the block hit L2.
template <int HINT>
__device__ __forceinline__ __half ld_pop(const __half *p) {
    if (HINT == 1) {
        unsigned short v;
        asm("ld.global.nc.L2::256B.b16 %0, [%1];" : "=h"(v) : "l"(p));
        return __ushort_as_half(v);
    }
    return __ldg(p);
}
template <int HINT>
__device__ __forceinline__ float ld_pop(const float *p) {
    if (HINT == 1) {
        float v;
        asm("ld.global.nc.L2::256B.f32 %0, [%1];" : "=f"(v) : "l"(p));
        return v;
    }
    return __ldg(p);
}
template <int HINT>
__device__ __forceinline__ f16c_t ld_pop(const f16c_t *p) {
    if (HINT == 1) {
        unsigned short v;
        asm("ld.global.nc.L2::256B.b16 %0, [%1];" : "=h"(v) : "l"(&p->bits));
        return f16c_t{v};
    }
    return f16c_t{__ldg(&p->bits)};
}
template <int HINT>
__device__ __forceinline__ double ld_pop(const double *p) {
    if (HINT == 1) {
        double v;
        asm("ld.global.nc.L2::256B.f64 %0, [%1];" : "=d"(v) : "l"(p));
        return v;
    }
    return __ldg(p);
}

template <int ST> struct Store;
// F32 holds f - shift: the deviation from the collision model's rest state in
// physics mode (shift 0 in reference mode, which keeps the reference's f).
template <> struct Store<LBM_STORE_F32> {
    using T = float;   // element type in HBM
    using R = float;   // arithmetic type
    __device__ static __forceinline__ R load(const T *p, float w, float) { return __ldg(p) + w; }
    __device__ static __forceinline__ R decode(T v, float w, float) { return v + w; }
    __device__ static __forceinline__ void store(T *p, R v, float w, float) { *p = v - w; }
    __device__ static __forceinline__ T encode(R v, float w, float) { return v - w; }
    // read-back and restart in FP64: f = v + w is exact in double, so a
    // decode64 / encode64 round trip returns the stored value
    __device__ static __forceinline__ double decode64(T v, float w, float) { return (double)v + (double)w; }
    __device__ static __forceinline__ T encode64(double v, float w, float) { return (float)(v - (double)w); }
};
template <> struct Store<LBM_STORE_F16S> {
    using T = __half;
    using R = float;
    __device__ static __forceinline__ R load(const T *p, float w, float inv_scale) {
        return fmaf(__half2float(__ldg(p)), inv_scale, w);
    }
    __device__ static __forceinline__ R decode(T v, float w, float inv_scale) {
        return fmaf(__half2float(v), inv_scale, w);
    }
    __device__ static __forceinline__ T encode(R v, float w, float scale) {
        return __float2half_rn((v - w) * scale);
    }
    __device__ static __forceinline__ void store(T *p, R v, float w, float scale) {
        *p = encode(v, w, scale);
    }
    __device__ static __forceinline__ double decode64(T v, float w, float inv_scale) {
        return (double)__half2float(v) * (double)inv_scale + (double)w;
    }
    __device__ static __forceinline__ T encode64(double v, float w, float scale) {
        return __float2half_rn((float)((v - (double)w) * (double)scale));
    }
};
template <> struct Store<LBM_STORE_F16C> {
    using T = f16c_t;
    using R = float;
    __device__ static __forceinline__ R load(const T *p, float w, float inv_scale) {
        return fmaf(f16c_to_float(T{__ldg(&p->bits)}), inv_scale, w);
    }
    __device__ static __forceinline__ R decode(T v, float w, float inv_scale) {
        return fmaf(f16c_to_float(v), inv_scale, w);
    }
    __device__ static __forceinline__ T encode(R v, float w, float scale) { return f16c_from_float((v - w) * scale); }
    __device__ static __forceinline__ void store(T *p, R v, float w, float scale) { *p = encode(v, w, scale); }
    __device__ static __forceinline__ double decode64(T v, float w, float inv_scale) {
        return (double)f16c_to_float(v) * (double)inv_scale + (double)w;
    }
    __device__ static __forceinline__ T encode64(double v, float w, float scale) {
        return f16c_from_float((float)((v - (double)w) * (double)scale));
    }
};
template <> struct Store<LBM_STORE_F64> {
    using T = double;
    using R = double;
    __device__ static __forceinline__ R load(const T *p, float, float) { return __ldg(p); }
    __device__ static __forceinline__ R decode(T v, float, float) { return v; }
    __device__ static __forceinline__ void store(T *p, R v, float, float) { *p = v; }
    __device__ static __forceinline__ T encode(R v, float, float) { return v; }
    __device__ static __forceinline__ double decode64(T v, float, float) { return v; }
    __device__ static __forceinline__ T encode64(double v, float, float) { return v; }
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
// omega, 1.4, omega, 1.4, omega, omega, omega, 1.98, 1.98, 1.98).
//
// The basis rows are even or odd under c -> -c, so with the nine opposite
// pairs (i, opp i) split into sums s = f_i + f_opp and differences
// a = f_i - f_opp, even moments need only the sums and odd moments only the
// differences; the correction c = M^T diag(1/|m_k|^2) S (m - m_eq) splits the
// same way, c_i = E + O and c_opp = E - O.  Shared partial sums bring the
// transform to about 200 FLOPs instead of two dense 19x19 products.
// Pairs (first member along +): X (1,2) Y (3,4) Z (5,6) A (7,10: +x+y)
// B (8,9: -x+y) C (11,14: +x+z) D (12,13: -x+z) E (15,18: +y+z) F (16,17: -y+z).
// REF reproduces the reference's unwritten direction 18 (GpuCollision.cu:1161):
// its post-collision value is the zero the buffer was initialised with.
template <bool REF, class R>
__host__ __device__ __forceinline__ void collide_mrt19(R (&f)[19], R rho, R ux, R uy, R uz, R omega) {
    const R sX = f[1] + f[2], aX = f[1] - f[2];
    const R sY = f[3] + f[4], aY = f[3] - f[4];
    const R sZ = f[5] + f[6], aZ = f[5] - f[6];
    const R sA = f[7] + f[10], aA = f[7] - f[10];
    const R sB = f[8] + f[9], aB = f[8] - f[9];
    const R sC = f[11] + f[14], aC = f[11] - f[14];
    const R sD = f[12] + f[13], aD = f[12] - f[13];
    const R sE = f[15] + f[18], aE = f[15] - f[18];
    const R sF = f[16] + f[17], aF = f[16] - f[17];
    const R sAxis = sX + sY + sZ;
    const R sABCD = (sA + sB) + (sC + sD), sEF = sE + sF;
    const R sDiag = sABCD + sEF;
    const R f0 = f[0];
    // non-conserved moments
    const R m1 = (R)-30 * f0 + (R)-11 * sAxis + (R)8 * sDiag;
    const R m2 = (R)12 * f0 + (R)-4 * sAxis + sDiag;
    const R m4 = (R)-4 * aX + ((aA - aB) + (aC - aD));
    const R m6 = (R)-4 * aY + ((aA + aB) + (aE - aF));
    const R m8 = (R)-4 * aZ + ((aC + aD) + (aE + aF));
    const R m9 = (R)2 * sX - (sY + sZ) + sABCD - (R)2 * sEF;
    const R m10 = (R)-4 * sX + (R)2 * (sY + sZ) + sABCD - (R)2 * sEF;
    const R m11 = (sY - sZ) + (sA + sB) - (sC + sD);
    const R m12 = (R)2 * (sZ - sY) + (sA + sB) - (sC + sD);
    const R m13 = sA - sB, m14 = sE - sF, m15 = sC - sD;
    const R m16 = (aA - aB) - (aC - aD);
    const R m17 = (aE - aF) - (aA + aB);
    const R m18 = (aC + aD) - (aE + aF);
    // relaxation towards the equilibria, scaled by 1/|row|^2
    const R jx = rho * ux, jy = rho * uy, jz = rho * uz;
    const R jx2 = jx * jx, jy2 = jy * jy, jz2 = jz * jz, jsq = jx2 + jy2 + jz2;
    const R d1 = (R)(1.19 / 2394.0) * (m1 - ((R)-11 * rho + (R)19 * jsq));
    const R d2 = (R)(1.4 / 252.0) * (m2 - (R)(-475.0 / 63.0) * jsq);
    const R d4 = (R)(1.2 / 40.0) * (m4 + (R)(2.0 / 3.0) * jx);
    const R d6 = (R)(1.2 / 40.0) * (m6 + (R)(2.0 / 3.0) * jy);
    const R d8 = (R)(1.2 / 40.0) * (m8 + (R)(2.0 / 3.0) * jz);
    const R w36 = omega * (R)(1.0 / 36.0), w12 = omega * (R)(1.0 / 12.0), w4 = omega * (R)0.25;
    const R d9 = w36 * (m9 - ((R)2 * jx2 - (jy2 + jz2)));
    const R d10 = (R)(1.4 / 72.0) * m10;
    const R d11 = w12 * (m11 - (jy2 - jz2));
    const R d12 = (R)(1.4 / 24.0) * m12;
    const R d13 = w4 * (m13 - jx * jy);
    const R d14 = w4 * (m14 - jy * jz);
    const R d15 = w4 * (m15 - jx * jz);
    const R d16 = (R)(1.98 / 8.0) * m16;
    const R d17 = (R)(1.98 / 8.0) * m17;
    const R d18 = (R)(1.98 / 8.0) * m18;
    // even (E) and odd (O) parts of the correction per pair
    const R P = (R)-11 * d1 + (R)-4 * d2;
    const R EX = P + (R)2 * d9 + (R)-4 * d10;
    const R EY = P - d9 + (R)2 * d10 + d11 + (R)-2 * d12;
    const R EZ = P - d9 + (R)2 * d10 - d11 + (R)2 * d12;
    const R G = (R)8 * d1 + d2, H = d9 + d10, K = d11 + d12;
    const R GHp = G + H + K, GHm = G + H - K, G2H = G - (R)2 * H;
    const R OA = (d4 + d6) + (d16 - d17), OB = (d6 - d4) - (d16 + d17);
    const R OC = (d4 + d8) + (d18 - d16), OD = (d8 - d4) + (d16 + d18);
    const R OE = (d6 + d8) + (d17 - d18), OF = (d8 - d6) - (d17 + d18);
    f[0] = f0 - ((R)-30 * d1 + (R)12 * d2);
    f[1] -= EX + (R)-4 * d4;
    f[2] -= EX - (R)-4 * d4;
    f[3] -= EY + (R)-4 * d6;
    f[4] -= EY - (R)-4 * d6;
    f[5] -= EZ + (R)-4 * d8;
    f[6] -= EZ - (R)-4 * d8;
    f[7] -= (GHp + d13) + OA;
    f[10] -= (GHp + d13) - OA;
    f[8] -= (GHp - d13) + OB;
    f[9] -= (GHp - d13) - OB;
    f[11] -= (GHm + d15) + OC;
    f[14] -= (GHm + d15) - OC;
    f[12] -= (GHm - d15) + OD;
    f[13] -= (GHm - d15) - OD;
    f[15] -= (G2H + d14) + OE;
    f[18] -= (G2H + d14) - OE;
    f[16] -= (G2H - d14) + OF;
    f[17] -= (G2H - d14) - OF;
    if (REF) f[18] = 0;
}

}  // namespace lbm
