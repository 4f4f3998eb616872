// Two-node fused step for sm_100-class GPUs (sm_103a here).
//
// Each thread owns the x-adjacent node pair (x, x+1), x even.  Populations of
// the pair travel as one 4-byte half2 (F16S) or 8-byte float2 (F32) per
// direction, and all arithmetic runs on packed FP32x2 (FFMA2/FADD2/FMUL2), so a
// warp instruction advances two lattice nodes.  Pulls with cx = 0 are one
// aligned pair load; pulls with cx = +/-1 take the source row's aligned pair
// and its left or right neighbour pair and pick the shifted elements.
//
// Arithmetic runs in storage space: h = (f - sigma w) * S, w the collision
// model's rest state, with S = scale for F16S and 1 for F32, sigma = 1 when
// the storage holds deviations (F16S, physics-mode F32) and 0 otherwise.
// Every collision operator is linear in f except through the equilibria, so
// it is applied to h directly with equilibria expressed in the same units; a
// load is one half2->float2 convert and a store one float2->half2 convert,
// with no per-population shift and scale, and the moments come from the small
// deviations instead of cancelling sums of O(w) values.  Boundary nodes
// convert to f and reuse the scalar boundary code.
#pragma once
#include "lbm_step.cuh"

namespace lbm {

struct f2 {
    float2 v;
    __device__ __forceinline__ f2() {}
    __device__ __forceinline__ f2(float s) : v(make_float2(s, s)) {}
    __device__ __forceinline__ f2(float a, float b) : v(make_float2(a, b)) {}
    __device__ __forceinline__ f2(float2 x) : v(x) {}
};
__device__ __forceinline__ f2 operator+(f2 a, f2 b) { return f2(__fadd2_rn(a.v, b.v)); }
__device__ __forceinline__ f2 operator*(f2 a, f2 b) { return f2(__fmul2_rn(a.v, b.v)); }
__device__ __forceinline__ f2 fma2(f2 a, f2 b, f2 c) { return f2(__ffma2_rn(a.v, b.v, c.v)); }
__device__ __forceinline__ f2 operator-(f2 a, f2 b) { return f2(__ffma2_rn(b.v, make_float2(-1.f, -1.f), a.v)); }
__device__ __forceinline__ f2 operator-(f2 a) { return f2(__fmul2_rn(a.v, make_float2(-1.f, -1.f))); }
__device__ __forceinline__ f2 &operator+=(f2 &a, f2 b) { return a = a + b; }
__device__ __forceinline__ f2 &operator-=(f2 &a, f2 b) { return a = a - b; }

// One lane: the same collision code on one node per thread (h_node).
struct f1 {
    float v;
    __device__ __forceinline__ f1() {}
    __device__ __forceinline__ f1(float s) : v(s) {}
};
__device__ __forceinline__ f1 operator+(f1 a, f1 b) { return f1(a.v + b.v); }
__device__ __forceinline__ f1 operator*(f1 a, f1 b) { return f1(a.v * b.v); }
__device__ __forceinline__ f1 fma2(f1 a, f1 b, f1 c) { return f1(fmaf(a.v, b.v, c.v)); }
__device__ __forceinline__ f1 operator-(f1 a, f1 b) { return f1(a.v - b.v); }
__device__ __forceinline__ f1 operator-(f1 a) { return f1(-a.v); }
__device__ __forceinline__ f1 &operator+=(f1 &a, f1 b) { return a = a + b; }
__device__ __forceinline__ f1 &operator-=(f1 &a, f1 b) { return a = a - b; }

// One stored value in storage units h and back: F32 as is, F16S as IEEE
// half, F16C as the 1-4-11 float (lbm_device.cuh).
template <int ST>
__device__ __forceinline__ float h_raw(const typename Store<ST>::T *q) {
    if constexpr (ST == LBM_STORE_F16S) return __half2float(__ldg(q));
    else if constexpr (ST == LBM_STORE_F16C) return f16c_to_float(f16c_t{__ldg(&q->bits)});
    else return __ldg(q);
}
template <int ST>
__device__ __forceinline__ void h_put(typename Store<ST>::T *q, float v) {
    if constexpr (ST == LBM_STORE_F16S) *q = __float2half_rn(v);
    else if constexpr (ST == LBM_STORE_F16C) *q = f16c_from_float(v);
    else *q = v;
}

// Pair storage: element type of a pair in HBM and its conversion to h.
template <int ST> struct Pair;
template <> struct Pair<LBM_STORE_F32> {
    using T = float2;
    __device__ static __forceinline__ f2 load(const float *p) { return f2(__ldg((const float2 *)p)); }
    __device__ static __forceinline__ float load1(const float *p) { return __ldg(p); }
    __device__ static __forceinline__ void store(float *p, f2 h) { *(float2 *)p = h.v; }
};
template <> struct Pair<LBM_STORE_F16S> {
    using T = __half2;
    __device__ static __forceinline__ f2 load(const __half *p) { return f2(__half22float2(__ldg((const __half2 *)p))); }
    __device__ static __forceinline__ float load1(const __half *p) { return __half2float(__ldg(p)); }
    __device__ static __forceinline__ void store(__half *p, f2 h) { *(__half2 *)p = __float22half2_rn(h.v); }
};

// Moments of the storage shift that h carries: D2Q9 shift w has
// (rho, e, eps) = (1, -2, 1); the D3Q19 BGK/TRT shift w has rho = 1 and the
// D3Q19 MRT shift w~ has (rho, e, eps) = (1, -11, 0); the other moments
// vanish by isotropy.

// BGK / TRT in h units: h_eq,d = S w_d [(rho - sigma) + rho (3 cu + 4.5 cu^2 - 1.5 u^2)].
template <int Q, class V>
__device__ __forceinline__ V heq(int d, V rho_m_sigma, V rho, V ux, V uy, V uz, V usq15, float S) {
    using L = Lat<Q>;
    V cu = 0.f;
    if (L::cx(d)) cu = L::cx(d) > 0 ? ux : -ux;
    if (L::cy(d)) cu = L::cy(d) > 0 ? cu + uy : cu - uy;
    if (L::cz(d)) cu = L::cz(d) > 0 ? cu + uz : cu - uz;
    // rho (3 cu + 4.5 cu^2 - 1.5 u^2) = rho (cu (3 + 4.5 cu) - usq15)
    const V poly = fma2(cu, fma2(cu, V(4.5f), V(3.f)), -usq15);
    return V((float)(L::w(d)) * S) * fma2(rho, poly, rho_m_sigma);
}

template <int Q, class V>
__device__ __forceinline__ void collide_bgk_x2(V (&h)[Q], V rho, V rms, V ux, V uy, V uz, float omega,
                                               float S) {
    const V usq15 = V(1.5f) * fma2(ux, ux, fma2(uy, uy, uz * uz));
    const V om(omega);
#pragma unroll
    for (int d = 0; d < Q; ++d) h[d] = fma2(-om, h[d] - heq<Q>(d, rms, rho, ux, uy, uz, usq15, S), h[d]);
}

template <int Q, class V>
__device__ __forceinline__ void collide_trt_x2(V (&h)[Q], V rho, V rms, V ux, V uy, V uz, float omega,
                                               float omega_m, float S) {
    using L = Lat<Q>;
    const V usq15 = V(1.5f) * fma2(ux, ux, fma2(uy, uy, uz * uz));
    V e[Q];
#pragma unroll
    for (int d = 0; d < Q; ++d) e[d] = heq<Q>(d, rms, rho, ux, uy, uz, usq15, S);
    V out[Q];
    const V hp(0.5f * omega), hm(0.5f * omega_m);
#pragma unroll
    for (int d = 0; d < Q; ++d) {
        const int o = L::opp(d);
        const V nd = h[d] - e[d], no = h[o] - e[o];
        out[d] = h[d] - fma2(hp, nd + no, hm * (nd - no));
    }
#pragma unroll
    for (int d = 0; d < Q; ++d) h[d] = out[d];
}

// D3Q19 MRT in h units, in the pair-sum form of collide_mrt19 (lbm_device.cuh):
// d_k = s_k/|m_k|^2 (m_k(h) - S (m_eq,k - sigma m_k(w~))), with w~ the
// model's rest state (rest_shift): m(w~) = (1, -11, 0, 0, ...).
template <bool REF, class V>
__device__ __forceinline__ void collide_mrt19_x2(V (&h)[19], V rho, V rms, V ux, V uy, V uz, float omega,
                                                 float sigma, float S) {
    const V sX = h[1] + h[2], aX = h[1] - h[2];
    const V sY = h[3] + h[4], aY = h[3] - h[4];
    const V sZ = h[5] + h[6], aZ = h[5] - h[6];
    const V sA = h[7] + h[10], aA = h[7] - h[10];
    const V sB = h[8] + h[9], aB = h[8] - h[9];
    const V sC = h[11] + h[14], aC = h[11] - h[14];
    const V sD = h[12] + h[13], aD = h[12] - h[13];
    const V sE = h[15] + h[18], aE = h[15] - h[18];
    const V sF = h[16] + h[17], aF = h[16] - h[17];
    const V sAxis = sX + sY + sZ;
    const V sAB = sA + sB, sCD = sC + sD, sEF = sE + sF;
    const V sABCD = sAB + sCD, sDiag = sABCD + sEF;
    const V h0 = h[0];
    const V tx = (aA - aB) + (aC - aD), ty = (aA + aB) + (aE - aF), tz = (aC + aD) + (aE + aF);
    const V m1 = fma2(V(-30.f), h0, fma2(V(-11.f), sAxis, V(8.f) * sDiag));
    const V m2 = fma2(V(12.f), h0, fma2(V(-4.f), sAxis, sDiag));
    const V m4 = fma2(V(-4.f), aX, tx);
    const V m6 = fma2(V(-4.f), aY, ty);
    const V m8 = fma2(V(-4.f), aZ, tz);
    const V sYZ = sY + sZ;
    const V m9 = fma2(V(2.f), sX - sEF, sABCD - sYZ);
    const V m10 = fma2(V(2.f), sYZ - sEF, fma2(V(-4.f), sX, sABCD));
    const V m11 = (sY - sZ) + (sAB - sCD);
    const V m12 = fma2(V(2.f), sZ - sY, sAB - sCD);
    const V m13 = sA - sB, m14 = sE - sF, m15 = sC - sD;
    const V m16 = (aA - aB) - (aC - aD);
    const V m17 = (aE - aF) - (aA + aB);
    const V m18 = (aC + aD) - (aE + aF);
    const V jx = rho * ux, jy = rho * uy, jz = rho * uz;
    const V jx2 = jx * jx, jy2 = jy * jy, jz2 = jz * jz;
    const V jsq = jx2 + jy2 + jz2;
    const V Sv(S);
    // S (m_eq,k - sigma m_k(w)) for the non-conserved moments
    const V E1 = Sv * fma2(V(-11.f), rms, V(19.f) * jsq);
    // the storage shift is this model's rest state, whose eps moment is 0
    const V E2 = Sv * (V((float)(-475.0 / 63.0)) * jsq);
    const V c23 = V((float)(-2.0 / 3.0) * S);
    const V d1 = V((float)(1.19 / 2394.0)) * (m1 - E1);
    const V d2 = V((float)(1.4 / 252.0)) * (m2 - E2);
    const V d4 = V((float)(1.2 / 40.0)) * (m4 - c23 * jx);
    const V d6 = V((float)(1.2 / 40.0)) * (m6 - c23 * jy);
    const V d8 = V((float)(1.2 / 40.0)) * (m8 - c23 * jz);
    const V d9 = V(omega / 36.f) * (m9 - Sv * (fma2(V(2.f), jx2, -jy2) - jz2));
    const V d10 = V((float)(1.4 / 72.0)) * m10;
    const V d11 = V(omega / 12.f) * (m11 - Sv * (jy2 - jz2));
    const V d12 = V((float)(1.4 / 24.0)) * m12;
    const V w4(0.25f * omega);
    const V d13 = w4 * (m13 - Sv * (jx * jy));
    const V d14 = w4 * (m14 - Sv * (jy * jz));
    const V d15 = w4 * (m15 - Sv * (jx * jz));
    const V g16(1.98f / 8.f);
    const V d16 = g16 * m16, d17 = g16 * m17, d18 = g16 * m18;
    const V P = fma2(V(-11.f), d1, V(-4.f) * d2);
    const V EX = fma2(V(2.f), d9, fma2(V(-4.f), d10, P));
    const V EYZb = fma2(V(2.f), d10, P - d9);
    const V K2 = fma2(V(-2.f), d12, d11);
    const V EY = EYZb + K2, EZ = EYZb - K2;
    const V G = fma2(V(8.f), d1, d2), H = d9 + d10, K = d11 + d12;
    const V GH = G + H;
    const V GHp = GH + K, GHm = GH - K, G2H = fma2(V(-2.f), H, G);
    const V OA = (d4 + d6) + (d16 - d17), OB = (d6 - d4) - (d16 + d17);
    const V OC = (d4 + d8) + (d18 - d16), OD = (d8 - d4) + (d16 + d18);
    const V OE = (d6 + d8) + (d17 - d18), OF = (d8 - d6) - (d17 + d18);
    const V m4d4 = V(-4.f) * d4, m4d6 = V(-4.f) * d6, m4d8 = V(-4.f) * d8;
    h[0] = h0 - fma2(V(-30.f), d1, V(12.f) * d2);
    h[1] -= EX + m4d4;
    h[2] -= EX - m4d4;
    h[3] -= EY + m4d6;
    h[4] -= EY - m4d6;
    h[5] -= EZ + m4d8;
    h[6] -= EZ - m4d8;
    const V eA = GHp + d13, eB = GHp - d13, eC = GHm + d15, eD = GHm - d15, eE = G2H + d14, eF = G2H - d14;
    h[7] -= eA + OA;
    h[10] -= eA - OA;
    h[8] -= eB + OB;
    h[9] -= eB - OB;
    h[11] -= eC + OC;
    h[14] -= eC - OC;
    h[12] -= eD + OD;
    h[13] -= eD - OD;
    h[15] -= eE + OE;
    h[18] -= eE - OE;
    h[16] -= eF + OF;
    h[17] -= eF - OF;
    if (REF) h[18] = V((float)(-sigma * rest_shift(19, LBM_MRT, 18)) * S);  // f18 = 0
}

// D2Q9 MRT in h units (CellFunctions.cu:7-63 basis and rates); REF keeps the
// reference's energy equilibria with the extra density factor.
template <bool REF, class V>
__device__ __forceinline__ void collide_mrt9_x2(V (&h)[9], V rho, V rms, V ux, V uy, float omega, float sigma,
                                                float S) {
    const V usq = fma2(ux, ux, uy * uy);
    const V ef = REF ? rho : V(1.f);
    const V Sv(S);
    const V rs = rho * usq * ef;
    V E[9];
    E[0] = 0.f;
    E[1] = Sv * fma2(V(3.f), rs, V(-2.f) * rms);
    E[2] = Sv * fma2(V(-3.f), rs, rms);
    E[3] = Sv * (rho * ux);
    E[4] = -E[3];
    E[5] = Sv * (rho * uy);
    E[6] = -E[5];
    E[7] = Sv * (rho * (ux * ux - uy * uy));
    E[8] = Sv * (rho * (ux * uy));
    // The moment transform of the D2Q9 matrix (mrt2) in pair form: with
    // opposite pairs (1,3), (2,4), (5,7), (6,8), the even moments (e, eps,
    // pxx, pxy) take the pair sums and the odd ones (qx, qy) the pair
    // differences; the back-transform adds a part S shared by a pair and a
    // part O with opposite signs.  Same operator as the 9 x 9 form, about
    // 40 % fewer instructions.
    const V A = h[1] + h[3], B = h[2] + h[4], C = h[5] + h[7], D = h[6] + h[8];
    const V a = h[1] - h[3], b = h[2] - h[4], c = h[5] - h[7], d = h[6] - h[8];
    const V AB = A + B, CD = C + D;
    const V m1 = fma2(V(2.f), CD, fma2(V(-4.f), h[0], -AB));   // e
    const V m2 = fma2(V(-2.f), AB, fma2(V(4.f), h[0], CD));    // eps
    const V m4 = fma2(V(-2.f), a, c - d);                      // qx
    const V m6 = fma2(V(-2.f), b, c + d);                      // qy
    const V m7 = A - B;                                        // pxx
    const V m8 = C - D;                                        // pxy
    const V dm1 = V(1.4f / 36.f) * (m1 - E[1]), dm2 = V(1.4f / 36.f) * (m2 - E[2]);
    const V dm4 = V(1.2f / 12.f) * (m4 - E[4]), dm6 = V(1.2f / 12.f) * (m6 - E[6]);
    const V dm7 = V(omega / 4.f) * (m7 - E[7]), dm8 = V(omega / 4.f) * (m8 - E[8]);
    const V t1 = fma2(V(-2.f), dm2, -dm1), t2 = fma2(V(2.f), dm1, dm2);
    const V S13 = t1 + dm7, S24 = t1 - dm7, S57 = t2 + dm8, S68 = t2 - dm8;
    const V O13 = V(-2.f) * dm4, O24 = V(-2.f) * dm6, O57 = dm4 + dm6, O68 = dm6 - dm4;
    h[0] -= V(4.f) * (dm2 - dm1);
    h[1] -= S13 + O13;
    h[3] -= S13 - O13;
    h[2] -= S24 + O24;
    h[4] -= S24 - O24;
    h[5] -= S57 + O57;
    h[7] -= S57 - O57;
    h[6] -= S68 + O68;
    h[8] -= S68 - O68;
}

// rms = rho - sigma, the density's deviation from the shift's density,
// formed as sum(h)/S by the caller: no FP32 cancellation of rho - 1.
template <int Q, int COLL, bool PHYS, class V>
__device__ __forceinline__ void collide_x2(V (&h)[Q], V rho, V rms, V ux, V uy, V uz, const StepParams &p,
                                           float sigma, float S) {
    if (COLL == LBM_BGKW) {
        collide_bgk_x2<Q>(h, rho, rms, ux, uy, uz, (float)p.omega, S);
    } else if (COLL == LBM_TRT) {
        collide_trt_x2<Q>(h, rho, rms, ux, uy, uz, (float)p.omega, (float)p.omega_m, S);
    } else {
        if constexpr (Q == 9)
            collide_mrt9_x2<!PHYS>(h, rho, rms, ux, uy, (float)p.omega, sigma, S);
        else
            collide_mrt19_x2<!PHYS>(h, rho, rms, ux, uy, uz, (float)p.omega, sigma, S);
    }
}

constexpr int X2_BLOCK = 128;

// One node pair (x0, x0 + 1) of the fused step; G and WRAP as in step_node.
template <int Q, int COLL, int ST, bool PHYS, bool WRAP, class G>
__device__ __forceinline__ void pair_node(const StepParams &p, const G &g, int x0, int y, int z) {
    using L = Lat<Q>;
    using T = typename Store<ST>::T;
    using PS = Pair<ST>;
    constexpr bool F16 = ST == LBM_STORE_F16S;
    const float sigma = p.sigma;
    const float S = F16 ? p.scale : 1.f;
    const float invS = F16 ? p.inv_scale : 1.f;

    const bool in_row = x0 < g.nx;
    const int row = y + g.ny * z;
    const int node = x0 + g.nx * row;   // flag words and macroscopic fields
    const long long idx = x0 + (long long)g.pitch * row;  // populations
    const T *in = (const T *)p.fin[0] + idx;
    T *out = (T *)p.fout[0] + idx;
    uint2 wp = make_uint2(0u, 0u);
    if (in_row) wp = __ldg((const uint2 *)(p.word + node));
    const bool fl0 = (wp.x & W_FLUID) != 0, fl1 = (wp.y & W_FLUID) != 0;
    const unsigned warp_fluid = __ballot_sync(0xffffffffu, fl0 || fl1);
    if (!fl0 && !fl1) {
        if (in_row && warp_fluid) {
#pragma unroll
            for (int d = 0; d < Q; ++d)
                PS::store(out + d * g.nx, f2(-p.shift[d] * S));
        }
        return;
    }

    const int plane = g.pitch * g.ny;
    int oym = -g.pitch, oyp = g.pitch, ozm = -plane, ozp = plane;
    // x offsets of the pair's pulls: node x0 from x0 - 1, node x0 + 1 from x0 + 2
    int oxm0 = -1, oxp1 = 1;
    if (WRAP) {
        oym = y == 0 ? (g.ny - 1) * g.pitch : -g.pitch;
        oyp = y == g.ny - 1 ? (1 - g.ny) * g.pitch : g.pitch;
        ozm = z == 0 ? (g.nz - 1) * plane : -plane;
        ozp = z == g.nz - 1 ? (1 - g.nz) * plane : plane;
        oxm0 = x0 == 0 ? g.nx - 1 : -1;
        oxp1 = x0 + 2 >= g.nx ? 1 - g.nx : 1;
    }

    // All loads first, none of their values used before the last is issued:
    // each element's address already selects the pull source or, across a
    // blocked link, the node's own population (direction d in reference
    // mode, opp(d) for half-way bounce-back), so there is no branch between
    // loads and the memory system sees every request of the thread at once.
    float hx[Q], hy[Q];
#pragma unroll
    for (int d = 0; d < Q; ++d) {
        const int oyz = (L::cy(d) == 1 ? oym : (L::cy(d) == -1 ? oyp : 0)) +
                        (L::cz(d) == 1 ? ozm : (L::cz(d) == -1 ? ozp : 0));
        const int s0 = d * g.nx + oyz + (L::cx(d) == 1 ? oxm0 : (L::cx(d) == -1 ? 1 : 0));
        const int s1 = d * g.nx + 1 + oyz + (L::cx(d) == 1 ? -1 : (L::cx(d) == -1 ? oxp1 : 0));
        if (d == 0) {
            hx[0] = PS::load1(in);
            hy[0] = PS::load1(in + 1);
            continue;
        }
        const int own = (PHYS ? L::opp(d) : d) * g.nx;
        const bool b0 = (wp.x >> d) & 1u, b1 = (wp.y >> d) & 1u;
        hx[d] = PS::load1(in + (b0 ? own : s0));
        hy[d] = PS::load1(in + (b1 ? own + 1 : s1));
    }
    const unsigned warp_blocked = __reduce_or_sync(0xffffffffu, (wp.x | wp.y) & 0x7FFFEu);
    f2 h[Q];
#pragma unroll
    for (int d = 0; d < Q; ++d) h[d] = f2(hx[d], hy[d]);

    bool keep0 = false, keep1 = false, zv0 = false, zv1 = false;
    if (((wp.x | wp.y) & W_SPECIAL) != 0) {
        // boundary nodes: to f, scalar boundary code, back to h
#pragma unroll
        for (int e = 0; e < 2; ++e) {
            const uint32_t we = e ? wp.y : wp.x;
            if (!(we & W_SPECIAL) || !(we & W_FLUID)) continue;
            float f[Q];
#pragma unroll
            for (int d = 0; d < Q; ++d)
                f[d] = fmaf(e ? h[d].v.y : h[d].v.x, invS, p.shift[d]);
            const int nd = node + e;
            const int sl = __ldg(p.slot + nd);
            const float u0 = (float)__ldg(p.bc_uvw + 3 * sl), v0 = (float)__ldg(p.bc_uvw + 3 * sl + 1),
                        w0 = (float)__ldg(p.bc_uvw + 3 * sl + 2);
            bool keep = false, zv = false;
            if constexpr (!PHYS) {
                const unsigned long long mk = __ldg(p.bc_mask + sl);
                if constexpr (Q == 9) {
                    bc_ref_d2q9<float>(f, (uint32_t)mk, u0, p.outlet_profile, zv);
                } else {
                    bc_ref3_inlet_wall<float>(f, mk, u0, v0, w0, p.ref_hh != 0);
                    ref3_periodic<ST, WRAP, G>(f, mk, nd, p, g);
                    bc_ref3_symm<float>(f, mk);
                    keep = ref3_keep_macro(mk, p.update_inlet_outlet);
                }
            } else {
                const int kind = __ldg(p.bc_kind + sl);
                if (kind & BCK_MOVING) {
                    bc_moving_wall<Q, float>(f, __ldg(p.bc_mask + sl), (float)p.rho0, u0, v0, w0);
                } else if (kind & BCK_ACTIVE) {
                    const float rset = (kind & BCK_OUTLET) ? (float)p.rho_out : (float)p.rho_in;
                    bc_phys<Q, float>(f, kind & BCK_FACE_MASK, (kind & BCK_PRESSURE) != 0, rset, u0, v0, w0);
                }
            }
#pragma unroll
            for (int d = 0; d < Q; ++d) {
                const float hv = (f[d] - p.shift[d]) * S;
                if (e) h[d].v.y = hv; else h[d].v.x = hv;
            }
            if (e) { keep1 = keep; zv1 = zv; } else { keep0 = keep; zv0 = zv; }
        }
        if constexpr (!PHYS) {
            // reference straight walls of the plain wall node of the pair
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                const uint32_t we = e ? wp.y : wp.x;
                if ((we & W_SPECIAL) || !(we & W_FLUID)) continue;
#pragma unroll
                for (int dir = 1; dir < Q; ++dir)
                    if ((we >> L::opp(dir)) & 1u) {
                        if (e) h[L::opp(dir)].v.y = h[dir].v.y; else h[L::opp(dir)].v.x = h[dir].v.x;
                    }
            }
        }
    } else if constexpr (!PHYS) {
        if (warp_blocked) {
#pragma unroll
            for (int dir = 1; dir < Q; ++dir) {
                const int o = L::opp(dir);
                const bool b0 = (wp.x >> o) & 1u, b1 = (wp.y >> o) & 1u;
                h[o] = f2(b0 ? h[dir].v.x : h[o].v.x, b1 ? h[dir].v.y : h[o].v.y);
            }
        }
    }

    // macroscopic moments: rho = sigma + sum(h)/S, j = sum(c h)/S
    f2 sum = h[0], jx = 0.f, jy = 0.f, jz = 0.f;
#pragma unroll
    for (int d = 1; d < Q; ++d) {
        sum += h[d];
        if (L::cx(d) == 1) jx += h[d]; else if (L::cx(d) == -1) jx -= h[d];
        if (L::cy(d) == 1) jy += h[d]; else if (L::cy(d) == -1) jy -= h[d];
        if (L::cz(d) == 1) jz += h[d]; else if (L::cz(d) == -1) jz -= h[d];
    }
    f2 rms = sum * f2(invS);
    f2 rho = rms + f2(sigma);
    const f2 irho(1.f / rho.v.x, 1.f / rho.v.y);
    const f2 sc = irho * f2(invS);
    f2 ux = fma2(jx, sc, f2((float)p.gshift)), uy = jy * sc, uz = jz * sc;
    if (zv0) uy.v.x = 0.f;
    if (zv1) uy.v.y = 0.f;
    if (keep0 || keep1) {
        if (keep0) {
            rho.v.x = p.rho[node]; ux.v.x = p.ux[node]; uy.v.x = p.uy[node]; uz.v.x = p.uz[node];
            rms.v.x = rho.v.x - sigma;
        }
        if (keep1) {
            rho.v.y = p.rho[node + 1]; ux.v.y = p.ux[node + 1]; uy.v.y = p.uy[node + 1]; uz.v.y = p.uz[node + 1];
            rms.v.y = rho.v.y - sigma;
        }
    }
    if (p.write_macro) {
        if (!keep0 && fl0) { p.rho[node] = rho.v.x; p.ux[node] = ux.v.x; p.uy[node] = uy.v.x; p.uz[node] = uz.v.x; }
        if (!keep1 && fl1) {
            p.rho[node + 1] = rho.v.y; p.ux[node + 1] = ux.v.y; p.uy[node + 1] = uy.v.y; p.uz[node + 1] = uz.v.y;
        }
    }

    collide_x2<Q, COLL, PHYS>(h, rho, rms, ux, uy, uz, p, sigma, S);

    // a solid node of a mixed pair keeps the zero encoding
    if (!fl0 || !fl1) {
#pragma unroll
        for (int d = 0; d < Q; ++d) {
            const float z0 = -p.shift[d] * S;
            if (!fl0) h[d].v.x = z0;
            if (!fl1) h[d].v.y = z0;
        }
    }
#pragma unroll
    for (int d = 0; d < Q; ++d) PS::store(out + d * g.nx, h[d]);
}

// One node per thread with pair_node's arithmetic (storage units h, lanes of
// type f1): no decode or encode per population and moments from deviations.
// The update of one fluid node in storage units: gather (pull or bounce
// back), boundary conditions, moments, collision; h receives the new state.
// The node's populations after streaming, in storage units: direction d
// pulls from the upstream neighbour, or, across a link the flag word marks
// blocked (bit d), takes the node's own population (its opposite in physics
// mode: half-way bounce-back).
template <int Q, int ST, bool PHYS, class G, int HB = 0>
__device__ __forceinline__ void h_gather(const G &g, uint32_t w, const typename Store<ST>::T *in, f1 (&h)[Q], int oxm,
                                         int oxp, int oym, int oyp, int ozm, int ozp) {
    using L = Lat<Q>;
    using T = typename Store<ST>::T;
    auto raw = [](const T *q) -> float { return h_raw<ST>(q); };
    h[0] = raw(in);
#pragma unroll
    for (int d = 1; d < Q; ++d) {
        const int pull = d * g.nx + (L::cx(d) == 1 ? oxm : (L::cx(d) == -1 ? oxp : 0)) +
                         (L::cy(d) == 1 ? oym : (L::cy(d) == -1 ? oyp : 0)) +
                         (L::cz(d) == 1 ? ozm : (L::cz(d) == -1 ? ozp : 0));
        const int own = (PHYS ? L::opp(d) : d) * g.nx;
        if constexpr (HB == 1) {
            // two exclusive loads at fixed offsets instead of an address
            // selected per direction
            float v;
            if ((w >> d) & 1u) v = raw(in + own);
            else v = raw(in + pull);
            h[d] = v;
        } else {
            h[d] = raw(in + (((w >> d) & 1u) ? own : pull));
        }
    }
}

// Boundary closures, moments, the macroscopic store and the collision of a
// fluid node whose streamed populations are in h (storage units).
template <int Q, int COLL, int ST, bool PHYS, bool WRAP, class G>
__device__ __forceinline__ void h_finish(const StepParams &p, const G &g, int node, uint32_t w, f1 (&h)[Q]) {
    using L = Lat<Q>;
    using T = typename Store<ST>::T;
    constexpr bool F16 = ST == LBM_STORE_F16S || ST == LBM_STORE_F16C;
    const float sigma = p.sigma;
    const float S = F16 ? p.scale : 1.f;
    const float invS = F16 ? p.inv_scale : 1.f;
    bool keep = false, zv = false;
    if constexpr (PHYS) {
        // physics-mode faces and moving walls stay in storage units: the
        // deviations keep their digits (an f-space detour rounds every
        // population to FP32 near w_d, 1e-4 of a slow flow's velocity)
        if (w & W_SPECIAL) {
            const int sl = __ldg(p.slot + node);
            const int kind = __ldg(p.bc_kind + sl);
            if (kind & (BCK_MOVING | BCK_ACTIVE)) {
                const float u0 = (float)__ldg(p.bc_uvw + 3 * sl), v0 = (float)__ldg(p.bc_uvw + 3 * sl + 1),
                            w0 = (float)__ldg(p.bc_uvw + 3 * sl + 2);
                float hv[Q];
#pragma unroll
                for (int d = 0; d < Q; ++d) hv[d] = h[d].v;
                if (kind & BCK_MOVING) {
                    bc_moving_wall_h<Q>(hv, __ldg(p.bc_mask + sl), (float)p.rho0, S, u0, v0, w0);
                } else if (kind & (BCK_EXTRAP1 | BCK_EXTRAP2 | BCK_HE)) {
                    phys_open_outlet<Q, ST, WRAP, G, float>(
                        hv, kind, sl, node, p, g, [](const T *q, int) { return h_raw<ST>(q); },
                        [&](int d, float r, float ux, float uy, float uz) {
                            const float usq15 = 1.5f * (ux * ux + uy * uy + uz * uz);
                            return (feq<Q, float>(d, r, ux, uy, uz, usq15) - sigma * p.shift[d]) * S;
                        });
                } else {
                    const double rset = (kind & BCK_OUTLET) ? p.rho_out : p.rho_in;
                    bc_phys_h<Q>(hv, kind & BCK_FACE_MASK, (kind & BCK_PRESSURE) != 0, (float)(rset - (double)sigma),
                                 sigma, S, invS, u0, v0, w0);
                }
#pragma unroll
                for (int d = 0; d < Q; ++d) h[d] = f1(hv[d]);
            }
        }
    } else {
        if ((w & W_SPECIAL) || (w & 0x7FFFEu)) {
            // boundary nodes and reference wall copies: to f, scalar code, back
            float f[Q];
#pragma unroll
            for (int d = 0; d < Q; ++d) f[d] = fmaf(h[d].v, invS, sigma * p.shift[d]);
            apply_bc<Q, ST, PHYS, WRAP, G>(f, w, node, p, g, keep, zv);
#pragma unroll
            for (int d = 0; d < Q; ++d) h[d] = f1((f[d] - sigma * p.shift[d]) * S);
        }
    }
    f1 sum = h[0], jx = 0.f, jy = 0.f, jz = 0.f;
#pragma unroll
    for (int d = 1; d < Q; ++d) {
        sum += h[d];
        if (L::cx(d) == 1) jx += h[d]; else if (L::cx(d) == -1) jx -= h[d];
        if (L::cy(d) == 1) jy += h[d]; else if (L::cy(d) == -1) jy -= h[d];
        if (L::cz(d) == 1) jz += h[d]; else if (L::cz(d) == -1) jz -= h[d];
    }
    f1 rms = sum * f1(invS);
    f1 rho = rms + f1(sigma);
    const f1 sc = f1(invS / rho.v);
    f1 ux = fma2(jx, sc, f1((float)p.gshift)), uy = jy * sc, uz = jz * sc;
    if (zv) uy = 0.f;
    if (PHYS && (w & W_SPECIAL) && p.bc_macro) {
        const int sl = __ldg(p.slot + node);
        if (__ldg(p.bc_kind + sl) & BCK_HE) {
            double *st = p.bc_macro + 4 * sl;
            st[0] = rho.v;
            st[1] = ux.v;
            st[2] = uy.v;
            st[3] = uz.v;
        }
    }
    if (keep) {
        rho = p.rho[node];
        rms = rho - f1(sigma);
        ux = p.ux[node];
        uy = p.uy[node];
        uz = p.uz[node];
    } else if (p.write_macro) {
        p.rho[node] = rho.v;
        p.ux[node] = ux.v;
        p.uy[node] = uy.v;
        p.uz[node] = uz.v;
    }
    collide_x2<Q, COLL, PHYS>(h, rho, rms, ux, uy, uz, p, sigma, S);
}

template <int Q, int COLL, int ST, bool PHYS, bool WRAP, class G, bool SPEC, int HB = 0>
__device__ __forceinline__ void h_update(const StepParams &p, const G &g, int x, int node, uint32_t w,
                                         const typename Store<ST>::T *in, f1 (&h)[Q],
                                         const float (&spec_pull)[SPEC ? Q : 1], const float (&spec_own)[SPEC ? Q : 1],
                                         int oxm, int oxp, int oym, int oyp, int ozm,
                                         int ozp) {
    if constexpr (SPEC) {
        h[0] = spec_pull[0];
#pragma unroll
        for (int d = 1; d < Q; ++d) h[d] = ((w >> d) & 1u) ? spec_own[d] : spec_pull[d];
    } else {
        h_gather<Q, ST, PHYS, G, HB>(g, w, in, h, oxm, oxp, oym, oyp, ozm, ozp);
    }
    h_finish<Q, COLL, ST, PHYS, WRAP, G>(p, g, node, w, h);
}

// SPEC: the pull values (guarded by the node's coordinates, not its flag
// word) and the node's own bounce-back values are loaded together with the
// flag word and selected once it arrives: one memory round trip per node
// instead of two (flag word, then the addresses it selects).
// MERGE: solid lanes of a warp with fluid nodes store their zero encoding in
// the fluid lanes' store instructions (one store per direction and warp);
// without it they store in a branch of their own, which keeps fewer
// registers live (the batch kernel, whose domains are mostly all fluid).
template <int Q, int COLL, int ST, bool PHYS, bool WRAP, class G, bool SPEC = false, bool MERGE = true, int HB = 0>
__device__ __forceinline__ void h_node_w(const StepParams &p, const G &g, int x, int y, int z, uint32_t w) {
    using L = Lat<Q>;
    using T = typename Store<ST>::T;
    constexpr bool F16 = ST == LBM_STORE_F16S || ST == LBM_STORE_F16C;
    const float sigma = p.sigma;
    const float S = F16 ? p.scale : 1.f;
    const float invS = F16 ? p.inv_scale : 1.f;
    const bool in_row = x < g.nx;
    const int row = y + g.ny * z;
    const int node = x + g.nx * row;
    const long long idx = x + (long long)g.pitch * row;
    const T *in = (const T *)p.fin[0] + idx;
    T *out = (T *)p.fout[0] + idx;
    auto raw = [](const T *q) -> float { return h_raw<ST>(q); };
    const int plane = g.pitch * g.ny;
    int oxm = -1, oxp = 1, oym = -g.pitch, oyp = g.pitch, ozm = -plane, ozp = plane;
    if (WRAP) {
        oxm = x == 0 ? g.nx - 1 : -1;
        oxp = x == g.nx - 1 ? 1 - g.nx : 1;
        oym = y == 0 ? (g.ny - 1) * g.pitch : -g.pitch;
        oyp = y == g.ny - 1 ? (1 - g.ny) * g.pitch : g.pitch;
        ozm = z == 0 ? (g.nz - 1) * plane : -plane;
        ozp = z == g.nz - 1 ? (1 - g.nz) * plane : plane;
    }
    float spec_pull[SPEC ? Q : 1], spec_own[SPEC ? Q : 1];
    if constexpr (SPEC) {
        // every address below lies inside the lattice: pulls only where the
        // source coordinate does (with WRAP every offset wraps into it)
        const bool xl = WRAP || x > 0, xh = WRAP || x < g.nx - 1, yl = WRAP || y > 0, yh = WRAP || y < g.ny - 1,
                   zl = WRAP || z > 0, zh = WRAP || z < g.nz - 1;
#pragma unroll
        for (int d = 1; d < Q; ++d) {
            const bool inside = in_row && (L::cx(d) == 1 ? xl : (L::cx(d) == -1 ? xh : true)) &&
                                (L::cy(d) == 1 ? yl : (L::cy(d) == -1 ? yh : true)) &&
                                (L::cz(d) == 1 ? zl : (L::cz(d) == -1 ? zh : true));
            const int pull = d * g.nx + (L::cx(d) == 1 ? oxm : (L::cx(d) == -1 ? oxp : 0)) +
                             (L::cy(d) == 1 ? oym : (L::cy(d) == -1 ? oyp : 0)) +
                             (L::cz(d) == 1 ? ozm : (L::cz(d) == -1 ? ozp : 0));
            spec_pull[d] = inside ? raw(in + pull) : 0.f;
            spec_own[d] = in_row ? raw(in + (PHYS ? L::opp(d) : d) * g.nx) : 0.f;
        }
        spec_pull[0] = in_row ? raw(in) : 0.f;
    }
    const bool fluid = (w & W_FLUID) != 0;
    auto put = [](T *q, float v) { h_put<ST>(q, v); };
    const unsigned warp_fluid = __ballot_sync(0xffffffffu, fluid);
    if (!warp_fluid) return;  // a warp of solid nodes writes nothing
    f1 h[Q];
    if constexpr (!MERGE) {
        if (!fluid) {
            if (in_row) {
#pragma unroll
                for (int d = 0; d < Q; ++d) put(out + d * g.nx, -sigma * p.shift[d] * S);
            }
            return;
        }
        h_update<Q, COLL, ST, PHYS, WRAP, G, SPEC, HB>(p, g, x, node, w, in, h, spec_pull, spec_own, oxm, oxp, oym, oyp,
                                                   ozm, ozp);
#pragma unroll
        for (int d = 0; d < Q; ++d) put(out + d * g.nx, h[d].v);
        return;
    }
    if (fluid) {
        h_update<Q, COLL, ST, PHYS, WRAP, G, SPEC, HB>(p, g, x, node, w, in, h, spec_pull, spec_own, oxm, oxp, oym, oyp,
                                                   ozm, ozp);
    } else {
        // solid lanes of a warp with fluid nodes store the zero encoding in
        // the same store instructions, so every store covers whole sectors
#pragma unroll
        for (int d = 0; d < Q; ++d) h[d] = f1(-sigma * p.shift[d] * S);
    }
    if (in_row) {
#pragma unroll
        for (int d = 0; d < Q; ++d) put(out + d * g.nx, h[d].v);
    }
}



// Two nodes of one column, (x, y, z) and (x, y, z + 1), updated together:
// each gathers by its own flag word (pull, or its own opposite population
// across a blocked link), then moments and collision run on packed FP32x2
// lanes (collide_x2 with f2), so one FFMA2 serves both nodes.  Neither node
// may be a boundary-slot node (the caller takes the one-node path for a warp
// that holds one).  A solid node loads nothing and stores its zero encoding,
// as in h_node_w.
template <int Q, int COLL, int ST, bool PHYS, bool WRAP, class G, int HB>
__device__ __forceinline__ void h_zpair_w(const StepParams &p, const G &g, int x, int y, int z, uint32_t w0,
                                          uint32_t w1) {
    using L = Lat<Q>;
    using T = typename Store<ST>::T;
    constexpr bool F16 = ST == LBM_STORE_F16S || ST == LBM_STORE_F16C;
    const float sigma = p.sigma;
    const float S = F16 ? p.scale : 1.f;
    const float invS = F16 ? p.inv_scale : 1.f;
    const bool in_row = x < g.nx;
    const int row0 = y + g.ny * z;
    const int node0 = x + g.nx * row0, node1 = node0 + g.nx * g.ny;
    const int plane = g.pitch * g.ny;
    const long long idx = x + (long long)g.pitch * row0;
    const T *in0 = (const T *)p.fin[0] + idx;
    const T *in1 = in0 + plane;
    T *out0 = (T *)p.fout[0] + idx;
    T *out1 = out0 + plane;
    const bool fl0 = (w0 & W_FLUID) != 0, fl1 = (w1 & W_FLUID) != 0;
    if (!__ballot_sync(0xffffffffu, fl0 || fl1)) return;  // a warp of solid nodes writes nothing
    int oxm = -1, oxp = 1, oym = -g.pitch, oyp = g.pitch;
    int ozm0 = -plane, ozp0 = plane, ozm1 = -plane, ozp1 = plane;
    if (WRAP) {
        oxm = x == 0 ? g.nx - 1 : -1;
        oxp = x == g.nx - 1 ? 1 - g.nx : 1;
        oym = y == 0 ? (g.ny - 1) * g.pitch : -g.pitch;
        oyp = y == g.ny - 1 ? (1 - g.ny) * g.pitch : g.pitch;
        // node 0 (at z < nz - 1) and node 1 (at z + 1 > 0) wrap on one side only
        ozm0 = z == 0 ? (g.nz - 1) * plane : -plane;
        ozp1 = z + 1 == g.nz - 1 ? (1 - g.nz) * plane : plane;
    }
    auto raw = [](const T *q) -> float { return h_raw<ST>(q); };
    f2 h[Q];
    {
        const float a0 = fl0 ? raw(in0) : 0.f, a1 = fl1 ? raw(in1) : 0.f;
        h[0] = f2(a0, a1);
    }
#pragma unroll
    for (int d = 1; d < Q; ++d) {
        const int pxy = d * g.nx + (L::cx(d) == 1 ? oxm : (L::cx(d) == -1 ? oxp : 0)) +
                        (L::cy(d) == 1 ? oym : (L::cy(d) == -1 ? oyp : 0));
        const int pull0 = pxy + (L::cz(d) == 1 ? ozm0 : (L::cz(d) == -1 ? ozp0 : 0));
        const int pull1 = pxy + (L::cz(d) == 1 ? ozm1 : (L::cz(d) == -1 ? ozp1 : 0));
        const int own = (PHYS ? L::opp(d) : d) * g.nx;
        float a0 = 0.f, a1 = 0.f;
        if constexpr (HB == 1) {
            if (fl0) {
                if ((w0 >> d) & 1u) a0 = raw(in0 + own);
                else a0 = raw(in0 + pull0);
            }
            if (fl1) {
                if ((w1 >> d) & 1u) a1 = raw(in1 + own);
                else a1 = raw(in1 + pull1);
            }
        } else {
            if (fl0) a0 = raw(in0 + (((w0 >> d) & 1u) ? own : pull0));
            if (fl1) a1 = raw(in1 + (((w1 >> d) & 1u) ? own : pull1));
        }
        h[d] = f2(a0, a1);
    }
    f2 sum = h[0], jx = 0.f, jy = 0.f, jz = 0.f;
#pragma unroll
    for (int d = 1; d < Q; ++d) {
        sum += h[d];
        if (L::cx(d) == 1) jx += h[d]; else if (L::cx(d) == -1) jx -= h[d];
        if (L::cy(d) == 1) jy += h[d]; else if (L::cy(d) == -1) jy -= h[d];
        if (L::cz(d) == 1) jz += h[d]; else if (L::cz(d) == -1) jz -= h[d];
    }
    const f2 rms = sum * f2(invS);
    const f2 rho = rms + f2(sigma);
    // a solid lane's rho is sigma + 0 = 1 (F16S/F32 shifted) or 0 (unshifted);
    // guard the reciprocal, its results are discarded
    const float r0 = fl0 ? rho.v.x : 1.f, r1 = fl1 ? rho.v.y : 1.f;
    const f2 sc(invS / r0, invS / r1);
    const f2 ux = fma2(jx, sc, f2((float)p.gshift)), uy = jy * sc, uz = jz * sc;
    if (p.write_macro) {
        if (fl0) {
            p.rho[node0] = rho.v.x;
            p.ux[node0] = ux.v.x;
            p.uy[node0] = uy.v.x;
            p.uz[node0] = uz.v.x;
        }
        if (fl1) {
            p.rho[node1] = rho.v.y;
            p.ux[node1] = ux.v.y;
            p.uy[node1] = uy.v.y;
            p.uz[node1] = uz.v.y;
        }
    }
    collide_x2<Q, COLL, PHYS>(h, rho, rms, ux, uy, uz, p, sigma, S);
    if (in_row) {
#pragma unroll
        for (int d = 0; d < Q; ++d) {
            const float zero = -sigma * p.shift[d] * S;
            h_put<ST>(out0 + d * g.nx, fl0 ? h[d].v.x : zero);
            h_put<ST>(out1 + d * g.nx, fl1 ? h[d].v.y : zero);
        }
    }
}

// One node: its flag word, then the update.
template <int Q, int COLL, int ST, bool PHYS, bool WRAP, class G, bool SPEC = false, bool MERGE = true, int HB = 0>
__device__ __forceinline__ void h_node(const StepParams &p, const G &g, int x, int y, int z) {
    const uint32_t w = x < g.nx ? __ldg(p.word + x + g.nx * (y + g.ny * z)) : 0u;
    h_node_w<Q, COLL, ST, PHYS, WRAP, G, SPEC, MERGE, HB>(p, g, x, y, z, w);
}

template <int Q, int COLL, int ST, bool PHYS>
__global__ void __launch_bounds__(STEP_BLOCK) step_kernel_h(const StepParams p) {
    const DynGeom g{p.nx, p.ny, p.nz, p.pitch};
    h_node<Q, COLL, ST, PHYS, true>(p, g, blockIdx.x * blockDim.x + threadIdx.x, blockIdx.y, blockIdx.z);
}

// h_node with the lattice extents fixed at compile time (built at run time).
// ZW > 1: a thread updates ZW nodes in a column along z, loading the next
// node's flag word before it works on the current one, so the populations'
// addresses do not wait a memory round trip for it (blockIdx.z = z / ZW).
// HB = 1: a population across a possibly blocked link comes from one of two
// loads at fixed offsets, predicated on the link's flag bit, instead of one
// load from an address selected per direction.
template <int Q, int COLL, int ST, bool PHYS, bool WRAP, int NX, int NY, int NZ, int BLOCK, int MINB, bool SPEC = false,
          int ZW = 1, int HB = 0, bool ZP = false>
__global__ void __launch_bounds__(BLOCK, MINB) step_kernel_h_fixed(const StepParams p) {
    using G = FixedGeom<NX, NY, NZ, Q * NX>;
    const G g;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if constexpr (ZW == 1) {
        h_node<Q, COLL, ST, PHYS, WRAP, G, SPEC, true, HB>(p, g, x, blockIdx.y, blockIdx.z);
    } else if constexpr (ZP) {
        // ZP: the column's nodes two at a time on packed FP32x2 (h_zpair_w);
        // a warp holding a boundary-slot node takes the one-node path
        const int y = blockIdx.y, z0 = blockIdx.z * ZW;
        const bool in_row = x < NX;
        auto flag = [&](int z) -> uint32_t { return in_row && z < NZ ? __ldg(p.word + x + NX * (y + NY * z)) : 0u; };
        uint32_t wa = flag(z0), wb = flag(z0 + 1);
#pragma unroll 1
        for (int k = 0; k < ZW; k += 2) {
            const int z = z0 + k;
            if (z >= NZ) break;  // the same z for every thread of the block
            const bool two = k + 1 < ZW && z + 1 < NZ;
            const uint32_t wc = k + 2 < ZW ? flag(z + 2) : 0u, wd = k + 3 < ZW ? flag(z + 3) : 0u;
            const bool special = __any_sync(0xffffffffu, ((wa | (two ? wb : 0u)) & W_SPECIAL) != 0);
            if (two && !special) {
                h_zpair_w<Q, COLL, ST, PHYS, WRAP, G, HB>(p, g, x, y, z, wa, wb);
            } else {
                h_node_w<Q, COLL, ST, PHYS, WRAP, G, SPEC, true, HB>(p, g, x, y, z, wa);
                if (two) h_node_w<Q, COLL, ST, PHYS, WRAP, G, SPEC, true, HB>(p, g, x, y, z + 1, wb);
            }
            wa = wc;
            wb = wd;
        }
    } else {
        const int y = blockIdx.y, z0 = blockIdx.z * ZW;
        const bool in_row = x < NX;
        uint32_t w = in_row ? __ldg(p.word + x + NX * (y + NY * z0)) : 0u;
#pragma unroll 1
        for (int k = 0; k < ZW; ++k) {
            const int z = z0 + k;
            if (z >= NZ) break;  // the same z for every thread of the block
            const uint32_t wn =
                in_row && k + 1 < ZW && z + 1 < NZ ? __ldg(p.word + x + NX * (y + NY * (z + 1))) : 0u;
            h_node_w<Q, COLL, ST, PHYS, WRAP, G, SPEC, true, HB>(p, g, x, y, z, w);
            w = wn;
        }
    }
}

template <int Q, int COLL, int ST, bool PHYS>
__global__ void __launch_bounds__(X2_BLOCK) step_kernel_x2(const StepParams p) {
    const DynGeom g{p.nx, p.ny, p.nz, p.pitch};
    pair_node<Q, COLL, ST, PHYS, true>(p, g, 2 * (blockIdx.x * blockDim.x + threadIdx.x), blockIdx.y, blockIdx.z);
}

// The pair step with the lattice extents fixed at compile time (built at run
// time, lbm_jit.cpp); BLOCK threads (pairs) along x.
template <int Q, int COLL, int ST, bool PHYS, bool WRAP, int NX, int NY, int NZ, int BLOCK, int MINB>
__global__ void __launch_bounds__(BLOCK, MINB) step_kernel_x2_fixed(const StepParams p) {
    const FixedGeom<NX, NY, NZ, Q * NX> g;
    pair_node<Q, COLL, ST, PHYS, WRAP>(p, g, 2 * (blockIdx.x * blockDim.x + threadIdx.x), blockIdx.y, blockIdx.z);
}

}  // namespace lbm
