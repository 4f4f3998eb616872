// Node-local boundary conditions applied in registers between pull-streaming
// and the macroscopic update.  Only "special" nodes (inlets, outlets,
// symmetry planes, mixed-type reference masks) reach these functions; plain
// wall nodes are handled inline by the step kernel from their blocked-link
// bits.
#pragma once
#include "lbm_device.cuh"

namespace lbm {

// Reference 2D BC mask bits (include/BcMacros.h:14-74).
__device__ __forceinline__ uint32_t m2(uint32_t type, int dir) { return type << ((dir - 1) * 2); }
constexpr uint32_t R2_INLT_B = 0x20000u, R2_CORNER = 0x40000u, R2_FLUID = 0x80000u;
// Reference 3D BC mask bits (include/BcMacros3D.h:16-170), 64-bit.
__device__ __forceinline__ uint64_t m3(uint64_t type, int dir) { return type << ((dir - 1) * 3); }
constexpr uint64_t R3_INLT_B = 2ull << 54, R3_OUTL_B = 3ull << 54, R3_SYMP_B = 5ull << 54,
                   R3_CORNER = 1ull << 57, R3_FLUID = 1ull << 58;

// ---------------------------------------------------------------------------
// Reference semantics, D2Q9: gpuBcInlet2D, gpuBcWall2D (straight), and the
// Zou-He branch of gpuBcOutlet2D (GpuBoundaries.cu:12-71, :400-443,
// :1562-1602), in that order, on the node's streamed populations.
// ---------------------------------------------------------------------------
template <class R>
__device__ __forceinline__ void bc_ref_d2q9(R (&f)[9], uint32_t mk, R u0, int outlet_profile,
                                            bool &zero_v) {
    if (!(mk & R2_FLUID)) return;
    if (mk & R2_INLT_B) {
        if ((mk & m2(2, 2)) && !(mk & R2_CORNER)) {  // north (lid)
            f[4] = f[2];
            const R t = (f[0] + f[1] + f[3] + (R)2 * (f[2] + f[6] + f[5])) * u0 / (R)6;
            f[8] = f[6] + t;
            f[7] = f[5] - t;
        }
        if ((mk & m2(2, 3)) && !(mk & R2_CORNER)) {  // west
            const R r = (f[0] + f[2] + f[4] + (R)2 * (f[3] + f[6] + f[7])) / ((R)1 - u0);
            f[1] = f[3] + (R)2 * r * u0 / (R)3;
            f[5] = f[7] + r * u0 / (R)6;
            f[8] = f[6] + r * u0 / (R)6;
        }
    }
#pragma unroll
    for (int dir = 1; dir < 9; ++dir)
        if ((mk & m2(3, dir)) == m2(1, dir)) f[Lat<9>::opp(dir)] = f[dir];
    if ((mk & m2(3, 1)) == m2(3, 1)) {  // east outlet
        if (outlet_profile == LBM_OUTLET_ZOUHE) {
            const R r = (f[0] + f[2] + f[4] + (R)2 * (f[1] + f[5] + f[8])) / ((R)1 - u0);
            f[3] = f[1] - (R)2 * r * u0 / (R)3;
            f[7] = f[5] - r * u0 / (R)6;
            f[6] = f[8] - r * u0 / (R)6;
        }
        zero_v = true;  // gpuUpdateMacro2D forces v = 0 on east outlets (GpuUpdateMacro.cu:30)
    }
}

// ---------------------------------------------------------------------------
// Reference semantics, D3Q19: gpuBcInlet3D faces W, E, S, N, B, T
// (GpuBoundaries.cu:92-394, including its west/east density denominators),
// gpuBcSimpleWall3D straight walls (:445-490) and gpuBcSymm3D (:2086-2168).
// ---------------------------------------------------------------------------
template <class R>
__device__ __forceinline__ void ref_face3(R (&f)[19], int face, R uu, R vv, R ww) {
    R d, n1, n2;
    switch (face) {
    case 2:  // WEST
        d = (R)1 / ((R)1 + uu) * (f[0] + f[3] + f[4] + f[5] + f[6] + f[15] + f[16] + f[17] + f[18] + (R)2 * (f[2] + f[8] + f[10] + f[12] + f[14]));
        n1 = (R)0.5 * (f[3] + f[15] + f[17] - (f[4] + f[16] + f[18])) - d * vv / (R)3;
        n2 = (R)0.5 * (f[5] + f[15] + f[16] - (f[6] + f[17] + f[18])) - d * ww / (R)3;
        f[1] = f[2] + d * uu / (R)3;
        f[7] = f[10] + d * (uu + vv) / (R)6 - n1;
        f[9] = f[8] + d * (uu - vv) / (R)6 + n1;
        f[11] = f[14] + d * (uu + ww) / (R)6 - n2;
        f[13] = f[12] + d * (uu - ww) / (R)6 + n2;
        break;
    case 1:  // EAST
        d = (R)1 / ((R)1 - uu) * (f[0] + f[3] + f[4] + f[5] + f[6] + f[15] + f[16] + f[17] + f[18] + (R)2 * (f[1] + f[7] + f[9] + f[11] + f[13]));
        n1 = (R)0.5 * (f[3] + f[15] + f[17] - (f[4] + f[16] + f[18])) - d * vv / (R)3;
        n2 = (R)0.5 * (f[5] + f[15] + f[16] - (f[6] + f[17] + f[18])) - d * ww / (R)3;
        f[2] = f[1] - d * uu / (R)3;
        f[8] = f[9] - d * (uu - vv) / (R)6 - n1;
        f[10] = f[7] - d * (uu + vv) / (R)6 + n1;
        f[12] = f[13] - d * (uu - ww) / (R)6 - n2;
        f[14] = f[11] - d * (uu + ww) / (R)6 + n2;
        break;
    case 4:  // SOUTH
        d = (R)1 / ((R)1 - vv) * (f[0] + f[1] + f[2] + f[5] + f[6] + f[11] + f[12] + f[13] + f[14] + (R)2 * (f[4] + f[9] + f[10] + f[16] + f[18]));
        n1 = (R)0.5 * (f[1] + f[11] + f[13] - (f[2] + f[12] + f[14])) - d * uu / (R)3;
        n2 = (R)0.5 * (f[5] + f[11] + f[12] - (f[6] + f[13] + f[14])) - d * ww / (R)3;
        f[3] = f[4] + d * vv / (R)3;
        f[7] = f[10] + d * (vv + uu) / (R)6 - n1;
        f[8] = f[9] + d * (vv - uu) / (R)6 + n1;
        f[15] = f[18] + d * (vv + ww) / (R)6 - n2;
        f[17] = f[16] + d * (vv - ww) / (R)6 + n2;
        break;
    case 3:  // NORTH
        d = (R)1 / ((R)1 + vv) * (f[0] + f[1] + f[2] + f[5] + f[6] + f[11] + f[12] + f[13] + f[14] + (R)2 * (f[3] + f[7] + f[8] + f[15] + f[17]));
        n1 = (R)0.5 * (f[1] + f[11] + f[13] - (f[2] + f[12] + f[14])) - d * uu / (R)3;
        n2 = (R)0.5 * (f[5] + f[11] + f[12] - (f[6] + f[13] + f[14])) - d * ww / (R)3;
        f[4] = f[3] - d * vv / (R)3;
        f[9] = f[8] - d * (vv - uu) / (R)6 - n1;
        f[10] = f[7] - d * (vv + uu) / (R)6 + n1;
        f[16] = f[17] - d * (vv - ww) / (R)6 - n2;
        f[18] = f[15] - d * (vv + ww) / (R)6 + n2;
        break;
    case 6:  // BOTTOM
        d = (R)1 / ((R)1 - ww) * (f[0] + f[1] + f[2] + f[3] + f[4] + f[7] + f[8] + f[9] + f[10] + (R)2 * (f[6] + f[13] + f[14] + f[17] + f[18]));
        n1 = (R)0.5 * (f[1] + f[7] + f[9] - (f[2] + f[8] + f[10])) - d * uu / (R)3;
        n2 = (R)0.5 * (f[3] + f[7] + f[8] - (f[4] + f[9] + f[10])) - d * vv / (R)3;
        f[5] = f[6] + d * ww / (R)3;
        f[11] = f[14] + d * (ww + uu) / (R)6 - n1;
        f[12] = f[13] + d * (ww - uu) / (R)6 + n1;
        f[15] = f[18] + d * (ww + vv) / (R)6 - n2;
        f[16] = f[17] + d * (ww - vv) / (R)6 + n2;
        break;
    default:  // 5: TOP
        d = (R)1 / ((R)1 + ww) * (f[0] + f[1] + f[2] + f[3] + f[4] + f[7] + f[8] + f[9] + f[10] + (R)2 * (f[5] + f[11] + f[12] + f[15] + f[16]));
        n1 = (R)0.5 * (f[1] + f[7] + f[9] - (f[2] + f[8] + f[10])) - d * uu / (R)3;
        n2 = (R)0.5 * (f[3] + f[7] + f[8] - (f[4] + f[9] + f[10])) - d * vv / (R)3;
        f[6] = f[5] - d * ww / (R)3;
        f[13] = f[12] - d * (ww - uu) / (R)6 - n1;
        f[14] = f[11] - d * (ww + uu) / (R)6 + n1;
        f[17] = f[16] - d * (ww - vv) / (R)6 - n2;
        f[18] = f[15] - d * (ww + vv) / (R)6 + n2;
        break;
    }
}

template <class R>
__device__ __forceinline__ void bc_ref_d3q19(R (&f)[19], uint64_t mk, R uu, R vv, R ww,
                                             int update_inlet_outlet, bool &keep_macro) {
    if (!(mk & R3_FLUID)) return;
    if (mk & R3_INLT_B) {
        const int faces[6] = {2, 1, 4, 3, 6, 5};
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            const int face = faces[k];
            const uint64_t inl = m3(2, face), all = mk & m3(7, face);
            const bool hit = (mk & inl) && !(mk & R3_CORNER) && (face == 1 ? all == inl : all == (mk & inl));
            if (hit) ref_face3(f, face, uu, vv, ww);
        }
    }
#pragma unroll
    for (int dir = 1; dir < 19; ++dir)
        if ((mk & m3(7, dir)) == m3(1, dir)) f[Lat<19>::opp(dir)] = f[dir];
    if (mk & R3_SYMP_B) {
        auto is = [&](int dir) { return (mk & m3(7, dir)) == m3(5, dir); };
        if (is(2)) { f[1] = f[2]; f[7] = f[8]; f[9] = f[10]; f[11] = f[12]; f[13] = f[14]; }
        if (is(1)) { f[2] = f[1]; f[8] = f[7]; f[10] = f[9]; f[12] = f[11]; f[14] = f[13]; }
        if (is(4)) { f[3] = f[4]; f[7] = f[9]; f[8] = f[10]; f[15] = f[16]; f[17] = f[18]; }
        if (is(3)) { f[4] = f[3]; f[9] = f[7]; f[10] = f[8]; f[16] = f[15]; f[18] = f[17]; }
        if (is(6)) { f[5] = f[6]; f[11] = f[13]; f[12] = f[14]; f[15] = f[17]; f[16] = f[18]; }
        if (is(5)) { f[6] = f[5]; f[13] = f[11]; f[14] = f[12]; f[17] = f[15]; f[18] = f[16]; }
    }
    // gpuUpdateMacro3D leaves inlet nodes untouched unless UpdateInltOutl
    // (GpuUpdateMacro.cu:150-151).
    if ((mk & R3_OUTL_B) == R3_INLT_B && !update_inlet_outlet) keep_macro = true;
}

// ---------------------------------------------------------------------------
// Physics semantics: mass-balanced Zou-He face with Hecht-Harting transverse
// corrections, for any lattice face.  FACE = inward normal: 0 +x (west face),
// 1 -x (east), 2 +y (south), 3 -y (north), 4 +z (bottom), 5 -z (top).
// Velocity faces impose (ux,uy,uz); pressure faces impose rho and a purely
// normal velocity.  With e the inward normal, unknowns are c.e = +1:
//   rho (1 - u.e) = S0 + 2 S-            (S0: c.e = 0, S-: c.e = -1)
//   f_e       = f_-e + 6 w_e rho (u.e)
//   f_(e+t)   = f_opp + rho (u.e)/6 + rho (u.t)/2 - (1/2) sum_{c.e=0} (c.t) f_c
// ---------------------------------------------------------------------------
template <int Q, int FACE, class R>
__device__ __forceinline__ void zou_he_face(R (&f)[Q], bool pressure, R rho_set, R ux, R uy, R uz) {
    using L = Lat<Q>;
    constexpr int ex = FACE == 0 ? 1 : (FACE == 1 ? -1 : 0);
    constexpr int ey = FACE == 2 ? 1 : (FACE == 3 ? -1 : 0);
    constexpr int ez = FACE == 4 ? 1 : (FACE == 5 ? -1 : 0);
    R s0 = 0, sm = 0;
#pragma unroll
    for (int d = 0; d < Q; ++d) {
        constexpr int dummy = 0;
        (void)dummy;
        const int ce = L::cx(d) * ex + L::cy(d) * ey + L::cz(d) * ez;
        if (ce == 0) s0 += f[d];
        if (ce == -1) sm += f[d];
    }
    R rho, ue;
    if (pressure) {
        rho = rho_set;
        ue = (R)1 - (s0 + (R)2 * sm) / rho;
        ux = ue * (R)ex;
        uy = ue * (R)ey;
        uz = ue * (R)ez;
    } else {
        ue = ux * (R)ex + uy * (R)ey + uz * (R)ez;
        rho = (s0 + (R)2 * sm) / ((R)1 - ue);
    }
#pragma unroll
    for (int d = 1; d < Q; ++d) {
        const int ce = L::cx(d) * ex + L::cy(d) * ey + L::cz(d) * ez;
        if (ce != 1) continue;
        const int tx = L::cx(d) - ex, ty = L::cy(d) - ey, tz = L::cz(d) - ez;
        const int o = L::opp(d);
        if (tx == 0 && ty == 0 && tz == 0) {
            f[d] = f[o] + (R)(6.0 * L::w(d)) * rho * ue;
        } else {
            R st = 0;
#pragma unroll
            for (int c = 0; c < Q; ++c) {
                const int cce = L::cx(c) * ex + L::cy(c) * ey + L::cz(c) * ez;
                const int ct = L::cx(c) * tx + L::cy(c) * ty + L::cz(c) * tz;
                if (cce == 0 && ct != 0) st += (R)ct * f[c];
            }
            const R ut = ux * (R)tx + uy * (R)ty + uz * (R)tz;
            f[d] = f[o] + rho * ue / (R)6 + rho * ut / (R)2 - st / (R)2;
        }
    }
}

// Moving wall (Ladd): after half-way bounce-back, each incoming population d
// of a wall link gains 6 w_d rho_0 (c_d . u_w), rho_0 the reference density.
// For a wall velocity tangential to the face the gains cancel pairwise, so the
// node's mass is unchanged.  (The node's own density in place of rho_0 feeds
// back on itself and slowly destabilises a cavity lid.)
template <int Q, class R>
__device__ __forceinline__ void bc_moving_wall(R (&f)[Q], unsigned long long links, R rho, R uwx, R uwy, R uwz) {
    using L = Lat<Q>;
#pragma unroll
    for (int d = 1; d < Q; ++d)
        if ((links >> d) & 1ull) {
            const R cu = (R)L::cx(d) * uwx + (R)L::cy(d) * uwy + (R)L::cz(d) * uwz;
            f[d] += (R)(6.0 * L::w(d)) * rho * cu;
        }
}

template <int Q, class R>
__device__ __forceinline__ void bc_phys(R (&f)[Q], int face, bool pressure, R rho_set, R ux, R uy, R uz) {
    switch (face) {
    case 0: zou_he_face<Q, 0>(f, pressure, rho_set, ux, uy, uz); break;
    case 1: zou_he_face<Q, 1>(f, pressure, rho_set, ux, uy, uz); break;
    case 2: zou_he_face<Q, 2>(f, pressure, rho_set, ux, uy, uz); break;
    case 3: zou_he_face<Q, 3>(f, pressure, rho_set, ux, uy, uz); break;
    case 4: if (Q == 19) zou_he_face<Q, 4>(f, pressure, rho_set, ux, uy, uz); break;
    case 5: if (Q == 19) zou_he_face<Q, 5>(f, pressure, rho_set, ux, uy, uz); break;
    default: break;
    }
}

}  // namespace lbm
