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
constexpr uint64_t R3_WALL_B = 1ull << 54, R3_INLT_B = 2ull << 54, R3_OUTL_B = 3ull << 54,
                   R3_CYCL_B = 4ull << 54, R3_SYMP_B = 5ull << 54, R3_CORNER = 1ull << 57, R3_FLUID = 1ull << 58;

// ---------------------------------------------------------------------------
// Reference semantics, D2Q9: gpuBcInlet2D, gpuBcWall2D (straight), and the
// east outlet of gpuBcOutlet2D (GpuBoundaries.cu:12-71, :400-443,
// :1562-1653), in that order, on the node's streamed populations.  CURVED:
// a wall link dir sets f_opp(dir) to cv[dir] (ref_curved) instead of f[dir].
// The extrapolation outlets rewrite f1, f5, f8 from the post-stream,
// post-wall values of the nodes one and two to the west, ext[0..2] and
// ext[3..5] (ref2_outlet_neighbours); with ext null, or HEmodel, which the
// 2D kernel has no case for, they leave the node as it is.
// ---------------------------------------------------------------------------
template <class R, bool CURVED = false>
__device__ __forceinline__ void bc_ref_d2q9(R (&f)[9], uint32_t mk, R u0, int outlet_profile,
                                            bool &zero_v, const R *cv = nullptr, const R *ext = nullptr) {
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
        if ((mk & m2(3, dir)) == m2(1, dir)) f[Lat<9>::opp(dir)] = CURVED ? cv[dir] : f[dir];
    if ((mk & m2(3, 1)) == m2(3, 1)) {  // east outlet
        if (outlet_profile == LBM_OUTLET_ZOUHE) {
            const R r = (f[0] + f[2] + f[4] + (R)2 * (f[1] + f[5] + f[8])) / ((R)1 - u0);
            f[3] = f[1] - (R)2 * r * u0 / (R)3;
            f[7] = f[5] - r * u0 / (R)6;
            f[6] = f[8] - r * u0 / (R)6;
        } else if (ext && outlet_profile == LBM_OUTLET_SECOND) {
            f[1] = (R)2 * ext[0] - ext[3];
            f[5] = (R)2 * ext[1] - ext[4];
            f[8] = (R)2 * ext[2] - ext[5];
        } else if (ext && outlet_profile == LBM_OUTLET_FIRST) {
            f[1] = ext[0];
            f[5] = ext[1];
            f[8] = ext[2];
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

// ---------------------------------------------------------------------------
// The reference's HH ("complex") wall, gpuBcComplexWall3D
// (GpuBoundaries.cu:492-1560), for walls at rest.  The kernel counts the
// node's wall-typed links and finds up to three inward wall normals from the
// wall bits of directions 1-6; then
//   5 wall links (face, normal e):  f_e = f_-e and, for each tangential axis
//     t, N_t = (1/2)(sum_{c.e=0, c_t=+1} f_c - sum_{c.e=0, c_t=-1} f_c),
//     f_(e+t) = f_(-e-t) - N_t, f_(e-t) = f_(-e+t) + N_t            (:558-861)
//   9 wall links (edge, normals a, b, third axis t):
//     N_t = -(f_(+t) - f_(-t))/4; f_a = f_-a, f_b = f_-b, f_(a+b) = f_(-a-b),
//     f_(n+t) = f_(-n-t) + N_t, f_(n-t) = f_(-n+t) - N_t for n = a, b; the
//     two buried links a-b and b-a get S/22 and the rest population 12 S/22,
//     S the sum of the other populations                             (:863-1364)
//   12 wall links (corner, normals a, b, c): f_n = f_-n for the three axes
//     and the three inward diagonals; the six buried diagonals get S/18 and
//     the rest population 12 S/18, S the sum over the twelve others  (:1366-1559)
// The wall velocity terms of the face formulas are zero and left out.
// ---------------------------------------------------------------------------
__host__ __device__ constexpr int dir19(int cx, int cy, int cz) {
    int r = -1;
    for (int d = 0; d < 19; ++d)
        if (Lat<19>::cx(d) == cx && Lat<19>::cy(d) == cy && Lat<19>::cz(d) == cz) r = d;
    return r;
}
// direction of s1 * unit(a1) + s2 * unit(a2) (s2 = 0: the axis direction)
__host__ __device__ constexpr int dir_of(int a1, int s1, int a2 = 0, int s2 = 0) {
    return dir19((a1 == 0 ? s1 : 0) + (a2 == 0 ? s2 : 0), (a1 == 1 ? s1 : 0) + (a2 == 1 ? s2 : 0),
                 (a1 == 2 ? s1 : 0) + (a2 == 2 ? s2 : 0));
}
template <int A>
__host__ __device__ constexpr int comp19(int d) {
    return A == 0 ? Lat<19>::cx(d) : (A == 1 ? Lat<19>::cy(d) : Lat<19>::cz(d));
}

template <int A, int S, class R>
__device__ __forceinline__ void hh_face(R (&f)[19]) {
    constexpr int T1 = A == 0 ? 1 : 0, T2 = A == 2 ? 1 : 2;
    R p1 = 0, m1 = 0, p2 = 0, m2 = 0;
#pragma unroll
    for (int d = 1; d < 19; ++d) {
        if (comp19<A>(d) != 0) continue;
        if (comp19<T1>(d) == 1) p1 += f[d];
        if (comp19<T1>(d) == -1) m1 += f[d];
        if (comp19<T2>(d) == 1) p2 += f[d];
        if (comp19<T2>(d) == -1) m2 += f[d];
    }
    const R n1 = (R)0.5 * (p1 - m1), n2 = (R)0.5 * (p2 - m2);
    f[dir_of(A, S)] = f[dir_of(A, -S)];
    f[dir_of(A, S, T1, 1)] = f[dir_of(A, -S, T1, -1)] - n1;
    f[dir_of(A, S, T1, -1)] = f[dir_of(A, -S, T1, 1)] + n1;
    f[dir_of(A, S, T2, 1)] = f[dir_of(A, -S, T2, -1)] - n2;
    f[dir_of(A, S, T2, -1)] = f[dir_of(A, -S, T2, 1)] + n2;
}

template <int A1, int S1, int A2, int S2, class R>
__device__ __forceinline__ void hh_edge(R (&f)[19]) {
    constexpr int T = 3 - A1 - A2;
    constexpr int b1 = dir_of(A1, S1, A2, -S2), b2 = dir_of(A1, -S1, A2, S2);
    const R nt = (R)-0.25 * (f[dir_of(T, 1)] - f[dir_of(T, -1)]);
    f[dir_of(A1, S1)] = f[dir_of(A1, -S1)];
    f[dir_of(A2, S2)] = f[dir_of(A2, -S2)];
    f[dir_of(A1, S1, A2, S2)] = f[dir_of(A1, -S1, A2, -S2)];
    f[dir_of(A1, S1, T, 1)] = f[dir_of(A1, -S1, T, -1)] + nt;
    f[dir_of(A1, S1, T, -1)] = f[dir_of(A1, -S1, T, 1)] - nt;
    f[dir_of(A2, S2, T, 1)] = f[dir_of(A2, -S2, T, -1)] + nt;
    f[dir_of(A2, S2, T, -1)] = f[dir_of(A2, -S2, T, 1)] - nt;
    R s = 0;
#pragma unroll
    for (int d = 1; d < 19; ++d)
        if (d != b1 && d != b2) s += f[d];
    f[b1] = s * (R)(1.0 / 22.0);
    f[b2] = s * (R)(1.0 / 22.0);
    f[0] = s * (R)(12.0 / 22.0);
}

template <int SX, int SY, int SZ, class R>
__device__ __forceinline__ void hh_corner(R (&f)[19]) {
    f[dir_of(0, SX)] = f[dir_of(0, -SX)];
    f[dir_of(1, SY)] = f[dir_of(1, -SY)];
    f[dir_of(2, SZ)] = f[dir_of(2, -SZ)];
    f[dir_of(0, SX, 1, SY)] = f[dir_of(0, -SX, 1, -SY)];
    f[dir_of(0, SX, 2, SZ)] = f[dir_of(0, -SX, 2, -SZ)];
    f[dir_of(1, SY, 2, SZ)] = f[dir_of(1, -SY, 2, -SZ)];
    // buried: diagonals whose two components have the opposite sign pattern
    // of the normal
    constexpr int b0 = dir_of(0, SX, 1, -SY), b1 = dir_of(0, -SX, 1, SY), b2 = dir_of(0, SX, 2, -SZ),
                  b3 = dir_of(0, -SX, 2, SZ), b4 = dir_of(1, SY, 2, -SZ), b5 = dir_of(1, -SY, 2, SZ);
    R s = 0;
#pragma unroll
    for (int d = 1; d < 19; ++d)
        if (d != b0 && d != b1 && d != b2 && d != b3 && d != b4 && d != b5) s += f[d];
    const R c = s * (R)(1.0 / 18.0);
    f[b0] = c; f[b1] = c; f[b2] = c; f[b3] = c; f[b4] = c; f[b5] = c;
    f[0] = (R)12 * c;
}

template <int A1, int A2, class R>
__device__ __forceinline__ void hh_edge_signed(R (&f)[19], int s1, int s2) {
    if (s1 > 0) {
        if (s2 > 0) hh_edge<A1, 1, A2, 1>(f); else hh_edge<A1, 1, A2, -1>(f);
    } else {
        if (s2 > 0) hh_edge<A1, -1, A2, 1>(f); else hh_edge<A1, -1, A2, -1>(f);
    }
}

template <class R>
__device__ __forceinline__ void hh_wall3(R (&f)[19], uint64_t mk) {
    int walls = 0;
#pragma unroll
    for (int d = 1; d < 19; ++d) walls += (mk & m3(7, d)) == m3(1, d);
    // inward normals: slot j = 0, 1, 2 takes the first of directions 1..6
    // whose wall bit is set and whose axis has no normal yet; a wall bit in
    // direction c gives the normal -c on its axis
    int sgn[3] = {0, 0, 0}, slot[3] = {-1, -1, -1};
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        bool done = false;
#pragma unroll
        for (int d = 1; d <= 6; ++d) {
            const int a = (d - 1) >> 1;
            if (!done && (mk & m3(1, d)) && slot[a] < 0) {
                slot[a] = j;
                sgn[a] = (d & 1) ? -1 : 1;
                done = true;
            }
        }
    }
    if (walls == 5 && (mk & R3_FLUID) && (mk & R3_WALL_B)) {
        auto is = [&](int d) { return (mk & m3(1, d)) && (mk & m3(7, d)) == (mk & m3(1, d)); };
        if (is(2)) hh_face<0, 1>(f);
        if (is(1)) hh_face<0, -1>(f);
        if (is(4)) hh_face<1, 1>(f);
        if (is(3)) hh_face<1, -1>(f);
        if (is(6)) hh_face<2, 1>(f);
        if (is(5)) hh_face<2, -1>(f);
    }
    if (walls == 9) {
        if (slot[0] == 0 && slot[2] == 1) hh_edge_signed<0, 2>(f, sgn[0], sgn[2]);
        if (slot[1] == 0 && slot[2] == 1) hh_edge_signed<1, 2>(f, sgn[1], sgn[2]);
        if (slot[0] == 0 && slot[1] == 1) hh_edge_signed<0, 1>(f, sgn[0], sgn[1]);
    }
    if (walls == 12 && slot[0] == 0 && slot[1] == 1 && slot[2] == 2) {
        const int k = (sgn[0] > 0) | ((sgn[1] > 0) << 1) | ((sgn[2] > 0) << 2);
        switch (k) {
        case 0: hh_corner<-1, -1, -1>(f); break;
        case 1: hh_corner<1, -1, -1>(f); break;
        case 2: hh_corner<-1, 1, -1>(f); break;
        case 3: hh_corner<1, 1, -1>(f); break;
        case 4: hh_corner<-1, -1, 1>(f); break;
        case 5: hh_corner<1, -1, 1>(f); break;
        case 6: hh_corner<-1, 1, 1>(f); break;
        default: hh_corner<1, 1, 1>(f); break;
        }
    }
}

// gpuBcInlet3D faces W, E, S, N, B, T (GpuBoundaries.cu:92-394) and the
// straight walls of gpuBcSimpleWall3D (:445-490) or the HH wall.  CURVED:
// the simple wall's curved branch, f_opp(dir) = cv[dir] (ref_curved).
template <class R, bool CURVED = false>
__device__ __forceinline__ void bc_ref3_inlet_wall(R (&f)[19], uint64_t mk, R uu, R vv, R ww, bool hh,
                                                   const R *cv = nullptr) {
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
    if (hh) {
        hh_wall3(f, mk);
    } else {
#pragma unroll
        for (int dir = 1; dir < 19; ++dir)
            if ((mk & m3(7, dir)) == m3(1, dir)) f[Lat<19>::opp(dir)] = CURVED ? cv[dir] : f[dir];
    }
}

// gpuBcSymm3D (GpuBoundaries.cu:2086-2168).
template <class R>
__device__ __forceinline__ void bc_ref3_symm(R (&f)[19], uint64_t mk) {
    if (!(mk & R3_FLUID) || !(mk & R3_SYMP_B)) return;
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
__device__ __forceinline__ bool ref3_keep_macro(uint64_t mk, int update_inlet_outlet) {
    return (mk & R3_FLUID) && (mk & R3_OUTL_B) == R3_INLT_B && !update_inlet_outlet;
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

// ---------------------------------------------------------------------------
// The physics-mode faces and moving walls in storage units: h = (f - sigma r) S
// with r the model's rest state (isotropic: r_d = r_opp(d), sum 1) and S the
// storage scale.  The same closures as zou_he_face and bc_moving_wall, with
// the O(1) sums that cancel to the normal velocity or the density replaced by
// identities of the shift: sum_{c.e=0} r + 2 sum_{c.e=-1} r = 1, r_d = r_opp(d)
// and sum_{c.e=0} (c.t) r_c = 0.  So with K = (sum_{c.e=0} h + 2 sum_{c.e=-1}
// h)/S the pressure face gives u_e = ((rho - sigma) - K)/rho and the velocity
// face rho = (sigma + K)/(1 - u_e), from deviations only: an FP32 face then
// keeps the digits that the f-space form loses to the cancellation (relative
// 1e-4 of a 1e-3 velocity per step).  rho_dev = rho_set - sigma, formed in FP64
// on the host.
// ---------------------------------------------------------------------------
template <int Q, int FACE>
__device__ __forceinline__ void zou_he_face_h(float (&h)[Q], bool pressure, float rho_dev, float sigma, float S,
                                              float invS, float ux, float uy, float uz) {
    using L = Lat<Q>;
    constexpr int ex = FACE == 0 ? 1 : (FACE == 1 ? -1 : 0);
    constexpr int ey = FACE == 2 ? 1 : (FACE == 3 ? -1 : 0);
    constexpr int ez = FACE == 4 ? 1 : (FACE == 5 ? -1 : 0);
    float h0 = 0.f, hm = 0.f;
#pragma unroll
    for (int d = 0; d < Q; ++d) {
        const int ce = L::cx(d) * ex + L::cy(d) * ey + L::cz(d) * ez;
        if (ce == 0) h0 += h[d];
        if (ce == -1) hm += h[d];
    }
    const float K = (h0 + 2.f * hm) * invS;
    float rho, ue;
    if (pressure) {
        rho = rho_dev + sigma;
        ue = (rho_dev - K) / rho;
        ux = ue * (float)ex;
        uy = ue * (float)ey;
        uz = ue * (float)ez;
    } else {
        ue = ux * (float)ex + uy * (float)ey + uz * (float)ez;
        rho = (sigma + K) / (1.f - ue);
    }
    const float rS = rho * S;
#pragma unroll
    for (int d = 1; d < Q; ++d) {
        const int ce = L::cx(d) * ex + L::cy(d) * ey + L::cz(d) * ez;
        if (ce != 1) continue;
        const int tx = L::cx(d) - ex, ty = L::cy(d) - ey, tz = L::cz(d) - ez;
        const int o = L::opp(d);
        if (tx == 0 && ty == 0 && tz == 0) {
            h[d] = fmaf((float)(6.0 * L::w(d)) * rS, ue, h[o]);
        } else {
            float st = 0.f;
#pragma unroll
            for (int c = 0; c < Q; ++c) {
                const int cce = L::cx(c) * ex + L::cy(c) * ey + L::cz(c) * ez;
                const int ct = L::cx(c) * tx + L::cy(c) * ty + L::cz(c) * tz;
                if (cce == 0 && ct != 0) st += (float)ct * h[c];
            }
            const float ut = ux * (float)tx + uy * (float)ty + uz * (float)tz;
            h[d] = h[o] + rS * (ue * (1.f / 6.f) + ut * 0.5f) - 0.5f * st;
        }
    }
}

template <int Q>
__device__ __forceinline__ void bc_phys_h(float (&h)[Q], int face, bool pressure, float rho_dev, float sigma, float S,
                                          float invS, float ux, float uy, float uz) {
    switch (face) {
    case 0: zou_he_face_h<Q, 0>(h, pressure, rho_dev, sigma, S, invS, ux, uy, uz); break;
    case 1: zou_he_face_h<Q, 1>(h, pressure, rho_dev, sigma, S, invS, ux, uy, uz); break;
    case 2: zou_he_face_h<Q, 2>(h, pressure, rho_dev, sigma, S, invS, ux, uy, uz); break;
    case 3: zou_he_face_h<Q, 3>(h, pressure, rho_dev, sigma, S, invS, ux, uy, uz); break;
    case 4: if (Q == 19) zou_he_face_h<Q, 4>(h, pressure, rho_dev, sigma, S, invS, ux, uy, uz); break;
    case 5: if (Q == 19) zou_he_face_h<Q, 5>(h, pressure, rho_dev, sigma, S, invS, ux, uy, uz); break;
    default: break;
    }
}

// Moving wall in storage units: h_d gains S 6 w_d rho_0 (c_d . u_w).
template <int Q>
__device__ __forceinline__ void bc_moving_wall_h(float (&h)[Q], unsigned long long links, float rho, float S,
                                                 float uwx, float uwy, float uwz) {
    using L = Lat<Q>;
#pragma unroll
    for (int d = 1; d < Q; ++d)
        if ((links >> d) & 1ull) {
            const float cu = (float)L::cx(d) * uwx + (float)L::cy(d) * uwy + (float)L::cz(d) * uwz;
            h[d] += (float)(6.0 * L::w(d)) * rho * S * cu;
        }
}

}  // namespace lbm
