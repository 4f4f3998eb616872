/*
 * CPU ORACLE for the lattice-Boltzmann time step -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain C++ restatement of the reference solver's single-phase time step
 * (ZPaulo/Thesis, "Source code/lbm-solver_final"), used by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU baseline as the checker.  The
 * product (thesis_gb300/) never links or calls it.
 *
 * Two semantics, selected per run by orc_params.mode:
 *   mode 0 (reference): the reference's loop and quirks, restated in the same
 *     expression order so FP32 results match the reference kernels compiled
 *     for the host (oracle/_ref) to the last bit on x86 without FMA.
 *   mode 1 (physics): the standard formulations the reference approximates:
 *     equilibrium start, half-way bounce-back from the node's own outgoing
 *     population, full Zou-He velocity/pressure faces, D2Q9 MRT equilibria
 *     without the extra density factor, D3Q19 MRT writing all 19 outputs,
 *     TRT in 3D, no forced v=0 on east outlets, and every link towards a
 *     solid or out-of-domain node treated as a wall link.
 *
 * Files restated (file:line within Source code/lbm-solver_final/):
 *   lattice tables          GpuInit.cu:94-99 (D2Q9), :822-842 (D3Q19)
 *   BC masks / stream flags GpuInit.cu:1055-1122 (2D), :1157-1238 (3D);
 *                           bit layouts include/BcMacros.h, include/BcMacros3D.h
 *   equilibria              GpuCollision.cu:21-32
 *   BGK                     GpuCollision.cu:528-550, :882-916
 *   TRT                     GpuCollision.cu:917-969 (omegaA GpuInit.cu:103)
 *   MRT                     GpuCollision.cu:971-1037, :1039-1170;
 *                           matrices CellFunctions.cu:7-153
 *   streaming               GpuStream.cu:8-28, :160-194
 *   inlet (Zou-He velocity) GpuBoundaries.cu:12-71 (2D), :73-399 (3D)
 *   straight walls          GpuBoundaries.cu:400-443 (2D), :445-490 (3D)
 *   2D outlets              GpuBoundaries.cu:1562-1653
 *   3D periodic / symmetry  GpuBoundaries.cu:2025-2168
 *   macroscopic update      GpuUpdateMacro.cu:6-41 (2D), :137-213 (3D)
 *   L2 residual             ComputeResiduals.cu:13-26
 *   loop order              Iterate.cu:385-518, Iterate3D.cu:493-653
 *   HH ("complex") 3D wall  GpuBoundaries.cu:492-1560
 *
 *   curved walls            GpuBoundaries.cu:414-432 (2D), :461-479 (3D);
 *                           link fractions GpuInit.cu:1086-1088, :1203-1207
 *
 * Not restated (the entry points return ORC_UNSUPPORTED): the
 * 3D outlet kernel (it addresses directions with the 2D plane size,
 * GpuBoundaries.cu:1662, so it rewrites other nodes) and the
 * INLET_PROF 3D profile the reference itself refuses (Iterate3D.cu:200-206).
 */
#include <math.h>
#include <cmath>
#include <stdint.h>
#include <string.h>

#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_OK 0
#define ORC_UNSUPPORTED 3
#define ORC_BAD_INPUT 4

namespace {

/* ---------------- lattice tables (reference ordering) ---------------- */
const int cx2[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1};
const int cy2[9] = {0, 0, 1, 0, -1, 1, 1, -1, -1};
const int opp2[9] = {0, 3, 4, 1, 2, 7, 8, 5, 6};

const int cx3[19] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0};
const int cy3[19] = {0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1};
const int cz3[19] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1};
const int opp3[19] = {0, 2, 1, 4, 3, 6, 5, 10, 9, 8, 7, 14, 13, 12, 11, 18, 17, 16, 15};

/* D2Q9 moment basis M (CellFunctions.cu:31-40) and diag(S) (:47-55). */
const double M2[81] = {
    1, 1, 1, 1, 1, 1, 1, 1, 1,      -4, -1, -1, -1, -1, 2, 2, 2, 2,
    4, -2, -2, -2, -2, 1, 1, 1, 1,  0, 1, 0, -1, 0, 1, -1, -1, 1,
    0, -2, 0, 2, 0, 1, -1, -1, 1,   0, 0, 1, 0, -1, 1, 1, -1, -1,
    0, 0, -2, 0, 2, 1, 1, -1, -1,   0, 1, -1, 1, -1, 0, 0, 0, 0,
    0, 0, 0, 0, 0, 1, -1, 1, -1};
/* D3Q19 moment basis (CellFunctions.cu:94-113), reference direction order. */
const double M3[361] = {
    1,   1,   1,   1,   1,   1,   1,   1, 1, 1, 1, 1, 1, 1, 1, 1,  1,  1,  1,
    -30, -11, -11, -11, -11, -11, -11, 8, 8, 8, 8, 8, 8, 8, 8, 8,  8,  8,  8,
    12,  -4,  -4,  -4,  -4,  -4,  -4,  1, 1, 1, 1, 1, 1, 1, 1, 1,  1,  1,  1,
    0,   1,   -1,  0,   0,   0,   0,   1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0,
    0,   -4,  4,   0,   0,   0,   0,   1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0,
    0,   0,   0,   1,   -1,  0,   0,   1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1,
    0,   0,   0,   -4,  4,   0,   0,   1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1,
    0,   0,   0,   0,   0,   1,   -1,  0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1,
    0,   0,   0,   0,   0,   -4,  4,   0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1,
    0,   2,   2,   -1,  -1,  -1,  -1,  1, 1, 1, 1, 1, 1, 1, 1, -2, -2, -2, -2,
    0,   -4,  -4,  2,   2,   2,   2,   1, 1, 1, 1, 1, 1, 1, 1, -2, -2, -2, -2,
    0,   0,   0,   1,   1,   -1,  -1,  1, 1, 1, 1, -1, -1, -1, -1, 0, 0, 0, 0,
    0,   0,   0,   -2,  -2,  2,   2,   1, 1, 1, 1, -1, -1, -1, -1, 0, 0, 0, 0,
    0,   0,   0,   0,   0,   0,   0,   1, -1, -1, 1, 0, 0, 0, 0, 0, 0, 0, 0,
    0,   0,   0,   0,   0,   0,   0,   0, 0, 0, 0, 0, 0, 0, 0, 1, -1, -1, 1,
    0,   0,   0,   0,   0,   0,   0,   0, 0, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0,
    0,   0,   0,   0,   0,   0,   0,   1, -1, 1, -1, -1, 1, -1, 1, 0, 0, 0, 0,
    0,   0,   0,   0,   0,   0,   0,   -1, -1, 1, 1, 0, 0, 0, 0, 1, -1, 1, -1,
    0,   0,   0,   0,   0,   0,   0,   0, 0, 0, 0, 1, 1, -1, -1, -1, -1, 1, 1};

/* Bit layout of the reference BC masks. */
inline uint64_t bc2_mask(uint64_t type, int dir) { return type << ((dir - 1) * 2); }
const uint64_t BC2_B_ALL = 3ull << 16, BC2_WALL_B = 1ull << 16, BC2_CORNER = 1ull << 18,
               BC2_FLUID = 1ull << 19, BC2_INLT_B = 2ull << 16;
inline uint64_t bc3_mask(uint64_t type, int dir) { return type << ((dir - 1) * 3); }
const uint64_t BC3_B_ALL = 7ull << 54, BC3_WALL_B = 1ull << 54, BC3_INLT_B = 2ull << 54,
               BC3_OUTL_B = 3ull << 54, BC3_CYCL_B = 4ull << 54, BC3_SYMP_B = 5ull << 54,
               BC3_CORNER = 1ull << 57, BC3_FLUID = 1ull << 58;

}  // namespace

extern "C" {

/* Mirrors the reference Arguments fields read by the loop, plus the values
 * Iterate2D/3D derive from the mesh, plus the extensions of this build. */
typedef struct {
    double u, v, w, rho, viscosity, g;
    int inlet_profile;   /* 1 INLET, 2 NO_INLET, 4 pressure inlet (physics) */
    int outlet_profile;  /* 1 OUTLET Zou-He, 2 SECOND, 3 FIRST, 4 HEmodel, 5 pressure (physics) */
    int collision_model; /* 1 BGKW, 2 TRT, 3 MRT */
    int boundary_type;   /* 1 CURVED, 2 STRAIGHT */
    int bc_wall_model;   /* 1 SIMPLE, 2 COMPLEX */
    int update_inlet_outlet;
    int boundary_id;
    double delta, min_inlet_y, max_inlet_y, min_inlet_z, max_inlet_z;
    int mode;            /* 0 reference semantics, 1 physics */
    int init_kind;       /* 0 f=0 (reference), 1 f=feq(rho,u) */
    double rho_in, rho_out;
    int periodic[3];     /* physics mode: axes whose out-of-domain pulls wrap */
    const double *link_q; /* CURVED: wall fraction of every BC link (NULL: all 1/2) */
} orc_params;

}  // extern "C"

namespace {

template <class T>
inline T feqc2(T u, T uc, T v, T vc, T rho, T w) {
    T vec = u * uc + v * vc;
    return rho * w * (1. + 3. * vec + 4.5 * vec * vec - 1.5 * (u * u + v * v));
}
template <class T>
inline T feqc3(T u, T uc, T v, T vc, T w, T wc, T rho, T weight) {
    T vec = u * uc + v * vc + w * wc;
    return rho * weight * (1. + 3. * vec + 4.5 * vec * vec - 1.5 * (u * u + v * v + w * w));
}

template <class T>
struct Lattice {
    int dims = 2, q = 9, n = 0, m = 0, h = 1, N = 0;
    orc_params p;
    T omega, omegaA;
    T w[19];
    int off[19]; /* linear pull offsets (c2D_d / c3D_d) */
    std::vector<int> fluid;
    std::vector<T> f, fc, rho, u, v, w3, u0, v0, w0;
    std::vector<uint64_t> mask;    /* reference BC mask per node */
    std::vector<uint8_t> stream;   /* (q-1)*N, 1 = streamed */
    std::vector<int> bcnodes;      /* collapsed BC node list, ascending */
    std::vector<T> qc;             /* CURVED: collapsed link fractions, (q-1) per BC node */
    T msc[361];                    /* reference M^-1 S, row-major */
    T mm[361];                     /* reference M */

    int X(int i) const { return i % n; }
    int Y(int i) const { return (i / n) % m; }
    int Z(int i) const { return i / (n * m); }

    /* Pull source of population d at node i: the reference adds a linear
     * offset; out-of-domain pulls wrap periodically here (the reference reads a
     * neighbouring row or past the array there, which the generator's
     * boundary links always prevent). */
    int src(int i, int d) const {
        int x = X(i), y = Y(i), z = Z(i);
        int cx = dims == 2 ? cx2[d] : cx3[d], cy = dims == 2 ? cy2[d] : cy3[d];
        int cz = dims == 2 ? 0 : cz3[d];
        x = (x - cx + n) % n;
        y = (y - cy + m) % m;
        z = (z - cz + h) % h;
        return x + n * (y + m * z);
    }
    int opp(int d) const { return dims == 2 ? opp2[d] : opp3[d]; }
};

/* ----------------------------- set-up ----------------------------------- */

template <class T>
void build_tables(Lattice<T> &L) {
    const int n = L.n, m = L.m;
    if (L.dims == 2) {
        const T w2[9] = {4. / 9., 1. / 9., 1. / 9., 1. / 9., 1. / 9., 1. / 36., 1. / 36., 1. / 36., 1. / 36.};
        const int c2[9] = {0, -1, -n, 1, n, -n - 1, -n + 1, n + 1, n - 1};
        for (int d = 0; d < 9; ++d) {
            L.w[d] = w2[d];
            L.off[d] = c2[d];
        }
    } else {
        const T w3[19] = {1. / 3.,  1. / 18., 1. / 18., 1. / 18., 1. / 18., 1. / 18., 1. / 18.,
                          1. / 36., 1. / 36., 1. / 36., 1. / 36., 1. / 36., 1. / 36., 1. / 36.,
                          1. / 36., 1. / 36., 1. / 36., 1. / 36., 1. / 36.};
        const int mn = m * n;
        const int c3[19] = {0,       -1,      1,       -n,      n,       -mn,     mn,
                            -n - 1,  -n + 1,  n - 1,   n + 1,   -mn - 1, -mn + 1, mn - 1,
                            mn + 1,  -mn - n, -mn + n, mn - n,  mn + n};
        for (int d = 0; d < 19; ++d) {
            L.w[d] = w3[d];
            L.off[d] = c3[d];
        }
    }
    /* GpuInit.cu:102-103 / :845-846, evaluated in the storage type. */
    L.omega = (T)(1.0 / (3. * (T)L.p.viscosity + 0.5));
    L.omegaA = (T)(8 * (2 - L.omega) / (8 - L.omega));
    /* MRT: M and M^-1 S with M^-1 = M^T diag(1/|row|^2) (the reference's
     * hard-coded M^-1 equals this exactly, CellFunctions.cu:14-24, :70-90). */
    const int q = L.q;
    const double *M = q == 9 ? M2 : M3;
    double s[19];
    if (q == 9) {
        const double s2[9] = {1.0, 1.4, 1.4, 1.0, 1.2, 1.0, 1.2, (double)L.omega, (double)L.omega};
        for (int k = 0; k < 9; ++k) s[k] = s2[k];
    } else {
        const double om = (double)L.omega;
        const double s3[19] = {0.0, 1.19, 1.4, 0.0, 1.2, 0.0, 1.2, 0.0, 1.2, om,
                               1.4, om,   1.4, om,  om,  om,  1.98, 1.98, 1.98};
        for (int k = 0; k < 19; ++k) s[k] = s3[k];
    }
    for (int k = 0; k < q; ++k) {
        double nrm = 0;
        for (int i = 0; i < q; ++i) nrm += M[k * q + i] * M[k * q + i];
        for (int i = 0; i < q; ++i) {
            L.mm[k * q + i] = (T)M[k * q + i];
            /* (M^-1 S)[i][k] = M[k][i] / |row k|^2 * s_k */
            L.msc[i * q + k] = (T)((T)(M[k * q + i] / nrm) * (T)s[k]);
        }
    }
}

/* initBoundaryConditions2D/3D + collapseBc2D/3D, restated. */
template <class T>
int build_masks(Lattice<T> &L, int nconn, const int *bi, const int *bj, const int *bk,
                const int *bdir, const int *btype, const int *bid) {
    const int N = L.N, q = L.q;
    L.mask.assign(N, 0ull);
    L.stream.assign((size_t)(q - 1) * N, 1);
    std::vector<int> flag(N, 0);
    for (int c = 0; c < nconn; ++c) {
        int ind = bi[c] + bj[c] * L.n + (L.dims == 3 ? bk[c] * L.n * L.m : 0);
        int dir = bdir[c];
        if (ind < 0 || ind >= N || dir < 1 || dir >= q) return ORC_BAD_INPUT;
        uint64_t &mk = L.mask[ind];
        uint64_t type = (uint64_t)btype[c];
        if (L.dims == 2) {
            mk |= bc2_mask(type, dir);
            mk |= (uint64_t)L.fluid[ind] << 19;
            if (!(mk & BC2_B_ALL)) {
                mk |= type << 16;
            } else if ((mk & BC2_B_ALL) != (type << 16)) {
                mk &= ~BC2_B_ALL;
                mk |= BC2_WALL_B;
                mk |= BC2_CORNER;
            }
            /* BOUND_ID(id) = id << 24 on a 32-bit int mask (BcMacros.h:74) */
            uint32_t m32 = (uint32_t)mk | ((uint32_t)bid[c] << 24);
            mk = m32;
        } else {
            mk |= bc3_mask(type, dir);
            mk |= (uint64_t)L.fluid[ind] << 58;
            if (!(mk & BC3_B_ALL)) {
                mk |= type << 54;
            } else if ((mk & BC3_B_ALL) != (type << 54)) {
                mk &= ~BC3_B_ALL;
                mk |= BC3_WALL_B;
                mk |= BC3_CORNER;
            }
        }
        L.stream[(size_t)(L.opp(dir) - 1) * N + ind] = 0; /* no stream opposite the BC link */
        flag[ind] = 1;
    }
    for (int c = 0; c < nconn; ++c) {
        int ind = bi[c] + bj[c] * L.n + (L.dims == 3 ? bk[c] * L.n * L.m : 0);
        uint64_t &mk = L.mask[ind];
        if (L.dims == 2) {
            if (mk & BC2_CORNER) {
                auto any = [&](int d) { return (mk & bc2_mask(3, d)) != 0; };
                if (any(1) && any(2)) { mk &= ~bc2_mask(3, 5); mk |= bc2_mask(1, 5); }
                if (any(3) && any(2)) { mk &= ~bc2_mask(3, 6); mk |= bc2_mask(1, 6); }
                if (any(3) && any(4)) { mk &= ~bc2_mask(3, 7); mk |= bc2_mask(1, 7); }
                if (any(1) && any(4)) { mk &= ~bc2_mask(3, 8); mk |= bc2_mask(1, 8); }
            }
        } else if (mk & BC3_CORNER) {
            /* every typed link of a mixed-type node becomes a wall link */
            for (int d = 1; d < 19; ++d)
                if (mk & bc3_mask(7, d)) {
                    mk &= ~bc3_mask(7, d);
                    mk |= bc3_mask(1, d);
                }
        }
    }
    L.bcnodes.clear();
    for (int i = 0; i < N; ++i)
        if (flag[i]) L.bcnodes.push_back(i);
    return ORC_OK;
}

/* ----------------------------- collision -------------------------------- */

template <class T>
void collide_node(Lattice<T> &L, int i) {
    const int N = L.N;
    const T om = L.omega;
    T *f = L.f.data();
    T *fc = L.fc.data();
    const T r = L.rho[i], u = L.u[i], v = L.v[i];
    const bool phys = L.p.mode == 1;
    if (L.dims == 2) {
        switch (L.p.collision_model) {
        case 1:
            for (int d = 0; d < 9; ++d)
                fc[i + d * N] = om * feqc2<T>(u, (T)cx2[d], v, (T)cy2[d], r, L.w[d]) + (1.0 - om) * f[i + d * N];
            break;
        case 2: {
            T feq[9], fl[9];
            for (int d = 0; d < 9; ++d) {
                feq[d] = feqc2<T>(u, (T)cx2[d], v, (T)cy2[d], r, L.w[d]);
                fl[d] = f[i + d * N];
            }
            for (int d = 0; d < 9; ++d) {
                int o = opp2[d];
                fc[i + d * N] = fl[d] - 0.5 * om * (fl[d] + fl[o] - feq[d] - feq[o]) -
                                0.5 * L.omegaA * (fl[d] - fl[o] - feq[d] + feq[o]);
            }
            break;
        }
        case 3: {
            T meq[9], mo[9], col[9], fl[9];
            meq[0] = r;
            if (!phys) {
                meq[1] = r * (-2. + 3. * r * (u * u + v * v));
                meq[2] = r * (1. - 3. * r * (u * u + v * v));
            } else { /* e_eq = -2 rho + 3 |j|^2 / rho, eps_eq = rho - 3 |j|^2 / rho */
                meq[1] = r * (-2. + 3. * (u * u + v * v));
                meq[2] = r * (1. - 3. * (u * u + v * v));
            }
            meq[3] = r * u;
            meq[4] = -r * u;
            meq[5] = r * v;
            meq[6] = -r * v;
            meq[7] = r * (u * u - v * v);
            meq[8] = r * u * v;
            for (int d = 0; d < 9; ++d) fl[d] = f[i + d * N];
            for (int a = 0; a < 9; ++a) {
                mo[a] = 0;
                for (int b = 0; b < 9; ++b) mo[a] += L.mm[a * 9 + b] * fl[b];
            }
            for (int a = 0; a < 9; ++a) {
                col[a] = 0;
                for (int b = 0; b < 9; ++b) col[a] += L.msc[a * 9 + b] * (mo[b] - meq[b]);
            }
            for (int d = 0; d < 9; ++d) fc[i + d * N] = fl[d] - col[d];
            break;
        }
        }
        return;
    }
    const T w = L.w3[i];
    switch (L.p.collision_model) {
    case 1:
        for (int d = 0; d < 19; ++d)
            fc[i + d * N] = om * feqc3<T>(u, (T)cx3[d], v, (T)cy3[d], w, (T)cz3[d], r, L.w[d]) + (1.0 - om) * f[i + d * N];
        break;
    case 2: { /* physics mode only: the reference has no 3D TRT */
        T feq[19], fl[19];
        for (int d = 0; d < 19; ++d) {
            feq[d] = feqc3<T>(u, (T)cx3[d], v, (T)cy3[d], w, (T)cz3[d], r, L.w[d]);
            fl[d] = f[i + d * N];
        }
        for (int d = 0; d < 19; ++d) {
            int o = opp3[d];
            fc[i + d * N] = fl[d] - 0.5 * om * (fl[d] + fl[o] - feq[d] - feq[o]) -
                            0.5 * L.omegaA * (fl[d] - fl[o] - feq[d] + feq[o]);
        }
        break;
    }
    case 3: {
        T meq[19], mo[19], col[19], fl[19];
        T jx = r * u, jy = r * v, jz = r * w;
        T wej = -475. / 63.;
        meq[0] = r;
        meq[1] = -11. * r + 19. * (jx * jx + jy * jy + jz * jz);
        meq[2] = wej * (jx * jx + jy * jy + jz * jz);
        meq[3] = jx;
        meq[4] = -(2. / 3.) * jx;
        meq[5] = jy;
        meq[6] = -(2. / 3.) * jy;
        meq[7] = jz;
        meq[8] = -(2. / 3.) * jz;
        meq[9] = (2 * jx * jx - (jy * jy + jz * jz));
        meq[10] = 0.0;
        meq[11] = jy * jy - jz * jz;
        meq[12] = 0.0;
        meq[13] = jx * jy;
        meq[14] = jy * jz;
        meq[15] = jx * jz;
        meq[16] = 0.0;
        meq[17] = 0.0;
        meq[18] = 0.0;
        for (int d = 0; d < 19; ++d) fl[d] = f[i + d * N];
        for (int a = 0; a < 19; ++a) {
            mo[a] = 0.;
            for (int b = 0; b < 19; ++b) mo[a] += L.mm[a * 19 + b] * fl[b];
        }
        for (int a = 0; a < 19; ++a) {
            col[a] = 0.;
            for (int b = 0; b < 19; ++b) col[a] += L.msc[a * 19 + b] * (mo[b] - meq[b]);
        }
        /* the reference never writes direction 18 (GpuCollision.cu:1161) */
        int last = phys ? 19 : 18;
        for (int d = 0; d < last; ++d) fc[i + d * N] = fl[d] - col[d];
        break;
    }
    }
}

template <class T>
void collide_all(Lattice<T> &L) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < L.N; ++i)
        if (L.fluid[i] == 1) collide_node(L, i);
}

/* ------------------------------ streaming -------------------------------- */

template <class T>
void stream_all(Lattice<T> &L) {
    const int N = L.N, q = L.q;
    const bool phys = L.p.mode == 1;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < N; ++i) {
        if (L.fluid[i] != 1) continue;
        L.f[i] = L.fc[i];
        for (int d = 1; d < q; ++d) {
            bool st = L.stream[(size_t)(d - 1) * N + i] != 0;
            int s = L.src(i, d);
            if (phys) {
                /* physics: a link is a wall link when the reference's stream
                 * flag is cleared by a non-periodic BC link, or when x - c_d is
                 * solid or outside a non-periodic domain */
                const int od = L.opp(d);
                const int b = L.dims == 2 ? 2 : 3;
                const uint64_t lt = (L.mask[i] >> ((od - 1) * b)) & (L.dims == 2 ? 3ull : 7ull);
                const bool periodic_link = !st && lt == 4;
                if (periodic_link) st = true;
                const int cx = L.dims == 2 ? cx2[d] : cx3[d], cy = L.dims == 2 ? cy2[d] : cy3[d];
                const int cz = L.dims == 2 ? 0 : cz3[d];
                const int sx = L.X(i) - cx, sy = L.Y(i) - cy, sz = L.Z(i) - cz;
                if (!periodic_link && ((!L.p.periodic[0] && (sx < 0 || sx >= L.n)) ||
                                       (!L.p.periodic[1] && (sy < 0 || sy >= L.m)) ||
                                       (!L.p.periodic[2] && (sz < 0 || sz >= L.h))))
                    st = false;
                if (st && L.fluid[s] != 1) st = false;
            }
            if (st)
                L.f[i + (size_t)d * N] = L.fc[s + (size_t)d * N];
            else if (phys) /* half-way bounce-back of the node's own outgoing population */
                L.f[i + (size_t)d * N] = L.fc[i + (size_t)L.opp(d) * N];
            else
                L.f[i + (size_t)d * N] = L.fc[i + (size_t)d * N];
        }
    }
}

/* --------------------------- 2D boundaries ------------------------------- */

/* Curved wall (CURVED branch of gpuBcWall2D / gpuBcSimpleWall3D,
 * GpuBoundaries.cu:414-432, :461-479): the population entering against wall
 * link dir of BC node number b, from this step's post-collision values.  The
 * first coefficient of the q < 1/2 branch reads entry b*(q-1)+dir of the
 * collapsed table, one past the link's own, and the upstream value sits at
 * the flat index i + dir*N + c(dir) of the SoA array (a neighbouring row, or
 * another direction's array, where the neighbour is outside the lattice);
 * past either end of the array the reference's read is undefined, 0 here. */
template <class T>
T curved_value(const Lattice<T> &L, int b, int i, int dir) {
    const size_t N = (size_t)L.N;
    const int D = L.q - 1;
    const T *fc = L.fc.data();
    const T q0 = L.qc[(size_t)b * D + dir - 1];
    if (q0 < 0.5) {
        const long long up = (long long)i + (long long)dir * (long long)N + L.off[dir];
        const T fu = up >= 0 && up < (long long)L.fc.size() ? fc[up] : (T)0;
        return 2 * L.qc[(size_t)b * D + dir] * fc[i + dir * N] + (1 - 2 * q0) * fu;
    }
    return fc[i + dir * N] / 2 / q0 + (2 * q0 - 1) / (2 * q0) * fc[i + (size_t)L.opp(dir) * N];
}

template <class T>
void bc_node_2d(Lattice<T> &L, int b, int i, uint64_t mk) {
    const int N = L.N;
    T *f = L.f.data();
    auto F = [&](int d) -> T & { return f[i + (size_t)d * N]; };
    if (!(mk & BC2_FLUID)) return;
    const T u0 = L.u0[i];
    /* inlet (GpuBoundaries.cu:12-71) */
    if (mk & BC2_INLT_B) {
        bool north = (mk & bc2_mask(2, 2)) && !(mk & BC2_CORNER);
        bool west = (mk & bc2_mask(2, 3)) && !(mk & BC2_CORNER);
        if (north) {
            F(4) = F(2);
            F(8) = F(6) + (F(0) + F(1) + F(3) + 2 * (F(2) + F(6) + F(5))) * u0 / 6.0;
            F(7) = F(5) - (F(0) + F(1) + F(3) + 2 * (F(2) + F(6) + F(5))) * u0 / 6.0;
        }
        if (west) {
            F(1) = F(3) + 2. * ((F(0) + F(2) + F(4) + 2. * (F(3) + F(6) + F(7))) / (1.0 - u0)) * u0 / 3;
            F(5) = F(7) + ((F(0) + F(2) + F(4) + 2. * (F(3) + F(6) + F(7))) / (1.0 - u0)) * u0 / 6;
            F(8) = F(6) + ((F(0) + F(2) + F(4) + 2. * (F(3) + F(6) + F(7))) / (1.0 - u0)) * u0 / 6;
        }
    }
    /* straight wall (GpuBoundaries.cu:400-443): f[opp(dir)] = f[dir] after
     * streaming, in direction order */
    for (int dir = 1; dir < 9; ++dir) {
        uint64_t all = mk & bc2_mask(3, dir), wall = mk & bc2_mask(1, dir);
        if (all == wall && wall) F(opp2[dir]) = L.p.boundary_type == 1 ? curved_value(L, b, i, dir) : F(dir);
    }
    /* east outlet (GpuBoundaries.cu:1562-1653) */
    if ((mk & bc2_mask(3, 1)) == bc2_mask(3, 1)) {
        switch (L.p.outlet_profile) {
        case 1:
            F(3) = F(1) - 2 * ((F(0) + F(2) + F(4) + 2 * (F(1) + F(5) + F(8))) / (1 - u0)) * u0 / 3;
            F(7) = F(5) - ((F(0) + F(2) + F(4) + 2 * (F(1) + F(5) + F(8))) / (1 - u0)) * u0 / 6;
            F(6) = F(8) - ((F(0) + F(2) + F(4) + 2 * (F(1) + F(5) + F(8))) / (1 - u0)) * u0 / 6;
            break;
        case 2:
            F(1) = 2 * f[i + N - 1] - f[i + N - 2];
            F(5) = 2 * f[i + 5 * N - 1] - f[i + 5 * N - 2];
            F(8) = 2 * f[i + 8 * N - 1] - f[i + 8 * N - 2];
            break;
        case 3:
            F(1) = f[i - 1 + N];
            F(5) = f[i - 1 + 5 * N];
            F(8) = f[i - 1 + 8 * N];
            break;
        }
    }
}

/* --------------------------- 3D boundaries ------------------------------- */

/* Zou-He velocity face of the reference (Hecht-Harting transverse
 * corrections, GpuBoundaries.cu:92-394), face order W,E,S,N,B,T.  The
 * reference's west and east densities divide by (1+u) and (1-u), the reverse
 * of the mass balance rho (1 -/+ u) = known sums that its other four faces
 * use; physics mode uses zou_he_face instead. */
template <class T>
void zou_he_3d(T *f, size_t N, int i, int face, T uu, T vv, T ww) {
    auto F = [&](int d) -> T & { return f[i + (size_t)d * N]; };
    T d_, n1, n2;
    switch (face) {
    case 2: /* WEST */
        d_ = 1.0 / (1.0 + uu) * (F(0) + F(3) + F(4) + F(5) + F(6) + F(15) + F(16) + F(17) + F(18) + 2.0 * (F(2) + F(8) + F(10) + F(12) + F(14)));
        n1 = 0.5 * (F(3) + F(15) + F(17) - (F(4) + F(16) + F(18))) - 1.0 / 3.0 * d_ * vv;
        n2 = 0.5 * (F(5) + F(15) + F(16) - (F(6) + F(17) + F(18))) - 1.0 / 3.0 * d_ * ww;
        F(1) = F(2) + 1.0 / 3.0 * d_ * uu;
        F(7) = F(10) + 1.0 / 6.0 * d_ * (uu + vv) - n1;
        F(9) = F(8) + 1.0 / 6.0 * d_ * (uu - vv) + n1;
        F(11) = F(14) + 1.0 / 6.0 * d_ * (uu + ww) - n2;
        F(13) = F(12) + 1.0 / 6.0 * d_ * (uu - ww) + n2;
        break;
    case 1: /* EAST */
        d_ = 1.0 / (1.0 - uu) * (F(0) + F(3) + F(4) + F(5) + F(6) + F(15) + F(16) + F(17) + F(18) + 2.0 * (F(1) + F(7) + F(9) + F(11) + F(13)));
        n1 = 0.5 * (F(3) + F(15) + F(17) - (F(4) + F(16) + F(18))) - 1.0 / 3.0 * d_ * vv;
        n2 = 0.5 * (F(5) + F(15) + F(16) - (F(6) + F(17) + F(18))) - 1.0 / 3.0 * d_ * ww;
        F(2) = F(1) - 1.0 / 3.0 * d_ * uu;
        F(8) = F(9) - 1.0 / 6.0 * d_ * (uu - vv) - n1;
        F(10) = F(7) - 1.0 / 6.0 * d_ * (uu + vv) + n1;
        F(12) = F(13) - 1.0 / 6.0 * d_ * (uu - ww) - n2;
        F(14) = F(11) - 1.0 / 6.0 * d_ * (uu + ww) + n2;
        break;
    case 4: /* SOUTH */
        d_ = 1.0 / (1.0 - vv) * (F(0) + F(1) + F(2) + F(5) + F(6) + F(11) + F(12) + F(13) + F(14) + 2.0 * (F(4) + F(9) + F(10) + F(16) + F(18)));
        n1 = 0.5 * (F(1) + F(11) + F(13) - (F(2) + F(12) + F(14))) - 1.0 / 3.0 * d_ * uu;
        n2 = 0.5 * (F(5) + F(11) + F(12) - (F(6) + F(13) + F(14))) - 1.0 / 3.0 * d_ * ww;
        F(3) = F(4) + 1.0 / 3.0 * d_ * vv;
        F(7) = F(10) + 1.0 / 6.0 * d_ * (vv + uu) - n1;
        F(8) = F(9) + 1.0 / 6.0 * d_ * (vv - uu) + n1;
        F(15) = F(18) + 1.0 / 6.0 * d_ * (vv + ww) - n2;
        F(17) = F(16) + 1.0 / 6.0 * d_ * (vv - ww) + n2;
        break;
    case 3: /* NORTH */
        d_ = 1.0 / (1.0 + vv) * (F(0) + F(1) + F(2) + F(5) + F(6) + F(11) + F(12) + F(13) + F(14) + 2.0 * (F(3) + F(7) + F(8) + F(15) + F(17)));
        n1 = 0.5 * (F(1) + F(11) + F(13) - (F(2) + F(12) + F(14))) - 1.0 / 3.0 * d_ * uu;
        n2 = 0.5 * (F(5) + F(11) + F(12) - (F(6) + F(13) + F(14))) - 1.0 / 3.0 * d_ * ww;
        F(4) = F(3) - 1.0 / 3.0 * d_ * vv;
        F(9) = F(8) - 1.0 / 6.0 * d_ * (vv - uu) - n1;
        F(10) = F(7) - 1.0 / 6.0 * d_ * (vv + uu) + n1;
        F(16) = F(17) - 1.0 / 6.0 * d_ * (vv - ww) - n2;
        F(18) = F(15) - 1.0 / 6.0 * d_ * (vv + ww) + n2;
        break;
    case 6: /* BOTTOM */
        d_ = 1.0 / (1.0 - ww) * (F(0) + F(1) + F(2) + F(3) + F(4) + F(7) + F(8) + F(9) + F(10) + 2.0 * (F(6) + F(13) + F(14) + F(17) + F(18)));
        n1 = 0.5 * (F(1) + F(7) + F(9) - (F(2) + F(8) + F(10))) - 1.0 / 3.0 * d_ * uu;
        n2 = 0.5 * (F(3) + F(7) + F(8) - (F(4) + F(9) + F(10))) - 1.0 / 3.0 * d_ * vv;
        F(5) = F(6) + 1.0 / 3.0 * d_ * ww;
        F(11) = F(14) + 1.0 / 6.0 * d_ * (ww + uu) - n1;
        F(12) = F(13) + 1.0 / 6.0 * d_ * (ww - uu) + n1;
        F(15) = F(18) + 1.0 / 6.0 * d_ * (ww + vv) - n2;
        F(16) = F(17) + 1.0 / 6.0 * d_ * (ww - vv) + n2;
        break;
    case 5: /* TOP */
        d_ = (1.0 / (1.0 + ww)) * (F(0) + F(1) + F(2) + F(3) + F(4) + F(7) + F(8) + F(9) + F(10) + 2.0 * (F(5) + F(11) + F(12) + F(15) + F(16)));
        n1 = 0.5 * (F(1) + F(7) + F(9) - (F(2) + F(8) + F(10))) - 1.0 / 3.0 * d_ * uu;
        n2 = 0.5 * (F(3) + F(7) + F(8) - (F(4) + F(9) + F(10))) - 1.0 / 3.0 * d_ * vv;
        F(6) = F(5) - 1.0 / 3.0 * d_ * ww;
        F(13) = F(12) - 1.0 / 6.0 * d_ * (ww - uu) - n1;
        F(14) = F(11) - 1.0 / 6.0 * d_ * (ww + uu) + n1;
        F(17) = F(16) - 1.0 / 6.0 * d_ * (ww - vv) - n2;
        F(18) = F(15) - 1.0 / 6.0 * d_ * (ww + vv) + n2;
        break;
    }
}

template <class T>
void bc_node_3d(Lattice<T> &L, int b, int i, uint64_t mk) {
    const size_t N = (size_t)L.N;
    T *f = L.f.data();
    if (!(mk & BC3_FLUID)) return;
    const T uu = L.u0[i], vv = L.v0[i], ww = L.w0[i];
    /* inlet (GpuBoundaries.cu:73-399) */
    if (mk & BC3_INLT_B) {
        const int faces[6] = {2, 1, 4, 3, 6, 5};
        for (int k = 0; k < 6; ++k) {
            int face = faces[k];
            uint64_t inl = bc3_mask(2, face), all = mk & bc3_mask(7, face);
            bool hit = (mk & inl) && !(mk & BC3_CORNER) &&
                       (face == 1 ? all == inl : all == (mk & inl));
            if (hit) zou_he_3d(f, N, i, face, uu, vv, ww);
        }
    }
    if (L.p.bc_wall_model == 2) return; /* HH wall: complex_wall_node_3d */
    /* straight simple wall (GpuBoundaries.cu:445-490) */
    for (int dir = 1; dir < 19; ++dir) {
        uint64_t all = mk & bc3_mask(7, dir), wall = mk & bc3_mask(1, dir);
        if (all == wall && wall)
            f[i + (size_t)opp3[dir] * N] = L.p.boundary_type == 1 ? curved_value(L, b, i, dir) : f[i + (size_t)dir * N];
    }
}

/* D3Q19 direction of s1 unit(a1) + s2 unit(a2) in the reference ordering. */
int dir3_of(int a1, int s1, int a2 = 0, int s2 = 0) {
    const int v[3] = {(a1 == 0 ? s1 : 0) + (a2 == 0 ? s2 : 0), (a1 == 1 ? s1 : 0) + (a2 == 1 ? s2 : 0),
                      (a1 == 2 ? s1 : 0) + (a2 == 2 ? s2 : 0)};
    for (int d = 0; d < 19; ++d)
        if (cx3[d] == v[0] && cy3[d] == v[1] && cz3[d] == v[2]) return d;
    return -1;
}
int comp3(int a, int d) { return a == 0 ? cx3[d] : (a == 1 ? cy3[d] : cz3[d]); }

/* HH ("complex") wall, gpuBcComplexWall3D (GpuBoundaries.cu:492-1560), wall
 * at rest.  FP32 evaluation follows the reference's: sums in FLOAT_TYPE,
 * products with double constants in double and rounded on assignment; the
 * zero wall-velocity terms of the face formulas add exact zeros and are left
 * out.  Runs for every node of the boundary list, as the kernel does (its edge
 * and corner branches do not test the fluid bit). */
template <class T>
void complex_wall_node_3d(Lattice<T> &L, int i, uint64_t mk) {
    const size_t N = (size_t)L.N;
    T *f = L.f.data();
    auto F = [&](int d) -> T & { return f[i + (size_t)d * N]; };
    int walls = 0;
    for (int d = 1; d < 19; ++d)
        if ((mk & bc3_mask(7, d)) == (mk & bc3_mask(1, d)) && (mk & bc3_mask(1, d))) ++walls;
    /* normal search (:513-556): slot j takes the first direction 1..6 with a
     * wall bit whose axis is still free; direction c gives normal -c */
    int slot[3] = {-1, -1, -1}, sgn[3] = {0, 0, 0};
    for (int j = 0; j < 3; ++j)
        for (int d = 1; d <= 6; ++d) {
            const int a = (d - 1) / 2;
            if ((mk & bc3_mask(1, d)) && slot[a] < 0) {
                slot[a] = j;
                sgn[a] = (d % 2) ? -1 : 1;
                break;
            }
        }
    if (walls == 5 && (mk & BC3_FLUID) && (mk & BC3_WALL_B)) {
        const int order[6] = {2, 1, 4, 3, 6, 5};
        for (int k = 0; k < 6; ++k) {
            const int dw = order[k];
            const uint64_t wb = mk & bc3_mask(1, dw);
            if (!(wb && (mk & bc3_mask(7, dw)) == wb)) continue;
            const int A = (dw - 1) / 2, S = (dw % 2) ? -1 : 1;  /* inward normal */
            int tang[2], nt = 0;
            for (int a = 0; a < 3; ++a)
                if (a != A) tang[nt++] = a;
            T N2[2];
            for (int t = 0; t < 2; ++t) {
                T ps = 0, ms = 0;
                bool pf = true, mf = true;
                for (int d = 1; d < 19; ++d) {
                    if (comp3(A, d) != 0) continue;
                    if (comp3(tang[t], d) == 1) { ps = pf ? F(d) : (T)(ps + F(d)); pf = false; }
                    if (comp3(tang[t], d) == -1) { ms = mf ? F(d) : (T)(ms + F(d)); mf = false; }
                }
                N2[t] = (T)(0.5 * (double)(T)(ps - ms));
            }
            F(dir3_of(A, S)) = F(dir3_of(A, -S));
            for (int t = 0; t < 2; ++t) {
                F(dir3_of(A, S, tang[t], 1)) = (T)((double)F(dir3_of(A, -S, tang[t], -1)) - (double)N2[t]);
                F(dir3_of(A, S, tang[t], -1)) = (T)((double)F(dir3_of(A, -S, tang[t], 1)) + (double)N2[t]);
            }
        }
    }
    if (walls == 9) {
        int a1 = -1, a2 = -1;
        if (slot[0] == 0 && slot[2] == 1) { a1 = 0; a2 = 2; }
        if (slot[1] == 0 && slot[2] == 1) { a1 = 1; a2 = 2; }
        if (slot[0] == 0 && slot[1] == 1) { a1 = 0; a2 = 1; }
        if (a1 >= 0) {
            const int s1 = sgn[a1], s2 = sgn[a2], t = 3 - a1 - a2;
            const T ntv = (T)(-0.25 * (double)(T)(F(dir3_of(t, 1)) - F(dir3_of(t, -1))));
            F(dir3_of(a1, s1)) = F(dir3_of(a1, -s1));
            F(dir3_of(a2, s2)) = F(dir3_of(a2, -s2));
            F(dir3_of(a1, s1, a2, s2)) = F(dir3_of(a1, -s1, a2, -s2));
            F(dir3_of(a1, s1, t, 1)) = (T)(F(dir3_of(a1, -s1, t, -1)) + ntv);
            F(dir3_of(a1, s1, t, -1)) = (T)(F(dir3_of(a1, -s1, t, 1)) - ntv);
            F(dir3_of(a2, s2, t, 1)) = (T)(F(dir3_of(a2, -s2, t, -1)) + ntv);
            F(dir3_of(a2, s2, t, -1)) = (T)(F(dir3_of(a2, -s2, t, 1)) - ntv);
            const int b1 = dir3_of(a1, s1, a2, -s2), b2 = dir3_of(a1, -s1, a2, s2);
            T sum = 0;
            bool first = true;
            for (int d = 1; d < 19; ++d) {
                if (d == b1 || d == b2) continue;
                sum = first ? F(d) : (T)(sum + F(d));
                first = false;
            }
            const int lo = b1 < b2 ? b1 : b2, hi = b1 < b2 ? b2 : b1;
            F(lo) = (T)((1. / 22.) * (double)sum);
            F(hi) = (T)((1. / 22.) * (double)sum);
            F(0) = (T)((12. / 22.) * (double)sum);
        }
    }
    if (walls == 12 && slot[0] == 0 && slot[1] == 1 && slot[2] == 2) {
        const int sx = sgn[0], sy = sgn[1], sz = sgn[2];
        F(dir3_of(0, sx)) = F(dir3_of(0, -sx));
        F(dir3_of(1, sy)) = F(dir3_of(1, -sy));
        F(dir3_of(2, sz)) = F(dir3_of(2, -sz));
        F(dir3_of(0, sx, 1, sy)) = F(dir3_of(0, -sx, 1, -sy));
        F(dir3_of(0, sx, 2, sz)) = F(dir3_of(0, -sx, 2, -sz));
        F(dir3_of(1, sy, 2, sz)) = F(dir3_of(1, -sy, 2, -sz));
        const int b[6] = {dir3_of(0, sx, 1, -sy), dir3_of(0, -sx, 1, sy), dir3_of(0, sx, 2, -sz),
                          dir3_of(0, -sx, 2, sz), dir3_of(1, sy, 2, -sz), dir3_of(1, -sy, 2, sz)};
        auto buried = [&](int d) {
            for (int k = 0; k < 6; ++k)
                if (b[k] == d) return true;
            return false;
        };
        T sum = 0;
        bool first = true;
        for (int d = 1; d < 19; ++d) {
            if (buried(d)) continue;
            sum = first ? F(d) : (T)(sum + F(d));
            first = false;
        }
        const T c = (T)((1. / 18.) * (double)sum);
        for (int d = 1; d < 19; ++d)
            if (buried(d)) F(d) = c;
        F(0) = (T)(12. * (double)c);
    }
}

/* 3D periodic copy from the opposite face (GpuBoundaries.cu:2025-2084) and
 * mirror symmetry (:2086-2168), reference mode.  The copies read every
 * partner's populations as they were before any periodic copy (`snap`): the
 * reference runs them as concurrent GPU threads, which agree with this where
 * a partner does not copy the same directions itself (one periodic axis) and
 * race where two periodic faces meet. */
template <class T>
void periodic_node_3d(Lattice<T> &L, const std::vector<T> &snap, int i, uint64_t mk) {
    const size_t N = (size_t)L.N;
    T *f = L.f.data();
    if (!(mk & BC3_FLUID) || !(mk & BC3_CYCL_B)) return;
    const int ox = L.n - 1, oy = L.n * (L.m - 1), oz = L.n * L.m * (L.h - 1);
    auto cp = [&](const int *ds, int off) {
        const long long pn = (long long)i + off;
        if (pn < 0 || pn >= (long long)N) return;
        for (int k = 0; k < 5; ++k) f[i + (size_t)ds[k] * N] = snap[(size_t)pn + (size_t)ds[k] * N];
    };
    const int dW[5] = {1, 7, 9, 11, 13}, dE[5] = {2, 8, 10, 12, 14}, dS[5] = {3, 7, 8, 15, 17},
              dN[5] = {4, 9, 10, 16, 18}, dB[5] = {5, 11, 12, 15, 16}, dT[5] = {6, 13, 14, 17, 18};
    if (mk & bc3_mask(4, 2)) cp(dW, ox);
    if (mk & bc3_mask(4, 1)) cp(dE, -ox);
    if (mk & bc3_mask(4, 4)) cp(dS, oy);
    if (mk & bc3_mask(4, 3)) cp(dN, -oy);
    if (mk & bc3_mask(4, 6)) cp(dB, oz);
    if (mk & bc3_mask(4, 5)) cp(dT, -oz);
}

template <class T>
void symm_node_3d(Lattice<T> &L, int i, uint64_t mk) {
    const size_t N = (size_t)L.N;
    T *f = L.f.data();
    if (!(mk & BC3_FLUID) || !(mk & BC3_SYMP_B)) return;
    auto F = [&](int d) -> T & { return f[i + (size_t)d * N]; };
    auto is = [&](int dir) {
        return (mk & bc3_mask(5, dir)) && (mk & bc3_mask(7, dir)) == bc3_mask(5, dir);
    };
    if (is(2)) { F(1) = F(2); F(7) = F(8); F(9) = F(10); F(11) = F(12); F(13) = F(14); }
    if (is(1)) { F(2) = F(1); F(8) = F(7); F(10) = F(9); F(12) = F(11); F(14) = F(13); }
    if (is(4)) { F(3) = F(4); F(7) = F(9); F(8) = F(10); F(15) = F(16); F(17) = F(18); }
    if (is(3)) { F(4) = F(3); F(9) = F(7); F(10) = F(8); F(16) = F(15); F(18) = F(17); }
    if (is(6)) { F(5) = F(6); F(11) = F(13); F(12) = F(14); F(15) = F(17); F(16) = F(18); }
    if (is(5)) { F(6) = F(5); F(13) = F(11); F(14) = F(12); F(17) = F(15); F(18) = F(16); }
}


/* Physics mode: mass-balanced Zou-He face with Hecht-Harting transverse
 * terms for any lattice face.  face = inward normal: 0 +x (west), 1 -x (east),
 * 2 +y (south), 3 -y (north), 4 +z (bottom), 5 -z (top).  With e the inward
 * normal: rho (1 - u.e) = S0 + 2 S- over the c.e = 0 and c.e = -1 populations;
 * the c.e = +1 unknowns are f_opp + rho (c.u)/3 (axis, D3Q19) or 2 rho (c.u)/3
 * (axis, D2Q9), and f_opp + rho (u.e)/6 + rho (u.t)/2 - (1/2) sum_{c.e=0}
 * (c.t) f_c for a diagonal c = e + t. */
template <class T>
void zou_he_face(Lattice<T> &L, int i, int face, bool pressure, T rho_set, T ux, T uy, T uz) {
    const size_t N = (size_t)L.N;
    T *f = L.f.data();
    const int q = L.q;
    const int *cx = q == 9 ? cx2 : cx3, *cy = q == 9 ? cy2 : cy3;
    static const int zero9[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    const int *cz = q == 9 ? zero9 : cz3;
    int e[3] = {0, 0, 0};
    e[face / 2] = (face % 2 == 0) ? 1 : -1;
    T s0 = 0, sm = 0;
    for (int d = 0; d < q; ++d) {
        const int ce = cx[d] * e[0] + cy[d] * e[1] + cz[d] * e[2];
        if (ce == 0) s0 += f[i + d * N];
        else if (ce == -1) sm += f[i + d * N];
    }
    T rho, un;
    T u[3] = {ux, uy, uz};
    if (pressure) {
        rho = rho_set;
        un = 1 - (s0 + 2 * sm) / rho;
        for (int a = 0; a < 3; ++a) u[a] = un * e[a];
    } else {
        un = u[0] * e[0] + u[1] * e[1] + u[2] * e[2];
        rho = (s0 + 2 * sm) / (1 - un);
    }
    for (int d = 1; d < q; ++d) {
        const int ce = cx[d] * e[0] + cy[d] * e[1] + cz[d] * e[2];
        if (ce != 1) continue;
        const int t[3] = {cx[d] - e[0], cy[d] - e[1], cz[d] - e[2]};
        const int o = L.opp(d);
        if (!t[0] && !t[1] && !t[2]) {
            f[i + d * N] = f[i + o * N] + (T)(q == 9 ? 2.0 / 3.0 : 1.0 / 3.0) * rho * un;
            continue;
        }
        T st = 0;
        for (int c = 0; c < q; ++c) {
            const int cce = cx[c] * e[0] + cy[c] * e[1] + cz[c] * e[2];
            const int ct = cx[c] * t[0] + cy[c] * t[1] + cz[c] * t[2];
            if (cce == 0 && ct) st += (T)ct * f[i + c * N];
        }
        const T ut = u[0] * t[0] + u[1] * t[1] + u[2] * t[2];
        f[i + d * N] = f[i + o * N] + rho * un / 6 + rho * ut / 2 - st / 2;
    }
}

/* Physics-mode boundary node: an inlet or outlet node (not a corner) gets a
 * Zou-He face normal to its first axis link of the node's type. */
template <class T>
int phys_face_kind(const Lattice<T> &L, uint64_t mk, int &face, bool &pressure, bool &outlet) {
    const int q = L.q;
    const bool d2 = q == 9;
    const uint64_t corner = d2 ? BC2_CORNER : BC3_CORNER;
    if (mk & corner) return 0;
    const uint64_t mt = d2 ? (mk >> 16) & 3ull : (mk >> 54) & 7ull;
    if (mt != 2 && mt != 3) return 0;
    face = -1;
    for (int d = 1; d < q && face < 0; ++d) {
        const uint64_t t = d2 ? (mk >> ((d - 1) * 2)) & 3ull : (mk >> ((d - 1) * 3)) & 7ull;
        if (t != mt) continue;
        const int cxd = d2 ? cx2[d] : cx3[d], cyd = d2 ? cy2[d] : cy3[d], czd = d2 ? 0 : cz3[d];
        if (cxd == -1 && !cyd && !czd) face = 0;
        else if (cxd == 1 && !cyd && !czd) face = 1;
        else if (cyd == -1 && !cxd && !czd) face = 2;
        else if (cyd == 1 && !cxd && !czd) face = 3;
        else if (czd == -1 && !cxd && !cyd) face = 4;
        else if (czd == 1 && !cxd && !cyd) face = 5;
    }
    if (face < 0) return 0;
    outlet = mt == 3;
    if (!outlet) {
        pressure = L.p.inlet_profile == 4;
        /* a velocity face with a tangential velocity is a moving wall */
        const double nrm = face < 2 ? L.p.u : (face < 4 ? L.p.v : (d2 ? 0.0 : L.p.w));
        if (!pressure && nrm == 0.0) return 2;
    } else {
        if (L.p.outlet_profile == 5) pressure = true;
        else if (L.p.outlet_profile == 1) pressure = false;
        else if (L.p.outlet_profile >= 2 && L.p.outlet_profile <= 4) return 3;
        else return -1;
    }
    return 1;
}

/* Physics-mode open outlet (the reference's OUTLET_SECOND, OUTLET_FIRST and
 * OUTLET_HEmodel of gpuBcOutlet2D/3D, GpuBoundaries.cu:1562-1874, on any face,
 * each population addressed at its own node): every population d entering
 * through the face (c_d . e = 1, e the inward normal) becomes
 *   first order   F_d(x + e),
 *   second order  2 F_d(x + e) - F_d(x + 2e),
 *   HEmodel       f_eq,d(rho, u) of the node's macroscopic state of the
 *                 previous step,
 * F the post-stream populations before any boundary condition (snap); a
 * neighbour outside the lattice or not fluid leaves the population as
 * streamed (second order falls back to first order without x + 2e). */
template <class T>
void open_outlet(Lattice<T> &L, const std::vector<T> &snap, int i, int face) {
    const size_t N = (size_t)L.N;
    const int q = L.q;
    const bool d2 = q == 9;
    int e[3] = {0, 0, 0};
    e[face / 2] = (face % 2 == 0) ? 1 : -1;
    const int x = L.X(i), y = L.Y(i), z = L.Z(i);
    auto inside_fluid = [&](int k, int &j) {
        const int yx = x + k * e[0], yy = y + k * e[1], yz = z + k * e[2];
        if (yx < 0 || yx >= L.n || yy < 0 || yy >= L.m || yz < 0 || yz >= L.h) return false;
        j = yx + L.n * (yy + L.m * yz);
        return L.fluid[j] == 1;
    };
    int j1 = -1, j2 = -1;
    const bool ok1 = inside_fluid(1, j1), ok2 = inside_fluid(2, j2);
    for (int d = 1; d < q; ++d) {
        const int cxd = d2 ? cx2[d] : cx3[d], cyd = d2 ? cy2[d] : cy3[d], czd = d2 ? 0 : cz3[d];
        if (cxd * e[0] + cyd * e[1] + czd * e[2] != 1) continue;
        T &fd = L.f[i + d * N];
        if (L.p.outlet_profile == 4) {
            fd = d2 ? feqc2<T>(L.u[i], (T)cxd, L.v[i], (T)cyd, L.rho[i], L.w[d])
                    : feqc3<T>(L.u[i], (T)cxd, L.v[i], (T)cyd, L.w3[i], (T)czd, L.rho[i], L.w[d]);
            continue;
        }
        if (!ok1) continue;
        const T f1 = snap[j1 + d * N];
        if (L.p.outlet_profile == 3 || !ok2) fd = f1;
        else fd = 2 * f1 - snap[j2 + d * N];
    }
}

/* Moving wall (Ladd): after half-way bounce-back each incoming population d of
 * an inlet link gains 6 w_d rho_0 (c_d . u_w), rho_0 the initial density
 * parameter; for a tangential wall velocity the gains cancel pairwise.  (The
 * node's own density in place of rho_0 feeds back on itself: a 24^2 cavity at
 * u = 0.1 blows up after about 70,000 steps.) */
template <class T>
void moving_wall(Lattice<T> &L, int i, uint64_t mk) {
    const int q = L.q;
    const bool d2 = q == 9;
    const size_t N = (size_t)L.N;
    T *f = L.f.data();
    const T rho = (T)L.p.rho;
    const T uw = L.u0[i], vw = L.v0[i], ww = d2 ? (T)0 : L.w0[i];
    for (int dir = 1; dir < q; ++dir) {
        const uint64_t t = d2 ? (mk >> ((dir - 1) * 2)) & 3ull : (mk >> ((dir - 1) * 3)) & 7ull;
        if (t != 2) continue;
        const int d = L.opp(dir);
        const int cxd = d2 ? cx2[d] : cx3[d], cyd = d2 ? cy2[d] : cy3[d], czd = d2 ? 0 : cz3[d];
        const T cu = (T)cxd * uw + (T)cyd * vw + (T)czd * ww;
        f[i + d * N] += (T)(6.0 * L.w[d]) * rho * cu;
    }
}

/* ------------------------------ macro ----------------------------------- */

template <class T>
void macro_all(Lattice<T> &L) {
    const size_t N = (size_t)L.N;
    const T *f = L.f.data();
    const bool phys = L.p.mode == 1;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < L.N; ++i) {
        if (L.fluid[i] != 1) continue;
        auto F = [&](int d) { return f[i + (size_t)d * N]; };
        if (L.dims == 2) {
            T r = F(0) + F(1) + F(2) + F(3) + F(4) + F(5) + F(6) + F(7) + F(8);
            T u = F(1) - F(3) + F(5) - F(6) - F(7) + F(8);
            T v = F(2) - F(4) + F(5) + F(6) - F(7) - F(8);
            L.rho[i] = r;
            L.u[i] = u / r;
            bool eout = (L.mask[i] & bc2_mask(3, 1)) == bc2_mask(3, 1);
            L.v[i] = (!phys && eout) ? (T)0.0 : v / r;
        } else {
            uint64_t mk = L.mask[i];
            bool inl = (mk & BC3_OUTL_B) == BC3_INLT_B;
            if (inl && !L.p.update_inlet_outlet) continue;
            T r = F(0) + F(1) + F(2) + F(3) + F(4) + F(5) + F(6) + F(7) + F(8) + F(9) + F(10) +
                  F(11) + F(12) + F(13) + F(14) + F(15) + F(16) + F(17) + F(18);
            T ru = F(1) - F(2) + F(7) - F(8) + F(9) - F(10) + F(11) - F(12) + F(13) - F(14);
            T rv = F(3) - F(4) + F(7) + F(8) - F(9) - F(10) + F(15) - F(16) + F(17) - F(18);
            T rw = F(5) - F(6) + F(11) + F(12) - F(13) - F(14) + F(15) + F(16) - F(17) - F(18);
            L.rho[i] = r;
            L.u[i] = ru / r + (T)L.p.g / (L.omega);
            L.v[i] = rv / r;
            L.w3[i] = rw / r;
        }
    }
}

template <class T>
double l2_residual(const Lattice<T> &L) {
    double s = 0.0;
    for (size_t k = 0; k < L.f.size(); ++k) {
        double d = (double)L.f[k] - (double)L.fc[k];
        s += d * d;
    }
    return sqrt(s);
}

/* ------------------------------ driver ---------------------------------- */

template <class T>
int run(int dims, int n, int m, int h, const int *node_type, int nconn, const int *bi,
        const int *bj, const int *bk, const int *bdir, const int *btype, const int *bid,
        const orc_params *p, const double *u_init, const double *v_init, const double *w_init,
        const double *rho_init, int steps, int extra_collide, double *out_f, double *out_fc,
        double *out_rho, double *out_u, double *out_v, double *out_w, uint64_t *out_mask,
        uint8_t *out_stream, int *out_count, double *out_resid) {
    if (n < 1 || m < 1 || h < 1 || (dims != 2 && dims != 3)) return ORC_BAD_INPUT;
    if (p->collision_model < 1 || p->collision_model > 3) return ORC_BAD_INPUT;
    if (p->boundary_type == 1 && p->mode == 1) return ORC_UNSUPPORTED;
    if (p->bc_wall_model == 2 && p->mode == 1) return ORC_UNSUPPORTED;
    if (dims == 3 && p->mode == 0 && p->collision_model == 2) return ORC_UNSUPPORTED;
    if (dims == 3 && p->inlet_profile == 1) return ORC_UNSUPPORTED;
    if (dims == 2 && p->inlet_profile == 1) return ORC_UNSUPPORTED;
    if (dims == 3 && p->outlet_profile != 5 && p->mode == 1) {
        /* physics mode supports only pressure outlets in 3D */
    }
    Lattice<T> L;
    L.dims = dims;
    L.q = dims == 2 ? 9 : 19;
    L.n = n;
    L.m = m;
    L.h = dims == 2 ? 1 : h;
    L.N = n * m * L.h;
    L.p = *p;
    const int N = L.N;
    build_tables(L);
    L.fluid.assign(node_type, node_type + N);
    int rc = build_masks(L, nconn, bi, bj, bk, bdir, btype, bid);
    if (rc) return rc;
    if (p->boundary_type == 1 && p->mode == 0) {
        if (dims == 3 && p->bc_wall_model == 2) {
            L.p.boundary_type = 2; /* the HH wall kernel has no curved branch */
        } else {
            /* per-node table filled with 1/2 (Iterate.cu:277, Iterate3D.cu:364),
             * link entries q[ind*(q-1)+dir-1] (GpuInit.cu:1088, :1203-1207),
             * collapsed in BC node order (GpuInit.cu:1125-1155, :1239-1277);
             * one more node's worth of 1/2 stands for what the reference reads
             * past the end of its device array */
            const int D = L.q - 1;
            std::vector<T> qn((size_t)D * N, (T)0.5);
            for (int c = 0; c < nconn; ++c) {
                const int ind = bi[c] + bj[c] * n + (dims == 3 ? bk[c] * n * m : 0);
                qn[(size_t)ind * D + bdir[c] - 1] = p->link_q ? (T)p->link_q[c] : (T)0.5;
            }
            L.qc.assign((L.bcnodes.size() + 1) * (size_t)D, (T)0.5);
            for (size_t b = 0; b < L.bcnodes.size(); ++b)
                for (int j = 0; j < D; ++j) L.qc[b * D + j] = qn[(size_t)L.bcnodes[b] * D + j];
        }
    }
    if (dims == 3 && p->mode == 0) {
        for (int i : L.bcnodes)
            if ((L.mask[i] & BC3_B_ALL) == BC3_OUTL_B) return ORC_UNSUPPORTED;
    }
    if (p->mode == 1) {
        for (int i : L.bcnodes) {
            int face;
            bool pr = false, ou = false;
            if (L.fluid[i] && phys_face_kind(L, L.mask[i], face, pr, ou) < 0) return ORC_UNSUPPORTED;
        }
    }
    L.rho.assign(N, (T)p->rho);
    L.u0.assign(N, (T)p->u);
    L.v0.assign(N, (T)p->v);
    L.w0.assign(N, (T)p->w);
    L.u = L.u0;
    L.v = L.v0;
    L.w3 = L.w0;
    if (u_init) for (int i = 0; i < N; ++i) L.u[i] = (T)u_init[i];
    if (v_init) for (int i = 0; i < N; ++i) L.v[i] = (T)v_init[i];
    if (w_init) for (int i = 0; i < N; ++i) L.w3[i] = (T)w_init[i];
    if (rho_init) for (int i = 0; i < N; ++i) L.rho[i] = (T)rho_init[i];
    L.f.assign((size_t)L.q * N, (T)0);
    L.fc.assign((size_t)L.q * N, (T)0);
    if (p->init_kind == 1) {
        for (int i = 0; i < N; ++i) {
            if (L.fluid[i] != 1) continue;
            for (int d = 0; d < L.q; ++d)
                L.f[i + (size_t)d * N] = dims == 2
                    ? feqc2<T>(L.u[i], (T)cx2[d], L.v[i], (T)cy2[d], L.rho[i], L.w[d])
                    : feqc3<T>(L.u[i], (T)cx3[d], L.v[i], (T)cy3[d], L.w3[i], (T)cz3[d], L.rho[i], L.w[d]);
        }
    }
    for (int it = 0; it < steps; ++it) {
        collide_all(L);
        stream_all(L);
        if (p->mode == 1) {
            const bool open = p->outlet_profile >= 2 && p->outlet_profile <= 4;
            std::vector<T> snap;
            if (open) snap = L.f;
            for (int i : L.bcnodes) {
                int face;
                bool pressure = false, outlet = false;
                if (!L.fluid[i]) continue;
                const int kind = phys_face_kind(L, L.mask[i], face, pressure, outlet);
                if (kind == 2) {
                    moving_wall(L, i, L.mask[i]);
                    continue;
                }
                if (kind == 3) {
                    open_outlet(L, snap, i, face);
                    continue;
                }
                if (kind != 1) continue;
                const T rset = (T)(outlet ? p->rho_out : p->rho_in);
                zou_he_face(L, i, face, pressure, rset, L.u0[i], L.v0[i], dims == 3 ? L.w0[i] : (T)0);
            }
        } else if (dims == 2) {
            for (size_t b = 0; b < L.bcnodes.size(); ++b) bc_node_2d(L, (int)b, L.bcnodes[b], L.mask[L.bcnodes[b]]);
        } else {
            for (size_t b = 0; b < L.bcnodes.size(); ++b) bc_node_3d(L, (int)b, L.bcnodes[b], L.mask[L.bcnodes[b]]);
            if (p->bc_wall_model == 2)
                for (int i : L.bcnodes) complex_wall_node_3d(L, i, L.mask[i]);
            if (p->mode == 0) {
                const std::vector<T> snap = L.f;
                for (int i : L.bcnodes) periodic_node_3d(L, snap, i, L.mask[i]);
                for (int i : L.bcnodes) symm_node_3d(L, i, L.mask[i]);
            }
        }
        macro_all(L);
        if (out_resid) out_resid[it] = l2_residual(L);
    }
    if (out_f) for (size_t k = 0; k < L.f.size(); ++k) out_f[k] = (double)L.f[k];
    if (extra_collide) collide_all(L);
    if (out_fc) for (size_t k = 0; k < L.fc.size(); ++k) out_fc[k] = (double)L.fc[k];
    for (int i = 0; i < N; ++i) {
        if (out_rho) out_rho[i] = (double)L.rho[i];
        if (out_u) out_u[i] = (double)L.u[i];
        if (out_v) out_v[i] = (double)L.v[i];
        if (out_w) out_w[i] = dims == 3 ? (double)L.w3[i] : 0.0;
    }
    if (out_mask) for (int i = 0; i < N; ++i) out_mask[i] = L.mask[i];
    if (out_stream) for (size_t k = 0; k < L.stream.size(); ++k) out_stream[k] = L.stream[k];
    if (out_count) *out_count = (int)L.bcnodes.size();
    return ORC_OK;
}

}  // namespace

extern "C" {

int orc_version(void) { return 1; }

int orc_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_set_threads(int t) {
#ifdef _OPENMP
    if (t > 0) omp_set_num_threads(t);
#else
    (void)t;
#endif
}

/* One run of the time-step loop.  dims 2 or 3; node arrays x-fastest;
 * bc_k may be NULL in 2D.  fp64 selects the storage/arithmetic type.
 * extra_collide: apply one more collision after the last step so out_fc holds
 * the post-collision populations the next step would stream.  Returns 0, or
 * ORC_UNSUPPORTED / ORC_BAD_INPUT. */
int orc_run(int fp64, int dims, int n, int m, int h, const int *node_type, int nconn,
            const int *bc_i, const int *bc_j, const int *bc_k, const int *bc_dir,
            const int *bc_type, const int *bc_id, const orc_params *p, const double *u_init,
            const double *v_init, const double *w_init, const double *rho_init, int steps,
            int extra_collide, double *out_f, double *out_fc, double *out_rho, double *out_u,
            double *out_v, double *out_w, uint64_t *out_mask, uint8_t *out_stream,
            int *out_count, double *out_resid) {
    static const int zero = 0;
    std::vector<int> kz;
    if (!bc_k) {
        kz.assign(nconn > 0 ? nconn : 1, zero);
        bc_k = kz.data();
    }
    if (fp64)
        return run<double>(dims, n, m, h, node_type, nconn, bc_i, bc_j, bc_k, bc_dir, bc_type,
                           bc_id, p, u_init, v_init, w_init, rho_init, steps, extra_collide,
                           out_f, out_fc, out_rho, out_u, out_v, out_w, out_mask, out_stream,
                           out_count, out_resid);
    return run<float>(dims, n, m, h, node_type, nconn, bc_i, bc_j, bc_k, bc_dir, bc_type, bc_id,
                      p, u_init, v_init, w_init, rho_init, steps, extra_collide, out_f, out_fc,
                      out_rho, out_u, out_v, out_w, out_mask, out_stream, out_count, out_resid);
}

}  // extern "C"

/* =====================================================================
 * Colour-gradient two-phase D2Q9 (restated from GpuCollision.cu:112-707,
 * GpuStream.cu:30-158, GpuUpdateMacro.cu:43-135, constants GpuInit.cu:144-203).
 *
 * One step, as the reference orders it (Iterate.cu:393-491):
 *   collide: colour gradient of phi = (rho_r - rho_b)/rho from the 3x3
 *     (cg_w = 4/12, 1/12) or 24-point (weights /5040) stencil, one BGK with
 *     omega_eff from the harmonic mean viscosity, phase-dependent rest weights
 *     phi_k + theta_k alpha_mean, perturbation A|g|(w_k (c.g)^2/|g|^2 - B_k)
 *     and recolouring +/- beta rho_r rho_b/rho cos(phi_k)(phi_k + theta_k alpha);
 *   stream both colours; macroscopic densities, f = r + b, u.
 * The lattice is periodic by index wrap in both axes (the reference copies
 * across a one-node overlap and uses one-sided gradients on its edges; its
 * interior formulas are what this follows).  Test infrastructure only.
 * ===================================================================== */
extern "C" {
typedef struct {
    double r_density, b_density, r_alpha, b_alpha, r_viscosity, b_viscosity;
    double beta, A, g_limit, control_param, g;
    int high_order, enhanced, external_force;
} orc_cg_params;
}

namespace {

const double CG_PHI[9] = {0.0, 0.2, 0.2, 0.2, 0.2, 0.05, 0.05, 0.05, 0.05};
const double CG_TETA[9] = {1.0, -0.2, -0.2, -0.2, -0.2, -0.05, -0.05, -0.05, -0.05};
const double CG_CHI[9] = {-8.0 / 3.0, -1.0 / 6.0, -1.0 / 6.0, -1.0 / 6.0, -1.0 / 6.0, 1.0 / 12.0, 1.0 / 12.0, 1.0 / 12.0, 1.0 / 12.0};
const double CG_PSI[9] = {0.0, 0.5, 0.5, 0.5, 0.5, 0.125, 0.125, 0.125, 0.125};
const double CG_WPERT[9] = {-4.0 / 27.0, 2.0 / 27.0, 2.0 / 27.0, 2.0 / 27.0, 2.0 / 27.0, 5.0 / 108.0, 5.0 / 108.0, 5.0 / 108.0, 5.0 / 108.0};
const double CG_W[9] = {0., 4. / 12., 4. / 12., 4. / 12., 4. / 12., 1. / 12., 1. / 12., 1. / 12., 1. / 12.};
const int HO_CX[25] = {0, 1, 0, -1, 0, 1, -1, -1, 1, 0, 1, 2, 2, 2, 2, 2, 1, 0, -1, -2, -2, -2, -2, -2, -1};
const int HO_CY[25] = {0, 0, 1, 0, -1, 1, 1, -1, -1, 2, 2, 2, 1, 0, -1, -2, -2, -2, -2, -2, -1, 0, 1, 2, 2};
const double HO_W[25] = {0., 960., 960., 960., 960., 448., 448., 448., 448., 84., 32., 1., 32., 84., 32., 1., 32., 84., 32., 1., 32., 84., 32., 1., 32.};

template <class T>
struct CgState {
    int n, m, N;
    orc_cg_params p;
    std::vector<T> rf, bf, rfc, bfc, rr, br, rho, u, v;
    int wrap(int x, int y) const { return ((x % n + n) % n) + n * ((y % m + m) % m); }
};

template <class T>
void cg_macro(CgState<T> &S) {
    const size_t N = (size_t)S.N;
    for (int i = 0; i < S.N; ++i) {
        T r = 0, b = 0, ju = 0, jv = 0;
        for (int d = 0; d < 9; ++d) {
            const T fd = S.rf[i + d * N] + S.bf[i + d * N];
            r += S.rf[i + d * N];
            b += S.bf[i + d * N];
            ju += (T)cx2[d] * fd;
            jv += (T)cy2[d] * fd;
        }
        const T rho = r + b;
        S.rr[i] = r;
        S.br[i] = b;
        S.rho[i] = rho;
        S.u[i] = ju / rho;
        S.v[i] = jv / rho;
    }
}

template <class T>
void cg_collide(CgState<T> &S) {
    const size_t N = (size_t)S.N;
    const orc_cg_params &p = S.p;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < S.N; ++i) {
        const int x = i % S.n, y = i / S.n;
        T cgx = 0, cgy = 0, grx = 0, gry = 0;
        if (p.high_order) {
            for (int k = 1; k < 25; ++k) {
                const int j = S.wrap(x + HO_CX[k], y + HO_CY[k]);
                const T w = (T)(HO_W[k] / 5040.0);
                const T a1 = w * (S.rr[j] - S.br[j]) / S.rho[j], a2 = w * S.rho[j];
                grx += a2 * (T)HO_CX[k];
                gry += a2 * (T)HO_CY[k];
                cgx += a1 * (T)HO_CX[k];
                cgy += a1 * (T)HO_CY[k];
            }
        } else {
            for (int k = 1; k < 9; ++k) {
                const int j = S.wrap(x + cx2[k], y + cy2[k]);
                const T a1 = (T)CG_W[k] * (S.rr[j] - S.br[j]) / S.rho[j], a2 = (T)CG_W[k] * S.rho[j];
                grx += a2 * (T)cx2[k];
                gry += a2 * (T)cy2[k];
                cgx += a1 * (T)cx2[k];
                cgy += a1 * (T)cy2[k];
            }
        }
        const T r_r = S.rr[i], b_r = S.br[i], r = S.rho[i], u = S.u[i], v = S.v[i];
        const T mean_nu = (T)1.0 / (r_r / (r * (T)p.r_viscosity) + b_r / (r * (T)p.b_viscosity));
        const T omega_eff = (T)1.0 / ((T)3.0 * mean_nu + (T)0.5);
        const T mean_alpha = (T)p.r_alpha * r_r / r + (T)p.b_alpha * b_r / r;
        const T gnorm = std::sqrt(cgx * cgx + cgy * cgy);
        const T k_r = r_r / r, k_b = b_r / r, k_k = (T)p.beta * r_r * b_r / r;
        const T cu1 = u * u + v * v;
        const T G1 = (T)2.0 * u * grx, G2 = u * gry + v * grx, G4 = (T)2.0 * v * gry;
        const T ugr = u * grx + v * gry;
        for (int k = 0; k < 9; ++k) {
            T pert = 0, cosin = 0;
            if (gnorm > (T)p.g_limit) {
                const T pcg = (T)cx2[k] * cgx + (T)cy2[k] * cgy;
                const T cn = k == 0 ? (T)0 : (k <= 4 ? (T)1 : (T)std::sqrt(2.0));
                cosin = k != 0 ? pcg / (gnorm * cn) : (T)0;
                const T wk = k == 0 ? (T)(4. / 9.) : (k <= 4 ? (T)(1. / 9.) : (T)(1. / 36.));
                pert = (T)p.A * gnorm * (wk * (pcg * pcg) / (gnorm * gnorm) - (T)CG_WPERT[k]);
            }
            const T wk = k == 0 ? (T)(4. / 9.) : (k <= 4 ? (T)(1. / 9.) : (T)(1. / 36.));
            const T cu2 = u * (T)cx2[k] + v * (T)cy2[k];
            const T rest = (T)CG_PHI[k] + (T)CG_TETA[k] * mean_alpha;
            T feq = r * (rest + wk * ((T)3. * cu2 + (T)4.5 * cu2 * cu2 - (T)1.5 * cu1));
            if (p.enhanced) {
                const T TC = G1 * (T)(cx2[k] * cx2[k]) + (T)2 * G2 * (T)(cx2[k] * cy2[k]) + G4 * (T)(cy2[k] * cy2[k]);
                feq += mean_nu * ((T)CG_CHI[k] * ugr + (T)CG_PSI[k] * TC);
            }
            const T fk = S.rf[i + k * N] + S.bf[i + k * N];
            const T fp = omega_eff * feq + ((T)1 - omega_eff) * fk + pert;
            S.rfc[i + k * N] = k_r * fp + k_k * cosin * rest;
            S.bfc[i + k * N] = k_b * fp - k_k * cosin * rest;
        }
    }
}

template <class T>
void cg_stream(CgState<T> &S) {
    const size_t N = (size_t)S.N;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < S.N; ++i) {
        const int x = i % S.n, y = i / S.n;
        for (int d = 0; d < 9; ++d) {
            const int j = S.wrap(x - cx2[d], y - cy2[d]);
            S.rf[i + d * N] = S.rfc[j + d * N];
            S.bf[i + d * N] = S.bfc[j + d * N];
        }
    }
}

template <class T>
int run_cg(int n, int m, const orc_cg_params *p, const double *r0, const double *b0, int steps,
           int extra_collide, double *out_rf, double *out_bf, double *out_rfc, double *out_bfc,
           double *out_rr, double *out_br, double *out_u, double *out_v, double *out_laplace) {
    CgState<T> S;
    S.n = n;
    S.m = m;
    S.N = n * m;
    S.p = *p;
    const size_t Q = 9 * (size_t)S.N;
    S.rf.assign(r0, r0 + Q);
    S.bf.assign(b0, b0 + Q);
    S.rfc.assign(Q, (T)0);
    S.bfc.assign(Q, (T)0);
    S.rr.assign(S.N, 0);
    S.br.assign(S.N, 0);
    S.rho.assign(S.N, 0);
    S.u.assign(S.N, 0);
    S.v.assign(S.N, 0);
    cg_macro(S);
    for (int it = 0; it < steps; ++it) {
        cg_collide(S);
        cg_stream(S);
        cg_macro(S);
    }
    if (extra_collide) cg_collide(S);
    for (size_t k = 0; k < Q; ++k) {
        if (out_rf) out_rf[k] = S.rf[k];
        if (out_bf) out_bf[k] = S.bf[k];
        if (out_rfc) out_rfc[k] = S.rfc[k];
        if (out_bfc) out_bfc[k] = S.bfc[k];
    }
    double pin = 0, pout = 0, nin = 0, nout = 0, umax = 0;
    for (int i = 0; i < S.N; ++i) {
        if (out_rr) out_rr[i] = S.rr[i];
        if (out_br) out_br[i] = S.br[i];
        if (out_u) out_u[i] = S.u[i];
        if (out_v) out_v[i] = S.v[i];
        const double chi = ((double)S.rr[i] - (double)S.br[i]) / (double)S.rho[i];
        if (chi >= p->control_param) { pin += S.rr[i]; nin += 1; }
        else if (chi <= -p->control_param) { pout += S.br[i]; nout += 1; }
        const double um = sqrt((double)S.u[i] * S.u[i] + (double)S.v[i] * S.v[i]);
        if (um > umax) umax = um;
    }
    if (out_laplace) {
        out_laplace[0] = pin;
        out_laplace[1] = nin;
        out_laplace[2] = pout;
        out_laplace[3] = nout;
        out_laplace[4] = umax;
    }
    return ORC_OK;
}

}  // namespace

extern "C" int orc_run_cg2d(int fp64, int n, int m, const orc_cg_params *p, const double *r0,
                            const double *b0, int steps, int extra_collide, double *out_rf,
                            double *out_bf, double *out_rfc, double *out_bfc, double *out_rr,
                            double *out_br, double *out_u, double *out_v, double *out_laplace) {
    if (n < 3 || m < 3 || !p || !r0 || !b0) return ORC_BAD_INPUT;
    if (p->g != 0.0) return ORC_UNSUPPORTED; /* body-force variants not restated */
    if (fp64)
        return run_cg<double>(n, m, p, r0, b0, steps, extra_collide, out_rf, out_bf, out_rfc, out_bfc,
                              out_rr, out_br, out_u, out_v, out_laplace);
    return run_cg<float>(n, m, p, r0, b0, steps, extra_collide, out_rf, out_bf, out_rfc, out_bfc, out_rr,
                         out_br, out_u, out_v, out_laplace);
}

/* One colour-gradient collision from given macroscopic fields and summed
 * populations (the inputs of gpuCollBgkwGC2D), for pinning against the
 * reference kernel. */
extern "C" int orc_cg2d_collide(int fp64, int n, int m, const orc_cg_params *p, const double *rho,
                                const double *r_rho, const double *b_rho, const double *u,
                                const double *v, const double *f, double *out_rfc, double *out_bfc) {
    auto go = [&](auto tag) {
        using T = decltype(tag);
        CgState<T> S;
        S.n = n;
        S.m = m;
        S.N = n * m;
        S.p = *p;
        const size_t Q = 9 * (size_t)S.N;
        S.rf.assign(f, f + Q);
        S.bf.assign(Q, (T)0);
        S.rfc.assign(Q, (T)0);
        S.bfc.assign(Q, (T)0);
        S.rr.assign(r_rho, r_rho + S.N);
        S.br.assign(b_rho, b_rho + S.N);
        S.rho.assign(rho, rho + S.N);
        S.u.assign(u, u + S.N);
        S.v.assign(v, v + S.N);
        cg_collide(S);
        for (size_t k = 0; k < Q; ++k) {
            out_rfc[k] = S.rfc[k];
            out_bfc[k] = S.bfc[k];
        }
        return ORC_OK;
    };
    return fp64 ? go(0.0) : go(0.0f);
}

/* =====================================================================
 * Colour-gradient two-phase D3Q19 (restated from gpuCollBgkwGC3D and
 * gpuCollEnhancedBgkwGC3D, GpuCollision.cu:283-526, :709-880; streaming
 * GpuStream.cu:196-250; macroscopic update gpuUpdateMacro3DCG,
 * GpuUpdateMacro.cu:215-360; constants GpuInit.cu:896-990).
 *
 * Same step as the D2Q9 path above, on a lattice periodic by index wrap in
 * all three axes.  The gradient stencils: the 18 lattice neighbours with
 * weights 1/6 (axes) and 1/12 (diagonals), or the 104-point isotropic set
 * of shells |c|^2 = 1, 2, 3, 4, 5, 6, 9 with weights 4/45, 1/21, 2/105,
 * 5/504, 1/315, 1/630, 1/5040 (Shan's eighth-order 3D set), summed here shell
 * by shell in lexicographic order (the reference sums its own table order).
 * Below the gradient limit the recolouring cosine is 0 (the reference's
 * non-enhanced kernel leaves it unset there).  No body force.
 * Test infrastructure only.
 * ===================================================================== */
namespace {

const double CG3_W[19] = {1. / 3., 1. / 18., 1. / 18., 1. / 18., 1. / 18., 1. / 18., 1. / 18., 1. / 36., 1. / 36.,
                          1. / 36., 1. / 36., 1. / 36., 1. / 36., 1. / 36., 1. / 36., 1. / 36., 1. / 36., 1. / 36., 1. / 36.};

inline double cg3_phi(int d) { return d == 0 ? 0.0 : (d <= 6 ? 1. / 12. : 1. / 24.); }
inline double cg3_teta(int d) { return d == 0 ? 1.0 : (d <= 6 ? -1. / 12. : -1. / 24.); }
inline double cg3_chi(int d) { return d == 0 ? -5.0 / 2.0 : (d <= 6 ? -1. / 6. : 1. / 24.); }
inline double cg3_psi(int d) { return d == 0 ? 0.0 : (d <= 6 ? 1. / 4. : 1. / 8.); }
inline double cg3_wpert(int d) { return d == 0 ? -2.0 / 9.0 : (d <= 6 ? 1.0 / 54.0 : 1.0 / 27.0); }
inline double cg3_gw(int d) { return d == 0 ? 0.0 : (d <= 6 ? 1. / 6. : 1. / 12.); }

struct Ho3 {
    int n = 0;
    int c[104][3];
    double w[104];
    Ho3() {
        const int shells[7] = {1, 2, 3, 4, 5, 6, 9};
        const double ws[7] = {4. / 45., 1. / 21., 2. / 105., 5. / 504., 1. / 315., 1. / 630., 1. / 5040.};
        for (int s = 0; s < 7; ++s)
            for (int x = -2; x <= 2; ++x)
                for (int y = -2; y <= 2; ++y)
                    for (int z = -2; z <= 2; ++z)
                        if (x * x + y * y + z * z == shells[s]) {
                            c[n][0] = x;
                            c[n][1] = y;
                            c[n][2] = z;
                            w[n] = ws[s];
                            ++n;
                        }
    }
};
const Ho3 HO3;

template <class T>
struct CgState3 {
    int n, m, h, N;
    orc_cg_params p;
    std::vector<T> rf, bf, rfc, bfc, rr, br, rho, u, v, w;
    int wrap(int x, int y, int z) const {
        return ((x % n + n) % n) + n * (((y % m + m) % m) + m * ((z % h + h) % h));
    }
};

template <class T>
void cg3_macro(CgState3<T> &S) {
    const size_t N = (size_t)S.N;
    for (int i = 0; i < S.N; ++i) {
        T r = 0, b = 0, ju = 0, jv = 0, jw = 0;
        for (int d = 0; d < 19; ++d) {
            const T fd = S.rf[i + d * N] + S.bf[i + d * N];
            r += S.rf[i + d * N];
            b += S.bf[i + d * N];
            ju += (T)cx3[d] * fd;
            jv += (T)cy3[d] * fd;
            jw += (T)cz3[d] * fd;
        }
        const T rho = r + b;
        S.rr[i] = r;
        S.br[i] = b;
        S.rho[i] = rho;
        S.u[i] = ju / rho;
        S.v[i] = jv / rho;
        S.w[i] = jw / rho;
    }
}

template <class T>
void cg3_collide(CgState3<T> &S) {
    const size_t N = (size_t)S.N;
    const orc_cg_params &p = S.p;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < S.N; ++i) {
        const int x = i % S.n, y = (i / S.n) % S.m, z = i / (S.n * S.m);
        T cgx = 0, cgy = 0, cgz = 0, grx = 0, gry = 0, grz = 0;
        auto add = [&](int ox, int oy, int oz, T wgt) {
            const int j = S.wrap(x + ox, y + oy, z + oz);
            const T a1 = wgt * (S.rr[j] - S.br[j]) / S.rho[j], a2 = wgt * S.rho[j];
            grx += a2 * (T)ox;
            gry += a2 * (T)oy;
            grz += a2 * (T)oz;
            cgx += a1 * (T)ox;
            cgy += a1 * (T)oy;
            cgz += a1 * (T)oz;
        };
        if (p.high_order) {
            for (int k = 0; k < HO3.n; ++k) add(HO3.c[k][0], HO3.c[k][1], HO3.c[k][2], (T)HO3.w[k]);
        } else {
            for (int k = 1; k < 19; ++k) add(cx3[k], cy3[k], cz3[k], (T)cg3_gw(k));
        }
        const T r_r = S.rr[i], b_r = S.br[i], r = S.rho[i], u = S.u[i], v = S.v[i], w = S.w[i];
        const T G1 = (T)2.0 * u * grx, G2 = u * gry + v * grx, G3 = u * grz + w * grx;
        const T G4 = G2, G5 = (T)2.0 * v * gry, G6 = v * grz + w * gry;
        const T G7 = G3, G8 = G6, G9 = (T)2.0 * w * grz;
        const T ugr = u * grx + v * gry + w * grz;
        const T cu1 = u * u + v * v + w * w;
        const T gnorm = std::sqrt(cgx * cgx + cgy * cgy + cgz * cgz);
        const T k_r = r_r / r, k_b = b_r / r, k_k = (T)p.beta * r_r * b_r / r;
        const T mean_nu = (T)1.0 / (r_r / (r * (T)p.r_viscosity) + b_r / (r * (T)p.b_viscosity));
        const T omega_eff = (T)1.0 / ((T)3.0 * mean_nu + (T)0.5);
        const T mean_alpha = (T)p.r_alpha * r_r / r + (T)p.b_alpha * b_r / r;
        for (int k = 0; k < 19; ++k) {
            const T cx = (T)cx3[k], cy = (T)cy3[k], cz = (T)cz3[k];
            const T wk = (T)CG3_W[k];
            T pert = 0, cosin = 0;
            if (gnorm > (T)p.g_limit) {
                const T pcg = cx * cgx + cy * cgy + cz * cgz;
                const T cn = (T)std::sqrt((double)(cx3[k] * cx3[k] + cy3[k] * cy3[k] + cz3[k] * cz3[k]));
                cosin = k != 0 ? pcg / (gnorm * cn) : (T)0;
                pert = (T)p.A * gnorm * (wk * (pcg * pcg) / (gnorm * gnorm) - (T)cg3_wpert(k));
            }
            const T cu2 = u * cx + v * cy + w * cz;
            const T rest = (T)cg3_phi(k) + (T)cg3_teta(k) * mean_alpha;
            T feq = r * (rest + wk * ((T)3. * cu2 + (T)4.5 * cu2 * cu2 - (T)1.5 * cu1));
            if (p.enhanced) {
                T TC = 0;
                TC += G1 * cx * cx;
                TC += G2 * cx * cy;
                TC += G3 * cx * cz;
                TC += G4 * cx * cy;
                TC += G5 * cy * cy;
                TC += G6 * cy * cz;
                TC += G7 * cx * cz;
                TC += G8 * cy * cz;
                TC += G9 * cz * cz;
                feq = mean_nu * ((T)cg3_chi(k) * ugr + (T)cg3_psi(k) * TC) + feq;
            }
            const T fk = S.rf[i + k * N] + S.bf[i + k * N];
            const T fp = omega_eff * feq + ((T)1 - omega_eff) * fk + pert;
            S.rfc[i + k * N] = k_r * fp + k_k * cosin * rest;
            S.bfc[i + k * N] = k_b * fp - k_k * cosin * rest;
        }
    }
}

template <class T>
void cg3_stream(CgState3<T> &S) {
    const size_t N = (size_t)S.N;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < S.N; ++i) {
        const int x = i % S.n, y = (i / S.n) % S.m, z = i / (S.n * S.m);
        for (int d = 0; d < 19; ++d) {
            const int j = S.wrap(x - cx3[d], y - cy3[d], z - cz3[d]);
            S.rf[i + d * N] = S.rfc[j + d * N];
            S.bf[i + d * N] = S.bfc[j + d * N];
        }
    }
}

template <class T>
void cg3_alloc(CgState3<T> &S, int n, int m, int h, const orc_cg_params *p) {
    S.n = n;
    S.m = m;
    S.h = h;
    S.N = n * m * h;
    S.p = *p;
    const size_t Q = 19 * (size_t)S.N;
    S.rf.assign(Q, (T)0);
    S.bf.assign(Q, (T)0);
    S.rfc.assign(Q, (T)0);
    S.bfc.assign(Q, (T)0);
    for (auto *a : {&S.rr, &S.br, &S.rho, &S.u, &S.v, &S.w}) a->assign(S.N, (T)0);
}

template <class T>
int run_cg3(int n, int m, int h, const orc_cg_params *p, const double *r0, const double *b0, int steps,
            int extra_collide, double *out_rfc, double *out_bfc, double *out_rr, double *out_br, double *out_u,
            double *out_v, double *out_w, double *out_laplace) {
    CgState3<T> S;
    cg3_alloc(S, n, m, h, p);
    const size_t Q = 19 * (size_t)S.N;
    for (size_t k = 0; k < Q; ++k) {
        S.rf[k] = (T)r0[k];
        S.bf[k] = (T)b0[k];
    }
    cg3_macro(S);
    for (int it = 0; it < steps; ++it) {
        cg3_collide(S);
        cg3_stream(S);
        cg3_macro(S);
    }
    if (extra_collide) cg3_collide(S);
    for (size_t k = 0; k < Q; ++k) {
        if (out_rfc) out_rfc[k] = S.rfc[k];
        if (out_bfc) out_bfc[k] = S.bfc[k];
    }
    double pin = 0, pout = 0, nin = 0, nout = 0, umax = 0;
    for (int i = 0; i < S.N; ++i) {
        if (out_rr) out_rr[i] = S.rr[i];
        if (out_br) out_br[i] = S.br[i];
        if (out_u) out_u[i] = S.u[i];
        if (out_v) out_v[i] = S.v[i];
        if (out_w) out_w[i] = S.w[i];
        const double chi = ((double)S.rr[i] - (double)S.br[i]) / (double)S.rho[i];
        if (chi >= p->control_param) { pin += S.rr[i]; nin += 1; }
        else if (chi <= -p->control_param) { pout += S.br[i]; nout += 1; }
        const double um = sqrt((double)S.u[i] * S.u[i] + (double)S.v[i] * S.v[i] + (double)S.w[i] * S.w[i]);
        if (um > umax) umax = um;
    }
    if (out_laplace) {
        out_laplace[0] = pin;
        out_laplace[1] = nin;
        out_laplace[2] = pout;
        out_laplace[3] = nout;
        out_laplace[4] = umax;
    }
    return ORC_OK;
}

}  // namespace

/* steps of the D3Q19 colour-gradient loop from post-streaming populations
 * r0, b0 (19*n*m*h each); extra_collide as in orc_run. */
extern "C" int orc_run_cg3d(int fp64, int n, int m, int h, const orc_cg_params *p, const double *r0,
                            const double *b0, int steps, int extra_collide, double *out_rfc, double *out_bfc,
                            double *out_rr, double *out_br, double *out_u, double *out_v, double *out_w,
                            double *out_laplace) {
    if (n < 5 || m < 5 || h < 5 || !p || !r0 || !b0) return ORC_BAD_INPUT;
    if (p->g != 0.0) return ORC_UNSUPPORTED;
    if (fp64)
        return run_cg3<double>(n, m, h, p, r0, b0, steps, extra_collide, out_rfc, out_bfc, out_rr, out_br, out_u,
                               out_v, out_w, out_laplace);
    return run_cg3<float>(n, m, h, p, r0, b0, steps, extra_collide, out_rfc, out_bfc, out_rr, out_br, out_u, out_v,
                          out_w, out_laplace);
}

/* One D3Q19 colour-gradient collision from given macroscopic fields and
 * summed populations f (the inputs of gpuCollBgkwGC3D), for pinning against
 * the reference kernel. */
extern "C" int orc_cg3d_collide(int fp64, int n, int m, int h, const orc_cg_params *p, const double *rho,
                                const double *r_rho, const double *b_rho, const double *u, const double *v,
                                const double *w, const double *f, double *out_rfc, double *out_bfc) {
    auto go = [&](auto tag) {
        using T = decltype(tag);
        CgState3<T> S;
        cg3_alloc(S, n, m, h, p);
        const size_t Q = 19 * (size_t)S.N;
        for (size_t k = 0; k < Q; ++k) S.rf[k] = (T)f[k];
        for (int i = 0; i < S.N; ++i) {
            S.rr[i] = (T)r_rho[i];
            S.br[i] = (T)b_rho[i];
            S.rho[i] = (T)rho[i];
            S.u[i] = (T)u[i];
            S.v[i] = (T)v[i];
            S.w[i] = (T)w[i];
        }
        cg3_collide(S);
        for (size_t k = 0; k < Q; ++k) {
            out_rfc[k] = S.rfc[k];
            out_bfc[k] = S.bfc[k];
        }
        return ORC_OK;
    };
    return fp64 ? go(0.0) : go(0.0f);
}
