// Fused lattice-Boltzmann time step: one launch per step does what the
// reference does in four (collision, streaming, boundary and macroscopic
// kernels with a host synchronisation after each, Iterate3D.cu:493-653):
//
//   for every fluid node, in registers:
//     f_d  <- post-collision population d of the neighbour x - c_d   (pull)
//             or, across a blocked link, the node's own population
//             (reference: f_d itself; physics: f_opp(d), half-way bounce-back)
//     boundary conditions (reference wall copies / Zou-He faces)
//     rho, u <- moments of f  (+ g/omega body-force shift in 3D)
//     f <- collide(f, rho, u)  and store to the other buffer
//
// The state between launches is the post-collision population field in a
// pull double buffer laid out as rows: for every lattice row (y, z) the Q
// directions follow each other, each a run of nx values (x fastest), so
// population d of node (x, y, z) sits at d*nx + x + pitch*(y + ny*z) with
// pitch = Q*nx.  A warp's loads and stores are 32 consecutive nodes of one
// direction, one row of one direction is contiguous (a single bulk copy),
// and all populations of a node are at fixed offsets from one base.  Per node the kernel reads one 32-bit flag word and Q
// populations and writes Q populations; macroscopic fields are written only
// on steps that need them (residuals, output).
#pragma once
#include "lbm_bc.cuh"

namespace lbm {

struct StepParams {
    const void *fin[19];
    void *fout[19];
    const uint32_t *word;
    const int32_t *slot;
    const unsigned long long *bc_mask;
    const int32_t *bc_kind;
    const double *bc_uvw;
    // reference curved walls: per boundary slot Q link fractions q (entry
    // dir-1 for link dir, entry Q-1 the next boundary node's direction-1
    // entry); null for straight walls
    const double *bc_q;
    // physics-mode HEmodel outlets: per boundary slot the node's rho, u, v, w
    // of the previous step (4 doubles, written by the node's own thread every
    // step; doubles so an F64 run keeps its precision)
    double *bc_macro;
    float *rho, *ux, *uy, *uz;
    int nx, ny, nz;
    int pitch;  // elements from one row of a direction to the next (Q * nx)
    int write_macro;
    double omega, omega_m, gshift;
    double rho_in, rho_out;
    double rho0;  // reference density (moving walls)
    int ref_hh;   // reference mode: the HH wall model instead of straight walls
    float scale, inv_scale;
    // F16S storage holds (f_d - shift_d) * scale and physics-mode F32 storage
    // f_d - shift_d: shift is the collision model's rest-state equilibrium
    // (0 for F64 and reference-mode F32); sigma is 1 when shift is applied
    float shift[19];
    float sigma;
    int outlet_profile;
    int update_inlet_outlet;
    // initial state (init kernel only): constants for the fields not given as
    // arrays (bit 0 rho, 1 ux, 2 uy, 3 uz set = read the array)
    double init_rho, init_ux, init_uy, init_uz;
    int init_from_arrays;
};

constexpr int STEP_BLOCK = 128;

template <int Q, int COLL, int ST, bool PHYS>
__device__ __forceinline__ void collide(typename Store<ST>::R (&f)[Q], typename Store<ST>::R rho,
                                        typename Store<ST>::R ux, typename Store<ST>::R uy,
                                        typename Store<ST>::R uz, const StepParams &p) {
    using R = typename Store<ST>::R;
    if (COLL == LBM_BGKW) {
        collide_bgk<Q, R>(f, rho, ux, uy, uz, (R)p.omega);
    } else if (COLL == LBM_TRT) {
        collide_trt<Q, R>(f, rho, ux, uy, uz, (R)p.omega, (R)p.omega_m);
    } else {
        if constexpr (Q == 9)
            collide_mrt9<!PHYS, R>(f, rho, ux, uy, (R)p.omega);
        else
            collide_mrt19<!PHYS, R>(f, rho, ux, uy, uz, (R)p.omega);
    }
}

// Lattice extents seen by the step: read from the parameters (DynGeom) or
// fixed at compile time (FixedGeom, the build specialised for one lattice,
// where every population offset becomes an immediate).
struct DynGeom {
    int nx, ny, nz, pitch;
};
template <int NX, int NY, int NZ, int PITCH>
struct FixedGeom {
    static constexpr int nx = NX, ny = NY, nz = NZ, pitch = PITCH;
};

template <int Q, int ST, bool PHYS, bool WRAP, class G, int HINT, bool PRED>
__device__ __forceinline__ void gather_node(const StepParams &p, const G &g, int x, int y, int z, uint32_t w,
                                            const typename Store<ST>::T *in, typename Store<ST>::R (&f)[Q]);

// The reference's curved (q-interpolated) wall: the CURVED branch of
// gpuBcWall2D / gpuBcSimpleWall3D (GpuBoundaries.cu:414-432, :461-479),
// linear interpolation (Bouzidi) between post-collision populations f* of the
// last step, i.e. the read buffer.  For every wall link dir of node x, with
// q0 the link's fraction and q1 the entry after it in the reference's
// per-node table (the link dir+1, and for the last direction the first link
// of the next boundary node: the reference reads its first coefficient one
// entry ahead, p.bc_q keeps that entry as the slot's last),
//   q0 < 1/2:  f_opp(dir) = 2 q1 f*_dir(x) + (1 - 2 q0) f*_dir(x - c_dir)
//   else:      f_opp(dir) = f*_dir(x) / 2 / q0 + (2 q0 - 1) / (2 q0) f*_opp(dir)(x)
// cv[dir] receives the value for each wall link.  The reference reads
// f*_dir(x - c_dir) at the flat index node + dir N + c(dir) of its SoA array
// (N nodes per direction, c(dir) the linear pull offset): the upstream node
// inside the lattice, a neighbouring row's or another direction's value
// where x - c_dir lies outside it; the same element is read here from the
// row layout, and 0 past either end of the array (undefined there in the
// reference).
template <int Q, int ST, class G>
__device__ __forceinline__ void ref_curved(typename Store<ST>::R (&cv)[Q], uint64_t mk, int sl, int node,
                                           const StepParams &p, const G &g) {
    using S = Store<ST>;
    using T = typename S::T;
    using R = typename S::R;
    using L = Lat<Q>;
    const int x = node % g.nx, row = node / g.nx;
    const T *base = (const T *)p.fin[0];
    const T *in = base + (x + (long long)g.pitch * row);
    const long long total = (long long)g.nx * g.ny * g.nz;
    const double *qs = p.bc_q + (long long)sl * Q;
#pragma unroll
    for (int dir = 1; dir < Q; ++dir) {
        bool wall;
        if constexpr (Q == 9)
            wall = ((uint32_t)mk & m2(3, dir)) == m2(1, dir);
        else
            wall = (mk & m3(7, dir)) == m3(1, dir);
        if (!wall) continue;
        const R own = S::decode(in[dir * g.nx], p.shift[dir], p.inv_scale);
        const R q0 = (R)qs[dir - 1];
        if (q0 < (R)0.5) {
            const long long flat = (long long)node + dir * total -
                                   (L::cx(dir) + (long long)L::cy(dir) * g.nx + (long long)L::cz(dir) * g.nx * g.ny);
            R up = (R)0;
            if (flat >= 0 && flat < Q * total) {
                const int du = (int)(flat / total);
                const long long nu = flat - du * total;
                const long long xu = nu % g.nx, ru = nu / g.nx;
                up = S::decode(base[du * g.nx + xu + (long long)g.pitch * ru], p.shift[du], p.inv_scale);
            }
            cv[dir] = (R)2 * (R)qs[dir] * own + ((R)1 - (R)2 * q0) * up;
        } else {
            const int o = L::opp(dir);
            const R own_o = S::decode(in[o * g.nx], p.shift[o], p.inv_scale);
            cv[dir] = own / (R)2 / q0 + ((R)2 * q0 - (R)1) / ((R)2 * q0) * own_o;
        }
    }
}

// The reference's 3D periodic copy (gpuBcPeriodic3D, GpuBoundaries.cu:
// 2025-2084): a node with a periodic link on a face takes the five
// populations entering through that face from the node one lattice length
// away (linear offsets n-1, n(m-1), nm(h-1)), as that node holds them after
// streaming, inlet and wall conditions.  The partner's populations are
// recomputed here from the read buffer (pull + its own boundary conditions),
// so every periodic node sees its partners' values from before any periodic
// copy; the reference runs the copies as concurrent threads, which agree with
// this wherever a partner does not itself copy the same directions (one
// periodic axis) and race where two periodic faces meet.
template <int ST, bool WRAP, class G>
__device__ __forceinline__ void ref3_periodic(typename Store<ST>::R (&f)[19], uint64_t mk, int node,
                                              const StepParams &p, const G &g) {
    using S = Store<ST>;
    using T = typename S::T;
    using R = typename S::R;
    using L = Lat<19>;
    if (!(mk & R3_FLUID) || !(mk & R3_CYCL_B)) return;
    const int n = g.nx, nm = g.nx * g.ny;
    const long long total = (long long)nm * g.nz;
#pragma unroll 1
    for (int k = 0; k < 6; ++k) {
        // faces in the reference's order W, E, S, N, B, T: periodic bit of
        // direction 2, 1, 4, 3, 6, 5; partner offset +-(n-1), +-n(m-1), +-nm(h-1)
        const int dir = (k & 1) ? k : k + 2;
        if (!(mk & m3(4, dir))) continue;
        const int axis_off = k < 2 ? n - 1 : (k < 4 ? n * (g.ny - 1) : nm * (g.nz - 1));
        const long long pn = (long long)node + ((k & 1) ? -axis_off : axis_off);
        if (pn < 0 || pn >= total) continue;
        const int px = (int)(pn % n), py = (int)((pn / n) % g.ny), pz = (int)(pn / nm);
        const uint32_t pw = __ldg(p.word + pn);
        R fb[19];
        if (pw & W_FLUID) {
            const T *in = (const T *)p.fin[0] + (px + (long long)g.pitch * (py + g.ny * pz));
            gather_node<19, ST, false, WRAP, G, 0, false>(p, g, px, py, pz, pw, in, fb);
            if (pw & W_SPECIAL) {
                const int sl = __ldg(p.slot + pn);
                const uint64_t pmk = __ldg(p.bc_mask + sl);
                const R pu = (R)__ldg(p.bc_uvw + 3 * sl), pv = (R)__ldg(p.bc_uvw + 3 * sl + 1),
                        pw0 = (R)__ldg(p.bc_uvw + 3 * sl + 2);
                if (p.bc_q) {
                    R cv[19];
                    ref_curved<19, ST, G>(cv, pmk, sl, (int)pn, p, g);
                    bc_ref3_inlet_wall<R, true>(fb, pmk, pu, pv, pw0, false, cv);
                } else {
                    bc_ref3_inlet_wall<R>(fb, pmk, pu, pv, pw0, p.ref_hh != 0);
                }
            } else {
#pragma unroll
                for (int d = 1; d < 19; ++d)
                    if ((pw >> L::opp(d)) & 1u) fb[L::opp(d)] = fb[d];
            }
        } else {
#pragma unroll
            for (int d = 0; d < 19; ++d) fb[d] = (R)0;
        }
        switch (k) {
        case 0: f[1] = fb[1]; f[7] = fb[7]; f[9] = fb[9]; f[11] = fb[11]; f[13] = fb[13]; break;
        case 1: f[2] = fb[2]; f[8] = fb[8]; f[10] = fb[10]; f[12] = fb[12]; f[14] = fb[14]; break;
        case 2: f[3] = fb[3]; f[7] = fb[7]; f[8] = fb[8]; f[15] = fb[15]; f[17] = fb[17]; break;
        case 3: f[4] = fb[4]; f[9] = fb[9]; f[10] = fb[10]; f[16] = fb[16]; f[18] = fb[18]; break;
        case 4: f[5] = fb[5]; f[11] = fb[11]; f[12] = fb[12]; f[15] = fb[15]; f[16] = fb[16]; break;
        default: f[6] = fb[6]; f[13] = fb[13]; f[14] = fb[14]; f[17] = fb[17]; f[18] = fb[18]; break;
        }
    }
}

// The 2D extrapolation outlets (OUTLET_SECOND / OUTLET_FIRST of
// gpuBcOutlet2D, GpuBoundaries.cu:1608-1638) read f1, f5 and f8 of the nodes
// one and two to the west (flat indices node - 1, node - 2) as they stand
// after streaming, inlet and wall conditions.  Those values are recomputed
// here from the read buffer: the neighbour's pull and its own inlet and wall
// conditions (curved walls included); a solid neighbour holds 0, as the
// reference's never-streamed solid nodes do.
template <int ST, bool WRAP, class G>
__device__ __forceinline__ void ref2_outlet_neighbours(typename Store<ST>::R (&ext)[6], int node, const StepParams &p,
                                                       const G &g) {
    using R = typename Store<ST>::R;
    using T = typename Store<ST>::T;
    using L = Lat<9>;
#pragma unroll 1
    for (int k = 0; k < 2; ++k) {
        const int nb = node - 1 - k;
        R fb[9];
#pragma unroll
        for (int d = 0; d < 9; ++d) fb[d] = (R)0;
        const uint32_t w = nb >= 0 ? __ldg(p.word + nb) : 0u;
        if (w & W_FLUID) {
            const int x = nb % g.nx, y = nb / g.nx;
            const T *in = (const T *)p.fin[0] + (x + (long long)g.pitch * y);
            gather_node<9, ST, false, WRAP, G, 0, false>(p, g, x, y, 0, w, in, fb);
            if (w & W_SPECIAL) {
                const int sl = __ldg(p.slot + nb);
                const uint64_t mk = __ldg(p.bc_mask + sl);
                const R u0 = (R)__ldg(p.bc_uvw + 3 * sl);
                bool zv;
                if (p.bc_q) {
                    R cv[9];
                    ref_curved<9, ST, G>(cv, mk, sl, nb, p, g);
                    bc_ref_d2q9<R, true>(fb, (uint32_t)mk, u0, LBM_OUTLET_HEMODEL, zv, cv);
                } else {
                    bc_ref_d2q9<R>(fb, (uint32_t)mk, u0, LBM_OUTLET_HEMODEL, zv);
                }
            } else {
#pragma unroll
                for (int dir = 1; dir < 9; ++dir)
                    if ((w >> L::opp(dir)) & 1u) fb[L::opp(dir)] = fb[dir];
            }
        }
        ext[3 * k] = fb[1];
        ext[3 * k + 1] = fb[5];
        ext[3 * k + 2] = fb[8];
    }
}

// The physics-mode open outlet of a boundary slot (BCK_EXTRAP1, BCK_EXTRAP2,
// BCK_HE): writes the populations that enter through the slot's face, the
// directions d with c_d . e = 1 for the inward normal e of face
// (kind & BCK_FACE_MASK), in storage units (ST's raw values; the caller's
// arithmetic form): R_OUT(raw) turns a stored value into it and
// EQ(d, rho, ux, uy, uz) gives an equilibrium in it.  The inward neighbours'
// values are their post-stream populations as the gather forms them: pulled
// from y - c_d, or across a blocked link y's own opp(d) (half-way
// bounce-back); a neighbour that is not fluid leaves the population as the
// node's own gather set it.
template <int Q, int ST, bool WRAP, class G, class V, class RAW, class EQ>
__device__ __forceinline__ void phys_open_outlet(V (&f)[Q], int kind, int sl, int node, const StepParams &p,
                                                 const G &g, RAW raw_to, EQ eq) {
    using L = Lat<Q>;
    using T = typename Store<ST>::T;
    const int face = kind & BCK_FACE_MASK;
    const int ex = face == 0 ? 1 : (face == 1 ? -1 : 0), ey = face == 2 ? 1 : (face == 3 ? -1 : 0),
              ez = face == 4 ? 1 : (face == 5 ? -1 : 0);
    const T *base = (const T *)p.fin[0];
    const int x = node % g.nx, y = (node / g.nx) % g.ny, z = node / (g.nx * g.ny);
    auto wrap = [](int a, int n) { return a < 0 ? a + n : (a >= n ? a - n : a); };
    // post-stream value of direction d at the node k steps inward
    auto value = [&](int k, int d, bool &ok) -> V {
        const int yx = x + k * ex, yy = y + k * ey, yz = z + k * ez;
        ok = yx >= 0 && yx < g.nx && yy >= 0 && yy < g.ny && yz >= 0 && yz < g.nz;
        if (!ok) return V(0);
        const uint32_t wy = __ldg(p.word + yx + g.nx * (yy + g.ny * yz));
        ok = (wy & W_FLUID) != 0;
        if (!ok) return V(0);
        if ((wy >> d) & 1u) return raw_to(base + L::opp(d) * g.nx + yx + (long long)g.pitch * (yy + g.ny * yz), d);
        int sx = yx - L::cx(d), sy = yy - L::cy(d), sz = yz - L::cz(d);
        if (WRAP) {
            sx = wrap(sx, g.nx);
            sy = wrap(sy, g.ny);
            sz = wrap(sz, g.nz);
        }
        return raw_to(base + d * g.nx + sx + (long long)g.pitch * (sy + g.ny * sz), d);
    };
    if (kind & BCK_HE) {
        const double *st = p.bc_macro + 4 * sl;
        const V r0 = V(st[0]), u0 = V(st[1]), v0 = V(st[2]), w0 = V(st[3]);
#pragma unroll
        for (int d = 1; d < Q; ++d)
            if (L::cx(d) * ex + L::cy(d) * ey + L::cz(d) * ez == 1) f[d] = eq(d, r0, u0, v0, w0);
        return;
    }
#pragma unroll
    for (int d = 1; d < Q; ++d) {
        if (L::cx(d) * ex + L::cy(d) * ey + L::cz(d) * ez != 1) continue;
        bool ok1 = false, ok2 = false;
        const V f1v = value(1, d, ok1);
        if (!ok1) continue;
        if (kind & BCK_EXTRAP1) {
            f[d] = f1v;
        } else {
            const V f2v = value(2, d, ok2);
            f[d] = ok2 ? V(2) * f1v - f2v : f1v;
        }
    }
}

// Boundary conditions of a fluid node whose populations are gathered
// (pulled, bounced back): Zou-He faces, moving walls, the reference's wall,
// periodic and symmetry copies.  keep_macro / zero_v report the reference's
// 3D inlet and 2D outlet special cases.
template <int Q, int ST, bool PHYS, bool WRAP, class G>
__device__ __forceinline__ void apply_bc(typename Store<ST>::R (&f)[Q], uint32_t w, int node, const StepParams &p,
                                         const G &g, bool &keep_macro, bool &zero_v) {
    using R = typename Store<ST>::R;
    using L = Lat<Q>;
    keep_macro = false;
    zero_v = false;
    if (w & W_SPECIAL) {
        const int sl = __ldg(p.slot + node);
        const R u0 = (R)__ldg(p.bc_uvw + 3 * sl), v0 = (R)__ldg(p.bc_uvw + 3 * sl + 1),
                w0 = (R)__ldg(p.bc_uvw + 3 * sl + 2);
        if constexpr (!PHYS) {
            const unsigned long long mk = __ldg(p.bc_mask + sl);
            // curved walls: the interpolated values come from the read buffer
            // only, so they are formed before any condition changes f
            R cv[Q];
            if (p.bc_q) ref_curved<Q, ST, G>(cv, mk, sl, node, p, g);
            if constexpr (Q == 9) {
                R ext[6];
                const bool extrap = (mk & R2_FLUID) && ((uint32_t)mk & m2(3, 1)) == m2(3, 1) &&
                                    (p.outlet_profile == LBM_OUTLET_SECOND || p.outlet_profile == LBM_OUTLET_FIRST);
                if (extrap) ref2_outlet_neighbours<ST, WRAP, G>(ext, node, p, g);
                if (p.bc_q)
                    bc_ref_d2q9<R, true>(f, (uint32_t)mk, u0, p.outlet_profile, zero_v, cv, extrap ? ext : nullptr);
                else
                    bc_ref_d2q9<R>(f, (uint32_t)mk, u0, p.outlet_profile, zero_v, nullptr, extrap ? ext : nullptr);
            } else {
                // the reference's kernel order: inlet, wall, (outlet), periodic, symmetry
                if (p.bc_q)
                    bc_ref3_inlet_wall<R, true>(f, mk, u0, v0, w0, false, cv);
                else
                    bc_ref3_inlet_wall<R>(f, mk, u0, v0, w0, p.ref_hh != 0);
                ref3_periodic<ST, WRAP, G>(f, mk, node, p, g);
                bc_ref3_symm<R>(f, mk);
                keep_macro = ref3_keep_macro(mk, p.update_inlet_outlet);
            }
        } else {
            const int kind = __ldg(p.bc_kind + sl);
            if (kind & BCK_MOVING) {
                bc_moving_wall<Q, R>(f, __ldg(p.bc_mask + sl), (R)p.rho0, u0, v0, w0);
            } else if (kind & (BCK_EXTRAP1 | BCK_EXTRAP2 | BCK_HE)) {
                using S = Store<ST>;
                phys_open_outlet<Q, ST, WRAP, G, R>(
                    f, kind, sl, node, p, g,
                    [&](const typename S::T *q, int d) { return (R)S::decode(*q, p.shift[d], p.inv_scale); },
                    [&](int d, R r, R ux, R uy, R uz) {
                        return feq<Q, R>(d, r, ux, uy, uz, (R)1.5 * (ux * ux + uy * uy + uz * uz));
                    });
            } else if (kind & BCK_ACTIVE) {
                const bool pressure = (kind & BCK_PRESSURE) != 0;
                const R rset = (kind & BCK_OUTLET) ? (R)p.rho_out : (R)p.rho_in;
                bc_phys<Q, R>(f, kind & BCK_FACE_MASK, pressure, rset, u0, v0, w0);
            }
        }
    } else if constexpr (!PHYS) {
        // reference straight walls: f[opp(dir)] = f[dir] for every wall link
        // dir in direction order (GpuBoundaries.cu:436, :483); on a plain wall
        // node the wall links are exactly the opposites of the blocked pulls.
#pragma unroll
        for (int dir = 1; dir < Q; ++dir)
            if ((w >> L::opp(dir)) & 1u) f[L::opp(dir)] = f[dir];
    }
}

template <int Q, int COLL, int ST, bool PHYS, bool WRAP, class G>
__device__ __forceinline__ void update_node(typename Store<ST>::R (&f)[Q], uint32_t w, int node,
                                            const StepParams &p, const G &g) {
    using R = typename Store<ST>::R;
    using L = Lat<Q>;
    bool keep_macro, zero_v;
    apply_bc<Q, ST, PHYS, WRAP, G>(f, w, node, p, g, keep_macro, zero_v);

    R rho = 0, jx = 0, jy = 0, jz = 0;
#pragma unroll
    for (int d = 0; d < Q; ++d) {
        rho += f[d];
        if (L::cx(d)) jx += (R)L::cx(d) * f[d];
        if (L::cy(d)) jy += (R)L::cy(d) * f[d];
        if (L::cz(d)) jz += (R)L::cz(d) * f[d];
    }
    R ux, uy, uz;
    if (keep_macro) {
        rho = (R)p.rho[node];
        ux = (R)p.ux[node];
        uy = (R)p.uy[node];
        uz = (R)p.uz[node];
    } else {
        const R inv = (R)1 / rho;
        ux = jx * inv + (R)p.gshift;
        uy = zero_v ? (R)0 : jy * inv;
        uz = jz * inv;
        if (p.write_macro) {
            p.rho[node] = (float)rho;
            p.ux[node] = (float)ux;
            p.uy[node] = (float)uy;
            p.uz[node] = (float)uz;
        }
        if (PHYS && (w & W_SPECIAL) && p.bc_macro) {
            const int sl = __ldg(p.slot + node);
            if (__ldg(p.bc_kind + sl) & BCK_HE) {
                double *st = p.bc_macro + 4 * sl;
                st[0] = (double)rho;
                st[1] = (double)ux;
                st[2] = (double)uy;
                st[3] = (double)uz;
            }
        }
    }

    collide<Q, COLL, ST, PHYS>(f, rho, ux, uy, uz, p);
}

// Populations of a fluid node after streaming: pulled from x - c_d, or
// across a blocked link the node's own population (opp(d) for half-way
// bounce-back, d itself in the reference's wall model).  `in` points at the
// node's own element of direction 0.
template <int Q, int ST, bool PHYS, bool WRAP, class G, int HINT, bool PRED>
__device__ __forceinline__ void gather_node(const StepParams &p, const G &g, int x, int y, int z, uint32_t w,
                                            const typename Store<ST>::T *in, typename Store<ST>::R (&f)[Q]) {
    using S = Store<ST>;
    using T = typename S::T;
    using L = Lat<Q>;
    // Pull offsets to the six face neighbours.  With WRAP, coordinates wrap
    // and links that must not wrap are blocked in the flag word, so a wrapped
    // address is only read where the lattice is periodic.
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

    f[0] = S::decode(ld_pop<HINT>(in), p.shift[0], p.inv_scale);
#pragma unroll
    for (int d = 1; d < Q; ++d) {
        const int pull = d * g.nx + (L::cx(d) == 1 ? oxm : (L::cx(d) == -1 ? oxp : 0)) +
                         (L::cy(d) == 1 ? oym : (L::cy(d) == -1 ? oyp : 0)) +
                         (L::cz(d) == 1 ? ozm : (L::cz(d) == -1 ? ozp : 0));
        // across a blocked link: the node's own population, opp(d) for
        // half-way bounce-back, d itself in the reference's wall model
        const int own = (PHYS ? L::opp(d) : d) * g.nx;
        const bool blocked = (w >> d) & 1u;
        T v;
        if (PRED) {
            if (blocked) v = ld_pop<HINT>(in + own);
            else v = ld_pop<HINT>(in + pull);
        } else {
            v = ld_pop<HINT>(in + (blocked ? own : pull));
        }
        f[d] = S::decode(v, p.shift[d], p.inv_scale);
    }
}

// One node of the fused step.  WRAP: coordinates wrap at the lattice faces
// (periodic lattices, or any out-of-domain link left open); without it the
// pull offsets are constants and every out-of-domain link must be blocked.
// HINT: population load form (ld_pop).  PRED: a blocked link is read by a
// second, predicated load instead of a selected address.
template <int Q, int COLL, int ST, bool PHYS, bool WRAP, class G, int HINT = 0, bool PRED = false>
__device__ __forceinline__ void step_node(const StepParams &p, const G &g, int x, int y, int z) {
    using S = Store<ST>;
    using T = typename S::T;
    using R = typename S::R;
    using L = Lat<Q>;
    const bool in_row = x < g.nx;
    const int row = y + g.ny * z;
    const int node = x + g.nx * row;    // flag words and macroscopic fields
    const long long idx = x + (long long)g.pitch * row;  // populations
    const uint32_t w = in_row ? __ldg(p.word + node) : 0u;
    const bool fluid = (w & W_FLUID) != 0;
    // Every population of the node is at a fixed offset from these bases.
    const T *in = (const T *)p.fin[0] + idx;
    T *out = (T *)p.fout[0] + idx;
    // Solid lanes of a warp that also holds fluid nodes store the zero
    // encoding, so the warp's stores cover whole 32-byte sectors instead of
    // forcing a read-modify-write of partly written ones in L2/DRAM.
    const unsigned warp_fluid = __ballot_sync(0xffffffffu, fluid);
    if (!fluid) {
        if (in_row && warp_fluid) {
#pragma unroll
            for (int d = 0; d < Q; ++d) out[d * g.nx] = S::encode((R)0, p.shift[d], p.scale);
        }
        return;
    }

    typename Store<ST>::R f[Q];
    gather_node<Q, ST, PHYS, WRAP, G, HINT, PRED>(p, g, x, y, z, w, in, f);

    update_node<Q, COLL, ST, PHYS, WRAP, G>(f, w, node, p, g);

#pragma unroll
    for (int d = 0; d < Q; ++d) S::store(out + d * g.nx, f[d], p.shift[d], p.scale);
}

template <int Q, int COLL, int ST, bool PHYS>
__global__ void __launch_bounds__(STEP_BLOCK) step_kernel(const StepParams p) {
    const DynGeom g{p.nx, p.ny, p.nz, p.pitch};
    step_node<Q, COLL, ST, PHYS, true>(p, g, blockIdx.x * blockDim.x + threadIdx.x, blockIdx.y, blockIdx.z);
}

// The same step with the lattice extents fixed at compile time: built at run
// time for one lattice (lbm_jit.cpp), so pull, bounce-back and store offsets
// are immediates of the loads and stores.
// BLOCK threads along x, HINT and PRED as in step_node: the knobs the
// autotuner (lbm_autotune) chooses among.
// MINB: minimum resident blocks per SM asked of the register allocator (1 =
// no constraint).
template <int Q, int COLL, int ST, bool PHYS, bool WRAP, int NX, int NY, int NZ, int BLOCK, int HINT, bool PRED,
          int MINB>
__global__ void __launch_bounds__(BLOCK, MINB) step_kernel_fixed(const StepParams p) {
    const FixedGeom<NX, NY, NZ, Q * NX> g;
    step_node<Q, COLL, ST, PHYS, WRAP, FixedGeom<NX, NY, NZ, Q * NX>, HINT, PRED>(
        p, g, blockIdx.x * blockDim.x + threadIdx.x, blockIdx.y, blockIdx.z);
}

// The reference's L2 residual (computeResidual2D/3D, ComputeResiduals.cu:13-26):
// sqrt of the sum over all populations of (f - fColl)^2, f the post-stream,
// post-boundary field and fColl the post-collision field it streams from.
// The state between steps is fColl, so this recomputes f (the next step's
// gather and boundary conditions, no collision) and sums per block in FP64;
// solid nodes contribute 0 as in the reference, which writes neither array
// there.
template <int Q, int ST, bool PHYS>
__global__ void __launch_bounds__(STEP_BLOCK) resid_l2_kernel(const StepParams p, double *partial) {
    using S = Store<ST>;
    using T = typename S::T;
    using R = typename S::R;
    const DynGeom g{p.nx, p.ny, p.nz, p.pitch};
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, z = blockIdx.z;
    double acc = 0.0;
    if (x < g.nx) {
        const int row = y + g.ny * z;
        const int node = x + g.nx * row;
        const uint32_t w = __ldg(p.word + node);
        if (w & W_FLUID) {
            const T *in = (const T *)p.fin[0] + (x + (long long)g.pitch * row);
            R f[Q];
            gather_node<Q, ST, PHYS, true, DynGeom, 0, false>(p, g, x, y, z, w, in, f);
            bool keep, zv;
            apply_bc<Q, ST, PHYS, true, DynGeom>(f, w, node, p, g, keep, zv);
#pragma unroll
            for (int d = 0; d < Q; ++d) {
                const double df = (double)f[d] - (double)S::decode(in[d * g.nx], p.shift[d], p.inv_scale);
                acc += df * df;
            }
        }
    }
    __shared__ double sm[STEP_BLOCK / 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int k = 0; k < STEP_BLOCK / 32; ++k) t += sm[k];
        partial[blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * (size_t)blockIdx.z)] = t;
    }
}

// Force on the solid nodes inside a box by momentum exchange (physics mode,
// half-way bounce-back): every blocked link of a fluid node x whose solid
// neighbour x - c_d lies in the box carries 2 c_opp(d) f*_opp(d)(x) to the
// wall per step, f* the post-collision state.  Per-block FP64 partials of the
// three components, stored component-major.
template <int Q, int ST>
__global__ void __launch_bounds__(STEP_BLOCK) momentum_exchange_kernel(const StepParams p, int4 lo, int4 hi,
                                                                        double *partial, long long nb) {
    using S = Store<ST>;
    using T = typename S::T;
    using L = Lat<Q>;
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, z = blockIdx.z;
    double F[3] = {0, 0, 0};
    if (x < p.nx) {
        const int row = y + p.ny * z;
        const uint32_t w = __ldg(p.word + x + p.nx * row);
        if ((w & W_FLUID) && (w & 0x7FFFEu)) {
            const T *in = (const T *)p.fin[0] + (x + (long long)p.pitch * row);
#pragma unroll
            for (int d = 1; d < Q; ++d) {
                if (!((w >> d) & 1u)) continue;
                const int sx = x - L::cx(d), sy = y - L::cy(d), sz = z - L::cz(d);
                if (sx < lo.x || sx > hi.x || sy < lo.y || sy > hi.y || sz < lo.z || sz > hi.z) continue;
                if (sx < 0 || sx >= p.nx || sy < 0 || sy >= p.ny || sz < 0 || sz >= p.nz) continue;
                const int o = L::opp(d);
                const double fo = S::decode64(in[o * p.nx], p.shift[o], p.inv_scale);
                F[0] += 2.0 * L::cx(o) * fo;
                F[1] += 2.0 * L::cy(o) * fo;
                F[2] += 2.0 * L::cz(o) * fo;
            }
        }
    }
    __shared__ double sm[3][STEP_BLOCK / 32];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        double v = F[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0) sm[k][threadIdx.x >> 5] = v;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double t = 0.0;
        for (int k = 0; k < STEP_BLOCK / 32; ++k) t += sm[threadIdx.x][k];
        partial[threadIdx.x * nb + blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * (size_t)blockIdx.z)] = t;
    }
}

// The reference's FdRelDiff residual (gpu_NewResidual, ComputeResiduals.cu:
// 56-64): per population of a fluid node, |f - f_prev| / |f_first|, f the
// post-stream, post-boundary field the next step pulls (as for the L2
// residual), f_prev and f_first snapshots in the reference's SoA order
// (d * N + node).  first = 1 records f in both snapshots.  Per block: the
// maximum (entries with f_first = 0 skipped) and the count of non-finite
// values, stored at partial[b] and partial[nb + b].
template <int Q, int ST, bool PHYS>
__global__ void __launch_bounds__(STEP_BLOCK) fd_rel_kernel(const StepParams p, float *fprev, float *ffirst,
                                                            int first, double *partial, long long nb) {
    using S = Store<ST>;
    using T = typename S::T;
    using R = typename S::R;
    const DynGeom g{p.nx, p.ny, p.nz, p.pitch};
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, z = blockIdx.z;
    const long long N = (long long)g.nx * g.ny * g.nz;
    double mx = 0.0, bad = 0.0;
    if (x < g.nx) {
        const int row = y + g.ny * z;
        const int node = x + g.nx * row;
        const uint32_t w = __ldg(p.word + node);
        if (w & W_FLUID) {
            const T *in = (const T *)p.fin[0] + (x + (long long)g.pitch * row);
            R f[Q];
            gather_node<Q, ST, PHYS, true, DynGeom, 0, false>(p, g, x, y, z, w, in, f);
            bool keep, zv;
            apply_bc<Q, ST, PHYS, true, DynGeom>(f, w, node, p, g, keep, zv);
#pragma unroll
            for (int d = 0; d < Q; ++d) {
                const long long i = d * N + node;
                const float fv = (float)f[d];
                if (first) {
                    ffirst[i] = fv;
                } else {
                    const double den = fabs((double)ffirst[i]);
                    const double rel = fabs((double)fv - (double)fprev[i]) / den;
                    if (!isfinite((double)fv)) bad += 1.0;
                    else if (den > 0.0 && rel > mx) mx = rel;
                }
                fprev[i] = fv;
            }
        }
    }
    __shared__ double sm[2][STEP_BLOCK / 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        mx = fmax(mx, __shfl_down_sync(0xffffffffu, mx, o));
        bad += __shfl_down_sync(0xffffffffu, bad, o);
    }
    if ((threadIdx.x & 31) == 0) {
        sm[0][threadIdx.x >> 5] = mx;
        sm[1][threadIdx.x >> 5] = bad;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double m = 0.0, b = 0.0;
        for (int k = 0; k < STEP_BLOCK / 32; ++k) {
            m = fmax(m, sm[0][k]);
            b += sm[1][k];
        }
        const size_t blk = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * (size_t)blockIdx.z);
        partial[blk] = m;
        partial[nb + blk] = b;
    }
}

// Maximum of n partials into out[0], sum of the next n into out[1].
static __global__ void __launch_bounds__(1024) max_partials_kernel(const double *partial, long long n, double *out) {
    __shared__ double sm[2][1024];
    double m = 0.0, b = 0.0;
    for (long long i = threadIdx.x; i < n; i += 1024) {
        m = fmax(m, partial[i]);
        b += partial[n + i];
    }
    sm[0][threadIdx.x] = m;
    sm[1][threadIdx.x] = b;
    __syncthreads();
    for (int s = 512; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            sm[0][threadIdx.x] = fmax(sm[0][threadIdx.x], sm[0][threadIdx.x + s]);
            sm[1][threadIdx.x] += sm[1][threadIdx.x + s];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[0] = sm[0][0];
        out[1] = sm[1][0];
    }
}

// Deterministic sum of n partials (one block of 1024 threads, fixed order).
static __global__ void __launch_bounds__(1024) sum_partials_kernel(const double *partial, long long n, double *out) {
    __shared__ double sm[1024];
    double t = 0.0;
    for (long long i = threadIdx.x; i < n; i += 1024) t += partial[i];
    sm[threadIdx.x] = t;
    __syncthreads();
    for (int s = 512; s > 0; s >>= 1) {
        if (threadIdx.x < s) sm[threadIdx.x] += sm[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = sm[0];
}

// First post-collision field: f0 = 0 (the reference's start, Iterate.cu:244)
// or f0 = f_eq(rho0, u0), collided with rho0, u0 read from the macro arrays.
// Solid nodes get f = 0 in both buffers, which is what a fluid node pulls
// from a solid neighbour when no boundary link blocks it (the reference never
// writes solid nodes).
template <int Q, int COLL, int ST, bool PHYS>
__global__ void __launch_bounds__(STEP_BLOCK) init_kernel(const StepParams p, const StepParams other,
                                                          int equilibrium_start) {
    using S = Store<ST>;
    using T = typename S::T;
    using R = typename S::R;
    using L = Lat<Q>;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= p.nx) return;
    const int row = blockIdx.y + p.ny * blockIdx.z;
    const int node = x + p.nx * row;
    const long long idx = x + (long long)p.pitch * row;
    const uint32_t w = p.word[node];
    if (!(w & W_FLUID)) {
#pragma unroll
        for (int d = 0; d < Q; ++d) {
            ((T *)p.fout[d])[idx] = S::encode((R)0, p.shift[d], p.scale);
            ((T *)other.fout[d])[idx] = S::encode((R)0, p.shift[d], p.scale);
        }
        return;
    }
    const int m = p.init_from_arrays;
    const R rho = (m & 1) ? (R)p.rho[node] : (R)p.init_rho;
    const R ux = (m & 2) ? (R)p.ux[node] : (R)p.init_ux;
    const R uy = (m & 4) ? (R)p.uy[node] : (R)p.init_uy;
    const R uz = (m & 8) ? (R)p.uz[node] : (R)p.init_uz;
    R f[Q];
    const R usq15 = (R)1.5 * (ux * ux + uy * uy + uz * uz);
#pragma unroll
    for (int d = 0; d < Q; ++d) f[d] = equilibrium_start ? feq<Q, R>(d, rho, ux, uy, uz, usq15) : (R)0;
    collide<Q, COLL, ST, PHYS>(f, rho, ux, uy, uz, p);
#pragma unroll
    for (int d = 0; d < Q; ++d) {
        S::store((T *)p.fout[d] + idx, f[d], p.shift[d], p.scale);
        // The other buffer's fluid entries are overwritten by the first step
        // before anything reads them; give them the same finite values.
        S::store((T *)other.fout[d] + idx, f[d], p.shift[d], p.scale);
    }
}

// Decode a population field to double in the reference's SoA order
// out[d*n + node] (host read-back of the state).
template <int Q, int ST>
__global__ void decode_kernel(const StepParams p, double *out, long long n) {
    using S = Store<ST>;
    using T = typename S::T;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const long long idx = i % p.nx + (long long)p.pitch * (i / p.nx);
#pragma unroll
    for (int d = 0; d < Q; ++d)
        out[d * n + i] = S::decode64(((const T *)p.fin[d])[idx], p.shift[d], p.inv_scale);
}

// The inverse of decode_kernel: a population field in the reference's SoA
// order, in[d*n + node], encoded into the buffer the next step reads.
template <int Q, int ST>
__global__ void encode_kernel(const StepParams p, const double *in, long long n) {
    using S = Store<ST>;
    using T = typename S::T;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const long long idx = i % p.nx + (long long)p.pitch * (i / p.nx);
#pragma unroll
    for (int d = 0; d < Q; ++d) ((T *)p.fin[d])[idx] = S::encode64(in[d * n + i], p.shift[d], p.scale);
}

}  // namespace lbm

