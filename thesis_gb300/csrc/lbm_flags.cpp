// Host-side lattice set-up: the reference's boundary masks and streaming flags
// and, from them, this engine's per-node flag words and boundary slots.
//
// Reference masks (restated from GpuInit.cu:1055-1122 and :1157-1238):
//   per BC link (node, dir, type):
//     mask |= type << (dir-1)*B             (B = 2 bits in 2D, 3 in 3D)
//     mask |= fluid << F                    (F = 19 / 58)
//     main type (bits 16 / 54): set to type if unset; if a different type was
//       set, main := WALL and the CORNER bit (18 / 57) is set
//     2D: mask |= boundary id << 24
//     stream flag of direction opp(dir) cleared
//   corner pass: 2D -- a corner node's diagonal links between two typed faces
//     become walls (NE, NW, SW, SE); 3D -- every typed link becomes a wall.
#include "lbm_flags.h"

#include <string.h>

#include <algorithm>

#include <thread>

namespace lbm {

namespace {
const int CX2[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1};
const int CY2[9] = {0, 0, 1, 0, -1, 1, 1, -1, -1};
const int OPP2[9] = {0, 3, 4, 1, 2, 7, 8, 5, 6};
const int CX3[19] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0};
const int CY3[19] = {0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1};
const int CZ3[19] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1};
const int OPP3[19] = {0, 2, 1, 4, 3, 6, 5, 10, 9, 8, 7, 14, 13, 12, 11, 18, 17, 16, 15};
}  // namespace

int lattice_cx(int q, int d) { return q == 9 ? CX2[d] : CX3[d]; }
int lattice_cy(int q, int d) { return q == 9 ? CY2[d] : CY3[d]; }
int lattice_cz(int q, int d) { return q == 9 ? 0 : CZ3[d]; }
int lattice_opp(int q, int d) { return q == 9 ? OPP2[d] : OPP3[d]; }

uint64_t ref_type(const RefMasks &r, size_t b, int dir) {
    const int bits = r.q == 9 ? 2 : 3;
    return (r.mask[b] >> ((dir - 1) * bits)) & (r.q == 9 ? 3ull : 7ull);
}

uint64_t ref_main_type(const RefMasks &r, size_t b) {
    return r.q == 9 ? (r.mask[b] >> 16) & 3ull : (r.mask[b] >> 54) & 7ull;
}

bool ref_corner(const RefMasks &r, size_t b) {
    return r.q == 9 ? (r.mask[b] >> 18) & 1ull : (r.mask[b] >> 57) & 1ull;
}

long long find_bc(const RefMasks &r, long long node) {
    auto it = std::lower_bound(r.bc_nodes.begin(), r.bc_nodes.end(), node);
    return it != r.bc_nodes.end() && *it == node ? (long long)(it - r.bc_nodes.begin()) : -1;
}

int build_ref_masks(const lbm_lattice_desc &L, RefMasks &r, std::string &err) {
    const int q = L.dims == 2 ? 9 : 19;
    const int h = L.dims == 2 ? 1 : L.h;
    const int nc = L.num_conns > 0 ? L.num_conns : 0;
    r.q = q;
    r.bc_nodes.clear();
    r.mask.clear();
    r.blocked.clear();
    r.linked.clear();
    // node of every link; the links of one node are combined below, so they
    // are visited node by node (BC files list them node-major already)
    std::vector<long long> li((size_t)nc);
    bool sorted = true;
    for (int c = 0; c < nc; ++c) {
        const int i = L.bc_i[c], j = L.bc_j[c], k = L.bc_k ? L.bc_k[c] : 0;
        const int dir = L.bc_dir[c];
        if (i < 0 || i >= L.n || j < 0 || j >= L.m || k < 0 || k >= h || dir < 1 || dir >= q) {
            err = "BC link " + std::to_string(c) + " out of range";
            return LBM_ERR_INVALID;
        }
        li[(size_t)c] = i + (long long)L.n * (j + (long long)L.m * k);
        if (c && li[(size_t)c] < li[(size_t)c - 1]) sorted = false;
    }
    std::vector<int> order((size_t)nc);
    for (int c = 0; c < nc; ++c) order[(size_t)c] = c;
    if (!sorted)
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return li[(size_t)a] < li[(size_t)b]; });
    for (size_t t = 0; t < (size_t)nc;) {
        const long long ind = li[(size_t)order[t]];
        const uint64_t fluid = (uint64_t)(L.node_type[ind] & 1);
        uint64_t mk = 0;
        uint32_t blocked = 0, linked = 0;
        for (; t < (size_t)nc && li[(size_t)order[t]] == ind; ++t) {
            const int c = order[t];
            const int dir = L.bc_dir[c];
            const uint64_t type = (uint64_t)L.bc_type[c];
            if (q == 9) {
                mk |= type << ((dir - 1) * 2);
                mk |= fluid << 19;
                const uint64_t all = 3ull << 16;
                if (!(mk & all)) {
                    mk |= type << 16;
                } else if ((mk & all) != (type << 16)) {
                    mk &= ~all;
                    mk |= 1ull << 16;
                    mk |= 1ull << 18;
                }
                const uint32_t id = L.bc_id ? (uint32_t)L.bc_id[c] : 0u;
                mk = (uint64_t)((uint32_t)mk | (id << 24));
            } else {
                mk |= type << ((dir - 1) * 3);
                mk |= fluid << 58;
                const uint64_t all = 7ull << 54;
                if (!(mk & all)) {
                    mk |= type << 54;
                } else if ((mk & all) != (type << 54)) {
                    mk &= ~all;
                    mk |= 1ull << 54;
                    mk |= 1ull << 57;
                }
            }
            blocked |= 1u << lattice_opp(q, dir);
            linked |= 1u << dir;
        }
        // corner pass
        if (q == 9) {
            if ((mk >> 18) & 1ull) {
                auto any = [&](int d) { return ((mk >> ((d - 1) * 2)) & 3ull) != 0; };
                auto wall = [&](int d) {
                    mk &= ~(3ull << ((d - 1) * 2));
                    mk |= 1ull << ((d - 1) * 2);
                };
                if (any(1) && any(2)) wall(5);
                if (any(3) && any(2)) wall(6);
                if (any(3) && any(4)) wall(7);
                if (any(1) && any(4)) wall(8);
            }
        } else if ((mk >> 57) & 1ull) {
            for (int d = 1; d < 19; ++d)
                if ((mk >> ((d - 1) * 3)) & 7ull) {
                    mk &= ~(7ull << ((d - 1) * 3));
                    mk |= 1ull << ((d - 1) * 3);
                }
        }
        r.bc_nodes.push_back(ind);
        r.mask.push_back(mk);
        r.blocked.push_back(blocked);
        r.linked.push_back(linked);
    }
    return LBM_OK;
}

// Face id (inward normal) of an axis link direction pointing out of the domain.
static int face_of_link(int q, int dir) {
    const int cx = lattice_cx(q, dir), cy = lattice_cy(q, dir), cz = lattice_cz(q, dir);
    if (cx == -1 && cy == 0 && cz == 0) return 0;  // link to x-: inward +x
    if (cx == 1 && cy == 0 && cz == 0) return 1;
    if (cy == -1 && cx == 0 && cz == 0) return 2;
    if (cy == 1 && cx == 0 && cz == 0) return 3;
    if (cz == -1 && cx == 0 && cy == 0) return 4;
    if (cz == 1 && cx == 0 && cy == 0) return 5;
    return -1;
}

bool curved_walls(const lbm_params &P, int q) {
    return P.mode != LBM_MODE_PHYSICS && P.boundary_type == LBM_CURVED &&
           !(q == 19 && P.bc_wall_model == LBM_WALL_COMPLEX);
}

bool one_node_boundaries(const lbm_params &P, int q) {
    const bool open_outlet = P.outlet_profile == LBM_OUTLET_SECOND || P.outlet_profile == LBM_OUTLET_FIRST ||
                             P.outlet_profile == LBM_OUTLET_HEMODEL;
    return curved_walls(P, q) || (q == 9 && P.mode != LBM_MODE_PHYSICS &&
                                  (P.outlet_profile == LBM_OUTLET_SECOND || P.outlet_profile == LBM_OUTLET_FIRST)) ||
           (P.mode == LBM_MODE_PHYSICS && open_outlet);
}

int build_device_flags(const lbm_lattice_desc &L, const lbm_params &P, const RefMasks &r,
                       DeviceFlags &out, std::string &err) {
    const int q = r.q;
    const int n = L.n, m = L.m, h = L.dims == 2 ? 1 : L.h;
    const long long N = (long long)n * m * h;
    const bool phys = P.mode == LBM_MODE_PHYSICS;
    out.word.resize((size_t)N);  // every entry written below
    out.slot.resize((size_t)N);
    out.mask.clear();
    out.kind.clear();
    out.slot_node.clear();

    if (P.boundary_type != LBM_CURVED && P.boundary_type != LBM_STRAIGHT) {
        err = "unknown boundary type";
        return LBM_ERR_INVALID;
    }
    if (P.boundary_type == LBM_CURVED && phys) {
        err = "curved (q-interpolated) walls are the reference's wall kernels; physics-mode walls are "
              "half-way bounce-back (use LBM_STRAIGHT)";
        return LBM_ERR_UNSUPPORTED;
    }
    if (P.bc_wall_model == LBM_WALL_COMPLEX && phys) {
        err = "the HH wall model is a reference-mode boundary; physics-mode walls are half-way bounce-back "
              "(use LBM_WALL_SIMPLE)";
        return LBM_ERR_UNSUPPORTED;
    }
    // reference 3D HH walls: every boundary node takes the wall kernel's
    // path (a node whose wall links match none of its face, edge and corner
    // cases keeps its streamed populations); the reference's 2D loop has
    // straight walls only (Iterate.cu), so there the model changes nothing
    const bool hh = !phys && q == 19 && P.bc_wall_model == LBM_WALL_COMPLEX;
    // reference curved walls (the simple wall kernels' CURVED branch; the HH
    // kernel has none): every node with a wall link takes the boundary path,
    // which interpolates between the node's own and upstream populations
    const bool curved = curved_walls(P, q);

    // fluid bit and blocked pulls, in parallel over node ranges; a range
    // walks the boundary-node list alongside
    const size_t nb = r.bc_nodes.size();
    int off[19];
    for (int d = 0; d < q; ++d)
        off[d] = lattice_cx(q, d) + n * lattice_cy(q, d) + n * m * lattice_cz(q, d);
    auto word_range = [&](long long lo, long long hi) {
        size_t b = (size_t)(std::lower_bound(r.bc_nodes.begin(), r.bc_nodes.end(), lo) - r.bc_nodes.begin());
        int x = (int)(lo % n), y = (int)((lo / n) % m), z = (int)(lo / ((long long)n * m));
        for (long long ind = lo; ind < hi; ++ind) {
            const bool isbc = b < nb && r.bc_nodes[b] == ind;
            const size_t bi = b;
            if (isbc) ++b;
            const int cx = x, cy = y, cz = z;
            if (++x == n) {
                x = 0;
                if (++y == m) {
                    y = 0;
                    ++z;
                }
            }
            out.slot[(size_t)ind] = -1;
            if (!(L.node_type[ind] & 1)) {
                out.word[(size_t)ind] = 0u;
                continue;
            }
            uint32_t w = W_FLUID | (isbc ? r.blocked[bi] : 0u);
            if (phys) {
                uint32_t bl = 0;
                const bool interior = cx > 0 && cx < n - 1 && cy > 0 && cy < m - 1 && (h == 1 || (cz > 0 && cz < h - 1));
                if (interior && !isbc) {
                    // no link leaves the lattice: only solid neighbours block
                    for (int d = 1; d < q; ++d)
                        if (!(L.node_type[ind - off[d]] & 1)) bl |= 1u << d;
                    out.word[(size_t)ind] = W_FLUID | bl;
                    continue;
                }
                for (int d = 1; d < q; ++d) {
                    const int opp = lattice_opp(q, d);
                    // a periodic-type link on the opposite direction streams by wrapping
                    const bool periodic_link =
                        isbc && ((r.linked[bi] >> opp) & 1u) && ref_type(r, bi, opp) == LBM_BC_PERIODIC;
                    if (((w >> d) & 1u) && !periodic_link) bl |= 1u << d;
                    int sx = cx - lattice_cx(q, d), sy = cy - lattice_cy(q, d), sz = cz - lattice_cz(q, d);
                    bool outside = false;
                    if (sx < 0 || sx >= n) { if (P.periodic[0] || periodic_link) sx = (sx + n) % n; else outside = true; }
                    if (sy < 0 || sy >= m) { if (P.periodic[1] || periodic_link) sy = (sy + m) % m; else outside = true; }
                    if (sz < 0 || sz >= h) { if (P.periodic[2] || periodic_link) sz = (sz + h) % h; else outside = true; }
                    if (outside) {
                        bl |= 1u << d;
                        continue;
                    }
                    const long long src = sx + (long long)n * (sy + (long long)m * sz);
                    if (!(L.node_type[src] & 1)) bl |= 1u << d;
                }
                w = W_FLUID | bl;
            }
            out.word[(size_t)ind] = w;
        }
    };
    {
        unsigned nt = std::thread::hardware_concurrency();
        nt = nt == 0 ? 1 : (nt > 32 ? 32 : nt);
        if (N < (1 << 16)) nt = 1;
        std::vector<std::thread> pool;
        const long long chunk = (N + nt - 1) / nt;
        for (unsigned t = 0; t < nt; ++t) {
            const long long lo = t * chunk, hi = lo + chunk < N ? lo + chunk : N;
            if (lo < hi) pool.emplace_back(word_range, lo, hi);
        }
        for (auto &th : pool) th.join();
    }

    // special nodes
    for (size_t node = 0; node < nb; ++node) {
        const long long ind = r.bc_nodes[node];
        if (!(L.node_type[ind] & 1)) continue;
        bool special = false;
        int kind = 0;
        if (!phys) {
            bool simple = !hh && !curved && ref_main_type(r, node) == LBM_BC_WALL;
            for (int d = 1; d < q && simple; ++d) {
                const uint64_t t = ref_type(r, node, d);
                const bool wall = t == LBM_BC_WALL;
                const bool blocked_opp = (r.blocked[node] >> lattice_opp(q, d)) & 1u;
                if (t > LBM_BC_WALL || wall != blocked_opp) simple = false;
            }
            special = !simple;
            if (special) {
                const uint64_t mt = ref_main_type(r, node);
                if (q == 19 && mt == LBM_BC_OUTLET) {
                    err = "the reference's 3D outlet kernel addresses populations with the 2D plane "
                          "size; 3D outlets are supported in physics mode only";
                    return LBM_ERR_UNSUPPORTED;
                }
                if (q == 9 && ref_type(r, node, 1) == LBM_BC_OUTLET &&
                    (P.outlet_profile < LBM_OUTLET_ZOUHE || P.outlet_profile > LBM_OUTLET_HEMODEL)) {
                    err = "unknown 2D outlet profile";
                    return LBM_ERR_INVALID;
                }
            }
        } else {
            if (ref_corner(r, node)) continue;  // mixed faces: walls only
            const uint64_t mt = ref_main_type(r, node);
            if (mt == LBM_BC_SYMMETRY) {
                err = "symmetry planes are supported in reference mode only";
                return LBM_ERR_UNSUPPORTED;
            }
            if (mt != LBM_BC_INLET && mt != LBM_BC_OUTLET) continue;
            int face = -1;
            for (int d = 1; d < q && face < 0; ++d)
                if (((r.linked[node] >> d) & 1u) && ref_type(r, node, d) == mt)
                    face = face_of_link(q, d);
            if (face < 0) continue;
            // a velocity inlet whose velocity has no component along the
            // face normal is a moving wall (a cavity lid): bounce-back plus
            // the wall's momentum on every inlet link conserves mass exactly,
            // where the Zou-He closure lets the mean density drift
            if (mt == LBM_BC_INLET && P.inlet_profile != LBM_INLET_PRESSURE) {
                const double nrm = face < 2 ? P.u : (face < 4 ? P.v : (q == 19 ? P.w : 0.0));
                if (nrm == 0.0) {
                    uint64_t moving = 0;
                    for (int d = 1; d < q; ++d)
                        if (((r.linked[node] >> d) & 1u) && ref_type(r, node, d) == LBM_BC_INLET)
                            moving |= 1ull << lattice_opp(q, d);
                    out.slot[(size_t)ind] = (int32_t)out.slot_node.size();
                    out.slot_node.push_back(ind);
                    out.mask.push_back(moving);
                    out.kind.push_back(face | BCK_ACTIVE | BCK_MOVING);
                    out.word[(size_t)ind] |= W_SPECIAL;
                    continue;
                }
            }
            kind = face | BCK_ACTIVE;
            if (mt == LBM_BC_INLET) {
                if (P.inlet_profile == LBM_INLET_PRESSURE) kind |= BCK_PRESSURE;
            } else {
                kind |= BCK_OUTLET;
                if (P.outlet_profile == LBM_OUTLET_PRESSURE)
                    kind |= BCK_PRESSURE;
                else if (P.outlet_profile == LBM_OUTLET_FIRST)
                    kind |= BCK_EXTRAP1;
                else if (P.outlet_profile == LBM_OUTLET_SECOND)
                    kind |= BCK_EXTRAP2;
                else if (P.outlet_profile == LBM_OUTLET_HEMODEL)
                    kind |= BCK_HE;
                else if (P.outlet_profile != LBM_OUTLET_ZOUHE) {
                    err = "unknown outlet profile";
                    return LBM_ERR_INVALID;
                }
            }
            special = true;
        }
        if (!special) continue;
        out.slot[(size_t)ind] = (int32_t)out.slot_node.size();
        out.slot_node.push_back(ind);
        out.mask.push_back(r.mask[node]);
        out.kind.push_back(kind);
        out.word[(size_t)ind] |= W_SPECIAL;
    }
    return LBM_OK;
}

}  // namespace lbm
