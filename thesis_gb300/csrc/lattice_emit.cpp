// Lattice emitters for the geometries the reference generator cannot mesh:
// a duct packed with random spheres, a 2D channel with circular and
// rectangular obstacles, and lid-driven cavities.  Each writes the Node and
// BC files in the reference's formats (3D: G/main.cpp:56-66 node lines and
// G/FluidTracking.cpp:229-236 BC lines; 2D: the layout readNodeFile and
// readConnFile read, S/FilesReading.cu:270-347), so a run reads its lattice
// the way the reference's solver does.
//
// Random geometry comes from SplitMix64 (Steele, Lea and Flood, "Fast
// splittable pseudorandom number generators", OOPSLA 2014), uniform doubles
// from its top 53 bits; thesis_gb300/lattice.py draws the same sequence, so
// the files and the Python builders give the same lattice for a seed.  All
// geometric tests are evaluated in the same order as there (the library's
// host code is built without floating-point contraction).
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "thesis_lbm.h"
#include "thesis_lbm_io.h"

namespace {

thread_local std::string g_emit_error;

int emit_fail(int code, const std::string &m) {
    g_emit_error = m;
    return code;
}

struct SplitMix64 {
    unsigned long long s;
    explicit SplitMix64(unsigned long long seed) : s(seed) {}
    unsigned long long next() {
        s += 0x9E3779B97F4A7C15ull;
        unsigned long long z = s;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uniform() { return (double)(next() >> 11) * 0x1.0p-53; }
    double uniform(double lo, double hi) { return lo + (hi - lo) * uniform(); }
};

const int CX2[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1};
const int CY2[9] = {0, 0, 1, 0, -1, 1, 1, -1, -1};
const int CX3[19] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0};
const int CY3[19] = {0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1};
const int CZ3[19] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1};

struct BcLine {
    int i, j, k, dir, type;
};

// Links of fluid nodes that leave the domain: face_type[2*axis + side] is the
// BC type of a link leaving through that face (0: none); a link leaving
// through several faces takes the first non-zero type in the order x-, x+,
// y-, y+, z-, z+.  Node-major, directions ascending.
std::vector<BcLine> boundary_links(int dims, int n, int m, int h, const std::vector<unsigned char> &fluid,
                                   const int face_type[6]) {
    std::vector<BcLine> out;
    const int q = dims == 2 ? 9 : 19;
    for (int z = 0; z < h; ++z)
        for (int y = 0; y < m; ++y)
            for (int x = 0; x < n; ++x) {
                const bool edge = x == 0 || x == n - 1 || y == 0 || y == m - 1 || (dims == 3 && (z == 0 || z == h - 1));
                if (!edge || !fluid[(size_t)x + (size_t)n * (y + (size_t)m * z)]) continue;
                for (int d = 1; d < q; ++d) {
                    const int tx = x + (dims == 2 ? CX2[d] : CX3[d]), ty = y + (dims == 2 ? CY2[d] : CY3[d]);
                    const int tz = z + (dims == 2 ? 0 : CZ3[d]);
                    const bool out_x0 = tx < 0, out_x1 = tx > n - 1, out_y0 = ty < 0, out_y1 = ty > m - 1;
                    const bool out_z0 = tz < 0, out_z1 = tz > h - 1;
                    const bool leaves = out_x0 || out_x1 || out_y0 || out_y1 || out_z0 || out_z1;
                    if (!leaves) continue;
                    int t = 0;
                    const bool sel[6] = {out_x0, out_x1, out_y0, out_y1, out_z0, out_z1};
                    for (int f = 0; f < 6 && !t; ++f)
                        if (sel[f] && face_type[f]) t = face_type[f];
                    if (t > 0) out.push_back({x, y, z, d, t});
                }
            }
    return out;
}

// "%.6f" of index * delta for every index of an axis, formatted once.
std::vector<std::string> coord_strings(int count, double delta) {
    std::vector<std::string> s((size_t)count);
    char buf[64];
    for (int i = 0; i < count; ++i) {
        snprintf(buf, sizeof(buf), "%.6f", (double)i * delta);
        s[(size_t)i] = buf;
    }
    return s;
}

int write_files(int dims, int n, int m, int h, const std::vector<unsigned char> &fluid,
                const std::vector<BcLine> &bc, const char *node_path, const char *bc_path) {
    const double delta = 1.0 / (double)std::max(n - 1, 1);
    const std::vector<std::string> sx = coord_strings(n, delta), sy = coord_strings(m, delta),
                                   sz = coord_strings(h, delta);
    FILE *nf = fopen(node_path, "wb");
    if (!nf) return emit_fail(LBM_ERR_FILE, std::string("cannot write ") + node_path);
    std::string chunk;
    chunk.reserve(1 << 22);
    char num[32];
    for (int z = 0; z < h; ++z)
        for (int y = 0; y < m; ++y)
            for (int x = 0; x < n; ++x) {
                const int f = fluid[(size_t)x + (size_t)n * (y + (size_t)m * z)];
                if (dims == 2) {
                    snprintf(num, sizeof(num), "%d %d ", x, y);
                    chunk += num;
                    chunk += sx[(size_t)x];
                    chunk += ' ';
                    chunk += sy[(size_t)y];
                    chunk += f ? " 1\n" : " 0\n";
                } else {
                    snprintf(num, sizeof(num), "%d\t%d\t%d\t", x, y, z);
                    chunk += num;
                    chunk += sx[(size_t)x];
                    chunk += '\t';
                    chunk += sy[(size_t)y];
                    chunk += '\t';
                    chunk += sz[(size_t)z];
                    chunk += f ? "\t1\n" : "\t0\n";
                }
                if (chunk.size() > (1u << 22) - 256) {
                    fwrite(chunk.data(), 1, chunk.size(), nf);
                    chunk.clear();
                }
            }
    fwrite(chunk.data(), 1, chunk.size(), nf);
    const bool nf_ok = ferror(nf) == 0;
    fclose(nf);
    if (!nf_ok) return emit_fail(LBM_ERR_FILE, std::string("write failed: ") + node_path);
    FILE *bf = fopen(bc_path, "wb");
    if (!bf) return emit_fail(LBM_ERR_FILE, std::string("cannot write ") + bc_path);
    chunk.clear();
    for (const BcLine &b : bc) {
        if (dims == 2) {
            snprintf(num, sizeof(num), "%d %d %d %d ", b.i, b.j, b.dir, b.type);
            chunk += num;
            chunk += sx[(size_t)b.i];
            chunk += ' ';
            chunk += sy[(size_t)b.j];
            chunk += " 0\n";
        } else {
            snprintf(num, sizeof(num), "%d\t%d\t%d\t\t%d\t%d\t", b.i, b.j, b.k, b.dir, b.type);
            chunk += num;
            chunk += sx[(size_t)b.i];
            chunk += '\t';
            chunk += sy[(size_t)b.j];
            chunk += '\t';
            chunk += sz[(size_t)b.k];
            chunk += "\t0\n";
        }
        if (chunk.size() > (1u << 22) - 256) {
            fwrite(chunk.data(), 1, chunk.size(), bf);
            chunk.clear();
        }
    }
    fwrite(chunk.data(), 1, chunk.size(), bf);
    const bool bf_ok = ferror(bf) == 0;
    fclose(bf);
    if (!bf_ok) return emit_fail(LBM_ERR_FILE, std::string("write failed: ") + bc_path);
    return LBM_OK;
}

}  // namespace

extern "C" {

const char *lbm_emit_last_error(void) { return g_emit_error.c_str(); }

int lbm_pack_spheres(int n, int m, int h, double porosity, double rmin, double rmax, unsigned long long seed,
                     int margin_axis, double margin, long long max_attempts, unsigned char *solid,
                     double *spheres, long long max_spheres, long long *num_spheres) {
    if (n < 1 || m < 1 || h < 1 || !solid || margin_axis < 0 || margin_axis > 2 || !(rmax >= rmin) || !(rmin > 0))
        return emit_fail(LBM_ERR_INVALID, "lbm_pack_spheres: invalid argument");
    const size_t N = (size_t)n * m * h;
    memset(solid, 0, N);
    const double target = (1.0 - porosity) * (double)n * (double)m * (double)h;
    const double ext[3] = {(double)(n - 1), (double)(m - 1), (double)(h - 1)};
    std::vector<double> cx, cy, cz, rad;
    SplitMix64 rng(seed);
    long long solid_count = 0, attempts = 0;
    while ((double)solid_count < target && attempts < max_attempts) {
        ++attempts;
        const double r = rng.uniform(rmin, rmax);
        double c[3];
        c[0] = rng.uniform() * ext[0];
        c[1] = rng.uniform() * ext[1];
        c[2] = rng.uniform() * ext[2];
        const double lo = margin + r, hi = ext[margin_axis] - margin - r;
        c[margin_axis] = lo + rng.uniform() * std::max(hi - lo, 0.0);
        bool overlap = false;
        for (size_t s = 0; s < rad.size() && !overlap; ++s) {
            const double dx = cx[s] - c[0], dy = cy[s] - c[1], dz = cz[s] - c[2];
            const double d2 = dx * dx + dy * dy + dz * dz;
            const double rr = rad[s] + r;
            overlap = d2 < rr * rr;
        }
        if (overlap) continue;
        cx.push_back(c[0]);
        cy.push_back(c[1]);
        cz.push_back(c[2]);
        rad.push_back(r);
        const int x0 = std::max((int)floor(c[0] - r), 0), x1 = std::min((int)ceil(c[0] + r) + 1, n);
        const int y0 = std::max((int)floor(c[1] - r), 0), y1 = std::min((int)ceil(c[1] + r) + 1, m);
        const int z0 = std::max((int)floor(c[2] - r), 0), z1 = std::min((int)ceil(c[2] + r) + 1, h);
        const double r2 = r * r;
        for (int z = z0; z < z1; ++z)
            for (int y = y0; y < y1; ++y)
                for (int x = x0; x < x1; ++x) {
                    const double dx = (double)x - c[0], dy = (double)y - c[1], dz = (double)z - c[2];
                    if (dx * dx + dy * dy + dz * dz <= r2) {
                        unsigned char &s = solid[(size_t)x + (size_t)n * (y + (size_t)m * z)];
                        if (!s) {
                            s = 1;
                            ++solid_count;
                        }
                    }
                }
    }
    const long long k = (long long)rad.size();
    if (num_spheres) *num_spheres = k;
    if (spheres)
        for (long long s = 0; s < std::min(k, max_spheres); ++s) {
            spheres[4 * s] = cx[s];
            spheres[4 * s + 1] = cy[s];
            spheres[4 * s + 2] = cz[s];
            spheres[4 * s + 3] = rad[s];
        }
    return LBM_OK;
}

int lbm_emit_sphere_duct(int n, int m, int h, double porosity, double rmin, double rmax, unsigned long long seed,
                         const char *node_path, const char *bc_path, long long *num_spheres) {
    if (!node_path || !bc_path) return emit_fail(LBM_ERR_INVALID, "null path");
    if (n < 2 || m < 2 || h < 2) return emit_fail(LBM_ERR_INVALID, "lattice too small");
    std::vector<unsigned char> solid((size_t)n * m * h);
    int rc = lbm_pack_spheres(n, m, h, porosity, rmin, rmax, seed, 2, 2.0, 2000000, solid.data(), nullptr, 0,
                              num_spheres);
    if (rc) return rc;
    std::vector<unsigned char> fluid(solid.size());
    for (size_t i = 0; i < solid.size(); ++i) fluid[i] = solid[i] ? 0 : 1;
    // pressure faces: inlet z = 0, outlet z = h-1; the side faces and the
    // spheres are walls without BC lines (physics mode bounces back there)
    const int ft[6] = {0, 0, 0, 0, 2, 3};
    return write_files(3, n, m, h, fluid, boundary_links(3, n, m, h, fluid, ft), node_path, bc_path);
}

int lbm_emit_channel2d(int n, int m, unsigned long long seed, int n_obstacles, double size_scale,
                       const char *node_path, const char *bc_path) {
    if (!node_path || !bc_path) return emit_fail(LBM_ERR_INVALID, "null path");
    if (n < 8 || m < 12) return emit_fail(LBM_ERR_INVALID, "channel too small");
    SplitMix64 rng(seed);
    int k = n_obstacles;
    if (k < 0) k = 1 + std::min((int)(rng.uniform() * 6.0), 5);
    std::vector<unsigned char> solid((size_t)n * m, 0);
    std::vector<double> boxes;  // x0, y0, x1, y1
    int placed = 0, tries = 0;
    const double s = size_scale;
    while (placed < k && tries < 10000) {
        ++tries;
        const double rmax = std::min(std::min(32.0 * s, (m - 8) / 2.0), n * 0.3);
        const double smax = std::min(std::min(60.0 * s, m - 8.0), n * 0.5);
        double bb[4];
        bool circle;
        double ccx = 0, ccy = 0, cr = 0, rx = 0, ry = 0, rw = 0, rh = 0;
        if (rng.uniform() < 0.5) {
            circle = true;
            cr = rng.uniform(std::min(8.0 * s, rmax), rmax);
            ccx = rng.uniform(n * 0.1 + cr, n * 0.85 - cr);
            ccy = rng.uniform(cr + 3, m - 4 - cr);
            bb[0] = ccx - cr;
            bb[1] = ccy - cr;
            bb[2] = ccx + cr;
            bb[3] = ccy + cr;
        } else {
            circle = false;
            rw = rng.uniform(std::min(10.0 * s, smax), smax);
            rh = rng.uniform(std::min(10.0 * s, smax), smax);
            rx = rng.uniform(n * 0.1, n * 0.85 - rw);
            ry = rng.uniform(3, m - 4 - rh);
            bb[0] = rx;
            bb[1] = ry;
            bb[2] = rx + rw;
            bb[3] = ry + rh;
        }
        bool clash = false;
        for (size_t b = 0; b < boxes.size() && !clash; b += 4) {
            const double *o = &boxes[b];
            clash = !(bb[2] + 2 < o[0] || o[2] + 2 < bb[0] || bb[3] + 2 < o[1] || o[3] + 2 < bb[1]);
        }
        if (clash) continue;
        boxes.insert(boxes.end(), bb, bb + 4);
        for (int y = 0; y < m; ++y)
            for (int x = 0; x < n; ++x) {
                bool in;
                if (circle) {
                    const double dx = (double)x - ccx, dy = (double)y - ccy;
                    in = dx * dx + dy * dy <= cr * cr;
                } else {
                    in = (double)x >= rx && (double)x <= rx + rw && (double)y >= ry && (double)y <= ry + rh;
                }
                if (in) solid[(size_t)x + (size_t)n * y] = 1;
            }
        ++placed;
    }
    std::vector<unsigned char> fluid(solid.size());
    for (size_t i = 0; i < solid.size(); ++i) fluid[i] = solid[i] ? 0 : 1;
    // inlet x = 0, outlet x = n-1, walls y = 0 and y = m-1
    const int ft[6] = {2, 3, 1, 1, 0, 0};
    return write_files(2, n, m, 1, fluid, boundary_links(2, n, m, 1, fluid, ft), node_path, bc_path);
}

int lbm_emit_cavity(int dims, int n, int m, int h, const char *node_path, const char *bc_path) {
    if (!node_path || !bc_path) return emit_fail(LBM_ERR_INVALID, "null path");
    if ((dims != 2 && dims != 3) || n < 2 || m < 2 || (dims == 3 && h < 2))
        return emit_fail(LBM_ERR_INVALID, "lbm_emit_cavity: invalid lattice");
    if (dims == 2) h = 1;
    std::vector<unsigned char> fluid((size_t)n * m * h, 1);
    // walls everywhere, the lid (y = m-1 in 2D, z = h-1 in 3D) an inlet
    int ft[6] = {1, 1, 1, 1, 1, 1};
    if (dims == 2) ft[3] = 2;
    else ft[5] = 2;
    return write_files(dims, n, m, h, fluid, boundary_links(dims, n, m, h, fluid, ft), node_path, bc_path);
}

}  // extern "C"
