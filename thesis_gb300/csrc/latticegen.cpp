// Lattice generator: STAR-CD geometry (.vrt nodes + .bnd quadrilateral
// boundary faces) to the solver's Node and BC files, byte-identical to the
// reference generator (Source code/latticegen2_W8).
//
// Algorithm (steps and floating-point comparisons kept identical, because the
// output is specified bit for bit by the reference's golden files):
//   * faces: type from the .bnd keyword (WALL/INLE/OUTL/CYCL/SYMP -> 1..5),
//     plane 3 (all x equal), 2 (all y equal), 1 (all z equal) or 0 (sloped,
//     never intersected), bounding box of the four corners
//     (GeomRead.cpp:59-187);
//   * grid: delta = (xmax - xmin)/(n - 1), m = ceil(ydom/delta) + 1,
//     h = ceil(zdom/delta) + 1, one padding layer on every side, node
//     (i, j, k) at (xmin + delta (i-1), ...) (MeshGen.cpp:17-79);
//   * flood fill from the node nearest the seed over the 18 D3Q19 links, in
//     FIFO order; a link that crosses a face is a boundary link, written when
//     its far node is not yet fluid (FluidTracking.cpp:94-212).  The seed is
//     marked fluid in the node list but not in the fill matrix, so it can be
//     queued twice, as in the reference;
//   * a link crosses a face when the face plane, clipped to the face box and
//     the link's box, holds the crossing point, and that point is not the far
//     node (Intersect.cpp:43-527).  The crossing point is one persistent state
//     shared by all tests, so coordinates a test does not set keep the value an
//     earlier test left, exactly as the reference's member array does.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <fstream>
#include <string>
#include <vector>

#include "thesis_lbm.h"

namespace {

struct Face {
    double id;
    int p[4];
    int type;
    int plane;
    double xmax, xmin, ymax, ymin, zmax, zmin;
};

struct Geometry {
    std::vector<double> x, y, z;  // STAR-CD vertices, 1-based ids map to index id-1
    std::vector<Face> faces;
};

bool read_geometry(const std::string &vrt, const std::string &bnd, Geometry &g, std::string &err) {
    std::ifstream vf(vrt.c_str()), bf(bnd.c_str());
    if (!vf.is_open() || !bf.is_open()) {
        err = "cannot open " + vrt + " or " + bnd;
        return false;
    }
    int id;
    double cx, cy, cz;
    while (vf >> id >> cx >> cy >> cz) {
        g.x.push_back(cx);
        g.y.push_back(cy);
        g.z.push_back(cz);
    }
    int i1, p1, p2, p3, p4, bcid, i2;
    std::string kw;
    const int nv = (int)g.x.size();
    while (bf >> i1 >> p1 >> p2 >> p3 >> p4 >> bcid >> i2 >> kw) {
        Face f{};
        f.id = bcid;
        f.p[0] = p1;
        f.p[1] = p2;
        f.p[2] = p3;
        f.p[3] = p4;
        for (int k = 0; k < 4; ++k)
            if (f.p[k] < 1 || f.p[k] > nv) {
                err = "face vertex out of range in " + bnd;
                return false;
            }
        f.type = kw == "WALL" ? 1 : kw == "INLE" ? 2 : kw == "OUTL" ? 3 : kw == "CYCL" ? 4 : kw == "SYMP" ? 5 : 0;
        auto X = [&](int k) { return g.x[f.p[k] - 1]; };
        auto Y = [&](int k) { return g.y[f.p[k] - 1]; };
        auto Z = [&](int k) { return g.z[f.p[k] - 1]; };
        if (X(0) == X(1) && X(1) == X(2) && X(2) == X(3))
            f.plane = 3;
        else if (Y(0) == Y(1) && Y(1) == Y(2) && Y(2) == Y(3))
            f.plane = 2;
        else if (Z(0) == Z(1) && Z(1) == Z(2) && Z(2) == Z(3))
            f.plane = 1;
        else
            f.plane = 0;
        f.xmax = std::max(std::max(std::max(X(1), X(0)), X(2)), X(3));
        f.xmin = std::min(std::min(std::min(X(1), X(0)), X(2)), X(3));
        f.ymax = std::max(std::max(std::max(Y(1), Y(0)), Y(2)), Y(3));
        f.ymin = std::min(std::min(std::min(Y(1), Y(0)), Y(2)), Y(3));
        f.zmax = std::max(std::max(std::max(Z(1), Z(0)), Z(2)), Z(3));
        f.zmin = std::min(std::min(std::min(Z(1), Z(0)), Z(2)), Z(3));
        g.faces.push_back(f);
    }
    if (g.x.empty()) {
        err = "no vertices in " + vrt;
        return false;
    }
    return true;
}

// One link-versus-faces test with the crossing point kept between calls.
struct Crossing {
    const Geometry &g;
    double I[3] = {0, 0, 0};
    double hit[3] = {0, 0, 0};
    int type = -1, id = -1;
    explicit Crossing(const Geometry &geo) : g(geo) {}

    // second vertex of a face, the point the reference takes the plane from
    double vx(const Face &f) const { return g.x[f.p[1] - 1]; }
    double vy(const Face &f) const { return g.y[f.p[1] - 1]; }
    double vz(const Face &f) const { return g.z[f.p[1] - 1]; }

    bool record(const Face &f, const double *a, const double *b) {
        if ((I[0] != b[0] || a[0] == b[0]) && (I[1] != b[1] || a[1] == b[1]) && (I[2] != b[2] || a[2] == b[2])) {
            id = (int)f.id;
            type = f.type;
            hit[0] = I[0];
            hit[1] = I[1];
            hit[2] = I[2];
            return true;
        }
        return false;
    }

    bool test(const double *a, const double *b) {
        const double maxX = std::max(a[0], b[0]), minX = std::min(a[0], b[0]);
        const double maxY = std::max(a[1], b[1]), minY = std::min(a[1], b[1]);
        const double maxZ = std::max(a[2], b[2]), minZ = std::min(a[2], b[2]);
        for (const Face &f : g.faces) {
            if (a[1] == b[1] && a[0] == b[0]) {  // link along z
                if (f.plane != 3 && f.plane != 2) {
                    I[0] = a[0];
                    I[1] = a[1];
                    if (f.plane == 1) {
                        I[2] = vz(f);
                        if (I[2] <= maxZ && I[2] >= minZ && I[0] <= f.xmax && I[0] >= f.xmin &&
                            I[1] <= f.ymax && I[1] >= f.ymin && record(f, a, b))
                            return true;
                    }
                }
            }
            if (a[1] == b[1] && a[2] == b[2]) {  // link along x
                if (f.plane != 1 && f.plane != 2) {
                    I[2] = a[2];
                    I[1] = a[1];
                    if (f.plane == 3) {
                        I[0] = vx(f);
                        if (I[0] <= maxX && I[0] >= minX && I[1] <= f.ymax && I[1] >= f.ymin &&
                            I[2] <= f.zmax && I[2] >= f.zmin && record(f, a, b))
                            return true;
                    }
                }
            }
            if (a[0] == b[0] && a[2] == b[2]) {  // link along y
                if (f.plane != 1 && f.plane != 3) {
                    I[2] = a[2];
                    I[0] = a[0];
                    if (f.plane == 2) {
                        I[1] = vy(f);
                        if (I[1] <= maxY && I[1] >= minY && I[0] <= f.xmax && I[0] >= f.xmin &&
                            I[2] <= f.zmax && I[2] >= f.zmin && record(f, a, b))
                            return true;
                    }
                }
            }
            if (a[0] != b[0] && a[1] != b[1] && a[2] == b[2]) {  // diagonal in the xy plane
                if (f.plane != 1) {
                    if (f.plane == 2) {
                        I[2] = a[2];
                        if (b[0] >= a[0] && b[0] < f.xmax)
                            I[0] = a[0] + fabs(vy(f) - a[1]);
                        else if (b[0] < a[0] && b[0] >= f.xmin)
                            I[0] = a[0] - fabs(vy(f) - a[1]);
                        if (a[1] <= f.ymax && a[0] >= f.xmin && a[1] == f.ymax) I[0] = a[0];
                        I[1] = vy(f);
                        if (I[0] <= maxX && I[0] >= minX && I[1] <= maxY && I[1] >= minY &&
                            I[2] <= f.zmax && I[2] >= f.zmin && record(f, a, b))
                            return true;
                    } else if (f.plane == 3) {
                        I[2] = a[2];
                        if (b[1] > a[1] && b[1] <= f.ymax)
                            I[1] = a[1] + fabs(vx(f) - a[0]);
                        else if (b[1] < a[1] && b[1] >= f.ymin)
                            I[1] = a[1] - fabs(vx(f) - a[0]);
                        if (a[1] <= f.ymax && a[1] >= f.ymin && a[0] == f.xmax) I[1] = a[1];
                        I[0] = vx(f);
                        if (I[0] <= maxX && I[0] >= minX && I[1] <= maxY && I[1] >= minY &&
                            I[2] <= f.zmax && I[2] >= f.zmin && record(f, a, b))
                            return true;
                    }
                }
            }
            if (a[0] != b[0] && a[2] != b[2] && a[1] == b[1]) {  // diagonal in the xz plane
                if (f.plane != 2) {
                    if (f.plane == 1) {
                        I[1] = a[1];
                        if (b[0] > a[0] && b[0] <= f.xmax)
                            I[0] = a[0] + fabs(vz(f) - a[2]);
                        else if (b[0] < a[0] && b[0] >= f.xmin)
                            I[0] = a[0] - fabs(vz(f) - a[2]);
                        if (a[0] <= f.xmax && a[0] >= f.xmin && a[2] == f.zmax) I[0] = a[0];
                        I[2] = vz(f);
                        if (I[0] <= maxX && I[0] >= minX && I[2] <= maxZ && I[2] >= minZ &&
                            I[1] <= f.ymax && I[1] >= f.ymin && record(f, a, b))
                            return true;
                    } else if (f.plane == 3) {
                        I[1] = a[1];
                        if (b[2] > a[2] && b[2] <= f.zmax)
                            I[2] = a[2] + fabs(vx(f) - a[0]);
                        else if (b[2] < a[2] && b[2] >= f.zmin)
                            I[2] = a[2] - fabs(vx(f) - a[0]);
                        if (a[2] <= f.zmax && a[2] >= f.zmin && a[0] == f.xmax) I[2] = a[2];
                        I[0] = vx(f);
                        if (I[0] <= maxX && I[0] >= minX && I[2] <= maxZ && I[2] >= minZ &&
                            I[1] <= f.ymax && I[1] >= f.ymin && record(f, a, b))
                            return true;
                    }
                }
            }
            if (a[2] != b[2] && a[1] != b[1] && a[0] == b[0]) {  // diagonal in the yz plane
                if (f.plane != 3) {
                    if (f.plane == 1) {
                        I[0] = a[0];
                        if (b[1] > a[1] && b[1] <= f.ymax)
                            I[1] = a[1] + fabs(vz(f) - a[2]);
                        else if (b[1] < a[1] && b[1] >= f.ymin)
                            I[1] = a[1] - fabs(vz(f) - a[2]);
                        if (a[1] <= f.ymax && a[1] >= f.ymin && a[2] == f.zmax) I[1] = a[1];
                        I[2] = vz(f);
                        if (I[2] <= maxZ && I[2] >= minZ && I[1] <= maxY && I[1] >= minY &&
                            I[0] <= f.xmax && I[0] >= f.xmin && record(f, a, b))
                            return true;
                    } else if (f.plane == 2) {
                        I[0] = a[0];
                        if (b[2] > a[2] && b[2] <= f.zmax)
                            I[2] = a[2] + fabs(vy(f) - a[1]);
                        else if (b[2] < a[2] && b[2] >= f.zmin)
                            I[2] = a[2] - fabs(vy(f) - a[1]);
                        if (a[2] <= f.zmax && a[2] >= f.zmin && a[1] == f.ymax) I[2] = a[2];
                        I[1] = vy(f);
                        if (I[2] <= maxZ && I[2] >= minZ && I[1] <= maxY && I[1] >= minY &&
                            I[0] <= f.xmax && I[0] >= f.xmin && record(f, a, b))
                            return true;
                    }
                }
            }
        }
        return false;
    }
};

const int CX[19] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0};
const int CY[19] = {0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1};
const int CZ[19] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1};

thread_local std::string g_gen_error;

}  // namespace

extern "C" {

const char *lbm_latticegen_error(void) { return g_gen_error.c_str(); }

int lbm_latticegen(const char *vrt_path, const char *bnd_path, int n_x, double xseed, double yseed,
                   double zseed, int complexity, const char *node_path, const char *bc_path,
                   int *out_dims) {
    Geometry g;
    std::string err;
    if (!vrt_path || !bnd_path || !node_path || !bc_path || n_x < 2) {
        g_gen_error = "invalid arguments";
        return LBM_ERR_INVALID;
    }
    if (!read_geometry(vrt_path, bnd_path, g, err)) {
        g_gen_error = err;
        return LBM_ERR_FILE;
    }
    // grid (MeshGen.cpp:35-79)
    double xmax = g.x[0], xmin = g.x[0], ymax = g.y[0], ymin = g.y[0], zmax = g.z[0], zmin = g.z[0];
    for (size_t v = 0; v < g.x.size(); ++v) {
        if (g.x[v] > xmax) xmax = g.x[v];
        if (g.y[v] > ymax) ymax = g.y[v];
        if (g.z[v] > zmax) zmax = g.z[v];
        if (g.x[v] < xmin) xmin = g.x[v];
        if (g.y[v] < ymin) ymin = g.y[v];
        if (g.z[v] < zmin) zmin = g.z[v];
    }
    const int n = n_x;
    const double delta = (xmax - xmin) / (n - 1);
    const int m = (int)ceil((ymax - ymin) / delta) + 1;
    const int h = (int)ceil((zmax - zmin) / delta) + 1;
    const long long NX = n + 2, NY = m + 2, NZ = h + 2, NT = NX * NY * NZ;
    if (m < 1 || h < 1 || NT > (1ll << 31)) {
        g_gen_error = "degenerate or oversized grid";
        return LBM_ERR_INVALID;
    }
    std::vector<double> px(NT), py(NT), pz(NT);
    for (long long k = 0; k < NZ; ++k)
        for (long long j = 0; j < NY; ++j)
            for (long long i = 0; i < NX; ++i) {
                const long long id = i + j * NX + k * NY * NX;
                px[id] = xmin + delta * (double)(i - 1);
                py[id] = ymin + delta * (double)(j - 1);
                pz[id] = zmin + delta * (double)(k - 1);
            }
    // seed: nearest node closer than the seed's distance from the origin
    double dist = sqrt(pow(xseed, 2) + pow(yseed, 2) + pow(zseed, 2));
    long long seed = -1;
    for (long long id = 0; id < NT; ++id) {
        const double d = sqrt(pow(px[id] - xseed, 2) + pow(py[id] - yseed, 2) + pow(pz[id] - zseed, 2));
        if (d < dist) {
            dist = d;
            seed = id;
        }
    }
    if (seed < 0) {
        g_gen_error = "no lattice node is nearer the seed than the origin is";
        return LBM_ERR_INVALID;
    }
    FILE *bcf = fopen(bc_path, "w");
    if (!bcf) {
        g_gen_error = std::string("cannot write ") + bc_path;
        return LBM_ERR_FILE;
    }
    std::vector<uint8_t> fluid_flag(NT, 0), filled(NT, 0);
    std::vector<long long> queue;
    queue.reserve(1024);
    queue.push_back(seed);
    fluid_flag[seed] = 1;
    Crossing X(g);
    auto write_link = [&](long long xi, long long yi, long long zi, int dir) {
        fprintf(bcf, "%lld\t%lld\t%lld\t%d\t%d\t%.6f\t%.6f\t%.6f\t%d\n", xi - 1, yi - 1, zi - 1, dir, X.type,
                (double)(float)X.hit[0], (double)(float)X.hit[1], (double)(float)X.hit[2], X.id);
    };
    auto decompose = [&](long long id, long long &xi, long long &yi, long long &zi) {
        zi = id / (NX * NY);
        yi = (id - zi * NX * NY) / NX;
        xi = id - zi * NX * NY - yi * NX;
    };
    for (size_t q = 0; q < queue.size(); ++q) {
        long long xi, yi, zi;
        decompose(queue[q], xi, yi, zi);
        if (!(xi > 0 && xi < n + 1 && yi > 0 && yi < m + 1 && zi > 0 && zi < h + 1)) continue;
        const double a[3] = {px[queue[q]], py[queue[q]], pz[queue[q]]};
        for (int dir = 1; dir < 19; ++dir) {
            const long long nb = (xi + CX[dir]) + (yi + CY[dir]) * NX + (zi + CZ[dir]) * NX * NY;
            const double b[3] = {px[nb], py[nb], pz[nb]};
            if (!X.test(a, b)) {
                if (!filled[nb]) {
                    queue.push_back(nb);
                    fluid_flag[nb] = 1;
                    filled[nb] = 1;
                }
            } else if (complexity == 1 && !filled[nb]) {
                write_link(xi, yi, zi, dir);
            }
        }
    }
    if (complexity == 2) {
        for (size_t q = 0; q < queue.size(); ++q) {
            long long xi, yi, zi;
            decompose(queue[q], xi, yi, zi);
            const double a[3] = {px[queue[q]], py[queue[q]], pz[queue[q]]};
            for (int dir = 1; dir < 19; ++dir) {
                if (!(xi > 0 && xi < n + 1 && yi > 0 && yi < m + 1 && zi > 0 && zi < h + 1)) continue;
                const long long nb = (xi + CX[dir]) + (yi + CY[dir]) * NX + (zi + CZ[dir]) * NX * NY;
                const double b[3] = {px[nb], py[nb], pz[nb]};
                if (X.test(a, b) && !filled[nb]) write_link(xi, yi, zi, dir);
            }
        }
    }
    fclose(bcf);
    FILE *nf = fopen(node_path, "w");
    if (!nf) {
        g_gen_error = std::string("cannot write ") + node_path;
        return LBM_ERR_FILE;
    }
    for (long long k = 1; k < h + 1; ++k)
        for (long long j = 1; j < m + 1; ++j)
            for (long long i = 1; i < n + 1; ++i) {
                const long long id = i + j * NX + k * NY * NX;
                fprintf(nf, "%lld\t%lld\t%lld\t%.6f\t%.6f\t%.6f\t%d\n", i - 1, j - 1, k - 1, px[id], py[id],
                        pz[id], (int)fluid_flag[id]);
            }
    fclose(nf);
    if (out_dims) {
        out_dims[0] = n;
        out_dims[1] = m;
        out_dims[2] = h;
    }
    return LBM_OK;
}

}  // extern "C"
