// The reference solver's file formats (include/thesis_lbm_io.h): init file,
// Node/BC lattice files, result writers and readers, result comparison.
// Restated from Source code/lbm-solver_final/FilesReading.cu,
// FilesWriting.cu and Check.cu; host code only.
#include "thesis_lbm_io.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <fstream>
#include <string>
#include <thread>
#include <vector>

#include "thesis_lbm.h"

namespace {

thread_local std::string g_io_error;

int io_fail(int code, const std::string &msg) {
    g_io_error = msg;
    return code;
}

// Text after the first "= " (the reference's value extraction); false when
// the line has none.
bool value_of(std::string &line) {
    const size_t p = line.find("= ");
    if (p == std::string::npos) return false;
    line = line.substr(p + 2);
    return true;
}

// Text between the first two double quotes.
bool quoted(std::string &s) {
    size_t p = s.find('"');
    if (p == std::string::npos) return false;
    s = s.substr(p + 1);
    p = s.find('"');
    if (p == std::string::npos) return false;
    s = s.substr(0, p);
    return true;
}

bool has(const std::string &s, const char *key) { return s.find(key) != std::string::npos; }

// The reference's default build parses into FP32 fields.
double f32(double v) { return (double)(float)v; }


// Whole file into memory; false when it cannot be read.
bool slurp(const char *path, std::vector<char> &buf) {
    FILE *f = path ? fopen(path, "rb") : nullptr;
    if (!f) return false;
    buf.clear();
    const size_t block = 1u << 24;
    size_t used = 0;
    for (;;) {
        buf.resize(used + block);
        const size_t got = fread(buf.data() + used, 1, block, f);
        used += got;
        if (got < block) break;
    }
    const bool ok = ferror(f) == 0;
    fclose(f);
    buf.resize(used);
    return ok;
}

// One whitespace-separated field of a record line, as fscanf's %d and %f
// read it (strtol / strtof: a float field keeps strtof's rounding).
bool next_int(const char *&p, const char *end, int &v) {
    while (p < end && (*p == ' ' || *p == '\t' || *p == '\r')) ++p;
    if (p >= end) return false;
    char *q = nullptr;
    const long x = strtol(p, &q, 10);
    if (q == p) return false;
    p = q;
    v = (int)x;
    return true;
}
bool next_float(const char *&p, const char *end, float &v) {
    while (p < end && (*p == ' ' || *p == '\t' || *p == '\r')) ++p;
    if (p >= end) return false;
    char *q = nullptr;
    const float x = strtof(p, &q);
    if (q == p) return false;
    p = q;
    v = x;
    return true;
}

// Records of a Node or BC file, one per non-blank line, parsed by
// `parse(line_begin, line_end, record)` on all host threads.  Records before
// the first malformed one are read, as the reference's fscanf loop stops
// there (FilesReading.cu:270-347); what lies from that record on is
// unspecified (the reference leaves it unset).
template <class F>
void parse_records(const std::vector<char> &buf, long long count, F parse) {
    const char *base = buf.data();
    const size_t size = buf.size();
    const int T = (int)std::max(1u, std::min(std::thread::hardware_concurrency(), 64u));
    std::vector<size_t> cut(T + 1, size);
    cut[0] = 0;
    for (int t = 1; t < T; ++t) {
        size_t c = std::max(size * t / T, cut[t - 1]);
        while (c < size && base[c - 1] != '\n') ++c;
        cut[t] = c;
    }
    auto is_blank = [](const char *a, const char *b) {
        for (; a < b; ++a)
            if (*a != ' ' && *a != '\t' && *a != '\r') return false;
        return true;
    };
    std::vector<long long> lines(T, 0);
    std::vector<std::thread> th;
    for (int t = 0; t < T; ++t)
        th.emplace_back([&, t] {
            const char *p = base + cut[t], *e = base + cut[t + 1];
            while (p < e) {
                const char *nl = (const char *)memchr(p, '\n', (size_t)(e - p));
                const char *le = nl ? nl : e;
                if (!is_blank(p, le)) ++lines[t];
                p = le + 1;
            }
        });
    for (auto &x : th) x.join();
    th.clear();
    std::vector<long long> first(T + 1, 0);
    for (int t = 0; t < T; ++t) first[t + 1] = first[t] + lines[t];
    std::atomic<long long> bad(count);
    for (int t = 0; t < T; ++t)
        th.emplace_back([&, t] {
            const char *p = base + cut[t], *e = base + cut[t + 1];
            long long r = first[t];
            while (p < e && r < count) {
                const char *nl = (const char *)memchr(p, '\n', (size_t)(e - p));
                const char *le = nl ? nl : e;
                if (!is_blank(p, le)) {
                    if (!parse(p, le, r)) {
                        long long cur = bad.load();
                        while (r < cur && !bad.compare_exchange_weak(cur, r)) {
                        }
                        return;
                    }
                    ++r;
                }
                p = le + 1;
            }
        });
    for (auto &x : th) x.join();
}
}  // namespace

extern "C" {

const char *lbm_io_last_error(void) { return g_io_error.c_str(); }

long long lbm_count_lines(const char *path) {
    FILE *f = path ? fopen(path, "rb") : nullptr;
    if (!f) return -1;
    long long lines = 0;
    std::vector<char> block(1u << 22);
    size_t got;
    while ((got = fread(block.data(), 1, block.size(), f)) > 0)
        for (size_t c = 0; c < got; ++c) lines += (block[c] == '\n') | (block[c] == '\r');
    fclose(f);
    return lines;
}

int lbm_read_init_file(const char *path, lbm_run_config *cfg) {
    if (!path || !cfg) return io_fail(LBM_ERR_INVALID, "null argument");
    memset(cfg, 0, sizeof(*cfg));
    std::ifstream in(path);
    if (!in) return io_fail(LBM_ERR_FILE, std::string("cannot open ") + path);
    std::string line[23];
    int bad = 0;
    for (int i = 0; i < 23; ++i) {
        std::getline(in, line[i]);
        if (!value_of(line[i])) ++bad;
    }
    if (quoted(line[0])) snprintf(cfg->problem_name, sizeof(cfg->problem_name), "%s", line[0].c_str());
    else ++bad;
    if (quoted(line[17]))
        snprintf(cfg->initial_conditions_name, sizeof(cfg->initial_conditions_name), "%s", line[17].c_str());
    else ++bad;
    cfg->u = f32(atof(line[1].c_str()));
    cfg->v = f32(atof(line[2].c_str()));
    cfg->w = f32(atof(line[3].c_str()));
    cfg->rho = f32(atof(line[4].c_str()));
    cfg->viscosity = f32(atof(line[5].c_str()));
    cfg->iterations = atoi(line[11].c_str());
    cfg->autosave_after = atoi(line[12].c_str());
    cfg->autosave_every = atoi(line[13].c_str());
    float sc[4] = {0, 0, 0, 0};
    sscanf(line[14].c_str(), "%f %f %f %f", &sc[0], &sc[1], &sc[2], &sc[3]);
    for (int k = 0; k < 4; ++k) cfg->stop_condition[k] = sc[k];
    cfg->show_macro_diff = atoi(line[19].c_str());
    cfg->g = f32(atof(line[20].c_str()));
    cfg->boundary_id = (int)(float)atof(line[21].c_str());
    if (has(line[15], "CSV")) cfg->output_format = LBM_OUT_CSV;
    else if (has(line[15], "DAT")) cfg->output_format = LBM_OUT_DAT;
    else if (has(line[15], "VTI")) cfg->output_format = LBM_OUT_VTI;
    else ++bad;
    if (has(line[16], "yes")) cfg->use_initial_conditions_file = 1;
    else if (has(line[16], "no")) cfg->use_initial_conditions_file = 0;
    else ++bad;
    if (has(line[6], "INLET_PROF")) cfg->inlet_profile = 1;
    else if (has(line[6], "INLET_CTE")) cfg->inlet_profile = 2;
    else if (has(line[6], "INLET_PUL")) cfg->inlet_profile = 3;
    else ++bad;
    if (has(line[7], "SRT")) cfg->collision_model = LBM_BGKW;
    else if (has(line[7], "TRT")) cfg->collision_model = LBM_TRT;
    else if (has(line[7], "MRT")) cfg->collision_model = LBM_MRT;
    else ++bad;
    if (has(line[8], "STRAIGHT")) cfg->boundary_type = LBM_STRAIGHT;
    else if (has(line[8], "CURVED")) cfg->boundary_type = LBM_CURVED;
    else ++bad;
    if (has(line[9], "BBack")) cfg->bc_wall_model = LBM_WALL_SIMPLE;
    else if (has(line[9], "HHmodel")) cfg->bc_wall_model = LBM_WALL_COMPLEX;
    else ++bad;
    // the reference maps the names to these enum values as written
    // (FilesReading.cu:171-190): 1stE -> 2, 2ndE -> 3
    if (has(line[10], "Vout")) cfg->outlet_profile = 1;
    else if (has(line[10], "1stE")) cfg->outlet_profile = 2;
    else if (has(line[10], "2ndE")) cfg->outlet_profile = 3;
    else if (has(line[10], "HEmodel")) cfg->outlet_profile = 4;
    else ++bad;
    if (has(line[18], "L2")) cfg->residual_model = LBM_RES_L2;
    else if (has(line[18], "MaxRelativeFdDiff")) cfg->residual_model = LBM_RES_FD_REL_DIFF;
    else if (has(line[18], "MaxMacroDiff")) cfg->residual_model = LBM_RES_MACRO_DIFF;
    else ++bad;
    if (has(line[22], "yes")) cfg->update_inlet_outlet = 1;
    else if (has(line[22], "no")) cfg->update_inlet_outlet = 0;
    else ++bad;
    cfg->unparsed_lines = bad;
    return LBM_OK;
}

int lbm_node_file_dims(const char *path) {
    FILE *f = path ? fopen(path, "r") : nullptr;
    if (!f) return -1;
    char buf[4096];
    const bool ok = fgets(buf, sizeof(buf), f) != nullptr;
    fclose(f);
    if (!ok) return -1;
    int i, j, k, t;
    float a, b, c;
    return sscanf(buf, "%d\t%d\t%d\t%f\t%f\t%f\t%d", &i, &j, &k, &a, &b, &c, &t) == 7 ? 3 : 2;
}

int lbm_read_node_file(const char *path, int dims, long long count, int *i, int *j, int *k, float *x, float *y,
                       float *z, int *type) {
    if (!i || !j || !x || !y || !type || (dims == 3 && (!k || !z))) return io_fail(LBM_ERR_INVALID, "null array");
    std::vector<char> buf;
    if (!slurp(path, buf)) return io_fail(LBM_ERR_FILE, std::string("cannot open ") + (path ? path : "(null)"));
    parse_records(buf, count, [&](const char *p, const char *e, long long r) {
        if (dims == 2) {
            if (k) k[r] = 0;
            if (z) z[r] = 0.f;
            return next_int(p, e, i[r]) && next_int(p, e, j[r]) && next_float(p, e, x[r]) && next_float(p, e, y[r]) &&
                   next_int(p, e, type[r]);
        }
        return next_int(p, e, i[r]) && next_int(p, e, j[r]) && next_int(p, e, k[r]) && next_float(p, e, x[r]) &&
               next_float(p, e, y[r]) && next_float(p, e, z[r]) && next_int(p, e, type[r]);
    });
    return LBM_OK;
}

int lbm_read_bc_file(const char *path, int dims, long long count, int *i, int *j, int *k, int *dir, int *type,
                     float *bx, float *by, float *bz, int *id) {
    if (!i || !j || !dir || !type || !bx || !by || !id || (dims == 3 && (!k || !bz)))
        return io_fail(LBM_ERR_INVALID, "null array");
    std::vector<char> buf;
    if (!slurp(path, buf)) return io_fail(LBM_ERR_FILE, std::string("cannot open ") + (path ? path : "(null)"));
    parse_records(buf, count, [&](const char *p, const char *e, long long r) {
        if (dims == 2) {
            if (k) k[r] = 0;
            if (bz) bz[r] = 0.f;
            return next_int(p, e, i[r]) && next_int(p, e, j[r]) && next_int(p, e, dir[r]) && next_int(p, e, type[r]) &&
                   next_float(p, e, bx[r]) && next_float(p, e, by[r]) && next_int(p, e, id[r]);
        }
        return next_int(p, e, i[r]) && next_int(p, e, j[r]) && next_int(p, e, k[r]) && next_int(p, e, dir[r]) &&
               next_int(p, e, type[r]) && next_float(p, e, bx[r]) && next_float(p, e, by[r]) &&
               next_float(p, e, bz[r]) && next_int(p, e, id[r]);
    });
    return LBM_OK;
}

int lbm_write_results(const char *path, int format, int n, int m, int h, const float *x, const float *y,
                      const float *z, const float *u, const float *v, const float *w, const float *rho) {
    if (!path || !x || !y || !z || !u || !v || !w || !rho) return io_fail(LBM_ERR_INVALID, "null argument");
    FILE *f = fopen(path, "w");
    if (!f) return io_fail(LBM_ERR_FILE, std::string("cannot write ") + path);
    const long long N = (long long)n * m * h;
    // vel_mag as the reference computes it: pow of the FP32 values in FP64
    auto vmag = [&](long long i) {
        return sqrt(pow((double)u[i], 2) + pow((double)v[i], 2) + pow((double)w[i], 2));
    };
    if (format == LBM_OUT_CSV) {
        fprintf(f, "x,y,z,u,v,w,vel_mag,rho,press\n");
        for (long long i = 0; i < N; ++i)
            fprintf(f, "%.10f, %.10f, %.10f, %.10f, %.10f, %.10f, %.10f, %.10f, %.10f\n", x[i], y[i], z[i], u[i],
                    v[i], w[i], vmag(i), rho[i], rho[i] / 3);  // pressure in FP32, rho / 3
    } else if (format == LBM_OUT_DAT) {
        fprintf(f, "Title = \"LBM results\"\n");
        fprintf(f, "Variables = \"x\",\"y\",\"z\",\"u\",\"v\",\"w\",\"vel mag\",\"rho\",\"press\"\n");
        fprintf(f, "Zone i=%d, j=%d, k=%d, f=point\n", n, m, h);
        for (long long i = 0; i < N; ++i)
            fprintf(f, "%.10f %.10f %.10f %.10f %.10f %.10f %.10f %.10f %.10f\n", x[i], y[i], z[i], u[i], v[i],
                    w[i], vmag(i), rho[i], rho[i] / 3);
    } else if (format == LBM_OUT_VTI) {
        fprintf(f, "<?xml version=\"1.0\"?>\n");
        fprintf(f, "<!-- 3D LBM Solver -->\n");
        fprintf(f, "<VTKFile type=\"ImageData\" version=\"0.1\" byte_order=\"LittleEndian\">\n");
        fprintf(f, "  <ImageData WholeExtent=\"0 %d 0 %d 0 %d\" Origin=\"0 0 0\" Spacing=\"1 1 1\">\n", n - 1,
                m - 1, h - 1);
        fprintf(f, "  <Piece Extent=\"0 %d 0 %d 0 %d\">\n", n - 1, m - 1, h - 1);
        fprintf(f, "    <PointData Scalars=\"scalars\">\n");
        fprintf(f, "      <DataArray type=\"Float32\" Name=\"Velocity\" NumberOfComponents=\"3\" format=\"ascii\">\n");
        for (long long i = 0; i < N; ++i) fprintf(f, "%.10f %.10f %.10f\n", u[i], v[i], w[i]);
        fprintf(f, "      </DataArray>\n");
        fprintf(f, "      <DataArray type=\"Float32\" Name=\"Density\" NumberOfComponents=\"1\" format=\"ascii\">\n");
        for (long long i = 0; i < N; ++i) fprintf(f, "%.10f\n", rho[i]);
        fprintf(f, "      </DataArray>\n");
        fprintf(f, "      <DataArray type=\"Float32\" Name=\"Pressure\" NumberOfComponents=\"1\" format=\"ascii\">\n");
        for (long long i = 0; i < N; ++i) fprintf(f, "%.10f\n", rho[i] / 3.0);  // FP64 here, as written
        fprintf(f, "      </DataArray>\n");
        fprintf(f, "    </PointData>\n");
        fprintf(f, "    <CellData>\n");
        fprintf(f, "    </CellData>\n");
        fprintf(f, "  </Piece>\n");
        fprintf(f, "  </ImageData>\n");
        fprintf(f, "</VTKFile>\n");
    } else {
        fclose(f);
        return io_fail(LBM_ERR_INVALID, "unknown output format");
    }
    const bool err = ferror(f) != 0;
    fclose(f);
    return err ? io_fail(LBM_ERR_FILE, std::string("write error on ") + path) : LBM_OK;
}

long long lbm_read_results(const char *path, long long count, double *cols) {
    if (!path || !cols) return io_fail(LBM_ERR_INVALID, "null argument") * -1;
    const long long n = lbm_count_lines(path);
    if (n <= 0) return -(long long)io_fail(LBM_ERR_FILE, std::string("empty or unreadable ") + path);
    FILE *f = fopen(path, "r");
    if (!f) return -(long long)io_fail(LBM_ERR_FILE, std::string("cannot open ") + path);
    for (long long i = 0; i < 9 * count; ++i) cols[i] = 0.0;
    char head[4096] = {0};
    if (!fgets(head, sizeof(head), f)) {
        fclose(f);
        return -(long long)io_fail(LBM_ERR_FILE, "empty result file");
    }
    long long rows = 0;
    float v[9];
    auto put = [&](long long r, int c, float val) {
        if (r < count) cols[(long long)c * count + r] = val;
    };
    char skip[4096];
    if (head[0] == 'x' && head[1] == ',') {  // CSV
        for (long long r = 0; r < n - 1; ++r) {
            if (fscanf(f, "%f, %f, %f, %f, %f, %f, %f, %f, %f\n", v, v + 1, v + 2, v + 3, v + 4, v + 5, v + 6, v + 7,
                       v + 8) != 9)
                break;
            for (int c = 0; c < 9; ++c) put(r, c, v[c]);
            rows = r + 1;
        }
    } else if (head[0] == 'T' && head[1] == 'i') {  // Tecplot
        if (!fgets(skip, sizeof(skip), f) || !fgets(skip, sizeof(skip), f)) {
            fclose(f);
            return -(long long)io_fail(LBM_ERR_FILE, "truncated Tecplot header");
        }
        for (long long r = 0; r < n - 3; ++r) {
            if (fscanf(f, "%f %f %f %f %f %f %f %f %f\n", v, v + 1, v + 2, v + 3, v + 4, v + 5, v + 6, v + 7,
                       v + 8) != 9)
                break;
            for (int c = 0; c < 9; ++c) put(r, c, v[c]);
            rows = r + 1;
        }
    } else if (head[0] == '<' && head[1] == '?') {  // ParaView image data
        for (int s = 0; s < 6; ++s)
            if (!fgets(skip, sizeof(skip), f)) break;
        const long long pts = (n - 18) / 3;
        for (long long r = 0; r < pts; ++r) {
            if (fscanf(f, "%f %f %f\n", v, v + 1, v + 2) != 3) break;
            put(r, 3, v[0]);
            put(r, 4, v[1]);
            put(r, 5, v[2]);
            rows = r + 1;
        }
        if (fgets(skip, sizeof(skip), f) && fgets(skip, sizeof(skip), f))
            for (long long r = 0; r < pts; ++r) {
                if (fscanf(f, "%f\n", v) != 1) break;
                put(r, 7, v[0]);
            }
    } else {
        fclose(f);
        return -(long long)io_fail(LBM_ERR_FILE, std::string("unknown result format in ") + path);
    }
    fclose(f);
    return rows;
}

int lbm_read_initial_conditions(const char *path, long long nodes, int n, int m, int h, float *u, float *v,
                                float *w, float *rho) {
    if (!u || !v || !w || !rho) return io_fail(LBM_ERR_INVALID, "null array");
    const long long lines = lbm_count_lines(path);
    if (lines <= 0) return io_fail(LBM_ERR_FILE, "empty/no initial condition file");
    FILE *f = fopen(path, "r");
    if (!f) return io_fail(LBM_ERR_FILE, std::string("cannot open ") + path);
    char head[4096] = {0};
    const bool got = fgets(head, sizeof(head), f) != nullptr;
    fclose(f);
    if (!got) return io_fail(LBM_ERR_FILE, "empty/no initial condition file");
    const long long N = (long long)n * m * h;
    const bool tecplot = lines - 3 == nodes && head[0] == 'T' && head[1] == 'i';
    const bool vti = head[0] == '<' && head[1] == '?' && lines == 18 + 3 * N;
    const bool csv = lines - 1 == nodes && head[0] == 'x' && head[1] == ',';
    if (!tecplot && !vti && !csv)
        return io_fail(LBM_ERR_FILE, "wrong file! Number of nodes in initial condition file is incorrect");
    std::vector<double> cols((size_t)9 * N);
    const long long rows = lbm_read_results(path, N, cols.data());
    if (rows < 0) return (int)-rows;
    for (long long i = 0; i < N; ++i) {
        u[i] = (float)cols[3 * N + i];
        v[i] = (float)cols[4 * N + i];
        w[i] = (float)cols[5 * N + i];
        rho[i] = (float)cols[7 * N + i];
    }
    return LBM_OK;
}

int lbm_write_midlines(const char *path, int dims, int n, int m, int h, const float *x, const float *y,
                       const float *z, const float *u, const float *v, const float *w, double ulid) {
    if (!path || !x || !y || !u || !v || (dims == 3 && (!z || !w)) || !(ulid != 0))
        return io_fail(LBM_ERR_INVALID, "invalid argument");
    FILE *f = fopen(path, "w");
    if (!f) return io_fail(LBM_ERR_FILE, std::string("cannot write ") + path);
    fprintf(f, "CASE: Ulid = %f Nx = %d\n", ulid, n);
    const float U = (float)ulid;
    if (dims == 3) {
        // the reference pairs the k-th node of one line with the k-th of the other
        fprintf(f, "U/Ulid\tZ\tX\tW/Ulid\n");
        std::vector<float> uz, zz, xx, wx;
        const int yc = m / 2, xc = n / 2, zc = h / 2;
        for (int k = 0; k < h; ++k)
            for (int i = 0; i < n; ++i) {
                const size_t id = (size_t)i + (size_t)n * (yc + (size_t)m * k);
                if (i == xc) {
                    uz.push_back(u[id] / U);
                    zz.push_back(z[id]);
                }
                if (k == zc) {
                    xx.push_back(x[id]);
                    wx.push_back(w[id] / U);
                }
            }
        for (size_t r = 0; r < uz.size(); ++r)
            fprintf(f, "%.8f\t%.8f\t%.8f\t%.8f\n", uz[r], zz[r], r < xx.size() ? xx[r] : 0.f,
                    r < wx.size() ? wx[r] : 0.f);
    } else {
        fprintf(f, "U/Ulid\tY\tX\tV/Ulid\n");
        const int xc = n / 2, yc = m / 2;
        const int rows = m > n ? m : n;
        for (int r = 0; r < rows; ++r) {
            const size_t a = (size_t)xc + (size_t)n * (r < m ? r : m - 1);  // along x = n/2
            const size_t b = (size_t)(r < n ? r : n - 1) + (size_t)n * yc;  // along y = m/2
            fprintf(f, "%.8f\t%.8f\t%.8f\t%.8f\n", r < m ? u[a] / U : 0.f, r < m ? y[a] : 0.f,
                    r < n ? x[b] : 0.f, r < n ? v[b] / U : 0.f);
        }
    }
    fclose(f);
    return LBM_OK;
}

int lbm_write_cross_section(const char *path, int n, int m, int h, const float *x, const float *y,
                            const float *z, const float *u, const float *v, const float *w, double uin) {
    if (!path || !x || !y || !z || !u || !v || !w) return io_fail(LBM_ERR_INVALID, "null argument");
    FILE *f = fopen(path, "w");
    if (!f) return io_fail(LBM_ERR_FILE, std::string("cannot write ") + path);
    fprintf(f, "CASE: Uin = %f Ny = %d\n", uin, m);
    fprintf(f, "X\tY\tZ\tU\tV\tW\n");
    const int xc = (int)((3. / 4.) * n);
    for (int k = 0; k < h; ++k)
        for (int j = 0; j < m; ++j) {
            const size_t id = (size_t)xc + (size_t)n * (j + (size_t)m * k);
            fprintf(f, "%.10f %.10f %.10f %.10f %.10f %.10f\n", x[id], y[id], z[id], u[id], v[id], w[id]);
        }
    fclose(f);
    return LBM_OK;
}

int lbm_compare_results(const char *f1, const char *f2, double *diff_sum, double *diff_max) {
    const long long l1 = lbm_count_lines(f1), l2 = lbm_count_lines(f2);
    if (l1 < 0 || l2 < 0) return io_fail(LBM_ERR_FILE, "cannot read a result file");
    if (l1 != l2) return io_fail(LBM_ERR_FILE, "Line number mismatch");
    std::vector<double> a((size_t)9 * l1), b((size_t)9 * l1);
    const long long ra = lbm_read_results(f1, l1, a.data()), rb = lbm_read_results(f2, l1, b.data());
    if (ra < 0 || rb < 0) return LBM_ERR_FILE;
    int differ = 0;
    for (int c = 0; c < 9; ++c) {
        double s = 0, mx = 0;
        for (long long r = 0; r < l1; ++r) {
            const double d = fabs(a[(size_t)c * l1 + r] - b[(size_t)c * l1 + r]);
            s += d;
            mx = d > mx ? d : mx;
        }
        if (diff_sum) diff_sum[c] = s;
        if (diff_max) diff_max[c] = mx;
        differ |= s > 0.001;
    }
    return differ;
}

}  // extern "C"
