// thesis_lbm_run: the reference solver's command line (Source code/
// lbm-solver_final/main.cu, Iterate.cu, Iterate3D.cu) on this engine.
//
//   thesis_lbm_run [-f <initfile>] [-o <dir>] [--physics] [--storage f32|f16s|f64]
//   thesis_lbm_run compare <result file> [<result file>]
//
// Reads the 23-line init file (default SetUpData.ini), the lattice
// Mesh/<Lattice>_Node.dat and Mesh/<Lattice>_BC.dat, optional initial
// conditions, runs the time steps on the GPU with the init file's residual
// checks, stop conditions and autosaves, and writes <dir>/FinalData.csv|.dat|.vti
// (default dir Results/) and <dir>/MacroDiffs.txt.  Exit status as
// Iterate2D/3D: 0 done, 1 diverged, 2 lattice not found; 3 for other errors.
// `compare` prints the reference's column table and exits 1 when a column's
// summed difference exceeds 0.001 (Check.cu compareFiles).
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>

#include <string>
#include <vector>

#include "thesis_lbm.h"
#include "thesis_lbm_io.h"

namespace {

int usage(const char *prog) {
    fprintf(stderr,
            "usage: %s [-f <initfile>] [-o <dir>] [--physics] [--storage f32|f16s|f64]\n"
            "       %s compare <result file> [<result file>]\n",
            prog, prog);
    return 3;
}

int compare(const char *a, const char *b) {
    printf("Comparing results\n");
    double sum[9], mx[9];
    const int rc = lbm_compare_results(a, b, sum, mx);
    if (rc == LBM_ERR_FILE) {
        printf("%s\n", lbm_io_last_error());
        return 1;
    }
    const char *names[] = {"x", "y", "z", "u", "v", "w", "vel_mag", "rho", "pressure"};
    const long long lines = lbm_count_lines(a);
    printf("     array |        diff sum |        diff max |      diff/nodes\n"
           "----------------------------------------------\n");
    for (int c = 0; c < 9; ++c)
        printf("%10s | %15g | %15g | %15g\n", names[c], sum[c], mx[c], sum[c] / (double)lines);
    return rc;
}

// Inlet extent for the 2D parabolic profile, as the reference finds it
// (FilesReading.cu:473-606): grid spacing from nodes (0,0) and (1,0), inlet
// links of directions 1-4, extended by half a spacing.
float grid_spacing(const std::vector<int> &ni, const std::vector<int> &nj, const std::vector<float> &nx) {
    float d1 = 0, d2 = 0;
    for (size_t i = 0; i < ni.size(); ++i)
        if (ni[i] == 0 && nj[i] == 0) {
            d1 = nx[i];
            break;
        }
    for (size_t i = 0; i < ni.size(); ++i)
        if (ni[i] == 1 && nj[i] == 0) {
            d2 = nx[i];
            break;
        }
    return fabsf(d2 - d1);
}

void inlet_extent(const std::vector<int> &ni, const std::vector<int> &nj, const std::vector<float> &nx,
                  const std::vector<int> &type, const std::vector<int> &dir, const std::vector<float> &by,
                  float &ymin, float &ymax) {
    const float delta = grid_spacing(ni, nj, nx);
    bool any = false;
    for (size_t i = 0; i < type.size(); ++i)
        if (type[i] == LBM_BC_INLET && dir[i] >= 1 && dir[i] <= 4) {
            if (!any || by[i] > ymax) ymax = by[i];
            if (!any || by[i] < ymin) ymin = by[i];
            any = true;
        }
    ymax += delta / 2;
    ymin -= delta / 2;
}

}  // namespace

int main(int argc, char **argv) {
    std::string init = "SetUpData.ini", out = "Results/";
    int mode = LBM_MODE_REFERENCE, storage = LBM_STORE_F32;
    if (argc >= 2 && strcmp(argv[1], "compare") == 0) {
        if (argc < 3) return usage(argv[0]);
        return compare(argv[2], argc >= 4 ? argv[3] : "Results/FinalData.csv");
    }
    for (int a = 1; a < argc; ++a) {
        const std::string s = argv[a];
        if ((s == "-f" || s == "--initfile") && a + 1 < argc) init = argv[++a];
        else if ((s == "-o" || s == "--output") && a + 1 < argc) out = argv[++a];
        else if (s == "--physics") mode = LBM_MODE_PHYSICS;
        else if (s == "--storage" && a + 1 < argc) {
            const std::string v = argv[++a];
            storage = v == "f16s" ? LBM_STORE_F16S : (v == "f64" ? LBM_STORE_F64 : LBM_STORE_F32);
        } else if (s == "-h" || s == "--help") {
            usage(argv[0]);
            return 0;
        } else
            return usage(argv[0]);
    }
    if (!out.empty() && out.back() != '/') out += '/';
    mkdir(out.c_str(), 0755);

    lbm_run_config cfg;
    if (lbm_read_init_file(init.c_str(), &cfg) != LBM_OK) {
        fprintf(stderr, "%s\n", lbm_io_last_error());
        return 3;
    }
    if (cfg.unparsed_lines) fprintf(stderr, "Error reading initial file (%d lines)\n", cfg.unparsed_lines);
    const std::string node = std::string("Mesh/") + cfg.problem_name + "_Node.dat";
    const std::string bcf = std::string("Mesh/") + cfg.problem_name + "_BC.dat";
    const int dims = lbm_node_file_dims(node.c_str());
    const long long nn = lbm_count_lines(node.c_str()), nc = lbm_count_lines(bcf.c_str());
    if (dims < 0 || nn <= 0 || nc < 0) {
        fprintf(stderr, "Error reading file %s\n", node.c_str());
        return 2;
    }
    std::vector<int> ni(nn), nj(nn), nk(nn), nt(nn);
    std::vector<float> x(nn), y(nn), z(nn);
    std::vector<int> bi(nc), bj(nc), bk(nc), bd(nc), bt(nc), bid(nc);
    std::vector<float> bx(nc), by(nc), bz(nc);
    if (lbm_read_node_file(node.c_str(), dims, nn, ni.data(), nj.data(), nk.data(), x.data(), y.data(), z.data(),
                           nt.data()) ||
        (nc && lbm_read_bc_file(bcf.c_str(), dims, nc, bi.data(), bj.data(), bk.data(), bd.data(), bt.data(),
                                bx.data(), by.data(), bz.data(), bid.data()))) {
        fprintf(stderr, "%s\n", lbm_io_last_error());
        return 2;
    }
    // extents from the last node, as Iterate* does (getLastValue)
    const int n = ni[nn - 1] + 1, m = nj[nn - 1] + 1, h = dims == 3 ? nk[nn - 1] + 1 : 1;
    if ((long long)n * m * h != nn) {
        fprintf(stderr, "node file holds %lld nodes, not %d x %d x %d\n", nn, n, m, h);
        return 2;
    }
    lbm_lattice_desc lat = {dims, n, m, h, nt.data(), (int)nc, bi.data(), bj.data(),
                            dims == 3 ? bk.data() : nullptr, bd.data(), bt.data(), bid.data()};
    lbm_params p;
    memset(&p, 0, sizeof(p));
    p.u = cfg.u;
    p.v = cfg.v;
    p.w = cfg.w;
    p.rho = cfg.rho;
    p.viscosity = cfg.viscosity;
    p.g = cfg.g;
    p.inlet_profile = cfg.inlet_profile;
    p.outlet_profile = cfg.outlet_profile;
    p.collision_model = cfg.collision_model;
    p.boundary_type = cfg.boundary_type;
    p.bc_wall_model = cfg.bc_wall_model;
    if (mode == LBM_MODE_PHYSICS && p.bc_wall_model == LBM_WALL_COMPLEX) {
        // physics-mode walls are half-way bounce-back whatever the init file names
        fprintf(stderr, "physics mode: walls are half-way bounce-back (BCwallModel HHmodel ignored)\n");
        p.bc_wall_model = LBM_WALL_SIMPLE;
    }
    if (mode == LBM_MODE_PHYSICS && p.boundary_type == LBM_CURVED) {
        fprintf(stderr, "physics mode: walls are half-way bounce-back (BoundaryType CURVED ignored)\n");
        p.boundary_type = LBM_STRAIGHT;
    }
    p.update_inlet_outlet = cfg.update_inlet_outlet;
    p.mode = mode;
    p.storage = storage;
    p.rho_in = p.rho_out = cfg.rho;
    p.init_equilibrium = mode == LBM_MODE_PHYSICS;
    lbm_handle hd;
    if (lbm_create(&lat, &p, &hd) != LBM_OK) {
        fprintf(stderr, "%s\n", lbm_last_error());
        return 3;
    }
    if (p.boundary_type == LBM_CURVED && !(dims == 3 && p.bc_wall_model == LBM_WALL_COMPLEX)) {
        // link fractions from the BC file's boundary points and the node
        // coordinates (initBoundaryConditions2D/3D; the reference's HH wall
        // kernel has no curved branch)
        std::vector<double> q((size_t)nc);
        if (lbm_link_q(dims, n, m, h, (int)nc, bi.data(), bj.data(), dims == 3 ? bk.data() : nullptr, bd.data(),
                       bx.data(), by.data(), dims == 3 ? bz.data() : nullptr, x.data(), y.data(),
                       dims == 3 ? z.data() : nullptr, grid_spacing(ni, nj, x), q.data()) != LBM_OK ||
            lbm_set_link_q(hd, q.data()) != LBM_OK) {
            fprintf(stderr, "%s\n", lbm_last_error());
            lbm_destroy(hd);
            return 3;
        }
    }
    const long long N = nn;
    std::vector<float> rho(N), u(N), v(N), w(N);
    if (dims == 2 && cfg.inlet_profile == LBM_INLET) {
        // parabolic inlet over the inlet's y extent (gpuInitInletProfile2D)
        float ymin = 0, ymax = 0;
        inlet_extent(ni, nj, x, bt, bd, by, ymin, ymax);
        const float len2 = (ymax - ymin) * (ymax - ymin);
        std::vector<float> u0(N), v0(N, (float)cfg.v);
        for (long long i = 0; i < N; ++i) u0[i] = 4 * 1.5f * (float)cfg.u * (y[i] - ymin) * (ymax - y[i]) / len2;
        lbm_set_inlet_velocity(hd, u0.data(), v0.data(), nullptr);
    }
    int rc;
    if (cfg.use_initial_conditions_file) {
        if (lbm_read_initial_conditions(cfg.initial_conditions_name, N, n, m, h, u.data(), v.data(), w.data(),
                                        rho.data()) != LBM_OK) {
            fprintf(stderr, "%s\n", lbm_io_last_error());
            lbm_destroy(hd);
            return 3;
        }
        rc = lbm_init(hd, rho.data(), u.data(), v.data(), w.data());
    } else {
        rc = lbm_init(hd, nullptr, nullptr, nullptr, nullptr);
    }
    if (rc != LBM_OK) {
        fprintf(stderr, "%s\n", lbm_last_error());
        lbm_destroy(hd);
        return 3;
    }
    const char *ext = cfg.output_format == LBM_OUT_DAT ? "dat" : (cfg.output_format == LBM_OUT_VTI ? "vti" : "csv");
    auto write = [&](const std::string &path) {
        lbm_get_macro(hd, rho.data(), u.data(), v.data(), w.data());
        if (lbm_write_results(path.c_str(), cfg.output_format, n, m, h, x.data(), y.data(), z.data(), u.data(),
                              v.data(), w.data(), rho.data()) != LBM_OK)
            fprintf(stderr, "%s\n", lbm_io_last_error());
    };
    FILE *md = fopen((out + "MacroDiffs.txt").c_str(), "w");
    if (md) fprintf(md, "iteration\tMax u diff\tMax v diff\tMax w diff\tMax rho diff\n");

    // the reference's residual file (writeResiduals, LogWriter.cu:190-205):
    // one row per iteration, filled at the checks; in 2D the norm column is
    // the L2 residual with the drag/lift sums of BoundaryId beside it
    // (Iterate.cu:548-571), in 3D the residual model's value (Iterate3D.cu:
    // 737-780) and no drag/lift.  The stop test uses the residual model in
    // both (the reference's 2D single-phase loop has none).
    const bool res_file = dims == 2 || cfg.residual_model != LBM_RES_MACRO_DIFF;
    std::vector<double> norm((size_t)(cfg.iterations > 0 ? cfg.iterations : 1), 0.0), drag(norm), lift(norm);
    if (cfg.residual_model == LBM_RES_FD_REL_DIFF) {
        // FdRelDiff measures against the populations at the start (f_prev and
        // f_first both taken here; the reference takes f_first at its first check)
        double r0;
        lbm_residual_fd_rel_diff(hd, &r0);
    }
    const int every = cfg.show_macro_diff > 0 ? cfg.show_macro_diff : cfg.iterations;
    int status = 0, autosave_it = 1;
    for (int iter = 0; iter < cfg.iterations;) {
        int chunk = every - iter % every;
        if (iter + chunk > cfg.iterations) chunk = cfg.iterations - iter;
        if (cfg.autosave_every > 0) {
            const int next_save = cfg.autosave_every * autosave_it;
            if (next_save > iter && next_save < iter + chunk) chunk = next_save - iter;
        }
        if (lbm_step(hd, chunk, 1, nullptr) != LBM_OK) {
            fprintf(stderr, "%s\n", lbm_last_error());
            status = 3;
            break;
        }
        iter += chunk;
        if (iter % every == 0 || iter == cfg.iterations) {
            double d[5];
            const int r = lbm_macro_diff(hd, d);
            if (r == LBM_DIVERGED) {
                fprintf(stderr, "\nDIVERGENCE!\n");
                status = 1;
                break;
            }
            if (md) fprintf(md, "%d\t\t%.10f\t%.10f\t%.10f\t%.10f\n", iter, d[0], d[1], d[2], d[3]);
            if (cfg.residual_model == LBM_RES_MACRO_DIFF && d[0] < cfg.stop_condition[0] &&
                d[1] < cfg.stop_condition[1] && d[2] < cfg.stop_condition[2] && d[3] < cfg.stop_condition[3]) {
                printf("simulation converged!\n");
                break;
            }
            // L2 and MaxRelativeFdDiff stop on |r| < StopCondition[0] (Iterate3D.cu:758-765)
            if (res_file) {
                double res = 0.0, l2 = 0.0;
                int rr = LBM_OK;
                if (cfg.residual_model == LBM_RES_FD_REL_DIFF) rr = lbm_residual_fd_rel_diff(hd, &res);
                if (rr == LBM_OK && (dims == 2 || cfg.residual_model == LBM_RES_L2)) rr = lbm_residual_l2(hd, &l2);
                if (cfg.residual_model == LBM_RES_L2) res = l2;
                if (rr == LBM_DIVERGED) {
                    fprintf(stderr, "\nDIVERGENCE!\n");
                    status = 1;
                    break;
                }
                norm[(size_t)iter - 1] = dims == 2 ? l2 : res;
                if (dims == 2 && cfg.boundary_id > 0) {
                    double dl[2];
                    if (lbm_reference_drag_lift(hd, cfg.boundary_id, x.data(), y.data(), dl) == LBM_OK) {
                        drag[(size_t)iter - 1] = dl[0];
                        lift[(size_t)iter - 1] = dl[1];
                    }
                }
                if (cfg.residual_model != LBM_RES_MACRO_DIFF && fabs(res) < cfg.stop_condition[0]) {
                    printf("simulation converged!\n");
                    break;
                }
            }
        }
        if (cfg.autosave_every > 0 && iter == cfg.autosave_every * autosave_it) {
            ++autosave_it;
            if (iter > cfg.autosave_after) write(out + "FinalData." + ext);
        }
    }
    if (md) fclose(md);
    if (res_file) {
        if (FILE *resf = fopen((out + "Residuals.txt").c_str(), "w")) {
            fprintf(resf, "Iter L2_norm L2_norm_weighted Drag Lift\n");
            for (int i = 0; i < cfg.iterations; ++i)
                fprintf(resf, "%d %5.4e %5.4e %f %f\n", i, norm[(size_t)i], norm[(size_t)i] / (double)N, drag[(size_t)i],
                        lift[(size_t)i]);
            fclose(resf);
        }
    }
    if (status != 3) write(out + "FinalData." + ext);
    lbm_destroy(hd);
    return status;
}
