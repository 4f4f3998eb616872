/*
 * The reference's serial CPU colour-gradient loop, driven from C.
 *
 * TEST INFRASTRUCTURE ONLY.  oracle/build_ref.sh compiles this file with the
 * reference's own Multiphase.cu and CellFunctions.cu (read in place, never
 * copied) into oracle/_ref/libref_multiphase.so.  ref_cpu_cg2d replays the
 * CPU branch of Iterate2D's multiphase loop
 * (Source code/lbm-solver_final/Iterate.cu:158-176, :178-207, :393-499):
 * createBubble (test case 1), then per step mp2DColl, streamMP,
 * peridicBoundaries and updateMacroMP.  It serves as the reference's own CPU
 * baseline for the colour-gradient workload; its arithmetic differs from the
 * reference's GPU kernels (which this project follows), so it is timed, not
 * compared.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "ArrayUtils.h"
#include "CellFunctions.h"
#include "FloatType.h"

void mp2DColl(int n, int m, FLOAT_TYPE *rho, FLOAT_TYPE *u, FLOAT_TYPE *v, FLOAT_TYPE *r_f, FLOAT_TYPE *b_f,
              FLOAT_TYPE *r_rho, FLOAT_TYPE *b_rho, FLOAT_TYPE *r_phi, FLOAT_TYPE *b_phi, FLOAT_TYPE *w_pert,
              FLOAT_TYPE *color_gradient, FLOAT_TYPE r_omega, FLOAT_TYPE b_omega, FLOAT_TYPE control_param,
              FLOAT_TYPE del, FLOAT_TYPE beta, FLOAT_TYPE g_limit, FLOAT_TYPE r_A, FLOAT_TYPE b_A,
              FLOAT_TYPE *r_fPert, FLOAT_TYPE *b_fPert, FLOAT_TYPE *weight, int *cx, int *cy, FLOAT_TYPE r_nu,
              FLOAT_TYPE b_nu);
void createBubble(FLOAT_TYPE *x, FLOAT_TYPE *y, int n, int m, FLOAT_TYPE radius, FLOAT_TYPE *r_f, FLOAT_TYPE *b_f,
                  FLOAT_TYPE *r_rho, FLOAT_TYPE *b_rho, FLOAT_TYPE r_density, FLOAT_TYPE b_density,
                  FLOAT_TYPE *r_phi, FLOAT_TYPE *b_phi, FLOAT_TYPE *rho, int test_case);
void updateMacroMP(int n, int m, FLOAT_TYPE *u, FLOAT_TYPE *v, FLOAT_TYPE *r_rho, FLOAT_TYPE *b_rho,
                   FLOAT_TYPE *r_f, FLOAT_TYPE *b_f, FLOAT_TYPE *rho, FLOAT_TYPE control_param, FLOAT_TYPE r_alpha,
                   FLOAT_TYPE b_alpha, FLOAT_TYPE bubble_radius, FLOAT_TYPE *st_error, int iteration,
                   FLOAT_TYPE st_predicted, int test_case);
void peridicBoundaries(int n, int m, FLOAT_TYPE *r_f, FLOAT_TYPE *b_f, FLOAT_TYPE *u, FLOAT_TYPE *v,
                       FLOAT_TYPE *r_rho, FLOAT_TYPE *b_rho, FLOAT_TYPE *rho, int test_case);
void streamMP(int n, int m, FLOAT_TYPE *r_f, FLOAT_TYPE *b_f, FLOAT_TYPE *r_fColl, FLOAT_TYPE *b_fColl);

/* ArrayUtils.h host allocator that Multiphase.cu calls (ArrayUtils.cu is
 * CUDA host code and is not built here). */
FLOAT_TYPE *createHostArrayFlt(int length, ArrayOption op, FLOAT_TYPE fill, FLOAT_TYPE *copy) {
    FLOAT_TYPE *a = (FLOAT_TYPE *)calloc(length > 0 ? (size_t)length : 1u, sizeof(FLOAT_TYPE));
    if (op == ARRAY_FILL) {
        for (int i = 0; i < length; ++i) a[i] = fill;
    } else if (op == ARRAY_COPY && copy) {
        memcpy(a, copy, sizeof(FLOAT_TYPE) * (size_t)length);
    }
    return a;
}

extern "C" {

typedef struct {
    double r_density, b_density, r_alpha, b_alpha, r_viscosity, b_viscosity;
    double beta, A, g_limit, control_param, bubble_radius;
} ref_cpu_cg_params;

/* steps of the reference's CPU colour-gradient loop on an n x m lattice
 * with node coordinates i/(n-1), j/(m-1); returns 0 and the final colour
 * densities (n*m each, may be NULL). */
int ref_cpu_cg2d(int n, int m, const ref_cpu_cg_params *p, int steps, double *out_r_rho, double *out_b_rho) {
    if (n < 3 || m < 3 || !p || steps < 0) return 4;
    const int ms = n * m;
    std::vector<FLOAT_TYPE> x(ms), y(ms), rho(ms, 1), u(ms, 0), v(ms, 0), r_rho(ms, 0), b_rho(ms, 0);
    for (int j = 0; j < m; ++j)
        for (int i = 0; i < n; ++i) {
            x[j * n + i] = (FLOAT_TYPE)i / (FLOAT_TYPE)(n - 1);
            y[j * n + i] = (FLOAT_TYPE)j / (FLOAT_TYPE)(m - 1);
        }
    std::vector<FLOAT_TYPE> r_f(9 * (size_t)ms, 0), b_f(9 * (size_t)ms, 0), r_fc(9 * (size_t)ms, 0),
        b_fc(9 * (size_t)ms, 0), cg(2 * (size_t)ms, 0), st_error(steps > 0 ? steps : 1, 0);
    FLOAT_TYPE r_phi[9], b_phi[9], w_pert[9];
    int cx[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1};
    int cy[9] = {0, 0, 1, 0, -1, 1, 1, -1, -1};
    FLOAT_TYPE weight[9] = {4.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0,
                            1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0};
    w_pert[0] = -4.0 / 27.0;
    r_phi[0] = (FLOAT_TYPE)p->r_alpha;
    b_phi[0] = (FLOAT_TYPE)p->b_alpha;
    for (int i = 1; i < 9; ++i) {
        w_pert[i] = i < 5 ? 2.0 / 27.0 : 5.0 / 108.0;
        r_phi[i] = (FLOAT_TYPE)((1.0 - p->r_alpha) / (i < 5 ? 5.0 : 20.0));
        b_phi[i] = (FLOAT_TYPE)((1.0 - p->b_alpha) / (i < 5 ? 5.0 : 20.0));
    }
    const FLOAT_TYPE aux1 = (FLOAT_TYPE)(p->r_density / ((p->r_density + p->b_density) * p->r_viscosity) +
                                         p->b_density / ((p->r_density + p->b_density) * p->b_viscosity));
    const FLOAT_TYPE mean_nu = 1.0 / aux1;
    const FLOAT_TYPE omega_eff = 1.0 / (3.0 * mean_nu + 0.5);
    const FLOAT_TYPE st_predicted = 4.0 * p->A / 9.0 / omega_eff;
    createBubble(x.data(), y.data(), n, m, (FLOAT_TYPE)p->bubble_radius, r_f.data(), b_f.data(), r_rho.data(),
                 b_rho.data(), (FLOAT_TYPE)p->r_density, (FLOAT_TYPE)p->b_density, r_phi, b_phi, rho.data(), 1);
    for (int it = 0; it < steps; ++it) {
        mp2DColl(n, m, rho.data(), u.data(), v.data(), r_f.data(), b_f.data(), r_rho.data(), b_rho.data(), r_phi,
                 b_phi, w_pert, cg.data(), omega_eff, omega_eff, (FLOAT_TYPE)p->control_param, (FLOAT_TYPE)0.1,
                 (FLOAT_TYPE)p->beta, (FLOAT_TYPE)p->g_limit, (FLOAT_TYPE)p->A, (FLOAT_TYPE)p->A, r_fc.data(),
                 b_fc.data(), weight, cx, cy, (FLOAT_TYPE)p->r_viscosity, (FLOAT_TYPE)p->b_viscosity);
        streamMP(n, m, r_f.data(), b_f.data(), r_fc.data(), b_fc.data());
        peridicBoundaries(n, m, r_f.data(), b_f.data(), u.data(), v.data(), r_rho.data(), b_rho.data(), rho.data(), 1);
        updateMacroMP(n, m, u.data(), v.data(), r_rho.data(), b_rho.data(), r_f.data(), b_f.data(), rho.data(),
                      (FLOAT_TYPE)p->control_param, (FLOAT_TYPE)p->r_alpha, (FLOAT_TYPE)p->b_alpha,
                      (FLOAT_TYPE)p->bubble_radius, st_error.data(), it, st_predicted, 1);
    }
    for (int i = 0; i < ms; ++i) {
        if (out_r_rho) out_r_rho[i] = r_rho[i];
        if (out_b_rho) out_b_rho[i] = b_rho[i];
    }
    return 0;
}

}  // extern "C"
