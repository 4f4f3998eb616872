/*
 * Reference-on-CPU harness.
 *
 * TEST INFRASTRUCTURE ONLY.  oracle/build_ref.sh compiles this file together
 * with the reference solver's own kernel and set-up sources (read in place
 * from the reference tree, never copied) into oracle/_ref/libreflbm_f32.so and
 * oracle/_ref/libreflbm_f64.so.  The harness replays the single-phase time
 * step loops of the reference, calling the reference's __global__ functions
 * once per emulated CUDA thread with the reference's own launch shapes:
 *
 *   2D: Source code/lbm-solver_final/Iterate.cu:211-293 (set-up) and
 *       :385-518 (collision, streaming, inlet, wall, outlet, macro)
 *   3D: Source code/lbm-solver_final/Iterate3D.cu:94-388 (set-up) and
 *       :493-653 (collision, streaming, inlet, wall, outlet, periodic,
 *       symmetry, macro)
 *
 * Emulating threads one at a time is exact for these kernels: every thread
 * writes only its own node (streaming writes f from fColl, boundary kernels
 * rewrite f of their own boundary node), so no kernel reads a value another
 * thread of the same launch writes.  The only product of this file is a
 * golden-vector generator and a pin for the oracle restatement; nothing under
 * thesis_gb300/ links it.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "ArrayUtils.h"
#include "BcMacros.h"
#include "BcMacros3D.h"
#include "CellFunctions.h"
#include "GpuFunctions.h"

thread_local shim_dim3 blockIdx, threadIdx, blockDim, gridDim;

/* ArrayUtils.h host allocator that GpuInit.cu calls for the MRT matrices. */
FLOAT_TYPE *createHostArrayFlt(int length, ArrayOption op, FLOAT_TYPE fill, FLOAT_TYPE *copy) {
    FLOAT_TYPE *a = (FLOAT_TYPE *)calloc(length > 0 ? (size_t)length : 1u, sizeof(FLOAT_TYPE));
    if (op == ARRAY_FILL) {
        for (int i = 0; i < length; ++i) a[i] = fill;
    } else if (op == ARRAY_COPY && copy) {
        memcpy(a, copy, sizeof(FLOAT_TYPE) * (size_t)length);
    }
    return a;
}

template <class Body>
static void launch(shim_dim3 grid, shim_dim3 block, Body body) {
    gridDim = grid;
    blockDim = block;
    for (unsigned bz = 0; bz < grid.z; ++bz)
        for (unsigned by = 0; by < grid.y; ++by)
            for (unsigned bx = 0; bx < grid.x; ++bx) {
                blockIdx = shim_dim3{bx, by, bz};
                for (unsigned tz = 0; tz < block.z; ++tz)
                    for (unsigned ty = 0; ty < block.y; ++ty)
                        for (unsigned tx = 0; tx < block.x; ++tx) {
                            threadIdx = shim_dim3{tx, ty, tz};
                            body();
                        }
            }
}

template <class T>
static void copy_out(void *dst, const std::vector<FLOAT_TYPE> &src) {
    if (!dst) return;
    T *d = (T *)dst;
    for (size_t i = 0; i < src.size(); ++i) d[i] = (T)src[i];
}

extern "C" {

/* Scalar inputs of one run: the fields of the reference's Arguments struct
 * (include/Arguments.h:86-135) that the single-phase loop reads, plus the
 * values Iterate2D/3D derive from the mesh files before initConstants*. */
typedef struct {
    double u, v, w, rho, viscosity, g;
    int inlet_profile;      /* InletProfile: 1 INLET, 2 NO_INLET */
    int outlet_profile;     /* OutletProfile: 1 OUTLET (Zou-He), 2 SECOND, 3 FIRST, 4 HEmodel */
    int collision_model;    /* CollisionModel: 1 BGKW, 2 TRT, 3 MRT */
    int boundary_type;      /* BoundaryType: 1 CURVED, 2 STRAIGHT */
    int bc_wall_model;      /* BCWallModel: 1 SIMPLE, 2 COMPLEX */
    int update_inlet_outlet;
    int boundary_id;
    double delta, min_inlet_y, max_inlet_y, min_inlet_z, max_inlet_z;
} ref_params;

int ref_float_bytes(void) { return (int)sizeof(FLOAT_TYPE); }

static void fill_args(Arguments *a, const ref_params *p) {
    memset(a, 0, sizeof(*a));
    a->u = (FLOAT_TYPE)p->u;
    a->v = (FLOAT_TYPE)p->v;
    a->w = (FLOAT_TYPE)p->w;
    a->rho = (FLOAT_TYPE)p->rho;
    a->viscosity = (FLOAT_TYPE)p->viscosity;
    a->g = (FLOAT_TYPE)p->g;
    a->inletProfile = (InletProfile)p->inlet_profile;
    a->outletProfile = (OutletProfile)p->outlet_profile;
    a->collisionModel = (CollisionModel)p->collision_model;
    a->boundaryType = (BoundaryType)p->boundary_type;
    a->bcwallmodel = (BCWallModel)p->bc_wall_model;
    a->UpdateInltOutl = p->update_inlet_outlet;
    a->boundaryId = p->boundary_id;
    a->multiPhase = 0; /* single-phase loop (main.cu:52 hard-codes 1; patched) */
}

static double l2_residual(const std::vector<FLOAT_TYPE> &f, const std::vector<FLOAT_TYPE> &fc) {
    /* computeResidual2D/3D (ComputeResiduals.cu:13-26): sqrt(sum (f-fColl)^2);
     * accumulated here in double. */
    double s = 0.0;
    for (size_t i = 0; i < f.size(); ++i) {
        double d = (double)f[i] - (double)fc[i];
        s += d * d;
    }
    return sqrt(s);
}

/*
 * Single-phase 2D run.  Node arrays are x-fastest (ind = i + j*n) and are the
 * columns of the Node file; BC arrays are the columns of the BC file.
 * Outputs (any may be NULL) are written as doubles: f/fColl are 9*n*m in the
 * reference's SoA layout f[d*n*m + ind]; bc_mask is the reference's int mask
 * per node; stream is the 8*n*m flag array; resid[steps] the L2 residual.
 */
int ref_run2d(int n, int m, const int *node_type, const double *node_x, const double *node_y,
              int num_conns, const int *bc_i, const int *bc_j, const int *bc_dir,
              const int *bc_type, const int *bc_id, const double *bc_x, const double *bc_y,
              const ref_params *p, int steps, double *out_f, double *out_fcoll,
              double *out_rho, double *out_u, double *out_v, int *out_bc_mask,
              int *out_stream, int *out_bc_count, double *out_resid) {
    const int ms = n * m;
    Arguments args;
    fill_args(&args, p);
    initConstants2D(&args, (FLOAT_TYPE)p->max_inlet_y, (FLOAT_TYPE)p->min_inlet_y,
                    (FLOAT_TYPE)p->delta, m, n);

    std::vector<int> fluid(node_type, node_type + ms);
    std::vector<FLOAT_TYPE> nx(ms), ny(ms);
    for (int i = 0; i < ms; ++i) {
        nx[i] = (FLOAT_TYPE)node_x[i];
        ny[i] = (FLOAT_TYPE)node_y[i];
    }
    std::vector<int> bi(bc_i, bc_i + num_conns), bj(bc_j, bc_j + num_conns);
    std::vector<int> bdir(bc_dir, bc_dir + num_conns), btype(bc_type, bc_type + num_conns);
    std::vector<int> bid(bc_id, bc_id + num_conns);
    std::vector<FLOAT_TYPE> bx(num_conns), by(num_conns);
    for (int i = 0; i < num_conns; ++i) {
        bx[i] = (FLOAT_TYPE)bc_x[i];
        by[i] = (FLOAT_TYPE)bc_y[i];
    }

    /* Iterate.cu:211, :231-240, :244-245, :274-277 */
    std::vector<FLOAT_TYPE> rho(ms, (FLOAT_TYPE)p->rho);
    std::vector<FLOAT_TYPE> u0(ms, 0), v0(ms, 0);
    shim_dim3 tpb{THREADS, 1, 1};
    shim_dim3 bpg1{(unsigned)(ms / THREADS) + 1, 1, 1};
    if (args.inletProfile == NO_INLET) {
        for (int i = 0; i < ms; ++i) {
            u0[i] = args.u;
            v0[i] = args.v;
        }
    }
    if (args.inletProfile == INLET) {
        launch(bpg1, tpb, [&] { gpuInitInletProfile2D(u0.data(), v0.data(), ny.data(), ms); });
    }
    std::vector<FLOAT_TYPE> drag(ms, 0), lift(ms, 0);
    std::vector<FLOAT_TYPE> f(9 * (size_t)ms, 0), fColl(9 * (size_t)ms, 0);
    std::vector<int> mask(ms, 0), bcMask(ms, 0), bcIdx(ms, 0);
    std::vector<FLOAT_TYPE> u(u0), v(v0);
    std::vector<int> stream(8 * (size_t)ms, 1);
    std::vector<FLOAT_TYPE> q(8 * (size_t)ms, (FLOAT_TYPE)0.5);

    int bcCount = initBoundaryConditions2D(bi.data(), bj.data(), q.data(), bid.data(), fluid.data(),
                                           bx.data(), by.data(), nx.data(), ny.data(), bdir.data(),
                                           stream.data(), btype.data(), bcMask.data(), bcIdx.data(),
                                           mask.data(), (FLOAT_TYPE)p->delta, m, n, num_conns);
    std::vector<int> bcIdxC(bcCount > 0 ? bcCount : 1), bcMaskC(bcCount > 0 ? bcCount : 1);
    /* one node's worth of 1/2 past the collapsed table: the curved wall's
     * first coefficient reads one entry ahead, past the end for the last node */
    std::vector<FLOAT_TYPE> qC(8 * (size_t)((bcCount > 0 ? bcCount : 1) + 1), (FLOAT_TYPE)0.5);
    collapseBc2D(bcIdx.data(), bcIdxC.data(), bcMask.data(), bcMaskC.data(), q.data(), qC.data(),
                 mask.data(), m, n, bcCount);
    shim_dim3 bpgB{(unsigned)(bcCount / THREADS) + 1, 1, 1};

    for (int iter = 0; iter < steps; ++iter) {
        switch (args.collisionModel) { /* Iterate.cu:390-418 */
        case BGKW:
            launch(bpg1, tpb, [&] { gpuCollBgkw2D(fluid.data(), rho.data(), u.data(), v.data(), f.data(), fColl.data()); });
            break;
        case TRT:
            launch(bpg1, tpb, [&] { gpuCollTrt(fluid.data(), rho.data(), u.data(), v.data(), f.data(), fColl.data()); });
            break;
        case MRT:
            launch(bpg1, tpb, [&] { gpuCollMrt2D(fluid.data(), rho.data(), u.data(), v.data(), f.data(), fColl.data()); });
            break;
        }
        launch(bpg1, tpb, [&] { gpuStreaming2D(fluid.data(), stream.data(), f.data(), fColl.data()); });
        launch(bpgB, tpb, [&] { gpuBcInlet2D(bcIdxC.data(), bcMaskC.data(), f.data(), u0.data(), v0.data(), bcCount); });
        launch(bpgB, tpb, [&] { gpuBcWall2D(bcIdxC.data(), bcMaskC.data(), f.data(), fColl.data(), qC.data(), bcCount); });
        launch(bpgB, tpb, [&] { gpuBcOutlet2D(bcIdxC.data(), bcMaskC.data(), f.data(), u0.data(), v0.data(), bcCount); });
        launch(bpg1, tpb, [&] {
            gpuUpdateMacro2D(fluid.data(), rho.data(), u.data(), v.data(), bcMask.data(), drag.data(),
                             lift.data(), nx.data(), ny.data(), f.data());
        });
        if (out_resid) out_resid[iter] = l2_residual(f, fColl);
    }

    copy_out<double>(out_f, f);
    copy_out<double>(out_fcoll, fColl);
    copy_out<double>(out_rho, rho);
    copy_out<double>(out_u, u);
    copy_out<double>(out_v, v);
    if (out_bc_mask) memcpy(out_bc_mask, bcMask.data(), sizeof(int) * (size_t)ms);
    if (out_stream) memcpy(out_stream, stream.data(), sizeof(int) * 8 * (size_t)ms);
    if (out_bc_count) *out_bc_count = bcCount;
    return 0;
}

/*
 * Single-phase 3D run (ind = i + j*n + k*n*m).  f/fColl are 19*n*m*h SoA;
 * bc_mask is the reference's 64-bit mask per node; stream is 18*n*m*h flags.
 * inlet_u/v/w (n*m*h, may be NULL) replace the constant u1 fill when given,
 * as a velocity field loaded from an initial-condition file would.
 */
int ref_run3d(int n, int m, int h, const int *node_type, const double *node_x,
              const double *node_y, const double *node_z, int num_conns, const int *bc_i,
              const int *bc_j, const int *bc_k, const int *bc_dir, const int *bc_type,
              const int *bc_id, const double *bc_x, const double *bc_y, const double *bc_z,
              const ref_params *p, int steps, double *out_f, double *out_fcoll,
              double *out_rho, double *out_u, double *out_v, double *out_w,
              unsigned long long *out_bc_mask, unsigned char *out_stream, int *out_bc_count,
              double *out_resid) {
    const int ms = n * m * h;
    Arguments args;
    fill_args(&args, p);
    initConstants3D(&args, (FLOAT_TYPE)p->max_inlet_y, (FLOAT_TYPE)p->min_inlet_y,
                    (FLOAT_TYPE)p->max_inlet_z, (FLOAT_TYPE)p->min_inlet_z, (FLOAT_TYPE)p->delta, m,
                    n, h);

    std::vector<int> fluid(node_type, node_type + ms);
    std::vector<FLOAT_TYPE> nx(ms), ny(ms), nz(ms);
    for (int i = 0; i < ms; ++i) {
        nx[i] = (FLOAT_TYPE)node_x[i];
        ny[i] = (FLOAT_TYPE)node_y[i];
        nz[i] = (FLOAT_TYPE)node_z[i];
    }
    std::vector<int> bi(bc_i, bc_i + num_conns), bj(bc_j, bc_j + num_conns), bk(bc_k, bc_k + num_conns);
    std::vector<int> bdir(bc_dir, bc_dir + num_conns), btype(bc_type, bc_type + num_conns);
    std::vector<int> bid(bc_id, bc_id + num_conns);
    std::vector<FLOAT_TYPE> bx(num_conns), by(num_conns), bz(num_conns);
    for (int i = 0; i < num_conns; ++i) {
        bx[i] = (FLOAT_TYPE)bc_x[i];
        by[i] = (FLOAT_TYPE)bc_y[i];
        bz[i] = (FLOAT_TYPE)bc_z[i];
    }
    if (args.inletProfile == INLET) {
        /* Iterate3D.cu:200-206: the 3D inlet profile is not available. */
        return 3;
    }

    shim_dim3 tpb{THREADS, THREADS, 1};
    unsigned side = (unsigned)(sqrt((double)(m * n * h)) / THREADS) + 1;
    shim_dim3 bpg1{side, side, 1};

    /* Iterate3D.cu:176-199, :301-302, :345-388 */
    std::vector<FLOAT_TYPE> rho(ms, args.rho);
    std::vector<FLOAT_TYPE> u1(ms, args.u), v1(ms, args.v), w1(ms, args.w);
    std::vector<FLOAT_TYPE> f(19 * (size_t)ms, 0), fColl(19 * (size_t)ms, 0);
    std::vector<int> mask(ms, 0), bcIdx(ms, 0);
    std::vector<unsigned long long> bcMask(ms, 0ull);
    std::vector<FLOAT_TYPE> u(u1), v(v1), w(w1);
    std::vector<unsigned char> streamBytes(18 * (size_t)ms, 1);
    bool *stream = (bool *)malloc(sizeof(bool) * 18 * (size_t)ms);
    for (size_t i = 0; i < 18 * (size_t)ms; ++i) stream[i] = true;
    std::vector<FLOAT_TYPE> q(18 * (size_t)ms, (FLOAT_TYPE)0.5);

    int bcCount = initBoundaryConditions3D(bi.data(), bj.data(), bk.data(), q.data(), bid.data(),
                                           fluid.data(), bx.data(), by.data(), bz.data(), nx.data(),
                                           ny.data(), nz.data(), bdir.data(), stream, btype.data(),
                                           bcMask.data(), bcIdx.data(), mask.data(),
                                           (FLOAT_TYPE)p->delta, m, n, h, num_conns,
                                           args.boundaryType);
    int cap = bcCount > 0 ? bcCount : 1;
    std::vector<int> bcIdxC(cap);
    std::vector<unsigned long long> bcMaskC(cap);
    std::vector<FLOAT_TYPE> qC(18 * (size_t)(cap + 1), (FLOAT_TYPE)0.5); /* as in 2D: one node past the end */
    collapseBc3D(bcIdx.data(), bcIdxC.data(), bcMask.data(), bcMaskC.data(), q.data(), qC.data(),
                 mask.data(), m, n, h, bcCount, args.boundaryType);
    unsigned sideB = (unsigned)(sqrt((double)bcCount) / THREADS) + 1;
    shim_dim3 bpgB{sideB, sideB, 1};
    /* gpuUpdateMacro3D reads bcMask_d indexed by node and the BC id by node. */
    std::vector<int> bcBoundIdNode(ms, 0);

    for (int iter = 0; iter < steps; ++iter) {
        switch (args.collisionModel) { /* Iterate3D.cu:497-526 */
        case BGKW:
            launch(bpg1, tpb, [&] { gpuCollBgkw3D(fluid.data(), rho.data(), u.data(), v.data(), w.data(), f.data(), fColl.data()); });
            break;
        case TRT:
            break; /* "TRT not implemented in 3D" (Iterate3D.cu:517-520) */
        case MRT:
            launch(bpg1, tpb, [&] { gpuCollMrt3D(fluid.data(), rho.data(), u.data(), v.data(), w.data(), f.data(), fColl.data()); });
            break;
        }
        launch(bpg1, tpb, [&] { gpuStreaming3D(fluid.data(), stream, f.data(), fColl.data()); });
        launch(bpgB, tpb, [&] { gpuBcInlet3D(bcIdxC.data(), bcMaskC.data(), f.data(), u1.data(), v1.data(), w1.data(), bcCount); });
        if (args.bcwallmodel == SIMPLE)
            launch(bpgB, tpb, [&] { gpuBcSimpleWall3D(bcIdxC.data(), bcMaskC.data(), f.data(), fColl.data(), qC.data(), bcCount); });
        else
            launch(bpgB, tpb, [&] { gpuBcComplexWall3D(bcIdxC.data(), bcMaskC.data(), f.data(), fColl.data(), qC.data(), bcCount); });
        launch(bpgB, tpb, [&] { gpuBcOutlet3D(bcIdxC.data(), bcMaskC.data(), f.data(), u.data(), v.data(), w.data(), rho.data(), bcCount); });
        launch(bpgB, tpb, [&] { gpuBcPeriodic3D(bcIdxC.data(), bcMaskC.data(), f.data(), bcCount); });
        launch(bpgB, tpb, [&] { gpuBcSymm3D(bcIdxC.data(), bcMaskC.data(), f.data(), bcCount); });
        launch(bpg1, tpb, [&] {
            gpuUpdateMacro3D(fluid.data(), rho.data(), u.data(), v.data(), w.data(), bcBoundIdNode.data(),
                             nx.data(), ny.data(), nz.data(), f.data(), args.g, bcMask.data(),
                             args.UpdateInltOutl);
        });
        if (out_resid) out_resid[iter] = l2_residual(f, fColl);
    }

    copy_out<double>(out_f, f);
    copy_out<double>(out_fcoll, fColl);
    copy_out<double>(out_rho, rho);
    copy_out<double>(out_u, u);
    copy_out<double>(out_v, v);
    copy_out<double>(out_w, w);
    if (out_bc_mask) memcpy(out_bc_mask, bcMask.data(), sizeof(unsigned long long) * (size_t)ms);
    if (out_stream)
        for (size_t i = 0; i < 18 * (size_t)ms; ++i) out_stream[i] = stream[i] ? 1 : 0;
    if (out_bc_count) *out_bc_count = bcCount;
    free(stream);
    (void)streamBytes;
    return 0;
}

/* Colour-gradient parameters (the multiphase fields of Arguments,
 * include/Arguments.h:113-128). */
typedef struct {
    double r_density, b_density, r_alpha, b_alpha, r_viscosity, b_viscosity;
    double beta, A, g_limit, control_param, g;
    int high_order, enhanced, external_force;
} ref_cg_params;

/* One call of the reference's gpuCollBgkwGC2D / gpuCollEnhancedBgkwGC2D
 * (GpuCollision.cu:552-707) on given fields; out_cgdir receives the
 * reference's gradient-direction map (GpuInit.cu:206-260). */
int ref_cg2d_collide(int n, int m, const ref_cg_params *cp, const double *rho, const double *r_rho,
                     const double *b_rho, const double *u, const double *v, const double *f,
                     double *out_rfc, double *out_bfc, int *out_cgdir) {
    const int ms = n * m;
    Arguments args;
    memset(&args, 0, sizeof(args));
    args.viscosity = (FLOAT_TYPE)0.1;
    args.multiPhase = 1;
    args.r_density = (FLOAT_TYPE)cp->r_density;
    args.b_density = (FLOAT_TYPE)cp->b_density;
    args.r_alpha = (FLOAT_TYPE)cp->r_alpha;
    args.b_alpha = (FLOAT_TYPE)cp->b_alpha;
    args.r_viscosity = (FLOAT_TYPE)cp->r_viscosity;
    args.b_viscosity = (FLOAT_TYPE)cp->b_viscosity;
    args.beta = (FLOAT_TYPE)cp->beta;
    args.A = (FLOAT_TYPE)cp->A;
    args.g_limit = (FLOAT_TYPE)cp->g_limit;
    args.control_param = (FLOAT_TYPE)cp->control_param;
    args.g = (FLOAT_TYPE)cp->g;
    args.external_force = cp->external_force != 0;
    args.bubble_radius = (FLOAT_TYPE)1.0;
    initConstants2D(&args, 0, 0, 1, m, n);
    std::vector<int> cgdir(ms, 0);
    if (cp->high_order)
        initHOColorGradient(cgdir.data(), n, m);
    else
        initColorGradient(cgdir.data(), n, m);
    std::vector<FLOAT_TYPE> R(ms), RR(ms), BR(ms), U(ms), V(ms), F(9 * (size_t)ms), RC(9 * (size_t)ms, 0),
        BC(9 * (size_t)ms, 0);
    for (int i = 0; i < ms; ++i) {
        R[i] = (FLOAT_TYPE)rho[i];
        RR[i] = (FLOAT_TYPE)r_rho[i];
        BR[i] = (FLOAT_TYPE)b_rho[i];
        U[i] = (FLOAT_TYPE)u[i];
        V[i] = (FLOAT_TYPE)v[i];
    }
    for (size_t k = 0; k < 9 * (size_t)ms; ++k) F[k] = (FLOAT_TYPE)f[k];
    shim_dim3 tpb{THREADS, 1, 1};
    shim_dim3 bpg1{(unsigned)(ms / THREADS) + 1, 1, 1};
    launch(bpg1, tpb, [&] {
        if (cp->enhanced)
            gpuCollEnhancedBgkwGC2D(R.data(), RR.data(), BR.data(), U.data(), V.data(), F.data(), RC.data(),
                                    BC.data(), cgdir.data(), cp->high_order != 0);
        else
            gpuCollBgkwGC2D(R.data(), RR.data(), BR.data(), U.data(), V.data(), F.data(), RC.data(), BC.data(),
                            cgdir.data(), cp->high_order != 0);
    });
    for (size_t k = 0; k < 9 * (size_t)ms; ++k) {
        out_rfc[k] = RC[k];
        out_bfc[k] = BC[k];
    }
    if (out_cgdir) memcpy(out_cgdir, cgdir.data(), sizeof(int) * (size_t)ms);
    return 0;
}

/* One D3Q19 colour-gradient collision by gpuCollBgkwGC3D /
 * gpuCollEnhancedBgkwGC3D (GpuCollision.cu:709-880) on given fields, with
 * the reference's gradient-direction map (GpuInit.cu:262-321) in
 * out_cgdir. */
int ref_cg3d_collide(int n, int m, int h, const ref_cg_params *cp, const double *rho, const double *r_rho,
                     const double *b_rho, const double *u, const double *v, const double *w, const double *f,
                     double *out_rfc, double *out_bfc, int *out_cgdir) {
    const int ms = n * m * h;
    Arguments args;
    memset(&args, 0, sizeof(args));
    args.viscosity = (FLOAT_TYPE)0.1;
    args.multiPhase = 1;
    args.r_density = (FLOAT_TYPE)cp->r_density;
    args.b_density = (FLOAT_TYPE)cp->b_density;
    args.r_alpha = (FLOAT_TYPE)cp->r_alpha;
    args.b_alpha = (FLOAT_TYPE)cp->b_alpha;
    args.r_viscosity = (FLOAT_TYPE)cp->r_viscosity;
    args.b_viscosity = (FLOAT_TYPE)cp->b_viscosity;
    args.beta = (FLOAT_TYPE)cp->beta;
    args.A = (FLOAT_TYPE)cp->A;
    args.g_limit = (FLOAT_TYPE)cp->g_limit;
    args.control_param = (FLOAT_TYPE)cp->control_param;
    args.g = (FLOAT_TYPE)cp->g;
    args.external_force = cp->external_force != 0;
    args.bubble_radius = (FLOAT_TYPE)1.0;
    initConstants3D(&args, 0, 0, 0, 0, 1, m, n, h);
    std::vector<int> cgdir(ms, 0), fluid(ms, 1);
    if (cp->high_order)
        initHOColorGradient3D(cgdir.data(), n, m, h);
    else
        initColorGradient3D(cgdir.data(), n, m, h);
    std::vector<FLOAT_TYPE> R(ms), RR(ms), BR(ms), U(ms), V(ms), W(ms), F(19 * (size_t)ms),
        RC(19 * (size_t)ms, 0), BC(19 * (size_t)ms, 0);
    for (int i = 0; i < ms; ++i) {
        R[i] = (FLOAT_TYPE)rho[i];
        RR[i] = (FLOAT_TYPE)r_rho[i];
        BR[i] = (FLOAT_TYPE)b_rho[i];
        U[i] = (FLOAT_TYPE)u[i];
        V[i] = (FLOAT_TYPE)v[i];
        W[i] = (FLOAT_TYPE)w[i];
    }
    for (size_t k = 0; k < 19 * (size_t)ms; ++k) F[k] = (FLOAT_TYPE)f[k];
    shim_dim3 tpb{THREADS, THREADS, 1};
    unsigned side = (unsigned)(sqrt((double)ms) / THREADS) + 1;
    shim_dim3 bpg1{side, side, 1};
    launch(bpg1, tpb, [&] {
        if (cp->enhanced)
            gpuCollEnhancedBgkwGC3D(fluid.data(), R.data(), RR.data(), BR.data(), U.data(), V.data(), W.data(),
                                    F.data(), RC.data(), BC.data(), cgdir.data(), cp->high_order != 0);
        else
            gpuCollBgkwGC3D(fluid.data(), R.data(), RR.data(), BR.data(), U.data(), V.data(), W.data(), F.data(),
                            RC.data(), BC.data(), cgdir.data(), cp->high_order != 0);
    });
    for (size_t k = 0; k < 19 * (size_t)ms; ++k) {
        out_rfc[k] = RC[k];
        out_bfc[k] = BC[k];
    }
    if (out_cgdir) memcpy(out_cgdir, cgdir.data(), sizeof(int) * (size_t)ms);
    return 0;
}

/* The reference's MRT matrices (CellFunctions.cu:7-153) for a given omega. */
void ref_mrt_matrices(int q, double omega, double *vel_mom_map, double *mom_coll_mtx) {
    int n = q * q;
    std::vector<FLOAT_TYPE> a(n), b(n);
    if (q == 9)
        MRTInitializer2D(a.data(), b.data(), (FLOAT_TYPE)omega);
    else
        MRTInitializer3D(a.data(), b.data(), (FLOAT_TYPE)omega);
    for (int i = 0; i < n; ++i) {
        vel_mom_map[i] = a[i];
        mom_coll_mtx[i] = b[i];
    }
}

} /* extern "C" */
