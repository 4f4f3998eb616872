/*
 * thesis_lbm.h -- C ABI of the GB300 lattice-Boltzmann time-step engine.
 *
 * Drop-in for the time-step loop of the reference solver
 * (ZPaulo/Thesis, "Source code/lbm-solver_final"):
 *
 *   int Iterate2D(InputFilenames*, Arguments*)   include/Iterate.h:64
 *   int Iterate3D(InputFilenames*, Arguments*)   include/Iterate.h:65
 *
 * The reference runs collision, streaming, boundary and macroscopic kernels
 * per step (Iterate3D.cu:493-653) on state it allocates itself.  This library
 * keeps the same inputs -- the columns of the Node and BC lattice files and the
 * Arguments fields the loop reads -- and runs one fused CUDA kernel per step.
 *
 * Conventions: plain pointers and sizes only; host buffers are owned by the
 * caller, device buffers by the handle; every call returns a status code
 * (never exits the process); one handle per host thread.
 */
#ifndef THESIS_LBM_H
#define THESIS_LBM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  1 and 2 keep the meaning of Iterate2D/3D's return values
 * (Iterate.cu:563, Iterate3D.cu:89-105). */
#define LBM_OK 0
#define LBM_DIVERGED 1
#define LBM_ERR_FILE 2
#define LBM_ERR_UNSUPPORTED 3
#define LBM_ERR_INVALID 4
#define LBM_ERR_CUDA 5
#define LBM_ERR_NOMEM 6

/* Population storage in HBM.  Arithmetic is FP32 for F32, F16S and F16C,
 * FP64 for F64.  F16S stores (f_i - w_i) * scale as IEEE half.  F16C stores
 * the same scaled deviation in a 16-bit float with 4 exponent and 11
 * mantissa bits (one significand bit more than IEEE half; the "FP16C" format
 * of Lehmann et al., Phys. Rev. E 106, 015308 (2022)): normal range
 * [2^-14, 2), subnormal step 2^-25, so |f_i - w_i| * scale must stay below 2
 * (scale defaults to 256 for F16C, 8 for the D3Q19 MRT whose equilibrium
 * start lies 0.143 from its rest state; values beyond saturate); physics mode and
 * the run-time specialised storage-unit kernels only. */
#define LBM_STORE_F32 0
#define LBM_STORE_F16S 1
#define LBM_STORE_F64 2
#define LBM_STORE_F16C 3

/* Semantics.  REFERENCE reproduces the reference loop including its quirks
 * (zero initial populations, post-stream wall copies, the lid Zou-He with
 * rho*u/6, D3Q19 MRT without direction 18, ...).  PHYSICS uses the standard
 * forms: half-way bounce-back, mass-balanced Zou-He velocity and pressure
 * faces, all 19 MRT outputs, TRT in 3D. */
#define LBM_MODE_REFERENCE 0
#define LBM_MODE_PHYSICS 1

/* Values of the reference's enums (include/Arguments.h:14-56). */
#define LBM_BGKW 1
#define LBM_TRT 2
#define LBM_MRT 3
#define LBM_INLET 1            /* InletProfile INLET (parabolic, 2D)        */
#define LBM_NO_INLET 2         /* InletProfile NO_INLET (constant u, v, w)  */
#define LBM_INLET_PRESSURE 4   /* extension: Zou-He pressure inlet, rho_in  */
#define LBM_OUTLET_ZOUHE 1     /* OutletProfile OUTLET                      */
#define LBM_OUTLET_SECOND 2
#define LBM_OUTLET_FIRST 3
#define LBM_OUTLET_HEMODEL 4
#define LBM_OUTLET_PRESSURE 5  /* extension: Zou-He pressure outlet, rho_out */
#define LBM_CURVED 1
#define LBM_STRAIGHT 2
#define LBM_WALL_SIMPLE 1
#define LBM_WALL_COMPLEX 2

/* BC file link types (latticegen: WALL/INLE/OUTL/CYCL/SYMP -> 1..5). */
#define LBM_BC_WALL 1
#define LBM_BC_INLET 2
#define LBM_BC_OUTLET 3
#define LBM_BC_PERIODIC 4
#define LBM_BC_SYMMETRY 5

/* The constants above are shared with the CUDA kernels, which the library
 * also compiles at run time (NVRTC), where host declarations are not allowed. */
#ifndef __CUDACC_RTC__

typedef struct lbm_handle_s *lbm_handle;

/* A lattice as the reference reads it: the Node file columns (i, j, [k,]
 * fluid) laid out x fastest, and the BC file columns (i, j, [k,] dir, type,
 * id) -- FilesReading.cu:270-347. */
typedef struct lbm_lattice_desc {
    int dims;                 /* 2 or 3 */
    int n, m, h;              /* nodes along x, y, z (h = 1 in 2D) */
    const int *node_type;     /* n*m*h entries: 1 fluid, 0 solid */
    int num_conns;            /* number of BC links */
    const int *bc_i, *bc_j;   /* node of each link */
    const int *bc_k;          /* NULL in 2D */
    const int *bc_dir;        /* lattice direction from the node into the boundary */
    const int *bc_type;       /* LBM_BC_* */
    const int *bc_id;         /* boundary id (2D drag/lift), may be NULL */
} lbm_lattice_desc;

/* The Arguments fields the time-step loop reads (include/Arguments.h:86-135),
 * plus this engine's options. */
typedef struct lbm_params {
    double u, v, w;           /* inlet / initial velocity */
    double rho;               /* initial density */
    double viscosity;         /* omega = 1 / (3 nu + 0.5) */
    double g;                 /* 3D body force, applied as u += g / omega */
    int inlet_profile;        /* LBM_NO_INLET, LBM_INLET_PRESSURE */
    int outlet_profile;       /* LBM_OUTLET_* */
    int collision_model;      /* LBM_BGKW, LBM_TRT, LBM_MRT */
    int boundary_type;        /* LBM_STRAIGHT, or LBM_CURVED: the reference's q-interpolated
                                 walls (reference mode, simple wall model; link fractions
                                 from lbm_set_link_q, 1/2 until then) */
    int bc_wall_model;        /* LBM_WALL_SIMPLE, or LBM_WALL_COMPLEX: the reference's HH wall
                                 (gpuBcComplexWall3D, GpuBoundaries.cu:492-1560), reference
                                 mode only; the reference's 2D loop has straight walls only */
    int update_inlet_outlet;  /* UpdateInltOutl */
    int mode;                 /* LBM_MODE_REFERENCE or LBM_MODE_PHYSICS */
    int storage;              /* LBM_STORE_* */
    double rho_in, rho_out;   /* pressure faces */
    double f16_scale;         /* F16S scale; 0 selects 1024 */
    int periodic[3];          /* physics mode: periodic x, y, z (reference mode follows the BC
                                 file's periodic links with the reference's copies from the
                                 opposite face, gpuBcPeriodic3D, GpuBoundaries.cu:2025-2084) */
    int init_equilibrium;     /* 0: f starts at 0 (reference); 1: f_eq(rho, u) */
} lbm_params;

/* Build a solver from a lattice description.  Computes the reference's BC
 * masks and streaming flags (GpuInit.cu:1055-1277), derives the per-node flag
 * words, allocates device state and uploads it. */
int lbm_create(const lbm_lattice_desc *lattice, const lbm_params *params, lbm_handle *out);

/* Per-node inlet/outlet velocity field (the reference's u0/u1 arrays); any
 * NULL component keeps the constant from params.  Host arrays of n*m*h. */
int lbm_set_inlet_velocity(lbm_handle h, const float *u, const float *v, const float *w);

/* Curved walls (boundary_type LBM_CURVED): the fraction q of each BC link
 * (num_conns values in the lattice's link order) at which the wall cuts the
 * link from the node, |node -> wall| / |c_dir| in lattice spacings.  The
 * reference computes q in initBoundaryConditions2D/3D (GpuInit.cu:1086-1088,
 * :1203-1207; links without an entry keep 1/2) and applies the CURVED
 * branch of gpuBcWall2D / gpuBcSimpleWall3D (GpuBoundaries.cu:414-432,
 * :461-479) on every wall link of a fluid node, interpolating between the
 * last step's post-collision populations (f* at the node and at its
 * upstream neighbour, or f* at the node and its opposite, for q < 1/2 and
 * q >= 1/2).  The reference's first coefficient of the q < 1/2 branch reads
 * the next entry of its per-node table (link dir+1; for the last direction
 * the next boundary node's first link, 1/2 past the last node), and it
 * reads the upstream value at the flat index node + dir N + c(dir) of its
 * direction-major array, which for a node whose upstream neighbour lies
 * outside the lattice is a neighbouring row's or another direction's value;
 * this engine does the same (0 past either end of the array, where the
 * reference's read is undefined).  Takes effect from the next step.  LBM_ERR_UNSUPPORTED
 * when the handle has no curved walls (straight walls, physics mode, or the
 * HH wall model, whose reference kernel has no curved branch). */
int lbm_set_link_q(lbm_handle h, const double *q);

/* The reference's link fractions from coordinates: q[c] = |B_c - X_c| /
 * (delta |c_dir|), B_c the BC file's boundary point of link c and X_c the
 * Node file's coordinates of its node (node_x/y/z hold n*m*h values indexed
 * by node, x fastest; bc_k, bc_z, node_z NULL in 2D), delta the grid spacing
 * (getGridSpacing, FilesReading.cu:473-489).  FP64 arithmetic.  Host only. */
int lbm_link_q(int dims, int n, int m, int h, int num_conns, const int *bc_i, const int *bc_j, const int *bc_k,
               const int *bc_dir, const float *bc_x, const float *bc_y, const float *bc_z, const float *node_x,
               const float *node_y, const float *node_z, double delta, double *q);

/* Initial macroscopic state (NULL = constant from params) and the first
 * collision, which produces the state lbm_step advances. */
int lbm_init(lbm_handle h, const float *rho, const float *u, const float *v, const float *w);

/* Advance nsteps time steps on `stream` (a cudaStream_t; NULL = the
 * handle's own stream).  write_macro_last: store rho, u on the last step. */
int lbm_step(lbm_handle h, int nsteps, int write_macro_last, void *stream);

/* Wait for queued steps, then copy the macroscopic fields written by the
 * last step that stored them into host arrays of n*m*h (any may be NULL). */
int lbm_get_macro(lbm_handle h, float *rho, float *u, float *v, float *w);

/* Copy the post-collision populations into a host array of Q*n*m*h doubles,
 * SoA f[d*n*m*h + node] in the reference's direction order. */
int lbm_get_populations(lbm_handle h, double *f);

/* Restart from a population field: replace the state with f (the layout
 * lbm_get_populations returns), encoded into the handle's storage.  Takes
 * the place of lbm_init; the residual snapshots (norms, MaxMacroDiff,
 * FdRelDiff) start again from zero fields.  A field read back by
 * lbm_get_populations is restored exactly except where a shifted storage's
 * deviation f - shift is below ~1e-16 of the shift (FP64 cannot hold
 * shift + deviation there); lbm_get_state / lbm_set_state are the exact
 * checkpoint.  The reference restarts from macroscopic fields only
 * (FilesReading.cu:224-268); these are the population-level counterparts. */
int lbm_set_populations(lbm_handle h, const double *f);

/* Exact checkpoint: the stored populations as they are held (F32, F64, or
 * F16S half deviations; lbm_state_bytes(h) bytes, SoA order state[d N +
 * node] of the storage element type).  A state saved by lbm_get_state and
 * loaded by lbm_set_state into a handle of the same lattice and parameters
 * continues bit for bit as the uninterrupted run; lbm_set_state takes the
 * place of lbm_init as lbm_set_populations does. */
long long lbm_state_bytes(lbm_handle h);
int lbm_get_state(lbm_handle h, void *state);
int lbm_set_state(lbm_handle h, const void *state);

/* FP64 norms over fluid nodes of the last stored macroscopic fields:
 * out[0] = sum |u - u_prev|^2, out[1] = sum |u|^2, out[2] = sum rho,
 * out[3] = number of fluid nodes, out[4] = sum rho*ux.  u_prev is the field
 * at the previous call (zero before the first).  Deterministic.  Returns
 * LBM_DIVERGED when a sum is not finite. */
#define LBM_NORMS 5
int lbm_macro_norms(lbm_handle h, double *out);

/* The reference's L2 residual (computeResidual2D/3D, ComputeResiduals.cu:13-26,
 * used when ResidualModel = L2): sqrt(sum over all populations of
 * (f - fColl)^2), fColl the post-collision state the last step left and f the
 * post-stream, post-boundary field the next step will pull from it.  Summed
 * in FP64 (the reference sums in FP32).  LBM_DIVERGED when not finite. */
int lbm_residual_l2(lbm_handle h, double *out);

/* The reference's FdRelDiff residual (ResidualModel = MaxRelativeFdDiff:
 * computeNewResidual3D / gpu_NewResidual, ComputeResiduals.cu:28-36, :56-64,
 * Iterate3D.cu:677-692): max over fluid nodes and directions of
 * |f - f_prev| / |f_first|, f the post-stream, post-boundary populations the
 * next step pulls, f_prev those at the previous call and f_first those at
 * the first call after lbm_init; the first call records both snapshots and
 * returns 0 (it allocates 2 Q N floats).  Entries with f_first = 0 are
 * skipped (the reference divides by zero there); the maximum is exact (the
 * reference's reduction adds on load, GpuSum.cu:160).  LBM_DIVERGED when a
 * population is not finite. */
int lbm_residual_fd_rel_diff(lbm_handle h, double *out);

/* Drag and lift by momentum exchange (physics mode): the force on the solid
 * nodes inside box = {x0, x1, y0, y1, z0, z1} (inclusive node indices), from
 * every bounced-back link of a fluid node into one of them, 2 c f* per link
 * and step, f* the post-collision state the last step left; force[0..2] in
 * lattice units, FP64 sums.  The reference's drag/lift (GpuUpdateMacro.cu:
 * 33-38) integrates a hard-wired pressure expression over the nodes of a
 * boundary id instead; this is the standard link-based force. */
int lbm_momentum_exchange(lbm_handle h, const int *box, double *force);

/* The reference's 2D drag and lift sums (gpuUpdateMacro2D,
 * GpuUpdateMacro.cu:33-38, summed by computeDragLift2D, ComputeResiduals.cu:
 * 39-45, into the Drag and Lift columns of its residual file): over the fluid
 * nodes whose BC mask carries boundary id boundary_id, out[0] =
 * sum 0.33333333 rho (20 - x) 0.2 and out[1] = sum 0.33333333 rho (20 - y) 0.2,
 * rho the last stored density and x, y the Node file's coordinates
 * (node_x/y hold n*m values by node).  A hard-wired expression of the
 * reference, not a force; lbm_momentum_exchange is the physical one.  Zero
 * for boundary_id <= 0 and in 3D, where the reference's loop has no such
 * term.  Per-node terms rounded to FP32 as the reference stores them, FP64
 * sum. */
int lbm_reference_drag_lift(lbm_handle h, int boundary_id, const float *node_x, const float *node_y, double *out);

/* The reference's MaxMacroDiff residual (Iterate3D.cu:696-735): out[0..3] =
 * max over all nodes of |u - u_prev|, |v - v_prev|, |w - w_prev|,
 * |rho - rho_prev| for the last stored macroscopic fields, where _prev is the
 * field at the previous call (the initial fields before the first); out[4] =
 * number of non-finite differences.  Returns LBM_DIVERGED when out[4] > 0. */
int lbm_macro_diff(lbm_handle h, double *out);

/* The same FP64 norms as lbm_macro_norms, for callers that must not allocate
 * device memory while they run (for example a host framework that owns a
 * fixed device arena and forbids cudaMalloc/cudaFree inside its step
 * callback, where allocation would synchronise the device or could fail).
 * This function has no counterpart in the reference.  All pointers are
 * device pointers the caller owns: the flag words and macroscopic fields of
 * n nodes, the previous-velocity arrays (read, then overwritten with u, v, w)
 * and `out`, LBM_NORMS doubles.  It allocates nothing: its per-block partial
 * sums live in a static device array (160 KiB per device context, kept until
 * the process exits), so n is limited to lbm_noalloc_max_nodes() (67,108,864)
 * and larger calls return LBM_ERR_INVALID.  Calls share that array, so calls
 * that overlap on the GPU race and must be serialised.  The first call on a
 * device looks up the array's address and keeps it; make it before any
 * stream capture.  That address lives as long as the device's context: after
 * cudaDeviceReset on a device, do not call this function on it again in the
 * same process.  A CUDA error pending at entry or raised by the launches
 * returns LBM_ERR_CUDA (message in lbm_noalloc_last_error()); pending errors
 * are left for the caller's own checks, not cleared.
 * Work is queued on `stream` (a cudaStream_t, NULL = legacy default). */
int lbm_fluid_norms_noalloc(const uint32_t *word, const float *rho, const float *u, const float *v,
                            const float *w, float *u_prev, float *v_prev, float *w_prev, long long n,
                            double *out, void *stream);
long long lbm_noalloc_max_nodes(void);
const char *lbm_noalloc_last_error(void);

/* Sticky status of the handle (LBM_OK, LBM_DIVERGED, LBM_ERR_CUDA). */
int lbm_status(lbm_handle h);

/* Number of fluid nodes (the lattice updates one step performs). */
long long lbm_fluid_nodes(lbm_handle h);

/* Step kernel of the handle, chosen at lbm_create: 4 (the default) the
 * one-node kernel specialised for this lattice's extents at run time (in
 * physics mode computing in storage units, deviations from the rest state;
 * THESIS_LBM_KERNEL=jith|jitf forces storage-unit or f-space, jiths the
 * storage-unit kernel that loads pull and bounce-back values before the flag
 * word arrives), 1 the
 * compiled-in one-node kernel (used when the run-time build is unavailable),
 * 2 two nodes per thread (even n, F32/F16S), 3 the row-staged bulk-copy
 * kernel.  THESIS_LBM_KERNEL=scalar|pair|tma|jit|jit2 in the environment at
 * lbm_create selects one (jit2: the run-time specialised two-node kernel); a
 * variant the lattice does not admit falls back to 1, except jit and jit2,
 * whose build failure lbm_create reports. */
int lbm_kernel_variant(lbm_handle h);

/* Empty when the handle runs the kernel lbm_create meant to use; otherwise
 * why it fell back (the run-time specialised kernel could not be built, for
 * example without NVRTC or the toolkit headers it compiles against), in
 * which case the handle runs the compiled-in one-node kernel, about 1.4x
 * slower.  The first fallback in a process is also printed on stderr; with
 * the environment variable THESIS_LBM_REQUIRE_JIT=1, lbm_create fails
 * instead (LBM_ERR_CUDA).  No counterpart in the reference. */
const char *lbm_kernel_warning(lbm_handle h);

/* Autotuner of the run-time specialised kernel: builds its variants (one
 * node per thread with blocks of 128 or 256 threads along x, plain or
 * L2-256-byte-prefetching loads, bounce-back by selected address or by
 * predicated loads; and, for even n with F32/F16S storage, two nodes per
 * thread with blocks of 64 or 128), times trial_steps steps of each on the
 * handle's stream and keeps the fastest, also for handles created later in
 * the process on the same lattice and parameters.  The trial steps leave the
 * populations undefined: call lbm_init afterwards.  The chosen knobs go to
 * block, hint (bit 0 L2-256-byte loads, bit 1 arithmetic in storage units,
 * one node per thread; bits 2 and up, storage units: nodes a thread updates
 * along z with the next flag word loaded ahead, 0 for one) and pred (bit 0
 * predicated bounce-back, or in storage units loads issued before the flag
 * word arrives; bit 1 two nodes per thread; bits 2 and up the minimum
 * resident blocks per SM asked of the register allocator, 0 for none); each
 * may be NULL.  In physics mode with
 * F32 storage only storage-unit variants are candidates (their moments come
 * from deviations from the rest state).  This function has no
 * counterpart in the reference. */
int lbm_autotune(lbm_handle h, int trial_steps, int *block, int *hint, int *pred);
/* The knobs of the handle's step kernel (defaults 128, 0, 0). */
int lbm_kernel_config(lbm_handle h, int *block, int *hint, int *pred);

/* Compile (no GPU needed, nothing is loaded) the run-time specialised step
 * kernel for the given template arguments and knobs (as lbm_autotune; pred
 * bit 1 selects the two-node kernel): a build check of the sources the
 * library embeds.  Returns LBM_OK or LBM_ERR_CUDA with the compiler log in
 * lbm_last_error(). */
int lbm_jit_check(int q, int coll, int storage, int phys, int wrap, int nx, int ny, int nz, int block, int hint,
                  int pred);

/* Bytes of HBM one step moves per fluid node for the populations alone. */
int lbm_bytes_per_update(lbm_handle h);

/* Message of the last failing call on this thread. */
const char *lbm_last_error(void);

void lbm_destroy(lbm_handle h);

/* Host only, needs no GPU: the reference's BC masks (one uint64 per node; 2D
 * masks in the low 32 bits), this engine's flag words (one uint32 per node:
 * bit 0 fluid, bit d blocked pull of direction d, bit 19 boundary slot) and
 * slot indices (int32 per node, -1 for none), and the number of nodes with BC
 * links.  Any output pointer may be NULL. */
int lbm_build_flags(const lbm_lattice_desc *lattice, const lbm_params *params, uint64_t *mask,
                    uint32_t *word, int32_t *slot, int *num_bc_nodes);

/* Lattice generator: STAR-CD geometry (.vrt vertices, .bnd quadrilateral
 * boundary faces) to the Node and BC files the solver reads, byte-identical to
 * the reference generator `latticegen <geom> <n> <xseed> <yseed> <zseed>
 * <out> <1|2>` (latticegen2_W8/main.cpp:19-66, FluidTracking.cpp:24-236).
 * n_x: nodes along x; seed: a point inside the fluid; complexity 1 writes a
 * boundary link when first met, 2 after the flood fill.  out_dims (may be
 * NULL) receives n, m, h. */
int lbm_latticegen(const char *vrt_path, const char *bnd_path, int n_x, double xseed, double yseed,
                   double zseed, int complexity, const char *node_path, const char *bc_path,
                   int *out_dims);
const char *lbm_latticegen_error(void);

/* ---- Batched independent domains -------------------------------------------
 * Many lattices of uneven sizes (a sweep over geometry and Reynolds number)
 * advanced together: one persistent launch per step over a packed table of
 * row tiles of all active domains, long runs replayed from a captured CUDA
 * graph, per-domain FP64 residuals, converged domains retired from the table.
 * The reference runs one lattice per process; this has no counterpart there.
 * All domains share dims, collision model and storage (F32 or F16S) and run
 * in physics mode; each has its own extents, viscosity, velocities and
 * boundary links. */
typedef struct lbm_batch_s *lbm_batch;
int lbm_batch_create(const lbm_lattice_desc *const *lattices, const lbm_params *params, int count,
                     lbm_batch *out);
/* Equilibrium start of every domain from its params' rho, u, v, w. */
int lbm_batch_init(lbm_batch b);
/* Per-node inlet/outlet velocity of one domain (host arrays of its n*m*h
 * nodes; a NULL component keeps the params' constant), as
 * lbm_set_inlet_velocity does for one lattice. */
int lbm_batch_set_inlet_velocity(lbm_batch b, int domain, const float *u, const float *v, const float *w);
/* Equilibrium start of one domain from macroscopic fields (host arrays of
 * n*m*h; NULL = the params' constant), e.g. a predicted steady state.  Call
 * after lbm_batch_init and before the first step. */
int lbm_batch_init_fields(lbm_batch b, int domain, const float *rho, const float *u, const float *v,
                          const float *w);
/* nsteps steps of every active domain (stream NULL = the batch's own). */
int lbm_batch_step(lbm_batch b, int nsteps, int write_macro_last, void *stream);
/* res[d]: sqrt(sum |u - u_prev|^2) / sqrt(sum |u|^2) over fluid nodes of the
 * last stored fields against those at the previous call (FP64; zero fields
 * before the first call).  LBM_DIVERGED when an active domain is not finite. */
int lbm_batch_residuals(lbm_batch b, double *res);
/* Retire (0) or re-activate (1) domains; retired domains keep their state. */
int lbm_batch_set_active(lbm_batch b, const int *active);
/* Step all active domains in chunks of check_every steps, retire each domain
 * whose residual falls below tol, until none is active or max_steps steps
 * ran.  steps[d] and res[d] (may be NULL) receive each domain's step count
 * and last residual. */
int lbm_batch_run_to_tolerance(lbm_batch b, double tol, int check_every, long long max_steps, long long *steps,
                               double *res);
int lbm_batch_get_macro(lbm_batch b, int domain, float *rho, float *u, float *v, float *w);
int lbm_batch_get_populations(lbm_batch b, int domain, double *f);
int lbm_batch_info(lbm_batch b, int *domains, long long *nodes, long long *fluid_nodes, int *active_tiles);
long long lbm_batch_active_fluid_nodes(lbm_batch b);
const char *lbm_batch_last_error(void);
void lbm_batch_destroy(lbm_batch b);

/* ---- Colour-gradient two-phase D2Q9 on a periodic lattice ----------------
 * The reference's multiphase 2D step (Iterate.cu:393-491): colour gradient
 * of (rho_r - rho_b)/rho over the 3x3 stencil or, with high_order, the
 * 24-point stencil (GpuCollision.cu:112-281), one BGK collision with the
 * harmonic-mean viscosity, phase-dependent rest weights, surface-tension
 * perturbation and recolouring (gpuCollBgkwGC2D, gpuCollEnhancedBgkwGC2D,
 * GpuCollision.cu:552-707), streaming of both colours (gpuStreaming2DCG,
 * GpuStream.cu:30-158) and the colour densities (gpuUpdateMacro2DCG,
 * GpuUpdateMacro.cu:43-135).  Both axes wrap periodically. */
typedef struct lbm_cg_handle_s *lbm_cg_handle;

typedef struct lbm_cg_params {
    double r_alpha, b_alpha;         /* rest-weight parameters of each colour */
    double r_viscosity, b_viscosity; /* kinematic viscosities */
    double beta;                     /* recolouring strength */
    double A;                        /* surface-tension perturbation amplitude */
    double g_limit;                  /* |colour gradient| above which a node is interface */
    double control_param;            /* |phi| threshold of the Laplace-law sums */
    int high_order;                  /* 1: 24-point gradient stencil */
    int enhanced;                    /* 1: enhanced equilibrium (GpuCollision.cu:630-707) */
    int storage;                     /* LBM_STORE_F32; LBM_STORE_F16S: per direction the
                                        summed population r+b as the FP16 of
                                        (r + b - w_d) * 1024 and the colour
                                        difference r - b as FP16, FP32
                                        arithmetic; LBM_STORE_F64: FP64 storage
                                        and arithmetic (the reference run for
                                        storage-precision checks) */
} lbm_cg_params;

/* n x m periodic lattice, n, m >= 5. */
int lbm_cg_create(int n, int m, const lbm_cg_params *params, lbm_cg_handle *out);
/* D3Q19: n x m x h lattice periodic in all three axes, n, m, h >= 5 (the
 * reference's 3D path, gpuCollBgkwGC3D / gpuCollEnhancedBgkwGC3D,
 * GpuCollision.cu:283-526, :709-880, with the 18-neighbour gradient or, when
 * high_order, the 104-point isotropic set).  The calls below take Q = 19
 * populations per node and SoA index d*N + x + n*(y + m*z). */
int lbm_cg_create3d(int n, int m, int h, const lbm_cg_params *params, lbm_cg_handle *out);
/* Post-streaming red and blue populations, host arrays of Q*N floats (Q = 9
 * in 2D) in SoA order f[d*N + x + n*y]; performs the first collision. */
int lbm_cg_init(lbm_cg_handle h, const float *r_f, const float *b_f);
/* nsteps of stream + densities + collide on `stream` (NULL = own stream);
 * write_macro_last stores rho, u, v on the last step. */
int lbm_cg_step(lbm_cg_handle h, int nsteps, int write_macro_last, void *stream);
/* Colour densities of the last step and the velocity of the last step that
 * stored it, host arrays of n*m (any may be NULL). */
int lbm_cg_get_macro(lbm_cg_handle h, float *r_rho, float *b_rho, float *u, float *v);
/* As lbm_cg_get_macro, with the z velocity (0 in 2D). */
int lbm_cg_get_macro3d(lbm_cg_handle h, float *r_rho, float *b_rho, float *u, float *v, float *w);
/* Post-collision red and blue populations, Q*N floats each. */
int lbm_cg_get_populations(lbm_cg_handle h, float *r_f, float *b_f);
/* FP64 Laplace-law sums (Iterate.cu:496-499): out[0] = sum rho_r where
 * phi >= control_param, out[1] = their count, out[2] = sum rho_b where
 * phi <= -control_param, out[3] = their count, out[4] = max |u| (3D:
 * gpuUpdateMacro3DCG's p_in / p_out sums, GpuUpdateMacro.cu:345-356).
 * Returns LBM_DIVERGED when a sum is not finite. */
int lbm_cg_laplace(lbm_cg_handle h, double *out);
long long lbm_cg_nodes(lbm_cg_handle h);
/* Populations per node: 9 or 19. */
int lbm_cg_q(lbm_cg_handle h);
const char *lbm_cg_last_error(void);
void lbm_cg_destroy(lbm_cg_handle h);

/* Library version, for load checks. */
int lbm_version(void);

#endif /* __CUDACC_RTC__ */

#ifdef __cplusplus
}
#endif

#endif /* THESIS_LBM_H */
