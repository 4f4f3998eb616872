/*
 * thesis_lbm_io.h -- the reference solver's file formats, host side.
 *
 * The drop-in keeps lbm-solver_final's inputs and outputs: the 23-line init
 * file, the Node and BC lattice files, the FinalData/InitialData result files
 * in CSV, Tecplot (.dat) and ParaView image data (.vti), and its result
 * comparison.  These functions restate the reference's readers and writers
 * (Source code/lbm-solver_final/FilesReading.cu, FilesWriting.cu, Check.cu)
 * so a driver written against include/thesis_lbm.h reads and writes the same
 * files.  Host only; no GPU needed.  Conventions as in thesis_lbm.h: caller
 * allocates, status codes returned.
 */
#ifndef THESIS_LBM_IO_H
#define THESIS_LBM_IO_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Output formats (OutputFormat, include/Arguments.h: CSV=1, TECPLOT, PARAVIEW). */
#define LBM_OUT_CSV 1
#define LBM_OUT_DAT 2
#define LBM_OUT_VTI 3

/* Residual models (ResidualsModel: L2=1, FdRelDiff, MacroDiff). */
#define LBM_RES_L2 1
#define LBM_RES_FD_REL_DIFF 2
#define LBM_RES_MACRO_DIFF 3

/* InletProfile values the init file can select: INLET_PROF -> 1, INLET_CTE
 * -> 2, INLET_PUL -> 3 (FilesReading.cu:125-137). */

/* The Arguments fields readInitFile sets (FilesReading.cu:60-222). */
typedef struct lbm_run_config {
    char problem_name[512];            /* line 1, quoted: Mesh/<name>_Node.dat, _BC.dat */
    double u, v, w, rho, viscosity;    /* lines 2-6 */
    int inlet_profile;                 /* line 7: INLET_PROF 1, INLET_CTE 2, INLET_PUL 3 */
    int collision_model;               /* line 8: SRT 1, TRT 2, MRT 3 */
    int boundary_type;                 /* line 9: CURVED 1, STRAIGHT 2 */
    int bc_wall_model;                 /* line 10: BBack 1, HHmodel 2 */
    int outlet_profile;                /* line 11: Vout 1, 1stE 2, 2ndE 3, HEmodel 4 */
    int iterations;                    /* line 12 */
    int autosave_after, autosave_every;/* lines 13-14 */
    double stop_condition[4];          /* line 15: u v w rho */
    int output_format;                 /* line 16: CSV 1, DAT 2, VTI 3 */
    int use_initial_conditions_file;   /* line 17: yes / no */
    char initial_conditions_name[512]; /* line 18, quoted */
    int residual_model;                /* line 19: L2 1, MaxRelativeFdDiff 2, MaxMacroDiff 3 */
    int show_macro_diff;               /* line 20: residual check interval */
    double g;                          /* line 21: body force */
    int boundary_id;                   /* line 22: drag/lift boundary id */
    int update_inlet_outlet;           /* line 23: yes / no */
    int unparsed_lines;                /* lines the reference would report as
                                          "Error reading initial file" */
} lbm_run_config;

/* Parse the init file.  Returns LBM_ERR_FILE (2) when it cannot be opened.
 * A line that does not parse leaves its field at zero and counts in
 * unparsed_lines, where the reference prints an error and continues. */
int lbm_read_init_file(const char *path, lbm_run_config *cfg);

/* Number of lines as the reference counts them: every '\n' and every '\r'
 * (getNumberOfLines, FilesReading.cu:17-46).  -1 when unreadable. */
long long lbm_count_lines(const char *path);

/* 3 when the first line of a Node file has the 7 tab-separated 3D columns,
 * else 2 (main.cu:107-139).  -1 when unreadable. */
int lbm_node_file_dims(const char *path);

/* Read `count` records of a Node file (readNodeFile, FilesReading.cu:270-305):
 * 2D "i j x y type", 3D "i j k x y z type".  k and z are zero in 2D.
 * Coordinates are read as FP32, as the reference's default build does. */
int lbm_read_node_file(const char *path, int dims, long long count, int *i, int *j, int *k, float *x, float *y,
                       float *z, int *type);

/* Read `count` records of a BC file (readConnFile, FilesReading.cu:307-347):
 * 2D "i j dir type x y id", 3D "i j k dir type x y z id". */
int lbm_read_bc_file(const char *path, int dims, long long count, int *i, int *j, int *k, int *dir, int *type,
                     float *bx, float *by, float *bz, int *id);

/* Write a result file (WriteResults3D, FilesWriting.cu:146-258; the 2D loop
 * writes the same file with z = w = 0): CSV "x,y,z,u,v,w,vel_mag,rho,press",
 * Tecplot point data, or ParaView image data with Velocity, Density and
 * Pressure arrays.  Arrays hold n*m*h nodes, x fastest. */
int lbm_write_results(const char *path, int format, int n, int m, int h, const float *x, const float *y,
                      const float *z, const float *u, const float *v, const float *w, const float *rho);

/* Read the nine columns of a result file (readResultFile, FilesReading.cu:
 * 348-467) into cols[c*count + row]; a .vti file fills u, v, w (3-5) and rho
 * (7) only.  Returns the number of rows read or a negative status. */
long long lbm_read_results(const char *path, long long count, double *cols);

/* Initial conditions for a restart (readInitConditionsFile, FilesReading.cu:
 * 224-268): checks that the file's line count matches `nodes` for its
 * format, then returns u, v, w, rho.  LBM_ERR_FILE when it does not. */
int lbm_read_initial_conditions(const char *path, long long nodes, int n, int m, int h, float *u, float *v,
                                float *w, float *rho);

/* Compare two result files column by column (compareFiles, Check.cu):
 * diff_sum[c] = sum |a - b| and diff_max[c] = max |a - b| (FP64 here) for the
 * nine columns x, y, z, u, v, w, vel_mag, rho, pressure.  Returns 0 when every
 * diff_sum is at most 0.001, 1 when one is larger, LBM_ERR_FILE (2) when the
 * line counts differ or a file is unreadable. */
int lbm_compare_results(const char *f1, const char *f2, double *diff_sum, double *diff_max);

/* Cavity centre lines (WriteLidDrivenCavityMidLines3D, FilesWriting.cu:
 * 260-302): 3D — for the nodes at y = m/2, u/Ulid and z along the line
 * x = n/2, and x and w/Ulid along the line z = h/2, one row per pair,
 * "%.8f\t%.8f\t%.8f\t%.8f"; 2D (the same layout for the 2D cavity) — u/Ulid
 * and y along x = n/2, x and v/Ulid along y = m/2.  Header lines
 * "CASE: Ulid = %f Nx = %d" and the column names. */
int lbm_write_midlines(const char *path, int dims, int n, int m, int h, const float *x, const float *y,
                       const float *z, const float *u, const float *v, const float *w, double ulid);

/* Channel cross-section (WriteChannelCrossSection3D, FilesWriting.cu:304-336):
 * every node of the plane x = (3/4) n, "x y z u v w". */
int lbm_write_cross_section(const char *path, int n, int m, int h, const float *x, const float *y,
                            const float *z, const float *u, const float *v, const float *w, double uin);

/* Message of the last failing call on this thread. */
const char *lbm_io_last_error(void);

/* ---- Lattice emitters (no counterpart in the reference) ------------------
 * Geometries the reference generator cannot mesh (it meshes axis-aligned
 * quadrilateral faces only, G/Intersect.cpp:98-110), written as Node and BC
 * files in the reference's formats (3D lines as G/main.cpp:56-66 and
 * G/FluidTracking.cpp:229-236 write them; 2D as readNodeFile/readConnFile
 * read them, S/FilesReading.cu:270-347), coordinates index/(n-1).  Random
 * geometry comes from SplitMix64(seed), uniform doubles from its top 53
 * bits.  Return LBM_OK, LBM_ERR_INVALID or LBM_ERR_FILE (message in
 * lbm_emit_last_error). */

/* Random sequential packing of non-overlapping spheres in an n x m x h box:
 * per attempt r = U(rmin, rmax), centre U(0,1) x (n-1, m-1, h-1), then the
 * margin axis' coordinate again, U within [margin + r, ext - margin - r];
 * a sphere that overlaps none is kept and its nodes (distance^2 <= r^2) turn
 * solid, until the solid fraction reaches 1 - porosity or max_attempts.
 * solid: n*m*h bytes, x fastest; spheres (may be NULL): up to max_spheres
 * (x, y, z, r) rows; num_spheres: the count kept. */
int lbm_pack_spheres(int n, int m, int h, double porosity, double rmin, double rmax, unsigned long long seed,
                     int margin_axis, double margin, long long max_attempts, unsigned char *solid,
                     double *spheres, long long max_spheres, long long *num_spheres);
/* Duct along z packed with spheres (margin axis z, margin 2): Zou-He
 * pressure faces z = 0 (inlet, BC type 2) and z = h-1 (outlet, type 3); the
 * side faces and the spheres carry no BC lines (walls in physics mode). */
int lbm_emit_sphere_duct(int n, int m, int h, double porosity, double rmin, double rmax, unsigned long long seed,
                         const char *node_path, const char *bc_path, long long *num_spheres);
/* 2D channel along x with n_obstacles (-1: 1 to 6 drawn) non-overlapping
 * circles (radius 8-32) and rectangles (sides 10-60), times size_scale,
 * clear of the inlet and outlet: inlet x = 0 (type 2), outlet x = n-1
 * (type 3), walls y = 0 and y = m-1 (type 1). */
int lbm_emit_channel2d(int n, int m, unsigned long long seed, int n_obstacles, double size_scale,
                       const char *node_path, const char *bc_path);
/* Lid-driven cavity, every node fluid: walls on all faces, the lid (y = m-1
 * in 2D, z = h-1 in 3D) an inlet. */
int lbm_emit_cavity(int dims, int n, int m, int h, const char *node_path, const char *bc_path);
const char *lbm_emit_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* THESIS_LBM_IO_H */
