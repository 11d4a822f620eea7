/*
 * lsmpqs_gpu.h -- C-ABI of the GB300 implementation of the lsmpqs
 * quasi-static level-set path (libqssgpu.so).
 *
 * Every function below keeps the name, signature, argument meaning, return
 * convention and side effects of the reference routine it replaces (cited as
 * file:line inside the lsmpqs-1.0 source tree), so a C caller of the
 * reference links against libqssgpu.so unchanged.  QSSLIB_REAL is double.
 * Arrays are host memory owned by the caller, laid out over the ghost box,
 * column-major (i fastest).  Inside, the arrays live in HBM between calls of
 * one top-level entry point; on return the caller's arrays hold exactly what
 * the reference would have left in them.
 *
 * Errors never abort the process: an entry point that fails returns the
 * reference's failure value where it has one (-1 from constCurvModel3d, 1 from
 * drainTop) and records a code and message for qssgpu_last_error().
 */
#ifndef LSMPQS_GPU_H
#define LSMPQS_GPU_H

#include <stdio.h>

#include "lsmpqs_types.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------- model drivers (the hot path) ---------------------------- */

/* src/level_set_evolution/drain_top.h:28 -- reads data/grid/mask files, runs
   drain_model3d, writes data_final; returns 0, or 1 on bad input / GPU error */
int drainTop(Options *options, char *fname_data_in, char *fname_grid_in, char *fname_mask_in);
/* src/level_set_evolution/imbibe_top.h (imbibeTop) */
int imbibeTop(Options *options, char *fname_data_in, char *fname_grid_in, char *fname_mask_in);

/* src/level_set_evolution/drain_model3d.h:31 -- increasing-curvature ladder;
   writes data_step_<n>(.gz) after every curvature step */
void drain_model3d(Options *options, QSS_DataArrays *p, Grid *g, FILE *fp_out);
/* src/level_set_evolution/imbibe_model3d.h -- decreasing-curvature ladder */
void imbibe_model3d(Options *options, QSS_DataArrays *p, Grid *g, FILE *fp_out);

/* src/level_set_evolution/constCurvModel3d.h:29 -- variable-coefficient model
   (contact angle > 0); returns the pseudo time reached, or -1 when the
   non-wetting saturation exceeds vol_frac_max or the phase vanishes */
QSSLIB_REAL constCurvModel3d(Options *options, QSS_DataArrays *p, Grid *g, FILE *fp_out);
/* src/level_set_evolution/constCurvModel3d.h:30 -- zero contact angle, scalar a */
QSSLIB_REAL constCurvModel3dNoVar(Options *options, QSS_DataArrays *p, Grid *g, FILE *fp_out,
                                  QSSLIB_REAL a);

/* src/connectivity/connectivity.h:27 -- trapped non-wetting / wetting masks */
void trapComponents_mask(QSS_DataArrays *p, Grid *g, Options *options);
/* src/connectivity/connectivity.h:23 -- 26-connected labels of phi_bin into
   connectivity: each component carries its largest linear index, 0 = background */
void findConnectivity3d(QSS_DataArrays *p, Grid *g);
/* src/connectivity/connectivity.h -- inlet/outlet reference points (host only) */
void getMainInd_new(Options *options, QSS_DataArrays *p, Grid *g);
/* src/reinitialization/reinitialize_top.h:28 -- Russo-Smereka subcell-fix
   reinitialisation of a host array, tmax_r / (0.5 dx) pseudo-time iterations */
void reinitializeSubcellFix3d(QSSLIB_REAL *data, Grid *g, Options *options);

/* src/utilities/qss_general_util.h (qss_general_util.c:82-143) -- stores one of
   this library's getrhs3d* routines in options->space_deriv_func */
void setSpaceDerivFunc(Grid *g, Options *options);
/* qss_general_util.c:150-207 -- overlap from the contact angle */
void setThetaOverlap(QSS_DataArrays *p, Grid *g, Options *options);
/* qss_general_util.c:422-706 -- signed linear extrapolation into the ghost
   layers; idx 0..5 one face, 6/7/8 an axis, 9 all faces in x, y, z order */
void signedLinearExtrapolationBCqss(QSSLIB_REAL *phi, Grid *g, int bdry_location_idx);
/* qss_general_util.c:711-728 */
void initializeDisconnectedMasks(QSSLIB_REAL *data, Grid *g);
/* qss_general_util.c:813-833 -- fills p->phi_extra */
void createReservoirInlet3d(QSS_DataArrays *p, Grid *g);

/* ---------------- kernel-level entry points (Fortran convention) ---------- */
/* The reference's Fortran kernels, same symbol names and argument lists
   (src/spatial_derivatives/qss_spatial_derivatives3d.h:22-32,
   src/time_integration/qss_tvd_runge_kutta3d.h:27-29,
   src/reinitialization/qss_reinitialization3d.h:42-45,
   src/utilities/qss_util3d.h:20-29).  Each call copies its host arrays to the
   GPU, runs one kernel over the given fill box and copies the outputs back. */
#define LSMPQS_GB6 const int *, const int *, const int *, const int *, const int *, const int *
void getrhs3d2ndconst_(const double *phi, const double *vel_n, const double *b, double *max_H_over_dX,
                       double *lse_rhs, LSMPQS_GB6, LSMPQS_GB6, const double *dx, const double *dy,
                       const double *dz);
void getrhs3d3rdconst_(const double *phi, const double *vel_n, const double *b, double *max_H_over_dX,
                       double *lse_rhs, LSMPQS_GB6, LSMPQS_GB6, const double *dx, const double *dy,
                       const double *dz);
void getrhs3d2nd_(const double *phi, const double *vel_n, const double *b, const double *vel_x,
                  const double *vel_y, const double *vel_z, double *max_H_over_dX, double *lse_rhs,
                  LSMPQS_GB6, LSMPQS_GB6, const double *dx, const double *dy, const double *dz);
void getrhs3d3rd_(const double *phi, const double *vel_n, const double *b, const double *vel_x,
                  const double *vel_y, const double *vel_z, double *max_H_over_dX, double *lse_rhs,
                  LSMPQS_GB6, LSMPQS_GB6, const double *dx, const double *dy, const double *dz);
void getrhs3d5th_(const double *phi, const double *vel_n, const double *b, const double *vel_x,
                  const double *vel_y, const double *vel_z, double *max_H_over_dX, double *lse_rhs,
                  LSMPQS_GB6, LSMPQS_GB6, const double *dx, const double *dy, const double *dz);
void getcentralgrad3dorder2_(double *phi_x, double *phi_y, double *phi_z, LSMPQS_GB6, const double *phi,
                             LSMPQS_GB6, LSMPQS_GB6, const double *dx, const double *dy, const double *dz);
void signedlinearextrapolation3d_(double *phi, LSMPQS_GB6, LSMPQS_GB6, const int *bdry_location_idx);
void setvarnorm3d_(const double *mask, const double *mask_x, const double *mask_y, const double *mask_z,
                   double *var_a, const double *a0, const double *ca, LSMPQS_GB6, LSMPQS_GB6,
                   const double *dx);
void setvarnorm3dtheta_(const double *mask, const double *mask_x, const double *mask_y,
                        const double *mask_z, double *var_a, const double *a0, const double *ca,
                        LSMPQS_GB6, LSMPQS_GB6, const double *dx);
void setvarcurvadv3d_(const double *mask, const double *mask_x, const double *mask_y,
                      const double *mask_z, double *var_b, double *vel_x, double *vel_y, double *vel_z,
                      double *b_max_over_dx, double *max_U_over_dx, const double *const_b, LSMPQS_GB6,
                      LSMPQS_GB6, const double *dx);
void qss3drk1step_(double *u_next, LSMPQS_GB6, const double *u_cur, LSMPQS_GB6, const double *rhs,
                   LSMPQS_GB6, LSMPQS_GB6, const double *dt);
void qss3dtvdrk2stage2_(double *u_stage2, LSMPQS_GB6, const double *u_stage1, LSMPQS_GB6,
                        const double *u_cur, LSMPQS_GB6, const double *rhs, LSMPQS_GB6, LSMPQS_GB6,
                        const double *dt);
void qss3dtvdrk3stage3_(double *u_next, LSMPQS_GB6, const double *u_stage2, LSMPQS_GB6,
                        const double *u_cur, LSMPQS_GB6, const double *rhs, LSMPQS_GB6, LSMPQS_GB6,
                        const double *dt);
void qss3dcomputedistanceforsubcellfix_(double *distance0, const double *phi0, LSMPQS_GB6, LSMPQS_GB6,
                                        const double *dx, const double *dy, const double *dz);
void qss3dcomputereinitializationeqnrhssubcellfixorder1_(double *reinit_rhs, const double *phi,
                                                         LSMPQS_GB6, const double *phi0,
                                                         const double *distance0, LSMPQS_GB6,
                                                         const double *dx, const double *dy,
                                                         const double *dz);
void qss3dmaxnormdifflocal_(double *max_norm_diff, const double *field1, LSMPQS_GB6,
                            const double *field2, LSMPQS_GB6, LSMPQS_GB6, const double *local_zone);
void imposemaskparallel_(double *phi_masked, const double *mask, const double *phi,
                         const double *overlap, LSMPQS_GB6, const int *cur_klo_gb,
                         const int *cur_khi_gb);
void qss3dvolumeregionphilessthanzero_(double *volume, const double *phi, LSMPQS_GB6, LSMPQS_GB6,
                                       const double *dx, const double *dy, const double *dz,
                                       const double *epsilon);
void imposetrapvelocity3d_(const double *phi_w, const double *phi_nw, double *normal_velocity,
                           double *curvature_coeff, double *vel_x, double *vel_y, double *vel_z,
                           LSMPQS_GB6, LSMPQS_GB6, const double *dx);
#undef LSMPQS_GB6

/* ---------------- data model, options, files (host) ------------------------ */
/* src/utilities/qss_data_arrays.h:84-182 */
QSS_DataArrays *allocateQSSDataArrays(void);
void allocateMemoryForQSSDataArrays(QSS_DataArrays *p, Grid *grid);
void destroyQSSDataArrays(QSS_DataArrays *p); /* also frees the device copy */
void writeDataArrayQSS(QSSLIB_REAL *data, Grid *grid, char *file_name, int zip_status);
void writeDataArrayRaw(QSSLIB_REAL *data, Grid *grid, char *file_name, int zip_status);
void writeDataArrayUchar(unsigned char *data, Grid *grid, char *file_name, int zip_status);
void writeDataArrayInt(int *data, Grid *grid, char *file_name, int zip_status);
void writeDataArrayUcharFB(unsigned char *data, Grid *grid, char *file_name, int zip_status);
QSSLIB_REAL *readDataArrayQSS(int *grid_dims_ghostbox, char *file_name);
int *readDataArrayInt(int *grid_dims_ghostbox, char *file_name);
/* src/geometry/qss_grid.h:103-340 */
Grid *allocateGrid(void);
Grid *createGridSetDx(int num_dims, QSSLIB_REAL dx, QSSLIB_REAL *x_lo, QSSLIB_REAL *x_hi,
                      QSSLIB_SPATIAL_DERIVATIVE_ACCURACY_TYPE accuracy);
Grid *createGridSetDxDyDz(int num_dims, QSSLIB_REAL dx, QSSLIB_REAL dy, QSSLIB_REAL dz,
                          QSSLIB_REAL *x_lo, QSSLIB_REAL *x_hi,
                          QSSLIB_SPATIAL_DERIVATIVE_ACCURACY_TYPE accuracy);
Grid *createGridSetGridDims(int num_dims, int *grid_dims, QSSLIB_REAL *x_lo, QSSLIB_REAL *x_hi,
                            QSSLIB_SPATIAL_DERIVATIVE_ACCURACY_TYPE accuracy);
Grid *copyGrid(Grid *grid);
void destroyGrid(Grid *grid);
void printGrid(Grid *grid, FILE *fp);
void writeGridToAsciiFile(Grid *grid, char *file_name, int zip_status);
void writeGridToBinaryFile(Grid *grid, char *file_name, int zip_status);
Grid *readGridFromBinaryFile(char *file_name);
/* src/utilities/qss_options.h:170-283 */
Options *allocateOptions(void);
Options *createOptionsDefault(void);
Options *createOptionsFromInputFile(char *filename);
void printOptions(Options *options, FILE *fp);
void destroyOptions(Options *options);
/* src/utilities/qss_file.h:30-58 */
void checkUnzipFile(char *file_name, int *pzip_status, char **pfile_base);
void zipFile(char *file_base, int zip_status);
/* src/geometry/qss_initialization3d.h (signed distances, evaluated on the GPU) */
void createIntersectionOfSpheres(QSSLIB_REAL *phi, int num_spheres, QSSLIB_REAL *center_x,
                                 QSSLIB_REAL *center_y, QSSLIB_REAL *center_z, QSSLIB_REAL *radius,
                                 int *inside_flag, Grid *grid);
void createSphere(QSSLIB_REAL *phi, QSSLIB_REAL center_x, QSSLIB_REAL center_y, QSSLIB_REAL center_z,
                  QSSLIB_REAL radius, int inside_flag, Grid *grid);
void createIntersectionOfHalfSpaces3d(QSSLIB_REAL *phi, int num_half_spaces, QSSLIB_REAL *normal_x,
                                      QSSLIB_REAL *normal_y, QSSLIB_REAL *normal_z,
                                      QSSLIB_REAL *point_x, QSSLIB_REAL *point_y,
                                      QSSLIB_REAL *point_z, Grid *grid);
void createPlane(QSSLIB_REAL *phi, QSSLIB_REAL normal_x, QSSLIB_REAL normal_y, QSSLIB_REAL normal_z,
                 QSSLIB_REAL point_x, QSSLIB_REAL point_y, QSSLIB_REAL point_z, Grid *grid);
void createPolyhedron3d(QSSLIB_REAL *phi, int num_planes, QSSLIB_REAL *normal_x,
                        QSSLIB_REAL *normal_y, QSSLIB_REAL *normal_z, QSSLIB_REAL *point_x,
                        QSSLIB_REAL *point_y, QSSLIB_REAL *point_z, Grid *grid);
void createIntersectionOfBoxes(QSSLIB_REAL *phi, int num_cuboids, QSSLIB_REAL *corner_x,
                               QSSLIB_REAL *corner_y, QSSLIB_REAL *corner_z,
                               QSSLIB_REAL *side_length_x, QSSLIB_REAL *side_length_y,
                               QSSLIB_REAL *side_length_z, int *inside_flag, Grid *grid);
void createBox(QSSLIB_REAL *phi, QSSLIB_REAL corner_x, QSSLIB_REAL corner_y, QSSLIB_REAL corner_z,
               QSSLIB_REAL side_length_x, QSSLIB_REAL side_length_y, QSSLIB_REAL side_length_z,
               int inside_flag, Grid *grid);
/* src/geometry/qss_initialization2d.h:235-241, 277-284 (2-D circles, evaluated on the
   host: the 2-D path is not on the GPU; createInitFromMask's 2-D branch calls
   them) */
void createIntersectionOfCircles(QSSLIB_REAL *phi, int num_circles, QSSLIB_REAL *center_x,
                                 QSSLIB_REAL *center_y, QSSLIB_REAL *radius, int *inside_flag,
                                 Grid *grid);
void createCircle(QSSLIB_REAL *phi, QSSLIB_REAL center_x, QSSLIB_REAL center_y, QSSLIB_REAL radius,
                  int inside_flag, Grid *grid);

/* ---------------- GB300 extensions (no counterpart in the reference) ------- */
/* error state: 0 = no error since the last clear */
int qssgpu_last_error(void);
const char *qssgpu_error_string(void);
void qssgpu_clear_error(void);
/* 1 if a CUDA device is usable by the library */
int qssgpu_device_available(void);
/* Number of z-slabs whose last voxels set the CFL step, i.e. the OpenMP thread
   count of the reference run to reproduce (default 1, or $QSSGPU_SLABS);
   0 restores the default */
void qssgpu_set_slabs(int nslabs);
/* WENO5 variable-coefficient stages: 0 one fused kernel per stage, 1 (the
   default) one kernel per axis + a combine kernel; also $QSSGPU_WENO_MODE;
   -1 restores the default; results are identical.  Returns the previous
   mode. */
int qssgpu_set_weno_split(int mode);
/* Share of the split WENO5 stage's FP64 arithmetic computed bit-exactly on
   the integer pipes: 0 none, 1 divisions, power-of-two scalings and
   comparisons, 2 (default, also $QSSGPU_EMU) level 1 plus part of the
   products and sums; -1 restores the default.  Results are identical at
   every level.  Returns the previous level. */
int qssgpu_set_emu_level(int level);
/* form of the WENO5 axis passes at levels >= 1: -1 (default) and 3 tiles
   of 16 lines x 16 voxels, one voxel per thread, every face and centre of a
   tile computed once into shared memory; 4 tiles of 8 lines x 27 voxels; 0
   sliding window in registers; 1 the window's scaled copies in shared
   memory and the smoothness squares on the integer pipes; 2 tuned: the
   first pass over each line shape times every distinct (form, segment
   length), the tile form included, and the fastest is kept for that shape
   (one stream synchronisation per new shape and axis); identical results;
   returns the previous setting.  No
   reference counterpart: the reference's getrhs3d5th_ (3d.f:1962-2246) is a
   loop over voxels with nothing to tune. */
int qssgpu_set_axis_variant(int variant);
/* the launch shapes chosen in tuned mode so far: at most max_rows rows of 7
   ints (arithmetic level, axis, lanes, lines per lane, line length, form,
   segment length) into rows (may be NULL); returns the number of shapes */
int qssgpu_axis_tuning(int* rows, int max_rows);
/* forgets the tuned launch shapes */
void qssgpu_axis_tuning_reset(void);
/* writes the tuned launch shapes to a text file, one shape a line (the 7
   numbers of qssgpu_axis_tuning); returns the number written, -1 on error */
int qssgpu_axis_tuning_save(const char *path);
/* adds the shapes of such a file to the table (a shape already there keeps
   its pick), so later processes in tuned mode (axis variant 2) skip the
   timing of those shapes; every line is checked first
   (level 1-2, axis 0-2, positive sizes, form 0 or 1 with 1 <= segment length
   <= line length, form 3 with segment length 16, form 4 with segment length
   27) and a file with any other line adds nothing; returns the number of
   shapes read, -1 on error */
int qssgpu_axis_tuning_load(const char *path);
/* Batched mode (no reference counterpart): the curvature ladder of
   drain_model3d (drain != 0) or imbibe_model3d on n independent volumes at
   once, each with its own Options (contact angle, curvature ladder), arrays
   and grid, on its own CUDA stream driven by one of `workers` host threads
   (0: one per volume; at most 64).  Every volume ends exactly as a single
   drain_model3d / imbibe_model3d call on it would leave it.  fp may be NULL
   or hold n FILE* (each may be NULL).  The per-step files of volume v are
   named prefix[v] + "data_step_<k>" ("" gives the reference's names); a
   NULL prefix array or entry writes no per-step files.  Volumes must not
   share arrays or options.  Returns 0, or the number of volumes that
   failed; qssgpu_last_error / qssgpu_error_string then describe the first. */
int qssgpu_ladder_batch(int drain, int n, Options *const *o, QSS_DataArrays *const *p, Grid *const *g,
                        FILE *const *fp, const char *const *prefix, int workers);
/* ---- pre- and post-processing on the GPU ---- */
/* qss_general_util.h: reinitialisation of p->mask (tmax_r / (0.5 dx)
   subcell-fix iterations); like the reference it leaves distance0 in
   scratch1, the initial mask in scratch2, the last RHS in lse_rhs (fill box)
   and the last iterate in phi_next */
void qss_reinitialize_mask(QSS_DataArrays *p, Grid *g, Options *o);
/* createMaskUBC (src/applications/createMaskUBC.c:76-112) as a library call:
   p->mask = +dx where the 8-bit fill-box image (x fastest) is 255 (grain),
   -dx elsewhere, zero on the ghost layers, then qss_reinitialize_mask;
   dx = o->dx as in the reference */
int qssgpu_create_mask_ubc(const unsigned char *ubc, QSS_DataArrays *p, Grid *g, Options *o);
/* createInitFromMask (createInitFromMask.c:55-85, 3-D): p->phi = max(p->mask,
   the inlet sphere of the reference: radius 0.7 (x_hi - x_lo) centred 0.7
   radius before x_lo, or radius 90 dx at the centre with o->center_inlet) */
int qssgpu_create_init_from_mask(QSS_DataArrays *p, Grid *g, Options *o);
/* makeDiffSteps (makeDiffSteps.c:54-132, 3-D): diff = max(-step_a, step_b -
   dx/2) (the lens between two saved steps), 26-connected labels of {diff < 0}
   with inlet and outlet slabs, *percolates = inlet and outlet connected;
   when it percolates and connected != NULL, connected = diff with the
   non-wetting voxels outside the percolating component flipped.  Ghost-box
   arrays. */
int qssgpu_diff_steps(const double *step_a, const double *step_b, Grid *g, double *diff, double *connected,
                      int *percolates);
/* makeRaw's phase images (src/applications/makeRaw.c:52-135): 1 where the
   selected level set is negative, else 0 (IMPOSE_UCHAR), for phase 'm' the
   mask, 'n' phi (non-wetting), 'w' max(mask, -phi) (wetting); bin_full gets
   the ghost-box image, bin_fb the fill box packed i fastest (copyDataFB);
   either may be NULL, phi / mask only where the phase reads them.  The
   reference writes its `_fb` images of phases n and w with the ghost-box
   byte count from a fill-box buffer (an over-read); here the fill-box image
   has exactly the fill-box bytes. */
int qssgpu_phase_uchar(const double *phi, const double *mask, Grid *g, char phase, unsigned char *bin_full,
                       unsigned char *bin_fb);
/* Adjoint mode (no reference counterpart).  Forward model: nsteps TVD-RK3
   steps of the variable-coefficient WENO5 update of constCurvModel3d with a
   fixed time step dt (no connectivity, reinitialisation or CFL), starting from
   p->phi, with the normal speed of setVarNorm3dTheta for the per-voxel contact
   angle theta[] (radians, ghost-box array; a0 = o->a, curvature coefficient
   o->b, imposition of p->mask - o->overlap); loss = sum over the fill box of
   (H_eps(phi_T) - target)^2, eps = 1.5 dx, H the reference's smoothed
   Heaviside, target a ghost-box array.  qssgpu_adjoint_theta returns the loss
   and d loss / d theta (ghost-box array, zero on the ghost layers) by a
   hand-written reverse pass that recomputes the states from checkpoints every
   ckpt steps (ckpt <= 0: one segment); qssgpu_forward_theta only the loss
   (and phi_T into phi_out, a ghost-box array, when phi_out is not NULL).
   Host arrays are read, not modified.  0 on success. */
int qssgpu_adjoint_theta(Options *o, QSS_DataArrays *p, Grid *g, const double *theta, const double *target,
                         int nsteps, double dt, int ckpt, double *loss, double *grad_theta);
int qssgpu_forward_theta(Options *o, QSS_DataArrays *p, Grid *g, const double *theta, const double *target,
                         int nsteps, double dt, double *loss, double *phi_out);
/* The sequentially rounded sum values[0] + values[1] + ... + values[n-1]
   (a plain C loop's result, bit for bit) computed on the GPU: in parallel
   by binade-wise integer sums for non-negative runs, element by element
   elsewhere; the volume integrals use the same code.  0 on success. */
int qssgpu_loop_sum(const double *values, long long n, double *out);
int qssgpu_get_slabs(const Grid *g);
/* frees the device copy kept for p (destroyQSSDataArrays calls it) */
void qssgpu_release(QSS_DataArrays *p);
/* page-locked, zeroed host memory for the arrays of a QSS_DataArrays (the
   copies to and from the device then skip the driver's staging); NULL on
   failure; release with qssgpu_host_free */
void *qssgpu_host_alloc(size_t bytes);
void qssgpu_host_free(void *h);
/* inner steps and outer iterations of the last top-level call on p */
void qssgpu_call_stats(const QSS_DataArrays *p, const Grid *g, long long *inner_steps,
                       long long *outer_iters);
/* host wall time (s) of the last top-level call on p by phase: out[0] total,
   out[1] set-up (device arrays), out[2] uploads, out[3] inner steps,
   out[4] trapping, out[5] reinitialisation, out[6] volume and max-norm
   reductions, out[7] downloads (out holds 8 doubles); device work is
   charged to the phase that waits for it, unless $QSSGPU_PHASE_SYNC=1 ends
   every phase with a stream synchronisation */
void qssgpu_call_times(const QSS_DataArrays *p, const Grid *g, double *out);
/* device time of the last top-level call on p by phase, from CUDA events
   recorded on the volume's stream where each phase begins and ends: out[1..7]
   as in qssgpu_call_times, out[0] their sum (out holds 8 doubles); waits for
   the recorded events */
void qssgpu_call_device_times(const QSS_DataArrays *p, const Grid *g, double *out);

/* Allocation-free smoothed volume of {phi < 0} (no counterpart in the
   reference; same result, bit for bit, as qss3dvolumeregionphilessthanzero_).
   For callers that must not allocate device memory while they run and that
   already hold their data on the GPU: a framework that reserved all of HBM
   up front for its own pool allocator (cudaMalloc then fails, or takes memory
   the framework has planned for something else), or one that keeps several
   streams busy and cannot afford the device-wide synchronisation that
   cudaFree implies.  d_phi (the ghost box gb = {0, nx-1, 0, ny-1, 0, nz-1})
   and d_volume (one double) are DEVICE pointers of the caller; ib is the
   summed box; work is queued on `stream` (a cudaStream_t, NULL = default
   stream) and the result is in *d_volume when the stream reaches it.  The
   per-voxel contributions live in one fixed device array of 2^21 doubles
   (16 MiB) that every GPU loading the library holds until the process exits:
   boxes of more than 2^21 voxels (128^3) are rejected with QSSGPU_ERR_ARG.
   Set-up: the first call on a device, with that device current, looks up the
   array's device address (the CUDA runtime loads this part of the library,
   and so creates the 16 MiB array, at that moment unless
   CUDA_MODULE_LOADING=EAGER is set).  Make that first call before any stream
   capture and before the caller's pool takes its memory.  The address is
   kept for the life of the process: a cudaDeviceReset after the first call
   is not supported.  All calls share the array, which keeps the previous
   call's contents (each call overwrites what it reads, nothing needs
   clearing): calls that can overlap on the GPU race.  Returns 0 or an error
   code (see qssgpu_last_error). */
int qssgpu_volume_noalloc(const double *d_phi, const int gb[6], const int ib[6], double dx, double dy,
                          double dz, double epsilon, double *d_volume, void *stream);

/* ---------------- diagnostics and benchmark support ---------------------- */
/* Measurement tools, not part of the path: nothing above calls them. */
/* Device self-test of the integer-pipe FP64 arithmetic against the native
   instructions on n generated operand pairs: counts[0..7] = mismatches of
   div, mul, add, sub, scale2, comparisons, max, sqrt; counts[8] = cases run
   (counts holds 9 values); first = {operation, x, y} of one mismatch (may
   be NULL). */
int qssgpu_emu_selftest(long long n, unsigned long long seed, long long *counts, double *first);
/* Throughput (G operations/s) of native / emulated division, multiplication
   and addition: out[0..5] = div native, div emulated, mul native, mul
   emulated, add native, add emulated; out[6] = multiplications with half
   of the chains native and half emulated (out holds 7 doubles). */
int qssgpu_op_rates(double *out);
/* benchmark support: drain_model3d's set-up for curvature a0 with the arrays
   left in HBM, then timing of `steps` inner steps after `warmup`
   (out[0] total ms, out[1] mean ms per launch of the stage kernel with the
   largest total time, out[2] kernels per step, out[3] ms inside stage
   kernels, out[4] kind of that kernel: 0 fused stage, 1/2/3 WENO5 x/y/z
   pass, 4 WENO5 combine; out[5..9] ms and out[10..14] launches per kind;
   out holds 15 doubles); FP64 throughput probe (TFLOP/s of DFMA, DADD) */
int qssgpu_prepare_step(Options *o, QSS_DataArrays *p, Grid *g, double a0);
int qssgpu_time_steps(Options *o, QSS_DataArrays *p, Grid *g, double a0, int warmup, int steps,
                      double *out);
int qssgpu_fp64_peak(double *out);

#ifdef __cplusplus
}
#endif

#endif /* LSMPQS_GPU_H */
