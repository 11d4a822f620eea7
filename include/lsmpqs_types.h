/*
 * lsmpqs_types.h -- the data model of the lsmpqs level-set library, as seen by
 * C callers of the GB300 implementation.
 *
 * The three structs below must be byte-for-byte identical to the reference
 * library built with QSSLIB_REAL = double, because existing callers allocate
 * and fill them and then hand them to drain_model3d() & co.  Field order,
 * types and names follow:
 *   Grid            src/geometry/qss_grid.h:29-81
 *   QSS_DataArrays  src/utilities/qss_data_arrays.h:24-73
 *   Options         src/utilities/qss_options.h:34-168
 * (tests/test_abi_layout.py checks every offset against a fixture generated
 * from the reference headers).
 *
 * Memory layout of every REAL/int/uchar array: the full ghost box
 * (grid_dims_ghostbox[0] x [1] x [2]), column-major, i fastest:
 *   idx = i + nx*(j + ny*k),  0 <= i < nx, ...
 */
#ifndef LSMPQS_TYPES_H
#define LSMPQS_TYPES_H

#ifndef QSSLIB_REAL
#define QSSLIB_REAL double
#endif
#ifndef LSMLIB_REAL
#define LSMLIB_REAL double
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* Accuracy id used to size the ghost layers (qss_grid.h:92-93).
   Ghost cells per accuracy: LOW 2, MEDIUM 3, HIGH 5, VERY_HIGH 4. */
typedef enum { LOW = 0, MEDIUM = 1, HIGH = 2, VERY_HIGH = 3 }
  QSSLIB_SPATIAL_DERIVATIVE_ACCURACY_TYPE;

typedef struct _Grid {
  int num_dims;
  QSSLIB_REAL x_lo[3];
  QSSLIB_REAL x_hi[3];
  QSSLIB_REAL x_lo_ghostbox[3];
  QSSLIB_REAL x_hi_ghostbox[3];
  int grid_dims[3];
  int grid_dims_ghostbox[3];
  QSSLIB_REAL dx[3];
  int num_gridpts;
  int ilo_gb, ihi_gb, jlo_gb, jhi_gb, klo_gb, khi_gb;
  int ilo_fb, ihi_fb, jlo_fb, jhi_fb, klo_fb, khi_fb;
  int ilo_D1_fb, ihi_D1_fb, jlo_D1_fb, jhi_D1_fb, klo_D1_fb, khi_D1_fb;
  int ilo_D2_fb, ihi_D2_fb, jlo_D2_fb, jhi_D2_fb, klo_D2_fb, khi_D2_fb;
  int ilo_D3_fb, ihi_D3_fb, jlo_D3_fb, jhi_D3_fb, klo_D3_fb, khi_D3_fb;
  int num_nb_levels;
  unsigned char mark_gb, mark_D1, mark_D2, mark_D3, mark_fb;
  QSSLIB_REAL beta, gamma;
} Grid;

typedef struct _QSS_DataArrays {
  QSSLIB_REAL *phi, *phi_next, *phi_extra;
  QSSLIB_REAL *phi_prev;
  QSSLIB_REAL *mask;
  QSSLIB_REAL *lse_rhs;
  QSSLIB_REAL *normal_velocity;
  QSSLIB_REAL *curvature_coeff;
  QSSLIB_REAL *external_velocity_x;
  QSSLIB_REAL *external_velocity_y;
  QSSLIB_REAL *external_velocity_z;
  QSSLIB_REAL *mask_x, *mask_y, *mask_z;
  QSSLIB_REAL *scratch1, *scratch2;
  int *connectivity;
  unsigned char *phi_bin;
  QSSLIB_REAL *mask_w, *mask_nw, *mask_disconn_init;
  QSSLIB_REAL *theta;
  QSSLIB_REAL *overlap;
} QSS_DataArrays;

/* Function-pointer members are declared without a prototype in the
   reference (K&R style); in C++ the closest spelling with the same size is a
   pointer to a variadic function. */
#ifdef __cplusplus
typedef void (*qss_untyped_fn)(...);
#else
typedef void (*qss_untyped_fn)();
#endif

typedef struct _Options {
  char outfile[256];
  char path[256];
  QSSLIB_REAL dx;
  QSSLIB_REAL tmax;
  QSSLIB_REAL tmax_r;
  QSSLIB_REAL tplot;
  char accuracy[20];
  QSSLIB_SPATIAL_DERIVATIVE_ACCURACY_TYPE accuracy_id;
  QSSLIB_REAL a;
  QSSLIB_REAL b;
  int save_data;
  int do_reinit;
  int do_mask;
  QSSLIB_REAL eps_stop;
  int subcell_fix;
  qss_untyped_fn reinit_func;
  QSSLIB_REAL dc;
  QSSLIB_REAL cmax;
  QSSLIB_REAL amax;
  QSSLIB_REAL amin;
  QSSLIB_REAL vol_frac_max;
  QSSLIB_REAL vol_frac_min;
  int mask_reinit;
  int narrow_band;
  int init_step;
  QSSLIB_REAL overlap;
  int stop_touch;
  QSSLIB_REAL eps_coefficient;
  int extrapol_id;
  qss_untyped_fn extrapol_func;
  qss_untyped_fn space_deriv_func;
  int order_space_accur;
  int order_time_accur;
  int checkpoint;
  int reservoir_inlet;
  QSSLIB_REAL theta;
  QSSLIB_REAL C;
  QSSLIB_REAL b_max_over_dx, max_U_over_dx;
  int check_connectivity;
  int phi_w_ind;
  int phi_nw_ind;
  QSSLIB_REAL err_check_zone;
  int use_var_theta;
  QSSLIB_REAL theta_1;
  QSSLIB_REAL theta_2;
  int print_details;
  int use_satn_stop;
  int conserve_imbibe;
  int center_inlet;
} Options;

/* zip_status values of the data-array / grid writers (qss_file.h) */
#define NO_ZIP 0
#define GZIP   1
#define BZIP2  2

#ifdef __cplusplus
}
#endif

#endif /* LSMPQS_TYPES_H */
