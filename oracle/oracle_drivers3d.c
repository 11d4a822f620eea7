/*
 * oracle_drivers3d.c -- TEST INFRASTRUCTURE (oracle), never part of the product.
 *
 * C restatement of the reference's C drivers on the quasi-static level-set
 * path (3-D only), built on the restated kernels of oracle_kernels3d.c.  It
 * exports the reference's own entry-point names so the tests can drive the
 * oracle, the reference C (when it can be compiled) and the GPU library with
 * the same calls.  The OpenMP structure follows the reference: z-slabs of
 * nslices*t/T per thread, serial boundary conditions and copies, so with
 * OMP_NUM_THREADS=T the results equal the reference run with T threads
 * (the CFL step depends on T through the last voxel of each slab).
 *
 * Sources followed (paths inside the reference project):
 *   constCurvModel3d / NoVar   src/level_set_evolution/constCurvModel3d.c:50-334, 336-610
 *   drain_model3d              src/level_set_evolution/drain_model3d.c:49-165
 *   imbibe_model3d             src/level_set_evolution/imbibe_model3d.c:49-161
 *   reinitializeSubcellFix3d   src/reinitialization/reinitialize_top.c:297-377
 *   qss_reinitialize_mask      src/utilities/qss_general_util.c:261-306
 *   createMaskUBC, createInitFromMask, makeDiffSteps, makeRaw (logic of the CLIs)
 *                              src/applications/createMaskUBC.c:76-112,
 *                              createInitFromMask.c:55-85, makeDiffSteps.c:54-132,
 *                              makeRaw.c:52-135
 *   trapComponents_mask        src/connectivity/trapComponents.c:156-375
 *   findConnectivity3d         src/connectivity/connectivity.c:48-217
 *   getMainInd_new             src/connectivity/connectivity.c:219-296
 *   BC / theta / masks / inlet src/utilities/qss_general_util.c:82-207, 422-706, 711-728, 813-833
 *   geometry                   src/geometry/qss_initialization3d.c:33-165, 440-522
 *   grid, arrays, options      src/geometry/qss_grid.c:47-250, 614-763, 789-1035;
 *                              src/utilities/qss_data_arrays.c:30-228;
 *                              src/utilities/qss_options.c:42-117
 *   array macros               src/utilities/qss_macros.h:38-264
 */
#include <float.h>
#include <math.h>
#include <omp.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define QSSLIB_REAL double
#include "../include/lsmpqs_types.h"
#include "oracle_kernels3d.h"

#define GBD(g) &(g)->ilo_gb, &(g)->ihi_gb, &(g)->jlo_gb, &(g)->jhi_gb, &(g)->klo_gb, &(g)->khi_gb
#define FBD(g) &(g)->ilo_fb, &(g)->ihi_fb, &(g)->jlo_fb, &(g)->jhi_fb, &(g)->klo_fb, &(g)->khi_fb

typedef void (*rhs_var_fn)(const double *, const double *, const double *, const double *,
                           const double *, const double *, double *, double *, ...);

/* ------------------------------------------------------------------ */
/* whole-array helpers (qss_macros.h)                                  */
static void arr_copy(double *dst, const double *src, int n)
{ for (int q = 0; q < n; q++) dst[q] = src[q]; }
static void arr_fill(double *dst, double v, int n)
{ for (int q = 0; q < n; q++) dst[q] = v; }
static void arr_max_into(double *out, const double *mask, const double *phi, int n)
{ for (int q = 0; q < n; q++) out[q] = (mask[q] > phi[q]) ? mask[q] : phi[q]; }
static void arr_min_into(double *out, const double *a, const double *b, int n)
{ for (int q = 0; q < n; q++) out[q] = (a[q] < b[q]) ? a[q] : b[q]; }
/* MERGE_SETS: pull trapped non-wetting blobs back into phi */
static void arr_merge(double *phi, const double *m, int n)
{ for (int q = 0; q < n; q++) phi[q] = (m[q] > 0) ? -m[q] : phi[q]; }

/* ------------------------------------------------------------------ */
/* file helpers (qss_file.c, qss_data_arrays.c)                        */
void zipFile(char *file_base, int zip_status)
{
  char cmd[600];
  if (zip_status == GZIP) { snprintf(cmd, sizeof cmd, "gzip -f %s", file_base); if (system(cmd)) {} }
  else if (zip_status == BZIP2) { snprintf(cmd, sizeof cmd, "bzip2 -f %s", file_base); if (system(cmd)) {} }
}

void checkUnzipFile(char *file_name, int *pzip_status, char **pfile_base)
{
  char cmd[600];
  char *base = (char *)malloc(256);
  int zs = NO_ZIP;
  if (strstr(file_name, ".gz")) {
    zs = GZIP;
    snprintf(cmd, sizeof cmd, "gunzip -f %s", file_name); if (system(cmd)) {}
    size_t L = strlen(file_name) - 3; memcpy(base, file_name, L); base[L] = 0;
  } else if (strstr(file_name, ".bz2")) {
    zs = BZIP2;
    snprintf(cmd, sizeof cmd, "bunzip2 -f %s", file_name); if (system(cmd)) {}
    size_t L = strlen(file_name) - 4; memcpy(base, file_name, L); base[L] = 0;
  } else {
    strcpy(base, file_name);
  }
  *pzip_status = zs;
  *pfile_base = base;
}

void writeDataArrayQSS(double *data, Grid *g, char *file_name, int zip_status)
{
  FILE *fp = fopen(file_name, "w");
  if (!fp) { printf("\nCould not open file %s\n", file_name); return; }
  fwrite(g->grid_dims_ghostbox, sizeof(int), 3, fp);
  fwrite(data, sizeof(double), (size_t)g->num_gridpts, fp);
  fclose(fp);
  zipFile(file_name, zip_status);
}

double *readDataArrayQSS(int *dims, char *file_name)
{
  int zs; char *base; double *data = NULL;
  checkUnzipFile(file_name, &zs, &base);
  FILE *fp = fopen(base, "r");
  if (fp) {
    if (fread(dims, sizeof(int), 3, fp) != 3) {}
    size_t n = (size_t)dims[0] * dims[1] * dims[2];
    data = (double *)malloc(n * sizeof(double));
    if (fread(data, sizeof(double), n, fp) != n) {}
    fclose(fp);
    zipFile(base, zs);
  } else {
    printf("\nCould not open file %s", file_name);
  }
  free(base);
  return data;
}

/* ------------------------------------------------------------------ */
/* geometry (qss_initialization3d.c)                                   */
void createIntersectionOfSpheres(double *phi, int num, double *cx, double *cy, double *cz,
                                 double *radius, int *inside_flag, Grid *g)
{
  int nx = g->grid_dims_ghostbox[0], ny = g->grid_dims_ghostbox[1], nz = g->grid_dims_ghostbox[2];
  for (int k = 0; k < nz; k++)
    for (int j = 0; j < ny; j++)
      for (int i = 0; i < nx; i++) {
        double x = g->x_lo_ghostbox[0] + g->dx[0] * i;
        double y = g->x_lo_ghostbox[1] + g->dx[1] * j;
        double z = g->x_lo_ghostbox[2] + g->dx[2] * k;
        double best = -FLT_MAX;
        for (int l = 0; l < num; l++) {
          double d = sqrt((x - cx[l]) * (x - cx[l]) + (y - cy[l]) * (y - cy[l])
                          + (z - cz[l]) * (z - cz[l])) - radius[l];
          if (inside_flag[l] >= 0) d = -d;
          if (d > best) best = d;
        }
        phi[i + nx * (j + ny * k)] = best;
      }
}

void createSphere(double *phi, double cx, double cy, double cz, double r, int inside, Grid *g)
{ createIntersectionOfSpheres(phi, 1, &cx, &cy, &cz, &r, &inside, g); }

void createIntersectionOfHalfSpaces3d(double *phi, int num, double *nxv, double *nyv, double *nzv,
                                      double *px, double *py, double *pz, Grid *g)
{
  int nx = g->grid_dims_ghostbox[0], ny = g->grid_dims_ghostbox[1], nz = g->grid_dims_ghostbox[2];
  for (int k = 0; k < nz; k++)
    for (int j = 0; j < ny; j++)
      for (int i = 0; i < nx; i++) {
        double x = g->x_lo_ghostbox[0] + g->dx[0] * i;
        double y = g->x_lo_ghostbox[1] + g->dx[1] * j;
        double z = g->x_lo_ghostbox[2] + g->dx[2] * k;
        double best = -FLT_MAX;
        for (int l = 0; l < num; l++) {
          double dot = (x - px[l]) * nxv[l] + (y - py[l]) * nyv[l] + (z - pz[l]) * nzv[l];
          double nrm = nxv[l] * nxv[l] + nyv[l] * nyv[l] + nzv[l] * nzv[l];
          nrm = sqrt(nrm);
          double d = dot / nrm;
          if (d > best) best = d;
        }
        phi[i + nx * (j + ny * k)] = best;
      }
}

void createIntersectionOfBoxes(double *phi, int num, double *cx, double *cy, double *cz,
                               double *sx, double *sy, double *sz, int *inside_flag, Grid *g)
{
  int n = g->num_gridpts;
  double *tmp = (double *)malloc((size_t)n * sizeof(double));
  for (int l = 0; l < num; l++) {
    double px[6], py[6], pz[6], nxv[6], nyv[6], nzv[6];
    for (int q = 0; q < 6; q++) {
      int lowside = q < 3, ax = q % 3;
      px[q] = lowside ? cx[l] : cx[l] + sx[l];
      py[q] = lowside ? cy[l] : cy[l] + sy[l];
      pz[q] = lowside ? cz[l] : cz[l] + sz[l];
      double s = lowside ? -1 : 1;
      nxv[q] = (ax == 0) ? s : 0;
      nyv[q] = (ax == 1) ? s : 0;
      nzv[q] = (ax == 2) ? s : 0;
    }
    createIntersectionOfHalfSpaces3d(tmp, 6, nxv, nyv, nzv, px, py, pz, g);
    if (inside_flag[l] >= 1)
      for (int q = 0; q < n; q++) tmp[q] = -tmp[q];
    if (l == 0) arr_copy(phi, tmp, n);
    else arr_max_into(phi, tmp, phi, n);
  }
  free(tmp);
}

void createBox(double *phi, double cx, double cy, double cz, double sx, double sy, double sz,
               int inside, Grid *g)
{ createIntersectionOfBoxes(phi, 1, &cx, &cy, &cz, &sx, &sy, &sz, &inside, g); }

/* ------------------------------------------------------------------ */
/* grid (qss_grid.c)                                                   */
static const int ghost_cells_for_accuracy[4] = {2, 3, 5, 4};

static void set_index_space_limits(QSSLIB_SPATIAL_DERIVATIVE_ACCURACY_TYPE acc, Grid *g)
{
  int n0 = g->grid_dims_ghostbox[0], n1 = g->grid_dims_ghostbox[1], n2 = g->grid_dims_ghostbox[2];
  g->mark_gb = 120; g->mark_D1 = 119; g->mark_D2 = 118; g->mark_D3 = 117;
  g->num_nb_levels = ghost_cells_for_accuracy[acc];
  g->mark_fb = (unsigned char)(g->mark_gb - g->num_nb_levels);
  if (acc > MEDIUM) { g->beta = 3 * g->dx[0]; g->gamma = 6 * g->dx[0]; }
  else              { g->beta = 2 * g->dx[0]; g->gamma = 4 * g->dx[0]; }
  g->ilo_gb = 0; g->ihi_gb = n0 - 1; g->jlo_gb = 0; g->jhi_gb = n1 - 1; g->klo_gb = 0; g->khi_gb = n2 - 1;
  g->ilo_D1_fb = 1; g->ihi_D1_fb = n0 - 2; g->jlo_D1_fb = 1; g->jhi_D1_fb = n1 - 2; g->klo_D1_fb = 1; g->khi_D1_fb = n2 - 2;
  g->ilo_D2_fb = 2; g->ihi_D2_fb = n0 - 3; g->jlo_D2_fb = 2; g->jhi_D2_fb = n1 - 3; g->klo_D2_fb = 2; g->khi_D2_fb = n2 - 3;
  g->ilo_D3_fb = 3; g->ihi_D3_fb = n0 - 4; g->jlo_D3_fb = 3; g->jhi_D3_fb = n1 - 4; g->klo_D3_fb = 3; g->khi_D3_fb = n2 - 4;
  int lo_i, hi_i, lo_j, hi_j, lo_k, hi_k;
  switch (acc) {
    case LOW: /* ENO1 */
      lo_i = g->ilo_D1_fb; hi_i = g->ihi_D1_fb - 1; lo_j = g->jlo_D1_fb; hi_j = g->jhi_D1_fb - 1;
      lo_k = g->klo_D1_fb; hi_k = g->khi_D1_fb - 1; break;
    case HIGH: /* ENO3 */
      lo_i = g->ilo_D3_fb + 1; hi_i = g->ihi_D3_fb - 2; lo_j = g->jlo_D3_fb + 1; hi_j = g->jhi_D3_fb - 2;
      lo_k = g->klo_D3_fb + 1; hi_k = g->khi_D3_fb - 2; break;
    case VERY_HIGH: /* WENO5 */
      lo_i = g->ilo_D1_fb + 2; hi_i = g->ihi_D1_fb - 3; lo_j = g->jlo_D1_fb + 2; hi_j = g->jhi_D1_fb - 3;
      lo_k = g->klo_D1_fb + 2; hi_k = g->khi_D1_fb - 3; break;
    default: /* MEDIUM, ENO2 */
      lo_i = g->ilo_D2_fb + 1; hi_i = g->ihi_D2_fb - 1; lo_j = g->jlo_D2_fb + 1; hi_j = g->jhi_D2_fb - 1;
      lo_k = g->klo_D2_fb + 1; hi_k = g->khi_D2_fb - 1; break;
  }
  g->ilo_fb = lo_i; g->ihi_fb = hi_i; g->jlo_fb = lo_j; g->jhi_fb = hi_j; g->klo_fb = lo_k; g->khi_fb = hi_k;
}

Grid *createGridSetGridDims(int num_dims, int *grid_dims, double *x_lo, double *x_hi,
                            QSSLIB_SPATIAL_DERIVATIVE_ACCURACY_TYPE acc)
{
  Grid *g = (Grid *)calloc(1, sizeof(Grid));
  int ng = ghost_cells_for_accuracy[acc];
  g->num_dims = (num_dims == 2 || num_dims == 3) ? num_dims : 2;
  g->num_gridpts = 1;
  for (int d = 0; d < g->num_dims; d++) {
    g->grid_dims[d] = grid_dims[d];
    g->x_hi[d] = x_hi[d];
    g->x_lo[d] = x_lo[d];
    g->dx[d] = (g->x_hi[d] - g->x_lo[d]) / g->grid_dims[d];
    g->grid_dims_ghostbox[d] = g->grid_dims[d] + 2 * ng;
    g->x_lo_ghostbox[d] = g->x_lo[d] - ng * g->dx[d];
    g->x_hi_ghostbox[d] = g->x_hi[d] + ng * g->dx[d];
    g->num_gridpts *= g->grid_dims_ghostbox[d];
  }
  if (g->num_dims == 2) {
    g->x_lo[2] = g->x_hi[2] = g->x_lo_ghostbox[2] = g->x_hi_ghostbox[2] = 0;
    g->grid_dims[2] = g->grid_dims_ghostbox[2] = 1;
    g->dx[2] = 0;
  }
  set_index_space_limits(acc, g);
  return g;
}

void destroyGrid(Grid *g) { free(g); }

/* ------------------------------------------------------------------ */
/* data arrays (qss_data_arrays.c)                                     */
#define DUMMY ((double *)(-1))
QSS_DataArrays *allocateQSSDataArrays(void)
{
  QSS_DataArrays *p = (QSS_DataArrays *)malloc(sizeof(QSS_DataArrays));
  double **r[] = {&p->phi, &p->phi_next, &p->phi_extra, &p->phi_prev, &p->mask, &p->lse_rhs,
                  &p->normal_velocity, &p->curvature_coeff, &p->external_velocity_x,
                  &p->external_velocity_y, &p->external_velocity_z, &p->mask_x, &p->mask_y,
                  &p->mask_z, &p->scratch1, &p->scratch2, &p->mask_w, &p->mask_nw,
                  &p->mask_disconn_init, &p->theta, &p->overlap};
  for (size_t q = 0; q < sizeof r / sizeof r[0]; q++) *r[q] = DUMMY;
  p->connectivity = (int *)(-1);
  p->phi_bin = (unsigned char *)(-1);
  return p;
}

void allocateMemoryForQSSDataArrays(QSS_DataArrays *p, Grid *g)
{
  size_t n = (size_t)g->num_gridpts;
  double **zeroed[] = {&p->phi, &p->phi_next, &p->phi_extra, &p->phi_prev, &p->mask};
  for (size_t q = 0; q < 5; q++) if (*zeroed[q] == DUMMY) *zeroed[q] = (double *)calloc(n, sizeof(double));
  double **plain[] = {&p->lse_rhs, &p->normal_velocity, &p->curvature_coeff,
                      &p->external_velocity_x, &p->external_velocity_y, &p->external_velocity_z,
                      &p->mask_x, &p->mask_y, &p->mask_z, &p->scratch1, &p->scratch2,
                      &p->theta, &p->overlap, &p->mask_w, &p->mask_nw, &p->mask_disconn_init};
  for (size_t q = 0; q < sizeof plain / sizeof plain[0]; q++) {
    int is_z = (plain[q] == &p->external_velocity_z || plain[q] == &p->mask_z);
    if (is_z && g->num_dims != 3) { *plain[q] = NULL; continue; }
    if (*plain[q] == DUMMY) *plain[q] = (double *)malloc(n * sizeof(double));
  }
  if (p->connectivity == (int *)(-1)) p->connectivity = (int *)malloc(n * sizeof(int));
  if (p->phi_bin == (unsigned char *)(-1)) p->phi_bin = (unsigned char *)malloc(n);
}

void destroyQSSDataArrays(QSS_DataArrays *p)
{
  if (!p) return;
  double *r[] = {p->phi, p->phi_next, p->phi_extra, p->phi_prev, p->mask, p->lse_rhs,
                 p->normal_velocity, p->curvature_coeff, p->external_velocity_x,
                 p->external_velocity_y, p->external_velocity_z, p->mask_x, p->mask_y,
                 p->mask_z, p->scratch1, p->scratch2, p->mask_w, p->mask_nw,
                 p->mask_disconn_init, p->theta, p->overlap};
  for (size_t q = 0; q < sizeof r / sizeof r[0]; q++) free(r[q]);
  free(p->connectivity);
  free(p->phi_bin);
  free(p);
}

/* ------------------------------------------------------------------ */
/* options (qss_options.c:42-117)                                      */
void signedLinearExtrapolationBCqss(double *phi, Grid *g, int idx);

Options *createOptionsDefault(void)
{
  Options *o = (Options *)calloc(1, sizeof(Options));
  snprintf(o->outfile, sizeof o->outfile, "out_file");
  snprintf(o->path, sizeof o->path, "./");
  o->dx = 0.04; o->tmax = 150.0; o->tplot = 0.5;
  snprintf(o->accuracy, sizeof o->accuracy, "medium");
  o->accuracy_id = MEDIUM;
  o->a = 0.15; o->b = 0.04;
  o->save_data = 1; o->do_reinit = 1; o->do_mask = 1;
  o->eps_stop = 0.014; o->narrow_band = 0; o->overlap = 0;
  o->init_step = 0; o->print_details = 1;
  o->tmax_r = 10 * o->dx;
  o->subcell_fix = 1; o->dc = 0.1;
  o->cmax = 1.0 / (o->dx / 2.0);
  o->amax = 10; o->amin = 0.05;
  o->vol_frac_max = 0.97; o->vol_frac_min = 0;
  o->mask_reinit = 1; o->stop_touch = 1;
  o->eps_coefficient = 1.5;
  o->extrapol_id = 0;
  o->extrapol_func = (qss_untyped_fn)signedLinearExtrapolationBCqss;
  o->space_deriv_func = (qss_untyped_fn)getrhs3d5th_;
  o->checkpoint = 0; o->reservoir_inlet = 1;
  o->theta = 0; o->C = 1;
  o->check_connectivity = 1;
  o->err_check_zone = 20 * o->dx;
  o->phi_w_ind = 0; o->phi_nw_ind = 0;
  o->use_var_theta = 0;
  o->order_space_accur = 3; o->order_time_accur = 3;
  o->use_satn_stop = 1; o->conserve_imbibe = 0; o->center_inlet = 0;
  return o;
}

void destroyOptions(Options *o) { free(o); }

/* ------------------------------------------------------------------ */
/* boundary conditions, scheme selection, overlap, masks, inlet        */
void signedLinearExtrapolationBCqss(double *phi, Grid *g, int idx)
{
  if (g->num_dims != 3) return; /* the 2-D path is outside this oracle */
  int faces[6], nf = 0;
  switch (idx) {
    case 0: case 1: case 2: case 3: case 4: case 5: faces[nf++] = idx; break;
    case 6: faces[nf++] = 0; faces[nf++] = 1; break;
    case 7: faces[nf++] = 2; faces[nf++] = 3; break;
    case 8: faces[nf++] = 4; faces[nf++] = 5; break;
    case 9: for (int f = 0; f < 6; f++) faces[nf++] = f; break;
    default: break;
  }
  for (int q = 0; q < nf; q++) signedlinearextrapolation3d_(phi, GBD(g), FBD(g), &faces[q]);
}

void setSpaceDerivFunc(Grid *g, Options *o)
{
  (void)g; /* 3-D selection of qss_general_util.c:115-141; '~use_var_theta' is always true */
  int plain = (o->theta == 0);
  switch (o->order_space_accur) {
    case 2: o->space_deriv_func = plain ? (qss_untyped_fn)getrhs3d2ndconst_ : (qss_untyped_fn)getrhs3d2nd_; break;
    case 3: case 4:
      o->space_deriv_func = plain ? (qss_untyped_fn)getrhs3d3rdconst_ : (qss_untyped_fn)getrhs3d3rd_; break;
    case 5: o->space_deriv_func = plain ? (qss_untyped_fn)getrhs3d3rdconst_ : (qss_untyped_fn)getrhs3d5th_; break;
    default: o->space_deriv_func = (qss_untyped_fn)getrhs3d3rd_;
  }
}

void setThetaOverlap(QSS_DataArrays *p, Grid *g, Options *o)
{
  (void)p; /* constant-theta branch only: '~use_var_theta' is always true */
  double rad = 3.14159 / 180;
  double th = o->theta;
  if (g->num_dims == 3) {
    if (th <= 20 * rad) o->overlap = 0;
    else if (th <= 40 * rad) o->overlap = 0.3 * g->dx[0];
    else if (th <= 50 * rad) o->overlap = 0.5 * g->dx[0];
    else if (th > 50 * rad) o->overlap = 1 * g->dx[0];
  } else {
    o->overlap = (th <= 20 * rad) ? 0 : 3 * g->dx[0];
  }
}

void initializeDisconnectedMasks(double *data, Grid *g)
{
  double cz = 0.5 * (g->x_lo[2] + g->x_hi[2]);
  double cy = 0.5 * (g->x_lo[1] + g->x_hi[1]);
  double cx = 0.5 * (g->x_lo[0] + g->x_hi[0]);
  double r = 2 * (g->x_hi[0] - g->x_lo[0]);
  createSphere(data, cx, cy, cz, r, -1, g);
}

void createReservoirInlet3d(QSS_DataArrays *p, Grid *g)
{
  createBox(p->phi_extra, g->x_lo_ghostbox[0], g->x_lo_ghostbox[1], g->x_lo_ghostbox[2],
            3 * g->dx[0], g->x_hi_ghostbox[1] - g->x_lo_ghostbox[1],
            g->x_hi_ghostbox[2] - g->x_lo_ghostbox[2], -1, g);
}

/* ------------------------------------------------------------------ */
/* reinitialisation (reinitialize_top.c:297-377)                        */
void reinitializeSubcellFix3d(double *data, Grid *g, Options *o)
{
  int n = g->num_gridpts;
  double *distance0 = (double *)malloc((size_t)n * sizeof(double));
  double *copy = (double *)malloc((size_t)n * sizeof(double));
  double *rhs = (double *)malloc((size_t)n * sizeof(double));
  double *next = (double *)malloc((size_t)n * sizeof(double));
  double t_r = 0, dt_r = 0.5 * g->dx[0];
  arr_copy(copy, data, n);
  qss3dcomputedistanceforsubcellfix_(distance0, copy, GBD(g), FBD(g), &g->dx[0], &g->dx[1], &g->dx[2]);
#pragma omp parallel
  {
    int T = omp_get_num_threads(), tid = omp_get_thread_num();
    int ns = g->khi_fb - g->klo_fb + 1;
    int klo = g->klo_fb + ns * tid / T;
    int khi = g->klo_fb + ns * (tid + 1) / T - 1;
#pragma omp barrier
    while (t_r < o->tmax_r) {
      qss3dcomputereinitializationeqnrhssubcellfixorder1_(
          rhs, data, GBD(g), copy, distance0, &g->ilo_fb, &g->ihi_fb, &g->jlo_fb, &g->jhi_fb,
          &klo, &khi, &g->dx[0], &g->dx[1], &g->dx[2]);
#pragma omp barrier
      qss3drk1step_(next, GBD(g), data, GBD(g), rhs, GBD(g), &g->ilo_fb, &g->ihi_fb,
                    &g->jlo_fb, &g->jhi_fb, &klo, &khi, &dt_r);
#pragma omp barrier
#pragma omp single
      signedLinearExtrapolationBCqss(next, g, 9);
#pragma omp single
      arr_copy(data, next, n);
#pragma omp single
      arr_fill(rhs, 0, n);
#pragma omp single
      t_r = t_r + dt_r;
    }
  }
  free(distance0); free(copy); free(rhs); free(next);
}

/* ------------------------------------------------------------------ */
/* mask reinitialisation (qss_general_util.c:261-306): serial, distance0 in
   scratch1, the initial mask in scratch2, the RHS in lse_rhs, the RK1
   output in phi_next                                                    */
void qss_reinitialize_mask(QSS_DataArrays *p, Grid *g, Options *o)
{
  double *distance0 = p->scratch1, *copy = p->scratch2;
  double t_r = 0, dt_r = 0.5 * g->dx[0];
  arr_copy(copy, p->mask, g->num_gridpts);
  qss3dcomputedistanceforsubcellfix_(distance0, copy, GBD(g), FBD(g), &g->dx[0], &g->dx[1], &g->dx[2]);
  while (t_r < o->tmax_r) {
    qss3dcomputereinitializationeqnrhssubcellfixorder1_(p->lse_rhs, p->mask, GBD(g), copy, distance0,
                                                        FBD(g), &g->dx[0], &g->dx[1], &g->dx[2]);
    qss3drk1step_(p->phi_next, GBD(g), p->mask, GBD(g), p->lse_rhs, GBD(g), FBD(g), &dt_r);
    signedLinearExtrapolationBCqss(p->phi_next, g, 9);
    arr_copy(p->mask, p->phi_next, g->num_gridpts);
    t_r = t_r + dt_r;
  }
}

/* createMaskUBC.c:76-112 on caller arrays: mask = +-dx from a 255/0 image of
   the fill box (x fastest), zero ghost layers, then the mask reinitialisation */
int oracle_create_mask_ubc(const unsigned char *ubc, QSS_DataArrays *p, Grid *g, Options *o)
{
  int nx = g->grid_dims_ghostbox[0], nxy = nx * g->grid_dims_ghostbox[1];
  int fx = g->ihi_fb - g->ilo_fb + 1, fy = g->jhi_fb - g->jlo_fb + 1;
  arr_fill(p->mask, 0.0, g->num_gridpts);
  for (int k = g->klo_fb; k <= g->khi_fb; k++)
    for (int j = g->jlo_fb; j <= g->jhi_fb; j++)
      for (int i = g->ilo_fb; i <= g->ihi_fb; i++) {
        int idx = (i - g->ilo_fb) + (j - g->jlo_fb) * fx + (k - g->klo_fb) * fx * fy;
        int idx_gb = (i - g->ilo_gb) + (j - g->jlo_gb) * nx + (k - g->klo_gb) * nxy;
        p->mask[idx_gb] = (ubc[idx] == 255) ? o->dx : -o->dx;
      }
  qss_reinitialize_mask(p, g, o);
  return 0;
}

/* createInitFromMask.c:55-85 (3-D): a sphere around the inlet, then
   IMPOSE_MASK(phi, mask, phi)                                            */
int oracle_create_init_from_mask(QSS_DataArrays *p, Grid *g, Options *o)
{
  double radius, cx, cy, cz;
  if (o->center_inlet) {
    radius = 90 * g->dx[0];
    cy = 0.5 * (g->x_lo[1] + g->x_hi[1]);
    cx = 0.5 * (g->x_lo[1] + g->x_hi[1]);
    cz = 0.5 * (g->x_lo[2] + g->x_hi[2]);
  } else {
    radius = 0.7 * (g->x_hi[0] - g->x_lo[0]);
    cy = 0.5 * (g->x_lo[1] + g->x_hi[1]);
    cx = (g->x_lo[0]) - radius * 0.7;
    cz = 0.5 * (g->x_lo[2] + g->x_hi[2]);
  }
  createSphere(p->phi, cx, cy, cz, radius, -1, g);
  arr_max_into(p->phi, p->mask, p->phi, g->num_gridpts);
  return 0;
}

/* makeDiffSteps.c:54-132 (3-D) on arrays: diff = max(-a, b - dx/2), then the
   inlet/outlet slabs, 26-connected labels and the percolation check; when
   it percolates, connected = diff with the non-wetting voxels outside the
   main component flipped                                                   */
void findConnectivity3d(QSS_DataArrays *p, Grid *g);
int oracle_diff_steps(const double *a, const double *b, Grid *g, double *diff, double *connected,
                      int *percolates)
{
  int n = g->num_gridpts, nx = g->grid_dims_ghostbox[0], nxy = nx * g->grid_dims_ghostbox[1];
  QSS_DataArrays q;
  memset(&q, 0, sizeof q);
  q.phi_bin = (unsigned char *)malloc((size_t)n);
  q.connectivity = (int *)malloc((size_t)n * sizeof(int));
  for (int i = 0; i < n; i++) {
    double m = -a[i];
    double ph = b[i];
    ph -= 0.5 * g->dx[0];
    diff[i] = (m > ph) ? m : ph;
    q.phi_bin[i] = (diff[i] < 0) ? 1 : 0;
  }
  for (int k = g->klo_fb; k <= g->khi_fb; k++)
    for (int j = g->jlo_fb; j <= g->jhi_fb; j++) {
      q.phi_bin[(g->ilo_fb - 1) + j * nx + k * nxy] = 1;
      q.phi_bin[(g->ihi_fb + 1) + j * nx + k * nxy] = 1;
    }
  findConnectivity3d(&q, g);
  int j = 0.5 * (g->jlo_fb + g->jhi_fb), k = 0.5 * (g->klo_fb + g->khi_fb);
  int inlet = (g->ilo_fb - 1) + j * nx + k * nxy, outlet = (g->ihi_fb + 1) + j * nx + k * nxy;
  *percolates = q.connectivity[inlet] == q.connectivity[outlet];
  if (*percolates && connected) {
    int main_val = q.connectivity[inlet];
    for (int i = 0; i < n; i++) {
      double ph = diff[i];
      if ((q.connectivity[i] != main_val) & (ph <= 0)) ph *= -1;
      connected[i] = ph;
    }
  }
  free(q.phi_bin);
  free(q.connectivity);
  return 0;
}

/* makeRaw.c:52-135: 0/1 image of f < 0 (IMPOSE_UCHAR) for f = mask ('m'),
   phi ('n') or max(mask, -phi) ('w': COPY_DATA, NEGATE_DATA, IMPOSE_MASK);
   full = ghost box, fb = fill box packed i fastest (copyDataFB)            */
int oracle_phase_uchar(const double *phi, const double *mask, Grid *g, char phase, unsigned char *full,
                       unsigned char *fb)
{
  int n = g->num_gridpts, nx = g->grid_dims_ghostbox[0], nxy = nx * g->grid_dims_ghostbox[1];
  unsigned char *img = (unsigned char *)malloc((size_t)n);
  double *s = (double *)malloc((size_t)n * sizeof(double));
  if (phase == 'm') {
    for (int i = 0; i < n; i++) img[i] = (mask[i] < 0) ? 1 : 0;
  } else if (phase == 'n') {
    for (int i = 0; i < n; i++) img[i] = (phi[i] < 0) ? 1 : 0;
  } else {
    for (int i = 0; i < n; i++) s[i] = phi[i];
    for (int i = 0; i < n; i++) s[i] = -s[i];
    for (int i = 0; i < n; i++) s[i] = (mask[i] > s[i]) ? mask[i] : s[i];
    for (int i = 0; i < n; i++) img[i] = (s[i] < 0) ? 1 : 0;
  }
  if (full) memcpy(full, img, (size_t)n);
  if (fb) {
    int fx = g->ihi_fb - g->ilo_fb + 1, fy = g->jhi_fb - g->jlo_fb + 1;
    for (int k = g->klo_fb; k <= g->khi_fb; k++)
      for (int j = g->jlo_fb; j <= g->jhi_fb; j++)
        for (int i = g->ilo_fb; i <= g->ihi_fb; i++)
          fb[(i - g->ilo_fb) + (j - g->jlo_fb) * fx + (k - g->klo_fb) * fx * fy] = img[i + j * nx + k * nxy];
  }
  free(img);
  free(s);
  return 0;
}

/* ------------------------------------------------------------------ */
/* connectivity (connectivity.c): union-find whose root is the largest
   linear ghost-box index of its component; 0 marks background          */
static int uf_find(int *parent, int n, int x)
{
  int root = x;
  while (parent[root] < n) root = parent[root];
  while (parent[x] < n) { int nx = parent[x]; parent[x] = root; x = nx; }
  return root;
}

static void uf_union(int *parent, int n, int a, int b)
{
  int ra = uf_find(parent, n, a), rb = uf_find(parent, n, b);
  if (ra == rb) return;
  if (ra < rb) parent[ra] = rb; else parent[rb] = ra;
}

void findConnectivity3d(QSS_DataArrays *p, Grid *g)
{
  int nx = g->grid_dims_ghostbox[0], ny = g->grid_dims_ghostbox[1], nz = g->grid_dims_ghostbox[2];
  int n = nx * ny * nz;
  int *parent = (int *)malloc((size_t)n * sizeof(int));
  for (int q = 0; q < n; q++) parent[q] = n; /* n marks a root */
  const unsigned char *bin = p->phi_bin;
  for (int k = 0; k < nz; k++)
    for (int j = 0; j < ny; j++)
      for (int i = 0; i < nx; i++) {
        int c = i + nx * (j + ny * k);
        if (!bin[c]) continue;
        for (int dk = -1; dk <= 1; dk++)
          for (int dj = -1; dj <= 1; dj++)
            for (int di = -1; di <= 1; di++) {
              if (!di && !dj && !dk) continue;
              int i2 = i + di, j2 = j + dj, k2 = k + dk;
              if (i2 < 0 || j2 < 0 || k2 < 0 || i2 >= nx || j2 >= ny || k2 >= nz) continue;
              int c2 = i2 + nx * (j2 + ny * k2);
              if (bin[c2]) uf_union(parent, n, c, c2);
            }
      }
  for (int c = 0; c < n; c++)
    p->connectivity[c] = bin[c] ? uf_find(parent, n, c) : 0;
  free(parent);
}

void getMainInd_new(Options *o, QSS_DataArrays *p, Grid *g)
{
  (void)p;
  int nx = g->grid_dims_ghostbox[0], nxy = nx * g->grid_dims_ghostbox[1];
  int yi = (int)(0.5 * (g->jlo_fb + g->jhi_fb));
  int zi = (int)(0.5 * (g->klo_fb + g->khi_fb));
  int nwx = o->center_inlet ? (int)(0.5 * (g->ilo_fb + g->ihi_fb)) : g->ilo_fb - 1;
  o->phi_nw_ind = nwx + yi * nx + zi * nxy;
  o->phi_w_ind = (g->ihi_fb + 1) + yi * nx + zi * nxy;
}

static void disconnected_flags(unsigned char *flag, const int *conn, int main_label, int n)
{
  for (int q = 0; q < n; q++) flag[q] = (conn[q] == main_label || conn[q] == 0) ? 0 : 1;
}

void trapComponents_mask(QSS_DataArrays *p, Grid *g, Options *o)
{
  int n = g->num_gridpts;
  int nx = g->grid_dims_ghostbox[0], nxy = nx * g->grid_dims_ghostbox[1];
  unsigned char *disc = (unsigned char *)malloc((size_t)n);
  double eps = 0;
  arr_merge(p->phi, p->mask_nw, n);
  for (int q = 0; q < n; q++) p->phi_bin[q] = (p->phi[q] < eps) ? 1 : 0;
  if (o->center_inlet) {
    int k = (int)(0.5 * (g->klo_fb + g->khi_fb)), i = (int)(0.5 * (g->ilo_fb + g->ihi_fb));
    for (int j = g->jlo_gb; j <= g->jhi_gb; j++) p->phi_bin[i + j * nx + k * nxy] = 1;
  } else {
    int i = g->ilo_fb - 1;
    for (int k = g->klo_fb; k <= g->khi_fb; k++)
      for (int j = g->jlo_fb; j <= g->jhi_fb; j++) p->phi_bin[i + j * nx + k * nxy] = 1;
  }
  findConnectivity3d(p, g);
  disconnected_flags(disc, p->connectivity, p->connectivity[o->phi_nw_ind], n);
  arr_fill(p->mask_nw, -20 * g->dx[0], n);
  for (int q = 0; q < n; q++)
    if (disc[q] == 1 && p->phi[q] < 0) p->mask_nw[q] = -p->phi[q];
  for (int q = 0; q < n; q++) p->connectivity[q] = 0;

  /* wetting phase */
  arr_copy(p->scratch1, p->phi, n);
  for (int q = 0; q < n; q++) p->scratch1[q] = -p->scratch1[q];
  arr_max_into(p->scratch1, p->mask, p->scratch1, n);
  arr_max_into(p->scratch1, p->mask_nw, p->scratch1, n);
  for (int q = 0; q < n; q++) p->phi_bin[q] = (p->scratch1[q] < eps) ? 1 : 0;
  if (o->center_inlet) {
    for (int j = g->jlo_gb; j <= g->jhi_gb; j++)
      for (int i = g->ilo_gb; i <= g->ihi_gb; i++) {
        p->phi_bin[i + j * nx + (g->klo_fb - 1) * nxy] = 1;
      }
    for (int j = g->jlo_gb; j <= g->jhi_gb; j++)
      for (int i = g->ilo_gb; i <= g->ihi_gb; i++) {
        p->phi_bin[i + j * nx + (g->khi_fb + 1) * nxy] = 1;
      }
    for (int j = g->jlo_gb; j <= g->jhi_gb; j++)
      for (int k = g->klo_gb; k <= g->khi_gb; k++) {
        p->phi_bin[(g->ilo_fb - 1) + j * nx + k * nxy] = 1;
      }
    for (int j = g->jlo_gb; j <= g->jhi_gb; j++)
      for (int k = g->klo_gb; k <= g->khi_gb; k++) {
        p->phi_bin[(g->ihi_fb + 1) + j * nx + k * nxy] = 1;
      }
  } else {
    int i = g->ihi_fb + 1;
    for (int k = g->klo_fb; k <= g->khi_fb; k++)
      for (int j = g->jlo_fb; j <= g->jhi_fb; j++) p->phi_bin[i + j * nx + k * nxy] = 1;
  }
  findConnectivity3d(p, g);
  disconnected_flags(disc, p->connectivity, p->connectivity[o->phi_w_ind], n);
  arr_fill(p->mask_w, -20 * g->dx[0], n);
  for (int q = 0; q < n; q++)
    if (disc[q] == 1 && p->scratch1[q] < 0) p->mask_w[q] = -p->scratch1[q];
  arr_fill(p->scratch1, 0, n);
  free(disc);
}

/* ------------------------------------------------------------------ */
/* the constant-curvature model (constCurvModel3d.c)                   */
static double volume_below_zero(const double *f, Grid *g, double eps)
{
  double v;
  qss3dvolumeregionphilessthanzero_(&v, f, GBD(g), FBD(g), &g->dx[0], &g->dx[1], &g->dx[2], &eps);
  return v;
}

typedef void (*rhs_const_fn)(const double *, const double *, const double *, double *, double *,
                             const int *, const int *, const int *, const int *, const int *,
                             const int *, const int *, const int *, const int *, const int *,
                             const int *, const int *, const double *, const double *,
                             const double *);
typedef void (*rhs_full_fn)(const double *, const double *, const double *, const double *,
                            const double *, const double *, double *, double *, const int *,
                            const int *, const int *, const int *, const int *, const int *,
                            const int *, const int *, const int *, const int *, const int *,
                            const int *, const double *, const double *, const double *);

/* the pseudo-time inner loop of constCurvModel3d.c:85-251; max_steps > 0
   stops after that many steps (used to time the CPU baseline) */
static void inner_loop(int var, Options *o, QSS_DataArrays *p, Grid *g, FILE *fp_out, double a,
                       double *dt_sub_p, double *cur_max_H_p, int max_steps)
{
  int n = g->num_gridpts;
  double zero = 0.0, disconn_overlap = 0.0, cfl = 0.5;
  double dt_sub = *dt_sub_p, cur_max_H = *cur_max_H_p;
  int steps = 0;
  rhs_const_fn rc = (rhs_const_fn)o->space_deriv_func;
  rhs_full_fn rf = (rhs_full_fn)o->space_deriv_func;
#pragma omp parallel
    {
      int T = omp_get_num_threads(), tid = omp_get_thread_num();
      int ns = g->khi_fb - g->klo_fb + 1;
      int klo = g->klo_fb + ns * tid / T;
      int khi = g->klo_fb + ns * (tid + 1) / T - 1;
      if (khi > g->khi_fb) khi = g->khi_fb;
      int kglo = (tid == 0) ? klo - 3 : klo;
      int kghi = (tid == T - 1) ? khi + 3 : khi;
      double my_H = -1, dt;
      double t1 = omp_get_wtime();
#define RHS_CALL(src)                                                                         \
      do {                                                                                     \
        if (var) rf(src, p->normal_velocity, p->curvature_coeff, p->external_velocity_x,       \
                    p->external_velocity_y, p->external_velocity_z, &my_H, p->lse_rhs, GBD(g), \
                    &g->ilo_fb, &g->ihi_fb, &g->jlo_fb, &g->jhi_fb, &klo, &khi, &g->dx[0],     \
                    &g->dx[1], &g->dx[2]);                                                     \
        else rc(src, &a, &o->b, &my_H, p->lse_rhs, GBD(g), &g->ilo_fb, &g->ihi_fb,             \
                &g->jlo_fb, &g->jhi_fb, &klo, &khi, &g->dx[0], &g->dx[1], &g->dx[2]);          \
      } while (0)

      while (dt_sub < o->tplot && (max_steps <= 0 || steps < max_steps)) {
        RHS_CALL(p->phi);
#pragma omp barrier
#pragma omp critical
        {
          if (my_H > cur_max_H) cur_max_H = my_H;
        }
#pragma omp barrier
        dt = cfl / (cur_max_H + o->b_max_over_dx + o->max_U_over_dx);
        qss3drk1step_(p->phi_next, GBD(g), p->phi, GBD(g), p->lse_rhs, GBD(g), &g->ilo_fb,
                      &g->ihi_fb, &g->jlo_fb, &g->jhi_fb, &klo, &khi, &dt);
#pragma omp barrier
#pragma omp single
        {
          signedLinearExtrapolationBCqss(p->phi_next, g, 9);
          cur_max_H = -1;
        }
        if (o->order_time_accur >= 2) {
          double *stage = var ? p->scratch2 : p->scratch1;
          RHS_CALL(p->phi_next);
#pragma omp barrier
          qss3dtvdrk2stage2_(stage, GBD(g), p->phi_next, GBD(g), p->phi, GBD(g), p->lse_rhs,
                             GBD(g), &g->ilo_fb, &g->ihi_fb, &g->jlo_fb, &g->jhi_fb, &klo, &khi,
                             &dt);
#pragma omp barrier
#pragma omp single
          arr_copy(p->phi_next, stage, n);
#pragma omp single
          signedLinearExtrapolationBCqss(p->phi_next, g, 9);
        }
        if (o->order_time_accur >= 3) {
          RHS_CALL(p->phi_next);
#pragma omp barrier
          qss3dtvdrk3stage3_(p->scratch2, GBD(g), p->phi_next, GBD(g), p->phi, GBD(g),
                             p->lse_rhs, GBD(g), &g->ilo_fb, &g->ihi_fb, &g->jlo_fb, &g->jhi_fb,
                             &klo, &khi, &dt);
#pragma omp barrier
#pragma omp single
          arr_copy(p->phi_next, p->scratch2, n);
#pragma omp single
          signedLinearExtrapolationBCqss(p->phi_next, g, 9);
        }
#pragma omp single
        {
          arr_fill(p->lse_rhs, zero, n);
          arr_fill(p->scratch1, zero, n);
          arr_fill(p->scratch2, zero, n);
          dt_sub += dt;
          steps++;
        }
#pragma omp barrier
        imposemaskparallel_(p->phi, p->mask, p->phi_next, &o->overlap, GBD(g), &kglo, &kghi);
#pragma omp barrier
        if (o->check_connectivity)
          imposemaskparallel_(p->phi, p->mask_w, p->phi, &disconn_overlap, GBD(g), &kglo, &kghi);
#pragma omp barrier
        if (o->check_connectivity)
          imposemaskparallel_(p->phi, p->mask_nw, p->phi, &disconn_overlap, GBD(g), &kglo, &kghi);
#pragma omp barrier
      }
#undef RHS_CALL
      if (tid == 0 && fp_out)
        fprintf(fp_out, "%d threads: Level set time = %lf\n", T, omp_get_wtime() - t1);
    }

  *dt_sub_p = dt_sub;
  *cur_max_H_p = cur_max_H;
}

/* var != 0: constCurvModel3d (coefficient arrays); var == 0: NoVar with scalar a */
static double const_curv_model(int var, Options *o, QSS_DataArrays *p, Grid *g, FILE *fp_out,
                               double a)
{
  int n = g->num_gridpts;
  double dt_sub = 0, t = 0, cur_max_H = -1;
  double max_abs_err = 100, vol_phi = 100;
  double vol_very_small = g->dx[0] * g->dx[1] * g->dx[2];
  double eps = o->eps_coefficient * g->dx[0];
  double max_satn = o->vol_frac_max;
  double vol_pore = volume_below_zero(p->mask, g, eps);
  vol_phi = volume_below_zero(p->phi, g, eps);
  double satn = vol_phi / vol_pore, satn_old;

  while ((t < o->tmax) && (max_abs_err > o->eps_stop)) {
    dt_sub = 0;
    arr_copy(p->phi_prev, p->phi, n);
    inner_loop(var, o, p, g, fp_out, a, &dt_sub, &cur_max_H, 0);

    t += dt_sub;
    if (var) arr_max_into(p->phi, p->mask, p->phi, n);
    if (o->check_connectivity) {
      trapComponents_mask(p, g, o);
      reinitializeSubcellFix3d(p->mask_w, g, o);
      reinitializeSubcellFix3d(p->mask_nw, g, o);
      if (var && o->conserve_imbibe)
        imposetrapvelocity3d_(p->mask_nw, p->mask_w, p->normal_velocity, p->curvature_coeff,
                              p->external_velocity_x, p->external_velocity_y,
                              p->external_velocity_z, GBD(g), FBD(g), &g->dx[0]);
      arr_merge(p->phi, p->mask_nw, n);
    }
    if (fp_out) fprintf(fp_out, "Reinitializing....");
    reinitializeSubcellFix3d(p->phi, g, o);
    if (fp_out) fprintf(fp_out, "Reinitialized\n");
    qss3dmaxnormdifflocal_(&max_abs_err, p->phi, GBD(g), p->phi_prev, GBD(g), FBD(g),
                           &o->err_check_zone);
    satn_old = satn;
    vol_phi = volume_below_zero(p->phi, g, eps);
    satn = vol_phi / vol_pore;
    if ((satn > max_satn) || (vol_phi <= vol_very_small)) return -1;
    if (o->checkpoint) {
      writeDataArrayQSS(p->phi, g, "checkpoint_phi", GZIP);
      writeDataArrayQSS(p->phi_prev, g, "checkpoint_phi_prev", GZIP);
      writeDataArrayQSS(p->mask_w, g, "mask_w", GZIP);
      writeDataArrayQSS(p->mask_nw, g, "mask_nw", GZIP);
    }
    if (fp_out) {
      fprintf(fp_out, "connectivity time = %lf\n", 0.0);
      fprintf(fp_out, "t = %4.1f\t", t);
      fprintf(fp_out, "max_abs_err = %4.3f,\t", max_abs_err);
      fprintf(fp_out, "nw phase satn pct = %4.3f\n", satn * 100);
      fflush(fp_out);
    }
    printf("t = %4.1f\t", t);
    printf("max_abs_err = %4.3f,\t", max_abs_err);
    printf("nw phase satn = %4.3f\n", satn * 100);
    if (o->use_satn_stop) {
      if (fabsf((float)(100 * (satn - satn_old))) < 0.001) break;
    }
  }
  return t;
}

double constCurvModel3d(Options *o, QSS_DataArrays *p, Grid *g, FILE *fp_out)
{ return const_curv_model(1, o, p, g, fp_out, 0.0); }

double constCurvModel3dNoVar(Options *o, QSS_DataArrays *p, Grid *g, FILE *fp_out, double a)
{ return const_curv_model(0, o, p, g, fp_out, a); }

/* ------------------------------------------------------------------ */
/* curvature ladders (drain_model3d.c, imbibe_model3d.c)                */
static void ladder(int drain, Options *o, QSS_DataArrays *p, Grid *g, FILE *fp_out)
{
  char fname[256];
  int dims[3];
  double a0 = o->a;
  double da = o->b * o->dc;
  int step = o->init_step + 1;
  int n = g->num_gridpts;
  initializeDisconnectedMasks(p->mask_w, g);
  initializeDisconnectedMasks(p->mask_nw, g);
  arr_copy(p->mask_disconn_init, p->mask_nw, n);
  createReservoirInlet3d(p, g);
  double amax = o->amax, amin = o->amin;
  if (drain && o->mask_reinit) reinitializeSubcellFix3d(p->mask, g, o);
  getcentralgrad3dorder2_(p->mask_x, p->mask_y, p->mask_z, GBD(g), p->mask, GBD(g), FBD(g),
                          &g->dx[0], &g->dx[1], &g->dx[2]);
  if (o->use_var_theta) {
    snprintf(fname, sizeof fname, "theta.gz");
    p->theta = readDataArrayQSS(dims, fname);
  }
  setSpaceDerivFunc(g, o);
  setThetaOverlap(p, g, o);
  if (o->reservoir_inlet) {
    arr_min_into(p->phi, p->phi, p->phi_extra, n);
    arr_max_into(p->phi, p->mask, p->phi, n);
  }
  getMainInd_new(o, p, g);
  int var = (o->theta > 0) || o->use_var_theta;
  while (drain ? (a0 < amax) : (a0 > amin)) {
    printf("\nStep %d: a = %f\n", step, a0);
    if (fp_out) fprintf(fp_out, "\nStep %d: a = %f\n", step, a0);
    if (var) {
      setvarcurvadv3d_(p->mask, p->mask_x, p->mask_y, p->mask_z, p->curvature_coeff,
                       p->external_velocity_x, p->external_velocity_y, p->external_velocity_z,
                       &o->b_max_over_dx, &o->max_U_over_dx, &o->b, GBD(g), FBD(g), &g->dx[0]);
    } else {
      double ix = 1 / g->dx[0], iy = 1 / g->dx[1], iz = 1 / g->dx[2];
      o->b_max_over_dx = 2 * o->b * (ix * ix + iy * iy + iz * iz);
      o->max_U_over_dx = 0;
    }
    if (!drain) o->conserve_imbibe = 1;
    if (var)
      setvarnorm3d_(p->mask, p->mask_x, p->mask_y, p->mask_z, p->normal_velocity, &a0, &o->theta,
                    GBD(g), FBD(g), &g->dx[0]);
    if (o->check_connectivity) trapComponents_mask(p, g, o);
    double t_step = var ? constCurvModel3d(o, p, g, fp_out) : constCurvModel3dNoVar(o, p, g, fp_out, a0);
    if (t_step == -1) break;
    if (drain) a0 += da; else a0 -= da;
    if (o->reservoir_inlet) arr_min_into(p->phi, p->phi, p->phi_extra, n);
    arr_max_into(p->phi, p->mask, p->phi, n);
    snprintf(fname, sizeof fname, "data_step_%d", step);
    step += 1;
    writeDataArrayQSS(p->phi, g, fname, GZIP);
  }
}

void drain_model3d(Options *o, QSS_DataArrays *p, Grid *g, FILE *fp_out) { ladder(1, o, p, g, fp_out); }
void imbibe_model3d(Options *o, QSS_DataArrays *p, Grid *g, FILE *fp_out) { ladder(0, o, p, g, fp_out); }

/* ------------------------------------------------------------------ */
/* test hooks                                                          */
/* CPU baseline: runs `steps` inner steps of the model on the current arrays
   and returns the wall time in seconds */
double oracle_time_inner_steps(Options *o, QSS_DataArrays *p, Grid *g, int var, double a, int steps)
{
  double dt_sub = 0, cur = -1;
  double t0 = omp_get_wtime();
  inner_loop(var, o, p, g, NULL, a, &dt_sub, &cur, steps);
  return omp_get_wtime() - t0;
}

void oracle_set_threads(int t) { omp_set_num_threads(t); }
int oracle_get_max_threads(void) { return omp_get_max_threads(); }
