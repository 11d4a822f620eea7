// qss_host_io.cpp -- data model, options and file formats of the lsmpqs C API.
//
// Host-side code: struct allocation, the text option file, and the binary
// grid / data-array files.  The formats and the option keywords are those of
// the reference so that existing input decks and result files are
// interchangeable:
//   grid file        src/geometry/qss_grid.c:614-763 (field order of Grid)
//   data array file  src/utilities/qss_data_arrays.c:214-381 (int[3] dims + values)
//   option file      src/utilities/qss_options.c:120-491 (keyword by leading letters)
//   defaults         src/utilities/qss_options.c:42-117
//   compression      src/utilities/qss_file.c:13-64 (gzip/bzip2 executables)
#include <cctype>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <initializer_list>
#include <string>

#include "../../include/lsmpqs_gpu.h"
#include "../../include/lsmpqs_types.h"
#include "qss_fortran_abi.h"

// qss_gzip.cpp: gzip file of head + data deflated on all host cores
bool qss_gzip_write(const char* path, const void* head, size_t head_len, const void* data, size_t len);

extern "C" {
void qssgpu_release(QSS_DataArrays* p);
void signedLinearExtrapolationBCqss(double* phi, Grid* g, int idx);
}

namespace {

const int kGhostCells[4] = {2, 3, 5, 4};  // LOW, MEDIUM, HIGH, VERY_HIGH

double* const kDummy = (double*)(-1);

void set_index_space_limits(QSSLIB_SPATIAL_DERIVATIVE_ACCURACY_TYPE acc, Grid* g) {
  const int n0 = g->grid_dims_ghostbox[0], n1 = g->grid_dims_ghostbox[1], n2 = g->grid_dims_ghostbox[2];
  g->mark_gb = 120;
  g->mark_D1 = 119;
  g->mark_D2 = 118;
  g->mark_D3 = 117;
  g->num_nb_levels = kGhostCells[acc];
  g->mark_fb = (unsigned char)(g->mark_gb - g->num_nb_levels);
  if (acc > MEDIUM) {
    g->beta = 3 * g->dx[0];
    g->gamma = 6 * g->dx[0];
  } else {
    g->beta = 2 * g->dx[0];
    g->gamma = 4 * g->dx[0];
  }
  g->ilo_gb = 0; g->ihi_gb = n0 - 1; g->jlo_gb = 0; g->jhi_gb = n1 - 1; g->klo_gb = 0; g->khi_gb = n2 - 1;
  g->ilo_D1_fb = 1; g->ihi_D1_fb = n0 - 2; g->jlo_D1_fb = 1; g->jhi_D1_fb = n1 - 2; g->klo_D1_fb = 1; g->khi_D1_fb = n2 - 2;
  g->ilo_D2_fb = 2; g->ihi_D2_fb = n0 - 3; g->jlo_D2_fb = 2; g->jhi_D2_fb = n1 - 3; g->klo_D2_fb = 2; g->khi_D2_fb = n2 - 3;
  g->ilo_D3_fb = 3; g->ihi_D3_fb = n0 - 4; g->jlo_D3_fb = 3; g->jhi_D3_fb = n1 - 4; g->klo_D3_fb = 3; g->khi_D3_fb = n2 - 4;
  // common fill box of the plus and minus one-sided stencils of each scheme
  int lo[3], hi[3];
  const int d1lo[3] = {g->ilo_D1_fb, g->jlo_D1_fb, g->klo_D1_fb}, d1hi[3] = {g->ihi_D1_fb, g->jhi_D1_fb, g->khi_D1_fb};
  const int d2lo[3] = {g->ilo_D2_fb, g->jlo_D2_fb, g->klo_D2_fb}, d2hi[3] = {g->ihi_D2_fb, g->jhi_D2_fb, g->khi_D2_fb};
  const int d3lo[3] = {g->ilo_D3_fb, g->jlo_D3_fb, g->klo_D3_fb}, d3hi[3] = {g->ihi_D3_fb, g->jhi_D3_fb, g->khi_D3_fb};
  for (int a = 0; a < 3; a++) {
    switch (acc) {
      case LOW: lo[a] = d1lo[a]; hi[a] = d1hi[a] - 1; break;
      case HIGH: lo[a] = d3lo[a] + 1; hi[a] = d3hi[a] - 2; break;
      case VERY_HIGH: lo[a] = d1lo[a] + 2; hi[a] = d1hi[a] - 3; break;
      default: lo[a] = d2lo[a] + 1; hi[a] = d2hi[a] - 1; break;
    }
  }
  g->ilo_fb = lo[0]; g->ihi_fb = hi[0]; g->jlo_fb = lo[1]; g->jhi_fb = hi[1]; g->klo_fb = lo[2]; g->khi_fb = hi[2];
}

void flatten_2d(Grid* g) {
  if (g->num_dims == 2) {
    g->x_lo[2] = g->x_hi[2] = g->x_lo_ghostbox[2] = g->x_hi_ghostbox[2] = 0;
    g->grid_dims[2] = g->grid_dims_ghostbox[2] = 1;
    g->dx[2] = 0;
  }
}

// `prog 'name'`: the name in single quotes (each ' as '\''), so that names
// with spaces or shell metacharacters reach the program as one argument
void run_on_file(const char* prog, const char* name) {
  std::string cmd = prog;
  cmd += " '";
  for (const char* c = name; *c; c++) {
    if (*c == '\'') cmd += "'\\''";
    else cmd += *c;
  }
  cmd += "'";
  if (system(cmd.c_str())) {
  }
}

int valid_dims(int d) {
  if (d == 2 || d == 3) return d;
  fprintf(stderr, "\nInvalid number of dimensions (%d).  Using to default value of 2.\n", d);
  return 2;
}

}  // namespace

extern "C" {

// ---------------------------------------------------------------- files
// As the reference: a name containing ".gz" (else ".bz2") is decompressed in
// place by the program and the base name is the name less its last 3 (4)
// characters.  The base is allocated to fit (the reference's fixed 256 bytes
// overflow on longer paths); free() it.
void checkUnzipFile(char* file_name, int* pzip_status, char** pfile_base) {
  const size_t len = strlen(file_name);
  char* base = (char*)malloc(len + 1);
  int zs = NO_ZIP;
  size_t keep = len;
  if (strstr(file_name, ".gz")) {
    zs = GZIP;
    run_on_file("gunzip -f", file_name);
    keep = len - 3;
  } else if (strstr(file_name, ".bz2")) {
    zs = BZIP2;
    run_on_file("bunzip2 -f", file_name);
    keep = len - 4;
  }
  memcpy(base, file_name, keep);
  base[keep] = 0;
  *pzip_status = zs;
  *pfile_base = base;
}

void zipFile(char* file_base, int zip_status) {
  if (zip_status == GZIP) run_on_file("gzip -f", file_base);
  else if (zip_status == BZIP2) run_on_file("bzip2 -f", file_base);
}

// ---------------------------------------------------------------- grid
Grid* allocateGrid(void) { return (Grid*)calloc(1, sizeof(Grid)); }

Grid* createGridSetDx(int num_dims, QSSLIB_REAL dx, QSSLIB_REAL* x_lo, QSSLIB_REAL* x_hi,
                      QSSLIB_SPATIAL_DERIVATIVE_ACCURACY_TYPE accuracy) {
  const int ng = kGhostCells[accuracy];
  Grid* g = allocateGrid();
  g->num_dims = valid_dims(num_dims);
  g->num_gridpts = 1;
  for (int i = 0; i < g->num_dims; i++) {
    g->dx[i] = dx;
    g->grid_dims[i] = (int)rint((x_hi[i] - x_lo[i]) / dx);
    g->x_lo[i] = x_lo[i];
    g->x_hi[i] = x_lo[i] + g->grid_dims[i] * dx;
    g->grid_dims_ghostbox[i] = g->grid_dims[i] + 2 * ng;
    g->x_lo_ghostbox[i] = g->x_lo[i] - ng * g->dx[i];
    g->x_hi_ghostbox[i] = g->x_hi[i] + ng * g->dx[i];
    g->num_gridpts *= g->grid_dims_ghostbox[i];
  }
  flatten_2d(g);
  set_index_space_limits(accuracy, g);
  return g;
}

Grid* createGridSetDxDyDz(int num_dims, QSSLIB_REAL dx, QSSLIB_REAL dy, QSSLIB_REAL dz, QSSLIB_REAL* x_lo,
                          QSSLIB_REAL* x_hi, QSSLIB_SPATIAL_DERIVATIVE_ACCURACY_TYPE accuracy) {
  const int ng = kGhostCells[accuracy];
  Grid* g = allocateGrid();
  g->num_dims = valid_dims(num_dims);
  g->num_gridpts = 1;
  g->dx[0] = dx;
  g->dx[1] = dy;
  g->dx[2] = dz;
  for (int i = 0; i < g->num_dims; i++) {
    g->grid_dims[i] = (int)rint((x_hi[i] - x_lo[i]) / g->dx[i]);
    g->x_lo[i] = x_lo[i];
    g->x_hi[i] = x_lo[i] + g->grid_dims[i] * g->dx[i];
    g->grid_dims_ghostbox[i] = g->grid_dims[i] + 2 * ng;
    g->x_lo_ghostbox[i] = g->x_lo[i] - ng * g->dx[i];
    g->x_hi_ghostbox[i] = g->x_hi[i] + ng * g->dx[i];
    g->num_gridpts *= g->grid_dims_ghostbox[i];
  }
  flatten_2d(g);
  set_index_space_limits(accuracy, g);
  return g;
}

Grid* createGridSetGridDims(int num_dims, int* grid_dims, QSSLIB_REAL* x_lo, QSSLIB_REAL* x_hi,
                            QSSLIB_SPATIAL_DERIVATIVE_ACCURACY_TYPE accuracy) {
  const int ng = kGhostCells[accuracy];
  Grid* g = allocateGrid();
  g->num_dims = valid_dims(num_dims);
  g->num_gridpts = 1;
  for (int i = 0; i < g->num_dims; i++) {
    g->grid_dims[i] = grid_dims[i];
    g->x_hi[i] = x_hi[i];
    g->x_lo[i] = x_lo[i];
    g->dx[i] = (g->x_hi[i] - g->x_lo[i]) / g->grid_dims[i];
    g->grid_dims_ghostbox[i] = g->grid_dims[i] + 2 * ng;
    g->x_lo_ghostbox[i] = g->x_lo[i] - ng * g->dx[i];
    g->x_hi_ghostbox[i] = g->x_hi[i] + ng * g->dx[i];
    g->num_gridpts *= g->grid_dims_ghostbox[i];
  }
  flatten_2d(g);
  set_index_space_limits(accuracy, g);
  return g;
}

Grid* copyGrid(Grid* grid) {
  Grid* g = allocateGrid();
  *g = *grid;
  return g;
}

void destroyGrid(Grid* grid) { free(grid); }

void printGrid(Grid* g, FILE* fp) {
  fprintf(fp, "Number of dimensions: %d\n", g->num_dims);
  if (g->num_dims == 2) {
    fprintf(fp, "Geometric limits (without ghostcells): [%g,%g] x [%g,%g]\n", g->x_lo[0], g->x_hi[0], g->x_lo[1],
            g->x_hi[1]);
    fprintf(fp, "Geometric limits (with ghostcells): [%g,%g] x [%g,%g]\n", g->x_lo_ghostbox[0], g->x_hi_ghostbox[0],
            g->x_lo_ghostbox[1], g->x_hi_ghostbox[1]);
    fprintf(fp, "Grid dimensions (without ghostcells): %d x %d\n", g->grid_dims[0], g->grid_dims[1]);
    fprintf(fp, "Grid dimensions (with ghostcells): %d x %d\n", g->grid_dims_ghostbox[0], g->grid_dims_ghostbox[1]);
    fprintf(fp, "Grid spacing: dx = %g, dy = %g\n", g->dx[0], g->dx[1]);
  } else {
    fprintf(fp, "Geometric limits (without ghostcells): [%g,%g] x [%g,%g] x [%g,%g]\n", g->x_lo[0], g->x_hi[0],
            g->x_lo[1], g->x_hi[1], g->x_lo[2], g->x_hi[2]);
    fprintf(fp, "Geometric limits (with ghostcells): [%g,%g] x [%g,%g] x [%g,%g]\n", g->x_lo_ghostbox[0],
            g->x_hi_ghostbox[0], g->x_lo_ghostbox[1], g->x_hi_ghostbox[1], g->x_lo_ghostbox[2], g->x_hi_ghostbox[2]);
    fprintf(fp, "Grid dimensions (without ghostcells): %d x %d x %d\n", g->grid_dims[0], g->grid_dims[1],
            g->grid_dims[2]);
    fprintf(fp, "Grid dimensions (with ghostcells): %d x %d x %d\n", g->grid_dims_ghostbox[0],
            g->grid_dims_ghostbox[1], g->grid_dims_ghostbox[2]);
    fprintf(fp, "Grid spacing: dx = %g, dy = %g, dz = %g\n", g->dx[0], g->dx[1], g->dx[2]);
  }
  fprintf(fp, "Total number of grid points: %d\n", g->num_gridpts);
  fprintf(fp, "Ghost box: [%d,%d] x [%d,%d] x [%d,%d]\n", g->ilo_gb, g->ihi_gb, g->jlo_gb, g->jhi_gb, g->klo_gb,
          g->khi_gb);
  fprintf(fp, "Fill box: [%d,%d] x [%d,%d] x [%d,%d]\n", g->ilo_fb, g->ihi_fb, g->jlo_fb, g->jhi_fb, g->klo_fb,
          g->khi_fb);
}

void writeGridToAsciiFile(Grid* grid, char* file_name, int zip_status) {
  FILE* fp = fopen(file_name, "w");
  if (!fp) return;
  printGrid(grid, fp);
  fclose(fp);
  zipFile(file_name, zip_status);
}

// Grid file: the Grid fields in declaration order, each written on its own
// (ints, REALs, unsigned chars), no padding.
#define GRID_FIELDS(X)                                                                                      \
  X(&g->num_dims, sizeof(int), 1) X(g->x_lo, sizeof(double), 3) X(g->x_hi, sizeof(double), 3)              \
  X(g->x_lo_ghostbox, sizeof(double), 3) X(g->x_hi_ghostbox, sizeof(double), 3)                            \
  X(g->grid_dims, sizeof(int), 3) X(g->grid_dims_ghostbox, sizeof(int), 3) X(g->dx, sizeof(double), 3)      \
  X(&g->num_gridpts, sizeof(int), 1) X(&g->ilo_gb, sizeof(int), 6) X(&g->ilo_fb, sizeof(int), 6)            \
  X(&g->ilo_D1_fb, sizeof(int), 6) X(&g->ilo_D2_fb, sizeof(int), 6) X(&g->ilo_D3_fb, sizeof(int), 6)        \
  X(&g->num_nb_levels, sizeof(int), 1) X(&g->mark_gb, 1, 5) X(&g->beta, sizeof(double), 1)                  \
  X(&g->gamma, sizeof(double), 1)

void writeGridToBinaryFile(Grid* grid, char* file_name, int zip_status) {
  Grid* g = grid;
  FILE* fp = fopen(file_name, "w");
  if (!fp) {
    printf("\nCould not open file %s", file_name);
    return;
  }
#define W(ptr, sz, cnt) fwrite(ptr, sz, cnt, fp);
  GRID_FIELDS(W)
#undef W
  fclose(fp);
  zipFile(file_name, zip_status);
}

Grid* readGridFromBinaryFile(char* file_name) {
  char* base;
  int zs;
  checkUnzipFile(file_name, &zs, &base);
  Grid* g = allocateGrid();
  FILE* fp = fopen(base, "r");
  if (fp) {
#define R(ptr, sz, cnt) \
  if (fread(ptr, sz, cnt, fp) != (size_t)(cnt)) {}
    GRID_FIELDS(R)
#undef R
    fclose(fp);
    zipFile(base, zs);
  } else {
    printf("\nCould not open file %s", base);
  }
  free(base);
  return g;
}

// ---------------------------------------------------------------- 2-D shapes
// The 2-D initial shapes some reference tools call (createInitFromMask's
// 2-D branch); host loops over the 2-D ghost box, as the reference
// (src/geometry/qss_initialization2d.c:127-178): the larger of the signed
// distances to the circles, each negated when its inside_flag is >= 0.
void createIntersectionOfCircles(QSSLIB_REAL* phi, int num_circles, QSSLIB_REAL* center_x, QSSLIB_REAL* center_y,
                                 QSSLIB_REAL* radius, int* inside_flag, Grid* grid) {
  const int nx = grid->grid_dims_ghostbox[0], ny = grid->grid_dims_ghostbox[1];
  for (int j = 0; j < ny; j++)
    for (int i = 0; i < nx; i++) {
      const double x = grid->x_lo_ghostbox[0] + grid->dx[0] * i;
      const double y = grid->x_lo_ghostbox[1] + grid->dx[1] * j;
      double best = -FLT_MAX;
      for (int c = 0; c < num_circles; c++) {
        const double ex = x - center_x[c], ey = y - center_y[c];
        double d = sqrt(ex * ex + ey * ey) - radius[c];
        if (inside_flag[c] >= 0) d = -d;
        if (d > best) best = d;
      }
      phi[i + j * nx] = best;
    }
}

void createCircle(QSSLIB_REAL* phi, QSSLIB_REAL center_x, QSSLIB_REAL center_y, QSSLIB_REAL radius, int inside_flag,
                  Grid* grid) {
  createIntersectionOfCircles(phi, 1, &center_x, &center_y, &radius, &inside_flag, grid);
}

// ---------------------------------------------------------------- data arrays
QSS_DataArrays* allocateQSSDataArrays(void) {
  QSS_DataArrays* p = (QSS_DataArrays*)malloc(sizeof(QSS_DataArrays));
  double** r[] = {&p->phi, &p->phi_next, &p->phi_extra, &p->phi_prev, &p->mask, &p->lse_rhs,
                  &p->normal_velocity, &p->curvature_coeff, &p->external_velocity_x, &p->external_velocity_y,
                  &p->external_velocity_z, &p->mask_x, &p->mask_y, &p->mask_z, &p->scratch1, &p->scratch2,
                  &p->mask_w, &p->mask_nw, &p->mask_disconn_init, &p->theta, &p->overlap};
  for (double** q : r) *q = kDummy;
  p->connectivity = (int*)(-1);
  p->phi_bin = (unsigned char*)(-1);
  return p;
}

void allocateMemoryForQSSDataArrays(QSS_DataArrays* p, Grid* g) {
  const size_t n = (size_t)g->num_gridpts;
  for (double** q : {&p->phi, &p->phi_next, &p->phi_extra, &p->phi_prev, &p->mask})
    if (*q == kDummy) *q = (double*)calloc(n, sizeof(double));
  double** plain[] = {&p->lse_rhs, &p->normal_velocity, &p->curvature_coeff, &p->external_velocity_x,
                      &p->external_velocity_y, &p->external_velocity_z, &p->mask_x, &p->mask_y, &p->mask_z,
                      &p->scratch1, &p->scratch2, &p->theta, &p->overlap, &p->mask_w, &p->mask_nw,
                      &p->mask_disconn_init};
  for (double** q : plain) {
    const bool z_only = (q == &p->external_velocity_z || q == &p->mask_z);
    if (z_only && g->num_dims != 3) {
      *q = nullptr;
      continue;
    }
    if (*q == kDummy) *q = (double*)malloc(n * sizeof(double));
  }
  if (p->connectivity == (int*)(-1)) p->connectivity = (int*)malloc(n * sizeof(int));
  if (p->phi_bin == (unsigned char*)(-1)) p->phi_bin = (unsigned char*)malloc(n);
}

void destroyQSSDataArrays(QSS_DataArrays* p) {
  if (!p) return;
  qssgpu_release(p);
  double* r[] = {p->phi, p->phi_next, p->phi_extra, p->phi_prev, p->mask, p->lse_rhs, p->normal_velocity,
                 p->curvature_coeff, p->external_velocity_x, p->external_velocity_y, p->external_velocity_z,
                 p->mask_x, p->mask_y, p->mask_z, p->scratch1, p->scratch2, p->mask_w, p->mask_nw,
                 p->mask_disconn_init, p->theta, p->overlap};
  for (double* q : r)
    if (q != kDummy) free(q);
  if (p->connectivity != (int*)(-1)) free(p->connectivity);
  if (p->phi_bin != (unsigned char*)(-1)) free(p->phi_bin);
  free(p);
}

static void write_array(const void* data, size_t elem, Grid* g, char* file_name, int zip_status, bool dims) {
  if (zip_status == GZIP) {
    // the final state of "write file_name, gzip -f file_name": file_name.gz
    // holds the bytes, file_name is gone (compressed on all host cores)
    char gz[600];
    snprintf(gz, sizeof gz, "%s.gz", file_name);
    if (qss_gzip_write(gz, g->grid_dims_ghostbox, dims ? 3 * sizeof(int) : 0, data,
                       elem * (size_t)g->num_gridpts)) {
      remove(file_name);
      return;
    }
  }
  FILE* fp = fopen(file_name, "w");
  if (!fp) {
    printf("\nCould not open file %s\n", file_name);
    return;
  }
  if (dims) fwrite(g->grid_dims_ghostbox, sizeof(int), 3, fp);
  fwrite(data, elem, (size_t)g->num_gridpts, fp);
  fclose(fp);
  zipFile(file_name, zip_status);
}

void writeDataArrayQSS(QSSLIB_REAL* data, Grid* grid, char* file_name, int zip_status) {
  write_array(data, sizeof(double), grid, file_name, zip_status, true);
}
void writeDataArrayRaw(QSSLIB_REAL* data, Grid* grid, char* file_name, int zip_status) {
  write_array(data, sizeof(double), grid, file_name, zip_status, false);
}
void writeDataArrayUchar(unsigned char* data, Grid* grid, char* file_name, int zip_status) {
  write_array(data, 1, grid, file_name, zip_status, true);
}
void writeDataArrayInt(int* data, Grid* grid, char* file_name, int zip_status) {
  write_array(data, sizeof(int), grid, file_name, zip_status, true);
}
void writeDataArrayUcharFB(unsigned char* data_fb, Grid* g, char* file_name, int zip_status) {
  const size_t nfb = (size_t)g->grid_dims[0] * g->grid_dims[1] * g->grid_dims[2];
  if (zip_status == GZIP) {
    char gz[600];
    snprintf(gz, sizeof gz, "%s.gz", file_name);
    if (qss_gzip_write(gz, nullptr, 0, data_fb, nfb)) {
      remove(file_name);
      return;
    }
  }
  FILE* fp = fopen(file_name, "w");
  if (!fp) return;
  fwrite(data_fb, 1, (size_t)g->grid_dims[0] * g->grid_dims[1] * g->grid_dims[2], fp);
  fclose(fp);
  zipFile(file_name, zip_status);
}

static void* read_array(int* dims, char* file_name, size_t elem) {
  char* base;
  int zs;
  void* data = nullptr;
  checkUnzipFile(file_name, &zs, &base);
  FILE* fp = fopen(base, "r");
  if (fp) {
    // a header that is missing or not three positive sizes reads as no array
    // (NULL) instead of sizing an allocation from it; a short payload leaves
    // the rest zero
    if (fread(dims, sizeof(int), 3, fp) == 3 && dims[0] > 0 && dims[1] > 0 && dims[2] > 0) {
      const size_t n = (size_t)dims[0] * dims[1] * dims[2];
      data = calloc(n, elem);
      if (data && fread(data, elem, n, fp) != n) {
        printf("\nFile %s is shorter than its header says", file_name);
      }
    } else {
      printf("\nFile %s has no valid array header", file_name);
    }
    fclose(fp);
    zipFile(base, zs);
  } else {
    printf("\nCould not open file %s", file_name);
  }
  free(base);
  return data;
}

QSSLIB_REAL* readDataArrayQSS(int* grid_dims_ghostbox, char* file_name) {
  return (QSSLIB_REAL*)read_array(grid_dims_ghostbox, file_name, sizeof(double));
}
int* readDataArrayInt(int* grid_dims_ghostbox, char* file_name) {
  return (int*)read_array(grid_dims_ghostbox, file_name, sizeof(int));
}

// ---------------------------------------------------------------- options
Options* allocateOptions(void) { return (Options*)calloc(1, sizeof(Options)); }

Options* createOptionsDefault(void) {
  Options* o = allocateOptions();
  snprintf(o->outfile, sizeof o->outfile, "out_file");
  snprintf(o->path, sizeof o->path, "./");
  o->dx = 0.04;
  o->tmax = 150.0;
  o->tplot = 0.5;
  snprintf(o->accuracy, sizeof o->accuracy, "medium");
  o->accuracy_id = MEDIUM;
  o->a = 0.15;
  o->b = 0.04;
  o->save_data = 1;
  o->do_reinit = 1;
  o->do_mask = 1;
  o->eps_stop = 0.014;
  o->narrow_band = 0;
  o->overlap = 0;
  o->init_step = 0;
  o->print_details = 1;
  o->tmax_r = 10 * o->dx;
  o->subcell_fix = 1;
  o->dc = 0.1;
  o->cmax = 1.0 / (o->dx / 2.0);
  o->amax = 10;
  o->amin = 0.05;
  o->vol_frac_max = 0.97;
  o->vol_frac_min = 0;
  o->mask_reinit = 1;
  o->stop_touch = 1;
  o->eps_coefficient = 1.5;
  o->extrapol_id = 0;
  o->extrapol_func = (qss_untyped_fn)signedLinearExtrapolationBCqss;
  o->space_deriv_func = (qss_untyped_fn)getrhs3d5th_;
  o->checkpoint = 0;
  o->reservoir_inlet = 1;
  o->theta = 0;
  o->C = 1;
  o->check_connectivity = 1;
  o->err_check_zone = 20 * o->dx;
  o->phi_w_ind = 0;
  o->phi_nw_ind = 0;
  o->use_var_theta = 0;
  o->order_space_accur = 3;
  o->order_time_accur = 3;
  o->use_satn_stop = 1;
  o->conserve_imbibe = 0;
  o->center_inlet = 0;
  return o;
}

static const char* const kAccuracyNames[4] = {"low", "medium", "high", "very_high"};

static int read_int(const char* s, int* out) { return sscanf(s, "%*s %d ", out) == 1; }
static int read_real(const char* s, double* out) { return sscanf(s, "%*s %lf ", out) == 1; }

// One "keyword value" per line; the keyword is recognised by its leading
// letters exactly as the reference parser does, so abbreviations and
// unknown words behave the same way.
Options* createOptionsFromInputFile(char* filename) {
  Options* o = createOptionsDefault();
  FILE* fp = fopen(filename, "r");
  if (!fp) {
    printf("\nCouldnt open file %s", filename);
    return o;
  }
  char line[100], word[100];
  // keywords are told apart by letters at fixed positions; past the end of
  // a short line those read as 0, never as a previous line's letters
  for (;;) {
    memset(line, 0, sizeof line);
    if (!fgets(line, 80, fp)) break;
    int n = 0;
    while (isspace((unsigned char)line[n])) n++;
    const char* s = line + n;
    const int c = tolower((unsigned char)s[0]);
    auto at = [&](int k) { return tolower((unsigned char)s[k]); };
    double r;
    int v;
    if (c == 'a') {
      if (at(1) == 'c') {
        if (sscanf(s, "accuracy %99s", word) == 1) {
          int found = 0;
          for (int i = 0; i < 4; i++)
            if (!strcmp(word, kAccuracyNames[i])) {
              found = 1;
              o->accuracy_id = (QSSLIB_SPATIAL_DERIVATIVE_ACCURACY_TYPE)i;
              snprintf(o->accuracy, sizeof o->accuracy, "%s", kAccuracyNames[i]);
            }
          if (!found) printf("\nAccuracy type %s not found, set to default.", word);
        }
      } else if (at(2) == 'a') {
        if (read_real(s, &r)) o->amax = r;
      } else if (at(2) == 'i') {
        if (read_real(s, &r)) o->amin = r;
      } else if (read_real(s, &r)) {
        o->a = r;
      }
    } else if (c == 'b') {
      if (read_real(s, &r)) o->b = r;
    } else if (c == 'c') {
      if (at(1) == 'm') {
        if (read_real(s, &r)) o->cmax = r;
      } else if (at(5) == 'p') {
        if (read_int(s, &v)) {
          if (v == 0 || v == 1) o->checkpoint = v;
          else printf("\nIncorrect checkpoint option %d, set to default.\n", v);
        }
      } else if (at(6) == 'c') {
        if (read_int(s, &v)) o->check_connectivity = v;
      } else if (at(1) == 'e') {
        if (read_int(s, &v)) o->center_inlet = v;
      }
    } else if (c == 'd') {
      if (at(1) == 'x') {
        if (read_real(s, &r)) o->dx = r;
      } else if (s[3] == 'r') {
        if (read_int(s, &v)) {
          if (v == 0 || v == 1) o->do_reinit = v;
          else printf("\nIncorrect do_reinit option %d, set to default.\n", v);
        }
      } else if (s[3] == 'm') {
        if (read_int(s, &v)) {
          if (v == 0 || v == 1) o->do_mask = v;
          else printf("\nIncorrect do_mask option %d, set to default.\n", v);
        }
      } else if (at(1) == 'c') {
        if (read_real(s, &r)) o->dc = r;
      }
    } else if (c == 'e') {
      if (at(1) == 'p' && at(4) == 'c') {
        if (read_real(s, &r)) {
          if (r > 0) o->eps_coefficient = r;
          else printf("\nIncorrect eps_coefficient option %g, set to default.\n", r);
        }
      } else if (at(1) == 'r' && at(10) == 'z') {
        if (read_real(s, &r)) o->err_check_zone = r;
      } else if (at(1) == 'p' && at(4) == 's') {
        if (read_real(s, &r)) o->eps_stop = r;
      } else if (at(1) == 'x' && at(2) == 't') {
        if (read_int(s, &v)) {
          if (v < 0 || v > 3) {
            printf("\nIncorrect extrapol_id option %d, set to default.\n", v);
            v = 0;
          }
          o->extrapol_id = v;
          o->extrapol_func = (qss_untyped_fn)signedLinearExtrapolationBCqss;
        }
      }
    } else if (c == 'i') {
      if (read_int(s, &v)) o->init_step = v;
    } else if (c == 'm' && s[1] == 'a') {
      if (read_int(s, &v)) {
        if (v == 0 || v == 1) o->mask_reinit = v;
        else printf("\nIncorrect mask_reinit option %d, set to default.\n", v);
      }
    } else if (c == 'n') {
      if (read_int(s, &v)) {
        if (v == 0 || v == 1) o->narrow_band = v;
        else printf("\nIncorrect narrow_band option %d, set to default.\n", v);
      }
    } else if (c == 'o' && s[1] == 'u') {
      if (sscanf(s, "outfile %99s", word) == 1) {
        snprintf(o->outfile, sizeof o->outfile, "%s", word);
        const char* slash = strrchr(o->outfile, '/');
        if (slash) {
          size_t L = (size_t)(slash - o->outfile) + 1;
          memcpy(o->path, o->outfile, L);
          o->path[L] = 0;
        } else {
          snprintf(o->path, sizeof o->path, "./");
        }
      }
    } else if (c == 'o' && s[1] == 'v') {
      if (read_real(s, &r)) o->overlap = r;
    } else if (c == 'r' && s[1] == 'e') {
      if (read_int(s, &v)) {
        if (v == 0 || v == 1) o->reservoir_inlet = v;
        else {
          printf("\nIncorrect reservoir_inlet option %d, set to default.\n", v);
          o->reservoir_inlet = 0;
        }
      }
    } else if (c == 's' && at(1) == 'a') {
      if (read_int(s, &v)) {
        if (v == 0 || v == 1) o->save_data = v;
        else printf("\nIncorrect save_data option %d, set to default.\n", v);
      }
    } else if (c == 's' && at(5) == 't') {
      if (read_int(s, &v)) {
        if (v == 0 || v == 1) o->stop_touch = v;
        else printf("\nIncorrect stop_touch option %d, set to default.\n", v);
      }
    } else if (c == 's' && at(1) == 'u') {
      if (read_int(s, &v)) {
        if (v == 0 || v == 1) o->subcell_fix = v;
        else printf("\nIncorrect subcell_fix option %d, set to default.\n", v);
      }
    } else if (c == 's' && at(1) == 'p') {
      if (read_int(s, &v)) o->order_space_accur = v;
    } else if (c == 't') {
      if (at(1) == 'm') {
        if (read_real(s, &r)) o->tmax = r;
      } else if (at(1) == 'p') {
        if (read_real(s, &r)) o->tplot = r;
      } else if (at(1) == 'i') {
        if (read_int(s, &v)) o->order_time_accur = v;
      } else if (at(1) == 'h') {
        if (read_real(s, &r)) o->theta = r * 3.14159 / 180;  // input in degrees
      }
    } else if (c == 'v') {
      if (at(9) == 'm' && at(10) == 'a') {
        if (read_real(s, &r)) o->vol_frac_max = r;
      } else if (at(9) == 'm' && at(10) == 'i') {
        if (read_real(s, &r)) o->vol_frac_min = r;
      }
    } else if (c == 'u') {
      if (at(4) == 'v') {
        if (read_int(s, &v)) o->use_var_theta = v;
      } else if (at(4) == 's') {
        if (read_int(s, &v)) o->use_satn_stop = v;
      }
    }
    if (c == 'p') {
      if (read_int(s, &v)) {
        if (v == 0 || v == 1) o->print_details = v;
        else {
          printf("\nIncorrect print_details option %d, set to default.\n", v);
          o->print_details = 1;
        }
      }
    }
  }
  fclose(fp);
  return o;
}

void printOptions(Options* o, FILE* fp) {
  const char* rule = "  -----------------------------------------------------------------------------\n";
  fprintf(fp, "%s  Geometry options: \n%s", rule, rule);
  fprintf(fp, "  dx                   %8g  [ grid spacing ]\n", o->dx);
  fprintf(fp, "  mask_reinit          %8d  [ reinitialize mask or not ]\n", o->mask_reinit);
  fprintf(fp, "  reservoir_inlet      %8d  [ impose reservoir at inlet or not ]\n", o->reservoir_inlet);
  fprintf(fp, "%s  Running options: \n%s", rule, rule);
  fprintf(fp, "  a                    %8g  [ Initial normal velocity (or cap pressure) ]\n", o->a);
  fprintf(fp, "  b                    %8g  [ Curvature coefficient   ]\n", o->b);
  fprintf(fp, "  dc                   %8g  [ curvature increment/decrement ]\n", o->dc);
  fprintf(fp, "   space accuracy       %8d [ accuracy options: low, medium, high, very_high ]\n", o->order_space_accur);
  fprintf(fp, "   time accuracy        %8d  [ accuracy options: low, medium, high, very_high ]\n", o->order_time_accur);
  fprintf(fp, "  theta                %8g  [ contact angle, in radians ]\n", o->theta);
  fprintf(fp, "  tplot                %8g  [ intervals for reinit, error ]\n", o->tplot);
  fprintf(fp, "  init_step            %8d  [ Initial step (if restarting a stopped simulation) ]\n", o->init_step);
  fprintf(fp, "  overlap              %8g  [ overlap between pore space and mask allowed ]\n", o->overlap);
  fprintf(fp, "  eps_coefficient      %8g  [ numerical width of smearing for Heaviside ]\n", o->eps_coefficient);
  fprintf(fp, "  check_connectivity   %8d  [ check for trapped components or not ]\n", o->check_connectivity);
  fprintf(fp, "  checkpoint           %8d  [ output checkpoint data or not ]\n", o->checkpoint);
  fprintf(fp, "  err_check_zone       %8g  [ distance from zero ls to check error ]\n", o->err_check_zone);
  fprintf(fp, "  do_reinit            %8d  [ reinitilize periodically (1) or not (0)]\n", o->do_reinit);
  fprintf(fp, "  do_mask              %8d  [ impose mask (1) or not (0)]\n", o->do_mask);
  fprintf(fp, "  print_details        %8d  [ print details (1) or not (0)   ]\n", o->print_details);
  fprintf(fp, "  center_inlet         %8d  [ Inlet at center or not \n", o->center_inlet);
  fprintf(fp, "%s  Stopping options: \n%s", rule, rule);
  fprintf(fp, "  tmax                 %8g  [ max running time allowed ]\n", o->tmax);
  fprintf(fp, "  eps_stop             %8g  [ criteria for stopping ]\n", o->eps_stop);
  fprintf(fp, "  tmax_reinit          %8g  [ max reinit time allowed ]\n", o->tmax_r);
  fprintf(fp, "  cmax                 %8g  [ maximum curvature ]\n", o->cmax);
  fprintf(fp, "  amax                 %8g  [ maximum a, for drainage ]\n", o->amax);
  fprintf(fp, "  amin                 %8g  [ minimum a, for imbibition ]\n", o->amin);
  fprintf(fp, "  vol_frac_max         %8g  [ maximum nw fraction allowed ]\n", o->vol_frac_max);
  fprintf(fp, "  stop_touch           %8d  [ stop the simulation when opp. bdry. is touched ]\n", o->stop_touch);
  fprintf(fp, "  save_data            %8d  [ save data (1) or not (0)       ]\n", o->save_data);
  fprintf(fp, "  outfile              %8s  [ output file name ]\n", o->outfile);
}

void destroyOptions(Options* o) { free(o); }

}  // extern "C"
