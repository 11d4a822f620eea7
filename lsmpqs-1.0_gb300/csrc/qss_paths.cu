// qss_paths.cu -- curvature ladders and the remaining path-level C entry points.
//
//   drain_model3d / imbibe_model3d  src/level_set_evolution/drain_model3d.c:49-165,
//                                   imbibe_model3d.c:49-161
//   drainTop / imbibeTop            src/level_set_evolution/drain_top.c:31-137, imbibe_top.c
//   trapComponents_mask             src/connectivity/trapComponents.c:156-375
//   findConnectivity3d, getMainInd_new  src/connectivity/connectivity.c:148-296
//   reinitializeSubcellFix3d        src/reinitialization/reinitialize_top.c:297-377
//   setSpaceDerivFunc, setThetaOverlap, signedLinearExtrapolationBCqss,
//   initializeDisconnectedMasks, createReservoirInlet3d
//                                   src/utilities/qss_general_util.c:82-207, 422-706, 711-728, 813-833
#include <cmath>
#include <cstring>
#include <initializer_list>
#include <memory>
#include <ctime>
#include <algorithm>
#include <atomic>
#include <chrono>
#include <string>
#include <thread>
#include <vector>

#include "qss_fortran_abi.h"
#include "qss_state.h"

extern "C" {
void writeDataArrayQSS(double* data, Grid* grid, char* file_name, int zip_status);
double* readDataArrayQSS(int* grid_dims_ghostbox, char* file_name);
Grid* readGridFromBinaryFile(char* file_name);
QSS_DataArrays* allocateQSSDataArrays(void);
void allocateMemoryForQSSDataArrays(QSS_DataArrays* p, Grid* g);
void destroyQSSDataArrays(QSS_DataArrays* p);
void destroyGrid(Grid* g);
void printOptions(Options* o, FILE* fp);
void printGrid(Grid* g, FILE* fp);
void setSpaceDerivFunc(Grid* g, Options* o);
void setThetaOverlap(QSS_DataArrays* p, Grid* g, Options* o);
void getMainInd_new(Options* o, QSS_DataArrays* p, Grid* g);
int qssgpu_last_error(void);
const char* qssgpu_error_string(void);
void qssgpu_clear_error(void);
}

namespace qss {
void path_reinit(DevVolume& v, double*& data, const Grid* g, const Options* o);
void path_trap(DevVolume& v, const Grid* g, const Options* o);
double path_const_curv(DevVolume& v, bool var, Options* o, QSS_DataArrays* p, Grid* g, FILE* fp, double a);
double path_inner_loop(DevVolume& v, Options* o, Grid* g, double a, int max_steps);
int path_kernels_per_step(DevVolume& v, const Options* o);

namespace {

void dev_sphere(DevVolume& v, double* dst, const Grid* g, double cx, double cy, double cz, double r, int inside) {
  launch_sphere(v.stream, v.box, dst, g->x_lo_ghostbox, g->dx, cx, cy, cz, r, inside);
}

// initializeDisconnectedMasks (3-D): a sphere of radius 2*(x_hi-x_lo) around
// the domain centre, negative inside
void dev_init_disconnected(DevVolume& v, double* dst, const Grid* g) {
  double cz = 0.5 * (g->x_lo[2] + g->x_hi[2]);
  double cy = 0.5 * (g->x_lo[1] + g->x_hi[1]);
  double cx = 0.5 * (g->x_lo[0] + g->x_hi[0]);
  double r = 2 * (g->x_hi[0] - g->x_lo[0]);
  dev_sphere(v, dst, g, cx, cy, cz, r, -1);
}

// createReservoirInlet3d: box 3 cells thick on the x-lo side of the ghost box
void dev_reservoir(DevVolume& v, const Grid* g) {
  const double corner[3] = {g->x_lo_ghostbox[0], g->x_lo_ghostbox[1], g->x_lo_ghostbox[2]};
  const double side[3] = {3 * g->dx[0], g->x_hi_ghostbox[1] - g->x_lo_ghostbox[1],
                          g->x_hi_ghostbox[2] - g->x_lo_ghostbox[2]};
  launch_box(v.stream, v.box, v.phi_extra, g->x_lo_ghostbox, g->dx, corner, side, -1);
}

// The ladder's per-step files, written while the device runs the next
// curvature step: each step's phi is copied into one of two host buffers
// and a host thread writes and compresses the file (the reference writes
// synchronously, drain_model3d.c:146-153).  At most two files are in
// flight; all are complete when the ladder returns, with the same contents.
class StepWriter {
 public:
  ~StepWriter() { join(); }
  void write(DevVolume& v, const Grid* g, const char* name) {
    const int b = next_;
    next_ ^= 1;
    if (th_[b].joinable()) th_[b].join();
    if (!buf_[b]) buf_[b].reset(new double[(size_t)v.n]);
    QSS_CK(cudaMemcpyAsync(buf_[b].get(), v.phi, (size_t)v.n * sizeof(double), cudaMemcpyDeviceToHost, v.stream));
    QSS_CK(cudaStreamSynchronize(v.stream));
    Grid gc = *g;
    std::string nm(name);
    double* data = buf_[b].get();
    th_[b] = std::thread([gc, nm, data]() mutable { writeDataArrayQSS(data, &gc, &nm[0], GZIP); });
  }
  void join() {
    for (auto& t : th_)
      if (t.joinable()) t.join();
  }

 private:
  std::unique_ptr<double[]> buf_[2];
  std::thread th_[2];
  int next_ = 0;
};

// The per-step files are named prefix + "data_step_<k>" (the reference's
// names for prefix ""); a null prefix writes none.
void dev_ladder(bool drain, Options* o, QSS_DataArrays* p, Grid* g, FILE* fp_out, bool outermost,
                const char* prefix) {
  DevVolume& v = volume_for(p, g);
  if (outermost) {
    v.inner_steps = v.outer_iters = 0;
    reset_phases(v);
  }
  PhaseTimer total(v, PH_TOTAL);
  if (outermost) {
    upload(v, p, H_PHI);
    upload(v, p, H_MASK);
    if (o->theta > 0 || o->use_var_theta)
      start_prefault(v, p, {H_PHI_NEXT, H_PHI_PREV, H_PHI_EXTRA, H_MASK_W, H_MASK_NW, H_MASK_DISCONN, H_MASK_X,
                            H_MASK_Y, H_MASK_Z, H_CONN, H_BIN, H_VEL_N, H_BCOEF, H_VX, H_VY, H_VZ});
    else
      start_prefault(v, p, {H_PHI_NEXT, H_PHI_PREV, H_PHI_EXTRA, H_MASK_W, H_MASK_NW, H_MASK_DISCONN, H_MASK_X,
                            H_MASK_Y, H_MASK_Z, H_CONN, H_BIN});
  }
  PrefaultGuard pg{v};
  StepWriter files;
  char fname[256];
  int dims[3];
  double a0 = o->a;
  const double da = o->b * o->dc;
  int step = o->init_step + 1;
  const int64_t n = v.n;

  dev_init_disconnected(v, v.mask_w, g);
  dev_init_disconnected(v, v.mask_nw, g);
  QSS_CK(cudaMemcpyAsync(v.mask_disconn, v.mask_nw, n * sizeof(double), cudaMemcpyDeviceToDevice, v.stream));
  dev_reservoir(v, g);
  for (HostArray h : {H_MASK_W, H_MASK_NW, H_MASK_DISCONN, H_PHI_EXTRA}) v.dirty[h] = true;
  const double amax = o->amax, amin = o->amin;
  if (drain && o->mask_reinit) {
    path_reinit(v, v.mask, g, o);
    v.dirty[H_MASK] = true;
  }
  launch_central_grad(v.stream, v.box, v.mask, v.mask_x, v.mask_y, v.mask_z, g->dx[0], g->dx[1], g->dx[2]);
  v.dirty[H_MASK_X] = v.dirty[H_MASK_Y] = v.dirty[H_MASK_Z] = true;
  if (o->use_var_theta) {
    snprintf(fname, sizeof fname, "theta.gz");
    p->theta = readDataArrayQSS(dims, fname);
  }
  setSpaceDerivFunc(g, o);
  setThetaOverlap(p, g, o);
  if (o->reservoir_inlet) {
    launch_min_into(v.stream, n, v.phi, v.phi, v.phi_extra);
    launch_max_into(v.stream, n, v.phi, v.mask, v.phi);
    v.dirty[H_PHI] = true;
  }
  getMainInd_new(o, p, g);
  const bool var = (o->theta > 0) || o->use_var_theta;
  while (drain ? (a0 < amax) : (a0 > amin)) {
    printf("\nStep %d: a = %f\n", step, a0);
    if (fp_out) fprintf(fp_out, "\nStep %d: a = %f\n", step, a0);
    if (var) {
      launch_setvarcurvadv(v.stream, v.box, v.mask, v.mask_x, v.mask_y, v.mask_z, v.bcoef, v.vx, v.vy, v.vz,
                           o->b, g->dx[0], v.red);
      unsigned long long keys[2];
      QSS_CK(cudaMemcpyAsync(keys, v.red, sizeof keys, cudaMemcpyDeviceToHost, v.stream));
      QSS_CK(cudaStreamSynchronize(v.stream));
      const double b_max = key_to_double(keys[0]);
      const double inv_dx = 1.0 / g->dx[0], inv_dy = 1.0 / g->dx[0], inv_dz = 1.0 / g->dx[0];
      o->b_max_over_dx = 2 * b_max * (inv_dx * inv_dx + inv_dy * inv_dy + inv_dz * inv_dz);
      o->max_U_over_dx = key_to_double(keys[1]);
      for (HostArray h : {H_BCOEF, H_VX, H_VY, H_VZ}) v.dirty[h] = true;
    } else {
      const double inv_dx = 1 / g->dx[0], inv_dy = 1 / g->dx[1], inv_dz = 1 / g->dx[2];
      o->b_max_over_dx = 2 * o->b * (inv_dx * inv_dx + inv_dy * inv_dy + inv_dz * inv_dz);
      o->max_U_over_dx = 0;
    }
    if (!drain) o->conserve_imbibe = 1;
    if (var) {
      launch_setvarnorm(v.stream, v.box, v.mask, v.mask_x, v.mask_y, v.mask_z, v.vel_n, a0, nullptr, o->theta,
                        g->dx[0]);
      v.nsrc_slabs = 0;
      v.dirty[H_VEL_N] = true;
    }
    if (o->check_connectivity) path_trap(v, g, o);
    const double t_step = path_const_curv(v, var, o, p, g, fp_out, a0);
    if (t_step == -1) break;
    if (drain) a0 += da;
    else a0 -= da;
    if (o->reservoir_inlet) launch_min_into(v.stream, n, v.phi, v.phi, v.phi_extra);
    launch_max_into(v.stream, n, v.phi, v.mask, v.phi);
    v.dirty[H_PHI] = true;
    if (prefix) {
      snprintf(fname, sizeof fname, "%sdata_step_%d", prefix, step);
      files.write(v, g, fname);
    }
    step += 1;
  }
  files.join();
  if (outermost) download_dirty(v, p);
}

}  // namespace
}  // namespace qss

using namespace qss;

#define QSS_API_BEGIN try {
#define QSS_API_END(ret)                  \
  }                                       \
  catch (const Error& e) {                \
    set_error(e.code, e.what());          \
    ret;                                  \
  }                                       \
  catch (const std::exception& e) {       \
    set_error(QSSGPU_ERR_CUDA, e.what()); \
    ret;                                  \
  }

extern "C" {

// drain_model3d.h:31
void drain_model3d(Options* o, QSS_DataArrays* p, Grid* g, FILE* fp_out) {
  CallScope scope;
  QSS_API_BEGIN
  dev_ladder(true, o, p, g, fp_out, scope.outermost(), "");
  QSS_API_END(return)
}

// imbibe_model3d.h
void imbibe_model3d(Options* o, QSS_DataArrays* p, Grid* g, FILE* fp_out) {
  CallScope scope;
  QSS_API_BEGIN
  dev_ladder(false, o, p, g, fp_out, scope.outermost(), "");
  QSS_API_END(return)
}

// See include/lsmpqs_gpu.h.
int qssgpu_ladder_batch(int drain, int n, Options* const* o, QSS_DataArrays* const* p, Grid* const* g,
                        FILE* const* fp, const char* const* prefix, int workers) {
  qssgpu_clear_error();
  if (n < 0 || (n > 0 && (!o || !p || !g))) {
    set_error(QSSGPU_ERR_ARG, "qssgpu_ladder_batch: bad arguments");
    return n > 0 ? n : 1;
  }
  for (int i = 0; i < n; i++)
    if (!o[i] || !p[i] || !g[i]) {
      set_error(QSSGPU_ERR_ARG, "qssgpu_ladder_batch: volume " + std::to_string(i) + " has a NULL option, array "
                                "or grid pointer");
      return n;
    }
  for (int i = 0; i < n; i++)
    for (int j = 0; j < i; j++)
      if (p[i] == p[j] || o[i] == o[j]) {
        set_error(QSSGPU_ERR_ARG, "qssgpu_ladder_batch: volumes must not share arrays or options");
        return n;
      }
  if (workers <= 0) workers = n;
  if (workers > 64) workers = 64;
  if (workers > n) workers = n;
  std::atomic<int> next{0};
  std::vector<int> codes(n, 0);
  std::vector<std::string> msgs(n);
  std::vector<double> setup(n, 0.0);
  // device arrays of every volume first: allocation serialises the device,
  // so it is done before the volumes run
  for (int v = 0; v < n; v++) {
    const auto t0 = std::chrono::steady_clock::now();
    try {
      volume_for(p[v], g[v]);
    } catch (const Error& e) {
      codes[v] = e.code ? e.code : 1;
      msgs[v] = e.what();
    } catch (const std::exception& e) {  // host memory for the volume's state
      codes[v] = QSSGPU_ERR_CUDA;
      msgs[v] = e.what();
    }
    setup[v] = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
  // largest volumes first, so that no large volume starts last and runs alone
  std::vector<int> order(n);
  for (int v = 0; v < n; v++) order[v] = v;
  std::stable_sort(order.begin(), order.end(),
                   [&](int x, int y) { return g[x]->num_gridpts > g[y]->num_gridpts; });
  auto work = [&]() {
    for (int k = next++; k < n; k = next++) {
      const int v = order[k];
      if (codes[v]) continue;
      qssgpu_clear_error();
      try {
        CallScope scope;  // each volume is an outermost call on its worker thread
        dev_ladder(drain != 0, o[v], p[v], g[v], fp ? fp[v] : nullptr, true, prefix ? prefix[v] : nullptr);
        volume_for(p[v], g[v]).phase_s[PH_SETUP] += setup[v];
        QSS_CK(cudaStreamSynchronize(volume_for(p[v], g[v]).stream));
      } catch (const Error& e) {
        set_error(e.code, e.what());
      } catch (const std::exception& e) {
        set_error(QSSGPU_ERR_CUDA, e.what());
      }
      codes[v] = qssgpu_last_error();
      if (codes[v]) msgs[v] = qssgpu_error_string();
    }
  };
  std::vector<std::thread> pool;
  for (int w = 1; w < workers; w++) pool.emplace_back(work);
  work();
  for (auto& t : pool) t.join();
  int failed = 0, first = -1;
  for (int v = 0; v < n; v++)
    if (codes[v]) {
      failed++;
      if (first < 0) first = v;
    }
  qssgpu_clear_error();
  if (first >= 0) set_error(codes[first], "volume " + std::to_string(first) + ": " + msgs[first]);
  return failed;
}

static int top_level(bool drain, Options* o, char* fdata, char* fgrid, char* fmask) {
  time_t t0;
  time(&t0);
  qssgpu_clear_error();
  if (!fdata || !fgrid || !fmask) {
    set_error(QSSGPU_ERR_ARG, "drainTop/imbibeTop need the data, grid and mask file names");
    return 1;
  }
  int n1[3], n2[3];
  QSS_DataArrays* p = allocateQSSDataArrays();
  p->phi = readDataArrayQSS(n1, fdata);
  p->mask = readDataArrayQSS(n2, fmask);
  Grid* g = readGridFromBinaryFile(fgrid);
  if (!p->phi || !p->mask) {
    set_error(QSSGPU_ERR_ARG, "could not read the data or mask file");
    return 1;
  }
  allocateMemoryForQSSDataArrays(p, g);
  for (int i = 0; i < 3; i++) {
    if (n1[i] != g->grid_dims_ghostbox[i] || n2[i] != g->grid_dims_ghostbox[i]) {
      printf("\nInput data dimensions n1[%d]=%d, n2[%d]=%d,", i, n1[i], i, n2[i]);
      printf(" (grid->grid_dims_ghostbox)[%d]=%d", i, g->grid_dims_ghostbox[i]);
      printf(" don't match\n");
      printf("\nTerminating...");
      return 1;
    }
  }
  FILE* fp = fopen(o->outfile, "a+");
  if (fp && o->print_details) {
    fprintf(fp, "Time Start %s\n", ctime(&t0));
    fprintf(fp, drain ? "Level Set Method simulation\n" : "Constant Curvature Model Level Set Method simulation\n");
    printOptions(o, fp);
    printGrid(g, fp);
  }
  if (fp) fflush(fp);
  if (g->num_dims == 3) {
    if (drain) drain_model3d(o, p, g, fp);
    else imbibe_model3d(o, p, g, fp);
  } else {
    set_error(QSSGPU_ERR_UNSUPPORTED, "only 3-D grids run on the GPU path");
  }
  if (o->save_data) {
    char fname[600];
    snprintf(fname, sizeof fname, "%s/data_final", o->path);
    writeDataArrayQSS(p->phi, g, fname, GZIP);
  }
  destroyQSSDataArrays(p);
  destroyGrid(g);
  if (fp) fclose(fp);
  return qssgpu_last_error() ? 1 : 0;
}

// drain_top.h:28
int drainTop(Options* o, char* fname_data_in, char* fname_grid_in, char* fname_mask_in) {
  return top_level(true, o, fname_data_in, fname_grid_in, fname_mask_in);
}

// imbibe_top.h
int imbibeTop(Options* o, char* fname_data_in, char* fname_grid_in, char* fname_mask_in) {
  return top_level(false, o, fname_data_in, fname_grid_in, fname_mask_in);
}

// connectivity.h:27
void trapComponents_mask(QSS_DataArrays* p, Grid* g, Options* o) {
  CallScope scope;
  QSS_API_BEGIN
  DevVolume& v = volume_for(p, g);
  if (scope.outermost()) {
    upload(v, p, H_PHI);
    upload(v, p, H_MASK);
    upload(v, p, H_MASK_NW);
  }
  path_trap(v, g, o);
  if (scope.outermost()) download_dirty(v, p);
  QSS_API_END(return)
}

// connectivity.h:23
void findConnectivity3d(QSS_DataArrays* p, Grid* g) {
  CallScope scope;
  QSS_API_BEGIN
  DevVolume& v = volume_for(p, g);
  if (scope.outermost()) upload(v, p, H_BIN);
  launch_label(v.stream, v.box, v.bin, v.labels, v.ctl);
  QSS_CK(cudaGetLastError());
  v.dirty[H_CONN] = true;
  if (scope.outermost()) download_dirty(v, p);
  QSS_API_END(return)
}

// connectivity.h: inlet (non-wetting) and outlet (wetting) reference points
void getMainInd_new(Options* o, QSS_DataArrays* p, Grid* g) {
  (void)p;
  const int nx = g->grid_dims_ghostbox[0], nxy = nx * g->grid_dims_ghostbox[1];
  if (g->num_dims == 3) {
    const int yi = (int)(0.5 * (g->jlo_fb + g->jhi_fb));
    const int zi = (int)(0.5 * (g->klo_fb + g->khi_fb));
    const int nwx = o->center_inlet ? (int)(0.5 * (g->ilo_fb + g->ihi_fb)) : g->ilo_fb - 1;
    o->phi_nw_ind = nwx + yi * nx + zi * nxy;
    o->phi_w_ind = (g->ihi_fb + 1) + yi * nx + zi * nxy;
  } else {
    const int yi = (int)(0.5 * (g->jlo_fb + g->jhi_fb));
    if (o->center_inlet) {
      o->phi_nw_ind = (int)(0.5 * (g->ilo_fb + g->ihi_fb)) + yi * nx;
      o->phi_w_ind = (g->ilo_fb - 1) + yi * nx;
    } else {
      o->phi_nw_ind = (g->ilo_fb - 1) + yi * nx;
      o->phi_w_ind = (g->ilo_fb + 1) + yi * nx;
    }
  }
}

// reinitialize_top.h:28 -- data is a host array of the caller
void reinitializeSubcellFix3d(double* data, Grid* g, Options* o) {
  QSS_API_BEGIN
  ensure_device();
  // a private device volume keyed by the host array
  thread_local QSS_DataArrays key;
  DevVolume& v = volume_for(&key, g);
  QSS_CK(cudaMemcpyAsync(v.scratch, data, v.n * sizeof(double), cudaMemcpyHostToDevice, v.stream));
  double* d = v.scratch;
  path_reinit(v, d, g, o);
  QSS_CK(cudaMemcpyAsync(data, d, v.n * sizeof(double), cudaMemcpyDeviceToHost, v.stream));
  QSS_CK(cudaStreamSynchronize(v.stream));
  if (d != v.scratch) std::swap(v.scratch, v.r_next);
  QSS_API_END(return)
}

// qss_general_util.c:422-706 -- faces 0..5, 6 = x, 7 = y, 8 = z, 9 = all, in order
void signedLinearExtrapolationBCqss(double* phi, Grid* g, int idx) {
  QSS_API_BEGIN
  ensure_device();
  if (g->num_dims != 3) throw Error(QSSGPU_ERR_UNSUPPORTED, "only 3-D grids run on the GPU path");
  int faces[6], nf = 0;
  switch (idx) {
    case 0: case 1: case 2: case 3: case 4: case 5: faces[nf++] = idx; break;
    case 6: faces[nf++] = 0; faces[nf++] = 1; break;
    case 7: faces[nf++] = 2; faces[nf++] = 3; break;
    case 8: faces[nf++] = 4; faces[nf++] = 5; break;
    case 9: for (int f = 0; f < 6; f++) faces[nf++] = f; break;
    default: return;
  }
  thread_local QSS_DataArrays key;
  DevVolume& v = volume_for(&key, g);
  QSS_CK(cudaMemcpyAsync(v.scratch, phi, v.n * sizeof(double), cudaMemcpyHostToDevice, v.stream));
  for (int q = 0; q < nf; q++) launch_face(v.stream, v.box, v.scratch, faces[q]);
  QSS_CK(cudaGetLastError());
  QSS_CK(cudaMemcpyAsync(phi, v.scratch, v.n * sizeof(double), cudaMemcpyDeviceToHost, v.stream));
  QSS_CK(cudaStreamSynchronize(v.stream));
  QSS_API_END(return)
}

// qss_general_util.c:82-143 (3-D; the '~use_var_theta' test of the reference is always true)
void setSpaceDerivFunc(Grid* g, Options* o) {
  (void)g;
  const bool plain = (o->theta == 0);
  switch (o->order_space_accur) {
    case 2: o->space_deriv_func = plain ? (qss_untyped_fn)getrhs3d2ndconst_ : (qss_untyped_fn)getrhs3d2nd_; break;
    case 3:
    case 4: o->space_deriv_func = plain ? (qss_untyped_fn)getrhs3d3rdconst_ : (qss_untyped_fn)getrhs3d3rd_; break;
    case 5: o->space_deriv_func = plain ? (qss_untyped_fn)getrhs3d3rdconst_ : (qss_untyped_fn)getrhs3d5th_; break;
    default: o->space_deriv_func = (qss_untyped_fn)getrhs3d3rd_;
  }
}

// qss_general_util.c:150-207 (constant-angle branch; see setSpaceDerivFunc)
void setThetaOverlap(QSS_DataArrays* p, Grid* g, Options* o) {
  (void)p;
  const double rad = 3.14159 / 180;
  const double th = o->theta;
  if (g->num_dims == 3) {
    if (th <= 20 * rad) o->overlap = 0;
    else if (th <= 40 * rad) o->overlap = 0.3 * g->dx[0];
    else if (th <= 50 * rad) o->overlap = 0.5 * g->dx[0];
    else if (th > 50 * rad) o->overlap = 1 * g->dx[0];
  } else {
    o->overlap = (th <= 20 * rad) ? 0 : 3 * g->dx[0];
  }
}

// qss_general_util.c:711-728 -- data is a host array
void initializeDisconnectedMasks(double* data, Grid* g) {
  QSS_API_BEGIN
  thread_local QSS_DataArrays key;
  DevVolume& v = volume_for(&key, g);
  dev_init_disconnected(v, v.scratch, g);
  QSS_CK(cudaMemcpyAsync(data, v.scratch, v.n * sizeof(double), cudaMemcpyDeviceToHost, v.stream));
  QSS_CK(cudaStreamSynchronize(v.stream));
  QSS_API_END(return)
}

// qss_general_util.c:813-833
void createReservoirInlet3d(QSS_DataArrays* p, Grid* g) {
  QSS_API_BEGIN
  DevVolume& v = volume_for(p, g);
  dev_reservoir(v, g);
  QSS_CK(cudaMemcpyAsync(p->phi_extra, v.phi_extra, v.n * sizeof(double), cudaMemcpyDeviceToHost, v.stream));
  QSS_CK(cudaStreamSynchronize(v.stream));
  QSS_API_END(return)
}

// ---------------------------------------------------------------------------
// Entry points for measuring the inner loop on device-resident data.

// Uploads phi and mask and runs the set-up of drain_model3d for curvature a0
// (mask gradient, scheme selection, overlap, coefficients of one curvature
// step, inlet/outlet points), without the trapping step or any time step.
int qssgpu_prepare_step(Options* o, QSS_DataArrays* p, Grid* g, double a0) {
  QSS_API_BEGIN
  DevVolume& v = volume_for(p, g);
  upload(v, p, H_PHI);
  upload(v, p, H_MASK);
  dev_init_disconnected(v, v.mask_w, g);
  dev_init_disconnected(v, v.mask_nw, g);
  launch_central_grad(v.stream, v.box, v.mask, v.mask_x, v.mask_y, v.mask_z, g->dx[0], g->dx[1], g->dx[2]);
  setSpaceDerivFunc(g, o);
  setThetaOverlap(p, g, o);
  getMainInd_new(o, p, g);
  const bool var = (o->theta > 0) || o->use_var_theta;
  if (var) {
    launch_setvarcurvadv(v.stream, v.box, v.mask, v.mask_x, v.mask_y, v.mask_z, v.bcoef, v.vx, v.vy, v.vz, o->b,
                         g->dx[0], v.red);
    unsigned long long keys[2];
    QSS_CK(cudaMemcpyAsync(keys, v.red, sizeof keys, cudaMemcpyDeviceToHost, v.stream));
    QSS_CK(cudaStreamSynchronize(v.stream));
    const double inv = 1.0 / g->dx[0];
    o->b_max_over_dx = 2 * key_to_double(keys[0]) * (inv * inv + inv * inv + inv * inv);
    o->max_U_over_dx = key_to_double(keys[1]);
    launch_setvarnorm(v.stream, v.box, v.mask, v.mask_x, v.mask_y, v.mask_z, v.vel_n, a0, nullptr, o->theta,
                      g->dx[0]);
    v.nsrc_slabs = 0;
  } else {
    const double ix = 1 / g->dx[0], iy = 1 / g->dx[1], iz = 1 / g->dx[2];
    o->b_max_over_dx = 2 * o->b * (ix * ix + iy * iy + iz * iz);
    o->max_U_over_dx = 0;
  }
  QSS_CK(cudaStreamSynchronize(v.stream));
  return 0;
  QSS_API_END(return 1)
}

// Runs `warmup` then `steps` inner steps on the device-resident volume with
// CUDA events on the volume's stream.  out[0] = device ms of the timed steps,
// out[1] = mean ms of one launch of the kernel with the largest total time,
// out[2] = kernel launches per step, out[3] = total ms inside the profiled
// stage kernels, out[4] = kind of that largest kernel (0 fused stage, 1..3
// WENO5 x/y/z pass, 4 combine), out[5..9] = total ms per kind, out[10..14] =
// launches per kind.
int qssgpu_time_steps(Options* o, QSS_DataArrays* p, Grid* g, double a0, int warmup, int steps, double* out) {
  QSS_API_BEGIN
  DevVolume& v = volume_for(p, g);
  Options oo = *o;
  oo.tplot = 1e300;
  path_inner_loop(v, &oo, g, a0, warmup > 0 ? warmup : 1);
  QSS_CK(cudaStreamSynchronize(v.stream));
  cudaEvent_t e0, e1;
  QSS_CK(cudaEventCreate(&e0));
  QSS_CK(cudaEventCreate(&e1));
  QSS_CK(cudaEventRecord(e0, v.stream));
  qss_profile_stage_begin(v.stream);
  path_inner_loop(v, &oo, g, a0, steps);
  QSS_CK(cudaEventRecord(e1, v.stream));
  QSS_CK(cudaEventSynchronize(e1));
  float ms = 0;
  QSS_CK(cudaEventElapsedTime(&ms, e0, e1));
  double kind_ms[kProfKinds];
  int kind_n[kProfKinds];
  qss_profile_stage_end(kind_ms, kind_n);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  int top = 0;
  double total = 0;
  for (int k = 0; k < kProfKinds; k++) {
    total += kind_ms[k];
    if (kind_ms[k] > kind_ms[top]) top = k;
  }
  out[0] = ms;
  out[1] = kind_n[top] ? kind_ms[top] / kind_n[top] : 0;
  out[2] = path_kernels_per_step(v, o);
  out[3] = total;
  out[4] = top;
  for (int k = 0; k < kProfKinds; k++) {
    out[5 + k] = kind_ms[k];
    out[5 + kProfKinds + k] = kind_n[k];
  }
  return 0;
  QSS_API_END(return 1)
}

}  // extern "C"
