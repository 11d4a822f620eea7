// qss_api.cu -- the lsmpqs C API of the quasi-static level-set path, on GB300.
//
// Every entry point keeps the reference's name, signature, return convention
// and side effects on the caller's host arrays, so existing C callers link
// against this library instead of liblsmpqs.a.  Inside, the data live in HBM
// (one DevVolume per QSS_DataArrays) and every numerical step is a kernel:
// the host only keeps the reference's scalar control flow (t, tmax, tplot,
// the curvature ladder, stopping tests) in the same order and precision.
//
// The outermost API call uploads the host arrays it reads and, on return,
// refreshes every host array the reference would have modified; nested calls
// (drain_model3d -> constCurvModel3d -> trapComponents_mask ...) stay on the
// device.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <initializer_list>
#include <string>

#include "qss_fortran_abi.h"
#include "qss_state.h"

// RHS routines exported by this library (qss_fortran_abi.cu); their addresses
// identify the scheme stored in Options::space_deriv_func.
extern "C" {
void signedLinearExtrapolationBCqss(double* phi, Grid* g, int idx);
void writeDataArrayQSS(double* data, Grid* grid, char* file_name, int zip_status);
double* readDataArrayQSS(int* grid_dims_ghostbox, char* file_name);
}

namespace qss {

namespace {

struct SchemeSel {
  int scheme;
  bool var;
};

SchemeSel scheme_of(const Options* o) {
  void* f = (void*)o->space_deriv_func;
  if (f == (void*)getrhs3d2ndconst_) return {ENO2, false};
  if (f == (void*)getrhs3d3rdconst_) return {ENO3, false};
  if (f == (void*)getrhs3d2nd_) return {ENO2, true};
  if (f == (void*)getrhs3d3rd_) return {ENO3, true};
  if (f == (void*)getrhs3d5th_) return {WENO5, true};
  throw Error(QSSGPU_ERR_ARG,
              "Options::space_deriv_func is not one of this library's RHS routines "
              "(call setSpaceDerivFunc first)");
}

void sync(DevVolume& v) { QSS_CK(cudaStreamSynchronize(v.stream)); }

void check_device_flags(DevVolume& v) {
  QSS_CK(cudaMemcpyAsync(v.h_ctl, v.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, v.stream));
  sync(v);
  if (v.h_ctl->err)
    throw Error(QSSGPU_ERR_DEVICE_CHECK, "a device-side iteration cap was reached (flags " +
                                             std::to_string(v.h_ctl->err) + ")");
}

ImposeArgs impose_args(DevVolume& v, const Options* o) {
  return ImposeArgs{v.mask, v.mask_w, v.mask_nw, o->overlap, o->check_connectivity ? 1 : 0};
}

Coef coef_of(DevVolume& v, const Options* o, bool var, double a) {
  Coef c;
  c.vel_n = v.vel_n;
  c.b = v.bcoef;
  c.vx = v.vx;
  c.vy = v.vy;
  c.vz = v.vz;
  c.a_const = var ? 0.0 : a;
  c.b_const = o->b;
  c.nsrc = v.nsrc;
  return c;
}

// source map of the carried normal term for the current vel_n and slab count
void ensure_nsrc(DevVolume& v, int nslabs) {
  if (v.nsrc_slabs == nslabs) return;
  launch_nsrc(v.stream, v.box, v.vel_n, v.nsrc, nslabs, v.rowlast, v.carry, v.count);
  QSS_CK(cudaGetLastError());
  v.nsrc_slabs = nslabs;
}

// ---------------------------------------------------------------------------
// reinitializeSubcellFix3d (reinitialize_top.c:297-377) on a device array

int reinit_iterations(const Grid* g, const Options* o) {
  double t_r = 0, dt_r = 0.5 * g->dx[0];
  int n = 0;
  while (t_r < o->tmax_r) {
    n++;
    t_r = t_r + dt_r;
    if (n > 100000000) throw Error(QSSGPU_ERR_ARG, "tmax_r / dx gives too many reinitialisation steps");
  }
  return n;
}

void dev_reinit(DevVolume& v, double*& data, const Grid* g, const Options* o) {
  PhaseTimer pt(v, PH_REINIT);
  const Box& b = v.box;
  const double dx = g->dx[0], dy = g->dx[1], dz = g->dx[2];
  const double dt_r = 0.5 * g->dx[0];
  const int iters = reinit_iterations(g, o);
  QSS_CK(cudaMemcpyAsync(v.r_phi0, data, v.n * sizeof(double), cudaMemcpyDeviceToDevice, v.stream));
  launch_distance0(v.stream, b, v.r_phi0, v.r_dist, dx, dy, dz);
  ImposeArgs none{};
  for (int it = 0; it < iters; it++) {
    launch_reinit_step(v.stream, b, data, v.r_phi0, v.r_dist, v.r_next, dt_r, dx, dy, dz);
    launch_ghost(v.stream, b, v.r_next, nullptr, none, nullptr);
    std::swap(data, v.r_next);
  }
  QSS_CK(cudaGetLastError());
}

// ---------------------------------------------------------------------------
// trapComponents_mask (trapComponents.c:156-375)

void dev_trap(DevVolume& v, const Grid* g, const Options* o) {
  PhaseTimer pt(v, PH_TRAP);
  const int64_t n = v.n;
  if (o->phi_nw_ind < 0 || o->phi_nw_ind >= n || o->phi_w_ind < 0 || o->phi_w_ind >= n)
    throw Error(QSSGPU_ERR_ARG, "phi_nw_ind / phi_w_ind outside the grid (call getMainInd_new)");
  const double fill = -20 * g->dx[0];
  launch_bin_nw(v.stream, n, v.phi, v.mask_nw, v.bin);
  launch_set_bin_slab(v.stream, v.box, v.bin, o->center_inlet, 0);
  launch_label(v.stream, v.box, v.bin, v.labels, v.ctl);
  launch_trap_nw(v.stream, n, v.labels, o->phi_nw_ind, v.phi, v.mask, v.mask_nw, v.scratch, v.bin, fill);
  launch_set_bin_slab(v.stream, v.box, v.bin, o->center_inlet, 1);
  launch_label(v.stream, v.box, v.bin, v.labels, v.ctl);
  launch_trap_w(v.stream, n, v.labels, o->phi_w_ind, v.scratch, v.mask_w, fill);
  QSS_CK(cudaGetLastError());
  for (HostArray a : {H_PHI, H_MASK_NW, H_MASK_W, H_CONN, H_BIN}) v.dirty[a] = true;
  v.zero_on_return[H_SCRATCH1] = true;
}

double dev_volume(DevVolume& v, const double* f, const Grid* g, double eps) {
  PhaseTimer pt(v, PH_REDUCE);
  launch_volume(v.stream, v.box, f, g->dx[0], g->dx[1], g->dx[2], eps, v.contrib, v.dscal);
  QSS_CK(cudaMemcpyAsync(v.h_scal, v.dscal, sizeof(double), cudaMemcpyDeviceToHost, v.stream));
  sync(v);
  return v.h_scal[0];
}

double dev_maxnorm(DevVolume& v, const Options* o) {
  PhaseTimer pt(v, PH_REDUCE);
  launch_maxnormdiff(v.stream, v.box, v.phi, v.phi_prev, o->err_check_zone, v.red + 2);
  unsigned long long key;
  QSS_CK(cudaMemcpyAsync(&key, v.red + 2, sizeof key, cudaMemcpyDeviceToHost, v.stream));
  sync(v);
  return key_to_double(key);
}

// ---------------------------------------------------------------------------
// one inner pseudo-time step (constCurvModel3d.c:127-243), predicated on the
// device loop condition

// one stage: RHS of `in` fused with the TVD-RK combination into `out`; on the
// last stage also the impositions into phi (in place)
void enqueue_stage(DevVolume& v, const SchemeSel& sc, const Coef& c, const ImposeArgs& im, int stage, bool fin,
                   const double* in, double* out, double* phi_new, const Grid* g) {
  const double dx = g->dx[0], dy = g->dx[1], dz = g->dx[2];
  const int mode = (sc.scheme == WENO5 && sc.var) ? weno_mode() : 0;
  if (mode == 1) {
    launch_weno_axes(v.stream, v.box, in, dx, dy, dz, v.dplus, v.dminus, v.ctl);
    launch_weno_combine(v.stream, stage, fin, v.box, dx, dy, dz, in, v.phi, out, phi_new, v.dplus, v.dminus, c,
                        im, v.ctl);
  } else {
    launch_stage(v.stream, sc.scheme, sc.var, stage, fin, v.box, dx, dy, dz, in, v.phi, out, phi_new, c, im,
                 v.ctl);
  }
}

void enqueue_step(DevVolume& v, const SchemeSel& sc, const Coef& c, const ImposeArgs& im, int order,
                  int nslabs, const Grid* g) {
  const Box& b = v.box;
  const double dx = g->dx[0], dy = g->dx[1], dz = g->dx[2];
  cudaStream_t s = v.stream;
  launch_dt(s, sc.scheme, sc.var, b, v.phi, c, nslabs, dx, dy, dz, v.ctl);
  if (order <= 1) {
    enqueue_stage(v, sc, c, im, 1, false, v.phi, v.s1, nullptr, g);
    launch_ghost(s, b, v.s1, nullptr, im, v.ctl);
    launch_impose_region(s, b, v.s1, v.phi, im, v.ctl);
    v.phi_next_buf = 1;
  } else if (order == 2) {
    enqueue_stage(v, sc, c, im, 1, false, v.phi, v.s1, nullptr, g);
    launch_ghost(s, b, v.s1, nullptr, im, v.ctl);
    enqueue_stage(v, sc, c, im, 2, true, v.s1, v.s2, v.phi, g);
    launch_ghost(s, b, v.s2, v.phi, im, v.ctl);
    v.phi_next_buf = 2;
  } else {
    enqueue_stage(v, sc, c, im, 1, false, v.phi, v.s1, nullptr, g);
    launch_ghost(s, b, v.s1, nullptr, im, v.ctl);
    enqueue_stage(v, sc, c, im, 2, false, v.s1, v.s2, nullptr, g);
    launch_ghost(s, b, v.s2, nullptr, im, v.ctl);
    enqueue_stage(v, sc, c, im, 3, true, v.s2, v.s1, v.phi, g);
    launch_ghost(s, b, v.s1, v.phi, im, v.ctl);
    v.phi_next_buf = 1;
  }
}

int kernels_per_step(int order, int mode) {
  const int per_stage = mode == 1 ? 4 : 1;
  const int stages = order <= 1 ? 1 : (order == 2 ? 2 : 3);
  return 1 + stages * (per_stage + 1) + (order <= 1 ? 1 : 0);
}

// Runs the inner loop to completion; returns dt_sub.
double dev_inner_loop(DevVolume& v, const SchemeSel& sc, const Options* o, const Grid* g, double a,
                      int max_steps) {
  PhaseTimer pt(v, PH_INNER);
  const int nslabs = num_slabs_for(g);
  if (sc.scheme == ENO3 && g->jhi_fb - g->jlo_gb > g->khi_gb - g->klo_gb)
    throw Error(QSSGPU_ERR_UNSUPPORTED,
                "the ENO3 x-stencil of the reference reads phi(i+3,j,j), which lies outside the grid "
                "when the y extent exceeds the z extent");
  if (sc.var) ensure_nsrc(v, nslabs);
  Ctl init{};
  init.dt = 0;
  init.dt_sub = 0;
  init.tplot = o->tplot;
  init.b_max_over_dx = o->b_max_over_dx;
  init.max_U_over_dx = o->max_U_over_dx;
  init.cur_max_H = -1;
  init.active = 1;
  init.steps = 0;
  init.max_steps = max_steps;
  init.err = 0;
  *v.h_ctl = init;
  QSS_CK(cudaMemcpyAsync(v.ctl, v.h_ctl, sizeof(Ctl), cudaMemcpyHostToDevice, v.stream));
  const Coef c = coef_of(v, o, sc.var, a);
  const ImposeArgs im = impose_args(v, o);
  int order = o->order_time_accur;
  // Steps are queued in batches; a step queued after the loop condition
  // turned false does nothing, so over-queueing only costs launches.  The
  // batch size follows the remaining pseudo time.
  int batch = 2;
  if (max_steps > 0 && batch > max_steps) batch = max_steps;
  for (int guard = 0;; guard++) {
    for (int q = 0; q < batch; q++) enqueue_step(v, sc, c, im, order, nslabs, g);
    QSS_CK(cudaGetLastError());
    QSS_CK(cudaMemcpyAsync(v.h_ctl, v.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, v.stream));
    sync(v);
    if (v.h_ctl->err) throw Error(QSSGPU_ERR_DEVICE_CHECK, "device check failed in the inner loop");
    if (!v.h_ctl->active) break;
    if (max_steps > 0 && v.h_ctl->steps >= max_steps) break;
    const double dt = v.h_ctl->dt;
    // a non-positive or NaN step would never reach tplot (the reference loops forever)
    if (!(dt > 0)) throw Error(QSSGPU_ERR_ARG, "the CFL time step is not positive (check b_max_over_dx / max_U_over_dx)");
    double remain = (o->tplot - v.h_ctl->dt_sub) / (dt > 0 ? dt : 1.0);
    if (!(remain >= 0)) remain = 1;
    batch = (int)std::min(256.0, remain + 2.0);
    if (max_steps > 0) batch = std::min(batch, max_steps - v.h_ctl->steps);
    if (batch < 1) batch = 1;
    if (guard > 10000000) throw Error(QSSGPU_ERR_DEVICE_CHECK, "inner loop does not terminate");
  }
  v.inner_steps += v.h_ctl->steps;
  if (v.h_ctl->steps > 0) {
    v.dirty[H_PHI] = v.dirty[H_PHI_NEXT] = true;
    v.zero_on_return[H_LSE_RHS] = v.zero_on_return[H_SCRATCH1] = v.zero_on_return[H_SCRATCH2] = true;
  }
  return v.h_ctl->dt_sub;
}

// constCurvModel3d / constCurvModel3dNoVar (constCurvModel3d.c:50-334 / 336-610)
double dev_const_curv(DevVolume& v, bool var, Options* o, QSS_DataArrays* p, Grid* g, FILE* fp_out,
                      double a) {
  SchemeSel sc = scheme_of(o);
  if (sc.var != var)
    throw Error(QSSGPU_ERR_ARG, var ? "constCurvModel3d needs a variable-coefficient RHS routine"
                                    : "constCurvModel3dNoVar needs a constant-coefficient RHS routine");
  double dt_sub = 0, t = 0;
  double max_abs_err = 100, vol_phi = 100;
  const double vol_very_small = g->dx[0] * g->dx[1] * g->dx[2];
  const double eps = o->eps_coefficient * g->dx[0];
  const double max_satn = o->vol_frac_max;
  const double vol_pore = dev_volume(v, v.mask, g, eps);
  vol_phi = dev_volume(v, v.phi, g, eps);
  double satn = vol_phi / vol_pore, satn_old;
  while ((t < o->tmax) && (max_abs_err > o->eps_stop)) {
    v.outer_iters++;
    dt_sub = 0;
    QSS_CK(cudaMemcpyAsync(v.phi_prev, v.phi, v.n * sizeof(double), cudaMemcpyDeviceToDevice, v.stream));
    v.dirty[H_PHI_PREV] = true;
    cudaEvent_t e0, e1;
    QSS_CK(cudaEventCreate(&e0));
    QSS_CK(cudaEventCreate(&e1));
    QSS_CK(cudaEventRecord(e0, v.stream));
    dt_sub = dev_inner_loop(v, sc, o, g, a, 0);
    QSS_CK(cudaEventRecord(e1, v.stream));
    sync(v);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (fp_out) fprintf(fp_out, "%d threads: Level set time = %lf\n", num_slabs_for(g), ms * 1e-3);

    t += dt_sub;
    if (var) {
      launch_max_into(v.stream, v.n, v.phi, v.mask, v.phi);
      v.dirty[H_PHI] = true;
    }
    if (o->check_connectivity) {
      dev_trap(v, g, o);
      dev_reinit(v, v.mask_w, g, o);
      dev_reinit(v, v.mask_nw, g, o);
      if (var && o->conserve_imbibe) {
        launch_trapvel(v.stream, v.box, v.mask_nw, v.vel_n, v.bcoef, v.vx, v.vy, v.vz, g->dx[0]);
        v.nsrc_slabs = 0;
        for (HostArray h : {H_VEL_N, H_BCOEF, H_VX, H_VY, H_VZ}) v.dirty[h] = true;
      }
      launch_merge(v.stream, v.n, v.phi, v.mask_nw);
    }
    if (fp_out) fprintf(fp_out, "Reinitializing....");
    dev_reinit(v, v.phi, g, o);
    if (fp_out) fprintf(fp_out, "Reinitialized\n");
    v.dirty[H_PHI] = true;
    max_abs_err = dev_maxnorm(v, o);
    satn_old = satn;
    vol_phi = dev_volume(v, v.phi, g, eps);
    check_device_flags(v);
    satn = vol_phi / vol_pore;
    if ((satn > max_satn) || (vol_phi <= vol_very_small)) return -1;
    if (o->checkpoint) {
      download_dirty(v, p);
      writeDataArrayQSS(p->phi, g, (char*)"checkpoint_phi", GZIP);
      writeDataArrayQSS(p->phi_prev, g, (char*)"checkpoint_phi_prev", GZIP);
      writeDataArrayQSS(p->mask_w, g, (char*)"mask_w", GZIP);
      writeDataArrayQSS(p->mask_nw, g, (char*)"mask_nw", GZIP);
    }
    if (fp_out) {
      fprintf(fp_out, "connectivity time = %lf\n", 0.0);
      fprintf(fp_out, "t = %4.1f\t", t);
      fprintf(fp_out, "max_abs_err = %4.3f,\t", max_abs_err);
      fprintf(fp_out, "nw phase satn pct = %4.3f\n", satn * 100);
    }
    printf("t = %4.1f\t", t);
    printf("max_abs_err = %4.3f,\t", max_abs_err);
    printf("nw phase satn = %4.3f\n", satn * 100);
    if (fp_out) fflush(fp_out);
    if (o->use_satn_stop) {
      if (fabsf((float)(100 * (satn - satn_old))) < 0.001) break;
    }
  }
  return t;
}

// uploads for a constant-curvature call made directly by the caller
void upload_for_const_curv(DevVolume& v, QSS_DataArrays* p, const Options* o, bool var) {
  upload(v, p, H_PHI);
  upload(v, p, H_MASK);
  if (o->check_connectivity) {
    upload(v, p, H_MASK_W);
    upload(v, p, H_MASK_NW);
  }
  if (var) {
    for (HostArray h : {H_VEL_N, H_BCOEF, H_VX, H_VY, H_VZ}) upload(v, p, h);
    v.nsrc_slabs = 0;
  }
}

}  // namespace

// shared with qss_fortran_abi.cu / qss_paths.cu
void path_reinit(DevVolume& v, double*& data, const Grid* g, const Options* o) { dev_reinit(v, data, g, o); }
void path_trap(DevVolume& v, const Grid* g, const Options* o) { dev_trap(v, g, o); }
double path_const_curv(DevVolume& v, bool var, Options* o, QSS_DataArrays* p, Grid* g, FILE* fp, double a) {
  return dev_const_curv(v, var, o, p, g, fp, a);
}
double path_inner_loop(DevVolume& v, Options* o, Grid* g, double a, int max_steps) {
  SchemeSel sc = scheme_of(o);
  return dev_inner_loop(v, sc, o, g, a, max_steps);
}
int path_kernels_per_step(DevVolume& v, const Options* o) {
  SchemeSel sc = scheme_of(o);
  return kernels_per_step(o->order_time_accur, (sc.scheme == WENO5 && sc.var) ? weno_mode() : 0);
}
void path_upload_for_const_curv(DevVolume& v, QSS_DataArrays* p, const Options* o, bool var) {
  upload_for_const_curv(v, p, o, var);
}

}  // namespace qss

using namespace qss;

#define QSS_API_BEGIN try {
#define QSS_API_END(ret)                                                   \
  }                                                                        \
  catch (const Error& e) {                                                 \
    set_error(e.code, e.what());                                           \
    ret;                                                                   \
  }                                                                        \
  catch (const std::exception& e) {                                        \
    set_error(QSSGPU_ERR_CUDA, e.what());                                  \
    ret;                                                                   \
  }

extern "C" {

// constCurvModel3d.h:29
double constCurvModel3d(Options* o, QSS_DataArrays* p, Grid* g, FILE* fp_out) {
  CallScope scope;
  QSS_API_BEGIN
  DevVolume& v = volume_for(p, g);
  if (scope.outermost()) {
    v.inner_steps = v.outer_iters = 0;
    reset_phases(v);
    upload_for_const_curv(v, p, o, true);
    if (o->check_connectivity)
      start_prefault(v, p, {H_PHI_NEXT, H_PHI_PREV, H_LSE_RHS, H_SCRATCH1, H_SCRATCH2, H_MASK_W, H_MASK_NW,
                            H_CONN, H_BIN});
    else
      start_prefault(v, p, {H_PHI_NEXT, H_PHI_PREV, H_LSE_RHS, H_SCRATCH1, H_SCRATCH2});
  }
  PrefaultGuard pg{v};
  double t = dev_const_curv(v, true, o, p, g, fp_out, 0.0);
  if (scope.outermost()) download_dirty(v, p);
  return t;
  QSS_API_END(return -1)
}

// constCurvModel3d.h:30
double constCurvModel3dNoVar(Options* o, QSS_DataArrays* p, Grid* g, FILE* fp_out, double a) {
  CallScope scope;
  QSS_API_BEGIN
  DevVolume& v = volume_for(p, g);
  if (scope.outermost()) {
    v.inner_steps = v.outer_iters = 0;
    reset_phases(v);
    upload_for_const_curv(v, p, o, false);
    if (o->check_connectivity)
      start_prefault(v, p, {H_PHI_NEXT, H_PHI_PREV, H_LSE_RHS, H_SCRATCH1, H_SCRATCH2, H_MASK_W, H_MASK_NW,
                            H_CONN, H_BIN});
    else
      start_prefault(v, p, {H_PHI_NEXT, H_PHI_PREV, H_LSE_RHS, H_SCRATCH1, H_SCRATCH2});
  }
  PrefaultGuard pg{v};
  double t = dev_const_curv(v, false, o, p, g, fp_out, a);
  if (scope.outermost()) download_dirty(v, p);
  return t;
  QSS_API_END(return -1)
}

// host wall time of the last top-level call on p by phase: out[0] total,
// [1] set-up, [2] uploads, [3] inner steps, [4] trapping, [5]
// reinitialisation, [6] volume and max-norm reductions, [7] downloads
void qssgpu_call_times(const QSS_DataArrays* p, const Grid* g, double* out) {
  try {
    DevVolume& v = volume_for(p, g);
    for (int k = 0; k < 8; k++) out[k] = v.phase_s[k];
  } catch (const Error& e) {
    set_error(e.code, e.what());
  }
}

// device time of the last top-level call on p by phase (CUDA events on the
// volume's stream): out[0] the sum, then set-up, uploads, inner steps,
// trapping, reinitialisation, reductions, downloads, as qssgpu_call_times
void qssgpu_call_device_times(const QSS_DataArrays* p, const Grid* g, double* out) {
  QSS_API_BEGIN
  DevVolume& v = volume_for(p, g);
  resolve_phase_events(v);
  double sum = 0;
  for (int k = 1; k < 8; k++) {
    out[k] = v.phase_dev_s[k];
    sum += out[k];
  }
  out[0] = sum;
  QSS_API_END(return)
}

// statistics of the last top-level call on p: inner steps and outer iterations
void qssgpu_call_stats(const QSS_DataArrays* p, const Grid* g, long long* inner_steps, long long* outer_iters) {
  QSS_API_BEGIN
  DevVolume& v = volume_for(p, g);
  if (inner_steps) *inner_steps = v.inner_steps;
  if (outer_iters) *outer_iters = v.outer_iters;
  QSS_API_END(return)
}

}  // extern "C"
