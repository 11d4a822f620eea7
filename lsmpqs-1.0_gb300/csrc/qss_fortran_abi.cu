// qss_fortran_abi.cu -- single-kernel entry points with the reference's
// Fortran calling convention, backed by the GB300 kernels.
//
// Each call copies its host arrays to HBM, runs one kernel over the given
// fill box and copies the outputs back; outside the fill box an output array
// keeps the caller's values, as with the Fortran routines.  These entry
// points exist for drop-in linking and per-kernel parity checks; the path
// drivers never use them (they keep the data resident).  Ghost boxes must
// start at index 0, as every lsmpqs grid does.
//
// Reference routines (3d.f = src/spatial_derivatives/qss_spatial_derivatives3d.f):
//   getRHS3d2ndConst 3d.f:302, getRHS3d3rdConst :572, getRHS3d2nd :1020,
//   getRHS3d3rd :1335, getRHS3d5th :1827, getCentralGrad3dOrder2 :2987,
//   signedLinearExtrapolation3d :3055, setVarNorm3d :13, setVarNorm3dTheta :94,
//   setVarCurvAdv3d :178; qss_tvd_runge_kutta3d.f:2, 61, 131;
//   qss_reinitialization3d.f:476, 585; qss_util3d.f:65, 130, 288, 499.
#include <cstring>
#include <vector>

#include "qss_fortran_abi.h"
#include "qss_state.h"

using namespace qss;

namespace {

cudaStream_t abi_stream() {
  thread_local cudaStream_t s = nullptr;
  if (!s) QSS_CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  return s;
}

struct DBuf {
  void* p = nullptr;
  size_t bytes = 0;
  explicit DBuf(size_t b) : bytes(b) { QSS_CK(cudaMalloc(&p, b ? b : 8)); }
  ~DBuf() {
    if (p) cudaFree(p);
  }
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  double* d() { return (double*)p; }
};

struct Bounds {
  int lo[3], hi[3];
};

Bounds read6(const int* a, const int* b, const int* c, const int* d, const int* e, const int* f) {
  return Bounds{{*a, *c, *e}, {*b, *d, *f}};
}

Box make_box(const Bounds& gb, const Bounds& fb) {
  for (int q = 0; q < 3; q++)
    if (gb.lo[q] != 0) throw Error(QSSGPU_ERR_UNSUPPORTED, "ghost boxes must start at index 0");
  Box b;
  b.nx = gb.hi[0] + 1;
  b.ny = gb.hi[1] + 1;
  b.nz = gb.hi[2] + 1;
  b.ilo = fb.lo[0];
  b.ihi = fb.hi[0];
  b.jlo = fb.lo[1];
  b.jhi = fb.hi[1];
  b.klo = fb.lo[2];
  b.khi = fb.hi[2];
  return b;
}

bool empty(const Box& b) { return b.ihi < b.ilo || b.jhi < b.jlo || b.khi < b.klo; }

// fill-box points whose stencil reaches `r` cells must stay inside the ghost box
void check_reach(const Box& b, int r) {
  if (empty(b)) return;
  if (b.ilo - r < 0 || b.jlo - r < 0 || b.klo - r < 0 || b.ihi + r >= b.nx || b.jhi + r >= b.ny ||
      b.khi + r >= b.nz)
    throw Error(QSSGPU_ERR_ARG, "fill box too close to the ghost-box edge for this stencil");
}

void h2d(DBuf& d, const void* h, size_t bytes) {
  QSS_CK(cudaMemcpyAsync(d.p, h, bytes, cudaMemcpyHostToDevice, abi_stream()));
}
void d2h(void* h, DBuf& d, size_t bytes) {
  QSS_CK(cudaMemcpyAsync(h, d.p, bytes, cudaMemcpyDeviceToHost, abi_stream()));
}
void finish() {
  QSS_CK(cudaGetLastError());
  QSS_CK(cudaStreamSynchronize(abi_stream()));
}

void rhs_entry(int scheme, bool var, const double* phi, const double* vel_n, const double* b, const double* vx,
               const double* vy, const double* vz, double* max_H, double* lse_rhs, const Bounds& gb,
               const Bounds& fb, double dx, double dy, double dz) {
  ensure_device();
  Box bx = make_box(gb, fb);
  if (empty(bx)) return;
  check_reach(bx, scheme == ENO2 ? 2 : 3);
  if (scheme == ENO3 && bx.jhi >= bx.nz)
    throw Error(QSSGPU_ERR_UNSUPPORTED, "the ENO3 x-stencil reads phi(i+3,j,j) outside the grid");
  const size_t bytes = (size_t)bx.npts() * sizeof(double);
  cudaStream_t s = abi_stream();
  DBuf dphi(bytes), drhs(bytes), dh(8);
  h2d(dphi, phi, bytes);
  h2d(drhs, lse_rhs, bytes);
  Coef c{};
  std::vector<DBuf*> keep;
  DBuf dv(var ? bytes : 8), db(var ? bytes : 8), dvx(var ? bytes : 8), dvy(var ? bytes : 8),
      dvz(var ? bytes : 8), dns(var ? (size_t)bx.npts() * sizeof(int) : 8),
      drow(var ? (size_t)bx.fby() * bx.fbz() * sizeof(int) : 8),
      dcar(var ? (size_t)bx.fby() * bx.fbz() * sizeof(int) : 8), dcnt(8);
  if (var) {
    h2d(dv, vel_n, bytes);
    h2d(db, b, bytes);
    h2d(dvx, vx, bytes);
    h2d(dvy, vy, bytes);
    h2d(dvz, vz, bytes);
    c.vel_n = dv.d();
    c.b = db.d();
    c.vx = dvx.d();
    c.vy = dvy.d();
    c.vz = dvz.d();
    c.nsrc = (int*)dns.p;
    // the temp_norm carry of the Fortran loop restarts at the start of the call
    launch_nsrc(s, bx, c.vel_n, (int*)dns.p, 1, (int*)drow.p, (int*)dcar.p, (unsigned long long*)dcnt.p);
  } else {
    c.a_const = *vel_n;
    c.b_const = *b;
  }
  ImposeArgs im{};
  const int mode = (scheme == WENO5 && var) ? weno_mode() : 0;
  if (mode != 0) {
    DBuf d0(bytes), d1(bytes), d2(bytes), d3(bytes), d4(bytes), d5(bytes);
    double* const dp[3] = {d0.d(), d1.d(), d2.d()};
    double* const dm[3] = {d3.d(), d4.d(), d5.d()};
    launch_weno_axes(s, bx, dphi.d(), dx, dy, dz, dp, dm, nullptr);
    launch_weno_combine(s, 0, false, bx, dx, dy, dz, dphi.d(), nullptr, drhs.d(), nullptr, dp, dm, c, im, nullptr);
    QSS_CK(cudaStreamSynchronize(s));
  } else {
    launch_stage(s, scheme, var, 0, false, bx, dx, dy, dz, dphi.d(), nullptr, drhs.d(), nullptr, c, im, nullptr);
  }
  launch_cfl_at(s, scheme, var, bx, dphi.d(), c, bx.ihi, bx.jhi, bx.khi, dx, dy, dz, dh.d());
  d2h(lse_rhs, drhs, bytes);
  double h;
  d2h(&h, dh, sizeof h);
  finish();
  *max_H = h;
}

#define ABI_BEGIN try {
#define ABI_END                             \
  }                                         \
  catch (const Error& e) {                  \
    set_error(e.code, e.what());            \
  }                                         \
  catch (const std::exception& e) {         \
    set_error(QSSGPU_ERR_CUDA, e.what());   \
  }

}  // namespace

#define GB6P const int *ilo_gb, const int *ihi_gb, const int *jlo_gb, const int *jhi_gb, const int *klo_gb, \
             const int *khi_gb
#define FB6P const int *ilo_fb, const int *ihi_fb, const int *jlo_fb, const int *jhi_fb, const int *klo_fb, \
             const int *khi_fb
#define GB read6(ilo_gb, ihi_gb, jlo_gb, jhi_gb, klo_gb, khi_gb)
#define FB read6(ilo_fb, ihi_fb, jlo_fb, jhi_fb, klo_fb, khi_fb)

extern "C" {

void getrhs3d2ndconst_(const double* phi, const double* vel_n, const double* b, double* max_H, double* lse_rhs,
                       GB6P, FB6P, const double* dx, const double* dy, const double* dz) {
  ABI_BEGIN rhs_entry(ENO2, false, phi, vel_n, b, nullptr, nullptr, nullptr, max_H, lse_rhs, GB, FB, *dx, *dy, *dz);
  ABI_END
}

void getrhs3d3rdconst_(const double* phi, const double* vel_n, const double* b, double* max_H, double* lse_rhs,
                       GB6P, FB6P, const double* dx, const double* dy, const double* dz) {
  ABI_BEGIN rhs_entry(ENO3, false, phi, vel_n, b, nullptr, nullptr, nullptr, max_H, lse_rhs, GB, FB, *dx, *dy, *dz);
  ABI_END
}

void getrhs3d2nd_(const double* phi, const double* vel_n, const double* b, const double* vx, const double* vy,
                  const double* vz, double* max_H, double* lse_rhs, GB6P, FB6P, const double* dx, const double* dy,
                  const double* dz) {
  ABI_BEGIN rhs_entry(ENO2, true, phi, vel_n, b, vx, vy, vz, max_H, lse_rhs, GB, FB, *dx, *dy, *dz);
  ABI_END
}

void getrhs3d3rd_(const double* phi, const double* vel_n, const double* b, const double* vx, const double* vy,
                  const double* vz, double* max_H, double* lse_rhs, GB6P, FB6P, const double* dx, const double* dy,
                  const double* dz) {
  ABI_BEGIN rhs_entry(ENO3, true, phi, vel_n, b, vx, vy, vz, max_H, lse_rhs, GB, FB, *dx, *dy, *dz);
  ABI_END
}

void getrhs3d5th_(const double* phi, const double* vel_n, const double* b, const double* vx, const double* vy,
                  const double* vz, double* max_H, double* lse_rhs, GB6P, FB6P, const double* dx, const double* dy,
                  const double* dz) {
  ABI_BEGIN rhs_entry(WENO5, true, phi, vel_n, b, vx, vy, vz, max_H, lse_rhs, GB, FB, *dx, *dy, *dz);
  ABI_END
}

void getcentralgrad3dorder2_(double* phi_x, double* phi_y, double* phi_z, const int* ilo_g, const int* ihi_g,
                             const int* jlo_g, const int* jhi_g, const int* klo_g, const int* khi_g,
                             const double* phi, GB6P, FB6P, const double* dx, const double* dy, const double* dz) {
  ABI_BEGIN
  ensure_device();
  Bounds g2 = read6(ilo_g, ihi_g, jlo_g, jhi_g, klo_g, khi_g), g1 = GB;
  for (int q = 0; q < 3; q++)
    if (g2.lo[q] != g1.lo[q] || g2.hi[q] != g1.hi[q])
      throw Error(QSSGPU_ERR_UNSUPPORTED, "gradient and phi must share one ghost box");
  Box bx = make_box(g1, FB);
  if (empty(bx)) return;
  check_reach(bx, 1);
  const size_t bytes = (size_t)bx.npts() * sizeof(double);
  DBuf dp(bytes), gx(bytes), gy(bytes), gz(bytes);
  h2d(dp, phi, bytes);
  h2d(gx, phi_x, bytes);
  h2d(gy, phi_y, bytes);
  h2d(gz, phi_z, bytes);
  launch_central_grad(abi_stream(), bx, dp.d(), gx.d(), gy.d(), gz.d(), *dx, *dy, *dz);
  d2h(phi_x, gx, bytes);
  d2h(phi_y, gy, bytes);
  d2h(phi_z, gz, bytes);
  finish();
  ABI_END
}

void signedlinearextrapolation3d_(double* phi, GB6P, FB6P, const int* bdry_location_idx) {
  ABI_BEGIN
  ensure_device();
  const int face = *bdry_location_idx;
  if (face < 0 || face > 5) return;
  Box bx = make_box(GB, FB);
  const size_t bytes = (size_t)bx.npts() * sizeof(double);
  DBuf dp(bytes);
  h2d(dp, phi, bytes);
  launch_face(abi_stream(), bx, dp.d(), face);
  d2h(phi, dp, bytes);
  finish();
  ABI_END
}

static void varnorm_entry(const double* mask, const double* mx, const double* my, const double* mz, double* var_a,
                          double a0, const double* ca_field, double ca, const Bounds& gb, const Bounds& fb,
                          double dx) {
  ensure_device();
  Box bx = make_box(gb, fb);
  if (empty(bx)) return;
  const size_t bytes = (size_t)bx.npts() * sizeof(double);
  DBuf dm(bytes), dx_(bytes), dy_(bytes), dz_(bytes), dout(bytes), dth(ca_field ? bytes : 8);
  h2d(dm, mask, bytes);
  h2d(dx_, mx, bytes);
  h2d(dy_, my, bytes);
  h2d(dz_, mz, bytes);
  h2d(dout, var_a, bytes);
  if (ca_field) h2d(dth, ca_field, bytes);
  launch_setvarnorm(abi_stream(), bx, dm.d(), dx_.d(), dy_.d(), dz_.d(), dout.d(), a0,
                    ca_field ? dth.d() : nullptr, ca, dx);
  d2h(var_a, dout, bytes);
  finish();
}

void setvarnorm3d_(const double* mask, const double* mask_x, const double* mask_y, const double* mask_z,
                   double* var_a, const double* a0, const double* ca, GB6P, FB6P, const double* dx) {
  ABI_BEGIN varnorm_entry(mask, mask_x, mask_y, mask_z, var_a, *a0, nullptr, *ca, GB, FB, *dx);
  ABI_END
}

void setvarnorm3dtheta_(const double* mask, const double* mask_x, const double* mask_y, const double* mask_z,
                        double* var_a, const double* a0, const double* ca, GB6P, FB6P, const double* dx) {
  ABI_BEGIN varnorm_entry(mask, mask_x, mask_y, mask_z, var_a, *a0, ca, 0.0, GB, FB, *dx);
  ABI_END
}

void setvarcurvadv3d_(const double* mask, const double* mask_x, const double* mask_y, const double* mask_z,
                      double* var_b, double* vel_x, double* vel_y, double* vel_z, double* b_max_over_dx,
                      double* max_U_over_dx, const double* const_b, GB6P, FB6P, const double* dx) {
  ABI_BEGIN
  ensure_device();
  Box bx = make_box(GB, FB);
  const size_t bytes = (size_t)bx.npts() * sizeof(double);
  DBuf dm(bytes), gx(bytes), gy(bytes), gz(bytes), ob(bytes), ox(bytes), oy(bytes), oz(bytes), red(16);
  h2d(dm, mask, bytes);
  h2d(gx, mask_x, bytes);
  h2d(gy, mask_y, bytes);
  h2d(gz, mask_z, bytes);
  h2d(ob, var_b, bytes);
  h2d(ox, vel_x, bytes);
  h2d(oy, vel_y, bytes);
  h2d(oz, vel_z, bytes);
  if (empty(bx)) {
    unsigned long long init[2] = {double_to_key(-1.0), double_to_key(-1.0)};
    QSS_CK(cudaMemcpyAsync(red.p, init, sizeof init, cudaMemcpyHostToDevice, abi_stream()));
  } else {
    launch_setvarcurvadv(abi_stream(), bx, dm.d(), gx.d(), gy.d(), gz.d(), ob.d(), ox.d(), oy.d(), oz.d(),
                         *const_b, *dx, (unsigned long long*)red.p);
  }
  d2h(var_b, ob, bytes);
  d2h(vel_x, ox, bytes);
  d2h(vel_y, oy, bytes);
  d2h(vel_z, oz, bytes);
  unsigned long long keys[2];
  d2h(keys, red, sizeof keys);
  finish();
  const double b_max = key_to_double(keys[0]);
  const double inv_dx = 1.0 / *dx, inv_dy = 1.0 / *dx, inv_dz = 1.0 / *dx;
  *max_U_over_dx = key_to_double(keys[1]);
  *b_max_over_dx = 2 * b_max * (inv_dx * inv_dx + inv_dy * inv_dy + inv_dz * inv_dz);
  ABI_END
}

static void same_boxes(const std::vector<Bounds>& v) {
  for (size_t q = 1; q < v.size(); q++)
    for (int a = 0; a < 3; a++)
      if (v[q].lo[a] != v[0].lo[a] || v[q].hi[a] != v[0].hi[a])
        throw Error(QSSGPU_ERR_UNSUPPORTED, "all arrays of one call must share the ghost box");
}

static void rk_entry(int stage, double* out, const Bounds& g_out, const double* u1, const Bounds& g1,
                     const double* u0, const Bounds& g0, const double* rhs, const Bounds& gr, const Bounds& fb,
                     double dt) {
  ensure_device();
  same_boxes(u0 ? std::vector<Bounds>{g_out, g1, g0, gr} : std::vector<Bounds>{g_out, g1, gr});
  Box bx = make_box(g_out, fb);
  if (empty(bx)) return;
  const size_t bytes = (size_t)bx.npts() * sizeof(double);
  DBuf dout(bytes), d1(bytes), d0(u0 ? bytes : 8), dr(bytes);
  h2d(dout, out, bytes);
  h2d(d1, u1, bytes);
  if (u0) h2d(d0, u0, bytes);
  h2d(dr, rhs, bytes);
  launch_rk(abi_stream(), bx, stage, dout.d(), d1.d(), u0 ? d0.d() : nullptr, dr.d(), dt);
  d2h(out, dout, bytes);
  finish();
}

#define GBN(n) const int *ilo_##n, const int *ihi_##n, const int *jlo_##n, const int *jhi_##n, const int *klo_##n, \
               const int *khi_##n
#define RGB(n) read6(ilo_##n, ihi_##n, jlo_##n, jhi_##n, klo_##n, khi_##n)

void qss3drk1step_(double* u_next, GBN(a), const double* u_cur, GBN(b), const double* rhs, GBN(c), FB6P,
                   const double* dt) {
  ABI_BEGIN rk_entry(1, u_next, RGB(a), u_cur, RGB(b), nullptr, RGB(b), rhs, RGB(c), FB, *dt);
  ABI_END
}

void qss3dtvdrk2stage2_(double* u_stage2, GBN(a), const double* u_stage1, GBN(b), const double* u_cur, GBN(c),
                        const double* rhs, GBN(d), FB6P, const double* dt) {
  ABI_BEGIN rk_entry(2, u_stage2, RGB(a), u_stage1, RGB(b), u_cur, RGB(c), rhs, RGB(d), FB, *dt);
  ABI_END
}

void qss3dtvdrk3stage3_(double* u_next, GBN(a), const double* u_stage2, GBN(b), const double* u_cur, GBN(c),
                        const double* rhs, GBN(d), FB6P, const double* dt) {
  ABI_BEGIN rk_entry(3, u_next, RGB(a), u_stage2, RGB(b), u_cur, RGB(c), rhs, RGB(d), FB, *dt);
  ABI_END
}

void qss3dcomputedistanceforsubcellfix_(double* distance0, const double* phi0, GB6P, FB6P, const double* dx,
                                        const double* dy, const double* dz) {
  ABI_BEGIN
  ensure_device();
  Box bx = make_box(GB, FB);
  if (empty(bx)) return;
  check_reach(bx, 1);
  const size_t bytes = (size_t)bx.npts() * sizeof(double);
  DBuf dp(bytes), dd(bytes);
  h2d(dp, phi0, bytes);
  h2d(dd, distance0, bytes);
  launch_distance0(abi_stream(), bx, dp.d(), dd.d(), *dx, *dy, *dz);
  d2h(distance0, dd, bytes);
  finish();
  ABI_END
}

void qss3dcomputereinitializationeqnrhssubcellfixorder1_(double* reinit_rhs, const double* phi, GB6P,
                                                         const double* phi0, const double* distance0, FB6P,
                                                         const double* dx, const double* dy, const double* dz) {
  ABI_BEGIN
  ensure_device();
  Box bx = make_box(GB, FB);
  if (empty(bx)) return;
  check_reach(bx, 1);
  const size_t bytes = (size_t)bx.npts() * sizeof(double);
  DBuf dr(bytes), dp(bytes), d0(bytes), dd(bytes);
  h2d(dr, reinit_rhs, bytes);
  h2d(dp, phi, bytes);
  h2d(d0, phi0, bytes);
  h2d(dd, distance0, bytes);
  launch_reinit_rhs(abi_stream(), bx, dp.d(), d0.d(), dd.d(), dr.d(), *dx, *dy, *dz);
  d2h(reinit_rhs, dr, bytes);
  finish();
  ABI_END
}

void qss3dmaxnormdifflocal_(double* max_norm_diff, const double* field1, GBN(a), const double* field2, GBN(b),
                            const int* ilo_ib, const int* ihi_ib, const int* jlo_ib, const int* jhi_ib,
                            const int* klo_ib, const int* khi_ib, const double* local_zone) {
  ABI_BEGIN
  ensure_device();
  same_boxes({RGB(a), RGB(b)});
  Box bx = make_box(RGB(a), read6(ilo_ib, ihi_ib, jlo_ib, jhi_ib, klo_ib, khi_ib));
  if (empty(bx)) {
    *max_norm_diff = -1.0;
    return;
  }
  const size_t bytes = (size_t)bx.npts() * sizeof(double);
  DBuf d1(bytes), d2(bytes), key(8);
  h2d(d1, field1, bytes);
  h2d(d2, field2, bytes);
  launch_maxnormdiff(abi_stream(), bx, d1.d(), d2.d(), *local_zone, (unsigned long long*)key.p);
  unsigned long long k;
  d2h(&k, key, sizeof k);
  finish();
  *max_norm_diff = key_to_double(k);
  ABI_END
}

void imposemaskparallel_(double* phi_masked, const double* mask, const double* phi, const double* overlap, GB6P,
                         const int* cur_klo_gb, const int* cur_khi_gb) {
  ABI_BEGIN
  ensure_device();
  Bounds g = GB;
  Bounds fb = g;
  Box bx = make_box(g, fb);
  if (*cur_klo_gb < 0 || *cur_khi_gb >= bx.nz)
    throw Error(QSSGPU_ERR_ARG, "imposemaskparallel: z range outside the ghost box");
  const size_t bytes = (size_t)bx.npts() * sizeof(double);
  DBuf dout(bytes), dm(bytes), dp(bytes);
  h2d(dout, phi_masked, bytes);
  h2d(dm, mask, bytes);
  h2d(dp, phi, bytes);
  launch_impose_slab(abi_stream(), bx, dout.d(), dm.d(), dp.d(), *overlap, *cur_klo_gb, *cur_khi_gb);
  d2h(phi_masked, dout, bytes);
  finish();
  ABI_END
}

void qss3dvolumeregionphilessthanzero_(double* volume, const double* phi, GB6P, const int* ilo_ib,
                                       const int* ihi_ib, const int* jlo_ib, const int* jhi_ib,
                                       const int* klo_ib, const int* khi_ib, const double* dx, const double* dy,
                                       const double* dz, const double* epsilon) {
  ABI_BEGIN
  ensure_device();
  Box bx = make_box(GB, read6(ilo_ib, ihi_ib, jlo_ib, jhi_ib, klo_ib, khi_ib));
  if (empty(bx)) {
    *volume = 0.0;
    return;
  }
  const size_t bytes = (size_t)bx.npts() * sizeof(double);
  DBuf dp(bytes), dc((size_t)volume_scratch_doubles((int64_t)bx.fbx() * bx.fby() * bx.fbz()) * sizeof(double)),
      dv(8);
  h2d(dp, phi, bytes);
  launch_volume(abi_stream(), bx, dp.d(), *dx, *dy, *dz, *epsilon, dc.d(), dv.d());
  double v;
  d2h(&v, dv, sizeof v);
  finish();
  *volume = v;
  ABI_END
}

void imposetrapvelocity3d_(const double* phi_w, const double* phi_nw, double* normal_velocity,
                           double* curvature_coeff, double* vel_x, double* vel_y, double* vel_z, GB6P, FB6P,
                           const double* dx) {
  ABI_BEGIN
  (void)phi_nw;
  ensure_device();
  Box bx = make_box(GB, FB);
  if (empty(bx)) return;
  const size_t bytes = (size_t)bx.npts() * sizeof(double);
  DBuf dt(bytes), dn(bytes), db(bytes), dx_(bytes), dy_(bytes), dz_(bytes);
  h2d(dt, phi_w, bytes);
  h2d(dn, normal_velocity, bytes);
  h2d(db, curvature_coeff, bytes);
  h2d(dx_, vel_x, bytes);
  h2d(dy_, vel_y, bytes);
  h2d(dz_, vel_z, bytes);
  launch_trapvel(abi_stream(), bx, dt.d(), dn.d(), db.d(), dx_.d(), dy_.d(), dz_.d(), *dx);
  d2h(normal_velocity, dn, bytes);
  d2h(curvature_coeff, db, bytes);
  d2h(vel_x, dx_, bytes);
  d2h(vel_y, dy_, bytes);
  d2h(vel_z, dz_, bytes);
  finish();
  ABI_END
}

}  // extern "C"
