// qss_geometry.cu -- signed-distance initialisers of the lsmpqs C API
// (src/geometry/qss_initialization3d.c:19-165, 440-522), evaluated on the GPU
// and returned in the caller's host array.  3-D grids only.
#include <vector>

#include "qss_state.h"

using namespace qss;

namespace {

Box full_box(const Grid* g) {
  if (!g || g->num_dims != 3) throw Error(QSSGPU_ERR_UNSUPPORTED, "only 3-D grids are supported");
  Box b;
  b.nx = g->grid_dims_ghostbox[0];
  b.ny = g->grid_dims_ghostbox[1];
  b.nz = g->grid_dims_ghostbox[2];
  b.ilo = 0;
  b.ihi = b.nx - 1;
  b.jlo = 0;
  b.jhi = b.ny - 1;
  b.klo = 0;
  b.khi = b.nz - 1;
  return b;
}

struct Dev {
  void* p = nullptr;
  explicit Dev(size_t bytes) { QSS_CK(cudaMalloc(&p, bytes ? bytes : 8)); }
  ~Dev() {
    if (p) cudaFree(p);
  }
  template <class T>
  T* as() {
    return (T*)p;
  }
};

template <class T>
void put(Dev& d, const T* h, int n) {
  QSS_CK(cudaMemcpy(d.p, h, (size_t)n * sizeof(T), cudaMemcpyHostToDevice));
}

void halfspaces_into(double* d_phi, const Box& b, const Grid* g, int num, const double* nx, const double* ny,
                     const double* nz, const double* px, const double* py, const double* pz) {
  Dev a(num * 8), bb(num * 8), c(num * 8), d(num * 8), e(num * 8), f(num * 8);
  put(a, nx, num);
  put(bb, ny, num);
  put(c, nz, num);
  put(d, px, num);
  put(e, py, num);
  put(f, pz, num);
  launch_halfspaces(nullptr, b, d_phi, g->x_lo_ghostbox, g->dx, a.as<double>(), bb.as<double>(), c.as<double>(),
                    d.as<double>(), e.as<double>(), f.as<double>(), num);
  QSS_CK(cudaGetLastError());
  QSS_CK(cudaDeviceSynchronize());
}

}  // namespace

#define GEO_BEGIN try {                        \
  ensure_device();
#define GEO_END                                \
  }                                            \
  catch (const Error& e) {                     \
    set_error(e.code, e.what());               \
  }                                            \
  catch (const std::exception& e) {            \
    set_error(QSSGPU_ERR_CUDA, e.what());      \
  }

extern "C" {

void createIntersectionOfSpheres(double* phi, int num, double* cx, double* cy, double* cz, double* radius,
                                 int* inside_flag, Grid* g) {
  GEO_BEGIN
  Box b = full_box(g);
  const size_t bytes = (size_t)b.npts() * sizeof(double);
  Dev dphi(bytes), a(num * 8), bb(num * 8), c(num * 8), r(num * 8), in(num * 4);
  put(a, cx, num);
  put(bb, cy, num);
  put(c, cz, num);
  put(r, radius, num);
  put(in, inside_flag, num);
  launch_spheres(nullptr, b, dphi.as<double>(), g->x_lo_ghostbox, g->dx, a.as<double>(), bb.as<double>(),
                 c.as<double>(), r.as<double>(), in.as<int>(), num);
  QSS_CK(cudaGetLastError());
  QSS_CK(cudaMemcpy(phi, dphi.p, bytes, cudaMemcpyDeviceToHost));
  GEO_END
}

void createSphere(double* phi, double cx, double cy, double cz, double radius, int inside_flag, Grid* g) {
  createIntersectionOfSpheres(phi, 1, &cx, &cy, &cz, &radius, &inside_flag, g);
}

void createIntersectionOfHalfSpaces3d(double* phi, int num, double* nx, double* ny, double* nz, double* px,
                                      double* py, double* pz, Grid* g) {
  GEO_BEGIN
  Box b = full_box(g);
  const size_t bytes = (size_t)b.npts() * sizeof(double);
  Dev dphi(bytes);
  halfspaces_into(dphi.as<double>(), b, g, num, nx, ny, nz, px, py, pz);
  QSS_CK(cudaMemcpy(phi, dphi.p, bytes, cudaMemcpyDeviceToHost));
  GEO_END
}

void createPlane(double* phi, double nx, double ny, double nz, double px, double py, double pz, Grid* g) {
  createIntersectionOfHalfSpaces3d(phi, 1, &nx, &ny, &nz, &px, &py, &pz, g);
}

void createPolyhedron3d(double* phi, int num, double* nx, double* ny, double* nz, double* px, double* py,
                        double* pz, Grid* g) {
  createIntersectionOfHalfSpaces3d(phi, num, nx, ny, nz, px, py, pz, g);
}

// each box is the intersection of its six faces; boxes combine by max
void createIntersectionOfBoxes(double* phi, int num, double* cx, double* cy, double* cz, double* sx, double* sy,
                               double* sz, int* inside_flag, Grid* g) {
  GEO_BEGIN
  Box b = full_box(g);
  const int64_t n = b.npts();
  Dev dphi(n * 8), tmp(n * 8);
  for (int l = 0; l < num; l++) {
    double px[6], py[6], pz[6], nxv[6], nyv[6], nzv[6];
    for (int q = 0; q < 6; q++) {
      const bool low = q < 3;
      const int ax = q % 3;
      px[q] = low ? cx[l] : cx[l] + sx[l];
      py[q] = low ? cy[l] : cy[l] + sy[l];
      pz[q] = low ? cz[l] : cz[l] + sz[l];
      const double s = low ? -1 : 1;
      nxv[q] = ax == 0 ? s : 0;
      nyv[q] = ax == 1 ? s : 0;
      nzv[q] = ax == 2 ? s : 0;
    }
    halfspaces_into(tmp.as<double>(), b, g, 6, nxv, nyv, nzv, px, py, pz);
    if (inside_flag[l] >= 1) launch_negate(nullptr, n, tmp.as<double>());
    if (l == 0) QSS_CK(cudaMemcpy(dphi.p, tmp.p, n * 8, cudaMemcpyDeviceToDevice));
    else launch_max_into(nullptr, n, dphi.as<double>(), tmp.as<double>(), dphi.as<double>());
  }
  QSS_CK(cudaGetLastError());
  QSS_CK(cudaMemcpy(phi, dphi.p, n * 8, cudaMemcpyDeviceToHost));
  GEO_END
}

void createBox(double* phi, double cx, double cy, double cz, double sx, double sy, double sz, int inside_flag,
               Grid* g) {
  createIntersectionOfBoxes(phi, 1, &cx, &cy, &cz, &sx, &sy, &sz, &inside_flag, g);
}

}  // extern "C"
