// qss_prepost.cu -- pre- and post-processing of the level-set path on the GPU.
//
//   qss_reinitialize_mask         src/utilities/qss_general_util.c:261-306
//   qssgpu_create_mask_ubc        src/applications/createMaskUBC.c:76-112
//   qssgpu_create_init_from_mask  src/applications/createInitFromMask.c:55-85 (3-D)
//   qssgpu_diff_steps             src/applications/makeDiffSteps.c:54-132 (3-D)
//   qssgpu_phase_uchar            src/applications/makeRaw.c:52-135 (phase images)
//
// The reference runs these as command-line programs (or, for the mask
// reinitialisation, a library routine they call); here each is one library
// call on host arrays whose work runs on the device, so that large images are
// converted, initialised and post-processed without the serial host loops.
// Every function writes exactly the arrays (and ranges) the reference writes,
// with the reference's operations in the same order.
#include <cmath>
#include <vector>

#include "qss_state.h"

using namespace qss;

namespace {

__global__ void k_ubc_mask(Box b, const unsigned char* __restrict__ ubc, double dx, double* mask) {
  const int64_t n = b.npts();
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(q % b.nx);
    const int64_t r = q / b.nx;
    const int j = (int)(r % b.ny), k = (int)(r / b.ny);
    double v = 0.0;  // ghost layers: a freshly allocated (zeroed) array
    if (i >= b.ilo && i <= b.ihi && j >= b.jlo && j <= b.jhi && k >= b.klo && k <= b.khi) {
      const int64_t s = (i - b.ilo) + (int64_t)b.fbx() * ((j - b.jlo) + (int64_t)b.fby() * (k - b.klo));
      v = (ubc[s] == 255) ? dx : -dx;  // 255 = grain
    }
    mask[q] = v;
  }
}

// makeDiffSteps.c:62-72: mask = -phi_a, phi = max(mask, phi_b - dx/2),
// phi_bin = phi < 0
__global__ void k_diff(int64_t n, const double* __restrict__ a, const double* __restrict__ bstep, double half_dx,
                       double* phi, unsigned char* bin) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
    const double m = -a[q];
    double p = bstep[q];
    p -= half_dx;
    p = (m > p) ? m : p;
    phi[q] = p;
    bin[q] = (p < 0.0) ? 1 : 0;
  }
}

// makeRaw's 0/1 phase images: bin = (f < 0) (IMPOSE_UCHAR, qss_macros.h:97-104)
// of f = mask (phase 'm', makeRaw.c:96), phi ('n', :107) or max(mask, -phi)
// ('w': COPY_DATA, NEGATE_DATA, IMPOSE_MASK, :123-128, qss_macros.h:56-86);
// the ghost-box image and/or the fill box packed i fastest (copyDataFB,
// makeRaw.c:52-73)
__global__ void k_phase_uchar(Box b, const double* __restrict__ phi, const double* __restrict__ mask, int phase,
                              unsigned char* full, unsigned char* fb) {
  const int64_t n = b.npts();
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
    double f;
    if (phase == 'm') {
      f = mask[q];
    } else if (phase == 'n') {
      f = phi[q];
    } else {
      const double s = -phi[q];
      const double m = mask[q];
      f = (m > s) ? m : s;
    }
    const unsigned char v = (f < 0) ? 1 : 0;
    if (full) full[q] = v;
    if (fb) {
      const int i = (int)(q % b.nx);
      const int64_t r = q / b.nx;
      const int j = (int)(r % b.ny), k = (int)(r / b.ny);
      if (i >= b.ilo && i <= b.ihi && j >= b.jlo && j <= b.jhi && k >= b.klo && k <= b.khi)
        fb[(i - b.ilo) + (int64_t)b.fbx() * ((j - b.jlo) + (int64_t)b.fby() * (k - b.klo))] = v;
    }
  }
}

// the inlet and outlet slabs of ones (makeDiffSteps.c:78-97)
__global__ void k_diff_slabs(Box b, unsigned char* bin) {
  const int64_t cnt = (int64_t)b.fby() * b.fbz();
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= cnt) return;
  const int j = b.jlo + (int)(t % b.fby()), k = b.klo + (int)(t / b.fby());
  bin[b.idx(b.ilo - 1, j, k)] = 1;
  bin[b.idx(b.ihi + 1, j, k)] = 1;
}

// makeDiffSteps.c:117-122: flip the sign of the non-wetting voxels that are
// not in the main (percolating) component
__global__ void k_diff_connected(int64_t n, const int* __restrict__ labels, int main_label, double* phi) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
    if ((labels[q] != main_label) & (phi[q] <= 0)) phi[q] *= -1;
  }
}

unsigned g1(int64_t n) {
  int64_t b = (n + 255) / 256;
  if (b > 152 * 16) b = 152 * 16;
  return (unsigned)(b < 1 ? 1 : b);
}

struct Buf {
  std::vector<void*> ptrs;
  template <class T>
  T* get(int64_t n) {
    void* p = nullptr;
    QSS_CK(cudaMalloc(&p, (size_t)(n > 0 ? n : 1) * sizeof(T)));
    ptrs.push_back(p);
    return (T*)p;
  }
  ~Buf() {
    for (void* p : ptrs) cudaFree(p);
  }
};

struct Stream {
  cudaStream_t s = nullptr;
  Stream() { QSS_CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking)); }
  ~Stream() {
    if (s) cudaStreamDestroy(s);
  }
};

void h2d(cudaStream_t s, void* d, const void* h, size_t bytes) {
  QSS_CK(cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, s));
}
void d2h(cudaStream_t s, void* h, const void* d, size_t bytes) {
  QSS_CK(cudaMemcpyAsync(h, d, bytes, cudaMemcpyDeviceToHost, s));
}

bool usable(const void* p) { return p != nullptr; }

// qss_reinitialize_mask on device copies of the arrays it uses
void reinit_mask_dev(cudaStream_t s, const Box& b, const Grid* g, const Options* o, double* mask, double* scratch1,
                     double* scratch2, double* rhs, double* next) {
  const int64_t n = b.npts();
  const double dx = g->dx[0], dy = g->dx[1], dz = g->dx[2];
  const double dt_r = 0.5 * g->dx[0];  // cfl_number 0.5
  QSS_CK(cudaMemcpyAsync(scratch2, mask, n * sizeof(double), cudaMemcpyDeviceToDevice, s));  // COPY_DATA
  launch_distance0(s, b, scratch2, scratch1, dx, dy, dz);
  ImposeArgs none{};
  double t_r = 0;
  while (t_r < o->tmax_r) {
    launch_reinit_rhs(s, b, mask, scratch2, scratch1, rhs, dx, dy, dz);
    launch_rk(s, b, 1, next, mask, nullptr, rhs, dt_r);
    launch_ghost(s, b, next, nullptr, none, nullptr);  // signedLinearExtrapolationBCqss(., 9)
    QSS_CK(cudaMemcpyAsync(mask, next, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
    t_r = t_r + dt_r;
  }
}

}  // namespace

extern "C" {

// qss_general_util.h: the mask reinitialisation (its side effects on
// scratch1 = distance0, scratch2 = the initial mask, lse_rhs and phi_next
// included)
void qss_reinitialize_mask(QSS_DataArrays* p, Grid* g, Options* o) {
  try {
    ensure_device();
    validate_grid(g);
    if (!p || !o || !usable(p->mask) || !usable(p->scratch1) || !usable(p->scratch2) || !usable(p->lse_rhs) ||
        !usable(p->phi_next))
      throw Error(QSSGPU_ERR_ARG, "qss_reinitialize_mask: arrays not allocated");
    const Box b = box_of(g);
    const int64_t n = b.npts();
    const size_t bytes = (size_t)n * sizeof(double);
    Stream st;
    Buf buf;
    double *mask = buf.get<double>(n), *s1 = buf.get<double>(n), *s2 = buf.get<double>(n),
           *rhs = buf.get<double>(n), *next = buf.get<double>(n);
    h2d(st.s, mask, p->mask, bytes);
    h2d(st.s, s1, p->scratch1, bytes);
    h2d(st.s, rhs, p->lse_rhs, bytes);
    h2d(st.s, next, p->phi_next, bytes);
    reinit_mask_dev(st.s, b, g, o, mask, s1, s2, rhs, next);
    d2h(st.s, p->mask, mask, bytes);
    d2h(st.s, p->scratch1, s1, bytes);
    d2h(st.s, p->scratch2, s2, bytes);
    d2h(st.s, p->lse_rhs, rhs, bytes);
    d2h(st.s, p->phi_next, next, bytes);
    QSS_CK(cudaStreamSynchronize(st.s));
  } catch (const std::exception& e) {
    report_exception(e);
  }
}

// See include/lsmpqs_gpu.h.
int qssgpu_create_mask_ubc(const unsigned char* ubc, QSS_DataArrays* p, Grid* g, Options* o) {
  try {
    ensure_device();
    validate_grid(g);
    if (!ubc || !p || !o || !usable(p->mask) || !usable(p->scratch1) || !usable(p->scratch2) ||
        !usable(p->lse_rhs) || !usable(p->phi_next))
      throw Error(QSSGPU_ERR_ARG, "qssgpu_create_mask_ubc: bad arguments");
    const Box b = box_of(g);
    const int64_t n = b.npts(), nfb = (int64_t)b.fbx() * b.fby() * b.fbz();
    const size_t bytes = (size_t)n * sizeof(double);
    Stream st;
    Buf buf;
    unsigned char* img = buf.get<unsigned char>(nfb);
    double *mask = buf.get<double>(n), *s1 = buf.get<double>(n), *s2 = buf.get<double>(n),
           *rhs = buf.get<double>(n), *next = buf.get<double>(n);
    h2d(st.s, img, ubc, (size_t)nfb);
    h2d(st.s, s1, p->scratch1, bytes);
    h2d(st.s, rhs, p->lse_rhs, bytes);
    h2d(st.s, next, p->phi_next, bytes);
    k_ubc_mask<<<g1(n), 256, 0, st.s>>>(b, img, o->dx, mask);
    reinit_mask_dev(st.s, b, g, o, mask, s1, s2, rhs, next);
    d2h(st.s, p->mask, mask, bytes);
    d2h(st.s, p->scratch1, s1, bytes);
    d2h(st.s, p->scratch2, s2, bytes);
    d2h(st.s, p->lse_rhs, rhs, bytes);
    d2h(st.s, p->phi_next, next, bytes);
    QSS_CK(cudaStreamSynchronize(st.s));
    return 0;
  } catch (const std::exception& e) {
    return report_exception(e);
  }
}

// See include/lsmpqs_gpu.h.
int qssgpu_create_init_from_mask(QSS_DataArrays* p, Grid* g, Options* o) {
  try {
    ensure_device();
    validate_grid(g);
    if (!p || !o || !usable(p->mask) || !usable(p->phi))
      throw Error(QSSGPU_ERR_ARG, "qssgpu_create_init_from_mask: bad arguments");
    const Box b = box_of(g);
    const int64_t n = b.npts();
    const size_t bytes = (size_t)n * sizeof(double);
    double radius, cx, cy, cz;
    if (o->center_inlet) {
      radius = 90 * g->dx[0];
      cy = 0.5 * (g->x_lo[1] + g->x_hi[1]);
      cx = 0.5 * (g->x_lo[1] + g->x_hi[1]);  // as the reference writes it (x from the y bounds)
      cz = 0.5 * (g->x_lo[2] + g->x_hi[2]);
    } else {
      radius = 0.7 * (g->x_hi[0] - g->x_lo[0]);
      cy = 0.5 * (g->x_lo[1] + g->x_hi[1]);
      cx = (g->x_lo[0]) - radius * 0.7;
      cz = 0.5 * (g->x_lo[2] + g->x_hi[2]);
    }
    Stream st;
    Buf buf;
    double *mask = buf.get<double>(n), *phi = buf.get<double>(n);
    h2d(st.s, mask, p->mask, bytes);
    launch_sphere(st.s, b, phi, g->x_lo_ghostbox, g->dx, cx, cy, cz, radius, -1);  // createSphere(.., -1, g)
    launch_max_into(st.s, n, phi, mask, phi);                                        // IMPOSE_MASK
    d2h(st.s, p->phi, phi, bytes);
    QSS_CK(cudaStreamSynchronize(st.s));
    return 0;
  } catch (const std::exception& e) {
    return report_exception(e);
  }
}

// See include/lsmpqs_gpu.h.
int qssgpu_diff_steps(const double* step_a, const double* step_b, Grid* g, double* diff, double* connected,
                      int* percolates) {
  try {
    ensure_device();
    validate_grid(g);
    if (!step_a || !step_b || !diff || !percolates) throw Error(QSSGPU_ERR_ARG, "qssgpu_diff_steps: bad arguments");
    const Box b = box_of(g);
    const int64_t n = b.npts();
    const size_t bytes = (size_t)n * sizeof(double);
    Stream st;
    Buf buf;
    double *a = buf.get<double>(n), *bb = buf.get<double>(n), *phi = buf.get<double>(n);
    unsigned char* bin = buf.get<unsigned char>(n);
    int* labels = buf.get<int>(n);
    Ctl* ctl = buf.get<Ctl>(1);
    QSS_CK(cudaMemsetAsync(ctl, 0, sizeof(Ctl), st.s));
    h2d(st.s, a, step_a, bytes);
    h2d(st.s, bb, step_b, bytes);
    k_diff<<<g1(n), 256, 0, st.s>>>(n, a, bb, 0.5 * g->dx[0], phi, bin);
    d2h(st.s, diff, phi, bytes);
    const int64_t cnt = (int64_t)b.fby() * b.fbz();
    k_diff_slabs<<<(unsigned)((cnt + 255) / 256), 256, 0, st.s>>>(b, bin);
    launch_label(st.s, b, bin, labels, ctl);
    // inlet (ilo_fb - 1, mid j, mid k) and outlet (ihi_fb + 1, mid j, mid k)
    const int j = (int)(0.5 * (g->jlo_fb + g->jhi_fb)), k = (int)(0.5 * (g->klo_fb + g->khi_fb));
    const int64_t inlet = b.idx(b.ilo - 1, j - g->jlo_gb, k - g->klo_gb);
    const int64_t outlet = b.idx(b.ihi + 1, j - g->jlo_gb, k - g->klo_gb);
    int li = 0, lo = 0;
    d2h(st.s, &li, labels + inlet, sizeof(int));
    d2h(st.s, &lo, labels + outlet, sizeof(int));
    Ctl hc;
    d2h(st.s, &hc, ctl, sizeof(Ctl));
    QSS_CK(cudaStreamSynchronize(st.s));
    if (hc.err) throw Error(QSSGPU_ERR_DEVICE_CHECK, "qssgpu_diff_steps: labelling check failed");
    *percolates = (li == lo) ? 1 : 0;
    if (*percolates && connected) {
      k_diff_connected<<<g1(n), 256, 0, st.s>>>(n, labels, li, phi);
      d2h(st.s, connected, phi, bytes);
      QSS_CK(cudaStreamSynchronize(st.s));
    }
    return 0;
  } catch (const std::exception& e) {
    return report_exception(e);
  }
}

// See include/lsmpqs_gpu.h.
int qssgpu_phase_uchar(const double* phi, const double* mask, Grid* g, char phase, unsigned char* bin_full,
                       unsigned char* bin_fb) {
  try {
    ensure_device();
    validate_grid(g);
    const bool need_phi = phase == 'n' || phase == 'w', need_mask = phase == 'm' || phase == 'w';
    if ((phase != 'm' && phase != 'n' && phase != 'w') || (need_phi && !phi) || (need_mask && !mask) ||
        (!bin_full && !bin_fb))
      throw Error(QSSGPU_ERR_ARG, "qssgpu_phase_uchar: bad arguments");
    const Box b = box_of(g);
    const int64_t n = b.npts(), nfb = (int64_t)b.fbx() * b.fby() * b.fbz();
    const size_t bytes = (size_t)n * sizeof(double);
    Stream st;
    Buf buf;
    double* dphi = need_phi ? buf.get<double>(n) : nullptr;
    double* dmask = need_mask ? buf.get<double>(n) : nullptr;
    unsigned char* dfull = bin_full ? buf.get<unsigned char>(n) : nullptr;
    unsigned char* dfb = bin_fb ? buf.get<unsigned char>(nfb) : nullptr;
    if (dphi) h2d(st.s, dphi, phi, bytes);
    if (dmask) h2d(st.s, dmask, mask, bytes);
    k_phase_uchar<<<g1(n), 256, 0, st.s>>>(b, dphi, dmask, phase, dfull, dfb);
    if (dfull) d2h(st.s, bin_full, dfull, (size_t)n);
    if (dfb) d2h(st.s, bin_fb, dfb, (size_t)nfb);
    QSS_CK(cudaStreamSynchronize(st.s));
    return 0;
  } catch (const std::exception& e) {
    return report_exception(e);
  }
}

}  // extern "C"
