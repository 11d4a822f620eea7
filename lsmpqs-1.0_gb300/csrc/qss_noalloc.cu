// qss_noalloc.cu -- an allocation-free variant of the smoothed volume integral.
//
// Some callers of this library must not allocate device memory while they
// run: a host framework that reserved all of HBM up front for its own pool
// allocator (a cudaMalloc then fails, or takes memory the framework planned
// for something else), or one that keeps several streams busy and cannot
// take the device-wide synchronisation that cudaFree implies.  Such callers
// already hold their inputs and outputs in device memory.
// qssgpu_volume_noalloc() serves them: it reads phi from a device pointer,
// writes the volume to a device pointer and keeps its only intermediate data
// -- one contribution per fill-box voxel, summed in the reference's loop
// order -- in the fixed array below.  Under CUDA's default lazy module
// loading the runtime loads this translation unit's module, and so creates
// the array on a device, at the first call on that device (the
// cudaGetSymbolAddress in scratch_on_current_device); with
// CUDA_MODULE_LOADING=EAGER it exists from library load.  Either way it stays
// until the process exits.  Nothing here calls cudaMalloc, cudaFree or any
// allocating library routine.
#include <mutex>

#include "qss_state.h"

using namespace qss;

// Largest fill box accepted: 2^21 voxels (128^3) -> 16 MiB of scratch per GPU
// (one contribution per voxel, plus 8 doubles per chunk of 4096 for the
// parallel loop-order sum and 64 of padding).
#define QSSGPU_NOALLOC_MAX_FB_VOXELS (1 << 21)
#define QSSGPU_NOALLOC_SCRATCH_DOUBLES (QSSGPU_NOALLOC_MAX_FB_VOXELS + 8 * (QSSGPU_NOALLOC_MAX_FB_VOXELS / 4096) + 64)

static __device__ __align__(256) double g_noalloc_contrib[QSSGPU_NOALLOC_SCRATCH_DOUBLES];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
double* g_scratch_addr[kMaxDevices] = {};

// Device address of the scratch array on the current device.  The array's
// name is only a host-side stand-in; the address is looked up once per device
// with that device current and kept for the life of the process (a
// cudaDeviceReset after the first call would leave it stale, so none is
// supported).
double* scratch_on_current_device() {
  int dev = 0;
  QSS_CK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) throw Error(QSSGPU_ERR_UNSUPPORTED, "device index out of range");
  std::lock_guard<std::mutex> lk(g_setup_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    QSS_CK(cudaGetSymbolAddress(&p, g_noalloc_contrib));
    g_scratch_addr[dev] = (double*)p;
  }
  return g_scratch_addr[dev];
}

}  // namespace

extern "C" {

// See include/lsmpqs_gpu.h.
int qssgpu_volume_noalloc(const double* d_phi, const int gb[6], const int ib[6], double dx, double dy, double dz,
                          double epsilon, double* d_volume, void* stream) {
  try {
    ensure_device();
    if (!d_phi || !d_volume || !gb || !ib) throw Error(QSSGPU_ERR_ARG, "qssgpu_volume_noalloc: null argument");
    if (gb[0] != 0 || gb[2] != 0 || gb[4] != 0)
      throw Error(QSSGPU_ERR_UNSUPPORTED, "qssgpu_volume_noalloc: ghost boxes must start at index 0");
    Box b;
    b.nx = gb[1] + 1;
    b.ny = gb[3] + 1;
    b.nz = gb[5] + 1;
    b.ilo = ib[0];
    b.ihi = ib[1];
    b.jlo = ib[2];
    b.jhi = ib[3];
    b.klo = ib[4];
    b.khi = ib[5];
    if (b.nx <= 0 || b.ny <= 0 || b.nz <= 0 || b.ilo < 0 || b.jlo < 0 || b.klo < 0 || b.ihi >= b.nx ||
        b.jhi >= b.ny || b.khi >= b.nz)
      throw Error(QSSGPU_ERR_ARG, "qssgpu_volume_noalloc: box outside the ghost box");
    cudaStream_t s = (cudaStream_t)stream;
    double* scratch = scratch_on_current_device();
    if (b.ihi < b.ilo || b.jhi < b.jlo || b.khi < b.klo) {  // empty box: volume 0
      QSS_CK(cudaMemsetAsync(d_volume, 0, sizeof(double), s));
      return 0;
    }
    const long long nfb = (long long)b.fbx() * b.fby() * b.fbz();
    if (nfb > QSSGPU_NOALLOC_MAX_FB_VOXELS)
      throw Error(QSSGPU_ERR_ARG, "qssgpu_volume_noalloc: the fill box has " + std::to_string(nfb) +
                                      " voxels, more than the fixed scratch holds (" +
                                      std::to_string(QSSGPU_NOALLOC_MAX_FB_VOXELS) +
                                      "); use qss3dvolumeregionphilessthanzero_ for larger boxes");
    // Every scratch entry the sum reads is written first by the contribution
    // and chunk kernels, so nothing has to be cleared between calls.
    static_assert(QSSGPU_NOALLOC_SCRATCH_DOUBLES >= QSSGPU_NOALLOC_MAX_FB_VOXELS + 8 * ((QSSGPU_NOALLOC_MAX_FB_VOXELS + 4095) / 4096) + 64,
                  "scratch below volume_scratch_doubles of the largest box");
    if (volume_scratch_doubles(nfb) > QSSGPU_NOALLOC_SCRATCH_DOUBLES)
      throw Error(QSSGPU_ERR_ARG, "qssgpu_volume_noalloc: scratch too small");
    launch_volume(s, b, d_phi, dx, dy, dz, epsilon, scratch, d_volume);
    QSS_CK(cudaGetLastError());
    return 0;
  } catch (const std::exception& e) {
    return report_exception(e);
  }
}

}  // extern "C"
