// qss_state.h -- device mirror of one QSS_DataArrays and shared host helpers.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <initializer_list>
#include <thread>
#include <utility>
#include <vector>

#include "../../include/lsmpqs_gpu.h"
#include "../../include/lsmpqs_types.h"
#include "qss_kernels.cuh"

namespace qss {

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

// error codes reported by qssgpu_last_error()
enum {
  QSSGPU_OK = 0,
  QSSGPU_ERR_CUDA = 1,
  QSSGPU_ERR_NO_DEVICE = 2,
  QSSGPU_ERR_ARG = 3,
  QSSGPU_ERR_UNSUPPORTED = 4,
  QSSGPU_ERR_DEVICE_CHECK = 5,
};

void set_error(int code, const std::string& msg);
void clear_error();

// Records an exception escaping an entry point as the calling thread's error
// (the library's Error with its code; any other, such as host memory
// exhausted, as QSSGPU_ERR_CUDA) and returns the code.
inline int report_exception(const std::exception& e) {
  const Error* q = dynamic_cast<const Error*>(&e);
  const int code = q && q->code ? q->code : QSSGPU_ERR_CUDA;
  set_error(code, e.what());
  return code;
}

#define QSS_CK(expr)                                                                            \
  do {                                                                                          \
    cudaError_t e_ = (expr);                                                                    \
    if (e_ != cudaSuccess)                                                                      \
      throw ::qss::Error(::qss::QSSGPU_ERR_CUDA,                                                \
                         std::string(#expr) + ": " + cudaGetErrorString(e_));                   \
  } while (0)

void ensure_device();

// Box of a Grid (ghost box origin 0, as every lsmpqs grid has)
Box box_of(const Grid* g);

// Identity of the host arrays of QSS_DataArrays, used to track which host
// arrays must be refreshed from the device when a top-level call returns.
enum HostArray {
  H_PHI, H_PHI_NEXT, H_PHI_EXTRA, H_PHI_PREV, H_MASK, H_LSE_RHS, H_VEL_N, H_BCOEF, H_VX, H_VY, H_VZ,
  H_MASK_X, H_MASK_Y, H_MASK_Z, H_SCRATCH1, H_SCRATCH2, H_CONN, H_BIN, H_MASK_W, H_MASK_NW,
  H_MASK_DISCONN, H_COUNT
};

// Background population of the host pages a call will copy results into.
// A device-to-host copy into anonymous pages that were never written runs at
// the speed of the page faults (~25 GB/s measured on the Grace host, ~190
// GB/s into resident pages), so the outermost call asks the kernel to make
// those pages resident and writable (madvise MADV_POPULATE_WRITE, which
// leaves their contents unchanged) on host threads while the device
// computes.  Kernels without that advice leave the pages as they are.
struct HostPrefault {
  std::vector<std::thread> workers;
  void start(const std::vector<std::pair<void*, size_t>>& ranges);
  void join();
  ~HostPrefault() { join(); }
};

struct DevVolume {
  const QSS_DataArrays* key = nullptr;
  Box box{};
  int64_t n = 0;
  int64_t nfb = 0;
  cudaStream_t stream = nullptr;
  // two more streams and their events for the downloads on return, which then
  // run on several copy engines at once (created with the volume)
  cudaStream_t xfer[2] = {nullptr, nullptr};
  cudaEvent_t xfer_ev[3] = {nullptr, nullptr, nullptr};
  // level set and the two stage buffers
  double *phi = nullptr, *s1 = nullptr, *s2 = nullptr, *phi_prev = nullptr;
  double *mask = nullptr, *mask_w = nullptr, *mask_nw = nullptr, *mask_disconn = nullptr;
  double *mask_x = nullptr, *mask_y = nullptr, *mask_z = nullptr, *phi_extra = nullptr;
  double *vel_n = nullptr, *bcoef = nullptr, *vx = nullptr, *vy = nullptr, *vz = nullptr;
  double *scratch = nullptr;                           // trapped-phase work array
  double *r_phi0 = nullptr, *r_dist = nullptr, *r_next = nullptr;  // reinitialisation
  double *contrib = nullptr;                           // volume contributions (fill box) + sum scratch
  double *dplus[3] = {}, *dminus[3] = {};              // WENO5 one-sided derivatives per axis
  int *labels = nullptr, *nsrc = nullptr, *rowlast = nullptr, *carry = nullptr;
  unsigned char* bin = nullptr;
  unsigned long long* red = nullptr;  // 4 reduction keys
  unsigned long long* count = nullptr;
  double* dscal = nullptr;  // device scalars (volume)
  Ctl* ctl = nullptr;
  Ctl* h_ctl = nullptr;  // pinned mirror
  double* h_scal = nullptr;  // pinned scalars
  // which stage buffer holds the reference's phi_next
  int phi_next_buf = 1;
  // nsrc describes the current vel_n for this many slabs (0 = stale)
  int nsrc_slabs = 0;
  unsigned long long nsrc_invalid = 0;
  // host arrays whose device copy is newer / that must be zero on return
  bool dirty[H_COUNT] = {};
  bool zero_on_return[H_COUNT] = {};
  // statistics of the last top-level call
  long long inner_steps = 0;
  long long outer_iters = 0;
  // host wall time per phase of the last top-level call (PhaseTimer)
  double phase_s[8] = {};
  int phase_open = -1;
  // device time per phase of the last top-level call: a pair of CUDA events
  // recorded on the volume's stream where each phase begins and ends,
  // resolved when the times are asked for
  double phase_dev_s[8] = {};
  std::vector<cudaEvent_t> ev_pool;
  std::vector<std::pair<int, int>> ev_marks;  // (phase, index of the begin event; the end event follows)
  HostPrefault prefault;
};

DevVolume& volume_for(const QSS_DataArrays* p, const Grid* g);
void release_volume(const QSS_DataArrays* p);

// host <-> device copies of one array of the struct
void upload(DevVolume& v, const QSS_DataArrays* p, HostArray which);
void download_dirty(DevVolume& v, QSS_DataArrays* p);
// populates in the background the host pages of the given arrays of p (the
// ones the call will write); download_dirty waits for it
void start_prefault(DevVolume& v, const QSS_DataArrays* p, std::initializer_list<HostArray> which);
// waits for the background population when the call leaves early (error)
struct PrefaultGuard {
  DevVolume& v;
  ~PrefaultGuard() { v.prefault.join(); }
};

int num_slabs_for(const Grid* g);
// throws unless g is a 3-D grid the device path supports (>= 3 ghost layers)
void validate_grid(const Grid* g);
// WENO5 variable-coefficient stages: 0 one fused kernel per stage, 1 (default)
// one kernel per axis + a combine kernel ($QSSGPU_WENO_MODE,
// qssgpu_set_weno_split); both give identical results
int weno_mode();
// share of the WENO5 stage's FP64 arithmetic done on the integer pipes
// (0 none, 1 divisions / power-of-two scalings / comparisons, 2 also part of
// the products and sums; $QSSGPU_EMU, qssgpu_set_emu_level); all levels give
// identical results
int emu_level();

// nesting depth of API calls: only the outermost call moves host data
// Host wall-time accounting of one volume's top-level call, by phase; a
// phase opened inside another is counted in the outer one only.
enum Phase { PH_TOTAL = 0, PH_SETUP, PH_UPLOAD, PH_INNER, PH_TRAP, PH_REINIT, PH_REDUCE, PH_DOWNLOAD };
struct PhaseTimer {
  DevVolume* v;
  int ph;
  double t0;
  int ev = -1;  // index of the begin event in v->ev_pool, -1 when none was recorded
  PhaseTimer(DevVolume& vol, int phase);
  ~PhaseTimer();
};
void reset_phases(DevVolume& v);
// adds the recorded phase events' durations to v.phase_dev_s (waits for them)
void resolve_phase_events(DevVolume& v);

struct CallScope {
  static thread_local int depth;
  CallScope() { depth++; }
  ~CallScope() { depth--; }
  bool outermost() const { return depth == 1; }
};

}  // namespace qss
