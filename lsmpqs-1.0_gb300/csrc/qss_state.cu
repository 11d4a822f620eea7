// qss_state.cu -- device state per QSS_DataArrays, host<->device transfers, errors.
#include <atomic>
#include <chrono>
#include <cstdlib>
#include <cstring>
#include <initializer_list>
#include <mutex>
#include <unordered_map>

#include <sys/mman.h>
#include <unistd.h>

#include "qss_state.h"

namespace qss {

thread_local int CallScope::depth = 0;

namespace {
// error state of the calling thread (the batch entry point reports the
// errors of its worker threads on the caller's)
thread_local int g_err = QSSGPU_OK;
thread_local char g_msg[1024] = "";
std::mutex g_mu;
std::unordered_map<const QSS_DataArrays*, DevVolume*> g_table;
int g_slabs_override = 0;
int g_weno_split = -1;  // -1: from the environment
int g_emu_level = -1;   // -1: from the environment
int g_axis_variant = -1;  // -1: from the environment, else by launch size
}  // namespace

// MADV_POPULATE_WRITE (Linux 5.14); older headers lack the name
#ifdef MADV_POPULATE_WRITE
constexpr int kMadvPopulateWrite = MADV_POPULATE_WRITE;
#else
constexpr int kMadvPopulateWrite = 23;
#endif

static double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// at most this many events per volume and call (a phase beyond it keeps its
// host time only)
constexpr size_t kMaxPhaseEvents = 8192;

PhaseTimer::PhaseTimer(DevVolume& vol, int phase) : v(&vol), ph(phase), t0(0) {
  if (v->phase_open >= 0 && phase != PH_TOTAL) {
    v = nullptr;  // nested: counted in the enclosing phase
    return;
  }
  if (phase != PH_TOTAL) {
    v->phase_open = phase;
    const size_t used = 2 * v->ev_marks.size();
    if (v->stream && used + 2 <= kMaxPhaseEvents) {
      while (v->ev_pool.size() < used + 2) {
        cudaEvent_t e = nullptr;
        if (cudaEventCreate(&e) != cudaSuccess) break;
        v->ev_pool.push_back(e);
      }
      if (v->ev_pool.size() >= used + 2 && cudaEventRecord(v->ev_pool[used], v->stream) == cudaSuccess) {
        ev = (int)used;
        v->ev_marks.emplace_back(phase, ev);
      }
    }
  }
  t0 = now_s();
}

// $QSSGPU_PHASE_SYNC=1 makes every phase end with a stream synchronisation,
// so that asynchronous device work is charged to the phase that queued it
// (diagnostic timing; off by default)
static bool phase_sync() {
  static const int on = [] {
    const char* e = getenv("QSSGPU_PHASE_SYNC");
    return e && atoi(e) == 1 ? 1 : 0;
  }();
  return on != 0;
}

PhaseTimer::~PhaseTimer() {
  if (!v) return;
  if (ev >= 0) cudaEventRecord(v->ev_pool[ev + 1], v->stream);
  if (phase_sync()) cudaStreamSynchronize(v->stream);
  v->phase_s[ph] += now_s() - t0;
  if (ph != PH_TOTAL) v->phase_open = -1;
}

void reset_phases(DevVolume& v) {
  for (double& t : v.phase_s) t = 0;
  for (double& t : v.phase_dev_s) t = 0;
  v.ev_marks.clear();
  v.phase_open = -1;
}

void resolve_phase_events(DevVolume& v) {
  for (const auto& m : v.ev_marks) {
    float ms = 0.f;
    cudaEvent_t b = v.ev_pool[m.second], e = v.ev_pool[m.second + 1];
    if (cudaEventSynchronize(e) == cudaSuccess && cudaEventElapsedTime(&ms, b, e) == cudaSuccess)
      v.phase_dev_s[m.first] += ms * 1e-3;
  }
  v.ev_marks.clear();
  (void)cudaGetLastError();
}

void set_error(int code, const std::string& msg) {
  g_err = code;
  snprintf(g_msg, sizeof g_msg, "%s", msg.c_str());
  fprintf(stderr, "qssgpu error %d: %s\n", code, g_msg);
}

void clear_error() {
  g_err = QSSGPU_OK;
  g_msg[0] = 0;
}

void ensure_device() {
  static std::atomic<int> state{-1};  // -1 unknown, 0 none, 1 ok
  if (state.load() == 1) return;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    state = 0;
    throw Error(QSSGPU_ERR_NO_DEVICE,
                std::string("no CUDA device available for the GB300 level-set library (") +
                    (e != cudaSuccess ? cudaGetErrorString(e) : "0 devices") + ")");
  }
  state = 1;
}

Box box_of(const Grid* g) {
  Box b;
  b.nx = g->grid_dims_ghostbox[0];
  b.ny = g->grid_dims_ghostbox[1];
  b.nz = g->grid_dims_ghostbox[2];
  b.ilo = g->ilo_fb - g->ilo_gb;
  b.ihi = g->ihi_fb - g->ilo_gb;
  b.jlo = g->jlo_fb - g->jlo_gb;
  b.jhi = g->jhi_fb - g->jlo_gb;
  b.klo = g->klo_fb - g->klo_gb;
  b.khi = g->khi_fb - g->klo_gb;
  return b;
}

static void check_grid(const Grid* g) {
  if (!g) throw Error(QSSGPU_ERR_ARG, "Grid is NULL");
  if (g->num_dims != 3) throw Error(QSSGPU_ERR_UNSUPPORTED, "only 3-D grids run on the GPU path");
  Box b = box_of(g);
  if (b.ilo < 3 || b.jlo < 3 || b.klo < 3 || b.nx - 1 - b.ihi < 3 || b.ny - 1 - b.jhi < 3 ||
      b.nz - 1 - b.khi < 3)
    throw Error(QSSGPU_ERR_ARG, "the level-set stencils need at least 3 ghost layers on every face");
  if (b.fbx() < 2 || b.fby() < 2 || b.fbz() < 2)
    throw Error(QSSGPU_ERR_ARG, "the fill box must span at least 2 cells per axis");
  if (b.npts() >= (int64_t)INT32_MAX) throw Error(QSSGPU_ERR_ARG, "ghost box exceeds 2^31 points");
}

void validate_grid(const Grid* g) { check_grid(g); }

int num_slabs_for(const Grid* g) {
  int t = g_slabs_override;
  if (t <= 0) {
    const char* e = getenv("QSSGPU_SLABS");
    t = e ? atoi(e) : 1;
  }
  if (t < 1) t = 1;
  int ns = g->khi_fb - g->klo_fb + 1;
  if (t > ns) t = ns;
  if (t > 1024) t = 1024;
  return t;
}

int weno_mode() {
  int m = g_weno_split;
  if (m < 0) {
    const char* e = getenv("QSSGPU_WENO_MODE");
    m = e ? atoi(e) : 1;
  }
  return m <= 0 ? 0 : 1;
}

int axis_variant() {
  int m = g_axis_variant;
  if (m < 0) {
    const char* e = getenv("QSSGPU_AXIS_VARIANT");
    m = e ? atoi(e) : -1;
  }
  return m < 0 ? -1 : (m > 4 ? 4 : m);
}

int emu_level() {
  int m = g_emu_level;
  if (m < 0) {
    const char* e = getenv("QSSGPU_EMU");
    m = e ? atoi(e) : 2;
  }
  return m < 0 ? 0 : (m > 2 ? 2 : m);
}

template <class T>
static void dalloc(T*& ptr, int64_t count) {
  if (!ptr) QSS_CK(cudaMalloc((void**)&ptr, (size_t)count * sizeof(T)));
}

static void destroy_volume(DevVolume* v) {
  if (v->stream) cudaStreamSynchronize(v->stream);
  void* ptrs[] = {v->phi, v->s1, v->s2, v->phi_prev, v->mask, v->mask_w, v->mask_nw, v->mask_disconn,
                  v->mask_x, v->mask_y, v->mask_z, v->phi_extra, v->vel_n, v->bcoef, v->vx, v->vy,
                  v->vz, v->scratch, v->r_phi0, v->r_dist, v->r_next, v->contrib, v->labels, v->nsrc,
                  v->bin, v->rowlast, v->carry, v->red, v->count, v->dscal, v->ctl};
  for (void* q : ptrs)
    if (q) cudaFree(q);
  for (int d = 0; d < 3; d++) {
    if (v->dplus[d]) cudaFree(v->dplus[d]);
    if (v->dminus[d]) cudaFree(v->dminus[d]);
  }
  for (cudaEvent_t e : v->ev_pool) cudaEventDestroy(e);
  if (v->h_ctl) cudaFreeHost(v->h_ctl);
  if (v->h_scal) cudaFreeHost(v->h_scal);
  for (cudaStream_t x : v->xfer)
    if (x) cudaStreamDestroy(x);
  for (cudaEvent_t e : v->xfer_ev)
    if (e) cudaEventDestroy(e);
  if (v->stream) cudaStreamDestroy(v->stream);
  delete v;
}

static void alloc_volume(DevVolume* v);

static bool same_box(const Box& a, const Box& b) {
  return a.nx == b.nx && a.ny == b.ny && a.nz == b.nz && a.ilo == b.ilo && a.ihi == b.ihi &&
         a.jlo == b.jlo && a.jhi == b.jhi && a.klo == b.klo && a.khi == b.khi;
}

DevVolume& volume_for(const QSS_DataArrays* p, const Grid* g) {
  ensure_device();
  check_grid(g);
  std::lock_guard<std::mutex> lk(g_mu);
  Box b = box_of(g);
  auto it = g_table.find(p);
  if (it != g_table.end()) {
    if (same_box(it->second->box, b)) return *it->second;
    destroy_volume(it->second);  // the grid changed under the same struct
    g_table.erase(it);
  }
  DevVolume* v = new DevVolume();
  v->key = p;
  v->box = b;
  v->n = b.npts();
  v->nfb = (int64_t)b.fbx() * b.fby() * b.fbz();
  try {
    alloc_volume(v);
  } catch (...) {
    // an allocation that failed (device memory exhausted) frees what was
    // already taken and clears the runtime's last error, so that later calls
    // (on smaller volumes, or after a release) start clean
    destroy_volume(v);
    cudaGetLastError();
    throw;
  }
  g_table[p] = v;
  return *v;
}

static void alloc_volume(DevVolume* v) {
  const Box& b = v->box;
  const int64_t n = v->n;
  QSS_CK(cudaStreamCreateWithFlags(&v->stream, cudaStreamNonBlocking));
  for (auto& x : v->xfer) QSS_CK(cudaStreamCreateWithFlags(&x, cudaStreamNonBlocking));
  for (auto& e : v->xfer_ev) QSS_CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  double** reals[] = {&v->phi, &v->s1, &v->s2, &v->phi_prev, &v->mask, &v->mask_w, &v->mask_nw,
                      &v->mask_disconn, &v->mask_x, &v->mask_y, &v->mask_z, &v->phi_extra,
                      &v->vel_n, &v->bcoef, &v->vx, &v->vy, &v->vz, &v->scratch,
                      &v->r_phi0, &v->r_dist, &v->r_next};
  for (double** r : reals) dalloc(*r, n);
  for (int d = 0; d < 3; d++) {
    dalloc(v->dplus[d], n);
    dalloc(v->dminus[d], n);
  }
  dalloc(v->contrib, volume_scratch_doubles(v->nfb));
  dalloc(v->labels, n);
  dalloc(v->nsrc, n);
  dalloc(v->bin, n);
  const int64_t rows = (int64_t)b.fby() * b.fbz();
  dalloc(v->rowlast, rows);
  dalloc(v->carry, rows);
  dalloc(v->red, 4);
  dalloc(v->count, 1);
  dalloc(v->dscal, 8);
  dalloc(v->ctl, 1);
  QSS_CK(cudaMallocHost((void**)&v->h_ctl, sizeof(Ctl)));
  QSS_CK(cudaMallocHost((void**)&v->h_scal, 8 * sizeof(double)));
  QSS_CK(cudaMemsetAsync(v->s1, 0, n * sizeof(double), v->stream));
  QSS_CK(cudaMemsetAsync(v->s2, 0, n * sizeof(double), v->stream));
  QSS_CK(cudaStreamSynchronize(v->stream));
}

void release_volume(const QSS_DataArrays* p) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_table.find(p);
  if (it == g_table.end()) return;
  destroy_volume(it->second);
  g_table.erase(it);
}

static void* host_ptr(const QSS_DataArrays* p, HostArray a) {
  switch (a) {
    case H_PHI: return p->phi;
    case H_PHI_NEXT: return p->phi_next;
    case H_PHI_EXTRA: return p->phi_extra;
    case H_PHI_PREV: return p->phi_prev;
    case H_MASK: return p->mask;
    case H_LSE_RHS: return p->lse_rhs;
    case H_VEL_N: return p->normal_velocity;
    case H_BCOEF: return p->curvature_coeff;
    case H_VX: return p->external_velocity_x;
    case H_VY: return p->external_velocity_y;
    case H_VZ: return p->external_velocity_z;
    case H_MASK_X: return p->mask_x;
    case H_MASK_Y: return p->mask_y;
    case H_MASK_Z: return p->mask_z;
    case H_SCRATCH1: return p->scratch1;
    case H_SCRATCH2: return p->scratch2;
    case H_CONN: return p->connectivity;
    case H_BIN: return p->phi_bin;
    case H_MASK_W: return p->mask_w;
    case H_MASK_NW: return p->mask_nw;
    case H_MASK_DISCONN: return p->mask_disconn_init;
    default: return nullptr;
  }
}

static void* dev_ptr(DevVolume& v, HostArray a) {
  switch (a) {
    case H_PHI: return v.phi;
    case H_PHI_NEXT: return v.phi_next_buf == 1 ? v.s1 : v.s2;
    case H_PHI_EXTRA: return v.phi_extra;
    case H_PHI_PREV: return v.phi_prev;
    case H_MASK: return v.mask;
    case H_VEL_N: return v.vel_n;
    case H_BCOEF: return v.bcoef;
    case H_VX: return v.vx;
    case H_VY: return v.vy;
    case H_VZ: return v.vz;
    case H_MASK_X: return v.mask_x;
    case H_MASK_Y: return v.mask_y;
    case H_MASK_Z: return v.mask_z;
    case H_CONN: return v.labels;
    case H_BIN: return v.bin;
    case H_MASK_W: return v.mask_w;
    case H_MASK_NW: return v.mask_nw;
    case H_MASK_DISCONN: return v.mask_disconn;
    default: return nullptr;  // lse_rhs, scratch1/2 have no device copy
  }
}

static size_t elem_size(HostArray a) {
  if (a == H_CONN) return sizeof(int);
  if (a == H_BIN) return 1;
  return sizeof(double);
}

// arrays the reference only ever writes on the fill box (mask gradient,
// model coefficients, trapped-velocity zeroing)
static bool fill_box_only(HostArray a) {
  switch (a) {
    case H_MASK_X: case H_MASK_Y: case H_MASK_Z: case H_VEL_N: case H_BCOEF: case H_VX: case H_VY: case H_VZ:
      return true;
    default:
      return false;
  }
}

static bool usable(const void* h) {
  return h != nullptr && h != (const void*)(intptr_t)-1;
}

void upload(DevVolume& v, const QSS_DataArrays* p, HostArray which) {
  PhaseTimer pt(v, PH_UPLOAD);
  void* h = host_ptr(p, which);
  void* d = dev_ptr(v, which);
  if (!usable(h) || !d) throw Error(QSSGPU_ERR_ARG, "input array is not allocated");
  QSS_CK(cudaMemcpyAsync(d, h, (size_t)v.n * elem_size(which), cudaMemcpyHostToDevice, v.stream));
}

void HostPrefault::start(const std::vector<std::pair<void*, size_t>>& ranges) {
  join();
  if (ranges.empty()) return;
  const uintptr_t page = (uintptr_t)sysconf(_SC_PAGESIZE);
  const size_t nw = ranges.size() < 2 ? ranges.size() : 2;
  for (size_t w = 0; w < nw; w++) {
    std::vector<std::pair<void*, size_t>> mine;
    for (size_t r = w; r < ranges.size(); r += nw) mine.push_back(ranges[r]);
    workers.emplace_back([mine, page] {
      for (const auto& r : mine) {
        const uintptr_t lo = (uintptr_t)r.first & ~(page - 1);
        const uintptr_t hi = ((uintptr_t)r.first + r.second + page - 1) & ~(page - 1);
        // failure (an older kernel, a mapping that refuses) leaves the pages as they are
        (void)madvise((void*)lo, hi - lo, kMadvPopulateWrite);
      }
    });
  }
}

void HostPrefault::join() {
  for (auto& t : workers)
    if (t.joinable()) t.join();
  workers.clear();
}

void start_prefault(DevVolume& v, const QSS_DataArrays* p, std::initializer_list<HostArray> which) {
  std::vector<std::pair<void*, size_t>> ranges;
  for (HostArray a : which) {
    void* h = host_ptr(p, a);
    if (usable(h)) ranges.emplace_back(h, (size_t)v.n * elem_size(a));
  }
  v.prefault.start(ranges);
}

void download_dirty(DevVolume& v, QSS_DataArrays* p) {
  PhaseTimer pt(v, PH_DOWNLOAD);
  v.prefault.join();
  // the copies go round-robin to the volume's stream and its two transfer
  // streams, which start after everything queued so far and are joined
  // before the return: three copy engines move the arrays at once
  QSS_CK(cudaEventRecord(v.xfer_ev[0], v.stream));
  for (cudaStream_t x : v.xfer) QSS_CK(cudaStreamWaitEvent(x, v.xfer_ev[0], 0));
  const cudaStream_t lanes[3] = {v.stream, v.xfer[0], v.xfer[1]};
  int next = 0;
  auto lane = [&]() { return lanes[next++ % 3]; };
  // arrays the reference leaves zero: copied from a zeroed device buffer (the
  // reinitialisation scratch, free once the call's work is queued) by the
  // copy engine, which writes host memory faster than a CPU memset
  bool zeroed = false;
  for (int a = 0; a < H_COUNT; a++) {
    HostArray w = (HostArray)a;
    void* h = host_ptr(p, w);
    if (!usable(h)) {
      v.dirty[a] = v.zero_on_return[a] = false;
      continue;
    }
    if (v.zero_on_return[a]) {
      const size_t bytes = (size_t)v.n * elem_size(w);  // at most n doubles
      if (!zeroed) {
        // cleared on the volume's stream, then made visible to the other two
        QSS_CK(cudaMemsetAsync(v.r_next, 0, (size_t)v.n * sizeof(double), v.stream));
        QSS_CK(cudaEventRecord(v.xfer_ev[0], v.stream));
        for (cudaStream_t x : v.xfer) QSS_CK(cudaStreamWaitEvent(x, v.xfer_ev[0], 0));
      }
      zeroed = true;
      QSS_CK(cudaMemcpyAsync(h, v.r_next, bytes, cudaMemcpyDeviceToHost, lane()));
    } else if (v.dirty[a]) {
      void* d = dev_ptr(v, w);
      if (!d) continue;
      if (fill_box_only(w)) {
        // the reference writes these arrays on the fill box only: the caller's
        // ghost values must survive, so only fill-box rows travel
        const Box& b = v.box;
        const size_t pitch = (size_t)b.nx * sizeof(double);
        const cudaStream_t st = lane();
        for (int k = b.klo; k <= b.khi; k++) {
          const size_t off = (size_t)b.idx(b.ilo, b.jlo, k) * sizeof(double);
          QSS_CK(cudaMemcpy2DAsync((char*)h + off, pitch, (const char*)d + off, pitch,
                                   (size_t)b.fbx() * sizeof(double), (size_t)b.fby(), cudaMemcpyDeviceToHost,
                                   st));
        }
      } else {
        QSS_CK(cudaMemcpyAsync(h, d, (size_t)v.n * elem_size(w), cudaMemcpyDeviceToHost, lane()));
      }
    }
    v.dirty[a] = v.zero_on_return[a] = false;
  }
  for (int x = 0; x < 2; x++) {
    QSS_CK(cudaEventRecord(v.xfer_ev[1 + x], v.xfer[x]));
    QSS_CK(cudaStreamWaitEvent(v.stream, v.xfer_ev[1 + x], 0));
  }
  QSS_CK(cudaStreamSynchronize(v.stream));
}

}  // namespace qss

using namespace qss;

extern "C" {

int qssgpu_last_error(void) { return g_err; }
const char* qssgpu_error_string(void) { return g_msg; }
void qssgpu_clear_error(void) { clear_error(); }

void qssgpu_set_slabs(int nslabs) { g_slabs_override = nslabs; }

int qssgpu_set_emu_level(int level) {
  const int prev = emu_level();
  g_emu_level = level < 0 ? -1 : (level > 2 ? 2 : level);
  return prev;
}

int qssgpu_set_axis_variant(int v) {
  const int prev = axis_variant();
  g_axis_variant = v < 0 ? -1 : (v > 4 ? 4 : v);
  return prev;
}

int qssgpu_set_weno_split(int mode) {
  const int prev = weno_mode();
  g_weno_split = mode < 0 ? -1 : (mode ? 1 : 0);
  return prev;
}

int qssgpu_get_slabs(const Grid* g) { return g ? num_slabs_for(g) : g_slabs_override; }

void qssgpu_release(QSS_DataArrays* p) { release_volume(p); }

// See include/lsmpqs_gpu.h.
void* qssgpu_host_alloc(size_t bytes) {
  try {
    ensure_device();
    void* h = nullptr;
    QSS_CK(cudaHostAlloc(&h, bytes ? bytes : 1, cudaHostAllocDefault));
    memset(h, 0, bytes);
    return h;
  } catch (const Error& e) {
    set_error(e.code, e.what());
    return nullptr;
  }
}

// See include/lsmpqs_gpu.h.
void qssgpu_host_free(void* h) {
  if (h) cudaFreeHost(h);
}

int qssgpu_device_available(void) {
  try {
    ensure_device();
    return 1;
  } catch (const Error&) {
    return 0;
  }
}

}  // extern "C"
