// qss_kernels.cuh -- launch interface of the GB300 kernels of the level-set path.
// All launches are asynchronous on the given stream; every pointer is device memory.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstring>
#include "qss_device.cuh"

namespace qss {

// Device-resident control block of the pseudo-time inner loop.  It replaces
// the host-side `while (dt_sub < tplot)` of constCurvModel3d.c:127 so that a
// batch of inner steps can be queued without a host round trip per step: the
// dt kernel of each step re-evaluates the loop condition and every later
// kernel of the step is a no-op once it is false.
struct Ctl {
  double dt;             // dt of the current step
  double dt_sub;         // accumulated pseudo time of this outer iteration
  double tplot;          // loop bound
  double b_max_over_dx;  // CFL terms from the options
  double max_U_over_dx;
  double cur_max_H;      // CFL estimate used for the current step
  int active;            // 1 while the loop condition holds
  int steps;             // inner steps executed
  int max_steps;         // optional cap on steps (0 = none), used by benchmarks
  int err;               // sticky error flags (QSSGPU_ERR_*)
};

enum { ERR_UF_LIMIT = 1, ERR_BAD_ARG = 2 };

// Coefficients of the right-hand side: arrays (variable model) or scalars.
struct Coef {
  const double* vel_n;
  const double* b;
  const double* vx;
  const double* vy;
  const double* vz;
  double a_const, b_const;
  const int* nsrc;  // per voxel: source voxel of the carried normal term, -1 for none
};

struct ImposeArgs {
  const double* mask;
  const double* mask_w;
  const double* mask_nw;
  double overlap;
  int check_conn;
};

#ifdef __CUDACC__
// the three mask impositions of one voxel (level_set_evolution/constCurvModel3d.c:228-241)
__device__ __forceinline__ double impose3(double v, int64_t idx, const ImposeArgs& im) {
  double t = im.mask[idx] - im.overlap;
  v = (t > v) ? t : v;
  if (im.check_conn) {
    t = im.mask_w[idx] - 0.0;
    v = (t > v) ? t : v;
    t = im.mask_nw[idx] - 0.0;
    v = (t > v) ? t : v;
  }
  return v;
}
#endif

// ---- inner step ---------------------------------------------------------
// dt kernel: CFL estimate at the last voxel of each of `nslabs` z-slabs of the
// stage-1 input, dt, loop condition.
void launch_dt(cudaStream_t s, int scheme, bool var, const Box& b, const double* phi, const Coef& c,
               int nslabs, double dx, double dy, double dz, Ctl* ctl);

// stage kernel.  stage: 0 = RHS only (out = rhs), 1 = RK1, 2 = TVD-RK2 stage 2,
// 3 = TVD-RK3 stage 3.  final: also write impose(out) into phi_new (fill box).
// ctl may be null only for stage 0.
void launch_stage(cudaStream_t s, int scheme, bool var, int stage, bool final_stage, const Box& b,
                  double dx, double dy, double dz, const double* phi_in, const double* u_cur,
                  double* out, double* phi_new, const Coef& c, const ImposeArgs& im, const Ctl* ctl);

// emulation level of the split WENO5 kernels (defined in qss_state.cu)
int emu_level();
// form of the WENO5 axis passes at integer-pipe levels >= 1: 0 the sliding
// window in registers, 1 the faces' scaled copies in shared memory with the
// smoothness squares on the integer pipes (faster from ~12 M fill voxels),
// -1 (default) chosen by the launch's size ($QSSGPU_AXIS_VARIANT,
// qssgpu_set_axis_variant); both give identical results
int axis_variant();

// WENO5 variable-coefficient stage as three axis passes (one-sided
// derivatives into dp[axis], dm[axis], ghost-box sized) and a combine kernel
// (qss_weno.cu); same results as launch_stage for scheme WENO5, var = true.
void launch_weno_axes(cudaStream_t s, const Box& b, const double* phi, double dx, double dy, double dz,
                      double* const dp[3], double* const dm[3], const Ctl* ctl);
void launch_weno_combine(cudaStream_t s, int stage, bool final_stage, const Box& b, double dx, double dy, double dz,
                         const double* phi_in, const double* u_cur, double* out, double* phi_new,
                         double* const dp[3], double* const dm[3], const Coef& c, const ImposeArgs& im,
                         const Ctl* ctl);

// CFL estimate of one voxel (for the RHS-only entry points)
void launch_cfl_at(cudaStream_t s, int scheme, bool var, const Box& b, const double* phi, const Coef& c,
                   int i, int j, int k, double dx, double dy, double dz, double* h_out);

// Ghost layers of `a` from its fill box (signed linear extrapolation, all six
// faces).  If phi_new is non-null its ghost points in z-range
// [klo-3, khi+3] receive impose(ghost value).
void launch_ghost(cudaStream_t s, const Box& b, double* a, double* phi_new, const ImposeArgs& im,
                  const Ctl* ctl);

// one face of the signed linear extrapolation (face 0..5 = x-lo, x-hi, y-lo,
// y-hi, z-lo, z-hi), over the full ghost range of the other two axes
void launch_face(cudaStream_t s, const Box& b, double* a, int face);

// Optional timing of every stage-kernel launch with CUDA events on the
// launching stream (used by the benchmark entry point).
// kinds of profiled kernels: fused stage, WENO5 x / y / z passes, combine
enum { kProfStage = 0, kProfAxisX = 1, kProfAxisY = 2, kProfAxisZ = 3, kProfCombine = 4, kProfKinds = 5 };
void qss_profile_stage_begin(cudaStream_t s);
void qss_profile_stage_end(double ms[kProfKinds], int launches[kProfKinds]);
// event before / after one profiled launch on s (no-ops unless s is profiled)
cudaEvent_t prof_open(cudaStream_t s);
void prof_close(cudaStream_t s, cudaEvent_t e0, int kind);

// phi_new = impose(src) over the whole ghost box restricted to z in [klo-3, khi+3]
void launch_impose_region(cudaStream_t s, const Box& b, const double* src, double* phi_new,
                          const ImposeArgs& im, const Ctl* ctl);

// ---- F8: carried normal term ------------------------------------------
// For every fill-box voxel with !(|vel_n| >= 1e-5) store in nsrc the ghost-box
// index of the closest preceding voxel (loop order i, j, k within its z-slab)
// with |vel_n| >= 1e-5, or -1.  Returns the count of such voxels in *d_count.
void launch_nsrc(cudaStream_t s, const Box& b, const double* vel_n, int* nsrc, int nslabs,
                 int* d_rowlast, int* d_carry, unsigned long long* d_count);

// ---- reinitialisation ---------------------------------------------------
void launch_distance0(cudaStream_t s, const Box& b, const double* phi0, double* distance0, double dx,
                      double dy, double dz);
void launch_reinit_step(cudaStream_t s, const Box& b, const double* data, const double* phi0,
                        const double* distance0, double* next, double dt_r, double dx, double dy,
                        double dz);
void launch_reinit_rhs(cudaStream_t s, const Box& b, const double* data, const double* phi0,
                       const double* distance0, double* rhs, double dx, double dy, double dz);

// ---- coefficients -------------------------------------------------------
void launch_central_grad(cudaStream_t s, const Box& b, const double* f, double* fx, double* fy,
                         double* fz, double dx, double dy, double dz);
void launch_setvarnorm(cudaStream_t s, const Box& b, const double* mask, const double* mx,
                       const double* my, const double* mz, double* vel_n, double a0,
                       const double* theta_field, double theta, double dx);
// b_max and max_U written as ordered keys into red[0], red[1] (see key_to_double)
void launch_setvarcurvadv(cudaStream_t s, const Box& b, const double* mask, const double* mx,
                          const double* my, const double* mz, double* vb, double* vx, double* vy,
                          double* vz, double const_b, double dx, unsigned long long* red);
void launch_trapvel(cudaStream_t s, const Box& b, const double* test, double* vel_n, double* vb,
                    double* vx, double* vy, double* vz, double dx);

// ---- whole-array operations (all ghost-box points) -----------------------
void launch_max_into(cudaStream_t s, int64_t n, double* out, const double* mask, const double* phi);
void launch_min_into(cudaStream_t s, int64_t n, double* out, const double* a, const double* b);
void launch_merge(cudaStream_t s, int64_t n, double* phi, const double* m);
void launch_fill(cudaStream_t s, int64_t n, double* out, double v);
void launch_rk(cudaStream_t s, const Box& b, int stage, double* out, const double* u1,
               const double* u0, const double* rhs, double dt);
void launch_impose_slab(cudaStream_t s, const Box& b, double* out, const double* mask,
                        const double* phi, double overlap, int k0, int k1);

// ---- reductions ------------------------------------------------------------
// key encoding of doubles whose unsigned order equals the numeric order
__host__ __device__ inline unsigned long long double_to_key(double v) {
  unsigned long long u;
  memcpy(&u, &v, 8);
  return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}
__host__ __device__ inline double key_to_double(unsigned long long k) {
  unsigned long long u = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
  double v;
  memcpy(&v, &u, 8);
  return v;
}
void launch_maxnormdiff(cudaStream_t s, const Box& b, const double* f1, const double* f2,
                        double zone, unsigned long long* key);
// sequential (loop-order) smoothed volume of {phi < 0}; contrib is fill-box sized scratch
// Smoothed volume of {phi < 0} summed in the reference's loop order;
// scratch holds volume_scratch_doubles(fill-box voxels) doubles.
void launch_volume(cudaStream_t s, const Box& b, const double* phi, double dx, double dy, double dz,
                   double eps, double* scratch, double* out);
// the sequentially rounded sum c[0] + c[1] + ... + c[n-1] (qss_volsum.cu);
// scratch holds loop_sum_scratch_doubles(n) doubles
int64_t loop_sum_scratch_doubles(int64_t n);
void launch_loop_sum(cudaStream_t s, const double* c, int64_t n, double* scratch, double* out);
inline int64_t volume_scratch_doubles(int64_t nfb) { return nfb + loop_sum_scratch_doubles(nfb); }

// ---- geometry ------------------------------------------------------------
void launch_sphere(cudaStream_t s, const Box& b, double* phi, const double* x_lo_gb, const double* dxv,
                   double cx, double cy, double cz, double r, int inside_flag);
void launch_box(cudaStream_t s, const Box& b, double* phi, const double* x_lo_gb, const double* dxv,
                const double corner[3], const double side[3], int inside_flag);

// signed distance to the intersection of spheres / half spaces for arrays
// of objects held in device memory (createIntersectionOfSpheres,
// createIntersectionOfHalfSpaces3d)
void launch_spheres(cudaStream_t s, const Box& b, double* phi, const double* x_lo_gb, const double* dxv,
                    const double* cx, const double* cy, const double* cz, const double* r, const int* inside,
                    int num);
void launch_halfspaces(cudaStream_t s, const Box& b, double* phi, const double* x_lo_gb, const double* dxv,
                       const double* nx, const double* ny, const double* nz, const double* px,
                       const double* py, const double* pz, int num);
void launch_negate(cudaStream_t s, int64_t n, double* a);

// ---- connectivity (qss_uf.cu) -----------------------------------------------
// labels[v] = largest ghost-box index of v's 26-connected component of bin,
// 0 for background; ctl->err gets ERR_UF_LIMIT if an iteration cap is hit.
void launch_label(cudaStream_t s, const Box& b, const unsigned char* bin, int* labels, Ctl* ctl);
// bin = (phi < 0) over all points (after MERGE_SETS when merge != null)
void launch_bin_nw(cudaStream_t s, int64_t n, double* phi, const double* mask_nw, unsigned char* bin);
void launch_set_bin_slab(cudaStream_t s, const Box& b, unsigned char* bin, int center_inlet, int outlet);
// mask_nw = -20dx, or -phi where the component is disconnected from `main_idx`;
// scratch = max(mask_nw, max(mask, -phi)); bin = scratch < 0
void launch_trap_nw(cudaStream_t s, int64_t n, const int* labels, int main_idx, const double* phi,
                    const double* mask, double* mask_nw, double* scratch, unsigned char* bin,
                    double fill);
void launch_trap_w(cudaStream_t s, int64_t n, const int* labels, int main_idx, const double* scratch,
                   double* mask_w, double fill);

}  // namespace qss
