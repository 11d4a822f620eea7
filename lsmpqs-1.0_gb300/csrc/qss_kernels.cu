// qss_kernels.cu -- GB300 (sm_103a) kernels of the quasi-static level-set path.
//
// FP64 throughout, compiled with --fmad=false so that each kernel reproduces
// the reference's Fortran arithmetic bit for bit (see qss_device.cuh).  On
// GB300 the FP64 pipe, not HBM, bounds the WENO5 stage kernel; the kernels
// therefore skip work the reference throws away (the per-voxel CFL estimate
// of which only the last voxel survives, 3d.f:490) and read the stencil
// through the read-only cache (the 7/5-point lines along x, y, z and the
// 12 mixed-derivative neighbours are shared between adjacent threads).
#include <cfloat>
#include <cstdlib>
#include <cstdio>
#include <utility>
#include <vector>
#include "qss_emu.cuh"
#include "qss_kernels.cuh"

namespace qss {

namespace {

constexpr double kZeroTol = 1.e-5;

inline dim3 fb_grid(const Box& b, dim3 blk) {
  return dim3((b.fbx() + blk.x - 1) / blk.x, (b.fby() + blk.y - 1) / blk.y, (b.fbz() + blk.z - 1) / blk.z);
}

inline unsigned blocks_for(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

// ---------------------------------------------------------------------------
// inner step: dt

template <int SCHEME, bool VAR>
__global__ void k_dt(Box b, const double* __restrict__ phi, Coef c, int nslabs, double dx, double dy,
                     double dz, Ctl* ctl) {
  __shared__ double sh[32];
  if (!ctl->active) return;
  const Inv inv{1.0 / dx, 1.0 / dy, 1.0 / dz};
  const int t = threadIdx.x;
  double h = -1.0;
  if (t < nslabs) {
    int ns = b.khi - b.klo + 1;
    int k = b.klo + (int)(((int64_t)ns * (t + 1)) / nslabs) - 1;
    if (k > b.khi) k = b.khi;
    int i = b.ihi, j = b.jhi;
    double pp[3], pm[3];
    upwind<SCHEME>(phi, b, i, j, k, inv, pp, pm);
    double vel = VAR ? c.vel_n[b.idx(i, j, k)] : c.a_const;
    h = cfl_h(vel, pp, pm, dx, dy, dz, inv);
  }
  // max over slabs (the reference's critical section), -1 if none
  for (int o = 16; o > 0; o >>= 1) h = dmax(h, __shfl_down_sync(0xffffffffu, h, o));
  if ((t & 31) == 0) sh[t >> 5] = h;
  __syncthreads();
  if (t == 0) {
    double m = -1.0;
    for (int w = 0; w < (int)((blockDim.x + 31) >> 5); w++) m = dmax(m, sh[w]);
    // loop condition of constCurvModel3d.c:127, evaluated before the step
    bool go = ctl->dt_sub < ctl->tplot;
    if (ctl->max_steps > 0 && ctl->steps >= ctl->max_steps) go = false;
    if (!go) {
      ctl->active = 0;
      return;
    }
    double cur = -1.0;
    if (m > cur) cur = m;
    double dt = 0.5 / (cur + ctl->b_max_over_dx + ctl->max_U_over_dx);
    ctl->cur_max_H = cur;
    ctl->dt = dt;
    ctl->dt_sub = ctl->dt_sub + dt;
    ctl->steps = ctl->steps + 1;
  }
}

// ---------------------------------------------------------------------------
// inner step: stage kernel (RHS fused with the TVD-RK combination and, for the
// last stage, with the three mask impositions)

struct StageArgs {
  Box b;
  Inv inv;
  Fac fac;
  const double* phi_in;
  const double* u_cur;
  double* out;
  double* phi_new;
  Coef c;
  ImposeArgs im;
  const Ctl* ctl;
};

template <int SCHEME, bool VAR, int STAGE, bool FINAL>
__global__ void __launch_bounds__(128) k_stage(StageArgs a) {
  if (STAGE != 0 && !a.ctl->active) return;
  const Box& b = a.b;
  const int i = b.ilo + blockIdx.x * blockDim.x + threadIdx.x;
  const int j = b.jlo + blockIdx.y * blockDim.y + threadIdx.y;
  const int k = b.klo + blockIdx.z * blockDim.z + threadIdx.z;
  if (i > b.ihi || j > b.jhi || k > b.khi) return;
  const int64_t idx = b.idx(i, j, k);
  const double* __restrict__ phi = a.phi_in;

  double pp[3], pm[3];
  upwind<SCHEME>(phi, b, i, j, k, a.inv, pp, pm);

  // Godunov normal term.  A voxel whose |vel_n| is below the tolerance keeps
  // the term of the closest preceding voxel of its slab (3d.f:459-486).
  const double vel = VAR ? a.c.vel_n[idx] : a.c.a_const;
  double temp_norm;
  if (fabs(vel) >= kZeroTol) {
    temp_norm = godunov_norm<SCHEME>(vel, pp, pm);
  } else if (VAR) {
    const int src = a.c.nsrc[idx];
    if (src < 0) {
      temp_norm = 0.0;
    } else {
      const int is = src % b.nx, js = (src / b.nx) % b.ny, ks = src / (b.nx * b.ny);
      double qp[3], qm[3];
      upwind<SCHEME>(phi, b, is, js, ks, a.inv, qp, qm);
      temp_norm = godunov_norm<SCHEME>(a.c.vel_n[src], qp, qm);
    }
  } else {
    temp_norm = 0.0;
  }

  double rhs;
  if (VAR) {
    const double vx = a.c.vx[idx], vy = a.c.vy[idx], vz = a.c.vz[idx];
    const double ax = (vx >= 0) ? pm[0] : pp[0];
    const double ay = (vy >= 0) ? pm[1] : pp[1];
    const double az = (vz >= 0) ? pm[2] : pp[2];
    const double temp_vel = -(vx * ax + vy * ay + vz * az);
    const double temp_curv = a.c.b[idx] * curvature(phi, b, idx, a.fac);
    rhs = temp_norm + temp_curv + temp_vel;
  } else {
    const double temp_curv = a.c.b_const * curvature(phi, b, idx, a.fac);
    rhs = temp_norm + temp_curv;
  }

  double out;
  if (STAGE == 0) {
    out = rhs;
  } else {
    const double dt = a.ctl->dt;
    if (STAGE == 1) {
      out = phi[idx] + dt * rhs;
    } else if (STAGE == 2) {
      out = 0.75 * a.u_cur[idx] + 0.25 * (phi[idx] + dt * rhs);
    } else {
      const double one_third = 1.0 / 3.0, two_thirds = 2.0 / 3.0;
      out = one_third * a.u_cur[idx] + two_thirds * (phi[idx] + dt * rhs);
    }
  }
  a.out[idx] = out;
  if (FINAL) a.phi_new[idx] = impose3(out, idx, a.im);
}

template <int SCHEME, bool VAR>
__global__ void k_cfl_at(Box b, const double* __restrict__ phi, Coef c, int i, int j, int k, double dx,
                         double dy, double dz, double* h_out) {
  const Inv inv{1.0 / dx, 1.0 / dy, 1.0 / dz};
  double pp[3], pm[3];
  upwind<SCHEME>(phi, b, i, j, k, inv, pp, pm);
  double vel = VAR ? c.vel_n[b.idx(i, j, k)] : c.a_const;
  *h_out = cfl_h(vel, pp, pm, dx, dy, dz, inv);
}

// ---------------------------------------------------------------------------
// ghost layers

__global__ void k_ghost(Box b, double* a, double* phi_new, ImposeArgs im, const Ctl* ctl) {
  if (ctl && !ctl->active) return;
  const int64_t nxy = (int64_t)b.nx * b.ny;
  const int nzg = b.klo + (b.nz - 1 - b.khi);    // z-ghost planes
  const int nyg = b.jlo + (b.ny - 1 - b.jhi);    // y-ghost rows per plane
  const int nxg = b.ilo + (b.nx - 1 - b.ihi);    // x-ghost points per row
  const int64_t nz_cells = (int64_t)nzg * nxy;
  const int64_t ny_cells = (int64_t)b.fbz() * nyg * b.nx;
  const int64_t nx_cells = (int64_t)b.fbz() * b.fby() * nxg;
  const int64_t total = nz_cells + ny_cells + nx_cells;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < total;
       q += (int64_t)gridDim.x * blockDim.x) {
    int i, j, k;
    if (q < nz_cells) {
      int p = (int)(q / nxy);
      int64_t r = q - (int64_t)p * nxy;
      k = (p < b.klo) ? p : b.khi + 1 + (p - b.klo);
      j = (int)(r / b.nx);
      i = (int)(r - (int64_t)j * b.nx);
    } else if (q < nz_cells + ny_cells) {
      int64_t r = q - nz_cells;
      int64_t per = (int64_t)nyg * b.nx;
      k = b.klo + (int)(r / per);
      r -= (int64_t)(k - b.klo) * per;
      int p = (int)(r / b.nx);
      i = (int)(r - (int64_t)p * b.nx);
      j = (p < b.jlo) ? p : b.jhi + 1 + (p - b.jlo);
    } else {
      int64_t r = q - nz_cells - ny_cells;
      int64_t per = (int64_t)b.fby() * nxg;
      k = b.klo + (int)(r / per);
      r -= (int64_t)(k - b.klo) * per;
      j = b.jlo + (int)(r / nxg);
      int p = (int)(r - (int64_t)(j - b.jlo) * nxg);
      i = (p < b.ilo) ? p : b.ihi + 1 + (p - b.ilo);
    }
    const double v = bc_xyz(a, b, i, j, k);
    const int64_t idx = b.idx(i, j, k);
    a[idx] = v;
    if (phi_new && k >= b.klo - 3 && k <= b.khi + 3) phi_new[idx] = impose3(v, idx, im);
  }
}

__global__ void k_face(Box b, double* a, int face) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (face < 2) {  // lines over (j,k)
    if (t >= b.ny * b.nz) return;
    const int j = t % b.ny, k = t / b.ny;
    const int f = face == 0 ? b.ilo : b.ihi, g = face == 0 ? b.ilo + 1 : b.ihi - 1;
    const double vf = a[b.idx(f, j, k)], vg = a[b.idx(g, j, k)];
    if (face == 0)
      for (int i = 0; i < b.ilo; i++) a[b.idx(i, j, k)] = extrap(vf, vg, b.ilo - i);
    else
      for (int i = b.ihi + 1; i < b.nx; i++) a[b.idx(i, j, k)] = extrap(vf, vg, i - b.ihi);
  } else if (face < 4) {  // lines over (i,k)
    if (t >= b.nx * b.nz) return;
    const int i = t % b.nx, k = t / b.nx;
    const int f = face == 2 ? b.jlo : b.jhi, g = face == 2 ? b.jlo + 1 : b.jhi - 1;
    const double vf = a[b.idx(i, f, k)], vg = a[b.idx(i, g, k)];
    if (face == 2)
      for (int j = 0; j < b.jlo; j++) a[b.idx(i, j, k)] = extrap(vf, vg, b.jlo - j);
    else
      for (int j = b.jhi + 1; j < b.ny; j++) a[b.idx(i, j, k)] = extrap(vf, vg, j - b.jhi);
  } else {  // lines over (i,j)
    if (t >= b.nx * b.ny) return;
    const int i = t % b.nx, j = t / b.nx;
    const int f = face == 4 ? b.klo : b.khi, g = face == 4 ? b.klo + 1 : b.khi - 1;
    const double vf = a[b.idx(i, j, f)], vg = a[b.idx(i, j, g)];
    if (face == 4)
      for (int k = 0; k < b.klo; k++) a[b.idx(i, j, k)] = extrap(vf, vg, b.klo - k);
    else
      for (int k = b.khi + 1; k < b.nz; k++) a[b.idx(i, j, k)] = extrap(vf, vg, k - b.khi);
  }
}

__global__ void k_impose_region(Box b, const double* src, double* phi_new, ImposeArgs im, const Ctl* ctl) {
  if (ctl && !ctl->active) return;
  int k0 = b.klo - 3 < 0 ? 0 : b.klo - 3;
  int k1 = b.khi + 3 > b.nz - 1 ? b.nz - 1 : b.khi + 3;
  const int64_t nxy = (int64_t)b.nx * b.ny;
  const int64_t total = (int64_t)(k1 - k0 + 1) * nxy;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < total;
       q += (int64_t)gridDim.x * blockDim.x) {
    int64_t idx = (int64_t)k0 * nxy + q;
    phi_new[idx] = impose3(src[idx], idx, im);
  }
}

// ---------------------------------------------------------------------------
// F8 source map: rows are (j,k) lines of the fill box in loop order

__device__ __forceinline__ bool vel_valid(double v) { return fabs(v) >= kZeroTol; }

__global__ void k_nsrc_rowlast(Box b, const double* __restrict__ vel, int* rowlast) {
  const int64_t nrows = (int64_t)b.fby() * b.fbz();
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nrows;
       r += (int64_t)gridDim.x * blockDim.x) {
    int j = b.jlo + (int)(r % b.fby()), k = b.klo + (int)(r / b.fby());
    int last = -1;
    for (int i = b.ihi; i >= b.ilo; i--) {
      int64_t idx = b.idx(i, j, k);
      if (vel_valid(vel[idx])) {
        last = (int)idx;
        break;
      }
    }
    rowlast[r] = last;
  }
}

// one block per slab: exclusive running max of rowlast over the slab's rows
__global__ void k_nsrc_carry(Box b, int nslabs, const int* rowlast, int* carry) {
  __shared__ int part[1024];
  const int t = blockIdx.x;
  const int ns = b.khi - b.klo + 1;
  const int k0 = b.klo + (int)(((int64_t)ns * t) / nslabs);
  int k1 = b.klo + (int)(((int64_t)ns * (t + 1)) / nslabs) - 1;
  if (k1 > b.khi) k1 = b.khi;
  const int64_t r0 = (int64_t)(k0 - b.klo) * b.fby();
  const int64_t r1 = (int64_t)(k1 - b.klo + 1) * b.fby();  // exclusive
  const int64_t len = r1 - r0;
  const int nt = blockDim.x;
  const int64_t chunk = (len + nt - 1) / nt;
  const int64_t a0 = r0 + threadIdx.x * chunk;
  const int64_t a1 = (a0 + chunk < r1) ? a0 + chunk : r1;
  int m = -1;
  for (int64_t r = a0; r < a1; r++) m = max(m, rowlast[r]);
  part[threadIdx.x] = m;
  __syncthreads();
  if (threadIdx.x == 0) {  // exclusive scan of the chunk maxima
    int run = -1;
    for (int q = 0; q < nt; q++) {
      int v = part[q];
      part[q] = run;
      run = max(run, v);
    }
  }
  __syncthreads();
  int run = part[threadIdx.x];
  for (int64_t r = a0; r < a1; r++) {
    carry[r] = run;
    run = max(run, rowlast[r]);
  }
}

__global__ void k_nsrc_fill(Box b, const double* __restrict__ vel, const int* carry, int* nsrc,
                            unsigned long long* count) {
  const int64_t nrows = (int64_t)b.fby() * b.fbz();
  unsigned long long local = 0;
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nrows;
       r += (int64_t)gridDim.x * blockDim.x) {
    int j = b.jlo + (int)(r % b.fby()), k = b.klo + (int)(r / b.fby());
    int cur = carry[r];
    for (int i = b.ilo; i <= b.ihi; i++) {
      int64_t idx = b.idx(i, j, k);
      if (vel_valid(vel[idx])) {
        cur = (int)idx;
        nsrc[idx] = -1;
      } else {
        nsrc[idx] = cur;
        local++;
      }
    }
  }
  if (local) atomicAdd(count, local);
}

// ---------------------------------------------------------------------------
// reinitialisation (src/reinitialization/qss_reinitialization3d.f:476-746)

__global__ void k_distance0(Box b, const double* __restrict__ phi0, double* distance0, double dx, double dy,
                            double dz) {
  const int i = b.ilo + blockIdx.x * blockDim.x + threadIdx.x;
  const int j = b.jlo + blockIdx.y * blockDim.y + threadIdx.y;
  const int k = b.klo + blockIdx.z * blockDim.z + threadIdx.z;
  if (i > b.ihi || j > b.jhi || k > b.khi) return;
  const int64_t c = b.idx(i, j, k), sy = b.sy(), sz = b.sz();
  const double zero_tol = 1.e-5, zero = 0.0;
  const double max_dx = dmax(dmax(dx, dy), dz);
  const double cc = phi0[c];
  const double n[6] = {phi0[c + 1], phi0[c - 1], phi0[c + sy], phi0[c - sy], phi0[c + sz], phi0[c - sz]};
  bool near = false;
#pragma unroll
  for (int q = 0; q < 6; q++) near = near || (n[q] > zero && cc <= zero) || (n[q] <= zero && cc > zero);
  if (!near) {
    distance0[c] = -1000.0 * max_dx;
    return;
  }
  double d1, d2, d3, delta;
  d1 = fabs(n[0] - n[1]) / 2.0;
  d2 = fabs(n[0] - cc);
  d3 = fabs(cc - n[1]);
  delta = dmax(dmax(dmax(d1, d2), d3), zero_tol);
  d1 = fabs(n[2] - n[3]) / 2.0;
  d2 = fabs(n[2] - cc);
  d3 = fabs(cc - n[3]);
  delta = dmax(dmax(dmax(d1, d2), d3), delta);
  d1 = fabs(n[4] - n[5]) / 2.0;
  d2 = fabs(n[4] - cc);
  d3 = fabs(cc - n[5]);
  delta = dmax(dmax(dmax(d1, d2), d3), delta);
  distance0[c] = cc / delta;
}

__device__ __forceinline__ double reinit_rhs_at(const double* __restrict__ phi, const double* __restrict__ phi0,
                                                const double* __restrict__ distance0, const Box& b, int64_t c,
                                                const Inv& inv, double max_dx) {
  const double zero_tol = 1.e-5;
  const int64_t sy = b.sy(), sz = b.sz();
  const double cc = __ldg(phi + c);
  double gp[3], gm[3];
  gp[0] = (__ldg(phi + c + 1) - cc) * inv.x;
  gm[0] = (cc - __ldg(phi + c - 1)) * inv.x;
  gp[1] = (__ldg(phi + c + sy) - cc) * inv.y;
  gm[1] = (cc - __ldg(phi + c - sy)) * inv.y;
  gp[2] = (__ldg(phi + c + sz) - cc) * inv.z;
  gm[2] = (cc - __ldg(phi + c - sz)) * inv.z;
  const double p0 = phi0[c];
  const double sgn = (fabs(p0) > zero_tol) ? copysign(1.0, p0) : 0.0;
  const double d0 = distance0[c];
  if (d0 == -1000.0 * max_dx) {
    double gs[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
      double a_, b_;
      if (cc > 0.0) {
        a_ = dmax(-gp[d], 0.0);
        b_ = dmax(gm[d], 0.0);
      } else {
        a_ = dmax(gp[d], 0.0);
        b_ = dmax(-gm[d], 0.0);
      }
      gs[d] = dmax(a_, b_);
    }
    if (fabs(cc) > zero_tol) {
      double ngps = gs[0] * gs[0] + gs[1] * gs[1] + gs[2] * gs[2];
      return sgn - sgn * sqrt(ngps);
    }
    return 0.0;
  }
  return d0 - sgn * fabs(cc) / max_dx;
}

// The same right-hand side with the sign tests, maxima, absolute values, the
// square root and the division on the integer pipes (qss_emu: IEEE results,
// bit for bit), leaving ~20 FP64 instructions per voxel; at EMU >= 2 the six
// scalings of the one-sided differences move there too.  Every branch
// computes exactly the native version's value:
//   dmax(-g, 0) = (g < 0 ? -g : +0) and dmax(g, 0) = (g > 0 ? g : +0) (only
//   their squares are used, so the sign of a zero does not matter);
//   sgn * s for sgn = +-1 is a sign flip; sgn = 0 keeps the native product.
template <int EMU>
__device__ __forceinline__ double reinit_rhs_e(const double* __restrict__ phi, const double* __restrict__ phi0,
                                               const double* __restrict__ distance0, const Box& b, int64_t c,
                                               const Inv& inv, double max_dx, uint64_t far_bits) {
  using namespace qss_emu;
  const uint64_t tol_bits = bits(1.e-5);
  const int64_t sy = b.sy(), sz = b.sz();
  auto scale = [](double d, double f) -> double { return EMU >= 2 ? qss_emu::mul(d, f) : d * f; };
  const double cc = __ldg(phi + c);
  const double p0 = phi0[c];
  const uint64_t ap0 = bits(p0) & kAbs;
  const bool sgn_nz = ap0 > tol_bits && ap0 <= 0x7ff0000000000000ull;  // fabs(p0) > 1e-5
  const bool sgn_neg = (int64_t)bits(p0) < 0;
  const double sgn = sgn_nz ? (sgn_neg ? -1.0 : 1.0) : 0.0;
  const double d0 = distance0[c];
  if (bits(d0) == far_bits) {
    const bool pos = gt0(cc);
    double gs[3];
    const int64_t st[3] = {1, sy, sz};
    const double iv[3] = {inv.x, inv.y, inv.z};
#pragma unroll
    for (int d = 0; d < 3; d++) {
      const double gp = scale(__ldg(phi + c + st[d]) - cc, iv[d]);
      const double gm = scale(cc - __ldg(phi + c - st[d]), iv[d]);
      double a_, b_;
      if (pos) {
        a_ = lt0(gp) ? qss_emu::neg(gp) : 0.0;
        b_ = gt0(gm) ? gm : 0.0;
      } else {
        a_ = gt0(gp) ? gp : 0.0;
        b_ = lt0(gm) ? qss_emu::neg(gm) : 0.0;
      }
      gs[d] = max_nonneg(a_, b_);
    }
    const uint64_t acc = bits(cc) & kAbs;
    if (acc > tol_bits && acc <= 0x7ff0000000000000ull) {  // fabs(cc) > 1e-5
      const double ngps = scale(gs[0], gs[0]) + scale(gs[1], gs[1]) + scale(gs[2], gs[2]);
      const double s = qss_emu::sqrt(ngps);
      if (!sgn_nz) return sgn - sgn * s;
      return sgn - (sgn_neg ? qss_emu::neg(s) : s);
    }
    return 0.0;
  }
  // d0 - sgn * fabs(cc) / max_dx
  const double acc = qss_emu::abs(cc);
  const double t = sgn_nz ? (sgn_neg ? qss_emu::neg(acc) : acc) : sgn * acc;
  return d0 - qss_emu::div(t, max_dx);
}

// The reinitialisation right-hand side of one voxel from its six scaled
// one-sided differences gp[d] = (phi(c + e_d) - phi(c)) inv_d and
// gm[d] = (phi(c) - phi(c - e_d)) inv_d, with the operations of reinit_rhs_e.
__device__ __forceinline__ double reinit_rhs_diffs(double cc, double p0, double d0, const double gp[3],
                                                   const double gm[3], double max_dx, uint64_t far_bits) {
  using namespace qss_emu;
  const uint64_t tol_bits = bits(1.e-5);
  auto scale = [](double d, double f) -> double { return qss_emu::mul(d, f); };
  const uint64_t ap0 = bits(p0) & kAbs;
  const bool sgn_nz = ap0 > tol_bits && ap0 <= 0x7ff0000000000000ull;  // fabs(p0) > 1e-5
  const bool sgn_neg = (int64_t)bits(p0) < 0;
  const double sgn = sgn_nz ? (sgn_neg ? -1.0 : 1.0) : 0.0;
  if (bits(d0) == far_bits) {
    const bool pos = gt0(cc);
    double gs[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
      double a_, b_;
      if (pos) {
        a_ = lt0(gp[d]) ? qss_emu::neg(gp[d]) : 0.0;
        b_ = gt0(gm[d]) ? gm[d] : 0.0;
      } else {
        a_ = gt0(gp[d]) ? gp[d] : 0.0;
        b_ = lt0(gm[d]) ? qss_emu::neg(gm[d]) : 0.0;
      }
      gs[d] = max_nonneg(a_, b_);
    }
    const uint64_t acc = bits(cc) & kAbs;
    if (acc > tol_bits && acc <= 0x7ff0000000000000ull) {  // fabs(cc) > 1e-5
      const double ngps = scale(gs[0], gs[0]) + scale(gs[1], gs[1]) + scale(gs[2], gs[2]);
      const double s = qss_emu::sqrt(ngps);
      if (!sgn_nz) return sgn - sgn * s;
      return sgn - (sgn_neg ? qss_emu::neg(s) : s);
    }
    return 0.0;
  }
  const double acc = qss_emu::abs(cc);
  const double t = sgn_nz ? (sgn_neg ? qss_emu::neg(acc) : acc) : sgn * acc;
  return d0 - qss_emu::div(t, max_dx);
}

// Reinitialisation step at level 2 with each face difference computed once:
// the difference (phi(c + e) - phi(c)) inv is the plus difference of c and
// the minus difference of c + e, the same operation on the same operands.
// A block of 4 warps covers 32 (i) x 4 (j) voxels, each warp an 8 x 4 patch
// (x neighbours one lane apart, y neighbours eight), and walks `walk` planes
// along k carrying the z difference; lanes on the patch's low edges and the
// first plane compute their minus difference themselves.  Per voxel about
// 3.4 differences instead of 6 for a walk of 16 planes.  Short walks keep
// small boxes' grids large enough to fill the GPU (see reinit_launch).
constexpr int kRWalkMax = 16;

__global__ void __launch_bounds__(128) k_reinit_walk(Box b, const double* __restrict__ data,
                                                     const double* __restrict__ phi0,
                                                     const double* __restrict__ distance0, double* __restrict__ next,
                                                     double dt_r, Inv inv, double max_dx, int rhs_only,
                                                     uint64_t far_bits, int walk) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int li = lane & 7, lj = lane >> 3;
  const int i_raw = b.ilo + blockIdx.x * 32 + 8 * warp + li;
  const int j_raw = b.jlo + blockIdx.y * 4 + lj;
  const bool ok = i_raw <= b.ihi && j_raw <= b.jhi;
  // lanes past the fill box work on its last row/column (in the box), store nothing
  const int i = i_raw <= b.ihi ? i_raw : b.ihi;
  const int j = j_raw <= b.jhi ? j_raw : b.jhi;
  const int k0 = b.klo + blockIdx.z * walk;
  const int k1 = k0 + walk - 1 < b.khi ? k0 + walk - 1 : b.khi;
  const int64_t sy = b.sy(), sz = b.sz();
  auto scale = [](double d, double f) -> double { return qss_emu::mul(d, f); };
  int64_t c = b.idx(i, j, k0);
  double cc = __ldg(data + c);
  double dzm = scale(cc - __ldg(data + c - sz), inv.z);
  for (int k = k0; k <= k1; k++) {
    const double zp = __ldg(data + c + sz);
    double gp[3], gm[3];
    gp[0] = scale(__ldg(data + c + 1) - cc, inv.x);
    gp[1] = scale(__ldg(data + c + sy) - cc, inv.y);
    gp[2] = scale(zp - cc, inv.z);
    const double xm = __shfl_up_sync(0xffffffffu, gp[0], 1);
    const double ym = __shfl_up_sync(0xffffffffu, gp[1], 8);
    gm[0] = li == 0 ? scale(cc - __ldg(data + c - 1), inv.x) : xm;
    gm[1] = lj == 0 ? scale(cc - __ldg(data + c - sy), inv.y) : ym;
    gm[2] = dzm;
    if (ok) {
      const double r = reinit_rhs_diffs(cc, phi0[c], distance0[c], gp, gm, max_dx, far_bits);
      next[c] = rhs_only ? r : data[c] + qss_emu::mul(dt_r, r);
    }
    dzm = gp[2];
    cc = zp;
    c += sz;
  }
}

template <int EMU>
__global__ void k_reinit_step(Box b, const double* __restrict__ data, const double* __restrict__ phi0,
                              const double* __restrict__ distance0, double* __restrict__ next, double dt_r,
                              Inv inv, double max_dx, int rhs_only, uint64_t far_bits) {
  const int i = b.ilo + blockIdx.x * blockDim.x + threadIdx.x;
  const int j = b.jlo + blockIdx.y * blockDim.y + threadIdx.y;
  const int k = b.klo + blockIdx.z * blockDim.z + threadIdx.z;
  if (i > b.ihi || j > b.jhi || k > b.khi) return;
  const int64_t c = b.idx(i, j, k);
  const double r = EMU == 0 ? reinit_rhs_at(data, phi0, distance0, b, c, inv, max_dx)
                            : reinit_rhs_e<EMU>(data, phi0, distance0, b, c, inv, max_dx, far_bits);
  next[c] = rhs_only ? r : data[c] + (EMU >= 2 ? qss_emu::mul(dt_r, r) : dt_r * r);
}

// ---------------------------------------------------------------------------
// coefficient set-up (3d.f:13-298, qss_util3d.f:499-581)

__global__ void k_central_grad(Box b, const double* __restrict__ f, double* fx, double* fy, double* fz,
                               Fac fac) {
  const int i = b.ilo + blockIdx.x * blockDim.x + threadIdx.x;
  const int j = b.jlo + blockIdx.y * blockDim.y + threadIdx.y;
  const int k = b.klo + blockIdx.z * blockDim.z + threadIdx.z;
  if (i > b.ihi || j > b.jhi || k > b.khi) return;
  const int64_t c = b.idx(i, j, k), sy = b.sy(), sz = b.sz();
  fx[c] = (f[c + 1] - f[c - 1]) * fac.x;
  fy[c] = (f[c + sy] - f[c - sy]) * fac.y;
  fz[c] = (f[c + sz] - f[c - sz]) * fac.z;
}

struct MaskGeom {
  double h1, h2, absgrad, s;
};

__device__ __forceinline__ MaskGeom mask_geom(double m, double mx, double my, double mz, double dx) {
  const double eps_var = 1.5 * dx;
  MaskGeom g;
  g.h1 = qss_heaviside(-m, eps_var);
  g.h2 = qss_heaviside(m, eps_var);
  double ag = mx * mx + my * my + mz * mz;
  ag = sqrt(ag);
  double x = m * m + ag * dx * ag * dx;
  x = sqrt(x);
  g.absgrad = ag;
  g.s = m / x;
  return g;
}

__global__ void k_setvarnorm(Box b, const double* __restrict__ mask, const double* __restrict__ mx,
                             const double* __restrict__ my, const double* __restrict__ mz, double* vel_n,
                             double a0, const double* theta_field, double theta, double dx) {
  const int i = b.ilo + blockIdx.x * blockDim.x + threadIdx.x;
  const int j = b.jlo + blockIdx.y * blockDim.y + threadIdx.y;
  const int k = b.klo + blockIdx.z * blockDim.z + threadIdx.z;
  if (i > b.ihi || j > b.jhi || k > b.khi) return;
  const int64_t c = b.idx(i, j, k);
  const double C2 = 1;
  MaskGeom g = mask_geom(mask[c], mx[c], my[c], mz[c], dx);
  const double ca = theta_field ? theta_field[c] : theta;
  vel_n[c] = g.h1 * a0 - g.s * g.h2 * C2 * portable_cos(ca) * g.absgrad;
}

__global__ void k_setvarcurvadv(Box b, const double* __restrict__ mask, const double* __restrict__ mx,
                                const double* __restrict__ my, const double* __restrict__ mz, double* vb,
                                double* vx, double* vy, double* vz, double const_b, double dx,
                                unsigned long long* red) {
  const int i = b.ilo + blockIdx.x * blockDim.x + threadIdx.x;
  const int j = b.jlo + blockIdx.y * blockDim.y + threadIdx.y;
  const int k = b.klo + blockIdx.z * blockDim.z + threadIdx.z;
  double bm = -1.0, um = -1.0;
  if (i <= b.ihi && j <= b.jhi && k <= b.khi) {
    const int64_t c = b.idx(i, j, k);
    const double C1 = const_b, C2 = 1;
    const double inv_dx = 1.0 / dx, inv_dy = 1.0 / dx, inv_dz = 1.0 / dx;
    const double gx = mx[c], gy = my[c], gz = mz[c];
    MaskGeom g = mask_geom(mask[c], gx, gy, gz, dx);
    const double bv = g.h1 * C1;
    vb[c] = bv;
    bm = bv;
    const double ux = g.s * C2 * gx * g.h2;
    const double uy = g.s * C2 * gy * g.h2;
    const double uz = g.s * C2 * gz * g.h2;
    vx[c] = ux;
    vy[c] = uy;
    vz[c] = uz;
    um = fabs(ux) * inv_dx + fabs(uy) * inv_dy + fabs(uz) * inv_dz;
  }
  for (int o = 16; o > 0; o >>= 1) {
    bm = dmax(bm, __shfl_down_sync(0xffffffffu, bm, o));
    um = dmax(um, __shfl_down_sync(0xffffffffu, um, o));
  }
  const int lane = (threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z)) & 31;
  if (lane == 0) {
    atomicMax(&red[0], double_to_key(bm));
    atomicMax(&red[1], double_to_key(um));
  }
}

__global__ void k_trapvel(Box b, const double* __restrict__ test, double* vel_n, double* vb, double* vx,
                          double* vy, double* vz, double dx) {
  const int i = b.ilo + blockIdx.x * blockDim.x + threadIdx.x;
  const int j = b.jlo + blockIdx.y * blockDim.y + threadIdx.y;
  const int k = b.klo + blockIdx.z * blockDim.z + threadIdx.z;
  if (i > b.ihi || j > b.jhi || k > b.khi) return;
  const int64_t c = b.idx(i, j, k);
  if (test[c] > 1.5 * dx) {
    vel_n[c] = 0;
    vb[c] = 0;
    vx[c] = 0;
    vy[c] = 0;
    vz[c] = 0;
  }
}

// ---------------------------------------------------------------------------
// whole-array operations

__global__ void k_max_into(int64_t n, double* out, const double* mask, const double* phi) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
    double m = mask[q], p = phi[q];
    out[q] = (m > p) ? m : p;
  }
}
__global__ void k_min_into(int64_t n, double* out, const double* a, const double* b) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
    double x = a[q], y = b[q];
    out[q] = (x < y) ? x : y;
  }
}
__global__ void k_merge(int64_t n, double* phi, const double* m) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
    double v = m[q];
    if (v > 0) phi[q] = -v;
  }
}
__global__ void k_fill(int64_t n, double* out, double v) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
    out[q] = v;
}

__global__ void k_rk(Box b, int stage, double* out, const double* u1, const double* u0, const double* rhs,
                     double dt) {
  const int i = b.ilo + blockIdx.x * blockDim.x + threadIdx.x;
  const int j = b.jlo + blockIdx.y * blockDim.y + threadIdx.y;
  const int k = b.klo + blockIdx.z * blockDim.z + threadIdx.z;
  if (i > b.ihi || j > b.jhi || k > b.khi) return;
  const int64_t c = b.idx(i, j, k);
  if (stage == 1) {
    out[c] = u1[c] + dt * rhs[c];
  } else if (stage == 2) {
    out[c] = 0.75 * u0[c] + 0.25 * (u1[c] + dt * rhs[c]);
  } else {
    const double one_third = 1.0 / 3.0, two_thirds = 2.0 / 3.0;
    out[c] = one_third * u0[c] + two_thirds * (u1[c] + dt * rhs[c]);
  }
}

__global__ void k_impose_slab(Box b, double* out, const double* mask, const double* phi, double overlap, int k0,
                              int k1) {
  const int64_t nxy = (int64_t)b.nx * b.ny;
  const int64_t total = (int64_t)(k1 - k0 + 1) * nxy;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < total;
       q += (int64_t)gridDim.x * blockDim.x) {
    int64_t c = (int64_t)k0 * nxy + q;
    double m = mask[c] - overlap, p = phi[c];
    out[c] = (m > p) ? m : p;
  }
}

// ---------------------------------------------------------------------------
// reductions

__global__ void k_maxnormdiff(Box b, const double* __restrict__ f1, const double* __restrict__ f2, double zone,
                              unsigned long long* key) {
  const int i = b.ilo + blockIdx.x * blockDim.x + threadIdx.x;
  const int j = b.jlo + blockIdx.y * blockDim.y + threadIdx.y;
  const int k = b.klo + blockIdx.z * blockDim.z + threadIdx.z;
  double m = -1.0;
  if (i <= b.ihi && j <= b.jhi && k <= b.khi) {
    const int64_t c = b.idx(i, j, k);
    const double a = f1[c];
    if (fabs(a) < zone) m = fabs(a - f2[c]);
  }
  for (int o = 16; o > 0; o >>= 1) m = dmax(m, __shfl_down_sync(0xffffffffu, m, o));
  const int lane = (threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z)) & 31;
  if (lane == 0 && m > -1.0) atomicMax(key, double_to_key(m));
}

// contribution of each fill-box voxel, stored in loop order (i fastest)
__global__ void k_vol_contrib(Box b, const double* __restrict__ phi, double dV, double eps, double* contrib) {
  const int64_t n = (int64_t)b.fbx() * b.fby() * b.fbz();
  const double pi = 3.14159265358979323846;
  const double one_over_pi = 0.31830988618379;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
    const int i = b.ilo + (int)(q % b.fbx());
    const int64_t r = q / b.fbx();
    const int j = b.jlo + (int)(r % b.fby());
    const int k = b.klo + (int)(r / b.fby());
    const double p = phi[b.idx(i, j, k)];
    const double rr = p / eps;
    double v = 0.0;
    if (p < -eps) {
      v = dV;
    } else if (p < eps) {
      const double one_minus_H = 0.5 * (1 - rr - one_over_pi * portable_sin(pi * rr));
      v = one_minus_H * dV;
    }
    contrib[q] = v;
  }
}

// ---------------------------------------------------------------------------
// geometry (src/geometry/qss_initialization3d.c:33-165, 440-522)

__global__ void k_sphere(Box b, double* phi, double x0, double y0, double z0, double dx, double dy, double dz,
                         double cx, double cy, double cz, double r, int inside) {
  const int64_t n = b.npts();
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(q % b.nx);
    const int64_t rr = q / b.nx;
    const int j = (int)(rr % b.ny), k = (int)(rr / b.ny);
    const double x = x0 + dx * i, y = y0 + dy * j, z = z0 + dz * k;
    double d = sqrt((x - cx) * (x - cx) + (y - cy) * (y - cy) + (z - cz) * (z - cz)) - r;
    if (inside >= 0) d = -d;
    double best = -FLT_MAX;
    if (d > best) best = d;
    phi[q] = best;
  }
}

__global__ void k_box(Box b, double* phi, double x0, double y0, double z0, double dx, double dy, double dz,
                      double c0, double c1, double c2, double s0, double s1, double s2, int inside) {
  const int64_t n = b.npts();
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(q % b.nx);
    const int64_t rr = q / b.nx;
    const int j = (int)(rr % b.ny), k = (int)(rr / b.ny);
    const double x = x0 + dx * i, y = y0 + dy * j, z = z0 + dz * k;
    double best = -FLT_MAX;
#pragma unroll
    for (int p = 0; p < 6; p++) {
      const bool low = p < 3;
      const int ax = p % 3;
      const double px = low ? c0 : c0 + s0, py = low ? c1 : c1 + s1, pz = low ? c2 : c2 + s2;
      const double sg = low ? -1 : 1;
      const double nx = (ax == 0) ? sg : 0, ny = (ax == 1) ? sg : 0, nz = (ax == 2) ? sg : 0;
      const double dot = (x - px) * nx + (y - py) * ny + (z - pz) * nz;
      double nrm = nx * nx + ny * ny + nz * nz;
      nrm = sqrt(nrm);
      const double d = dot / nrm;
      if (d > best) best = d;
    }
    phi[q] = (inside >= 1) ? -best : best;
  }
}

__global__ void k_spheres(Box b, double* phi, double x0, double y0, double z0, double dx, double dy, double dz,
                          const double* __restrict__ cx, const double* __restrict__ cy,
                          const double* __restrict__ cz, const double* __restrict__ rad,
                          const int* __restrict__ inside, int num) {
  const int64_t n = b.npts();
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(q % b.nx);
    const int64_t rr = q / b.nx;
    const int j = (int)(rr % b.ny), k = (int)(rr / b.ny);
    const double x = x0 + dx * i, y = y0 + dy * j, z = z0 + dz * k;
    double best = -FLT_MAX;
    for (int l = 0; l < num; l++) {
      double d = sqrt((x - cx[l]) * (x - cx[l]) + (y - cy[l]) * (y - cy[l]) + (z - cz[l]) * (z - cz[l])) - rad[l];
      if (inside[l] >= 0) d = -d;
      if (d > best) best = d;
    }
    phi[q] = best;
  }
}

__global__ void k_halfspaces(Box b, double* phi, double x0, double y0, double z0, double dx, double dy, double dz,
                             const double* __restrict__ nxv, const double* __restrict__ nyv,
                             const double* __restrict__ nzv, const double* __restrict__ px,
                             const double* __restrict__ py, const double* __restrict__ pz, int num) {
  const int64_t n = b.npts();
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(q % b.nx);
    const int64_t rr = q / b.nx;
    const int j = (int)(rr % b.ny), k = (int)(rr / b.ny);
    const double x = x0 + dx * i, y = y0 + dy * j, z = z0 + dz * k;
    double best = -FLT_MAX;
    for (int l = 0; l < num; l++) {
      const double dot = (x - px[l]) * nxv[l] + (y - py[l]) * nyv[l] + (z - pz[l]) * nzv[l];
      double nrm = nxv[l] * nxv[l] + nyv[l] * nyv[l] + nzv[l] * nzv[l];
      nrm = sqrt(nrm);
      const double d = dot / nrm;
      if (d > best) best = d;
    }
    phi[q] = best;
  }
}

__global__ void k_negate(int64_t n, double* a) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
    a[q] = -a[q];
}

}  // namespace

// ===========================================================================
// launch wrappers

static const dim3 kBlk3(32, 4, 1);

// stage-kernel timing (host side): event pairs recorded around each launch
// of a stage kernel on the profiled stream, tagged with the kernel's kind
namespace {
struct StageProfiler {
  bool on = false;
  cudaStream_t stream = nullptr;
  struct Rec {
    int kind;
    cudaEvent_t e0, e1;
  };
  std::vector<Rec> ev;
} g_prof;
}  // namespace

void qss_profile_stage_begin(cudaStream_t s) {
  g_prof.on = true;
  g_prof.stream = s;
  g_prof.ev.clear();
}

void qss_profile_stage_end(double ms[kProfKinds], int launches[kProfKinds]) {
  for (int k = 0; k < kProfKinds; k++) {
    ms[k] = 0;
    launches[k] = 0;
  }
  for (auto& e : g_prof.ev) {
    cudaEventSynchronize(e.e1);
    float t = 0;
    cudaEventElapsedTime(&t, e.e0, e.e1);
    ms[e.kind] += t;
    launches[e.kind]++;
    cudaEventDestroy(e.e0);
    cudaEventDestroy(e.e1);
  }
  g_prof.ev.clear();
  g_prof.on = false;
}

cudaEvent_t prof_open(cudaStream_t s) {
  if (!g_prof.on || s != g_prof.stream) return nullptr;
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  cudaEventRecord(e, s);
  return e;
}

void prof_close(cudaStream_t s, cudaEvent_t e0, int kind) {
  if (!e0) return;
  cudaEvent_t e1 = nullptr;
  cudaEventCreate(&e1);
  cudaEventRecord(e1, s);
  g_prof.ev.push_back({kind, e0, e1});
}

static const int kBlk1 = 256;

static unsigned grid1(int64_t n) {
  int64_t b = (n + kBlk1 - 1) / kBlk1;
  if (b > 152 * 32) b = 152 * 32;
  if (b < 1) b = 1;
  return (unsigned)b;
}

void launch_dt(cudaStream_t s, int scheme, bool var, const Box& b, const double* phi, const Coef& c, int nslabs,
               double dx, double dy, double dz, Ctl* ctl) {
  int threads = ((nslabs + 31) / 32) * 32;
  if (threads < 32) threads = 32;
#define QSS_DT(S, V) k_dt<S, V><<<1, threads, 0, s>>>(b, phi, c, nslabs, dx, dy, dz, ctl)
  if (scheme == ENO2) { if (var) QSS_DT(ENO2, true); else QSS_DT(ENO2, false); }
  else if (scheme == ENO3) { if (var) QSS_DT(ENO3, true); else QSS_DT(ENO3, false); }
  else { if (var) QSS_DT(WENO5, true); else QSS_DT(WENO5, false); }
#undef QSS_DT
}

template <int S, bool V>
static void stage_dispatch(cudaStream_t s, int stage, bool fin, dim3 g, dim3 blk, const StageArgs& a) {
  switch (stage) {
    case 0: k_stage<S, V, 0, false><<<g, blk, 0, s>>>(a); break;
    case 1: if (fin) k_stage<S, V, 1, true><<<g, blk, 0, s>>>(a); else k_stage<S, V, 1, false><<<g, blk, 0, s>>>(a); break;
    case 2: if (fin) k_stage<S, V, 2, true><<<g, blk, 0, s>>>(a); else k_stage<S, V, 2, false><<<g, blk, 0, s>>>(a); break;
    default: if (fin) k_stage<S, V, 3, true><<<g, blk, 0, s>>>(a); else k_stage<S, V, 3, false><<<g, blk, 0, s>>>(a); break;
  }
}

void launch_stage(cudaStream_t s, int scheme, bool var, int stage, bool final_stage, const Box& b, double dx,
                  double dy, double dz, const double* phi_in, const double* u_cur, double* out, double* phi_new,
                  const Coef& c, const ImposeArgs& im, const Ctl* ctl) {
  StageArgs a;
  a.b = b;
  a.inv = Inv{1.0 / dx, 1.0 / dy, 1.0 / dz};
  a.fac = Fac{0.5 / dx, 0.5 / dy, 0.5 / dz};
  a.phi_in = phi_in;
  a.u_cur = u_cur;
  a.out = out;
  a.phi_new = phi_new;
  a.c = c;
  a.im = im;
  a.ctl = ctl;
  dim3 g = fb_grid(b, kBlk3);
  cudaEvent_t e0 = stage != 0 ? prof_open(s) : nullptr;
  if (scheme == ENO2) { if (var) stage_dispatch<ENO2, true>(s, stage, final_stage, g, kBlk3, a); else stage_dispatch<ENO2, false>(s, stage, final_stage, g, kBlk3, a); }
  else if (scheme == ENO3) { if (var) stage_dispatch<ENO3, true>(s, stage, final_stage, g, kBlk3, a); else stage_dispatch<ENO3, false>(s, stage, final_stage, g, kBlk3, a); }
  else { if (var) stage_dispatch<WENO5, true>(s, stage, final_stage, g, kBlk3, a); else stage_dispatch<WENO5, false>(s, stage, final_stage, g, kBlk3, a); }
  prof_close(s, e0, kProfStage);
}

void launch_cfl_at(cudaStream_t s, int scheme, bool var, const Box& b, const double* phi, const Coef& c, int i,
                   int j, int k, double dx, double dy, double dz, double* h_out) {
#define QSS_CFL(S, V) k_cfl_at<S, V><<<1, 1, 0, s>>>(b, phi, c, i, j, k, dx, dy, dz, h_out)
  if (scheme == ENO2) { if (var) QSS_CFL(ENO2, true); else QSS_CFL(ENO2, false); }
  else if (scheme == ENO3) { if (var) QSS_CFL(ENO3, true); else QSS_CFL(ENO3, false); }
  else { if (var) QSS_CFL(WENO5, true); else QSS_CFL(WENO5, false); }
#undef QSS_CFL
}

void launch_ghost(cudaStream_t s, const Box& b, double* a, double* phi_new, const ImposeArgs& im, const Ctl* ctl) {
  const int64_t total = b.npts() - (int64_t)b.fbx() * b.fby() * b.fbz();
  k_ghost<<<grid1(total), kBlk1, 0, s>>>(b, a, phi_new, im, ctl);
}

void launch_face(cudaStream_t s, const Box& b, double* a, int face) {
  int lines = face < 2 ? b.ny * b.nz : (face < 4 ? b.nx * b.nz : b.nx * b.ny);
  k_face<<<(lines + 255) / 256, 256, 0, s>>>(b, a, face);
}

void launch_impose_region(cudaStream_t s, const Box& b, const double* src, double* phi_new, const ImposeArgs& im,
                          const Ctl* ctl) {
  k_impose_region<<<grid1(b.npts()), kBlk1, 0, s>>>(b, src, phi_new, im, ctl);
}

void launch_nsrc(cudaStream_t s, const Box& b, const double* vel_n, int* nsrc, int nslabs, int* d_rowlast,
                 int* d_carry, unsigned long long* d_count) {
  const int64_t nrows = (int64_t)b.fby() * b.fbz();
  cudaMemsetAsync(d_count, 0, sizeof(unsigned long long), s);
  k_nsrc_rowlast<<<grid1(nrows), kBlk1, 0, s>>>(b, vel_n, d_rowlast);
  k_nsrc_carry<<<nslabs, 1024, 0, s>>>(b, nslabs, d_rowlast, d_carry);
  k_nsrc_fill<<<grid1(nrows), kBlk1, 0, s>>>(b, vel_n, d_carry, nsrc, d_count);
}

void launch_distance0(cudaStream_t s, const Box& b, const double* phi0, double* distance0, double dx, double dy,
                      double dz) {
  k_distance0<<<fb_grid(b, kBlk3), kBlk3, 0, s>>>(b, phi0, distance0, dx, dy, dz);
}

// $QSSGPU_REINIT_WALK=0 selects the one-voxel-per-thread reinitialisation
// step at level 2 (identical results)
static bool reinit_walk() {
  static const int on = [] {
    const char* e = getenv("QSSGPU_REINIT_WALK");
    return e && atoi(e) == 0 ? 0 : 1;
  }();
  return on != 0;
}

static void reinit_launch(cudaStream_t s, const Box& b, const double* data, const double* phi0,
                          const double* distance0, double* out, double dt_r, double dx, double dy, double dz,
                          int rhs_only) {
  const double max_dx = (dx > dy ? dx : dy) > dz ? (dx > dy ? dx : dy) : dz;
  const Inv inv{1.0 / dx, 1.0 / dy, 1.0 / dz};
  const uint64_t far_bits = qss_emu::bits(-1000.0 * max_dx);  // distance0 of voxels away from the interface
  const int lvl = emu_level();
  const dim3 grid = fb_grid(b, kBlk3);
  if (lvl >= 2 && reinit_walk()) {
    // planes per thread: up to kRWalkMax while the grid keeps ~16 blocks per SM
    const int64_t xy = (int64_t)((b.fbx() + 31) / 32) * ((b.fby() + 3) / 4);
    int64_t walk = xy * b.fbz() / (152 * 16);
    walk = walk < 1 ? 1 : (walk > kRWalkMax ? kRWalkMax : walk);
    const dim3 gw((b.fbx() + 31) / 32, (b.fby() + 3) / 4, (unsigned)((b.fbz() + walk - 1) / walk));
    k_reinit_walk<<<gw, 128, 0, s>>>(b, data, phi0, distance0, out, dt_r, inv, max_dx, rhs_only, far_bits,
                                     (int)walk);
  } else if (lvl >= 2)
    k_reinit_step<2><<<grid, kBlk3, 0, s>>>(b, data, phi0, distance0, out, dt_r, inv, max_dx, rhs_only, far_bits);
  else if (lvl == 1)
    k_reinit_step<1><<<grid, kBlk3, 0, s>>>(b, data, phi0, distance0, out, dt_r, inv, max_dx, rhs_only, far_bits);
  else
    k_reinit_step<0><<<grid, kBlk3, 0, s>>>(b, data, phi0, distance0, out, dt_r, inv, max_dx, rhs_only, far_bits);
}

void launch_reinit_step(cudaStream_t s, const Box& b, const double* data, const double* phi0,
                        const double* distance0, double* next, double dt_r, double dx, double dy, double dz) {
  reinit_launch(s, b, data, phi0, distance0, next, dt_r, dx, dy, dz, 0);
}

void launch_reinit_rhs(cudaStream_t s, const Box& b, const double* data, const double* phi0,
                       const double* distance0, double* rhs, double dx, double dy, double dz) {
  reinit_launch(s, b, data, phi0, distance0, rhs, 0.0, dx, dy, dz, 1);
}

void launch_central_grad(cudaStream_t s, const Box& b, const double* f, double* fx, double* fy, double* fz,
                         double dx, double dy, double dz) {
  k_central_grad<<<fb_grid(b, kBlk3), kBlk3, 0, s>>>(b, f, fx, fy, fz, Fac{0.5 / dx, 0.5 / dy, 0.5 / dz});
}

void launch_setvarnorm(cudaStream_t s, const Box& b, const double* mask, const double* mx, const double* my,
                       const double* mz, double* vel_n, double a0, const double* theta_field, double theta,
                       double dx) {
  k_setvarnorm<<<fb_grid(b, kBlk3), kBlk3, 0, s>>>(b, mask, mx, my, mz, vel_n, a0, theta_field, theta, dx);
}

void launch_setvarcurvadv(cudaStream_t s, const Box& b, const double* mask, const double* mx, const double* my,
                          const double* mz, double* vb, double* vx, double* vy, double* vz, double const_b,
                          double dx, unsigned long long* red) {
  unsigned long long init[2] = {double_to_key(-1.0), double_to_key(-1.0)};
  cudaMemcpyAsync(red, init, sizeof init, cudaMemcpyHostToDevice, s);
  k_setvarcurvadv<<<fb_grid(b, kBlk3), kBlk3, 0, s>>>(b, mask, mx, my, mz, vb, vx, vy, vz, const_b, dx, red);
}

void launch_trapvel(cudaStream_t s, const Box& b, const double* test, double* vel_n, double* vb, double* vx,
                    double* vy, double* vz, double dx) {
  k_trapvel<<<fb_grid(b, kBlk3), kBlk3, 0, s>>>(b, test, vel_n, vb, vx, vy, vz, dx);
}

void launch_max_into(cudaStream_t s, int64_t n, double* out, const double* mask, const double* phi) {
  k_max_into<<<grid1(n), kBlk1, 0, s>>>(n, out, mask, phi);
}
void launch_min_into(cudaStream_t s, int64_t n, double* out, const double* a, const double* b) {
  k_min_into<<<grid1(n), kBlk1, 0, s>>>(n, out, a, b);
}
void launch_merge(cudaStream_t s, int64_t n, double* phi, const double* m) {
  k_merge<<<grid1(n), kBlk1, 0, s>>>(n, phi, m);
}
void launch_fill(cudaStream_t s, int64_t n, double* out, double v) { k_fill<<<grid1(n), kBlk1, 0, s>>>(n, out, v); }

void launch_rk(cudaStream_t s, const Box& b, int stage, double* out, const double* u1, const double* u0,
               const double* rhs, double dt) {
  k_rk<<<fb_grid(b, kBlk3), kBlk3, 0, s>>>(b, stage, out, u1, u0, rhs, dt);
}

void launch_impose_slab(cudaStream_t s, const Box& b, double* out, const double* mask, const double* phi,
                        double overlap, int k0, int k1) {
  if (k1 < k0) return;
  k_impose_slab<<<grid1((int64_t)(k1 - k0 + 1) * b.nx * b.ny), kBlk1, 0, s>>>(b, out, mask, phi, overlap, k0, k1);
}

void launch_maxnormdiff(cudaStream_t s, const Box& b, const double* f1, const double* f2, double zone,
                        unsigned long long* key) {
  unsigned long long init = double_to_key(-1.0);
  cudaMemcpyAsync(key, &init, sizeof init, cudaMemcpyHostToDevice, s);
  k_maxnormdiff<<<fb_grid(b, kBlk3), kBlk3, 0, s>>>(b, f1, f2, zone, key);
}

void launch_volume(cudaStream_t s, const Box& b, const double* phi, double dx, double dy, double dz, double eps,
                   double* scratch, double* out) {
  const int64_t n = (int64_t)b.fbx() * b.fby() * b.fbz();
  const double dV = dx * dy * dz;
  k_vol_contrib<<<grid1(n), kBlk1, 0, s>>>(b, phi, dV, eps, scratch);
  launch_loop_sum(s, scratch, n, scratch + n, out);
}

void launch_sphere(cudaStream_t s, const Box& b, double* phi, const double* x_lo_gb, const double* dxv, double cx,
                   double cy, double cz, double r, int inside_flag) {
  k_sphere<<<grid1(b.npts()), kBlk1, 0, s>>>(b, phi, x_lo_gb[0], x_lo_gb[1], x_lo_gb[2], dxv[0], dxv[1], dxv[2],
                                              cx, cy, cz, r, inside_flag);
}

void launch_box(cudaStream_t s, const Box& b, double* phi, const double* x_lo_gb, const double* dxv,
                const double corner[3], const double side[3], int inside_flag) {
  k_box<<<grid1(b.npts()), kBlk1, 0, s>>>(b, phi, x_lo_gb[0], x_lo_gb[1], x_lo_gb[2], dxv[0], dxv[1], dxv[2],
                                           corner[0], corner[1], corner[2], side[0], side[1], side[2], inside_flag);
}

void launch_spheres(cudaStream_t s, const Box& b, double* phi, const double* x_lo_gb, const double* dxv,
                    const double* cx, const double* cy, const double* cz, const double* r, const int* inside,
                    int num) {
  k_spheres<<<grid1(b.npts()), kBlk1, 0, s>>>(b, phi, x_lo_gb[0], x_lo_gb[1], x_lo_gb[2], dxv[0], dxv[1], dxv[2], cx,
                                               cy, cz, r, inside, num);
}

void launch_halfspaces(cudaStream_t s, const Box& b, double* phi, const double* x_lo_gb, const double* dxv,
                       const double* nx, const double* ny, const double* nz, const double* px, const double* py,
                       const double* pz, int num) {
  k_halfspaces<<<grid1(b.npts()), kBlk1, 0, s>>>(b, phi, x_lo_gb[0], x_lo_gb[1], x_lo_gb[2], dxv[0], dxv[1],
                                                  dxv[2], nx, ny, nz, px, py, pz, num);
}

void launch_negate(cudaStream_t s, int64_t n, double* a) { k_negate<<<grid1(n), kBlk1, 0, s>>>(n, a); }

}  // namespace qss
