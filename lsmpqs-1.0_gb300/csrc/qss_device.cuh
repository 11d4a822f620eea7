// qss_device.cuh -- device-side numerics of the quasi-static level-set path.
//
// Every function here evaluates the same IEEE-754 double operations, in the
// same order, as the lsmpqs Fortran kernels it replaces, so that results are
// bit-identical to an FP64 build of the reference.  The translation unit must
// be compiled with --fmad=false (no contraction of a*b+c into FMA); division
// and square root are the IEEE round-to-nearest versions (nvcc defaults).
//
// "3d.f" = src/spatial_derivatives/qss_spatial_derivatives3d.f of the reference.
#pragma once
#include <cstdint>

namespace qss {

// Index space of one volume: ghost box [0,nx)x[0,ny)x[0,nz), fill box
// [ilo,ihi]x[jlo,jhi]x[klo,khi], column-major with i fastest.
struct Box {
  int nx, ny, nz;
  int ilo, ihi, jlo, jhi, klo, khi;
  __host__ __device__ int64_t sx() const { return 1; }
  __host__ __device__ int64_t sy() const { return nx; }
  __host__ __device__ int64_t sz() const { return (int64_t)nx * ny; }
  __host__ __device__ int64_t idx(int i, int j, int k) const {
    return (int64_t)i + (int64_t)nx * ((int64_t)j + (int64_t)ny * k);
  }
  __host__ __device__ int64_t npts() const { return (int64_t)nx * ny * nz; }
  __host__ __device__ int fbx() const { return ihi - ilo + 1; }
  __host__ __device__ int fby() const { return jhi - jlo + 1; }
  __host__ __device__ int fbz() const { return khi - klo + 1; }
};

enum Scheme { ENO2 = 2, ENO3 = 3, WENO5 = 5 };

__device__ __forceinline__ double dmax(double a, double b) { return (a > b) ? a : b; }
__device__ __forceinline__ double dmin(double a, double b) { return (a < b) ? a : b; }

// ---------------------------------------------------------------------------
// Portable sine/cosine: Cody-Waite reduction by pi/2 (three-part constant,
// P1/P2 with 33 significant bits) and Taylor polynomials (1/n! coefficients,
// Horner form) on |r| <= pi/4.  The CPU oracle evaluates the identical
// sequence, so both sides agree bit for bit; the error is about 1 ulp.
__device__ __forceinline__ double trig_core(double x, int q) {
  const double two_over_pi = 0x1.45f306dc9c883p-1;
  const double P1 = 0x1.921fb54400000p+0, P2 = 0x1.0b4611a600000p-34, P3 = 0x1.3198a2e037073p-69;
  double k = rint(x * two_over_pi);
  double r = __dsub_rn(__dsub_rn(__dsub_rn(x, __dmul_rn(k, P1)), __dmul_rn(k, P2)), __dmul_rn(k, P3));
  int n = ((int)k + q) & 3;
  double r2 = r * r;
  double v;
  if (n & 1) {
    double p = 0x1.ae7f3e733b81fp-45 + r2 * (-0x1.6827863b97d97p-53);
    p = -0x1.93974a8c07c9dp-37 + r2 * p;
    p = 0x1.1eed8eff8d898p-29 + r2 * p;
    p = -0x1.27e4fb7789f5cp-22 + r2 * p;
    p = 0x1.a01a01a01a01ap-16 + r2 * p;
    p = -0x1.6c16c16c16c17p-10 + r2 * p;
    p = 0x1.5555555555555p-5 + r2 * p;
    v = (1.0 - 0.5 * r2) + (r2 * r2) * p;
  } else {
    double p = -0x1.ae7f3e733b81fp-41 + r2 * 0x1.952c77030ad4ap-49;
    p = 0x1.6124613a86d09p-33 + r2 * p;
    p = -0x1.ae64567f544e4p-26 + r2 * p;
    p = 0x1.71de3a556c734p-19 + r2 * p;
    p = -0x1.a01a01a01a01ap-13 + r2 * p;
    p = 0x1.1111111111111p-7 + r2 * p;
    p = -0x1.5555555555555p-3 + r2 * p;
    v = r + (r * r2) * p;
  }
  return (n & 2) ? -v : v;
}
__device__ __forceinline__ double portable_sin(double x) { return trig_core(x, 0); }
__device__ __forceinline__ double portable_cos(double x) { return trig_core(x, 1); }

// qss_util3d.f:450-493
__device__ __forceinline__ double basic_heaviside(double x) {
  if (x < 0) return 0.0;
  if (x > 0) return 1.0;
  return 0.5;
}
__device__ __forceinline__ double qss_heaviside(double x, double eps) {
  const double pi = 3.14159265358979323846;
  const double one_over_pi = 0.31830988618379;
  double v1 = basic_heaviside(x + eps);
  double v2 = basic_heaviside(eps - x);
  double v3 = basic_heaviside(x - eps);
  return (0.5 + x / (2 * eps) + (0.5 * one_over_pi) * portable_sin((pi * x) / eps)) * v1 * v2 + v3;
}

// ---------------------------------------------------------------------------
// One-sided derivatives along one axis.  s[] holds phi at offsets -R..+R.

// HJ ENO2, 3d.f:387-458 (R = 2)
__device__ __forceinline__ void eno2_pm(const double s[5], double inv, double& plus, double& minus) {
  const double half = 0.5;
  double D1 = s[2] - s[1];
  double D1p = s[3] - s[2];
  double D2 = s[3] + s[1] - 2 * s[2];
  double D2p = s[4] + s[2] - 2 * s[3];
  double D2m = s[0] + s[2] - 2 * s[1];
  plus = (fabs(D2) < fabs(D2p)) ? (D1p - half * D2) * inv : (D1p - half * D2p) * inv;
  minus = (fabs(D2m) < fabs(D2)) ? (D1 + half * D2m) * inv : (D1 + half * D2) * inv;
}

// HJ ENO3, 3d.f:672-903 (R = 3); the y/z minus derivatives are scaled by
// inv_dx in the reference, so the two scalings are passed separately.
__device__ __forceinline__ void eno3_pm(const double s[7], double inv_p, double inv_m, double& plus,
                                        double& minus) {
  const double half = 0.5, third = 1.0 / 3.0, sixth = 1.0 / 6.0;
  double D1 = s[3] - s[2], D1p = s[4] - s[3], D1m = s[2] - s[1], D1mm = s[1] - s[0];
  double D1pp = s[5] - s[4], D1ppp = s[6] - s[5];
  double D2 = D1p - D1, D2p = D1pp - D1p, D2m = D1 - D1m, D2pp = D1ppp - D1pp, D2mm = D1m - D1mm;
  double D3 = D2 - D2m, D3p = D2p - D2, D3pp = D2pp - D2p, D3m = D2m - D2mm;
  double p = D1p;
  if (fabs(D2) < fabs(D2p)) {
    p = p - half * D2;
    p = (fabs(D3) < fabs(D3p)) ? p - sixth * D3 : p - sixth * D3p;
  } else {
    p = p - half * D2p;
    p = (fabs(D3p) < fabs(D3pp)) ? p + third * D3p : p + third * D3pp;
  }
  plus = p * inv_p;
  double m = D1;
  if (fabs(D2m) < fabs(D2)) {
    m = m + half * D2m;
    m = (fabs(D3m) < fabs(D3)) ? m + third * D3m : m + third * D3;
  } else {
    m = m + half * D2;
    m = (fabs(D3) < fabs(D3p)) ? m - sixth * D3 : m - sixth * D3p;
  }
  minus = m * inv_m;
}

// HJ WENO5 weights and reconstruction of one side, 3d.f:1976-2005
__device__ __forceinline__ double weno5_side(double v1, double v2, double v3, double v4, double v5) {
  const double tiny_nonzero_number = 1.0e-35;
  const double one_third = 1.0 / 3.0, seven_sixths = 7.0 / 6.0, eleven_sixths = 11.0 / 6.0;
  const double one_sixth = 1.0 / 6.0, five_sixths = 5.0 / 6.0;
  const double thirteen_twelfths = 13.0 / 12.0, one_fourth = 0.25;
  double m = dmax(dmax(dmax(dmax(v1 * v1, v2 * v2), v3 * v3), v4 * v4), v5 * v5);
  double eps = 1e-6 * m + tiny_nonzero_number;
  double p1 = one_third * v1 - seven_sixths * v2 + eleven_sixths * v3;
  double p2 = -(one_sixth * v2) + five_sixths * v3 + one_third * v4;
  double p3 = one_third * v3 + five_sixths * v4 - one_sixth * v5;
  double t, S1, S2, S3;
  t = v1 - 2.0 * v2 + v3;       S1 = thirteen_twelfths * (t * t);
  t = v1 - 4.0 * v2 + 3.0 * v3; S1 = S1 + one_fourth * (t * t);
  t = v2 - 2.0 * v3 + v4;       S2 = thirteen_twelfths * (t * t);
  t = v2 - v4;                  S2 = S2 + one_fourth * (t * t);
  t = v3 - 2.0 * v4 + v5;       S3 = thirteen_twelfths * (t * t);
  t = 3.0 * v3 - 4.0 * v4 + v5; S3 = S3 + one_fourth * (t * t);
  double a1, a2, a3;
  t = S1 + eps; a1 = 0.1 / (t * t);
  t = S2 + eps; a2 = 0.6 / (t * t);
  t = S3 + eps; a3 = 0.3 / (t * t);
  double inv_sum_a = 1.0 / (a1 + a2 + a3);
  a1 = a1 * inv_sum_a;
  a2 = a2 * inv_sum_a;
  a3 = a3 * inv_sum_a;
  return a1 * p1 + a2 * p2 + a3 * p3;
}

// 3d.f:1962-2049 (R = 3)
__device__ __forceinline__ void weno5_pm(const double s[7], double inv, double& plus, double& minus) {
  double D1 = s[3] - s[2], D1p = s[4] - s[3], D1m = s[2] - s[1];
  double D1pp = s[5] - s[4], D1ppp = s[6] - s[5], D1mm = s[1] - s[0];
  plus = weno5_side(D1ppp * inv, D1pp * inv, D1p * inv, D1 * inv, D1m * inv);
  minus = weno5_side(D1mm * inv, D1m * inv, D1 * inv, D1p * inv, D1pp * inv);
}

struct Inv {
  double x, y, z;
};

// Upwind plus/minus derivatives of phi at (i,j,k) for the given scheme.
// The ENO3 x-stencil reproduces the reference's read of phi(i+3,j,j).
template <int SCHEME>
__device__ __forceinline__ void upwind(const double* __restrict__ phi, const Box& b, int i, int j, int k,
                                       const Inv& inv, double pp[3], double pm[3]) {
  const int64_t c = b.idx(i, j, k), sy = b.sy(), sz = b.sz();
  if (SCHEME == ENO2) {
    double sx_[5], sy_[5], sz_[5];
#pragma unroll
    for (int o = -2; o <= 2; o++) {
      sx_[o + 2] = __ldg(phi + c + o);
      sy_[o + 2] = __ldg(phi + c + o * sy);
      sz_[o + 2] = __ldg(phi + c + o * sz);
    }
    eno2_pm(sx_, inv.x, pp[0], pm[0]);
    eno2_pm(sy_, inv.y, pp[1], pm[1]);
    eno2_pm(sz_, inv.z, pp[2], pm[2]);
  } else {
    double sx_[7], sy_[7], sz_[7];
#pragma unroll
    for (int o = -3; o <= 3; o++) {
      sx_[o + 3] = __ldg(phi + c + o);
      sy_[o + 3] = __ldg(phi + c + o * sy);
      sz_[o + 3] = __ldg(phi + c + o * sz);
    }
    if (SCHEME == ENO3) {
      sx_[6] = __ldg(phi + b.idx(i + 3, j, j));  // 3d.f:677
      eno3_pm(sx_, inv.x, inv.x, pp[0], pm[0]);
      eno3_pm(sy_, inv.y, inv.x, pp[1], pm[1]);
      eno3_pm(sz_, inv.z, inv.x, pp[2], pm[2]);
    } else {
      weno5_pm(sx_, inv.x, pp[0], pm[0]);
      weno5_pm(sy_, inv.y, pp[1], pm[1]);
      weno5_pm(sz_, inv.z, pp[2], pm[2]);
    }
  }
}

// Godunov normal term; WENO5 adds +vel*|grad| (3d.f:2276), the others subtract.
template <int SCHEME>
__device__ __forceinline__ double godunov_norm(double vel, const double pp[3], const double pm[3]) {
  double ngps;
  if (vel > 0.0) {
    double ax = dmax(pm[0], 0.0), bx = dmin(pp[0], 0.0);
    double ay = dmax(pm[1], 0.0), by = dmin(pp[1], 0.0);
    double az = dmax(pm[2], 0.0), bz = dmin(pp[2], 0.0);
    ngps = dmax(ax * ax, bx * bx) + dmax(ay * ay, by * by) + dmax(az * az, bz * bz);
  } else {
    double ax = dmin(pm[0], 0.0), bx = dmax(pp[0], 0.0);
    double ay = dmin(pm[1], 0.0), by = dmax(pp[1], 0.0);
    double az = dmin(pm[2], 0.0), bz = dmax(pp[2], 0.0);
    ngps = dmax(ax * ax, bx * bx) + dmax(ay * ay, by * by) + dmax(az * az, bz * bz);
  }
  if (SCHEME == WENO5) return vel * sqrt(ngps);
  return -(vel * sqrt(ngps));
}

// CFL estimate H/dx of one voxel (3d.f:490-512)
__device__ __forceinline__ double cfl_h(double vel, const double pp[3], const double pm[3], double dx,
                                        double dy, double dz, const Inv& inv) {
  double mdx = dmax(dmax(dx, dy), dz);
  double max_dx_sq = mdx * mdx;
  double pxc = dmax(fabs(pp[0]), fabs(pm[0]));
  double pyc = dmax(fabs(pp[1]), fabs(pm[1]));
  double pzc = dmax(fabs(pp[2]), fabs(pm[2]));
  double ngp = sqrt(pxc * pxc + pyc * pyc + pzc * pzc + max_dx_sq);
  return fabs(vel) / ngp * (pxc * inv.x + pyc * inv.y + pzc * inv.z);
}

struct Fac {
  double x, y, z;  // 0.5/dx ...
};

// Central curvature term b*kappa|grad phi| with 2-cell second differences
// (3d.f:2337-2379)
__device__ __forceinline__ double curvature(const double* __restrict__ phi, const Box& b, int64_t c,
                                            const Fac& f) {
  const int64_t sy = b.sy(), sz = b.sz();
  const double zero_tol = 1.e-5;
  double cc = __ldg(phi + c);
  double phi_x = (__ldg(phi + c + 1) - __ldg(phi + c - 1)) * f.x;
  double phi_y = (__ldg(phi + c + sy) - __ldg(phi + c - sy)) * f.y;
  double phi_z = (__ldg(phi + c + sz) - __ldg(phi + c - sz)) * f.z;
  double phi_xx = (__ldg(phi + c + 2) + __ldg(phi + c - 2) - 2 * cc) * f.x * f.x;
  double phi_zz = (__ldg(phi + c + 2 * sz) + __ldg(phi + c - 2 * sz) - 2 * cc) * f.z * f.z;
  double phi_yy = (__ldg(phi + c + 2 * sy) + __ldg(phi + c - 2 * sy) - 2 * cc) * f.y * f.y;
  double phi_xy = (__ldg(phi + c + 1 + sy) + __ldg(phi + c - 1 - sy) - __ldg(phi + c - 1 + sy) -
                   __ldg(phi + c + 1 - sy)) * f.x * f.y;
  double phi_xz = (__ldg(phi + c + 1 + sz) + __ldg(phi + c - 1 - sz) - __ldg(phi + c - 1 + sz) -
                   __ldg(phi + c + 1 - sz)) * f.x * f.z;
  double phi_yz = (__ldg(phi + c + sy + sz) + __ldg(phi + c - sy - sz) - __ldg(phi + c - sy + sz) -
                   __ldg(phi + c + sy - sz)) * f.y * f.z;
  double grad_mag2 = phi_x * phi_x + phi_y * phi_y + phi_z * phi_z;
  if (grad_mag2 < zero_tol) return 0.0;
  double curv = phi_xx * phi_y * phi_y + phi_yy * phi_x * phi_x - 2 * phi_xy * phi_x * phi_y +
                phi_xx * phi_z * phi_z + phi_zz * phi_x * phi_x - 2 * phi_xz * phi_x * phi_z +
                phi_yy * phi_z * phi_z + phi_zz * phi_y * phi_y - 2 * phi_yz * phi_y * phi_z;
  return curv / grad_mag2;
}

// Signed linear extrapolation of the six faces applied in the reference's
// order x-lo, x-hi, y-lo, y-hi, z-lo, z-hi (3d.f:3055-3191,
// qss_general_util.c:630-698), written as a closed function of fill-box
// values: the value stored at a ghost point equals the one the sequential
// face sweeps would leave there.
__device__ __forceinline__ double extrap(double f, double g, int dist) {
  double s = copysign(1.0, f);
  double slope = s * fabs(f - g);
  return f + slope * (double)dist;
}

// value after the x faces at (i, j, k) with j, k inside the fill box
__device__ __forceinline__ double bc_x(const double* __restrict__ a, const Box& b, int i, int j, int k) {
  if (i < b.ilo) return extrap(a[b.idx(b.ilo, j, k)], a[b.idx(b.ilo + 1, j, k)], b.ilo - i);
  if (i > b.ihi) return extrap(a[b.idx(b.ihi, j, k)], a[b.idx(b.ihi - 1, j, k)], i - b.ihi);
  return a[b.idx(i, j, k)];
}
// value after the x and y faces at (i, j, k) with k inside the fill box
__device__ __forceinline__ double bc_xy(const double* __restrict__ a, const Box& b, int i, int j, int k) {
  if (j < b.jlo) return extrap(bc_x(a, b, i, b.jlo, k), bc_x(a, b, i, b.jlo + 1, k), b.jlo - j);
  if (j > b.jhi) return extrap(bc_x(a, b, i, b.jhi, k), bc_x(a, b, i, b.jhi - 1, k), j - b.jhi);
  return bc_x(a, b, i, j, k);
}
// value after all six faces at any ghost-box point
__device__ __forceinline__ double bc_xyz(const double* __restrict__ a, const Box& b, int i, int j, int k) {
  if (k < b.klo) return extrap(bc_xy(a, b, i, j, b.klo), bc_xy(a, b, i, j, b.klo + 1), b.klo - k);
  if (k > b.khi) return extrap(bc_xy(a, b, i, j, b.khi), bc_xy(a, b, i, j, b.khi - 1), k - b.khi);
  return bc_xy(a, b, i, j, k);
}

}  // namespace qss
