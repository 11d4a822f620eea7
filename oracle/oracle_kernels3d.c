/*
 * oracle_kernels3d.c -- TEST INFRASTRUCTURE (oracle), never part of the product.
 *
 * C restatement of the 3-D Fortran-77 kernels of lsmpqs-1.0 that lie on the
 * quasi-static level-set path.  The Fortran sources cannot be compiled here
 * (no Fortran compiler), so this file stands in for them, with the same
 * symbol names and the Fortran calling convention (every argument by
 * pointer, arrays column-major with the ghost-box lower bounds), so that the
 * reference's own C drivers link against it unchanged.
 *
 * Arithmetic is the FP64 build of the reference (QSSLIB_REAL = double,
 * default REAL kind 8, so literals such as 1e-6 and 1.e-5 are doubles).
 * Expressions are evaluated in Fortran source order, left to right, one IEEE
 * operation at a time (build with -ffp-contract=off): x**2 is x*x, unary minus
 * binds looser than '*'.  Quirks of the reference are kept on purpose:
 *   - the CFL estimate max_H_over_dX is reset inside the voxel loop, so each
 *     call returns H of the LAST voxel of its box (3d.f:490, 935, 1222, 1712,
 *     2282);
 *   - getRHS3d5th adds +vel_n*|grad phi| where every other variant subtracts
 *     it (3d.f:2276 vs 484);
 *   - the ENO3 x-stencil reads phi(i+3,j,j) and the y/z minus derivatives are
 *     scaled by inv_dx (3d.f:677, 823, 900, 1454, 1600, 1677);
 *   - temp_norm is not reset when |vel_n| < 1e-5, so the previous voxel's value
 *     (in loop order) is reused.  The reference leaves it uninitialised at the
 *     start of a call; this restatement starts every call with 0.
 * Sine and cosine use the portable evaluation in oracle_math.h instead of
 * libm (see there for the reason).
 *
 * "3d.f" below is src/spatial_derivatives/qss_spatial_derivatives3d.f.
 */
#include <math.h>
#include <stddef.h>
#include "oracle_math.h"

#define GB_ARGS const int *ilo_gb, const int *ihi_gb, const int *jlo_gb, \
                const int *jhi_gb, const int *klo_gb, const int *khi_gb
#define FB_ARGS const int *ilo_fb, const int *ihi_fb, const int *jlo_fb, \
                const int *jhi_fb, const int *klo_fb, const int *khi_fb

/* column-major offset of (i,j,k) in an array with the given lower/upper bounds */
#define OFF(i, j, k, il, ih, jl, jh, kl)                                   \
  ((ptrdiff_t)((i) - (il)) + (ptrdiff_t)((ih) - (il) + 1) *               \
   ((ptrdiff_t)((j) - (jl)) + (ptrdiff_t)((jh) - (jl) + 1) * (ptrdiff_t)((k) - (kl))))

#define P(a, i, j, k) (a)[OFF(i, j, k, *ilo_gb, *ihi_gb, *jlo_gb, *jhi_gb, *klo_gb)]

static inline double fabs_(double x) { return fabs(x); }
static inline double max2(double a, double b) { return (a > b) ? a : b; }
static inline double min2(double a, double b) { return (a < b) ? a : b; }
/* Fortran SIGN(1.0, x): magnitude 1 with the sign bit of x */
static inline double sign1(double x) { return copysign(1.0, x); }

/* ------------------------------------------------------------------------ */
/* qss_util3d.f:450-493  smoothed Heaviside                                  */
static double basic_heaviside(double x)
{
  if (x < 0) return 0.0;
  if (x > 0) return 1.0;
  return 0.5; /* x == 0 (a NaN leaves the Fortran result undefined) */
}

static double qss_heaviside(double x, double eps)
{
  const double pi = 3.14159265358979323846;
  const double one_over_pi = 0.31830988618379;
  double v1 = basic_heaviside(x + eps);
  double v2 = basic_heaviside(eps - x);
  double v3 = basic_heaviside(x - eps);
  return (0.5 + x / (2 * eps) + (0.5 * one_over_pi) * oracle_sin((pi * x) / eps)) * v1 * v2 + v3;
}

/* ------------------------------------------------------------------------ */
/* 3d.f:13-87  normal velocity with constant contact angle                   */
void setvarnorm3d_(const double *mask, const double *mask_x, const double *mask_y,
                   const double *mask_z, double *var_a, const double *a0,
                   const double *ca, GB_ARGS, FB_ARGS, const double *dx)
{
  double eps_var = 1.5 * (*dx);
  double C2 = 1;
  for (int k = *klo_fb; k <= *khi_fb; k++)
    for (int j = *jlo_fb; j <= *jhi_fb; j++)
      for (int i = *ilo_fb; i <= *ihi_fb; i++) {
        double m = P(mask, i, j, k);
        double h1 = qss_heaviside(-m, eps_var);
        double h2 = qss_heaviside(m, eps_var);
        double mx = P(mask_x, i, j, k), my = P(mask_y, i, j, k), mz = P(mask_z, i, j, k);
        double absgrad = mx * mx + my * my + mz * mz;
        absgrad = sqrt(absgrad);
        double x = m * m + absgrad * (*dx) * absgrad * (*dx);
        x = sqrt(x);
        double s = m / x;
        P(var_a, i, j, k) = h1 * (*a0) - s * h2 * C2 * oracle_cos(*ca) * absgrad;
      }
}

/* 3d.f:94-172  normal velocity with a contact-angle field (dead in the
   reference drivers because of the '~' test, kept for completeness) */
void setvarnorm3dtheta_(const double *mask, const double *mask_x, const double *mask_y,
                        const double *mask_z, double *var_a, const double *a0,
                        const double *ca, GB_ARGS, FB_ARGS, const double *dx)
{
  double eps_var = 1.5 * (*dx);
  double C2 = 1;
  for (int k = *klo_fb; k <= *khi_fb; k++)
    for (int j = *jlo_fb; j <= *jhi_fb; j++)
      for (int i = *ilo_fb; i <= *ihi_fb; i++) {
        double m = P(mask, i, j, k);
        double h1 = qss_heaviside(-m, eps_var);
        double h2 = qss_heaviside(m, eps_var);
        double mx = P(mask_x, i, j, k), my = P(mask_y, i, j, k), mz = P(mask_z, i, j, k);
        double absgrad = mx * mx + my * my + mz * mz;
        absgrad = sqrt(absgrad);
        double x = m * m + absgrad * (*dx) * absgrad * (*dx);
        x = sqrt(x);
        double s = m / x;
        P(var_a, i, j, k) = h1 * (*a0) - s * h2 * C2 * oracle_cos(P(ca, i, j, k)) * absgrad;
      }
}

/* 3d.f:178-298  curvature coefficient b(x), advection field V(x) and the two
   CFL bounds (true maxima here, unlike the RHS routines) */
void setvarcurvadv3d_(const double *mask, const double *mask_x, const double *mask_y,
                      const double *mask_z, double *var_b, double *vel_x, double *vel_y,
                      double *vel_z, double *b_max_over_dx, double *max_U_over_dx,
                      const double *const_b, GB_ARGS, FB_ARGS, const double *dx)
{
  double eps_var = 1.5 * (*dx);
  double C1 = *const_b;
  double C2 = 1;
  *max_U_over_dx = -1.0;
  double b_max = -1.0;
  double inv_dx = 1.0 / (*dx), inv_dy = 1.0 / (*dx), inv_dz = 1.0 / (*dx);
  for (int k = *klo_fb; k <= *khi_fb; k++)
    for (int j = *jlo_fb; j <= *jhi_fb; j++)
      for (int i = *ilo_fb; i <= *ihi_fb; i++) {
        double m = P(mask, i, j, k);
        double h1 = qss_heaviside(-m, eps_var);
        double h2 = qss_heaviside(m, eps_var);
        double mx = P(mask_x, i, j, k), my = P(mask_y, i, j, k), mz = P(mask_z, i, j, k);
        double absgrad = mx * mx + my * my + mz * mz;
        absgrad = sqrt(absgrad);
        double x = m * m + absgrad * (*dx) * absgrad * (*dx);
        x = sqrt(x);
        double s = m / x;
        double vb = h1 * C1;
        P(var_b, i, j, k) = vb;
        if (vb > b_max) b_max = vb;
        double vx = s * C2 * mx * h2;
        double vy = s * C2 * my * h2;
        double vz = s * C2 * mz * h2;
        P(vel_x, i, j, k) = vx;
        P(vel_y, i, j, k) = vy;
        P(vel_z, i, j, k) = vz;
        double u = fabs_(vx) * inv_dx + fabs_(vy) * inv_dy + fabs_(vz) * inv_dz;
        if (u > *max_U_over_dx) *max_U_over_dx = u;
      }
  *b_max_over_dx = 2 * b_max * (inv_dx * inv_dx + inv_dy * inv_dy + inv_dz * inv_dz);
}

/* ------------------------------------------------------------------------ */
/* Upwind one-sided derivatives.  Each helper returns (plus, minus) for one
   direction at one voxel, written exactly as the Fortran statements. */

/* HJ ENO2 (3d.f:387-458): st[0..4] = phi at offsets -2..+2 along the axis */
static void eno2_pm(const double st[5], double inv, double *plus, double *minus)
{
  const double half = 0.5;
  double D1 = st[2] - st[1];
  double D1p = st[3] - st[2];
  double D2 = st[3] + st[1] - 2 * st[2];
  double D2p = st[4] + st[2] - 2 * st[3];
  double D2m = st[0] + st[2] - 2 * st[1];
  if (fabs_(D2) < fabs_(D2p)) *plus = (D1p - half * D2) * inv;
  else                        *plus = (D1p - half * D2p) * inv;
  if (fabs_(D2m) < fabs_(D2)) *minus = (D1 + half * D2m) * inv;
  else                        *minus = (D1 + half * D2) * inv;
}

/* HJ ENO3 (3d.f:672-903): st[0..6] = phi at offsets -3..+3; the caller
   substitutes the off-plane value for st[6] to keep the x typo, and passes
   inv_plus / inv_minus separately to keep the inv_dx scaling quirk. */
static void eno3_pm(const double st[7], double inv_plus, double inv_minus,
                    double *plus, double *minus)
{
  const double half = 0.5, third = 1.0 / 3.0, sixth = 1.0 / 6.0;
  double D1 = st[3] - st[2];
  double D1p = st[4] - st[3];
  double D1m = st[2] - st[1];
  double D1mm = st[1] - st[0];
  double D1pp = st[5] - st[4];
  double D1ppp = st[6] - st[5];
  double D2 = D1p - D1;
  double D2p = D1pp - D1p;
  double D2m = D1 - D1m;
  double D2pp = D1ppp - D1pp;
  double D2mm = D1m - D1mm;
  double D3 = D2 - D2m;
  double D3p = D2p - D2;
  double D3pp = D2pp - D2p;
  double D3m = D2m - D2mm;
  double p = D1p;
  if (fabs_(D2) < fabs_(D2p)) {
    p = p - half * D2;
    if (fabs_(D3) < fabs_(D3p)) p = p - sixth * D3;
    else                        p = p - sixth * D3p;
  } else {
    p = p - half * D2p;
    if (fabs_(D3p) < fabs_(D3pp)) p = p + third * D3p;
    else                           p = p + third * D3pp;
  }
  *plus = p * inv_plus;
  double m = D1;
  if (fabs_(D2m) < fabs_(D2)) {
    m = m + half * D2m;
    if (fabs_(D3m) < fabs_(D3)) m = m + third * D3m;
    else                        m = m + third * D3;
  } else {
    m = m + half * D2;
    if (fabs_(D3) < fabs_(D3p)) m = m - sixth * D3;
    else                        m = m - sixth * D3p;
  }
  *minus = m * inv_minus;
}

/* HJ WENO5 weights and reconstruction for one side (3d.f:1976-2005) */
static double weno5_side(double v1, double v2, double v3, double v4, double v5)
{
  const double tiny_nonzero_number = 1.0e-35;
  const double one_third = 1.0 / 3.0, seven_sixths = 7.0 / 6.0, eleven_sixths = 11.0 / 6.0;
  const double one_sixth = 1.0 / 6.0, five_sixths = 5.0 / 6.0;
  const double thirteen_twelfths = 13.0 / 12.0, one_fourth = 0.25;
  double m = max2(max2(max2(max2(v1 * v1, v2 * v2), v3 * v3), v4 * v4), v5 * v5);
  double eps = 1e-6 * m + tiny_nonzero_number;
  double p1 = one_third * v1 - seven_sixths * v2 + eleven_sixths * v3;
  double p2 = -(one_sixth * v2) + five_sixths * v3 + one_third * v4;
  double p3 = one_third * v3 + five_sixths * v4 - one_sixth * v5;
  double t;
  double S1, S2, S3;
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

/* st[0..6] = phi at offsets -3..+3 along the axis (3d.f:1962-2049) */
static void weno5_pm(const double st[7], double inv, double *plus, double *minus)
{
  double D1 = st[3] - st[2];
  double D1p = st[4] - st[3];
  double D1m = st[2] - st[1];
  double D1pp = st[5] - st[4];
  double D1ppp = st[6] - st[5];
  double D1mm = st[1] - st[0];
  *plus = weno5_side(D1ppp * inv, D1pp * inv, D1p * inv, D1 * inv, D1m * inv);
  *minus = weno5_side(D1mm * inv, D1m * inv, D1 * inv, D1p * inv, D1pp * inv);
}

/* ------------------------------------------------------------------------ */
/* Shared tail of every RHS routine: Godunov normal term, CFL estimate of the
   current voxel, upwind advection and the central curvature term. */
enum { RHS_ENO2 = 2, RHS_ENO3 = 3, RHS_WENO5 = 5 };

static void rhs_generic(int scheme, int var, const double *phi, const double *vel_n,
                        const double *b, const double *vel_x, const double *vel_y,
                        const double *vel_z, double *max_H_over_dX, double *lse_rhs,
                        GB_ARGS, FB_ARGS, const double *dx, const double *dy,
                        const double *dz)
{
  const double zero_tol = 1.e-5;
  double dx_factor = 0.5 / (*dx), dy_factor = 0.5 / (*dy), dz_factor = 0.5 / (*dz);
  double inv_dx = 1.0 / (*dx), inv_dy = 1.0 / (*dy), inv_dz = 1.0 / (*dz);
  double temp_norm = 0.0; /* carried over between voxels, see header */
  for (int k = *klo_fb; k <= *khi_fb; k++)
    for (int j = *jlo_fb; j <= *jhi_fb; j++)
      for (int i = *ilo_fb; i <= *ihi_fb; i++) {
        double pxp, pxm, pyp, pym, pzp, pzm;
        if (scheme == RHS_ENO2) {
          double sx[5], sy[5], sz[5];
          for (int o = -2; o <= 2; o++) {
            sx[o + 2] = P(phi, i + o, j, k);
            sy[o + 2] = P(phi, i, j + o, k);
            sz[o + 2] = P(phi, i, j, k + o);
          }
          eno2_pm(sx, inv_dx, &pxp, &pxm);
          eno2_pm(sy, inv_dy, &pyp, &pym);
          eno2_pm(sz, inv_dz, &pzp, &pzm);
        } else {
          double sx[7], sy[7], sz[7];
          for (int o = -3; o <= 3; o++) {
            sx[o + 3] = P(phi, i + o, j, k);
            sy[o + 3] = P(phi, i, j + o, k);
            sz[o + 3] = P(phi, i, j, k + o);
          }
          if (scheme == RHS_ENO3) {
            sx[6] = P(phi, i + 3, j, j); /* 3d.f:677 reads phi(i+3,j,j) */
            eno3_pm(sx, inv_dx, inv_dx, &pxp, &pxm);
            eno3_pm(sy, inv_dy, inv_dx, &pyp, &pym);
            eno3_pm(sz, inv_dz, inv_dx, &pzp, &pzm);
          } else {
            weno5_pm(sx, inv_dx, &pxp, &pxm);
            weno5_pm(sy, inv_dy, &pyp, &pym);
            weno5_pm(sz, inv_dz, &pzp, &pzm);
          }
        }

        double vel_n_cur = var ? P(vel_n, i, j, k) : *vel_n;
        if (fabs_(vel_n_cur) >= zero_tol) {
          double ngps;
          if (vel_n_cur > 0.0) {
            double ax = max2(pxm, 0.0), bx = min2(pxp, 0.0);
            double ay = max2(pym, 0.0), by = min2(pyp, 0.0);
            double az = max2(pzm, 0.0), bz = min2(pzp, 0.0);
            ngps = max2(ax * ax, bx * bx) + max2(ay * ay, by * by) + max2(az * az, bz * bz);
          } else {
            double ax = min2(pxm, 0.0), bx = max2(pxp, 0.0);
            double ay = min2(pym, 0.0), by = max2(pyp, 0.0);
            double az = min2(pzm, 0.0), bz = max2(pzp, 0.0);
            ngps = max2(ax * ax, bx * bx) + max2(ay * ay, by * by) + max2(az * az, bz * bz);
          }
          if (scheme == RHS_WENO5) temp_norm = vel_n_cur * sqrt(ngps);
          else                     temp_norm = -(vel_n_cur * sqrt(ngps));
        }

        /* CFL estimate of this voxel; the reset makes the last voxel win */
        *max_H_over_dX = -1.0;
        double mdx = max2(max2(*dx, *dy), *dz);
        double max_dx_sq = mdx * mdx;
        double pxc = max2(fabs_(pxp), fabs_(pxm));
        double pyc = max2(fabs_(pyp), fabs_(pym));
        double pzc = max2(fabs_(pzp), fabs_(pzm));
        double ngp = sqrt(pxc * pxc + pyc * pyc + pzc * pzc + max_dx_sq);
        double vabs = fabs_(var ? P(vel_n, i, j, k) : *vel_n);
        double H = vabs / ngp * (pxc * inv_dx + pyc * inv_dy + pzc * inv_dz);
        if (H > *max_H_over_dX) *max_H_over_dX = H;

        double temp_vel = 0.0;
        if (var) {
          double ax = (P(vel_x, i, j, k) >= 0) ? pxm : pxp;
          double ay = (P(vel_y, i, j, k) >= 0) ? pym : pyp;
          double az = (P(vel_z, i, j, k) >= 0) ? pzm : pzp;
          temp_vel = -(P(vel_x, i, j, k) * ax + P(vel_y, i, j, k) * ay + P(vel_z, i, j, k) * az);
        }

        double c = P(phi, i, j, k);
        double phi_x = (P(phi, i + 1, j, k) - P(phi, i - 1, j, k)) * dx_factor;
        double phi_y = (P(phi, i, j + 1, k) - P(phi, i, j - 1, k)) * dy_factor;
        double phi_z = (P(phi, i, j, k + 1) - P(phi, i, j, k - 1)) * dz_factor;
        double phi_xx = (P(phi, i + 2, j, k) + P(phi, i - 2, j, k) - 2 * c) * dx_factor * dx_factor;
        double phi_zz = (P(phi, i, j, k + 2) + P(phi, i, j, k - 2) - 2 * c) * dz_factor * dz_factor;
        double phi_yy = (P(phi, i, j + 2, k) + P(phi, i, j - 2, k) - 2 * c) * dy_factor * dy_factor;
        double phi_xy = (P(phi, i + 1, j + 1, k) + P(phi, i - 1, j - 1, k)
                         - P(phi, i - 1, j + 1, k) - P(phi, i + 1, j - 1, k)) * dx_factor * dy_factor;
        double phi_xz = (P(phi, i + 1, j, k + 1) + P(phi, i - 1, j, k - 1)
                         - P(phi, i - 1, j, k + 1) - P(phi, i + 1, j, k - 1)) * dx_factor * dz_factor;
        double phi_yz = (P(phi, i, j + 1, k + 1) + P(phi, i, j - 1, k - 1)
                         - P(phi, i, j - 1, k + 1) - P(phi, i, j + 1, k - 1)) * dy_factor * dz_factor;
        double grad_mag2 = phi_x * phi_x + phi_y * phi_y + phi_z * phi_z;
        double curv;
        if (grad_mag2 < zero_tol) {
          curv = 0.0;
        } else {
          curv = phi_xx * phi_y * phi_y
               + phi_yy * phi_x * phi_x
               - 2 * phi_xy * phi_x * phi_y
               + phi_xx * phi_z * phi_z
               + phi_zz * phi_x * phi_x
               - 2 * phi_xz * phi_x * phi_z
               + phi_yy * phi_z * phi_z
               + phi_zz * phi_y * phi_y
               - 2 * phi_yz * phi_y * phi_z;
          curv = curv / grad_mag2;
        }
        double temp_curv = (var ? P(b, i, j, k) : *b) * curv;
        if (var) P(lse_rhs, i, j, k) = temp_norm + temp_curv + temp_vel;
        else     P(lse_rhs, i, j, k) = temp_norm + temp_curv;
      }
}

/* 3d.f:302-567 */
void getrhs3d2ndconst_(const double *phi, const double *vel_n, const double *b,
                       double *max_H_over_dX, double *lse_rhs, GB_ARGS, FB_ARGS,
                       const double *dx, const double *dy, const double *dz)
{
  rhs_generic(RHS_ENO2, 0, phi, vel_n, b, 0, 0, 0, max_H_over_dX, lse_rhs,
              ilo_gb, ihi_gb, jlo_gb, jhi_gb, klo_gb, khi_gb,
              ilo_fb, ihi_fb, jlo_fb, jhi_fb, klo_fb, khi_fb, dx, dy, dz);
}

/* 3d.f:572-1011 */
void getrhs3d3rdconst_(const double *phi, const double *vel_n, const double *b,
                       double *max_H_over_dX, double *lse_rhs, GB_ARGS, FB_ARGS,
                       const double *dx, const double *dy, const double *dz)
{
  rhs_generic(RHS_ENO3, 0, phi, vel_n, b, 0, 0, 0, max_H_over_dX, lse_rhs,
              ilo_gb, ihi_gb, jlo_gb, jhi_gb, klo_gb, khi_gb,
              ilo_fb, ihi_fb, jlo_fb, jhi_fb, klo_fb, khi_fb, dx, dy, dz);
}

/* 3d.f:1020-1326 */
void getrhs3d2nd_(const double *phi, const double *vel_n, const double *b,
                  const double *vel_x, const double *vel_y, const double *vel_z,
                  double *max_H_over_dX, double *lse_rhs, GB_ARGS, FB_ARGS,
                  const double *dx, const double *dy, const double *dz)
{
  rhs_generic(RHS_ENO2, 1, phi, vel_n, b, vel_x, vel_y, vel_z, max_H_over_dX, lse_rhs,
              ilo_gb, ihi_gb, jlo_gb, jhi_gb, klo_gb, khi_gb,
              ilo_fb, ihi_fb, jlo_fb, jhi_fb, klo_fb, khi_fb, dx, dy, dz);
}

/* 3d.f:1335-1817 */
void getrhs3d3rd_(const double *phi, const double *vel_n, const double *b,
                  const double *vel_x, const double *vel_y, const double *vel_z,
                  double *max_H_over_dX, double *lse_rhs, GB_ARGS, FB_ARGS,
                  const double *dx, const double *dy, const double *dz)
{
  rhs_generic(RHS_ENO3, 1, phi, vel_n, b, vel_x, vel_y, vel_z, max_H_over_dX, lse_rhs,
              ilo_gb, ihi_gb, jlo_gb, jhi_gb, klo_gb, khi_gb,
              ilo_fb, ihi_fb, jlo_fb, jhi_fb, klo_fb, khi_fb, dx, dy, dz);
}

/* 3d.f:1827-2386 */
void getrhs3d5th_(const double *phi, const double *vel_n, const double *b,
                  const double *vel_x, const double *vel_y, const double *vel_z,
                  double *max_H_over_dX, double *lse_rhs, GB_ARGS, FB_ARGS,
                  const double *dx, const double *dy, const double *dz)
{
  rhs_generic(RHS_WENO5, 1, phi, vel_n, b, vel_x, vel_y, vel_z, max_H_over_dX, lse_rhs,
              ilo_gb, ihi_gb, jlo_gb, jhi_gb, klo_gb, khi_gb,
              ilo_fb, ihi_fb, jlo_fb, jhi_fb, klo_fb, khi_fb, dx, dy, dz);
}

/* ------------------------------------------------------------------------ */
/* 3d.f:2987-3048 */
void getcentralgrad3dorder2_(double *phi_x, double *phi_y, double *phi_z,
                             const int *ilo_g, const int *ihi_g, const int *jlo_g,
                             const int *jhi_g, const int *klo_g, const int *khi_g,
                             const double *phi, GB_ARGS, FB_ARGS,
                             const double *dx, const double *dy, const double *dz)
{
  double fx = 0.5 / (*dx), fy = 0.5 / (*dy), fz = 0.5 / (*dz);
  (void)khi_g;
  for (int k = *klo_fb; k <= *khi_fb; k++)
    for (int j = *jlo_fb; j <= *jhi_fb; j++)
      for (int i = *ilo_fb; i <= *ihi_fb; i++) {
        ptrdiff_t o = OFF(i, j, k, *ilo_g, *ihi_g, *jlo_g, *jhi_g, *klo_g);
        phi_x[o] = (P(phi, i + 1, j, k) - P(phi, i - 1, j, k)) * fx;
        phi_y[o] = (P(phi, i, j + 1, k) - P(phi, i, j - 1, k)) * fy;
        phi_z[o] = (P(phi, i, j, k + 1) - P(phi, i, j, k - 1)) * fz;
      }
}

/* 3d.f:3055-3191  signed linear extrapolation of one face */
void signedlinearextrapolation3d_(double *phi, GB_ARGS, FB_ARGS, const int *bdry_location_idx)
{
  int b = *bdry_location_idx;
  if (b == 0 || b == 1) {
    int f = (b == 0) ? *ilo_fb : *ihi_fb;
    int g = (b == 0) ? *ilo_fb + 1 : *ihi_fb - 1;
    for (int k = *klo_gb; k <= *khi_gb; k++)
      for (int j = *jlo_gb; j <= *jhi_gb; j++) {
        double s = sign1(P(phi, f, j, k));
        double slope = s * fabs_(P(phi, f, j, k) - P(phi, g, j, k));
        if (b == 0)
          for (int i = *ilo_gb; i <= *ilo_fb - 1; i++)
            P(phi, i, j, k) = P(phi, f, j, k) + slope * (double)(*ilo_fb - i);
        else
          for (int i = *ihi_fb + 1; i <= *ihi_gb; i++)
            P(phi, i, j, k) = P(phi, f, j, k) + slope * (double)(i - *ihi_fb);
      }
  } else if (b == 2 || b == 3) {
    int f = (b == 2) ? *jlo_fb : *jhi_fb;
    int g = (b == 2) ? *jlo_fb + 1 : *jhi_fb - 1;
    for (int i = *ilo_gb; i <= *ihi_gb; i++)
      for (int k = *klo_gb; k <= *khi_gb; k++) {
        double s = sign1(P(phi, i, f, k));
        double slope = s * fabs_(P(phi, i, f, k) - P(phi, i, g, k));
        if (b == 2)
          for (int j = *jlo_gb; j <= *jlo_fb - 1; j++)
            P(phi, i, j, k) = P(phi, i, f, k) + slope * (double)(*jlo_fb - j);
        else
          for (int j = *jhi_fb + 1; j <= *jhi_gb; j++)
            P(phi, i, j, k) = P(phi, i, f, k) + slope * (double)(j - *jhi_fb);
      }
  } else if (b == 4 || b == 5) {
    int f = (b == 4) ? *klo_fb : *khi_fb;
    int g = (b == 4) ? *klo_fb + 1 : *khi_fb - 1;
    for (int i = *ilo_gb; i <= *ihi_gb; i++)
      for (int j = *jlo_gb; j <= *jhi_gb; j++) {
        double s = sign1(P(phi, i, j, f));
        double slope = s * fabs_(P(phi, i, j, f) - P(phi, i, j, g));
        if (b == 4)
          for (int k = *klo_gb; k <= *klo_fb - 1; k++)
            P(phi, i, j, k) = P(phi, i, j, f) + slope * (double)(*klo_fb - k);
        else
          for (int k = *khi_fb + 1; k <= *khi_gb; k++)
            P(phi, i, j, k) = P(phi, i, j, f) + slope * (double)(k - *khi_fb);
      }
  }
}

/* ------------------------------------------------------------------------ */
/* src/time_integration/qss_tvd_runge_kutta3d.f:2-200.  All arrays share the
   same ghost box in every call of the path, so one set of bounds is used for
   indexing (the Fortran accepts separate bounds per array). */
#define RK_GB(n) const int *ilo_##n, const int *ihi_##n, const int *jlo_##n, \
                 const int *jhi_##n, const int *klo_##n, const int *khi_##n
#define PX(a, n, i, j, k) (a)[OFF(i, j, k, *ilo_##n, *ihi_##n, *jlo_##n, *jhi_##n, *klo_##n)]

void qss3drk1step_(double *u_next, RK_GB(a), const double *u_cur, RK_GB(b),
                   const double *rhs, RK_GB(c), FB_ARGS, const double *dt)
{
  (void)khi_a; (void)khi_b; (void)khi_c;
  for (int k = *klo_fb; k <= *khi_fb; k++)
    for (int j = *jlo_fb; j <= *jhi_fb; j++)
      for (int i = *ilo_fb; i <= *ihi_fb; i++)
        PX(u_next, a, i, j, k) = PX(u_cur, b, i, j, k) + (*dt) * PX(rhs, c, i, j, k);
}

void qss3dtvdrk2stage2_(double *u_stage2, RK_GB(a), const double *u_stage1, RK_GB(b),
                        const double *u_cur, RK_GB(c), const double *rhs, RK_GB(d),
                        FB_ARGS, const double *dt)
{
  (void)khi_a; (void)khi_b; (void)khi_c; (void)khi_d;
  for (int k = *klo_fb; k <= *khi_fb; k++)
    for (int j = *jlo_fb; j <= *jhi_fb; j++)
      for (int i = *ilo_fb; i <= *ihi_fb; i++)
        PX(u_stage2, a, i, j, k) = 0.75 * PX(u_cur, c, i, j, k)
                                 + 0.25 * (PX(u_stage1, b, i, j, k) + (*dt) * PX(rhs, d, i, j, k));
}

void qss3dtvdrk3stage3_(double *u_next, RK_GB(a), const double *u_stage2, RK_GB(b),
                        const double *u_cur, RK_GB(c), const double *rhs, RK_GB(d),
                        FB_ARGS, const double *dt)
{
  const double one_third = 1.0 / 3.0, two_thirds = 2.0 / 3.0;
  (void)khi_a; (void)khi_b; (void)khi_c; (void)khi_d;
  for (int k = *klo_fb; k <= *khi_fb; k++)
    for (int j = *jlo_fb; j <= *jhi_fb; j++)
      for (int i = *ilo_fb; i <= *ihi_fb; i++)
        PX(u_next, a, i, j, k) = one_third * PX(u_cur, c, i, j, k)
                               + two_thirds * (PX(u_stage2, b, i, j, k) + (*dt) * PX(rhs, d, i, j, k));
}

/* ------------------------------------------------------------------------ */
/* src/reinitialization/qss_reinitialization3d.f:476-579  Russo-Smereka
   subcell distance, -1000*max_dx away from the interface */
void qss3dcomputedistanceforsubcellfix_(double *distance0, const double *phi0, GB_ARGS,
                                        FB_ARGS, const double *dx, const double *dy,
                                        const double *dz)
{
  const double zero_tol = 1.e-5, zero = 0.0;
  double max_dx = max2(max2(*dx, *dy), *dz);
  double flag = -1000.0 * max_dx;
  for (int k = *klo_fb; k <= *khi_fb; k++)
    for (int j = *jlo_fb; j <= *jhi_fb; j++)
      for (int i = *ilo_fb; i <= *ihi_fb; i++) {
        double c = P(phi0, i, j, k);
        double n[6] = {P(phi0, i + 1, j, k), P(phi0, i - 1, j, k), P(phi0, i, j + 1, k),
                       P(phi0, i, j - 1, k), P(phi0, i, j, k + 1), P(phi0, i, j, k - 1)};
        int near = 0;
        for (int q = 0; q < 6; q++)
          near = near || (n[q] > zero && c <= zero) || (n[q] <= zero && c > zero);
        if (!near) {
          P(distance0, i, j, k) = flag;
        } else {
          double d1, d2, d3, delta;
          d1 = fabs_(n[0] - n[1]) / 2.0;
          d2 = fabs_(n[0] - c);
          d3 = fabs_(c - n[1]);
          delta = max2(max2(max2(d1, d2), d3), zero_tol);
          d1 = fabs_(n[2] - n[3]) / 2.0;
          d2 = fabs_(n[2] - c);
          d3 = fabs_(c - n[3]);
          delta = max2(max2(max2(d1, d2), d3), delta);
          d1 = fabs_(n[4] - n[5]) / 2.0;
          d2 = fabs_(n[4] - c);
          d3 = fabs_(c - n[5]);
          delta = max2(max2(max2(d1, d2), d3), delta);
          P(distance0, i, j, k) = c / delta;
        }
      }
}

/* qss_reinitialization3d.f:585-746  first-order Godunov reinitialisation RHS
   with the subcell fix near the interface */
void qss3dcomputereinitializationeqnrhssubcellfixorder1_(
    double *reinit_rhs, const double *phi, GB_ARGS, const double *phi0,
    const double *distance0, FB_ARGS, const double *dx, const double *dy, const double *dz)
{
  const double zero_tol = 1.e-5;
  double max_dx = max2(max2(*dx, *dy), *dz);
  double flag = -1000.0 * max_dx;
  double inv_dx = 1.0 / (*dx), inv_dy = 1.0 / (*dy), inv_dz = 1.0 / (*dz);
  for (int k = *klo_fb; k <= *khi_fb; k++)
    for (int j = *jlo_fb; j <= *jhi_fb; j++)
      for (int i = *ilo_fb; i <= *ihi_fb; i++) {
        double c = P(phi, i, j, k);
        double gp[3], gm[3];
        gp[0] = (P(phi, i + 1, j, k) - c) * inv_dx;
        gm[0] = (c - P(phi, i - 1, j, k)) * inv_dx;
        gp[1] = (P(phi, i, j + 1, k) - c) * inv_dy;
        gm[1] = (c - P(phi, i, j - 1, k)) * inv_dy;
        gp[2] = (P(phi, i, j, k + 1) - c) * inv_dz;
        gm[2] = (c - P(phi, i, j, k - 1)) * inv_dz;
        double p0 = P(phi0, i, j, k);
        double sgn = (fabs_(p0) > zero_tol) ? sign1(p0) : 0.0;
        double out;
        if (P(distance0, i, j, k) == flag) {
          double gs[3];
          for (int d = 0; d < 3; d++) {
            double a, bb;
            if (c > 0.0) { a = max2(-gp[d], 0.0); bb = max2(gm[d], 0.0); }
            else         { a = max2(gp[d], 0.0);  bb = max2(-gm[d], 0.0); }
            gs[d] = max2(a, bb);
          }
          if (fabs_(c) > zero_tol) {
            double ngps = gs[0] * gs[0] + gs[1] * gs[1] + gs[2] * gs[2];
            out = sgn - sgn * sqrt(ngps);
          } else {
            out = 0.0;
          }
        } else {
          out = P(distance0, i, j, k) - sgn * fabs_(c) / max_dx;
        }
        P(reinit_rhs, i, j, k) = out;
      }
}

/* ------------------------------------------------------------------------ */
/* qss_util3d.f:65-124 */
void qss3dmaxnormdifflocal_(double *max_norm_diff, const double *field1, GB_ARGS,
                            const double *field2, RK_GB(b), const int *ilo_ib,
                            const int *ihi_ib, const int *jlo_ib, const int *jhi_ib,
                            const int *klo_ib, const int *khi_ib, const double *local_zone)
{
  (void)khi_b;
  *max_norm_diff = -1.0;
  for (int k = *klo_ib; k <= *khi_ib; k++)
    for (int j = *jlo_ib; j <= *jhi_ib; j++)
      for (int i = *ilo_ib; i <= *ihi_ib; i++) {
        double f1 = P(field1, i, j, k);
        if (fabs_(f1) < *local_zone) {
          double d = fabs_(f1 - PX(field2, b, i, j, k));
          if (d > *max_norm_diff) *max_norm_diff = d;
        }
      }
}

/* qss_util3d.f:130-175 */
void imposemaskparallel_(double *phi_masked, const double *mask, const double *phi,
                         const double *overlap, GB_ARGS, const int *cur_klo_gb,
                         const int *cur_khi_gb)
{
  for (int k = *cur_klo_gb; k <= *cur_khi_gb; k++)
    for (int j = *jlo_gb; j <= *jhi_gb; j++)
      for (int i = *ilo_gb; i <= *ihi_gb; i++) {
        double m = P(mask, i, j, k) - *overlap;
        double p = P(phi, i, j, k);
        P(phi_masked, i, j, k) = (m > p) ? m : p;
      }
}

/* qss_util3d.f:181-228 (note: stores mask, not mask - overlap) */
void imposemaskparallelvar_(double *phi_masked, const double *mask, const double *phi,
                            const double *overlap, GB_ARGS, const int *cur_klo_gb,
                            const int *cur_khi_gb)
{
  for (int k = *cur_klo_gb; k <= *cur_khi_gb; k++)
    for (int j = *jlo_gb; j <= *jhi_gb; j++)
      for (int i = *ilo_gb; i <= *ihi_gb; i++) {
        double p = P(phi, i, j, k);
        if (P(mask, i, j, k) - P(overlap, i, j, k) > p) P(phi_masked, i, j, k) = P(mask, i, j, k);
        else                                           P(phi_masked, i, j, k) = p;
      }
}

/* qss_util3d.f:288-358  smoothed volume of {phi < 0}, summed in loop order */
void qss3dvolumeregionphilessthanzero_(double *volume, const double *phi, GB_ARGS,
                                       const int *ilo_ib, const int *ihi_ib,
                                       const int *jlo_ib, const int *jhi_ib,
                                       const int *klo_ib, const int *khi_ib,
                                       const double *dx, const double *dy,
                                       const double *dz, const double *epsilon)
{
  const double pi = 3.14159265358979323846;
  const double one_over_pi = 0.31830988618379;
  double dV = (*dx) * (*dy) * (*dz);
  double vol = 0.0;
  for (int k = *klo_ib; k <= *khi_ib; k++)
    for (int j = *jlo_ib; j <= *jhi_ib; j++)
      for (int i = *ilo_ib; i <= *ihi_ib; i++) {
        double phi_cur = P(phi, i, j, k);
        double r = phi_cur / (*epsilon);
        if (phi_cur < -(*epsilon)) {
          vol = vol + dV;
        } else if (phi_cur < *epsilon) {
          double one_minus_H = 0.5 * (1 - r - one_over_pi * oracle_sin(pi * r));
          vol = vol + one_minus_H * dV;
        }
      }
  *volume = vol;
}

/* qss_util3d.f:499-581.  The first array argument is the one tested; the
   drivers pass mask_nw there. */
void imposetrapvelocity3d_(const double *phi_w, const double *phi_nw, double *normal_velocity,
                           double *curvature_coeff, double *vel_x, double *vel_y,
                           double *vel_z, GB_ARGS, FB_ARGS, const double *dx)
{
  (void)phi_nw;
  double eps_var = 1.5 * (*dx);
  for (int k = *klo_fb; k <= *khi_fb; k++)
    for (int j = *jlo_fb; j <= *jhi_fb; j++)
      for (int i = *ilo_fb; i <= *ihi_fb; i++)
        if (P(phi_w, i, j, k) > eps_var) {
          P(normal_velocity, i, j, k) = 0;
          P(curvature_coeff, i, j, k) = 0;
          P(vel_x, i, j, k) = 0;
          P(vel_y, i, j, k) = 0;
          P(vel_z, i, j, k) = 0;
        }
}

/* Portable sine exported so tests can compare it with the GPU's copy. */
double oracle_portable_sin(double x) { return oracle_sin(x); }
double oracle_portable_cos(double x) { return oracle_cos(x); }
