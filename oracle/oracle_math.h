/*
 * oracle_math.h -- TEST INFRASTRUCTURE (oracle).  Portable sine/cosine used by
 * the oracle's restatement of the smoothed Heaviside and the volume integral.
 *
 * The reference evaluates SIN/COS through the platform libm (Fortran
 * intrinsics in src/utilities/qss_util3d.f:346-348, 466-467 and
 * src/spatial_derivatives/qss_spatial_derivatives3d.f:81, 166).  libm results
 * differ in the last bit between x86-64 and aarch64 builds and from any GPU
 * implementation, which would make bit-exact parity impossible.  Both the
 * oracle and the GPU kernels therefore evaluate sine with the same published
 * method, so the results agree bit for bit on every machine:
 *   - Cody & Waite argument reduction by pi/2 with a three-part constant
 *     (W. J. Cody, W. Waite, "Software Manual for the Elementary Functions",
 *     1980): P1, P2 carry 33 significant bits each, so k*P1 and k*P2 are exact
 *     for |k| < 2^20;
 *   - Taylor polynomials of sin (to r^17) and cos (to r^18) on |r| <= pi/4,
 *     evaluated by Horner's rule with coefficients 1/n! rounded to nearest.
 * The truncation error is below 1e-17 relative; the result is within about
 * one ulp of the true value.  Must be compiled without FMA contraction
 * (-ffp-contract=off).
 */
#ifndef ORACLE_MATH_H
#define ORACLE_MATH_H

#include <math.h>

#define QSSM_TWO_OVER_PI 0x1.45f306dc9c883p-1
#define QSSM_P1 0x1.921fb54400000p+0
#define QSSM_P2 0x1.0b4611a600000p-34
#define QSSM_P3 0x1.3198a2e037073p-69

#define QSSM_S3  0x1.5555555555555p-3
#define QSSM_S5  0x1.1111111111111p-7
#define QSSM_S7  0x1.a01a01a01a01ap-13
#define QSSM_S9  0x1.71de3a556c734p-19
#define QSSM_S11 0x1.ae64567f544e4p-26
#define QSSM_S13 0x1.6124613a86d09p-33
#define QSSM_S15 0x1.ae7f3e733b81fp-41
#define QSSM_S17 0x1.952c77030ad4ap-49

#define QSSM_C4  0x1.5555555555555p-5
#define QSSM_C6  0x1.6c16c16c16c17p-10
#define QSSM_C8  0x1.a01a01a01a01ap-16
#define QSSM_C10 0x1.27e4fb7789f5cp-22
#define QSSM_C12 0x1.1eed8eff8d898p-29
#define QSSM_C14 0x1.93974a8c07c9dp-37
#define QSSM_C16 0x1.ae7f3e733b81fp-45
#define QSSM_C18 0x1.6827863b97d97p-53

/* quarter-period polynomial: returns sin(x + q*pi/2) for the reduced r */
static inline double oracle_trig_core(double x, int q)
{
  double k = rint(x * QSSM_TWO_OVER_PI);
  double r = ((x - k * QSSM_P1) - k * QSSM_P2) - k * QSSM_P3;
  int n = ((int)k + q) & 3;
  double r2 = r * r;
  double v;
  if (n & 1) {
    double p = QSSM_C16 + r2 * (-QSSM_C18);
    p = -QSSM_C14 + r2 * p;
    p = QSSM_C12 + r2 * p;
    p = -QSSM_C10 + r2 * p;
    p = QSSM_C8 + r2 * p;
    p = -QSSM_C6 + r2 * p;
    p = QSSM_C4 + r2 * p;
    v = (1.0 - 0.5 * r2) + (r2 * r2) * p;
  } else {
    double p = -QSSM_S15 + r2 * QSSM_S17;
    p = QSSM_S13 + r2 * p;
    p = -QSSM_S11 + r2 * p;
    p = QSSM_S9 + r2 * p;
    p = -QSSM_S7 + r2 * p;
    p = QSSM_S5 + r2 * p;
    p = -QSSM_S3 + r2 * p;
    v = r + (r * r2) * p;
  }
  return (n & 2) ? -v : v;
}

#ifdef ORACLE_LIBM
/* The reference as linked: the platform libm's sine and cosine (the Fortran
 * intrinsics SIN/COS of qss_util3d.f:348, 467 and
 * qss_spatial_derivatives3d.f:81, 166).  Built as liboracle_libm.so, it
 * bounds what the portable evaluation changes in the results. */
static inline double oracle_sin(double x) { return sin(x); }
static inline double oracle_cos(double x) { return cos(x); }
#else
static inline double oracle_sin(double x) { return oracle_trig_core(x, 0); }
static inline double oracle_cos(double x) { return oracle_trig_core(x, 1); }
#endif

#endif
