// qss_emu.cuh -- IEEE-754 binary64 arithmetic (round to nearest even) on the
// integer pipes.
//
// On GB300 the FP64 pipe issues one warp instruction per ~64 cycles per
// scheduler, while the integer pipes accept one every one or two cycles, and
// the WENO5 kernels of this library keep the FP64 pipe 80-85 % busy with the
// integer pipes nearly idle.  The functions below compute the correctly
// rounded IEEE results of x/y, sqrt(x), x*y, x+y, exact power-of-two
// scalings and comparisons from the operands' bit patterns with 32/64-bit integer
// instructions, so that part of the FP64 work moves to otherwise idle
// pipes.  Each function has a fast path for normal operands whose result is
// normal (plus signed zeros where cheap) and falls back to the native FP64
// instruction for everything else (subnormals, infinities, NaNs, overflow,
// underflow), so every result is bit-identical to the native operation on
// all inputs.  The division reciprocal is seeded by the single-precision
// reciprocal approximation and refined by two Newton steps in fixed point;
// the quotient is then verified and corrected with its exact 128-bit integer
// remainder, so the reciprocal's accuracy affects only speed, never the
// result (a quotient still off after one correction falls back to native).
//
// The header compiles for the host too (g++), where the same code is tested
// against the host's IEEE double arithmetic.
#pragma once
#include <math.h>
#include <stdint.h>
#ifndef __CUDACC__
#include <string.h>
#endif

#ifdef __CUDACC__
#define QSS_EMU_HD __host__ __device__ __forceinline__
#else
#define QSS_EMU_HD static inline
#endif

// hooks for the host check: count fallbacks, perturb the reciprocal seed
#ifndef QSS_EMU_FALLBACK
#define QSS_EMU_FALLBACK(op, expr) (expr)
#endif
#ifndef QSS_EMU_SEED_ADJUST
#define QSS_EMU_SEED_ADJUST(rb) (rb)
#endif

namespace qss_emu {

constexpr uint64_t kMant = (1ull << 52) - 1;
constexpr uint64_t kHidden = 1ull << 52;
constexpr uint64_t kSign = 1ull << 63;
constexpr uint64_t kAbs = ~kSign;

QSS_EMU_HD uint64_t bits(double x) {
#ifdef __CUDA_ARCH__
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t u;
  memcpy(&u, &x, 8);
  return u;
#endif
}

QSS_EMU_HD double from_bits(uint64_t u) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)u);
#else
  double x;
  memcpy(&x, &u, 8);
  return x;
#endif
}

QSS_EMU_HD uint64_t umulhi(uint64_t a, uint64_t b) {
#ifdef __CUDA_ARCH__
  return __umul64hi(a, b);
#else
  return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

QSS_EMU_HD int clz64(uint64_t x) {
#ifdef __CUDA_ARCH__
  return __clzll((long long)x);
#else
  return x ? __builtin_clzll(x) : 64;
#endif
}

// 53 x 53-bit product of two mantissas as (hi, lo) of a 128-bit value, from
// four 32 x 32 -> 64-bit products (the high words are below 2^21)
QSS_EMU_HD void mul53(uint64_t a, uint64_t b, uint64_t& hi, uint64_t& lo) {
  const uint32_t a0 = (uint32_t)a, a1 = (uint32_t)(a >> 32);
  const uint32_t b0 = (uint32_t)b, b1 = (uint32_t)(b >> 32);
  const uint64_t p00 = (uint64_t)a0 * b0;
  const uint64_t mid = (uint64_t)a0 * b1 + (uint64_t)a1 * b0;  // < 2^54
  const uint64_t p11 = (uint64_t)a1 * b1;
  lo = p00 + (mid << 32);
  hi = p11 + (mid >> 32) + (lo < p00 ? 1u : 0u);
}

// ---------------------------------------------------------------------------
// reciprocal of a mantissa m in (2^52, 2^53): V ~ 2^116 / m in (2^63, 2^64)
//
// With D = m 2^11 in [2^63, 2^64) and Dh = D >> 32, the top 32 bits of V are
// S ~ 2^63 / Dh.  The seed S0 comes from the single-precision reciprocal
// approximation (about 2^-22 relative); one Newton step in 32-bit fixed
// point gives S1 to about 2^-31; one more step against the full D gives V to
// about 2^-62.  Only speed depends on these accuracies (see div()).

QSS_EMU_HD uint32_t recip_seed32(uint64_t D) {
  // single-precision value of the top 24 bits of D / 2^63, in [1, 2)
  const uint32_t fb = 0x3f800000u | (uint32_t)((D >> 40) & 0x7fffffu);
#ifdef __CUDA_ARCH__
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(__uint_as_float(fb)));
  uint32_t rb = __float_as_uint(r);
#else
  float f, r;
  memcpy(&f, &fb, 4);
  r = 1.0f / f;
  uint32_t rb;
  memcpy(&rb, &r, 4);
  rb = QSS_EMU_SEED_ADJUST(rb);
#endif
  // 1/f lies in (0.5, 1]; an approximation outside [0.5, 1) is clamped to the
  // nearest end, which keeps the seed within 2^-22 of the true value
  if (rb >= 0x3f800000u) return 0xffffffffu;
  if (rb < 0x3f000000u) return 0x80000000u;
  return ((rb & 0x7fffffu) | 0x800000u) << 8;  // r 2^32
}

QSS_EMU_HD uint64_t recip116(uint64_t m) {
  const uint64_t D = m << 11;
  const uint32_t Dh = (uint32_t)(D >> 32);
  uint32_t S = recip_seed32(D);
  {
    // E = 2^63 - Dh S (|E| < 2^43 for a seed within 2^-20), S <- S + S E / 2^63
    const int64_t E = (int64_t)((1ull << 63) - (uint64_t)Dh * S);
    const int64_t c = ((int64_t)S * (E >> 12)) >> 51;
    S = (uint32_t)((int64_t)S + c);
  }
  // T = D S (96 bits) as T >> 32; e = (2^95 - T) >> 32 (|e| < 2^34 for S
  // within 2^-29), V = S 2^32 + S e / 2^31
  const uint64_t lo = (D & 0xffffffffull) * S, hi = (D >> 32) * S;
  const uint64_t T32 = hi + (lo >> 32);
  const int64_t e = (int64_t)((1ull << 63) - T32);
  const int64_t c = ((int64_t)S * (e >> 3)) >> 28;
  return ((uint64_t)S << 32) + (uint64_t)c;
}

// ---------------------------------------------------------------------------
// x / y

QSS_EMU_HD double div(double x, double y) {
  const uint64_t bx = bits(x), by = bits(y);
  const uint32_t ex = (uint32_t)(bx >> 52) & 0x7ffu, ey = (uint32_t)(by >> 52) & 0x7ffu;
  if (ex - 1u < 2046u && ey - 1u < 2046u) {
    const uint64_t sign = (bx ^ by) & kSign;
    const uint64_t mx = (bx & kMant) | kHidden, my = (by & kMant) | kHidden;
    const int s = mx < my ? 1 : 0;
    const uint64_t N = mx << s;                  // N / my in [1, 2)
    const int e = (int)ex - (int)ey + 1023 - s;  // biased exponent of the quotient
    if (e >= 1 && e <= 2046) {
      uint64_t Q = N, R = 0;  // power-of-two divisor: exact
      bool ok = true;
      if (my != kHidden) {
        Q = umulhi(N, recip116(my));  // ~ floor(N 2^52 / my)
        // exact 128-bit N 2^52 - Q my = (rhi, rlo)
        uint64_t phi, plo;
        mul53(Q, my, phi, plo);
        const uint64_t nlo = N << 52;
        R = nlo - plo;
        const uint64_t rhi = (N >> 12) - phi - (nlo < plo ? 1u : 0u);
        if (rhi == 0) {
          if (R >= my) {  // Q one too small
            Q += 1;
            R -= my;
            ok = R < my;
          }
        } else if (rhi == ~0ull && R + my < my) {  // -my <= R < 0: Q one too large
          Q -= 1;
          R += my;
        } else {
          ok = false;
        }
      }
      if (ok && Q >= kHidden && Q < (kHidden << 1)) {
        const uint64_t r2 = R << 1;
        const uint64_t up = (r2 > my || (r2 == my && (Q & 1))) ? 1u : 0u;
        // (e - 1) << 52 plus the 53-bit significand: a carry out of the
        // significand increments the exponent (to infinity at the top)
        return from_bits(sign | ((((uint64_t)(e - 1)) << 52) + Q + up));
      }
    }
  }
  return QSS_EMU_FALLBACK(0, x / y);
}

// ---------------------------------------------------------------------------
// sqrt(x)
//
// x = M 2^(2k-52) with M = mx or 2 mx (53-54 bits) so that v = M / 2^52 lies
// in [1, 4); the significand is Q = floor(sqrt(M 2^52)) in [2^52, 2^53),
// rounded up when the remainder M 2^52 - Q^2 exceeds Q (no ties exist).  Q
// comes from the single-precision reciprocal square root, one Newton step in
// 32-bit fixed point and one correction against the full M; the exact
// 128-bit remainder then verifies and corrects it.

QSS_EMU_HD double sqrt(double x) {
  const uint64_t bx = bits(x);
  const uint32_t ex = (uint32_t)(bx >> 52);  // sign bit included: negative x fails the test
  if (ex - 1u < 2046u) {
    const int E = (int)ex - 1023;
    const int odd = E & 1;
    const uint64_t M = ((bx & kMant) | kHidden) << odd;  // v = M / 2^52 in [1, 4)
    const uint32_t fb = ((uint32_t)(127 + odd) << 23) | (uint32_t)((bx >> 29) & 0x7fffffu);
#ifdef __CUDA_ARCH__
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(__uint_as_float(fb)));
    uint32_t rb = __float_as_uint(r);
#else
    float f, r;
    memcpy(&f, &fb, 4);
    r = 1.0f / ::sqrtf(f);
    uint32_t rb;
    memcpy(&rb, &r, 4);
    rb = QSS_EMU_SEED_ADJUST(rb);
#endif
    // 1/sqrt(v) in (0.5, 1] as Y = r 2^32 (clamped to the interval)
    uint32_t Y;
    if (rb >= 0x3f800000u) Y = 0xffffffffu;
    else if (rb < 0x3f000000u) Y = 0x80000000u;
    else Y = ((rb & 0x7fffffu) | 0x800000u) << 8;
    const uint32_t Mt = (uint32_t)(M >> 22);  // v 2^30
    {
      // Newton step for the reciprocal square root: Y <- Y (3 - v Y^2) / 2
      const uint64_t G = (uint64_t)Mt * Y;                   // v r 2^62
      const uint64_t H = umulhi(G, (uint64_t)Y << 32);       // v r^2 2^62
      const int64_t d = (int64_t)((3ull << 62) - H);          // ~ 2^63 (3 - v r^2)/2 ... scaled below
      // Y (3 - v r^2) / 2 = Y d / 2^63
      const uint64_t t = umulhi((uint64_t)Y << 32, (uint64_t)d);  // Y d / 2^32
      Y = (uint32_t)(t >> 31);
    }
    // q0 = v r 2^52 (about 2^-30 relative), then q1 = q0 + (T - q0^2) r / 2
    uint64_t Q = ((uint64_t)Mt * Y) >> 10;
    {
      uint64_t shi, slo;
      mul53(Q, Q, shi, slo);
      const uint64_t tlo = M << 52, thi = M >> 12;
      const uint64_t elo = tlo - slo;
      const uint64_t ehi = thi - shi - (tlo < slo ? 1u : 0u);
      // e = (ehi:elo) signed, |e| < 2^80; e >> 16 fits 64 bits
      const int64_t e16 = (int64_t)((ehi << 48) | (elo >> 16));
      const bool neg = e16 < 0;
      const uint64_t ae = neg ? (uint64_t)(-e16) : (uint64_t)e16;
      // e r / 2 in units of Q: e16 2^16 Y / 2^32 / 2 / 2^52 = e16 Y / 2^69
      const uint64_t c = umulhi(ae, (uint64_t)Y << 32) >> 37;
      Q = neg ? Q - c : Q + c;
    }
    // exact remainder T - Q^2 and a correction of at most one unit
    uint64_t shi, slo;
    mul53(Q, Q, shi, slo);
    const uint64_t tlo = M << 52, thi = M >> 12;
    uint64_t R = tlo - slo;
    const uint64_t rhi = thi - shi - (tlo < slo ? 1u : 0u);
    bool ok = true;
    if (rhi == 0) {
      if (R > 2 * Q) {  // Q one too small
        Q += 1;
        R -= 2 * Q - 1;
        ok = R <= 2 * Q;
      }
    } else if (rhi == ~0ull && R + 2 * Q - 1 < 2 * Q - 1) {  // -(2Q - 1) <= R < 0: Q one too large
      R += 2 * Q - 1;
      Q -= 1;
    } else {
      ok = false;
    }
    if (ok && Q >= kHidden && Q < (kHidden << 1)) {
      const uint64_t up = R > Q ? 1u : 0u;
      const uint64_t eb = (uint64_t)((E >> 1) + 1023);
      return from_bits(((eb - 1) << 52) + Q + up);
    }
  } else if ((bx & kAbs) == 0) {
    return x;  // sqrt(+-0) = +-0
  }
  return QSS_EMU_FALLBACK(3, ::sqrt(x));
}

// ---------------------------------------------------------------------------
// x * y

QSS_EMU_HD double mul(double x, double y) {
  const uint64_t bx = bits(x), by = bits(y);
  const uint32_t ex = (uint32_t)(bx >> 52) & 0x7ffu, ey = (uint32_t)(by >> 52) & 0x7ffu;
  const uint64_t sign = (bx ^ by) & kSign;
  if (ex - 1u < 2046u && ey - 1u < 2046u) {
    const uint64_t mx = (bx & kMant) | kHidden, my = (by & kMant) | kHidden;
    uint64_t hi, lo;
    mul53(mx, my, hi, lo);  // product in [2^104, 2^106)
    const int top = (int)(hi >> 41);  // 1 if the product is >= 2^105
    const int e = (int)ex + (int)ey - 1023 + top;
    if (e >= 1 && e <= 2046) {
      uint64_t sig, rem, half;
      if (top) {
        sig = (hi << 11) | (lo >> 53);
        rem = lo & ((1ull << 53) - 1);
        half = 1ull << 52;
      } else {
        sig = (hi << 12) | (lo >> 52);
        rem = lo & ((1ull << 52) - 1);
        half = 1ull << 51;
      }
      const uint64_t up = (rem > half || (rem == half && (sig & 1))) ? 1u : 0u;
      return from_bits(sign | ((((uint64_t)(e - 1)) << 52) + sig + up));
    }
  } else if ((((bx & kAbs) == 0) && ey - 1u < 2046u) || (((by & kAbs) == 0) && ex - 1u < 2046u) ||
             (((bx | by) & kAbs) == 0)) {
    return from_bits(sign);  // zero times a finite nonzero normal, or zero times zero
  }
  return QSS_EMU_FALLBACK(1, x * y);
}

// ---------------------------------------------------------------------------
// x + y

QSS_EMU_HD double add(double x, double y) {
  uint64_t ba = bits(x), bb = bits(y);
  // order by magnitude: |a| >= |b|
  if ((bb & kAbs) > (ba & kAbs)) {
    const uint64_t t = ba;
    ba = bb;
    bb = t;
  }
  const uint32_t ea = (uint32_t)(ba >> 52) & 0x7ffu, eb = (uint32_t)(bb >> 52) & 0x7ffu;
  if (ea - 1u < 2046u) {
    if ((bb & kAbs) == 0) return from_bits(ba);  // a + (+-0) = a for a nonzero normal
    if (eb != 0) {
      const uint64_t A = ((ba & kMant) | kHidden) << 10;  // 63 bits
      uint64_t B = ((bb & kMant) | kHidden) << 10;
      const uint32_t d = ea - eb;
      if (d > 0) {
        if (d >= 63) {
          B = 1;  // only the sticky bit survives
        } else {
          const uint64_t lost = B & ((1ull << d) - 1);
          B = (B >> d) | (lost ? 1u : 0u);
        }
      }
      uint64_t S;
      int e = (int)ea;
      if (((ba ^ bb) & kSign) == 0) {
        S = A + B;  // < 2^64
        if (S >> 63) {
          S = (S >> 1) | (S & 1);
          e += 1;
        }
      } else {
        S = A - B;
        if (S == 0) return 0.0;  // exact cancellation: +0 in round-to-nearest
        const int sh = clz64(S) - 1;  // bring the leading one to bit 62
        S <<= sh;
        e -= sh;
      }
      if (e >= 1 && e <= 2046) {
        const uint64_t sig = S >> 10, rb = S & 0x3ffu;
        const uint64_t up = (rb > 0x200u || (rb == 0x200u && (sig & 1))) ? 1u : 0u;
        return from_bits((ba & kSign) | ((((uint64_t)(e - 1)) << 52) + sig + up));
      }
    }
  } else if ((ba & kAbs) == 0) {  // both zero
    return from_bits(ba & bb & kSign);
  }
  return QSS_EMU_FALLBACK(2, x + y);
}

QSS_EMU_HD double neg(double x);
QSS_EMU_HD double sub(double x, double y) { return add(x, neg(y)); }

// x * 2^k for a small integer k (exact unless the result leaves the normal range)
QSS_EMU_HD double scale2(double x, int k) {
  const uint64_t b = bits(x);
  const int e = (int)((b >> 52) & 0x7ffu);
  if (e >= 1 && e <= 2046 && e + k >= 1 && e + k <= 2046)
    return from_bits(b + ((uint64_t)(int64_t)k << 52));
  if ((b & kAbs) == 0) return x;
#ifdef __CUDA_ARCH__
  return x * __longlong_as_double((long long)((uint64_t)(1023 + k) << 52));
#else
  return x * from_bits((uint64_t)(1023 + k) << 52);
#endif
}

// ---------------------------------------------------------------------------
// sign flip and absolute value on the integer pipes.  Written as plain bit
// operations the compiler recognises them as FP64 negation / fabs and may
// issue them as FP64-pipe additions; the PTX logic op on the high word keeps
// them integer instructions.

QSS_EMU_HD double neg(double x) {
#ifdef __CUDA_ARCH__
  int hi = __double2hiint(x);
  asm("xor.b32 %0, %0, 0x80000000;" : "+r"(hi));
  return __hiloint2double(hi, __double2loint(x));
#else
  return from_bits(bits(x) ^ kSign);
#endif
}

QSS_EMU_HD double abs(double x) {
#ifdef __CUDA_ARCH__
  int hi = __double2hiint(x);
  asm("and.b32 %0, %0, 0x7fffffff;" : "+r"(hi));
  return __hiloint2double(hi, __double2loint(x));
#else
  return from_bits(bits(x) & kAbs);
#endif
}

// ---------------------------------------------------------------------------
// comparisons with IEEE semantics (false for NaN operands, -0 == +0)

QSS_EMU_HD bool isnan_bits(uint64_t b) { return (b & kAbs) > 0x7ff0000000000000ull; }

// x > 0
QSS_EMU_HD bool gt0(double x) {
  const int64_t b = (int64_t)bits(x);
  return b > 0 && (uint64_t)b <= 0x7ff0000000000000ull;
}
// x >= 0
QSS_EMU_HD bool ge0(double x) {
  const uint64_t b = bits(x);
  return ((int64_t)b >= 0 && b <= 0x7ff0000000000000ull) || b == kSign;
}
// x < 0
QSS_EMU_HD bool lt0(double x) {
  const uint64_t b = bits(x);
  return (int64_t)b < 0 && b != kSign && b <= 0xfff0000000000000ull;
}

// x > y
QSS_EMU_HD bool gt(double x, double y) {
  const uint64_t a = bits(x), b = bits(y);
  if (isnan_bits(a) || isnan_bits(b)) return false;
  if (((a | b) & kAbs) == 0) return false;  // both zero
  const int64_t ka = (int64_t)a >= 0 ? (int64_t)a : -(int64_t)(a & kAbs);
  const int64_t kb = (int64_t)b >= 0 ? (int64_t)b : -(int64_t)(b & kAbs);
  return ka > kb;
}

// max of two non-negative, non-NaN values (e.g. squares): bit patterns order
// like the values
QSS_EMU_HD double max_nonneg(double a, double b) {
  const int64_t ia = (int64_t)bits(a), ib = (int64_t)bits(b);
  return from_bits((uint64_t)(ia > ib ? ia : ib));
}

}  // namespace qss_emu
