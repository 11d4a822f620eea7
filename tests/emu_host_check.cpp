// Host check of the integer-pipe FP64 arithmetic (qss_emu.cuh) against the
// host's IEEE-754 double arithmetic: every emulated result must equal the
// native one bit for bit.  Usage: emu_host_check <cases per family> <seed>
// Prints one line per operation with the number of mismatches; exit code 1
// when any mismatch is found.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cstdint>
#include <initializer_list>

static long long g_fallback[4];
static int g_family;  // operand family of the current case (fallbacks are counted for family 1)
#define QSS_EMU_FALLBACK(op, expr) ((g_family == 1 ? g_fallback[op]++ : 0), (expr))
static uint64_t g_jitter_state = 1;
static int g_jitter;  // perturbs the reciprocal seed by up to +-g_jitter units in the last place
static uint32_t jitter(uint32_t rb) {
  if (!g_jitter) return rb;
  g_jitter_state = g_jitter_state * 6364136223846793005ull + 1442695040888963407ull;
  const int d = (int)((g_jitter_state >> 33) % (uint64_t)(2 * g_jitter + 1)) - g_jitter;
  return rb + (uint32_t)d;
}
#define QSS_EMU_SEED_ADJUST(rb) jitter(rb)
#include "qss_emu.cuh"

namespace {

uint64_t g_state;
uint64_t rnd() {  // xorshift64*
  g_state ^= g_state >> 12;
  g_state ^= g_state << 25;
  g_state ^= g_state >> 27;
  return g_state * 2685821657736338717ull;
}

double dbl(uint64_t b) {
  double x;
  memcpy(&x, &b, 8);
  return x;
}
uint64_t bts(double x) {
  uint64_t b;
  memcpy(&b, &x, 8);
  return b;
}

// operand families: raw bit patterns (all classes), normals in a moderate
// range, short significands (exact products / sums / ties), neighbours of
// another operand (cancellation, quotients near 1), special values
double operand(int fam, double other) {
  switch (fam) {
    case 0:
      return dbl(rnd());
    case 1: {
      const uint64_t e = 1023 - 60 + rnd() % 120;
      return dbl((rnd() & (1ull << 63)) | (e << 52) | (rnd() & qss_emu::kMant));
    }
    case 2: {
      const uint64_t e = 1023 - 8 + rnd() % 16;
      const int keep = 1 + (int)(rnd() % 30);
      const uint64_t m = rnd() & qss_emu::kMant & ~((1ull << (52 - keep)) - 1);
      return dbl((rnd() & (1ull << 63)) | (e << 52) | m);
    }
    case 3: {
      const int64_t d = (int64_t)(rnd() % 2001) - 1000;
      uint64_t b = bts(other) + (uint64_t)d;
      if (rnd() & 1) b ^= 1ull << 63;
      return dbl(b);
    }
    case 4: {
      static const double sp[] = {0.0, -0.0, 1.0, -1.0, 0.5, 2.0, 0.1, 0.6, 0.3, 1e-35, 1e-300,
                                  1e300, 4.9e-324, 2.2250738585072014e-308, 1.7976931348623157e308,
                                  INFINITY, -INFINITY, NAN};
      return sp[rnd() % (sizeof sp / sizeof sp[0])];
    }
    default: {  // near the edges of the normal range
      const uint64_t e = (rnd() & 1) ? 1 + rnd() % 60 : 2046 - rnd() % 60;
      return dbl((rnd() & (1ull << 63)) | (e << 52) | (rnd() & qss_emu::kMant));
    }
  }
}

bool same(double a, double b) {
  if (std::isnan(a) && std::isnan(b)) return true;  // NaN payloads may differ
  return bts(a) == bts(b);
}

struct Count {
  const char* name;
  long long bad = 0, n = 0;
};

}  // namespace

int main(int argc, char** argv) {
  const long long cases = argc > 1 ? atoll(argv[1]) : 1000000;
  g_state = argc > 2 ? strtoull(argv[2], nullptr, 10) | 1 : 88172645463325252ull;
  g_jitter = argc > 3 ? atoi(argv[3]) : 0;
  long long fam1 = 0;
  Count c_sqrt{"sqrt"}, c_div{"div"}, c_mul{"mul"}, c_add{"add"}, c_sub{"sub"}, c_sc{"scale2"}, c_cmp{"compare"},
      c_max{"max_nonneg"}, c_sign{"neg_abs"};
  int shown = 0;
  auto report = [&](const char* op, double x, double y, double got, double want) {
    if (shown++ < 12)
      printf("  %s(%a, %a) = %a, native %a\n", op, x, y, got, want);
  };
  for (long long i = 0; i < cases; i++) {
    const int fx = (int)(rnd() % 6), fy = (int)(rnd() % 6);
    const double x = operand(fx == 3 ? 1 : fx, 1.0);
    const double y = operand(fy, x);
    g_family = (fx == 1 || fx == 3) && fy == 1 ? 1 : 0;
    fam1 += g_family;
    double g, w;
    g = qss_emu::sqrt(x), w = std::sqrt(x);
    c_sqrt.n++;
    if (!same(g, w)) c_sqrt.bad++, report("sqrt", x, 0, g, w);
    g = qss_emu::div(x, y), w = x / y;
    c_div.n++;
    if (!same(g, w)) c_div.bad++, report("div", x, y, g, w);
    g = qss_emu::mul(x, y), w = x * y;
    c_mul.n++;
    if (!same(g, w)) c_mul.bad++, report("mul", x, y, g, w);
    g = qss_emu::add(x, y), w = x + y;
    c_add.n++;
    if (!same(g, w)) c_add.bad++, report("add", x, y, g, w);
    g = qss_emu::sub(x, y), w = x - y;
    c_sub.n++;
    if (!same(g, w)) c_sub.bad++, report("sub", x, y, g, w);
    // sign flip and magnitude: bit for bit, NaN sign bits included
    c_sign.n++;
    if (bts(qss_emu::neg(x)) != bts(-x) || bts(qss_emu::abs(x)) != bts(std::fabs(x)))
      c_sign.bad++, report("neg_abs", x, 0, qss_emu::neg(x), -x);
    const int k = (int)(rnd() % 9) - 4;
    g = qss_emu::scale2(x, k), w = x * std::ldexp(1.0, k);
    c_sc.n++;
    if (!same(g, w)) c_sc.bad++, report("scale2", x, (double)k, g, w);
    c_cmp.n++;
    if (qss_emu::gt0(x) != (x > 0) || qss_emu::ge0(x) != (x >= 0) || qss_emu::lt0(x) != (x < 0) ||
        qss_emu::gt(x, y) != (x > y))
      c_cmp.bad++, report("compare", x, y, 0, 0);
    const double sx = x * x, sy = y * y;
    if (!std::isnan(sx) && !std::isnan(sy)) {
      c_max.n++;
      if (!same(qss_emu::max_nonneg(sx, sy), sx > sy ? sx : sy)) c_max.bad++, report("max", sx, sy, 0, 0);
    }
  }
  // positive normal operands: the square root takes the integer path
  g_family = 1;
  const long long fb0 = g_fallback[3];
  long long sq_pos = 0;
  for (long long i = 0; i < cases / 4; i++) {
    const double x = std::fabs(operand(1, 1.0));
    sq_pos++;
    const double g = qss_emu::sqrt(x), w = std::sqrt(x);
    c_sqrt.n++;
    if (!same(g, w)) c_sqrt.bad++, report("sqrt", x, 0, g, w);
  }
  printf("sqrt_positive %lld %lld\n", sq_pos, g_fallback[3] - fb0);
  long long bad = 0;
  for (const Count* c : {&c_sqrt, &c_div, &c_mul, &c_add, &c_sub, &c_sc, &c_cmp, &c_max, &c_sign}) {
    printf("%s %lld %lld\n", c->name, c->n, c->bad);
    bad += c->bad;
  }
  printf("fallbacks_normal %lld %lld %lld %lld %lld\n", fam1, g_fallback[0], g_fallback[1], g_fallback[2],
         g_fallback[3]);
  return bad ? 1 : 0;
}
