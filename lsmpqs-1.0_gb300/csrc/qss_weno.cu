// qss_weno.cu -- WENO5 stage of the variable-coefficient model with shared
// sub-expressions.
//
// The reference evaluates, for every voxel and axis, two WENO5 reconstructions
// from ten scaled first differences (3d.f:1962-2246).  Most of that work
// depends only on one cell face or one cell centre and is therefore repeated
// by up to six neighbouring voxels: the scaled difference v of a face, its
// square, its multiples by 3 and by the five stencil coefficients, and the
// smoothness terms of a centre.  Each of those values is an IEEE operation
// on identical operands wherever it appears, so computing it once per line
// and reusing it reproduces the reference's values bit for bit while cutting
// the FP64 instructions per voxel -- the resource that bounds this kernel on
// GB300 (one FP64 warp instruction per ~64 cycles per scheduler).
//
// A stage runs as three axis passes and one combine kernel:
//   k_weno_tile<AX> (the default): a block computes every face and centre of
//     a tile of lines once into shared memory, then one thread per voxel the
//     two reconstructions, and writes the plus and minus one-sided
//     derivatives of that axis (2 doubles per voxel);
//   k_weno_axis<AX> (selectable): each thread walks a segment of voxels along
//     axis AX with a sliding window of faces / centres, same outputs;
//   k_weno_combine: Godunov normal term (with the carried term of voxels whose
//     speed is below 1e-5), upwind advection, central curvature, TVD-RK
//     combination and, on the last stage, the three mask impositions.
// The extra traffic (48 B written + 48 B read per voxel and stage) costs about
// 2 % of the stage time at 512^3; HBM is idle otherwise.
//
// Identities used (v(m) = (phi(m) - phi(m-1)) * inv for face m, c a centre):
//   plus(i):  v1..v5 = v(i+3), v(i+2), v(i+1), v(i), v(i-1)
//   minus(i): v1..v5 = v(i-2), v(i-1), v(i),   v(i+1), v(i+2)
//   A(c) = 13/12((v(c+1) - 2v(c)) + v(c-1))^2   first term of S1+(c-2), S2+(c-1), S3+(c)
//   B(c) = 13/12((v(c-1) - 2v(c)) + v(c+1))^2   first term of S1-(c+1), S2-(c), S3-(c-1)
//   E(c) = 1/4 (v(c+1) - v(c-1))^2              second term of S2+(c-1) and S2-(c)
//   eps-(i) = eps+(i-1)                          (same five squares, max is exact)
#include <array>
#include <cstdlib>
#include <cstdio>
#include <map>
#include <mutex>
#include <vector>

#include "qss_emu.cuh"
#include "qss_kernels.cuh"

namespace qss {

namespace {

constexpr double k1312 = 13.0 / 12.0;
constexpr double kC13 = 1.0 / 3.0, kC76 = 7.0 / 6.0, kC116 = 11.0 / 6.0, kC16 = 1.0 / 6.0, kC56 = 5.0 / 6.0;
constexpr int SEG = 16;  // voxels per thread along the pass axis

// Arithmetic of one emulation level (all levels give identical results):
//   0: native FP64 instructions only;
//   1: divisions, square roots, power-of-two scalings and comparisons on the
//      integer pipes;
//   2: level 1 plus a share of the products: in the axis passes the five
//      scaled copies of each face and the normalised weights, in the combine
//      kernel the second derivatives and the curvature numerator.  The
//      combine kernel runs ~10 warps per scheduler and overlaps these with
//      its FP64 work; the axis passes hold ~120 registers per thread (4 warps
//      per scheduler) and gain only a few percent from them.
template <int EMU>
struct Ar {
  static __device__ __forceinline__ double div(double a, double b) {
    if (EMU >= 1) return qss_emu::div(a, b);
    return a / b;
  }
  // x * 2^k
  static __device__ __forceinline__ double s2(double x, int k) {
    if (EMU >= 1) return qss_emu::scale2(x, k);
    return x * (k == 1 ? 2.0 : k == 2 ? 4.0 : k == -2 ? 0.25 : k == -1 ? 0.5 : 1.0);
  }
  // products moved at level 2
  static __device__ __forceinline__ double mul2(double a, double b) {
    if (EMU >= 2) return qss_emu::mul(a, b);
    return a * b;
  }
};

// out-of-line copies of integer-pipe routines: one copy of the code instead of
// one per call site keeps the kernels' instruction footprint small
__device__ __noinline__ double div_outline(double a, double b) { return qss_emu::div(a, b); }
__device__ __noinline__ double mul_outline(double a, double b) { return qss_emu::mul(a, b); }

struct Face {
  double v, w, t3, c13, c76, c116, c16, c56;
};

__device__ __forceinline__ Face make_face(double hi, double lo, double inv) {
  Face f;
  const double d = hi - lo;
  f.v = d * inv;
  f.w = f.v * f.v;
  f.t3 = 3.0 * f.v;
  f.c13 = kC13 * f.v;
  f.c76 = kC76 * f.v;
  f.c116 = kC116 * f.v;
  f.c16 = kC16 * f.v;
  f.c56 = kC56 * f.v;
  return f;
}

// the same face with its five scaled copies on the integer pipes at EMU >= 2
template <int EMU>
__device__ __forceinline__ Face make_face_e(double hi, double lo, double inv) {
  if (EMU < 2) return make_face(hi, lo, inv);
  using qss_emu::mul;
  Face f;
  const double d = hi - lo;
  f.v = d * inv;
  f.w = f.v * f.v;
  f.t3 = 3.0 * f.v;
  f.c13 = mul(kC13, f.v);
  f.c76 = mul(kC76, f.v);
  f.c116 = mul(kC116, f.v);
  f.c16 = mul(kC16, f.v);
  f.c56 = mul(kC56, f.v);
  return f;
}

// the face with its square and 3v on the integer pipes as well (tile form)
__device__ __forceinline__ Face make_face_i(double hi, double lo, double inv) {
  using qss_emu::mul;
  Face f;
  const double d = hi - lo;
  f.v = d * inv;
  f.w = mul(f.v, f.v);
  f.t3 = mul(3.0, f.v);
  f.c13 = mul(kC13, f.v);
  f.c76 = mul(kC76, f.v);
  f.c116 = mul(kC116, f.v);
  f.c16 = mul(kC16, f.v);
  f.c56 = mul(kC56, f.v);
  return f;
}

struct Centre {
  double s1p, s2p, s3p, s1m, s2m, s3m;
};

// smoothness terms of centre c from its faces a = c-1, b = c, d = c+1: the
// three indicators of the plus side (S1+(c-2), S2+(c-1), S3+(c)) and of the
// minus side (S1-(c+1), S2-(c), S3-(c-1)), each as first term + second term
// in the reference's order of operations
template <int EMU, bool SQ>
__device__ __forceinline__ Centre make_centre(const Face& a, const Face& b, const Face& d) {
  using Q = Ar<EMU>;
  // squares (and the 13/12 products) on the integer pipes when SQ
  auto sq = [](double t) { return SQ ? Q::mul2(t, t) : t * t; };
  auto k13 = [](double x) { return SQ ? Q::mul2(k1312, x) : k1312 * x; };
  const double t2 = Q::s2(b.v, 1), t4 = Q::s2(b.v, 2);
  double t;
  t = (d.v - t2) + a.v;
  const double A = k13(sq(t));
  t = (a.v - t2) + d.v;
  const double B = k13(sq(t));
  t = (d.v - t4) + a.t3;
  const double Cp = Q::s2(sq(t), -2);
  t = (d.t3 - t4) + a.v;
  const double Dp = Q::s2(sq(t), -2);
  t = (a.v - t4) + d.t3;
  const double Cm = Q::s2(sq(t), -2);
  t = (a.t3 - t4) + d.v;
  const double Dm = Q::s2(sq(t), -2);
  t = d.v - a.v;
  const double E = Q::s2(sq(t), -2);
  Centre c;
  c.s1p = A + Cp;
  c.s2p = A + E;
  c.s3p = A + Dp;
  c.s1m = B + Cm;
  c.s2m = B + E;
  c.s3m = B + Dm;
  return c;
}

__device__ __forceinline__ double eps_of(double w1, double w2, double w3, double w4, double w5) {
  using qss_emu::max_nonneg;
  const double m = max_nonneg(max_nonneg(max_nonneg(max_nonneg(w1, w2), w3), w4), w5);
  return 1e-6 * m + 1.0e-35;
}

// weights and combination of one side (3d.f:1996-2005) given the candidate
// stencils and smoothness indicators

template <int EMU, bool SQ, bool MULC = false, bool OUTLINE = false, bool OUTMUL = false>
__device__ __forceinline__ double weno_weights(double p1, double p2, double p3, double S1, double S2, double S3,
                                               double eps) {
  using Q = Ar<EMU>;
  auto m2 = [](double x, double y) { return (OUTMUL && EMU >= 2) ? mul_outline(x, y) : Q::mul2(x, y); };
  auto sq = [&](double t) { return SQ ? m2(t, t) : t * t; };
  auto dv = [](double x, double y) { return (OUTLINE && EMU >= 1) ? div_outline(x, y) : Q::div(x, y); };
  double t, a1, a2, a3;
  t = S1 + eps;
  a1 = dv(0.1, sq(t));
  t = S2 + eps;
  a2 = dv(0.6, sq(t));
  t = S3 + eps;
  a3 = dv(0.3, sq(t));
  const double inv_sum_a = dv(1.0, a1 + a2 + a3);
  a1 = m2(a1, inv_sum_a);
  a2 = m2(a2, inv_sum_a);
  a3 = m2(a3, inv_sum_a);
  // the combination's products on the integer pipes too when MULC
  if (MULC) return m2(a1, p1) + m2(a2, p2) + m2(a3, p3);
  return a1 * p1 + a2 * p2 + a3 * p3;
}

struct AxisArgs {
  Box b;
  const double* phi;
  double* dplus;
  double* dminus;
  double inv;
  const Ctl* ctl;
  int seg_len;  // voxels per thread at EMU >= 1 (SEG at EMU 0)
};

// One thread: SEG consecutive voxels along axis AX starting at s0, inside
// the fill box of that axis.  Faces s0-2 .. s0+SEG+2, centres s0-1 .. s0+SEG.
template <int AX, int EMU, bool RING>
__global__ void __launch_bounds__(128, RING ? 5 : 4) k_weno_axis(AxisArgs a) {
  if (a.ctl && !a.ctl->active) return;
  const Box& b = a.b;
  // lanes run along i for the y and z passes (coalesced); for the x pass they
  // run along j and each thread streams its own row through L1
  int p, q, seg;
  int lo, hi;
  if (AX == 0) {
    p = b.jlo + blockIdx.x * blockDim.x + threadIdx.x;  // j
    q = b.klo + blockIdx.y;                              // k
    seg = blockIdx.z;
    if (p > b.jhi) return;
    lo = b.ilo;
    hi = b.ihi;
  } else {
    p = b.ilo + blockIdx.x * blockDim.x + threadIdx.x;  // i
    q = (AX == 1 ? b.klo : b.jlo) + blockIdx.y;          // k for the y pass, j for the z pass
    seg = blockIdx.z;
    if (p > b.ihi) return;
    lo = (AX == 1) ? b.jlo : b.klo;
    hi = (AX == 1) ? b.jhi : b.khi;
  }
  const int len = EMU == 0 ? SEG : a.seg_len;
  const int s0 = lo + seg * len;
  if (s0 > hi) return;
  int64_t base, stride;
  if (AX == 0) {
    base = b.idx(0, p, q);
    stride = 1;
  } else if (AX == 1) {
    base = b.idx(p, 0, q);
    stride = b.nx;
  } else {
    base = b.idx(p, q, 0);
    stride = (int64_t)b.nx * b.ny;
  }
  const double* __restrict__ phi = a.phi;
  const double inv = a.inv;
  // phi along the line, clamped to the last ghost point for the tail segment
  const int last = (AX == 0 ? b.nx : (AX == 1 ? b.ny : b.nz)) - 1;
  auto ld = [&](int m) -> double {
    const int mm = m > last ? last : m;
    return __ldg(phi + base + (int64_t)mm * stride);
  };

  // prologue: faces s0-2 .. s0+2, centres s0-1 .. s0+1, eps+(s0-1)
  double pm3 = ld(s0 - 3), pm2 = ld(s0 - 2), pm1 = ld(s0 - 1), p0 = ld(s0), pp1 = ld(s0 + 1), pp2 = ld(s0 + 2);
  Face fm2 = make_face_e<EMU>(pm2, pm3, inv);  // face s0-2
  Face fm1 = make_face_e<EMU>(pm1, pm2, inv);  // face s0-1
  Face f0 = make_face_e<EMU>(p0, pm1, inv);    // face s0
  Face f1 = make_face_e<EMU>(pp1, p0, inv);    // face s0+1
  Face f2 = make_face_e<EMU>(pp2, pp1, inv);   // face s0+2
  Centre cm1 = make_centre<EMU, RING>(fm2, fm1, f0);  // centre s0-1
  Centre c0 = make_centre<EMU, RING>(fm1, f0, f1);    // centre s0
  Centre c1 = make_centre<EMU, RING>(f0, f1, f2);     // centre s0+1
  double eps_prev = eps_of(f2.w, f1.w, f0.w, fm1.w, fm2.w);  // eps+(s0-1): faces s0-2 .. s0+2
  double plast = pp2;

  // At EMU >= 1 the five scaled copies of each face of the window live in
  // shared memory, one column per thread (no sharing between threads, no
  // barrier): the sliding window then holds ~30 fewer registers per thread
  // and more warps stay resident.  Face r of the segment (r = m - s0 + 2)
  // uses slot r mod 6.
  // (the register form declares no shared memory: its x pass streams rows
  // through L1, which a shared-memory carve-out would shrink)
  double* ring = nullptr;
  if constexpr (RING) {
    __shared__ double ring_mem[6 * 5 * 128];
    ring = ring_mem;
  }
  const int tx = RING ? threadIdx.x : 0;
  auto R = [&](int slot, int k) -> double& { return ring[(slot * 5 + k) * 128 + tx]; };
  auto put = [&](int slot, const Face& f) {
    if (!RING) return;
    R(slot, 0) = f.c13;
    R(slot, 1) = f.c76;
    R(slot, 2) = f.c116;
    R(slot, 3) = f.c16;
    R(slot, 4) = f.c56;
  };
  int sm2 = 0, sm1 = 1, sz = 2, sp1 = 3, sp2 = 4, sp3 = 5;
  put(sm2, fm2);
  put(sm1, fm1);
  put(sz, f0);
  put(sp1, f1);
  put(sp2, f2);

  // fully unrolled, the loop with the integer-pipe arithmetic no longer fits
  // the instruction cache; the window then rotates by register moves
#pragma unroll(EMU == 0 ? SEG : 1)
  for (int t = 0; t < (EMU == 0 ? SEG : len); t++) {
    const int i = s0 + t;
    // window: faces i-2 (fm2) .. i+2 (f2); centres i-1 (cm1) .. i+1 (c1)
    const double pnext = ld(i + 3);
    const Face f3 = make_face_e<EMU>(pnext, plast, inv);  // face i+3
    put(sp3, f3);
    const Centre c2 = make_centre<EMU, RING>(f1, f2, f3);     // centre i+2
    const double eps_i = eps_of(f3.w, f2.w, f1.w, f0.w, fm1.w);  // eps+(i): faces i-1 .. i+3
    if (i <= hi) {
      // the scaled copies of faces i-2 .. i+2
      double c13m2, c76m1, c16m1, c13z, c116z, c56z, c13p1, c116p1, c56p1, c76p2, c16p2;
      if (RING) {
        c13m2 = R(sm2, 0);
        c76m1 = R(sm1, 1);
        c16m1 = R(sm1, 3);
        c13z = R(sz, 0);
        c116z = R(sz, 2);
        c56z = R(sz, 4);
        c13p1 = R(sp1, 0);
        c116p1 = R(sp1, 2);
        c56p1 = R(sp1, 4);
        c76p2 = R(sp2, 1);
        c16p2 = R(sp2, 3);
      } else {
        c13m2 = fm2.c13;
        c76m1 = fm1.c76;
        c16m1 = fm1.c16;
        c13z = f0.c13;
        c116z = f0.c116;
        c56z = f0.c56;
        c13p1 = f1.c13;
        c116p1 = f1.c116;
        c56p1 = f1.c56;
        c76p2 = f2.c76;
        c16p2 = f2.c16;
      }
      // plus: v1..v5 = faces i+3, i+2, i+1, i, i-1
      const double pp1_ = (f3.c13 - c76p2) + c116p1;
      const double pp2_ = (-c16p2 + c56p1) + c13z;
      const double pp3_ = (c13p1 + c56z) - c16m1;
      const double plus = weno_weights<EMU, RING>(pp1_, pp2_, pp3_, c2.s1p, c1.s2p, c0.s3p, eps_i);
      // minus: v1..v5 = faces i-2, i-1, i, i+1, i+2
      const double pm1_ = (c13m2 - c76m1) + c116z;
      const double pm2_ = (-c16m1 + c56z) + c13p1;
      const double pm3_ = (c13z + c56p1) - c16p2;
      const double minus = weno_weights<EMU, RING>(pm1_, pm2_, pm3_, cm1.s1m, c0.s2m, c1.s3m, eps_prev);
      const int64_t o = base + (int64_t)i * stride;
      a.dplus[o] = plus;
      a.dminus[o] = minus;
    }
    // slide the window by one voxel
    fm2 = fm1;
    fm1 = f0;
    f0 = f1;
    f1 = f2;
    f2 = f3;
    cm1 = c0;
    c0 = c1;
    c1 = c2;
    eps_prev = eps_i;
    plast = pnext;
    const int sfree = sm2;
    sm2 = sm1;
    sm1 = sz;
    sz = sp1;
    sp1 = sp2;
    sp2 = sp3;
    sp3 = sfree;
  }
}

// Tile form of the axis pass: one block holds a tile of TL lines x TP voxels
// along the pass axis, and every face, centre and eps value of the tile is
// computed once, by one thread, into shared memory; after a barrier each
// thread finishes one voxel (the two weight sets and the combinations).
// Unlike the sliding-window forms no thread carries a window of faces and
// centres in registers, so the kernel fits 48 registers per thread and five
// blocks (ten warps per scheduler) stay resident to hide the latency of the
// integer-pipe arithmetic and of the tile's barriers.  The cost is the tile's
// halo: 21 faces and 19 centres for 16 voxels of a line (about 7 % more FP64
// work per voxel than a long window).  Lanes run over the tile's lines (16)
// and its positions (2 per warp row), so every warp instruction of every
// phase is full.  Measured on GB300 (whole WENO5 stage, M voxel-steps/s,
// by-size default of the window forms -> tiles): 64^3 188 -> 338, 128^3
// 418 -> 476, 192^3 411 -> 501, 256^3 474 -> 509, 384^3 485 -> 514, 512^3
// 497 -> 516; the FP64 pipe runs 76 % busy at 192^3 (ncu, 4 blocks per SM)
// against 57 % for the window form.
// A tile shape: L lines (a power of two) x P voxels along the axis, handled
// by L * NS threads; thread t works on line t % L and position slot t / L,
// taking positions slot, slot + NS, ... in each phase.
template <int L_, int P_, int NS_, int MB_, int MUL_>
struct TileGeom {
  static constexpr int L = L_, P = P_, NS = NS_;
  static constexpr int MB = MB_;    // resident blocks per SM the kernel is compiled for
  static constexpr int MUL = MUL_;  // default integer-pipe / out-of-line arithmetic (tile_mul)
  static constexpr int F = P + 5;  // faces s0-2 .. s0+P+2
  static constexpr int C = P + 3;  // centres s0-1 .. s0+P+1
  static constexpr int E = P + 1;  // eps+ of voxels s0-1 .. s0+P-1
  static constexpr int NT = L * NS;
  static constexpr size_t BYTES = sizeof(double) * (8 * F + 6 * C + E) * L;
};
// 16 lines x 16 voxels, 256 threads (faces and centres of the halo take a
// second round for 5 and 3 slots)
using Tile16 = TileGeom<16, 16, 16, 5, 6>;
// 8 lines x 27 voxels, 32 slots, 256 threads: the 32 faces take one round,
// the 30 centres one (2 slots idle), the 27 voxels one (5 slots idle); lines
// of a multiple of 27 voxels lose nothing to the last tile; compiled for 6
// blocks per SM (40 registers): 565 against 553 M voxel-steps/s for the whole
// stage at 512^3 on GB300 (16 x 16 tiles lose with 6 blocks: 518 against 522
// M at 192^3)
using Tile27 = TileGeom<8, 27, 32, 6, 14>;

// the tile kernels ask for all of the unified L1 / shared memory as shared
// memory, so that five or six blocks of a tile fit on an SM (once per
// process and kernel)
template <typename K>
void tile_smem_attr(K kernel, bool& done) {
  if (done) return;
  cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
  done = true;
}

// MUL bit 0: the faces' squares and 3v on the integer pipes; bit 1: the
// weights' products with the candidate stencils as well (EMU 2 only)
template <int AX, int EMU, typename G, int MUL = 0>
__global__ void __launch_bounds__(G::NT, G::MB) k_weno_tile(AxisArgs a) {
  if (a.ctl && !a.ctl->active) return;
  constexpr int TL = G::L, TP = G::P, NS = G::NS, TF = G::F, TC = G::C, TE = G::E;
  const Box& b = a.b;
  // faces: v, w, 3v and the five scaled copies; centres: six smoothness
  // indicators; eps+ per voxel; all [field][position][line], in dynamic
  // shared memory (G::BYTES)
  extern __shared__ double tile_smem[];
  auto sf = reinterpret_cast<double(*)[TF][TL]>(tile_smem);
  auto sc = reinterpret_cast<double(*)[TC][TL]>(tile_smem + 8 * TF * TL);
  auto se = reinterpret_cast<double(*)[TL]>(tile_smem + (8 * TF + 6 * TC) * TL);
  const int line = threadIdx.x % TL;
  const int slot = threadIdx.x / TL;  // 0..NS-1: position within a round
  int p, q, lo, hi, plast_line;
  if (AX == 0) {
    p = b.jlo + blockIdx.x * TL + line;  // j
    q = b.klo + blockIdx.y;              // k
    lo = b.ilo;
    hi = b.ihi;
    plast_line = b.jhi;
  } else {
    p = b.ilo + blockIdx.x * TL + line;  // i
    q = (AX == 1 ? b.klo : b.jlo) + blockIdx.y;
    lo = (AX == 1) ? b.jlo : b.klo;
    hi = (AX == 1) ? b.jhi : b.khi;
    plast_line = b.ihi;
  }
  const bool line_ok = p <= plast_line;
  if (!line_ok) p = plast_line;  // loads stay in the box; nothing is stored
  const int s0 = lo + blockIdx.z * TP;
  int64_t base, stride;
  if (AX == 0) {
    base = b.idx(0, p, q);
    stride = 1;
  } else if (AX == 1) {
    base = b.idx(p, 0, q);
    stride = b.nx;
  } else {
    base = b.idx(p, q, 0);
    stride = (int64_t)b.nx * b.ny;
  }
  const double* __restrict__ phi = a.phi;
  const int last = (AX == 0 ? b.nx : (AX == 1 ? b.ny : b.nz)) - 1;
  auto ld = [&](int m) -> double {
    const int mm = m > last ? last : m;
    return __ldg(phi + base + (int64_t)mm * stride);
  };

  // faces m = s0-2+f (between voxels m-1 and m)
  for (int f = slot; f < TF; f += NS) {
    const int m = s0 - 2 + f;
    const Face fc = (EMU >= 2 && (MUL & 1)) ? make_face_i(ld(m), ld(m - 1), a.inv)
                                            : make_face_e<EMU>(ld(m), ld(m - 1), a.inv);
    sf[0][f][line] = fc.v;
    sf[1][f][line] = fc.w;
    sf[2][f][line] = fc.t3;
    sf[3][f][line] = fc.c13;
    sf[4][f][line] = fc.c76;
    sf[5][f][line] = fc.c116;
    sf[6][f][line] = fc.c16;
    sf[7][f][line] = fc.c56;
  }
  __syncthreads();
  // centres s0-1+c from faces c, c+1, c+2; eps+ of voxel s0-1+e from faces e .. e+4
  for (int c = slot; c < TC; c += NS) {
    Face fa{}, fb{}, fd{};
    fa.v = sf[0][c][line];
    fa.t3 = sf[2][c][line];
    fb.v = sf[0][c + 1][line];
    fd.v = sf[0][c + 2][line];
    fd.t3 = sf[2][c + 2][line];
    const Centre ct = make_centre<EMU, true>(fa, fb, fd);
    sc[0][c][line] = ct.s1p;
    sc[1][c][line] = ct.s2p;
    sc[2][c][line] = ct.s3p;
    sc[3][c][line] = ct.s1m;
    sc[4][c][line] = ct.s2m;
    sc[5][c][line] = ct.s3m;
    if (c < TE)
      se[c][line] = eps_of(sf[1][c + 4][line], sf[1][c + 3][line], sf[1][c + 2][line], sf[1][c + 1][line],
                           sf[1][c][line]);
  }
  __syncthreads();
  const int t = slot;
  const int i = s0 + t;
  if (!line_ok || t >= TP || i > hi) return;
  auto F = [&](int field, int f) -> double { return sf[field][f][line]; };
  // plus: v1..v5 = faces i+3, i+2, i+1, i, i-1 (tile faces t+5 .. t+1)
  const double pp1_ = (F(3, t + 5) - F(4, t + 4)) + F(5, t + 3);
  const double pp2_ = (-F(6, t + 4) + F(7, t + 3)) + F(3, t + 2);
  const double pp3_ = (F(3, t + 3) + F(7, t + 2)) - F(6, t + 1);
  const double plus =
      weno_weights<EMU, true, EMU >= 2 && (MUL & 2), (MUL & 4) != 0, (MUL & 8) != 0>(pp1_, pp2_, pp3_, sc[0][t + 3][line], sc[1][t + 2][line], sc[2][t + 1][line],
                              se[t + 1][line]);
  // minus: v1..v5 = faces i-2, i-1, i, i+1, i+2 (tile faces t .. t+4)
  const double pm1_ = (F(3, t) - F(4, t + 1)) + F(5, t + 2);
  const double pm2_ = (-F(6, t + 1) + F(7, t + 2)) + F(3, t + 3);
  const double pm3_ = (F(3, t + 2) + F(7, t + 3)) - F(6, t + 4);
  const double minus =
      weno_weights<EMU, true, EMU >= 2 && (MUL & 2), (MUL & 4) != 0, (MUL & 8) != 0>(pm1_, pm2_, pm3_, sc[3][t][line], sc[4][t + 1][line], sc[5][t + 2][line],
                              se[t][line]);
  const int64_t o = base + (int64_t)i * stride;
  a.dplus[o] = plus;
  a.dminus[o] = minus;
}

struct CombineArgs {
  Box b;
  Fac fac;
  const double* phi_in;
  const double* u_cur;
  double* out;
  double* phi_new;
  const double* dp[3];
  const double* dm[3];
  Coef c;
  ImposeArgs im;
  const Ctl* ctl;
};

// Godunov normal term of the WENO5 scheme, vel * |grad| (3d.f:2251-2276),
// with the sign tests and maxima on the integer pipes at EMU >= 1
template <int EMU>
__device__ __forceinline__ double godunov5(double vel, const double pp[3], const double pm[3]) {
  if (EMU == 0) return godunov_norm<WENO5>(vel, pp, pm);
  using namespace qss_emu;
  double ngps;
  if (gt0(vel)) {
    double s[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
      const double a = gt0(pm[d]) ? pm[d] : 0.0, c = lt0(pp[d]) ? pp[d] : 0.0;
      s[d] = max_nonneg(a * a, c * c);
    }
    ngps = s[0] + s[1] + s[2];
  } else {
    double s[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
      const double a = lt0(pm[d]) ? pm[d] : 0.0, c = gt0(pp[d]) ? pp[d] : 0.0;
      s[d] = max_nonneg(a * a, c * c);
    }
    ngps = s[0] + s[1] + s[2];
  }
  return vel * qss_emu::sqrt(ngps);
}

// |v| >= 1e-5 (false for NaN)
__device__ __forceinline__ bool speed_valid(double v) {
  const uint64_t a = qss_emu::bits(v) & qss_emu::kAbs;
  return a >= qss_emu::bits(1.e-5) && a <= 0x7ff0000000000000ull;
}

// central curvature term (3d.f:2337-2379), same operations as curvature()
// with the exact doublings, the threshold test and the division moved to the
// integer pipes at EMU >= 1
template <int EMU>
__device__ __forceinline__ double curvature_e(const double* __restrict__ phi, const Box& b, int64_t c, const Fac& f) {
  if (EMU == 0) return curvature(phi, b, c, f);
  using Q = Ar<EMU>;
  const int64_t sy = b.sy(), sz = b.sz();
  const double cc = __ldg(phi + c);
  const double cc2 = Q::s2(cc, 1);
  const double phi_x = (__ldg(phi + c + 1) - __ldg(phi + c - 1)) * f.x;
  const double phi_y = (__ldg(phi + c + sy) - __ldg(phi + c - sy)) * f.y;
  const double phi_z = (__ldg(phi + c + sz) - __ldg(phi + c - sz)) * f.z;
  const double phi_xx = Q::mul2((__ldg(phi + c + 2) + __ldg(phi + c - 2) - cc2) * f.x, f.x);
  const double phi_zz = Q::mul2((__ldg(phi + c + 2 * sz) + __ldg(phi + c - 2 * sz) - cc2) * f.z, f.z);
  const double phi_yy = Q::mul2((__ldg(phi + c + 2 * sy) + __ldg(phi + c - 2 * sy) - cc2) * f.y, f.y);
  const double phi_xy = Q::mul2((__ldg(phi + c + 1 + sy) + __ldg(phi + c - 1 - sy) - __ldg(phi + c - 1 + sy) -
                                 __ldg(phi + c + 1 - sy)) * f.x, f.y);
  const double phi_xz = Q::mul2((__ldg(phi + c + 1 + sz) + __ldg(phi + c - 1 - sz) - __ldg(phi + c - 1 + sz) -
                                 __ldg(phi + c + 1 - sz)) * f.x, f.z);
  const double phi_yz = Q::mul2((__ldg(phi + c + sy + sz) + __ldg(phi + c - sy - sz) - __ldg(phi + c - sy + sz) -
                                 __ldg(phi + c + sy - sz)) * f.y, f.z);
  const double grad_mag2 = Q::mul2(phi_x, phi_x) + Q::mul2(phi_y, phi_y) + Q::mul2(phi_z, phi_z);
  // grad_mag2 < 1e-5: a sum of squares is +0, positive or NaN
  if (qss_emu::bits(grad_mag2) < qss_emu::bits(1.e-5)) return 0.0;
  // at level 2 the products of the curvature numerator run on the integer
  // pipes (the FP64 pipe is the combine kernel's bound; its integer pipes idle)
  const double curv = phi_xx * phi_y * phi_y + Q::mul2(Q::mul2(phi_yy, phi_x), phi_x) -
                      Q::mul2(Q::mul2(Q::s2(phi_xy, 1), phi_x), phi_y) + Q::mul2(Q::mul2(phi_xx, phi_z), phi_z) +
                      Q::mul2(Q::mul2(phi_zz, phi_x), phi_x) - Q::mul2(Q::mul2(Q::s2(phi_xz, 1), phi_x), phi_z) +
                      Q::mul2(Q::mul2(phi_yy, phi_z), phi_z) + Q::mul2(Q::mul2(phi_zz, phi_y), phi_y) -
                      Q::mul2(Q::mul2(Q::s2(phi_yz, 1), phi_y), phi_z);
  return Q::div(curv, grad_mag2);
}

// the three mask impositions with the comparisons on the integer pipes
template <int EMU>
__device__ __forceinline__ double impose3_e(double v, int64_t idx, const ImposeArgs& im) {
  if (EMU == 0) return impose3(v, idx, im);
  double t = im.mask[idx] - im.overlap;
  v = qss_emu::gt(t, v) ? t : v;
  if (im.check_conn) {
    t = im.mask_w[idx] - 0.0;
    v = qss_emu::gt(t, v) ? t : v;
    t = im.mask_nw[idx] - 0.0;
    v = qss_emu::gt(t, v) ? t : v;
  }
  return v;
}

// One block: 32 (i) x 4 (j) voxels of one k plane; each warp covers an 8 x 4
// patch of them, so that the warps that lie wholly where the curvature
// coefficient is zero (inside the grains) skip the curvature term together.
// Compiled for 10 resident blocks per SM (48 registers; 64 without the bound):
// 557 against 553 M voxel-steps/s for the whole stage at 512^3 on GB300.
template <int STAGE, bool FINAL, int EMU>
__global__ void __launch_bounds__(128, 10) k_weno_combine(CombineArgs a) {
  if (STAGE != 0 && !a.ctl->active) return;
  using Q = Ar<EMU>;
  const Box& b = a.b;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int i = b.ilo + blockIdx.x * 32 + 8 * warp + (lane & 7);
  const int j = b.jlo + blockIdx.y * 4 + (lane >> 3);
  const int k = b.klo + blockIdx.z;
  if (i > b.ihi || j > b.jhi || k > b.khi) return;
  const int64_t idx = b.idx(i, j, k);
  double pp[3], pm[3];
#pragma unroll
  for (int d = 0; d < 3; d++) {
    pp[d] = a.dp[d][idx];
    pm[d] = a.dm[d][idx];
  }
  const double vel = a.c.vel_n[idx];
  double temp_norm;
  if (EMU >= 1 ? speed_valid(vel) : fabs(vel) >= 1.e-5) {
    temp_norm = godunov5<EMU>(vel, pp, pm);
  } else {
    const int src = a.c.nsrc[idx];
    if (src < 0) {
      temp_norm = 0.0;
    } else {
      double qp[3], qm[3];
#pragma unroll
      for (int d = 0; d < 3; d++) {
        qp[d] = a.dp[d][src];
        qm[d] = a.dm[d][src];
      }
      temp_norm = godunov5<EMU>(a.c.vel_n[src], qp, qm);
    }
  }
  const double vx = a.c.vx[idx], vy = a.c.vy[idx], vz = a.c.vz[idx];
  double ax, ay, az;
  if (EMU >= 1) {
    ax = qss_emu::ge0(vx) ? pm[0] : pp[0];
    ay = qss_emu::ge0(vy) ? pm[1] : pp[1];
    az = qss_emu::ge0(vz) ? pm[2] : pp[2];
  } else {
    ax = (vx >= 0) ? pm[0] : pp[0];
    ay = (vy >= 0) ? pm[1] : pp[1];
    az = (vz >= 0) ? pm[2] : pp[2];
  }
  const double temp_vel = -(vx * ax + vy * ay + vz * az);
  // b * kappa is +-0 where b is +0, and (temp_norm + (+-0)) equals
  // (temp_norm + 0.0) unless temp_norm is -0: there the curvature (finite:
  // its denominator is at least 1e-5) changes nothing and is skipped
  const double bco = a.c.b[idx];
  const double temp_curv = (qss_emu::bits(bco) == 0 && qss_emu::bits(temp_norm) != qss_emu::kSign)
                               ? 0.0
                               : bco * curvature_e<EMU>(a.phi_in, b, idx, a.fac);
  const double rhs = temp_norm + temp_curv + temp_vel;
  double out;
  if (STAGE == 0) {
    out = rhs;
  } else {
    const double dt = a.ctl->dt;
    const double* __restrict__ phi = a.phi_in;
    if (STAGE == 1) {
      out = phi[idx] + dt * rhs;
    } else if (STAGE == 2) {
      out = 0.75 * a.u_cur[idx] + Q::s2(phi[idx] + dt * rhs, -2);
    } else {
      const double one_third = 1.0 / 3.0, two_thirds = 2.0 / 3.0;
      out = one_third * a.u_cur[idx] + two_thirds * (phi[idx] + dt * rhs);
    }
  }
  a.out[idx] = out;
  if (FINAL) a.phi_new[idx] = impose3_e<EMU>(out, idx, a.im);
}

constexpr int64_t kRingVoxels = 12LL << 20;

// a segment recomputes 5 faces and 3 centres before its first voxel:
// segments as long as the line allows while the launch still fills about
// `waves` waves of 12 warps on every SM, and at most `most` segments a line
int seg_len_for(int64_t lines, int along, int64_t waves, int64_t most) {
  const int64_t want = waves * 152 * 12 * 32;
  int64_t nseg = (want + lines - 1) / lines;
  if (nseg > most) nseg = most;
  if (nseg < 1) nseg = 1;
  return (int)((along + nseg - 1) / nseg);
}

// The default segment length of each form follows the tuned mode's picks on
// cubes (GB300).  Register form: ~8 waves, segments of about SEG voxels or
// more (192^3: the tuned pick is this rule's).  Shared-memory form: ~16
// waves with segments of at least 64 voxels; tuned picks 64 / 55 / 128
// voxels at 256^3 / 384^3 / 512^3 (this rule: 64 / 64 / 128), where the
// earlier rule of ~4 waves gave 64 / 192 / 512 and the stage ran at
// 473 / 456 / 487 M voxel-steps/s against 473 / 487 / 496 tuned.
int default_seg_len(int var, int64_t lines, int along) {
  return var ? seg_len_for(lines, along, 16, along / 64) : seg_len_for(lines, along, 8, (along + SEG - 1) / SEG);
}

template <int EMU, typename G, int MUL>
void launch_tile_m(cudaStream_t s, int ax, const AxisArgs& a, int lanes, int other, int along) {
  const dim3 gt((lanes + G::L - 1) / G::L, other, (along + G::P - 1) / G::P);
  static bool done[3] = {false, false, false};
  if (ax == 0) {
    tile_smem_attr(k_weno_tile<0, EMU, G, MUL>, done[0]);
    k_weno_tile<0, EMU, G, MUL><<<gt, G::NT, G::BYTES, s>>>(a);
  } else if (ax == 1) {
    tile_smem_attr(k_weno_tile<1, EMU, G, MUL>, done[1]);
    k_weno_tile<1, EMU, G, MUL><<<gt, G::NT, G::BYTES, s>>>(a);
  } else {
    tile_smem_attr(k_weno_tile<2, EMU, G, MUL>, done[2]);
    k_weno_tile<2, EMU, G, MUL><<<gt, G::NT, G::BYTES, s>>>(a);
  }
}

// $QSSGPU_TILE_MUL (0, 2, 6 or 14; default per geometry, TileGeom::MUL):
// bit 1 the weights' products with the candidate stencils on the integer
// pipes, bit 2 one out-of-line copy of the integer-pipe division, bit 3 one
// out-of-line copy of the integer-pipe product (in the weights); identical
// results.  GB300, whole WENO5 stage, M voxel-steps/s at 512^3 (8 x 27
// tiles) / 192^3 (16 x 16): 0: 553.7 / 522.1, 2: 558.5 / 524.5,
// 6: 580.8 / 546.1, 14: 592.4 / 539.4 (bit 0, the faces' squares and 3v on
// the integer pipes: no gain; an out-of-line square root and division in the
// combine kernel: none either; an out-of-line product in the centres' squares:
// 578.7 / 539.1, a loss).
int tile_mul() {
  static const int m = [] {
    const char* e = getenv("QSSGPU_TILE_MUL");
    const int v = e ? atoi(e) : -1;
    return v == 0 || v == 2 || v == 6 || v == 14 ? v : -1;
  }();
  return m;
}

template <int EMU, typename G>
void launch_tile(cudaStream_t s, int ax, const AxisArgs& a, int lanes, int other, int along) {
  switch (EMU >= 2 ? (tile_mul() >= 0 ? tile_mul() : G::MUL) : 0) {
    case 0: launch_tile_m<EMU, G, 0>(s, ax, a, lanes, other, along); break;
    case 2: launch_tile_m<EMU, G, 2>(s, ax, a, lanes, other, along); break;
    case 6: launch_tile_m<EMU, G, 6>(s, ax, a, lanes, other, along); break;
    default: launch_tile_m<EMU, G, 14>(s, ax, a, lanes, other, along); break;
  }
}

template <int EMU>
void launch_axis(cudaStream_t s, int ax, int var, AxisArgs a, int lanes, int other, int along, int len) {
  a.seg_len = len;
  if (var >= 3 && EMU != 0) {
    if (var == 4) launch_tile<EMU, Tile27>(s, ax, a, lanes, other, along);
    else launch_tile<EMU, Tile16>(s, ax, a, lanes, other, along);
    return;
  }
  dim3 g((lanes + 127) / 128, other, (along + len - 1) / len);
  if (EMU == 0 || var == 0) {
    if (ax == 0) k_weno_axis<0, EMU, false><<<g, 128, 0, s>>>(a);
    else if (ax == 1) k_weno_axis<1, EMU, false><<<g, 128, 0, s>>>(a);
    else k_weno_axis<2, EMU, false><<<g, 128, 0, s>>>(a);
  } else {
    if (ax == 0) k_weno_axis<0, EMU, EMU != 0><<<g, 128, 0, s>>>(a);
    else if (ax == 1) k_weno_axis<1, EMU, EMU != 0><<<g, 128, 0, s>>>(a);
    else k_weno_axis<2, EMU, EMU != 0><<<g, 128, 0, s>>>(a);
  }
}

// Tuned launch shapes (axis variant 2): per line shape (level, axis, lanes,
// lines per lane row, line length) the form and segment length that ran
// fastest the first time that shape was met.
using TuneKey = std::array<int, 5>;
std::mutex g_tune_mu;
std::map<TuneKey, std::array<int, 2>> g_tune;

// Times every distinct (form, segment length) candidate of one axis pass on
// stream s, one launch each after one untimed launch, and returns the
// fastest in var / len.  Every candidate writes the same derivatives bit for
// bit, so the timing launches are the pass itself and leave the same
// result.  Returns false (nothing to cache) when timing failed or the step
// was inactive (its kernels returned at once, so the times mean nothing).
template <int EMU>
bool tune_axis(cudaStream_t s, int ax, const AxisArgs& a, int lanes, int other, int along, int& var, int& len) {
  const int64_t lines = (int64_t)lanes * other;
  std::vector<std::array<int, 2>> cand;
  auto add = [&](int v, int l) {
    const std::array<int, 2> c{v, l};
    bool seen = false;
    for (const auto& d : cand) seen = seen || d == c;
    if (!seen) cand.push_back(c);
  };
  add(3, Tile16::P);  // the tile forms (their segment is the tile)
  add(4, Tile27::P);
  for (int v = 0; v < 2; v++) {
    add(v, default_seg_len(v, lines, along));
    for (int64_t waves : {2, 4, 8, 16, 32}) add(v, seg_len_for(lines, along, waves, (along + SEG - 1) / SEG));
  }
  const size_t n = cand.size();
  std::vector<cudaEvent_t> ev(n + 1, nullptr);
  bool ok = true;
  for (auto& e : ev) ok = ok && cudaEventCreate(&e) == cudaSuccess;
  int active = 1;
  if (ok) {
    launch_axis<EMU>(s, ax, cand[0][0], a, lanes, other, along, cand[0][1]);
    cudaEventRecord(ev[0], s);
    for (size_t c = 0; c < n; c++) {
      launch_axis<EMU>(s, ax, cand[c][0], a, lanes, other, along, cand[c][1]);
      cudaEventRecord(ev[c + 1], s);
    }
    if (a.ctl) ok = cudaMemcpyAsync(&active, &a.ctl->active, sizeof(int), cudaMemcpyDeviceToHost, s) == cudaSuccess;
    ok = cudaStreamSynchronize(s) == cudaSuccess && ok;
    float best = 0.0f;
    for (size_t c = 0; ok && c < n; c++) {
      float t = 0.0f;
      ok = cudaEventElapsedTime(&t, ev[c], ev[c + 1]) == cudaSuccess;
      if (ok && (c == 0 || t < best)) {
        best = t;
        var = cand[c][0];
        len = cand[c][1];
      }
    }
  }
  for (auto& e : ev)
    if (e) cudaEventDestroy(e);
  return ok && active;
}

// The default tile: 8 x 27 where the line splits into 27-voxel tiles with at
// most 2 % of the last tile unused, else 16 x 16 (whole WENO5 stage on GB300,
// M voxel-steps/s, 16 x 16 / 8 x 27: 512^3 516 / 532 (1.2 % unused),
// 192^3 501 / 485 (12.5 % unused)).
int tile_form_for(int along) {
  const int tiles = (along + Tile27::P - 1) / Tile27::P;
  return (int64_t)tiles * Tile27::P * 50 <= (int64_t)along * 51 ? 4 : 3;
}

template <int EMU>
void axes_at(cudaStream_t s, const Box& b, const double* phi, const double invs[3], double* const dp[3],
             double* const dm[3], const Ctl* ctl) {
  const int mode = axis_variant();
  for (int ax = 0; ax < 3; ax++) {
    const int along = ax == 0 ? b.fbx() : (ax == 1 ? b.fby() : b.fbz());
    const int lanes = ax == 0 ? b.fby() : b.fbx();
    const int other = ax == 2 ? b.fby() : b.fbz();
    // by default a tile form (tile_form_for), the fastest at every size
    // measured on GB300 (64^3 .. 512^3, see k_weno_tile); of the two window forms, which are
    // kept selectable, the shared-memory one is the faster from ~12 M fill
    // voxels on (register / shared-memory form, M voxel-steps/s: 128^3
    // 420 / 383, 192^3 411 / 385, 256^3 458 / 473, 512^3 469 / 488)
    int var = mode == 0 || mode == 1 || mode == 3 || mode == 4 ? mode : tile_form_for(along);
    if (mode == 2) var = (int64_t)lanes * other * along >= kRingVoxels ? 1 : 0;
    int len = EMU == 0 ? SEG : default_seg_len(var, (int64_t)lanes * other, along);
    AxisArgs a{b, phi, dp[ax], dm[ax], invs[ax], ctl, len};
    if (mode == 2 && EMU != 0) {
      const TuneKey key{EMU, ax, lanes, other, along};
      bool found = false;
      {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        const auto it = g_tune.find(key);
        if (it != g_tune.end()) {
          var = it->second[0];
          len = it->second[1];
          found = true;
        }
      }
      int tv = var, tl = len;
      if (!found && tune_axis<EMU>(s, ax, a, lanes, other, along, tv, tl)) {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune.emplace(key, std::array<int, 2>{tv, tl});
        var = tv;
        len = tl;
      }
    }
    cudaEvent_t e0 = ctl ? prof_open(s) : nullptr;
    launch_axis<EMU>(s, ax, var, a, lanes, other, along, len);
    prof_close(s, e0, kProfAxisX + ax);
  }
}

template <int EMU>
void combine_at(cudaStream_t s, int stage, bool final_stage, dim3 g, dim3 blk, const CombineArgs& a) {
  switch (stage) {
    case 0: k_weno_combine<0, false, EMU><<<g, blk, 0, s>>>(a); break;
    case 1: if (final_stage) k_weno_combine<1, true, EMU><<<g, blk, 0, s>>>(a); else k_weno_combine<1, false, EMU><<<g, blk, 0, s>>>(a); break;
    case 2: if (final_stage) k_weno_combine<2, true, EMU><<<g, blk, 0, s>>>(a); else k_weno_combine<2, false, EMU><<<g, blk, 0, s>>>(a); break;
    default: if (final_stage) k_weno_combine<3, true, EMU><<<g, blk, 0, s>>>(a); else k_weno_combine<3, false, EMU><<<g, blk, 0, s>>>(a); break;
  }
}

}  // namespace

void launch_weno_axes(cudaStream_t s, const Box& b, const double* phi, double dx, double dy, double dz,
                      double* const dp[3], double* const dm[3], const Ctl* ctl) {
  const double invs[3] = {1.0 / dx, 1.0 / dy, 1.0 / dz};
  const int lv = emu_level();
  if (lv == 0) axes_at<0>(s, b, phi, invs, dp, dm, ctl);
  else if (lv == 1) axes_at<1>(s, b, phi, invs, dp, dm, ctl);
  else axes_at<2>(s, b, phi, invs, dp, dm, ctl);
}

void launch_weno_combine(cudaStream_t s, int stage, bool final_stage, const Box& b, double dx, double dy, double dz,
                         const double* phi_in, const double* u_cur, double* out, double* phi_new,
                         double* const dp[3], double* const dm[3], const Coef& c, const ImposeArgs& im,
                         const Ctl* ctl) {
  CombineArgs a;
  a.b = b;
  a.fac = Fac{0.5 / dx, 0.5 / dy, 0.5 / dz};
  a.phi_in = phi_in;
  a.u_cur = u_cur;
  a.out = out;
  a.phi_new = phi_new;
  for (int d = 0; d < 3; d++) {
    a.dp[d] = dp[d];
    a.dm[d] = dm[d];
  }
  a.c = c;
  a.im = im;
  a.ctl = ctl;
  const dim3 blk(128, 1, 1);
  const dim3 g((b.fbx() + 31) / 32, (b.fby() + 3) / 4, b.fbz());
  cudaEvent_t e0 = stage != 0 ? prof_open(s) : nullptr;
  switch (emu_level()) {
    case 0: combine_at<0>(s, stage, final_stage, g, blk, a); break;
    case 1: combine_at<1>(s, stage, final_stage, g, blk, a); break;
    default: combine_at<2>(s, stage, final_stage, g, blk, a); break;
  }
  prof_close(s, e0, kProfCombine);
}

}  // namespace qss

extern "C" {

int qssgpu_axis_tuning(int* rows, int max_rows) {
  std::lock_guard<std::mutex> lk(qss::g_tune_mu);
  int n = 0;
  for (const auto& kv : qss::g_tune) {
    if (rows && n < max_rows) {
      int* r = rows + 7 * n;
      for (int k = 0; k < 5; k++) r[k] = kv.first[k];
      r[5] = kv.second[0];
      r[6] = kv.second[1];
    }
    n++;
  }
  return n;
}

void qssgpu_axis_tuning_reset(void) {
  std::lock_guard<std::mutex> lk(qss::g_tune_mu);
  qss::g_tune.clear();
}

int qssgpu_axis_tuning_save(const char* path) {
  if (!path) return -1;
  FILE* fp = fopen(path, "w");
  if (!fp) return -1;
  std::lock_guard<std::mutex> lk(qss::g_tune_mu);
  int n = 0;
  fprintf(fp, "# level axis lanes lines_per_lane line form seg_len\n");
  for (const auto& kv : qss::g_tune) {
    fprintf(fp, "%d %d %d %d %d %d %d\n", kv.first[0], kv.first[1], kv.first[2], kv.first[3], kv.first[4],
            kv.second[0], kv.second[1]);
    n++;
  }
  return fclose(fp) == 0 ? n : -1;
}

int qssgpu_axis_tuning_load(const char* path) {
  if (!path) return -1;
  FILE* fp = fopen(path, "r");
  if (!fp) return -1;
  // every row is checked before any is added: a launch shape from the file
  // must be one the tuner itself could have picked
  std::vector<std::pair<qss::TuneKey, std::array<int, 2>>> rows;
  char line[256];
  bool ok = true;
  while (ok && fgets(line, sizeof line, fp)) {
    const char* c = line;
    while (*c == ' ' || *c == '\t') c++;
    if (*c == '#' || *c == '\n' || *c == 0) continue;
    int v[7];
    char tail;
    ok = sscanf(c, "%d %d %d %d %d %d %d %c", &v[0], &v[1], &v[2], &v[3], &v[4], &v[5], &v[6], &tail) == 7 &&
         v[0] >= 1 && v[0] <= 2 && v[1] >= 0 && v[1] <= 2 && v[2] > 0 && v[3] > 0 && v[4] > 0 &&
         (v[5] == 0 || v[5] == 1 || v[5] == 3 || v[5] == 4) && v[6] >= 1 &&
         (v[5] == 3 ? v[6] == qss::Tile16::P : v[5] == 4 ? v[6] == qss::Tile27::P : v[6] <= v[4]);
    if (ok) rows.push_back({qss::TuneKey{v[0], v[1], v[2], v[3], v[4]}, std::array<int, 2>{v[5], v[6]}});
  }
  fclose(fp);
  if (!ok) return -1;
  std::lock_guard<std::mutex> lk(qss::g_tune_mu);
  for (const auto& r : rows) qss::g_tune.emplace(r.first, r.second);
  return (int)rows.size();
}

}  // extern "C"
