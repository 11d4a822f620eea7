// qss_adjoint.cu -- adjoint of the constant-curvature update with respect to a
// spatially varying contact angle (no counterpart in the reference).
//
// Model (the var-coefficient inner step of constCurvModel3d.c:127-243 with
// check_connectivity = 0 and a fixed time step):
//   vel_n(x) = setVarNorm3dTheta(mask, grad mask, a0, theta(x))   (3d.f:94-172)
//   phi^{n+1} = impose(BC(s3)),  s1 = phi^n + dt L(phi^n)          (RK1)
//     s2 = 3/4 phi^n + 1/4 (BC(s1) + dt L(BC(s1)))                 (TVD-RK2 stage, F10)
//     s3 = 1/3 phi^n + 2/3 (BC(s2) + dt L(BC(s2)))                 (TVD-RK3 stage 3)
//   L = vel_n |grad phi|_Godunov(WENO5) + b kappa - V . grad phi_upwind   (getRHS3d5th)
//   BC = signed linear extrapolation of the six faces, impose = max(mask - overlap, .)
//   loss = sum over the fill box of (H_eps(phi^T) - target)^2, eps = 1.5 dx
// The forward runs the production kernels (split WENO5 passes + combine);
// the time step is an input, so no gradient flows through the CFL estimate.
//
// Backward (reverse mode by hand, FP64), per stage: k_adj_point takes each
// fill-box voxel's adjoint weight through the Godunov normal term, the upwind
// advection and the curvature, giving the adjoints of its six one-sided
// WENO5 derivatives and the partials of the curvature with respect to its
// central differences; k_adj_axis (one per axis) takes the derivative
// adjoints back to phi line by line, one WENO5 face window at a time for the
// minus derivative of one voxel and the plus derivative of its neighbour
// together (they share the window's smoothness indicators); k_adj_curv
// gathers the curvature partials.  Every point's adjoint is summed in a fixed
// order (deterministic); voxels whose normal term is carried from an earlier
// voxel (|vel_n| < 1e-5, 3d.f:459-486) add their (rare) contributions to
// that voxel's derivative adjoints by atomics.  The boundary extrapolation
// is reversed face by face (z, then y, then x), the imposition passes the
// adjoint where the stage value was kept.  Steps are
// recomputed from checkpoints every `ckpt` steps, storing the stage states
// of one segment at a time.
//
// This translation unit is compiled with FMA contraction: the reverse
// arithmetic has no reference bit pattern to reproduce (the forward steps run
// the uncontracted production kernels), and fused multiply-adds cut the FP64
// instructions of the reverse kernel, which is bound by the FP64 pipe.
#include <cstdlib>
#include <vector>

#include "qss_emu.cuh"
#include "qss_state.h"

namespace qss {

namespace {

constexpr double kC13 = 1.0 / 3.0, kC76 = 7.0 / 6.0, kC116 = 11.0 / 6.0, kC16 = 1.0 / 6.0, kC56 = 5.0 / 6.0;
constexpr double k1312 = 13.0 / 12.0, k136 = 13.0 / 6.0;

// Godunov term of WENO5 (3d.f:2251-2276) and its partials: dtn/d(pp, pm), dtn/dvel
__device__ __forceinline__ double godunov_bwd(double vel, const double pp[3], const double pm[3], double ppb[3],
                                              double pmb[3], double& velb) {
  double a[3], c[3];
  bool use_a[3];
  double ngps = 0;
  const bool vpos = qss_emu::gt0(vel);
#pragma unroll
  for (int d = 0; d < 3; d++) {
    if (vpos) {
      a[d] = qss_emu::gt0(pm[d]) ? pm[d] : 0.0;
      c[d] = qss_emu::lt0(pp[d]) ? pp[d] : 0.0;
    } else {
      a[d] = qss_emu::lt0(pm[d]) ? pm[d] : 0.0;
      c[d] = qss_emu::gt0(pp[d]) ? pp[d] : 0.0;
    }
    const double aa = a[d] * a[d], cc = c[d] * c[d];
    use_a[d] = (long long)qss_emu::bits(aa) > (long long)qss_emu::bits(cc);
    ngps += use_a[d] ? aa : cc;
  }
  const double norm = qss_emu::sqrt(ngps);
  velb = norm;
  const double nb = qss_emu::gt0(norm) ? qss_emu::div(vel, 2.0 * norm) : 0.0;
#pragma unroll
  for (int d = 0; d < 3; d++) {
    if (use_a[d]) pmb[d] = nb * 2.0 * a[d];
    else ppb[d] = nb * 2.0 * c[d];
  }
  return vel * norm;
}

struct AdjPointArgs {
  Box b;
  const double* phi;     // stage input, ghosts valid
  const double* dp[3];   // its WENO5 plus/minus derivatives (production axis passes)
  const double* dm[3];
  const double* lam_in;  // adjoint of the stage output; weight of the RHS = coef_l * lam_in (fill box)
  double coef_l;
  const double* vel_n;
  const double* bcoef;
  const double* vx;
  const double* vy;
  const double* vz;
  const int* nsrc;
  double fac[3];         // 1 / (2 dx) per axis
  double f2[6];          // fac products: xx, yy, zz, xy, xz, yz
  double* bp[3];         // out: adjoint of the plus / minus derivative per axis (fill box)
  double* bm[3];
  double* cc;            // out: 9 arrays of npts, the curvature's partials (see k_adj_curv)
  double* adj_vel;       // += dRHS/dvel * weight
  int64_t npts;
};

// Per fill-box voxel: the adjoints of the six one-sided WENO5 derivatives
// (Godunov normal term and upwind advection) and the partials of the
// curvature term b kappa (3d.f:2337-2379) with respect to its ten central
// differences, each times the voxel's adjoint weight.  Voxels whose normal
// term is carried from an earlier voxel leave that term to k_adj_carry.
// A block of 32 x 4 threads covers 32 (i) x 4 (j) voxels; each warp an 8 x 4
// patch of them, so that warps inside the grains (b = 0) skip the curvature
// partials together.
__global__ void __launch_bounds__(128) k_adj_point(AdjPointArgs a) {
  const Box& b = a.b;
  const int lane = threadIdx.x, warp = threadIdx.y;
  const int i = b.ilo + blockIdx.x * 32 + 8 * warp + (lane & 7);
  const int j = b.jlo + blockIdx.y * 4 + (lane >> 3);
  const int k = b.klo + blockIdx.z;
  if (i > b.ihi || j > b.jhi || k > b.khi) return;
  const int64_t q = b.idx(i, j, k);
  const double w = a.coef_l * a.lam_in[q];
  const int64_t st[3] = {1, (int64_t)b.nx, (int64_t)b.nx * b.ny};
  const double* __restrict__ phi = a.phi;
  double pp[3], pm[3];
#pragma unroll
  for (int d = 0; d < 3; d++) {
    pp[d] = a.dp[d][q];
    pm[d] = a.dm[d][q];
  }
  const double vel = a.vel_n[q];
  double ppb[3] = {0, 0, 0}, pmb[3] = {0, 0, 0};
  if (fabs(vel) >= 1.e-5) {
    double velb;
    godunov_bwd(vel, pp, pm, ppb, pmb, velb);
    a.adj_vel[q] += w * velb;
  }
  const double vxyz[3] = {a.vx[q], a.vy[q], a.vz[q]};
#pragma unroll
  for (int d = 0; d < 3; d++) {
    if (qss_emu::ge0(vxyz[d])) pmb[d] += -vxyz[d];
    else ppb[d] += -vxyz[d];
    a.bp[d][q] = w * ppb[d];
    a.bm[d][q] = w * pmb[d];
  }
  double out[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  {
    const double fx = a.fac[0], fy = a.fac[1], fz = a.fac[2];
    // first differences as the forward computes them (the threshold test on
    // their squares must take the forward's branch)
    const double phx = (phi[q + st[0]] - phi[q - st[0]]) * fx;
    const double phy = (phi[q + st[1]] - phi[q - st[1]]) * fy;
    const double phz = (phi[q + st[2]] - phi[q - st[2]]) * fz;
    const double grad = __dadd_rn(__dadd_rn(__dmul_rn(phx, phx), __dmul_rn(phy, phy)), __dmul_rn(phz, phz));
    // nothing flows through b kappa where b is zero (grain interiors)
    if (w != 0.0 && a.bcoef[q] != 0.0 && qss_emu::bits(grad) >= qss_emu::bits(1.e-5)) {  // grad >= 1e-5
      const double cc = phi[q];
      const double pxx = (phi[q + 2 * st[0]] + phi[q - 2 * st[0]] - 2 * cc) * a.f2[0];
      const double pyy = (phi[q + 2 * st[1]] + phi[q - 2 * st[1]] - 2 * cc) * a.f2[1];
      const double pzz = (phi[q + 2 * st[2]] + phi[q - 2 * st[2]] - 2 * cc) * a.f2[2];
      const double pxy = (phi[q + st[0] + st[1]] + phi[q - st[0] - st[1]] - phi[q - st[0] + st[1]] -
                          phi[q + st[0] - st[1]]) * a.f2[3];
      const double pxz = (phi[q + st[0] + st[2]] + phi[q - st[0] - st[2]] - phi[q - st[0] + st[2]] -
                          phi[q + st[0] - st[2]]) * a.f2[4];
      const double pyz = (phi[q + st[1] + st[2]] + phi[q - st[1] - st[2]] - phi[q - st[1] + st[2]] -
                          phi[q + st[1] - st[2]]) * a.f2[5];
      const double sx = phx * phx, sy = phy * phy, sz = phz * phz;
      // kappa numerator (3d.f:2337-2379), regrouped
      const double curv = pxx * (sy + sz) + pyy * (sx + sz) + pzz * (sx + sy) -
                          2 * (pxy * phx * phy + pxz * phx * phz + pyz * phy * phz);
      const double ig = qss_emu::div(1.0, grad);
      const double cb = w * a.bcoef[q] * ig;  // d RHS / d numerator
      const double gb = -cb * curv * ig;      // d RHS / d grad
      out[0] = 2 * (phx * (cb * (pyy + pzz) + gb) - cb * (pxy * phy + pxz * phz)) * fx;
      out[1] = 2 * (phy * (cb * (pxx + pzz) + gb) - cb * (pxy * phx + pyz * phz)) * fy;
      out[2] = 2 * (phz * (cb * (pxx + pyy) + gb) - cb * (pxz * phx + pyz * phy)) * fz;
      out[3] = cb * (sy + sz) * a.f2[0];
      out[4] = cb * (sx + sz) * a.f2[1];
      out[5] = cb * (sx + sy) * a.f2[2];
      const double m2cb = -2 * cb;
      out[6] = m2cb * phx * phy * a.f2[3];
      out[7] = m2cb * phx * phz * a.f2[4];
      out[8] = m2cb * phy * phz * a.f2[5];
    }
  }
#pragma unroll
  for (int o = 0; o < 9; o++) a.cc[o * a.npts + q] = out[o];
}

// Voxels whose normal term is carried from an earlier voxel (|vel_n| < 1e-5,
// 3d.f:459-486): their weight times the source voxel's Godunov partials goes
// to the source's derivative adjoints (atomics; such voxels are rare).  Runs
// after k_adj_point, which writes the source's own values.
__global__ void __launch_bounds__(128) k_adj_carry(AdjPointArgs a) {
  const Box& b = a.b;
  const int i = b.ilo + blockIdx.x * blockDim.x + threadIdx.x;
  const int j = b.jlo + blockIdx.y * blockDim.y + threadIdx.y;
  const int k = b.klo + blockIdx.z * blockDim.z + threadIdx.z;
  if (i > b.ihi || j > b.jhi || k > b.khi) return;
  const int64_t q = b.idx(i, j, k);
  if (fabs(a.vel_n[q]) >= 1.e-5) return;
  const double w = a.coef_l * a.lam_in[q];
  const int src = a.nsrc[q];
  if (w == 0.0 || src < 0) return;
  double sp[3], sm[3];
#pragma unroll
  for (int d = 0; d < 3; d++) {
    sp[d] = a.dp[d][src];
    sm[d] = a.dm[d][src];
  }
  double spb[3] = {0, 0, 0}, smb[3] = {0, 0, 0}, velb;
  godunov_bwd(a.vel_n[src], sp, sm, spb, smb, velb);
  atomicAdd(a.adj_vel + src, w * velb);
#pragma unroll
  for (int d = 0; d < 3; d++) {
    if (spb[d] != 0.0) atomicAdd(a.bp[d] + src, w * spb[d]);
    if (smb[d] != 0.0) atomicAdd(a.bm[d] + src, w * smb[d]);
  }
}

// Reverse of the WENO5 one-sided derivatives along one axis (3d.f:1962-2246),
// one face window at a time.  With v(m) = (phi(m) - phi(m-1)) inv the scaled
// difference of face m, the minus derivative of voxel c and the plus
// derivative of voxel c-1 are the same WENO5 reconstruction of the window
// u0..u4 = v(c-2..c+2), read in opposite directions: they share the three
// smoothness indicators (S1+ = S3-, S2+ = S2-, S3+ = S1-) and eps, and
// differ in the ideal weights (0.1, 0.6, 0.3 against 0.3, 0.6, 0.1 on
// S1, S2, S3) and the candidate stencils.  Per window the adjoints of both
// (the minus adjoint of voxel c, the plus adjoint of voxel c-1) are pushed
// to the five faces at once:
//   d value / d T_k = -2 w_k (p_k - value) / T_k,   T_k = S_k + eps,
//   d value / d p_k = w_k,  d eps / d u_j = 2e-6 u_j at the maximum square
// (the later operand of the reference's MAX chain on ties, per side).
// Each thread owns one of nseg equal segments of a line's points and
// recomputes the windows on either side of it whose faces it needs, so every
// point's adjoint is written once, in a fixed order: lam(p) += inv (F(p) -
// F(p+1)), F the face adjoints.
struct AdjAxisArgs {
  Box b;
  const double* phi;
  const double* bp;
  const double* bm;
  double* lam;
  double inv;
  int nseg;
};

template <int AX>
__global__ void __launch_bounds__(128) k_adj_axis(AdjAxisArgs a) {
  const Box& b = a.b;
  int p, q, lo, hi;
  if (AX == 0) {
    p = b.jlo + blockIdx.x * blockDim.x + threadIdx.x;  // j
    q = b.klo + blockIdx.y;                              // k
    if (p > b.jhi) return;
    lo = b.ilo;
    hi = b.ihi;
  } else {
    p = b.ilo + blockIdx.x * blockDim.x + threadIdx.x;  // i
    q = (AX == 1 ? b.klo : b.jlo) + blockIdx.y;
    if (p > b.ihi) return;
    lo = (AX == 1) ? b.jlo : b.klo;
    hi = (AX == 1) ? b.jhi : b.khi;
  }
  const int len = hi - lo + 7;  // points lo-3 .. hi+3
  const int p0 = lo - 3 + (int)(((int64_t)blockIdx.z * len) / a.nseg);
  const int pend = lo - 3 + (int)(((int64_t)(blockIdx.z + 1) * len) / a.nseg) - 1;
  if (pend < p0) return;
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
  const int last = (AX == 0 ? b.nx : (AX == 1 ? b.ny : b.nz)) - 1;
  // loads outside the line only feed windows without adjoints
  auto ld = [&](int m) -> double {
    const int mm = m < 0 ? 0 : (m > last ? last : m);
    return __ldg(phi + base + (int64_t)mm * stride);
  };
  auto ldbar = [&](const double* arr, int m) -> double {
    return (m >= lo && m <= hi) ? __ldg(arr + base + (int64_t)m * stride) : 0.0;
  };
  using qss_emu::bits;
  // window c = p0 - 2 first: faces c-2 .. c+1 now, face c+2 in the loop
  const int c0 = p0 - 2;
  double f_m3 = ld(c0 - 3), f_m2 = ld(c0 - 2), f_m1 = ld(c0 - 1), f_0 = ld(c0), f_p1 = ld(c0 + 1);
  double u0 = (f_m2 - f_m3) * inv, u1 = (f_m1 - f_m2) * inv, u2 = (f_0 - f_m1) * inv, u3 = (f_p1 - f_0) * inv;
  double s0 = u0 * u0, s1 = u1 * u1, s2 = u2 * u2, s3 = u3 * u3;
  double plast = f_p1;
  double F0 = 0, F1 = 0, F2 = 0, F3 = 0, F4 = 0;  // adjoints of faces c-2 .. c+2
  double prevF = 0;                                // completed adjoint of face c-3
  // the second difference a(m) = v(m-1) - 2 v(m) + v(m+1) of centre m and its
  // term 13/12 a^2 enter S1 of window m+1, S2 of window m and S3 of window
  // m-1: kept for centres c-1, c (c+1 computed per window), their adjoints
  // summed over the three windows
  double am_ = (u0 - 2.0 * u1) + u2, a0_ = (u1 - 2.0 * u2) + u3;
  double Am_ = k1312 * (am_ * am_), A0_ = k1312 * (a0_ * a0_);
  double BAm = 0, BA0 = 0, BAp = 0;  // adjoints of the terms of centres c-1, c, c+1
#pragma unroll 1
  for (int c = c0; c <= pend + 3; c++) {
    const double pn = ld(c + 2);
    const double u4 = (pn - plast) * inv;
    plast = pn;
    const double s4 = u4 * u4;
    const double ap_ = (u2 - 2.0 * u3) + u4;
    const double Ap_ = k1312 * (ap_ * ap_);
    const double gm = ldbar(a.bm, c), gp = ldbar(a.bp, c - 1);
    if (gm != 0.0 || gp != 0.0) {
      // eps and the position of the largest square for each reading direction
      const long long b0 = (long long)bits(s0), b1 = (long long)bits(s1), b2 = (long long)bits(s2),
                      b3 = (long long)bits(s3), b4 = (long long)bits(s4);
      long long mx = b0;
      int im = 0;  // minus: u0 .. u4, later wins ties
      if (b1 >= mx) { mx = b1; im = 1; }
      if (b2 >= mx) { mx = b2; im = 2; }
      if (b3 >= mx) { mx = b3; im = 3; }
      if (b4 >= mx) { mx = b4; im = 4; }
      long long mp = b4;
      int ip = 4;  // plus: u4 .. u0, later wins ties
      if (b3 >= mp) { mp = b3; ip = 3; }
      if (b2 >= mp) { mp = b2; ip = 2; }
      if (b1 >= mp) { mp = b1; ip = 1; }
      if (b0 >= mp) { mp = b0; ip = 0; }
      const double eps = 1e-6 * qss_emu::from_bits((unsigned long long)mx) + 1.0e-35;
      const double b1t = (u0 - 4.0 * u1) + 3.0 * u2, e2 = u1 - u3, b3t = (3.0 * u2 - 4.0 * u3) + u4;
      const double S1 = Am_ + 0.25 * (b1t * b1t);
      const double S2 = A0_ + 0.25 * (e2 * e2);
      const double S3 = Ap_ + 0.25 * (b3t * b3t);
      const double r1 = qss_emu::div(1.0, S1 + eps), r2 = qss_emu::div(1.0, S2 + eps),
                   r3 = qss_emu::div(1.0, S3 + eps);
      // products of the weights on the integer pipes (the FP64 pipe bounds
      // this kernel, its integer pipes are ~90 % idle)
      using qss_emu::mul;
      const double q1 = mul(r1, r1), q2 = mul(r2, r2), q3 = mul(r3, r3);
      const double am2 = mul(0.6, q2);
      const double am1 = mul(0.1, q1), am3 = mul(0.3, q3);  // minus: 0.1, 0.6, 0.3
      const double ap1 = mul(0.3, q1), ap3 = mul(0.1, q3);  // plus (on S1, S2, S3): 0.3, 0.6, 0.1
      const double iam = qss_emu::div(1.0, am1 + am2 + am3), iap = qss_emu::div(1.0, ap1 + am2 + ap3);
      const double wm1 = mul(am1, iam), wm2 = mul(am2, iam), wm3 = mul(am3, iam);
      const double wp1 = mul(ap1, iap), wp2 = mul(am2, iap), wp3 = mul(ap3, iap);
      // candidate stencils: minus reads u0..u4, plus reads u4..u0
      const double pm1 = kC13 * u0 - kC76 * u1 + kC116 * u2;
      const double pm2 = -kC16 * u1 + kC56 * u2 + kC13 * u3;
      const double pm3 = kC13 * u2 + kC56 * u3 - kC16 * u4;
      const double pq1 = -kC16 * u0 + kC56 * u1 + kC13 * u2;  // plus stencil on S1 (its third)
      const double pq2 = kC13 * u1 + kC56 * u2 - kC16 * u3;   // on S2
      const double pq3 = kC116 * u2 - kC76 * u3 + kC13 * u4;  // on S3 (its first)
      const double vm = wm1 * pm1 + wm2 * pm2 + wm3 * pm3;
      const double vp = wp1 * pq1 + wp2 * pq2 + wp3 * pq3;
      const double P1 = mul(gm, wm1), P2 = mul(gm, wm2), P3 = mul(gm, wm3);
      const double Q1 = mul(gp, wp1), Q2 = mul(gp, wp2), Q3 = mul(gp, wp3);
      const double x1 = qss_emu::scale2(r1, 1), x2 = qss_emu::scale2(r2, 1), x3 = qss_emu::scale2(r3, 1);
      // x_k = 2 r_k; the minus sign of d value / d T_k is folded into the differences
      const double m1 = P1 * (vm - pm1) * x1, m2 = P2 * (vm - pm2) * x2, m3 = P3 * (vm - pm3) * x3;
      const double n1 = Q1 * (vp - pq1) * x1, n2 = Q2 * (vp - pq2) * x2, n3 = Q3 * (vp - pq3) * x3;
      const double bS1 = m1 + n1, bS2 = m2 + n2, bS3 = m3 + n3;
      const double bem = m1 + m2 + m3, bep = n1 + n2 + n3;
      BAm += bS1;
      BA0 += bS2;
      BAp += bS3;
      const double bb1 = bS1 * qss_emu::scale2(b1t, -1);
      const double be2 = bS2 * qss_emu::scale2(e2, -1);
      const double bb3 = bS3 * qss_emu::scale2(b3t, -1);
      double d0 = bb1 + kC13 * P1 - kC16 * Q1;
      double d1 = -4.0 * bb1 + be2 - kC76 * P1 - kC16 * P2 + kC56 * Q1 + kC13 * Q2;
      double d2 = 3.0 * bb1 + 3.0 * bb3 + kC116 * P1 + kC56 * P2 + kC13 * P3 + kC13 * Q1 + kC56 * Q2 +
                  kC116 * Q3;
      double d3 = -be2 - 4.0 * bb3 + kC13 * P2 + kC56 * P3 - kC16 * Q2 - kC76 * Q3;
      double d4 = bb3 - kC16 * P3 + kC13 * Q3;
      // eps = 1e-6 max(u^2) + 1e-35, per reading direction
      {
        // both directions usually pick the same face: one sum, then selects
        const double um = im == 0 ? u0 : im == 1 ? u1 : im == 2 ? u2 : im == 3 ? u3 : u4;
        const double up = ip == 0 ? u0 : ip == 1 ? u1 : ip == 2 ? u2 : ip == 3 ? u3 : u4;
        const double cm = 2e-6 * um * bem, cp = 2e-6 * up * bep;
        const double cs = (im == ip) ? cm + cp : cm;
        auto ex = [&](int j) { return j == im ? cs : (j == ip && im != ip ? cp : 0.0); };
        d0 += ex(0);
        d1 += ex(1);
        d2 += ex(2);
        d3 += ex(3);
        d4 += ex(4);
      }
      F0 += d0;
      F1 += d1;
      F2 += d2;
      F3 += d3;
      F4 += d4;
    }
    // centre c-1 is complete: its term 13/12 a^2 back to faces c-2, c-1, c
    {
      const double ba = BAm * (k136 * am_);
      F0 += ba;
      F1 -= 2.0 * ba;
      F2 += ba;
    }
    // face c-2 is complete: the point between faces c-3 and c-2 is done
    const int m = c - 2;
    if (m > p0) {
      const int pt = m - 1;
      double* l = a.lam + base + (int64_t)pt * stride;
      *l += inv * (prevF - F0);
    }
    prevF = F0;
    // slide the window by one face
    u0 = u1;
    u1 = u2;
    u2 = u3;
    u3 = u4;
    s0 = s1;
    s1 = s2;
    s2 = s3;
    s3 = s4;
    F0 = F1;
    F1 = F2;
    F2 = F3;
    F3 = F4;
    F4 = 0;
    am_ = a0_;
    a0_ = ap_;
    Am_ = A0_;
    A0_ = Ap_;
    BAm = BA0;
    BA0 = BAp;
    BAp = 0;
  }
}

// lam_out[p] += coef * lam_in[p] (fill box) + the curvature partials of the
// fill-box voxels whose central stencil holds p, in a fixed order:
//   cc[0..2] first derivatives (+ at p-e, - at p+e), cc[3..5] second
//   derivatives (+ at p -+ 2e, -2 at p), cc[6..8] mixed xy, xz, yz
//   (+ at p -+ (e1 + e2), - at p + (e1 - e2) and p - (e1 - e2))
__global__ void k_adj_curv(Box b, const double* __restrict__ cc, int64_t npts, const double* lam_in, double coef,
                           double* lam_out) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < npts; p += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(p % b.nx);
    const int64_t r = p / b.nx;
    const int j = (int)(r % b.ny), k = (int)(r / b.ny);
    auto in_fill = [&](int ii, int jj, int kk) {
      return ii >= b.ilo && ii <= b.ihi && jj >= b.jlo && jj <= b.jhi && kk >= b.klo && kk <= b.khi;
    };
    auto at = [&](int o, int di, int dj, int dk) -> double {
      const int ii = i + di, jj = j + dj, kk = k + dk;
      return in_fill(ii, jj, kk) ? cc[o * npts + b.idx(ii, jj, kk)] : 0.0;
    };
    double s = in_fill(i, j, k) ? coef * lam_in[p] : 0.0;
    s += at(0, -1, 0, 0) - at(0, 1, 0, 0);
    s += at(1, 0, -1, 0) - at(1, 0, 1, 0);
    s += at(2, 0, 0, -1) - at(2, 0, 0, 1);
    s += at(3, -2, 0, 0) + at(3, 2, 0, 0) - 2.0 * at(3, 0, 0, 0);
    s += at(4, 0, -2, 0) + at(4, 0, 2, 0) - 2.0 * at(4, 0, 0, 0);
    s += at(5, 0, 0, -2) + at(5, 0, 0, 2) - 2.0 * at(5, 0, 0, 0);
    s += at(6, -1, -1, 0) + at(6, 1, 1, 0) - at(6, 1, -1, 0) - at(6, -1, 1, 0);
    s += at(7, -1, 0, -1) + at(7, 1, 0, 1) - at(7, 1, 0, -1) - at(7, -1, 0, 1);
    s += at(8, 0, -1, -1) + at(8, 0, 1, 1) - at(8, 0, 1, -1) - at(8, 0, -1, 1);
    lam_out[p] += s;
  }
}

// adjoint of the ghost extrapolation of one face sweep: per line, the ghost
// layers' adjoints go to the two boundary points they were built from, and
// are cleared.  axis 2: all (i, j); axis 1: all i, k in the fill box;
// axis 0: j, k in the fill box (the forward's sweep domains).
__device__ __forceinline__ void extrap_bwd(double f, double g, int dist, double gb, double& fb, double& gbb) {
  const double s = copysign(1.0, f);
  const double dsd = (f - g) > 0 ? 1.0 : ((f - g) < 0 ? -1.0 : 0.0);
  fb += gb * (1.0 + s * dsd * dist);
  gbb += gb * (-s * dsd * dist);
}

__global__ void k_adj_bc(Box b, int axis, const double* __restrict__ val, double* lam) {
  int n1, n2;
  if (axis == 2) {
    n1 = b.nx;
    n2 = b.ny;
  } else if (axis == 1) {
    n1 = b.nx;
    n2 = b.fbz();
  } else {
    n1 = b.fby();
    n2 = b.fbz();
  }
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n1 * n2) return;
  const int u = t % n1, w = t / n1;
  int64_t base, st;
  int lo, hi, len;
  if (axis == 2) {
    base = b.idx(u, w, 0);
    st = (int64_t)b.nx * b.ny;
    lo = b.klo;
    hi = b.khi;
    len = b.nz;
  } else if (axis == 1) {
    base = b.idx(u, 0, b.klo + w);
    st = b.nx;
    lo = b.jlo;
    hi = b.jhi;
    len = b.ny;
  } else {
    base = b.idx(0, b.jlo + u, b.klo + w);
    st = 1;
    lo = b.ilo;
    hi = b.ihi;
    len = b.nx;
  }
  double blo = 0, blo1 = 0, bhi = 0, bhi1 = 0;
  const double flo = val[base + lo * st], flo1 = val[base + (lo + 1) * st];
  const double fhi = val[base + hi * st], fhi1 = val[base + (hi - 1) * st];
  for (int m = 0; m < lo; m++) {
    const int64_t p = base + m * st;
    extrap_bwd(flo, flo1, lo - m, lam[p], blo, blo1);
    lam[p] = 0.0;
  }
  for (int m = hi + 1; m < len; m++) {
    const int64_t p = base + m * st;
    extrap_bwd(fhi, fhi1, m - hi, lam[p], bhi, bhi1);
    lam[p] = 0.0;
  }
  lam[base + lo * st] += blo;
  lam[base + (lo + 1) * st] += blo1;
  lam[base + hi * st] += bhi;
  lam[base + (hi - 1) * st] += bhi1;
}

// adjoint of phi = max(mask - overlap, s): passes where s was kept
__global__ void k_adj_impose(int64_t n, const double* __restrict__ s, const double* __restrict__ mask,
                             double overlap, const double* lam_in, double* lam_out) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    const double t = mask[p] - overlap;
    lam_out[p] = (t > s[p]) ? 0.0 : lam_in[p];
  }
}

// loss contributions (H(phi) - target)^2 in loop order, and the adjoint of phi^T
__global__ void k_adj_loss(Box b, const double* __restrict__ phi, const double* __restrict__ target, double eps,
                           double* contrib, double* lam) {
  const int64_t n = (int64_t)b.fbx() * b.fby() * b.fbz();
  const double pi = 3.14159265358979323846;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
    const int i = b.ilo + (int)(q % b.fbx());
    const int64_t r = q / b.fbx();
    const int j = b.jlo + (int)(r % b.fby());
    const int k = b.klo + (int)(r / b.fby());
    const int64_t p = b.idx(i, j, k);
    const double x = phi[p];
    const double H = qss_heaviside(x, eps);
    const double dH = (x > -eps && x < eps) ? (1.0 + portable_cos(pi * x / eps)) / (2 * eps) : 0.0;
    const double d = H - target[p];
    contrib[q] = d * d;
    lam[p] = 2.0 * d * dH;
  }
}

// lam_out += coef * lam_in on the fill box
__global__ void k_axpy_fill(Box b, const double* __restrict__ lam_in, double coef, double* lam_out) {
  const int64_t n = b.npts();
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(p % b.nx);
    const int64_t r = p / b.nx;
    const int j = (int)(r % b.ny), k = (int)(r / b.ny);
    if (i >= b.ilo && i <= b.ihi && j >= b.jlo && j <= b.jhi && k >= b.klo && k <= b.khi)
      lam_out[p] += coef * lam_in[p];
  }
}

// d vel_n / d theta = s h2 sin(theta) |grad mask| (from setVarNorm3dTheta)
__global__ void k_adj_theta(Box b, const double* __restrict__ mask, const double* __restrict__ mx,
                            const double* __restrict__ my, const double* __restrict__ mz,
                            const double* __restrict__ theta, const double* __restrict__ adj_vel, double dx,
                            double* grad) {
  const int i = b.ilo + blockIdx.x * blockDim.x + threadIdx.x;
  const int j = b.jlo + blockIdx.y * blockDim.y + threadIdx.y;
  const int k = b.klo + blockIdx.z * blockDim.z + threadIdx.z;
  if (i > b.ihi || j > b.jhi || k > b.khi) return;
  const int64_t c = b.idx(i, j, k);
  const double eps_var = 1.5 * dx;
  const double m = mask[c];
  const double h2 = qss_heaviside(m, eps_var);
  const double absgrad = sqrt(mx[c] * mx[c] + my[c] * my[c] + mz[c] * mz[c]);
  const double x = sqrt(m * m + absgrad * dx * absgrad * dx);
  const double s = m / x;
  grad[c] = adj_vel[c] * s * h2 * portable_sin(theta[c]) * absgrad;
}

// wgt = coef * lam on the fill box, 0 elsewhere
__global__ void k_scale_fill(Box b, const double* __restrict__ lam, double coef, double* wgt) {
  const int64_t n = b.npts();
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(p % b.nx);
    const int64_t r = p / b.nx;
    const int j = (int)(r % b.ny), k = (int)(r / b.ny);
    const bool fill = i >= b.ilo && i <= b.ihi && j >= b.jlo && j <= b.jhi && k >= b.klo && k <= b.khi;
    wgt[p] = fill ? coef * lam[p] : 0.0;
  }
}

unsigned g1(int64_t n) {
  int64_t b = (n + 255) / 256;
  if (b > 152 * 16) b = 152 * 16;
  return (unsigned)(b < 1 ? 1 : b);
}

struct DBufs {
  std::vector<double*> ptrs;
  double* get(int64_t n) {
    double* p = nullptr;
    QSS_CK(cudaMalloc(&p, (size_t)(n > 0 ? n : 1) * sizeof(double)));
    ptrs.push_back(p);
    return p;
  }
  ~DBufs() {
    for (double* p : ptrs) cudaFree(p);
  }
};

struct AdjCtx {
  Box b;
  cudaStream_t s;
  int64_t n;
  double dx[3];
  Coef c;
  ImposeArgs im;
  Ctl* ctl;
  double* dp[3];
  double* dm[3];
};

// WENO5 derivatives of the three stage inputs of one step (6 arrays each)
struct StageDerivs {
  double* d[3][6] = {};  // [stage][dp x, y, z, dm x, y, z]
};

// the stage states (and, when device memory allows, the stage inputs' WENO5
// derivatives) of the steps of one checkpoint segment
struct SegBufs {
  std::vector<double*> sphi, ss1, ss2, ss3;
  std::vector<StageDerivs> sder;
  // one allocation for the whole segment (4 states and, with derivs, 18
  // derivative arrays per step, each starting on a 256-byte boundary): a
  // trajectory kept whole at 128^3 / 200 steps is 4400 arrays, and a
  // cudaMalloc / cudaFree pair per array (cudaFree synchronises the device)
  // is host time the GPU waits through
  void alloc(DBufs& buf, int steps, int64_t n, bool derivs) {
    const int64_t pitch = (n + 31) / 32 * 32;
    const int64_t per_step = 4 + (derivs ? 18 : 0);
    double* slab = buf.get(pitch * per_step * steps);
    auto next = [&]() {
      double* p = slab;
      slab += pitch;
      return p;
    };
    for (int q = 0; q < steps; q++) {
      sphi.push_back(next());
      ss1.push_back(next());
      ss2.push_back(next());
      ss3.push_back(next());
    }
    if (derivs) {
      sder.resize(steps);
      for (auto& sd : sder)
        for (int st = 0; st < 3; st++)
          for (int c = 0; c < 6; c++) sd.d[st][c] = next();
    }
  }
  const StageDerivs* keep(int q) const { return sder.empty() ? nullptr : &sder[q]; }
};

// one forward step from phin: stage states s1, s2, s3 (ghosts valid) and
// phi^{n+1}; with keep, the stage inputs' WENO5 derivatives stay in *keep
void fwd_step(AdjCtx& a, const double* phin, double* s1, double* s2, double* s3, double* next,
              const StageDerivs* keep = nullptr) {
  const Box& b = a.b;
  const double* in[3] = {phin, s1, s2};
  double* out[3] = {s1, s2, s3};
  for (int st = 0; st < 3; st++) {
    double* dp[3] = {a.dp[0], a.dp[1], a.dp[2]};
    double* dm[3] = {a.dm[0], a.dm[1], a.dm[2]};
    if (keep)
      for (int d = 0; d < 3; d++) {
        dp[d] = keep->d[st][d];
        dm[d] = keep->d[st][3 + d];
      }
    launch_weno_axes(a.s, b, in[st], a.dx[0], a.dx[1], a.dx[2], dp, dm, a.ctl);
    launch_weno_combine(a.s, st + 1, st == 2, b, a.dx[0], a.dx[1], a.dx[2], in[st], phin, out[st],
                        st == 2 ? next : nullptr, dp, dm, a.c, a.im, a.ctl);
    launch_ghost(a.s, b, out[st], st == 2 ? next : nullptr, a.im, a.ctl);
  }
}

}  // namespace

}  // namespace qss

using namespace qss;

namespace {

// shared by the forward-only and the adjoint entry points
int adjoint_run(Options* o, QSS_DataArrays* p, Grid* g, const double* theta, const double* target, int nsteps,
                double dt, int ckpt, double* loss, double* grad_theta, double* phi_out) {
  CallScope scope;
  try {
    ensure_device();
    if (!o || !p || !g || !theta || !target || !loss || nsteps < 0 || !(dt > 0) || !p->phi || !p->mask)
      throw Error(QSSGPU_ERR_ARG, "qssgpu adjoint: bad arguments");
    validate_grid(g);
    if (ckpt <= 0 || ckpt > nsteps) ckpt = nsteps > 0 ? nsteps : 1;
    const Box b = box_of(g);
    const int64_t n = b.npts();
    const size_t bytes = (size_t)n * sizeof(double);
    AdjCtx a;
    a.b = b;
    a.n = n;
    for (int d = 0; d < 3; d++) a.dx[d] = g->dx[d];
    QSS_CK(cudaStreamCreateWithFlags(&a.s, cudaStreamNonBlocking));
    DBufs buf;
    double* mask = buf.get(n);
    double* mxyz[3] = {buf.get(n), buf.get(n), buf.get(n)};
    double* th = buf.get(n);
    double* tgt = buf.get(n);
    double* vel = buf.get(n);
    double* bco = buf.get(n);
    double* vv[3] = {buf.get(n), buf.get(n), buf.get(n)};
    for (int d = 0; d < 3; d++) {
      a.dp[d] = buf.get(n);
      a.dm[d] = buf.get(n);
    }
    int* nsrc = nullptr;
    QSS_CK(cudaMalloc(&nsrc, (size_t)n * sizeof(int)));
    const int64_t rows = (int64_t)b.fby() * b.fbz();
    int *rowlast = nullptr, *carry = nullptr;
    unsigned long long* cnt = nullptr;
    unsigned long long* red = nullptr;
    QSS_CK(cudaMalloc(&rowlast, (size_t)rows * sizeof(int)));
    QSS_CK(cudaMalloc(&carry, (size_t)rows * sizeof(int)));
    QSS_CK(cudaMalloc(&cnt, sizeof(unsigned long long)));
    QSS_CK(cudaMalloc(&red, 4 * sizeof(unsigned long long)));
    QSS_CK(cudaMalloc(&a.ctl, sizeof(Ctl)));
    QSS_CK(cudaMemcpyAsync(mask, p->mask, bytes, cudaMemcpyHostToDevice, a.s));
    QSS_CK(cudaMemcpyAsync(th, theta, bytes, cudaMemcpyHostToDevice, a.s));
    QSS_CK(cudaMemcpyAsync(tgt, target, bytes, cudaMemcpyHostToDevice, a.s));
    // coefficients as drain_model3d sets them (3d.f:13-298)
    launch_central_grad(a.s, b, mask, mxyz[0], mxyz[1], mxyz[2], g->dx[0], g->dx[1], g->dx[2]);
    launch_setvarcurvadv(a.s, b, mask, mxyz[0], mxyz[1], mxyz[2], bco, vv[0], vv[1], vv[2], o->b, g->dx[0], red);
    launch_setvarnorm(a.s, b, mask, mxyz[0], mxyz[1], mxyz[2], vel, o->a, th, o->theta, g->dx[0]);
    launch_nsrc(a.s, b, vel, nsrc, 1, rowlast, carry, cnt);
    Ctl init{};
    init.dt = dt;
    init.active = 1;
    init.tplot = 1e300;
    QSS_CK(cudaMemcpyAsync(a.ctl, &init, sizeof(Ctl), cudaMemcpyHostToDevice, a.s));
    a.c = Coef{};
    a.c.vel_n = vel;
    a.c.b = bco;
    a.c.vx = vv[0];
    a.c.vy = vv[1];
    a.c.vz = vv[2];
    a.c.nsrc = nsrc;
    a.im = ImposeArgs{mask, nullptr, nullptr, o->overlap, 0};

    const bool want_grad = grad_theta != nullptr;
    const int nseg = (nsteps + ckpt - 1) / ckpt;
    const int last0 = (nseg - 1) * ckpt;  // first step of the last segment
    // checkpoints phi^{k ckpt} of the segments before the last; the segment
    // buffers hold the stage states of one segment (the last one straight
    // from this forward pass, the others recomputed in the backward pass)
    std::vector<double*> cp(nseg, nullptr);
    // segment buffers; with two sets (when device memory allows) segment k-1
    // is recomputed on a second stream while the reverse sweep runs over
    // segment k
    SegBufs sets[2];
    int nsets = 0;
    if (want_grad) {
      for (int k = 0; k < nseg - 1; k++) cp[k] = buf.get(n);
      size_t free_b = 0, total_b = 0;
      QSS_CK(cudaMemGetInfo(&free_b, &total_b));
      const double per_set = (double)ckpt * (4 + 18) * bytes;
      const double rest = (double)(15 + 8) * bytes;
      const bool derivs = per_set + rest < 0.6 * (double)free_b;
      // (two sets need the kept derivatives: without them both streams
      // would share the derivative scratch)
      nsets = (derivs && nseg > 1 && 2 * per_set + rest < 0.6 * (double)free_b) ? 2 : 1;
      for (int k = 0; k < nsets; k++) sets[k].alloc(buf, ckpt, n, derivs);
    }
    double* cur = buf.get(n);
    double* nxt = buf.get(n);
    double* t1 = buf.get(n);
    double* t2 = buf.get(n);
    double* t3 = buf.get(n);
    QSS_CK(cudaMemcpyAsync(cur, p->phi, bytes, cudaMemcpyHostToDevice, a.s));
    for (int st = 0; st < nsteps; st++) {
      if (want_grad && st % ckpt == 0 && st < last0)
        QSS_CK(cudaMemcpyAsync(cp[st / ckpt], cur, bytes, cudaMemcpyDeviceToDevice, a.s));
      if (want_grad && st >= last0) {
        SegBufs& sb = sets[(nseg - 1) % nsets];
        const int q = st - last0;
        if (q == 0) QSS_CK(cudaMemcpyAsync(sb.sphi[0], cur, bytes, cudaMemcpyDeviceToDevice, a.s));
        double* next = (st + 1 < nsteps) ? sb.sphi[q + 1] : nxt;
        fwd_step(a, sb.sphi[q], sb.ss1[q], sb.ss2[q], sb.ss3[q], next, sb.keep(q));
        cur = next;
      } else {
        fwd_step(a, cur, t1, t2, t3, nxt);
        std::swap(cur, nxt);
      }
    }
    // loss
    const int64_t nfb = (int64_t)b.fbx() * b.fby() * b.fbz();
    double* lc = buf.get(volume_scratch_doubles(nfb));
    double* lam = buf.get(n);
    double* dl = buf.get(1);
    launch_fill(a.s, n, lam, 0.0);
    k_adj_loss<<<g1(nfb), 256, 0, a.s>>>(b, cur, tgt, 1.5 * g->dx[0], lc, lam);
    launch_loop_sum(a.s, lc, nfb, lc + nfb, dl);
    QSS_CK(cudaMemcpyAsync(loss, dl, sizeof(double), cudaMemcpyDeviceToHost, a.s));
    if (phi_out) QSS_CK(cudaMemcpyAsync(phi_out, cur, bytes, cudaMemcpyDeviceToHost, a.s));
    QSS_CK(cudaGetLastError());
    if (!want_grad) {
      QSS_CK(cudaStreamSynchronize(a.s));
      cudaFree(nsrc);
      cudaFree(rowlast);
      cudaFree(carry);
      cudaFree(cnt);
      cudaFree(red);
      cudaFree(a.ctl);
      cudaStreamDestroy(a.s);
      return 0;
    }
    // backward
    double* bars = buf.get(6 * n);  // adjoints of the plus / minus derivatives per axis
    double* cc = buf.get(9 * n);    // curvature partials
    launch_fill(a.s, 9 * n, cc, 0.0);  // outside the fill box they stay zero
    double* adj_vel = buf.get(n);
    double* lam3 = buf.get(n);
    double* lam2 = buf.get(n);
    double* lam1 = buf.get(n);
    double* lamphi = buf.get(n);
    double* wgt = buf.get(n);
    double* gth = buf.get(n);
    launch_fill(a.s, n, adj_vel, 0.0);
    AdjPointArgs ar;
    ar.b = b;
    ar.vel_n = vel;
    ar.bcoef = bco;
    ar.vx = vv[0];
    ar.vy = vv[1];
    ar.vz = vv[2];
    ar.nsrc = nsrc;
    for (int d = 0; d < 3; d++) ar.fac[d] = 0.5 / g->dx[d];
    ar.f2[0] = ar.fac[0] * ar.fac[0];
    ar.f2[1] = ar.fac[1] * ar.fac[1];
    ar.f2[2] = ar.fac[2] * ar.fac[2];
    ar.f2[3] = ar.fac[0] * ar.fac[1];
    ar.f2[4] = ar.fac[0] * ar.fac[2];
    ar.f2[5] = ar.fac[1] * ar.fac[2];
    for (int d = 0; d < 3; d++) {
      ar.bp[d] = bars + (int64_t)d * n;
      ar.bm[d] = bars + (int64_t)(3 + d) * n;
    }
    ar.cc = cc;
    ar.adj_vel = adj_vel;
    ar.npts = n;
    const dim3 blk(32, 4, 1);
    const dim3 grd((b.fbx() + 31) / 32, (b.fby() + 3) / 4, b.fbz());
    // line kernels: lanes along i for the y and z passes, along j for x; each
    // line cut into equal segments of at least 32 points (the windows a
    // segment recomputes at its ends cost 5 per segment), enough of them for
    // about two waves of 20 warps per SM
    auto nseg_of = [&](int ax) {
      const int len = (ax == 0 ? b.fbx() : ax == 1 ? b.fby() : b.fbz()) + 6;
      const int64_t lines = (ax == 0) ? (int64_t)b.fby() * b.fbz()
                                      : (ax == 1 ? (int64_t)b.fbx() * b.fbz() : (int64_t)b.fbx() * b.fby());
      const int64_t want = 2LL * 152 * 20 * 32;
      int64_t ns = (want + lines - 1) / lines;
      if (ns > len / 32) ns = len / 32;
      return (int)(ns < 1 ? 1 : ns);
    };
    const int ns0 = nseg_of(0), ns1 = nseg_of(1), ns2 = nseg_of(2);
    const dim3 ag0((unsigned)((b.fby() + 127) / 128), (unsigned)b.fbz(), (unsigned)ns0);
    const dim3 ag1((unsigned)((b.fbx() + 127) / 128), (unsigned)b.fbz(), (unsigned)ns1);
    const dim3 ag2((unsigned)((b.fbx() + 127) / 128), (unsigned)b.fby(), (unsigned)ns2);
    auto bc_bwd = [&](const double* val, double* l) {
      const int n2 = b.nx * b.ny, n1 = b.nx * b.fbz(), n0 = b.fby() * b.fbz();
      k_adj_bc<<<(n2 + 255) / 256, 256, 0, a.s>>>(b, 2, val, l);
      k_adj_bc<<<(n1 + 255) / 256, 256, 0, a.s>>>(b, 1, val, l);
      k_adj_bc<<<(n0 + 255) / 256, 256, 0, a.s>>>(b, 0, val, l);
    };
    // lam_out += coef_id * lam_in(fill) + J_L(in)^T (coef_l * lam_in)
    // stage_bwd's derivatives: kept from the forward pass (sd) or recomputed
    auto stage_bwd = [&](const double* in, const double* lam_in, double coef_id, double coef_l, double* lam_out,
                         const StageDerivs* sd, int st) {
      if (sd) {
        for (int d = 0; d < 3; d++) {
          ar.dp[d] = sd->d[st][d];
          ar.dm[d] = sd->d[st][3 + d];
        }
      } else {
        launch_weno_axes(a.s, b, in, a.dx[0], a.dx[1], a.dx[2], a.dp, a.dm, a.ctl);
        for (int d = 0; d < 3; d++) {
          ar.dp[d] = a.dp[d];
          ar.dm[d] = a.dm[d];
        }
      }
      ar.phi = in;
      ar.lam_in = lam_in;
      ar.coef_l = coef_l;
      k_adj_point<<<grd, blk, 0, a.s>>>(ar);
      k_adj_carry<<<grd, blk, 0, a.s>>>(ar);
      AdjAxisArgs ax{b, in, nullptr, nullptr, lam_out, 0.0, 1};
      ax.bp = ar.bp[0];
      ax.bm = ar.bm[0];
      ax.inv = 1.0 / g->dx[0];
      ax.nseg = ns0;
      k_adj_axis<0><<<ag0, 128, 0, a.s>>>(ax);
      ax.bp = ar.bp[1];
      ax.bm = ar.bm[1];
      ax.inv = 1.0 / g->dx[1];
      ax.nseg = ns1;
      k_adj_axis<1><<<ag1, 128, 0, a.s>>>(ax);
      ax.bp = ar.bp[2];
      ax.bm = ar.bm[2];
      ax.inv = 1.0 / g->dx[2];
      ax.nseg = ns2;
      k_adj_axis<2><<<ag2, 128, 0, a.s>>>(ax);
      k_adj_curv<<<g1(n), 256, 0, a.s>>>(b, cc, n, lam_in, coef_id, lam_out);
    };
    // recomputation of segment k's states from its checkpoint, on stream st
    AdjCtx a2 = a;
    cudaStream_t s2 = a.s;
    if (nsets == 2) QSS_CK(cudaStreamCreateWithFlags(&s2, cudaStreamNonBlocking));
    a2.s = s2;
    cudaEvent_t recomputed[2] = {}, released[2] = {};
    for (int k = 0; k < 2; k++) {
      QSS_CK(cudaEventCreateWithFlags(&recomputed[k], cudaEventDisableTiming));
      QSS_CK(cudaEventCreateWithFlags(&released[k], cudaEventDisableTiming));
    }
    auto recompute = [&](int k) {
      SegBufs& sb = sets[k % nsets];
      AdjCtx& c = (nsets == 2) ? a2 : a;
      const int s0 = k * ckpt, s1 = std::min(nsteps, s0 + ckpt);
      QSS_CK(cudaMemcpyAsync(sb.sphi[0], cp[k], bytes, cudaMemcpyDeviceToDevice, c.s));
      for (int st = s0; st < s1; st++) {
        const int q = st - s0;
        double* next = (q + 1 < s1 - s0) ? sb.sphi[q + 1] : t1;
        fwd_step(c, sb.sphi[q], sb.ss1[q], sb.ss2[q], sb.ss3[q], next, sb.keep(q));
      }
      QSS_CK(cudaEventRecord(recomputed[k % 2], c.s));
    };
    if (nsets == 2 && nseg >= 2) {
      // the checkpoints and coefficients come from work queued on a.s
      QSS_CK(cudaEventRecord(released[(nseg - 1) % 2], a.s));
      QSS_CK(cudaStreamWaitEvent(s2, released[(nseg - 1) % 2], 0));
      recompute(nseg - 2);
    }
    for (int k = nseg - 1; k >= 0; k--) {
      const int s0 = k * ckpt, s1 = std::min(nsteps, s0 + ckpt);
      SegBufs& sb = sets[k % nsets];
      if (k < nseg - 1) {
        if (nsets == 2) QSS_CK(cudaStreamWaitEvent(a.s, recomputed[k % 2], 0));
        else recompute(k);
      }
      // the set of segment k-1 is the one the reverse sweep of segment k+1
      // has released: recompute it now, beside the sweep over segment k
      if (nsets == 2 && k >= 1 && k - 1 < nseg - 2) {
        QSS_CK(cudaStreamWaitEvent(s2, released[(k + 1) % 2], 0));
        recompute(k - 1);
      }
      for (int st = s1 - 1; st >= s0; st--) {
        const int q = st - s0;
        // phi^{n+1} = impose(BC(s3))
        k_adj_impose<<<g1(n), 256, 0, a.s>>>(n, sb.ss3[q], mask, o->overlap, lam, lam3);
        bc_bwd(sb.ss3[q], lam3);
        // stage 3: s3 = 1/3 phi^n + 2/3 (s2 + dt L(s2))
        launch_fill(a.s, n, lamphi, 0.0);
        launch_fill(a.s, n, lam2, 0.0);
        const StageDerivs* sd = sb.keep(q);
        stage_bwd(sb.ss2[q], lam3, 2.0 / 3.0, 2.0 / 3.0 * dt, lam2, sd, 2);
        k_axpy_fill<<<g1(n), 256, 0, a.s>>>(b, lam3, 1.0 / 3.0, lamphi);
        bc_bwd(sb.ss2[q], lam2);
        // stage 2: s2 = 3/4 phi^n + 1/4 (s1 + dt L(s1))
        launch_fill(a.s, n, lam1, 0.0);
        stage_bwd(sb.ss1[q], lam2, 0.25, 0.25 * dt, lam1, sd, 1);
        k_axpy_fill<<<g1(n), 256, 0, a.s>>>(b, lam2, 0.75, lamphi);
        bc_bwd(sb.ss1[q], lam1);
        // stage 1: s1 = phi^n + dt L(phi^n)
        stage_bwd(sb.sphi[q], lam1, 1.0, dt, lamphi, sd, 0);
        std::swap(lam, lamphi);
      }
      QSS_CK(cudaEventRecord(released[k % 2], a.s));
    }
    QSS_CK(cudaStreamSynchronize(s2));
    for (int k = 0; k < 2; k++) {
      cudaEventDestroy(recomputed[k]);
      cudaEventDestroy(released[k]);
    }
    if (nsets == 2) cudaStreamDestroy(s2);
    k_adj_theta<<<grd, blk, 0, a.s>>>(b, mask, mxyz[0], mxyz[1], mxyz[2], th, adj_vel, g->dx[0], gth);
    QSS_CK(cudaGetLastError());
    // gradient on the fill box, zero on the ghost layers
    k_scale_fill<<<g1(n), 256, 0, a.s>>>(b, gth, 1.0, wgt);
    QSS_CK(cudaMemcpyAsync(grad_theta, wgt, bytes, cudaMemcpyDeviceToHost, a.s));
    QSS_CK(cudaStreamSynchronize(a.s));
    unsigned long long host_err = 0;
    Ctl hc;
    QSS_CK(cudaMemcpy(&hc, a.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost));
    host_err = hc.err;
    cudaFree(nsrc);
    cudaFree(rowlast);
    cudaFree(carry);
    cudaFree(cnt);
    cudaFree(red);
    cudaFree(a.ctl);
    cudaStreamDestroy(a.s);
    if (host_err) throw Error(QSSGPU_ERR_DEVICE_CHECK, "device check failed in the adjoint run");
    return 0;
  } catch (const std::exception& e) {
    return report_exception(e);
  }
}

}  // namespace

extern "C" {

// See include/lsmpqs_gpu.h.
int qssgpu_adjoint_theta(Options* o, QSS_DataArrays* p, Grid* g, const double* theta, const double* target,
                         int nsteps, double dt, int ckpt, double* loss, double* grad_theta) {
  if (!grad_theta) {
    set_error(QSSGPU_ERR_ARG, "qssgpu_adjoint_theta: grad_theta is NULL");
    return QSSGPU_ERR_ARG;
  }
  return adjoint_run(o, p, g, theta, target, nsteps, dt, ckpt, loss, grad_theta, nullptr);
}

// See include/lsmpqs_gpu.h.
int qssgpu_forward_theta(Options* o, QSS_DataArrays* p, Grid* g, const double* theta, const double* target,
                         int nsteps, double dt, double* loss, double* phi_out) {
  return adjoint_run(o, p, g, theta, target, nsteps, dt, 0, loss, nullptr, phi_out);
}

}  // extern "C"
