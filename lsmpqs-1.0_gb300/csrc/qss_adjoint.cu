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
// Backward (reverse mode by hand, FP64): for each stage, one thread per
// fill-box voxel recomputes the stage's RHS at that voxel and its partials
// with respect to the 31 stencil values it reads (axis offsets +-1..3, the 12
// edge neighbours of the mixed derivatives, the centre) and to vel_n, and
// stores partial x adjoint weight per offset; a gather kernel then forms
// each point's adjoint as the sum over the voxels whose stencil contains it,
// in a fixed order (deterministic, no atomics).  Voxels whose normal term is
// carried from an earlier voxel (|vel_n| < 1e-5, 3d.f:459-486) add their
// (rare) contributions to that voxel's stencil by atomics.  The boundary
// extrapolation is reversed face by face (z, then y, then x), the
// imposition passes the adjoint where the stage value was kept.  Steps are
// recomputed from checkpoints every `ckpt` steps, storing the stage states
// of one segment at a time.
#include <vector>

#include "qss_emu.cuh"
#include "qss_state.h"

namespace qss {

namespace {

constexpr int kOff = 31;  // stencil offsets of one voxel's RHS

// offset o -> (di, dj, dk):  0 centre; 1..18 axis d = (o-1)/6, distance
// -3,-2,-1,+1,+2,+3; 19..22 xy (+1,+1)(-1,-1)(-1,+1)(+1,-1); 23..26 xz; 27..30 yz
__host__ __device__ __forceinline__ void offset_of(int o, int& di, int& dj, int& dk) {
  di = dj = dk = 0;
  if (o == 0) return;
  if (o <= 18) {
    const int d = (o - 1) / 6, r = (o - 1) % 6;
    const int k = r < 3 ? r - 3 : r - 2;
    if (d == 0) di = k;
    else if (d == 1) dj = k;
    else dk = k;
    return;
  }
  const int e = (o - 19) / 4, r = (o - 19) % 4;
  const int a = (r == 0) ? 1 : (r == 1 ? -1 : (r == 2 ? -1 : 1));
  const int c = (r == 0) ? 1 : (r == 1 ? -1 : (r == 2 ? 1 : -1));
  if (e == 0) {
    di = a;
    dj = c;
  } else if (e == 1) {
    di = a;
    dk = c;
  } else {
    dj = a;
    dk = c;
  }
}

__device__ __forceinline__ int axis_off(int d, int k) { return 1 + 6 * d + (k < 0 ? k + 3 : k + 2); }

constexpr double kC13 = 1.0 / 3.0, kC76 = 7.0 / 6.0, kC116 = 11.0 / 6.0, kC16 = 1.0 / 6.0, kC56 = 5.0 / 6.0;
constexpr double k1312 = 13.0 / 12.0;

// adjoint of one WENO5 side (3d.f:1999-2014): accumulates into vb[0..4] the
// partials of the side's value times gbar (four divisions, on the integer
// pipes)
__device__ __forceinline__ void weno_side_bwd(const double v[5], double gbar, double vb[5]) {
  // eps: the reference's chain of MAX keeps the later operand on ties; the
  // squares are non-negative, so their bit patterns order like the values
  // (integer compares, static indices only: no local memory)
  long long mb = (long long)qss_emu::bits(v[0] * v[0]);
  int im = 0;
  double vim = v[0];
#pragma unroll
  for (int i = 1; i < 5; i++) {
    const long long qb = (long long)qss_emu::bits(v[i] * v[i]);
    if (!(mb > qb)) {
      mb = qb;
      im = i;
      vim = v[i];
    }
  }
  const double eps = 1e-6 * qss_emu::from_bits((unsigned long long)mb) + 1.0e-35;
  const double p1 = kC13 * v[0] - kC76 * v[1] + kC116 * v[2];
  const double p2 = -(kC16 * v[1]) + kC56 * v[2] + kC13 * v[3];
  const double p3 = kC13 * v[2] + kC56 * v[3] - kC16 * v[4];
  const double t1a = v[0] - 2.0 * v[1] + v[2], t1b = v[0] - 4.0 * v[1] + 3.0 * v[2];
  const double t2a = v[1] - 2.0 * v[2] + v[3], t2b = v[1] - v[3];
  const double t3a = v[2] - 2.0 * v[3] + v[4], t3b = 3.0 * v[2] - 4.0 * v[3] + v[4];
  const double S1 = k1312 * (t1a * t1a) + 0.25 * (t1b * t1b);
  const double S2 = k1312 * (t2a * t2a) + 0.25 * (t2b * t2b);
  const double S3 = k1312 * (t3a * t3a) + 0.25 * (t3b * t3b);
  const double iT1 = qss_emu::div(1.0, S1 + eps), iT2 = qss_emu::div(1.0, S2 + eps),
               iT3 = qss_emu::div(1.0, S3 + eps);
  const double a1 = 0.1 * iT1 * iT1, a2 = 0.6 * iT2 * iT2, a3 = 0.3 * iT3 * iT3;
  const double iA = qss_emu::div(1.0, a1 + a2 + a3);
  const double w1 = a1 * iA, w2 = a2 * iA, w3 = a3 * iA;
  // reverse
  const double pb1 = gbar * w1, pb2 = gbar * w2, pb3 = gbar * w3;
  const double wb1 = gbar * p1, wb2 = gbar * p2, wb3 = gbar * p3;
  const double sw = wb1 * w1 + wb2 * w2 + wb3 * w3;
  const double Tb1 = -2.0 * (wb1 - sw) * iA * a1 * iT1, Tb2 = -2.0 * (wb2 - sw) * iA * a2 * iT2,
               Tb3 = -2.0 * (wb3 - sw) * iA * a3 * iT3;
  const double epsb = Tb1 + Tb2 + Tb3;
  {
    // vb[im] += d eps / d v[im] * epsb, with the index resolved by selects
    double t = vb[0];
#pragma unroll
    for (int i = 1; i < 5; i++) t = (im == i) ? vb[i] : t;
    t += epsb * 2e-6 * vim;
#pragma unroll
    for (int i = 0; i < 5; i++) vb[i] = (im == i) ? t : vb[i];
  }
  const double t1ab = Tb1 * 2.0 * k1312 * t1a, t1bb = Tb1 * 0.5 * t1b;
  vb[0] += t1ab + t1bb;
  vb[1] += -2.0 * t1ab - 4.0 * t1bb;
  vb[2] += t1ab + 3.0 * t1bb;
  const double t2ab = Tb2 * 2.0 * k1312 * t2a, t2bb = Tb2 * 0.5 * t2b;
  vb[1] += t2ab + t2bb;
  vb[2] += -2.0 * t2ab;
  vb[3] += t2ab - t2bb;
  const double t3ab = Tb3 * 2.0 * k1312 * t3a, t3bb = Tb3 * 0.5 * t3b;
  vb[2] += t3ab + 3.0 * t3bb;
  vb[3] += -2.0 * t3ab - 4.0 * t3bb;
  vb[4] += t3ab + t3bb;
  vb[0] += kC13 * pb1;
  vb[1] += -kC76 * pb1 - kC16 * pb2;
  vb[2] += kC116 * pb1 + kC56 * pb2 + kC13 * pb3;
  vb[3] += kC13 * pb2 + kC56 * pb3;
  vb[4] += -kC16 * pb3;
}

// adjoint of the WENO5 plus/minus derivatives along one axis: P[0..6] =
// phi(q-3..q+3), output adjoints (pb, mb), accumulated into Pb[0..6]
__device__ __forceinline__ void weno_axis_bwd(const double P[7], double inv, double pb, double mb, double Pb[7]) {
  double F[6];  // faces q-2 .. q+3: F[m] = (P[m+1] - P[m]) inv
#pragma unroll
  for (int m = 0; m < 6; m++) F[m] = (P[m + 1] - P[m]) * inv;
  double Fb[6] = {0, 0, 0, 0, 0, 0};
  if (pb != 0.0) {
    const double v[5] = {F[5], F[4], F[3], F[2], F[1]};  // plus: faces i+3 .. i-1
    double vb[5] = {0, 0, 0, 0, 0};
    weno_side_bwd(v, pb, vb);
    Fb[5] += vb[0];
    Fb[4] += vb[1];
    Fb[3] += vb[2];
    Fb[2] += vb[3];
    Fb[1] += vb[4];
  }
  if (mb != 0.0) {
    const double v[5] = {F[0], F[1], F[2], F[3], F[4]};  // minus: faces i-2 .. i+2
    double vb[5] = {0, 0, 0, 0, 0};
    weno_side_bwd(v, mb, vb);
#pragma unroll
    for (int m = 0; m < 5; m++) Fb[m] += vb[m];
  }
#pragma unroll
  for (int m = 0; m < 6; m++) {
    Pb[m + 1] += Fb[m] * inv;
    Pb[m] -= Fb[m] * inv;
  }
}

// Godunov term of WENO5 (3d.f:2245-2276) and its partials: dtn/d(pp, pm), dtn/dvel
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

struct AdjRhsArgs {
  Box b;
  const double* phi;     // stage input, ghosts valid
  const double* dp[3];   // its WENO5 plus/minus derivatives (production axis passes)
  const double* dm[3];
  const double* wgt;     // adjoint weight of the voxel's RHS (fill box)
  const double* vel_n;
  const double* bcoef;
  const double* vx;
  const double* vy;
  const double* vz;
  const int* nsrc;
  double inv[3];
  double fac[3];
  double* contrib;       // kOff arrays of npts: contrib[o * npts + q]
  double* adj_vel;       // += dRHS/dvel * weight
  double* lam_out;       // target of the carried-term scatter
  int64_t npts;
};

__global__ void __launch_bounds__(128) k_adj_rhs(AdjRhsArgs a) {
  const Box& b = a.b;
  const int i = b.ilo + blockIdx.x * blockDim.x + threadIdx.x;
  const int j = b.jlo + blockIdx.y * blockDim.y + threadIdx.y;
  const int k = b.klo + blockIdx.z * blockDim.z + threadIdx.z;
  if (i > b.ihi || j > b.jhi || k > b.khi) return;
  const int64_t q = b.idx(i, j, k);
  const double w = a.wgt[q];
  double g[kOff];
#pragma unroll
  for (int o = 0; o < kOff; o++) g[o] = 0.0;
  const int64_t st[3] = {1, (int64_t)b.nx, (int64_t)b.nx * b.ny};
  const double* __restrict__ phi = a.phi;
  // forward values of the axis derivatives (for the upwind choices)
  double pp[3], pm[3];
#pragma unroll
  for (int d = 0; d < 3; d++) {
    pp[d] = a.dp[d][q];
    pm[d] = a.dm[d][q];
  }
  // Godunov normal term (or the carried term of an earlier voxel)
  const double vel = a.vel_n[q];
  double ppb[3] = {0, 0, 0}, pmb[3] = {0, 0, 0};
  const bool own = fabs(vel) >= 1.e-5;
  if (own) {
    double velb;
    godunov_bwd(vel, pp, pm, ppb, pmb, velb);
    a.adj_vel[q] += w * velb;
  }
  // advection
  const double vxyz[3] = {a.vx[q], a.vy[q], a.vz[q]};
#pragma unroll
  for (int d = 0; d < 3; d++) {
    if (qss_emu::ge0(vxyz[d])) pmb[d] += -vxyz[d];
    else ppb[d] += -vxyz[d];
  }
  // chain the axis derivatives to the stencil
#pragma unroll
  for (int d = 0; d < 3; d++) {
    double P[7], Pb[7];
#pragma unroll
    for (int m = 0; m < 7; m++) {
      P[m] = phi[q + (m - 3) * st[d]];
      Pb[m] = 0.0;
    }
    weno_axis_bwd(P, a.inv[d], ppb[d], pmb[d], Pb);
#pragma unroll
    for (int m = 0; m < 7; m++) {
      if (m == 3) g[0] += Pb[m];
      else g[axis_off(d, m - 3)] += Pb[m];
    }
  }
  // curvature b kappa (3d.f:2336-2378)
  {
    const double fx = a.fac[0], fy = a.fac[1], fz = a.fac[2];
    const double cc = phi[q];
    const double phx = (phi[q + st[0]] - phi[q - st[0]]) * fx;
    const double phy = (phi[q + st[1]] - phi[q - st[1]]) * fy;
    const double phz = (phi[q + st[2]] - phi[q - st[2]]) * fz;
    const double pxx = (phi[q + 2 * st[0]] + phi[q - 2 * st[0]] - 2 * cc) * fx * fx;
    const double pyy = (phi[q + 2 * st[1]] + phi[q - 2 * st[1]] - 2 * cc) * fy * fy;
    const double pzz = (phi[q + 2 * st[2]] + phi[q - 2 * st[2]] - 2 * cc) * fz * fz;
    const double pxy = (phi[q + st[0] + st[1]] + phi[q - st[0] - st[1]] - phi[q - st[0] + st[1]] -
                        phi[q + st[0] - st[1]]) * fx * fy;
    const double pxz = (phi[q + st[0] + st[2]] + phi[q - st[0] - st[2]] - phi[q - st[0] + st[2]] -
                        phi[q + st[0] - st[2]]) * fx * fz;
    const double pyz = (phi[q + st[1] + st[2]] + phi[q - st[1] - st[2]] - phi[q - st[1] + st[2]] -
                        phi[q + st[1] - st[2]]) * fy * fz;
    const double grad = phx * phx + phy * phy + phz * phz;
    if (qss_emu::bits(grad) >= qss_emu::bits(1.e-5)) {  // grad >= 1e-5 (a sum of squares)
      const double curv = pxx * phy * phy + pyy * phx * phx - 2 * pxy * phx * phy + pxx * phz * phz +
                          pzz * phx * phx - 2 * pxz * phx * phz + pyy * phz * phz + pzz * phy * phy -
                          2 * pyz * phy * phz;
      const double kb = a.bcoef[q];
      const double ig = qss_emu::div(1.0, grad);
      const double cb = kb * ig, gb = -kb * curv * ig * ig;
      const double xb = cb * (2 * pyy * phx - 2 * pxy * phy + 2 * pzz * phx - 2 * pxz * phz) + gb * 2 * phx;
      const double yb = cb * (2 * pxx * phy - 2 * pxy * phx + 2 * pzz * phy - 2 * pyz * phz) + gb * 2 * phy;
      const double zb = cb * (2 * pxx * phz - 2 * pxz * phx + 2 * pyy * phz - 2 * pyz * phy) + gb * 2 * phz;
      const double xxb = cb * (phy * phy + phz * phz) * fx * fx;
      const double yyb = cb * (phx * phx + phz * phz) * fy * fy;
      const double zzb = cb * (phx * phx + phy * phy) * fz * fz;
      const double xyb = cb * (-2 * phx * phy) * fx * fy;
      const double xzb = cb * (-2 * phx * phz) * fx * fz;
      const double yzb = cb * (-2 * phy * phz) * fy * fz;
      g[axis_off(0, 1)] += xb * fx;
      g[axis_off(0, -1)] -= xb * fx;
      g[axis_off(1, 1)] += yb * fy;
      g[axis_off(1, -1)] -= yb * fy;
      g[axis_off(2, 1)] += zb * fz;
      g[axis_off(2, -1)] -= zb * fz;
      g[axis_off(0, 2)] += xxb;
      g[axis_off(0, -2)] += xxb;
      g[axis_off(1, 2)] += yyb;
      g[axis_off(1, -2)] += yyb;
      g[axis_off(2, 2)] += zzb;
      g[axis_off(2, -2)] += zzb;
      g[0] -= 2 * (xxb + yyb + zzb);
      g[19] += xyb;
      g[20] += xyb;
      g[21] -= xyb;
      g[22] -= xyb;
      g[23] += xzb;
      g[24] += xzb;
      g[25] -= xzb;
      g[26] -= xzb;
      g[27] += yzb;
      g[28] += yzb;
      g[29] -= yzb;
      g[30] -= yzb;
    }
  }
#pragma unroll
  for (int o = 0; o < kOff; o++) a.contrib[o * a.npts + q] = w * g[o];
  // carried normal term: its partials belong to the source voxel's stencil
  if (!own && w != 0.0) {
    const int src = a.nsrc[q];
    if (src >= 0) {
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
        double P[7], Pb[7];
#pragma unroll
        for (int m = 0; m < 7; m++) {
          P[m] = phi[src + (m - 3) * st[d]];
          Pb[m] = 0.0;
        }
        weno_axis_bwd(P, a.inv[d], spb[d], smb[d], Pb);
#pragma unroll
        for (int m = 0; m < 7; m++) atomicAdd(a.lam_out + src + (m - 3) * st[d], w * Pb[m]);
      }
    }
  }
}

// lam_out[p] = coef * lam_in[p] (fill box) + sum over offsets of contrib[o][p - off(o)]
__global__ void k_adj_gather(Box b, const double* __restrict__ contrib, int64_t npts, const double* lam_in,
                             double coef, double* lam_out) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < npts; p += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(p % b.nx);
    const int64_t r = p / b.nx;
    const int j = (int)(r % b.ny), k = (int)(r / b.ny);
    const bool fill = i >= b.ilo && i <= b.ihi && j >= b.jlo && j <= b.jhi && k >= b.klo && k <= b.khi;
    double s = fill ? coef * lam_in[p] : 0.0;
    for (int o = 0; o < kOff; o++) {
      int di, dj, dk;
      offset_of(o, di, dj, dk);
      const int qi = i - di, qj = j - dj, qk = k - dk;
      if (qi < b.ilo || qi > b.ihi || qj < b.jlo || qj > b.jhi || qk < b.klo || qk > b.khi) continue;
      s += contrib[o * npts + b.idx(qi, qj, qk)];
    }
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
    std::vector<double*> sphi, ss1, ss2, ss3;
    std::vector<StageDerivs> sder;  // per segment step, when device memory allows
    if (want_grad) {
      for (int k = 0; k < nseg - 1; k++) cp[k] = buf.get(n);
      for (int q = 0; q < ckpt; q++) {
        sphi.push_back(buf.get(n));
        ss1.push_back(buf.get(n));
        ss2.push_back(buf.get(n));
        ss3.push_back(buf.get(n));
      }
      size_t free_b = 0, total_b = 0;
      QSS_CK(cudaMemGetInfo(&free_b, &total_b));
      const double need = (double)ckpt * 18 * bytes + (double)(kOff + 8) * bytes;
      if (need < 0.6 * (double)free_b) {
        sder.resize(ckpt);
        for (auto& sd : sder)
          for (int st = 0; st < 3; st++)
            for (int c = 0; c < 6; c++) sd.d[st][c] = buf.get(n);
      }
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
        const int q = st - last0;
        if (q == 0) QSS_CK(cudaMemcpyAsync(sphi[0], cur, bytes, cudaMemcpyDeviceToDevice, a.s));
        double* next = (st + 1 < nsteps) ? sphi[q + 1] : nxt;
        fwd_step(a, sphi[q], ss1[q], ss2[q], ss3[q], next, sder.empty() ? nullptr : &sder[q]);
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
    double* contrib = buf.get((int64_t)kOff * n);
    double* adj_vel = buf.get(n);
    double* lam3 = buf.get(n);
    double* lam2 = buf.get(n);
    double* lam1 = buf.get(n);
    double* lamphi = buf.get(n);
    double* wgt = buf.get(n);
    double* gth = buf.get(n);
    launch_fill(a.s, n, adj_vel, 0.0);
    AdjRhsArgs ar;
    ar.b = b;
    ar.vel_n = vel;
    ar.bcoef = bco;
    ar.vx = vv[0];
    ar.vy = vv[1];
    ar.vz = vv[2];
    ar.nsrc = nsrc;
    for (int d = 0; d < 3; d++) {
      ar.inv[d] = 1.0 / g->dx[d];
      ar.fac[d] = 0.5 / g->dx[d];
    }
    ar.contrib = contrib;
    ar.adj_vel = adj_vel;
    ar.npts = n;
    const dim3 blk(32, 4, 1);
    const dim3 grd((b.fbx() + 31) / 32, (b.fby() + 3) / 4, b.fbz());
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
      k_scale_fill<<<g1(n), 256, 0, a.s>>>(b, lam_in, coef_l, wgt);
      ar.phi = in;
      ar.wgt = wgt;
      ar.lam_out = lam_out;
      k_adj_rhs<<<grd, blk, 0, a.s>>>(ar);
      k_adj_gather<<<g1(n), 256, 0, a.s>>>(b, contrib, n, lam_in, coef_id, lam_out);
    };
    for (int k = nseg - 1; k >= 0; k--) {
      const int s0 = k * ckpt, s1 = std::min(nsteps, s0 + ckpt);
      // recompute the segment's states (the last segment's are still there)
      if (k < nseg - 1) {
        QSS_CK(cudaMemcpyAsync(sphi[0], cp[k], bytes, cudaMemcpyDeviceToDevice, a.s));
        for (int st = s0; st < s1; st++) {
          const int q = st - s0;
          double* next = (q + 1 < s1 - s0) ? sphi[q + 1] : t1;
          fwd_step(a, sphi[q], ss1[q], ss2[q], ss3[q], next, sder.empty() ? nullptr : &sder[q]);
        }
      }
      for (int st = s1 - 1; st >= s0; st--) {
        const int q = st - s0;
        // phi^{n+1} = impose(BC(s3))
        k_adj_impose<<<g1(n), 256, 0, a.s>>>(n, ss3[q], mask, o->overlap, lam, lam3);
        bc_bwd(ss3[q], lam3);
        // stage 3: s3 = 1/3 phi^n + 2/3 (s2 + dt L(s2))
        launch_fill(a.s, n, lamphi, 0.0);
        launch_fill(a.s, n, lam2, 0.0);
        const StageDerivs* sd = sder.empty() ? nullptr : &sder[q];
        stage_bwd(ss2[q], lam3, 2.0 / 3.0, 2.0 / 3.0 * dt, lam2, sd, 2);
        k_axpy_fill<<<g1(n), 256, 0, a.s>>>(b, lam3, 1.0 / 3.0, lamphi);
        bc_bwd(ss2[q], lam2);
        // stage 2: s2 = 3/4 phi^n + 1/4 (s1 + dt L(s1))
        launch_fill(a.s, n, lam1, 0.0);
        stage_bwd(ss1[q], lam2, 0.25, 0.25 * dt, lam1, sd, 1);
        k_axpy_fill<<<g1(n), 256, 0, a.s>>>(b, lam2, 0.75, lamphi);
        bc_bwd(ss1[q], lam1);
        // stage 1: s1 = phi^n + dt L(phi^n)
        stage_bwd(sphi[q], lam1, 1.0, dt, lamphi, sd, 0);
        std::swap(lam, lamphi);
      }
    }
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
  } catch (const Error& e) {
    set_error(e.code, e.what());
    return e.code ? e.code : 1;
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
