// qss_volsum.cu -- the reference's loop-order volume sum, in parallel and
// bit-identical.
//
// qss3dVolumeRegionPhiLessThanZero (qss_util3d.f:288-358) adds one
// contribution per fill-box voxel to a running double in loop order.
// Floating-point addition is not associative, so the result is the
// sequentially rounded sum, not the exact one; a dependent chain of FP64
// additions on GB300 costs ~85 ns per voxel.
//
// The contributions (1 - H(phi)) dV are non-negative, so the running sum s
// never decreases.  While s stays inside one binade [2^E, 2^(E+1)), every
// representable value there is a multiple of u = 2^(E-52), and
//     RN(s + c) = s + u * rne(c / u)
// where rne rounds to the nearest integer -- unless c / u is exactly halfway
// between two integers (then the tie goes to the even significand, which
// depends on s).  So for a chunk of contributions and a known binade, the
// chunk's effect on s is one integer R = sum of rne(c / u), computable in
// parallel and exactly (int64), valid when no element is a tie or not a
// finite non-negative number and s / u + R stays below 2^53 - 1.
//
//   1. k_vol_chunk_sum: per chunk of 4096 contributions, its double sum (any
//      order) -- only to estimate where the running sum stands;
//   2. k_vol_scan: exclusive scan of those sums -> an estimate of s at the
//      start of each chunk, good to far better than a factor of 2;
//   3. k_vol_chunk_r: per chunk, R and a "not applicable" flag for the
//      estimated binade and its two neighbours;
//   4. k_vol_walk: one warp walks the chunks in order with the exact running
//      sum: a chunk whose flag is clear for the binade s is actually in, and
//      that does not reach the top of it, advances s by u * R in one integer
//      addition; any other chunk (the first ones, binade crossings, ties,
//      special values) is added element by element with native FP64
//      additions in loop order.
// Every result equals the sequential loop's bit for bit.
#include "qss_state.h"

namespace qss {

namespace {

constexpr int kVolChunk = 4096;
constexpr int kVolThreads = 256;
constexpr int kWalkBatch = 512;  // chunk descriptors staged in shared memory per round

__device__ __forceinline__ uint64_t dbits(double x) { return (uint64_t)__double_as_longlong(x); }
__device__ __forceinline__ double dfrom(uint64_t b) { return __longlong_as_double((long long)b); }

// unbiased exponent of a positive normal double, or a sentinel
__device__ __forceinline__ int exp_of(double x) {
  const uint64_t b = dbits(x);
  const int e = (int)((b >> 52) & 0x7ff);
  if ((b >> 63) || e == 0 || e == 0x7ff) return -100000;
  return e - 1023;
}

// rne(c / u) for u = 2^(E - 52) (below 2^52 + 1, so 4096 of them fit in
// 64 bits); bad = a tie, a negative or non-finite c, or c >= 2^E
__device__ __forceinline__ uint64_t rne_units(double c, int E, bool& bad) {
  const uint64_t b = dbits(c);
  if ((b << 1) == 0) return 0;  // +-0 leaves s unchanged
  const int ec = (int)((b >> 52) & 0x7ff);
  if ((b >> 63) || ec == 0x7ff) {
    bad = true;
    return 0;
  }
  uint64_t m = b & ((1ull << 52) - 1);
  int ce;  // c = m 2^ce
  if (ec == 0) {
    ce = -1074;
  } else {
    m |= 1ull << 52;
    ce = ec - 1075;
  }
  const int sh = (E - 52) - ce;  // c / u = m / 2^sh
  if (sh <= 0) {  // c >= 2^E: s leaves the binade within this chunk
    bad = true;
    return 0;
  }
  if (sh >= 64) return 0;  // m < 2^53 <= 2^(sh-11): far below half a unit
  const uint64_t q = m >> sh, rem = m & ((1ull << sh) - 1), half = 1ull << (sh - 1);
  if (rem == half) bad = true;
  return q + (rem > half ? 1u : 0u);
}

__global__ void __launch_bounds__(kVolThreads) k_vol_chunk_sum(const double* __restrict__ c, int64_t n,
                                                               double* csum) {
  __shared__ double red[kVolThreads];
  const int64_t base = (int64_t)blockIdx.x * kVolChunk;
  double s = 0;
  for (int t = threadIdx.x; t < kVolChunk; t += kVolThreads) {
    const int64_t q = base + t;
    if (q < n) s += c[q];
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = kVolThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) csum[blockIdx.x] = red[0];
}

// exclusive scan of nc chunk sums in one block of 1024 threads
__global__ void __launch_bounds__(1024) k_vol_scan(const double* __restrict__ csum, int64_t nc, double* est) {
  __shared__ double part[1024];
  const int64_t per = (nc + 1023) / 1024;
  const int64_t lo = threadIdx.x * per, hi = lo + per < nc ? lo + per : nc;
  double s = 0;
  for (int64_t j = lo; j < hi; j++) s += csum[j];
  part[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double run = 0;
    for (int t = 0; t < 1024; t++) {
      const double x = part[t];
      part[t] = run;
      run += x;
    }
  }
  __syncthreads();
  double run = part[threadIdx.x];
  for (int64_t j = lo; j < hi; j++) {
    est[j] = run;
    run += csum[j];
  }
}

// R[3j+q], F[3j+q] for E = exp(est[j]) - 1 + q
__global__ void __launch_bounds__(kVolThreads) k_vol_chunk_r(const double* __restrict__ c, int64_t n,
                                                             const double* __restrict__ est, int64_t* R,
                                                             int64_t* F) {
  __shared__ unsigned long long rs[3][kVolThreads];
  __shared__ int fs[3][kVolThreads];
  const int64_t j = blockIdx.x;
  const int E0 = exp_of(est[j]);
  const int64_t base = j * kVolChunk;
  unsigned long long r[3] = {0, 0, 0};
  bool bad[3] = {E0 < -1000, E0 < -1000, E0 < -1000};
  if (E0 >= -1000) {
    for (int t = threadIdx.x; t < kVolChunk; t += kVolThreads) {
      const int64_t q = base + t;
      if (q >= n) break;
      const double x = c[q];
#pragma unroll
      for (int k = 0; k < 3; k++) r[k] += rne_units(x, E0 - 1 + k, bad[k]);
    }
  }
#pragma unroll
  for (int k = 0; k < 3; k++) {
    rs[k][threadIdx.x] = r[k];
    fs[k][threadIdx.x] = bad[k] ? 1 : 0;
  }
  __syncthreads();
  for (int w = kVolThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
#pragma unroll
      for (int k = 0; k < 3; k++) {
        rs[k][threadIdx.x] += rs[k][threadIdx.x + w];
        fs[k][threadIdx.x] |= fs[k][threadIdx.x + w];
      }
    }
    __syncthreads();
  }
  if (threadIdx.x < 3) {
    const int k = threadIdx.x;
    // a chunk sum that does not fit the significand range is not applicable
    R[3 * j + k] = (int64_t)rs[k][0];
    F[3 * j + k] = (fs[k][0] || rs[k][0] >= (1ull << 53)) ? 1 : 0;
  }
}

// one warp: the exact running sum over the chunks in loop order
__global__ void __launch_bounds__(32) k_vol_walk(const double* __restrict__ c, int64_t n, int64_t nc,
                                                 const double* __restrict__ est, const int64_t* __restrict__ R,
                                                 const int64_t* __restrict__ F, double* out) {
  __shared__ double s_est[kWalkBatch];
  __shared__ long long s_r[3 * kWalkBatch];
  __shared__ int s_f[3 * kWalkBatch];
  __shared__ int s_fast;
  __shared__ double s_sum;
  const int lane = threadIdx.x;
  if (lane == 0) s_sum = 0.0;
  for (int64_t j0 = 0; j0 < nc; j0 += kWalkBatch) {
    const int cnt = (int)((nc - j0) < kWalkBatch ? (nc - j0) : kWalkBatch);
    __syncwarp();
    for (int t = lane; t < cnt; t += 32) s_est[t] = est[j0 + t];
    for (int t = lane; t < 3 * cnt; t += 32) {
      s_r[t] = R[3 * j0 + t];
      s_f[t] = (int)F[3 * j0 + t];
    }
    __syncwarp();
    for (int t = 0; t < cnt; t++) {
      if (lane == 0) {
        s_fast = 0;
        const double s = s_sum;
        const int E = exp_of(s), E0 = exp_of(s_est[t]);
        const int k = E - (E0 - 1);
        if (E > -1000 && E0 > -1000 && k >= 0 && k <= 2 && !s_f[3 * t + k]) {
          const uint64_t M = (dbits(s) & ((1ull << 52) - 1)) | (1ull << 52);
          const uint64_t Rj = (uint64_t)s_r[3 * t + k];
          if (M + Rj < (1ull << 53) - 1) {
            s_sum = dfrom(((uint64_t)(E + 1023) << 52) | (M + Rj - (1ull << 52)));
            s_fast = 1;
          }
        }
      }
      __syncwarp();
      if (!s_fast) {
        // element by element, in loop order, skipping exact zeros
        double v = s_sum;
        const int64_t base = (j0 + t) * kVolChunk;
        const int64_t end = base + kVolChunk < n ? base + kVolChunk : n;
        for (int64_t b = base; b < end; b += 32) {
          const int64_t q = b + lane;
          const double x = (q < end) ? c[q] : 0.0;
          unsigned nz = __ballot_sync(0xffffffffu, x != 0.0);
          while (nz) {
            const int l = __ffs(nz) - 1;
            nz &= nz - 1;
            v = v + __shfl_sync(0xffffffffu, x, l);
          }
        }
        if (lane == 0) s_sum = v;
      }
      __syncwarp();
    }
  }
  if (lane == 0) *out = s_sum;
}

}  // namespace

int64_t loop_sum_scratch_doubles(int64_t n) {
  const int64_t nc = (n + kVolChunk - 1) / kVolChunk;
  return 8 * nc + 64;
}

void launch_loop_sum(cudaStream_t s, const double* c, int64_t n, double* scratch, double* out) {
  if (n <= 0) {
    QSS_CK(cudaMemsetAsync(out, 0, sizeof(double), s));
    return;
  }
  const int64_t nc = (n + kVolChunk - 1) / kVolChunk;
  double* csum = scratch;
  double* est = csum + nc;
  int64_t* R = reinterpret_cast<int64_t*>(est + nc);
  int64_t* F = R + 3 * nc;
  k_vol_chunk_sum<<<(unsigned)nc, kVolThreads, 0, s>>>(c, n, csum);
  k_vol_scan<<<1, 1024, 0, s>>>(csum, nc, est);
  k_vol_chunk_r<<<(unsigned)nc, kVolThreads, 0, s>>>(c, n, est, R, F);
  k_vol_walk<<<1, 32, 0, s>>>(c, n, nc, est, R, F, out);
}

}  // namespace qss

using namespace qss;

// ---------------------------------------------------------------------------
extern "C" {

// See include/lsmpqs_gpu.h.
int qssgpu_loop_sum(const double* values, long long n, double* out) {
  try {
    ensure_device();
    if (n < 0 || (n > 0 && !values) || !out) throw Error(QSSGPU_ERR_ARG, "qssgpu_loop_sum: bad argument");
    cudaStream_t s = nullptr;
    QSS_CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    double *dv = nullptr, *scratch = nullptr, *dout = nullptr;
    const int64_t nn = n > 0 ? n : 1;
    QSS_CK(cudaMalloc(&dv, nn * sizeof(double)));
    QSS_CK(cudaMalloc(&scratch, loop_sum_scratch_doubles(nn) * sizeof(double)));
    QSS_CK(cudaMalloc(&dout, sizeof(double)));
    if (n > 0) QSS_CK(cudaMemcpyAsync(dv, values, n * sizeof(double), cudaMemcpyHostToDevice, s));
    launch_loop_sum(s, dv, n, scratch, dout);
    QSS_CK(cudaGetLastError());
    QSS_CK(cudaMemcpyAsync(out, dout, sizeof(double), cudaMemcpyDeviceToHost, s));
    QSS_CK(cudaStreamSynchronize(s));
    cudaFree(dv);
    cudaFree(scratch);
    cudaFree(dout);
    cudaStreamDestroy(s);
    return 0;
  } catch (const std::exception& e) {
    return report_exception(e);
  }
}

}  // extern "C"
