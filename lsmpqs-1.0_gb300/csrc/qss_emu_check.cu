// qss_emu_check.cu -- device self-test and throughput probe of the
// integer-pipe FP64 arithmetic (qss_emu.cuh).
//
// qssgpu_emu_selftest compares every emulated operation (and the square root
// of x and |x|) with the native FP64 instruction on n generated operand pairs (raw bit patterns, moderate
// normals, short significands, near neighbours, special values, edges of the
// normal range) and counts mismatches.  qssgpu_op_rates measures the
// throughput of native and emulated division, multiplication and addition
// with 8 independent dependency chains per thread.
#include "qss_emu.cuh"
#include "qss_state.h"

using namespace qss;

namespace {

__device__ __forceinline__ uint64_t splitmix(uint64_t& s) {
  uint64_t z = (s += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

__device__ double gen_operand(int fam, double other, uint64_t& s) {
  using qss_emu::from_bits;
  switch (fam) {
    case 0:
      return from_bits(splitmix(s));
    case 1: {
      const uint64_t r = splitmix(s);
      const uint64_t e = 1023 - 60 + (r >> 8) % 120;
      return from_bits((r & (1ull << 63)) | (e << 52) | (splitmix(s) & qss_emu::kMant));
    }
    case 2: {
      const uint64_t r = splitmix(s);
      const uint64_t e = 1023 - 8 + (r >> 8) % 16;
      const int keep = 1 + (int)((r >> 20) % 30);
      const uint64_t m = splitmix(s) & qss_emu::kMant & ~((1ull << (52 - keep)) - 1);
      return from_bits((r & (1ull << 63)) | (e << 52) | m);
    }
    case 3: {
      const uint64_t r = splitmix(s);
      uint64_t b = qss_emu::bits(other) + (uint64_t)((int64_t)((r >> 8) % 2001) - 1000);
      if (r & 1) b ^= 1ull << 63;
      return from_bits(b);
    }
    case 4: {
      const double sp[] = {0.0, -0.0, 1.0, -1.0, 0.5, 2.0, 0.1, 0.6, 0.3, 1e-35, 1e-300, 1e300,
                           4.9e-324, 2.2250738585072014e-308, 1.7976931348623157e308,
                           __longlong_as_double(0x7ff0000000000000ll),
                           __longlong_as_double((long long)0xfff0000000000000ull),
                           __longlong_as_double(0x7ff8000000000000ll)};
      return sp[splitmix(s) % 18];
    }
    default: {
      const uint64_t r = splitmix(s);
      const uint64_t e = (r & 1) ? 1 + (r >> 8) % 60 : 2046 - (r >> 8) % 60;
      return from_bits((r & (1ull << 63)) | (e << 52) | (splitmix(s) & qss_emu::kMant));
    }
  }
}

__device__ __forceinline__ bool same(double a, double b) {
  if (a != a && b != b) return true;  // NaN payloads may differ
  return qss_emu::bits(a) == qss_emu::bits(b);
}

__device__ void note(unsigned long long* counts, int op, double x, double y, int* first_flag, double* first) {
  atomicAdd(counts + op, 1ull);
  if (atomicCAS(first_flag, 0, 1) == 0) {
    first[0] = op;
    first[1] = x;
    first[2] = y;
  }
}

__global__ void k_emu_selftest(long long n, uint64_t seed, unsigned long long* counts, int* first_flag,
                               double* first) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    uint64_t s = seed ^ ((uint64_t)i * 0xd1342543de82ef95ull);
    const uint64_t r = splitmix(s);
    const int fx = (int)(r % 6), fy = (int)((r >> 8) % 6);
    const double x = gen_operand(fx == 3 ? 1 : fx, 1.0, s);
    const double y = gen_operand(fy, x, s);
    if (!same(qss_emu::div(x, y), __ddiv_rn(x, y))) note(counts, 0, x, y, first_flag, first);
    if (!same(qss_emu::mul(x, y), __dmul_rn(x, y))) note(counts, 1, x, y, first_flag, first);
    if (!same(qss_emu::add(x, y), __dadd_rn(x, y))) note(counts, 2, x, y, first_flag, first);
    if (!same(qss_emu::sub(x, y), __dsub_rn(x, y))) note(counts, 3, x, y, first_flag, first);
    const int k = (int)((r >> 16) % 9) - 4;
    const double p2 = qss_emu::from_bits((uint64_t)(1023 + k) << 52);  // 2^k
    if (!same(qss_emu::scale2(x, k), __dmul_rn(x, p2))) note(counts, 4, x, (double)k, first_flag, first);
    if (qss_emu::gt0(x) != (x > 0) || qss_emu::ge0(x) != (x >= 0) || qss_emu::lt0(x) != (x < 0) ||
        qss_emu::gt(x, y) != (x > y))
      note(counts, 5, x, y, first_flag, first);
    const double sx = __dmul_rn(x, x), sy = __dmul_rn(y, y);
    if (sx == sx && sy == sy && !same(qss_emu::max_nonneg(sx, sy), sx > sy ? sx : sy))
      note(counts, 6, sx, sy, first_flag, first);
    if (!same(qss_emu::sqrt(x), __dsqrt_rn(x))) note(counts, 7, x, 0.0, first_flag, first);
    const double ax = fabs(x);
    if (!same(qss_emu::sqrt(ax), __dsqrt_rn(ax))) note(counts, 7, ax, 0.0, first_flag, first);
    atomicAdd(counts + 8, 1ull);
  }
}

// OP 0: x <- c / x; OP 1: x <- x * a; OP 2: x <- x + b; EMU selects the
// emulated operation; OP 3: x <- x * a on four chains natively and on four
// emulated (shows whether the two kinds of work overlap)
template <int OP, bool EMU>
__global__ void k_op_rate(double* out, int iters, double a, double b, double c) {
  double x[8];
#pragma unroll
  for (int q = 0; q < 8; q++) x[q] = 1.0 + threadIdx.x * 1e-3 + q * 0.125;
  for (int it = 0; it < iters; it++) {
#pragma unroll
    for (int q = 0; q < 8; q++) {
      if (OP == 0) x[q] = EMU ? qss_emu::div(c, x[q]) : __ddiv_rn(c, x[q]);
      else if (OP == 1) x[q] = EMU ? qss_emu::mul(x[q], a) : __dmul_rn(x[q], a);
      else if (OP == 2) x[q] = EMU ? qss_emu::add(x[q], b) : __dadd_rn(x[q], b);
      else x[q] = (q & 1) ? qss_emu::mul(x[q], a) : __dmul_rn(x[q], a);  // half of the chains each way
    }
  }
  double s = 0;
#pragma unroll
  for (int q = 0; q < 8; q++) s += x[q];
  if (s == 1234.5) out[0] = s;  // keeps the chains alive
}

template <int OP, bool EMU>
float time_rate(double* d, int blocks, int threads, int iters) {
  cudaEvent_t e0, e1;
  QSS_CK(cudaEventCreate(&e0));
  QSS_CK(cudaEventCreate(&e1));
  float best = 1e30f;
  for (int rep = 0; rep < 3; rep++) {
    QSS_CK(cudaEventRecord(e0));
    k_op_rate<OP, EMU><<<blocks, threads>>>(d, iters, 1.0 + 0x1p-40, 1e-9, 1.2345678901234567);
    QSS_CK(cudaEventRecord(e1));
    QSS_CK(cudaEventSynchronize(e1));
    float ms = 0;
    QSS_CK(cudaEventElapsedTime(&ms, e0, e1));
    if (rep > 0 && ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return best;
}

}  // namespace

extern "C" {

// See include/lsmpqs_gpu.h.
int qssgpu_emu_selftest(long long n, unsigned long long seed, long long* counts, double* first) {
  try {
    ensure_device();
    if (n < 0 || !counts) throw Error(QSSGPU_ERR_ARG, "qssgpu_emu_selftest: bad argument");
    unsigned long long* dc = nullptr;
    int* dflag = nullptr;
    double* dfirst = nullptr;
    QSS_CK(cudaMalloc(&dc, 9 * sizeof(unsigned long long)));
    QSS_CK(cudaMalloc(&dflag, sizeof(int)));
    QSS_CK(cudaMalloc(&dfirst, 3 * sizeof(double)));
    QSS_CK(cudaMemset(dc, 0, 9 * sizeof(unsigned long long)));
    QSS_CK(cudaMemset(dflag, 0, sizeof(int)));
    QSS_CK(cudaMemset(dfirst, 0, 3 * sizeof(double)));
    int dev = 0, sms = 0;
    QSS_CK(cudaGetDevice(&dev));
    QSS_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    k_emu_selftest<<<sms * 4, 256>>>(n, seed, dc, dflag, dfirst);
    QSS_CK(cudaGetLastError());
    unsigned long long hc[9];
    double hf[3];
    QSS_CK(cudaMemcpy(hc, dc, sizeof hc, cudaMemcpyDeviceToHost));
    QSS_CK(cudaMemcpy(hf, dfirst, sizeof hf, cudaMemcpyDeviceToHost));
    cudaFree(dc);
    cudaFree(dflag);
    cudaFree(dfirst);
    for (int q = 0; q < 9; q++) counts[q] = (long long)hc[q];
    if (first)
      for (int q = 0; q < 3; q++) first[q] = hf[q];
    return 0;
  } catch (const std::exception& e) {
    report_exception(e);
    return 1;
  }
}

// See include/lsmpqs_gpu.h.
int qssgpu_op_rates(double* out) {
  try {
    ensure_device();
    int dev = 0, sms = 0;
    QSS_CK(cudaGetDevice(&dev));
    QSS_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    double* d = nullptr;
    QSS_CK(cudaMalloc(&d, sizeof(double)));
    const int threads = 256, blocks = sms * 4, iters = 512;
    const double ops = (double)blocks * threads * iters * 8;
    const float t[7] = {time_rate<0, false>(d, blocks, threads, iters), time_rate<0, true>(d, blocks, threads, iters),
                        time_rate<1, false>(d, blocks, threads, iters), time_rate<1, true>(d, blocks, threads, iters),
                        time_rate<2, false>(d, blocks, threads, iters), time_rate<2, true>(d, blocks, threads, iters),
                        time_rate<3, false>(d, blocks, threads, iters)};
    for (int q = 0; q < 7; q++) out[q] = ops / (t[q] * 1e-3) / 1e9;
    cudaFree(d);
    return 0;
  } catch (const std::exception& e) {
    report_exception(e);
    return 1;
  }
}

}  // extern "C"
