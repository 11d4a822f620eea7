// qss_bench.cu -- FP64 throughput probe used to state the roofline of the
// FP64-bound stencil kernels (the measured-peaks file of the pool carries HBM
// and bf16 figures only).  Each thread runs 8 independent dependency chains
// so the FP64 pipe, not latency, limits the rate.
#include "qss_state.h"

using namespace qss;

namespace {

template <int KIND>
__global__ void k_fp64_probe(double* out, int iters, double a, double b) {
  double x[8];
#pragma unroll
  for (int q = 0; q < 8; q++) x[q] = threadIdx.x * 1e-3 + q;
  for (int it = 0; it < iters; it++) {
#pragma unroll
    for (int q = 0; q < 8; q++) {
      if (KIND == 0) x[q] = __fma_rn(x[q], a, b);  // DFMA: 2 flops
      else x[q] = __dadd_rn(x[q], b);              // DADD: 1 flop
    }
  }
  double s = 0;
#pragma unroll
  for (int q = 0; q < 8; q++) s += x[q];
  if (s == 1234.5) out[0] = s;  // keeps the chains alive
}

}  // namespace

extern "C" {

// out[0] = DFMA TFLOP/s (2 flops per FMA), out[1] = DADD TFLOP/s; returns 0 on success
int qssgpu_fp64_peak(double* out) {
  try {
    ensure_device();
    int dev = 0, sms = 0;
    QSS_CK(cudaGetDevice(&dev));
    QSS_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    double* d = nullptr;
    QSS_CK(cudaMalloc(&d, sizeof(double)));
    const int iters = 4096, threads = 256, blocks = sms * 8;
    cudaEvent_t e0, e1;
    QSS_CK(cudaEventCreate(&e0));
    QSS_CK(cudaEventCreate(&e1));
    for (int kind = 0; kind < 2; kind++) {
      float best = 1e30f;
      for (int rep = 0; rep < 4; rep++) {
        QSS_CK(cudaEventRecord(e0));
        if (kind == 0) k_fp64_probe<0><<<blocks, threads>>>(d, iters, 0.999999, 1e-7);
        else k_fp64_probe<1><<<blocks, threads>>>(d, iters, 0.999999, 1e-7);
        QSS_CK(cudaEventRecord(e1));
        QSS_CK(cudaEventSynchronize(e1));
        float ms = 0;
        QSS_CK(cudaEventElapsedTime(&ms, e0, e1));
        if (rep > 0 && ms < best) best = ms;
      }
      const double ops = (double)blocks * threads * iters * 8;
      out[kind] = ops * (kind == 0 ? 2.0 : 1.0) / (best * 1e-3) / 1e12;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(d);
    return 0;
  } catch (const std::exception& e) {
    report_exception(e);
    return 1;
  }
}

}  // extern "C"
