// Measured FP64 FMA rate of the device (elp_peak_fp64): the roofline of the
// plain FP64 path and of the assembly kernels is FP64 arithmetic, and the
// device's FP64 rate is far below its FP32 and tensor rates, so it is
// measured here rather than taken from a data sheet.
#include <cuda_runtime.h>

#include "device.cuh"

namespace elp {
namespace {

// every thread runs 8 independent FMA chains of `iters` steps; the result is
// written only when it equals a value the chains never reach, so the
// compiler keeps the arithmetic
__global__ void k_fp64_fma(int iters, double seed, double* __restrict__ sink) {
  double a0 = seed + threadIdx.x, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3, a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6,
         a7 = a0 + 7;
  const double m = 0.999999, c = 1e-7;
  for (int i = 0; i < iters; ++i) {
    a0 = fma(a0, m, c); a1 = fma(a1, m, c); a2 = fma(a2, m, c); a3 = fma(a3, m, c);
    a4 = fma(a4, m, c); a5 = fma(a5, m, c); a6 = fma(a6, m, c); a7 = fma(a7, m, c);
  }
  const double s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
  if (s == -1.0) sink[blockIdx.x] = s;
}

}  // namespace
}  // namespace elp

using namespace elp;

extern "C" int elp_peak_fp64(double* tflops) {
  if (!tflops) { set_error("null argument"); return ELP_ERR_ARG; }
  int dev = 0, sms = 0;
  ELP_CUDA(cudaGetDevice(&dev));
  ELP_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  DevBuf<double> sink;
  ELP_CUDA(sink.alloc(1024 * 8));
  const int blocks = sms * 8, threads = 256, iters = 1 << 14;
  cudaEvent_t e0, e1;
  ELP_CUDA(cudaEventCreate(&e0));
  ELP_CUDA(cudaEventCreate(&e1));
  k_fp64_fma<<<blocks, threads>>>(iters / 16, 1.0, sink.p);  // warm-up
  ELP_CUDA(cudaGetLastError());
  ELP_CUDA(cudaEventRecord(e0));
  for (int r = 0; r < 3; ++r) k_fp64_fma<<<blocks, threads>>>(iters, 1.0 + r, sink.p);
  ELP_CUDA(cudaEventRecord(e1));
  ELP_CUDA(cudaEventSynchronize(e1));
  float ms = 0.f;
  ELP_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  const double flops = 3.0 * blocks * threads * (double)iters * 8.0 * 2.0;
  *tflops = flops / (ms * 1e-3) / 1e12;
  return ELP_OK;
}
