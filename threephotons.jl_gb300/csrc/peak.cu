// Measured FP32 FMA peak of the device: the roofline denominator of the coupling
// stage (SIMT FP32), which measured copy bandwidth and BF16 GEMM peaks do not
// cover.  Every thread runs 8 independent FMA chains; the grid fills every SM with
// 2048 threads.  No reference counterpart.
#include <cuda_runtime.h>

#include <algorithm>

#include "ctx_internal.h"

namespace {

constexpr int kPeakThreads = 256;
constexpr int kPeakChains = 8;
constexpr int kPeakIters = 4096;

__global__ void __launch_bounds__(kPeakThreads) k_ffma_peak(float x, float y, float* sink) {
  float a[kPeakChains];
#pragma unroll
  for (int c = 0; c < kPeakChains; ++c) a[c] = (float)(threadIdx.x + c) * 1e-3f;
  for (int it = 0; it < kPeakIters; ++it) {
#pragma unroll
    for (int c = 0; c < kPeakChains; ++c) a[c] = fmaf(a[c], x, y);
  }
  float s = 0.f;
#pragma unroll
  for (int c = 0; c < kPeakChains; ++c) s += a[c];
  // the sum is a bounded fixed-point iterate (|x| < 1); the store keeps the chains live
  if (s == 12345.678f) sink[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

extern "C" {

int tp3_measure_fp32_peak(tp3_ctx* c, double* tflops) {
  if (int r = tp3::ctx_check(c)) return r;
  if (!tflops) return tp3::ctx_fail(c, TP3_ERR_ARG, "NULL pointer");
  int sms = 0;
  cudaError_t e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
  if (e != cudaSuccess) return tp3::ctx_cuda_fail(c, e, "SM count");
  const int blocks = sms * (2048 / kPeakThreads);
  float* sink = nullptr;
  cudaEvent_t a = nullptr, b = nullptr;
  if ((e = cudaMalloc(&sink, (size_t)blocks * kPeakThreads * sizeof(float))) != cudaSuccess ||
      (e = cudaEventCreate(&a)) != cudaSuccess || (e = cudaEventCreate(&b)) != cudaSuccess) {
    cudaFree(sink);
    if (a) cudaEventDestroy(a);
    return tp3::ctx_cuda_fail(c, e, "peak setup");
  }
  double best = 0.0;
  for (int rep = 0; rep < 4 && e == cudaSuccess; ++rep) {  // the first run warms up
    cudaEventRecord(a, c->stream);
    k_ffma_peak<<<blocks, kPeakThreads, 0, c->stream>>>(0.9999f, 1e-4f, sink);
    cudaEventRecord(b, c->stream);
    if ((e = cudaEventSynchronize(b)) != cudaSuccess) break;
    float ms = 0.f;
    if ((e = cudaEventElapsedTime(&ms, a, b)) != cudaSuccess) break;
    const double flop = 2.0 * (double)blocks * kPeakThreads * kPeakChains * kPeakIters;
    if (rep > 0 && ms > 0.f) best = std::max(best, flop / (ms * 1e-3) / 1e12);
  }
  if (e == cudaSuccess) e = cudaGetLastError();
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(sink);
  if (e != cudaSuccess) return tp3::ctx_cuda_fail(c, e, "peak kernel");
  *tflops = best;
  return TP3_OK;
}

}  // extern "C"
