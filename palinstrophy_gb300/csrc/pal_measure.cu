// Measurement support: the FP64 FMA throughput of the GPU, the ceiling of the
// FP64 plain path (its kernels are bound by the FP64 pipe, not by HBM).  No
// counterpart in the reference.
//
// k_fp64_fma: every thread runs kChains independent FMA chains x <- x a + b for
// `iters` rounds (8 * iters FMAs, 2 flops each); the chains are independent so
// the pipe, not the FMA latency, sets the rate, and the values stay bounded
// (a < 1).  The sum of the chains is stored so nothing is optimised away.
#include <cuda_runtime.h>

#include <algorithm>

#include "palgpu.h"

namespace {

constexpr int kChains = 8;
constexpr int kThreads = 256;

__global__ void __launch_bounds__(kThreads) k_fp64_fma(double* out, int iters, double a, double b) {
  double x[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) x[c] = 1.0 + 1e-3 * (threadIdx.x + c);
#pragma unroll 1
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = fma(x[c], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < kChains; ++c) s += x[c];
  out[blockIdx.x * kThreads + threadIdx.x] = s;
}

}  // namespace

extern "C" int pal_fp64_peak(double* tflops, double* ms) {
  if (!tflops) return PAL_ERR_INVALID;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return PAL_ERR_CUDA;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return PAL_ERR_CUDA;
  const int blocks = sms * 8;  // 2048 resident threads per SM at 256 x 8
  const int iters = 1 << 14;
  double* out = nullptr;
  cudaStream_t s = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = PAL_OK;
  float best = 0.0f;
  if (cudaMalloc(&out, sizeof(double) * blocks * kThreads) != cudaSuccess) return PAL_ERR_OOM;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
      cudaEventCreate(&e1) != cudaSuccess) {
    rc = PAL_ERR_CUDA;
  } else {
    k_fp64_fma<<<blocks, kThreads, 0, s>>>(out, iters, 0.999999, 1e-6);  // warm-up
    for (int t = 0; t < 5 && rc == PAL_OK; ++t) {
      cudaEventRecord(e0, s);
      k_fp64_fma<<<blocks, kThreads, 0, s>>>(out, iters, 0.999999, 1e-6);
      cudaEventRecord(e1, s);
      float m = 0.0f;
      if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&m, e0, e1) != cudaSuccess)
        rc = PAL_ERR_CUDA;
      else if (best == 0.0f || m < best)
        best = m;
    }
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (s) cudaStreamDestroy(s);
  cudaFree(out);
  if (rc != PAL_OK || best <= 0.0f) return rc != PAL_OK ? rc : PAL_ERR_CUDA;
  const double flops = 2.0 * kChains * (double)iters * (double)blocks * kThreads;
  *tflops = flops / (best * 1e-3) / 1e12;
  if (ms) *ms = best;
  return PAL_OK;
}
