// measure.cu -- the FP32 rate of this GPU, measured: the denominator of the line-profile kernel's
// roofline (that kernel is bound by FP32 instruction issue, not by memory).
//
// fma_rate_kernel: every thread runs kChains independent FMA chains of kIters steps; the grid holds
// eight CTAs of 256 threads per SM, so that every scheduler has enough independent work.  The
// chains stay finite (|a| shrinks towards c / (1 - b)), and their sum is stored so that nothing is
// optimised away.  Two FLOPs per FMA.
#include <cuda_runtime.h>

#include <string>

#include "../../include/relxill_gb300.h"

namespace relx {

constexpr int kChains = 8;
constexpr int kIters = 8192;
constexpr int kRateThreads = 256;

__global__ void __launch_bounds__(kRateThreads) fma_rate_kernel(float b, float c, float *out) {
  float a[kChains];
#pragma unroll
  for (int k = 0; k < kChains; k++) a[k] = (float) (threadIdx.x + k);
  for (int i = 0; i < kIters; i++) {
#pragma unroll
    for (int k = 0; k < kChains; k++) a[k] = fmaf(a[k], b, c);
  }
  float s = 0.0f;
#pragma unroll
  for (int k = 0; k < kChains; k++) s += a[k];
  out[blockIdx.x * kRateThreads + threadIdx.x] = s;
}

}  // namespace relx

extern "C" int relx_fp32_rate(double *gflops) {
  if (!gflops) return 9;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return 6;
  const int blocks = sms * 8;
  float *out = nullptr;
  if (cudaMalloc(&out, sizeof(float) * (size_t) blocks * relx::kRateThreads) != cudaSuccess) return 7;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  relx::fma_rate_kernel<<<blocks, relx::kRateThreads>>>(0.999f, 1e-3f, out);  // warm-up
  float best = 1e30f;
  for (int r = 0; r < 5; r++) {
    cudaEventRecord(e0);
    relx::fma_rate_kernel<<<blocks, relx::kRateThreads>>>(0.999f, 1e-3f, out);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  const cudaError_t e = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (e != cudaSuccess) return 6;
  const double flops = 2.0 * relx::kChains * (double) relx::kIters * blocks * relx::kRateThreads;
  *gflops = flops / (best * 1e-3) / 1e9;
  return 0;
}
