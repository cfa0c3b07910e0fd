// w3g_peak.cu -- measurement helper: sustained FP64 FMA throughput of the
// device, the roofline denominator of the FP64-bound element kernels.
// Not part of the WARP3D interface; bench.py calls it once per run.
#include <cuda_runtime.h>
#include "../../include/w3g.h"

namespace {

constexpr int kChains = 8;

__global__ void __launch_bounds__(256) k_dfma_chains(double* out, int iters) {
  double a[kChains];
#pragma unroll
  for (int k = 0; k < kChains; ++k) a[k] = 1.0 + 1e-9 * (threadIdx.x + k);
  const double b = 0.9999999999, c = 1e-12;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < kChains; ++k) a[k] = fma(a[k], b, c);
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < kChains; ++k) s += a[k];
  if (s == 12345.678) out[0] = s;   // keeps the chains live
}

}  // namespace

extern "C" int w3g_measure_fp64_peak(int device, double* tflops) {
  if (!tflops) return W3G_EARG;
  if (cudaSetDevice(device) != cudaSuccess) return W3G_ECUDA;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  double* out = nullptr;
  if (cudaMalloc(&out, sizeof(double)) != cudaSuccess) return W3G_ECUDA;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int blocks = sms * 8, threads = 256, iters = 8192;
  k_dfma_chains<<<blocks, threads>>>(out, 64);   // warm-up
  float best = 1e30f;
  for (int r = 0; r < 5; ++r) {
    cudaEventRecord(e0);
    k_dfma_chains<<<blocks, threads>>>(out, iters);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (err != cudaSuccess) return W3G_ECUDA;
  const double flops = 2.0 * kChains * (double)iters * blocks * threads;
  *tflops = flops / (best * 1e-3) / 1e12;
  return 0;
}
