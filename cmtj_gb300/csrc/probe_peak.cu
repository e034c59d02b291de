// Measurement probe (libcmtj_probe.so, used by bench.py only): FP32 FMA
// throughput of this GPU, the denominator of the FP32 roofline.  Each
// thread runs 8 independent FMA chains so the pipe, not latency, bounds it.
#include <cuda_runtime.h>
#include <stdint.h>

__global__ void k_fma_peak(int iters, float seed, float *out) {
  float a[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) a[k] = seed + threadIdx.x * 1e-7f + k;
  const float b = 0.999999f, c = 1e-7f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = fmaf(a[k], b, c);
  }
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += a[k];
  if (s == 1234.5f) out[0] = s;  // keeps the chains live
}

// Runs the probe `reps` times; returns the best FP32 FLOP/s (2 per FMA).
extern "C" double cmtj_probe_fp32_peak(int reps) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  float *out = nullptr;
  if (cudaMalloc(&out, sizeof(float)) != cudaSuccess) return -1.0;
  const int threads = 256, blocks = sms * 8, iters = 1 << 14;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_fma_peak<<<blocks, threads>>>(iters, 1.0f, out);
  double best = 0.0;
  for (int r = 0; r < reps; ++r) {
    cudaEventRecord(e0);
    k_fma_peak<<<blocks, threads>>>(iters, 1.0f, out);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    const double flops = 2.0 * 8.0 * (double)iters * threads * blocks;
    if (ms > 0 && flops / (ms * 1e-3) > best) best = flops / (ms * 1e-3);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  return best;
}
