// Measurement probe of bench.py (built into _build/libbench_peak.so by
// bench.build_peak_probe, never part of libcmtj_gpu.so): FP32 FMA
// throughput of this GPU, the denominator of the FP32 roofline.  Each
// thread runs 8 independent FMA chains so the pipe, not latency, bounds it.
// Two forms: scalar FFMA, and the packed two-lane __ffma2_rn (sm_100+).
// Also the cycles one warp spends per FP64 FMA, with one dependent chain
// and with several independent ones: the cost model of the FP64 plain form.
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

__global__ void k_fma2_peak(int iters, float seed, float *out) {
  float2 a[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) a[k] = make_float2(seed + threadIdx.x * 1e-7f + k, seed - k);
  const float2 b = make_float2(0.999999f, 0.999998f), c = make_float2(1e-7f, 2e-7f);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = __ffma2_rn(a[k], b, c);
  }
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += a[k].x + a[k].y;
  if (s == 1234.5f) out[0] = s;
}

// One warp: CH independent chains of dependent DFMAs, clock64 around the
// loop; cycles[0] gets the elapsed SM cycles.
template <int CH>
__global__ void k_dfma_cycles(int iters, double seed, long long *cycles, double *sink) {
  double a[CH];
#pragma unroll
  for (int k = 0; k < CH; ++k) a[k] = seed + threadIdx.x * 1e-9 + k;
  const double b = 0.9999999, c = 1e-12;
  const long long t0 = clock64();
#pragma unroll 4
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < CH; ++k) a[k] = fma(a[k], b, c);
  }
  const long long t1 = clock64();
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < CH; ++k) s += a[k];
  if (s == 1234.5) sink[0] = s;
  if (threadIdx.x == 0) cycles[0] = t1 - t0;
}

namespace {
template <int CH>
double dfma_cycles() {
  long long *cyc = nullptr;
  double *sink = nullptr;
  if (cudaMalloc(&cyc, sizeof(long long)) != cudaSuccess) return -1.0;
  if (cudaMalloc(&sink, sizeof(double)) != cudaSuccess) {
    cudaFree(cyc);
    return -1.0;
  }
  const int iters = 1 << 12;
  long long c = 0;
  double best = -1.0;
  for (int r = 0; r < 3; ++r) {  // the first run warms the instruction cache
    k_dfma_cycles<CH><<<1, 32>>>(iters, 1.0, cyc, sink);
    if (cudaMemcpy(&c, cyc, sizeof(c), cudaMemcpyDeviceToHost) != cudaSuccess) break;
    const double per = (double)c / ((double)iters * CH);
    if (r > 0 && (best < 0 || per < best)) best = per;
  }
  cudaFree(cyc);
  cudaFree(sink);
  return best;
}

// Runs one probe kernel `reps` times; returns the best FLOP/s (2 per lane FMA).
template <typename K>
double time_probe(K kernel, int reps, double lanes) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  float *out = nullptr;
  if (cudaMalloc(&out, sizeof(float)) != cudaSuccess) return -1.0;
  const int threads = 256, blocks = sms * 8, iters = 1 << 14;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  kernel<<<blocks, threads>>>(iters, 1.0f, out);
  double best = 0.0;
  for (int r = 0; r < reps; ++r) {
    cudaEventRecord(e0);
    kernel<<<blocks, threads>>>(iters, 1.0f, out);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    const double flops = 2.0 * lanes * 8.0 * (double)iters * threads * blocks;
    if (ms > 0 && flops / (ms * 1e-3) > best) best = flops / (ms * 1e-3);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  return best;
}
}  // namespace

// Best FP32 FLOP/s of scalar FFMA over `reps` runs.
extern "C" double cmtj_probe_fp32_peak(int reps) { return time_probe(k_fma_peak, reps, 1.0); }
// Best FP32 FLOP/s of packed FFMA2 (two FMAs per lane per instruction).
extern "C" double cmtj_probe_fp32x2_peak(int reps) { return time_probe(k_fma2_peak, reps, 2.0); }
// SM cycles per DFMA of one warp: one dependent chain (chains = 1) or four
// independent chains (chains = 4, the issue interval); -1 on error.
extern "C" double cmtj_probe_fp64_cycles(int chains) {
  return chains == 4 ? dfma_cycles<4>() : dfma_cycles<1>();
}
