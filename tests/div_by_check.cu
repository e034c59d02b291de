// Test harness (built by tests/test_gpu_div_by.py, not part of the library):
// div_by() of cmtj_gb300/csrc/recip.cuh against the IEEE quotient a / b, bit
// for bit, for n (a, b) pairs.
#include <cuda_runtime.h>
#include <stdint.h>

#include "recip.cuh"

__global__ void k_div_check(const double *a, const double *b, int n, unsigned long long *fast,
                            unsigned long long *ieee) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const cmtjd::Recip R = cmtjd::recip_of(b[i]);
  fast[i] = (unsigned long long)__double_as_longlong(cmtjd::div_by(a[i], R));
  ieee[i] = (unsigned long long)__double_as_longlong(a[i] / b[i]);
}

// Host entry: copies in, runs, copies both bit patterns out.  0 on success.
extern "C" int run_div_check(const double *a, const double *b, int n, unsigned long long *fast,
                             unsigned long long *ieee) {
  double *da = nullptr, *db = nullptr;
  unsigned long long *df = nullptr, *di = nullptr;
  const size_t sd = (size_t)n * sizeof(double), su = (size_t)n * sizeof(unsigned long long);
  int rc = 1;
  if (cudaMalloc(&da, sd) == cudaSuccess && cudaMalloc(&db, sd) == cudaSuccess && cudaMalloc(&df, su) == cudaSuccess &&
      cudaMalloc(&di, su) == cudaSuccess && cudaMemcpy(da, a, sd, cudaMemcpyHostToDevice) == cudaSuccess &&
      cudaMemcpy(db, b, sd, cudaMemcpyHostToDevice) == cudaSuccess) {
    k_div_check<<<(n + 255) / 256, 256>>>(da, db, n, df, di);
    if (cudaDeviceSynchronize() == cudaSuccess && cudaMemcpy(fast, df, su, cudaMemcpyDeviceToHost) == cudaSuccess &&
        cudaMemcpy(ieee, di, su, cudaMemcpyDeviceToHost) == cudaSuccess)
      rc = 0;
  }
  cudaFree(da);
  cudaFree(db);
  cudaFree(df);
  cudaFree(di);
  return rc;
}
