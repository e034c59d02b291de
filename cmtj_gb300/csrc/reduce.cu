// On-device reductions of batched logs.
//
// cmtj_spectrum_f32 replaces the per-junction numpy/scipy post-processing of
// PIMM_procedure (cmtj/utils/procedures.py:28-39, compute_spectrum_strip:
// |scipy.fft.fft(m)| truncated to a frequency range): one CTA per log row
// loads the last n_fft samples into shared memory, runs an in-place
// radix-2 decimation-in-time FFT (bit-reversed load, log2(n_fft) butterfly
// stages, twiddles from sincospif), and writes |X[k]| for k in [bin_lo,
// bin_hi).  Work per row is O(n log n) FP32 in shared memory; the kernel is
// bound by reading the log rows from HBM.
#include "common.cuh"

namespace {

constexpr int kMaxFft = 8192;
constexpr int kFftThreads = 512;

__global__ void __launch_bounds__(kFftThreads) k_spectrum(const float *__restrict__ series, int64_t row_stride,
                                                          int32_t series_len, int32_t log2n, int32_t bin_lo,
                                                          int32_t bin_hi, float *__restrict__ out) {
  extern __shared__ __align__(16) float sm[];
  const int n = 1 << log2n;
  float *re = sm;
  float *im = sm + n;
  float *twc = sm + 2 * n;       // cos(2 pi k / n), k < n/2
  float *tws = twc + n / 2;      // sin(2 pi k / n)
  const int64_t row = blockIdx.x;
  const float *src = series + row * row_stride + (series_len - n);
  for (int k = threadIdx.x; k < n / 2; k += blockDim.x) {
    float s, c;
    sincospif(2.0f * (float)k / (float)n, &s, &c);
    twc[k] = c;
    tws[k] = s;
  }
  for (int t = threadIdx.x; t < n; t += blockDim.x) {
    const int r = __brev(t) >> (32 - log2n);
    re[r] = src[t];
    im[r] = 0.f;
  }
  __syncthreads();
  for (int s = 0; s < log2n; ++s) {
    const int half = 1 << s;
    const int tstep = n >> (s + 1);
    for (int b = threadIdx.x; b < n / 2; b += blockDim.x) {
      const int pos = b & (half - 1);
      const int i = ((b >> s) << (s + 1)) + pos;
      const int j = i + half;
      const float wr = twc[pos * tstep], wi = -tws[pos * tstep];  // exp(-2 pi i k/n)
      const float xr = re[j], xi = im[j];
      const float tr = fmaf(wr, xr, -wi * xi);
      const float ti = fmaf(wr, xi, wi * xr);
      const float ar = re[i], ai = im[i];
      re[i] = ar + tr;
      im[i] = ai + ti;
      re[j] = ar - tr;
      im[j] = ai - ti;
    }
    __syncthreads();
  }
  const int nb = bin_hi - bin_lo;
  float *dst = out + row * (int64_t)nb;
  for (int k = threadIdx.x; k < nb; k += blockDim.x) {
    const int q = bin_lo + k;
    dst[k] = sqrtf(fmaf(re[q], re[q], im[q] * im[q]));
  }
}

}  // namespace

extern "C" int cmtj_spectrum_f32(const float *d_series, int64_t row_stride, int32_t n_rows, int32_t series_len,
                                 int32_t n_fft, int32_t bin_lo, int32_t bin_hi, float *d_out, void *stream) {
  int log2n = 0;
  while ((1 << log2n) < n_fft) ++log2n;
  if (n_rows < 0 || n_fft < 2 || (1 << log2n) != n_fft || n_fft > kMaxFft) {
    cmtj_set_error("cmtj_spectrum_f32: n_fft must be a power of two in [2, %d], got %d", kMaxFft, n_fft);
    return CMTJ_ERR_ARG;
  }
  if (series_len < n_fft || row_stride < series_len || bin_lo < 0 || bin_hi > n_fft || bin_lo >= bin_hi) {
    cmtj_set_error("cmtj_spectrum_f32: bad window (series_len=%d, stride=%lld, bins [%d,%d))", series_len,
                   (long long)row_stride, bin_lo, bin_hi);
    return CMTJ_ERR_ARG;
  }
  if (n_rows == 0) return CMTJ_OK;
  if (!d_series || !d_out) {
    cmtj_set_error("cmtj_spectrum_f32: null buffer");
    return CMTJ_ERR_ARG;
  }
  const size_t smem = (size_t)(3 * n_fft) * sizeof(float);
  if (smem > 48 * 1024) {
    CMTJ_CUDA_TRY(cudaFuncSetAttribute(k_spectrum, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  }
  k_spectrum<<<n_rows, kFftThreads, smem, cmtj_stream(stream)>>>(d_series, row_stride, series_len, log2n, bin_lo,
                                                                  bin_hi, d_out);
  CMTJ_LAUNCH_CHECK("k_spectrum");
  return CMTJ_OK;
}
