// On-device reductions of batched logs.
//
// cmtj_spectrum_f32 replaces the per-junction numpy/scipy post-processing of
// PIMM_procedure (cmtj/utils/procedures.py:28-39, compute_spectrum_strip:
// |scipy.fft.fft(m)| truncated to a frequency range).  One CTA of n/16
// threads transforms one log row.  The row is real, so its n-point spectrum
// comes from an n/2-point complex FFT of (even, odd) sample pairs and one
// unpacking pass over the kept bins.  The complex FFT is a Stockham FFT
// (self-sorting, no bit reversal) in radix-8 stages, with a final radix-4
// or radix-2 stage when log2(n/2) is not a multiple of 3.  Every thread
// keeps its 8 points in registers through a stage; stages exchange through
// one shared-memory buffer (n/2 complex floats, one padding word per 32
// against bank conflicts in the strided stores), so an n = 4096 spectrum
// takes 4 stages and 8 CTA barriers.  The first stage reads the row
// straight from HBM (coalesced); the last pass writes |X[k]| for k in
// [bin_lo, bin_hi).
#include "common.cuh"

namespace {

constexpr int kMaxFft = 8192;

// Shared-memory slot of point i: one padding word after every 32, so the
// strided stores of the first stages (stride 8 in the first radix-8 stage)
// fall in distinct banks.
__device__ __forceinline__ int pad(int i) { return i + (i >> 5); }

struct C2 {
  float r, i;
};
__device__ __forceinline__ C2 c2(float r, float i) {
  C2 z;
  z.r = r;
  z.i = i;
  return z;
}
__device__ __forceinline__ C2 cadd(C2 a, C2 b) { return c2(a.r + b.r, a.i + b.i); }
__device__ __forceinline__ C2 csub(C2 a, C2 b) { return c2(a.r - b.r, a.i - b.i); }
__device__ __forceinline__ C2 cmul(C2 a, C2 b) { return c2(fmaf(a.r, b.r, -a.i * b.i), fmaf(a.r, b.i, a.i * b.r)); }
// multiplication by -i (forward-transform rotation)
__device__ __forceinline__ C2 mul_mi(C2 a) { return c2(a.i, -a.r); }

// In-register DFTs of size 2, 4, 8 (forward, e^{-2 pi i jk/R}).
__device__ __forceinline__ void dft2(C2 &a, C2 &b) {
  const C2 t = a;
  a = cadd(t, b);
  b = csub(t, b);
}
__device__ __forceinline__ void dft4(C2 *v) {
  C2 a0 = v[0], a1 = v[1], a2 = v[2], a3 = v[3];
  dft2(a0, a2);
  dft2(a1, a3);
  a3 = mul_mi(a3);
  dft2(a0, a1);
  dft2(a2, a3);
  v[0] = a0;
  v[1] = a2;
  v[2] = a1;
  v[3] = a3;
}
__device__ __forceinline__ void dft8(C2 *v) {
  const float h = 0.70710678118654752f;
  C2 e[4] = {v[0], v[2], v[4], v[6]}, o[4] = {v[1], v[3], v[5], v[7]};
  dft4(e);
  dft4(o);
  // o[k] *= e^{-2 pi i k/8}
  o[1] = c2(h * (o[1].r + o[1].i), h * (o[1].i - o[1].r));
  o[2] = mul_mi(o[2]);
  o[3] = c2(h * (o[3].i - o[3].r), -h * (o[3].r + o[3].i));
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    v[k] = cadd(e[k], o[k]);
    v[k + 4] = csub(e[k], o[k]);
  }
}

// One Stockham stage of radix R over n points, `groups` R-point groups per
// thread.  Group g reads x[g + r*n/R], twiddles by w^(r*k) with
// w = e^{-2 pi i / (Ns R)}, k = g mod Ns, and writes y[(g/Ns) Ns R + k + r Ns].
template <int R>
__device__ __forceinline__ void stage(const float *__restrict__ src_re, const float *__restrict__ src_im,
                                      float *dst_re, float *dst_im, int n, int Ns, bool from_global,
                                      const float *__restrict__ grow, bool first) {
  constexpr int G = 8 / R;
  C2 v[G][R];
  const int stride = n / R;
#pragma unroll
  for (int q = 0; q < G; ++q) {
    const int g = threadIdx.x * G + q;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int idx = g + r * stride;
      // from global: point idx of the half-length complex sequence
      // z[m] = x[2m] + i x[2m+1] of the real row x
      v[q][r] = from_global ? c2(grow[2 * idx], grow[2 * idx + 1]) : c2(src_re[pad(idx)], src_im[pad(idx)]);
    }
    const int k = g % Ns;
    if (!first && k) {
      float sn, cs;
      sincospif(-2.0f * (float)k / (float)(Ns * R), &sn, &cs);
      const C2 w1 = c2(cs, sn);
      C2 w = w1;
#pragma unroll
      for (int r = 1; r < R; ++r) {
        v[q][r] = cmul(v[q][r], w);
        w = cmul(w, w1);
      }
    }
    if (R == 8) dft8(v[q]);
    else if (R == 4) dft4(v[q]);
    else dft2(v[q][0], v[q][1]);
  }
  __syncthreads();  // everyone has read src before anyone overwrites it
#pragma unroll
  for (int q = 0; q < G; ++q) {
    const int g = threadIdx.x * G + q;
    const int k = g % Ns;
    const int base = (g / Ns) * Ns * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      dst_re[pad(base + r * Ns)] = v[q][r].r;
      dst_im[pad(base + r * Ns)] = v[q][r].i;
    }
  }
  __syncthreads();
}

// |X[k]| of a real row x of n points, from the n/2-point complex FFT Z of
// z[m] = x[2m] + i x[2m+1]:  with E = FFT(x even), O = FFT(x odd),
// E[k] = (Z[k] + conj Z[h-k]) / 2, O[k] = (Z[k] - conj Z[h-k]) / 2i and
// X[k] = E[k] + W_n^k O[k] (h = n/2, indices mod h); bins above n/2 use
// |X[k]| = |X[n-k]|.
__global__ void __launch_bounds__(512, 2) k_spectrum(const float *__restrict__ series, int64_t row_stride,
                                                  int32_t series_len, int32_t n, int32_t bin_lo, int32_t bin_hi,
                                                  float *__restrict__ out) {
  extern __shared__ __align__(16) float sm[];
  const int h = n / 2;
  float *re = sm;
  float *im = sm + pad(h);
  const int64_t row = blockIdx.x;
  const float *src = series + row * row_stride + (series_len - n);
  int Ns = 1;
  bool first = true;
  while (Ns < h) {
    const int left = h / Ns;
    if (left >= 8) {
      stage<8>(re, im, re, im, h, Ns, first, src, first);
      Ns *= 8;
    } else if (left == 4) {
      stage<4>(re, im, re, im, h, Ns, first, src, first);
      Ns *= 4;
    } else {
      stage<2>(re, im, re, im, h, Ns, first, src, first);
      Ns *= 2;
    }
    first = false;
  }
  const int nb = bin_hi - bin_lo;
  float *dst = out + row * (int64_t)nb;
  for (int k = threadIdx.x; k < nb; k += blockDim.x) {
    int q = bin_lo + k;
    if (q > h) q = n - q;
    const int a = q == h ? 0 : q;
    const int b = q == 0 ? 0 : h - q;
    const C2 zk = c2(re[pad(a)], im[pad(a)]);
    const C2 zc = c2(re[pad(b)], -im[pad(b)]);
    const C2 e = c2(0.5f * (zk.r + zc.r), 0.5f * (zk.i + zc.i));
    const C2 o = c2(0.5f * (zk.i - zc.i), -0.5f * (zk.r - zc.r));
    float sn, cs;
    sincospif(-2.0f * (float)q / (float)n, &sn, &cs);
    const C2 x = cadd(e, cmul(c2(cs, sn), o));
    dst[k] = sqrtf(fmaf(x.r, x.r, x.i * x.i));
  }
}

}  // namespace

extern "C" int cmtj_spectrum_f32(const float *d_series, int64_t row_stride, int32_t n_rows, int32_t series_len,
                                 int32_t n_fft, int32_t bin_lo, int32_t bin_hi, float *d_out, void *stream) {
  int log2n = 0;
  while ((1 << log2n) < n_fft) ++log2n;
  if (n_rows < 0 || n_fft < 64 || (1 << log2n) != n_fft || n_fft > kMaxFft) {
    cmtj_set_error("cmtj_spectrum_f32: n_fft must be a power of two in [64, %d], got %d", kMaxFft, n_fft);
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
  // n/2 complex points, re and im each padded by one word per 32
  const size_t smem = 2 * (size_t)(n_fft / 2 + n_fft / 64) * sizeof(float);
  if (smem > 48 * 1024) {
    CMTJ_CUDA_TRY(cudaFuncSetAttribute(k_spectrum, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  }
  k_spectrum<<<n_rows, n_fft / 16, smem, cmtj_stream(stream)>>>(d_series, row_stride, series_len, n_fft, bin_lo,
                                                                bin_hi, d_out);
  CMTJ_LAUNCH_CHECK("k_spectrum");
  return CMTJ_OK;
}
