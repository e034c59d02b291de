// Buffered 1/f^alpha noise on the device: BufferedAlphaNoise::fillBuffer
// (core/noise.hpp:138-241) for many buffers at once.
//
// The reference colours N white Gaussian draws w (standard deviation std)
// with the filter h[0] = 1, h[i] = h[i-1] * (alpha/2 + i - 1) / i (float,
// noise.hpp:171-176): both are zero-padded to 2N, transformed, multiplied
// in bins [0, N), bins 0 and N-1 are halved, bins [N, 2N) are dropped, and
// the real part of the inverse transform's first N values divided by N is
// the buffer (noise.hpp:186-225).  With C the 2N-point spectrum of the
// linear convolution c = h * w (C = H W), that is exactly
//
//   out[n] = c[n] - [C_N (-1)^n + Re(C_{N-1} e^{i pi (N-1) n / N})] / 2N
//          = c[n] - (-1)^n [H_N W_N + Re(C_{N-1} e^{-i pi n / N})] / 2N,
//
// with H_N = sum_j h_j (-1)^j and H_{N-1} = sum_j h_j e^{-i pi j (N-1)/N}
// (W alike): the causal filter of the white draws, less the two top bins
// the reference's halving and dropping leave out.  Here c comes from one
// power-of-two FFT convolution of size M >= 2N - 1, and the four bin sums
// from FP64 reductions over h and w.
//
// Per batch of buffer rows (scratch: three M-point complex rows each, plus
// a header of six doubles):
//   k_alpha_fill     white draws (Philox, or the caller's), the factors of
//                    the filter recurrence, zero padding
//   k_alpha_weights  h as the reference's sequential float product, one
//                    warp per row
//   k_alpha_bins     H_N, H_{N-1}, W_N, W_{N-1} (FP64 sums, fixed order)
//   k_fft_pass<R>    Stockham radix-4 passes (radix-2 tail), forward h and
//                    w, pointwise product, inverse
//   k_alpha_finish   c / M less the top-bin term, rounded to float
// This runs once per simulation run, before its time loop; it is HBM-bound
// (each FFT pass reads and writes M complex floats per row).
#include "common.cuh"
#include "philox.cuh"

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
// i * a
__device__ __forceinline__ float2 cmuli(float2 a) { return make_float2(-a.y, a.x); }

// White draws and zero padding: A[row][m] = w_m (m < N), 0 beyond.  The
// weight row gets the factors of the filter recurrence (noise.hpp:171-176),
// in the reference's float arithmetic: Hh[0] = 1 and, for 1 <= m < N,
// Hh[m] = (float)(0.5 * alpha + (float)(m - 1)) / (float)m; 0 beyond.
// alpha outside [0, 2] (which setAlphaNoise rejects) gives a NaN row.
__global__ void k_alpha_fill(const cmtj_alpha_noise_t *__restrict__ specs, int row0, int rows, uint32_t N,
                             uint32_t M, const float *__restrict__ white, float2 *__restrict__ A,
                             float2 *__restrict__ Hh) {
  const uint64_t total = (uint64_t)rows * M;
  for (uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (uint64_t)gridDim.x * blockDim.x) {
    const int r = (int)(idx / M);
    const uint32_t m = (uint32_t)(idx % M);
    const cmtj_alpha_noise_t &s = specs[row0 + r];
    float w = 0.f, h = 0.f;
    if (m < N) {
      if (white) {
        w = white[(size_t)(row0 + r) * N + m];
      } else {
        const int c = s.component < 0 ? 0 : (s.component > 2 ? 2 : s.component);
        w = (float)(s.std * cmtj_alpha_gaussian_f64(s.seed_lo, s.seed_hi, s.counter + m, c));
      }
      const bool ok = s.alpha >= 0.0 && s.alpha <= 2.0;
      h = !ok ? __int_as_float(0x7fffffff)
              : (m == 0 ? 1.0f : (float)(0.5 * s.alpha + (double)(float)(m - 1)) / (float)m);
    }
    A[idx] = make_float2(w, 0.f);
    Hh[idx] = make_float2(h, 0.f);
  }
}

// h_m = h_{m-1} * factor_m over each weight row, in place: the reference's
// sequential float product, in order.  One warp per row: each round the
// warp loads 32 x 8 factors (coalesced), then the running product passes
// from lane to lane, each lane multiplying through its 8; the next round's
// loads are issued before this round's chain.
__global__ void __launch_bounds__(128) k_alpha_weights(int rows, uint32_t N, uint32_t M, float2 *__restrict__ Hh) {
  constexpr int K = 8, CH = 32 * K;
  const int lane = threadIdx.x & 31;
  const int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (r >= rows) return;
  float2 *h = Hh + (size_t)r * M;
  float v = h[0].x;  // 1 (or NaN)
  float cur[K], nxt[K];
  auto load = [&](uint32_t base, float *dst) {
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const uint32_t i = base + (uint32_t)(lane * K + k);
      dst[k] = i < N ? h[i].x : 1.0f;
    }
  };
  load(1, cur);
  for (uint32_t base = 1; base < N; base += CH) {
    if (base + CH < N) load(base + CH, nxt);
    for (int L = 0; L < 32; ++L) {
      if (lane == L) {
#pragma unroll
        for (int k = 0; k < K; ++k) {
          v = v * cur[k];
          cur[k] = v;
        }
      }
      v = __shfl_sync(0xffffffffu, v, L);
    }
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const uint32_t i = base + (uint32_t)(lane * K + k);
      if (i < N) h[i] = make_float2(cur[k], 0.f);
      cur[k] = nxt[k];
    }
  }
}

// H_N, Re/Im H_{N-1}, W_N, Re/Im W_{N-1} of each row, summed in FP64 in a
// fixed order (one block per row).  The twiddle of bin N-1 comes from the
// exact integer phase j (N-1) mod 2N through the float sincospi: its
// ~1e-7 error enters only the top-bin term, itself of order 1/sqrt(N) of
// the samples.
__global__ void __launch_bounds__(kThreads) k_alpha_bins(int rows, uint32_t N, uint32_t M,
                                                         const float2 *__restrict__ A,
                                                         const float2 *__restrict__ Hh, double *__restrict__ bins) {
  const int r = blockIdx.x;
  if (r >= rows) return;
  const float2 *w = A + (size_t)r * M;
  const float2 *h = Hh + (size_t)r * M;
  double acc[6] = {0, 0, 0, 0, 0, 0};
  const uint64_t twoN = 2ull * N;
  for (uint32_t j = threadIdx.x; j < N; j += blockDim.x) {
    const double hj = h[j].x, wj = w[j].x;
    const double sgn = (j & 1u) ? -1.0 : 1.0;
    // e^{-2 pi i j (N-1) / 2N}: the phase j (N-1) mod 2N in integers
    const uint32_t q = (uint32_t)(((uint64_t)j * (uint64_t)(N - 1)) % twoN);
    float sf, cf;
    sincospif(-(float)q / (float)N, &sf, &cf);
    const double s = sf, c = cf;
    acc[0] += hj * sgn;
    acc[1] += hj * c;
    acc[2] += hj * s;
    acc[3] += wj * sgn;
    acc[4] += wj * c;
    acc[5] += wj * s;
  }
  __shared__ double red[6][kThreads];
#pragma unroll
  for (int k = 0; k < 6; ++k) red[k][threadIdx.x] = acc[k];
  __syncthreads();
  for (int stride = kThreads / 2; stride > 0; stride >>= 1) {
    if ((int)threadIdx.x < stride) {
#pragma unroll
      for (int k = 0; k < 6; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + stride];
    }
    __syncthreads();
  }
  if (threadIdx.x < 6) bins[(size_t)r * 8 + threadIdx.x] = red[threadIdx.x][0];
}

// One Stockham pass of radix R over `rows` rows of M points: butterfly j of
// a row takes src[j + r M/R], twiddled by e^{sign 2 pi i r k / (Ns R)}
// (k = j mod Ns), and writes its R-point DFT to dst[(j/Ns) Ns R + k + r Ns]
// (Govindaraju et al., "High performance discrete Fourier transforms on
// graphics processors", SC'08).  Self-sorting: no bit reversal.
template <int R>
__global__ void __launch_bounds__(kThreads) k_fft_pass(const float2 *__restrict__ src, float2 *__restrict__ dst,
                                                       int rows, uint32_t M, uint32_t log2M, uint32_t Ns,
                                                       uint32_t log2NsR, int sign) {
  const uint32_t per = M / R;
  const uint64_t total = (uint64_t)rows * per;
  for (uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t base = (idx / per) << log2M;
    const uint32_t j = (uint32_t)(idx % per);
    const uint32_t k = j & (Ns - 1);
    float2 v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      v[r] = src[base + j + (uint64_t)r * per];
      if (r > 0 && k > 0) {
        // angle = sign 2 pi r k / (Ns R); r k < Ns R <= M <= 2^24 is exact
        // in float, and so is the power-of-two scaling
        float s, c;
        sincospif(ldexpf((float)(r * k), 1 - (int)log2NsR) * (float)sign, &s, &c);
        v[r] = cmul(v[r], make_float2(c, s));
      }
    }
    if constexpr (R == 2) {
      const float2 a = v[0], b = v[1];
      v[0] = cadd(a, b);
      v[1] = csub(a, b);
    } else {
      const float2 t0 = cadd(v[0], v[2]), t1 = csub(v[0], v[2]);
      const float2 t2 = cadd(v[1], v[3]), t3 = csub(v[1], v[3]);
      const float2 it3 = cmuli(t3);  // i t3
      v[0] = cadd(t0, t2);
      v[2] = csub(t0, t2);
      // forward (sign -1): X1 = t1 - i t3, X3 = t1 + i t3; inverse: swapped
      v[1] = sign < 0 ? csub(t1, it3) : cadd(t1, it3);
      v[3] = sign < 0 ? cadd(t1, it3) : csub(t1, it3);
    }
    const uint64_t d = base + (uint64_t)(j / Ns) * Ns * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) dst[d + (uint64_t)r * Ns] = v[r];
  }
}

__global__ void k_cmul_rows(float2 *__restrict__ a, const float2 *__restrict__ b, uint64_t total) {
  for (uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (uint64_t)gridDim.x * blockDim.x)
    a[idx] = cmul(a[idx], b[idx]);
}

// out[n] = c[n] - (-1)^n [H_N W_N + Re(C_{N-1} e^{-i pi n/N})] / 2N, with
// c = Re(inverse FFT) / M.
__global__ void k_alpha_finish(int row0, int rows, uint32_t N, uint32_t M, const float2 *__restrict__ C,
                               const double *__restrict__ bins, float *__restrict__ out) {
  const uint64_t total = (uint64_t)rows * N;
  const float invM = 1.0f / (float)M;  // a power of two: exact
  for (uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (uint64_t)gridDim.x * blockDim.x) {
    const int r = (int)(idx / N);
    const uint32_t n = (uint32_t)(idx % N);
    const double *b = bins + (size_t)r * 8;
    const double cN = b[0] * b[3];
    const double c1re = b[1] * b[4] - b[2] * b[5], c1im = b[1] * b[5] + b[2] * b[4];
    float s, c;
    sincospif(-(float)n / (float)N, &s, &c);
    const double corr = (cN + c1re * (double)c - c1im * (double)s) / (2.0 * (double)N);
    const double cn = (double)(C[(size_t)r * M + n].x * invM);
    // N = 1: bins 0 and N-1 coincide and the reference halves it twice
    const double v = N == 1 ? 0.25 * cn : cn - ((n & 1u) ? -corr : corr);
    out[(size_t)(row0 + r) * N + n] = (float)v;
  }
}

uint32_t fft_size(uint32_t N) {
  uint32_t M = 1;
  while (M < 2u * N - 1u) M <<= 1;
  return M < 2u ? 2u : M;
}

int grid_for(uint64_t work) {
  uint64_t b = (work + kThreads - 1) / kThreads;
  const uint64_t cap = 152ull * 16;  // a grid-stride wave of the GPU
  return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

// In-place (ping-pong) FFT of `rows` rows of M points in *x, with *y as the
// other buffer; on return *x holds the result (the pointers are swapped
// when the pass count is odd).
int fft_rows(float2 **x, float2 **y, int rows, uint32_t M, int sign, cudaStream_t s) {
  uint32_t log2M = 0;
  while ((1u << log2M) < M) ++log2M;
  uint32_t Ns = 1, logNs = 0;
  while (Ns < M) {
    const int R = (M / Ns >= 4) ? 4 : 2;
    const uint32_t logR = R == 4 ? 2 : 1;
    const uint64_t work = (uint64_t)rows * (M / R);
    if (R == 4)
      k_fft_pass<4><<<grid_for(work), kThreads, 0, s>>>(*x, *y, rows, M, log2M, Ns, logNs + logR, sign);
    else
      k_fft_pass<2><<<grid_for(work), kThreads, 0, s>>>(*x, *y, rows, M, log2M, Ns, logNs + logR, sign);
    CMTJ_LAUNCH_CHECK("k_fft_pass");
    float2 *t = *x;
    *x = *y;
    *y = t;
    Ns <<= logR;
    logNs += logR;
  }
  return CMTJ_OK;
}

}  // namespace

extern "C" size_t cmtj_alpha_noise_scratch_bytes(uint32_t n) {
  if (n == 0 || n > CMTJ_ALPHA_MAX_LEN) return 0;
  return (size_t)fft_size(n) * 3 * sizeof(float2) + 8 * sizeof(double);
}

extern "C" int cmtj_alpha_noise_f32(const cmtj_alpha_noise_t *d_specs, int32_t n_buffers, uint32_t n,
                                    const float *d_white, float *d_out, void *d_scratch, size_t scratch_bytes,
                                    void *stream) {
  if (n_buffers < 0) {
    cmtj_set_error("cmtj_alpha_noise_f32: n_buffers %d < 0", n_buffers);
    return CMTJ_ERR_ARG;
  }
  if (n_buffers == 0) return CMTJ_OK;
  if (n == 0 || n > CMTJ_ALPHA_MAX_LEN) {
    cmtj_set_error("cmtj_alpha_noise_f32: buffer length %u outside [1, %u]", n, CMTJ_ALPHA_MAX_LEN);
    return CMTJ_ERR_LIMIT;
  }
  if (!d_specs || !d_out || !d_scratch) {
    cmtj_set_error("cmtj_alpha_noise_f32: null device buffer");
    return CMTJ_ERR_ARG;
  }
  const size_t per_row = cmtj_alpha_noise_scratch_bytes(n);
  const uint32_t M = fft_size(n);
  const size_t chunk = scratch_bytes / per_row;
  if (chunk < 1 || ((uintptr_t)d_scratch & 15u)) {
    cmtj_set_error("cmtj_alpha_noise_f32: scratch of %zu bytes (16-byte aligned) holds no buffer row; one needs %zu",
                   scratch_bytes, per_row);
    return CMTJ_ERR_LIMIT;
  }
  cudaStream_t s = cmtj_stream(stream);
  for (int row0 = 0; row0 < n_buffers; row0 += (int)chunk) {
    const int rows = (int)((size_t)(n_buffers - row0) < chunk ? (size_t)(n_buffers - row0) : chunk);
    float2 *P0 = static_cast<float2 *>(d_scratch);
    float2 *P1 = P0 + (size_t)rows * M;
    float2 *P2 = P1 + (size_t)rows * M;
    double *bins = reinterpret_cast<double *>(P2 + (size_t)rows * M);
    const uint64_t elems = (uint64_t)rows * M;
    k_alpha_fill<<<grid_for(elems), kThreads, 0, s>>>(d_specs, row0, rows, n, M, d_white, P0, P1);
    CMTJ_LAUNCH_CHECK("k_alpha_fill");
    k_alpha_weights<<<(rows + 3) / 4, 128, 0, s>>>(rows, n, M, P1);
    CMTJ_LAUNCH_CHECK("k_alpha_weights");
    k_alpha_bins<<<rows, kThreads, 0, s>>>(rows, n, M, P0, P1, bins);
    CMTJ_LAUNCH_CHECK("k_alpha_bins");
    // W = FFT(w) with P2 as the other buffer, then H = FFT(h) with whichever
    // of P0 / P2 does not hold W
    float2 *w = P0, *other = P2;
    int rc = fft_rows(&w, &other, rows, M, -1, s);
    if (rc != CMTJ_OK) return rc;
    float2 *h = P1;
    rc = fft_rows(&h, &other, rows, M, -1, s);
    if (rc != CMTJ_OK) return rc;
    k_cmul_rows<<<grid_for(elems), kThreads, 0, s>>>(w, h, elems);
    CMTJ_LAUNCH_CHECK("k_cmul_rows");
    // inverse (unnormalised); `h` is free now
    rc = fft_rows(&w, &h, rows, M, +1, s);
    if (rc != CMTJ_OK) return rc;
    k_alpha_finish<<<grid_for((uint64_t)rows * n), kThreads, 0, s>>>(row0, rows, n, M, w, bins, d_out);
    CMTJ_LAUNCH_CHECK("k_alpha_finish");
  }
  return CMTJ_OK;
}
