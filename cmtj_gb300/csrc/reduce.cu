// On-device reductions of batched logs.
//
// cmtj_spectrum_f32 replaces the per-junction numpy/scipy post-processing of
// PIMM_procedure (cmtj/utils/procedures.py:28-39, compute_spectrum_strip:
// |scipy.fft.fft(m)| truncated to a frequency range).  The row is real, so
// its n-point spectrum comes from an n/2-point complex FFT of (even, odd)
// sample pairs and one unpacking pass over the kept bins.  The complex FFT
// is a Stockham FFT (self-sorting, no bit reversal) in radix-8 stages, with
// a final radix-4 or radix-2 stage when log2(n/2) is not a multiple of 3.
//
// The kernel is instantiated per FFT size, so every index, stride and
// shift is a compile-time constant.  CTAs of n/16 threads are persistent:
// each builds the twiddle table of every stage in shared memory once
// (entry (r-1) NS + k of a stage holds e^{-2 pi i k r/(NS R)}, so a warp's
// lanes read consecutive entries) and then transforms rows blockIdx.x,
// blockIdx.x + gridDim.x, ...  Every thread keeps 8 points in registers
// through a stage; stages exchange through one shared buffer of float2
// points with one point of padding after every 16 (no bank conflicts on
// the loads, few on the strided stores).  The first stage reads the row
// straight from HBM (coalesced, any alignment); the last pass writes |X[k]|
// for k in [bin_lo, bin_hi).  (Prefetching the next row into shared memory
// with cp.async was slower: the staging buffer cost a resident CTA per SM.)
#include <utility>

#include "common.cuh"

namespace {

constexpr int kMaxFft = 8192;

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
// multiplication by -i (forward-transform rotation)
__device__ __forceinline__ float2 mul_mi(float2 a) { return make_float2(a.y, -a.x); }

// In-register DFTs of size 2, 4, 8 (forward, e^{-2 pi i jk/R}).
__device__ __forceinline__ void dft2(float2 &a, float2 &b) {
  const float2 t = a;
  a = cadd(t, b);
  b = csub(t, b);
}
__device__ __forceinline__ void dft4(float2 *v) {
  float2 a0 = v[0], a1 = v[1], a2 = v[2], a3 = v[3];
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
__device__ __forceinline__ void dft8(float2 *v) {
  const float h = 0.70710678118654752f;
  float2 e[4] = {v[0], v[2], v[4], v[6]}, o[4] = {v[1], v[3], v[5], v[7]};
  dft4(e);
  dft4(o);
  // o[k] *= e^{-2 pi i k/8}
  o[1] = make_float2(h * (o[1].x + o[1].y), h * (o[1].y - o[1].x));
  o[2] = mul_mi(o[2]);
  o[3] = make_float2(h * (o[3].y - o[3].x), -h * (o[3].x + o[3].y));
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    v[k] = cadd(e[k], o[k]);
    v[k + 4] = csub(e[k], o[k]);
  }
}
template <int R>
__device__ __forceinline__ void dft(float2 *v) {
  if constexpr (R == 8) dft8(v);
  else if constexpr (R == 4) dft4(v);
  else dft2(v[0], v[1]);
}

// Shared slot of complex point i: one float2 of padding after every 16.
__device__ __forceinline__ int pad(int i) { return i + (i >> 4); }
// Slot of point a + c, given pa = pad(a): for c a multiple of 16 it is
// pa + c + c/16 (no carry reaches the low four bits).
template <int C>
__device__ __forceinline__ int slot_plus(int pa, int a) {
  if constexpr (C % 16 == 0) return pa + C + C / 16;
  else return pad(a + C);
}

// Offset of the twiddle table of the stage with NS = 2^NSL: the tables of
// the earlier stages hold (R - 1) NS entries each.
template <int L>
__host__ __device__ constexpr int table_offset(int NSL) {
  int off = 0;
  for (int nsl = 3; nsl < NSL;) {
    const int lr = L - nsl >= 3 ? 3 : L - nsl;
    off += ((1 << lr) - 1) << nsl;
    nsl += lr;
  }
  return off;
}

// Sizes of the 2^(L+1)-point real transform: H complex points, T threads;
// shared memory = the padded points and the stages' twiddle tables.
template <int L>
struct Fft {
  static constexpr int H = 1 << L;
  static constexpr int N = 2 * H;
  static constexpr int T = H / 8;
  static constexpr int SLOTS = H + H / 16;
  static constexpr int TABLE = table_offset<L>(L);
  static constexpr size_t kSmem = (size_t)(SLOTS + TABLE) * sizeof(float2);
};

// Fills the table of every stage after the first: entry (r - 1) NS + k of
// the stage with NS = 2^NSL and radix R is e^{-2 pi i k r / (NS R)}.
template <int L, int NSL>
__device__ __forceinline__ void build_tables(float2 *tab) {
  if constexpr (NSL < L) {
    constexpr int LR = (L - NSL) >= 3 ? 3 : (L - NSL);
    constexpr int R = 1 << LR, NS = 1 << NSL, OFF = table_offset<L>(NSL);
    for (int idx = threadIdx.x; idx < (R - 1) * NS; idx += Fft<L>::T) {
      const int r = (idx >> NSL) + 1, k = idx & (NS - 1);
      float sn, cs;
      sincospif(-2.0f * (float)(k * r) / (float)(NS * R), &sn, &cs);
      tab[OFF + idx] = make_float2(cs, sn);
    }
    build_tables<L, NSL + LR>(tab);
  }
}

// Unrolled over r = 0..R-1: f(r) with r a compile-time constant.
template <int R, class F, int... I>
__device__ __forceinline__ void each_r(F &&f, std::integer_sequence<int, I...>) {
  (f(std::integral_constant<int, I>{}), ...);
}

// One Stockham stage of radix R = 2^LR after the first (NS = 2^NSL points
// per already-transformed block), in place in buf.  Group g = q T + t
// (G = 8/R per thread, so a warp's lanes take consecutive groups) reads
// point g + r H/R, twiddles it by e^{-2 pi i k r/(NS R)} (k = g mod NS,
// from the stage's table, consecutive k in consecutive slots) and writes
// point (g/NS) NS R + k + r NS.
template <int L, int LR, int NSL>
__device__ __forceinline__ void stage(float2 *buf, const float2 *tab) {
  constexpr int R = 1 << LR, G = 8 / R, NS = 1 << NSL, STRIDE = Fft<L>::H / R;
  const float2 *tw = tab + table_offset<L>(NSL);
  float2 v[G][R];
#pragma unroll
  for (int q = 0; q < G; ++q) {
    const int g = q * Fft<L>::T + threadIdx.x;
    const int pg = pad(g);
    each_r<R>([&](auto r) { v[q][decltype(r)::value] = buf[slot_plus<decltype(r)::value * STRIDE>(pg, g)]; },
              std::make_integer_sequence<int, R>{});
    const int k = g & (NS - 1);
#pragma unroll
    for (int r = 1; r < R; ++r) v[q][r] = cmul(v[q][r], tw[(r - 1) * NS + k]);
    dft<R>(v[q]);
  }
  __syncthreads();  // everyone has read the points before anyone overwrites them
#pragma unroll
  for (int q = 0; q < G; ++q) {
    const int g = q * Fft<L>::T + threadIdx.x;
    const int base = ((g >> NSL) << (NSL + LR)) + (g & (NS - 1));
    const int pb = pad(base);
    each_r<R>([&](auto r) { buf[slot_plus<decltype(r)::value * NS>(pb, base)] = v[q][decltype(r)::value]; },
              std::make_integer_sequence<int, R>{});
  }
  __syncthreads();
}

// The stages after the first, NSL = log2 of the transformed block size.
template <int L, int NSL>
__device__ __forceinline__ void stages(float2 *buf, const float2 *tab) {
  if constexpr (NSL < L) {
    constexpr int LR = (L - NSL) >= 3 ? 3 : (L - NSL);
    stage<L, LR, NSL>(buf, tab);
    stages<L, NSL + LR>(buf, tab);
  }
}

// |X[k]| of a real row x of n points, from the n/2-point complex FFT Z of
// z[m] = x[2m] + i x[2m+1]:  with E = FFT(x even), O = FFT(x odd),
// E[k] = (Z[k] + conj Z[h-k]) / 2, O[k] = (Z[k] - conj Z[h-k]) / 2i and
// X[k] = E[k] + W_n^k O[k] (h = n/2, indices mod h); bins above n/2 use
// |X[k]| = |X[n-k]|.
template <int L>
__global__ void __launch_bounds__(Fft<L>::T) k_spectrum(const float *__restrict__ series, int64_t row_stride,
                                                       int32_t series_len, int32_t n_rows, int32_t bin_lo,
                                                       int32_t bin_hi, float *__restrict__ out) {
  constexpr int H = Fft<L>::H, N = Fft<L>::N, T = Fft<L>::T;
  extern __shared__ __align__(16) float2 smem2[];
  float2 *buf = smem2;
  float2 *tab = smem2 + Fft<L>::SLOTS;
  build_tables<L, 3>(tab);
  // (the first row's barriers order the tables before any use)
  const int nb = bin_hi - bin_lo;
  for (int64_t row = blockIdx.x; row < n_rows; row += gridDim.x) {
    // first stage, radix 8, from HBM: point m of z is (x[2m], x[2m+1])
    float2 v[8];
    {
      const float *src = series + row * row_stride + (series_len - N);
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        const int idx = threadIdx.x + r * (H / 8);
        v[r] = make_float2(__ldg(src + 2 * idx), __ldg(src + 2 * idx + 1));
      }
    }
    dft8(v);
    __syncthreads();  // the previous row's last pass has read buf
    {
      // point 8t + r (r < 8) shares the 16-point block of 8t: slot 8t + t/2 + r
      const int s0 = 8 * threadIdx.x + (threadIdx.x >> 1);
#pragma unroll
      for (int r = 0; r < 8; ++r) buf[s0 + r] = v[r];
    }
    __syncthreads();
    stages<L, 3>(buf, tab);
    float *dst = out + row * (int64_t)nb;
    for (int kk = threadIdx.x; kk < nb; kk += T) {
      int q = bin_lo + kk;
      if (q > H) q = N - q;
      const int a = q == H ? 0 : q;
      const int b = q == 0 ? 0 : H - q;
      const float2 zk = buf[pad(a)];
      const float2 zb = buf[pad(b)];
      const float2 zc = make_float2(zb.x, -zb.y);
      const float2 e = make_float2(0.5f * (zk.x + zc.x), 0.5f * (zk.y + zc.y));
      const float2 o = make_float2(0.5f * (zk.y - zc.y), -0.5f * (zk.x - zc.x));
      float sn, cs;
      sincospif(-2.0f * (float)q / (float)N, &sn, &cs);
      const float2 x = cadd(e, cmul(make_float2(cs, sn), o));
      dst[kk] = sqrtf(fmaf(x.x, x.x, x.y * x.y));
    }
  }
}

template <int L>
cudaError_t launch_spectrum(const float *d_series, int64_t row_stride, int32_t n_rows, int32_t series_len,
                            int32_t bin_lo, int32_t bin_hi, float *d_out, cudaStream_t stream) {
  constexpr size_t smem = Fft<L>::kSmem;
  cudaError_t e = cudaSuccess;
  if (smem > 48 * 1024) {
    e = cudaFuncSetAttribute(k_spectrum<L>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  int dev = 0, sms = 0, per_sm = 0;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
  if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
  if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_spectrum<L>, Fft<L>::T, smem)) != cudaSuccess)
    return e;
  const int64_t resident = (int64_t)sms * (per_sm > 0 ? per_sm : 1);
  const int grid = (int)(n_rows < resident ? n_rows : resident);
  k_spectrum<L><<<grid, Fft<L>::T, smem, stream>>>(d_series, row_stride, series_len, n_rows, bin_lo, bin_hi, d_out);
  return cudaGetLastError();
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
  const cudaStream_t s = cmtj_stream(stream);
  cudaError_t e = cudaSuccess;
  switch (log2n) {
    case 6: e = launch_spectrum<5>(d_series, row_stride, n_rows, series_len, bin_lo, bin_hi, d_out, s); break;
    case 7: e = launch_spectrum<6>(d_series, row_stride, n_rows, series_len, bin_lo, bin_hi, d_out, s); break;
    case 8: e = launch_spectrum<7>(d_series, row_stride, n_rows, series_len, bin_lo, bin_hi, d_out, s); break;
    case 9: e = launch_spectrum<8>(d_series, row_stride, n_rows, series_len, bin_lo, bin_hi, d_out, s); break;
    case 10: e = launch_spectrum<9>(d_series, row_stride, n_rows, series_len, bin_lo, bin_hi, d_out, s); break;
    case 11: e = launch_spectrum<10>(d_series, row_stride, n_rows, series_len, bin_lo, bin_hi, d_out, s); break;
    case 12: e = launch_spectrum<11>(d_series, row_stride, n_rows, series_len, bin_lo, bin_hi, d_out, s); break;
    default: e = launch_spectrum<12>(d_series, row_stride, n_rows, series_len, bin_lo, bin_hi, d_out, s); break;
  }
  if (e != cudaSuccess) {
    cmtj_set_error("launch of k_spectrum failed: %s", cudaGetErrorString(e));
    return CMTJ_ERR_CUDA;
  }
  return CMTJ_OK;
}
