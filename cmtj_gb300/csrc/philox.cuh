// Philox4x32-10 counter-based generator (Salmon, Moraes, Dror, Shaw,
// "Parallel random numbers: as easy as 1, 2, 3", SC'11) and the thermal-field
// Gaussian draws built on it.
//
// Stream definition (shared by every solver form, so FP32 and FP64 runs see
// the same noise up to the FP32 transform's error): for a layer with key
// (seed_lo, seed_hi) at absolute step s, one Philox block with counter
// {s_lo, s_hi, 0x7E4D, 0} gives four words w0..w3; u_k = (w_k + 0.5) * 2^-32
// lies in (0, 1); the Box-Muller transform gives g0, g1 from (u0, u1) and g2
// from (u2, u3).
#pragma once
#include <stdint.h>

#define CMTJ_PHILOX_M0 0xD2511F53u
#define CMTJ_PHILOX_M1 0xCD9E8D57u
#define CMTJ_PHILOX_W0 0x9E3779B9u
#define CMTJ_PHILOX_W1 0xBB67AE85u
#define CMTJ_THERMAL_TAG 0x7E4Du

__device__ __forceinline__ uint4 cmtj_philox4x32_10(uint4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint32_t hi0 = __umulhi(CMTJ_PHILOX_M0, c.x), lo0 = CMTJ_PHILOX_M0 * c.x;
    const uint32_t hi1 = __umulhi(CMTJ_PHILOX_M1, c.z), lo1 = CMTJ_PHILOX_M1 * c.z;
    c = make_uint4(hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0);
    k0 += CMTJ_PHILOX_W0;
    k1 += CMTJ_PHILOX_W1;
  }
  return c;
}

__device__ __forceinline__ uint4 cmtj_thermal_words(uint32_t seed_lo, uint32_t seed_hi, uint64_t step) {
  return cmtj_philox4x32_10(make_uint4((uint32_t)step, (uint32_t)(step >> 32), CMTJ_THERMAL_TAG, 0u),
                            seed_lo, seed_hi);
}

// The white draws of a layer's buffered 1/f^alpha noise: the same key and
// transform as the thermal draws, with counter {i_lo, i_hi, 0xA1F4, 0} for
// draw i, an independent stream.
#define CMTJ_ALPHA_TAG 0xA1F4u

// FP64 Box-Muller of one Philox block (plain form).
__device__ __forceinline__ void cmtj_gaussian3_of_words(uint4 w, double &g0, double &g1, double &g2) {
  const double s = 2.3283064365386963e-10;  // 2^-32
  const double u0 = ((double)w.x + 0.5) * s, u1 = ((double)w.y + 0.5) * s;
  const double u2 = ((double)w.z + 0.5) * s, u3 = ((double)w.w + 0.5) * s;
  const double r0 = sqrt(-2.0 * log(u0)), r1 = sqrt(-2.0 * log(u2));
  const double a0 = 6.283185307179586 * u1, a1 = 6.283185307179586 * u3;
  g0 = r0 * cos(a0);
  g1 = r0 * sin(a0);
  g2 = r1 * cos(a1);
}

// FP64 thermal draws (plain form).
__device__ __forceinline__ void cmtj_gaussian3_f64(uint32_t seed_lo, uint32_t seed_hi, uint64_t step,
                                                   double &g0, double &g1, double &g2) {
  cmtj_gaussian3_of_words(cmtj_thermal_words(seed_lo, seed_hi, step), g0, g1, g2);
}

// Normal `c` (0, 1 or 2) of the alpha-noise stream's draw i alone: the
// same operations as that component of cmtj_alpha_gaussian3_f64, so the
// same bits, without the other two transcendental chains.
__device__ __forceinline__ double cmtj_alpha_gaussian_f64(uint32_t seed_lo, uint32_t seed_hi, uint64_t i, int c) {
  const uint4 w =
      cmtj_philox4x32_10(make_uint4((uint32_t)i, (uint32_t)(i >> 32), CMTJ_ALPHA_TAG, 0u), seed_lo, seed_hi);
  const double s = 2.3283064365386963e-10;  // 2^-32
  if (c < 2) {
    const double u0 = ((double)w.x + 0.5) * s, u1 = ((double)w.y + 0.5) * s;
    const double r0 = sqrt(-2.0 * log(u0));
    const double a0 = 6.283185307179586 * u1;
    return c == 0 ? r0 * cos(a0) : r0 * sin(a0);
  }
  const double u2 = ((double)w.z + 0.5) * s, u3 = ((double)w.w + 0.5) * s;
  const double r1 = sqrt(-2.0 * log(u2));
  const double a1 = 6.283185307179586 * u3;
  return r1 * cos(a1);
}

// FP64 white draws of the buffered alpha noise.
__device__ __forceinline__ void cmtj_alpha_gaussian3_f64(uint32_t seed_lo, uint32_t seed_hi, uint64_t i,
                                                         double &g0, double &g1, double &g2) {
  cmtj_gaussian3_of_words(
      cmtj_philox4x32_10(make_uint4((uint32_t)i, (uint32_t)(i >> 32), CMTJ_ALPHA_TAG, 0u), seed_lo, seed_hi), g0, g1,
      g2);
}

// FP32 draws (batched form): the same words, transformed in single
// precision with the hardware approximations (the draws only have to be
// right in distribution; they agree with the FP64 draws to a few 1e-6).
// The radius uniforms keep 32 bits, (w + 0.5) 2^-32 (tails to 6.8 sigma).
// The angle uniform comes from the top 23 bits as v = u - 1/2 in
// [-1/2, 1/2), where the hardware sine and cosine are most accurate; the
// angle 2 pi v is the FP64 angle minus pi, so the products are negated to
// give the FP64 draws' signs.  __logf has a small absolute error near u = 1
// that can make -2 log(u) slightly negative; the radius is 0 there.
__device__ __forceinline__ float cmtj_bm_radius(uint32_t w) {
  const float u = ((float)w + 0.5f) * 2.3283064365386963e-10f;
  const float x = -2.0f * __logf(u);
  return x > 0.f ? x * rsqrtf(x) : 0.f;
}
__device__ __forceinline__ float cmtj_bm_angle(uint32_t w) {
  return 6.2831853f * (__uint_as_float(0x3f800000u | (w >> 9)) - 1.5f);
}
__device__ __forceinline__ void cmtj_gaussian3_f32(uint32_t seed_lo, uint32_t seed_hi, uint64_t step,
                                                   float &g0, float &g1, float &g2) {
  const uint4 w = cmtj_thermal_words(seed_lo, seed_hi, step);
  const float r0 = cmtj_bm_radius(w.x), r1 = cmtj_bm_radius(w.z);
  float s0, c0;
  __sincosf(cmtj_bm_angle(w.y), &s0, &c0);
  g0 = -r0 * c0;
  g1 = -r0 * s0;
  g2 = -r1 * __cosf(cmtj_bm_angle(w.w));
}
