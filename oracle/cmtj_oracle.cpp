// cmtj_oracle.cpp -- CPU restatement of the reference macrospin time loop.
//
// TEST INFRASTRUCTURE ONLY.  This file is the oracle: the tests, the smoke
// check and the CPU-baseline leg of bench.py call it to check (and time) the
// GPU solver.  The product (cmtj_gb300 and libcmtj_gpu.so) never links,
// loads or calls it.
//
// It restates, in plain FP64 C++ with no FMA contraction (build with
// -ffp-contract=off), the arithmetic of LemurPwned/cmtj:
//   core/drivers.hpp:73-108, 262-305   ScalarDriver::getCurrentScalarValue
//   core/cvector.hpp:179-192           CVector length / normalize
//   core/junction.hpp:54-72            calculate_tensor_interaction
//   core/junction.hpp:580-701          calculateHeff and its field terms
//   core/junction.hpp:716-831          solveLLG (LLG + STT + SOT), stochasticTorque
//   core/junction.hpp:866-1002         Layer::dormand_prince_step
//   core/junction.hpp:1017-1041        Layer::rk4_step
//   core/junction.hpp:1111-1136        thermal field standard deviation, getOneFVector
//   core/noise.hpp:160-225, 280-290    BufferedAlphaNoise::fillBuffer, VectorAlphaNoise::tickVector
//   core/junction.hpp:1580-1636        logLayerParams
//   core/junction.hpp:1668-1815        runners (single/multi layer, Euler-Heun, Heun)
//   core/junction.hpp:1835-1867        strip / classic magnetoresistance
//   core/junction.hpp:1948-1981        runSimulation fixed-step loop
//   core/junction.hpp:1982-2045        runSimulation Dormand-Prince loop
//   core/reservoir.hpp:61-151, 185-230 GroupInteraction (dipole-coupled groups)
// keeping the reference's expression order so that deterministic runs are
// bit-identical to the reference build (checked by tests/test_oracle_pin.py).
//
// The thermal field uses Philox4x32-10 (Salmon et al., SC'11) and the
// Box-Muller transform instead of the reference's unseeded std::mt19937, so
// thermal runs are reproducible; against the reference they agree in
// statistics only.
//
// The scalar type is a template parameter so that the same code, run on a
// counting type, yields the FLOP count per layer-step used for the roofline.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>
#include <algorithm>
#include <atomic>
#include <complex>

#include "../include/cmtj_gpu.h"

namespace oracle {
using std::cos;
using std::erf;
using std::exp;
using std::fabs;
using std::log;
using std::pow;
using std::sin;
using std::sqrt;

// ---------------------------------------------------------------- vectors
template <typename T> struct V3 {
  T x, y, z;
  V3() : x(0.0), y(0.0), z(0.0) {}
  V3(T a, T b, T c) : x(a), y(b), z(c) {}
  V3 operator+(const V3 &v) const { return V3(x + v.x, y + v.y, z + v.z); }
  V3 operator-(const V3 &v) const { return V3(x - v.x, y - v.y, z - v.z); }
  V3 operator*(const T &s) const { return V3(x * s, y * s, z * s); }
  V3 operator/(const T &s) const { return V3(x / s, y / s, z / s); }
};
template <typename T> V3<T> smul(const T &s, const V3<T> &v) { return V3<T>(s * v.x, s * v.y, s * v.z); }
template <typename T> T dot(const V3<T> &a, const V3<T> &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <typename T> V3<T> cross(const V3<T> &a, const V3<T> &b) {
  return V3<T>(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
template <typename T> T sq(const T &a) { return a * a; }  // pow(a, 2): GCC folds it to a*a
template <typename T> V3<T> normalized(const V3<T> &v) {
  const T mag = sqrt(sq(v.x) + sq(v.y) + sq(v.z));
  if (mag != 0) return V3<T>(v.x / mag, v.y / mag, v.z / mag);
  return v;
}
template <typename T> V3<T> tensor_mul(const V3<T> &m, const double *t, const T &Ms, const T &mu0) {
  V3<T> r(t[0] * m.x + t[1] * m.y + t[2] * m.z, t[3] * m.x + t[4] * m.y + t[5] * m.z,
          t[6] * m.x + t[7] * m.y + t[8] * m.z);
  return r * (Ms / mu0);
}
template <typename T> V3<T> v3(const double *p) { return V3<T>(p[0], p[1], p[2]); }

// ---------------------------------------------------------------- drivers
// drivers.hpp:262-305; table drivers hold host-sampled custom callbacks.
template <typename T> struct Tables {
  const double *data = nullptr;
  uint32_t step = 0;   // current iteration (table row)
  int stage = 0;       // 0: t, 1: t + dt/2, 2: t + dt
};

template <typename T> T driver_value(const cmtj_driver_t &d, const T &time, const Tables<T> &tb) {
  T rv = d.constantValue;
  switch (d.update) {
  case CMTJ_DRV_CONSTANT: break;
  case CMTJ_DRV_PULSE: {
    const int n = (int)(double)(time / d.period);
    const T dT = d.cycle * d.period;
    const T nT = n * d.period;
    if (nT <= time && time <= (nT + dT)) rv = rv + d.amplitude;
    break;
  }
  case CMTJ_DRV_SINE: rv = rv + d.amplitude * sin(2 * M_PI * time * d.frequency + d.phase); break;
  case CMTJ_DRV_POSINE: rv = rv + fabs(d.amplitude * sin(2 * M_PI * time * d.frequency + d.phase)); break;
  case CMTJ_DRV_HALFSINE: {
    const T tamp = d.amplitude * sin(2 * M_PI * time * d.frequency + d.phase);
    if (tamp <= 0) rv = rv + tamp;
    break;
  }
  case CMTJ_DRV_STEP:
    if (time >= d.timeStart && time <= d.timeStop) rv = rv + d.amplitude;
    break;
  case CMTJ_DRV_TRAPEZOID: {
    const double ts = d.timeStart, e = d.edgeTime, s = d.steadyTime, a = d.amplitude;
    T add = 0.0;
    if (time < ts) add = 0.0;
    else if (time <= ts + e) add = (a / e) * (time - ts);
    else if (time <= ts + e + s) add = a;
    else if (time <= ts + 2 * e + s) add = a - (a / e) * (time - (ts + e + s));
    rv = rv + add;
    break;
  }
  case CMTJ_DRV_GAUSSIMPULSE:
    rv = rv + d.amplitude * exp(-sq(time - d.timeStart) / (2 * sq(T(d.edgeTime))));
    break;
  case CMTJ_DRV_GAUSSSTEP:
    rv = rv + 0.5 * d.amplitude * (1 + erf((time - d.timeStart) / (sqrt(2.0) * d.edgeTime)));
    break;
  case CMTJ_DRV_TABLE:
    return tb.data[d.table_offset + (int64_t)tb.step * 3 + tb.stage];
  default: break;
  }
  return rv;
}

// ---------------------------------------------------------------- philox
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), counter-based.
struct U4 { uint32_t v[4]; };
inline U4 philox4x32_10(U4 c, uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = (uint64_t)M0 * c.v[0];
    const uint64_t p1 = (uint64_t)M1 * c.v[2];
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    U4 n;
    n.v[0] = hi1 ^ c.v[1] ^ k0;
    n.v[1] = lo1;
    n.v[2] = hi0 ^ c.v[3] ^ k1;
    n.v[3] = lo0;
    c = n;
    k0 += W0;
    k1 += W1;
  }
  return c;
}
// Three N(0,1) draws of one layer at one step: Box-Muller on the four
// 32-bit words, u = (w + 0.5) / 2^32 in (0, 1).  The counter's third word
// tags the stream: 0x7E4D the thermal field, 0xA1F4 the white draws of the
// buffered alpha noise.
inline void gaussian3_tag(uint32_t tag, uint32_t seed_lo, uint32_t seed_hi, uint64_t step, double g[3]) {
  U4 c;
  c.v[0] = (uint32_t)step;
  c.v[1] = (uint32_t)(step >> 32);
  c.v[2] = tag;
  c.v[3] = 0u;
  const U4 w = philox4x32_10(c, seed_lo, seed_hi);
  const double s = 2.3283064365386963e-10;  // 2^-32
  const double u0 = ((double)w.v[0] + 0.5) * s, u1 = ((double)w.v[1] + 0.5) * s;
  const double u2 = ((double)w.v[2] + 0.5) * s, u3 = ((double)w.v[3] + 0.5) * s;
  const double r0 = sqrt(-2.0 * log(u0)), r1 = sqrt(-2.0 * log(u2));
  const double a0 = 6.283185307179586 * u1, a1 = 6.283185307179586 * u3;
  g[0] = r0 * cos(a0);
  g[1] = r0 * sin(a0);
  g[2] = r1 * cos(a1);
}
inline void gaussian3(uint32_t seed_lo, uint32_t seed_hi, uint64_t step, double g[3]) {
  gaussian3_tag(0x7E4Du, seed_lo, seed_hi, step, g);
}

// ------------------------------------------------------ buffered alpha noise
// Iterative radix-2 complex FFT in FP64 (size a power of two); sign -1
// forward, +1 inverse (unnormalised).
inline void fft_pow2(std::vector<std::complex<double>> &a, int sign) {
  const size_t n = a.size();
  for (size_t i = 1, j = 0; i < n; ++i) {
    size_t bit = n >> 1;
    for (; j & bit; bit >>= 1) j ^= bit;
    j ^= bit;
    if (i < j) std::swap(a[i], a[j]);
  }
  for (size_t len = 2; len <= n; len <<= 1) {
    const double ang = sign * 2.0 * M_PI / (double)len;
    for (size_t i = 0; i < n; i += len) {
      for (size_t k = 0; k < len / 2; ++k) {
        const std::complex<double> w(std::cos(ang * (double)k), std::sin(ang * (double)k));
        const std::complex<double> u = a[i + k], v = a[i + k + len / 2] * w;
        a[i + k] = u + v;
        a[i + k + len / 2] = u - v;
      }
    }
  }
}

// BufferedAlphaNoise::fillBuffer (noise.hpp:186-225) of one buffer of n
// samples.  White draws: `white` when given, else std times normal
// `component` of the alpha-noise Philox stream at counter + m (the
// reference: std::normal_distribution<float>(0, std) on mt19937).  Filter
// weights: the reference's float recurrence (171-176).  The reference
// multiplies the 2n-point spectra of the zero-padded white and weight rows
// in bins [0, n), halves bins 0 and n-1, drops bins [n, 2n), and keeps
// Re(inverse)[m] / n.  With C = H W the 2n-point spectrum of the linear
// convolution c = h * w, that is c[m] - (C_n (-1)^m + Re(C_{n-1}
// e^{i pi (n-1) m / n})) / 2n for n >= 2 (bins 0 and n-1 distinct) and C_0 / 4
// for n = 1 (the one bin halved twice).  c comes from a power-of-two FFT
// convolution, the two bins from direct sums, all in FP64.
inline void alpha_fill(const cmtj_alpha_noise_t &sp, uint32_t n, const float *white, float *out) {
  std::vector<float> w(n), h(n);
  for (uint32_t m = 0; m < n; ++m) {
    if (white) {
      w[m] = white[m];
    } else {
      double g[3];
      gaussian3_tag(0xA1F4u, sp.seed_lo, sp.seed_hi, sp.counter + m, g);
      const int c = sp.component < 0 ? 0 : (sp.component > 2 ? 2 : sp.component);
      w[m] = (float)(sp.std * g[c]);
    }
  }
  float v = (sp.alpha >= 0.0 && sp.alpha <= 2.0) ? 1.0f : NAN;
  h[0] = v;
  for (uint32_t i = 1; i < n; ++i) {
    const float weight = (float)(0.5 * sp.alpha + (double)(float)(i - 1)) / (float)i;
    v = v * weight;
    h[i] = v;
  }
  size_t M = 2;
  while (M < 2 * (size_t)n - 1) M <<= 1;
  std::vector<std::complex<double>> A(M), B(M);
  for (uint32_t m = 0; m < n; ++m) {
    A[m] = w[m];
    B[m] = h[m];
  }
  fft_pow2(A, -1);
  fft_pow2(B, -1);
  for (size_t k = 0; k < M; ++k) A[k] *= B[k];
  fft_pow2(A, +1);
  if (n == 1) {
    out[0] = (float)(0.25 * A[0].real() / (double)M);
    return;
  }
  // the 2n-point bins n and n-1 of h and w
  double hN = 0, wN = 0;
  std::complex<double> h1(0, 0), w1(0, 0);
  for (uint32_t j = 0; j < n; ++j) {
    const double sg = (j & 1u) ? -1.0 : 1.0;
    hN += h[j] * sg;
    wN += w[j] * sg;
    const uint64_t q = ((uint64_t)j * (uint64_t)(n - 1)) % (2ull * n);
    const std::complex<double> e(std::cos(M_PI * (double)q / (double)n), -std::sin(M_PI * (double)q / (double)n));
    h1 += (double)h[j] * e;
    w1 += (double)w[j] * e;
  }
  const double cN = hN * wN;
  const std::complex<double> c1 = h1 * w1;
  for (uint32_t m = 0; m < n; ++m) {
    const uint64_t q = ((uint64_t)m * (uint64_t)(n - 1)) % (2ull * n);
    const std::complex<double> e(std::cos(M_PI * (double)q / (double)n), std::sin(M_PI * (double)q / (double)n));
    const double corr = (cN * ((m & 1u) ? -1.0 : 1.0) + (c1 * e).real()) / (2.0 * (double)n);
    out[m] = (float)(A[m].real() / (double)M - corr);
  }
}

// ---------------------------------------------------------------- physics
template <typename T> struct Side {  // side effects logged with calculateEnergies
  T K = 0.0, K2 = 0.0, Jb = 0.0, Jt = 0.0, I = 0.0;
  V3<T> Hext, Hiec, Hanis, Hdemag, Hfl, Hdl;
};

template <typename T> struct Ctx {
  const cmtj_layer_t *L;
  const cmtj_constants_t *c;
  Tables<T> tb;
  Side<T> *side;
};

template <typename T> V3<T> axial(const cmtj_layer_t &L, int slot, const T &t, const Tables<T> &tb) {
  return V3<T>(driver_value<T>(L.drv[slot], t, tb), driver_value<T>(L.drv[slot + 1], t, tb),
               driver_value<T>(L.drv[slot + 2], t, tb));
}

// calculateHeff (junction.hpp:580-622).
template <typename T>
V3<T> heff(Ctx<T> &cx, const T &time, const V3<T> &m, const V3<T> &bottom, const V3<T> &top) {
  const cmtj_layer_t &L = *cx.L;
  const T mu0 = cx.c->mu0;
  const T Ms = L.Ms;
  const V3<T> Hdipole = tensor_mul<T>(bottom, L.dipole_bottom, Ms, mu0) + tensor_mul<T>(top, L.dipole_top, Ms, mu0);
  const V3<T> Hext = axial<T>(L, CMTJ_SLOT_HEXT, time, cx.tb);
  const V3<T> Hoe = axial<T>(L, CMTJ_SLOT_HOE, time, cx.tb);
  const V3<T> Hdemag = tensor_mul<T>(m, L.demag, Ms, mu0);
  // calculateIEC (654-675)
  const T Jb = driver_value<T>(L.drv[CMTJ_SLOT_IEC_BOTTOM], time, cx.tb);
  const T Jt = driver_value<T>(L.drv[CMTJ_SLOT_IEC_TOP], time, cx.tb);
  const T J2b = driver_value<T>(L.drv[CMTJ_SLOT_IECQ_BOTTOM], time, cx.tb);
  const T J2t = driver_value<T>(L.drv[CMTJ_SLOT_IECQ_TOP], time, cx.tb);
  const T Mst = Ms * T(L.thickness);
  const V3<T> Hiec = (bottom * (Jb + 2 * J2b * dot(bottom, m))) / Mst + (top * (Jt + 2 * J2t * dot(top, m))) / Mst;
  // calculateIDMI (677-701)
  const V3<T> Db = axial<T>(L, CMTJ_SLOT_IDMI_BOTTOM, time, cx.tb);
  const V3<T> Dt = axial<T>(L, CMTJ_SLOT_IDMI_TOP, time, cx.tb);
  const V3<T> Hidmi = smul<T>(-1.0, cross(Db, bottom)) / Mst + smul<T>(-1.0, cross(Dt, top)) / Mst;
  // calculateAnisotropy (638-643)
  const V3<T> anis = v3<T>(L.anis);
  const T K = driver_value<T>(L.drv[CMTJ_SLOT_ANIS], time, cx.tb);
  const V3<T> Hanis = anis * ((2 * K) * dot(anis, m) / Ms);
  const V3<T> Hdmi = axial<T>(L, CMTJ_SLOT_HDMI, time, cx.tb);
  const V3<T> Hres = axial<T>(L, CMTJ_SLOT_HRES, time, cx.tb);
  // calculateSecondOrderAnisotropy (645-652)
  const T K2 = driver_value<T>(L.drv[CMTJ_SLOT_ANIS2], time, cx.tb);
  const T da = dot(anis, m);
  const V3<T> Hanis2 = anis * ((4 * K2) * pow(da, 3) / Ms);
  const V3<T> Hfl;  // Hfluctuation default argument: zero vector
  const V3<T> H = Hext + Hanis + Hanis2 + Hiec + Hidmi + Hoe + Hdmi + Hfl - Hdemag - Hdipole + Hres;
  if (cx.side) {
    cx.side->K = K; cx.side->K2 = K2; cx.side->Jb = Jb; cx.side->Jt = Jt;
    cx.side->Hext = Hext; cx.side->Hiec = Hiec; cx.side->Hanis = Hanis; cx.side->Hdemag = Hdemag;
  }
  return H;
}

// solveLLG (junction.hpp:716-815).
template <typename T>
V3<T> llg(Ctx<T> &cx, const T &time, const V3<T> &m, const V3<T> &bottom, const V3<T> &top, const V3<T> &H) {
  const cmtj_layer_t &L = *cx.L;
  const T GYRO = cx.c->gyro;
  const T damping = L.damping;
  const V3<T> prod = cross(m, H);
  const V3<T> prod2 = cross(m, prod);
  const T convTerm = 1 / (1 + sq(damping));
  const V3<T> dmdt = prod + prod2 * damping;
  V3<T> reference;
  switch (L.referenceType) {
  case CMTJ_REF_FIXED: reference = v3<T>(L.ref); break;
  case CMTJ_REF_TOP: reference = top; break;
  case CMTJ_REF_BOTTOM: reference = bottom; break;
  default: break;
  }
  if (L.includeSTT) {
    const T I = driver_value<T>(L.drv[CMTJ_SLOT_CURRENT], time, cx.tb);
    if (cx.side) cx.side->I = I;
    const T aJ = cx.c->hbar * I / (cx.c->echarge * L.Ms * L.thickness);
    T eta = 0;
    if (L.alternativeSTT) {
      eta = (L.spinPolarisation) / (1 + L.slonczewski * dot(m, reference));
    } else {
      const T slonSq = sq(T(L.slonczewski));
      eta = (L.spinPolarisation * slonSq) / (slonSq + 1 + (slonSq - 1) * dot(m, reference));
    }
    const T sttTerm = GYRO * aJ * eta;
    const V3<T> fieldLike = cross(m, reference);
    const V3<T> dampingLike = cross(m, fieldLike);
    return (dmdt * -GYRO + dampingLike * -sttTerm * T(L.kappa) + fieldLike * sttTerm * T(L.beta)) * convTerm;
  } else if (L.includeSOT) {
    T Hdl = 0, Hfl = 0, Hdl2 = 0, Hfl2 = 0;
    if (L.dynamicSOT) {
      Hdl = driver_value<T>(L.drv[CMTJ_SLOT_DL], time, cx.tb);
      Hfl = driver_value<T>(L.drv[CMTJ_SLOT_FL], time, cx.tb);
      Hdl2 = driver_value<T>(L.drv[CMTJ_SLOT_DL2], time, cx.tb);
      Hfl2 = driver_value<T>(L.drv[CMTJ_SLOT_FL2], time, cx.tb);
    } else {
      const T I = driver_value<T>(L.drv[CMTJ_SLOT_CURRENT], time, cx.tb);
      if (cx.side) cx.side->I = I;
      Hdl = L.dampingLikeTorque * I;
      Hfl = L.fieldLikeTorque * I;
    }
    const V3<T> ref2 = v3<T>(L.ref2);
    if (cx.side) {
      cx.side->Hfl = reference * (Hfl - damping * Hdl);
      cx.side->Hdl = reference * (Hdl + damping * Hfl);
    }
    const V3<T> cm_p = cross(m, reference);
    const V3<T> ccm_p = cross(m, cm_p);
    const V3<T> cm_s = cross(m, ref2);
    const V3<T> ccm_s = cross(m, cm_s);
    const V3<T> flp = cm_p * (Hfl - damping * Hdl);
    const V3<T> dlp = ccm_p * (Hdl + damping * Hfl);
    const V3<T> fls = cm_s * (Hfl2 - damping * Hdl2);
    const V3<T> dls = ccm_s * (Hdl2 + damping * Hfl2);
    return (dmdt + flp + dlp + fls + dls) * -GYRO * convTerm;
  }
  return dmdt * -GYRO * convTerm;
}

template <typename T>
V3<T> rhs(Ctx<T> &cx, const T &time, const V3<T> &m, const V3<T> &bottom, const V3<T> &top) {
  const V3<T> H = heff<T>(cx, time, m, bottom, top);
  return llg<T>(cx, time, m, bottom, top, H);
}

// stochasticTorque (junction.hpp:824-831).
template <typename T> V3<T> stoch_torque(const cmtj_layer_t &L, const cmtj_constants_t &c, const V3<T> &m, const V3<T> &dW) {
  const T convTerm = -T(c.gyro) / (1. + sq(T(L.damping)));
  const V3<T> th = cross(m, dW);
  const V3<T> th2 = cross(m, th);
  return (th + th2 * T(L.damping)) * convTerm;
}

// getOneFVector (junction.hpp:1130-1136) through VectorAlphaNoise::
// tickVector (noise.hpp:280-290): the float samples of iteration `step`
// (all three normalised for Axis::all, else the one axis) times the scale.
template <typename T> V3<T> alpha_sample(const cmtj_layer_t &L, uint64_t step) {
  if (!L.alpha_buf || step >= L.alpha_len) return V3<T>();
  const float *b = L.alpha_buf + step;
  const size_t n = L.alpha_len;
  const int ax = L.alpha_axis;
  V3<T> v((ax == 0 || ax == 3) ? (double)b[0] : 0.0, (ax == 1 || ax == 3) ? (double)b[n] : 0.0,
          (ax == 2 || ax == 3) ? (double)b[2 * n] : 0.0);
  if (ax == 3) v = normalized(v);
  return v * T(L.alpha_scale);
}

// getStochasticLangevinVector (junction.hpp:1111-1128) plus getOneFVector:
// the dW of the Euler-Heun and Heun runners (1726-1727, 1792-1793).
template <typename T> V3<T> langevin(const cmtj_layer_t &L, const cmtj_constants_t &c, const T &time,
                                     uint64_t step, const Tables<T> &tb) {
  V3<T> dW;
  if (L.temperatureSet) {
    const T temp = driver_value<T>(L.drv[CMTJ_SLOT_TEMPERATURE], time, tb);
    const T mainFactor = (2 * T(L.damping) * T(c.kB) * temp) / (T(L.Ms) * T(L.cellVolume) * T(c.gyro));
    const T sigma = sqrt(mainFactor);
    double g[3];
    gaussian3(L.seed_lo, L.seed_hi, L.noise_step + step, g);
    dW = V3<T>(g[0], g[1], g[2]) * sigma;
  }
  if (L.alpha_buf) dW = dW + alpha_sample<T>(L, step);
  return dW;
}

// --------------------------------------------------------------- junction
template <typename T> struct JunctionRun {
  const cmtj_junction_t &J;
  cmtj_layer_t *layers;  // J.n_layers entries
  const cmtj_sim_params_t &p;
  const double *tables;
  std::vector<V3<T>> mag;
  std::vector<Side<T>> side;

  JunctionRun(const cmtj_junction_t &J_, cmtj_layer_t *layers_, const cmtj_sim_params_t &p_, const double *tables_)
      : J(J_), layers(layers_), p(p_), tables(tables_), mag(J_.n_layers), side(J_.n_layers) {
    for (int l = 0; l < J.n_layers; ++l) mag[l] = V3<T>(layers[l].mag[0], layers[l].mag[1], layers[l].mag[2]);
  }

  Ctx<T> ctx(int l, uint32_t step, int stage, bool record) {
    Ctx<T> cx;
    cx.L = &layers[l];
    cx.c = &p.c;
    cx.tb.data = tables;
    cx.tb.step = step;
    cx.tb.stage = stage;
    cx.side = (record && p.calculate_energies) ? &side[l] : nullptr;
    return cx;
  }

  // rk4_step (junction.hpp:1017-1041); false on NaN.
  bool rk4(int l, const T &t, uint32_t i, const V3<T> &bottom, const V3<T> &top) {
    const T dt = p.time_step;
    V3<T> m_t = mag[l];
    Ctx<T> c0 = ctx(l, i, 0, false), c1 = ctx(l, i, 1, false), c2 = ctx(l, i, 2, true);
    const V3<T> k1 = rhs<T>(c0, t, m_t, bottom, top) * dt;
    const V3<T> k2 = rhs<T>(c1, t + 0.5 * dt, m_t + k1 * 0.5, bottom, top) * dt;
    const V3<T> k3 = rhs<T>(c1, t + 0.5 * dt, m_t + k2 * 0.5, bottom, top) * dt;
    const V3<T> k4 = rhs<T>(c2, t + dt, m_t + k3, bottom, top) * dt;
    m_t = m_t + (k1 + (k2 * 2.0) + (k3 * 2.0) + k4) / 6.0;
    mag[l] = normalized(m_t);
    return !std::isnan((double)mag[l].x);
  }

  // runSingleLayerSolver / runMultiLayerSolver (1668-1707).
  bool step_rk4(const T &t, uint32_t i) {
    const int n = J.n_layers;
    std::vector<V3<T>> copies(n + 2);
    for (int l = 0; l < n; ++l) copies[l + 1] = mag[l];
    for (int l = 0; l < n; ++l)
      if (!rk4(l, t, i, copies[l], copies[l + 2])) return false;
    return true;
  }

  // eulerHeunSolverStep (1709-1754).
  void step_euler_heun(const T &t, uint32_t i) {
    const int n = J.n_layers;
    const T dt = p.time_step;
    std::vector<V3<T>> mPrime(n);
    for (int l = 0; l < n; ++l) {
      Ctx<T> c0 = ctx(l, i, 0, true);
      const V3<T> dW = langevin<T>(layers[l], p.c, t, i, c0.tb);
      const V3<T> bottom = (l == 0) ? V3<T>() : mag[l - 1];
      const V3<T> top = (l == n - 1) ? V3<T>() : mag[l + 1];
      const V3<T> f = rhs<T>(c0, t, mag[l], bottom, top);
      const V3<T> g = stoch_torque<T>(layers[l], p.c, mag[l], dW);
      const V3<T> mNext = mag[l] + g * sqrt(dt);
      const V3<T> g2 = stoch_torque<T>(layers[l], p.c, mNext, dW);
      mPrime[l] = mag[l] + f * dt + smul<T>(0.5, g + g2) * sqrt(dt);
    }
    for (int l = 0; l < n; ++l) mag[l] = normalized(mPrime[l]);
  }

  // heunSolverStep (1756-1815).
  void step_heun(const T &t, uint32_t i) {
    const int n = J.n_layers;
    const T dt = p.time_step;
    std::vector<V3<T>> fn(n), gn(n), dW(n), mNext(n);
    for (int l = 0; l < n; ++l) {
      const V3<T> bottom = (l == 0) ? V3<T>() : mag[l - 1];
      const V3<T> top = (l == n - 1) ? V3<T>() : mag[l + 1];
      Ctx<T> c0 = ctx(l, i, 0, false);
      fn[l] = rhs<T>(c0, t, mag[l], bottom, top);
      dW[l] = langevin<T>(layers[l], p.c, t, i, c0.tb);
      gn[l] = stoch_torque<T>(layers[l], p.c, mag[l], dW[l]);
      mNext[l] = mag[l] + fn[l] * dt + gn[l] * sqrt(dt);
    }
    for (int l = 0; l < n; ++l) {
      const V3<T> bottom = (l == 0) ? V3<T>() : mNext[l - 1];
      const V3<T> top = (l == n - 1) ? V3<T>() : mNext[l + 1];
      Ctx<T> c2 = ctx(l, i, 2, true);
      const V3<T> f2 = rhs<T>(c2, t + dt, mNext[l], bottom, top);
      const V3<T> g2 = stoch_torque<T>(layers[l], p.c, mNext[l], dW[l]);
      mag[l] = mag[l] + smul<T>(0.5 * dt, fn[l] + f2) + smul<T>(0.5, gn[l] + g2) * sqrt(dt);
      mag[l] = normalized(mag[l]);
    }
  }

  // logLayerParams (1580-1636) into one row of log_width doubles.
  void log_row(double *row, const T &t) {
    const int n = J.n_layers;
    int col = 0;
    for (int l = 0; l < n; ++l) {
      if (p.calculate_energies) {
        const Side<T> &s = side[l];
        const T vals[26] = {s.K, s.K2, s.Jb, s.Jt, s.I,
                            s.Hext.x, s.Hext.y, s.Hext.z, s.Hiec.x, s.Hiec.y, s.Hiec.z,
                            s.Hanis.x, s.Hanis.y, s.Hanis.z, s.Hdemag.x, s.Hdemag.y, s.Hdemag.z,
                            0.0, 0.0, 0.0,
                            s.Hfl.x, s.Hfl.y, s.Hfl.z, s.Hdl.x, s.Hdl.y, s.Hdl.z};
        for (int k = 0; k < 26; ++k) row[col++] = (double)vals[k];
      }
      row[col++] = (double)mag[l].x;
      row[col++] = (double)mag[l].y;
      row[col++] = (double)mag[l].z;
    }
    T r0 = 0.0, r1 = 0.0, r2 = 0.0;
    if (J.mr_mode == CMTJ_MR_CLASSIC && n == 1) {
      const T cosT = dot(mag[0], v3<T>(layers[0].ref));
      r0 = J.Rp + (((J.Rap - J.Rp) / 2.0) * (1.0 - cosT));
    } else if (J.mr_mode == CMTJ_MR_CLASSIC && n > 1) {
      const T cosT = dot(mag[0], mag[1]);
      r0 = J.Rp + (((J.Rap - J.Rp) / 2.0) * (1.0 - cosT));
    } else if (J.mr_mode == CMTJ_MR_STRIP) {
      T Rx_acc = 0.0, Ry_acc = 0.0;
      for (int l = 0; l < n; ++l) {
        const T Rx = J.Rx0[l] + J.AMR_X[l] * (mag[l].x * mag[l].x) + J.SMR_X[l] * (mag[l].y * mag[l].y);
        const T Ry = J.Ry0[l] + 0.5 * J.AHE[l] * mag[l].z + (J.AMR_Y[l] + J.SMR_Y[l]) * mag[l].x * mag[l].y;
        Rx_acc = Rx_acc + 1. / Rx;
        Ry_acc = Ry_acc + 1. / Ry;
      }
      r0 = 1 / Rx_acc;
      r1 = 1 / Ry_acc;
      r2 = 0.;
    }
    row[col++] = (double)r0;
    row[col++] = (double)r1;
    row[col++] = (double)r2;
    row[col++] = (double)t;
  }

  // dormand_prince_step (junction.hpp:866-1002) of layer l: tries a step
  // of size ts from time t; updates ts to the next step size (accepted or
  // not) and the layer's PID state.  Returns accepted; nan set when an
  // accepted m is NaN (the reference throws "NAN magnetisation").
  bool dp(int l, const T &t, T &ts, const V3<T> &bottom, const V3<T> &top, bool &nan) {
    cmtj_adaptive_t &ap = layers[l].adaptive;
    const V3<T> m_t = mag[l];
    const T c2 = 1.0 / 5.0, c3 = 3.0 / 10.0, c4 = 4.0 / 5.0, c5 = 8.0 / 9.0, c6 = 1.0, c7 = 1.0;
    Ctx<T> c0 = ctx(l, 0, 0, false), cl = ctx(l, 0, 0, true);
    const V3<T> k1 = rhs<T>(c0, t, m_t, bottom, top) * ts;
    const V3<T> k2 = rhs<T>(c0, t + c2 * ts, m_t + k1 * (c2), bottom, top) * ts;
    const V3<T> k3 = rhs<T>(c0, t + c3 * ts, m_t + k1 * (3.0 / 40.0) + k2 * (9.0 / 40.0), bottom, top) * ts;
    const V3<T> k4 = rhs<T>(c0, t + c4 * ts, m_t + k1 * (44.0 / 45.0) + k2 * (-56.0 / 15.0) + k3 * (32.0 / 9.0),
                            bottom, top) * ts;
    const V3<T> k5 = rhs<T>(c0, t + c5 * ts,
                            m_t + k1 * (19372.0 / 6561.0) + k2 * (-25360.0 / 2187.0) + k3 * (64448.0 / 6561.0) +
                                k4 * (-212.0 / 729.0),
                            bottom, top) * ts;
    const V3<T> k6 = rhs<T>(c0, t + c6 * ts,
                            m_t + k1 * (9017.0 / 3168.0) + k2 * (-355.0 / 33.0) + k3 * (46732.0 / 5247.0) +
                                k4 * (49.0 / 176.0) + k5 * (-5103.0 / 18656.0),
                            bottom, top) * ts;
    const V3<T> k7 = rhs<T>(cl, t + c7 * ts,
                            m_t + k1 * (35.0 / 384.0) + k3 * (500.0 / 1113.0) + k4 * (125.0 / 192.0) +
                                k5 * (-2187.0 / 6784.0) + k6 * (11.0 / 84.0),
                            bottom, top) * ts;
    V3<T> m5 = m_t + k1 * (35.0 / 384.0) + k3 * (500.0 / 1113.0) + k4 * (125.0 / 192.0) + k5 * (-2187.0 / 6784.0) +
               k6 * (11.0 / 84.0);
    const V3<T> m4 = m_t + k1 * (5179.0 / 57600.0) + k3 * (7571.0 / 16695.0) + k4 * (393.0 / 640.0) +
                     k5 * (-92097.0 / 339200.0) + k6 * (187.0 / 2100.0) + k7 * (1.0 / 40.0);
    const V3<T> err = m5 - m4;
    const T err_norm = sqrt(sq(err.x) + sq(err.y) + sq(err.z));
    const T tol = ap.abs_tol + ap.rel_tol * sqrt(sq(m_t.x) + sq(m_t.y) + sq(m_t.z));
    T ratio = err_norm / tol;
    if (tol < 1e-15 || std::isnan(ratio) || std::isinf(ratio)) ratio = 10.0;
    T factor;
    if (ap.use_pid_control) {
      const T e_n = log(ratio);
      ap.integral_error += e_n;
      factor = exp(ap.kp * e_n + ap.ki * ap.integral_error + ap.kd * (e_n - ap.prev_error_ratio));
      ap.prev_error_ratio = e_n;
    } else {
      factor = ap.safety_factor * pow(1.0 / ratio, 0.2);
    }
    if (std::isnan(factor) || std::isinf(factor)) factor = ap.min_factor;
    factor = std::min(factor, T(ap.max_factor));
    factor = std::max(factor, T(ap.min_factor));
    T next = ts * factor;
    if (std::isnan(next) || std::isinf(next) || next <= 0) next = ts * ap.min_factor;
    if (ratio <= 1.0) {
      mag[l] = normalized(m5);
      if (std::isnan(mag[l].x)) nan = true;
      ts = next;
      return true;
    }
    ts = next;
    return false;
  }

  // runSimulation's Dormand-Prince loop (1982-2045) with runSingleLayerSolver
  // / runMultiLayerSolver (1668-1707).  Every layer's step sees the step size
  // the previous layer's step chose (one shared timeStep reference), and t
  // advances by the step size chosen for the NEXT step, both as in the
  // reference.  A multi-layer rejection stops with CMTJ_STATUS_DP_STALL
  // where the reference would continue from hopt = -1 without end.
  uint32_t run_dp(double *log) {
    const int n = J.n_layers;
    const T total = p.total_time, wf = p.write_frequency;
    T t = 0.0, next_write = 0.0, cur = p.time_step;
    uint32_t row = 0, status = CMTJ_STATUS_OK;
    uint64_t attempts = 0;
    std::vector<V3<T>> copies(n + 2);
    while (t < total) {
      if (++attempts > p.max_attempts) { status = CMTJ_STATUS_LIMIT; break; }
      if (t + cur > total) cur = total - t;
      int consecutive = 0;
      if (std::isnan(cur) || std::isinf(cur) || cur <= 0) {
        cur = p.time_step;
        consecutive++;
      }
      bool accepted, nan = false;
      if (n > 1) {
        accepted = true;
        for (int l = 0; l < n; ++l) copies[l + 1] = mag[l];
        for (int l = 0; l < n; ++l)
          if (!dp(l, t, cur, copies[l], copies[l + 2], nan)) accepted = false;
        if (!accepted) { status = CMTJ_STATUS_DP_STALL; break; }
      } else {
        accepted = dp(0, t, cur, V3<T>(), V3<T>(), nan);
      }
      if (nan) { status = CMTJ_STATUS_NAN; break; }
      if (!accepted && (cur < 1e-15 || consecutive >= 10)) {
        accepted = true;
        consecutive = 0;
      }
      if (accepted) {
        t += cur;
        if (t >= next_write) {
          if (row >= p.n_log) { status = CMTJ_STATUS_LIMIT; break; }
          log_row(log + (size_t)row * p.log_width, t);
          ++row;
          next_write = ((double)(uint32_t)(t / wf) + 1) * wf;
        }
      }
    }
    rows = row;
    for (int l = 0; l < n; ++l) {
      layers[l].mag[0] = (double)mag[l].x;
      layers[l].mag[1] = (double)mag[l].y;
      layers[l].mag[2] = (double)mag[l].z;
    }
    return status;
  }

  // runSimulation fixed-step loop (1966-1981).
  uint32_t rows = 0;
  uint32_t run(double *log) {
    uint32_t row = 0;
    uint32_t status = CMTJ_STATUS_OK;
    for (uint32_t i = 0; i < p.total_iterations; ++i) {
      const T t = (double)i * p.time_step;
      if (p.solver == CMTJ_RK4) {
        if (!step_rk4(t, i)) { status = CMTJ_STATUS_NAN; break; }
      } else if (p.solver == CMTJ_EULER_HEUN) {
        step_euler_heun(t, i);
      } else {
        step_heun(t, i);
      }
      if (!(i % p.write_every)) {
        log_row(log + (size_t)row * p.log_width, t);
        ++row;
      }
    }
    rows = row;
    for (int l = 0; l < J.n_layers; ++l) {
      layers[l].mag[0] = (double)mag[l].x;
      layers[l].mag[1] = (double)mag[l].y;
      layers[l].mag[2] = (double)mag[l].z;
    }
    return status;
  }
};

}  // namespace oracle

namespace oracle_cnt {
// ------------------------------------------------------------ op counting
// A double that counts the arithmetic done on it; used once to fix the FLOP
// count per layer-step.  add/sub/mul/div/sqrt count 1, transcendental 1.
struct Counter { static thread_local uint64_t add, mul, div, sqrt_, trans; };
thread_local uint64_t Counter::add = 0, Counter::mul = 0, Counter::div = 0, Counter::sqrt_ = 0, Counter::trans = 0;
struct CD {
  double v;
  CD() : v(0) {}
  CD(double x) : v(x) {}
  explicit operator double() const { return v; }
};
inline CD operator+(CD a, CD b) { ++Counter::add; return CD(a.v + b.v); }
inline CD operator-(CD a, CD b) { ++Counter::add; return CD(a.v - b.v); }
inline CD operator*(CD a, CD b) { ++Counter::mul; return CD(a.v * b.v); }
inline CD operator/(CD a, CD b) { ++Counter::div; return CD(a.v / b.v); }
inline CD operator-(CD a) { return CD(-a.v); }
inline CD operator+(CD a, double b) { return a + CD(b); }
inline CD operator+(double a, CD b) { return CD(a) + b; }
inline CD operator-(CD a, double b) { return a - CD(b); }
inline CD operator-(double a, CD b) { return CD(a) - b; }
inline CD operator*(CD a, double b) { return a * CD(b); }
inline CD operator*(double a, CD b) { return CD(a) * b; }
inline CD operator/(CD a, double b) { return a / CD(b); }
inline CD operator/(double a, CD b) { return CD(a) / b; }
inline CD operator*(int a, CD b) { return CD((double)a) * b; }
inline CD operator+(int a, CD b) { return CD((double)a) + b; }
inline CD operator/(int a, CD b) { return CD((double)a) / b; }
inline bool operator<(CD a, CD b) { return a.v < b.v; }
inline bool operator<=(CD a, CD b) { return a.v <= b.v; }
inline bool operator>=(CD a, CD b) { return a.v >= b.v; }
inline bool operator<(CD a, double b) { return a.v < b; }
inline bool operator<=(CD a, double b) { return a.v <= b; }
inline bool operator<=(CD a, int b) { return a.v <= b; }
inline bool operator>=(CD a, double b) { return a.v >= b; }
inline bool operator<=(double a, CD b) { return a <= b.v; }
inline bool operator!=(CD a, int b) { return a.v != b; }
inline CD sqrt(CD a) { ++Counter::sqrt_; return CD(std::sqrt(a.v)); }
inline CD sin(CD a) { ++Counter::trans; return CD(std::sin(a.v)); }
inline CD exp(CD a) { ++Counter::trans; return CD(std::exp(a.v)); }
inline CD erf(CD a) { ++Counter::trans; return CD(std::erf(a.v)); }
inline CD fabs(CD a) { return CD(std::fabs(a.v)); }
inline CD pow(CD a, int n) { CD r = a; for (int k = 1; k < n; ++k) r = r * a; return r; }

}  // namespace oracle_cnt

// ----------------------------------------------------------------- C ABI
extern "C" {

int oracle_log_width(int n_layers, int calculate_energies) {
  return n_layers * (calculate_energies ? CMTJ_ENERGY_COLS : 3) + 4;
}

// Junction::runSimulation on the CPU for n_junctions junctions, using
// n_threads host threads (junctions are independent).  Same packed inputs,
// log layout and [n][2] status words as cmtj_run_simulation_f64.
int oracle_run_simulation(const cmtj_junction_t *junctions, int32_t n_junctions, cmtj_layer_t *layers,
                          const double *tables, const cmtj_sim_params_t *p, double *log, uint32_t *status,
                          int32_t n_threads) {
  if (n_junctions < 0 || !p || p->write_every == 0) return CMTJ_ERR_ARG;
  std::atomic<int32_t> next(0);
  auto worker = [&]() {
    for (;;) {
      const int32_t j = next.fetch_add(1);
      if (j >= n_junctions) break;
      const cmtj_junction_t &J = junctions[j];
      oracle::JunctionRun<double> run(J, layers + J.layer_offset, *p, tables);
      double *out = log + (size_t)j * p->n_log * p->log_width;
      status[2 * j] = p->solver == CMTJ_DORMAND_PRINCE ? run.run_dp(out) : run.run(out);
      status[2 * j + 1] = run.rows;
    }
  };
  if (n_threads <= 1) {
    worker();
  } else {
    std::vector<std::thread> pool;
    for (int k = 0; k < n_threads; ++k) pool.emplace_back(worker);
    for (auto &t : pool) t.join();
  }
  return CMTJ_OK;
}

// GroupInteraction::runSimulation (reservoir.hpp:185-230) with
// stepFunctionalSolver (130-151), for n_groups groups.  The fixed pair
// geometry comes from the host (cmtj_pair_t, formed with the reference's own
// expressions); each step freezes every top layer's m, sums each junction's
// interaction field from all others in index order (computeDipoleInteraction
// 77-97 or the tensor form 99-122), sets it as the top layer's reserved
// interaction field, then steps every junction with the last junction's
// runner.  Same inputs, log layout and status words as cmtj_run_group_f64.
int oracle_run_group(const cmtj_junction_t *junctions, cmtj_layer_t *layers, const double *tables,
                     const cmtj_group_t *groups, int32_t n_groups, const cmtj_pair_t *pairs, const int32_t *top,
                     const cmtj_sim_params_t *p, double *log, uint32_t *status) {
  using oracle::V3;
  if (n_groups < 0 || !p || p->write_every == 0) return CMTJ_ERR_ARG;
  for (int32_t g = 0; g < n_groups; ++g) {
    const cmtj_group_t &G = groups[g];
    const int N = G.n_junctions;
    std::vector<oracle::JunctionRun<double>> runs;
    runs.reserve(N);
    for (int k = 0; k < N; ++k) {
      const cmtj_junction_t &J = junctions[G.first_junction + k];
      runs.emplace_back(J, layers + J.layer_offset, *p, tables);
      cmtj_layer_t &T = layers[J.layer_offset + top[G.first_junction + k]];
      for (int c = 0; c < 3; ++c) T.drv[CMTJ_SLOT_HRES + c].update = CMTJ_DRV_CONSTANT;
    }
    uint32_t row = 0, code = CMTJ_STATUS_OK;
    std::vector<V3<double>> frozen(N);
    for (uint32_t i = 0; i < p->total_iterations && code == CMTJ_STATUS_OK; ++i) {
      const double t = (double)i * p->time_step;
      for (int k = 0; k < N; ++k) frozen[k] = runs[k].mag[top[G.first_junction + k]];
      for (int k = 0; k < N; ++k) {
        V3<double> H;
        if (G.interaction != CMTJ_INTERACTION_NULL) {
          for (int q = 0; q < N; ++q) {
            if (q == k) continue;
            const cmtj_pair_t &pr = pairs[G.pair_offset + (int64_t)k * N + q];
            const V3<double> &m = frozen[q];
            V3<double> term;
            if (G.interaction == CMTJ_INTERACTION_DIPOLE) {
              const V3<double> rij(pr.g[0], pr.g[1], pr.g[2]);
              const double s = 3 * (m.x * rij.x + m.y * rij.y + m.z * rij.z);
              term = oracle::smul<double>(pr.scale, oracle::smul<double>(s, rij) / pr.g[4] - m / pr.g[3]);
            } else {
              const double *tt = pr.g;
              term = V3<double>(tt[0] * m.x + tt[1] * m.y + tt[2] * m.z, tt[3] * m.x + tt[4] * m.y + tt[5] * m.z,
                                tt[6] * m.x + tt[7] * m.y + tt[8] * m.z) * pr.scale;
            }
            H = H + term;
          }
        }
        const cmtj_junction_t &J = junctions[G.first_junction + k];
        cmtj_layer_t &T = layers[J.layer_offset + top[G.first_junction + k]];
        T.drv[CMTJ_SLOT_HRES + 0].constantValue = H.x;
        T.drv[CMTJ_SLOT_HRES + 1].constantValue = H.y;
        T.drv[CMTJ_SLOT_HRES + 2].constantValue = H.z;
      }
      for (int k = 0; k < N && code == CMTJ_STATUS_OK; ++k) {
        if (p->solver == CMTJ_RK4) {
          const bool ok = G.single_layer_runner ? runs[k].rk4(0, t, i, V3<double>(), V3<double>())
                                                : runs[k].step_rk4(t, i);
          if (!ok) code = CMTJ_STATUS_NAN;
        } else if (p->solver == CMTJ_EULER_HEUN) {
          runs[k].step_euler_heun(t, i);
        } else {
          runs[k].step_heun(t, i);
        }
      }
      if (code != CMTJ_STATUS_OK) break;
      if (!(i % p->write_every)) {
        for (int k = 0; k < N; ++k)
          runs[k].log_row(log + ((size_t)(G.first_junction + k) * p->n_log + row) * p->log_width, t);
        ++row;
      }
    }
    for (int k = 0; k < N; ++k) {
      const int gj = G.first_junction + k;
      cmtj_layer_t *Ls = layers + junctions[gj].layer_offset;
      for (int l = 0; l < junctions[gj].n_layers; ++l) {
        Ls[l].mag[0] = runs[k].mag[l].x;
        Ls[l].mag[1] = runs[k].mag[l].y;
        Ls[l].mag[2] = runs[k].mag[l].z;
      }
      status[2 * gj] = code;
      status[2 * gj + 1] = row;
    }
  }
  return CMTJ_OK;
}

// FLOP count of one junction run on the counting scalar type:
// out[0] adds+subs, out[1] muls, out[2] divs, out[3] sqrts, out[4] sin/exp/erf.
int oracle_count_flops(const cmtj_junction_t *junction, cmtj_layer_t *layers, const double *tables,
                       const cmtj_sim_params_t *p, double *log, uint64_t *out) {
  using oracle_cnt::Counter;
  Counter::add = Counter::mul = Counter::div = Counter::sqrt_ = Counter::trans = 0;
  oracle::JunctionRun<oracle_cnt::CD> run(*junction, layers, *p, tables);
  run.run(log);
  out[0] = Counter::add;
  out[1] = Counter::mul;
  out[2] = Counter::div;
  out[3] = Counter::sqrt_;
  out[4] = Counter::trans;
  return CMTJ_OK;
}

// Three Gaussian draws of the thermal stream, exposed for the noise tests.
void oracle_gaussian3(uint32_t seed_lo, uint32_t seed_hi, uint64_t step, double *g) {
  oracle::gaussian3(seed_lo, seed_hi, step, g);
}

// BufferedAlphaNoise::fillBuffer for n_buffers rows of n samples (the
// restatement of cmtj_alpha_noise_f32): out[r*n ..] from specs[r], white
// draws from white[r*n ..] when white is not null.  Rows run on n_threads
// host threads.
int oracle_alpha_noise(const cmtj_alpha_noise_t *specs, int32_t n_buffers, uint32_t n, const float *white,
                       float *out, int32_t n_threads) {
  if (n_buffers < 0 || n == 0 || !specs || !out) return CMTJ_ERR_ARG;
  std::atomic<int> next(0);
  auto work = [&]() {
    for (int r = next++; r < n_buffers; r = next++)
      oracle::alpha_fill(specs[r], n, white ? white + (size_t)r * n : nullptr, out + (size_t)r * n);
  };
  const int t = std::max(1, std::min<int>(n_threads, n_buffers));
  std::vector<std::thread> pool;
  for (int k = 1; k < t; ++k) pool.emplace_back(work);
  work();
  for (auto &th : pool) th.join();
  return CMTJ_OK;
}

}  // extern "C"
