// FP32 batched form: persistent, work-stealing macrospin integrator.
//
// Each thread owns one junction at a time: its magnetisations, RK4
// accumulators, driver waves and reductions live in registers.  Layers are
// unrolled at compile time (L = 1..4), the solver and the set of active
// field/torque terms (FEAT) are template parameters, so a partition of
// uniform junctions runs straight-line FP32 FMA code.  When a junction
// ends, its lane takes the next one from a warp-aggregated atomic ticket,
// so uneven durations keep every lane busy until the queue drains.
//
// Arithmetic (core/junction.hpp:580-831, 1017-1041, 1709-1815 of the
// reference) is restated with constants folded on the host: the field terms
// arrive pre-divided by Ms, Ms*t and mu0 (cmtj_f32_layer_t), |m| is
// renormalised with rsqrt every step, driver time enters through integer
// step counts and Q0.64 phases (no FP32 time accumulator).
//
// Logs are staged per thread in shared memory and written to global memory
// with cp.async.bulk (TMA bulk copy, shared::cta -> global), one copy per
// completed tile of log_tile samples.
#pragma once
#include "common.cuh"
#include "philox.cuh"

namespace cmtjf {

struct F3 {
  float x, y, z;
};
__device__ __forceinline__ F3 f3(float x, float y, float z) {
  F3 r;
  r.x = x;
  r.y = y;
  r.z = z;
  return r;
}
__device__ __forceinline__ F3 operator+(F3 a, F3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ F3 operator-(F3 a, F3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ F3 operator*(F3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ F3 fma3(F3 a, float s, F3 b) { return f3(fmaf(a.x, s, b.x), fmaf(a.y, s, b.y), fmaf(a.z, s, b.z)); }
__device__ __forceinline__ float dot(F3 a, F3 b) { return fmaf(a.x, b.x, fmaf(a.y, b.y, a.z * b.z)); }
__device__ __forceinline__ F3 cross(F3 a, F3 b) {
  return f3(fmaf(a.y, b.z, -a.z * b.y), fmaf(a.z, b.x, -a.x * b.z), fmaf(a.x, b.y, -a.y * b.x));
}
__device__ __forceinline__ F3 ld3(const float *p) { return f3(p[0], p[1], p[2]); }
__device__ __forceinline__ F3 renorm(F3 m) { return m * rsqrtf(dot(m, m)); }
__device__ __forceinline__ F3 matvec(const float *t, F3 m) {
  return f3(fmaf(t[0], m.x, fmaf(t[1], m.y, t[2] * m.z)), fmaf(t[3], m.x, fmaf(t[4], m.y, t[5] * m.z)),
            fmaf(t[6], m.x, fmaf(t[7], m.y, t[8] * m.z)));
}

// sin(2 pi x) of a phase fraction x in [0, 1) taken from a 64-bit
// fixed-point phase (its top 24 bits).  The hardware sine is accurate to
// ~1e-6 in [-pi, pi), so the argument is shifted there: sin(2 pi (x - 1/2))
// = -sin(2 pi x).  An error of 1e-6 of a driver's amplitude is far below the
// FP32 form's 1e-4 bound on m.
__device__ __forceinline__ float sin2pi_phase(uint64_t ph) {
  const float x = (float)(uint32_t)(ph >> 40) * 5.9604644775390625e-08f;  // 2^-24
  return -__sinf(6.2831853f * (x - 0.5f));
}

// Neumaier compensated accumulation.
__device__ __forceinline__ void kadd(float &s, float &c, float v) {
  const float t = s + v;
  c += (fabsf(s) >= fabsf(v)) ? ((s - t) + v) : ((v - t) + s);
  s = t;
}

template <int FEAT> struct Feat {
  static constexpr bool full_demag = (FEAT & CMTJ_FEAT_FULL_DEMAG) != 0;
  static constexpr bool dipole = (FEAT & CMTJ_FEAT_DIPOLE) != 0;
  static constexpr bool idmi = (FEAT & CMTJ_FEAT_IDMI) != 0;
  static constexpr bool k2 = (FEAT & CMTJ_FEAT_K2) != 0;
  static constexpr bool stt = (FEAT & CMTJ_FEAT_STT) != 0;
  static constexpr bool sot = (FEAT & CMTJ_FEAT_SOT) != 0;
  static constexpr bool waves = (FEAT & CMTJ_FEAT_WAVES) != 0;
  static constexpr bool swaves = (FEAT & CMTJ_FEAT_SCALAR_WAVES) != 0;
  static constexpr bool iec2 = (FEAT & CMTJ_FEAT_IEC2) != 0;
  static constexpr bool twaves = waves && (stt || sot);  // current / torque waves
  static constexpr bool offaxis = (FEAT & CMTJ_FEAT_OFFAXIS) != 0;
  // anisotropy (constant K along a coordinate axis) + diagonal demag fold
  // into one diagonal tensor: H += M m with M_i = 2K a_i^2/(mu0 Ms) - N_ii
  static constexpr bool diag = !full_demag && !k2 && !swaves && !offaxis;
  // every field term is stored pre-multiplied by the layer's gamma dt
  // prefactor, so the torque needs no final scaling (not with SOT, whose
  // torques add to the LL term before the scaling, nor with scalar waves,
  // whose deltas add to the unscaled coefficients)
  static constexpr bool prescale = !sot && !swaves;
};

// Per-layer constants held in registers for the life of a junction.
template <int FEAT> struct LayerP {
  F3 a;
  F3 M;  // diag: the folded anisotropy + demag tensor (times gdt when prescale)
  float kc, k2c;
  float N[9];
  float Db[9], Dt[9];
  F3 h0;
  float jb, jt, j2b, j2t;
  F3 dmib, dmit;
  float gam, gdt, alpha;  // -gamma/(1+alpha^2), and that times dt (or dt/6 for RK4)
  F3 ref, ref2;
  int rtype, flags;
  float sttc, sttp, sttl, sttb, sttk, i0, fl0, dl0, fl20, dl20;  // sttc carries dt (dt/6 for RK4)
  float sigc, t0, sig;  // sig = sqrt(sigc * t0): the thermal scale at constant T
  uint32_t seed_lo, seed_hi;
  uint64_t nstep0;

  // rk4: load the dt/6 prefactors (k' = k/6), else the dt ones
  __device__ __forceinline__ void load(const cmtj_f32_layer_t &r, bool rk4) {
    using F = Feat<FEAT>;
    a = ld3(r.anis);
    kc = r.kc;
    k2c = F::k2 ? r.k2c : 0.f;
    if (F::full_demag) {
#pragma unroll
      for (int q = 0; q < 9; ++q) N[q] = r.demag[q];
    } else {
      N[0] = r.demag[0];
      N[4] = r.demag[4];
      N[8] = r.demag[8];
    }
    if (F::dipole) {
#pragma unroll
      for (int q = 0; q < 9; ++q) {
        Db[q] = r.dip_b[q];
        Dt[q] = r.dip_t[q];
      }
    }
    h0 = ld3(r.h0);
    jb = r.jb;
    jt = r.jt;
    j2b = r.j2b;
    j2t = r.j2t;
    if (F::idmi) {
      dmib = ld3(r.dmi_b);
      dmit = ld3(r.dmi_t);
    }
    gam = r.gam;
    gdt = rk4 ? r.gdt6 : r.gdt;
    alpha = r.alpha;
    rtype = r.ref_type;
    flags = r.flags;
    if (F::stt || F::sot) {
      ref = ld3(r.ref);
      ref2 = ld3(r.ref2);
      sttc = rk4 ? r.stt_cdt6 : r.stt_cdt;
      sttp = r.stt_p;
      sttl = r.stt_l;
      sttb = r.stt_beta;
      sttk = r.stt_kappa;
      i0 = r.i0;
      fl0 = r.fl0;
      dl0 = r.dl0;
      fl20 = r.fl20;
      dl20 = r.dl20;
    }
    if (F::diag) {
      M = f3(fmaf(kc * a.x, a.x, -N[0]), fmaf(kc * a.y, a.y, -N[4]), fmaf(kc * a.z, a.z, -N[8]));
    }
    if (F::prescale) {
      h0 = h0 * gdt;
      jb *= gdt;
      jt *= gdt;
      j2b *= gdt;
      j2t *= gdt;
      if (F::diag) {
        M = M * gdt;
      } else {
        kc *= gdt;
        k2c *= gdt;
        if (F::full_demag) {
#pragma unroll
          for (int q = 0; q < 9; ++q) N[q] *= gdt;
        } else {
          N[0] *= gdt;
          N[4] *= gdt;
          N[8] *= gdt;
        }
      }
      if (F::dipole) {
#pragma unroll
        for (int q = 0; q < 9; ++q) {
          Db[q] *= gdt;
          Dt[q] *= gdt;
        }
      }
      if (F::idmi) {
        dmib = dmib * gdt;
        dmit = dmit * gdt;
      }
    }
    sigc = r.sig_c;
    t0 = r.t0;
    sig = sqrtf(fmaxf(sigc * t0, 0.f));
    seed_lo = r.seed_lo;
    seed_hi = r.seed_hi;
    nstep0 = ((uint64_t)r.noise_step_hi << 32) | r.noise_step_lo;
  }
};

// Time-dependent additions to one layer's terms at one stage time.  Only
// the targets the variant supports are kept (the host routes any other wave
// to a variant that has them), so unused fields cost no registers.
template <int FEAT> struct Delta {
  using F = Feat<FEAT>;
  F3 dH;
  float dK, dK2, dJb, dJt, dJ2b, dJ2t, dI, dFL, dDL, dFL2, dDL2, dT;
  // dH starts at the layer's constant field h0, so the right-hand side
  // reads the whole field from it without a separate add
  __device__ __forceinline__ void clear(F3 h0) {
    dH = h0;
    dK = dK2 = dJb = dJt = dJ2b = dJ2t = dI = dFL = dDL = dFL2 = dDL2 = dT = 0.f;
  }
  __device__ __forceinline__ void add(int target, float v) {
    if (target == CMTJ_TGT_HX) dH.x += v;
    else if (target == CMTJ_TGT_HY) dH.y += v;
    else if (target == CMTJ_TGT_HZ) dH.z += v;
    else if (F::twaves && target == CMTJ_TGT_I) dI += v;
    else if (F::twaves && F::sot && target == CMTJ_TGT_FL) dFL += v;
    else if (F::twaves && F::sot && target == CMTJ_TGT_DL) dDL += v;
    else if (F::twaves && F::sot && target == CMTJ_TGT_FL2) dFL2 += v;
    else if (F::twaves && F::sot && target == CMTJ_TGT_DL2) dDL2 += v;
    else if (F::swaves) {
      switch (target) {
      case CMTJ_TGT_K: dK += v; break;
      case CMTJ_TGT_K2: dK2 += v; break;
      case CMTJ_TGT_JB: dJb += v; break;
      case CMTJ_TGT_JT: dJt += v; break;
      case CMTJ_TGT_J2B: dJ2b += v; break;
      case CMTJ_TGT_J2T: dJ2t += v; break;
      case CMTJ_TGT_T: dT += v; break;
      default: break;
      }
    }
  }
};

// One time-dependent driver in registers.
template <int L> struct WaveR {
  int target, kind;
  bool field;   // targets HX/HY/HZ: added as hdir[l] * u, no target dispatch
  float amp[L];
  F3 hdir[L];
  float p0, p1, p2;
  uint32_t thr32;
  int32_t i0;
  uint64_t ph0, dph, dphh;
  uint32_t on0, off0, on1, off1, on2, off2;

  // hscale[l]: factor on layer l's field contributions (its gamma dt
  // prefactor when the variant pre-scales fields, else 1)
  __device__ __forceinline__ void load(const cmtj_wave_t &w, const float *hscale) {
    target = w.target;
    kind = w.kind;
    field = target <= CMTJ_TGT_HZ;
#pragma unroll
    for (int l = 0; l < L; ++l) {
      amp[l] = ((w.layer_mask >> l) & 1) ? w.amp : 0.f;
      const float h = amp[l] * hscale[l];
      hdir[l] = f3(target == CMTJ_TGT_HX ? h : 0.f, target == CMTJ_TGT_HY ? h : 0.f, target == CMTJ_TGT_HZ ? h : 0.f);
    }
    p0 = w.p0;
    p1 = w.p1;
    p2 = w.p2;
    thr32 = w.thr32;
    i0 = w.i0;
    ph0 = w.ph0;
    dph = w.dph;
    dphh = w.dph_half;
    on0 = w.on[0];
    off0 = w.off[0];
    on1 = w.on[1];
    off1 = w.off[1];
    on2 = w.on[2];
    off2 = w.off[2];
  }

  // True when the waveform is 0 at every stage of steps [i0_, i1_): a step
  // driver whose stage windows [on_s, off_s] all miss that range.
  __device__ __forceinline__ bool off_during(uint32_t i0_, uint32_t i1_) const {
    if (kind != CMTJ_WAVE_STEP || i1_ <= i0_) return false;
    const uint32_t lo = min(on0, min(on1, on2)), hi = max(off0, max(off1, off2));
    return i1_ - 1u < lo || i0_ > hi;
  }

  // Unit waveform at step i, stage s (0: t, 1: t + dt/2, 2: t + dt).
  __device__ __forceinline__ float unit(uint32_t i, int s, float dtf) const {
    switch (kind) {
    case CMTJ_WAVE_SINE:
    case CMTJ_WAVE_POSINE:
    case CMTJ_WAVE_HALFSINE: {
      const uint64_t ph = ph0 + (uint64_t)i * dph + (s == 0 ? 0ull : (s == 1 ? dphh : dph));
      const float v = sin2pi_phase(ph);
      if (kind == CMTJ_WAVE_POSINE) return fabsf(v);
      if (kind == CMTJ_WAVE_HALFSINE) return (p0 * v <= 0.f) ? v : 0.f;
      return v;
    }
    case CMTJ_WAVE_PULSE: {
      const uint64_t ph = ph0 + (uint64_t)i * dph + (s == 0 ? 0ull : (s == 1 ? dphh : dph));
      return ((uint32_t)(ph >> 32) <= thr32) ? 1.f : 0.f;
    }
    case CMTJ_WAVE_STEP: {
      const uint32_t on = s == 0 ? on0 : (s == 1 ? on1 : on2);
      const uint32_t off = s == 0 ? off0 : (s == 1 ? off1 : off2);
      return (i >= on && i <= off) ? 1.f : 0.f;
    }
    default: {
      const float tau = fmaf((float)((int32_t)i - i0), dtf, fmaf((float)s, 0.5f * dtf, p2));
      if (kind == CMTJ_WAVE_TRAPEZOID) {
        if (tau < 0.f) return 0.f;
        if (tau <= p0) return tau / p0;
        if (tau <= p0 + p1) return 1.f;
        if (tau <= 2.f * p0 + p1) return 1.f - (tau - (p0 + p1)) / p0;
        return 0.f;
      }
      if (kind == CMTJ_WAVE_GAUSSIMPULSE) {
        const float u = tau * p0;
        return __expf(-0.5f * u * u);
      }
      return 0.5f * (1.f + erff(tau * p0));  // GAUSSSTEP
    }
    }
  }
};

// Adds wave w's value at (step, stage) to every layer's deltas.  Variants
// without scalar or torque waves only ever see field waves (the host routes
// others elsewhere), so they take the branch-free field path.
template <int L, int FEAT>
__device__ __forceinline__ void add_wave(const WaveR<L> &w, uint32_t step, int s, float dtf, Delta<FEAT> *d) {
  using F = Feat<FEAT>;
  const float u = w.unit(step, s, dtf);
  if (!(F::swaves || F::twaves) || w.field) {
#pragma unroll
    for (int l = 0; l < L; ++l) d[l].dH = fma3(w.hdir[l], u, d[l].dH);
  } else {
#pragma unroll
    for (int l = 0; l < L; ++l) d[l].add(w.target, w.amp[l] * u);
  }
}

// The part of one layer's effective field that does not depend on its own
// m (junction.hpp:590-622, 654-701): the constant + wave field, then the
// neighbour terms (bilinear IEC, IDMI, dipole) from the neighbour
// magnetisations mb / mt.  The RK4 runner freezes neighbours for the whole
// step (junction.hpp:1682-1707), so this sum is formed once per stage time,
// not once per stage.  Quadratic IEC depends on m and stays in rhs().
template <int FEAT, bool HB, bool HT>
__device__ __forceinline__ F3 hbase(const LayerP<FEAT> &P, F3 mb, F3 mt, const Delta<FEAT> &d) {
  using F = Feat<FEAT>;
  F3 H = F::waves ? d.dH : P.h0;
  if (HB) {
    if (!F::iec2) H = fma3(mb, F::swaves ? P.jb + d.dJb : P.jb, H);
    if (F::idmi) H = H + cross(mb, P.dmib);
    if (F::dipole) H = H - matvec(P.Db, mb);
  }
  if (HT) {
    if (!F::iec2) H = fma3(mt, F::swaves ? P.jt + d.dJt : P.jt, H);
    if (F::idmi) H = H + cross(mt, P.dmit);
    if (F::dipole) H = H - matvec(P.Dt, mt);
  }
  return H;
}

// Effective field + LL torque of one layer (junction.hpp:580-815) given its
// hbase() sum H, returned already multiplied by dt (Euler-Heun, Heun: f dt)
// or by dt/6 (RK4: k/6).
template <int FEAT, bool HB, bool HT>
__device__ __forceinline__ F3 rhs(const LayerP<FEAT> &P, F3 m, F3 mb, F3 mt, const Delta<FEAT> &d, F3 H) {
  using F = Feat<FEAT>;
  if (F::diag) {
    H = f3(fmaf(P.M.x, m.x, H.x), fmaf(P.M.y, m.y, H.y), fmaf(P.M.z, m.z, H.z));
  } else {
    const float da = dot(P.a, m);
    float ka = F::swaves ? P.kc + d.dK : P.kc;
    if (F::k2) ka = fmaf(F::swaves ? P.k2c + d.dK2 : P.k2c, da * da, ka);
    H = fma3(P.a, ka * da, H);
  }
  if (F::iec2) {
    if (HB) {
      const float jb = F::swaves ? P.jb + d.dJb : P.jb;
      H = fma3(mb, fmaf(F::swaves ? P.j2b + d.dJ2b : P.j2b, dot(mb, m), jb), H);
    }
    if (HT) {
      const float jt = F::swaves ? P.jt + d.dJt : P.jt;
      H = fma3(mt, fmaf(F::swaves ? P.j2t + d.dJ2t : P.j2t, dot(mt, m), jt), H);
    }
  }
  if (F::full_demag) {
    H = H - matvec(P.N, m);
  } else if (!F::diag) {
    H = f3(fmaf(-P.N[0], m.x, H.x), fmaf(-P.N[4], m.y, H.y), fmaf(-P.N[8], m.z, H.z));
  }
  const F3 mxH = cross(m, H);
  F3 acc = fma3(cross(m, mxH), P.alpha, mxH);
  if (F::stt || F::sot) {
    F3 p = P.ref;
    if (P.rtype == CMTJ_REF_TOP) p = HT ? mt : f3(0.f, 0.f, 0.f);
    else if (P.rtype == CMTJ_REF_BOTTOM) p = HB ? mb : f3(0.f, 0.f, 0.f);
    else if (P.rtype == CMTJ_REF_NONE) p = f3(0.f, 0.f, 0.f);
    if (F::stt && (P.flags & CMTJ_F32_STT)) {
      const float I = F::twaves ? P.i0 + d.dI : P.i0;
      const float mp = dot(m, p);
      float eta;
      if (P.flags & CMTJ_F32_ALT_STT) {
        eta = __fdividef(P.sttp, fmaf(P.sttl, mp, 1.f));
      } else {
        const float l2 = P.sttl * P.sttl;
        eta = __fdividef(P.sttp * l2, fmaf(l2 - 1.f, mp, l2 + 1.f));
      }
      const float s = P.sttc * I * eta;
      const F3 fl = cross(m, p);
      const F3 dl = cross(m, fl);
      // gdt carries -gamma dt/(1+alpha^2), sttc dt/(1+alpha^2) (each /6 for RK4).
      return fma3(fl, s * P.sttb, fma3(dl, -s * P.sttk, F::prescale ? acc : acc * P.gdt));
    }
    if (F::sot && (P.flags & CMTJ_F32_SOT)) {
      float hfl, hdl, hfl2 = 0.f, hdl2 = 0.f;
      if (P.flags & CMTJ_F32_SOT_STATIC) {
        const float I = F::twaves ? P.i0 + d.dI : P.i0;
        hfl = P.fl0 * I;
        hdl = P.dl0 * I;
      } else {
        hfl = F::twaves ? P.fl0 + d.dFL : P.fl0;
        hdl = F::twaves ? P.dl0 + d.dDL : P.dl0;
        hfl2 = F::twaves ? P.fl20 + d.dFL2 : P.fl20;
        hdl2 = F::twaves ? P.dl20 + d.dDL2 : P.dl20;
      }
      const F3 cp = cross(m, p);
      acc = fma3(cp, fmaf(-P.alpha, hdl, hfl), acc);
      acc = fma3(cross(m, cp), fmaf(P.alpha, hfl, hdl), acc);
      const F3 cs = cross(m, P.ref2);
      acc = fma3(cs, fmaf(-P.alpha, hdl2, hfl2), acc);
      acc = fma3(cross(m, cs), fmaf(P.alpha, hfl2, hdl2), acc);
    }
  }
  return F::prescale ? acc : acc * P.gdt;
}

// stochasticTorque (junction.hpp:824-831).
template <int FEAT>
__device__ __forceinline__ F3 stoch(const LayerP<FEAT> &P, F3 m, F3 dW) {
  const F3 th = cross(m, dW);
  return fma3(cross(m, th), P.alpha, th) * P.gam;
}

// Layer l of an L-layer stack: which neighbours it has (edge layers see a
// zero vector, junction.hpp:1686-1695).
template <int L, int FEAT>
__device__ __forceinline__ F3 hbase_at(int l, const LayerP<FEAT> &P, F3 mb, F3 mt, const Delta<FEAT> &d) {
  if (L == 1) return hbase<FEAT, false, false>(P, mb, mt, d);
  if (l == 0) return hbase<FEAT, false, true>(P, mb, mt, d);
  if (l == L - 1) return hbase<FEAT, true, false>(P, mb, mt, d);
  return hbase<FEAT, true, true>(P, mb, mt, d);
}
template <int L, int FEAT>
__device__ __forceinline__ F3 rhs_at(int l, const LayerP<FEAT> &P, F3 m, F3 mb, F3 mt, const Delta<FEAT> &d, F3 H) {
  if (L == 1) return rhs<FEAT, false, false>(P, m, mb, mt, d, H);
  if (l == 0) return rhs<FEAT, false, true>(P, m, mb, mt, d, H);
  if (l == L - 1) return rhs<FEAT, true, false>(P, m, mb, mt, d, H);
  return rhs<FEAT, true, true>(P, m, mb, mt, d, H);
}

// ---- Packed two-layer form.  A 2-layer junction runs both layers through
// the same arithmetic, so each float2 holds (layer 0, layer 1) and every
// vector operation is one packed FFMA2 / FMUL2 / FADD2 instead of two
// scalar ones: half the issue slots for the same FMA-pipe work.  Each lane
// repeats the scalar path's operations in the same order, so both forms give
// the same bits.
struct V2 {
  float2 x, y, z;
};
__device__ __forceinline__ float2 bc2(float s) { return make_float2(s, s); }
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ V2 v2(float2 x, float2 y, float2 z) {
  V2 r;
  r.x = x;
  r.y = y;
  r.z = z;
  return r;
}
__device__ __forceinline__ V2 pack2(F3 a, F3 b) {
  return v2(make_float2(a.x, b.x), make_float2(a.y, b.y), make_float2(a.z, b.z));
}
__device__ __forceinline__ F3 lane0(V2 v) { return f3(v.x.x, v.y.x, v.z.x); }
__device__ __forceinline__ F3 lane1(V2 v) { return f3(v.x.y, v.y.y, v.z.y); }
__device__ __forceinline__ V2 swap2(V2 v) {
  return v2(make_float2(v.x.y, v.x.x), make_float2(v.y.y, v.y.x), make_float2(v.z.y, v.z.x));
}
__device__ __forceinline__ V2 v2add(V2 a, V2 b) {
  return v2(__fadd2_rn(a.x, b.x), __fadd2_rn(a.y, b.y), __fadd2_rn(a.z, b.z));
}
__device__ __forceinline__ V2 v2mul(V2 a, float2 s) {
  return v2(__fmul2_rn(a.x, s), __fmul2_rn(a.y, s), __fmul2_rn(a.z, s));
}
// a * s + b, s per layer
__device__ __forceinline__ V2 v2fma(V2 a, float2 s, V2 b) {
  return v2(__ffma2_rn(a.x, s, b.x), __ffma2_rn(a.y, s, b.y), __ffma2_rn(a.z, s, b.z));
}
// a * s + b componentwise
__device__ __forceinline__ V2 v2fmav(V2 a, V2 s, V2 b) {
  return v2(__ffma2_rn(a.x, s.x, b.x), __ffma2_rn(a.y, s.y, b.y), __ffma2_rn(a.z, s.z, b.z));
}
__device__ __forceinline__ float2 v2dot(V2 a, V2 b) {
  return __ffma2_rn(a.x, b.x, __ffma2_rn(a.y, b.y, __fmul2_rn(a.z, b.z)));
}
__device__ __forceinline__ V2 v2cross(V2 a, V2 b) {
  return v2(__ffma2_rn(a.y, b.z, neg2(__fmul2_rn(a.z, b.y))), __ffma2_rn(a.z, b.x, neg2(__fmul2_rn(a.x, b.z))),
            __ffma2_rn(a.x, b.y, neg2(__fmul2_rn(a.y, b.x))));
}
__device__ __forceinline__ V2 v2renorm(V2 m) {
  const float2 q = v2dot(m, m);
  return v2mul(m, make_float2(rsqrtf(q.x), rsqrtf(q.y)));
}

// Constants of a layer pair (layers 2p, 2p+1) of a junction whose variant
// has only the constant field, field waves, uniaxial anisotropy, diagonal
// demag and bilinear IEC, with every field term pre-scaled by the layer's
// gamma dt prefactor (LayerP with Feat::prescale).  DIAG: the anisotropy
// axis lies on a coordinate axis and folds with the demag into M.  A pair
// whose second layer does not exist (an odd layer count) carries a pad lane
// with every coefficient zero: its m = (0, 0, 1) never moves.
template <bool DIAG> struct PairC {
  V2 A;          // DIAG: folded tensor M; else the anisotropy axis a
  V2 nN;         // !DIAG: -diag(N)
  V2 h0;         // constant field
  float2 kc;     // !DIAG: anisotropy coefficient
  float2 alpha;
  float2 jb, jt; // IEC coefficient of each lane's bottom / top neighbour (0 at an edge)
  template <int FEAT, int L>
  __device__ __forceinline__ void load(const LayerP<FEAT> *P, int p) {
    const int l0 = 2 * p, l1 = 2 * p + 1;
    const bool has1 = l1 < L;
    const F3 z = f3(0.f, 0.f, 0.f);
    if (DIAG) {
      A = pack2(P[l0].M, has1 ? P[l1].M : z);
    } else {
      A = pack2(P[l0].a, has1 ? P[l1].a : z);
      nN = pack2(f3(-P[l0].N[0], -P[l0].N[4], -P[l0].N[8]),
                 has1 ? f3(-P[l1].N[0], -P[l1].N[4], -P[l1].N[8]) : z);
      kc = make_float2(P[l0].kc, has1 ? P[l1].kc : 0.f);
    }
    h0 = pack2(P[l0].h0, has1 ? P[l1].h0 : z);
    alpha = make_float2(P[l0].alpha, has1 ? P[l1].alpha : 0.f);
    jb = make_float2(l0 > 0 ? P[l0].jb : 0.f, has1 ? P[l1].jb : 0.f);
    jt = make_float2(has1 ? P[l0].jt : 0.f, (has1 && l1 + 1 < L) ? P[l1].jt : 0.f);
  }
};

// rhs() of both lanes of a pair, given their hbase() sums.
template <bool DIAG>
__device__ __forceinline__ V2 rhs2(const PairC<DIAG> &Q, V2 m, V2 H) {
  if (DIAG) {
    H = v2fmav(Q.A, m, H);
  } else {
    const float2 da = v2dot(Q.A, m);
    H = v2fma(Q.A, __fmul2_rn(Q.kc, da), H);
    H = v2fmav(Q.nN, m, H);
  }
  const V2 mxH = v2cross(m, H);
  return v2fma(v2cross(m, mxH), Q.alpha, mxH);
}

// One packed RK4 step of a 2-layer junction (the scalar RK4 of k_batch,
// lane by lane): the two layers are each other's only neighbour, so the
// neighbour vector is the swapped pair.  WAVES: evaluate the waves at the
// three stage times; otherwise the field base is time-independent and
// formed once.
template <bool DIAG, bool WAVES, int NW>
__device__ __forceinline__ void packed_rk4_step(V2 &mp, const PairC<DIAG> &Q, const WaveR<2> *W, const V2 *HD,
                                                int nw, uint32_t step, float dtf) {
  const V2 nb = swap2(mp);  // frozen neighbours: layer 0 sees layer 1, layer 1 sees layer 0
  const float2 jn = make_float2(Q.jt.x, Q.jb.y);
  V2 hb = v2fma(nb, jn, Q.h0), acc, kp;
#pragma unroll
  for (int st = 0; st < 4; ++st) {
    const int s = st == 0 ? 0 : (st == 3 ? 2 : 1);
    if (WAVES && st != 2) {
      hb = Q.h0;
#pragma unroll
      for (int w = 0; w < NW; ++w)
        if (w < nw) hb = v2fma(HD[w], bc2(W[w].unit(step, s, dtf)), hb);
      hb = v2fma(nb, jn, hb);
    }
    const V2 ms = st == 0 ? mp : v2fma(kp, bc2(st == 3 ? 6.f : 3.f), mp);
    kp = rhs2<DIAG>(Q, ms, hb);
    if (st == 0) acc = kp;
    else if (st == 3) acc = v2add(acc, kp);
    else acc = v2fma(kp, bc2(2.f), acc);
  }
  mp = v2renorm(v2add(mp, acc));
}

// One packed RK4 step of a 3- or 4-layer junction as NP layer pairs.  Lane 0
// of pair p is layer 2p (bottom neighbour: lane 1 of pair p-1, top: lane 1
// of pair p); lane 1 is layer 2p+1 (bottom: lane 0 of pair p, top: lane 0
// of pair p+1).  Neighbour terms add bottom then top, as hbase() does.
template <int L, bool DIAG, bool WAVES, int NW>
__device__ __forceinline__ void packed_rk4_step_pairs(V2 *mp, const PairC<DIAG> *Q, const WaveR<L> *W,
                                                      const V2 (*HD)[(L + 1) / 2], int nw, uint32_t step,
                                                      float dtf) {
  constexpr int NP = (L + 1) / 2;
  V2 nbB[NP], nbT[NP], hb[NP], acc[NP], kp[NP];
#pragma unroll
  for (int q = 0; q < NP; ++q) {
    const V2 below = q > 0 ? mp[q - 1] : v2(bc2(0.f), bc2(0.f), bc2(0.f));
    const V2 above = q + 1 < NP ? mp[q + 1] : v2(bc2(0.f), bc2(0.f), bc2(0.f));
    nbB[q] = v2(make_float2(below.x.y, mp[q].x.x), make_float2(below.y.y, mp[q].y.x),
                make_float2(below.z.y, mp[q].z.x));
    nbT[q] = v2(make_float2(mp[q].x.y, above.x.x), make_float2(mp[q].y.y, above.y.x),
                make_float2(mp[q].z.y, above.z.x));
    hb[q] = v2fma(nbT[q], Q[q].jt, v2fma(nbB[q], Q[q].jb, Q[q].h0));
  }
#pragma unroll
  for (int st = 0; st < 4; ++st) {
    const int s = st == 0 ? 0 : (st == 3 ? 2 : 1);
    if (WAVES && st != 2) {
      float u[NW];  // each waveform once per stage time, shared by the pairs
#pragma unroll
      for (int w = 0; w < NW; ++w) u[w] = w < nw ? W[w].unit(step, s, dtf) : 0.f;
#pragma unroll
      for (int q = 0; q < NP; ++q) {
        V2 h = Q[q].h0;
#pragma unroll
        for (int w = 0; w < NW; ++w)
          if (w < nw) h = v2fma(HD[w][q], bc2(u[w]), h);
        hb[q] = v2fma(nbT[q], Q[q].jt, v2fma(nbB[q], Q[q].jb, h));
      }
    }
#pragma unroll
    for (int q = 0; q < NP; ++q) {
      const V2 ms = st == 0 ? mp[q] : v2fma(kp[q], bc2(st == 3 ? 6.f : 3.f), mp[q]);
      kp[q] = rhs2<DIAG>(Q[q], ms, hb[q]);
      if (st == 0) acc[q] = kp[q];
      else if (st == 3) acc[q] = v2add(acc[q], kp[q]);
      else acc[q] = v2fma(kp[q], bc2(2.f), acc[q]);
    }
  }
#pragma unroll
  for (int q = 0; q < NP; ++q) mp[q] = v2renorm(v2add(mp[q], acc[q]));
}

struct Args {
  const cmtj_f32_junction_t *J;
  const cmtj_f32_layer_t *Ly;
  cmtj_f32_state_t *S;
  const int32_t *order;
  int32_t n;
  cmtj_f32_params_t p;
  float *log;
  uint32_t *ticket;
};

__device__ __forceinline__ void bulk_store(float *gdst, const float *ssrc, uint32_t bytes) {
  // Generic-proxy writes to shared memory must be visible to the async proxy.
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  const uint32_t s = (uint32_t)__cvta_generic_to_shared(ssrc);
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(gdst), "r"(s), "r"(bytes)
               : "memory");
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}
__device__ __forceinline__ void bulk_wait_read() {
  asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}

// Resistance of one junction: CLASSIC R = Rp + (Rap - Rp)/2 (1 - cos)
// (junction.hpp:1865-1867, cos against layer 1 or the layer-0 reference),
// STRIP Rx = 1 / sum_l 1/(Rx0 + AMR_X mx^2 + SMR_X my^2) (1835-1857), SERIES
// Rx = sum_l (Rx0 + AMR_X mx^2 + SMR_X my^2) (cmtj/utils/resistance.py:121-150).
template <int L>
__device__ __forceinline__ float resistance(const cmtj_f32_junction_t *J, const float *ref0, const F3 *m) {
  const int mr = J->mr_mode;
  if (mr == CMTJ_MR_CLASSIC) {
    const F3 other = L > 1 ? m[L > 1 ? 1 : 0] : ld3(ref0);
    return fmaf((J->Rap - J->Rp) * 0.5f, 1.f - dot(m[0], other), J->Rp);
  }
  float acc = 0.f;
  if (mr == CMTJ_MR_SERIES) {
#pragma unroll
    for (int l = 0; l < L; ++l)
      acc += fmaf(J->AMR_X[l], m[l].x * m[l].x, fmaf(J->SMR_X[l], m[l].y * m[l].y, J->Rx0[l]));
    return acc;
  }
#pragma unroll
  for (int l = 0; l < L; ++l)
    acc += 1.f / fmaf(J->AMR_X[l], m[l].x * m[l].x, fmaf(J->SMR_X[l], m[l].y * m[l].y, J->Rx0[l]));
  return 1.f / acc;
}

// Constants of the on-device reductions, cached per thread in shared memory
// when its junction is loaded, word k of thread t at rk[k * kRedStride + t]:
// a warp reads 32 consecutive words, one wavefront.  Read from the junction
// records instead (536 B apart, in length order) every load of a warp
// gathers 32 cache lines, and with R reduced every step those gathers kept
// the L1 busy.  Words: 0 MR mode; CLASSIC 1 (Rap - Rp) / 2, 2 Rp, 3-5 the
// layer-0 reference (1 layer); SERIES / STRIP 1 + 3l, 2 + 3l, 3 + 3l
// AMR_X, SMR_X, Rx0 of layer l; then vsd_ph0, vsd_dph (low, high words)
// and red_total.  Integers are stored as their bits.
constexpr int kRedStride = 128;  // threads per CTA of k_batch
template <int L> __host__ __device__ constexpr int red_mr_words() { return 1 + (3 * L > 5 ? 3 * L : 5); }
template <int L> __host__ __device__ constexpr int red_words() { return red_mr_words<L>() + 5; }

template <int L>
__device__ __forceinline__ void red_cache(float *rk, const cmtj_f32_junction_t &J, const float *ref0) {
  const int mr = J.mr_mode;
  rk[0] = __int_as_float(mr);
  if (mr == CMTJ_MR_CLASSIC) {
    rk[1 * kRedStride] = (J.Rap - J.Rp) * 0.5f;
    rk[2 * kRedStride] = J.Rp;
    if (L == 1) {
      rk[3 * kRedStride] = ref0[0];
      rk[4 * kRedStride] = ref0[1];
      rk[5 * kRedStride] = ref0[2];
    }
  } else {
#pragma unroll
    for (int l = 0; l < L; ++l) {
      rk[(1 + 3 * l) * kRedStride] = J.AMR_X[l];
      rk[(2 + 3 * l) * kRedStride] = J.SMR_X[l];
      rk[(3 + 3 * l) * kRedStride] = J.Rx0[l];
    }
  }
  constexpr int b = red_mr_words<L>();
  rk[b * kRedStride] = __uint_as_float((uint32_t)J.vsd_ph0);
  rk[(b + 1) * kRedStride] = __uint_as_float((uint32_t)(J.vsd_ph0 >> 32));
  rk[(b + 2) * kRedStride] = __uint_as_float((uint32_t)J.vsd_dph);
  rk[(b + 3) * kRedStride] = __uint_as_float((uint32_t)(J.vsd_dph >> 32));
  rk[(b + 4) * kRedStride] = __uint_as_float(J.red_total);
}
__device__ __forceinline__ uint64_t red_u64(const float *rk, int k) {
  return ((uint64_t)__float_as_uint(rk[(k + 1) * kRedStride]) << 32) | __float_as_uint(rk[k * kRedStride]);
}

// resistance() on the cached constants: the same operations in the same
// order, so the same bits.
template <int L> __device__ __forceinline__ float resistance_cached(const float *rk, const F3 *m) {
  const int mr = __float_as_int(rk[0]);
  if (mr == CMTJ_MR_CLASSIC) {
    const F3 other = L > 1 ? m[L > 1 ? 1 : 0] : f3(rk[3 * kRedStride], rk[4 * kRedStride], rk[5 * kRedStride]);
    return fmaf(rk[1 * kRedStride], 1.f - dot(m[0], other), rk[2 * kRedStride]);
  }
  float acc = 0.f;
  if (mr == CMTJ_MR_SERIES) {
#pragma unroll
    for (int l = 0; l < L; ++l)
      acc += fmaf(rk[(1 + 3 * l) * kRedStride], m[l].x * m[l].x,
                  fmaf(rk[(2 + 3 * l) * kRedStride], m[l].y * m[l].y, rk[(3 + 3 * l) * kRedStride]));
    return acc;
  }
#pragma unroll
  for (int l = 0; l < L; ++l)
    acc += 1.f / fmaf(rk[(1 + 3 * l) * kRedStride], m[l].x * m[l].x,
                      fmaf(rk[(2 + 3 * l) * kRedStride], m[l].y * m[l].y, rk[(3 + 3 * l) * kRedStride]));
  return 1.f / acc;
}

template <int L> __device__ __forceinline__ int log_channels(int mode) {
  return mode == CMTJ_LOG_M ? 3 * L : (mode == CMTJ_LOG_NONE ? 0 : 1);
}

// Resident CTAs of 128 threads per SM the specialised variants are built
// for (register cap); the catch-all CMTJ_FEAT_ALL variants take what they
// need.  The packed two-layer RK4 variants have their own bound.
#ifndef CMTJ_BATCH_MINB
#define CMTJ_BATCH_MINB 5
#endif
#ifndef CMTJ_BATCH_MINB_PACKED
#define CMTJ_BATCH_MINB_PACKED CMTJ_BATCH_MINB
#endif
#ifndef CMTJ_BATCH_MINB_STOCH
#define CMTJ_BATCH_MINB_STOCH 4  // Euler-Heun / Heun variants (the p-bit sweep: 4 beat 5 and 6 by 6-7 %)
#endif
#ifndef CMTJ_BATCH_MINB_WIDE
#define CMTJ_BATCH_MINB_WIDE 2  // packed 3- and 4-layer variants (best of 2/3/4/5 measured)
#endif

// Layer-packed RK4: 2-4 layers, only constant / wave fields, uniaxial
// anisotropy (on an axis or off it), diagonal demag and bilinear IEC.
template <int L, int SOLVER, int FEAT>
__host__ __device__ constexpr bool packed_variant() {
  return L >= 2 && SOLVER == CMTJ_RK4 && (FEAT & ~(CMTJ_FEAT_WAVES | CMTJ_FEAT_OFFAXIS)) == 0;
}
template <int L, int SOLVER, int FEAT>
__host__ __device__ constexpr int min_blocks() {
  return FEAT == CMTJ_FEAT_ALL ? 1
         : (packed_variant<L, SOLVER, FEAT>() ? (L == 2 ? CMTJ_BATCH_MINB_PACKED : CMTJ_BATCH_MINB_WIDE)
                                               : (SOLVER == CMTJ_RK4 ? CMTJ_BATCH_MINB : CMTJ_BATCH_MINB_STOCH));
}

// The second, lower-occupancy instantiation of every specialised variant:
// fewer resident CTAs per SM, so more registers per thread.  A batch too
// small to fill the GPU gains from it; the run-time autotuner
// (cmtj_gb300/autotune.py) picks between the two per partition.
template <int L, int SOLVER, int FEAT>
__host__ __device__ constexpr int low_min_blocks() {
  return packed_variant<L, SOLVER, FEAT>() && L > 2 ? 1 : 2;
}

// MB > 0 overrides the variant's resident-CTA bound.
template <int L, int SOLVER, int FEAT, int NW, int MB = 0>
__global__ void __launch_bounds__(128, (MB > 0 ? MB : min_blocks<L, SOLVER, FEAT>())) k_batch(Args A) {
  using F = Feat<FEAT>;
  extern __shared__ __align__(16) float smem[];
  const int lane = threadIdx.x & 31;
  const cmtj_f32_params_t &p = A.p;
  const float dtf = (float)p.dt;
  const float sqdt = (float)sqrt(p.dt);
  const int C = log_channels<L>(p.log_mode);
  const uint32_t T = p.log_tile;
  // shared memory per thread: its log tile; after all tiles, when
  // p.red_weights is set, the (sum, compensation) pair of the weighted sum;
  // then, when reducing, the reduction constants (red_cache, one column per
  // thread)
  const uint32_t tile_floats = C > 0 ? T * (uint32_t)C : 1u;
  float *tile = smem + (size_t)threadIdx.x * tile_floats;
  float *wsum = smem + (size_t)blockDim.x * tile_floats + 2u * threadIdx.x;
  float *rk = smem + (size_t)blockDim.x * (tile_floats + (p.red_weights ? 2u : 0u)) + threadIdx.x;

  // Packed two-layer RK4 for the variants with only constant / wave fields,
  // uniaxial anisotropy, diagonal demag and bilinear IEC.
  constexpr bool kPacked = packed_variant<L, SOLVER, FEAT>();
  constexpr bool kDiag = Feat<FEAT>::diag;
  constexpr int NP = (L + 1) / 2;  // layer pairs of the packed path
  static_assert(!kPacked || Feat<FEAT>::prescale, "the packed path reads pre-scaled fields");

  // junction-lifetime registers
  LayerP<FEAT> P[L];
  WaveR<L> W[NW > 0 ? NW : 1];
  PairC<kDiag> Q[NP];                  // kPacked: each layer pair's constants
  V2 HD[NW > 0 ? NW : 1][NP];          // kPacked: each wave's field direction x amplitude, per pair
  int nw = 0;
  F3 m[L];
  int32_t jid = -1;
  bool retired = false;
  uint32_t step = 0, end = 0, stop_all = 0, n_logged = 0, tcount = 0, n_red = 0, win = 0;
  uint32_t next_log = 0xffffffffu, next_red = 0xffffffffu;  // next steps that log / reduce
  // junction constants used only when logging or reducing stay in the
  // record (read through L1 when needed), not in registers
  const cmtj_f32_junction_t *Jp = nullptr;
  const float *ref0 = nullptr;
  float rs = 0.f, rc = 0.f, vs = 0.f, vc = 0.f;
  float *logrow = nullptr;

  for (;;) {
    // ---- refill lanes that have no junction (warp-aggregated ticket)
    const bool need = (jid < 0) && !retired;
    const unsigned needmask = __ballot_sync(0xffffffffu, need);
    if (needmask) {
      const int leader = __ffs(needmask) - 1;
      uint32_t base = 0;
      if (lane == leader) base = atomicAdd(A.ticket, (uint32_t)__popc(needmask));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (need) {
        const uint32_t k = base + __popc(needmask & ((1u << lane) - 1u));
        if (k >= (uint32_t)A.n) {
          retired = true;
        } else {
          jid = A.order[k];
          const cmtj_f32_junction_t &J = A.J[jid];
          const cmtj_f32_state_t &S = A.S[jid];
          if (J.n_layers != L) {
            // wrong partition: never read past this junction's layers
            A.S[jid].status = CMTJ_STATUS_BAD_INPUT;
            jid = -1;
          } else {
#pragma unroll
            for (int l = 0; l < L; ++l) P[l].load(A.Ly[J.layer_offset + l], SOLVER == CMTJ_RK4);
            if (F::waves) {
              float hs[L];
#pragma unroll
              for (int l = 0; l < L; ++l) hs[l] = F::prescale ? P[l].gdt : 1.f;
              nw = J.n_waves < NW ? J.n_waves : NW;
#pragma unroll
              for (int w = 0; w < NW; ++w)
                if (w < nw) W[w].load(J.waves[w], hs);
            }
            if constexpr (kPacked) {
#pragma unroll
              for (int q = 0; q < NP; ++q) {
                Q[q].template load<FEAT, L>(P, q);
#pragma unroll
                for (int w = 0; w < NW; ++w)
                  if (w < nw)
                    HD[w][q] = pack2(W[w].hdir[2 * q], 2 * q + 1 < L ? W[w].hdir[2 * q + 1] : f3(0.f, 0.f, 0.f));
              }
            }
            step = S.step;
            if (step == 0) {
#pragma unroll
              for (int l = 0; l < L; ++l) m[l] = ld3(A.Ly[J.layer_offset + l].m);
            } else {
#pragma unroll
              for (int l = 0; l < L; ++l) m[l] = ld3(S.m[l]);
            }
            end = J.n_steps;
            stop_all = (end - step > p.chunk_steps) ? step + p.chunk_steps : end;
            n_logged = S.n_logged;
            n_red = S.n_red;
            rs = S.r_sum;
            rc = S.r_c;
            vs = S.v_sum;
            vc = S.v_c;
            if (p.red_weights) {
              wsum[0] = S.vw_sum;
              wsum[1] = S.vw_c;
            }
            win = J.win_start;
            Jp = &J;
            ref0 = A.Ly[J.layer_offset].ref;
            if (p.red_every) red_cache<L>(rk, J, ref0);
            tcount = 0;
            logrow = A.log + (size_t)J.log_offset * 4u;
            // next sampling steps: log at step % log_every == 0, reductions
            // at (step - win) % red_every == 0 for step >= win
            next_log = (C > 0 && p.log_every) ? step + (p.log_every - step % p.log_every) % p.log_every
                                              : 0xffffffffu;
            next_red = !p.red_every ? 0xffffffffu
                       : (step >= win ? step + (p.red_every - (step - win) % p.red_every) % p.red_every : win);
          }
        }
      }
    }
    // leave only when every lane has drained the queue
    if (__ballot_sync(0xffffffffu, !retired) == 0) break;
    if (jid < 0) continue;

    // ---- run a burst of steps, sampling only at the steps that log or
    // reduce (the reference logs after stepping at i % writeEvery == 0)
    const uint32_t burst_end = (stop_all - step > 64u) ? step + 64u : stop_all;
    while (step < burst_end) {
      const uint32_t next_ev = next_log < next_red ? next_log : next_red;
      const uint32_t stop = (next_ev < burst_end) ? next_ev + 1 : burst_end;
      // When every wave is a step driver whose on-windows miss this whole
      // burst, u = 0 at every stage and the waves are skipped: adding
      // amp * 0 would leave every term's bits unchanged.
      bool quiet = true;
#pragma unroll
      for (int w = 0; w < NW; ++w)
        if (w < nw) quiet = quiet && W[w].off_during(step, stop);
      if constexpr (kPacked) {
        // RK4 on layer pairs (the scalar RK4 below, lane by lane); a quiet
        // burst forms the field base once per step
        V2 mp[NP];
#pragma unroll
        for (int q = 0; q < NP; ++q) mp[q] = pack2(m[2 * q], 2 * q + 1 < L ? m[2 * q + 1] : f3(0.f, 0.f, 1.f));
        if constexpr (L == 2) {
          if (quiet) {
            for (; step < stop; ++step) packed_rk4_step<kDiag, false, NW>(mp[0], Q[0], W, &HD[0][0], nw, step, dtf);
          } else {
            for (; step < stop; ++step)
              packed_rk4_step<kDiag, F::waves, NW>(mp[0], Q[0], W, &HD[0][0], nw, step, dtf);
          }
        } else {
          if (quiet) {
            for (; step < stop; ++step) packed_rk4_step_pairs<L, kDiag, false, NW>(mp, Q, W, HD, nw, step, dtf);
          } else {
            for (; step < stop; ++step) packed_rk4_step_pairs<L, kDiag, F::waves, NW>(mp, Q, W, HD, nw, step, dtf);
          }
        }
#pragma unroll
        for (int q = 0; q < NP; ++q) {
          m[2 * q] = lane0(mp[q]);
          if (2 * q + 1 < L) m[2 * q + 1] = lane1(mp[q]);
        }
      } else {
      for (; step < stop; ++step) {
      if (SOLVER == CMTJ_RK4) {
        // neighbours frozen at their start-of-step values (junction.hpp:1682-1707)
        F3 acc[L], kp[L], hb[L];
        Delta<FEAT> d[L];
#pragma unroll
        for (int st = 0; st < 4; ++st) {
          const int s = st == 0 ? 0 : (st == 3 ? 2 : 1);
          if ((F::waves && st != 2) || (!F::waves && st == 0)) {
#pragma unroll
            for (int l = 0; l < L; ++l) d[l].clear(P[l].h0);
            if (F::waves && !quiet) {
#pragma unroll
              for (int w = 0; w < NW; ++w)
                if (w < nw) add_wave<L, FEAT>(W[w], step, s, dtf, d);
            }
#pragma unroll
            for (int l = 0; l < L; ++l)
              hb[l] = hbase_at<L, FEAT>(l, P[l], l > 0 ? m[l - 1] : f3(0.f, 0.f, 0.f),
                                        l < L - 1 ? m[l + 1] : f3(0.f, 0.f, 0.f), d[l]);
          }
          // k' = k/6 through the host's dt/6 prefactors, so the stage
          // offsets (3k', 3k', 6k') and weights (1, 2, 2, 1) are exact; the
          // increment is summed apart from m and added to m once, so only one
          // rounding per step happens at the scale of |m| = 1
          const float c = st == 3 ? 6.f : 3.f;
#pragma unroll
          for (int l = 0; l < L; ++l) {
            const F3 ms = st == 0 ? m[l] : fma3(kp[l], c, m[l]);
            const F3 mb = l > 0 ? m[l - 1] : f3(0.f, 0.f, 0.f);
            const F3 mt = l < L - 1 ? m[l + 1] : f3(0.f, 0.f, 0.f);
            const F3 k = rhs_at<L, FEAT>(l, P[l], ms, mb, mt, d[l], hb[l]);
            kp[l] = k;
            if (st == 0) acc[l] = k;
            else if (st == 3) acc[l] = acc[l] + k;
            else acc[l] = fma3(k, 2.f, acc[l]);
          }
        }
#pragma unroll
        for (int l = 0; l < L; ++l) m[l] = renorm(m[l] + acc[l]);
      } else {
        // Euler-Heun (1709-1754) and Heun (1756-1815), neighbours un-updated
        Delta<FEAT> d[L];
#pragma unroll
        for (int l = 0; l < L; ++l) d[l].clear(P[l].h0);
        if (F::waves && !quiet) {
#pragma unroll
          for (int w = 0; w < NW; ++w)
            if (w < nw) add_wave<L, FEAT>(W[w], step, 0, dtf, d);
        }
        F3 f[L], g[L], dW[L], mn[L];
#pragma unroll
        for (int l = 0; l < L; ++l) {
          // without scalar waves T is constant: sigma was formed at load
          const float sigma = F::swaves ? sqrtf(fmaxf(P[l].sigc * (P[l].t0 + d[l].dT), 0.f)) : P[l].sig;
          if (sigma > 0.f) {
            float g0, g1, g2;
            cmtj_gaussian3_f32(P[l].seed_lo, P[l].seed_hi, P[l].nstep0 + step, g0, g1, g2);
            dW[l] = f3(g0, g1, g2) * sigma;
          } else {
            dW[l] = f3(0.f, 0.f, 0.f);
          }
          const F3 mb = l > 0 ? m[l - 1] : f3(0.f, 0.f, 0.f);
          const F3 mt = l < L - 1 ? m[l + 1] : f3(0.f, 0.f, 0.f);
          f[l] = rhs_at<L, FEAT>(l, P[l], m[l], mb, mt, d[l], hbase_at<L, FEAT>(l, P[l], mb, mt, d[l]));
          g[l] = stoch<FEAT>(P[l], m[l], dW[l]);
        }
        if (SOLVER == CMTJ_EULER_HEUN) {
#pragma unroll
          for (int l = 0; l < L; ++l) {
            const F3 mN = fma3(g[l], sqdt, m[l]);
            const F3 g2 = stoch<FEAT>(P[l], mN, dW[l]);
            mn[l] = m[l] + fma3(g[l] + g2, 0.5f * sqdt, f[l]);  // one rounding at |m|
          }
#pragma unroll
          for (int l = 0; l < L; ++l) m[l] = renorm(mn[l]);
        } else {
#pragma unroll
          for (int l = 0; l < L; ++l) mn[l] = m[l] + fma3(g[l], sqdt, f[l]);
          if (F::waves && !quiet) {
#pragma unroll
            for (int l = 0; l < L; ++l) d[l].clear(P[l].h0);
#pragma unroll
            for (int w = 0; w < NW; ++w)
              if (w < nw) add_wave<L, FEAT>(W[w], step, 2, dtf, d);
          }
#pragma unroll
          for (int l = 0; l < L; ++l) {
            // the corrector sees the predicted neighbours (junction.hpp:1790-1800)
            const F3 mb = l > 0 ? mn[l - 1] : f3(0.f, 0.f, 0.f);
            const F3 mt = l < L - 1 ? mn[l + 1] : f3(0.f, 0.f, 0.f);
            const F3 f2 = rhs_at<L, FEAT>(l, P[l], mn[l], mb, mt, d[l], hbase_at<L, FEAT>(l, P[l], mb, mt, d[l]));
            const F3 g2 = stoch<FEAT>(P[l], mn[l], dW[l]);
            m[l] = renorm(m[l] + fma3(g[l] + g2, 0.5f * sqdt, (f[l] + f2) * 0.5f));
          }
        }
      }
      }  // steps up to (and including) the next sampling step
      }
      const uint32_t last = step - 1;

      // ---- reductions: R and I(t) R(t) from win_start on
      if (last == next_red) {
        next_red = (next_red > 0xffffffffu - p.red_every) ? 0xffffffffu : next_red + p.red_every;
        constexpr int b = red_mr_words<L>();
        const float R = resistance_cached<L>(rk, m);
        kadd(rs, rc, R);
        const uint64_t vdph = red_u64(rk, b + 2);
        if (vdph) {
          const uint64_t ph = red_u64(rk, b) + (uint64_t)last * vdph;
          const float I = sin2pi_phase(ph);
          kadd(vs, vc, I * R);
          if (p.red_weights) {
            const uint32_t tot = __float_as_uint(rk[(b + 4) * kRedStride]);
            const float w = __ldg(p.red_weights + (tot > n_red ? tot - 1u - n_red : 0u));
            float ws = wsum[0], wc = wsum[1];
            kadd(ws, wc, w * (I * R));
            wsum[0] = ws;
            wsum[1] = wc;
          }
        }
        ++n_red;
      }
      // ---- log (i % log_every == 0, like logLayerParams at 1978-1980)
      if (last == next_log) {
        next_log = (next_log > 0xffffffffu - p.log_every) ? 0xffffffffu : next_log + p.log_every;
        if (tcount == 0) bulk_wait_read();
        float *dst = tile + tcount * C;
        if (p.log_mode == CMTJ_LOG_M) {
#pragma unroll
          for (int l = 0; l < L; ++l) {
            dst[3 * l] = m[l].x;
            dst[3 * l + 1] = m[l].y;
            dst[3 * l + 2] = m[l].z;
          }
        } else if (p.log_mode == CMTJ_LOG_MIX) {
          float v = 0.f;
#pragma unroll
          for (int l = 0; l < L; ++l)
            v = fmaf(Jp->mix_w[l], p.log_axis == 0 ? m[l].x : (p.log_axis == 1 ? m[l].y : m[l].z), v);
          dst[0] = v;
        } else {
          dst[0] = resistance<L>(Jp, ref0, m);
        }
        ++tcount;
        ++n_logged;
        if (tcount == T) {
          bulk_store(logrow + (size_t)(n_logged - T) * C, tile, T * C * 4u);
          tcount = 0;
        }
      }
    }

    if (step == stop_all) {
      // ---- junction (or chunk) done: flush the partial tile, save state
      if (tcount > 0) {
        const uint32_t t4 = (tcount + 3u) & ~3u;
        bulk_store(logrow + (size_t)(n_logged - tcount) * C, tile, t4 * C * 4u);
        tcount = 0;
      }
      cmtj_f32_state_t &S = A.S[jid];
#pragma unroll
      for (int l = 0; l < L; ++l) {
        S.m[l][0] = m[l].x;
        S.m[l][1] = m[l].y;
        S.m[l][2] = m[l].z;
      }
      bool bad = false;
#pragma unroll
      for (int l = 0; l < L; ++l) bad |= isnan(m[l].x);
      S.step = step;
      S.status = bad ? CMTJ_STATUS_NAN : CMTJ_STATUS_OK;
      S.n_logged = n_logged;
      S.n_red = n_red;
      S.r_sum = rs;
      S.r_c = rc;
      S.v_sum = vs;
      S.v_c = vc;
      if (p.red_weights) {
        S.vw_sum = wsum[0];
        S.vw_c = wsum[1];
      }
      jid = -1;
    }
  }
  // Bulk stores still reading shared memory must finish before the CTA exits.
  bulk_wait_read();
}

}  // namespace cmtjf
