// FP64 plain-form device physics shared by every FP64 kernel (single
// junctions, stacks, groups; a thread or lanes per junction).  Every
// expression keeps the reference's operand order; units that include this
// header are compiled with --fmad=false so nothing is contracted into an
// FMA.
#pragma once
#include "common.cuh"
#include "philox.cuh"

// Functions are static: each including unit gets its own copy.
namespace cmtjd {


struct DriverCtx;

// A 3-vector held whole by one lane.  The physics below is written once
// for any vector type V with this interface (plain_lanes_f64.cu adds one
// that spreads the components over lanes).
struct D3 {
  double x, y, z;
  static constexpr int kLanes = 1;  // lanes per layer
  static __device__ __forceinline__ D3 zero();
  static __device__ __forceinline__ D3 load(const double *p);
  static __device__ __forceinline__ D3 make(double x, double y, double z);
  static __device__ __forceinline__ D3 axial(const cmtj_layer_t &L, int s, double t, const DriverCtx &dc, uint32_t dyn);
};

template <class T>
struct NoDeduce {
  using type = T;
};
static __device__ __forceinline__ D3 d3(double x, double y, double z) {
  D3 r;
  r.x = x;
  r.y = y;
  r.z = z;
  return r;
}
static __device__ __forceinline__ D3 zero3() { return d3(0.0, 0.0, 0.0); }
static __device__ __forceinline__ D3 operator+(const D3 &a, const D3 &b) { return d3(a.x + b.x, a.y + b.y, a.z + b.z); }
static __device__ __forceinline__ D3 operator-(const D3 &a, const D3 &b) { return d3(a.x - b.x, a.y - b.y, a.z - b.z); }
static __device__ __forceinline__ D3 operator*(const D3 &a, double s) { return d3(a.x * s, a.y * s, a.z * s); }
static __device__ __forceinline__ D3 operator/(const D3 &a, double s) { return d3(a.x / s, a.y / s, a.z / s); }
static __device__ __forceinline__ D3 smul(double s, const D3 &a) { return d3(s * a.x, s * a.y, s * a.z); }
static __device__ __forceinline__ double dot(const D3 &a, const D3 &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static __device__ __forceinline__ D3 cross(const D3 &a, const D3 &b) {
  return d3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static __device__ __forceinline__ D3 load3(const double *p) { return d3(p[0], p[1], p[2]); }

// CVector::normalize (cvector.hpp:185-192); pow(v, 2) is v*v, and
// dot(v, v) forms x*x + y*y + z*z in that order.
template <class V>
static __device__ __forceinline__ V normalized(const V &v) {
  const double mag = sqrt(dot(v, v));
  if (mag != 0) return v / mag;
  return v;
}

// calculate_tensor_interaction (junction.hpp:54-72).
// ms_mu0 = Ms / mu0, evaluated once by the host (cmtj_layer_t.ms_over_mu0).
static __device__ __forceinline__ D3 tensor_mul(const D3 &m, const double *t, double ms_mu0) {
  const D3 r = d3(t[0] * m.x + t[1] * m.y + t[2] * m.z, t[3] * m.x + t[4] * m.y + t[5] * m.z,
                  t[6] * m.x + t[7] * m.y + t[8] * m.z);
  return r * ms_mu0;
}

// True when every component is +0 or -0 (integer test: no FP64 instruction).
static __device__ __forceinline__ bool is_zero3(const D3 &v) {
  const unsigned long long mask = 0x7fffffffffffffffull;
  return ((__double_as_longlong(v.x) | __double_as_longlong(v.y) | __double_as_longlong(v.z)) & mask) == 0ull;
}

// x^3 rounded once: x*x is split exactly into hi + lo (FMA error-free
// product), then (hi + lo) * x is formed with one final rounding.  This is
// what a correctly rounded pow(x, 3.0) returns, up to rare ties.
static __device__ __forceinline__ double cube_rn(double x) {
  const double ph = x * x;
  const double pl = fma(x, x, -ph);
  const double th = ph * x;
  const double tl = fma(ph, x, -th) + pl * x;
  return th + tl;
}

struct DriverCtx {
  const double *tables;
  uint32_t step;
  int stage;  // 0: t, 1: t + dt/2, 2: t + dt
};

// ScalarDriver::getCurrentScalarValue (drivers.hpp:262-305).
static __device__ double drv(const cmtj_driver_t &d, double time, const DriverCtx &dc) {
  const int u = d.update;
  double rv = d.constantValue;
  if (u == CMTJ_DRV_CONSTANT) return rv;
  if (u == CMTJ_DRV_PULSE) {
    const int n = (int)(time / d.period);
    const double dT = d.cycle * d.period;
    const double nT = n * d.period;
    if (nT <= time && time <= (nT + dT)) rv = rv + d.amplitude;
  } else if (u == CMTJ_DRV_SINE) {
    rv = rv + d.amplitude * sin(2 * M_PI * time * d.frequency + d.phase);
  } else if (u == CMTJ_DRV_POSINE) {
    rv = rv + fabs(d.amplitude * sin(2 * M_PI * time * d.frequency + d.phase));
  } else if (u == CMTJ_DRV_HALFSINE) {
    const double tamp = d.amplitude * sin(2 * M_PI * time * d.frequency + d.phase);
    if (tamp <= 0) rv = rv + tamp;
  } else if (u == CMTJ_DRV_STEP) {
    if (time >= d.timeStart && time <= d.timeStop) rv = rv + d.amplitude;
  } else if (u == CMTJ_DRV_TRAPEZOID) {
    const double ts = d.timeStart, e = d.edgeTime, s = d.steadyTime, a = d.amplitude;
    double add = 0.0;
    if (time < ts) add = 0.0;
    else if (time <= ts + e) add = (a / e) * (time - ts);
    else if (time <= ts + e + s) add = a;
    else if (time <= ts + 2 * e + s) add = a - (a / e) * (time - (ts + e + s));
    rv = rv + add;
  } else if (u == CMTJ_DRV_GAUSSIMPULSE) {
    const double dtt = time - d.timeStart;
    rv = rv + d.amplitude * exp(-(dtt * dtt) / (2 * (d.edgeTime * d.edgeTime)));
  } else if (u == CMTJ_DRV_GAUSSSTEP) {
    rv = rv + 0.5 * d.amplitude * (1 + erf((time - d.timeStart) / (sqrt(2.0) * d.edgeTime)));
  } else if (u == CMTJ_DRV_TABLE) {
    return dc.tables[d.table_offset + (int64_t)dc.step * 3 + dc.stage];
  }
  return rv;
}

static __device__ __forceinline__ D3 axial(const cmtj_layer_t &L, int slot, double t, const DriverCtx &dc) {
  return d3(drv(L.drv[slot], t, dc), drv(L.drv[slot + 1], t, dc), drv(L.drv[slot + 2], t, dc));
}

// One out-of-line copy of the driver dispatch for callers that reach it
// only for the few time-dependent slots.
static __device__ __noinline__ double drv_call(const cmtj_driver_t &d, double time, DriverCtx dc) {
  return drv(d, time, dc);
}

// Driver slot s at `time`.  Bit s of dyn marks a slot whose driver is not
// CMTJ_DRV_CONSTANT; the other slots return constantValue, which is what
// drv() returns for them, without the dispatch.  dyn = ~0u evaluates every
// slot through drv().
static __device__ __forceinline__ double slot_at(const cmtj_layer_t &L, int s, double time, const DriverCtx &dc,
                                                 uint32_t dyn) {
  if (dyn == 0xffffffffu) return drv(L.drv[s], time, dc);
  return ((dyn >> s) & 1u) ? drv_call(L.drv[s], time, dc) : L.drv[s].constantValue;
}
static __device__ __forceinline__ D3 axial_at(const cmtj_layer_t &L, int s, double time, const DriverCtx &dc,
                                              uint32_t dyn) {
  return d3(slot_at(L, s, time, dc, dyn), slot_at(L, s + 1, time, dc, dyn), slot_at(L, s + 2, time, dc, dyn));
}

__device__ __forceinline__ D3 D3::zero() { return zero3(); }
__device__ __forceinline__ D3 D3::load(const double *p) { return load3(p); }
__device__ __forceinline__ D3 D3::make(double x, double y, double z) { return d3(x, y, z); }
__device__ __forceinline__ D3 D3::axial(const cmtj_layer_t &L, int s, double t, const DriverCtx &dc, uint32_t dyn) {
  return axial_at(L, s, t, dc, dyn);
}

// Bit s set when driver slot s of L is time-dependent (not CMTJ_DRV_CONSTANT).
static __device__ __forceinline__ uint32_t dynamic_slots(const cmtj_layer_t &L) {
  uint32_t m = 0;
  for (int s = 0; s < CMTJ_NUM_SLOTS; ++s)
    if (L.drv[s].update != CMTJ_DRV_CONSTANT) m |= 1u << s;
  return m;
}

// Values the reference keeps on the Layer as side effects of the last field
// evaluation and logs with calculateEnergies (junction.hpp:1589-1613).
template <class V>
struct SideT {
  double K, K2, Jb, Jt, I;
  V Hext, Hiec, Hanis, Hdemag, Hfl, Hdl;
};
using Side = SideT<D3>;

// calculateHeff + solveLLG (junction.hpp:580-815, 855-864).
template <class V>
static __device__ V rhs(const cmtj_layer_t &L, const cmtj_constants_t &c, double time, const V &m, const V &bottom,
                        const V &top, const DriverCtx &dc, typename NoDeduce<SideT<V>>::type *side,
                        const cmtj_driver_t *cur = nullptr, uint32_t dyn = 0xffffffffu,
                        const double *hres = nullptr) {
  const double Ms = L.Ms;
  const uint32_t zt = L.zero_terms;
  // --- calculateHeff (580-622).  Terms the host marked identically zero
  // (CMTJ_ZERO_*), and IEC / IDMI against a zero neighbour vector, are left
  // out of the sum: adding an exact zero changes no value.
  const bool zb = is_zero3(bottom), ztop = is_zero3(top);
  V Hdipole = V::zero();
  if (!(zt & CMTJ_ZERO_DIPOLE))
    Hdipole = tensor_mul(bottom, L.dipole_bottom, L.ms_over_mu0) + tensor_mul(top, L.dipole_top, L.ms_over_mu0);
  const V Hext = V::axial(L, CMTJ_SLOT_HEXT, time, dc, dyn);
  const V Hoe = V::axial(L, CMTJ_SLOT_HOE, time, dc, dyn);
  const V Hdemag = tensor_mul(m, L.demag, L.ms_over_mu0);
  const double Jb = slot_at(L, CMTJ_SLOT_IEC_BOTTOM, time, dc, dyn);
  const double Jt = slot_at(L, CMTJ_SLOT_IEC_TOP, time, dc, dyn);
  const double Mst = Ms * L.thickness;
  V Hiec = V::zero();
  if (zt & CMTJ_ZERO_J2) {
    // Jx + 2*0*dot = Jx exactly
    if (!zb && !ztop) Hiec = (bottom * Jb) / Mst + (top * Jt) / Mst;
    else if (!zb) Hiec = (bottom * Jb) / Mst;
    else if (!ztop) Hiec = (top * Jt) / Mst;
  } else {
    const double J2b = slot_at(L, CMTJ_SLOT_IECQ_BOTTOM, time, dc, dyn);
    const double J2t = slot_at(L, CMTJ_SLOT_IECQ_TOP, time, dc, dyn);
    Hiec = (bottom * (Jb + 2 * J2b * dot(bottom, m))) / Mst + (top * (Jt + 2 * J2t * dot(top, m))) / Mst;
  }
  V Hidmi = V::zero();
  if (!(zt & CMTJ_ZERO_IDMI)) {
    const V Db = V::axial(L, CMTJ_SLOT_IDMI_BOTTOM, time, dc, dyn);
    const V Dt = V::axial(L, CMTJ_SLOT_IDMI_TOP, time, dc, dyn);
    Hidmi = smul(-1.0, cross(Db, bottom)) / Mst + smul(-1.0, cross(Dt, top)) / Mst;
  }
  const V anis = V::load(L.anis);
  const double K = slot_at(L, CMTJ_SLOT_ANIS, time, dc, dyn);
  const V Hanis = anis * ((2 * K) * dot(anis, m) / Ms);
  const V Hdmi = V::axial(L, CMTJ_SLOT_HDMI, time, dc, dyn);
  // hres: the reserved interaction field a group sets for this step (the
  // value its constant HRES drivers would return)
  const V Hres = hres ? V::make(hres[0], hres[1], hres[2]) : V::axial(L, CMTJ_SLOT_HRES, time, dc, dyn);
  double K2 = 0.0;
  V H = Hext + Hanis;
  if (!(zt & CMTJ_ZERO_K2)) {
    K2 = slot_at(L, CMTJ_SLOT_ANIS2, time, dc, dyn);
    H = H + anis * ((4 * K2) * cube_rn(dot(anis, m)) / Ms);
  }
  H = H + Hiec;
  if (!(zt & CMTJ_ZERO_IDMI)) H = H + Hidmi;
  H = H + Hoe + Hdmi - Hdemag;  // + Hfluct (zero without a thermal field here)
  if (!(zt & CMTJ_ZERO_DIPOLE)) H = H - Hdipole;
  H = H + Hres;
  if (side) {
    side->K = K;
    side->K2 = K2;
    side->Jb = Jb;
    side->Jt = Jt;
    side->Hext = Hext;
    side->Hiec = Hiec;
    side->Hanis = Hanis;
    side->Hdemag = Hdemag;
  }
  // --- solveLLG (716-815)
  const double GYRO = c.gyro;
  const double damping = L.damping;
  const V prod = cross(m, H);
  const V prod2 = cross(m, prod);
  const double convTerm = L.conv_term;  // 1 / (1 + damping^2)
  const V dmdt = prod + prod2 * damping;
  V reference = V::zero();
  if (L.referenceType == CMTJ_REF_FIXED) reference = V::load(L.ref);
  else if (L.referenceType == CMTJ_REF_TOP) reference = top;
  else if (L.referenceType == CMTJ_REF_BOTTOM) reference = bottom;
  if (L.includeSTT) {
    const double I = cur ? drv(*cur, time, dc) : slot_at(L, CMTJ_SLOT_CURRENT, time, dc, dyn);
    if (side) side->I = I;
    const double aJ = c.hbar * I / (c.echarge * L.Ms * L.thickness);
    double eta = 0;
    if (L.alternativeSTT) {
      eta = (L.spinPolarisation) / (1 + L.slonczewski * dot(m, reference));
    } else {
      const double slonSq = L.slonczewski * L.slonczewski;
      eta = (L.spinPolarisation * slonSq) / (slonSq + 1 + (slonSq - 1) * dot(m, reference));
    }
    const double sttTerm = GYRO * aJ * eta;
    const V fieldLike = cross(m, reference);
    const V dampingLike = cross(m, fieldLike);
    return (dmdt * -GYRO + dampingLike * -sttTerm * L.kappa + fieldLike * sttTerm * L.beta) * convTerm;
  } else if (L.includeSOT) {
    double Hdl = 0, Hfl = 0, Hdl2 = 0, Hfl2 = 0;
    if (L.dynamicSOT) {
      Hdl = slot_at(L, CMTJ_SLOT_DL, time, dc, dyn);
      Hfl = slot_at(L, CMTJ_SLOT_FL, time, dc, dyn);
      Hdl2 = slot_at(L, CMTJ_SLOT_DL2, time, dc, dyn);
      Hfl2 = slot_at(L, CMTJ_SLOT_FL2, time, dc, dyn);
    } else {
      const double I = cur ? drv(*cur, time, dc) : slot_at(L, CMTJ_SLOT_CURRENT, time, dc, dyn);
      if (side) side->I = I;
      Hdl = L.dampingLikeTorque * I;
      Hfl = L.fieldLikeTorque * I;
    }
    const V ref2 = V::load(L.ref2);
    if (side) {
      side->Hfl = reference * (Hfl - damping * Hdl);
      side->Hdl = reference * (Hdl + damping * Hfl);
    }
    const V cm_p = cross(m, reference);
    const V ccm_p = cross(m, cm_p);
    const V cm_s = cross(m, ref2);
    const V ccm_s = cross(m, cm_s);
    const V flp = cm_p * (Hfl - damping * Hdl);
    const V dlp = ccm_p * (Hdl + damping * Hfl);
    const V fls = cm_s * (Hfl2 - damping * Hdl2);
    const V dls = ccm_s * (Hdl2 + damping * Hfl2);
    return (dmdt + flp + dlp + fls + dls) * -GYRO * convTerm;
  }
  return dmdt * -GYRO * convTerm;
}

// stochasticTorque (junction.hpp:824-831).
template <class V>
static __device__ __forceinline__ V stoch_torque(const cmtj_layer_t &L, const cmtj_constants_t &c, const V &m,
                                                 const V &dW) {
  const double convTerm = L.stoch_conv;  // -gyro / (1 + damping^2)
  const V th = cross(m, dW);
  const V th2 = cross(m, th);
  return (th + th2 * L.damping) * convTerm;
}

// getOneFVector (junction.hpp:1130-1136): the layer's buffered 1/f^alpha
// sample of iteration i, VectorAlphaNoise::tickVector (noise.hpp:280-290):
// the float samples of the active axis (all three, normalised, for
// Axis::all) times the scale.  Iterations beyond the buffer read zero.
template <class V>
static __device__ __forceinline__ V alpha_sample(const cmtj_layer_t &L, uint32_t i) {
  if (i >= L.alpha_len) return V::zero();
  const float *b = L.alpha_buf + i;
  const size_t n = L.alpha_len;
  const int ax = L.alpha_axis;
  const double x = (ax == 0 || ax == 3) ? (double)b[0] : 0.0;
  const double y = (ax == 1 || ax == 3) ? (double)b[n] : 0.0;
  const double z = (ax == 2 || ax == 3) ? (double)b[2 * n] : 0.0;
  V v = V::make(x, y, z);
  if (ax == 3) v = normalized(v);
  return v * L.alpha_scale;
}

// The thermal field's standard deviation at temperature temp
// (getLangevinStochasticStandardDeviation, junction.hpp:1111-1120).
static __device__ __forceinline__ double langevin_sigma(const cmtj_layer_t &L, const cmtj_constants_t &c,
                                                        double temp) {
  const double mainFactor = (2 * L.damping * c.kB * temp) / (L.Ms * L.cellVolume * c.gyro);
  return sqrt(mainFactor);
}

// getStochasticLangevinVector (junction.hpp:1111-1128), plus the buffered
// alpha noise where the layer has one: dW of the Euler-Heun and Heun
// runners (junction.hpp:1726-1727, 1792-1793).  sigma_run: the lane's sigma
// formed once for the run (langevin_sigma of its constant temperature; the
// same value every step), or -1 to form it at this step (the test reads the
// sign bit: no FP64 compare).
template <class V = D3>
static __device__ __forceinline__ V langevin(const cmtj_layer_t &L, const cmtj_constants_t &c, double time,
                                       uint32_t i, const DriverCtx &dc, uint32_t dyn = 0xffffffffu,
                                       double sigma_run = -1.0) {
  V dW = V::zero();
  if (L.temperatureSet) {
    const double sigma = (__double_as_longlong(sigma_run) >= 0)
                             ? sigma_run
                             : langevin_sigma(L, c, slot_at(L, CMTJ_SLOT_TEMPERATURE, time, dc, dyn));
    double g0, g1, g2;
    cmtj_gaussian3_f64(L.seed_lo, L.seed_hi, L.noise_step + i, g0, g1, g2);
    dW = V::make(g0, g1, g2) * sigma;
  }
  if (L.alpha_buf) dW = dW + alpha_sample<V>(L, i);
  return dW;
}


// One iteration of the runner chosen by getSolver (junction.hpp:1668-1815)
// for the n layers of one junction, on one thread (the stack and group
// kernels for stacks and groups too wide for lanes; out of line, since they
// run rarely and it shortens their build).  single_layer:
// runSingleLayerSolver is in force (a Stack whose last junction has one
// layer steps only layer 0 of every junction).  Returns false on a NaN
// magnetisation (rk4_step throws).
static __device__ __noinline__ bool junction_step(int n, const cmtj_layer_t *Ls, D3 *mag, D3 *work, Side *side, uint32_t i, double t,
                              const cmtj_sim_params_t &p, const double *tables, const cmtj_driver_t *cur,
                              bool single_layer) {
  const cmtj_constants_t c = p.c;
  const double dt = p.time_step;
  const bool energies = p.calculate_energies != 0;
  if (single_layer && p.solver == CMTJ_RK4) n = 1;
    if (p.solver == CMTJ_RK4) {
      // runSingleLayerSolver / runMultiLayerSolver (1668-1707): neighbours
      // frozen at their start-of-step values for all four stages.
      work[0] = zero3();
      work[n + 1] = zero3();
      for (int l = 0; l < n; ++l) work[l + 1] = mag[l];
      bool nan_seen = false;
      for (int l = 0; l < n; ++l) {
        const cmtj_layer_t &L = Ls[l];
        const D3 bottom = work[l], top = work[l + 2];
        DriverCtx d0 = {tables, i, 0}, d1 = {tables, i, 1}, d2 = {tables, i, 2};
        // Layer::rk4_step (1017-1041)
        D3 m_t = mag[l];
        const D3 k1 = rhs(L, c, t, m_t, bottom, top, d0, nullptr, cur) * dt;
        const D3 k2 = rhs(L, c, t + 0.5 * dt, m_t + k1 * 0.5, bottom, top, d1, nullptr, cur) * dt;
        const D3 k3 = rhs(L, c, t + 0.5 * dt, m_t + k2 * 0.5, bottom, top, d1, nullptr, cur) * dt;
        const D3 k4 = rhs(L, c, t + dt, m_t + k3, bottom, top, d2, energies ? &side[l] : nullptr, cur) * dt;
        m_t = m_t + (k1 + (k2 * 2.0) + (k3 * 2.0) + k4) / 6.0;
        mag[l] = normalized(m_t);
        if (isnan(mag[l].x)) {
          nan_seen = true;
          break;
        }
      }
      if (nan_seen) return false;
    } else if (p.solver == CMTJ_EULER_HEUN) {
      // eulerHeunSolverStep (1709-1754)
      for (int l = 0; l < n; ++l) {
        const cmtj_layer_t &L = Ls[l];
        DriverCtx d0 = {tables, i, 0};
        const D3 dW = langevin(L, c, t, i, d0);
        const D3 bottom = (l == 0) ? zero3() : mag[l - 1];
        const D3 top = (l == n - 1) ? zero3() : mag[l + 1];
        const D3 f = rhs(L, c, t, mag[l], bottom, top, d0, energies ? &side[l] : nullptr, cur);
        const D3 g = stoch_torque(L, c, mag[l], dW);
        const D3 mNext = mag[l] + g * sqrt(dt);
        const D3 g2 = stoch_torque(L, c, mNext, dW);
        work[l] = mag[l] + f * dt + smul(0.5, g + g2) * sqrt(dt);
      }
      for (int l = 0; l < n; ++l) mag[l] = normalized(work[l]);
    } else {
      // heunSolverStep (1756-1815)
      D3 fn[CMTJ_MAX_LAYERS], gn[CMTJ_MAX_LAYERS], dW[CMTJ_MAX_LAYERS];
      for (int l = 0; l < n; ++l) {
        const cmtj_layer_t &L = Ls[l];
        DriverCtx d0 = {tables, i, 0};
        const D3 bottom = (l == 0) ? zero3() : mag[l - 1];
        const D3 top = (l == n - 1) ? zero3() : mag[l + 1];
        fn[l] = rhs(L, c, t, mag[l], bottom, top, d0, nullptr, cur);
        dW[l] = langevin(L, c, t, i, d0);
        gn[l] = stoch_torque(L, c, mag[l], dW[l]);
        work[l] = mag[l] + fn[l] * dt + gn[l] * sqrt(dt);
      }
      for (int l = 0; l < n; ++l) {
        const cmtj_layer_t &L = Ls[l];
        DriverCtx d2 = {tables, i, 2};
        const D3 bottom = (l == 0) ? zero3() : work[l - 1];
        const D3 top = (l == n - 1) ? zero3() : work[l + 1];
        const D3 f2 = rhs(L, c, t + dt, work[l], bottom, top, d2, energies ? &side[l] : nullptr, cur);
        const D3 g2 = stoch_torque(L, c, work[l], dW[l]);
        mag[l] = mag[l] + smul(0.5 * dt, fn[l] + f2) + smul(0.5, gn[l] + g2) * sqrt(dt);
        mag[l] = normalized(mag[l]);
      }
    }

  return true;
}

// isnan of a vector's x component, on every lane that holds the vector.
static __device__ __forceinline__ bool x_nan_all(const D3 &a) { return isnan(a.x); }

// Layer::dormand_prince_step (junction.hpp:866-1002) of one layer: tries a
// step of size ts from time t, sets ts to the next step size (whether the
// step is accepted or not) and updates the layer's PID state in place.
// Returns accepted; nan is set when an accepted m is NaN.  Custom drivers
// are rejected by the host (their tables hold fixed-step times only).
template <class V>
static __device__ bool dp_layer(const cmtj_layer_t &L, cmtj_adaptive_t &ap, const cmtj_constants_t &c, double t,
                                double &ts, V &mag, const V &bottom, const V &top, const double *tables,
                                typename NoDeduce<SideT<V>>::type *side, bool &nan) {
  const DriverCtx dc = {tables, 0u, 0};
  const V m_t = mag;
  const double c2 = 1.0 / 5.0, c3 = 3.0 / 10.0, c4 = 4.0 / 5.0, c5 = 8.0 / 9.0, c6 = 1.0, c7 = 1.0;
  const V k1 = rhs(L, c, t, m_t, bottom, top, dc, nullptr) * ts;
  const V k2 = rhs(L, c, t + c2 * ts, m_t + k1 * (c2), bottom, top, dc, nullptr) * ts;
  const V k3 = rhs(L, c, t + c3 * ts, m_t + k1 * (3.0 / 40.0) + k2 * (9.0 / 40.0), bottom, top, dc, nullptr) * ts;
  const V k4 = rhs(L, c, t + c4 * ts, m_t + k1 * (44.0 / 45.0) + k2 * (-56.0 / 15.0) + k3 * (32.0 / 9.0), bottom,
                    top, dc, nullptr) * ts;
  const V k5 = rhs(L, c, t + c5 * ts,
                    m_t + k1 * (19372.0 / 6561.0) + k2 * (-25360.0 / 2187.0) + k3 * (64448.0 / 6561.0) +
                        k4 * (-212.0 / 729.0),
                    bottom, top, dc, nullptr) * ts;
  const V k6 = rhs(L, c, t + c6 * ts,
                    m_t + k1 * (9017.0 / 3168.0) + k2 * (-355.0 / 33.0) + k3 * (46732.0 / 5247.0) +
                        k4 * (49.0 / 176.0) + k5 * (-5103.0 / 18656.0),
                    bottom, top, dc, nullptr) * ts;
  const V k7 = rhs(L, c, t + c7 * ts,
                    m_t + k1 * (35.0 / 384.0) + k3 * (500.0 / 1113.0) + k4 * (125.0 / 192.0) +
                        k5 * (-2187.0 / 6784.0) + k6 * (11.0 / 84.0),
                    bottom, top, dc, side) * ts;
  const V m5 = m_t + k1 * (35.0 / 384.0) + k3 * (500.0 / 1113.0) + k4 * (125.0 / 192.0) +
                k5 * (-2187.0 / 6784.0) + k6 * (11.0 / 84.0);
  const V m4 = m_t + k1 * (5179.0 / 57600.0) + k3 * (7571.0 / 16695.0) + k4 * (393.0 / 640.0) +
                k5 * (-92097.0 / 339200.0) + k6 * (187.0 / 2100.0) + k7 * (1.0 / 40.0);
  const V err = m5 - m4;
  const double err_norm = sqrt(dot(err, err));  // x*x + y*y + z*z
  const double tol = ap.abs_tol + ap.rel_tol * sqrt(dot(m_t, m_t));
  double ratio = err_norm / tol;
  if (tol < 1e-15 || isnan(ratio) || isinf(ratio)) ratio = 10.0;
  double factor;
  if (ap.use_pid_control) {
    const double e_n = log(ratio);
    ap.integral_error += e_n;
    factor = exp(ap.kp * e_n + ap.ki * ap.integral_error + ap.kd * (e_n - ap.prev_error_ratio));
    ap.prev_error_ratio = e_n;
  } else {
    factor = ap.safety_factor * pow(1.0 / ratio, 0.2);
  }
  if (isnan(factor) || isinf(factor)) factor = ap.min_factor;
  factor = fmin(factor, ap.max_factor);
  factor = fmax(factor, ap.min_factor);
  double next = ts * factor;
  if (isnan(next) || isinf(next) || next <= 0) next = ts * ap.min_factor;
  ts = next;
  if (ratio <= 1.0) {
    mag = normalized(m5);
    if (x_nan_all(mag)) nan = true;
    return true;
  }
  return false;
}

// logLayerParams (junction.hpp:1580-1636) into one row of p.log_width doubles.
static __device__ void log_row(double *r, const cmtj_junction_t &J, int n, const cmtj_layer_t *Ls, const D3 *mag,
                        const Side *side, double t, bool energies) {
  int col = 0;
  for (int l = 0; l < n; ++l) {
    if (energies) {
      const Side &s = side[l];
      r[col++] = s.K;
      r[col++] = s.K2;
      r[col++] = s.Jb;
      r[col++] = s.Jt;
      r[col++] = s.I;
      const D3 v[7] = {s.Hext, s.Hiec, s.Hanis, s.Hdemag, zero3(), s.Hfl, s.Hdl};
      for (int q = 0; q < 7; ++q) {
        r[col++] = v[q].x;
        r[col++] = v[q].y;
        r[col++] = v[q].z;
      }
    }
    r[col++] = mag[l].x;
    r[col++] = mag[l].y;
    r[col++] = mag[l].z;
  }
  double r0 = 0.0, r1 = 0.0, r2 = 0.0;
  if (J.mr_mode == CMTJ_MR_CLASSIC && n == 1) {
    const double cosT = dot(mag[0], load3(Ls[0].ref));
    r0 = J.Rp + (((J.Rap - J.Rp) / 2.0) * (1.0 - cosT));
  } else if (J.mr_mode == CMTJ_MR_CLASSIC && n > 1) {
    const double cosT = dot(mag[0], mag[1]);
    r0 = J.Rp + (((J.Rap - J.Rp) / 2.0) * (1.0 - cosT));
  } else if (J.mr_mode == CMTJ_MR_STRIP) {
    // stripMagnetoResistance (1835-1857)
    double Rx_acc = 0.0, Ry_acc = 0.0;
    for (int l = 0; l < n; ++l) {
      const double Rx = J.Rx0[l] + J.AMR_X[l] * (mag[l].x * mag[l].x) + J.SMR_X[l] * (mag[l].y * mag[l].y);
      const double Ry = J.Ry0[l] + 0.5 * J.AHE[l] * mag[l].z + (J.AMR_Y[l] + J.SMR_Y[l]) * mag[l].x * mag[l].y;
      Rx_acc = Rx_acc + 1. / Rx;
      Ry_acc = Ry_acc + 1. / Ry;
    }
    r0 = 1 / Rx_acc;
    r1 = 1 / Ry_acc;
  }
  r[col++] = r0;
  r[col++] = r1;
  r[col++] = r2;
  r[col++] = t;
}

// magnetoresistance of a CLASSIC junction (getMagnetoresistance()[0], 1869-1879)
static __device__ __forceinline__ double classic_R(const cmtj_junction_t &J, int n, const cmtj_layer_t *Ls, const D3 *mag) {
  const double cosT = n == 1 ? dot(mag[0], load3(Ls[0].ref)) : dot(mag[0], mag[1]);
  return J.Rp + (((J.Rap - J.Rp) / 2.0) * (1.0 - cosT));
}

}  // namespace cmtjd
