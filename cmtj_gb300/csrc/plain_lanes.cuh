// Device building blocks of the FP64 fixed-step runners with a junction's
// layers side by side on lanes (plain_lanes_f64.cu, stack_lanes_f64.cu,
// group_lanes_f64.cu).
//
// A junction holds `span` = G * P consecutive lanes of one warp: G layer
// slots (at least its layer count) of P lanes each (P = 1 for D3, 4 for C3).
// Every function here is called by every lane of the warp, in uniform
// control flow: the warp shuffles and ballots below name the whole warp.
// Lanes that have nothing to compute pass step = false.
#pragma once
#include "lane3.cuh"
#include "plain_f64.cuh"
#include "recip.cuh"

namespace cmtjd {

constexpr unsigned kWarpAll = 0xffffffffu;

struct LaneGeo {
  int lane;       // lane in the warp
  int jl;         // lane within the junction's span
  int l;          // layer slot of this lane
  int lead;       // warp lane of the junction's first lane
  int span;       // lanes per junction
  int below_src;  // lane holding the same component of layer l - 1
  int above_src;  // ... of layer l + 1
  unsigned group; // the junction's lanes
};

template <class V>
__device__ __forceinline__ LaneGeo lane_geo(int G) {
  constexpr int P = V::kLanes;
  LaneGeo g;
  g.span = G * P;
  g.lane = threadIdx.x & 31;
  g.jl = g.lane % g.span;
  g.l = g.jl / P;
  g.lead = g.lane - g.jl;
  g.below_src = g.l > 0 ? g.lane - P : g.lane;
  g.above_src = g.l + 1 < G ? g.lane + P : g.lane;
  g.group = (g.span == 32 ? kWarpAll : ((1u << g.span) - 1u)) << g.lead;
  return g;
}

// A field-only layer: no dipole, IDMI, second-order anisotropy or
// biquadratic IEC term (CMTJ_ZERO_*), no STT and no SOT.  rhs() of such a
// layer reads only m, the neighbours and the slots HEXT, HOE, HDMI, HRES,
// ANIS, IEC_TOP and IEC_BOTTOM.  With those constant, everything but m and
// the neighbours is fixed for the whole run, and FieldOnly holds it in
// registers.  The field and anisotropy slots may also be time-dependent
// (rhs_field_only with DYN reads them at each stage time); the IEC slots
// may not, because the IEC term is formed once per step.
__device__ __forceinline__ bool field_only(const cmtj_layer_t &L) {
  const uint32_t all = CMTJ_ZERO_DIPOLE | CMTJ_ZERO_IDMI | CMTJ_ZERO_K2 | CMTJ_ZERO_J2;
  return (L.zero_terms & all) == all && !L.includeSTT && !L.includeSOT;
}
// The driver slots whose dynamic_slots() bit keeps a field-only layer off
// the field-only loop.
constexpr uint32_t kFieldOnlyFixedSlots = (1u << CMTJ_SLOT_IEC_TOP) | (1u << CMTJ_SLOT_IEC_BOTTOM);

template <class V>
struct FieldOnly {
  V Hext, Hoe, Hdmi, Hres, anis;
  double K, Jb, Jt, Ms, Mst, ms_mu0, damping, conv, gyro;
  Recip rMs, rMst;  // division by Ms and by Ms * thickness (recip.cuh)
  const double *demag;
  // the same on every lane of the warp (field_only_flags): every lane's
  // demag rows have +-0 off the diagonal; every lane's Hoe / Hdmi / Hres
  // slot is constant and +-0
  bool diag, zoe, zdmi, zres;
};

static __device__ __forceinline__ unsigned long long dbits(double x) {
  return (unsigned long long)__double_as_longlong(x);
}

// x + z for z = +-0 (rounding to nearest): x, except -0 + +0 = +0.  No
// FP64 instruction.
static __device__ __forceinline__ double add_zero(double x, double z) {
  return (dbits(x) == 0x8000000000000000ull && dbits(z) == 0ull) ? 0.0 : x;
}
static __device__ __forceinline__ C3 add_zero(const C3 &a, const C3 &z) { return C3{add_zero(a.v, z.v)}; }
static __device__ __forceinline__ D3 add_zero(const D3 &a, const D3 &z) {
  return d3(add_zero(a.x, z.x), add_zero(a.y, z.y), add_zero(a.z, z.z));
}

// A tensor row times m as tensor_mul forms it, out of line: a predicated
// inline copy would still hold the FP64 pipe for its five instructions on
// every call of diag_row.
static __device__ __noinline__ double row_full(const double *r, double mx, double my, double mz) {
  return r[0] * mx + r[1] * my + r[2] * mz;
}
// (r0 mx + r1 my) + r2 mz, as tensor_mul forms it, for a row whose entries
// other than r[c] are +-0: the zero products change the diagonal product d
// in no bit unless d is itself zero, and then the sum is a zero that is -0
// only when all three products are -0.  An inf or NaN component takes the
// full sum (row_full).  One FP64 instruction instead of five.
static __device__ __forceinline__ double diag_row(const double *r, int c, double mx, double my, double mz) {
  const unsigned long long e = 0x7ff0000000000000ull;
  const unsigned long long bx = dbits(mx), by = dbits(my), bz = dbits(mz);
  if ((bx & e) == e || (by & e) == e || (bz & e) == e) return row_full(r, mx, my, mz);
  const double d = r[c] * (c == 0 ? mx : (c == 1 ? my : mz));
  if ((dbits(d) << 1) != 0ull) return d;
  const unsigned long long neg = (dbits(r[0]) ^ bx) & (dbits(r[1]) ^ by) & (dbits(r[2]) ^ bz);
  return (neg >> 63) ? -0.0 : 0.0;
}
static __device__ __forceinline__ C3 tensor_mul_diag(const C3 &m, const double *t, double ms_mu0) {
  const double mx = quad_get(m.v, 0), my = quad_get(m.v, 1), mz = quad_get(m.v, 2);
  const int c = quad_comp();
  return C3{diag_row(t + 3 * c, c, mx, my, mz) * ms_mu0};
}
static __device__ __forceinline__ D3 tensor_mul_diag(const D3 &m, const double *t, double ms_mu0) {
  return d3(diag_row(t, 0, m.x, m.y, m.z), diag_row(t + 3, 1, m.x, m.y, m.z), diag_row(t + 6, 2, m.x, m.y, m.z)) *
         ms_mu0;
}
// The components the lane holds are +-0 (a warp vote over every lane then
// covers every component of every layer).
static __device__ __forceinline__ bool lane_zero(const C3 &a) { return (dbits(a.v) << 1) == 0ull; }
static __device__ __forceinline__ bool lane_zero(const D3 &a) {
  return ((dbits(a.x) | dbits(a.y) | dbits(a.z)) << 1) == 0ull;
}
// The lane's demag rows (C3: its component's row; D3: all three) have +-0
// off the diagonal.
static __device__ __forceinline__ bool offdiag_zero(const double *t, const C3 &) {
  const int c = quad_comp();
  bool z = true;
  for (int i = 0; i < 3; ++i)
    if (i != c) z = z && (dbits(t[3 * c + i]) << 1) == 0ull;
  return z;
}
static __device__ __forceinline__ bool offdiag_zero(const double *t, const D3 &) {
  return ((dbits(t[1]) | dbits(t[2]) | dbits(t[3]) | dbits(t[5]) | dbits(t[6]) | dbits(t[7])) << 1) == 0ull;
}

// v / R.b componentwise, each quotient correctly rounded (recip.cuh).
static __device__ __forceinline__ C3 vdiv(const C3 &a, const Recip &R) { return C3{div_by(a.v, R)}; }
static __device__ __forceinline__ D3 vdiv(const D3 &a, const Recip &R) {
  return d3(div_by(a.x, R), div_by(a.y, R), div_by(a.z, R));
}
// 6 split as recip_of(6.0) would: RN(1/6) and RN(1/6 - RN(1/6)).
static __device__ __forceinline__ Recip recip_six() {
  Recip R;
  R.b = 6.0;
  R.zh = 0x1.5555555555555p-3;
  R.zl = 0x1.5555555555555p-57;
  return R;
}

// The constants of a field-only layer whose driver slots are all constant
// (each slot reads constantValue, as slot_at does with a zero slot mask).
template <class V>
__device__ __forceinline__ FieldOnly<V> field_only_load(const cmtj_layer_t &L, const cmtj_constants_t &c) {
  const DriverCtx dc = {nullptr, 0u, 0};
  FieldOnly<V> f;
  f.Hext = V::axial(L, CMTJ_SLOT_HEXT, 0.0, dc, 0u);
  f.Hoe = V::axial(L, CMTJ_SLOT_HOE, 0.0, dc, 0u);
  f.Hdmi = V::axial(L, CMTJ_SLOT_HDMI, 0.0, dc, 0u);
  f.Hres = V::axial(L, CMTJ_SLOT_HRES, 0.0, dc, 0u);
  f.anis = V::load(L.anis);
  f.K = L.drv[CMTJ_SLOT_ANIS].constantValue;
  f.Jb = L.drv[CMTJ_SLOT_IEC_BOTTOM].constantValue;
  f.Jt = L.drv[CMTJ_SLOT_IEC_TOP].constantValue;
  f.Ms = L.Ms;
  f.Mst = L.Ms * L.thickness;
  f.rMs = recip_of(f.Ms);
  f.rMst = recip_of(f.Mst);
  f.ms_mu0 = L.ms_over_mu0;
  f.damping = L.damping;
  f.conv = L.conv_term;
  f.gyro = c.gyro;
  f.demag = L.demag;
  return f;
}

static __device__ __forceinline__ C3 vsel(bool c, const C3 &a, const C3 &b) { return C3{c ? a.v : b.v}; }
static __device__ __forceinline__ D3 vsel(bool c, const D3 &a, const D3 &b) { return c ? a : b; }

// The warp-uniform flags of FieldOnly.  Called by every lane of the warp;
// dyn: the lane's time-dependent slots (0 when none may be).
template <class V>
__device__ __forceinline__ void field_only_flags(FieldOnly<V> &f, uint32_t dyn) {
  f.diag = __all_sync(kWarpAll, offdiag_zero(f.demag, f.anis));
  f.zoe = __all_sync(kWarpAll, lane_zero(f.Hoe) && !(dyn & (7u << CMTJ_SLOT_HOE)));
  f.zdmi = __all_sync(kWarpAll, lane_zero(f.Hdmi) && !(dyn & (7u << CMTJ_SLOT_HDMI)));
  f.zres = __all_sync(kWarpAll, lane_zero(f.Hres) && !(dyn & (7u << CMTJ_SLOT_HRES)));
}

// rhs()'s IEC term of a field-only layer (the CMTJ_ZERO_J2 form), which
// depends only on the neighbours, frozen for an RK4 step.  one_nb: no lane
// of the warp has two neighbours (its junctions have at most two layers, so
// at least one neighbour of every lane is the zero vector of an edge).  Then
// each lane forms its one term with its own operands, the same operations
// as the branch it would take, and the warp runs one division instead of
// both branches in turn.
template <class V>
__device__ __forceinline__ V field_only_iec(const FieldOnly<V> &f, const V &bottom, const V &top, bool one_nb) {
  const bool zb = is_zero3(bottom), ztop = is_zero3(top);
  if (one_nb) {
    const V r = vdiv(vsel(zb, top, bottom) * (zb ? f.Jt : f.Jb), f.rMst);
    return vsel(zb && ztop, V::zero(), r);
  }
  if (!zb && !ztop) return vdiv(bottom * f.Jb, f.rMst) + vdiv(top * f.Jt, f.rMst);
  if (!zb) return vdiv(bottom * f.Jb, f.rMst);
  if (!ztop) return vdiv(top * f.Jt, f.rMst);
  return V::zero();
}

// rhs() (calculateHeff + solveLLG, junction.hpp:580-815) of a field-only
// layer: the same operations in the same order, with the terms rhs()
// leaves out for such a layer absent and the constant ones preloaded.
// DYN: the field and anisotropy slots are read through slot_at() at the
// stage time (dyn: dynamic_slots(L)), as rhs() reads them.
template <class V, bool DYN>
__device__ __forceinline__ V rhs_field_only(const FieldOnly<V> &f, const cmtj_layer_t &L, double time,
                                            const DriverCtx &dc, uint32_t dyn, const V &m, const V &Hiec,
                                            typename NoDeduce<SideT<V>>::type *side) {
  const V Hext = DYN ? V::axial(L, CMTJ_SLOT_HEXT, time, dc, dyn) : f.Hext;
  const V Hoe = DYN ? V::axial(L, CMTJ_SLOT_HOE, time, dc, dyn) : f.Hoe;
  const V Hdmi = DYN ? V::axial(L, CMTJ_SLOT_HDMI, time, dc, dyn) : f.Hdmi;
  const V Hres = DYN ? V::axial(L, CMTJ_SLOT_HRES, time, dc, dyn) : f.Hres;
  const double K = DYN ? slot_at(L, CMTJ_SLOT_ANIS, time, dc, dyn) : f.K;
  // A layer per lane (D3, large batches, bound by FP64 issue): a diagonal
  // demag tensor takes one product per component, and a slot that is a
  // constant +-0 on every lane of the warp is added without an FP64 add,
  // both bit-exactly.  The quad layout (small batches, bound by the step's
  // latency) ran 3 % slower with them, so it keeps the plain sums.
  constexpr bool kExact0 = V::kLanes == 1;
  const V Hdemag =
      (kExact0 && f.diag) ? tensor_mul_diag(m, f.demag, f.ms_mu0) : tensor_mul(m, f.demag, f.ms_mu0);
  const V Hanis = f.anis * div_by((2 * K) * dot(f.anis, m), f.rMs);
  V H = Hext + Hanis;
  H = H + Hiec;
  // H + Hoe + Hdmi - Hdemag, then + Hres
  H = (kExact0 && f.zoe) ? add_zero(H, Hoe) : H + Hoe;
  H = (kExact0 && f.zdmi) ? add_zero(H, Hdmi) : H + Hdmi;
  H = H - Hdemag;
  H = (kExact0 && f.zres) ? add_zero(H, Hres) : H + Hres;
  if (side) {
    side->K = K;
    side->K2 = 0.0;
    side->Jb = f.Jb;
    side->Jt = f.Jt;
    side->Hext = Hext;
    side->Hiec = Hiec;
    side->Hanis = Hanis;
    side->Hdemag = Hdemag;
  }
  const V prod = cross(m, H);
  const V prod2 = cross(m, prod);
  const V dmdt = prod + prod2 * f.damping;
  return dmdt * -f.gyro * f.conv;
}

// ---- CMTJ_ARITH_FUSED: field-only RK4 layers ------------------------------
// On GB300 every FP64 warp instruction holds its SM sub-partition's FP64
// pipe for about 64 cycles whatever the lane mask, and independent FP64
// instructions of one warp do not overlap, so a step costs about 64 cycles
// per FP64 instruction on its warp.  The reference's operation order needs
// about 290 per RK4 step of a field-only layer (four divisions by Ms, the
// IEC division, the division by 6, a square root and a division in the
// normalisation, each a sequence of about nine).  With constant anisotropy
// and IEC, calculateHeff of such a layer is affine in m:
//   H = Hext + Hoe + Hdmi + Hres + Hiec + A m,
//   A = (2K/Ms) k k^T - N Ms/mu0,
// so the fused form evaluates it as three FMAs per component from a matrix
// formed once per run, with g = -gyro * convTerm * dt folded into A and the
// constant field so that k = dt * dm/dt = p + damping * (m x p), p = m x gH.
// About 50 FP64 instructions per step.

// a * s + b, one rounding per component.
static __device__ __forceinline__ C3 fmav(const C3 &a, double s, const C3 &b) { return C3{fma(a.v, s, b.v)}; }
static __device__ __forceinline__ D3 fmav(const D3 &a, double s, const D3 &b) {
  return d3(fma(a.x, s, b.x), fma(a.y, s, b.y), fma(a.z, s, b.z));
}
// a x b, each component a_i b_j - a_j b_i as fma(a_i, b_j, -(a_j b_i)).
static __device__ __forceinline__ C3 cross_fused(const C3 &a, const C3 &b) {
  const int c = quad_comp();
  const int i = c == 2 ? 0 : c + 1, j = c == 0 ? 2 : c - 1;
  const double ai = quad_get(a.v, i), aj = quad_get(a.v, j), bi = quad_get(b.v, i), bj = quad_get(b.v, j);
  return C3{fma(ai, bj, -(aj * bi))};
}
static __device__ __forceinline__ D3 cross_fused(const D3 &a, const D3 &b) {
  return d3(fma(a.y, b.z, -(a.z * b.y)), fma(a.z, b.x, -(a.x * b.z)), fma(a.x, b.y, -(a.y * b.x)));
}

// v / |v| (CVector::normalize, cvector.hpp:185-192) with 1/|v| from the
// series 1 - e/2 + 3e^2/8 in e = |v|^2 - 1: the first omitted term is below
// 2^-54 for |e| < 2^-27 (two terms) and below 0.6 ulp for |e| < 2^-17 (three
// terms); beyond that 1/|v| is rsqrt(|v|^2).  A zero vector is returned as
// is.  The range tests read the exponent bits of e (integer instructions).
// Every lane of a C3 quad forms the same s, so the quad branches together.
template <class V>
__device__ __forceinline__ V normalized_fused(const V &v) {
  const double x = comp_of(v, 0), y = comp_of(v, 1), z = comp_of(v, 2);
  const double s = fma(z, z, fma(y, y, x * x));
  const double e = s - 1.0;
  const unsigned ex = (unsigned)((unsigned long long)__double_as_longlong(e) >> 52) & 0x7ffu;
  double r;
  if (ex < 1023u - 27u) {
    r = fma(e, -0.5, 1.0);
  } else if (ex < 1023u - 17u) {
    r = fma(e, fma(e, 0.375, -0.5), 1.0);
  } else {
    if ((__double_as_longlong(s) & 0x7fffffffffffffffll) == 0) return v;
    r = rsqrt(s);
  }
  return v * r;
}

// The per-run constants of a fused field-only layer: the columns of g A,
// g times the constant field slots, g Jbottom/(Ms t), g Jtop/(Ms t).
template <class V>
struct Fused {
  V a0, a1, a2, gHc;
  double gcb, gct, g, alpha;
};

template <class V>
__device__ __forceinline__ Fused<V> fused_load(const FieldOnly<V> &f, double dt) {
  Fused<V> u;
  const double g = -f.gyro * f.conv * dt;
  const double kk = (2 * f.K) / f.Ms;
  const double ax = comp_of(f.anis, 0), ay = comp_of(f.anis, 1), az = comp_of(f.anis, 2);
  const double *N = f.demag;
  u.a0 = (f.anis * (kk * ax) - V::make(N[0], N[3], N[6]) * f.ms_mu0) * g;
  u.a1 = (f.anis * (kk * ay) - V::make(N[1], N[4], N[7]) * f.ms_mu0) * g;
  u.a2 = (f.anis * (kk * az) - V::make(N[2], N[5], N[8]) * f.ms_mu0) * g;
  u.gHc = (f.Hext + f.Hoe + f.Hdmi + f.Hres) * g;
  u.gcb = g * (f.Jb / f.Mst);
  u.gct = g * (f.Jt / f.Mst);
  u.g = g;
  u.alpha = f.damping;
  return u;
}

// One RK4 step (Layer::rk4_step, junction.hpp:1017-1041, neighbours frozen
// as in runMultiLayerSolver 1680-1707) of a fused field-only layer.  DYN:
// the field slots are read at each stage time.  Returns as lane_step does.
template <class V, bool DYN>
__device__ __forceinline__ int lane_step_fused(const cmtj_layer_t &L, const Fused<V> &u, V &mag, bool step,
                                               const LaneGeo &g, int n, uint32_t i, double t, double dt,
                                               const double *tables, uint32_t dyn) {
  V below = shfl_vec(mag, g.below_src), above = shfl_vec(mag, g.above_src);
  if (g.l == 0) below = V::zero();
  if (g.l >= n - 1) above = V::zero();
  V next = mag;
  bool nan = false;
  if (step) {
    const V giec = fmav(above, u.gct, below * u.gcb);
    const V gs = DYN ? V::zero() : u.gHc + giec;
    V k = V::zero(), acc = V::zero(), mi = mag;
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      V gh = gs;
      if (DYN) {
        const double ts = s == 0 ? t : (s == 3 ? t + dt : t + 0.5 * dt);
        const DriverCtx dc = {tables, i, s == 0 ? 0 : (s == 3 ? 2 : 1)};
        const V Hc = V::axial(L, CMTJ_SLOT_HEXT, ts, dc, dyn) + V::axial(L, CMTJ_SLOT_HOE, ts, dc, dyn) +
                     V::axial(L, CMTJ_SLOT_HDMI, ts, dc, dyn) + V::axial(L, CMTJ_SLOT_HRES, ts, dc, dyn);
        gh = fmav(Hc, u.g, giec);
      }
      const double mx = comp_of(mi, 0), my = comp_of(mi, 1), mz = comp_of(mi, 2);
      const V h = fmav(u.a2, mz, fmav(u.a1, my, fmav(u.a0, mx, gh)));
      const V p = cross_fused(mi, h);
      const V p2 = cross_fused(mi, p);
      k = fmav(p2, u.alpha, p);
      acc = s == 0 ? k : (s == 3 ? acc + k : fmav(k, 2.0, acc));
      mi = s < 2 ? fmav(k, 0.5, mag) : mag + k;
    }
    next = normalized_fused(fmav(acc, 1.0 / 6.0, mag));
    nan = x_is_nan(next);
  }
  const unsigned bad = __ballot_sync(kWarpAll, nan) & g.group;
  if (bad) {
    const int first = (__ffs(bad) - 1 - g.lead) / V::kLanes;
    if (step && g.l <= first) mag = next;
    return first;
  }
  if (step) mag = next;
  return -1;
}

// One iteration of the fixed-step runner (RK4, Euler-Heun or Heun;
// core/junction.hpp:1668-1815) for the lane's layer of a junction whose
// n layers step (1 under runSingleLayerSolver).  cur overrides the current
// driver (stacks), hres the reserved interaction field (groups).  fo: RK4
// only, the layer is field-only (FieldOnly), with constant drivers or, under
// FDYN, time-dependent field and anisotropy drivers; edge_only: no junction
// of the warp has three or more layers, so no lane has two neighbours;
// sigma_run: the lane's thermal sigma for the whole run (langevin), or -1.
// Returns the first layer whose m became NaN (RK4: the layers above it
// keep their start-of-step m, as when rk4_step throws), or -1.
template <int SOLVER, class V, bool FDYN = false>
__device__ __forceinline__ int lane_step(const cmtj_layer_t &L, const cmtj_constants_t &c, V &mag,
                                         SideT<V> &side, bool step, const LaneGeo &g, int n, uint32_t i, double t,
                                         double dt, const double *tables, bool energies,
                                         const cmtj_driver_t *cur, uint32_t dyn, const double *hres = nullptr,
                                         const FieldOnly<V> *fo = nullptr, bool edge_only = false,
                                         double sigma_run = -1.0) {
  // neighbours at the start of the step; zero beyond the stack's ends
  V below = shfl_vec(mag, g.below_src), above = shfl_vec(mag, g.above_src);
  if (g.l == 0) below = V::zero();
  if (g.l >= n - 1) above = V::zero();
  if constexpr (SOLVER == CMTJ_RK4) {
    // Layer::rk4_step (1017-1041); neighbours frozen for all four stages
    // (runMultiLayerSolver, 1680-1707)
    V next = mag;
    bool nan = false;
    if (step) {
      V k = V::zero(), acc = V::zero();
      if (fo) {
        const V hiec = field_only_iec(*fo, below, above, edge_only);
#pragma unroll
        for (int s = 0; s < 4; ++s) {
          const double ts = s == 0 ? t : (s == 3 ? t + dt : t + 0.5 * dt);
          const V mi = s == 0 ? mag : (s == 3 ? mag + k : mag + k * 0.5);
          const DriverCtx dc = {tables, i, s == 0 ? 0 : (s == 3 ? 2 : 1)};
          k = rhs_field_only<V, FDYN>(*fo, L, ts, dc, dyn, mi, hiec, (s == 3 && energies) ? &side : nullptr) * dt;
          acc = s == 0 ? k : acc + (s == 3 ? k : k * 2.0);
        }
      } else {
#pragma unroll 1
        for (int s = 0; s < 4; ++s) {
          const double ts = s == 0 ? t : (s == 3 ? t + dt : t + 0.5 * dt);
          const V mi = s == 0 ? mag : (s == 3 ? mag + k : mag + k * 0.5);
          const DriverCtx dc = {tables, i, s == 0 ? 0 : (s == 3 ? 2 : 1)};
          k = rhs(L, c, ts, mi, below, above, dc, (s == 3 && energies) ? &side : nullptr, cur, dyn, hres) * dt;
          acc = s == 0 ? k : acc + (s == 3 ? k : k * 2.0);
        }
      }
      next = normalized(mag + vdiv(acc, recip_six()));
      nan = x_is_nan(next);
    }
    const unsigned bad = __ballot_sync(kWarpAll, nan) & g.group;
    if (bad) {
      const int first = (__ffs(bad) - 1 - g.lead) / V::kLanes;
      if (step && g.l <= first) mag = next;
      return first;
    }
    if (step) mag = next;
  } else if constexpr (SOLVER == CMTJ_EULER_HEUN) {
    // eulerHeunSolverStep (1709-1754)
    if (step) {
      const DriverCtx d0 = {tables, i, 0};
      const V dW = langevin<V>(L, c, t, i, d0, dyn, sigma_run);
      const V f = rhs(L, c, t, mag, below, above, d0, energies ? &side : nullptr, cur, dyn, hres);
      const V gt = stoch_torque(L, c, mag, dW);
      const V mNext = mag + gt * sqrt(dt);
      const V g2 = stoch_torque(L, c, mNext, dW);
      mag = normalized(mag + f * dt + smul(0.5, gt + g2) * sqrt(dt));
    }
  } else {
    // heunSolverStep (1756-1815): the corrector sees the neighbours'
    // predictions
    V fn = V::zero(), gn = V::zero(), dW = V::zero(), pred = V::zero();
    if (step) {
      const DriverCtx d0 = {tables, i, 0};
      fn = rhs(L, c, t, mag, below, above, d0, nullptr, cur, dyn, hres);
      dW = langevin<V>(L, c, t, i, d0, dyn, sigma_run);
      gn = stoch_torque(L, c, mag, dW);
      pred = mag + fn * dt + gn * sqrt(dt);
    }
    V pb = shfl_vec(pred, g.below_src), pa = shfl_vec(pred, g.above_src);
    if (g.l == 0) pb = V::zero();
    if (g.l >= n - 1) pa = V::zero();
    if (step) {
      const DriverCtx d2 = {tables, i, 2};
      const V f2 = rhs(L, c, t + dt, pred, pb, pa, d2, energies ? &side : nullptr, cur, dyn, hres);
      const V g2 = stoch_torque(L, c, pred, dW);
      mag = mag + smul(0.5 * dt, fn + f2) + smul(0.5, gn + g2) * sqrt(dt);
      mag = normalized(mag);
    }
  }
  return -1;
}

// The columns of one layer in a log row (logLayerParams, junction.hpp:
// 1580-1636): the energy-log side values, then m.
template <class V>
__device__ __forceinline__ void layer_cols(double *r, const SideT<V> &s, const V &m, bool energies) {
  double *mcol = r;
  if (energies) {
    if (scalar_owner(m)) {
      r[0] = s.K;
      r[1] = s.K2;
      r[2] = s.Jb;
      r[3] = s.Jt;
      r[4] = s.I;
    }
    store3(r + 5, s.Hext);
    store3(r + 8, s.Hiec);
    store3(r + 11, s.Hanis);
    store3(r + 14, s.Hdemag);
    store3(r + 17, V::zero());
    store3(r + 20, s.Hfl);
    store3(r + 23, s.Hdl);
    mcol = r + 26;
  }
  store3(mcol, m);
}

// cos of the angle the CLASSIC magnetoresistance uses (calculate-
// Magnetoresistance 1865-1867): m0 . ref for one layer, m0 . m1 otherwise;
// valid on the lanes of layer 0.
template <class V>
__device__ __forceinline__ double classic_cos(const cmtj_layer_t &L, const V &mag, const LaneGeo &g, int n, int G,
                                              bool layer0) {
  const V m1 = shfl_vec(mag, g.l == 0 && G > 1 ? g.lane + V::kLanes : g.lane);
  const double c01 = dot(mag, m1);
  const double cref = (layer0 && n == 1) ? dot(mag, V::load(L.ref)) : 0.0;
  return n == 1 ? cref : c01;
}

// (Rap - Rp) / 2.0 of calculateMagnetoresistance (junction.hpp:1865-1867),
// the same value on every call: kernels form it once per junction.
__device__ __forceinline__ double classic_half_span(const cmtj_junction_t &J) { return (J.Rap - J.Rp) / 2.0; }

// One log row of the junction (logLayerParams, junction.hpp:1580-1636, and
// the R columns of stripMagnetoResistance 1835-1857).  write: the junction
// logs this step (the same on all its lanes); mine: the lane holds a layer;
// half_span: classic_half_span() of the junction.
template <class V>
__device__ __forceinline__ void lane_log_row(double *r, bool write, bool mine, const cmtj_junction_t *junctions,
                                             int j, const cmtj_layer_t &L, const V &mag, const SideT<V> &side,
                                             const LaneGeo &g, int n, int G, int mr_mode, bool energies, double t,
                                             double half_span) {
  const int width = energies ? CMTJ_ENERGY_COLS : 3;
  // each MR form only when some junction of the warp logs it now (the
  // warp-wide shuffles inside stay converged)
  const double cosT = __any_sync(kWarpAll, write && mr_mode == CMTJ_MR_CLASSIC)
                          ? classic_cos(L, mag, g, n, G, write && g.l == 0)
                          : 0.0;
  double Rx_acc = 0.0, Ry_acc = 0.0;
  if (__any_sync(kWarpAll, write && mr_mode == CMTJ_MR_STRIP)) {
    const double mx = comp_of(mag, 0), my = comp_of(mag, 1), mz = comp_of(mag, 2);
    double inv_x = 0.0, inv_y = 0.0;
    if (write && mine && mr_mode == CMTJ_MR_STRIP) {
      const cmtj_junction_t &J = junctions[j];
      const double Rx = J.Rx0[g.l] + J.AMR_X[g.l] * (mx * mx) + J.SMR_X[g.l] * (my * my);
      const double Ry = J.Ry0[g.l] + 0.5 * J.AHE[g.l] * mz + (J.AMR_Y[g.l] + J.SMR_Y[g.l]) * mx * my;
      inv_x = 1. / Rx;
      inv_y = 1. / Ry;
    }
    for (int q = 0; q < G; ++q) {
      const double a = __shfl_sync(kWarpAll, inv_x, g.lead + q * V::kLanes);
      const double b = __shfl_sync(kWarpAll, inv_y, g.lead + q * V::kLanes);
      if (q < n) {
        Rx_acc = Rx_acc + a;
        Ry_acc = Ry_acc + b;
      }
    }
  }
  if (!write) return;
  if (mine) layer_cols(r + g.l * width, side, mag, energies);
  if (g.jl == 0) {
    const cmtj_junction_t &J = junctions[j];
    double r0 = 0.0, r1 = 0.0;
    if (mr_mode == CMTJ_MR_CLASSIC) {
      r0 = J.Rp + (half_span * (1.0 - cosT));
    } else if (mr_mode == CMTJ_MR_STRIP) {
      r0 = 1 / Rx_acc;
      r1 = 1 / Ry_acc;
    }
    double *rr = r + n * width;
    rr[0] = r0;
    rr[1] = r1;
    rr[2] = 0.0;
    rr[3] = t;
  }
}

}  // namespace cmtjd
