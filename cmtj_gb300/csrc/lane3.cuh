// C3: a 3-vector spread over a quad of lanes (lanes 4q, 4q+1, 4q+2 hold x,
// y, z; lane 4q+3 repeats z), for the FP64 plain-form physics of
// plain_f64.cuh.
//
// Each operation forms the same IEEE operations in the same order as the
// one-lane D3 version: a dot product is (ax*bx + ay*by) + az*bz with the
// three products gathered from the quad, a cross product component is
// a_i*b_j - a_j*b_i from the quad's other two lanes, and a tensor row is
// (t0*mx + t1*my) + t2*mz.  Values therefore do not depend on the layout.
// A step is bound by its warp's FP64 instructions (each holds the SM
// sub-partition's FP64 pipe for about 64 cycles on GB300, whatever the lane
// mask), so spreading the components cuts a step's FP64 instructions about
// 2.5-fold for a few shuffles.  The lanes of a quad always take the same
// branches (they hold one layer), so the quad-masked shuffles below are
// always converged.
#pragma once
#include "plain_f64.cuh"

namespace cmtjd {

static __device__ __forceinline__ int quad_comp() {
  const int c = threadIdx.x & 3;
  return c < 2 ? c : 2;
}
static __device__ __forceinline__ bool quad_owner() { return (threadIdx.x & 3) != 3; }
static __device__ __forceinline__ int quad_lead() { return (threadIdx.x & 31) & ~3; }
static __device__ __forceinline__ unsigned quad_mask() { return 0xFu << quad_lead(); }
static __device__ __forceinline__ double quad_get(double v, int k) {
  return __shfl_sync(quad_mask(), v, k, 4);  // lane k of this lane's quad
}

struct C3 {
  double v;  // this lane's component
  static constexpr int kLanes = 4;
  static __device__ __forceinline__ C3 zero() { return C3{0.0}; }
  static __device__ __forceinline__ C3 load(const double *p) { return C3{p[quad_comp()]}; }
  static __device__ __forceinline__ C3 make(double x, double y, double z) {
    const int c = quad_comp();
    return C3{c == 0 ? x : (c == 1 ? y : z)};
  }
  static __device__ __forceinline__ C3 axial(const cmtj_layer_t &L, int s, double t, const DriverCtx &dc,
                                             uint32_t dyn) {
    return C3{slot_at(L, s + quad_comp(), t, dc, dyn)};
  }
};

static __device__ __forceinline__ C3 operator+(const C3 &a, const C3 &b) { return C3{a.v + b.v}; }
static __device__ __forceinline__ C3 operator-(const C3 &a, const C3 &b) { return C3{a.v - b.v}; }
static __device__ __forceinline__ C3 operator*(const C3 &a, double s) { return C3{a.v * s}; }
static __device__ __forceinline__ C3 operator/(const C3 &a, double s) { return C3{a.v / s}; }
static __device__ __forceinline__ C3 smul(double s, const C3 &a) { return C3{s * a.v}; }
static __device__ __forceinline__ double dot(const C3 &a, const C3 &b) {
  const double p = a.v * b.v;
  return quad_get(p, 0) + quad_get(p, 1) + quad_get(p, 2);
}
static __device__ __forceinline__ C3 cross(const C3 &a, const C3 &b) {
  const int c = quad_comp();
  const int i = c == 2 ? 0 : c + 1, j = c == 0 ? 2 : c - 1;
  const double ai = quad_get(a.v, i), aj = quad_get(a.v, j), bi = quad_get(b.v, i), bj = quad_get(b.v, j);
  return C3{ai * bj - aj * bi};
}
static __device__ __forceinline__ C3 tensor_mul(const C3 &m, const double *t, double ms_mu0) {
  const double mx = quad_get(m.v, 0), my = quad_get(m.v, 1), mz = quad_get(m.v, 2);
  const double *r = t + 3 * quad_comp();
  return C3{(r[0] * mx + r[1] * my + r[2] * mz) * ms_mu0};
}
static __device__ __forceinline__ bool is_zero3(const C3 &a) {
  const bool nz = (__double_as_longlong(a.v) & 0x7fffffffffffffffull) != 0ull;
  return (__ballot_sync(quad_mask(), nz) & quad_mask()) == 0u;
}

// Component k (0, 1, 2) of a vector, on every lane of the quad / the lane.
static __device__ __forceinline__ double comp_of(const C3 &a, int k) { return quad_get(a.v, k); }
static __device__ __forceinline__ double comp_of(const D3 &a, int k) { return k == 0 ? a.x : (k == 1 ? a.y : a.z); }

// Stores a vector at dst[0..2] (each owning lane its component).
static __device__ __forceinline__ void store3(double *dst, const C3 &a) {
  if (quad_owner()) dst[quad_comp()] = a.v;
}
static __device__ __forceinline__ void store3(double *dst, const D3 &a) {
  dst[0] = a.x;
  dst[1] = a.y;
  dst[2] = a.z;
}

// The lane that writes a layer's scalars.
static __device__ __forceinline__ bool scalar_owner(const C3 &) { return (threadIdx.x & 3) == 0; }
static __device__ __forceinline__ bool scalar_owner(const D3 &) { return true; }

// isnan(v) as an integer test on the bits (exponent all ones, mantissa
// non-zero), which takes no FP64 pipe slot.
static __device__ __forceinline__ bool nan_bits(double v) {
  return ((unsigned long long)__double_as_longlong(v) << 1) > 0xffe0000000000000ull;
}

// isnan of the x component, true on the lane that holds it.
static __device__ __forceinline__ bool x_is_nan(const C3 &a) { return (threadIdx.x & 3) == 0 && nan_bits(a.v); }
static __device__ __forceinline__ bool x_is_nan(const D3 &a) { return nan_bits(a.x); }

// isnan of the x component, on every lane of the quad.
static __device__ __forceinline__ bool x_nan_all(const C3 &a) {
  return (__ballot_sync(quad_mask(), x_is_nan(a)) & quad_mask()) != 0u;
}

// The same component of the vector another lane holds.
static __device__ __forceinline__ C3 shfl_vec(const C3 &a, int src) { return C3{__shfl_sync(0xffffffffu, a.v, src)}; }
static __device__ __forceinline__ D3 shfl_vec(const D3 &a, int src) {
  return d3(__shfl_sync(0xffffffffu, a.x, src), __shfl_sync(0xffffffffu, a.y, src),
            __shfl_sync(0xffffffffu, a.z, src));
}

}  // namespace cmtjd
