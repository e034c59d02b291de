// Correctly rounded division by a per-run constant, in three FP64
// instructions and an integer test instead of a full division.
//
// b > 0 is split once as zh + zl with zh = RN(1/b) and zl = RN(1/b - zh)
// (recip_of).  For a / b (div_by):
//   q = RN(a zh + RN(a zl)) is within an ulp of a/b (zh + zl is 1/b to about
//       2^-105 relative), so
//   r = a - q b is exact and comes out of one FMA, and
//   q = RN(a/b) exactly when |a/b - q| < ulp(q)/2, i.e. |r| < b ulp(q)/2:
//   a quotient of two doubles is never a midpoint, so no tie arises.  When
//   |q| is a power of two the doubles below it are twice as dense, and the
//   test uses b ulp(q)/4 on both sides (conservative).
// The bound b 2^(E(q) - 53) is formed on b's exponent bits and compared with
// |r| as integers (both non-negative doubles).  a = +-0 returns a.  When the
// test fails, or q or the bound would leave the normal range, a / b is
// divided in full, so the result is always the IEEE quotient.
#pragma once

namespace cmtjd {

struct Recip {
  double b, zh, zl;
};

static __device__ __forceinline__ Recip recip_of(double b) {
  Recip R;
  R.b = b;
  R.zh = 1.0 / b;
  R.zl = fma(-R.zh, b, 1.0) / b;  // 1 - zh b is exact
  return R;
}

// The full IEEE division, kept out of line so that it runs only when the
// test below fails.
static __device__ __noinline__ double div_full(double a, double b) { return a / b; }

static __device__ __forceinline__ double div_by(double a, const Recip &R) {
  const unsigned long long ab = (unsigned long long)__double_as_longlong(a);
  if ((ab << 1) == 0ull) return a;  // +-0 / b
  const double q = fma(a, R.zh, a * R.zl);
  const double r = fma(-q, R.b, a);
  const unsigned long long qb = (unsigned long long)__double_as_longlong(q);
  const int eq = (int)((qb >> 52) & 0x7ffu);
  const int pow2 = (qb & 0xfffffffffffffull) == 0ull ? 1 : 0;
  const unsigned long long bb = (unsigned long long)__double_as_longlong(R.b);
  const int eh = (int)(bb >> 52) + (eq - 1023) - 53 - pow2;
  const unsigned long long rb = (unsigned long long)__double_as_longlong(r) & 0x7fffffffffffffffull;
  const unsigned long long hb = (bb & 0xfffffffffffffull) | ((unsigned long long)(eh > 0 ? eh : 0) << 52);
  // eh > 54: every multiple of ulp(q) ulp(b) below the bound is a double,
  // so r is exact even where it falls below the normal range
  const bool ok = eq > 64 && eq < 1983 && eh > 54 && eh < 2047 && rb < hb;
  if (ok) return q;
  return div_full(a, R.b);
}

}  // namespace cmtjd
