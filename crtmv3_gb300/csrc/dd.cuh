// Double-float numbers: an unevaluated sum hi + lo of two FP32 values, about
// 48 significant bits while |x| > ~1e-30 (below that the low word leaves
// FP32's normal range and the precision falls towards FP32's; the layer
// solver's values stay far above it, or are negligible terms).  GB300 issues
// FP32 fused multiply-adds at roughly 64 times its FP64 rate, so the
// scattering layer solver (MOM: eigenproblem, inversions, products) runs on
// these in the mixed form; FP64 stays in the all-FP64 form.
//
// Algorithms: the error-free transformations two-sum (Knuth) and two-product
// with a fused multiply-add, with renormalisation by fast two-sum (Dekker),
// as published for float-float arithmetic on GPUs; division and square root
// by one correction step of the FP32 quotient / root.  exp goes through FP64
// (a handful of calls per layer).
#pragma once

#include <math.h>

#ifndef CRTM_HD
#ifdef __CUDACC__
#define CRTM_HD __host__ __device__ inline
#else
#define CRTM_HD inline
#endif
#endif

namespace crtm {

struct DD {
  float hi, lo;
  CRTM_HD DD() : hi(0.0f), lo(0.0f) {}
  CRTM_HD DD(double x) {   // NOLINT: implicit from double
    hi = (float)x;
    lo = (float)(x - (double)hi);
  }
  CRTM_HD DD(float h, float l, int) : hi(h), lo(l) {}
  CRTM_HD explicit operator double() const { return (double)hi + (double)lo; }
  CRTM_HD explicit operator float() const { return hi + lo; }
};

namespace dd_detail {
// s + e = a + b exactly
CRTM_HD DD two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  const float e = (a - (s - bb)) + (b - bb);
  return DD(s, e, 0);
}
// s + e = a + b exactly when |a| >= |b|
CRTM_HD DD fast_two_sum(float a, float b) {
  const float s = a + b;
  return DD(s, b - (s - a), 0);
}
}  // namespace dd_detail

CRTM_HD DD operator+(const DD& a, const DD& b) {
  DD s = dd_detail::two_sum(a.hi, b.hi);
  const DD t = dd_detail::two_sum(a.lo, b.lo);
  s.lo += t.hi;
  s = dd_detail::fast_two_sum(s.hi, s.lo);
  s.lo += t.lo;
  return dd_detail::fast_two_sum(s.hi, s.lo);
}
CRTM_HD DD operator-(const DD& a) { return DD(-a.hi, -a.lo, 0); }
CRTM_HD DD operator-(const DD& a, const DD& b) { return a + (-b); }
CRTM_HD DD operator*(const DD& a, const DD& b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  return dd_detail::fast_two_sum(p, e);
}
CRTM_HD DD operator/(const DD& a, const DD& b) {
  const float q1 = a.hi / b.hi;
  // r = a - q1 b, exactly enough for the correction
  const float p = q1 * b.hi;
  const float pe = fmaf(q1, b.hi, -p);
  const DD r = a - DD(p, fmaf(q1, b.lo, pe), 0);
  const float q2 = r.hi / b.hi;
  return dd_detail::fast_two_sum(q1, q2);
}
CRTM_HD DD& operator+=(DD& a, const DD& b) { return a = a + b; }
CRTM_HD DD& operator-=(DD& a, const DD& b) { return a = a - b; }
CRTM_HD DD& operator*=(DD& a, const DD& b) { return a = a * b; }
CRTM_HD DD& operator/=(DD& a, const DD& b) { return a = a / b; }

CRTM_HD bool operator<(const DD& a, const DD& b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
CRTM_HD bool operator>(const DD& a, const DD& b) { return b < a; }
CRTM_HD bool operator<=(const DD& a, const DD& b) { return !(b < a); }
CRTM_HD bool operator>=(const DD& a, const DD& b) { return !(a < b); }
CRTM_HD bool operator==(const DD& a, const DD& b) { return a.hi == b.hi && a.lo == b.lo; }
CRTM_HD bool operator!=(const DD& a, const DD& b) { return !(a == b); }
// comparisons with plain constants (thresholds)
CRTM_HD bool operator<(const DD& a, double b) { return a < DD(b); }
CRTM_HD bool operator>(const DD& a, double b) { return a > DD(b); }
CRTM_HD bool operator<=(const DD& a, double b) { return a <= DD(b); }
CRTM_HD bool operator>=(const DD& a, double b) { return a >= DD(b); }
CRTM_HD bool operator==(const DD& a, double b) { return a == DD(b); }

CRTM_HD DD fabs(const DD& a) { return a.hi < 0.0f ? -a : a; }
CRTM_HD DD sqrt(const DD& a) {
  if (!(a.hi > 0.0f)) return DD();
  const float s = sqrtf(a.hi);
  // one Newton step on s: s + (a - s^2) / (2 s)
  const float p = s * s;
  const DD r = a - DD(p, fmaf(s, s, -p), 0);
  return dd_detail::fast_two_sum(s, r.hi / (2.0f * s));
}
CRTM_HD DD exp(const DD& a) { return DD(::exp((double)a)); }
CRTM_HD DD expm1(const DD& a) { return DD(::expm1((double)a)); }

CRTM_HD double value_of(const DD& x) { return (double)x; }
CRTM_HD bool is_zero(const DD& x) { return x.hi == 0.0f && x.lo == 0.0f; }

// Jacobi convergence threshold on (off-diagonal / diagonal) squared norms
template <class T> struct JacobiEps { static constexpr double value = 1.0e-32; };
template <> struct JacobiEps<float> { static constexpr double value = 1.0e-14; };
template <> struct JacobiEps<DD> { static constexpr double value = 1.0e-27; };

}  // namespace crtm
