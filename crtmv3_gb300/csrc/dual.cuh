// Forward-mode derivative numbers: a value and N directional derivatives, in
// the scalar S (double, or double-float in the mixed form).  The cloudy
// K-matrix evaluates each layer's optics (cloud/aerosol LUT, combine, phase,
// MOM) on these to get the derivatives of the layer's transmission,
// reflection and source with respect to its gas optical depth, temperature
// and the clouds' and aerosols' amounts and radii.
#pragma once

#include <math.h>

#include "dd.cuh"

#ifndef CRTM_HD
#ifdef __CUDACC__
#define CRTM_HD __host__ __device__ inline
#else
#define CRTM_HD inline
#endif
#endif

namespace crtm {

// keep the plain overloads visible next to the Dual and DD ones
using ::exp;
using ::expm1;
using ::fabs;
using ::sqrt;

template <int N, class S = double>
struct Dual {
  S v;
  S d[N];
  CRTM_HD Dual() : v(0.0) { for (int i = 0; i < N; i++) d[i] = S(0.0); }
  CRTM_HD Dual(double x) : v(x) { for (int i = 0; i < N; i++) d[i] = S(0.0); }   // NOLINT: implicit
  CRTM_HD Dual(const S& x, int) : v(x) { for (int i = 0; i < N; i++) d[i] = S(0.0); }
  CRTM_HD explicit operator double() const { return (double)v; }
  CRTM_HD Dual& operator+=(const Dual& b) { v += b.v; for (int i = 0; i < N; i++) d[i] += b.d[i]; return *this; }
  CRTM_HD Dual& operator-=(const Dual& b) { v -= b.v; for (int i = 0; i < N; i++) d[i] -= b.d[i]; return *this; }
  CRTM_HD Dual& operator*=(const Dual& b) {
    for (int i = 0; i < N; i++) d[i] = d[i] * b.v + v * b.d[i];
    v *= b.v;
    return *this;
  }
  CRTM_HD Dual& operator/=(const Dual& b) {
    const S r = S(1.0) / b.v, q = v * r;
    for (int i = 0; i < N; i++) d[i] = (d[i] - q * b.d[i]) * r;
    v = q;
    return *this;
  }
};

template <int N, class S> CRTM_HD Dual<N, S> operator+(Dual<N, S> a, const Dual<N, S>& b) { return a += b; }
template <int N, class S> CRTM_HD Dual<N, S> operator-(Dual<N, S> a, const Dual<N, S>& b) { return a -= b; }
template <int N, class S> CRTM_HD Dual<N, S> operator*(Dual<N, S> a, const Dual<N, S>& b) { return a *= b; }
template <int N, class S> CRTM_HD Dual<N, S> operator/(Dual<N, S> a, const Dual<N, S>& b) { return a /= b; }
template <int N, class S> CRTM_HD Dual<N, S> operator+(Dual<N, S> a, double b) { a.v += S(b); return a; }
template <int N, class S> CRTM_HD Dual<N, S> operator+(double b, Dual<N, S> a) { a.v += S(b); return a; }
template <int N, class S> CRTM_HD Dual<N, S> operator-(Dual<N, S> a, double b) { a.v -= S(b); return a; }
template <int N, class S> CRTM_HD Dual<N, S> operator-(double b, const Dual<N, S>& a) {
  Dual<N, S> r;
  r.v = S(b) - a.v;
  for (int i = 0; i < N; i++) r.d[i] = -a.d[i];
  return r;
}
template <int N, class S> CRTM_HD Dual<N, S> operator*(Dual<N, S> a, double b) {
  const S bs(b);
  a.v *= bs;
  for (int i = 0; i < N; i++) a.d[i] *= bs;
  return a;
}
template <int N, class S> CRTM_HD Dual<N, S> operator*(double b, Dual<N, S> a) { return a * b; }
template <int N, class S> CRTM_HD Dual<N, S> operator/(Dual<N, S> a, double b) { return a * (1.0 / b); }
template <int N, class S> CRTM_HD Dual<N, S> operator/(double b, const Dual<N, S>& a) { return Dual<N, S>(b) / a; }
template <int N, class S> CRTM_HD Dual<N, S> operator-(const Dual<N, S>& a) { return 0.0 - a; }

template <int N, class S> CRTM_HD bool operator<(const Dual<N, S>& a, const Dual<N, S>& b) { return a.v < b.v; }
template <int N, class S> CRTM_HD bool operator>(const Dual<N, S>& a, const Dual<N, S>& b) { return a.v > b.v; }
template <int N, class S> CRTM_HD bool operator<=(const Dual<N, S>& a, const Dual<N, S>& b) { return a.v <= b.v; }
template <int N, class S> CRTM_HD bool operator>=(const Dual<N, S>& a, const Dual<N, S>& b) { return a.v >= b.v; }
template <int N, class S> CRTM_HD bool operator<(const Dual<N, S>& a, double b) { return a.v < b; }
template <int N, class S> CRTM_HD bool operator>(const Dual<N, S>& a, double b) { return a.v > b; }
template <int N, class S> CRTM_HD bool operator<=(const Dual<N, S>& a, double b) { return a.v <= b; }
template <int N, class S> CRTM_HD bool operator>=(const Dual<N, S>& a, double b) { return a.v >= b; }
template <int N, class S> CRTM_HD bool operator==(const Dual<N, S>& a, double b) { return a.v == b; }

template <int N, class S> CRTM_HD Dual<N, S> sqrt(const Dual<N, S>& a) {
  Dual<N, S> r;
  r.v = sqrt(a.v);
  const S g = S(0.5) / r.v;
  for (int i = 0; i < N; i++) r.d[i] = a.d[i] * g;
  return r;
}
template <int N, class S> CRTM_HD Dual<N, S> exp(const Dual<N, S>& a) {
  Dual<N, S> r;
  r.v = exp(a.v);
  for (int i = 0; i < N; i++) r.d[i] = a.d[i] * r.v;
  return r;
}
template <int N, class S> CRTM_HD Dual<N, S> expm1(const Dual<N, S>& a) {
  Dual<N, S> r;
  r.v = expm1(a.v);
  const S e = r.v + S(1.0);
  for (int i = 0; i < N; i++) r.d[i] = a.d[i] * e;
  return r;
}
template <int N, class S> CRTM_HD Dual<N, S> fabs(const Dual<N, S>& a) { return a.v < 0.0 ? -a : a; }

CRTM_HD double value_of(double x) { return x; }
CRTM_HD bool is_zero(double x) { return x == 0.0; }
CRTM_HD bool is_zero(float x) { return x == 0.0f; }
template <int N, class S> CRTM_HD bool is_zero(const Dual<N, S>& x) {
  if (!is_zero(x.v)) return false;
  for (int i = 0; i < N; i++)
    if (!is_zero(x.d[i])) return false;
  return true;
}
template <int N, class S> CRTM_HD double value_of(const Dual<N, S>& x) { return value_of(x.v); }
// derivative part i as a double
CRTM_HD double part(double x) { return x; }
CRTM_HD double part(const DD& x) { return (double)x; }

}  // namespace crtm
