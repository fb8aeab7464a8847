// Forward-mode derivative numbers: a value and N directional derivatives.
// The cloudy K-matrix evaluates each layer's optics (cloud/aerosol LUT,
// combine, phase, MOM) on these to get the layer's transmission, reflection
// and source together with their derivatives with respect to the layer's gas
// optical depth and temperature.
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

// keep the plain overloads visible next to the Dual ones below
using ::exp;
using ::fabs;
using ::sqrt;

template <int N>
struct Dual {
  double v;
  double d[N];
  CRTM_HD Dual() : v(0.0) { for (int i = 0; i < N; i++) d[i] = 0.0; }
  CRTM_HD Dual(double x) : v(x) { for (int i = 0; i < N; i++) d[i] = 0.0; }   // NOLINT: implicit from double
  CRTM_HD explicit operator double() const { return v; }
  CRTM_HD Dual& operator+=(const Dual& b) { v += b.v; for (int i = 0; i < N; i++) d[i] += b.d[i]; return *this; }
  CRTM_HD Dual& operator-=(const Dual& b) { v -= b.v; for (int i = 0; i < N; i++) d[i] -= b.d[i]; return *this; }
  CRTM_HD Dual& operator*=(const Dual& b) {
    for (int i = 0; i < N; i++) d[i] = d[i] * b.v + v * b.d[i];
    v *= b.v;
    return *this;
  }
  CRTM_HD Dual& operator/=(const Dual& b) {
    const double r = 1.0 / b.v, q = v * r;
    for (int i = 0; i < N; i++) d[i] = (d[i] - q * b.d[i]) * r;
    v = q;
    return *this;
  }
};

template <int N> CRTM_HD Dual<N> operator+(Dual<N> a, const Dual<N>& b) { return a += b; }
template <int N> CRTM_HD Dual<N> operator-(Dual<N> a, const Dual<N>& b) { return a -= b; }
template <int N> CRTM_HD Dual<N> operator*(Dual<N> a, const Dual<N>& b) { return a *= b; }
template <int N> CRTM_HD Dual<N> operator/(Dual<N> a, const Dual<N>& b) { return a /= b; }
template <int N> CRTM_HD Dual<N> operator+(Dual<N> a, double b) { a.v += b; return a; }
template <int N> CRTM_HD Dual<N> operator+(double b, Dual<N> a) { a.v += b; return a; }
template <int N> CRTM_HD Dual<N> operator-(Dual<N> a, double b) { a.v -= b; return a; }
template <int N> CRTM_HD Dual<N> operator-(double b, const Dual<N>& a) {
  Dual<N> r;
  r.v = b - a.v;
  for (int i = 0; i < N; i++) r.d[i] = -a.d[i];
  return r;
}
template <int N> CRTM_HD Dual<N> operator*(Dual<N> a, double b) { a.v *= b; for (int i = 0; i < N; i++) a.d[i] *= b; return a; }
template <int N> CRTM_HD Dual<N> operator*(double b, Dual<N> a) { return a * b; }
template <int N> CRTM_HD Dual<N> operator/(Dual<N> a, double b) { return a * (1.0 / b); }
template <int N> CRTM_HD Dual<N> operator/(double b, const Dual<N>& a) { return Dual<N>(b) / a; }
template <int N> CRTM_HD Dual<N> operator-(const Dual<N>& a) { return 0.0 - a; }

template <int N> CRTM_HD bool operator<(const Dual<N>& a, const Dual<N>& b) { return a.v < b.v; }
template <int N> CRTM_HD bool operator>(const Dual<N>& a, const Dual<N>& b) { return a.v > b.v; }
template <int N> CRTM_HD bool operator<=(const Dual<N>& a, const Dual<N>& b) { return a.v <= b.v; }
template <int N> CRTM_HD bool operator>=(const Dual<N>& a, const Dual<N>& b) { return a.v >= b.v; }
template <int N> CRTM_HD bool operator<(const Dual<N>& a, double b) { return a.v < b; }
template <int N> CRTM_HD bool operator>(const Dual<N>& a, double b) { return a.v > b; }
template <int N> CRTM_HD bool operator<=(const Dual<N>& a, double b) { return a.v <= b; }
template <int N> CRTM_HD bool operator>=(const Dual<N>& a, double b) { return a.v >= b; }
template <int N> CRTM_HD bool operator==(const Dual<N>& a, double b) { return a.v == b; }

template <int N> CRTM_HD Dual<N> sqrt(const Dual<N>& a) {
  Dual<N> r;
  r.v = ::sqrt(a.v);
  const double g = 0.5 / r.v;
  for (int i = 0; i < N; i++) r.d[i] = a.d[i] * g;
  return r;
}
template <int N> CRTM_HD Dual<N> exp(const Dual<N>& a) {
  Dual<N> r;
  r.v = ::exp(a.v);
  for (int i = 0; i < N; i++) r.d[i] = a.d[i] * r.v;
  return r;
}
template <int N> CRTM_HD Dual<N> fabs(const Dual<N>& a) { return a.v < 0.0 ? -a : a; }

CRTM_HD double value_of(double x) { return x; }
CRTM_HD bool is_zero(double x) { return x == 0.0; }
CRTM_HD bool is_zero(float x) { return x == 0.0f; }
template <int N> CRTM_HD bool is_zero(const Dual<N>& x) {
  if (x.v != 0.0) return false;
  for (int i = 0; i < N; i++)
    if (x.d[i] != 0.0) return false;
  return true;
}
template <int N> CRTM_HD double value_of(const Dual<N>& x) { return x.v; }

}  // namespace crtm
