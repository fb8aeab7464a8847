// Floating-point operation count of one scattering layer's MOM work in the
// cloudy K-matrix (the scatter_reverse_kernel's layer: phase blocks, the
// loss-form MOM forward and its reverse sweep, the phase blocks' adjoint),
// taken by running the library's own header code on a counting number type.
// Every +, -, *, / and every sqrt / exp / expm1 counts as one operation (a
// fused multiply-add as two).  The benchmark's roofline numerator for that
// stage is a fit to these counts.
#include <cmath>
#include <cstdint>

static int64_t g_ops = 0;

struct FC {
  float v;
  FC() : v(0.0f) {}
  FC(double x) : v((float)x) {}
  explicit operator double() const { return v; }
  FC& operator+=(const FC& b) { v += b.v; g_ops++; return *this; }
  FC& operator-=(const FC& b) { v -= b.v; g_ops++; return *this; }
  FC& operator*=(const FC& b) { v *= b.v; g_ops++; return *this; }
  FC& operator/=(const FC& b) { v /= b.v; g_ops++; return *this; }
};
inline FC operator+(FC a, const FC& b) { return a += b; }
inline FC operator-(FC a, const FC& b) { return a -= b; }
inline FC operator*(FC a, const FC& b) { return a *= b; }
inline FC operator/(FC a, const FC& b) { return a /= b; }
inline FC operator-(const FC& a) { FC r; r.v = -a.v; return r; }
inline bool operator<(const FC& a, const FC& b) { return a.v < b.v; }
inline bool operator>(const FC& a, const FC& b) { return a.v > b.v; }
inline bool operator<=(const FC& a, const FC& b) { return a.v <= b.v; }
inline bool operator>=(const FC& a, const FC& b) { return a.v >= b.v; }
inline bool operator==(const FC& a, const FC& b) { return a.v == b.v; }
inline bool operator!=(const FC& a, const FC& b) { return a.v != b.v; }
inline FC sqrt(const FC& a) { g_ops++; return FC(std::sqrt(a.v)); }
inline FC exp(const FC& a) { g_ops++; return FC(std::exp(a.v)); }
inline FC expm1(const FC& a) { g_ops++; return FC(std::expm1(a.v)); }
inline FC fabs(const FC& a) { return FC(std::fabs(a.v)); }
inline double value_of(const FC& x) { return x.v; }
inline bool is_zero(const FC& x) { return x.v == 0.0f; }

#include "scatter_adjoint.cuh"

namespace crtm {
template <> struct JacobiEps<FC> { static constexpr double value = 1.0e-14; };
}  // namespace crtm

using namespace crtm;

static GaussTable make_gauss() {
  GaussTable g;
  gauss_table_host(g);
  return g;
}

// Operations of one layer at nleg Legendre terms (nS = (nleg + 2) / 2 quadrature
// angles, plus the sensor angle when it is not one of them), single-scattering
// albedo w and optical depth tau; returns -1 where MOM fails.
extern "C" long long fc_layer_ops(int nleg, double mu_sensor, double w, double tau) {
  static GaussTable gt = make_gauss();
  StreamSet<SC_NZ_MAX, double> S;
  if (stream_set<SC_NZ_MAX, double>(nleg, mu_sensor, -1, gt, S)) return -1;
  const int nS = S.nS, nZ = S.nZ;
  FC mu[SC_NZ_MAX], wt[SC_NZ_MAX], P[SC_NZ_MAX][SC_NLEG_MAX + 1], pc[SC_NLEG_MAX + 1];
  for (int i = 0; i < nZ; i++) {
    mu[i] = FC(S.mu[i]);
    wt[i] = FC(S.wt[i]);
    for (int l = 0; l <= nleg; l++) P[i][l] = FC(S.P[i][l]);
  }
  for (int l = 0; l <= nleg; l++) pc[l] = FC(0.5 * std::pow(0.7, l));
  Mat<SC_NZ_MAX, FC> ff, bb, Tb, Rb, ffb, bbb;
  FC sb[SC_NZ_MAX], wb, tb, Bb, pcb[SC_NLEG_MAX + 1];
  for (int i = 0; i < nZ; i++) {
    sb[i] = FC(0.3 + 0.01 * i);
    for (int j = 0; j < nZ; j++) { Tb.a[i][j] = FC(0.1 * (i + 1) - 0.02 * j); Rb.a[i][j] = FC(0.05 * (j + 1)); }
  }
  g_ops = 0;
  phase_blocks<SC_NZ_MAX, FC>(nS, nZ, nleg, pc, P, wt, ff, bb);
  double gap = 1.0;
  if (!ada_layer_adjoint<SC_NZ_MAX, FC>(nS, nZ, FC(w), FC(tau), mu, wt, ff, bb, FC(1.0), Tb, Rb, sb, &wb, &tb,
                                         ffb, bbb, &Bb, &gap))
    return -1;
  phase_blocks_adjoint<SC_NZ_MAX, FC>(nS, nZ, nleg, pc, P, wt, ffb, bbb, pcb);
  return g_ops;
}
