// Cloud scattering and the ADA solver for one (profile, channel): the physics
// of the cloudy forward path, written for one GPU thread per pair and
// compiled for the CPU as well (tests/harness).
//
// Reference behaviour followed (JCSDA/CRTMv3):
//   LUT interpolation   src/Interpolation/CRTM_Interpolation.f90 (Find_Random_Index
//                       :769-788, LPoly :832-860, Interp_1D/2D/3D :226-275)
//   cloud optics        src/AtmScatter/CRTM_CloudScatter.f90:221-399, :927-1009, :1269-1416
//   stream count        src/RTSolution/CRTM_RTSolution.f90:1204-1260
//   combine             src/AtmOptics/CRTM_AtmOptics.f90:369-432
//   angles and phase    src/RTSolution/Common_RTSolution.f90:189-458, 1857-1943, 2885-2940
//   ADA                 src/RTSolution/ADA/ADA_Module.f90:97-258, 262-354, 552-743
//
// Differences of form (same numbers):
//   - Layer optics are computed inside the adding loop, one layer at a time
//     from the surface up, so no per-layer phase arrays are kept.
//   - MOM's eigenproblem HH = (PP-PM)(PP+PM) is solved in its symmetric form
//     (Cholesky of the PD matrix D^-1/2 (I - s W^1/2 (F+B) W^1/2) D^-1/2 and
//     Jacobi rotations).  Only the eigenvalues and the eigenvectors' span
//     enter the layer transmission and reflection; their scaling and order
//     cancel in MOM's formulas.
#pragma once

#include <math.h>

#include <type_traits>

#include "dual.cuh"
#include "odps_physics.cuh"

namespace crtm {

constexpr int SC_NLEG_MAX = 16;          // MAX_N_LEGENDRE_TERMS
constexpr int SC_NZ_MAX = 10;            // 9 streams (16-stream option) + the sensor angle
constexpr int SC_KMAX = 1024;            // layers of a profile with clouds or aerosols
constexpr int SC_NC_MAX = 8;             // clouds (and aerosols) of a profile
constexpr double WATER_CONTENT_THRESHOLD = 1.0e-6;   // CRTM_Parameters.f90:256
constexpr double AEROSOL_CONTENT_THRESHOLD = 1.0e-9; // CRTM_Parameters.f90:255
constexpr double MIN_COVERAGE = 1.0e-12;             // CRTM_Parameters.f90:257
constexpr double FRACTIONAL_COVERAGE = 1.0e-6;       // CRTM_Atmosphere.f90:164
constexpr double BS_THRESHOLD = 1.0e-10;             // CRTM_Parameters.f90:260
constexpr double MAX_ALBEDO = 0.999999;              // RTV_Define.f90:77
constexpr double PHASE_THRESHOLD = 1.0e-7;           // RTV_Define.f90:74
constexpr double DELTA_OPTICAL_DEPTH = 1.0e-8;       // RTV_Define.f90:76
constexpr double ANGLE_THRESHOLD = 1.0e-7;           // RTV_Define.f90:70
// K-matrix contraction: relative gap between a MOM quadrature eigenvalue and
// the sensor angle's below which the derivatives are taken at shifted sensor
// angles mu (1 +- SENSOR_SHIFT)
constexpr double SENSOR_GAP_MIN = 1.0e-3;
constexpr double SENSOR_SHIFT = 1.0e-3;
// FP32 layer solver: below these relative gaps (forward; reverse sweep) the
// sensor angle's MOM eigenvector, which divides by the gap, loses too much
// of FP32's precision (about eps/gap in T and R, eps/gap^2 in their
// derivatives); such a layer is solved at sensor angles mu (1 +- h),
// mu (1 +- 2h), h = FP32_SENSOR_SHIFT, and extrapolated, in FP32.
constexpr double FP32_GAP_MIN = 3.0e-3;
constexpr double FP32_ADJ_GAP_MIN = 3.0e-3;
constexpr double FP32_SENSOR_SHIFT = 1.0e-2;
// FP32 reverse sweep: layers whose single-scattering albedo is within this
// of 1 are differentiated in FP64 (the albedo's adjoint loses eps / (1 - ssa))
constexpr double FP32_COALBEDO_MIN = 3.0e-4;

// Device copy of the CloudCoeff LUT (phase element 1 only).  Tables keep the
// file's Fortran order (frequency fastest).
struct CloudLut {
  int nfm, nrm, nt, nd, nfi, nri, nleg;
  const double* f_mw, *r_mw, *t, *f_ir, *r_ir;
  const double* ke_l, *w_l, *pc_l;   // [nt][nrm][nfm], pc: [nleg+1][nt][nrm][nfm]
  const double* ke_s, *w_s, *pc_s;   // [nd][nrm][nfm],  pc: [nleg+1][nd][nrm][nfm]
  const double* ke_ir, *w_ir, *pc_ir; // [nd+1][nri][nfi], pc: [nleg][nd+1][nri][nfi]
  // lagrange4_recip_table of the radius and temperature axes (null: formed per lookup)
  const double* rc_rmw = nullptr, *rc_rir = nullptr, *rc_t = nullptr;
};

// Gauss-Legendre angles/weights on (0,1) for 1..9 streams (Double_Gauss_Quadrature).
// P[n][i][l]: Legendre polynomial l of angle i of the n-point set, l up to
// the largest stream set's term count (the streams' P of every layer).
struct GaussTable {
  double mu[10][SC_NZ_MAX];
  double w[10][SC_NZ_MAX];
  double P[10][9][SC_NLEG_MAX + 1];
};

// ---- interpolation ----------------------------------------------------------
// Weights in S: the radius axis and the temperature axis of the liquid-cloud
// tables carry derivatives in the cloudy K-matrix; frequency is a plain double.
template <class S>
struct Lagrange4T {
  int i0;          // first of the 4 points
  S wl[3], wr[3];  // left and right quadratic weights, already blended
};
using Lagrange4 = Lagrange4T<double>;

// The seven reciprocal denominators of the 4-point window starting at node
// i0 of an axis: 1/d12 and the left and right quadratics' 1/(d..d..).
CRTM_HD void lagrange4_recip(const double* p, double* r) {
  const double d01 = p[0] - p[1], d02 = p[0] - p[2], d12 = p[1] - p[2], d13 = p[1] - p[3],
               d23 = p[2] - p[3];
  r[0] = 1.0 / d12;
  r[1] = 1.0 / (d01 * d02);
  r[2] = -1.0 / (d01 * d12);
  r[3] = 1.0 / (d02 * d12);
  r[4] = 1.0 / (d12 * d13);
  r[5] = -1.0 / (d12 * d23);
  r[6] = 1.0 / (d13 * d23);
}

// Host: an axis's table of lagrange4_recip for every window (n - 3 rows of 7;
// empty for axes of fewer than 4 nodes).
inline void lagrange4_recip_table(const double* ax, int n, double* out) {
  for (int i0 = 0; i0 + 3 < n; i0++) lagrange4_recip(ax + i0, out + 7 * i0);
}

// Clamp x into the axis, bracket it with 4 points and form the blended
// quadratic weights (the reference's LPoly applied to a 4-point window).
// rec: the axis's lagrange4_recip_table (null: the reciprocals are formed
// here); the weights carry S's derivative parts through multiplications only.
template <class S>
CRTM_HD Lagrange4T<S> lagrange4(const double* ax, int n, S x, const double* rec = nullptr) {
  if (x < ax[0]) x = S(ax[0]);
  if (x > ax[n - 1]) x = S(ax[n - 1]);
  int lo = 0, hi = n - 1;             // first node >= x, by bisection
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (x > ax[mid]) lo = mid + 1;
    else hi = mid;
  }
  int i0 = lo - 2;
  i0 = i0 < 0 ? 0 : (i0 > n - 4 ? n - 4 : i0);
  const double* p = ax + i0;
  const S a0 = x - p[0], a1 = x - p[1], a2 = x - p[2], a3 = x - p[3];
  double rw[7];
  if (rec) {
    for (int q = 0; q < 7; q++) rw[q] = rec[7 * i0 + q];
  } else {
    lagrange4_recip(p, rw);
  }
  const double r12 = rw[0], rl0 = rw[1], rl1 = rw[2], rl2 = rw[3], rr0 = rw[4], rr1 = rw[5], rr2 = rw[6];
  S wr = (x < p[1]) ? S(0.0) : ((x > p[2]) ? S(1.0) : a1 * (-r12));
  const S wl = 1.0 - wr;
  Lagrange4T<S> L;
  L.i0 = i0;
  L.wl[0] = wl * (a1 * a2 * rl0);
  L.wl[1] = wl * (a0 * a2 * rl1);
  L.wl[2] = wl * (a0 * a1 * rl2);
  L.wr[0] = wr * (a2 * a3 * rr0);
  L.wr[1] = wr * (a1 * a3 * rr1);
  L.wr[2] = wr * (a1 * a2 * rr2);
  return L;
}

template <class S, class Z>
CRTM_HD S lerp4(const Z* z, size_t stride, const Lagrange4T<S>& L) {
  const Z z0 = z[0], z1 = z[stride], z2 = z[2 * stride], z3 = z[3 * stride];
  return (L.wl[0] * z0 + L.wl[1] * z1 + L.wl[2] * z2) + (L.wr[0] * z1 + L.wr[1] * z2 + L.wr[2] * z3);
}

// 2-D: dimension u (frequency, plain) fastest, v with stride nu.
template <class S>
CRTM_HD S lerp4x4(const double* z, int nu, const Lagrange4& U, const Lagrange4T<S>& V) {
  double a[4];
  const double* b = z + (size_t)V.i0 * nu + U.i0;
  for (int j = 0; j < 4; j++) a[j] = lerp4(b + (size_t)j * nu, 1, U);
  return lerp4(a, 1, V);
}

// 3-D: frequency (plain), radius and temperature in S.
template <class S>
CRTM_HD S lerp4x4x4(const double* z, int nu, int nv, const Lagrange4& U, const Lagrange4T<S>& V,
                    const Lagrange4T<S>& W) {
  S a[4];
  for (int k = 0; k < 4; k++) a[k] = lerp4x4(z + (size_t)(W.i0 + k) * nu * nv, nu, U, V);
  return lerp4(a, 1, W);
}

// The cloud tables of one sensor already interpolated to each channel's
// frequency (the frequency step of lerp4x4 / lerp4x4x4 done once per channel
// at init, cloud_chan_kernel): plane q of the tables at radius row r for
// channel ch is z[(q * rows + r) * L + ch], channels fastest, rows = the
// radius axis.  Planes (cloud_chan_plane):
//   infrared:  ke, w of the nd + 1 density slots, then Legendre term t
//              (t = 0..nleg-1, the file's pc index) of each slot;
//   microwave: liquid ke, w of the nt temperatures and term t (0..nleg) of
//              each temperature, then solid ke, w of the nd density slots and
//              term t of each slot.
// A null z: the lookups interpolate in frequency themselves.
struct CloudChan {
  const double* z = nullptr;
  size_t L = 0;
  int ch = 0;
};

CRTM_HD int cloud_chan_planes(const CloudLut& C, bool microwave) {
  return microwave ? (2 + C.nleg + 1) * (C.nt + C.nd) : (2 + C.nleg) * (C.nd + 1);
}

// Plane index of table `tab` (0 ke, 1 w, 2 + t Legendre term t) of slot j
// (temperature index of a liquid table, density slot otherwise).
CRTM_HD int cloud_chan_plane(const CloudLut& C, bool microwave, bool solid, int tab, int j) {
  if (!microwave) return tab * (C.nd + 1) + j;
  return solid ? (2 + C.nleg + 1) * C.nt + tab * C.nd + j : tab * C.nt + j;
}

// The file table behind plane q (rows of nf frequencies, stride nf).
CRTM_HD const double* cloud_chan_source(const CloudLut& C, bool microwave, int q) {
  if (!microwave) {
    const size_t plane = (size_t)C.nfi * C.nri, vol = plane * (C.nd + 1);
    const int tab = q / (C.nd + 1), j = q % (C.nd + 1);
    return tab == 0 ? C.ke_ir + j * plane : (tab == 1 ? C.w_ir + j * plane : C.pc_ir + (tab - 2) * vol + j * plane);
  }
  const size_t plane = (size_t)C.nfm * C.nrm;
  const int nliq = (2 + C.nleg + 1) * C.nt;
  if (q < nliq) {
    const size_t vol = plane * C.nt;
    const int tab = q / C.nt, j = q % C.nt;
    return tab == 0 ? C.ke_l + j * plane : (tab == 1 ? C.w_l + j * plane : C.pc_l + (tab - 2) * vol + j * plane);
  }
  q -= nliq;
  const size_t vol = plane * C.nd;
  const int tab = q / C.nd, j = q % C.nd;
  return tab == 0 ? C.ke_s + j * plane : (tab == 1 ? C.w_s + j * plane : C.pc_s + (tab - 2) * vol + j * plane);
}

// Legendre offset of the stream set (CloudCoeff_Define.f90:83-84).
CRTM_HD int legendre_offset(int nleg) {
  return nleg == 2 || nleg == 4 ? 0 : (nleg == 6 ? 5 : (nleg == 8 ? 12 : (nleg == 16 ? 21 : -1)));
}

// The lookups of cloud_layer_optics through channel tables of element type
// TZ (zc: the tables at this channel; L: the channel stride).
template <class S, class TZ>
CRTM_HD bool cloud_optics_chan(const CloudLut& C, bool microwave, int type, S reff, S temp, int nleg, int loff,
                               S* ke, S* w, S* pc, const TZ* zc, size_t L) {
  const bool solid = microwave && !(type == 1 || type == 3);
  const int rows = microwave ? C.nrm : C.nri;
  const size_t ps = (size_t)rows * L;
  auto plane = [&](int tab, int j) { return zc + (size_t)cloud_chan_plane(C, microwave, solid, tab, j) * ps; };
  int kd;
  if (!microwave)
    kd = (type == 1 || type == 3) ? 0 : (type == 4 ? 1 : (type == 5 ? 2 : (type == 2 || type == 6 ? 3 : -1)));
  else
    kd = solid ? (type == 4 ? 0 : (type == 5 ? 1 : (type == 2 || type == 6 ? 2 : -1))) : 0;
  if (kd < 0) return false;
  if (microwave && !solid) {    // liquid: temperature axis
    const Lagrange4T<S> T = lagrange4(C.t, C.nt, temp, C.rc_t);
    if (type == 1) {            // cloud water: (frequency, temperature) at the first radius
      double a[4];
      for (int k = 0; k < 4; k++) a[k] = plane(0, T.i0 + k)[0];
      *ke = lerp4(a, 1, T);
      return true;
    }
    const Lagrange4T<S> R = lagrange4(C.r_mw, C.nrm, reff, C.rc_rmw);
    const size_t r0 = (size_t)R.i0 * L;
    auto tr = [&](int tab) {
      S a[4];
      for (int k = 0; k < 4; k++) a[k] = lerp4(plane(tab, T.i0 + k) + r0, L, R);
      return lerp4(a, 1, T);
    };
    *ke = tr(0);
    *w = tr(1);
    pc[0] = S(0.5);
    for (int l = 1; l <= nleg; l++) pc[l] = tr(2 + l + loff);
    return true;
  }
  if (microwave && type == 2) {   // cloud ice: frequency only, first radius
    *ke = S(plane(0, kd)[0]);
    return true;
  }
  const Lagrange4T<S> R = lagrange4(microwave ? C.r_mw : C.r_ir, rows, reff, microwave ? C.rc_rmw : C.rc_rir);
  const size_t r0 = (size_t)R.i0 * L;
  *ke = lerp4(plane(0, kd) + r0, L, R);
  *w = lerp4(plane(1, kd) + r0, L, R);
  pc[0] = S(0.5);
  const int t0 = microwave ? loff : loff - 1;   // the infrared tables have no term 0
  for (int l = 1; l <= nleg; l++) pc[l] = lerp4(plane(2 + l + t0, kd) + r0, L, R);
  return true;
}

// Optical properties of one cloud layer: ke (m^2/kg), w and the phase terms
// pc[0..nleg].  Only the liquid microwave tables depend on temperature; the
// effective radius and the temperature carry S's derivatives.  Returns false
// for an unknown cloud type.  With the channel tables Z the same values come
// from the frequency-interpolated planes (the same arithmetic, one step done
// once per channel).
template <class S>
CRTM_HD bool cloud_layer_optics(const CloudLut& C, bool microwave, double freq, int type, S reff,
                                S temp, int nleg, int loff, S* ke, S* w, S* pc, const CloudChan& Z = CloudChan()) {
  for (int l = 0; l <= nleg; l++) pc[l] = S(0.0);
  *w = S(0.0);
  if (Z.z) return cloud_optics_chan<S, double>(C, microwave, type, reff, temp, nleg, loff, ke, w, pc, Z.z + Z.ch, Z.L);
  if (!microwave) {
    // density slot of Get_Cloud_Opt_IR: liquid 1, snow 2, graupel 3, ice/hail 4
    const int kd = (type == 1 || type == 3) ? 0 : (type == 4 ? 1 : (type == 5 ? 2 : (type == 2 || type == 6 ? 3 : -1)));
    if (kd < 0) return false;
    const Lagrange4 F = lagrange4(C.f_ir, C.nfi, freq);
    const Lagrange4T<S> R = lagrange4(C.r_ir, C.nri, reff);
    const size_t plane = (size_t)C.nfi * C.nri, vol = plane * (C.nd + 1);
    *ke = lerp4x4(C.ke_ir + kd * plane, C.nfi, F, R);
    *w = lerp4x4(C.w_ir + kd * plane, C.nfi, F, R);
    pc[0] = S(0.5);
    for (int l = 1; l <= nleg; l++) pc[l] = lerp4x4(C.pc_ir + (l + loff - 1) * vol + kd * plane, C.nfi, F, R);
    return true;
  }
  const Lagrange4 F = lagrange4(C.f_mw, C.nfm, freq);
  const size_t plane = (size_t)C.nfm * C.nrm;
  if (type == 1 || type == 3) {   // liquid: temperature axis
    const Lagrange4T<S> T = lagrange4(C.t, C.nt, temp);
    if (type == 1) {              // cloud water: (frequency, temperature) at the first radius
      double a[4];
      for (int k = 0; k < 4; k++) a[k] = lerp4(C.ke_l + (size_t)(T.i0 + k) * plane + F.i0, 1, F);
      *ke = lerp4(a, 1, T);
      return true;
    }
    const Lagrange4T<S> R = lagrange4(C.r_mw, C.nrm, reff);
    const size_t vol = plane * C.nt;
    *ke = lerp4x4x4(C.ke_l, C.nfm, C.nrm, F, R, T);
    *w = lerp4x4x4(C.w_l, C.nfm, C.nrm, F, R, T);
    pc[0] = S(0.5);
    for (int l = 1; l <= nleg; l++) pc[l] = lerp4x4x4(C.pc_l + (l + loff) * vol, C.nfm, C.nrm, F, R, T);
    return true;
  }
  const int kd = type == 4 ? 0 : (type == 5 ? 1 : (type == 2 || type == 6 ? 2 : -1));
  if (kd < 0) return false;
  if (type == 2) {                // cloud ice: frequency only, first radius
    *ke = S(lerp4(C.ke_s + kd * plane + F.i0, 1, F));
    return true;
  }
  const Lagrange4T<S> R = lagrange4(C.r_mw, C.nrm, reff);
  const size_t vol = plane * C.nd;
  *ke = lerp4x4(C.ke_s + kd * plane, C.nfm, F, R);
  *w = lerp4x4(C.w_s + kd * plane, C.nfm, F, R);
  pc[0] = S(0.5);
  for (int l = 1; l <= nleg; l++) pc[l] = lerp4x4(C.pc_s + (l + loff) * vol + kd * plane, C.nfm, F, R);
  return true;
}

// Device copy of the AerosolCoeff LUT, scheme 'CRTM' (first RH and sigma of
// each type; phase element 1).  Tables in the file's Fortran order.
// CRTM_Init's Aerosol_Model: the LUT's layout and interpolation axes
constexpr int AEROSOL_CRTM = 0, AEROSOL_CMAQ = 1, AEROSOL_GOCART = 2, AEROSOL_NAAPS = 3;

struct AerosolLut {
  int nw, nrh, nr, ns, nt, nleg;
  int scheme;               // AEROSOL_CRTM .. AEROSOL_NAAPS
  int nrh_axis;             // entries of the RH axis (n_RH_Radii or n_RH)
  const int* type_id;       // [nt]
  const double* freq;       // [nw] cm^-1, increasing
  const double* reff;       // [nt][nr]
  const double* rsig;       // [nt][ns]
  const double* rh;         // [nrh_axis]
  const double* ke, *w;     // [nt][ns][nr][nrh][nw]
  const double* pc;         // [nleg+1][nt][ns][nr][nrh][nw]
  // lagrange4_recip_table of the axes (per type for radius and sigma: rows of
  // (nr - 3) * 7 and (ns - 3) * 7); null: formed per lookup
  const double* rc_freq = nullptr, *rc_reff = nullptr, *rc_rsig = nullptr, *rc_rh = nullptr;
};

// Get_Aerosol_Opt (CRTM_AerosolScatter.f90:772-918).  'CRTM': frequency x
// radius at the first RH and sigma; 'CMAQ': frequency x radius x sigma at the
// first RH; 'GOCART-GEOS5' / 'NAAPS': frequency x RH at the first radius and
// sigma.  Radius, sigma (Effective_Variance) and RH carry S's derivatives.
template <class S>
CRTM_HD bool aerosol_layer_optics(const AerosolLut& A, double wavenumber, int type, S reff, S rsig, S rh,
                                  int nleg, int loff, S* ke, S* w, S* pc) {
  int k = -1;
  for (int t = 0; t < A.nt; t++)
    if (A.type_id[t] == type) { k = t; break; }
  if (k < 0) return false;
  const Lagrange4 F = lagrange4(A.freq, A.nw, wavenumber, A.rc_freq);
  const double* rcr = A.rc_reff ? A.rc_reff + (size_t)k * (A.nr - 3) * 7 : nullptr;
  const double* rcs = A.rc_rsig ? A.rc_rsig + (size_t)k * (A.ns - 3) * 7 : nullptr;
  const int nu = A.nw * A.nrh;                     // radius stride
  const size_t base = (size_t)k * A.nw * A.nrh * A.nr * A.ns;
  const size_t n5 = (size_t)A.nw * A.nrh * A.nr * A.ns * A.nt;
  pc[0] = S(0.5);
  if (A.scheme == AEROSOL_CRTM) {
    const Lagrange4T<S> Rr = lagrange4(A.reff + (size_t)k * A.nr, A.nr, reff, rcr);
    *ke = lerp4x4(A.ke + base, nu, F, Rr);
    *w = lerp4x4(A.w + base, nu, F, Rr);
    for (int l = 1; l <= nleg; l++) pc[l] = lerp4x4(A.pc + n5 * (l + loff) + base, nu, F, Rr);
  } else if (A.scheme == AEROSOL_CMAQ) {
    const Lagrange4T<S> Rr = lagrange4(A.reff + (size_t)k * A.nr, A.nr, reff, rcr);
    const Lagrange4T<S> Sg = lagrange4(A.rsig + (size_t)k * A.ns, A.ns, rsig, rcs);
    *ke = lerp4x4x4(A.ke + base, nu, A.nr, F, Rr, Sg);
    *w = lerp4x4x4(A.w + base, nu, A.nr, F, Rr, Sg);
    for (int l = 1; l <= nleg; l++) pc[l] = lerp4x4x4(A.pc + n5 * (l + loff) + base, nu, A.nr, F, Rr, Sg);
  } else {
    const Lagrange4T<S> H = lagrange4(A.rh, A.nrh, rh, A.rc_rh);
    *ke = lerp4x4(A.ke + base, A.nw, F, H);
    *w = lerp4x4(A.w + base, A.nw, F, H);
    for (int l = 1; l <= nleg; l++) pc[l] = lerp4x4(A.pc + n5 * (l + loff) + base, A.nw, F, H);
  }
  return true;
}

// IR sea-surface emissivity table (IRwaterCoeff_Define.f90:86-106), Fortran
// order (angle fastest, then frequency, wind speed, temperature).
struct IRWaterLut {
  int na, nf, nv, nt;
  int nalli2;               // 'Nalli2' classification: temperature is an axis too
  const double* angle;      // [na] degrees
  const double* freq;       // [nf] cm^-1
  const double* wind;       // [nv] m/s
  const double* temp;       // [nt] K
  const double* e;          // [nt][nv][nf][na]
};

// CRTM_Compute_IRSSEM (CRTM_IRSSEM.f90:204-334) at one angle (degrees): the
// 4-point blended Lagrange interpolation in angle, frequency and wind speed,
// and water temperature for a 'Nalli2' table, each clamped to its axis as
// Find_Random_Index does.  Wind speed and temperature carry S's derivatives.
template <class S>
CRTM_HD S irssem(const IRWaterLut& W, S water_temperature, S wind_speed, double frequency, double angle) {
  const Lagrange4 A = lagrange4(W.angle, W.na, fabs(angle));
  const Lagrange4T<S> F = lagrange4(W.freq, W.nf, S(frequency));
  const Lagrange4T<S> V = lagrange4(W.wind, W.nv, wind_speed);
  if (!W.nalli2) return lerp4x4x4(W.e, W.na, W.nf, A, F, V);
  const Lagrange4T<S> T = lagrange4(W.temp, W.nt, water_temperature);
  const size_t n3 = (size_t)W.na * W.nf * W.nv;
  S a[4];
  for (int l = 0; l < 4; l++) a[l] = lerp4x4x4(W.e + (size_t)(T.i0 + l) * n3, W.na, W.nf, A, F, V);
  return lerp4(a, 1, T);
}

// ---- small dense matrices (row-major, fixed capacity NZ x NZ) --------------
template <int NZ, class T>
struct Mat {
  T a[NZ][NZ];
};

template <int NZ, class T>
CRTM_HD void mat_mul(int n, const Mat<NZ, T>& A, const Mat<NZ, T>& B, Mat<NZ, T>& C) {
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      T s = T(0.0);
      for (int k = 0; k < n; k++) s += A.a[i][k] * B.a[k][j];
      C.a[i][j] = s;
    }
}

// In-place inverse by Gauss-Jordan elimination with partial pivoting.
template <int NZ, class T>
CRTM_HD bool mat_invert(int n, Mat<NZ, T>& A) {
  int perm[NZ];
  for (int i = 0; i < n; i++) perm[i] = i;
  for (int k = 0; k < n; k++) {
    int p = k;
    T best = fabs(A.a[k][k]);
    for (int i = k + 1; i < n; i++)
      if (fabs(A.a[i][k]) > best) { best = fabs(A.a[i][k]); p = i; }
    if (!(best > T(1.0e-40))) return false;
    if (p != k) {
      for (int j = 0; j < n; j++) { const T t = A.a[p][j]; A.a[p][j] = A.a[k][j]; A.a[k][j] = t; }
      const int t = perm[p]; perm[p] = perm[k]; perm[k] = t;
    }
    const T d = T(1.0) / A.a[k][k];
    for (int j = 0; j < n; j++) A.a[k][j] *= d;
    A.a[k][k] = d;
    for (int i = 0; i < n; i++) {
      if (i == k) continue;
      const T f = A.a[i][k];
      if (is_zero(f)) continue;
      for (int j = 0; j < n; j++) A.a[i][j] -= f * A.a[k][j];
      A.a[i][k] = -f * d;
    }
  }
  // undo the row interchanges as column interchanges of the inverse
  T tmp[NZ];
  for (int i = 0; i < n; i++) {
    for (int j = 0; j < n; j++) tmp[perm[j]] = A.a[i][j];
    for (int j = 0; j < n; j++) A.a[i][j] = tmp[j];
  }
  return true;
}

// Symmetric eigenproblem S = V diag(lam) V^T by cyclic Jacobi rotations.
template <int NZ, class T>
CRTM_HD void jacobi(int n, Mat<NZ, T>& S, T* lam, Mat<NZ, T>& V) {
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) V.a[i][j] = (i == j) ? T(1.0) : T(0.0);
  for (int sweep = 0; sweep < 60; sweep++) {
    T off = T(0.0), diag = T(0.0);
    for (int i = 0; i < n; i++) {
      diag += S.a[i][i] * S.a[i][i];
      for (int j = i + 1; j < n; j++) off += S.a[i][j] * S.a[i][j];
    }
    if (off <= T(JacobiEps<T>::value) * diag) break;
    for (int p = 0; p < n - 1; p++)
      for (int q = p + 1; q < n; q++) {
        const T apq = S.a[p][q];
        if (apq == T(0.0)) continue;
        const T th = (S.a[q][q] - S.a[p][p]) / (T(2.0) * apq);
        const T t = (th >= T(0.0) ? T(1.0) : -T(1.0)) / (fabs(th) + sqrt(th * th + T(1.0)));
        const T c = T(1.0) / sqrt(t * t + T(1.0)), s = t * c;
        for (int k = 0; k < n; k++) {
          const T kp = S.a[k][p], kq = S.a[k][q];
          S.a[k][p] = c * kp - s * kq;
          S.a[k][q] = s * kp + c * kq;
        }
        for (int k = 0; k < n; k++) {
          const T pk = S.a[p][k], qk = S.a[q][k];
          S.a[p][k] = c * pk - s * qk;
          S.a[q][k] = s * pk + c * qk;
        }
        for (int k = 0; k < n; k++) {
          const T kp = V.a[k][p], kq = V.a[k][q];
          V.a[k][p] = c * kp - s * kq;
          V.a[k][q] = s * kp + c * kq;
        }
      }
  }
  for (int i = 0; i < n; i++) lam[i] = S.a[i][i];
}

// Symmetric eigenproblem on derivative numbers: eigenpairs of the value
// part by Jacobi, then their derivatives by first-order perturbation:
// d(lambda_i) = v_i' dS v_i and dv_i = sum_{j != i} v_j (v_j' dS v_i) / (lambda_i - lambda_j).
template <int NZ, int N, class Q>
CRTM_HD void jacobi(int n, Mat<NZ, Dual<N, Q>>& S, Dual<N, Q>* lam, Mat<NZ, Dual<N, Q>>& V) {
  Mat<NZ, Q> S0, V0;
  Q l0[NZ];
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) S0.a[i][j] = S.a[i][j].v;
  jacobi<NZ, Q>(n, S0, l0, V0);
  for (int i = 0; i < n; i++) {
    lam[i] = Dual<N, Q>(l0[i], 0);
    for (int j = 0; j < n; j++) V.a[i][j] = Dual<N, Q>(V0.a[i][j], 0);
  }
  for (int q = 0; q < N; q++) {
    // M = V0' dS V0
    Q M[NZ][NZ], T1[NZ][NZ];
    for (int i = 0; i < n; i++)
      for (int j = 0; j < n; j++) {
        Q v = Q(0.0);
        for (int k = 0; k < n; k++) v += S.a[i][k].d[q] * V0.a[k][j];
        T1[i][j] = v;
      }
    for (int i = 0; i < n; i++)
      for (int j = 0; j < n; j++) {
        Q v = Q(0.0);
        for (int k = 0; k < n; k++) v += V0.a[k][i] * T1[k][j];
        M[i][j] = v;
      }
    for (int i = 0; i < n; i++) lam[i].d[q] = M[i][i];
    for (int r = 0; r < n; r++)     // row r of dV = V0 C, C_ji = M_ji / (l_i - l_j)
      for (int i = 0; i < n; i++) {
        Q v = Q(0.0);
        for (int j = 0; j < n; j++)
          if (j != i) v += V0.a[r][j] * M[j][i] / (l0[i] - l0[j]);
        V.a[r][i].d[q] = v;
      }
  }
}

// Eigenpairs of MOM's HH = (PP - PM)(PP + PM) for a layer of scaled albedo s
// (CRTM_AMOM_layer / MOM, ADA_Module.f90:262-354 and :552-743): the
// eigenvectors in the columns of E, the eigenvalues in lam.  The quadrature
// block is solved in its symmetric form, the sensor angle's eigenpair from
// the block-triangular structure.  On return X = PP - PM and Y = PP + PM over
// all nZ angles; V and W are scratch.  Returns false on a failed
// factorisation.  gap: see ada_layer.
template <int NZ, class T>
CRTM_HD bool mom_eigen(int nS, int nZ, T s, const T* mu, const T* wt, const Mat<NZ, T>& ff, const Mat<NZ, T>& bb,
                       Mat<NZ, T>& E, T* lam, Mat<NZ, T>& X, Mat<NZ, T>& Y, Mat<NZ, T>& V, Mat<NZ, T>& W,
                       double* gap) {
  // symmetric form of the quadrature block
  T sq[NZ];
  for (int i = 0; i < nS; i++) sq[i] = sqrt(wt[i]);
  for (int i = 0; i < nS; i++)
    for (int j = 0; j < nS; j++) {
      const T sw = s * sq[i] * sq[j], dd = T(1.0) / sqrt(mu[i] * mu[j]);
      const T id = (i == j) ? T(1.0) : T(0.0);
      X.a[i][j] = (id - sw * (ff.a[i][j] - bb.a[i][j])) * dd;
      Y.a[i][j] = (id - sw * (ff.a[i][j] + bb.a[i][j])) * dd;
    }
  // Cholesky Y = L L^T (lower triangle of Y overwritten by L)
  for (int j = 0; j < nS; j++) {
    T d = Y.a[j][j];
    for (int k = 0; k < j; k++) d -= Y.a[j][k] * Y.a[j][k];
    if (!(d > T(0.0))) return false;
    d = sqrt(d);
    Y.a[j][j] = d;
    for (int i = j + 1; i < nS; i++) {
      T v = Y.a[i][j];
      for (int k = 0; k < j; k++) v -= Y.a[i][k] * Y.a[j][k];
      Y.a[i][j] = v / d;
    }
  }
  // S = L^T X L in V (temporary X L in W)
  for (int i = 0; i < nS; i++)
    for (int j = 0; j < nS; j++) {
      T v = T(0.0);
      for (int k = j; k < nS; k++) v += X.a[i][k] * Y.a[k][j];
      W.a[i][j] = v;
    }
  for (int i = 0; i < nS; i++)
    for (int j = i; j < nS; j++) {
      T v = T(0.0);
      for (int k = i; k < nS; k++) v += Y.a[k][i] * W.a[k][j];
      V.a[i][j] = v;
    }
  for (int i = 0; i < nS; i++)
    for (int j = 0; j < i; j++) V.a[i][j] = V.a[j][i];
  jacobi(nS, V, lam, X);   // eigenvectors u in the columns of X
  // E = W^-1/2 D^-1/2 L^-T u: eigenvectors of HH, in E
  for (int c = 0; c < nS; c++) {
    for (int i = nS - 1; i >= 0; i--) {
      T v = X.a[i][c];
      for (int k = i + 1; k < nS; k++) v -= Y.a[k][i] * E.a[k][c];
      E.a[i][c] = v / Y.a[i][i];
    }
    for (int i = 0; i < nS; i++) E.a[i][c] /= sqrt(wt[i] * mu[i]);
  }
  // PP, PM for the full set of angles: PPM = PP - PM kept in X, PPP in Y
  for (int i = 0; i < nZ; i++) {
    const T c = s / mu[i];
    for (int j = 0; j < nZ; j++) {
      const T f = c * ff.a[i][j] * wt[j] - (i == j ? T(1.0) / mu[i] : T(0.0)), b = c * bb.a[i][j] * wt[j];
      X.a[i][j] = f - b;
      Y.a[i][j] = f + b;
    }
  }
  if (nZ > nS) {   // sensor angle (weight 0): HH is block lower triangular
    const int z = nZ - 1;
    T hz[NZ];
    for (int k = 0; k < nZ; k++) {
      T v = T(0.0);
      for (int m = 0; m < nZ; m++) v += X.a[z][m] * Y.a[m][k];
      hz[k] = v;   // row z of HH
    }
    for (int c = 0; c < nS; c++) {
      T v = T(0.0);
      for (int k = 0; k < nS; k++) v += hz[k] * E.a[k][c];
      E.a[z][c] = v / (lam[c] - hz[z]);
      if (gap) {
        const double g = fabs(value_of(lam[c]) - value_of(hz[z])) / fabs(value_of(lam[c]));
        if (g < *gap) *gap = g;
      }
    }
    for (int i = 0; i < nS; i++) E.a[i][z] = T(0.0);
    E.a[z][z] = T(1.0);
    lam[z] = hz[z];
  }
  return true;
}

// Layer optics of a scattering layer for the adding method (CRTM_AMOM_layer +
// MOM, azimuth order 0, no solar source), in loss form: U = I - T (T the
// layer's transmission), the reflection R and the thermal source (identical
// up and down).  ff/bb are the normalised forward/backward phase blocks.
// Returns false on a failed factorisation.
//
// MOM gives T and R as ratios of differences that cancel as the layer thins
// (T -> I, R -> 0 as tau -> 0): with D = I - diag(exp(-lambda tau)) from expm1,
// P = Gm^-1 Gp, Q = Gm - Gp P and e = I - D, the reference's
//   T = (Gm e - Gp A2)(Gm - Gp e A2)^-1,  R = (Gp - Gm e A2)(...)^-1,  A2 = P e
// are rewritten with GA = Q + Gp (D P e + P D) as
//   U = (Q D + Gp (D P e + P D)) GA^-1,  R = (Gp D + Gm D P e) GA^-1,
// every term of which is O(D): U, R and the source (1 - row sums of T + R)
// keep the arithmetic's relative precision for thin layers, which FP32
// records need.
// gap (optional): the smallest |lambda_c - h_zz| / |lambda_c| between the
// quadrature eigenvalues and the sensor angle's diagonal term of HH (1 when
// there is no separate sensor angle).  Near 0 the eigenbasis is nearly
// defective: the layer's T and R stay smooth, but their derivatives through
// the eigenvectors lose about eps / gap^2 of their accuracy.
template <int NZ, class T>
CRTM_HD bool ada_layer_loss(int nS, int nZ, T w, T tau, const T* mu, const T* wt, const Mat<NZ, T>& ff,
                            const Mat<NZ, T>& bb, T B, Mat<NZ, T>& Um, Mat<NZ, T>& Rm, T* src,
                            double* gap = nullptr) {
  if (gap) *gap = 1.0;
  const bool sensor_row = nZ == nS + 1;
  if (tau < T(DELTA_OPTICAL_DEPTH)) {   // thin layer: first-order scattering
    const T s = tau * w;
    for (int i = 0; i < nZ; i++) {
      const T c = s / mu[i];
      T a = T(0.0);
      for (int j = 0; j < nZ; j++) {
        Rm.a[i][j] = c * bb.a[i][j] * wt[j];
        Um.a[i][j] = (i == j ? tau / mu[i] : T(0.0)) - c * ff.a[i][j] * wt[j];
        a += Um.a[i][j] - Rm.a[i][j];
      }
      src[i] = a * B;
    }
    return true;
  }
  const T s = w < T(MAX_ALBEDO) ? w : T(MAX_ALBEDO);
  Mat<NZ, T> X, Y, V;
  T lam[NZ];
  if (!mom_eigen<NZ, T>(nS, nZ, s, mu, wt, ff, bb, Rm, lam, X, Y, V, Um, gap)) return false;
  // MOM with the eigenpairs (E in R, eigenvalues lam)
  if (!mat_invert(nZ, X)) return false;   // inverse of PP - PM
  T ex[NZ], dx[NZ];
  for (int i = 0; i < nZ; i++) {
    lam[i] = lam[i] > T(0.0) ? sqrt(lam[i]) : T(0.0);
    ex[i] = exp(-lam[i] * tau);
    dx[i] = -expm1(-lam[i] * tau);
  }
  // EF = (PP-PM)^-1 E diag(lam);  Gp = (E + EF)/2 in Y, Gm = (E - EF)/2 in V
  for (int i = 0; i < nZ; i++)
    for (int j = 0; j < nZ; j++) {
      T v = T(0.0);
      for (int k = 0; k < nZ; k++) v += X.a[i][k] * Rm.a[k][j];
      v *= lam[j];
      Y.a[i][j] = T(0.5) * (Rm.a[i][j] + v);
      V.a[i][j] = T(0.5) * (Rm.a[i][j] - v);
    }
  // P = Gm^-1 Gp (in Rm)
  for (int i = 0; i < nZ; i++)
    for (int j = 0; j < nZ; j++) X.a[i][j] = V.a[i][j];
  if (!mat_invert(nZ, X)) return false;    // Gm^-1
  mat_mul(nZ, X, Y, Rm);
  // W = D P e + P D (in X);  Q = Gm - Gp P (in Um)
  for (int i = 0; i < nZ; i++)
    for (int j = 0; j < nZ; j++) {
      X.a[i][j] = dx[i] * Rm.a[i][j] * ex[j] + Rm.a[i][j] * dx[j];
      T v = T(0.0);
      for (int k = 0; k < nZ; k++) v += Y.a[i][k] * Rm.a[k][j];
      Um.a[i][j] = V.a[i][j] - v;
    }
  // GA = Q + Gp W (in A);  U numerator Q D + Gp W (in Um);  R numerator Gp D + Gm D P e (in Rn)
  Mat<NZ, T> A, Rn;
  for (int i = 0; i < nZ; i++)
    for (int j = 0; j < nZ; j++) {
      T gw = T(0.0), gd = T(0.0);
      for (int k = 0; k < nZ; k++) {
        gw += Y.a[i][k] * X.a[k][j];
        gd += V.a[i][k] * dx[k] * Rm.a[k][j];
      }
      A.a[i][j] = Um.a[i][j] + gw;
      Um.a[i][j] = Um.a[i][j] * dx[j] + gw;
      Rn.a[i][j] = Y.a[i][j] * dx[j] + gd * ex[j];
    }
  if (!mat_invert(nZ, A)) return false;    // GA^-1
  mat_mul(nZ, Um, A, X);
  mat_mul(nZ, Rn, A, V);
  for (int i = 0; i < nZ; i++)
    for (int j = 0; j < nZ; j++) { Um.a[i][j] = X.a[i][j]; Rm.a[i][j] = V.a[i][j]; }
  // source (1 - row sum of T + R) B over the quadrature columns (and T's
  // diagonal on the sensor row) = (row sum of U - row sum of R) B
  for (int i = 0; i < nZ; i++) {
    T a = T(0.0);
    for (int j = 0; j < nS; j++) a += Um.a[i][j] - Rm.a[i][j];
    if (sensor_row && i == nZ - 1) a += Um.a[i][i];
    src[i] = a * B;
  }
  return true;
}

// ada_layer_loss with the transmission T = I - U.
template <int NZ, class T>
CRTM_HD bool ada_layer(int nS, int nZ, T w, T tau, const T* mu, const T* wt, const Mat<NZ, T>& ff,
                       const Mat<NZ, T>& bb, T B, Mat<NZ, T>& Tm, Mat<NZ, T>& Rm, T* src, double* gap = nullptr) {
  if (!ada_layer_loss<NZ, T>(nS, nZ, w, tau, mu, wt, ff, bb, B, Tm, Rm, src, gap)) return false;
  for (int i = 0; i < nZ; i++)
    for (int j = 0; j < nZ; j++) Tm.a[i][j] = (i == j ? T(1.0) : T(0.0)) - Tm.a[i][j];
  return true;
}

// Forward/backward phase blocks of one layer from its Legendre terms
// (CRTM_Phase_Matrix, m = 0) and their normalisation (Normalize_Phase).
template <int NZ, class T>
CRTM_HD void phase_blocks(int nS, int nZ, int nleg, const T* pc, const T (*P)[SC_NLEG_MAX + 1],
                                 const T* wt, Mat<NZ, T>& ff, Mat<NZ, T>& bb) {
  for (int i = 0; i < nZ; i++)
    for (int j = i; j < nZ; j++) {
      T f = T(0.0), b = T(0.0);
      for (int l = 0; l < nleg; l++) {
        const T t = pc[l] * P[i][l] * P[j][l];
        f += t;
        b += (l & 1) ? -t : t;
      }
      ff.a[i][j] = ff.a[j][i] = f < T(0.0) ? T(PHASE_THRESHOLD) : f;
      bb.a[i][j] = bb.a[j][i] = b < T(0.0) ? T(PHASE_THRESHOLD) : b;
    }
  T carried = T(0.0);
  for (int i = 0; i < nS; i++) {
    T nf = T(0.0);
    for (int j = i; j < nZ; j++) nf += (ff.a[i][j] + bb.a[i][j]) * wt[j];
    const T sc = (T(1.0) - carried) / nf;
    for (int j = i; j < nZ; j++) {
      ff.a[i][j] *= sc; bb.a[i][j] *= sc;
      ff.a[j][i] = ff.a[i][j]; bb.a[j][i] = bb.a[i][j];
    }
    carried = T(0.0);
    if (i + 1 < nZ)
      for (int j = 0; j <= i; j++) carried += (ff.a[i + 1][j] + bb.a[i + 1][j]) * wt[j];
  }
  if (nS < nZ) {
    const int z = nZ - 1;
    for (int j = 0; j < nZ; j++) {
      ff.a[j][z] /= carried; bb.a[j][z] /= carried;
      if (j < z) { ff.a[z][j] = ff.a[j][z]; bb.a[z][j] = bb.a[j][z]; }
    }
  }
}

// SOI layer doubling (SOI_Module.f90: CRTM_Truncated_Doubling :697-827 uses
// I + R R in place of (I - R R)^-1; CRTM_Doubling_layer :1091-1234 inverts):
// from a first-order layer of optical depth tau / 2^n, n doublings give the
// layer's transmission T, reflection R and thermal source.
template <int NZ, class T>
CRTM_HD bool soi_doubling(bool trunc, int nS, int nZ, T w, T tau, const T* mu, const T* wt,
                          const Mat<NZ, T>& ff, const Mat<NZ, T>& bb, T B, Mat<NZ, T>& Tm,
                          Mat<NZ, T>& Rm, T* src) {
  if (tau < 1.0e-6) {   // OPTICAL_DEPTH_THRESHOLD: transparent, no source
    for (int i = 0; i < nZ; i++) {
      src[i] = T(0.0);
      for (int j = 0; j < nZ; j++) { Tm.a[i][j] = T((i == j) ? 1.0 : 0.0); Rm.a[i][j] = T(0.0); }
    }
    return true;
  }
  int nd = (int)(log(value_of(tau) / DELTA_OPTICAL_DEPTH) / log(2.0)) + 1;
  if (nd < 1) nd = 1;
  T dt;
  if (nd <= 55) {                      // MAX_N_DOUBLING
    dt = tau;
    for (int i = 0; i < nd; i++) dt = dt * 0.5;
  } else {
    nd = 55;
    dt = T(DELTA_OPTICAL_DEPTH);
  }
  const T s = dt * w;
  for (int i = 0; i < nZ; i++) {
    const T c = s / mu[i];
    for (int j = 0; j < nZ; j++) {
      Rm.a[i][j] = c * bb.a[i][j] * wt[j];
      Tm.a[i][j] = c * ff.a[i][j] * wt[j] + (i == j ? 1.0 - dt / mu[i] : T(0.0));
    }
  }
  Mat<NZ, T> G, A, Bq;
  for (int L = 0; L < nd; L++) {
    mat_mul<NZ, T>(nZ, Rm, Rm, G);
    for (int i = 0; i < nZ; i++)
      for (int j = 0; j < nZ; j++) G.a[i][j] = (trunc ? G.a[i][j] : -G.a[i][j]) + T(i == j ? 1.0 : 0.0);
    if (!trunc && !mat_invert<NZ, T>(nZ, G)) {
      // the reference falls back to the clear layer
      for (int i = 0; i < nZ; i++) {
        src[i] = T(0.0);
        for (int j = 0; j < nZ; j++) { Tm.a[i][j] = (i == j) ? exp(-tau / mu[i]) : T(0.0); Rm.a[i][j] = T(0.0); }
      }
      return true;
    }
    mat_mul<NZ, T>(nZ, Tm, G, A);    // term2 = T (I -/+ R R)^(-1 or +1)
    mat_mul<NZ, T>(nZ, A, Rm, G);    // term2 R
    mat_mul<NZ, T>(nZ, G, Tm, Bq);   // term2 R T
    for (int i = 0; i < nZ; i++)
      for (int j = 0; j < nZ; j++) Rm.a[i][j] += Bq.a[i][j];
    mat_mul<NZ, T>(nZ, A, Tm, G);
    Tm = G;
  }
  for (int i = 0; i < nZ; i++) {
    T c1 = T(0.0), c2 = T(0.0);
    for (int j = 0; j < nS; j++) { c1 += Tm.a[i][j]; c2 += Rm.a[i][j]; }
    if (i == nZ - 1 && nZ == nS + 1) c1 += Tm.a[i][i];
    src[i] = (1.0 - c1 - c2) * B;
  }
  return true;
}

// Total cloud cover of a profile (Compute_CloudCover,
// CRTM_CloudCover_Define.f90:447-642) after its coverage flag
// (CRTM_Atmosphere_Coverage, CRTM_Atmosphere.f90:158-203).  cf: the layers'
// Cloud_Fraction (null: 1), values below 1e-12 count as 0 and drop the
// layer's clouds; wc: n_clouds rows of stride cstride.  Returns the total
// cover of a FRACTIONAL profile (a cloudy layer with a fraction above 1e-6),
// -1 for a profile whose clouds fill the column, -2 for an invalid overlap id
// (1 maximum, 2 random, 3 maximum-random, 4 average, 5 overcast).
CRTM_HD double total_cloud_cover(int Ku, int n_clouds, const double* cf, const double* wc, size_t cstride,
                                 int overlap) {
  auto frac = [&](int k) {
    const double f = cf ? cf[k] : 1.0;
    return f < MIN_COVERAGE ? 0.0 : f;
  };
  auto lwc = [&](int k) {   // cloud water of the layer above the threshold
    double s = 0.0;
    if (frac(k) == 0.0) return s;
    for (int c = 0; c < n_clouds; c++) {
      const double w = wc[c * cstride + k];
      if (w > WATER_CONTENT_THRESHOLD) s += w;
    }
    return s;
  };
  bool fractional = false;
  for (int k = 0; k < Ku && !fractional; k++) fractional = frac(k) > FRACTIONAL_COVERAGE && lwc(k) > 0.0;
  if (!fractional) return -1.0;
  double tcc = 0.0;
  switch (overlap) {
    case 1:   // maximum
      for (int k = 0; k < Ku; k++) tcc = frac(k) > tcc ? frac(k) : tcc;
      break;
    case 2: {   // random
      double prod = 1.0;
      for (int k = 0; k < Ku; k++)
        if (frac(k) > MIN_COVERAGE) prod *= 1.0 - frac(k);
      tcc = 1.0 - prod;
      break;
    }
    case 3: {   // maximum-random
      double prod = 1.0 - frac(0);
      for (int k = 1; k < Ku; k++) {
        const double a = frac(k - 1), b = frac(k);
        const double mc = 1.0 - (a > b ? a : b);
        prod = (prod == 0.0 && 1.0 - a == 0.0) ? mc : prod * (mc / (1.0 - a));
      }
      tcc = 1.0 - prod;
      break;
    }
    case 4: {   // average, weighted by the layers' cloud water
      double ws = 0.0, cws = 0.0;
      for (int k = 0; k < Ku; k++) {
        const double w = lwc(k);
        ws += w;
        cws += frac(k) * w;
      }
      tcc = ws > 0.0 ? cws / ws : 0.0;
      break;
    }
    case 5:   // overcast
      tcc = 1.0;
      break;
    default:
      return -2.0;
  }
  return tcc;
}

// Inputs of one (profile, channel) for the cloudy solver.
struct CloudyColumn {
  int Ku, n_clouds, nleg;                // nleg: Legendre terms of the stream set
  bool microwave;
  double freq;                           // GHz (MW) or cm^-1 (IR): LUT axis
  double mu_sensor, emissivity, planck_surface, cosmic;
  double c1, c2, b1, b2;                 // Planck constants of the channel
  const double* temperature;             // [Ku]
  const int* cloud_type;                 // [n_clouds]
  const double* wc;                      // [n_clouds] rows of stride cstride
  const double* reff;
  size_t cstride;
  bool soi;                              // Options%RT_Algorithm_Id == RT_SOI
  int n_aerosols;                        // used for non-microwave sensors only
  double wavenumber;                     // aerosol LUT axis, cm^-1
  const int* aerosol_type;               // [n_aerosols]
  const double* conc;                    // [n_aerosols] rows of stride cstride, kg/m^2
  const double* aer_reff;
  const double* aer_var = nullptr;       // Effective_Variance rows ('CMAQ'), null: 0
  const double* rh = nullptr;            // [Ku] Relative_Humidity ('GOCART-GEOS5', 'NAAPS'), null: 0
  const AerosolLut* alut;
  // Cloud_Fraction of the profile's layers (null: 1): clouds are dropped
  // where it is below 1e-12 (CRTM_Forward_Module.f90:367-376); water content
  // divided by the total cloud cover of a fractional profile (Compute_CloudCover,
  // CRTM_CloudCover_Define.f90:512-519), 1 otherwise.
  const double* cf = nullptr;
  double wc_div = 1.0;
  CloudChan zc;                          // the sensor's channel-interpolated cloud tables (optional)
};

// Stream angles of a (profile, channel): Gauss angles of the stream set plus
// the sensor angle with weight 0 unless it is one of them (Assign_Common_Input),
// and Legendre polynomials P_l(mu_i), l = 0..nleg (Legendre_M, m = 0).
template <int NZ, class T>
struct StreamSet {
  int nleg, loff, nS, nZ, isat;
  T mu[NZ], wt[NZ];
  T P[NZ][SC_NLEG_MAX + 1];
};

// Returns 0 or an error code (1-3: stream set does not fit).
template <int NZ, class T>
CRTM_HD int stream_set(int nleg, double mu_sensor, int lut_nleg, const GaussTable& gt, StreamSet<NZ, T>& S) {
  S.nleg = nleg;
  S.loff = legendre_offset(nleg);
  if (S.loff < 0 || nleg > SC_NLEG_MAX) return 1;
  if (lut_nleg >= 0 && lut_nleg < nleg + S.loff) return 2;   // lut_nleg < 0: no clouds
  S.nS = (nleg + 2) / 2;
  if (S.nS + 1 > NZ || S.nS > 9) return 3;
  S.nZ = S.nS;
  S.isat = -1;
  for (int i = 0; i < S.nS; i++) {
    S.mu[i] = T(gt.mu[S.nS][i]);
    S.wt[i] = T(gt.w[S.nS][i]);
    if (S.isat < 0 && fabs(gt.mu[S.nS][i] - mu_sensor) < ANGLE_THRESHOLD) S.isat = i;
  }
  if (S.isat < 0) { S.nZ = S.nS + 1; S.isat = S.nS; S.mu[S.nS] = T(mu_sensor); S.wt[S.nS] = T(0); }
  // the quadrature angles' Legendre values from the table; the sensor
  // angle's by the recurrence
  for (int i = 0; i < S.nS; i++)
    for (int l = 0; l <= nleg; l++) S.P[i][l] = T(gt.P[S.nS][i][l]);
  for (int i = S.nS; i < S.nZ; i++) {
    S.P[i][0] = T(1);
    if (nleg > 0) S.P[i][1] = S.mu[i];
    for (int j = 1; j < nleg; j++)
      S.P[i][j + 1] = (T(2 * j + 1) * S.mu[i] * S.P[i][j] - T(j) * S.P[i][j - 1]) / T(j + 1);
  }
  return 0;
}

// Species seeds of a derivative evaluation: seed(s, amount, c1, c2) may set
// the derivative parts of species s's layer amount (cloud water content after
// the cover scaling, or aerosol concentration) and of its LUT coordinates:
// c1 the effective radius (clouds; aerosols of the 'CRTM' and 'CMAQ' schemes)
// or the layer's relative humidity as this aerosol's lookup sees it
// ('GOCART-GEOS5', 'NAAPS'); c2 the effective variance ('CMAQ'; unused
// otherwise).  Species are the clouds 0..n_clouds-1, then the aerosols.
struct NoSeed {
  template <class S>
  CRTM_HD void operator()(int, S&, S&, S&) const {}
};

// Species s's additive share of layer k's optics: the optical depth
// ke * amount, the scattering bs = ke * w * amount and the phase sums
// pc[l] * bs (l = 1..nleg for a cloud, 0..nleg for an aerosol) are added to
// od, bs_sum and pcs.  Species 0..n_clouds-1 are the clouds
// (CRTM_Compute_CloudScatter, CRTM_CloudScatter.f90:221-399), then the
// aerosols (CRTM_Compute_AerosolScatter, CRTM_AerosolScatter.f90:170-317).
// A species below its amount threshold (or a cloud in a layer whose
// Cloud_Fraction drops it) adds nothing.  Returns 0 or a negative error.
template <class S, class Seed>
CRTM_HD int species_share(const CloudyColumn& in, const CloudLut& lut, int nleg, int loff, int k, int sp, S tk,
                          Seed seed, S* od, S* bs_sum, S* pcs) {
  S pc[SC_NLEG_MAX + 1];
  if (sp < in.n_clouds) {
    if (in.cf && in.cf[k] < MIN_COVERAGE) return 0;
    const double wcv = in.wc[sp * in.cstride + k] / in.wc_div;
    if (!(wcv > WATER_CONTENT_THRESHOLD)) return 0;
    S wc(wcv), re(in.reff[sp * in.cstride + k]), unused(0.0);
    seed(sp, wc, re, unused);
    S ke, w;
    if (!cloud_layer_optics<S>(lut, in.microwave, in.freq, in.cloud_type[sp], re, tk, nleg, loff, &ke, &w, pc,
                               in.zc))
      return -4;
    if (ke <= 0.0) { ke = S(0.0); w = S(0.0); }
    if (w <= 0.0) { w = S(0.0); for (int l = 0; l <= nleg; l++) pc[l] = S(0.0); }
    if (w >= 1.0) w = S(1.0);
    *od += ke * wc;
    const S bs = ke * w * wc;
    *bs_sum += bs;
    for (int l = 1; l <= nleg; l++) pcs[l] += pc[l] * bs;
    return 0;
  }
  const int c = sp - in.n_clouds;
  const double concv = in.conc[c * in.cstride + k];
  if (!(concv > AEROSOL_CONTENT_THRESHOLD)) return 0;
  S conc(concv), re(in.aer_reff[c * in.cstride + k]);
  S sg(in.aer_var ? in.aer_var[c * in.cstride + k] : 0.0), rh(in.rh ? in.rh[k] : 0.0);
  seed(sp, conc, in.alut->scheme >= AEROSOL_GOCART ? rh : re, sg);
  S ke, w;
  if (!aerosol_layer_optics<S>(*in.alut, in.wavenumber, in.aerosol_type[c], re, sg, rh, nleg, loff, &ke, &w, pc))
    return -9;
  if (ke <= 0.0) { ke = S(0.0); w = S(0.0); }
  if (w <= 0.0) { w = S(0.0); for (int l = 0; l <= nleg; l++) pc[l] = S(0.0); }
  if (w >= 1.0) w = S(1.0);
  *od += ke * conc;
  const S bs = conc * ke * w;
  *bs_sum += bs;
  for (int l = 0; l <= nleg; l++) pcs[l] += pc[l] * bs;
  return 0;
}

// Number of species of a column whose optics enter the layers: its clouds,
// and its aerosols for an infrared sensor.  Returns -8 when the aerosol table
// cannot serve the stream set.
CRTM_HD int scattering_species(const CloudyColumn& in, int nleg, int loff) {
  if (in.n_aerosols > 0 && !in.microwave) {
    if (nleg == 2 || !in.alut || in.alut->nleg < nleg + loff) return -8;
    return in.n_clouds + in.n_aerosols;
  }
  return in.n_clouds;
}

// Sum of every species' share of layer k (species_share), clouds first.
template <class S, class Seed>
CRTM_HD int species_sums(const CloudyColumn& in, const CloudLut& lut, int nleg, int loff, int k, S tk, Seed seed,
                         S* od, S* bs_sum, S* pcs) {
  for (int c = 0; c < in.n_clouds; c++)
    if (const int rc = species_share<S>(in, lut, nleg, loff, k, c, tk, seed, od, bs_sum, pcs)) return rc;
  const int nsp = scattering_species(in, nleg, loff);
  if (nsp < 0) return nsp;
  for (int c = in.n_clouds; c < nsp; c++)
    if (const int rc = species_share<S>(in, lut, nleg, loff, k, c, tk, seed, od, bs_sum, pcs)) return rc;
  return 0;
}

// Optics of layer k for the adding method: cloud and aerosol optics summed
// over the species, combine and delta truncation, and for a scattering layer
// the phase blocks and the layer's transmission, reflection and source
// (ada_layer, or SOI doubling).  Computed in S (FP64, FP32 in the mixed
// form's ADA layers, or derivative numbers), stored in T.  Returns 1 for a
// scattering layer, 0 for a clear one (od is then the layer optical depth),
// negative on failure.  bs_out (optional): the layer's scattering
// coefficient before the delta truncation where it is significant, else 0
// (its term of the scattering optical depth, CRTM_AtmOptics.f90:425-427).
template <int NZ, class T, class S = double, class Seed = NoSeed>
CRTM_HD int layer_optics(const CloudyColumn& in, const CloudLut& lut, const StreamSet<NZ, double>& St, int k,
                         S gas_od, S tk, T* od_out, Mat<NZ, T>& Tm, Mat<NZ, T>& Rm, T* src,
                         Seed seed = Seed(), double* gap = nullptr, double* bs_out = nullptr) {
  const int nleg = St.nleg;
  S od = gas_od, bs_sum = S(0.0);
  S pcs[SC_NLEG_MAX + 1];
  for (int l = 0; l <= nleg; l++) pcs[l] = S(0.0);
  if (const int rc = species_sums<S>(in, lut, nleg, St.loff, k, tk, seed, &od, &bs_sum, pcs)) return rc;
  if (bs_out) *bs_out = bs_sum > BS_THRESHOLD ? double(value_of(bs_sum)) : 0.0;
  S ssa = bs_sum;
  if (bs_sum > BS_THRESHOLD) {   // CRTM_AtmOptics_Combine
    const S w = bs_sum / od;
    const S ib = 1.0 / bs_sum;
    for (int l = 1; l <= nleg; l++) pcs[l] *= ib;
    pcs[0] = S(0.5);
    const S f = pcs[nleg];
    od = (1.0 - f * w) * od;
    ssa = (1.0 - f) * w / (1.0 - f * w);
  }
  *od_out = T(od);
  if (!(ssa > BS_THRESHOLD)) return 0;
  // Phase blocks and MOM in S; the stored layer record is in T.
  Mat<NZ, S> ff, bb, Td, Rd;
  S mu[NZ], wt[NZ], P[NZ][SC_NLEG_MAX + 1], srcd[NZ];
  for (int i = 0; i < St.nZ; i++) {
    mu[i] = S(St.mu[i]);
    wt[i] = S(St.wt[i]);
    for (int l = 0; l <= nleg; l++) P[i][l] = S(St.P[i][l]);
  }
  phase_blocks<NZ, S>(St.nS, St.nZ, nleg, pcs, P, wt, ff, bb);
  const S B = in.c1 / (exp(in.c2 / (in.b1 + in.b2 * tk)) - 1.0);
  if (in.soi) {   // SOI: doubling, then the direct beam taken out of the diagonal
    soi_doubling<NZ, S>(ssa < 0.8 && od < 4.0, St.nS, St.nZ, ssa, od, mu, wt, ff, bb, B, Td, Rd, srcd);
    for (int i = 0; i < St.nZ; i++) Td.a[i][i] -= exp(-od / mu[i]);
  } else {
    S mx = S(0.0);
    for (int i = 0; i < St.nZ; i++)
      for (int j = 0; j < St.nZ; j++) mx = fabs(ff.a[i][j]) > mx ? fabs(ff.a[i][j]) : mx;
    if (!(mx > 0.0)) return 0;
    // loss form U = I - T: the record's T = I - U is formed in the record's
    // type, so a layer solved in FP32 keeps its relative precision in FP64 records
    double g32 = 1.0;
    const bool ok = ada_layer_loss<NZ, S>(St.nS, St.nZ, ssa, od, mu, wt, ff, bb, B, Td, Rd, srcd,
                                          gap ? gap : &g32);
    if constexpr (std::is_same<S, float>::value) {
      bool in_fp64 = !ok;
      if (ok && (gap ? *gap : g32) < FP32_GAP_MIN && St.nZ == St.nS + 1) {
        // the sensor angle nearly meets a MOM eigenvalue: the layer at sensor
        // angles mu (1 +- h), mu (1 +- 2h), combined as (4 M(h) - M(2h)) / 3
        // of the symmetric means (T, R and the source are smooth in the
        // sensor angle; error O(h^4)); FP64 if a shifted angle fails too
        const int zz = St.nZ - 1;
        Mat<NZ, S> Ta, Ra, f2, b2, T2, R2;
        S sa[NZ], s2[NZ], m2[NZ], P2[NZ][SC_NLEG_MAX + 1];
        for (int i = 0; i < St.nZ; i++) {
          sa[i] = S(0.0);
          m2[i] = mu[i];
          for (int l = 0; l <= nleg; l++) P2[i][l] = P[i][l];
          for (int j = 0; j < St.nZ; j++) { Ta.a[i][j] = S(0.0); Ra.a[i][j] = S(0.0); }
        }
#pragma unroll 1
        for (int side = 0; side < 4 && !in_fp64; side++) {
          const double fsh = (side & 1 ? -1.0 : 1.0) * (side < 2 ? FP32_SENSOR_SHIFT : 2.0 * FP32_SENSOR_SHIFT);
          const S wgt = S((side < 2 ? 4.0 : -1.0) / 6.0);
          const double ms = St.mu[zz] * (1.0 + fsh);
          double q[SC_NLEG_MAX + 1];
          q[0] = 1.0;
          if (nleg > 0) q[1] = ms;
          for (int j = 1; j < nleg; j++) q[j + 1] = ((2 * j + 1) * ms * q[j] - j * q[j - 1]) / (j + 1);
          m2[zz] = S(ms);
          for (int l = 0; l <= nleg; l++) P2[zz][l] = S(q[l]);
          phase_blocks<NZ, S>(St.nS, St.nZ, nleg, pcs, P2, wt, f2, b2);
          double g2 = 1.0;
          if (!ada_layer_loss<NZ, S>(St.nS, St.nZ, ssa, od, m2, wt, f2, b2, B, T2, R2, s2, &g2) ||
              g2 < FP32_GAP_MIN) {
            in_fp64 = true;
            break;
          }
          for (int i = 0; i < St.nZ; i++) {
            sa[i] += wgt * s2[i];
            for (int j = 0; j < St.nZ; j++) { Ta.a[i][j] += wgt * T2.a[i][j]; Ra.a[i][j] += wgt * R2.a[i][j]; }
          }
        }
        if (!in_fp64)
          for (int i = 0; i < St.nZ; i++) {
            srcd[i] = sa[i];
            for (int j = 0; j < St.nZ; j++) { Td.a[i][j] = Ta.a[i][j]; Rd.a[i][j] = Ra.a[i][j]; }
          }
      }
      if (in_fp64) {   // this layer in FP64
        Mat<NZ, double> f2, b2, T2, R2;
        double m2[NZ], w2[NZ], s2[NZ];
        for (int i = 0; i < St.nZ; i++) {
          m2[i] = St.mu[i];
          w2[i] = St.wt[i];
          for (int j = 0; j < St.nZ; j++) { f2.a[i][j] = double(ff.a[i][j]); b2.a[i][j] = double(bb.a[i][j]); }
        }
        if (!ada_layer_loss<NZ, double>(St.nS, St.nZ, double(ssa), double(od), m2, w2, f2, b2, double(B), T2, R2,
                                        s2))
          return -5;
        for (int i = 0; i < St.nZ; i++) {
          srcd[i] = S(s2[i]);
          for (int j = 0; j < St.nZ; j++) { Td.a[i][j] = S(T2.a[i][j]); Rd.a[i][j] = S(R2.a[i][j]); }
        }
      }
    } else {
      if (!ok) return -5;
    }
    for (int i = 0; i < St.nZ; i++) {
      src[i] = T(srcd[i]);
      for (int j = 0; j < St.nZ; j++) {
        Tm.a[i][j] = (i == j ? T(1.0) : T(0.0)) - T(Td.a[i][j]);
        Rm.a[i][j] = T(Rd.a[i][j]);
      }
    }
    return 1;
  }
  for (int i = 0; i < St.nZ; i++) {
    src[i] = T(srcd[i]);
    for (int j = 0; j < St.nZ; j++) { Tm.a[i][j] = T(Td.a[i][j]); Rm.a[i][j] = T(Rd.a[i][j]); }
  }
  return 1;
}

// Adding state: reflectivity of everything below the current level (Rup) and
// upwelling radiance there (rad), in the adding's arithmetic A (FP64 in the
// FP64 form and the forward; the mixed form's K-matrix and adjoint run the
// adding and its adjoint in FP32 with the (I - Rup R)^-1 inversions in FP64).
template <int NZ, class A = double>
struct AddingState {
  Mat<NZ, A> Rup;
  A rad[NZ];
};

// Gamma = G^-1 in place for G = I - Rup R.  In FP32, where the coupling is
// weak (||I - G||_inf < 1/2, so cond(G) < 3 and FP32 elimination keeps ~1e-7
// relative) the elimination runs in FP32; otherwise in FP64 (thick, nearly
// conservative layers over a reflecting column, where G nears singular).
constexpr double ADDING_FP32_COUPLING = 0.5;
template <int NZ, class A>
CRTM_HD bool invert_fp64(int n, Mat<NZ, A>& G) {
  if constexpr (sizeof(A) == sizeof(double)) {
    return mat_invert<NZ, A>(n, G);
  } else {
    A cpl = A(0.0);
    for (int i = 0; i < n; i++) {
      A r = A(0.0);
      for (int j = 0; j < n; j++) r += fabs((i == j ? A(1.0) : A(0.0)) - G.a[i][j]);
      cpl = r > cpl ? r : cpl;
    }
    if (cpl < A(ADDING_FP32_COUPLING)) return mat_invert<NZ, A>(n, G);
    Mat<NZ, double> D;
    for (int i = 0; i < n; i++)
      for (int j = 0; j < n; j++) D.a[i][j] = double(G.a[i][j]);
    if (!mat_invert<NZ, double>(n, D)) return false;
    for (int i = 0; i < n; i++)
      for (int j = 0; j < n; j++) G.a[i][j] = A(D.a[i][j]);
    return true;
  }
}

template <int NZ, class A = double>
CRTM_HD void adding_init(AddingState<NZ, A>& S, int nZ, double emissivity, double planck_surface) {
  for (int i = 0; i < nZ; i++) {
    for (int j = 0; j < nZ; j++) S.Rup.a[i][j] = A(0.0);
    S.Rup.a[i][i] = A(1.0 - emissivity);
    S.rad[i] = A(emissivity * planck_surface);
  }
}

// Clear layer: diagonal transmission exp(-od/mu_i), source B (1 - t_i).
template <int NZ, class A = double>
CRTM_HD void adding_clear(AddingState<NZ, A>& S, int nZ, const double* mu, double od, double B) {
  A tr[NZ], src[NZ], tmp[NZ];
  for (int i = 0; i < nZ; i++) {
    const A x = A(-od / mu[i]);
    tr[i] = exp(x);
    src[i] = -A(B) * expm1(x);
  }
  for (int i = 0; i < nZ; i++) {
    A v = S.rad[i];
    for (int j = 0; j < nZ; j++) v += S.Rup.a[i][j] * src[j];
    tmp[i] = src[i] + tr[i] * v;
  }
  for (int i = 0; i < nZ; i++) {
    S.rad[i] = tmp[i];
    for (int j = 0; j < nZ; j++) S.Rup.a[i][j] *= tr[i] * tr[j];
  }
}

// Scattering layer (ADA_Module.f90:169-190): Gamma = (I - Rup R)^-1,
// rad <- src + T Gamma (Rup src + rad),  Rup <- R + T Gamma Rup T.
template <int NZ, class A = double>
CRTM_HD bool adding_scatter(AddingState<NZ, A>& S, int nZ, const Mat<NZ, A>& Tm, const Mat<NZ, A>& Rm,
                            const A* src) {
  Mat<NZ, A> G, IGT;
  A tmp[NZ];
  for (int i = 0; i < nZ; i++)
    for (int j = 0; j < nZ; j++) {
      A v = A(0.0);
      for (int m = 0; m < nZ; m++) v += S.Rup.a[i][m] * Rm.a[m][j];
      G.a[i][j] = (i == j ? A(1.0) : A(0.0)) - v;
    }
  if (!invert_fp64<NZ, A>(nZ, G)) return false;
  mat_mul<NZ, A>(nZ, Tm, G, IGT);
  for (int i = 0; i < nZ; i++) {
    A v = S.rad[i];
    for (int j = 0; j < nZ; j++) v += S.Rup.a[i][j] * src[j];
    tmp[i] = v;
  }
  for (int i = 0; i < nZ; i++) {
    A v = src[i];
    for (int j = 0; j < nZ; j++) v += IGT.a[i][j] * tmp[j];
    S.rad[i] = v;
  }
  mat_mul<NZ, A>(nZ, S.Rup, Tm, G);    // Rup T
  mat_mul<NZ, A>(nZ, IGT, G, S.Rup);   // T Gamma Rup T
  for (int i = 0; i < nZ; i++)
    for (int j = 0; j < nZ; j++) S.Rup.a[i][j] += Rm.a[i][j];
  return true;
}

template <int NZ, class A = double>
CRTM_HD double adding_toa(const AddingState<NZ, A>& S, int nZ, int isat, double cosmic) {
  double s = 0.0;
  for (int j = 0; j < nZ; j++) s += double(S.Rup.a[isat][j]);
  return double(S.rad[isat]) + s * cosmic;
}

// ---- adjoint of the adding (reverse mode), unit TOA radiance seed ----------
// The forward adding maps (Rup, rad) below a layer to (Rup', rad') above it.
// Given the adjoints of (Rup', rad'), these give the adjoints of (Rup, rad)
// and of the layer's inputs.  The forward state below the layer is passed in.

// Clear layer (diagonal transmission t_i = exp(-od/mu_i), source B (1 - t_i)):
// returns d/d(od) and d/dB.
template <int NZ, class A = double>
CRTM_HD void adding_clear_adjoint(int nZ, const double* mu, double od, double B, const Mat<NZ, A>& Rup,
                                  const A* rad, Mat<NZ, A>& Rup_b, A* rad_b, double* od_b, double* B_b) {
  A tr[NZ], src[NZ], om[NZ], t[NZ], tr_b[NZ], src_b[NZ], t_b[NZ];
  const A Bw = A(B);
  for (int i = 0; i < nZ; i++) {
    const A x = A(-od / mu[i]);
    tr[i] = exp(x);
    om[i] = -expm1(x);   // 1 - t_i
    src[i] = Bw * om[i];
  }
  for (int i = 0; i < nZ; i++) {
    A v = rad[i];
    for (int j = 0; j < nZ; j++) v += Rup.a[i][j] * src[j];
    t[i] = v;
  }
  // rad'_i = src_i + tr_i t_i ;  Rup'_ij = tr_i Rup_ij tr_j
  for (int i = 0; i < nZ; i++) {
    src_b[i] = rad_b[i];
    tr_b[i] = rad_b[i] * t[i];
    t_b[i] = rad_b[i] * tr[i];
  }
  for (int i = 0; i < nZ; i++)
    for (int j = 0; j < nZ; j++) {
      const A g = Rup_b.a[i][j];
      tr_b[i] += g * Rup.a[i][j] * tr[j];
      tr_b[j] += g * tr[i] * Rup.a[i][j];
      Rup_b.a[i][j] = g * tr[i] * tr[j];
    }
  // t_i = rad_i + sum_j Rup_ij src_j
  for (int i = 0; i < nZ; i++) {
    rad_b[i] = t_b[i];
    for (int j = 0; j < nZ; j++) {
      Rup_b.a[i][j] += t_b[i] * src[j];
      src_b[j] += t_b[i] * Rup.a[i][j];
    }
  }
  A ob = A(0.0), bb = A(0.0);
  for (int i = 0; i < nZ; i++) {
    bb += src_b[i] * om[i];
    tr_b[i] -= src_b[i] * Bw;
    ob -= tr_b[i] * tr[i] / A(mu[i]);
  }
  *od_b = double(ob);
  *B_b = double(bb);
}

// Scattering layer (transmission T, reflection R, source src): adjoints of the
// layer's T, R and src.  Returns false on a singular (I - Rup R).
template <int NZ, class A = double>
CRTM_HD bool adding_scatter_adjoint(int nZ, const Mat<NZ, A>& Tm, const Mat<NZ, A>& Rm, const A* src,
                                    const Mat<NZ, A>& Rup, const A* rad, Mat<NZ, A>& Rup_b, A* rad_b,
                                    Mat<NZ, A>& T_b, Mat<NZ, A>& R_b, A* src_b) {
  Mat<NZ, A> G, IGT, RT, M1, M2;
  A t[NZ], t_b[NZ];
  for (int i = 0; i < nZ; i++)
    for (int j = 0; j < nZ; j++) {
      A v = A(0.0);
      for (int m = 0; m < nZ; m++) v += Rup.a[i][m] * Rm.a[m][j];
      G.a[i][j] = (i == j ? A(1.0) : A(0.0)) - v;
    }
  if (!invert_fp64<NZ, A>(nZ, G)) return false;     // G now holds Gamma
  mat_mul<NZ, A>(nZ, Tm, G, IGT);
  mat_mul<NZ, A>(nZ, Rup, Tm, RT);
  for (int i = 0; i < nZ; i++) {
    A v = rad[i];
    for (int j = 0; j < nZ; j++) v += Rup.a[i][j] * src[j];
    t[i] = v;
  }
  // IGT_b = rad'_b t^T + Rup'_b RT^T  (in M1);  t_b = IGT^T rad'_b;  RT_b = IGT^T Rup'_b (in M2)
  for (int i = 0; i < nZ; i++) {
    src_b[i] = rad_b[i];
    for (int j = 0; j < nZ; j++) {
      A v = rad_b[i] * t[j];
      for (int m = 0; m < nZ; m++) v += Rup_b.a[i][m] * RT.a[j][m];
      M1.a[i][j] = v;
    }
  }
  for (int j = 0; j < nZ; j++) {
    A v = A(0.0);
    for (int i = 0; i < nZ; i++) v += IGT.a[i][j] * rad_b[i];
    t_b[j] = v;
  }
  for (int i = 0; i < nZ; i++)
    for (int j = 0; j < nZ; j++) {
      A v = A(0.0);
      for (int m = 0; m < nZ; m++) v += IGT.a[m][i] * Rup_b.a[m][j];
      M2.a[i][j] = v;
      R_b.a[i][j] = Rup_b.a[i][j];
    }
  // RT = Rup T:  Rup_b = RT_b T^T ;  T_b = Rup^T RT_b
  Mat<NZ, A> Rb_new;
  for (int i = 0; i < nZ; i++)
    for (int j = 0; j < nZ; j++) {
      A a = A(0.0), b = A(0.0);
      for (int m = 0; m < nZ; m++) {
        a += M2.a[i][m] * Tm.a[j][m];
        b += Rup.a[m][i] * M2.a[m][j];
      }
      Rb_new.a[i][j] = a;
      T_b.a[i][j] = b;
    }
  // t = rad + Rup src
  for (int i = 0; i < nZ; i++) {
    rad_b[i] = t_b[i];
    for (int j = 0; j < nZ; j++) {
      Rb_new.a[i][j] += t_b[i] * src[j];
      src_b[j] += t_b[i] * Rup.a[i][j];
    }
  }
  // IGT = T Gamma:  T_b += IGT_b Gamma^T ;  Gamma_b = T^T IGT_b (in M2)
  for (int i = 0; i < nZ; i++)
    for (int j = 0; j < nZ; j++) {
      A a = A(0.0), b = A(0.0);
      for (int m = 0; m < nZ; m++) {
        a += M1.a[i][m] * G.a[j][m];
        b += Tm.a[m][i] * M1.a[m][j];
      }
      T_b.a[i][j] += a;
      M2.a[i][j] = b;
    }
  // Gamma = G^-1:  G_b = -Gamma^T Gamma_b Gamma^T (in M1)
  for (int i = 0; i < nZ; i++)
    for (int j = 0; j < nZ; j++) {
      A v = A(0.0);
      for (int m = 0; m < nZ; m++) v += M2.a[i][m] * G.a[j][m];
      IGT.a[i][j] = v;   // Gamma_b Gamma^T
    }
  for (int i = 0; i < nZ; i++)
    for (int j = 0; j < nZ; j++) {
      A v = A(0.0);
      for (int m = 0; m < nZ; m++) v += G.a[m][i] * IGT.a[m][j];
      M1.a[i][j] = -v;
    }
  // G = I - Rup R:  Rup_b -= G_b R^T ;  R_b -= Rup^T G_b
  for (int i = 0; i < nZ; i++)
    for (int j = 0; j < nZ; j++) {
      A a = A(0.0), b = A(0.0);
      for (int m = 0; m < nZ; m++) {
        a += M1.a[i][m] * Rm.a[j][m];
        b += Rup.a[m][i] * M1.a[m][j];
      }
      Rb_new.a[i][j] -= a;
      R_b.a[i][j] -= b;
    }
  Rup_b = Rb_new;
  return true;
}

// One order of interaction n (1-based) of CRTM_SOI (SOI_Module.f90:63-283):
// the order's downwelling and upwelling fields go to field slot cur, computed
// from the previous order's in slot prev (not read for n = 1).  Order 1
// carries the thermal sources, the surface emission and the cosmic
// background; each later order scatters the previous order's diffuse fields
// through the layers' T (direct beam removed) and R; between scattering events
// the fields propagate with the direct transmission exp(-od / mu).
// lod(k, &kind, &od, &B) gives layer k's kind (0 clear, 1 scattering), optical
// depth and Planck radiance; lsrc(k, src) and ltr(k, T, R) its source and
// matrices (scattering layers).  fld(slot, f, k, i): field f (0 down, 1 up) at
// level k (0 top, Ku surface), angle i.  Returns the order's upwelling
// radiance at the top in the sensor angle.
template <int NZ, class LodFn, class SrcFn, class TrFn, class FldFn>
CRTM_HD double soi_order(int n, int cur, int prev, int nZ, int Ku, int isat, const double* mu,
                         double emissivity, double planck_surface, double cosmic, LodFn lod, SrcFn lsrc,
                         TrFn ltr, FldFn fld) {
  Mat<NZ, double> Tm, Rm;
  double sv[NZ], etr[NZ];
  for (int i = 0; i < nZ; i++) fld(cur, 0, 0, i) = n == 1 ? cosmic : 0.0;
  for (int dir = 0; dir < 2; dir++) {   // down from the top, then up from the surface
    if (dir == 1)
      for (int i = 0; i < nZ; i++)
        fld(cur, 1, Ku, i) = (1.0 - emissivity) * fld(cur, 0, Ku, i) + (n == 1 ? emissivity * planck_surface : 0.0);
    for (int m = 0; m < Ku; m++) {
      const int k = dir == 0 ? m : Ku - 1 - m;
      int kind;
      double od, B;
      lod(k, &kind, &od, &B);
      for (int i = 0; i < nZ; i++) etr[i] = exp(-od / mu[i]);
      if (n == 1) {
        if (kind == 1)
          lsrc(k, sv);
        else
          for (int i = 0; i < nZ; i++) sv[i] = B * (1.0 - etr[i]);
      } else if (kind == 1 && od >= 1.0e-6) {
        ltr(k, Tm, Rm);
        const Mat<NZ, double>& A = dir == 0 ? Tm : Rm;   // acts on the downwelling field above
        const Mat<NZ, double>& C = dir == 0 ? Rm : Tm;   // acts on the upwelling field below
        for (int i = 0; i < nZ; i++) {
          double v = 0.0;
          for (int j = 0; j < nZ; j++) v += A.a[i][j] * fld(prev, 0, k, j) + C.a[i][j] * fld(prev, 1, k + 1, j);
          sv[i] = v;
        }
      } else {
        for (int i = 0; i < nZ; i++) sv[i] = 0.0;
      }
      if (dir == 0)
        for (int i = 0; i < nZ; i++) fld(cur, 0, k + 1, i) = fld(cur, 0, k, i) * etr[i] + sv[i];
      else
        for (int i = 0; i < nZ; i++) fld(cur, 1, k, i) = fld(cur, 1, k + 1, i) * etr[i] + sv[i];
    }
  }
  return fld(cur, 1, 0, isat);
}

// CRTM_SOI: orders until the newest adds less than 1e-4 of the radiance (at
// least 2, at most 75: MAX_N_SOI_ITERATIONS), fields in two slots.
constexpr int SOI_MAX_ORDERS = 75;
template <int NZ, class LodFn, class SrcFn, class TrFn, class FldFn>
CRTM_HD int soi_solve(int nZ, int Ku, int isat, const double* mu, double emissivity, double planck_surface,
                      double cosmic, LodFn lod, SrcFn lsrc, TrFn ltr, FldFn fld, double* radiance) {
  double total = 0.0, change = 1.0e10;
  int n = 0;
  while ((change > 1.0e-4 && n + 1 <= SOI_MAX_ORDERS) || n < 2) {
    n++;
    const double rad = soi_order<NZ>(n, (n - 1) & 1, n & 1, nZ, Ku, isat, mu, emissivity, planck_surface, cosmic,
                                     lod, lsrc, ltr, fld);
    total += rad;
    change = rad / total;
  }
  *radiance = total;
  return 0;
}

// Adjoint of the SOI for a unit radiance seed (CRTM_SOI_AD,
// SOI_Module.f90:477-): every order of interaction is linear in the previous
// order's fields, so the reverse runs from the last order down, each order's
// fields' adjoints collecting the seed (its share of the radiance), the next
// order's scattering sources and the propagation.  Accumulates into
// ab(k, e) layer k's record adjoints in the record layout (e = 0 kind, 1 od_b,
// then T_b, R_b, src_b for a scattering layer, 2 the Planck radiance's B_b for
// a clear one) and returns the radiance, dR/de and dR/d(surface Planck).
//
// Field storage: n_slots order fields fld(slot, ...) (at least 17) and two
// adjoint fields lam(b, f, k, i), b = 0, 1.  With the orders' count N at most
// n_slots every order is kept; beyond, orders c, 2c, ... are kept as
// checkpoints (c the smallest with (N-1)/c + c <= n_slots) and each segment
// of c orders is recomputed from its checkpoint before its reverse.
template <int NZ, class LodFn, class SrcFn, class TrFn, class FldFn, class LamFn, class AbFn>
CRTM_HD int soi_adjoint(int nZ, int Ku, int isat, const double* mu, double emissivity, double planck_surface,
                        double cosmic, int n_slots, LodFn lod, SrcFn lsrc, TrFn ltr, FldFn fld, LamFn lam,
                        AbFn ab, double* radiance, double* e_b, double* Bs_b, int* n_orders = nullptr) {
  constexpr int NE_T = 2, NE_R = 2 + NZ * NZ, NE_S = 2 + 2 * NZ * NZ;
  if (n_slots < 17) return 12;
  // forward: orders into slots 0..n_slots-1, beyond that alternately into the last two
  const int M = n_slots;
  auto slot1 = [&](int n) { return n <= M ? n - 1 : M - 1 - ((n - M) & 1); };
  double total = 0.0, change = 1.0e10;
  int N = 0;
  while ((change > 1.0e-4 && N + 1 <= SOI_MAX_ORDERS) || N < 2) {
    N++;
    const double rad = soi_order<NZ>(N, slot1(N), N > 1 ? slot1(N - 1) : 0, nZ, Ku, isat, mu, emissivity,
                                     planck_surface, cosmic, lod, lsrc, ltr, fld);
    total += rad;
    change = rad / total;
  }
  *radiance = total;
  if (n_orders) *n_orders = N;
  // segments: c orders each, checkpoints at orders c, 2c, ..., nck c
  int c = N, nck = 0;
  if (N > M) {
    for (c = 2; c <= N; c++)
      if ((N - 1) / c + c <= M) break;
    nck = (N - 1) / c;
  }
  auto slot2 = [&](int n) { return (n % c == 0 && n / c <= nck) ? n / c - 1 : nck + (n - 1) % c; };
  auto slot = [&](int n) { return N <= M ? n - 1 : slot2(n); };
  auto order_into = [&](int n) {
    soi_order<NZ>(n, slot(n), n > 1 ? slot(n - 1) : 0, nZ, Ku, isat, mu, emissivity, planck_surface, cosmic, lod,
                  lsrc, ltr, fld);
  };
  if (N > M)
    for (int n = 1; n <= nck * c; n++) order_into(n);   // the checkpoints
  // record adjoints and adjoint fields start at zero
  for (int k = 0; k < Ku; k++) {
    int kind;
    double od, B;
    lod(k, &kind, &od, &B);
    ab(k, 0) = kind;
    ab(k, 1) = 0.0;
    if (kind == 1) {
      for (int i = 0; i < nZ; i++) {
        for (int j = 0; j < nZ; j++) { ab(k, NE_T + i * NZ + j) = 0.0; ab(k, NE_R + i * NZ + j) = 0.0; }
        ab(k, NE_S + i) = 0.0;
      }
    } else {
      ab(k, 2) = 0.0;
    }
  }
  for (int b = 0; b < 2; b++)
    for (int f = 0; f < 2; f++)
      for (int k = 0; k <= Ku; k++)
        for (int i = 0; i < nZ; i++) lam(b, f, k, i) = 0.0;
  double eb = 0.0, bsb = 0.0;
  Mat<NZ, double> Tm, Rm;
  double etr[NZ], sd[NZ], su[NZ];
  for (int s = nck; s >= 0; s--) {
    const int a0 = s * c + 1, b0 = s == nck ? N : (s + 1) * c;
    if (N > M)
      for (int n = a0; n <= b0; n++) order_into(n);
    for (int n = b0; n >= a0; n--) {
      const int cur = slot(n), prv = n > 1 ? slot(n - 1) : 0, lc = n & 1, lp = lc ^ 1;
      lam(lc, 1, 0, isat) += 1.0;
      // up(k) = up(k+1) etr + sv_up(k), k = Ku-1 .. 0
      for (int k = 0; k < Ku; k++) {
        int kind;
        double od, B;
        lod(k, &kind, &od, &B);
        double g = 0.0;
        for (int i = 0; i < nZ; i++) {
          const double e = exp(-od / mu[i]), lu = lam(lc, 1, k, i);
          lam(lc, 1, k + 1, i) += lu * e;
          g += lu * fld(cur, 1, k + 1, i) * e / mu[i];
        }
        ab(k, 1) -= g;
      }
      // surface: up(Ku) = (1 - e) dn(Ku) + [n = 1] e Bs
      for (int i = 0; i < nZ; i++) {
        const double lu = lam(lc, 1, Ku, i);
        lam(lc, 0, Ku, i) += (1.0 - emissivity) * lu;
        eb += lu * ((n == 1 ? planck_surface : 0.0) - fld(cur, 0, Ku, i));
        if (n == 1) bsb += emissivity * lu;
      }
      // dn(k+1) = dn(k) etr + sv_dn(k), k = 0 .. Ku-1; then the sources of layer k
      for (int k = Ku - 1; k >= 0; k--) {
        int kind;
        double od, B;
        lod(k, &kind, &od, &B);
        double g = 0.0;
        for (int i = 0; i < nZ; i++) {
          etr[i] = exp(-od / mu[i]);
          const double ld = lam(lc, 0, k + 1, i);
          lam(lc, 0, k, i) += ld * etr[i];
          g += ld * fld(cur, 0, k, i) * etr[i] / mu[i];
          sd[i] = ld;
          su[i] = lam(lc, 1, k, i);
        }
        ab(k, 1) -= g;
        if (n == 1) {
          if (kind == 1) {
            for (int i = 0; i < nZ; i++) ab(k, NE_S + i) += sd[i] + su[i];
          } else {
            double gb = 0.0, go = 0.0;
            for (int i = 0; i < nZ; i++) {
              const double w = sd[i] + su[i];
              gb += w * (1.0 - etr[i]);
              go += w * B * etr[i] / mu[i];
            }
            ab(k, 2) += gb;
            ab(k, 1) += go;
          }
        } else if (kind == 1 && od >= 1.0e-6) {
          // sv_dn = T dn'(k) + R up'(k+1), sv_up = R dn'(k) + T up'(k+1) (' order n-1)
          ltr(k, Tm, Rm);
          for (int i = 0; i < nZ; i++)
            for (int j = 0; j < nZ; j++) {
              const double dj = fld(prv, 0, k, j), uj = fld(prv, 1, k + 1, j);
              ab(k, NE_T + i * NZ + j) += sd[i] * dj + su[i] * uj;
              ab(k, NE_R + i * NZ + j) += sd[i] * uj + su[i] * dj;
            }
          for (int j = 0; j < nZ; j++) {
            double ad = 0.0, au = 0.0;
            for (int i = 0; i < nZ; i++) {
              ad += Tm.a[i][j] * sd[i] + Rm.a[i][j] * su[i];
              au += Rm.a[i][j] * sd[i] + Tm.a[i][j] * su[i];
            }
            lam(lp, 0, k, j) += ad;
            lam(lp, 1, k + 1, j) += au;
          }
        }
      }
      // order n's adjoints are spent: the buffer becomes order n-2's
      for (int f = 0; f < 2; f++)
        for (int k = 0; k <= Ku; k++)
          for (int i = 0; i < nZ; i++) lam(lc, f, k, i) = 0.0;
    }
  }
  *e_b = eb;
  *Bs_b = bsb;
  return 0;
}

// The whole (profile, channel) in one pass, FP64 (the layer-parallel GPU
// kernels split it into layer_optics for every layer, then the adding).
template <int NZ, class OdFn>
CRTM_HD int cloudy_radiance(const CloudyColumn& in, const CloudLut& lut, const GaussTable& gt,
                            OdFn od_of, double* radiance) {
  if (in.soi) return 7;   // SOI needs every layer's record: the layered form
  StreamSet<NZ, double> S;
  if (int rc = stream_set<NZ, double>(in.nleg, in.mu_sensor, in.n_clouds > 0 ? lut.nleg : -1, gt, S)) return rc;
  AddingState<NZ> A;
  adding_init<NZ>(A, S.nZ, in.emissivity, in.planck_surface);
  Mat<NZ, double> Tm, Rm;
  double src[NZ];
  for (int k = in.Ku - 1; k >= 0; k--) {
    double od;
    const int kind = layer_optics<NZ, double>(in, lut, S, k, od_of(k), in.temperature[k], &od, Tm, Rm, src);
    if (kind < 0) return -kind;
    if (kind == 1) {
      if (!adding_scatter<NZ>(A, S.nZ, Tm, Rm, src)) return 6;
    } else {
      const double tk = in.temperature[k];
      adding_clear<NZ>(A, S.nZ, S.mu, od, in.c1 / (exp(in.c2 / (in.b1 + in.b2 * tk)) - 1.0));
    }
  }
  *radiance = adding_toa<NZ>(A, S.nZ, S.isat, in.cosmic);
  return 0;
}

// A layer's optics on derivative numbers (layer_optics with S = T = D), with
// the derivatives of a nearly defective MOM eigenbasis taken at shifted
// sensor angles.
template <int NZ, int N, class Q, class Seed>
CRTM_HD int layer_optics_dual(const CloudyColumn& in, const CloudLut& lut, const StreamSet<NZ, double>& S, int k,
                              Dual<N, Q> gd, Dual<N, Q> tt, Dual<N, Q>* odd, Mat<NZ, Dual<N, Q>>& Td,
                              Mat<NZ, Dual<N, Q>>& Rd, Dual<N, Q>* srcd, Seed seed) {
  using D = Dual<N, Q>;
  double gap = 1.0;
  const int kind = layer_optics<NZ, D, D>(in, lut, S, k, gd, tt, odd, Td, Rd, srcd, seed, &gap);
  if (kind == 1 && gap < SENSOR_GAP_MIN && S.nZ == S.nS + 1) {
    // A quadrature eigenvalue of MOM nearly meets the sensor angle's: the
    // eigenbasis is nearly defective and the derivatives through it lose
    // about eps / gap^2.  T, R and the source are smooth in the sensor angle:
    // their derivatives come from sensor angles mu (1 +- h), h = 1e-3 and
    // 2e-3 (gaps >= 1e-3 there), as the Richardson extrapolation
    // (4 D(h) - D(2h)) / 3 of the symmetric means, accurate to O(h^4).
    Mat<NZ, D> T2, R2;
    D s2[NZ], o2;
    Mat<NZ, D> Ta, Ra;
    D sa[NZ], oa;
    int n_ok = 0;
    for (int side = 0; side < 4; side++) {
      const double f = (side & 1 ? -1.0 : 1.0) * (side < 2 ? SENSOR_SHIFT : 2.0 * SENSOR_SHIFT);
      const double wgt = (side < 2 ? 4.0 : -1.0) / 6.0;   // (4 mean(h) - mean(2h)) / 3
      StreamSet<NZ, double> S2 = S;
      const int z = S.nZ - 1;
      S2.mu[z] = S.mu[z] * (1.0 + f);
      S2.P[z][0] = 1.0;
      if (S2.nleg > 0) S2.P[z][1] = S2.mu[z];
      for (int j = 1; j < S2.nleg; j++)
        S2.P[z][j + 1] = ((2 * j + 1) * S2.mu[z] * S2.P[z][j] - j * S2.P[z][j - 1]) / (j + 1);
      if (layer_optics<NZ, D, D>(in, lut, S2, k, gd, tt, &o2, T2, R2, s2, seed) != 1) break;
      for (int i = 0; i < S.nZ; i++) {
        for (int j = 0; j < S.nZ; j++)
          for (int q = 0; q < N; q++) {
            const Q t = T2.a[i][j].d[q] * wgt, r = R2.a[i][j].d[q] * wgt;
            Ta.a[i][j].d[q] = n_ok ? Ta.a[i][j].d[q] + t : t;
            Ra.a[i][j].d[q] = n_ok ? Ra.a[i][j].d[q] + r : r;
          }
        for (int q = 0; q < N; q++) sa[i].d[q] = n_ok ? sa[i].d[q] + s2[i].d[q] * wgt : s2[i].d[q] * wgt;
      }
      for (int q = 0; q < N; q++) oa.d[q] = n_ok ? oa.d[q] + o2.d[q] * wgt : o2.d[q] * wgt;
      n_ok++;
    }
    if (n_ok == 4) {   // else (a shifted angle changed the layer's kind) keep the direct derivatives
      for (int i = 0; i < S.nZ; i++) {
        for (int j = 0; j < S.nZ; j++)
          for (int q = 0; q < N; q++) { Td.a[i][j].d[q] = Ta.a[i][j].d[q]; Rd.a[i][j].d[q] = Ra.a[i][j].d[q]; }
        for (int q = 0; q < N; q++) srcd[i].d[q] = sa[i].d[q];
      }
      for (int q = 0; q < N; q++) odd->d[q] = oa.d[q];
    }
  }
  return kind;
}

// Directions of one derivative evaluation of a layer's optics: the gas
// optical depth and the temperature (when gas_t; directions 0 and 1), then
// for each listed species its amount and its first LUT coordinate c1
// (directions base + 2i and base + 2i + 1, base = 2 or 0), or with second
// set its second coordinate c2 only (direction base + i).  Species index:
// clouds 0..n_clouds-1, then aerosols.
struct LayerDirections {
  bool gas_t;
  int nsp;
  int sp[4];
  bool second = false;   // the listed species' second LUT coordinate (c2), direction i each
};

// Contraction of one layer's optics derivatives with the adjoints of its
// record: for a scattering layer g[d] = sum(T_b dT/dd) + sum(R_b dR/dd) +
// sum(src_b dsrc/dd) + od_b dod/dd (od_b is 0 for ADA, whose adding takes
// the layer's optical depth only through T, R and the source; SOI propagates
// between layers with exp(-od / mu)); for a clear one g[d] = od_b dod/dd, plus B_b dB/dT in
// the temperature direction (its Planck radiance enters the adding outside
// the layer optics).  The optics are evaluated on derivative numbers with N
// directions.  Returns the layer kind of that evaluation.
template <int NZ, int N, class Q = double>
CRTM_HD int layer_contract(const CloudyColumn& in, const CloudLut& lut, const StreamSet<NZ, double>& S, int k,
                           double gas_od, const LayerDirections& dir, const Mat<NZ, double>& T_b,
                           const Mat<NZ, double>& R_b, const double* src_b, double od_b, double B_b, double* g) {
  using D = Dual<N, Q>;
  D gd(gas_od), tt(in.temperature[k]);
  const int base = dir.gas_t ? 2 : 0;
  if (dir.gas_t) {
    gd.d[0] = 1.0;
    tt.d[1] = 1.0;
  }
  auto seed = [&](int s, D& amount, D& c1, D& c2) {
    for (int i = 0; i < dir.nsp; i++)
      if (dir.sp[i] == s) {
        if (dir.second) {
          c2.d[base + i] = 1.0;
        } else {
          amount.d[base + 2 * i] = 1.0;
          c1.d[base + 2 * i + 1] = 1.0;
        }
      }
  };
  Mat<NZ, D> Td, Rd;
  D srcd[NZ], odd;
  const int kind = layer_optics_dual<NZ>(in, lut, S, k, gd, tt, &odd, Td, Rd, srcd, seed);
  for (int d = 0; d < N; d++) g[d] = 0.0;
  if (kind == 1) {
    for (int d = 0; d < N; d++) g[d] = od_b * part(odd.d[d]);   // SOI's direct transmission
    for (int i = 0; i < S.nZ; i++)
      for (int d = 0; d < N; d++) {
        double acc = src_b[i] * part(srcd[i].d[d]);
        for (int j = 0; j < S.nZ; j++)
          acc += T_b.a[i][j] * part(Td.a[i][j].d[d]) + R_b.a[i][j] * part(Rd.a[i][j].d[d]);
        g[d] += acc;
      }
  } else if (kind == 0) {
    for (int d = 0; d < N; d++) g[d] = od_b * part(odd.d[d]);
    if (dir.gas_t) {
      const double te = in.b1 + in.b2 * in.temperature[k];
      const double ee = exp(in.c2 / te);
      g[1] += B_b * in.c1 * in.c2 * ee * in.b2 / (te * te * (ee - 1.0) * (ee - 1.0));
    }
  }
  return kind;
}

// Adjoint of the adding for one (profile, channel) through ADA, for a unit
// TOA radiance seed.  Forward adding with every level's (Rup, rad) kept in
// state(level, i) (nZ*nZ + nZ values per level, level Ku = surface), then the
// adding adjoint from the top down.  layer(k, kind, od, T, R, src) gives the
// layer records of the forward pass; adj(k, kind, T_b, R_b, src_b, od_b, B_b)
// receives each layer's record adjoints (scattering layer: T_b, R_b, src_b;
// clear layer: od_b and the Planck radiance's B_b).  Returns the radiance and
// the derivatives with respect to the surface emissivity (reflectivity 1 - e)
// and the surface Planck radiance.
template <int NZ, class LayerFn, class StateFn, class AdjFn, class A = double>
CRTM_HD int cloudy_adjoint(const CloudyColumn& in, const StreamSet<NZ, double>& S, LayerFn layer,
                           StateFn state, AdjFn adj, double* radiance, double* e_b, double* Bs_b) {
  const int nZ = S.nZ, Ku = in.Ku;
  auto planck = [&](int k) -> double {   // the layer's Planck radiance, in A
    const A te = A(in.b1) + A(in.b2) * A(in.temperature[k]);
    return double(A(in.c1) / (exp(A(in.c2) / te) - A(1.0)));
  };
  AddingState<NZ, A> St;
  adding_init<NZ, A>(St, nZ, in.emissivity, in.planck_surface);
  auto save = [&](int lev) {
    for (int i = 0; i < nZ; i++) {
      for (int j = 0; j < nZ; j++) state(lev, i * NZ + j) = St.Rup.a[i][j];
      state(lev, NZ * NZ + i) = St.rad[i];
    }
  };
  auto load = [&](int lev, Mat<NZ, A>& Rup, A* rad) {
    for (int i = 0; i < nZ; i++) {
      for (int j = 0; j < nZ; j++) Rup.a[i][j] = state(lev, i * NZ + j);
      rad[i] = state(lev, NZ * NZ + i);
    }
  };
  save(Ku);
  Mat<NZ, A> Tm, Rm;
  A src[NZ];
  for (int k = Ku - 1; k >= 0; k--) {
    int kind;
    double od;
    layer(k, &kind, &od, Tm, Rm, src);
    if (kind < 0) return -kind;
    if (kind == 1) {
      if (!adding_scatter<NZ, A>(St, nZ, Tm, Rm, src)) return 6;
    } else {
      adding_clear<NZ, A>(St, nZ, S.mu, od, planck(k));
    }
    save(k);
  }
  *radiance = adding_toa<NZ, A>(St, nZ, S.isat, in.cosmic);
  // adjoint of the TOA radiance
  Mat<NZ, A> Rup_b, Rup, T_b, R_b;
  A rad_b[NZ], rad[NZ], src_b[NZ];
  for (int i = 0; i < nZ; i++) {
    rad_b[i] = (i == S.isat) ? A(1.0) : A(0.0);
    for (int j = 0; j < nZ; j++) Rup_b.a[i][j] = (i == S.isat) ? A(in.cosmic) : A(0.0);
  }
  for (int k = 0; k < Ku; k++) {
    load(k + 1, Rup, rad);
    int kind;
    double od;
    layer(k, &kind, &od, Tm, Rm, src);
    if (kind == 1) {
      if (!adding_scatter_adjoint<NZ, A>(nZ, Tm, Rm, src, Rup, rad, Rup_b, rad_b, T_b, R_b, src_b)) return 6;
      adj(k, kind, T_b, R_b, src_b, 0.0, 0.0);
    } else {
      const double B = planck(k);
      double od_b, B_b;
      adding_clear_adjoint<NZ, A>(nZ, S.mu, od, B, Rup, rad, Rup_b, rad_b, &od_b, &B_b);
      adj(k, kind, T_b, R_b, src_b, od_b, B_b);
    }
  }
  double tr = 0.0, sr = 0.0;
  for (int i = 0; i < nZ; i++) { tr += double(Rup_b.a[i][i]); sr += double(rad_b[i]); }
  *e_b = -tr + in.planck_surface * sr;
  *Bs_b = in.emissivity * sr;
  return 0;
}

// Derivatives of the total cloud cover (total_cloud_cover) with respect to
// each layer's cloud fraction (dcf) and, for the average overlap, to the
// water content of a cloud whose content is above the threshold in that layer
// (dwc; 0 for the other schemes): the reverse of Compute_CloudCover
// (CRTM_CloudCover_Define.f90:522-638).  tcc >= 0 (a fractional profile).
CRTM_HD void cloud_cover_derivatives(int Ku, int n_clouds, const double* cf, const double* wc, size_t cstride,
                                     int overlap, double tcc, double* dcf, double* dwc) {
  auto frac = [&](int k) {
    const double f = cf ? cf[k] : 1.0;
    return f < MIN_COVERAGE ? 0.0 : f;
  };
  for (int k = 0; k < Ku; k++) dcf[k] = dwc[k] = 0.0;
  if (overlap == 1) {          // running maximum: the first layer that reaches it
    int km = 0;
    for (int k = 1; k < Ku; k++)
      if (frac(k) > frac(km)) km = k;
    if (cf && cf[km] >= MIN_COVERAGE) dcf[km] = 1.0;
  } else if (overlap == 2) {   // 1 - prod(1 - cf) over the layers above the threshold
    double pre = 1.0;
    for (int k = 0; k < Ku; k++) {
      dcf[k] = pre;            // product over the layers above k
      if (frac(k) > MIN_COVERAGE) pre *= 1.0 - frac(k);
    }
    double suf = 1.0;
    for (int k = Ku - 1; k >= 0; k--) {
      const bool on = frac(k) > MIN_COVERAGE;
      dcf[k] = on ? dcf[k] * suf : 0.0;
      if (on) suf *= 1.0 - frac(k);
    }
  } else if (overlap == 3) {   // maximum-random: reverse of the product recursion
    double prod[SC_KMAX];
    const int n = Ku < SC_KMAX ? Ku : SC_KMAX;
    prod[0] = 1.0 - frac(0);
    for (int k = 1; k < n; k++) {
      const double a = frac(k - 1), b = frac(k), mc = 1.0 - (a > b ? a : b);
      prod[k] = (prod[k - 1] == 0.0 && 1.0 - a == 0.0) ? mc : prod[k - 1] * (mc / (1.0 - a));
    }
    double pb = -1.0;          // d tcc / d prod(n-1)
    for (int k = n - 1; k >= 1; k--) {
      const double a = frac(k - 1), b = frac(k), mc = 1.0 - (a > b ? a : b);
      double mcb;
      if (prod[k - 1] == 0.0 && 1.0 - a == 0.0) {
        mcb = pb;
        pb = 0.0;
      } else {
        const double r = 1.0 / (1.0 - a);
        mcb = pb * prod[k - 1] * r;
        dcf[k - 1] += pb * prod[k - 1] * mc * r * r;
        pb = pb * mc * r;
      }
      if (a > b) dcf[k - 1] -= mcb; else dcf[k] -= mcb;
    }
    dcf[0] -= pb;
    for (int k = 0; k < n; k++)
      if (cf && cf[k] < MIN_COVERAGE) dcf[k] = 0.0;
  } else if (overlap == 4) {   // water-content weighted average
    double ws = 0.0;
    for (int k = 0; k < Ku; k++) {
      if (frac(k) == 0.0) continue;
      for (int c = 0; c < n_clouds; c++) {
        const double w = wc[c * cstride + k];
        if (w > WATER_CONTENT_THRESHOLD) ws += w;
      }
    }
    for (int k = 0; k < Ku && ws > 0.0; k++) {
      if (frac(k) == 0.0) continue;
      double lwc = 0.0;
      for (int c = 0; c < n_clouds; c++) {
        const double w = wc[c * cstride + k];
        if (w > WATER_CONTENT_THRESHOLD) lwc += w;
      }
      dcf[k] = lwc / ws;
      dwc[k] = (frac(k) - tcc) / ws;
    }
  }
}

// Stream rule (CRTM_Compute_nStreams): Legendre terms 2/4/6 from the Mie
// parameter of the largest effective radius in the profile.
CRTM_HD int stream_rule_nleg(double max_reff, double wavenumber) {
  const double mie = 2.0 * PI_D * max_reff * wavenumber / 10000.0;
  return mie < 0.01 ? 2 : (mie < 1.0 ? 4 : 6);
}

// Double_Gauss_Quadrature for n points on (0,1).
inline void double_gauss_host(int n, double* x, double* w) {
  const int k = (n + 1) / 2;
  for (int j = 1; j <= k; j++) {
    double X = cos(PI_D * (j - 0.25) / (n + 0.5)), XP, PL = 0, PL1, PL2, DPL = 1;
    for (int it = 0; it < 10; it++) {
      PL1 = 1.0;
      PL = X;
      for (int l = 2; l <= n; l++) {
        PL2 = PL1;
        PL1 = PL;
        PL = ((2 * l - 1) * X * PL1 - (l - 1) * PL2) / l;
      }
      DPL = n * (X * PL - PL1) / (X * X - 1.0);
      XP = X;
      X = XP - PL / DPL;
      if (!(fabs(X - XP) > 3.0e-14)) break;
    }
    x[j - 1] = (1.0 - X) / 2.0;
    x[n - j] = (1.0 + X) / 2.0;
    w[j - 1] = w[n - j] = 1.0 / ((1.0 - X * X) * DPL * DPL);
  }
}

// The Gauss table: angles and weights of the 1..9-point sets and their
// Legendre values P_l(mu_i), l = 0..SC_NLEG_MAX (Legendre_M, m = 0).
inline void gauss_table_host(GaussTable& g) {
  g = GaussTable{};
  for (int n = 1; n <= 9; n++) {
    double_gauss_host(n, g.mu[n], g.w[n]);
    for (int i = 0; i < n; i++) {
      double* P = g.P[n][i];
      P[0] = 1.0;
      P[1] = g.mu[n][i];
      for (int j = 1; j < SC_NLEG_MAX; j++) P[j + 1] = ((2 * j + 1) * g.mu[n][i] * P[j] - j * P[j - 1]) / (j + 1);
    }
  }
}

}  // namespace crtm
