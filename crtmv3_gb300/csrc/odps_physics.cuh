// Per-profile ODPS physics shared by the GPU kernels and the CPU unit-test
// harness: user->ODPS layer mapping, integrated predictor variables,
// predictors and the sparse table of predictor partial derivatives that the
// K-matrix / adjoint kernels contract with the regression coefficients.
//
// Everything here is __host__ __device__ and works on one profile through
// plain pointers, so tests can compile it with g++ and compare it with the
// oracle without a GPU.
#pragma once

#include <math.h>
#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define CRTM_HD __host__ __device__ __forceinline__
#else
#define CRTM_HD inline
#endif

namespace crtm {

constexpr int MAX_LAYERS = 200;     // MAX_N_LAYERS (src/CRTM_Parameters.f90:64)
constexpr int MAX_ABS = 6;          // ODPS absorbers of group 1
constexpr int MAX_BAND = 32;        // user layers per reference layer in the mapping weights
constexpr int MAX_UBAND = 16;       // reference layers per user layer (transposed band)
constexpr double PI_D = 3.141592653589793238462643383279;
constexpr double DEG2RAD = PI_D / 180.0;
constexpr double MAX_TRANS_ZENITH_ANGLE = 63.6122;   // CRTM_Parameters.f90:205
constexpr double EARTH_RADIUS = 6370.0;              // CRTM_Parameters.f90:184
constexpr double MAX_OD = 20.0;                      // ODPS_AtmAbsorption.f90:49
constexpr double EPS_FP = 2.220446049250313e-16;     // EPSILON(1.0_fp)
// Geopotential height factors (ODPS_CoordinateMapping.f90:48-52 with the
// constants of Profile_Utility_Parameters.f90 / Fundamental_Constants.f90)
constexpr double MW_H2O = 18.01528, MW_DRYAIR = 28.9648, R0_GAS = 8.314472, G0_GRAV = 9.80665;
constexpr double C_TV = (1.0 / (MW_H2O / MW_DRYAIR) - 1.0) / 1000.0;
constexpr double CC_H = 0.001 * (R0_GAS / (MW_DRYAIR * 1.0e-3)) / G0_GRAV;

// Status bits written per profile
enum : int {
  ST_OK = 0,
  ST_BAD_LAYERS = 1,      // layer count out of range
  ST_BAND_OVERFLOW = 2,   // mapping band wider than MAX_BAND
  ST_LAYERAVG_FAIL = 4,   // degenerate pressure grid in the layer averaging
  ST_UBAND_OVERFLOW = 8,  // more than MAX_UBAND reference layers map to one user layer
};

// ---------------------------------------------------------------------------
// Predictor group layouts (ODPS_Predictor.f90:85-116).  Slot s = OFF[j] + i
// numbers the predictors of all components of a group densely.
// Variables of the partial-derivative table: q = 0 local temperature,
// q = 1+a local absorber a, q = 1+JM Tz, 2+JM Tzp, 3+JM+a GAzp_a,
// 3+2JM+a GATzp_a.  Integrated-variable partials are stored already divided
// by the reference running sum at that layer.
// ---------------------------------------------------------------------------
template <int G> struct Group;
template <> struct Group<1> {
  static constexpr int J = 8, JM = 6, NS = 89, NV = 3 + 3 * 6;
  static constexpr int NPRED[8] = {7, 18, 7, 11, 11, 14, 10, 11};
  static constexpr int OFF[9] = {0, 7, 25, 32, 43, 54, 68, 78, 89};
};
template <> struct Group<2> {
  static constexpr int J = 5, JM = 3, NS = 50, NV = 3 + 3 * 3;
  static constexpr int NPRED[5] = {7, 15, 7, 11, 10};
  static constexpr int OFF[6] = {0, 7, 22, 29, 40, 50};
};
template <> struct Group<3> {
  static constexpr int J = 2, JM = 1, NS = 21, NV = 3 + 3 * 1;
  static constexpr int NPRED[2] = {7, 14};
  static constexpr int OFF[3] = {0, 7, 21};
};

CRTM_HD int group_ns(int g) { return g == 1 ? 89 : (g == 2 ? 50 : 21); }
CRTM_HD int group_jm(int g) { return g == 1 ? 6 : (g == 2 ? 3 : 1); }
CRTM_HD int group_j(int g) { return g == 1 ? 8 : (g == 2 ? 5 : 2); }

// ---------------------------------------------------------------------------
// Per-layer state handed to the predictor and partial-derivative functions.
// ---------------------------------------------------------------------------
// T is the arithmetic type of the predictor and partial-derivative evaluation.
template <class T>
struct LayerStateT {
  T sec, T_, Tref, pdp;
  T dT;   // T_ - Tref, formed in FP64 before any rounding to T (it cancels)
  T A[MAX_ABS], Aref[MAX_ABS];
  T tz, tzp, tz_ref, tzp_ref;
  T gazp[MAX_ABS], gatzp[MAX_ABS], gazp_ref[MAX_ABS], gatzp_ref[MAX_ABS];
};
using LayerState = LayerStateT<double>;

// Variable index helpers
template <int G> CRTM_HD constexpr int qT() { return 0; }
template <int G> CRTM_HD constexpr int qA(int a) { return 1 + a; }
template <int G> CRTM_HD constexpr int qTz() { return 1 + Group<G>::JM; }
template <int G> CRTM_HD constexpr int qTzp() { return 2 + Group<G>::JM; }
template <int G> CRTM_HD constexpr int qGazp(int a) { return 3 + Group<G>::JM + a; }
template <int G> CRTM_HD constexpr int qGatzp(int a) { return 3 + 2 * Group<G>::JM + a; }

// ---------------------------------------------------------------------------
// Predictors X[s] of one layer (ODPS_Compute_Predictor, ODPS_Predictor.f90:775-1093).
// ---------------------------------------------------------------------------
template <int G, class R, class T = double>
CRTM_HD void layer_predictors(const LayerStateT<T>& L, R* X) {
  const T s = L.sec, t = L.T_ / L.Tref, t2 = t * t, dT = L.dT;
  const T dT2 = dT * fabs(dT);
  const T H = L.A[0] / L.Aref[0], Ha = s * H, Hr = sqrt(Ha), Hs = Ha * Ha;
  const T Hd = H / L.gatzp[0];
  // dry component (slots 0..6)
  X[0] = R(s); X[1] = R(s * t); X[2] = R(s * t2); X[3] = R(t); X[4] = R(s * s); X[5] = R(t2);
  X[6] = R(L.tz);
  if (G == 3) {
    R* w = X + 7;
    const T g = L.gazp[0];
    w[0] = R(Ha / t); w[1] = R(Ha / t * H); w[2] = R(Ha / t2 * H / t2); w[3] = R(Ha / t2);
    w[4] = R(Ha / t2 * H); w[5] = R(Ha / (t2 * t2)); w[6] = R(Ha); w[7] = R(Ha * dT);
    w[8] = R((s * g) * (s * g)); w[9] = R(s * g); w[10] = R(s); w[11] = R(Hs * Ha);
    w[12] = R(Hs * Hs); w[13] = R(Hd);
    return;
  }
  constexpr int oWLO = 7, oWCO = (G == 1 ? 25 : 22), oOZO = (G == 1 ? 32 : 29),
                oCO2 = (G == 1 ? 43 : 40);
  const T O = L.A[1] / L.Aref[1], Oa = s * O, Or = sqrt(Oa), go = L.gazp[1];
  const T C2 = L.A[2] / L.Aref[2], gc = L.gazp[2], tzp = L.tzp, gh = L.gazp[0];
  R* wl = X + oWLO;
  wl[0] = R(Ha); wl[1] = R(Ha * dT); wl[2] = R(Hs); wl[3] = R(Ha * dT2); wl[4] = R(sqrt(Hr));
  wl[5] = R(Hs * Ha); wl[6] = R(Hr); wl[7] = R(Hr * dT); wl[8] = R(Hs * Hs); wl[9] = R(Hd);
  wl[10] = R(Hr * Hd); wl[11] = R((s * gh) * (s * gh)); wl[12] = R(s * gh); wl[13] = R(s);
  wl[14] = R(s * C2);
  R* wc = X + oWCO;
  wc[0] = R(Ha / t); wc[1] = R(Ha / t * H); wc[2] = R(Ha / t2 * H / t2); wc[3] = R(Ha / t2);
  wc[4] = R(Ha / t2 * H); wc[5] = R(Ha / (t2 * t2)); wc[6] = R(Ha);
  R* oz = X + oOZO;
  oz[0] = R(Oa); oz[1] = R(Oa * dT); oz[2] = R(Oa * O * go); oz[3] = R(Oa * Oa); oz[4] = R(Oa * go);
  oz[5] = R(Oa * sqrt(s * go)); oz[6] = R(Or * dT); oz[7] = R(Or); oz[8] = R(Or * O / go);
  oz[9] = R(s * go); oz[10] = R((s * go) * (s * go));
  R* c2 = X + oCO2;
  c2[0] = R(s * t); c2[1] = R(s * t2); c2[2] = R(t); c2[3] = R(t2); c2[4] = R(s); c2[5] = R(s * C2);
  c2[6] = R(s * tzp); c2[7] = R((s * gc) * (s * gc)); c2[8] = R(tzp * tzp * tzp);
  c2[9] = R(s * tzp * sqrt(t));
  if (G == 1) {
    const T N = L.A[3] / L.Aref[3], Na = s * N, Nr = sqrt(Na), gn = L.gazp[3];
    const T Cr = L.A[4] / L.Aref[4], COa = s * Cr, COr = sqrt(COa), gco = L.gazp[4];
    const T COc = COa * Cr / gco;
    const T M = L.A[5] / L.Aref[5], Ma = s * M, Mr = sqrt(Ma), gm = L.gazp[5], Mz = s * gm;
    c2[10] = R(COa);
    wl[15] = R(Ma); wl[16] = R(Ma * Ma * dT); wl[17] = R(COa);
    R* np = X + 54;
    np[0] = R(Na * dT); np[1] = R(Nr); np[2] = R(N * dT); np[3] = R(pow(Na, T(0.25))); np[4] = R(Na);
    np[5] = R(s * gn); np[6] = R(s * L.gatzp[3]); np[7] = R(Na * Na); np[8] = R(L.gatzp[3]);
    np[9] = R(Nr * N / gn); np[10] = R(Ma); np[11] = R(Ma * gm); np[12] = R(COa);
    np[13] = R(COa * s * gco);
    R* cp = X + 68;
    cp[0] = R(COa); cp[1] = R(COa * dT); cp[2] = R(sqrt(COr)); cp[3] = R(COr * dT);
    cp[4] = R(COa * COa); cp[5] = R(COr); cp[6] = R(COa * dT2); cp[7] = R(COc);
    cp[8] = R(COc / COr); cp[9] = R(COc * sqrt(gco));
    R* mp = X + 78;
    mp[0] = R(Ma * dT); mp[1] = R(Mr); mp[2] = R(Ma * Ma); mp[3] = R(Ma); mp[4] = R(M * dT);
    mp[5] = R(Mz); mp[6] = R(Mz * Mz); mp[7] = R(sqrt(Mr)); mp[8] = R(L.gatzp[5]);
    mp[9] = R(s * L.gatzp[5]); mp[10] = R(Mr * M / gm);
  }
}

// ---------------------------------------------------------------------------
// Sparse partial derivatives dX[s]/dv[q] of one layer.
//
// Each group has a fixed list of (slot, variable) pairs; PD_ENTRIES_G<n>
// lists them together with the expression of the partial, so the table of
// pairs (used by the contraction kernels) and the values (written here) are
// generated from one list.  Derived by hand from the predictor formulas
// above; the tests check them against finite differences and, through the
// K-matrix, against the oracle's reverse-mode adjoint.
// ---------------------------------------------------------------------------

// Shared locals available to the entry expressions.
#define CRTM_PD_LOCALS(G)                                                         \
  const T s = L.sec, iT = T(1.0) / L.Tref, t = L.T_ * iT, t2 = t * t;            \
  const T dT = L.dT, adT = fabs(dT), dT2 = dT * adT;                          \
  const T iA0 = T(1.0) / L.Aref[0], H = L.A[0] * iA0, Ha = s * H, Hr = sqrt(Ha); \
  const T gt0 = L.gatzp[0];                                                  \
  const T dt2 = T(2.0) * t * iT; /* d(t^2)/dT */                                \
  (void)dt2; (void)dT2; (void)Hr; (void)gt0;

#define PD_DRY(E)                                       \
  E(1, 0, s * iT)                                       \
  E(2, 0, s * dt2)                                      \
  E(3, 0, iT)                                           \
  E(5, 0, dt2)                                          \
  E(6, QTZ, T(1.0) / L.tz_ref)

// water vapour continuum (group 1/2) or first seven wet predictors (group 3)
#define PD_WCO(E, o)                                                        \
  E(o + 0, QA0, s * iA0 / t)                                                \
  E(o + 0, 0, -Ha / (t * t) * iT)                                           \
  E(o + 1, QA0, T(2.0) * Ha * iA0 / t)                                         \
  E(o + 1, 0, -Ha * H / (t * t) * iT)                                       \
  E(o + 2, QA0, T(2.0) * Ha * iA0 / (t2 * t2))                                 \
  E(o + 2, 0, -T(2.0) * Ha * H / (t2 * t2 * t2) * dt2)                         \
  E(o + 3, QA0, s * iA0 / t2)                                               \
  E(o + 3, 0, -Ha / (t2 * t2) * dt2)                                        \
  E(o + 4, QA0, T(2.0) * Ha * iA0 / t2)                                        \
  E(o + 4, 0, -Ha * H / (t2 * t2) * dt2)                                    \
  E(o + 5, QA0, s * iA0 / (t2 * t2))                                        \
  E(o + 5, 0, -T(2.0) * Ha / (t2 * t2 * t2) * dt2)                             \
  E(o + 6, QA0, s * iA0)

// group 3 wet predictors 8..14
#define PD_WET_TAIL(E)                                                      \
  E(14, QA0, s * iA0 * dT)                                                  \
  E(14, 0, Ha)                                                              \
  E(15, QGAZP0, T(2.0) * s * s * L.gazp[0] / L.gazp_ref[0])                    \
  E(16, QGAZP0, s / L.gazp_ref[0])                                          \
  E(18, QA0, T(3.0) * Ha * Ha * s * iA0)                                       \
  E(19, QA0, T(4.0) * Ha * Ha * Ha * s * iA0)                                  \
  E(20, QA0, iA0 / gt0)                                                     \
  E(20, QGATZP0, -H / (gt0 * gt0) / L.gatzp_ref[0])

// water vapour line, slots 7..21 (+ 22..24 for group 1)
#define PD_WLO(E)                                                           \
  E(7, QA0, s * iA0)                                                        \
  E(8, QA0, s * iA0 * dT)                                                   \
  E(8, 0, Ha)                                                               \
  E(9, QA0, T(2.0) * Ha * s * iA0)                                             \
  E(10, QA0, s * iA0 * dT2)                                                 \
  E(10, 0, Ha * T(2.0) * adT)                                                  \
  E(11, QA0, T(0.25) * sqrt(Hr) / Ha * s * iA0)                                \
  E(12, QA0, T(3.0) * Ha * Ha * s * iA0)                                       \
  E(13, QA0, T(0.5) / Hr * s * iA0)                                            \
  E(14, QA0, T(0.5) / Hr * s * iA0 * dT)                                       \
  E(14, 0, Hr)                                                              \
  E(15, QA0, T(4.0) * Ha * Ha * Ha * s * iA0)                                  \
  E(16, QA0, iA0 / gt0)                                                     \
  E(16, QGATZP0, -H / (gt0 * gt0) / L.gatzp_ref[0])                         \
  E(17, QA0, (T(0.5) / Hr * s * (H / gt0) + Hr / gt0) * iA0)                   \
  E(17, QGATZP0, -Hr * H / (gt0 * gt0) / L.gatzp_ref[0])                    \
  E(18, QGAZP0, T(2.0) * s * s * L.gazp[0] / L.gazp_ref[0])                    \
  E(19, QGAZP0, s / L.gazp_ref[0])                                          \
  E(21, QA2, s / L.Aref[2])

#define PD_WLO_G1(E)                                                        \
  E(22, QA5, s / L.Aref[5])                                                 \
  E(23, QA5, T(2.0) * (s * L.A[5] / L.Aref[5]) * s / L.Aref[5] * dT)           \
  E(23, 0, (s * L.A[5] / L.Aref[5]) * (s * L.A[5] / L.Aref[5]))             \
  E(24, QA4, s / L.Aref[4])

// ozone, offset o
#define PD_OZO(E, o)                                                                     \
  E(o + 0, QA1, s / L.Aref[1])                                                           \
  E(o + 1, QA1, s / L.Aref[1] * dT)                                                      \
  E(o + 1, 0, s * L.A[1] / L.Aref[1])                                                    \
  E(o + 2, QA1, T(2.0) * (s * L.A[1] / L.Aref[1]) * L.gazp[1] / L.Aref[1])                  \
  E(o + 2, QGAZP1, (s * L.A[1] / L.Aref[1]) * (L.A[1] / L.Aref[1]) / L.gazp_ref[1])      \
  E(o + 3, QA1, T(2.0) * (s * L.A[1] / L.Aref[1]) * s / L.Aref[1])                          \
  E(o + 4, QA1, s / L.Aref[1] * L.gazp[1])                                               \
  E(o + 4, QGAZP1, (s * L.A[1] / L.Aref[1]) / L.gazp_ref[1])                             \
  E(o + 5, QA1, s / L.Aref[1] * sqrt(s * L.gazp[1]))                                     \
  E(o + 5, QGAZP1, T(0.5) * (s * L.A[1] / L.Aref[1]) * sqrt(s / L.gazp[1]) / L.gazp_ref[1]) \
  E(o + 6, QA1, T(0.5) / sqrt(s * L.A[1] / L.Aref[1]) * s / L.Aref[1] * dT)                 \
  E(o + 6, 0, sqrt(s * L.A[1] / L.Aref[1]))                                              \
  E(o + 7, QA1, T(0.5) / sqrt(s * L.A[1] / L.Aref[1]) * s / L.Aref[1])                      \
  E(o + 8, QA1,                                                                          \
    (T(0.5) / sqrt(s * L.A[1] / L.Aref[1]) * s * (L.A[1] / L.Aref[1]) +                     \
     sqrt(s * L.A[1] / L.Aref[1])) / L.gazp[1] / L.Aref[1])                              \
  E(o + 8, QGAZP1,                                                                       \
    -sqrt(s * L.A[1] / L.Aref[1]) * (L.A[1] / L.Aref[1]) / (L.gazp[1] * L.gazp[1]) /     \
        L.gazp_ref[1])                                                                   \
  E(o + 9, QGAZP1, s / L.gazp_ref[1])                                                    \
  E(o + 10, QGAZP1, T(2.0) * s * s * L.gazp[1] / L.gazp_ref[1])

// carbon dioxide, offset o (slot o+10 only in group 1)
#define PD_CO2(E, o)                                                                  \
  E(o + 0, 0, s * iT)                                                                 \
  E(o + 1, 0, s * dt2)                                                                \
  E(o + 2, 0, iT)                                                                     \
  E(o + 3, 0, dt2)                                                                    \
  E(o + 5, QA2, s / L.Aref[2])                                                        \
  E(o + 6, QTZP, s / L.tzp_ref)                                                       \
  E(o + 7, QGAZP2, T(2.0) * s * s * L.gazp[2] / L.gazp_ref[2])                           \
  E(o + 8, QTZP, T(3.0) * L.tzp * L.tzp / L.tzp_ref)                                     \
  E(o + 9, QTZP, s * sqrt(t) / L.tzp_ref)                                             \
  E(o + 9, 0, s * L.tzp * T(0.5) / sqrt(t) * iT)

#define PD_CO2_G1(E) E(53, QA4, s / L.Aref[4])

// N2O (group 1, slots 54..67)
#define PD_N2O(E)                                                                        \
  E(54, QA3, s / L.Aref[3] * dT)                                                         \
  E(54, 0, s * L.A[3] / L.Aref[3])                                                       \
  E(55, QA3, T(0.5) / sqrt(s * L.A[3] / L.Aref[3]) * s / L.Aref[3])                         \
  E(56, QA3, dT / L.Aref[3])                                                             \
  E(56, 0, L.A[3] / L.Aref[3])                                                           \
  E(57, QA3, T(0.25) * pow(s * L.A[3] / L.Aref[3], -T(0.75)) * s / L.Aref[3])                  \
  E(58, QA3, s / L.Aref[3])                                                              \
  E(59, QGAZP3, s / L.gazp_ref[3])                                                       \
  E(60, QGATZP3, s / L.gatzp_ref[3])                                                     \
  E(61, QA3, T(2.0) * (s * L.A[3] / L.Aref[3]) * s / L.Aref[3])                             \
  E(62, QGATZP3, T(1.0) / L.gatzp_ref[3])                                                   \
  E(63, QA3,                                                                             \
    (T(0.5) / sqrt(s * L.A[3] / L.Aref[3]) * s * (L.A[3] / L.Aref[3]) +                     \
     sqrt(s * L.A[3] / L.Aref[3])) / L.gazp[3] / L.Aref[3])                              \
  E(63, QGAZP3,                                                                          \
    -sqrt(s * L.A[3] / L.Aref[3]) * (L.A[3] / L.Aref[3]) / (L.gazp[3] * L.gazp[3]) /     \
        L.gazp_ref[3])                                                                   \
  E(64, QA5, s / L.Aref[5])                                                              \
  E(65, QA5, s / L.Aref[5] * L.gazp[5])                                                  \
  E(65, QGAZP5, (s * L.A[5] / L.Aref[5]) / L.gazp_ref[5])                                \
  E(66, QA4, s / L.Aref[4])                                                              \
  E(67, QA4, s / L.Aref[4] * s * L.gazp[4])                                              \
  E(67, QGAZP4, (s * L.A[4] / L.Aref[4]) * s / L.gazp_ref[4])

// CO (group 1, slots 68..77); COc = COa*Cr/gco
#define PD_CO(E)                                                                         \
  E(68, QA4, s / L.Aref[4])                                                              \
  E(69, QA4, s / L.Aref[4] * dT)                                                         \
  E(69, 0, s * L.A[4] / L.Aref[4])                                                       \
  E(70, QA4, T(0.25) * sqrt(sqrt(s * L.A[4] / L.Aref[4])) / (s * L.A[4] / L.Aref[4]) * s /  \
                 L.Aref[4])                                                              \
  E(71, QA4, T(0.5) / sqrt(s * L.A[4] / L.Aref[4]) * s / L.Aref[4] * dT)                    \
  E(71, 0, sqrt(s * L.A[4] / L.Aref[4]))                                                 \
  E(72, QA4, T(2.0) * (s * L.A[4] / L.Aref[4]) * s / L.Aref[4])                             \
  E(73, QA4, T(0.5) / sqrt(s * L.A[4] / L.Aref[4]) * s / L.Aref[4])                         \
  E(74, QA4, s / L.Aref[4] * dT2)                                                        \
  E(74, 0, (s * L.A[4] / L.Aref[4]) * T(2.0) * adT)                                         \
  E(75, QA4, T(2.0) * s * (L.A[4] / L.Aref[4]) / L.gazp[4] / L.Aref[4])                     \
  E(75, QGAZP4, -COc / L.gazp[4] / L.gazp_ref[4])                                        \
  E(76, QA4,                                                                             \
    ((T(2.0) * s * (L.A[4] / L.Aref[4]) / L.gazp[4]) / sqrt(s * L.A[4] / L.Aref[4]) -       \
     COc * T(0.5) * s / (sqrt(s * L.A[4] / L.Aref[4]) * (s * L.A[4] / L.Aref[4]))) /        \
        L.Aref[4])                                                                       \
  E(76, QGAZP4, -COc / sqrt(s * L.A[4] / L.Aref[4]) / L.gazp[4] / L.gazp_ref[4])         \
  E(77, QA4, T(2.0) * s * (L.A[4] / L.Aref[4]) / L.gazp[4] * sqrt(L.gazp[4]) / L.Aref[4])   \
  E(77, QGAZP4, -T(0.5) * COc / sqrt(L.gazp[4]) / L.gazp_ref[4])

// CH4 (group 1, slots 78..88)
#define PD_CH4(E)                                                                        \
  E(78, QA5, s / L.Aref[5] * dT)                                                         \
  E(78, 0, s * L.A[5] / L.Aref[5])                                                       \
  E(79, QA5, T(0.5) / sqrt(s * L.A[5] / L.Aref[5]) * s / L.Aref[5])                         \
  E(80, QA5, T(2.0) * (s * L.A[5] / L.Aref[5]) * s / L.Aref[5])                             \
  E(81, QA5, s / L.Aref[5])                                                              \
  E(82, QA5, dT / L.Aref[5])                                                             \
  E(82, 0, L.A[5] / L.Aref[5])                                                           \
  E(83, QGAZP5, s / L.gazp_ref[5])                                                       \
  E(84, QGAZP5, T(2.0) * s * L.gazp[5] * s / L.gazp_ref[5])                                 \
  E(85, QA5, T(0.25) * sqrt(sqrt(s * L.A[5] / L.Aref[5])) / (s * L.A[5] / L.Aref[5]) * s /  \
                 L.Aref[5])                                                              \
  E(86, QGATZP5, T(1.0) / L.gatzp_ref[5])                                                   \
  E(87, QGATZP5, s / L.gatzp_ref[5])                                                     \
  E(88, QA5,                                                                             \
    (T(0.5) / sqrt(s * L.A[5] / L.Aref[5]) * s * (L.A[5] / L.Aref[5]) +                     \
     sqrt(s * L.A[5] / L.Aref[5])) / L.gazp[5] / L.Aref[5])                              \
  E(88, QGAZP5,                                                                          \
    -sqrt(s * L.A[5] / L.Aref[5]) * (L.A[5] / L.Aref[5]) / (L.gazp[5] * L.gazp[5]) /     \
        L.gazp_ref[5])

// Full entry lists per group
#define PD_ENTRIES_G1(E) \
  PD_DRY(E) PD_WLO(E) PD_WLO_G1(E) PD_WCO(E, 25) PD_OZO(E, 32) PD_CO2(E, 43) PD_CO2_G1(E) \
  PD_N2O(E) PD_CO(E) PD_CH4(E)
#define PD_ENTRIES_G2(E) PD_DRY(E) PD_WLO(E) PD_WCO(E, 22) PD_OZO(E, 29) PD_CO2(E, 40)
#define PD_ENTRIES_G3(E) PD_DRY(E) PD_WCO(E, 7) PD_WET_TAIL(E)

// variable codes used in the entry lists
#define CRTM_PD_QCODES(G)                                                    \
  constexpr int QA0 = qA<G>(0), QA1 = qA<G>(1), QA2 = qA<G>(2), QA3 = qA<G>(3), \
                QA4 = qA<G>(4), QA5 = qA<G>(5);                              \
  constexpr int QTZ = qTz<G>(), QTZP = qTzp<G>();                            \
  constexpr int QGAZP0 = qGazp<G>(0), QGAZP1 = qGazp<G>(1), QGAZP2 = qGazp<G>(2), \
                QGAZP3 = qGazp<G>(3), QGAZP4 = qGazp<G>(4), QGAZP5 = qGazp<G>(5); \
  constexpr int QGATZP0 = qGatzp<G>(0), QGATZP3 = qGatzp<G>(3), QGATZP5 = qGatzp<G>(5); \
  (void)QA0; (void)QA1; (void)QA2; (void)QA3; (void)QA4; (void)QA5; (void)QTZ; (void)QTZP; \
  (void)QGAZP0; (void)QGAZP1; (void)QGAZP2; (void)QGAZP3; (void)QGAZP4; (void)QGAZP5; \
  (void)QGATZP0; (void)QGATZP3; (void)QGATZP5;

#define CRTM_PD_COUNT(slot, q, expr) +1
constexpr int PD_NNZ_G1 = 0 PD_ENTRIES_G1(CRTM_PD_COUNT);
constexpr int PD_NNZ_G2 = 0 PD_ENTRIES_G2(CRTM_PD_COUNT);
constexpr int PD_NNZ_G3 = 0 PD_ENTRIES_G3(CRTM_PD_COUNT);

template <int G> struct PdNnz;
template <> struct PdNnz<1> { static constexpr int value = PD_NNZ_G1; };
template <> struct PdNnz<2> { static constexpr int value = PD_NNZ_G2; };
template <> struct PdNnz<3> { static constexpr int value = PD_NNZ_G3; };

// Value writer: D[e] for the e-th entry, in list order.
#define CRTM_PD_VALUE(slot, q, expr) D[e++] = R(expr);

template <int G, class R, class T = double>
CRTM_HD void layer_partials(const LayerStateT<T>& L, R* D) {
  CRTM_PD_LOCALS(G)
  CRTM_PD_QCODES(G)
  int e = 0;
  if (G == 1) {
    const T COc = (s * L.A[4] / L.Aref[4]) * (L.A[4] / L.Aref[4]) / L.gazp[4];
    (void)COc;
    PD_ENTRIES_G1(CRTM_PD_VALUE)
  } else if (G == 2) {
    PD_ENTRIES_G2(CRTM_PD_VALUE)
  } else {
    PD_ENTRIES_G3(CRTM_PD_VALUE)
  }
}

// (slot, variable) pairs of the entries, in list order.
#define CRTM_PD_PAIR(slot, q, expr) {slot, q},
struct PdPair { int slot, q; };

// Host-usable pattern tables (built from the lists with G's variable codes).
template <int G>
inline void pd_pattern(PdPair* out) {
  CRTM_PD_QCODES(G)
  const PdPair tab1[] = {PD_ENTRIES_G1(CRTM_PD_PAIR)};
  const PdPair tab2[] = {PD_ENTRIES_G2(CRTM_PD_PAIR)};
  const PdPair tab3[] = {PD_ENTRIES_G3(CRTM_PD_PAIR)};
  const PdPair* t = G == 1 ? tab1 : (G == 2 ? tab2 : tab3);
  const int n = G == 1 ? PD_NNZ_G1 : (G == 2 ? PD_NNZ_G2 : PD_NNZ_G3);
  for (int i = 0; i < n; i++) out[i] = t[i];
}

// ---------------------------------------------------------------------------
// Geometry (CRTM_GeometryInfo.f90:100-143)
// ---------------------------------------------------------------------------
struct Geom {
  double cos_sensor_zenith, sec_sensor_zenith, trans_zenith_radian, sec_trans_zenith;
};
CRTM_HD Geom geometry(double zenith_deg) {
  Geom g;
  const double zr = DEG2RAD * zenith_deg;
  g.cos_sensor_zenith = cos(zr);
  g.sec_sensor_zenith = 1.0 / g.cos_sensor_zenith;
  if (zenith_deg > MAX_TRANS_ZENITH_ANGLE) {
    g.trans_zenith_radian = DEG2RAD * MAX_TRANS_ZENITH_ANGLE;
    g.sec_trans_zenith = 1.0 / cos(g.trans_zenith_radian);
  } else {
    g.trans_zenith_radian = zr;
    g.sec_trans_zenith = g.sec_sensor_zenith;
  }
  return g;
}

// ---------------------------------------------------------------------------
// Layer-averaging weights of user layers for one reference layer ki
// (LayerAvg, ODPS_CoordinateMapping.f90:1108-1320).  px1: reference layer
// ln p (kn1 of them), px2: user layer ln p (kn2).  Writes the band start i0,
// width nw and normalised weights w[0..nw).  `istart` is where the search
// over user layers begins: the reference passes the previous column's first
// weight index; any index not after the column's first contributing user
// layer gives the same weights (user layers below it cannot contribute), so
// columns can also be computed independently from a binary-search bound
// (layer_avg_start).  Returns status bits.
// ---------------------------------------------------------------------------
CRTM_HD void layer_avg_edges(const double* px1, int kn1, const double* px2, int kn2, int ki,
                             double& z1, double& z2, double& z3, int& iskip) {
  z2 = px1[ki];
  z1 = (ki == 0) ? 2.0 * z2 - px1[ki + 1] : px1[ki - 1];
  z3 = (ki == kn1 - 1) ? 2.0 * z2 - z1 : px1[ki + 1];
  if (z3 > px2[kn2 - 1]) z3 = px2[kn2 - 1];
  iskip = 0;
  if (z2 >= px2[kn2 - 1]) { z3 = px2[kn2 - 1]; z2 = px2[kn2 - 1]; iskip = 1; }
}

// First user layer j (0-based) with px2[j+1] > min(z1,z2,z3): no user layer
// before it contributes to column ki.
CRTM_HD int layer_avg_start(const double* px1, int kn1, const double* px2, int kn2, int ki) {
  double z1, z2, z3;
  int iskip;
  layer_avg_edges(px1, kn1, px2, kn2, ki, z1, z2, z3, iskip);
  double zmin = z1 < z2 ? z1 : z2;
  if (z3 < zmin) zmin = z3;
  int lo = 0, hi = kn2 - 1;  // answer in [0, kn2-1]
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (px2[mid + 1] > zmin) hi = mid; else lo = mid + 1;
  }
  return lo;
}

CRTM_HD int layer_avg_column(const double* px1, int kn1, const double* px2, int kn2, int ki,
                             int istart, int* i0, int* nw, double* w) {
  const double SMALLDIFF = 1.0e-20;
  double z1, z2, z3;
  int iskip;
  layer_avg_edges(px1, kn1, px2, kn2, ki, z1, z2, z3, iskip);
  double pz[MAX_BAND + 2];
  for (int i = 0; i < MAX_BAND + 2; i++) pz[i] = 0.0;
  int ic = 0, jend = kn2 - 1, j, bad = 0;
  for (j = istart; j < kn2 - 1; j++) {
    if (px2[j] > z3) { jend = j; break; }
    for (int pass = 0; pass < 2; pass++) {
      const double za = pass == 0 ? z1 : z3;  // the edge used by this half-layer
      const bool hit = pass == 0 ? (px2[j] <= z2 && px2[j + 1] > z1)
                                 : (px2[j] < z3 && px2[j + 1] >= z2 && iskip == 0);
      if (!hit) continue;
      const double zb = pass == 0 ? z3 : z1;  // the opposite edge
      int itop = 0, ibot = 0;
      double y1, y2;
      if (za < zb) {
        y1 = za; if (px2[j] > za) { y1 = px2[j]; itop = 1; }
        y2 = z2; if (px2[j + 1] < z2) { y2 = px2[j + 1]; ibot = 1; }
      } else {
        y1 = z2; if (px2[j] > z2) { y1 = px2[j]; itop = 1; }
        y2 = za; if (px2[j + 1] < za) { y2 = px2[j + 1]; ibot = 1; }
      }
      const double dy = y2 - y1, dz = za - z2;
      if (fabs(dz) < SMALLDIFF) { bad = 1; break; }
      const double dzd = 1.0 / dz;
      double zw1 = (za - y1) * dzd * dy, zw2 = (za - y2) * dzd * dy;
      const double dx = px2[j + 1] - px2[j];
      if (fabs(dx) < SMALLDIFF) { bad = 1; break; }
      const double d = (px2[j + 1] - z2) * (1.0 / dx);
      if (za < zb && ibot == 0) { zw1 = zw1 + zw2 * d; zw2 = zw2 * (1.0 - d); }
      else if (za > zb && itop == 0) { zw2 = zw2 + zw1 * (1.0 - d); zw1 = zw1 * d; }
      const int r = j - istart;
      if (r + 1 >= MAX_BAND + 2) { bad = 2; break; }
      pz[r] += zw1; pz[r + 1] += zw2; ic = 1;
    }
    if (bad) break;
  }
  if (bad) {
    *i0 = istart < kn2 ? istart : kn2 - 1; *nw = 1; w[0] = 1.0;
    return (bad == 2) ? ST_BAND_OVERFLOW : ST_LAYERAVG_FAIL;
  }
  if (j >= kn2 - 1) jend = kn2 - 1;
  if (ic == 0) {
    const int r = jend - istart;
    if (r < 0 || r >= MAX_BAND + 2) { *i0 = jend; *nw = 1; w[0] = 1.0; return ST_OK; }
    pz[r] = 1.0;
  }
  int f = -1;
  for (int r = 0; r < MAX_BAND + 2 && istart + r < kn2; r++)
    if (pz[r] != 0.0) { f = r; break; }
  if (f < 0) f = 0;
  int n = 0;
  for (int r = f; r < MAX_BAND + 2 && istart + r < kn2; r++) {
    if (pz[r] == 0.0) break;
    n++;
  }
  int status = ST_OK;
  if (n > MAX_BAND) { status = ST_BAND_OVERFLOW; n = MAX_BAND; }
  double zsum = 0.0;
  for (int r = f; r < f + n; r++) zsum += pz[r];
  *i0 = istart + f;
  *nw = n;
  for (int r = 0; r < n; r++) w[r] = pz[f + r] / zsum;
  return status;
}

// All columns in the reference's order.  Each search starts at the later of
// the previous column's first weight index (the reference's start) and the
// column's binary-search bound, which keeps the band inside the fixed window.
CRTM_HD int layer_avg_weights(const double* px1, int kn1, const double* px2, int kn2, int* i0,
                              int* nw, double* w) {
  int status = ST_OK, istart = 0;
  for (int ki = 0; ki < kn1; ki++) {
    const int lb = layer_avg_start(px1, kn1, px2, kn2, ki);
    status |= layer_avg_column(px1, kn1, px2, kn2, ki, istart > lb ? istart : lb, i0 + ki, nw + ki,
                               w + ki * MAX_BAND);
    istart = i0[ki];
  }
  return status;
}

// Compute_Interp_Index (ODPS_CoordinateMapping.f90:963-1012): for user level
// iu, the 1-based reference level pair (k1[iu], k2[iu]).
CRTM_HD void interp_index(const double* x, int nx, const double* u, int nu, int* k1o, int* k2o) {
  int k1 = nu + 1, k2 = 0;
  for (int iu = 1; iu <= nu; iu++) {
    if (u[iu - 1] < x[0]) { k1o[iu - 1] = 1; k2o[iu - 1] = 1; }
    else { k1 = iu; break; }
  }
  for (int iu = nu; iu >= k1; iu--) {
    if (u[iu - 1] > x[nx - 1]) { k1o[iu - 1] = nx; k2o[iu - 1] = nx; }
    else { k2 = iu; break; }
  }
  int j = 1;
  for (int iu = k1; iu <= k2; iu++)
    for (int ix = j; ix <= nx - 1; ix++)
      if (u[iu - 1] >= x[ix - 1] && u[iu - 1] <= x[ix]) {
        k1o[iu - 1] = ix; k2o[iu - 1] = ix + 1; j = ix;
        break;
      }
}

// Planck radiance and derivatives (CRTM_Planck_Functions.f90:116-136,358-385,470-492,697-723)
template <class R>
CRTM_HD R planck_radiance(R c1, R c2, R b1, R b2, R T) {
  R te = b1 + b2 * T;
  return c1 / (exp(c2 / te) - R(1));
}
template <class R>
CRTM_HD R planck_radiance_dT(R c1, R c2, R b1, R b2, R T) {
  R te = b1 + b2 * T;
  R e = exp(c2 / te);
  R d = te * (e - R(1));
  return c1 * c2 * e * b2 / (d * d);
}
// Exact float -> double conversion with integer operations.  On GB300 the
// hardware conversion runs on the narrow FP64 pipe; kernels that store FP64
// results of FP32 arithmetic (one conversion per output element) use this
// instead.  Handles zeros, subnormals, infinities and NaNs.
CRTM_HD double f32_to_f64_exact(float f) {
  uint32_t u;
  memcpy(&u, &f, 4);
  const uint32_t sign = u & 0x80000000u;
  uint32_t e = (u >> 23) & 0xffu, m = u & 0x7fffffu;
  uint32_t hi;
  if (e == 0xffu) {
    hi = sign | 0x7ff00000u | (m >> 3);
  } else if (e == 0) {
    if (m == 0) {
      hi = sign;
    } else {   // subnormal float: normalise (the double is normal)
      int sh = 0;
      while (!(m & 0x800000u)) { m <<= 1; sh++; }
      m &= 0x7fffffu;
      hi = sign | ((uint32_t)(1 - sh + 896) << 20) | (m >> 3);
    }
  } else {
    hi = sign | ((e + 896u) << 20) | (m >> 3);
  }
  const uint64_t bits = ((uint64_t)hi << 32) | ((uint64_t)(m & 7u) << 29);
  double d;
  memcpy(&d, &bits, 8);
  return d;
}
CRTM_HD double to_f64(float f) { return f32_to_f64_exact(f); }
CRTM_HD double to_f64(double d) { return d; }

CRTM_HD double planck_temperature(double c1, double c2, double b1, double b2, double R) {
  double te = c2 / log(c1 / R + 1.0);
  return (te - b1) / b2;
}
CRTM_HD double planck_temperature_dR(double c1, double c2, double b1, double b2, double R) {
  double arg = c1 / R + 1.0;
  double d = R * log(arg);
  return c1 * c2 / (b2 * arg * d * d);
}
// Both of the above from one logarithm (CRTM_Planck_Temperature and its adjoint,
// CRTM_Planck_Functions.f90:470-492,697-723).
CRTM_HD void planck_temperature_with_dR(double c1, double c2, double b1, double b2, double R,
                                        double* T, double* dTdR) {
  const double arg = c1 / R + 1.0;
  const double lg = log(arg);
  *T = (c2 / lg - b1) / b2;
  const double d = R * lg;
  *dTdR = c1 * c2 / (b2 * arg * d * d);
}

}  // namespace crtm
