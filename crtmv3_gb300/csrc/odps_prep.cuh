// Per-profile preparation of the ODPS path (one profile per call):
//   Map_Input (ODPS_CoordinateMapping.f90:151-319), the integrated predictor
//   variables (ODPS_Predictor.f90:707-759), predictors X, the predictor
//   partial-derivative table D, the user-layer mapping band used by the
//   Map_Input adjoint, and the reference->user level interpolation of the
//   optical-depth path (ODPS_AtmAbsorption.f90:224-254).
// __host__ __device__: the GPU prep kernel and the CPU unit-test harness
// both call prep_profile().
#pragma once

#include "odps_physics.cuh"

namespace crtm {

// Sensor-constant tables (host or device pointers).
struct SensorTables {
  int group, K, J, Jm, L, sensor_type, h2o_idx;
  const double* ref_lev;       // [K+1] hPa
  const double* ref_lev_lnp;   // [K+1]
  const double* ref_lnp;       // [K]   ln of the layer pressures
  const double* ref_t;         // [K]
  const double* ref_a;         // [Jm][K]
  const double* min_a;         // [Jm][K]
  const double* max_a;         // [Jm][K]
  const double* pdp;           // [K]
  const double* zgeo;          // [K+1] geopotential height of the reference levels (Z(K)=0)
  const double* ref_p;         // [K]   layer pressures (the OPTRAN predictors)
  double o_alpha, o_c1, o_c2;  // OPTRAN absorber transform (Alpha, Alpha_C1, Alpha_C2)
};

// One profile of the batch (host or device pointers into the batch arrays).
struct ProfileIn {
  int n_layers, n_abs;
  const double* level_pressure;   // [n_layers+1]
  const double* pressure;         // [n_layers]
  const double* temperature;      // [n_layers]
  const double* absorber;         // [n_abs][abs_stride]
  int abs_stride;
  const int* idx_map;             // [Jm]: user absorber of each ODPS absorber or -1
  double zenith_deg, surface_altitude;
};

// Per-profile prep outputs.  Arrays are per profile; X and D use R.
template <class R>
struct ProfileOut {
  R* X;              // [K][NS]
  R* D;              // [K][NNZ] or nullptr (forward only)
  double* T;         // [K]   mapped temperature
  double* A;         // [Jm][K] mapped (clamped) absorber amounts
  unsigned char* amask;  // [Jm][K] 1 where the Map_Input adjoint passes (A > EPSILON)
  int* band_i0;      // [K]
  int* band_n;       // [K]
  double* band_w;    // [K][MAX_BAND]
  int* ulev_k1;      // [Ku+1] 0-based reference level of the lower bracket
  int* ulev_k2;      // [Ku+1]
  double* ulev_fac;  // [Ku+1] interpolation factor (0 when k1 == k2)
  int* ulay_k0;      // [Ku] first reference layer whose band covers user layer ku
  int* ulay_k1;      // [Ku] last such layer (k0 > k1: none)
  double* scal;      // [4]: sec_surface, u (=cos sensor zenith), unused, unused
  int* status;       // [1]
};

// Map_Input + predictors + partials for one profile.
template <int G, class R>
CRTM_HD void prep_profile(const SensorTables& S, const ProfileIn& P, const ProfileOut<R>& O) {
  const int K = S.K, Jm = S.Jm, Ku = P.n_layers;
  int status = ST_OK;
  if (Ku < 2 || Ku > MAX_LAYERS) {
    O.status[0] = ST_BAD_LAYERS;
    return;
  }
  // user ln p (layers and levels)
  double ulnp[MAX_LAYERS], ulev[MAX_LAYERS + 1];
  for (int k = 0; k < Ku; k++) ulnp[k] = log(P.pressure[k]);
  ulev[0] = (P.level_pressure[0] <= 0.0) ? log(P.level_pressure[1] / 2.0) : log(P.level_pressure[0]);
  for (int k = 1; k <= Ku; k++) ulev[k] = log(P.level_pressure[k]);
  // ODPS surface index and fraction
  int sfc_idx = K;
  double sfc_frac = 0.0;
  const double psfc = P.level_pressure[Ku];
  if (S.ref_lev[K] > psfc) {
    for (int k = K; k >= 0; k--)
      if (S.ref_lev[k] < psfc) {
        sfc_idx = k + 1;
        sfc_frac = (S.ref_lev_lnp[sfc_idx] - ulev[Ku]) / (S.ref_lev_lnp[sfc_idx] - S.ref_lev_lnp[k]);
        break;
      }
  }
  // layer-averaging weights and mapped profiles
  status |= layer_avg_weights(S.ref_lnp, K, ulnp, Ku, O.band_i0, O.band_n, O.band_w);
  for (int k = 0; k < K; k++) {
    const int i0 = O.band_i0[k], n = O.band_n[k];
    const double* w = O.band_w + k * MAX_BAND;
    double acc = 0.0;
    for (int i = 0; i < n; i++) acc += w[i] * P.temperature[i0 + i];
    O.T[k] = acc;
  }
  for (int j = 0; j < Jm; j++) {
    const int map = P.idx_map[j];
    for (int k = 0; k < K; k++) {
      double a;
      unsigned char pass = 0;
      if (map >= 0) {
        const int i0 = O.band_i0[k], n = O.band_n[k];
        const double* w = O.band_w + k * MAX_BAND;
        const double* au = P.absorber + (size_t)map * P.abs_stride;
        a = 0.0;
        for (int i = 0; i < n; i++) a += w[i] * au[i0 + i];
        if (a <= EPS_FP) a = EPS_FP;
        if (a < S.min_a[j * K + k]) a = S.min_a[j * K + k];
        if (a > S.max_a[j * K + k]) a = S.max_a[j * K + k];
        // ODPS_CoordinateMapping.f90:521-523 tests the final (clamped) amount
        pass = (a > EPS_FP) ? 1 : 0;
      } else {
        a = S.ref_a[j * K + k];
      }
      O.A[j * K + k] = a;
      O.amask[j * K + k] = pass;
    }
  }
  // height-dependent secant (reference geopotential heights + offset)
  const Geom g = geometry(P.zenith_deg);
  double zoff;
  if (S.ref_lev[K] >= psfc)
    zoff = -(S.zgeo[sfc_idx] + sfc_frac * (S.zgeo[sfc_idx - 1] - S.zgeo[sfc_idx])) + P.surface_altitude;
  else
    zoff = CC_H * S.ref_t[K - 1] * log(1013.0 / S.ref_lev[K]);
  const double sv = (EARTH_RADIUS + P.surface_altitude) * sin(g.trans_zenith_radian);
  // integrated variables + predictors + partials, layer by layer
  LayerState L;
  double tz_r = 0, tz_s = 0, tzp_r = 0, tzp_s = 0;
  double gazp_r[MAX_ABS], gazp_s[MAX_ABS], gatzp_r[MAX_ABS], gatzp_s[MAX_ABS];
  for (int j = 0; j < MAX_ABS; j++) {
    gazp_r[j] = gazp_s[j] = gatzp_r[j] = gatzp_s[j] = 0.0;
    L.A[j] = L.Aref[j] = 1.0;
    L.gazp[j] = L.gatzp[j] = L.gazp_ref[j] = L.gatzp_ref[j] = 1.0;
  }
  constexpr int NS = Group<G>::NS, NNZ = PdNnz<G>::value;
  for (int k = 0; k < K; k++) {
    const double sa = sv / (EARTH_RADIUS + (S.zgeo[k + 1] + zoff));
    L.sec = 1.0 / sqrt(1.0 - sa * sa);
    L.T_ = O.T[k];
    L.Tref = S.ref_t[k];
    L.dT = O.T[k] - S.ref_t[k];
    const double pdp = S.pdp[k];
    L.pdp = pdp;
    tz_r += S.ref_t[k]; tz_s += L.T_;
    L.tz_ref = tz_r; L.tz = tz_s / tz_r;
    tzp_r += pdp * S.ref_t[k]; tzp_s += pdp * L.T_;
    L.tzp_ref = tzp_r; L.tzp = tzp_s / tzp_r;
    for (int j = 0; j < Jm; j++) {
      const double a = O.A[j * K + k], ar = S.ref_a[j * K + k];
      L.A[j] = a; L.Aref[j] = ar;
      gazp_r[j] += pdp * ar; gazp_s[j] += pdp * a;
      L.gazp_ref[j] = gazp_r[j]; L.gazp[j] = gazp_s[j] / gazp_r[j];
      gatzp_r[j] += pdp * ar * S.ref_t[k]; gatzp_s[j] += pdp * a * L.T_;
      L.gatzp_ref[j] = gatzp_r[j]; L.gatzp[j] = gatzp_s[j] / gatzp_r[j];
    }
    layer_predictors<G, R>(L, O.X + (size_t)k * NS);
    if (O.D) layer_partials<G, R>(L, O.D + (size_t)k * NNZ);
  }
  // reference -> user level interpolation of the optical-depth path
  int k1[MAX_LAYERS + 1], k2[MAX_LAYERS + 1];
  interp_index(S.ref_lev_lnp, K + 1, ulev, Ku + 1, k1, k2);
  for (int i = 0; i <= Ku; i++) {
    const int a = k1[i] - 1, b = k2[i] - 1;
    O.ulev_k1[i] = a;
    O.ulev_k2[i] = b;
    O.ulev_fac[i] = (a == b) ? 0.0
                             : (ulev[i] - S.ref_lev_lnp[a]) / (S.ref_lev_lnp[b] - S.ref_lev_lnp[a]);
  }
  // reverse band: reference layers contributing to each user layer
  for (int ku = 0; ku < Ku; ku++) { O.ulay_k0[ku] = K; O.ulay_k1[ku] = -1; }
  for (int k = 0; k < K; k++)
    for (int i = 0; i < O.band_n[k]; i++) {
      const int ku = O.band_i0[k] + i;
      if (ku < 0 || ku >= Ku) continue;
      if (k < O.ulay_k0[ku]) O.ulay_k0[ku] = k;
      if (k > O.ulay_k1[ku]) O.ulay_k1[ku] = k;
    }
  O.scal[0] = g.sec_trans_zenith;
  O.scal[1] = 1.0 / g.sec_sensor_zenith;   // Common_RTSolution.f90:227
  O.scal[2] = 0.0;
  O.scal[3] = 0.0;
  O.status[0] = status;
}

}  // namespace crtm
