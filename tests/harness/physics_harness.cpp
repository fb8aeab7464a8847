// CPU harness around the GPU library's __host__ __device__ physics headers.
// Test infrastructure only: lets the per-profile prep (mapping, predictors,
// partial-derivative table) be checked against the oracle without a GPU.
#include <cstring>
#include <vector>

#include "odps_prep.cuh"

using namespace crtm;

extern "C" {

int hx_nnz(int group) {
  return group == 1 ? PD_NNZ_G1 : (group == 2 ? PD_NNZ_G2 : PD_NNZ_G3);
}

void hx_pattern(int group, int* slot, int* q) {
  std::vector<PdPair> p(hx_nnz(group));
  if (group == 1) pd_pattern<1>(p.data());
  else if (group == 2) pd_pattern<2>(p.data());
  else pd_pattern<3>(p.data());
  for (size_t i = 0; i < p.size(); i++) { slot[i] = p[i].slot; q[i] = p[i].q; }
}

// Layer predictors and partials for an explicit layer state (arrays of MAX_ABS).
void hx_layer(int group, const double* st, double* X, double* D) {
  LayerState L;
  L.sec = st[0]; L.T_ = st[1]; L.Tref = st[2]; L.pdp = st[3]; L.dT = st[1] - st[2];
  L.tz = st[4]; L.tzp = st[5]; L.tz_ref = st[6]; L.tzp_ref = st[7];
  for (int a = 0; a < MAX_ABS; a++) {
    L.A[a] = st[8 + a]; L.Aref[a] = st[14 + a];
    L.gazp[a] = st[20 + a]; L.gatzp[a] = st[26 + a];
    L.gazp_ref[a] = st[32 + a]; L.gatzp_ref[a] = st[38 + a];
  }
  if (group == 1) { layer_predictors<1, double>(L, X); layer_partials<1, double>(L, D); }
  else if (group == 2) { layer_predictors<2, double>(L, X); layer_partials<2, double>(L, D); }
  else { layer_predictors<3, double>(L, X); layer_partials<3, double>(L, D); }
}

// Full per-profile prep.  tables: ref_lev[K+1], ref_t[K], ref_p[K], ref_a/min_a/max_a [Jm][K]
// (the sensor constants are derived here as the library derives them).
int hx_prep(int group, int K, const double* ref_lev, const double* ref_p, const double* ref_t,
            const double* ref_a, const double* min_a, const double* max_a, int h2o_idx,
            int Ku, const double* lev, const double* lay, const double* temp, int n_abs,
            const double* absorber, int abs_stride, const int* idx_map, double zenith,
            double* X, double* D, double* T, double* A, unsigned char* amask, int* band_i0,
            int* band_n, double* band_w, int* k1, int* k2, double* fac, int* uk0, int* uk1,
            double* scal) {
  const int Jm = group_jm(group);
  std::vector<double> lev_lnp(K + 1), lnp(K), pdp(K), z(K + 1);
  for (int k = 0; k <= K; k++) lev_lnp[k] = log(ref_lev[k]);
  for (int k = 0; k < K; k++) lnp[k] = log(ref_p[k]);
  for (int k = 0; k < K; k++)
    pdp[k] = (k == 0) ? ref_lev[0] * (ref_lev[1] - ref_lev[0]) : ref_lev[k + 1] * (ref_lev[k + 1] - ref_lev[k]);
  z[K] = 0.0;
  for (int k = K; k >= 1; k--)
    z[k - 1] = z[k] + CC_H * ref_t[k - 1] * (1.0 + C_TV * ref_a[h2o_idx * K + k - 1]) *
                          log(ref_lev[k] / ref_lev[k - 1]);
  SensorTables S{group, K, group_j(group), Jm, 0, 0, h2o_idx, ref_lev, lev_lnp.data(), lnp.data(),
                 ref_t, ref_a, min_a, max_a, pdp.data(), z.data()};
  ProfileIn P{Ku, n_abs, lev, lay, temp, absorber, abs_stride, idx_map, zenith, 0.0};
  int status = 0;
  ProfileOut<double> O{X, D, T, A, amask, band_i0, band_n, band_w, k1, k2, fac, uk0, uk1, scal, &status};
  if (group == 1) prep_profile<1, double>(S, P, O);
  else if (group == 2) prep_profile<2, double>(S, P, O);
  else prep_profile<3, double>(S, P, O);
  return status;
}
}

extern "C" {
// Layer-averaging bands computed in the reference's sequential order and
// column by column from the binary-search start; returns 1 if they differ.
int hx_layer_avg_compare(const double* px1, int kn1, const double* px2, int kn2, int* max_band) {
  std::vector<int> a0(kn1), an(kn1), b0(kn1), bn(kn1);
  std::vector<double> aw((size_t)kn1 * MAX_BAND), bw((size_t)kn1 * MAX_BAND);
  int sa = layer_avg_weights(px1, kn1, px2, kn2, a0.data(), an.data(), aw.data());
  int sb = 0;
  for (int ki = 0; ki < kn1; ki++) {
    int st = layer_avg_start(px1, kn1, px2, kn2, ki);
    sb |= layer_avg_column(px1, kn1, px2, kn2, ki, st, &b0[ki], &bn[ki], &bw[(size_t)ki * MAX_BAND]);
  }
  int mb = 0;
  for (int ki = 0; ki < kn1; ki++) {
    if (an[ki] > mb) mb = an[ki];
    if (a0[ki] != b0[ki] || an[ki] != bn[ki]) return 1;
    for (int r = 0; r < an[ki]; r++)
      if (aw[(size_t)ki * MAX_BAND + r] != bw[(size_t)ki * MAX_BAND + r]) return 1;
  }
  *max_band = mb;
  return (sa != sb) ? 2 : 0;
}
}
extern "C" int hx_layer_avg_debug(const double* px1, int kn1, const double* px2, int kn2, int* out) {
  std::vector<int> a0(kn1), an(kn1);
  std::vector<double> aw((size_t)kn1 * MAX_BAND);
  layer_avg_weights(px1, kn1, px2, kn2, a0.data(), an.data(), aw.data());
  for (int ki = 0; ki < kn1; ki++) {
    int b0, bn; double bw[MAX_BAND];
    int st = layer_avg_start(px1, kn1, px2, kn2, ki);
    layer_avg_column(px1, kn1, px2, kn2, ki, st, &b0, &bn, bw);
    int prev = ki ? a0[ki-1] : 0;
    if (a0[ki] != b0 || an[ki] != bn) { out[0]=ki; out[1]=a0[ki]; out[2]=an[ki]; out[3]=b0; out[4]=bn; out[5]=st; out[6]=prev; return 1; }
    for (int r = 0; r < bn; r++) if (aw[(size_t)ki*MAX_BAND+r] != bw[r]) { out[0]=ki; out[1]=-r; out[5]=st; out[6]=prev; return 2; }
  }
  return 0;
}

extern "C" double hx_f32_to_f64(float f) { return f32_to_f64_exact(f); }
