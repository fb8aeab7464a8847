// CPU harness around the GPU library's cloud/ADA physics header (test
// infrastructure only): one ADA layer and one cloudy (profile, channel).
#include <algorithm>
#include <cmath>
#include <vector>

#include "scatter_adjoint.cuh"

using namespace crtm;

namespace {
GaussTable make_gauss() {
  GaussTable g;
  gauss_table_host(g);
  return g;
}
}  // namespace

extern "C" {


int sx_ada_layer(int nS, int nZ, double w, double tau, const double* mu, const double* wt,
                 const double* ff, const double* bb, double B, double* T, double* R, double* src) {
  Mat<SC_NZ_MAX, double> F, Bm, Tm, Rm;
  for (int i = 0; i < nZ; i++)
    for (int j = 0; j < nZ; j++) { F.a[i][j] = ff[i * nZ + j]; Bm.a[i][j] = bb[i * nZ + j]; }
  if (!ada_layer<SC_NZ_MAX, double>(nS, nZ, w, tau, mu, wt, F, Bm, B, Tm, Rm, src)) return 1;
  for (int i = 0; i < nZ; i++)
    for (int j = 0; j < nZ; j++) { T[i * nZ + j] = Tm.a[i][j]; R[i * nZ + j] = Rm.a[i][j]; }
  return 0;
}

// One ADA layer in double-float (the mixed form's layer solver).
int sx_ada_layer_dd(int nS, int nZ, double w, double tau, const double* mu, const double* wt,
                    const double* ff, const double* bb, double B, double* T, double* R, double* src) {
  Mat<SC_NZ_MAX, DD> F, Bm, Tm, Rm;
  DD mud[SC_NZ_MAX], wtd[SC_NZ_MAX], s[SC_NZ_MAX];
  for (int i = 0; i < nZ; i++) {
    mud[i] = DD(mu[i]);
    wtd[i] = DD(wt[i]);
    for (int j = 0; j < nZ; j++) { F.a[i][j] = DD(ff[i * nZ + j]); Bm.a[i][j] = DD(bb[i * nZ + j]); }
  }
  if (!ada_layer<SC_NZ_MAX, DD>(nS, nZ, DD(w), DD(tau), mud, wtd, F, Bm, DD(B), Tm, Rm, s)) return 1;
  for (int i = 0; i < nZ; i++) {
    src[i] = (double)s[i];
    for (int j = 0; j < nZ; j++) { T[i * nZ + j] = (double)Tm.a[i][j]; R[i * nZ + j] = (double)Rm.a[i][j]; }
  }
  return 0;
}

// Double-float arithmetic checks: a op b for op = 0 +, 1 -, 2 *, 3 /, 4 sqrt(a), 5 exp(a).
double sx_dd_op(int op, double a, double b) {
  const DD x(a), y(b);
  switch (op) {
    case 0: return (double)(x + y);
    case 1: return (double)(x - y);
    case 2: return (double)(x * y);
    case 3: return (double)(x / y);
    case 4: return (double)sqrt(x);
    default: return (double)exp(x);
  }
}

// dims: nfm nrm nt nd nfi nri nleg; arrays in the file's Fortran order.
int sx_cloudy_radiance(const int* dims, const double* f_mw, const double* r_mw, const double* t,
                       const double* f_ir, const double* r_ir, const double* ke_l, const double* w_l,
                       const double* pc_l, const double* ke_s, const double* w_s, const double* pc_s,
                       const double* ke_ir, const double* w_ir, const double* pc_ir, int Ku, int n_clouds,
                       int nleg, int microwave, double freq, double mu_sensor, double emissivity,
                       double planck_surface, double cosmic, const double* planck, const double* temp,
                       const int* cloud_type, const double* wc, const double* reff, int cstride,
                       const double* od, int soi, int n_aer, const int* aer_type, const double* conc,
                       const double* aer_reff, const double* aer_var, const double* rh_layers,
                       const int* adims, const int* atypes, const double* afreq, const double* areff,
                       const double* arsig, const double* arh, const double* ake, const double* aw,
                       const double* apc, double wavenumber, double* radiance) {
  // adims: nw nrh nr ns nt nleg scheme n_rh_axis
  AerosolLut A{};
  if (n_aer > 0) {
    A.nw = adims[0]; A.nrh = adims[1]; A.nr = adims[2]; A.ns = adims[3]; A.nt = adims[4]; A.nleg = adims[5];
    A.scheme = adims[6]; A.nrh_axis = adims[7];
    A.type_id = atypes; A.freq = afreq; A.reff = areff; A.rsig = arsig; A.rh = arh; A.ke = ake; A.w = aw;
    A.pc = apc;
  }
  CloudLut L{dims[0], dims[1], dims[2], dims[3], dims[4], dims[5], dims[6], f_mw, r_mw, t, f_ir, r_ir,
             ke_l, w_l, pc_l, ke_s, w_s, pc_s, ke_ir, w_ir, pc_ir};
  static const GaussTable gt = make_gauss();
  CloudyColumn c{};
  c.Ku = Ku; c.n_clouds = n_clouds; c.nleg = nleg; c.microwave = microwave != 0; c.freq = freq;
  c.mu_sensor = mu_sensor; c.emissivity = emissivity; c.planck_surface = planck_surface; c.cosmic = cosmic;
  c.c1 = planck[0]; c.c2 = planck[1]; c.b1 = planck[2]; c.b2 = planck[3];
  c.temperature = temp; c.cloud_type = cloud_type; c.wc = wc; c.reff = reff; c.cstride = (size_t)cstride;
  c.n_aerosols = n_aer; c.wavenumber = wavenumber; c.aerosol_type = aer_type; c.conc = conc;
  c.aer_reff = aer_reff; c.aer_var = aer_var; c.rh = rh_layers; c.alut = &A;
  c.soi = soi != 0;
  if (soi >= 2 && soi <= 5) {   // layered ADA as the GPU kernels run it (records with NZ = 10);
    c.soi = false;               // layer optics in FP64 (2), double-float (3), FP32 (4; 5: FP32 records)
    constexpr int NZ = SC_NZ_MAX, NE = 2 + 2 * NZ * NZ + NZ;
    StreamSet<NZ, double> S;
    if (int rc = stream_set<NZ, double>(nleg, mu_sensor, n_clouds > 0 ? L.nleg : -1, gt, S)) return rc;
    std::vector<double> rec((size_t)Ku * NE);
    for (int k = 0; k < Ku; k++) {
      Mat<NZ, double> Tm, Rm;
      double srcv[NZ], o;
      int kind;
      if (soi == 3)
        kind = layer_optics<NZ, double, DD>(c, L, S, k, DD(od[k]), DD(temp[k]), &o, Tm, Rm, srcv);
      else if (soi == 4)
        kind = layer_optics<NZ, double, float>(c, L, S, k, float(od[k]), float(temp[k]), &o, Tm, Rm, srcv);
      else if (soi == 5) {   // FP32 layer solver and FP32 records (the mixed forward)
        Mat<NZ, float> Tf, Rf;
        float sf[NZ], of;
        kind = layer_optics<NZ, float, float>(c, L, S, k, float(od[k]), float(temp[k]), &of, Tf, Rf, sf);
        o = of;
        for (int i = 0; i < NZ; i++) {
          srcv[i] = sf[i];
          for (int j = 0; j < NZ; j++) { Tm.a[i][j] = Tf.a[i][j]; Rm.a[i][j] = Rf.a[i][j]; }
        }
      }
      else
        kind = layer_optics<NZ, double>(c, L, S, k, od[k], temp[k], &o, Tm, Rm, srcv);
      double* r = &rec[(size_t)k * NE];
      r[0] = kind;
      r[1] = o;
      if (kind != 1) continue;
      for (int i = 0; i < S.nZ; i++) {
        for (int j = 0; j < S.nZ; j++) { r[2 + i * NZ + j] = Tm.a[i][j]; r[2 + NZ * NZ + i * NZ + j] = Rm.a[i][j]; }
        r[2 + 2 * NZ * NZ + i] = srcv[i];
      }
    }
    AddingState<NZ> A;
    adding_init<NZ>(A, S.nZ, emissivity, planck_surface);
    for (int k = Ku - 1; k >= 0; k--) {
      const double* r = &rec[(size_t)k * NE];
      const int kind = (int)r[0];
      if (kind < 0) return -kind;
      if (kind == 1) {
        Mat<NZ, double> Tm, Rm;
        double srcv[NZ];
        for (int i = 0; i < S.nZ; i++) {
          for (int j = 0; j < S.nZ; j++) { Tm.a[i][j] = r[2 + i * NZ + j]; Rm.a[i][j] = r[2 + NZ * NZ + i * NZ + j]; }
          srcv[i] = r[2 + 2 * NZ * NZ + i];
        }
        if (!adding_scatter<NZ>(A, S.nZ, Tm, Rm, srcv)) return 6;
      } else {
        adding_clear<NZ>(A, S.nZ, S.mu, r[1], c.c1 / (exp(c.c2 / (c.b1 + c.b2 * temp[k])) - 1.0));
      }
    }
    *radiance = adding_toa<NZ>(A, S.nZ, S.isat, cosmic);
    return 0;
  }
  if (!c.soi) return cloudy_radiance<SC_NZ_MAX>(c, L, gt, [&](int k) { return od[k]; }, radiance);
  // SOI: every layer's record first, then the orders of interaction
  constexpr int NZ = SC_NZ_MAX;
  StreamSet<NZ, double> S;
  if (int rc = stream_set<NZ, double>(nleg, mu_sensor, n_clouds > 0 ? L.nleg : -1, gt, S)) return rc;
  std::vector<int> kind(Ku);
  std::vector<double> ods(Ku);
  std::vector<Mat<NZ, double>> T(Ku), R(Ku);
  std::vector<double> src((size_t)Ku * NZ);
  for (int k = 0; k < Ku; k++) {
    kind[k] = layer_optics<NZ, double>(c, L, S, k, od[k], temp[k], &ods[k], T[k], R[k], &src[(size_t)k * NZ]);
    if (kind[k] < 0) return -kind[k];
  }
  auto lod = [&](int k, int* kd, double* o, double* B) {
    *kd = kind[k];
    *o = ods[k];
    *B = c.c1 / (exp(c.c2 / (c.b1 + c.b2 * temp[k])) - 1.0);
  };
  auto lsrc = [&](int k, double* sv) { for (int i = 0; i < NZ; i++) sv[i] = src[(size_t)k * NZ + i]; };
  auto ltr = [&](int k, Mat<NZ, double>& Tm, Mat<NZ, double>& Rm) { Tm = T[k]; Rm = R[k]; };
  std::vector<double> f((size_t)4 * (Ku + 1) * NZ);
  auto fld = [&](int b, int fi, int k, int i) -> double& { return f[((size_t)(2 * fi + b) * (Ku + 1) + k) * NZ + i]; };
  return soi_solve<NZ>(S.nZ, Ku, S.isat, S.mu, emissivity, planck_surface, cosmic, lod, lsrc, ltr, fld, radiance);
}

int sx_stream_rule(double max_reff, double wavenumber) { return stream_rule_nleg(max_reff, wavenumber); }
double sx_total_cloud_cover(int Ku, int n_clouds, const double* cf, const double* wc, int cstride, int overlap) {
  return total_cloud_cover(Ku, n_clouds, cf, wc, (size_t)cstride, overlap);
}
void sx_cloud_cover_derivatives(int Ku, int n_clouds, const double* cf, const double* wc, int cstride, int overlap,
                                double tcc, double* dcf, double* dwc) {
  cloud_cover_derivatives(Ku, n_clouds, cf, wc, (size_t)cstride, overlap, tcc, dcf, dwc);
}
}


// One layer's record (od, T, R, src: 1 + 2 nZ^2 + nZ values) for gas optical
// depth gas and temperature tk, with its derivatives d/dgas and d/dtk from the
// derivative-number evaluation.  Same LUT and column arguments as above.
extern "C" int sx_layer_record(const int* dims, const double* f_mw, const double* r_mw, const double* t,
                               const double* f_ir, const double* r_ir, const double* ke_l, const double* w_l,
                               const double* pc_l, const double* ke_s, const double* w_s, const double* pc_s,
                               const double* ke_ir, const double* w_ir, const double* pc_ir, int n_clouds,
                               int nleg, int microwave, double freq, double mu_sensor, const double* planck,
                               const int* cloud_type, const double* wc, const double* reff, int cstride, int k,
                               double gas, double tk, double* val, double* dgas, double* dtk, int* nz_out) {
  CloudLut L{dims[0], dims[1], dims[2], dims[3], dims[4], dims[5], dims[6], f_mw, r_mw, t, f_ir, r_ir,
             ke_l, w_l, pc_l, ke_s, w_s, pc_s, ke_ir, w_ir, pc_ir};
  static const GaussTable gt = make_gauss();
  CloudyColumn c{};
  c.Ku = k + 1; c.n_clouds = n_clouds; c.nleg = nleg; c.microwave = microwave != 0; c.freq = freq;
  c.mu_sensor = mu_sensor;
  c.c1 = planck[0]; c.c2 = planck[1]; c.b1 = planck[2]; c.b2 = planck[3];
  c.cloud_type = cloud_type; c.wc = wc; c.reff = reff; c.cstride = (size_t)cstride;
  constexpr int NZ = SC_NZ_MAX;
  StreamSet<NZ, double> S;
  if (int rc = stream_set<NZ, double>(nleg, mu_sensor, L.nleg, gt, S)) return -100 - rc;
  using D = Dual<2>;
  D g(gas), tt(tk);
  g.d[0] = 1.0;
  tt.d[1] = 1.0;
  Mat<NZ, D> Tm, Rm;
  D src[NZ], od;
  const int kind = layer_optics<NZ, D, D>(c, L, S, k, g, tt, &od, Tm, Rm, src);
  const int nZ = S.nZ;
  *nz_out = nZ;
  auto put = [&](const D& x, int i) { val[i] = x.v; dgas[i] = x.d[0]; dtk[i] = x.d[1]; };
  put(od, 0);
  for (int i = 0; i < nZ; i++)
    for (int j = 0; j < nZ; j++) { put(Tm.a[i][j], 1 + i * nZ + j); put(Rm.a[i][j], 1 + nZ * nZ + i * nZ + j); }
  for (int i = 0; i < nZ; i++) put(src[i], 1 + 2 * nZ * nZ + i);
  return kind;
}


// K-matrix of one cloudy (profile, channel) through ADA for a unit radiance
// seed: radiance, dR/d(gas OD_k), dR/dT_k, dR/de and dR/dB_surface.
extern "C" int sx_cloudy_kmatrix(const int* dims, const double* f_mw, const double* r_mw, const double* t,
                                 const double* f_ir, const double* r_ir, const double* ke_l, const double* w_l,
                                 const double* pc_l, const double* ke_s, const double* w_s, const double* pc_s,
                                 const double* ke_ir, const double* w_ir, const double* pc_ir, int Ku,
                                 int n_clouds, int nleg, int microwave, double freq, double mu_sensor,
                                 double emissivity, double planck_surface, double cosmic, const double* planck,
                                 const double* temp, const int* cloud_type, const double* wc, const double* reff,
                                 int cstride, const double* od, double* radiance, double* dgas, double* dT,
                                 double* e_b, double* Bs_b, double* dwc, double* dre, int dd, int soi_slots,
                                 int* n_orders) {
  CloudLut L{dims[0], dims[1], dims[2], dims[3], dims[4], dims[5], dims[6], f_mw, r_mw, t, f_ir, r_ir,
             ke_l, w_l, pc_l, ke_s, w_s, pc_s, ke_ir, w_ir, pc_ir};
  static const GaussTable gt = make_gauss();
  CloudyColumn c{};
  c.Ku = Ku; c.n_clouds = n_clouds; c.nleg = nleg; c.microwave = microwave != 0; c.freq = freq;
  c.mu_sensor = mu_sensor; c.emissivity = emissivity; c.planck_surface = planck_surface; c.cosmic = cosmic;
  c.c1 = planck[0]; c.c2 = planck[1]; c.b1 = planck[2]; c.b2 = planck[3];
  c.temperature = temp; c.cloud_type = cloud_type; c.wc = wc; c.reff = reff; c.cstride = (size_t)cstride;
  constexpr int NZ = SC_NZ_MAX;
  StreamSet<NZ, double> S;
  if (int rc = stream_set<NZ, double>(nleg, mu_sensor, L.nleg, gt, S)) return rc;
  auto layer = [&](int k, int* kind, double* o, Mat<NZ, double>& Tm, Mat<NZ, double>& Rm, double* src) {
    *kind = layer_optics<NZ, double>(c, L, S, k, od[k], temp[k], o, Tm, Rm, src);
  };
  std::vector<double> st((size_t)(Ku + 1) * (NZ * NZ + NZ));
  auto state = [&](int lev, int i) -> double& { return st[(size_t)lev * (NZ * NZ + NZ) + i]; };
  int bad = 0;
  auto adj = [&](int k, int kind, const Mat<NZ, double>& T_b, const Mat<NZ, double>& R_b, const double* src_b,
                 double od_b, double B_b) {
    // gas and temperature, then each cloud's (water content, radius), one cloud per pass
    LayerDirections d{true, 0, {0, 0, 0, 0}};
    double g[4];
    auto contract = [&](const LayerDirections& dir) {
      return dd ? layer_contract<NZ, 2, DD>(c, L, S, k, od[k], dir, T_b, R_b, src_b, od_b, B_b, g)
                : layer_contract<NZ, 2>(c, L, S, k, od[k], dir, T_b, R_b, src_b, od_b, B_b, g);
    };
    if (contract(d) != kind) bad = 7;
    dgas[k] = g[0];
    dT[k] = g[1];
    for (int cc = 0; cc < n_clouds; cc++) {
      d = LayerDirections{false, 1, {cc, 0, 0, 0}};
      if (contract(d) != kind) bad = 7;
      if (dwc) dwc[(size_t)cc * cstride + k] = g[0];
      if (dre) dre[(size_t)cc * cstride + k] = g[1];
    }
  };
  if (soi_slots <= 0) {
    const int rc = cloudy_adjoint<NZ>(c, S, layer, state, adj, radiance, e_b, Bs_b);
    return rc ? rc : bad;
  }
  // SOI (soi_slots order-field slots): records first, the orders' adjoint,
  // then the same contraction of every layer's record adjoints
  c.soi = true;
  constexpr int NE = 2 + 2 * NZ * NZ + NZ;
  std::vector<double> rec((size_t)Ku * NE), rab((size_t)Ku * NE);
  for (int k = 0; k < Ku; k++) {
    Mat<NZ, double> Tm, Rm;
    double sv[NZ], o;
    const int kind = layer_optics<NZ, double>(c, L, S, k, od[k], temp[k], &o, Tm, Rm, sv);
    if (kind < 0) return -kind;
    double* r = &rec[(size_t)k * NE];
    r[0] = kind;
    r[1] = o;
    for (int i = 0; i < NZ; i++) {
      for (int j = 0; j < NZ; j++) { r[2 + i * NZ + j] = Tm.a[i][j]; r[2 + NZ * NZ + i * NZ + j] = Rm.a[i][j]; }
      r[2 + 2 * NZ * NZ + i] = sv[i];
    }
  }
  const int nZ = S.nZ;
  auto lod = [&](int k, int* kd, double* o, double* B) {
    *kd = (int)rec[(size_t)k * NE];
    *o = rec[(size_t)k * NE + 1];
    *B = c.c1 / (exp(c.c2 / (c.b1 + c.b2 * temp[k])) - 1.0);
  };
  auto lsrc = [&](int k, double* sv) { for (int i = 0; i < nZ; i++) sv[i] = rec[(size_t)k * NE + 2 + 2 * NZ * NZ + i]; };
  auto ltr = [&](int k, Mat<NZ, double>& Tm, Mat<NZ, double>& Rm) {
    for (int i = 0; i < nZ; i++)
      for (int j = 0; j < nZ; j++) {
        Tm.a[i][j] = rec[(size_t)k * NE + 2 + i * NZ + j];
        Rm.a[i][j] = rec[(size_t)k * NE + 2 + NZ * NZ + i * NZ + j];
      }
  };
  std::vector<double> fs((size_t)soi_slots * 2 * (Ku + 1) * NZ, 0.0), lm((size_t)4 * (Ku + 1) * NZ, 0.0);
  auto fld = [&](int sl, int f, int k, int i) -> double& { return fs[(((size_t)sl * 2 + f) * (Ku + 1) + k) * NZ + i]; };
  auto lam = [&](int b, int f, int k, int i) -> double& { return lm[(((size_t)b * 2 + f) * (Ku + 1) + k) * NZ + i]; };
  auto ab = [&](int k, int e) -> double& { return rab[(size_t)k * NE + e]; };
  const int rc = soi_adjoint<NZ>(nZ, Ku, S.isat, S.mu, emissivity, planck_surface, cosmic, soi_slots, lod, lsrc, ltr,
                                 fld, lam, ab, radiance, e_b, Bs_b, n_orders);
  if (rc) return rc;
  for (int k = 0; k < Ku; k++) {
    const double* r = &rab[(size_t)k * NE];
    Mat<NZ, double> T_b, R_b;
    double src_b[NZ];
    const int kind = (int)r[0];
    for (int i = 0; i < NZ; i++) {
      for (int j = 0; j < NZ; j++) {
        T_b.a[i][j] = kind == 1 ? r[2 + i * NZ + j] : 0.0;
        R_b.a[i][j] = kind == 1 ? r[2 + NZ * NZ + i * NZ + j] : 0.0;
      }
      src_b[i] = kind == 1 ? r[2 + 2 * NZ * NZ + i] : 0.0;
    }
    adj(k, kind, T_b, R_b, src_b, r[1], kind == 1 ? 0.0 : r[2]);
  }
  return bad;
}



// One aerosol-only layer's record (od, T, R, src) and its derivatives with
// respect to aerosol a's concentration and first LUT coordinate (radius, or
// the layer's relative humidity for 'GOCART-GEOS5' / 'NAAPS'), from the
// derivative-number evaluation the K-matrix contraction uses
// (layer_optics_dual), and the MOM eigenvalue gap at the sensor angle.
// adims as sx_cloudy_radiance's.
extern "C" int sx_aerosol_layer_record(const int* adims, const int* atypes, const double* afreq,
                                       const double* areff, const double* arsig, const double* arh,
                                       const double* ake, const double* aw, const double* apc, int n_aer,
                                       const int* aer_type, const double* conc, const double* aer_reff,
                                       const double* aer_var, double rh_layer, int nleg, double mu_sensor,
                                       const double* planck, double wavenumber, double gas, double tk, int a,
                                       double* val, double* dconc, double* dc1, int* nz_out, double* gap_out) {
  AerosolLut A{};
  A.nw = adims[0]; A.nrh = adims[1]; A.nr = adims[2]; A.ns = adims[3]; A.nt = adims[4]; A.nleg = adims[5];
  A.scheme = adims[6]; A.nrh_axis = adims[7];
  A.type_id = atypes; A.freq = afreq; A.reff = areff; A.rsig = arsig; A.rh = arh; A.ke = ake; A.w = aw;
  A.pc = apc;
  CloudLut L{};
  static const GaussTable gt = make_gauss();
  CloudyColumn c{};
  c.Ku = 1; c.n_clouds = 0; c.nleg = nleg; c.microwave = false; c.freq = wavenumber; c.mu_sensor = mu_sensor;
  c.c1 = planck[0]; c.c2 = planck[1]; c.b1 = planck[2]; c.b2 = planck[3];
  c.n_aerosols = n_aer; c.wavenumber = wavenumber; c.aerosol_type = aer_type; c.conc = conc;
  c.aer_reff = aer_reff; c.aer_var = aer_var; c.rh = &rh_layer; c.cstride = 1; c.alut = &A;
  constexpr int NZ = SC_NZ_MAX;
  StreamSet<NZ, double> S;
  if (int rc = stream_set<NZ, double>(nleg, mu_sensor, -1, gt, S)) return -100 - rc;
  using D = Dual<2>;
  auto seed = [&](int s, D& amount, D& c1, D&) {
    if (s == a) { amount.d[0] = 1.0; c1.d[1] = 1.0; }
  };
  Mat<NZ, D> Tm, Rm;
  D src[NZ], od;
  const int kind = layer_optics_dual<NZ>(c, L, S, 0, D(gas), D(tk), &od, Tm, Rm, src, seed);
  const int nZ = S.nZ;
  *nz_out = nZ;
  if (gap_out) {   // the MOM eigenvalue gap at the sensor angle (plain evaluation)
    Mat<NZ, double> T0, R0;
    double s0[NZ], o0;
    *gap_out = 1.0;
    layer_optics<NZ, double>(c, L, S, 0, gas, tk, &o0, T0, R0, s0, NoSeed(), gap_out);
  }
  auto put = [&](const D& x, int i) { val[i] = x.v; dconc[i] = x.d[0]; dc1[i] = x.d[1]; };
  put(od, 0);
  for (int i = 0; i < nZ; i++)
    for (int j = 0; j < nZ; j++) { put(Tm.a[i][j], 1 + i * nZ + j); put(Rm.a[i][j], 1 + nZ * nZ + i * nZ + j); }
  for (int i = 0; i < nZ; i++) put(src[i], 1 + 2 * nZ * nZ + i);
  return kind;
}

// IR sea-surface emissivity (irssem) with its wind-speed and temperature derivatives.
extern "C" double sx_irssem(const int* dims, int nalli2, const double* angle, const double* freq, const double* wind,
                            const double* temp, const double* e, double water_temperature, double wind_speed,
                            double frequency, double ang, double* de_dv, double* de_dt) {
  const IRWaterLut W{dims[0], dims[1], dims[2], dims[3], nalli2, angle, freq, wind, temp, e};
  Dual<2> t(water_temperature), v(wind_speed);
  v.d[0] = 1.0;
  t.d[1] = 1.0;
  const Dual<2> r = irssem<Dual<2>>(W, t, v, frequency, ang);
  *de_dv = r.d[0];
  *de_dt = r.d[1];
  return irssem<double>(W, water_temperature, wind_speed, frequency, ang);
}


// One layer's optics adjoint two ways, for record adjoints T_b, R_b, src_b
// (scattering layer) or od_b, B_b (clear layer): the reverse sweep
// (layer_adjoint, FP64) and the contraction on derivative numbers
// (layer_contract).  Outputs per method: g[0] gas optical depth, g[1]
// temperature, then per species s (clouds, then aerosols) amount, c1, c2 at
// g[2 + 3 s ..].  Column and LUT arguments as sx_cloudy_radiance's.  Returns
// the layer kind of the reverse sweep (or its negative error), and
// *kind_dual that of the derivative-number evaluation.
extern "C" int sx_layer_adjoint_compare(
    const int* dims, const double* f_mw, const double* r_mw, const double* t, const double* f_ir,
    const double* r_ir, const double* ke_l, const double* w_l, const double* pc_l, const double* ke_s,
    const double* w_s, const double* pc_s, const double* ke_ir, const double* w_ir, const double* pc_ir, int Ku,
    int n_clouds, int nleg, int microwave, double freq, double mu_sensor, const double* planck, const double* temp,
    const int* cloud_type, const double* wc, const double* reff, int cstride, int n_aer, const int* aer_type,
    const double* conc, const double* aer_reff, const double* aer_var, const double* rh_layers, const int* adims,
    const int* atypes, const double* afreq, const double* areff, const double* arsig, const double* arh,
    const double* ake, const double* aw, const double* apc, double wavenumber, int k, double gas,
    const double* tb, const double* rb, const double* sb, double od_b, double B_b, double* g_rev, double* g_dual,
    int* kind_dual, int* nz_out) {
  AerosolLut A{};
  if (n_aer > 0) {
    A.nw = adims[0]; A.nrh = adims[1]; A.nr = adims[2]; A.ns = adims[3]; A.nt = adims[4]; A.nleg = adims[5];
    A.scheme = adims[6]; A.nrh_axis = adims[7];
    A.type_id = atypes; A.freq = afreq; A.reff = areff; A.rsig = arsig; A.rh = arh; A.ke = ake; A.w = aw;
    A.pc = apc;
  }
  CloudLut L{dims[0], dims[1], dims[2], dims[3], dims[4], dims[5], dims[6], f_mw, r_mw, t, f_ir, r_ir,
             ke_l, w_l, pc_l, ke_s, w_s, pc_s, ke_ir, w_ir, pc_ir};
  static const GaussTable gt = make_gauss();
  CloudyColumn c{};
  c.Ku = Ku; c.n_clouds = n_clouds; c.nleg = nleg; c.microwave = microwave != 0; c.freq = freq;
  c.mu_sensor = mu_sensor;
  c.c1 = planck[0]; c.c2 = planck[1]; c.b1 = planck[2]; c.b2 = planck[3];
  c.temperature = temp; c.cloud_type = cloud_type; c.wc = wc; c.reff = reff; c.cstride = (size_t)cstride;
  c.n_aerosols = n_aer; c.wavenumber = wavenumber; c.aerosol_type = aer_type; c.conc = conc;
  c.aer_reff = aer_reff; c.aer_var = aer_var; c.rh = rh_layers; c.alut = &A;
  constexpr int NZ = SC_NZ_MAX;
  StreamSet<NZ, double> S;
  if (int rc = stream_set<NZ, double>(nleg, mu_sensor, n_clouds > 0 ? L.nleg : -1, gt, S)) return -100 - rc;
  const int nZ = S.nZ;
  *nz_out = nZ;
  Mat<NZ, double> T_b, R_b;
  double src_b[NZ];
  for (int i = 0; i < nZ; i++) {
    src_b[i] = sb[i];
    for (int j = 0; j < nZ; j++) { T_b.a[i][j] = tb[i * nZ + j]; R_b.a[i][j] = rb[i * nZ + j]; }
  }
  const int nsp = n_clouds + (microwave ? 0 : n_aer);
  // the record's kind from the plain forward
  Mat<NZ, double> T0, R0;
  double s0[NZ], o0;
  const int kind = layer_optics<NZ, double>(c, L, S, k, gas, temp[k], &o0, T0, R0, s0);
  if (kind < 0) return kind;
  double g[2], gs[2 * SC_NC_MAX][3];
  const int kr = layer_adjoint<NZ, double>(c, L, S, k, gas, kind, T_b, R_b, src_b, kind == 1 ? 0.0 : od_b,
                                           kind == 1 ? 0.0 : B_b, g, gs);
  g_rev[0] = g[0];
  g_rev[1] = g[1];
  for (int s = 0; s < nsp; s++)
    for (int q = 0; q < 3; q++) g_rev[2 + 3 * s + q] = gs[s][q];
  double gd[4];
  LayerDirections d{true, 0, {0, 0, 0, 0}};
  *kind_dual = layer_contract<NZ, 2>(c, L, S, k, gas, d, T_b, R_b, src_b, kind == 1 ? 0.0 : od_b,
                                     kind == 1 ? 0.0 : B_b, gd);
  g_dual[0] = gd[0];
  g_dual[1] = gd[1];
  for (int s = 0; s < nsp; s++) {
    d = LayerDirections{false, 1, {s, 0, 0, 0}};
    layer_contract<NZ, 2>(c, L, S, k, gas, d, T_b, R_b, src_b, kind == 1 ? 0.0 : od_b, 0.0, gd);
    g_dual[2 + 3 * s] = gd[0];
    g_dual[3 + 3 * s] = gd[1];
    d.second = true;
    layer_contract<NZ, 2>(c, L, S, k, gas, d, T_b, R_b, src_b, kind == 1 ? 0.0 : od_b, 0.0, gd);
    g_dual[4 + 3 * s] = gd[0];
  }
  return kr;
}


// K-matrix of one cloudy (profile, channel) through ADA as the mixed form
// computes it (mixed != 0: layer records from the FP32 layer solver in loss
// form, the adding and its adjoint in FP32 with the (I - Rup R)^-1 inversions
// in FP64, the layers' reverse sweep in FP32) or the FP64 form (mixed = 0):
// radiance, dR/d(gas OD_k), dR/dT_k, dR/de, dR/dB_surface and each cloud's
// dR/dwc, dR/dre.  Arguments as sx_cloudy_kmatrix's.
template <class A>
static int cloudy_kmatrix_form(const CloudyColumn& c, const CloudLut& L, const StreamSet<SC_NZ_MAX, double>& S,
                               const double* od, double* radiance, double* dgas, double* dT, double* e_b,
                               double* Bs_b, double* dwc, double* dre, int cstride) {
  constexpr int NZ = SC_NZ_MAX;
  auto layer = [&](int k, int* kind, double* o, Mat<NZ, A>& Tm, Mat<NZ, A>& Rm, A* src) {
    A ow;
    *kind = layer_optics<NZ, A, A>(c, L, S, k, A(od[k]), A(c.temperature[k]), &ow, Tm, Rm, src);
    *o = double(ow);
  };
  std::vector<A> st((size_t)(c.Ku + 1) * (NZ * NZ + NZ));
  auto state = [&](int lev, int i) -> A& { return st[(size_t)lev * (NZ * NZ + NZ) + i]; };
  int bad = 0;
  auto adj = [&](int k, int kind, const Mat<NZ, A>& T_b, const Mat<NZ, A>& R_b, const A* src_b, double od_b,
                 double B_b) {
    Mat<NZ, double> Tb, Rb;
    double sb[NZ];
    for (int i = 0; i < NZ; i++) {
      sb[i] = kind == 1 ? double(src_b[i]) : 0.0;
      for (int j = 0; j < NZ; j++) {
        Tb.a[i][j] = kind == 1 ? double(T_b.a[i][j]) : 0.0;
        Rb.a[i][j] = kind == 1 ? double(R_b.a[i][j]) : 0.0;
      }
    }
    double g[2], gs[2 * SC_NC_MAX][3];
    const int kr = layer_adjoint<NZ, A>(c, L, S, k, od[k], kind, Tb, Rb, sb, kind == 1 ? 0.0 : od_b,
                                        kind == 1 ? 0.0 : B_b, g, gs);
    if (kr != kind) bad = 7;
    dgas[k] = g[0];
    dT[k] = g[1];
    for (int cc = 0; cc < c.n_clouds; cc++) {
      dwc[(size_t)cc * cstride + k] = gs[cc][0];
      dre[(size_t)cc * cstride + k] = gs[cc][1];
    }
  };
  const int rc = cloudy_adjoint<NZ, decltype(layer), decltype(state), decltype(adj), A>(c, S, layer, state, adj,
                                                                                        radiance, e_b, Bs_b);
  return rc ? rc : bad;
}

extern "C" int sx_cloudy_kmatrix_form(const int* dims, const double* f_mw, const double* r_mw, const double* t,
                                      const double* f_ir, const double* r_ir, const double* ke_l, const double* w_l,
                                      const double* pc_l, const double* ke_s, const double* w_s, const double* pc_s,
                                      const double* ke_ir, const double* w_ir, const double* pc_ir, int Ku,
                                      int n_clouds, int nleg, int microwave, double freq, double mu_sensor,
                                      double emissivity, double planck_surface, double cosmic, const double* planck,
                                      const double* temp, const int* cloud_type, const double* wc, const double* reff,
                                      int cstride, const double* od, double* radiance, double* dgas, double* dT,
                                      double* e_b, double* Bs_b, double* dwc, double* dre, int mixed) {
  CloudLut L{dims[0], dims[1], dims[2], dims[3], dims[4], dims[5], dims[6], f_mw, r_mw, t, f_ir, r_ir,
             ke_l, w_l, pc_l, ke_s, w_s, pc_s, ke_ir, w_ir, pc_ir};
  static const GaussTable gt = make_gauss();
  CloudyColumn c{};
  c.Ku = Ku; c.n_clouds = n_clouds; c.nleg = nleg; c.microwave = microwave != 0; c.freq = freq;
  c.mu_sensor = mu_sensor; c.emissivity = emissivity; c.planck_surface = planck_surface; c.cosmic = cosmic;
  c.c1 = planck[0]; c.c2 = planck[1]; c.b1 = planck[2]; c.b2 = planck[3];
  c.temperature = temp; c.cloud_type = cloud_type; c.wc = wc; c.reff = reff; c.cstride = (size_t)cstride;
  StreamSet<SC_NZ_MAX, double> S;
  if (int rc = stream_set<SC_NZ_MAX, double>(nleg, mu_sensor, L.nleg, gt, S)) return rc;
  return mixed ? cloudy_kmatrix_form<float>(c, L, S, od, radiance, dgas, dT, e_b, Bs_b, dwc, dre, cstride)
               : cloudy_kmatrix_form<double>(c, L, S, od, radiance, dgas, dT, e_b, Bs_b, dwc, dre, cstride);
}


// The channel-interpolated cloud tables (CloudChan, built here as
// cloud_chan_kernel builds them on the GPU, for the channels at frequencies
// freq[0..L-1]) against the direct lookups: every cloud type, radius and
// temperature of the grids given, every Legendre term of the stream sets
// nleg = 2..16 (with their offsets), value and radius / temperature
// derivatives (Dual<2>).  Returns the largest |difference|.
extern "C" double sx_cloud_chan_compare(const int* dims, const double* f_mw, const double* r_mw, const double* t,
                                        const double* f_ir, const double* r_ir, const double* ke_l,
                                        const double* w_l, const double* pc_l, const double* ke_s, const double* w_s,
                                        const double* pc_s, const double* ke_ir, const double* w_ir,
                                        const double* pc_ir, int microwave, int L, const double* freq, int n_re,
                                        const double* re_grid, int n_t, const double* t_grid) {
  CloudLut C{dims[0], dims[1], dims[2], dims[3], dims[4], dims[5], dims[6], f_mw, r_mw, t, f_ir, r_ir,
             ke_l, w_l, pc_l, ke_s, w_s, pc_s, ke_ir, w_ir, pc_ir};
  const bool mw = microwave != 0;
  const int rows = mw ? C.nrm : C.nri, nf = mw ? C.nfm : C.nfi;
  const long long n = (long long)cloud_chan_planes(C, mw) * rows * L;
  std::vector<double> z((size_t)n);
  for (long long i = 0; i < n; i++) {
    const int ch = (int)(i % L);
    const long long qr = i / L;
    const int r = (int)(qr % rows), q = (int)(qr / rows);
    const Lagrange4 U = lagrange4(mw ? C.f_mw : C.f_ir, nf, freq[ch]);
    z[(size_t)i] = lerp4(cloud_chan_source(C, mw, q) + (size_t)r * nf + U.i0, 1, U);
  }
  // the radius and temperature axes' reciprocal tables, as the library builds them
  std::vector<double> rmw((size_t)std::max(C.nrm - 3, 0) * 7), rir((size_t)std::max(C.nri - 3, 0) * 7),
      rt((size_t)std::max(C.nt - 3, 0) * 7);
  lagrange4_recip_table(C.r_mw, C.nrm, rmw.data());
  lagrange4_recip_table(C.r_ir, C.nri, rir.data());
  lagrange4_recip_table(C.t, C.nt, rt.data());
  CloudLut CR = C;
  CR.rc_rmw = C.nrm >= 4 ? rmw.data() : nullptr;
  CR.rc_rir = C.nri >= 4 ? rir.data() : nullptr;
  CR.rc_t = C.nt >= 4 ? rt.data() : nullptr;
  using D = Dual<2>;
  double worst = 0.0;
  const int nlegs[5] = {2, 4, 6, 8, 16};
  for (int ch = 0; ch < L; ch++)
    for (int type = 1; type <= 6; type++)
      for (int a = 0; a < n_re; a++)
        for (int b = 0; b < n_t; b++)
          for (int q = 0; q < 5; q++) {
            const int nleg = nlegs[q], loff = legendre_offset(nleg);
            if (nleg + loff > C.nleg) continue;
            D re(re_grid[a]), tk(t_grid[b]);
            re.d[0] = 1.0;
            tk.d[1] = 1.0;
            D ke0, w0, pc0[SC_NLEG_MAX + 1], ke1, w1, pc1[SC_NLEG_MAX + 1];
            const CloudChan Z{z.data(), (size_t)L, ch};
            const bool ok0 = cloud_layer_optics<D>(C, mw, freq[ch], type, re, tk, nleg, loff, &ke0, &w0, pc0);
            const bool ok1 = cloud_layer_optics<D>(CR, mw, freq[ch], type, re, tk, nleg, loff, &ke1, &w1, pc1, Z);
            if (ok0 != ok1) return 1e300;
            if (!ok0) continue;
            auto cmp = [&](const D& x, const D& y) {
              worst = std::max(worst, std::fabs(x.v - y.v));
              for (int d = 0; d < 2; d++) worst = std::max(worst, std::fabs(x.d[d] - y.d[d]));
            };
            cmp(ke0, ke1);
            cmp(w0, w1);
            for (int l = 0; l <= nleg; l++) cmp(pc0[l], pc1[l]);
          }
  return worst;
}

