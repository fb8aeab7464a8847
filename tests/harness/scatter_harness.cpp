// CPU harness around the GPU library's cloud/ADA physics header (test
// infrastructure only): one ADA layer and one cloudy (profile, channel).
#include <vector>

#include "scatter_physics.cuh"

using namespace crtm;

namespace {
GaussTable make_gauss() {
  GaussTable g{};
  for (int n = 1; n <= 9; n++) double_gauss_host(n, g.mu[n], g.w[n]);
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

// dims: nfm nrm nt nd nfi nri nleg; arrays in the file's Fortran order.
int sx_cloudy_radiance(const int* dims, const double* f_mw, const double* r_mw, const double* t,
                       const double* f_ir, const double* r_ir, const double* ke_l, const double* w_l,
                       const double* pc_l, const double* ke_s, const double* w_s, const double* pc_s,
                       const double* ke_ir, const double* w_ir, const double* pc_ir, int Ku, int n_clouds,
                       int nleg, int microwave, double freq, double mu_sensor, double emissivity,
                       double planck_surface, double cosmic, const double* planck, const double* temp,
                       const int* cloud_type, const double* wc, const double* reff, int cstride,
                       const double* od, double* radiance) {
  CloudLut L{dims[0], dims[1], dims[2], dims[3], dims[4], dims[5], dims[6], f_mw, r_mw, t, f_ir, r_ir,
             ke_l, w_l, pc_l, ke_s, w_s, pc_s, ke_ir, w_ir, pc_ir};
  static const GaussTable gt = make_gauss();
  CloudyColumn c{};
  c.Ku = Ku; c.n_clouds = n_clouds; c.nleg = nleg; c.microwave = microwave != 0; c.freq = freq;
  c.mu_sensor = mu_sensor; c.emissivity = emissivity; c.planck_surface = planck_surface; c.cosmic = cosmic;
  c.c1 = planck[0]; c.c2 = planck[1]; c.b1 = planck[2]; c.b2 = planck[3];
  c.temperature = temp; c.cloud_type = cloud_type; c.wc = wc; c.reff = reff; c.cstride = (size_t)cstride;
  return cloudy_radiance<SC_NZ_MAX>(c, L, gt, [&](int k) { return od[k]; }, radiance);
}

int sx_stream_rule(double max_reff, double wavenumber) { return stream_rule_nleg(max_reff, wavenumber); }
}
