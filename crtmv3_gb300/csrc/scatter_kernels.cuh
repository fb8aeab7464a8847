// Cloudy forward kernels, after the column kernel has stored the gas layer
// optical depths:
//
//   scatter_layers_kernel  one thread per (profile, layer, channel): cloud
//                          optics, combine, phase blocks and, for scattering
//                          layers, the layer transmission/reflection/source
//                          (MOM), in the working precision R.  Layers are
//                          independent, so this is where the parallelism is.
//   scatter_adding_kernel  one thread per (profile, channel): the adding
//                          recursion from the surface to the top (ADA) or the
//                          successive orders of interaction (SOI), FP64 in
//                          every form, then the FP64 Planck inversion.
//
// Per-layer results go through HBM with channels fastest:
// LB[p][k][e][l], e = 0 kind (0 clear, 1 scattering, <0 error), 1 optical
// depth, then T (NZ*NZ), R (NZ*NZ) and the source (NZ).
//
// K-matrix and adjoint of scattering profiles (ADA), between the two column
// launches:
//
//   scatter_layers_k_kernel  one thread per (profile, layer, channel): the
//                            layer optics on derivative numbers (directions:
//                            gas optical depth, temperature); the record adds
//                            the derivatives of T, R, the source and the
//                            optical depth (layer_record_k).
//   scatter_kmatrix_kernel   one thread per (profile, channel): the adding
//                            from the surface with the level states kept in
//                            AS, then the adding adjoint from the top down,
//                            contracted with the layer derivatives.  Writes,
//                            for a unit radiance seed, dR/dtau of each user
//                            layer (TODc), the Planck part of the temperature
//                            derivative (PT), and the radiance and surface
//                            derivatives (CB).  The second column launch
//                            mixes them with the clear column of a
//                            fractional profile, applies the Planck-inversion
//                            seed and maps dR/dtau onto the reference levels.
#pragma once

#include "odps_kernels.cuh"
#include "scatter_physics.cuh"

namespace crtm {

__constant__ GaussTable c_gauss;

template <int NZ>
constexpr int layer_record() { return 2 + 2 * NZ * NZ + NZ; }
// K-matrix layer record: kind, optical depth, the values of T, R and the
// source (NV = 2 NZ^2 + NZ), their derivatives with respect to the gas optical
// depth and to the temperature (NV each), then the optical depth's two.
template <int NZ>
constexpr int layer_record_k() { return 4 + 3 * (2 * NZ * NZ + NZ); }
// adding state per level: Rup (NZ*NZ) and the upwelling radiance (NZ)
template <int NZ>
constexpr int adding_state_size() { return NZ * NZ + NZ; }

template <class R>
struct ScatterArgs {
  int K, L, Kmax, p_begin, n_chunk, microwave;
  BatchView b;
  SpecView sp;
  PrepView<R> pv;
  CloudLut lut;
  int max_clouds;
  const int* n_clouds;          // [P]
  const int* cloud_type;        // [P][NC]
  const double* wc, *reff;      // [P][NC][Kmax]
  const int* n_streams;         // [P] or null
  const int* rt_algorithm;      // [P] or null (ADA)
  AerosolLut alut;
  int max_aerosols;
  const int* n_aerosols;        // [P] (null when max_aerosols = 0)
  const int* aerosol_type;      // [P][NA]
  const double* conc, *aer_reff;   // [P][NA][Kmax]
  double* FB;                   // SOI fields [n][2][2][Kmax+1][NZ][L], or null
  const R* TAU;                 // [n][Kmax][L] gas layer optical depths
  R* LB;                        // [n][Kmax][NE][L] layer records
  const double* cloud_fraction; // [P][Kmax] or null (1)
  const int* overlap;           // [P] Options%Overlap_Id or null (4, average)
  double* maxreff;              // [n]
  double* cover;                // [n] total cloud cover, -1: no clear part
  double* radiance, *bt;        // [P][L]
  int* status;                  // [P] or null
  int* error;                   // first failing code (device), 0 if none
  // K-matrix and adjoint: the cloudy column's derivatives for a unit
  // radiance seed, combined with the clear column by the second column launch
  R* TODc;                      // [n][Kmax][L] dR/dtau of the user layers
  R* PT;                        // [n][Kmax][L] dR/dT at fixed gas optical depth
  double* CB;                   // [n][3][L] radiance, dR/d(emissivity), dR/d(surface Planck)
  double* AS;                   // [n][Kmax+1][NS][L] adding states
};

constexpr int SCATTER_THREADS = 128;

// Per profile, one warp each: the largest effective radius of its clouds and
// aerosols (stream rule input; clouds dropped by a fraction below 1e-12 do
// not count) and the total cloud cover of a fractional profile.
template <class R>
__global__ void scatter_profile_kernel(ScatterArgs<R> a) {
  const int p = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (p >= a.n_chunk) return;
  const int gp = a.p_begin + p, Ku = a.b.n_layers[gp];
  const int nc = a.max_clouds > 0 ? a.n_clouds[gp] : 0, na = a.max_aerosols > 0 ? a.n_aerosols[gp] : 0;
  const double* cf = a.cloud_fraction ? a.cloud_fraction + (size_t)gp * a.Kmax : nullptr;
  double mr = 0.0;
  for (int i = lane; i < nc * Ku; i += 32) {
    if (cf && cf[i % Ku] < MIN_COVERAGE) continue;
    const double r = a.reff[((size_t)gp * a.max_clouds + i / Ku) * a.Kmax + (i % Ku)];
    mr = r > mr ? r : mr;
  }
  for (int i = lane; i < na * Ku; i += 32) {
    const double r = a.aer_reff[((size_t)gp * a.max_aerosols + i / Ku) * a.Kmax + (i % Ku)];
    mr = r > mr ? r : mr;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const double v = __shfl_xor_sync(FULL, mr, o);
    mr = v > mr ? v : mr;
  }
  if (lane == 0) {
    a.maxreff[p] = mr;
    double tcc = -1.0;
    if (nc > 0) {
      tcc = total_cloud_cover(Ku, nc, cf, a.wc + (size_t)gp * a.max_clouds * a.Kmax, (size_t)a.Kmax,
                              a.overlap ? a.overlap[gp] : 4);
      if (tcc < -1.5) {
        atomicCAS(a.error, 0, 11);
        if (a.status) atomicOr(a.status + gp, 1 << 4);
        tcc = -1.0;
      }
    }
    a.cover[p] = tcc;
  }
}

// Radiance of the clear column (gas optical depths tau, stride L; Emission
// solver in FP64), the clear part of a fractional profile.
template <class R>
__device__ double clear_column_radiance(const CloudyColumn& c, const R* tau, int L) {
  const double inv_u = 1.0 / c.mu_sensor;
  double down = c.cosmic, tr_tot = 1.0, src = 0.0;
  for (int k = 0; k < c.Ku; k++) {
    const double t = exp(-double(tau[(size_t)k * L]) * inv_u);
    const double B = c.c1 / (exp(c.c2 / (c.b1 + c.b2 * c.temperature[k])) - 1.0);
    src += tr_tot * B * (1.0 - t);
    down = down * t + B * (1.0 - t);
    tr_tot *= t;
  }
  return src + tr_tot * (c.emissivity * c.planck_surface + (1.0 - c.emissivity) * down);
}

template <class R>
__device__ __forceinline__ CloudyColumn column_inputs(const ScatterArgs<R>& a, int p, int gp, int l) {
  CloudyColumn c;
  c.Ku = a.b.n_layers[gp];
  c.n_clouds = a.max_clouds > 0 ? a.n_clouds[gp] : 0;
  const int ns = a.n_streams ? a.n_streams[gp] : 0;
  c.nleg = ns > 0 ? ns : stream_rule_nleg(a.maxreff[p], a.sp.wn[l]);
  c.microwave = a.microwave != 0;
  c.freq = a.microwave ? a.sp.freq[l] : a.sp.wn[l];
  c.mu_sensor = a.pv.scal[(size_t)p * 4 + 1];
  const size_t pl = (size_t)gp * a.L + l;
  c.emissivity = a.b.emissivity[pl];
  c.c1 = a.sp.c1[l]; c.c2 = a.sp.c2[l]; c.b1 = a.sp.b1[l]; c.b2 = a.sp.b2[l];
  const double ts = a.b.land_cov[gp] * a.b.land_t[gp] + a.b.water_cov[gp] * a.b.water_t[gp] +
                    a.b.snow_cov[gp] * a.b.snow_t[gp] + a.b.ice_cov[gp] * a.b.ice_t[gp];
  c.planck_surface = c.c1 / (exp(c.c2 / (c.b1 + c.b2 * ts)) - 1.0);
  c.cosmic = a.sp.cbr[l];
  c.temperature = a.b.temperature + (size_t)gp * a.Kmax;
  c.cloud_type = a.max_clouds > 0 ? a.cloud_type + (size_t)gp * a.max_clouds : nullptr;
  c.wc = a.max_clouds > 0 ? a.wc + (size_t)gp * a.max_clouds * a.Kmax : nullptr;
  c.reff = a.max_clouds > 0 ? a.reff + (size_t)gp * a.max_clouds * a.Kmax : nullptr;
  c.cstride = (size_t)a.Kmax;
  c.soi = a.rt_algorithm && a.rt_algorithm[gp] == 168;   // RT_SOI
  c.n_aerosols = a.max_aerosols > 0 ? a.n_aerosols[gp] : 0;
  c.wavenumber = a.sp.wn[l];
  c.aerosol_type = a.max_aerosols > 0 ? a.aerosol_type + (size_t)gp * a.max_aerosols : nullptr;
  c.conc = a.max_aerosols > 0 ? a.conc + (size_t)gp * a.max_aerosols * a.Kmax : nullptr;
  c.aer_reff = a.max_aerosols > 0 ? a.aer_reff + (size_t)gp * a.max_aerosols * a.Kmax : nullptr;
  c.alut = &a.alut;
  c.cf = a.cloud_fraction && c.n_clouds > 0 ? a.cloud_fraction + (size_t)gp * a.Kmax : nullptr;
  const double tcc = a.cover[p];
  c.wc_div = tcc > MIN_COVERAGE ? tcc : 1.0;
  return c;
}

template <int NZ, class R>
__global__ void __launch_bounds__(SCATTER_THREADS) scatter_layers_kernel(ScatterArgs<R> a) {
  constexpr int NE = layer_record<NZ>();
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int L = a.L, Kmax = a.Kmax;
  if (idx >= (long long)a.n_chunk * Kmax * L) return;
  const int l = (int)(idx % L);
  const int k = (int)((idx / L) % Kmax);
  const int p = (int)(idx / ((long long)L * Kmax));
  const int gp = a.p_begin + p;
  if (a.pv.status[p] != 0 || k >= a.b.n_layers[gp]) return;
  R* rec = a.LB + ((size_t)p * Kmax + k) * NE * L + l;
  const CloudyColumn c = column_inputs(a, p, gp, l);
  if (c.n_clouds == 0 && c.n_aerosols == 0) return;
  StreamSet<NZ, double> S;
  if (int rc = stream_set<NZ, double>(c.nleg, c.mu_sensor, c.n_clouds > 0 ? a.lut.nleg : -1, c_gauss, S)) {
    rec[0] = R(-rc);
    return;
  }
  Mat<NZ, R> Tm, Rm;
  R src[NZ], od;
  const double gas = double(a.TAU[((size_t)p * Kmax + k) * L + l]);
  const int kind = layer_optics<NZ, R>(c, a.lut, S, k, gas, c.temperature[k], &od, Tm, Rm, src);
  rec[0] = R(kind);
  rec[(size_t)L] = od;
  if (kind != 1) return;
  const int nZ = S.nZ;
  for (int i = 0; i < nZ; i++)
    for (int j = 0; j < nZ; j++) {
      rec[(size_t)(2 + i * NZ + j) * L] = Tm.a[i][j];
      rec[(size_t)(2 + NZ * NZ + i * NZ + j) * L] = Rm.a[i][j];
    }
  for (int i = 0; i < nZ; i++) rec[(size_t)(2 + 2 * NZ * NZ + i) * L] = src[i];
}

template <int NZ, class R>
__global__ void __launch_bounds__(SCATTER_THREADS) scatter_adding_kernel(ScatterArgs<R> a) {
  constexpr int NE = layer_record<NZ>();
  const int L = a.L, Kmax = a.Kmax;
  const int p = blockIdx.y, gp = a.p_begin + p;
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= L) return;
  const size_t pl = (size_t)gp * L + l;
  if (a.pv.status[p] != 0) {
    a.radiance[pl] = 0.0;
    a.bt[pl] = 0.0;
    return;
  }
  const CloudyColumn c = column_inputs(a, p, gp, l);
  const R* tau = a.TAU + (size_t)p * Kmax * L + l;
  double rad = 0.0;
  int code = 0;
  if (c.n_clouds == 0 && c.n_aerosols == 0) {   // clear profile: Emission solver, FP64 here
    rad = clear_column_radiance(c, tau, L);
  } else if (c.soi) {
    return;   // SOI profiles: scatter_soi_kernel
  } else {
    StreamSet<NZ, double> S;
    code = stream_set<NZ, double>(c.nleg, c.mu_sensor, c.n_clouds > 0 ? a.lut.nleg : -1, c_gauss, S);
    if (!code) {
      const int nZ = S.nZ;
      AddingState<NZ> A;
      adding_init<NZ>(A, nZ, c.emissivity, c.planck_surface);
      Mat<NZ, double> Tm, Rm;
      double src[NZ];
      for (int k = c.Ku - 1; k >= 0 && !code; k--) {
        const R* rec = a.LB + ((size_t)p * Kmax + k) * NE * L + l;
        const int kind = (int)rec[0];
        const double od = double(rec[(size_t)L]);
        if (kind < 0) { code = -kind; break; }
        if (kind == 1) {
          for (int i = 0; i < nZ; i++)
            for (int j = 0; j < nZ; j++) {
              Tm.a[i][j] = double(rec[(size_t)(2 + i * NZ + j) * L]);
              Rm.a[i][j] = double(rec[(size_t)(2 + NZ * NZ + i * NZ + j) * L]);
            }
          for (int i = 0; i < nZ; i++) src[i] = double(rec[(size_t)(2 + 2 * NZ * NZ + i) * L]);
          if (!adding_scatter<NZ>(A, nZ, Tm, Rm, src)) code = 6;
        } else {
          const double tk = c.temperature[k];
          adding_clear<NZ>(A, nZ, S.mu, od, c.c1 / (exp(c.c2 / (c.b1 + c.b2 * tk)) - 1.0));
        }
      }
      if (!code) rad = adding_toa<NZ>(A, nZ, S.isat, c.cosmic);
      const double tcc = a.cover[p];
      if (!code && tcc >= 0.0) rad = (1.0 - tcc) * clear_column_radiance(c, tau, L) + tcc * rad;
    }
  }
  if (code) {
    atomicCAS(a.error, 0, code);
    if (a.status) atomicOr(a.status + gp, 1 << 4);
    rad = 0.0;
  }
  a.radiance[pl] = rad;
  a.bt[pl] = code ? 0.0 : planck_temperature(c.c1, c.c2, c.b1, c.b2, rad);
}


// SOI profiles (Options%RT_Algorithm_Id = RT_SOI): successive orders of
// interaction over the layer records, fields in FB.
template <int NZ, class R>
__global__ void __launch_bounds__(SCATTER_THREADS) scatter_soi_kernel(ScatterArgs<R> a) {
  constexpr int NE = layer_record<NZ>();
  const int L = a.L, Kmax = a.Kmax;
  const int p = blockIdx.y, gp = a.p_begin + p;
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= L || a.pv.status[p] != 0) return;
  const CloudyColumn c = column_inputs(a, p, gp, l);
  if ((c.n_clouds == 0 && c.n_aerosols == 0) || !c.soi) return;
  const size_t pl = (size_t)gp * L + l;
  double rad = 0.0;
  int code = 0;
  StreamSet<NZ, double> S;
  code = stream_set<NZ, double>(c.nleg, c.mu_sensor, c.n_clouds > 0 ? a.lut.nleg : -1, c_gauss, S);
  if (!code) {
    const int nZ = S.nZ;
    auto layer = [&](int k, int* kind, double* od, double* B, Mat<NZ, double>& Tm, Mat<NZ, double>& Rm,
                     double* src) {
      const R* rec = a.LB + ((size_t)p * Kmax + k) * NE * L + l;
      *kind = (int)rec[0];
      *od = double(rec[(size_t)L]);
      const double tk = c.temperature[k];
      *B = c.c1 / (exp(c.c2 / (c.b1 + c.b2 * tk)) - 1.0);
      if (*kind != 1) return;
      for (int i = 0; i < nZ; i++) {
        for (int j = 0; j < nZ; j++) {
          Tm.a[i][j] = double(rec[(size_t)(2 + i * NZ + j) * L]);
          Rm.a[i][j] = double(rec[(size_t)(2 + NZ * NZ + i * NZ + j) * L]);
        }
        src[i] = double(rec[(size_t)(2 + 2 * NZ * NZ + i) * L]);
      }
    };
    double* fb = a.FB + (size_t)p * 4 * (Kmax + 1) * NZ * L + l;
    const size_t lev = (size_t)NZ * L, buf = (size_t)(Kmax + 1) * lev;
    auto dn = [&](int k, int i, int b) -> double& { return fb[b * buf + k * lev + (size_t)i * L]; };
    auto up = [&](int k, int i, int b) -> double& { return fb[(2 + b) * buf + k * lev + (size_t)i * L]; };
    for (int k = 0; k < c.Ku && !code; k++)
      if ((int)a.LB[((size_t)p * Kmax + k) * NE * L + l] < 0) code = -(int)a.LB[((size_t)p * Kmax + k) * NE * L + l];
    if (!code) soi_solve<NZ>(nZ, c.Ku, S.isat, S.mu, c.emissivity, c.planck_surface, c.cosmic, layer, dn, up, &rad);
    const double tcc = a.cover[p];
    if (!code && tcc >= 0.0)
      rad = (1.0 - tcc) * clear_column_radiance(c, a.TAU + (size_t)p * Kmax * L + l, L) + tcc * rad;
  }
  if (code) {
    atomicCAS(a.error, 0, code);
    if (a.status) atomicOr(a.status + gp, 1 << 4);
    rad = 0.0;
  }
  a.radiance[pl] = rad;
  a.bt[pl] = code ? 0.0 : planck_temperature(c.c1, c.c2, c.b1, c.b2, rad);
}

template <int NZ, class R>
__global__ void __launch_bounds__(SCATTER_THREADS) scatter_layers_k_kernel(ScatterArgs<R> a) {
  constexpr int NE = layer_record_k<NZ>(), NV = 2 * NZ * NZ + NZ;
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int L = a.L, Kmax = a.Kmax;
  if (idx >= (long long)a.n_chunk * Kmax * L) return;
  const int l = (int)(idx % L);
  const int k = (int)((idx / L) % Kmax);
  const int p = (int)(idx / ((long long)L * Kmax));
  const int gp = a.p_begin + p;
  if (a.pv.status[p] != 0 || k >= a.b.n_layers[gp]) return;
  R* rec = a.LB + ((size_t)p * Kmax + k) * NE * L + l;
  const CloudyColumn c = column_inputs(a, p, gp, l);
  if (c.n_clouds == 0 && c.n_aerosols == 0) return;
  if (c.soi) { rec[0] = R(-10); return; }   // SOI K-matrix: not available
  StreamSet<NZ, double> S;
  if (int rc = stream_set<NZ, double>(c.nleg, c.mu_sensor, c.n_clouds > 0 ? a.lut.nleg : -1, c_gauss, S)) {
    rec[0] = R(-rc);
    return;
  }
  using D = Dual<2>;
  D gd(double(a.TAU[((size_t)p * Kmax + k) * L + l])), tt(c.temperature[k]);
  gd.d[0] = 1.0;
  tt.d[1] = 1.0;
  Mat<NZ, D> Tm, Rm;
  D src[NZ], od;
  const int kind = layer_optics<NZ, D, D>(c, a.lut, S, k, gd, tt, &od, Tm, Rm, src);
  rec[0] = R(kind);
  rec[(size_t)L] = R(od.v);
  rec[(size_t)(2 + 3 * NV) * L] = R(od.d[0]);
  rec[(size_t)(3 + 3 * NV) * L] = R(od.d[1]);
  if (kind != 1) return;
  const int nZ = S.nZ;
  for (int i = 0; i < nZ; i++) {
    for (int j = 0; j < nZ; j++) {
      const size_t et = (size_t)(2 + i * NZ + j), er = et + NZ * NZ;
      rec[et * L] = R(Tm.a[i][j].v);
      rec[(et + NV) * L] = R(Tm.a[i][j].d[0]);
      rec[(et + 2 * NV) * L] = R(Tm.a[i][j].d[1]);
      rec[er * L] = R(Rm.a[i][j].v);
      rec[(er + NV) * L] = R(Rm.a[i][j].d[0]);
      rec[(er + 2 * NV) * L] = R(Rm.a[i][j].d[1]);
    }
    const size_t es = (size_t)(2 + 2 * NZ * NZ + i);
    rec[es * L] = R(src[i].v);
    rec[(es + NV) * L] = R(src[i].d[0]);
    rec[(es + 2 * NV) * L] = R(src[i].d[1]);
  }
}

template <int NZ, class R>
__global__ void __launch_bounds__(SCATTER_THREADS) scatter_kmatrix_kernel(ScatterArgs<R> a) {
  constexpr int NE = layer_record_k<NZ>(), NV = 2 * NZ * NZ + NZ, NS = adding_state_size<NZ>();
  const int L = a.L, Kmax = a.Kmax;
  const int p = blockIdx.y, gp = a.p_begin + p;
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= L || a.pv.status[p] != 0) return;
  const CloudyColumn c = column_inputs(a, p, gp, l);
  if (c.n_clouds == 0 && c.n_aerosols == 0) return;   // clear: the column kernel's Emission adjoint
  R* tod = a.TODc + (size_t)p * Kmax * L + l;
  R* pt = a.PT + (size_t)p * Kmax * L + l;
  double rad = 0.0, e_b = 0.0, Bs_b = 0.0;
  StreamSet<NZ, double> S;
  int code = stream_set<NZ, double>(c.nleg, c.mu_sensor, c.n_clouds > 0 ? a.lut.nleg : -1, c_gauss, S);
  if (!code) {
    const int nZ = S.nZ;
    auto rec_of = [&](int k) { return a.LB + ((size_t)p * Kmax + k) * NE * L + l; };
    auto layer = [&](int k, int* kind, double* od, Mat<NZ, double>& Tm, Mat<NZ, double>& Rm, double* src) {
      const R* rec = rec_of(k);
      *kind = (int)rec[0];
      *od = double(rec[(size_t)L]);
      if (*kind != 1) return;
      for (int i = 0; i < nZ; i++) {
        for (int j = 0; j < nZ; j++) {
          Tm.a[i][j] = double(rec[(size_t)(2 + i * NZ + j) * L]);
          Rm.a[i][j] = double(rec[(size_t)(2 + NZ * NZ + i * NZ + j) * L]);
        }
        src[i] = double(rec[(size_t)(2 + 2 * NZ * NZ + i) * L]);
      }
    };
    double* as = a.AS + (size_t)p * (Kmax + 1) * NS * L + l;
    auto state = [&](int lev, int i) -> double& { return as[((size_t)lev * NS + i) * L]; };
    auto contract = [&](int k, int kind, const Mat<NZ, double>& T_b, const Mat<NZ, double>& R_b,
                        const double* src_b, double od_b, double* g) {
      const R* rec = rec_of(k);
      if (kind != 1) {
        g[0] = od_b * double(rec[(size_t)(2 + 3 * NV) * L]);
        g[1] = od_b * double(rec[(size_t)(3 + 3 * NV) * L]);
        return true;
      }
      for (int d = 0; d < 2; d++) {
        const R* r = rec + (size_t)(2 + (1 + d) * NV) * L;
        double acc = 0.0;
        for (int i = 0; i < nZ; i++) {
          for (int j = 0; j < nZ; j++)
            acc += T_b.a[i][j] * double(r[(size_t)(i * NZ + j) * L]) +
                   R_b.a[i][j] * double(r[(size_t)(NZ * NZ + i * NZ + j) * L]);
          acc += src_b[i] * double(r[(size_t)(2 * NZ * NZ + i) * L]);
        }
        g[d] = acc;
      }
      return true;
    };
    auto out = [&](int k, double g, double t) {
      tod[(size_t)k * L] = R(g);
      pt[(size_t)k * L] = R(t);
    };
    code = cloudy_kmatrix<NZ>(c, S, layer, state, contract, out, &rad, &e_b, &Bs_b);
  }
  if (code) {
    atomicCAS(a.error, 0, code);
    if (a.status) atomicOr(a.status + gp, 1 << 4);
    rad = e_b = Bs_b = 0.0;
    for (int k = 0; k < c.Ku; k++) { tod[(size_t)k * L] = R(0); pt[(size_t)k * L] = R(0); }
  }
  double* cb = a.CB + (size_t)p * 3 * L + l;
  cb[0] = rad;
  cb[(size_t)L] = e_b;
  cb[2 * (size_t)L] = Bs_b;
}

}  // namespace crtm
