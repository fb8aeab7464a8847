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
// K-matrix and adjoint of scattering profiles.  After the first column launch
// and scatter_layers_kernel (the forward layer records):
//
//   scatter_kmatrix_kernel   one thread per (profile, channel): the adding
//                            from the surface with the level states kept in
//                            AS, then the adding adjoint from the top down.
//                            Writes each layer's record adjoints (LBA, FP64:
//                            kind, od_b, B_b, then T_b, R_b, src_b) and the
//                            cloudy radiance, its surface derivatives and the
//                            clear-column radiance of a fractional profile (CB).
//   scatter_soi_k_kernel     the same for the SOI profiles: the orders of
//                            interaction with their fields kept (FS), then
//                            their adjoint from the last order down.
//   scatter_contract_kernel  one thread per (profile, layer, channel): the
//                            layer optics on derivative numbers (gas optical
//                            depth, temperature, and each active cloud or
//                            aerosol's amount and radius), contracted with
//                            the record adjoints: dR/dtau (TODc), dR/dT at
//                            fixed gas optical depth (PT) and the species
//                            Jacobians (CJ, CR), all for a unit radiance seed.
//
// The second column launch mixes TODc, PT and CB with the clear column of a
// fractional profile, applies the Planck-inversion seed (SC) and maps dR/dtau
// onto the reference levels; scatter_species_kernel then applies the cover
// chain rule and SC to the species and cloud-fraction Jacobians, and
// species_k_out_kernel / species_ad_out_kernel write them out.
#pragma once

#include "odps_kernels.cuh"
#include "scatter_adjoint.cuh"

namespace crtm {

// Gauss angles and weights.  Internal linkage: every translation unit that
// launches scattering kernels holds its own copy, uploaded at init.
static __constant__ GaussTable c_gauss;

template <int NZ>
constexpr int layer_record() { return 2 + 2 * NZ * NZ + NZ; }
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
  const double* lut_chan;   // the sensor's channel-interpolated cloud tables (CloudChan; null: none)
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
  const double* aer_var;        // [P][NA][Kmax] Effective_Variance ('CMAQ'), or null (0)
  const double* rh;             // [P][Kmax] Relative_Humidity ('GOCART-GEOS5', 'NAAPS'), or null (0)
  double* FB;                   // SOI fields [n][2][2][Kmax+1][NZ][L], or null (K-matrix/adjoint:
                                // the orders' adjoint fields)
  double* FS;                   // SOI K-matrix/adjoint: [n][soi_slots][2][Kmax+1][NZ][L] order fields
  int soi_slots;
  const R* TAU;                 // [n][Kmax][L] gas layer optical depths
  R* LB;                        // [n][Kmax][NE][L] layer records (forward)
  R* LBK;                       // [n][Kmax][NE][L] layer records of the K-matrix / adjoint (the
                                // layer solver's T in loss form keeps FP32 records accurate)
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
  double* CB;                   // [n][4][L] radiance, dR/de, dR/d(surface Planck), clear radiance
  R* AS;                        // [n][Kmax+1][NS][L] adding states
  R* LBA;                       // [n][Kmax][NE][L] record adjoints
  // species Jacobians: slots 0..max_clouds-1 clouds, then aerosols
  int n_slots;                  // max_clouds + max_aerosols when requested, else 0
  double* CJ, *CR;              // [n][n_slots][Kmax][L] amount and radius
  double* CF;                   // [n][Kmax][L] cloud fraction, or null
  double* CV;                   // [n][n_slots][Kmax][L] aerosol effective variance ('CMAQ'), or null
  double* CH;                   // [n][Kmax][L] relative humidity ('GOCART-GEOS5', 'NAAPS'), or null
  double* TD;                   // [n][2][Kmax] d tcc / d cf, d tcc / d wc (fractional profiles)
  const R* SC;                  // [n][L] dBT/dR x seed (after the second column launch)
  // further RTSolution components: the layer kernel writes the layers'
  // optical depths and accumulates the scattering optical depth; the forward
  // solvers write the cloud cover, the clear column and the stream count
  // (the K-matrix kernels the stream count; the second column launch the rest)
  RtsExt x;
};

constexpr int SCATTER_THREADS = 128;

// The layer solver's arithmetic C is a template parameter of the layer and
// contraction kernels: double in the all-FP64 form, DD (double-float on the
// FP32 pipe: about 48 bits at a quarter of the cost of GB300's FP64) in the
// mixed form.

// Per profile, one warp each: the largest effective radius of its clouds and
// aerosols (stream rule input; clouds dropped by a fraction below 1e-12 do
// not count) and the total cloud cover of a fractional profile.
template <class R>
__global__ void scatter_profile_kernel(ScatterArgs<R> a) {
  const int p = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (p >= a.n_chunk) return;
  const int gp = batch_profile(a.b, a.p_begin + p), Ku = a.b.n_layers[gp];
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
    const int ov = a.overlap ? a.overlap[gp] : 4;
    const double* wc = nc > 0 ? a.wc + (size_t)gp * a.max_clouds * a.Kmax : nullptr;
    if (nc > 0) {
      tcc = total_cloud_cover(Ku, nc, cf, wc, (size_t)a.Kmax, ov);
      if (tcc < -1.5) {
        atomicCAS(a.error, 0, 11);
        if (a.status) atomicOr(a.status + gp, 1 << 4);
        tcc = -1.0;
      }
    }
    a.cover[p] = tcc;
    if (a.TD && tcc >= 0.0)
      cloud_cover_derivatives(Ku, nc, cf, wc, (size_t)a.Kmax, ov, tcc, a.TD + (size_t)p * 2 * a.Kmax,
                              a.TD + (size_t)p * 2 * a.Kmax + a.Kmax);
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
  c.aer_var = a.max_aerosols > 0 && a.aer_var ? a.aer_var + (size_t)gp * a.max_aerosols * a.Kmax : nullptr;
  c.rh = a.max_aerosols > 0 && a.rh ? a.rh + (size_t)gp * a.Kmax : nullptr;
  c.alut = &a.alut;
  c.cf = a.cloud_fraction && c.n_clouds > 0 ? a.cloud_fraction + (size_t)gp * a.Kmax : nullptr;
  c.zc.z = a.lut_chan;
  c.zc.L = (size_t)a.L;
  c.zc.ch = l;
  const double tcc = a.cover[p];
  c.wc_div = tcc > MIN_COVERAGE ? tcc : 1.0;
  return c;
}

template <int NZ, class R, class Rec, class C>
__global__ void __launch_bounds__(SCATTER_THREADS) scatter_layers_kernel(ScatterArgs<R> a, Rec* LBr) {
  constexpr int NE = layer_record<NZ>();
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int L = a.L, Kmax = a.Kmax;
  if (idx >= (long long)a.n_chunk * Kmax * L) return;
  const int l = (int)(idx % L);
  const int k = (int)((idx / L) % Kmax);
  const int p = (int)(idx / ((long long)L * Kmax));
  const int gp = batch_profile(a.b, a.p_begin + p);
  if (a.pv.status[p] != 0 || k >= a.b.n_layers[gp]) return;
  Rec* rec = LBr + ((size_t)p * Kmax + k) * NE * L + l;
  const CloudyColumn c = column_inputs(a, p, gp, l);
  if (c.n_clouds == 0 && c.n_aerosols == 0) return;
  StreamSet<NZ, double> S;
  if (int rc = stream_set<NZ, double>(c.nleg, c.mu_sensor, c.n_clouds > 0 ? a.lut.nleg : -1, c_gauss, S)) {
    rec[0] = Rec(-rc);
    return;
  }
  Mat<NZ, Rec> Tm, Rm;
  Rec src[NZ], od;
  const double gas = double(a.TAU[((size_t)p * Kmax + k) * L + l]);
  double bs = 0.0;
  const int kind = layer_optics<NZ, Rec, C>(c, a.lut, S, k, C(gas), C(c.temperature[k]), &od, Tm, Rm, src,
                                            NoSeed(), nullptr, a.x.sod ? &bs : nullptr);
  if (kind >= 0) {
    const size_t pl = (size_t)gp * L + l;
    if (a.x.lod) a.x.lod[pl * Kmax + k] = double(od);
    if (a.x.sod && bs > 0.0) atomicAdd(a.x.sod + pl, bs);
  }
  rec[0] = Rec(kind);
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

// The forward's further RTSolution components of pair pl (profile p of the
// chunk): total cloud cover and the clear column of a fractional profile;
// R_clear / Tb_clear the profile's own radiance where it has no clouds or
// its cover is below 1e-12 (CRTM_Forward_Module.f90:1086-1119); the stream
// count (CRTM_Forward_Module.f90:866-874).
template <class R>
__device__ void forward_rts_ext(const ScatterArgs<R>& a, const CloudyColumn& c, int p, int gp, size_t pl,
                                int code, double rad_clear) {
  const RtsExt& x = a.x;
  const double tcc = a.cover[p];
  const bool frac = tcc >= 0.0 && !code;
  if (x.tcc) x.tcc[pl] = frac ? tcc : 0.0;
  double rc = frac ? rad_clear : 0.0, bc = frac ? planck_temperature(c.c1, c.c2, c.b1, c.b2, rad_clear) : 0.0;
  if (!code && (c.n_clouds == 0 || (tcc >= 0.0 && tcc < MIN_COVERAGE))) {
    rc = a.radiance[pl];
    bc = a.bt[pl];
  }
  if (x.r_clear) x.r_clear[pl] = rc;
  if (x.tb_clear) x.tb_clear[pl] = bc;
  const int ns = a.n_streams ? a.n_streams[gp] : 0;
  if (x.nfs) x.nfs[pl] = (c.n_clouds > 0 || c.n_aerosols > 0) ? c.nleg + 2 : (ns > 0 ? ns + 2 : 0);
}

template <int NZ, class R>
__global__ void __launch_bounds__(SCATTER_THREADS) scatter_adding_kernel(ScatterArgs<R> a) {
  constexpr int NE = layer_record<NZ>();
  const int L = a.L, Kmax = a.Kmax;
  const int p = blockIdx.y, gp = batch_profile(a.b, a.p_begin + p);
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
  double rad = 0.0, rad_clear = 0.0;
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
      if (!code && tcc >= 0.0) {
        rad_clear = clear_column_radiance(c, tau, L);
        rad = (1.0 - tcc) * rad_clear + tcc * rad;
      }
    }
  }
  if (code) {
    atomicCAS(a.error, 0, code);
    if (a.status) atomicOr(a.status + gp, 1 << 4);
    rad = 0.0;
  }
  a.radiance[pl] = rad;
  a.bt[pl] = code ? 0.0 : planck_temperature(c.c1, c.c2, c.b1, c.b2, rad);
  forward_rts_ext(a, c, p, gp, pl, code, rad_clear);
}


// SOI profiles (Options%RT_Algorithm_Id = RT_SOI): successive orders of
// interaction over the layer records, fields in FB.
template <int NZ, class R>
__global__ void __launch_bounds__(SCATTER_THREADS) scatter_soi_kernel(ScatterArgs<R> a) {
  constexpr int NE = layer_record<NZ>();
  const int L = a.L, Kmax = a.Kmax;
  const int p = blockIdx.y, gp = batch_profile(a.b, a.p_begin + p);
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= L || a.pv.status[p] != 0) return;
  const CloudyColumn c = column_inputs(a, p, gp, l);
  if ((c.n_clouds == 0 && c.n_aerosols == 0) || !c.soi) return;
  const size_t pl = (size_t)gp * L + l;
  double rad = 0.0, rad_clear = 0.0;
  int code = 0;
  StreamSet<NZ, double> S;
  code = stream_set<NZ, double>(c.nleg, c.mu_sensor, c.n_clouds > 0 ? a.lut.nleg : -1, c_gauss, S);
  if (!code) {
    const int nZ = S.nZ;
    const R* rec0 = a.LB + (size_t)p * Kmax * NE * L + l;
    auto rec = [&](int k, int e) { return double(rec0[((size_t)k * NE + e) * L]); };
    auto lod = [&](int k, int* kind, double* od, double* B) {
      *kind = (int)rec(k, 0);
      *od = rec(k, 1);
      *B = c.c1 / (exp(c.c2 / (c.b1 + c.b2 * c.temperature[k])) - 1.0);
    };
    auto lsrc = [&](int k, double* src) {
      for (int i = 0; i < nZ; i++) src[i] = rec(k, 2 + 2 * NZ * NZ + i);
    };
    auto ltr = [&](int k, Mat<NZ, double>& Tm, Mat<NZ, double>& Rm) {
      for (int i = 0; i < nZ; i++)
        for (int j = 0; j < nZ; j++) {
          Tm.a[i][j] = rec(k, 2 + i * NZ + j);
          Rm.a[i][j] = rec(k, 2 + NZ * NZ + i * NZ + j);
        }
    };
    double* fb = a.FB + (size_t)p * 4 * (Kmax + 1) * NZ * L + l;
    auto fld = [&](int b, int f, int k, int i) -> double& {
      return fb[(((size_t)(2 * f + b) * (Kmax + 1) + k) * NZ + i) * L];
    };
    for (int k = 0; k < c.Ku && !code; k++)
      if ((int)rec(k, 0) < 0) code = -(int)rec(k, 0);
    if (!code)
      soi_solve<NZ>(nZ, c.Ku, S.isat, S.mu, c.emissivity, c.planck_surface, c.cosmic, lod, lsrc, ltr, fld, &rad);
    const double tcc = a.cover[p];
    if (!code && tcc >= 0.0) {
      rad_clear = clear_column_radiance(c, a.TAU + (size_t)p * Kmax * L + l, L);
      rad = (1.0 - tcc) * rad_clear + tcc * rad;
    }
  }
  if (code) {
    atomicCAS(a.error, 0, code);
    if (a.status) atomicOr(a.status + gp, 1 << 4);
    rad = 0.0;
  }
  a.radiance[pl] = rad;
  a.bt[pl] = code ? 0.0 : planck_temperature(c.c1, c.c2, c.b1, c.b2, rad);
  forward_rts_ext(a, c, p, gp, pl, code, rad_clear);
}

template <int NZ, class R>
__global__ void __launch_bounds__(SCATTER_THREADS) scatter_kmatrix_kernel(ScatterArgs<R> a) {
  constexpr int NE = layer_record<NZ>(), NS = adding_state_size<NZ>();
  const int L = a.L, Kmax = a.Kmax;
  const int p = blockIdx.y, gp = batch_profile(a.b, a.p_begin + p);
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= L || a.pv.status[p] != 0) return;
  const CloudyColumn c = column_inputs(a, p, gp, l);
  if (c.n_clouds == 0 && c.n_aerosols == 0) return;   // clear: the column kernel's Emission adjoint
  if (c.soi) return;                                   // scatter_soi_k_kernel
  if (a.x.nfs) a.x.nfs[(size_t)gp * L + l] = c.nleg + 2;
  double rad = 0.0, e_b = 0.0, Bs_b = 0.0;
  StreamSet<NZ, double> S;
  int code = stream_set<NZ, double>(c.nleg, c.mu_sensor, c.n_clouds > 0 ? a.lut.nleg : -1, c_gauss, S);
  if (!code) {
    const int nZ = S.nZ;
    auto layer = [&](int k, int* kind, double* od, Mat<NZ, R>& Tm, Mat<NZ, R>& Rm, R* src) {
      const R* rec = a.LBK + ((size_t)p * Kmax + k) * NE * L + l;
      *kind = (int)rec[0];
      *od = double(rec[(size_t)L]);
      if (*kind != 1) return;
      for (int i = 0; i < nZ; i++) {
        for (int j = 0; j < nZ; j++) {
          Tm.a[i][j] = rec[(size_t)(2 + i * NZ + j) * L];
          Rm.a[i][j] = rec[(size_t)(2 + NZ * NZ + i * NZ + j) * L];
        }
        src[i] = rec[(size_t)(2 + 2 * NZ * NZ + i) * L];
      }
    };
    R* as = a.AS + (size_t)p * (Kmax + 1) * NS * L + l;
    auto state = [&](int lev, int i) -> R& { return as[((size_t)lev * NS + i) * L]; };
    auto adj = [&](int k, int kind, const Mat<NZ, R>& T_b, const Mat<NZ, R>& R_b, const R* src_b,
                   double od_b, double B_b) {
      R* rb = a.LBA + ((size_t)p * Kmax + k) * NE * L + l;
      rb[0] = R(kind);
      rb[(size_t)L] = R(od_b);
      if (kind != 1) {
        rb[2 * (size_t)L] = R(B_b);
        return;
      }
      for (int i = 0; i < nZ; i++) {
        for (int j = 0; j < nZ; j++) {
          rb[(size_t)(2 + i * NZ + j) * L] = T_b.a[i][j];
          rb[(size_t)(2 + NZ * NZ + i * NZ + j) * L] = R_b.a[i][j];
        }
        rb[(size_t)(2 + 2 * NZ * NZ + i) * L] = src_b[i];
      }
    };
    code = cloudy_adjoint<NZ, decltype(layer), decltype(state), decltype(adj), R>(c, S, layer, state, adj, &rad,
                                                                                         &e_b, &Bs_b);
  }
  if (code) {
    atomicCAS(a.error, 0, code);
    if (a.status) atomicOr(a.status + gp, 1 << 4);
    rad = e_b = Bs_b = 0.0;
    for (int k = 0; k < c.Ku; k++) a.LBA[((size_t)p * Kmax + k) * NE * L + l] = R(-1.0);
  }
  double* cb = a.CB + (size_t)p * 4 * L + l;
  cb[0] = rad;
  cb[(size_t)L] = e_b;
  cb[2 * (size_t)L] = Bs_b;
  cb[3 * (size_t)L] = a.cover[p] >= 0.0 ? clear_column_radiance(c, a.TAU + (size_t)p * Kmax * L + l, L) : 0.0;
}

// K-matrix / adjoint of the SOI profiles (Options%RT_Algorithm_Id = RT_SOI),
// one thread per (profile, channel): the orders of interaction over the FP64
// layer records with every order's fields kept in FS (checkpoints and
// recomputation beyond soi_slots orders), then their adjoint from the last
// order down into the record adjoints (LBA) and CB, as scatter_kmatrix_kernel
// does for ADA.
template <int NZ>
__global__ void __launch_bounds__(SCATTER_THREADS) scatter_soi_k_kernel(ScatterArgs<double> a) {
  constexpr int NE = layer_record<NZ>();
  const int L = a.L, Kmax = a.Kmax;
  const int p = blockIdx.y, gp = batch_profile(a.b, a.p_begin + p);
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= L || a.pv.status[p] != 0) return;
  const CloudyColumn c = column_inputs(a, p, gp, l);
  if ((c.n_clouds == 0 && c.n_aerosols == 0) || !c.soi) return;
  if (a.x.nfs) a.x.nfs[(size_t)gp * L + l] = c.nleg + 2;
  double rad = 0.0, e_b = 0.0, Bs_b = 0.0;
  StreamSet<NZ, double> S;
  int code = stream_set<NZ, double>(c.nleg, c.mu_sensor, c.n_clouds > 0 ? a.lut.nleg : -1, c_gauss, S);
  const double* rec0 = a.LBK + (size_t)p * Kmax * NE * L + l;
  auto rec = [&](int k, int e) { return rec0[((size_t)k * NE + e) * L]; };
  for (int k = 0; k < c.Ku && !code; k++)
    if ((int)rec(k, 0) < 0) code = -(int)rec(k, 0);
  if (!code) {
    const int nZ = S.nZ;
    auto lod = [&](int k, int* kind, double* od, double* B) {
      *kind = (int)rec(k, 0);
      *od = rec(k, 1);
      *B = c.c1 / (exp(c.c2 / (c.b1 + c.b2 * c.temperature[k])) - 1.0);
    };
    auto lsrc = [&](int k, double* src) {
      for (int i = 0; i < nZ; i++) src[i] = rec(k, 2 + 2 * NZ * NZ + i);
    };
    auto ltr = [&](int k, Mat<NZ, double>& Tm, Mat<NZ, double>& Rm) {
      for (int i = 0; i < nZ; i++)
        for (int j = 0; j < nZ; j++) {
          Tm.a[i][j] = rec(k, 2 + i * NZ + j);
          Rm.a[i][j] = rec(k, 2 + NZ * NZ + i * NZ + j);
        }
    };
    const size_t lev = (size_t)NZ * L, fsz = (size_t)(Kmax + 1) * lev;
    double* fs = a.FS + (size_t)p * a.soi_slots * 2 * fsz + l;
    double* fb = a.FB + (size_t)p * 4 * fsz + l;
    auto fld = [&](int sl, int f, int k, int i) -> double& {
      return fs[(size_t)(2 * sl + f) * fsz + k * lev + (size_t)i * L];
    };
    auto lam = [&](int b, int f, int k, int i) -> double& {
      return fb[(size_t)(2 * b + f) * fsz + k * lev + (size_t)i * L];
    };
    double* rb = a.LBA + (size_t)p * Kmax * NE * L + l;
    auto ab = [&](int k, int e) -> double& { return rb[((size_t)k * NE + e) * L]; };
    code = soi_adjoint<NZ>(nZ, c.Ku, S.isat, S.mu, c.emissivity, c.planck_surface, c.cosmic, a.soi_slots, lod, lsrc,
                           ltr, fld, lam, ab, &rad, &e_b, &Bs_b);
  }
  if (code) {
    atomicCAS(a.error, 0, code);
    if (a.status) atomicOr(a.status + gp, 1 << 4);
    rad = e_b = Bs_b = 0.0;
    for (int k = 0; k < c.Ku; k++) a.LBA[((size_t)p * Kmax + k) * NE * L + l] = -1.0;
  }
  double* cb = a.CB + (size_t)p * 4 * L + l;
  cb[0] = rad;
  cb[(size_t)L] = e_b;
  cb[2 * (size_t)L] = Bs_b;
  cb[3 * (size_t)L] = a.cover[p] >= 0.0 ? clear_column_radiance(c, a.TAU + (size_t)p * Kmax * L + l, L) : 0.0;
}

// Active species of layer k (clouds above the water-content threshold after
// the cover scaling and not dropped, aerosols above theirs for non-microwave
// sensors), as seed indices of layer_optics.
CRTM_HD int active_species(const CloudyColumn& c, int k, int* sp) {
  int n = 0;
  if (!(c.cf && c.cf[k] < MIN_COVERAGE))
    for (int i = 0; i < c.n_clouds; i++)
      if (c.wc[i * c.cstride + k] / c.wc_div > WATER_CONTENT_THRESHOLD) sp[n++] = i;
  if (!c.microwave)
    for (int i = 0; i < c.n_aerosols; i++)
      if (c.conc[i * c.cstride + k] > AEROSOL_CONTENT_THRESHOLD) sp[n++] = c.n_clouds + i;
  return n;
}

template <int NZ, class R, class C>
__global__ void __launch_bounds__(SCATTER_THREADS) scatter_contract_kernel(ScatterArgs<R> a) {
  constexpr int NE = layer_record<NZ>();
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int L = a.L, Kmax = a.Kmax;
  if (idx >= (long long)a.n_chunk * Kmax * L) return;
  const int l = (int)(idx % L);
  const int k = (int)((idx / L) % Kmax);
  const int p = (int)(idx / ((long long)L * Kmax));
  const int gp = batch_profile(a.b, a.p_begin + p);
  if (a.pv.status[p] != 0 || k >= a.b.n_layers[gp]) return;
  const CloudyColumn c = column_inputs(a, p, gp, l);
  if (c.n_clouds == 0 && c.n_aerosols == 0) return;
  if (!c.soi) return;   // ADA profiles: scatter_reverse_kernel
  const size_t kl = ((size_t)p * Kmax + k) * L + l;
  auto slot = [&](int s) { return s < c.n_clouds ? s : a.max_clouds + (s - c.n_clouds); };
  if (a.n_slots > 0)
    for (int s = 0; s < a.n_slots; s++) {
      a.CJ[((size_t)p * a.n_slots + s) * Kmax * L + (size_t)k * L + l] = 0.0;
      a.CR[((size_t)p * a.n_slots + s) * Kmax * L + (size_t)k * L + l] = 0.0;
      if (a.CV) a.CV[((size_t)p * a.n_slots + s) * Kmax * L + (size_t)k * L + l] = 0.0;
    }
  const double* rb = a.LBA + ((size_t)p * Kmax + k) * NE * L + l;
  const int kind = (int)rb[0];
  if (kind < 0) {
    a.TODc[kl] = R(0);
    a.PT[kl] = R(0);
    return;
  }
  StreamSet<NZ, double> S;
  if (stream_set<NZ, double>(c.nleg, c.mu_sensor, c.n_clouds > 0 ? a.lut.nleg : -1, c_gauss, S)) return;
  const int nZ = S.nZ;
  Mat<NZ, double> T_b, R_b;
  double src_b[NZ];
  const double od_b = rb[(size_t)L], B_b = kind == 1 ? 0.0 : rb[2 * (size_t)L];
  if (kind == 1)
    for (int i = 0; i < nZ; i++) {
      for (int j = 0; j < nZ; j++) {
        T_b.a[i][j] = rb[(size_t)(2 + i * NZ + j) * L];
        R_b.a[i][j] = rb[(size_t)(2 + NZ * NZ + i * NZ + j) * L];
      }
      src_b[i] = rb[(size_t)(2 + 2 * NZ * NZ + i) * L];
    }
  const double gas = double(a.TAU[kl]);
  int sp[2 * SC_NC_MAX];
  const int nsp = a.n_slots > 0 ? active_species(c, k, sp) : 0;
  double g[4];
  int done = 0;
  if (nsp == 0) {
    const LayerDirections d{true, 0, {0, 0, 0, 0}};
    layer_contract<NZ, 2, C>(c, a.lut, S, k, gas, d, T_b, R_b, src_b, od_b, B_b, g);
  } else {   // gas, temperature and the first species in one pass
    const LayerDirections d{true, 1, {sp[0], 0, 0, 0}};
    layer_contract<NZ, 4, C>(c, a.lut, S, k, gas, d, T_b, R_b, src_b, od_b, B_b, g);
    const size_t o = ((size_t)p * a.n_slots + slot(sp[0])) * Kmax * L + (size_t)k * L + l;
    a.CJ[o] = g[2];
    a.CR[o] = g[3];
    done = 1;
  }
  a.TODc[kl] = R(g[0]);
  a.PT[kl] = R(g[1]);
  while (done < nsp) {   // two more species per pass
    const int m = nsp - done >= 2 ? 2 : 1;
    const LayerDirections d{false, m, {sp[done], m == 2 ? sp[done + 1] : 0, 0, 0}};
    layer_contract<NZ, 4, C>(c, a.lut, S, k, gas, d, T_b, R_b, src_b, od_b, B_b, g);
    for (int i = 0; i < m; i++) {
      const size_t o = ((size_t)p * a.n_slots + slot(sp[done + i])) * Kmax * L + (size_t)k * L + l;
      a.CJ[o] = g[2 * i];
      a.CR[o] = g[2 * i + 1];
    }
    done += m;
  }
  if (a.CV && a.alut.scheme == AEROSOL_CMAQ) {   // the aerosols' effective variance, four per pass
    int av[2 * SC_NC_MAX], nav = 0;
    for (int i = 0; i < nsp; i++)
      if (sp[i] >= c.n_clouds) av[nav++] = sp[i];
    for (int i0 = 0; i0 < nav; i0 += 4) {
      const int m = nav - i0 < 4 ? nav - i0 : 4;
      LayerDirections d{false, m, {av[i0], m > 1 ? av[i0 + 1] : 0, m > 2 ? av[i0 + 2] : 0, m > 3 ? av[i0 + 3] : 0}};
      d.second = true;
      layer_contract<NZ, 4, C>(c, a.lut, S, k, gas, d, T_b, R_b, src_b, od_b, B_b, g);
      for (int i = 0; i < m; i++)
        a.CV[((size_t)p * a.n_slots + slot(av[i0 + i])) * Kmax * L + (size_t)k * L + l] = g[i];
    }
  }
}

// The same contraction for the ADA profiles (and the clear layers of any
// profile not on SOI), one thread per (profile, layer, channel), by the
// reverse sweep through the layer's optics (layer_adjoint): all of the
// layer's inputs in one pass, in the arithmetic C.
// (FP32 sweep with 10 angles: 3 CTAs per SM, 168 registers, measured 8 %
// faster than the register-limited 2; the 5-angle sweep is fastest at 2)
template <int NZ, class R, class C>
__global__ void __launch_bounds__(SCATTER_THREADS, (NZ > 5 && sizeof(C) == 4) ? 3 : 1)
    scatter_reverse_kernel(ScatterArgs<R> a) {
  constexpr int NE = layer_record<NZ>();
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int L = a.L, Kmax = a.Kmax;
  if (idx >= (long long)a.n_chunk * Kmax * L) return;
  const int l = (int)(idx % L);
  const int k = (int)((idx / L) % Kmax);
  const int p = (int)(idx / ((long long)L * Kmax));
  const int gp = batch_profile(a.b, a.p_begin + p);
  if (a.pv.status[p] != 0 || k >= a.b.n_layers[gp]) return;
  const CloudyColumn c = column_inputs(a, p, gp, l);
  if (c.n_clouds == 0 && c.n_aerosols == 0) return;
  if (c.soi) return;    // SOI profiles: scatter_contract_kernel
  const size_t kl = ((size_t)p * Kmax + k) * L + l;
  auto slot = [&](int s) { return s < c.n_clouds ? s : a.max_clouds + (s - c.n_clouds); };
  auto jac = [&](double* X, int s) -> double& {
    return X[((size_t)p * a.n_slots + s) * Kmax * L + (size_t)k * L + l];
  };
  if (a.n_slots > 0)
    for (int s = 0; s < a.n_slots; s++) {
      jac(a.CJ, s) = 0.0;
      jac(a.CR, s) = 0.0;
      if (a.CV) jac(a.CV, s) = 0.0;
    }
  const R* rb = a.LBA + ((size_t)p * Kmax + k) * NE * L + l;
  const int kind = (int)rb[0];
  if (kind < 0) {
    a.TODc[kl] = R(0);
    a.PT[kl] = R(0);
    return;
  }
  StreamSet<NZ, double> S;
  if (stream_set<NZ, double>(c.nleg, c.mu_sensor, c.n_clouds > 0 ? a.lut.nleg : -1, c_gauss, S)) return;
  const int nZ = S.nZ;
  Mat<NZ, double> T_b, R_b;
  double src_b[NZ];
  const double od_b = double(rb[(size_t)L]), B_b = kind == 1 ? 0.0 : double(rb[2 * (size_t)L]);
  if (kind == 1)
    for (int i = 0; i < nZ; i++) {
      for (int j = 0; j < nZ; j++) {
        T_b.a[i][j] = double(rb[(size_t)(2 + i * NZ + j) * L]);
        R_b.a[i][j] = double(rb[(size_t)(2 + NZ * NZ + i * NZ + j) * L]);
      }
      src_b[i] = double(rb[(size_t)(2 + 2 * NZ * NZ + i) * L]);
    }
  double g[2], gs[2 * SC_NC_MAX][3];
  const int kr = layer_adjoint<NZ, C>(c, a.lut, S, k, double(a.TAU[kl]), kind, T_b, R_b, src_b,
                                      kind == 1 ? 0.0 : od_b, B_b, g, gs);
  if (kr < 0) {
    atomicCAS(a.error, 0, -kr);
    if (a.status) atomicOr(a.status + gp, 1 << 4);
    a.TODc[kl] = R(0);
    a.PT[kl] = R(0);
    return;
  }
  a.TODc[kl] = R(g[0]);
  a.PT[kl] = R(g[1]);
  if (a.n_slots > 0) {
    const int nsp = c.n_clouds + (c.microwave ? 0 : c.n_aerosols);
    for (int s = 0; s < nsp; s++) {
      jac(a.CJ, slot(s)) = gs[s][0];
      jac(a.CR, slot(s)) = gs[s][1];
      if (a.CV && a.alut.scheme == AEROSOL_CMAQ && s >= c.n_clouds) jac(a.CV, slot(s)) = gs[s][2];
    }
  }
}

// Species and cloud-fraction Jacobians of one (profile, channel), in place:
// a fractional profile's radiance is (1 - tcc) R_clear + tcc R_cloudy(wc / tcc),
// so d/dwc = dRc/dwc' + dR/dtcc dtcc/dwc, d/dradius and the aerosols' = tcc dRc,
// d/dcf = dR/dtcc dtcc/dcf with dR/dtcc = Rc - R_clear - sum(wc dRc/dwc') / tcc;
// then x SC (dBT/dR x seed).
template <class R>
__global__ void scatter_species_kernel(ScatterArgs<R> a) {
  const int L = a.L, Kmax = a.Kmax;
  const int p = blockIdx.y, gp = batch_profile(a.b, a.p_begin + p);
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= L) return;
  const int Ku = a.b.n_layers[gp];
  const int nc = a.max_clouds > 0 ? a.n_clouds[gp] : 0, na = a.max_aerosols > 0 ? a.n_aerosols[gp] : 0;
  const bool live = a.pv.status[p] == 0 && (nc > 0 || na > 0);
  const double sc = live ? double(a.SC[(size_t)p * L + l]) : 0.0;
  const double tcc = live ? a.cover[p] : -1.0;
  const double w = tcc < 0.0 ? 1.0 : tcc;
  const double* wc = nc > 0 ? a.wc + (size_t)gp * a.max_clouds * Kmax : nullptr;
  const double* cf = a.cloud_fraction && nc > 0 ? a.cloud_fraction + (size_t)gp * Kmax : nullptr;
  auto J = [&](double* X, int s, int k) -> double& {
    return X[((size_t)p * a.n_slots + s) * Kmax * L + (size_t)k * L + l];
  };
  double dtcc = 0.0;   // dR/dtcc
  if (tcc >= 0.0) {
    const double* cb = a.CB + (size_t)p * 4 * L + l;
    dtcc = cb[0] - cb[3 * (size_t)L];
    if (tcc > MIN_COVERAGE) {
      double sum = 0.0;
      for (int c = 0; c < nc; c++)
        for (int k = 0; k < Ku; k++) sum += wc[(size_t)c * Kmax + k] * J(a.CJ, c, k);
      dtcc -= sum / tcc;
    }
  }
  const double* dcf = tcc >= 0.0 && a.TD ? a.TD + (size_t)p * 2 * Kmax : nullptr;
  // GOCART-GEOS5 / NAAPS: an aerosol's second slot holds its lookup's RH
  // derivative; the layer's RH Jacobian is their sum, the radius one is zero
  const bool rh_slots = a.max_aerosols > 0 && a.alut.scheme >= AEROSOL_GOCART;
  for (int s = 0; s < a.n_slots; s++) {
    const bool cloud = s < a.max_clouds;
    for (int k = 0; k < Kmax; k++) {
      double& x = J(a.CJ, s, k);
      double& r = J(a.CR, s, k);
      double* v2 = a.CV ? &J(a.CV, s, k) : nullptr;
      if (k >= Ku || !live) {
        x = r = 0.0;
        if (v2) *v2 = 0.0;
        continue;
      }
      if (cloud) {
        double v = x;
        const double wk = s < nc ? wc[(size_t)s * Kmax + k] : 0.0;
        if (dcf && wk > WATER_CONTENT_THRESHOLD && !(cf && cf[k] < MIN_COVERAGE)) v += dtcc * dcf[Kmax + k];
        x = sc * v;
        r = sc * w * r;
      } else {
        x = sc * w * x;
        r = sc * w * r;
        if (v2) *v2 = sc * w * *v2;
      }
    }
  }
  if (a.CH)
    for (int k = 0; k < Kmax; k++) {
      double h = 0.0;
      for (int s = a.max_clouds; s < a.n_slots && rh_slots; s++) h += J(a.CR, s, k);
      a.CH[((size_t)p * Kmax + k) * L + l] = h;
    }
  if (rh_slots)
    for (int s = a.max_clouds; s < a.n_slots; s++)
      for (int k = 0; k < Kmax; k++) J(a.CR, s, k) = 0.0;
  if (a.CF)
    for (int k = 0; k < Kmax; k++)
      a.CF[((size_t)p * Kmax + k) * L + l] = (live && dcf && k < Ku) ? sc * dtcc * dcf[k] : 0.0;
}

// K-matrix outputs of the species Jacobians: X[n][S][Kmax][L] slots s0..s0+ns-1
// to out[P][L][ns][Kmax] (a shared-memory transpose of 32 x 32 tiles).
static __global__ void species_k_out_kernel(const double* X, int S, int s0, int ns, int Kmax, int L, int p_begin,
                                     int n, double* out, const int* perm) {
  __shared__ double tile[32][33];
  const int k0 = blockIdx.y * 32, l0 = blockIdx.x * 32;
  for (int ps = blockIdx.z; ps < n * ns; ps += gridDim.z) {
    const int p = ps / ns, s = ps % ns;
    const double* in = X + ((size_t)p * S + s0 + s) * Kmax * L;
    __syncthreads();
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
      const int k = k0 + i, l = l0 + threadIdx.x;
      tile[i][threadIdx.x] = (k < Kmax && l < L) ? in[(size_t)k * L + l] : 0.0;
    }
    __syncthreads();
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
      const int l = l0 + i, k = k0 + threadIdx.x;
      const size_t gp = perm ? perm[p_begin + p] : p_begin + p;
      if (l < L && k < Kmax) out[((gp * L + l) * ns + s) * Kmax + k] = tile[threadIdx.x][i];
    }
  }
}

// Adjoint outputs: out[P][ns][Kmax] = sum over channels of slots s0..s0+ns-1
// (one warp per row, lanes over channels).
static __global__ void species_ad_out_kernel(const double* X, int S, int s0, int ns, int Kmax, int L, int p_begin,
                                      int n, double* out, const int* perm) {
  const long long row = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (row >= (long long)n * ns * Kmax) return;
  const int k = (int)(row % Kmax), s = (int)((row / Kmax) % ns), p = (int)(row / ((long long)Kmax * ns));
  const double* in = X + (((size_t)p * S + s0 + s) * Kmax + k) * L;
  double acc = 0.0;
  for (int l = lane; l < L; l += 32) acc += in[l];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(FULL, acc, o);
  const size_t gp = perm ? perm[p_begin + p] : p_begin + p;
  if (lane == 0) out[(gp * ns + s) * Kmax + k] = acc;
}

// Zero rows of `row` doubles of out for the batch profiles perm[0..n-1] (the
// scattering Jacobians of a bucket's clear profiles).
static __global__ void zero_profile_rows_kernel(double* out, const int* perm, int n, size_t row) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (size_t)n * row) return;
  out[(size_t)perm[i / row] * row + i % row] = 0.0;
}

}  // namespace crtm
