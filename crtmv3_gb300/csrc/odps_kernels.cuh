// CUDA kernels of the clear-sky ODPS + Emission forward / K-matrix / adjoint path.
//
// A batch is processed in chunks of profiles.  Per chunk:
//   prep_kernel        one thread per profile: Map_Input, predictors X, partials D
//   absorb_fwd_kernel  one thread per (channel, NP profiles): OD(k) = sum C*X
//                      (ODPS_AtmAbsorption.f90:169-208), reference-layer ODs
//   column_kernel      one thread per (profile, channel): clamp, path, level
//                      interpolation (ODPS_AtmAbsorption.f90:213-254), Planck,
//                      Emission forward (Emission_Module.f90:54-174), Planck
//                      inversion, and for K/AD the Emission adjoint
//                      (Emission_Module.f90:280-395) and the optical-depth
//                      path adjoint (ODPS_AtmAbsorption.f90:487-540)
//   absorb_ad_kernel   one thread per (channel, NP profiles): contraction of
//                      the coefficients with the predictor partials and the
//                      reverse running sums (ODPS_AtmAbsorption.f90:543-598 +
//                      ODPS_Predictor.f90:1783-2643)
//   map_kernel         Map_Input adjoint to user layers (ODPS_CoordinateMapping.f90:480-547)
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>
#include <utility>

#include "odps_prep.cuh"

namespace crtm {

// (slot, variable) pattern of the partial-derivative table as device constants.
#define CRTM_PD_QCODES_MEMBERS(G)                                                       \
  static constexpr int QA0 = qA<G>(0), QA1 = qA<G>(1), QA2 = qA<G>(2), QA3 = qA<G>(3),  \
                       QA4 = qA<G>(4), QA5 = qA<G>(5);                                  \
  static constexpr int QTZ = qTz<G>(), QTZP = qTzp<G>();                                \
  static constexpr int QGAZP0 = qGazp<G>(0), QGAZP1 = qGazp<G>(1), QGAZP2 = qGazp<G>(2), \
                       QGAZP3 = qGazp<G>(3), QGAZP4 = qGazp<G>(4), QGAZP5 = qGazp<G>(5); \
  static constexpr int QGATZP0 = qGatzp<G>(0), QGATZP3 = qGatzp<G>(3), QGATZP5 = qGatzp<G>(5);

#define CRTM_PD_SLOT(slot, q, expr) slot,
#define CRTM_PD_VAR(slot, q, expr) q,

template <int G> struct PdTab;
template <> struct PdTab<1> {
  CRTM_PD_QCODES_MEMBERS(1)
  static constexpr int n = PD_NNZ_G1;
  static constexpr int slot[PD_NNZ_G1] = {PD_ENTRIES_G1(CRTM_PD_SLOT)};
  static constexpr int q[PD_NNZ_G1] = {PD_ENTRIES_G1(CRTM_PD_VAR)};
};
template <> struct PdTab<2> {
  CRTM_PD_QCODES_MEMBERS(2)
  static constexpr int n = PD_NNZ_G2;
  static constexpr int slot[PD_NNZ_G2] = {PD_ENTRIES_G2(CRTM_PD_SLOT)};
  static constexpr int q[PD_NNZ_G2] = {PD_ENTRIES_G2(CRTM_PD_VAR)};
};
template <> struct PdTab<3> {
  CRTM_PD_QCODES_MEMBERS(3)
  static constexpr int n = PD_NNZ_G3;
  static constexpr int slot[PD_NNZ_G3] = {PD_ENTRIES_G3(CRTM_PD_SLOT)};
  static constexpr int q[PD_NNZ_G3] = {PD_ENTRIES_G3(CRTM_PD_VAR)};
};

// Component of slot s (evaluated at compile time only).
template <int G>
constexpr int slot_component(int s) {
  int j = 0;
  while (j + 1 < Group<G>::J && Group<G>::OFF[j + 1] <= s) j++;
  return j;
}

// Compile-time loop: f(std::integral_constant<int, i>) for i = 0..N-1.
template <class F, int... Is>
__device__ __forceinline__ void static_for_impl(F&& f, std::integer_sequence<int, Is...>) {
  (f(std::integral_constant<int, Is>{}), ...);
}
template <int N, class F>
__device__ __forceinline__ void static_for(F&& f) {
  static_for_impl(f, std::make_integer_sequence<int, N>{});
}

// ---------------------------------------------------------------------------
// Device views
// ---------------------------------------------------------------------------
struct BatchView {
  int n_profiles, max_layers, n_abs;
  const int* n_layers;
  const double* level_pressure;
  const double* pressure;
  const double* temperature;
  const double* absorber;
  const double* land_cov, *water_cov, *snow_cov, *ice_cov;
  const double* land_t, *water_t, *snow_t, *ice_t;
  const double* zenith;
  const double* altitude;
  const double* emissivity;
};

struct SpecView {
  const double* c1, *c2, *b1, *b2, *cbr;
};

template <class R>
struct PrepView {
  R* X;
  R* D;
  double* T;
  double* A;
  unsigned char* amask;
  int* band_i0;
  int* band_n;
  double* band_w;
  int* ulev_k1;
  int* ulev_k2;
  double* ulev_fac;
  int* ulay_k0;
  int* ulay_k1;
  double* scal;
  int* status;
  int K, NS, NNZ, Jm, Kmax;

  __device__ ProfileOut<R> profile(int p) const {
    ProfileOut<R> o;
    o.X = X + (size_t)p * K * NS;
    o.D = D ? D + (size_t)p * K * NNZ : nullptr;
    o.T = T + (size_t)p * K;
    o.A = A + (size_t)p * Jm * K;
    o.amask = amask + (size_t)p * Jm * K;
    o.band_i0 = band_i0 + (size_t)p * K;
    o.band_n = band_n + (size_t)p * K;
    o.band_w = band_w + (size_t)p * K * MAX_BAND;
    o.ulev_k1 = ulev_k1 + (size_t)p * (Kmax + 1);
    o.ulev_k2 = ulev_k2 + (size_t)p * (Kmax + 1);
    o.ulev_fac = ulev_fac + (size_t)p * (Kmax + 1);
    o.ulay_k0 = ulay_k0 + (size_t)p * Kmax;
    o.ulay_k1 = ulay_k1 + (size_t)p * Kmax;
    o.scal = scal + (size_t)p * 4;
    o.status = status + p;
    return o;
  }
};

// ---------------------------------------------------------------------------
// 1. prep
// ---------------------------------------------------------------------------
template <int G, class R>
__global__ void prep_kernel(SensorTables S, BatchView b, PrepView<R> pv, const int* idx_map,
                            int p_begin, int n_chunk) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n_chunk) return;
  const int gp = p_begin + p;
  ProfileIn in;
  in.n_layers = b.n_layers[gp];
  in.n_abs = b.n_abs;
  in.level_pressure = b.level_pressure + (size_t)gp * (b.max_layers + 1);
  in.pressure = b.pressure + (size_t)gp * b.max_layers;
  in.temperature = b.temperature + (size_t)gp * b.max_layers;
  in.absorber = b.absorber + (size_t)gp * b.n_abs * b.max_layers;
  in.abs_stride = b.max_layers;
  in.idx_map = idx_map;
  in.zenith_deg = b.zenith[gp];
  in.surface_altitude = b.altitude ? b.altitude[gp] : 0.0;
  if (in.n_layers > b.max_layers) {
    pv.status[p] = ST_BAD_LAYERS;
    return;
  }
  prep_profile<G, R>(S, in, pv.profile(p));
}

// ---------------------------------------------------------------------------
// 2. absorption forward: OD[p][k][l] = sum_s C[k][s][l] * X[p][k][s]
// ---------------------------------------------------------------------------
template <int G, class R, int NP>
__global__ void __launch_bounds__(128) absorb_fwd_kernel(int K, int L, int n_chunk,
                                                         const float* __restrict__ C,
                                                         const unsigned* __restrict__ cmask,
                                                         const R* __restrict__ X,
                                                         R* __restrict__ OD) {
  constexpr int NS = Group<G>::NS, J = Group<G>::J;
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  const int p0 = blockIdx.y * NP;
  const bool active = l < L;
  const unsigned wmask = __reduce_or_sync(0xffffffffu, active ? cmask[l] : 0u);
  const int lc = active ? l : 0;
  const R* Xp[NP];
#pragma unroll
  for (int p = 0; p < NP; p++) Xp[p] = X + (size_t)min(p0 + p, n_chunk - 1) * K * NS;
  for (int k = 0; k < K; k++) {
    R acc[NP];
#pragma unroll
    for (int p = 0; p < NP; p++) acc[p] = R(0);
    const float* Ck = C + (size_t)k * NS * L + lc;
    static_for<J>([&](auto jc) {
      constexpr int j = decltype(jc)::value;
      constexpr int s0 = Group<G>::OFF[j], s1 = Group<G>::OFF[j + 1];
      if (!(wmask & (1u << j))) return;
#pragma unroll
      for (int s = s0; s < s1; s++) {
        const R c = R(__ldg(Ck + (size_t)s * L));
#pragma unroll
        for (int p = 0; p < NP; p++) acc[p] += c * __ldg(Xp[p] + (size_t)k * NS + s);
      }
    });
    if (active) {
#pragma unroll
      for (int p = 0; p < NP; p++)
        if (p0 + p < n_chunk) OD[((size_t)(p0 + p) * K + k) * L + l] = acc[p];
    }
  }
}

// ---------------------------------------------------------------------------
// 3. per-(profile, channel) column: path, interpolation, Emission, Planck.
// mode 0: forward; 1: K-matrix; 2: adjoint.
// ---------------------------------------------------------------------------
template <class R>
struct ColumnArgs {
  int K, L, Kmax, p_begin, n_chunk, mode;
  BatchView b;
  SpecView sp;
  PrepView<R> pv;
  R* OD;                  // [n_chunk][K][L] in: reference ODs, out (K/AD): OD adjoint
  R* TAU, *RD, *RU, *TODAD, *BAD;  // [n_chunk][Kmax][L] scratch
  const double* seed;     // [P][L] or null (=1)
  double* radiance, *bt;  // [P][L]
  double* kt;             // K-matrix: [P][L][Kmax] (Planck part); adjoint: PT scratch [n_chunk][Kmax][L]
  double* tsk, *ek;       // [P][L] (adjoint: [n_chunk][L] scratch for tsk)
  int* status;            // [P] or null
};

template <class R>
__device__ __forceinline__ R clamp_od(R v) {
  return v < R(0) ? R(0) : (v > R(MAX_OD) ? R(MAX_OD) : v);
}

template <class R>
__global__ void __launch_bounds__(256) column_kernel(ColumnArgs<R> a) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)a.n_chunk * a.L) return;
  const int p = (int)(idx / a.L), l = (int)(idx % a.L);
  const int gp = a.p_begin + p;
  const int K = a.K, L = a.L, Kmax = a.Kmax;
  const int st = a.pv.status[p];
  if (a.status && l == 0) a.status[gp] = st;
  const int Ku = a.b.n_layers[gp];
  const size_t pl = (size_t)gp * L + l;
  if (st != 0) {
    a.radiance[pl] = 0.0;
    a.bt[pl] = 0.0;
    return;
  }
  const double* sc = a.pv.scal + (size_t)p * 4;
  const double sec_sfc = sc[0], u = sc[1];
  const R ru = R(u), rsd = R(1.0 / u);
  const R rsec = R(sec_sfc);
  const R c1 = R(a.sp.c1[l]), c2 = R(a.sp.c2[l]), b1 = R(a.sp.b1[l]), b2 = R(a.sp.b2[l]);
  const double* tu = a.b.temperature + (size_t)gp * Kmax;
  const double ts = a.b.land_cov[gp] * a.b.land_t[gp] + a.b.water_cov[gp] * a.b.water_t[gp] +
                    a.b.snow_cov[gp] * a.b.snow_t[gp] + a.b.ice_cov[gp] * a.b.ice_t[gp];
  const double e = a.b.emissivity[pl];
  const R re = R(e), rr = R(1.0 - e);
  const R Bs = planck_radiance<R>(c1, c2, b1, b2, R(ts));
  const int* k1 = a.pv.ulev_k1 + (size_t)p * (Kmax + 1);
  const int* k2 = a.pv.ulev_k2 + (size_t)p * (Kmax + 1);
  const double* fac = a.pv.ulev_fac + (size_t)p * (Kmax + 1);
  R* od = a.OD + (size_t)p * K * L + l;
  const size_t cs = (size_t)p * Kmax * L + l;   // column scratch base, stride L

  // sweep 1 (top -> surface): user-level OD path, layer ODs, downwelling
  R cur = R(0), up_prev = R(0), rad_down = R(a.sp.cbr[l]);
  R src = R(0), tr = R(1);   // forward-only accumulation of the TOA radiance
  int lvl = 0;
  for (int i = 0; i <= Ku; i++) {
    const int ka = k1[i], kb = k2[i];
    while (lvl < ka) { cur += clamp_od(od[(size_t)lvl * L]); lvl++; }
    R upi = cur;
    if (kb != ka) {
      const R yb = cur + clamp_od(od[(size_t)ka * L]);
      upi = cur + (yb - cur) * R(fac[i]);
    }
    if (i > 0) {
      const int ku = i - 1;
      const R tau = (upi - up_prev) / rsec;
      const R B = planck_radiance<R>(c1, c2, b1, b2, R(tu[ku]));
      const R d = exp(-tau * rsd);
      if (a.mode == 0) {
        const R t = exp(-tau / ru);
        src += tr * B * (R(1) - t);
        tr *= t;
      } else {
        a.TAU[cs + (size_t)ku * L] = tau;
        a.RD[cs + (size_t)ku * L] = rad_down;
      }
      rad_down = rad_down * d + B * (R(1) - d);
    }
    up_prev = upi;
  }
  R rad_toa;
  if (a.mode == 0) {
    rad_toa = src + tr * (re * Bs + rr * rad_down);
  } else {
    // sweep 2 (surface -> top): upwelling radiance
    R rad_up = re * Bs + rr * rad_down;
    for (int ku = Ku - 1; ku >= 0; ku--) {
      const R tau = a.TAU[cs + (size_t)ku * L];
      const R t = exp(-tau / ru);
      const R B = planck_radiance<R>(c1, c2, b1, b2, R(tu[ku]));
      a.RU[cs + (size_t)ku * L] = rad_up;
      rad_up = rad_up * t + B * (R(1) - t);
    }
    rad_toa = rad_up;
  }
  const double Rd = double(rad_toa);
  const double Td = planck_temperature(a.sp.c1[l], a.sp.c2[l], a.sp.b1[l], a.sp.b2[l], Rd);
  a.radiance[pl] = Rd;
  a.bt[pl] = Td;
  if (a.mode == 0) return;

  // Adjoint: Pre_Process_RTSolution_K (Planck inversion adjoint), then Emission_AD
  const double seed = a.seed ? a.seed[pl] : 1.0;
  R up_ad = R(planck_temperature_dR(a.sp.c1[l], a.sp.c2[l], a.sp.b1[l], a.sp.b2[l], Rd) * seed);
  // sweep 3 (top -> surface): upwelling part
  for (int ku = 0; ku < Ku; ku++) {
    const R tau = a.TAU[cs + (size_t)ku * L];
    const R t = exp(-tau / ru);
    const R B = planck_radiance<R>(c1, c2, b1, b2, R(tu[ku]));
    R a_ad = a.RU[cs + (size_t)ku * L] * t * up_ad;
    const R src_ad = up_ad;
    up_ad = up_ad * t;
    a_ad -= B * t * src_ad;
    a.TODAD[cs + (size_t)ku * L] = -a_ad / ru;
    a.BAD[cs + (size_t)ku * L] = src_ad * (R(1) - t);
  }
  const R e_ad = up_ad * Bs;
  const R bs_ad = re * up_ad;
  const R refl_ad = up_ad * rad_down;
  R down_ad = rr * up_ad;
  const double ts_ad =
      a.b.water_cov[gp] * planck_radiance_dT<double>(a.sp.c1[l], a.sp.c2[l], a.sp.b1[l],
                                                     a.sp.b2[l], ts) * double(bs_ad);
  if (a.mode == 1) {
    a.tsk[pl] = ts_ad;
    a.ek[pl] = double(e_ad - refl_ad);
  } else {
    a.tsk[(size_t)p * L + l] = ts_ad;
  }
  // sweep 4 (surface -> top): downwelling part, Planck adjoint, OD path adjoint
  R pa_lo = R(0), pa_hi = R(0), suffix = R(0), ua_hi = R(0);
  int plvl = K - 1;
  auto flush = [&](void) {
    suffix += pa_hi;
    const R odr = od[(size_t)plvl * L];
    od[(size_t)plvl * L] = (odr < R(0) || odr > R(MAX_OD)) ? R(0) : suffix;
    pa_hi = pa_lo;
    pa_lo = R(0);
    plvl--;
  };
  auto scatter = [&](int i, R v) {
    const int ka = k1[i], kb = k2[i];
    while (ka < plvl) flush();
    if (ka == kb) {
      if (ka == plvl) pa_lo += v; else pa_hi += v;
    } else {
      const R f = R(fac[i]);
      if (ka == plvl) { pa_lo += (R(1) - f) * v; pa_hi += f * v; }
      else { pa_hi += (R(1) - f) * v; }   // ka == plvl+1 implies kb > K: unreachable
    }
  };
  double* kt_row = (a.mode == 1) ? a.kt + pl * Kmax : nullptr;
  for (int ku = Ku - 1; ku >= 0; ku--) {
    const R tau = a.TAU[cs + (size_t)ku * L];
    const R d = exp(-tau * rsd);
    const R B = planck_radiance<R>(c1, c2, b1, b2, R(tu[ku]));
    R a_ad = a.RD[cs + (size_t)ku * L] * d * down_ad;
    const R src_ad = down_ad;
    down_ad = down_ad * d;
    const R bad = a.BAD[cs + (size_t)ku * L] + src_ad * (R(1) - d);
    a_ad -= B * d * src_ad;
    const R tod = a.TODAD[cs + (size_t)ku * L] - a_ad * rsd;
    const R pterm = planck_radiance_dT<R>(c1, c2, b1, b2, R(tu[ku])) * bad;
    if (a.mode == 1) kt_row[ku] = double(pterm);
    else a.kt[cs + (size_t)ku * L] = double(pterm);
    // user-level path adjoint (ODPS_AtmAbsorption.f90:519-530)
    ua_hi += tod / rsec;
    scatter(ku + 1, ua_hi);
    ua_hi = -tod / rsec;
  }
  scatter(0, ua_hi);
  while (plvl >= 0) flush();
  if (a.mode == 1)
    for (int ku = Ku; ku < Kmax; ku++) kt_row[ku] = 0.0;
}

// ---------------------------------------------------------------------------
// 4. absorption adjoint: reference-layer adjoints of T and the ODPS absorbers
//    RA[p][v][k][l], v = 0 temperature, 1+a absorber a.
// ---------------------------------------------------------------------------
template <int G, class R, int NP>
__global__ void __launch_bounds__(128) absorb_ad_kernel(int K, int L, int n_chunk,
                                                        const float* __restrict__ C,
                                                        const unsigned* __restrict__ cmask,
                                                        const R* __restrict__ D,
                                                        const R* __restrict__ ODAD,
                                                        const double* __restrict__ Tm,
                                                        const double* __restrict__ Am,
                                                        const unsigned char* __restrict__ amask,
                                                        const double* __restrict__ pdp,
                                                        R* __restrict__ RA) {
  constexpr int NS = Group<G>::NS, JM = Group<G>::JM, NV = Group<G>::NV;
  constexpr int NNZ = PdNnz<G>::value;
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  const int p0 = blockIdx.y * NP;
  const bool active = l < L;
  const unsigned wmask = __reduce_or_sync(0xffffffffu, active ? cmask[l] : 0u);
  const int lc = active ? l : 0;
  int pp[NP];
#pragma unroll
  for (int p = 0; p < NP; p++) pp[p] = min(p0 + p, n_chunk - 1);
  R Stz[NP], Stzp[NP], Sgazp[NP][JM], Sgatzp[NP][JM];
#pragma unroll
  for (int p = 0; p < NP; p++) {
    Stz[p] = Stzp[p] = R(0);
#pragma unroll
    for (int a = 0; a < JM; a++) Sgazp[p][a] = Sgatzp[p][a] = R(0);
  }
  for (int k = K - 1; k >= 0; k--) {
    R E[NP][NV];
#pragma unroll
    for (int p = 0; p < NP; p++)
#pragma unroll
      for (int q = 0; q < NV; q++) E[p][q] = R(0);
    const float* Ck = C + (size_t)k * NS * L + lc;
    static_for<NNZ>([&](auto ec) {
      constexpr int e = decltype(ec)::value;
      constexpr int s = PdTab<G>::slot[e], q = PdTab<G>::q[e];
      constexpr int j = slot_component<G>(s);
      if (!(wmask & (1u << j))) return;
      const R c = R(__ldg(Ck + (size_t)s * L));
#pragma unroll
      for (int p = 0; p < NP; p++) E[p][q] += c * __ldg(D + ((size_t)pp[p] * K + k) * NNZ + e);
    });
    const R pd = R(pdp[k]);
#pragma unroll
    for (int p = 0; p < NP; p++) {
      const R oda = active ? ODAD[((size_t)pp[p] * K + k) * L + l] : R(0);
      Stz[p] += oda * E[p][qTz<G>()];
      Stzp[p] += oda * E[p][qTzp<G>()];
      const R Tk = R(Tm[(size_t)pp[p] * K + k]);
      R tad = oda * E[p][0] + Stz[p] + pd * Stzp[p];
      R aad[JM];
#pragma unroll
      for (int a = 0; a < JM; a++) {
        Sgazp[p][a] += oda * E[p][qGazp<G>(a)];
        Sgatzp[p][a] += oda * E[p][qGatzp<G>(a)];
        const R Ak = R(Am[((size_t)pp[p] * JM + a) * K + k]);
        tad += pd * Ak * Sgatzp[p][a];
        aad[a] = oda * E[p][qA<G>(a)] + pd * Sgazp[p][a] + pd * Tk * Sgatzp[p][a];
        if (!amask[((size_t)pp[p] * JM + a) * K + k]) aad[a] = R(0);
      }
      if (active && p0 + p < n_chunk) {
        R* out = RA + (((size_t)(p0 + p) * (1 + JM)) * K + k) * L + l;
        out[0] = tad;
#pragma unroll
        for (int a = 0; a < JM; a++) out[(size_t)(1 + a) * K * L] = aad[a];
      }
    }
  }
}

// ---------------------------------------------------------------------------
// 5. Map_Input adjoint to user layers: K-matrix outputs.
// ---------------------------------------------------------------------------
template <class R>
struct MapArgs {
  int K, L, Kmax, Jm, n_abs, p_begin, n_chunk;
  BatchView b;
  PrepView<R> pv;
  const R* RA;            // [n_chunk][1+Jm][K][L]
  const int* abs_of_user; // [n_abs]: ODPS absorber index of each user absorber, or -1
  double* kt;             // [P][L][Kmax] holds the Planck part on entry
  double* ka;             // [P][L][n_abs][Kmax]
};

template <class R>
__global__ void __launch_bounds__(256) map_kernel(MapArgs<R> m) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)m.n_chunk * m.L) return;
  const int p = (int)(idx / m.L), l = (int)(idx % m.L);
  const int gp = m.p_begin + p;
  const int K = m.K, L = m.L, Kmax = m.Kmax;
  const size_t pl = (size_t)gp * L + l;
  double* kt = m.kt + pl * Kmax;
  double* ka = m.ka + pl * m.n_abs * Kmax;
  const int Ku = m.pv.status[p] ? 0 : m.b.n_layers[gp];
  const int* i0 = m.pv.band_i0 + (size_t)p * K;
  const int* nb = m.pv.band_n + (size_t)p * K;
  const double* w = m.pv.band_w + (size_t)p * K * MAX_BAND;
  const int* uk0 = m.pv.ulay_k0 + (size_t)p * Kmax;
  const int* uk1 = m.pv.ulay_k1 + (size_t)p * Kmax;
  const R* ra = m.RA + (size_t)p * (1 + m.Jm) * K * L + l;
  for (int ku = 0; ku < Kmax; ku++) {
    if (ku >= Ku) {
      kt[ku] = 0.0;
      for (int j = 0; j < m.n_abs; j++) ka[(size_t)j * Kmax + ku] = 0.0;
      continue;
    }
    const int ka0 = uk0[ku], ka1 = uk1[ku];
    double acc = 0.0;
    for (int k = ka1; k >= ka0; k--) {
      const int i = ku - i0[k];
      if (i < 0 || i >= nb[k]) continue;
      acc += w[k * MAX_BAND + i] * double(ra[(size_t)k * L]);
    }
    kt[ku] += acc;
    for (int j = 0; j < m.n_abs; j++) {
      const int a = m.abs_of_user[j];
      double acc_a = 0.0;
      if (a >= 0) {
        const R* rav = ra + (size_t)(1 + a) * K * L;
        for (int k = ka1; k >= ka0; k--) {
          const int i = ku - i0[k];
          if (i < 0 || i >= nb[k]) continue;
          acc_a += w[k * MAX_BAND + i] * double(rav[(size_t)k * L]);
        }
      }
      ka[(size_t)j * Kmax + ku] = acc_a;
    }
  }
}

// ---------------------------------------------------------------------------
// Adjoint mode: sums over channels, then the Map_Input adjoint per profile.
// ---------------------------------------------------------------------------
// rows [n_chunk][nrow][L] -> out [n_chunk][nrow]; one warp per row.
template <class T>
__global__ void sum_channels_kernel(const T* __restrict__ in, double* __restrict__ out,
                                    long long n_rows, int L) {
  const long long row = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (row >= n_rows) return;
  const T* r = in + row * L;
  double acc = 0.0;
  for (int l = lane; l < L; l += 32) acc += double(r[l]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) out[row] = acc;
}

template <class R>
struct AdjMapArgs {
  int K, Kmax, Jm, n_abs, p_begin, n_chunk;
  BatchView b;
  PrepView<R> pv;
  const double* ras;      // [n_chunk][1+Jm][K] channel sums of RA
  const double* pts;      // [n_chunk][Kmax] channel sums of the Planck part
  const double* tss;      // [n_chunk] channel sums of the skin temperature adjoint
  const int* abs_of_user;
  double* t_ad;           // [P][Kmax]
  double* a_ad;           // [P][n_abs][Kmax]
  double* ts_ad;          // [P]
};

template <class R>
__global__ void adjoint_map_kernel(AdjMapArgs<R> m) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)m.n_chunk * m.Kmax) return;
  const int p = (int)(idx / m.Kmax), ku = (int)(idx % m.Kmax);
  const int gp = m.p_begin + p;
  const int K = m.K, Kmax = m.Kmax;
  const int Ku = m.pv.status[p] ? 0 : m.b.n_layers[gp];
  if (ku == 0) m.ts_ad[gp] = m.tss[p];
  double* to = m.t_ad + (size_t)gp * Kmax;
  double* ao = m.a_ad + (size_t)gp * m.n_abs * Kmax;
  if (ku >= Ku) {
    to[ku] = 0.0;
    for (int j = 0; j < m.n_abs; j++) ao[(size_t)j * Kmax + ku] = 0.0;
    return;
  }
  const int* i0 = m.pv.band_i0 + (size_t)p * K;
  const int* nb = m.pv.band_n + (size_t)p * K;
  const double* w = m.pv.band_w + (size_t)p * K * MAX_BAND;
  const int k0 = m.pv.ulay_k0[(size_t)p * Kmax + ku], k1 = m.pv.ulay_k1[(size_t)p * Kmax + ku];
  const double* ras = m.ras + (size_t)p * (1 + m.Jm) * K;
  double acc = m.pts[(size_t)p * Kmax + ku];
  for (int k = k1; k >= k0; k--) {
    const int i = ku - i0[k];
    if (i < 0 || i >= nb[k]) continue;
    acc += w[k * MAX_BAND + i] * ras[k];
  }
  to[ku] = acc;
  for (int j = 0; j < m.n_abs; j++) {
    const int a = m.abs_of_user[j];
    double acc_a = 0.0;
    if (a >= 0)
      for (int k = k1; k >= k0; k--) {
        const int i = ku - i0[k];
        if (i < 0 || i >= nb[k]) continue;
        acc_a += w[k * MAX_BAND + i] * ras[(size_t)(1 + a) * K + k];
      }
    ao[(size_t)j * Kmax + ku] = acc_a;
  }
}

}  // namespace crtm
