// CUDA kernels of the clear-sky ODPS + Emission forward / K-matrix / adjoint path.
//
// A batch is processed in chunks of profiles.  Per chunk:
//   prep_kernel        one warp per profile: Map_Input (ODPS_CoordinateMapping.f90:151-319),
//                      running sums by warp scans, predictors X
//                      (ODPS_Predictor.f90:645-1095) and the predictor
//                      partial-derivative table D; mapping bands for the adjoint
//   absorb_fwd_kernel  one thread per (channel, NPF profiles): reference-layer
//                      OD = sum C*X (ODPS_AtmAbsorption.f90:169-208)
//   column_kernel      one CTA per (profile, 32 channels), one warp per channel,
//                      layers across lanes: clamp + path + level interpolation
//                      (ODPS_AtmAbsorption.f90:213-254), Planck, Emission
//                      (Emission_Module.f90:54-174) as affine warp scans, Planck
//                      inversion; for K/AD the Emission adjoint
//                      (Emission_Module.f90:280-395) and the optical-depth path
//                      adjoint (ODPS_AtmAbsorption.f90:487-540), also as scans
//   absorb_ad_kernel   one thread per (channel, NPA profiles): coefficient x
//                      predictor-partial contraction and reverse running sums
//                      (ODPS_AtmAbsorption.f90:543-598, ODPS_Predictor.f90:1783-2643)
//   map_kernel         one warp per (profile, channel): Map_Input adjoint to
//                      user layers (ODPS_CoordinateMapping.f90:480-547), K output
//   adjoint_*          CRTM_Adjoint: sums over channels, then the Map_Input adjoint
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>
#include <utility>

#include "odps_prep.cuh"
#include "optran.cuh"

namespace crtm {

constexpr int MAX_OUT_ABS = 8;   // absorber Jacobians per K-matrix call
constexpr unsigned FULL = 0xffffffffu;

// (slot, variable) pattern of the partial-derivative table.
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
  static constexpr int slot[PD_NNZ_G1] = {PD_ENTRIES_G1(CRTM_PD_SLOT)};
  static constexpr int q[PD_NNZ_G1] = {PD_ENTRIES_G1(CRTM_PD_VAR)};
};
template <> struct PdTab<2> {
  CRTM_PD_QCODES_MEMBERS(2)
  static constexpr int slot[PD_NNZ_G2] = {PD_ENTRIES_G2(CRTM_PD_SLOT)};
  static constexpr int q[PD_NNZ_G2] = {PD_ENTRIES_G2(CRTM_PD_VAR)};
};
template <> struct PdTab<3> {
  CRTM_PD_QCODES_MEMBERS(3)
  static constexpr int slot[PD_NNZ_G3] = {PD_ENTRIES_G3(CRTM_PD_SLOT)};
  static constexpr int q[PD_NNZ_G3] = {PD_ENTRIES_G3(CRTM_PD_VAR)};
};

// Entries of D per layer: the partials, then pdp*A_a (a < JM), pdp*T and the
// Map_Input adjoint pass mask (bit a set: absorber a passes).
template <int G> struct DLayout {
  static constexpr int NNZ = PdNnz<G>::value;
  static constexpr int NX = NNZ + Group<G>::JM + 2;
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
// Warp scans (lanes own consecutive blocks of elements)
// ---------------------------------------------------------------------------
template <class T>
__device__ __forceinline__ T warp_excl_sum(T v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const T n = __shfl_up_sync(FULL, v, o);
    if (lane >= o) v += n;
  }
  const T e = __shfl_up_sync(FULL, v, 1);
  return lane == 0 ? T(0) : e;
}
template <class T>
__device__ __forceinline__ T warp_rexcl_sum(T v) {   // sum over lanes > lane
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const T n = __shfl_down_sync(FULL, v, o);
    if (lane + o < 32) v += n;
  }
  const T e = __shfl_down_sync(FULL, v, 1);
  return lane == 31 ? T(0) : e;
}
template <class T>
__device__ __forceinline__ T warp_excl_prod(T v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const T n = __shfl_up_sync(FULL, v, o);
    if (lane >= o) v *= n;
  }
  const T e = __shfl_up_sync(FULL, v, 1);
  return lane == 0 ? T(1) : e;
}
template <class T>
__device__ __forceinline__ T warp_rexcl_prod(T v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const T n = __shfl_down_sync(FULL, v, o);
    if (lane + o < 32) v *= n;
  }
  const T e = __shfl_down_sync(FULL, v, 1);
  return lane == 31 ? T(1) : e;
}
// Affine maps x -> a*x + b.  Forward: lower lanes applied first; on return
// (a, b) is the composition of the maps of lanes < lane.
template <class T>
__device__ __forceinline__ void warp_affine_excl(T& a, T& b) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const T an = __shfl_up_sync(FULL, a, o), bn = __shfl_up_sync(FULL, b, o);
    if (lane >= o) { b = a * bn + b; a = an * a; }
  }
  const T ae = __shfl_up_sync(FULL, a, 1), be = __shfl_up_sync(FULL, b, 1);
  a = lane == 0 ? T(1) : ae;
  b = lane == 0 ? T(0) : be;
}
// Reverse: higher lanes applied first; composition of the maps of lanes > lane.
template <class T>
__device__ __forceinline__ void warp_affine_rexcl(T& a, T& b) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const T an = __shfl_down_sync(FULL, a, o), bn = __shfl_down_sync(FULL, b, o);
    if (lane + o < 32) { b = a * bn + b; a = an * a; }
  }
  const T ae = __shfl_down_sync(FULL, a, 1), be = __shfl_down_sync(FULL, b, 1);
  a = lane == 31 ? T(1) : ae;
  b = lane == 31 ? T(0) : be;
}

// Vector loads of N consecutive values (N a multiple of 4 floats / 2 doubles,
// source 16-byte aligned).
template <class R, int N>
__device__ __forceinline__ void load_group(const R* __restrict__ src, R* dst) {
  if constexpr (sizeof(R) == 4) {
#pragma unroll
    for (int i = 0; i < N; i += 4) {
      const float4 v = __ldg(reinterpret_cast<const float4*>(src + i));
      dst[i] = v.x; dst[i + 1] = v.y; dst[i + 2] = v.z; dst[i + 3] = v.w;
    }
  } else {
#pragma unroll
    for (int i = 0; i < N; i += 2) {
      const double2 v = __ldg(reinterpret_cast<const double2*>(src + i));
      dst[i] = v.x; dst[i + 1] = v.y;
    }
  }
}

// Asynchronous global->shared copies (16 bytes; src_bytes 0 zero-fills).
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem, int src_bytes) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem), "r"(src_bytes));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Coefficient tile of one reference layer: NS slots x 32 channels starting at
// channel l0 of C[k][s][Lp] (Lp a multiple of 32, rows 128-byte aligned).
template <int NS>
__device__ __forceinline__ void load_c_tile(float (*dst)[32], const float* __restrict__ C, int k,
                                            int Lp, int l0, int tid, int nthreads) {
  for (int i = tid; i < NS * 8; i += nthreads) {
    const int s = i >> 3, q = i & 7;
    cp_async16(&dst[s][q * 4], C + ((size_t)k * NS + s) * Lp + l0 + q * 4, 16);
  }
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
  // Profile order of the pipeline: chunk position i (p_begin + p) is batch
  // profile perm[i]; null for the batch's own order.  The pipeline runs the
  // profiles of one bucket (clear, cloudy with up to 6 streams, cloudy with
  // 8-16 streams) at a time.
  const int* perm = nullptr;
};

// Batch profile of pipeline position i.
CRTM_HD int batch_profile(const BatchView& b, int i) { return b.perm ? b.perm[i] : i; }

// The RTSolution components beyond radiance and brightness temperature
// (crtm_gpu_rtsolution), each null when not wanted: [P][L] and, for the
// layer arrays, [P][L][Kmax].
struct RtsExt {
  double* tb_clear = nullptr, *r_clear = nullptr, *tcc = nullptr, *sod = nullptr, *emis = nullptr;
  double* up = nullptr, *down = nullptr, *bs = nullptr;
  int* nfs = nullptr;
  double* lod = nullptr, *upw = nullptr, *ovc = nullptr;
};

// Zero the layer array row [from, Kmax) of output o at pair pl, if o is wanted.
CRTM_HD void zero_row(double* o, size_t pl, int Kmax, int from) {
  if (!o) return;
  double* r = o + pl * Kmax;
  for (int k = from; k < Kmax; k++) r[k] = 0.0;
}

struct SpecView {
  const double* c1, *c2, *b1, *b2, *cbr;
  const double* freq, *wn;   // GHz, cm^-1
};

// Running sums of the reference profile (the *_ref terms of ODPS_Predictor.f90:707-759).
struct RefSums {
  const double* tz_ref;     // [K]
  const double* tzp_ref;    // [K]
  const double* gazp_ref;   // [Jm][K]
  const double* gatzp_ref;  // [Jm][K]
};

template <class R>
struct PrepView {
  R* Xg;               // [ceil(n/npf)][K][NS][npf]
  R* Dg;               // [ceil(n/npa)][K][NX][npa] (K/AD only)
  int* band_i0;        // [n][K]
  int* band_n;         // [n][K]
  double* band_w;      // [n][K][MAX_BAND]
  int* ulev_k1;        // [n][Kmax+1]  0-based reference level bracket of user level i
  int* ulev_k2;        // [n][Kmax+1]
  double* ulev_fac;    // [n][Kmax+1]
  int* rlev_ilo;       // [n][K+1] user levels whose bracket touches reference level j
  int* rlev_ihi;       // [n][K+1]
  int* ub_k0;          // [n][Kmax] first reference layer mapping to user layer ku
  int* ub_n;           // [n][Kmax]
  double* ub_w;        // [n][Kmax][MAX_UBAND]
  double* scal;        // [n][4]: sec_surface, u = cos(sensor zenith)
  int* status;         // [n]
  double* opt;         // [n][K][OPT_NS] OPTRAN predictor state, or null (no OPTRAN channels)
  int K, Kmax, npf, npa;
};

template <int G>
inline size_t prep_smem_bytes(int K) {
  return sizeof(double) * ((size_t)(4 + 3 * Group<G>::JM) * K + 2 * MAX_LAYERS + 1) +
         sizeof(int) * (size_t)K;
}

// ---------------------------------------------------------------------------
// 1. prep: one warp (= one CTA) per profile
// ---------------------------------------------------------------------------
template <int G, class R>
__global__ void __launch_bounds__(32) prep_kernel(SensorTables S, RefSums RS, BatchView b,
                                                  PrepView<R> pv, const int* __restrict__ idx_map,
                                                  int p_begin, int n_chunk) {
  constexpr int JM = Group<G>::JM, NS = Group<G>::NS, NNZ = DLayout<G>::NNZ, NX = DLayout<G>::NX;
  extern __shared__ double psm[];
  const int lane = threadIdx.x;
  const int p = blockIdx.x;
  if (p >= n_chunk) return;
  const int gp = batch_profile(b, p_begin + p);
  const int K = S.K, Kmax = pv.Kmax;
  const int Ku = b.n_layers[gp];
  if (Ku < 2 || Ku > Kmax || Ku > MAX_LAYERS) {
    if (lane == 0) pv.status[p] = ST_BAD_LAYERS;
    return;
  }
  double* sT = psm;                      // [K]     mapped temperature
  double* sA = sT + K;                   // [JM][K] mapped absorber amounts
  double* sTz = sA + (size_t)JM * K;     // [K]     running sum of T
  double* sTzp = sTz + K;                // [K]     running sum of pdp*T
  double* sGz = sTzp + K;                // [JM][K] running sum of pdp*A
  double* sGt = sGz + (size_t)JM * K;    // [JM][K] running sum of pdp*A*T
  double* ulnp = sGt + (size_t)JM * K;   // [MAX_LAYERS]
  double* ulev = ulnp + MAX_LAYERS;      // [MAX_LAYERS+1]
  int* sPass = reinterpret_cast<int*>(ulev + MAX_LAYERS + 1);  // [K]
  const double* lev = b.level_pressure + (size_t)gp * (Kmax + 1);
  const double* lay = b.pressure + (size_t)gp * Kmax;
  const double* tu = b.temperature + (size_t)gp * Kmax;
  for (int k = lane; k < Ku; k += 32) ulnp[k] = log(lay[k]);
  for (int k = lane; k <= Ku; k += 32)
    ulev[k] = (k == 0) ? ((lev[0] <= 0.0) ? log(lev[1] / 2.0) : log(lev[0])) : log(lev[k]);
  __syncwarp();
  int status = ST_OK;
  int* bi0 = pv.band_i0 + (size_t)p * K;
  int* bn = pv.band_n + (size_t)p * K;
  double* bw = pv.band_w + (size_t)p * K * MAX_BAND;
  // ---- mapping of T and absorbers to the reference layers (lanes stride over layers)
  for (int k = lane; k < K; k += 32) {
    const int st = layer_avg_start(S.ref_lnp, K, ulnp, Ku, k);
    int i0, n;
    double* w = bw + (size_t)k * MAX_BAND;
    status |= layer_avg_column(S.ref_lnp, K, ulnp, Ku, k, st, &i0, &n, w);
    bi0[k] = i0;
    bn[k] = n;
    double acc = 0.0;
    for (int i = 0; i < n; i++) acc += w[i] * tu[i0 + i];
    sT[k] = acc;
    int pass = 0;
#pragma unroll
    for (int a = 0; a < JM; a++) {
      const int map = idx_map[a];
      double v;
      if (map >= 0) {
        const double* au = b.absorber + ((size_t)gp * b.n_abs + map) * Kmax;
        v = 0.0;
        for (int i = 0; i < n; i++) v += w[i] * au[i0 + i];
        if (v <= EPS_FP) v = EPS_FP;
        if (v < S.min_a[a * K + k]) v = S.min_a[a * K + k];
        if (v > S.max_a[a * K + k]) v = S.max_a[a * K + k];
        if (v > EPS_FP) pass |= 1 << a;   // ODPS_CoordinateMapping.f90:521-523
      } else {
        v = S.ref_a[a * K + k];
      }
      sA[a * K + k] = v;
    }
    sPass[k] = pass;
  }
  __syncwarp();
  // ---- running sums: contiguous block per lane, warp scan of the block totals
  {
    const int per = (K + 31) / 32, k0 = min(K, lane * per), k1 = min(K, k0 + per);
    for (int qn = 0; qn < 2 + 2 * JM; qn++) {
      // qn: 0 T, 1 pdp*T, 2+a pdp*A_a, 2+JM+a pdp*A_a*T
      const int a = (qn < 2) ? 0 : (qn - 2) % JM;
      double* out = qn == 0 ? sTz : (qn == 1 ? sTzp : (qn < 2 + JM ? sGz + a * K : sGt + a * K));
      double c = 0.0;
      for (int k = k0; k < k1; k++) {
        const double v = qn == 0 ? sT[k] : (qn == 1 ? S.pdp[k] * sT[k]
                         : (qn < 2 + JM ? S.pdp[k] * sA[a * K + k] : S.pdp[k] * sA[a * K + k] * sT[k]));
        c += v;
      }
      double run = warp_excl_sum(c);
      for (int k = k0; k < k1; k++) {
        const double v = qn == 0 ? sT[k] : (qn == 1 ? S.pdp[k] * sT[k]
                         : (qn < 2 + JM ? S.pdp[k] * sA[a * K + k] : S.pdp[k] * sA[a * K + k] * sT[k]));
        run += v;
        out[k] = run;
      }
    }
  }
  __syncwarp();
  // ---- height-dependent secants (ODPS_CoordinateMapping.f90:285-306)
  const Geom g = geometry(b.zenith[gp]);
  const double alt = b.altitude ? b.altitude[gp] : 0.0;
  const double psfc = lev[Ku];
  int sfc_idx = K;
  double sfc_frac = 0.0;
  if (S.ref_lev[K] > psfc) {
    for (int k = K; k >= 0; k--)
      if (S.ref_lev[k] < psfc) {
        sfc_idx = k + 1;
        sfc_frac = (S.ref_lev_lnp[sfc_idx] - ulev[Ku]) / (S.ref_lev_lnp[sfc_idx] - S.ref_lev_lnp[k]);
        break;
      }
  }
  double zoff;
  if (S.ref_lev[K] >= psfc)
    zoff = -(S.zgeo[sfc_idx] + sfc_frac * (S.zgeo[sfc_idx - 1] - S.zgeo[sfc_idx])) + alt;
  else
    zoff = CC_H * S.ref_t[K - 1] * log(1013.0 / S.ref_lev[K]);
  const double sv = (EARTH_RADIUS + alt) * sin(g.trans_zenith_radian);
  // ---- predictors and partials (lanes stride over layers)
  const int pgf = p / pv.npf, pof = p % pv.npf;
  const int pga = pv.npa ? p / pv.npa : 0, poa = pv.npa ? p % pv.npa : 0;
  for (int k = lane; k < K; k += 32) {
    // the predictors and partials are evaluated in R: FP32 in the mixed form
    LayerStateT<R> Ls;
    const double sa = sv / (EARTH_RADIUS + (S.zgeo[k + 1] + zoff));
    Ls.sec = R(1.0 / sqrt(1.0 - sa * sa));
    Ls.T_ = R(sT[k]);
    Ls.Tref = R(S.ref_t[k]);
    Ls.dT = R(sT[k] - S.ref_t[k]);
    Ls.pdp = R(S.pdp[k]);
    Ls.tz_ref = R(RS.tz_ref[k]);
    Ls.tz = R(sTz[k] / RS.tz_ref[k]);
    Ls.tzp_ref = R(RS.tzp_ref[k]);
    Ls.tzp = R(sTzp[k] / RS.tzp_ref[k]);
#pragma unroll
    for (int a = 0; a < MAX_ABS; a++) {
      if (a < JM) {
        Ls.A[a] = R(sA[a * K + k]);
        Ls.Aref[a] = R(S.ref_a[a * K + k]);
        Ls.gazp_ref[a] = R(RS.gazp_ref[a * K + k]);
        Ls.gatzp_ref[a] = R(RS.gatzp_ref[a * K + k]);
        Ls.gazp[a] = R(sGz[a * K + k] / RS.gazp_ref[a * K + k]);
        Ls.gatzp[a] = R(sGt[a * K + k] / RS.gatzp_ref[a * K + k]);
      } else {
        Ls.A[a] = Ls.Aref[a] = Ls.gazp[a] = Ls.gatzp[a] = Ls.gazp_ref[a] = Ls.gatzp_ref[a] = R(1);
      }
    }
    R X[NS];
    layer_predictors<G, R, R>(Ls, X);
    R* xo = pv.Xg + ((size_t)pgf * K + k) * NS * pv.npf + pof;
#pragma unroll
    for (int s = 0; s < NS; s++) xo[(size_t)s * pv.npf] = X[s];
    if (pv.Dg) {
      R D[NNZ];
      layer_partials<G, R, R>(Ls, D);
      R* dO = pv.Dg + ((size_t)pga * K + k) * NX * pv.npa + poa;
#pragma unroll
      for (int e = 0; e < NNZ; e++) dO[(size_t)e * pv.npa] = D[e];
#pragma unroll
      for (int a = 0; a < JM; a++) dO[(size_t)(NNZ + a) * pv.npa] = R(S.pdp[k] * sA[a * K + k]);
      dO[(size_t)(NNZ + JM) * pv.npa] = R(S.pdp[k] * sT[k]);
      dO[(size_t)(NNZ + JM + 1) * pv.npa] = R(float(sPass[k]));
    }
  }
  // ---- compact-OPTRAN predictors (ODPS_Predictor.f90:336-347): a running
  // sum over the layers, on lane 0, in FP64
  if (pv.opt) {
    __syncwarp();
    if (lane == 0) {
      double secl[MAX_LAYERS];
      for (int k = 0; k < K; k++) {
        const double sa = sv / (EARTH_RADIUS + (S.zgeo[k + 1] + zoff));
        secl[k] = 1.0 / sqrt(1.0 - sa * sa);
      }
      optran_profile(K, sT, sA + (size_t)S.h2o_idx * K, secl, sPass, S.ref_lev, S.ref_p, S.o_alpha, S.o_c1,
                     S.o_c2, pv.opt + (size_t)p * K * OPT_NS);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) status |= __shfl_xor_sync(FULL, status, o);
  // ---- reference -> user level brackets (Compute_Interp_Index, sequential on lane 0)
  int* k1o = pv.ulev_k1 + (size_t)p * (Kmax + 1);
  int* k2o = pv.ulev_k2 + (size_t)p * (Kmax + 1);
  double* fo = pv.ulev_fac + (size_t)p * (Kmax + 1);
  for (int i = lane; i <= Ku; i += 32) { k1o[i] = 0; k2o[i] = 0; }   // every entry a valid level
  __syncwarp();
  if (lane == 0) {
    const double* x = S.ref_lev_lnp;
    const int nx = K + 1, nu = Ku + 1;
    int k1 = nu + 1, k2 = 0;
    for (int iu = 1; iu <= nu; iu++) {
      if (ulev[iu - 1] < x[0]) { k1o[iu - 1] = 0; k2o[iu - 1] = 0; }
      else { k1 = iu; break; }
    }
    for (int iu = nu; iu >= k1; iu--) {
      if (ulev[iu - 1] > x[nx - 1]) { k1o[iu - 1] = nx - 1; k2o[iu - 1] = nx - 1; }
      else { k2 = iu; break; }
    }
    int jj = 1;
    for (int iu = k1; iu <= k2; iu++)
      for (int ix = jj; ix <= nx - 1; ix++)
        if (ulev[iu - 1] >= x[ix - 1] && ulev[iu - 1] <= x[ix]) {
          k1o[iu - 1] = ix - 1; k2o[iu - 1] = ix; jj = ix;
          break;
        }
    for (int i = 0; i < nu; i++) {
      const int a = k1o[i], c = k2o[i];
      fo[i] = (a == c) ? 0.0 : (ulev[i] - x[a]) / (x[c] - x[a]);
    }
    pv.scal[(size_t)p * 4 + 0] = g.sec_trans_zenith;
    pv.scal[(size_t)p * 4 + 1] = 1.0 / g.sec_sensor_zenith;  // Common_RTSolution.f90:227
  }
  __syncwarp();
  // ---- reference level j <- user levels whose bracket touches it (path adjoint)
  int* ilo = pv.rlev_ilo + (size_t)p * (K + 1);
  int* ihi = pv.rlev_ihi + (size_t)p * (K + 1);
  for (int jl = lane; jl <= K; jl += 32) {
    int lo = Ku + 1, hi = -1;
    for (int i = 0; i <= Ku; i++)
      if (k1o[i] == jl || k2o[i] == jl) { if (i < lo) lo = i; hi = i; }
    ilo[jl] = lo;
    ihi[jl] = hi;
  }
  // ---- user layer ku <- reference layers mapping to it (Map_Input adjoint)
  int* uk0 = pv.ub_k0 + (size_t)p * Kmax;
  int* un = pv.ub_n + (size_t)p * Kmax;
  double* uw = pv.ub_w + (size_t)p * Kmax * MAX_UBAND;
  int ust = 0;
  for (int ku = lane; ku < Ku; ku += 32) {
    int k0 = -1, k1 = -1;
    for (int k = 0; k < K; k++)
      if (ku >= bi0[k] && ku < bi0[k] + bn[k]) { if (k0 < 0) k0 = k; k1 = k; }
    int n = (k0 < 0) ? 0 : k1 - k0 + 1;
    if (n > MAX_UBAND) { ust |= ST_UBAND_OVERFLOW; n = MAX_UBAND; }
    uk0[ku] = k0 < 0 ? 0 : k0;
    un[ku] = n;
    for (int i = 0; i < n; i++) {
      const int k = k0 + i, r = ku - bi0[k];
      uw[(size_t)ku * MAX_UBAND + i] = (r >= 0 && r < bn[k]) ? bw[(size_t)k * MAX_BAND + r] : 0.0;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) ust |= __shfl_xor_sync(FULL, ust, o);
  if (lane == 0) pv.status[p] = status | ust;
}

// ---------------------------------------------------------------------------
// 2. absorption forward: OD[p][k][l] = sum_s C[k][s][l] * X[p][k][s].
//    CTA = 32 channels (lanes) x FWD_WARPS warps, each warp NP profiles; the
//    coefficient slice of each layer is staged in shared memory (double
//    buffered, cp.async) and used by all warps.
// ---------------------------------------------------------------------------
constexpr int FWD_WARPS = 4;
constexpr int FWD_CH = 64;   // channels per CTA: 2 per lane

// Coefficient tile of one reference layer: NS slots x FWD_CH channels from l0.
template <int NS>
__device__ __forceinline__ void load_c_tile64(float (*dst)[FWD_CH], const float* __restrict__ C,
                                              int k, int Lp, int l0, int tid, int nthreads) {
  for (int i = tid; i < NS * (FWD_CH / 4); i += nthreads) {
    const int s = i / (FWD_CH / 4), q = i % (FWD_CH / 4);
    const int l = l0 + q * 4;
    // rows are padded to a multiple of 32 channels; a half tile past the end reads zeros
    cp_async16(&dst[s][q * 4], C + ((size_t)k * NS + s) * Lp + (l < Lp ? l : 0), l < Lp ? 16 : 0);
  }
}

template <int G, class R, int NP>
constexpr size_t fwd_smem_bytes() {
  return sizeof(float) * 2 * Group<G>::NS * FWD_CH + sizeof(R) * 2 * FWD_WARPS * Group<G>::NS * NP;
}

template <int G, class R, int NP>
__global__ void __launch_bounds__(32 * FWD_WARPS) absorb_fwd_kernel(int K, int L, int Lp, int n_chunk,
                                                                    const float* __restrict__ C,
                                                                    const unsigned* __restrict__ cmask,
                                                                    const R* __restrict__ Xg,
                                                                    R* __restrict__ OD) {
  constexpr int NS = Group<G>::NS, J = Group<G>::J;
  constexpr int XCH = NS * NP * (int)sizeof(R) / 16;   // 16-byte chunks of one warp's X slice
  extern __shared__ __align__(16) unsigned char fwd_smem[];
  auto cs = reinterpret_cast<float (*)[NS][FWD_CH]>(fwd_smem);                       // [2][NS][FWD_CH]
  auto xs = reinterpret_cast<R (*)[FWD_WARPS][NS * NP]>(fwd_smem + sizeof(float) * 2 * NS * FWD_CH);
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int l0 = blockIdx.x * FWD_CH;
  const int la = l0 + lane, lb = l0 + 32 + lane;
  const int pg = blockIdx.y * FWD_WARPS + wib;
  const int p0 = pg * NP;
  const unsigned wmask = __reduce_or_sync(FULL, (la < L ? cmask[la] : 0u) | (lb < L ? cmask[lb] : 0u));
  const R* Xb = Xg + (size_t)pg * K * NS * NP;
  const bool group_ok = p0 < n_chunk;
  auto stage = [&](int k, int buf) {
    load_c_tile64<NS>(cs[buf], C, k, Lp, l0, threadIdx.x, 32 * FWD_WARPS);
    if (group_ok) {
      const R* src = Xb + (size_t)k * NS * NP;
      for (int i = lane; i < XCH; i += 32)
        cp_async16(&xs[buf][wib][i * (16 / sizeof(R))], src + i * (16 / sizeof(R)), 16);
    }
    cp_async_commit();
  };
  stage(0, 0);
  for (int k = 0; k < K; k++) {
    cp_async_wait_all();
    __syncthreads();
    if (k + 1 < K) stage(k + 1, (k + 1) & 1);
    if (!group_ok) continue;
    const float (*ct)[FWD_CH] = cs[k & 1];
    const R* xk = xs[k & 1][wib];
    R acc0[NP], acc1[NP];
#pragma unroll
    for (int p = 0; p < NP; p++) acc0[p] = acc1[p] = R(0);
    static_for<J>([&](auto jc) {
      constexpr int j = decltype(jc)::value;
      constexpr int s0 = Group<G>::OFF[j], s1 = Group<G>::OFF[j + 1];
      if (!(wmask & (1u << j))) return;
#pragma unroll
      for (int s = s0; s < s1; s++) {
        const R ca = R(ct[s][lane]), cb = R(ct[s][32 + lane]);
        R x[NP];
#pragma unroll
        for (int p = 0; p < NP; p++) x[p] = xk[s * NP + p];
#pragma unroll
        for (int p = 0; p < NP; p++) { acc0[p] += ca * x[p]; acc1[p] += cb * x[p]; }
      }
    });
#pragma unroll
    for (int p = 0; p < NP; p++) {
      if (p0 + p >= n_chunk) break;
      R* o = OD + ((size_t)(p0 + p) * K + k) * L;
      if (la < L) o[la] = acc0[p];
      if (lb < L) o[lb] = acc1[p];
    }
  }
}

// ---------------------------------------------------------------------------
// 3. column: one thread per (profile, channel), two passes over the user layers.
//    mode 0 forward, 1 K-matrix, 2 adjoint, 3 layer optical depths only.
//
//    Pass 1 (top down) follows the forward model: OD path and its interpolation
//    to the user levels, layer transmittance, Planck radiance and the
//    downwelling recursion.  Pass 2 (bottom up) runs the upwelling recursion
//    and, alongside it, the Emission adjoint and the OD-path adjoint for a
//    unit radiance seed.  The Planck-inversion adjoint seed dBT/dR * seed is
//    known only once the TOA radiance is, so it is written per (profile,
//    channel) and applied by the kernels that consume the adjoints (the
//    adjoint is linear in it).
// ---------------------------------------------------------------------------
template <class R>
struct ColumnArgs {
  int K, L, Kmax, p_begin, n_chunk, mode;
  BatchView b;
  SpecView sp;
  PrepView<R> pv;
  R* OD;                  // [n][K][L]: in reference ODs, out (K/AD) unit-seed OD adjoint
  R* TAU, *DTOP;          // [n][Kmax][L] scratch: layer OD and downwelling at the layer top
  R* PT;                  // [n][Kmax][L] unit-seed Planck part of the temperature adjoint
  R* SC;                  // [n][L] adjoint seed dBT/dR * seed
  const double* seed;     // [P][L] or null (=1)
  double* radiance, *bt;  // [P][L]
  double* tsk, *ek;       // K-matrix: [P][L] water temperature, emissivity; adjoint: tsk is [n][L]
                          // scratch of dBT/dTs x seed
  double* tsk_land, *tsk_snow, *tsk_ice;   // K-matrix: [P][L] or null
  // IR sea-surface emissivity model (batch emissivity from CRTM_IRSSEM): its
  // derivatives de/d(wind speed), de/d(water temperature) [P][L], or null;
  // wind_k receives dBT/d(wind speed): K-matrix [P][L], adjoint [n][L]
  const double* sfc_ev, *sfc_et;
  double* wind_k;
  int* status;            // [P] or null
  // Scattering profiles in a K-matrix/adjoint call: launched twice.  pass 1
  // stores TAU/DTOP and stops; the scattering K kernel then writes the cloudy
  // column's unit-seed derivatives; pass 2 finishes clear profiles as usual
  // and, for scattering profiles, mixes the cloudy column with the clear one
  // (weights tcc and 1 - tcc of a fractional profile; 1 and 0 otherwise).
  int pass;                      // 0: one launch (no scattering profiles)
  const int* n_clouds, *n_aerosols;   // [P] or null
  const R* TODc;                 // [n][Kmax][L] cloudy dR/dtau (PT holds the cloudy dR/dT)
  const double* CB;              // [n][4][L] cloudy radiance, dR/de, dR/dBs, clear radiance
  const double* cover;           // [n] total cloud cover, -1: no clear part
  // further RTSolution components.  A profile solved here with the Emission
  // solver gets them all; for a profile with clouds or aerosols the launch
  // before the scattering kernels (mode 3, pass 1) writes the emissivity and
  // zeros the Emission-only components and the scattering optical depth
  // (which the layer kernel accumulates), and pass 2 writes the cloud cover
  // and the clear column.
  RtsExt x;
  const int* n_streams;          // [P] Options%n_Streams or null
};

template <class R>
__device__ __forceinline__ R clamp_od(R v) {
  return v < R(0) ? R(0) : (v > R(MAX_OD) ? R(MAX_OD) : v);
}

template <class R>
inline size_t column_smem_bytes(int K, int Kmax) {
  return sizeof(double) * (size_t)(Kmax + 1) + sizeof(R) * (size_t)Kmax +
         sizeof(int) * (2 * (size_t)(Kmax + 1) + 2 * (size_t)(K + 1)) + 16;
}

// EXT: the call asks for further RTSolution components (a.x); without them
// the component code compiles out.
template <class R, bool EXT>
__global__ void __launch_bounds__(128) column_kernel(ColumnArgs<R> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int K = a.K, L = a.L, Kmax = a.Kmax;
  const int p = blockIdx.y, gp = batch_profile(a.b, a.p_begin + p);
  const int tid = threadIdx.x;
  const int l = blockIdx.x * blockDim.x + tid;
  // interpolation factors in R, converted once per CTA (the slot is sized for doubles)
  R* facd = reinterpret_cast<R*>(smem_raw);              // [Kmax+1]
  R* tus = reinterpret_cast<R*>(reinterpret_cast<double*>(smem_raw) + Kmax + 1);   // [Kmax]
  int* k1s = reinterpret_cast<int*>(tus + Kmax);         // [Kmax+1]
  int* k2s = k1s + (Kmax + 1);
  int* ilos = k2s + (Kmax + 1);                          // [K+1]
  int* ihis = ilos + (K + 1);
  const int st = a.pv.status[p];
  const int Ku = a.b.n_layers[gp];
  if (blockIdx.x == 0 && tid == 0 && a.status) a.status[gp] = st;
  const RtsExt x = EXT ? a.x : RtsExt{};
  auto ext_scalars = [&](size_t pl, double e, double up, double down, double bs) {
    if (x.emis) x.emis[pl] = e;
    if (x.up) x.up[pl] = up;
    if (x.down) x.down[pl] = down;
    if (x.bs) x.bs[pl] = bs;
  };
  if (st != 0) {
    if (l < L) {
      const size_t pl = (size_t)gp * L + l;
      a.radiance[pl] = 0.0;
      a.bt[pl] = 0.0;
      ext_scalars(pl, 0.0, 0.0, 0.0, 0.0);
      if (x.tb_clear) x.tb_clear[pl] = 0.0;
      if (x.r_clear) x.r_clear[pl] = 0.0;
      if (x.tcc) x.tcc[pl] = 0.0;
      if (x.sod) x.sod[pl] = 0.0;
      if (x.nfs) x.nfs[pl] = 0;
      zero_row(x.lod, pl, Kmax, 0);
      zero_row(x.upw, pl, Kmax, 0);
      zero_row(x.ovc, pl, Kmax, 0);
      if (a.mode == 1) { a.tsk[pl] = 0.0; a.ek[pl] = 0.0; }
      if (a.mode == 1 || a.mode == 2) a.SC[(size_t)p * L + l] = R(0);
      if (a.mode == 2) a.tsk[(size_t)p * L + l] = 0.0;
      if (a.wind_k) a.wind_k[a.mode == 1 ? pl : (size_t)p * L + l] = 0.0;
    }
    return;
  }
  const double* tug = a.b.temperature + (size_t)gp * Kmax;
  for (int i = tid; i < Kmax; i += blockDim.x) tus[i] = R(i < Ku ? tug[i] : 0.0);
  const int* k1g = a.pv.ulev_k1 + (size_t)p * (Kmax + 1);
  const int* k2g = a.pv.ulev_k2 + (size_t)p * (Kmax + 1);
  const double* fg = a.pv.ulev_fac + (size_t)p * (Kmax + 1);
  for (int i = tid; i <= Ku; i += blockDim.x) { k1s[i] = k1g[i]; k2s[i] = k2g[i]; facd[i] = R(fg[i]); }
  if (a.mode) {
    const int* ilg = a.pv.rlev_ilo + (size_t)p * (K + 1);
    const int* ihg = a.pv.rlev_ihi + (size_t)p * (K + 1);
    for (int i = tid; i <= K; i += blockDim.x) { ilos[i] = ilg[i]; ihis[i] = ihg[i]; }
  }
  __syncthreads();
  if (l >= L) return;
  const size_t pl = (size_t)gp * L + l;
  const double* sc = a.pv.scal + (size_t)p * 4;
  const R inv_sec = R(1.0 / sc[0]);
  const R inv_u = R(1.0 / sc[1]);
  const double c1d = a.sp.c1[l], c2d = a.sp.c2[l], b1d = a.sp.b1[l], b2d = a.sp.b2[l];
  const R c1 = R(c1d), c2 = R(c2d), b1 = R(b1d), b2 = R(b2d);
  const double e = a.b.emissivity[pl];
  const R re = R(e), rr = R(1.0 - e);
  const double tsd = a.b.land_cov[gp] * a.b.land_t[gp] + a.b.water_cov[gp] * a.b.water_t[gp] +
                     a.b.snow_cov[gp] * a.b.snow_t[gp] + a.b.ice_cov[gp] * a.b.ice_t[gp];
  // surface Planck radiance and its temperature derivative in R (the Planck
  // inversion at the end stays in FP64)
  const R ted = b1 + b2 * R(tsd);
  const R eed = exp(c2 / ted);
  const R Bs = c1 / (eed - R(1));
  R* od = a.OD + (size_t)p * K * L + l;
  const size_t cs = (size_t)p * Kmax * L + l;   // scratch base, stride L

  // ---- pass 1 (top down): OD path, user-level interpolation, downwelling.
  // Reference levels are walked in order (OD loads prefetched two levels
  // ahead); each user level is emitted once the upper level of its bracket
  // is reached.
  // a profile with clouds or aerosols (solved by the scattering kernels):
  // every profile of a forward launch in mode 3, those with clouds or
  // aerosols in the K-matrix / adjoint launches around the scattering kernels
  const bool scat_p = a.mode == 3 ||
                      ((a.pass == 1 || a.pass == 2) &&
                       ((a.n_clouds && a.n_clouds[gp] > 0) || (a.n_aerosols && a.n_aerosols[gp] > 0)));
  double* lod_row = (x.lod && a.pass != 2) ? x.lod + pl * Kmax : nullptr;
  double* ovc_row = (x.ovc && a.pass != 2 && !scat_p) ? x.ovc + pl * Kmax : nullptr;
  // mode 0: the layer optical depths wait in the upwelling row for the upwelling sweep
  double* stash = (x.upw && a.mode == 0) ? x.upw + pl * Kmax : nullptr;
  R rad_down = R(a.sp.cbr[l]);
  R src = R(0), tr = R(1), total = R(0);   // atmospheric upwelling at the top, accumulated top down
  R path_prev = R(0), path_cur = R(0), up_prev = R(0);
  R od1 = K > 0 ? od[0] : R(0), od2 = K > 1 ? od[L] : R(0);
  int i = 0;
  for (int k = 0; k <= K; k++) {
    while (i <= Ku && k2s[i] == k) {
      const int ka = k1s[i];
      const R upi = (ka == k) ? path_cur : path_prev + (path_cur - path_prev) * facd[i];
      if (i > 0) {
        const int ku = i - 1;
        const R tau = (upi - up_prev) * inv_sec;
        const R t = exp(-tau * inv_u);
        const R te = b1 + b2 * tus[ku];
        const R B = c1 / (exp(c2 / te) - R(1));
        if (ovc_row) ovc_row[ku] = double(src + tr * B);   // a black cloud filling layer ku
        if (lod_row) lod_row[ku] = double(tau);
        if (stash) stash[ku] = double(tau);
        src += tr * B * (R(1) - t);
        if (a.mode != 0 && a.pass != 2) {
          a.TAU[cs + (size_t)ku * L] = tau;
          if (a.mode != 3) a.DTOP[cs + (size_t)ku * L] = rad_down;
        }
        tr *= t;
        total += tau;
        rad_down = rad_down * t + B * (R(1) - t);
      }
      up_prev = upi;
      i++;
    }
    if (k == K) break;
    const R v = clamp_od(od1);
    od1 = od2;
    if (k + 2 < K) od2 = od[(size_t)(k + 2) * L];
    path_prev = path_cur;
    path_cur += v;
  }
  const R Dn = rad_down, Tn = tr;
  const int nsu = a.n_streams ? a.n_streams[gp] : 0;
  if (a.mode == 0) {
    const double Rd = double(src + Tn * (re * Bs + rr * Dn));
    const double btv = planck_temperature(c1d, c2d, b1d, b2d, Rd);
    a.radiance[pl] = Rd;
    a.bt[pl] = btv;
    ext_scalars(pl, e, double(src), double(Dn), double(Bs));
    if (x.tb_clear) x.tb_clear[pl] = btv;   // no clouds (CRTM_Forward_Module.f90:1115-1119)
    if (x.r_clear) x.r_clear[pl] = Rd;
    if (x.tcc) x.tcc[pl] = 0.0;
    if (x.sod) x.sod[pl] = 0.0;
    if (x.nfs) x.nfs[pl] = nsu > 0 ? nsu + 2 : 0;
    if (stash) {   // upwelling at each layer's bottom, surface to top
      R U = re * Bs + rr * Dn;
      for (int ku = Ku - 1; ku >= 0; ku--) {
        const R tau = R(stash[ku]);
        stash[ku] = double(U);
        const R t = exp(-tau * inv_u);
        const R B = c1 / (exp(c2 / (b1 + b2 * tus[ku])) - R(1));
        U = t * U + B * (R(1) - t);
      }
    }
    zero_row(x.lod, pl, Kmax, Ku);
    zero_row(x.upw, pl, Kmax, Ku);
    zero_row(x.ovc, pl, Kmax, Ku);
    return;
  }
  if (a.mode == 3 || a.pass == 1) {
    if (scat_p) {   // Emission-only components zero; the scattering kernels fill the rest
      ext_scalars(pl, e, 0.0, 0.0, 0.0);
      if (x.sod) x.sod[pl] = 0.0;
      zero_row(x.lod, pl, Kmax, Ku);
      zero_row(x.upw, pl, Kmax, 0);
      zero_row(x.ovc, pl, Kmax, 0);
    }
    // mode 3: gas layer optical depths only (the cloudy solver follows);
    // pass 1: TAU/DTOP stored, the scattering K kernel runs next
    return;
  }
  // ---- pass 2 (bottom up): upwelling, Emission adjoint, OD path adjoint (unit seed)
  R U = re * Bs + rr * Dn;
  R P = R(1);                 // transmittance of the layers below the current one
  const R down0 = rr * Tn;    // downwelling adjoint at the surface (unit seed)
  R cum = R(0);               // OD of the layers below the current one
  R pa_lo = R(0), pa_hi = R(0), suffix = R(0), ua_hi = R(0);
  int plvl = K - 1;
  R odm = od[(size_t)plvl * L];   // reference OD of layer plvl (clamp test), prefetched
  auto flush = [&]() {
    suffix += pa_hi;
    od[(size_t)plvl * L] = (odm < R(0) || odm > R(MAX_OD)) ? R(0) : suffix;
    pa_hi = pa_lo;
    pa_lo = R(0);
    plvl--;
    if (plvl >= 0) odm = od[(size_t)plvl * L];
  };
  auto scatter = [&](int iu, R v) {
    const int ka = k1s[iu], kb = k2s[iu];
    while (ka < plvl) flush();
    if (ka == kb) {
      if (ka == plvl) pa_lo += v; else pa_hi += v;
    } else {
      const R f = facd[iu];
      pa_lo += (R(1) - f) * v;
      pa_hi += f * v;
    }
  };
  const bool scat = a.pass == 2 && ((a.n_clouds && a.n_clouds[gp] > 0) || (a.n_aerosols && a.n_aerosols[gp] > 0));
  double wcloud = 0.0;   // weight of the cloudy column
  if (scat) wcloud = a.cover[p] < 0.0 ? 1.0 : a.cover[p];
  const R wclr = R(1.0 - wcloud), wcl = R(wcloud);
  double* upw_row = (x.upw && !scat) ? x.upw + pl * Kmax : nullptr;
  R tau_n = a.TAU[cs + (size_t)(Ku - 1) * L], dt_n = a.DTOP[cs + (size_t)(Ku - 1) * L];
  for (int ku = Ku - 1; ku >= 0; ku--) {
    const R tau = tau_n, Dtop = dt_n;
    if (ku > 0) { tau_n = a.TAU[cs + (size_t)(ku - 1) * L]; dt_n = a.DTOP[cs + (size_t)(ku - 1) * L]; }
    const R t = exp(-tau * inv_u);
    const R te = b1 + b2 * tus[ku];
    const R ee = exp(c2 / te);
    const R em1 = ee - R(1);
    const R B = c1 / em1;
    const R den = te * em1;
    const R dB = c1 * c2 * ee * b2 / (den * den);
    const R Tprev = exp(-(total - cum - tau) * inv_u);   // TOA to the top of this layer
    // upwelling part (Emission_AD first loop)
    R tod = -(Tprev * (U - B) * t) * inv_u;
    R Bad = Tprev * (R(1) - t);
    // downwelling part (Emission_AD second loop)
    const R dad = down0 * P;
    Bad += dad * (R(1) - t);
    tod -= ((Dtop - B) * t * dad) * inv_u;
    R ptv = dB * Bad;
    if (upw_row) upw_row[ku] = double(U);   // upwelling at this layer's bottom
    if (scat) {
      ptv = wclr * ptv + wcl * a.PT[cs + (size_t)ku * L];
      tod = wclr * tod + wcl * a.TODc[cs + (size_t)ku * L];
    }
    a.PT[cs + (size_t)ku * L] = ptv;
    U = t * U + B * (R(1) - t);
    P *= t;
    cum += tau;
    // user-level path adjoint (ODPS_AtmAbsorption.f90:519-530) and its scatter to
    // the reference levels (Interpolate_Profile_F1_AD), flushing finished layers
    ua_hi += tod * inv_sec;
    scatter(ku + 1, ua_hi);
    ua_hi = -tod * inv_sec;
  }
  scatter(0, ua_hi);
  while (plvl >= 0) flush();
  for (int ku = Ku; ku < Kmax; ku++) a.PT[cs + (size_t)ku * L] = R(0);
  // ---- TOA radiance, brightness temperature and the adjoint seed; the
  // surface derivatives for a unit radiance seed (emissivity with the
  // reflectivity 1 - e, and the surface Planck radiance)
  double Rd = double(U);
  double e_b = double(Tn) * (double(Bs) - double(Dn));
  double Bs_b = e * double(Tn);
  if (scat) {
    const double* cb = a.CB + (size_t)p * 4 * L + l;
    Rd = (1.0 - wcloud) * Rd + wcloud * cb[0];
    e_b = (1.0 - wcloud) * e_b + wcloud * cb[(size_t)L];
    Bs_b = (1.0 - wcloud) * Bs_b + wcloud * cb[2 * (size_t)L];
  }
  a.radiance[pl] = Rd;
  double btv, dtdr;
  planck_temperature_with_dR(c1d, c2d, b1d, b2d, Rd, &btv, &dtdr);
  a.bt[pl] = btv;
  // further RTSolution components: the K-matrix and adjoint fill R_clear and
  // Tb_clear for fractional profiles only (CRTM_K_Matrix_Module.f90:1328-1336)
  if (scat) {
    const bool frac = a.cover[p] >= 0.0;
    const double Rc = double(U);
    if (x.tcc) x.tcc[pl] = frac ? a.cover[p] : 0.0;
    if (x.r_clear) x.r_clear[pl] = frac ? Rc : 0.0;
    if (x.tb_clear) x.tb_clear[pl] = frac ? planck_temperature(c1d, c2d, b1d, b2d, Rc) : 0.0;
  } else {
    ext_scalars(pl, e, double(src), double(Dn), double(Bs));
    if (x.tcc) x.tcc[pl] = 0.0;
    if (x.r_clear) x.r_clear[pl] = 0.0;
    if (x.tb_clear) x.tb_clear[pl] = 0.0;
    if (x.sod) x.sod[pl] = 0.0;
    if (x.nfs) x.nfs[pl] = nsu > 0 ? nsu + 2 : 0;
    zero_row(x.lod, pl, Kmax, Ku);
    zero_row(x.upw, pl, Kmax, Ku);
    zero_row(x.ovc, pl, Kmax, Ku);
  }
  const double seed = a.seed ? a.seed[pl] : 1.0;
  const double scale = dtdr * seed;
  a.SC[(size_t)p * L + l] = R(scale);
  const R dden = ted * (eed - R(1));
  const R dBs = c1 * c2 * eed * b2 / (dden * dden);
  // surface temperature: Ts = sum of the coverage-weighted cover temperatures
  // (CRTM_Compute_SurfaceT), so each cover's adjoint is its coverage x dBT/dTs
  const double ts_ad = double(dBs) * Bs_b * scale;
  // emissivity model (water coverage 1): de/dT adds to the water temperature
  // adjoint, de/dv gives the wind speed's (CRTM_Compute_IRSSEM_AD)
  const double e_ad = scale * e_b;   // emissivity_AD - reflectivity_AD
  const double ts_e = a.sfc_et ? e_ad * a.sfc_et[pl] : 0.0;
  if (a.mode == 1) {
    a.tsk[pl] = a.b.water_cov[gp] * ts_ad + ts_e;
    if (a.tsk_land) a.tsk_land[pl] = a.b.land_cov[gp] * ts_ad;
    if (a.tsk_snow) a.tsk_snow[pl] = a.b.snow_cov[gp] * ts_ad;
    if (a.tsk_ice) a.tsk_ice[pl] = a.b.ice_cov[gp] * ts_ad;
    a.ek[pl] = e_ad;
    if (a.wind_k) a.wind_k[pl] = e_ad * a.sfc_ev[pl];
  } else {
    a.tsk[(size_t)p * L + l] = ts_ad + ts_e;
    if (a.wind_k) a.wind_k[(size_t)p * L + l] = e_ad * a.sfc_ev[pl];
  }
}

// ---------------------------------------------------------------------------
// 4. absorption adjoint: reference-layer adjoints RA[p][v][k][l], v = 0 the
//    temperature, v = 1+j the j-th requested absorber.  CTA = 32 channels
//    (lanes) x 4 warps, each warp NP profiles; the coefficient slice of layer k
//    for the CTA's channels is staged in shared memory and used by all warps.
// ---------------------------------------------------------------------------
struct OutAbs {
  int n;                  // requested absorber adjoints
  int odps[MAX_OUT_ABS];  // ODPS absorber of each, or -1 (absorber unknown to the sensor)
};

constexpr int AD_WARPS = 4;

// OUTSET 0: adjoints of every ODPS absorber; 1: only absorbers 0 and 1 (H2O and,
// for groups 1-2, O3), which skips the partials the other absorbers' own
// adjoints need (their GATzp terms still feed the temperature adjoint).
template <int G, int OUTSET>
__host__ __device__ constexpr bool q_needed(int q) {
  constexpr int JM = Group<G>::JM;
  if (OUTSET == 0) return true;
  if (q >= 1 && q <= JM) return (q - 1) < 2;                          // local absorber
  if (q >= 3 + JM && q < 3 + 2 * JM) return (q - 3 - JM) < 2;          // GAzp
  return true;
}

template <int G, class R, int NP, int OUTSET>
__global__ void __launch_bounds__(32 * AD_WARPS) absorb_ad_kernel(
    int K, int L, int Lp, int n_chunk, const float* __restrict__ C,
    const unsigned* __restrict__ cmask, const R* __restrict__ Dg,
    const double* __restrict__ pdp_tab, const R* __restrict__ ODAD, const R* __restrict__ SC,
    OutAbs oa, R* __restrict__ RA) {
  constexpr int NS = Group<G>::NS, JM = Group<G>::JM, NV = Group<G>::NV;
  constexpr int NNZ = DLayout<G>::NNZ, NX = DLayout<G>::NX;
  constexpr int DCH = NX * NP * (int)sizeof(R) / 16;   // 16-byte chunks of one warp's D slice
  __shared__ __align__(16) float cs[2][NS][32];
  __shared__ __align__(16) R ds[2][AD_WARPS][NX * NP];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int l0 = blockIdx.x * 32, l = l0 + lane;
  const int pg = blockIdx.y * AD_WARPS + wib;
  const int p0 = pg * NP;
  const bool active = l < L;
  const unsigned wmask = __reduce_or_sync(FULL, active ? cmask[l] : 0u);
  const int nv = 1 + oa.n;
  const R* Db = Dg + (size_t)pg * K * NX * NP;
  const bool group_ok = p0 < n_chunk;
  R scl[NP];
#pragma unroll
  for (int p = 0; p < NP; p++)
    scl[p] = (active && p0 + p < n_chunk) ? SC[(size_t)(p0 + p) * L + l] : R(0);
  R Stz[NP], Stzp[NP], Sgazp[NP][JM], Sgatzp[NP][JM];
#pragma unroll
  for (int p = 0; p < NP; p++) {
    Stz[p] = Stzp[p] = R(0);
#pragma unroll
    for (int a = 0; a < JM; a++) Sgazp[p][a] = Sgatzp[p][a] = R(0);
  }
  auto stage = [&](int k, int buf) {
    load_c_tile<NS>(cs[buf], C, k, Lp, l0, threadIdx.x, 32 * AD_WARPS);
    if (group_ok) {
      const R* src = Db + (size_t)k * NX * NP;
      for (int i = lane; i < DCH; i += 32) cp_async16(&ds[buf][wib][i * (16 / sizeof(R))], src + i * (16 / sizeof(R)), 16);
    }
    cp_async_commit();
  };
  // OD adjoints of the next layer are loaded one iteration ahead
  R odn[NP];
#pragma unroll
  for (int p = 0; p < NP; p++)
    odn[p] = (active && p0 + p < n_chunk) ? ODAD[((size_t)(p0 + p) * K + (K - 1)) * L + l] : R(0);
  stage(K - 1, (K - 1) & 1);
  for (int k = K - 1; k >= 0; k--) {
    cp_async_wait_all();
    __syncthreads();
    if (k > 0) stage(k - 1, (k - 1) & 1);
    if (!group_ok) continue;
    R odc[NP];
#pragma unroll
    for (int p = 0; p < NP; p++) {
      odc[p] = odn[p];
      if (k > 0 && active && p0 + p < n_chunk) odn[p] = ODAD[((size_t)(p0 + p) * K + (k - 1)) * L + l];
    }
    const float (*ct)[32] = cs[k & 1];
    const R* Dk = ds[k & 1][wib];
    R E[NP][NV];
#pragma unroll
    for (int p = 0; p < NP; p++)
#pragma unroll
      for (int q = 0; q < NV; q++) E[p][q] = R(0);
    static_for<NNZ>([&](auto ec) {
      constexpr int e = decltype(ec)::value;
      constexpr int s = PdTab<G>::slot[e], q = PdTab<G>::q[e];
      constexpr int j = slot_component<G>(s);
      if constexpr (!q_needed<G, OUTSET>(q)) return;
      if (!(wmask & (1u << j))) return;
      const R c = R(ct[s][lane]);
#pragma unroll
      for (int p = 0; p < NP; p++) E[p][q] += c * Dk[e * NP + p];
    });
    const R pdp = R(pdp_tab[k]);
#pragma unroll
    for (int p = 0; p < NP; p++) {
      const bool valid = active && (p0 + p < n_chunk);
      const R oda = valid ? odc[p] * scl[p] : R(0);
      const R pT = Dk[(NNZ + JM) * NP + p];
      const unsigned mask = (unsigned)Dk[(NNZ + JM + 1) * NP + p];
      Stz[p] += oda * E[p][qTz<G>()];
      Stzp[p] += oda * E[p][qTzp<G>()];
      // T_ad(k) = local + S_Tz + pdp*S_Tzp + sum_a (pdp*A_a)*S_GATzp_a
      R tad = oda * E[p][0] + Stz[p] + pdp * Stzp[p];
      R aad[JM];
#pragma unroll
      for (int a = 0; a < JM; a++) {
        Sgatzp[p][a] += oda * E[p][qGatzp<G>(a)];
        const R pA = Dk[(NNZ + a) * NP + p];
        tad += pA * Sgatzp[p][a];
        if (OUTSET == 0 || a < 2) {
          Sgazp[p][a] += oda * E[p][qGazp<G>(a)];
          // A_ad(k,a) = local + pdp*S_GAzp_a + (pdp*T)*S_GATzp_a, zero where Map_Input's
          // adjoint blocks it (ODPS_CoordinateMapping.f90:521-523)
          aad[a] = ((mask >> a) & 1u)
                       ? oda * E[p][qA<G>(a)] + pdp * Sgazp[p][a] + pT * Sgatzp[p][a]
                       : R(0);
        } else {
          aad[a] = R(0);
        }
      }
      if (valid) {
        R* out = RA + ((size_t)(p0 + p) * nv * K + k) * L + l;
        out[0] = tad;
        for (int jo = 0; jo < oa.n; jo++) {
          const int aj = oa.odps[jo];
          R vout = R(0);
#pragma unroll
          for (int a = 0; a < JM; a++)
            if (a == aj) vout = aad[a];
          out[(size_t)(1 + jo) * K * L] = vout;
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// 5. Map_Input adjoint to user layers and the K-matrix outputs.  CTA = one
//    profile x CT channels: the reference-layer adjoint tiles RA[v][k][CT] and
//    the Planck part PT[ku][CT] are staged in shared memory, then each warp
//    writes whole output rows (lanes across user layers).
// ---------------------------------------------------------------------------
template <class R>
struct MapArgs {
  int K, L, Kmax, p_begin, n_chunk, nv, ct;
  BatchView b;
  PrepView<R> pv;
  const R* RA;   // [n][nv][K][L]
  const R* PT;   // [n][Kmax][L]
  const R* SC;   // [n][L]
  double* kt;    // [P][L][Kmax]
  double* ka;    // [P][L][nv-1][Kmax]
};

template <class R>
inline size_t map_smem_bytes(int K, int Kmax, int nv, int ct) {
  return sizeof(R) * ((size_t)nv * K * (ct + 1) + (size_t)Kmax * (ct + 1) + ct +
                      (size_t)Kmax * MAX_UBAND) +
         sizeof(int) * 2 * (size_t)Kmax + 16;
}

template <class R>
__global__ void __launch_bounds__(256) map_kernel(MapArgs<R> m) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int K = m.K, L = m.L, Kmax = m.Kmax, nv = m.nv, CT = m.ct, CS = m.ct + 1;
  const int cshift = __ffs(CT) - 1;   // CT is a power of two
  const int p = blockIdx.y, gp = batch_profile(m.b, m.p_begin + p);
  const int l0 = blockIdx.x * CT;
  const int tid = threadIdx.x, wib = tid >> 5, lane = tid & 31;
  R* rat = reinterpret_cast<R*>(smem_raw);        // [nv][K][CS]
  R* ptt = rat + (size_t)nv * K * CS;             // [Kmax][CS]
  R* sct = ptt + (size_t)Kmax * CS;               // [CT]
  R* uws = sct + CT;                              // [MAX_UBAND][Kmax]
  int* uk0 = reinterpret_cast<int*>(uws + (size_t)Kmax * MAX_UBAND);
  int* un = uk0 + Kmax;
  const int Ku = m.pv.status[p] ? 0 : m.b.n_layers[gp];
  const int ncl = min(CT, L - l0);
  {
    const R* src = m.RA + (size_t)p * nv * K * L + l0;
    const int total = nv * K << cshift;
    for (int i = tid; i < total; i += 256) {
      const int row = i >> cshift, c = i & (CT - 1);
      rat[row * CS + c] = c < ncl ? src[(size_t)row * L + c] : R(0);
    }
    const R* pts = m.PT + (size_t)p * Kmax * L + l0;
    const int tp = Ku << cshift;
    for (int i = tid; i < tp; i += 256) {
      const int ku = i >> cshift, c = i & (CT - 1);
      ptt[ku * CS + c] = c < ncl ? pts[(size_t)ku * L + c] : R(0);
    }
  }
  if (tid < CT) sct[tid] = tid < ncl ? m.SC[(size_t)p * L + l0 + tid] : R(0);
  for (int i = tid; i < Ku; i += 256) {
    uk0[i] = m.pv.ub_k0[(size_t)p * Kmax + i];
    un[i] = m.pv.ub_n[(size_t)p * Kmax + i];
  }
  {
    const double* uwg = m.pv.ub_w + (size_t)p * Kmax * MAX_UBAND;
    for (int i = tid; i < Ku * MAX_UBAND; i += 256) {
      const int ku = i / MAX_UBAND, j = i % MAX_UBAND;   // stored [j][ku]: conflict-free reads
      uws[j * Kmax + ku] = R(uwg[i]);
    }
  }
  __syncthreads();
  // each lane owns user layers ku = lane + 32*t; weights are read once per layer
  for (int ku0 = 0; ku0 < Kmax; ku0 += 32) {
    const int ku = ku0 + lane;
    const bool live = ku < Ku;
    const int k0 = live ? uk0[ku] : 0, n = live ? un[ku] : 0;
    R w[4];
#pragma unroll
    for (int i = 0; i < 4; i++) w[i] = i < n ? uws[i * Kmax + ku] : R(0);
    for (int c = wib; c < ncl; c += 8) {
      const size_t pl = (size_t)gp * L + l0 + c;
      const R scl = sct[c];
      for (int v = 0; v < nv; v++) {
        double* out = v == 0 ? m.kt + pl * Kmax : m.ka + (pl * (nv - 1) + (v - 1)) * Kmax;
        if (ku >= Kmax) continue;
        if (!live) { out[ku] = 0.0; continue; }
        const R* rav = rat + (size_t)(v * K + k0) * CS + c;
        R acc = (v == 0) ? ptt[ku * CS + c] * scl : R(0);
#pragma unroll
        for (int i = 3; i >= 0; i--)
          if (i < n) acc += w[i] * rav[i * CS];
        for (int i = 4; i < n; i++) acc += uws[i * Kmax + ku] * rav[i * CS];
        out[ku] = double(acc);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// 6. CRTM_Adjoint: sums over channels in a fixed order, then the Map_Input adjoint.
// ---------------------------------------------------------------------------
// out[row] = sum_l in[row][l] * (w ? w[row / rows_per_w][l] : 1); one warp per row.
template <class T>
__global__ void channel_sum_kernel(const T* __restrict__ in, const T* __restrict__ w,
                                   int rows_per_w, long long n_rows, int L, double* __restrict__ out) {
  const long long row = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (row >= n_rows) return;
  const T* r = in + row * L;
  const T* wr = w ? w + (row / rows_per_w) * L : nullptr;
  double acc = 0.0;
  for (int l = lane; l < L; l += 32) acc += double(r[l]) * (wr ? double(wr[l]) : 1.0);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(FULL, acc, o);
  if (lane == 0) out[row] = acc;
}

template <class R>
struct AdjMapArgs {
  int K, Kmax, nv, p_begin, n_chunk;
  BatchView b;
  PrepView<R> pv;
  const double* ras;   // [n][nv][K] channel sums of RA
  const double* pts;   // [n][Kmax] channel sums of SC * PT
  const double* tss;   // [n] channel sums of the skin temperature adjoint
  double* t_ad;        // [P][Kmax]
  double* a_ad;        // [P][nv-1][Kmax]
  double* ts_ad;       // [P] water temperature
  double* ts_land, *ts_snow, *ts_ice;   // [P] or null
};

template <class R>
__global__ void adjoint_map_kernel(AdjMapArgs<R> m) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)m.n_chunk * m.Kmax) return;
  const int p = (int)(idx / m.Kmax), ku = (int)(idx % m.Kmax);
  const int gp = batch_profile(m.b, m.p_begin + p);
  const int K = m.K, Kmax = m.Kmax, nv = m.nv;
  const int Ku = m.pv.status[p] ? 0 : m.b.n_layers[gp];
  if (ku == 0) {
    m.ts_ad[gp] = m.b.water_cov[gp] * m.tss[p];
    if (m.ts_land) m.ts_land[gp] = m.b.land_cov[gp] * m.tss[p];
    if (m.ts_snow) m.ts_snow[gp] = m.b.snow_cov[gp] * m.tss[p];
    if (m.ts_ice) m.ts_ice[gp] = m.b.ice_cov[gp] * m.tss[p];
  }
  for (int v = 0; v < nv; v++) {
    double* out = v == 0 ? m.t_ad + (size_t)gp * Kmax : m.a_ad + ((size_t)gp * (nv - 1) + (v - 1)) * Kmax;
    if (ku >= Ku) { out[ku] = 0.0; continue; }
    double acc = (v == 0) ? m.pts[(size_t)p * Kmax + ku] : 0.0;
    const int k0 = m.pv.ub_k0[(size_t)p * Kmax + ku], n = m.pv.ub_n[(size_t)p * Kmax + ku];
    const double* uw = m.pv.ub_w + ((size_t)p * Kmax + ku) * MAX_UBAND;
    const double* row = m.ras + ((size_t)p * nv + v) * K;
    for (int i = n - 1; i >= 0; i--) acc += uw[i] * row[k0 + i];
    out[ku] = acc;
  }
}

}  // namespace crtm
