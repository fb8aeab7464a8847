// Compact-OPTRAN water-vapour-line term of the ODPS absorption model
// (A9): for a channel whose OSignificance is 1 the OComponent_Index
// component's layer optical depth is chi(k) dA(k) instead of the ODPS
// regression, with ln chi(k) = b_0(k) + sum_i b_i(k) OX(k, OP_Index(i)) and
// each b_i a polynomial of the transformed integrated water vapour.
//
// Reference behaviour followed (JCSDA/CRTMv3):
//   ODPS_Compute_Predictor_ODAS     src/AtmAbsorption/ODPS/ODPS_Predictor.f90:2716-2816
//   ODPS_Compute_Predictor_ODAS_AD  src/AtmAbsorption/ODPS/ODPS_Predictor.f90:3092-3230
//   Add_OPTRAN_wloOD                src/AtmAbsorption/ODPS/ODPS_AtmAbsorption.f90:664-727
//   Add_OPTRAN_wloOD_AD             src/AtmAbsorption/ODPS/ODPS_AtmAbsorption.f90:911-984
//
// Layout: the profile state of the OPTRAN predictors is computed once per
// profile by the prep kernel (lane 0, a sequential pass over the reference
// layers: the integrated water vapour is a running sum) into
// OPT[n][K][OPT_NS] doubles; the forward kernel adds each OPTRAN channel's
// optical depths to OD, one thread per (profile, OPTRAN channel) walking the
// layers; the adjoint kernel walks the layers bottom up per (profile, OPTRAN
// channel) and adds the temperature and water vapour adjoints into the
// reference-layer adjoints RA.  Both in FP64 in every form: ln chi is a sum
// of large predictors times small coefficients.
#pragma once

#include "odps_physics.cuh"

namespace crtm {

constexpr int OPT_NU = 7;        // N_PREDICTOR_USED_OPTRAN + 1 (ODPS_Define.f90:103)
constexpr int OPT_ORDER = 10;    // MAX_OPTRAN_ORDER (ODPS_Predictor_Define.f90:94)
// per (profile, reference layer): OX(1:14) at 0..13, Ap^1..Ap^10 at 14..23,
// then dA, the integrated water vapour, its layer mean, the inverse, the
// running T* and P* sums and Map_Input's pass mask
constexpr int OPT_AP = 14, OPT_DA = 24, OPT_IV = 25, OPT_AVE = 26, OPT_INV = 27, OPT_ST = 28, OPT_SP = 29,
              OPT_MASK = 30, OPT_NS = 31;
constexpr double OPT_RECIPROCAL_GRAVITY = 1.0 / 980.665;   // CRTM_Parameters.f90:164
constexpr double OPT_MIN_ABSORBER = 1.0e-76;               // CRTM_Parameters.f90:140
constexpr double OPT_LIMIT_EXP = 20.0, OPT_LIMIT_LOG = 4.8e+08;   // CRTM_Parameters.f90:150-151

// The sensor's OPTRAN channels (device tables; n = 0: none).
struct OptranView {
  int n;                  // OPTRAN channels among the processed ones
  const int* ch;          // [n] channel position in the processed list
  const int* idx;         // [n][8]: predictor count, OP_Index(1:6), polynomial order
  const double* coef;     // [n][OPT_NU][OPT_ORDER + 1] OC, zero past the count and order
  double alpha, alpha_c1, alpha_c2;
};

// ODPS_Compute_Predictor_ODAS for one profile (one thread): mapped T[k],
// water vapour V[k], secants sec[k], Map_Input's pass mask bits, the
// reference pressures; OPT[k][OPT_NS] out.
CRTM_HD void optran_profile(int K, const double* T, const double* V, const double* sec, const int* pass,
                            const double* ref_lev, const double* ref_p, double alpha, double c1, double c2,
                            double* opt) {
  double ivp = 0.0, st = 0.0, sp = 0.0, xlt_prev = 0.0, xlp_prev = 0.0;
  for (int k = 0; k < K; k++) {
    double* o = opt + (size_t)k * OPT_NS;
    const double t = T[k], P = ref_p[k], v = V[k], t2 = t * t, p2 = P * P;
    o[0] = t; o[1] = P; o[2] = t2; o[3] = p2; o[4] = t * P; o[5] = t2 * P; o[6] = t * p2; o[7] = t2 * p2;
    o[8] = sqrt(sqrt(P)); o[9] = v; o[10] = v / t2; o[13] = sec[k];
    const double dA = OPT_RECIPROCAL_GRAVITY * (ref_lev[k + 1] - ref_lev[k]) * v * sec[k];
    const double iv = ivp + dA, ave = 0.5 * (ivp + iv);
    st += t * dA;
    sp += P * dA;
    const double inv = iv > OPT_MIN_ABSORBER ? 1.0 / iv : 0.0;
    const double xlt = 0.5 * st * inv, xlp = 0.5 * sp * inv;
    o[11] = xlt + xlt_prev;
    o[12] = xlp + xlp_prev;
    xlt_prev = xlt;
    xlp_prev = xlp;
    const double ap1 = log((ave - c2) / c1) / alpha;
    double ap = 1.0;
    for (int i = 0; i < OPT_ORDER; i++) {
      ap *= ap1;
      o[OPT_AP + i] = ap;
    }
    o[OPT_DA] = dA; o[OPT_IV] = iv; o[OPT_AVE] = ave; o[OPT_INV] = inv; o[OPT_ST] = st; o[OPT_SP] = sp;
    o[OPT_MASK] = double(pass[k]);
    ivp = iv;
  }
}

// ln chi of one OPTRAN channel at one layer, with the polynomials b(0:np).
CRTM_HD double optran_lnchi(const double* o, const int* idx, const double* coef, double* b) {
  const int np = idx[0], ord = idx[7];
  double x = 0.0;
  for (int i = 0; i <= np; i++) {
    const double* c = coef + i * (OPT_ORDER + 1);
    double v = c[0];
    for (int j = 1; j <= ord; j++) v += c[j] * o[OPT_AP + j - 1];
    b[i] = v;
    x += i ? v * o[idx[i] - 1] : v;
  }
  return x;
}

// Add_OPTRAN_wloOD: OD[p][k][l] += chi(k) dA(k) for the OPTRAN channels, one
// thread per (profile, OPTRAN channel).
template <class R>
__global__ void optran_fwd_kernel(int K, int L, int n_chunk, OptranView O, const double* __restrict__ opt,
                                  R* __restrict__ OD) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x, p = blockIdx.y;
  if (c >= O.n || p >= n_chunk) return;
  const int l = O.ch[c];
  const int* idx = O.idx + (size_t)c * 8;
  if (idx[0] <= 0) return;
  const double* coef = O.coef + (size_t)c * OPT_NU * (OPT_ORDER + 1);
  const double* op = opt + (size_t)p * K * OPT_NS;
  R* od = OD + (size_t)p * K * L + l;
  for (int k = 0; k < K; k++) {
    const double* o = op + (size_t)k * OPT_NS;
    double b[OPT_NU];
    const double x = optran_lnchi(o, idx, coef, b);
    const double chi = x > OPT_LIMIT_EXP ? OPT_LIMIT_LOG : (x < -OPT_LIMIT_EXP ? 0.0 : exp(x));
    od[(size_t)k * L] += R(chi * o[OPT_DA]);
  }
}

// Add_OPTRAN_wloOD_AD + ODPS_Compute_Predictor_ODAS_AD for one (profile,
// OPTRAN channel): the layer optical depth adjoints ODAD x the seed SC to the
// mapped temperature and water vapour adjoints, added into RA[p][0][k][l]
// and RA[p][1 + h2o_out][k][l] (h2o_out < 0: the water vapour Jacobian is not
// requested; Map_Input's adjoint blocks it where the mask bit h2o_bit is 0).
template <class R>
__global__ void optran_ad_kernel(int K, int L, int n_chunk, int nv, int h2o_out, int h2o_bit, OptranView O,
                                 const double* __restrict__ opt, const double* __restrict__ ref_lev,
                                 const R* __restrict__ ODAD,
                                 const R* __restrict__ SC, R* __restrict__ RA) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x, p = blockIdx.y;
  if (c >= O.n || p >= n_chunk) return;
  const int l = O.ch[c];
  const int* idx = O.idx + (size_t)c * 8;
  const int np = idx[0], ord = idx[7];
  if (np <= 0) return;
  const double* coef = O.coef + (size_t)c * OPT_NU * (OPT_ORDER + 1);
  const double* op = opt + (size_t)p * K * OPT_NS;
  const double scl = double(SC[(size_t)p * L + l]);
  R* rt = RA + (size_t)p * nv * K * L + l;
  R* rv = h2o_out >= 0 ? rt + (size_t)(1 + h2o_out) * K * L : nullptr;
  double iv_ad = 0.0, st_ad = 0.0, sp_ad = 0.0, x12_next = 0.0, x13_next = 0.0;
  for (int k = K - 1; k >= 0; k--) {
    const double* o = op + (size_t)k * OPT_NS;
    const double oda = double(ODAD[((size_t)p * K + k) * L + l]) * scl;
    // Add_OPTRAN_wloOD_AD at layer k
    double b[OPT_NU];
    const double x = optran_lnchi(o, idx, coef, b);
    const bool in_range = x <= OPT_LIMIT_EXP && x >= -OPT_LIMIT_EXP;
    const double chi = x > OPT_LIMIT_EXP ? OPT_LIMIT_LOG : (in_range ? exp(x) : 0.0);
    const double da_ad = oda * chi;
    const double x_ad = in_range ? chi * oda * o[OPT_DA] : 0.0;
    double ox_ad[14];
    for (int i = 0; i < 14; i++) ox_ad[i] = 0.0;
    double ap1_ad = 0.0;
    for (int i = 0; i <= np; i++) {
      const double* cc = coef + i * (OPT_ORDER + 1);
      const double b_ad = i ? x_ad * o[idx[i] - 1] : x_ad;
      if (i) ox_ad[idx[i] - 1] += x_ad * b[i];
      // b_i = sum_j c_j Ap1^j: d b_i / d Ap1 = sum_j j c_j Ap1^(j-1)
      double db = 0.0;
      for (int j = 1; j <= ord; j++) db += j * cc[j] * (j == 1 ? 1.0 : o[OPT_AP + j - 2]);
      ap1_ad += db * b_ad;
    }
    // ODPS_Compute_Predictor_ODAS_AD at layer k: the integrated part
    const double t = o[0], P = o[1], v = o[9], t2 = o[2];
    const double ave_ad = ap1_ad / (O.alpha * (o[OPT_AVE] - O.alpha_c2));
    const double xlt_ad = ox_ad[11] + x12_next, xlp_ad = ox_ad[12] + x13_next;
    x12_next = ox_ad[11];
    x13_next = ox_ad[12];
    st_ad += 0.5 * o[OPT_INV] * xlt_ad;
    sp_ad += 0.5 * o[OPT_INV] * xlp_ad;
    const double inv_ad = 0.5 * o[OPT_ST] * xlt_ad + 0.5 * o[OPT_SP] * xlp_ad;
    if (o[OPT_IV] > OPT_MIN_ABSORBER) iv_ad += -inv_ad / (o[OPT_IV] * o[OPT_IV]);
    iv_ad += 0.5 * ave_ad;
    const double dA_ad = da_ad + iv_ad + P * sp_ad + t * st_ad;
    double T_ad = o[OPT_DA] * st_ad;
    double V_ad = OPT_RECIPROCAL_GRAVITY * (ref_lev[k + 1] - ref_lev[k]) * o[13] * dA_ad;
    iv_ad += 0.5 * ave_ad;   // the integrated amount above layer k
    // the local predictors
    const double p2 = P * P;
    T_ad += ox_ad[0] + P * ox_ad[4] + p2 * ox_ad[6];
    const double t2_ad = ox_ad[2] + P * ox_ad[5] + p2 * ox_ad[7] - (v / (t2 * t2)) * ox_ad[10];
    V_ad += ox_ad[9] + ox_ad[10] / t2;
    T_ad += 2.0 * t * t2_ad;
    rt[(size_t)k * L] += R(T_ad);
    if (rv && ((int)o[OPT_MASK] >> h2o_bit & 1)) rv[(size_t)k * L] += R(V_ad);
  }
}

}  // namespace crtm
