// Reverse mode of one scattering layer's optics for the cloudy K-matrix and
// adjoint: from the adjoints of the layer's transmission T, reflection R and
// source (what the adding adjoint hands back) to the adjoints of its gas
// optical depth, temperature and each cloud's / aerosol's amount and LUT
// coordinates, in one sweep for all of them.
//
// Reference behaviour followed (JCSDA/CRTMv3):
//   MOM_AD, CRTM_AMOM_layer_AD   src/RTSolution/ADA/ADA_Module.f90:439-549, 1760-2084
//   ASYMTX_AD                    src/CRTM_Utility/CRTM_Utility.f90:1158-1193
//   Phase matrix adjoint         src/RTSolution/Common_RTSolution.f90:2548-2940
//   AtmOptics_Combine_AD         src/AtmOptics/CRTM_AtmOptics.f90:628-784
//   CloudScatter_AD, AerosolScatter_AD (LUT part: derivative numbers here)
//                                src/AtmScatter/CRTM_CloudScatter.f90:737-926,
//                                src/AtmScatter/CRTM_AerosolScatter.f90:614-771
//
// Differences of form (same derivatives):
//   - The eigen-decomposition's adjoint uses the general formula for
//     HH = E diag(lam) E^-1 with the eigenvectors' scaling left free: MOM's
//     T, R and source do not depend on that scaling, so the adjoint of E is
//     orthogonal to it and no normalisation convention enters.
//   - The forward quantities the adjoint needs are recomputed from the
//     layer's inputs inside the call instead of being read from a tape.
//   - The LUT interpolation of each species is differentiated in forward mode
//     (its four inputs: amount, two LUT coordinates, temperature), in FP64,
//     which costs a few LUT evaluations and no matrix work.
#pragma once

#include "scatter_physics.cuh"

namespace crtm {

// C = A^T B
template <int NZ, class T>
CRTM_HD void mat_mul_tn(int n, const Mat<NZ, T>& A, const Mat<NZ, T>& B, Mat<NZ, T>& C) {
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      T s = T(0.0);
      for (int k = 0; k < n; k++) s += A.a[k][i] * B.a[k][j];
      C.a[i][j] = s;
    }
}

// C = A B^T
template <int NZ, class T>
CRTM_HD void mat_mul_nt(int n, const Mat<NZ, T>& A, const Mat<NZ, T>& B, Mat<NZ, T>& C) {
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      T s = T(0.0);
      for (int k = 0; k < n; k++) s += A.a[i][k] * B.a[j][k];
      C.a[i][j] = s;
    }
}

// Adjoint of an inverse Y = X^-1 given Y and Y_b: X_b = -Y^T Y_b Y^T, in Xb
// (tmp is scratch).
template <int NZ, class T>
CRTM_HD void inverse_adjoint(int n, const Mat<NZ, T>& Y, const Mat<NZ, T>& Yb, Mat<NZ, T>& Xb, Mat<NZ, T>& tmp) {
  mat_mul_tn(n, Y, Yb, tmp);   // Y^T Y_b
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      T s = T(0.0);
      for (int k = 0; k < n; k++) s += tmp.a[i][k] * Y.a[j][k];
      Xb.a[i][j] = -s;
    }
}

// Adjoint of ada_layer (CRTM_AMOM_layer + MOM for one scattering layer,
// azimuth order 0, thermal source only).  Given the adjoints T_b, R_b, src_b
// of the layer's transmission, reflection and source, returns the adjoints of
// its single-scattering albedo (w_b), optical depth (tau_b), forward and
// backward phase blocks (ff_b, bb_b, full nZ x nZ: an entry's adjoint as that
// entry is read) and Planck radiance (B_b).  Returns false where the forward
// factorisation fails.  gap: as in ada_layer.
template <int NZ, class T>
CRTM_HD bool ada_layer_adjoint(int nS, int nZ, T w, T tau, const T* mu, const T* wt, const Mat<NZ, T>& ff,
                               const Mat<NZ, T>& bb, T B, const Mat<NZ, T>& T_b, const Mat<NZ, T>& R_b,
                               const T* src_b, T* w_b, T* tau_b, Mat<NZ, T>& ff_b, Mat<NZ, T>& bb_b, T* B_b,
                               double* gap = nullptr) {
  const int n = nZ;
  const bool sensor_row = nZ == nS + 1;
  if (gap) *gap = 1.0;
  if (tau < T(DELTA_OPTICAL_DEPTH)) {   // thin layer (first-order scattering)
    const T s = tau * w;
    T s_b = T(0.0), tb = T(0.0), bsum = T(0.0);
    for (int i = 0; i < n; i++) {
      const T c = s / mu[i];
      T th = T(0.0);
      for (int j = 0; j < n; j++)
        th += c * (bb.a[i][j] + ff.a[i][j]) * wt[j] + (i == j ? T(1.0) - tau / mu[i] : T(0.0));
      bsum += src_b[i] * (T(1.0) - th);
      const T th_b = -src_b[i] * B;
      T c_b = T(0.0);
      for (int j = 0; j < n; j++) {
        const T rb = R_b.a[i][j] + th_b, tbij = T_b.a[i][j] + th_b;
        c_b += (rb * bb.a[i][j] + tbij * ff.a[i][j]) * wt[j];
        bb_b.a[i][j] = rb * c * wt[j];
        ff_b.a[i][j] = tbij * c * wt[j];
        if (i == j) tb -= tbij / mu[i];
      }
      s_b += c_b / mu[i];
    }
    *tau_b = tb + s_b * w;
    *w_b = s_b * tau;
    *B_b = bsum;
    return true;
  }
  // ---- forward, keeping what the reverse sweep reads ----
  const T s = w < T(MAX_ALBEDO) ? w : T(MAX_ALBEDO);
  Mat<NZ, T> E, iX, Gp, Gm, iGm, A2, iGA, Tm, Rm, M1, M2, M3;
  T lam[NZ], ev[NZ], ex[NZ];
  if (!mom_eigen<NZ, T>(nS, nZ, s, mu, wt, ff, bb, E, lam, iX, M1, M2, M3, gap)) return false;
  if (!mat_invert(n, iX)) return false;   // (PP - PM)^-1
  for (int i = 0; i < n; i++) {
    ev[i] = lam[i] > T(0.0) ? sqrt(lam[i]) : T(0.0);
    ex[i] = exp(-ev[i] * tau);
  }
  // EF = (PP-PM)^-1 E diag(ev);  Gp = (E + EF)/2, Gm = (E - EF)/2
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      T v = T(0.0);
      for (int k = 0; k < n; k++) v += iX.a[i][k] * E.a[k][j];
      v *= ev[j];
      Gp.a[i][j] = T(0.5) * (E.a[i][j] + v);
      Gm.a[i][j] = T(0.5) * (E.a[i][j] - v);
    }
  iGm = Gm;
  if (!mat_invert(n, iGm)) return false;
  // A2 = Gm^-1 Gp diag(ex)
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      T v = T(0.0);
      for (int k = 0; k < n; k++) v += iGm.a[i][k] * Gp.a[k][j];
      A2.a[i][j] = v * ex[j];
    }
  // GA = Gm - Gp diag(ex) A2;  Tt = Gm diag(ex) - Gp A2 (M1);  Rt = Gp - Gm diag(ex) A2 (M2)
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      T a5 = T(0.0), a3 = T(0.0), a6 = T(0.0);
      for (int k = 0; k < n; k++) {
        a5 += Gp.a[i][k] * ex[k] * A2.a[k][j];
        a3 += Gp.a[i][k] * A2.a[k][j];
        a6 += Gm.a[i][k] * ex[k] * A2.a[k][j];
      }
      iGA.a[i][j] = Gm.a[i][j] - a5;
      M1.a[i][j] = Gm.a[i][j] * ex[j] - a3;
      M2.a[i][j] = Gp.a[i][j] - a6;
    }
  if (!mat_invert(n, iGA)) return false;
  mat_mul(n, M1, iGA, Tm);
  mat_mul(n, M2, iGA, Rm);
  // ---- reverse ----
  // Scratch schedule (12 matrices): E, iX, Gp, Gm, iGm, A2, iGA are the
  // forward's; Tm, Rm, M1, M2, M3 are reused as each earlier value dies.
  // src_i = (1 - th_i) B with th_i the row sum of T + R over the quadrature
  // columns (and T's diagonal on the sensor row).
  Mat<NZ, T>& Tb = M1;   // total T adjoint
  Mat<NZ, T>& Rb = M2;   // total R adjoint
  T bsum = T(0.0);
  for (int i = 0; i < n; i++) {
    T th = T(0.0);
    for (int j = 0; j < nS; j++) th += Tm.a[i][j] + Rm.a[i][j];
    if (sensor_row && i == n - 1) th += Tm.a[i][i];
    bsum += src_b[i] * (T(1.0) - th);
    const T th_b = -src_b[i] * B;
    for (int j = 0; j < n; j++) {
      const bool in_th = j < nS || (sensor_row && i == n - 1 && j == i);
      Tb.a[i][j] = T_b.a[i][j] + (in_th ? th_b : T(0.0));
      Rb.a[i][j] = R_b.a[i][j] + (j < nS ? th_b : T(0.0));
    }
  }
  *B_b = bsum;
  // T = Tt GA^-1, R = Rt GA^-1:
  //   GA_b = -(T^T Tb + R^T Rb) GA^-T;  Tt_b = Tb GA^-T;  Rt_b = Rb GA^-T
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      T v = T(0.0);
      for (int k = 0; k < n; k++) v += Tm.a[k][i] * Tb.a[k][j] + Rm.a[k][i] * Rb.a[k][j];
      M3.a[i][j] = v;
    }
  Mat<NZ, T>& GAb = Tm;
  mat_mul_nt(n, M3, iGA, GAb);
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) GAb.a[i][j] = -GAb.a[i][j];
  Mat<NZ, T>& Ttb = Rm;
  Mat<NZ, T>& Rtb = M3;
  mat_mul_nt(n, Tb, iGA, Ttb);
  mat_mul_nt(n, Rb, iGA, Rtb);
  // Tt = Gm diag(ex) - Gp A2;  Rt = Gp - Gm diag(ex) A2;  GA = Gm - Gp diag(ex) A2:
  //   Gm_b = GA_b + (Tt_b - Rt_b A2^T) diag(ex)
  //   Gp_b = Rt_b - Tt_b A2^T - GA_b A2^T diag(ex)
  //   ex_b_j = sum_i Gm_ij (Tt_b - Rt_b A2^T)_ij - Gp_ij (GA_b A2^T)_ij
  //   A2_b = -(Gp^T Tt_b + diag(ex) (Gm^T Rt_b + Gp^T GA_b))
  Mat<NZ, T>& Gmb = M1;   // Tb, Rb are dead
  Mat<NZ, T>& Gpb = M2;
  T ex_b[NZ];
  for (int j = 0; j < n; j++) ex_b[j] = T(0.0);
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      T rA = T(0.0), tA = T(0.0), gA = T(0.0);
      for (int k = 0; k < n; k++) {
        rA += Rtb.a[i][k] * A2.a[j][k];
        tA += Ttb.a[i][k] * A2.a[j][k];
        gA += GAb.a[i][k] * A2.a[j][k];
      }
      Gmb.a[i][j] = GAb.a[i][j] + (Ttb.a[i][j] - rA) * ex[j];
      Gpb.a[i][j] = Rtb.a[i][j] - tA - gA * ex[j];
      ex_b[j] += Gm.a[i][j] * (Ttb.a[i][j] - rA) - Gp.a[i][j] * gA;
    }
  Mat<NZ, T>& A2b = iGA;  // iGA is dead
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      T v = T(0.0);
      for (int k = 0; k < n; k++)
        v += Gp.a[k][i] * Ttb.a[k][j] + ex[i] * (Gm.a[k][i] * Rtb.a[k][j] + Gp.a[k][i] * GAb.a[k][j]);
      A2b.a[i][j] = -v;
    }
  // A2 = Gm^-1 A1 with A1 = Gp diag(ex):  A1_b = Gm^-T A2_b;  (Gm^-1)_b = A2_b A1^T;
  //   Gp_b += A1_b diag(ex);  ex_b_j += sum_i A1_b_ij Gp_ij;  Gm_b += -Gm^-T (Gm^-1)_b Gm^-T
  Mat<NZ, T>& A1b = Tm;   // GA_b, Tt_b, Rt_b are dead
  Mat<NZ, T>& iGmb = Rm;
  mat_mul_tn(n, iGm, A2b, A1b);
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      T v = T(0.0);
      for (int k = 0; k < n; k++) v += A2b.a[i][k] * Gp.a[j][k] * ex[k];
      iGmb.a[i][j] = v;
    }
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      Gpb.a[i][j] += A1b.a[i][j] * ex[j];
      ex_b[j] += A1b.a[i][j] * Gp.a[i][j];
    }
  inverse_adjoint(n, iGm, iGmb, M3, A1b);
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) Gmb.a[i][j] += M3.a[i][j];
  // Gp = (E + EF)/2, Gm = (E - EF)/2
  Mat<NZ, T>& Eb = M2;
  Mat<NZ, T>& EFb = M1;
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      const T p = Gpb.a[i][j], q = Gmb.a[i][j];
      Eb.a[i][j] = T(0.5) * (p + q);
      EFb.a[i][j] = T(0.5) * (p - q);
    }
  // EF = iX E diag(ev):  iX_b = EF_b (E diag(ev))^T;  EV_b = iX^T EF_b;
  //   E_b += EV_b diag(ev);  ev_b_j = sum_i EV_b_ij E_ij
  Mat<NZ, T>& iXb = Tm;
  Mat<NZ, T>& EVb = Rm;
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      T v = T(0.0);
      for (int k = 0; k < n; k++) v += EFb.a[i][k] * E.a[j][k] * ev[k];
      iXb.a[i][j] = v;
    }
  mat_mul_tn(n, iX, EFb, EVb);
  T lam_b[NZ];
  T tb = T(0.0);
  for (int j = 0; j < n; j++) {
    T v = T(0.0);
    for (int i = 0; i < n; i++) {
      v += EVb.a[i][j] * E.a[i][j];
      Eb.a[i][j] += EVb.a[i][j] * ev[j];
    }
    // ex_j = exp(-ev_j tau), ev_j = sqrt(lam_j)
    const T ev_b = v - tau * ex[j] * ex_b[j];
    tb -= ev[j] * ex[j] * ex_b[j];
    lam_b[j] = lam[j] > T(0.0) ? T(0.5) * ev_b / ev[j] : T(0.0);
  }
  *tau_b = tb;
  // X = PP - PM inverted:  X_b = -iX^T iX_b iX^T  (in M3)
  inverse_adjoint(n, iX, iXb, M3, A2);
  // HH = E diag(lam) E^-1:  HH_b = E^-T (diag(lam_b) + F o (E^T E_b)) E^T,
  // F_ij = 1 / (lam_j - lam_i) off the diagonal
  Mat<NZ, T>& Ei = Gp;    // Gp, Gm, iGm are dead
  Mat<NZ, T>& Mx = Gm;
  Ei = E;
  if (!mat_invert(n, Ei)) return false;
  mat_mul_tn(n, E, Eb, Mx);
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++)
      Mx.a[i][j] = (i == j) ? lam_b[i] : Mx.a[i][j] / (lam[j] - lam[i]);
  Mat<NZ, T>& HHb = Rm;
  mat_mul_tn(n, Ei, Mx, Tm);   // E^-T M
  mat_mul_nt(n, Tm, E, HHb);   // (E^-T M) E^T
  // HH = X Y with X = PP - PM, Y = PP + PM (rebuilt from the phase blocks):
  //   X_b += HH_b Y^T;  Y_b = X^T HH_b
  Mat<NZ, T>& X = iGm;
  Mat<NZ, T>& Y = A2;
  for (int i = 0; i < n; i++) {
    const T c = s / mu[i];
    for (int j = 0; j < n; j++) {
      const T f = c * ff.a[i][j] * wt[j] - (i == j ? T(1.0) / mu[i] : T(0.0)), b = c * bb.a[i][j] * wt[j];
      X.a[i][j] = f - b;
      Y.a[i][j] = f + b;
    }
  }
  Mat<NZ, T>& Yb = Tm;
  mat_mul_tn(n, X, HHb, Yb);
  mat_mul_nt(n, HHb, Y, M1);
  // f = c_i ff_ij wt_j - delta_ij / mu_i, b = c_i bb_ij wt_j, c_i = s / mu_i;
  // X = f - b, Y = f + b
  T s_b = T(0.0);
  for (int i = 0; i < n; i++) {
    const T c = s / mu[i];
    T c_b = T(0.0);
    for (int j = 0; j < n; j++) {
      const T xb = M3.a[i][j] + M1.a[i][j];
      const T fb = xb + Yb.a[i][j], bbv = Yb.a[i][j] - xb;
      ff_b.a[i][j] = fb * c * wt[j];
      bb_b.a[i][j] = bbv * c * wt[j];
      c_b += (fb * ff.a[i][j] + bbv * bb.a[i][j]) * wt[j];
    }
    s_b += c_b / mu[i];
  }
  *w_b = w < T(MAX_ALBEDO) ? s_b : T(0.0);
  return true;
}


// Adjoint of phase_blocks (CRTM_Phase_Matrix for m = 0 and Normalize_Phase):
// given the adjoints ff_b, bb_b of the normalised forward/backward blocks
// (full matrices, an entry's adjoint as that entry is read), returns the
// adjoints pc_b[l] of the Legendre terms pc[l], l < nleg.  The normalisation
// scales row i of the upper triangle by sc_i = (1 - carried_i) / nf_i in
// turn, with carried_i the weighted sum of row i's already-normalised
// entries left of the diagonal; the sensor angle's column is divided by the
// carried sum of its row.  The forward values are recomputed here.
template <int NZ, class T>
CRTM_HD void phase_blocks_adjoint(int nS, int nZ, int nleg, const T* pc, const T (*P)[SC_NLEG_MAX + 1], const T* wt,
                                  const Mat<NZ, T>& ff_b, const Mat<NZ, T>& bb_b, T* pc_b) {
  Mat<NZ, T> f0, b0, fb, bq;   // clamped unscaled blocks (upper triangle) and their adjoints
  unsigned clampf[NZ] = {0}, clampb[NZ] = {0};
  for (int i = 0; i < nZ; i++)
    for (int j = i; j < nZ; j++) {
      T f = T(0.0), b = T(0.0);
      for (int l = 0; l < nleg; l++) {
        const T t = pc[l] * P[i][l] * P[j][l];
        f += t;
        b += (l & 1) ? -t : t;
      }
      if (f < T(0.0)) { f = T(PHASE_THRESHOLD); clampf[i] |= 1u << j; }
      if (b < T(0.0)) { b = T(PHASE_THRESHOLD); clampb[i] |= 1u << j; }
      f0.a[i][j] = f;
      b0.a[i][j] = b;
      fb.a[i][j] = T(0.0);
      bq.a[i][j] = T(0.0);
    }
  // forward scales
  T sc[NZ], nf[NZ];
  T carried = T(0.0);
  for (int i = 0; i < nS; i++) {
    T v = T(0.0);
    for (int j = i; j < nZ; j++) v += (f0.a[i][j] + b0.a[i][j]) * wt[j];
    nf[i] = v;
    sc[i] = (T(1.0) - carried) / v;
    carried = T(0.0);
    if (i + 1 < nZ)
      for (int j = 0; j <= i; j++) carried += (f0.a[j][i + 1] + b0.a[j][i + 1]) * sc[j] * wt[j];
  }
  const bool sensor = nS < nZ;
  const int z = nZ - 1;
  const T cz = carried;   // the sensor column's divisor (when sensor)
  T sc_b[NZ];
  for (int i = 0; i < nZ; i++) sc_b[i] = T(0.0);
  T cz_b = T(0.0);
  // final entries: (i <= j) f0_ij sc_i, the sensor column further / cz
  for (int i = 0; i < nZ; i++)
    for (int j = i; j < nZ; j++) {
      const T hf = (i == j) ? ff_b.a[i][i] : ff_b.a[i][j] + ff_b.a[j][i];
      const T hb = (i == j) ? bb_b.a[i][i] : bb_b.a[i][j] + bb_b.a[j][i];
      const T si = i < nS ? sc[i] : T(1.0);
      if (sensor && j == z) {
        fb.a[i][j] += hf * si / cz;
        bq.a[i][j] += hb * si / cz;
        if (i < nS) sc_b[i] += (hf * f0.a[i][j] + hb * b0.a[i][j]) / cz;
        cz_b -= (hf * f0.a[i][j] + hb * b0.a[i][j]) * si / (cz * cz);
      } else {
        fb.a[i][j] += hf * si;
        bq.a[i][j] += hb * si;
        sc_b[i] += hf * f0.a[i][j] + hb * b0.a[i][j];
      }
    }
  if (sensor)   // cz = sum_{j < z} (f0_jz + b0_jz) sc_j wt_j
    for (int j = 0; j < z; j++) {
      fb.a[j][z] += cz_b * sc[j] * wt[j];
      bq.a[j][z] += cz_b * sc[j] * wt[j];
      sc_b[j] += cz_b * (f0.a[j][z] + b0.a[j][z]) * wt[j];
    }
  for (int i = nS - 1; i >= 0; i--) {   // sc_i = (1 - carried_i) / nf_i
    const T car_b = -sc_b[i] / nf[i], nf_b = -sc_b[i] * sc[i] / nf[i];
    for (int j = i; j < nZ; j++) {
      fb.a[i][j] += nf_b * wt[j];
      bq.a[i][j] += nf_b * wt[j];
    }
    for (int j = 0; j < i; j++) {   // carried_i = sum_{j < i} (f0_ji + b0_ji) sc_j wt_j
      fb.a[j][i] += car_b * sc[j] * wt[j];
      bq.a[j][i] += car_b * sc[j] * wt[j];
      sc_b[j] += car_b * (f0.a[j][i] + b0.a[j][i]) * wt[j];
    }
  }
  for (int l = 0; l < nleg; l++) pc_b[l] = T(0.0);
  for (int i = 0; i < nZ; i++)
    for (int j = i; j < nZ; j++) {
      const T gf = (clampf[i] >> j) & 1u ? T(0.0) : fb.a[i][j];
      const T gb = (clampb[i] >> j) & 1u ? T(0.0) : bq.a[i][j];
      for (int l = 0; l < nleg; l++) pc_b[l] += ((l & 1) ? gf - gb : gf + gb) * P[i][l] * P[j][l];
    }
}

// Bulk optics of a layer in T: the species sums (optical depth od0, scattering
// bs, phase sums ps[l]) and the combine with delta truncation
// (CRTM_AtmOptics_Combine): optical depth od, single-scattering albedo ssa and
// the normalised Legendre terms p[l] (p[0] = 1/2).
template <class T>
struct LayerBulk {
  T od0, bs, od, ssa;
  T ps[SC_NLEG_MAX + 1], p[SC_NLEG_MAX + 1];
};

template <class T>
CRTM_HD int layer_bulk(const CloudyColumn& in, const CloudLut& lut, int nleg, int loff, int k, T gas_od, T tk,
                       LayerBulk<T>& L) {
  L.od0 = gas_od;
  L.bs = T(0.0);
  for (int l = 0; l <= nleg; l++) L.ps[l] = T(0.0);
  if (const int rc = species_sums<T>(in, lut, nleg, loff, k, tk, NoSeed(), &L.od0, &L.bs, L.ps)) return rc;
  L.od = L.od0;
  L.ssa = L.bs;
  if (L.bs > T(BS_THRESHOLD)) {
    const T w = L.bs / L.od0;
    for (int l = 1; l <= nleg; l++) L.p[l] = L.ps[l] / L.bs;
    L.p[0] = T(0.5);
    const T f = L.p[nleg];
    L.od = (T(1.0) - f * w) * L.od0;
    L.ssa = (T(1.0) - f) * w / (T(1.0) - f * w);
  }
  return 0;
}

// Seed of one species' forward-mode pass: amount, first and second LUT
// coordinate on directions 0, 1, 2 (temperature on 3 is seeded by the caller).
struct SpeciesSeed {
  int sp;
  template <class S>
  CRTM_HD void operator()(int s, S& amount, S& c1, S& c2) const {
    if (s != sp) return;
    amount.d[0] = 1.0;
    c1.d[1] = 1.0;
    c2.d[2] = 1.0;
  }
};

// The adjoints a layer's record hands to its optics, folded to the bulk
// quantities: optical depth (od_b), single-scattering albedo (ssa_b),
// normalised Legendre terms (p_b[l], l < nleg) and Planck radiance (B_b).
template <class T>
struct BulkAdjoint {
  T od_b, ssa_b, B_b;
  T p_b[SC_NLEG_MAX + 1];
};

// Reverse of the combine and the species sums: from a layer's bulk adjoint to
// the adjoints of its gas optical depth (g[0]), temperature (g[1]) and each
// species' amount and LUT coordinates (gs[sp][0..2]; nsp species).
template <class T>
CRTM_HD int bulk_to_inputs(const CloudyColumn& in, const CloudLut& lut, int nleg, int loff, int k, T tk,
                           const LayerBulk<T>& L, const BulkAdjoint<T>& A, int nsp, double* g, double (*gs)[3]) {
  // combine: w = bs / od0, p_l = ps_l / bs, f = p_nleg,
  //   od = (1 - f w) od0, ssa = (1 - f) w / (1 - f w)
  T od0_b = A.od_b, bs_b = T(0.0), ps_b[SC_NLEG_MAX + 1];
  for (int l = 0; l <= nleg; l++) ps_b[l] = T(0.0);
  if (L.bs > T(BS_THRESHOLD)) {
    const T w = L.bs / L.od0, f = L.p[nleg], D = T(1.0) - f * w;
    const T f_b = A.ssa_b * w * (w - T(1.0)) / (D * D) - A.od_b * w * L.od0;
    const T w_b = A.ssa_b * (T(1.0) - f) / (D * D) - A.od_b * f * L.od0;
    od0_b = A.od_b * D - w_b * w / L.od0;
    bs_b = w_b / L.od0;
    for (int l = 1; l <= nleg; l++) {
      const T pb = l < nleg ? A.p_b[l] : f_b;
      ps_b[l] = pb / L.bs;
      bs_b -= pb * L.p[l] / L.bs;
    }
  } else {
    bs_b = A.ssa_b;
  }
  g[0] = (double)od0_b;
  // Planck radiance of the layer temperature
  const double te = in.b1 + in.b2 * (double)tk, ee = exp(in.c2 / te);
  double gt = (double)A.B_b * in.c1 * in.c2 * ee * in.b2 / (te * te * (ee - 1.0) * (ee - 1.0));
  // each species' share in forward mode: amount, c1, c2 and the temperature,
  // in FP64 in every form (the LUT derivatives are differences of nearby
  // table values: in FP32 they cost the radius Jacobians ~1e-3; the LUT work
  // is a small part of the layer's)
  using D4 = Dual<4, double>;
  for (int sp = 0; sp < nsp; sp++) {
    D4 od(0.0), bs(0.0), ps[SC_NLEG_MAX + 1];
    D4 td(double(tk), 0);
    td.d[3] = 1.0;
    if (const int rc = species_share<D4>(in, lut, nleg, loff, k, sp, td, SpeciesSeed{sp}, &od, &bs, ps)) return rc;
    double gg[4];
    for (int d = 0; d < 4; d++) {
      double v = double(od0_b) * od.d[d] + double(bs_b) * bs.d[d];
      for (int l = 1; l <= nleg; l++) v += double(ps_b[l]) * ps[l].d[d];
      gg[d] = v;
    }
    gs[sp][0] = gg[0];
    gs[sp][1] = gg[1];
    gs[sp][2] = gg[2];
    gt += gg[3];
  }
  g[1] = gt;
  return 0;
}

// Reverse mode of layer_optics for an ADA or clear layer (not SOI): given the
// adjoints of the layer's record (scattering layer: T_b, R_b, src_b; clear
// layer: od_b, and B_b of its Planck radiance, which the adding reads outside
// the record), g[0] = d/d(gas optical depth), g[1] = d/d(temperature) and
// gs[sp][0..2] = d/d(amount, c1, c2) of species sp (the contraction of the
// layer's optics derivatives with those adjoints).  Layers whose MOM
// eigenbasis is nearly defective take the derivatives through MOM at shifted
// sensor angles, as layer_optics_dual does.  Returns the layer kind (1
// scattering, 0 clear) or a negative error; kind_rec is the record's kind
// (the forward's); a mismatch returns -7.
template <int NZ, class T>
CRTM_HD int layer_adjoint(const CloudyColumn& in, const CloudLut& lut, const StreamSet<NZ, double>& St, int k,
                          double gas_od, int kind_rec, const Mat<NZ, double>& T_b, const Mat<NZ, double>& R_b,
                          const double* src_b, double od_b, double B_b, double* g, double (*gs)[3]) {
  const int nleg = St.nleg, nS = St.nS, nZ = St.nZ;
  const T tk = T(in.temperature[k]);
  LayerBulk<T> L;
  if (const int rc = layer_bulk<T>(in, lut, nleg, St.loff, k, T(gas_od), tk, L)) return rc;
  const int nsp = scattering_species(in, nleg, St.loff);
  if (nsp < 0) return nsp;
  BulkAdjoint<T> A;
  A.ssa_b = T(0.0);
  for (int l = 0; l <= nleg; l++) A.p_b[l] = T(0.0);
  int kind = L.ssa > T(BS_THRESHOLD) ? 1 : 0;
  T mu[NZ], wt[NZ], P[NZ][SC_NLEG_MAX + 1];
  Mat<NZ, T> ff, bb;
  if (kind == 1) {
    for (int i = 0; i < nZ; i++) {
      mu[i] = T(St.mu[i]);
      wt[i] = T(St.wt[i]);
      for (int l = 0; l <= nleg; l++) P[i][l] = T(St.P[i][l]);
    }
    phase_blocks<NZ, T>(nS, nZ, nleg, L.p, P, wt, ff, bb);
    T mx = T(0.0);
    for (int i = 0; i < nZ; i++)
      for (int j = 0; j < nZ; j++) mx = fabs(ff.a[i][j]) > mx ? fabs(ff.a[i][j]) : mx;
    if (!(mx > T(0.0))) kind = 0;
  }
  if (kind != kind_rec) return -7;
  if (kind == 0) {
    A.od_b = T(od_b);
    A.B_b = T(B_b);
  } else {
    const double te = in.b1 + in.b2 * in.temperature[k];
    const T B = T(in.c1 / (exp(in.c2 / te) - 1.0));
    Mat<NZ, T> Tb, Rb, ffb, bbb;
    T sb[NZ];
    for (int i = 0; i < nZ; i++) {
      sb[i] = T(src_b[i]);
      for (int j = 0; j < nZ; j++) { Tb.a[i][j] = T(T_b.a[i][j]); Rb.a[i][j] = T(R_b.a[i][j]); }
    }
    double gap = 1.0;
    T w_b, tau_b, Bb;
    const bool ok = ada_layer_adjoint<NZ, T>(nS, nZ, L.ssa, L.od, mu, wt, ff, bb, B, Tb, Rb, sb, &w_b, &tau_b, ffb,
                                             bbb, &Bb, &gap);
    if constexpr (std::is_same<T, float>::value) {
      // the FP32 reverse sweep near a nearly defective eigenbasis, or where
      // its factorisation failed: this layer in FP64
      if (!ok || gap < FP32_ADJ_GAP_MIN)
        return layer_adjoint<NZ, double>(in, lut, St, k, gas_od, kind_rec, T_b, R_b, src_b, od_b, B_b, g, gs);
    }
    if (!ok) return -5;
    if (gap < SENSOR_GAP_MIN && nZ == nS + 1) {
      // A quadrature eigenvalue of MOM nearly meets the sensor angle's: the
      // derivatives through the nearly defective eigenbasis lose about
      // eps / gap^2.  T, R and the source are smooth in the sensor angle, so
      // the layer's bulk adjoints are taken at sensor angles mu (1 +- h),
      // h = 1e-3 and 2e-3, as the Richardson extrapolation
      // (4 D(h) - D(2h)) / 3 of the symmetric means.
      BulkAdjoint<T> S2;
      S2.od_b = S2.ssa_b = S2.B_b = T(0.0);
      for (int l = 0; l <= nleg; l++) S2.p_b[l] = T(0.0);
      int n_ok = 0;
      const int zz = nZ - 1;
      for (int side = 0; side < 4; side++) {
        const double fsh = (side & 1 ? -1.0 : 1.0) * (side < 2 ? SENSOR_SHIFT : 2.0 * SENSOR_SHIFT);
        const T wgt = T((side < 2 ? 4.0 : -1.0) / 6.0);
        T mu2[NZ], P2[NZ][SC_NLEG_MAX + 1];
        for (int i = 0; i < nZ; i++) {
          mu2[i] = mu[i];
          for (int l = 0; l <= nleg; l++) P2[i][l] = P[i][l];
        }
        const double m2 = St.mu[zz] * (1.0 + fsh);
        double q[SC_NLEG_MAX + 1];
        q[0] = 1.0;
        if (nleg > 0) q[1] = m2;
        for (int j = 1; j < nleg; j++) q[j + 1] = ((2 * j + 1) * m2 * q[j] - j * q[j - 1]) / (j + 1);
        mu2[zz] = T(m2);
        for (int l = 0; l <= nleg; l++) P2[zz][l] = T(q[l]);
        Mat<NZ, T> ff2, bb2, ffb2, bbb2;
        phase_blocks<NZ, T>(nS, nZ, nleg, L.p, P2, wt, ff2, bb2);
        T w2, t2, B2, pb2[SC_NLEG_MAX + 1];
        if (!ada_layer_adjoint<NZ, T>(nS, nZ, L.ssa, L.od, mu2, wt, ff2, bb2, B, Tb, Rb, sb, &w2, &t2, ffb2, bbb2,
                                      &B2))
          break;
        phase_blocks_adjoint<NZ, T>(nS, nZ, nleg, L.p, P2, wt, ffb2, bbb2, pb2);
        S2.od_b += wgt * t2;
        S2.ssa_b += wgt * w2;
        S2.B_b += wgt * B2;
        for (int l = 0; l < nleg; l++) S2.p_b[l] += wgt * pb2[l];
        n_ok++;
      }
      if (n_ok == 4) {   // else (a shifted angle failed) keep the direct derivatives
        if (const int rc = bulk_to_inputs<T>(in, lut, nleg, St.loff, k, tk, L, S2, nsp, g, gs)) return rc;
        return 1;
      }
    }
    A.od_b = tau_b;
    A.ssa_b = w_b;
    A.B_b = Bb;
    phase_blocks_adjoint<NZ, T>(nS, nZ, nleg, L.p, P, wt, ffb, bbb, A.p_b);
  }
  if (const int rc = bulk_to_inputs<T>(in, lut, nleg, St.loff, k, tk, L, A, nsp, g, gs)) return rc;
  return kind;
}
}  // namespace crtm
