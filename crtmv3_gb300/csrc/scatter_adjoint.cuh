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
  // ---- forward in the loss form of ada_layer_loss, keeping what the
  // reverse sweep reads.  With P = Gm^-1 Gp, D = diag(1 - exp(-ev tau)) and
  // e = diag(exp(-ev tau)):  W = D P e + P D,  Q = Gm - Gp P,  GA = Q + Gp W,
  // U = (Q D + Gp W) GA^-1 = I - T,  R = (Gp D + Gm D P e) GA^-1.  Every
  // term of U and R is O(tau) for a thin layer, and so is every adjoint that
  // reaches the eigen-decomposition below: the FP32 form keeps its relative
  // accuracy where the plain form T = Tt GA^-1 loses it to cancellation.
  const T s = w < T(MAX_ALBEDO) ? w : T(MAX_ALBEDO);
  Mat<NZ, T> E, iX, Gp, Gm, iGm, P, W, iGA, Um, Rm, T1, T2;
  T lam[NZ], ev[NZ], ex[NZ], dx[NZ], buf[NZ];
  if (!mom_eigen<NZ, T>(nS, nZ, s, mu, wt, ff, bb, E, lam, iX, T1, T2, Um, gap)) return false;
  if (!mat_invert(n, iX)) return false;   // (PP - PM)^-1
  for (int i = 0; i < n; i++) {
    ev[i] = lam[i] > T(0.0) ? sqrt(lam[i]) : T(0.0);
    ex[i] = exp(-ev[i] * tau);
    dx[i] = -expm1(-ev[i] * tau);
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
  mat_mul(n, iGm, Gp, P);
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) W.a[i][j] = dx[i] * P.a[i][j] * ex[j] + P.a[i][j] * dx[j];
  for (int i = 0; i < n; i++)   // Q (T1)
    for (int j = 0; j < n; j++) {
      T v = T(0.0);
      for (int k = 0; k < n; k++) v += Gp.a[i][k] * P.a[k][j];
      T1.a[i][j] = Gm.a[i][j] - v;
    }
  // GA (iGA), U numerator (T1, in place over Q), R numerator (T2)
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      T gw = T(0.0), gd = T(0.0);
      for (int k = 0; k < n; k++) {
        gw += Gp.a[i][k] * W.a[k][j];
        gd += Gm.a[i][k] * dx[k] * P.a[k][j];
      }
      iGA.a[i][j] = T1.a[i][j] + gw;
      T1.a[i][j] = T1.a[i][j] * dx[j] + gw;
      T2.a[i][j] = Gp.a[i][j] * dx[j] + gd * ex[j];
    }
  if (!mat_invert(n, iGA)) return false;
  mat_mul(n, T1, iGA, Um);
  mat_mul(n, T2, iGA, Rm);
  // ---- reverse ----
  // src_i = a_i B with a_i the row sum of U - R over the quadrature columns
  // (and U's diagonal on the sensor row); U_b = -T_b.  U_b in T1, R_b in T2.
  T bsum = T(0.0);
  for (int i = 0; i < n; i++) {
    T a = T(0.0);
    for (int j = 0; j < nS; j++) a += Um.a[i][j] - Rm.a[i][j];
    if (sensor_row && i == n - 1) a += Um.a[i][i];
    bsum += src_b[i] * a;
    const T sb = src_b[i] * B;
    for (int j = 0; j < n; j++) {
      const bool in_a = j < nS || (sensor_row && i == n - 1 && j == i);
      T1.a[i][j] = (in_a ? sb : T(0.0)) - T_b.a[i][j];
      T2.a[i][j] = R_b.a[i][j] - (j < nS ? sb : T(0.0));
    }
  }
  *B_b = bsum;
  // U = Un GA^-1, R = Rn GA^-1:  Un_b = U_b GA^-T, Rn_b = R_b GA^-T (row by
  // row in place), then GA_b = -(U^T Un_b + R^T Rn_b) into iGA
  for (int i = 0; i < n; i++) {
    for (int j = 0; j < n; j++) {
      T v = T(0.0);
      for (int k = 0; k < n; k++) v += T1.a[i][k] * iGA.a[j][k];
      buf[j] = v;
    }
    for (int j = 0; j < n; j++) T1.a[i][j] = buf[j];
    for (int j = 0; j < n; j++) {
      T v = T(0.0);
      for (int k = 0; k < n; k++) v += T2.a[i][k] * iGA.a[j][k];
      buf[j] = v;
    }
    for (int j = 0; j < n; j++) T2.a[i][j] = buf[j];
  }
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      T v = T(0.0);
      for (int k = 0; k < n; k++) v += Um.a[k][i] * T1.a[k][j] + Rm.a[k][i] * T2.a[k][j];
      iGA.a[i][j] = -v;
    }
  Mat<NZ, T>& GAb = iGA;
  Mat<NZ, T>& Qb = Um;   // U, R are dead
  Mat<NZ, T>& Wb = Rm;
  T dx_b[NZ], ex_b[NZ];
  for (int j = 0; j < n; j++) { dx_b[j] = T(0.0); ex_b[j] = T(0.0); }
  // Un = Q D + Gp W, GA = Q + Gp W:  Q_b = Un_b D + GA_b;  dx_b_j += sum_i Un_b_ij Q_ij;
  //   with S = Un_b + GA_b (T1):  W_b = Gp^T S;  Gp_b = S W^T
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      T v = T(0.0);
      for (int k = 0; k < n; k++) v += Gp.a[i][k] * P.a[k][j];
      dx_b[j] += T1.a[i][j] * (Gm.a[i][j] - v);
      Qb.a[i][j] = T1.a[i][j] * dx[j] + GAb.a[i][j];
      T1.a[i][j] += GAb.a[i][j];
    }
  mat_mul_tn(n, Gp, T1, Wb);
  Mat<NZ, T>& Gpb = iGA;   // GA_b is dead
  mat_mul_nt(n, T1, W, Gpb);
  Mat<NZ, T>& Gmb = T1;    // S is dead
  // Rn = Gp D + Gm D P e:  Gp_b += Rn_b D;  dx_b_j += sum_i Rn_b_ij Gp_ij;
  //   ex_b_j += sum_i Rn_b_ij (Gm D P)_ij;  with Z = Rn_b e:  Gm_b = Z P^T D,
  //   dx_b_k += sum_i Gm_ik (Z P^T)_ik;  P_b = D Gm^T Z (column by column into T2)
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      const T rb = T2.a[i][j];
      Gpb.a[i][j] += rb * dx[j];
      T g = T(0.0);
      for (int k = 0; k < n; k++) g += Gm.a[i][k] * dx[k] * P.a[k][j];
      dx_b[j] += rb * Gp.a[i][j];
      ex_b[j] += rb * g;
    }
  for (int i = 0; i < n; i++)
    for (int k = 0; k < n; k++) {
      T zp = T(0.0);
      for (int j = 0; j < n; j++) zp += T2.a[i][j] * ex[j] * P.a[k][j];
      Gmb.a[i][k] = zp * dx[k];
      dx_b[k] += Gm.a[i][k] * zp;
    }
  for (int j = 0; j < n; j++) {
    for (int k = 0; k < n; k++) {
      T v = T(0.0);
      for (int i = 0; i < n; i++) v += Gm.a[i][k] * T2.a[i][j];
      buf[k] = dx[k] * v * ex[j];
    }
    for (int k = 0; k < n; k++) T2.a[k][j] = buf[k];
  }
  Mat<NZ, T>& Pb = T2;
  // Q = Gm - Gp P:  Gm_b += Q_b;  Gp_b -= Q_b P^T;  P_b -= Gp^T Q_b
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      T a = T(0.0), b = T(0.0);
      for (int k = 0; k < n; k++) {
        a += Qb.a[i][k] * P.a[j][k];
        b += Gp.a[k][i] * Qb.a[k][j];
      }
      Gmb.a[i][j] += Qb.a[i][j];
      Gpb.a[i][j] -= a;
      Pb.a[i][j] -= b;
    }
  // W_ij = dx_i P_ij ex_j + P_ij dx_j
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      const T wb = Wb.a[i][j], pij = P.a[i][j];
      Pb.a[i][j] += wb * (dx[i] * ex[j] + dx[j]);
      dx_b[i] += wb * pij * ex[j];
      ex_b[j] += wb * dx[i] * pij;
      dx_b[j] += wb * pij;
    }
  // P = Gm^-1 Gp:  K = Gm^-T P_b;  Gp_b += K;  Gm_b -= K P^T
  Mat<NZ, T>& Kt = Um;   // Q_b is dead
  mat_mul_tn(n, iGm, Pb, Kt);
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      T v = T(0.0);
      for (int k = 0; k < n; k++) v += Kt.a[i][k] * P.a[j][k];
      Gpb.a[i][j] += Kt.a[i][j];
      Gmb.a[i][j] -= v;
    }
  // Gp = (E + EF)/2, Gm = (E - EF)/2
  Mat<NZ, T>& Eb = Gpb;
  Mat<NZ, T>& EFb = Gmb;
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      const T p = Gpb.a[i][j], q = Gmb.a[i][j];
      Eb.a[i][j] = T(0.5) * (p + q);
      EFb.a[i][j] = T(0.5) * (p - q);
    }
  // EF = iX E diag(ev):  iX_b = EF_b (E diag(ev))^T;  EV_b = iX^T EF_b;
  //   E_b += EV_b diag(ev);  ev_b_j = sum_i EV_b_ij E_ij
  Mat<NZ, T>& iXb = Um;   // K is dead
  Mat<NZ, T>& EVb = Rm;   // W_b is dead
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
    // ex_j = exp(-ev_j tau), dx_j = 1 - ex_j, ev_j = sqrt(lam_j)
    const T d = dx_b[j] - ex_b[j];
    const T ev_b = v + tau * ex[j] * d;
    tb += ev[j] * ex[j] * d;
    lam_b[j] = lam[j] > T(0.0) ? T(0.5) * ev_b / ev[j] : T(0.0);
  }
  *tau_b = tb;
  // X = PP - PM inverted:  X_b = -iX^T iX_b iX^T  (in P; W is scratch)
  Mat<NZ, T>& Xb = P;
  inverse_adjoint(n, iX, iXb, Xb, W);
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
  Mat<NZ, T>& HHb = Rm;   // EV_b is dead
  mat_mul_tn(n, Ei, Mx, T2);   // E^-T M  (P_b is dead)
  mat_mul_nt(n, T2, E, HHb);   // (E^-T M) E^T
  // HH = X Y with X = PP - PM, Y = PP + PM (rebuilt from the phase blocks):
  //   X_b += HH_b Y^T;  Y_b = X^T HH_b
  Mat<NZ, T>& X = iGm;
  Mat<NZ, T>& Y = W;
  for (int i = 0; i < n; i++) {
    const T c = s / mu[i];
    for (int j = 0; j < n; j++) {
      const T f = c * ff.a[i][j] * wt[j] - (i == j ? T(1.0) / mu[i] : T(0.0)), b = c * bb.a[i][j] * wt[j];
      X.a[i][j] = f - b;
      Y.a[i][j] = f + b;
    }
  }
  Mat<NZ, T>& Yb = T2;
  mat_mul_tn(n, X, HHb, Yb);
  mat_mul_nt(n, HHb, Y, Um);   // iX_b is dead
  // f = c_i ff_ij wt_j - delta_ij / mu_i, b = c_i bb_ij wt_j, c_i = s / mu_i;
  // X = f - b, Y = f + b
  T s_b = T(0.0);
  for (int i = 0; i < n; i++) {
    const T c = s / mu[i];
    T c_b = T(0.0);
    for (int j = 0; j < n; j++) {
      const T xb = Xb.a[i][j] + Um.a[i][j];
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
    const T ib = T(1.0) / L.bs;
    for (int l = 1; l <= nleg; l++) L.p[l] = L.ps[l] * ib;
    L.p[0] = T(0.5);
    const T f = L.p[nleg];
    L.od = (T(1.0) - f * w) * L.od0;
    L.ssa = (T(1.0) - f) * w / (T(1.0) - f * w);
  }
  return 0;
}

// Seed of one species' forward-mode pass: the amount on direction 0, the
// first LUT coordinate on 1 and the second on c2 (-1: not a direction of this
// pass; the temperature's direction is seeded by the caller).
struct SpeciesSeed {
  int sp, c2;
  template <class S>
  CRTM_HD void operator()(int s, S& amount, S& a1, S& a2) const {
    if (s != sp) return;
    amount.d[0] = 1.0;
    a1.d[1] = 1.0;
    if (c2 >= 0) a2.d[c2] = 1.0;
  }
};

// One species' forward-mode pass on N directions (amount, first coordinate,
// and, for N = 3, the second coordinate or the temperature), contracted with
// the species sums' adjoints: gg[d] = od0_b dod/dd + bs_b dbs/dd
// + sum_l ps_b[l] dps_l/dd.
template <int N>
CRTM_HD int species_contract(const CloudyColumn& in, const CloudLut& lut, int nleg, int loff, int k, int sp,
                             double tk, int c2_dir, int t_dir, double od0_b, double bs_b, const double* ps_b,
                             double* gg) {
  using D = Dual<N, double>;
  D od(0.0), bs(0.0), ps[SC_NLEG_MAX + 1];
  D td(tk, 0);
  if (t_dir >= 0) td.d[t_dir] = 1.0;
  if (const int rc = species_share<D>(in, lut, nleg, loff, k, sp, td, SpeciesSeed{sp, c2_dir}, &od, &bs, ps))
    return rc;
  for (int d = 0; d < N; d++) {
    double v = od0_b * od.d[d] + bs_b * bs.d[d];
    for (int l = 1; l <= nleg; l++) v += ps_b[l] * ps[l].d[d];
    gg[d] = v;
  }
  return 0;
}

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
// species' amount and LUT coordinates (gs[sp][0..2]; nsp species).  In FP64
// whatever the adjoint's type: bs_b gathers -p_l pb_l / bs over the Legendre
// terms, which cancel against the ps_b terms in the contraction with the
// species' derivatives (a phase moment moves little while the scattering
// coefficient moves much with the radius), so the bulk values L are FP64 too.
template <class T>
CRTM_HD int bulk_to_inputs(const CloudyColumn& in, const CloudLut& lut, int nleg, int loff, int k, double tk,
                           const LayerBulk<double>& L, const BulkAdjoint<T>& A, int nsp, double* g,
                           double (*gs)[3]) {
  // combine: w = bs / od0, p_l = ps_l / bs, f = p_nleg,
  //   od = (1 - f w) od0, ssa = (1 - f) w / (1 - f w)
  const double od_b = double(A.od_b), ssa_b = double(A.ssa_b);
  double od0_b = od_b, bs_b = 0.0, ps_b[SC_NLEG_MAX + 1];
  for (int l = 0; l <= nleg; l++) ps_b[l] = 0.0;
  if (L.bs > BS_THRESHOLD) {
    const double w = L.bs / L.od0, f = L.p[nleg], D = 1.0 - f * w;
    const double f_b = ssa_b * w * (w - 1.0) / (D * D) - od_b * w * L.od0;
    const double w_b = ssa_b * (1.0 - f) / (D * D) - od_b * f * L.od0;
    od0_b = od_b * D - w_b * w / L.od0;
    bs_b = w_b / L.od0;
    const double ib = 1.0 / L.bs;
    for (int l = 1; l <= nleg; l++) {
      const double pb = l < nleg ? double(A.p_b[l]) : f_b;
      ps_b[l] = pb * ib;
      bs_b -= pb * L.p[l] * ib;
    }
  } else {
    bs_b = ssa_b;
  }
  g[0] = od0_b;
  // Planck radiance of the layer temperature
  const double te = in.b1 + in.b2 * tk, ee = exp(in.c2 / te);
  double gt = (double)A.B_b * in.c1 * in.c2 * ee * in.b2 / (te * te * (ee - 1.0) * (ee - 1.0));
  // each species' share in forward mode on the directions its lookup has:
  // the amount and the first coordinate (radius, or relative humidity for
  // 'GOCART-GEOS5' / 'NAAPS'), and a third only for the liquid microwave
  // tables (temperature) and 'CMAQ' (sigma); in FP64 in every form (the LUT
  // derivatives are differences of nearby table values: in FP32 they cost
  // the radius Jacobians ~1e-3)
  for (int sp = 0; sp < nsp; sp++) {
    const bool cloud = sp < in.n_clouds;
    const int type = cloud ? in.cloud_type[sp] : 0;
    const bool t_dep = cloud && in.microwave && (type == 1 || type == 3);
    const bool c2_dep = !cloud && in.alut && in.alut->scheme == AEROSOL_CMAQ;
    double gg[3] = {0.0, 0.0, 0.0};
    const int rc = (t_dep || c2_dep)
                       ? species_contract<3>(in, lut, nleg, loff, k, sp, tk, c2_dep ? 2 : -1, t_dep ? 2 : -1, od0_b,
                                             bs_b, ps_b, gg)
                       : species_contract<2>(in, lut, nleg, loff, k, sp, tk, -1, -1, od0_b, bs_b, ps_b, gg);
    if (rc) return rc;
    gs[sp][0] = gg[0];
    gs[sp][1] = gg[1];
    gs[sp][2] = c2_dep ? gg[2] : 0.0;
    if (t_dep) gt += gg[2];
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
// (the forward's); a mismatch returns -7.  In FP32, *in_fp64 is set (and
// nothing written) where the layer must be taken in FP64; layer_adjoint
// below then runs the FP64 instance.
template <int NZ, class T>
CRTM_HD int layer_adjoint_in(const CloudyColumn& in, const CloudLut& lut, const StreamSet<NZ, double>& St, int k,
                             double gas_od, int kind_rec, const Mat<NZ, double>& T_b, const Mat<NZ, double>& R_b,
                             const double* src_b, double od_b, double B_b, double* g, double (*gs)[3],
                             bool* in_fp64) {
  constexpr bool fp32 = std::is_same<T, float>::value;
  const int nleg = St.nleg, nS = St.nS, nZ = St.nZ;
  // the layer's bulk optics in FP64 (the combine's adjoint needs them there;
  // the LUT work is small), and in T for the MOM work
  LayerBulk<double> Ld;
  if (const int rc = layer_bulk<double>(in, lut, nleg, St.loff, k, gas_od, in.temperature[k], Ld)) return rc;
  LayerBulk<T> L;
  L.od0 = T(Ld.od0); L.bs = T(Ld.bs); L.od = T(Ld.od); L.ssa = T(Ld.ssa);
  for (int l = 0; l <= nleg; l++) { L.ps[l] = T(Ld.ps[l]); L.p[l] = T(Ld.p[l]); }
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
    // FP32: a nearly conservative layer: the smallest eigenvalue of MOM's
    // (PP - PM)(PP + PM), about 1 - ssa, carries FP32's absolute error, and
    // the single-scattering albedo's adjoint loses eps / (1 - ssa): in FP64
    if (fp32 && 1.0 - Ld.ssa < FP32_COALBEDO_MIN) {
      *in_fp64 = true;
      return 0;
    }
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
    if (!ok) {
      if (!fp32) return -5;
      *in_fp64 = true;   // a failed FP32 factorisation: this layer in FP64
      return 0;
    }
    bool rich = false;
    const double gap_min = fp32 ? FP32_ADJ_GAP_MIN : SENSOR_GAP_MIN;
    if (gap < gap_min && nZ == nS + 1) {
      // A quadrature eigenvalue of MOM nearly meets the sensor angle's: the
      // derivatives through the nearly defective eigenbasis lose about
      // eps / gap^2.  T, R and the source are smooth in the sensor angle, so
      // the layer's bulk adjoints are taken at sensor angles mu (1 +- h) and
      // mu (1 +- 2h), as the Richardson extrapolation (4 D(h) - D(2h)) / 3
      // of the symmetric means (error O(h^4)): h = 1e-3 in FP64, 1e-2 in
      // FP32, where the shifted gaps must be wider.  An FP32 layer whose
      // shifted angles still meet an eigenvalue, or fail, is taken in FP64.
      const double shift = fp32 ? FP32_SENSOR_SHIFT : SENSOR_SHIFT;
      BulkAdjoint<T> S2;
      S2.od_b = S2.ssa_b = S2.B_b = T(0.0);
      for (int l = 0; l <= nleg; l++) S2.p_b[l] = T(0.0);
      int n_ok = 0;
      const int zz = nZ - 1;
#pragma unroll 1
      for (int side = 0; side < 4; side++) {
        const double fsh = (side & 1 ? -1.0 : 1.0) * (side < 2 ? shift : 2.0 * shift);
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
        double gap2 = 1.0;
        if (!ada_layer_adjoint<NZ, T>(nS, nZ, L.ssa, L.od, mu2, wt, ff2, bb2, B, Tb, Rb, sb, &w2, &t2, ffb2, bbb2,
                                      &B2, &gap2))
          break;
        if (fp32 && gap2 < gap_min) break;
        phase_blocks_adjoint<NZ, T>(nS, nZ, nleg, L.p, P2, wt, ffb2, bbb2, pb2);
        S2.od_b += wgt * t2;
        S2.ssa_b += wgt * w2;
        S2.B_b += wgt * B2;
        for (int l = 0; l < nleg; l++) S2.p_b[l] += wgt * pb2[l];
        n_ok++;
      }
      if (n_ok == 4) {
        A = S2;
        rich = true;
      } else if (fp32) {   // a shifted angle failed: FP32 goes to FP64; FP64 keeps the direct derivatives
        *in_fp64 = true;
        return 0;
      }
    }
    if (!rich) {
      A.od_b = tau_b;
      A.ssa_b = w_b;
      A.B_b = Bb;
      phase_blocks_adjoint<NZ, T>(nS, nZ, nleg, L.p, P, wt, ffb, bbb, A.p_b);
    }
  }
  if (const int rc = bulk_to_inputs<T>(in, lut, nleg, St.loff, k, in.temperature[k], Ld, A, nsp, g, gs))
    return rc;
  return kind;
}
template <int NZ, class T>
CRTM_HD int layer_adjoint(const CloudyColumn& in, const CloudLut& lut, const StreamSet<NZ, double>& St, int k,
                          double gas_od, int kind_rec, const Mat<NZ, double>& T_b, const Mat<NZ, double>& R_b,
                          const double* src_b, double od_b, double B_b, double* g, double (*gs)[3]) {
  bool in_fp64 = false;
  const int r = layer_adjoint_in<NZ, T>(in, lut, St, k, gas_od, kind_rec, T_b, R_b, src_b, od_b, B_b, g, gs,
                                        &in_fp64);
  if constexpr (std::is_same<T, float>::value) {
    // one call site of the FP64 instance for every FP32 fallback
    if (in_fp64)
      return layer_adjoint_in<NZ, double>(in, lut, St, k, gas_od, kind_rec, T_b, R_b, src_b, od_b, B_b, g, gs,
                                          &in_fp64);
  }
  return r;
}
}  // namespace crtm
