/*
 * CPU FP64 oracle for the CRTM ODPS + Emission forward / K-matrix / adjoint path.
 *
 * TEST INFRASTRUCTURE ONLY (see crtm_oracle.h): the checker of the GPU
 * library and the timed CPU baseline; never on the product path.
 *
 * Parity unpinned against reference outputs (none can be produced or found
 * here); pinned by known answers, finite differences and TL/AD symmetry.
 *
 * Every routine below is a from-scratch restatement of the reference's
 * behaviour, written in C, citing the Fortran routine it follows.  Arrays are
 * 0-based; where the reference uses 1-based indices the comments say so.
 */
#include "crtm_oracle.h"

#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ---- constants (src/CRTM_Parameters.f90, src/Utility/Fundamental_Constants.f90,
 *      src/Utility/Profile_Utility/Profile_Utility_Parameters.f90) ---------- */
#define OR_PI 3.141592653589793238462643383279
#define DEG2RAD (OR_PI / 180.0)
#define MAX_TRANS_ZENITH_ANGLE 63.6122
#define EARTH_RADIUS 6370.0
#define MAX_OD 20.0 /* ODPS_AtmAbsorption.f90:49 */
#define MAXK 200    /* MAX_N_LAYERS, CRTM_Parameters.f90:64 */
#define MAXJ 8
#define MAXI 18
#define MAXJM 6

static const double G0 = 9.80665, R0 = 8.314472;
static const double MW_H2O = 18.01528, MW_DRYAIR = 28.9648;

static double c_tv(void) { return (1.0 / (MW_H2O / MW_DRYAIR) - 1.0) / 1000.0; }
static double cc_h(void) { return 0.001 * (R0 / (MW_DRYAIR * 1.0e-3)) / G0; }

static const int N_COMPONENTS_G[4] = {0, 8, 5, 2};
static const int N_ABSORBERS_G[4] = {0, 6, 3, 1};

static char g_err[512];
const char* or_last_error(void) { return g_err; }
static void set_err(const char* m) { snprintf(g_err, sizeof g_err, "%s", m); }

struct or_handle_s {
  int group, K, J, Jm, L, sensor_type;
  double ref_lev[MAXK + 1], ref_p[MAXK], ref_t[MAXK];
  double ref_a[MAXJM][MAXK], min_a[MAXJM][MAXK], max_a[MAXJM][MAXK];
  int absorber_id[MAXJM];
  int* n_pred; /* [L][J] */
  int* pos;    /* [L][J], 1-based */
  float* c;
  double *wn, *c1, *c2, *b1, *b2, *cbr, *solar, *freq;
  /* compact-OPTRAN term (oracle_optran.inc); n_oc = 0: none */
  int n_oc, ocomp;
  int* osig, *oorder, *opidx, *opos;
  double* oc;
  double alpha, alpha_c1, alpha_c2;
};

/* ---------------- Fortran sequential record reader ------------------------ */
typedef struct {
  const unsigned char* p;
  size_t n, off;
  int swap;
} recrd;

static uint32_t rd32(const unsigned char* q, int swap) {
  uint32_t v;
  memcpy(&v, q, 4);
  if (swap) v = (v >> 24) | ((v >> 8) & 0xff00u) | ((v << 8) & 0xff0000u) | (v << 24);
  return v;
}

static int next_record(recrd* r, const unsigned char** data, size_t* len) {
  if (r->off + 4 > r->n) return -1;
  uint32_t a = rd32(r->p + r->off, r->swap);
  if (r->off + 8 + a > r->n) return -1;
  uint32_t b = rd32(r->p + r->off + 4 + a, r->swap);
  if (a != b) return -1;
  *data = r->p + r->off + 4;
  *len = a;
  r->off += 8 + a;
  return 0;
}

static void copy_i32(int* dst, const unsigned char* src, size_t n, int swap) {
  for (size_t i = 0; i < n; i++) dst[i] = (int)rd32(src + 4 * i, swap);
}
static void copy_f64(double* dst, const unsigned char* src, size_t n, int swap) {
  for (size_t i = 0; i < n; i++) {
    unsigned char b[8];
    memcpy(b, src + 8 * i, 8);
    if (swap)
      for (int k = 0; k < 4; k++) {
        unsigned char t = b[k];
        b[k] = b[7 - k];
        b[7 - k] = t;
      }
    memcpy(dst + i, b, 8);
  }
}
static void copy_f32(float* dst, const unsigned char* src, size_t n, int swap) {
  for (size_t i = 0; i < n; i++) {
    uint32_t v = rd32(src + 4 * i, swap);
    memcpy(dst + i, &v, 4);
  }
}

static unsigned char* slurp(const char* path, size_t* n) {
  FILE* f = fopen(path, "rb");
  if (!f) return NULL;
  fseek(f, 0, SEEK_END);
  long sz = ftell(f);
  fseek(f, 0, SEEK_SET);
  unsigned char* buf = (unsigned char*)malloc((size_t)sz);
  if (buf && fread(buf, 1, (size_t)sz, f) != (size_t)sz) {
    free(buf);
    buf = NULL;
  }
  fclose(f);
  *n = (size_t)sz;
  return buf;
}

/* Magic-number record decides the byte order (Binary_File_Utility.f90:154-260). */
static int open_records(recrd* r, const unsigned char* buf, size_t n) {
  r->p = buf;
  r->n = n;
  r->off = 0;
  for (int swap = 0; swap < 2; swap++) {
    if (n < 12) return -1;
    if (rd32(buf, swap) == 4 && rd32(buf + 4, swap) == 123456789u) {
      r->swap = swap;
      r->off = 12;
      return 0;
    }
  }
  return -1;
}

/* Read_ODPS_Binary record order (ODPS_Binary_IO.f90:586-900). */
static int load_optran(or_handle* h, recrd* r, int n_oc);

static int load_taucoeff(or_handle* h, const char* path) {
  size_t n;
  unsigned char* buf = slurp(path, &n);
  if (!buf) { set_err("cannot read TauCoeff file"); return -1; }
  recrd r;
  const unsigned char* d;
  size_t len;
  int ok = -1;
  int dims[7];
  if (open_records(&r, buf, n)) { set_err("TauCoeff: bad magic number"); goto done; }
  if (next_record(&r, &d, &len) || len != 8) goto bad;          /* release, version */
  if ((int)rd32(d, r.swap) != 2) { set_err("TauCoeff: unsupported ODPS release"); goto done; }
  if (next_record(&r, &d, &len) || len != 4) goto bad;          /* algorithm */
  if ((int)rd32(d, r.swap) != 2) { set_err("TauCoeff: not an ODPS file"); goto done; }
  if (next_record(&r, &d, &len) || len != 28) goto bad;
  copy_i32(dims, d, 7, r.swap);
  h->K = dims[0]; h->J = dims[1]; h->Jm = dims[2]; h->L = dims[3];
  if (h->K < 1 || h->K > MAXK || h->J > MAXJ || h->Jm > MAXJM || h->L < 1) {
    set_err("TauCoeff: dimensions out of range"); goto done;
  }
  if (next_record(&r, &d, &len) || len != 4) goto bad;
  h->group = (int)rd32(d, r.swap);
  if (h->group < 1 || h->group > 3 || N_COMPONENTS_G[h->group] != h->J ||
      N_ABSORBERS_G[h->group] != h->Jm) { set_err("TauCoeff: bad group"); goto done; }
  if (next_record(&r, &d, &len) || len != 32) goto bad;         /* sensor id + 3 ints */
  h->sensor_type = (int)rd32(d + 28, r.swap);
  if (next_record(&r, &d, &len) || len != 4u * h->L) goto bad;  /* channels */
  if (next_record(&r, &d, &len) || len != 4u * h->J) goto bad;  /* component ids */
  if (next_record(&r, &d, &len) || len != 4u * h->Jm) goto bad; /* absorber ids */
  copy_i32(h->absorber_id, d, h->Jm, r.swap);
  if (next_record(&r, &d, &len) || len != 8u * ((h->K + 1) + 2 * h->K + 3 * h->K * h->Jm)) goto bad;
  {
    size_t o = 0;
    copy_f64(h->ref_lev, d, h->K + 1, r.swap); o += 8 * (h->K + 1);
    copy_f64(h->ref_p, d + o, h->K, r.swap); o += 8 * h->K;
    copy_f64(h->ref_t, d + o, h->K, r.swap); o += 8 * h->K;
    for (int j = 0; j < h->Jm; j++) { copy_f64(h->ref_a[j], d + o, h->K, r.swap); o += 8 * h->K; }
    for (int j = 0; j < h->Jm; j++) { copy_f64(h->min_a[j], d + o, h->K, r.swap); o += 8 * h->K; }
    for (int j = 0; j < h->Jm; j++) { copy_f64(h->max_a[j], d + o, h->K, r.swap); o += 8 * h->K; }
  }
  if (next_record(&r, &d, &len) || len != 8u * h->J * h->L) goto bad;
  h->n_pred = (int*)malloc(sizeof(int) * h->J * h->L);
  h->pos = (int*)malloc(sizeof(int) * h->J * h->L);
  copy_i32(h->n_pred, d, (size_t)h->J * h->L, r.swap);
  copy_i32(h->pos, d + 4u * h->J * h->L, (size_t)h->J * h->L, r.swap);
  h->c = (float*)malloc(sizeof(float) * (dims[4] > 0 ? dims[4] : 1));
  if (dims[4] > 0) {
    if (next_record(&r, &d, &len) || len != 4u * dims[4]) goto bad;
    copy_f32(h->c, d, dims[4], r.swap);
  }
  for (int l = 0; l < h->L; l++)
    for (int j = 0; j < h->J; j++) {
      int np = h->n_pred[l * h->J + j], p0 = h->pos[l * h->J + j];
      if (np > 0 && (p0 < 1 || (long)p0 - 1 + (long)np * h->K > dims[4])) {
        set_err("TauCoeff: Pos_Index out of range"); goto done;
      }
    }
  if (dims[6] > 0 && load_optran(h, &r, dims[6])) goto done;
  ok = 0;
  goto done;
bad:
  set_err("TauCoeff: corrupt or truncated record");
done:
  free(buf);
  return ok;
}

/* SpcCoeff release 8 version 3 record order (SpcCoeff_Binary_IO.f90:660-711). */
static int load_spccoeff(or_handle* h, const char* path) {
  size_t n;
  unsigned char* buf = slurp(path, &n);
  if (!buf) { set_err("cannot read SpcCoeff file"); return -1; }
  recrd r;
  const unsigned char* d;
  size_t len;
  int ok = -1, L;
  if (open_records(&r, buf, n)) { set_err("SpcCoeff: bad magic number"); goto done; }
  if (next_record(&r, &d, &len) || len != 8) goto bad;
  if ((int)rd32(d + 4, r.swap) < 3) { set_err("SpcCoeff: version < 3 not supported"); goto done; }
  if (next_record(&r, &d, &len) || len != 4) goto bad;
  L = (int)rd32(d, r.swap);
  if (L != h->L) { set_err("SpcCoeff and TauCoeff channel counts differ"); goto done; }
  if (next_record(&r, &d, &len) || len != 32) goto bad;
  if (next_record(&r, &d, &len) || len != (size_t)L * (4 + 4 + 8 + 4 + 8 * 8)) goto bad;
  {
    double* tmp = (double*)malloc(sizeof(double) * 8 * L);
    copy_f64(tmp, d + (size_t)L * 20, (size_t)8 * L, r.swap);
    h->wn = (double*)malloc(sizeof(double) * 8 * L);
    h->freq = h->wn + 7 * L; memcpy(h->freq, tmp, sizeof(double) * L);
    memcpy(h->wn, tmp + 1 * L, sizeof(double) * L);
    h->c1 = h->wn + L; memcpy(h->c1, tmp + 2 * L, sizeof(double) * L);
    h->c2 = h->wn + 2 * L; memcpy(h->c2, tmp + 3 * L, sizeof(double) * L);
    h->b1 = h->wn + 3 * L; memcpy(h->b1, tmp + 4 * L, sizeof(double) * L);
    h->b2 = h->wn + 4 * L; memcpy(h->b2, tmp + 5 * L, sizeof(double) * L);
    h->cbr = h->wn + 5 * L; memcpy(h->cbr, tmp + 6 * L, sizeof(double) * L);
    h->solar = h->wn + 6 * L; memcpy(h->solar, tmp + 7 * L, sizeof(double) * L);
    free(tmp);
  }
  ok = 0;
  goto done;
bad:
  set_err("SpcCoeff: corrupt or truncated record");
done:
  free(buf);
  return ok;
}

or_handle* or_init(const char* dir, const char* sensor_id) {
  or_handle* h = (or_handle*)calloc(1, sizeof(or_handle));
  char path[4096];
  snprintf(path, sizeof path, "%s/%s.TauCoeff.bin", dir, sensor_id);
  if (load_taucoeff(h, path)) { or_destroy(h); return NULL; }
  snprintf(path, sizeof path, "%s/%s.SpcCoeff.bin", dir, sensor_id);
  if (load_spccoeff(h, path)) { or_destroy(h); return NULL; }
  return h;
}

void or_destroy(or_handle* h) {
  if (!h) return;
  free(h->n_pred); free(h->pos); free(h->c); free(h->wn);
  free(h);
}
int or_n_channels(const or_handle* h) { return h->L; }
int or_n_ref_layers(const or_handle* h) { return h->K; }
int or_group(const or_handle* h) { return h->group; }

/* ---------------- geometry (CRTM_GeometryInfo.f90:100-143) --------------- */
typedef struct {
  double cos_sensor_zenith, sec_sensor_zenith, trans_zenith_radian, sec_trans_zenith;
  double surface_altitude;
} geom;

static void geometry_compute(double zenith_deg, double altitude, geom* g) {
  double zr = DEG2RAD * zenith_deg;
  g->cos_sensor_zenith = cos(zr);
  g->sec_sensor_zenith = 1.0 / g->cos_sensor_zenith;
  if (zenith_deg > MAX_TRANS_ZENITH_ANGLE) {
    g->trans_zenith_radian = DEG2RAD * MAX_TRANS_ZENITH_ANGLE;
    g->sec_trans_zenith = 1.0 / cos(g->trans_zenith_radian);
  } else {
    g->trans_zenith_radian = zr;
    g->sec_trans_zenith = g->sec_sensor_zenith;
  }
  g->surface_altitude = altitude;
}

/* ---------------- per-profile predictor state ------------------------------ */
typedef struct {
  int Ku, K;
  double user_lev_lnp[MAXK + 1], ref_lev_lnp[MAXK + 1];
  int odps2user[MAXK + 1][2]; /* 1-based into ref levels */
  double T[MAXK], A[MAXJM][MAXK], sec[MAXK], sec_surface;
  /* layer-averaging weights: w[k][i] for user layer wi0[k]+i (0-based) */
  int wi0[MAXK], wn[MAXK];
  double w[MAXK][MAXK];
  int idx_map[MAXJM];
  /* integrated predictor variables (ODPS_Predictor.f90:707-759) */
  double pdp[MAXK], tz_ref[MAXK], tzp_ref[MAXK], tz[MAXK], tzp[MAXK];
  double gazp_ref[MAXJM][MAXK], gatzp_ref[MAXJM][MAXK], gazp[MAXJM][MAXK], gatzp[MAXJM][MAXK];
  double X[MAXK][MAXJ][MAXI];
  /* OPTRAN predictors (index 1-14 as the reference's OX(k, 1:14)), powers of
   * the transformed integrated water vapour, layer water vapour amounts and
   * the integrated sums the adjoint reads */
  double OX[MAXK][15], oAp[MAXK][11], odA[MAXK], oiv[MAXK], oave[MAXK], oinv[MAXK], ost[MAXK], osp[MAXK];
} pstate;

#include "oracle_optran.inc"

/* adjoints of the OPTRAN predictors, accumulated over channels like X_AD */
typedef struct {
  double ox[MAXK][OPT_NX + 1], ap[MAXK][OPT_ORDER + 1], da[MAXK];
} optran_adj;

/* LayerAvg (ODPS_CoordinateMapping.f90:1108-1320): weights of the user layers
 * (ln p at px2, n2 of them) for each reference layer (ln p at px1, n1). */
static void layer_avg(const double* px1, int kn1, const double* px2, int kn2, pstate* s) {
  int istart = 0; /* 0-based */
  static const double SMALLDIFF = 1.0e-20;
  double* pz = (double*)malloc(sizeof(double) * kn2);
  for (int ki = 0; ki < kn1; ki++) {
    double z2 = px1[ki], z1, z3;
    z1 = (ki == 0) ? 2.0 * z2 - px1[ki + 1] : px1[ki - 1];
    z3 = (ki == kn1 - 1) ? 2.0 * z2 - z1 : px1[ki + 1];
    if (z3 > px2[kn2 - 1]) z3 = px2[kn2 - 1];
    int iskip = 0;
    if (z2 >= px2[kn2 - 1]) { z3 = px2[kn2 - 1]; z2 = px2[kn2 - 1]; iskip = 1; }
    for (int j = 0; j < kn2; j++) pz[j] = 0.0;
    int ic = 0, jend = kn2 - 1, j;
    for (j = istart; j < kn2 - 1; j++) {
      if (px2[j] > z3) { jend = j; goto tail; }
      if (px2[j] <= z2 && px2[j + 1] > z1) {
        int itop = 0, ibot = 0;
        double y1, y2;
        if (z1 < z3) {
          y1 = z1; if (px2[j] > z1) { y1 = px2[j]; itop = 1; }
          y2 = z2; if (px2[j + 1] < z2) { y2 = px2[j + 1]; ibot = 1; }
        } else {
          y1 = z2; if (px2[j] > z2) { y1 = px2[j]; itop = 1; }
          y2 = z1; if (px2[j + 1] < z1) { y2 = px2[j + 1]; ibot = 1; }
        }
        double dy = y2 - y1, dz = z1 - z2;
        if (fabs(dz) < SMALLDIFF) goto abort_profile;
        double dzd = 1.0 / dz;
        double zw1 = (z1 - y1) * dzd * dy, zw2 = (z1 - y2) * dzd * dy;
        double dx = px2[j + 1] - px2[j];
        if (fabs(dx) < SMALLDIFF) goto abort_profile;
        double d = (px2[j + 1] - z2) * (1.0 / dx);
        if (z1 < z3 && ibot == 0) { zw1 = zw1 + zw2 * d; zw2 = zw2 * (1.0 - d); }
        else if (z1 > z3 && itop == 0) { zw2 = zw2 + zw1 * (1.0 - d); zw1 = zw1 * d; }
        pz[j] += zw1; pz[j + 1] += zw2; ic = 1;
      }
      if (px2[j] < z3 && px2[j + 1] >= z2 && iskip == 0) {
        int itop = 0, ibot = 0;
        double y1, y2;
        if (z3 < z1) {
          y1 = z3; if (px2[j] > z3) { y1 = px2[j]; itop = 1; }
          y2 = z2; if (px2[j + 1] < z2) { y2 = px2[j + 1]; ibot = 1; }
        } else {
          y1 = z2; if (px2[j] > z2) { y1 = px2[j]; itop = 1; }
          y2 = z3; if (px2[j + 1] < z3) { y2 = px2[j + 1]; ibot = 1; }
        }
        double dy = y2 - y1, dz = z3 - z2;
        if (fabs(dz) < SMALLDIFF) goto abort_profile;
        double dzd = 1.0 / dz;
        double zw1 = (z3 - y1) * dzd * dy, zw2 = (z3 - y2) * dzd * dy;
        double dx = px2[j + 1] - px2[j];
        if (fabs(dx) < SMALLDIFF) goto abort_profile;
        double d = (px2[j + 1] - z2) * (1.0 / dx);
        if (z3 < z1 && ibot == 0) { zw1 = zw1 + zw2 * d; zw2 = zw2 * (1.0 - d); }
        else if (z3 > z1 && itop == 0) { zw2 = zw2 + zw1 * (1.0 - d); zw1 = zw1 * d; }
        pz[j] += zw1; pz[j + 1] += zw2; ic = 1;
      }
    }
    jend = kn2 - 1;
  tail:
    if (ic == 0) pz[jend] = 1.0;
    {
      int i1 = -1;
      for (int ii = istart; ii < kn2; ii++)
        if (pz[ii] != 0.0) { i1 = ii; break; }
      if (i1 < 0) i1 = istart; /* unreachable for monotone grids */
      istart = i1;
      int i2 = kn2 - 1;
      for (int ii = i1 + 1; ii < kn2; ii++)
        if (pz[ii] == 0.0) { i2 = ii - 1; break; }
      double zsum = 0.0;
      for (int ii = i1; ii <= i2; ii++) zsum += pz[ii];
      s->wi0[ki] = i1;
      s->wn[ki] = i2 - i1 + 1;
      for (int ii = i1; ii <= i2; ii++) s->w[ki][ii - i1] = pz[ii] / zsum;
    }
    continue;
  abort_profile:
    /* the reference prints an error and returns, leaving later weights unset */
    s->wi0[ki] = 0; s->wn[ki] = 0;
  }
  free(pz);
}

/* Compute_Interp_Index (ODPS_CoordinateMapping.f90:963-1012); idx 1-based into x. */
static void compute_interp_index(const double* x, int nx, const double* u, int nu, int (*idx)[2]) {
  int k1 = nu + 1, k2 = 0;
  for (int iu = 1; iu <= nu; iu++) {
    if (u[iu - 1] < x[0]) { idx[iu - 1][0] = 1; idx[iu - 1][1] = 1; }
    else { k1 = iu; break; }
  }
  for (int iu = nu; iu >= k1; iu--) {
    if (u[iu - 1] > x[nx - 1]) { idx[iu - 1][0] = nx; idx[iu - 1][1] = nx; }
    else { k2 = iu; break; }
  }
  int j = 1;
  for (int iu = k1; iu <= k2; iu++) {
    for (int ix = j; ix <= nx - 1; ix++) {
      if (u[iu - 1] >= x[ix - 1] && u[iu - 1] <= x[ix]) {
        idx[iu - 1][0] = ix; idx[iu - 1][1] = ix + 1; j = ix;
        break;
      }
    }
  }
}

/* Map_Input (ODPS_CoordinateMapping.f90:151-319). */
static void map_input(const or_handle* h, const or_batch* b, int m, const geom* g, pstate* s) {
  const int K = h->K, Ku = b->n_layers[m], Kmax = b->max_layers;
  const double* lev = b->level_pressure + (size_t)m * (Kmax + 1);
  const double* lay = b->pressure + (size_t)m * Kmax;
  const double* tu = b->temperature + (size_t)m * Kmax;
  const double tol = 2.220446049250313e-16; /* EPSILON(1.0_fp) */
  double ref_lnp[MAXK], user_lnp[MAXK];
  s->K = K;
  s->Ku = Ku;
  for (int k = 0; k < K; k++) ref_lnp[k] = log(h->ref_p[k]);
  for (int k = 0; k < Ku; k++) user_lnp[k] = log(lay[k]);
  for (int k = 0; k <= K; k++) s->ref_lev_lnp[k] = log(h->ref_lev[k]);
  s->user_lev_lnp[0] = (lev[0] <= 0.0) ? log(lev[1] / 2.0) : log(lev[0]);
  for (int k = 1; k <= Ku; k++) s->user_lev_lnp[k] = log(lev[k]);
  int sfc_idx = K;
  double sfc_frac = 0.0;
  if (h->ref_lev[K] > lev[Ku]) {
    for (int k = K; k >= 0; k--) {
      if (h->ref_lev[k] < lev[Ku]) {
        sfc_idx = k + 1;
        sfc_frac = (s->ref_lev_lnp[sfc_idx] - s->user_lev_lnp[Ku]) /
                   (s->ref_lev_lnp[sfc_idx] - s->ref_lev_lnp[k]);
        break;
      }
    }
  }
  layer_avg(ref_lnp, K, user_lnp, Ku, s);
  for (int k = 0; k < K; k++) {
    double acc = 0.0;
    for (int i = 0; i < s->wn[k]; i++) acc += s->w[k][i] * tu[s->wi0[k] + i];
    s->T[k] = acc;
  }
  for (int j = 0; j < h->Jm; j++) {
    int map = -1;
    for (int jj = 0; jj < b->n_absorbers; jj++)
      if (b->absorber_id[jj] == h->absorber_id[j]) { map = jj; break; }
    s->idx_map[j] = map;
    if (map >= 0) {
      const double* au = b->absorber + ((size_t)m * b->n_absorbers + map) * Kmax;
      for (int k = 0; k < K; k++) {
        double acc = 0.0;
        for (int i = 0; i < s->wn[k]; i++) acc += s->w[k][i] * au[s->wi0[k] + i];
        if (acc <= tol) acc = tol;
        if (acc < h->min_a[j][k]) acc = h->min_a[j][k];
        if (acc > h->max_a[j][k]) acc = h->max_a[j][k];
        s->A[j][k] = acc;
      }
    } else {
      for (int k = 0; k < K; k++) s->A[j][k] = h->ref_a[j][k];
    }
  }
  /* H2O_idx: reset to 1 inside the absorber loop, so it ends as 1 unless the
   * last absorber is water vapour (ODPS_CoordinateMapping.f90:251-256). */
  int h2o = (h->absorber_id[h->Jm - 1] == 1) ? h->Jm - 1 : 0;
  /* Geopotential_Height (ODPS_CoordinateMapping.f90:607-634) on the reference profile */
  double z[MAXK + 1];
  z[K] = 0.0;
  for (int k = K; k >= 1; k--) {
    double tv = h->ref_t[k - 1] * (1.0 + c_tv() * h->ref_a[h2o][k - 1]);
    z[k - 1] = z[k] + cc_h() * tv * log(h->ref_lev[k] / h->ref_lev[k - 1]);
  }
  double zoff;
  if (h->ref_lev[K] >= lev[Ku])
    zoff = -(z[sfc_idx] + sfc_frac * (z[sfc_idx - 1] - z[sfc_idx])) + g->surface_altitude;
  else
    zoff = cc_h() * h->ref_t[K - 1] * log(1013.0 / h->ref_lev[K]);
  double sv = (EARTH_RADIUS + g->surface_altitude) * sin(g->trans_zenith_radian);
  for (int k = 1; k <= K; k++) {
    double sa = sv / (EARTH_RADIUS + (z[k] + zoff));
    s->sec[k - 1] = 1.0 / sqrt(1.0 - sa * sa);
  }
  s->sec_surface = g->sec_trans_zenith;
  compute_interp_index(s->ref_lev_lnp, K + 1, s->user_lev_lnp, Ku + 1, s->odps2user);
}

/* ODPS_Compute_Predictor (ODPS_Predictor.f90:645-1095), groups 1-3. */
static void compute_predictors(const or_handle* h, pstate* s) {
  const int K = h->K, Jm = h->Jm, G = h->group;
  double tz_r = 0, tz_s = 0, tzp_r = 0, tzp_s = 0;
  double gazp_r[MAXJM] = {0}, gazp_s[MAXJM] = {0}, gatzp_r[MAXJM] = {0}, gatzp_s[MAXJM] = {0};
  memset(s->X, 0, sizeof s->X);
  for (int k = 0; k < K; k++) {
    double pdp = (k == 0) ? h->ref_lev[0] * (h->ref_lev[1] - h->ref_lev[0])
                          : h->ref_lev[k + 1] * (h->ref_lev[k + 1] - h->ref_lev[k]);
    /* note: the reference's level index k (1-based layer k) is ref_lev[k] here for k>=1 */
    s->pdp[k] = pdp;
    tz_r += h->ref_t[k]; tz_s += s->T[k];
    s->tz_ref[k] = tz_r; s->tz[k] = tz_s / tz_r;
    tzp_r += pdp * h->ref_t[k]; tzp_s += pdp * s->T[k];
    s->tzp_ref[k] = tzp_r; s->tzp[k] = tzp_s / tzp_r;
    for (int j = 0; j < Jm; j++) {
      gazp_r[j] += pdp * h->ref_a[j][k]; gazp_s[j] += pdp * s->A[j][k];
      s->gazp_ref[j][k] = gazp_r[j]; s->gazp[j][k] = gazp_s[j] / gazp_r[j];
      gatzp_r[j] += pdp * h->ref_a[j][k] * h->ref_t[k];
      gatzp_s[j] += pdp * s->A[j][k] * s->T[k];
      s->gatzp_ref[j][k] = gatzp_r[j]; s->gatzp[j][k] = gatzp_s[j] / gatzp_r[j];
    }
  }
  for (int k = 0; k < K; k++) {
    double (*X)[MAXI] = s->X[k];
    const double sec = s->sec[k];
    const double dT = s->T[k] - h->ref_t[k], t = s->T[k] / h->ref_t[k];
    const double t2 = t * t, dT2 = dT * fabs(dT);
    const double h2o = s->A[0][k] / h->ref_a[0][k];
    const double h2o_a = sec * h2o, h2o_r = sqrt(h2o_a), h2o_s = h2o_a * h2o_a;
    const double h2o_r4 = sqrt(h2o_r), hd = h2o / s->gatzp[0][k];
    X[0][0] = sec; X[0][1] = sec * t; X[0][2] = sec * t2; X[0][3] = t;
    X[0][4] = sec * sec; X[0][5] = t2; X[0][6] = s->tz[k];
    if (G == 3) {
      const double g = s->gazp[0][k];
      double* w = X[1];
      w[0] = h2o_a / t; w[1] = h2o_a / t * h2o; w[2] = h2o_a / t2 * h2o / t2; w[3] = h2o_a / t2;
      w[4] = h2o_a / t2 * h2o; w[5] = h2o_a / (t2 * t2); w[6] = h2o_a; w[7] = h2o_a * dT;
      w[8] = (sec * g) * (sec * g); w[9] = sec * g; w[10] = sec; w[11] = h2o_s * h2o_a;
      w[12] = h2o_s * h2o_s; w[13] = hd;
      continue;
    }
    const double o3 = s->A[1][k] / h->ref_a[1][k], co2 = s->A[2][k] / h->ref_a[2][k];
    const double o3_a = sec * o3, o3_r = sqrt(o3_a), go3 = s->gazp[1][k];
    double* wco = X[2];
    wco[0] = h2o_a / t; wco[1] = h2o_a / t * h2o; wco[2] = h2o_a / t2 * h2o / t2;
    wco[3] = h2o_a / t2; wco[4] = h2o_a / t2 * h2o; wco[5] = h2o_a / (t2 * t2); wco[6] = h2o_a;
    double* oz = X[3];
    oz[0] = o3_a; oz[1] = o3_a * dT; oz[2] = o3_a * o3 * go3; oz[3] = o3_a * o3_a;
    oz[4] = o3_a * go3; oz[5] = o3_a * sqrt(sec * go3); oz[6] = o3_r * dT; oz[7] = o3_r;
    oz[8] = o3_r * o3 / go3; oz[9] = sec * go3; oz[10] = (sec * go3) * (sec * go3);
    double* c2 = X[4];
    const double tzp = s->tzp[k], gco2 = s->gazp[2][k];
    c2[0] = sec * t; c2[1] = sec * t2; c2[2] = t; c2[3] = t2; c2[4] = sec; c2[5] = sec * co2;
    c2[6] = sec * tzp; c2[7] = (sec * gco2) * (sec * gco2); c2[8] = tzp * tzp * tzp;
    c2[9] = sec * tzp * sqrt(t);
    double* wl = X[1];
    const double gh = s->gazp[0][k];
    wl[0] = h2o_a; wl[1] = h2o_a * dT; wl[2] = h2o_s; wl[3] = h2o_a * dT2; wl[4] = h2o_r4;
    wl[5] = h2o_s * h2o_a; wl[6] = h2o_r; wl[7] = h2o_r * dT; wl[8] = h2o_s * h2o_s; wl[9] = hd;
    wl[10] = h2o_r * hd; wl[11] = (sec * gh) * (sec * gh); wl[12] = sec * gh; wl[13] = sec;
    wl[14] = sec * co2;
    if (G == 1) {
      const double co = s->A[4][k] / h->ref_a[4][k], n2o = s->A[3][k] / h->ref_a[3][k];
      const double ch4 = s->A[5][k] / h->ref_a[5][k];
      const double n2o_a = sec * n2o, n2o_r = sqrt(n2o_a), n2o_s = n2o_a * n2o_a;
      const double co_a = sec * co, co_r = sqrt(co_a), co_s = co_a * co_a;
      const double gco = s->gazp[4][k], gch4 = s->gazp[5][k], gn2o = s->gazp[3][k];
      const double coc = co_a * co / gco;
      const double ch4_a = sec * ch4, ch4_r = sqrt(ch4_a), ch4z = sec * gch4;
      c2[10] = co_a;
      wl[15] = ch4_a; wl[16] = ch4_a * ch4_a * dT; wl[17] = co_a;
      double* cp = X[6];
      cp[0] = co_a; cp[1] = co_a * dT; cp[2] = sqrt(co_r); cp[3] = co_r * dT; cp[4] = co_s;
      cp[5] = co_r; cp[6] = co_a * dT2; cp[7] = coc; cp[8] = coc / co_r; cp[9] = coc * sqrt(gco);
      double* mp = X[7];
      mp[0] = ch4_a * dT; mp[1] = ch4_r; mp[2] = ch4_a * ch4_a; mp[3] = ch4_a; mp[4] = ch4 * dT;
      mp[5] = ch4z; mp[6] = ch4z * ch4z; mp[7] = sqrt(ch4_r); mp[8] = s->gatzp[5][k];
      mp[9] = sec * s->gatzp[5][k]; mp[10] = ch4_r * ch4 / gch4;
      double* np_ = X[5];
      np_[0] = n2o_a * dT; np_[1] = n2o_r; np_[2] = n2o * dT; np_[3] = pow(n2o_a, 0.25);
      np_[4] = n2o_a; np_[5] = sec * gn2o; np_[6] = sec * s->gatzp[3][k]; np_[7] = n2o_s;
      np_[8] = s->gatzp[3][k]; np_[9] = n2o_r * n2o / gn2o; np_[10] = ch4_a;
      np_[11] = ch4_a * gch4; np_[12] = co_a; np_[13] = co_a * sec * gco;
    }
  }
  if (h->n_oc > 0) optran_predictors(h, s);   /* ODPS_Predictor.f90:336-347 */
}

/* Adjoint of compute_predictors: X_AD -> T_AD, A_AD on reference layers.
 * Exact reverse of the forward above; the reference's ODPS_Compute_Predictor_AD
 * (ODPS_Predictor.f90:1783-2643) is likewise the exact adjoint. */
static void compute_predictors_ad(const or_handle* h, const pstate* s, double (*XA)[MAXJ][MAXI],
                                  double* T_ad, double (*A_ad)[MAXK], optran_adj* oa) {
  const int K = h->K, Jm = h->Jm, G = h->group;
  double tz_ad[MAXK], tzp_ad[MAXK], gazp_ad[MAXJM][MAXK], gatzp_ad[MAXJM][MAXK];
  memset(tz_ad, 0, sizeof tz_ad); memset(tzp_ad, 0, sizeof tzp_ad);
  memset(gazp_ad, 0, sizeof gazp_ad); memset(gatzp_ad, 0, sizeof gatzp_ad);
  for (int k = K - 1; k >= 0; k--) {
    double (*x)[MAXI] = XA[k];
    const double sec = s->sec[k];
    const double dT = s->T[k] - h->ref_t[k], t = s->T[k] / h->ref_t[k];
    const double t2 = t * t;
    const double h2o = s->A[0][k] / h->ref_a[0][k];
    const double h2o_a = sec * h2o, h2o_r = sqrt(h2o_a), h2o_s = h2o_a * h2o_a;
    const double G0h = s->gatzp[0][k], hd = h2o / G0h;
    double t_ad = 0, t2_ad = 0, dT_ad = 0, dT2_ad = 0;
    double h2o_ad = 0, h2o_a_ad = 0, h2o_r_ad = 0, h2o_s_ad = 0, h2o_r4_ad = 0, hd_ad = 0;
    double ratio_ad[MAXJM] = {0};
    /* dry */
    t_ad += x[0][1] * sec + x[0][3];
    t2_ad += x[0][2] * sec + x[0][5];
    tz_ad[k] += x[0][6];
    if (G == 3) {
      const double* w = x[1];
      const double g = s->gazp[0][k];
      h2o_a_ad += w[0] / t + w[1] * h2o / t + w[2] * h2o / (t2 * t2) + w[3] / t2 +
                  w[4] * h2o / t2 + w[5] / (t2 * t2) + w[6] + w[7] * dT + w[11] * h2o_s;
      t_ad -= w[0] * h2o_a / (t * t) + w[1] * h2o_a * h2o / (t * t);
      h2o_ad += w[1] * h2o_a / t + w[2] * h2o_a / (t2 * t2) + w[4] * h2o_a / t2;
      t2_ad -= w[2] * 2.0 * h2o_a * h2o / (t2 * t2 * t2) + w[3] * h2o_a / (t2 * t2) +
               w[4] * h2o_a * h2o / (t2 * t2) + w[5] * 2.0 * h2o_a / (t2 * t2 * t2);
      dT_ad += w[7] * h2o_a;
      gazp_ad[0][k] += w[8] * 2.0 * sec * sec * g + w[9] * sec;
      h2o_s_ad += w[11] * h2o_a + w[12] * 2.0 * h2o_s;
      hd_ad += w[13];
    } else {
      const double o3 = s->A[1][k] / h->ref_a[1][k];
      const double o3_a = sec * o3, o3_r = sqrt(o3_a), go3 = s->gazp[1][k];
      double o3_ad = 0, o3_a_ad = 0, o3_r_ad = 0, co2_ad = 0;
      double co_a_ad = 0, ch4_a_ad = 0;
      const double* wc = x[2];
      h2o_a_ad += wc[0] / t + wc[1] * h2o / t + wc[2] * h2o / (t2 * t2) + wc[3] / t2 +
                  wc[4] * h2o / t2 + wc[5] / (t2 * t2) + wc[6];
      t_ad -= wc[0] * h2o_a / (t * t) + wc[1] * h2o_a * h2o / (t * t);
      h2o_ad += wc[1] * h2o_a / t + wc[2] * h2o_a / (t2 * t2) + wc[4] * h2o_a / t2;
      t2_ad -= wc[2] * 2.0 * h2o_a * h2o / (t2 * t2 * t2) + wc[3] * h2o_a / (t2 * t2) +
               wc[4] * h2o_a * h2o / (t2 * t2) + wc[5] * 2.0 * h2o_a / (t2 * t2 * t2);
      const double* oz = x[3];
      o3_a_ad += oz[0] + oz[1] * dT + oz[2] * o3 * go3 + oz[3] * 2.0 * o3_a + oz[4] * go3 +
                 oz[5] * sqrt(sec * go3);
      dT_ad += oz[1] * o3_a + oz[6] * o3_r;
      o3_ad += oz[2] * o3_a * go3 + oz[8] * o3_r / go3;
      gazp_ad[1][k] += oz[2] * o3_a * o3 + oz[4] * o3_a + oz[5] * 0.5 * o3_a * sqrt(sec / go3) -
                       oz[8] * o3_r * o3 / (go3 * go3) + oz[9] * sec + oz[10] * 2.0 * sec * sec * go3;
      o3_r_ad += oz[6] * dT + oz[7] + oz[8] * o3 / go3;
      const double* c2 = x[4];
      const double tzp = s->tzp[k];
      t_ad += c2[0] * sec + c2[2] + c2[9] * sec * (0.5 * tzp / sqrt(t));
      t2_ad += c2[1] * sec + c2[3];
      co2_ad += c2[5] * sec;
      tzp_ad[k] += c2[6] * sec + c2[8] * 3.0 * tzp * tzp + c2[9] * sec * sqrt(t);
      gazp_ad[2][k] += c2[7] * 2.0 * sec * sec * s->gazp[2][k];
      const double* wl = x[1];
      h2o_a_ad += wl[0] + wl[1] * dT + wl[3] * (dT * fabs(dT)) + wl[5] * h2o_s;
      dT_ad += wl[1] * h2o_a + wl[7] * h2o_r;
      h2o_s_ad += wl[2] + wl[5] * h2o_a + wl[8] * 2.0 * h2o_s;
      dT2_ad += wl[3] * h2o_a;
      h2o_r4_ad += wl[4];
      h2o_r_ad += wl[6] + wl[7] * dT + wl[10] * hd;
      hd_ad += wl[9] + wl[10] * h2o_r;
      gazp_ad[0][k] += wl[11] * 2.0 * sec * sec * s->gazp[0][k] + wl[12] * sec;
      co2_ad += wl[14] * sec;
      if (G == 1) {
        const double co = s->A[4][k] / h->ref_a[4][k], n2o = s->A[3][k] / h->ref_a[3][k];
        const double ch4 = s->A[5][k] / h->ref_a[5][k];
        const double n2o_a = sec * n2o, n2o_r = sqrt(n2o_a);
        const double co_a = sec * co, co_r = sqrt(co_a);
        const double gco = s->gazp[4][k], gch4 = s->gazp[5][k], gn2o = s->gazp[3][k];
        const double coc = co_a * co / gco;
        const double ch4_a = sec * ch4, ch4_r = sqrt(ch4_a), ch4z = sec * gch4;
        double co_ad = 0, co_r_ad = 0, co_s_ad = 0, coc_ad = 0;
        double ch4_ad = 0, ch4_r_ad = 0, ch4z_ad = 0;
        double n2o_ad = 0, n2o_a_ad = 0, n2o_r_ad = 0, n2o_s_ad = 0;
        co_a_ad += wl[17] + c2[10];
        ch4_a_ad += wl[15] + wl[16] * 2.0 * ch4_a * dT;
        dT_ad += wl[16] * ch4_a * ch4_a;
        const double* cp = x[6];
        co_a_ad += cp[0] + cp[1] * dT + cp[6] * (dT * fabs(dT));
        dT_ad += cp[1] * co_a + cp[3] * co_r;
        co_r_ad += cp[2] * 0.5 / sqrt(co_r) + cp[3] * dT + cp[5] - cp[8] * coc / (co_r * co_r);
        co_s_ad += cp[4];
        dT2_ad += cp[6] * co_a;
        coc_ad += cp[7] + cp[8] / co_r + cp[9] * sqrt(gco);
        gazp_ad[4][k] += cp[9] * 0.5 * coc / sqrt(gco);
        const double* mp = x[7];
        ch4_a_ad += mp[0] * dT + mp[2] * 2.0 * ch4_a + mp[3];
        dT_ad += mp[0] * ch4_a + mp[4] * ch4;
        ch4_r_ad += mp[1] + mp[7] * 0.5 / sqrt(ch4_r) + mp[10] * ch4 / gch4;
        ch4_ad += mp[4] * dT + mp[10] * ch4_r / gch4;
        ch4z_ad += mp[5] + mp[6] * 2.0 * ch4z;
        gatzp_ad[5][k] += mp[8] + mp[9] * sec;
        gazp_ad[5][k] -= mp[10] * ch4_r * ch4 / (gch4 * gch4);
        const double* np_ = x[5];
        n2o_a_ad += np_[0] * dT + np_[3] * 0.25 * pow(n2o_a, -0.75) + np_[4];
        dT_ad += np_[0] * n2o_a + np_[2] * n2o;
        n2o_r_ad += np_[1] + np_[9] * n2o / gn2o;
        n2o_ad += np_[2] * dT + np_[9] * n2o_r / gn2o;
        gazp_ad[3][k] += np_[5] * sec - np_[9] * n2o_r * n2o / (gn2o * gn2o);
        gatzp_ad[3][k] += np_[6] * sec + np_[8];
        n2o_s_ad += np_[7];
        ch4_a_ad += np_[10] + np_[11] * gch4;
        gazp_ad[5][k] += np_[11] * ch4_a;
        co_a_ad += np_[12] + np_[13] * sec * gco;
        gazp_ad[4][k] += np_[13] * co_a * sec;
        /* intermediates */
        gazp_ad[5][k] += sec * ch4z_ad;
        ch4_a_ad += (0.5 / sqrt(ch4_a)) * ch4_r_ad;
        ch4_ad += sec * ch4_a_ad;
        gazp_ad[4][k] -= coc_ad * co_a * co / (gco * gco);
        co_a_ad += coc_ad * co / gco + co_s_ad * 2.0 * co_a + co_r_ad * 0.5 / sqrt(co_a);
        co_ad += coc_ad * co_a / gco + co_a_ad * sec;
        n2o_a_ad += n2o_r_ad * 0.5 / sqrt(n2o_a) + n2o_s_ad * 2.0 * n2o_a;
        n2o_ad += n2o_a_ad * sec;
        ratio_ad[5] += ch4_ad;
        ratio_ad[3] += n2o_ad;
        ratio_ad[4] += co_ad;
      }
      o3_a_ad += o3_r_ad * 0.5 / sqrt(o3_a);
      o3_ad += o3_a_ad * sec;
      ratio_ad[1] += o3_ad;
      ratio_ad[2] += co2_ad;
    }
    gatzp_ad[0][k] -= hd_ad * h2o / (G0h * G0h);
    h2o_r_ad += h2o_r4_ad * 0.5 / sqrt(h2o_r);
    h2o_a_ad += h2o_s_ad * 2.0 * h2o_a + h2o_r_ad * 0.5 / sqrt(h2o_a);
    h2o_ad += h2o_a_ad * sec + hd_ad / G0h;
    ratio_ad[0] += h2o_ad;
    dT_ad += dT2_ad * 2.0 * fabs(dT);
    t_ad += t2_ad * 2.0 * t;
    for (int j = 0; j < Jm; j++) A_ad[j][k] += ratio_ad[j] / h->ref_a[j][k];
    T_ad[k] += t_ad / h->ref_t[k] + dT_ad;
  }
  /* reverse of the running integrals */
  double tz_sum = 0, tzp_sum = 0, gazp_sum[MAXJM] = {0}, gatzp_sum[MAXJM] = {0};
  for (int k = K - 1; k >= 0; k--) {
    for (int j = Jm - 1; j >= 0; j--) {
      gatzp_sum[j] += gatzp_ad[j][k] / s->gatzp_ref[j][k];
      gazp_sum[j] += gazp_ad[j][k] / s->gazp_ref[j][k];
      T_ad[k] += gatzp_sum[j] * s->pdp[k] * s->A[j][k];
      A_ad[j][k] += gazp_sum[j] * s->pdp[k] + gatzp_sum[j] * s->pdp[k] * s->T[k];
    }
    tzp_sum += tzp_ad[k] / s->tzp_ref[k];
    tz_sum += tz_ad[k] / s->tz_ref[k];
    T_ad[k] += tz_sum + s->pdp[k] * tzp_sum;
  }
  if (h->n_oc > 0) optran_predictors_ad(h, s, oa->ox, oa->ap, oa->da, T_ad, A_ad[0]);
}

/* ODPS_Compute_AtmAbsorption (ODPS_AtmAbsorption.f90:133-256): user-layer
 * optical depth of channel l; od_ref returns the unclamped reference-layer OD. */
static void atm_absorption(const or_handle* h, const pstate* s, int l, double* od_ref,
                           double* layer_od) {
  const int K = h->K;
  for (int k = 0; k < K; k++) od_ref[k] = 0.0;
  for (int j = 0; j < h->J; j++) {
    int np = h->n_pred[l * h->J + j];
    if (np <= 0) continue;
    if (j == h->ocomp - 1 && optran_channel(h, l)) {   /* ODPS_AtmAbsorption.f90:184-195 */
      optran_od(h, s, l, od_ref);
      continue;
    }
    int j0 = h->pos[l * h->J + j] - 1;
    for (int i = 0; i < np; i++) {
      const float* c = h->c + j0 + (size_t)i * K;
      for (int k = 0; k < K; k++) od_ref[k] += (double)c[k] * s->X[k][j][i];
    }
  }
  double path[MAXK + 1];
  path[0] = 0.0;
  for (int k = 0; k < K; k++) {
    double v = od_ref[k];
    if (v < 0.0) v = 0.0;
    else if (v > MAX_OD) v = MAX_OD;
    path[k + 1] = path[k] + v;
  }
  double up[MAXK + 1];
  for (int i = 0; i <= s->Ku; i++) {
    int k1 = s->odps2user[i][0], k2 = s->odps2user[i][1];
    if (k1 == k2) up[i] = path[k1 - 1];
    else {
      double x1 = s->ref_lev_lnp[k1 - 1], x2 = s->ref_lev_lnp[k2 - 1];
      up[i] = path[k1 - 1] + (path[k2 - 1] - path[k1 - 1]) * (s->user_lev_lnp[i] - x1) / (x2 - x1);
    }
  }
  for (int k = 0; k < s->Ku; k++) layer_od[k] = (up[k + 1] - up[k]) / s->sec_surface;
}

/* ODPS_Compute_AtmAbsorption_AD (ODPS_AtmAbsorption.f90:487-600): adds C*OD_AD to X_AD. */
static void atm_absorption_ad(const or_handle* h, const pstate* s, int l, const double* od_ref,
                              const double* layer_od_ad, double (*XA)[MAXJ][MAXI], optran_adj* oa) {
  const int K = h->K, Ku = s->Ku;
  double up_ad[MAXK + 1], path_ad[MAXK + 1], od_ad[MAXK];
  up_ad[Ku] = 0.0;
  for (int k = Ku; k >= 1; k--) {
    up_ad[k] += layer_od_ad[k - 1] / s->sec_surface;
    up_ad[k - 1] = -layer_od_ad[k - 1] / s->sec_surface;
  }
  for (int k = 0; k <= K; k++) path_ad[k] = 0.0;
  for (int i = Ku; i >= 0; i--) {
    int k1 = s->odps2user[i][0], k2 = s->odps2user[i][1];
    if (k1 == k2) path_ad[k1 - 1] += up_ad[i];
    else {
      double x1 = s->ref_lev_lnp[k1 - 1], x2 = s->ref_lev_lnp[k2 - 1];
      double fac = (s->user_lev_lnp[i] - x1) / (x2 - x1);
      path_ad[k1 - 1] += (1.0 - fac) * up_ad[i];
      path_ad[k2 - 1] += fac * up_ad[i];
    }
  }
  for (int k = K; k >= 1; k--) {
    path_ad[k - 1] += path_ad[k];
    od_ad[k - 1] = path_ad[k];
    path_ad[k] = 0.0;
    if (od_ref[k - 1] < 0.0 || od_ref[k - 1] > MAX_OD) od_ad[k - 1] = 0.0;
  }
  for (int j = 0; j < h->J; j++) {
    int np = h->n_pred[l * h->J + j];
    if (np <= 0) continue;
    if (j == h->ocomp - 1 && optran_channel(h, l)) {   /* ODPS_AtmAbsorption.f90:573-580 */
      optran_od_ad(h, s, l, od_ad, oa->ox, oa->ap, oa->da);
      continue;
    }
    int j0 = h->pos[l * h->J + j] - 1;
    for (int i = 0; i < np; i++) {
      const float* c = h->c + j0 + (size_t)i * K;
      for (int k = K - 1; k >= 0; k--) XA[k][j][i] += (double)c[k] * od_ad[k];
    }
  }
}

/* Map_Input_AD (ODPS_CoordinateMapping.f90:480-547): note that only absorber
 * amounts clamped to EPSILON lose their adjoint; the Min/Max_Absorber clamps
 * pass it through, as in the reference. */
static void map_input_ad(const or_handle* h, const or_batch* b, const pstate* s,
                         const double* T_ad, double (*A_ad)[MAXK], double* Tk, double* Ak) {
  const double tol = 2.220446049250313e-16;
  const int K = h->K, Kmax = b->max_layers;
  for (int j = h->Jm - 1; j >= 0; j--) {
    int map = s->idx_map[j];
    if (map < 0 || (b->k_absorber_mask && !b->k_absorber_mask[map])) continue;
    double* out = Ak + (size_t)map * Kmax;
    for (int k = K - 1; k >= 0; k--) {
      double a = (s->A[j][k] <= tol) ? 0.0 : A_ad[j][k];
      for (int i = 0; i < s->wn[k]; i++) out[s->wi0[k] + i] += s->w[k][i] * a;
    }
  }
  for (int k = K - 1; k >= 0; k--)
    for (int i = 0; i < s->wn[k]; i++) Tk[s->wi0[k] + i] += s->w[k][i] * T_ad[k];
}

/* CRTM_Planck_Functions.f90:116-136, 358-385, 470-492, 697-723 */
static double planck_radiance(const or_handle* h, int l, double T) {
  double te = h->b1[l] + h->b2[l] * T;
  return h->c1[l] / (exp(h->c2[l] / te) - 1.0);
}
static double planck_radiance_dT(const or_handle* h, int l, double T) {
  double te = h->b1[l] + h->b2[l] * T;
  double e = exp(h->c2[l] / te);
  double d = te * (e - 1.0);
  return h->c1[l] * h->c2[l] * e * h->b2[l] / (d * d);
}
static double planck_temperature(const or_handle* h, int l, double R) {
  double te = h->c2[l] / log(h->c1[l] / R + 1.0);
  return (te - h->b1[l]) / h->b2[l];
}
static double planck_temperature_dR(const or_handle* h, int l, double R) {
  double arg = h->c1[l] / R + 1.0;
  double d = R * log(arg);
  return h->c1[l] * h->c2[l] / (h->b2[l] * arg * d * d);
}

/* CRTM_Emission (Emission_Module.f90:54-174) for a specular surface, no solar term. */
typedef struct {
  double trans_up[MAXK], trans_down[MAXK], rad_down[MAXK + 1], rad_up[MAXK + 1];
  double sec_down;
} rtv;

static double emission(int n, double u, const double* tod, const double* B, double Bs,
                       double emis, double refl, double cbr, rtv* r) {
  r->sec_down = 1.0 / u;
  r->rad_down[0] = cbr;
  for (int k = 0; k < n; k++) {
    r->trans_down[k] = exp(-tod[k] * r->sec_down);
    r->rad_down[k + 1] = r->rad_down[k] * r->trans_down[k] + B[k] * (1.0 - r->trans_down[k]);
    r->trans_up[k] = exp(-tod[k] / u);
  }
  r->rad_up[n] = emis * Bs + refl * r->rad_down[n];
  for (int k = n - 1; k >= 0; k--)
    r->rad_up[k] = r->rad_up[k + 1] * r->trans_up[k] + B[k] * (1.0 - r->trans_up[k]);
  return r->rad_up[0];
}

/* CRTM_Emission_AD (Emission_Module.f90:280-395). */
static void emission_ad(int n, double u, const double* B, double Bs, double emis, double refl,
                        const rtv* r, double up_ad, double* tod_ad, double* B_ad, double* Bs_ad,
                        double* emis_ad, double* refl_ad) {
  for (int k = 0; k < n; k++) { tod_ad[k] = 0.0; B_ad[k] = 0.0; }
  for (int k = 0; k < n; k++) {
    double a_ad = r->rad_up[k + 1] * r->trans_up[k] * up_ad;
    double src_ad = up_ad;
    up_ad = up_ad * r->trans_up[k];
    B_ad[k] += src_ad * (1.0 - r->trans_up[k]);
    a_ad -= B[k] * r->trans_up[k] * src_ad;
    tod_ad[k] -= a_ad / u;
  }
  *emis_ad = up_ad * Bs;
  *Bs_ad = emis * up_ad;
  *refl_ad = up_ad * r->rad_down[n];
  double down_ad = refl * up_ad;
  for (int k = n - 1; k >= 0; k--) {
    double a_ad = r->rad_down[k] * r->trans_down[k] * down_ad;
    double src_ad = down_ad;
    down_ad = down_ad * r->trans_down[k];
    B_ad[k] += src_ad * (1.0 - r->trans_down[k]);
    a_ad -= B[k] * r->trans_down[k] * src_ad;
    tod_ad[k] -= a_ad * r->sec_down;
  }
}

/* ---------------- drivers --------------------------------------------------- */
static double surface_temperature(const or_batch* b, int m) {
  /* CRTM_Compute_SurfaceT (CRTM_SfcOptics.f90:204-217) */
  return b->surface_land_coverage[m] * b->surface_land_temperature[m] +
         b->surface_water_coverage[m] * b->surface_water_temperature[m] +
         b->surface_snow_coverage[m] * b->surface_snow_temperature[m] +
         b->surface_ice_coverage[m] * b->surface_ice_temperature[m];
}

static int check_batch(const or_handle* h, const or_batch* b) {
  for (int m = 0; m < b->n_profiles; m++)
    if (b->n_layers[m] < 1 || b->n_layers[m] > b->max_layers || b->n_layers[m] > MAXK) {
      set_err("profile layer count out of range");
      return 3;
    }
  (void)h;
  return 0;
}

/* One profile: forward over all channels, and optionally the K-matrix/adjoint. */
static void profile_solution(const or_handle* h, const or_batch* b, int m, const double* seed,
                             double* rad, double* bt, double* lod, double* tk, double* ak,
                             double* tsk, double* ek, int adjoint_mode, double* tad,
                             double* aad, double* tsad) {
  const int L = h->L, Kmax = b->max_layers, Ku = b->n_layers[m], Jab = b->n_absorbers;
  pstate* s = (pstate*)malloc(sizeof(pstate));
  geom g;
  geometry_compute(b->sensor_zenith_angle[m], b->surface_altitude ? b->surface_altitude[m] : 0.0, &g);
  map_input(h, b, m, &g, s);
  compute_predictors(h, s);
  const double u = 1.0 / g.sec_sensor_zenith; /* Common_RTSolution.f90:227 */
  const double ts = surface_temperature(b, m);
  const double* tu = b->temperature + (size_t)m * Kmax;
  double od_ref[MAXK], lod_k[MAXK], B[MAXK], tod_ad[MAXK], B_ad[MAXK];
  double (*XA)[MAXJ][MAXI] = NULL;
  optran_adj* oa = NULL;
  double T_ad[MAXK], A_ad[MAXJM][MAXK];
  rtv r;
  int want_ad = (tk != NULL) || adjoint_mode;
  if (want_ad) {
    XA = (double (*)[MAXJ][MAXI])calloc(MAXK, sizeof *XA);
    oa = (optran_adj*)calloc(1, sizeof *oa);
  }
  for (int l = 0; l < L; l++) {
    atm_absorption(h, s, l, od_ref, lod_k);
    for (int k = 0; k < Ku; k++) B[k] = planck_radiance(h, l, tu[k]);
    double Bs = planck_radiance(h, l, ts);
    double e = b->emissivity[(size_t)m * L + l];
    double R = emission(Ku, u, lod_k, B, Bs, e, 1.0 - e, h->cbr[l], &r);
    double T = planck_temperature(h, l, R);
    size_t ml = (size_t)m * L + l;
    if (rad) rad[ml] = R;
    if (bt) bt[ml] = T;
    if (lod) for (int k = 0; k < Ku; k++) lod[ml * Kmax + k] = lod_k[k];
    if (!want_ad) continue;
    double seed_v = seed ? seed[ml] : 1.0;
    double r_ad = planck_temperature_dR(h, l, R) * seed_v;
    double Bs_ad, e_ad, refl_ad;
    emission_ad(Ku, u, B, Bs, e, 1.0 - e, &r, r_ad, tod_ad, B_ad, &Bs_ad, &e_ad, &refl_ad);
    if (!adjoint_mode) {
      memset(XA, 0, sizeof(double) * MAXK * MAXJ * MAXI);
      memset(oa, 0, sizeof *oa);
    }
    atm_absorption_ad(h, s, l, od_ref, tod_ad, XA, oa);
    double* tko = adjoint_mode ? tad + (size_t)m * Kmax : tk + ml * Kmax;
    for (int k = 0; k < Ku; k++) tko[k] += planck_radiance_dT(h, l, tu[k]) * B_ad[k];
    double st_ad = planck_radiance_dT(h, l, ts) * Bs_ad;
    if (adjoint_mode) {
      tsad[m] += b->surface_water_coverage[m] * st_ad;
    } else {
      tsk[ml] = b->surface_water_coverage[m] * st_ad;
      ek[ml] = e_ad - refl_ad;
      memset(T_ad, 0, sizeof T_ad);
      memset(A_ad, 0, sizeof A_ad);
      compute_predictors_ad(h, s, XA, T_ad, A_ad, oa);
      map_input_ad(h, b, s, T_ad, A_ad, tko, ak + ml * Jab * Kmax);
    }
  }
  if (adjoint_mode) {
    /* CRTM_Adjoint_Module.f90:1396: predictor adjoint once, after the channel loop */
    memset(T_ad, 0, sizeof T_ad);
    memset(A_ad, 0, sizeof A_ad);
    compute_predictors_ad(h, s, XA, T_ad, A_ad, oa);
    map_input_ad(h, b, s, T_ad, A_ad, tad + (size_t)m * Kmax, aad + (size_t)m * Jab * Kmax);
  }
  free(XA);
  free(oa);
  free(s);
}

int or_forward(const or_handle* h, const or_batch* b, double* radiance, double* bt,
               double* layer_od, int n_threads) {
  int st = check_batch(h, b);
  if (st) return st;
#pragma omp parallel for schedule(dynamic, 1) num_threads(n_threads > 0 ? n_threads : 1)
  for (int m = 0; m < b->n_profiles; m++)
    profile_solution(h, b, m, NULL, radiance, bt, layer_od, NULL, NULL, NULL, NULL, 0, NULL, NULL,
                     NULL);
  return 0;
}

int or_k_matrix(const or_handle* h, const or_batch* b, const double* bt_k, double* radiance,
                double* bt, double* temperature_k, double* absorber_k, double* water_temperature_k,
                double* surface_emissivity_k, int n_threads) {
  int st = check_batch(h, b);
  if (st) return st;
  const size_t PL = (size_t)b->n_profiles * h->L;
  memset(temperature_k, 0, sizeof(double) * PL * b->max_layers);
  memset(absorber_k, 0, sizeof(double) * PL * b->n_absorbers * b->max_layers);
#pragma omp parallel for schedule(dynamic, 1) num_threads(n_threads > 0 ? n_threads : 1)
  for (int m = 0; m < b->n_profiles; m++)
    profile_solution(h, b, m, bt_k, radiance, bt, NULL, temperature_k, absorber_k,
                     water_temperature_k, surface_emissivity_k, 0, NULL, NULL, NULL);
  return 0;
}

int or_adjoint(const or_handle* h, const or_batch* b, const double* bt_ad, double* radiance,
               double* bt, double* temperature_ad, double* absorber_ad,
               double* water_temperature_ad, int n_threads) {
  int st = check_batch(h, b);
  if (st) return st;
  memset(temperature_ad, 0, sizeof(double) * b->n_profiles * b->max_layers);
  memset(absorber_ad, 0, sizeof(double) * b->n_profiles * b->n_absorbers * b->max_layers);
  memset(water_temperature_ad, 0, sizeof(double) * b->n_profiles);
#pragma omp parallel for schedule(dynamic, 1) num_threads(n_threads > 0 ? n_threads : 1)
  for (int m = 0; m < b->n_profiles; m++)
    profile_solution(h, b, m, bt_ad, radiance, bt, NULL, NULL, NULL, NULL, NULL, 1, temperature_ad,
                     absorber_ad, water_temperature_ad);
  return 0;
}

int or_tangent_fd(const or_handle* hd, const or_batch* b, const double* temperature_tl,
                  const double* absorber_tl, const double* water_temperature_tl, double step,
                  double* bt_tl, int n_threads) {
  const int P = b->n_profiles, Kmax = b->max_layers, Jab = b->n_absorbers, L = hd->L;
  size_t nT = (size_t)P * Kmax, nA = (size_t)P * Jab * Kmax;
  double* t2 = (double*)malloc(sizeof(double) * nT);
  double* a2 = (double*)malloc(sizeof(double) * nA);
  double* w2 = (double*)malloc(sizeof(double) * P);
  double* bp = (double*)malloc(sizeof(double) * P * L);
  double* bm = (double*)malloc(sizeof(double) * P * L);
  or_batch c = *b;
  c.surface_water_temperature = w2;
  c.temperature = t2;
  c.absorber = a2;
  for (int sgn = 0; sgn < 2; sgn++) {
    double f = sgn ? -step : step;
    for (size_t i = 0; i < nT; i++) t2[i] = b->temperature[i] + f * temperature_tl[i];
    for (size_t i = 0; i < nA; i++) a2[i] = b->absorber[i] + f * absorber_tl[i];
    for (int i = 0; i < P; i++) w2[i] = b->surface_water_temperature[i] + f * water_temperature_tl[i];
    int st = or_forward(hd, &c, NULL, sgn ? bm : bp, NULL, n_threads);
    if (st) return st;
  }
  for (size_t i = 0; i < (size_t)P * L; i++) bt_tl[i] = (bp[i] - bm[i]) / (2.0 * step);
  free(t2); free(a2); free(w2); free(bp); free(bm);
  return 0;
}

/* Test hook: the mapped profile and predictors of profile m (X as [K][J][18]). */
int or_profile_state(const or_handle* h, const or_batch* b, int m, double* T, double* A,
                     double* sec, double* X) {
  pstate* s = (pstate*)malloc(sizeof(pstate));
  geom g;
  geometry_compute(b->sensor_zenith_angle[m], b->surface_altitude ? b->surface_altitude[m] : 0.0, &g);
  map_input(h, b, m, &g, s);
  compute_predictors(h, s);
  for (int k = 0; k < h->K; k++) {
    T[k] = s->T[k];
    sec[k] = s->sec[k];
    for (int j = 0; j < h->Jm; j++) A[j * h->K + k] = s->A[j][k];
    for (int j = 0; j < h->J; j++)
      for (int i = 0; i < MAXI; i++) X[(k * h->J + j) * MAXI + i] = s->X[k][j][i];
  }
  free(s);
  return 0;
}

/* ---- scattering (clouds, ADA) ------------------------------------------- */
#include "oracle_scatter.inc"
#include "oracle_scatter_k.inc"

/* ---- CRTM_Atmosphere_AddLayers for one profile -----------------------------
 * src/Atmosphere/CRTM_Atmosphere.f90:248-400 with Extra_Layers :1043-1050,
 * Layer_P / Layer_X :1054-1066, Interp_LPoly / Interp_Linear :1070-1084 and
 * Shift_Profile :1088-1098; the model rows come from CRTM_Get_Model_Profile
 * (src/Atmosphere/CRTM_Model_Profiles.f90:1120-1141).
 *
 * mlp[nlev]: model level pressures; mlt[nlev]: the model's level
 * temperatures; mla[J][nlev]: its level amounts of the profile's J absorbers.
 * top: the profile's Level_Pressure(0); up, ut: its first two layer
 * pressures / temperatures; ua[J][2]: its first two layers' absorber amounts.
 * Writes the n added layers: pl[n+1] level pressures, p[n], t[n], a[J][n].
 * Returns n, or 0 when no model level lies at or below the top. */
int or_add_layers(int nlev, const double* mlp, const double* mlt, const double* mla, int J,
                  double top, const double* up, const double* ut, const double* ua,
                  double* pl, double* p, double* t, double* a) {
  int n = 0;
  for (int k = 1; k < nlev; k++) {   /* 1-based DO n = 1, SIZE(...) over the 0-based levels */
    if (mlp[k] >= top) { n = k; break; }
  }
  if (n < 1) return 0;
  double tl[128], al[128];
  if (n + 1 > 128) return 0;
  for (int k = 0; k <= n; k++) { pl[k] = mlp[k]; tl[k] = mlt[k]; }
  const double w = (log(top) - log(pl[n - 1])) / (log(pl[n]) - log(pl[n - 1]));
  pl[n] = top;
  tl[n] = (tl[n] - tl[n - 1]) * w + tl[n - 1];
  for (int k = 1; k <= n; k++) {
    p[k - 1] = (pl[k] - pl[k - 1]) / log(pl[k] / pl[k - 1]);
    t[k - 1] = 0.5 * (tl[k - 1] + tl[k]);
  }
  const double e = (log(p[n - 1]) - log(up[0])) / (log(up[1]) - log(up[0]));
  const double dt = ((ut[1] - ut[0]) * e + ut[0]) - t[n - 1];
  for (int k = 0; k < n; k++) t[k] += dt;
  for (int j = 0; j < J; j++) {
    for (int k = 0; k <= n; k++) al[k] = mla[(size_t)j * nlev + k];
    al[n] = (al[n] - al[n - 1]) * w + al[n - 1];
    double* aj = a + (size_t)j * n;
    for (int k = 1; k <= n; k++) aj[k - 1] = 0.5 * (al[k - 1] + al[k]);
    const double da = ((ua[2 * j + 1] - ua[2 * j]) * e + ua[2 * j]) - aj[n - 1];
    for (int k = 0; k < n; k++) {
      aj[k] += da;
      if (aj[k] < 0.0) aj[k] = 1.0e-76;   /* MINIMUM_ABSORBER_AMOUNT, CRTM_Parameters.f90:140 */
    }
  }
  return n;
}
