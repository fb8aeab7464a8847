// Host runtime and C-ABI of the GB300 CRTM forward / K-matrix / adjoint library.
//
// crtm_gpu_init reads each sensor's SpcCoeff and ODPS TauCoeff binary files
// (the reference's record layouts: SpcCoeff_Binary_IO.f90:660-711,
// ODPS_Binary_IO.f90:586-900), builds the device tables once and keeps them
// for the life of the handle (the reference keeps them in module globals
// SC/TC after CRTM_Init, src/Coefficients/CRTM_SharedData.f90).  Each call
// then runs the chunked kernel pipeline of odps_kernels.cuh on the handle's
// stream.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "../../include/crtm_gpu.h"
#include "odps_kernels.cuh"
#include "scatter_kernels.cuh"
#include "scatter_launch.h"

using namespace crtm;

// Scratch of crtm_gpu_k_matrix_device_static: one fixed block per device,
// reserved when this library's device code is loaded on that device, so that
// the call itself allocates nothing.  With CUDA's lazy module loading (the
// default) that load happens on the module's first use on the device:
// crtm_gpu_init takes the block's address there (static_scratch_slot), which
// loads it, so a later static call never triggers the load.  128 MiB holds the intermediates of at least one profile for up to ~8500
// channels at 200 layers with 8 absorber Jacobians in FP64; larger batches
// are processed in chunks that fit.
static constexpr size_t STATIC_SCRATCH_BYTES = (size_t)CRTM_GPU_STATIC_SCRATCH_MIB << 20;
static __device__ __align__(256) unsigned char g_static_scratch[STATIC_SCRATCH_BYTES];

namespace {

thread_local std::string g_init_error;

// Device address of g_static_scratch, looked up once per device.
constexpr int MAX_STATIC_DEVICES = 64;
struct StaticScratchSlot {
  std::once_flag once;
  void* ptr = nullptr;
  cudaError_t err = cudaSuccess;
};
StaticScratchSlot g_static_slots[MAX_STATIC_DEVICES];

// The slot of device dev (current), its address looked up on first use.
StaticScratchSlot* static_scratch_slot(int dev) {
  if (dev < 0 || dev >= MAX_STATIC_DEVICES) return nullptr;
  StaticScratchSlot& slot = g_static_slots[dev];
  std::call_once(slot.once, [&slot] { slot.err = cudaGetSymbolAddress(&slot.ptr, g_static_scratch); });
  return &slot;
}

// ---------------------------------------------------------------------------
// Fortran sequential record files
// ---------------------------------------------------------------------------
struct Records {
  std::vector<unsigned char> buf;
  size_t off = 0;
  bool swap = false;

  static uint32_t bswap(uint32_t v) {
    return (v >> 24) | ((v >> 8) & 0xff00u) | ((v << 8) & 0xff0000u) | (v << 24);
  }
  uint32_t u32(size_t at) const {
    uint32_t v;
    memcpy(&v, buf.data() + at, 4);
    return swap ? bswap(v) : v;
  }
  bool open(const std::string& path, std::string& err) {
    FILE* f = fopen(path.c_str(), "rb");
    if (!f) { err = "cannot open " + path; return false; }
    fseek(f, 0, SEEK_END);
    long n = ftell(f);
    fseek(f, 0, SEEK_SET);
    buf.resize(n > 0 ? (size_t)n : 0);
    bool ok = n > 0 && fread(buf.data(), 1, buf.size(), f) == buf.size();
    fclose(f);
    if (!ok || buf.size() < 12) { err = "cannot read " + path; return false; }
    for (int s = 0; s < 2; s++) {
      swap = s == 1;
      if (u32(0) == 4 && u32(4) == 123456789u && u32(8) == 4) { off = 12; return true; }
    }
    err = path + ": not a CRTM binary file (magic number)";
    return false;
  }
  // next record; returns false on corruption
  bool next(const unsigned char*& data, size_t& len) {
    if (off + 4 > buf.size()) return false;
    uint32_t a = u32(off);
    if (off + 8 + (size_t)a > buf.size() || u32(off + 4 + a) != a) return false;
    data = buf.data() + off + 4;
    len = a;
    off += 8 + (size_t)a;
    return true;
  }
  int i32(const unsigned char* p) const {
    uint32_t v;
    memcpy(&v, p, 4);
    return (int)(swap ? bswap(v) : v);
  }
  double f64(const unsigned char* p) const {
    unsigned char b[8];
    memcpy(b, p, 8);
    if (swap) std::reverse(b, b + 8);
    double d;
    memcpy(&d, b, 8);
    return d;
  }
  float f32(const unsigned char* p) const {
    uint32_t v;
    memcpy(&v, p, 4);
    if (swap) v = bswap(v);
    float f;
    memcpy(&f, &v, 4);
    return f;
  }
};

// ---------------------------------------------------------------------------
// Sensor coefficients: host copies and device tables
// ---------------------------------------------------------------------------
struct Sensor {
  std::string id;
  int group = 0, K = 0, J = 0, Jm = 0, L = 0, Lp = 0, sensor_type = 0, h2o_idx = 0, NS = 0;
  std::vector<int> absorber_id;
  std::vector<double> ref_lev, ref_p, ref_t, ref_a, min_a, max_a;  // [Jm][K] for absorbers
  std::vector<double> c1, c2, b1, b2, cbr, freq, wn;
  // device
  float* d_C = nullptr;          // [K][NS][Lp]
  unsigned* d_cmask = nullptr;   // [L]
  double* d_tab = nullptr;       // concatenated tables
  double* d_spec = nullptr;      // c1,c2,b1,b2,cbr,frequency,wavenumber [7][L]
  SensorTables tables{};
  RefSums refsums{};
  SpecView spec{};
  // tuning per arithmetic form ([0] FP64, [1] mixed), set by
  // crtm_gpu_set_tuning or crtm_gpu_autotune_k_matrix_device: channels per
  // map_kernel CTA (0 = the handle default) and a cap on the profiles per
  // pipeline pass (0 = as many as the workspace budget holds)
  int tune_map[2] = {0, 0};
  int tune_chunk[2] = {0, 0};
  double tune_ms[2] = {0.0, 0.0};
  // all the file's channels (host copies), for channel subsets
  // (crtm_gpu_set_channel_subset): L and the device arrays above hold the
  // processed channels only
  int L_all = 0, Lp_all = 0;
  std::vector<float> C_all;          // [K][NS][Lp_all]
  std::vector<unsigned> cmask_all;   // [L_all]
  std::vector<double> spec_all;      // [7][L_all]
  std::vector<int> processed;        // file positions of the processed channels; empty: all
  // compact-OPTRAN term (host copies per file channel; o_n[l] = 0: not an OPTRAN channel)
  std::vector<int> o_n, o_idx;       // [L_all] predictor count; [L_all][8] count, OP_Index(1:6), order
  std::vector<double> o_coef;        // [L_all][OPT_NU][OPT_ORDER+1]
  double o_alpha = 1.0, o_c1 = 1.0, o_c2 = 0.0;
  int* d_oidx = nullptr;             // device: the processed OPTRAN channels' tables
  int* d_och = nullptr;
  double* d_ocoef = nullptr;
  OptranView ov{};
  // the cloud tables interpolated to the processed channels' frequencies
  // (CloudChan layout; built when the handle has a CloudCoeff table)
  double* d_zc = nullptr;
};

// The OPTRAN tables of the processed channels (file positions `pos`; all
// when empty) on the device.
bool upload_optran(Sensor& s, const std::vector<int>& pos, std::string& err) {
  cudaFree(s.d_oidx); cudaFree(s.d_och); cudaFree(s.d_ocoef);
  s.d_oidx = nullptr; s.d_och = nullptr; s.d_ocoef = nullptr;
  s.ov = OptranView{};
  s.ov.alpha = s.o_alpha; s.ov.alpha_c1 = s.o_c1; s.ov.alpha_c2 = s.o_c2;
  std::vector<int> ch, ix;
  std::vector<double> cf;
  const int n = pos.empty() ? s.L_all : (int)pos.size();
  const size_t nc = (size_t)OPT_NU * (OPT_ORDER + 1);
  for (int l = 0; l < n; l++) {
    const int q = pos.empty() ? l : pos[l];
    if (q < 0 || q >= (int)s.o_n.size() || s.o_n[q] <= 0) continue;
    ch.push_back(l);
    ix.insert(ix.end(), s.o_idx.begin() + (size_t)q * 8, s.o_idx.begin() + (size_t)q * 8 + 8);
    cf.insert(cf.end(), s.o_coef.begin() + (size_t)q * nc, s.o_coef.begin() + (size_t)q * nc + nc);
  }
  if (ch.empty()) return true;
  cudaError_t ce;
  if ((ce = cudaMalloc(&s.d_och, ch.size() * sizeof(int))) != cudaSuccess ||
      (ce = cudaMalloc(&s.d_oidx, ix.size() * sizeof(int))) != cudaSuccess ||
      (ce = cudaMalloc(&s.d_ocoef, cf.size() * sizeof(double))) != cudaSuccess ||
      (ce = cudaMemcpy(s.d_och, ch.data(), ch.size() * sizeof(int), cudaMemcpyHostToDevice)) != cudaSuccess ||
      (ce = cudaMemcpy(s.d_oidx, ix.data(), ix.size() * sizeof(int), cudaMemcpyHostToDevice)) != cudaSuccess ||
      (ce = cudaMemcpy(s.d_ocoef, cf.data(), cf.size() * sizeof(double), cudaMemcpyHostToDevice)) != cudaSuccess) {
    err = std::string("device upload of the OPTRAN tables failed: ") + cudaGetErrorString(ce);
    return false;
  }
  s.ov.n = (int)ch.size();
  s.ov.ch = s.d_och; s.ov.idx = s.d_oidx; s.ov.coef = s.d_ocoef;
  return true;
}

bool load_sensor(const std::string& dir, const std::string& id, Sensor& s, std::string& err) {
  s.id = id;
  Records r;
  const unsigned char* d;
  size_t len;
  std::string tau = dir + "/" + id + ".TauCoeff.bin";
  if (!r.open(tau, err)) return false;
  auto bad = [&](const char* what) { err = tau + ": " + what; return false; };
  if (!r.next(d, len) || len != 8) return bad("corrupt Release/Version record");
  if (r.i32(d) != 2) return bad("unsupported ODPS release");
  if (!r.next(d, len) || len != 4) return bad("corrupt Algorithm record");
  if (r.i32(d) != 2) return bad("TauCoeff algorithm is not ODPS");
  if (!r.next(d, len) || len != 28) return bad("corrupt dimension record");
  int dims[7];
  for (int i = 0; i < 7; i++) dims[i] = r.i32(d + 4 * i);
  s.K = dims[0]; s.J = dims[1]; s.Jm = dims[2]; s.L = dims[3];
  const long long n_coeffs = dims[4];
  if (s.K < 2 || s.K > MAX_LAYERS || s.L < 1) return bad("dimensions out of range");
  if (!r.next(d, len) || len != 4) return bad("corrupt Group record");
  s.group = r.i32(d);
  if (s.group < 1 || s.group > 3 || group_j(s.group) != s.J || group_jm(s.group) != s.Jm)
    return bad("unsupported ODPS predictor group");
  s.NS = group_ns(s.group);
  if (!r.next(d, len) || len != 32) return bad("corrupt sensor-id record");
  s.sensor_type = r.i32(d + 28);
  if (!r.next(d, len) || len != 4u * s.L) return bad("corrupt channel record");
  if (!r.next(d, len) || len != 4u * s.J) return bad("corrupt component record");
  if (!r.next(d, len) || len != 4u * s.Jm) return bad("corrupt absorber record");
  s.absorber_id.resize(s.Jm);
  for (int j = 0; j < s.Jm; j++) s.absorber_id[j] = r.i32(d + 4 * j);
  const size_t nref = (size_t)(s.K + 1) + 2 * s.K + 3 * (size_t)s.K * s.Jm;
  if (!r.next(d, len) || len != 8 * nref) return bad("corrupt reference-profile record");
  size_t o = 0;
  auto take = [&](std::vector<double>& v, size_t n) {
    v.resize(n);
    for (size_t i = 0; i < n; i++) v[i] = r.f64(d + 8 * (o + i));
    o += n;
  };
  take(s.ref_lev, s.K + 1);
  take(s.ref_p, s.K);
  take(s.ref_t, s.K);
  take(s.ref_a, (size_t)s.K * s.Jm);
  take(s.min_a, (size_t)s.K * s.Jm);
  take(s.max_a, (size_t)s.K * s.Jm);
  for (int k = 0; k < s.K; k++)
    if (!(s.ref_lev[k + 1] > s.ref_lev[k]) || !(s.ref_p[k] > 0.0) || !(s.ref_t[k] > 0.0))
      return bad("reference profile is not monotone / positive");
  if (!r.next(d, len) || len != 8u * s.J * s.L) return bad("corrupt n_Predictors record");
  std::vector<int> npred((size_t)s.J * s.L), pos((size_t)s.J * s.L);
  for (size_t i = 0; i < npred.size(); i++) {
    npred[i] = r.i32(d + 4 * i);
    pos[i] = r.i32(d + 4 * (npred.size() + i));
  }
  std::vector<float> C(n_coeffs > 0 ? (size_t)n_coeffs : 0);
  if (n_coeffs > 0) {
    if (!r.next(d, len) || len != 4u * (size_t)n_coeffs) return bad("corrupt coefficient record");
    for (long long i = 0; i < n_coeffs; i++) C[i] = r.f32(d + 4 * i);
  }
  // compact OPTRAN (ODPS_Binary_IO.f90:778-800): OSignificance(L), Order(L),
  // OP_Index(0:6, L), OPos_Index(L), OC(n), Alpha, Alpha_C1, Alpha_C2,
  // OComponent_Index
  const long long n_oc = dims[6];
  int ocomp = -1;
  s.o_n.assign(s.L, 0);
  if (n_oc > 0) {
    const size_t want = 4u * (size_t)s.L * (3 + OPT_NU) + 8u * (size_t)n_oc + 24 + 4;
    if (!r.next(d, len) || len != want) return bad("corrupt OPTRAN record");
    const int L = s.L;
    size_t o2 = 0;
    std::vector<int> sig(L), ord(L), opi((size_t)L * OPT_NU), opos(L);
    for (int l = 0; l < L; l++) sig[l] = r.i32(d + o2 + 4 * l);
    o2 += 4u * L;
    for (int l = 0; l < L; l++) ord[l] = r.i32(d + o2 + 4 * l);
    o2 += 4u * L;
    for (size_t i = 0; i < opi.size(); i++) opi[i] = r.i32(d + o2 + 4 * i);
    o2 += 4u * opi.size();
    for (int l = 0; l < L; l++) opos[l] = r.i32(d + o2 + 4 * l);
    o2 += 4u * L;
    std::vector<double> oc(n_oc);
    for (long long i = 0; i < n_oc; i++) oc[i] = r.f64(d + o2 + 8 * i);
    o2 += 8u * (size_t)n_oc;
    s.o_alpha = r.f64(d + o2); s.o_c1 = r.f64(d + o2 + 8); s.o_c2 = r.f64(d + o2 + 16);
    ocomp = r.i32(d + o2 + 24) - 1;
    if (ocomp < 0 || ocomp >= s.J) return bad("OPTRAN OComponent_Index out of range");
    if (!(s.o_alpha != 0.0) || !(s.o_c1 != 0.0)) return bad("OPTRAN Alpha or Alpha_C1 is zero");
    s.o_idx.assign((size_t)L * 8, 0);
    s.o_coef.assign((size_t)L * OPT_NU * (OPT_ORDER + 1), 0.0);
    for (int l = 0; l < L; l++) {
      // OPTRAN replaces the component where the channel has it at all
      // (ODPS_AtmAbsorption.f90:172-195); Add_OPTRAN_wloOD adds nothing
      // where OP_Index(0) is 0
      if (sig[l] != 1 || npred[(size_t)l * s.J + ocomp] <= 0) continue;
      const int np = opi[(size_t)l * OPT_NU], od = ord[l];
      if (np < 0 || np > OPT_NU - 1 || od < 0 || od > OPT_ORDER) return bad("OPTRAN order or predictor count");
      s.o_n[l] = -1;   // the ODPS component is replaced
      if (np == 0) continue;
      for (int i = 1; i <= np; i++)
        if (opi[(size_t)l * OPT_NU + i] < 1 || opi[(size_t)l * OPT_NU + i] > 14) return bad("OPTRAN OP_Index");
      const long long p0 = (long long)opos[l] - 1;
      if (p0 < 0 || p0 + (long long)(np + 1) * (od + 1) > n_oc) return bad("OPTRAN OPos_Index out of range");
      s.o_n[l] = np;
      int* ix = &s.o_idx[(size_t)l * 8];
      ix[0] = np;
      for (int i = 1; i <= np; i++) ix[i] = opi[(size_t)l * OPT_NU + i];
      ix[7] = od;
      double* cf = &s.o_coef[(size_t)l * OPT_NU * (OPT_ORDER + 1)];
      for (int i = 0; i <= np; i++)
        for (int j = 0; j <= od; j++) cf[i * (OPT_ORDER + 1) + j] = oc[p0 + (size_t)i * (od + 1) + j];
    }
  }
  // dense coefficient array [K][NS][L] and component masks
  const int K = s.K, L = s.L, NS = s.NS;
  s.Lp = (L + 31) / 32 * 32;   // 128-byte aligned coefficient rows
  const int Lp = s.Lp;
  std::vector<float> Cd((size_t)K * NS * Lp, 0.0f);
  std::vector<unsigned> cmask(L, 0u);
  static const int npmax[3][8] = {{7, 18, 7, 11, 11, 14, 10, 11}, {7, 15, 7, 11, 10}, {7, 14}};
  for (int l = 0; l < L; l++) {
    int off = 0;
    for (int j = 0; j < s.J; j++) {
      const int np = npred[(size_t)l * s.J + j];
      const int mx = npmax[s.group - 1][j];
      if (np > mx) return bad("n_Predictors exceeds the group's predictor count");
      if (np > 0 && !(j == ocomp && s.o_n[l] != 0)) {   // an OPTRAN channel's component: OPTRAN instead
        const long long p0 = (long long)pos[(size_t)l * s.J + j] - 1;
        if (p0 < 0 || p0 + (long long)np * K > n_coeffs) return bad("Pos_Index out of range");
        cmask[l] |= 1u << j;
        for (int i = 0; i < np; i++)
          for (int k = 0; k < K; k++)
            Cd[((size_t)k * NS + off + i) * Lp + l] = C[p0 + (size_t)i * K + k];
      }
      off += mx;
    }
  }
  // SpcCoeff
  Records sr;
  std::string spc = dir + "/" + id + ".SpcCoeff.bin";
  if (!sr.open(spc, err)) return false;
  auto sbad = [&](const char* what) { err = spc + ": " + what; return false; };
  if (!sr.next(d, len) || len != 8) return sbad("corrupt Release/Version record");
  if (sr.i32(d + 4) < 3) return sbad("SpcCoeff version < 3 is not supported");
  if (!sr.next(d, len) || len != 4) return sbad("corrupt dimension record");
  if (sr.i32(d) != L) return sbad("channel count differs from the TauCoeff file");
  if (!sr.next(d, len) || len != 32) return sbad("corrupt sensor-id record");
  if (!sr.next(d, len) || len != (size_t)L * (4 + 4 + 8 + 4 + 8 * 8)) return sbad("corrupt channel record");
  const size_t base = (size_t)L * 20;  // after channel, polarization, pol angle, flag
  auto col = [&](int f, std::vector<double>& v) {
    v.resize(L);
    for (int l = 0; l < L; l++) v[l] = sr.f64(d + base + 8 * ((size_t)f * L + l));
  };
  // fields after the integer/polangle block: Frequency(0) Wavenumber(1) C1(2) C2(3) B1(4) B2(5) CBR(6) Solar(7)
  col(0, s.freq); col(1, s.wn); col(2, s.c1); col(3, s.c2); col(4, s.b1); col(5, s.b2); col(6, s.cbr);
  s.h2o_idx = (s.absorber_id[s.Jm - 1] == 1) ? s.Jm - 1 : 0;
  // derived tables
  std::vector<double> lev_lnp(K + 1), lnp(K), pdp(K), z(K + 1);
  for (int k = 0; k <= K; k++) lev_lnp[k] = std::log(s.ref_lev[k]);
  for (int k = 0; k < K; k++) lnp[k] = std::log(s.ref_p[k]);
  for (int k = 0; k < K; k++)  // ODPS_Predictor.f90:690-700
    pdp[k] = (k == 0) ? s.ref_lev[0] * (s.ref_lev[1] - s.ref_lev[0])
                      : s.ref_lev[k + 1] * (s.ref_lev[k + 1] - s.ref_lev[k]);
  z[K] = 0.0;  // Geopotential_Height, ODPS_CoordinateMapping.f90:607-634
  for (int k = K; k >= 1; k--)
    z[k - 1] = z[k] + CC_H * s.ref_t[k - 1] * (1.0 + C_TV * s.ref_a[(size_t)s.h2o_idx * K + k - 1]) *
                          std::log(s.ref_lev[k] / s.ref_lev[k - 1]);
  std::vector<double> tab;
  auto put = [&](const std::vector<double>& v) { size_t at = tab.size(); tab.insert(tab.end(), v.begin(), v.end()); return at; };
  size_t o_lev = put(s.ref_lev), o_levl = put(lev_lnp), o_lnp = put(lnp), o_t = put(s.ref_t);
  size_t o_a = put(s.ref_a), o_mn = put(s.min_a), o_mx = put(s.max_a), o_pdp = put(pdp), o_z = put(z);
  size_t o_rp = put(s.ref_p);
  // running sums of the reference profile (ODPS_Predictor.f90:707-759, the *_ref terms)
  std::vector<double> tzr(K), tzpr(K), gzr((size_t)s.Jm * K), gtr((size_t)s.Jm * K);
  {
    double a0 = 0, a1 = 0;
    for (int k = 0; k < K; k++) { a0 += s.ref_t[k]; a1 += pdp[k] * s.ref_t[k]; tzr[k] = a0; tzpr[k] = a1; }
    for (int j = 0; j < s.Jm; j++) {
      double g0 = 0, g1 = 0;
      for (int k = 0; k < K; k++) {
        const double ra = s.ref_a[(size_t)j * K + k];
        g0 += pdp[k] * ra;
        g1 += pdp[k] * ra * s.ref_t[k];
        gzr[(size_t)j * K + k] = g0;
        gtr[(size_t)j * K + k] = g1;
      }
    }
  }
  size_t o_tzr = put(tzr), o_tzpr = put(tzpr), o_gzr = put(gzr), o_gtr = put(gtr);
  std::vector<double> spec;
  for (auto* v : {&s.c1, &s.c2, &s.b1, &s.b2, &s.cbr, &s.freq, &s.wn}) spec.insert(spec.end(), v->begin(), v->end());
  s.L_all = L;
  s.Lp_all = Lp;
  s.C_all = Cd;
  s.cmask_all = cmask;
  s.spec_all = spec;
  cudaError_t ce;
  if ((ce = cudaMalloc(&s.d_C, Cd.size() * sizeof(float))) != cudaSuccess ||
      (ce = cudaMalloc(&s.d_cmask, cmask.size() * sizeof(unsigned))) != cudaSuccess ||
      (ce = cudaMalloc(&s.d_tab, tab.size() * sizeof(double))) != cudaSuccess ||
      (ce = cudaMalloc(&s.d_spec, spec.size() * sizeof(double))) != cudaSuccess ||
      (ce = cudaMemcpy(s.d_C, Cd.data(), Cd.size() * sizeof(float), cudaMemcpyHostToDevice)) != cudaSuccess ||
      (ce = cudaMemcpy(s.d_cmask, cmask.data(), cmask.size() * sizeof(unsigned), cudaMemcpyHostToDevice)) != cudaSuccess ||
      (ce = cudaMemcpy(s.d_tab, tab.data(), tab.size() * sizeof(double), cudaMemcpyHostToDevice)) != cudaSuccess ||
      (ce = cudaMemcpy(s.d_spec, spec.data(), spec.size() * sizeof(double), cudaMemcpyHostToDevice)) != cudaSuccess) {
    err = std::string("device upload of ") + id + " coefficients failed: " + cudaGetErrorString(ce);
    return false;
  }
  SensorTables& t = s.tables;
  t.group = s.group; t.K = K; t.J = s.J; t.Jm = s.Jm; t.L = L; t.sensor_type = s.sensor_type;
  t.h2o_idx = s.h2o_idx;
  t.ref_lev = s.d_tab + o_lev; t.ref_lev_lnp = s.d_tab + o_levl; t.ref_lnp = s.d_tab + o_lnp;
  t.ref_t = s.d_tab + o_t; t.ref_a = s.d_tab + o_a; t.min_a = s.d_tab + o_mn; t.max_a = s.d_tab + o_mx;
  t.pdp = s.d_tab + o_pdp; t.zgeo = s.d_tab + o_z; t.ref_p = s.d_tab + o_rp;
  t.o_alpha = s.o_alpha; t.o_c1 = s.o_c1; t.o_c2 = s.o_c2;
  if (!upload_optran(s, std::vector<int>(), err)) return false;
  s.refsums.tz_ref = s.d_tab + o_tzr; s.refsums.tzp_ref = s.d_tab + o_tzpr;
  s.refsums.gazp_ref = s.d_tab + o_gzr; s.refsums.gatzp_ref = s.d_tab + o_gtr;
  s.spec.c1 = s.d_spec; s.spec.c2 = s.d_spec + L; s.spec.b1 = s.d_spec + 2 * L;
  s.spec.b2 = s.d_spec + 3 * L; s.spec.cbr = s.d_spec + 4 * L;
  s.spec.freq = s.d_spec + 5 * L; s.spec.wn = s.d_spec + 6 * L;
  return true;
}

// The device arrays of the channels at file positions `pos` (all channels
// when empty): coefficients [K][NS][Lp], component masks and SpcCoeff
// columns, gathered from the host copies.
bool upload_channels(Sensor& s, const std::vector<int>& pos, std::string& err) {
  const int K = s.K, NS = s.NS;
  const bool all = pos.empty();
  const int L = all ? s.L_all : (int)pos.size();
  const int Lp = std::max(32, (L + 31) / 32 * 32);
  std::vector<float> Cd((size_t)K * NS * Lp, 0.0f);
  std::vector<unsigned> cmask(std::max(L, 1), 0u);
  std::vector<double> spec((size_t)7 * std::max(L, 1), 0.0);
  for (int l = 0; l < L; l++) {
    const int q = all ? l : pos[l];
    for (size_t r = 0; r < (size_t)K * NS; r++) Cd[r * Lp + l] = s.C_all[r * s.Lp_all + q];
    cmask[l] = s.cmask_all[q];
    for (int f = 0; f < 7; f++) spec[(size_t)f * L + l] = s.spec_all[(size_t)f * s.L_all + q];
  }
  float* dC = nullptr;
  unsigned* dm = nullptr;
  double* ds = nullptr;
  cudaError_t ce;
  if ((ce = cudaMalloc(&dC, Cd.size() * sizeof(float))) != cudaSuccess ||
      (ce = cudaMalloc(&dm, cmask.size() * sizeof(unsigned))) != cudaSuccess ||
      (ce = cudaMalloc(&ds, spec.size() * sizeof(double))) != cudaSuccess ||
      (ce = cudaMemcpy(dC, Cd.data(), Cd.size() * sizeof(float), cudaMemcpyHostToDevice)) != cudaSuccess ||
      (ce = cudaMemcpy(dm, cmask.data(), cmask.size() * sizeof(unsigned), cudaMemcpyHostToDevice)) != cudaSuccess ||
      (ce = cudaMemcpy(ds, spec.data(), spec.size() * sizeof(double), cudaMemcpyHostToDevice)) != cudaSuccess) {
    cudaFree(dC); cudaFree(dm); cudaFree(ds);
    err = std::string("device upload of the channel subset failed: ") + cudaGetErrorString(ce);
    return false;
  }
  cudaFree(s.d_C); cudaFree(s.d_cmask); cudaFree(s.d_spec);
  s.d_C = dC; s.d_cmask = dm; s.d_spec = ds;
  s.L = L; s.Lp = Lp; s.tables.L = L;
  s.spec.c1 = ds; s.spec.c2 = ds + L; s.spec.b1 = ds + 2 * L;
  s.spec.b2 = ds + 3 * L; s.spec.cbr = ds + 4 * L;
  s.spec.freq = ds + 5 * L; s.spec.wn = ds + 6 * L;
  for (int f = 0; f < 7; f++) {
    std::vector<double>* v[7] = {&s.c1, &s.c2, &s.b1, &s.b2, &s.cbr, &s.freq, &s.wn};
    v[f]->assign(spec.begin() + (size_t)f * L, spec.begin() + (size_t)f * L + L);
  }
  s.processed = pos;
  return upload_optran(s, pos, err);
}

void free_sensor(Sensor& s) {
  cudaFree(s.d_C); cudaFree(s.d_cmask); cudaFree(s.d_tab); cudaFree(s.d_spec);
  cudaFree(s.d_oidx); cudaFree(s.d_och); cudaFree(s.d_ocoef); cudaFree(s.d_zc);
  s.d_C = nullptr; s.d_cmask = nullptr; s.d_tab = nullptr; s.d_spec = nullptr;
  s.d_oidx = nullptr; s.d_och = nullptr; s.d_ocoef = nullptr; s.d_zc = nullptr;
}

// The cloud tables at each processed channel's frequency (CloudChan layout):
// one thread per (plane, radius row, channel), the frequency step of the
// lookups' 4-point Lagrange interpolation.
__global__ void cloud_chan_kernel(CloudLut C, int microwave, const double* freq, int L, long long n, double* z) {
  const int rows = microwave ? C.nrm : C.nri, nf = microwave ? C.nfm : C.nfi;
  const double* fax = microwave ? C.f_mw : C.f_ir;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int ch = (int)(i % L);
    const long long qr = i / L;
    const int r = (int)(qr % rows), q = (int)(qr / rows);
    const Lagrange4 U = lagrange4(fax, nf, freq[ch]);
    z[i] = lerp4(cloud_chan_source(C, microwave != 0, q) + (size_t)r * nf + U.i0, 1, U);
  }
}

// (Re)build a sensor's channel-interpolated cloud tables for its processed
// channels; none without a cloud table or channels.
bool build_cloud_chan(const CloudLut& C, bool has_clouds, Sensor& s, std::string& err) {
  cudaFree(s.d_zc);
  s.d_zc = nullptr;
  if (!has_clouds || s.L <= 0) return true;
  const bool mw = s.sensor_type == 1;
  const long long n = (long long)cloud_chan_planes(C, mw) * (mw ? C.nrm : C.nri) * s.L;
  cudaError_t ce = cudaMalloc(&s.d_zc, (size_t)n * sizeof(double));
  if (ce == cudaSuccess) {
    const long long blocks = std::min<long long>((n + 255) / 256, 152LL * 16);
    cloud_chan_kernel<<<(unsigned)blocks, 256>>>(C, mw ? 1 : 0, mw ? s.spec.freq : s.spec.wn, s.L, n, s.d_zc);
    ce = cudaGetLastError();
    if (ce == cudaSuccess) ce = cudaDeviceSynchronize();
  }
  if (ce != cudaSuccess) {
    cudaFree(s.d_zc);
    s.d_zc = nullptr;
    err = std::string("channel cloud tables: ") + cudaGetErrorString(ce);
    return false;
  }
  return true;
}

// CloudCoeff.bin (CloudCoeff_Binary_IO.f90:360-460): Release/Version, 8
// dimensions, the axis vectors, then (ke, w, g, pcoeff) for the MW liquid,
// MW solid and IR tables.  Only phase element 1 of pcoeff is kept; g is not
// used by this path.
bool load_cloudcoeff(const std::string& path, std::vector<double>& buf, int* dims, size_t* off,
                     std::string& err) {
  Records r;
  if (!r.open(path, err)) return false;
  const unsigned char* d;
  size_t len;
  auto bad = [&](const char* what) { err = path + ": " + what; return false; };
  if (!r.next(d, len) || len != 8) return bad("corrupt Release/Version record");
  if (r.i32(d) != 3) return bad("unsupported CloudCoeff release");
  if (!r.next(d, len) || len != 32) return bad("corrupt dimension record");
  int nd8[8];
  for (int i = 0; i < 8; i++) nd8[i] = r.i32(d + 4 * i);
  const int nfm = nd8[0], nrm = nd8[1], nfi = nd8[2], nri = nd8[3], nt = nd8[4], nd = nd8[5],
            nleg = nd8[6], nph = nd8[7];
  if (nfm < 4 || nrm < 4 || nfi < 4 || nri < 4 || nt < 4 || nd < 1 || nleg < 1 || nleg > 64 || nph < 1)
    return bad("dimensions out of range");
  buf.clear();
  auto take = [&](const unsigned char* src, size_t n) {
    size_t at = buf.size();
    for (size_t i = 0; i < n; i++) buf.push_back(r.f64(src + 8 * i));
    return at;
  };
  const size_t na = (size_t)nfm + nfi + nrm + nri + nt + nd;
  if (!r.next(d, len) || len != 8 * na) return bad("corrupt axis record");
  off[0] = take(d, nfm);                                   // frequency MW
  off[1] = take(d + 8 * nfm, nfi);                         // frequency IR
  off[2] = take(d + 8 * ((size_t)nfm + nfi), nrm);         // radius MW
  off[3] = take(d + 8 * ((size_t)nfm + nfi + nrm), nri);   // radius IR
  off[4] = take(d + 8 * ((size_t)nfm + nfi + nrm + nri), nt);   // temperature
  const size_t n3[3] = {(size_t)nfm * nrm * nt, (size_t)nfm * nrm * nd, (size_t)nfi * nri * (nd + 1)};
  const size_t nl[3] = {(size_t)nleg + 1, (size_t)nleg + 1, (size_t)nleg};
  for (int bk = 0; bk < 3; bk++) {
    const size_t np = n3[bk] * nl[bk] * nph;
    if (!r.next(d, len) || len != 8 * (3 * n3[bk] + np)) return bad("corrupt LUT record");
    off[5 + 3 * bk] = take(d, n3[bk]);                          // ke
    off[6 + 3 * bk] = take(d + 8 * n3[bk], n3[bk]);             // w
    off[7 + 3 * bk] = take(d + 8 * 3 * n3[bk], n3[bk] * nl[bk]); // pcoeff, phase element 1
  }
  dims[0] = nfm; dims[1] = nrm; dims[2] = nt; dims[3] = nd; dims[4] = nfi; dims[5] = nri; dims[6] = nleg;
  return true;
}

// AerosolCoeff file (AerosolCoeff_Binary_IO.f90:396-530): Release/Version,
// 7 dimensions, n_RH_Radii ('CRTM' and 'CMAQ' files only), the data-source
// string, type ids, type names, (wavelength, Reff, Rsig, RH), then (ke, w, g,
// pcoeff).  The RH axis has n_RH_Radii entries in 'CRTM' / 'CMAQ' files and
// n_RH in 'GOCART-GEOS5' / 'NAAPS' ones (AerosolCoeff_Define.f90:342-354).
// Version > 300 files carry kb as well and are refused here.  dims: nw nrh nr
// ns nt nleg n_rh_axis; off: freq reff ke w pc rsig rh.
bool load_aerosolcoeff(const std::string& path, int scheme, std::vector<double>& buf, std::vector<int>& types,
                       int* dims, size_t* off, std::string& err) {
  Records r;
  if (!r.open(path, err)) return false;
  const unsigned char* d;
  size_t len;
  auto bad = [&](const char* what) { err = path + ": " + what; return false; };
  if (!r.next(d, len) || len != 8) return bad("corrupt Release/Version record");
  if (r.i32(d) != 4) return bad("unsupported AerosolCoeff release");
  if (r.i32(d + 4) > 300) return bad("AerosolCoeff files with kb (Version > 300) are not supported");
  if (!r.next(d, len) || len != 28) return bad("corrupt dimension record");
  int dm[7];
  for (int i = 0; i < 7; i++) dm[i] = r.i32(d + 4 * i);
  const int nw = dm[0], nr = dm[1], ns = dm[2], nt = dm[3], nrh = dm[4], nleg = dm[5], nph = dm[6];
  if (nw < 4 || nr < 1 || ns < 1 || nt < 1 || nrh < 1 || nleg < 1 || nleg > 64 || nph < 1)
    return bad("dimensions out of range");
  // the interpolated axes need the 4-point window
  if ((scheme <= AEROSOL_CMAQ && nr < 4) || (scheme == AEROSOL_CMAQ && ns < 4) ||
      (scheme >= AEROSOL_GOCART && nrh < 4))
    return bad("an axis that the aerosol scheme interpolates has fewer than 4 entries");
  int nrr = nrh;
  if (scheme <= AEROSOL_CMAQ) {
    if (!r.next(d, len) || len != 4) return bad("corrupt n_RH_Radii record");
    nrr = r.i32(d);
    if (nrr < 1) return bad("n_RH_Radii out of range");
  }
  if (!r.next(d, len) || len != 4) return bad("corrupt string-length record");
  if (!r.next(d, len)) return bad("corrupt data-source record");
  if (!r.next(d, len) || len != 4u * nt) return bad("corrupt type record");
  types.resize(nt);
  for (int t = 0; t < nt; t++) types[t] = r.i32(d + 4 * t);
  if (!r.next(d, len) || len != 4) return bad("corrupt string-length record");
  if (!r.next(d, len)) return bad("corrupt type-name record");
  const size_t nax = (size_t)nw + (size_t)nr * nt + (size_t)ns * nt + nrr;
  if (!r.next(d, len) || len != 8 * nax) return bad("corrupt axis record");
  buf.clear();
  off[0] = 0;
  for (int i = 0; i < nw; i++) buf.push_back(1.0e4 / r.f64(d + 8 * i));   // micron_to_inverse_cm
  for (int i = 1; i < nw; i++)
    if (!(buf[i] > buf[i - 1])) return bad("frequencies (10^4/wavelength) must increase");
  off[1] = buf.size();
  for (size_t i = 0; i < (size_t)nr * nt; i++) buf.push_back(r.f64(d + 8 * (nw + i)));
  off[5] = buf.size();
  for (size_t i = 0; i < (size_t)ns * nt; i++) buf.push_back(r.f64(d + 8 * (nw + (size_t)nr * nt + i)));
  off[6] = buf.size();
  for (size_t i = 0; i < (size_t)nrr; i++) buf.push_back(r.f64(d + 8 * (nw + (size_t)(nr + ns) * nt + i)));
  const size_t n5 = (size_t)nw * nrh * nr * ns * nt;
  if (!r.next(d, len) || len != 8 * (3 * n5 + n5 * (nleg + 1) * nph)) return bad("corrupt LUT record");
  off[2] = buf.size();
  for (size_t i = 0; i < n5; i++) buf.push_back(r.f64(d + 8 * i));
  off[3] = buf.size();
  for (size_t i = 0; i < n5; i++) buf.push_back(r.f64(d + 8 * (n5 + i)));
  off[4] = buf.size();
  for (size_t i = 0; i < n5 * (nleg + 1); i++) buf.push_back(r.f64(d + 8 * (3 * n5 + i)));
  dims[0] = nw; dims[1] = nrh; dims[2] = nr; dims[3] = ns; dims[4] = nt; dims[5] = nleg; dims[6] = nrr;
  return true;
}

// IRwaterCoeff file (IRwaterCoeff_Define.f90:805-984): Release/Version, the
// 4 dimensions, 5 global attributes (a length record, then the text when the
// length is not 0), the classification name, the axes (angle, frequency,
// wind speed, temperature), the emissivity.  dims: na nf nv nt nalli2;
// off: angle freq wind temp e.
bool load_irwatercoeff(const std::string& path, std::vector<double>& buf, int* dims, size_t* off,
                       std::string& err) {
  Records r;
  if (!r.open(path, err)) return false;
  const unsigned char* d;
  size_t len;
  auto bad = [&](const char* what) { err = path + ": " + what; return false; };
  if (!r.next(d, len) || len != 8) return bad("corrupt Release/Version record");
  if (r.i32(d) != 4) return bad("unsupported IRwaterCoeff release");
  if (!r.next(d, len) || len != 16) return bad("corrupt dimension record");
  const int na = r.i32(d), nf = r.i32(d + 4), nv = r.i32(d + 8), nt = r.i32(d + 12);
  if (na < 4 || nf < 4 || nv < 4 || nt < 1) return bad("dimensions out of range");
  for (int g = 0; g < 5; g++) {
    if (!r.next(d, len) || len != 4) return bad("corrupt global attribute");
    if (r.i32(d) > 0 && !r.next(d, len)) return bad("corrupt global attribute");
  }
  if (!r.next(d, len) || len != 80) return bad("corrupt classification record");
  const std::string name(reinterpret_cast<const char*>(d), 80);
  const bool nalli2 = name.compare(0, 6, "Nalli2") == 0 && (name.size() == 6 || name[6] == ' ');
  if (nalli2 && nt < 4) return bad("a Nalli2 table needs at least 4 temperatures");
  const size_t nax = (size_t)na + nf + nv + nt, ne = (size_t)na * nf * nv * nt;
  if (!r.next(d, len) || len != 8 * nax) return bad("corrupt axis record");
  buf.clear();
  for (size_t i = 0; i < nax; i++) buf.push_back(r.f64(d + 8 * i));
  off[0] = 0; off[1] = na; off[2] = na + nf; off[3] = na + nf + nv; off[4] = nax;
  if (!r.next(d, len) || len != 8 * ne) return bad("corrupt emissivity record");
  for (size_t i = 0; i < ne; i++) buf.push_back(r.f64(d + 8 * i));
  dims[0] = na; dims[1] = nf; dims[2] = nv; dims[3] = nt; dims[4] = nalli2 ? 1 : 0;
  return true;
}

// Grow-only device buffer
struct DevBuf {
  void* p = nullptr;
  size_t n = 0;
  bool ensure(size_t bytes) {
    if (bytes <= n) return true;
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
    if (cudaMalloc(&p, bytes) != cudaSuccess) return false;
    n = bytes;
    return true;
  }
  void release() { if (p) cudaFree(p); p = nullptr; n = 0; }
};

}  // namespace

struct crtm_gpu_context {
  std::vector<Sensor> sensors;
  int precision = CRTM_GPU_FP64;
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string error;
  long long launches = 0;
  size_t workspace_budget = (size_t)8 << 30;
  int map_channels = 16;   // channels per map_kernel CTA (power of two, 8..32; 16 measured fastest on C2)
  int soi_slots = 20;      // SOI K-matrix/adjoint: order fields kept per (profile, channel), 17..75
  DevBuf ws;        // chunk workspace
  DevBuf io_in, io_out;  // device copies for the host entry points
  DevBuf io_tl;          // tangent-linear inputs of the host entry point
  DevBuf tl_k;           // tangent linear: the K-matrix it contracts
  // the trajectory of crtm_gpu_linearize (its K-matrix in tl_k, the profiles'
  // layer counts and status in lin_meta)
  struct {
    bool valid = false;
    int sensor = -1, P = 0, L = 0, Km = 0, J = 0, NC = 0, NA = 0;
    crtm_gpu_kmatrix k{};
    int* n_layers = nullptr;
    int* status = nullptr;
  } lin;
  DevBuf lin_meta;
  DevBuf small;     // idx maps
  // cloud LUT (CloudCoeff.bin), when present
  bool has_clouds = false;
  double* d_cloud = nullptr;
  CloudLut lut{};
  // aerosol LUT (AerosolCoeff.bin, scheme 'CRTM'), when present
  bool has_aerosols = false;
  double* d_aero = nullptr;
  int* d_aero_type = nullptr;
  AerosolLut alut{};
  // IR sea-surface emissivity table (Nalli.IRwater.EmisCoeff.bin), when present
  bool has_irwater = false;
  double* d_irw = nullptr;
  IRWaterLut irw{};
  DevBuf sfc;               // emissivity model: e, de/dv, de/dT [P][L]
  bool model_call = false;  // the last call used the emissivity model
  int* d_error = nullptr;   // first failure code of the scattering kernel
  cudaStream_t copy_stream = nullptr;   // device-to-host copies of finished chunks
  std::vector<cudaEvent_t> chunk_events;
  // Calls on a handle share its workspace and buffers, whatever stream each
  // call uses: every call waits for this event, recorded at the end of the
  // previous call's work on that call's stream.
  cudaEvent_t order_event = nullptr;
  bool order_pending = false;
  // stage profiling
  bool profiling = false;
  struct Pending { int stage; cudaEvent_t a, b; };
  std::vector<Pending> pending;
  std::vector<cudaEvent_t> event_pool;
  static constexpr int N_STAGES = 10;
  double stage_ms[N_STAGES] = {0};
  long long stage_n[N_STAGES] = {0};
};

namespace {

int fail(crtm_gpu_handle h, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (h) h->error = buf; else g_init_error = buf;
  return CRTM_GPU_FAILURE;
}

#define CK_LAUNCH(h)                                                                    \
  do {                                                                                  \
    (h)->launches++;                                                                    \
    cudaError_t _e = cudaGetLastError();                                                \
    if (_e != cudaSuccess) return fail(h, "kernel launch failed: %s", cudaGetErrorString(_e)); \
  } while (0)

cudaEvent_t take_event(crtm_gpu_handle h) {
  if (!h->event_pool.empty()) {
    cudaEvent_t e = h->event_pool.back();
    h->event_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

// Brackets one kernel launch with events when profiling is enabled.
struct StageScope {
  crtm_gpu_handle h;
  int stage;
  cudaStream_t st;
  cudaEvent_t a = nullptr;
  StageScope(crtm_gpu_handle h_, int s_, cudaStream_t st_) : h(h_), stage(s_), st(st_) {
    if (h->profiling) { a = take_event(h); cudaEventRecord(a, st); }
  }
  ~StageScope() {
    if (a) {
      cudaEvent_t b = take_event(h);
      cudaEventRecord(b, st);
      h->pending.push_back({stage, a, b});
    }
  }
};

void collect_stage_times(crtm_gpu_handle h) {
  for (auto& p : h->pending) {
    float ms = 0.0f;
    if (cudaEventSynchronize(p.b) == cudaSuccess && cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
      h->stage_ms[p.stage] += ms;
      h->stage_n[p.stage] += 1;
    }
    h->event_pool.push_back(p.a);
    h->event_pool.push_back(p.b);
  }
  h->pending.clear();
}

size_t align_up(size_t x) { return (x + 255) & ~(size_t)255; }

// Workspace carving for one chunk
template <class R>
struct Work {
  PrepView<R> pv;
  R* OD;            // [n][K][L]
  R* TAU, *DTOP;    // [n][Kmax][L]
  R* PT;            // [n][Kmax][L]
  R* SC;            // [n][L]
  double* TSK;      // adjoint: [n][L]
  R* RA;            // [n][nv][K][L]
  R* LB;            // cloudy forward: [n][Kmax][NE][L] layer records
  R* LBK;           // scattering K-matrix/adjoint: [n][Kmax][NE][L] layer records
  double* FB;       // SOI: [n][2][2][Kmax+1][NZ][L] fields (forward), adjoint fields (K-matrix/adjoint)
  double* FS;       // SOI K-matrix/adjoint: [n][slots][2][Kmax+1][NZ][L] order fields
  double* maxreff;  // scattering: [n]
  double* cover;    // scattering: [n] total cloud cover
  R* AS;            // scattering K-matrix/adjoint: [n][Kmax+1][NZ*NZ+NZ][L] adding states
  R* TODc;          // scattering K-matrix/adjoint: [n][Kmax][L] cloudy dR/dtau
  double* CB;       // scattering K-matrix/adjoint: [n][4][L] cloudy radiance, surface terms, clear radiance
  R* LBA;           // scattering K-matrix/adjoint: [n][Kmax][NE][L] layer record adjoints
  double* CJ, *CR;  // species Jacobians: [n][slots][Kmax][L]
  double* CF;       // cloud-fraction Jacobian: [n][Kmax][L]
  double* CV;       // aerosol effective-variance Jacobians ('CMAQ'): [n][slots][Kmax][L]
  double* CH;       // relative-humidity Jacobian ('GOCART-GEOS5', 'NAAPS'): [n][Kmax][L]
  double* WS;       // adjoint with the emissivity model: [n][L] wind-speed adjoints
  double* TD;       // cloud-cover derivatives: [n][2][Kmax]
  double* ras;      // adjoint: [n][nv][K]
  double* pts;      // adjoint: [n][Kmax]
  double* tss;      // adjoint: [n]
  int* idx_map;     // [Jm]
};

template <int G, class R> struct Tune;
template <> struct Tune<1, double> { static constexpr int FWD = 4, AD = 2; };
template <> struct Tune<1, float> { static constexpr int FWD = 8, AD = 4; };
template <> struct Tune<2, double> { static constexpr int FWD = 4, AD = 2; };
template <> struct Tune<2, float> { static constexpr int FWD = 8, AD = 4; };
template <> struct Tune<3, double> { static constexpr int FWD = 4, AD = 4; };
template <> struct Tune<3, float> { static constexpr int FWD = 8, AD = 8; };
// profiles per absorb_ad CTA
template <int G, class R> constexpr int ad_profiles() { return Tune<G, R>::AD * AD_WARPS; }

// Scattering part of a chunk's workspace: layer record length (0: none),
// angles of the kernels, SOI fields, adding states of the K-matrix.
struct ScatterWork {
  int rec = 0, nz = 0;
  bool soi = false, kstate = false;
  int soi_slots = 0;     // SOI order-field slots of the K-matrix/adjoint
  int slots = 0;         // species Jacobian slots (max_clouds + max_aerosols), 0: none
  bool cf = false;       // cloud-fraction Jacobian
  bool cv = false, ch = false;   // aerosol effective-variance / relative-humidity Jacobians
  bool wind = false;     // adjoint through the emissivity model: per-(profile, channel) wind-speed adjoints
};

template <int G, class R>
size_t work_bytes(const Sensor& s, int n, int Kmax, int nv, int mode, Work<R>* w, char* base,
                  const ScatterWork& sw = ScatterWork()) {
  const int K = s.K, L = s.L, NS = s.NS, NX = DLayout<G>::NX;
  const int npf = Tune<G, R>::FWD, npa = Tune<G, R>::AD;
  size_t off = 0;
  auto carve = [&](size_t bytes) -> char* { char* p = base ? base + off : nullptr; off += align_up(bytes); return p; };
  const size_t nn = (size_t)n;
  const size_t ngf = ((nn + npf * FWD_WARPS - 1) / (npf * FWD_WARPS)) * FWD_WARPS;
  const size_t nga = ((nn + ad_profiles<G, R>() - 1) / ad_profiles<G, R>()) * AD_WARPS;
  PrepView<R> pv;
  pv.Xg = (R*)carve(ngf * npf * K * NS * sizeof(R));
  const bool adj = mode == 1 || mode == 2;
  pv.Dg = adj ? (R*)carve(nga * npa * K * NX * sizeof(R)) : nullptr;
  pv.band_i0 = (int*)carve(nn * K * sizeof(int));
  pv.band_n = (int*)carve(nn * K * sizeof(int));
  pv.band_w = (double*)carve(nn * K * MAX_BAND * sizeof(double));
  pv.ulev_k1 = (int*)carve(nn * (Kmax + 1) * sizeof(int));
  pv.ulev_k2 = (int*)carve(nn * (Kmax + 1) * sizeof(int));
  pv.ulev_fac = (double*)carve(nn * (Kmax + 1) * sizeof(double));
  pv.rlev_ilo = (int*)carve(nn * (K + 1) * sizeof(int));
  pv.rlev_ihi = (int*)carve(nn * (K + 1) * sizeof(int));
  pv.ub_k0 = (int*)carve(nn * Kmax * sizeof(int));
  pv.ub_n = (int*)carve(nn * Kmax * sizeof(int));
  pv.ub_w = (double*)carve(nn * Kmax * MAX_UBAND * sizeof(double));
  pv.scal = (double*)carve(nn * 4 * sizeof(double));
  pv.status = (int*)carve(nn * sizeof(int));
  pv.opt = s.ov.n > 0 ? (double*)carve(nn * K * OPT_NS * sizeof(double)) : nullptr;
  pv.K = K; pv.Kmax = Kmax; pv.npf = npf; pv.npa = adj ? npa : 0;
  Work<R> wk{};
  wk.pv = pv;
  wk.OD = (R*)carve(nn * K * L * sizeof(R));
  if (mode == 3) wk.TAU = (R*)carve(nn * Kmax * L * sizeof(R));
  if (sw.rec > 0) {
    if (sw.kstate)
      wk.LBK = (R*)carve(nn * Kmax * (size_t)sw.rec * L * sizeof(R));
    else
      wk.LB = (R*)carve(nn * Kmax * (size_t)sw.rec * L * sizeof(R));
    wk.maxreff = (double*)carve(nn * sizeof(double));
    wk.cover = (double*)carve(nn * sizeof(double));
    // SOI fields: 2 fields x 2 buffers x levels x angles
    wk.FB = sw.soi ? (double*)carve(nn * 4 * (size_t)(Kmax + 1) * sw.nz * L * sizeof(double)) : nullptr;
    wk.FS = sw.soi && sw.kstate
                ? (double*)carve(nn * (size_t)sw.soi_slots * 2 * (Kmax + 1) * sw.nz * L * sizeof(double))
                : nullptr;
    wk.AS = sw.kstate ? (R*)carve(nn * (size_t)(Kmax + 1) * (sw.nz * sw.nz + sw.nz) * L * sizeof(R))
                      : nullptr;
    wk.TODc = sw.kstate ? (R*)carve(nn * Kmax * L * sizeof(R)) : nullptr;
    wk.CB = sw.kstate ? (double*)carve(nn * 4 * L * sizeof(double)) : nullptr;
    wk.LBA = sw.kstate ? (R*)carve(nn * Kmax * (size_t)sw.rec * L * sizeof(R)) : nullptr;
    const size_t sj = nn * (size_t)sw.slots * Kmax * L * sizeof(double);
    wk.CJ = sw.slots ? (double*)carve(sj) : nullptr;
    wk.CR = sw.slots ? (double*)carve(sj) : nullptr;
    wk.CF = sw.cf ? (double*)carve(nn * Kmax * L * sizeof(double)) : nullptr;
    wk.CV = sw.cv ? (double*)carve(sj) : nullptr;
    wk.CH = sw.ch ? (double*)carve(nn * Kmax * L * sizeof(double)) : nullptr;
    wk.TD = sw.kstate && (sw.slots || sw.cf) ? (double*)carve(nn * 2 * Kmax * sizeof(double)) : nullptr;
  }
  if (adj) {
    wk.TAU = (R*)carve(nn * Kmax * L * sizeof(R));
    wk.DTOP = (R*)carve(nn * Kmax * L * sizeof(R));
    wk.PT = (R*)carve(nn * Kmax * L * sizeof(R));
    wk.SC = (R*)carve(nn * L * sizeof(R));
    wk.RA = (R*)carve(nn * nv * K * L * sizeof(R));
  }
  if (mode == 2 && sw.wind) wk.WS = (double*)carve(nn * L * sizeof(double));
  if (mode == 2) {
    wk.TSK = (double*)carve(nn * L * sizeof(double));
    wk.ras = (double*)carve(nn * nv * K * sizeof(double));
    wk.pts = (double*)carve(nn * Kmax * sizeof(double));
    wk.tss = (double*)carve(nn * sizeof(double));
  }
  wk.idx_map = (int*)carve(MAX_ABS * sizeof(int));
  if (w) *w = wk;
  return off;
}

BatchView make_view(const crtm_gpu_batch* b) {
  BatchView v;
  v.n_profiles = b->n_profiles; v.max_layers = b->max_layers; v.n_abs = b->n_absorbers;
  v.n_layers = b->n_layers; v.level_pressure = b->level_pressure; v.pressure = b->pressure;
  v.temperature = b->temperature; v.absorber = b->absorber;
  v.land_cov = b->land_coverage; v.water_cov = b->water_coverage;
  v.snow_cov = b->snow_coverage; v.ice_cov = b->ice_coverage;
  v.land_t = b->land_temperature; v.water_t = b->water_temperature;
  v.snow_t = b->snow_temperature; v.ice_t = b->ice_temperature;
  v.zenith = b->sensor_zenith_angle; v.altitude = b->surface_altitude;
  v.emissivity = b->emissivity;
  return v;
}

template <class F>
int reserve_smem(crtm_gpu_handle h, F kernel, size_t bytes, const char* what) {
  if (bytes > 48 * 1024 &&
      cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) != cudaSuccess)
    return fail(h, "cannot reserve %zu bytes of shared memory for the %s kernel", bytes, what);
  return CRTM_GPU_SUCCESS;
}

// Per-profile output slabs copied to host buffers as each chunk finishes
// (host entry points only): element i covers bytes [p*per[i], (p+n)*per[i]).
struct HostCopy {
  int n = 0;
  void* dst[40];
  const void* src[40];
  size_t per[40];
  int max_chunk = 0;   // cap on the chunk size so that copies overlap compute
};

// The further RTSolution components of an output set, in a fixed order:
// their pointers and byte sizes (P x L pairs, Km layers).
constexpr int N_RTS_EXT = 12;
void rts_ext_list(const crtm_gpu_rtsolution* r, size_t PL, size_t Km, void** ptr, size_t* bytes) {
  void* const p[N_RTS_EXT] = {r->tb_clear, r->r_clear, r->total_cloud_cover, r->sod, r->surface_emissivity,
                              r->up_radiance, r->down_radiance, r->surface_planck_radiance, r->n_full_streams,
                              r->layer_optical_depth, r->upwelling_radiance, r->upwelling_overcast_radiance};
  for (int i = 0; i < N_RTS_EXT; i++) {
    ptr[i] = p[i];
    bytes[i] = !p[i] ? 0 : i == 8 ? PL * sizeof(int) : i >= 9 ? PL * Km * sizeof(double) : PL * sizeof(double);
  }
}
void rts_ext_set(crtm_gpu_rtsolution* r, void* const* p) {
  r->tb_clear = (double*)p[0]; r->r_clear = (double*)p[1]; r->total_cloud_cover = (double*)p[2];
  r->sod = (double*)p[3]; r->surface_emissivity = (double*)p[4]; r->up_radiance = (double*)p[5];
  r->down_radiance = (double*)p[6]; r->surface_planck_radiance = (double*)p[7]; r->n_full_streams = (int*)p[8];
  r->layer_optical_depth = (double*)p[9]; r->upwelling_radiance = (double*)p[10];
  r->upwelling_overcast_radiance = (double*)p[11];
}
// Whether a call asks for any of the further RTSolution components.
bool rts_ext_any(const RtsExt& x) {
  return x.tb_clear || x.r_clear || x.tcc || x.sod || x.emis || x.up || x.down || x.bs || x.nfs || x.lod || x.upw ||
         x.ovc;
}

RtsExt make_ext(const crtm_gpu_rtsolution* r) {
  RtsExt x;
  x.tb_clear = r->tb_clear; x.r_clear = r->r_clear; x.tcc = r->total_cloud_cover; x.sod = r->sod;
  x.emis = r->surface_emissivity; x.up = r->up_radiance; x.down = r->down_radiance;
  x.bs = r->surface_planck_radiance; x.nfs = r->n_full_streams; x.lod = r->layer_optical_depth;
  x.upw = r->upwelling_radiance; x.ovc = r->upwelling_overcast_radiance;
  return x;
}

// Caller-owned scratch of fixed size used instead of the handle's workspace
// (crtm_gpu_k_matrix_device_static).
struct FixedScratch {
  char* base;
  size_t bytes;
};

// IR sea-surface emissivity model of a call (batch emissivity NULL):
// de/d(wind speed) and de/d(water temperature) [P][L] (the latter null unless
// the table is 'Nalli2').
struct SfcModel {
  const double* ev = nullptr;
  const double* et = nullptr;
};

// CRTM_Compute_IR_Water_SfcOptics (CRTM_IR_Water_SfcOptics.f90:179-254) for
// the Emission solver: the emissivity at the sensor zenith angle (the one
// angle of a clear-sky column; specular, reflectivity 1 - e) and its wind
// speed / water temperature derivatives, one thread per (profile, channel).
// Profiles whose water coverage is not 1 raise error 13 (the land, snow and
// ice models are not built).
__global__ void irwater_kernel(IRWaterLut W, int P, int L, const double* wn, const double* zenith,
                               const double* t_water, const double* water_cov, const double* wind, double* E,
                               double* EV, double* ET, int* error) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)P * L) return;
  const int p = (int)(i / L), l = (int)(i % L);
  if (fabs(water_cov[p] - 1.0) > 1.0e-12) atomicCAS(error, 0, 13);
  Dual<2> t(t_water[p]), v(wind ? wind[p] : 5.0);   // DEFAULT_WIND_SPEED
  v.d[0] = 1.0;
  t.d[1] = 1.0;
  const Dual<2> e = irssem<Dual<2>>(W, t, v, wn[l], zenith[p]);
  E[i] = e.v;
  EV[i] = e.d[0];
  ET[i] = e.d[1];
}

int copy_chunk(crtm_gpu_handle h, const HostCopy* hc, int p0, int n, cudaStream_t st) {
  if (!h->copy_stream && cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking) != cudaSuccess)
    return fail(h, "cannot create the copy stream");
  cudaEvent_t ev = nullptr;
  if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess)
    return fail(h, "cannot create a chunk event");
  h->chunk_events.push_back(ev);
  if (cudaEventRecord(ev, st) != cudaSuccess || cudaStreamWaitEvent(h->copy_stream, ev, 0) != cudaSuccess)
    return fail(h, "chunk event failed");
  for (int i = 0; i < hc->n; i++) {
    if (!hc->dst[i] || !hc->per[i]) continue;
    if (cudaMemcpyAsync((char*)hc->dst[i] + (size_t)p0 * hc->per[i],
                        (const char*)hc->src[i] + (size_t)p0 * hc->per[i], (size_t)n * hc->per[i],
                        cudaMemcpyDeviceToHost, h->copy_stream) != cudaSuccess)
      return fail(h, "device-to-host copy failed");
  }
  return CRTM_GPU_SUCCESS;
}

// mode 0 forward, 1 K-matrix, 2 adjoint
// perm: device array of the batch profiles the pipeline runs, in order
// (b->n_profiles of them), or null for all of the batch's profiles in its
// own order.  nz_max: scattering kernels for up to 16 streams (else the
// stream rule's, up to 6).
template <int G, class R>
int run_pipeline(crtm_gpu_handle h, const Sensor& s, const crtm_gpu_batch* b, int mode,
                 const double* seed, crtm_gpu_rtsolution* rts, crtm_gpu_kmatrix* kk,
                 crtm_gpu_adjoint_out* ad, cudaStream_t st, const HostCopy* hc,
                 const FixedScratch* fixed, bool scat, const SfcModel* sm, const int* perm, bool nz_max) {
  const int P = b->n_profiles, Kmax = b->max_layers, L = s.L, K = s.K, n_abs = b->n_absorbers;
  if (P <= 0) return CRTM_GPU_SUCCESS;
  if (Kmax < 2 || Kmax > MAX_LAYERS) return fail(h, "max_layers %d out of range [2, %d]", Kmax, MAX_LAYERS);
  if (n_abs < 0 || n_abs > MAX_OUT_ABS || (n_abs > 0 && !b->absorber_id))
    return fail(h, "absorber count %d out of range [0, %d] or ids missing", n_abs, MAX_OUT_ABS);
  // absorber maps (host): ODPS absorber -> first user absorber with the same id
  int idx_map[MAX_ABS];
  std::vector<int> abs_of_user(n_abs > 0 ? n_abs : 1, -1);
  for (int j = 0; j < s.Jm; j++) {
    idx_map[j] = -1;
    for (int jj = 0; jj < n_abs; jj++)
      if (b->absorber_id[jj] == s.absorber_id[j]) { idx_map[j] = jj; break; }
    if (idx_map[j] >= 0) abs_of_user[idx_map[j]] = j;
  }
  // requested absorber adjoints: K-matrix selection (default all) or, for the adjoint, all
  OutAbs oa{};
  if (mode == 1 && kk->n_k_absorbers > 0) {
    if (kk->n_k_absorbers > n_abs || !kk->k_absorber_index) return fail(h, "bad K-matrix absorber selection");
    oa.n = kk->n_k_absorbers;
    for (int j = 0; j < oa.n; j++) {
      const int ja = kk->k_absorber_index[j];
      if (ja < 0 || ja >= n_abs) return fail(h, "K-matrix absorber index %d out of range", ja);
      oa.odps[j] = abs_of_user[ja];
    }
  } else {
    oa.n = n_abs;
    for (int j = 0; j < n_abs; j++) oa.odps[j] = abs_of_user[j];
  }
  const int nv = 1 + oa.n;
  const bool soi = scat && b->rt_algorithm_id != nullptr;
  // scattering Jacobian outputs that the caller asked for
  double* o_wc = nullptr, *o_re = nullptr, *o_cf = nullptr, *o_ac = nullptr, *o_ar = nullptr;
  double* o_av = nullptr, *o_rh = nullptr;
  if (mode == 1) {
    o_wc = kk->cloud_water_content; o_re = kk->cloud_effective_radius; o_cf = kk->cloud_fraction;
    o_ac = kk->aerosol_concentration; o_ar = kk->aerosol_effective_radius;
    o_av = kk->aerosol_effective_variance; o_rh = kk->relative_humidity;
  } else if (mode == 2) {
    o_wc = ad->cloud_water_content; o_re = ad->cloud_effective_radius; o_cf = ad->cloud_fraction;
    o_ac = ad->aerosol_concentration; o_ar = ad->aerosol_effective_radius;
    o_av = ad->aerosol_effective_variance; o_rh = ad->relative_humidity;
  }
  const int NCb = b->max_clouds > 0 ? b->max_clouds : 0, NAb = b->max_aerosols > 0 ? b->max_aerosols : 0;
  if (NCb == 0) o_wc = o_re = o_cf = nullptr;
  if (NAb == 0) o_ac = o_ar = o_av = o_rh = nullptr;
  // the scheme's second aerosol coordinate: effective variance ('CMAQ') or
  // relative humidity ('GOCART-GEOS5', 'NAAPS'); the other output stays zero
  const int ascheme = h->has_aerosols ? h->alut.scheme : AEROSOL_CRTM;
  const bool want_av = o_av && ascheme == AEROSOL_CMAQ, want_rh = o_rh && ascheme >= AEROSOL_GOCART;
  ScatterWork sw;
  if (scat) {
    sw.nz = nz_max ? SC_NZ_MAX : 5;
    sw.soi = soi;
    sw.kstate = mode != 3;
    sw.soi_slots = soi && sw.kstate ? h->soi_slots : 0;
    sw.rec = nz_max ? layer_record<SC_NZ_MAX>() : layer_record<5>();
    if (sw.kstate && (o_wc || o_re || o_cf || o_ac || o_ar || o_av || o_rh)) sw.slots = NCb + NAb;
    sw.cf = sw.kstate && o_cf != nullptr;
    sw.cv = sw.kstate && want_av;
    sw.ch = sw.kstate && want_rh;
  }
  sw.wind = mode == 2 && sm && sm->ev && ad->wind_speed;
  // chunk size from the workspace budget
  const size_t per = work_bytes<G, R>(s, 64, Kmax, nv, mode, nullptr, nullptr, sw) / 64 + 1;
  int chunk = (int)std::max<size_t>(1, std::min<size_t>((size_t)P, h->workspace_budget / per));
  if (hc && hc->max_chunk > 0) chunk = std::min(chunk, hc->max_chunk);
  constexpr int form = sizeof(R) == sizeof(float) ? 1 : 0;
  if (!fixed && s.tune_chunk[form] > 0) chunk = std::min(chunk, s.tune_chunk[form]);
  char* ws_base;
  if (fixed) {
    // largest chunk whose workspace fits the fixed scratch
    chunk = (int)std::min<size_t>((size_t)chunk, fixed->bytes / per);
    while (chunk > 1 && work_bytes<G, R>(s, chunk, Kmax, nv, mode, nullptr, nullptr, sw) > fixed->bytes) chunk--;
    const size_t one = work_bytes<G, R>(s, 1, Kmax, nv, mode, nullptr, nullptr, sw);
    if (chunk < 1 || one > fixed->bytes)
      return fail(h, "one profile of this call needs %zu bytes of scratch (%d channels, max_layers %d, "
                     "%d absorber Jacobians); the static scratch holds %zu bytes",
                  one, L, Kmax, nv - 1, fixed->bytes);
    ws_base = fixed->base;
  } else {
    const size_t need = work_bytes<G, R>(s, chunk, Kmax, nv, mode, nullptr, nullptr, sw);
    if (!h->ws.ensure(need)) return fail(h, "cannot allocate %zu bytes of workspace", need);
    ws_base = (char*)h->ws.p;
  }
  Work<R> w;
  work_bytes<G, R>(s, chunk, Kmax, nv, mode, &w, ws_base, sw);
  if (cudaMemcpyAsync(w.idx_map, idx_map, sizeof(int) * s.Jm, cudaMemcpyHostToDevice, st) != cudaSuccess)
    return fail(h, "absorber map upload failed");
  BatchView bv = make_view(b);
  bv.perm = perm;
  constexpr int NPF = Tune<G, R>::FWD, NPA = Tune<G, R>::AD;
  const size_t prep_smem = prep_smem_bytes<G>(K);
  const size_t col_smem = column_smem_bytes<R>(K, Kmax);
  // channels per map CTA: 16 (more resident CTAs hide the tile loads; C2:
  // 6.4 ms against 7.4 ms with 32 and 8.1 ms with 8), fewer if the tiles exceed
  // the shared-memory budget (CRTM_GPU_MAP_CHANNELS: 8, 16 or 32 overrides;
  // a sensor's tuning overrides both)
  int map_ct = s.tune_map[form] > 0 ? s.tune_map[form] : h->map_channels;
  while (map_ct > 8 && map_smem_bytes<R>(K, Kmax, nv, map_ct) > 200 * 1024) map_ct >>= 1;
  const size_t map_smem = map_smem_bytes<R>(K, Kmax, nv, map_ct);
  constexpr size_t fwd_smem = fwd_smem_bytes<G, R, NPF>();
  if (reserve_smem(h, absorb_fwd_kernel<G, R, NPF>, fwd_smem, "absorb_fwd") ||
      reserve_smem(h, column_kernel<R, false>, col_smem, "column") ||
      reserve_smem(h, column_kernel<R, true>, col_smem, "column") ||
      reserve_smem(h, map_kernel<R>, map_smem, "map"))
    return CRTM_GPU_FAILURE;
  const bool ho_only = [&] {
    for (int j = 0; j < oa.n; j++)
      if (oa.odps[j] >= 2) return false;
    return true;
  }();
  for (int p0 = 0; p0 < P; p0 += chunk) {
    const int n = std::min(chunk, P - p0);
    {
      StageScope sc(h, 0, st);
      prep_kernel<G, R><<<n, 32, prep_smem, st>>>(s.tables, s.refsums, bv, w.pv, w.idx_map, p0, n);
      CK_LAUNCH(h);
    }
    {
      StageScope sc(h, 1, st);
      dim3 gf((L + FWD_CH - 1) / FWD_CH, (n + NPF * FWD_WARPS - 1) / (NPF * FWD_WARPS));
      absorb_fwd_kernel<G, R, NPF><<<gf, 32 * FWD_WARPS, fwd_smem, st>>>(K, L, s.Lp, n, s.d_C, s.d_cmask,
                                                                   w.pv.Xg, w.OD);
      CK_LAUNCH(h);
      if (s.ov.n > 0) {   // the OPTRAN channels' water-vapour-line component
        optran_fwd_kernel<R><<<dim3((s.ov.n + 127) / 128, n), 128, 0, st>>>(K, L, n, s.ov, w.pv.opt, w.OD);
        CK_LAUNCH(h);
      }
    }
    ColumnArgs<R> ca{};
    ca.K = K; ca.L = L; ca.Kmax = Kmax; ca.p_begin = p0; ca.n_chunk = n; ca.mode = mode;
    ca.b = bv; ca.sp = s.spec; ca.pv = w.pv; ca.OD = w.OD;
    ca.TAU = w.TAU; ca.DTOP = w.DTOP; ca.PT = w.PT; ca.SC = w.SC;
    ca.seed = seed; ca.radiance = rts->radiance; ca.bt = rts->brightness_temperature;
    ca.tsk = mode == 1 ? kk->water_temperature : (mode == 2 ? w.TSK : nullptr);
    ca.ek = mode == 1 ? kk->surface_emissivity : nullptr;
    if (mode == 1) { ca.tsk_land = kk->land_temperature; ca.tsk_snow = kk->snow_temperature; ca.tsk_ice = kk->ice_temperature; }
    if (sm && sm->ev) {   // emissivity model
      ca.sfc_ev = sm->ev;
      ca.sfc_et = sm->et;
      ca.wind_k = mode == 1 ? kk->wind_speed : (mode == 2 ? w.WS : nullptr);
    }
    ca.status = rts->status;
    ca.x = make_ext(rts);
    ca.n_streams = b->n_streams;
    // scattering K-matrix/adjoint: the column runs twice around the scattering kernels
    const bool split = scat && mode != 3;
    if (split) {
      ca.pass = 1;
      ca.n_clouds = b->max_clouds > 0 ? b->n_clouds : nullptr;
      ca.n_aerosols = b->max_aerosols > 0 ? b->n_aerosols : nullptr;
      ca.TODc = w.TODc; ca.CB = w.CB; ca.cover = w.cover;
    }
    dim3 gc((L + 127) / 128, n);
    {
      StageScope sc(h, 2, st);
      if (rts_ext_any(ca.x))
        column_kernel<R, true><<<gc, 128, col_smem, st>>>(ca);
      else
        column_kernel<R, false><<<gc, 128, col_smem, st>>>(ca);
      CK_LAUNCH(h);
    }
    if (scat) {   // layer optics, then the adding from the surface (and its adjoint)
      ScatterArgs<R> sa{};
      sa.K = K; sa.L = L; sa.Kmax = Kmax; sa.p_begin = p0; sa.n_chunk = n;
      sa.microwave = s.sensor_type == 1;
      sa.b = bv; sa.sp = s.spec; sa.pv = w.pv; sa.lut = h->lut; sa.lut_chan = s.d_zc;
      sa.max_clouds = b->max_clouds; sa.n_clouds = b->n_clouds; sa.cloud_type = b->cloud_type;
      sa.wc = b->cloud_water_content; sa.reff = b->cloud_effective_radius; sa.n_streams = b->n_streams;
      sa.rt_algorithm = b->rt_algorithm_id; sa.FB = w.FB; sa.FS = w.FS; sa.soi_slots = sw.soi_slots;
      sa.alut = h->alut; sa.max_aerosols = b->max_aerosols > 0 ? b->max_aerosols : 0;
      sa.n_aerosols = b->n_aerosols; sa.aerosol_type = b->aerosol_type;
      sa.conc = b->aerosol_concentration; sa.aer_reff = b->aerosol_effective_radius;
      sa.aer_var = sa.max_aerosols > 0 ? b->aerosol_effective_variance : nullptr;
      sa.rh = sa.max_aerosols > 0 ? b->relative_humidity : nullptr;
      sa.CV = w.CV; sa.CH = w.CH;
      if (b->max_clouds <= 0) sa.max_clouds = 0;
      sa.TAU = w.TAU; sa.LB = w.LB; sa.LBK = w.LBK; sa.maxreff = w.maxreff; sa.cover = w.cover;
      sa.cloud_fraction = sa.max_clouds > 0 ? b->cloud_fraction : nullptr;
      sa.overlap = sa.max_clouds > 0 ? b->overlap_id : nullptr;
      sa.radiance = rts->radiance; sa.bt = rts->brightness_temperature;
      sa.status = rts->status; sa.error = h->d_error;
      sa.x = make_ext(rts);
      sa.TODc = w.TODc; sa.PT = w.PT; sa.CB = w.CB; sa.AS = w.AS; sa.LBA = w.LBA;
      sa.n_slots = sw.slots; sa.CJ = w.CJ; sa.CR = w.CR; sa.CF = w.CF; sa.TD = w.TD; sa.SC = w.SC;
      const long long nlay = (long long)n * Kmax * L;
      const unsigned gl = (unsigned)((nlay + SCATTER_THREADS - 1) / SCATTER_THREADS);
      dim3 ga((L + SCATTER_THREADS - 1) / SCATTER_THREADS, n);
      {
        StageScope sc(h, 6, st);
        scatter_profile_kernel<R><<<(n + 3) / 4, 128, 0, st>>>(sa);
        CK_LAUNCH(h);
        if (split) {   // K-matrix / adjoint: FP64 records, layer solver in R
          if (nz_max)
            launch_scatter_layers_k<SC_NZ_MAX, R, R>(sa, gl, st);
          else
            launch_scatter_layers_k<5, R, R>(sa, gl, st);
        } else if (soi) {   // forward with SOI profiles: FP64 layer solver (records in R)
          if (nz_max)
            scatter_layers_kernel<SC_NZ_MAX, R, R, double><<<gl, SCATTER_THREADS, 0, st>>>(sa, w.LB);
          else
            scatter_layers_kernel<5, R, R, double><<<gl, SCATTER_THREADS, 0, st>>>(sa, w.LB);
        } else {   // forward: layer solver in R (records in R)
          if (nz_max)
            scatter_layers_kernel<SC_NZ_MAX, R, R, R><<<gl, SCATTER_THREADS, 0, st>>>(sa, w.LB);
          else
            scatter_layers_kernel<5, R, R, R><<<gl, SCATTER_THREADS, 0, st>>>(sa, w.LB);
        }
        CK_LAUNCH(h);
      }
      if (split) {
        {
          StageScope sc(h, 7, st);
          if (nz_max)
            launch_scatter_kmatrix<SC_NZ_MAX, R>(sa, ga, st, soi);
          else
            launch_scatter_kmatrix<5, R>(sa, ga, st, soi);
          CK_LAUNCH(h);
        }
        {
          StageScope sc(h, 8, st);
          if (nz_max)
            launch_scatter_reverse<SC_NZ_MAX, R, R>(sa, gl, st);
          else
            launch_scatter_reverse<5, R, R>(sa, gl, st);
          CK_LAUNCH(h);
          if constexpr (std::is_same<R, double>::value) {
            if (soi) {   // the SOI profiles' layers
              if (nz_max)
                launch_scatter_contract<SC_NZ_MAX, double>(sa, gl, st);
              else
                launch_scatter_contract<5, double>(sa, gl, st);
              CK_LAUNCH(h);
            }
          } else if (soi) {
            return fail(h, "internal: SOI K-matrix in the mixed form");
          }
        }
        {
          ca.pass = 2;
          StageScope sc(h, 2, st);
          if (rts_ext_any(ca.x))
        column_kernel<R, true><<<gc, 128, col_smem, st>>>(ca);
      else
        column_kernel<R, false><<<gc, 128, col_smem, st>>>(ca);
          CK_LAUNCH(h);
        }
        if (sw.slots || sw.cf) {   // species and cloud-fraction Jacobians: cover chain rule, seed, outputs
          StageScope sc(h, 9, st);
          scatter_species_kernel<R><<<ga, SCATTER_THREADS, 0, st>>>(sa);
          CK_LAUNCH(h);
          struct Out { double* o; const double* X; int S, s0, ns; };
          const Out outs[7] = {{o_wc, w.CJ, sw.slots, 0, NCb}, {o_re, w.CR, sw.slots, 0, NCb},
                               {o_ac, w.CJ, sw.slots, NCb, NAb}, {o_ar, w.CR, sw.slots, NCb, NAb},
                               {o_cf, w.CF, 1, 0, 1}, {o_av, w.CV, sw.slots, NCb, NAb},
                               {o_rh, w.CH, 1, 0, 1}};
          for (const Out& o : outs) {
            if (!o.o || !o.X || o.ns == 0) continue;
            if (mode == 1) {
              dim3 gt((L + 31) / 32, (Kmax + 31) / 32, std::min(n * o.ns, 65535));
              species_k_out_kernel<<<gt, dim3(32, 8), 0, st>>>(o.X, o.S, o.s0, o.ns, Kmax, L, p0, n, o.o,
                                                               perm);
            } else {
              const long long rows = (long long)n * o.ns * Kmax;
              species_ad_out_kernel<<<(unsigned)((rows + 7) / 8), 256, 0, st>>>(o.X, o.S, o.s0, o.ns, Kmax, L,
                                                                              p0, n, o.o, perm);
            }
            CK_LAUNCH(h);
          }
        }
        // outputs of a coordinate that the handle's aerosol scheme does not have: zero
        const size_t rows_k = mode == 1 ? (size_t)L * Kmax : (size_t)Kmax;
        const auto clear_rows = [&](double* o, size_t row) {
          if (perm) {
            const size_t nel = (size_t)n * row;
            zero_profile_rows_kernel<<<(unsigned)((nel + 255) / 256), 256, 0, st>>>(o, perm + p0, n, row);
            return cudaGetLastError() == cudaSuccess;
          }
          return cudaMemsetAsync(o + (size_t)p0 * row, 0, (size_t)n * row * sizeof(double), st) == cudaSuccess;
        };
        if (o_av && !sw.cv && !clear_rows(o_av, NAb * rows_k)) return fail(h, "output clear failed");
        if (o_rh && !sw.ch && !clear_rows(o_rh, rows_k)) return fail(h, "output clear failed");
      } else {
        StageScope sc(h, 7, st);
        if (nz_max)
          scatter_adding_kernel<SC_NZ_MAX, R><<<ga, SCATTER_THREADS, 0, st>>>(sa);
        else
          scatter_adding_kernel<5, R><<<ga, SCATTER_THREADS, 0, st>>>(sa);
        CK_LAUNCH(h);
        if (soi) {
          if (nz_max)
            scatter_soi_kernel<SC_NZ_MAX, R><<<ga, SCATTER_THREADS, 0, st>>>(sa);
          else
            scatter_soi_kernel<5, R><<<ga, SCATTER_THREADS, 0, st>>>(sa);
          CK_LAUNCH(h);
        }
      }
    }
    if (mode == 0 || mode == 3) {
      if (hc && hc->n) {
        if (int rc = copy_chunk(h, hc, p0, n, st)) return rc;
      }
      continue;
    }
    {
      StageScope sc(h, 3, st);
      dim3 ga((L + 31) / 32, (n + ad_profiles<G, R>() - 1) / ad_profiles<G, R>());
      if (ho_only)
        absorb_ad_kernel<G, R, NPA, 1><<<ga, 32 * AD_WARPS, 0, st>>>(
            K, L, s.Lp, n, s.d_C, s.d_cmask, w.pv.Dg, s.tables.pdp, w.OD, w.SC, oa, w.RA);
      else
        absorb_ad_kernel<G, R, NPA, 0><<<ga, 32 * AD_WARPS, 0, st>>>(
            K, L, s.Lp, n, s.d_C, s.d_cmask, w.pv.Dg, s.tables.pdp, w.OD, w.SC, oa, w.RA);
      CK_LAUNCH(h);
      if (s.ov.n > 0) {   // the OPTRAN terms' temperature and water vapour adjoints
        int h2o_out = -1;
        for (int j = 0; j < oa.n; j++)
          if (oa.odps[j] == s.h2o_idx) h2o_out = j;
        optran_ad_kernel<R><<<dim3((s.ov.n + 127) / 128, n), 128, 0, st>>>(
            K, L, n, nv, h2o_out, s.h2o_idx, s.ov, w.pv.opt, s.tables.ref_lev, w.OD, w.SC, w.RA);
        CK_LAUNCH(h);
      }
    }
    if (mode == 1) {
      MapArgs<R> ma{};
      ma.K = K; ma.L = L; ma.Kmax = Kmax; ma.p_begin = p0; ma.n_chunk = n; ma.nv = nv; ma.ct = map_ct;
      ma.b = bv; ma.pv = w.pv; ma.RA = w.RA; ma.PT = w.PT; ma.SC = w.SC;
      ma.kt = kk->temperature; ma.ka = kk->absorber;
      StageScope sc(h, 4, st);
      dim3 gm((L + map_ct - 1) / map_ct, n);
      map_kernel<R><<<gm, 256, map_smem, st>>>(ma);
      CK_LAUNCH(h);
    } else {
      StageScope sc(h, 5, st);
      const long long rows_ra = (long long)n * nv * K;
      channel_sum_kernel<R><<<(unsigned)((rows_ra * 32 + 255) / 256), 256, 0, st>>>(
          w.RA, nullptr, 1, rows_ra, L, w.ras);
      CK_LAUNCH(h);
      const long long rows_pt = (long long)n * Kmax;
      channel_sum_kernel<R><<<(unsigned)((rows_pt * 32 + 255) / 256), 256, 0, st>>>(
          w.PT, w.SC, Kmax, rows_pt, L, w.pts);
      CK_LAUNCH(h);
      channel_sum_kernel<double><<<(unsigned)(((long long)n * 32 + 255) / 256), 256, 0, st>>>(
          w.TSK, nullptr, 1, n, L, w.tss);
      CK_LAUNCH(h);
      if (w.WS) {   // Surface_AD%Wind_Speed through the emissivity model
        channel_sum_kernel<double><<<(unsigned)(((long long)n * 32 + 255) / 256), 256, 0, st>>>(
            w.WS, nullptr, 1, n, L, ad->wind_speed + p0);
        CK_LAUNCH(h);
      }
      AdjMapArgs<R> am{};
      am.K = K; am.Kmax = Kmax; am.nv = nv; am.p_begin = p0; am.n_chunk = n;
      am.b = bv; am.pv = w.pv; am.ras = w.ras; am.pts = w.pts; am.tss = w.tss;
      am.t_ad = ad->temperature; am.a_ad = ad->absorber; am.ts_ad = ad->water_temperature;
      am.ts_land = ad->land_temperature; am.ts_snow = ad->snow_temperature; am.ts_ice = ad->ice_temperature;
      const long long na = (long long)n * Kmax;
      adjoint_map_kernel<R><<<(unsigned)((na + 255) / 256), 256, 0, st>>>(am);
      CK_LAUNCH(h);
    }
    if (hc && hc->n) {
      if (int rc = copy_chunk(h, hc, p0, n, st)) return rc;
    }
  }
  return CRTM_GPU_SUCCESS;
}

// Order this call's work on st after the previous call's, and mark the end
// of this call's work (see order_event).
void order_after_previous(crtm_gpu_handle h, cudaStream_t st) {
  if (h->order_pending && h->order_event) cudaStreamWaitEvent(st, h->order_event, 0);
}
void mark_done(crtm_gpu_handle h, cudaStream_t st) {
  if (h->order_event && cudaEventRecord(h->order_event, st) == cudaSuccess) h->order_pending = true;
}

int dispatch(crtm_gpu_handle h, int sensor, const crtm_gpu_batch* b, int mode, const double* seed,
             crtm_gpu_rtsolution* rts, crtm_gpu_kmatrix* kk, crtm_gpu_adjoint_out* ad,
             cudaStream_t st, const HostCopy* hc = nullptr, const FixedScratch* fixed = nullptr) {
  if (!h) return CRTM_GPU_FAILURE;
  if (sensor < 0 || sensor >= (int)h->sensors.size()) return fail(h, "sensor index %d out of range", sensor);
  if (h->sensors[sensor].L == 0) return CRTM_GPU_SUCCESS;   // an empty channel subset: nothing to compute
  if (!b || !rts || !rts->radiance || !rts->brightness_temperature) return fail(h, "missing batch or RTSolution buffers");
  if (!b->n_layers || !b->level_pressure || !b->pressure || !b->temperature ||
      !b->land_coverage || !b->water_coverage || !b->snow_coverage || !b->ice_coverage ||
      !b->land_temperature || !b->water_temperature || !b->snow_temperature ||
      !b->ice_temperature || !b->sensor_zenith_angle || (b->n_absorbers > 0 && !b->absorber))
    return fail(h, "missing batch input arrays");
  if (mode == 1 && (!kk || !kk->temperature || !kk->absorber || !kk->water_temperature || !kk->surface_emissivity))
    return fail(h, "missing K-matrix output buffers");
  if (mode == 2 && (!ad || !ad->temperature || !ad->absorber || !ad->water_temperature))
    return fail(h, "missing adjoint output buffers");
  if (cudaSetDevice(h->device) != cudaSuccess) return fail(h, "cudaSetDevice failed");
  const Sensor& s = h->sensors[sensor];
  const bool scat = b->max_clouds > 0 || b->max_aerosols > 0;
  // The mixed form runs the gas optics and the scattering layer solver in
  // FP32 and the adding in FP64.  The K-matrix and adjoint of a batch with
  // SOI profiles (Options%RT_Algorithm_Id given) run in the FP64 form: the SOI
  // layers' doubling and its derivative-number contraction are FP64 only.
  const bool fp64 = h->precision == CRTM_GPU_FP64 ||
                    (scat && (mode == 1 || mode == 2) && b->rt_algorithm_id != nullptr);
  if (scat) {
    if (b->max_clouds > SC_NC_MAX || b->max_aerosols > SC_NC_MAX)
      return fail(h, "at most %d clouds and %d aerosols per profile", SC_NC_MAX, SC_NC_MAX);
    if (b->max_layers > SC_KMAX) return fail(h, "at most %d layers in a batch with clouds or aerosols", SC_KMAX);
    if (b->max_clouds > 0 && !h->has_clouds) return fail(h, "batch has clouds but no CloudCoeff.bin was loaded at init");
    if (b->max_aerosols > 0 && !h->has_aerosols && s.sensor_type != 1)
      return fail(h, "batch has aerosols but no AerosolCoeff.bin was loaded at init");
    if (b->max_clouds > 0 && (!b->n_clouds || !b->cloud_type || !b->cloud_water_content || !b->cloud_effective_radius))
      return fail(h, "cloud arrays missing for max_clouds = %d", b->max_clouds);
    if (b->max_aerosols > 0 && (!b->n_aerosols || !b->aerosol_type || !b->aerosol_concentration ||
                                !b->aerosol_effective_radius))
      return fail(h, "aerosol arrays missing for max_aerosols = %d", b->max_aerosols);
    if (cudaMemsetAsync(h->d_error, 0, sizeof(int), st) != cudaSuccess) return fail(h, "error flag reset failed");
    if (mode == 0) mode = 3;
  }
  // no emissivity given: the IR sea-surface emissivity model (clear sky, water)
  const bool model = b->emissivity == nullptr;
  h->model_call = model;
  if (model) {
    if (!h->has_irwater)
      return fail(h, "no emissivity given and no Nalli.IRwater.EmisCoeff.bin was loaded at init");
    if (s.sensor_type != 2)
      return fail(h, "no emissivity given: the surface emissivity model is built for infrared sensors (IR water)");
    if (scat)
      return fail(h, "no emissivity given: the IR water emissivity model is built for clear-sky batches; "
                     "supply Options%%Emissivity for batches with clouds or aerosols");
  }
  crtm_gpu_batch bm;
  SfcModel sm{};
  FixedScratch fixed_rest{};
  double* E = nullptr;
  if (model) {
    const size_t PL = (size_t)b->n_profiles * s.L, eb = 3 * PL * sizeof(double);
    if (fixed) {
      // a call that may not allocate takes the model's e, de/dv and de/dT
      // from the front of its fixed scratch and runs the pipeline on the rest
      const size_t take = (eb + 255) & ~(size_t)255;
      if (take >= fixed->bytes)
        return fail(h, "the emissivity model's %zu bytes (%d profiles x %d channels) do not fit the static "
                       "scratch of %zu bytes: pass an emissivity or fewer profiles per call",
                    eb, b->n_profiles, s.L, fixed->bytes);
      E = (double*)fixed->base;
      fixed_rest = FixedScratch{fixed->base + take, fixed->bytes - take};
      fixed = &fixed_rest;
    } else {
      if (!h->sfc.ensure(eb)) return fail(h, "cannot allocate the emissivity model's buffers");
      E = (double*)h->sfc.p;
    }
  }
  order_after_previous(h, st);
  if (model) {
    const size_t PL = (size_t)b->n_profiles * s.L;
    if (cudaMemsetAsync(h->d_error, 0, sizeof(int), st) != cudaSuccess) return fail(h, "error flag reset failed");
    irwater_kernel<<<(unsigned)((PL + 255) / 256), 256, 0, st>>>(h->irw, b->n_profiles, s.L, s.spec.wn,
                                                                 b->sensor_zenith_angle, b->water_temperature,
                                                                 b->water_coverage, b->wind_speed, E, E + PL,
                                                                 E + 2 * PL, h->d_error);
    CK_LAUNCH(h);
    bm = *b;
    bm.emissivity = E;
    b = &bm;
    sm.ev = E + PL;
    sm.et = h->irw.nalli2 ? E + 2 * PL : nullptr;
  }
  auto run = [&](const crtm_gpu_batch* bb, int md, const HostCopy* hcc, const FixedScratch* fx, bool sc,
                 const int* perm, bool nzm) {
    switch (s.group) {
      case 1: return fp64 ? run_pipeline<1, double>(h, s, bb, md, seed, rts, kk, ad, st, hcc, fx, sc, &sm, perm, nzm)
                          : run_pipeline<1, float>(h, s, bb, md, seed, rts, kk, ad, st, hcc, fx, sc, &sm, perm, nzm);
      case 2: return fp64 ? run_pipeline<2, double>(h, s, bb, md, seed, rts, kk, ad, st, hcc, fx, sc, &sm, perm, nzm)
                          : run_pipeline<2, float>(h, s, bb, md, seed, rts, kk, ad, st, hcc, fx, sc, &sm, perm, nzm);
      default: return fp64 ? run_pipeline<3, double>(h, s, bb, md, seed, rts, kk, ad, st, hcc, fx, sc, &sm, perm, nzm)
                           : run_pipeline<3, float>(h, s, bb, md, seed, rts, kk, ad, st, hcc, fx, sc, &sm, perm, nzm);
    }
  };
  int rc = CRTM_GPU_SUCCESS;
  if (!scat || b->n_profiles <= 0) {
    rc = run(b, mode, hc, fixed, scat, nullptr, scat && b->n_streams != nullptr);
  } else {
    // Buckets of a batch with clouds or aerosols: its clear profiles (the
    // clear-sky pipeline), its cloudy ones on the stream rule or up to 6
    // streams (kernels for 5 angles) and those with 8 or 16 streams (10
    // angles), each run as its own pipeline, so that every chunk's
    // scattering work space and grids hold only profiles that use them.  The
    // profile counts, clouds and stream options are read back to the host
    // first (the call waits for the stream to reach this point).
    const int P = b->n_profiles;
    std::vector<int> nc(P, 0), na(P, 0), ns(P, 0);
    bool ok = true;
    if (b->max_clouds > 0)
      ok &= cudaMemcpyAsync(nc.data(), b->n_clouds, sizeof(int) * P, cudaMemcpyDeviceToHost, st) == cudaSuccess;
    if (b->max_aerosols > 0)
      ok &= cudaMemcpyAsync(na.data(), b->n_aerosols, sizeof(int) * P, cudaMemcpyDeviceToHost, st) == cudaSuccess;
    if (b->n_streams)
      ok &= cudaMemcpyAsync(ns.data(), b->n_streams, sizeof(int) * P, cudaMemcpyDeviceToHost, st) == cudaSuccess;
    if (!ok || cudaStreamSynchronize(st) != cudaSuccess) return fail(h, "reading the batch's cloud counts failed");
    int cnt[3] = {0, 0, 0};
    std::vector<int> cls(P);
    for (int p = 0; p < P; p++) {
      cls[p] = (nc[p] > 0 || na[p] > 0) ? (ns[p] > 6 ? 2 : 1) : 0;
      cnt[cls[p]]++;
    }
    const int start[3] = {0, cnt[0], cnt[0] + cnt[1]};
    const int n_buckets = (cnt[0] > 0) + (cnt[1] > 0) + (cnt[2] > 0);
    const int* dperm = nullptr;
    FixedScratch fx_rest{};
    if (n_buckets > 1) {   // the profiles in bucket order (stable)
      std::vector<int> perm(P);
      int pos[3] = {start[0], start[1], start[2]};
      for (int p = 0; p < P; p++) perm[pos[cls[p]]++] = p;
      const size_t pb = ((size_t)P * sizeof(int) + 255) & ~(size_t)255;
      int* dp;
      if (fixed) {
        if (pb >= fixed->bytes) return fail(h, "the profile order of %d profiles does not fit the static scratch", P);
        dp = (int*)fixed->base;
        fx_rest = FixedScratch{fixed->base + pb, fixed->bytes - pb};
        fixed = &fx_rest;
      } else {
        if (!h->small.ensure(pb)) return fail(h, "cannot allocate the profile order");
        dp = (int*)h->small.p;
      }
      if (cudaMemcpyAsync(dp, perm.data(), sizeof(int) * P, cudaMemcpyHostToDevice, st) != cudaSuccess)
        return fail(h, "profile order upload failed");
      dperm = dp;
    }
    for (int c = 0; c < 3 && rc == CRTM_GPU_SUCCESS; c++) {
      if (!cnt[c]) continue;
      crtm_gpu_batch bc = *b;
      bc.n_profiles = cnt[c];
      rc = run(&bc, c == 0 && mode == 3 ? 0 : mode, dperm ? nullptr : hc, fixed, c != 0,
               dperm ? dperm + start[c] : nullptr, c == 2);
    }
    // the scattering Jacobians of the clear profiles are zero
    if (rc == CRTM_GPU_SUCCESS && cnt[0] > 0 && (mode == 1 || mode == 2)) {
      const int NCb = b->max_clouds > 0 ? b->max_clouds : 0, NAb = b->max_aerosols > 0 ? b->max_aerosols : 0;
      const size_t lead = mode == 1 ? (size_t)s.L * b->max_layers : (size_t)b->max_layers;
      double* const outs[7] = {
          mode == 1 ? kk->cloud_water_content : ad->cloud_water_content,
          mode == 1 ? kk->cloud_effective_radius : ad->cloud_effective_radius,
          mode == 1 ? kk->cloud_fraction : ad->cloud_fraction,
          mode == 1 ? kk->aerosol_concentration : ad->aerosol_concentration,
          mode == 1 ? kk->aerosol_effective_radius : ad->aerosol_effective_radius,
          mode == 1 ? kk->aerosol_effective_variance : ad->aerosol_effective_variance,
          mode == 1 ? kk->relative_humidity : ad->relative_humidity};
      const size_t rows[7] = {lead * NCb, lead * NCb, NCb ? lead : 0, lead * NAb, lead * NAb, lead * NAb,
                              NAb ? lead : 0};
      for (int i = 0; i < 7; i++) {
        if (!outs[i] || !rows[i]) continue;
        if (dperm) {
          const size_t nel = (size_t)cnt[0] * rows[i];
          zero_profile_rows_kernel<<<(unsigned)((nel + 255) / 256), 256, 0, st>>>(outs[i], dperm, cnt[0], rows[i]);
          CK_LAUNCH(h);
        } else if (cudaMemsetAsync(outs[i], 0, (size_t)P * rows[i] * sizeof(double), st) != cudaSuccess) {
          rc = fail(h, "output clear failed");
        }
      }
    }
    if (rc == CRTM_GPU_SUCCESS && dperm && hc && hc->n) rc = copy_chunk(h, hc, 0, P, st);
  }
  mark_done(h, st);
  return rc;
}

int check_call(crtm_gpu_handle h, const crtm_gpu_batch* b, const crtm_gpu_rtsolution* rts);

// Host entry points: copy inputs to the device, run, copy outputs back.
// Copy a host batch (and an optional [P][L] seed) into the handle's input
// buffer; db receives the batch with device pointers.
int stage_batch(crtm_gpu_handle h, const crtm_gpu_batch* b, int L, const double* seed, crtm_gpu_batch* db_out,
                const double** dseed_out) {
  const int P = b->n_profiles, Km = b->max_layers, J = b->n_absorbers;
  order_after_previous(h, h->stream);
  // input layout: doubles then ints
  struct Item { const void* src; size_t bytes; };
  const size_t PD = (size_t)P * sizeof(double);
  std::vector<Item> items = {
      {b->level_pressure, (size_t)P * (Km + 1) * 8}, {b->pressure, (size_t)P * Km * 8},
      {b->temperature, (size_t)P * Km * 8},           {b->absorber, (size_t)P * J * Km * 8},
      {b->land_coverage, PD}, {b->water_coverage, PD}, {b->snow_coverage, PD}, {b->ice_coverage, PD},
      {b->land_temperature, PD}, {b->water_temperature, PD}, {b->snow_temperature, PD},
      {b->ice_temperature, PD}, {b->sensor_zenith_angle, PD}, {b->surface_altitude, PD},
      {b->emissivity, (size_t)P * L * 8}, {seed, (size_t)P * L * 8}, {b->n_layers, (size_t)P * 4}};
  const int NC = b->max_clouds > 0 ? b->max_clouds : 0;
  const int NA = b->max_aerosols > 0 ? b->max_aerosols : 0;
  if (NA > 0) {
    if (!b->n_aerosols || !b->aerosol_type || !b->aerosol_concentration || !b->aerosol_effective_radius)
      return fail(h, "aerosol arrays missing for max_aerosols = %d", NA);
    for (int m = 0; m < P; m++)
      if (b->n_aerosols[m] < 0 || b->n_aerosols[m] > NA)
        return fail(h, "profile %d: n_aerosols %d outside [0, max_aerosols=%d]", m, b->n_aerosols[m], NA);
  }
  if (NC > 0) {
    if (!b->n_clouds || !b->cloud_type || !b->cloud_water_content || !b->cloud_effective_radius)
      return fail(h, "cloud arrays missing for max_clouds = %d", NC);
    for (int m = 0; m < P; m++)
      if (b->n_clouds[m] < 0 || b->n_clouds[m] > NC)
        return fail(h, "profile %d: n_clouds %d outside [0, max_clouds=%d]", m, b->n_clouds[m], NC);
    items.insert(items.end(), {{b->cloud_water_content, (size_t)P * NC * Km * 8},
                               {b->cloud_effective_radius, (size_t)P * NC * Km * 8},
                               {b->n_clouds, (size_t)P * 4}, {b->cloud_type, (size_t)P * NC * 4},
                               {b->n_streams, b->n_streams ? (size_t)P * 4 : 0},
                               {b->rt_algorithm_id, b->rt_algorithm_id ? (size_t)P * 4 : 0},
                               {b->cloud_fraction, b->cloud_fraction ? (size_t)P * Km * 8 : 0},
                               {b->overlap_id, b->overlap_id ? (size_t)P * 4 : 0}});
  }
  const size_t aer0 = items.size();
  if (NA > 0)
    items.insert(items.end(), {{b->aerosol_concentration, (size_t)P * NA * Km * 8},
                               {b->aerosol_effective_radius, (size_t)P * NA * Km * 8},
                               {b->n_aerosols, (size_t)P * 4}, {b->aerosol_type, (size_t)P * NA * 4}});
  const size_t wind0 = items.size();
  items.push_back({b->wind_speed, b->wind_speed ? PD : 0});
  const size_t aer1 = items.size();
  if (NA > 0)
    items.insert(items.end(),
                 {{b->aerosol_effective_variance, b->aerosol_effective_variance ? (size_t)P * NA * Km * 8 : 0},
                  {b->relative_humidity, b->relative_humidity ? (size_t)P * Km * 8 : 0}});
  if (NC == 0 && b->max_clouds <= 0 && (b->n_streams || b->rt_algorithm_id) && NA > 0) {
    // options without clouds (aerosol-only batch)
    items.insert(items.end(), {{b->n_streams, b->n_streams ? (size_t)P * 4 : 0},
                               {b->rt_algorithm_id, b->rt_algorithm_id ? (size_t)P * 4 : 0}});
  }
  size_t tot = 0;
  for (auto& it : items) tot += align_up(it.bytes);
  if (!h->io_in.ensure(tot)) return fail(h, "cannot allocate %zu bytes for inputs", tot);
  std::vector<void*> dptr(items.size(), nullptr);
  size_t off = 0;
  cudaStream_t st = h->stream;
  for (size_t i = 0; i < items.size(); i++) {
    if (items[i].src && items[i].bytes) {
      dptr[i] = (char*)h->io_in.p + off;
      if (cudaMemcpyAsync(dptr[i], items[i].src, items[i].bytes, cudaMemcpyHostToDevice, st) != cudaSuccess)
        return fail(h, "host-to-device copy failed");
    }
    off += align_up(items[i].bytes);
  }
  crtm_gpu_batch& db = *db_out;
  db = *b;
  db.level_pressure = (const double*)dptr[0]; db.pressure = (const double*)dptr[1];
  db.temperature = (const double*)dptr[2]; db.absorber = (const double*)dptr[3];
  db.land_coverage = (const double*)dptr[4]; db.water_coverage = (const double*)dptr[5];
  db.snow_coverage = (const double*)dptr[6]; db.ice_coverage = (const double*)dptr[7];
  db.land_temperature = (const double*)dptr[8]; db.water_temperature = (const double*)dptr[9];
  db.snow_temperature = (const double*)dptr[10]; db.ice_temperature = (const double*)dptr[11];
  db.sensor_zenith_angle = (const double*)dptr[12]; db.surface_altitude = (const double*)dptr[13];
  db.emissivity = (const double*)dptr[14];
  const double* dseed = (const double*)dptr[15];
  db.n_layers = (const int*)dptr[16];
  if (NC > 0) {
    db.cloud_water_content = (const double*)dptr[17];
    db.cloud_effective_radius = (const double*)dptr[18];
    db.n_clouds = (const int*)dptr[19];
    db.cloud_type = (const int*)dptr[20];
    db.n_streams = (const int*)dptr[21];
    db.rt_algorithm_id = (const int*)dptr[22];
    db.cloud_fraction = (const double*)dptr[23];
    db.overlap_id = (const int*)dptr[24];
  } else {
    db.cloud_fraction = nullptr;
    db.overlap_id = nullptr;
  }
  db.wind_speed = (const double*)dptr[wind0];
  if (NA > 0) {
    db.aerosol_concentration = (const double*)dptr[aer0];
    db.aerosol_effective_radius = (const double*)dptr[aer0 + 1];
    db.n_aerosols = (const int*)dptr[aer0 + 2];
    db.aerosol_type = (const int*)dptr[aer0 + 3];
    if (NC == 0) {
      db.n_streams = b->n_streams ? (const int*)dptr[aer1 + 2] : nullptr;
      db.rt_algorithm_id = b->rt_algorithm_id ? (const int*)dptr[aer1 + 3] : nullptr;
    }
    db.aerosol_effective_variance = (const double*)dptr[aer1];
    db.relative_humidity = (const double*)dptr[aer1 + 1];
  } else {
    db.aerosol_effective_variance = nullptr;
    db.relative_humidity = nullptr;
  }
  *dseed_out = dseed;
  return CRTM_GPU_SUCCESS;
}

int host_call(crtm_gpu_handle h, int sensor, const crtm_gpu_batch* b, int mode, const double* seed,
              crtm_gpu_kmatrix* kk, crtm_gpu_adjoint_out* ad, crtm_gpu_rtsolution* rts) {
  if (!h) return CRTM_GPU_FAILURE;
  if (sensor < 0 || sensor >= (int)h->sensors.size()) return fail(h, "sensor index %d out of range", sensor);
  if (!b || b->n_profiles < 0 || b->max_layers < 1 || b->n_absorbers < 0) return fail(h, "bad batch dimensions");
  if (cudaSetDevice(h->device) != cudaSuccess) return fail(h, "cudaSetDevice failed");
  const int P = b->n_profiles, Km = b->max_layers, J = b->n_absorbers, L = h->sensors[sensor].L;
  if (P == 0 || L == 0) return CRTM_GPU_SUCCESS;
  for (int m = 0; m < P; m++)
    if (b->n_layers[m] < 2 || b->n_layers[m] > Km)
      return fail(h, "profile %d: n_layers %d outside [2, max_layers=%d]", m, b->n_layers[m], Km);
  crtm_gpu_batch db;
  const double* dseed = nullptr;
  if (int rc = stage_batch(h, b, L, seed, &db, &dseed)) return rc;
  const int NC = b->max_clouds > 0 ? b->max_clouds : 0;
  const int NA = b->max_aerosols > 0 ? b->max_aerosols : 0;
  const size_t PD = (size_t)P * sizeof(double);
  cudaStream_t st = h->stream;
  size_t off = 0;
  // outputs
  const size_t PL = (size_t)P * L;
  std::vector<std::pair<void*, size_t>> outs = {{rts->radiance, PL * 8}, {rts->brightness_temperature, PL * 8},
                                                {rts->status, rts->status ? (size_t)P * 4 : 0}};
  const int JK = (mode == 1 && kk->n_k_absorbers > 0) ? kk->n_k_absorbers : J;
  const size_t NCo = NC, NAo = NA;
  if (mode == 1)
    outs.insert(outs.end(), {{kk->temperature, PL * Km * 8}, {kk->absorber, PL * JK * Km * 8},
                             {kk->water_temperature, PL * 8}, {kk->surface_emissivity, PL * 8},
                             {kk->cloud_water_content, NCo ? PL * NCo * Km * 8 : 0},
                             {kk->cloud_effective_radius, NCo ? PL * NCo * Km * 8 : 0},
                             {kk->cloud_fraction, NCo ? PL * Km * 8 : 0},
                             {kk->aerosol_concentration, NAo ? PL * NAo * Km * 8 : 0},
                             {kk->aerosol_effective_radius, NAo ? PL * NAo * Km * 8 : 0},
                             {kk->land_temperature, PL * 8}, {kk->snow_temperature, PL * 8},
                             {kk->ice_temperature, PL * 8},
                             {kk->aerosol_effective_variance, NAo ? PL * NAo * Km * 8 : 0},
                             {kk->relative_humidity, NAo ? PL * Km * 8 : 0}, {kk->wind_speed, PL * 8}});
  if (mode == 2)
    outs.insert(outs.end(), {{ad->temperature, (size_t)P * Km * 8}, {ad->absorber, (size_t)P * J * Km * 8},
                             {ad->water_temperature, PD},
                             {ad->cloud_water_content, NCo ? (size_t)P * NCo * Km * 8 : 0},
                             {ad->cloud_effective_radius, NCo ? (size_t)P * NCo * Km * 8 : 0},
                             {ad->cloud_fraction, NCo ? (size_t)P * Km * 8 : 0},
                             {ad->aerosol_concentration, NAo ? (size_t)P * NAo * Km * 8 : 0},
                             {ad->aerosol_effective_radius, NAo ? (size_t)P * NAo * Km * 8 : 0},
                             {ad->land_temperature, PD}, {ad->snow_temperature, PD}, {ad->ice_temperature, PD},
                             {ad->aerosol_effective_variance, NAo ? (size_t)P * NAo * Km * 8 : 0},
                             {ad->relative_humidity, NAo ? (size_t)P * Km * 8 : 0}, {ad->wind_speed, PD}});
  const size_t ext0 = outs.size();
  {
    void* ep[N_RTS_EXT];
    size_t eb[N_RTS_EXT];
    rts_ext_list(rts, PL, (size_t)Km, ep, eb);
    for (int i = 0; i < N_RTS_EXT; i++) outs.push_back({ep[i], eb[i]});
  }
  size_t tout = 0;
  for (auto& o : outs) tout += align_up(o.second);
  if (!h->io_out.ensure(tout)) return fail(h, "cannot allocate %zu bytes for outputs", tout);
  std::vector<void*> dout(outs.size(), nullptr);
  off = 0;
  for (size_t i = 0; i < outs.size(); i++) {
    if (outs[i].first && outs[i].second) dout[i] = (char*)h->io_out.p + off;
    off += align_up(outs[i].second);
  }
  crtm_gpu_rtsolution drts{(double*)dout[0], (double*)dout[1], (int*)dout[2]};
  rts_ext_set(&drts, dout.data() + ext0);
  crtm_gpu_kmatrix dk{};
  crtm_gpu_adjoint_out dad{};
  if (mode == 1)
    dk = {(double*)dout[3], (double*)dout[4], (double*)dout[5], (double*)dout[6], kk->n_k_absorbers,
          kk->k_absorber_index, (double*)dout[7], (double*)dout[8], (double*)dout[9], (double*)dout[10],
          (double*)dout[11], (double*)dout[12], (double*)dout[13], (double*)dout[14], (double*)dout[15],
          (double*)dout[16], (double*)dout[17]};
  if (mode == 2)
    dad = {(double*)dout[3], (double*)dout[4], (double*)dout[5], (double*)dout[6], (double*)dout[7],
           (double*)dout[8], (double*)dout[9], (double*)dout[10], (double*)dout[11], (double*)dout[12],
           (double*)dout[13], (double*)dout[14], (double*)dout[15], (double*)dout[16]};
  HostCopy hc;
  hc.n = (int)outs.size();
  for (size_t i = 0; i < outs.size(); i++) {
    hc.dst[i] = dout[i] ? outs[i].first : nullptr;
    hc.src[i] = dout[i];
    hc.per[i] = outs[i].second / (size_t)P;
  }
  // several chunks so that the copies of finished chunks overlap the next ones
  hc.max_chunk = std::max(32, (P + 5) / 6);
  int rc = dispatch(h, sensor, &db, mode, dseed, &drts, mode == 1 ? &dk : nullptr,
                    mode == 2 ? &dad : nullptr, st, &hc);
  cudaError_t e = cudaStreamSynchronize(st);
  cudaError_t e2 = h->copy_stream ? cudaStreamSynchronize(h->copy_stream) : cudaSuccess;
  for (auto ev : h->chunk_events) cudaEventDestroy(ev);
  h->chunk_events.clear();
  if (rc != CRTM_GPU_SUCCESS) return rc;
  if (e != cudaSuccess || e2 != cudaSuccess)
    return fail(h, "CUDA error: %s", cudaGetErrorString(e != cudaSuccess ? e : e2));
  if (h->profiling) collect_stage_times(h);
  return check_call(h, b, rts);
}

// After a host entry point's work has finished: the scattering error flag and
// the per-profile status words.
int check_call(crtm_gpu_handle h, const crtm_gpu_batch* b, const crtm_gpu_rtsolution* rts) {
  if (b->max_clouds > 0 || b->max_aerosols > 0 || h->model_call) {
    int code = 0;
    if (cudaMemcpy(&code, h->d_error, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
      return fail(h, "cannot read the scattering error flag");
    if (code) return fail(h, "radiative transfer failed (code %d: 1-3 stream set, 4 cloud type, "
                             "5-6 singular matrix, 8 aerosol stream set or LUT, 9 aerosol type, 11 invalid "
                             "Options%Overlap_Id, 12 SOI order-field slots below 17, 13 emissivity model with a water "
                             "coverage other than 1)", code);
  }
  if (rts->status)
    for (int m = 0; m < b->n_profiles; m++)
      if (rts->status[m] != 0) return fail(h, "profile %d failed (status bits 0x%x)", m, rts->status[m]);
  return CRTM_GPU_SUCCESS;
}

// Tangent linear as the K-matrix contracted with the perturbations.
struct TLArgs {
  int P, L, Km, J, NC, NA;
  const int* n_layers;
  const int* status;
  const double* kt, *ka, *kw, *kl, *ks, *ki, *ke, *kwc, *kre, *kcf, *kac, *kar, *kav, *krh, *kws;
  crtm_gpu_tl_in d;
  double* bt_tl;
};

// One warp per (profile, TL_CH consecutive channels), lanes over the layers:
// each perturbation value is loaded once for the warp's channels, whose
// TL_CH sums are independent accumulations (the same order per channel as a
// warp per channel would take).
constexpr int TL_CH = 8;

__global__ void tl_kernel(TLArgs a) {
  const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int groups = (a.L + TL_CH - 1) / TL_CH;
  if (w >= (long long)a.P * groups) return;
  const int p = (int)(w / groups), l0 = (int)(w % groups) * TL_CH;
  const int nch = min(TL_CH, a.L - l0);
  const int Ku = a.n_layers[p];
  double s[TL_CH];
#pragma unroll
  for (int c = 0; c < TL_CH; c++) s[c] = 0.0;
  auto rows = [&](const double* K, const double* D, int nrow) {
    if (!K || !D) return;
    const size_t cstride = (size_t)nrow * a.Km;   // one channel's rows
    const double* k0 = K + ((size_t)p * a.L + l0) * cstride;
    for (int r = 0; r < nrow; r++) {
      const double* dr = D + ((size_t)p * nrow + r) * a.Km;
      const double* kr = k0 + (size_t)r * a.Km;
      for (int k = lane; k < Ku; k += 32) {
        const double d = dr[k];
#pragma unroll
        for (int c = 0; c < TL_CH; c++)
          if (c < nch) s[c] += kr[c * cstride + k] * d;
      }
    }
  };
  rows(a.kt, a.d.temperature, 1);
  rows(a.ka, a.d.absorber, a.J);
  rows(a.kwc, a.d.cloud_water_content, a.NC);
  rows(a.kre, a.d.cloud_effective_radius, a.NC);
  rows(a.kcf, a.d.cloud_fraction, 1);
  rows(a.kac, a.d.aerosol_concentration, a.NA);
  rows(a.kar, a.d.aerosol_effective_radius, a.NA);
  rows(a.kav, a.d.aerosol_effective_variance, a.NA);
  rows(a.krh, a.d.relative_humidity, 1);
  double mine = 0.0;
#pragma unroll
  for (int c = 0; c < TL_CH; c++) {
    double v = s[c];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == c) mine = v;
  }
  if (lane >= nch) return;
  const size_t pl = (size_t)p * a.L + l0 + lane;
  double t = mine;
  if (a.d.water_temperature) t += a.kw[pl] * a.d.water_temperature[p];
  if (a.d.land_temperature) t += a.kl[pl] * a.d.land_temperature[p];
  if (a.d.snow_temperature) t += a.ks[pl] * a.d.snow_temperature[p];
  if (a.d.ice_temperature) t += a.ki[pl] * a.d.ice_temperature[p];
  if (a.d.emissivity) t += a.ke[pl] * a.d.emissivity[pl];
  if (a.d.wind_speed && a.kws) t += a.kws[pl] * a.d.wind_speed[p];
  a.bt_tl[pl] = (a.status && a.status[p]) ? 0.0 : t;
}

// The trajectory's K-matrix into the handle's scratch: every Jacobian the
// batch has (want == NULL), or those of the perturbations `want` gives; the
// profiles' layer counts and status words beside it.  Enqueued on st.
int linearize(crtm_gpu_handle h, int sensor, const crtm_gpu_batch* b, crtm_gpu_rtsolution* rts,
              const crtm_gpu_tl_in* want, cudaStream_t st) {
  if (!h) return CRTM_GPU_FAILURE;
  h->lin.valid = false;
  if (sensor < 0 || sensor >= (int)h->sensors.size()) return fail(h, "sensor index %d out of range", sensor);
  if (!b || b->n_profiles < 0 || b->max_layers < 1) return fail(h, "bad batch dimensions");
  if (!rts || !rts->radiance || !rts->brightness_temperature) return fail(h, "missing RTSolution buffers");
  const size_t P = b->n_profiles, L = h->sensors[sensor].L, Km = b->max_layers, J = b->n_absorbers;
  const size_t NC = b->max_clouds > 0 ? b->max_clouds : 0, NA = b->max_aerosols > 0 ? b->max_aerosols : 0;
  const bool wc = NC && (!want || want->cloud_water_content || want->cloud_effective_radius);
  const bool cf = NC && (!want || want->cloud_fraction);
  const bool aer = NA && (!want || want->aerosol_concentration || want->aerosol_effective_radius);
  const bool av = NA && (!want || want->aerosol_effective_variance);
  const bool rh = NA && (!want || want->relative_humidity);
  const bool ws = !b->emissivity && (!want || want->wind_speed);   // the emissivity model's wind speed
  const size_t PL = P * L;
  const size_t n_el = PL * Km * (1 + J) + 5 * PL + (wc ? 2 * PL * NC * Km : 0) + (cf ? PL * Km : 0) +
                      (aer ? 2 * PL * NA * Km : 0) + (av ? PL * NA * Km : 0) + (rh ? PL * Km : 0) +
                      (ws ? PL : 0);
  if (cudaSetDevice(h->device) != cudaSuccess) return fail(h, "cudaSetDevice failed");
  if (!h->tl_k.ensure(std::max<size_t>(n_el, 1) * sizeof(double)))
    return fail(h, "cannot allocate %zu bytes for the trajectory's K-matrix", n_el * sizeof(double));
  if (!h->lin_meta.ensure(std::max<size_t>(2 * P, 1) * sizeof(int)))
    return fail(h, "cannot allocate the trajectory's profile table");
  if (P == 0 || L == 0) {
    h->lin = {};
    h->lin.valid = true;
    h->lin.sensor = sensor;
    h->lin.P = (int)P; h->lin.L = (int)L; h->lin.Km = (int)Km; h->lin.J = (int)J;
    return CRTM_GPU_SUCCESS;
  }
  double* q = (double*)h->tl_k.p;
  auto take = [&](size_t n) { double* r = q; q += n; return r; };
  crtm_gpu_kmatrix kk{};
  kk.temperature = take(PL * Km);
  kk.absorber = take(PL * J * Km);
  kk.water_temperature = take(PL);
  kk.land_temperature = take(PL);
  kk.snow_temperature = take(PL);
  kk.ice_temperature = take(PL);
  kk.surface_emissivity = take(PL);
  if (wc) { kk.cloud_water_content = take(PL * NC * Km); kk.cloud_effective_radius = take(PL * NC * Km); }
  if (cf) kk.cloud_fraction = take(PL * Km);
  if (aer) { kk.aerosol_concentration = take(PL * NA * Km); kk.aerosol_effective_radius = take(PL * NA * Km); }
  if (av) kk.aerosol_effective_variance = take(PL * NA * Km);
  if (rh) kk.relative_humidity = take(PL * Km);
  if (ws) kk.wind_speed = take(PL);
  if (int rc = dispatch(h, sensor, b, 1, nullptr, rts, &kk, nullptr, st)) return rc;
  int* meta = (int*)h->lin_meta.p;
  if (cudaMemcpyAsync(meta, b->n_layers, P * sizeof(int), cudaMemcpyDeviceToDevice, st) != cudaSuccess ||
      (rts->status ? cudaMemcpyAsync(meta + P, rts->status, P * sizeof(int), cudaMemcpyDeviceToDevice, st)
                   : cudaMemsetAsync(meta + P, 0, P * sizeof(int), st)) != cudaSuccess)
    return fail(h, "trajectory profile table copy failed");
  h->lin.valid = true;
  h->lin.sensor = sensor;
  h->lin.P = (int)P; h->lin.L = (int)L; h->lin.Km = (int)Km; h->lin.J = (int)J;
  h->lin.NC = (int)NC; h->lin.NA = (int)NA;
  h->lin.k = kk;
  h->lin.n_layers = meta;
  h->lin.status = meta + P;
  mark_done(h, st);
  return CRTM_GPU_SUCCESS;
}

// The tangent linear about the stored trajectory: bt_tl [P][L] from the
// perturbations tl (device pointers), one read of the stored Jacobians.
int tl_apply(crtm_gpu_handle h, const crtm_gpu_tl_in* tl, double* bt_tl, cudaStream_t st) {
  if (!h) return CRTM_GPU_FAILURE;
  if (!h->lin.valid) return fail(h, "no trajectory: call crtm_gpu_linearize first");
  if (!tl || !bt_tl) return fail(h, "missing tangent-linear inputs or output");
  const auto& g = h->lin;
  auto need = [&](const double* d, const double* k, const char* what) {
    return d && !k ? fail(h, "the trajectory holds no %s Jacobian", what) : CRTM_GPU_SUCCESS;
  };
  if (int rc = need(tl->cloud_water_content, g.k.cloud_water_content, "cloud water content")) return rc;
  if (int rc = need(tl->cloud_effective_radius, g.k.cloud_effective_radius, "cloud effective radius")) return rc;
  if (int rc = need(tl->cloud_fraction, g.k.cloud_fraction, "cloud fraction")) return rc;
  if (int rc = need(tl->aerosol_concentration, g.k.aerosol_concentration, "aerosol concentration")) return rc;
  if (int rc = need(tl->aerosol_effective_radius, g.k.aerosol_effective_radius, "aerosol radius")) return rc;
  if (int rc = need(tl->aerosol_effective_variance, g.k.aerosol_effective_variance, "effective variance")) return rc;
  if (int rc = need(tl->relative_humidity, g.k.relative_humidity, "relative humidity")) return rc;
  if (g.P == 0 || g.L == 0) return CRTM_GPU_SUCCESS;
  if (cudaSetDevice(h->device) != cudaSuccess) return fail(h, "cudaSetDevice failed");
  order_after_previous(h, st);
  TLArgs ta{};
  ta.P = g.P; ta.L = g.L; ta.Km = g.Km; ta.J = g.J; ta.NC = g.NC; ta.NA = g.NA;
  ta.n_layers = g.n_layers; ta.status = g.status; ta.d = *tl; ta.bt_tl = bt_tl;
  ta.kt = g.k.temperature; ta.ka = g.k.absorber; ta.kw = g.k.water_temperature; ta.kl = g.k.land_temperature;
  ta.ks = g.k.snow_temperature; ta.ki = g.k.ice_temperature; ta.ke = g.k.surface_emissivity;
  ta.kwc = g.k.cloud_water_content; ta.kre = g.k.cloud_effective_radius; ta.kcf = g.k.cloud_fraction;
  ta.kac = g.k.aerosol_concentration; ta.kar = g.k.aerosol_effective_radius;
  ta.kav = g.k.aerosol_effective_variance; ta.krh = g.k.relative_humidity; ta.kws = g.k.wind_speed;
  const long long threads = (long long)g.P * ((g.L + TL_CH - 1) / TL_CH) * 32;
  tl_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(ta);
  CK_LAUNCH(h);
  mark_done(h, st);
  return CRTM_GPU_SUCCESS;
}

// out[p][j] = sum_l w[p][l] K[p][l][j] (j over a block's rows x layers), zero
// for profiles whose trajectory status is not 0: one thread per (p, j), the
// channels' rows read coalesced across j.
__global__ void channel_contract_kernel(const double* __restrict__ K, int P, int L, int rowlen,
                                        const double* __restrict__ w, const int* __restrict__ status,
                                        double* __restrict__ out) {
  const int p = blockIdx.y;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P || j >= rowlen) return;
  double acc = 0.0;
  if (!status[p]) {
    const double* kp = K + (size_t)p * L * rowlen + j;
    const double* wp = w + (size_t)p * L;
    for (int l = 0; l < L; l++) acc += wp[l] * kp[(size_t)l * rowlen];
  }
  out[(size_t)p * rowlen + j] = acc;
}

// The adjoint about the stored trajectory: the outputs of CRTM_Adjoint for
// the seed bt_ad [P][L] (device pointers), one read of the stored Jacobians.
int ad_apply(crtm_gpu_handle h, const double* bt_ad, crtm_gpu_adjoint_out* ad, cudaStream_t st) {
  if (!h) return CRTM_GPU_FAILURE;
  if (!h->lin.valid) return fail(h, "no trajectory: call crtm_gpu_linearize first");
  if (!bt_ad || !ad || !ad->temperature || !ad->absorber || !ad->water_temperature)
    return fail(h, "missing adjoint seed or outputs");
  const auto& g = h->lin;
  if (g.P == 0) return CRTM_GPU_SUCCESS;
  if (cudaSetDevice(h->device) != cudaSuccess) return fail(h, "cudaSetDevice failed");
  order_after_previous(h, st);
  const int Km = g.Km;
  struct Block { const double* k; double* out; int rowlen; const char* what; };
  const Block blocks[] = {
      {g.k.temperature, ad->temperature, Km, "temperature"},
      {g.k.absorber, ad->absorber, g.J * Km, "absorber"},
      {g.k.water_temperature, ad->water_temperature, 1, "water temperature"},
      {g.k.land_temperature, ad->land_temperature, 1, "land temperature"},
      {g.k.snow_temperature, ad->snow_temperature, 1, "snow temperature"},
      {g.k.ice_temperature, ad->ice_temperature, 1, "ice temperature"},
      {g.k.cloud_water_content, ad->cloud_water_content, g.NC * Km, "cloud water content"},
      {g.k.cloud_effective_radius, ad->cloud_effective_radius, g.NC * Km, "cloud effective radius"},
      {g.k.cloud_fraction, ad->cloud_fraction, Km, "cloud fraction"},
      {g.k.aerosol_concentration, ad->aerosol_concentration, g.NA * Km, "aerosol concentration"},
      {g.k.aerosol_effective_radius, ad->aerosol_effective_radius, g.NA * Km, "aerosol radius"},
      {g.k.aerosol_effective_variance, ad->aerosol_effective_variance, g.NA * Km, "effective variance"},
      {g.k.relative_humidity, ad->relative_humidity, Km, "relative humidity"},
      {g.k.wind_speed, ad->wind_speed, 1, "wind speed"},
  };
  for (const Block& x : blocks) {
    if (!x.out) continue;
    if (!x.k) return fail(h, "the trajectory holds no %s Jacobian", x.what);
    if (x.rowlen <= 0) continue;
    if (g.L == 0) {
      if (cudaMemsetAsync(x.out, 0, (size_t)g.P * x.rowlen * sizeof(double), st) != cudaSuccess)
        return fail(h, "cudaMemsetAsync failed");
      continue;
    }
    const dim3 grid((unsigned)((x.rowlen + 127) / 128), (unsigned)g.P);
    channel_contract_kernel<<<grid, 128, 0, st>>>(x.k, g.P, g.L, x.rowlen, bt_ad, g.status, x.out);
    CK_LAUNCH(h);
  }
  mark_done(h, st);
  return CRTM_GPU_SUCCESS;
}

int tl_device(crtm_gpu_handle h, int sensor, const crtm_gpu_batch* b, const crtm_gpu_tl_in* tl,
              crtm_gpu_rtsolution* rts, double* bt_tl, cudaStream_t st) {
  if (!h) return CRTM_GPU_FAILURE;
  if (!tl || !bt_tl) return fail(h, "missing tangent-linear inputs or output");
  if (int rc = linearize(h, sensor, b, rts, tl, st)) return rc;
  return tl_apply(h, tl, bt_tl, st);
}

int tl_host(crtm_gpu_handle h, int sensor, const crtm_gpu_batch* b, const crtm_gpu_tl_in* tl,
            crtm_gpu_rtsolution* rts, double* bt_tl) {
  if (!h) return CRTM_GPU_FAILURE;
  if (!tl || !bt_tl || !rts || !rts->radiance || !rts->brightness_temperature)
    return fail(h, "missing tangent-linear inputs or outputs");
  if (sensor < 0 || sensor >= (int)h->sensors.size()) return fail(h, "sensor index %d out of range", sensor);
  if (!b || b->n_profiles < 0 || b->max_layers < 1 || b->n_absorbers < 0) return fail(h, "bad batch dimensions");
  if (cudaSetDevice(h->device) != cudaSuccess) return fail(h, "cudaSetDevice failed");
  const size_t P = b->n_profiles, L = h->sensors[sensor].L, Km = b->max_layers, J = b->n_absorbers;
  const size_t NC = b->max_clouds > 0 ? b->max_clouds : 0, NA = b->max_aerosols > 0 ? b->max_aerosols : 0;
  if (P == 0 || L == 0) return CRTM_GPU_SUCCESS;
  for (size_t m = 0; m < P; m++)
    if (b->n_layers[m] < 2 || b->n_layers[m] > (int)Km)
      return fail(h, "profile %zu: n_layers %d outside [2, max_layers=%zu]", m, b->n_layers[m], Km);
  crtm_gpu_batch db;
  const double* dseed = nullptr;
  if (int rc = stage_batch(h, b, (int)L, nullptr, &db, &dseed)) return rc;
  cudaStream_t st = h->stream;
  // perturbations
  constexpr int NTL = 15;
  const double* srcs[NTL] = {tl->temperature, tl->absorber, tl->land_temperature, tl->water_temperature,
                             tl->snow_temperature, tl->ice_temperature, tl->emissivity, tl->cloud_water_content,
                             tl->cloud_effective_radius, tl->cloud_fraction, tl->aerosol_concentration,
                             tl->aerosol_effective_radius, tl->aerosol_effective_variance, tl->relative_humidity,
                             tl->wind_speed};
  const size_t sz[NTL] = {P * Km, P * J * Km, P, P, P, P, P * L, P * NC * Km, P * NC * Km, NC ? P * Km : 0,
                          P * NA * Km, P * NA * Km, P * NA * Km, NA ? P * Km : 0, P};
  size_t tot = 0;
  for (int i = 0; i < NTL; i++) tot += srcs[i] && sz[i] ? align_up(sz[i] * 8) : 0;
  if (!h->io_tl.ensure(tot + 256)) return fail(h, "cannot allocate %zu bytes for the perturbations", tot);
  const double* dsrc[NTL] = {};
  size_t off = 0;
  for (int i = 0; i < NTL; i++) {
    if (!srcs[i] || !sz[i]) continue;
    dsrc[i] = (const double*)((char*)h->io_tl.p + off);
    if (cudaMemcpyAsync((void*)dsrc[i], srcs[i], sz[i] * 8, cudaMemcpyHostToDevice, st) != cudaSuccess)
      return fail(h, "host-to-device copy failed");
    off += align_up(sz[i] * 8);
  }
  const crtm_gpu_tl_in dtl = {dsrc[0], dsrc[1], dsrc[2],  dsrc[3],  dsrc[4],  dsrc[5],  dsrc[6], dsrc[7],
                              dsrc[8], dsrc[9], dsrc[10], dsrc[11], dsrc[12], dsrc[13], dsrc[14]};
  // outputs
  const size_t PL = P * L;
  const size_t o_bt = align_up(PL * 8), o_tl = o_bt + align_up(PL * 8), o_st = o_tl + align_up(PL * 8);
  void* ep[N_RTS_EXT];
  size_t eb[N_RTS_EXT], eo[N_RTS_EXT];
  rts_ext_list(rts, PL, Km, ep, eb);
  size_t o_end = o_st + align_up(P * 4);
  for (int i = 0; i < N_RTS_EXT; i++) { eo[i] = o_end; o_end += align_up(eb[i]); }
  if (!h->io_out.ensure(o_end)) return fail(h, "cannot allocate the outputs");
  char* ob = (char*)h->io_out.p;
  crtm_gpu_rtsolution drts{(double*)ob, (double*)(ob + o_bt), rts->status ? (int*)(ob + o_st) : nullptr};
  void* dep[N_RTS_EXT];
  for (int i = 0; i < N_RTS_EXT; i++) dep[i] = ep[i] ? ob + eo[i] : nullptr;
  rts_ext_set(&drts, dep);
  int rc = tl_device(h, sensor, &db, &dtl, &drts, (double*)(ob + o_tl), st);
  for (int i = 0; i < N_RTS_EXT && rc == CRTM_GPU_SUCCESS; i++)
    if (ep[i] && cudaMemcpyAsync(ep[i], dep[i], eb[i], cudaMemcpyDeviceToHost, st) != cudaSuccess)
      rc = fail(h, "device-to-host copy failed");
  if (rc == CRTM_GPU_SUCCESS) {
    if (cudaMemcpyAsync(rts->radiance, drts.radiance, PL * 8, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaMemcpyAsync(rts->brightness_temperature, drts.brightness_temperature, PL * 8, cudaMemcpyDeviceToHost,
                        st) != cudaSuccess ||
        cudaMemcpyAsync(bt_tl, ob + o_tl, PL * 8, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        (rts->status && cudaMemcpyAsync(rts->status, drts.status, P * 4, cudaMemcpyDeviceToHost, st) != cudaSuccess))
      rc = fail(h, "device-to-host copy failed");
  }
  const cudaError_t e = cudaStreamSynchronize(st);
  if (rc != CRTM_GPU_SUCCESS) return rc;
  if (e != cudaSuccess) return fail(h, "CUDA error: %s", cudaGetErrorString(e));
  if (h->profiling) collect_stage_times(h);
  return check_call(h, b, rts);
}

}  // namespace

extern "C" {

int crtm_gpu_init(const char* coeff_path, int n_sensors, const char* const* sensor_ids,
                  crtm_gpu_handle* handle) {
  return crtm_gpu_init_aerosol(coeff_path, n_sensors, sensor_ids, nullptr, nullptr, handle);
}

int crtm_gpu_init_aerosol(const char* coeff_path, int n_sensors, const char* const* sensor_ids,
                          const char* aerosol_model, const char* aerosol_coeff_file, crtm_gpu_handle* handle) {
  if (!handle) return fail(nullptr, "null handle pointer");
  *handle = nullptr;
  if (!coeff_path || n_sensors < 1 || !sensor_ids) return fail(nullptr, "bad init arguments");
  int scheme = AEROSOL_CRTM;
  if (aerosol_model) {
    const std::string m = aerosol_model;
    if (m == "CRTM") scheme = AEROSOL_CRTM;
    else if (m == "CMAQ") scheme = AEROSOL_CMAQ;
    else if (m == "GOCART-GEOS5") scheme = AEROSOL_GOCART;
    else if (m == "NAAPS") scheme = AEROSOL_NAAPS;
    else return fail(nullptr, "unknown Aerosol_Model '%s' (CRTM, CMAQ, GOCART-GEOS5 or NAAPS)", aerosol_model);
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return fail(nullptr, "no CUDA device");
  crtm_gpu_context* h = new crtm_gpu_context();
  h->device = dev;
  if (const char* e = getenv("CRTM_GPU_WORKSPACE_MB")) h->workspace_budget = (size_t)atoll(e) << 20;
  if (const char* e = getenv("CRTM_GPU_MAP_CHANNELS")) {
    const int v = atoi(e);
    if (v == 8 || v == 16 || v == 32) h->map_channels = v;
  }
  if (const char* e = getenv("CRTM_GPU_SOI_SLOTS")) {
    const int v = atoi(e);
    if (v >= 17 && v <= 75) h->soi_slots = v;
  }

  if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&h->order_event, cudaEventDisableTiming) != cudaSuccess) {
    delete h;
    return fail(nullptr, "cudaStreamCreate failed");
  }
  // load the device code (and with it the static scratch) on this device now
  static_scratch_slot(dev);
  h->sensors.resize(n_sensors);
  for (int i = 0; i < n_sensors; i++) {
    std::string err;
    if (!sensor_ids[i] || !load_sensor(coeff_path, sensor_ids[i], h->sensors[i], err)) {
      g_init_error = err.empty() ? "bad sensor id" : err;
      crtm_gpu_destroy(h);
      return CRTM_GPU_FAILURE;
    }
  }
  {
    // the cloud LUT is optional: without it, batches with clouds are refused
    const std::string cpath = std::string(coeff_path) + "/CloudCoeff.bin";
    FILE* f = fopen(cpath.c_str(), "rb");
    if (f) {
      fclose(f);
      std::vector<double> buf;
      int dims[7];
      size_t off[14];
      std::string err;
      if (!load_cloudcoeff(cpath, buf, dims, off, err)) {
        g_init_error = err;
        crtm_gpu_destroy(h);
        return CRTM_GPU_FAILURE;
      }
      // the radius and temperature axes' Lagrange reciprocals, after the tables
      const int rc_n[3] = {dims[1], dims[5], dims[2]};   // r_mw, r_ir, t
      const size_t rc_ax[3] = {off[2], off[3], off[4]};
      size_t rc_off[3];
      for (int a = 0; a < 3; a++) {
        rc_off[a] = buf.size();
        if (rc_n[a] >= 4) {
          buf.resize(buf.size() + (size_t)(rc_n[a] - 3) * 7);
          lagrange4_recip_table(buf.data() + rc_ax[a], rc_n[a], buf.data() + rc_off[a]);
        }
      }
      if (cudaMalloc(&h->d_cloud, buf.size() * sizeof(double)) != cudaSuccess ||
          cudaMemcpy(h->d_cloud, buf.data(), buf.size() * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess) {
        g_init_error = "device upload of CloudCoeff.bin failed";
        crtm_gpu_destroy(h);
        return CRTM_GPU_FAILURE;
      }
      CloudLut& L = h->lut;
      L.nfm = dims[0]; L.nrm = dims[1]; L.nt = dims[2]; L.nd = dims[3]; L.nfi = dims[4]; L.nri = dims[5];
      L.nleg = dims[6];
      const double* b0 = h->d_cloud;
      L.f_mw = b0 + off[0]; L.f_ir = b0 + off[1]; L.r_mw = b0 + off[2]; L.r_ir = b0 + off[3]; L.t = b0 + off[4];
      L.ke_l = b0 + off[5]; L.w_l = b0 + off[6]; L.pc_l = b0 + off[7];
      L.ke_s = b0 + off[8]; L.w_s = b0 + off[9]; L.pc_s = b0 + off[10];
      L.ke_ir = b0 + off[11]; L.w_ir = b0 + off[12]; L.pc_ir = b0 + off[13];
      L.rc_rmw = rc_n[0] >= 4 ? b0 + rc_off[0] : nullptr;
      L.rc_rir = rc_n[1] >= 4 ? b0 + rc_off[1] : nullptr;
      L.rc_t = rc_n[2] >= 4 ? b0 + rc_off[2] : nullptr;
      h->has_clouds = true;
      for (auto& s : h->sensors)
        if (!build_cloud_chan(h->lut, true, s, err)) {
          g_init_error = err;
          crtm_gpu_destroy(h);
          return CRTM_GPU_FAILURE;
        }
    }
    const std::string apath =
        std::string(coeff_path) + "/" + (aerosol_coeff_file ? aerosol_coeff_file : "AerosolCoeff.bin");
    FILE* fa = fopen(apath.c_str(), "rb");
    if (!fa && aerosol_coeff_file) {   // a named LUT must exist
      g_init_error = apath + ": cannot open";
      crtm_gpu_destroy(h);
      return CRTM_GPU_FAILURE;
    }
    if (fa) {
      fclose(fa);
      std::vector<double> abuf;
      std::vector<int> types;
      int adims[7];
      size_t aoff[7];
      std::string err;
      if (!load_aerosolcoeff(apath, scheme, abuf, types, adims, aoff, err)) {
        g_init_error = err;
        crtm_gpu_destroy(h);
        return CRTM_GPU_FAILURE;
      }
      // the axes' Lagrange reciprocals (radius and sigma per type), after the tables
      const int ant = adims[4], anr = adims[2], ans = adims[3];
      size_t ar_off[4] = {0, 0, 0, 0};
      auto add_rec = [&](size_t ax, int n, int rows) -> size_t {
        const size_t o = abuf.size();
        if (n < 4) return 0;
        abuf.resize(abuf.size() + (size_t)rows * (n - 3) * 7);
        for (int r = 0; r < rows; r++)
          lagrange4_recip_table(abuf.data() + ax + (size_t)r * n, n, abuf.data() + o + (size_t)r * (n - 3) * 7);
        return o;
      };
      ar_off[0] = add_rec(aoff[0], adims[0], 1);
      ar_off[1] = add_rec(aoff[1], anr, ant);
      ar_off[2] = add_rec(aoff[5], ans, ant);
      ar_off[3] = add_rec(aoff[6], adims[6], 1);
      if (cudaMalloc(&h->d_aero, abuf.size() * sizeof(double)) != cudaSuccess ||
          cudaMalloc(&h->d_aero_type, types.size() * sizeof(int)) != cudaSuccess ||
          cudaMemcpy(h->d_aero, abuf.data(), abuf.size() * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
          cudaMemcpy(h->d_aero_type, types.data(), types.size() * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess) {
        g_init_error = "device upload of AerosolCoeff.bin failed";
        crtm_gpu_destroy(h);
        return CRTM_GPU_FAILURE;
      }
      AerosolLut& A = h->alut;
      A.nw = adims[0]; A.nrh = adims[1]; A.nr = adims[2]; A.ns = adims[3]; A.nt = adims[4]; A.nleg = adims[5];
      A.nrh_axis = adims[6];
      A.scheme = scheme;
      A.type_id = h->d_aero_type;
      A.freq = h->d_aero + aoff[0]; A.reff = h->d_aero + aoff[1]; A.ke = h->d_aero + aoff[2];
      A.w = h->d_aero + aoff[3]; A.pc = h->d_aero + aoff[4]; A.rsig = h->d_aero + aoff[5];
      A.rh = h->d_aero + aoff[6];
      A.rc_freq = ar_off[0] ? h->d_aero + ar_off[0] : nullptr;
      A.rc_reff = ar_off[1] ? h->d_aero + ar_off[1] : nullptr;
      A.rc_rsig = ar_off[2] ? h->d_aero + ar_off[2] : nullptr;
      A.rc_rh = ar_off[3] ? h->d_aero + ar_off[3] : nullptr;
      h->has_aerosols = true;
    }
    const std::string wpath = std::string(coeff_path) + "/Nalli.IRwater.EmisCoeff.bin";
    if (FILE* fw = fopen(wpath.c_str(), "rb")) {   // the reference's default IRwaterCoeff_File
      fclose(fw);
      std::vector<double> wbuf;
      int wd[5];
      size_t wo[5];
      std::string err;
      if (!load_irwatercoeff(wpath, wbuf, wd, wo, err)) {
        g_init_error = err;
        crtm_gpu_destroy(h);
        return CRTM_GPU_FAILURE;
      }
      if (cudaMalloc(&h->d_irw, wbuf.size() * sizeof(double)) != cudaSuccess ||
          cudaMemcpy(h->d_irw, wbuf.data(), wbuf.size() * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess) {
        g_init_error = "device upload of Nalli.IRwater.EmisCoeff.bin failed";
        crtm_gpu_destroy(h);
        return CRTM_GPU_FAILURE;
      }
      IRWaterLut& W = h->irw;
      W.na = wd[0]; W.nf = wd[1]; W.nv = wd[2]; W.nt = wd[3]; W.nalli2 = wd[4];
      W.angle = h->d_irw + wo[0]; W.freq = h->d_irw + wo[1]; W.wind = h->d_irw + wo[2];
      W.temp = h->d_irw + wo[3]; W.e = h->d_irw + wo[4];
      h->has_irwater = true;
    }
    GaussTable gt;
    gauss_table_host(gt);
    if (cudaMemcpyToSymbol(c_gauss, &gt, sizeof gt) != cudaSuccess || scatter_k_set_gauss(gt) ||
        cudaMalloc(&h->d_error, sizeof(int)) != cudaSuccess) {
      g_init_error = "device set-up of the scattering tables failed";
      crtm_gpu_destroy(h);
      return CRTM_GPU_FAILURE;
    }
  }
  *handle = h;
  return CRTM_GPU_SUCCESS;
}

int crtm_gpu_destroy(crtm_gpu_handle h) {
  if (!h) return CRTM_GPU_SUCCESS;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  for (auto& s : h->sensors) free_sensor(s);
  h->ws.release(); h->io_in.release(); h->io_out.release(); h->small.release(); h->sfc.release();
  cudaFree(h->d_irw);
  cudaFree(h->d_cloud);
  cudaFree(h->d_aero);
  cudaFree(h->d_aero_type);
  cudaFree(h->d_error);
  collect_stage_times(h);
  if (h->order_event) {   // the last call's work, whatever stream it ran on
    cudaEventSynchronize(h->order_event);
    cudaEventDestroy(h->order_event);
  }
  for (auto e : h->event_pool) cudaEventDestroy(e);
  if (h->copy_stream) cudaStreamSynchronize(h->copy_stream);
  if (h->stream) cudaStreamDestroy(h->stream);
  if (h->copy_stream) cudaStreamDestroy(h->copy_stream);
  delete h;
  return CRTM_GPU_SUCCESS;
}

int crtm_gpu_n_channels(crtm_gpu_handle h, int sensor) {
  if (!h || sensor < 0 || sensor >= (int)h->sensors.size()) return -1;
  return h->sensors[sensor].L;
}

int crtm_gpu_set_channel_subset(crtm_gpu_handle h, int sensor, int n, const int* channel_index) {
  if (!h) return CRTM_GPU_FAILURE;
  if (sensor < 0 || sensor >= (int)h->sensors.size()) return fail(h, "sensor index %d out of range", sensor);
  if (cudaSetDevice(h->device) != cudaSuccess) return fail(h, "cudaSetDevice failed");
  Sensor& s = h->sensors[sensor];
  std::vector<int> pos;
  if (n >= 0) {
    if (n > 0 && !channel_index) return fail(h, "missing channel subset");
    if (n > s.L_all) return fail(h, "channel subset of %d channels for a sensor of %d", n, s.L_all);
    pos.assign(channel_index, channel_index + n);
    std::sort(pos.begin(), pos.end());
    for (int i = 0; i < n; i++) {
      if (pos[i] < 0 || pos[i] >= s.L_all)
        return fail(h, "channel subset index %d out of range [0, %d)", pos[i], s.L_all);
      if (i > 0 && pos[i] == pos[i - 1]) return fail(h, "channel %d given twice in the subset", pos[i]);
    }
    if (n == 0) pos.push_back(-1);   // marker: no channels
  }
  // wait for calls in flight on the handle's stream before the tables change
  if (cudaStreamSynchronize(h->stream) != cudaSuccess) return fail(h, "stream synchronisation failed");
  if (h->lin.sensor == sensor) h->lin.valid = false;   // its Jacobians have the old channels
  std::string err;
  if (!pos.empty() && pos[0] == -1) {
    s.L = 0;
    s.processed = pos;
    build_cloud_chan(h->lut, false, s, err);
    return CRTM_GPU_SUCCESS;
  }
  if (!upload_channels(s, pos, err)) return fail(h, "%s", err.c_str());
  if (!build_cloud_chan(h->lut, h->has_clouds, s, err)) return fail(h, "%s", err.c_str());
  return CRTM_GPU_SUCCESS;
}

int crtm_gpu_get_channel_subset(crtm_gpu_handle h, int sensor, int capacity, int* channel_index) {
  if (!h || sensor < 0 || sensor >= (int)h->sensors.size()) return -1;
  const Sensor& s = h->sensors[sensor];
  for (int l = 0; l < s.L && channel_index && l < capacity; l++)
    channel_index[l] = s.processed.empty() ? l : s.processed[l];
  return s.L;
}

int crtm_gpu_set_precision(crtm_gpu_handle h, int precision) {
  if (!h) return CRTM_GPU_FAILURE;
  if (precision != CRTM_GPU_FP64 && precision != CRTM_GPU_MIXED) return fail(h, "unknown precision %d", precision);
  h->precision = precision;
  return CRTM_GPU_SUCCESS;
}

int crtm_gpu_forward(crtm_gpu_handle h, int sensor, const crtm_gpu_batch* b, crtm_gpu_rtsolution* rts) {
  if (!rts) return fail(h, "missing RTSolution");
  return host_call(h, sensor, b, 0, nullptr, nullptr, nullptr, rts);
}

int crtm_gpu_k_matrix(crtm_gpu_handle h, int sensor, const crtm_gpu_batch* b, const double* bt_k,
                      crtm_gpu_kmatrix* k, crtm_gpu_rtsolution* rts) {
  if (!rts || !k) return fail(h, "missing K-matrix or RTSolution outputs");
  return host_call(h, sensor, b, 1, bt_k, k, nullptr, rts);
}

int crtm_gpu_adjoint(crtm_gpu_handle h, int sensor, const crtm_gpu_batch* b, const double* bt_ad,
                     crtm_gpu_adjoint_out* ad, crtm_gpu_rtsolution* rts) {
  if (!rts || !ad || !bt_ad) return fail(h, "missing adjoint seed or outputs");
  return host_call(h, sensor, b, 2, bt_ad, nullptr, ad, rts);
}

int crtm_gpu_tangent_linear(crtm_gpu_handle h, int sensor, const crtm_gpu_batch* b, const crtm_gpu_tl_in* tl,
                            crtm_gpu_rtsolution* rts, double* bt_tl) {
  return tl_host(h, sensor, b, tl, rts, bt_tl);
}

int crtm_gpu_tangent_linear_device(crtm_gpu_handle h, int sensor, const crtm_gpu_batch* b,
                                   const crtm_gpu_tl_in* tl, crtm_gpu_rtsolution* rts, double* bt_tl,
                                   void* stream) {
  if (!rts || !rts->radiance || !rts->brightness_temperature) return fail(h, "missing RTSolution buffers");
  return tl_device(h, sensor, b, tl, rts, bt_tl, (cudaStream_t)stream);
}

int crtm_gpu_linearize(crtm_gpu_handle h, int sensor, const crtm_gpu_batch* b, crtm_gpu_rtsolution* rts,
                       void* stream) {
  return linearize(h, sensor, b, rts, nullptr, (cudaStream_t)stream);
}

int crtm_gpu_tangent_linear_apply(crtm_gpu_handle h, const crtm_gpu_tl_in* tl, double* bt_tl, void* stream) {
  return tl_apply(h, tl, bt_tl, (cudaStream_t)stream);
}

int crtm_gpu_adjoint_apply(crtm_gpu_handle h, const double* bt_ad, crtm_gpu_adjoint_out* ad, void* stream) {
  return ad_apply(h, bt_ad, ad, (cudaStream_t)stream);
}

int crtm_gpu_forward_device(crtm_gpu_handle h, int sensor, const crtm_gpu_batch* b,
                            crtm_gpu_rtsolution* rts, void* stream) {
  return dispatch(h, sensor, b, 0, nullptr, rts, nullptr, nullptr,
                  (cudaStream_t)stream);
}

int crtm_gpu_k_matrix_device(crtm_gpu_handle h, int sensor, const crtm_gpu_batch* b,
                             const double* bt_k, crtm_gpu_kmatrix* k, crtm_gpu_rtsolution* rts,
                             void* stream) {
  return dispatch(h, sensor, b, 1, bt_k, rts, k, nullptr,
                  (cudaStream_t)stream);
}

int crtm_gpu_adjoint_device(crtm_gpu_handle h, int sensor, const crtm_gpu_batch* b,
                            const double* bt_ad, crtm_gpu_adjoint_out* ad, crtm_gpu_rtsolution* rts,
                            void* stream) {
  if (!bt_ad) return fail(h, "missing adjoint seed");
  return dispatch(h, sensor, b, 2, bt_ad, rts, nullptr, ad,
                  (cudaStream_t)stream);
}

// The K-matrix of crtm_gpu_k_matrix_device with its intermediates in
// g_static_scratch instead of the handle's grow-on-demand workspace.  Some
// callers cannot let a call allocate: a host model whose device memory is
// already held by its own caching allocator (a cudaMalloc here would fail or
// force that cache to be released), or an assimilation loop that calls the
// operator every iteration on a few profiles, where cudaMalloc and cudaFree
// would synchronise the whole device and stall its other streams.
//
// crtm_gpu_init looks up the scratch address on its device with that device
// current (cudaGetSymbolAddress); if that lookup has not happened on the
// handle's device, the first call here does it, and that first call should
// come before any stream capture.  Calls only enqueue kernels and one small
// copy of the absorber map.  Without a batch emissivity the IR sea-surface
// emissivity model's three [P][L] arrays are taken from the front of the
// scratch as well.  No part of the scratch is read before the same call's
// kernels write it, so nothing needs clearing between calls.  The scratch is
// shared by every handle on the device: two calls that overlap in time (on
// different streams, handles or host threads) overwrite each other's
// intermediates, so callers must order them (one stream, or events).
int crtm_gpu_k_matrix_device_static(crtm_gpu_handle h, int sensor, const crtm_gpu_batch* b,
                                    const double* bt_k, crtm_gpu_kmatrix* k,
                                    crtm_gpu_rtsolution* rts, void* stream) {
  if (!h) return CRTM_GPU_FAILURE;
  if (h->device < 0 || h->device >= MAX_STATIC_DEVICES)
    return fail(h, "device %d has no static scratch slot", h->device);
  if (cudaSetDevice(h->device) != cudaSuccess) return fail(h, "cudaSetDevice failed");
  const StaticScratchSlot* slot = static_scratch_slot(h->device);
  if (slot->err != cudaSuccess || !slot->ptr)
    return fail(h, "static scratch lookup failed: %s", cudaGetErrorString(slot->err));
  const FixedScratch fx{(char*)slot->ptr, STATIC_SCRATCH_BYTES};
  return dispatch(h, sensor, b, 1, bt_k, rts, k, nullptr,
                  (cudaStream_t)stream, nullptr, &fx);
}

int crtm_gpu_get_tuning(crtm_gpu_handle h, int sensor, int precision, crtm_gpu_tuning* out) {
  if (!h) return CRTM_GPU_FAILURE;
  if (sensor < 0 || sensor >= (int)h->sensors.size()) return fail(h, "sensor index %d out of range", sensor);
  if (precision != CRTM_GPU_FP64 && precision != CRTM_GPU_MIXED) return fail(h, "unknown precision %d", precision);
  if (!out) return fail(h, "missing tuning output");
  const Sensor& s = h->sensors[sensor];
  const int f = precision == CRTM_GPU_MIXED ? 1 : 0;
  out->map_channels = s.tune_map[f] > 0 ? s.tune_map[f] : h->map_channels;
  out->chunk_profiles = s.tune_chunk[f];
  out->ms_per_call = s.tune_ms[f];
  return CRTM_GPU_SUCCESS;
}

int crtm_gpu_set_tuning(crtm_gpu_handle h, int sensor, int precision, const crtm_gpu_tuning* t) {
  if (!h) return CRTM_GPU_FAILURE;
  if (sensor < 0 || sensor >= (int)h->sensors.size()) return fail(h, "sensor index %d out of range", sensor);
  if (precision != CRTM_GPU_FP64 && precision != CRTM_GPU_MIXED) return fail(h, "unknown precision %d", precision);
  if (!t) return fail(h, "missing tuning");
  if (t->map_channels != 0 && t->map_channels != 8 && t->map_channels != 16 && t->map_channels != 32)
    return fail(h, "map_channels must be 0, 8, 16 or 32 (got %d)", t->map_channels);
  if (t->chunk_profiles < 0) return fail(h, "chunk_profiles must be >= 0 (got %d)", t->chunk_profiles);
  Sensor& s = h->sensors[sensor];
  const int f = precision == CRTM_GPU_MIXED ? 1 : 0;
  s.tune_map[f] = t->map_channels;
  s.tune_chunk[f] = t->chunk_profiles;
  s.tune_ms[f] = 0.0;
  return CRTM_GPU_SUCCESS;
}

// Times the K-matrix of this batch (device buffers, as
// crtm_gpu_k_matrix_device) under each candidate tuning and keeps the
// fastest for the sensor and the arithmetic form the call runs in.
// Candidates: 16, 8 and 32 channels per map CTA, each with no cap on the
// profiles per pipeline pass, with P/2 and with P/4.  Each candidate runs
// once untimed (workspace growth, shared-memory attributes), then `reps`
// times between two CUDA events on `stream`.  The per-output arithmetic of
// the pipeline does not depend on either setting, so every trial writes the
// same K-matrix and RTSolution; the outputs hold it when the call returns.
int crtm_gpu_autotune_k_matrix_device(crtm_gpu_handle h, int sensor, const crtm_gpu_batch* b,
                                      const double* bt_k, crtm_gpu_kmatrix* k,
                                      crtm_gpu_rtsolution* rts, void* stream, int reps,
                                      crtm_gpu_tuning* trials, int max_trials, int* n_trials,
                                      crtm_gpu_tuning* chosen) {
  if (!h) return CRTM_GPU_FAILURE;
  if (sensor < 0 || sensor >= (int)h->sensors.size()) return fail(h, "sensor index %d out of range", sensor);
  if (!b || b->n_profiles < 1) return fail(h, "autotune needs a batch of at least one profile");
  if (reps < 1 || reps > 1000) return fail(h, "reps must be in 1..1000 (got %d)", reps);
  if (cudaSetDevice(h->device) != cudaSuccess) return fail(h, "cudaSetDevice failed");
  const cudaStream_t st = (cudaStream_t)stream;
  const bool scat = b->max_clouds > 0 || b->max_aerosols > 0;
  // the form dispatch runs the K-matrix in (batches with clouds or aerosols: FP64)
  const int f = (h->precision == CRTM_GPU_MIXED && !scat) ? 1 : 0;
  Sensor& s = h->sensors[sensor];
  const int old_map = s.tune_map[f], old_chunk = s.tune_chunk[f];
  const double old_ms = s.tune_ms[f];
  const int P = b->n_profiles;
  std::vector<std::pair<int, int>> cand;
  for (int mc : {16, 8, 32}) {
    int last = -1;
    for (int cap : {0, (P + 1) / 2, (P + 3) / 4}) {
      if (cap >= P) cap = 0;   // a cap at or above the batch is no cap
      if (cap == last) continue;
      cand.emplace_back(mc, cap);
      last = cap;
    }
  }
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    if (e0) cudaEventDestroy(e0);
    return fail(h, "cudaEventCreate failed");
  }
  int best = -1;
  double best_ms = 0.0;
  int rc = CRTM_GPU_SUCCESS;
  int n = 0;
  for (size_t i = 0; i < cand.size(); i++) {
    s.tune_map[f] = cand[i].first;
    s.tune_chunk[f] = cand[i].second;
    rc = dispatch(h, sensor, b, 1, bt_k, rts, k, nullptr, st);
    if (rc != CRTM_GPU_SUCCESS) break;
    if (cudaEventRecord(e0, st) != cudaSuccess) { rc = fail(h, "cudaEventRecord failed"); break; }
    for (int r = 0; r < reps && rc == CRTM_GPU_SUCCESS; r++) rc = dispatch(h, sensor, b, 1, bt_k, rts, k, nullptr, st);
    if (rc != CRTM_GPU_SUCCESS) break;
    float ms = 0.0f;
    if (cudaEventRecord(e1, st) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
        cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
      rc = fail(h, "timing the trial failed: %s", cudaGetErrorString(cudaGetLastError()));
      break;
    }
    const double per = (double)ms / reps;
    if (trials && n < max_trials) trials[n] = crtm_gpu_tuning{cand[i].first, cand[i].second, per};
    n++;
    if (best < 0 || per < best_ms) { best = (int)i; best_ms = per; }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (n_trials) *n_trials = n;
  if (rc != CRTM_GPU_SUCCESS || best < 0) {
    s.tune_map[f] = old_map;
    s.tune_chunk[f] = old_chunk;
    s.tune_ms[f] = old_ms;
    return rc != CRTM_GPU_SUCCESS ? rc : fail(h, "autotune ran no trial");
  }
  s.tune_map[f] = cand[best].first;
  s.tune_chunk[f] = cand[best].second;
  s.tune_ms[f] = best_ms;
  if (chosen) *chosen = crtm_gpu_tuning{cand[best].first, cand[best].second, best_ms};
  return CRTM_GPU_SUCCESS;
}

int crtm_gpu_last_error(crtm_gpu_handle h, char* buf, int n) {
  const std::string& e = h ? h->error : g_init_error;
  if (buf && n > 0) {
    snprintf(buf, (size_t)n, "%s", e.c_str());
  }
  return (int)e.size();
}

long long crtm_gpu_launch_count(crtm_gpu_handle h) { return h ? h->launches : 0; }

int crtm_gpu_set_profiling(crtm_gpu_handle h, int enable) {
  if (!h) return CRTM_GPU_FAILURE;
  h->profiling = enable != 0;
  return CRTM_GPU_SUCCESS;
}

int crtm_gpu_stage_times(crtm_gpu_handle h, double* ms, long long* launches, int n, int reset) {
  if (!h) return 0;
  cudaSetDevice(h->device);
  collect_stage_times(h);
  const int N = crtm_gpu_context::N_STAGES;
  for (int i = 0; i < n && i < N; i++) {
    if (ms) ms[i] = h->stage_ms[i];
    if (launches) launches[i] = h->stage_n[i];
  }
  if (reset)
    for (int i = 0; i < N; i++) { h->stage_ms[i] = 0.0; h->stage_n[i] = 0; }
  return N;
}

}  // extern "C"
