// Cloudy forward kernel: one thread per (profile, channel) runs the cloud
// optics, the combine, the phase matrices and the ADA adding method
// (scatter_physics.cuh) over the profile's layers, from the gas layer optical
// depths the column kernel stored.  The scattering arithmetic is FP64 in
// every form: the reference keeps its matrix inversions and thin-layer
// initialisation in FP64.
#pragma once

#include "odps_kernels.cuh"
#include "scatter_physics.cuh"

namespace crtm {

__constant__ GaussTable c_gauss;

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
  const R* TAU;                 // [n][Kmax][L] gas layer optical depths
  double* radiance, *bt;        // [P][L]
  int* status;                  // [P] or null
  int* error;                   // first failing code (device), 0 if none
};

constexpr int SCATTER_THREADS = 128;

template <int NZ, class R>
__global__ void __launch_bounds__(SCATTER_THREADS) scatter_kernel(ScatterArgs<R> a) {
  __shared__ double s_maxreff;
  const int L = a.L, Kmax = a.Kmax;
  const int p = blockIdx.y, gp = a.p_begin + p;
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  const int st = a.pv.status[p];
  const int Ku = a.b.n_layers[gp];
  const int nc = a.n_clouds[gp];
  // largest effective radius of the profile's clouds (stream rule input)
  if (threadIdx.x == 0) s_maxreff = 0.0;
  __syncthreads();
  if (st == 0 && nc > 0) {
    double mr = 0.0;
    const double* rp = a.reff + (size_t)gp * a.max_clouds * Kmax;
    for (int i = threadIdx.x; i < nc * Ku; i += blockDim.x) {
      const double r = rp[(size_t)(i / Ku) * Kmax + (i % Ku)];
      mr = r > mr ? r : mr;
    }
    for (int o = 16; o > 0; o >>= 1) {
      const double v = __shfl_xor_sync(FULL, mr, o);
      mr = v > mr ? v : mr;
    }
    if ((threadIdx.x & 31) == 0 && mr > 0.0) {
      // non-negative doubles order like their bit patterns
      atomicMax(reinterpret_cast<unsigned long long*>(&s_maxreff), (unsigned long long)__double_as_longlong(mr));
    }
  }
  __syncthreads();
  if (l >= L) return;
  const size_t pl = (size_t)gp * L + l;
  if (st != 0) {
    a.radiance[pl] = 0.0;
    a.bt[pl] = 0.0;
    return;
  }
  const double c1 = a.sp.c1[l], c2 = a.sp.c2[l], b1 = a.sp.b1[l], b2 = a.sp.b2[l];
  const double e = a.b.emissivity[pl];
  const double ts = a.b.land_cov[gp] * a.b.land_t[gp] + a.b.water_cov[gp] * a.b.water_t[gp] +
                    a.b.snow_cov[gp] * a.b.snow_t[gp] + a.b.ice_cov[gp] * a.b.ice_t[gp];
  const double Bs = c1 / (exp(c2 / (b1 + b2 * ts)) - 1.0);
  const double mu = a.pv.scal[(size_t)p * 4 + 1];
  const double* tu = a.b.temperature + (size_t)gp * Kmax;
  const R* tau = a.TAU + (size_t)p * Kmax * L + l;
  double rad = 0.0;
  int code = 0;
  if (nc == 0) {   // clear profile: Emission solver, in FP64 here
    const double inv_u = 1.0 / mu;
    double down = a.sp.cbr[l], tr_tot = 1.0, src = 0.0;
    for (int k = 0; k < Ku; k++) {
      const double t = exp(-double(tau[(size_t)k * L]) * inv_u);
      const double B = c1 / (exp(c2 / (b1 + b2 * tu[k])) - 1.0);
      src += tr_tot * B * (1.0 - t);
      down = down * t + B * (1.0 - t);
      tr_tot *= t;
    }
    rad = src + tr_tot * (e * Bs + (1.0 - e) * down);
  } else {
    CloudyColumn c;
    c.Ku = Ku;
    c.n_clouds = nc;
    const int ns = a.n_streams ? a.n_streams[gp] : 0;
    c.nleg = ns > 0 ? ns : stream_rule_nleg(s_maxreff, a.sp.wn[l]);
    c.microwave = a.microwave != 0;
    c.freq = a.microwave ? a.sp.freq[l] : a.sp.wn[l];
    c.mu_sensor = mu;
    c.emissivity = e;
    c.planck_surface = Bs;
    c.cosmic = a.sp.cbr[l];
    c.c1 = c1; c.c2 = c2; c.b1 = b1; c.b2 = b2;
    c.temperature = tu;
    c.cloud_type = a.cloud_type + (size_t)gp * a.max_clouds;
    c.wc = a.wc + (size_t)gp * a.max_clouds * Kmax;
    c.reff = a.reff + (size_t)gp * a.max_clouds * Kmax;
    c.cstride = (size_t)Kmax;
    code = cloudy_radiance<NZ>(c, a.lut, c_gauss, [&](int k) { return double(tau[(size_t)k * L]); }, &rad);
  }
  if (code) {
    atomicCAS(a.error, 0, code);
    if (a.status) atomicOr(a.status + gp, 1 << 4);
    rad = 0.0;
  }
  a.radiance[pl] = rad;
  a.bt[pl] = code ? 0.0 : planck_temperature(c1, c2, b1, b2, rad);
}

}  // namespace crtm
