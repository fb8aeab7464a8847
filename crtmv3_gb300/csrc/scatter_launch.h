// Host launchers of the scattering K-matrix/adjoint kernels.  R is the gas
// optics' arithmetic (double in the FP64 form, float in the mixed form), C
// the layer solver's (the same); the adding and its adjoint are FP64 in both.
// A batch with SOI profiles runs in the FP64 form.  Translation units per
// angle capacity (d5: the stream rule's 2-6 streams, d10: Options%n_Streams
// up to 16): scatter_k_*.cu (records, adding adjoint, reverse sweep of the ADA
// layers; the f units for the mixed form) and scatter_soi_*.cu (the SOI
// layers' derivative-number contraction); they compile in parallel.
#pragma once

#include <cuda_runtime.h>

namespace crtm {

struct GaussTable;
template <class R> struct ScatterArgs;

// Upload the Gauss table into each unit's constant memory; 0 on success.
int scatter_k_d5_set_gauss(const GaussTable& g);
int scatter_k_d10_set_gauss(const GaussTable& g);
int scatter_k_d5f_set_gauss(const GaussTable& g);
int scatter_k_d10f_set_gauss(const GaussTable& g);
int scatter_soi_d5_set_gauss(const GaussTable& g);
int scatter_soi_d10_set_gauss(const GaussTable& g);
inline int scatter_k_set_gauss(const GaussTable& g) {
  return scatter_k_d5_set_gauss(g) | scatter_k_d10_set_gauss(g) | scatter_k_d5f_set_gauss(g) |
         scatter_k_d10f_set_gauss(g) | scatter_soi_d5_set_gauss(g) | scatter_soi_d10_set_gauss(g);
}

// layer records (in R) with the layer solver in C
template <int NZ, class R, class C>
void launch_scatter_layers_k(const ScatterArgs<R>& a, unsigned grid, cudaStream_t st);
// the ADA adding adjoint, then (FP64 form, soi) the SOI orders' adjoint of the SOI profiles
template <int NZ, class R>
void launch_scatter_kmatrix(const ScatterArgs<R>& a, dim3 grid, cudaStream_t st, bool soi);
// the ADA profiles' layer contraction (reverse sweep in C)
template <int NZ, class R, class C>
void launch_scatter_reverse(const ScatterArgs<R>& a, unsigned grid, cudaStream_t st);
// the SOI profiles' layer contraction (derivative numbers, FP64 form)
template <int NZ, class C>
void launch_scatter_contract(const ScatterArgs<double>& a, unsigned grid, cudaStream_t st);

}  // namespace crtm
