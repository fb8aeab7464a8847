// Host launchers of the scattering K-matrix/adjoint kernels.  The K-matrix
// and adjoint of a batch with clouds or aerosols run the gas optics and the
// layer solver in FP64 in both forms (ScatterArgs<double>, C = double).  Two
// translation units per angle capacity (d5: the stream rule's 2-6 streams,
// d10: Options%n_Streams up to 16): scatter_k_*.cu (records, adding adjoint,
// reverse sweep of the ADA layers) and scatter_soi_*.cu (the SOI layers'
// derivative-number contraction); they compile in parallel with the rest of
// the library.
#pragma once

#include <cuda_runtime.h>

namespace crtm {

struct GaussTable;
template <class R> struct ScatterArgs;

// Upload the Gauss table into each unit's constant memory; 0 on success.
int scatter_k_d5_set_gauss(const GaussTable& g);
int scatter_k_d10_set_gauss(const GaussTable& g);
int scatter_soi_d5_set_gauss(const GaussTable& g);
int scatter_soi_d10_set_gauss(const GaussTable& g);
inline int scatter_k_set_gauss(const GaussTable& g) {
  return scatter_k_d5_set_gauss(g) | scatter_k_d10_set_gauss(g) | scatter_soi_d5_set_gauss(g) |
         scatter_soi_d10_set_gauss(g);
}

template <int NZ, class C>
void launch_scatter_layers_k(const ScatterArgs<double>& a, unsigned grid, cudaStream_t st);
// the ADA adding adjoint, then (soi) the SOI orders' adjoint of the SOI profiles
template <int NZ>
void launch_scatter_kmatrix(const ScatterArgs<double>& a, dim3 grid, cudaStream_t st, bool soi);
// the ADA profiles' layer contraction (reverse sweep)
template <int NZ, class C>
void launch_scatter_reverse(const ScatterArgs<double>& a, unsigned grid, cudaStream_t st);
// the SOI profiles' layer contraction (derivative numbers)
template <int NZ, class C>
void launch_scatter_contract(const ScatterArgs<double>& a, unsigned grid, cudaStream_t st);

}  // namespace crtm
