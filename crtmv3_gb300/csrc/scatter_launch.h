// Host launchers of the scattering K-matrix/adjoint kernels.  They live in
// their own translation units, one per (angle capacity, working precision):
// scatter_k_{f,d}5.cu for the stream rule's 2-6 streams, scatter_k_{f,d}10.cu
// for Options%n_Streams up to 16; the units compile in parallel with the rest
// of the library.
#pragma once

#include <cuda_runtime.h>

namespace crtm {

struct GaussTable;
template <class R> struct ScatterArgs;

// Upload the Gauss table into each unit's constant memory; 0 on success.
int scatter_k_f5_set_gauss(const GaussTable& g);
int scatter_k_d5_set_gauss(const GaussTable& g);
int scatter_k_f10_set_gauss(const GaussTable& g);
int scatter_k_d10_set_gauss(const GaussTable& g);
inline int scatter_k_set_gauss(const GaussTable& g) {
  return scatter_k_f5_set_gauss(g) | scatter_k_d5_set_gauss(g) | scatter_k_f10_set_gauss(g) |
         scatter_k_d10_set_gauss(g);
}

template <int NZ, class R>
void launch_scatter_layers_k(const ScatterArgs<R>& a, unsigned grid, cudaStream_t st);
template <int NZ, class R>
void launch_scatter_kmatrix(const ScatterArgs<R>& a, dim3 grid, cudaStream_t st);
template <int NZ, class R>
void launch_scatter_contract(const ScatterArgs<R>& a, unsigned grid, cudaStream_t st);

}  // namespace crtm
