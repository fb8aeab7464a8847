// Scattering K-matrix/adjoint kernels for NZ = 10 angles (Options%n_Streams up to 16), FP64:
// the layer records, the adding adjoint (and the SOI orders' adjoint), and
// the reverse sweep through the ADA layers' optics.  One translation unit per
// angle capacity so that the library compiles in parallel.
#include "scatter_kernels.cuh"
#include "scatter_launch.h"

namespace crtm {

int scatter_k_d10_set_gauss(const GaussTable& g) {
  return cudaMemcpyToSymbol(c_gauss, &g, sizeof g) == cudaSuccess ? 0 : 1;
}

template <int NZ, class C>
void launch_scatter_layers_k(const ScatterArgs<double>& a, unsigned grid, cudaStream_t st) {
  scatter_layers_kernel<NZ, double, double, C><<<grid, SCATTER_THREADS, 0, st>>>(a, a.LBK);
}

template <int NZ>
void launch_scatter_kmatrix(const ScatterArgs<double>& a, dim3 grid, cudaStream_t st, bool soi) {
  scatter_kmatrix_kernel<NZ, double><<<grid, SCATTER_THREADS, 0, st>>>(a);
  if (soi) scatter_soi_k_kernel<NZ><<<grid, SCATTER_THREADS, 0, st>>>(a);
}

template <int NZ, class C>
void launch_scatter_reverse(const ScatterArgs<double>& a, unsigned grid, cudaStream_t st) {
  scatter_reverse_kernel<NZ, double, C><<<grid, SCATTER_THREADS, 0, st>>>(a);
}

template void launch_scatter_layers_k<10, double>(const ScatterArgs<double>&, unsigned, cudaStream_t);
template void launch_scatter_kmatrix<10>(const ScatterArgs<double>&, dim3, cudaStream_t, bool);
template void launch_scatter_reverse<10, double>(const ScatterArgs<double>&, unsigned, cudaStream_t);

}  // namespace crtm
