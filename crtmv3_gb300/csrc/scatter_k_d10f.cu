// Scattering K-matrix/adjoint kernels for NZ = 10 angles (Options%n_Streams up to 16), mixed form (FP32 gas optics and layer solver, FP64 adding):
// the layer records, the adding adjoint (and, FP64 form, the SOI orders'
// adjoint), and the reverse sweep through the ADA layers' optics.  One
// translation unit per angle capacity and form so that the library compiles
// in parallel.
#include "scatter_kernels.cuh"
#include "scatter_launch.h"

namespace crtm {

int scatter_k_d10f_set_gauss(const GaussTable& g) {
  return cudaMemcpyToSymbol(c_gauss, &g, sizeof g) == cudaSuccess ? 0 : 1;
}

template <int NZ, class R, class C>
void launch_scatter_layers_k(const ScatterArgs<R>& a, unsigned grid, cudaStream_t st) {
  scatter_layers_kernel<NZ, R, R, C><<<grid, SCATTER_THREADS, 0, st>>>(a, a.LBK);
}

template <int NZ, class R>
void launch_scatter_kmatrix(const ScatterArgs<R>& a, dim3 grid, cudaStream_t st, bool soi) {
  scatter_kmatrix_kernel<NZ, R><<<grid, SCATTER_THREADS, 0, st>>>(a);
  if constexpr (std::is_same<R, double>::value)
    if (soi) scatter_soi_k_kernel<NZ><<<grid, SCATTER_THREADS, 0, st>>>(a);
}

template <int NZ, class R, class C>
void launch_scatter_reverse(const ScatterArgs<R>& a, unsigned grid, cudaStream_t st) {
  scatter_reverse_kernel<NZ, R, C><<<grid, SCATTER_THREADS, 0, st>>>(a);
}

template void launch_scatter_layers_k<10, float, float>(const ScatterArgs<float>&, unsigned, cudaStream_t);
template void launch_scatter_kmatrix<10, float>(const ScatterArgs<float>&, dim3, cudaStream_t, bool);
template void launch_scatter_reverse<10, float, float>(const ScatterArgs<float>&, unsigned, cudaStream_t);

}  // namespace crtm
