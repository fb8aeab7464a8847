// SOI profiles' layer contraction for NZ = 10 angles (Options%n_Streams up to 16): each
// layer's optics (LUT, combine, phase, SOI doubling) on derivative numbers,
// contracted with the record adjoints.  Its own translation unit: it is the
// slowest to compile and builds in parallel with the rest.
#include "scatter_kernels.cuh"
#include "scatter_launch.h"

namespace crtm {

int scatter_soi_d10_set_gauss(const GaussTable& g) {
  return cudaMemcpyToSymbol(c_gauss, &g, sizeof g) == cudaSuccess ? 0 : 1;
}

template <int NZ, class C>
void launch_scatter_contract(const ScatterArgs<double>& a, unsigned grid, cudaStream_t st) {
  scatter_contract_kernel<NZ, double, C><<<grid, SCATTER_THREADS, 0, st>>>(a);
}

template void launch_scatter_contract<10, double>(const ScatterArgs<double>&, unsigned, cudaStream_t);

}  // namespace crtm
