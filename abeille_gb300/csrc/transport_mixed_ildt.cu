// Mixed-precision translation unit, implicit-leakage delta tracking (the
// delta-tracking kernels and the launch dispatch are in transport_mixed.cu).
#include "transport_loop.cuh"
#include "launch.h"

namespace abx {

template __global__ void transport_kernel<float, ABX_TRACK_IMPLICIT_LEAKAGE, false>(
    const __grid_constant__ TransportArgs<float>);
template __global__ void transport_kernel<float, ABX_TRACK_IMPLICIT_LEAKAGE, true>(
    const __grid_constant__ TransportArgs<float>);

void launch_transport_f_ildt(const TransportArgs<float>& A, bool iso, int grid, int block, cudaStream_t s) {
  if (iso) transport_kernel<float, ABX_TRACK_IMPLICIT_LEAKAGE, true><<<grid, block, 0, s>>>(A);
  else transport_kernel<float, ABX_TRACK_IMPLICIT_LEAKAGE, false><<<grid, block, 0, s>>>(A);
}

int occupancy_f_ildt(bool iso, int block) {
  int nb = 0;
  if (iso)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, transport_kernel<float, ABX_TRACK_IMPLICIT_LEAKAGE, true>,
                                                  block, 0);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, transport_kernel<float, ABX_TRACK_IMPLICIT_LEAKAGE, false>,
                                                  block, 0);
  return nb;
}

}  // namespace abx
