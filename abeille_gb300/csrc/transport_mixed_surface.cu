// Mixed-precision translation unit, surface tracking (the delta-tracking
// kernels and the launch dispatch are in transport_mixed.cu).
#include "transport_loop.cuh"
#include "launch.h"

namespace abx {

template __global__ void transport_kernel<float, ABX_TRACK_SURFACE, false>(const __grid_constant__ TransportArgs<float>);
template __global__ void transport_kernel<float, ABX_TRACK_SURFACE, true>(const __grid_constant__ TransportArgs<float>);

void launch_transport_f_surface(const TransportArgs<float>& A, bool iso, int grid, int block, cudaStream_t s) {
  if (iso) transport_kernel<float, ABX_TRACK_SURFACE, true><<<grid, block, 0, s>>>(A);
  else transport_kernel<float, ABX_TRACK_SURFACE, false><<<grid, block, 0, s>>>(A);
}

int occupancy_f_surface(bool iso, int block) {
  int nb = 0;
  if (iso) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, transport_kernel<float, ABX_TRACK_SURFACE, true>, block, 0);
  else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, transport_kernel<float, ABX_TRACK_SURFACE, false>, block, 0);
  return nb;
}

int transport_regs_f_surface() {
  cudaFuncAttributes a;
  cudaFuncGetAttributes(&a, transport_kernel<float, ABX_TRACK_SURFACE, false>);
  return a.numRegs;
}

}  // namespace abx
