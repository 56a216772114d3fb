// Pooled transport kernels, FP32 tracking, surface tracking: compiled with the
// same fast single-precision math as the surface-tracking history kernel
// (transport_mixed_surface.cu), so the two give the same FP32 results.
#include "transport_pool.cuh"
#include "launch.h"

namespace abx {

template __global__ void transport_pool_kernel<float, ABX_TRACK_SURFACE, false>(const __grid_constant__ TransportArgs<float>);
template __global__ void transport_pool_kernel<float, ABX_TRACK_SURFACE, true>(const __grid_constant__ TransportArgs<float>);

void launch_pool_f_surface(const TransportArgs<float>& A, bool iso, int grid, int block, cudaStream_t s) {
  if (iso) transport_pool_kernel<float, ABX_TRACK_SURFACE, true><<<grid, block, 0, s>>>(A);
  else transport_pool_kernel<float, ABX_TRACK_SURFACE, false><<<grid, block, 0, s>>>(A);
}

int occupancy_pool_f_surface(bool iso, int block) {
  int nb = 0;
  if (iso) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, transport_pool_kernel<float, ABX_TRACK_SURFACE, true>, block, 0);
  else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, transport_pool_kernel<float, ABX_TRACK_SURFACE, false>, block, 0);
  return nb;
}

}  // namespace abx
