// Mixed-precision translation unit: the branchless collisions of the
// branchless k-eigenvalue simulation, with delta and surface tracking (the
// branching kernels are in transport_mixed.cu and transport_mixed_surface.cu).
#include "transport_loop.cuh"
#include "launch.h"

namespace abx {

constexpr int BL_DELTA = ABX_TRACK_DELTA | ABX_KERNEL_BRANCHLESS;
constexpr int BL_SURFACE = ABX_TRACK_SURFACE | ABX_KERNEL_BRANCHLESS;

template __global__ void transport_kernel<float, BL_DELTA, false>(const __grid_constant__ TransportArgs<float>);
template __global__ void transport_kernel<float, BL_DELTA, true>(const __grid_constant__ TransportArgs<float>);
template __global__ void transport_kernel<float, BL_SURFACE, false>(const __grid_constant__ TransportArgs<float>);
template __global__ void transport_kernel<float, BL_SURFACE, true>(const __grid_constant__ TransportArgs<float>);

void launch_transport_f_branchless(const TransportArgs<float>& A, int tracking, bool iso, int grid, int block,
                                   cudaStream_t s) {
  if (tracking == ABX_TRACK_SURFACE) {
    if (iso) transport_kernel<float, BL_SURFACE, true><<<grid, block, 0, s>>>(A);
    else transport_kernel<float, BL_SURFACE, false><<<grid, block, 0, s>>>(A);
  } else {
    if (iso) transport_kernel<float, BL_DELTA, true><<<grid, block, 0, s>>>(A);
    else transport_kernel<float, BL_DELTA, false><<<grid, block, 0, s>>>(A);
  }
}

int occupancy_f_branchless(int tracking, bool iso, int block) {
  int nb = 0;
  if (tracking == ABX_TRACK_SURFACE) {
    if (iso) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, transport_kernel<float, BL_SURFACE, true>, block, 0);
    else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, transport_kernel<float, BL_SURFACE, false>, block, 0);
  } else {
    if (iso) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, transport_kernel<float, BL_DELTA, true>, block, 0);
    else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, transport_kernel<float, BL_DELTA, false>, block, 0);
  }
  return nb;
}

}  // namespace abx
