// Mixed-precision translation unit, the other delta-tracking transporters:
// implicit-leakage delta tracking and Carter tracking (delta tracking and the
// launch dispatch are in transport_mixed.cu).
#include "transport_loop.cuh"
#include "launch.h"

namespace abx {

template __global__ void transport_kernel<float, ABX_TRACK_IMPLICIT_LEAKAGE, false>(
    const __grid_constant__ TransportArgs<float>);
template __global__ void transport_kernel<float, ABX_TRACK_IMPLICIT_LEAKAGE, true>(
    const __grid_constant__ TransportArgs<float>);
template __global__ void transport_kernel<float, ABX_TRACK_CARTER, false>(const __grid_constant__ TransportArgs<float>);
template __global__ void transport_kernel<float, ABX_TRACK_CARTER, true>(const __grid_constant__ TransportArgs<float>);

void launch_transport_f_variant(const TransportArgs<float>& A, int tracking, bool iso, int grid, int block,
                                cudaStream_t s) {
  if (tracking == ABX_TRACK_CARTER) {
    if (iso) transport_kernel<float, ABX_TRACK_CARTER, true><<<grid, block, 0, s>>>(A);
    else transport_kernel<float, ABX_TRACK_CARTER, false><<<grid, block, 0, s>>>(A);
  } else {
    if (iso) transport_kernel<float, ABX_TRACK_IMPLICIT_LEAKAGE, true><<<grid, block, 0, s>>>(A);
    else transport_kernel<float, ABX_TRACK_IMPLICIT_LEAKAGE, false><<<grid, block, 0, s>>>(A);
  }
}

int occupancy_f_variant(int tracking, bool iso, int block) {
  int nb = 0;
  if (tracking == ABX_TRACK_CARTER) {
    if (iso) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, transport_kernel<float, ABX_TRACK_CARTER, true>, block, 0);
    else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, transport_kernel<float, ABX_TRACK_CARTER, false>, block, 0);
  } else if (iso) {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, transport_kernel<float, ABX_TRACK_IMPLICIT_LEAKAGE, true>,
                                                  block, 0);
  } else {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, transport_kernel<float, ABX_TRACK_IMPLICIT_LEAKAGE, false>,
                                                  block, 0);
  }
  return nb;
}

}  // namespace abx
