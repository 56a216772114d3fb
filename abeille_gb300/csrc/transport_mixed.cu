// Mixed-precision translation unit: positions, directions, flight distances
// and cross sections in FP32; scores, tallies and k in FP64.
#include "transport_loop.cuh"
#include "launch.h"

namespace abx {

template __global__ void transport_kernel<float, ABX_TRACK_DELTA>(const __grid_constant__ TransportArgs<float>);
template __global__ void transport_kernel<float, ABX_TRACK_SURFACE>(const __grid_constant__ TransportArgs<float>);

void launch_transport_f(const TransportArgs<float>& A, int tracking, bool trace, int grid, int block,
                        cudaStream_t s) {
  if (tracking == ABX_TRACK_DELTA) {
    transport_kernel<float, ABX_TRACK_DELTA><<<grid, block, 0, s>>>(A);
  } else {
    transport_kernel<float, ABX_TRACK_SURFACE><<<grid, block, 0, s>>>(A);
  }
}

int occupancy_f(int tracking, int block) {
  int nb = 0;
  if (tracking == ABX_TRACK_DELTA)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, transport_kernel<float, ABX_TRACK_DELTA>, block, 0);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, transport_kernel<float, ABX_TRACK_SURFACE>, block, 0);
  return nb;
}

int transport_regs_f(int tracking) {
  cudaFuncAttributes a;
  if (tracking == ABX_TRACK_DELTA) cudaFuncGetAttributes(&a, transport_kernel<float, ABX_TRACK_DELTA>);
  else cudaFuncGetAttributes(&a, transport_kernel<float, ABX_TRACK_SURFACE>);
  return a.numRegs;
}

}  // namespace abx
