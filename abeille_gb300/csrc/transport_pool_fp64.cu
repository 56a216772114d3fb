// Pooled transport kernels, FP64 parity mode (transport_pool.cuh; compiled
// with --fmad=false like every FP64 kernel): delta and surface tracking.
#include "transport_pool.cuh"
#include "launch.h"

namespace abx {

template __global__ void transport_pool_kernel<double, ABX_TRACK_DELTA, false>(const __grid_constant__ TransportArgs<double>);
template __global__ void transport_pool_kernel<double, ABX_TRACK_SURFACE, false>(const __grid_constant__ TransportArgs<double>);

void launch_pool_d(const TransportArgs<double>& A, int tracking, int grid, int block, cudaStream_t s) {
  if ((tracking & 0xff) == ABX_TRACK_DELTA) transport_pool_kernel<double, ABX_TRACK_DELTA, false><<<grid, block, 0, s>>>(A);
  else transport_pool_kernel<double, ABX_TRACK_SURFACE, false><<<grid, block, 0, s>>>(A);
}

int occupancy_pool_d(int tracking, int block) {
  int nb = 0;
  if ((tracking & 0xff) == ABX_TRACK_DELTA)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, transport_pool_kernel<double, ABX_TRACK_DELTA, false>, block, 0);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, transport_pool_kernel<double, ABX_TRACK_SURFACE, false>, block, 0);
  return nb;
}

size_t pool_slot_bytes_d() { return sizeof(PoolSlot<double>); }

}  // namespace abx
