// Pooled transport kernels, FP32 tracking (transport_pool.cuh): delta
// tracking, with an instantiation for problems whose materials all scatter
// isotropically; the surface-tracking ones are in
// transport_pool_mixed_surface.cu (compiled with the surface-tracking
// history kernel's flags).
#include "transport_pool.cuh"
#include "launch.h"

namespace abx {

constexpr int POOL_DELTA_SINGLE = ABX_TRACK_DELTA | ABX_KERNEL_SINGLE;
template __global__ void transport_pool_kernel<float, POOL_DELTA_SINGLE, false>(const __grid_constant__ TransportArgs<float>);
template __global__ void transport_pool_kernel<float, POOL_DELTA_SINGLE, true>(const __grid_constant__ TransportArgs<float>);
template __global__ void transport_pool_kernel<float, ABX_TRACK_DELTA, false>(const __grid_constant__ TransportArgs<float>);
template __global__ void transport_pool_kernel<float, ABX_TRACK_DELTA, true>(const __grid_constant__ TransportArgs<float>);

template <bool ISO> static const void* pool_fn_f(int tracking) {
  if (tracking == POOL_DELTA_SINGLE) return (const void*)transport_pool_kernel<float, POOL_DELTA_SINGLE, ISO>;
  return (const void*)transport_pool_kernel<float, ABX_TRACK_DELTA, ISO>;
}

void launch_pool_f(const TransportArgs<float>& A, int tracking, bool iso, int grid, int block, cudaStream_t s) {
  if (tracking == POOL_DELTA_SINGLE) {
    if (iso) transport_pool_kernel<float, POOL_DELTA_SINGLE, true><<<grid, block, 0, s>>>(A);
    else transport_pool_kernel<float, POOL_DELTA_SINGLE, false><<<grid, block, 0, s>>>(A);
  } else if ((tracking & 0xff) == ABX_TRACK_DELTA) {
    if (iso) transport_pool_kernel<float, ABX_TRACK_DELTA, true><<<grid, block, 0, s>>>(A);
    else transport_pool_kernel<float, ABX_TRACK_DELTA, false><<<grid, block, 0, s>>>(A);
  } else {
    launch_pool_f_surface(A, iso, grid, block, s);
  }
}

int occupancy_pool_f(int tracking, bool iso, int block) {
  if ((tracking & 0xff) == ABX_TRACK_SURFACE) return occupancy_pool_f_surface(iso, block);
  int nb = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, iso ? pool_fn_f<true>(tracking) : pool_fn_f<false>(tracking),
                                                block, 0);
  return nb;
}

size_t pool_slot_bytes_f() { return sizeof(PoolSlot<float>); }

}  // namespace abx
