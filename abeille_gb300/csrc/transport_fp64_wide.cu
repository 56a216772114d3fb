// FP64 parity kernels for large launches: delta and surface tracking with four
// 256-thread blocks per SM (64 registers) instead of three.  Measured on one
// GB300: +4 % on the 1M-history pin assembly, +6 % on the 2M-history ring-pin
// lattice, but 25 % slower on a 10,000-history launch, whose lanes each run
// one history and gain nothing from more of them; so contexts whose
// generations hold at least FP64_WIDE_MIN_HISTORIES histories use these.
// Same arithmetic as transport_fp64.cu (--fmad=false): the results are the same
// bit for bit, only the register allocation differs.
#include "transport_loop.cuh"
#include "launch.h"

namespace abx {

template __global__ void transport_kernel<double, ABX_TRACK_DELTA | ABX_KERNEL_WIDE, false>(
    const __grid_constant__ TransportArgs<double>);
template __global__ void transport_kernel<double, ABX_TRACK_SURFACE | ABX_KERNEL_WIDE, false>(
    const __grid_constant__ TransportArgs<double>);

void launch_transport_d_wide(const TransportArgs<double>& A, int tracking, int grid, int block, cudaStream_t s) {
  if ((tracking & 0xff) == ABX_TRACK_DELTA)
    transport_kernel<double, ABX_TRACK_DELTA | ABX_KERNEL_WIDE, false><<<grid, block, 0, s>>>(A);
  else
    transport_kernel<double, ABX_TRACK_SURFACE | ABX_KERNEL_WIDE, false><<<grid, block, 0, s>>>(A);
}

int occupancy_d_wide(int tracking, int block) {
  int nb = 0;
  if ((tracking & 0xff) == ABX_TRACK_DELTA)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, transport_kernel<double, ABX_TRACK_DELTA | ABX_KERNEL_WIDE, false>,
                                                  block, 0);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &nb, transport_kernel<double, ABX_TRACK_SURFACE | ABX_KERNEL_WIDE, false>, block, 0);
  return nb;
}

}  // namespace abx
