// FP64 parity translation unit: every kernel here runs in double, in the
// reference's operation order, compiled with --fmad=false so no
// multiply-add is contracted.
#include "transport_loop.cuh"
#include "launch.h"
#include "sources.cuh"

namespace abx {

template __global__ void transport_kernel<double, ABX_TRACK_DELTA, false>(const __grid_constant__ TransportArgs<double>);
template __global__ void transport_kernel<double, ABX_TRACK_SURFACE, false>(const __grid_constant__ TransportArgs<double>);
template __global__ void transport_kernel<double, ABX_TRACK_IMPLICIT_LEAKAGE, false>(
    const __grid_constant__ TransportArgs<double>);
template __global__ void transport_kernel<double, ABX_TRACK_CARTER, false>(const __grid_constant__ TransportArgs<double>);
// branchless collisions (the branchless k-eigenvalue simulation)
template __global__ void transport_kernel<double, ABX_TRACK_DELTA | ABX_KERNEL_BRANCHLESS, false>(
    const __grid_constant__ TransportArgs<double>);
template __global__ void transport_kernel<double, ABX_TRACK_SURFACE | ABX_KERNEL_BRANCHLESS, false>(
    const __grid_constant__ TransportArgs<double>);

void launch_transport_d(const TransportArgs<double>& A, int tracking, bool trace, int grid, int block,
                        cudaStream_t s) {
  tracking &= ~ABX_KERNEL_SINGLE;  // FP64 kernels serve single problems and batches alike
  if (tracking & ABX_KERNEL_WIDE) {
    launch_transport_d_wide(A, tracking, grid, block, s);
  } else if (tracking == (ABX_TRACK_DELTA | ABX_KERNEL_BRANCHLESS)) {
    transport_kernel<double, ABX_TRACK_DELTA | ABX_KERNEL_BRANCHLESS, false><<<grid, block, 0, s>>>(A);
  } else if (tracking == (ABX_TRACK_SURFACE | ABX_KERNEL_BRANCHLESS)) {
    transport_kernel<double, ABX_TRACK_SURFACE | ABX_KERNEL_BRANCHLESS, false><<<grid, block, 0, s>>>(A);
  } else if (tracking == ABX_TRACK_DELTA) {
    transport_kernel<double, ABX_TRACK_DELTA, false><<<grid, block, 0, s>>>(A);
  } else if (tracking == ABX_TRACK_IMPLICIT_LEAKAGE) {
    transport_kernel<double, ABX_TRACK_IMPLICIT_LEAKAGE, false><<<grid, block, 0, s>>>(A);
  } else if (tracking == ABX_TRACK_CARTER) {
    transport_kernel<double, ABX_TRACK_CARTER, false><<<grid, block, 0, s>>>(A);
  } else {
    transport_kernel<double, ABX_TRACK_SURFACE, false><<<grid, block, 0, s>>>(A);
  }
}

int occupancy_d(int tracking, int block) {
  int nb = 0;
  tracking &= ~ABX_KERNEL_SINGLE;
  if (tracking & ABX_KERNEL_WIDE) return occupancy_d_wide(tracking, block);
  if (tracking == (ABX_TRACK_DELTA | ABX_KERNEL_BRANCHLESS))
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &nb, transport_kernel<double, ABX_TRACK_DELTA | ABX_KERNEL_BRANCHLESS, false>, block, 0);
  else if (tracking == (ABX_TRACK_SURFACE | ABX_KERNEL_BRANCHLESS))
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &nb, transport_kernel<double, ABX_TRACK_SURFACE | ABX_KERNEL_BRANCHLESS, false>, block, 0);
  else if (tracking == ABX_TRACK_DELTA)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, transport_kernel<double, ABX_TRACK_DELTA, false>, block, 0);
  else if (tracking == ABX_TRACK_IMPLICIT_LEAKAGE)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, transport_kernel<double, ABX_TRACK_IMPLICIT_LEAKAGE, false>,
                                                  block, 0);
  else if (tracking == ABX_TRACK_CARTER)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, transport_kernel<double, ABX_TRACK_CARTER, false>, block, 0);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, transport_kernel<double, ABX_TRACK_SURFACE, false>, block, 0);
  return nb;
}

int transport_regs_d(int tracking) {
  cudaFuncAttributes a;
  if (tracking == ABX_TRACK_DELTA) cudaFuncGetAttributes(&a, transport_kernel<double, ABX_TRACK_DELTA, false>);
  else cudaFuncGetAttributes(&a, transport_kernel<double, ABX_TRACK_SURFACE, false>);
  return a.numRegs;
}

void launch_sources(const SourceArgs& A, cudaStream_t s) {
  if (A.n == 0) return;
  uint64_t blocks = (A.n + 127) / 128;
  if (blocks > 152 * 64) blocks = 152 * 64;
  sources_kernel<double><<<(unsigned)blocks, 128, 0, s>>>(A);
}

}  // namespace abx
