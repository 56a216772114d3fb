// Mixed-precision translation unit, delta tracking: positions, directions,
// flight distances and cross sections in FP32; scores, tallies and k in FP64.
// Each tracking mode has one instantiation for problems whose materials all
// scatter isotropically and one general; the surface-tracking pair lives in
// transport_mixed_surface.cu so the two compile in parallel.
#include "transport_loop.cuh"
#include "launch.h"
#include "sources.cuh"

namespace abx {

template __global__ void transport_kernel<float, ABX_TRACK_DELTA, false>(const __grid_constant__ TransportArgs<float>);
template __global__ void transport_kernel<float, ABX_TRACK_DELTA, true>(const __grid_constant__ TransportArgs<float>);
// one problem, no per-problem bookkeeping (the power iteration, transport
// steps and fixed-source runs of a single problem)
constexpr int DELTA_SINGLE = ABX_TRACK_DELTA | ABX_KERNEL_SINGLE;
template __global__ void transport_kernel<float, DELTA_SINGLE, false>(const __grid_constant__ TransportArgs<float>);
template __global__ void transport_kernel<float, DELTA_SINGLE, true>(const __grid_constant__ TransportArgs<float>);

void launch_transport_f(const TransportArgs<float>& A, int tracking, bool iso, bool trace, int grid, int block,
                        cudaStream_t s) {
  if (tracking == DELTA_SINGLE) {
    if (iso) transport_kernel<float, DELTA_SINGLE, true><<<grid, block, 0, s>>>(A);
    else transport_kernel<float, DELTA_SINGLE, false><<<grid, block, 0, s>>>(A);
    return;
  }
  tracking &= ~ABX_KERNEL_SINGLE;  // the other kernels serve single problems too
  if (tracking & ABX_KERNEL_BRANCHLESS) {
    launch_transport_f_branchless(A, tracking & 0xff, iso, grid, block, s);
  } else if (tracking == ABX_TRACK_SURFACE) {
    launch_transport_f_surface(A, iso, grid, block, s);
  } else if (tracking == ABX_TRACK_IMPLICIT_LEAKAGE || tracking == ABX_TRACK_CARTER) {
    launch_transport_f_variant(A, tracking, iso, grid, block, s);
  } else if (iso) {
    transport_kernel<float, ABX_TRACK_DELTA, true><<<grid, block, 0, s>>>(A);
  } else {
    transport_kernel<float, ABX_TRACK_DELTA, false><<<grid, block, 0, s>>>(A);
  }
}

int occupancy_f(int tracking, bool iso, int block) {
  if (tracking == DELTA_SINGLE) {
    int nb = 0;
    if (iso) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, transport_kernel<float, DELTA_SINGLE, true>, block, 0);
    else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, transport_kernel<float, DELTA_SINGLE, false>, block, 0);
    return nb;
  }
  tracking &= ~ABX_KERNEL_SINGLE;
  if (tracking & ABX_KERNEL_BRANCHLESS) return occupancy_f_branchless(tracking & 0xff, iso, block);
  if (tracking == ABX_TRACK_SURFACE) return occupancy_f_surface(iso, block);
  if (tracking == ABX_TRACK_IMPLICIT_LEAKAGE || tracking == ABX_TRACK_CARTER)
    return occupancy_f_variant(tracking, iso, block);
  int nb = 0;
  if (iso) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, transport_kernel<float, ABX_TRACK_DELTA, true>, block, 0);
  else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, transport_kernel<float, ABX_TRACK_DELTA, false>, block, 0);
  return nb;
}

void launch_sources_f(const SourceArgs& A, cudaStream_t s) {
  if (A.n == 0) return;
  uint64_t blocks = (A.n + 127) / 128;
  if (blocks > 152 * 64) blocks = 152 * 64;
  sources_kernel<float><<<(unsigned)blocks, 128, 0, s>>>(A);
}

int transport_regs_f(int tracking) {
  cudaFuncAttributes a;
  if (tracking == ABX_TRACK_DELTA) cudaFuncGetAttributes(&a, transport_kernel<float, ABX_TRACK_DELTA, false>);
  else return transport_regs_f_surface();
  return a.numRegs;
}

}  // namespace abx
