// Host-side launchers exported by the kernel translation units.
#pragma once

#include <cuda_runtime.h>

#include "tables.h"

namespace abx {

template <class R> struct TransportArgs;
template <class R> struct BankT;

struct SourceArgs {
  Tables T;
  int prob;                 // problem index whose sources are sampled
  uint64_t first_hid;
  uint64_t n;
  // output bank (double SoA; the FP32 sampler writes the float arrays)
  double *x, *y, *z, *ux, *uy, *uz, *E, *w, *w2;
  float *fx, *fy, *fz, *fux, *fuy, *fuz, *fE, *fw, *fw2;
  uint64_t* rng;
  uint64_t* hid;
  uint64_t* fam;
  int32_t* probv;           // optional per-history problem index output
  uint64_t out_off;         // write offset into the output arrays
  DevState* st;
  // batches of problems: output index i belongs to segment s with
  // seg_off[s] <= i < seg_off[s+1]: problem seg_prob[s], history id
  // seg_hid0[s] + (i - seg_off[s]).  nseg == 0: one problem (prob, first_hid).
  const uint64_t* seg_off;
  const int32_t* seg_prob;
  const uint64_t* seg_hid0;
  int nseg;
};

// transport_fp64.cu
void launch_transport_d(const TransportArgs<double>& A, int tracking, bool trace, int grid, int block,
                        cudaStream_t s);
void launch_sources(const SourceArgs& A, cudaStream_t s);
void launch_sources_f(const SourceArgs& A, cudaStream_t s);  // transport_mixed.cu
int transport_regs_d(int tracking);
// transport_fp64_wide.cu: the FP64 delta/surface kernels at four blocks per SM
void launch_transport_d_wide(const TransportArgs<double>& A, int tracking, int grid, int block, cudaStream_t s);
int occupancy_d_wide(int tracking, int block);

// transport_mixed.cu (+ transport_mixed_surface.cu); `iso`: every material
// of the problem scatters isotropically; `tracking` is a kernel code (the
// tracking mode, or'd with ABX_KERNEL_BRANCHLESS for branchless collisions)
void launch_transport_f(const TransportArgs<float>& A, int tracking, bool iso, bool trace, int grid, int block,
                        cudaStream_t s);
void launch_transport_f_surface(const TransportArgs<float>& A, bool iso, int grid, int block, cudaStream_t s);
void launch_transport_f_variant(const TransportArgs<float>& A, int tracking, bool iso, int grid, int block,
                                cudaStream_t s);
int occupancy_f_variant(int tracking, bool iso, int block);
// transport_mixed_branchless.cu: `tracking` delta or surface
void launch_transport_f_branchless(const TransportArgs<float>& A, int tracking, bool iso, int grid, int block,
                                   cudaStream_t s);
int occupancy_f_branchless(int tracking, bool iso, int block);
int transport_regs_f(int tracking);
int transport_regs_f_surface();

// transport_pool_mixed.cu / transport_pool_fp64.cu: the pooled kernels
// (delta tracking, surface tracking); `A.pool` holds pool_slot_bytes_*()
// bytes for each of the 32 * POOL_K slots of every warp of the launch
void launch_pool_f(const TransportArgs<float>& A, int tracking, bool iso, int grid, int block, cudaStream_t s);
int occupancy_pool_f(int tracking, bool iso, int block);
size_t pool_slot_bytes_f();
// transport_pool_mixed_surface.cu: the FP32 surface-tracking pooled kernels
void launch_pool_f_surface(const TransportArgs<float>& A, bool iso, int grid, int block, cudaStream_t s);
int occupancy_pool_f_surface(bool iso, int block);
void launch_pool_d(const TransportArgs<double>& A, int tracking, int grid, int block, cudaStream_t s);
int occupancy_pool_d(int tracking, int block);
size_t pool_slot_bytes_d();
constexpr int POOL_SLOTS_PER_WARP = 128;

// occupancy helpers
int occupancy_d(int tracking, int block);
int occupancy_f(int tracking, bool iso, int block);
int occupancy_f_surface(bool iso, int block);

}  // namespace abx
