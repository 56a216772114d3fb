// FP64 parity translation unit: every kernel here runs in double, in the
// reference's operation order, compiled with --fmad=false so no
// multiply-add is contracted.
#include "transport_loop.cuh"
#include "launch.h"

namespace abx {

template __global__ void transport_kernel<double, ABX_TRACK_DELTA, false>(const __grid_constant__ TransportArgs<double>);
template __global__ void transport_kernel<double, ABX_TRACK_SURFACE, false>(const __grid_constant__ TransportArgs<double>);
template __global__ void transport_kernel<double, ABX_TRACK_IMPLICIT_LEAKAGE, false>(
    const __grid_constant__ TransportArgs<double>);
template __global__ void transport_kernel<double, ABX_TRACK_CARTER, false>(const __grid_constant__ TransportArgs<double>);

void launch_transport_d(const TransportArgs<double>& A, int tracking, bool trace, int grid, int block,
                        cudaStream_t s) {
  if (tracking == ABX_TRACK_DELTA) {
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
  if (tracking == ABX_TRACK_DELTA)
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

// Simulation::sample_sources + Source::generate_particle
// (src/simulation.cpp:55-77, src/source.cpp:44-90), one thread per history.
__global__ void __launch_bounds__(128) sources_kernel(const SourceArgs A) {
  const Tables& T = A.T;
  const View<double> V = make_view<double>(T);
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < A.n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    int prob = A.prob;
    uint64_t hid = A.first_hid + i;
    if (A.nseg > 0) {
      // last segment whose first index is <= i
      int lo = 0, hi = A.nseg - 1;
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (A.seg_off[mid] <= i) lo = mid; else hi = mid - 1;
      }
      prob = A.seg_prob[lo];
      hid = A.seg_hid0[lo] + (i - A.seg_off[lo]);
    }
    const ProbT& P = T.probs[prob];
    uint64_t rng = pcg_advance(pcg_seeded(P.seed), P.stride * hid);
    int si = P.src_first + discrete<double>(rng, T.src_cdf + P.src_cdf_off, P.src_count);
    const abx_source S = T.sources[si];
    V3<double> u;
    if (S.direction == ABX_DIR_ISOTROPIC) {
      // Isotropic::sample (src/isotropic.cpp:28-36) -> Direction(mu, phi)
      const double PI = 3.14159265358979323846264338327950288;
      double mu = 2. * canon_d(rng) - 1.;
      double phi = 2. * PI * canon_d(rng);
      if (mu < -1.) mu = -1.; else if (mu > 1.) mu = 1.;
      if (phi < 0.) phi = 0.; else if (phi > 2 * PI) phi = 2 * PI;
      double x = sqrt(1. - mu * mu) * cos(phi);
      double y = sqrt(1. - mu * mu) * sin(phi);
      u = dir3<double>(x, y, mu);
    } else {
      u = dir3<double>(S.dir[0], S.dir[1], S.dir[2]);
    }
    double E = S.energy_value;  // MonoEnergetic: no draw, sampled twice by the reference
    auto pos = [&]() -> V3<double> {
      if (S.spatial == ABX_SPATIAL_POINT) return mk<double>(S.low[0], S.low[1], S.low[2]);
      double x = (S.hi[0] - S.low[0]) * canon_d(rng) + S.low[0];
      double y = (S.hi[1] - S.low[1]) * canon_d(rng) + S.low[1];
      double z = (S.hi[2] - S.low[2]) * canon_d(rng) + S.low[2];
      return mk<double>(x, y, z);
    };
    V3<double> r = pos();
    Trk<double> k;
    k.r = r; k.u = u; k.token = 0; k.err = 0;
    trk_restart(T, V, P, k);
    int guard = 0;
    bool bad = false;
    while (k.cell < 0) {
      if (S.spatial == ABX_SPATIAL_POINT || ++guard > 100000) { bad = true; break; }
      r = pos();
      trk_set_r(k, r);
      trk_restart(T, V, P, k);
    }
    if (!bad && S.fissile_only) {
      int count = 0;
      while (k.cell < 0 || !T.mats[T.cells[k.cell].fill].fissile) {
        if (count == 201) { bad = true; break; }
        r = pos();
        trk_set_r(k, r);
        trk_restart(T, V, P, k);
        count++;
      }
    }
    if (bad || k.err) {
      if (atomicCAS(&A.st->err, 0, bad ? ABX_ERR_INVALID : k.err) == 0) A.st->err_hist = hid;
      continue;
    }
    const uint64_t o = A.out_off + i;
    A.x[o] = r.x; A.y[o] = r.y; A.z[o] = r.z;
    A.ux[o] = u.x; A.uy[o] = u.y; A.uz[o] = u.z;
    A.E[o] = E; A.w[o] = 1.0; A.w2[o] = 0.;
    A.rng[o] = rng; A.hid[o] = hid;
    if (A.fam) A.fam[o] = hid;
    if (A.probv) A.probv[o] = prob;
  }
}

void launch_sources(const SourceArgs& A, cudaStream_t s) {
  if (A.n == 0) return;
  uint64_t blocks = (A.n + 127) / 128;
  if (blocks > 152 * 64) blocks = 152 * 64;
  sources_kernel<<<(unsigned)blocks, 128, 0, s>>>(A);
}

}  // namespace abx
