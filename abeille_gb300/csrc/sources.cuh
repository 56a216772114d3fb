// Source sampling kernel, templated on the precision it samples in.  FP64
// follows the reference's arithmetic (parity mode); FP32 (the mixed mode)
// samples directions and positions in FP32 straight into the FP32 bank.
#pragma once

#include "kernels.cuh"
#include "launch.h"

namespace abx {

// Simulation::sample_sources + Source::generate_particle
// (src/simulation.cpp:55-77, src/source.cpp:44-90), one thread per history.
template <class R>
__global__ void __launch_bounds__(128) sources_kernel(const SourceArgs A) {
  const Tables& T = A.T;
  const View<R> V = make_view<R>(T);
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
    int si = P.src_first + discrete<double>(rng, T.src_cdf + P.src_cdf_off, P.src_count);  // FP64 CDF both modes
    const abx_source S = T.sources[si];
    V3<R> u;
    if (S.direction == ABX_DIR_ISOTROPIC) {
      // Isotropic::sample (src/isotropic.cpp:28-36) -> Direction(mu, phi)
      R mu = R(2) * canon<R>(rng) - R(1);
      if (mu < R(-1)) mu = R(-1); else if (mu > R(1)) mu = R(1);
      R c, sn;
      if constexpr (sizeof(R) == 8) {
        const double PI = 3.14159265358979323846264338327950288;
        double phi = 2. * PI * canon_d(rng);
        if (phi < 0.) phi = 0.; else if (phi > 2 * PI) phi = 2 * PI;
        c = cos(phi);
        sn = sin(phi);
      } else {
        azimuth(canon<R>(rng), c, sn);  // FP32: cos and sin of 2*pi*u
      }
      R x = sqrt_1m<R>(mu * mu) * c;
      R y = sqrt_1m<R>(mu * mu) * sn;
      u = dir3<R>(x, y, mu);
    } else {
      u = dir3<R>((R)S.dir[0], (R)S.dir[1], (R)S.dir[2]);
    }
    R E = (R)S.energy_value;  // MonoEnergetic: no draw, sampled twice by the reference
    auto pos = [&]() -> V3<R> {
      if (S.spatial == ABX_SPATIAL_POINT) return mk<R>((R)S.low[0], (R)S.low[1], (R)S.low[2]);
      R x = ((R)S.hi[0] - (R)S.low[0]) * canon<R>(rng) + (R)S.low[0];
      R y = ((R)S.hi[1] - (R)S.low[1]) * canon<R>(rng) + (R)S.low[1];
      R z = ((R)S.hi[2] - (R)S.low[2]) * canon<R>(rng) + (R)S.low[2];
      return mk<R>(x, y, z);
    };
    V3<R> r = pos();
    Trk<R> k;
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
    if constexpr (sizeof(R) == 8) {
      A.x[o] = r.x; A.y[o] = r.y; A.z[o] = r.z;
      A.ux[o] = u.x; A.uy[o] = u.y; A.uz[o] = u.z;
      A.E[o] = E; A.w[o] = 1.0; A.w2[o] = 0.;
    } else {
      A.fx[o] = r.x; A.fy[o] = r.y; A.fz[o] = r.z;
      A.fux[o] = u.x; A.fuy[o] = u.y; A.fuz[o] = u.z;
      A.fE[o] = E; A.fw[o] = 1.f; A.fw2[o] = 0.f;
    }
    A.rng[o] = rng; A.hid[o] = hid;
    if (A.fam) A.fam[o] = hid;
    if (A.probv) A.probv[o] = prob;
  }
}

}  // namespace abx
