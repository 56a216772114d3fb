// Device building blocks of the transport loop, templated on the tracking
// precision R: argument and bank layouts, score accumulators, the collision
// (Transporter::collision and its helpers) and the mesh-tally estimators.
// Included by transport_loop.cuh, which transport_fp64.cu (R = double,
// --fmad=false) and transport_mixed.cu (R = float) instantiate.
//
// Fission sites are appended with warp-aggregated atomics and keyed by
// (history, daughter) so a counting sort restores the reference's bank order.
#pragma once

#include <cooperative_groups.h>
#include <cooperative_groups/reduce.h>
#include <cooperative_groups/scan.h>

#include "device.cuh"

namespace abx {

namespace cg = cooperative_groups;

template <class R> struct BankT {
  R *x, *y, *z, *ux, *uy, *uz, *E, *w, *w2;
  uint64_t* rng;
  uint64_t* hid;
  uint64_t* fam;
  int32_t* prob;  // problem index per history, or nullptr for problem 0
};

template <class R> struct SiteT {
  R *x, *y, *z, *ux, *uy, *uz, *E, *w;
  uint32_t* hist;
  uint32_t* dau;
};

template <class R> struct TransportArgs {
  Tables T;
  BankT<R> bank;
  SiteT<R> sites;
  uint64_t site_cap;
  uint32_t* hist_count;
  R* sec;              // secondary stacks: [thread][sec_cap][9]
  uint32_t sec_cap;
  DevState* st;
  abx_trace_rec* trace;
  uint32_t trace_nhist;
  uint64_t trace_cap;
  uint64_t max_events;
  // batches of problems: per-problem score sums [prob][ABX_PSCORES] and
  // counters [prob][ABX_PCOUNTS]; nullptr when one problem runs alone
  double* pscore;
  unsigned long long* pcount;
  // pooled kernel: 32 * POOL_K slot records per warp of the launch
  void* pool;
  // history kernel: histories a warp takes before it retires (0: no limit).
  // With a grid larger than the GPU holds at once, blocks then finish and
  // leave their SM slots to later blocks -- and to launches of other
  // streams -- while the launch runs; the grid must cover the histories
  // (grid * warps per block * quota >= histories).
  uint32_t warp_quota;
};

enum : int { ABX_PSCORES = 5, ABX_PCOUNTS = 4 };
// transport kernel codes: the tracking mode (ABX_TRACK_*) or'd with these
// bits: branchless collisions; one problem without per-problem scores (every
// history of the launch belongs to problem 0, the batch bookkeeping compiled
// out)
// ABX_KERNEL_WIDE: the FP64 instantiation with four blocks per SM, for large launches
enum : int { ABX_KERNEL_BRANCHLESS = 0x100, ABX_KERNEL_SINGLE = 0x200, ABX_KERNEL_WIDE = 0x800 };  // counters: collisions flights histories lost

template <class R> ABX_DEV View<R> make_view(const Tables& T);
template <> ABX_DEV View<double> make_view<double>(const Tables& T) {
  return View<double>{T.surf_d, T.lat_d, T.xs_d, T.cdf_d, T.ang_d, T.eb_d, T.maj_d, T.dg_d};
}
template <> ABX_DEV View<float> make_view<float>(const Tables& T) {
  return View<float>{T.surf_f, T.lat_f, T.xs_f, T.cdf_f, T.ang_f, T.eb_f, T.maj_f, T.dg_f};
}
template <class R> ABX_DEV const R* tally_eb(const Tables& T);
template <> ABX_DEV const double* tally_eb<double>(const Tables& T) { return T.tally_eb; }
template <> ABX_DEV const float* tally_eb<float>(const Tables& T) { return T.tally_eb_f; }

template <class R> ABX_DEV void tally_geom(const TallyT& t, R low[3], R hi[3], R d[3], R dinv[3]);
template <> ABX_DEV void tally_geom<double>(const TallyT& t, double low[3], double hi[3], double d[3], double dinv[3]) {
  for (int a = 0; a < 3; a++) { low[a] = t.low[a]; hi[a] = t.hi[a]; d[a] = t.d[a]; dinv[a] = t.dinv[a]; }
}
template <> ABX_DEV void tally_geom<float>(const TallyT& t, float low[3], float hi[3], float d[3], float dinv[3]) {
  for (int a = 0; a < 3; a++) { low[a] = t.lowf[a]; hi[a] = t.hif[a]; d[a] = t.df[a]; dinv[a] = t.dinvf[a]; }
}

// Score accumulators.  Each history sums its terms in the tracking precision;
// at the end of the history the five totals are added, in FP64, to the block's
// shared accumulators (one FP64 atomic each), which the block adds to the
// global scores when it retires; in a batch of problems they go straight to
// the history's own problem.  In FP64 mode every term is a double, so
// the sums are FP64 throughout, as the reference's ThreadLocalScores.
template <class R> struct Acc {
  R hcol = 0, habs = 0, htrk = 0, hleak = 0, hmig = 0;
  ABX_DEV void flush(double* sh) {
    atomicAdd(sh + 0, (double)hcol);
    atomicAdd(sh + 1, (double)habs);
    atomicAdd(sh + 2, (double)htrk);
    atomicAdd(sh + 3, (double)hleak);
    atomicAdd(sh + 4, (double)hmig);
    hcol = habs = htrk = hleak = hmig = R(0);
  }
};

template <class R> struct Lane {
  V3<R> r, u, rb;
  R E, w, w2;
  int g;
  uint64_t rng;
  uint32_t h;
  int pid;
  int mat;
  uint32_t dau;
  uint32_t nsec;
  uint32_t events;  // flights of this history (secondaries included)
  uint32_t hcoll;   // real collisions of this history
  uint32_t npos, nneg;
};

ABX_DEV void raise_err(DevState* st, int code, uint64_t hist) {
  if (atomicCAS(&st->err, 0, code) == 0) st->err_hist = hist;
}

template <class R> ABX_DEV int group_of(const R* eb, int G, R E) {
  // MGNuclide::energy_grid_index (src/mg_nuclide.cpp:382-392)
  int i;
  for (i = 0; i < G; i++)
    if (eb[i] <= E && E < eb[i + 1]) break;
  return i;
}

// Trace records and track-length scoring are called from several places of
// the loop but run rarely (tracing is a test hook; the track-length tally only
// exists in some problems).  They are compiled once, out of line, with plain
// scalar arguments, so the loop's hot code stays compact.
static __device__ __noinline__ void trace_write(abx_trace_rec* trace, uint64_t cap, unsigned long long* counter,
                                         uint32_t h, int kind, int g, int cell, uint64_t rng, double rx,
                                         double ry, double rz, double ux, double uy, double uz, double w) {
  unsigned long long i = atomicAdd(counter, 1ull);
  if (i >= cap) return;
  abx_trace_rec t;
  t.hist = h; t.kind = kind; t.group = g; t.cell = cell; t.rng_state = rng;
  t.r[0] = rx; t.r[1] = ry; t.r[2] = rz;
  t.u[0] = ux; t.u[1] = uy; t.u[2] = uz;
  t.wgt = w;
  trace[i] = t;
}

template <class R> ABX_DEV void trace_rec(const TransportArgs<R>& A, const Lane<R>& L, int kind, int cell) {
  if (L.h >= A.trace_nhist) return;
  trace_write(A.trace, A.trace_cap, &A.st->trace_n, L.h, kind, L.g, cell, L.rng, (double)L.r.x, (double)L.r.y,
              (double)L.r.z, (double)L.u.x, (double)L.u.y, (double)L.u.z, (double)L.w);
}

// Quantity multiplier (src/collision_mesh_tally.cpp:66-100).
template <class R> ABX_DEV R qfactor(const View<R>& V, const MatT& M, int q, int g, R w) {
  switch (q) {
    case ABX_Q_ELASTIC: return w * V.xs[M.xs_off + XS_ES * M.G + g];
    case ABX_Q_ABSORPTION: return w * V.xs[M.xs_off + XS_EABS * M.G + g];
    case ABX_Q_FISSION: return w * V.xs[M.xs_off + XS_EF * M.G + g];
    case ABX_Q_TOTAL: return w * V.xs[M.xs_off + XS_ET * M.G + g];
    default: return w;
  }
}

template <class R> ABX_DEV int tally_ebin(const R* eb, int ne, R E) {
  for (int e = 0; e < ne; e++)
    if (eb[e] <= E && E <= eb[e + 1]) return e;
  return -1;
}

// CollisionMeshTally::score_collision (src/collision_mesh_tally.cpp:33-108)
template <class R>
ABX_DEV void score_collision(const Tables& T, const View<R>& V, const ProbT& P, const MatT& M, const Lane<R>& L) {
  const R* teb = tally_eb<R>(T);
  for (int ti = P.tally_first; ti < P.tally_first + P.tally_count; ti++) {
    const TallyT& t = T.tallies[ti];
    if (t.est != ABX_EST_COLLISION) continue;
    R low[3], hi[3], d[3], dinv[3];
    tally_geom<R>(t, low, hi, d, dinv);
    R Et = V.xs[M.xs_off + XS_ET * M.G + L.g];
    R scr = R(1) / (Et * (R)P.nparticles);
    int i = (int)m_floor((L.r.x - low[0]) * dinv[0]);
    int j = (int)m_floor((L.r.y - low[1]) * dinv[1]);
    int k = (int)m_floor((L.r.z - low[2]) * dinv[2]);
    int l = tally_ebin<R>(teb + t.eb_off, t.ne, L.E);
    if (l < 0) continue;
    if (i >= 0 && i < t.n[0] && j >= 0 && j < t.n[1] && k >= 0 && k < t.n[2]) {
      scr *= qfactor(V, M, t.quantity, L.g, L.w);
      int64_t idx = t.bin_off + (((int64_t)l * t.n[0] + i) * t.n[1] + j) * t.n[2] + k;
      atomicAdd(T.tally_gen + idx, (double)scr);
    }
  }
}

// TrackLengthMeshTally::score_flight (src/track_length_mesh_tally.cpp:77-435)
template <class R>
__device__ __noinline__ void score_flight_ool(const TallyT* tallies, double* tally_gen, const R* teb, const R* xs,
                                              const MatT* mats, int tally_first, int tally_count,
                                              double nparticles, R rx, R ry, R rz, R ux, R uy, R uz, R w, R E,
                                              int g, int mat, R dfl) {
  for (int ti = tally_first; ti < tally_first + tally_count; ti++) {
    const TallyT& t = tallies[ti];
    if (t.est != ABX_EST_TRACK_LENGTH) continue;
    R low[3], hi[3], d[3], dinv[3];
    tally_geom<R>(t, low, hi, d, dinv);
    V3<R> r = mk<R>(rx, ry, rz);
    const V3<R> u = mk<R>(ux, uy, uz);
    int ijk[3], on[3];
    auto init_idx = [&](V3<R> rr) {
      R rc[3] = {rr.x, rr.y, rr.z}, uc[3] = {u.x, u.y, u.z};
#pragma unroll
      for (int a = 0; a < 3; a++) {
        ijk[a] = (int)m_floor((rc[a] - low[a]) * dinv[a]);
        on[a] = 0;
        R c = low[a] + ijk[a] * d[a] + R(0.5) * d[a];
        R lo = c - R(0.5) * d[a], hi = c + R(0.5) * d[a];
        if (m_abs(lo - rc[a]) < Tol<R>::SC) {
          if (uc[a] < R(0)) { ijk[a]--; on[a] = 1; } else { on[a] = -1; }
        } else if (m_abs(hi - rc[a]) < Tol<R>::SC) {
          if (uc[a] < R(0)) { on[a] = 1; } else { ijk[a]++; on[a] = -1; }
        }
      }
    };
    init_idx(r);
    bool inside = ijk[0] >= 0 && ijk[0] < t.n[0] && ijk[1] >= 0 && ijk[1] < t.n[1] && ijk[2] >= 0 && ijk[2] < t.n[2];
    R dd = dfl;
    if (!inside) {
      // find_entry_point (src/track_length_mesh_tally.cpp:185-247)
      const R ix = R(1) / u.x, iy = R(1) / u.y, iz = R(1) / u.z;
      R dmin = (low[0] - r.x) * ix, dmax = (hi[0] - r.x) * ix, tmp;
      if (dmin > dmax) { tmp = dmin; dmin = dmax; dmax = tmp; }
      R dymin = (low[1] - r.y) * iy, dymax = (hi[1] - r.y) * iy;
      if (dymin > dymax) { tmp = dymin; dymin = dymax; dymax = tmp; }
      if ((dmin > dymax) || (dymin > dmax)) continue;
      if (dymin > dmin) dmin = dymin;
      if (dymax < dmax) dmax = dymax;
      R dzmin = (low[2] - r.z) * iz, dzmax = (hi[2] - r.z) * iz;
      if (dzmin > dzmax) { tmp = dzmin; dzmin = dzmax; dzmax = tmp; }
      if ((dmin > dzmax) || (dzmin > dmax)) continue;
      if (dzmin > dmin) dmin = dzmin;
      if (dzmax < dmax) dmax = dzmax;
      if (dmax < dmin) { tmp = dmax; dmax = dmin; dmin = tmp; }
      if ((dmax < R(0)) && (dmin < R(0))) continue;
      if (dmin < R(0)) continue;
      r = add(r, scl(u, dmin));
      dd -= dmin;
      init_idx(r);
    }
    const MatT& M = mats[mat];
    R base = R(1) / (R)nparticles;
    switch (t.quantity) {  // src/collision_mesh_tally.cpp:66-100, as qfactor
      case ABX_Q_ELASTIC: base *= w * xs[M.xs_off + XS_ES * M.G + g]; break;
      case ABX_Q_ABSORPTION: base *= w * xs[M.xs_off + XS_EABS * M.G + g]; break;
      case ABX_Q_FISSION: base *= w * xs[M.xs_off + XS_EF * M.G + g]; break;
      case ABX_Q_TOTAL: base *= w * xs[M.xs_off + XS_ET * M.G + g]; break;
      default: base *= w;
    }
    int l = tally_ebin<R>(teb + t.eb_off, t.ne, E);
    if (l < 0) continue;
    R rem = dd;
    for (int guard = 0; guard < (1 << 22) && rem > R(0); guard++) {
      R xc = low[0] + ijk[0] * d[0] + R(0.5) * d[0];
      R yc = low[1] + ijk[1] * d[1] + R(0.5) * d[1];
      R zc = low[2] + ijk[2] * d[2] + R(0.5) * d[2];
      V3<R> rt = mk<R>(r.x - xc, r.y - yc, r.z - zc);
      R dist = Tol<R>::INF;
      int key = 0;
      const R a = (-d[0] * R(0.5) - rt.x) * (R(1) / u.x), b = (d[0] * R(0.5) - rt.x) * (R(1) / u.x);
      const R c = (-d[1] * R(0.5) - rt.y) * (R(1) / u.y), e = (d[1] * R(0.5) - rt.y) * (R(1) / u.y);
      const R f = (-d[2] * R(0.5) - rt.z) * (R(1) / u.z), h = (d[2] * R(0.5) - rt.z) * (R(1) / u.z);
      if (a > R(0) && a < dist && on[0] != -1) { dist = a; key = -1; }
      if (b > R(0) && b < dist && on[0] != 1) { dist = b; key = 1; }
      if (c > R(0) && c < dist && on[1] != -1) { dist = c; key = -2; }
      if (e > R(0) && e < dist && on[1] != 1) { dist = e; key = 2; }
      if (f > R(0) && f < dist && on[2] != -1) { dist = f; key = -3; }
      if (h > R(0) && h < dist && on[2] != 1) { dist = h; key = 3; }
      if (dist == Tol<R>::INF) break;
      R dt = dist < rem ? dist : rem;
      if (ijk[0] >= 0 && ijk[0] < t.n[0] && ijk[1] >= 0 && ijk[1] < t.n[1] && ijk[2] >= 0 && ijk[2] < t.n[2]) {
        int64_t idx = t.bin_off + (((int64_t)l * t.n[0] + ijk[0]) * t.n[1] + ijk[1]) * t.n[2] + ijk[2];
        atomicAdd(tally_gen + idx, (double)(dt * base));
      } else {
        break;
      }
      rem -= dt;
      if (rem <= R(0)) break;
      r = add(r, scl(u, dt));
      on[0] = on[1] = on[2] = 0;
      switch (key) {
        case -1: ijk[0]--; on[0] = 1; break;
        case 1: ijk[0]++; on[0] = -1; break;
        case -2: ijk[1]--; on[1] = 1; break;
        case 2: ijk[1]++; on[1] = -1; break;
        case -3: ijk[2]--; on[2] = 1; break;
        case 3: ijk[2]++; on[2] = -1; break;
        default: break;
      }
    }
  }
}

template <class R>
ABX_DEV void score_flight(const Tables& T, const View<R>& V, const ProbT& P, const Lane<R>& L, R dfl) {
  score_flight_ool<R>(T.tallies, T.tally_gen, tally_eb<R>(T), V.xs, T.mats, P.tally_first, P.tally_count,
                      P.nparticles, L.r.x, L.r.y, L.r.z, L.u.x, L.u.y, L.u.z, L.w, L.E, L.g, L.mat, dfl);
}

// MGAngleDistribution::sample_mu (include/materials/mg_angle_distribution.hpp:45-60,92-101)
// ISO: every material of the problem scatters isotropically (the launch
// picks this instantiation), so the table path is compiled out.
template <class R, bool ISO>
ABX_DEV R sample_mu(const Tables& T, const View<R>& V, const MatT& M, int gi, int go, uint64_t& rng) {
  const R xi = canon<R>(rng);
  if (ISO || M.iso) {
    // the two-point {-1,1} table with pdf {0.5,0.5}: histogram branch
    if (xi == R(0)) return R(-1);
    return R(-1) + ((xi - R(0)) / R(0.5));
  }
  const AngHdr a = T.ang_hdr[M.ang_off + gi * M.G + go];
  const R* mu = V.ang + a.off;
  const R* pdf = mu + a.n;
  const R* cdf = pdf + a.n;
  int l = lower_bound<R>(cdf, a.n, xi);
  if (xi == cdf[l]) return mu[l];
  l--;
  R out;
  if (pdf[l] == pdf[l + 1]) {
    out = mu[l] + ((xi - cdf[l]) / pdf[l]);
  } else {
    R m = (pdf[l + 1] - pdf[l]) / (mu[l + 1] - mu[l]);
    R arg = pdf[l] * pdf[l] + R(2) * m * (xi - cdf[l]);
    if (sizeof(R) == 4 && arg < R(0)) arg = R(0);
    out = mu[l] + (R(1) / m) * (m_sqrt(arg) - pdf[l]);
  }
  if (sizeof(R) == 4) out = out < R(-1) ? R(-1) : (out > R(1) ? R(1) : out);  // FP32 rounding
  return out;
}

template <class R> ABX_DEV R group_mid(const View<R>& V, const ProbT& P, int g) {
  return R(0.5) * (V.ebnd[P.eb_off + g] + V.ebnd[P.eb_off + g + 1]);
}

// The neutrons of one fission event (Transporter::make_fission_neutrons,
// src/transporter.cpp:400-487; MGNuclide::sample_fission,
// src/mg_nuclide.cpp:504-544): per neutron a chi-row draw, an isotropic
// direction, the delayed test, then the site (k-eigenvalue) or a secondary
// on the history's stack (fixed source).  A few percent of collisions bank
// neutrons, so this runs out of line with scalar arguments and hands back
// the advanced random state.
struct FissionOut {
  uint64_t rng;
  uint32_t nsec;
};

template <class R>
ABX_DEV FissionOut fission_neutrons_body(const TransportArgs<R>& A, const R* chi, const R* ebnd,
                                                    const R* dgcdf, int G, int ndg, R P_delayed, int n_new,
                                                    uint64_t base, uint64_t rng, R rx, R ry, R rz, R ux, R uy,
                                                    R uz, bool positive, uint32_t h, uint32_t dau, uint32_t nsec,
                                                    bool keig) {
  const V3<R> u0 = mk<R>(ux, uy, uz);
  const R wgt = positive ? R(1) : R(-1);
  for (int i = 0; i < n_new; i++) {
    int ei = discrete<R>(rng, chi, G);
    R E_out = R(0.5) * (ebnd[ei] + ebnd[ei + 1]);  // group_mid
    R mu = R(2) * canon<R>(rng) - R(1);
    R c, s;
    azimuth(canon<R>(rng), c, s);
    V3<R> uo = rotate(u0, mu, c, s);
    if (canon<R>(rng) < P_delayed) (void)discrete<R>(rng, dgcdf, ndg);
    if (keig) {
      uint64_t j = base + i;
      if (j < A.site_cap) {
        A.sites.x[j] = rx; A.sites.y[j] = ry; A.sites.z[j] = rz;
        A.sites.ux[j] = uo.x; A.sites.uy[j] = uo.y; A.sites.uz[j] = uo.z;
        A.sites.E[j] = E_out; A.sites.w[j] = wgt;
        A.sites.hist[j] = h; A.sites.dau[j] = dau + (uint32_t)i;
      }
    } else {
      uint32_t gt = blockIdx.x * blockDim.x + threadIdx.x;
      if (nsec < A.sec_cap) {
        R* sp = A.sec + ((uint64_t)gt * A.sec_cap + nsec) * 9;
        sp[0] = rx; sp[1] = ry; sp[2] = rz;
        sp[3] = uo.x; sp[4] = uo.y; sp[5] = uo.z;
        sp[6] = E_out; sp[7] = wgt; sp[8] = R(0);
        nsec++;
      } else {
        raise_err(A.st, ABX_ERR_CAPACITY, h);
        atomicAdd(&A.st->sec_overflow, 1ull);
      }
    }
  }
  return FissionOut{rng, nsec};
}

// Out of line in FP32 tracking (measured faster on the 51x51-pin assembly), inline in FP64.
// The out-of-line function's name decides where it lands in the module; this
// placement measured 38 % faster on the nested-cylinder lattice than the alternatives tried.
template <class R>
__device__ __noinline__ FissionOut fission_neutrons(const TransportArgs<R>& A, const R* chi, const R* ebnd,
                                                        const R* dgcdf, int G, int ndg, R P_delayed, int n_new,
                                                        uint64_t base, uint64_t rng, R rx, R ry, R rz, R ux,
                                                        R uy, R uz, bool positive, uint32_t h, uint32_t dau,
                                                        uint32_t nsec, bool keig) {
  return fission_neutrons_body<R>(A, chi, ebnd, dgcdf, G, ndg, P_delayed, n_new, base, rng, rx, ry, rz, ux, uy, uz,
                                  positive, h, dau, nsec, keig);
}

template <class R>
ABX_DEV FissionOut fission_dispatch(const TransportArgs<R>& A, const R* chi, const R* ebnd, const R* dgcdf, int G,
                                    int ndg, R P_delayed, int n_new, uint64_t base, uint64_t rng, R rx, R ry, R rz,
                                    R ux, R uy, R uz, bool positive, uint32_t h, uint32_t dau, uint32_t nsec,
                                    bool keig) {
  if constexpr (sizeof(R) == 4)
    return fission_neutrons<R>(A, chi, ebnd, dgcdf, G, ndg, P_delayed, n_new, base, rng, rx, ry, rz, ux, uy, uz,
                                   positive, h, dau, nsec, keig);
  else
    return fission_neutrons_body<R>(A, chi, ebnd, dgcdf, G, ndg, P_delayed, n_new, base, rng, rx, ry, rz, ux, uy,
                                    uz, positive, h, dau, nsec, keig);
}

// Transporter::collision + branching_collision + russian_roulette +
// make_fission_neutrons + do_scatter (src/transporter.cpp:35-93, 269-347, 358-487),
// MGNuclide::sample_scatter / sample_fission (src/mg_nuclide.cpp:442-461, 504-544)
// Particle::split (include/simulation/particle.hpp:165-173): n > 1 particles
// of equal weight, the n - 1 copies on the history's secondary stack.
template <class R> ABX_DEV void split_lane(const TransportArgs<R>& A, Lane<R>& L, int n) {
  if (n <= 1) return;
  L.w = L.w / (R)n;
  L.w2 = L.w2 / (R)n;
  const uint32_t gt = blockIdx.x * blockDim.x + threadIdx.x;
  for (int i = 0; i < n - 1; i++) {
    if (L.nsec < A.sec_cap) {
      R* sp = A.sec + ((uint64_t)gt * A.sec_cap + L.nsec) * 9;
      sp[0] = L.r.x; sp[1] = L.r.y; sp[2] = L.r.z;
      sp[3] = L.u.x; sp[4] = L.u.y; sp[5] = L.u.z;
      sp[6] = L.E; sp[7] = L.w; sp[8] = L.w2;
      L.nsec++;
    } else {
      raise_err(A.st, ABX_ERR_CAPACITY, L.h);
      atomicAdd(&A.st->sec_overflow, 1ull);
      return;
    }
  }
}

// Transporter::branchless_collision_iso / branchless_collision_mat
// (src/transporter.cpp:95-267), after the collision scores: the collision
// either scatters, its weight multiplied by m = (nu Sigma_f + Sigma_s) /
// Sigma_t, or ends the history in one fission site of weight w m.  The
// per-nuclide form draws the nuclide, scores k_abs, plays roulette, then
// draws the reaction; the per-material form draws the reaction, then the
// nuclide, scores k_abs scaled by m / m_i, then plays roulette.  A scattered
// particle splits (floor(|w|) copies per nuclide, ceil(|w|) per material)
// when splitting is on and |w| reaches wgt_split.
template <class R, bool ISO>
ABX_DEV void branchless_collide(const TransportArgs<R>& A, const Tables& T, const View<R>& V, const ProbT& P,
                                const MatT& M, Lane<R>& L, Acc<R>& acc, bool& alive) {
  const int G = M.G, g = L.g;
  const R* xs = V.xs + M.xs_off;
  const R Et = xs[XS_ET * G + g];
  const R Eabs = xs[XS_EABS * G + g];
  const R Ef = xs[XS_EF * G + g];
  const R nu = xs[XS_NU * G + g];
  const bool per_mat = (P.branchless & ABX_BRANCHLESS_MATERIAL) != 0;
  bool scatter = false;
  R m;
  if (per_mat) {
    const R Es = xs[XS_ES * G + g];
    const R vEf = xs[XS_VEF * G + g];
    const R Pscatter = Es / (vEf + Es);
    m = (vEf + Es) / Et;
    scatter = canon<R>(L.rng) < Pscatter;
    (void)canon<R>(L.rng);  // sample_branchless_nuclide's draw (material_helper.hpp:226-271)
    const R m_i = (nu * Ef + (Et - Eabs)) / Et;
    acc.habs += (m / m_i) * L.w * nu * Ef / Et;
  } else {
    (void)canon<R>(L.rng);  // sample_nuclide's draw (material_helper.hpp:178-224)
    acc.habs += L.w * nu * Ef / Et;
  }
  const R Pscatter_iso = (Et - Eabs) / (nu * Ef + (Et - Eabs));
  if (!per_mat) m = (nu * Ef + (Et - Eabs)) / Et;
  // russian roulette (src/transporter.cpp:35-58)
  if (m_abs(L.w) < (R)P.wgt_cutoff) {
    R P_kill = R(1) - (m_abs(L.w) / (R)P.wgt_survival);
    if (canon<R>(L.rng) < P_kill) L.w = R(0);
    else L.w = copysign((R)P.wgt_survival, L.w);
  }
  if (m_abs(L.w2) < (R)P.wgt_cutoff) {
    R P_kill = R(1) - (m_abs(L.w2) / (R)P.wgt_survival);
    if (canon<R>(L.rng) < P_kill) L.w2 = R(0);
    else L.w2 = copysign((R)P.wgt_survival, L.w2);
  }
  const bool live = !(L.w == R(0) && L.w2 == R(0));
  if (live && !per_mat) scatter = canon<R>(L.rng) < Pscatter_iso;
  const bool fis = live && !scatter;
  // one atomic per warp reserves the sites of every lane that ends in fission
  uint64_t base = 0;
  if (__any_sync(__activemask(), fis)) {
    cg::coalesced_group grp = cg::coalesced_threads();
    const unsigned my = fis ? 1u : 0u;
    const unsigned pre = cg::exclusive_scan(grp, my);
    const unsigned tot = cg::reduce(grp, my, cg::plus<unsigned>());
    const double wsum = cg::reduce(grp, fis ? (double)(L.w * m) : 0., cg::plus<double>());
    unsigned long long b0 = 0;
    if (grp.thread_rank() == 0 && tot) {
      b0 = atomicAdd(&A.st->site_count, (unsigned long long)tot);
      atomicAdd(&A.st->site_wsum, wsum);
    }
    b0 = grp.shfl(b0, 0);
    base = b0 + pre;
  }
  if (!live) {
    alive = false;
  } else if (scatter) {
    int ei = discrete<R>(L.rng, V.cdf + M.cdf_off + g * G, G);
    R E_out = group_mid(V, P, ei);
    R mu = sample_mu<R, ISO>(T, V, M, g, ei, L.rng);
    R c, s;
    azimuth(canon<R>(L.rng), c, s);
    L.u = rotate(L.u, mu, c, s);
    L.E = E_out;
    L.g = ei;
    L.w = L.w * m * R(1);
    L.w2 = L.w2 * m * R(1);
    if ((double)L.E < P.min_energy) alive = false;
    if ((P.branchless & ABX_BRANCHLESS_SPLITTING) && alive && m_abs(L.w) >= (R)P.wgt_split)
      split_lane(A, L, per_mat ? (int)ceil((double)m_abs(L.w)) : (int)floor((double)m_abs(L.w)));
  } else {
    // MGNuclide::sample_fission (src/mg_nuclide.cpp:504-544), one neutron
    const R P_delayed = xs[XS_NUD * G + g] / nu;
    int ei = discrete<R>(L.rng, V.cdf + M.cdf_off + G * G + g * G, G);
    R E_out = group_mid(V, P, ei);
    R mu = R(2) * canon<R>(L.rng) - R(1);
    R c, s;
    azimuth(canon<R>(L.rng), c, s);
    const V3<R> uo = rotate(L.u, mu, c, s);
    if (canon<R>(L.rng) < P_delayed) (void)discrete<R>(L.rng, V.dgcdf + M.dg_off, M.ndg);
    const R wsite = L.w * m;
    if (base < A.site_cap) {
      A.sites.x[base] = L.r.x; A.sites.y[base] = L.r.y; A.sites.z[base] = L.r.z;
      A.sites.ux[base] = uo.x; A.sites.uy[base] = uo.y; A.sites.uz[base] = uo.z;
      A.sites.E[base] = E_out; A.sites.w[base] = wsite;
      A.sites.hist[base] = L.h; A.sites.dau[base] = L.dau;
    }
    L.dau++;
    if (wsite > R(0)) L.npos++;
    else L.nneg++;
    alive = false;
  }
}

// RESYNC reconverges the colliding lanes after the fission block (measured
// faster with surface tracking only).  BL: branchless collisions.
template <class R, bool ISO, bool RESYNC, bool BL>
ABX_DEV void collide(const TransportArgs<R>& A, const Tables& T, const View<R>& V, const ProbT& P,
                     Lane<R>& L, Acc<R>& acc, bool converged, R kcol, bool& alive) {
  const unsigned cmask = RESYNC ? __activemask() : 0u;
  const MatT M = T.mats[L.mat];
  const int G = M.G, g = L.g;
  const R* xs = V.xs + M.xs_off;
  if (converged && P.has_coll) score_collision(T, V, P, M, L);
  const R Et = xs[XS_ET * G + g];
  const R Eabs = xs[XS_EABS * G + g];
  const R Ef = xs[XS_EF * G + g];
  const R nu = xs[XS_NU * G + g];
  const R vEf = xs[XS_VEF * G + g];
  {
    R k_col_scr = L.w * vEf / Et;
    V3<R> dd = sub(L.r, L.rb);
    R mig_dist = m_sqrt(dd.x * dd.x + dd.y * dd.y + dd.z * dd.z);
    R mig_scr = L.w * Eabs / Et * mig_dist * mig_dist;
    acc.hcol += k_col_scr;
    acc.hmig += mig_scr;
  }
  if constexpr (BL) {
    branchless_collide<R, ISO>(A, T, V, P, M, L, acc, alive);
    return;
  }
  (void)canon<R>(L.rng);  // sample_nuclide's draw (include/materials/material_helper.hpp:189)
  acc.habs += L.w * nu * Ef / Et;
  {
    R kabs2 = L.w * nu * Ef / Et;
    int n_new;
    if (P.mode == ABX_MODE_K_EIGENVALUE) n_new = (int)m_floor(m_abs(kabs2) / kcol + canon<R>(L.rng));
    else n_new = (int)m_floor(m_abs(kabs2) + canon<R>(L.rng));
    if (n_new < 0) n_new = 0;
    R P_delayed = xs[XS_NUD * G + g] / nu;
    uint64_t base = 0;
    const bool keig = P.mode == ABX_MODE_K_EIGENVALUE;
    if (keig && __any_sync(__activemask(), n_new > 0)) {
      // one atomic per warp reserves the sites of every colliding lane
      cg::coalesced_group grp = cg::coalesced_threads();
      unsigned my = (unsigned)n_new;
      unsigned pre = cg::exclusive_scan(grp, my);
      unsigned tot = cg::reduce(grp, my, cg::plus<unsigned>());
      unsigned long long b0 = 0;
      if (grp.thread_rank() == 0 && tot) b0 = atomicAdd(&A.st->site_count, (unsigned long long)tot);
      b0 = grp.shfl(b0, 0);
      base = b0 + pre;
      if (L.w > R(0)) L.npos += (uint32_t)n_new;
      else L.nneg += (uint32_t)n_new;
    }
    if (n_new > 0) {
      const FissionOut o = fission_dispatch<R>(A, V.cdf + M.cdf_off + G * G + g * G, V.ebnd + P.eb_off,
                                               V.dgcdf + M.dg_off, G, M.ndg, P_delayed, n_new, base, L.rng,
                                               L.r.x, L.r.y, L.r.z, L.u.x, L.u.y, L.u.z, L.w > R(0), L.h, L.dau,
                                               L.nsec, keig);
      L.rng = o.rng;
      L.dau += (uint32_t)n_new;
      L.nsec = o.nsec;
    }
  }
  if (RESYNC) __syncwarp(cmask);
  // implicit capture
  L.w = L.w * (R(1) - (Eabs + R(0)) / Et);
  L.w2 = L.w2 * (R(1) - (Eabs + R(0)) / Et);
  // russian roulette
  if (m_abs(L.w) < (R)P.wgt_cutoff) {
    R P_kill = R(1) - (m_abs(L.w) / (R)P.wgt_survival);
    if (canon<R>(L.rng) < P_kill) L.w = R(0);
    else L.w = copysign((R)P.wgt_survival, L.w);
  }
  if (m_abs(L.w2) < (R)P.wgt_cutoff) {
    R P_kill = R(1) - (m_abs(L.w2) / (R)P.wgt_survival);
    if (canon<R>(L.rng) < P_kill) L.w2 = R(0);
    else L.w2 = copysign((R)P.wgt_survival, L.w2);
  }
  if (L.w == R(0) && L.w2 == R(0)) alive = false;
  if (alive) {
    int ei = discrete<R>(L.rng, V.cdf + M.cdf_off + g * G, G);
    R E_out = group_mid(V, P, ei);
    R mu = sample_mu<R, ISO>(T, V, M, g, ei, L.rng);
    R c, s;
    azimuth(canon<R>(L.rng), c, s);
    L.u = rotate(L.u, mu, c, s);
    L.E = E_out;
    L.g = ei;
    L.w = L.w * R(1);
    L.w2 = L.w2 * R(1);
    if ((double)L.E < P.min_energy) alive = false;
  }
}

}  // namespace abx
