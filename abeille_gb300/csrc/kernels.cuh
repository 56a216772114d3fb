// Transport kernels of the GB300 multigroup engine, templated on the tracking
// precision R.  Included by transport_fp64.cu (R = double, --fmad=false) and
// transport_mixed.cu (R = float).
//
// Design: one persistent launch per transport call.  Each lane owns one
// history at a time with its whole state (position, direction, weight, pcg32
// state and the geometry tree) in registers.  A lane whose history ends takes
// the next one from a global work counter (warp-aggregated), so lanes never
// wait for a slow neighbour ("lane refill"); every loop iteration advances
// each lane by exactly one flight, plus one collision when the flight ends in
// a real collision.  Fission sites are appended with warp-aggregated atomics
// and keyed by (history, daughter) so a counting sort restores the
// reference's bank order.
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
};

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
// global scores when it retires.  In FP64 mode every term is a double, so
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
  uint32_t events;
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

template <class R> ABX_DEV void trace_rec(const TransportArgs<R>& A, const Lane<R>& L, int kind, int cell) {
  if (L.h >= A.trace_nhist) return;
  unsigned long long i = atomicAdd(&A.st->trace_n, 1ull);
  if (i >= A.trace_cap) return;
  abx_trace_rec t;
  t.hist = L.h; t.kind = kind; t.group = L.g; t.cell = cell; t.rng_state = L.rng;
  t.r[0] = (double)L.r.x; t.r[1] = (double)L.r.y; t.r[2] = (double)L.r.z;
  t.u[0] = (double)L.u.x; t.u[1] = (double)L.u.y; t.u[2] = (double)L.u.z;
  t.wgt = (double)L.w;
  A.trace[i] = t;
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
ABX_DEV void score_flight(const Tables& T, const View<R>& V, const ProbT& P, const Lane<R>& L, R dfl) {
  const R* teb = tally_eb<R>(T);
  for (int ti = P.tally_first; ti < P.tally_first + P.tally_count; ti++) {
    const TallyT& t = T.tallies[ti];
    if (t.est != ABX_EST_TRACK_LENGTH) continue;
    R low[3], hi[3], d[3], dinv[3];
    tally_geom<R>(t, low, hi, d, dinv);
    V3<R> r = L.r;
    const V3<R> u = L.u;
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
    const MatT& M = T.mats[L.mat];
    R base = R(1) / (R)P.nparticles;
    base *= qfactor(V, M, t.quantity, L.g, L.w);
    int l = tally_ebin<R>(teb + t.eb_off, t.ne, L.E);
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
        atomicAdd(T.tally_gen + idx, (double)(dt * base));
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

// MGAngleDistribution::sample_mu (include/materials/mg_angle_distribution.hpp:45-60,92-101)
template <class R>
ABX_DEV R sample_mu(const Tables& T, const View<R>& V, const MatT& M, int gi, int go, uint64_t& rng) {
  const R xi = canon<R>(rng);
  if (M.iso) {
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
  if (pdf[l] == pdf[l + 1]) return mu[l] + ((xi - cdf[l]) / pdf[l]);
  R m = (pdf[l + 1] - pdf[l]) / (mu[l + 1] - mu[l]);
  return mu[l] + (R(1) / m) * (m_sqrt(pdf[l] * pdf[l] + R(2) * m * (xi - cdf[l])) - pdf[l]);
}

template <class R> ABX_DEV R group_mid(const View<R>& V, const ProbT& P, int g) {
  return R(0.5) * (V.ebnd[P.eb_off + g] + V.ebnd[P.eb_off + g + 1]);
}

// Transporter::collision + branching_collision + russian_roulette +
// make_fission_neutrons + do_scatter (src/transporter.cpp:35-93, 269-347, 358-487),
// MGNuclide::sample_scatter / sample_fission (src/mg_nuclide.cpp:442-461, 504-544)
template <class R>
ABX_DEV void collide(const TransportArgs<R>& A, const Tables& T, const View<R>& V, const ProbT& P,
                     Lane<R>& L, Acc<R>& acc, bool converged, R kcol, bool& alive) {
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
    if (keig) {
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
    const R* chi = V.cdf + M.cdf_off + G * G + g * G;
    for (int i = 0; i < n_new; i++) {
      int ei = discrete<R>(L.rng, chi, G);
      R E_out = group_mid(V, P, ei);
      R mu = R(2) * canon<R>(L.rng) - R(1);
      R c, s;
      azimuth(canon<R>(L.rng), c, s);
      V3<R> uo = rotate(L.u, mu, c, s);
      if (canon<R>(L.rng) < P_delayed) (void)discrete<R>(L.rng, V.dgcdf + M.dg_off, M.ndg);
      R wgt = L.w > R(0) ? R(1) : R(-1);
      if (keig) {
        uint64_t j = base + i;
        if (j < A.site_cap) {
          A.sites.x[j] = L.r.x; A.sites.y[j] = L.r.y; A.sites.z[j] = L.r.z;
          A.sites.ux[j] = uo.x; A.sites.uy[j] = uo.y; A.sites.uz[j] = uo.z;
          A.sites.E[j] = E_out; A.sites.w[j] = wgt;
          A.sites.hist[j] = L.h; A.sites.dau[j] = L.dau;
        }
        L.dau++;
      } else {
        L.dau++;
        uint32_t gt = blockIdx.x * blockDim.x + threadIdx.x;
        if (L.nsec < A.sec_cap) {
          R* sp = A.sec + ((uint64_t)gt * A.sec_cap + L.nsec) * 9;
          sp[0] = L.r.x; sp[1] = L.r.y; sp[2] = L.r.z;
          sp[3] = uo.x; sp[4] = uo.y; sp[5] = uo.z;
          sp[6] = E_out; sp[7] = wgt; sp[8] = R(0);
          L.nsec++;
        } else {
          raise_err(A.st, ABX_ERR_CAPACITY, L.h);
          atomicAdd(&A.st->sec_overflow, 1ull);
        }
      }
    }
  }
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
    R mu = sample_mu(T, V, M, g, ei, L.rng);
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

template <class R>
ABX_DEV void do_reflection(const Tables& T, const View<R>& V, const ProbT& P, Trk<R>& k, Lane<R>& L, const Bound<R>& b) {
  // Tracker::do_reflection (tracker.hpp:314-359); the surface token it sets is
  // cleared by set_r, and previous-position bookkeeping only feeds cancellation.
  const SurfT<R> s = V.surf[b.si];
  V3<R> r_on = add(L.r, scl(L.u, b.dist));
  if (sizeof(R) == 4) {  // mixed mode: put the point exactly on an axis plane
    if (s.type == ABX_SURF_XPLANE) r_on.x = s.c[0];
    else if (s.type == ABX_SURF_YPLANE) r_on.y = s.c[0];
    else if (s.type == ABX_SURF_ZPLANE) r_on.z = s.c[0];
  }
  V3<R> n = surf_norm(s, r_on);
  R c2 = R(2) * dot(L.u, n);
  V3<R> nd = sub(L.u, scl(n, c2));
  // the side token the reference computes before set_r clears it
  const int32_t side = sizeof(R) == 4 && b.token != 0 ? b.token
                       : (surf_sign(s, L.r, L.u) < 0 ? -(b.si + 1) : (b.si + 1));
  L.r = r_on;
  L.u = dir3(nd.x, nd.y, nd.z);
  trk_set_r(k, L.r);
  k.u = L.u;
  // Mixed mode keeps it: the particle sits on the plane, and with no FP32
  // distance band the token is what marks that plane as the one it is on.
  if (sizeof(R) == 4) k.token = side;
  trk_restart(T, V, P, k);
}

// Load history h into a lane and locate it (Tracker ctor, DeltaTracker::transport
// src/delta_tracker.cpp:87-103).
template <class R>
ABX_DEV bool lane_load(const TransportArgs<R>& A, const Tables& T, const View<R>& V, Lane<R>& L, Trk<R>& k, uint32_t h) {
  L.h = h;
  L.r = mk<R>(A.bank.x[h], A.bank.y[h], A.bank.z[h]);
  L.u = mk<R>(A.bank.ux[h], A.bank.uy[h], A.bank.uz[h]);
  L.E = A.bank.E[h];
  L.w = A.bank.w[h];
  L.w2 = A.bank.w2 ? A.bank.w2[h] : R(0);
  L.rng = A.bank.rng[h];
  L.pid = A.bank.prob ? A.bank.prob[h] : 0;
  L.rb = L.r;
  L.dau = 0;
  L.nsec = 0;
  L.events = 0;
  const ProbT& P = T.probs[L.pid];
  L.g = group_of<R>(V.ebnd + P.eb_off, P.G, L.E);
  k.r = L.r; k.u = L.u; k.token = 0; k.err = 0;
  if (L.g >= P.G) {  // energy outside the group structure
    k.err = ABX_ERR_INVALID;
    L.mat = -1;
    return false;
  }
  trk_restart(T, V, P, k);
  if (k.cell < 0) {
    L.mat = -1;
    return false;
  }
  L.mat = T.cells[k.cell].fill;
  return true;
}

template <class R, int TRACK>
__global__ void __launch_bounds__(256, 2) transport_kernel(const TransportArgs<R> A) {
  const bool TRACE = A.trace != nullptr;
  const Tables& T = A.T;
  const View<R> V = make_view<R>(T);
  DevState* st = A.st;
  const unsigned lane = threadIdx.x & 31u;
  const unsigned long long n_hist = st->n_hist;
  const R kcol = (R)st->kcol;
  const bool converged = st->converged != 0;

  __shared__ double sh_acc[5];
  if (threadIdx.x < 5) sh_acc[threadIdx.x] = 0.;
  __syncthreads();

  Lane<R> L;
  Trk<R> k;
  Acc<R> acc;
  uint32_t ncoll = 0, nflight = 0, nlost = 0;
  bool active = false, done = false;
  L.h = 0xffffffffu;
  L.pid = 0;
  L.mat = -1;
  L.nsec = 0;
  L.dau = 0;
  L.npos = 0;
  L.nneg = 0;
  k.depth = 0;

  while (true) {
    // ------------------------------------------------ lane refill
    bool need = !active && !done;
    unsigned m = __ballot_sync(0xffffffffu, need);
    if (m) {
      unsigned leader = __ffs(m) - 1;
      unsigned long long base = 0;
      if (lane == leader) base = atomicAdd(&st->next_hist, (unsigned long long)__popc(m));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (need) {
        unsigned long long h = base + __popc(m & ((1u << lane) - 1u));
        if (h >= n_hist || st->err) {
          done = true;
        } else {
          active = lane_load(A, T, V, L, k, (uint32_t)h);
          if (k.err) { raise_err(st, k.err, L.h); done = true; active = false; }
          else if (!active) {
            nlost++;
            A.hist_count[h] = 0;
          }
        }
      }
    }
    if (__all_sync(0xffffffffu, done)) break;
    if (!active) continue;

    // ------------------------------------------------ one flight
    const ProbT& P = T.probs[L.pid];
    bool alive = true;
    bool had_collision = false;
    L.events++;
    nflight++;
    if (TRACK == ABX_TRACK_DELTA) {
      const R Emaj = V.maj[P.maj_off + L.g];
      R d_coll = Emaj == R(0) ? Tol<R>::INF : -m_log(R(1) - canon<R>(L.rng)) / Emaj;
      Bound<R> bound{Tol<R>::INF, -1, ABX_BC_NORMAL, 0};
      bool crossed = false;
      trk_move(k, d_coll);
      trk_current(T, V, P, k);
      if (k.cell < 0) {
        trk_set_r(k, L.r);
        trk_current(T, V, P, k);
        // Mixed mode: the search is direction-aware at axis planes, so a
        // particle within the FP32 coincidence band of the wall it leaves
        // through finds that wall (trk_bc_mixed).
        bound = sizeof(R) == 8 ? trk_bc(T, V, P, k) : trk_bc_mixed(T, V, P, k);
        crossed = true;
      }
      if (converged && P.has_tle) score_flight(T, V, P, L, d_coll < bound.dist ? d_coll : bound.dist);
      if (crossed) {
        if (bound.btype == ABX_BC_VACUUM) {
          alive = false;
          acc.hleak += L.w;
          V3<R> rl = add(L.r, scl(L.u, bound.dist));
          V3<R> dl = sub(rl, L.rb);
          acc.hmig += dot(scl(dl, L.w), dl);
          if (TRACE) trace_rec(A, L, 2, k.cell);
        } else if (bound.btype == ABX_BC_REFLECTIVE) {
          do_reflection(T, V, P, k, L, bound);
          if (k.cell < 0) {
            if (sizeof(R) == 8) { raise_err(st, ABX_ERR_LOST_PARTICLE, L.h); done = true; active = false; continue; }
            nlost++;  // mixed mode: counted in `lost` and killed
            alive = false;
          }
          if (TRACE) trace_rec(A, L, 3, k.cell);
        } else {
          if (sizeof(R) == 8) { raise_err(st, ABX_ERR_LOST_PARTICLE, L.h); done = true; active = false; continue; }
          nlost++;
          alive = false;
        }
      } else {
        L.r = add(L.r, scl(L.u, d_coll));
        L.mat = T.cells[k.cell].fill;
        const MatT& M = T.mats[L.mat];
        const R Et = V.xs[M.xs_off + XS_ET * M.G + L.g];
        if (Et - Emaj > Tol<R>::MAJ) { raise_err(st, ABX_ERR_MAJORANT, L.h); done = true; active = false; continue; }
        if (canon<R>(L.rng) < (Et / Emaj)) had_collision = true;
        if (TRACE) trace_rec(A, L, had_collision ? 1 : 0, k.cell);
      }
    } else {
      const MatT& M = T.mats[L.mat];
      const R Et = V.xs[M.xs_off + XS_ET * M.G + L.g];
      R d_coll = Et == R(0) ? Tol<R>::INF : -m_log(R(1) - canon<R>(L.rng)) / Et;
      Bound<R> bound = sizeof(R) == 8 ? trk_nearest(T, V, P, k) : trk_nearest_mixed(T, V, P, k);
      R dmin = d_coll < bound.dist ? d_coll : bound.dist;
      if (converged && P.has_tle) score_flight(T, V, P, L, dmin);
      acc.htrk += L.w * dmin * V.xs[M.xs_off + XS_VEF * M.G + L.g];
      if (bound.dist < d_coll || m_abs(bound.dist - d_coll) < Tol<R>::BTOL) {
        if (bound.btype == ABX_BC_VACUUM) {
          alive = false;
          acc.hleak += L.w;
          V3<R> rl = add(L.r, scl(L.u, bound.dist));
          V3<R> dl = sub(rl, L.rb);
          acc.hmig += dot(scl(dl, L.w), dl);
          if (TRACE) trace_rec(A, L, 2, k.cell);
        } else if (bound.btype == ABX_BC_REFLECTIVE) {
          do_reflection(T, V, P, k, L, bound);
          if (k.cell < 0) {
            if (sizeof(R) == 8) { raise_err(st, ABX_ERR_LOST_PARTICLE, L.h); done = true; active = false; continue; }
            nlost++;  // mixed mode: counted in `lost` and killed
            alive = false;
          }
          if (TRACE) trace_rec(A, L, 3, k.cell);
        } else {
          const int prev = k.cell;
          trk_move(k, bound.dist);
          k.token = -bound.token;
          trk_current(T, V, P, k);
          L.r = add(L.r, scl(L.u, bound.dist));
          if (sizeof(R) == 4 && (k.cell < 0 || (k.cell == prev && bound.dist == R(0)))) {
            // mixed mode: step off a surface crossing FP32 cannot resolve
            L.r = add(L.r, scl(L.u, R(4) * Tol<R>::SC));
            trk_set_r(k, L.r);
            trk_restart(T, V, P, k);
          }
          if (k.cell < 0) {
            if (sizeof(R) == 8) { raise_err(st, ABX_ERR_LOST_PARTICLE, L.h); done = true; active = false; continue; }
            nlost++;
            alive = false;
          } else {
            L.mat = T.cells[k.cell].fill;
          }
          if (TRACE) trace_rec(A, L, 5, k.cell);
        }
      } else {
        L.r = add(L.r, scl(L.u, d_coll));
        trk_move(k, d_coll);
        had_collision = true;
        if (TRACE) trace_rec(A, L, 1, k.cell);
      }
    }
    if (k.err) { raise_err(st, k.err, L.h); done = true; active = false; continue; }
    if (alive && had_collision) {
      ncoll++;
      collide(A, T, V, P, L, acc, converged, kcol, alive);
      k.u = L.u;
      if (TRACE) trace_rec(A, L, 4, k.cell);
    }
    if (!alive) {
      if (L.nsec > 0) {
        // Particle::resurect (include/simulation/particle.hpp:170-182)
        L.nsec--;
        uint32_t gt = blockIdx.x * blockDim.x + threadIdx.x;
        const R* sp = A.sec + ((uint64_t)gt * A.sec_cap + L.nsec) * 9;
        L.r = mk<R>(sp[0], sp[1], sp[2]);
        L.u = mk<R>(sp[3], sp[4], sp[5]);
        L.E = sp[6]; L.w = sp[7]; L.w2 = sp[8];
        L.g = group_of<R>(V.ebnd + P.eb_off, P.G, L.E);
        if (L.g >= P.G) { raise_err(st, ABX_ERR_INVALID, L.h); done = true; active = false; continue; }
        trk_set_r(k, L.r);
        k.u = L.u;
        trk_restart(T, V, P, k);
        if (k.cell < 0 || k.err) { raise_err(st, ABX_ERR_LOST_PARTICLE, L.h); done = true; active = false; continue; }
        L.mat = T.cells[k.cell].fill;
        if (TRACE) trace_rec(A, L, 6, k.cell);
      } else {
        A.hist_count[L.h] = L.dau;
        acc.flush(sh_acc);
        active = false;
      }
    } else if (sizeof(R) == 4 && L.events > 100000u) {
      // mixed mode: a history this long is a geometry rounding trap, not
      // physics; it is counted in `lost` and ended
      nlost++;
      A.hist_count[L.h] = L.dau;
      acc.flush(sh_acc);
      active = false;
    } else if (L.events > A.max_events) {
      raise_err(st, ABX_ERR_TIMEOUT, L.h);
      done = true;
      active = false;
    }
  }
  acc.flush(sh_acc);
  unsigned long long c[5] = {ncoll, nflight, nlost, (unsigned long long)L.npos, (unsigned long long)L.nneg};
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
    for (int i = 0; i < 5; i++) c[i] += __shfl_down_sync(0xffffffffu, c[i], o);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    atomicAdd(&st->scores[0], sh_acc[0]);
    atomicAdd(&st->scores[1], sh_acc[1]);
    atomicAdd(&st->scores[2], sh_acc[2]);
    atomicAdd(&st->scores[4], sh_acc[3]);
    atomicAdd(&st->scores[5], sh_acc[4]);
  }
  if (lane == 0) {
    atomicAdd(&st->collisions, c[0]);
    atomicAdd(&st->flights, c[1]);
    atomicAdd(&st->lost, c[2]);
    atomicAdd(&st->site_pos, c[3]);
    atomicAdd(&st->site_neg, c[4]);
  }
}

}  // namespace abx
