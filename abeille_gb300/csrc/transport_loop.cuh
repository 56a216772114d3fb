// The transport loop: one persistent launch, one lane per history, written as
// a per-lane event state machine.
//
// Every lane keeps its history's state in registers and sits in one phase.
// Each pass of the loop visits the phases in a fixed order, and the lanes in
// a phase execute it together: refill (take the next history), flight
// (sample a distance, move, check the geometry tree), descend (re-locate in
// the CSG tree: the only copy of the descent code), start / reflect / cross /
// resurrect checks, moved (real-or-virtual test), boundary (leak or reflect),
// collide, dead.  A lane runs through as many phases per pass as its history
// allows (a tile crossing followed by a real collision is one pass).  Each
// history still performs exactly the reference's sequence of operations and
// draws; only the interleaving across lanes changes.
#pragma once

#include "kernels.cuh"

namespace abx {

enum : int {
  PH_REFILL = 0,
  PH_WAIT,     // waiting for the descend phase; continues in `after`
  PH_START,
  PH_FLIGHT,
  PH_MOVED,
  PH_LOST,
  PH_REFL,
  PH_CROSSED,
  PH_COLL,
  PH_DEAD,
  PH_RES,
  PH_DONE
};

// Load history h into a lane (DeltaTracker::transport, src/delta_tracker.cpp:87-103);
// its location is found by the next descend phase.
template <class R, bool SINGLE>
ABX_DEV bool lane_load(const TransportArgs<R>& A, const Tables& T, const View<R>& V, Lane<R>& L, Trk<R>& k,
                       uint32_t h) {
  L.h = h;
  L.r = mk<R>(A.bank.x[h], A.bank.y[h], A.bank.z[h]);
  L.u = mk<R>(A.bank.ux[h], A.bank.uy[h], A.bank.uz[h]);
  L.E = A.bank.E[h];
  L.w = A.bank.w[h];
  L.w2 = A.bank.w2 ? A.bank.w2[h] : R(0);
  L.rng = A.bank.rng[h];
  L.pid = (!SINGLE && A.bank.prob) ? A.bank.prob[h] : 0;
  L.rb = L.r;
  L.dau = 0;
  L.nsec = 0;
  L.events = 0;
  L.hcoll = 0;
  const ProbT& P = T.probs[SINGLE ? 0 : L.pid];
  L.g = group_of<R>(V.ebnd + P.eb_off, P.G, L.E);
  k.r = L.r;
  k.u = L.u;
  k.token = 0;
  k.err = 0;
  k.depth = 0;
  if (L.g >= P.G) {  // energy outside the group structure
    k.err = ABX_ERR_INVALID;
    return false;
  }
  return true;
}

// Tracker::do_reflection (tracker.hpp:314-359) without the re-location, which
// the descend phase performs.  The surface token it sets is cleared by set_r
// in the reference; the mixed mode keeps it (the particle sits on the plane
// and, with no FP32 distance band, the token marks it as the one it is on).
// Previous-position bookkeeping only feeds cancellation and is not carried.
template <class R>
ABX_DEV void reflect_move(const View<R>& V, Trk<R>& k, Lane<R>& L, const Bound<R>& b) {
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
  const int32_t side = sizeof(R) == 4 && b.token != 0 ? b.token
                       : (surf_sign(s, L.r, L.u) < 0 ? -(b.si + 1) : (b.si + 1));
  L.r = r_on;
  L.u = dir3(nd.x, nd.y, nd.z);
  trk_set_r(k, L.r);
  k.u = L.u;
  if (sizeof(R) == 4) k.token = side;
}

// rare and long: the boundary-condition search runs out of line
template <class R>
__device__ __noinline__ Bound<R> trk_bc_ool(const Tables& T, const ProbT& P, const Trk<R>& k) {
  const View<R> V = make_view<R>(T);
  return sizeof(R) == 8 ? trk_bc(T, V, P, k) : trk_bc_mixed(T, V, P, k);
}

// Particle::split (include/simulation/particle.hpp:165-173) as Carter tracking
// applies it after every collision, real or virtual (src/carter_tracker.cpp:
// 218-222): a weight of magnitude wgt_split or more becomes ceil(|w|)
// particles of equal weight, the copies on the history's secondary stack.
template <class R>
ABX_DEV void carter_split(const TransportArgs<R>& A, const ProbT& P, Lane<R>& L) {
  if (!(m_abs(L.w) >= (R)P.wgt_split)) return;
  const int n_new = (int)ceil((double)m_abs(L.w));
  if (n_new <= 1) return;
  L.w = L.w / (R)n_new;
  L.w2 = L.w2 / (R)n_new;
  const uint32_t gt = blockIdx.x * blockDim.x + threadIdx.x;
  for (int i = 0; i < n_new - 1; i++) {
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

// End of a history: its fission-site count (for the bank sort) and its score
// totals, to the block's accumulators or, in a batch of problems, to its
// problem's sums and counters.
template <class R, bool SINGLE>
ABX_DEV void history_end(const TransportArgs<R>& A, const Lane<R>& L, Acc<R>& acc, double* sh_acc) {
  A.hist_count[L.h] = L.dau;
  if (!SINGLE && A.pscore) {
    acc.flush(A.pscore + (size_t)L.pid * ABX_PSCORES);
    unsigned long long* c = A.pcount + (size_t)L.pid * ABX_PCOUNTS;
    atomicAdd(c + 0, (unsigned long long)L.hcoll);
    atomicAdd(c + 1, (unsigned long long)L.events);
    atomicAdd(c + 2, 1ull);
  } else {
    acc.flush(sh_acc);
  }
}

// Occupancy (measured on the 51x51-pin assembly and the 70-group
// nested-cylinder lattice): FP32 delta tracking (and implicit-leakage delta
// tracking) runs four 256-thread blocks per SM (64 registers), FP32 surface
// tracking three (80 registers), FP64 three (80) or, for large launches
// (ABX_KERNEL_WIDE), four (64).
// TRACK: the tracking mode, or'd with ABX_KERNEL_BRANCHLESS for the
// branchless collisions of the branchless k-eigenvalue simulation.
template <class R, int TRACK, bool ISO>
__global__ void __launch_bounds__(256, sizeof(R) == 4 ? ((TRACK & 0xff) != ABX_TRACK_SURFACE ? 4 : 3)
                                                    : ((TRACK & ABX_KERNEL_WIDE) ? 4 : 3))
    transport_kernel(const __grid_constant__ TransportArgs<R> A) {
  constexpr int TRK = TRACK & 0xff;
  constexpr bool BL = (TRACK & ABX_KERNEL_BRANCHLESS) != 0;
  constexpr bool SINGLE = (TRACK & ABX_KERNEL_SINGLE) != 0;
  // Event traces are a parity-test hook of the FP64 mode (abx_set_trace
  // refuses mixed contexts): the FP32 kernels carry none of their code
  // (the nested-cylinder lattice +5 %, the pin assembly within noise).
  const bool TRACE = sizeof(R) == 8 && A.trace != nullptr;
  const Tables& T = A.T;
  const View<R> V = make_view<R>(T);
  DevState* st = A.st;
  const unsigned lane = threadIdx.x & 31u;
  const unsigned long long n_hist = st->n_hist;
  const R kcol = (R)st->kcol;
  const bool converged = st->converged != 0;
  const uint32_t ev_limit = sizeof(R) == 4 ? 100000u : (uint32_t)(A.max_events < 0xffffffffull ? A.max_events : 0xffffffffull);

  __shared__ double sh_acc[5];
  if (threadIdx.x < 5) sh_acc[threadIdx.x] = 0.;
  __syncthreads();

  Lane<R> L;
  Trk<R> k;
  Acc<R> acc;
  uint32_t ncoll = 0, nflight = 0, nlost = 0;
  int ph = PH_REFILL, after = PH_REFILL, dmode = 0, dui = 0, dfr = 0, prev_cell = -1;
  R dcol = R(0);
  bool done = false;
  L.h = 0xffffffffu;
  L.pid = 0;
  L.mat = -1;
  L.nsec = 0;
  L.dau = 0;
  L.npos = 0;
  L.nneg = 0;
  L.events = 0;
  L.g = 0;
  k.depth = 0;
  k.cell = -1;
  k.err = 0;

#define ABX_FAIL(code)            \
  {                               \
    raise_err(st, (code), L.h);   \
    done = true;                  \
    ph = PH_DONE;                 \
  }
#define ABX_LOST()                                                                              \
  {                                                                                             \
    nlost++;                                                                                    \
    if (!SINGLE && A.pcount) atomicAdd(A.pcount + (size_t)L.pid * ABX_PCOUNTS + 3, 1ull);       \
    if (TRACE) trace_rec(A, L, 7, k.cell);                                                      \
  }

  uint32_t wtaken = 0;  // histories this warp took (warp-uniform)
  while (true) {
    // ---------------------------------------------------------------- refill
    const bool need = ph == PH_REFILL && !done;
    const unsigned m = __ballot_sync(0xffffffffu, need);
    if (m) {
      const unsigned leader = __ffs(m) - 1;
      const bool quota_left = A.warp_quota == 0 || wtaken < A.warp_quota;
      unsigned long long base = 0;
      if (lane == leader && quota_left) base = atomicAdd(&st->next_hist, (unsigned long long)__popc(m));
      base = __shfl_sync(0xffffffffu, base, leader);
      wtaken += __popc(m);
      if (need) {
        const unsigned long long h = base + __popc(m & ((1u << lane) - 1u));
        if (!quota_left || h >= n_hist || st->err) {
          done = true;
          ph = PH_DONE;
        } else if (!lane_load<R, SINGLE>(A, T, V, L, k, (uint32_t)h)) {
          ABX_FAIL(k.err);
        } else {
          dmode = 1;
          after = PH_START;
          ph = PH_WAIT;
        }
      }
    }
    if (__all_sync(0xffffffffu, done)) break;

    // ---------------------------------------------------------------- flight
    if (ph == PH_FLIGHT) {
      const ProbT& P = T.probs[SINGLE ? 0 : L.pid];
      L.events++;
      nflight++;
      if (TRK == ABX_TRACK_IMPLICIT_LEAKAGE) {
        // ImplicitLeakageDeltaTracker::transport
        // (src/implicit_leakage_delta_tracker.cpp:104-214): the nearest
        // boundary condition before every flight; towards a vacuum boundary
        // the weight that would leak is scored at once and the flight is
        // sampled within the boundary distance.
        const R Emaj = V.maj[P.maj_off + L.g];
        const Bound<R> b = trk_bc_ool<R>(T, P, k);
        if (b.btype == ABX_BC_VACUUM) {
          const R P_leak = m_exp(-Emaj * b.dist);
          const R P_no_leak = R(1) - P_leak;
          const R wgt_leak = L.w * P_leak, wgt2_leak = L.w2 * P_leak;
          const R wgt_coll = L.w * P_no_leak, wgt2_coll = L.w2 * P_no_leak;
          acc.hleak += wgt_leak;
          const V3<R> dl = sub(add(L.r, scl(L.u, b.dist)), L.rb);
          acc.hmig += dot(scl(dl, wgt_leak), dl);
          dcol = -m_log(R(1) - P_no_leak * canon<R>(L.rng)) / Emaj;
          if (converged && P.has_tle) {
            L.w = wgt_leak;
            L.w2 = wgt2_leak;
            score_flight(T, V, P, L, b.dist);
          }
          L.w = wgt_coll;
          L.w2 = wgt2_coll;
          if (converged && P.has_tle) score_flight(T, V, P, L, dcol);
        } else {
          dcol = Emaj == R(0) ? Tol<R>::INF : -m_log(R(1) - canon<R>(L.rng)) / Emaj;
          if (converged && P.has_tle) score_flight(T, V, P, L, dcol < b.dist ? dcol : b.dist);
        }
        if (b.dist < dcol || m_abs(b.dist - dcol) < Tol<R>::BTOL) {
          if (b.btype == ABX_BC_VACUUM) {
            acc.hleak += L.w;
            const V3<R> dl = sub(add(L.r, scl(L.u, b.dist)), L.rb);
            acc.hmig += dot(scl(dl, L.w), dl);
            if (TRACE) trace_rec(A, L, 2, k.cell);
            ph = PH_DEAD;
          } else if (b.btype == ABX_BC_REFLECTIVE) {
            reflect_move(V, k, L, b);
            dmode = 1;
            after = PH_REFL;
            ph = PH_WAIT;
          } else if (sizeof(R) == 8) {
            ABX_FAIL(ABX_ERR_LOST_PARTICLE);
          } else {
            ABX_LOST();
            ph = PH_DEAD;
          }
        } else {
          trk_move(k, dcol);
          const int r = trk_check(T, V, k, dui, dfr);
          if (r) {
            dmode = r;
            after = PH_MOVED;
            ph = PH_WAIT;
          } else {
            ph = PH_MOVED;
          }
        }
      } else if (TRK == ABX_TRACK_DELTA || TRK == ABX_TRACK_CARTER) {
        // DeltaTracker::transport (src/delta_tracker.cpp:105-118); Carter
        // tracking flies the same way on its sampling cross section
        // (src/carter_tracker.cpp:124-138), stored after the majorant
        const R Emaj = V.maj[P.maj_off + (TRK == ABX_TRACK_CARTER ? P.G : 0) + L.g];
        dcol = Emaj == R(0) ? Tol<R>::INF : -m_log(R(1) - canon<R>(L.rng)) / Emaj;
        trk_move(k, dcol);
        const int r = trk_check(T, V, k, dui, dfr);
        if (r) {
          dmode = r;
          after = PH_MOVED;
          ph = PH_WAIT;
        } else {
          ph = PH_MOVED;
        }
      } else {
        // SurfaceTracker::transport (src/surface_tracker.cpp:72-150)
        const MatT& M = T.mats[L.mat];
        const R Et = V.xs[M.xs_off + XS_ET * M.G + L.g];
        dcol = Et == R(0) ? Tol<R>::INF : -m_log(R(1) - canon<R>(L.rng)) / Et;
        const Bound<R> b = sizeof(R) == 8 ? trk_nearest(T, V, P, k) : trk_nearest_mixed(T, V, P, k);
        const R dmin = dcol < b.dist ? dcol : b.dist;
        if (converged && P.has_tle) score_flight(T, V, P, L, dmin);
        acc.htrk += L.w * dmin * V.xs[M.xs_off + XS_VEF * M.G + L.g];
        if (b.dist < dcol || m_abs(b.dist - dcol) < Tol<R>::BTOL) {
          if (b.btype == ABX_BC_VACUUM) {
            acc.hleak += L.w;
            const V3<R> dl = sub(add(L.r, scl(L.u, b.dist)), L.rb);
            acc.hmig += dot(scl(dl, L.w), dl);
            if (TRACE) trace_rec(A, L, 2, k.cell);
            ph = PH_DEAD;
          } else if (b.btype == ABX_BC_REFLECTIVE) {
            reflect_move(V, k, L, b);
            dmode = 1;
            after = PH_REFL;
            ph = PH_WAIT;
          } else {
            // Tracker::cross_surface + get_current (tracker.hpp:227-231)
            prev_cell = k.cell;
            trk_move(k, b.dist);
            k.token = -b.token;
            L.r = add(L.r, scl(L.u, b.dist));
            dcol = b.dist;
            const int r = trk_check(T, V, k, dui, dfr);
            if (r) {
              dmode = r;
              after = PH_CROSSED;
              ph = PH_WAIT;
            } else {
              ph = PH_CROSSED;
            }
          }
        } else {
          L.r = add(L.r, scl(L.u, dcol));
          trk_move(k, dcol);
          if (TRACE) trace_rec(A, L, 1, k.cell);
          ph = PH_COLL;
        }
      }
    }

    // --------------------------------------------------------------- descend
    // Every phase starts at an explicit warp reconvergence point: the lanes
    // that arrive from different branches of the previous phase run it
    // together (measured faster than the compiler's own reconvergence).
    __syncwarp();
    if (ph == PH_WAIT) {
      // CellUniverse/RectLattice::get_cell: re-descent from the first invalid
      // pad, or from the root (restart_get_current) when that fails or when the
      // tree must be rebuilt.
      const ProbT& P = T.probs[SINGLE ? 0 : L.pid];
      int cell = -1;
      if (dmode == 2) {
        cell = univ_get_cell(T, V, k, dui, dfr, k.getfr(dfr));
        if (cell < 0) dmode = 1;
      }
      if (dmode == 1) {
        k.depth = 0;
        cell = univ_get_cell(T, V, k, P.root, 0, k.r);
      }
      k.cell = cell;
      dmode = 0;
      ph = after;
      if (k.err) ABX_FAIL(k.err);
    }

    // ------------------------------------------------ post-descend checks
    __syncwarp();
    if (ph == PH_START) {
      if (k.cell < 0) {  // lost at birth: a warning in the reference, the particle is killed
        ABX_LOST();
        history_end<R, SINGLE>(A, L, acc, sh_acc);
        ph = PH_REFILL;
      } else {
        L.mat = T.cells[k.cell].fill;
        ph = PH_FLIGHT;
      }
    } else if (ph == PH_RES) {
      if (k.cell < 0) {
        // a secondary starting on a boundary that FP32 rounding puts outside:
        // counted in `lost` and killed in the mixed mode, fatal in FP64
        if (sizeof(R) == 8) ABX_FAIL(ABX_ERR_LOST_PARTICLE) else {
          ABX_LOST();
          ph = PH_DEAD;
        }
      } else {
        L.mat = T.cells[k.cell].fill;
        if (TRACE) trace_rec(A, L, 6, k.cell);
        ph = PH_FLIGHT;
      }
    } else if (ph == PH_REFL) {
      if (k.cell < 0) {
        if (sizeof(R) == 8) ABX_FAIL(ABX_ERR_LOST_PARTICLE) else {
          ABX_LOST();  // mixed mode: counted in `lost` and killed
          ph = PH_DEAD;
        }
      } else {
        if (TRACE) trace_rec(A, L, 3, k.cell);
        ph = PH_FLIGHT;
      }
    } else if (ph == PH_CROSSED) {
      if (sizeof(R) == 4 && prev_cell != -2 && (k.cell < 0 || (k.cell == prev_cell && dcol == R(0)))) {
        // mixed mode: step off a surface crossing FP32 cannot resolve
        L.r = add(L.r, scl(L.u, R(4) * Tol<R>::SC));
        trk_set_r(k, L.r);
        prev_cell = -2;
        dmode = 1;
        after = PH_CROSSED;
        ph = PH_WAIT;
      } else if (k.cell < 0) {
        if (sizeof(R) == 8) ABX_FAIL(ABX_ERR_LOST_PARTICLE) else {
          ABX_LOST();
          ph = PH_DEAD;
        }
      } else {
        L.mat = T.cells[k.cell].fill;
        if (TRACE) trace_rec(A, L, 5, k.cell);
        ph = PH_FLIGHT;
      }
    }

    // ----------------------------------------------------------------- moved
    __syncwarp();
    if (ph == PH_MOVED) {
      if (k.cell < 0 && (TRK == ABX_TRACK_DELTA || TRK == ABX_TRACK_CARTER)) {
        // flew out of the geometry: back to the last position, find the
        // boundary condition (src/delta_tracker.cpp:120-127)
        trk_set_r(k, L.r);
        dmode = 1;
        after = PH_LOST;
        ph = PH_WAIT;
      } else if (k.cell < 0) {
        // implicit leakage: flights end inside the boundary conditions
        if (sizeof(R) == 8) ABX_FAIL(ABX_ERR_LOST_PARTICLE) else {
          ABX_LOST();
          ph = PH_DEAD;
        }
      } else {
        const ProbT& P = T.probs[SINGLE ? 0 : L.pid];
        if (TRK != ABX_TRACK_IMPLICIT_LEAKAGE && converged && P.has_tle) score_flight(T, V, P, L, dcol);
        L.r = add(L.r, scl(L.u, dcol));
        L.mat = T.cells[k.cell].fill;
        const MatT& M = T.mats[L.mat];
        const R Et = V.xs[M.xs_off + XS_ET * M.G + L.g];
        if (TRK == ABX_TRACK_CARTER) {
          // src/carter_tracker.cpp:184-207: where the sampling cross section
          // falls below the total one the collision is always "real" with
          // probability D and carries weight factors +-F
          const R Es = V.maj[P.maj_off + P.G + L.g];
          bool real;
          if (Es >= Et) {
            real = canon<R>(L.rng) < (Et / Es);
          } else {
            const R D = Et / (R(2) * Et - Es);
            const R F = Et / (D * Es);
            real = (D - canon<R>(L.rng)) > R(0);
            L.w = real ? L.w * F : -L.w * F;
          }
          if (TRACE) trace_rec(A, L, real ? 1 : 0, k.cell);
          if (real) {
            ph = PH_COLL;
          } else {
            carter_split(A, P, L);
            ph = PH_FLIGHT;
          }
        } else {
          const R Emaj = V.maj[P.maj_off + L.g];
          if (Et - Emaj > Tol<R>::MAJ) ABX_FAIL(ABX_ERR_MAJORANT) else {
            const bool real = canon<R>(L.rng) < (Et / Emaj);
            if (TRACE) trace_rec(A, L, real ? 1 : 0, k.cell);
            ph = real ? PH_COLL : PH_FLIGHT;
          }
        }
      }
    }

    // -------------------------------------------------------------- boundary
    if (ph == PH_LOST) {
      const ProbT& P = T.probs[SINGLE ? 0 : L.pid];
      const Bound<R> b = trk_bc_ool<R>(T, P, k);
      if (converged && P.has_tle) score_flight(T, V, P, L, dcol < b.dist ? dcol : b.dist);
      if (b.btype == ABX_BC_VACUUM) {
        acc.hleak += L.w;
        const V3<R> dl = sub(add(L.r, scl(L.u, b.dist)), L.rb);
        acc.hmig += dot(scl(dl, L.w), dl);
        if (TRACE) trace_rec(A, L, 2, k.cell);
        ph = PH_DEAD;
      } else if (b.btype == ABX_BC_REFLECTIVE) {
        reflect_move(V, k, L, b);
        dmode = 1;
        after = PH_REFL;
        ph = PH_WAIT;
      } else if (sizeof(R) == 8) {
        ABX_FAIL(ABX_ERR_LOST_PARTICLE);
      } else {
        ABX_LOST();
        ph = PH_DEAD;
      }
    }

    // --------------------------------------------------------------- collide
    __syncwarp();
    if (ph == PH_COLL) {
      const ProbT& P = T.probs[SINGLE ? 0 : L.pid];
      bool alive = true;
      ncoll++;
      L.hcoll++;
      collide<R, ISO, TRK == ABX_TRACK_SURFACE, BL>(A, T, V, P, L, acc, converged, kcol, alive);
      if (sizeof(R) == 4 && !(m_abs(L.u.x) <= R(1) && m_abs(L.u.y) <= R(1) && m_abs(L.u.z) <= R(1))) {
        // mixed mode: a direction that is not finite cannot be tracked
        ABX_LOST();
        alive = false;
      }
      k.u = L.u;
      if (TRACE) trace_rec(A, L, 4, k.cell);
      if (TRK == ABX_TRACK_CARTER && alive) carter_split(A, P, L);
      ph = alive ? PH_FLIGHT : PH_DEAD;
    }

    // ------------------------------------------------------------------ dead
    __syncwarp();
    if (ph == PH_DEAD) {
      if (L.nsec > 0) {
        // Particle::resurect (include/simulation/particle.hpp:170-182)
        const ProbT& P = T.probs[SINGLE ? 0 : L.pid];
        L.nsec--;
        const uint32_t gt = blockIdx.x * blockDim.x + threadIdx.x;
        const R* sp = A.sec + ((uint64_t)gt * A.sec_cap + L.nsec) * 9;
        L.r = mk<R>(sp[0], sp[1], sp[2]);
        L.u = mk<R>(sp[3], sp[4], sp[5]);
        L.E = sp[6];
        L.w = sp[7];
        L.w2 = sp[8];
        L.g = group_of<R>(V.ebnd + P.eb_off, P.G, L.E);
        if (L.g >= P.G) ABX_FAIL(ABX_ERR_INVALID) else {
          trk_set_r(k, L.r);
          k.u = L.u;
          dmode = 1;
          after = PH_RES;
          ph = PH_WAIT;
        }
      } else {
        history_end<R, SINGLE>(A, L, acc, sh_acc);
        ph = PH_REFILL;
      }
    }

    if (ph != PH_REFILL && ph != PH_DONE && L.events > ev_limit) {
      if (sizeof(R) == 4) {
        // mixed mode: a history this long is a geometry rounding trap, not
        // physics; it is counted in `lost` and ended
        ABX_LOST();
        history_end<R, SINGLE>(A, L, acc, sh_acc);
        ph = PH_REFILL;
      } else {
        ABX_FAIL(ABX_ERR_TIMEOUT);
      }
    }
  }
#undef ABX_FAIL
#undef ABX_LOST
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
