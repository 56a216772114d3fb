// The pooled transport loop: event-sorted execution inside one persistent
// launch.
//
// The history kernel (transport_loop.cuh) gives every lane one history and
// runs the phases of the lanes' event machines one after another, each with
// the lanes that happen to be in it: on the 51x51-pin assembly 5.7 of 32
// lanes execute an average instruction.  Here every warp owns a pool of
// 32 * POOL_K particle slots in device memory (AoS records of the full
// history state: particle, tracker tree, score accumulators, event-machine
// registers).  A warp visits the event kinds in a fixed order -- refill,
// flight (+ the real/virtual test), descend (+ the checks after it),
// boundary, collide, history end -- and for each kind gathers the slots of
// its pool in that kind (one ballot per 32 slots), 32 at a time, so each
// warp-step runs one event kind with every lane busy.  A slot's history goes
// through exactly the reference's sequence of operations and draws; only the
// interleaving across histories changes, as in the history kernel.
//
// No grid-wide synchronisation, no queues in global memory: each warp sorts
// its own pool, slots refill from the global history counter as their
// histories end, and a warp retires when its pool is empty.
#pragma once

#include "transport_loop.cuh"

namespace abx {

constexpr int POOL_K = 4;              // slots per lane
constexpr int POOL_NS = 32 * POOL_K;   // slots per warp

// Everything a history carries between two of its events.
template <class R> struct __align__(16) PoolSlot {
  Lane<R> L;
  Trk<R> k;
  Acc<R> acc;
  R dcol;
  int32_t after, dmode, dui, dfr, prev_cell;
};

// Stored event kinds of a slot (a subset of the PH_* codes; the others are
// transient within one warp-step).
enum : uint8_t { PS_REFILL = 0, PS_FLIGHT, PS_WAIT, PS_LOST, PS_COLL, PS_DEAD, PS_DONE };

// Position of the j-th (0-based) set bit of m, j < popc(m).
ABX_DEV int pool_nth_bit(unsigned m, int j) {
  int pos = 0, c;
  c = __popc(m & 0xffffu); if (j >= c) { j -= c; m >>= 16; pos += 16; }
  c = __popc(m & 0xffu);   if (j >= c) { j -= c; m >>= 8;  pos += 8; }
  c = __popc(m & 0xfu);    if (j >= c) { j -= c; m >>= 4;  pos += 4; }
  c = __popc(m & 0x3u);    if (j >= c) { j -= c; m >>= 2;  pos += 2; }
  if (j >= (int)(m & 1u)) pos += 1;
  return pos;
}

template <class R> size_t pool_slot_bytes() { return sizeof(PoolSlot<R>); }

// TRACK: the tracking mode (delta, surface or implicit-leakage delta
// tracking), or'd with ABX_KERNEL_SINGLE for one problem.  Histories that
// may put particles on a secondary stack (fixed-source fission, Carter
// tracking, branchless splitting) run in the history kernel.
template <class R, int TRACK, bool ISO>
__global__ void __launch_bounds__(256, sizeof(R) == 4 ? ((TRACK & 0xff) != ABX_TRACK_SURFACE ? 4 : 3) : 3)
    transport_pool_kernel(const __grid_constant__ TransportArgs<R> A) {
  constexpr int TRK = TRACK & 0xff;
  constexpr bool SINGLE = (TRACK & ABX_KERNEL_SINGLE) != 0;
  const bool TRACE = sizeof(R) == 8 && A.trace != nullptr;
  const Tables& T = A.T;
  const View<R> V = make_view<R>(T);
  DevState* st = A.st;
  const unsigned lane = threadIdx.x & 31u;
  const unsigned wib = threadIdx.x >> 5;
  const uint64_t gwarp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  PoolSlot<R>* pool = reinterpret_cast<PoolSlot<R>*>(A.pool) + gwarp * POOL_NS;
  const unsigned long long n_hist = st->n_hist;
  const R kcol = (R)st->kcol;
  const bool converged = st->converged != 0;
  const uint32_t ev_limit = sizeof(R) == 4 ? 100000u : (uint32_t)(A.max_events < 0xffffffffull ? A.max_events : 0xffffffffull);

  __shared__ double sh_acc[5];
  __shared__ uint8_t codes[8][POOL_NS];
  if (threadIdx.x < 5) sh_acc[threadIdx.x] = 0.;
  uint8_t* cw = codes[wib];
#pragma unroll
  for (int j = 0; j < POOL_K; j++) cw[lane + 32 * j] = PS_REFILL;
  __syncthreads();

  uint32_t ncoll = 0, nflight = 0, nlost = 0;
  unsigned long long npos = 0, nneg = 0;

  // the event kinds in the order a round visits them
  const uint8_t order[6] = {PS_REFILL, PS_FLIGHT, PS_WAIT, PS_LOST, PS_COLL, PS_DEAD};
  // Rare kinds (refill, boundary, history end) wait until a quarter warp of
  // slots needs them while at least half the pool is in the common ones
  // (flight, descend, collide); the common count is the last round's.
  int common = 0;

  for (;;) {
    int common_now = 0;
#pragma unroll 1
    for (int oi = 0; oi < 6; oi++) {
      const uint8_t kind = order[oi];
      unsigned m[POOL_K];
      int tot = 0;
#pragma unroll
      for (int j = 0; j < POOL_K; j++) {
        m[j] = __ballot_sync(0xffffffffu, cw[lane + 32 * j] == kind);
        tot += __popc(m[j]);
      }
      const bool rare = kind == PS_REFILL || kind == PS_LOST || kind == PS_DEAD;
      if (!rare) common_now += tot;
      if (rare && tot < 8 && common >= POOL_NS / 2) continue;
#pragma unroll 1
      for (int c0 = 0; c0 < tot; c0 += 32) {
        // this lane's slot: the (c0 + lane)-th slot of the pool in `kind`
        int s = -1;
        {
          int n = c0 + (int)lane, base = 0;
#pragma unroll
          for (int j = 0; j < POOL_K; j++) {
            const int c = __popc(m[j]);
            if (s < 0 && n < tot && n < base + c) s = 32 * j + pool_nth_bit(m[j], n - base);
            base += c;
          }
        }
        const bool act = s >= 0;
        PoolSlot<R> S;
        int ph = PH_DONE;
        if (act) {
          if (kind != PS_REFILL) S = pool[s];
          ph = kind == PS_REFILL ? PH_REFILL
             : kind == PS_FLIGHT ? PH_FLIGHT
             : kind == PS_WAIT   ? PH_WAIT
             : kind == PS_LOST   ? PH_LOST
             : kind == PS_COLL   ? PH_COLL
                                 : PH_DEAD;
        }
        Lane<R>& L = S.L;
        Trk<R>& k = S.k;
        Acc<R>& acc = S.acc;

#define ABX_FAIL(code)          \
  {                             \
    raise_err(st, (code), L.h); \
    ph = PH_DONE;               \
  }
#define ABX_LOST()                                                                        \
  {                                                                                       \
    nlost++;                                                                              \
    if (!SINGLE && A.pcount) atomicAdd(A.pcount + (size_t)L.pid * ABX_PCOUNTS + 3, 1ull); \
    if (TRACE) trace_rec(A, L, 7, k.cell);                                                \
  }

        if (kind == PS_DEAD && act) {
          // ---------------------------------------------------- history end
          history_end<R, SINGLE>(A, L, acc, sh_acc);
          npos += L.npos;
          nneg += L.nneg;
          ph = PH_REFILL;
        }
        if (kind == PS_REFILL || kind == PS_DEAD) {
          // ------------------------------------------------------ refill
          // (a slot whose history just ended takes the next one at once)
          const unsigned mm = __ballot_sync(0xffffffffu, act);
          const unsigned leader = __ffs(mm) - 1;
          unsigned long long base = 0;
          if (lane == leader) base = atomicAdd(&st->next_hist, (unsigned long long)__popc(mm));
          base = __shfl_sync(0xffffffffu, base, leader);
          if (act) {
            const unsigned long long h = base + __popc(mm & ((1u << lane) - 1u));
            L.npos = 0;
            L.nneg = 0;
            if (h >= n_hist || st->err) {
              ph = PH_DONE;
            } else if (!lane_load<R, SINGLE>(A, T, V, L, k, (uint32_t)h)) {
              ABX_FAIL(k.err);
            } else {
              acc = Acc<R>();
              L.mat = -1;
              S.prev_cell = -1;
              S.dcol = R(0);
              S.dmode = 1;
              S.after = PH_START;
              ph = PH_WAIT;
            }
          }
        } else if (kind == PS_FLIGHT) {
          // ------------------------------------------------------ flight
          if (act) {
            const ProbT& P = T.probs[SINGLE ? 0 : L.pid];
            L.events++;
            nflight++;
            if (TRK == ABX_TRACK_IMPLICIT_LEAKAGE) {
              // ImplicitLeakageDeltaTracker::transport
              // (src/implicit_leakage_delta_tracker.cpp:104-214)
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
                S.dcol = -m_log(R(1) - P_no_leak * canon<R>(L.rng)) / Emaj;
                if (converged && P.has_tle) {
                  L.w = wgt_leak;
                  L.w2 = wgt2_leak;
                  score_flight(T, V, P, L, b.dist);
                }
                L.w = wgt_coll;
                L.w2 = wgt2_coll;
                if (converged && P.has_tle) score_flight(T, V, P, L, S.dcol);
              } else {
                S.dcol = Emaj == R(0) ? Tol<R>::INF : -m_log(R(1) - canon<R>(L.rng)) / Emaj;
                if (converged && P.has_tle) score_flight(T, V, P, L, S.dcol < b.dist ? S.dcol : b.dist);
              }
              if (b.dist < S.dcol || m_abs(b.dist - S.dcol) < Tol<R>::BTOL) {
                if (b.btype == ABX_BC_VACUUM) {
                  acc.hleak += L.w;
                  const V3<R> dl = sub(add(L.r, scl(L.u, b.dist)), L.rb);
                  acc.hmig += dot(scl(dl, L.w), dl);
                  if (TRACE) trace_rec(A, L, 2, k.cell);
                  ph = PH_DEAD;
                } else if (b.btype == ABX_BC_REFLECTIVE) {
                  reflect_move(V, k, L, b);
                  S.dmode = 1;
                  S.after = PH_REFL;
                  ph = PH_WAIT;
                } else if (sizeof(R) == 8) {
                  ABX_FAIL(ABX_ERR_LOST_PARTICLE);
                } else {
                  ABX_LOST();
                  ph = PH_DEAD;
                }
              } else {
                trk_move(k, S.dcol);
                const int r = trk_check(T, V, k, S.dui, S.dfr);
                if (r) {
                  S.dmode = r;
                  S.after = PH_MOVED;
                  ph = PH_WAIT;
                } else {
                  ph = PH_MOVED;
                }
              }
            } else if (TRK == ABX_TRACK_DELTA) {
              // DeltaTracker::transport (src/delta_tracker.cpp:105-118)
              const R Emaj = V.maj[P.maj_off + L.g];
              S.dcol = Emaj == R(0) ? Tol<R>::INF : -m_log(R(1) - canon<R>(L.rng)) / Emaj;
              trk_move(k, S.dcol);
              const int r = trk_check(T, V, k, S.dui, S.dfr);
              if (r) {
                S.dmode = r;
                S.after = PH_MOVED;
                ph = PH_WAIT;
              } else {
                ph = PH_MOVED;
              }
            } else {
              // SurfaceTracker::transport (src/surface_tracker.cpp:72-150)
              const MatT& M = T.mats[L.mat];
              const R Et = V.xs[M.xs_off + XS_ET * M.G + L.g];
              S.dcol = Et == R(0) ? Tol<R>::INF : -m_log(R(1) - canon<R>(L.rng)) / Et;
              const Bound<R> b = sizeof(R) == 8 ? trk_nearest(T, V, P, k) : trk_nearest_mixed(T, V, P, k);
              const R dmin = S.dcol < b.dist ? S.dcol : b.dist;
              if (converged && P.has_tle) score_flight(T, V, P, L, dmin);
              acc.htrk += L.w * dmin * V.xs[M.xs_off + XS_VEF * M.G + L.g];
              if (b.dist < S.dcol || m_abs(b.dist - S.dcol) < Tol<R>::BTOL) {
                if (b.btype == ABX_BC_VACUUM) {
                  acc.hleak += L.w;
                  const V3<R> dl = sub(add(L.r, scl(L.u, b.dist)), L.rb);
                  acc.hmig += dot(scl(dl, L.w), dl);
                  if (TRACE) trace_rec(A, L, 2, k.cell);
                  ph = PH_DEAD;
                } else if (b.btype == ABX_BC_REFLECTIVE) {
                  reflect_move(V, k, L, b);
                  S.dmode = 1;
                  S.after = PH_REFL;
                  ph = PH_WAIT;
                } else {
                  // Tracker::cross_surface + get_current (tracker.hpp:227-231)
                  S.prev_cell = k.cell;
                  trk_move(k, b.dist);
                  k.token = -b.token;
                  L.r = add(L.r, scl(L.u, b.dist));
                  S.dcol = b.dist;
                  const int r = trk_check(T, V, k, S.dui, S.dfr);
                  if (r) {
                    S.dmode = r;
                    S.after = PH_CROSSED;
                    ph = PH_WAIT;
                  } else {
                    ph = PH_CROSSED;
                  }
                }
              } else {
                L.r = add(L.r, scl(L.u, S.dcol));
                trk_move(k, S.dcol);
                if (TRACE) trace_rec(A, L, 1, k.cell);
                ph = PH_COLL;
              }
            }
          }
        } else if (kind == PS_WAIT) {
          // ----------------------------------------------------- descend
          if (act) {
            const ProbT& P = T.probs[SINGLE ? 0 : L.pid];
            int cell = -1;
            if (S.dmode == 2) {
              cell = univ_get_cell(T, V, k, S.dui, S.dfr, k.getfr(S.dfr));
              if (cell < 0) S.dmode = 1;
            }
            if (S.dmode == 1) {
              k.depth = 0;
              cell = univ_get_cell(T, V, k, P.root, 0, k.r);
            }
            k.cell = cell;
            S.dmode = 0;
            ph = S.after;
            if (k.err) ABX_FAIL(k.err);
          }
        }

        // ------------------------------------------ checks after a descent
        // (transient kinds: reached from the descend step, or from a flight
        // whose tree stayed valid)
        if (act && ph == PH_START) {
          if (k.cell < 0) {  // lost at birth: a warning in the reference, the particle is killed
            ABX_LOST();
            history_end<R, SINGLE>(A, L, acc, sh_acc);
            npos += L.npos;
            nneg += L.nneg;
            ph = PH_REFILL;
          } else {
            L.mat = T.cells[k.cell].fill;
            ph = PH_FLIGHT;
          }
        } else if (act && ph == PH_REFL) {
          if (k.cell < 0) {
            if (sizeof(R) == 8) ABX_FAIL(ABX_ERR_LOST_PARTICLE) else {
              ABX_LOST();
              ph = PH_DEAD;
            }
          } else {
            if (TRACE) trace_rec(A, L, 3, k.cell);
            ph = PH_FLIGHT;
          }
        } else if (act && ph == PH_CROSSED) {
          if (sizeof(R) == 4 && S.prev_cell != -2 && (k.cell < 0 || (k.cell == S.prev_cell && S.dcol == R(0)))) {
            // mixed mode: step off a surface crossing FP32 cannot resolve
            L.r = add(L.r, scl(L.u, R(4) * Tol<R>::SC));
            trk_set_r(k, L.r);
            S.prev_cell = -2;
            S.dmode = 1;
            S.after = PH_CROSSED;
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

        // --------------------------------------------------------- moved
        if (act && ph == PH_MOVED) {
          if (k.cell < 0 && TRK == ABX_TRACK_DELTA) {
            // flew out of the geometry: back to the last position (located
            // again by the next descend step), then find the boundary
            // condition (src/delta_tracker.cpp:120-127)
            trk_set_r(k, L.r);
            S.dmode = 1;
            S.after = PH_LOST;
            ph = PH_WAIT;
          } else if (k.cell < 0) {
            if (sizeof(R) == 8) ABX_FAIL(ABX_ERR_LOST_PARTICLE) else {
              ABX_LOST();
              ph = PH_DEAD;
            }
          } else {
            const ProbT& P = T.probs[SINGLE ? 0 : L.pid];
            if (TRK != ABX_TRACK_IMPLICIT_LEAKAGE && converged && P.has_tle) score_flight(T, V, P, L, S.dcol);
            L.r = add(L.r, scl(L.u, S.dcol));
            L.mat = T.cells[k.cell].fill;
            const MatT& M = T.mats[L.mat];
            const R Et = V.xs[M.xs_off + XS_ET * M.G + L.g];
            const R Emaj = V.maj[P.maj_off + L.g];
            if (Et - Emaj > Tol<R>::MAJ) ABX_FAIL(ABX_ERR_MAJORANT) else {
              const bool real = canon<R>(L.rng) < (Et / Emaj);
              if (TRACE) trace_rec(A, L, real ? 1 : 0, k.cell);
              ph = real ? PH_COLL : PH_FLIGHT;
            }
          }
        }

        if (kind == PS_LOST && act) {
          // ------------------------------------------------------ boundary
          const ProbT& P = T.probs[SINGLE ? 0 : L.pid];
          const Bound<R> b = trk_bc_ool<R>(T, P, k);
          if (converged && P.has_tle) score_flight(T, V, P, L, S.dcol < b.dist ? S.dcol : b.dist);
          if (b.btype == ABX_BC_VACUUM) {
            acc.hleak += L.w;
            const V3<R> dl = sub(add(L.r, scl(L.u, b.dist)), L.rb);
            acc.hmig += dot(scl(dl, L.w), dl);
            if (TRACE) trace_rec(A, L, 2, k.cell);
            ph = PH_DEAD;
          } else if (b.btype == ABX_BC_REFLECTIVE) {
            reflect_move(V, k, L, b);
            S.dmode = 1;
            S.after = PH_REFL;
            ph = PH_WAIT;
          } else if (sizeof(R) == 8) {
            ABX_FAIL(ABX_ERR_LOST_PARTICLE);
          } else {
            ABX_LOST();
            ph = PH_DEAD;
          }
        } else if (kind == PS_COLL && act) {
          // ------------------------------------------------------- collide
          const ProbT& P = T.probs[SINGLE ? 0 : L.pid];
          bool alive = true;
          ncoll++;
          L.hcoll++;
          collide<R, ISO, TRK == ABX_TRACK_SURFACE, false>(A, T, V, P, L, acc, converged, kcol, alive);
          if (sizeof(R) == 4 && !(m_abs(L.u.x) <= R(1) && m_abs(L.u.y) <= R(1) && m_abs(L.u.z) <= R(1))) {
            // mixed mode: a direction that is not finite cannot be tracked
            ABX_LOST();
            alive = false;
          }
          k.u = L.u;
          if (TRACE) trace_rec(A, L, 4, k.cell);
          ph = alive ? PH_FLIGHT : PH_DEAD;
        }

        if (act && ph != PH_REFILL && ph != PH_DONE && L.events > ev_limit) {
          if (sizeof(R) == 4) {
            // mixed mode: a history this long is a geometry rounding trap,
            // not physics; it is counted in `lost` and ended
            ABX_LOST();
            history_end<R, SINGLE>(A, L, acc, sh_acc);
            npos += L.npos;
            nneg += L.nneg;
            ph = PH_REFILL;
          } else {
            ABX_FAIL(ABX_ERR_TIMEOUT);
          }
        }
#undef ABX_FAIL
#undef ABX_LOST
        if (act) {
          uint8_t code;
          switch (ph) {
            case PH_REFILL: code = PS_REFILL; break;
            case PH_FLIGHT: code = PS_FLIGHT; break;
            case PH_WAIT: code = PS_WAIT; break;
            case PH_LOST: code = PS_LOST; break;
            case PH_COLL: code = PS_COLL; break;
            case PH_DEAD: code = PS_DEAD; break;
            default: code = PS_DONE; break;
          }
          if (code != PS_DONE && code != PS_REFILL) pool[s] = S;
          cw[s] = code;
        }
        __syncwarp();
      }
    }
    common = common_now;
    bool left = false;
#pragma unroll
    for (int j = 0; j < POOL_K; j++) left |= cw[lane + 32 * j] != PS_DONE;
    if (!__any_sync(0xffffffffu, left)) break;
  }

  unsigned long long c[5] = {ncoll, nflight, nlost, npos, nneg};
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
