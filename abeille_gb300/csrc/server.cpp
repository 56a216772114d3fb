// Request loop for fixed-source problems: a host scheduler over the C-ABI.
//
// Submission copies the problem (the caller's buffers are not retained) and
// queues it with an estimate of its device footprint.  A preparation thread
// admits queued requests in arrival order into a round while the footprints
// of everything admitted and not yet finished fit the HBM budget, and
// derives the round's tables on the host.  Several GPU lanes -- threads
// that each own a batch context, hence its own CUDA stream and device
// buffers -- take prepared rounds as they come free: a lane installs the
// round's tables, runs every batch of every request of the round in one
// transport launch, and copies results and tally bins back.  Rounds of
// different lanes run on the device at the same time.  Their launches use a
// history quantum: each warp retires after a bounded number of histories
// and the grid covers the rest with later blocks, so blocks finish all
// through a launch and the SM slots they free go to whichever launch is
// waiting -- a round admitted while others run starts on the device as
// slots free up, instead of after them.  A request's HBM share returns to
// the budget when its round completes.
//
// A request's results do not depend on its round or lane: batch b of a
// problem always transports its histories b*n .. (b+1)*n-1, each seeded by
// skip-ahead on the problem's own stream, and its tallies and scores are its
// own.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "abeille_gb300.h"

namespace abx {
void set_error_string(const char* msg);  // engine.cu: the thread's abx_last_error_string
// engine.cu: abx_batch_replace in a host half and a device half
void* batch_prepare(const abx_problem* problems, int n_problems, int* rc);
int batch_install(abx_ctx* c, void* prepared);
void batch_discard(void* prepared);
}

namespace {

using Clock = std::chrono::steady_clock;

double ms_between(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double, std::milli>(b - a).count();
}

int srv_fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  abx::set_error_string(buf);
  return code;
}

// Deep copy of an abx_problem; `p` points into the vectors.
struct ProblemCopy {
  abx_problem p{};
  std::vector<double> eb, mg, teb;
  std::vector<abx_surface> surf;
  std::vector<abx_cell> cells;
  std::vector<int32_t> rpn, lists, lat;
  std::vector<abx_universe> univ;
  std::vector<abx_material> mats;
  std::vector<abx_mesh_tally> tallies;
  std::vector<abx_source> src;

  template <class T> static void take(std::vector<T>& v, const T* a, int64_t n) {
    v.assign(a, a + (n > 0 && a ? n : 0));
  }
  void copy_from(const abx_problem& q) {
    p = q;
    take(eb, q.energy_bounds, q.settings.ngroups + 1);
    take(mg, q.mg_data, q.n_mg_data);
    take(teb, q.tally_ebounds, q.n_tally_ebounds);
    take(surf, q.surfaces, q.n_surfaces);
    take(cells, q.cells, q.n_cells);
    take(rpn, q.rpn, q.n_rpn);
    take(lists, q.cell_lists, q.n_cell_lists);
    take(lat, q.lattice_elems, q.n_lattice_elems);
    take(univ, q.universes, q.n_universes);
    take(mats, q.materials, q.n_materials);
    take(tallies, q.tallies, q.n_tallies);
    take(src, q.sources, q.n_sources);
    p.energy_bounds = eb.data();
    p.mg_data = mg.data();
    p.tally_ebounds = teb.data();
    p.surfaces = surf.data();
    p.cells = cells.data();
    p.rpn = rpn.data();
    p.cell_lists = lists.data();
    p.lattice_elems = lat.data();
    p.universes = univ.data();
    p.materials = mats.data();
    p.tallies = tallies.data();
    p.sources = src.data();
  }
  uint64_t tally_bins() const {
    uint64_t n = 0;
    for (const abx_mesh_tally& t : tallies)
      n += (uint64_t)std::max(0, t.n_ebounds - 1) * (uint64_t)std::max(0, t.shape[0]) *
           (uint64_t)std::max(0, t.shape[1]) * (uint64_t)std::max(0, t.shape[2]);
    return n;
  }
  // Device bytes while the request runs with `nb` batches: a per-batch FP64
  // copy of every tally bin plus the average and variance, the two banks of
  // the transport precision (nine reals, three 64-bit words and a problem
  // index per history: 64 B in FP32, 100 B in FP64) and two sort counters
  // for all its histories, and the tables (four copies of the cross-section
  // data covers the derived CDFs, angle tables and FP32 mirrors).
  uint64_t footprint(int nb, bool mixed) const {
    const uint64_t hist = (uint64_t)(p.settings.nparticles > 0 ? p.settings.nparticles : 0) * (uint64_t)nb;
    const uint64_t per_hist = 2 * (mixed ? 64 : 100) + 8;
    return 8 * ((uint64_t)nb + 2) * tally_bins() + per_hist * hist + 32 * (uint64_t)mg.size() +
           16 * (uint64_t)(surf.size() + cells.size() + rpn.size() + univ.size() + lat.size()) + (64u << 10);
  }
};

struct Request {
  uint64_t id = 0, tag = 0;
  std::unique_ptr<ProblemCopy> prob;
  uint64_t footprint = 0;
  Clock::time_point t_submit;
};

struct Done {
  abx_request_result r{};
  std::vector<double> avg, var;
};

struct Round {
  std::vector<Request> reqs;
  void* prepared = nullptr;  // host tables of the batch
  int number = 0;
  uint64_t bytes = 0;        // admitted footprint, returned when the round ends
  Clock::time_point t_admit;
  double prep_ms = 0.;
};

}  // namespace

struct abx_server {
  abx_server_options opt{};
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Request> queue;
  std::deque<uint64_t> ready;                  // finished, not yet polled
  std::unordered_map<uint64_t, Done> results;  // finished, not yet released
  uint64_t next_id = 1;
  bool stop = false;
  abx_server_stats stats{};
  std::vector<std::thread> lanes;
  std::thread preparer;
  int round = 0;
  uint64_t inflight_bytes = 0;    // footprint of admitted, unfinished requests
  int idle_lanes = 0;
  std::unique_ptr<Round> staged;  // prepared, waiting for a lane
  bool prep_done = false;         // the preparation thread has exited
  std::condition_variable cv_staged;

  void run_round(Round& rd, abx_ctx*& ctx);
  void finish(Request& q, Done&& d, double queue_ms);
  void fail_request(Request& q, int status, double queue_ms);
  void prep_loop();
  void lane_loop();
};

void abx_server::fail_request(Request& q, int status, double queue_ms) {
  Done d;
  d.r.status = status;
  d.r.n_tallies = q.prob->p.n_tallies;
  finish(q, std::move(d), queue_ms);
}

void abx_server::finish(Request& q, Done&& d, double queue_ms) {
  d.r.request_id = q.id;
  d.r.tag = q.tag;
  d.r.queue_ms = queue_ms;
  std::lock_guard<std::mutex> g(mu);
  d.r.latency_ms = ms_between(q.t_submit, Clock::now());
  stats.completed++;
  if (d.r.status != ABX_OK) stats.failed++;
  ready.push_back(q.id);
  results.emplace(q.id, std::move(d));
  cv_done.notify_all();
}

void abx_server::run_round(Round& rd, abx_ctx*& ctx) {
  std::vector<Request>& reqs = rd.reqs;
  const int n = (int)reqs.size();
  const Clock::time_point t_start = rd.t_admit;
  const Clock::time_point c0 = Clock::now();
  // the context is kept across rounds; a round installs its prepared tables
  int rc;
  if (ctx) {
    rc = abx::batch_install(ctx, rd.prepared);
  } else {
    abx::batch_discard(rd.prepared);
    std::vector<abx_problem> arr((size_t)n);
    for (int i = 0; i < n; i++) arr[(size_t)i] = reqs[(size_t)i].prob->p;
    rc = abx_create_batch(arr.data(), n, opt.device, &ctx);
    if (rc == ABX_OK) rc = abx_set_history_quantum(ctx, opt.history_quantum);
  }
  rd.prepared = nullptr;
  const Clock::time_point c1 = Clock::now();
  std::vector<abx_problem_result> res((size_t)n);
  abx_run_stats st{};
  if (rc == ABX_OK) rc = abx_run_fixed_source_batch(ctx, opt.nbatches, res.data(), &st);
  const Clock::time_point c2 = Clock::now();
  std::vector<double> avg, var;
  if (rc == ABX_OK && opt.keep_tallies) {
    size_t nb = 0;
    rc = abx_tally_read_all(ctx, nullptr, nullptr, 0, &nb);
    if (rc == ABX_OK) {
      avg.resize(nb);
      var.resize(nb);
      rc = abx_tally_read_all(ctx, avg.data(), var.data(), nb, &nb);
    }
  }
  const Clock::time_point c3 = Clock::now();
  if (ctx && rc != ABX_OK) {
    // start the next round from a fresh context
    abx_destroy(ctx);
    ctx = nullptr;
  }
  const Clock::time_point c4 = Clock::now();
  {
    std::lock_guard<std::mutex> g(mu);
    stats.rounds++;
    stats.load_ms += rd.prep_ms + ms_between(c0, c1);
    stats.run_ms += ms_between(c1, c2);
    stats.readback_ms += ms_between(c2, c3);
    stats.free_ms += ms_between(c3, c4);
    if (rc == ABX_OK) {
      stats.collisions += st.collisions;
      stats.flights += st.flights;
      stats.histories += st.histories;
      stats.transport_ms += st.transport_ms;
    }
  }
  uint64_t bin0 = 0;
  for (int i = 0; i < n; i++) {
    Request& q = reqs[(size_t)i];
    Done d;
    d.r.status = rc;
    d.r.round = rd.number;
    d.r.round_problems = n;
    d.r.n_tallies = q.prob->p.n_tallies;
    d.r.n_tally_bins = q.prob->tally_bins();
    if (rc == ABX_OK) {
      d.r.result = res[(size_t)i];
      if (opt.keep_tallies) {
        d.avg.assign(avg.begin() + (long)bin0, avg.begin() + (long)(bin0 + d.r.n_tally_bins));
        d.var.assign(var.begin() + (long)bin0, var.begin() + (long)(bin0 + d.r.n_tally_bins));
      }
    }
    bin0 += d.r.n_tally_bins;
    finish(q, std::move(d), ms_between(q.t_submit, t_start));
  }
}

// Preparation thread: admits the next round and derives its host tables while
// the GPU thread runs the current one.  A request whose problem cannot be
// prepared fails on its own; the others of its round still run.
void abx_server::prep_loop() {
  auto prepare = [](std::vector<Request>& rs, int* rc) {
    std::vector<abx_problem> arr(rs.size());
    for (size_t i = 0; i < rs.size(); i++) arr[i] = rs[i].prob->p;
    return abx::batch_prepare(arr.data(), (int)arr.size(), rc);
  };
  for (;;) {
    std::unique_ptr<Round> rd(new Round());
    {
      std::unique_lock<std::mutex> lk(mu);
      // a round is formed when a lane can take it and the first queued
      // request fits next to what is already on the device
      auto can_admit = [&] {
        return !queue.empty() && !staged && idle_lanes > 0 &&
               (inflight_bytes == 0 || inflight_bytes + queue.front().footprint <= opt.hbm_budget_bytes);
      };
      cv_work.wait(lk, [&] { return stop || can_admit(); });
      if (stop) break;
      while (!queue.empty()) {
        const Request& h = queue.front();
        if (!rd->reqs.empty() && inflight_bytes + h.footprint > opt.hbm_budget_bytes) break;
        if (opt.max_round_problems > 0 && (int)rd->reqs.size() >= opt.max_round_problems) break;
        inflight_bytes += h.footprint;
        rd->bytes += h.footprint;
        rd->reqs.push_back(std::move(queue.front()));
        queue.pop_front();
      }
      rd->number = ++round;
      idle_lanes--;  // reserved for this round
    }
    rd->t_admit = Clock::now();
    int rc = ABX_OK;
    rd->prepared = prepare(rd->reqs, &rc);
    if (rc != ABX_OK) {
      // isolate the malformed requests
      std::vector<Request> good;
      for (Request& q : rd->reqs) {
        std::vector<Request> one;
        one.push_back(std::move(q));
        int rc1 = ABX_OK;
        abx::batch_discard(prepare(one, &rc1));
        if (rc1 != ABX_OK) fail_request(one[0], rc1, ms_between(one[0].t_submit, rd->t_admit));
        else good.push_back(std::move(one[0]));
      }
      rd->reqs = std::move(good);
      rc = ABX_OK;
      rd->prepared = rd->reqs.empty() ? nullptr : prepare(rd->reqs, &rc);
      if (!rd->reqs.empty() && rc != ABX_OK) {
        for (Request& q : rd->reqs) fail_request(q, rc, ms_between(q.t_submit, rd->t_admit));
        rd->reqs.clear();
      }
      // the failed requests' footprints go back to the budget
      uint64_t kept = 0;
      for (const Request& q : rd->reqs) kept += q.footprint;
      {
        std::lock_guard<std::mutex> g(mu);
        inflight_bytes -= rd->bytes - kept;
        rd->bytes = kept;
        if (rd->reqs.empty()) idle_lanes++;
      }
      if (rd->reqs.empty()) {
        cv_work.notify_all();
        continue;
      }
    }
    rd->prep_ms = ms_between(rd->t_admit, Clock::now());
    std::lock_guard<std::mutex> g(mu);
    staged = std::move(rd);
    cv_staged.notify_all();
  }
  std::lock_guard<std::mutex> g(mu);
  prep_done = true;
  cv_staged.notify_all();
}

// GPU lane: takes prepared rounds as they come and runs them in its own
// batch context (own stream, own device buffers), concurrently with the
// other lanes.
void abx_server::lane_loop() {
  abx_ctx* ctx = nullptr;
  for (;;) {
    std::unique_ptr<Round> rd;
    {
      std::unique_lock<std::mutex> lk(mu);
      cv_staged.wait(lk, [&] { return staged || prep_done; });
      if (!staged) break;
      rd = std::move(staged);
      cv_work.notify_all();  // the preparation thread may stage the next round
    }
    const Clock::time_point t0 = Clock::now();
    run_round(*rd, ctx);
    {
      std::lock_guard<std::mutex> g(mu);
      stats.busy_ms += ms_between(t0, Clock::now());
      inflight_bytes -= rd->bytes;  // the round's HBM share is free again
      idle_lanes++;
    }
    cv_work.notify_all();
  }
  if (ctx) abx_destroy(ctx);
}

// After the lanes stop: cancel what is still queued or staged.
static void cancel_queued(abx_server* s) {
  std::lock_guard<std::mutex> g(s->mu);
  std::vector<Request> left;
  while (!s->queue.empty()) {
    left.push_back(std::move(s->queue.front()));
    s->queue.pop_front();
  }
  if (s->staged) {
    for (Request& q : s->staged->reqs) left.push_back(std::move(q));
    s->staged->reqs.clear();
  }
  for (Request& q : left) {
    Done d;
    d.r.request_id = q.id;
    d.r.tag = q.tag;
    d.r.status = ABX_ERR_CANCELLED;
    d.r.latency_ms = ms_between(q.t_submit, Clock::now());
    s->stats.completed++;
    s->stats.failed++;
    s->ready.push_back(q.id);
    s->results.emplace(q.id, std::move(d));
  }
  s->cv_done.notify_all();
}

extern "C" int abx_server_create(const abx_server_options* options, abx_server** out) {
  if (!options || !out) return srv_fail(ABX_ERR_INVALID, "bad arguments");
  *out = nullptr;
  if (options->nbatches < 1) return srv_fail(ABX_ERR_INVALID, "nbatches must be >= 1");
  if (options->precision != ABX_PREC_FP64 && options->precision != ABX_PREC_MIXED)
    return srv_fail(ABX_ERR_INVALID, "precision %d", options->precision);
  if (options->tracking < ABX_TRACK_DELTA || options->tracking > ABX_TRACK_CARTER)
    return srv_fail(ABX_ERR_INVALID, "tracking %d", options->tracking);
  if (options->lanes < 0 || options->lanes > 16) return srv_fail(ABX_ERR_INVALID, "lanes %d out of range", options->lanes);
  abx_server* s = new abx_server();
  s->opt = *options;
  if (!s->opt.hbm_budget_bytes) s->opt.hbm_budget_bytes = 150ull * 1000 * 1000 * 1000;
  if (!s->opt.lanes) s->opt.lanes = 3;
  if (!s->opt.history_quantum) s->opt.history_quantum = 256;
  s->idle_lanes = s->opt.lanes;
  for (int i = 0; i < s->opt.lanes; i++) s->lanes.emplace_back([s] { s->lane_loop(); });
  s->preparer = std::thread([s] { s->prep_loop(); });
  *out = s;
  return ABX_OK;
}

extern "C" int abx_server_destroy(abx_server* s) {
  if (!s) return ABX_OK;
  {
    std::lock_guard<std::mutex> g(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  s->cv_staged.notify_all();
  if (s->preparer.joinable()) s->preparer.join();
  for (std::thread& t : s->lanes)
    if (t.joinable()) t.join();
  cancel_queued(s);
  if (s->staged && s->staged->prepared) abx::batch_discard(s->staged->prepared);
  delete s;
  return ABX_OK;
}

extern "C" int abx_server_submit(abx_server* s, const abx_problem* problem, uint64_t tag, uint64_t* request_id) {
  if (!s || !problem) return srv_fail(ABX_ERR_INVALID, "bad arguments");
  const abx_settings& st = problem->settings;
  if (st.mode != ABX_MODE_FIXED_SOURCE) return srv_fail(ABX_ERR_UNSUPPORTED, "the request loop runs fixed-source problems");
  if (st.precision != s->opt.precision || st.tracking != s->opt.tracking)
    return srv_fail(ABX_ERR_UNSUPPORTED, "request precision/tracking differ from the server's");
  if (st.ngroups < 1 || !problem->energy_bounds || !(st.nparticles >= 1))
    return srv_fail(ABX_ERR_INVALID, "malformed problem");
  Request q;
  q.prob.reset(new ProblemCopy());
  q.prob->copy_from(*problem);
  q.footprint = q.prob->footprint(s->opt.nbatches, s->opt.precision == ABX_PREC_MIXED);
  q.tag = tag;
  if (q.footprint > s->opt.hbm_budget_bytes)
    return srv_fail(ABX_ERR_BUDGET, "request needs ~%llu bytes, budget %llu", (unsigned long long)q.footprint,
                    (unsigned long long)s->opt.hbm_budget_bytes);
  {
    std::lock_guard<std::mutex> g(s->mu);
    if (s->stop) return srv_fail(ABX_ERR_CANCELLED, "server is stopping");
    q.id = s->next_id++;
    q.t_submit = Clock::now();
    if (request_id) *request_id = q.id;
    s->stats.submitted++;
    s->queue.push_back(std::move(q));
  }
  s->cv_work.notify_one();
  return ABX_OK;
}

extern "C" int abx_server_poll(abx_server* s, abx_request_result* out, int capacity, int* n_out, int timeout_ms) {
  if (!s || !n_out || (capacity > 0 && !out)) return srv_fail(ABX_ERR_INVALID, "bad arguments");
  *n_out = 0;
  std::unique_lock<std::mutex> lk(s->mu);
  auto have = [&] { return !s->ready.empty(); };
  if (!have() && timeout_ms != 0) {
    if (timeout_ms < 0) {
      s->cv_done.wait(lk, [&] { return have() || (s->stop && s->queue.empty()); });
    } else {
      s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), have);
    }
  }
  int k = 0;
  while (k < capacity && !s->ready.empty()) {
    const uint64_t id = s->ready.front();
    s->ready.pop_front();
    auto it = s->results.find(id);
    if (it == s->results.end()) continue;
    out[k++] = it->second.r;
    if (!s->opt.keep_tallies) s->results.erase(it);  // nothing left to read
  }
  *n_out = k;
  return ABX_OK;
}

extern "C" int abx_server_tally(abx_server* s, uint64_t request_id, double* avg, double* var, size_t capacity) {
  if (!s) return srv_fail(ABX_ERR_INVALID, "bad arguments");
  std::lock_guard<std::mutex> g(s->mu);
  auto it = s->results.find(request_id);
  if (it == s->results.end()) return srv_fail(ABX_ERR_INVALID, "request %llu has no result", (unsigned long long)request_id);
  const Done& d = it->second;
  if (!s->opt.keep_tallies) return srv_fail(ABX_ERR_UNSUPPORTED, "server was created without keep_tallies");
  if (capacity < d.avg.size()) return srv_fail(ABX_ERR_CAPACITY, "%zu bins, capacity %zu", d.avg.size(), capacity);
  if (avg && !d.avg.empty()) memcpy(avg, d.avg.data(), d.avg.size() * sizeof(double));
  if (var && !d.var.empty()) memcpy(var, d.var.data(), d.var.size() * sizeof(double));
  return ABX_OK;
}

extern "C" int abx_server_release(abx_server* s, uint64_t request_id) {
  if (!s) return srv_fail(ABX_ERR_INVALID, "bad arguments");
  std::lock_guard<std::mutex> g(s->mu);
  s->results.erase(request_id);
  return ABX_OK;
}

extern "C" int abx_server_get_stats(abx_server* s, abx_server_stats* out) {
  if (!s || !out) return srv_fail(ABX_ERR_INVALID, "bad arguments");
  std::lock_guard<std::mutex> g(s->mu);
  *out = s->stats;
  return ABX_OK;
}
