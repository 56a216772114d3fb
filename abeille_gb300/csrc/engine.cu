// Host side of the GB300 multigroup transport engine: the C-ABI declared in
// include/abeille_gb300.h, device pools (the tables come from
// problem_tables.cpp), and the device-resident generation loop (bank sort,
// weight normalisation, entropy, k and tally statistics) that replaces the
// reference's PowerIterator / FixedSource bookkeeping.  Compiled with
// --fmad=false and host -ffp-contract=off: every double derived here rounds
// as the reference's does.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstddef>
#include <random>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "kernels.cuh"
#include "launch.h"
#include "problem_tables.h"

using namespace abx;

// ------------------------------------------------------------------ errors
static thread_local std::string g_err;
static int fail(int code, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}
#define CUDA_TRY(x)                                                                    \
  do {                                                                                 \
    cudaError_t e_ = (x);                                                              \
    if (e_ != cudaSuccess) {                                                           \
      return fail(e_ == cudaErrorMemoryAllocation ? ABX_ERR_OOM : ABX_ERR_CUDA,         \
                  "%s failed: %s (%s:%d)", #x, cudaGetErrorString(e_), __FILE__, __LINE__); \
    }                                                                                  \
  } while (0)

extern "C" const char* abx_last_error_string(void) { return g_err.c_str(); }
namespace abx {
void set_error_string(const char* msg) { g_err = msg; }
}
extern "C" int abx_version(int* a, int* b, int* c) {
  if (a) *a = 0;
  if (b) *b = 4;
  if (c) *c = 0;
  return ABX_OK;
}

// ------------------------------------------------------------ device pools
// Buffers that follow the size of the work grow by half again when they must
// grow: every reallocation frees device memory, and cudaFree waits for the
// whole device -- in the request loop, for the launches of the other lanes.
static size_t headroom(size_t n) { return n + n / 2; }

// Device copies of the pools.  upload() fills the slots in a fixed order, so
// a context whose problems are replaced reuses each slot's allocation when it
// is large enough.
struct DevPools {
  std::vector<void*> allocs;
  std::vector<size_t> caps;
  size_t slot = 0;
  Tables T{};
  template <class X> int up(const std::vector<X>& v, const X** out) {
    const size_t bytes = std::max<size_t>(v.size(), 1) * sizeof(X);
    if (slot == allocs.size()) {
      allocs.push_back(nullptr);
      caps.push_back(0);
    }
    if (caps[slot] < bytes) {
      if (allocs[slot]) cudaFree(allocs[slot]);
      allocs[slot] = nullptr;
      caps[slot] = 0;
      CUDA_TRY(cudaMalloc(&allocs[slot], headroom(bytes)));
      caps[slot] = headroom(bytes);
    }
    void* p = allocs[slot++];
    if (!v.empty()) CUDA_TRY(cudaMemcpy(p, v.data(), v.size() * sizeof(X), cudaMemcpyHostToDevice));
    *out = (const X*)p;
    return ABX_OK;
  }
  void release() {
    for (void* p : allocs)
      if (p) cudaFree(p);
    allocs.clear();
    caps.clear();
    slot = 0;
  }
};

template <class X> static std::vector<float> to_f(const std::vector<X>& v) {
  std::vector<float> o(v.size());
  for (size_t i = 0; i < v.size(); i++) o[i] = (float)v[i];
  return o;
}

// Table uploads are synchronous copies on the legacy stream, which is not
// ordered with the context's (non-blocking) stream: make the stream wait for
// them before it runs kernels that read the tables (other contexts' streams
// keep running meanwhile).
static int after_host_copies(cudaStream_t s) {
  cudaEvent_t e = nullptr;
  if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return ABX_ERR_CUDA;
  cudaError_t r = cudaEventRecord(e, 0);
  if (r == cudaSuccess) r = cudaStreamWaitEvent(s, e, 0);
  cudaEventDestroy(e);
  return r == cudaSuccess ? ABX_OK : ABX_ERR_CUDA;
}

static int upload(const Pools& P, DevPools& D) {
  int rc;
  D.slot = 0;
#define UP(v, dst)                                  \
  if ((rc = D.up(v, &dst)) != ABX_OK) return rc;
  UP(P.cells, D.T.cells);
  UP(P.rpn, D.T.rpn);
  UP(P.univ, D.T.univ);
  UP(P.cell_lists, D.T.cell_lists);
  UP(P.lat_elems, D.T.lat_elems);
  UP(P.mats, D.T.mats);
  UP(P.ang_hdr, D.T.ang_hdr);
  UP(P.probs, D.T.probs);
  UP(P.tallies, D.T.tallies);
  UP(P.sources, D.T.sources);
  UP(P.src_cdf, D.T.src_cdf);
  UP(P.surf_d, D.T.surf_d);
  UP(P.lat_d, D.T.lat_d);
  UP(P.xs_d, D.T.xs_d);
  UP(P.cdf_d, D.T.cdf_d);
  UP(P.ang_d, D.T.ang_d);
  UP(P.eb_d, D.T.eb_d);
  UP(P.maj_d, D.T.maj_d);
  UP(P.dg_d, D.T.dg_d);
  UP(P.tally_eb, D.T.tally_eb);
  // FP32 mirrors for the mixed mode
  std::vector<SurfT<float>> sf(P.surf_d.size());
  for (size_t i = 0; i < sf.size(); i++) {
    sf[i].type = P.surf_d[i].type;
    sf[i].bc = P.surf_d[i].bc;
    for (int k = 0; k < 4; k++) sf[i].c[k] = (float)P.surf_d[i].c[k];
  }
  UP(sf, D.T.surf_f);
  std::vector<LatT<float>> lf(P.lat_d.size());
  for (size_t i = 0; i < lf.size(); i++)
    for (int a = 0; a < 3; a++) {
      lf[i].p[a] = (float)P.lat_d[i].p[a];
      lf[i].lo[a] = (float)P.lat_d[i].lo[a];
      lf[i].pinv[a] = 1.f / lf[i].p[a];
    }
  UP(lf, D.T.lat_f);
  std::vector<float> xf = to_f(P.xs_d);
  UP(xf, D.T.xs_f);
  std::vector<float> cf = to_f(P.cdf_d);
  UP(cf, D.T.cdf_f);
  std::vector<float> af = to_f(P.ang_d);
  UP(af, D.T.ang_f);
  std::vector<float> ef = to_f(P.eb_d);
  UP(ef, D.T.eb_f);
  // float majorant: the rounded group maxima bound the rounded cross sections
  std::vector<float> mf = to_f(P.maj_d);
  UP(mf, D.T.maj_f);
  std::vector<float> df = to_f(P.dg_d);
  UP(df, D.T.dg_f);
  std::vector<float> tf = to_f(P.tally_eb);
  UP(tf, D.T.tally_eb_f);
#undef UP
  D.T.nprob = (int)P.probs.size();
  return ABX_OK;
}

// ---------------------------------------------------------------- context
template <class R> struct BankBuf {
  BankT<R> b{};
  size_t cap = 0;
  std::vector<void*> mem;
  int alloc(size_t n, bool with_prob) {
    free_();
    cap = n;
    R** rs[] = {&b.x, &b.y, &b.z, &b.ux, &b.uy, &b.uz, &b.E, &b.w, &b.w2};
    for (R** p : rs) {
      void* m;
      CUDA_TRY(cudaMalloc(&m, std::max<size_t>(n, 1) * sizeof(R)));
      mem.push_back(m);
      *p = (R*)m;
    }
    uint64_t** us[] = {&b.rng, &b.hid, &b.fam};
    for (uint64_t** p : us) {
      void* m;
      CUDA_TRY(cudaMalloc(&m, std::max<size_t>(n, 1) * sizeof(uint64_t)));
      mem.push_back(m);
      *p = (uint64_t*)m;
    }
    b.prob = nullptr;
    if (with_prob) {
      void* m;
      CUDA_TRY(cudaMalloc(&m, std::max<size_t>(n, 1) * sizeof(int32_t)));
      mem.push_back(m);
      b.prob = (int32_t*)m;
    }
    return ABX_OK;
  }
  void free_() {
    for (void* m : mem) cudaFree(m);
    mem.clear();
    cap = 0;
  }
};

template <class R> struct SiteBuf {
  SiteT<R> s{};
  size_t cap = 0;
  std::vector<void*> mem;
  int alloc(size_t n) {
    free_();
    cap = n;
    R** rs[] = {&s.x, &s.y, &s.z, &s.ux, &s.uy, &s.uz, &s.E, &s.w};
    for (R** p : rs) {
      void* m;
      CUDA_TRY(cudaMalloc(&m, std::max<size_t>(n, 1) * sizeof(R)));
      mem.push_back(m);
      *p = (R*)m;
    }
    uint32_t** us[] = {&s.hist, &s.dau};
    for (uint32_t** p : us) {
      void* m;
      CUDA_TRY(cudaMalloc(&m, std::max<size_t>(n, 1) * sizeof(uint32_t)));
      mem.push_back(m);
      *p = (uint32_t*)m;
    }
    return ABX_OK;
  }
  void free_() {
    for (void* m : mem) cudaFree(m);
    mem.clear();
    cap = 0;
  }
};

struct RunAcc {
  double kcol_avg, kcol_var, kabs_avg, kabs_var, ktrk_avg, ktrk_var, leak_avg, leak_var, mig_avg, mig_var;
  int active;
  int gen;
  unsigned long long global_hist;
  unsigned long long total_coll, total_flights, total_hist;
};

struct abx_context {
  int device = 0;
  int nsm = 152;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  Pools P;
  DevPools D;
  ProbT prob0{};
  bool fissile_any = false;
  bool fp64_wide = false;  // FP64 delta/surface launches at four blocks per SM
  double* tally_gen = nullptr;
  double* tally_avg = nullptr;
  double* tally_var = nullptr;
  int tally_g = 0;
  DevState* st = nullptr;
  DevState* st_host = nullptr;
  RunAcc* run = nullptr;
  abx_gen_record* gen_rec = nullptr;
  int hist_cap = 0;
  double* ent_bins = nullptr;
  double* ent_total = nullptr;
  size_t ent_nbins = 0;
  BankBuf<double> bd[2];
  BankBuf<float> bf[2];
  SiteBuf<double> sd;
  SiteBuf<float> sf;
  uint32_t* hist_count = nullptr;
  uint32_t* offsets = nullptr;
  uint32_t* block_sums = nullptr;
  size_t count_cap = 0;
  void* sec = nullptr;
  uint32_t sec_cap = 16;
  size_t sec_threads = 0;
  abx_particle* aos_in = nullptr;
  abx_site* aos_out = nullptr;
  size_t aos_in_cap = 0, aos_out_cap = 0;
  abx_trace_rec* trace = nullptr;
  uint32_t trace_nhist = 0;
  size_t trace_cap = 0;
  int block = 256;
  int grid = 0;
  double last_ms = 0.;
  uint64_t max_events = 10000000ull;
  int prec = ABX_PREC_FP64;
  bool all_iso = false;  // every material scatters isotropically
  void* flush = nullptr;
  size_t flush_bytes = 0;
  // batches of problems
  int nprob = 1;
  bool batch_scores = false;  // transport launches score per problem
  double* pscore = nullptr;
  unsigned long long* pcount = nullptr;
  void* prun = nullptr;
  uint64_t* seg_off = nullptr;
  int32_t* seg_prob = nullptr;
  uint64_t* seg_hid0 = nullptr;
  // the (problem, batch) layout of the last batch run
  int vb_nb = 0;
  uint64_t vb_total = 0;
  ProbT* vprobs = nullptr;
  TallyT* vtallies = nullptr;
  size_t tally_gen_cap = 0;
  size_t vcap[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  size_t tally_rv_cap = 0;  // capacity of tally_avg / tally_var, in bins
  Tables batch_tables{};
  // captured generation step (one graph per bank parity)
  bool use_graphs = true;
  // the bank parity holding the next generation's source after a power
  // iteration (-1: none, or overwritten since), its size and k_col
  int pi_bank = -1;
  size_t pi_n = 0;
  double pi_kcol = 1.;
  // a source bank to start the next power iteration from (x y z ux uy uz E
  // w w2 per particle), set by abx_set_source_bank; empty: sample the sources
  std::vector<double> restart_src;
  cudaGraphExec_t gen_exec[2] = {nullptr, nullptr};
  cudaGraph_t gen_graph[2] = {nullptr, nullptr};  // kept: exec updates name its nodes
  cudaGraphNode_t gen_ev_node[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
  cudaEvent_t gen_ev_ph[2] = {nullptr, nullptr};
  size_t gen_cap = 0;
  int gen_nignored = -1;
  std::vector<const void*> gen_sig;  // buffers the captured launches point at
  std::vector<cudaEvent_t> ev_pool;  // per-generation timing events
  // transport kernel choice (ABX_TRANSPORT_KERNEL_*) and the pooled kernel's
  // slot records
  int kernel_mode = ABX_TRANSPORT_KERNEL_AUTO;
  void* pool = nullptr;
  size_t pool_bytes = 0;
  // batch runs: histories per warp before it retires (0: persistent warps),
  // and the quota of the launch being made
  uint32_t warp_quota = 0;
  uint32_t launch_quota = 0;
};

static void ctx_free(abx_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  c->D.release();
  for (auto& b : c->bd) b.free_();
  for (auto& b : c->bf) b.free_();
  c->sd.free_();
  c->sf.free_();
  if (c->pool) cudaFree(c->pool);
  c->pool = nullptr;
  void* ps[] = {c->tally_gen, c->tally_avg, c->tally_var, c->st, c->run, c->gen_rec,
                c->ent_bins, c->ent_total, c->hist_count, c->offsets, c->block_sums, c->sec,
                c->aos_in, c->aos_out, c->trace, c->flush, c->pscore, c->pcount, c->prun,
                c->seg_off, c->seg_prob, c->seg_hid0, c->vprobs, c->vtallies};
  for (void* p : ps)
    if (p) cudaFree(p);
  if (c->st_host) cudaFreeHost(c->st_host);
  for (auto& e : c->gen_exec)
    if (e) cudaGraphExecDestroy(e);
  for (auto& g : c->gen_graph)
    if (g) cudaGraphDestroy(g);
  for (auto& e : c->gen_ev_ph)
    if (e) cudaEventDestroy(e);
  for (auto& e : c->ev_pool) cudaEventDestroy(e);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}


// ------------------------------------------------------------- utilities
__global__ void k_zero_d(double* p, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) p[i] = 0.;
}
static void zero_d(double* p, size_t n, cudaStream_t s) {
  if (!n) return;
  size_t b = std::min<size_t>((n + 255) / 256, 152 * 32);
  k_zero_d<<<(unsigned)b, 256, 0, s>>>(p, n);
}

// Resets the per-step counters; the next step transports `n` histories (or the
// device-held count when n == ~0).
__global__ void k_step_begin(DevState* st, unsigned long long n, double kcol, int converged, int use_dev) {
  st->next_hist = 0;
  if (!use_dev) {
    st->n_hist = n;
    st->kcol = kcol;
    st->converged = converged;
    st->err = 0;
    st->err_hist = 0;
  }
  st->site_count = 0;
  st->site_pos = 0;
  st->site_neg = 0;
  st->site_wsum = 0.;
  st->collisions = 0;
  st->flights = 0;
  st->lost = 0;
  for (int i = 0; i < 6; i++) st->scores[i] = 0.;
  st->trace_n = 0;
}

// Exclusive scan of hist_count[0..n) (n read on the device): three phases.
constexpr int SCAN_T = 256, SCAN_V = 8, SCAN_CHUNK = SCAN_T * SCAN_V;
// histories per generation from which FP64 contexts use the four-block kernels:
// about twice the 155,648 threads four 256-thread blocks on 152 SMs hold
constexpr double FP64_WIDE_MIN_HISTORIES = 300000.;
__global__ void k_scan_reduce(const uint32_t* in, const DevState* st, uint32_t* bsum) {
  __shared__ uint32_t sh[SCAN_T];
  const unsigned long long n = st->n_hist;
  unsigned long long base = (unsigned long long)blockIdx.x * SCAN_CHUNK;
  uint32_t acc = 0;
  for (int v = 0; v < SCAN_V; v++) {
    unsigned long long i = base + (unsigned long long)v * SCAN_T + threadIdx.x;
    if (i < n) acc += in[i];
  }
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int s = SCAN_T / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) bsum[blockIdx.x] = sh[0];
}
__global__ void k_scan_blocks(uint32_t* bsum, int nb) {
  __shared__ uint32_t sh[1024];
  // serial carry over tiles of 1024
  uint32_t carry = 0;
  for (int t0 = 0; t0 < nb; t0 += 1024) {
    int i = t0 + threadIdx.x;
    uint32_t v = i < nb ? bsum[i] : 0;
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
      uint32_t a = threadIdx.x >= (unsigned)o ? sh[threadIdx.x - o] : 0;
      __syncthreads();
      sh[threadIdx.x] += a;
      __syncthreads();
    }
    if (i < nb) bsum[i] = carry + sh[threadIdx.x] - v;
    uint32_t tot = sh[1023];
    __syncthreads();
    carry += tot;
  }
}
__global__ void k_scan_apply(const uint32_t* in, const DevState* st, const uint32_t* bsum, uint32_t* out) {
  __shared__ uint32_t sh[SCAN_T];
  const unsigned long long n = st->n_hist;
  unsigned long long base = (unsigned long long)blockIdx.x * SCAN_CHUNK + (unsigned long long)threadIdx.x * SCAN_V;
  uint32_t loc[SCAN_V];
  uint32_t acc = 0;
  for (int v = 0; v < SCAN_V; v++) {
    unsigned long long i = base + v;
    loc[v] = i < n ? in[i] : 0;
    acc += loc[v];
  }
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int o = 1; o < SCAN_T; o <<= 1) {
    uint32_t a = threadIdx.x >= (unsigned)o ? sh[threadIdx.x - o] : 0;
    __syncthreads();
    sh[threadIdx.x] += a;
    __syncthreads();
  }
  uint32_t run = bsum[blockIdx.x] + sh[threadIdx.x] - acc;
  for (int v = 0; v < SCAN_V; v++) {
    unsigned long long i = base + v;
    if (i < n) out[i] = run;
    run += loc[v];
  }
}

// Counting sort of the fission sites into BankedParticle::operator< order
// (include/simulation/particle.hpp:59-65), fused with the construction of the
// next generation (src/power_iterator.cpp:359-404): weight normalisation to
// nparticles/W, history ids in bank order, per-history skip-ahead seeding,
// and the pre-normalisation Shannon entropy (src/entropy.cpp:32-64).
template <class R>
__global__ void k_next_bank(SiteT<R> S, DevState* st, const uint32_t* off, BankT<R> cur, BankT<R> nxt,
                            const ProbT* probs, RunAcc* run, uint64_t cap, double* ent_bins, double* ent_total) {
  const unsigned long long ns = st->site_count;
  const ProbT& P = probs[0];
  // normalize_weights (src/power_iterator.cpp:538-586): N over the bank's net
  // weight, sites of weight +-1 unless the collisions are branchless
  const double W = P.branchless ? st->site_wsum : (double)st->site_pos - (double)st->site_neg;
  // a combed bank is normalised on the host, in the reference's summation order
  const double wpp = (P.branchless & ABX_BRANCHLESS_COMBING) ? 1. : P.nparticles / W;
  const unsigned long long g0 = run->global_hist;
  double w_in_mesh = 0.;  // this thread's share of the entropy total
  for (unsigned long long j = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; j < ns && j < cap;
       j += (unsigned long long)gridDim.x * blockDim.x) {
    uint32_t h = S.hist[j];
    uint64_t d = (uint64_t)off[h] + S.dau[j];
    if (d >= cap) continue;
    R x = S.x[j], y = S.y[j], z = S.z[j];
    R ws = S.w[j];
    nxt.x[d] = x; nxt.y[d] = y; nxt.z[d] = z;
    nxt.ux[d] = S.ux[j]; nxt.uy[d] = S.uy[j]; nxt.uz[d] = S.uz[j];
    nxt.E[d] = S.E[j];
    nxt.w[d] = (R)((double)ws * wpp);
    nxt.w2[d] = R(0);
    uint64_t hid = g0 + d;
    nxt.hid[d] = hid;
    nxt.rng[d] = pcg_advance(pcg_seeded(P.seed), P.stride * hid);
    nxt.fam[d] = cur.fam[h];
    if (P.ent_on) {
      int nx = (int)floor(((double)x - P.ent_low[0]) / P.ent_d[0]);
      int ny = (int)floor(((double)y - P.ent_low[1]) / P.ent_d[1]);
      int nz = (int)floor(((double)z - P.ent_low[2]) / P.ent_d[2]);
      if (nx >= 0 && nx < P.ent_shape[0] && ny >= 0 && ny < P.ent_shape[1] && nz >= 0 && nz < P.ent_shape[2]) {
        w_in_mesh += (double)ws;
        atomicAdd(ent_bins + ((size_t)P.ent_shape[1] * P.ent_shape[2] * nx + (size_t)P.ent_shape[2] * ny + nz), (double)ws);
      }
    }
  }
  // the entropy total: one atomic per warp instead of one per site on a
  // single address
  if (P.ent_on) {
    for (int o = 16; o > 0; o >>= 1) w_in_mesh += __shfl_down_sync(0xffffffffu, w_in_mesh, o);
    if ((threadIdx.x & 31u) == 0 && w_in_mesh != 0.) atomicAdd(ent_total, w_in_mesh);
  }
}

// Tallies::update_avg_and_var (src/tallies.cpp:268-280)
__device__ void upd(int gen, double x, double& avg, double& var) {
  double dgen = (double)gen, a0 = avg, v0 = var;
  avg = a0 + (x - a0) / dgen;
  if (gen > 1) var = v0 + ((x - a0) * (x - a0) / dgen) - (v0 / (dgen - 1.));
}

// End of a generation: Tallies::calc_gen_values (src/tallies.cpp:159-181),
// Entropy::calculate_entropy (src/entropy.cpp:74-93), scalar record_generation,
// and the bank swap bookkeeping.  One block.
__global__ void k_gen_end(DevState* st, RunAcc* run, const ProbT* probs, abx_gen_record* rec, int hist_cap,
                          double* ent_bins, const double* ent_total, size_t nbins, uint64_t cap, int keig,
                          int nignored) {
  __shared__ double sh[1024];
  const ProbT& P = probs[0];
  double acc = 0.;
  double tw = ent_total ? *ent_total : 0.;
  for (size_t b = threadIdx.x; b < nbins; b += blockDim.x) {
    double p = fabs(ent_bins[b]) / tw;
    if (p > 1.0) {
    } else if (p != 0.) {
      acc -= p * log2(p);
    }
  }
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < (unsigned)s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  __syncthreads();
  for (size_t b = threadIdx.x; b < nbins; b += blockDim.x) ent_bins[b] = 0.;
  if (threadIdx.x != 0) return;
  const double N = P.nparticles;
  double k_col = st->scores[0] / N, k_abs = st->scores[1] / N, k_trk = st->scores[2] / N;
  double leak = st->scores[4] / N, mig = st->scores[5] / N;
  int g = run->gen;  // 0-based index of this generation
  if (g < hist_cap) {
    abx_gen_record& r = rec[g];
    r.kcol = k_col;
    r.entropy = P.ent_on ? sh[0] : 0.;
    r.collisions = st->collisions;
    r.flights = st->flights;
    r.histories = st->n_hist;
    r.sites = st->site_count;
    r.lost = st->lost;
  }
  run->total_coll += st->collisions;
  run->total_flights += st->flights;
  run->total_hist += st->n_hist;
  if (st->converged) {
    run->active++;
    upd(run->active, k_col, run->kcol_avg, run->kcol_var);
    upd(run->active, k_abs, run->kabs_avg, run->kabs_var);
    upd(run->active, k_trk, run->ktrk_avg, run->ktrk_var);
    upd(run->active, leak, run->leak_avg, run->leak_var);
    upd(run->active, mig, run->mig_avg, run->mig_var);
  }
  run->gen = g + 1;
  if (ent_total) *(double*)ent_total = 0.;
  if (keig) {
    unsigned long long ns = st->site_count;
    if (ns == 0 && st->err == 0) st->err = ABX_ERR_NO_FISSION;
    if (ns > cap && st->err == 0) st->err = ABX_ERR_CAPACITY;
    run->global_hist += ns;
    st->n_hist = ns > cap ? cap : ns;
    st->kcol = k_col;
    st->converged = (nignored == 0) || (g + 1 >= nignored) ? 1 : 0;
  }
}

// Per-problem batch statistics of a batch context.  Batch b of problem p was
// scored as virtual problem v = p*nb + b; the leakage estimator of
// Tallies::calc_gen_values / record_generation (src/tallies.cpp:159-203,
// 268-280) is applied to batches 0..nb-1 in order, as the reference's loop
// over generations does, then the per-batch sums are cleared.
struct ProbRun {
  double leak_avg, leak_var;
  unsigned long long coll, flights, hist, lost;
};
__global__ void k_prob_record(double* ps, unsigned long long* pc, ProbRun* pr, const ProbT* probs, int np,
                              int nb) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
    ProbRun r{};
    for (int b = 0; b < nb; b++) {
      double* s = ps + ((size_t)p * nb + b) * ABX_PSCORES;
      unsigned long long* c = pc + ((size_t)p * nb + b) * ABX_PCOUNTS;
      upd(b + 1, s[3] / probs[p].nparticles, r.leak_avg, r.leak_var);
      r.coll += c[0];
      r.flights += c[1];
      r.hist += c[2];
      r.lost += c[3];
      for (int k = 0; k < ABX_PSCORES; k++) s[k] = 0.;
      for (int k = 0; k < ABX_PCOUNTS; k++) c[k] = 0ull;
    }
    pr[p] = r;
  }
}

// MeshTally::record_generation + clear_generation (src/mesh_tally.cpp:121-152)
// for nb batches scored side by side: bin i of batch b sits at gen[b*n + i];
// the batches are recorded in order into avg/var (which start from zero).
__global__ void k_tally_record_batches(double* gen, double* avg, double* var, size_t n, int nb) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    double a = 0., v = 0.;
    for (int b = 0; b < nb; b++) {
      const double dg = (double)(b + 1);
      const double val = gen[(size_t)b * n + i];
      const double old_avg = a;
      a = old_avg + (val - old_avg) / dg;
      v = v + (((val - old_avg) * (val - a) - (v)) / dg);
      gen[(size_t)b * n + i] = 0.;
    }
    avg[i] = a;
    var[i] = v;
  }
}

// The same, with the generation's bookkeeping read on the device (for the
// captured generation step): a generation is recorded when it is active
// (DevState::converged, set by the previous k_gen_end), as active generation
// number RunAcc::active + 1.
__global__ void k_tally_record_dev(double* gen, double* avg, double* var, size_t n, const DevState* st,
                                   const struct RunAcc* run);

// MeshTally::record_generation + clear_generation (src/mesh_tally.cpp:121-152)
__global__ void k_tally_record(double* gen, double* avg, double* var, size_t n, double mult, int rec,
                               double dg) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    if (rec) {
      double old_avg = avg[i];
      double val = gen[i] * mult;
      double a = old_avg + (val - old_avg) / dg;
      avg[i] = a;
      double v = var[i];
      v = v + (((val - old_avg) * (val - a) - (v)) / dg);
      var[i] = v;
    }
    gen[i] = 0.;
  }
}

__global__ void k_tally_record_dev(double* gen, double* avg, double* var, size_t n, const DevState* st,
                                   const RunAcc* run) {
  const int rec = st->converged;
  const double dg = (double)(run->active + 1);
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    if (rec) {
      double old_avg = avg[i];
      double val = gen[i];
      double a = old_avg + (val - old_avg) / dg;
      avg[i] = a;
      double v = var[i];
      v = v + (((val - old_avg) * (val - a) - (v)) / dg);
      var[i] = v;
    }
    gen[i] = 0.;
  }
}

// AoS host particles -> SoA device bank.
template <class R> __global__ void k_bank_from_aos(const abx_particle* in, size_t n, BankT<R> b) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const abx_particle p = in[i];
    b.x[i] = (R)p.r[0]; b.y[i] = (R)p.r[1]; b.z[i] = (R)p.r[2];
    b.ux[i] = (R)p.u[0]; b.uy[i] = (R)p.u[1]; b.uz[i] = (R)p.u[2];
    b.E[i] = (R)p.E; b.w[i] = (R)p.wgt; b.w2[i] = (R)p.wgt2;
    b.rng[i] = p.rng_state; b.hid[i] = p.history_id; b.fam[i] = p.family_id;
  }
}
// SoA device bank -> AoS particles.
template <class R> __global__ void k_bank_to_aos(BankT<R> b, size_t n, abx_particle* out) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    abx_particle p;
    p.r[0] = b.x[i]; p.r[1] = b.y[i]; p.r[2] = b.z[i];
    p.u[0] = b.ux[i]; p.u[1] = b.uy[i]; p.u[2] = b.uz[i];
    p.E = b.E[i]; p.wgt = b.w[i]; p.wgt2 = b.w2[i];
    p.rng_state = b.rng[i]; p.history_id = b.hid[i]; p.family_id = b.fam[i];
    out[i] = p;
  }
}
// Sorted sites -> AoS BankedParticles.  `cap` bounds both the site arrays
// and `out`: the transport kernel counts sites past its capacity without
// storing them, so entries at or beyond `cap` were never written.
template <class R>
__global__ void k_sites_to_aos(SiteT<R> S, const DevState* st, const uint32_t* off, BankT<R> cur, abx_site* out,
                               uint64_t cap) {
  const unsigned long long ns = st->site_count < cap ? st->site_count : (unsigned long long)cap;
  for (unsigned long long j = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; j < ns;
       j += (unsigned long long)gridDim.x * blockDim.x) {
    uint32_t h = S.hist[j];
    uint64_t d = (uint64_t)off[h] + S.dau[j];
    if (d >= cap) continue;
    abx_site s;
    s.r[0] = S.x[j]; s.r[1] = S.y[j]; s.r[2] = S.z[j];
    s.u[0] = S.ux[j]; s.u[1] = S.uy[j]; s.u[2] = S.uz[j];
    s.E = S.E[j]; s.wgt = S.w[j]; s.wgt2 = 0.;
    s.parent_history_id = cur.hid[h];
    s.parent_daughter_id = S.dau[j];
    s.family_id = cur.fam[h];
    out[d] = s;
  }
}

// ------------------------------------------------------------ ctx helpers

static int ensure_counts(abx_ctx* c, size_t n) {
  if (n <= c->count_cap) return ABX_OK;
  size_t cap = std::max<size_t>(headroom(n), 1024);
  if (c->hist_count) cudaFree(c->hist_count);
  if (c->offsets) cudaFree(c->offsets);
  if (c->block_sums) cudaFree(c->block_sums);
  c->hist_count = c->offsets = c->block_sums = nullptr;
  CUDA_TRY(cudaMalloc(&c->hist_count, cap * sizeof(uint32_t)));
  CUDA_TRY(cudaMalloc(&c->offsets, cap * sizeof(uint32_t)));
  CUDA_TRY(cudaMalloc(&c->block_sums, ((cap + SCAN_CHUNK - 1) / SCAN_CHUNK + 1) * sizeof(uint32_t)));
  c->count_cap = cap;
  return ABX_OK;
}

static int ensure_banks(abx_ctx* c, size_t n, bool mixed, bool with_prob) {
  int rc;
  c->pi_bank = -1;  // every caller writes bank 0 next
  // banks of the transport precision only (mixed runs sample in FP32)
  for (int i = 0; i < 2; i++) {
    if (!mixed && (c->bd[i].cap < n || (with_prob && !c->bd[i].b.prob)))
      if ((rc = c->bd[i].alloc(headroom(n), with_prob)) != ABX_OK) return rc;
    if (mixed && (c->bf[i].cap < n || (with_prob && !c->bf[i].b.prob)))
      if ((rc = c->bf[i].alloc(headroom(n), with_prob)) != ABX_OK) return rc;
  }
  return ensure_counts(c, n);
}

static int ensure_sites(abx_ctx* c, size_t n, bool mixed) {
  int rc;
  if (mixed) {
    if (c->sf.cap < n && (rc = c->sf.alloc(headroom(n))) != ABX_OK) return rc;
  } else {
    if (c->sd.cap < n && (rc = c->sd.alloc(headroom(n))) != ABX_OK) return rc;
  }
  return ABX_OK;
}

// The AoS staging buffers of the C-ABI's host records grow with headroom,
// like the work buffers: a reallocation's cudaFree waits for the whole device,
// and bank sizes move from one call to the next.
static int ensure_aos_in(abx_ctx* c, size_t n) {
  if (c->aos_in_cap >= n) return ABX_OK;
  if (c->aos_in) cudaFree(c->aos_in);
  c->aos_in = nullptr;
  c->aos_in_cap = 0;
  const size_t cap = headroom(n);
  CUDA_TRY(cudaMalloc(&c->aos_in, cap * sizeof(abx_particle)));
  c->aos_in_cap = cap;
  return ABX_OK;
}
static int ensure_aos_out(abx_ctx* c, size_t n) {
  if (c->aos_out_cap >= n) return ABX_OK;
  if (c->aos_out) cudaFree(c->aos_out);
  c->aos_out = nullptr;
  c->aos_out_cap = 0;
  const size_t cap = headroom(n);
  CUDA_TRY(cudaMalloc(&c->aos_out, cap * sizeof(abx_site)));
  c->aos_out_cap = cap;
  return ABX_OK;
}

static int kernel_code(const abx_ctx* c);

// Histories of this context can put particles on a secondary stack:
// fission in fixed-source problems, splitting in Carter tracking and in
// branchless collisions with splitting.
static bool needs_stacks(const abx_ctx* c) {
  const bool bl_split = (c->prob0.branchless & ABX_BRANCHLESS_SPLITTING) != 0;
  return c->prob0.tracking == ABX_TRACK_CARTER || bl_split ||
         (c->prob0.mode == ABX_MODE_FIXED_SOURCE && c->fissile_any);
}

// The pooled kernel serves delta and surface tracking with branching
// collisions and no secondary stacks; everything else runs in the history
// kernel.
static bool pool_eligible(const abx_ctx* c) {
  return (c->prob0.tracking == ABX_TRACK_DELTA || c->prob0.tracking == ABX_TRACK_SURFACE) && !c->prob0.branchless &&
         !needs_stacks(c) && c->block <= 256;
}
static bool use_pool(const abx_ctx* c) {
  if (c->kernel_mode == ABX_TRANSPORT_KERNEL_HISTORY || !pool_eligible(c)) return false;
  if (c->kernel_mode == ABX_TRANSPORT_KERNEL_POOL) return true;
  return false;  // automatic choice: the history kernel
}
static int occupancy_of(const abx_ctx* c, bool mixed, int block) {
  if (use_pool(c)) return mixed ? occupancy_pool_f(kernel_code(c), c->all_iso, block) : occupancy_pool_d(kernel_code(c), block);
  return mixed ? occupancy_f(kernel_code(c), c->all_iso, block) : occupancy_d(kernel_code(c), block);
}
static int ensure_pool(abx_ctx* c, bool mixed) {
  if (!use_pool(c)) return ABX_OK;
  const size_t warps = ((size_t)c->grid * c->block + 31) / 32;
  const size_t need = warps * POOL_SLOTS_PER_WARP * (mixed ? pool_slot_bytes_f() : pool_slot_bytes_d());
  if (c->pool && c->pool_bytes >= need) return ABX_OK;
  if (c->pool) cudaFree(c->pool);
  c->pool = nullptr;
  c->pool_bytes = 0;
  CUDA_TRY(cudaMalloc(&c->pool, need));
  c->pool_bytes = need;
  return ABX_OK;
}

static int ensure_stacks(abx_ctx* c, bool mixed);
static int ensure_sec(abx_ctx* c, bool mixed) {
  int rc = ensure_stacks(c, mixed);
  if (rc != ABX_OK) return rc;
  return ensure_pool(c, mixed);
}

static int ensure_stacks(abx_ctx* c, bool mixed) {
  // secondaries: fission in fixed-source problems, splitting in Carter tracking
  // splitting (Carter tracking, branchless collisions) needs the stack in
  // every mode
  const bool bl_split = (c->prob0.branchless & ABX_BRANCHLESS_SPLITTING) != 0;
  const bool carter = c->prob0.tracking == ABX_TRACK_CARTER || bl_split;
  if (!carter && (c->prob0.mode != ABX_MODE_FIXED_SOURCE || !c->fissile_any)) return ABX_OK;
  // branchless splitting piles copies up within a history (the oracle saw
  // 190 pending copies in 2e6 histories of the critical slabs)
  const uint32_t want = bl_split ? 512 : 64;
  if (carter && c->sec_cap < want) {
    if (c->sec) cudaFree(c->sec);
    c->sec = nullptr;
    c->sec_threads = 0;
    c->sec_cap = want;
  }
  size_t threads = (size_t)c->grid * c->block;
  size_t need = threads * c->sec_cap * 9 * (mixed ? sizeof(float) : sizeof(double));
  if (c->sec && c->sec_threads >= threads) return ABX_OK;
  if (c->sec) cudaFree(c->sec);
  c->sec = nullptr;
  CUDA_TRY(cudaMalloc(&c->sec, need));
  c->sec_threads = threads;
  return ABX_OK;
}

static int check_state(abx_ctx* c) {
  CUDA_TRY(cudaMemcpyAsync(c->st_host, c->st, sizeof(DevState), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  int e = c->st_host->err;
  if (e) {
    const char* what = e == ABX_ERR_LOST_PARTICLE ? "a particle became lost"
                       : e == ABX_ERR_MAJORANT   ? "total cross section exceeded the majorant"
                       : e == ABX_ERR_CAPACITY   ? "fission bank or secondary stack capacity exceeded"
                       : e == ABX_ERR_TIMEOUT    ? "a history exceeded the event limit"
                       : e == ABX_ERR_NO_FISSION ? "No fission neutrons were produced."
                                                 : "invalid geometry or particle state";
    return fail(e, "%s (history %llu)", what, (unsigned long long)c->st_host->err_hist);
  }
  return ABX_OK;
}

// which transport kernel: the tracking mode, plus the branchless-collision
// bit, plus the single-problem bit outside runs that score per problem, plus
// the four-block bit of large FP64 contexts
static int kernel_code(const abx_ctx* c) {
  return c->prob0.tracking | (c->prob0.branchless ? ABX_KERNEL_BRANCHLESS : 0) |
         (c->batch_scores ? 0 : ABX_KERNEL_SINGLE) | (c->fp64_wide ? ABX_KERNEL_WIDE : 0);
}

template <class R> static TransportArgs<R> make_args(abx_ctx* c, const BankT<R>& bank, const SiteT<R>& sites,
                                                     size_t site_cap) {
  TransportArgs<R> A{};
  A.T = c->batch_scores ? c->batch_tables : c->D.T;
  A.T.tally_gen = c->tally_gen;
  A.bank = bank;
  A.sites = sites;
  A.site_cap = site_cap;
  A.hist_count = c->hist_count;
  A.sec = (R*)c->sec;
  A.sec_cap = c->sec_cap;
  A.st = c->st;
  A.trace = c->trace_nhist ? c->trace : nullptr;
  A.trace_nhist = c->trace_nhist;
  A.trace_cap = c->trace_cap;
  A.max_events = c->max_events;
  A.pscore = c->batch_scores ? c->pscore : nullptr;
  A.pcount = c->batch_scores ? c->pcount : nullptr;
  A.pool = use_pool(c) ? c->pool : nullptr;
  A.warp_quota = c->launch_quota;
  return A;
}

static int launch_transport(abx_ctx* c, bool mixed, int which_bank, size_t site_cap) {
  const bool pooled = use_pool(c);
  if (pooled && !c->pool) return fail(ABX_ERR_INVALID, "pooled transport kernel without its slot records");
  if (mixed) {
    TransportArgs<float> A = make_args<float>(c, c->bf[which_bank].b, c->sf.s, site_cap);
    if (pooled) launch_pool_f(A, kernel_code(c), c->all_iso, c->grid, c->block, c->stream);
    else launch_transport_f(A, kernel_code(c), c->all_iso, c->trace_nhist > 0, c->grid, c->block, c->stream);
  } else {
    TransportArgs<double> A = make_args<double>(c, c->bd[which_bank].b, c->sd.s, site_cap);
    if (pooled) launch_pool_d(A, kernel_code(c), c->grid, c->block, c->stream);
    else launch_transport_d(A, kernel_code(c), c->trace_nhist > 0, c->grid, c->block, c->stream);
  }
  CUDA_TRY(cudaGetLastError());
  return ABX_OK;
}

static void launch_scan(abx_ctx* c, size_t cap) {
  unsigned nb = (unsigned)((cap + SCAN_CHUNK - 1) / SCAN_CHUNK);
  if (nb == 0) nb = 1;
  k_scan_reduce<<<nb, SCAN_T, 0, c->stream>>>(c->hist_count, c->st, c->block_sums);
  k_scan_blocks<<<1, 1024, 0, c->stream>>>(c->block_sums, (int)nb);
  k_scan_apply<<<nb, SCAN_T, 0, c->stream>>>(c->hist_count, c->st, c->block_sums, c->offsets);
}

static unsigned grid_for(size_t n) {
  size_t b = (n + 255) / 256;
  if (b < 1) b = 1;
  if (b > 152 * 16) b = 152 * 16;
  return (unsigned)b;
}

// ------------------------------------------------------------------- C-ABI
static int create_ctx(const abx_problem* problems, int nprob, int device, abx_ctx** out) {
  if (!out) return fail(ABX_ERR_INVALID, "null output pointer");
  *out = nullptr;
  if (!problems || nprob <= 0) return fail(ABX_ERR_INVALID, "no problems");
  const abx_problem* problem = &problems[0];
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) return fail(ABX_ERR_CUDA, "no CUDA device available");
  if (device < 0 || device >= ndev) return fail(ABX_ERR_INVALID, "device %d out of range", device);
  abx_ctx* c = new abx_context();
  c->device = device;
  c->nprob = nprob;
  int rc = ABX_OK;
  for (int i = 0; i < nprob && rc == ABX_OK; i++) {
    const abx_settings& s = problems[i].settings;
    if (nprob > 1 && (s.mode != ABX_MODE_FIXED_SOURCE || s.tracking != problem->settings.tracking ||
                      s.precision != problem->settings.precision))
      rc = fail(ABX_ERR_UNSUPPORTED,
                "problem %d: a batch holds fixed-source problems of one tracking mode and one precision", i);
    else
      rc = append_problem(c->P, &problems[i]);
  }
  if (rc) {
    delete c;
    return rc;
  }
  c->prob0 = c->P.probs[0];
  for (const MatT& m : c->P.mats) c->fissile_any |= m.fissile != 0;
  c->all_iso = true;
  for (const MatT& m : c->P.mats) c->all_iso = c->all_iso && m.iso != 0;
  const int prec = problem->settings.precision;
  if (prec != ABX_PREC_FP64 && prec != ABX_PREC_MIXED) {
    delete c;
    return fail(ABX_ERR_INVALID, "precision %d", prec);
  }
  c->prec = prec;
  // generations large enough to fill four FP64 blocks per SM twice over run
  // the four-block FP64 kernels (transport_fp64_wide.cu)
  c->fp64_wide = prec == ABX_PREC_FP64 && !c->prob0.branchless &&
                 (c->prob0.tracking == ABX_TRACK_DELTA || c->prob0.tracking == ABX_TRACK_SURFACE) &&
                 problem->settings.nparticles >= FP64_WIDE_MIN_HISTORIES;
  auto bail = [&](int code) {
    ctx_free(c);
    return code;
  };
  if (cudaSetDevice(device) != cudaSuccess) return bail(fail(ABX_ERR_CUDA, "cudaSetDevice failed"));
  cudaDeviceProp prop;
  cudaGetDeviceProperties(&prop, device);
  c->nsm = prop.multiProcessorCount;
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess)
    return bail(fail(ABX_ERR_CUDA, "stream creation failed"));
  cudaEventCreate(&c->ev0);
  cudaEventCreate(&c->ev1);
  if ((rc = upload(c->P, c->D)) != ABX_OK) return bail(rc);
  size_t nb = (size_t)std::max<int64_t>(c->P.tally_bins, 1);
  if (cudaMalloc(&c->tally_gen, nb * 8) || cudaMalloc(&c->tally_avg, nb * 8) || cudaMalloc(&c->tally_var, nb * 8))
    return bail(fail(ABX_ERR_OOM, "tally allocation failed"));
  c->tally_gen_cap = nb;
  c->tally_rv_cap = nb;
  cudaMemset(c->tally_gen, 0, nb * 8);
  cudaMemset(c->tally_avg, 0, nb * 8);
  cudaMemset(c->tally_var, 0, nb * 8);
  if (cudaMalloc(&c->st, sizeof(DevState)) || cudaMallocHost(&c->st_host, sizeof(DevState)) ||
      cudaMalloc(&c->run, sizeof(RunAcc)))
    return bail(fail(ABX_ERR_OOM, "state allocation failed"));
  cudaMemset(c->st, 0, sizeof(DevState));
  cudaMemset(c->run, 0, sizeof(RunAcc));
  c->ent_nbins = problem->entropy.enabled
                     ? (size_t)problem->entropy.shape[0] * problem->entropy.shape[1] * problem->entropy.shape[2]
                     : 1;
  if (cudaMalloc(&c->ent_bins, c->ent_nbins * 8) || cudaMalloc(&c->ent_total, 8))
    return bail(fail(ABX_ERR_OOM, "entropy allocation failed"));
  cudaMemset(c->ent_bins, 0, c->ent_nbins * 8);
  cudaMemset(c->ent_total, 0, 8);
  int block = problem->settings.block_size > 0 ? problem->settings.block_size : 256;
  block = std::max(32, std::min(256, block / 32 * 32));
  c->block = block;
  int occ = occupancy_of(c, prec == ABX_PREC_MIXED, block);
  if (occ < 1) occ = 1;
  c->grid = c->nsm * occ;
  if (cudaDeviceSynchronize() != cudaSuccess) return bail(fail(ABX_ERR_CUDA, "device sync failed"));
  *out = c;
  return ABX_OK;
}

extern "C" int abx_create(const abx_problem* problem, int device, abx_ctx** out) {
  if (!problem) {
    if (out) *out = nullptr;
    return fail(ABX_ERR_INVALID, "null problem");
  }
  return create_ctx(problem, 1, device, out);
}

extern "C" int abx_create_batch(const abx_problem* problems, int n_problems, int device, abx_ctx** out) {
  return create_ctx(problems, n_problems, device, out);
}

extern "C" int abx_destroy(abx_ctx* c) {
  ctx_free(c);
  return ABX_OK;
}

static bool mixed_of(const abx_ctx* c) { return c->prec == ABX_PREC_MIXED; }

// Samples S.n source histories into bank 0 of the transport precision: FP64
// runs sample in FP64 (the reference's arithmetic), mixed runs sample in FP32
// straight into the float bank.  S carries the tables, counts and segments.
static void sample_bank0(abx_ctx* c, SourceArgs& S, bool mixed, bool with_prob) {
  S.out_off = 0;
  S.st = c->st;
  if (mixed) {
    BankT<float>& b = c->bf[0].b;
    S.fx = b.x; S.fy = b.y; S.fz = b.z; S.fux = b.ux; S.fuy = b.uy; S.fuz = b.uz; S.fE = b.E; S.fw = b.w;
    S.fw2 = b.w2; S.rng = b.rng; S.hid = b.hid; S.fam = b.fam; S.probv = with_prob ? b.prob : nullptr;
    launch_sources_f(S, c->stream);
  } else {
    BankT<double>& b = c->bd[0].b;
    S.x = b.x; S.y = b.y; S.z = b.z; S.ux = b.ux; S.uy = b.uy; S.uz = b.uz; S.E = b.E; S.w = b.w;
    S.w2 = b.w2; S.rng = b.rng; S.hid = b.hid; S.fam = b.fam; S.probv = with_prob ? b.prob : nullptr;
    launch_sources(S, c->stream);
  }
}

extern "C" int abx_sample_sources(abx_ctx* c, uint64_t first, size_t n, abx_particle* out) {
  if (!c || (!out && n)) return fail(ABX_ERR_INVALID, "bad arguments");
  if (c->prob0.src_count <= 0) return fail(ABX_ERR_INVALID, "problem has no sources");
  if (n == 0) return ABX_OK;
  cudaSetDevice(c->device);
  int rc;
  if ((rc = ensure_banks(c, n, false, false)) != ABX_OK) return rc;
  CUDA_TRY(cudaMemsetAsync(c->st, 0, sizeof(DevState), c->stream));
  SourceArgs S{};
  S.T = c->D.T;
  S.prob = 0;
  S.first_hid = first;
  S.n = n;
  BankT<double>& b = c->bd[0].b;
  S.x = b.x; S.y = b.y; S.z = b.z; S.ux = b.ux; S.uy = b.uy; S.uz = b.uz; S.E = b.E; S.w = b.w; S.w2 = b.w2;
  S.rng = b.rng; S.hid = b.hid; S.fam = b.fam; S.probv = nullptr; S.out_off = 0; S.st = c->st;
  launch_sources(S, c->stream);
  if ((rc = ensure_aos_in(c, n)) != ABX_OK) return rc;
  k_bank_to_aos<double><<<grid_for(n), 256, 0, c->stream>>>(b, n, c->aos_in);
  CUDA_TRY(cudaGetLastError());
  if ((rc = check_state(c)) != ABX_OK) return rc;
  CUDA_TRY(cudaMemcpyAsync(out, c->aos_in, n * sizeof(abx_particle), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  return ABX_OK;
}

extern "C" int abx_transport(abx_ctx* c, const abx_particle* bank, size_t n, double kcol, int converged,
                             abx_site* sites, size_t site_capacity, size_t* n_sites, abx_scores* scores) {
  if (!c || (!bank && n)) return fail(ABX_ERR_INVALID, "bad arguments");
  if (!(kcol > 0)) return fail(ABX_ERR_INVALID, "kcol must be positive");
  if (n > 0xffffffffull) return fail(ABX_ERR_INVALID, "at most 2^32-1 histories per call");
  if (c->nprob > 1)
    return fail(ABX_ERR_UNSUPPORTED, "a batch context transports through abx_run_fixed_source_batch only");
  cudaSetDevice(c->device);
  const bool mixed = mixed_of(c);
  const bool keig = c->prob0.mode == ABX_MODE_K_EIGENVALUE;
  int rc;
  size_t cap = std::max<size_t>(n, 1);
  if ((rc = ensure_banks(c, cap, mixed, false)) != ABX_OK) return rc;
  size_t scap = keig ? std::max<size_t>(site_capacity, 1) : 1;
  if ((rc = ensure_sites(c, scap, mixed)) != ABX_OK) return rc;
  if ((rc = ensure_sec(c, mixed)) != ABX_OK) return rc;
  if ((rc = ensure_aos_in(c, cap)) != ABX_OK) return rc;
  if (n) CUDA_TRY(cudaMemcpyAsync(c->aos_in, bank, n * sizeof(abx_particle), cudaMemcpyHostToDevice, c->stream));
  if (mixed) k_bank_from_aos<float><<<grid_for(n), 256, 0, c->stream>>>(c->aos_in, n, c->bf[0].b);
  else k_bank_from_aos<double><<<grid_for(n), 256, 0, c->stream>>>(c->aos_in, n, c->bd[0].b);
  k_step_begin<<<1, 1, 0, c->stream>>>(c->st, n, kcol, converged, 0);
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaEventRecord(c->ev0, c->stream));
  if ((rc = launch_transport(c, mixed, 0, keig ? scap : 0)) != ABX_OK) return rc;
  CUDA_TRY(cudaEventRecord(c->ev1, c->stream));
  if ((rc = check_state(c)) != ABX_OK) return rc;
  float ms = 0.f;
  cudaEventElapsedTime(&ms, c->ev0, c->ev1);
  c->last_ms = ms;
  const DevState& h = *c->st_host;
  size_t ns = keig ? (size_t)h.site_count : 0;
  if (n_sites) *n_sites = ns;
  if (scores) {
    scores->k_col = h.scores[0];
    scores->k_abs = h.scores[1];
    scores->k_trk = h.scores[2];
    scores->k_tot = h.scores[3];
    scores->leakage = h.scores[4];
    scores->mig_area = h.scores[5];
    scores->collisions = h.collisions;
    scores->flights = h.flights;
    scores->lost = h.lost;
  }
  if (keig && ns > site_capacity)
    return fail(ABX_ERR_CAPACITY, "fission bank capacity %zu < %zu sites", site_capacity, ns);
  if (keig && ns && sites) {
    launch_scan(c, n);
    if ((rc = ensure_aos_out(c, ns)) != ABX_OK) return rc;
    if (mixed) k_sites_to_aos<float><<<grid_for(ns), 256, 0, c->stream>>>(c->sf.s, c->st, c->offsets, c->bf[0].b, c->aos_out, ns);
    else k_sites_to_aos<double><<<grid_for(ns), 256, 0, c->stream>>>(c->sd.s, c->st, c->offsets, c->bd[0].b, c->aos_out, ns);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaMemcpyAsync(sites, c->aos_out, ns * sizeof(abx_site), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
  }
  return ABX_OK;
}

// ------------------------------------------------------------- autotuner
// Picks the transport launch shape (threads per block, resident blocks per
// SM) by timing the problem's own first-generation bank: `n_probe` source
// histories are sampled once, then transported three times per candidate
// (the same histories each time, so every candidate does identical work;
// tallies scored as in active generations; the first run warms the caches)
// and the shape with the fastest run is kept for the context.  Results do not depend on the shape.
extern "C" int abx_autotune(abx_ctx* c, size_t n_probe, int* block_out, int* grid_out, double* best_ms) {
  if (!c || n_probe == 0 || n_probe > 0xffffffffull) return fail(ABX_ERR_INVALID, "bad arguments");
  if (c->prob0.src_count <= 0) return fail(ABX_ERR_INVALID, "problem has no sources");
  cudaSetDevice(c->device);
  const bool mixed = mixed_of(c);
  const bool keig = c->prob0.mode == ABX_MODE_K_EIGENVALUE;
  int rc;
  const size_t scap = keig ? 3 * n_probe + 4096 : 1;
  if ((rc = ensure_banks(c, n_probe, mixed, false)) != ABX_OK) return rc;
  if ((rc = ensure_sites(c, scap, mixed)) != ABX_OK) return rc;
  CUDA_TRY(cudaMemsetAsync(c->st, 0, sizeof(DevState), c->stream));
  SourceArgs S{};
  S.T = c->D.T;
  S.prob = 0;
  S.first_hid = 0;
  S.n = n_probe;
  sample_bank0(c, S, mixed, false);
  if ((rc = check_state(c)) != ABX_OK) return rc;
  // The probes score the problem's tallies, as active generations do, into a
  // scratch copy of the tally bins: the context's own bins stay untouched.
  double* probe_bins = nullptr;
  const size_t nbins = (size_t)std::max<int64_t>(c->P.tally_bins, 0);
  if (nbins && nbins <= (size_t(1) << 27)) CUDA_TRY(cudaMalloc(&probe_bins, nbins * 8));
  std::swap(c->tally_gen, probe_bins);
  const int converged = c->tally_gen != nullptr && nbins ? 1 : 0;
  const int block0 = c->block, grid0 = c->grid;
  int best_block = block0, best_grid = grid0;
  float best = -1.f;
  for (int block : {128, 256}) {
    const int occ = occupancy_of(c, mixed, block);
    for (int per_sm = 1; per_sm <= occ; per_sm++) {
      c->block = block;
      c->grid = c->nsm * per_sm;
      if ((rc = ensure_sec(c, mixed)) != ABX_OK) break;
      float ms = 0.f;
      for (int rep = 0; rep < 3; rep++) {  // the first run warms the caches; the faster of two counts
        k_step_begin<<<1, 1, 0, c->stream>>>(c->st, n_probe, 1.0, converged, 0);
        if (cudaEventRecord(c->ev0, c->stream) != cudaSuccess) { rc = fail(ABX_ERR_CUDA, "event record"); break; }
        if ((rc = launch_transport(c, mixed, 0, keig ? scap : 0)) != ABX_OK) break;
        if (cudaEventRecord(c->ev1, c->stream) != cudaSuccess) { rc = fail(ABX_ERR_CUDA, "event record"); break; }
        if ((rc = check_state(c)) != ABX_OK) break;
        float t = 0.f;
        cudaEventElapsedTime(&t, c->ev0, c->ev1);
        if (rep == 1 || (rep == 2 && t < ms)) ms = t;
      }
      if (rc) break;
      if (best < 0.f || ms < best) {
        best = ms;
        best_block = block;
        best_grid = c->grid;
      }
    }
    if (rc) break;
  }
  std::swap(c->tally_gen, probe_bins);
  if (probe_bins) cudaFree(probe_bins);
  c->block = rc ? block0 : best_block;
  c->grid = rc ? grid0 : best_grid;
  if (rc) return rc;
  if ((rc = ensure_sec(c, mixed)) != ABX_OK) return rc;
  if (block_out) *block_out = c->block;
  if (grid_out) *grid_out = c->grid;
  if (best_ms) *best_ms = best;
  return ABX_OK;
}

// ------------------------------------------------- transport, no allocation
// abx_transport_noalloc: the transport step for callers that must not
// allocate device memory while they run -- hosts that route every device
// allocation through their own pool and forbid direct cudaMalloc, loops that
// cannot afford the device synchronisation cudaMalloc/cudaFree imply, and
// processes running at their memory budget, where a late allocation can
// fail.  The caller owns the bank and
// site buffers (device memory); every per-call scratch array -- the SoA bank
// and fission-site arrays, per-history site counts, their prefix sums --
// lives in one file-scope device array of fixed size, reserved when the
// library is loaded on a device and held until the process exits.
static constexpr size_t NA_HIST = 16384;          // histories per call
static constexpr size_t NA_SITES = 4 * NA_HIST;   // fission sites per call
static constexpr size_t na_round(size_t b) { return (b + 255) / 256 * 256; }
static constexpr size_t NA_BANK_ARRAY = na_round(NA_HIST * 8);   // one SoA bank column (8-byte worst case)
static constexpr size_t NA_SITE_ARRAY = na_round(NA_SITES * 8);  // one SoA site column
static constexpr size_t NA_BLOCKS = (NA_HIST + SCAN_CHUNK - 1) / SCAN_CHUNK + 1;
static constexpr size_t NA_BYTES = 12 * NA_BANK_ARRAY + 8 * NA_SITE_ARRAY + 2 * na_round(NA_SITES * 4) +
                                   2 * na_round(NA_HIST * 4) + na_round(NA_BLOCKS * 4);
static __device__ __align__(256) unsigned char g_transport_scratch[NA_BYTES];

// The array's device address, looked up once per device with that device
// current (host code cannot use the symbol itself as a device pointer).
static std::mutex g_scratch_mu;
static void* g_scratch_addr[256];
static int scratch_address(int device, unsigned char** out) {
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (device < 0 || device >= 256) return fail(ABX_ERR_INVALID, "device %d out of range", device);
  if (!g_scratch_addr[device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_transport_scratch);
    if (e != cudaSuccess || !p)
      return fail(ABX_ERR_CUDA, "cudaGetSymbolAddress(transport scratch) failed: %s", cudaGetErrorString(e));
    g_scratch_addr[device] = p;
  }
  *out = (unsigned char*)g_scratch_addr[device];
  return ABX_OK;
}

template <class R> static void na_carve(unsigned char* base, BankT<R>& b, SiteT<R>& s, uint32_t*& counts,
                                        uint32_t*& offsets, uint32_t*& blocks) {
  unsigned char* p = base;
  R** br[] = {&b.x, &b.y, &b.z, &b.ux, &b.uy, &b.uz, &b.E, &b.w, &b.w2};
  for (R** a : br) { *a = (R*)p; p += NA_BANK_ARRAY; }
  uint64_t** bu[] = {&b.rng, &b.hid, &b.fam};
  for (uint64_t** a : bu) { *a = (uint64_t*)p; p += NA_BANK_ARRAY; }
  b.prob = nullptr;
  R** sr[] = {&s.x, &s.y, &s.z, &s.ux, &s.uy, &s.uz, &s.E, &s.w};
  for (R** a : sr) { *a = (R*)p; p += NA_SITE_ARRAY; }
  s.hist = (uint32_t*)p; p += na_round(NA_SITES * 4);
  s.dau = (uint32_t*)p; p += na_round(NA_SITES * 4);
  counts = (uint32_t*)p; p += na_round(NA_HIST * 4);
  offsets = (uint32_t*)p; p += na_round(NA_HIST * 4);
  blocks = (uint32_t*)p;
}

template <class R>
static int transport_noalloc_impl(abx_ctx* c, unsigned char* scratch, const abx_particle* bank_dev, size_t n,
                                  size_t site_cap, abx_site* sites_dev) {
  BankT<R> b;
  SiteT<R> s;
  uint32_t *counts, *offsets, *blocks;
  na_carve<R>(scratch, b, s, counts, offsets, blocks);
  k_bank_from_aos<R><<<grid_for(n), 256, 0, c->stream>>>(bank_dev, n, b);
  TransportArgs<R> A{};
  A.T = c->batch_scores ? c->batch_tables : c->D.T;
  A.T.tally_gen = c->tally_gen;
  A.bank = b;
  A.sites = s;
  A.site_cap = c->prob0.mode == ABX_MODE_K_EIGENVALUE ? std::min(site_cap, NA_SITES) : 0;
  A.hist_count = counts;
  A.sec = nullptr;
  A.sec_cap = 0;
  A.st = c->st;
  A.trace = nullptr;
  A.max_events = c->max_events;
  if constexpr (sizeof(R) == 4) launch_transport_f(A, kernel_code(c), c->all_iso, false, c->grid, c->block, c->stream);
  else launch_transport_d(A, kernel_code(c), false, c->grid, c->block, c->stream);
  CUDA_TRY(cudaGetLastError());
  unsigned nb = (unsigned)((n + SCAN_CHUNK - 1) / SCAN_CHUNK);
  if (nb == 0) nb = 1;
  k_scan_reduce<<<nb, SCAN_T, 0, c->stream>>>(counts, c->st, blocks);
  k_scan_blocks<<<1, 1024, 0, c->stream>>>(blocks, (int)nb);
  k_scan_apply<<<nb, SCAN_T, 0, c->stream>>>(counts, c->st, blocks, offsets);
  if (sites_dev && A.site_cap)
    k_sites_to_aos<R><<<grid_for(A.site_cap), 256, 0, c->stream>>>(s, c->st, offsets, b, sites_dev, A.site_cap);
  CUDA_TRY(cudaGetLastError());
  return ABX_OK;
}

extern "C" int abx_transport_noalloc(abx_ctx* c, const abx_particle* bank_dev, size_t n, double kcol, int converged,
                                     abx_site* sites_dev, size_t site_capacity, size_t* n_sites, abx_scores* scores) {
  if (!c || (!bank_dev && n)) return fail(ABX_ERR_INVALID, "bad arguments");
  if (!(kcol > 0)) return fail(ABX_ERR_INVALID, "kcol must be positive");
  if (c->nprob > 1)
    return fail(ABX_ERR_UNSUPPORTED, "a batch context transports through abx_run_fixed_source_batch only");
  if (n > NA_HIST)
    return fail(ABX_ERR_CAPACITY, "abx_transport_noalloc takes at most %zu histories per call (got %zu)", NA_HIST, n);
  if (site_capacity > NA_SITES)
    return fail(ABX_ERR_CAPACITY, "abx_transport_noalloc holds at most %zu fission sites per call (asked for %zu)",
                NA_SITES, site_capacity);
  if (c->prob0.mode == ABX_MODE_FIXED_SOURCE && c->fissile_any)
    return fail(ABX_ERR_UNSUPPORTED, "fixed-source fission secondaries need abx_transport");
  if (c->prob0.tracking == ABX_TRACK_CARTER || (c->prob0.branchless & ABX_BRANCHLESS_SPLITTING))
    return fail(ABX_ERR_UNSUPPORTED, "splitting puts particles on stacks: use abx_transport");
  if (cudaSetDevice(c->device) != cudaSuccess) return fail(ABX_ERR_CUDA, "cudaSetDevice failed");
  unsigned char* scratch = nullptr;
  int rc = scratch_address(c->device, &scratch);
  if (rc) return rc;
  const bool keig = c->prob0.mode == ABX_MODE_K_EIGENVALUE;
  k_step_begin<<<1, 1, 0, c->stream>>>(c->st, n, kcol, converged, 0);
  rc = mixed_of(c) ? transport_noalloc_impl<float>(c, scratch, bank_dev, n, site_capacity, sites_dev)
                   : transport_noalloc_impl<double>(c, scratch, bank_dev, n, site_capacity, sites_dev);
  if (rc) return rc;
  if ((rc = check_state(c)) != ABX_OK) return rc;
  const DevState& h = *c->st_host;
  size_t ns = keig ? (size_t)h.site_count : 0;
  if (n_sites) *n_sites = ns;
  if (scores) {
    scores->k_col = h.scores[0];
    scores->k_abs = h.scores[1];
    scores->k_trk = h.scores[2];
    scores->k_tot = h.scores[3];
    scores->leakage = h.scores[4];
    scores->mig_area = h.scores[5];
    scores->collisions = h.collisions;
    scores->flights = h.flights;
    scores->lost = h.lost;
  }
  if (keig && ns > site_capacity)
    return fail(ABX_ERR_CAPACITY, "fission bank capacity %zu < %zu sites", site_capacity, ns);
  return ABX_OK;
}

extern "C" int abx_set_l2_flush(abx_ctx* c, size_t bytes) {
  if (!c) return fail(ABX_ERR_INVALID, "bad arguments");
  cudaSetDevice(c->device);
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  if (c->flush) cudaFree(c->flush);
  c->flush = nullptr;
  c->flush_bytes = 0;
  if (!bytes) return ABX_OK;
  CUDA_TRY(cudaMalloc(&c->flush, bytes));
  c->flush_bytes = bytes;
  return ABX_OK;
}

extern "C" int abx_last_transport_ms(abx_ctx* c, double* ms) {
  if (!c || !ms) return fail(ABX_ERR_INVALID, "bad arguments");
  *ms = c->last_ms;
  return ABX_OK;
}

static int tally_record(abx_ctx* c, double mult, bool force) {
  size_t n = (size_t)c->P.tally_bins;
  if (!n) return ABX_OK;
  k_tally_record<<<grid_for(n), 256, 0, c->stream>>>(c->tally_gen, c->tally_avg, c->tally_var, n, mult,
                                                     force ? 1 : 0, (double)(c->tally_g + 1));
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  c->tally_g++;
  return ABX_OK;
}

extern "C" int abx_tally_record_generation(abx_ctx* c, double mult) {
  if (!c) return fail(ABX_ERR_INVALID, "null context");
  cudaSetDevice(c->device);
  return tally_record(c, mult, true);
}

extern "C" int abx_tally_clear_generation(abx_ctx* c) {
  if (!c) return fail(ABX_ERR_INVALID, "null context");
  cudaSetDevice(c->device);
  zero_d(c->tally_gen, (size_t)c->P.tally_bins, c->stream);
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  return ABX_OK;
}

extern "C" int abx_tally_size(abx_ctx* c, int id, size_t* n) {
  if (!c || !n || id < 0 || id >= (int)c->P.tallies.size()) return fail(ABX_ERR_INVALID, "bad tally id");
  const TallyT& t = c->P.tallies[id];
  *n = (size_t)t.ne * t.n[0] * t.n[1] * t.n[2];
  return ABX_OK;
}

extern "C" int abx_tally_read(abx_ctx* c, int id, double* gen, double* avg, double* var, int* generations) {
  size_t n;
  int rc = abx_tally_size(c, id, &n);
  if (rc) return rc;
  cudaSetDevice(c->device);
  const TallyT& t = c->P.tallies[id];
  if (gen) CUDA_TRY(cudaMemcpyAsync(gen, c->tally_gen + t.bin_off, n * 8, cudaMemcpyDeviceToHost, c->stream));
  if (avg) CUDA_TRY(cudaMemcpyAsync(avg, c->tally_avg + t.bin_off, n * 8, cudaMemcpyDeviceToHost, c->stream));
  if (var) CUDA_TRY(cudaMemcpyAsync(var, c->tally_var + t.bin_off, n * 8, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  if (generations) *generations = c->tally_g;
  return ABX_OK;
}

extern "C" int abx_tally_read_all(abx_ctx* c, double* avg, double* var, size_t capacity, size_t* n_bins) {
  if (!c || !n_bins) return fail(ABX_ERR_INVALID, "bad arguments");
  const size_t n = (size_t)c->P.tally_bins;
  *n_bins = n;
  if (!avg && !var) return ABX_OK;
  if (capacity < n) return fail(ABX_ERR_CAPACITY, "%zu tally bins, capacity %zu", n, capacity);
  cudaSetDevice(c->device);
  if (avg && n) CUDA_TRY(cudaMemcpyAsync(avg, c->tally_avg, n * 8, cudaMemcpyDeviceToHost, c->stream));
  if (var && n) CUDA_TRY(cudaMemcpyAsync(var, c->tally_var, n * 8, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  return ABX_OK;
}

// Entropy::add_point + calculate_entropy (src/entropy.cpp:32-93), Sign::Total,
// FP64, over n points of any record with r[3] and wgt.
template <class Pt> static double entropy_of(const ProbT& P, const Pt* s, size_t n) {
  if (!P.ent_on) return 0.;
  size_t nb = (size_t)P.ent_shape[0] * P.ent_shape[1] * P.ent_shape[2];
  std::vector<double> bins(nb, 0.);
  double tw = 0.;
  for (size_t i = 0; i < n; i++) {
    int nx = (int)std::floor((s[i].r[0] - P.ent_low[0]) / P.ent_d[0]);
    int ny = (int)std::floor((s[i].r[1] - P.ent_low[1]) / P.ent_d[1]);
    int nz = (int)std::floor((s[i].r[2] - P.ent_low[2]) / P.ent_d[2]);
    if (nx >= 0 && nx < P.ent_shape[0] && ny >= 0 && ny < P.ent_shape[1] && nz >= 0 && nz < P.ent_shape[2]) {
      tw += s[i].wgt;
      bins[(size_t)P.ent_shape[1] * P.ent_shape[2] * nx + (size_t)P.ent_shape[2] * ny + nz] += s[i].wgt;
    }
  }
  double sum = 0.;
  for (double b : bins) {
    double p = std::fabs(b) / tw;
    if (p > 1.0) {
    } else if (p != 0.) {
      sum -= p * std::log2(p);
    }
  }
  return sum;
}

extern "C" int abx_entropy(abx_ctx* c, const abx_site* s, size_t n, double* H) {
  if (!c || !H || (!s && n)) return fail(ABX_ERR_INVALID, "bad arguments");
  *H = entropy_of(c->prob0, s, n);
  return ABX_OK;
}

extern "C" int abx_set_trace(abx_ctx* c, uint32_t n_hist, size_t cap) {
  if (!c) return fail(ABX_ERR_INVALID, "null context");
  if (mixed_of(c) && n_hist && cap) return fail(ABX_ERR_UNSUPPORTED, "event traces are recorded in the FP64 mode");
  cudaSetDevice(c->device);
  if (c->trace) cudaFree(c->trace);
  c->trace = nullptr;
  c->trace_nhist = 0;
  c->trace_cap = 0;
  if (n_hist == 0 || cap == 0) return ABX_OK;
  CUDA_TRY(cudaMalloc(&c->trace, cap * sizeof(abx_trace_rec)));
  c->trace_nhist = n_hist;
  c->trace_cap = cap;
  return ABX_OK;
}

extern "C" int abx_get_trace(abx_ctx* c, abx_trace_rec* out, size_t cap, size_t* n_out) {
  if (!c || !n_out) return fail(ABX_ERR_INVALID, "bad arguments");
  cudaSetDevice(c->device);
  CUDA_TRY(cudaMemcpy(c->st_host, c->st, sizeof(DevState), cudaMemcpyDeviceToHost));
  size_t n = std::min<size_t>(c->st_host->trace_n, c->trace_cap);
  *n_out = n;
  if (!out || !c->trace) return ABX_OK;
  std::vector<abx_trace_rec> v(n);
  if (n) CUDA_TRY(cudaMemcpy(v.data(), c->trace, n * sizeof(abx_trace_rec), cudaMemcpyDeviceToHost));
  // records of one history were appended in program order: a stable sort on
  // the history index gives each history's event sequence
  std::stable_sort(v.begin(), v.end(), [](const abx_trace_rec& a, const abx_trace_rec& b) { return a.hist < b.hist; });
  size_t m = std::min(n, cap);
  if (m) memcpy(out, v.data(), m * sizeof(abx_trace_rec));
  return ABX_OK;
}

// PowerIterator::initialize + run (src/power_iterator.cpp:46-166, 305-473),
// device resident: the host only launches.
static int ensure_records(abx_ctx* c, int n) {
  if (c->hist_cap >= n) return ABX_OK;
  if (c->gen_rec) cudaFree(c->gen_rec);
  c->gen_rec = nullptr;
  CUDA_TRY(cudaMalloc(&c->gen_rec, (size_t)n * sizeof(abx_gen_record)));
  CUDA_TRY(cudaMemset(c->gen_rec, 0, (size_t)n * sizeof(abx_gen_record)));
  c->hist_cap = n;
  return ABX_OK;
}

// One power-iteration generation on the stream (src/power_iterator.cpp:
// 333-404): transport of bank `cur`, the site count scan, the next bank
// (bank order, weights, ids, streams, entropy bins) into bank 1-cur, the
// tally record and the end-of-generation statistics.  `device_book`: the
// tally record reads its active flag and count on the device (captured
// graphs); otherwise they come from the host (`conv`, `active`).
static int generation_step(abx_ctx* c, bool mixed, int cur, size_t cap, int nignored, cudaEvent_t ev_t0,
                           cudaEvent_t ev_t1, bool device_book, bool conv, int active) {
  int rc;
  // under stream capture (device_book) the records are external, so they
  // become event-record nodes of the graph
  const unsigned evf = device_book ? cudaEventRecordExternal : cudaEventRecordDefault;
  k_step_begin<<<1, 1, 0, c->stream>>>(c->st, 0, 0., 0, 1);
  CUDA_TRY(cudaEventRecordWithFlags(ev_t0, c->stream, evf));
  if ((rc = launch_transport(c, mixed, cur, cap)) != ABX_OK) return rc;
  CUDA_TRY(cudaEventRecordWithFlags(ev_t1, c->stream, evf));
  launch_scan(c, cap);
  if (mixed)
    k_next_bank<float><<<grid_for(cap), 256, 0, c->stream>>>(c->sf.s, c->st, c->offsets, c->bf[cur].b,
                                                             c->bf[1 - cur].b, c->D.T.probs, c->run, cap,
                                                             c->ent_bins, c->ent_total);
  else
    k_next_bank<double><<<grid_for(cap), 256, 0, c->stream>>>(c->sd.s, c->st, c->offsets, c->bd[cur].b,
                                                              c->bd[1 - cur].b, c->D.T.probs, c->run, cap,
                                                              c->ent_bins, c->ent_total);
  if (c->P.tally_bins) {
    if (device_book)
      k_tally_record_dev<<<grid_for((size_t)c->P.tally_bins), 256, 0, c->stream>>>(
          c->tally_gen, c->tally_avg, c->tally_var, (size_t)c->P.tally_bins, c->st, c->run);
    else
      k_tally_record<<<grid_for((size_t)c->P.tally_bins), 256, 0, c->stream>>>(
          c->tally_gen, c->tally_avg, c->tally_var, (size_t)c->P.tally_bins, 1.0, conv ? 1 : 0,
          (double)std::max(active, 1));
  }
  k_gen_end<<<1, 1024, 0, c->stream>>>(c->st, c->run, c->D.T.probs, c->gen_rec, c->hist_cap, c->ent_bins,
                                       c->ent_total, c->ent_nbins, cap, 1, nignored);
  CUDA_TRY(cudaGetLastError());
  return ABX_OK;
}

// Captures the generation step once per bank parity (the launches of a
// generation never change between generations: every per-generation value
// lives in device memory), so a generation is one graph launch.
static int ensure_gen_graphs(abx_ctx* c, bool mixed, size_t cap, int nignored) {
  // everything a captured launch points at; a reallocation forces a new capture
  std::vector<const void*> sig = {c->bd[0].b.x, c->bd[1].b.x, c->bf[0].b.x, c->bf[1].b.x, c->sd.s.x, c->sf.s.x,
                                  c->hist_count, c->offsets, c->block_sums, c->tally_gen, c->tally_avg,
                                  c->tally_var, c->ent_bins, c->ent_total, c->sec, c->st, c->run, c->gen_rec,
                                  c->D.T.probs, (const void*)(uintptr_t)c->grid, (const void*)(uintptr_t)c->block,
                                  (const void*)(uintptr_t)mixed, (const void*)(uintptr_t)c->hist_cap,
                                  (const void*)(uintptr_t)c->ent_nbins, c->pool,
                                  (const void*)(uintptr_t)use_pool(c)};
  if (c->gen_exec[0] && c->gen_cap == cap && c->gen_nignored == nignored && sig == c->gen_sig) return ABX_OK;
  for (auto& e : c->gen_exec)
    if (e) cudaGraphExecDestroy(e);
  for (auto& g : c->gen_graph)
    if (g) cudaGraphDestroy(g);
  c->gen_exec[0] = c->gen_exec[1] = nullptr;
  c->gen_graph[0] = c->gen_graph[1] = nullptr;
  for (auto& e : c->gen_ev_ph)
    if (!e) CUDA_TRY(cudaEventCreate(&e));
  for (int cur = 0; cur < 2; cur++) {
    cudaGraph_t graph = nullptr;
    CUDA_TRY(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    int rc = generation_step(c, mixed, cur, cap, nignored, c->gen_ev_ph[0], c->gen_ev_ph[1], true, false, 0);
    cudaError_t ce = cudaStreamEndCapture(c->stream, &graph);
    if (rc != ABX_OK) {
      if (graph) cudaGraphDestroy(graph);
      return rc;
    }
    if (ce != cudaSuccess) return fail(ABX_ERR_CUDA, "generation capture failed: %s", cudaGetErrorString(ce));
    // the two event-record nodes, to point them at each generation's events
    size_t nn = 0;
    cudaGraphGetNodes(graph, nullptr, &nn);
    std::vector<cudaGraphNode_t> nodes(nn);
    cudaGraphGetNodes(graph, nodes.data(), &nn);
    c->gen_ev_node[cur][0] = c->gen_ev_node[cur][1] = nullptr;
    for (cudaGraphNode_t n : nodes) {
      cudaGraphNodeType ty;
      cudaGraphNodeGetType(n, &ty);
      if (ty != cudaGraphNodeTypeEventRecord) continue;
      cudaEvent_t e;
      cudaGraphEventRecordNodeGetEvent(n, &e);
      if (e == c->gen_ev_ph[0]) c->gen_ev_node[cur][0] = n;
      if (e == c->gen_ev_ph[1]) c->gen_ev_node[cur][1] = n;
    }
    if (!c->gen_ev_node[cur][0] || !c->gen_ev_node[cur][1]) {
      cudaGraphDestroy(graph);
      return fail(ABX_ERR_CUDA, "generation graph: transport event nodes not found");
    }
    ce = cudaGraphInstantiate(&c->gen_exec[cur], graph, 0);
    c->gen_graph[cur] = graph;
    if (ce != cudaSuccess) return fail(ABX_ERR_CUDA, "generation graph instantiation failed: %s", cudaGetErrorString(ce));
  }
  c->gen_cap = cap;
  c->gen_nignored = nignored;
  c->gen_sig = sig;
  return ABX_OK;
}

extern "C" int abx_set_transport_kernel(abx_ctx* c, int kind) {
  if (!c) return fail(ABX_ERR_INVALID, "null context");
  if (kind != ABX_TRANSPORT_KERNEL_AUTO && kind != ABX_TRANSPORT_KERNEL_HISTORY && kind != ABX_TRANSPORT_KERNEL_POOL)
    return fail(ABX_ERR_INVALID, "unknown transport kernel %d", kind);
  if (kind == ABX_TRANSPORT_KERNEL_POOL && !pool_eligible(c))
    return fail(ABX_ERR_UNSUPPORTED,
                "the pooled kernel serves delta and surface tracking without secondary stacks or branchless collisions");
  cudaSetDevice(c->device);
  c->kernel_mode = kind;
  // the launch shape follows the kernel's occupancy
  int occ = occupancy_of(c, mixed_of(c), c->block);
  if (occ < 1) occ = 1;
  c->grid = c->nsm * occ;
  return ensure_sec(c, mixed_of(c));
}

extern "C" int abx_set_history_quantum(abx_ctx* c, uint32_t histories_per_warp) {
  if (!c) return fail(ABX_ERR_INVALID, "null context");
  c->warp_quota = histories_per_warp;
  return ABX_OK;
}

extern "C" int abx_get_transport_kernel(abx_ctx* c, int* kind) {
  if (!c || !kind) return fail(ABX_ERR_INVALID, "bad arguments");
  *kind = use_pool(c) ? ABX_TRANSPORT_KERNEL_POOL : ABX_TRANSPORT_KERNEL_HISTORY;
  return ABX_OK;
}

extern "C" int abx_set_graphs(abx_ctx* c, int enabled) {
  if (!c) return fail(ABX_ERR_INVALID, "bad arguments");
  c->use_graphs = enabled != 0;
  return ABX_OK;
}

// The reference's global stream (settings::rng, a pcg32) on the host, as a
// uniform random bit generator for libstdc++'s std::shuffle and
// uniform_real_distribution, the calls BranchlessPowerIterator makes.
struct GlobalStream {
  using result_type = uint32_t;
  uint64_t state;
  static constexpr result_type min() { return 0u; }
  static constexpr result_type max() { return 0xffffffffu; }
  result_type operator()() {
    const uint64_t old = state;
    state = old * PCG_MULT + PCG_INC;
    const uint32_t rot = (uint32_t)(old >> 59);
    const uint32_t xs = (uint32_t)(((old >> 18) ^ old) >> 27);
    return (xs >> rot) | (xs << ((32u - rot) & 31u));
  }
};

// The host half of a branchless generation with combing, after the device
// wrote the next bank (unnormalised, in the reference's order) into bank
// `nxt`: BranchlessPowerIterator::normalize_weights and comb_particles
// (src/branchless_power_iterator.cpp:541-650), then the bank rebuilt as
// PowerIterator does (new history ids in order, streams seeded at them,
// src/branchless_power_iterator.cpp:415-423) and the entropy of the combed
// bank (compute_post_cancellation_entropy) put in the generation's record.
static int comb_generation(abx_ctx* c, bool mixed, int nxt, int g, GlobalStream& gs, size_t cap) {
  int rc;
  if ((rc = check_state(c)) != ABX_OK) return rc;
  const size_t ns = (size_t)c->st_host->n_hist;
  std::vector<abx_particle> bank(ns);
  {
    const int rc_in = ensure_aos_in(c, std::max(ns, cap));
    if (rc_in != ABX_OK) return rc_in;
  }
  if (ns) {
    if (mixed) k_bank_to_aos<float><<<grid_for(ns), 256, 0, c->stream>>>(c->bf[nxt].b, ns, c->aos_in);
    else k_bank_to_aos<double><<<grid_for(ns), 256, 0, c->stream>>>(c->bd[nxt].b, ns, c->aos_in);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaMemcpyAsync(bank.data(), c->aos_in, ns * sizeof(abx_particle), cudaMemcpyDeviceToHost, c->stream));
  }
  RunAcc ra;
  CUDA_TRY(cudaMemcpyAsync(&ra, c->run, sizeof ra, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  // normalize_weights
  double W_pos = 0., W_neg = 0.;
  for (const abx_particle& p : bank) {
    if (p.wgt > 0.) W_pos += p.wgt;
    else W_neg -= p.wgt;
  }
  const double wpp = c->prob0.nparticles / (W_pos - W_neg);
  for (abx_particle& p : bank) p.wgt *= wpp;
  // comb_particles: only positive weights occur with branchless collisions
  std::vector<abx_particle> pos;
  pos.reserve(ns);
  double Wpos = 0.;
  for (const abx_particle& p : bank) {
    if (!(p.wgt > 0.)) return fail(ABX_ERR_UNSUPPORTED, "combing a bank with non-positive weights");
    Wpos += p.wgt;
    pos.push_back(p);
  }
  const size_t Npos = (size_t)std::ceil(Wpos);
  std::shuffle(pos.begin(), pos.end(), gs);
  std::uniform_real_distribution<double> unit(0., 1.);  // RNG::rand (include/utils/rng.hpp:41)
  const double avg_pos = Wpos / (double)Npos;
  double comb_pos = unit(gs) * avg_pos;
  double current = 0.;
  std::vector<abx_particle> next;
  next.reserve(Npos + 4);
  for (const abx_particle& p : pos) {
    current += p.wgt;
    while (comb_pos < current) {
      next.push_back(p);
      next.back().wgt = avg_pos;
      comb_pos += avg_pos;
    }
  }
  (void)unit(gs);  // the comb position of the (empty) negative part
  std::shuffle(next.begin(), next.end(), gs);
  const size_t m = next.size();
  if (m == 0) return fail(ABX_ERR_NO_FISSION, "No fission neutrons were produced.");
  if (m > cap) return fail(ABX_ERR_CAPACITY, "combed bank of %zu particles, capacity %zu", m, cap);
  // the next generation's particles: history ids from the global counter
  const uint64_t base = ra.global_hist - ns;
  for (size_t i = 0; i < m; i++) {
    abx_particle& p = next[i];
    p.wgt2 = 0.;
    p.history_id = base + i;
    p.rng_state = pcg_advance(pcg_seeded(c->prob0.seed), c->prob0.stride * p.history_id);
  }
  ra.global_hist = base + m;
  const double H = entropy_of(c->prob0, next.data(), m);
  CUDA_TRY(cudaMemcpyAsync(c->aos_in, next.data(), m * sizeof(abx_particle), cudaMemcpyHostToDevice, c->stream));
  if (mixed) k_bank_from_aos<float><<<grid_for(m), 256, 0, c->stream>>>(c->aos_in, m, c->bf[nxt].b);
  else k_bank_from_aos<double><<<grid_for(m), 256, 0, c->stream>>>(c->aos_in, m, c->bd[nxt].b);
  CUDA_TRY(cudaGetLastError());
  const unsigned long long n_hist = m;
  CUDA_TRY(cudaMemcpyAsync((char*)c->st + offsetof(DevState, n_hist), &n_hist, sizeof n_hist,
                           cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(cudaMemcpyAsync((char*)c->run + offsetof(RunAcc, global_hist), &ra.global_hist,
                           sizeof ra.global_hist, cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(cudaMemcpyAsync((char*)(c->gen_rec + (g - 1)) + offsetof(abx_gen_record, entropy), &H, sizeof H,
                           cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(cudaStreamSynchronize(c->stream));  // host vectors are pageable and go out of scope
  return ABX_OK;
}

// PowerIterator::load_source_from_file (src/power_iterator.cpp:60-132): the
// stored particles become histories 0..n-1 (family = history id), each
// stream seeded at its id.  The caller has already set nparticles to the
// rounded total weight on the host; it is copied to the device here (and
// stays so for the context).
static int load_restart_bank(abx_ctx* c, bool mixed, size_t cap, size_t* n_out) {
  const size_t n = c->restart_src.size() / 9;
  if (n > cap) return fail(ABX_ERR_CAPACITY, "source bank of %zu particles, capacity %zu", n, cap);
  std::vector<abx_particle> bank(n);
  for (size_t i = 0; i < n; i++) {
    const double* q = c->restart_src.data() + 9 * i;
    abx_particle& p = bank[i];
    for (int a = 0; a < 3; a++) { p.r[a] = q[a]; p.u[a] = q[3 + a]; }
    p.E = q[6];
    p.wgt = q[7];
    p.wgt2 = q[8];
    p.history_id = i;
    p.family_id = i;
    p.rng_state = pcg_advance(pcg_seeded(c->prob0.seed), c->prob0.stride * (uint64_t)i);
  }
  // the run's nparticles (set from the bank's total weight) on the device
  CUDA_TRY(cudaMemcpyAsync((void*)c->D.T.probs, &c->P.probs[0], sizeof(ProbT), cudaMemcpyHostToDevice, c->stream));
  {
    const int rc_in = ensure_aos_in(c, n);
    if (rc_in != ABX_OK) return rc_in;
  }
  CUDA_TRY(cudaMemcpyAsync(c->aos_in, bank.data(), n * sizeof(abx_particle), cudaMemcpyHostToDevice, c->stream));
  if (mixed) k_bank_from_aos<float><<<grid_for(n), 256, 0, c->stream>>>(c->aos_in, n, c->bf[0].b);
  else k_bank_from_aos<double><<<grid_for(n), 256, 0, c->stream>>>(c->aos_in, n, c->bd[0].b);
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaStreamSynchronize(c->stream));  // `bank` is pageable host memory
  *n_out = n;
  return ABX_OK;
}

extern "C" int abx_set_source_bank(abx_ctx* c, const double* source, size_t n) {
  if (!c || (!source && n)) return fail(ABX_ERR_INVALID, "bad arguments");
  if (c->prob0.mode != ABX_MODE_K_EIGENVALUE) return fail(ABX_ERR_INVALID, "problem is not k-eigenvalue");
  if (n == 0) {
    c->restart_src.clear();
    return ABX_OK;
  }
  const double* eb = c->P.eb_d.data() + c->prob0.eb_off;
  for (size_t i = 0; i < n; i++) {
    const double* q = source + 9 * i;
    for (int a = 0; a < 9; a++)
      if (!std::isfinite(q[a])) return fail(ABX_ERR_INVALID, "source particle %zu: value %d is not finite", i, a);
    if (!(q[6] >= eb[0] && q[6] <= eb[c->prob0.G]))
      return fail(ABX_ERR_INVALID, "source particle %zu: energy outside the group structure", i);
  }
  c->restart_src.assign(source, source + 9 * n);
  return ABX_OK;
}

extern "C" int abx_run_power_iteration_ex(abx_ctx* c, int ngen, int nignored, abx_run_stats* stats,
                                          abx_gen_record* per_gen) {
  if (!c || ngen <= 0 || nignored < 0) return fail(ABX_ERR_INVALID, "bad arguments");
  if (c->prob0.mode != ABX_MODE_K_EIGENVALUE) return fail(ABX_ERR_INVALID, "problem is not k-eigenvalue");
  cudaSetDevice(c->device);
  const bool mixed = mixed_of(c);
  int rc;
  const size_t n_restart = c->restart_src.size() / 9;
  if (n_restart) {
    // settings::nparticles and the tallies' total weight become the source
    // bank's rounded total weight (src/power_iterator.cpp:124-131)
    double tot_wgt = 0.;
    for (size_t i = 0; i < n_restart; i++) tot_wgt += c->restart_src[9 * i + 7];
    const double np = std::round(tot_wgt);
    if (!(np > 0.)) return fail(ABX_ERR_INVALID, "source bank has no positive total weight");
    for (ProbT* q : {&c->prob0, &c->P.probs[0]}) {
      q->nparticles = np;
      q->inv_np = 1. / np;
    }
  }
  const size_t N = (size_t)c->prob0.nparticles;
  const size_t cap = 3 * std::max(N, n_restart) + 4096;
  if ((rc = ensure_banks(c, cap, mixed, false)) != ABX_OK) return rc;
  if ((rc = ensure_sites(c, cap, mixed)) != ABX_OK) return rc;
  if ((rc = ensure_records(c, ngen)) != ABX_OK) return rc;
  auto t0 = std::chrono::steady_clock::now();
  CUDA_TRY(cudaMemsetAsync(c->st, 0, sizeof(DevState), c->stream));
  CUDA_TRY(cudaMemsetAsync(c->run, 0, sizeof(RunAcc), c->stream));
  zero_d(c->tally_gen, (size_t)c->P.tally_bins, c->stream);
  zero_d(c->tally_avg, (size_t)c->P.tally_bins, c->stream);
  zero_d(c->tally_var, (size_t)c->P.tally_bins, c->stream);
  c->tally_g = 0;
  size_t N0 = N;  // histories of the first generation
  if (c->restart_src.empty()) {
    // initial source bank, histories 0..N-1 (src/power_iterator.cpp:135-166)
    SourceArgs S{};
    S.T = c->D.T;
    S.prob = 0;
    S.first_hid = 0;
    S.n = N;
    sample_bank0(c, S, mixed, false);
  } else if ((rc = load_restart_bank(c, mixed, cap, &N0)) != ABX_OK) {
    return rc;
  }
  {
    // RunAcc.global_hist = N0; DevState: n_hist = N0, kcol = 1, converged
    RunAcc ra{};
    ra.global_hist = N0;
    CUDA_TRY(cudaMemcpyAsync(c->run, &ra, sizeof ra, cudaMemcpyHostToDevice, c->stream));
  }
  if ((rc = check_state(c)) != ABX_OK) return rc;
  k_step_begin<<<1, 1, 0, c->stream>>>(c->st, N0, 1.0, nignored == 0 ? 1 : 0, 0);
  if ((rc = ensure_sec(c, mixed)) != ABX_OK) return rc;
  // the generation events come from the context's pool and live as long as
  // the context: a captured graph's event nodes keep pointing at them
  while (c->ev_pool.size() < 4 * (size_t)ngen) {
    cudaEvent_t e;
    CUDA_TRY(cudaEventCreate(&e));
    c->ev_pool.push_back(e);
  }
  const std::vector<cudaEvent_t> evs(c->ev_pool.begin(), c->ev_pool.begin() + 4 * (size_t)ngen);
  int cur = 0;
  int active_tally = 0;
  // branchless combing: a host step after every generation, so no graphs;
  // its stream starts as a default-constructed pcg32 after the deck's draws
  const bool combing = (c->prob0.branchless & ABX_BRANCHLESS_COMBING) != 0;
  GlobalStream gs{pcg_advance(pcg_seeded(0xcafef00dd15ea5e5ULL), (uint64_t)std::max(0, c->prob0.global_rng_skip))};
  const bool graphs = c->use_graphs && c->trace_nhist == 0 && !combing;
  if (graphs && (rc = ensure_gen_graphs(c, mixed, cap, nignored)) != ABX_OK) return rc;
  for (int g = 1; g <= ngen; g++) {
    if (c->flush_bytes) CUDA_TRY(cudaMemsetAsync(c->flush, g & 0xff, c->flush_bytes, c->stream));
    cudaEventRecord(evs[4 * (g - 1)], c->stream);
    bool conv = (nignored == 0) || (g > nignored);
    if (conv) active_tally++;
    if (graphs) {
      // the captured step, its transport bracketed by this generation's events
      CUDA_TRY(cudaGraphExecEventRecordNodeSetEvent(c->gen_exec[cur], c->gen_ev_node[cur][0], evs[4 * (g - 1) + 1]));
      CUDA_TRY(cudaGraphExecEventRecordNodeSetEvent(c->gen_exec[cur], c->gen_ev_node[cur][1], evs[4 * (g - 1) + 2]));
      CUDA_TRY(cudaGraphLaunch(c->gen_exec[cur], c->stream));
    } else {
      if ((rc = generation_step(c, mixed, cur, cap, nignored, evs[4 * (g - 1) + 1], evs[4 * (g - 1) + 2], false,
                                conv, active_tally)) != ABX_OK)
        break;
    }
    cudaEventRecord(evs[4 * (g - 1) + 3], c->stream);
    CUDA_TRY(cudaGetLastError());
    cur = 1 - cur;
    if (combing && (rc = comb_generation(c, mixed, cur, g, gs, cap)) != ABX_OK) break;
    if ((g & 7) == 0 || g == ngen) {
      if ((rc = check_state(c)) != ABX_OK) break;
    }
  }
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  c->tally_g = active_tally;
  if (rc == ABX_OK) {
    // the last check_state read DevState after the final generation end
    c->pi_bank = cur;
    c->pi_n = (size_t)c->st_host->n_hist;
    c->pi_kcol = c->st_host->kcol;
  }
  double tms = 0.;
  std::vector<abx_gen_record> recs(ngen);
  if (rc == ABX_OK) CUDA_TRY(cudaMemcpy(recs.data(), c->gen_rec, ngen * sizeof(abx_gen_record), cudaMemcpyDeviceToHost));
  for (int g = 0; g < ngen && rc == ABX_OK; g++) {
    float ms = 0.f, ts = 0.f;
    cudaEventElapsedTime(&ms, evs[4 * g], evs[4 * g + 3]);
    cudaEventElapsedTime(&ts, evs[4 * g + 1], evs[4 * g + 2]);
    recs[g].step_ms = ms;
    recs[g].transport_ms = ts;
    tms += ts;
  }
  if (rc) return rc;
  auto t1 = std::chrono::steady_clock::now();
  RunAcc ra;
  CUDA_TRY(cudaMemcpy(&ra, c->run, sizeof ra, cudaMemcpyDeviceToHost));
  if (per_gen) memcpy(per_gen, recs.data(), ngen * sizeof(abx_gen_record));
  if (stats) {
    memset(stats, 0, sizeof *stats);
    stats->generations = ra.gen;
    stats->active = ra.active;
    stats->kcol_avg = ra.kcol_avg;
    stats->kcol_std = ra.active ? std::sqrt(ra.kcol_var / ra.active) : 0.;
    stats->ktrk_avg = ra.ktrk_avg;
    stats->ktrk_std = ra.active ? std::sqrt(ra.ktrk_var / ra.active) : 0.;
    stats->leak_avg = ra.leak_avg;
    stats->leak_std = ra.active ? std::sqrt(ra.leak_var / ra.active) : 0.;
    stats->mig_avg = ra.mig_avg;
    stats->mig_std = ra.active ? std::sqrt(ra.mig_var / ra.active) : 0.;
    stats->collisions = ra.total_coll;
    stats->flights = ra.total_flights;
    stats->histories = ra.total_hist;
    stats->transport_ms = tms;
    stats->total_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
  }
  return ABX_OK;
}

extern "C" int abx_read_source_bank(abx_ctx* c, abx_particle* out, size_t capacity, size_t* n_out,
                                    double* kcol_out) {
  if (!c || !n_out) return fail(ABX_ERR_INVALID, "bad arguments");
  if (c->pi_bank < 0) return fail(ABX_ERR_INVALID, "no source bank: no power iteration since the banks were last written");
  const size_t n = c->pi_n;
  *n_out = n;
  if (kcol_out) *kcol_out = c->pi_kcol;
  if (!out || n == 0) return ABX_OK;
  if (capacity < n) return fail(ABX_ERR_CAPACITY, "source bank of %zu particles, capacity %zu", n, capacity);
  cudaSetDevice(c->device);
  {
    const int rc_in = ensure_aos_in(c, n);
    if (rc_in != ABX_OK) return rc_in;
  }
  if (mixed_of(c)) k_bank_to_aos<float><<<grid_for(n), 256, 0, c->stream>>>(c->bf[c->pi_bank].b, n, c->aos_in);
  else k_bank_to_aos<double><<<grid_for(n), 256, 0, c->stream>>>(c->bd[c->pi_bank].b, n, c->aos_in);
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaMemcpyAsync(out, c->aos_in, n * sizeof(abx_particle), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  return ABX_OK;
}

extern "C" int abx_run_power_iteration(abx_ctx* c, int ngen, int nignored, abx_run_stats* stats, double* kcol_gen,
                                       double* ent_gen) {
  if (ngen <= 0) return fail(ABX_ERR_INVALID, "bad arguments");
  std::vector<abx_gen_record> r(ngen);
  int rc = abx_run_power_iteration_ex(c, ngen, nignored, stats, r.data());
  if (rc) return rc;
  for (int g = 0; g < ngen; g++) {
    if (kcol_gen) kcol_gen[g] = r[g].kcol;
    if (ent_gen) ent_gen[g] = r[g].entropy;
  }
  return ABX_OK;
}

// FixedSource::run (src/fixed_source.cpp:81-173): batches of fresh source
// histories; fission makes in-history secondaries.
extern "C" int abx_run_fixed_source(abx_ctx* c, int nbatches, uint64_t npart, abx_run_stats* stats) {
  if (!c || nbatches <= 0 || npart == 0) return fail(ABX_ERR_INVALID, "bad arguments");
  if (c->prob0.mode != ABX_MODE_FIXED_SOURCE) return fail(ABX_ERR_INVALID, "problem is not fixed-source");
  cudaSetDevice(c->device);
  const bool mixed = mixed_of(c);
  int rc;
  if ((rc = ensure_banks(c, npart, mixed, false)) != ABX_OK) return rc;
  if ((rc = ensure_sites(c, 1, mixed)) != ABX_OK) return rc;
  if ((rc = ensure_sec(c, mixed)) != ABX_OK) return rc;
  if ((rc = ensure_records(c, nbatches)) != ABX_OK) return rc;
  auto t0 = std::chrono::steady_clock::now();
  CUDA_TRY(cudaMemsetAsync(c->st, 0, sizeof(DevState), c->stream));
  CUDA_TRY(cudaMemsetAsync(c->run, 0, sizeof(RunAcc), c->stream));
  zero_d(c->tally_gen, (size_t)c->P.tally_bins, c->stream);
  zero_d(c->tally_avg, (size_t)c->P.tally_bins, c->stream);
  zero_d(c->tally_var, (size_t)c->P.tally_bins, c->stream);
  c->tally_g = 0;
  std::vector<cudaEvent_t> evs(2 * (size_t)nbatches);
  for (auto& e : evs) cudaEventCreate(&e);
  uint64_t hc = 0;
  for (int g = 1; g <= nbatches; g++) {
    SourceArgs S{};
    S.T = c->D.T;
    S.prob = 0;
    S.first_hid = hc;
    S.n = npart;
    sample_bank0(c, S, mixed, false);
    hc += npart;
    k_step_begin<<<1, 1, 0, c->stream>>>(c->st, npart, 1.0, 1, 0);
    cudaEventRecord(evs[2 * (g - 1)], c->stream);
    if ((rc = launch_transport(c, mixed, 0, 0)) != ABX_OK) break;
    cudaEventRecord(evs[2 * (g - 1) + 1], c->stream);
    if (c->P.tally_bins)
      k_tally_record<<<grid_for((size_t)c->P.tally_bins), 256, 0, c->stream>>>(
          c->tally_gen, c->tally_avg, c->tally_var, (size_t)c->P.tally_bins, 1.0, 1, (double)g);
    k_gen_end<<<1, 1024, 0, c->stream>>>(c->st, c->run, c->D.T.probs, c->gen_rec, c->hist_cap, c->ent_bins,
                                         nullptr, 0, npart, 0, 0);
    CUDA_TRY(cudaGetLastError());
    if ((rc = check_state(c)) != ABX_OK) break;
  }
  double tms = 0.;
  for (int g = 0; g < nbatches && rc == ABX_OK; g++) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, evs[2 * g], evs[2 * g + 1]);
    tms += ms;
  }
  for (auto& e : evs) cudaEventDestroy(e);
  if (rc) return rc;
  c->tally_g = nbatches;
  auto t1 = std::chrono::steady_clock::now();
  RunAcc ra;
  CUDA_TRY(cudaMemcpy(&ra, c->run, sizeof ra, cudaMemcpyDeviceToHost));
  if (stats) {
    memset(stats, 0, sizeof *stats);
    stats->generations = ra.gen;
    stats->active = ra.active;
    stats->leak_avg = ra.leak_avg;
    stats->leak_std = ra.active ? std::sqrt(ra.leak_var / ra.active) : 0.;
    stats->mig_avg = ra.mig_avg;
    stats->mig_std = ra.active ? std::sqrt(ra.mig_var / ra.active) : 0.;
    stats->collisions = ra.total_coll;
    stats->flights = ra.total_flights;
    stats->histories = ra.total_hist;
    stats->transport_ms = tms;
    stats->total_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
  }
  return ABX_OK;
}

// abx_batch_replace in two halves, for callers that derive the next batch's
// tables on the host while the GPU still runs the current batch: the host
// half touches no device state; the device half uploads into the context.
namespace abx {
struct PreparedBatch {
  Pools P;
  int n = 0, tracking = 0, prec = 0;
};

void* batch_prepare(const abx_problem* problems, int n_problems, int* rc_out) {
  int rc = ABX_OK;
  PreparedBatch* b = nullptr;
  if (!problems || n_problems <= 0) {
    rc = fail(ABX_ERR_INVALID, "bad arguments");
  } else {
    b = new PreparedBatch();
    b->n = n_problems;
    b->tracking = problems[0].settings.tracking;
    b->prec = problems[0].settings.precision;
    // the pools sized up front: no reallocation while appending
    size_t nxs = 0, ncdf = 0, nmat = 0, ndg = 0, neb = 0, nsurf = 0, ncell = 0, nrpn = 0, nuniv = 0, nlist = 0,
           nlat = 0, ntal = 0, nteb = 0, nsrc = 0;
    auto cnt = [](int v) { return (size_t)std::max(0, v); };
    for (int i = 0; i < n_problems; i++) {
      const abx_problem& q = problems[i];
      const size_t G = cnt(q.settings.ngroups), nm = cnt(q.n_materials);
      nxs += nm * XS_ROWS * G;
      ncdf += nm * 2 * G * G;
      nmat += nm;
      if (q.materials)
        for (size_t m = 0; m < nm; m++) ndg += (size_t)std::max(1, q.materials[m].n_delayed);
      neb += G + 1;
      nsurf += cnt(q.n_surfaces);
      ncell += cnt(q.n_cells);
      nrpn += 2 * cnt(q.n_rpn);  // cell regions and the boundary half-spaces of each universe
      nuniv += cnt(q.n_universes);
      nlist += cnt(q.n_cell_lists);
      nlat += cnt(q.n_lattice_elems);
      ntal += cnt(q.n_tallies);
      nteb += cnt(q.n_tally_ebounds);
      nsrc += cnt(q.n_sources);
    }
    Pools& P = b->P;
    P.xs_d.reserve(nxs);
    P.cdf_d.reserve(ncdf);
    P.mats.reserve(nmat);
    P.dg_d.reserve(ndg);
    P.eb_d.reserve(neb);
    P.maj_d.reserve(2 * neb);
    P.probs.reserve(n_problems);
    P.surf_d.reserve(nsurf);
    P.cells.reserve(ncell);
    P.rpn.reserve(nrpn);
    P.univ.reserve(nuniv);
    P.cell_lists.reserve(nlist);
    P.lat_elems.reserve(nlat);
    P.tallies.reserve(ntal);
    P.tally_eb.reserve(nteb);
    P.sources.reserve(nsrc);
    P.src_cdf.reserve(nsrc + n_problems);
    for (int i = 0; i < n_problems && rc == ABX_OK; i++) {
      const abx_settings& s = problems[i].settings;
      if (s.mode != ABX_MODE_FIXED_SOURCE || s.tracking != b->tracking || s.precision != b->prec)
        rc = fail(ABX_ERR_UNSUPPORTED,
                  "problem %d: a batch holds fixed-source problems of one tracking mode and precision", i);
      else
        rc = append_problem(b->P, &problems[i]);
    }
    if (rc) {
      delete b;
      b = nullptr;
    }
  }
  if (rc_out) *rc_out = rc;
  return b;
}

void batch_discard(void* prepared) { delete static_cast<PreparedBatch*>(prepared); }

static int install_prepared(abx_ctx* c, PreparedBatch* b);

int batch_install(abx_ctx* c, void* prepared) {
  PreparedBatch* b = static_cast<PreparedBatch*>(prepared);
  int rc = (c && b) ? install_prepared(c, b) : fail(ABX_ERR_INVALID, "bad arguments");
  delete b;
  return rc;
}
}  // namespace abx

extern "C" int abx_batch_replace(abx_ctx* c, const abx_problem* problems, int n_problems) {
  if (!c) return fail(ABX_ERR_INVALID, "bad arguments");
  int rc;
  void* b = abx::batch_prepare(problems, n_problems, &rc);
  if (rc) return rc;  // the context keeps its previous problems
  return abx::batch_install(c, b);
}

static int abx::install_prepared(abx_ctx* c, PreparedBatch* b) {
  if (b->tracking != c->prob0.tracking || b->prec != c->prec)
    return fail(ABX_ERR_UNSUPPORTED, "the batch's tracking mode or precision differs from the context's");
  const int n_problems = b->n;
  cudaSetDevice(c->device);
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  c->P = std::move(b->P);
  c->nprob = n_problems;
  c->prob0 = c->P.probs[0];
  c->fissile_any = false;
  for (const MatT& m : c->P.mats) c->fissile_any |= m.fissile != 0;
  c->all_iso = true;
  for (const MatT& m : c->P.mats) c->all_iso = c->all_iso && m.iso != 0;
  int rc = upload(c->P, c->D);
  if (rc) return rc;
  if (after_host_copies(c->stream) != ABX_OK) return fail(ABX_ERR_CUDA, "stream ordering of the table upload failed");
  const size_t R = (size_t)std::max<int64_t>(c->P.tally_bins, 1);
  if (c->tally_rv_cap < R) {
    cudaFree(c->tally_avg);
    cudaFree(c->tally_var);
    c->tally_avg = c->tally_var = nullptr;
    c->tally_rv_cap = 0;
    CUDA_TRY(cudaMalloc(&c->tally_avg, headroom(R) * 8));
    CUDA_TRY(cudaMalloc(&c->tally_var, headroom(R) * 8));
    c->tally_rv_cap = headroom(R);
  }
  if (c->tally_gen_cap < R) {
    cudaFree(c->tally_gen);
    c->tally_gen = nullptr;
    c->tally_gen_cap = 0;
    CUDA_TRY(cudaMalloc(&c->tally_gen, headroom(R) * 8));
    c->tally_gen_cap = headroom(R);
  }
  zero_d(c->tally_gen, R, c->stream);
  zero_d(c->tally_avg, R, c->stream);
  zero_d(c->tally_var, R, c->stream);
  c->tally_g = 0;
  c->vb_nb = 0;
  CUDA_TRY(cudaGetLastError());
  return ABX_OK;
}

// Every batch of every problem of a batch context in one transport launch.
// Batch b of problem p runs as virtual problem v = p*nb + b: a copy of the
// problem's settings whose tallies are the b-th copy of the problem's tally
// bins, so the per-batch bookkeeping of FixedSource::run
// (src/fixed_source.cpp:105-150) is applied afterwards, batch by batch, for
// every problem at once.
static int ensure_virtual(abx_ctx* c, int nb) {
  const int np = c->nprob;
  const size_t R = (size_t)c->P.tally_bins;
  const int RT = (int)c->P.tallies.size();
  if (c->vb_nb == nb) return ABX_OK;
  std::vector<ProbT> vp((size_t)np * nb);
  std::vector<TallyT> vt((size_t)RT * nb);
  for (int p = 0; p < np; p++)
    for (int b = 0; b < nb; b++) {
      ProbT q = c->P.probs[p];
      q.tally_first = b * RT + q.tally_first;
      vp[(size_t)p * nb + b] = q;
    }
  for (int b = 0; b < nb; b++)
    for (int t = 0; t < RT; t++) {
      TallyT u = c->P.tallies[t];
      u.bin_off += (int64_t)b * (int64_t)R;
      vt[(size_t)b * RT + t] = u;
    }
  c->vb_nb = 0;
  auto grow = [&](void** ptr, size_t* cap, size_t bytes) -> int {
    if (*cap >= bytes) return ABX_OK;
    if (*ptr) cudaFree(*ptr);
    *ptr = nullptr;
    *cap = 0;
    CUDA_TRY(cudaMalloc(ptr, headroom(bytes)));
    *cap = headroom(bytes);
    return ABX_OK;
  };
  const size_t nv = (size_t)np * nb;
  int rc;
  if ((rc = grow((void**)&c->vprobs, &c->vcap[0], vp.size() * sizeof(ProbT))) ||
      (rc = grow((void**)&c->vtallies, &c->vcap[1], std::max<size_t>(vt.size(), 1) * sizeof(TallyT))) ||
      (rc = grow((void**)&c->pscore, &c->vcap[2], nv * ABX_PSCORES * sizeof(double))) ||
      (rc = grow((void**)&c->pcount, &c->vcap[3], nv * ABX_PCOUNTS * sizeof(unsigned long long))) ||
      (rc = grow((void**)&c->seg_off, &c->vcap[4], (nv + 1) * sizeof(uint64_t))) ||
      (rc = grow((void**)&c->seg_prob, &c->vcap[5], nv * sizeof(int32_t))) ||
      (rc = grow((void**)&c->seg_hid0, &c->vcap[6], nv * sizeof(uint64_t))) ||
      (rc = grow((void**)&c->prun, &c->vcap[7], (size_t)np * sizeof(ProbRun))))
    return rc;
  CUDA_TRY(cudaMemcpy(c->vprobs, vp.data(), vp.size() * sizeof(ProbT), cudaMemcpyHostToDevice));
  if (!vt.empty()) CUDA_TRY(cudaMemcpy(c->vtallies, vt.data(), vt.size() * sizeof(TallyT), cudaMemcpyHostToDevice));
  const size_t need = std::max<size_t>(R * (size_t)nb, 1);
  if (c->tally_gen_cap < need) {
    if (c->tally_gen) cudaFree(c->tally_gen);
    c->tally_gen = nullptr;
    c->tally_gen_cap = 0;
    CUDA_TRY(cudaMalloc(&c->tally_gen, headroom(need) * 8));
    c->tally_gen_cap = headroom(need);
  }
  // segments: virtual problem v = p*nb + b holds histories b*n_p .. (b+1)*n_p-1
  std::vector<uint64_t> off(nv + 1), hid0(nv);
  std::vector<int32_t> vid(nv);
  uint64_t total = 0;
  for (int p = 0; p < np; p++) {
    const uint64_t n_p = (uint64_t)c->P.probs[p].nparticles;
    for (int b = 0; b < nb; b++) {
      const size_t v = (size_t)p * nb + b;
      off[v] = total;
      hid0[v] = (uint64_t)b * n_p;  // src/fixed_source.cpp:152-155
      vid[v] = (int32_t)v;
      total += n_p;
    }
  }
  off[nv] = total;
  CUDA_TRY(cudaMemcpy(c->seg_off, off.data(), off.size() * sizeof(uint64_t), cudaMemcpyHostToDevice));
  CUDA_TRY(cudaMemcpy(c->seg_prob, vid.data(), vid.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
  CUDA_TRY(cudaMemcpy(c->seg_hid0, hid0.data(), hid0.size() * sizeof(uint64_t), cudaMemcpyHostToDevice));
  c->vb_total = total;
  c->vb_nb = nb;
  return ABX_OK;
}

extern "C" int abx_run_fixed_source_batch(abx_ctx* c, int nbatches, abx_problem_result* results,
                                          abx_run_stats* stats) {
  if (!c || nbatches <= 0) return fail(ABX_ERR_INVALID, "bad arguments");
  if (c->prob0.mode != ABX_MODE_FIXED_SOURCE) return fail(ABX_ERR_INVALID, "problem is not fixed-source");
  cudaSetDevice(c->device);
  const bool mixed = mixed_of(c);
  const int np = c->nprob;
  uint64_t total = 0;
  for (int p = 0; p < np; p++) {
    if (c->P.probs[p].src_count <= 0) return fail(ABX_ERR_INVALID, "problem %d has no sources", p);
    total += (uint64_t)c->P.probs[p].nparticles * (uint64_t)nbatches;
  }
  if (total == 0 || total > 0xffffffffull)
    return fail(ABX_ERR_CAPACITY, "%llu histories in one launch", (unsigned long long)total);
  int rc;
  if ((rc = ensure_virtual(c, nbatches)) != ABX_OK) return rc;
  if (after_host_copies(c->stream) != ABX_OK) return fail(ABX_ERR_CUDA, "stream ordering of the batch layout failed");
  if ((rc = ensure_banks(c, total, mixed, true)) != ABX_OK) return rc;
  if ((rc = ensure_sites(c, 1, mixed)) != ABX_OK) return rc;
  if ((rc = ensure_sec(c, mixed)) != ABX_OK) return rc;
  if ((rc = ensure_records(c, 1)) != ABX_OK) return rc;
  const size_t nv = (size_t)np * nbatches;
  const size_t R = (size_t)c->P.tally_bins;
  CUDA_TRY(cudaMemsetAsync(c->st, 0, sizeof(DevState), c->stream));
  CUDA_TRY(cudaMemsetAsync(c->run, 0, sizeof(RunAcc), c->stream));
  CUDA_TRY(cudaMemsetAsync(c->pscore, 0, nv * ABX_PSCORES * sizeof(double), c->stream));
  CUDA_TRY(cudaMemsetAsync(c->pcount, 0, nv * ABX_PCOUNTS * sizeof(unsigned long long), c->stream));
  zero_d(c->tally_gen, R * nbatches, c->stream);
  c->tally_g = 0;
  Tables TV = c->D.T;
  TV.probs = c->vprobs;
  TV.tallies = c->vtallies;
  TV.nprob = (int)nv;
  cudaEvent_t ev[4];
  for (auto& e : ev) cudaEventCreate(&e);
  cudaEventRecord(ev[0], c->stream);
  SourceArgs S{};
  S.T = TV;
  S.n = total;
  S.seg_off = c->seg_off;
  S.seg_prob = c->seg_prob;
  S.seg_hid0 = c->seg_hid0;
  S.nseg = (int)nv;
  sample_bank0(c, S, mixed, true);
  k_step_begin<<<1, 1, 0, c->stream>>>(c->st, total, 1.0, 1, 0);
  cudaEventRecord(ev[1], c->stream);
  c->batch_tables = TV;
  c->batch_scores = true;
  // with a history quota, warps retire after `warp_quota` histories and the
  // grid grows to cover the launch: blocks finish and hand their SM slots
  // to the launches of other contexts' streams while this one runs
  const int grid0 = c->grid;
  if (c->warp_quota && !needs_stacks(c) && !use_pool(c)) {
    const uint64_t per_block = (uint64_t)c->warp_quota * (uint64_t)(c->block / 32);
    const uint64_t need_blocks = (total + per_block - 1) / per_block;
    if (need_blocks > (uint64_t)c->grid) c->grid = (int)std::min<uint64_t>(need_blocks, 0x7fffffffull);
    c->launch_quota = c->warp_quota;
  }
  rc = launch_transport(c, mixed, 0, 0);
  c->launch_quota = 0;
  c->grid = grid0;
  c->batch_scores = false;
  cudaEventRecord(ev[2], c->stream);
  if (rc == ABX_OK) {
    if (R)
      k_tally_record_batches<<<grid_for(R), 256, 0, c->stream>>>(c->tally_gen, c->tally_avg, c->tally_var, R,
                                                                  nbatches);
    k_prob_record<<<(np + 255) / 256, 256, 0, c->stream>>>(c->pscore, c->pcount, (ProbRun*)c->prun, c->D.T.probs,
                                                           np, nbatches);
    k_gen_end<<<1, 1024, 0, c->stream>>>(c->st, c->run, c->D.T.probs, c->gen_rec, c->hist_cap, c->ent_bins,
                                         nullptr, 0, total, 0, 0);
    cudaEventRecord(ev[3], c->stream);
    if (cudaGetLastError() != cudaSuccess) rc = fail(ABX_ERR_CUDA, "launch failed");
  }
  if (rc == ABX_OK) rc = check_state(c);
  float sms = 0.f, tms = 0.f;
  if (rc == ABX_OK) {
    cudaEventElapsedTime(&sms, ev[0], ev[3]);
    cudaEventElapsedTime(&tms, ev[1], ev[2]);
  }
  for (auto& e : ev) cudaEventDestroy(e);
  if (rc) return rc;
  c->tally_g = nbatches;
  c->last_ms = tms;
  std::vector<ProbRun> pr((size_t)np);
  CUDA_TRY(cudaMemcpy(pr.data(), c->prun, (size_t)np * sizeof(ProbRun), cudaMemcpyDeviceToHost));
  RunAcc ra;
  CUDA_TRY(cudaMemcpy(&ra, c->run, sizeof ra, cudaMemcpyDeviceToHost));
  if (results) {
    for (int p = 0; p < np; p++) {
      abx_problem_result& r = results[p];
      memset(&r, 0, sizeof r);
      r.leak_avg = pr[p].leak_avg;
      r.leak_std = std::sqrt(pr[p].leak_var / nbatches);
      r.collisions = pr[p].coll;
      r.flights = pr[p].flights;
      r.histories = pr[p].hist;
      r.lost = pr[p].lost;
      r.batches = nbatches;
      r.tally_first = c->P.probs[p].tally_first;
    }
  }
  if (stats) {
    memset(stats, 0, sizeof *stats);
    stats->generations = nbatches;
    stats->active = nbatches;
    stats->collisions = ra.total_coll;
    stats->flights = ra.total_flights;
    stats->histories = ra.total_hist;
    stats->transport_ms = tms;
    stats->total_ms = sms;
  }
  return ABX_OK;
}
