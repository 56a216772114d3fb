// Device table layouts of the GB300 transport engine (shared by host and device code).
//
// A problem is flattened into pools whose indices are global, so one launch can
// carry many problems (batched fixed-source) with no per-problem pointers.
#pragma once

#include <cstdint>

#include "../../include/abeille_gb300.h"

namespace abx {

template <class R> struct SurfT {
  int32_t type, bc;
  R c[4];
};

template <class R> struct LatT {
  R p[3];     // pitch
  R lo[3];    // low corner: origin - N*0.5*pitch (src/rect_lattice.cpp:49-51)
  R pinv[3];  // 1/pitch
};

struct CellT {
  int32_t rpn_off, rpn_len;
  int32_t simple;    // no complement/union: operators stripped (src/cell.cpp:222-246)
  int32_t has_bc;    // any vacuum/reflective surface (src/cell.cpp:208-220)
  int32_t fill_kind, fill;
  int32_t reentry;   // universe index universe_id_to_indx[cell id] yields
  int32_t pad_;
};

struct UnivT {
  int32_t kind, list_off, list_len;
  int32_t n[3];
  int32_t outer;
  int32_t has_bc;
  int32_t lat;  // index into the lattice parameter pool
  // distinct boundary-condition half-spaces of the universe's cells (region
  // tokens in the rpn pool), or bc_len = -1 when a cell is not a plain
  // intersection; used by the mixed-mode boundary search
  int32_t bc_off, bc_len;
};

// Per material: xs block (7 rows of G: Et, Eabs, Ef, nu_tot, nu_d, Es, vEf),
// CDF block (scatter rows [G][G] then chi rows [G][G]), angle headers [G][G].
enum { XS_ET = 0, XS_EABS = 1, XS_EF = 2, XS_NU = 3, XS_NUD = 4, XS_ES = 5, XS_VEF = 6, XS_ROWS = 7 };
struct MatT {
  int32_t xs_off;
  int32_t cdf_off;
  int32_t ang_off;
  int32_t dg_off, ndg;
  int32_t fissile;
  int32_t G;
  int32_t iso;  // every angle table is the isotropic two-point table
};

struct AngHdr {
  int32_t off, n;  // mu at off, pdf at off+n, cdf at off+2n
};

struct TallyT {
  int32_t est, quantity;
  int32_t n[3];
  int32_t ne, eb_off;
  int32_t pad_;
  int64_t bin_off;  // into the tally pool
  double low[3], hi[3], d[3], dinv[3];
  float lowf[3], hif[3], df[3], dinvf[3];
};

struct ProbT {
  int32_t root;
  int32_t G;
  int32_t eb_off;      // energy bounds (G+1) in the bounds pool
  int32_t maj_off;     // majorant (G), then the Carter sampling xs (G), in the majorant pool
  int32_t tally_first, tally_count;
  int32_t mode, tracking;
  int32_t has_tle, has_coll;
  uint64_t seed, stride;
  double wgt_cutoff, wgt_survival;
  double nparticles;
  double inv_np;       // 1/nparticles
  double min_energy;
  float wgt_cutoff_f, wgt_survival_f;
  int32_t ent_on;
  int32_t ent_shape[3];
  double ent_low[3], ent_d[3];
  int32_t src_first, src_count;   // into the source pool
  int32_t src_cdf_off;            // discrete CDF over source weights
  float wgt_split_f;
  double wgt_split;               // Carter tracking and branchless splitting split at |weight| >= this
  int32_t branchless;             // ABX_BRANCHLESS_* flags (0: branching collisions)
  int32_t global_rng_skip;        // combing: outputs the global stream drew before the run
};

struct Tables {
  const CellT* cells;
  const int32_t* rpn;
  const UnivT* univ;
  const int32_t* cell_lists;
  const int32_t* lat_elems;
  const MatT* mats;
  const AngHdr* ang_hdr;
  const ProbT* probs;
  int32_t nprob;
  int32_t pad_;
  const TallyT* tallies;
  double* tally_gen;
  const abx_source* sources;
  const double* src_cdf;
  // precision-specific pools
  const SurfT<double>* surf_d;
  const SurfT<float>* surf_f;
  const LatT<double>* lat_d;
  const LatT<float>* lat_f;
  const double* xs_d;
  const float* xs_f;
  const double* cdf_d;
  const float* cdf_f;
  const double* ang_d;
  const float* ang_f;
  const double* eb_d;
  const float* eb_f;
  const double* maj_d;
  const float* maj_f;
  const double* dg_d;
  const float* dg_f;
  const double* tally_eb;   // tally energy bounds pool (double)
  const float* tally_eb_f;
};

// Device-resident run state (one per context / launch).
struct DevState {
  unsigned long long next_hist;   // work counter
  unsigned long long n_hist;      // histories in the current bank
  unsigned long long site_count;  // fission sites appended
  unsigned long long site_pos, site_neg;
  unsigned long long collisions, flights, lost;
  double scores[6];               // k_col k_abs k_trk k_tot leak mig
  double kcol;                    // previous generation's k_col
  int converged;
  int err;
  unsigned long long err_hist;
  unsigned long long trace_n;
  unsigned long long sec_overflow;
  double site_wsum;               // sum of the fission sites' weights (branchless collisions)
};

}  // namespace abx
