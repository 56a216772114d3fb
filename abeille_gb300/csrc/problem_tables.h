// Host pools of the flattened problem tables: every problem of a context is
// appended here with global indices, then uploaded as one set of device
// pools (and FP32 mirrors).
#pragma once

#include <cstdint>
#include <vector>

#include "tables.h"

namespace abx {

struct Pools {
  std::vector<CellT> cells;
  std::vector<int32_t> rpn;
  std::vector<UnivT> univ;
  std::vector<int32_t> cell_lists, lat_elems;
  std::vector<MatT> mats;
  std::vector<AngHdr> ang_hdr;
  std::vector<ProbT> probs;
  std::vector<TallyT> tallies;
  std::vector<abx_source> sources;
  std::vector<double> src_cdf;
  std::vector<SurfT<double>> surf_d;
  std::vector<LatT<double>> lat_d;
  std::vector<double> xs_d, cdf_d, ang_d, eb_d, maj_d, dg_d, tally_eb;
  int64_t tally_bins = 0;
  int max_depth = 0;
};

// Appends one problem (the reference's parsed globals, src/parser.cpp:77-1054)
// to the pools, deriving the tables the transport reads: surface and cell
// layouts, universe boundary half-spaces, group-transfer and chi CDFs
// (MGNuclide, src/mg_nuclide.cpp:37-118), angle tables
// (LegendreDistribution::linearize), majorant and Carter sampling cross
// section, tallies, sources and settings.  ABX_OK or an error code with the
// thread's error string set.
int append_problem(Pools& P, const abx_problem* pr);

}  // namespace abx
