// Host table derivation of the GB300 transport engine: one abx_problem
// appended to the flat pools (problem_tables.h).  Compiled with host
// -ffp-contract=off: every double derived here rounds as the reference's does.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "problem_tables.h"

namespace abx {

void set_error_string(const char* msg);  // engine.cu: the thread's C-ABI error string

static int fail(int code, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  set_error_string(buf);
  return code;
}

// discrete_distribution param init (libstdc++ bits/random.tcc:2657-2678)
static void discrete_cdf(const double* w, int n, double* cp) {
  if (n < 2) return;
  double sum = 0.0;
  for (int i = 0; i < n; i++) sum += w[i];
  double acc = 0.0;
  for (int i = 0; i < n; i++) {
    double p = w[i] / sum;
    acc = (i == 0) ? p : acc + p;
    cp[i] = acc;
  }
  cp[n - 1] = 1.0;
}

static double legendre_p(unsigned n, double x) {
  // LegendreDistribution::legendre (include/materials/legendre_distribution.hpp:160-193)
  switch (n) {
    case 0: return 1.;
    case 1: return x;
    case 2: return 0.5 * (3. * x * x - 1.);
    case 3: return 0.5 * (5. * x * x * x - 3. * x);
    case 4: { const double x2 = x * x; return 0.125 * (35. * x2 * x2 - 30. * x2 + 3.); }
    default: {
      const double x2 = x * x, x3 = x2 * x, x4 = x3 * x;
      double p3 = 0.5 * (5. * x3 - 3. * x), p4 = 0.125 * (35. * x4 - 30. * x2 + 3.);
      unsigned l = 4;
      while (l < n) {
        std::swap(p3, p4);
        p4 = ((2. * l + 1.) * x * p3 - l * p4) / (l + 1.);
        l++;
      }
      return p4;
    }
  }
}

// LegendreDistribution::linearize (src/legendre_distribution.cpp:105-155)
static bool linearize(const std::vector<double>& a, std::vector<double>& mu, std::vector<double>& p,
                      std::vector<double>& c) {
  auto pdf = [&](double m) {
    double s = 0;
    for (size_t l = 0; l < a.size(); l++) s += a[l] * legendre_p((unsigned)l, m);
    return s;
  };
  mu = {-1., 1.};
  p = {pdf(-1.), pdf(1.)};
  size_t i = 0;
  while (i < mu.size() - 1) {
    double mid = 0.5 * (mu[i] + mu[i + 1]);
    double pi = 0.5 * (p[i] + p[i + 1]);
    double pr = pdf(mid);
    double rel = std::fabs(pi - pr) / pr;
    if (rel > 0.0001) {
      mu.insert(mu.begin() + (long)i + 1, mid);
      p.insert(p.begin() + (long)i + 1, pr);
      if (mu.size() > 100000) return false;
    } else {
      i++;
    }
  }
  c.assign(mu.size(), 0.);
  for (size_t k = 0; k + 1 < mu.size(); k++) c[k + 1] = ((mu[k + 1] - mu[k]) * 0.5 * (p[k + 1] + p[k])) + c[k];
  const double norm = c.back();
  for (size_t k = 0; k < c.size(); k++) {
    p[k] /= norm;
    c[k] /= norm;
  }
  return true;
}

// Appends one problem to the pools, offsetting every index so the pools can
// hold many problems.
int append_problem(Pools& P, const abx_problem* pr) {
  if (!pr) return fail(ABX_ERR_INVALID, "null problem");
  const abx_settings& s = pr->settings;
  const int G = s.ngroups;
  if (G < 1 || G > 1024) return fail(ABX_ERR_INVALID, "ngroups %d out of range", G);
  if (s.mode != ABX_MODE_K_EIGENVALUE && s.mode != ABX_MODE_FIXED_SOURCE)
    return fail(ABX_ERR_UNSUPPORTED, "simulation mode %d is outside the multigroup transport path", s.mode);
  if (s.tracking < ABX_TRACK_DELTA || s.tracking > ABX_TRACK_CARTER)
    return fail(ABX_ERR_UNSUPPORTED, "tracking mode %d not supported", s.tracking);
  if (!pr->energy_bounds) return fail(ABX_ERR_INVALID, "no energy bounds");
  for (int g = 0; g < G; g++)
    if (!(pr->energy_bounds[g] < pr->energy_bounds[g + 1]))
      return fail(ABX_ERR_INVALID, "energy bounds must be strictly ascending");
  if (pr->n_surfaces < 0 || pr->n_cells <= 0 || pr->n_universes <= 0 || pr->n_materials <= 0)
    return fail(ABX_ERR_INVALID, "problem needs surfaces, cells, universes and materials");
  if (pr->root_universe < 0 || pr->root_universe >= pr->n_universes)
    return fail(ABX_ERR_INVALID, "root universe index %d out of range", pr->root_universe);
  if (!(s.nparticles > 0)) return fail(ABX_ERR_INVALID, "nparticles must be positive");

  const int surf0 = (int)P.surf_d.size(), cell0 = (int)P.cells.size(), univ0 = (int)P.univ.size();
  const int mat0 = (int)P.mats.size(), lat0 = (int)P.lat_d.size();
  // surfaces
  for (int i = 0; i < pr->n_surfaces; i++) {
    const abx_surface& a = pr->surfaces[i];
    if (a.type < ABX_SURF_XPLANE || a.type > ABX_SURF_SPHERE) return fail(ABX_ERR_INVALID, "surface %d: bad type", i);
    if (a.bc < ABX_BC_VACUUM || a.bc > ABX_BC_NORMAL) return fail(ABX_ERR_INVALID, "surface %d: bad boundary", i);
    SurfT<double> t;
    t.type = a.type;
    t.bc = a.bc;
    for (int k = 0; k < 4; k++) t.c[k] = a.c[k];
    P.surf_d.push_back(t);
  }
  // cells (Cell ctor: simplify + check_for_bc, src/cell.cpp:37-67,208-246)
  for (int i = 0; i < pr->n_cells; i++) {
    const abx_cell& c = pr->cells[i];
    if (c.rpn_offset < 0 || c.rpn_len < 0 || c.rpn_offset + c.rpn_len > pr->n_rpn)
      return fail(ABX_ERR_INVALID, "cell %u: region out of range", c.id);
    const int32_t* r = pr->rpn + c.rpn_offset;
    bool simple = true;
    for (int k = 0; k < c.rpn_len; k++)
      if (r[k] == ABX_OP_COMP || r[k] == ABX_OP_UNIN) simple = false;
    CellT t{};
    t.rpn_off = (int)P.rpn.size();
    int depth = 0, maxd = 0;
    for (int k = 0; k < c.rpn_len; k++) {
      int32_t tok = r[k];
      if (tok >= ABX_OP_UNIN) {
        if (tok == ABX_OP_LPAR || tok == ABX_OP_RPAR) return fail(ABX_ERR_INVALID, "cell %u: parentheses in RPN", c.id);
        if (tok != ABX_OP_COMP) depth--;
        if (simple) continue;
        P.rpn.push_back(tok);
        continue;
      }
      int a = tok < 0 ? -tok : tok;
      if (a < 1 || a > pr->n_surfaces) return fail(ABX_ERR_INVALID, "cell %u: surface token %d out of range", c.id, tok);
      int bc = pr->surfaces[a - 1].bc;
      if (bc == ABX_BC_VACUUM || bc == ABX_BC_REFLECTIVE) t.has_bc = 1;
      P.rpn.push_back(tok > 0 ? tok + surf0 : tok - surf0);
      depth++;
      maxd = std::max(maxd, depth);
    }
    if (!simple && maxd > 60) return fail(ABX_ERR_INVALID, "cell %u: region too deep", c.id);
    t.rpn_len = (int)P.rpn.size() - t.rpn_off;
    t.simple = simple;
    t.fill_kind = c.fill_kind;
    if (c.fill_kind == ABX_FILL_MATERIAL) {
      if (c.fill < 0 || c.fill >= pr->n_materials) return fail(ABX_ERR_INVALID, "cell %u: material out of range", c.id);
      t.fill = c.fill + mat0;
    } else if (c.fill_kind == ABX_FILL_UNIVERSE) {
      if (c.fill < 0 || c.fill >= pr->n_universes) return fail(ABX_ERR_INVALID, "cell %u: universe out of range", c.id);
      t.fill = c.fill + univ0;
    } else {
      return fail(ABX_ERR_INVALID, "cell %u: bad fill kind", c.id);
    }
    // universe_id_to_indx[cell id] (tracker.hpp:284-285 on a Cell pad)
    t.reentry = univ0;
    for (int u = 0; u < pr->n_universes; u++)
      if (pr->universes[u].id == c.id) { t.reentry = univ0 + u; break; }
    P.cells.push_back(t);
  }
  // universes
  for (int i = 0; i < pr->n_universes; i++) {
    const abx_universe& u = pr->universes[i];
    UnivT t{};
    t.kind = u.kind;
    t.outer = -1;
    t.lat = -1;
    if (u.kind == ABX_UNIV_CELLS) {
      if (u.list_offset < 0 || u.list_len <= 0 || u.list_offset + u.list_len > pr->n_cell_lists)
        return fail(ABX_ERR_INVALID, "universe %u: cell list out of range", u.id);
      t.list_off = (int)P.cell_lists.size();
      t.list_len = u.list_len;
      for (int k = 0; k < u.list_len; k++) {
        int ci = pr->cell_lists[u.list_offset + k];
        if (ci < 0 || ci >= pr->n_cells) return fail(ABX_ERR_INVALID, "universe %u: cell index out of range", u.id);
        P.cell_lists.push_back(ci + cell0);
        if (P.cells[ci + cell0].has_bc) t.has_bc = 1;
      }
    } else if (u.kind == ABX_UNIV_RECT_LATTICE) {
      int64_t n = (int64_t)u.shape[0] * u.shape[1] * u.shape[2];
      if (u.shape[0] <= 0 || u.shape[1] <= 0 || u.shape[2] <= 0 || n != u.list_len ||
          u.list_offset < 0 || u.list_offset + n > pr->n_lattice_elems)
        return fail(ABX_ERR_INVALID, "lattice %u: shape/elements mismatch", u.id);
      if (u.shape[0] > 500 || u.shape[1] > 500 || u.shape[2] > 500)
        return fail(ABX_ERR_UNSUPPORTED, "lattice %u: more than 500 tiles along an axis", u.id);
      t.list_off = (int)P.lat_elems.size();
      t.list_len = (int)n;
      for (int a = 0; a < 3; a++) t.n[a] = u.shape[a];
      for (int64_t k = 0; k < n; k++) {
        int e = pr->lattice_elems[u.list_offset + k];
        if (e >= pr->n_universes) return fail(ABX_ERR_INVALID, "lattice %u: element out of range", u.id);
        P.lat_elems.push_back(e < 0 ? -1 : e + univ0);
      }
      if (u.outer >= pr->n_universes) return fail(ABX_ERR_INVALID, "lattice %u: outer universe out of range", u.id);
      t.outer = u.outer < 0 ? -1 : u.outer + univ0;
      // RectLattice ctor (src/rect_lattice.cpp:33-52)
      LatT<double> L;
      for (int a = 0; a < 3; a++) {
        if (!(u.pitch[a] > 0)) return fail(ABX_ERR_INVALID, "lattice %u: pitch must be positive", u.id);
        L.p[a] = u.pitch[a];
        L.pinv[a] = 1. / u.pitch[a];
        L.lo[a] = u.origin[a] - (double)u.shape[a] * 0.5 * u.pitch[a];
      }
      t.lat = (int)P.lat_d.size();
      P.lat_d.push_back(L);
    } else {
      return fail(ABX_ERR_INVALID, "universe %u: bad kind", u.id);
    }
    P.univ.push_back(t);
  }
  // distinct boundary-condition tokens per cell universe (mixed-mode search)
  for (int i = univ0; i < (int)P.univ.size(); i++) {
    UnivT& U = P.univ[i];
    U.bc_off = (int)P.rpn.size();
    U.bc_len = 0;
    if (U.kind != ABX_UNIV_CELLS || !U.has_bc) continue;
    std::vector<int32_t> toks;
    for (int j = 0; j < U.list_len && U.bc_len >= 0; j++) {
      const CellT& c = P.cells[P.cell_lists[U.list_off + j]];
      if (!c.has_bc) continue;
      if (!c.simple) {
        U.bc_len = -1;
        break;
      }
      for (int k = 0; k < c.rpn_len; k++) {
        const int32_t t = P.rpn[c.rpn_off + k];
        if (P.surf_d[std::abs(t) - 1].bc == ABX_BC_NORMAL) continue;
        if (std::find(toks.begin(), toks.end(), t) == toks.end()) toks.push_back(t);
      }
    }
    if (U.bc_len < 0) continue;
    P.rpn.insert(P.rpn.end(), toks.begin(), toks.end());
    U.bc_len = (int)toks.size();
  }
  // lattices inherit their outer universe's boundary flag (src/lattice.cpp:45-53)
  for (int pass = 0; pass < 16; pass++)
    for (int i = univ0; i < (int)P.univ.size(); i++)
      if (P.univ[i].kind == ABX_UNIV_RECT_LATTICE) P.univ[i].has_bc = P.univ[i].outer >= 0 ? P.univ[P.univ[i].outer].has_bc : 0;
  (void)lat0;
  // materials (MGNuclide ctor + get_micro_xs, src/mg_nuclide.cpp:37-118, 394-411)
  std::vector<double> row(G), pr_row(G);
  ProbT pt{};
  pt.eb_off = (int)P.eb_d.size();
  for (int g = 0; g <= G; g++) P.eb_d.push_back(pr->energy_bounds[g]);
  pt.maj_off = (int)P.maj_d.size();
  std::vector<double> maj(G, 0.);
  for (int m = 0; m < pr->n_materials; m++) {
    const abx_material& mt = pr->materials[m];
    if (mt.n_legendre < 0 || mt.n_legendre > 5 || mt.n_delayed < 0)
      return fail(ABX_ERR_INVALID, "material %u: bad Legendre/delayed counts", mt.id);
    int64_t need = (int64_t)5 * G + 2LL * G * G + (int64_t)mt.n_legendre * G * G + 2LL * mt.n_delayed;
    if (mt.data_offset < 0 || mt.data_offset + need > pr->n_mg_data)
      return fail(ABX_ERR_INVALID, "material %u: data out of range", mt.id);
    const double* d = pr->mg_data + mt.data_offset;
    const double *tot = d, *abs_ = d + G, *fis = d + 2 * G, *nup = d + 3 * G, *nud = d + 4 * G;
    const double* chi = d + 5 * G;
    const double* sct = chi + (size_t)G * G;
    const double* legm = sct + (size_t)G * G;
    const double* dgp = legm + (size_t)mt.n_legendre * G * G;
    // the input checks of make_mg_nuclide (src/mg_nuclide.cpp:604-636, 720-738, 826-834)
    for (int g = 0; g < G; g++) {
      if (fis[g] < 0.) return fail(ABX_ERR_INVALID, "Negative fission xs in material %u.", mt.id);
      for (int o = 0; o < G; o++) {
        if (sct[(size_t)g * G + o] < 0.)
          return fail(ABX_ERR_INVALID,
                      "Negative scattering component at row %d, column %d of the scattering matrix for material %u.",
                      g, o, mt.id);
        if (chi[(size_t)g * G + o] < 0.)
          return fail(ABX_ERR_INVALID, "chi[%d][%d] is negative in material %u.", g, o, mt.id);
      }
    }
    MatT M{};
    M.G = G;
    M.xs_off = (int)P.xs_d.size();
    P.xs_d.resize(P.xs_d.size() + (size_t)XS_ROWS * G);
    double* xs = P.xs_d.data() + M.xs_off;
    for (int g = 0; g < G; g++) {
      xs[XS_ET * G + g] = tot[g];
      xs[XS_EF * G + g] = fis[g];
      xs[XS_EABS * G + g] = fis[g] + (abs_[g] - fis[g]);
      xs[XS_NU * G + g] = nup[g] + nud[g];
      xs[XS_NUD * G + g] = nud[g];
      xs[XS_VEF * G + g] = 1. * (nup[g] + nud[g]) * fis[g];
      if (fis[g] != 0. && (nup[g] + nud[g]) > 0.) M.fissile = 1;
      if (tot[g] > maj[g]) maj[g] = tot[g];
    }
    M.cdf_off = (int)P.cdf_d.size();
    P.cdf_d.resize(P.cdf_d.size() + 2 * (size_t)G * G);
    double* cdf = P.cdf_d.data() + M.cdf_off;
    for (int g = 0; g < G; g++) {
      double es = 0.;
      for (int o = 0; o < G; o++) es += sct[(size_t)g * G + o];
      xs[XS_ES * G + g] = es;
      for (int o = 0; o < G; o++) row[o] = sct[(size_t)g * G + o] / es;
      discrete_cdf(row.data(), G, cdf + (size_t)g * G);
      if (!M.fissile) continue;  // no fission neutron is ever sampled: the chi rows stay zero
      double ci = 0.;
      for (int o = 0; o < G; o++) ci += chi[(size_t)g * G + o];
      for (int o = 0; o < G; o++) row[o] = chi[(size_t)g * G + o] / ci;
      discrete_cdf(row.data(), G, cdf + (size_t)G * G + (size_t)g * G);
    }
    M.ndg = mt.n_delayed;
    M.dg_off = (int)P.dg_d.size();
    P.dg_d.resize(P.dg_d.size() + (size_t)std::max(1, mt.n_delayed));
    discrete_cdf(dgp, mt.n_delayed, P.dg_d.data() + M.dg_off);
    // angle tables; none when every Legendre moment is zero (isotropic
    // scattering, whose flat tables sampling inverts directly)
    const size_t hdr0 = P.ang_hdr.size(), ang0 = P.ang_d.size();
    M.ang_off = (int)hdr0;
    M.iso = 1;
    bool all_flat = true;
    for (size_t q = 0, nq = (size_t)mt.n_legendre * G * G; q < nq && all_flat; q++) all_flat = legm[q] == 0.;
    for (int gi = 0; gi < G && !all_flat; gi++)
      for (int go = 0; go < G; go++) {
        double ac[6] = {0.5, 0., 0., 0., 0., 0.};
        bool flat = true;
        for (int l = 1; l <= mt.n_legendre; l++) {
          double coeff = legm[((size_t)(l - 1) * G + gi) * G + go];
          ac[l] = coeff * (2. * (double)l + 1.) / 2.;
          flat = flat && ac[l] == 0.;
        }
        AngHdr h{(int)P.ang_d.size(), 2};
        if (flat) {
          // pdf 1/2 on [-1, 1]: linearize stops at once with mu {-1, 1},
          // p {1/2, 1/2}, cdf {0, 1}
          const double iso_tab[6] = {-1., 1., 0.5, 0.5, 0., 1.};
          P.ang_d.insert(P.ang_d.end(), iso_tab, iso_tab + 6);
          P.ang_hdr.push_back(h);
          continue;
        }
        const std::vector<double> a(ac, ac + mt.n_legendre + 1);
        std::vector<double> mu, pp, cc;
        if (!linearize(a, mu, pp, cc)) return fail(ABX_ERR_INVALID, "material %u: angle table did not converge", mt.id);
        // MGAngleDistribution's check (src/mg_angle_distribution.cpp:53-58)
        for (double p : pp)
          if (p < 0.)
            return fail(ABX_ERR_INVALID, "material %u: the angle distribution from group %d to group %d has a "
                        "negative pdf (PDF is less than 0)", mt.id, gi, go);
        bool iso = mu.size() == 2 && pp[0] == 0.5 && pp[1] == 0.5 && cc[0] == 0. && cc[1] == 1.;
        if (!iso) M.iso = 0;
        h.n = (int)mu.size();
        P.ang_d.insert(P.ang_d.end(), mu.begin(), mu.end());
        P.ang_d.insert(P.ang_d.end(), pp.begin(), pp.end());
        P.ang_d.insert(P.ang_d.end(), cc.begin(), cc.end());
        P.ang_hdr.push_back(h);
      }
    if (M.iso) {
      // every (g, g') table is the flat one, which sampling inverts directly
      P.ang_hdr.resize(hdr0);
      P.ang_d.resize(ang0);
      M.ang_off = -1;
    }
    P.mats.push_back(M);
  }
  // majorant (src/majorant.cpp:132-176), then the sampling cross section of
  // Carter tracking, majorant x sampling-xs-ratio (src/carter_tracker.cpp:60-72)
  for (int g = 0; g < G; g++) P.maj_d.push_back(maj[g]);
  for (int g = 0; g < G; g++) {
    const double ratio = pr->sampling_xs_ratio ? pr->sampling_xs_ratio[g] : 1.0;
    if (!(ratio > 0.)) return fail(ABX_ERR_INVALID, "sampling-xs-ratio must be positive (group %d)", g);
    P.maj_d.push_back(maj[g] * ratio);
  }
  // tallies (src/mesh_tally.cpp:62-119)
  pt.tally_first = (int)P.tallies.size();
  pt.tally_count = pr->n_tallies;
  for (int i = 0; i < pr->n_tallies; i++) {
    const abx_mesh_tally& d = pr->tallies[i];
    if (d.estimator != ABX_EST_COLLISION && d.estimator != ABX_EST_TRACK_LENGTH)
      return fail(ABX_ERR_UNSUPPORTED, "tally %d: estimator not supported", i);
    if (d.quantity < ABX_Q_FLUX || d.quantity > ABX_Q_TOTAL) return fail(ABX_ERR_UNSUPPORTED, "tally %d: quantity", i);
    if (d.shape[0] <= 0 || d.shape[1] <= 0 || d.shape[2] <= 0 || d.n_ebounds < 2 || d.ebounds_offset < 0 ||
        d.ebounds_offset + d.n_ebounds > pr->n_tally_ebounds)
      return fail(ABX_ERR_INVALID, "tally %d: bad shape or energy bounds", i);
    TallyT t{};
    t.est = d.estimator;
    t.quantity = d.quantity;
    for (int a = 0; a < 3; a++) {
      t.n[a] = d.shape[a];
      t.low[a] = d.low[a];
      t.hi[a] = d.hi[a];
      t.d[a] = (d.hi[a] - d.low[a]) / (double)d.shape[a];
      t.dinv[a] = 1. / t.d[a];
      t.lowf[a] = (float)t.low[a];
      t.hif[a] = (float)t.hi[a];
      t.df[a] = (float)t.d[a];
      t.dinvf[a] = 1.f / t.df[a];
    }
    t.ne = d.n_ebounds - 1;
    t.eb_off = (int)P.tally_eb.size();
    for (int k = 0; k < d.n_ebounds; k++) P.tally_eb.push_back(pr->tally_ebounds[d.ebounds_offset + k]);
    t.bin_off = P.tally_bins;
    P.tally_bins += (int64_t)t.ne * t.n[0] * t.n[1] * t.n[2];
    if (d.estimator == ABX_EST_TRACK_LENGTH) pt.has_tle = 1;
    else pt.has_coll = 1;
    P.tallies.push_back(t);
  }
  // sources (src/simulation.cpp:58-69)
  pt.src_first = (int)P.sources.size();
  pt.src_count = pr->n_sources;
  pt.src_cdf_off = (int)P.src_cdf.size();
  {
    std::vector<double> w(std::max(1, pr->n_sources), 0.);
    for (int i = 0; i < pr->n_sources; i++) {
      const abx_source& so = pr->sources[i];
      if (so.spatial != ABX_SPATIAL_POINT && so.spatial != ABX_SPATIAL_BOX)
        return fail(ABX_ERR_UNSUPPORTED, "source %d: spatial distribution", i);
      if (so.direction != ABX_DIR_ISOTROPIC && so.direction != ABX_DIR_MONO)
        return fail(ABX_ERR_UNSUPPORTED, "source %d: direction distribution", i);
      if (so.energy != ABX_ENERGY_MONO) return fail(ABX_ERR_UNSUPPORTED, "source %d: energy distribution", i);
      if (!(so.weight > 0)) return fail(ABX_ERR_INVALID, "source %d: weight must be positive", i);
      P.sources.push_back(so);
      w[i] = so.weight;
    }
    P.src_cdf.resize(P.src_cdf.size() + w.size());
    discrete_cdf(w.data(), pr->n_sources, P.src_cdf.data() + pt.src_cdf_off);
  }
  // settings
  pt.root = pr->root_universe + univ0;
  pt.G = G;
  pt.mode = s.mode;
  pt.tracking = s.tracking;
  pt.seed = s.seed;
  pt.stride = s.stride;
  pt.wgt_cutoff = s.wgt_cutoff;
  pt.wgt_survival = s.wgt_survival;
  pt.wgt_cutoff_f = (float)s.wgt_cutoff;
  pt.wgt_survival_f = (float)s.wgt_survival;
  pt.wgt_split = s.wgt_split > 0. ? s.wgt_split : 2.0;  // src/settings.cpp:64
  pt.wgt_split_f = (float)pt.wgt_split;
  if (s.tracking == ABX_TRACK_CARTER && !(pt.wgt_split > s.wgt_survival))
    return fail(ABX_ERR_INVALID, "wgt-split must exceed wgt-survival (src/parser.cpp:689-697)");
  pt.branchless = 0;
  if (s.branchless) {
    if (s.branchless & ~(ABX_BRANCHLESS_ON | ABX_BRANCHLESS_MATERIAL | ABX_BRANCHLESS_SPLITTING |
                         ABX_BRANCHLESS_COMBING) ||
        !(s.branchless & ABX_BRANCHLESS_ON))
      return fail(ABX_ERR_INVALID, "branchless flags %d", s.branchless);
    if (s.mode != ABX_MODE_K_EIGENVALUE)
      return fail(ABX_ERR_UNSUPPORTED, "branchless collisions belong to the branchless k-eigenvalue simulation");
    if (s.tracking != ABX_TRACK_DELTA && s.tracking != ABX_TRACK_SURFACE)
      return fail(ABX_ERR_UNSUPPORTED, "branchless collisions with delta or surface tracking only");
    pt.branchless = s.branchless;
    pt.global_rng_skip = s.global_rng_skip;
  }
  pt.nparticles = s.nparticles;
  pt.inv_np = 1. / s.nparticles;
  pt.min_energy = std::max(0., pr->energy_bounds[0]);  // src/parser.cpp:157-168
  pt.ent_on = pr->entropy.enabled;
  for (int a = 0; a < 3; a++) {
    pt.ent_shape[a] = pr->entropy.enabled ? pr->entropy.shape[a] : 1;
    pt.ent_low[a] = pr->entropy.low[a];
    pt.ent_d[a] = pr->entropy.enabled ? (pr->entropy.hi[a] - pr->entropy.low[a]) / (double)pr->entropy.shape[a] : 1.;
  }
  if (pr->entropy.enabled && (pr->entropy.shape[0] <= 0 || pr->entropy.shape[1] <= 0 || pr->entropy.shape[2] <= 0))
    return fail(ABX_ERR_INVALID, "entropy mesh shape must be positive");
  P.probs.push_back(pt);
  return ABX_OK;
}

}  // namespace abx
