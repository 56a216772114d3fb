/*
 * Oracle: CPU restatement of Abeille's multigroup transport loop.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle.h).  Every function below names the
 * reference file:line it restates (paths relative to the Abeille v0.4.0 source
 * tree).  Arithmetic is written in the reference's operand order and the file
 * is compiled with -ffp-contract=off, so each double operation rounds exactly
 * where the reference's does.  libm's log/sin/cos/sqrt are called just as the
 * reference calls them.
 *
 * Third-party arithmetic restated here (absent from the reference tree):
 *  - pcg32 = pcg_engines::setseq_xsh_rr_64_32 of pcg-cpp (fork
 *    HunterBelanger/pcg-cpp@feature/cmake, unpinned branch): 64-bit LCG with
 *    multiplier 6364136223846793005 and default increment
 *    1442695040888963407, XSH-RR output of the previous state, seeding
 *    state = (seed + inc) * mult + inc, jump-ahead by Brown's algorithm.
 *  - libstdc++ 13 <random>: generate_canonical<double,53> from two 32-bit
 *    outputs, exponential_distribution = -log(1-u)/lambda,
 *    discrete_distribution = normalise, partial sum, last entry forced to 1,
 *    lower_bound; no draw with fewer than two weights.
 * Both are pinned by golden vectors made from the real libraries.
 */
#include "oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <stdarg.h>

#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------ constants */
/* include/utils/constants.hpp:42-57 */
static const double INF_ = 1.7976931348623157e308; /* std::numeric_limits<double>::max() */
static const double PI_ = 3.14159265358979323846264338327950288;
#define SURFACE_COINCIDENT 1e-12
static double BOUNDRY_TOL_ = 0.0;   /* 500. * SURFACE_COINCIDENT, set at init */
static double TILE_TOL_ = 0.0;      /* 100 * SURFACE_COINCIDENT (src/rect_lattice.cpp:270-281) */
#define TOLERANCE_LIN 0.0001        /* constants.hpp TOLERANCE */
#define MAXPADS 16

static char g_err[512];
static void set_err(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof g_err, fmt, ap);
  va_end(ap);
}
const char* oracle_last_error(void) { return g_err; }

/* --------------------------------------------------------------- vectors */
/* include/utils/{vector,position,direction}.hpp */
typedef struct { double x, y, z; } V3;
static inline V3 v3(double x, double y, double z) { V3 v; v.x = x; v.y = y; v.z = z; return v; }
static inline V3 vadd(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline V3 vsub(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
/* c * Direction -> Vector(d.x()*c, ...) (direction.hpp:112-114) */
static inline V3 vscale(V3 v, double c) { return v3(v.x * c, v.y * c, v.z * c); }
static inline double vdot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline double vnorm(V3 a) { return sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
/* Direction(x,y,z) renormalises (direction.hpp:37-42) */
static inline V3 dir3(double x, double y, double z) {
  double m = sqrt(x * x + y * y + z * z);
  return v3(x / m, y / m, z / m);
}
/* Direction(mu, phi) (direction.hpp:43-62) */
static V3 dir_mu_phi(double mu, double phi) {
  if (mu < -1.) mu = -1.;
  else if (mu > 1.) mu = 1.;
  if (phi < 0.) phi = 0.;
  else if (phi > 2 * PI_) phi = 2 * PI_;
  double x = sqrt(1. - mu * mu) * cos(phi);
  double y = sqrt(1. - mu * mu) * sin(phi);
  double z = mu;
  return dir3(x, y, z);
}
/* rotate_direction (direction.hpp:130-151) */
static V3 rotate_direction(V3 u, double mu, double phi) {
  double c = cos(phi);
  double s = sin(phi);
  double sqrt_mu = sqrt(1. - mu * mu);
  double sqrt_w = sqrt(1. - u.z * u.z);
  double ux, uy, uz;
  if (sqrt_w > 1.E-10) {
    ux = mu * u.x + sqrt_mu * (u.x * u.z * c - u.y * s) / sqrt_w;
    uy = mu * u.y + sqrt_mu * (u.y * u.z * c + u.x * s) / sqrt_w;
    uz = mu * u.z - sqrt_mu * sqrt_w * c;
  } else {
    double sqrt_v = sqrt(1. - u.y * u.y);
    ux = mu * u.x + sqrt_mu * (u.x * u.y * c + u.z * s) / sqrt_v;
    uy = mu * u.y - sqrt_mu * sqrt_v * c;
    uz = mu * u.z + sqrt_mu * (u.y * u.z * c - u.x * s) / sqrt_v;
  }
  return dir3(ux, uy, uz);
}

/* ------------------------------------------------------------------ RNG */
#define PCG_MULT 6364136223846793005ULL
#define PCG_INC 1442695040888963407ULL

void oracle_pcg32_seed(uint64_t seed, uint64_t* state) {
  *state = (seed + PCG_INC) * PCG_MULT + PCG_INC;
}
uint32_t oracle_pcg32_next(uint64_t* state) {
  uint64_t old = *state;
  *state = old * PCG_MULT + PCG_INC;
  uint32_t rot = (uint32_t)(old >> 59);
  uint32_t xs = (uint32_t)(((old >> 18) ^ old) >> 27);
  return (xs >> rot) | (xs << ((32u - rot) & 31u));
}
/* F. B. Brown, "Random number generation with arbitrary strides" (1994). */
void oracle_pcg32_advance(uint64_t* state, uint64_t delta) {
  uint64_t cur_mult = PCG_MULT, cur_plus = PCG_INC;
  uint64_t acc_mult = 1u, acc_plus = 0u;
  while (delta > 0) {
    if (delta & 1u) {
      acc_mult *= cur_mult;
      acc_plus = acc_plus * cur_mult + cur_plus;
    }
    cur_plus = (cur_mult + 1u) * cur_plus;
    cur_mult *= cur_mult;
    delta >>= 1;
  }
  *state = acc_mult * *state + acc_plus;
}
/* libstdc++ generate_canonical<double,53> over a 32-bit engine
 * (bits/random.tcc:3349-3380): two outputs, sum in double, scaled by 2^-64. */
double oracle_canonical(uint64_t* st) {
  double sum = (double)oracle_pcg32_next(st);
  sum += (double)oracle_pcg32_next(st) * 4294967296.0;
  double ret = sum / 18446744073709551616.0;
  if (ret >= 1.0) ret = 0x1.fffffffffffffp-1; /* nextafter(1, 0) */
  return ret;
}
/* libstdc++ uniform_int_distribution<unsigned long>{0, range} over a 32-bit
 * engine (bits/uniform_int_dist.h): for range < 2^32 - 1 the engine's range
 * is larger, and the draw is Lemire's nearly divisionless method (D. Lemire,
 * "Fast random integer generation in an interval", ACM TOMACS 29(1), 2019)
 * on 64-bit products: the high half of output * (range + 1), redrawn while
 * the low half falls below 2^32 mod (range + 1).  Ranges of 2^32 - 1 or more
 * (banks of four billion particles) are not needed here. */
static uint64_t uniform_upto(uint64_t* st, uint64_t range) {
  const uint32_t uerange = (uint32_t)(range + 1u);
  uint64_t product = (uint64_t)oracle_pcg32_next(st) * (uint64_t)uerange;
  uint32_t low = (uint32_t)product;
  if (low < uerange) {
    const uint32_t threshold = (uint32_t)(0u - uerange) % uerange;
    while (low < threshold) {
      product = (uint64_t)oracle_pcg32_next(st) * (uint64_t)uerange;
      low = (uint32_t)product;
    }
  }
  return product >> 32;
}

/* std::shuffle over a 32-bit engine (libstdc++ bits/stl_algo.h): when
 * n * n fits the engine's range (n <= 65535) the swap positions of two
 * successive elements come from one draw over [0, (i+1)(i+2)), an even n
 * first swapping element 1 with a draw over [0, 1]; otherwise one draw over
 * [0, i] per element i = 1 .. n-1. */
static void swap_elems(unsigned char* base, size_t sz, size_t i, size_t j, unsigned char* tmp) {
  if (i == j) return;
  memcpy(tmp, base + i * sz, sz);
  memcpy(base + i * sz, base + j * sz, sz);
  memcpy(base + j * sz, tmp, sz);
}
void oracle_shuffle(void* data, size_t n, size_t sz, uint64_t* st) {
  if (n == 0) return;
  unsigned char* base = (unsigned char*)data;
  unsigned char* tmp = (unsigned char*)calloc(1, sz ? sz : 1);
  if (!tmp) return;
  const uint64_t urngrange = 0xffffffffULL, urange = n;
  if (urngrange / urange >= urange) {
    size_t i = 1;
    if ((urange % 2) == 0) {
      swap_elems(base, sz, i, (size_t)uniform_upto(st, 1), tmp);
      i++;
    }
    while (i != n) {
      const uint64_t swap_range = (uint64_t)i + 1;
      const uint64_t x = uniform_upto(st, swap_range * (swap_range + 1) - 1);
      swap_elems(base, sz, i, (size_t)(x / (swap_range + 1)), tmp);
      i++;
      swap_elems(base, sz, i, (size_t)(x % (swap_range + 1)), tmp);
      i++;
    }
  } else {
    for (size_t i = 1; i < n; i++) swap_elems(base, sz, i, (size_t)uniform_upto(st, i), tmp);
  }
  free(tmp);
}

/* RNG::exponential (include/utils/rng.hpp:72-77) + exponential_distribution */
double oracle_exponential(uint64_t* st, double lambda) {
  if (lambda == 0.) return INF_;
  return -log(1.0 - oracle_canonical(st)) / lambda;
}
/* std::lower_bound on a cumulative table: first i with !(cp[i] < u). */
static int lower_bound_d(const double* cp, int n, double u) {
  int first = 0, count = n;
  while (count > 0) {
    int step = count / 2;
    int it = first + step;
    if (cp[it] < u) {
      first = it + 1;
      count -= step + 1;
    } else {
      count = step;
    }
  }
  return first;
}
/* discrete_distribution param init (bits/random.tcc:2657-2678) */
static void make_discrete_cdf(const double* w, int n, double* cp) {
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
/* discrete_distribution::operator() (bits/random.tcc:2697-2714) */
static int sample_discrete_cdf(uint64_t* st, const double* cp, int n) {
  if (n < 2) return 0;
  double u = oracle_canonical(st);
  return lower_bound_d(cp, n, u);
}
int oracle_discrete(uint64_t* st, const double* w, int n) {
  double cp[256];
  if (n > 256) return -1;
  make_discrete_cdf(w, n, cp);
  return sample_discrete_cdf(st, cp, n);
}

/* ------------------------------------------------------------ problem */
typedef struct {
  int n;          /* points */
  int off;        /* into ang_pool */
} AngleTab;

typedef struct {
  double distance;
  int surface_index;
  int btype;
  int32_t token;
} Boundary;

typedef struct {
  int est, quantity;
  int N[3];
  double low[3], hi[3], d[3], dinv[3];
  int ne;
  double* eb;
  double* gen; double* avg; double* var;
  size_t nbins;
  int g;
} OTally;

struct oracle_ctx {
  abx_settings set;
  int G;
  double* eb;
  double min_energy, max_energy;
  /* geometry */
  int nsurf; abx_surface* surf;
  int ncell; abx_cell* cell; int32_t** crpn; int* crpn_len; int* csimple; int* chasbc;
  int* creentry; /* universe index that universe_id_to_indx[cell id] yields */
  int nuniv; abx_universe* univ; int* uhasbc;
  double* lat_xl; double* lat_yl; double* lat_zl;   /* shifted low corners */
  double* lat_pxi; double* lat_pyi; double* lat_pzi;
  int32_t* cell_lists; int32_t* lat_elems;
  int root;
  /* materials */
  int M;
  double *Et, *Eabs, *Ef, *nu_tot, *nu_d, *Es, *vEf;
  double *ps_cdf, *chi_cdf;  /* [M][G][G] */
  int* fissile;
  int* n_dg; double** dg_cdf; double** dg_lambda;
  AngleTab* ang; double* ang_mu; double* ang_pdf; double* ang_cdf; int ang_n;
  double* maj;
  double* smp;   /* Carter tracking sampling cross section per group */
  /* tallies */
  int ntally; OTally* tally;
  int ent_on; int ent_shape[3]; double ent_low[3], ent_d[3];
  /* sources */
  int nsrc; abx_source* src; double* src_cdf;
  /* trace */
  uint32_t tr_nhist; size_t tr_cap; size_t tr_n; abx_trace_rec* tr;
  /* source bank to restart power iterations from ([n][9]), or NULL */
  double* restart; size_t n_restart;
  /* status */
  int err;
};

#define MAT_AT(arr, m, g) ((arr)[(size_t)(m) * ctx->G + (g)])

static void* xcalloc(size_t n, size_t s) {
  void* p = calloc(n ? n : 1, s ? s : 1);
  return p;
}

/* ------------------------------------------------------------ surfaces */
/* src/{x,y,z}plane.cpp:32-56, plane.cpp:33-60, {x,y,z}cylinder.cpp:33-80, sphere.cpp:33-80 */
static V3 surf_norm(const abx_surface* s, V3 r) {
  switch (s->type) {
    case ABX_SURF_XPLANE: return dir3(1., 0., 0.);
    case ABX_SURF_YPLANE: return dir3(0., 1., 0.);
    case ABX_SURF_ZPLANE: return dir3(0., 0., 1.);
    case ABX_SURF_PLANE: return dir3(s->c[0], s->c[1], s->c[2]);
    case ABX_SURF_XCYLINDER: return dir3(0., r.y - s->c[0], r.z - s->c[1]);
    case ABX_SURF_YCYLINDER: return dir3(r.x - s->c[0], 0., r.z - s->c[1]);
    case ABX_SURF_ZCYLINDER: return dir3(r.x - s->c[0], r.y - s->c[1], 0.);
    default: return dir3(r.x - s->c[0], r.y - s->c[1], r.z - s->c[2]);
  }
}

static int surf_sign(const abx_surface* s, V3 r, V3 u) {
  double eval;
  switch (s->type) {
    case ABX_SURF_XPLANE: eval = r.x - s->c[0]; break;
    case ABX_SURF_YPLANE: eval = r.y - s->c[0]; break;
    case ABX_SURF_ZPLANE: eval = r.z - s->c[0]; break;
    case ABX_SURF_PLANE:
      eval = s->c[0] * r.x + s->c[1] * r.y + s->c[2] * r.z - s->c[3];
      break;
    case ABX_SURF_XCYLINDER: {
      double y = r.y - s->c[0], z = r.z - s->c[1], R = s->c[2];
      eval = y * y + z * z - R * R;
    } break;
    case ABX_SURF_YCYLINDER: {
      double x = r.x - s->c[0], z = r.z - s->c[1], R = s->c[2];
      eval = x * x + z * z - R * R;
    } break;
    case ABX_SURF_ZCYLINDER: {
      double x = r.x - s->c[0], y = r.y - s->c[1], R = s->c[2];
      eval = y * y + x * x - R * R;
    } break;
    default: {
      double x = r.x - s->c[0], y = r.y - s->c[1], z = r.z - s->c[2], R = s->c[3];
      eval = (x * x) + (y * y) + (z * z) - R * R;
    } break;
  }
  if (eval > SURFACE_COINCIDENT) return 1;
  if (eval < -SURFACE_COINCIDENT) return -1;
  if (vdot(u, surf_norm(s, r)) > 0.) return 1;
  return -1;
}

static double plane_axis_distance(double diff, double ua, int on_surf) {
  if (on_surf || fabs(diff) < SURFACE_COINCIDENT || ua == 0.) return INF_;
  if (diff / ua < 0.) return INF_;
  return diff / ua;
}

static double quad_distance(double a, double k, double c, double quad, int on_surf) {
  if (quad < 0.) return INF_;
  if (on_surf || fabs(c) < SURFACE_COINCIDENT) {
    if (k >= 0.) return INF_;
    return (-k + sqrt(quad)) / a;
  }
  if (c < 0.) return (-k + sqrt(quad)) / a;
  double d = (-k - sqrt(quad)) / a;
  if (d < 0.) return INF_;
  return d;
}

static double surf_distance(const abx_surface* s, V3 r, V3 u, int on_surf) {
  switch (s->type) {
    case ABX_SURF_XPLANE: return plane_axis_distance(s->c[0] - r.x, u.x, on_surf);
    case ABX_SURF_YPLANE: return plane_axis_distance(s->c[0] - r.y, u.y, on_surf);
    case ABX_SURF_ZPLANE: return plane_axis_distance(s->c[0] - r.z, u.z, on_surf);
    case ABX_SURF_PLANE: {
      double A = s->c[0], B = s->c[1], C = s->c[2], D = s->c[3];
      double num = D - A * r.x - B * r.y - C * r.z;
      double denom = A * u.x + B * u.y + C * u.z;
      double d = num / denom;
      if (on_surf || fabs(d) < SURFACE_COINCIDENT || denom == 0.) return INF_;
      if (d < 0.) return INF_;
      return d;
    }
    case ABX_SURF_XCYLINDER: {
      double a = u.y * u.y + u.z * u.z;
      if (a == 0.) return INF_;
      double y = r.y - s->c[0], z = r.z - s->c[1], R = s->c[2];
      double k = y * u.y + z * u.z;
      double c = y * y + z * z - R * R;
      double quad = k * k - a * c;
      return quad_distance(a, k, c, quad, on_surf);
    }
    case ABX_SURF_YCYLINDER: {
      double a = u.x * u.x + u.z * u.z;
      if (a == 0.) return INF_;
      double x = r.x - s->c[0], z = r.z - s->c[1], R = s->c[2];
      double k = x * u.x + z * u.z;
      double c = x * x + z * z - R * R;
      double quad = k * k - a * c;
      return quad_distance(a, k, c, quad, on_surf);
    }
    case ABX_SURF_ZCYLINDER: {
      double a = u.y * u.y + u.x * u.x;
      if (a == 0.) return INF_;
      double x = r.x - s->c[0], y = r.y - s->c[1], R = s->c[2];
      double k = y * u.y + x * u.x;
      double c = y * y + x * x - R * R;
      double quad = k * k - a * c;
      return quad_distance(a, k, c, quad, on_surf);
    }
    default: {
      double x = r.x - s->c[0], y = r.y - s->c[1], z = r.z - s->c[2], R = s->c[3];
      double k = x * u.x + y * u.y + z * u.z;
      double c = x * x + y * y + z * z - R * R;
      double quad = k * k - c;
      if (quad < 0.) return INF_;
      if (on_surf || fabs(c) < SURFACE_COINCIDENT) {
        if (k >= 0.) return INF_;
        return -k + sqrt(quad);
      }
      if (c < 0.) return -k + sqrt(quad);
      double d = -k - sqrt(quad);
      if (d < 0.) return INF_;
      return d;
    }
  }
}

/* ---------------------------------------------------------------- cells */
/* Cell::is_inside_simple / is_inside_complex (src/cell.cpp:147-199) */
static int cell_is_inside(oracle_ctx* ctx, int ci, V3 r, V3 u, int32_t on_surf) {
  const int32_t* rpn = ctx->crpn[ci];
  int n = ctx->crpn_len[ci];
  if (ctx->csimple[ci]) {
    for (int i = 0; i < n; i++) {
      int32_t t = rpn[i];
      if (t == on_surf) {
      } else if (-t == on_surf) {
        return 0;
      } else {
        int sg = surf_sign(&ctx->surf[abs(t) - 1], r, u);
        if ((sg > 0 && t < 0) || (sg < 0 && t > 0)) return 0;
      }
    }
    return 1;
  }
  unsigned char stck[256];
  int i_st = -1;
  for (int i = 0; i < n; i++) {
    int32_t t = rpn[i];
    if (t == ABX_OP_UNIN) {
      stck[i_st - 1] = stck[i_st - 1] || stck[i_st];
      i_st--;
    } else if (t == ABX_OP_INTR) {
      stck[i_st - 1] = stck[i_st - 1] && stck[i_st];
      i_st--;
    } else if (t == ABX_OP_COMP) {
      stck[i_st] = !stck[i_st];
    } else {
      i_st++;
      if (t == on_surf) stck[i_st] = 1;
      else if (-t == on_surf) stck[i_st] = 0;
      else {
        int sg = surf_sign(&ctx->surf[abs(t) - 1], r, u);
        stck[i_st] = ((sg > 0 && t > 0) || (sg < 0 && t < 0)) ? 1 : 0;
      }
    }
  }
  if (i_st == 0) return stck[0];
  return 1;
}

/* Cell::distance_to_boundary (src/cell.cpp:79-106) and
 * distance_to_boundary_condition (src/cell.cpp:108-141) */
static void cell_distance(oracle_ctx* ctx, int ci, V3 r, V3 u, int32_t on_surf,
                          int bc_only, double* dist, int32_t* isurf) {
  double min_dist = INF_;
  int32_t i_surf = 0;
  if (bc_only && !ctx->chasbc[ci]) {
    *dist = INF_;
    *isurf = 0;
    return;
  }
  const int32_t* rpn = ctx->crpn[ci];
  for (int i = 0; i < ctx->crpn_len[ci]; i++) {
    int32_t t = rpn[i];
    if (t >= ABX_OP_UNIN) continue;
    int coincident = abs(t) == abs(on_surf);
    const abx_surface* s = &ctx->surf[abs(t) - 1];
    if (bc_only && s->bc == ABX_BC_NORMAL) continue;
    double d = surf_distance(s, r, u, coincident);
    if (d < min_dist) {
      if (fabs(d - min_dist) / min_dist >= 1e-14) {
        min_dist = d;
        i_surf = -t;
      }
    }
  }
  *dist = min_dist;
  *isurf = i_surf;
}

/* ------------------------------------------------------------ lattices */
/* RectLattice::tile_center (src/rect_lattice.cpp:304-310) */
static V3 tile_center(oracle_ctx* ctx, int li, int nx, int ny, int nz) {
  const abx_universe* L = &ctx->univ[li];
  double x = ((double)nx + 0.5) * L->pitch[0] + ctx->lat_xl[li];
  double y = ((double)ny + 0.5) * L->pitch[1] + ctx->lat_yl[li];
  double z = ((double)nz + 0.5) * L->pitch[2] + ctx->lat_zl[li];
  return v3(x, y, z);
}
/* RectLattice::get_tile (src/rect_lattice.cpp:207-237) */
static void get_tile(oracle_ctx* ctx, int li, V3 r, V3 u, int t[3]) {
  const abx_universe* L = &ctx->univ[li];
  int32_t nx = (int32_t)floor((r.x - ctx->lat_xl[li]) * ctx->lat_pxi[li]);
  int32_t ny = (int32_t)floor((r.y - ctx->lat_yl[li]) * ctx->lat_pyi[li]);
  int32_t nz = (int32_t)floor((r.z - ctx->lat_zl[li]) * ctx->lat_pzi[li]);
  V3 rt = tile_center(ctx, li, nx, ny, nz);
  double Px = L->pitch[0], Py = L->pitch[1], Pz = L->pitch[2];
  double xl = rt.x - Px * 0.5;
  if (fabs(xl - r.x) < SURFACE_COINCIDENT && u.x < 0.) nx--;
  double xh = rt.x + Px * 0.5;
  if (fabs(xh - r.x) < SURFACE_COINCIDENT && u.x >= 0.) nx++;
  double yl = rt.y - Py * 0.5;
  if (fabs(yl - r.y) < SURFACE_COINCIDENT && u.y < 0.) ny--;
  double yh = rt.y + Py * 0.5;
  if (fabs(yh - r.y) < SURFACE_COINCIDENT && u.y >= 0.) ny++;
  double zl = rt.z - Pz * 0.5;
  if (fabs(zl - r.z) < SURFACE_COINCIDENT && u.z < 0.) nz--;
  double zh = rt.z + Pz * 0.5;
  if (fabs(zh - r.z) < SURFACE_COINCIDENT && u.z >= 0.) nz++;
  t[0] = nx; t[1] = ny; t[2] = nz;
}
/* RectLattice::distance_to_tile_boundary (src/rect_lattice.cpp:239-282) */
static double dist_to_tile(oracle_ctx* ctx, int li, V3 rl, V3 u, const int t[3]) {
  const abx_universe* L = &ctx->univ[li];
  V3 c = tile_center(ctx, li, t[0], t[1], t[2]);
  V3 rt = vsub(rl, c);
  double dist = INF_;
  double Px = L->pitch[0], Py = L->pitch[1], Pz = L->pitch[2];
  const double diff_xl = -Px * 0.5 - rt.x;
  const double diff_xh = Px * 0.5 - rt.x;
  const double diff_yl = -Py * 0.5 - rt.y;
  const double diff_yh = Py * 0.5 - rt.y;
  const double diff_zl = -Pz * 0.5 - rt.z;
  const double diff_zh = Pz * 0.5 - rt.z;
  const double ux_inv = 1. / u.x, uy_inv = 1. / u.y, uz_inv = 1. / u.z;
  const double d_xl = diff_xl * ux_inv, d_xh = diff_xh * ux_inv;
  const double d_yl = diff_yl * uy_inv, d_yh = diff_yh * uy_inv;
  const double d_zl = diff_zl * uz_inv, d_zh = diff_zh * uz_inv;
  if (d_xl > 0. && d_xl < dist && fabs(diff_xl) > TILE_TOL_) dist = d_xl;
  if (d_xh > 0. && d_xh < dist && fabs(diff_xh) > TILE_TOL_) dist = d_xh;
  if (d_yl > 0. && d_yl < dist && fabs(diff_yl) > TILE_TOL_) dist = d_yl;
  if (d_yh > 0. && d_yh < dist && fabs(diff_yh) > TILE_TOL_) dist = d_yh;
  if (d_zl > 0. && d_zl < dist && fabs(diff_zl) > TILE_TOL_) dist = d_zl;
  if (d_zh > 0. && d_zh < dist && fabs(diff_zh) > TILE_TOL_) dist = d_zh;
  return dist;
}

/* ---------------------------------------------------------------- tree */
enum { PAD_UNIV = 0, PAD_LATT = 1, PAD_CELL = 2 };
typedef struct {
  int type, idx;
  V3 r;
  int tile[3];
} Pad;

typedef struct {
  V3 r, u;
  int32_t token;
  Pad tree[MAXPADS];
  int depth;
  int cell; /* current material cell, -1 lost */
} Tracker;

static int push_pad(oracle_ctx* ctx, Tracker* t, int type, int idx, V3 r, const int* tile) {
  if (t->depth >= MAXPADS) {
    ctx->err = ABX_ERR_INVALID;
    set_err("geometry tree deeper than %d levels", MAXPADS);
    return 0;
  }
  Pad* p = &t->tree[t->depth++];
  p->type = type; p->idx = idx; p->r = r;
  p->tile[0] = tile ? tile[0] : 0;
  p->tile[1] = tile ? tile[1] : 0;
  p->tile[2] = tile ? tile[2] : 0;
  return 1;
}

/* CellUniverse::get_cell(stack,...) (src/cell_universe.cpp:69-104) and
 * RectLattice::get_cell(stack,...) (src/rect_lattice.cpp:131-205) */
static int univ_get_cell(oracle_ctx* ctx, int ui, Tracker* t, V3 r, V3 u, int32_t on_surf) {
  for (int guard = 0; guard < 64; guard++) {
    const abx_universe* U = &ctx->univ[ui];
    if (U->kind == ABX_UNIV_CELLS) {
      if (!push_pad(ctx, t, PAD_UNIV, ui, r, NULL)) return -1;
      int found = -1;
      for (int k = 0; k < U->list_len; k++) {
        int ci = ctx->cell_lists[U->list_offset + k];
        if (cell_is_inside(ctx, ci, r, u, on_surf)) { found = ci; break; }
      }
      if (found < 0) return -1;
      if (!push_pad(ctx, t, PAD_CELL, found, r, NULL)) return -1;
      if (ctx->cell[found].fill_kind == ABX_FILL_MATERIAL) return found;
      ui = ctx->cell[found].fill;
      continue;
    }
    int tl[3];
    get_tile(ctx, ui, r, u, tl);
    int Nx = U->shape[0], Ny = U->shape[1], Nz = U->shape[2];
    int inside = !(tl[0] < 0 || tl[0] >= Nx || tl[1] < 0 || tl[1] >= Ny || tl[2] < 0 || tl[2] >= Nz);
    int fill = -1;
    if (inside) {
      size_t lin = (size_t)((uint32_t)tl[2] * ((uint32_t)Nx * (uint32_t)Ny) + (uint32_t)tl[0] * (uint32_t)Ny + (uint32_t)tl[1]);
      fill = ctx->lat_elems[U->list_offset + lin];
    }
    if (fill >= 0) {
      V3 rl = vsub(r, tile_center(ctx, ui, tl[0], tl[1], tl[2]));
      if (!push_pad(ctx, t, PAD_LATT, ui, r, tl)) return -1;
      r = rl;
      ui = fill;
      continue;
    }
    if (!push_pad(ctx, t, PAD_LATT, ui, r, tl)) return -1;
    if (U->outer >= 0) {
      ui = U->outer;
      continue;
    }
    return -1;
  }
  ctx->err = ABX_ERR_INVALID;
  set_err("universe nesting too deep");
  return -1;
}

/* CellUniverse::get_boundary_condition (src/cell_universe.cpp:107-147),
 * Lattice::get_boundary_condition (src/lattice.cpp:77-91) */
static Boundary univ_get_bc(oracle_ctx* ctx, int ui, V3 r, V3 u, int32_t on_surf) {
  Boundary b = {INF_, -1, ABX_BC_VACUUM, 0};
  for (int guard = 0; guard < 64; guard++) {
    const abx_universe* U = &ctx->univ[ui];
    if (U->kind == ABX_UNIV_RECT_LATTICE) {
      if (ctx->uhasbc[ui]) { ui = U->outer; continue; }
      return b;
    }
    if (ctx->uhasbc[ui]) {
      for (int k = 0; k < U->list_len; k++) {
        int ci = ctx->cell_lists[U->list_offset + k];
        if (!ctx->chasbc[ci]) continue;
        double d; int32_t ts;
        cell_distance(ctx, ci, r, u, on_surf, 1, &d, &ts);
        if (d < b.distance && fabs(d - b.distance) > BOUNDRY_TOL_) {
          int32_t tmp = abs(ts);
          if (tmp) {
            b.token = tmp;
            b.distance = d;
            b.surface_index = tmp - 1;
          } else {
            continue;
          }
          b.btype = ctx->surf[b.surface_index].bc;
          if (surf_sign(&ctx->surf[b.surface_index], r, u) < 0) b.token *= -1;
        }
      }
    }
    return b;
  }
  return b;
}

/* Tracker::restart_get_current (include/simulation/tracker.hpp:59-71) */
static void trk_restart(oracle_ctx* ctx, Tracker* t) {
  t->depth = 0;
  t->cell = univ_get_cell(ctx, ctx->root, t, t->r, t->u, t->token);
}
/* Tracker ctor (tracker.hpp:43-50) */
static void trk_init(oracle_ctx* ctx, Tracker* t, V3 r, V3 u) {
  t->r = r; t->u = u; t->token = 0;
  trk_restart(ctx, t);
}
/* Tracker::move (tracker.hpp:76-85) */
static void trk_move(Tracker* t, double d) {
  t->r = vadd(t->r, vscale(t->u, d));
  for (int k = 0; k < t->depth; k++) t->tree[k].r = vadd(t->tree[k].r, vscale(t->u, d));
  t->token = 0;
}
static void trk_set_r(Tracker* t, V3 r) { t->r = r; t->token = 0; }
static int trk_check_tree(const Tracker* t) {
  return t->r.x == t->tree[0].r.x && t->r.y == t->tree[0].r.y && t->r.z == t->tree[0].r.z;
}
/* Tracker::get_current (tracker.hpp:235-306) */
static void trk_get_current(oracle_ctx* ctx, Tracker* t) {
  if (!trk_check_tree(t)) {
    trk_restart(ctx, t);
    if (!trk_check_tree(t)) {
      ctx->err = ABX_ERR_LOST_PARTICLE;
      set_err("BAD POSITIONS in get_current");
      return;
    }
  }
  int first_bad = t->depth;
  for (int k = 0; k < t->depth; k++) {
    Pad* p = &t->tree[k];
    if (p->type == PAD_CELL) {
      if (!cell_is_inside(ctx, p->idx, p->r, t->u, t->token)) { first_bad = k; break; }
    } else if (p->type == PAD_LATT) {
      int tl[3];
      get_tile(ctx, p->idx, p->r, t->u, tl);
      if (p->tile[0] != tl[0] || p->tile[1] != tl[1] || p->tile[2] != tl[2]) { first_bad = k; break; }
    }
  }
  if (first_bad == t->depth) return;
  if (first_bad == 0) { trk_restart(ctx, t); return; }
  t->depth = first_bad;
  Pad back = t->tree[t->depth - 1];
  /* universe_id_to_indx[tree.back().id]: for a Cell pad this looks a universe
   * up by the cell's id (std::map::operator[] yields index 0 when absent). */
  int ui = back.type == PAD_CELL ? ctx->creentry[back.idx] : back.idx;
  t->depth--;
  t->cell = univ_get_cell(ctx, ui, t, back.r, t->u, t->token);
  if (t->cell < 0) trk_restart(ctx, t);
}
/* Tracker::get_boundary_condition (tracker.hpp:94-161) */
static Boundary trk_get_bc(oracle_ctx* ctx, const Tracker* t) {
  if (t->cell < 0) return univ_get_bc(ctx, ctx->root, t->r, t->u, t->token);
  Boundary b = {INF_, -1, ABX_BC_VACUUM, 0};
  for (int k = 0; k < t->depth; k++) {
    const Pad* p = &t->tree[k];
    if (p->type == PAD_CELL) {
      if (!ctx->chasbc[p->idx]) continue;
      double d; int32_t ts;
      cell_distance(ctx, p->idx, p->r, t->u, t->token, 1, &d, &ts);
      if (d < b.distance && fabs(d - b.distance) > BOUNDRY_TOL_) {
        int32_t tmp = abs(ts);
        if (tmp) {
          b.distance = d;
          b.token = tmp;
          b.surface_index = tmp - 1;
        } else {
          continue;
        }
        b.btype = ctx->surf[b.surface_index].bc;
        if (surf_sign(&ctx->surf[b.surface_index], p->r, t->u) < 0) b.token *= -1;
      }
    } else {
      if (ctx->uhasbc[p->idx]) {
        Boundary ub = univ_get_bc(ctx, p->idx, p->r, t->u, t->token);
        if (ub.distance < b.distance && fabs(ub.distance - b.distance) > BOUNDRY_TOL_) {
          b = ub;
        }
      }
    }
  }
  return b;
}
/* Tracker::get_nearest_boundary (tracker.hpp:163-225) */
static Boundary trk_nearest(oracle_ctx* ctx, const Tracker* t) {
  if (t->cell < 0) {
    ctx->err = ABX_ERR_LOST_PARTICLE;
    set_err("nearest boundary asked of a lost tracker");
    Boundary b = {INF_, -1, ABX_BC_VACUUM, 0};
    return b;
  }
  Boundary b = trk_get_bc(ctx, t);
  for (int k = 0; k < t->depth; k++) {
    const Pad* p = &t->tree[k];
    if (p->type == PAD_LATT) {
      double d = dist_to_tile(ctx, p->idx, p->r, t->u, p->tile);
      if (d < b.distance && fabs(d - b.distance) > BOUNDRY_TOL_) {
        b.distance = d;
        b.btype = ABX_BC_NORMAL;
        b.surface_index = -1;
        b.token = 0;
      }
    } else if (p->type == PAD_CELL) {
      double d; int32_t ts;
      cell_distance(ctx, p->idx, p->r, t->u, t->token, 0, &d, &ts);
      if (d < b.distance && fabs(d - b.distance) > BOUNDRY_TOL_) {
        b.distance = d;
        b.token = abs(ts);
        b.surface_index = b.token ? b.token - 1 : -1;
        b.btype = b.surface_index >= 0 ? ctx->surf[b.surface_index].bc : ABX_BC_NORMAL;
        if (b.surface_index >= 0 && surf_sign(&ctx->surf[b.surface_index], p->r, t->u) < 0)
          b.token *= -1;
      }
    }
  }
  return b;
}

/* ------------------------------------------------------------ particle */
typedef struct {
  V3 r, u;
  double E, w, w2;
} PState;

typedef struct {
  PState s;
  uint64_t rng;
  uint64_t hid, family;
  V3 r_birth;
  int alive;
  uint64_t daughter;
  PState* sec; int nsec, capsec;
} Part;

typedef struct {
  double k_col, k_abs, k_trk, k_tot, leak, mig;
  uint64_t coll, flights, lost;
} Scores;

typedef struct {
  abx_site* v; size_t n, cap;
  uint32_t* hist;
} SiteBuf;

typedef struct {
  abx_trace_rec* v; size_t n, cap;
} TraceBuf;

static int group_of(oracle_ctx* ctx, double E) {
  /* MGNuclide::energy_grid_index (src/mg_nuclide.cpp:382-392) */
  int i;
  for (i = 0; i < ctx->G; i++)
    if (ctx->eb[i] <= E && E < ctx->eb[i + 1]) break;
  return i;
}

static void trace(oracle_ctx* ctx, TraceBuf* tb, uint32_t h, int kind, const Part* p, int cell) {
  if (!tb || h >= ctx->tr_nhist) return;
  if (tb->n == tb->cap) {
    size_t nc = tb->cap ? 2 * tb->cap : 1024;
    abx_trace_rec* nv = (abx_trace_rec*)realloc(tb->v, nc * sizeof *nv);
    if (!nv) return;
    tb->v = nv; tb->cap = nc;
  }
  abx_trace_rec* r = &tb->v[tb->n++];
  memset(r, 0, sizeof *r);
  r->hist = h; r->kind = kind;
  r->group = group_of(ctx, p->s.E);
  r->cell = cell;
  r->rng_state = p->rng;
  r->r[0] = p->s.r.x; r->r[1] = p->s.r.y; r->r[2] = p->s.r.z;
  r->u[0] = p->s.u.x; r->u[1] = p->s.u.y; r->u[2] = p->s.u.z;
  r->wgt = p->s.w;
}

static int site_push(SiteBuf* sb, uint32_t h, const abx_site* s) {
  if (sb->n == sb->cap) {
    size_t nc = sb->cap ? 2 * sb->cap : 4096;
    abx_site* nv = (abx_site*)realloc(sb->v, nc * sizeof *nv);
    uint32_t* nh = (uint32_t*)realloc(sb->hist, nc * sizeof *nh);
    if (!nv || !nh) return 0;
    sb->v = nv; sb->hist = nh; sb->cap = nc;
  }
  sb->v[sb->n] = *s;
  sb->hist[sb->n] = h;
  sb->n++;
  return 1;
}

static int sec_push(Part* p, PState s) {
  if (p->nsec == p->capsec) {
    int nc = p->capsec ? 2 * p->capsec : 8;
    PState* nv = (PState*)realloc(p->sec, (size_t)nc * sizeof *nv);
    if (!nv) return 0;
    p->sec = nv; p->capsec = nc;
  }
  p->sec[p->nsec++] = s;
  return 1;
}

/* ------------------------------------------------------------- tallies */
static int ebin(const OTally* T, double E) {
  for (int e = 0; e < T->ne; e++)
    if (T->eb[e] <= E && E <= T->eb[e + 1]) return e;
  return -1;
}

static double quantity_factor(oracle_ctx* ctx, int q, int mat, int g, double w) {
  switch (q) {
    case ABX_Q_ELASTIC: return w * MAT_AT(ctx->Es, mat, g);
    case ABX_Q_ABSORPTION: return w * MAT_AT(ctx->Eabs, mat, g);
    case ABX_Q_FISSION: return w * MAT_AT(ctx->Ef, mat, g);
    case ABX_Q_TOTAL: return w * MAT_AT(ctx->Et, mat, g);
    default: return w;
  }
}

static void tally_add(double* a, double v) {
#ifdef _OPENMP
#pragma omp atomic
#endif
  *a += v;
}

/* CollisionMeshTally::score_collision (src/collision_mesh_tally.cpp:33-108) */
static void score_collision(oracle_ctx* ctx, const Part* p, int mat) {
  for (int ti = 0; ti < ctx->ntally; ti++) {
    OTally* T = &ctx->tally[ti];
    if (T->est != ABX_EST_COLLISION) continue;
    int g = group_of(ctx, p->s.E);
    double Et = MAT_AT(ctx->Et, mat, g);
    double scr = 1. / (Et * ctx->set.nparticles);
    int i = (int)floor((p->s.r.x - T->low[0]) * T->dinv[0]);
    int j = (int)floor((p->s.r.y - T->low[1]) * T->dinv[1]);
    int k = (int)floor((p->s.r.z - T->low[2]) * T->dinv[2]);
    int l = ebin(T, p->s.E);
    if (l == -1) continue;
    if (i >= 0 && i < T->N[0] && j >= 0 && j < T->N[1] && k >= 0 && k < T->N[2]) {
      scr *= quantity_factor(ctx, T->quantity, mat, g, p->s.w);
      size_t idx = (((size_t)l * T->N[0] + i) * T->N[1] + j) * T->N[2] + k;
      tally_add(&T->gen[idx], scr);
    }
  }
}

/* TrackLengthMeshTally::initialize_indices (src/track_length_mesh_tally.cpp:249-317) */
static void tle_init_idx(const OTally* T, V3 r, V3 u, int* i, int* j, int* k, int on[3]) {
  *i = (int)floor((r.x - T->low[0]) * T->dinv[0]);
  *j = (int)floor((r.y - T->low[1]) * T->dinv[1]);
  *k = (int)floor((r.z - T->low[2]) * T->dinv[2]);
  on[0] = on[1] = on[2] = 0;
  double dx = T->d[0], dy = T->d[1], dz = T->d[2];
  double xc = T->low[0] + *i * dx + 0.5 * dx;
  double yc = T->low[1] + *j * dy + 0.5 * dy;
  double zc = T->low[2] + *k * dz + 0.5 * dz;
  double xl = xc - 0.5 * dx, xh = xc + 0.5 * dx;
  double yl = yc - 0.5 * dy, yh = yc + 0.5 * dy;
  double zl = zc - 0.5 * dz, zh = zc + 0.5 * dz;
  if (fabs(xl - r.x) < SURFACE_COINCIDENT) {
    if (u.x < 0.) { (*i)--; on[0] = 1; } else { on[0] = -1; }
  } else if (fabs(xh - r.x) < SURFACE_COINCIDENT) {
    if (u.x < 0.) { on[0] = 1; } else { (*i)++; on[0] = -1; }
  }
  if (fabs(yl - r.y) < SURFACE_COINCIDENT) {
    if (u.y < 0.) { (*j)--; on[1] = 1; } else { on[1] = -1; }
  } else if (fabs(yh - r.y) < SURFACE_COINCIDENT) {
    if (u.y < 0.) { on[1] = 1; } else { (*j)++; on[1] = -1; }
  }
  if (fabs(zl - r.z) < SURFACE_COINCIDENT) {
    if (u.z < 0.) { (*k)--; on[2] = 1; } else { on[2] = -1; }
  } else if (fabs(zh - r.z) < SURFACE_COINCIDENT) {
    if (u.z < 0.) { on[2] = 1; } else { (*k)++; on[2] = -1; }
  }
}
/* TrackLengthMeshTally::find_entry_point (src/track_length_mesh_tally.cpp:185-247) */
static int tle_entry(const OTally* T, V3* r, V3 u, double* dfl) {
  const double uxi = 1. / u.x, uyi = 1. / u.y, uzi = 1. / u.z;
  double dmin = (T->low[0] - r->x) * uxi, dmax = (T->hi[0] - r->x) * uxi, tmp;
  if (dmin > dmax) { tmp = dmin; dmin = dmax; dmax = tmp; }
  double dymin = (T->low[1] - r->y) * uyi, dymax = (T->hi[1] - r->y) * uyi;
  if (dymin > dymax) { tmp = dymin; dymin = dymax; dymax = tmp; }
  if ((dmin > dymax) || (dymin > dmax)) return 0;
  if (dymin > dmin) dmin = dymin;
  if (dymax < dmax) dmax = dymax;
  double dzmin = (T->low[2] - r->z) * uzi, dzmax = (T->hi[2] - r->z) * uzi;
  if (dzmin > dzmax) { tmp = dzmin; dzmin = dzmax; dzmax = tmp; }
  if ((dmin > dzmax) || (dzmin > dmax)) return 0;
  if (dzmin > dmin) dmin = dzmin;
  if (dzmax < dmax) dmax = dzmax;
  if (dmax < dmin) { tmp = dmax; dmax = dmin; dmin = tmp; }
  if ((dmax < 0.) && (dmin < 0.)) return 0;
  if (dmin < 0.) return 0;
  *r = vadd(*r, vscale(u, dmin));
  *dfl -= dmin;
  return 1;
}
/* TrackLengthMeshTally::distance_to_next_index (src/track_length_mesh_tally.cpp:319-385) */
static double tle_next(const OTally* T, V3 r, V3 u, int i, int j, int k, const int on[3], int* key) {
  double dx = T->d[0], dy = T->d[1], dz = T->d[2];
  double xc = T->low[0] + i * dx + 0.5 * dx;
  double yc = T->low[1] + j * dy + 0.5 * dy;
  double zc = T->low[2] + k * dz + 0.5 * dz;
  V3 rt = v3(r.x - xc, r.y - yc, r.z - zc);
  double dist = INF_;
  *key = 0;
  const double diff_xl = -dx * 0.5 - rt.x, diff_xh = dx * 0.5 - rt.x;
  const double diff_yl = -dy * 0.5 - rt.y, diff_yh = dy * 0.5 - rt.y;
  const double diff_zl = -dz * 0.5 - rt.z, diff_zh = dz * 0.5 - rt.z;
  const double uxi = 1. / u.x, uyi = 1. / u.y, uzi = 1. / u.z;
  const double d_xl = diff_xl * uxi, d_xh = diff_xh * uxi;
  const double d_yl = diff_yl * uyi, d_yh = diff_yh * uyi;
  const double d_zl = diff_zl * uzi, d_zh = diff_zh * uzi;
  if (d_xl > 0. && d_xl < dist && on[0] != -1) { dist = d_xl; *key = -1; }
  if (d_xh > 0. && d_xh < dist && on[0] != 1) { dist = d_xh; *key = 1; }
  if (d_yl > 0. && d_yl < dist && on[1] != -1) { dist = d_yl; *key = -2; }
  if (d_yh > 0. && d_yh < dist && on[1] != 1) { dist = d_yh; *key = 2; }
  if (d_zl > 0. && d_zl < dist && on[2] != -1) { dist = d_zl; *key = -3; }
  if (d_zh > 0. && d_zh < dist && on[2] != 1) { dist = d_zh; *key = 3; }
  return dist;
}
/* TrackLengthMeshTally::score_flight (src/track_length_mesh_tally.cpp:77-183) */
static void score_flight(oracle_ctx* ctx, const Part* p, double d, int mat) {
  for (int ti = 0; ti < ctx->ntally; ti++) {
    OTally* T = &ctx->tally[ti];
    if (T->est != ABX_EST_TRACK_LENGTH) continue;
    V3 r = p->s.r, u = p->s.u;
    int i, j, k, on[3];
    double dd = d;
    tle_init_idx(T, r, u, &i, &j, &k, on);
    int inside = i >= 0 && i < T->N[0] && j >= 0 && j < T->N[1] && k >= 0 && k < T->N[2];
    if (!inside) {
      if (!tle_entry(T, &r, u, &dd)) continue;
      tle_init_idx(T, r, u, &i, &j, &k, on);
    }
    int g = group_of(ctx, p->s.E);
    double base = 1. / ctx->set.nparticles;
    base *= quantity_factor(ctx, T->quantity, mat, g, p->s.w);
    int l = ebin(T, p->s.E);
    if (l == -1) continue;
    double rem = dd;
    while (rem > 0.) {
      int key;
      double nt = tle_next(T, r, u, i, j, k, on, &key);
      if (nt == INF_) break;
      double dt = nt < rem ? nt : rem;
      if (i >= 0 && i < T->N[0] && j >= 0 && j < T->N[1] && k >= 0 && k < T->N[2]) {
        size_t idx = (((size_t)l * T->N[0] + i) * T->N[1] + j) * T->N[2] + k;
        tally_add(&T->gen[idx], dt * base);
      } else {
        break;
      }
      rem -= dt;
      if (rem <= 0.) break;
      r = vadd(r, vscale(u, dt));
      on[0] = on[1] = on[2] = 0;
      switch (key) {
        case -1: i--; on[0] = 1; break;
        case 1: i++; on[0] = -1; break;
        case -2: j--; on[1] = 1; break;
        case 2: j++; on[1] = -1; break;
        case -3: k--; on[2] = 1; break;
        case 3: k++; on[2] = -1; break;
        default: break;
      }
    }
  }
}

/* ------------------------------------------------------------- physics */
/* MGAngleDistribution::sample_mu (include/materials/mg_angle_distribution.hpp:45-60,92-101) */
static double sample_mu(oracle_ctx* ctx, int mat, int gi, int go, uint64_t* rng) {
  const AngleTab* a = &ctx->ang[((size_t)mat * ctx->G + gi) * ctx->G + go];
  const double* mu = ctx->ang_mu + a->off;
  const double* pdf = ctx->ang_pdf + a->off;
  const double* cdf = ctx->ang_cdf + a->off;
  const double xi = oracle_canonical(rng);
  int l = lower_bound_d(cdf, a->n, xi);
  if (xi == cdf[l]) return mu[l];
  l--;
  if (pdf[l] == pdf[l + 1]) return mu[l] + ((xi - cdf[l]) / pdf[l]);
  double m = (pdf[l + 1] - pdf[l]) / (mu[l + 1] - mu[l]);
  return mu[l] + (1. / m) * (sqrt(pdf[l] * pdf[l] + 2. * m * (xi - cdf[l])) - pdf[l]);
}

static double group_mid(oracle_ctx* ctx, int g) { return 0.5 * (ctx->eb[g] + ctx->eb[g + 1]); }

/* Transporter::russian_roulette (src/transporter.cpp:35-58) */
static void russian_roulette(oracle_ctx* ctx, Part* p) {
  if (fabs(p->s.w) < ctx->set.wgt_cutoff) {
    double P_kill = 1.0 - (fabs(p->s.w) / ctx->set.wgt_survival);
    if (oracle_canonical(&p->rng) < P_kill) p->s.w = 0.;
    else p->s.w = copysign(ctx->set.wgt_survival, p->s.w);
  }
  if (fabs(p->s.w2) < ctx->set.wgt_cutoff) {
    double P_kill = 1.0 - (fabs(p->s.w2) / ctx->set.wgt_survival);
    if (oracle_canonical(&p->rng) < P_kill) p->s.w2 = 0.;
    else p->s.w2 = copysign(ctx->set.wgt_survival, p->s.w2);
  }
  if (p->s.w == 0. && p->s.w2 == 0.) p->alive = 0;
}

/* Transporter::branchless_collision_iso / branchless_collision_mat
 * (src/transporter.cpp:95-267), after Transporter::collision's scores: the
 * collision scatters with the weight multiplied by m, or ends the history in
 * one fission site of weight w m.  Splitting: Particle::split
 * (include/simulation/particle.hpp:165-173). */
static int branchless_collision(oracle_ctx* ctx, Part* p, int mat, int g, Scores* sc, SiteBuf* sb, uint32_t h) {
  const int G = ctx->G;
  const double Et = MAT_AT(ctx->Et, mat, g);
  const double Eabs = MAT_AT(ctx->Eabs, mat, g);
  const double Ef = MAT_AT(ctx->Ef, mat, g);
  const double nu = MAT_AT(ctx->nu_tot, mat, g);
  const int per_mat = (ctx->set.branchless & ABX_BRANCHLESS_MATERIAL) != 0;
  const int splitting = (ctx->set.branchless & ABX_BRANCHLESS_SPLITTING) != 0;
  const double wgt_split = ctx->set.wgt_split > 0. ? ctx->set.wgt_split : 2.0;
  int scatter;
  double m;
  if (per_mat) {
    /* branchless_collision_mat (src/transporter.cpp:185-267) */
    const double Es = MAT_AT(ctx->Es, mat, g);
    const double vEf = MAT_AT(ctx->vEf, mat, g);
    const double Pscatter = Es / (vEf + Es);
    m = (vEf + Es) / Et;
    scatter = oracle_canonical(&p->rng) < Pscatter;
    (void)oracle_canonical(&p->rng); /* sample_branchless_nuclide (material_helper.hpp:226-271) */
    const double m_i = (nu * Ef + (Et - Eabs)) / Et;
    sc->k_abs += (m / m_i) * p->s.w * nu * Ef / Et;
    russian_roulette(ctx, p);
    if (!p->alive) return ABX_OK;
  } else {
    /* branchless_collision_iso (src/transporter.cpp:104-183) */
    (void)oracle_canonical(&p->rng); /* sample_nuclide */
    sc->k_abs += p->s.w * nu * Ef / Et;
    const double Pscatter = (Et - Eabs) / (nu * Ef + (Et - Eabs));
    m = (nu * Ef + (Et - Eabs)) / Et;
    russian_roulette(ctx, p);
    if (!p->alive) return ABX_OK;
    scatter = oracle_canonical(&p->rng) < Pscatter;
  }
  if (scatter) {
    int ei = sample_discrete_cdf(&p->rng, ctx->ps_cdf + ((size_t)mat * G + g) * G, G);
    double E_out = group_mid(ctx, ei);
    double mu = sample_mu(ctx, mat, g, ei, &p->rng);
    double phi = 2. * PI_ * oracle_canonical(&p->rng);
    p->s.E = E_out;
    p->s.u = rotate_direction(p->s.u, mu, phi);
    p->s.w = p->s.w * m * 1.;
    p->s.w2 = p->s.w2 * m * 1.;
    if (p->s.E < ctx->min_energy) p->alive = 0;
    if (splitting && p->alive && fabs(p->s.w) >= wgt_split) {
      int n_new = per_mat ? (int)ceil(fabs(p->s.w)) : (int)floor(fabs(p->s.w));
      if (n_new > 1) {
        p->s.w = p->s.w / (double)n_new;
        p->s.w2 = p->s.w2 / (double)n_new;
        for (int k = 0; k < n_new - 1; k++)
          if (!sec_push(p, p->s)) { set_err("out of memory"); return ABX_ERR_OOM; }
      }
    }
  } else {
    /* MGNuclide::sample_fission (src/mg_nuclide.cpp:504-544), one neutron */
    double P_delayed = MAT_AT(ctx->nu_d, mat, g) / nu;
    int ei = sample_discrete_cdf(&p->rng, ctx->chi_cdf + ((size_t)mat * G + g) * G, G);
    double E_out = group_mid(ctx, ei);
    double mu = 2. * oracle_canonical(&p->rng) - 1.;
    double phi = 2. * PI_ * oracle_canonical(&p->rng);
    V3 uout = rotate_direction(p->s.u, mu, phi);
    if (oracle_canonical(&p->rng) < P_delayed) (void)sample_discrete_cdf(&p->rng, ctx->dg_cdf[mat], ctx->n_dg[mat]);
    abx_site s;
    s.r[0] = p->s.r.x; s.r[1] = p->s.r.y; s.r[2] = p->s.r.z;
    s.u[0] = uout.x; s.u[1] = uout.y; s.u[2] = uout.z;
    s.E = E_out; s.wgt = p->s.w * m; s.wgt2 = 0.; /* the next generation starts from wgt alone */
    s.parent_history_id = p->hid;
    s.parent_daughter_id = p->daughter++;
    s.family_id = p->family;
    if (!site_push(sb, h, &s)) { set_err("out of memory"); return ABX_ERR_OOM; }
    p->alive = 0;
  }
  return ABX_OK;
}

/* Transporter::collision + branching_collision + make_fission_neutrons +
 * do_scatter (src/transporter.cpp:60-93, 269-347, 358-487) and
 * MGNuclide::sample_scatter / sample_fission (src/mg_nuclide.cpp:442-461, 504-544) */
static int collision(oracle_ctx* ctx, Part* p, int mat, double kcol, int converged,
                     Scores* sc, SiteBuf* sb, uint32_t h) {
  const int G = ctx->G;
  int g = group_of(ctx, p->s.E);
  if (converged) score_collision(ctx, p, mat);
  const double Et = MAT_AT(ctx->Et, mat, g);
  const double Eabs = MAT_AT(ctx->Eabs, mat, g);
  const double Ef = MAT_AT(ctx->Ef, mat, g);
  const double nu = MAT_AT(ctx->nu_tot, mat, g);
  const double vEf = MAT_AT(ctx->vEf, mat, g);
  {
    double k_col_scr = p->s.w * vEf / Et;
    double mig_dist = vnorm(vsub(p->s.r, p->r_birth));
    double mig_area_scr = p->s.w * Eabs / Et * mig_dist * mig_dist;
    sc->k_col += k_col_scr;
    sc->mig += mig_area_scr;
  }
  if (ctx->set.branchless) return branchless_collision(ctx, p, mat, g, sc, sb, h);
  /* sample_nuclide: one draw even with a single component (material_helper.hpp:178-224) */
  (void)oracle_canonical(&p->rng);
  double k_abs_scr = p->s.w * nu * Ef / Et;
  sc->k_abs += k_abs_scr;
  /* make_fission_neutrons */
  {
    double kabs2 = p->s.w * nu * Ef / Et;
    int n_new;
    if (ctx->set.mode == ABX_MODE_K_EIGENVALUE)
      n_new = (int)floor(fabs(kabs2) / kcol + oracle_canonical(&p->rng));
    else
      n_new = (int)floor(fabs(kabs2) + oracle_canonical(&p->rng));
    double P_delayed = MAT_AT(ctx->nu_d, mat, g) / nu;
    for (int i = 0; i < n_new; i++) {
      int ei = sample_discrete_cdf(&p->rng, ctx->chi_cdf + ((size_t)mat * G + g) * G, G);
      double E_out = group_mid(ctx, ei);
      double mu = 2. * oracle_canonical(&p->rng) - 1.;
      double phi = 2. * PI_ * oracle_canonical(&p->rng);
      V3 uout = rotate_direction(p->s.u, mu, phi);
      if (oracle_canonical(&p->rng) < P_delayed) {
        (void)sample_discrete_cdf(&p->rng, ctx->dg_cdf[mat], ctx->n_dg[mat]);
      }
      double wgt = p->s.w > 0. ? 1. : -1.;
      if (ctx->set.mode == ABX_MODE_K_EIGENVALUE) {
        abx_site s;
        s.r[0] = p->s.r.x; s.r[1] = p->s.r.y; s.r[2] = p->s.r.z;
        s.u[0] = uout.x; s.u[1] = uout.y; s.u[2] = uout.z;
        s.E = E_out; s.wgt = wgt; s.wgt2 = 0.;
        s.parent_history_id = p->hid;
        s.parent_daughter_id = p->daughter++;
        s.family_id = p->family;
        if (!site_push(sb, h, &s)) { set_err("out of memory"); return ABX_ERR_OOM; }
      } else {
        PState ns;
        ns.r = p->s.r; ns.u = uout; ns.E = E_out; ns.w = wgt; ns.w2 = 0.;
        p->daughter++;
        if (!sec_push(p, ns)) { set_err("out of memory"); return ABX_ERR_OOM; }
      }
    }
  }
  /* implicit capture */
  p->s.w = p->s.w * (1. - (Eabs + 0.) / Et);
  p->s.w2 = p->s.w2 * (1. - (Eabs + 0.) / Et);
  russian_roulette(ctx, p);
  if (p->alive) {
    int ei = sample_discrete_cdf(&p->rng, ctx->ps_cdf + ((size_t)mat * G + g) * G, G);
    double E_out = group_mid(ctx, ei);
    double mu = sample_mu(ctx, mat, g, ei, &p->rng);
    double phi = 2. * PI_ * oracle_canonical(&p->rng);
    V3 uout = rotate_direction(p->s.u, mu, phi);
    p->s.u = uout;
    p->s.E = E_out;
    p->s.w = p->s.w * 1.;
    p->s.w2 = p->s.w2 * 1.;
    if (p->s.E < ctx->min_energy) p->alive = 0;
  }
  return ABX_OK;
}

/* Particle::resurect (include/simulation/particle.hpp:170-182) */
static void resurrect(Part* p) {
  if (!p->alive && p->nsec > 0) {
    p->alive = 1;
    p->s = p->sec[--p->nsec];
  }
}

static void do_reflection(oracle_ctx* ctx, Tracker* t, Part* p, Boundary b) {
  /* Tracker::do_reflection (tracker.hpp:314-359); the surface token it sets
   * is cleared again by set_r, and previous-position bookkeeping only feeds
   * cancellation, so neither is carried. */
  const abx_surface* s = &ctx->surf[b.surface_index];
  V3 u = p->s.u;
  V3 r_on = vadd(p->s.r, vscale(u, b.distance));
  V3 n = surf_norm(s, r_on);
  double c2 = 2. * vdot(u, n);
  V3 nd = vsub(u, vscale(n, c2));
  V3 unew = dir3(nd.x, nd.y, nd.z);
  p->s.r = r_on;
  p->s.u = unew;
  trk_set_r(t, p->s.r);
  t->u = p->s.u;
  trk_restart(ctx, t);
}

/* One history: DeltaTracker::transport loop body (src/delta_tracker.cpp:87-229)
 * or SurfaceTracker::transport loop body (src/surface_tracker.cpp:55-199). */
static int run_history(oracle_ctx* ctx, const abx_particle* in, uint32_t h, double kcol,
                       int converged, Scores* sc, SiteBuf* sb, TraceBuf* tb) {
  Part p;
  memset(&p, 0, sizeof p);
  p.s.r = v3(in->r[0], in->r[1], in->r[2]);
  p.s.u = v3(in->u[0], in->u[1], in->u[2]);
  p.s.E = in->E; p.s.w = in->wgt; p.s.w2 = in->wgt2;
  p.rng = in->rng_state; p.hid = in->history_id; p.family = in->family_id;
  p.r_birth = p.s.r;
  p.alive = 1;
  Tracker t;
  trk_init(ctx, &t, p.s.r, p.s.u);
  if (ctx->err) return ctx->err;
  if (t.cell < 0) {
    sc->lost++;
    p.alive = 0;
  }
  int mat = t.cell >= 0 ? ctx->cell[t.cell].fill : -1;
  const int delta = ctx->set.tracking == ABX_TRACK_DELTA;
  const int ildt = ctx->set.tracking == ABX_TRACK_IMPLICIT_LEAKAGE;
  const int carter = ctx->set.tracking == ABX_TRACK_CARTER;
  const double wgt_split = ctx->set.wgt_split > 0. ? ctx->set.wgt_split : 2.0;
  int rc = ABX_OK;
  while (p.alive) {
    int had_collision = 0;
    int g = group_of(ctx, p.s.E);
    if (ildt) {
      /* ImplicitLeakageDeltaTracker::transport
       * (src/implicit_leakage_delta_tracker.cpp:104-214): the nearest
       * boundary condition before every flight; towards a vacuum boundary the
       * weight that would leak is scored as leakage at once and the flight is
       * sampled within the boundary distance. */
      double Emaj = ctx->maj[g];
      Boundary bound = trk_get_bc(ctx, &t);
      if (ctx->err) return ctx->err;
      double d_coll;
      sc->flights++;
      if (bound.btype == ABX_BC_VACUUM) {
        const double P_leak = exp(-Emaj * bound.distance);
        const double P_no_leak = 1. - P_leak;
        const double wgt_leak = p.s.w * P_leak, wgt2_leak = p.s.w2 * P_leak;
        const double wgt_coll = p.s.w * P_no_leak, wgt2_coll = p.s.w2 * P_no_leak;
        sc->leak += wgt_leak;
        V3 r_leak = vadd(p.s.r, vscale(p.s.u, bound.distance));
        V3 dl = vsub(r_leak, p.r_birth);
        sc->mig += vdot(vscale(dl, wgt_leak), dl);
        d_coll = -log(1. - P_no_leak * oracle_canonical(&p.rng)) / Emaj;
        p.s.w = wgt_leak;
        p.s.w2 = wgt2_leak;
        if (converged) score_flight(ctx, &p, bound.distance, mat);
        p.s.w = wgt_coll;
        p.s.w2 = wgt2_coll;
        if (converged) score_flight(ctx, &p, d_coll, mat);
      } else {
        d_coll = oracle_exponential(&p.rng, Emaj);
        if (converged) score_flight(ctx, &p, d_coll < bound.distance ? d_coll : bound.distance, mat);
      }
      if (bound.distance < d_coll || fabs(bound.distance - d_coll) < BOUNDRY_TOL_) {
        if (bound.btype == ABX_BC_VACUUM) {
          p.alive = 0;
          sc->leak += p.s.w;
          V3 r_leak = vadd(p.s.r, vscale(p.s.u, bound.distance));
          V3 dl = vsub(r_leak, p.r_birth);
          sc->mig += vdot(vscale(dl, p.s.w), dl);
          trace(ctx, tb, h, 2, &p, t.cell);
        } else if (bound.btype == ABX_BC_REFLECTIVE) {
          do_reflection(ctx, &t, &p, bound);
          if (ctx->err) return ctx->err;
          if (t.cell < 0) {
            set_err("particle %llu lost after reflection", (unsigned long long)p.hid);
            return ABX_ERR_LOST_PARTICLE;
          }
          trace(ctx, tb, h, 3, &p, t.cell);
        } else {
          set_err("boundary crossing without a boundary condition");
          return ABX_ERR_LOST_PARTICLE;
        }
      } else {
        p.s.r = vadd(p.s.r, vscale(p.s.u, d_coll));
        trk_move(&t, d_coll);
        trk_get_current(ctx, &t);
        if (ctx->err) return ctx->err;
        if (t.cell < 0) {
          set_err("particle %llu lost after a flight of %g cm", (unsigned long long)p.hid, d_coll);
          return ABX_ERR_LOST_PARTICLE;
        }
        mat = ctx->cell[t.cell].fill;
        double Et = MAT_AT(ctx->Et, mat, g);
        if (Et - Emaj > 1.E-10) {
          set_err("Total cross section excedeed majorant: Et = %g, Emaj = %g", Et, Emaj);
          return ABX_ERR_MAJORANT;
        }
        if (oracle_canonical(&p.rng) < (Et / Emaj)) had_collision = 1;
        trace(ctx, tb, h, had_collision ? 1 : 0, &p, t.cell);
      }
    } else if (delta || carter) {
      /* CarterTracker::transport (src/carter_tracker.cpp:124-222) flies like
       * the delta tracker, on its sampling cross section */
      double Emaj = carter ? ctx->smp[g] : ctx->maj[g];
      double d_coll = oracle_exponential(&p.rng, Emaj);
      Boundary bound = {INF_, -1, ABX_BC_NORMAL, 0};
      int crossed = 0;
      trk_move(&t, d_coll);
      trk_get_current(ctx, &t);
      if (ctx->err) return ctx->err;
      if (t.cell < 0) {
        trk_set_r(&t, p.s.r);
        trk_get_current(ctx, &t);
        if (ctx->err) return ctx->err;
        bound = trk_get_bc(ctx, &t);
        crossed = 1;
      }
      sc->flights++;
      if (converged) score_flight(ctx, &p, d_coll < bound.distance ? d_coll : bound.distance, mat);
      if (crossed) {
        if (bound.btype == ABX_BC_VACUUM) {
          p.alive = 0;
          sc->leak += p.s.w;
          V3 r_leak = vadd(p.s.r, vscale(p.s.u, bound.distance));
          V3 dl = vsub(r_leak, p.r_birth);
          sc->mig += vdot(vscale(dl, p.s.w), dl);
          trace(ctx, tb, h, 2, &p, t.cell);
        } else if (bound.btype == ABX_BC_REFLECTIVE) {
          do_reflection(ctx, &t, &p, bound);
          if (ctx->err) return ctx->err;
          if (t.cell < 0) {
            set_err("particle %llu lost after reflection", (unsigned long long)p.hid);
            return ABX_ERR_LOST_PARTICLE;
          }
          trace(ctx, tb, h, 3, &p, t.cell);
        } else {
          set_err("boundary crossing without a boundary condition");
          return ABX_ERR_LOST_PARTICLE;
        }
      } else {
        p.s.r = vadd(p.s.r, vscale(p.s.u, d_coll));
        mat = ctx->cell[t.cell].fill;
        double Et = MAT_AT(ctx->Et, mat, g);
        if (carter) {
          /* src/carter_tracker.cpp:188-207 */
          const double Esample = Emaj;
          if (Esample >= Et) {
            if (oracle_canonical(&p.rng) < (Et / Esample)) had_collision = 1;
          } else {
            double D = Et / (2. * Et - Esample);
            double F = Et / (D * Esample);
            if ((D - oracle_canonical(&p.rng)) > 0.) {
              p.s.w = p.s.w * F;
              had_collision = 1;
            } else {
              p.s.w = -p.s.w * F;
            }
          }
        } else {
          if (Et - Emaj > 1.E-10) {
            set_err("Total cross section excedeed majorant: Et = %g, Emaj = %g", Et, Emaj);
            return ABX_ERR_MAJORANT;
          }
          if (oracle_canonical(&p.rng) < (Et / Emaj)) had_collision = 1;
        }
        trace(ctx, tb, h, had_collision ? 1 : 0, &p, t.cell);
      }
    } else {
      double Et = MAT_AT(ctx->Et, mat, g);
      double d_coll = oracle_exponential(&p.rng, Et);
      Boundary bound = trk_nearest(ctx, &t);
      if (ctx->err) return ctx->err;
      double dmin = d_coll < bound.distance ? d_coll : bound.distance;
      sc->flights++;
      if (converged) score_flight(ctx, &p, dmin, mat);
      sc->k_trk += p.s.w * dmin * MAT_AT(ctx->vEf, mat, g);
      if (bound.distance < d_coll || fabs(bound.distance - d_coll) < BOUNDRY_TOL_) {
        if (bound.btype == ABX_BC_VACUUM) {
          p.alive = 0;
          sc->leak += p.s.w;
          V3 r_leak = vadd(p.s.r, vscale(p.s.u, bound.distance));
          V3 dl = vsub(r_leak, p.r_birth);
          sc->mig += vdot(vscale(dl, p.s.w), dl);
          trace(ctx, tb, h, 2, &p, t.cell);
        } else if (bound.btype == ABX_BC_REFLECTIVE) {
          do_reflection(ctx, &t, &p, bound);
          if (ctx->err) return ctx->err;
          if (t.cell < 0) {
            set_err("particle %llu lost after reflection", (unsigned long long)p.hid);
            return ABX_ERR_LOST_PARTICLE;
          }
          trace(ctx, tb, h, 3, &p, t.cell);
        } else {
          /* Tracker::cross_surface + get_current (tracker.hpp:227-231) */
          trk_move(&t, bound.distance);
          t.token = -bound.token;
          trk_get_current(ctx, &t);
          if (ctx->err) return ctx->err;
          p.s.r = vadd(p.s.r, vscale(p.s.u, bound.distance));
          if (t.cell < 0) {
            set_err("particle %llu lost crossing a surface", (unsigned long long)p.hid);
            return ABX_ERR_LOST_PARTICLE;
          }
          mat = ctx->cell[t.cell].fill;
          trace(ctx, tb, h, 5, &p, t.cell);
        }
      } else {
        p.s.r = vadd(p.s.r, vscale(p.s.u, d_coll));
        trk_move(&t, d_coll);
        had_collision = 1;
        trace(ctx, tb, h, 1, &p, t.cell);
      }
    }
    if (p.alive && had_collision) {
      sc->coll++;
      rc = collision(ctx, &p, mat, kcol, converged, sc, sb, h);
      if (rc) return rc;
      t.u = p.s.u;
      trace(ctx, tb, h, 4, &p, t.cell);
    }
    if (carter && p.alive && fabs(p.s.w) >= wgt_split) {
      /* Particle::split (include/simulation/particle.hpp:165-173) */
      int n_new = (int)ceil(fabs(p.s.w));
      if (n_new > 1) {
        p.s.w = p.s.w / (double)n_new;
        p.s.w2 = p.s.w2 / (double)n_new;
        for (int k = 0; k < n_new - 1; k++)
          if (!sec_push(&p, p.s)) { set_err("out of memory"); return ABX_ERR_OOM; }
      }
    }
    if (!p.alive) {
      resurrect(&p);
      if (p.alive) {
        trk_set_r(&t, p.s.r);
        t.u = p.s.u;
        trk_restart(ctx, &t);
        if (ctx->err) return ctx->err;
        if (t.cell < 0) {
          set_err("particle %llu lost at resurrection", (unsigned long long)p.hid);
          return ABX_ERR_LOST_PARTICLE;
        }
        mat = ctx->cell[t.cell].fill;
        trace(ctx, tb, h, 6, &p, t.cell);
      }
    }
  }
  free(p.sec);
  return rc;
}

/* ---------------------------------------------------------- transport */
int oracle_transport(oracle_ctx* ctx, const abx_particle* bank, size_t n, double kcol,
                     int converged, abx_site* sites, size_t cap, size_t* n_sites,
                     abx_scores* out_scores, int nthreads) {
  if (!ctx) return ABX_ERR_INVALID;
  ctx->err = 0;
  int use_trace = ctx->tr_nhist > 0;
  if (use_trace) nthreads = 1;
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#else
  nthreads = 1;
#endif
  SiteBuf* sbs = (SiteBuf*)xcalloc((size_t)nthreads, sizeof(SiteBuf));
  Scores* scs = (Scores*)xcalloc((size_t)nthreads, sizeof(Scores));
  TraceBuf tbuf = {0};
  int rc_all = ABX_OK;
  if (!sbs || !scs) { free(sbs); free(scs); set_err("out of memory"); return ABX_ERR_OOM; }
#ifdef _OPENMP
#pragma omp parallel num_threads(nthreads)
#endif
  {
    int tid = 0;
#ifdef _OPENMP
    tid = omp_get_thread_num();
#endif
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 16)
#endif
    for (size_t i = 0; i < n; i++) {
      if (rc_all) continue;
      int rc = run_history(ctx, &bank[i], (uint32_t)i, kcol, converged, &scs[tid], &sbs[tid],
                           use_trace ? &tbuf : NULL);
      if (rc) {
#ifdef _OPENMP
#pragma omp critical
#endif
        rc_all = rc;
      }
    }
  }
  /* Per-history banks concatenated in bank order (src/delta_tracker.cpp:251-253):
   * counting sort on the history index; within a history sites are in order. */
  size_t total = 0;
  for (int t = 0; t < nthreads; t++) total += sbs[t].n;
  if (!rc_all && n_sites) *n_sites = total;
  if (!rc_all && total > cap && ctx->set.mode == ABX_MODE_K_EIGENVALUE) {
    set_err("fission bank capacity %zu < %zu sites", cap, total);
    rc_all = ABX_ERR_CAPACITY;
  }
  if (!rc_all && total > 0 && sites) {
    size_t* cnt = (size_t*)xcalloc(n + 1, sizeof(size_t));
    for (int t = 0; t < nthreads; t++)
      for (size_t s = 0; s < sbs[t].n; s++) cnt[sbs[t].hist[s] + 1]++;
    for (size_t i = 0; i < n; i++) cnt[i + 1] += cnt[i];
    for (int t = 0; t < nthreads; t++)
      for (size_t s = 0; s < sbs[t].n; s++) sites[cnt[sbs[t].hist[s]]++] = sbs[t].v[s];
    free(cnt);
  }
  abx_scores S;
  memset(&S, 0, sizeof S);
  for (int t = 0; t < nthreads; t++) {
    S.k_col += scs[t].k_col; S.k_abs += scs[t].k_abs; S.k_trk += scs[t].k_trk;
    S.k_tot += scs[t].k_tot; S.leakage += scs[t].leak; S.mig_area += scs[t].mig;
    S.collisions += scs[t].coll; S.flights += scs[t].flights; S.lost += scs[t].lost;
  }
  if (out_scores) *out_scores = S;
  for (int t = 0; t < nthreads; t++) { free(sbs[t].v); free(sbs[t].hist); }
  free(sbs); free(scs);
  if (use_trace) {
    size_t m = tbuf.n < ctx->tr_cap ? tbuf.n : ctx->tr_cap;
    free(ctx->tr);
    ctx->tr = (abx_trace_rec*)xcalloc(m, sizeof(abx_trace_rec));
    if (m) memcpy(ctx->tr, tbuf.v, m * sizeof(abx_trace_rec));
    ctx->tr_n = m;
    free(tbuf.v);
  }
  return rc_all;
}

/* ----------------------------------------------------------- sources */
/* Source::generate_particle (src/source.cpp:44-90) */
static V3 src_position(const abx_source* s, uint64_t* rng) {
  if (s->spatial == ABX_SPATIAL_POINT) return v3(s->low[0], s->low[1], s->low[2]);
  double x = (s->hi[0] - s->low[0]) * oracle_canonical(rng) + s->low[0];
  double y = (s->hi[1] - s->low[1]) * oracle_canonical(rng) + s->low[1];
  double z = (s->hi[2] - s->low[2]) * oracle_canonical(rng) + s->low[2];
  return v3(x, y, z);
}

int oracle_sample_sources(oracle_ctx* ctx, uint64_t first, size_t n, abx_particle* out) {
  if (!ctx || ctx->nsrc <= 0) { set_err("no sources"); return ABX_ERR_INVALID; }
  ctx->err = 0;
  for (size_t i = 0; i < n; i++) {
    uint64_t hid = first + i;
    uint64_t rng;
    oracle_pcg32_seed(ctx->set.seed, &rng);
    oracle_pcg32_advance(&rng, ctx->set.stride * hid);
    int indx = sample_discrete_cdf(&rng, ctx->src_cdf, ctx->nsrc);
    const abx_source* s = &ctx->src[indx];
    V3 u;
    if (s->direction == ABX_DIR_ISOTROPIC) {
      double mu = 2. * oracle_canonical(&rng) - 1.;
      double phi = 2. * PI_ * oracle_canonical(&rng);
      u = dir_mu_phi(mu, phi);
    } else {
      u = dir3(s->dir[0], s->dir[1], s->dir[2]);
    }
    double E = s->energy_value;
    int E_count = 0;
    do {
      if (E_count > 200) { set_err("Exceded 200 samplings of energy."); return ABX_ERR_INVALID; }
      E = s->energy_value;
      E_count++;
    } while (E <= ctx->min_energy || ctx->max_energy <= E);
    V3 r = src_position(s, &rng);
    Tracker t;
    trk_init(ctx, &t, r, u);
    int guard = 0;
    while (t.cell < 0) {
      if (s->spatial == ABX_SPATIAL_POINT || ++guard > 1000000) {
        set_err("source position outside the geometry");
        return ABX_ERR_LOST_PARTICLE;
      }
      r = src_position(s, &rng);
      trk_set_r(&t, r);
      trk_restart(ctx, &t);
    }
    if (s->fissile_only) {
      int count = 0;
      while (t.cell < 0 || !ctx->fissile[ctx->cell[t.cell].fill]) {
        if (count == 201) {
          set_err("Exceded 200 samplings of position in fissile-only source.");
          return ABX_ERR_INVALID;
        }
        r = src_position(s, &rng);
        trk_set_r(&t, r);
        trk_restart(ctx, &t);
        count++;
      }
    }
    if (ctx->err) return ctx->err;
    abx_particle* p = &out[i];
    p->r[0] = r.x; p->r[1] = r.y; p->r[2] = r.z;
    p->u[0] = u.x; p->u[1] = u.y; p->u[2] = u.z;
    p->E = E; p->wgt = 1.0; p->wgt2 = 0.;
    p->history_id = hid;
    p->rng_state = rng;
    p->family_id = hid;
  }
  return ABX_OK;
}

/* -------------------------------------------------- tallies lifecycle */
/* MeshTally::record_generation (src/mesh_tally.cpp:121-150) */
int oracle_tally_record_generation(oracle_ctx* ctx, double multiplier) {
  for (int ti = 0; ti < ctx->ntally; ti++) {
    OTally* T = &ctx->tally[ti];
    T->g++;
    const double dg = (double)T->g;
    for (size_t i = 0; i < T->nbins; i++) {
      double old_avg = T->avg[i];
      double val = T->gen[i] * multiplier;
      double avg = old_avg + (val - old_avg) / dg;
      T->avg[i] = avg;
      double var = T->var[i];
      var = var + (((val - old_avg) * (val - avg) - (var)) / dg);
      T->var[i] = var;
    }
  }
  return ABX_OK;
}
int oracle_tally_clear_generation(oracle_ctx* ctx) {
  for (int ti = 0; ti < ctx->ntally; ti++)
    memset(ctx->tally[ti].gen, 0, ctx->tally[ti].nbins * sizeof(double));
  return ABX_OK;
}
int oracle_tally_size(oracle_ctx* ctx, int id, size_t* n) {
  if (id < 0 || id >= ctx->ntally) return ABX_ERR_INVALID;
  *n = ctx->tally[id].nbins;
  return ABX_OK;
}
int oracle_tally_read(oracle_ctx* ctx, int id, double* gen, double* avg, double* var, int* g) {
  if (id < 0 || id >= ctx->ntally) return ABX_ERR_INVALID;
  OTally* T = &ctx->tally[id];
  if (gen) memcpy(gen, T->gen, T->nbins * sizeof(double));
  if (avg) memcpy(avg, T->avg, T->nbins * sizeof(double));
  if (var) memcpy(var, T->var, T->nbins * sizeof(double));
  if (g) *g = T->g;
  return ABX_OK;
}

/* Entropy::add_point + calculate_entropy (src/entropy.cpp:32-93), Sign::Total */
int oracle_entropy(oracle_ctx* ctx, const abx_site* s, size_t n, double* H) {
  if (!ctx->ent_on) { *H = 0.; return ABX_OK; }
  size_t nb = (size_t)ctx->ent_shape[0] * ctx->ent_shape[1] * ctx->ent_shape[2];
  double* bins = (double*)xcalloc(nb, sizeof(double));
  double tw = 0.;
  for (size_t i = 0; i < n; i++) {
    int32_t nx = (int32_t)floor((s[i].r[0] - ctx->ent_low[0]) / ctx->ent_d[0]);
    int32_t ny = (int32_t)floor((s[i].r[1] - ctx->ent_low[1]) / ctx->ent_d[1]);
    int32_t nz = (int32_t)floor((s[i].r[2] - ctx->ent_low[2]) / ctx->ent_d[2]);
    if (nx >= 0 && nx < ctx->ent_shape[0] && ny >= 0 && ny < ctx->ent_shape[1] && nz >= 0 &&
        nz < ctx->ent_shape[2]) {
      tw += s[i].wgt;
      bins[(size_t)ctx->ent_shape[1] * ctx->ent_shape[2] * nx + (size_t)ctx->ent_shape[2] * ny + nz] += s[i].wgt;
    }
  }
  double sum = 0.;
  for (size_t b = 0; b < nb; b++) {
    double p = fabs(bins[b]) / tw;
    if (p > 1.0) {
    } else if (p != 0.) {
      sum -= p * log2(p);
    }
  }
  free(bins);
  *H = sum;
  return ABX_OK;
}

/* ------------------------------------------------------------ drivers */
static void update_avg_var(int gen, double x, double* avg, double* var) {
  /* Tallies::update_avg_and_var (src/tallies.cpp:268-280) */
  double dgen = (double)gen;
  double a0 = *avg, v0 = *var;
  *avg = a0 + (x - a0) / dgen;
  if (gen > 1) *var = v0 + ((x - a0) * (x - a0) / dgen) - (v0 / (dgen - 1.));
}

static double now_ms(void) {
#ifdef _OPENMP
  return omp_get_wtime() * 1e3;
#else
  return 0.;
#endif
}

/* PowerIterator::initialize + run (src/power_iterator.cpp:46-166, 305-473, 538-586) */
/* BranchlessPowerIterator::comb_particles (src/branchless_power_iterator.cpp:
 * 592-650) on the normalised bank: positive and negative sites apart, each
 * shuffled with the global stream and combed into ceil(W) sites of equal
 * weight (a comb position drawn in [0, W/N) then steps of W/N), the result
 * shuffled again.  Negative weights do not occur with branchless collisions
 * alone; a bank holding some is refused. */
static int comb_sites(abx_site** psites, size_t* pn, uint64_t* gs) {
  abx_site* s = *psites;
  const size_t n = *pn;
  abx_site* pos = (abx_site*)xcalloc(n, sizeof(abx_site));
  size_t np = 0;
  double Wpos = 0., Wneg = 0.;
  for (size_t i = 0; i < n; i++) {
    if (s[i].wgt > 0.) { Wpos += s[i].wgt; pos[np++] = s[i]; }
    else Wneg += s[i].wgt;
  }
  if (np != n) { free(pos); set_err("combing a bank with non-positive weights"); return ABX_ERR_UNSUPPORTED; }
  const size_t Npos = (size_t)ceil(Wpos);
  oracle_shuffle(pos, np, sizeof(abx_site), gs);
  const double avg_pos = Wpos / (double)Npos;
  double comb_pos = oracle_canonical(gs) * avg_pos;
  double cur = 0.;
  size_t cap = Npos + 4, m = 0;
  abx_site* out = (abx_site*)xcalloc(cap, sizeof(abx_site));
  for (size_t i = 0; i < np; i++) {
    cur += pos[i].wgt;
    while (comb_pos < cur) {
      if (m == cap) {
        cap *= 2;
        abx_site* nv = (abx_site*)realloc(out, cap * sizeof(abx_site));
        if (!nv) { free(out); free(pos); set_err("out of memory"); return ABX_ERR_OOM; }
        out = nv;
      }
      out[m] = pos[i];
      out[m].wgt = avg_pos;
      m++;
      comb_pos += avg_pos;
    }
  }
  /* the negative sites: none to shuffle or comb, but the comb position is drawn */
  (void)oracle_canonical(gs);
  (void)Wneg;
  oracle_shuffle(out, m, sizeof(abx_site), gs);
  free(pos);
  free(s);
  *psites = out;
  *pn = m;
  return ABX_OK;
}

/* PowerIterator::load_source_from_file (src/power_iterator.cpp:60-132):
 * rows x y z ux uy uz E wgt wgt2 become histories 0..n-1 (family = history
 * id), each stream seeded at its id; nparticles becomes the rounded total
 * weight. */
int oracle_set_source_bank(oracle_ctx* ctx, const double* src, size_t n) {
  free(ctx->restart);
  ctx->restart = NULL;
  ctx->n_restart = 0;
  if (n == 0) return ABX_OK;
  ctx->restart = (double*)xcalloc(9 * n, sizeof(double));
  memcpy(ctx->restart, src, 9 * n * sizeof(double));
  ctx->n_restart = n;
  return ABX_OK;
}

int oracle_run_power_iteration(oracle_ctx* ctx, int ngen, int nignored, int nthreads,
                               abx_run_stats* st, double* kcol_gen, double* ent_gen) {
  double t0 = now_ms();
  int rc;
  abx_particle* bank;
  size_t N;
  if (ctx->n_restart) {
    N = ctx->n_restart;
    bank = (abx_particle*)xcalloc(N, sizeof(abx_particle));
    double tot_wgt = 0.;
    for (size_t i = 0; i < N; i++) {
      const double* q = ctx->restart + 9 * i;
      abx_particle* p = &bank[i];
      memcpy(p->r, q, 3 * sizeof(double));
      memcpy(p->u, q + 3, 3 * sizeof(double));
      p->E = q[6]; p->wgt = q[7]; p->wgt2 = q[8];
      p->history_id = i;
      p->family_id = i;
      oracle_pcg32_seed(ctx->set.seed, &p->rng_state);
      oracle_pcg32_advance(&p->rng_state, ctx->set.stride * p->history_id);
      tot_wgt += q[7];
    }
    ctx->set.nparticles = round(tot_wgt);
  } else {
    N = (size_t)ctx->set.nparticles;
    bank = (abx_particle*)xcalloc(N, sizeof(abx_particle));
    rc = oracle_sample_sources(ctx, 0, N, bank);
    if (rc) { free(bank); return rc; }
  }
  uint64_t global = N;
  size_t nb = N;
  /* the global stream the combing draws from: a default-constructed pcg32
   * (src/settings.cpp:59) after the draws made while the deck was read */
  const int combing = (ctx->set.branchless & ABX_BRANCHLESS_COMBING) != 0;
  uint64_t gstream;
  oracle_pcg32_seed(0xcafef00dd15ea5e5ULL, &gstream);
  oracle_pcg32_advance(&gstream, (uint64_t)(ctx->set.global_rng_skip > 0 ? ctx->set.global_rng_skip : 0));
  double kcol = 1.0;
  int converged = nignored == 0;
  int active = 0;
  double kcol_avg = 0, kcol_var = 0, ktrk_avg = 0, ktrk_var = 0, leak_avg = 0, leak_var = 0,
         mig_avg = 0, mig_var = 0, kabs_avg = 0, kabs_var = 0;
  abx_run_stats S;
  memset(&S, 0, sizeof S);
  double ttr = 0.;
  for (int g = 1; g <= ngen; g++) {
    size_t cap = 3 * nb + 1024;
    abx_site* sites = (abx_site*)xcalloc(cap, sizeof(abx_site));
    size_t ns = 0;
    abx_scores sc;
    double ta = now_ms();
    rc = oracle_transport(ctx, bank, nb, kcol, converged, sites, cap, &ns, &sc, nthreads);
    ttr += now_ms() - ta;
    if (rc) { free(sites); free(bank); return rc; }
    S.collisions += sc.collisions; S.flights += sc.flights; S.histories += nb;
    if (ns == 0) { free(sites); free(bank); set_err("No fission neutrons were produced."); return ABX_ERR_NO_FISSION; }
    if (ent_gen && !combing) { double H; oracle_entropy(ctx, sites, ns, &H); ent_gen[g - 1] = H; }
    double tw = ctx->set.nparticles;
    double k_col = sc.k_col / tw, k_abs = sc.k_abs / tw, k_trk = sc.k_trk / tw;
    double leak = sc.leakage / tw, mig = sc.mig_area / tw;
    if (kcol_gen) kcol_gen[g - 1] = k_col;
    /* normalize_weights */
    double W_pos = 0., W_neg = 0.;
    for (size_t i = 0; i < ns; i++) {
      if (sites[i].wgt > 0.) W_pos += sites[i].wgt;
      else W_neg -= sites[i].wgt;
    }
    double W = W_pos - W_neg;
    double wpp = (double)ctx->set.nparticles / W;
    for (size_t i = 0; i < ns; i++) sites[i].wgt *= wpp;
    if (combing) {
      rc = comb_sites(&sites, &ns, &gstream);
      if (rc) { free(sites); free(bank); return rc; }
      /* the entropy of the combed bank (compute_post_cancellation_entropy) */
      if (ent_gen) { double H; oracle_entropy(ctx, sites, ns, &H); ent_gen[g - 1] = H; }
    }
    if (converged) {
      active++;
      update_avg_var(active, k_col, &kcol_avg, &kcol_var);
      update_avg_var(active, k_abs, &kabs_avg, &kabs_var);
      update_avg_var(active, k_trk, &ktrk_avg, &ktrk_var);
      update_avg_var(active, leak, &leak_avg, &leak_var);
      update_avg_var(active, mig, &mig_avg, &mig_var);
      oracle_tally_record_generation(ctx, 1.0);
    }
    oracle_tally_clear_generation(ctx);
    free(bank);
    bank = (abx_particle*)xcalloc(ns, sizeof(abx_particle));
    for (size_t i = 0; i < ns; i++) {
      abx_particle* p = &bank[i];
      memcpy(p->r, sites[i].r, sizeof p->r);
      memcpy(p->u, sites[i].u, sizeof p->u);
      p->E = sites[i].E; p->wgt = sites[i].wgt; p->wgt2 = 0.;
      p->history_id = global + i;
      oracle_pcg32_seed(ctx->set.seed, &p->rng_state);
      oracle_pcg32_advance(&p->rng_state, ctx->set.stride * p->history_id);
      p->family_id = sites[i].family_id;
    }
    global += ns;
    nb = ns;
    free(sites);
    kcol = k_col;
    S.generations = g;
    if (g == nignored) converged = 1;
  }
  free(bank);
  S.active = active;
  S.kcol_avg = kcol_avg; S.kcol_std = active ? sqrt(kcol_var / active) : 0.;
  S.ktrk_avg = ktrk_avg; S.ktrk_std = active ? sqrt(ktrk_var / active) : 0.;
  S.leak_avg = leak_avg; S.leak_std = active ? sqrt(leak_var / active) : 0.;
  S.mig_avg = mig_avg; S.mig_std = active ? sqrt(mig_var / active) : 0.;
  S.transport_ms = ttr;
  S.total_ms = now_ms() - t0;
  if (st) *st = S;
  return ABX_OK;
}

/* FixedSource::run (src/fixed_source.cpp:81-173) */
int oracle_run_fixed_source(oracle_ctx* ctx, int nbatches, uint64_t npart, int nthreads,
                            abx_run_stats* st) {
  abx_run_stats S;
  memset(&S, 0, sizeof S);
  uint64_t hc = 0;
  double leak_avg = 0, leak_var = 0, mig_avg = 0, mig_var = 0;
  double t0 = now_ms(), ttr = 0.;
  abx_particle* bank = (abx_particle*)xcalloc(npart, sizeof(abx_particle));
  for (int g = 1; g <= nbatches; g++) {
    int rc = oracle_sample_sources(ctx, hc, npart, bank);
    if (rc) { free(bank); return rc; }
    hc += npart;
    abx_scores sc;
    size_t ns = 0;
    double ta = now_ms();
    rc = oracle_transport(ctx, bank, npart, 1.0, 1, NULL, 0, &ns, &sc, nthreads);
    ttr += now_ms() - ta;
    if (rc) { free(bank); return rc; }
    S.collisions += sc.collisions; S.flights += sc.flights; S.histories += npart;
    double tw = ctx->set.nparticles;
    update_avg_var(g, sc.leakage / tw, &leak_avg, &leak_var);
    update_avg_var(g, sc.mig_area / tw, &mig_avg, &mig_var);
    oracle_tally_record_generation(ctx, 1.0);
    oracle_tally_clear_generation(ctx);
    S.generations = g;
  }
  free(bank);
  S.active = S.generations;
  S.leak_avg = leak_avg; S.leak_std = S.active ? sqrt(leak_var / S.active) : 0.;
  S.mig_avg = mig_avg; S.mig_std = S.active ? sqrt(mig_var / S.active) : 0.;
  S.transport_ms = ttr;
  S.total_ms = now_ms() - t0;
  if (st) *st = S;
  return ABX_OK;
}

int oracle_set_trace(oracle_ctx* ctx, uint32_t n_hist, size_t cap) {
  ctx->tr_nhist = n_hist;
  ctx->tr_cap = cap;
  return ABX_OK;
}
int oracle_get_trace(oracle_ctx* ctx, abx_trace_rec* out, size_t cap, size_t* n_out) {
  size_t m = ctx->tr_n < cap ? ctx->tr_n : cap;
  if (m && out) memcpy(out, ctx->tr, m * sizeof(abx_trace_rec));
  *n_out = ctx->tr_n;
  return ABX_OK;
}

/* ------------------------------------------------------- construction */
static double leg(unsigned n, double x) {
  /* LegendreDistribution::legendre (include/materials/legendre_distribution.hpp:160-193) */
  switch (n) {
    case 0: return 1.;
    case 1: return x;
    case 2: return 0.5 * (3. * x * x - 1.);
    case 3: return 0.5 * (5. * x * x * x - 3. * x);
    case 4: { const double x2 = x * x; return 0.125 * (35. * x2 * x2 - 30. * x2 + 3.); }
    default: {
      const double x2 = x * x, x3 = x2 * x, x4 = x3 * x;
      double p3 = 0.5 * (5. * x3 - 3. * x);
      double p4 = 0.125 * (35. * x4 - 30. * x2 + 3.);
      unsigned l = 4;
      while (l < n) {
        double tmp = p3; p3 = p4; p4 = tmp;
        p4 = ((2. * l + 1.) * x * p3 - l * p4) / (l + 1.);
        l++;
      }
      return p4;
    }
  }
}
static double leg_pdf(const double* a, int na, double mu) {
  double p = 0;
  for (int l = 0; l < na; l++) p += a[l] * leg((unsigned)l, mu);
  return p;
}

/* LegendreDistribution::linearize (src/legendre_distribution.cpp:105-155) */
static int linearize(const double* a, int na, double** mu_o, double** p_o, double** c_o, int* n_o) {
  int cap = 64, n = 2;
  double* mu = (double*)malloc((size_t)cap * sizeof(double));
  double* p = (double*)malloc((size_t)cap * sizeof(double));
  mu[0] = -1.; mu[1] = 1.;
  p[0] = leg_pdf(a, na, -1.);
  p[1] = leg_pdf(a, na, 1.);
  int i = 0;
  while (i < n - 1) {
    double mu_mid = 0.5 * (mu[i] + mu[i + 1]);
    double p_interp = 0.5 * (p[i] + p[i + 1]);
    double p_real = leg_pdf(a, na, mu_mid);
    double rel = fabs(p_interp - p_real) / p_real;
    if (rel > TOLERANCE_LIN) {
      if (n == cap) {
        cap *= 2;
        mu = (double*)realloc(mu, (size_t)cap * sizeof(double));
        p = (double*)realloc(p, (size_t)cap * sizeof(double));
      }
      memmove(mu + i + 2, mu + i + 1, (size_t)(n - i - 1) * sizeof(double));
      memmove(p + i + 2, p + i + 1, (size_t)(n - i - 1) * sizeof(double));
      mu[i + 1] = mu_mid;
      p[i + 1] = p_real;
      n++;
      if (n > 100000) return 0;
    } else {
      i++;
    }
  }
  double* c = (double*)calloc((size_t)n, sizeof(double));
  for (int k = 0; k < n - 1; k++) c[k + 1] = ((mu[k + 1] - mu[k]) * 0.5 * (p[k + 1] + p[k])) + c[k];
  const double norm = c[n - 1];
  for (int k = 0; k < n; k++) { p[k] /= norm; c[k] /= norm; }
  *mu_o = mu; *p_o = p; *c_o = c; *n_o = n;
  return 1;
}

void oracle_destroy(oracle_ctx* ctx) {
  if (!ctx) return;
  free(ctx->eb); free(ctx->surf); free(ctx->cell);
  if (ctx->crpn) for (int i = 0; i < ctx->ncell; i++) free(ctx->crpn[i]);
  free(ctx->crpn); free(ctx->crpn_len); free(ctx->csimple); free(ctx->chasbc); free(ctx->creentry);
  free(ctx->univ); free(ctx->uhasbc);
  free(ctx->lat_xl); free(ctx->lat_yl); free(ctx->lat_zl);
  free(ctx->lat_pxi); free(ctx->lat_pyi); free(ctx->lat_pzi);
  free(ctx->cell_lists); free(ctx->lat_elems);
  free(ctx->Et); free(ctx->Eabs); free(ctx->Ef); free(ctx->nu_tot); free(ctx->nu_d);
  free(ctx->restart);
  free(ctx->Es); free(ctx->vEf); free(ctx->ps_cdf); free(ctx->chi_cdf); free(ctx->fissile);
  if (ctx->dg_cdf) for (int m = 0; m < ctx->M; m++) { free(ctx->dg_cdf[m]); free(ctx->dg_lambda[m]); }
  free(ctx->dg_cdf); free(ctx->dg_lambda); free(ctx->n_dg);
  free(ctx->ang); free(ctx->ang_mu); free(ctx->ang_pdf); free(ctx->ang_cdf); free(ctx->maj); free(ctx->smp);
  for (int t = 0; t < ctx->ntally; t++) {
    free(ctx->tally[t].eb); free(ctx->tally[t].gen); free(ctx->tally[t].avg); free(ctx->tally[t].var);
  }
  free(ctx->tally); free(ctx->src); free(ctx->src_cdf); free(ctx->tr);
  free(ctx);
}

int oracle_majorant(oracle_ctx* ctx, double* out) {
  memcpy(out, ctx->maj, (size_t)ctx->G * sizeof(double));
  return ABX_OK;
}
int oracle_scatter_cdf(oracle_ctx* ctx, int mat, int g, double* out) {
  if (mat < 0 || mat >= ctx->M || g < 0 || g >= ctx->G) return ABX_ERR_INVALID;
  memcpy(out, ctx->ps_cdf + ((size_t)mat * ctx->G + g) * ctx->G, (size_t)ctx->G * sizeof(double));
  return ABX_OK;
}

int oracle_create(const abx_problem* P, oracle_ctx** out) {
  BOUNDRY_TOL_ = 500. * SURFACE_COINCIDENT;
  TILE_TOL_ = 100 * SURFACE_COINCIDENT;
  if (!P || !out) return ABX_ERR_INVALID;
  oracle_ctx* ctx = (oracle_ctx*)xcalloc(1, sizeof(oracle_ctx));
  ctx->set = P->settings;
  const int G = ctx->G = P->settings.ngroups;
  if (G < 1 || G > 256) { set_err("bad ngroups"); oracle_destroy(ctx); return ABX_ERR_INVALID; }
  ctx->eb = (double*)xcalloc((size_t)G + 1, sizeof(double));
  memcpy(ctx->eb, P->energy_bounds, ((size_t)G + 1) * sizeof(double));
  /* settings::min/max_energy from the materials' energy bounds (src/parser.cpp:157-168) */
  ctx->min_energy = 0.;
  ctx->max_energy = 100000.;
  if (ctx->eb[0] > ctx->min_energy) ctx->min_energy = ctx->eb[0];
  if (ctx->eb[G] < ctx->max_energy) ctx->max_energy = ctx->eb[G];
  /* geometry */
  ctx->nsurf = P->n_surfaces;
  ctx->surf = (abx_surface*)xcalloc((size_t)P->n_surfaces, sizeof(abx_surface));
  memcpy(ctx->surf, P->surfaces, (size_t)P->n_surfaces * sizeof(abx_surface));
  ctx->ncell = P->n_cells;
  ctx->cell = (abx_cell*)xcalloc((size_t)P->n_cells, sizeof(abx_cell));
  memcpy(ctx->cell, P->cells, (size_t)P->n_cells * sizeof(abx_cell));
  ctx->crpn = (int32_t**)xcalloc((size_t)P->n_cells, sizeof(int32_t*));
  ctx->crpn_len = (int*)xcalloc((size_t)P->n_cells, sizeof(int));
  ctx->csimple = (int*)xcalloc((size_t)P->n_cells, sizeof(int));
  ctx->chasbc = (int*)xcalloc((size_t)P->n_cells, sizeof(int));
  ctx->creentry = (int*)xcalloc((size_t)P->n_cells, sizeof(int));
  for (int c = 0; c < P->n_cells; c++) {
    const abx_cell* C = &P->cells[c];
    const int32_t* r = P->rpn + C->rpn_offset;
    int simple = 1;
    for (int k = 0; k < C->rpn_len; k++)
      if (r[k] == ABX_OP_COMP || r[k] == ABX_OP_UNIN) { simple = 0; break; }
    /* Cell::simplify (src/cell.cpp:222-246) */
    ctx->crpn[c] = (int32_t*)xcalloc((size_t)C->rpn_len, sizeof(int32_t));
    int n = 0;
    for (int k = 0; k < C->rpn_len; k++) {
      if (simple && r[k] >= ABX_OP_UNIN) continue;
      int32_t t = r[k];
      if (t < ABX_OP_UNIN && (abs(t) < 1 || abs(t) > P->n_surfaces)) {
        set_err("cell %u references surface token %d out of range", C->id, t);
        oracle_destroy(ctx);
        return ABX_ERR_INVALID;
      }
      ctx->crpn[c][n++] = t;
    }
    ctx->crpn_len[c] = n;
    ctx->csimple[c] = simple;
    /* Cell::check_for_bc (src/cell.cpp:208-220) */
    for (int k = 0; k < n; k++) {
      int32_t t = ctx->crpn[c][k];
      if (t >= ABX_OP_UNIN) continue;
      int bc = P->surfaces[abs(t) - 1].bc;
      if (bc == ABX_BC_VACUUM || bc == ABX_BC_REFLECTIVE) ctx->chasbc[c] = 1;
    }
    ctx->creentry[c] = 0;
    for (int u = 0; u < P->n_universes; u++)
      if (P->universes[u].id == C->id) { ctx->creentry[c] = u; break; }
  }
  ctx->nuniv = P->n_universes;
  ctx->univ = (abx_universe*)xcalloc((size_t)P->n_universes, sizeof(abx_universe));
  memcpy(ctx->univ, P->universes, (size_t)P->n_universes * sizeof(abx_universe));
  ctx->cell_lists = (int32_t*)xcalloc((size_t)P->n_cell_lists, sizeof(int32_t));
  memcpy(ctx->cell_lists, P->cell_lists, (size_t)P->n_cell_lists * sizeof(int32_t));
  ctx->lat_elems = (int32_t*)xcalloc((size_t)P->n_lattice_elems, sizeof(int32_t));
  memcpy(ctx->lat_elems, P->lattice_elems, (size_t)P->n_lattice_elems * sizeof(int32_t));
  ctx->uhasbc = (int*)xcalloc((size_t)ctx->nuniv, sizeof(int));
  ctx->lat_xl = (double*)xcalloc((size_t)ctx->nuniv, sizeof(double));
  ctx->lat_yl = (double*)xcalloc((size_t)ctx->nuniv, sizeof(double));
  ctx->lat_zl = (double*)xcalloc((size_t)ctx->nuniv, sizeof(double));
  ctx->lat_pxi = (double*)xcalloc((size_t)ctx->nuniv, sizeof(double));
  ctx->lat_pyi = (double*)xcalloc((size_t)ctx->nuniv, sizeof(double));
  ctx->lat_pzi = (double*)xcalloc((size_t)ctx->nuniv, sizeof(double));
  for (int u = 0; u < ctx->nuniv; u++) {
    const abx_universe* U = &ctx->univ[u];
    if (U->kind == ABX_UNIV_CELLS) {
      /* CellUniverse ctor (src/cell_universe.cpp:30-41) */
      for (int k = 0; k < U->list_len; k++)
        if (ctx->chasbc[ctx->cell_lists[U->list_offset + k]]) { ctx->uhasbc[u] = 1; break; }
    } else {
      /* RectLattice ctor (src/rect_lattice.cpp:33-52) */
      ctx->lat_pxi[u] = 1. / U->pitch[0];
      ctx->lat_pyi[u] = 1. / U->pitch[1];
      ctx->lat_pzi[u] = 1. / U->pitch[2];
      ctx->lat_xl[u] = U->origin[0] - (double)U->shape[0] * 0.5 * U->pitch[0];
      ctx->lat_yl[u] = U->origin[1] - (double)U->shape[1] * 0.5 * U->pitch[1];
      ctx->lat_zl[u] = U->origin[2] - (double)U->shape[2] * 0.5 * U->pitch[2];
    }
  }
  /* Lattice::set_outisde_universe (src/lattice.cpp:45-53): lattices inherit
   * the outer universe's flag; resolve in index order (outer universes are
   * created before the lattice that names them). */
  for (int pass = 0; pass < 8; pass++)
    for (int u = 0; u < ctx->nuniv; u++) {
      const abx_universe* U = &ctx->univ[u];
      if (U->kind == ABX_UNIV_RECT_LATTICE)
        ctx->uhasbc[u] = U->outer >= 0 ? ctx->uhasbc[U->outer] : 0;
    }
  ctx->root = P->root_universe;
  /* materials (src/mg_nuclide.cpp:37-118, 394-411) */
  const int M = ctx->M = P->n_materials;
  ctx->Et = (double*)xcalloc((size_t)M * G, sizeof(double));
  ctx->Eabs = (double*)xcalloc((size_t)M * G, sizeof(double));
  ctx->Ef = (double*)xcalloc((size_t)M * G, sizeof(double));
  ctx->nu_tot = (double*)xcalloc((size_t)M * G, sizeof(double));
  ctx->nu_d = (double*)xcalloc((size_t)M * G, sizeof(double));
  ctx->Es = (double*)xcalloc((size_t)M * G, sizeof(double));
  ctx->vEf = (double*)xcalloc((size_t)M * G, sizeof(double));
  ctx->ps_cdf = (double*)xcalloc((size_t)M * G * G, sizeof(double));
  ctx->chi_cdf = (double*)xcalloc((size_t)M * G * G, sizeof(double));
  ctx->fissile = (int*)xcalloc((size_t)M, sizeof(int));
  ctx->n_dg = (int*)xcalloc((size_t)M, sizeof(int));
  ctx->dg_cdf = (double**)xcalloc((size_t)M, sizeof(double*));
  ctx->dg_lambda = (double**)xcalloc((size_t)M, sizeof(double*));
  ctx->ang = (AngleTab*)xcalloc((size_t)M * G * G, sizeof(AngleTab));
  int ang_cap = 4 * M * G * G + 16;
  ctx->ang_mu = (double*)xcalloc((size_t)ang_cap, sizeof(double));
  ctx->ang_pdf = (double*)xcalloc((size_t)ang_cap, sizeof(double));
  ctx->ang_cdf = (double*)xcalloc((size_t)ang_cap, sizeof(double));
  ctx->ang_n = 0;
  double* row = (double*)xcalloc((size_t)G, sizeof(double));
  for (int m = 0; m < M; m++) {
    const abx_material* mt = &P->materials[m];
    const double* d = P->mg_data + mt->data_offset;
    const double* tot = d;
    const double* abs_ = d + G;
    const double* fis = d + 2 * G;
    const double* nup = d + 3 * G;
    const double* nud = d + 4 * G;
    const double* chi = d + 5 * G;
    const double* sct = d + 5 * G + G * G;
    const double* leg_m = d + 5 * G + 2 * G * G;
    const double* dgp = leg_m + (size_t)mt->n_legendre * G * G;
    const double* dgl = dgp + mt->n_delayed;
    for (int g = 0; g < G; g++) {
      MAT_AT(ctx->Et, m, g) = tot[g];
      MAT_AT(ctx->Ef, m, g) = fis[g];
      MAT_AT(ctx->Eabs, m, g) = fis[g] + (abs_[g] - fis[g]);
      MAT_AT(ctx->nu_tot, m, g) = nup[g] + nud[g];
      MAT_AT(ctx->nu_d, m, g) = nud[g];
      MAT_AT(ctx->vEf, m, g) = 1. * (nup[g] + nud[g]) * fis[g];
      if (fis[g] != 0. && (nup[g] + nud[g]) > 0.) ctx->fissile[m] = 1;
      /* make_scatter_xs: row sums, row-normalised Ps */
      double es = 0.;
      for (int o = 0; o < G; o++) es += sct[(size_t)g * G + o];
      MAT_AT(ctx->Es, m, g) = es;
      for (int o = 0; o < G; o++) row[o] = sct[(size_t)g * G + o] / es;
      make_discrete_cdf(row, G, ctx->ps_cdf + ((size_t)m * G + g) * G);
      /* normalize_chi */
      double ci = 0.;
      for (int o = 0; o < G; o++) ci += chi[(size_t)g * G + o];
      for (int o = 0; o < G; o++) row[o] = chi[(size_t)g * G + o] / ci;
      make_discrete_cdf(row, G, ctx->chi_cdf + ((size_t)m * G + g) * G);
    }
    ctx->n_dg[m] = mt->n_delayed;
    ctx->dg_cdf[m] = (double*)xcalloc((size_t)mt->n_delayed + 1, sizeof(double));
    ctx->dg_lambda[m] = (double*)xcalloc((size_t)mt->n_delayed + 1, sizeof(double));
    make_discrete_cdf(dgp, mt->n_delayed, ctx->dg_cdf[m]);
    memcpy(ctx->dg_lambda[m], dgl, (size_t)mt->n_delayed * sizeof(double));
    /* angle tables: LegendreDistribution default a_={0.5}, set_moment(l,c)
     * a_[l] = c*(2l+1)/2 (legendre_distribution.hpp:92-103) */
    for (int gi = 0; gi < G; gi++)
      for (int go = 0; go < G; go++) {
        double a[6] = {0.5, 0, 0, 0, 0, 0};
        int na = 1;
        for (int l = 1; l <= mt->n_legendre; l++) {
          double coeff = leg_m[((size_t)(l - 1) * G + gi) * G + go];
          a[l] = coeff * (2. * (double)l + 1.) / 2.;
          na = l + 1;
        }
        double *mu, *pp, *cc;
        int npt;
        if (!linearize(a, na, &mu, &pp, &cc, &npt)) {
          set_err("angle linearisation did not converge");
          free(row); oracle_destroy(ctx); return ABX_ERR_INVALID;
        }
        if (ctx->ang_n + npt > ang_cap) {
          ang_cap = 2 * (ctx->ang_n + npt);
          ctx->ang_mu = (double*)realloc(ctx->ang_mu, (size_t)ang_cap * sizeof(double));
          ctx->ang_pdf = (double*)realloc(ctx->ang_pdf, (size_t)ang_cap * sizeof(double));
          ctx->ang_cdf = (double*)realloc(ctx->ang_cdf, (size_t)ang_cap * sizeof(double));
        }
        AngleTab* at = &ctx->ang[((size_t)m * G + gi) * G + go];
        at->off = ctx->ang_n; at->n = npt;
        memcpy(ctx->ang_mu + ctx->ang_n, mu, (size_t)npt * sizeof(double));
        memcpy(ctx->ang_pdf + ctx->ang_n, pp, (size_t)npt * sizeof(double));
        memcpy(ctx->ang_cdf + ctx->ang_n, cc, (size_t)npt * sizeof(double));
        ctx->ang_n += npt;
        free(mu); free(pp); free(cc);
      }
  }
  free(row);
  /* make_majorant_xs, multigroup branch (src/majorant.cpp:132-176); the
   * piecewise-constant grid evaluates to the group's value at any energy
   * inside the group. */
  ctx->maj = (double*)xcalloc((size_t)G, sizeof(double));
  for (int m = 0; m < M; m++)
    for (int g = 0; g < G; g++) {
      double xs = MAT_AT(ctx->Et, m, g);
      if (xs > ctx->maj[g]) ctx->maj[g] = xs;
    }
  /* CarterTracker ctor (src/carter_tracker.cpp:60-72): the majorant at the
   * group's mid energy times the deck's sampling-xs-ratio */
  ctx->smp = (double*)xcalloc((size_t)G, sizeof(double));
  for (int g = 0; g < G; g++) ctx->smp[g] = ctx->maj[g] * (P->sampling_xs_ratio ? P->sampling_xs_ratio[g] : 1.0);
  /* tallies */
  ctx->ntally = P->n_tallies;
  ctx->tally = (OTally*)xcalloc((size_t)P->n_tallies, sizeof(OTally));
  for (int t = 0; t < P->n_tallies; t++) {
    const abx_mesh_tally* D = &P->tallies[t];
    OTally* T = &ctx->tally[t];
    T->est = D->estimator; T->quantity = D->quantity;
    for (int a = 0; a < 3; a++) {
      T->N[a] = D->shape[a]; T->low[a] = D->low[a]; T->hi[a] = D->hi[a];
      T->d[a] = (D->hi[a] - D->low[a]) / (double)D->shape[a];
      T->dinv[a] = 1. / T->d[a];
    }
    T->ne = D->n_ebounds - 1;
    T->eb = (double*)xcalloc((size_t)D->n_ebounds, sizeof(double));
    memcpy(T->eb, P->tally_ebounds + D->ebounds_offset, (size_t)D->n_ebounds * sizeof(double));
    T->nbins = (size_t)T->ne * T->N[0] * T->N[1] * T->N[2];
    T->gen = (double*)xcalloc(T->nbins, sizeof(double));
    T->avg = (double*)xcalloc(T->nbins, sizeof(double));
    T->var = (double*)xcalloc(T->nbins, sizeof(double));
  }
  ctx->ent_on = P->entropy.enabled;
  for (int a = 0; a < 3; a++) {
    ctx->ent_shape[a] = P->entropy.shape[a];
    ctx->ent_low[a] = P->entropy.low[a];
    ctx->ent_d[a] = P->entropy.enabled ? (P->entropy.hi[a] - P->entropy.low[a]) / (double)P->entropy.shape[a] : 1.;
  }
  /* sources (src/simulation.cpp:58-59) */
  ctx->nsrc = P->n_sources;
  ctx->src = (abx_source*)xcalloc((size_t)P->n_sources, sizeof(abx_source));
  memcpy(ctx->src, P->sources, (size_t)P->n_sources * sizeof(abx_source));
  ctx->src_cdf = (double*)xcalloc((size_t)P->n_sources + 1, sizeof(double));
  {
    double* w = (double*)xcalloc((size_t)P->n_sources + 1, sizeof(double));
    for (int s = 0; s < P->n_sources; s++) w[s] = P->sources[s].weight;
    make_discrete_cdf(w, P->n_sources, ctx->src_cdf);
    free(w);
  }
  *out = ctx;
  return ABX_OK;
}
