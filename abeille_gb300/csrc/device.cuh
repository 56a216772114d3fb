// Device-side building blocks of the GB300 multigroup transport engine.
//
// Everything here is templated on the tracking precision R (double for the
// FP64 parity mode, float for the mixed mode).  The FP64 instantiations live in
// a translation unit compiled with --fmad=false, so every double operation
// rounds where the reference's does (Abeille v0.4.0, paths below relative to
// its source tree).
#pragma once

#include <cfloat>
#include <cstdint>

#include "tables.h"

namespace abx {

#define ABX_DEV __device__ __forceinline__

// ------------------------------------------------------------- tolerances
// FP64 values are the reference's (include/utils/constants.hpp:42-57,
// src/rect_lattice.cpp:270-281, src/cell.cpp:97-101, direction.hpp:140).
// FP32 values are the mixed mode's: a few float ulps at the 100 cm scale.
template <class R> struct Tol;
template <> struct Tol<double> {
  static constexpr double INF = DBL_MAX;
  static constexpr double SC = 1e-12;             // SURFACE_COINCIDENT
  static constexpr double SCD = 1e-12;            // plane on-surface band
  static constexpr double SCQ = 1e-12;            // quadric on-surface band
  static constexpr double BTOL = 500. * 1e-12;    // BOUNDRY_TOL
  static constexpr double TILE = 100 * 1e-12;     // tile-wall skip
  static constexpr double REL = 1e-14;            // relative distance tie
  static constexpr double ROT = 1.E-10;           // rotate_direction pole test
  static constexpr double MAJ = 1.E-10;           // Et > majorant check
};
template <> struct Tol<float> {
  static constexpr float INF = FLT_MAX;
  static constexpr float SC = 2e-5f;   // sign ties and lattice-face nudges
  static constexpr float SCD = 0.f;    // planes: "on surface" only through the surface token
  static constexpr float SCQ = 1e-6f;  // quadrics: |c| band treated as on-surface
  static constexpr float BTOL = 4e-5f;
  static constexpr float TILE = 4e-5f;
  static constexpr float REL = 1e-6f;
  static constexpr float ROT = 1e-2f;
  static constexpr float MAJ = 0.f;
};

ABX_DEV double m_log(double x) { return log(x); }
ABX_DEV float m_log(float x) { return logf(x); }
ABX_DEV double m_exp(double x) { return exp(x); }
ABX_DEV float m_exp(float x) { return expf(x); }
ABX_DEV double m_sqrt(double x) { return sqrt(x); }
ABX_DEV float m_sqrt(float x) { return sqrtf(x); }
ABX_DEV double m_floor(double x) { return floor(x); }
ABX_DEV float m_floor(float x) { return floorf(x); }
ABX_DEV double m_abs(double x) { return fabs(x); }
ABX_DEV float m_abs(float x) { return fabsf(x); }

template <class R> struct V3 {
  R x, y, z;
};
template <class R> ABX_DEV V3<R> mk(R x, R y, R z) { V3<R> v; v.x = x; v.y = y; v.z = z; return v; }
template <class R> ABX_DEV V3<R> add(V3<R> a, V3<R> b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
template <class R> ABX_DEV V3<R> sub(V3<R> a, V3<R> b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
template <class R> ABX_DEV V3<R> scl(V3<R> v, R c) { return mk(v.x * c, v.y * c, v.z * c); }
template <class R> ABX_DEV R dot(V3<R> a, V3<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class R> ABX_DEV V3<R> dir3(R x, R y, R z) {
  // Direction(x,y,z) renormalises (include/utils/direction.hpp:37-42)
  R m = m_sqrt(x * x + y * y + z * z);
  return mk(x / m, y / m, z / m);
}

// --------------------------------------------------------------- pcg32
// pcg-cpp setseq_xsh_rr_64_32 on its default stream: LCG step with the
// previous state's XSH-RR output (O'Neill, "PCG: A Family of Simple Fast
// Space-Efficient Statistically Good Algorithms for RNG", 2014).
constexpr uint64_t PCG_MULT = 6364136223846793005ULL;
constexpr uint64_t PCG_INC = 1442695040888963407ULL;

ABX_DEV uint32_t pcg_next(uint64_t& s) {
  uint64_t old = s;
  s = old * PCG_MULT + PCG_INC;
  uint32_t rot = (uint32_t)(old >> 59);
  uint32_t xs = (uint32_t)(((old >> 18) ^ old) >> 27);
  return __funnelshift_r(xs, xs, rot);
}
// Jump ahead by delta steps (F. B. Brown, "Random number generation with
// arbitrary strides", Trans. Am. Nucl. Soc. 71, 1994).
__host__ __device__ inline uint64_t pcg_advance(uint64_t state, uint64_t delta) {
  uint64_t cm = PCG_MULT, cp = PCG_INC, am = 1u, ap = 0u;
  while (delta > 0) {
    if (delta & 1u) {
      am *= cm;
      ap = ap * cm + cp;
    }
    cp = (cm + 1u) * cp;
    cm *= cm;
    delta >>= 1;
  }
  return am * state + ap;
}
__host__ __device__ inline uint64_t pcg_seeded(uint64_t seed) {
  return (seed + PCG_INC) * PCG_MULT + PCG_INC;
}

// libstdc++ generate_canonical<double,53> over a 32-bit engine: two outputs.
ABX_DEV double canon_d(uint64_t& s) {
  double sum = (double)pcg_next(s);
  sum += (double)pcg_next(s) * 4294967296.0;
  double r = sum / 18446744073709551616.0;
  if (r >= 1.0) r = 0x1.fffffffffffffp-1;
  return r;
}
// Mixed mode: the same two outputs, truncated to 24 bits (always < 1).
ABX_DEV float canon_f(uint64_t& s) {
  (void)pcg_next(s);
  uint32_t hi = pcg_next(s);
  return (float)(hi >> 8) * 0x1p-24f;
}
template <class R> ABX_DEV R canon(uint64_t& s);
template <> ABX_DEV double canon<double>(uint64_t& s) { return canon_d(s); }
template <> ABX_DEV float canon<float>(uint64_t& s) { return canon_f(s); }

// std::lower_bound: first i with !(cp[i] < u).
template <class R> ABX_DEV int lower_bound(const R* __restrict__ cp, int n, R u) {
  int first = 0, count = n;
  while (count > 0) {
    int step = count >> 1;
    int it = first + step;
    if (__ldg(cp + it) < u) {
      first = it + 1;
      count -= step + 1;
    } else {
      count = step;
    }
  }
  return first;
}
// discrete_distribution::operator(): no draw with fewer than two weights.
template <class R> ABX_DEV int discrete(uint64_t& s, const R* cp, int n) {
  if (n < 2) return 0;
  R u = canon<R>(s);
  return lower_bound<R>(cp, n, u);
}

// ----------------------------------------------------------- table views
template <class R> struct View {
  const SurfT<R>* __restrict__ surf;
  const LatT<R>* __restrict__ lat;
  const R* __restrict__ xs;     // per material: Et Eabs Ef nu_tot nu_d Es vEf (G each)
  const R* __restrict__ cdf;    // scatter and chi CDF rows
  const R* __restrict__ ang;    // angle tables: mu | pdf | cdf runs
  const R* __restrict__ ebnd;   // energy bounds pool
  const R* __restrict__ maj;    // majorant pool
  const R* __restrict__ dgcdf;  // delayed-group CDFs
};

// ------------------------------------------------------------- surfaces
// src/{x,y,z}plane.cpp:32-56, plane.cpp:33-60, {x,y,z}cylinder.cpp:33-80, sphere.cpp:33-80
template <class R> ABX_DEV V3<R> surf_norm(const SurfT<R>& s, V3<R> r) {
  switch (s.type) {
    case ABX_SURF_XPLANE: return dir3<R>(1, 0, 0);
    case ABX_SURF_YPLANE: return dir3<R>(0, 1, 0);
    case ABX_SURF_ZPLANE: return dir3<R>(0, 0, 1);
    case ABX_SURF_PLANE: return dir3<R>(s.c[0], s.c[1], s.c[2]);
    case ABX_SURF_XCYLINDER: return dir3<R>(0, r.y - s.c[0], r.z - s.c[1]);
    case ABX_SURF_YCYLINDER: return dir3<R>(r.x - s.c[0], 0, r.z - s.c[1]);
    case ABX_SURF_ZCYLINDER: return dir3<R>(r.x - s.c[0], r.y - s.c[1], 0);
    default: return dir3<R>(r.x - s.c[0], r.y - s.c[1], r.z - s.c[2]);
  }
}

template <class R> ABX_DEV R surf_eval(const SurfT<R>& s, V3<R> r) {
  switch (s.type) {
    case ABX_SURF_XPLANE: return r.x - s.c[0];
    case ABX_SURF_YPLANE: return r.y - s.c[0];
    case ABX_SURF_ZPLANE: return r.z - s.c[0];
    case ABX_SURF_PLANE: return s.c[0] * r.x + s.c[1] * r.y + s.c[2] * r.z - s.c[3];
    case ABX_SURF_XCYLINDER: {
      R y = r.y - s.c[0], z = r.z - s.c[1], Rr = s.c[2];
      return y * y + z * z - Rr * Rr;
    }
    case ABX_SURF_YCYLINDER: {
      R x = r.x - s.c[0], z = r.z - s.c[1], Rr = s.c[2];
      return x * x + z * z - Rr * Rr;
    }
    case ABX_SURF_ZCYLINDER: {
      R x = r.x - s.c[0], y = r.y - s.c[1], Rr = s.c[2];
      return y * y + x * x - Rr * Rr;
    }
    default: {
      R x = r.x - s.c[0], y = r.y - s.c[1], z = r.z - s.c[2], Rr = s.c[3];
      return (x * x) + (y * y) + (z * z) - Rr * Rr;
    }
  }
}

template <class R> ABX_DEV int surf_sign(const SurfT<R>& s, V3<R> r, V3<R> u) {
  R e = surf_eval(s, r);
  if (e > Tol<R>::SC) return 1;
  if (e < -Tol<R>::SC) return -1;
  return dot(u, surf_norm(s, r)) > R(0) ? 1 : -1;
}

template <class R> ABX_DEV R axis_dist(R diff, R ua, bool on) {
  if (on || m_abs(diff) < Tol<R>::SCD || ua == R(0)) return Tol<R>::INF;
  if (diff / ua < R(0)) return Tol<R>::INF;
  return diff / ua;
}

// Quadratic surface distance.  In the mixed mode the root is recomputed in
// FP64 when the discriminant is small against k^2 (grazing incidence), where
// FP32 cancellation would dominate.
template <class R> ABX_DEV R quad_dist(R a, R k, R c, R quad, bool on) {
  if (quad < R(0)) return Tol<R>::INF;
  if (on || m_abs(c) < Tol<R>::SCQ) {
    if (k >= R(0)) return Tol<R>::INF;
    return (-k + m_sqrt(quad)) / a;
  }
  if (c < R(0)) return (-k + m_sqrt(quad)) / a;
  R d = (-k - m_sqrt(quad)) / a;
  if (d < R(0)) return Tol<R>::INF;
  return d;
}

template <class R> ABX_DEV R grazing_fix(R a, R k, R c, bool on) {
  double ad = a, kd = k, cd = c;
  double q = kd * kd - ad * cd;
  if (q < 0.) return Tol<R>::INF;
  if (on || fabs(cd) < (double)Tol<R>::SCQ) {
    if (kd >= 0.) return Tol<R>::INF;
    return (R)((-kd + sqrt(q)) / ad);
  }
  if (cd < 0.) return (R)((-kd + sqrt(q)) / ad);
  double d = (-kd - sqrt(q)) / ad;
  if (d < 0.) return Tol<R>::INF;
  return (R)d;
}

template <class R> ABX_DEV R surf_dist(const SurfT<R>& s, V3<R> r, V3<R> u, bool on) {
  switch (s.type) {
    case ABX_SURF_XPLANE: return axis_dist<R>(s.c[0] - r.x, u.x, on);
    case ABX_SURF_YPLANE: return axis_dist<R>(s.c[0] - r.y, u.y, on);
    case ABX_SURF_ZPLANE: return axis_dist<R>(s.c[0] - r.z, u.z, on);
    case ABX_SURF_PLANE: {
      R num = s.c[3] - s.c[0] * r.x - s.c[1] * r.y - s.c[2] * r.z;
      R den = s.c[0] * u.x + s.c[1] * u.y + s.c[2] * u.z;
      R d = num / den;
      if (on || m_abs(d) < Tol<R>::SCD || den == R(0)) return Tol<R>::INF;
      if (d < R(0)) return Tol<R>::INF;
      return d;
    }
    case ABX_SURF_SPHERE: {
      R x = r.x - s.c[0], y = r.y - s.c[1], z = r.z - s.c[2], Rr = s.c[3];
      R k = x * u.x + y * u.y + z * u.z;
      R c = x * x + y * y + z * z - Rr * Rr;
      R quad = k * k - c;
      if (sizeof(R) == 4 && quad >= R(0) && quad < R(1e-3) * k * k) return grazing_fix<R>(R(1), k, c, on);
      return quad_dist<R>(R(1), k, c, quad, on);
    }
    default: {
      R p, q, up, uq, Rr = s.c[2];
      if (s.type == ABX_SURF_ZCYLINDER) {
        p = r.y - s.c[1]; q = r.x - s.c[0]; up = u.y; uq = u.x;
      } else if (s.type == ABX_SURF_XCYLINDER) {
        p = r.y - s.c[0]; q = r.z - s.c[1]; up = u.y; uq = u.z;
      } else {
        p = r.x - s.c[0]; q = r.z - s.c[1]; up = u.x; uq = u.z;
      }
      R a = up * up + uq * uq;
      if (a == R(0)) return Tol<R>::INF;
      R k = p * up + q * uq;
      R c = p * p + q * q - Rr * Rr;
      R quad = k * k - a * c;
      if (sizeof(R) == 4 && quad >= R(0) && quad < R(1e-3) * k * k) return grazing_fix<R>(a, k, c, on);
      return quad_dist<R>(a, k, c, quad, on);
    }
  }
}

// ----------------------------------------------------------------- cells
// Cell::is_inside_simple / is_inside_complex (src/cell.cpp:147-199).
// Called from the validity check after every flight and from the descent;
// compiled once, out of line, with pointer arguments: one copy of the
// surface-sign code instead of one per caller measurably cuts the loop's
// instruction-fetch stalls.
template <class R>
__device__ __noinline__ bool cell_inside_at(const CellT* __restrict__ cells, const int32_t* __restrict__ rpn_pool,
                                            const SurfT<R>* __restrict__ surf, int ci, V3<R> r, V3<R> u,
                                            int32_t on) {
  const CellT c = cells[ci];
  const int32_t* __restrict__ rpn = rpn_pool + c.rpn_off;
  if (c.simple) {
    for (int i = 0; i < c.rpn_len; i++) {
      int32_t t = __ldg(rpn + i);
      if (t == on) continue;
      if (-t == on) return false;
      int sg = surf_sign(surf[abs(t) - 1], r, u);
      if ((sg > 0 && t < 0) || (sg < 0 && t > 0)) return false;
    }
    return true;
  }
  uint64_t st = 0;  // bit stack
  int sp = -1;
  for (int i = 0; i < c.rpn_len; i++) {
    int32_t t = __ldg(rpn + i);
    if (t == ABX_OP_UNIN || t == ABX_OP_INTR) {
      uint64_t a = (st >> (sp - 1)) & 1u, b = (st >> sp) & 1u;
      uint64_t v = (t == ABX_OP_UNIN) ? (a | b) : (a & b);
      st = (st & ~(1ull << (sp - 1))) | (v << (sp - 1));
      sp--;
    } else if (t == ABX_OP_COMP) {
      st ^= (1ull << sp);
    } else {
      sp++;
      bool v;
      if (t == on) v = true;
      else if (-t == on) v = false;
      else {
        int sg = surf_sign(surf[abs(t) - 1], r, u);
        v = (sg > 0 && t > 0) || (sg < 0 && t < 0);
      }
      st = (st & ~(1ull << sp)) | ((uint64_t)v << sp);
    }
  }
  if (sp == 0) return (st & 1u) != 0;
  return true;
}

template <class R>
ABX_DEV bool cell_inside(const Tables& T, const View<R>& V, int ci, V3<R> r, V3<R> u, int32_t on) {
  return cell_inside_at<R>(T.cells, T.rpn, V.surf, ci, r, u, on);
}

// Cell::distance_to_boundary / distance_to_boundary_condition (src/cell.cpp:79-141)
template <class R>
ABX_DEV void cell_dist(const Tables& T, const View<R>& V, int ci, V3<R> r, V3<R> u, int32_t on,
                       bool bc_only, R& dist, int32_t& isurf) {
  const CellT c = T.cells[ci];
  R mind = Tol<R>::INF;
  int32_t is = 0;
  if (bc_only && !c.has_bc) {
    dist = mind;
    isurf = 0;
    return;
  }
  const int32_t* __restrict__ rpn = T.rpn + c.rpn_off;
  for (int i = 0; i < c.rpn_len; i++) {
    int32_t t = __ldg(rpn + i);
    if (t >= ABX_OP_UNIN) continue;
    bool co = abs(t) == abs(on);
    const SurfT<R> s = V.surf[abs(t) - 1];
    if (bc_only && s.bc == ABX_BC_NORMAL) continue;
    R d = surf_dist(s, r, u, co);
    if (d < mind) {
      if (m_abs(d - mind) / mind >= Tol<R>::REL) {
        mind = d;
        is = -t;
      }
    }
  }
  dist = mind;
  isurf = is;
}

// ------------------------------------------------------------- lattices
// RectLattice::tile_center / get_tile / distance_to_tile_boundary
// (src/rect_lattice.cpp:207-310)
template <class R> ABX_DEV V3<R> tile_center(const LatT<R>& L, int nx, int ny, int nz) {
  return mk<R>(((R)nx + R(0.5)) * L.p[0] + L.lo[0], ((R)ny + R(0.5)) * L.p[1] + L.lo[1],
               ((R)nz + R(0.5)) * L.p[2] + L.lo[2]);
}
template <class R> ABX_DEV void get_tile(const LatT<R>& L, V3<R> r, V3<R> u, int t[3]) {
  int nx = (int)m_floor((r.x - L.lo[0]) * L.pinv[0]);
  int ny = (int)m_floor((r.y - L.lo[1]) * L.pinv[1]);
  int nz = (int)m_floor((r.z - L.lo[2]) * L.pinv[2]);
  V3<R> c = tile_center(L, nx, ny, nz);
  R h0 = L.p[0] * R(0.5), h1 = L.p[1] * R(0.5), h2 = L.p[2] * R(0.5);
  R xl = c.x - h0, xh = c.x + h0, yl = c.y - h1, yh = c.y + h1, zl = c.z - h2, zh = c.z + h2;
  if (m_abs(xl - r.x) < Tol<R>::SC && u.x < R(0)) nx--;
  if (m_abs(xh - r.x) < Tol<R>::SC && u.x >= R(0)) nx++;
  if (m_abs(yl - r.y) < Tol<R>::SC && u.y < R(0)) ny--;
  if (m_abs(yh - r.y) < Tol<R>::SC && u.y >= R(0)) ny++;
  if (m_abs(zl - r.z) < Tol<R>::SC && u.z < R(0)) nz--;
  if (m_abs(zh - r.z) < Tol<R>::SC && u.z >= R(0)) nz++;
  t[0] = nx; t[1] = ny; t[2] = nz;
}
template <class R> ABX_DEV R tile_dist(const LatT<R>& L, V3<R> rl, V3<R> u, const int t[3]) {
  V3<R> rt = sub(rl, tile_center(L, t[0], t[1], t[2]));
  R dist = Tol<R>::INF;
  const R dxl = -L.p[0] * R(0.5) - rt.x, dxh = L.p[0] * R(0.5) - rt.x;
  const R dyl = -L.p[1] * R(0.5) - rt.y, dyh = L.p[1] * R(0.5) - rt.y;
  const R dzl = -L.p[2] * R(0.5) - rt.z, dzh = L.p[2] * R(0.5) - rt.z;
  const R ix = R(1) / u.x, iy = R(1) / u.y, iz = R(1) / u.z;
  const R a = dxl * ix, b = dxh * ix, c = dyl * iy, d = dyh * iy, e = dzl * iz, f = dzh * iz;
  if (a > R(0) && a < dist && m_abs(dxl) > Tol<R>::TILE) dist = a;
  if (b > R(0) && b < dist && m_abs(dxh) > Tol<R>::TILE) dist = b;
  if (c > R(0) && c < dist && m_abs(dyl) > Tol<R>::TILE) dist = c;
  if (d > R(0) && d < dist && m_abs(dyh) > Tol<R>::TILE) dist = d;
  if (e > R(0) && e < dist && m_abs(dzl) > Tol<R>::TILE) dist = e;
  if (f > R(0) && f < dist && m_abs(dzh) > Tol<R>::TILE) dist = f;
  return dist;
}

// --------------------------------------------------------- boundary type
template <class R> struct Bound {
  R dist;
  int si;
  int btype;
  int32_t token;
};

// CellUniverse::get_boundary_condition (src/cell_universe.cpp:107-147) and
// Lattice::get_boundary_condition (src/lattice.cpp:77-91)
template <class R>
ABX_DEV Bound<R> univ_bc(const Tables& T, const View<R>& V, int ui, V3<R> r, V3<R> u, int32_t on) {
  Bound<R> b{Tol<R>::INF, -1, ABX_BC_VACUUM, 0};
  for (int guard = 0; guard < 16; guard++) {
    const UnivT U = T.univ[ui];
    if (U.kind == ABX_UNIV_RECT_LATTICE) {
      if (U.has_bc) { ui = U.outer; continue; }
      return b;
    }
    if (U.has_bc) {
      for (int k = 0; k < U.list_len; k++) {
        int ci = __ldg(T.cell_lists + U.list_off + k);
        if (!T.cells[ci].has_bc) continue;
        R d; int32_t ts;
        cell_dist(T, V, ci, r, u, on, true, d, ts);
        if (d < b.dist && m_abs(d - b.dist) > Tol<R>::BTOL) {
          int32_t tmp = abs(ts);
          if (!tmp) continue;
          b.token = tmp; b.dist = d; b.si = tmp - 1;
          b.btype = V.surf[b.si].bc;
          if (surf_sign(V.surf[b.si], r, u) < 0) b.token = -b.token;
        }
      }
    }
    return b;
  }
  return b;
}

// ------------------------------------------------------------- tracker
// Per-particle navigation state (include/simulation/tracker.hpp:41-372).
// The reference keeps a vector of GeoLilyPad{type,id,r_local,tile}; pads
// created together hold equal r_local and move together, so positions are
// stored once per coordinate frame (a new frame starts at each lattice
// descent) and each pad records its frame.
constexpr int MAXD = 6;  // pads
constexpr int MAXF = 3;  // frames (lattice nesting + 1)
enum { PAD_UNIV = 0, PAD_LATT = 1, PAD_CELL = 2 };

ABX_DEV uint32_t pad_pack(int type, int frame, int idx) {
  return (uint32_t)type | ((uint32_t)frame << 2) | ((uint32_t)idx << 4);
}
ABX_DEV int pad_type(uint32_t p) { return (int)(p & 3u); }
ABX_DEV int pad_frame(uint32_t p) { return (int)((p >> 2) & 3u); }
ABX_DEV int pad_idx(uint32_t p) { return (int)(p >> 4); }
// Tile indices packed as three 10-bit fields, clamped to [-512, 511].  Lattice
// shapes are limited to 500 per axis, so every in-lattice tile is exact; two
// out-of-lattice tiles that clamp alike both send a lookup to the outer
// universe, so the clamp never changes which cell is found.
ABX_DEV uint32_t tile_pack(const int t[3]) {
  auto c = [](int v) -> uint32_t {
    v = v < -512 ? -512 : (v > 511 ? 511 : v);
    return (uint32_t)(v + 512) & 0x3FFu;
  };
  return c(t[0]) | (c(t[1]) << 10) | (c(t[2]) << 20);
}
ABX_DEV void tile_unpack(uint32_t p, int t[3]) {
  t[0] = (int)(p & 0x3FFu) - 512;
  t[1] = (int)((p >> 10) & 0x3FFu) - 512;
  t[2] = (int)((p >> 20) & 0x3FFu) - 512;
}

template <class R> struct Trk {
  V3<R> r, u;
  int32_t token;
  int depth;
  int cell;       // material cell, -1 when lost
  int err;        // first error
  uint32_t pad[MAXD];
  uint32_t tl[MAXD];
  V3<R> fr[MAXF];

  ABX_DEV uint32_t getpad(int k) const {
    uint32_t v = 0;
#pragma unroll
    for (int i = 0; i < MAXD; i++) if (i == k) v = pad[i];
    return v;
  }
  ABX_DEV uint32_t gettile(int k) const {
    uint32_t v = 0;
#pragma unroll
    for (int i = 0; i < MAXD; i++) if (i == k) v = tl[i];
    return v;
  }
  ABX_DEV V3<R> getfr(int f) const {
    V3<R> v = fr[0];
#pragma unroll
    for (int i = 1; i < MAXF; i++) if (i == f) v = fr[i];
    return v;
  }
  ABX_DEV void setfr(int f, V3<R> v) {
#pragma unroll
    for (int i = 0; i < MAXF; i++) if (i == f) fr[i] = v;
  }
  ABX_DEV bool push(uint32_t p, uint32_t t) {
    if (depth >= MAXD || pad_frame(p) >= MAXF) {
      err = ABX_ERR_INVALID;
      return false;
    }
#pragma unroll
    for (int i = 0; i < MAXD; i++)
      if (i == depth) { pad[i] = p; tl[i] = t; }
    depth++;
    return true;
  }
};

// CellUniverse::get_cell(stack,...) (src/cell_universe.cpp:69-104) and
// RectLattice::get_cell(stack,...) (src/rect_lattice.cpp:131-205), iterative.
template <class R>
ABX_DEV int univ_get_cell(const Tables& T, const View<R>& V, Trk<R>& k, int ui, int frame, V3<R> r) {
  k.setfr(frame, r);
  for (int guard = 0; guard < 16; guard++) {
    const UnivT U = T.univ[ui];
    if (U.kind == ABX_UNIV_CELLS) {
      if (!k.push(pad_pack(PAD_UNIV, frame, ui), 0)) return -1;
      int found = -1;
      for (int j = 0; j < U.list_len; j++) {
        int ci = __ldg(T.cell_lists + U.list_off + j);
        if (cell_inside(T, V, ci, r, k.u, k.token)) { found = ci; break; }
      }
      if (found < 0) return -1;
      if (!k.push(pad_pack(PAD_CELL, frame, found), 0)) return -1;
      const CellT c = T.cells[found];
      if (c.fill_kind == ABX_FILL_MATERIAL) return found;
      ui = c.fill;
      continue;
    }
    const LatT<R> L = V.lat[U.lat];
    int t[3];
    get_tile(L, r, k.u, t);
    bool inside = !(t[0] < 0 || t[0] >= U.n[0] || t[1] < 0 || t[1] >= U.n[1] || t[2] < 0 || t[2] >= U.n[2]);
    int fill = -1;
    if (inside) {
      uint32_t lin = (uint32_t)t[2] * ((uint32_t)U.n[0] * (uint32_t)U.n[1]) + (uint32_t)t[0] * (uint32_t)U.n[1] + (uint32_t)t[1];
      fill = __ldg(T.lat_elems + U.list_off + lin);
    }
    if (!k.push(pad_pack(PAD_LATT, frame, ui), tile_pack(t))) return -1;
    if (fill >= 0) {
      r = sub(r, tile_center(L, t[0], t[1], t[2]));
      frame++;
      if (frame >= MAXF) { k.err = ABX_ERR_INVALID; return -1; }
      k.setfr(frame, r);
      ui = fill;
      continue;
    }
    if (U.outer >= 0) { ui = U.outer; continue; }
    return -1;
  }
  k.err = ABX_ERR_INVALID;
  return -1;
}

// Tracker::restart_get_current (tracker.hpp:59-71)
template <class R> ABX_DEV void trk_restart(const Tables& T, const View<R>& V, const ProbT& P, Trk<R>& k) {
  k.depth = 0;
  k.cell = univ_get_cell(T, V, k, P.root, 0, k.r);
}
// Tracker::move (tracker.hpp:76-85): every frame moves by d*u.
template <class R> ABX_DEV void trk_move(Trk<R>& k, R d) {
  V3<R> du = scl(k.u, d);
  k.r = add(k.r, du);
  int nf = k.depth > 0 ? pad_frame(k.getpad(k.depth - 1)) + 1 : 1;
#pragma unroll
  for (int i = 0; i < MAXF; i++)
    if (i < nf) k.fr[i] = add(k.fr[i], du);
  k.token = 0;
}
template <class R> ABX_DEV void trk_set_r(Trk<R>& k, V3<R> r) {
  k.r = r;
  k.token = 0;
}

// Tracker::get_current (tracker.hpp:235-306)
template <class R> ABX_DEV void trk_current(const Tables& T, const View<R>& V, const ProbT& P, Trk<R>& k) {
  if (!(k.r.x == k.fr[0].x && k.r.y == k.fr[0].y && k.r.z == k.fr[0].z)) {
    trk_restart(T, V, P, k);
    return;  // a fresh tree is valid by construction
  }
  int first_bad = k.depth;
#pragma unroll
  for (int i = 0; i < MAXD; i++) {
    if (i < k.depth && first_bad == k.depth) {
      uint32_t p = k.pad[i];
      int ty = pad_type(p);
      V3<R> rl = k.getfr(pad_frame(p));
      if (ty == PAD_CELL) {
        if (!cell_inside(T, V, pad_idx(p), rl, k.u, k.token)) first_bad = i;
      } else if (ty == PAD_LATT) {
        int t[3];
        get_tile(V.lat[T.univ[pad_idx(p)].lat], rl, k.u, t);
        if (tile_pack(t) != k.tl[i]) first_bad = i;
      }
    }
  }
  if (first_bad == k.depth) return;
  if (first_bad == 0) {
    trk_restart(T, V, P, k);
    return;
  }
  uint32_t back = k.getpad(first_bad - 1);
  k.depth = first_bad - 1;
  // universe_id_to_indx[tree.back().id]: a Cell pad is looked up by the
  // cell's id (cells[].reentry precomputes what that lookup yields).
  int ui = pad_type(back) == PAD_CELL ? T.cells[pad_idx(back)].reentry : pad_idx(back);
  int f = pad_frame(back);
  k.cell = univ_get_cell(T, V, k, ui, f, k.getfr(f));
  if (k.cell < 0) trk_restart(T, V, P, k);
}

// The check half of Tracker::get_current (tracker.hpp:235-306): walks the
// tree and reports what must be re-located, without descending.  Returns
// 0 when every pad is still valid, 1 when the tree must be rebuilt from the
// root, 2 when it must be re-descended from universe `ui` in frame `fr` (the
// tree is already truncated).  The descent itself runs once per iteration of
// the transport loop for every lane that needs one (descend()).
template <class R> ABX_DEV int trk_check(const Tables& T, const View<R>& V, Trk<R>& k, int& ui, int& fr) {
  if (!(k.r.x == k.fr[0].x && k.r.y == k.fr[0].y && k.r.z == k.fr[0].z)) return 1;
  int first_bad = k.depth;
#pragma unroll 1
  for (int i = 0; i < k.depth; i++) {
    const uint32_t p = k.getpad(i);
    const int ty = pad_type(p);
    if (ty == PAD_UNIV) continue;
    const V3<R> rl = k.getfr(pad_frame(p));
    if (ty == PAD_CELL) {
      if (!cell_inside(T, V, pad_idx(p), rl, k.u, k.token)) { first_bad = i; break; }
    } else {
      int t[3];
      get_tile(V.lat[T.univ[pad_idx(p)].lat], rl, k.u, t);
      if (tile_pack(t) != k.gettile(i)) { first_bad = i; break; }
    }
  }
  if (first_bad == k.depth) return 0;
  if (first_bad == 0) return 1;
  const uint32_t back = k.getpad(first_bad - 1);
  k.depth = first_bad - 1;
  // universe_id_to_indx[tree.back().id]: a Cell pad is looked up by the
  // cell's id (cells[].reentry precomputes what that lookup yields).
  ui = pad_type(back) == PAD_CELL ? T.cells[pad_idx(back)].reentry : pad_idx(back);
  fr = pad_frame(back);
  return 2;
}

// Tracker::get_boundary_condition (tracker.hpp:94-161)
template <class R> ABX_DEV Bound<R> trk_bc(const Tables& T, const View<R>& V, const ProbT& P, const Trk<R>& k) {
  if (k.cell < 0) return univ_bc(T, V, P.root, k.r, k.u, k.token);
  Bound<R> b{Tol<R>::INF, -1, ABX_BC_VACUUM, 0};
#pragma unroll 1
  for (int i = 0; i < k.depth; i++) {
    {
      uint32_t p = k.getpad(i);
      int ty = pad_type(p), id = pad_idx(p);
      V3<R> rl = k.getfr(pad_frame(p));
      if (ty == PAD_CELL) {
        if (T.cells[id].has_bc) {
          R d; int32_t ts;
          cell_dist(T, V, id, rl, k.u, k.token, true, d, ts);
          if (d < b.dist && m_abs(d - b.dist) > Tol<R>::BTOL) {
            int32_t tmp = abs(ts);
            if (tmp) {
              b.dist = d; b.token = tmp; b.si = tmp - 1;
              b.btype = V.surf[b.si].bc;
              if (surf_sign(V.surf[b.si], rl, k.u) < 0) b.token = -b.token;
            }
          }
        }
      } else if (T.univ[id].has_bc) {
        Bound<R> ub = univ_bc(T, V, id, rl, k.u, k.token);
        if (ub.dist < b.dist && m_abs(ub.dist - b.dist) > Tol<R>::BTOL) b = ub;
      }
    }
  }
  return b;
}

// Tracker::get_nearest_boundary (tracker.hpp:163-225)
template <class R> ABX_DEV Bound<R> trk_nearest(const Tables& T, const View<R>& V, const ProbT& P, const Trk<R>& k) {
  Bound<R> b = trk_bc(T, V, P, k);
#pragma unroll 1
  for (int i = 0; i < k.depth; i++) {
    {
      uint32_t p = k.getpad(i);
      int ty = pad_type(p), id = pad_idx(p);
      V3<R> rl = k.getfr(pad_frame(p));
      if (ty == PAD_LATT) {
        int t[3];
        tile_unpack(k.gettile(i), t);
        R d = tile_dist(V.lat[T.univ[id].lat], rl, k.u, t);
        if (d < b.dist && m_abs(d - b.dist) > Tol<R>::BTOL) {
          b.dist = d; b.btype = ABX_BC_NORMAL; b.si = -1; b.token = 0;
        }
      } else if (ty == PAD_CELL) {
        R d; int32_t ts;
        cell_dist(T, V, id, rl, k.u, k.token, false, d, ts);
        if (d < b.dist && m_abs(d - b.dist) > Tol<R>::BTOL) {
          b.dist = d;
          b.token = abs(ts);
          b.si = b.token ? b.token - 1 : -1;
          b.btype = b.si >= 0 ? V.surf[b.si].bc : ABX_BC_NORMAL;
          if (b.si >= 0 && surf_sign(V.surf[b.si], rl, k.u) < 0) b.token = -b.token;
        }
      }
    }
  }
  return b;
}


// ------------------------------------------------- mixed-mode exit distances
// FP32 positions carry ~1e-6 relative error, so the reference's 1e-12
// "on the surface" bands cannot be reproduced.  The mixed mode measures, for
// each half-space of the current cell (region token t: t > 0 is the side where
// the surface function is positive), the distance along u until the particle
// leaves that half-space: infinite when moving inward or parallel, clamped to
// 0 when the point is already (within rounding) on the far side.  This needs
// no tolerance and cannot pick a wall the particle is moving away from.
//
// `on_it`: the particle sits on this surface (the tracker's surface token, set
// by the crossing or reflection that put it there).  For a quadric the side is
// then taken from the token and c = 0 exactly: FP32 rounding of c would
// otherwise put a particle that just crossed outward back inside, and the
// next flight would cross again at distance 0, back and forth.
template <class R, bool FAST32 = false>
ABX_DEV R exit_dist(const SurfT<R>& s, int32_t t, V3<R> r, V3<R> u, bool on_it) {
  const R INF = Tol<R>::INF;
  if (s.type <= ABX_SURF_PLANE) {
    R eval = surf_eval(s, r);
    R rate = s.type == ABX_SURF_XPLANE ? u.x
             : s.type == ABX_SURF_YPLANE ? u.y
             : s.type == ABX_SURF_ZPLANE ? u.z
                                         : s.c[0] * u.x + s.c[1] * u.y + s.c[2] * u.z;
    bool exiting = t > 0 ? rate < R(0) : rate > R(0);
    if (!exiting) return INF;
    R d = -eval / rate;
    return d > R(0) ? d : R(0);
  }
  R p, q, w = R(0), up, uq, uw = R(0), Rr;
  if (s.type == ABX_SURF_SPHERE) {
    p = r.x - s.c[0]; q = r.y - s.c[1]; w = r.z - s.c[2]; up = u.x; uq = u.y; uw = u.z; Rr = s.c[3];
  } else if (s.type == ABX_SURF_ZCYLINDER) {
    p = r.y - s.c[1]; q = r.x - s.c[0]; up = u.y; uq = u.x; Rr = s.c[2];
  } else if (s.type == ABX_SURF_XCYLINDER) {
    p = r.y - s.c[0]; q = r.z - s.c[1]; up = u.y; uq = u.z; Rr = s.c[2];
  } else {
    p = r.x - s.c[0]; q = r.z - s.c[1]; up = u.x; uq = u.z; Rr = s.c[2];
  }
  const R a = up * up + uq * uq + uw * uw;
  const R k = p * up + q * uq + w * uw;
  const R c = p * p + q * q + w * w - Rr * Rr;
  if (on_it) {
    if (a == R(0)) return INF;  // moving along the surface
    if (t > 0) return k >= R(0) ? INF : R(0);  // outside: leaves only by turning inward at once
    if (k > R(0)) return R(0);                 // inside but heading out
    const R d = R(-2) * k / a;                 // far root with c = 0
    return d > R(0) ? d : R(0);
  }
  if (a == R(0)) return ((t < 0) == (c > R(0))) ? R(0) : INF;
  // roots of a s^2 + 2 k s + c = 0.  With FAST32 (the nearest-boundary search
  // of surface tracking) away from grazing incidence in FP32, in the
  // cancellation-free form: with qq = -(k + sign(k) sqrt(k^2 - a c)) the roots
  // are qq / a and c / qq.  FP64 otherwise, and always when the discriminant is
  // small against k^2 (grazing incidence), where FP32 cancellation in
  // k^2 - a c dominates.  (The boundary-condition search, shared with delta
  // tracking, keeps the FP64 form: delta tracking measured faster with it.)
  if (FAST32 && sizeof(R) == 4) {
    const R quadf = k * k - a * c;
    if (quadf > R(1e-3) * k * k) {
      const R sq = m_sqrt(quadf);
      const R qq = k >= R(0) ? -(k + sq) : sq - k;
      if (qq != R(0)) {
        const R lo = qq / a, hi = c / qq;  // k >= 0: lo <= hi; k < 0: the other way round
        const R nearr = k >= R(0) ? lo : hi, farr = k >= R(0) ? hi : lo;
        if (t < 0) {  // inside: leave through the far root
          if (c > R(0) && k >= R(0)) return R(0);
          return farr > R(0) ? farr : R(0);
        }
        if (c < R(0)) return R(0);  // outside region but within the quadric
        if (k >= R(0)) return INF;
        return nearr > R(0) ? nearr : R(0);
      }
    }
  }
  double ad = a, kd = k, cd = c;
  double quad = kd * kd - ad * cd;
  if (t < 0) {  // inside: leave through the far root
    if (c > R(0) && k >= R(0)) return R(0);
    if (quad < 0.) return R(0);
    double d = (-kd + sqrt(quad)) / ad;
    return d > 0. ? (R)d : R(0);
  }
  if (c < R(0)) return R(0);  // outside region but within the quadric
  if (k >= R(0) || quad < 0.) return INF;
  double d = (-kd - sqrt(quad)) / ad;
  return d > 0. ? (R)d : R(0);
}

// Distance to leave a simple cell (intersection of half-spaces); for a cell
// with unions or complements the reference's per-surface distances are used.
template <class R, bool FAST32 = false>
ABX_DEV void cell_exit(const Tables& T, const View<R>& V, int ci, V3<R> r, V3<R> u, int32_t on, bool bc_only,
                       R& dist, int32_t& isurf) {
  const CellT c = T.cells[ci];
  if (!c.simple) {
    cell_dist(T, V, ci, r, u, on, bc_only, dist, isurf);
    return;
  }
  R mind = Tol<R>::INF;
  int32_t is = 0;
  const int32_t* __restrict__ rpn = T.rpn + c.rpn_off;
  for (int i = 0; i < c.rpn_len; i++) {
    int32_t t = __ldg(rpn + i);
    const SurfT<R> s = V.surf[abs(t) - 1];
    if (bc_only && s.bc == ABX_BC_NORMAL) continue;
    R d = exit_dist<R, FAST32>(s, t, r, u, t == on);
    if (d < mind) { mind = d; is = -t; }
  }
  dist = mind;
  isurf = is;
}

// Distance to leave the current lattice tile in the direction of motion.
template <class R> ABX_DEV R tile_exit(const LatT<R>& L, V3<R> rl, V3<R> u, const int t[3]) {
  V3<R> rt = sub(rl, tile_center(L, t[0], t[1], t[2]));
  const R h[3] = {L.p[0] * R(0.5), L.p[1] * R(0.5), L.p[2] * R(0.5)};
  const R x[3] = {rt.x, rt.y, rt.z}, v[3] = {u.x, u.y, u.z};
  R dist = Tol<R>::INF;
#pragma unroll
  for (int a = 0; a < 3; a++) {
    if (v[a] == R(0)) continue;
    R d = ((v[a] > R(0) ? h[a] : -h[a]) - x[a]) / v[a];
    d = d > R(0) ? d : R(0);
    if (d < dist) dist = d;
  }
  return dist;
}

// Mixed-mode boundary-condition search (used after a flight has left the
// geometry) and nearest-boundary search (surface tracking): the reference's
// walks over the tree, with exit distances in place of the banded ones.
template <class R>
ABX_DEV Bound<R> cells_bc_mixed(const Tables& T, const View<R>& V, int ci, V3<R> r, V3<R> u, int32_t on, Bound<R> b) {
  if (!T.cells[ci].has_bc) return b;
  R d;
  int32_t is;
  cell_exit(T, V, ci, r, u, on, true, d, is);
  if (is != 0 && d < b.dist) {
    b.dist = d;
    b.si = abs(is) - 1;
    b.token = -is;  // the cell's own side of the surface
    b.btype = V.surf[b.si].bc;
  }
  return b;
}

template <class R> ABX_DEV Bound<R> trk_bc_mixed(const Tables& T, const View<R>& V, const ProbT& P, const Trk<R>& k) {
  Bound<R> b{Tol<R>::INF, -1, ABX_BC_VACUUM, 0};
#pragma unroll 1
  for (int i = 0; i < k.depth; i++) {
    {
      uint32_t p = k.getpad(i);
      int ty = pad_type(p), id = pad_idx(p);
      V3<R> rl = k.getfr(pad_frame(p));
      if (ty == PAD_CELL) {
        b = cells_bc_mixed(T, V, id, rl, k.u, k.token, b);
      } else if (T.univ[id].has_bc) {
        int ui = id;
        for (int guard = 0; guard < 16; guard++) {
          const UnivT U = T.univ[ui];
          if (U.kind == ABX_UNIV_RECT_LATTICE) {
            if (!U.has_bc) break;
            ui = U.outer;
            continue;
          }
          if (U.bc_len >= 0) {
            // each distinct boundary half-space once, not once per cell
            for (int j = 0; j < U.bc_len; j++) {
              const int32_t t = __ldg(T.rpn + U.bc_off + j);
              const SurfT<R> s = V.surf[abs(t) - 1];
              const R d = exit_dist(s, t, rl, k.u, t == k.token);
              if (d < b.dist) {
                b.dist = d;
                b.si = abs(t) - 1;
                b.token = t;
                b.btype = s.bc;
              }
            }
          } else {
            for (int j = 0; j < U.list_len; j++)
              b = cells_bc_mixed(T, V, __ldg(T.cell_lists + U.list_off + j), rl, k.u, k.token, b);
          }
          break;
        }
      }
    }
  }
  return b;
}

template <class R> ABX_DEV Bound<R> trk_nearest_mixed(const Tables& T, const View<R>& V, const ProbT& P, const Trk<R>& k) {
  Bound<R> b = trk_bc_mixed(T, V, P, k);
#pragma unroll 1
  for (int i = 0; i < k.depth; i++) {
    {
      uint32_t p = k.getpad(i);
      int ty = pad_type(p), id = pad_idx(p);
      V3<R> rl = k.getfr(pad_frame(p));
      if (ty == PAD_LATT) {
        int t[3];
        tile_unpack(k.gettile(i), t);
        R d = tile_exit(V.lat[T.univ[id].lat], rl, k.u, t);
        // A tile wall that coincides with a boundary-condition surface (a
        // lattice filling its outer box) is that surface; FP32 rounding of the
        // two distances must not hand the tie to the tile wall.
        const bool bc_tie = b.si >= 0 && b.btype != ABX_BC_NORMAL && d > b.dist - Tol<R>::TILE;
        if (d < b.dist && !bc_tie) { b.dist = d; b.btype = ABX_BC_NORMAL; b.si = -1; b.token = 0; }
      } else if (ty == PAD_CELL) {
        R d; int32_t ts;
        cell_exit<R, true>(T, V, id, rl, k.u, k.token, false, d, ts);
        if (d < b.dist) {
          b.dist = d;
          b.token = -ts;  // the cell's own side: crossing flips it
          b.si = ts ? abs(ts) - 1 : -1;
          b.btype = b.si >= 0 ? V.surf[b.si].bc : ABX_BC_NORMAL;
        }
      }
    }
  }
  return b;
}

// rotate_direction (include/utils/direction.hpp:130-151)
// In FP32 a cosine can round just outside [-1, 1]; the square roots then take
// a clamped argument (FP64 keeps the reference's expressions unchanged).
template <class R> ABX_DEV R sqrt_1m(R x2) {
  const R a = R(1) - x2;
  return m_sqrt(sizeof(R) == 4 && a < R(0) ? R(0) : a);
}

template <class R> ABX_DEV V3<R> rotate(V3<R> u, R mu, R c, R s) {
  R sqrt_mu = sqrt_1m<R>(mu * mu);
  R sqrt_w = sqrt_1m<R>(u.z * u.z);
  R ux, uy, uz;
  if (sqrt_w > Tol<R>::ROT) {
    ux = mu * u.x + sqrt_mu * (u.x * u.z * c - u.y * s) / sqrt_w;
    uy = mu * u.y + sqrt_mu * (u.y * u.z * c + u.x * s) / sqrt_w;
    uz = mu * u.z - sqrt_mu * sqrt_w * c;
  } else {
    R sqrt_v = sqrt_1m<R>(u.y * u.y);
    ux = mu * u.x + sqrt_mu * (u.x * u.y * c + u.z * s) / sqrt_v;
    uy = mu * u.y - sqrt_mu * sqrt_v * c;
    uz = mu * u.z + sqrt_mu * (u.y * u.z * c - u.x * s) / sqrt_v;
  }
  return dir3(ux, uy, uz);
}

// Azimuth: the reference forms phi = 2*PI*u and calls cos/sin; the mixed
// mode evaluates cos(2*pi*u), sin(2*pi*u) with sincospif.
ABX_DEV void azimuth(double u, double& c, double& s) {
  const double PI = 3.14159265358979323846264338327950288;
  double phi = 2. * PI * u;
  c = cos(phi);
  s = sin(phi);
}
ABX_DEV void azimuth(float u, float& c, float& s) { sincospif(2.f * u, &s, &c); }

}  // namespace abx
