// Reference-format decks read natively: the multigroup YAML deck of the
// reference (src/parser.cpp:77-1054) flattened into an abx_problem, so a
// caller holding the deck text -- the reference's own transporter adapter,
// for one -- can build a context without any host-side problem code.
//
// The reader takes the YAML subset the reference's decks use (block maps
// and sequences, flow lists and maps that may span lines, plain and quoted
// scalars, comments).  The flattening follows the reference parser's
// conventions: surface tokens are +-(surface index + 1) and regions go
// through its infix->RPN conversion (src/cell.cpp:250-360); universes are
// indexed in the order the parser creates them (src/parser.cpp:177-257,
// src/rect_lattice.cpp:364-424); a one-row chi is repeated for every incoming
// group (src/mg_nuclide.cpp:834-854); `fissile-only` is read on the source
// entry (src/source.cpp:104-110); `sampling-xs-ratio` is a top-level list
// (src/parser.cpp:425-434).  It gives the same problem, bit for bit, as the
// package's Python deck reader (abeille_gb300/deck.py + decks.py +
// problem.py), which the tests check.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <set>
#include <stdexcept>
#include <string>
#include <vector>

#include "abeille_gb300.h"

namespace abx {
void set_error_string(const char* msg);
}

namespace {

struct DeckError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

[[noreturn]] void bad(const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  throw DeckError(buf);
}

// ---------------------------------------------------------------- values
struct Val {
  enum Kind { NONE, SCALAR, SEQ, MAP } kind = NONE;
  std::string s;  // scalar text (quotes removed)
  bool quoted = false;
  std::vector<Val> seq;
  std::vector<std::pair<std::string, Val>> map;

  const Val* get(const std::string& k) const {
    if (kind != MAP) return nullptr;
    for (const auto& kv : map)
      if (kv.first == k) return &kv.second;
    return nullptr;
  }
  const Val& at(const std::string& k) const {
    const Val* v = get(k);
    if (!v) bad("deck entry '%s' missing", k.c_str());
    return *v;
  }
  bool is_null() const { return kind == NONE || (kind == SCALAR && !quoted && (s == "null" || s == "~" || s.empty())); }
  double num() const {
    if (kind != SCALAR) bad("expected a number");
    std::string t = s;
    if (t == ".inf" || t == "+.inf" || t == ".Inf") return INFINITY;
    if (t == "-.inf" || t == "-.Inf") return -INFINITY;
    char* end = nullptr;
    double d = strtod(t.c_str(), &end);
    if (end == t.c_str() || *end) bad("'%s' is not a number", t.c_str());
    return d;
  }
  long long integer() const {
    double d = num();
    if (d != std::floor(d)) bad("'%s' is not an integer", s.c_str());
    return (long long)d;
  }
  bool boolean() const {
    if (kind == SCALAR && (s == "true" || s == "True")) return true;
    if (kind == SCALAR && (s == "false" || s == "False")) return false;
    bad("'%s' is not a boolean", s.c_str());
  }
  std::string str() const {
    if (kind != SCALAR) bad("expected a scalar");
    return s;
  }
  std::vector<double> nums() const {
    if (kind != SEQ) bad("expected a list of numbers");
    std::vector<double> o;
    for (const Val& v : seq) o.push_back(v.num());
    return o;
  }
};

Val scalar(std::string t) {
  // strip, unquote
  size_t a = t.find_first_not_of(" \t"), b = t.find_last_not_of(" \t");
  t = a == std::string::npos ? "" : t.substr(a, b - a + 1);
  Val v;
  v.kind = Val::SCALAR;
  if (t.size() >= 2 && t.front() == t.back() && (t[0] == '"' || t[0] == '\'')) {
    v.s = t.substr(1, t.size() - 2);
    v.quoted = true;
  } else {
    v.s = t;
  }
  return v;
}

std::string strip_comment(const std::string& line) {
  std::string out;
  char quote = 0;
  for (size_t i = 0; i < line.size(); i++) {
    char ch = line[i];
    if (quote) {
      if (ch == quote) quote = 0;
    } else if (ch == '"' || ch == '\'') {
      quote = ch;
    } else if (ch == '#' && (i == 0 || line[i - 1] == ' ' || line[i - 1] == '\t')) {
      break;
    }
    out += ch;
  }
  size_t e = out.find_last_not_of(" \t\r");
  return e == std::string::npos ? "" : out.substr(0, e + 1);
}

int depth(const std::string& t) {
  int d = 0;
  char quote = 0;
  for (char ch : t) {
    if (quote) {
      if (ch == quote) quote = 0;
    } else if (ch == '"' || ch == '\'') {
      quote = ch;
    } else if (ch == '[' || ch == '{') {
      d++;
    } else if (ch == ']' || ch == '}') {
      d--;
    }
  }
  return d;
}

struct Line {
  int indent;
  std::string text;
};

std::vector<Line> logical_lines(const std::string& text) {
  std::vector<Line> out;
  std::string pending;
  bool have_pending = false;
  int indent = 0;
  size_t p = 0;
  while (p <= text.size()) {
    size_t q = text.find('\n', p);
    if (q == std::string::npos) q = text.size();
    std::string raw = text.substr(p, q - p);
    p = q + 1;
    std::string tabbed;
    for (char ch : raw) {
      if (ch == '\t') tabbed += "    ";
      else tabbed += ch;
    }
    std::string line = strip_comment(tabbed);
    size_t first = line.find_first_not_of(' ');
    if (first == std::string::npos) {
      if (q == text.size()) break;
      continue;
    }
    std::string content = line.substr(first);
    if (have_pending) {
      pending += " " + content;
      if (depth(pending) <= 0) {
        out.push_back({indent, pending});
        have_pending = false;
      }
    } else {
      indent = (int)first;
      if (depth(content) > 0) {
        pending = content;
        have_pending = true;
      } else {
        out.push_back({indent, content});
      }
    }
    if (q == text.size()) break;
  }
  if (have_pending) bad("unterminated flow collection in deck");
  return out;
}

Val flow(const std::string& t, size_t& i) {
  const size_t n = t.size();
  while (i < n && t[i] == ' ') i++;
  if (i < n && t[i] == '[') {
    i++;
    Val v;
    v.kind = Val::SEQ;
    for (;;) {
      while (i < n && (t[i] == ' ' || t[i] == ',')) i++;
      if (i >= n) bad("unterminated flow list");
      if (t[i] == ']') {
        i++;
        return v;
      }
      v.seq.push_back(flow(t, i));
    }
  }
  if (i < n && t[i] == '{') {
    i++;
    Val v;
    v.kind = Val::MAP;
    for (;;) {
      while (i < n && (t[i] == ' ' || t[i] == ',')) i++;
      if (i >= n) bad("unterminated flow map");
      if (t[i] == '}') {
        i++;
        return v;
      }
      size_t j = i;
      while (j < n && t[j] != ':') j++;
      std::string key = scalar(t.substr(i, j - i)).s;
      i = j + 1;
      v.map.emplace_back(key, flow(t, i));
    }
  }
  size_t j = i;
  char quote = 0;
  while (j < n) {
    char ch = t[j];
    if (quote) {
      if (ch == quote) quote = 0;
    } else if (ch == '"' || ch == '\'') {
      quote = ch;
    } else if (ch == ',' || ch == ']' || ch == '}') {
      break;
    }
    j++;
  }
  Val v = scalar(t.substr(i, j - i));
  i = j;
  return v;
}

Val value(const std::string& text) {
  size_t a = text.find_first_not_of(' ');
  std::string t = a == std::string::npos ? "" : text.substr(a);
  if (!t.empty() && (t[0] == '[' || t[0] == '{')) {
    size_t i = 0;
    return flow(t, i);
  }
  return scalar(t);
}

bool split_key(const std::string& c, std::string& key, std::string& rest) {
  char quote = 0;
  for (size_t i = 0; i < c.size(); i++) {
    char ch = c[i];
    if (quote) {
      if (ch == quote) quote = 0;
    } else if (ch == '"' || ch == '\'') {
      quote = ch;
    } else if (ch == ':' && (i + 1 == c.size() || c[i + 1] == ' ')) {
      key = scalar(c.substr(0, i)).s;
      std::string r = c.substr(i + 1);
      size_t a = r.find_first_not_of(' ');
      rest = a == std::string::npos ? "" : r.substr(a);
      return true;
    }
  }
  return false;
}

bool is_item(const std::string& t) { return t == "-" || t.rfind("- ", 0) == 0; }

Val block(const std::vector<Line>& L, size_t& i, int indent) {
  if (is_item(L[i].text)) {
    Val out;
    out.kind = Val::SEQ;
    while (i < L.size() && L[i].indent == indent && is_item(L[i].text)) {
      std::string rest = L[i].text == "-" ? "" : L[i].text.substr(2);
      size_t a = rest.find_first_not_of(' ');
      rest = a == std::string::npos ? "" : rest.substr(a);
      if (rest.empty()) {
        i++;
        if (i < L.size() && L[i].indent > indent) out.seq.push_back(block(L, i, L[i].indent));
        else out.seq.push_back(Val());
        continue;
      }
      std::string k, r;
      if (rest[0] == '[' || rest[0] == '{' || !split_key(rest, k, r)) {
        out.seq.push_back(value(rest));
        i++;
        continue;
      }
      // an inline mapping: its further keys sit at the column of the first
      const int item_indent = indent + (int)(L[i].text.size() - rest.size());
      std::vector<Line> sub{{item_indent, rest}};
      size_t j = i + 1;
      while (j < L.size() && L[j].indent > indent) sub.push_back(L[j++]);
      size_t s0 = 0;
      out.seq.push_back(block(sub, s0, item_indent));
      i = j;
    }
    return out;
  }
  Val out;
  out.kind = Val::MAP;
  while (i < L.size() && L[i].indent == indent) {
    std::string key, rest;
    if (!split_key(L[i].text, key, rest)) bad("expected 'key: value', got '%s'", L[i].text.c_str());
    i++;
    if (!rest.empty()) {
      out.map.emplace_back(key, value(rest));
    } else if (i < L.size() && L[i].indent > indent) {
      out.map.emplace_back(key, block(L, i, L[i].indent));
    } else if (i < L.size() && L[i].indent == indent && is_item(L[i].text)) {
      out.map.emplace_back(key, block(L, i, indent));  // a sequence may sit at its key's column
    } else {
      out.map.emplace_back(key, Val());
    }
  }
  return out;
}

Val parse(const std::string& text) {
  std::vector<Line> L = logical_lines(text);
  if (L.empty()) return Val();
  size_t i = 0;
  Val v = block(L, i, L[0].indent);
  if (i != L.size()) bad("unparsed deck content from '%s'", L[i].text.c_str());
  return v;
}

// ------------------------------------------------------------ flattening
// region operators as tokens (the reference's values, include/geometry/cell.hpp:42-48)
constexpr int32_t OP_LPAR = ABX_OP_LPAR, OP_RPAR = ABX_OP_RPAR, OP_COMP = ABX_OP_COMP, OP_INTR = ABX_OP_INTR,
                  OP_UNIN = ABX_OP_UNIN;

}  // namespace

// The flattened problem and the storage its pointers point into.
struct abx_deck {
  abx_problem p{};
  std::vector<double> eb, mg, teb, smp;
  std::vector<abx_surface> surf;
  std::vector<abx_cell> cells;
  std::vector<int32_t> rpn, lists, lat;
  std::vector<abx_universe> univ;
  std::vector<abx_material> mats;
  std::vector<abx_mesh_tally> tallies;
  std::vector<abx_source> src;
};

namespace {

int op_token(char ch) {
  switch (ch) {
    case '&': return OP_INTR;
    case '(': return OP_LPAR;
    case ')': return OP_RPAR;
    case 'U': return OP_UNIN;
    default: return OP_COMP;  // '~'
  }
}

// Cell region string -> infix tokens (src/cell.cpp:309-360)
std::vector<int32_t> tokenize(const std::string& region, const std::map<long long, int>& surf_index) {
  std::vector<int32_t> out;
  std::string temp;
  auto flush = [&] {
    if (temp.empty()) return;
    long long sid = std::strtoll(temp.c_str(), nullptr, 10);
    auto it = surf_index.find(sid < 0 ? -sid : sid);
    if (it == surf_index.end()) bad("region references unknown surface id %lld", sid < 0 ? -sid : sid);
    int tok = it->second + 1;
    out.push_back(sid < 0 ? -tok : tok);
    temp.clear();
  };
  for (char ch : region) {
    if (ch == '&' || ch == '(' || ch == ')' || ch == 'U' || ch == '~') {
      flush();
      out.push_back(op_token(ch));
    } else if (ch == '+' || ch == '-' || (ch >= '0' && ch <= '9')) {
      temp += ch;
    } else if (ch != ' ') {
      bad("invalid character '%c' in region", ch);
    }
  }
  flush();
  return out;
}

// Shunting yard with the reference's precedences (src/cell.cpp:250-299)
std::vector<int32_t> to_rpn(const std::vector<int32_t>& infix) {
  std::vector<int32_t> rpn, stack;
  for (int32_t t : infix) {
    if (t < OP_UNIN) {
      rpn.push_back(t);
    } else if (t < OP_RPAR) {
      while (!stack.empty()) {
        int32_t op = stack.back();
        if (op < OP_RPAR && ((t == OP_COMP && t < op) || (t != OP_COMP && t <= op))) {
          rpn.push_back(op);
          stack.pop_back();
        } else {
          break;
        }
      }
      stack.push_back(t);
    } else if (t == OP_LPAR) {
      stack.push_back(t);
    } else {
      while (!stack.empty() && stack.back() != OP_LPAR) {
        rpn.push_back(stack.back());
        stack.pop_back();
      }
      if (stack.empty()) bad("mismatched parentheses in region");
      stack.pop_back();
    }
  }
  while (!stack.empty()) {
    int32_t op = stack.back();
    stack.pop_back();
    if (op >= OP_RPAR) bad("mismatched parentheses in region");
    rpn.push_back(op);
  }
  return rpn;
}

std::vector<double> flat(const Val& v, size_t n, const char* what, long long id) {
  std::vector<double> o;
  std::vector<const Val*> st{&v};
  while (!st.empty()) {  // depth-first, in order
    const Val* x = st.back();
    st.pop_back();
    if (x->kind == Val::SEQ) {
      for (size_t k = x->seq.size(); k-- > 0;) st.push_back(&x->seq[k]);
    } else {
      o.push_back(x->num());
    }
  }
  if (n && o.size() != n) bad("material %lld: %s has %zu entries, expected %zu", id, what, o.size(), n);
  return o;
}

void build(const Val& d, int precision, abx_deck& D) {
  if (d.kind != Val::MAP) bad("deck is not a map");
  const Val& st = d.at("settings");
  const Val* em = st.get("energy-mode");
  if (em && em->str() != "multi-group") bad("only multigroup decks run on this engine");
  const int G = (int)st.at("ngroups").integer();
  if (G < 1) bad("ngroups must be positive");
  D.eb = st.at("energy-bounds").nums();
  if ((int)D.eb.size() != G + 1) bad("energy-bounds must have ngroups+1 entries");
  abx_settings& S = D.p.settings;
  const std::string sim = st.at("simulation").str();
  if (sim == "k-eigenvalue" || sim == "branchless-k-eigenvalue") S.mode = ABX_MODE_K_EIGENVALUE;
  else if (sim == "fixed-source") S.mode = ABX_MODE_FIXED_SOURCE;
  else bad("simulation '%s' is outside the multigroup transport path", sim.c_str());
  const Val* tr = st.get("transport");
  const std::string trk = tr ? tr->str() : "surface-tracking";
  if (trk == "delta-tracking") S.tracking = ABX_TRACK_DELTA;
  else if (trk == "surface-tracking") S.tracking = ABX_TRACK_SURFACE;
  else if (trk == "implicit-leakage-delta-tracking") S.tracking = ABX_TRACK_IMPLICIT_LEAKAGE;
  else if (trk == "carter-tracking") S.tracking = ABX_TRACK_CARTER;
  else bad("transport '%s' unknown", trk.c_str());
  S.precision = precision;
  S.ngroups = G;
  auto opt_num = [&](const char* k, double dflt) { const Val* v = st.get(k); return v ? v->num() : dflt; };
  auto opt_bool = [&](const char* k, bool dflt) { const Val* v = st.get(k); return v ? v->boolean() : dflt; };
  S.nparticles = (double)st.at("nparticles").integer();
  S.seed = st.get("seed") ? (uint64_t)std::strtoull(st.at("seed").str().c_str(), nullptr, 10) : 19073486328125ull;
  S.stride = st.get("stride") ? (uint64_t)std::strtoull(st.at("stride").str().c_str(), nullptr, 10) : 152917ull;
  S.wgt_cutoff = opt_num("wgt-cutoff", 0.25);
  S.wgt_survival = opt_num("wgt-survival", 1.0);
  S.wgt_split = opt_num("wgt-split", 2.0);
  const Val* canc = st.get("cancellation");
  if (canc && canc->boolean()) bad("regional cancellation is outside the multigroup transport path");

  const Val& mats = d.at("materials");
  const Val& cells = d.at("cells");
  if (sim == "branchless-k-eigenvalue") {
    S.branchless = ABX_BRANCHLESS_ON | (opt_bool("branchless-material", true) ? ABX_BRANCHLESS_MATERIAL : 0) |
                   (opt_bool("branchless-splitting", false) ? ABX_BRANCHLESS_SPLITTING : 0) |
                   (opt_bool("branchless-combing", true) ? ABX_BRANCHLESS_COMBING : 0);
    // the global stream draws a plot colour for every cell and every material
    // without one while the deck is read (src/cell.cpp:445-448, src/material.cpp:440-449)
    int uncoloured = 0;
    for (const Val& m : mats.seq) {
      const Val* c = m.get("color");
      if (!(c && c->kind == Val::SEQ && c->seq.size() == 3)) uncoloured++;
    }
    S.global_rng_skip = 6 * ((int)cells.seq.size() + uncoloured);
  }
  if (const Val* smp = d.get("sampling-xs-ratio")) {
    D.smp = smp->nums();
    if ((int)D.smp.size() != G) bad("sampling-xs-ratio needs one entry per group");
  }

  // materials (src/mg_nuclide.cpp:579-922)
  std::map<long long, int> mat_index;
  for (const Val& m : mats.seq) {
    const long long id = m.at("id").integer();
    std::vector<double> tot = flat(m.at("total"), G, "total", id), ab = flat(m.at("absorption"), G, "absorption", id);
    std::vector<double> sc = flat(m.at("scatter"), (size_t)G * G, "scatter", id);
    std::vector<double> fi(G, 0.), nup(G, 0.), nud(G, 0.), ch((size_t)G * G, 0.);
    if (const Val* f = m.get("fission")) if (!f->is_null()) fi = flat(*f, G, "fission", id);
    bool fissile = false;
    for (double x : fi) fissile |= x > 0;
    if (fissile) {
      const Val* nu = m.get("nu");
      if (!nu || nu->is_null()) bad("material %lld: fissile material needs nu", id);
      nup = flat(*nu, G, "nu", id);
      const Val* chi = m.get("chi");
      if (!chi || chi->is_null()) bad("material %lld: fissile material needs chi", id);
      std::vector<double> c = flat(*chi, 0, "chi", id);
      if ((int)c.size() == G) {
        for (int g = 0; g < G; g++) std::copy(c.begin(), c.end(), ch.begin() + (size_t)g * G);
      } else if (c.size() == (size_t)G * G) {
        ch = c;
      } else {
        bad("material %lld: chi has %zu entries", id, c.size());
      }
    }
    int L = 0;
    for (int l = 1; l <= 5; l++)
      if (m.get("P" + std::to_string(l))) L = l;
    std::vector<double> mom((size_t)L * G * G, 0.);
    for (int l = 1; l <= L; l++) {
      const Val* pl = m.get("P" + std::to_string(l));
      if (!pl) continue;
      std::vector<double> v = flat(*pl, (size_t)G * G, "Legendre moment", id);
      std::copy(v.begin(), v.end(), mom.begin() + (size_t)(l - 1) * G * G);
    }
    abx_material am{};
    am.id = (uint32_t)id;
    am.data_offset = (int32_t)D.mg.size();
    am.n_legendre = L;
    am.n_delayed = 0;
    for (auto* v : {&tot, &ab, &fi, &nup, &nud, &ch, &sc, &mom}) D.mg.insert(D.mg.end(), v->begin(), v->end());
    mat_index[id] = (int)D.mats.size();
    D.mats.push_back(am);
  }

  // surfaces
  std::map<long long, int> surf_index;
  static const std::map<std::string, std::pair<int, std::vector<const char*>>> kinds = {
      {"xplane", {ABX_SURF_XPLANE, {"x0"}}},
      {"yplane", {ABX_SURF_YPLANE, {"y0"}}},
      {"zplane", {ABX_SURF_ZPLANE, {"z0"}}},
      {"plane", {ABX_SURF_PLANE, {"A", "B", "C", "D"}}},
      {"xcylinder", {ABX_SURF_XCYLINDER, {"y0", "z0", "r"}}},
      {"ycylinder", {ABX_SURF_YCYLINDER, {"x0", "z0", "r"}}},
      {"zcylinder", {ABX_SURF_ZCYLINDER, {"x0", "y0", "r"}}},
      {"sphere", {ABX_SURF_SPHERE, {"x0", "y0", "z0", "r"}}}};
  for (const Val& s : d.at("surfaces").seq) {
    auto k = kinds.find(s.at("type").str());
    if (k == kinds.end()) bad("surface type '%s' is outside the multigroup path", s.at("type").str().c_str());
    abx_surface as{};
    as.type = k->second.first;
    const long long id = s.at("id").integer();
    if (surf_index.count(id)) bad("surface id %lld used twice", id);
    as.id = (uint32_t)id;
    const Val* b = s.get("boundary");
    const std::string bc = b ? b->str() : "normal";
    as.bc = bc == "vacuum" ? ABX_BC_VACUUM : bc == "reflective" ? ABX_BC_REFLECTIVE : ABX_BC_NORMAL;
    int c = 0;
    for (const char* key : k->second.second) {
      const Val* v = s.get(key);
      as.c[c++] = v ? v->num() : 0.;
    }
    surf_index[id] = (int)D.surf.size();
    D.surf.push_back(as);
  }

  // universes in the reference parser's order
  struct U {
    bool lattice;
    std::vector<long long> cells;
    std::vector<long long> tiles;
    int shape[3];
    double pitch[3], origin[3];
    long long outer;
  };
  std::map<long long, U> unis;
  std::vector<long long> decl;
  for (const Val& u : d.at("universes").seq) {
    U x{};
    const long long id = u.at("id").integer();
    if (const Val* cl = u.get("cells")) {
      x.lattice = false;
      for (const Val& c : cl->seq) x.cells.push_back(c.integer());
    } else {
      x.lattice = true;
      std::vector<double> sh = u.at("shape").nums(), pi = u.at("pitch").nums(), og = u.at("origin").nums();
      if (sh.size() != 3 || pi.size() != 3 || og.size() != 3) bad("lattice %lld: shape, pitch and origin need 3 entries", id);
      for (int a = 0; a < 3; a++) {
        x.shape[a] = (int)sh[a];
        x.pitch[a] = pi[a];
        x.origin[a] = og[a];
      }
      std::vector<double> t = flat(u.at("universes"), 0, "lattice universes", id);
      for (double v : t) x.tiles.push_back((long long)v);
      if ((long long)x.tiles.size() != (long long)x.shape[0] * x.shape[1] * x.shape[2])
        bad("lattice %lld: universes do not match its shape", id);
      const Val* o = u.get("outer");
      x.outer = o && !o->is_null() ? o->integer() : -1;
    }
    unis[id] = x;
    decl.push_back(id);
  }
  std::map<long long, const Val*> cell_by_id;
  for (const Val& c : cells.seq) cell_by_id[c.at("id").integer()] = &c;
  std::vector<long long> order;
  std::set<long long> made;
  std::function<void(long long)> make = [&](long long uid) {
    if (made.count(uid)) return;
    auto it = unis.find(uid);
    if (it == unis.end()) bad("unknown universe id %lld", uid);
    const U& u = it->second;
    if (u.lattice) {
      for (long long t : u.tiles)
        if (t != -1) make(t);
      if (u.outer != -1) make(u.outer);
    } else {
      for (long long cid : u.cells)
        if (!cell_by_id.count(cid)) bad("universe %lld references unknown cell %lld", uid, cid);
    }
    made.insert(uid);
    order.push_back(uid);
  };
  for (const Val& c : cells.seq)
    if (const Val* u = c.get("universe")) if (!u->is_null()) make(u->integer());
  for (long long uid : decl) make(uid);
  std::map<long long, int> uni_index, cell_index;
  for (size_t i = 0; i < order.size(); i++) uni_index[order[i]] = (int)i;
  for (size_t i = 0; i < cells.seq.size(); i++) cell_index[cells.seq[i].at("id").integer()] = (int)i;

  for (const Val& c : cells.seq) {
    abx_cell ac{};
    ac.id = (uint32_t)c.at("id").integer();
    std::vector<int32_t> r = to_rpn(tokenize(c.at("region").str(), surf_index));
    ac.rpn_offset = (int32_t)D.rpn.size();
    ac.rpn_len = (int32_t)r.size();
    D.rpn.insert(D.rpn.end(), r.begin(), r.end());
    const Val* m = c.get("material");
    const Val* u = c.get("universe");
    const bool has_m = m && !m->is_null(), has_u = u && !u->is_null();
    if (has_m == has_u) bad("cell %u has exactly one of material/universe", ac.id);
    if (has_m) {
      auto it = mat_index.find(m->integer());
      if (it == mat_index.end()) bad("cell %u: unknown material %lld", ac.id, m->integer());
      ac.fill_kind = ABX_FILL_MATERIAL;
      ac.fill = it->second;
    } else {
      ac.fill_kind = ABX_FILL_UNIVERSE;
      ac.fill = uni_index.at(u->integer());
    }
    D.cells.push_back(ac);
  }
  for (long long uid : order) {
    const U& u = unis.at(uid);
    abx_universe au{};
    au.id = (uint32_t)uid;
    if (!u.lattice) {
      au.kind = ABX_UNIV_CELLS;
      au.list_offset = (int32_t)D.lists.size();
      au.list_len = (int32_t)u.cells.size();
      for (long long cid : u.cells) D.lists.push_back(cell_index.at(cid));
      au.outer = -1;
    } else {
      au.kind = ABX_UNIV_RECT_LATTICE;
      au.list_offset = (int32_t)D.lat.size();
      au.list_len = (int32_t)u.tiles.size();
      for (long long t : u.tiles) D.lat.push_back(t == -1 ? -1 : uni_index.at(t));
      au.outer = u.outer == -1 ? -1 : uni_index.at(u.outer);
      for (int a = 0; a < 3; a++) {
        au.shape[a] = u.shape[a];
        au.pitch[a] = u.pitch[a];
        au.origin[a] = u.origin[a];
      }
    }
    D.univ.push_back(au);
  }
  const long long root = d.at("root-universe").integer();
  if (!uni_index.count(root)) bad("unknown root universe %lld", root);

  // tallies, entropy, sources
  if (const Val* ts = d.get("tallies")) {
    for (const Val& t : ts->seq) {
      abx_mesh_tally at{};
      const Val* e = t.get("estimator");
      const std::string est = e ? e->str() : "collision";
      if (est == "collision") at.estimator = ABX_EST_COLLISION;
      else if (est == "track-length") at.estimator = ABX_EST_TRACK_LENGTH;
      else bad("tally estimator '%s' is outside the multigroup path", est.c_str());
      const Val* q = t.get("quantity");
      const std::string qs = q ? q->str() : "flux";
      static const std::map<std::string, int> qn = {{"flux", ABX_Q_FLUX}, {"elastic", ABX_Q_ELASTIC},
                                                    {"absorption", ABX_Q_ABSORPTION}, {"fission", ABX_Q_FISSION},
                                                    {"total", ABX_Q_TOTAL}};
      auto qi = qn.find(qs);
      if (qi == qn.end()) bad("tally quantity '%s' is outside the multigroup path", qs.c_str());
      at.quantity = qi->second;
      std::vector<double> sh = t.at("shape").nums(), lo = t.at("low").nums(), hi = t.at("hi").nums();
      for (int a = 0; a < 3; a++) {
        at.shape[a] = (int32_t)sh.at(a);
        at.low[a] = lo.at(a);
        at.hi[a] = hi.at(a);
      }
      const Val* eb = t.get("energy-bounds");
      std::vector<double> e2 = eb && !eb->is_null() ? eb->nums() : D.eb;
      at.ebounds_offset = (int32_t)D.teb.size();
      at.n_ebounds = (int32_t)e2.size();
      D.teb.insert(D.teb.end(), e2.begin(), e2.end());
      D.tallies.push_back(at);
    }
  }
  if (const Val* e = d.get("entropy")) {
    if (e->kind == Val::MAP) {
      abx_entropy_mesh& E = D.p.entropy;
      E.enabled = 1;
      std::vector<double> sh = e->at("shape").nums(), lo = e->at("low").nums(), hi = e->at("hi").nums();
      for (int a = 0; a < 3; a++) {
        E.shape[a] = (int32_t)sh.at(a);
        E.low[a] = lo.at(a);
        E.hi[a] = hi.at(a);
      }
    }
  }
  if (const Val* ss = d.get("sources")) {
    for (const Val& s : ss->seq) {
      abx_source so{};
      const Val& sp = s.at("spatial");
      const std::string kind = sp.at("type").str();
      const Val& en = s.at("energy");
      if (en.at("type").str() != "mono-energetic") bad("only mono-energetic sources are in the multigroup path");
      const Val& dr = s.at("direction");
      so.energy = ABX_ENERGY_MONO;
      so.energy_value = en.at("energy").num();
      so.weight = s.at("weight").num();
      if (const Val* f = s.get("fissile-only")) so.fissile_only = f->boolean() ? 1 : 0;
      std::vector<double> lo, hi;
      if (kind == "point") {
        so.spatial = ABX_SPATIAL_POINT;
        lo = sp.at("position").nums();
        hi = lo;
      } else if (kind == "box") {
        so.spatial = ABX_SPATIAL_BOX;
        lo = sp.at("low").nums();
        hi = sp.at("hi").nums();
      } else {
        bad("spatial distribution '%s' is outside the multigroup path", kind.c_str());
      }
      const std::string dt = dr.at("type").str();
      so.direction = dt == "isotropic" ? ABX_DIR_ISOTROPIC : ABX_DIR_MONO;
      std::vector<double> dv = so.direction == ABX_DIR_MONO ? dr.at("direction").nums() : std::vector<double>{1., 0., 0.};
      for (int a = 0; a < 3; a++) {
        so.low[a] = lo.at(a);
        so.hi[a] = hi.at(a);
        so.dir[a] = dv.at(a);
      }
      D.src.push_back(so);
    }
  }

  // pointers
  abx_problem& p = D.p;
  p.energy_bounds = D.eb.data();
  p.surfaces = D.surf.data();
  p.n_surfaces = (int32_t)D.surf.size();
  p.cells = D.cells.data();
  p.n_cells = (int32_t)D.cells.size();
  p.rpn = D.rpn.data();
  p.n_rpn = (int32_t)D.rpn.size();
  p.universes = D.univ.data();
  p.n_universes = (int32_t)D.univ.size();
  p.cell_lists = D.lists.data();
  p.n_cell_lists = (int32_t)D.lists.size();
  p.lattice_elems = D.lat.data();
  p.n_lattice_elems = (int32_t)D.lat.size();
  p.root_universe = uni_index.at(root);
  p.materials = D.mats.data();
  p.n_materials = (int32_t)D.mats.size();
  p.mg_data = D.mg.data();
  p.n_mg_data = (int64_t)D.mg.size();
  p.tallies = D.tallies.data();
  p.n_tallies = (int32_t)D.tallies.size();
  p.tally_ebounds = D.teb.data();
  p.n_tally_ebounds = (int32_t)D.teb.size();
  p.sources = D.src.data();
  p.n_sources = (int32_t)D.src.size();
  p.sampling_xs_ratio = D.smp.empty() ? nullptr : D.smp.data();
}

}  // namespace

extern "C" int abx_deck_read(const char* text, int precision, abx_deck** out, const abx_problem** problem) {
  if (!text || !out) {
    abx::set_error_string("bad arguments");
    return ABX_ERR_INVALID;
  }
  *out = nullptr;
  if (precision != ABX_PREC_FP64 && precision != ABX_PREC_MIXED) {
    abx::set_error_string("precision must be ABX_PREC_FP64 or ABX_PREC_MIXED");
    return ABX_ERR_INVALID;
  }
  std::unique_ptr<abx_deck> d(new abx_deck());
  try {
    build(parse(text), precision, *d);
  } catch (const std::exception& e) {
    abx::set_error_string(e.what());
    return ABX_ERR_INVALID;
  }
  if (problem) *problem = &d->p;
  *out = d.release();
  return ABX_OK;
}

extern "C" int abx_deck_free(abx_deck* d) {
  delete d;
  return ABX_OK;
}

extern "C" int abx_create_from_deck(const char* text, int precision, int device, abx_ctx** out) {
  abx_deck* d = nullptr;
  const abx_problem* p = nullptr;
  int rc = abx_deck_read(text, precision, &d, &p);
  if (rc != ABX_OK) return rc;
  rc = abx_create(p, device, out);
  abx_deck_free(d);
  return rc;
}
