"""Generate golden vectors for the random-number layer of the transport path.

Abeille draws every random number through pcg-cpp's ``pcg32`` and libstdc++'s
``<random>`` distributions (include/utils/rng.hpp:41-96,
include/simulation/particle.hpp:188-193, src/simulation.cpp:63-67).  Neither
library's source lives in the reference tree, so this script compiles a small
C++ program against the real ones -- the pcg-cpp copy vendored inside pyarrow
and the system libstdc++ -- and records what they produce:

  * pcg32 internal state after seeding, and after ``advance(stride * id)``;
  * raw 32-bit outputs;
  * ``std::uniform_real_distribution<double>(0,1)`` (== RNG::rand);
  * ``std::exponential_distribution<double>``;
  * ``std::discrete_distribution<int>`` on several weight vectors, followed by
    one more canonical draw to show how many outputs each sample consumed;
  * the state of a default-constructed ``pcg32`` (settings::rng) and
    ``std::shuffle`` of 1 .. 70001 elements (checksum, first elements and the
    next output), as the branchless power iteration's combing uses them.

Run it where pyarrow and g++ are installed; it rewrites rng_golden.json next
to this file.  The tests read only the JSON.
"""
import json
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))

CPP = r"""
#include <cstdio>
#include <cstdint>
#include <random>
#include <sstream>
#include <vector>
#include <algorithm>
#include "pcg_random.hpp"
using pcg32 = arrow_vendored::pcg32;

static uint64_t state_of(const pcg32& r) {
  std::ostringstream os; os << r;  // "multiplier increment state"
  std::istringstream is(os.str());
  unsigned long long m, i, s; is >> m >> i >> s; return (uint64_t)s;
}
static void vec(const char* key, const std::vector<double>& v, bool last=false) {
  std::printf("\"%s\": [", key);
  for (size_t i = 0; i < v.size(); i++) std::printf("%s\"%a\"", i ? ", " : "", v[i]);
  std::printf("]%s\n", last ? "" : ",");
}
int main() {
  std::printf("{\n");
  // seeding + raw outputs
  const uint64_t seeds[] = {19073486328125ULL, 0ULL, 1ULL, 12345678901234567ULL};
  std::printf("\"seed\": [\n");
  for (int k = 0; k < 4; k++) {
    pcg32 r(seeds[k]);
    std::printf("%s{\"seed\": %llu, \"state\": %llu, \"out\": [", k ? "," : "",
                (unsigned long long)seeds[k], (unsigned long long)state_of(r));
    for (int i = 0; i < 8; i++) std::printf("%s%u", i ? ", " : "", (unsigned)r());
    std::printf("]}\n");
  }
  std::printf("],\n");
  // skip-ahead as Particle::initialize_rng does
  const uint64_t ids[] = {0ULL, 1ULL, 2ULL, 999ULL, 1000000ULL, 123456789012ULL};
  std::printf("\"advance\": [\n");
  for (int k = 0; k < 6; k++) {
    pcg32 r; r.seed(19073486328125ULL);
    r.advance(152917ULL * ids[k]);
    std::printf("%s{\"id\": %llu, \"state\": %llu, \"out\": [", k ? "," : "",
                (unsigned long long)ids[k], (unsigned long long)state_of(r));
    for (int i = 0; i < 4; i++) std::printf("%s%u", i ? ", " : "", (unsigned)r());
    std::printf("]}\n");
  }
  std::printf("],\n");
  {
    pcg32 r(19073486328125ULL);
    std::uniform_real_distribution<double> U(0., 1.);
    std::vector<double> v;
    for (int i = 0; i < 64; i++) v.push_back(U(r));
    vec("canonical", v);
  }
  {
    const double lams[] = {0.2, 1.0, 3.0, 0.3264};
    std::printf("\"exponential\": [\n");
    for (int k = 0; k < 4; k++) {
      pcg32 r(7ULL + k);
      std::exponential_distribution<double> E(lams[k]);
      std::printf("%s{\"lambda\": \"%a\", \"seed\": %d, \"v\": [", k ? "," : "", lams[k], 7 + k);
      for (int i = 0; i < 16; i++) std::printf("%s\"%a\"", i ? ", " : "", E(r));
      std::printf("]}\n");
    }
    std::printf("],\n");
  }
  {
    std::vector<std::vector<double>> W = {
      {1.0},
      {0.6, 0.35, 0.05, 0., 0., 0., 0.},
      {0.2, 0., 0.8},
      {1e-9, 1., 0.},
      {0.0, 0.0, 3.0, 0.0},
    };
    std::vector<double> w70;
    pcg32 g(99ULL);
    std::uniform_real_distribution<double> U(0., 1.);
    for (int i = 0; i < 70; i++) w70.push_back(U(g) * (i % 5 == 0 ? 0.0 : 1.0));
    W.push_back(w70);
    std::printf("\"discrete\": [\n");
    for (size_t k = 0; k < W.size(); k++) {
      pcg32 r(31ULL + k);
      std::printf("%s{\"seed\": %d, \"w\": [", k ? "," : "", (int)(31 + k));
      for (size_t i = 0; i < W[k].size(); i++) std::printf("%s\"%a\"", i ? ", " : "", W[k][i]);
      std::printf("], \"idx\": [");
      std::discrete_distribution<int> D(W[k].begin(), W[k].end());
      for (int i = 0; i < 32; i++) std::printf("%s%d", i ? ", " : "", D(r));
      std::uniform_real_distribution<double> U2(0., 1.);
      std::printf("], \"next\": \"%a\"}\n", U2(r));
    }
    std::printf("],\n");
  }
  {
    // settings::rng (src/settings.cpp:59) is a default-constructed pcg32
    pcg32 d;
    std::printf("\"default_state\": %llu,\n", (unsigned long long)state_of(d));
    // std::shuffle over a pcg32, as BranchlessPowerIterator::comb_particles
    // uses it (src/branchless_power_iterator.cpp:619-650): both of
    // libstdc++'s paths (swap positions drawn in pairs up to 65535 elements,
    // one at a time above)
    const size_t sizes[] = {1, 2, 3, 4, 7, 10, 101, 65535, 65536, 70001};
    std::printf("\"shuffle\": [\n");
    for (int k = 0; k < 10; k++) {
      const size_t n = sizes[k];
      pcg32 r(5ULL + k);
      std::vector<uint32_t> v(n);
      for (size_t i = 0; i < n; i++) v[i] = (uint32_t)i;
      std::shuffle(v.begin(), v.end(), r);
      unsigned long long check = 0;
      for (size_t i = 0; i < n; i++) check = check * 1000003ULL + v[i];
      std::printf("%s{\"n\": %zu, \"seed\": %d, \"head\": [", k ? "," : "", n, 5 + k);
      for (size_t i = 0; i < n && i < 12; i++) std::printf("%s%u", i ? ", " : "", v[i]);
      std::printf("], \"check\": %llu, \"next\": %u}\n", check, (unsigned)r());
    }
    std::printf("]\n");
  }
  std::printf("}\n");
  return 0;
}
"""


def main():
    import pyarrow  # noqa: F401  (only to locate the vendored pcg-cpp)
    inc = os.path.join(os.path.dirname(pyarrow.__file__), "include", "arrow", "vendored", "pcg")
    if not os.path.exists(os.path.join(inc, "pcg_random.hpp")):
        sys.exit("pcg_random.hpp not found under pyarrow")
    with tempfile.TemporaryDirectory() as td:
        src = os.path.join(td, "gen.cpp")
        exe = os.path.join(td, "gen")
        with open(src, "w") as f:
            f.write(CPP)
        subprocess.check_call(["g++", "-O0", "-std=c++17", "-I", inc, src, "-o", exe])
        out = subprocess.check_output([exe]).decode()
    data = json.loads(out)
    data["_provenance"] = {
        "pcg": "pcg-cpp vendored in pyarrow " + __import__("pyarrow").__version__,
        "libstdcxx": subprocess.check_output(["g++", "-dumpfullversion"]).decode().strip(),
        "script": "tests/golden/make_rng_golden.py",
    }
    with open(os.path.join(HERE, "rng_golden.json"), "w") as f:
        json.dump(data, f, indent=1)
    print("wrote", os.path.join(HERE, "rng_golden.json"))


if __name__ == "__main__":
    main()
