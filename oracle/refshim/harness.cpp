// Driver for the reference's own multigroup transport code, built from its
// unmodified sources by oracle/refshim/build_ref.py (test infrastructure:
// only tests/ run it, to pin the oracle to the reference).
//
//   abeille_ref DECK.json NSAMPLE BANK_IN KCOL CONVERGED OUT_PREFIX
//
// DECK.json: a reference-format deck as JSON (the dictionary a deck's YAML
// reads as).  The reference's own parser functions build the problem from
// it (src/parser.cpp: make_settings, make_materials, make_geometry,
// make_tallies, make_transporter, make_sources, make_simulation).
// NSAMPLE > 0: Simulation::sample_sources(NSAMPLE) (src/simulation.cpp:55-77)
// writes OUT_PREFIX.bank; BANK_IN ("-" for none): a bank of abx_particle
// records to transport with Transporter::transport (delta_tracker.cpp,
// surface_tracker.cpp, ...) after setting Tallies::kcol to KCOL and
// settings::converged to CONVERGED.  Writes OUT_PREFIX.sites (abx_site
// records, the returned fission bank in its order), OUT_PREFIX.scores (the
// raw generation sums k_col k_abs k_trk leakage k_tot mig_area) and
// OUT_PREFIX.tally<i> (the generation array of every mesh tally, collision
// estimators first, then track-length ones, each [Ne][Nx][Ny][Nz] doubles).
//
// The particle's pcg32 state is moved in and out through pcg-cpp's own
// stream operators ("multiplier increment state").

#include <yaml-cpp/yaml.h>

#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <list>
#include <sstream>
#include <string>
#include <vector>

// The harness reads private members of Tallies and MeshTally (the scores
// and tally arrays have no public accessors); the reference's own
// translation units are compiled without this.
#define private public
#define protected public
#include <geometry/geometry.hpp>
#include <materials/material.hpp>
#include <simulation/collision_mesh_tally.hpp>
#include <simulation/mesh_tally.hpp>
#include <simulation/particle.hpp>
#include <simulation/simulation.hpp>
#include <simulation/tallies.hpp>
#include <simulation/track_length_mesh_tally.hpp>
#include <simulation/transporter.hpp>
#include <utils/parser.hpp>
#include <utils/settings.hpp>
#undef private
#undef protected

extern "C" {
#include "../../include/abeille_gb300.h"
}

void make_entropy_mesh(const YAML::Node& entropy);

// ------------------------------------------------------------ pcg32 state
static uint64_t rng_state_of(const pcg32& rng) {
  std::stringstream ss;
  ss << rng;
  unsigned long long mult, inc, state;
  ss >> mult >> inc >> state;
  return state;
}
static void set_rng_state(pcg32& rng, uint64_t state) {
  std::stringstream in;
  in << rng;
  unsigned long long mult, inc, old;
  in >> mult >> inc >> old;
  std::stringstream out;
  out << mult << ' ' << inc << ' ' << (unsigned long long)state;
  out >> rng;
  if (out.fail() || rng_state_of(rng) != state) throw std::runtime_error("could not set the pcg32 state");
}

static void write_bin(const std::string& path, const void* p, std::size_t bytes) {
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) throw std::runtime_error("cannot write " + path);
  if (bytes) std::fwrite(p, 1, bytes, f);
  std::fclose(f);
}

int main(int argc, char** argv) {
  if (argc != 7) {
    std::fprintf(stderr, "usage: abeille_ref DECK.json NSAMPLE BANK_IN KCOL CONVERGED OUT_PREFIX\n");
    return 2;
  }
  try {
    // the reference prints progress to stdout; keep it out of the way
    std::cout.setstate(std::ios::failbit);
    const YAML::Node input = YAML::LoadFile(argv[1]);
    const long nsample = std::atol(argv[2]);
    const std::string bank_in = argv[3];
    const double kcol = std::atof(argv[4]);
    const bool converged = std::atoi(argv[5]) != 0;
    const std::string out = argv[6];

    // src/parser.cpp:77-137 (parse_input_file), without the output file
    make_settings(input);
    make_materials(input);
    make_geometry(input);
    make_tallies(input);
    make_transporter();
    make_sources(input);
    make_simulation();
    if (input["entropy"] && input["entropy"].IsMap()) make_entropy_mesh(input["entropy"]);

    if (nsample > 0) {
      std::vector<Particle> src = simulation->sample_sources(static_cast<std::size_t>(nsample));
      std::vector<abx_particle> outp(src.size());
      for (std::size_t i = 0; i < src.size(); i++) {
        const Particle& p = src[i];
        abx_particle& q = outp[i];
        q.r[0] = p.r().x(); q.r[1] = p.r().y(); q.r[2] = p.r().z();
        q.u[0] = p.u().x(); q.u[1] = p.u().y(); q.u[2] = p.u().z();
        q.E = p.E(); q.wgt = p.wgt(); q.wgt2 = p.wgt2();
        q.history_id = p.history_id();
        q.rng_state = rng_state_of(p.rng);
        q.family_id = p.family_id();
      }
      write_bin(out + ".bank", outp.data(), outp.size() * sizeof(abx_particle));
    }

    if (bank_in != "-") {
      std::ifstream f(bank_in, std::ios::binary);
      std::vector<char> raw((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
      const std::size_t n = raw.size() / sizeof(abx_particle);
      const abx_particle* in = reinterpret_cast<const abx_particle*>(raw.data());
      std::vector<Particle> bank;
      bank.reserve(n);
      for (std::size_t i = 0; i < n; i++) {
        const abx_particle& q = in[i];
        bank.emplace_back(Position(q.r[0], q.r[1], q.r[2]), Direction(q.u[0], q.u[1], q.u[2]), q.E, q.wgt, q.wgt2,
                          q.history_id);
        bank.back().set_family_id(q.family_id);
        set_rng_state(bank.back().rng, q.rng_state);
      }
      settings::converged = converged;
      tallies->set_kcol(kcol);
      tallies->set_total_weight(1.);
      std::vector<BankedParticle> sites = transporter->transport(bank);
      std::vector<abx_site> outs(sites.size());
      for (std::size_t i = 0; i < sites.size(); i++) {
        const BankedParticle& b = sites[i];
        abx_site& s = outs[i];
        s.r[0] = b.r.x(); s.r[1] = b.r.y(); s.r[2] = b.r.z();
        s.u[0] = b.u.x(); s.u[1] = b.u.y(); s.u[2] = b.u.z();
        s.E = b.E; s.wgt = b.wgt; s.wgt2 = b.wgt2;
        s.parent_history_id = b.parent_history_id;
        s.parent_daughter_id = b.parent_daughter_id;
        s.family_id = b.family_id;
      }
      write_bin(out + ".sites", outs.data(), outs.size() * sizeof(abx_site));
      FILE* fs = std::fopen((out + ".scores").c_str(), "w");
      std::fprintf(fs, "%.17g %.17g %.17g %.17g %.17g %.17g\n", tallies->k_col_score, tallies->k_abs_score,
                   tallies->k_trk_score, tallies->leak_score, tallies->k_tot_score, tallies->mig_area_score);
      std::fclose(fs);
      int ti = 0;
      for (const auto& t : tallies->collision_mesh_tallies_)
        write_bin(out + ".tally" + std::to_string(ti++), t->tally_gen.data(), t->tally_gen.size() * sizeof(double));
      for (const auto& t : tallies->track_length_mesh_tallies_)
        write_bin(out + ".tally" + std::to_string(ti++), t->tally_gen.data(), t->tally_gen.size() * sizeof(double));
    }
  } catch (const std::exception& e) {
    std::fprintf(stderr, "abeille_ref: %s\n", e.what());
    return 1;
  }
  return 0;
}
