/*
 * Reference-side binding of the GB300 engine: a Transporter for Abeille's
 * own build.  Interface replaced: Transporter::transport
 * (include/simulation/transporter.hpp:43-46 of the reference).  This header
 * is compiled inside the reference, against its headers, and linked with
 * libabeille_gb300.so; nothing else of the reference changes -- the factory
 * hook that constructs it is shown in INTEGRATION.md.
 *
 *   GpuTransporter t(tallies, deck_text, ABX_PREC_FP64);   // or ABX_PREC_MIXED
 *   std::vector<BankedParticle> sites = t.transport(bank);
 *
 * The context is built from the deck text itself (abx_create_from_deck: the
 * library reads and flattens the multigroup deck with the reference parser's
 * conventions), so the reference's private geometry and material objects are
 * not needed.  As the reference's transporters do, transport() consumes the
 * bank (cleared on return, src/delta_tracker.cpp:262), returns the fission
 * bank in BankedParticle::operator< order, and adds the generation's scores
 * to the shared Tallies through its public score functions.  Each particle's
 * pcg32 state crosses the boundary through pcg-cpp's own stream operators
 * (no accessor is added to Particle).  The deck's mesh tallies live on the
 * device: call record_generation() where the driver calls
 * Tallies::record_generation, and read them with abx_tally_read.  Errors
 * become the reference's fatal_error (src/error.cpp), its convention for
 * every failure on this path.
 */
#ifndef ABEILLE_GB300_TRANSPORTER_HPP
#define ABEILLE_GB300_TRANSPORTER_HPP

#include <simulation/particle.hpp>
#include <simulation/tallies.hpp>
#include <simulation/transporter.hpp>
#include <utils/error.hpp>
#include <utils/settings.hpp>

#include <cstdint>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "abeille_gb300.h"

class GpuTransporter : public Transporter {
 public:
  GpuTransporter(std::shared_ptr<Tallies> t, const std::string& deck_text, int precision = ABX_PREC_FP64,
                 int device = 0)
      : Transporter(t) {
    if (abx_create_from_deck(deck_text.c_str(), precision, device, &ctx_) != ABX_OK)
      fatal_error(std::string("GPU transporter: ") + abx_last_error_string());
  }
  ~GpuTransporter() override { abx_destroy(ctx_); }
  GpuTransporter(const GpuTransporter&) = delete;
  GpuTransporter& operator=(const GpuTransporter&) = delete;

  std::vector<BankedParticle> transport(std::vector<Particle>& bank, bool noise = false,
                                        std::vector<BankedParticle>* noise_bank = nullptr,
                                        const NoiseMaker* noise_maker = nullptr) override {
    if (noise || noise_bank || noise_maker) fatal_error("noise transport is not on the GPU path");
    std::vector<abx_particle> in(bank.size());
    for (std::size_t i = 0; i < bank.size(); i++) {
      const Particle& q = bank[i];
      abx_particle& o = in[i];
      o.r[0] = q.r().x(); o.r[1] = q.r().y(); o.r[2] = q.r().z();
      o.u[0] = q.u().x(); o.u[1] = q.u().y(); o.u[2] = q.u().z();
      o.E = q.E();
      o.wgt = q.wgt();
      o.wgt2 = q.wgt2();
      o.history_id = q.history_id();
      o.rng_state = rng_state(q.rng);
      o.family_id = q.family_id();
    }
    std::vector<abx_site> out(4 * bank.size() + 64);
    std::size_t n_out = 0;
    abx_scores s{};
    int rc = abx_transport(ctx_, in.data(), in.size(), tallies->kcol(), settings::converged ? 1 : 0, out.data(),
                           out.size(), &n_out, &s);
    if (rc == ABX_ERR_CAPACITY && n_out > out.size()) {  // a larger bank than 4 sites per history
      out.resize(n_out);
      rc = abx_transport(ctx_, in.data(), in.size(), tallies->kcol(), settings::converged ? 1 : 0, out.data(),
                         out.size(), &n_out, &s);
    }
    if (rc != ABX_OK) fatal_error(std::string("GPU transporter: ") + abx_last_error_string());
    tallies->score_k_col(s.k_col);
    tallies->score_k_abs(s.k_abs);
    tallies->score_k_trk(s.k_trk);
    tallies->score_k_tot(s.k_tot);
    tallies->score_leak(s.leakage);
    tallies->score_mig_area(s.mig_area);
    std::vector<BankedParticle> sites(n_out);
    for (std::size_t i = 0; i < n_out; i++) {
      const abx_site& o = out[i];
      BankedParticle& b = sites[i];
      b.r = Position(o.r[0], o.r[1], o.r[2]);
      b.u = Direction(o.u[0], o.u[1], o.u[2]);
      b.E = o.E;
      b.wgt = o.wgt;
      b.wgt2 = o.wgt2;
      b.parent_history_id = o.parent_history_id;
      b.parent_daughter_id = o.parent_daughter_id;
      b.family_id = o.family_id;
    }
    bank.clear();
    return sites;
  }

  // MeshTally::record_generation for the deck's mesh tallies on the device.
  void record_generation(double multiplier = 1.) {
    if (abx_tally_record_generation(ctx_, multiplier) != ABX_OK)
      fatal_error(std::string("GPU transporter: ") + abx_last_error_string());
  }

  abx_ctx* context() const { return ctx_; }

  // The state word of a pcg32 ("multiplier increment state" in pcg-cpp's
  // stream form).
  static uint64_t rng_state(const pcg32& rng) {
    std::stringstream ss;
    ss << rng;
    unsigned long long mult = 0, inc = 0, state = 0;
    ss >> mult >> inc >> state;
    return state;
  }

 private:
  abx_ctx* ctx_ = nullptr;
};

#endif
