// Compile-only stand-ins for the continuous-energy classes of PapillonNDL that
// the reference's headers name.  The shim build runs multigroup decks only;
// every accessor throws.  Test infrastructure (oracle/refshim).
#pragma once
#include <PapillonNDL/cross_section.hpp>
#include <stdexcept>
#include <string>

namespace pndl {
[[noreturn]] inline void pndl_absent() { throw std::runtime_error("PapillonNDL is not available in the shim build"); }
struct ACE {
  enum class Type { ASCII, BINARY };
  static constexpr Type ASCII = Type::ASCII, BINARY = Type::BINARY;
  ACE(const std::string&, Type = Type::ASCII) { pndl_absent(); }
};
struct Tab1Stub {
  const std::vector<double>& x() const { pndl_absent(); }
  const std::vector<double>& y() const { pndl_absent(); }
  double operator()(double) const { pndl_absent(); }
};
struct XSPacket {
  double total = 0, elastic = 0, inelastic = 0, absorption = 0, capture = 0, fission = 0, heating = 0;
};
struct AngleEnergyPacket {
  double cos_angle = 0, energy = 0;
};
struct LinLin {};
class PCTable {
 public:
  PCTable() = default;
  template <class... A> PCTable(const A&...) {}
  template <class RNG> double sample_value(double, RNG&) const { pndl_absent(); }
  double sample_value(double) const { pndl_absent(); }
  double min_value() const { pndl_absent(); }
  double max_value() const { pndl_absent(); }
  const std::vector<double>& values() const { pndl_absent(); }
  const std::vector<double>& pdf() const { pndl_absent(); }
  const std::vector<double>& cdf() const { pndl_absent(); }
};
class STIncoherentInelastic {
 public:
  const Tab1Stub& xs() const { pndl_absent(); }
};
class STCoherentElastic {
 public:
  const std::vector<double>& bragg_edges() const { pndl_absent(); }
};
class STThermalScatteringLaw {
 public:
  const STIncoherentInelastic& incoherent_inelastic() const { pndl_absent(); }
  const STCoherentElastic& coherent_elastic() const { pndl_absent(); }
  double max_energy() const { pndl_absent(); }
  double temperature() const { pndl_absent(); }
};
struct URRPTablesStub {
  const std::vector<double>& energy() const { pndl_absent(); }
};
class STNeutron {
 public:
  const URRPTablesStub& urr_ptables() const { pndl_absent(); }
  const EnergyGrid& energy_grid() const { pndl_absent(); }
  double temperature() const { pndl_absent(); }
  double awr() const { pndl_absent(); }
  uint32_t zaid() const { pndl_absent(); }
};
class ElasticDBRC {};
struct PNDLException : std::runtime_error { using std::runtime_error::runtime_error; };
}  // namespace pndl
