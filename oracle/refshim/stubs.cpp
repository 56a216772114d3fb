// Stand-ins for the reference functions whose translation units the shim
// build leaves out (continuous-energy nuclear data, tabulated source
// energies, exact cancellation: they need PapillonNDL data or the Sobol
// tables, and the multigroup path never calls them).  Each throws if
// reached.  Test infrastructure (oracle/refshim).
#include <materials/ce_nuclide.hpp>
#include <simulation/basic_exact_mg_cancelator.hpp>
#include <simulation/exact_mg_cancelator.hpp>
#include <simulation/tabulated_energy.hpp>
#include <utils/nd_directory.hpp>

#include <stdexcept>

[[noreturn]] static void outside_mg(const char* what) {
  throw std::runtime_error(std::string(what) + " is outside the multigroup path of the shim build");
}

bool CENuclide::has_urr() const { outside_mg("CENuclide"); }
uint32_t CENuclide::zaid() const { outside_mg("CENuclide"); }
NDDirectory::NDDirectory(const std::filesystem::path&, TemperatureInterpolation, bool) { outside_mg("NDDirectory"); }
NDDirectory::CENuclidePacket NDDirectory::load_nuclide(const std::string&, double) { outside_mg("NDDirectory"); }
void NDDirectory::set_dbrc_nuclides(const std::vector<std::string>&) { outside_mg("NDDirectory"); }
std::shared_ptr<BasicExactMGCancelator> make_basic_exact_mg_cancelator(const YAML::Node&) {
  outside_mg("exact cancellation");
}
std::shared_ptr<ExactMGCancelator> make_exact_mg_cancelator(const YAML::Node&) { outside_mg("exact cancellation"); }
std::shared_ptr<TabulatedEnergy> make_tabulated_energy(const YAML::Node&) { outside_mg("tabulated energy"); }
