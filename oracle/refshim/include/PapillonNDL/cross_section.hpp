// Stand-in for PapillonNDL's CrossSection: values on an EnergyGrid, linearly
// interpolated between the grid point at the lower index and the next one
// (on the multigroup majorant grid both points of a group carry the same
// value, so the result is that value).  Test infrastructure (oracle/refshim).
#pragma once
#include <PapillonNDL/energy_grid.hpp>

namespace pndl {
class CrossSection {
 public:
  CrossSection(const std::vector<double>& xs, std::shared_ptr<EnergyGrid> grid, std::size_t index = 0)
      : xs_(xs), grid_(grid), index_(index) {}
  double evaluate(double E, std::size_t i) const {
    const std::vector<double>& g = grid_->grid();
    if (i + 1 >= g.size() || E <= g[i]) return xs_[i];
    const double E0 = g[i], E1 = g[i + 1];
    if (E1 == E0) return xs_[i];
    return xs_[i] + (E - E0) / (E1 - E0) * (xs_[i + 1] - xs_[i]);
  }
  double evaluate(double E) const { return evaluate(E, grid_->get_lower_index(E)); }
  double operator()(double E) const { return evaluate(E); }
  double operator()(double E, std::size_t i) const { return evaluate(E, i); }
  std::size_t index() const { return index_; }
  const std::vector<double>& xs() const { return xs_; }
 private:
  std::vector<double> xs_;
  std::shared_ptr<EnergyGrid> grid_;
  std::size_t index_;
};
}  // namespace pndl
