// Stand-in for PapillonNDL's EnergyGrid (the reference's third-party nuclear
// data library, absent here).  Only the lookup the multigroup majorant uses is
// functional: get_lower_index(E) is the index i of the last grid point with
// grid[i] <= E (clamped to the grid), as an interpolation search must return
// for a grid with repeated points [b0, b1, b1, b2, ...].  Test infrastructure
// for building the reference's own sources (oracle/refshim).
#pragma once
#include <algorithm>
#include <cstddef>
#include <memory>
#include <vector>

namespace pndl {
class EnergyGrid {
 public:
  EnergyGrid(const std::vector<double>& grid, uint32_t = 0) : grid_(grid) {}
  const std::vector<double>& grid() const { return grid_; }
  std::size_t size() const { return grid_.size(); }
  double min_energy() const { return grid_.front(); }
  double max_energy() const { return grid_.back(); }
  std::size_t get_lower_index(double E) const {
    if (E <= grid_.front()) return 0;
    if (E >= grid_.back()) return grid_.size() - 1;
    return static_cast<std::size_t>(std::upper_bound(grid_.begin(), grid_.end(), E) - grid_.begin()) - 1;
  }
 private:
  std::vector<double> grid_;
};
}  // namespace pndl
