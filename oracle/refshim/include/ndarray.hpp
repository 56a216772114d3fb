// Minimal row-major N-dimensional array standing in for the NDArray library
// the reference uses for tally arrays ([Ne][Nx][Ny][Nz], last index
// fastest) and source-file tables.  Test infrastructure (oracle/refshim).
#pragma once
#include <cstddef>
#include <initializer_list>
#include <stdexcept>
#include <string>
#include <vector>

template <class T> class NDArray {
 public:
  NDArray() = default;
  NDArray(const std::vector<std::size_t>& shape) { reallocate(shape); }
  NDArray(std::initializer_list<std::size_t> shape) { reallocate(std::vector<std::size_t>(shape)); }
  void reallocate(const std::vector<std::size_t>& shape) {
    shape_ = shape;
    std::size_t n = 1;
    for (auto s : shape_) n *= s;
    data_.assign(n, T());
  }
  void reallocate(std::initializer_list<std::size_t> shape) { reallocate(std::vector<std::size_t>(shape)); }
  void fill(const T& v) { std::fill(data_.begin(), data_.end(), v); }
  std::size_t size() const { return data_.size(); }
  const std::vector<std::size_t>& shape() const { return shape_; }
  std::vector<T>& data_vector() { return data_; }
  const std::vector<T>& data_vector() const { return data_; }
  T* data() { return data_.data(); }
  T& operator[](std::size_t i) { return data_[i]; }
  const T& operator[](std::size_t i) const { return data_[i]; }
  template <class... I> T& operator()(I... idx) { return data_[lin({static_cast<std::size_t>(idx)...})]; }
  template <class... I> const T& operator()(I... idx) const { return data_[lin({static_cast<std::size_t>(idx)...})]; }
  static NDArray load(const std::string&) { throw std::runtime_error("NDArray::load is not available in the shim build"); }
  void save(const std::string&) const {}
 private:
  std::size_t lin(std::initializer_list<std::size_t> idx) const {
    std::size_t i = 0, d = 0;
    for (auto v : idx) i = i * shape_[d++] + v;
    return i;
  }
  std::vector<std::size_t> shape_;
  std::vector<T> data_;
};
