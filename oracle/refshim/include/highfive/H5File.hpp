// Compile-only, do-nothing stand-in for HighFive (the reference's HDF5
// writer): the shim build writes no result file.  Test infrastructure
// (oracle/refshim).
#pragma once
#include <cstddef>
#include <string>
#include <vector>

namespace H5 {
struct DataSpace {
  template <class... A> DataSpace(const A&...) {}
  template <class T> static DataSpace From(const T&) { return DataSpace(); }
};
struct DataSpaceRead {
  std::vector<std::size_t> getDimensions() const { return {}; }
};
struct DataSet {
  DataSpaceRead getSpace() const { return {}; }
  template <class T> void read(T*) const {}
  template <class T> void write(const T&) {}
  template <class T> void write_raw(const T*) {}
  template <class T> DataSet& createAttribute(const std::string&, const T&) { return *this; }
};
struct Group {
  DataSet getDataSet(const std::string&) const { return {}; }
  template <class T> DataSet createDataSet(const std::string&, const DataSpace&) { return {}; }
  template <class T> DataSet createDataSet(const std::string&, const T&) { return {}; }
  template <class T> Group& createAttribute(const std::string&, const T&) { return *this; }
  Group createGroup(const std::string&) { return {}; }
};
struct File : Group {
  enum : unsigned { ReadOnly = 0, ReadWrite = 1, Create = 2, Truncate = 4, Overwrite = 4 };
  template <class... A> File(const A&...) {}
};
}  // namespace H5
namespace HighFive = H5;
