// Shim: boost::unordered_flat_map as std::unordered_map (same interface for
// the lookups the reference makes).  Test infrastructure (oracle/refshim).
#pragma once
#include <unordered_map>
namespace boost {
namespace unordered {
template <class K, class V, class H = std::hash<K>, class E = std::equal_to<K>,
          class A = std::allocator<std::pair<const K, V>>>
using unordered_flat_map = std::unordered_map<K, V, H, E, A>;
}
using unordered::unordered_flat_map;
}  // namespace boost
