// Minimal stand-in for yaml-cpp (absent here): a tree of scalars (kept as
// text, converted on as<T>() like yaml-cpp's stream conversion), sequences
// and maps, with the accessors the reference's parser uses.  The shim
// build's harness fills it from JSON (oracle/refshim/harness.cpp), so the
// reference's own make_settings / make_materials / make_geometry / ...
// build the problem.  Test infrastructure (oracle/refshim).
#pragma once
#include <algorithm>
#include <array>
#include <cstddef>
#include <cstdint>
#include <cstdlib>
#include <fstream>
#include <functional>
#include <iostream>
#include <map>
#include <memory>
#include <optional>
#include <set>
#include <sstream>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <unordered_map>
#include <utility>
#include <vector>

namespace YAML {
struct Mark { int line = 0, column = 0, pos = 0; };
enum class NodeTypeValue { Undefined, Null, Scalar, Sequence, Map };
namespace NodeType {
using value = NodeTypeValue;
constexpr auto Undefined = NodeTypeValue::Undefined, Null = NodeTypeValue::Null, Scalar = NodeTypeValue::Scalar,
               Sequence = NodeTypeValue::Sequence, Map = NodeTypeValue::Map;
}  // namespace NodeType

struct BadConversion : std::runtime_error {
  using std::runtime_error::runtime_error;
};

class Node;
template <class T> struct convert;

class Node {
 public:
  struct Impl {
    NodeTypeValue type = NodeTypeValue::Undefined;
    std::string scalar;
    std::vector<Node> seq;
    std::vector<std::pair<std::string, Node>> map;
  };

  Node() : p_(std::make_shared<Impl>()) {}
  static Node make(NodeTypeValue t) {
    Node n;
    n.p_->type = t;
    return n;
  }
  static Node scalar_node(const std::string& s) {
    Node n = make(NodeTypeValue::Scalar);
    n.p_->scalar = s;
    return n;
  }
  void push_back(const Node& n) { p_->seq.push_back(n); }
  void set(const std::string& k, const Node& n) { p_->map.emplace_back(k, n); }

  Node operator[](const std::string& key) const {
    if (p_->type == NodeTypeValue::Map)
      for (const auto& kv : p_->map)
        if (kv.first == key) return kv.second;
    return Node();
  }
  Node operator[](const char* key) const { return (*this)[std::string(key)]; }
  Node operator[](std::size_t i) const {
    if (p_->type == NodeTypeValue::Sequence && i < p_->seq.size()) return p_->seq[i];
    return Node();
  }
  Node operator[](int i) const { return (*this)[static_cast<std::size_t>(i)]; }
  explicit operator bool() const { return IsDefined(); }
  bool operator!() const { return !IsDefined(); }
  bool IsDefined() const { return p_->type != NodeTypeValue::Undefined; }
  bool IsNull() const { return p_->type == NodeTypeValue::Null; }
  bool IsScalar() const { return p_->type == NodeTypeValue::Scalar; }
  bool IsSequence() const { return p_->type == NodeTypeValue::Sequence; }
  bool IsMap() const { return p_->type == NodeTypeValue::Map; }
  std::size_t size() const {
    return p_->type == NodeTypeValue::Sequence ? p_->seq.size() : (p_->type == NodeTypeValue::Map ? p_->map.size() : 0);
  }
  NodeTypeValue Type() const { return p_->type; }
  Mark Mark_() const { return {}; }
  const std::string& Scalar() const { return p_->scalar; }
  const std::string& Tag() const {
    static const std::string t;
    return t;
  }
  template <class T> T as() const { return convert<T>::get(*this); }
  template <class T, class S> T as(const S& fallback) const {
    try {
      return as<T>();
    } catch (const BadConversion&) {
      return static_cast<T>(fallback);
    }
  }

  struct iterator_value;
  struct iterator {
    iterator_value operator*() const;
    const iterator_value* operator->() const;
    iterator& operator++() { return *this; }
    iterator operator++(int) { return *this; }
    bool operator!=(const iterator&) const { return false; }
    bool operator==(const iterator&) const { return true; }
  };
  using const_iterator = iterator;
  iterator begin() const { return {}; }
  iterator end() const { return {}; }

 private:
  std::shared_ptr<Impl> p_;
};

struct Node::iterator_value : Node {
  Node first, second;
};
inline Node::iterator_value Node::iterator::operator*() const { throw BadConversion("map iteration is not supported"); }
inline const Node::iterator_value* Node::iterator::operator->() const {
  throw BadConversion("map iteration is not supported");
}

template <class T> struct convert {
  static T get(const Node& n) {
    if constexpr (std::is_same_v<T, std::string>) {
      if (!n.IsScalar()) throw BadConversion("not a scalar");
      return n.Scalar();
    } else if constexpr (std::is_same_v<T, bool>) {
      if (!n.IsScalar()) throw BadConversion("not a scalar");
      const std::string& s = n.Scalar();
      if (s == "true" || s == "True" || s == "TRUE" || s == "yes" || s == "on") return true;
      if (s == "false" || s == "False" || s == "FALSE" || s == "no" || s == "off") return false;
      throw BadConversion("not a bool: " + s);
    } else if constexpr (std::is_arithmetic_v<T>) {
      if (!n.IsScalar()) throw BadConversion("not a scalar");
      std::istringstream in(n.Scalar());
      in.imbue(std::locale::classic());
      if constexpr (sizeof(T) == 1) {
        int v;
        in >> v;
        if (in.fail()) throw BadConversion("not a number: " + n.Scalar());
        return static_cast<T>(v);
      } else {
        T v;
        in >> v;
        if (in.fail()) throw BadConversion("not a number: " + n.Scalar());
        return v;
      }
    } else {
      // std::vector<U>
      using U = typename T::value_type;
      if (!n.IsSequence()) throw BadConversion("not a sequence");
      T out;
      for (std::size_t i = 0; i < n.size(); i++) out.push_back(n[i].template as<U>());
      return out;
    }
  }
};

Node LoadFile(const std::string& fname);
Node Load(const std::string& text);
}  // namespace YAML
