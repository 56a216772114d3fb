// YAML::Load / LoadFile of the shim build: the deck arrives as JSON (the
// dictionary a reference deck's YAML reads as) and becomes the stand-in
// YAML::Node tree the reference's parser functions walk.  Test
// infrastructure (oracle/refshim).
#include <yaml-cpp/yaml.h>

#include <fstream>
#include <sstream>
#include <stdexcept>
#include <string>

// ------------------------------------------------------------ JSON -> Node
namespace {
struct Json {
  const std::string& s;
  std::size_t i = 0;
  explicit Json(const std::string& t) : s(t) {}
  void ws() {
    while (i < s.size() && (s[i] == ' ' || s[i] == '\n' || s[i] == '\t' || s[i] == '\r')) i++;
  }
  [[noreturn]] void bad(const char* what) {
    throw std::runtime_error(std::string("deck JSON: ") + what + " at " + std::to_string(i));
  }
  std::string str() {
    if (s[i] != '"') bad("expected a string");
    i++;
    std::string out;
    while (i < s.size() && s[i] != '"') {
      if (s[i] == '\\') {
        i++;
        char c = s[i];
        out += c == 'n' ? '\n' : c == 't' ? '\t' : c;
      } else {
        out += s[i];
      }
      i++;
    }
    if (i >= s.size()) bad("unterminated string");
    i++;
    return out;
  }
  YAML::Node value() {
    ws();
    if (i >= s.size()) bad("unexpected end");
    char c = s[i];
    if (c == '{') {
      i++;
      YAML::Node m = YAML::Node::make(YAML::NodeTypeValue::Map);
      ws();
      if (s[i] == '}') { i++; return m; }
      for (;;) {
        ws();
        std::string k = str();
        ws();
        if (s[i] != ':') bad("expected ':'");
        i++;
        m.set(k, value());
        ws();
        if (s[i] == ',') { i++; continue; }
        if (s[i] == '}') { i++; return m; }
        bad("expected ',' or '}'");
      }
    }
    if (c == '[') {
      i++;
      YAML::Node q = YAML::Node::make(YAML::NodeTypeValue::Sequence);
      ws();
      if (s[i] == ']') { i++; return q; }
      for (;;) {
        q.push_back(value());
        ws();
        if (s[i] == ',') { i++; continue; }
        if (s[i] == ']') { i++; return q; }
        bad("expected ',' or ']'");
      }
    }
    if (c == '"') return YAML::Node::scalar_node(str());
    if (s.compare(i, 4, "null") == 0) {
      i += 4;
      return YAML::Node::make(YAML::NodeTypeValue::Null);
    }
    std::size_t j = i;
    while (j < s.size() && s[j] != ',' && s[j] != ']' && s[j] != '}' && s[j] != ' ' && s[j] != '\n') j++;
    std::string tok = s.substr(i, j - i);
    i = j;
    return YAML::Node::scalar_node(tok);
  }
};
}  // namespace

namespace YAML {
Node Load(const std::string& text) {
  Json j(text);
  return j.value();
}
Node LoadFile(const std::string& fname) {
  std::ifstream f(fname);
  std::stringstream b;
  b << f.rdbuf();
  return Load(b.str());
}
}  // namespace YAML

