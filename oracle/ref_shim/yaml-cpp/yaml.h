// Stand-in for yaml-cpp: an inert node type, enough for exaDEM's YAML decoders
// to compile.  The harness never decodes YAML (the functions below are declared
// only and never called).
#pragma once
#include <cstddef>
#include <string>
namespace YAML {
class Node {
 public:
  bool IsMap() const;
  bool IsSequence() const;
  bool IsScalar() const;
  bool IsDefined() const;
  bool IsNull() const;
  std::size_t size() const;
  Node operator[](const char* key) const;
  Node operator[](const std::string& key) const;
  Node operator[](std::size_t index) const;
  template <class T>
  T as() const;
  std::string Scalar() const;
  explicit operator bool() const;
};
template <class T>
struct convert;
}  // namespace YAML
