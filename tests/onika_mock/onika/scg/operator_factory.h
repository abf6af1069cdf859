// Compile-only stand-in: the operator factory and the static registration macro.
#pragma once
#include <onika/scg/operator.h>
namespace onika {
namespace scg {
struct OperatorNodeFactory {
  static OperatorNodeFactory* instance() {
    static OperatorNodeFactory f;
    return &f;
  }
  template <class F>
  void register_factory(const char*, F) {}
};
}  // namespace scg
}  // namespace onika
#define ONIKA_AUTORUN_INIT(name)                                    \
  static void name##_autorun();                                     \
  [[maybe_unused]] static const int name##_autorun_registered = (name##_autorun(), 0); \
  static void name##_autorun()
