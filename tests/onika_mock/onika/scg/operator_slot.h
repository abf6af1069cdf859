// Compile-only stand-in for ADD_SLOT: a member holding a value of the slot's type.
#pragma once
#include <onika/scg/operator.h>
namespace onika {
namespace scg {
template <class T>
struct OperatorSlot {
  T value{};
  bool present = false;
  template <class... A>
  OperatorSlot(A&&...) {}
  T& operator*() { return value; }
  T* operator->() { return &value; }
  bool has_value() const { return present; }
};
}  // namespace scg
}  // namespace onika
#define ADD_SLOT(T, name, ...) ::onika::scg::OperatorSlot<T> name{__VA_ARGS__}
