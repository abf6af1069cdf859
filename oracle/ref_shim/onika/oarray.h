#pragma once
#include <cstddef>
namespace onika {
template <class T, std::size_t N>
struct oarray_t {
  T x[N];
  T& operator[](std::size_t i) { return x[i]; }
  const T& operator[](std::size_t i) const { return x[i]; }
};
}  // namespace onika
