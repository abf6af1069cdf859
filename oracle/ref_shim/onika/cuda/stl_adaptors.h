// Stand-in: vector accessors over std::vector, and a pointer + size span.
#pragma once
#include <cstddef>
#include <vector>
#include <onika/cuda/cuda.h>
namespace onika {
namespace cuda {
template <class V>
inline auto vector_data(V& v) -> decltype(v.data()) { return v.data(); }
template <class V>
inline std::size_t vector_size(const V& v) { return v.size(); }
template <class T>
struct span {
  T* m_start = nullptr;
  std::size_t m_size = 0;
  T* begin() const { return m_start; }
  T* end() const { return m_start + m_size; }
  std::size_t size() const { return m_size; }
  T& operator[](std::size_t i) const { return m_start[i]; }
};
template <class T>
inline span<T> make_span(std::vector<T>& v) { return span<T>{v.data(), v.size()}; }
}  // namespace cuda
}  // namespace onika
