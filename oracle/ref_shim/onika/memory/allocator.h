// Stand-in: onika's managed-memory vector is a plain host vector here.
#pragma once
#include <cstddef>
#include <vector>
namespace onika {
namespace memory {
template <class T>
using CudaMMVector = std::vector<T>;
template <class T>
struct MemoryUsage {
  static inline std::size_t memory_bytes(const T&) { return sizeof(T); }
};
template <class T>
inline std::size_t memory_bytes(const T&) { return sizeof(T); }
}  // namespace memory
}  // namespace onika
