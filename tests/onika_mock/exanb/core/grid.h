// Compile-only stand-in for an exaNBody grid with exaDEM's fields: per-cell
// arrays addressed by field tags (cells[c][field::rx][p]).
#pragma once
#include <cstddef>
#include <cstdint>
#include <vector>
#include <onika/math/basic_types.h>
namespace exanb {
namespace field {
template <class T, int K>
struct Tag {
  using value_type = T;
};
inline constexpr Tag<double, 0> rx{};
inline constexpr Tag<double, 1> ry{};
inline constexpr Tag<double, 2> rz{};
inline constexpr Tag<double, 3> vx{};
inline constexpr Tag<double, 4> vy{};
inline constexpr Tag<double, 5> vz{};
inline constexpr Tag<double, 6> fx{};
inline constexpr Tag<double, 7> fy{};
inline constexpr Tag<double, 8> fz{};
inline constexpr Tag<uint64_t, 9> id{};
inline constexpr Tag<uint8_t, 10> type{};
inline constexpr Tag<double, 11> mass{};
inline constexpr Tag<double, 12> radius{};
inline constexpr Tag<double, 13> homothety{};
inline constexpr Tag<uint32_t, 14> group{};
inline constexpr Tag<Quaternion, 15> orient{};
inline constexpr Tag<Vec3d, 16> vrot{};
inline constexpr Tag<Vec3d, 17> arot{};
inline constexpr Tag<Vec3d, 18> mom{};
inline constexpr Tag<Vec3d, 19> inertia{};
inline constexpr Tag<double, 20> cluster{};
}  // namespace field
struct MockCell {
  std::size_t size() const { return 0; }
  template <class T, int K>
  T* operator[](field::Tag<T, K>) {
    static std::vector<T> v(1);
    return v.data();
  }
};
struct MockGrid {
  std::vector<MockCell> c;
  MockCell* cells() { return c.data(); }
  std::size_t number_of_cells() const { return c.size(); }
  bool is_ghost_cell(std::size_t) const { return false; }
};
}  // namespace exanb
