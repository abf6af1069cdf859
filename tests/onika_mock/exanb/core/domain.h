// Compile-only stand-in for exaNBody's Domain (bounds, periodicity, cell size).
#pragma once
#include <onika/math/basic_types.h>
namespace exanb {
struct Domain {
  AABB bounds() const { return AABB{}; }
  bool periodic_boundary_x() const { return false; }
  bool periodic_boundary_y() const { return false; }
  bool periodic_boundary_z() const { return false; }
  double cell_size() const { return 1.0; }
};
}  // namespace exanb
