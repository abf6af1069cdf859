// Stand-in: a physical quantity is its value in the internal unit system.
#pragma once
#include <yaml-cpp/yaml.h>
namespace onika {
namespace physics {
struct Quantity {
  double m_value = 0.0;
  double convert() const { return m_value; }
};
}  // namespace physics
}  // namespace onika
using onika::physics::Quantity;
