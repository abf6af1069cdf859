// Compile-only stand-in: instantiates the operator on the mock grid, so every
// operator class of a plugin is compiled.
#pragma once
#include <memory>
#include <exanb/core/grid.h>
#include <onika/scg/operator.h>
namespace exanb {
template <template <class> class Op>
std::shared_ptr<onika::scg::OperatorNode> make_grid_variant_operator() {
  auto op = std::make_shared<Op<MockGrid>>();
  op->execute();
  return op;
}
}  // namespace exanb
