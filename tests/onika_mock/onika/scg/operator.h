// Compile-only stand-in: the operator base class and slot flags of onika::scg.
#pragma once
#include <memory>
#include <string>
namespace onika {
namespace scg {
class OperatorNode {
 public:
  virtual ~OperatorNode() = default;
  virtual void execute() = 0;
};
struct DocString {
  const char* text;
};
enum SlotFlag { INPUT, OUTPUT, INPUT_OUTPUT, PRIVATE, REQUIRED, OPTIONAL };
}  // namespace scg
}  // namespace onika
namespace exaDEM {
using onika::scg::DocString;
using onika::scg::OperatorNode;
using namespace onika::scg;
}  // namespace exaDEM
