// Stand-in: onika's error stream writes to stderr; its output and debug streams are dropped
// (the harness calls exaDEM's checks many times; their warnings are not needed).
#pragma once
#include <iostream>
#include <ostream>
#include <streambuf>
namespace onika {
struct NullBuf : std::streambuf {
  int overflow(int c) override { return c; }
};
inline std::ostream& null_stream() {
  static NullBuf b;
  static std::ostream s(&b);
  return s;
}
static std::ostream& lout = null_stream();
static std::ostream& lerr = std::cerr;
static std::ostream& ldbg = null_stream();
}  // namespace onika
namespace exanb {
using onika::ldbg;
using onika::lerr;
using onika::lout;
}  // namespace exanb
