// mul_policy.cuh -- where the FP64 multiplies (and additions) of a kernel run.
// MulFP64: the FP64 pipe.  MulInt: the branch-free integer-pipe IEEE multiply
// of emu64.cuh, which returns the same bits; failed() reports an operand
// outside its fast path (subnormal, infinite, NaN, out-of-range product),
// after which the caller recomputes its block of arithmetic with MulFP64.
// AllInt: multiplies and additions on the integer pipe, same contract.
// A kernel instance is compiled per placement mode: bit 0 places the
// rotation multiplies of the integration, bit 1 its linear ones (Verlet
// pushes, quotient estimates), bit 2 the contact law's on the integer pipe.
#pragma once
#include <type_traits>

#include "emu64.cuh"

namespace dem {

struct MulFP64 {
  __device__ __forceinline__ double mul(double a, double b) const { return __dmul_rn(a, b); }
  __device__ __forceinline__ double add(double a, double b) const { return __dadd_rn(a, b); }
  __device__ __forceinline__ double sub(double a, double b) const { return __dsub_rn(a, b); }
  __device__ __forceinline__ double twice(double a) const { return __dmul_rn(a, 2.0); }
  __device__ __forceinline__ double half(double a) const { return __dmul_rn(a, 0.5); }
  __device__ __forceinline__ double neghalf(double a) const { return __dmul_rn(a, -0.5); }
  __device__ __forceinline__ bool failed() const { return false; }
};
struct MulInt {
  bool bad = false;
  __device__ __forceinline__ double mul(double a, double b) { return emu_dmul_nb(a, b, bad); }
  __device__ __forceinline__ double add(double a, double b) const { return __dadd_rn(a, b); }
  __device__ __forceinline__ double sub(double a, double b) const { return __dsub_rn(a, b); }
  __device__ __forceinline__ double twice(double a) { return emu_mul2_nb(a, bad); }
  __device__ __forceinline__ double half(double a) { return emu_mulhalf_nb(a, bad); }
  __device__ __forceinline__ double neghalf(double a) { return emu_mulnhalf_nb(a, bad); }
  __device__ __forceinline__ bool failed() const { return bad; }
};
// multiplies and additions on the integer pipe (emu_dmul_nb, emu_dadd_nb): a
// kernel that is bound by the FP64 pipe runs a share of its work items with it,
// so both pipes work at once; square roots and divisions stay on the FP64 pipe
struct AllInt {
  bool bad = false;
  __device__ __forceinline__ double mul(double a, double b) { return emu_dmul_nb(a, b, bad); }
  __device__ __forceinline__ double add(double a, double b) { return emu_dadd_nb(a, b, bad); }
  __device__ __forceinline__ double sub(double a, double b) { return emu_dsub_nb(a, b, bad); }
  __device__ __forceinline__ double twice(double a) { return emu_mul2_nb(a, bad); }
  __device__ __forceinline__ double half(double a) { return emu_mulhalf_nb(a, bad); }
  __device__ __forceinline__ double neghalf(double a) { return emu_mulnhalf_nb(a, bad); }
  __device__ __forceinline__ bool failed() const { return bad; }
};
template <int Mode>
using RotMul = typename std::conditional<(Mode & 1) != 0, MulInt, MulFP64>::type;
template <int Mode>
using LinMul = typename std::conditional<(Mode & 2) != 0, MulInt, MulFP64>::type;

// the kernel instance compiled for a multiply placement
template <class F>
F by_mode(int mode, F m0, F m1, F m2, F m3) {
  switch (mode & 3) {
    case 1: return m1;
    case 2: return m2;
    case 3: return m3;
    default: return m0;
  }
}

}  // namespace dem
