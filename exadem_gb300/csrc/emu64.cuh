// emu64.cuh -- IEEE 754 binary64 multiplication, round to nearest even,
// computed on the integer pipe.
//
// On sm_103a the FP64 pipe retires about two lanes per clock per SM, 1/64 of
// the FP32 rate, while the integer pipe retires 64.  A warp's FP64 multiply
// holds its sub-partition's FP64 unit for ~64 clocks; the same product formed
// from 32-bit integer partial products takes ~40 integer instructions on a
// pipe that is otherwise idle in the integration and contact kernels.  Kernels
// that are bound by the FP64 pipe therefore route part of their multiplies
// here, and the two pipes run concurrently.
//
// emu_dmul(a, b) returns exactly the bits of RN(a * b) (the IEEE 754-2008
// multiplication, roundTiesToEven), by the textbook method: unpack the
// significands with their hidden bit, form the 106-bit product from four
// 32 x 32 -> 64 partial products, normalise it (the top bit is bit 104 or
// 105), round on the guard bit with a sticky bit, and pack.  The rounding
// increment is added to the packed exponent+significand word, so a carry out
// of the significand bumps the exponent, and an exponent that reaches 2047
// packs to infinity, the correctly rounded overflow.
//
// Fast path: both operands normal.  Zero times a normal operand returns the
// signed zero.  Subnormal, infinite or NaN operands, and products whose
// exponent falls outside the normal range, go to the hardware multiply.
//
// The header compiles for the host too (plain C++, no intrinsics), where the
// fallback is the host's IEEE multiply; the host build is exercised by a CPU
// test against the host's own products.
#pragma once
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define EMU_HD __host__ __device__ __forceinline__
#else
#define EMU_HD inline
#endif

namespace dem {

// The bits of x through an opaque move: the compiler cannot tell that the
// integer came from a double, so it cannot turn integer tests of the bits
// (zero, exponent range) back into floating-point compares, which would
// issue on the FP64 pipe (one per multiply, measured with the per-pipe
// instruction counters).
EMU_HD uint64_t emu_bits(double x) {
#if defined(__CUDA_ARCH__)
  uint64_t u;
  asm("mov.b64 %0, %1;" : "=l"(u) : "d"(x));
  return u;
#else
  uint64_t u;
  memcpy(&u, &x, 8);
  return u;
#endif
}

EMU_HD double emu_double(uint64_t u) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)u);
#else
  double x;
  memcpy(&x, &u, 8);
  return x;
#endif
}

EMU_HD double emu_native_mul(double a, double b) {
#if defined(__CUDA_ARCH__)
  return __dmul_rn(a, b);
#else
  return a * b;
#endif
}

// Operands outside the fast path: a zero times a normal number is a signed
// zero; everything else (subnormal, infinite, NaN) is the hardware product.
EMU_HD double emu_dmul_special(double a, double b, uint64_t ua, uint64_t ub, uint32_t ea, uint32_t eb) {
  const uint64_t mag = 0x7fffffffffffffffull;
  const bool za = (ua & mag) == 0, zb = (ub & mag) == 0;
  if ((za && eb - 1u < 2046u) || (zb && ea - 1u < 2046u) || (za && zb))
    return emu_double((ua ^ ub) & ~mag);
  return emu_native_mul(a, b);
}

EMU_HD double emu_dmul(double a, double b) {
  const uint64_t ua = emu_bits(a), ub = emu_bits(b);
  const uint32_t ha = (uint32_t)(ua >> 32), hb = (uint32_t)(ub >> 32);
  const uint32_t ea = (ha >> 20) & 0x7ffu, eb = (hb >> 20) & 0x7ffu;
  if (ea - 1u >= 2046u || eb - 1u >= 2046u) return emu_dmul_special(a, b, ua, ub, ea, eb);
  // significands with the hidden bit: ma = (ma_hi : la), 21 + 32 bits
  const uint32_t la = (uint32_t)ua, lb = (uint32_t)ub;
  const uint32_t ma = (ha & 0xfffffu) | 0x100000u, mb = (hb & 0xfffffu) | 0x100000u;
  const uint64_t ll = (uint64_t)la * lb;                          // < 2^64
  const uint64_t mid = (uint64_t)la * mb + (uint64_t)ma * lb;     // < 2^54
  const uint64_t hh = (uint64_t)ma * mb;                          // < 2^42
  const uint64_t lo = ll + (mid << 32);
  const uint64_t hi = hh + (mid >> 32) + (lo < ll ? 1u : 0u);     // product = hi * 2^64 + lo, in [2^104, 2^106)
  const uint32_t t = (uint32_t)(hi >> 41);                        // 1 when the top bit is bit 105
  const uint32_t sh = 12u - t;
  const uint64_t m = (hi << sh) | (lo >> (64u - sh));             // 53-bit significand, bit 52 set
  const uint64_t rest = lo << sh;                                 // guard bit 63, sticky bits 62..0
  const int e = (int)(ea + eb) - 1023 + (int)t;                   // biased exponent of the result
  if ((uint32_t)(e - 1) >= 2046u) return emu_native_mul(a, b);    // subnormal / zero / overflowing result
  const uint64_t inc = (rest >> 63) & (uint64_t)(((rest << 1) != 0) | (uint32_t)(m & 1u));
  const uint64_t sign = (ua ^ ub) & 0x8000000000000000ull;
  return emu_double(sign | ((((uint64_t)(e - 1)) << 52) + m + inc));
}

// Branch-free form for kernels that chain many multiplies: no branch splits
// the instruction stream, so independent products interleave.  A zero times a
// normal number or a zero is handled inline (the signed zero); every other
// case outside the fast path (subnormal, infinite or NaN operand, product out
// of the normal range) sets `bad`, returns an unspecified value, and the
// caller recomputes its whole block of arithmetic with hardware multiplies.
EMU_HD double emu_dmul_nb(double a, double b, bool& bad) {
  const uint64_t ua = emu_bits(a), ub = emu_bits(b);
  const uint32_t ha = (uint32_t)(ua >> 32), hb = (uint32_t)(ub >> 32);
  const uint32_t ea = (ha >> 20) & 0x7ffu, eb = (hb >> 20) & 0x7ffu;
  const uint32_t la = (uint32_t)ua, lb = (uint32_t)ub;
  const uint32_t ma = (ha & 0xfffffu) | 0x100000u, mb = (hb & 0xfffffu) | 0x100000u;
  const uint64_t ll = (uint64_t)la * lb;
  const uint64_t mid = (uint64_t)la * mb + (uint64_t)ma * lb;
  const uint64_t hh = (uint64_t)ma * mb;
  const uint64_t lo = ll + (mid << 32);
  const uint64_t hi = hh + (mid >> 32) + (lo < ll ? 1u : 0u);
  const uint32_t t = (uint32_t)(hi >> 41);
  const uint32_t sh = 12u - t;
  const uint64_t m = (hi << sh) | (lo >> (64u - sh));
  const uint64_t rest = lo << sh;
  const int e = (int)(ea + eb) - 1023 + (int)t;
  const uint64_t inc = (rest >> 63) & (uint64_t)(((rest << 1) != 0) | (uint32_t)(m & 1u));
  const uint64_t sign = (ua ^ ub) & 0x8000000000000000ull;
  const bool na = ea - 1u < 2046u, nb = eb - 1u < 2046u;
  const bool za = (ua << 1) == 0, zb = (ub << 1) == 0;
  const bool zero = (za && (nb || zb)) || (zb && na);
  const bool fast = na && nb && (uint32_t)(e - 1) < 2046u;
  bad |= !(fast || zero);
  return emu_double(zero ? sign : (sign | ((((uint64_t)(e - 1)) << 52) + m + inc)));
}

// x * 2, x * 0.5, x * -0.5 in the same branch-free form: an exponent step for
// normal x whose result stays normal, x itself (sign adjusted) for a zero.
EMU_HD double emu_mul2_nb(double x, bool& bad) {
  const uint64_t u = emu_bits(x);
  const uint32_t e = (uint32_t)(u >> 52) & 0x7ffu;
  const bool z = (u << 1) == 0;
  bad |= !(e - 1u < 2045u || z);
  return z ? x : emu_double(u + (1ull << 52));
}

EMU_HD double emu_mulhalf_nb(double x, bool& bad) {
  const uint64_t u = emu_bits(x);
  const uint32_t e = (uint32_t)(u >> 52) & 0x7ffu;
  const bool z = (u << 1) == 0;
  bad |= !(e - 2u < 2045u || z);
  return z ? x : emu_double(u - (1ull << 52));
}

EMU_HD double emu_mulnhalf_nb(double x, bool& bad) {
  const uint64_t u = emu_bits(x);
  const uint32_t e = (uint32_t)(u >> 52) & 0x7ffu;
  const bool z = (u << 1) == 0;
  bad |= !(e - 2u < 2045u || z);
  return emu_double((z ? u : u - (1ull << 52)) ^ 0x8000000000000000ull);
}

// x * 2 and x * 0.5 for normal x whose result stays normal: exponent +-1.
// Both are exact, so the result equals the IEEE product; other inputs take
// the hardware multiply.
EMU_HD double emu_mul2(double x) {
  const uint64_t u = emu_bits(x);
  const uint32_t e = (uint32_t)(u >> 52) & 0x7ffu;
  if (e - 1u < 2045u) return emu_double(u + (1ull << 52));
  return emu_native_mul(x, 2.0);
}

EMU_HD double emu_mulhalf(double x) {
  const uint64_t u = emu_bits(x);
  const uint32_t e = (uint32_t)(u >> 52) & 0x7ffu;
  if (e - 2u < 2045u) return emu_double(u - (1ull << 52));
  return emu_native_mul(x, 0.5);
}

// x * -0.5: the exact halving with the sign flipped, otherwise the hardware
// multiply by -0.5 (so NaN operands keep the hardware's bits).
EMU_HD double emu_mulnhalf(double x) {
  const uint64_t u = emu_bits(x);
  const uint32_t e = (uint32_t)(u >> 52) & 0x7ffu;
  if (e - 2u < 2045u) return emu_double((u - (1ull << 52)) ^ 0x8000000000000000ull);
  return emu_native_mul(x, -0.5);
}

// IEEE 754 binary64 addition, round to nearest even, on the integer pipe, in
// the branch-free form of emu_dmul_nb.  Textbook method (as in Hauser's
// SoftFloat): order the operands by magnitude, place both significands with
// their hidden bit at bit 62 (10 bits below the result's last bit), shift the
// smaller one right by the exponent difference with every bit shifted out
// ORed into bit 0 ("jamming"), add or subtract, normalise the top bit back to
// bit 62 (a carry shifts right, jamming again; a cancellation shifts left,
// exactly, since it only happens when nothing was shifted out or by one
// place), then round on bit 9 with the bits below as sticky and pack.  The
// jammed bit 0 makes the computed sum odd whenever bits were lost, so it can
// never sit on a rounding boundary (multiples of 2^8): it rounds like the
// exact sum.  Operands that are zero or normal stay on the fast path; an exact
// cancellation gives +0 and the sum of two zeros the zero that is negative
// only when both are.  A subnormal, infinite or NaN operand, or a result
// below the normal range or overflowing before rounding, sets `bad` (the
// caller recomputes with the FP64 pipe); rounding that carries into the
// exponent 2047 packs to infinity, the correctly rounded overflow.
EMU_HD int emu_clz64(uint64_t x) {
#if defined(__CUDA_ARCH__)
  return __clzll((long long)x);
#else
  return x ? __builtin_clzll(x) : 64;
#endif
}
EMU_HD double emu_dadd_nb(double a, double b, bool& bad) {
  const uint64_t ua = emu_bits(a), ub = emu_bits(b);
  const uint64_t mag = 0x7fffffffffffffffull, frac = 0xfffffffffffffull;
  const bool sw = (ua & mag) < (ub & mag);
  const uint64_t ux = sw ? ub : ua, uy = sw ? ua : ub;  // |x| >= |y|
  const uint32_t ex = (uint32_t)(ux >> 52) & 0x7ffu, ey = (uint32_t)(uy >> 52) & 0x7ffu;
  const bool zx = (ux << 1) == 0, zy = (uy << 1) == 0;
  const bool ok_in = (ex - 1u < 2046u || zx) && (ey - 1u < 2046u || zy);
  const uint64_t mx = zx ? 0ull : (((ux & frac) | (1ull << 52)) << 10);
  const uint64_t my0 = zy ? 0ull : (((uy & frac) | (1ull << 52)) << 10);
  const uint32_t d = zy ? 63u : (ex - ey < 63u ? ex - ey : 63u);
  const uint64_t lost = d ? (my0 << (64u - d)) : 0ull;
  const uint64_t my = (my0 >> d) | (lost != 0 ? 1ull : 0ull);
  const bool sub = ((ux ^ uy) >> 63) != 0;
  uint64_t r = sub ? mx - my : mx + my;
  const uint32_t c = (uint32_t)(r >> 63);
  r = c ? ((r >> 1) | (r & 1ull)) : r;
  const int lz = r ? emu_clz64(r) - 1 : 0;
  r <<= lz;
  const int e = (int)ex + (int)c - lz;
  const uint64_t m = r >> 10;
  const uint64_t inc = ((r >> 9) & 1ull) & (((r & 0x1ffull) != 0 ? 1ull : 0ull) | (m & 1ull));
  const uint64_t sx = ux & 0x8000000000000000ull;
  const uint64_t zsign = sub ? 0ull : sx;  // x + (-x) = +0; -0 + -0 = -0
  bad |= !(ok_in && (r == 0 || (uint32_t)(e - 1) < 2046u));
  return emu_double(r == 0 ? zsign : (sx | ((((uint64_t)(e - 1)) << 52) + m + inc)));
}
EMU_HD double emu_dsub_nb(double a, double b, bool& bad) {
  return emu_dadd_nb(a, emu_double(emu_bits(b) ^ 0x8000000000000000ull), bad);
}

// Sums with a zero addend, decided on the integer pipe: a + z for z = +-0
// (sign bit zs) is a itself for a nonzero, non-NaN a, and for a zero a the
// zero that is negative only when both are (round to nearest).  ok is false
// for a NaN a (the hardware's NaN result is used then).
EMU_HD double emu_add_zero(double a, uint64_t zs, bool& ok) {
  const uint64_t ua = emu_bits(a);
  ok = (ua << 1) <= 0xffe0000000000000ull;  // not NaN
  return (ua << 1) != 0 ? a : emu_double((ua & (zs << 63)) & 0x8000000000000000ull);
}
EMU_HD bool emu_is_zero(double x) { return (emu_bits(x) << 1) == 0; }
EMU_HD uint64_t emu_sign(double x) { return emu_bits(x) >> 63; }
// a finite, non-negative factor (sign 0, exponent below 2047): its product with
// a zero is the zero of the other factor's sign
EMU_HD bool emu_nonneg_finite(double x) { return emu_bits(x) < 0x7ff0000000000000ull; }

// IEEE comparisons decided from the bits on the integer pipe (an FP64
// compare occupies the FP64 pipe like an add).  NaN compares false; -0 and +0
// compare equal.
EMU_HD bool emu_gt0(double x) {  // x > 0
  const uint64_t b = emu_bits(x);
  return (int64_t)b > 0 && b <= 0x7ff0000000000000ull;
}
EMU_HD bool emu_lt0(double x) {  // x < 0
  const uint64_t b = emu_bits(x);
  return b > 0x8000000000000000ull && b <= 0xfff0000000000000ull;
}
EMU_HD bool emu_ge0(double x) { return !emu_lt0(x) && (emu_bits(x) << 1) <= 0xffe0000000000000ull; }  // x >= 0
EMU_HD bool emu_le0(double x) { return !emu_gt0(x) && (emu_bits(x) << 1) <= 0xffe0000000000000ull; }  // x <= 0
// order key: monotone in the value, equal for -0 and +0 (caller excludes NaN)
EMU_HD uint64_t emu_key(double x) {
  uint64_t b = emu_bits(x);
  if ((b << 1) == 0) b = 0;
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
EMU_HD bool emu_isnan(double x) { return (emu_bits(x) << 1) > 0xffe0000000000000ull; }
EMU_HD bool emu_lt(double a, double b) { return !emu_isnan(a) && !emu_isnan(b) && emu_key(a) < emu_key(b); }
EMU_HD bool emu_le(double a, double b) { return !emu_isnan(a) && !emu_isnan(b) && emu_key(a) <= emu_key(b); }
// a > b and a >= b for a, b that are +0, positive or NaN (sums of squares)
EMU_HD bool emu_gt_nonneg(double a, double b) {
  const uint64_t ua = emu_bits(a), ub = emu_bits(b);
  return ua > ub && ua <= 0x7ff0000000000000ull;
}
EMU_HD bool emu_ge_nonneg(double a, double b) {
  const uint64_t ua = emu_bits(a), ub = emu_bits(b);
  return ua >= ub && ua <= 0x7ff0000000000000ull && ub <= 0x7ff0000000000000ull;
}

}  // namespace dem
