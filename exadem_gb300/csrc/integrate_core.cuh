// integrate_core.cuh -- per-particle bodies of the Verlet prolog and epilog,
// shared by the operator kernels (k_particles.cu) and the fused step kernels
// (k_step_fused.cu) so both keep the same FP64 operation order.
//   prolog: combined_compute_prolog.cu:94-116 with PushVec3SecondOrder /
//           PushVec3FirstOrder (exaNBody) and PushToQuaternionFunctor
//           (push_to_quaternion.hpp:26-38);
//   epilog: combined_compute_epilog.cu:94-113 with angular_acceleration.hpp:27-43,
//           angular_velocity.hpp:27-33.
// Quaternion arithmetic restates onika's operators following exaDEM's quat type
// (src/shape/include/exaDEM/type/quat.hpp:79-96,233-242).
//
// Multiply placement (Mode, fused kernels only).  Every multiply below goes
// through a policy: MulFP64 is the FP64 pipe, MulInt the integer-pipe IEEE
// multiply of emu64.cuh.  Both return the same bits, so the mode changes only
// which pipe does the work.  Mode bit 0 places the rotation multiplies
// (quaternion rotations, quaternion derivative, normalisation, Euler terms),
// bit 1 the rest (Verlet pushes, gravity, quotient estimates).  Additions,
// the FMAs of div_rn, the square root and the division stay on the FP64 pipe,
// so with both bits set the two pipes share the work roughly evenly.
#pragma once
#include "dem_ctx.cuh"
#include "emu64.cuh"
#include "math_exact.cuh"
#include "mul_policy.cuh"

namespace dem {

// div_rn (math_exact.cuh) with its quotient estimate a*y through M
template <class M>
__device__ __forceinline__ double div_rn_m(M& mm, double a, double b, double y) {
  // a == 0, decided on the integer pipe; a * y is a itself for y >= +0 finite
  if ((emu_bits(a) << 1) == 0) return emu_nonneg_finite(y) ? a : mm.mul(a, y);
  if (exp_in_safe_range(a) && exp_in_safe_range(b)) {
    const double q = mm.mul(a, y);
    const double r = fma(-q, b, a);
    return fma(r, y, q);
  }
  return a / b;
}

struct Q4 {
  double w, x, y, z;
};
__device__ __forceinline__ V3 qrotate(Q4 q, V3 v) {
  const V3 qv = mk(q.x, q.y, q.z);
  V3 uv = cross(qv, v);
  V3 uuv = cross(qv, uv);
  uv = uv * (2.0 * q.w);
  uuv = uuv * 2.0;
  return v + uv + uuv;
}

// v rotated by q (q v q*), in the form v + 2w (u x v) + 2 u x (u x v), the
// operation order of qrotate, multiplies through M
template <class M>
__device__ __forceinline__ V3 qrotate_m(M& mm, Q4 q, V3 v) {
  V3 uv = mk(mm.mul(q.y, v.z) - mm.mul(q.z, v.y), mm.mul(q.z, v.x) - mm.mul(q.x, v.z),
             mm.mul(q.x, v.y) - mm.mul(q.y, v.x));
  V3 uuv = mk(mm.mul(q.y, uv.z) - mm.mul(q.z, uv.y), mm.mul(q.z, uv.x) - mm.mul(q.x, uv.z),
              mm.mul(q.x, uv.y) - mm.mul(q.y, uv.x));
  const double w2 = mm.twice(q.w);
  uv = mk(mm.mul(uv.x, w2), mm.mul(uv.y, w2), mm.mul(uv.z, w2));
  uuv = mk(mm.twice(uuv.x), mm.twice(uuv.y), mm.twice(uuv.z));
  return mk(v.x + uv.x + uuv.x, v.y + uv.y + uuv.y, v.z + uv.z + uuv.z);
}

// x += v dt + a dt^2/2; v += a dt/2; Q <- normalize(Q + dot(Q, w) dt); w += dt/2 arot
struct ProlState {
  V3 r, v, a, w, arot;
  Q4 q;
};
// Quaternion step of a particle without spin (w = +0,+0,+0), finite Q and
// 0 < dt < inf: every product w_k Q_l is a zero with the sign of Q_l, so the
// derivative d is a signed zero whose sign follows from the signs of Q
// (round to nearest: a sum of zeros is -0 only when every term is -0; a - b
// adds -b); Q + d dt keeps every nonzero component and gives a zero component
// the sign (sign(Q_c) and sign(d_c)).  spin_free_quaternion computes exactly
// that with integer sign logic instead of the 24 FP64 operations.
__device__ __forceinline__ bool spin_free_step(const Q4& Q, V3 om, double delta_t) {
  const uint64_t ew = emu_bits(Q.w) >> 52 & 0x7ffu, ex = emu_bits(Q.x) >> 52 & 0x7ffu,
                 ey = emu_bits(Q.y) >> 52 & 0x7ffu, ez = emu_bits(Q.z) >> 52 & 0x7ffu;
  return (emu_bits(om.x) | emu_bits(om.y) | emu_bits(om.z)) == 0 && ew != 0x7ffu && ex != 0x7ffu &&
         ey != 0x7ffu && ez != 0x7ffu && (emu_bits(delta_t) - 1u) < 0x7fefffffffffffffull;
}
__device__ __forceinline__ Q4 spin_free_quaternion(const Q4& Q) {
  const uint64_t bw = emu_bits(Q.w), bx = emu_bits(Q.x), by = emu_bits(Q.y), bz = emu_bits(Q.z);
  const uint64_t sw = bw >> 63, sx = bx >> 63, sy = by >> 63, sz = bz >> 63;
  const uint64_t dx = sz & (sy ^ 1u) & sw;  // sign of d.x = half((w_y Q_z - w_z Q_y) + w_x Q_w)
  const uint64_t dy = sx & (sz ^ 1u) & sw;
  const uint64_t dz = sy & (sx ^ 1u) & sw;
  const uint64_t dw = (sx & sy & sz) ^ 1u;  // -half(...) flips the sign
  auto step = [](uint64_t b, uint64_t s, uint64_t sd) {
    return (b << 1) == 0 ? emu_double((s & sd) << 63) : emu_double(b);
  };
  return Q4{step(bw, sw, dw), step(bx, sx, dx), step(by, sy, dy), step(bz, sz, dz)};
}

// The rotational half of the prolog: Q <- normalize(Q + dot(Q, w) dt) and
// w += dt/2 arot.  spin_free: the caller has checked spin_free_step, and the
// signed-zero derivative replaces the 24 FP64 operations.
template <class R, class L, bool Shortcuts>
__device__ __forceinline__ void quat_math(R& rm, L& lm, Q4& Q, V3& w, V3 arot, bool spin_free, double delta_t,
                                          double half_delta_t) {
  const V3 om = w;
  bool still = false;  // spin-free with arot = +0: w = +0 + (dt/2)(+0) stays +0
  if (Shortcuts && spin_free) {
    Q = spin_free_quaternion(Q);
    still = (emu_bits(arot.x) | emu_bits(arot.y) | emu_bits(arot.z)) == 0;
  } else {
    Q4 d;
    d.x = rm.half(rm.mul(om.y, Q.z) - rm.mul(om.z, Q.y) + rm.mul(om.x, Q.w));
    d.y = rm.half(rm.mul(om.z, Q.x) - rm.mul(om.x, Q.z) + rm.mul(om.y, Q.w));
    d.z = rm.half(rm.mul(om.x, Q.y) - rm.mul(om.y, Q.x) + rm.mul(om.z, Q.w));
    d.w = rm.neghalf(rm.mul(om.x, Q.x) + rm.mul(om.y, Q.y) + rm.mul(om.z, Q.z));
    Q.w = Q.w + rm.mul(d.w, delta_t);
    Q.x = Q.x + rm.mul(d.x, delta_t);
    Q.y = Q.y + rm.mul(d.y, delta_t);
    Q.z = Q.z + rm.mul(d.z, delta_t);
  }
  const double norm2 = rm.mul(Q.w, Q.w) + (rm.mul(Q.x, Q.x) + rm.mul(Q.y, Q.y) + rm.mul(Q.z, Q.z));
  // Shortcuts compare on the integer pipe: norm2 is +0, positive or NaN, so
  // its bits order like its value (NaN above every number)
  const uint64_t nb = emu_bits(norm2);
  if (Shortcuts ? nb <= 0x3e112e0be826d695ull /* bits of 1e-9 */ : norm2 <= 1e-9) {
    Q = {1.0, 0.0, 0.0, 0.0};
  } else if (!(Shortcuts && nb == 0x3ff0000000000000ull)) {  // norm2 == 1: 1/sqrt(1) = 1 and Q * 1 = Q exactly
    const double inv = 1.0 / sqrt(norm2);
    Q = {rm.mul(Q.w, inv), rm.mul(Q.x, inv), rm.mul(Q.y, inv), rm.mul(Q.z, inv)};
  }
  if (!still)  // (spin_free_step checked 0 < dt < inf, so (dt/2) * +0 = +0)
    w = mk(om.x + lm.mul(half_delta_t, arot.x), om.y + lm.mul(half_delta_t, arot.y),
           om.z + lm.mul(half_delta_t, arot.z));
}

// The translational half: x += v dt + a dt^2/2; v += a dt/2
template <class L>
__device__ __forceinline__ void transl_math(L& lm, V3& r, V3& v, V3 a, double delta_t, double half_delta_t,
                                            double delta_t2_2) {
  r = mk(r.x + (lm.mul(v.x, delta_t) + lm.mul(a.x, delta_t2_2)), r.y + (lm.mul(v.y, delta_t) + lm.mul(a.y, delta_t2_2)),
         r.z + (lm.mul(v.z, delta_t) + lm.mul(a.z, delta_t2_2)));
  v = mk(v.x + lm.mul(a.x, half_delta_t), v.y + lm.mul(a.y, half_delta_t), v.z + lm.mul(a.z, half_delta_t));
}

// One component of transl_math for the fused kernels.  With v = +-0 and a = +-0
// (and finite non-negative steps: zok) every product is the zero of the
// factor's sign, v dt + a dt^2/2 and v + a dt/2 are the zero that is negative
// only when both are, and r + that zero is r (emu_add_zero): decided on the
// integer pipe.  A particle at rest along an axis (free fall under a gravity
// along z) skips those FP64 operations.
template <class L>
__device__ __forceinline__ void transl_comp_z(L& lm, double& r, double& v, double a, double delta_t,
                                              double half_delta_t, double delta_t2_2, bool zok) {
  if (zok && emu_is_zero(v) && emu_is_zero(a)) {
    const uint64_t sp = emu_sign(v) & emu_sign(a);
    bool ok;
    const double rz = emu_add_zero(r, sp, ok);
    if (ok) {
      r = rz;
      v = emu_double(sp << 63);
      return;
    }
  }
  r = r + (lm.mul(v, delta_t) + lm.mul(a, delta_t2_2));
  v = v + lm.mul(a, half_delta_t);
}
template <class L>
__device__ __forceinline__ void transl_math_z(L& lm, V3& r, V3& v, V3 a, double delta_t, double half_delta_t,
                                              double delta_t2_2) {
  const bool zok = emu_nonneg_finite(delta_t) && emu_nonneg_finite(half_delta_t) && emu_nonneg_finite(delta_t2_2);
  transl_comp_z(lm, r.x, v.x, a.x, delta_t, half_delta_t, delta_t2_2, zok);
  transl_comp_z(lm, r.y, v.y, a.y, delta_t, half_delta_t, delta_t2_2, zok);
  transl_comp_z(lm, r.z, v.z, a.z, delta_t, half_delta_t, delta_t2_2, zok);
}

template <class R, class L, bool Shortcuts = false>
__device__ __forceinline__ ProlState prolog_math(R& rm, L& lm, const ProlState& in, double delta_t,
                                                 double half_delta_t, double delta_t2_2) {
  ProlState o = in;
  if (Shortcuts)
    transl_math_z(lm, o.r, o.v, in.a, delta_t, half_delta_t, delta_t2_2);
  else
    transl_math(lm, o.r, o.v, in.a, delta_t, half_delta_t, delta_t2_2);
  quat_math<R, L, Shortcuts>(rm, lm, o.q, o.w, in.arot, Shortcuts && spin_free_step(in.q, in.w, delta_t), delta_t,
                             half_delta_t);
  return o;
}

// Split form of the fused sphere prolog.  prolog_cheap: the translation and,
// for a spin-free particle, its rotational half; returns true when the
// particle spins (its rotational half is left to prolog_rotation).  The two
// halves read disjoint inputs and write disjoint outputs, so running them in
// separate launches gives the same bits as prolog_math.
template <int Mode>
__device__ __forceinline__ bool prolog_cheap(const PArrays& P, uint64_t s, double delta_t, double half_delta_t,
                                             double delta_t2_2) {
  const Q4 q0 = {P.f[QW][s], P.f[QX][s], P.f[QY][s], P.f[QZ][s]};
  const V3 w0 = mk(P.f[WX][s], P.f[WY][s], P.f[WZ][s]);
  const bool spin_free = spin_free_step(q0, w0, delta_t);
  auto run = [&](auto& rm, auto& lm, V3& r, V3& v, Q4& q, V3& w) {
    r = mk(P.f[RX][s], P.f[RY][s], P.f[RZ][s]);
    v = mk(P.f[VX][s], P.f[VY][s], P.f[VZ][s]);
    transl_math_z(lm, r, v, mk(P.f[FX][s], P.f[FY][s], P.f[FZ][s]), delta_t, half_delta_t, delta_t2_2);
    q = {P.f[QW][s], P.f[QX][s], P.f[QY][s], P.f[QZ][s]};
    w = mk(P.f[WX][s], P.f[WY][s], P.f[WZ][s]);
    if (spin_free)
      quat_math<std::remove_reference_t<decltype(rm)>, std::remove_reference_t<decltype(lm)>, true>(
          rm, lm, q, w, mk(P.f[AX][s], P.f[AY][s], P.f[AZ][s]), true, delta_t, half_delta_t);
  };
  RotMul<Mode> rm;
  LinMul<Mode> lm;
  V3 r, v, w;
  Q4 q;
  run(rm, lm, r, v, q, w);
  if (rm.failed() || lm.failed()) {
    asm volatile("" ::: "memory");  // nothing is stored yet: reload
    MulFP64 n;
    run(n, n, r, v, q, w);
  }
  P.f[RX][s] = r.x;
  P.f[RY][s] = r.y;
  P.f[RZ][s] = r.z;
  P.f[VX][s] = v.x;
  P.f[VY][s] = v.y;
  P.f[VZ][s] = v.z;
  if (spin_free) {
    P.f[QW][s] = q.w;
    P.f[QX][s] = q.x;
    P.f[QY][s] = q.y;
    P.f[QZ][s] = q.z;
    P.f[WX][s] = w.x;
    P.f[WY][s] = w.y;
    P.f[WZ][s] = w.z;
  }
  return !spin_free;
}

template <int Mode>
__device__ __forceinline__ void prolog_rotation(const PArrays& P, uint64_t s, double delta_t, double half_delta_t) {
  auto run = [&](auto& rm, auto& lm, Q4& q, V3& w) {
    q = {P.f[QW][s], P.f[QX][s], P.f[QY][s], P.f[QZ][s]};
    w = mk(P.f[WX][s], P.f[WY][s], P.f[WZ][s]);
    quat_math<std::remove_reference_t<decltype(rm)>, std::remove_reference_t<decltype(lm)>, true>(
        rm, lm, q, w, mk(P.f[AX][s], P.f[AY][s], P.f[AZ][s]), false, delta_t, half_delta_t);
  };
  RotMul<Mode> rm;
  LinMul<Mode> lm;
  Q4 q;
  V3 w;
  run(rm, lm, q, w);
  if (rm.failed() || lm.failed()) {
    asm volatile("" ::: "memory");
    MulFP64 n;
    run(n, n, q, w);
  }
  P.f[QW][s] = q.w;
  P.f[QX][s] = q.x;
  P.f[QY][s] = q.y;
  P.f[QZ][s] = q.z;
  P.f[WX][s] = w.x;
  P.f[WY][s] = w.y;
  P.f[WZ][s] = w.z;
}

// Fused = true (the fused prolog kernels) takes the exact spin-free and unit
// norm shortcuts of prolog_math; the operator kernel runs the plain formula.
template <int Mode = 0, bool Fused = false>
__device__ __forceinline__ void prolog_one(const PArrays& P, uint64_t s, double delta_t, double half_delta_t,
                                           double delta_t2_2) {
  auto load = [&]() {
    ProlState in;
    in.r = mk(P.f[RX][s], P.f[RY][s], P.f[RZ][s]);
    in.v = mk(P.f[VX][s], P.f[VY][s], P.f[VZ][s]);
    in.a = mk(P.f[FX][s], P.f[FY][s], P.f[FZ][s]);
    in.q = {P.f[QW][s], P.f[QX][s], P.f[QY][s], P.f[QZ][s]};
    in.w = mk(P.f[WX][s], P.f[WY][s], P.f[WZ][s]);
    in.arot = mk(P.f[AX][s], P.f[AY][s], P.f[AZ][s]);
    return in;
  };
  RotMul<Mode> rm;
  LinMul<Mode> lm;
  ProlState o = prolog_math<RotMul<Mode>, LinMul<Mode>, Fused>(rm, lm, load(), delta_t, half_delta_t, delta_t2_2);
  if (rm.failed() || lm.failed()) {
    // nothing is stored yet: reload the inputs (the barrier keeps the main
    // path from holding them in registers for this rare case)
    asm volatile("" ::: "memory");
    MulFP64 n;
    o = prolog_math<MulFP64, MulFP64, Fused>(n, n, load(), delta_t, half_delta_t, delta_t2_2);
  }
  P.f[RX][s] = o.r.x;
  P.f[RY][s] = o.r.y;
  P.f[RZ][s] = o.r.z;
  P.f[VX][s] = o.v.x;
  P.f[VY][s] = o.v.y;
  P.f[VZ][s] = o.v.z;
  P.f[QW][s] = o.q.w;
  P.f[QX][s] = o.q.x;
  P.f[QY][s] = o.q.y;
  P.f[QZ][s] = o.q.z;
  P.f[WX][s] = o.w.x;
  P.f[WY][s] = o.w.y;
  P.f[WZ][s] = o.w.z;
}

// arot from the torque (Euler equations in the body frame), w += arot dt/2, v += a dt/2.
// a is the acceleration (f after force_to_accel).  FastDiv: divisions by the
// inertia through the precomputed reciprocals (div_rn, exact).
struct EpiOut {
  V3 arot, w, v;
};
template <bool FastDiv, class R, class L>
__device__ __forceinline__ EpiOut epilog_math(R& rm, L& lm, Q4 Q, V3 vrot, V3 I, V3 II, V3 vel, V3 a, V3 mom,
                                              double half_delta_t) {
  const Q4 Qinv = {Q.w, -Q.x, -Q.y, -Q.z};
  const V3 omega = qrotate_m(rm, Qinv, vrot);
  const V3 M = qrotate_m(rm, Qinv, mom);
  const double nx = M.x - rm.mul(rm.mul(I.z - I.y, omega.y), omega.z);
  const double ny = M.y - rm.mul(rm.mul(I.x - I.z, omega.z), omega.x);
  const double nz = M.z - rm.mul(rm.mul(I.y - I.x, omega.x), omega.y);
  V3 domega;
  if (FastDiv) {
    domega = mk(div_rn_m(lm, nx, I.x, II.x), div_rn_m(lm, ny, I.y, II.y), div_rn_m(lm, nz, I.z, II.z));
  } else {
    domega = mk(nx / I.x, ny / I.y, nz / I.z);
  }
  EpiOut o;
  o.arot = qrotate_m(rm, Q, domega);
  o.w = mk(vrot.x + lm.mul(o.arot.x, half_delta_t), vrot.y + lm.mul(o.arot.y, half_delta_t),
           vrot.z + lm.mul(o.arot.z, half_delta_t));
  o.v = mk(vel.x + lm.mul(a.x, half_delta_t), vel.y + lm.mul(a.y, half_delta_t), vel.z + lm.mul(a.z, half_delta_t));
  return o;
}

// A particle whose spin and torque are all +0.0 keeps arot = +0 and w = +0
// bit for bit, provided the quaternion is finite and the inertia and its
// reciprocal are positive and finite: every product of a quaternion or inertia
// component with +0 is +-0; a sum whose first operand is +0 and whose other
// operands are +-0 is +0 (round to nearest: -0 only for (-0) + (-0)); so
// omega = qrotate(Q^-1, +0) = +0 and M = +0, the Euler numerators are
// +0 - (+-0) = +0, div_rn(+0, I, 1/I) = +0 * (1/I) = +0, arot = qrotate(Q, +0)
// = +0 and w = +0 + (+0 * dt/2) = +0.
__device__ __forceinline__ bool finite_bits(double x) { return ((emu_bits(x) >> 52) & 0x7ffu) != 0x7ffu; }
__device__ __forceinline__ bool positive_finite_bits(double x) { return (emu_bits(x) >> 52) < 0x7ffu; }
__device__ __forceinline__ bool rotation_idle(Q4 Q, V3 vrot, V3 mom, V3 I, V3 II) {
  const uint64_t z = emu_bits(vrot.x) | emu_bits(vrot.y) | emu_bits(vrot.z) | emu_bits(mom.x) | emu_bits(mom.y) |
                     emu_bits(mom.z);
  return z == 0 && finite_bits(Q.w) && finite_bits(Q.x) && finite_bits(Q.y) && finite_bits(Q.z) &&
         positive_finite_bits(I.x) && positive_finite_bits(I.y) && positive_finite_bits(I.z) &&
         positive_finite_bits(II.x) && positive_finite_bits(II.y) && positive_finite_bits(II.z);
}

template <bool FastDiv>
__device__ __forceinline__ void epilog_one(const PArrays& P, uint64_t s, double half_delta_t, V3 a, V3 mom) {
  MulFP64 rm, lm;
  const Q4 Q = {P.f[QW][s], P.f[QX][s], P.f[QY][s], P.f[QZ][s]};
  const V3 vrot = mk(P.f[WX][s], P.f[WY][s], P.f[WZ][s]);
  const V3 I = mk(P.f[IX][s], P.f[IY][s], P.f[IZ][s]);
  const V3 II = FastDiv ? mk(P.f[IIX][s], P.f[IIY][s], P.f[IIZ][s]) : mk(0.0, 0.0, 0.0);
  const V3 vel = mk(P.f[VX][s], P.f[VY][s], P.f[VZ][s]);
  const EpiOut o = epilog_math<FastDiv>(rm, lm, Q, vrot, I, II, vel, a, mom, half_delta_t);
  P.f[AX][s] = o.arot.x;
  P.f[AY][s] = o.arot.y;
  P.f[AZ][s] = o.arot.z;
  P.f[WX][s] = o.w.x;
  P.f[WY][s] = o.w.y;
  P.f[WZ][s] = o.w.z;
  P.f[VX][s] = o.v.x;
  P.f[VY][s] = o.v.y;
  P.f[VZ][s] = o.v.z;
}

// The rotational half of the fused epilog (arot and w from the torque stored
// in mom; the velocity update is done by the caller), the operation order of
// epilog_math.  An integer-pipe multiply that leaves its fast path makes the
// whole half run again on the FP64 pipe from the stored inputs.
template <int Mode>
__device__ __forceinline__ void epilog_rotation(const PArrays& P, uint64_t s, double half_delta_t, V3 mom) {
  auto run = [&](auto& rm, auto& lm, V3 tq, V3& arot, V3& w) {
    const Q4 Q = {P.f[QW][s], P.f[QX][s], P.f[QY][s], P.f[QZ][s]};
    const V3 vrot = mk(P.f[WX][s], P.f[WY][s], P.f[WZ][s]);
    const V3 I = mk(P.f[IX][s], P.f[IY][s], P.f[IZ][s]);
    const V3 II = mk(P.f[IIX][s], P.f[IIY][s], P.f[IIZ][s]);
    const Q4 Qinv = {Q.w, -Q.x, -Q.y, -Q.z};
    const V3 omega = qrotate_m(rm, Qinv, vrot);
    const V3 M = qrotate_m(rm, Qinv, tq);
    const double nx = M.x - rm.mul(rm.mul(I.z - I.y, omega.y), omega.z);
    const double ny = M.y - rm.mul(rm.mul(I.x - I.z, omega.z), omega.x);
    const double nz = M.z - rm.mul(rm.mul(I.y - I.x, omega.x), omega.y);
    const V3 domega = mk(div_rn_m(lm, nx, I.x, II.x), div_rn_m(lm, ny, I.y, II.y), div_rn_m(lm, nz, I.z, II.z));
    arot = qrotate_m(rm, Q, domega);
    w = mk(vrot.x + lm.mul(arot.x, half_delta_t), vrot.y + lm.mul(arot.y, half_delta_t),
           vrot.z + lm.mul(arot.z, half_delta_t));
  };
  RotMul<Mode> rm;
  LinMul<Mode> lm;
  V3 arot, w;
  run(rm, lm, mom, arot, w);
  if (rm.failed() || lm.failed()) {
    asm volatile("" ::: "memory");  // reload the inputs, nothing is stored yet
    MulFP64 n;
    run(n, n, mk(P.f[MX][s], P.f[MY][s], P.f[MZ][s]), arot, w);
  }
  P.f[AX][s] = arot.x;
  P.f[AY][s] = arot.y;
  P.f[AZ][s] = arot.z;
  P.f[WX][s] = w.x;
  P.f[WY][s] = w.y;
  P.f[WZ][s] = w.z;
}

}  // namespace dem
