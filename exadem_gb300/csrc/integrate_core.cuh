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
#pragma once
#include "dem_ctx.cuh"
#include "math_exact.cuh"

namespace dem {

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

// x += v dt + a dt^2/2; v += a dt/2; Q <- normalize(Q + dot(Q, w) dt); w += dt/2 arot
__device__ __forceinline__ void prolog_one(const PArrays& P, uint64_t s, double delta_t, double half_delta_t,
                                           double delta_t2_2) {
#pragma unroll
  for (int d = 0; d < 3; d++) {
    const double v = P.f[VX + d][s], a = P.f[FX + d][s];
    P.f[RX + d][s] = P.f[RX + d][s] + (v * delta_t + a * delta_t2_2);
    P.f[VX + d][s] = v + a * half_delta_t;
  }
  Q4 Q = {P.f[QW][s], P.f[QX][s], P.f[QY][s], P.f[QZ][s]};
  const V3 om = mk(P.f[WX][s], P.f[WY][s], P.f[WZ][s]);
  Q4 d;
  d.x = 0.5 * (om.y * Q.z - om.z * Q.y + om.x * Q.w);
  d.y = 0.5 * (om.z * Q.x - om.x * Q.z + om.y * Q.w);
  d.z = 0.5 * (om.x * Q.y - om.y * Q.x + om.z * Q.w);
  d.w = -0.5 * (om.x * Q.x + om.y * Q.y + om.z * Q.z);
  Q.w = Q.w + d.w * delta_t;
  Q.x = Q.x + d.x * delta_t;
  Q.y = Q.y + d.y * delta_t;
  Q.z = Q.z + d.z * delta_t;
  const double norm2 = Q.w * Q.w + (Q.x * Q.x + Q.y * Q.y + Q.z * Q.z);
  if (norm2 <= 1e-9) {
    Q = {1.0, 0.0, 0.0, 0.0};
  } else {
    const double inv = 1.0 / sqrt(norm2);
    Q = {Q.w * inv, Q.x * inv, Q.y * inv, Q.z * inv};
  }
  P.f[QW][s] = Q.w;
  P.f[QX][s] = Q.x;
  P.f[QY][s] = Q.y;
  P.f[QZ][s] = Q.z;
  P.f[WX][s] = om.x + half_delta_t * P.f[AX][s];
  P.f[WY][s] = om.y + half_delta_t * P.f[AY][s];
  P.f[WZ][s] = om.z + half_delta_t * P.f[AZ][s];
}

// arot from the torque (Euler equations in the body frame), w += arot dt/2, v += a dt/2.
// a is the acceleration (f after force_to_accel).  FastDiv: divisions by the
// inertia through the precomputed reciprocals (div_rn, exact).
template <bool FastDiv>
__device__ __forceinline__ void epilog_one(const PArrays& P, uint64_t s, double half_delta_t, V3 a, V3 mom) {
  const Q4 Q = {P.f[QW][s], P.f[QX][s], P.f[QY][s], P.f[QZ][s]};
  const Q4 Qinv = {Q.w, -Q.x, -Q.y, -Q.z};
  const V3 vrot = mk(P.f[WX][s], P.f[WY][s], P.f[WZ][s]);
  const V3 I = mk(P.f[IX][s], P.f[IY][s], P.f[IZ][s]);
  const V3 omega = qrotate(Qinv, vrot);
  const V3 M = qrotate(Qinv, mom);
  const double nx = M.x - (I.z - I.y) * omega.y * omega.z;
  const double ny = M.y - (I.x - I.z) * omega.z * omega.x;
  const double nz = M.z - (I.y - I.x) * omega.x * omega.y;
  V3 domega;
  if (FastDiv) {
    domega = mk(div_rn(nx, I.x, P.f[IIX][s]), div_rn(ny, I.y, P.f[IIY][s]), div_rn(nz, I.z, P.f[IIZ][s]));
  } else {
    domega = mk(nx / I.x, ny / I.y, nz / I.z);
  }
  const V3 arot = qrotate(Q, domega);
  P.f[AX][s] = arot.x;
  P.f[AY][s] = arot.y;
  P.f[AZ][s] = arot.z;
  P.f[WX][s] = vrot.x + arot.x * half_delta_t;
  P.f[WY][s] = vrot.y + arot.y * half_delta_t;
  P.f[WZ][s] = vrot.z + arot.z * half_delta_t;
  P.f[VX][s] = P.f[VX][s] + a.x * half_delta_t;
  P.f[VY][s] = P.f[VY][s] + a.y * half_delta_t;
  P.f[VZ][s] = P.f[VZ][s] + a.z * half_delta_t;
}

}  // namespace dem
