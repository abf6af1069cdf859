// Stand-in for onika's vector and quaternion types (host only).
//
// Vec3d operators are component-wise (Vec3d * Vec3d too); dot sums x, y, z left to right; norm is
// sqrt(dot(v, v)).  The quaternion rotation, time derivative and normalisation
// use the formulas of exaDEM's own quat type
// (src/shape/include/exaDEM/type/quat.hpp, operator*(vec3r), dot(omega),
// normalize()).  These formulas are the part of the comparison that exaDEM's
// sources do not pin (onika is not vendored).
#pragma once
#include <cmath>
#include <ostream>
#include <onika/cuda/cuda.h>
#include <onika/memory/allocator.h>

namespace onika {
namespace math {
struct Vec3d {
  double x, y, z;
  Vec3d() = default;
  constexpr Vec3d(double a, double b, double c) : x(a), y(b), z(c) {}
};
inline Vec3d operator+(const Vec3d& a, const Vec3d& b) { return Vec3d(a.x + b.x, a.y + b.y, a.z + b.z); }
inline Vec3d operator-(const Vec3d& a, const Vec3d& b) { return Vec3d(a.x - b.x, a.y - b.y, a.z - b.z); }
inline Vec3d operator-(const Vec3d& a) { return Vec3d(-a.x, -a.y, -a.z); }
inline Vec3d operator*(const Vec3d& a, double s) { return Vec3d(a.x * s, a.y * s, a.z * s); }
inline Vec3d operator*(double s, const Vec3d& a) { return Vec3d(s * a.x, s * a.y, s * a.z); }
inline Vec3d operator*(const Vec3d& a, const Vec3d& b) { return Vec3d(a.x * b.x, a.y * b.y, a.z * b.z); }
inline Vec3d operator/(const Vec3d& a, double s) { return Vec3d(a.x / s, a.y / s, a.z / s); }
inline Vec3d& operator+=(Vec3d& a, const Vec3d& b) { a.x += b.x; a.y += b.y; a.z += b.z; return a; }
inline Vec3d& operator-=(Vec3d& a, const Vec3d& b) { a.x -= b.x; a.y -= b.y; a.z -= b.z; return a; }
inline Vec3d& operator*=(Vec3d& a, double s) { a.x *= s; a.y *= s; a.z *= s; return a; }
inline Vec3d& operator/=(Vec3d& a, double s) { a.x /= s; a.y /= s; a.z /= s; return a; }
inline bool operator==(const Vec3d& a, const Vec3d& b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
inline bool operator!=(const Vec3d& a, const Vec3d& b) { return !(a == b); }
inline double dot(const Vec3d& a, const Vec3d& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline Vec3d cross(const Vec3d& a, const Vec3d& b) {
  return Vec3d(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline double norm2(const Vec3d& a) { return dot(a, a); }
inline double norm(const Vec3d& a) { return std::sqrt(dot(a, a)); }

inline std::ostream& operator<<(std::ostream& o, const Vec3d& v) { return o << v.x << "," << v.y << "," << v.z; }

struct AABB {
  Vec3d bmin, bmax;
};

struct Quaternion {
  double w, x, y, z;
};
inline Quaternion operator+(const Quaternion& a, const Quaternion& b) {
  return Quaternion{a.w + b.w, a.x + b.x, a.y + b.y, a.z + b.z};
}
inline Quaternion operator*(const Quaternion& a, double s) { return Quaternion{a.w * s, a.x * s, a.y * s, a.z * s}; }
inline Quaternion operator*(double s, const Quaternion& a) { return Quaternion{s * a.w, s * a.x, s * a.y, s * a.z}; }
// Rotation of v by Q: v + 2w (q x v) + 2 q x (q x v), q the vector part.
inline Vec3d operator*(const Quaternion& Q, const Vec3d& v) {
  const Vec3d q(Q.x, Q.y, Q.z);
  Vec3d uv = cross(q, v);
  Vec3d uuv = cross(q, uv);
  uv *= (2.0 * Q.w);
  uuv *= 2.0;
  return v + uv + uuv;
}
inline Quaternion get_conjugated(const Quaternion& Q) { return Quaternion{Q.w, -Q.x, -Q.y, -Q.z}; }
// Time derivative of Q under the angular velocity om.
inline Quaternion dot(const Quaternion& Q, const Vec3d& om) {
  Quaternion r;
  r.x = 0.5 * (om.y * Q.z - om.z * Q.y + om.x * Q.w);
  r.y = 0.5 * (om.z * Q.x - om.x * Q.z + om.y * Q.w);
  r.z = 0.5 * (om.x * Q.y - om.y * Q.x + om.z * Q.w);
  r.w = -0.5 * (om.x * Q.x + om.y * Q.y + om.z * Q.z);
  return r;
}
inline Quaternion normalize(const Quaternion& Q) {
  const double n2 = Q.w * Q.w + (Q.x * Q.x + Q.y * Q.y + Q.z * Q.z);
  if (n2 <= 1e-9) return Quaternion{1.0, 0.0, 0.0, 0.0};
  const double inv = 1.0 / std::sqrt(n2);
  return Quaternion{Q.w * inv, Q.x * inv, Q.y * inv, Q.z * inv};
}
}  // namespace math
}  // namespace onika

namespace exanb {
using onika::math::AABB;
using onika::math::cross;
using onika::math::dot;
using onika::math::get_conjugated;
using onika::math::norm;
using onika::math::norm2;
using onika::math::normalize;
using onika::math::Quaternion;
using onika::math::Vec3d;
}  // namespace exanb
