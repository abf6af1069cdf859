// poly_f32.cuh -- FP32 decisions of the polyhedron broad-phase tests.
//
// Each function evaluates the same formula as its FP64 counterpart in
// poly_core.cuh (OBB::intersect, filter_vv/ve/vf/ee, which follow
// src/polyhedra/include/exaDEM/shape/shape_detection.hpp) in FP32, together
// with a first-order bound of the FP32 error, and returns
//   DEC_FALSE / DEC_TRUE  when every comparison of the formula is further from
//                         its threshold than 8x the error bound, so that the
//                         FP64 evaluation takes the same branch;
//   DEC_UNDECIDED         otherwise: the caller runs the FP64 function.
// The result of a decided test is therefore the FP64 result, bit for bit.
//
// Inputs: coordinates relative to the centre of the owner particle A, as FP32.
// With S a bound of every |coordinate| (S = |r_B - r_A| + both particles'
// max vertex radii and Minkowski radii + skin), each input coordinate carries
// an error of at most 3 u S (conversion of v - r, of r_B - r_A and their sum,
// u = 2^-24); vector differences of inputs therefore carry at most
// ETA = 2^-19 S (a factor 3 above 2 * sqrt(3) * 3 u S).
#pragma once
#include <cstdint>

#include "poly_core.cuh"

namespace dem {

struct F3 {
  float x, y, z;
};
__device__ __forceinline__ F3 f3(float x, float y, float z) { return F3{x, y, z}; }
__device__ __forceinline__ F3 operator+(F3 a, F3 b) { return F3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ F3 operator-(F3 a, F3 b) { return F3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ F3 operator*(F3 a, float s) { return F3{a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ float fdot(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float flen(F3 a) { return sqrtf(fdot(a, a)); }
__device__ __forceinline__ F3 fcross(F3 a, F3 b) {
  return F3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}

// FP32 vertices of one particle (relative to the centre of A) in SoA layout
struct FView {
  const float* x;
  const float* y;
  const float* z;
  F3 off;
  __device__ __forceinline__ F3 operator[](int k) const { return F3{x[k] + off.x, y[k] + off.y, z[k] + off.z}; }
};

struct OBBf {
  F3 c, e[3];
  float ext[3];
};

__device__ __forceinline__ OBBf obb_f32(const OBBd& o, V3 origin) {
  OBBf r;
  r.c = f3((float)(o.c.x - origin.x), (float)(o.c.y - origin.y), (float)(o.c.z - origin.z));
  r.e[0] = f3((float)o.e1.x, (float)o.e1.y, (float)o.e1.z);
  r.e[1] = f3((float)o.e2.x, (float)o.e2.y, (float)o.e2.z);
  r.e[2] = f3((float)o.e3.x, (float)o.e3.y, (float)o.e3.z);
  r.ext[0] = (float)o.ext.x;
  r.ext[1] = (float)o.ext.y;
  r.ext[2] = (float)o.ext.z;
  return r;
}

// Per-particle FP32 boxes written at a rebuild (floats, stride FBOX_STRIDE):
//   [0, 15)  gate OBB as OBBf (centre relative to the particle centre, axes, extents)
//   [15, 24) three unit slab directions d_k
//   [24, 27) slab centres c_k and [27, 30) half widths h_k: every vertex v of the
//            particle (relative to its centre) has |v.d_k - c_k| <= h_k
constexpr int FBOX_STRIDE = 32;

__device__ __forceinline__ void store_obbf(float* w, const OBBf& o) {
  w[0] = o.c.x;
  w[1] = o.c.y;
  w[2] = o.c.z;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    w[3 + 3 * k] = o.e[k].x;
    w[4 + 3 * k] = o.e[k].y;
    w[5 + 3 * k] = o.e[k].z;
    w[12 + k] = o.ext[k];
  }
}

__device__ __forceinline__ OBBf load_obbf(const float* w, F3 off) {
  OBBf o;
  o.c = f3(w[0], w[1], w[2]) + off;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    o.e[k] = f3(w[3 + 3 * k], w[4 + 3 * k], w[5 + 3 * k]);
    o.ext[k] = w[12 + k];
  }
  return o;
}

// Vertex slabs of a particle moved to another origin (off = centre - origin)
struct Slabs {
  F3 d[3];
  float c[3], h[3];
};

__device__ __forceinline__ Slabs load_slabs(const float* w, F3 off) {
  Slabs s;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    s.d[k] = f3(w[15 + 3 * k], w[16 + 3 * k], w[17 + 3 * k]);
    s.c[k] = w[24 + k] + fdot(off, s.d[k]);
    s.h[k] = w[27 + k];
  }
  return s;
}

// Necessary conditions for a feature to lie within distance lim of the other
// particle's vertex hull (which the slabs contain): false when some slab,
// widened by lim, misses the feature.  lim includes a margin m >= 2^-14 S, far
// above the FP32 error of the projections (about 2^-20 S).
__device__ __forceinline__ bool slab_near_point(const Slabs& s, F3 p, float lim) {
#pragma unroll
  for (int k = 0; k < 3; k++)
    if (fabsf(fdot(p, s.d[k]) - s.c[k]) > s.h[k] + lim) return false;
  return true;
}
// segment p0-p1 extended by ext * |p1 - p0| at both ends
__device__ __forceinline__ bool slab_near_segment(const Slabs& s, F3 p0, F3 p1, float ext, float lim) {
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const float a = fdot(p0, s.d[k]) - s.c[k], b = fdot(p1, s.d[k]) - s.c[k];
    const float x = ext * fabsf(b - a);
    if (fminf(a, b) - x > s.h[k] + lim || fmaxf(a, b) + x < -(s.h[k] + lim)) return false;
  }
  return true;
}
__device__ __forceinline__ bool slab_near_face(const Slabs& s, const FView& v, const ShapeDev& sh, int face,
                                               float lim) {
  const int b = sh.fo[face], nf = sh.fo[face + 1] - b;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    float lo = 3.4e38f, hi = -3.4e38f;
    for (int q = 0; q < nf; q++) {
      const float pr = fdot(v[sh.fv[b + q]], s.d[k]) - s.c[k];
      lo = fminf(lo, pr);
      hi = fmaxf(hi, pr);
    }
    if (lo > s.h[k] + lim || hi < -(s.h[k] + lim)) return false;
  }
  return true;
}

enum : int { DEC_FALSE = 0, DEC_TRUE = 1, DEC_UNDECIDED = 2 };

constexpr float F32_U = 5.9604645e-08f;  // 2^-24
constexpr float F32_ETA = 1.9073486e-06f;  // 2^-19: ETA / S
constexpr float F32_SAFE = 8.f;             // decided only beyond 8x the bound


// FP32 rotation by a quaternion (w, x, y, z), the formula of qrotate: v + 2w (u x v) + 2 u x (u x v)
__device__ __forceinline__ F3 qrotate_f32(float4 q, F3 v) {
  const F3 u = f3(q.y, q.z, q.w);
  F3 uv = fcross(u, v);
  F3 uuv = fcross(u, uv);
  uv = uv * (2.0f * q.x);
  uuv = uuv * 2.0f;
  return v + uv + uuv;
}

// vertex_displ_over for one vertex (backup_dem.hpp:65-110): over when
// |v - v_backup|^2 >= thr^2.  FP32 displacement (r - r_b) + (q v0' - q_b v0'),
// v0' = h v0; dp = FP32 rounding of r - r_b (FP64 difference), qn, qb = FP32
// roundings of the quaternions, q2 = max(1, |qn|^2, |qb|^2), pabs = |r|_1.
// Error bound E = 2u|dp| + 26u |v0'| q2 + 2u|d| + 2^-51 (pabs + |v0'|) + u thr
// (FP32 rounding of each term and of the quaternions, and the FP64 rounding of
// the reference's absolute vertices); decided beyond 8 E of thr.
__device__ __forceinline__ int decide_displ(F3 dp, float4 qn, float4 qb, F3 v0h, float q2, float pabs, float thr) {
  const float u = F32_U;
  const F3 d = dp + (qrotate_f32(qn, v0h) - qrotate_f32(qb, v0h));
  const float dl = flen(d), lv = flen(v0h);
  const float E = 2.f * u * flen(dp) + 26.f * u * lv * q2 + 2.f * u * dl + 4.440892e-16f * (pabs + lv) + u * thr;
  return dl > thr + F32_SAFE * E ? DEC_TRUE : (dl < thr - F32_SAFE * E ? DEC_FALSE : DEC_UNDECIDED);
}


// one comparison "x > thr" with error bound e: +1 surely greater, -1 surely not, 0 unknown
__device__ __forceinline__ int cmp_gt(float x, float thr, float e) {
  const float m = F32_SAFE * e;
  return x > thr + m ? 1 : (x < thr - m ? -1 : 0);
}

// Vertex gate: OBB::intersect(obb, box(p, rv)) with the box's axes the world axes.
// The FP64 test returns false at the first of 15 axes with |t_L| > ra_L + rb_L.
// Error of every axis test, with T = |c - p| + sum(ext) + rv + S:
// obb centre and extents are FP32 roundings of the FP64 values (u T), axes
// u per component, p carries ETA; every |t_L| and radius sum is a sum of at most
// 6 products of magnitude <= 2T with |factor| <= 1 + tol.  Bound: 2^-17 T.
// A cross axis A_k x W_l weighs t by the two entries R[k1][l], R[k2][l]: the
// error of its projection is at most (2^-17 T + 4u T)(|R[k1][l]| + |R[k2][l]|)
// (each t within 2^-17 T, each entry an FP32 rounding), that of its radius sum
// at most 8u of it.  When A_k is nearly a world axis (the covariance OBB of a
// cube is the world-aligned one) both entries vanish and this bound, far below
// 2^-17 T, still decides the axis.
__device__ __forceinline__ int decide_gate(const OBBf& o, F3 p, float rv, float S) {
  const float tol = 1.1920929e-07f;
  const F3 tt = o.c - p;
  const float T = flen(tt) + o.ext[0] + o.ext[1] + o.ext[2] + rv + S;
  const float e = 7.6293945e-06f * T;  // 2^-17 T
  // rows: A axes; B axes are the world axes, so R[k][l] = component l of e_k
  float R[3][3], Ab[3][3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    R[k][0] = o.e[k].x;
    R[k][1] = o.e[k].y;
    R[k][2] = o.e[k].z;
#pragma unroll
    for (int l = 0; l < 3; l++) Ab[k][l] = fabsf(R[k][l]) + tol;
  }
  const float t[3] = {fdot(tt, o.e[0]), fdot(tt, o.e[1]), fdot(tt, o.e[2])};
  // p inside the OBB (beyond the bound): the two boxes share p, so no axis
  // separates them (every projection of t stays below the OBB's radius on it)
  const float in = F32_SAFE * e;
  if (fabsf(t[0]) < o.ext[0] - in && fabsf(t[1]) < o.ext[1] - in && fabsf(t[2]) < o.ext[2] - in) return DEC_TRUE;
  bool undecided = false;
  // A's axes
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const int c = cmp_gt(fabsf(t[k]), o.ext[k] + rv * (Ab[k][0] + Ab[k][1] + Ab[k][2]), e);
    if (c > 0) return DEC_FALSE;
    undecided |= c == 0;
  }
  // B's (world) axes
#pragma unroll
  for (int l = 0; l < 3; l++) {
    const float ra = o.ext[0] * Ab[0][l] + o.ext[1] * Ab[1][l] + o.ext[2] * Ab[2][l];
    const int c = cmp_gt(fabsf(t[0] * R[0][l] + t[1] * R[1][l] + t[2] * R[2][l]), ra + rv, e);
    if (c > 0) return DEC_FALSE;
    undecided |= c == 0;
  }
  // cross axes A_k x B_l, with (k1, k2) the other two A axes
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const int k1 = (k + 1) % 3, k2 = (k + 2) % 3;
#pragma unroll
    for (int l = 0; l < 3; l++) {
      const int l1 = (l + 1) % 3, l2 = (l + 2) % 3;
      const float ra = o.ext[k1] * Ab[k2][l] + o.ext[k2] * Ab[k1][l];
      const float rb = rv * (Ab[k][l2] + Ab[k][l1]);
      const float lhs = fabsf(t[k2] * R[k1][l] - t[k1] * R[k2][l]), rhs = ra + rb;
      const float ex = (e + 4.f * F32_U * T) * (fabsf(R[k1][l]) + fabsf(R[k2][l])) + 8.f * F32_U * (lhs + rhs);
      const int c = cmp_gt(lhs, rhs, fminf(e, ex));
      if (c > 0) return DEC_FALSE;
      undecided |= c == 0;
    }
  }
  return undecided ? DEC_UNDECIDED : DEC_TRUE;
}

// filter_vv: |vi - vj|^2 <= R^2.  |d| carries 2 ETA + 4u|d|.
__device__ __forceinline__ int decide_vv(F3 vi, F3 vj, float R, float S) {
  const float d = flen(vi - vj);
  const int c = cmp_gt(d, R, 2.f * F32_ETA * S + 4.f * F32_U * (d + R));
  return c > 0 ? DEC_FALSE : (c < 0 ? DEC_TRUE : DEC_UNDECIDED);
}

// filter_ve: r = E.w / E.E in [-rV, 1 + rV] and |w - E r|^2 < R^2.
__device__ __forceinline__ int decide_ve(F3 vi, F3 vf, F3 vs, float R, float rV, float S) {
  const float eta = F32_ETA * S;
  const F3 E = vs - vf, w = vi - vf;
  const float L2 = fdot(E, E), L = sqrtf(L2), W = flen(w);
  if (!(L2 > 0.f)) return DEC_UNDECIDED;
  const float r = fdot(E, w) / L2;
  const float ar = fabsf(r);
  // |d(E.w)| <= eta (W + L) + 4u L W ; |d(E.E)| <= 2 eta L + 4u L^2 ; plus 2u |r| for the division
  const float er = (eta * (W + L) + 4.f * F32_U * L * W + ar * (2.f * eta * L + 4.f * F32_U * L2)) / L2 +
                   2.f * F32_U * ar;
  const int c0 = cmp_gt(-rV, r, er);  // r < -rV
  const int c1 = cmp_gt(r, 1.f + rV, er + F32_U * (1.f + rV));
  if (c0 > 0 || c1 > 0) return DEC_FALSE;
  if (c0 == 0 || c1 == 0) return DEC_UNDECIDED;
  const F3 dv = w - E * r;
  const float d = flen(dv);
  // |d(w - E r)| <= eta + eta |r| + L er + 4u (W + L |r|)
  const float ed = eta * (1.f + ar) + L * er + 4.f * F32_U * (W + L * ar) + 4.f * F32_U * (d + R);
  const int c = cmp_gt(d, R, ed);
  return c < 0 ? DEC_TRUE : (c > 0 ? DEC_FALSE : DEC_UNDECIDED);
}

// filter_vf (vf_core): vertex vi against face `face` of the shape with vertices vf.
// The frame (v1, n, v2 = n x v1) is built from the face's first, second and last
// vertices as in the FP64 code.  Decided when the plane distance and every
// comparison of the crossing-parity test are beyond their bounds.
// The face is given by its vertex count nf and V(k), its k-th vertex.
template <class VertF>
__device__ inline int decide_vf_list(F3 vi, int nf, VertF&& vtx, float lim, float S) {
  const float eta = F32_ETA * S;
  const F3 va = vtx(0);
  const F3 e1 = vtx(1) - va;
  const F3 e2 = vtx(nf - 1) - va;
  const float L1 = flen(e1), L2 = flen(e2);
  if (!(L1 > 0.f)) return DEC_UNDECIDED;
  const F3 v1 = e1 * (1.f / L1);
  const F3 cr = fcross(v1, e2);
  const float lc = flen(cr);
  if (!(lc > 1e-3f * L2)) return DEC_UNDECIDED;  // face frame ill-conditioned in FP32
  const F3 n = cr * (1.f / lc);
  // direction errors: v1 <= 2 eta / L1 + 3u ; n <= 2 (|dv1| L2 + eta + 4u L2) / lc + 3u
  const float ev1 = 2.f * eta / L1 + 3.f * F32_U;
  const float en = 2.f * (ev1 * L2 + eta + 4.f * F32_U * L2) / lc + 3.f * F32_U;
  const float ef = ev1 + en + 3.f * F32_U;  // frame error (v2 included)
  const F3 v = vi - va;
  const float V = flen(v);
  const float dist = fabsf(fdot(n, v));
  const float edist = en * V + eta + 4.f * F32_U * V;
  const int cd = cmp_gt(dist, lim, edist + F32_U * lim);
  if (cd > 0) return DEC_FALSE;
  const F3 v2 = fcross(n, v1);
  // in-plane coordinates of the face vertices relative to the projection P of vi:
  // D1 = (v_k - vi).v1 + dist n.v1 ; D2 likewise with v2 (n.v1, n.v2 are O(ef))
  const float eD = ef * (2.f * S + dist) + eta + 6.f * F32_U * 2.f * S;
  // P outside the face's extent along v1 or v2 (every D1, or every D2, beyond 0 on
  // one side): along v2 no edge straddles the line through P; along v1 every
  // straddling edge crosses it on the same side of P, and a closed polygon has an
  // even number of straddling edges.  The parity is then even, so the FP64 test
  // is false whatever its ties in the other direction or its plane distance.
  // Taken where a comparison is undecided: coplanar neighbours put P on the line
  // of a face edge.
  auto outside = [&]() -> bool {
    int lo1 = 0, hi1 = 0, lo2 = 0, hi2 = 0;
    for (int k = 0; k < nf; k++) {
      const F3 p = vtx(k) - vi;
      const int c1 = cmp_gt(fdot(p, v1), 0.f, eD), c2 = cmp_gt(fdot(p, v2), 0.f, eD);
      lo1 += c1 < 0;
      hi1 += c1 > 0;
      lo2 += c2 < 0;
      hi2 += c2 > 0;
    }
    return lo1 == nf || hi1 == nf || lo2 == nf || hi2 == nf;
  };
  if (cd == 0) return outside() ? DEC_FALSE : DEC_UNDECIDED;
  int odd = 0;
  F3 pa = vtx(0) - vi;
  float a1 = fdot(pa, v1), a2 = fdot(pa, v2);
  const int s_first = cmp_gt(a2, 0.f, eD);
  if (s_first == 0) return outside() ? DEC_FALSE : DEC_UNDECIDED;
  int sa = s_first;
  for (int k = 0; k < nf; k++) {
    float b1, b2;
    int sb;
    if (k + 1 == nf) {
      const F3 pb = vtx(0) - vi;
      b1 = fdot(pb, v1);
      b2 = fdot(pb, v2);
      sb = s_first;
    } else {
      const F3 pb = vtx(k + 1) - vi;
      b1 = fdot(pb, v1);
      b2 = fdot(pb, v2);
      sb = cmp_gt(b2, 0.f, eD);
      if (sb == 0) return outside() ? DEC_FALSE : DEC_UNDECIDED;
    }
    if (sa != sb) {  // the edge straddles the line through P along v1
      // crossing abscissa relative to P: X = a1 + t (b1 - a1), t = -a2 / (b2 - a2) in [0, 1]
      const float den = b2 - a2;
      const float t = -a2 / den;
      const float X = a1 + t * (b1 - a1);
      const float et = 3.f * eD / fabsf(den) + 2.f * F32_U;
      const float eX = eD + et * fabsf(b1 - a1) + 2.f * eD + 3.f * F32_U * (fabsf(a1) + fabsf(b1 - a1));
      const int cx = cmp_gt(0.f, X, eX);  // X < 0
      if (cx == 0) return outside() ? DEC_FALSE : DEC_UNDECIDED;
      if (cx > 0) odd ^= 1;
    }
    a1 = b1;
    a2 = b2;
    sa = sb;
  }
  return odd ? DEC_TRUE : DEC_FALSE;
}

__device__ __forceinline__ int decide_vf(F3 vi, const FView& vf, const ShapeDev& sf, int face, float lim, float S) {
  const int b = sf.fo[face];
  return decide_vf_list(vi, sf.fo[face + 1] - b, [&](int k) { return vf[sf.fv[b + k]]; }, lim, S);
}

// filter_ee: closest points of the two lines at s, t strictly inside (0, 1) and
// |pi - pj|^2 <= R^2; near-parallel edges (|f| within 8x its bound of 1e-12) are undecided.
__device__ inline int decide_ee(F3 vfi, F3 vsi, F3 vfj, F3 vsj, float R, float S) {
  const float eta = F32_ETA * S, u = F32_U;
  const F3 Ei = vsi - vfi, Ej = vsj - vfj, v = vfi - vfj;
  const float c = fdot(Ei, Ei), d = fdot(Ej, Ej), e = fdot(Ei, Ej);
  const float Li = sqrtf(c), Lj = sqrtf(d), V = flen(v);
  const float f = c * d - e * e;
  const float ae = fabsf(e);
  const float dc = 2.f * Li * eta + 4.f * u * c, dd = 2.f * Lj * eta + 4.f * u * d;
  const float de = (Li + Lj) * eta + 4.f * u * Li * Lj;
  const float df = dc * d + c * dd + 2.f * ae * de + 3.f * u * (c * d + e * e);
  const int cf = cmp_gt(fabsf(f), 1.0e-12f, df);
  if (cf < 0) return DEC_FALSE;
  if (cf == 0) return DEC_UNDECIDED;
  const float a = fdot(Ei, v), bb = fdot(Ej, v);
  const float aa = fabsf(a), ab = fabsf(bb);
  const float da = (Li + V) * eta + 4.f * u * Li * V, db = (Lj + V) * eta + 4.f * u * Lj * V;
  const float inv = 1.f / f, af = fabsf(f);
  const float s = (e * bb - a * d) * inv;
  const float t = (c * bb - e * a) * inv;
  const float as = fabsf(s), at = fabsf(t);
  const float ds = (de * ab + ae * db + da * d + aa * dd + 3.f * u * (ae * ab + aa * d) + as * df) / af + 3.f * u * as;
  const float dt = (dc * ab + c * db + de * aa + ae * da + 3.f * u * (c * ab + ae * aa) + at * df) / af + 3.f * u * at;
  const int s0 = cmp_gt(s, 0.f, ds), s1 = cmp_gt(1.f, s, ds + u);
  const int t0 = cmp_gt(t, 0.f, dt), t1 = cmp_gt(1.f, t, dt + u);
  if (s0 < 0 || s1 < 0 || t0 < 0 || t1 < 0) return DEC_FALSE;
  if (s0 == 0 || s1 == 0 || t0 == 0 || t1 == 0) return DEC_UNDECIDED;
  const F3 nv = v + Ei * s - Ej * t;
  const float dn = flen(nv);
  const float edn = eta * (1.f + as + at) + Li * ds + Lj * dt + 5.f * u * (V + Li * as + Lj * at) + 4.f * u * (dn + R);
  const int cn = cmp_gt(dn, R, edn);
  return cn < 0 ? DEC_TRUE : (cn > 0 ? DEC_FALSE : DEC_UNDECIDED);
}

// ---- contact screen of the polyhedron contact law (k_pdetect)
// Inputs are FP32 roundings of the FP64 world vertices (error u |x| per
// coordinate).  With W a bound of every |coordinate| involved, a difference of
// two inputs carries at most 3 u W per coordinate, so its norm at most
// ETA = 6 u W.  Each test returns true only when the FP64 detection
// (shape_detection_core.hpp: detection_vertex_vertex / _edge / _face,
// detection_edge_edge) provably finds no contact: a lower bound of the distance
// that a contact needs below R (the sum of the Minkowski radii) exceeds R by
// 8x its error bound.  Otherwise the FP64 detection runs.
__device__ __forceinline__ float fmaxabs(F3 a) { return fmaxf(fabsf(a.x), fmaxf(fabsf(a.y), fabsf(a.z))); }

// vertex-vertex: a contact needs |pi - pj| < R
__device__ inline bool apart_vv(F3 a, F3 b, float R) {
  const float eta = 6.f * F32_U * fmaxf(fmaxabs(a), fmaxabs(b));
  const float d = flen(a - b);
  return d > R + 8.f * (eta + 4.f * F32_U * (d + R));
}
// vertex-edge: a contact needs the projection parameter in (0, 1) and the
// distance to the line at most R, so the point-segment distance at most R.  The
// clamped distance min_t |w - e t| moves by at most |dw| + |de| under input
// errors; the FP32 projection parameter is off the minimiser by at most
// 8u (|w| + |e|) / |e|, which adds at most 8u (|w| + |e|)
__device__ inline bool apart_ve(F3 p, F3 a, F3 b, float R) {
  const float eta = 6.f * F32_U * fmaxf(fmaxabs(p), fmaxf(fmaxabs(a), fmaxabs(b)));
  const F3 e = b - a, w = p - a;
  const float ee = fdot(e, e);
  if (!(ee > 0.f)) return false;
  const float t = fminf(fmaxf(fdot(w, e) / ee, 0.f), 1.f);
  const float d = flen(w - e * t);
  const float err = 2.f * eta + 8.f * F32_U * (flen(w) + sqrtf(ee)) + 4.f * F32_U * (d + R);
  return d > R + 8.f * err;
}
// vertex-face: a contact needs the distance to the plane through va with normal
// (vb - va) x (vc - va) (vf_core's frame: first, second and last face vertex)
// at most R.  The unit normal's error is at most 4 ETA L / |c| (L the longer of
// the two edges, c their cross product); faces with |c| <= 1e-3 L^2 are not
// screened
__device__ inline bool apart_vf(F3 p, F3 va, F3 vb, F3 vc, float R) {
  const float eta = 6.f * F32_U * fmaxf(fmaxf(fmaxabs(p), fmaxabs(va)), fmaxf(fmaxabs(vb), fmaxabs(vc)));
  const F3 e1 = vb - va, e2 = vc - va, w = p - va;
  const F3 c = fcross(e1, e2);
  const float cl = flen(c), L = fmaxf(flen(e1), flen(e2));
  if (!(cl > 1e-3f * L * L)) return false;
  const float dist = fabsf(fdot(c, w)) / cl;
  const float W = flen(w);
  const float err = 4.f * eta * L * W / cl + eta + 8.f * F32_U * (W + dist + R);
  return dist > R + 8.f * err;
}
// edge-edge: a contact needs non-parallel edges, the closest points of the two
// lines inside both edges and their distance at most R, so the distance of the
// two lines, |v . c| / |c| with c = Ei x Ej, at most R.  Pairs with
// |c| <= 0.05 |Ei| |Ej| are not screened
__device__ inline bool apart_ee(F3 a0, F3 a1, F3 b0, F3 b1, float R) {
  const float eta =
      6.f * F32_U * fmaxf(fmaxf(fmaxabs(a0), fmaxabs(a1)), fmaxf(fmaxabs(b0), fmaxabs(b1)));
  const F3 Ei = a1 - a0, Ej = b1 - b0, v = a0 - b0;
  const F3 c = fcross(Ei, Ej);
  const float Li = flen(Ei), Lj = flen(Ej), cl = flen(c), V = flen(v);
  if (!(cl > 0.05f * Li * Lj)) return false;
  const float D = fabsf(fdot(v, c)) / cl;
  const float dc = eta * (Li + Lj) + 4.f * F32_U * Li * Lj;  // bound of |c - c_exact|
  const float err = eta + (V + D) * dc / cl + 8.f * F32_U * (V + D + R);
  return D > R + 8.f * err;
}

}  // namespace dem
