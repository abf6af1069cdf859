// poly_core.cuh -- device restatement of exaDEM's sphero-polyhedron geometry.
//
//   shape table           src/shape/include/exaDEM/shape.hpp:50-68,245-262
//   compute_obb           src/shape/include/exaDEM/basic_types.hpp:37-48
//   OBB::intersect (SAT)  src/shape/include/exaDEM/type/OBB.hpp:90-220 (tol = FLT_EPSILON)
//   filters               src/shape/include/exaDEM/shape_detection_core.hpp:43-53 (VV),
//                         :83-101 (VE), :246-309 (VF), :468-504 (EE)
//   detection cores       :57-81 (VV), :122-148 (VE), :398-466 (VF), :521-566 (EE)
// Same FP64 operation order as the reference (compiled with --fmad=false).
// A rejected detection returns dn = 0, like the reference's default `contact`.
#pragma once
#include "integrate_core.cuh"

namespace dem {

constexpr int SH_MAXV = DEM_MAX_SHAPE_VERTICES;
constexpr int SH_MAXE = 64;
constexpr int SH_MAXF = 32;
constexpr int SH_MAXFV = 128;

struct ShapeDev {
  int nv, ne, nf;
  double r;        // Minkowski radius
  double maxv;     // max |v0|
  double obb[15];  // center, e1, e2, e3, extent
  double v[3 * SH_MAXV];
  int e[2 * SH_MAXE];
  int fo[SH_MAXF + 1];  // face offsets into fv
  int fv[SH_MAXFV];
  float vf[3 * SH_MAXV];  // FP32 copy of v (split-precision displacement test)
};

struct OBBd {
  V3 c, e1, e2, e3, ext;
};

__device__ __forceinline__ V3 sh_v(const ShapeDev& s, int k) { return mk(s.v[3 * k], s.v[3 * k + 1], s.v[3 * k + 2]); }

// world vertex p + q * (h * v0)
__device__ __forceinline__ V3 world_vertex(const ShapeDev& s, int k, V3 p, Q4 q, double h) {
  return p + qrotate(q, h * sh_v(s, k));
}

__device__ __forceinline__ OBBd compute_obb(const ShapeDev& s, V3 p, Q4 q, double h) {
  OBBd o;
  o.c = mk(s.obb[0], s.obb[1], s.obb[2]);
  o.e1 = qrotate(q, mk(s.obb[3], s.obb[4], s.obb[5]));
  o.e2 = qrotate(q, mk(s.obb[6], s.obb[7], s.obb[8]));
  o.e3 = qrotate(q, mk(s.obb[9], s.obb[10], s.obb[11]));
  o.c = qrotate(q, o.c);
  o.ext = mk(s.obb[12], s.obb[13], s.obb[14]);
  if (h != 1.0) {
    o.ext = o.ext * h;
    o.c = o.c * h;
  }
  o.c = o.c + p;
  return o;
}

__device__ __forceinline__ void obb_enlarge(OBBd& o, double m) {
  o.ext.x += m;
  o.ext.y += m;
  o.ext.z += m;
}

__device__ inline bool obb_intersect(const OBBd& A, const OBBd& B) {
  const double tol = 1.1920928955078125e-07;
  double ra, rb;
  const double Rxx = dot(A.e1, B.e1), Rxy = dot(A.e1, B.e2), Rxz = dot(A.e1, B.e3);
  const double Axx = fabs(Rxx) + tol, Axy = fabs(Rxy) + tol, Axz = fabs(Rxz) + tol;
  const V3 tt = A.c - B.c;
  const V3 t = mk(dot(tt, A.e1), dot(tt, A.e2), dot(tt, A.e3));
  ra = A.ext.x;
  rb = B.ext.x * Axx + B.ext.y * Axy + B.ext.z * Axz;
  if (fabs(t.x) > ra + rb) return false;
  const double Ryx = dot(A.e2, B.e1);
  const double Ayx = fabs(Ryx) + tol;
  const double Ryy = dot(A.e2, B.e2);
  const double Ayy = fabs(Ryy) + tol;
  const double Ryz = dot(A.e2, B.e3);
  const double Ayz = fabs(Ryz) + tol;
  ra = A.ext.y;
  rb = B.ext.x * Ayx + B.ext.y * Ayy + B.ext.z * Ayz;
  if (fabs(t.y) > ra + rb) return false;
  const double Rzx = dot(A.e3, B.e1);
  const double Azx = fabs(Rzx) + tol;
  const double Rzy = dot(A.e3, B.e2);
  const double Azy = fabs(Rzy) + tol;
  const double Rzz = dot(A.e3, B.e3);
  const double Azz = fabs(Rzz) + tol;
  ra = A.ext.z;
  rb = B.ext.x * Azx + B.ext.y * Azy + B.ext.z * Azz;
  if (fabs(t.z) > ra + rb) return false;
  ra = A.ext.x * Axx + A.ext.y * Ayx + A.ext.z * Azx;
  rb = B.ext.x;
  if (fabs(t.x * Rxx + t.y * Ryx + t.z * Rzx) > ra + rb) return false;
  ra = A.ext.x * Axy + A.ext.y * Ayy + A.ext.z * Azy;
  rb = B.ext.y;
  if (fabs(t.x * Rxy + t.y * Ryy + t.z * Rzy) > ra + rb) return false;
  ra = A.ext.x * Axz + A.ext.y * Ayz + A.ext.z * Azz;
  rb = B.ext.z;
  if (fabs(t.x * Rxz + t.y * Ryz + t.z * Rzz) > ra + rb) return false;
  ra = A.ext.y * Azx + A.ext.z * Ayx;
  rb = B.ext.y * Axz + B.ext.z * Axy;
  if (fabs(t.z * Ryx - t.y * Rzx) > ra + rb) return false;
  ra = A.ext.y * Azy + A.ext.z * Ayy;
  rb = B.ext.x * Axz + B.ext.z * Axx;
  if (fabs(t.z * Ryy - t.y * Rzy) > ra + rb) return false;
  ra = A.ext.y * Azz + A.ext.z * Ayz;
  rb = B.ext.x * Axy + B.ext.y * Axx;
  if (fabs(t.z * Ryz - t.y * Rzz) > ra + rb) return false;
  ra = A.ext.x * Azx + A.ext.z * Axx;
  rb = B.ext.y * Ayz + B.ext.z * Ayy;
  if (fabs(t.x * Rzx - t.z * Rxx) > ra + rb) return false;
  ra = A.ext.x * Azy + A.ext.z * Axy;
  rb = B.ext.x * Ayz + B.ext.z * Ayx;
  if (fabs(t.x * Rzy - t.z * Rxy) > ra + rb) return false;
  ra = A.ext.x * Azz + A.ext.z * Axz;
  rb = B.ext.x * Ayy + B.ext.y * Ayx;
  if (fabs(t.x * Rzz - t.z * Rxz) > ra + rb) return false;
  ra = A.ext.x * Ayx + A.ext.y * Axx;
  rb = B.ext.y * Azz + B.ext.z * Azy;
  if (fabs(t.y * Rxx - t.x * Ryx) > ra + rb) return false;
  ra = A.ext.x * Ayy + A.ext.y * Axy;
  rb = B.ext.x * Azz + B.ext.z * Azx;
  if (fabs(t.y * Rxy - t.x * Ryy) > ra + rb) return false;
  ra = A.ext.x * Ayz + A.ext.y * Axz;
  rb = B.ext.x * Azy + B.ext.y * Azx;
  if (fabs(t.y * Rxz - t.x * Ryz) > ra + rb) return false;
  return true;
}

__device__ __forceinline__ V3 vnormalized(V3 v) { return v / vnorm(v); }  // _normalize

// ---- filters
__device__ __forceinline__ bool filter_vv(double rV, V3 vi, double ri, V3 vj, double rj) {
  const double R = ri + rj + rV;
  const V3 dist = vi - vj;
  const double d2 = dot(dist, dist);
  return d2 <= R * R;
}
__device__ __forceinline__ bool filter_ve(double rV, V3 vi, double ri, V3 vf, V3 vs, double rj) {
  const V3 distfs = vs - vf;
  const V3 distfi = vi - vf;
  const double r = (dot(distfs, distfi)) / (dot(distfs, distfs));
  if (r < -rV || r > 1.0 + rV) return false;
  const V3 dist = distfi - distfs * r;
  const double Rmax = ri + rj + rV;
  return (dot(dist, dist) < (Rmax * Rmax));
}

// Vertex array of a particle: world vertices stored with stride MV per particle.
struct VView {
  const double* x;
  const double* y;
  const double* z;
  __device__ __forceinline__ V3 operator[](int k) const { return mk(x[k], y[k], z[k]); }
};

// point-in-face core shared by the face filter and detection; returns inside,
// sets dist (unsigned plane distance) and n (oriented normal).  The face is the
// vertex list fv[0 .. nf) of vaj.
__device__ inline bool vf_core_list(double lim, V3 vi, const VView& vaj, const int* fv, int nf, double& dist_out,
                                    V3& n_out) {
  const V3 va = vaj[fv[0]];
  const V3 vb = vaj[fv[1]];
  const V3 vc = vaj[fv[nf - 1]];
  const V3 v = vi - va;
  V3 v1 = vb - va;
  V3 v2 = vc - va;
  v1 = vnormalized(v1);
  V3 n = cross(v1, v2);
  n = vnormalized(n);
  double dist = dot(n, v);
  if (dist < 0) {
    n = n * (-1);
    dist = -dist;
  }
  dist_out = dist;
  n_out = n;
  if (dist > lim) return false;
  const V3 P = vi - n * dist;
  int ODD = 0;
  v2 = cross(n, v1);
  const double ori1 = dot(P, v1);
  const double ori2 = dot(P, v2);
  for (int iva = 0; iva < nf; ++iva) {
    int ivb = iva + 1;
    if (ivb == nf) ivb = 0;
    const V3 _va = vaj[fv[iva]];
    const V3 _vb = vaj[fv[ivb]];
    const double pa1 = dot(_va, v1);
    const double pb1 = dot(_vb, v1);
    const double pa2 = dot(_va, v2);
    const double pb2 = dot(_vb, v2);
    if ((pa2 < ori2 && pb2 >= ori2) || (pb2 < ori2 && pa2 >= ori2)) {
      if (pa1 + (ori2 - pa2) / (pb2 - pa2) * (pb1 - pa1) < ori1) ODD = 1 - ODD;
    }
  }
  return ODD == 1;
}
__device__ __forceinline__ bool vf_core(double lim, V3 vi, const VView& vaj, const ShapeDev& sj, int face,
                                        double& dist_out, V3& n_out) {
  const int b = sj.fo[face];
  return vf_core_list(lim, vi, vaj, sj.fv + b, sj.fo[face + 1] - b, dist_out, n_out);
}
__device__ __forceinline__ bool filter_vf(double rV, V3 vi, double ri, const VView& vaj, const ShapeDev& sj, int face,
                                          double rj) {
  double dist;
  V3 n;
  return vf_core(ri + rj + rV, vi, vaj, sj, face, dist, n);
}
__device__ inline bool filter_ee(double rV, V3 vfi, V3 vsi, double ri, V3 vfj, V3 vsj, double rj) {
  const double R = ri + rj + rV;
  const V3 Ei = vsi - vfi;
  const V3 Ej = vsj - vfj;
  const V3 v = vfi - vfj;
  const double c = dot(Ei, Ei);
  const double d = dot(Ej, Ej);
  const double e = dot(Ei, Ej);
  double f = (c * d) - (e * e);
  if (fabs(f) > 1.0e-12) {
    f = 1.0 / f;
    const double a = dot(Ei, v);
    const double b = dot(Ej, v);
    const double s_ = (e * b - a * d) * f;
    const double t_ = (c * b - e * a) * f;
    if (s_ <= 0.0 || s_ >= 1.0 || t_ <= 0.0 || t_ >= 1.0) return false;
    const V3 pi = vfi + Ei * s_;
    const V3 pj = vfj + Ej * t_;
    const V3 n = pi - pj;
    return (dot(n, n) <= (R * R));
  }
  return false;
}

// ---- detection cores
struct DetD {
  bool c;
  double dn;
  V3 n, cp;
};
__device__ __forceinline__ DetD det_none() { return DetD{false, 0.0, mk(0, 0, 0), mk(0, 0, 0)}; }

__device__ __forceinline__ DetD detect_vv(V3 pi, double ri, V3 pj, double rj) {
  const double R = ri + rj;
  const V3 dist = pi - pj;
  const double dist_norm = vnorm(dist);
  const double inv_dist_norm = 1.0 / dist_norm;
  const double dn = dist_norm - R;
  const V3 n = dist * inv_dist_norm;
  const V3 cp = pi - n * (ri + 0.5 * dn);
  return DetD{dn < 0, dn, n, cp};
}
__device__ inline DetD detect_ve(V3 vi, double ri, V3 vf, V3 vs, double rj) {
  const V3 distfs = vs - vf;
  const V3 distfi = vi - vf;
  const double r = (dot(distfs, distfi)) / (dot(distfs, distfs));
  if (r <= 0 || r >= 1.0) return det_none();
  V3 n = distfi - distfs * r;
  const double dn = vnorm(n) - (ri + rj);
  if (dn > 0) return det_none();
  n = vnormalized(n);
  const V3 cp = vi - n * (ri + 0.5 * dn);
  return DetD{true, dn, n, cp};
}
__device__ inline DetD detect_vf(V3 vi, double ri, const VView& vaj, const ShapeDev& sj, int face, double rj) {
  double dist;
  V3 n;
  const bool inside = vf_core(ri + rj, vi, vaj, sj, face, dist, n);
  if (dist > (ri + rj)) return det_none();
  const double dn = dist - (ri + rj);
  const V3 cp = vi - n * (ri + 0.5 * dn);
  return DetD{inside, dn, n, cp};
}
__device__ inline DetD detect_ee(V3 vfi, V3 vsi, double ri, V3 vfj, V3 vsj, double rj) {
  const double R = ri + rj;
  const V3 Ei = vsi - vfi;
  const V3 Ej = vsj - vfj;
  const V3 v = vfi - vfj;
  const double c = dot(Ei, Ei);
  const double d = dot(Ej, Ej);
  const double e = dot(Ei, Ej);
  double f = (c * d) - (e * e);
  if (fabs(f) > 1.0e-12) {
    f = 1.0 / f;
    const double a = dot(Ei, v);
    const double b = dot(Ej, v);
    const double s_ = (e * b - a * d) * f;
    const double t_ = (c * b - e * a) * f;
    if (s_ <= 0.0 || s_ >= 1.0 || t_ <= 0.0 || t_ >= 1.0) return det_none();
    const V3 pi = vfi + Ei * s_;
    const V3 pj = vfj + Ej * t_;
    V3 n = pi - pj;
    const double dn = vnorm(n) - R;
    if (dn > 0) return det_none();
    n = vnormalized(n);
    const V3 cp = pi - n * (ri + 0.5 * dn);
    return DetD{dn <= 0, dn, n, cp};
  }
  return det_none();
}

}  // namespace dem
