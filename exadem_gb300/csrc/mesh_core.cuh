// mesh_core.cuh -- a sphere against the vertices, edges and faces of a mesh
// driver (RShapeDriver): the Verlet filters of detection_sphere_driver
// (sphere/nbh_sphere.hpp:25-86) and the detectors detect<7|8|9> for spheres
// (shape_detection_api.hpp:357-386, shape_detection_core.hpp:57-220).  The
// sphere is a vertex of radius rad; the mesh has homothety 1 and its
// Minkowski radius.  World vertices are precomputed once (the mesh does not
// move), which gives the values shape::get_vertex computes per call.
#pragma once
#include "../../include/dem_hotpath.h"
#include "poly_core.cuh"
#include "poly_f32.cuh"

namespace dem {

__device__ __forceinline__ VView mesh_view(const MeshDev& m) { return VView{m.x, m.y, m.z}; }

// kind 0 vertex, 1 edge, 2 face: filter_vertex_vertex_v2, filter_vertex_edge,
// filter_vertex_face with rVerlet = the skin
__device__ inline bool mesh_filter(const MeshDev& m, uint32_t kind, uint32_t j, double rV, V3 p, double rad) {
  const VView v = mesh_view(m);
  if (kind == 0) return filter_vv(rV, p, rad, v[j], m.r);
  if (kind == 1) return filter_ve(rV, p, rad, v[m.e[2 * j]], v[m.e[2 * j + 1]], m.r);
  double dist;
  V3 n;
  const int b = m.fo[j];
  return vf_core_list(rad + m.r + rV, p, v, m.fv + b, m.fo[j + 1] - b, dist, n);
}

// mesh_filter decided in FP32 first (poly_f32.cuh): coordinates relative to the
// sphere centre p, each an FP32 rounding of the FP64 difference (error u S with
// S a bound of their lengths plus the filter range); a decided test has the
// FP64 result, an undecided one runs mesh_filter
__device__ inline bool mesh_filter_f32(const MeshDev& m, uint32_t kind, uint32_t j, double rV, V3 p, double rad) {
  const VView v = mesh_view(m);
  auto rel = [&](int k) {
    const V3 w = v[k];
    return f3((float)(w.x - p.x), (float)(w.y - p.y), (float)(w.z - p.z));
  };
  const float R = (float)(rad + m.r + rV);
  int dec;
  if (kind == 0) {
    const F3 a = rel((int)j);
    dec = decide_vv(f3(0.f, 0.f, 0.f), a, R, flen(a) * 1.000001f + R);
  } else if (kind == 1) {
    const F3 a = rel(m.e[2 * j]), b = rel(m.e[2 * j + 1]);
    dec = decide_ve(f3(0.f, 0.f, 0.f), a, b, R, (float)rV, fmaxf(flen(a), flen(b)) * 1.000001f + R);
  } else {
    const int b = m.fo[j], nf = m.fo[j + 1] - b;
    float S = 0.f;
    for (int k = 0; k < nf; k++) S = fmaxf(S, flen(rel(m.fv[b + k])));
    dec = decide_vf_list(f3(0.f, 0.f, 0.f), nf, [&](int k) { return rel(m.fv[b + k]); }, R, S * 1.000001f + R);
  }
  if (dec != DEC_UNDECIDED) return dec == DEC_TRUE;
  return mesh_filter(m, kind, j, rV, p, rad);
}

// detect<type> for a sphere and mesh feature j
__device__ inline DetD mesh_detect(const MeshDev& m, uint32_t type, uint32_t j, V3 p, double rad) {
  const VView v = mesh_view(m);
  if (type == DEM_ITYPE_VERTEX_MESH_VERTEX) return detect_vv(p, rad, v[j], m.r);
  if (type == DEM_ITYPE_VERTEX_MESH_EDGE) return detect_ve(p, rad, v[m.e[2 * j]], v[m.e[2 * j + 1]], m.r);
  // detection_vertex_face for spheres (shape_detection_core.hpp:151-220)
  const double R = rad + m.r;
  double dist;
  V3 n;
  const int b = m.fo[j];
  const bool inside = vf_core_list(R, p, v, m.fv + b, m.fo[j + 1] - b, dist, n);
  if (dist > R) return det_none();
  const double dn = dist - R;
  return DetD{inside, dn, n, p - n * (rad + 0.5 * dn)};
}

// detect<7..12> for a polyhedron (shape_detection_api.hpp:357-405): its vertex,
// edge or face osub (world vertices va, shape sh, Minkowski radius ra) against
// the mesh's feature psub; 11 and 12 take the mesh vertex as the vertex side
__device__ inline DetD poly_mesh_detect(const MeshDev& m, uint32_t type, uint32_t osub, uint32_t psub,
                                        const VView& va, const ShapeDev& sh, double ra) {
  const VView mv = mesh_view(m);
  switch (type) {
    case DEM_ITYPE_VERTEX_MESH_VERTEX: return detect_vv(va[osub], ra, mv[psub], m.r);
    case DEM_ITYPE_VERTEX_MESH_EDGE: return detect_ve(va[osub], ra, mv[m.e[2 * psub]], mv[m.e[2 * psub + 1]], m.r);
    case DEM_ITYPE_VERTEX_MESH_FACE: {
      const double R = ra + m.r;
      double dist;
      V3 n;
      const int b = m.fo[psub];
      const bool inside = vf_core_list(R, va[osub], mv, m.fv + b, m.fo[psub + 1] - b, dist, n);
      if (dist > R) return det_none();
      const double dn = dist - R;
      return DetD{inside, dn, n, va[osub] - n * (ra + 0.5 * dn)};
    }
    case DEM_ITYPE_EDGE_MESH_EDGE:
      return detect_ee(va[sh.e[2 * osub]], va[sh.e[2 * osub + 1]], ra, mv[m.e[2 * psub]], mv[m.e[2 * psub + 1]], m.r);
    case DEM_ITYPE_MESH_VERTEX_EDGE: return detect_ve(mv[psub], m.r, va[sh.e[2 * osub]], va[sh.e[2 * osub + 1]], ra);
    default: return detect_vf(mv[psub], m.r, va, sh, (int)osub, ra);
  }
}

// the bin of p: false outside the bin grid (no feature can pass there)
__device__ inline bool mesh_bin_of(const MeshDev& m, V3 p, uint64_t& b) {
  const double fx = (p.x - m.lo[0]) * m.inv_bs;
  const double fy = (p.y - m.lo[1]) * m.inv_bs;
  const double fz = (p.z - m.lo[2]) * m.inv_bs;
  if (!(fx >= 0.0 && fx < (double)m.dims[0] && fy >= 0.0 && fy < (double)m.dims[1] && fz >= 0.0 &&
        fz < (double)m.dims[2]))
    return false;
  b = (uint64_t)(int)fx + (uint64_t)m.dims[0] * ((uint64_t)(int)fy + (uint64_t)m.dims[1] * (int)fz);
  return true;
}

}  // namespace dem
