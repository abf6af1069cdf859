// mesh_bins.hpp -- host construction of a mesh driver's feature bins (plain
// C++, no CUDA: the library uploads the result, a CPU test checks it).
//
// The reference lists, per grid cell, the mesh features whose enlarged OBB
// meets the cell (grid_rshape_driver, grid_stl_mesh.cpp:30-265); a particle
// keeps the features of its cell that pass their Verlet filter
// (nbh_sphere.hpp:25-86, nbh_polyhedron_driver.hpp:61-192).  Here a uniform
// bin grid over the mesh lists, per bin, every feature whose filter can pass
// for a point of the bin: a bin lists a feature when its centre is within
// E + margin + half its diagonal of the feature's region, E = the largest
// particle radius + the mesh's Minkowski radius + the skin.  The regions:
//   vertex  the vertex;
//   edge    the segment extended by the skin in its line parameter
//           (filter_vertex_edge_core compares that parameter with rVerlet);
//   face    the polygon (fan-split into triangles: a superset when non-convex).
// Items of a bin are (kind << 30 | index), kind 0 vertex, 1 edge, 2 face, in
// (kind, index) order.  The bin of a point is floor((p - lo) * inv_bs) per axis.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

namespace dem {
namespace meshbins {

struct Input {
  int nv, ne, nf;
  const double* x;  // world vertices
  const double* y;
  const double* z;
  const int* e;   // 2 ne
  const int* fo;  // nf + 1
  const int* fv;
  double r;  // Minkowski radius
};

struct Output {
  double lo[3] = {0, 0, 0};
  double inv_bs = 0.0;
  int dims[3] = {0, 0, 0};
  std::vector<uint32_t> boff;   // bins + 1
  std::vector<uint32_t> items;  // boff[bins]
  // per feature (vertices, edges, faces): FP32 bounding sphere x, y, z, r of
  // its region (the edge's extended by the skin), radius rounded up
  std::vector<float> sph;
};

enum : int { OK = 0, NONFINITE = 1, OVERFLOW_ = 2 };

struct P3 {
  double x, y, z;
};
inline P3 sub3(P3 a, P3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline double dot3(P3 a, P3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline P3 axpy(P3 a, double t, P3 d) { return {a.x + t * d.x, a.y + t * d.y, a.z + t * d.z}; }
inline double dist3(P3 a, P3 b) { return std::sqrt(dot3(sub3(a, b), sub3(a, b))); }
// distance from c to the segment a + t (b - a), t in [t0, t1]
inline double seg_dist(P3 c, P3 a, P3 b, double t0, double t1) {
  const P3 d = sub3(b, a);
  const double dd = dot3(d, d);
  double t = dd > 0.0 ? dot3(sub3(c, a), d) / dd : 0.0;
  t = std::min(std::max(t, t0), t1);
  return dist3(c, axpy(a, t, d));
}
// distance from p to the triangle abc (closest point on a triangle, Ericson's
// Real-Time Collision Detection 5.1.5)
inline double tri_dist(P3 p, P3 a, P3 b, P3 c) {
  const P3 ab = sub3(b, a), ac = sub3(c, a), ap = sub3(p, a);
  const double d1 = dot3(ab, ap), d2 = dot3(ac, ap);
  if (d1 <= 0.0 && d2 <= 0.0) return dist3(p, a);
  const P3 bp = sub3(p, b);
  const double d3 = dot3(ab, bp), d4 = dot3(ac, bp);
  if (d3 >= 0.0 && d4 <= d3) return dist3(p, b);
  const double vc = d1 * d4 - d3 * d2;
  if (vc <= 0.0 && d1 >= 0.0 && d3 <= 0.0) return dist3(p, axpy(a, d1 / (d1 - d3), ab));
  const P3 cp = sub3(p, c);
  const double d5 = dot3(ab, cp), d6 = dot3(ac, cp);
  if (d6 >= 0.0 && d5 <= d6) return dist3(p, c);
  const double vb = d5 * d2 - d1 * d6;
  if (vb <= 0.0 && d2 >= 0.0 && d6 <= 0.0) return dist3(p, axpy(a, d2 / (d2 - d6), ac));
  const double va = d3 * d6 - d5 * d4;
  if (va <= 0.0 && (d4 - d3) >= 0.0 && (d5 - d6) >= 0.0)
    return dist3(p, axpy(b, (d4 - d3) / ((d4 - d3) + (d5 - d6)), sub3(c, b)));
  const double den = 1.0 / (va + vb + vc);
  const double v = vb * den, w = vc * den;
  return dist3(p, axpy(axpy(a, v, ab), w, ac));
}

// the bin of p (the device's mesh_bin_of); false outside the grid
inline bool bin_of(const Output& o, double px, double py, double pz, uint64_t& b) {
  const double f[3] = {(px - o.lo[0]) * o.inv_bs, (py - o.lo[1]) * o.inv_bs, (pz - o.lo[2]) * o.inv_bs};
  for (int d = 0; d < 3; d++)
    if (!(f[d] >= 0.0 && f[d] < (double)o.dims[d])) return false;
  b = (uint64_t)(int)f[0] + (uint64_t)o.dims[0] * ((uint64_t)(int)f[1] + (uint64_t)o.dims[1] * (int)f[2]);
  return true;
}

// bins for particles of radius <= rad and the skin; OK, NONFINITE or OVERFLOW_
inline int build(const Input& m, double rad, double skin, Output& out) {
  const int nv = m.nv, ne = m.ne, nf = m.nf;
  const double E = rad + m.r + skin;  // Rmax of the vertex, edge and face filters
  auto V = [&](int k) { return P3{m.x[k], m.y[k], m.z[k]}; };
  struct Box {
    double lo[3], hi[3];
  };
  auto empty = [] { return Box{{HUGE_VAL, HUGE_VAL, HUGE_VAL}, {-HUGE_VAL, -HUGE_VAL, -HUGE_VAL}}; };
  auto grow = [](Box& b, P3 p) {
    const double c[3] = {p.x, p.y, p.z};
    for (int d = 0; d < 3; d++) {
      b.lo[d] = std::min(b.lo[d], c[d]);
      b.hi[d] = std::max(b.hi[d], c[d]);
    }
  };
  double amax = 0.0;
  for (int k = 0; k < nv; k++) amax = std::max(amax, std::max(std::fabs(m.x[k]), std::max(std::fabs(m.y[k]), std::fabs(m.z[k]))));
  std::vector<Box> box;
  box.reserve((size_t)nv + ne + nf);
  for (int k = 0; k < nv; k++) {
    Box b = empty();
    grow(b, V(k));
    box.push_back(b);
  }
  double span = 0.0;
  for (int k = 0; k < ne; k++) {
    const P3 a = V(m.e[2 * k]), d = sub3(V(m.e[2 * k + 1]), a);
    Box b = empty();
    grow(b, axpy(a, -skin, d));
    grow(b, axpy(a, 1.0 + skin, d));
    span = std::max(span, std::max(b.hi[0] - b.lo[0], std::max(b.hi[1] - b.lo[1], b.hi[2] - b.lo[2])));
    box.push_back(b);
  }
  // The face filter (filter_vertex_face) projects on the plane through the face's
  // first, second and last vertices.  A point it keeps lies within E of that
  // plane above the projected polygon, hence within E + flat[k] of the fan of
  // the face's own triangles, flat[k] being the largest distance of a face
  // vertex from that plane (0 for a planar face).
  std::vector<double> flat(nf, 0.0);
  for (int k = 0; k < nf; k++) {
    Box b = empty();
    for (int q = m.fo[k]; q < m.fo[k + 1]; q++) grow(b, V(m.fv[q]));
    const int b0 = m.fo[k], nvf = m.fo[k + 1] - b0;
    if (nvf > 3) {
      const P3 o = V(m.fv[b0]);
      const P3 u = sub3(V(m.fv[b0 + 1]), o), w = sub3(V(m.fv[b0 + nvf - 1]), o);
      P3 nn = {u.y * w.z - u.z * w.y, u.z * w.x - u.x * w.z, u.x * w.y - u.y * w.x};
      const double len = std::sqrt(nn.x * nn.x + nn.y * nn.y + nn.z * nn.z);
      double dmax = 0.0;
      if (len > 0.0) {
        nn = {nn.x / len, nn.y / len, nn.z / len};
        for (int q = 2; q + 1 < nvf; q++) {
          const P3 r = sub3(V(m.fv[b0 + q]), o);
          dmax = std::max(dmax, std::fabs(r.x * nn.x + r.y * nn.y + r.z * nn.z));
        }
      } else {  // degenerate first corner: bound by the face's extent
        for (int d = 0; d < 3; d++) dmax = std::max(dmax, b.hi[d] - b.lo[d]);
      }
      flat[k] = dmax * (1.0 + 1e-12);
    }
    for (int d = 0; d < 3; d++) {
      b.lo[d] -= flat[k];
      b.hi[d] += flat[k];
    }
    box.push_back(b);
  }
  const double margin = 1e-7 * (E + amax + span) + 1e-12;
  Box all = empty();
  for (Box& b : box) {
    for (int d = 0; d < 3; d++) {
      b.lo[d] -= E + margin;
      b.hi[d] += E + margin;
    }
    grow(all, {b.lo[0], b.lo[1], b.lo[2]});
    grow(all, {b.hi[0], b.hi[1], b.hi[2]});
  }
  for (int d = 0; d < 3; d++)
    if (box.empty() || !std::isfinite(all.lo[d]) || !std::isfinite(all.hi[d])) return NONFINITE;
  // bin size: about the filter range, at most 2^22 bins
  const double ext = std::max(all.hi[0] - all.lo[0], std::max(all.hi[1] - all.lo[1], all.hi[2] - all.lo[2]));
  double bs = std::max(E, ext / 256.0);
  int* dims = out.dims;
  for (;;) {
    uint64_t tot = 1;
    for (int d = 0; d < 3; d++) {
      dims[d] = (int)std::floor((all.hi[d] - all.lo[d]) * (1.0 / bs)) + 1;
      tot *= (uint64_t)dims[d];
    }
    if (tot <= (1u << 22)) break;
    bs *= 1.5;
  }
  for (int d = 0; d < 3; d++) out.lo[d] = all.lo[d];
  out.inv_bs = 1.0 / bs;
  // the bin range of a box: the index formula of bin_of, monotone in the coordinate
  auto index = [&](double x, int d) {
    const double f = (x - out.lo[d]) * out.inv_bs;
    return std::min(std::max((int)std::floor(f), 0), dims[d] - 1);
  };
  const uint64_t nb = (uint64_t)dims[0] * dims[1] * dims[2];
  const double reach = E + 2.0 * margin + 0.8660254037844387 * bs * (1.0 + 1e-12);
  auto near = [&](size_t k, P3 ctr) {
    if (k < (size_t)nv) return dist3(ctr, V((int)k)) <= reach;
    if (k < (size_t)nv + ne) {
      const int q = (int)(k - nv);
      return seg_dist(ctr, V(m.e[2 * q]), V(m.e[2 * q + 1]), -skin, 1.0 + skin) <= reach;
    }
    const int f = (int)(k - nv - ne), b0 = m.fo[f], nvf = m.fo[f + 1] - b0;
    for (int q = 1; q + 1 < nvf; q++)
      if (tri_dist(ctr, V(m.fv[b0]), V(m.fv[b0 + q]), V(m.fv[b0 + q + 1])) <= reach + flat[f]) return true;
    return false;
  };
  auto for_bins = [&](size_t k, auto&& f) {
    const Box& b = box[k];
    const int x0 = index(b.lo[0], 0), x1 = index(b.hi[0], 0);
    const int y0 = index(b.lo[1], 1), y1 = index(b.hi[1], 1);
    const int z0 = index(b.lo[2], 2), z1 = index(b.hi[2], 2);
    for (int z = z0; z <= z1; z++)
      for (int y = y0; y <= y1; y++)
        for (int x = x0; x <= x1; x++) {
          const P3 ctr = {out.lo[0] + (x + 0.5) * bs, out.lo[1] + (y + 0.5) * bs, out.lo[2] + (z + 0.5) * bs};
          if (near(k, ctr)) f((uint64_t)x + (uint64_t)dims[0] * ((uint64_t)y + (uint64_t)dims[1] * z));
        }
  };
  std::vector<uint32_t>& cnt = out.boff;
  cnt.assign(nb + 1, 0);
  uint64_t total = 0;
  for (size_t k = 0; k < box.size(); k++)
    for_bins(k, [&](uint64_t q) {
      cnt[q + 1]++;
      total++;
    });
  if (total >= (1ull << 32)) return OVERFLOW_;
  for (uint64_t q = 0; q < nb; q++) cnt[q + 1] += cnt[q];
  out.items.assign(total, 0);
  std::vector<uint32_t> cur(cnt.begin(), cnt.end() - 1);
  for (size_t k = 0; k < box.size(); k++) {  // (kind, index) order: vertices, edges, faces
    const uint32_t kind = k < (size_t)nv ? 0u : (k < (size_t)nv + ne ? 1u : 2u);
    const uint32_t idx = (uint32_t)(kind == 0 ? k : (kind == 1 ? k - nv : k - nv - ne));
    for_bins(k, [&](uint64_t q) { out.items[cur[q]++] = (kind << 30) | idx; });
  }
  // bounding spheres (centre rounded to FP32, radius rounded up)
  out.sph.assign(4 * box.size(), 0.f);
  auto put = [&](size_t k, P3 c, double r) {
    out.sph[4 * k] = (float)c.x;
    out.sph[4 * k + 1] = (float)c.y;
    out.sph[4 * k + 2] = (float)c.z;
    out.sph[4 * k + 3] = (float)(r * (1.0 + 1e-6)) + 1e-6f;
  };
  for (int k = 0; k < nv; k++) put(k, V(k), 0.0);
  for (int k = 0; k < ne; k++) {
    const P3 a = V(m.e[2 * k]), d = sub3(V(m.e[2 * k + 1]), a);
    put((size_t)nv + k, axpy(a, 0.5, d), (0.5 + skin) * std::sqrt(dot3(d, d)));
  }
  for (int f = 0; f < nf; f++) {
    P3 cgm = {0, 0, 0};
    const int b0 = m.fo[f], nvf = m.fo[f + 1] - b0;
    for (int q = 0; q < nvf; q++) cgm = axpy(cgm, 1.0 / nvf, V(m.fv[b0 + q]));
    double r = 0.0;
    for (int q = 0; q < nvf; q++) r = std::max(r, dist3(cgm, V(m.fv[b0 + q])));
    put((size_t)nv + ne + f, cgm, r + flat[f]);  // the filter's projected polygon lies within flat[f] of the face
  }
  return OK;
}

}  // namespace meshbins
}  // namespace dem
