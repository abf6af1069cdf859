// k_mesh.cu -- mesh drivers (register_stl_mesh / register_rshape,
// register_stl_mesh.cpp:40-147, rshape.hpp:104-420).
//
// The reference lists, per grid cell, the mesh features whose enlarged OBB
// meets the cell (grid_rshape_driver, grid_stl_mesh.cpp:30-265), and a sphere
// keeps the features of its cell that pass their Verlet filter
// (nbh_sphere.hpp:25-86).  With cells that cover the filter range that list
// is the set of features passing the filter, which is what is built here: a
// uniform bin grid of its own over the mesh lists, per bin, every feature whose
// filter can pass for a point of the bin (a sphere centre, a polyhedron vertex
// or edge point: the feature's box enlarged by the filter range with the
// largest particle radius, with a margin for rounding), and the neighbour pass
// runs the exact filter on the features of the bins it visits.
#include <algorithm>
#include <cmath>
#include <vector>

#include "../../include/dem_hotpath.h"
#include "dem_ctx.cuh"
#include "integrate_core.cuh"

namespace dem {
namespace {

// shape::get_vertex(i, center, 1.0, quat) = center + quat * (1.0 * v)
__global__ void k_mesh_world(const double* __restrict__ v0, uint64_t nv, Q4 q, V3 c, double* __restrict__ out) {
  const uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nv) return;
  const V3 v = mk(v0[3 * k], v0[3 * k + 1], v0[3 * k + 2]);
  const V3 w = c + qrotate(q, 1.0 * v);
  out[k] = w.x;
  out[nv + k] = w.y;
  out[2 * nv + k] = w.z;
}

struct Box {
  double lo[3], hi[3];
};

// ---- host geometry for the bin lists (distances from a bin centre)
struct P3 {
  double x, y, z;
};
inline P3 sub3(P3 a, P3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline double dot3(P3 a, P3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline P3 axpy(P3 a, double t, P3 d) { return {a.x + t * d.x, a.y + t * d.y, a.z + t * d.z}; }
inline double dist3(P3 a, P3 b) { return std::sqrt(dot3(sub3(a, b), sub3(a, b))); }
// distance from c to the segment a + t (b - a), t in [t0, t1]
double seg_dist(P3 c, P3 a, P3 b, double t0, double t1) {
  const P3 d = sub3(b, a);
  const double dd = dot3(d, d);
  double t = dd > 0.0 ? dot3(sub3(c, a), d) / dd : 0.0;
  t = std::min(std::max(t, t0), t1);
  return dist3(c, axpy(a, t, d));
}
// distance from c to the triangle abc (closest point on a triangle, Ericson's
// Real-Time Collision Detection 5.1.5)
double tri_dist(P3 p, P3 a, P3 b, P3 c) {
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

// bins of one mesh for spheres of radius <= rad and the skin
int build_bins(dem_ctx* c, MeshStore& m, double rad, double skin) {
  const int nv = m.dev.nv, ne = m.dev.ne, nf = m.dev.nf;
  const double E = rad + m.dev.r + skin;  // Rmax of the vertex, edge and face filters
  double amax = 0.0;
  for (int k = 0; k < nv; k++)
    amax = std::max(amax, std::max(std::fabs(m.hx[k]), std::max(std::fabs(m.hy[k]), std::fabs(m.hz[k]))));
  std::vector<Box> box;
  box.reserve((size_t)nv + ne + nf);
  auto grow = [&](Box& b, double x, double y, double z) {
    b.lo[0] = std::min(b.lo[0], x);
    b.lo[1] = std::min(b.lo[1], y);
    b.lo[2] = std::min(b.lo[2], z);
    b.hi[0] = std::max(b.hi[0], x);
    b.hi[1] = std::max(b.hi[1], y);
    b.hi[2] = std::max(b.hi[2], z);
  };
  auto empty = [] { return Box{{HUGE_VAL, HUGE_VAL, HUGE_VAL}, {-HUGE_VAL, -HUGE_VAL, -HUGE_VAL}}; };
  // vertices: |p - v| <= E
  for (int k = 0; k < nv; k++) {
    Box b = empty();
    grow(b, m.hx[k], m.hy[k], m.hz[k]);
    box.push_back(b);
  }
  // edges: p = vf + r (vs - vf) + d with r in [-skin, 1 + skin] and |d| < E
  // (filter_vertex_edge_core compares the line parameter r with rVerlet)
  double span = 0.0;
  for (int k = 0; k < ne; k++) {
    const int a = m.he[2 * k], s = m.he[2 * k + 1];
    const double d[3] = {m.hx[s] - m.hx[a], m.hy[s] - m.hy[a], m.hz[s] - m.hz[a]};
    Box b = empty();
    for (double t : {-skin, 1.0 + skin}) grow(b, m.hx[a] + t * d[0], m.hy[a] + t * d[1], m.hz[a] + t * d[2]);
    span = std::max(span, std::max(b.hi[0] - b.lo[0], std::max(b.hi[1] - b.lo[1], b.hi[2] - b.lo[2])));
    box.push_back(b);
  }
  // faces: p within E of the face's plane, projected inside the face
  for (int k = 0; k < nf; k++) {
    Box b = empty();
    for (int q = m.hfo[k]; q < m.hfo[k + 1]; q++) grow(b, m.hx[m.hfv[q]], m.hy[m.hfv[q]], m.hz[m.hfv[q]]);
    box.push_back(b);
  }
  const double margin = 1e-7 * (E + amax + span) + 1e-12;
  Box all = empty();
  for (Box& b : box) {
    for (int d = 0; d < 3; d++) {
      b.lo[d] -= E + margin;
      b.hi[d] += E + margin;
    }
    grow(all, b.lo[0], b.lo[1], b.lo[2]);
    grow(all, b.hi[0], b.hi[1], b.hi[2]);
  }
  MeshDev& D = m.dev;
  if (box.empty() || !(std::isfinite(all.lo[0]) && std::isfinite(all.hi[0]) && std::isfinite(all.lo[1]) &&
                       std::isfinite(all.hi[1]) && std::isfinite(all.lo[2]) && std::isfinite(all.hi[2])))
    return c->fail(DEM_ERR_INVALID_ARG, "mesh: non-finite vertices");
  // bin size: about the filter range, at most 2^22 bins (each axis below 2^21)
  double ext = std::max(all.hi[0] - all.lo[0], std::max(all.hi[1] - all.lo[1], all.hi[2] - all.lo[2]));
  double bs = std::max(E, ext / 256.0);
  int dims[3];
  for (;;) {
    uint64_t tot = 1;
    for (int d = 0; d < 3; d++) {
      dims[d] = (int)std::floor((all.hi[d] - all.lo[d]) * (1.0 / bs)) + 1;
      tot *= (uint64_t)dims[d];
    }
    if (tot <= (1u << 22)) break;
    bs *= 1.5;
  }
  for (int d = 0; d < 3; d++) D.lo[d] = all.lo[d];
  D.inv_bs = 1.0 / bs;
  for (int d = 0; d < 3; d++) D.dims[d] = dims[d];
  // the bin range of a box: the index formula of mesh_bin_of (mesh_core.cuh), monotone in the coordinate
  auto index = [&](double x, int d) {
    const double f = (x - D.lo[d]) * D.inv_bs;
    return std::min(std::max((int)std::floor(f), 0), dims[d] - 1);
  };
  const uint64_t nb = (uint64_t)dims[0] * dims[1] * dims[2];
  std::vector<uint32_t> cnt(nb + 1, 0);
  // a bin lists a feature when its centre is within E + margin + half its
  // diagonal of the feature's region (vertex; edge segment extended by the skin
  // in its parameter; face polygon, fan-split: a superset for a non-convex one),
  // which holds for every bin holding a point that passes the filter
  const double reach = E + 2.0 * margin + 0.8660254037844387 * bs * (1.0 + 1e-12);
  auto near = [&](size_t k, P3 ctr) {
    if (k < (size_t)nv) return dist3(ctr, {m.hx[k], m.hy[k], m.hz[k]}) <= reach;
    if (k < (size_t)nv + ne) {
      const int a = m.he[2 * (k - nv)], b = m.he[2 * (k - nv) + 1];
      return seg_dist(ctr, {m.hx[a], m.hy[a], m.hz[a]}, {m.hx[b], m.hy[b], m.hz[b]}, -skin, 1.0 + skin) <= reach;
    }
    const int f = (int)(k - nv - ne), b0 = m.hfo[f], nvf = m.hfo[f + 1] - b0;
    const int i0 = m.hfv[b0];
    const P3 a = {m.hx[i0], m.hy[i0], m.hz[i0]};
    for (int q = 1; q + 1 < nvf; q++) {
      const int i1 = m.hfv[b0 + q], i2 = m.hfv[b0 + q + 1];
      if (tri_dist(ctr, a, {m.hx[i1], m.hy[i1], m.hz[i1]}, {m.hx[i2], m.hy[i2], m.hz[i2]}) <= reach) return true;
    }
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
          const P3 ctr = {D.lo[0] + (x + 0.5) * bs, D.lo[1] + (y + 0.5) * bs, D.lo[2] + (z + 0.5) * bs};
          if (near(k, ctr)) f((uint64_t)x + (uint64_t)dims[0] * ((uint64_t)y + (uint64_t)dims[1] * z));
        }
  };
  uint64_t total = 0;
  for (size_t k = 0; k < box.size(); k++)
    for_bins(k, [&](uint64_t q) {
      cnt[q + 1]++;
      total++;
    });
  if (total >= (1ull << 32)) return c->fail(DEM_ERR_OVERFLOW, "mesh: too many bin entries");
  for (uint64_t q = 0; q < nb; q++) cnt[q + 1] += cnt[q];
  std::vector<uint32_t> items(total);
  std::vector<uint32_t> cur(cnt.begin(), cnt.end() - 1);
  // in (kind, index) order: vertices, edges, faces
  for (size_t k = 0; k < box.size(); k++) {
    const uint32_t kind = k < (size_t)nv ? 0u : (k < (size_t)nv + ne ? 1u : 2u);
    const uint32_t idx = (uint32_t)(kind == 0 ? k : (kind == 1 ? k - nv : k - nv - ne));
    for_bins(k, [&](uint64_t q) { items[cur[q]++] = (kind << 30) | idx; });
  }
  cudaFree(m.boff);
  cudaFree(m.bitem);
  cudaFree(m.fsph);
  m.boff = nullptr;
  m.bitem = nullptr;
  m.fsph = nullptr;
  // bounding spheres of the features (centre rounded to FP32, radius rounded up)
  std::vector<float4> sph(box.size());
  auto put = [&](size_t k, double x, double y, double z, double r) {
    sph[k] = make_float4((float)x, (float)y, (float)z, (float)(r * (1.0 + 1e-6)) + 1e-6f);
  };
  for (int k = 0; k < nv; k++) put(k, m.hx[k], m.hy[k], m.hz[k], 0.0);
  for (int k = 0; k < ne; k++) {
    const int a = m.he[2 * k], b = m.he[2 * k + 1];
    const P3 pa = {m.hx[a], m.hy[a], m.hz[a]}, d = sub3({m.hx[b], m.hy[b], m.hz[b]}, pa);
    const P3 mid = axpy(pa, 0.5, d);
    put((size_t)nv + k, mid.x, mid.y, mid.z, (0.5 + skin) * std::sqrt(dot3(d, d)));
  }
  for (int f = 0; f < nf; f++) {
    P3 cgm = {0, 0, 0};
    const int b0 = m.hfo[f], nvf = m.hfo[f + 1] - b0;
    for (int q = 0; q < nvf; q++) cgm = axpy(cgm, 1.0 / nvf, {m.hx[m.hfv[b0 + q]], m.hy[m.hfv[b0 + q]], m.hz[m.hfv[b0 + q]]});
    double r = 0.0;
    for (int q = 0; q < nvf; q++) r = std::max(r, dist3(cgm, {m.hx[m.hfv[b0 + q]], m.hy[m.hfv[b0 + q]], m.hz[m.hfv[b0 + q]]}));
    put((size_t)nv + ne + f, cgm.x, cgm.y, cgm.z, r);
  }
  DEM_CUDA_TRY(c, cudaMalloc(&m.fsph, sph.size() * sizeof(float4)));
  DEM_CUDA_TRY(c, cudaMemcpyAsync(m.fsph, sph.data(), sph.size() * sizeof(float4), cudaMemcpyHostToDevice, c->stream));
  D.fsph = m.fsph;
  DEM_CUDA_TRY(c, cudaMalloc(&m.boff, (nb + 1) * 4));
  DEM_CUDA_TRY(c, cudaMalloc(&m.bitem, std::max<uint64_t>(total, 1) * 4));
  DEM_CUDA_TRY(c, cudaMemcpyAsync(m.boff, cnt.data(), (nb + 1) * 4, cudaMemcpyHostToDevice, c->stream));
  if (total)
    DEM_CUDA_TRY(c, cudaMemcpyAsync(m.bitem, items.data(), total * 4, cudaMemcpyHostToDevice, c->stream));
  DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  D.boff = m.boff;
  D.bitem = m.bitem;
  m.bin_rad = rad;
  m.bin_skin = skin;
  return DEM_OK;
}

int upload_mesh_table(dem_ctx* c) {
  cudaFree(c->mesh_dev);
  c->mesh_dev = nullptr;
  if (c->meshes.empty()) return DEM_OK;
  std::vector<MeshDev> h;
  for (const MeshStore& m : c->meshes) h.push_back(m.dev);
  DEM_CUDA_TRY(c, cudaMalloc(&c->mesh_dev, h.size() * sizeof(MeshDev)));
  DEM_CUDA_TRY(c, cudaMemcpyAsync(c->mesh_dev, h.data(), h.size() * sizeof(MeshDev), cudaMemcpyHostToDevice,
                                  c->stream));
  DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return DEM_OK;
}
}  // namespace

int ensure_mesh_bins(dem_ctx* c) {
  if (!c->meshes.empty() && !c->poly && c->mesh_cnt_cap < std::max<uint64_t>(c->pcap, 1)) {
    if (c->capturing) return c->fail(DEM_ERR_STATE, "mesh count buffer too small inside a graph capture");
    cudaFree(c->mesh_cnt);
    c->mesh_cnt = nullptr;
    c->mesh_cnt_cap = 0;
    const uint64_t cap = std::max<uint64_t>(c->pcap, 1);
    DEM_CUDA_TRY(c, cudaMalloc(&c->mesh_cnt, cap * 4));
    c->mesh_cnt_cap = cap;
    c->gen++;  // captured kernels hold the old buffer
  }
  if (!c->meshes.empty() && c->poly && c->prm.learned_sizing)
    return c->fail(DEM_ERR_UNSUPPORTED, "learned record sizing does not bound mesh units: learned_sizing = 0");
  bool changed = false;
  const double rad = c->rad_max, skin = c->prm.rcut_inc;
  for (MeshStore& m : c->meshes) {
    // bins built for a larger radius bound and skin list a superset: still exact
    if (m.boff && m.bin_rad >= rad && m.bin_skin >= skin) continue;
    if (c->capturing) return c->fail(DEM_ERR_STATE, "mesh bins are stale inside a graph capture");
    const int rc = build_bins(c, m, rad, skin);
    if (rc) return rc;
    changed = true;
  }
  if (!changed) return DEM_OK;
  c->gen++;  // captured kernels hold the old mesh table
  return upload_mesh_table(c);
}

void free_meshes(dem_ctx* c) {
  for (MeshStore& m : c->meshes) {
    cudaFree(m.vtx);
    cudaFree(m.e);
    cudaFree(m.fo);
    cudaFree(m.fv);
    cudaFree(m.boff);
    cudaFree(m.bitem);
    cudaFree(m.fsph);
  }
  c->meshes.clear();
  cudaFree(c->mesh_dev);
  c->mesh_dev = nullptr;
  cudaFree(c->mesh_cnt);
  c->mesh_cnt = nullptr;
  c->mesh_cnt_cap = 0;
}
}  // namespace dem

using namespace dem;

extern "C" int dem_register_mesh(dem_ctx* c, const dem_mesh* s) {
  if (!c || !s) return DEM_ERR_INVALID_ARG;
  const int nv = s->nv, ne = s->ne, nf = s->nf;
  if (nv < 0 || ne < 0 || nf < 0 || nv + ne + nf == 0)
    return c->fail(DEM_ERR_INVALID_ARG, "mesh: no vertex, no edge and no face (RShape::initialize)");
  if (nv >= 0xffff || ne >= 0xffff || nf >= 0xffff)
    return c->fail(DEM_ERR_UNSUPPORTED, "mesh: 65535 or more vertices, edges or faces");
  if ((nv && !s->vertices) || (ne && !s->edges) || (nf && (!s->face_offsets || !s->face_vertices)))
    return c->fail(DEM_ERR_INVALID_ARG, "mesh: missing arrays");
  if (!(s->minkowski >= 0.0) || !std::isfinite(s->minkowski))
    return c->fail(DEM_ERR_INVALID_ARG, "mesh: Minkowski radius must be finite and >= 0");
  for (int k = 0; k < 3 * nv; k++)
    if (!std::isfinite(s->vertices[k])) return c->fail(DEM_ERR_INVALID_ARG, "mesh: non-finite vertex");
  for (int k = 0; k < 2 * ne; k++)
    if (s->edges[k] < 0 || s->edges[k] >= nv) return c->fail(DEM_ERR_INVALID_ARG, "mesh: edge vertex out of range");
  if (nf && s->face_offsets[0] != 0) return c->fail(DEM_ERR_INVALID_ARG, "mesh: face_offsets[0] must be 0");
  for (int k = 0; k < nf; k++)
    if (s->face_offsets[k + 1] - s->face_offsets[k] < 3)
      return c->fail(DEM_ERR_INVALID_ARG, "mesh: a face needs at least 3 vertices");
  const int nfv = nf ? s->face_offsets[nf] : 0;
  for (int k = 0; k < nfv; k++)
    if (s->face_vertices[k] < 0 || s->face_vertices[k] >= nv)
      return c->fail(DEM_ERR_INVALID_ARG, "mesh: face vertex out of range");
  const Q4 q{s->quat[0], s->quat[1], s->quat[2], s->quat[3]};
  const V3 ctr = mk(s->center[0], s->center[1], s->center[2]);
  for (double x : {q.w, q.x, q.y, q.z, ctr.x, ctr.y, ctr.z})
    if (!std::isfinite(x)) return c->fail(DEM_ERR_INVALID_ARG, "mesh: non-finite center or quaternion");

  MeshStore m;
  m.dev.nv = nv;
  m.dev.ne = ne;
  m.dev.nf = nf;
  m.dev.r = s->minkowski;
  double* v0 = nullptr;
  auto fail_free = [&](int rc) {
    cudaFree(v0);
    cudaFree(m.vtx);
    cudaFree(m.e);
    cudaFree(m.fo);
    cudaFree(m.fv);
    return rc;
  };
  const size_t vb = (size_t)std::max(nv, 1) * 3 * sizeof(double);
  if (cudaMalloc(&m.vtx, vb) != cudaSuccess || cudaMalloc(&v0, vb) != cudaSuccess ||
      cudaMalloc(&m.e, (size_t)std::max(2 * ne, 1) * 4) != cudaSuccess ||
      cudaMalloc(&m.fo, (size_t)(nf + 1) * 4) != cudaSuccess ||
      cudaMalloc(&m.fv, (size_t)std::max(nfv, 1) * 4) != cudaSuccess)
    return fail_free(c->fail(DEM_ERR_CUDA, "mesh: device allocation failed"));
  m.he.assign(s->edges, s->edges + 2 * ne);
  m.hfo.assign(1, 0);
  if (nf) m.hfo.assign(s->face_offsets, s->face_offsets + nf + 1);
  m.hfv.assign(s->face_vertices, s->face_vertices + nfv);
  bool ok = true;
  if (nv) ok = ok && cudaMemcpyAsync(v0, s->vertices, (size_t)nv * 24, cudaMemcpyHostToDevice, c->stream) == cudaSuccess;
  if (ne) ok = ok && cudaMemcpyAsync(m.e, m.he.data(), (size_t)ne * 8, cudaMemcpyHostToDevice, c->stream) == cudaSuccess;
  ok = ok && cudaMemcpyAsync(m.fo, m.hfo.data(), m.hfo.size() * 4, cudaMemcpyHostToDevice, c->stream) == cudaSuccess;
  if (nfv) ok = ok && cudaMemcpyAsync(m.fv, m.hfv.data(), (size_t)nfv * 4, cudaMemcpyHostToDevice, c->stream) == cudaSuccess;
  if (nv) {
    k_mesh_world<<<(unsigned)((nv + 255) / 256), 256, 0, c->stream>>>(v0, (uint64_t)nv, q, ctr, m.vtx);
    ok = ok && cudaGetLastError() == cudaSuccess;
  }
  m.hx.resize(nv);
  m.hy.resize(nv);
  m.hz.resize(nv);
  if (nv) {
    ok = ok && cudaMemcpyAsync(m.hx.data(), m.vtx, (size_t)nv * 8, cudaMemcpyDeviceToHost, c->stream) == cudaSuccess;
    ok = ok && cudaMemcpyAsync(m.hy.data(), m.vtx + nv, (size_t)nv * 8, cudaMemcpyDeviceToHost, c->stream) == cudaSuccess;
    ok = ok && cudaMemcpyAsync(m.hz.data(), m.vtx + 2 * (size_t)nv, (size_t)nv * 8, cudaMemcpyDeviceToHost,
                               c->stream) == cudaSuccess;
  }
  ok = ok && cudaStreamSynchronize(c->stream) == cudaSuccess;
  cudaFree(v0);
  v0 = nullptr;
  if (!ok) return fail_free(c->fail(DEM_ERR_CUDA, "mesh: upload failed"));
  m.dev.x = m.vtx;
  m.dev.y = m.vtx + nv;
  m.dev.z = m.vtx + 2 * (size_t)nv;
  m.dev.e = m.e;
  m.dev.fo = m.fo;
  m.dev.fv = m.fv;
  if (c->ndrv >= DEM_MAX_DRIVERS) return fail_free(c->fail(DEM_ERR_INVALID_ARG, "too many drivers"));
  DriverDev d{};
  d.kind = 2;
  d.mesh = (int)c->meshes.size();
  for (int k = 0; k < 3; k++) d.center[k] = s->center[k];  // driver.position(); velocities 0 (STATIONARY)
  c->meshes.push_back(m);
  MeshStore& mm = c->meshes.back();
  mm.dev.boff = nullptr;  // built by the next neighbour pass (ensure_mesh_bins)
  int rc = upload_mesh_table(c);
  if (rc) return rc;
  return ext_add_driver(c, d);
}
