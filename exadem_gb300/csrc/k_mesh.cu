// k_mesh.cu -- mesh drivers (register_stl_mesh / register_rshape,
// register_stl_mesh.cpp:40-147, rshape.hpp:104-420): registration, world
// vertices, and the upload of the feature bins that mesh_bins.hpp builds.
#include <algorithm>
#include <cmath>
#include <vector>

#include "../../include/dem_hotpath.h"
#include "dem_ctx.cuh"
#include "integrate_core.cuh"
#include "mesh_bins.hpp"

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

// bins of one mesh for particles of radius <= rad and the skin (mesh_bins.hpp), uploaded
int build_bins(dem_ctx* c, MeshStore& m, double rad, double skin) {
  meshbins::Input in{m.dev.nv, m.dev.ne, m.dev.nf, m.hx.data(), m.hy.data(), m.hz.data(),
                     m.he.data(), m.hfo.data(), m.hfv.data(), m.dev.r};
  meshbins::Output o;
  const int rc = meshbins::build(in, rad, skin, o);
  if (rc == meshbins::NONFINITE) return c->fail(DEM_ERR_INVALID_ARG, "mesh: non-finite vertices");
  if (rc == meshbins::OVERFLOW_) return c->fail(DEM_ERR_OVERFLOW, "mesh: too many bin entries");
  MeshDev& D = m.dev;
  for (int d = 0; d < 3; d++) {
    D.lo[d] = o.lo[d];
    D.dims[d] = o.dims[d];
  }
  D.inv_bs = o.inv_bs;
  cudaFree(m.boff);
  cudaFree(m.bitem);
  cudaFree(m.fsph);
  m.boff = nullptr;
  m.bitem = nullptr;
  m.fsph = nullptr;
  const uint64_t nb1 = o.boff.size(), total = o.items.size(), nfeat = o.sph.size() / 4;
  DEM_CUDA_TRY(c, cudaMalloc(&m.fsph, std::max<uint64_t>(nfeat, 1) * sizeof(float4)));
  DEM_CUDA_TRY(c, cudaMalloc(&m.boff, nb1 * 4));
  DEM_CUDA_TRY(c, cudaMalloc(&m.bitem, std::max<uint64_t>(total, 1) * 4));
  if (nfeat)
    DEM_CUDA_TRY(c, cudaMemcpyAsync(m.fsph, o.sph.data(), nfeat * sizeof(float4), cudaMemcpyHostToDevice, c->stream));
  DEM_CUDA_TRY(c, cudaMemcpyAsync(m.boff, o.boff.data(), nb1 * 4, cudaMemcpyHostToDevice, c->stream));
  if (total) DEM_CUDA_TRY(c, cudaMemcpyAsync(m.bitem, o.items.data(), total * 4, cudaMemcpyHostToDevice, c->stream));
  DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  D.fsph = m.fsph;
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
  const int ndrv0 = c->ndrv;
  c->meshes.push_back(m);
  MeshStore& mm = c->meshes.back();
  mm.dev.boff = nullptr;  // built by the next neighbour pass (ensure_mesh_bins)
  int rc = upload_mesh_table(c);
  if (rc == DEM_OK) rc = ext_add_driver(c, d);
  if (rc && c->ndrv == ndrv0) {
    // the driver was not added: take the mesh back out so that no mesh is left without its driver
    MeshStore gone = c->meshes.back();
    c->meshes.pop_back();
    cudaFree(gone.vtx);
    cudaFree(gone.e);
    cudaFree(gone.fo);
    cudaFree(gone.fv);
    upload_mesh_table(c);
  }
  return rc;
}
