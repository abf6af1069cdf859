// k_analysis.cu -- contact state readback and the stress tensor
// (stress_tensor.cu:30-160, classifier/contact_state.hpp:22-50).
#include <algorithm>
#include <numeric>
#include <vector>

#include "../../include/dem_hotpath.h"
#include "dem_ctx.cuh"

namespace dem {
namespace {

// m += u v^T (exanb::tensor, row major), added component by component
__device__ __forceinline__ void add_tensor(double* m, V3 u, V3 v) {
  m[0] = m[0] + u.x * v.x;
  m[1] = m[1] + u.x * v.y;
  m[2] = m[2] + u.x * v.z;
  m[3] = m[3] + u.y * v.x;
  m[4] = m[4] + u.y * v.y;
  m[5] = m[5] + u.y * v.z;
  m[6] = m[6] + u.z * v.x;
  m[7] = m[7] + u.z * v.y;
  m[8] = m[8] + u.z * v.z;
}

// ComputeStressTensorFunc (stress_tensor.cu:40-75) for every pair of a particle:
// its own pairs, then those where it is the partner (the canonical order of
// the force gather); a pair counts when dn < 0.  The state is in the contact
// law's frame: its particle i (I.i() = pi_) takes +(fn + ft), its particle j
// -(fn + ft).  pi_ is the owner unless the polyhedron pair is swapped
// (interaction_pair.hpp:70-112; swap = bit 15 of meta, nullptr for spheres).
__global__ void k_stress(PArrays P, ContactStateArrays cs, const uint32_t* __restrict__ meta,
                         const uint32_t* __restrict__ own_off, const uint32_t* __restrict__ rev_off,
                         const uint32_t* __restrict__ rev_idx, uint64_t n, double* __restrict__ out) {
  const uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const V3 r = mk(P.f[RX][s], P.f[RY][s], P.f[RZ][s]);
  double m[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (uint32_t k = own_off[s]; k < own_off[s + 1]; k++) {
    if (!(cs.dn[k] < 0.0)) continue;
    const V3 fij = mk(cs.fn[0][k], cs.fn[1][k], cs.fn[2][k]) + mk(cs.ft[0][k], cs.ft[1][k], cs.ft[2][k]);
    const V3 cij = mk(cs.cp[0][k], cs.cp[1][k], cs.cp[2][k]) - r;
    const bool swap = meta && ((meta[k] >> 15) & 1u);
    add_tensor(m, swap ? -fij : fij, cij);
  }
  for (uint32_t q = rev_off[s]; q < rev_off[s + 1]; q++) {
    const uint32_t k = rev_idx[q];
    if (!(cs.dn[k] < 0.0)) continue;
    const V3 fij = mk(cs.fn[0][k], cs.fn[1][k], cs.fn[2][k]) + mk(cs.ft[0][k], cs.ft[1][k], cs.ft[2][k]);
    const V3 cji = mk(cs.cp[0][k], cs.cp[1][k], cs.cp[2][k]) - r;
    const bool swap = meta && ((meta[k] >> 15) & 1u);
    add_tensor(m, swap ? fij : -fij, cji);
  }
  for (int c = 0; c < 9; c++) out[9 * s + c] = m[c];
}

int need_analysis(dem_ctx* c) {
  if (!c->analysis || !c->cs.dn) return c->fail(DEM_ERR_STATE, "analysis is off: dem_set_analysis(ctx, 1) before the step");
  if (!c->have_list) return c->fail(DEM_ERR_STATE, "no interaction list");
  return DEM_OK;
}
}  // namespace
}  // namespace dem

using namespace dem;

extern "C" int dem_set_analysis(dem_ctx* c, int on) {
  if (!c) return DEM_ERR_INVALID_ARG;
  c->analysis = on != 0;
  c->gen++;  // captured kernels hold the old state pointers
  return ext_ensure_contact_state(c);
}

extern "C" int dem_get_contact_state(dem_ctx* c, dem_contact_state* out) {
  if (!c || !out) return DEM_ERR_INVALID_ARG;
  int rc = need_analysis(c);
  if (rc) return rc;
  const uint64_t ni = c->ni, n = c->n;
  out->count = ni;
  if (out->capacity < ni) return c->fail(DEM_ERR_INVALID_ARG, "contact state capacity too small");
  std::vector<uint32_t> owner(ni);
  std::vector<uint64_t> id(n);
  std::vector<double> h[10];
  for (auto& v : h) v.resize(ni);
  if (ni) {
    DEM_CUDA_TRY(c, cudaMemcpyAsync(owner.data(), c->I[c->icur].owner, ni * 4, cudaMemcpyDeviceToHost, c->stream));
    DEM_CUDA_TRY(c, cudaMemcpyAsync(h[0].data(), c->cs.dn, ni * 8, cudaMemcpyDeviceToHost, c->stream));
    for (int d = 0; d < 3; d++) {
      DEM_CUDA_TRY(c, cudaMemcpyAsync(h[1 + d].data(), c->cs.cp[d], ni * 8, cudaMemcpyDeviceToHost, c->stream));
      DEM_CUDA_TRY(c, cudaMemcpyAsync(h[4 + d].data(), c->cs.fn[d], ni * 8, cudaMemcpyDeviceToHost, c->stream));
      DEM_CUDA_TRY(c, cudaMemcpyAsync(h[7 + d].data(), c->cs.ft[d], ni * 8, cudaMemcpyDeviceToHost, c->stream));
    }
  }
  if (n) DEM_CUDA_TRY(c, cudaMemcpyAsync(id.data(), c->P[c->pcur].id, n * 8, cudaMemcpyDeviceToHost, c->stream));
  DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  // the order of dem_get_interactions: owners by id, each owner's pairs in key order
  std::vector<uint64_t> seg;
  for (uint64_t k = 0; k < ni; k++)
    if (k == 0 || owner[k] != owner[k - 1]) seg.push_back(k);
  std::vector<size_t> order(seg.size());
  std::iota(order.begin(), order.end(), 0);
  std::sort(order.begin(), order.end(), [&](size_t a, size_t b) { return id[owner[seg[a]]] < id[owner[seg[b]]]; });
  uint64_t w = 0;
  for (size_t o : order) {
    const uint64_t b = seg[o], e = (o + 1 < seg.size()) ? seg[o + 1] : ni;
    for (uint64_t k = b; k < e; k++, w++) {
      if (out->dn) out->dn[w] = h[0][k];
      for (int d = 0; d < 3; d++) {
        if (out->cp) out->cp[3 * w + d] = h[1 + d][k];
        if (out->fn) out->fn[3 * w + d] = h[4 + d][k];
        if (out->ft) out->ft[3 * w + d] = h[7 + d][k];
      }
    }
  }
  return DEM_OK;
}

extern "C" int dem_stress_tensor(dem_ctx* c, double* stress, double* total) {
  if (!c) return DEM_ERR_INVALID_ARG;
  int rc = need_analysis(c);
  if (rc) return rc;
  const uint64_t n = c->n;
  std::vector<double> h(9 * n);
  std::vector<uint64_t> id(n);
  if (n) {
    double* d = nullptr;
    DEM_CUDA_TRY(c, cudaMalloc(&d, 9 * n * sizeof(double)));
    const uint32_t* meta = c->poly ? c->I[c->icur].meta : nullptr;
    k_stress<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(c->P[c->pcur], c->cs, meta, c->own_off[c->icur],
                                                                  c->rev_off, c->rev_idx, n, d);
    const cudaError_t e = cudaGetLastError();
    DEM_CUDA_TRY(c, cudaMemcpyAsync(h.data(), d, 9 * n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    DEM_CUDA_TRY(c, cudaMemcpyAsync(id.data(), c->P[c->pcur].id, n * 8, cudaMemcpyDeviceToHost, c->stream));
    DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    cudaFree(d);
    if (e != cudaSuccess) return c->fail(DEM_ERR_CUDA, cudaGetErrorString(e));
  }
  if (stress) std::copy(h.begin(), h.end(), stress);
  if (total) {
    std::vector<uint64_t> by_id(n);
    std::iota(by_id.begin(), by_id.end(), 0);
    std::sort(by_id.begin(), by_id.end(), [&](uint64_t a, uint64_t b) { return id[a] < id[b]; });
    for (int q = 0; q < 9; q++) total[q] = 0.0;
    for (uint64_t s : by_id)
      for (int q = 0; q < 9; q++) total[q] = total[q] + h[9 * s + q];
  }
  return DEM_OK;
}
