// dem_api.cu -- C ABI of the GB300 DEM hot path: context, memory, operator entry points.
//
// Each dem_* function stands in for one exaDEM operator (see include/dem_hotpath.h
// for the reference citations).  Host code only orchestrates: all per-particle
// and per-interaction work runs in the kernels of k_*.cu on the context's stream.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <numeric>
#include <unordered_map>
#include <vector>

#include "../../include/dem_learned.h"
#include "dem_ctx.cuh"
#include "poly_core.cuh"

using namespace dem;

namespace {

int check_params(dem_ctx* c, const dem_params* p) {
  if (!p) return c->fail(DEM_ERR_INVALID_ARG, "params is NULL");
  for (int d = 0; d < 3; d++)
    if (!(p->bounds_hi[d] > p->bounds_lo[d])) return c->fail(DEM_ERR_INVALID_ARG, "empty domain bounds");
  if (!(p->rcut_inc >= 0)) return c->fail(DEM_ERR_INVALID_ARG, "rcut_inc must be >= 0");
  if (!(p->dt > 0)) return c->fail(DEM_ERR_INVALID_ARG, "dt must be > 0");
  if (p->symetric != 1) return c->fail(DEM_ERR_UNSUPPORTED, "only symetric: true is supported");
  if (p->law != DEM_LAW_HOOKE_NONE && p->law != DEM_LAW_HOOKE_COHESIVE && p->law != DEM_LAW_HOOKE_DMT)
    return c->fail(DEM_ERR_UNSUPPORTED, "unknown contact law");
  if (p->law != DEM_LAW_HOOKE_COHESIVE && (p->config.dncut > 0 || p->config_driver.dncut > 0))
    return c->fail(DEM_ERR_INVALID_ARG,
                   "dncut is != 0 while the cohesive force is not used (contact_force_sphere.cu.in:280-292)");
  if (p->law == DEM_LAW_HOOKE_COHESIVE && (p->config.dncut == 0 || p->config_driver.dncut == 0))
    return c->fail(DEM_ERR_INVALID_ARG, "cohesive law needs dncut > 0");
  return DEM_OK;
}

// every particle group must index the multi-material table (the reference asserts it)
int check_multimat_groups(dem_ctx* c) {
  if (!c->mm_pp || !c->n) return DEM_OK;
  std::vector<uint32_t> g(c->n);
  DEM_CUDA_TRY(c, cudaMemcpy(g.data(), c->P[c->pcur].group, c->n * sizeof(uint32_t), cudaMemcpyDeviceToHost));
  for (uint32_t x : g)
    if (x >= (uint32_t)c->mm_ng) return c->fail(DEM_ERR_INVALID_ARG, "a particle group is outside the multi-material table");
  return DEM_OK;
}

void free_particles(dem_ctx* c) {
  for (int b = 0; b < 2; b++) {
    if (c->pblock[b]) cudaFree(c->pblock[b]);
    c->pblock[b] = nullptr;
    c->P[b] = PArrays{};
  }
  c->pcap = 0;
}

int alloc_particles(dem_ctx* c, uint64_t n) {
  if (n <= c->pcap && c->pblock[0]) return DEM_OK;
  free_particles(c);
  const uint64_t cap = std::max<uint64_t>(n, 1);
  const size_t per = NPF * sizeof(double) + sizeof(uint64_t) + 2 * sizeof(uint32_t);
  for (int b = 0; b < 2; b++) {
    DEM_CUDA_TRY(c, cudaMalloc(&c->pblock[b], per * cap + 1024));
    char* base = static_cast<char*>(c->pblock[b]);
    for (int f = 0; f < NPF; f++) c->P[b].f[f] = reinterpret_cast<double*>(base + (size_t)f * cap * sizeof(double));
    base += (size_t)NPF * cap * sizeof(double);
    c->P[b].id = reinterpret_cast<uint64_t*>(base);
    base += cap * sizeof(uint64_t);
    c->P[b].type = reinterpret_cast<uint32_t*>(base);
    base += cap * sizeof(uint32_t);
    c->P[b].group = reinterpret_cast<uint32_t*>(base);
  }
  // per-particle index arrays
  cudaFree(c->cell_of);
  cudaFree(c->cell_tmp);
  cudaFree(c->perm);
  cudaFree(c->pcnt);
  cudaFree(c->srec);
  cudaFree(c->rev_off);
  cudaFree(c->rev_cnt);
  cudaFree(c->rev_nlong);
  cudaFree(c->own_off[0]);
  cudaFree(c->own_off[1]);
  DEM_CUDA_TRY(c, cudaMalloc(&c->cell_of, cap * 4));
  DEM_CUDA_TRY(c, cudaMalloc(&c->cell_tmp, cap * 4));
  DEM_CUDA_TRY(c, cudaMalloc(&c->perm, cap * 4));
  DEM_CUDA_TRY(c, cudaMalloc(&c->pcnt, (cap + 1) * 4));
  DEM_CUDA_TRY(c, cudaMalloc(&c->srec, cap * 16 * 4));
  DEM_CUDA_TRY(c, cudaMalloc(&c->rev_off, (cap + 1) * 4));
  DEM_CUDA_TRY(c, cudaMalloc(&c->rev_cnt, (cap + 1) * 4));
  DEM_CUDA_TRY(c, cudaMalloc(&c->rev_nlong, sizeof(unsigned int)));
  DEM_CUDA_TRY(c, cudaMalloc(&c->own_off[0], (cap + 1) * 4));
  DEM_CUDA_TRY(c, cudaMalloc(&c->own_off[1], (cap + 1) * 4));
  for (int q = 0; q < 4; q++) {
    cudaFree(c->crel[q]);
    DEM_CUDA_TRY(c, cudaMalloc(&c->crel[q], cap * sizeof(float)));
  }
  cudaFree(c->rot_list);
  DEM_CUDA_TRY(c, cudaMalloc(&c->rot_list, cap * 4));
  c->pcap = cap;
  return DEM_OK;
}

void free_iarrays(IArrays& I) {
  cudaFree(I.owner);
  cudaFree(I.partner);
  cudaFree(I.pid);
  cudaFree(I.meta);
  cudaFree(I.sub);
  for (int d = 0; d < 3; d++) {
    cudaFree(I.ft[d]);
    cudaFree(I.mo[d]);
  }
  cudaFree(I.damp);
  I = IArrays{};
}

int alloc_iarrays(dem_ctx* c, int b, uint64_t need) {
  if (need <= c->icap[b] && c->I[b].owner) return DEM_OK;
  free_iarrays(c->I[b]);
  c->icap[b] = 0;
  const uint64_t cap = need + need / 4 + 4096;
  IArrays& I = c->I[b];
  DEM_CUDA_TRY(c, cudaMalloc(&I.owner, cap * 4));
  DEM_CUDA_TRY(c, cudaMalloc(&I.partner, cap * 4));
  DEM_CUDA_TRY(c, cudaMalloc(&I.pid, cap * 8));
  DEM_CUDA_TRY(c, cudaMalloc(&I.meta, cap * 4));
  DEM_CUDA_TRY(c, cudaMalloc(&I.sub, cap * 4));
  for (int d = 0; d < 3; d++) {
    DEM_CUDA_TRY(c, cudaMalloc(&I.ft[d], cap * 8));
    DEM_CUDA_TRY(c, cudaMalloc(&I.mo[d], cap * 8));
  }
  DEM_CUDA_TRY(c, cudaMalloc(&I.damp, cap * 8));
  c->icap[b] = cap;
  return DEM_OK;
}

void free_compact(dem_ctx* c) {
  cudaFree(c->L1);
  cudaFree(c->L2);
  c->L1 = c->L2 = nullptr;
  for (int q = 0; q < 7; q++) {
    cudaFree(c->Dscr[q]);
    c->Dscr[q] = nullptr;
  }
}

int ensure_contact_state(dem_ctx* c);

int alloc_records(dem_ctx* c, uint64_t need) {
  if (need <= c->rcap && c->rev_idx) return DEM_OK;
  for (int d = 0; d < 3; d++) {
    cudaFree(c->R.f[d]);
    cudaFree(c->R.ti[d]);
    cudaFree(c->R.tj[d]);
  }
  cudaFree(c->R.live);
  c->R = Records{};
  cudaFree(c->rev_idx);
  c->rev_idx = nullptr;
  free_compact(c);
  c->rcap = 0;
  const uint64_t cap = need + need / 4 + 4096;
  for (int d = 0; d < 3; d++) {
    DEM_CUDA_TRY(c, cudaMalloc(&c->R.f[d], cap * 8));
    DEM_CUDA_TRY(c, cudaMalloc(&c->R.ti[d], cap * 8));
    DEM_CUDA_TRY(c, cudaMalloc(&c->R.tj[d], cap * 8));
  }
  DEM_CUDA_TRY(c, cudaMalloc(&c->rev_idx, cap * 4));
  DEM_CUDA_TRY(c, cudaMalloc(&c->L1, cap * 4));
  DEM_CUDA_TRY(c, cudaMalloc(&c->L2, cap * 4));
  for (int q = 0; q < 7; q++) DEM_CUDA_TRY(c, cudaMalloc(&c->Dscr[q], cap * 8));
  DEM_CUDA_TRY(c, cudaMalloc(&c->R.live, cap));
  DEM_CUDA_TRY(c, cudaMemsetAsync(c->R.live, 1, cap, c->stream));
  c->rcap = cap;
  return ensure_contact_state(c);
}

void free_contact_state(dem_ctx* c) {
  cudaFree(c->cs.dn);
  for (int d = 0; d < 3; d++) {
    cudaFree(c->cs.cp[d]);
    cudaFree(c->cs.fn[d]);
    cudaFree(c->cs.ft[d]);
  }
  c->cs = ContactStateArrays{};
  c->cs_cap = 0;
}

// contact state arrays of the records' capacity while analysis is on
int ensure_contact_state(dem_ctx* c) {
  if (!c->analysis) {
    free_contact_state(c);
    return DEM_OK;
  }
  if (c->cs_cap >= c->rcap && c->cs.dn) return DEM_OK;
  free_contact_state(c);
  const uint64_t cap = std::max<uint64_t>(c->rcap, 1);
  DEM_CUDA_TRY(c, cudaMalloc(&c->cs.dn, cap * 8));
  for (int d = 0; d < 3; d++) {
    DEM_CUDA_TRY(c, cudaMalloc(&c->cs.cp[d], cap * 8));
    DEM_CUDA_TRY(c, cudaMalloc(&c->cs.fn[d], cap * 8));
    DEM_CUDA_TRY(c, cudaMalloc(&c->cs.ft[d], cap * 8));
  }
  c->cs_cap = cap;
  return DEM_OK;
}



// Cell grid: cell size >= nbh_dist = 2*r_max + rcut_inc (dem_rcut_max.cpp:60, config_globals.msp:35-37).
// Cell grid of one system: cs = max(cell_size, nbh_dist) with nbh_dist =
// 2 r_max + rcut_inc (dem_rcut_max.cpp:60, config_globals.msp:35-37);
// periodic axes get floor(L / cs) cells of L / dims, the others ceil(L / cs).
static int make_grid(dem_ctx* c, const double* lo, const double* hi, const int32_t* periodic, GridDev& g,
                     uint64_t& nc) {
  const dem_params& p = c->prm;
  const double nd = 2 * c->rad_max + p.rcut_inc;
  const double cs = std::max(p.cell_size, nd);
  if (!(cs > 0)) return c->fail(DEM_ERR_INVALID_ARG, "cell size must be > 0");
  g = GridDev{};
  nc = 1;
  for (int d = 0; d < 3; d++) {
    g.lo[d] = lo[d];
    g.hi[d] = hi[d];
    g.L[d] = hi[d] - lo[d];
    if (!(g.L[d] > 0)) return c->fail(DEM_ERR_INVALID_ARG, "empty domain");
    g.periodic[d] = periodic[d] ? 1 : 0;
    if (g.periodic[d]) {
      g.dims[d] = std::max(1, (int)std::floor(g.L[d] / cs));
      if (g.dims[d] < 3) return c->fail(DEM_ERR_INVALID_ARG, "periodic dimension needs at least 3 cells");
      g.csz[d] = g.L[d] / g.dims[d];
    } else {
      g.dims[d] = std::max(1, (int)std::ceil(g.L[d] / cs));
      g.csz[d] = cs;
    }
    nc *= (uint64_t)g.dims[d];
  }
  return DEM_OK;
}

// Grids of all systems, their cell offsets, particle and driver ranges, uploaded.
int setup_grid(dem_ctx* c) {
  const dem_params& p = c->prm;
  std::vector<dem_system> sys = c->systems;
  if (sys.empty()) {
    dem_system one{};
    one.first = 0;
    one.count = c->n;
    for (int d = 0; d < 3; d++) {
      one.bounds_lo[d] = p.bounds_lo[d];
      one.bounds_hi[d] = p.bounds_hi[d];
      one.periodic[d] = p.periodic[d];
    }
    one.driver_first = 0;
    one.driver_count = c->ndrv;
    sys.push_back(one);
  }
  const int ns = (int)sys.size();
  std::vector<GridDev> g(ns);
  std::vector<uint32_t> coff(ns + 1);
  std::vector<uint64_t> pfirst(ns + 1);
  std::vector<int2> dr(ns);
  uint64_t nc = 0;
  for (int k = 0; k < ns; k++) {
    uint64_t nck = 0;
    int rc = make_grid(c, sys[k].bounds_lo, sys[k].bounds_hi, sys[k].periodic, g[k], nck);
    if (rc) return rc;
    coff[k] = (uint32_t)nc;
    nc += nck;
    if (nc > (1ull << 31)) return c->fail(DEM_ERR_INVALID_ARG, "cell grid too large; raise cell_size");
    pfirst[k] = sys[k].first;
    dr[k] = make_int2(sys[k].driver_first, sys[k].driver_count);
  }
  coff[ns] = (uint32_t)nc;
  pfirst[ns] = c->n;
  if (ns > c->sys_cap) {
    cudaFree(c->grids_dev);
    cudaFree(c->coff_dev);
    cudaFree(c->pfirst_dev);
    cudaFree(c->drange_dev);
    cudaFree(c->trig_dev);
    c->grids_dev = nullptr;
    c->coff_dev = nullptr;
    c->pfirst_dev = nullptr;
    c->drange_dev = nullptr;
    c->trig_dev = nullptr;
    c->sys_cap = 0;
    DEM_CUDA_TRY(c, cudaMalloc(&c->grids_dev, ns * sizeof(GridDev)));
    DEM_CUDA_TRY(c, cudaMalloc(&c->coff_dev, (ns + 1) * sizeof(uint32_t)));
    DEM_CUDA_TRY(c, cudaMalloc(&c->pfirst_dev, (ns + 1) * sizeof(uint64_t)));
    DEM_CUDA_TRY(c, cudaMalloc(&c->drange_dev, ns * sizeof(int2)));
    DEM_CUDA_TRY(c, cudaMalloc(&c->trig_dev, ns * sizeof(uint32_t)));
    c->sys_cap = ns;
  }
  DEM_CUDA_TRY(c, cudaMemsetAsync(c->trig_dev, 0xff, ns * sizeof(uint32_t), c->stream));  // next rebuild: all
  DEM_CUDA_TRY(c, cudaMemcpyAsync(c->grids_dev, g.data(), ns * sizeof(GridDev), cudaMemcpyHostToDevice, c->stream));
  DEM_CUDA_TRY(c, cudaMemcpyAsync(c->coff_dev, coff.data(), (ns + 1) * 4, cudaMemcpyHostToDevice, c->stream));
  DEM_CUDA_TRY(c, cudaMemcpyAsync(c->pfirst_dev, pfirst.data(), (ns + 1) * 8, cudaMemcpyHostToDevice, c->stream));
  DEM_CUDA_TRY(c, cudaMemcpyAsync(c->drange_dev, dr.data(), ns * sizeof(int2), cudaMemcpyHostToDevice, c->stream));
  DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  c->nsys = ns;
  c->grid = g[0];
  c->ncell = nc;
  if (nc + 1 > c->ccap) {
    cudaFree(c->cell_cnt);
    cudaFree(c->cell_start);
    c->cell_cnt = c->cell_start = nullptr;
    c->ccap = 0;
    DEM_CUDA_TRY(c, cudaMalloc(&c->cell_cnt, (nc + 1) * 4));
    DEM_CUDA_TRY(c, cudaMalloc(&c->cell_start, (nc + 1) * 4));
    c->ccap = nc + 1;
  }
  return DEM_OK;
}

void free_poly(dem_ctx* c) {
  for (int d = 0; d < 3; d++) {
    cudaFree(c->vtx[d]);
    cudaFree(c->bvtx[d]);
    cudaFree(c->vrf[d]);
    cudaFree(c->vwf[d]);
    c->vtx[d] = c->bvtx[d] = nullptr;
    c->vrf[d] = c->vwf[d] = nullptr;
  }
  cudaFree(c->pobb);
  cudaFree(c->pfbox);
  cudaFree(c->pqb);
  cudaFree(c->vneed);
  cudaFree(c->vneed_off);
  cudaFree(c->vlist);
  cudaFree(c->u_off);
  cudaFree(c->urec);
  c->urec = nullptr;
  c->pobb = nullptr;
  c->pfbox = nullptr;
  c->pqb = nullptr;
  c->vneed = c->vneed_off = c->vlist = nullptr;
  c->nvlist = 0;
  c->u_off = nullptr;
  c->vcap = 0;
}

int alloc_poly(dem_ctx* c) {
  if (!c->poly) return DEM_OK;
  const uint64_t need = std::max<uint64_t>(c->n, 1) * (uint64_t)std::max(c->MV, 1);
  if (need <= c->vcap && c->pobb && c->u_off) return DEM_OK;
  free_poly(c);
  for (int d = 0; d < 3; d++) {
    DEM_CUDA_TRY(c, cudaMalloc(&c->vtx[d], need * 8));
    DEM_CUDA_TRY(c, cudaMalloc(&c->bvtx[d], need * 8));
    DEM_CUDA_TRY(c, cudaMalloc(&c->vrf[d], need * 4));
    DEM_CUDA_TRY(c, cudaMalloc(&c->vwf[d], need * 4));
  }
  DEM_CUDA_TRY(c, cudaMalloc(&c->pobb, std::max<uint64_t>(c->pcap, 1) * 15 * 8));
  DEM_CUDA_TRY(c, cudaMalloc(&c->urec, std::max<uint64_t>(c->pcap, 1) * 16 * 4));
  DEM_CUDA_TRY(c, cudaMalloc(&c->pfbox, std::max<uint64_t>(c->pcap, 1) * 32 * 4));
  DEM_CUDA_TRY(c, cudaMalloc(&c->pqb, std::max<uint64_t>(c->pcap, 1) * sizeof(float4)));
  DEM_CUDA_TRY(c, cudaMalloc(&c->vneed, (std::max<uint64_t>(c->pcap, 1) + 1) * 4));
  DEM_CUDA_TRY(c, cudaMalloc(&c->vneed_off, (std::max<uint64_t>(c->pcap, 1) + 1) * 4));
  DEM_CUDA_TRY(c, cudaMalloc(&c->vlist, std::max<uint64_t>(c->pcap, 1) * 4));
  DEM_CUDA_TRY(c, cudaMalloc(&c->u_off, (std::max<uint64_t>(c->pcap, 1) + 1) * 4));
  c->vcap = need;
  return DEM_OK;
}

void free_units(dem_ctx* c) {
  cudaFree(c->u_owner);
  cudaFree(c->u_partner);
  cudaFree(c->u_pid);
  cudaFree(c->u_kind);
  cudaFree(c->u_pass);
  cudaFree(c->u_slots);
  cudaFree(c->u_types);
  cudaFree(c->u_slotoff);
  cudaFree(c->u_order);
  cudaFree(c->u_x);
  cudaFree(c->u_rates);
  c->u_types = c->u_slotoff = c->u_order = nullptr;
  c->u_x = c->u_rates = nullptr;
  c->slot_cap = 0;
  cudaFree(c->f_cnt);
  cudaFree(c->f_off);
  cudaFree(c->u_rec);
  cudaFree(c->t_cnt);
  cudaFree(c->t_off);
  cudaFree(c->t_keep);
  c->u_rec = c->t_cnt = c->t_off = c->t_keep = nullptr;
  c->t_keepcap = 0;
  c->u_owner = c->u_partner = c->u_kind = c->f_cnt = c->f_off = nullptr;
  c->u_pid = nullptr;
  c->u_pass = nullptr;
  c->u_slots = nullptr;
  c->ucap = 0;
}

int grow_units(dem_ctx* c, uint64_t need) {
  if (need <= c->ucap && c->u_owner) return DEM_OK;
  free_units(c);
  const uint64_t cap = need + need / 4 + 1024;
  DEM_CUDA_TRY(c, cudaMalloc(&c->u_owner, cap * 4));
  DEM_CUDA_TRY(c, cudaMalloc(&c->u_partner, cap * 4));
  DEM_CUDA_TRY(c, cudaMalloc(&c->u_pid, cap * 8));
  DEM_CUDA_TRY(c, cudaMalloc(&c->u_kind, cap * 4));
  DEM_CUDA_TRY(c, cudaMalloc(&c->u_pass, cap));
  DEM_CUDA_TRY(c, cudaMalloc(&c->u_slots, cap * FEAT_SLOTS * sizeof(uint16_t)));
  c->slot_cap = cap * FEAT_SLOTS;
  DEM_CUDA_TRY(c, cudaMalloc(&c->u_types, cap * 4));
  DEM_CUDA_TRY(c, cudaMalloc(&c->u_slotoff, (cap + 1) * 4));
  DEM_CUDA_TRY(c, cudaMalloc(&c->u_order, cap * 4));
  DEM_CUDA_TRY(c, cudaMalloc(&c->u_x, cap * DEM_MLP_IN * sizeof(float)));
  DEM_CUDA_TRY(c, cudaMalloc(&c->u_rates, cap * DEM_MLP_OUT * sizeof(float)));
  DEM_CUDA_TRY(c, cudaMalloc(&c->f_cnt, (cap + 1) * 4));
  DEM_CUDA_TRY(c, cudaMalloc(&c->f_off, (cap + 1) * 4));
  DEM_CUDA_TRY(c, cudaMalloc(&c->u_rec, cap * 64));
  DEM_CUDA_TRY(c, cudaMalloc(&c->t_cnt, (6 * cap + 1) * 4));
  DEM_CUDA_TRY(c, cudaMalloc(&c->t_off, (6 * cap + 1) * 4));
  c->ucap = cap;
  return DEM_OK;
}

int alloc_records(dem_ctx* c, uint64_t need);
int alloc_iarrays(dem_ctx* c, int b, uint64_t need);

// nbh_polyhedron rebuild: bin + reorder, vertices/backup/OBBs, units, SAT, count, fill, reverse lists
int update_neighbors_poly(dem_ctx* c) {
  if (c->nsys != 1) return c->fail(DEM_ERR_UNSUPPORTED, "batched systems are implemented for spheres only");
  for (int d = 0; d < 3; d++)
    if (c->prm.periodic[d]) return c->fail(DEM_ERR_UNSUPPORTED, "periodic boundaries are not supported for polyhedra");
  if (c->n == 0) {
    c->ni = 0;
    c->have_list = true;
    return DEM_OK;
  }
  int rc;
  if ((rc = ensure_mesh_bins(c))) return rc;
  if ((rc = alloc_poly(c))) return rc;
  if ((rc = bonds_before_reorder(c))) return rc;  // broken bonds -> history, interfaces
  if ((rc = launch_bin_particles(c))) return rc;
  if ((rc = launch_reorder_particles(c))) return rc;
  if ((rc = bonds_after_reorder(c))) return rc;   // bonds follow the particles
  if ((rc = launch_poly_vertices(c, 2))) return rc;
  uint64_t nu = 0;
  if ((rc = launch_poly_units(c, &nu, grow_units))) return rc;
  c->learned_slots = false;
  if (c->prm.learned_sizing && c->prm.fp32_broad_phase && mlp_ready(c) && nu) {
    if ((rc = launch_unit_features(c, nu))) return rc;
    if ((rc = launch_learned_sizing(c, nu))) return rc;  // sets learned_slots
  }
  uint32_t total = 0;
  if ((rc = launch_poly_feature_count(c, nu, &total))) return rc;
  const int nw = 1 - c->icur;
  if ((rc = alloc_iarrays(c, nw, total))) return rc;
  if ((rc = alloc_records(c, total))) return rc;
  if ((rc = launch_poly_feature_fill(c, nu))) return rc;
  c->icur = nw;
  c->ni = total;
  c->have_list = true;
  c->hist_valid = true;
  if ((rc = launch_reverse_lists(c))) return rc;
  if ((rc = launch_vertex_list(c))) return rc;
  c->rebuilds++;
  return DEM_OK;
}

// every system rebuilds as if its own trigger fired (explicit neighbour updates)
int mark_all_triggered(dem_ctx* c) {
  DEM_CUDA_TRY(c, cudaMemsetAsync(c->trig_dev, 0xff, c->nsys * sizeof(uint32_t), c->stream));
  return DEM_OK;
}

int update_neighbors(dem_ctx* c) {
  c->gen++;  // buffers may move: a captured step graph is stale
  if (c->poly) {
    const int rc = update_neighbors_poly(c);
    return rc ? rc : mark_records_live(c);
  }
  if (c->n == 0) {
    c->ni = 0;
    c->have_list = true;
    return DEM_OK;
  }
  int rc;
  if (!c->capturing && (rc = ensure_mesh_bins(c))) return rc;
  if ((rc = launch_bin_particles(c))) return rc;
  if ((rc = launch_reorder_particles(c))) return rc;
  if ((rc = launch_count_sphere(c))) return rc;
  const int nw = 1 - c->icur;
  uint32_t* new_off = c->own_off[nw];
  if ((rc = scan_exclusive_u32(c, c->pcnt, new_off, c->n))) return rc;
  uint32_t total = 0;
  DEM_CUDA_TRY(c, cudaMemcpyAsync(&total, new_off + c->n, 4, cudaMemcpyDeviceToHost, c->stream));
  DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  if ((rc = alloc_iarrays(c, nw, total))) return rc;
  if ((rc = alloc_records(c, total))) return rc;
  if ((rc = launch_fill_sphere(c, new_off, total))) return rc;
  c->damp_stale = false;  // the new list's damping is that of the current parameters
  c->icur = nw;
  c->ni = total;
  c->have_list = true;
  c->hist_valid = true;
  if ((rc = launch_reverse_lists(c))) return rc;
  if ((rc = mark_records_live(c))) return rc;  // new list indices: every record is stale
  DEM_CUDA_TRY(c, cudaMemsetAsync(c->trig_dev, 0, c->nsys * sizeof(uint32_t), c->stream));
  c->rebuilds++;
  return DEM_OK;
}

// gravity, contact laws, gather; then the inner bonds (config_fragmentation.msp compute_force)
int compute_force(dem_ctx* c) {
  int rc;
  if ((rc = launch_gravity(c))) return rc;
  if ((rc = c->poly ? launch_contact_poly(c) : launch_contact_sphere(c))) return rc;
  if ((rc = launch_gather_forces(c))) return rc;
  return c->poly ? launch_bond_force(c) : DEM_OK;
}

int need_list(dem_ctx* c) {
  if (!c->have_list) return c->fail(DEM_ERR_STATE, "no interaction list: call dem_update_particle_neighbors first");
  return DEM_OK;
}

// Copies device scalar idx to the pinned host mirror and waits.
int read_flag(dem_ctx* c, int idx) {
  DEM_CUDA_TRY(c, cudaMemcpyAsync(c->h_scalars + idx, c->d_scalars + idx, sizeof(unsigned long long),
                                  cudaMemcpyDeviceToHost, c->stream));
  DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return DEM_OK;
}

int copy_field(dem_ctx* c, double* dst, const double* src, uint64_t n, cudaMemcpyKind k) {
  if (!dst || !src || !n) return DEM_OK;
  DEM_CUDA_TRY(c, cudaMemcpyAsync(dst, src, n * sizeof(double), k, c->stream));
  return DEM_OK;
}

}  // namespace

namespace dem {
int ext_alloc_iarrays(dem_ctx* c, int b, uint64_t need) { return alloc_iarrays(c, b, need); }
int ext_alloc_records(dem_ctx* c, uint64_t need) { return alloc_records(c, need); }
int ext_ensure_contact_state(dem_ctx* c) { return ensure_contact_state(c); }
// every record may be nonzero again (list rebuilt, state restored, or written by
// a kernel that does not keep the flags)
int mark_records_live(dem_ctx* c) {
  if (c->R.live && c->rcap) DEM_CUDA_TRY(c, cudaMemsetAsync(c->R.live, 1, c->rcap, c->stream));
  return DEM_OK;
}
void ext_free_iarrays(IArrays& I) { free_iarrays(I); }
int ext_update_neighbors(dem_ctx* c) {
  int rc = mark_all_triggered(c);
  return rc ? rc : update_neighbors(c);
}
int ext_setup_grid(dem_ctx* c) { return setup_grid(c); }
}  // namespace dem

extern "C" {

int dem_set_systems(dem_ctx* c, const dem_system* systems, int nsystems) {
  if (!c || !systems || nsystems < 1 || nsystems > DEM_MAX_SYSTEMS) return DEM_ERR_INVALID_ARG;
  if (c->poly) return c->fail(DEM_ERR_UNSUPPORTED, "batched systems are implemented for spheres only");
  // all systems rebuild when one triggers; with cohesion a rebuild off a system's
  // own schedule adds attracting pairs earlier than the system alone would
  if (nsystems > 1 && c->prm.law == DEM_LAW_HOOKE_COHESIVE)
    return c->fail(DEM_ERR_UNSUPPORTED, "batched systems need a law without cohesion");
  uint64_t next = 0;
  for (int k = 0; k < nsystems; k++) {
    const dem_system& q = systems[k];
    if (q.first != next || q.count == 0)
      return c->fail(DEM_ERR_INVALID_ARG, "systems must be non-empty consecutive particle ranges from 0");
    next += q.count;
    if (q.driver_first < 0 || q.driver_count < 0 || q.driver_first + q.driver_count > c->ndrv)
      return c->fail(DEM_ERR_INVALID_ARG, "system driver range outside the registered drivers");
    for (int d = 0; d < 3; d++)
      if (!(q.bounds_hi[d] > q.bounds_lo[d])) return c->fail(DEM_ERR_INVALID_ARG, "system with an empty domain");
  }
  if (next != c->n) return c->fail(DEM_ERR_INVALID_ARG, "systems must cover all particles");
  DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  c->gen++;
  const std::vector<dem_system> keep = c->systems;
  c->systems.assign(systems, systems + nsystems);
  int rc = setup_grid(c);
  if (rc) {
    c->systems = keep;
    return rc;
  }
  c->have_list = false;
  c->hist_valid = false;
  return DEM_OK;
}

int dem_system_count(dem_ctx* c, int* out) {
  if (!c || !out) return DEM_ERR_INVALID_ARG;
  *out = c->nsys;
  return DEM_OK;
}

int dem_simulation_state_systems(dem_ctx* c, dem_state* out, int nsystems) {
  if (!c || !out || nsystems != c->nsys) return DEM_ERR_INVALID_ARG;
  return launch_state_systems(c, out);
}


int dem_ctx_create(const dem_params* params, dem_ctx** out) {
  if (!out) return DEM_ERR_INVALID_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return DEM_ERR_NO_DEVICE;
  dem_ctx* c = new (std::nothrow) dem_ctx();
  if (!c) return DEM_ERR_OOM;
  int rc = check_params(c, params);
  if (rc) {
    delete c;
    return rc;
  }
  c->prm = *params;
  cudaGetDevice(&c->device);
  cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, c->device);
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMalloc(&c->d_scalars, DEM_NSCALARS * sizeof(unsigned long long)) != cudaSuccess ||
      cudaMallocHost(&c->h_scalars, 8 * sizeof(unsigned long long)) != cudaSuccess ||
      cudaMalloc(&c->drv_dev, DEM_MAX_DRIVERS * sizeof(DriverDev)) != cudaSuccess) {
    dem_ctx_destroy(c);
    return DEM_ERR_CUDA;
  }
  c->red_cap = std::max<uint64_t>(7ull * 2 * c->num_sms + 16, 4096);
  if (cudaMalloc(&c->d_red, c->red_cap * sizeof(double)) != cudaSuccess) {
    dem_ctx_destroy(c);
    return DEM_ERR_CUDA;
  }
  cudaMemset(c->d_scalars, 0, DEM_NSCALARS * sizeof(unsigned long long));
  for (int d = 0; d < 3; d++) c->grid.L[d] = c->prm.bounds_hi[d] - c->prm.bounds_lo[d];
  *out = c;
  return DEM_OK;
}

int dem_ctx_destroy(dem_ctx* c) {
  if (!c) return DEM_OK;
  if (c->stream) cudaStreamSynchronize(c->stream);
  cudaFree(c->mm_pp);
  cudaFree(c->mm_pd);
  free_contact_state(c);
  c->fold_events();
  for (cudaEvent_t e : c->ev_pool) cudaEventDestroy(e);
  c->ev_pool.clear();
  free_particles(c);
  for (int b = 0; b < 2; b++) {
    free_iarrays(c->I[b]);
    cudaFree(c->own_off[b]);
  }
  for (int d = 0; d < 3; d++) {
    cudaFree(c->R.f[d]);
    cudaFree(c->R.ti[d]);
    cudaFree(c->R.tj[d]);
  }
  cudaFree(c->R.live);
  cudaFree(c->rev_idx);
  free_compact(c);
  free_poly(c);
  free_units(c);
  free_bonds(c);
  cudaFree(c->shapes_dev);
  cudaFree(c->rev_off);
  cudaFree(c->rev_nlong);
  cudaFree(c->rev_cnt);
  cudaFree(c->cell_cnt);
  cudaFree(c->cell_start);
  cudaFree(c->cell_of);
  cudaFree(c->cell_tmp);
  cudaFree(c->perm);
  cudaFree(c->srec);
  cudaFree(c->pcnt);
  for (int q = 0; q < 4; q++) cudaFree(c->crel[q]);
  cudaFree(c->rot_list);
  cudaFree(c->scan_blk);
  cudaFree(c->d_scalars);
  cudaFree(c->d_red);
  free_graph(c);
  mlp_free(c);
  cudaFree(c->drv_dev);
  free_meshes(c);
  cudaFree(c->grids_dev);
  cudaFree(c->coff_dev);
  cudaFree(c->pfirst_dev);
  cudaFree(c->drange_dev);
  cudaFree(c->trig_dev);
  if (c->h_scalars) cudaFreeHost(c->h_scalars);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return DEM_OK;
}

const char* dem_last_error(const dem_ctx* c) { return c ? c->last_err.c_str() : "null context"; }

int dem_ctx_stream(dem_ctx* c, void** stream) {
  if (!c || !stream) return DEM_ERR_INVALID_ARG;
  *stream = (void*)c->stream;
  return DEM_OK;
}

int dem_set_params(dem_ctx* c, const dem_params* p) {
  if (!c || !p) return DEM_ERR_INVALID_ARG;
  if (c->systems.size() > 1 && p->law == DEM_LAW_HOOKE_COHESIVE)
    return c->fail(DEM_ERR_UNSUPPORTED, "batched systems need a law without cohesion");
  c->gen++;
  int rc = check_params(c, p);
  if (rc) return rc;
  if (std::memcmp(&p->config, &c->prm.config, sizeof(p->config)) ||
      std::memcmp(&p->config_driver, &c->prm.config_driver, sizeof(p->config_driver)))
    c->damp_stale = true;  // the per-pair damping of the current list (refresh_pair_damp)
  const bool grid_changed = std::memcmp(p->bounds_lo, c->prm.bounds_lo, sizeof(p->bounds_lo)) ||
                            std::memcmp(p->bounds_hi, c->prm.bounds_hi, sizeof(p->bounds_hi)) ||
                            std::memcmp(p->periodic, c->prm.periodic, sizeof(p->periodic)) ||
                            p->rcut_inc != c->prm.rcut_inc || p->cell_size != c->prm.cell_size;
  c->prm = *p;
  if (grid_changed && c->n) {
    if ((rc = setup_grid(c))) return rc;
    c->have_list = false;  // a new skin or domain needs a rebuild (history is kept by key)
  }
  return DEM_OK;
}

int dem_set_particles(dem_ctx* c, const dem_particles* p, int on_device) {
  if (!c || !p) return DEM_ERR_INVALID_ARG;
  if (p->n >= (1ull << 31)) return c->fail(DEM_ERR_INVALID_ARG, "too many particles");
  if (!p->rx || !p->ry || !p->rz || !p->radius)
    return c->fail(DEM_ERR_INVALID_ARG, "positions and radius are required");
  DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  c->gen++;
  const uint64_t n = p->n;
  int rc = alloc_particles(c, n);
  if (rc) return rc;
  c->pcur = 0;
  PArrays& P = c->P[0];
  const cudaMemcpyKind k = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  const double* src[NPF] = {p->rx, p->ry, p->rz, p->vx, p->vy, p->vz, p->fx, p->fy, p->fz, p->vrotx, p->vroty,
                            p->vrotz, p->arotx, p->aroty, p->arotz, p->momx, p->momy, p->momz, p->qw, p->qx,
                            p->qy, p->qz, p->inertiax, p->inertiay, p->inertiaz, p->mass, p->radius, p->homothety,
                            nullptr, nullptr, nullptr, nullptr, p->rx, p->ry, p->rz};
  // defaults for absent fields: 0, except orientation w, inertia, mass and homothety = 1
  std::vector<double> ones(n ? n : 1, 1.0);
  for (int f = 0; f < NPF; f++) {
    if (f >= IMASS && f <= IIZ) continue;  // derived below
    if (src[f]) {
      if ((rc = copy_field(c, P.f[f], src[f], n, k))) return rc;
    } else if (f == QW || f == IX || f == IY || f == IZ || f == MASS || f == HOM) {
      if ((rc = copy_field(c, P.f[f], ones.data(), n, cudaMemcpyHostToDevice))) return rc;
    } else if (n) {
      DEM_CUDA_TRY(c, cudaMemsetAsync(P.f[f], 0, n * sizeof(double), c->stream));
    }
  }
  std::vector<uint64_t> ids;
  if (p->id) {
    DEM_CUDA_TRY(c, cudaMemcpyAsync(P.id, p->id, n * 8, k, c->stream));
  } else if (n) {
    ids.resize(n);
    std::iota(ids.begin(), ids.end(), 0ull);
    DEM_CUDA_TRY(c, cudaMemcpyAsync(P.id, ids.data(), n * 8, cudaMemcpyHostToDevice, c->stream));
  }
  if (p->type) {
    DEM_CUDA_TRY(c, cudaMemcpyAsync(P.type, p->type, n * 4, k, c->stream));
  } else if (n) {
    DEM_CUDA_TRY(c, cudaMemsetAsync(P.type, 0, n * 4, c->stream));
  }
  if (p->group) {
    DEM_CUDA_TRY(c, cudaMemcpyAsync(P.group, p->group, n * 4, k, c->stream));
  } else if (n) {
    DEM_CUDA_TRY(c, cudaMemsetAsync(P.group, 0, n * 4, c->stream));
  }
  if ((rc = launch_reciprocals(c, n))) return rc;
  // r_max for nbh_dist (dem_rcut_max.cpp:49-66)
  std::vector<double> rad(n);
  if (n) {
    DEM_CUDA_TRY(c, cudaMemcpyAsync(rad.data(), P.f[RAD], n * 8, cudaMemcpyDeviceToHost, c->stream));
  }
  DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  double rmax = 0.0;
  for (double r : rad) rmax = std::max(rmax, r);
  c->rad_max = rmax;
  c->n = n;
  c->systems.clear();
  c->ni = 0;
  c->have_list = false;
  c->hist_valid = false;
  c->rebuilds = 0;
  clear_bonds(c);  // bonds refer to the particles they were made for
  if ((rc = alloc_poly(c))) return rc;
  if ((rc = check_multimat_groups(c))) return rc;
  return setup_grid(c);
}

int dem_set_multimat(dem_ctx* c, int ngroups, const dem_contact_params* pairs, int ndrivers,
                     const dem_contact_params* drivers) {
  if (!c || ngroups < 0 || ndrivers < 0) return DEM_ERR_INVALID_ARG;
  auto clear = [c]() {
    cudaFree(c->mm_pp);
    cudaFree(c->mm_pd);
    c->mm_pp = c->mm_pd = nullptr;
    c->mm_ng = c->mm_nd = 0;
  };
  c->gen++;  // the kernels of a captured step hold the old table
  c->damp_stale = true;
  if (ngroups == 0) {
    clear();
    return DEM_OK;
  }
  if (!pairs || (ndrivers > 0 && !drivers)) return DEM_ERR_INVALID_ARG;
  if (ndrivers != c->ndrv) return c->fail(DEM_ERR_INVALID_ARG, "ndrivers must equal the number of registered drivers");
  const size_t npp = (size_t)ngroups * ngroups, npd = (size_t)ngroups * ndrivers;
  for (int a = 0; a < ngroups; a++)
    for (int b = 0; b < ngroups; b++)
      if (std::memcmp(&pairs[a * ngroups + b], &pairs[b * ngroups + a], sizeof(dem_contact_params)))
        return c->fail(DEM_ERR_INVALID_ARG, "the pair table must be symmetric (register_multimat, multimat_parameters.hpp:181-186)");
  for (size_t k = 0; k < npp + npd; k++) {
    const dem_contact_params& q = k < npp ? pairs[k] : drivers[k - npp];
    if (c->prm.law != DEM_LAW_HOOKE_COHESIVE && q.dncut > 0)
      return c->fail(DEM_ERR_INVALID_ARG, "dncut is != 0 while the cohesive force is not used");
    if (c->prm.law == DEM_LAW_HOOKE_COHESIVE && q.dncut == 0)
      return c->fail(DEM_ERR_INVALID_ARG, "cohesive law needs dncut > 0");
  }
  clear();
  DEM_CUDA_TRY(c, cudaMalloc(&c->mm_pp, npp * sizeof(dem_contact_params)));
  DEM_CUDA_TRY(c, cudaMalloc(&c->mm_pd, std::max<size_t>(npd, 1) * sizeof(dem_contact_params)));
  DEM_CUDA_TRY(c, cudaMemcpy(c->mm_pp, pairs, npp * sizeof(dem_contact_params), cudaMemcpyHostToDevice));
  if (npd) DEM_CUDA_TRY(c, cudaMemcpy(c->mm_pd, drivers, npd * sizeof(dem_contact_params), cudaMemcpyHostToDevice));
  c->mm_ng = ngroups;
  c->mm_nd = ndrivers;
  const int rc = check_multimat_groups(c);
  if (rc) clear();
  return rc;
}

int dem_get_particles(dem_ctx* c, dem_particles* out, int on_device) {
  if (!c || !out) return DEM_ERR_INVALID_ARG;
  if (out->n < c->n) return c->fail(DEM_ERR_INVALID_ARG, "output arrays too small");
  const uint64_t n = c->n;
  const PArrays& P = c->P[c->pcur];
  const cudaMemcpyKind k = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  double* dst[NUSER] = {out->rx, out->ry, out->rz, out->vx, out->vy, out->vz, out->fx, out->fy, out->fz,
                     out->vrotx, out->vroty, out->vrotz, out->arotx, out->aroty, out->arotz, out->momx,
                     out->momy, out->momz, out->qw, out->qx, out->qy, out->qz, out->inertiax, out->inertiay,
                     out->inertiaz, out->mass, out->radius, out->homothety};
  int rc;
  for (int f = 0; f < NUSER; f++)
    if ((rc = copy_field(c, dst[f], P.f[f], n, k))) return rc;
  if (out->id && n) DEM_CUDA_TRY(c, cudaMemcpyAsync(out->id, P.id, n * 8, k, c->stream));
  if (out->type && n) DEM_CUDA_TRY(c, cudaMemcpyAsync(out->type, P.type, n * 4, k, c->stream));
  if (out->group && n) DEM_CUDA_TRY(c, cudaMemcpyAsync(out->group, P.group, n * 4, k, c->stream));
  DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  out->n = n;
  return DEM_OK;
}

static int add_driver(dem_ctx* c, const DriverDev& d) {
  if (c->ndrv >= DEM_MAX_DRIVERS) return c->fail(DEM_ERR_INVALID_ARG, "too many drivers");
  c->gen++;
  c->drv_host[c->ndrv] = d;
  DEM_CUDA_TRY(c, cudaMemcpyAsync(c->drv_dev + c->ndrv, &c->drv_host[c->ndrv], sizeof(DriverDev),
                                  cudaMemcpyHostToDevice, c->stream));
  DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  c->ndrv++;
  c->have_list = false;
  if (c->systems.empty() && c->n) return setup_grid(c);  // single system: all drivers
  return DEM_OK;
}


int dem_register_surface(dem_ctx* c, const dem_surface* s) {
  if (!c || !s) return DEM_ERR_INVALID_ARG;
  DriverDev d{};
  d.kind = 0;
  d.offset = s->offset;
  for (int k = 0; k < 3; k++) {
    d.normal[k] = s->normal[k];
    d.vel[k] = s->vel[k];
    d.vrot[k] = s->vrot[k];
    d.center_proj[k] = d.offset * d.normal[k];  // Surface::initialize (surface.hpp:138)
  }
  const bool vrot0 = s->vrot[0] == 0.0 && s->vrot[1] == 0.0 && s->vrot[2] == 0.0;
  const bool c0 = s->center[0] == 0.0 && s->center[1] == 0.0 && s->center[2] == 0.0;
  for (int k = 0; k < 3; k++) d.center[k] = (vrot0 && c0) ? d.offset * d.normal[k] : s->center[k];
  // Surface::initialize replaces a centre off the plane on the normal's side (surface.hpp:166-173)
  double off = 0.0, back = 0.0;
  off = (d.center[0] - d.center_proj[0]) * d.normal[0] + (d.center[1] - d.center_proj[1]) * d.normal[1] +
        (d.center[2] - d.center_proj[2]) * d.normal[2];
  if (off >= 1e-14) {
    back = (d.center_proj[0] - d.center[0]) * d.normal[0] + (d.center_proj[1] - d.center[1]) * d.normal[1] +
           (d.center_proj[2] - d.center[2]) * d.normal[2];
    for (int k = 0; k < 3; k++) d.center[k] = back * d.normal[k] + d.center_proj[k];
  }
  return add_driver(c, d);
}

int dem_register_cylinder(dem_ctx* c, const dem_cylinder* cy) {
  if (!c || !cy) return DEM_ERR_INVALID_ARG;
  if (!(cy->radius > 0)) return c->fail(DEM_ERR_INVALID_ARG, "cylinder radius must be > 0");
  DriverDev d{};
  d.kind = 1;
  d.radius = cy->radius;
  for (int k = 0; k < 3; k++) {
    d.axis[k] = cy->axis[k];
    d.center[k] = cy->axis[k] * cy->center[k];  // Cylinder::initialize (cylinder.hpp:89-99)
    d.vel[k] = cy->vel[k];
    d.vrot[k] = cy->vrot[k];
  }
  return add_driver(c, d);
}

int dem_particle_displ_over(dem_ctx* c, int* result) {
  if (!c || !result) return DEM_ERR_INVALID_ARG;
  int rc = launch_displ_over(c);
  if (rc) return rc;
  DEM_CUDA_TRY(c, cudaMemcpyAsync(c->h_scalars, c->d_scalars, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                                  c->stream));
  DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  *result = c->h_scalars[0] ? 1 : 0;
  return DEM_OK;
}

int dem_update_particle_neighbors(dem_ctx* c) {
  if (!c) return DEM_ERR_INVALID_ARG;
  int rc = mark_all_triggered(c);
  if (rc) return rc;
  return update_neighbors(c);
}

int dem_reset_force_moment(dem_ctx* c) {
  if (!c) return DEM_ERR_INVALID_ARG;
  return launch_reset_force_moment(c);
}

int dem_gravity_force(dem_ctx* c) {
  if (!c) return DEM_ERR_INVALID_ARG;
  return launch_gravity(c);
}

int dem_contact_sphere(dem_ctx* c) {
  if (!c) return DEM_ERR_INVALID_ARG;
  if (c->poly)
    return c->fail(DEM_ERR_STATE,
                   "The contact operator for spheres is being used, but polyhedron interactions are defined "
                   "(contact_force_sphere.cu.in:225-233)");
  int rc = need_list(c);
  if (rc) return rc;
  if ((rc = launch_contact_sphere(c))) return rc;
  return launch_gather_forces(c);
}

int dem_contact_polyhedron(dem_ctx* c) {
  if (!c) return DEM_ERR_INVALID_ARG;
  if (!c->poly) return c->fail(DEM_ERR_STATE, "no shapes: call dem_set_shapes first");
  int rc = need_list(c);
  if (rc) return rc;
  if ((rc = launch_contact_poly(c))) return rc;
  return launch_gather_forces(c);
}

int dem_compute_vertices(dem_ctx* c) {
  if (!c) return DEM_ERR_INVALID_ARG;
  if (!c->poly) return c->fail(DEM_ERR_STATE, "no shapes: call dem_set_shapes first");
  int rc = alloc_poly(c);
  if (rc) return rc;
  return launch_poly_vertices(c, 0);
}

int dem_vertex_displ_over(dem_ctx* c, int* result) {
  if (!c || !result) return DEM_ERR_INVALID_ARG;
  if (!c->poly) return c->fail(DEM_ERR_STATE, "no shapes: call dem_set_shapes first");
  if (!c->have_list) return c->fail(DEM_ERR_STATE, "no backup vertices: build the neighbour list first");
  int rc = launch_poly_vertices(c, 1);
  if (rc) return rc;
  if ((rc = read_flag(c, 0))) return rc;
  *result = c->h_scalars[0] ? 1 : 0;
  return DEM_OK;
}

int dem_set_shapes(dem_ctx* c, const dem_shape* shapes, int nshapes) {
  if (!c || !shapes || nshapes <= 0) return DEM_ERR_INVALID_ARG;
  if (!c->systems.empty()) return c->fail(DEM_ERR_UNSUPPORTED, "batched systems are implemented for spheres only");
  c->gen++;
  std::vector<ShapeDev> h(nshapes);
  int mv = 0;
  for (int k = 0; k < nshapes; k++) {
    const dem_shape& d = shapes[k];
    ShapeDev& o = h[k];
    std::memset(&o, 0, sizeof(o));
    if (d.nv < 1 || d.nv > SH_MAXV || d.ne < 0 || d.ne > SH_MAXE || d.nf < 0 || d.nf > SH_MAXF || !d.vertices ||
        (d.ne && !d.edges) || (d.nf && (!d.face_sizes || !d.face_vertices)))
      return c->fail(DEM_ERR_INVALID_ARG, "shape exceeds the supported sizes (32 vertices, 64 edges, 32 faces)");
    o.nv = d.nv;
    o.ne = d.ne;
    o.nf = d.nf;
    o.r = d.radius;
    double mx = 0;
    for (int i = 0; i < 3 * d.nv; i++) {
      o.v[i] = d.vertices[i];
      o.vf[i] = (float)d.vertices[i];
    }
    for (int i = 0; i < d.nv; i++)
      mx = std::max(mx, std::sqrt(o.v[3 * i] * o.v[3 * i] + o.v[3 * i + 1] * o.v[3 * i + 1] + o.v[3 * i + 2] * o.v[3 * i + 2]));
    o.maxv = mx;
    for (int i = 0; i < 2 * d.ne; i++) {
      if (d.edges[i] < 0 || d.edges[i] >= d.nv) return c->fail(DEM_ERR_INVALID_ARG, "edge vertex out of range");
      o.e[i] = d.edges[i];
    }
    int off = 0;
    for (int f = 0; f < d.nf; f++) {
      o.fo[f] = off;
      if (d.face_sizes[f] < 3 || off + d.face_sizes[f] > SH_MAXFV)
        return c->fail(DEM_ERR_INVALID_ARG, "face needs >= 3 vertices (128 face vertices at most)");
      for (int q = 0; q < d.face_sizes[f]; q++) {
        const int v = d.face_vertices[off + q];
        if (v < 0 || v >= d.nv) return c->fail(DEM_ERR_INVALID_ARG, "face vertex out of range");
        o.fv[off + q] = v;
      }
      off += d.face_sizes[f];
    }
    o.fo[d.nf] = off;
    for (int q = 0; q < 3; q++) {
      o.obb[q] = d.obb_center[q];
      o.obb[3 + q] = d.obb_e1[q];
      o.obb[6 + q] = d.obb_e2[q];
      o.obb[9 + q] = d.obb_e3[q];
      o.obb[12 + q] = d.obb_extent[q];
    }
    mv = std::max(mv, d.nv);
  }
  DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  cudaFree(c->shapes_dev);
  c->shapes_dev = nullptr;
  DEM_CUDA_TRY(c, cudaMalloc(&c->shapes_dev, sizeof(ShapeDev) * nshapes));
  DEM_CUDA_TRY(c, cudaMemcpy(c->shapes_dev, h.data(), sizeof(ShapeDev) * nshapes, cudaMemcpyHostToDevice));
  c->shapes_host.assign(reinterpret_cast<const char*>(h.data()),
                        reinterpret_cast<const char*>(h.data()) + sizeof(ShapeDev) * nshapes);
  c->nshapes = nshapes;
  if (mv != c->MV) free_poly(c);
  c->MV = mv;
  c->poly = true;
  c->have_list = false;
  c->hist_valid = false;
  return alloc_poly(c);
}

int dem_force_to_accel(dem_ctx* c) {
  if (!c) return DEM_ERR_INVALID_ARG;
  return launch_force_to_accel(c);
}

int dem_combined_compute_prolog(dem_ctx* c) {
  if (!c) return DEM_ERR_INVALID_ARG;
  return launch_prolog(c);
}

int dem_combined_compute_epilog(dem_ctx* c) {
  if (!c) return DEM_ERR_INVALID_ARG;
  return launch_epilog(c);
}

int dem_simulation_state(dem_ctx* c, dem_state* out) {
  if (!c || !out) return DEM_ERR_INVALID_ARG;
  return launch_state(c, out);
}

int dem_first_iteration(dem_ctx* c) {
  if (!c) return DEM_ERR_INVALID_ARG;
  int rc;
  if ((rc = mark_all_triggered(c))) return rc;
  if ((rc = update_neighbors(c))) return rc;
  if ((rc = launch_reset_force_moment(c))) return rc;
  return compute_force(c);
}

int dem_step(dem_ctx* c, int nsteps) {
  if (!c || nsteps < 0) return DEM_ERR_INVALID_ARG;
  int rc = need_list(c);
  if (rc) return rc;
  if (c->mm_pp && c->mm_nd != c->ndrv)
    return c->fail(DEM_ERR_STATE, "drivers were registered after dem_set_multimat: set the table again");
  if ((rc = refresh_pair_damp(c))) return rc;  // contact parameters changed since the list was built
  if ((rc = ensure_mesh_bins(c))) return rc;    // before a graph capture of the rebuild
  // graph replay unless per-kernel timing is on (events cannot be recorded inside a graph)
  if (c->prm.graph_step && c->prm.fused_step && !c->poly && nsteps > 0 && !c->prof_on) return step_graph(c, nsteps);
  for (int s = 0; s < nsteps; s++) {
    if (c->poly && c->prm.fused_step) {
      // prolog + vertex_displ_over decided in FP32; interface criterion (raises the
      // same flag); rebuild (all vertices) or the vertices of the particles in the
      // list and the bonds; contact; gather + f2a + epilog (with bonds: gather,
      // bond pass, f2a, epilog)
      if ((rc = launch_poly_fused_prolog(c))) return rc;
      if ((rc = launch_bond_criterion(c))) return rc;
      if ((rc = read_flag(c, 0))) return rc;
      if (c->h_scalars[0]) {
        if ((rc = update_neighbors(c))) return rc;
      } else if ((rc = launch_poly_vertices_listed(c))) {
        return rc;
      }
      if ((rc = launch_contact_poly(c))) return rc;
      if (c->nb) {
        if ((rc = launch_reset_force_moment(c))) return rc;
        if ((rc = launch_gravity(c))) return rc;
        if ((rc = launch_gather_forces(c))) return rc;
        if ((rc = launch_bond_force(c))) return rc;
        if ((rc = launch_force_to_accel(c))) return rc;
        if ((rc = launch_epilog(c))) return rc;
      } else if ((rc = launch_fused_epilog(c))) {
        return rc;
      }
      continue;
    }
    if (c->poly) {
      // prolog, vertices + vertex_displ_over, interface criterion, rebuild if
      // needed, forces, force_to_accel, epilog
      if ((rc = launch_prolog(c))) return rc;
      if ((rc = launch_poly_vertices(c, 1))) return rc;
      if ((rc = launch_bond_criterion(c))) return rc;
      if ((rc = read_flag(c, 0))) return rc;
      if (c->h_scalars[0] && (rc = update_neighbors(c))) return rc;
      if ((rc = launch_contact_poly(c))) return rc;
      if (c->prm.fused_step && !c->nb) {
        if ((rc = launch_fused_epilog(c))) return rc;
      } else {
        if ((rc = launch_reset_force_moment(c))) return rc;
        if ((rc = launch_gravity(c))) return rc;
        if ((rc = launch_gather_forces(c))) return rc;
        if ((rc = launch_bond_force(c))) return rc;
        if ((rc = launch_force_to_accel(c))) return rc;
        if ((rc = launch_epilog(c))) return rc;
      }
      continue;
    }
    if (c->prm.fused_step) {
      // prolog + trigger; rebuild if needed; three-pass contact; gather + f2a + epilog
      if ((rc = launch_fused_prolog(c))) return rc;
      if ((rc = read_flag(c, 0))) return rc;
      if (c->h_scalars[0] && (rc = update_neighbors(c))) return rc;
      if ((rc = launch_contact_compact(c))) return rc;
      if ((rc = launch_fused_epilog(c))) return rc;
      continue;
    }
    if ((rc = launch_prolog(c))) return rc;
    int over = 0;
    if ((rc = dem_particle_displ_over(c, &over))) return rc;
    if (over && (rc = update_neighbors(c))) return rc;
    if ((rc = launch_reset_force_moment(c))) return rc;
    if ((rc = compute_force(c))) return rc;
    if ((rc = launch_force_to_accel(c))) return rc;
    if ((rc = launch_epilog(c))) return rc;
  }
  DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return DEM_OK;
}

int dem_set_graph_capacity(dem_ctx* c, uint64_t capacity) {
  if (!c || capacity == 0) return DEM_ERR_INVALID_ARG;
  c->gcap = capacity;
  c->gen++;  // recapture with the new capacity
  return DEM_OK;
}

int dem_set_mul_mode(dem_ctx* c, int mode) {
  if (!c || mode < 0 || mode > 7) return DEM_ERR_INVALID_ARG;
  c->mul_mode = mode;
  c->gen++;  // a captured step holds the kernel instance of the old mode
  return DEM_OK;
}

int dem_set_contact_int_share(dem_ctx* c, int eighths) {
  if (!c || eighths < 0 || eighths > 8) return DEM_ERR_INVALID_ARG;
  c->tune_int_share = eighths;
  c->gen++;  // a captured step holds the kernel arguments of the old share
  return DEM_OK;
}

int dem_set_sphere_cell_broad_phase(dem_ctx* c, int on) {
  if (!c || on < 0 || on > 1) return DEM_ERR_INVALID_ARG;
  c->cell_broad_phase = on;
  c->gen++;  // a captured step holds the broad-phase kernels of the old choice
  return DEM_OK;
}

int dem_get_mul_mode(dem_ctx* c, int* mode) {
  if (!c || !mode) return DEM_ERR_INVALID_ARG;
  *mode = c->mul_mode;
  return DEM_OK;
}

int dem_rebuild_count(dem_ctx* c, uint64_t* out) {
  if (!c || !out) return DEM_ERR_INVALID_ARG;
  *out = c->rebuilds;
  return DEM_OK;
}

int dem_interaction_count(dem_ctx* c, uint64_t* out) {
  if (!c || !out) return DEM_ERR_INVALID_ARG;
  *out = c->ni;
  return DEM_OK;
}

// read_dump_particle_interaction: the history of a saved list, installed as the
// previous list of the particles currently set, for the next build to carry over
int dem_set_interactions(dem_ctx* c, const dem_interaction_list* l) {
  if (!c || !l) return DEM_ERR_INVALID_ARG;
  const uint64_t m = l->count, n = c->n;
  if (m && (!l->owner_id || !l->partner_id || !l->type || !l->swap || !l->owner_sub || !l->partner_sub ||
            !l->friction || !l->moment))
    return c->fail(DEM_ERR_INVALID_ARG, "set_interactions: every array of the list is needed");
  if (m >= (1ull << 31)) return c->fail(DEM_ERR_INVALID_ARG, "set_interactions: too many interactions");
  DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  std::vector<uint64_t> id(n);
  if (n) DEM_CUDA_TRY(c, cudaMemcpy(id.data(), c->P[c->pcur].id, n * 8, cudaMemcpyDeviceToHost));
  std::unordered_map<uint64_t, uint32_t> slot;
  slot.reserve(n * 2 + 1);
  for (uint64_t s2 = 0; s2 < n; s2++)
    if (!slot.emplace(id[s2], (uint32_t)s2).second) return c->fail(DEM_ERR_INVALID_ARG, "set_interactions: duplicate particle id");
  auto driver_base = [&](uint32_t sl) -> uint64_t {  // inverse of dem_get_interactions' per-system driver index
    if (c->systems.empty()) return 0;
    size_t lo = 0, hi = c->systems.size() - 1;
    while (lo < hi) {
      const size_t mid = (lo + hi + 1) / 2;
      if (c->systems[mid].first <= sl)
        lo = mid;
      else
        hi = mid - 1;
    }
    return (uint64_t)c->systems[lo].driver_first;
  };
  struct Row {
    uint32_t owner, partner, meta, sub;
    uint64_t pid;
    double h[6];
  };
  std::vector<Row> rows(m);
  for (uint64_t k = 0; k < m; k++) {
    const auto it = slot.find(l->owner_id[k]);
    if (it == slot.end()) return c->fail(DEM_ERR_INVALID_ARG, "set_interactions: owner id is not a particle");
    Row& r = rows[k];
    r.owner = it->second;
    const uint32_t t = l->type[k];
    const bool drv = t == DEM_ITYPE_VERTEX_CYLINDER || t == DEM_ITYPE_VERTEX_SURFACE ||
                     (t >= DEM_ITYPE_VERTEX_MESH_VERTEX && t <= DEM_ITYPE_MESH_VERTEX_FACE);
    if (drv) {
      r.pid = l->partner_id[k] + driver_base(r.owner);
      if (r.pid >= (uint64_t)c->ndrv) return c->fail(DEM_ERR_INVALID_ARG, "set_interactions: unknown driver");
      r.partner = (uint32_t)r.pid;
    } else {
      const auto jt = slot.find(l->partner_id[k]);
      if (jt == slot.end()) return c->fail(DEM_ERR_INVALID_ARG, "set_interactions: partner id is not a particle");
      r.pid = l->partner_id[k];
      r.partner = jt->second;
    }
    r.meta = (t & 0xffu) | ((uint32_t)(l->swap[k] & 1u) << 15);
    const uint32_t ps = l->partner_sub[k] == 0xffffffffu ? 0xffffu : (l->partner_sub[k] & 0xffffu);
    r.sub = (l->owner_sub[k] & 0xffffu) | (ps << 16);
    for (int d = 0; d < 3; d++) {
      r.h[d] = l->friction[3 * k + d];
      r.h[3 + d] = l->moment[3 * k + d];
    }
  }
  // the order the builds' binary searches assume inside an owner: spheres (partner id, type, sub),
  // polyhedra (partner id, type, swap, owner sub, partner sub)
  auto skey = [](const Row& r) {
    return ((uint64_t)(r.meta & 0xffu) << 48) | ((uint64_t)((r.meta >> 15) & 1u) << 40) |
           ((uint64_t)(r.sub & 0xffffu) << 20) | (uint64_t)(r.sub >> 16);
  };
  const bool poly = c->poly;
  std::stable_sort(rows.begin(), rows.end(), [&](const Row& a, const Row& b) {
    if (a.owner != b.owner) return a.owner < b.owner;
    if (a.pid != b.pid) return a.pid < b.pid;
    if (poly) return skey(a) < skey(b);
    if ((a.meta & 0xffu) != (b.meta & 0xffu)) return (a.meta & 0xffu) < (b.meta & 0xffu);
    return a.sub < b.sub;
  });
  const int b = c->icur;
  int rc = alloc_iarrays(c, b, m);
  if (rc) return rc;
  std::vector<uint32_t> owner(m), partner(m), meta(m), sub(m), off(n + 1, 0);
  std::vector<uint64_t> pid(m);
  std::vector<double> h[6];
  for (int q = 0; q < 6; q++) h[q].resize(m);
  for (uint64_t k = 0; k < m; k++) {
    owner[k] = rows[k].owner;
    partner[k] = rows[k].partner;
    meta[k] = rows[k].meta;
    sub[k] = rows[k].sub;
    pid[k] = rows[k].pid;
    for (int q = 0; q < 6; q++) h[q][k] = rows[k].h[q];
    off[rows[k].owner + 1]++;
  }
  for (uint64_t s2 = 0; s2 < n; s2++) off[s2 + 1] += off[s2];
  const IArrays& I = c->I[b];
  if (m) {
    DEM_CUDA_TRY(c, cudaMemcpy(I.owner, owner.data(), m * 4, cudaMemcpyHostToDevice));
    DEM_CUDA_TRY(c, cudaMemcpy(I.partner, partner.data(), m * 4, cudaMemcpyHostToDevice));
    DEM_CUDA_TRY(c, cudaMemcpy(I.meta, meta.data(), m * 4, cudaMemcpyHostToDevice));
    DEM_CUDA_TRY(c, cudaMemcpy(I.sub, sub.data(), m * 4, cudaMemcpyHostToDevice));
    DEM_CUDA_TRY(c, cudaMemcpy(I.pid, pid.data(), m * 8, cudaMemcpyHostToDevice));
    for (int d = 0; d < 3; d++) {
      DEM_CUDA_TRY(c, cudaMemcpy(I.ft[d], h[d].data(), m * 8, cudaMemcpyHostToDevice));
      DEM_CUDA_TRY(c, cudaMemcpy(I.mo[d], h[3 + d].data(), m * 8, cudaMemcpyHostToDevice));
    }
    DEM_CUDA_TRY(c, cudaMemset(I.damp, 0, m * 8));
  }
  DEM_CUDA_TRY(c, cudaMemcpy(c->own_off[b], off.data(), (n + 1) * 4, cudaMemcpyHostToDevice));
  c->ni = m;
  c->gen++;
  c->damp_stale = true;  // the installed list carries no damping
  c->have_list = false;  // the next build makes the list; this one only holds the history
  c->hist_valid = true;
  return mark_all_triggered(c);
}

int dem_get_interactions(dem_ctx* c, dem_interaction_list* l) {
  if (!c || !l) return DEM_ERR_INVALID_ARG;
  l->count = c->ni;
  if (l->capacity < c->ni) return c->fail(DEM_ERR_INVALID_ARG, "interaction list capacity too small");
  const uint64_t ni = c->ni, n = c->n;
  std::vector<uint32_t> owner(ni), meta(ni), sub(ni);
  std::vector<uint64_t> pid(ni), id(n);
  std::vector<double> h[6];
  const IArrays& I = c->I[c->icur];
  for (int k = 0; k < 6; k++) h[k].resize(ni);
  if (ni) {
    DEM_CUDA_TRY(c, cudaMemcpyAsync(owner.data(), I.owner, ni * 4, cudaMemcpyDeviceToHost, c->stream));
    DEM_CUDA_TRY(c, cudaMemcpyAsync(meta.data(), I.meta, ni * 4, cudaMemcpyDeviceToHost, c->stream));
    DEM_CUDA_TRY(c, cudaMemcpyAsync(sub.data(), I.sub, ni * 4, cudaMemcpyDeviceToHost, c->stream));
    DEM_CUDA_TRY(c, cudaMemcpyAsync(pid.data(), I.pid, ni * 8, cudaMemcpyDeviceToHost, c->stream));
    for (int d = 0; d < 3; d++) {
      DEM_CUDA_TRY(c, cudaMemcpyAsync(h[d].data(), I.ft[d], ni * 8, cudaMemcpyDeviceToHost, c->stream));
      DEM_CUDA_TRY(c, cudaMemcpyAsync(h[3 + d].data(), I.mo[d], ni * 8, cudaMemcpyDeviceToHost, c->stream));
    }
  }
  if (n) DEM_CUDA_TRY(c, cudaMemcpyAsync(id.data(), c->P[c->pcur].id, n * 8, cudaMemcpyDeviceToHost, c->stream));
  DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  // owners' segments are contiguous and key-sorted inside; order the segments by owner id
  std::vector<uint64_t> seg_start;
  for (uint64_t k = 0; k < ni; k++)
    if (k == 0 || owner[k] != owner[k - 1]) seg_start.push_back(k);
  std::vector<size_t> order(seg_start.size());
  std::iota(order.begin(), order.end(), 0);
  std::sort(order.begin(), order.end(),
            [&](size_t a, size_t b) { return id[owner[seg_start[a]]] < id[owner[seg_start[b]]]; });
  // driver partners are stored by global driver index; report the index inside
  // the owner's system (each system numbers its drivers from 0, as a run of its own)
  auto driver_base = [&](uint32_t slot) -> uint64_t {
    if (c->systems.empty()) return 0;
    size_t lo = 0, hi = c->systems.size() - 1;
    while (lo < hi) {
      const size_t mid = (lo + hi + 1) / 2;
      if (c->systems[mid].first <= slot)
        lo = mid;
      else
        hi = mid - 1;
    }
    return (uint64_t)c->systems[lo].driver_first;
  };
  uint64_t w = 0;
  for (size_t o : order) {
    const uint64_t b = seg_start[o], e = (o + 1 < seg_start.size()) ? seg_start[o + 1] : ni;
    for (uint64_t k = b; k < e; k++, w++) {
      if (l->owner_id) l->owner_id[w] = id[owner[k]];
      if (l->partner_id) {
        const uint32_t t = meta_type(meta[k]);
        const bool drv = t == DEM_ITYPE_VERTEX_CYLINDER || t == DEM_ITYPE_VERTEX_SURFACE ||
                         (t >= DEM_ITYPE_VERTEX_MESH_VERTEX && t <= DEM_ITYPE_VERTEX_MESH_FACE);
        l->partner_id[w] = drv ? pid[k] - driver_base(owner[k]) : pid[k];
      }
      if (l->type) l->type[w] = (uint16_t)meta_type(meta[k]);
      if (l->swap) l->swap[w] = (uint8_t)((meta[k] >> 15) & 1u);
      if (l->owner_sub) l->owner_sub[w] = sub[k] & 0xffffu;
      if (l->partner_sub) l->partner_sub[w] = (sub[k] >> 16) == 0xffffu ? 0xffffffffu : (sub[k] >> 16);
      if (l->friction)
        for (int d = 0; d < 3; d++) l->friction[3 * w + d] = h[d][k];
      if (l->moment)
        for (int d = 0; d < 3; d++) l->moment[3 * w + d] = h[3 + d][k];
    }
  }
  return DEM_OK;
}

int dem_profile(dem_ctx* c, int enable) {
  if (!c) return DEM_ERR_INVALID_ARG;
  c->prof_on = enable != 0;
  return DEM_OK;
}

int dem_kernel_stats(dem_ctx* c, dem_kernel_stat* out, int capacity, int* count) {
  if (!c || !count) return DEM_ERR_INVALID_ARG;
  DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  c->fold_events();
  int m = 0;
  for (int k = 0; k < K_NCLASS; k++) {
    if (out && m < capacity) {
      std::memset(out[m].name, 0, sizeof(out[m].name));
      std::strncpy(out[m].name, kDemKClassNames[k], sizeof(out[m].name) - 1);
      out[m].launches = c->launches[k];
      out[m].timed = c->prof_n[k];
      out[m].total_ms = c->prof_ms[k];
    }
    m++;
  }
  *count = m;
  return DEM_OK;
}

int dem_reset_kernel_stats(dem_ctx* c) {
  if (!c) return DEM_ERR_INVALID_ARG;
  DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  c->fold_events();
  for (int k = 0; k < K_NCLASS; k++) {
    c->launches[k] = 0;
    c->prof_ms[k] = 0;
    c->prof_n[k] = 0;
  }
  return DEM_OK;
}

int dem_packing_profile(dem_ctx* c, int nslabs, double zlo, double zhi, double* out) {
  if (!c || !out || nslabs <= 0 || !(zhi > zlo)) return DEM_ERR_INVALID_ARG;
  return launch_profile(c, nslabs, zlo, zhi, out);
}

}  // extern "C"

// add_driver for dem_register_mesh (k_mesh.cu)
namespace dem {
int ext_add_driver(dem_ctx* c, const DriverDev& d) { return add_driver(c, d); }
}  // namespace dem
