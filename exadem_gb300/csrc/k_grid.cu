// k_grid.cu -- cell binning and particle reorder at a neighbour rebuild.
//
// Stands in for exaNBody's move_particles / migrate_cell_particles / grid
// (periodic wrap into the domain, particles stored cell by cell).  Steps:
//   k_bin:       periodic wrap, cell index, cell histogram (atomics on counts)
//   scan:        cell starts
//   k_scatter:   slot of each particle inside its cell (atomic cursor)
//   k_cell_sort: order inside one cell by particle id, so the layout is
//                deterministic whatever order the atomics ran in
//   k_reorder:   gather every field into the other particle buffer
// All of it is integer / copy work: HBM-bound, one read and one write per field.
// Batched contexts: each system bins into its own block of the cell index
// space, so the sort keeps every particle inside its system's slot range.
#include "dem_ctx.cuh"

namespace dem {
namespace {

__global__ void k_bin(PArrays P, uint64_t n, SysView sv, uint32_t* __restrict__ cell_tmp,
                      uint32_t* __restrict__ cell_cnt) {
  const uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const int sys = sv.of(s);
  if (!sv.triggered(sys)) return;  // kept in place (k_sys_block counts it)
  const GridDev& g = sv.g[sys];
  int k[3];
#pragma unroll
  for (int d = 0; d < 3; d++) {
    double x = P.f[RX + d][s];
    if (g.periodic[d]) {
      const double lo = g.lo[d], hi = g.hi[d], Ld = g.L[d];
      if (x < lo) {
        x = x + Ld;
        if (x >= hi) x = lo;
      } else if (x >= hi) {
        x = x - Ld;
        if (x < lo) x = lo;
      }
      P.f[RX + d][s] = x;
    }
    double q = floor((x - g.lo[d]) / g.csz[d]);
    long kk = (q < 0.0) ? 0 : (q >= (double)g.dims[d] ? g.dims[d] - 1 : (long)q);
    if (kk < 0) kk = 0;
    if (kk >= g.dims[d]) kk = g.dims[d] - 1;
    k[d] = (int)kk;
  }
  const uint32_t c =
      sv.coff[sys] + (uint32_t)k[0] + (uint32_t)g.dims[0] * ((uint32_t)k[1] + (uint32_t)g.dims[1] * (uint32_t)k[2]);
  cell_tmp[s] = c;
  atomicAdd(&cell_cnt[c], 1u);
}

__global__ void k_scatter(const uint32_t* __restrict__ cell_tmp, uint64_t n, const uint32_t* __restrict__ cell_start,
                          uint32_t* __restrict__ cursor, uint32_t* __restrict__ perm, SysView sv) {
  const uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  if (!sv.triggered(sv.of(s))) return;  // slot kept (k_perm_keep)
  const uint32_t c = cell_tmp[s];
  const uint32_t pos = cell_start[c] + atomicAdd(&cursor[c], 1u);
  perm[pos] = (uint32_t)s;
}

__global__ void k_cell_sort(uint64_t ncell, const uint32_t* __restrict__ cell_start, const uint64_t* __restrict__ id,
                            uint32_t* __restrict__ perm, SysView sv) {
  const uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncell) return;
  if (sv.nsys > 1) {  // cells of systems rebuilt without their own trigger are not used
    int lo = 0, hi = sv.nsys - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (sv.coff[mid] <= c)
        lo = mid;
      else
        hi = mid - 1;
    }
    if (!sv.triggered(lo)) return;
  }
  const uint32_t b = cell_start[c], e = cell_start[c + 1];
  for (uint32_t a = b + 1; a < e; a++) {
    const uint32_t v = perm[a];
    const uint64_t key = id[v];
    uint32_t q = a;
    while (q > b && id[perm[q - 1]] > key) {
      perm[q] = perm[q - 1];
      q--;
    }
    perm[q] = v;
  }
}

// A system rebuilt without its own trigger is one block of its particle count
// in its first cell, so that every system's cells start at its first slot.
__global__ void k_sys_block(SysView sv, uint32_t* __restrict__ cell_cnt) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= sv.nsys || sv.triggered(k)) return;
  atomicAdd(&cell_cnt[sv.coff[k]], (uint32_t)(sv.pfirst[k + 1] - sv.pfirst[k]));
}

__global__ void k_reorder(PArrays src, PArrays dst, uint64_t n, const uint32_t* __restrict__ perm,
                          const uint32_t* __restrict__ cell_tmp, uint32_t* __restrict__ cell_of, SysView sv,
                          float* __restrict__ xr, float* __restrict__ yr, float* __restrict__ zr,
                          float* __restrict__ rf) {
  const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int sys = sv.of(t);  // the slot stays in the particle's system range
  if (!sv.triggered(sys)) return;  // kept in place
  const uint32_t o = perm[t];
#pragma unroll
  for (int k = 0; k < BX; k++) dst.f[k][t] = src.f[k][o];
  // FP32 coordinates relative to the origin of the particle's cell, for the FP32 broad phase
  const GridDev& g = sv.g[sys];
  const uint32_t c = cell_tmp[o] - sv.coff[sys];
  const uint32_t kx = c % (uint32_t)g.dims[0], ky = (c / (uint32_t)g.dims[0]) % (uint32_t)g.dims[1],
                 kz = c / ((uint32_t)g.dims[0] * (uint32_t)g.dims[1]);
  xr[t] = (float)(src.f[RX][o] - (g.lo[0] + (double)kx * g.csz[0]));
  yr[t] = (float)(src.f[RY][o] - (g.lo[1] + (double)ky * g.csz[1]));
  zr[t] = (float)(src.f[RZ][o] - (g.lo[2] + (double)kz * g.csz[2]));
  rf[t] = (float)src.f[RAD][o];
  // backup_r: positions at this rebuild, for the displacement trigger
  dst.f[BX][t] = src.f[RX][o];
  dst.f[BY][t] = src.f[RY][o];
  dst.f[BZ][t] = src.f[RZ][o];
  dst.id[t] = src.id[o];
  dst.type[t] = src.type[o];
  dst.group[t] = src.group[o];
  cell_of[t] = cell_tmp[o];
}

// several systems: the reordered slots of the triggered systems back into the
// current buffer (the others were not touched, so the buffers do not swap)
__global__ void k_copy_back(PArrays from, PArrays to, uint64_t n, SysView sv) {
  const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n || !sv.triggered(sv.of(t))) return;
#pragma unroll
  for (int k = 0; k < NPF; k++) to.f[k][t] = from.f[k][t];
  to.id[t] = from.id[t];
  to.type[t] = from.type[t];
  to.group[t] = from.group[t];
}

// Systems rebuilt without their own trigger keep every particle in its slot
// (their interaction lists are then copied unchanged).
__global__ void k_perm_keep(uint32_t* __restrict__ perm, uint64_t n, SysView sv) {
  const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  if (!sv.triggered(sv.of(t))) perm[t] = (uint32_t)t;
}

__global__ void k_zero_u32(uint32_t* p, uint64_t n) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = 0u;
}
}  // namespace

// Sets up the grid, wraps, bins, scans and scatters; leaves perm = new slot -> old slot.
int launch_bin_particles(dem_ctx* c) {
  const uint64_t n = c->n;
  const uint64_t nc = c->ncell;
  cudaStream_t st = c->stream;
  int rc;
  {
  ProfScope ps(c, K_BIN, n ? 2 : 1);
  k_zero_u32<<<grid_for(nc + 1, 256), 256, 0, st>>>(c->cell_cnt, nc + 1);
  if (n) k_bin<<<grid_for(n, 256), 256, 0, st>>>(c->P[c->pcur], n, c->sysview(), c->cell_tmp, c->cell_cnt);
  if (c->nsys > 1) k_sys_block<<<(c->nsys + 255) / 256, 256, 0, st>>>(c->sysview(), c->cell_cnt);
  }
  rc = scan_exclusive_u32(c, c->cell_cnt, c->cell_start, nc);
  if (rc) return rc;
  ProfScope ps(c, K_BIN, n ? 3 : 2);
  k_zero_u32<<<grid_for(nc + 1, 256), 256, 0, st>>>(c->cell_cnt, nc + 1);
  if (n)
    k_scatter<<<grid_for(n, 256), 256, 0, st>>>(c->cell_tmp, n, c->cell_start, c->cell_cnt, c->perm, c->sysview());
  k_cell_sort<<<grid_for(nc, 256), 256, 0, st>>>(nc, c->cell_start, c->P[c->pcur].id, c->perm, c->sysview());
  if (c->nsys > 1 && n) k_perm_keep<<<grid_for(n, 256), 256, 0, st>>>(c->perm, n, c->sysview());
  DEM_CUDA_TRY(c, cudaGetLastError());
  return DEM_OK;
}

// Gathers all particle fields into the other buffer in cell order and swaps.
// Several systems: only the triggered systems' slots are gathered, then copied
// back, and the buffers do not swap.
int launch_reorder_particles(dem_ctx* c) {
  const uint64_t n = c->n;
  const bool part = c->nsys > 1;
  ProfScope ps(c, K_REORDER, n ? (part ? 2 : 1) : 0);
  if (n) {
    k_reorder<<<grid_for(n, 256), 256, 0, c->stream>>>(c->P[c->pcur], c->P[1 - c->pcur], n, c->perm, c->cell_tmp,
                                                        c->cell_of, c->sysview(), c->crel[0], c->crel[1], c->crel[2],
                                                        c->crel[3]);
    if (part) k_copy_back<<<grid_for(n, 256), 256, 0, c->stream>>>(c->P[1 - c->pcur], c->P[c->pcur], n, c->sysview());
  }
  DEM_CUDA_TRY(c, cudaGetLastError());
  if (!part) c->pcur = 1 - c->pcur;
  return DEM_OK;
}
}  // namespace dem
