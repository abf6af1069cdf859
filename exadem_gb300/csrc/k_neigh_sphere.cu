// k_neigh_sphere.cu -- sphere interaction-list rebuild (exact two-pass count / fill).
//
// Replaces chunk_neighbors_contact (src/grid/chunk_neighbors_contact.cpp:45-57),
// nbh_sphere in symetric mode (src/sphere/nbh_sphere.cu:64-309) and
// classify_interactions (src/interaction/classify_interactions.cpp:52-136):
//   - drivers first: Surface / Cylinder filters with r + rcut_inc
//     (nbh_sphere.cu:140-233, surface.hpp:320-324, cylinder.hpp:225-235);
//   - particle pairs over the 27-cell stencil with the FP64 filter
//     d2 > 0 && d2 < (r_a + r_b + rcut_inc)^2 && d2 < nbh_dist^2;
//     a pair is owned by the smaller id, except when the partner is a periodic
//     ghost image, which is kept from both sides (nbh_sphere.cu:244-249);
//   - each owner's list sorted by InteractionPair order, history (friction,
//     moment) carried over from the previous list by key equality
//     (interaction_manager.hpp:89-112, placeholder_interaction.hpp:398-408).
// Plain FP64 path (k_count / k_fill): one thread per owner particle; particles
// are in cell order so the stencil reads of neighbouring threads hit the same
// cells (L1/L2 reuse).  FP32 broad phase (k_cell_count / k_cell_fill): one warp
// per cell, its 27-cell neighbourhood staged in shared memory, candidates
// compacted with ballots, each owner's list ordered by a warp rank sort; the
// drivers per particle (k_pre_count / k_pre_fill).  In a batched context the particle's system gives the grid, its cell block and
// its drivers; a system rebuilt without its own trigger kept its slots, and
// its previous list is copied as is (so its list is the one it has alone).
#include "dem_ctx.cuh"
#include "mesh_core.cuh"

namespace dem {
namespace {

struct BPArgs {
  PArrays P;
  uint64_t n;
  SysView sv;
  const uint32_t* cell_start;
  const uint32_t* cell_of;
  const DriverDev* drv;
  int ndrv;
  const MeshDev* mesh;  // mesh drivers (DriverDev::mesh)
  int has_mesh;         // a mesh driver is registered: k_mesh_count / k_mesh_fill ran
  const uint32_t* mcnt;  // per sphere: its mesh candidates (k_mesh_count)
  double skin;
  double rcut2;
  // FP32 broad phase: cell-relative coordinates and radii, cell sizes, skin
  const float* xr;
  const float* yr;
  const float* zr;
  const float* rf;
  float skin_f;
  uint64_t cap;  // interaction buffer capacity (graph step): a fill beyond it writes nothing
  // FP32 path: the count pass's candidates of each particle (SREC per particle:
  // partner, meta), read by the fill when they fit
  uint32_t* srec;
  // per-pair damping damp_rate 2 sqrt(kn meff), in the operation order of the
  // contact law: (damp_rate * 2) * sqrt(kn * meff), meff = (m_i m_j)/(m_i + m_j)
  // for particle pairs, m_i for drivers; the pair's parameter set
  dem_contact_params cp, cpd;
  ParamTable pt;
};

__device__ __forceinline__ double pair_damp(const BPArgs& a, uint32_t i, uint32_t j, uint32_t meta) {
  const double mi = a.P.f[MASS][i];
  if (meta_type(meta) == DEM_ITYPE_VERTEX_VERTEX) {
    const dem_contact_params& q = a.pt.pair(a.cp, a.P.group[i], a.P.group[j]);
    const double mj = a.P.f[MASS][j];
    const double meff = (mi * mj) / (mi + mj);
    return q.damp_rate * 2.0 * sqrt(q.kn * meff);
  }
  const dem_contact_params& q = a.pt.drv(a.cpd, a.P.group[i], j);
  return q.damp_rate * 2.0 * sqrt(q.kn * mi);
}

// FP32 decision of the broad-phase filter d2 > 0 && d2 < (r_i + r_j + skin)^2.
// Coordinates are relative to each particle's cell origin, so |x_rel| is
// about one cell and the FP32 difference vector has an absolute error below
// 2^-22 (|x_rel_i| + |x_rel_j| + cell): three roundings of magnitudes bounded by
// that sum (conversion of each coordinate, then subtraction and addition of the
// cell offset).  The FP32 radius sum has a relative error below 2^-22.  m is 8x
// the sum of both bounds; outside [rm - m, rm + m] the FP32 comparison equals
// the FP64 one; inside, and near d = 0, the caller runs the exact FP64 test.
// Returns 1 = keep, 0 = drop, -1 = undecided.
__device__ __forceinline__ int f32_decide(float ex, float ey, float ez, float si, float sj, float cmax, float rm) {
  const float d2f = ex * ex + ey * ey + ez * ez;
  const float m = (si + sj + cmax) * 1.9073486e-06f /* 2^-19 */ + rm * 9.5367432e-07f /* 2^-20 */;
  const float hi = rm + m;
  if (d2f > hi * hi) return 0;
  const float lo = rm - m;
  if (lo > 0.f && d2f < lo * lo && d2f > 4.f * m * m) return 1;
  return -1;
}

__device__ inline bool driver_filter(const DriverDev& d, double rcut, V3 p) {
  if (d.kind == 0) {
    const V3 nrm = mk(d.normal[0], d.normal[1], d.normal[2]);
    const V3 proj = dot(p, nrm) * nrm;
    const double dd = vnorm(proj - mk(d.center_proj[0], d.center_proj[1], d.center_proj[2]));
    return dd <= rcut;
  }
  const V3 proj = p * mk(d.axis[0], d.axis[1], d.axis[2]);
  const V3 dir = proj - mk(d.center[0], d.center[1], d.center[2]);
  const double dd = vnorm(dir);
  const double dn = d.radius - (dd + rcut);
  return dn <= 0;
}

// the stationary drivers (surfaces, cylinders) of particle s's system that pass the filter
template <class Emit>
__device__ inline void for_each_driver(const BPArgs& a, uint32_t s, int sys, Emit&& emit) {
  const V3 ri = mk(a.P.f[RX][s], a.P.f[RY][s], a.P.f[RZ][s]);
  const double radi = a.P.f[RAD][s];
  const int2 dr = a.sv.drange[sys];
  for (int k = dr.x; k < dr.x + dr.y; k++) {
    const DriverDev& d = a.drv[k];
    if (d.kind == 2) continue;  // mesh drivers: mesh_phase
    if (driver_filter(d, radi + a.skin, ri))
      emit((uint32_t)k, (uint64_t)k,
           make_meta(d.kind == 0 ? DEM_ITYPE_VERTEX_SURFACE : DEM_ITYPE_VERTEX_CYLINDER, 0, 0, 0, false), 0u);
  }
}

// the particle candidates of owner s over the 27-cell stencil, in stencil order
template <bool F32, class Emit>
__device__ inline void for_each_particle(const BPArgs& a, uint32_t s, int sys, Emit&& emit) {
  const double* __restrict__ rx = a.P.f[RX];
  const double* __restrict__ ry = a.P.f[RY];
  const double* __restrict__ rz = a.P.f[RZ];
  const double* __restrict__ rad = a.P.f[RAD];
  const uint64_t* __restrict__ id = a.P.id;
  const V3 ri = mk(rx[s], ry[s], rz[s]);
  const double radi = rad[s];
  const uint64_t idi = id[s];
  const GridDev& g = a.sv.g[sys];
  const uint32_t coff = a.sv.coff[sys];
  float xri = 0.f, yri = 0.f, zri = 0.f, rfi = 0.f, si = 0.f, cmax = 0.f;
  const float csx = (float)g.csz[0], csy = (float)g.csz[1], csz = (float)g.csz[2];
  if (F32) {
    xri = a.xr[s];
    yri = a.yr[s];
    zri = a.zr[s];
    rfi = a.rf[s];
    si = fmaxf(fabsf(xri), fmaxf(fabsf(yri), fabsf(zri)));
    cmax = fmaxf(csx, fmaxf(csy, csz));
  }
  const uint32_t c = a.cell_of[s] - coff;
  const int d0 = g.dims[0], d1 = g.dims[1], d2n = g.dims[2];
  const int cx = (int)(c % (uint32_t)d0);
  const int cy = (int)((c / (uint32_t)d0) % (uint32_t)d1);
  const int cz = (int)(c / ((uint32_t)d0 * (uint32_t)d1));
  for (int dz = -1; dz <= 1; dz++) {
    int z = cz + dz, sz = 0;
    if (z < 0) {
      if (!g.periodic[2]) continue;
      z += d2n;
      sz = -1;
    } else if (z >= d2n) {
      if (!g.periodic[2]) continue;
      z -= d2n;
      sz = 1;
    }
    for (int dy = -1; dy <= 1; dy++) {
      int y = cy + dy, sy = 0;
      if (y < 0) {
        if (!g.periodic[1]) continue;
        y += d1;
        sy = -1;
      } else if (y >= d1) {
        if (!g.periodic[1]) continue;
        y -= d1;
        sy = 1;
      }
      for (int dx = -1; dx <= 1; dx++) {
        int x = cx + dx, sx = 0;
        if (x < 0) {
          if (!g.periodic[0]) continue;
          x += d0;
          sx = -1;
        } else if (x >= d0) {
          if (!g.periodic[0]) continue;
          x -= d0;
          sx = 1;
        }
        const uint32_t cc = coff + (uint32_t)x + (uint32_t)d0 * ((uint32_t)y + (uint32_t)d1 * (uint32_t)z);
        uint32_t qb = a.cell_start[cc];
        const uint32_t qe = a.cell_start[cc + 1];
        const bool ghost = (sx | sy | sz) != 0;
        const float oxf = (float)dx * csx, oyf = (float)dy * csy, ozf = (float)dz * csz;
        if (!ghost) {  // a cell's particles are in id order: the owner rule keeps the suffix above idi
          uint32_t hi = qe;
          while (qb < hi) {
            const uint32_t mid = (qb + hi) >> 1;
            if (id[mid] <= idi)
              qb = mid + 1;
            else
              hi = mid;
          }
        }
        for (uint32_t q = qb; q < qe; q++) {
          const uint64_t idj = id[q];
          if (!ghost && idi >= idj) continue;  // owner rule (kept: the suffix already satisfies it)
          int keep = -1;
          if (F32) {
            const float xj = a.xr[q], yj = a.yr[q], zj = a.zr[q];
            const float sj = fmaxf(fabsf(xj), fmaxf(fabsf(yj), fabsf(zj)));
            keep = f32_decide((xj - xri) + oxf, (yj - yri) + oyf, (zj - zri) + ozf, si, sj, cmax,
                              rfi + a.rf[q] + a.skin_f);
          }
          if (keep < 0) {
            V3 rj = mk(rx[q], ry[q], rz[q]);
            if (sx) rj.x = rj.x + (double)sx * g.L[0];
            if (sy) rj.y = rj.y + (double)sy * g.L[1];
            if (sz) rj.z = rj.z + (double)sz * g.L[2];
            const double ddx = rj.x - ri.x, ddy = rj.y - ri.y, ddz = rj.z - ri.z;
            const double d2 = ddx * ddx + ddy * ddy + ddz * ddz;
            const double rmax = radi + rad[q] + a.skin;
            keep = (d2 > 0.0 && d2 < rmax * rmax && d2 < a.rcut2) ? 1 : 0;
          }
          if (!keep) continue;
          emit(q, idj, make_meta(DEM_ITYPE_VERTEX_VERTEX, sx, sy, sz, ghost), 0u);
        }
      }
    }
  }
}

// drivers, then particles (the emission order of the thread-per-owner kernels)
template <bool F32, class Emit>
__device__ inline void for_each_candidate(const BPArgs& a, uint32_t s, Emit&& emit) {
  const int sys = a.sv.of(s);
  for_each_driver(a, s, sys, emit);
  for_each_particle<F32>(a, s, sys, emit);
}

// Mesh candidates (detection_sphere_driver, nbh_sphere.hpp:25-86): every mesh
// vertex, edge and face of the sphere's bin that passes its filter, partner
// sub = the feature.  A sphere's bin can list hundreds of features (where many
// triangles meet), so the whole warp serves its spheres one at a time, a lane
// per bin item; with Fill the passing items go, in bin order, to the start of
// the sphere's segment [b, e) (the per-sphere sort orders the segment).
// Returns the lane's own sphere's count.  Every lane of the warp calls it.
template <bool F32, bool Fill>
__device__ uint32_t mesh_phase(const BPArgs& a, uint64_t s, bool want, uint32_t b, uint32_t e, IArrays dst) {
  const int lane = threadIdx.x & 31;
  uint32_t mine = 0;
  unsigned todo = __ballot_sync(0xffffffffu, want);
  while (todo) {
    const int L = __ffs(todo) - 1;
    todo &= todo - 1u;
    const uint32_t sL = (uint32_t)__shfl_sync(0xffffffffu, (unsigned long long)s, L);
    const uint32_t bL = __shfl_sync(0xffffffffu, b, L), eL = __shfl_sync(0xffffffffu, e, L);
    const V3 p = mk(a.P.f[RX][sL], a.P.f[RY][sL], a.P.f[RZ][sL]);
    const double rad = a.P.f[RAD][sL];
    const int2 dr = a.sv.drange[a.sv.of(sL)];
    uint32_t n = 0;
    for (int k = dr.x; k < dr.x + dr.y; k++) {
      const DriverDev& d = a.drv[k];
      if (d.kind != 2) continue;
      const MeshDev& m = a.mesh[d.mesh];
      uint64_t bb;
      if (!mesh_bin_of(m, p, bb)) continue;
      const uint32_t q0 = m.boff[bb], q1 = m.boff[bb + 1];
      for (uint32_t t0 = q0; t0 < q1; t0 += 32) {
        const uint32_t t = t0 + lane;
        bool pass = false;
        uint32_t kind = 0, j = 0;
        if (t < q1) {
          const uint32_t it = m.bitem[t];
          kind = it >> 30;
          j = it & 0x3fffffffu;
          pass = F32 ? mesh_filter_f32(m, kind, j, a.skin, p, rad) : mesh_filter(m, kind, j, a.skin, p, rad);
        }
        const unsigned pm = __ballot_sync(0xffffffffu, pass);
        if (Fill && pass) {
          const uint32_t w = bL + n + __popc(pm & ((1u << lane) - 1u));
          if (w < eL) {
            dst.partner[w] = (uint32_t)k;
            dst.pid[w] = (uint64_t)k;
            dst.meta[w] = make_meta(DEM_ITYPE_VERTEX_MESH_VERTEX + kind, 0, 0, 0, false);
            dst.sub[w] = j << 16;
          }
        }
        n += __popc(pm);
      }
    }
    if (lane == L) mine = n;
  }
  __syncwarp();  // the items other lanes wrote are read by the sphere's own lane
  return mine;
}

// the mesh candidates of each triggered sphere, one warp per sphere (lane 0
// asks mesh_phase for its sphere): a sphere whose bin lists hundreds of
// features gets a warp of its own.  Kept out of k_count / k_fill so the
// particle-pair passes keep their register budget.
template <bool F32>
__global__ void k_mesh_count(BPArgs a, uint32_t* __restrict__ mcnt) {
  const uint64_t s = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (s >= a.n) return;  // the whole warp
  const bool lead = (threadIdx.x & 31) == 0;
  const bool trig = a.sv.triggered(a.sv.of(s));
  const uint32_t m = mesh_phase<F32, false>(a, s, lead && trig, 0u, 0u, IArrays{});
  if (lead) mcnt[s] = trig ? m : 0u;
}
template <bool F32>
__global__ void k_mesh_fill(BPArgs a, const uint32_t* __restrict__ off, IArrays dst) {
  const uint64_t s = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (s >= a.n) return;  // the whole warp
  const uint32_t b = off[s], e = off[s + 1];
  const bool trig = e <= a.cap && a.sv.triggered(a.sv.of(s));
  mesh_phase<F32, true>(a, s, (threadIdx.x & 31) == 0 && trig, b, e, dst);
}

constexpr uint32_t SREC = 8;

template <bool F32>
__global__ void k_count(BPArgs a, uint32_t* __restrict__ cnt, const uint32_t* __restrict__ old_off) {
  const uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= a.n) return;
  if (!a.sv.triggered(a.sv.of(s))) {  // slot kept (k_perm_keep): the previous list is copied
    cnt[s] = old_off[s + 1] - old_off[s];
    return;
  }
  const uint32_t m0 = a.has_mesh ? a.mcnt[s] : 0u;
  uint32_t m = m0;
  uint32_t* rec = F32 ? a.srec + s * (2 * SREC) : nullptr;
  for_each_candidate<F32>(a, (uint32_t)s, [&](uint32_t q, uint64_t, uint32_t meta, uint32_t) {
    if (F32 && m - m0 < SREC) {
      rec[2 * (m - m0)] = q;
      rec[2 * (m - m0) + 1] = meta;
    }
    m++;
  });
  cnt[s] = m;
}

// InteractionPair order inside the owner: (partner id, type, partner sub); swap
// and the owner sub are 0 for spheres
__device__ inline bool key_less(uint64_t pa, uint32_t ta, uint32_t sa, uint64_t pb, uint32_t tb, uint32_t sb) {
  return pa < pb || (pa == pb && (ta < tb || (ta == tb && sa < sb)));
}

// orders owner s's segment [b, e) by InteractionPair order and carries the
// history over from the previous list
__device__ inline void finish_owner(const BPArgs& a, uint32_t s, uint32_t b, uint32_t e, IArrays dst, IArrays old,
                                    const uint32_t* __restrict__ old_off, const uint32_t* __restrict__ perm,
                                    int have_old, int reuse_damp) {
  for (uint32_t x = b + 1; x < e; x++) {
    const uint64_t pk = dst.pid[x];
    const uint32_t mk_ = dst.meta[x], qk = dst.partner[x], sk = dst.sub[x];
    const uint32_t tk = meta_type(mk_);
    uint32_t y = x;
    while (y > b && key_less(pk, tk, sk, dst.pid[y - 1], meta_type(dst.meta[y - 1]), dst.sub[y - 1])) {
      dst.pid[y] = dst.pid[y - 1];
      dst.meta[y] = dst.meta[y - 1];
      dst.partner[y] = dst.partner[y - 1];
      dst.sub[y] = dst.sub[y - 1];
      y--;
    }
    dst.pid[y] = pk;
    dst.meta[y] = mk_;
    dst.partner[y] = qk;
    dst.sub[y] = sk;
  }
  // history carry-over: binary search in the previous list of the same particle
  uint32_t ob = 0, oe = 0;
  if (have_old) {
    const uint32_t os = perm[s];
    ob = old_off[os];
    oe = old_off[os + 1];
  }
  for (uint32_t x = b; x < e; x++) {
    dst.owner[x] = s;
    double h[6] = {0, 0, 0, 0, 0, 0};
    const uint64_t pk = dst.pid[x];
    const uint32_t tk = meta_type(dst.meta[x]), sk = dst.sub[x];
    uint32_t lo = ob, hi = oe;
    while (lo < hi) {
      const uint32_t mid = (lo + hi) >> 1;
      if (key_less(old.pid[mid], meta_type(old.meta[mid]), old.sub[mid], pk, tk, sk))
        lo = mid + 1;
      else
        hi = mid;
    }
    if (lo < oe && old.pid[lo] == pk && meta_type(old.meta[lo]) == tk && old.sub[lo] == sk) {
      h[0] = old.ft[0][lo];
      h[1] = old.ft[1][lo];
      h[2] = old.ft[2][lo];
      h[3] = old.mo[0][lo];
      h[4] = old.mo[1][lo];
      h[5] = old.mo[2][lo];
      // the same pair in the previous list: the same masses and (reuse_damp) the
      // same parameters, so the same damping bits, without the FP64 square root
      // and division
      dst.damp[x] = reuse_damp ? old.damp[lo] : pair_damp(a, s, dst.partner[x], dst.meta[x]);
    } else {
      dst.damp[x] = pair_damp(a, s, dst.partner[x], dst.meta[x]);
    }
    dst.ft[0][x] = h[0];
    dst.ft[1][x] = h[1];
    dst.ft[2][x] = h[2];
    dst.mo[0][x] = h[3];
    dst.mo[1][x] = h[4];
    dst.mo[2][x] = h[5];
  }
}

// reuse_damp: the previous list's damping was computed with the current contact
// parameters (no dem_set_params / dem_set_multimat since, not a list installed by
// dem_set_interactions), so a pair found in it keeps its damping bits.
template <bool F32>
__global__ void k_fill(BPArgs a, const uint32_t* __restrict__ off, IArrays dst, IArrays old,
                       const uint32_t* __restrict__ old_off, const uint32_t* __restrict__ perm, int have_old,
                       int reuse_damp) {
  const uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= a.n) return;
  const uint32_t b = off[s], e = off[s + 1];
  if (e > a.cap) return;
  if (!a.sv.triggered(a.sv.of(s))) {  // slot kept, partners of the same system kept: copy
    const uint32_t ob = old_off[s];
    for (uint32_t x = b; x < e; x++) {
      const uint32_t y = ob + (x - b);
      dst.owner[x] = (uint32_t)s;
      dst.partner[x] = old.partner[y];
      dst.pid[x] = old.pid[y];
      dst.meta[x] = old.meta[y];
      dst.sub[x] = old.sub[y];
#pragma unroll
      for (int d = 0; d < 3; d++) {
        dst.ft[d][x] = old.ft[d][y];
        dst.mo[d][x] = old.mo[d][y];
      }
      dst.damp[x] = old.damp[y];
    }
    return;
  }
  uint32_t w = b + (a.has_mesh ? a.mcnt[s] : 0u);  // mesh items first (k_mesh_fill)
  if (F32 && e - w <= SREC) {  // the count pass recorded the drivers and particles
    const uint32_t* rec = a.srec + s * (2 * SREC);
    for (uint32_t x = w; x < e; x++) {
      const uint32_t q = rec[2 * (x - w)], meta = rec[2 * (x - w) + 1];
      dst.partner[x] = q;
      dst.pid[x] = meta_type(meta) == DEM_ITYPE_VERTEX_VERTEX ? a.P.id[q] : (uint64_t)q;
      dst.meta[x] = meta;
      dst.sub[x] = 0u;
    }
  } else {
    for_each_candidate<F32>(a, (uint32_t)s, [&](uint32_t q, uint64_t pid, uint32_t meta, uint32_t sub) {
      if (w < e) {
        dst.partner[w] = q;
        dst.pid[w] = pid;
        dst.meta[w] = meta;
        dst.sub[w] = sub;
      }
      w++;
    });
  }
  finish_owner(a, (uint32_t)s, b, e, dst, old, old_off, perm, have_old, reuse_damp);
}

// ---- warp-per-cell broad phase (FP32 decisions)
// One warp per cell.  The particles of the cell's 27 stencil cells are staged
// in shared memory (FP32 cell-relative coordinates and radius, id, index and
// stencil slot, in stencil order), and the warp tests each owner of the cell
// against them 32 candidates at a time, compacting the kept ones with ballots.
// A neighbourhood of more than CELL_STAGE particles is walked per owner, lanes
// over owners (for_each_particle).  The decisions are those of for_each_particle
// (same FP32 expressions, same FP64 fallback), so the lists are the same.
// Drivers are tested per particle (k_pre_count / k_pre_fill), where every lane
// has an owner; in an owner's segment the mesh items come first, the particle
// candidates next and the drivers last, and k_fill_finish then orders each
// segment with the sort of k_fill.  The keys of a segment are distinct (a
// periodic dimension has at least three cells, each at least the reach, so a
// partner is in reach through one image at most), so the order of the
// segment's parts does not matter.
constexpr int CELL_WARPS = 4;
constexpr int CELL_STAGE = 128;  // staged neighbourhood particles per warp
constexpr uint8_t SLOT_OFF = 0x80u;  // stencil slot outside a non-periodic grid

struct CellStage {
  uint32_t q0[27];   // first particle of stencil slot l
  uint32_t pre[28];  // staged candidates before slot l; pre[27] = all
  uint8_t sh[27];    // (sx + 1) | (sy + 1) << 2 | (sz + 1) << 4 of slot l, or SLOT_OFF
  float x[CELL_STAGE], y[CELL_STAGE], z[CELL_STAGE], r[CELL_STAGE];
  uint64_t id[CELL_STAGE];
  uint32_t q[CELL_STAGE];
  uint8_t l[CELL_STAGE];
};

// stencil slots of cell c (local index in its system's grid) and the staging of
// their particles; returns the neighbourhood's particle count (staged when at most CELL_STAGE)
__device__ inline uint32_t stage_cell(const BPArgs& a, const GridDev& g, uint32_t coff, uint32_t c, CellStage& st,
                                      int lane) {
  uint32_t n = 0;
  if (lane < 27) {
    const int dz = lane / 9 - 1, dy = (lane / 3) % 3 - 1, dx = lane % 3 - 1;
    const int d0 = g.dims[0], d1 = g.dims[1], d2n = g.dims[2];
    const int cx = (int)(c % (uint32_t)d0);
    const int cy = (int)((c / (uint32_t)d0) % (uint32_t)d1);
    const int cz = (int)(c / ((uint32_t)d0 * (uint32_t)d1));
    int x = cx + dx, y = cy + dy, z = cz + dz, sx = 0, sy = 0, sz = 0;
    bool ok = true;
    if (x < 0) { ok &= g.periodic[0] != 0; x += d0; sx = -1; } else if (x >= d0) { ok &= g.periodic[0] != 0; x -= d0; sx = 1; }
    if (y < 0) { ok &= g.periodic[1] != 0; y += d1; sy = -1; } else if (y >= d1) { ok &= g.periodic[1] != 0; y -= d1; sy = 1; }
    if (z < 0) { ok &= g.periodic[2] != 0; z += d2n; sz = -1; } else if (z >= d2n) { ok &= g.periodic[2] != 0; z -= d2n; sz = 1; }
    uint32_t q0 = 0;
    if (ok) {
      const uint32_t cc = coff + (uint32_t)x + (uint32_t)d0 * ((uint32_t)y + (uint32_t)d1 * (uint32_t)z);
      q0 = a.cell_start[cc];
      n = a.cell_start[cc + 1] - q0;
    }
    st.q0[lane] = q0;
    st.sh[lane] = ok ? (uint8_t)((sx + 1) | ((sy + 1) << 2) | ((sz + 1) << 4)) : SLOT_OFF;
  }
  uint32_t v = n;  // inclusive scan over the slots
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += t;
  }
  if (lane < 27) st.pre[lane] = v - n;
  const uint32_t T = __shfl_sync(0xffffffffu, v, 31);
  if (lane == 0) st.pre[27] = T;
  __syncwarp();
  if (T <= (uint32_t)CELL_STAGE) {
    for (uint32_t i = (uint32_t)lane; i < T; i += 32) {
      int lo = 0, hi = 27;  // last slot l with pre[l] <= i (a slot holding i is not empty)
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (st.pre[mid] <= i)
          lo = mid;
        else
          hi = mid - 1;
      }
      const uint32_t q = st.q0[lo] + (i - st.pre[lo]);
      st.x[i] = a.xr[q];
      st.y[i] = a.yr[q];
      st.z[i] = a.zr[q];
      st.r[i] = a.rf[q];
      st.id[i] = a.P.id[q];
      st.q[i] = q;
      st.l[i] = (uint8_t)lo;
    }
  }
  __syncwarp();
  return T;
}

// staged candidate i against owner s: for_each_particle's decision
__device__ __forceinline__ bool cell_keep(const BPArgs& a, const GridDev& g, const CellStage& st, uint32_t i,
                                          uint64_t idi, float xri, float yri, float zri, float rfi, float si,
                                          float cmax, V3 ri, double radi, uint32_t& meta) {
  const int l = st.l[i];
  const int sh = st.sh[l];
  const int sx = (sh & 3) - 1, sy = ((sh >> 2) & 3) - 1, sz = ((sh >> 4) & 3) - 1;
  const bool ghost = (sx | sy | sz) != 0;
  if (!ghost && idi >= st.id[i]) return false;  // owner rule first
  const float oxf = (float)(l % 3 - 1) * (float)g.csz[0], oyf = (float)((l / 3) % 3 - 1) * (float)g.csz[1],
              ozf = (float)(l / 9 - 1) * (float)g.csz[2];
  const float xj = st.x[i], yj = st.y[i], zj = st.z[i];
  const float sj = fmaxf(fabsf(xj), fmaxf(fabsf(yj), fabsf(zj)));
  int keep = f32_decide((xj - xri) + oxf, (yj - yri) + oyf, (zj - zri) + ozf, si, sj, cmax, rfi + st.r[i] + a.skin_f);
  if (keep < 0) {
    const uint32_t q = st.q[i];
    V3 rj = mk(a.P.f[RX][q], a.P.f[RY][q], a.P.f[RZ][q]);
    if (sx) rj.x = rj.x + (double)sx * g.L[0];
    if (sy) rj.y = rj.y + (double)sy * g.L[1];
    if (sz) rj.z = rj.z + (double)sz * g.L[2];
    const double ddx = rj.x - ri.x, ddy = rj.y - ri.y, ddz = rj.z - ri.z;
    const double d2 = ddx * ddx + ddy * ddy + ddz * ddz;
    const double rmax = radi + a.P.f[RAD][q] + a.skin;
    keep = (d2 > 0.0 && d2 < rmax * rmax && d2 < a.rcut2) ? 1 : 0;
  }
  meta = make_meta(DEM_ITYPE_VERTEX_VERTEX, sx, sy, sz, ghost);
  return keep != 0;
}

// the particle candidates of every owner of cell C: counted (Fill = false: added
// to cnt) or written at b + mesh items (Fill = true)
template <bool Fill>
__device__ inline void cell_particles(const BPArgs& a, uint32_t C, uint32_t o0, uint32_t o1, int sys, CellStage& st,
                                      int lane, uint32_t* cnt, const uint32_t* off, IArrays dst) {
  const GridDev& g = a.sv.g[sys];
  const uint32_t coff = a.sv.coff[sys];
  const uint32_t T = stage_cell(a, g, coff, C - coff, st, lane);
  const uint32_t lt = (1u << lane) - 1u;
  if (T > (uint32_t)CELL_STAGE) {  // dense neighbourhood: lanes over owners
    for (uint32_t s = o0 + (uint32_t)lane; s < o1; s += 32) {
      if (Fill) {
        const uint32_t b = off[s], e = off[s + 1];
        if (e > a.cap) continue;
        uint32_t w = b + (a.has_mesh ? a.mcnt[s] : 0u);
        for_each_particle<true>(a, s, sys, [&](uint32_t q, uint64_t pid, uint32_t meta, uint32_t sub) {
          if (w < e) {
            dst.partner[w] = q;
            dst.pid[w] = pid;
            dst.meta[w] = meta;
            dst.sub[w] = sub;
          }
          w++;
        });
      } else {
        uint32_t m = 0;
        for_each_particle<true>(a, s, sys, [&](uint32_t, uint64_t, uint32_t, uint32_t) { m++; });
        cnt[s] += m;
      }
    }
    __syncwarp();
    return;
  }
  const float cmax = fmaxf((float)g.csz[0], fmaxf((float)g.csz[1], (float)g.csz[2]));
  for (uint32_t s = o0; s < o1; s++) {
    uint32_t w = 0, e = 0;
    if (Fill) {
      e = off[s + 1];
      if (e > a.cap) continue;
      w = off[s] + (a.has_mesh ? a.mcnt[s] : 0u);
    }
    const float xri = a.xr[s], yri = a.yr[s], zri = a.zr[s], rfi = a.rf[s];
    const float si = fmaxf(fabsf(xri), fmaxf(fabsf(yri), fabsf(zri)));
    const uint64_t idi = a.P.id[s];
    const V3 ri = mk(a.P.f[RX][s], a.P.f[RY][s], a.P.f[RZ][s]);
    const double radi = a.P.f[RAD][s];
    uint32_t m = 0;
    for (uint32_t c0 = 0; c0 < T; c0 += 32) {
      const uint32_t i = c0 + (uint32_t)lane;
      uint32_t meta = 0;
      const bool keep = i < T && cell_keep(a, g, st, i, idi, xri, yri, zri, rfi, si, cmax, ri, radi, meta);
      const unsigned bm = __ballot_sync(0xffffffffu, keep);
      if (Fill && keep) {
        const uint32_t x = w + m + __popc(bm & lt);
        if (x < e) {
          dst.partner[x] = st.q[i];
          dst.pid[x] = st.id[i];
          dst.meta[x] = meta;
          dst.sub[x] = 0u;
        }
      }
      m += __popc(bm);
    }
    if (!Fill && lane == 0) cnt[s] += m;
  }
}

// drivers of each particle (after the mesh items, counted in k_mesh_count), or
// the previous count of a particle whose system kept its list
__global__ void k_pre_count(BPArgs a, uint32_t* __restrict__ cnt, const uint32_t* __restrict__ old_off) {
  const uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= a.n) return;
  const int sys = a.sv.of(s);
  if (!a.sv.triggered(sys)) {
    cnt[s] = old_off[s + 1] - old_off[s];
    return;
  }
  uint32_t m = a.has_mesh ? a.mcnt[s] : 0u;
  for_each_driver(a, (uint32_t)s, sys, [&](uint32_t, uint64_t, uint32_t, uint32_t) { m++; });
  cnt[s] = m;
}

// drivers at the end of each particle's segment; a particle whose system kept
// its list copies it
__global__ void k_pre_fill(BPArgs a, const uint32_t* __restrict__ off, IArrays dst, IArrays old,
                           const uint32_t* __restrict__ old_off) {
  const uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= a.n) return;
  const uint32_t b = off[s], e = off[s + 1];
  if (e > a.cap) return;
  const int sys = a.sv.of(s);
  if (!a.sv.triggered(sys)) {
    const uint32_t ob = old_off[s];
    for (uint32_t x = b; x < e; x++) {
      const uint32_t y = ob + (x - b);
      dst.owner[x] = (uint32_t)s;
      dst.partner[x] = old.partner[y];
      dst.pid[x] = old.pid[y];
      dst.meta[x] = old.meta[y];
      dst.sub[x] = old.sub[y];
#pragma unroll
      for (int d = 0; d < 3; d++) {
        dst.ft[d][x] = old.ft[d][y];
        dst.mo[d][x] = old.mo[d][y];
      }
      dst.damp[x] = old.damp[y];
    }
    return;
  }
  uint32_t nd = 0;
  for_each_driver(a, (uint32_t)s, sys, [&](uint32_t, uint64_t, uint32_t, uint32_t) { nd++; });
  uint32_t w = e - nd;
  for_each_driver(a, (uint32_t)s, sys, [&](uint32_t k, uint64_t pid, uint32_t meta, uint32_t sub) {
    dst.partner[w] = k;
    dst.pid[w] = pid;
    dst.meta[w] = meta;
    dst.sub[w] = sub;
    w++;
  });
}

__global__ void __launch_bounds__(CELL_WARPS * 32) k_cell_count(BPArgs a, uint32_t* __restrict__ cnt,
                                                                uint64_t ncell) {
  __shared__ CellStage stage[CELL_WARPS];
  const int lane = threadIdx.x & 31;
  CellStage& st = stage[threadIdx.x >> 5];
  const uint64_t nw = (uint64_t)gridDim.x * CELL_WARPS;
  for (uint64_t C = (uint64_t)blockIdx.x * CELL_WARPS + (threadIdx.x >> 5); C < ncell; C += nw) {
    const uint32_t o0 = a.cell_start[C], o1 = a.cell_start[C + 1];
    if (o0 == o1) continue;
    const int sys = a.sv.of(o0);
    if (!a.sv.triggered(sys)) continue;
    cell_particles<false>(a, (uint32_t)C, o0, o1, sys, st, lane, cnt, nullptr, IArrays{});
  }
}

__global__ void __launch_bounds__(CELL_WARPS * 32) k_cell_fill(BPArgs a, const uint32_t* __restrict__ off,
                                                               IArrays dst, uint64_t ncell) {
  __shared__ CellStage stage[CELL_WARPS];
  const int lane = threadIdx.x & 31;
  CellStage& st = stage[threadIdx.x >> 5];
  const uint64_t nw = (uint64_t)gridDim.x * CELL_WARPS;
  for (uint64_t C = (uint64_t)blockIdx.x * CELL_WARPS + (threadIdx.x >> 5); C < ncell; C += nw) {
    const uint32_t o0 = a.cell_start[C], o1 = a.cell_start[C + 1];
    if (o0 == o1) continue;
    const int sys = a.sv.of(o0);
    if (!a.sv.triggered(sys)) continue;
    cell_particles<true>(a, (uint32_t)C, o0, o1, sys, st, lane, nullptr, off, dst);
  }
}

// after k_mesh_fill, k_pre_fill and k_cell_fill: each owner's segment ordered and
// its history carried over, one thread per owner
__global__ void k_fill_finish(BPArgs a, const uint32_t* __restrict__ off, IArrays dst, IArrays old,
                              const uint32_t* __restrict__ old_off, const uint32_t* __restrict__ perm, int have_old,
                              int reuse_damp) {
  const uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= a.n) return;
  const uint32_t b = off[s], e = off[s + 1];
  if (e > a.cap || !a.sv.triggered(a.sv.of(s))) return;
  finish_owner(a, (uint32_t)s, b, e, dst, old, old_off, perm, have_old, reuse_damp);
}

// per-pair damping of a kept list after the contact parameters changed
__global__ void k_pair_damp(BPArgs a, IArrays I, uint64_t ni) {
  for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < ni; k += (uint64_t)gridDim.x * blockDim.x)
    I.damp[k] = pair_damp(a, I.owner[k], I.partner[k], I.meta[k]);
}

__global__ void k_zero_u32(uint32_t* p, uint64_t n) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = 0u;
}

// partner-side lists: interactions whose partner is a real particle that receives -f
// ni_dev != nullptr: the interaction count is read on the device (graph step)
__global__ void k_rev_count(IArrays I, uint64_t ni, const unsigned long long* ni_dev, uint32_t* __restrict__ cnt) {
  const uint64_t nn = ni_dev ? *ni_dev : ni;
  for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nn; k += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t m = I.meta[k];
    if (meta_type(m) <= DEM_ITYPE_EDGE_EDGE && !meta_owner_only(m)) atomicAdd(&cnt[I.partner[k]], 1u);
  }
}
__global__ void k_rev_fill(IArrays I, uint64_t ni, const unsigned long long* ni_dev, const uint32_t* __restrict__ off,
                           uint32_t* __restrict__ cursor, uint32_t* __restrict__ idx) {
  const uint64_t nn = ni_dev ? *ni_dev : ni;
  for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nn; k += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t m = I.meta[k];
    if (meta_type(m) <= DEM_ITYPE_EDGE_EDGE && !meta_owner_only(m)) {
      const uint32_t j = I.partner[k];
      idx[off[j] + atomicAdd(&cursor[j], 1u)] = (uint32_t)k;
    }
  }
}
// order of the partner-side contributions: InteractionPair order = (owner id, index).
// A list of at most REV_SHORT entries (spheres: a few) is copied from `unsorted`
// and insertion-sorted by its particle's thread; a longer one (polyhedra: tens)
// is queued in `longs` for k_rev_rank.
constexpr uint32_t REV_SHORT = 12;
__global__ void k_rev_short(uint64_t n, const uint32_t* __restrict__ off, const uint32_t* __restrict__ owner,
                            const uint64_t* __restrict__ id, const uint32_t* __restrict__ unsorted,
                            uint32_t* __restrict__ idx, uint32_t* __restrict__ longs, unsigned int* __restrict__ nlong) {
  const uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const uint32_t b = off[s], e = off[s + 1];
  if (e - b > REV_SHORT) {
    longs[atomicAdd(nlong, 1u)] = (uint32_t)s;
    return;
  }
  for (uint32_t x = b; x < e; x++) {
    const uint32_t k = unsorted[x];
    const uint64_t ok = id[owner[k]];
    uint32_t y = x;
    while (y > b) {
      const uint32_t kp = idx[y - 1];
      const uint64_t op = id[owner[kp]];
      if (op < ok || (op == ok && kp < k)) break;
      idx[y] = kp;
      y--;
    }
    idx[y] = k;
  }
}
// One warp per queued particle: the entries of its reverse list go to idx at
// their rank, the number of entries of the list with a smaller (owner id,
// index) key (keys are distinct: the index is).  Lanes hold 32 entries at a time
// and count against every chunk of 32 of the list broadcast by shuffles.
__global__ void __launch_bounds__(256) k_rev_rank(const unsigned int* __restrict__ nlong,
                                                  const uint32_t* __restrict__ longs, const uint32_t* __restrict__ off,
                                                  const uint32_t* __restrict__ owner,
                                                  const uint64_t* __restrict__ id,
                                                  const uint32_t* __restrict__ unsorted, uint32_t* __restrict__ idx) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  const uint64_t nl = *nlong;
  for (uint64_t t = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < nl; t += nw) {
    const uint32_t s = longs[t];
    const uint32_t b = off[s], m = off[s + 1] - b;
    for (uint32_t i0 = 0; i0 < m; i0 += 32) {
      const bool have = i0 + lane < m;
      const uint32_t k = have ? unsorted[b + i0 + lane] : 0u;
      const uint64_t o = have ? id[owner[k]] : 0ull;
      uint32_t rank = 0;
      for (uint32_t j0 = 0; j0 < m; j0 += 32) {
        uint32_t kj = k;
        uint64_t oj = o;
        if (j0 != i0) {
          const bool hj = j0 + lane < m;
          kj = hj ? unsorted[b + j0 + lane] : 0u;
          oj = hj ? id[owner[kj]] : 0ull;
        }
        const uint32_t nj = m - j0 < 32u ? m - j0 : 32u;
        for (uint32_t q = 0; q < nj; q++) {
          const uint32_t kq = __shfl_sync(0xffffffffu, kj, (int)q);
          const uint64_t oq = __shfl_sync(0xffffffffu, oj, (int)q);
          rank += (oq < o || (oq == o && kq < k)) ? 1u : 0u;
        }
      }
      if (have) idx[b + rank] = k;
    }
  }
}

BPArgs make_args(dem_ctx* c) {
  BPArgs a;
  a.P = c->P[c->pcur];
  a.n = c->n;
  a.sv = c->sysview();
  a.cell_start = c->cell_start;
  a.cell_of = c->cell_of;
  a.drv = c->drv_dev;
  a.ndrv = c->ndrv;
  a.mesh = c->mesh_dev;
  a.has_mesh = c->meshes.empty() ? 0 : 1;
  a.mcnt = c->mesh_cnt;
  a.skin = c->prm.rcut_inc;
  const double nd = 2 * c->rad_max + c->prm.rcut_inc;
  a.rcut2 = nd * nd;
  a.xr = c->crel[0];
  a.yr = c->crel[1];
  a.zr = c->crel[2];
  a.rf = c->crel[3];
  a.skin_f = (float)c->prm.rcut_inc;
  a.cap = c->capturing ? c->gcap : ~0ull;
  a.srec = c->srec;
  a.cp = c->prm.config;
  a.cpd = c->prm.config_driver;
  a.pt = c->ptable();
  return a;
}
}  // namespace

// recomputes the per-pair damping of the current sphere list (after dem_set_params)
int refresh_pair_damp(dem_ctx* c) {
  if (!c->damp_stale) return DEM_OK;
  if (!c->have_list) return DEM_OK;  // still stale: the next build computes every pair's damping
  c->damp_stale = false;
  if (c->poly || !c->ni) return DEM_OK;
  k_pair_damp<<<c->num_sms * 4, 256, 0, c->stream>>>(make_args(c), c->I[c->icur], c->ni);
  DEM_CUDA_TRY(c, cudaGetLastError());
  return DEM_OK;
}

// the warp-per-cell kernels: a grid-stride loop over the cells
static unsigned cell_grid(const dem_ctx* c) {
  const uint64_t want = (c->ncell + CELL_WARPS - 1) / CELL_WARPS;
  return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(want, (uint64_t)c->num_sms * 16));
}

int launch_count_sphere(dem_ctx* c) {
  const bool mesh = !c->meshes.empty();
  ProfScope ps(c, K_BROAD_COUNT, c->n ? (mesh ? 2 : 1) : 0);
  if (c->n && mesh) {
    if (!c->mesh_cnt) return c->fail(DEM_ERR_STATE, "mesh count buffer missing");
    if (c->prm.fp32_broad_phase)
      k_mesh_count<true><<<grid_for(c->n * 32, 128), 128, 0, c->stream>>>(make_args(c), c->mesh_cnt);
    else
      k_mesh_count<false><<<grid_for(c->n * 32, 128), 128, 0, c->stream>>>(make_args(c), c->mesh_cnt);
  }
  if (c->n) {
    if (c->prm.fp32_broad_phase && c->cell_broad_phase) {
      const BPArgs a = make_args(c);
      k_pre_count<<<grid_for(c->n, 128), 128, 0, c->stream>>>(a, c->pcnt, c->own_off[c->icur]);
      k_cell_count<<<cell_grid(c), CELL_WARPS * 32, 0, c->stream>>>(a, c->pcnt, c->ncell);
    } else if (c->prm.fp32_broad_phase) {
      k_count<true><<<grid_for(c->n, 128), 128, 0, c->stream>>>(make_args(c), c->pcnt, c->own_off[c->icur]);
    } else {
      k_count<false><<<grid_for(c->n, 128), 128, 0, c->stream>>>(make_args(c), c->pcnt, c->own_off[c->icur]);
    }
  }
  DEM_CUDA_TRY(c, cudaGetLastError());
  return DEM_OK;
}

int launch_fill_sphere(dem_ctx* c, uint32_t* new_off, uint64_t total) {
  (void)total;
  const int nw = 1 - c->icur;
  const bool mesh = !c->meshes.empty();
  ProfScope ps(c, K_BROAD_FILL, c->n ? (mesh ? 2 : 1) : 0);
  if (c->n && mesh) {
    if (c->prm.fp32_broad_phase)
      k_mesh_fill<true><<<grid_for(c->n * 32, 128), 128, 0, c->stream>>>(make_args(c), new_off, c->I[nw]);
    else
      k_mesh_fill<false><<<grid_for(c->n * 32, 128), 128, 0, c->stream>>>(make_args(c), new_off, c->I[nw]);
  }
  if (c->n) {
    const int have_old = c->hist_valid ? 1 : 0, reuse = (c->hist_valid && !c->damp_stale) ? 1 : 0;
    if (c->prm.fp32_broad_phase && c->cell_broad_phase) {
      const BPArgs a = make_args(c);
      k_pre_fill<<<grid_for(c->n, 128), 128, 0, c->stream>>>(a, new_off, c->I[nw], c->I[c->icur],
                                                             c->own_off[c->icur]);
      k_cell_fill<<<cell_grid(c), CELL_WARPS * 32, 0, c->stream>>>(a, new_off, c->I[nw], c->ncell);
      k_fill_finish<<<grid_for(c->n, 128), 128, 0, c->stream>>>(a, new_off, c->I[nw], c->I[c->icur],
                                                                c->own_off[c->icur], c->perm, have_old, reuse);
    } else if (c->prm.fp32_broad_phase)
      k_fill<true><<<grid_for(c->n, 128), 128, 0, c->stream>>>(make_args(c), new_off, c->I[nw], c->I[c->icur],
                                                               c->own_off[c->icur], c->perm, have_old, reuse);
    else
      k_fill<false><<<grid_for(c->n, 128), 128, 0, c->stream>>>(make_args(c), new_off, c->I[nw], c->I[c->icur],
                                                                c->own_off[c->icur], c->perm, have_old, reuse);
  }
  DEM_CUDA_TRY(c, cudaGetLastError());
  return DEM_OK;
}

int launch_reverse_lists(dem_ctx* c) {
  const uint64_t n = c->n, ni = c->ni;
  cudaStream_t st = c->stream;
  const IArrays& I = c->I[c->icur];
  // in a graph capture the count is on the device: persistent grids over d_ni
  const unsigned long long* nd = c->capturing ? c->d_ni : nullptr;
  const bool go = c->capturing || ni;
  const unsigned gi = c->capturing ? (unsigned)c->num_sms * 8u : grid_for(ni, 256);
  {
  ProfScope ps(c, K_REVERSE, go ? 2 : 1);
  k_zero_u32<<<grid_for(n + 1, 256), 256, 0, st>>>(c->rev_cnt, n + 1);
  if (go) k_rev_count<<<gi, 256, 0, st>>>(I, ni, nd, c->rev_cnt);
  }
  int rc = scan_exclusive_u32(c, c->rev_cnt, c->rev_off, n);
  if (rc) return rc;
  ProfScope ps(c, K_REVERSE, 1 + (go ? 1 : 0) + (n ? 2 : 0));
  // the contact work list L1 (capacity rcap, like rev_idx) holds the unsorted
  // lists: the step's contact phase, after the rebuild, refills it
  uint32_t* unsorted = c->L1;
  k_zero_u32<<<grid_for(n + 1, 256), 256, 0, st>>>(c->rev_cnt, n + 1);
  if (go) k_rev_fill<<<gi, 256, 0, st>>>(I, ni, nd, c->rev_off, c->rev_cnt, unsorted);
  if (n) {
    // rev_cnt (the fill's cursors) is free again: the queue of long lists
    DEM_CUDA_TRY(c, cudaMemsetAsync(c->rev_nlong, 0, sizeof(unsigned int), st));
    k_rev_short<<<grid_for(n, 256), 256, 0, st>>>(n, c->rev_off, I.owner, c->P[c->pcur].id, unsorted, c->rev_idx,
                                                  c->rev_cnt, c->rev_nlong);
    k_rev_rank<<<(unsigned)c->num_sms * 16u, 256, 0, st>>>(c->rev_nlong, c->rev_cnt, c->rev_off, I.owner,
                                                           c->P[c->pcur].id, unsorted, c->rev_idx);
  }
  DEM_CUDA_TRY(c, cudaGetLastError());
  return DEM_OK;
}
}  // namespace dem
