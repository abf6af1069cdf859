// k_poly.cu -- sphero-polyhedron hot path: vertices, interaction-list rebuild, contact law.
//
// Replaces compute_vertices (src/polyhedron/compute_vertices.cu:68-108),
// vertex_displ_over + backup_dem (src/polyhedron/vertex_displ_over.cu:74-134,
// backup_dem.hpp:65-110), nbh_polyhedron + add_driver_interaction
// (src/polyhedron/nbh_polyhedron.cpp:75-384, nbh_polyhedron_driver.hpp:216-238)
// and the contact_polyhedron operators (polyhedron/contact.hpp:123-303).
//
// Rebuild, exact two-pass count / fill:
//   units   per owner A: one unit per neighbour B with id_A < id_B whose bounding
//           spheres are within the skin (the chunk_neighbors filter), one unit per
//           driver that can reach A; sorted by (partner id, kind);
//   SAT     one thread per unit: OBB(A), OBB(B) enlarged by skin/2, separating axis test;
//   features  one warp per surviving unit: per-vertex OBB gates (one lane per
//           vertex), then every gated feature test enumerated in InteractionPair
//           order -- VV, VE, VE(swap), VF, VF(swap), EE -- so the ballot-compacted
//           output of the fill pass is already sorted; history by full key.
// Contact: dense detection pass over all feature interactions (types 0-3 and
// vertex-driver 4/5), overlapping ones appended to a list for the Hooke pass.
// Force records are in the owner frame (for swap = 1 the contact law's particle
// i is the partner), so the per-particle gather is the one of the sphere path.
#include <algorithm>

#include "contact_core.cuh"
#include "integrate_core.cuh"
#include "mesh_core.cuh"
#include "poly_core.cuh"
#include "poly_f32.cuh"

namespace dem {
namespace {

constexpr int PT = 128;

struct PolyArgs {
  PArrays P;
  uint64_t n;
  const ShapeDev* shapes;
  int MV;
  double* vx;
  double* vy;
  double* vz;
  double* bx;
  double* by;
  double* bz;
  double* obb;  // 15 per particle
  float* fx;    // FP32 vertices relative to the centre
  float* fy;
  float* fz;
  float* fbox;  // FBOX_STRIDE per particle: FP32 gate OBB and vertex slabs (rebuild time)
  float4* qb;   // FP32 orientation at the last rebuild
  float* wx;    // FP32 roundings of the world vertices (written with vx, vy, vz)
  float* wy;
  float* wz;
  double rV;
};

// ---------------------------------------------------------------- vertices
template <bool Displ, bool Backup>
__global__ void k_poly_vertices(PolyArgs a, double thr2, unsigned long long* flag) {
  const uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  bool over = false;
  if (s < a.n) {
    const ShapeDev& sh = a.shapes[a.P.type[s]];
    const V3 p = mk(a.P.f[RX][s], a.P.f[RY][s], a.P.f[RZ][s]);
    const Q4 q = {a.P.f[QW][s], a.P.f[QX][s], a.P.f[QY][s], a.P.f[QZ][s]};
    const double h = a.P.f[HOM][s];
    for (int k = 0; k < sh.nv; k++) {
      const V3 v = world_vertex(sh, k, p, q, h);
      const uint64_t idx = s * (uint64_t)a.MV + k;
      a.vx[idx] = v.x;
      a.vy[idx] = v.y;
      a.vz[idx] = v.z;
      a.wx[idx] = (float)v.x;
      a.wy[idx] = (float)v.y;
      a.wz[idx] = (float)v.z;
      if (Displ) {
        const V3 dr = v - mk(a.bx[idx], a.by[idx], a.bz[idx]);
        over |= dot(dr, dr) >= thr2;
      }
      if (Backup) {
        a.bx[idx] = v.x;
        a.by[idx] = v.y;
        a.bz[idx] = v.z;
        a.fx[idx] = (float)(v.x - p.x);
        a.fy[idx] = (float)(v.y - p.y);
        a.fz[idx] = (float)(v.z - p.z);
      }
    }
    if (Backup) {
      const OBBd o = compute_obb(sh, p, q, h);
      double* w = a.obb + s * 15;
      const double vals[15] = {o.c.x, o.c.y, o.c.z, o.e1.x, o.e1.y, o.e1.z, o.e2.x, o.e2.y, o.e2.z,
                               o.e3.x, o.e3.y, o.e3.z, o.ext.x, o.ext.y, o.ext.z};
#pragma unroll
      for (int k = 0; k < 15; k++) w[k] = vals[k];
      a.qb[s] = make_float4((float)q.w, (float)q.x, (float)q.y, (float)q.z);
      // FP32 copy of the gate OBB (relative to the centre, enlarged by 0.5 rV twice as
      // in the feature enumeration) and vertex slabs along its normalised axes
      float* fb = a.fbox + s * FBOX_STRIDE;
      OBBd g = o;
      obb_enlarge(g, 0.5 * a.rV);
      obb_enlarge(g, 0.5 * a.rV);
      const OBBf gf = obb_f32(g, p);
      store_obbf(fb, gf);
      const uint64_t base = s * (uint64_t)a.MV;
#pragma unroll
      for (int k = 0; k < 3; k++) {
        F3 d = gf.e[k];
        const float dl = flen(d);
        d = dl > 0.f ? d * (1.f / dl) : f3(k == 0, k == 1, k == 2);
        float lo = 3.4e38f, hi = -3.4e38f;
        for (int m = 0; m < sh.nv; m++) {
          const float pr = fdot(f3(a.fx[base + m], a.fy[base + m], a.fz[base + m]), d);
          lo = fminf(lo, pr);
          hi = fmaxf(hi, pr);
        }
        fb[15 + 3 * k] = d.x;
        fb[16 + 3 * k] = d.y;
        fb[17 + 3 * k] = d.z;
        fb[24 + k] = 0.5f * (lo + hi);
        fb[27 + k] = 0.5f * (hi - lo);
      }
    }
  }
  if (Displ) {
    if (__any_sync(0xffffffffu, over) && (threadIdx.x & 31) == 0) atomicOr(flag, 1ull);
  }
}

// prolog (integration) + vertex_displ_over (backup_dem.hpp:65-110) decided in
// FP32 per vertex (decide_displ); an undecided vertex is recomputed in FP64
// exactly as the reference does (world vertex minus the stored backup vertex).
// No vertex is written.
template <int Mode>
__global__ void __launch_bounds__(256, (Mode ? 3 : 1)) k_poly_fused_prolog(PolyArgs a, double delta_t, double half_delta_t, double delta_t2_2,
                                    double thr2, float thr, unsigned long long* flag) {
  const uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  bool over = false;
  if (s < a.n) {
    prolog_one<Mode, true>(a.P, s, delta_t, half_delta_t, delta_t2_2);
    const ShapeDev& sh = a.shapes[a.P.type[s]];
    const double h = a.P.f[HOM][s];
    const V3 p = mk(a.P.f[RX][s], a.P.f[RY][s], a.P.f[RZ][s]);
    const Q4 q = {a.P.f[QW][s], a.P.f[QX][s], a.P.f[QY][s], a.P.f[QZ][s]};
    const F3 dp = f3((float)(p.x - a.P.f[BX][s]), (float)(p.y - a.P.f[BY][s]), (float)(p.z - a.P.f[BZ][s]));
    const float4 qn = make_float4((float)q.w, (float)q.x, (float)q.y, (float)q.z);
    const float4 qb = a.qb[s];
    const float hf = (float)h;
    const float q2 = fmaxf(fmaxf(qn.x * qn.x + qn.y * qn.y + qn.z * qn.z + qn.w * qn.w,
                                 qb.x * qb.x + qb.y * qb.y + qb.z * qb.z + qb.w * qb.w),
                           1.f);
    bool k_skip_vertices = false;
    const float pabs = (float)(fabs(p.x) + fabs(p.y) + fabs(p.z));
    // Rigid-body bound on every vertex displacement: with F(q) = q v q* in the
    // form v + 2w (u x v) + 2 u x (u x v), |dF/dq| <= 6 |q| |v| |dq|, so
    // |F(q) v0' - F(q_b) v0'| <= 6 max(|q|, |q_b|) |q - q_b| |v0'|.  The FP32
    // |q - q_b| carries at most 4u max|q| of rounding (both quaternions rounded
    // to FP32), the other terms a relative 1e-5; below thr (1 - 1e-4) no vertex
    // can reach the threshold and the per-vertex test is skipped.
    {
      const float qm = sqrtf(q2);
      const float dqx = qn.x - qb.x, dqy = qn.y - qb.y, dqz = qn.z - qb.z, dqw = qn.w - qb.w;
      const float dq = sqrtf(dqx * dqx + dqy * dqy + dqz * dqz + dqw * dqw) + 8.f * 5.9604645e-08f * qm;
      const float bound = (flen(dp) + 6.f * qm * dq * hf * (float)sh.maxv) * 1.00001f + 4.440892e-16f * pabs;
      if (bound < thr * 0.9999f) over = false, k_skip_vertices = true;
    }
    for (int k = 0; k < sh.nv && !over && !k_skip_vertices; k++) {
      const F3 v0 = f3(sh.vf[3 * k], sh.vf[3 * k + 1], sh.vf[3 * k + 2]) * hf;
      const int d = decide_displ(dp, qn, qb, v0, q2, pabs, thr);
      if (d == DEC_UNDECIDED) {
        const V3 v = world_vertex(sh, k, p, q, h);
        const uint64_t idx = s * (uint64_t)a.MV + k;
        const V3 dr = v - mk(a.bx[idx], a.by[idx], a.bz[idx]);
        over = dot(dr, dr) >= thr2;
      } else {
        over = d == DEC_TRUE;
      }
    }
  }
  if (__any_sync(0xffffffffu, over) && (threadIdx.x & 31) == 0) atomicOr(flag, 1ull);
}

// vertices of the listed particles (those in the interaction list), FP64
// One thread per (listed particle, vertex): world_vertex p + q (h v0) with the
// multiplies of the rotation through the placement policy (mode bit 0) and the
// product h v0 skipped for h = 1 (1 * x = x); an operand outside the integer
// multiply's fast path makes the vertex run world_vertex itself.
template <int Mode>
__global__ void k_poly_vertices_listed(PolyArgs a, const uint32_t* __restrict__ list, uint64_t count) {
  const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= count * (uint64_t)a.MV) return;
  const uint32_t s = list[t / (uint64_t)a.MV];
  const int k = (int)(t % (uint64_t)a.MV);
  const ShapeDev& sh = a.shapes[a.P.type[s]];
  if (k >= sh.nv) return;
  const V3 p = mk(a.P.f[RX][s], a.P.f[RY][s], a.P.f[RZ][s]);
  const Q4 q = {a.P.f[QW][s], a.P.f[QX][s], a.P.f[QY][s], a.P.f[QZ][s]};
  const double h = a.P.f[HOM][s];
  RotMul<Mode> rm;
  const V3 v0 = sh_v(sh, k);
  const V3 hv = emu_bits(h) == 0x3ff0000000000000ull ? v0 : mk(rm.mul(h, v0.x), rm.mul(h, v0.y), rm.mul(h, v0.z));
  V3 v = p + qrotate_m(rm, q, hv);
  if (rm.failed()) v = world_vertex(sh, k, p, q, h);
  const uint64_t idx = (uint64_t)s * a.MV + k;
  a.vx[idx] = v.x;
  a.vy[idx] = v.y;
  a.vz[idx] = v.z;
  a.wx[idx] = (float)v.x;
  a.wy[idx] = (float)v.y;
  a.wz[idx] = (float)v.z;
}

// marks the particles whose vertices the interaction list uses: both sides of the
// vertex/edge/face types, the owner of the driver types
__global__ void k_vertex_needs(IArrays I, uint64_t ni, uint32_t* __restrict__ need) {
  const uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= ni) return;
  need[I.owner[k]] = 1u;
  if (meta_type(I.meta[k]) <= DEM_ITYPE_EDGE_EDGE) need[I.partner[k]] = 1u;
}

__global__ void k_vertex_compact(const uint32_t* __restrict__ need, const uint32_t* __restrict__ off, uint64_t n,
                                 uint32_t* __restrict__ list) {
  const uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s < n && need[s]) list[off[s]] = (uint32_t)s;
}

__device__ __forceinline__ OBBd load_obb(const double* o) {
  OBBd r;
  r.c = mk(o[0], o[1], o[2]);
  r.e1 = mk(o[3], o[4], o[5]);
  r.e2 = mk(o[6], o[7], o[8]);
  r.e3 = mk(o[9], o[10], o[11]);
  r.ext = mk(o[12], o[13], o[14]);
  return r;
}

// ---------------------------------------------------------------- units
struct UnitArgs {
  PArrays P;
  uint64_t n;
  GridDev g;
  const uint32_t* cell_start;
  const uint32_t* cell_of;
  const DriverDev* drv;
  int ndrv;
  const MeshDev* mesh;
  const ShapeDev* shapes;
  double rV;
  double rcut2;
  const float* xr;
  const float* yr;
  const float* zr;
  const float* rf;
  float csz[3];
  float skin_f;
  int f32;
  // bonds owned by each slot (nullptr: no bonds): nothing is listed between
  // bonded particles, nor with a driver whose index is a bonded partner's id
  const uint32_t* b_first;
  const uint32_t* b_cnt;
  const uint64_t* b_idj;
  // the count pass's units of each particle (UREC per particle: kind << 31 |
  // partner), read by the fill when they fit
  uint32_t* urec;
};
constexpr uint32_t UREC = 16;

__device__ __forceinline__ bool bonded_to(const UnitArgs& a, uint32_t s, uint64_t id) {
  if (!a.b_cnt) return false;
  const uint32_t cn = a.b_cnt[s];
  if (!cn) return false;
  const uint32_t b0 = a.b_first[s];
  for (uint32_t k = b0; k < b0 + cn; k++)
    if (a.b_idj[k] == id) return true;
  return false;
}

__device__ __forceinline__ bool driver_reach(const DriverDev& d, double rcut, V3 p) {
  if (d.kind == 0) {
    const V3 nrm = mk(d.normal[0], d.normal[1], d.normal[2]);
    const V3 proj = dot(p, nrm) * nrm;
    const double dd = vnorm(proj - mk(d.center_proj[0], d.center_proj[1], d.center_proj[2]));
    return dd <= rcut;
  }
  const V3 proj = p * mk(d.axis[0], d.axis[1], d.axis[2]);
  const V3 dir = proj - mk(d.center[0], d.center[1], d.center[2]);
  const double dd = vnorm(dir);
  return d.radius - (dd + rcut) <= 0;
}

// FP32 decision of the bounding-sphere filter (same bound as the sphere broad phase).
__device__ __forceinline__ int f32_pair(float ex, float ey, float ez, float si, float sj, float cmax, float rm) {
  const float d2f = ex * ex + ey * ey + ez * ez;
  const float m = (si + sj + cmax) * 1.9073486e-06f + rm * 9.5367432e-07f;
  const float hi = rm + m;
  if (d2f > hi * hi) return 0;
  const float lo = rm - m;
  if (lo > 0.f && d2f < lo * lo && d2f > 4.f * m * m) return 1;
  return -1;
}

// emit(kind, partner, pid): kind 0 = particle, 1 = driver
template <class Emit>
__device__ inline void for_each_unit(const UnitArgs& a, uint32_t s, Emit&& emit) {
  const V3 ri = mk(a.P.f[RX][s], a.P.f[RY][s], a.P.f[RZ][s]);
  const uint64_t idi = a.P.id[s];
  if (a.ndrv) {
    // a vertex of A can reach a driver only if the centre is within h*(max|v0| + r) + skin (+ rounding margin)
    const ShapeDev& sh = a.shapes[a.P.type[s]];
    const double h = a.P.f[HOM][s];
    const double reach = h * (sh.maxv + sh.r) + a.rV;
    const double rc = reach + 1e-9 * (1.0 + reach + fabs(ri.x) + fabs(ri.y) + fabs(ri.z));
    for (int k = 0; k < a.ndrv; k++) {
      const DriverDev& d = a.drv[k];
      if (bonded_to(a, s, (uint64_t)k)) continue;
      if (d.kind == 2) {  // a mesh unit when the reach sphere meets the mesh's bin grid
        const MeshDev& m = a.mesh[d.mesh];
        const double bs = 1.0 / m.inv_bs;
        const bool meet = ri.x + rc >= m.lo[0] && ri.x - rc <= m.lo[0] + (m.dims[0] + 1) * bs &&
                          ri.y + rc >= m.lo[1] && ri.y - rc <= m.lo[1] + (m.dims[1] + 1) * bs &&
                          ri.z + rc >= m.lo[2] && ri.z - rc <= m.lo[2] + (m.dims[2] + 1) * bs;
        if (meet) emit(1u, (uint32_t)k, (uint64_t)k);
      } else if (driver_reach(d, rc, ri)) {
        emit(1u, (uint32_t)k, (uint64_t)k);
      }
    }
  }
  float xri = 0.f, yri = 0.f, zri = 0.f, rfi = 0.f, si = 0.f, cmax = 0.f;
  if (a.f32) {
    xri = a.xr[s];
    yri = a.yr[s];
    zri = a.zr[s];
    rfi = a.rf[s];
    si = fmaxf(fabsf(xri), fmaxf(fabsf(yri), fabsf(zri)));
    cmax = fmaxf(a.csz[0], fmaxf(a.csz[1], a.csz[2]));
  }
  const uint32_t c = a.cell_of[s];
  const int d0 = a.g.dims[0], d1 = a.g.dims[1], d2n = a.g.dims[2];
  const int cx = (int)(c % (uint32_t)d0);
  const int cy = (int)((c / (uint32_t)d0) % (uint32_t)d1);
  const int cz = (int)(c / ((uint32_t)d0 * (uint32_t)d1));
  const double radi = a.P.f[RAD][s];
  for (int dz = -1; dz <= 1; dz++) {
    const int z = cz + dz;
    if (z < 0 || z >= d2n) continue;
    for (int dy = -1; dy <= 1; dy++) {
      const int y = cy + dy;
      if (y < 0 || y >= d1) continue;
      for (int dx = -1; dx <= 1; dx++) {
        const int x = cx + dx;
        if (x < 0 || x >= d0) continue;
        const uint32_t cc = (uint32_t)x + (uint32_t)d0 * ((uint32_t)y + (uint32_t)d1 * (uint32_t)z);
        const float oxf = (float)dx * a.csz[0], oyf = (float)dy * a.csz[1], ozf = (float)dz * a.csz[2];
        // a cell's particles are in id order (k_cell_sort): the owner rule keeps
        // the suffix of ids above idi, found by bisection
        uint32_t q0 = a.cell_start[cc], q1 = a.cell_start[cc + 1];
        while (q0 < q1) {
          const uint32_t mid = (q0 + q1) >> 1;
          if (a.P.id[mid] <= idi)
            q0 = mid + 1;
          else
            q1 = mid;
        }
        for (uint32_t q = q0; q < a.cell_start[cc + 1]; q++) {
          const uint64_t idj = a.P.id[q];
          int keep = -1;
          if (a.f32) {
            const float xj = a.xr[q], yj = a.yr[q], zj = a.zr[q];
            const float sj = fmaxf(fabsf(xj), fmaxf(fabsf(yj), fabsf(zj)));
            keep = f32_pair((xj - xri) + oxf, (yj - yri) + oyf, (zj - zri) + ozf, si, sj, cmax,
                            rfi + a.rf[q] + a.skin_f);
          }
          if (keep < 0) {
            const double ddx = a.P.f[RX][q] - ri.x, ddy = a.P.f[RY][q] - ri.y, ddz = a.P.f[RZ][q] - ri.z;
            const double d2 = ddx * ddx + ddy * ddy + ddz * ddz;
            const double rmax = radi + a.P.f[RAD][q] + a.rV;
            keep = (d2 > 0.0 && d2 < rmax * rmax && d2 < a.rcut2) ? 1 : 0;
          }
          // the bond list (the ignore list of inner_bond_interaction.hpp) only for
          // the pairs in reach: the same units, fewer list walks
          if (keep && !bonded_to(a, s, idj)) emit(0u, q, idj);
        }
      }
    }
  }
}

__global__ void k_unit_count(UnitArgs a, uint32_t* __restrict__ cnt) {
  const uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= a.n) return;
  uint32_t m = 0;
  uint32_t* rec = a.urec + s * UREC;
  for_each_unit(a, (uint32_t)s, [&](uint32_t kind, uint32_t partner, uint64_t) {
    if (m < UREC) rec[m] = (kind << 31) | partner;
    m++;
  });
  cnt[s] = m;
}

__global__ void k_unit_fill(UnitArgs a, const uint32_t* __restrict__ off, uint32_t* __restrict__ u_owner,
                            uint32_t* __restrict__ u_partner, uint64_t* __restrict__ u_pid,
                            uint32_t* __restrict__ u_kind) {
  const uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= a.n) return;
  const uint32_t b = off[s], e = off[s + 1];
  if (e - b <= UREC) {  // the count pass recorded them
    const uint32_t* rec = a.urec + s * UREC;
    for (uint32_t x = b; x < e; x++) {
      const uint32_t r = rec[x - b], kind = r >> 31, partner = r & 0x7fffffffu;
      u_owner[x] = (uint32_t)s;
      u_partner[x] = partner;
      u_pid[x] = kind ? (uint64_t)partner : a.P.id[partner];
      u_kind[x] = kind;
    }
  } else {
    uint32_t w = b;
    for_each_unit(a, (uint32_t)s, [&](uint32_t kind, uint32_t partner, uint64_t pid) {
      if (w < e) {
        u_owner[w] = (uint32_t)s;
        u_partner[w] = partner;
        u_pid[w] = pid;
        u_kind[w] = kind;
      }
      w++;
    });
  }
  // (partner id, kind): particle features (types 0-3) before driver features (types 4-5)
  for (uint32_t x = b + 1; x < e; x++) {
    const uint64_t pk = u_pid[x];
    const uint32_t kk = u_kind[x], qk = u_partner[x];
    uint32_t y = x;
    while (y > b && (u_pid[y - 1] > pk || (u_pid[y - 1] == pk && u_kind[y - 1] > kk))) {
      u_pid[y] = u_pid[y - 1];
      u_kind[y] = u_kind[y - 1];
      u_partner[y] = u_partner[y - 1];
      y--;
    }
    u_pid[y] = pk;
    u_kind[y] = kk;
    u_partner[y] = qk;
  }
}

// separating axis test of the two world OBBs enlarged by skin/2 (nbh_polyhedron.cpp:264-273)
__global__ void k_unit_sat(uint64_t nu, const uint32_t* __restrict__ u_owner, const uint32_t* __restrict__ u_partner,
                           const uint32_t* __restrict__ u_kind, const double* __restrict__ obb, double rV,
                           uint8_t* __restrict__ pass) {
  const uint64_t u = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= nu) return;
  if (u_kind[u]) {
    pass[u] = 1;
    return;
  }
  OBBd A = load_obb(obb + (uint64_t)u_owner[u] * 15);
  OBBd B = load_obb(obb + (uint64_t)u_partner[u] * 15);
  obb_enlarge(A, 0.5 * rV);
  obb_enlarge(B, 0.5 * rV);
  pass[u] = obb_intersect(A, B) ? 1 : 0;
}

// ---------------------------------------------------------------- features
struct FeatArgs {
  PArrays P;
  const ShapeDev* shapes;
  const DriverDev* drv;
  const MeshDev* mesh;
  int MV;
  const double* vx;
  const double* vy;
  const double* vz;
  const double* obb;
  double rV;
  uint64_t nu;
  const uint32_t* u_owner;
  const uint32_t* u_partner;
  const uint64_t* u_pid;
  const uint32_t* u_kind;
  const uint8_t* pass;
  uint32_t* fcnt;        // count pass: features per unit
  const uint32_t* foff;  // fill pass: offsets (nu+1)
  IArrays dst;
  IArrays old;
  const uint32_t* old_off;
  const uint32_t* perm;
  int have_old;
  const float* fvx;  // FP32 vertices relative to the particle centre
  const float* fvy;
  const float* fvz;
  const float* fbox;  // FP32 gate OBBs and vertex slabs
  uint16_t* slots;    // per unit: (segment, i, j) of the features found by the count pass
  const uint32_t* slot_off;  // learned sizing: record of unit u = [slot_off[u], slot_off[u+1]); else FEAT_SLOTS each
  const uint32_t* order;     // warp bins: the count pass visits units in this order (else 0, 1, ...)
  uint32_t* utypes;          // count pass: VV, VE, VF, EE counts of each unit (u8 x 4, saturated)
  // bonds broken since the last build, as vertex-vertex history in key order
  // (owner id, partner id, owner sub | partner sub << 16); searched when the
  // old list has no entry for a vertex-vertex pair
  const uint64_t* bh_oid;
  const uint64_t* bh_pid;
  const uint32_t* bh_sub;
  const double* bh_ft[3];
  uint64_t nbh;
};

__device__ __forceinline__ VView vview(const FeatArgs& a, uint32_t s) {
  const uint64_t o = (uint64_t)s * a.MV;
  return VView{a.vx + o, a.vy + o, a.vz + o};
}

__device__ __forceinline__ int nth_bit(uint32_t mask, int r) {  // position of the r-th set bit
  for (int k = 0; k < r; k++) mask &= mask - 1u;
  return __ffs(mask) - 1;
}

// secondary key: type, swap, owner sub, partner sub (InteractionPair order after the partner id)
__device__ __forceinline__ uint64_t skey(uint32_t type, uint32_t swap, uint32_t osub, uint32_t psub) {
  return ((uint64_t)type << 48) | ((uint64_t)swap << 40) | ((uint64_t)(osub & 0xfffffu) << 20) |
         (uint64_t)(psub & 0xfffffu);
}

// The history of a new feature is searched in [hlo, hhi) of the previous list:
// the owner's previous entries, or (the fill of one unit) the part of them with
// the unit's partner id, which holds every entry the owner's range would match.
__device__ void write_feature_in(const FeatArgs& a, uint32_t w, uint32_t owner, uint32_t partner, uint64_t pid,
                                 uint32_t type, uint32_t swap, uint32_t osub, uint32_t psub, uint32_t hlo,
                                 uint32_t hhi) {
  a.dst.owner[w] = owner;
  a.dst.partner[w] = partner;
  a.dst.pid[w] = pid;
  a.dst.meta[w] = type | (swap << 15);
  a.dst.sub[w] = (osub & 0xffffu) | ((psub & 0xffffu) << 16);
  double h[6] = {0, 0, 0, 0, 0, 0};
  bool found = false;
  if (a.have_old) {
    uint32_t lo = hlo, hi = hhi;
    const uint32_t oe = hi;
    const uint64_t sk = skey(type, swap, osub & 0xffffu, psub & 0xffffu);
    while (lo < hi) {
      const uint32_t mid = (lo + hi) >> 1;
      const uint32_t om = a.old.meta[mid], osb = a.old.sub[mid];
      const uint64_t ok = skey(meta_type(om), (om >> 15) & 1u, osb & 0xffffu, osb >> 16);
      if (a.old.pid[mid] < pid || (a.old.pid[mid] == pid && ok < sk))
        lo = mid + 1;
      else
        hi = mid;
    }
    if (lo < oe && a.old.pid[lo] == pid) {
      const uint32_t om = a.old.meta[lo], osb = a.old.sub[lo];
      if (skey(meta_type(om), (om >> 15) & 1u, osb & 0xffffu, osb >> 16) == sk) {
        found = true;
        h[0] = a.old.ft[0][lo];
        h[1] = a.old.ft[1][lo];
        h[2] = a.old.ft[2][lo];
        h[3] = a.old.mo[0][lo];
        h[4] = a.old.mo[1][lo];
        h[5] = a.old.mo[2][lo];
      }
    }
  }
  if (!found && a.nbh && type == DEM_ITYPE_VERTEX_VERTEX && swap == 0u) {
    // a broken bond of this vertex pair (broke_interaction: friction, moment 0)
    const uint64_t oid = a.P.id[owner];
    const uint32_t os = osub & 0xffffu, ps = psub & 0xffffu;
    uint64_t lo = 0, hi = a.nbh;
    auto less = [&](uint64_t m) {  // entry m < key
      if (a.bh_oid[m] != oid) return a.bh_oid[m] < oid;
      if (a.bh_pid[m] != pid) return a.bh_pid[m] < pid;
      const uint32_t ms = a.bh_sub[m];
      if ((ms & 0xffffu) != os) return (ms & 0xffffu) < os;
      return (ms >> 16) < ps;
    };
    while (lo < hi) {
      const uint64_t mid = (lo + hi) >> 1;
      if (less(mid))
        lo = mid + 1;
      else
        hi = mid;
    }
    if (lo < a.nbh && a.bh_oid[lo] == oid && a.bh_pid[lo] == pid && a.bh_sub[lo] == (os | (ps << 16))) {
      h[0] = a.bh_ft[0][lo];
      h[1] = a.bh_ft[1][lo];
      h[2] = a.bh_ft[2][lo];
    }
  }
  a.dst.ft[0][w] = h[0];
  a.dst.ft[1][w] = h[1];
  a.dst.ft[2][w] = h[2];
  a.dst.mo[0][w] = h[3];
  a.dst.mo[1][w] = h[4];
  a.dst.mo[2][w] = h[5];
}

__device__ void write_feature(const FeatArgs& a, uint32_t w, uint32_t owner, uint32_t partner, uint64_t pid,
                              uint32_t type, uint32_t swap, uint32_t osub, uint32_t psub) {
  uint32_t lo = 0, hi = 0;
  if (a.have_old) {
    const uint32_t os = a.perm[owner];
    lo = a.old_off[os];
    hi = a.old_off[os + 1];
  }
  write_feature_in(a, w, owner, partner, pid, type, swap, osub, psub, lo, hi);
}

// ---------------------------------------------------------------- split precision
// k_feat<Fill, true> decides every vertex gate and every feature test in FP32
// first (poly_f32.cuh): a decided test has the FP64 result by construction, an
// undecided one (its FP32 value within 8x its error bound of a threshold) runs
// the FP64 function.  Only the rare undecided lanes touch the FP64 pipe.
__device__ __forceinline__ uint32_t seg_type(int seg) {
  return seg == 0 ? DEM_ITYPE_VERTEX_VERTEX
                  : (seg <= 2 ? DEM_ITYPE_VERTEX_EDGE : (seg <= 4 ? DEM_ITYPE_VERTEX_FACE : DEM_ITYPE_EDGE_EDGE));
}
__device__ __forceinline__ uint32_t seg_swap(int seg) { return (seg == 2 || seg == 4) ? 1u : 0u; }

// Polyhedron A against a mesh driver (add_driver_interaction for RShapeDriver,
// nbh_polyhedron_driver.hpp:61-192): types 7 (A vertex - mesh vertex), 8 (A
// vertex - mesh edge), 9 (A vertex - mesh face), 10 (A edge - mesh edge), 11
// (mesh vertex - A edge) and 12 (mesh vertex - A face), each through its Verlet
// filter; 11 and 12 only for the mesh vertices whose box (vertex +- Minkowski
// radius) meets A's OBB rotated and translated (homothety not applied) and
// enlarged by rVerlet, the reference's gate.  The reference's type 9 gate (the
// face's OBB against the vertex box) holds whenever the face filter passes and
// is not evaluated.  Candidates are the mesh features listed in the bins under
// A's box (mesh vertices: under the gate OBB's box too), each taken in the
// first of those bins (scan order z, y, x) that lists it; the fill pass writes
// a unit's items in lane order and k_mesh_unit_sort puts them in
// InteractionPair order.
struct MeshQuery {
  int lo[3], hi[3];
  bool empty;
};
__device__ __forceinline__ MeshQuery mesh_query(const MeshDev& m, V3 lo, V3 hi) {
  MeshQuery q;
  q.empty = false;
  const double l[3] = {lo.x, lo.y, lo.z}, h[3] = {hi.x, hi.y, hi.z};
  for (int d = 0; d < 3; d++) {
    const double fl = (l[d] - m.lo[d]) * m.inv_bs, fh = (h[d] - m.lo[d]) * m.inv_bs;
    if (!(fh >= 0.0) || !(fl < (double)m.dims[d])) q.empty = true;
    q.lo[d] = fl <= 0.0 ? 0 : (int)fl;
    q.hi[d] = fh >= (double)m.dims[d] ? m.dims[d] - 1 : (fh <= 0.0 ? 0 : (int)fh);
  }
  return q;
}

// FP32 context of a mesh unit's decided tests (k_feat_dec): A's vertices
// relative to its centre cA (the FP32 arrays of the list build), mesh vertices
// relative to cA rounded to FP32, S a bound of every such |coordinate| for the
// feature at hand, Rf / rVf the filter range and rVerlet in FP32
struct MeshDecCtx {
  FView fa;
  V3 cA;
  float S, Rf, rVf;
};

// tests of one mesh feature against A's vertices, edges or faces; Write: items at
// w.  Dec: each filter decided in FP32 first (poly_f32.cuh), the FP64 filter
// where undecided, so the result is the FP64 one
template <bool Write, bool Dec>
__device__ uint32_t mesh_feature_tests(const FeatArgs& a, const MeshDev& m, uint32_t kind, uint32_t j,
                                       const ShapeDev& SA, double ra, const VView& va, const OBBd& gate,
                                       uint32_t A, uint32_t k, uint32_t w, const MeshDecCtx& dc) {
  const VView mv = mesh_view(m);
  const double rV = a.rV, mr = m.r;
  uint32_t n = 0;
  auto out = [&](uint32_t type, int osub) {
    if (Write) write_feature(a, w + n, A, k, (uint64_t)k, type, 0u, (uint32_t)osub, j);
    n++;
  };
  auto mrel = [&](int q) {
    const V3 v = mv[q];
    return f3((float)(v.x - dc.cA.x), (float)(v.y - dc.cA.y), (float)(v.z - dc.cA.z));
  };
  // decided result, else the FP64 test
  auto pass = [&](int dec, auto&& exact) { return Dec && dec != DEC_UNDECIDED ? dec == DEC_TRUE : (bool)exact(); };
  if (kind == 0) {
    const V3 p = mv[j];
    const F3 pf = Dec ? mrel((int)j) : f3(0.f, 0.f, 0.f);
    for (int i = 0; i < SA.nv; i++)
      if (pass(Dec ? decide_vv(dc.fa[i], pf, dc.Rf, dc.S) : DEC_UNDECIDED,
               [&] { return filter_vv(rV, va[i], ra, p, mr); }))
        out(DEM_ITYPE_VERTEX_MESH_VERTEX, i);
    OBBd ov;
    ov.c = p;
    ov.e1 = mk(1, 0, 0);
    ov.e2 = mk(0, 1, 0);
    ov.e3 = mk(0, 0, 1);
    ov.ext = mk(0, 0, 0);
    obb_enlarge(ov, mr);
    if (obb_intersect(ov, gate)) {  // obb_v_rshape_j.intersect(obb_i)
      for (int e = 0; e < SA.ne; e++)
        if (pass(Dec ? decide_ve(pf, dc.fa[SA.e[2 * e]], dc.fa[SA.e[2 * e + 1]], dc.Rf, dc.rVf, dc.S) : DEC_UNDECIDED,
                 [&] { return filter_ve(rV, p, mr, va[SA.e[2 * e]], va[SA.e[2 * e + 1]], ra); }))
          out(DEM_ITYPE_MESH_VERTEX_EDGE, e);
      for (int f = 0; f < SA.nf; f++)
        if (pass(Dec ? decide_vf(pf, dc.fa, SA, f, dc.Rf, dc.S) : DEC_UNDECIDED,
                 [&] { return filter_vf(rV, p, mr, va, SA, f, ra); }))
          out(DEM_ITYPE_MESH_VERTEX_FACE, f);
    }
  } else if (kind == 1) {
    const V3 m0 = mv[m.e[2 * j]], m1 = mv[m.e[2 * j + 1]];
    const F3 f0 = Dec ? mrel(m.e[2 * j]) : f3(0.f, 0.f, 0.f), f1 = Dec ? mrel(m.e[2 * j + 1]) : f3(0.f, 0.f, 0.f);
    for (int i = 0; i < SA.nv; i++)
      if (pass(Dec ? decide_ve(dc.fa[i], f0, f1, dc.Rf, dc.rVf, dc.S) : DEC_UNDECIDED,
               [&] { return filter_ve(rV, va[i], ra, m0, m1, mr); }))
        out(DEM_ITYPE_VERTEX_MESH_EDGE, i);
    for (int e = 0; e < SA.ne; e++)
      if (pass(Dec ? decide_ee(dc.fa[SA.e[2 * e]], dc.fa[SA.e[2 * e + 1]], f0, f1, dc.Rf, dc.S) : DEC_UNDECIDED,
               [&] { return filter_ee(rV, va[SA.e[2 * e]], va[SA.e[2 * e + 1]], ra, m0, m1, mr); }))
        out(DEM_ITYPE_EDGE_MESH_EDGE, e);
  } else {
    const int b = m.fo[j], nf = m.fo[j + 1] - b;
    for (int i = 0; i < SA.nv; i++) {
      const int dec = Dec ? decide_vf_list(dc.fa[i], nf, [&](int q) { return mrel(m.fv[b + q]); }, dc.Rf, dc.S)
                          : DEC_UNDECIDED;
      if (pass(dec, [&] {
            double dist;
            V3 nn;
            return vf_core_list(ra + mr + rV, va[i], mv, m.fv + b, nf, dist, nn);
          }))
        out(DEM_ITYPE_VERTEX_MESH_FACE, i);
    }
  }
  return n;
}

// whether a bin of R before (x, y, z) in scan order lists item it (bin lists are sorted)
__device__ inline bool listed_before(const MeshDev& m, const MeshQuery& R, int x, int y, int z, uint32_t it) {
  for (int zz = R.lo[2]; zz <= z; zz++)
    for (int yy = R.lo[1]; yy <= R.hi[1]; yy++) {
      if (zz == z && yy > y) return false;
      for (int xx = R.lo[0]; xx <= R.hi[0]; xx++) {
        if (zz == z && yy == y && xx >= x) return false;
        const uint64_t bb = (uint64_t)xx + (uint64_t)m.dims[0] * ((uint64_t)yy + (uint64_t)m.dims[1] * zz);
        uint32_t lo = m.boff[bb], hi = m.boff[bb + 1];
        while (lo < hi) {
          const uint32_t mid = (lo + hi) >> 1;
          if (m.bitem[mid] < it)
            lo = mid + 1;
          else
            hi = mid;
        }
        if (lo < m.boff[bb + 1] && m.bitem[lo] == it) return true;
      }
    }
  return false;
}

template <bool Fill, bool Dec>
__device__ void mesh_unit(const FeatArgs& a, uint64_t u, uint32_t A, const ShapeDev& SA, double ra, const VView& va,
                          uint32_t base, int lane, uint32_t lt) {
  const uint32_t k = a.u_partner[u];
  const MeshDev& m = a.mesh[a.drv[k].mesh];
  // A's vertex box
  V3 lo = mk(HUGE_VAL, HUGE_VAL, HUGE_VAL), hi = mk(-HUGE_VAL, -HUGE_VAL, -HUGE_VAL);
  for (int i = lane; i < SA.nv; i += 32) {
    const V3 v = va[i];
    lo = mk(fmin(lo.x, v.x), fmin(lo.y, v.y), fmin(lo.z, v.z));
    hi = mk(fmax(hi.x, v.x), fmax(hi.y, v.y), fmax(hi.z, v.z));
  }
  for (int o = 16; o; o >>= 1) {
    lo = mk(fmin(lo.x, __shfl_xor_sync(0xffffffffu, lo.x, o)), fmin(lo.y, __shfl_xor_sync(0xffffffffu, lo.y, o)),
            fmin(lo.z, __shfl_xor_sync(0xffffffffu, lo.z, o)));
    hi = mk(fmax(hi.x, __shfl_xor_sync(0xffffffffu, hi.x, o)), fmax(hi.y, __shfl_xor_sync(0xffffffffu, hi.y, o)),
            fmax(hi.z, __shfl_xor_sync(0xffffffffu, hi.z, o)));
  }
  // the gate OBB: compute_obb with homothety 1, enlarged by rVerlet; its box with a margin for the SAT tolerance
  const Q4 q{a.P.f[QW][A], a.P.f[QX][A], a.P.f[QY][A], a.P.f[QZ][A]};
  OBBd gate = compute_obb(SA, mk(a.P.f[RX][A], a.P.f[RY][A], a.P.f[RZ][A]), q, 1.0);
  obb_enlarge(gate, a.rV);
  const V3 he = mk(fabs(gate.e1.x) * gate.ext.x + fabs(gate.e2.x) * gate.ext.y + fabs(gate.e3.x) * gate.ext.z,
                   fabs(gate.e1.y) * gate.ext.x + fabs(gate.e2.y) * gate.ext.y + fabs(gate.e3.y) * gate.ext.z,
                   fabs(gate.e1.z) * gate.ext.x + fabs(gate.e2.z) * gate.ext.y + fabs(gate.e3.z) * gate.ext.z);
  const double gm = 1e-6 * (1.0 + fabs(gate.c.x) + fabs(gate.c.y) + fabs(gate.c.z) + he.x + he.y + he.z);
  const V3 glo = gate.c - he - mk(gm, gm, gm), ghi = gate.c + he + mk(gm, gm, gm);
  const MeshQuery r12 = mesh_query(m, lo, hi);
  const MeshQuery r0 = mesh_query(m, mk(fmin(lo.x, glo.x), fmin(lo.y, glo.y), fmin(lo.z, glo.z)),
                                  mk(fmax(hi.x, ghi.x), fmax(hi.y, ghi.y), fmax(hi.z, ghi.z)));
  // reach of A: a feature whose bounding sphere is farther than this from A's
  // centre passes none of the six filters (A's vertices lie within h maxv of the
  // centre, its edges extended by rVerlet in their parameter within
  // h maxv (1 + 2 rVerlet), and every filter range is ra + mr + rVerlet)
  const float rp = (float)(a.P.f[HOM][A] * SA.maxv * (1.0 + 2.0 * a.rV) + ra + m.r + a.rV);
  const F3 cA = f3((float)a.P.f[RX][A], (float)a.P.f[RY][A], (float)a.P.f[RZ][A]);
  const float rpm = rp + 1e-4f * (1.f + fabsf(cA.x) + fabsf(cA.y) + fabsf(cA.z) + rp);
  const uint32_t noff[3] = {0u, (uint32_t)m.nv, (uint32_t)(m.nv + m.ne)};
  MeshDecCtx dc;
  if (Dec) {
    const uint64_t oA = (uint64_t)A * a.MV;
    dc.fa = FView{a.fvx + oA, a.fvy + oA, a.fvz + oA, f3(0.f, 0.f, 0.f)};
    dc.cA = mk(a.P.f[RX][A], a.P.f[RY][A], a.P.f[RZ][A]);
    dc.Rf = (float)(ra + m.r + a.rV);
    dc.rVf = (float)a.rV;
  }
  const float hm = (float)(a.P.f[HOM][A] * SA.maxv);
  uint32_t total = 0;
  if (!r0.empty) {
    for (int z = r0.lo[2]; z <= r0.hi[2]; z++)
      for (int y = r0.lo[1]; y <= r0.hi[1]; y++)
        for (int x = r0.lo[0]; x <= r0.hi[0]; x++) {
          const bool in12 = !r12.empty && x >= r12.lo[0] && x <= r12.hi[0] && y >= r12.lo[1] && y <= r12.hi[1] &&
                            z >= r12.lo[2] && z <= r12.hi[2];
          const uint64_t bb = (uint64_t)x + (uint64_t)m.dims[0] * ((uint64_t)y + (uint64_t)m.dims[1] * z);
          const uint32_t q0 = m.boff[bb], q1 = m.boff[bb + 1];
          for (uint32_t t0 = q0; t0 < q1; t0 += 32) {
            const uint32_t t = t0 + lane;
            uint32_t kind = 3, j = 0;
            float Sitem = 0.f;
            if (t < q1) {
              const uint32_t it = m.bitem[t];
              kind = it >> 30;
              j = it & 0x3fffffffu;
              const float4 sp = m.fsph[noff[kind] + j];
              const float dx = sp.x - cA.x, dy = sp.y - cA.y, dz = sp.z - cA.z, lim = sp.w + rpm;
              const float d2 = dx * dx + dy * dy + dz * dz;
              // bound of |coordinate| relative to A's centre: the feature's vertices, A's vertices
              Sitem = (sqrtf(d2) + sp.w + hm) * 1.001f + dc.Rf + 1e-3f + 1e-6f * (fabsf(cA.x) + fabsf(cA.y) + fabsf(cA.z));
              if (d2 > lim * lim)
                kind = 3;  // out of A's reach
              else if ((kind != 0 && !in12) || listed_before(m, kind == 0 ? r0 : r12, x, y, z, it))
                kind = 3;  // an earlier bin of the box lists it, or the vertex box does not reach it
            }
            MeshDecCtx dci = dc;
            dci.S = Sitem;
            uint32_t n = kind < 3 ? mesh_feature_tests<false, Dec>(a, m, kind, j, SA, ra, va, gate, A, k, 0, dci) : 0u;
            if (Fill) {
              uint32_t pre = n;  // inclusive warp scan of the per-lane counts
              for (int o = 1; o < 32; o <<= 1) {
                const uint32_t v = __shfl_up_sync(0xffffffffu, pre, o);
                if (lane >= o) pre += v;
              }
              if (n) mesh_feature_tests<true, Dec>(a, m, kind, j, SA, ra, va, gate, A, k, base + total + pre - n, dci);
              total += __shfl_sync(0xffffffffu, pre, 31);
            } else {
              for (int o = 16; o; o >>= 1) n += __shfl_xor_sync(0xffffffffu, n, o);
              total += n;
            }
          }
        }
  }
  (void)lt;
  if (!Fill && lane == 0) a.fcnt[u] = total;
}

// vertex - driver unit (add_driver_interaction): filter(rV + minkowski(h), vertex)
template <bool Fill>
__device__ __forceinline__ void driver_unit(const FeatArgs& a, uint64_t u, uint32_t A, const ShapeDev& SA, double ra,
                                            const VView& va, uint32_t base, int lane, uint32_t lt) {
  const uint32_t k = a.u_partner[u];
  const DriverDev& d = a.drv[k];
  if (d.kind == 2) return;  // mesh units: k_mesh_units
  const uint32_t type = d.kind == 0 ? DEM_ITYPE_VERTEX_SURFACE : DEM_ITYPE_VERTEX_CYLINDER;
  const bool keep = lane < SA.nv && driver_reach(d, a.rV + ra, va[lane]);
  const unsigned m = __ballot_sync(0xffffffffu, keep);
  if (Fill) {
    if (keep) write_feature(a, base + __popc(m & lt), A, k, a.u_pid[u], type, 0, lane, 0xffffu);
  } else if (lane == 0) {
    a.fcnt[u] = __popc(m);
  }
}

// One warp per mesh unit (the other units are skipped): kept out of k_feat /
// k_feat_dec so that the particle-pair enumeration keeps its register budget.
// Fill = false: counts into fcnt; Fill = true: writes at foff.  Dec: the
// FP32-decided tests (the FP32 broad phase).
template <bool Fill, bool Dec>
__global__ void __launch_bounds__(PT) k_mesh_units(FeatArgs a) {
  const int lane = threadIdx.x & 31;
  const uint64_t warp = ((uint64_t)blockIdx.x * PT + threadIdx.x) >> 5;
  const uint64_t nwarps = ((uint64_t)gridDim.x * PT) >> 5;
  for (uint64_t u = warp; u < a.nu; u += nwarps) {
    if (!a.u_kind[u] || !a.pass[u] || a.drv[a.u_partner[u]].kind != 2) continue;
    const uint32_t A = a.u_owner[u];
    const ShapeDev& SA = a.shapes[a.P.type[A]];
    const double ra = SA.r * a.P.f[HOM][A];
    mesh_unit<Fill, Dec>(a, u, A, SA, ra, vview(a, A), Fill ? a.foff[u] : 0u, lane, 0u);
  }
}

// exact FP64 filter of test (i, j) of segment seg (warp-uniform seg)
__device__ __noinline__ bool exact_filter(int seg, int i, int j, double rV, const VView& va, double ra,
                                          const ShapeDev& SA, const VView& vb, double rb, const ShapeDev& SB) {
  switch (seg) {
    case 0: return filter_vv(rV, va[i], ra, vb[j], rb);
    case 1: return filter_ve(rV, va[i], ra, vb[SB.e[2 * j]], vb[SB.e[2 * j + 1]], rb);
    case 2: return filter_ve(rV, vb[j], rb, va[SA.e[2 * i]], va[SA.e[2 * i + 1]], ra);
    case 3: return filter_vf(rV, va[i], ra, vb, SB, j, rb);
    case 4: return filter_vf(rV, vb[j], rb, va, SA, i, ra);
    default:
      return filter_ee(rV, va[SA.e[2 * i]], va[SA.e[2 * i + 1]], ra, vb[SB.e[2 * j]], vb[SB.e[2 * j + 1]], rb);
  }
}

__device__ __noinline__ bool vertex_gate(const OBBd& obb, V3 v, double rv) {
  OBBd ov;
  ov.c = v;
  ov.e1 = mk(1, 0, 0);
  ov.e2 = mk(0, 1, 0);
  ov.e3 = mk(0, 0, 1);
  ov.ext = mk(0, 0, 0);
  obb_enlarge(ov, rv);
  return obb_intersect(obb, ov);
}

// One warp per unit.  Fill = false: counts into fcnt; Fill = true: writes at foff.
// Plain FP64 enumeration in InteractionPair order: gated A vertices against all
// B vertices (VV), edges (VE) and faces (VF), all A edges (VE swap) and faces
// (VF swap) against gated B vertices, all edge pairs (EE), one segment (one
// filter type) at a time.
template <bool Fill>
__global__ void __launch_bounds__(PT) k_feat(FeatArgs a) {
  const int lane = threadIdx.x & 31;
  const uint64_t warp = ((uint64_t)blockIdx.x * PT + threadIdx.x) >> 5;
  const uint64_t nwarps = ((uint64_t)gridDim.x * PT) >> 5;
  const uint32_t lt = (1u << lane) - 1u;
  for (uint64_t u = warp; u < a.nu; u += nwarps) {
    uint32_t count = 0;
    const uint32_t base = Fill ? a.foff[u] : 0;
    if (!a.pass[u]) {
      if (!Fill && lane == 0) a.fcnt[u] = 0;
      continue;
    }
    const uint32_t A = a.u_owner[u];
    const ShapeDev& SA = a.shapes[a.P.type[A]];
    const double ra = SA.r * a.P.f[HOM][A];
    const VView va = vview(a, A);
    if (a.u_kind[u]) {
      driver_unit<Fill>(a, u, A, SA, ra, va, base, lane, lt);
      continue;
    }
    const uint32_t B = a.u_partner[u];
    const uint64_t pid = a.u_pid[u];
    const ShapeDev& SB = a.shapes[a.P.type[B]];
    const double rb = SB.r * a.P.f[HOM][B];
    const VView vb = vview(a, B);
    OBBd obb_i = load_obb(a.obb + (uint64_t)A * 15);
    OBBd obb_j = load_obb(a.obb + (uint64_t)B * 15);
    obb_enlarge(obb_i, 0.5 * a.rV);
    obb_enlarge(obb_j, 0.5 * a.rV);
    obb_enlarge(obb_i, 0.5 * a.rV);
    obb_enlarge(obb_j, 0.5 * a.rV);
    const bool ga = lane < SA.nv && vertex_gate(obb_j, va[lane], ra);
    const bool gb = lane < SB.nv && vertex_gate(obb_i, vb[lane], rb);
    const uint32_t gA = __ballot_sync(0xffffffffu, ga), gB = __ballot_sync(0xffffffffu, gb);
    const int nA = __popc(gA), nB = __popc(gB);
#pragma unroll 1
    for (int seg = 0; seg < 6; seg++) {
      int rows, cols;
      switch (seg) {
        case 0: rows = nA; cols = SB.nv; break;
        case 1: rows = nA; cols = SB.ne; break;
        case 2: rows = SA.ne; cols = nB; break;
        case 3: rows = nA; cols = SB.nf; break;
        case 4: rows = SA.nf; cols = nB; break;
        default: rows = SA.ne; cols = SB.ne;
      }
      const uint32_t ns = (uint32_t)rows * (uint32_t)cols;
      for (uint32_t t0 = 0; t0 < ns; t0 += 32) {
        const uint32_t t = t0 + lane;
        int i = 0, j = 0;
        bool keep = false;
        if (t < ns) {
          const int r = (int)(t / (uint32_t)cols), c = (int)(t % (uint32_t)cols);
          i = (seg == 0 || seg == 1 || seg == 3) ? nth_bit(gA, r) : r;
          j = (seg == 2 || seg == 4) ? nth_bit(gB, c) : c;
          keep = exact_filter(seg, i, j, a.rV, va, ra, SA, vb, rb, SB);
        }
        const unsigned m = __ballot_sync(0xffffffffu, keep);
        if (Fill && keep)
          write_feature(a, base + count + __popc(m & lt), A, B, pid, seg_type(seg), seg_swap(seg), i, j);
        count += __popc(m);
      }
    }
    if (!Fill && lane == 0) a.fcnt[u] = count;
  }
}

// ---- FP32-decided enumeration
// The same feature tests as k_feat, restricted by necessary conditions and
// decided in FP32 (poly_f32.cuh):
//   * vertex gates decided in FP32 (FP64 OBB::intersect only when undecided);
//   * a B vertex can pass filter_vv only within R of A's vertex hull, a face
//     (VF) only within R of the other particle's hull, an edge (VE, EE) only
//     when the edge, extended by rV times its length at both ends (VE accepts
//     r in [-rV, 1 + rV]), comes within R of it; the hulls are bounded by the
//     per-particle vertex slabs, so the other features are skipped;
//   * every remaining test is decided in FP32; undecided lanes run the FP64 filter.
// Enumeration order, and therefore the written list, is that of k_feat.
struct DecUnit {
  uint64_t u;
  uint32_t sbase, scap;  // feature record of the unit
  uint32_t A, B;
  uint64_t pid;
  const ShapeDev* SA;
  const ShapeDev* SB;
  double ra, rb;
  VView va, vb;
  FView fa, fb;
  float R, rV, S;
};

__device__ __noinline__ int decide_vf_nf(F3 vi, const FView& vf, const ShapeDev& sf, int face, float lim, float S) {
  return decide_vf(vi, vf, sf, face, lim, S);
}

template <int SEG, bool Fill>
__device__ __forceinline__ void dec_segment(const FeatArgs& a, const DecUnit& x, const uint8_t* Lr, int nr,
                                            const uint8_t* Lc, int nc, uint32_t& count, uint32_t base, int lane,
                                            uint32_t lt) {
  const uint32_t ns = (uint32_t)nr * (uint32_t)nc;
  for (uint32_t t0 = 0; t0 < ns; t0 += 32) {
    const uint32_t t = t0 + lane;
    int i = 0, j = 0;
    bool keep = false;
    if (t < ns) {
      const uint32_t r = t / (uint32_t)nc;
      i = Lr[r];
      j = Lc[t - r * (uint32_t)nc];
      int d;
      if (SEG == 0) {
        d = decide_vv(x.fa[i], x.fb[j], x.R, x.S);
      } else if (SEG == 1) {
        d = decide_ve(x.fa[i], x.fb[x.SB->e[2 * j]], x.fb[x.SB->e[2 * j + 1]], x.R, x.rV, x.S);
      } else if (SEG == 2) {
        d = decide_ve(x.fb[j], x.fa[x.SA->e[2 * i]], x.fa[x.SA->e[2 * i + 1]], x.R, x.rV, x.S);
      } else if (SEG == 3) {
        d = decide_vf_nf(x.fa[i], x.fb, *x.SB, j, x.R, x.S);
      } else if (SEG == 4) {
        d = decide_vf_nf(x.fb[j], x.fa, *x.SA, i, x.R, x.S);
      } else {
        d = decide_ee(x.fa[x.SA->e[2 * i]], x.fa[x.SA->e[2 * i + 1]], x.fb[x.SB->e[2 * j]],
                      x.fb[x.SB->e[2 * j + 1]], x.R, x.S);
      }
      keep = d == DEC_TRUE;
      if (d == DEC_UNDECIDED) keep = exact_filter(SEG, i, j, a.rV, x.va, x.ra, *x.SA, x.vb, x.rb, *x.SB);
    }
    const unsigned m = __ballot_sync(0xffffffffu, keep);
    if (keep) {
      const uint32_t pos = count + __popc(m & lt);
      if (Fill)
        write_feature(a, base + pos, x.A, x.B, x.pid, seg_type(SEG), seg_swap(SEG), i, j);
      else if (pos < x.scap)
        a.slots[x.sbase + pos] = (uint16_t)((SEG << 12) | (i << 6) | j);
    }
    count += __popc(m);
  }
}

// appends the lanes with keep set (index idx0 + lane) to L at off; returns the new length
__device__ __forceinline__ int list_append(uint8_t* L, int off, bool keep, int idx0, int lane, uint32_t lt) {
  const unsigned m = __ballot_sync(0xffffffffu, keep);
  if (keep) L[off + __popc(m & lt)] = (uint8_t)(idx0 + lane);
  return off + __popc(m);
}

template <bool Fill>
__global__ void __launch_bounds__(PT, 4) k_feat_dec(FeatArgs a) {
  // per warp: gated A vertices, gated B vertices, B vertices near A, A edges near B,
  // B edges near A, A faces near B, B faces near A
  __shared__ uint8_t lists[PT / 32][288];
  const int lane = threadIdx.x & 31;
  uint8_t* LgA = lists[threadIdx.x >> 5];
  uint8_t* LgB = LgA + 32;
  uint8_t* LvB = LgA + 64;
  uint8_t* LeA = LgA + 96;
  uint8_t* LeB = LgA + 160;
  uint8_t* LfA = LgA + 224;
  uint8_t* LfB = LgA + 256;
  const uint64_t warp = ((uint64_t)blockIdx.x * PT + threadIdx.x) >> 5;
  const uint64_t nwarps = ((uint64_t)gridDim.x * PT) >> 5;
  const uint32_t lt = (1u << lane) - 1u;
  for (uint64_t tt = warp; tt < a.nu; tt += nwarps) {
    const uint64_t u = (!Fill && a.order) ? a.order[tt] : tt;
    uint32_t count = 0;
    const uint32_t base = Fill ? a.foff[u] : 0;
    if (!a.pass[u]) {
      if (!Fill && lane == 0) {
        a.fcnt[u] = 0;
        a.utypes[u] = 0u;
      }
      continue;
    }
    DecUnit x;
    x.u = u;
    x.sbase = a.slot_off ? a.slot_off[u] : (uint32_t)(u * FEAT_SLOTS);
    x.scap = a.slot_off ? a.slot_off[u + 1] - x.sbase : (uint32_t)FEAT_SLOTS;
    x.A = a.u_owner[u];
    x.SA = &a.shapes[a.P.type[x.A]];
    x.ra = x.SA->r * a.P.f[HOM][x.A];
    x.va = vview(a, x.A);
    if (a.u_kind[u]) {
      driver_unit<Fill>(a, u, x.A, *x.SA, x.ra, x.va, base, lane, lt);
      if (!Fill && lane == 0) a.utypes[u] = 0u;
      continue;
    }
    const ShapeDev& SA = *x.SA;
    x.B = a.u_partner[u];
    x.pid = a.u_pid[u];
    x.SB = &a.shapes[a.P.type[x.B]];
    const ShapeDev& SB = *x.SB;
    x.rb = SB.r * a.P.f[HOM][x.B];
    x.vb = vview(a, x.B);
    const uint32_t A = x.A, B = x.B;
    if (Fill) {  // the count pass recorded the features of this unit unless they overflowed its record
      const uint32_t cnt = a.foff[u + 1] - base;
      if (cnt <= x.scap) {
        for (uint32_t q = lane; q < cnt; q += 32) {
          const uint32_t w = a.slots[x.sbase + q];
          const int seg = (int)(w >> 12);
          write_feature(a, base + q, A, B, x.pid, seg_type(seg), seg_swap(seg), (w >> 6) & 63u, w & 63u);
        }
        continue;
      }
    }
    const F3 dR = f3((float)(a.P.f[RX][B] - a.P.f[RX][A]), (float)(a.P.f[RY][B] - a.P.f[RY][A]),
                     (float)(a.P.f[RZ][B] - a.P.f[RZ][A]));
    const F3 zero = f3(0.f, 0.f, 0.f);
    const uint64_t oA = (uint64_t)A * a.MV, oB = (uint64_t)B * a.MV;
    x.fa = FView{a.fvx + oA, a.fvy + oA, a.fvz + oA, zero};
    x.fb = FView{a.fvx + oB, a.fvy + oB, a.fvz + oB, dR};
    // S bounds every |coordinate| relative to A's centre: measured on the vertices
    float sv = fmaxf(lane < SA.nv ? flen(x.fa[lane]) : 0.f, lane < SB.nv ? flen(x.fb[lane]) : 0.f);
#pragma unroll
    for (int o = 16; o; o >>= 1) sv = fmaxf(sv, __shfl_xor_sync(0xffffffffu, sv, o));
    x.S = sv * 1.001f + (float)(x.ra + x.rb + a.rV);
    x.R = (float)(x.ra + x.rb + a.rV);
    x.rV = (float)a.rV;
    const float lim = x.R + x.S * 6.1035156e-05f;  // R + 2^-14 S
    const float* bA = a.fbox + (uint64_t)A * FBOX_STRIDE;
    const float* bB = a.fbox + (uint64_t)B * FBOX_STRIDE;
    // Lanes are packed over both particles' features, A's first: a lane of side A
    // tests its feature against B's boxes, a lane of side B against A's.
    int nA = 0, nB = 0, nvB = 0, neA = 0, neB = 0, nfA = 0, nfB = 0;
    // vertex gates (OBB::intersect of the vertex box with the other particle's OBB) and
    // B vertices near A (VV columns)
    for (int k0 = 0; k0 < SA.nv + SB.nv; k0 += 32) {
      const int k = k0 + lane;
      const bool sideA = k < SA.nv, valid = k < SA.nv + SB.nv;
      const int vi = sideA ? k : k - SA.nv;
      int d = DEC_FALSE;
      bool near = false;
      F3 p = zero;
      if (valid) {
        p = sideA ? x.fa[vi] : x.fb[vi];
        d = decide_gate(load_obbf(sideA ? bB : bA, sideA ? dR : zero), p, (float)(sideA ? x.ra : x.rb), x.S);
        if (!sideA) near = slab_near_point(load_slabs(bA, zero), p, lim);
      }
      bool g = d == DEC_TRUE;
      if (__any_sync(0xffffffffu, d == DEC_UNDECIDED) && d == DEC_UNDECIDED) {
        OBBd o = load_obb(a.obb + (uint64_t)(sideA ? B : A) * 15);
        obb_enlarge(o, 0.5 * a.rV);
        obb_enlarge(o, 0.5 * a.rV);
        g = vertex_gate(o, sideA ? x.va[vi] : x.vb[vi], sideA ? x.ra : x.rb);
      }
      nA = list_append(LgA, nA, g && sideA, vi - lane, lane, lt);
      nB = list_append(LgB, nB, g && valid && !sideA, vi - lane, lane, lt);
      nvB = list_append(LvB, nvB, near, vi - lane, lane, lt);
    }
    // edges (extended by rV times their length) and faces near the other particle
    for (int k0 = 0; k0 < SA.ne + SB.ne; k0 += 32) {
      const int k = k0 + lane;
      const bool sideA = k < SA.ne, valid = k < SA.ne + SB.ne;
      const int e = sideA ? k : k - SA.ne;
      bool near = false;
      if (valid) {
        const FView& fv = sideA ? x.fa : x.fb;
        const int* ev = sideA ? SA.e : SB.e;
        near = slab_near_segment(load_slabs(sideA ? bB : bA, sideA ? dR : zero), fv[ev[2 * e]], fv[ev[2 * e + 1]],
                                 x.rV, lim);
      }
      neA = list_append(LeA, neA, near && sideA, e - lane, lane, lt);
      neB = list_append(LeB, neB, near && !sideA, e - lane, lane, lt);
    }
    for (int k0 = 0; k0 < SA.nf + SB.nf; k0 += 32) {
      const int k = k0 + lane;
      const bool sideA = k < SA.nf, valid = k < SA.nf + SB.nf;
      const int f = sideA ? k : k - SA.nf;
      bool near = false;
      if (valid)
        near = slab_near_face(load_slabs(sideA ? bB : bA, sideA ? dR : zero), sideA ? x.fa : x.fb,
                              sideA ? SA : SB, f, lim);
      nfA = list_append(LfA, nfA, near && sideA, f - lane, lane, lt);
      nfB = list_append(LfB, nfB, near && !sideA, f - lane, lane, lt);
    }
    __syncwarp();
    dec_segment<0, Fill>(a, x, LgA, nA, LvB, nvB, count, base, lane, lt);
    const uint32_t c_vv = count;
    dec_segment<1, Fill>(a, x, LgA, nA, LeB, neB, count, base, lane, lt);
    dec_segment<2, Fill>(a, x, LeA, neA, LgB, nB, count, base, lane, lt);
    const uint32_t c_ve = count;
    dec_segment<3, Fill>(a, x, LgA, nA, LfB, nfB, count, base, lane, lt);
    dec_segment<4, Fill>(a, x, LfA, nfA, LgB, nB, count, base, lane, lt);
    const uint32_t c_vf = count;
    dec_segment<5, Fill>(a, x, LeA, neA, LeB, neB, count, base, lane, lt);
    __syncwarp();
    if (!Fill && lane == 0) {
      a.fcnt[u] = count;
      auto sat = [](uint32_t v) { return v > 255u ? 255u : v; };
      a.utypes[u] = sat(c_vv) | (sat(c_ve - c_vv) << 8) | (sat(c_vf - c_ve) << 16) | (sat(count - c_vf) << 24);
    }
  }
}

// ---- flattened FP32-decided enumeration (count pass without learned sizing)
// The tests of k_feat_dec, spread over the whole GPU instead of a warp per unit:
//   k_feat_prep   one warp per unit: the vertex gates and the near-feature
//                 filters of k_feat_dec, kept as bit masks (UnitRec), and the
//                 test count of each of the six segments;
//   scan          over the (segment, unit) test counts, segment-major: the test
//                 index space is (segment, unit, row, column);
//   k_feat_test   32 consecutive tests per warp: every lane of a warp runs the
//                 same decision (one segment) on its own test, so the FP32
//                 arithmetic is dense and the kernel small; one kept-bit per test;
//   k_feat_collect one warp per unit: the kept bits of its six segments, in
//                 segment order, give its count (and its types), or in the fill
//                 pass its features in the order k_feat writes them.
// The decisions and the FP64 fallback are those of dec_segment, so the list is
// the same bit for bit.
struct UnitRec {
  uint32_t gA, gB, vB, fA, fB;  // gated A vertices, gated B vertices, B vertices near A, A / B faces near the other
  uint32_t eA[2], eB[2];        // A / B edges near the other (64 bits)
  float dRx, dRy, dRz, S, R;
  uint32_t pad[2];
};
static_assert(sizeof(UnitRec) == 64, "UnitRec is one 64-byte line");

__device__ __forceinline__ uint64_t u64of(uint32_t lo, uint32_t hi) { return (uint64_t)lo | ((uint64_t)hi << 32); }
__device__ __forceinline__ int nth_bit64(uint64_t m, int r) {
  const uint32_t lo = (uint32_t)m;
  const int pl = __popc(lo);
  return r < pl ? nth_bit(lo, r) : 32 + nth_bit((uint32_t)(m >> 32), r - pl);
}
// rows and columns of segment seg (see dec_segment)
__device__ __forceinline__ void seg_masks(const UnitRec& q, int seg, uint64_t& rows, uint64_t& cols) {
  const uint64_t eA = u64of(q.eA[0], q.eA[1]), eB = u64of(q.eB[0], q.eB[1]);
  rows = (seg == 2 || seg == 5) ? eA : (seg == 4 ? (uint64_t)q.fA : (uint64_t)q.gA);
  cols = seg == 0 ? (uint64_t)q.vB : (seg == 1 || seg == 5 ? eB : (seg == 3 ? (uint64_t)q.fB : (uint64_t)q.gB));
}

__global__ void __launch_bounds__(PT, 4) k_feat_prep(FeatArgs a, UnitRec* __restrict__ rec, uint32_t* __restrict__ tcnt) {
  const int lane = threadIdx.x & 31;
  const uint64_t warp = ((uint64_t)blockIdx.x * PT + threadIdx.x) >> 5;
  const uint64_t nwarps = ((uint64_t)gridDim.x * PT) >> 5;
  for (uint64_t u = warp; u < a.nu; u += nwarps) {
    if (!a.pass[u] || a.u_kind[u]) {
      if (lane < 6) tcnt[(uint64_t)lane * a.nu + u] = 0u;
      continue;
    }
    const uint32_t A = a.u_owner[u], B = a.u_partner[u];
    const ShapeDev& SA = a.shapes[a.P.type[A]];
    const ShapeDev& SB = a.shapes[a.P.type[B]];
    const double ra = SA.r * a.P.f[HOM][A], rb = SB.r * a.P.f[HOM][B];
    const F3 dR = f3((float)(a.P.f[RX][B] - a.P.f[RX][A]), (float)(a.P.f[RY][B] - a.P.f[RY][A]),
                     (float)(a.P.f[RZ][B] - a.P.f[RZ][A]));
    const F3 zero = f3(0.f, 0.f, 0.f);
    const uint64_t oA = (uint64_t)A * a.MV, oB = (uint64_t)B * a.MV;
    const FView fa{a.fvx + oA, a.fvy + oA, a.fvz + oA, zero};
    const FView fb{a.fvx + oB, a.fvy + oB, a.fvz + oB, dR};
    float sv = fmaxf(lane < SA.nv ? flen(fa[lane]) : 0.f, lane < SB.nv ? flen(fb[lane]) : 0.f);
#pragma unroll
    for (int o = 16; o; o >>= 1) sv = fmaxf(sv, __shfl_xor_sync(0xffffffffu, sv, o));
    const float S = sv * 1.001f + (float)(ra + rb + a.rV);
    const float R = (float)(ra + rb + a.rV);
    const float lim = R + S * 6.1035156e-05f;  // R + 2^-14 S
    const float* bA = a.fbox + (uint64_t)A * FBOX_STRIDE;
    const float* bB = a.fbox + (uint64_t)B * FBOX_STRIDE;
    UnitRec q{};
    for (int k0 = 0; k0 < SA.nv + SB.nv; k0 += 32) {
      const int k = k0 + lane;
      const bool sideA = k < SA.nv, valid = k < SA.nv + SB.nv;
      const int vi = sideA ? k : k - SA.nv;
      int d = DEC_FALSE;
      bool near = false;
      if (valid) {
        const F3 p = sideA ? fa[vi] : fb[vi];
        d = decide_gate(load_obbf(sideA ? bB : bA, sideA ? dR : zero), p, (float)(sideA ? ra : rb), S);
        if (!sideA) near = slab_near_point(load_slabs(bA, zero), p, lim);
      }
      bool g = d == DEC_TRUE;
      if (__any_sync(0xffffffffu, d == DEC_UNDECIDED) && d == DEC_UNDECIDED) {
        OBBd o = load_obb(a.obb + (uint64_t)(sideA ? B : A) * 15);
        obb_enlarge(o, 0.5 * a.rV);
        obb_enlarge(o, 0.5 * a.rV);
        g = vertex_gate(o, sideA ? vview(a, A)[vi] : vview(a, B)[vi], sideA ? ra : rb);
      }
      q.gA |= __reduce_or_sync(0xffffffffu, (g && sideA) ? 1u << vi : 0u);
      q.gB |= __reduce_or_sync(0xffffffffu, (g && valid && !sideA) ? 1u << vi : 0u);
      q.vB |= __reduce_or_sync(0xffffffffu, near ? 1u << vi : 0u);
    }
    for (int k0 = 0; k0 < SA.ne + SB.ne; k0 += 32) {
      const int k = k0 + lane;
      const bool sideA = k < SA.ne, valid = k < SA.ne + SB.ne;
      const int e = sideA ? k : k - SA.ne;
      bool near = false;
      if (valid) {
        const FView& fv = sideA ? fa : fb;
        const int* ev = sideA ? SA.e : SB.e;
        near = slab_near_segment(load_slabs(sideA ? bB : bA, sideA ? dR : zero), fv[ev[2 * e]], fv[ev[2 * e + 1]],
                                 (float)a.rV, lim);
      }
      const uint32_t lo = (near && e < 32) ? 1u << e : 0u, hi = (near && e >= 32) ? 1u << (e - 32) : 0u;
      q.eA[0] |= __reduce_or_sync(0xffffffffu, sideA ? lo : 0u);
      q.eA[1] |= __reduce_or_sync(0xffffffffu, sideA ? hi : 0u);
      q.eB[0] |= __reduce_or_sync(0xffffffffu, sideA ? 0u : lo);
      q.eB[1] |= __reduce_or_sync(0xffffffffu, sideA ? 0u : hi);
    }
    for (int k0 = 0; k0 < SA.nf + SB.nf; k0 += 32) {
      const int k = k0 + lane;
      const bool sideA = k < SA.nf, valid = k < SA.nf + SB.nf;
      const int f = sideA ? k : k - SA.nf;
      bool near = false;
      if (valid)
        near = slab_near_face(load_slabs(sideA ? bB : bA, sideA ? dR : zero), sideA ? fa : fb, sideA ? SA : SB, f,
                              lim);
      q.fA |= __reduce_or_sync(0xffffffffu, (near && sideA) ? 1u << f : 0u);
      q.fB |= __reduce_or_sync(0xffffffffu, (near && !sideA) ? 1u << f : 0u);
    }
    if (lane == 0) {
      q.dRx = dR.x;
      q.dRy = dR.y;
      q.dRz = dR.z;
      q.S = S;
      q.R = R;
      rec[u] = q;
    }
    if (lane < 6) {
      uint64_t rows, cols;
      seg_masks(q, lane, rows, cols);
      tcnt[(uint64_t)lane * a.nu + u] = (uint32_t)(__popcll(rows) * __popcll(cols));
    }
  }
}

// last group g in [lo, hi] with off[g] <= t (a group holding t is not empty)
__device__ __forceinline__ uint32_t group_of(const uint32_t* __restrict__ off, uint32_t lo, uint32_t hi, uint32_t t) {
  while (lo < hi) {
    const uint32_t mid = lo + ((hi - lo + 1) >> 1);
    if (off[mid] <= t)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

__global__ void __launch_bounds__(PT, 8) k_feat_test(FeatArgs a, const UnitRec* __restrict__ rec,
                                                  const uint32_t* __restrict__ toff, uint32_t ntests,
                                                  uint32_t* __restrict__ keep) {
  const int lane = threadIdx.x & 31;
  const uint32_t ng = (uint32_t)(6 * a.nu);
  const uint32_t nu = (uint32_t)a.nu;
  const uint64_t nwarps = ((uint64_t)gridDim.x * PT) >> 5;
  for (uint64_t w = ((uint64_t)blockIdx.x * PT + threadIdx.x) >> 5; w * 32 < ntests; w += nwarps) {
    const uint32_t T0 = (uint32_t)(w * 32), Tl = min(T0 + 31u, ntests - 1u);
    uint32_t gb = 0;
    if (lane == 0) gb = group_of(toff, 0u, ng - 1u, T0);
    if (lane == 31) gb = group_of(toff, 0u, ng - 1u, Tl);
    const uint32_t g0 = __shfl_sync(0xffffffffu, gb, 0), g1 = __shfl_sync(0xffffffffu, gb, 31);
    const uint32_t T = T0 + (uint32_t)lane;
    bool kp = false;
    if (T < ntests) {
      const uint32_t g = group_of(toff, g0, g1, T);
      const int seg = (int)(g / nu);
      const uint32_t u = g - (uint32_t)seg * nu;
      const uint32_t loc = T - toff[g];
      const UnitRec q = rec[u];
      uint64_t rows, cols;
      seg_masks(q, seg, rows, cols);
      const uint32_t nc = (uint32_t)__popcll(cols);
      const uint32_t r = loc / nc;
      const int i = nth_bit64(rows, (int)r), j = nth_bit64(cols, (int)(loc - r * nc));
      const uint32_t A = a.u_owner[u], B = a.u_partner[u];
      const ShapeDev& SA = a.shapes[a.P.type[A]];
      const ShapeDev& SB = a.shapes[a.P.type[B]];
      const uint64_t oA = (uint64_t)A * a.MV, oB = (uint64_t)B * a.MV;
      const FView fa{a.fvx + oA, a.fvy + oA, a.fvz + oA, f3(0.f, 0.f, 0.f)};
      const FView fb{a.fvx + oB, a.fvy + oB, a.fvz + oB, f3(q.dRx, q.dRy, q.dRz)};
      int d;
      if (seg == 0) {
        d = decide_vv(fa[i], fb[j], q.R, q.S);
      } else if (seg == 1) {
        d = decide_ve(fa[i], fb[SB.e[2 * j]], fb[SB.e[2 * j + 1]], q.R, (float)a.rV, q.S);
      } else if (seg == 2) {
        d = decide_ve(fb[j], fa[SA.e[2 * i]], fa[SA.e[2 * i + 1]], q.R, (float)a.rV, q.S);
      } else if (seg == 3) {
        d = decide_vf_nf(fa[i], fb, SB, j, q.R, q.S);
      } else if (seg == 4) {
        d = decide_vf_nf(fb[j], fa, SA, i, q.R, q.S);
      } else {
        d = decide_ee(fa[SA.e[2 * i]], fa[SA.e[2 * i + 1]], fb[SB.e[2 * j]], fb[SB.e[2 * j + 1]], q.R, q.S);
      }
      kp = d == DEC_TRUE;
      if (d == DEC_UNDECIDED)
        kp = exact_filter(seg, i, j, a.rV, vview(a, A), SA.r * a.P.f[HOM][A], SA, vview(a, B),
                          SB.r * a.P.f[HOM][B], SB);
    }
    const unsigned m = __ballot_sync(0xffffffffu, kp);
    if (lane == 0) keep[w] = m;
  }
}

// Fill = false: counts per unit (fcnt, utypes) and per (segment, unit) group (kc);
// Fill = true: the driver units' features (the pairs' come from k_feat_fill_flat)
template <bool Fill>
__global__ void __launch_bounds__(PT) k_feat_collect(FeatArgs a, const UnitRec* __restrict__ rec,
                                                     const uint32_t* __restrict__ toff,
                                                     const uint32_t* __restrict__ keep, uint32_t* __restrict__ kc) {
  const int lane = threadIdx.x & 31;
  const uint32_t lt = (1u << lane) - 1u;
  const uint64_t warp = ((uint64_t)blockIdx.x * PT + threadIdx.x) >> 5;
  const uint64_t nwarps = ((uint64_t)gridDim.x * PT) >> 5;
  for (uint64_t u = warp; u < a.nu; u += nwarps) {
    const uint32_t base = Fill ? a.foff[u] : 0u;
    if (!a.pass[u]) {
      if (!Fill && lane == 0) {
        a.fcnt[u] = 0;
        a.utypes[u] = 0u;
      }
      continue;
    }
    const uint32_t A = a.u_owner[u];
    if (a.u_kind[u]) {
      const ShapeDev& SA = a.shapes[a.P.type[A]];
      driver_unit<Fill>(a, u, A, SA, SA.r * a.P.f[HOM][A], vview(a, A), base, lane, lt);
      if (!Fill && lane == 0) a.utypes[u] = 0u;
      continue;
    }
    if (Fill) continue;  // pair units: k_feat_fill_flat
    const UnitRec q = rec[u];
    const uint32_t B = a.u_partner[u];
    const uint64_t pid = a.u_pid[u];
    uint32_t hlo = 0, hhi = 0;  // previous entries of the pair (owner A, partner id pid)
    if (Fill && a.have_old) {
      const uint32_t os = a.perm[A];
      hlo = a.old_off[os];
      hhi = a.old_off[os + 1];
      uint32_t lo = hlo, hi = hhi;
      while (lo < hi) {  // first entry with partner id >= pid
        const uint32_t mid = (lo + hi) >> 1;
        if (a.old.pid[mid] < pid)
          lo = mid + 1;
        else
          hi = mid;
      }
      hlo = lo;
      hi = hhi;
      while (lo < hi) {  // first entry with partner id > pid
        const uint32_t mid = (lo + hi) >> 1;
        if (a.old.pid[mid] <= pid)
          lo = mid + 1;
        else
          hi = mid;
      }
      hhi = lo;
    }
    uint32_t count = 0, ty[4] = {0u, 0u, 0u, 0u};
    for (int seg = 0; seg < 6; seg++) {
      const uint64_t g = (uint64_t)seg * a.nu + u;
      const uint32_t b = toff[g], e = toff[g + 1];
      uint32_t n = 0;
      if (Fill) {
        uint64_t rows, cols;
        seg_masks(q, seg, rows, cols);
        const uint32_t nc = (uint32_t)__popcll(cols);
        for (uint32_t t0 = b; t0 < e; t0 += 32) {
          const uint32_t t = t0 + (uint32_t)lane;
          const bool kp = t < e && ((keep[t >> 5] >> (t & 31u)) & 1u);
          const unsigned m = __ballot_sync(0xffffffffu, kp);
          if (kp) {
            const uint32_t loc = t - b, r = loc / nc;
            write_feature_in(a, base + count + n + __popc(m & lt), A, B, pid, seg_type(seg), seg_swap(seg),
                             nth_bit64(rows, (int)r), nth_bit64(cols, (int)(loc - r * nc)), hlo, hhi);
          }
          n += __popc(m);
        }
      } else {
        uint32_t c = 0;
        for (uint32_t w0 = (b >> 5); w0 <= ((e - 1u) >> 5) && b < e; w0 += 32) {
          const uint32_t wd = w0 + (uint32_t)lane;
          if (wd <= ((e - 1u) >> 5)) {
            uint32_t bits = keep[wd];
            const uint32_t lo = wd << 5;  // first test of the word
            if (b > lo) bits &= ~0u << (b - lo);
            if (e - lo < 32u) bits &= (1u << (e - lo)) - 1u;
            c += __popc(bits);
          }
        }
        n = __reduce_add_sync(0xffffffffu, c);
        if (lane == 0) kc[g] = n;
      }
      count += n;
      ty[(seg + 1) >> 1] += n;
    }
    if (!Fill && lane == 0) {
      a.fcnt[u] = count;
      auto sat = [](uint32_t v) { return v > 255u ? 255u : v; };
      a.utypes[u] = sat(ty[0]) | (sat(ty[1]) << 8) | (sat(ty[2]) << 16) | (sat(ty[3]) << 24);
    }
  }
}

// The fill of the pair units: one thread per test, 32 tests per warp; a kept
// test goes to foff[u] + the kept tests of u's earlier segments + the kept
// tests before it in its (segment, unit) group, which is k_feat's order.
__global__ void __launch_bounds__(PT) k_feat_fill_flat(FeatArgs a, const UnitRec* __restrict__ rec,
                                                       const uint32_t* __restrict__ toff, uint32_t ntests,
                                                       const uint32_t* __restrict__ keep,
                                                       const uint32_t* __restrict__ kc) {
  const int lane = threadIdx.x & 31;
  const uint32_t ng = (uint32_t)(6 * a.nu);
  const uint32_t nu = (uint32_t)a.nu;
  const uint64_t nwarps = ((uint64_t)gridDim.x * PT) >> 5;
  for (uint64_t w = ((uint64_t)blockIdx.x * PT + threadIdx.x) >> 5; w * 32 < ntests; w += nwarps) {
    const uint32_t bits = keep[w];
    if (!bits) continue;
    const uint32_t T = (uint32_t)(w * 32) + (uint32_t)lane;
    if (!((bits >> lane) & 1u)) continue;
    const uint32_t g = group_of(toff, 0u, ng - 1u, T);
    const int seg = (int)(g / nu);
    const uint32_t u = g - (uint32_t)seg * nu;
    const uint32_t b = toff[g];
    // kept tests of the group before T
    uint32_t before = 0;
    for (uint32_t wd = b >> 5; wd <= (T >> 5); wd++) {
      uint32_t m = keep[wd];
      const uint32_t lo = wd << 5;
      if (b > lo) m &= ~0u << (b - lo);
      if (T - lo < 32u) m &= (1u << (T - lo)) - 1u;
      before += __popc(m);
    }
    uint32_t pos = a.foff[u] + before;
    for (int s2 = 0; s2 < seg; s2++) pos += kc[(uint64_t)s2 * a.nu + u];
    const UnitRec q = rec[u];
    uint64_t rows, cols;
    seg_masks(q, seg, rows, cols);
    const uint32_t nc = (uint32_t)__popcll(cols);
    const uint32_t loc = T - b, r = loc / nc;
    write_feature(a, pos, a.u_owner[u], a.u_partner[u], a.u_pid[u], seg_type(seg), seg_swap(seg),
                  nth_bit64(rows, (int)r), nth_bit64(cols, (int)(loc - r * nc)));
  }
}

// ---------------------------------------------------------------- learned part
// MLP inputs of unit u (dem_learned.h): B's centre in A's body frame / (r_A + r_B),
// q_A^-1 q_B (w >= 0), one-hot of the unordered shape pair (types mod 3), and
// OBB overlap with each OBB enlarged by 0, skin/4, skin/2.  Inputs need no
// exactness: all in FP32, from the FP32 gate OBBs of the rebuild (which carry
// the skin/2 + skin/2 enlargement of the enumeration, taken off here).
__device__ __forceinline__ bool obb_overlap_f32(const OBBf& A, const OBBf& B, float grow) {
  float R[3][3], AR[3][3];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      R[i][j] = fdot(A.e[i], B.e[j]);
      AR[i][j] = fabsf(R[i][j]) + 1e-6f;
    }
  const F3 d = B.c - A.c;
  const float t[3] = {fdot(d, A.e[0]), fdot(d, A.e[1]), fdot(d, A.e[2])};
  const float ea[3] = {A.ext[0] + grow, A.ext[1] + grow, A.ext[2] + grow};
  const float eb[3] = {B.ext[0] + grow, B.ext[1] + grow, B.ext[2] + grow};
#pragma unroll
  for (int i = 0; i < 3; i++)
    if (fabsf(t[i]) > ea[i] + eb[0] * AR[i][0] + eb[1] * AR[i][1] + eb[2] * AR[i][2]) return false;
#pragma unroll
  for (int j = 0; j < 3; j++)
    if (fabsf(t[0] * R[0][j] + t[1] * R[1][j] + t[2] * R[2][j]) >
        eb[j] + ea[0] * AR[0][j] + ea[1] * AR[1][j] + ea[2] * AR[2][j])
      return false;
#pragma unroll
  for (int i = 0; i < 3; i++) {
    const int i1 = (i + 1) % 3, i2 = (i + 2) % 3;
#pragma unroll
    for (int j = 0; j < 3; j++) {
      const int j1 = (j + 1) % 3, j2 = (j + 2) % 3;
      const float ra = ea[i1] * AR[i2][j] + ea[i2] * AR[i1][j];
      const float rb = eb[j1] * AR[i][j2] + eb[j2] * AR[i][j1];
      if (fabsf(t[i2] * R[i1][j] - t[i1] * R[i2][j]) > ra + rb) return false;
    }
  }
  return true;
}

__global__ void k_unit_features(uint64_t nu, PArrays P, const uint32_t* __restrict__ u_owner,
                                const uint32_t* __restrict__ u_partner, const uint32_t* __restrict__ u_kind,
                                const uint8_t* __restrict__ pass, const float* __restrict__ fbox, float rV,
                                float* __restrict__ X) {
  const uint64_t u = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= nu) return;
  float x[16];
#pragma unroll
  for (int k = 0; k < 16; k++) x[k] = 0.f;
  if (!u_kind[u] && pass[u]) {
    const uint32_t A = u_owner[u], B = u_partner[u];
    const F3 d = f3((float)(P.f[RX][B] - P.f[RX][A]), (float)(P.f[RY][B] - P.f[RY][A]),
                    (float)(P.f[RZ][B] - P.f[RZ][A]));
    const float4 qa = make_float4((float)P.f[QW][A], (float)P.f[QX][A], (float)P.f[QY][A], (float)P.f[QZ][A]);
    const float4 qb = make_float4((float)P.f[QW][B], (float)P.f[QX][B], (float)P.f[QY][B], (float)P.f[QZ][B]);
    const float4 qc = make_float4(qa.x, -qa.y, -qa.z, -qa.w);  // (w, x, y, z) conjugate
    const F3 dl = qrotate_f32(qc, d);
    const float sc = 1.f / (float)(P.f[RAD][A] + P.f[RAD][B]);
    x[0] = dl.x * sc;
    x[1] = dl.y * sc;
    x[2] = dl.z * sc;
    // q_A^-1 q_B, components (w, x, y, z) = (.x, .y, .z, .w)
    float w = qc.x * qb.x - qc.y * qb.y - qc.z * qb.z - qc.w * qb.w;
    float qx = qc.x * qb.y + qc.y * qb.x + qc.z * qb.w - qc.w * qb.z;
    float qy = qc.x * qb.z - qc.y * qb.w + qc.z * qb.x + qc.w * qb.y;
    float qz = qc.x * qb.w + qc.y * qb.z - qc.z * qb.y + qc.w * qb.x;
    if (w < 0.f) w = -w, qx = -qx, qy = -qy, qz = -qz;
    x[3] = w;
    x[4] = qx;
    x[5] = qy;
    x[6] = qz;
    const uint32_t ta = P.type[A] % 3u, tb = P.type[B] % 3u;
    const uint32_t lo = ta < tb ? ta : tb, hi = ta < tb ? tb : ta;
    const int pair = lo == 0 ? (int)hi : (lo == 1 ? 2 + (int)hi : 5);  // (0,0) (0,1) (0,2) (1,1) (1,2) (2,2)
    x[7 + pair] = 1.f;
    const OBBf oa = load_obbf(fbox + (uint64_t)A * FBOX_STRIDE, f3(0.f, 0.f, 0.f));
    const OBBf ob = load_obbf(fbox + (uint64_t)B * FBOX_STRIDE, d);
#pragma unroll
    for (int q = 0; q < 3; q++) x[13 + q] = obb_overlap_f32(oa, ob, (0.25f * q - 1.f) * rV) ? 1.f : 0.f;
  }
  float* o = X + u * 16;
#pragma unroll
  for (int k = 0; k < 16; k++) o[k] = x[k];
}

// record size from the predicted rates (mean + 3 sd + 2 of the Poisson total,
// capped at 64), exact bound nv_A for driver units; bin = predicted dominant
// contact type (1..4), 0 for near-empty pairs, 5 for drivers, 6 for no-pass
__global__ void k_learned_caps(uint64_t nu, PArrays P, const ShapeDev* __restrict__ shapes,
                               const uint32_t* __restrict__ u_owner, const uint32_t* __restrict__ u_kind,
                               const uint8_t* __restrict__ pass, const float* __restrict__ rates,
                               uint32_t* __restrict__ cap, uint32_t* __restrict__ bin,
                               unsigned int* __restrict__ bin_cnt) {
  const uint64_t u = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= nu) return;
  uint32_t cp = 0, b = 6;
  if (pass[u]) {
    if (u_kind[u]) {
      cp = (uint32_t)shapes[P.type[u_owner[u]]].nv;
      b = 5;
    } else {
      const float* r = rates + u * 4;
      const float tot = r[0] + r[1] + r[2] + r[3];
      const float c = ceilf(tot + 3.f * sqrtf(tot) + 2.f);
      cp = c >= 64.f ? 64u : (c < 1.f ? 1u : (uint32_t)c);
      if (tot < 0.5f) {
        b = 0;
      } else {
        int k = 0;
        for (int q = 1; q < 4; q++)
          if (r[q] > r[k]) k = q;
        b = 1 + k;
      }
    }
  }
  cap[u] = cp;
  bin[u] = b;
  atomicAdd(&bin_cnt[b], 1u);
}

// counting sort of the units by bin (order inside a bin is free: the count
// pass writes each unit's results at the unit's own index)
__global__ void k_learned_order(uint64_t nu, const uint32_t* __restrict__ bin, unsigned int* __restrict__ cursor,
                                uint32_t* __restrict__ order) {
  const uint64_t u = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= nu) return;
  order[atomicAdd(&cursor[bin[u]], 1u)] = (uint32_t)u;
}

__global__ void k_learned_overflow(uint64_t nu, const uint32_t* __restrict__ fcnt, const uint32_t* __restrict__ off,
                                   unsigned long long* __restrict__ over) {
  const uint64_t u = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= nu) return;
  if (fcnt[u] > off[u + 1] - off[u]) atomicAdd(over, 1ull);
}

// harvest: particle-pair units that pass the OBB test, in unit order
__global__ void k_harvest_flags(uint64_t nu, const uint32_t* __restrict__ u_kind, const uint8_t* __restrict__ pass,
                                uint32_t* __restrict__ flag) {
  const uint64_t u = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (u < nu) flag[u] = (!u_kind[u] && pass[u]) ? 1u : 0u;
}
__global__ void k_harvest_write(uint64_t nu, const uint32_t* __restrict__ flag, const uint32_t* __restrict__ pos,
                                const float* __restrict__ X, const uint32_t* __restrict__ types, uint64_t capacity,
                                float* __restrict__ xo, uint8_t* __restrict__ yo) {
  const uint64_t u = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= nu || !flag[u]) return;
  const uint64_t p = pos[u];
  if (p >= capacity) return;
#pragma unroll
  for (int k = 0; k < 16; k++) xo[p * 16 + k] = X[u * 16 + k];
  const uint32_t t = types[u];
#pragma unroll
  for (int k = 0; k < 4; k++) yo[p * 4 + k] = (uint8_t)((t >> (8 * k)) & 255u);
}

// InteractionPair order inside a mesh unit (the fill pass wrote it in lane order)
__global__ void k_mesh_unit_sort(uint64_t nu, const uint32_t* __restrict__ u_kind, const uint32_t* __restrict__ u_partner,
                                 const DriverDev* __restrict__ drv, const uint32_t* __restrict__ foff, IArrays I) {
  const uint64_t u = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= nu || !u_kind[u] || drv[u_partner[u]].kind != 2) return;
  const uint32_t b = foff[u], e = foff[u + 1];
  auto key = [&](uint32_t x) {
    const uint32_t m = I.meta[x], s = I.sub[x];
    return skey(meta_type(m), (m >> 15) & 1u, s & 0xffffu, s >> 16);
  };
  for (uint32_t x = b + 1; x < e; x++) {
    const uint64_t kx = key(x);
    const uint32_t mx = I.meta[x], sx = I.sub[x];
    double h[6] = {I.ft[0][x], I.ft[1][x], I.ft[2][x], I.mo[0][x], I.mo[1][x], I.mo[2][x]};
    uint32_t y = x;
    while (y > b && key(y - 1) > kx) {
      I.meta[y] = I.meta[y - 1];
      I.sub[y] = I.sub[y - 1];
      for (int d = 0; d < 3; d++) {
        I.ft[d][y] = I.ft[d][y - 1];
        I.mo[d][y] = I.mo[d][y - 1];
      }
      y--;
    }
    I.meta[y] = mx;
    I.sub[y] = sx;
    for (int d = 0; d < 3; d++) {
      I.ft[d][y] = h[d];
      I.mo[d][y] = h[3 + d];
    }
  }
}

// own_off[s] = feature offset of the first unit of s
__global__ void k_own_from_units(uint64_t n, const uint32_t* __restrict__ uoff, const uint32_t* __restrict__ foff,
                                 uint32_t* __restrict__ own) {
  const uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s > n) return;
  own[s] = foff[uoff[s]];
}

// ---------------------------------------------------------------- contact
struct PCArgs {
  PArrays P;
  IArrays I;
  Records R;
  uint64_t ni;
  const ShapeDev* shapes;
  const DriverDev* drv;
  int MV;
  const double* vx;
  const double* vy;
  const double* vz;
  const float* wx;  // FP32 roundings of the world vertices (contact screen)
  const float* wy;
  const float* wz;
  int screen;       // FP32 contact screen of the particle pairs (fused step, no cohesion, no analysis)
  dem_contact_params cp, cpd;
  double dt;
  int cohesive;
  int dmt;        // Hooke_DMT law combination
  ParamTable pt;  // multi-material parameters (pt.pp == nullptr: cp / cpd)
  ContactStateArrays cs;  // analysis, in the contact law's frame (cs.dn == nullptr: off)
  const MeshDev* mesh;
  uint32_t* L2;
  double* D[7];
  unsigned long long* cnt;  // [1] = L2 count, [2] = L2 entries with dn >= 0 (cohesive mesh items)
  unsigned long long* n_active;
};

__device__ __forceinline__ void pwrite(const PCArgs& a, uint64_t k, V3 ft, V3 mo, V3 f, V3 ti, V3 tj) {
  a.I.ft[0][k] = ft.x;
  a.I.ft[1][k] = ft.y;
  a.I.ft[2][k] = ft.z;
  a.I.mo[0][k] = mo.x;
  a.I.mo[1][k] = mo.y;
  a.I.mo[2][k] = mo.z;
  a.R.f[0][k] = f.x;
  a.R.f[1][k] = f.y;
  a.R.f[2][k] = f.z;
  a.R.ti[0][k] = ti.x;
  a.R.ti[1][k] = ti.y;
  a.R.ti[2][k] = ti.z;
  a.R.tj[0][k] = tj.x;
  a.R.tj[1][k] = tj.y;
  a.R.tj[2][k] = tj.z;
}

__device__ __forceinline__ uint32_t warp_append2(bool want, unsigned long long* counter) {
  const unsigned mask = __ballot_sync(0xffffffffu, want);
  const int lane = threadIdx.x & 31;
  unsigned long long base = 0;
  if (mask) {
    const int leader = __ffs(mask) - 1;
    if (lane == leader) base = atomicAdd(counter, (unsigned long long)__popc(mask));
    base = __shfl_sync(0xffffffffu, base, leader);
  }
  return (uint32_t)base + (uint32_t)__popc(mask & ((1u << lane) - 1u));
}

// Roles of an interaction in the contact law: i = pi_, j = pj_ (swap exchanges owner and partner).
struct Roles {
  uint32_t ip, jp, sub_i, sub_j;
};
__device__ __forceinline__ Roles roles(const PCArgs& a, uint64_t k) {
  const uint32_t meta = a.I.meta[k], sb = a.I.sub[k];
  const uint32_t osub = sb & 0xffffu, psub = sb >> 16;
  const uint32_t A = a.I.owner[k], B = a.I.partner[k];
  if ((meta >> 15) & 1u) return Roles{B, A, psub, osub};
  return Roles{A, B, osub, psub};
}

__device__ __forceinline__ VView pview(const PCArgs& a, uint32_t s) {
  const uint64_t o = (uint64_t)s * a.MV;
  return VView{a.vx + o, a.vy + o, a.vz + o};
}

__global__ void __launch_bounds__(PT) k_pdetect(PCArgs a) {
  const uint64_t k = (uint64_t)blockIdx.x * PT + threadIdx.x;
  bool heavy = false;
  DetD d = det_none();
  if (k < a.ni) {
    const uint32_t meta = a.I.meta[k];
    const uint32_t type = meta_type(meta);
    const V3 mo = mk(a.I.mo[0][k], a.I.mo[1][k], a.I.mo[2][k]);
    bool contact;
    V3 ri, rj = mk(0, 0, 0);
    bool is_pp = type <= DEM_ITYPE_EDGE_EDGE;
    bool is_mesh = false;  // mesh items go to the Hooke pass (types 11, 12 swap the law's roles)
    double dncut;
    const dem_contact_params* hp = &a.cp;
    uint32_t swap = (meta >> 15) & 1u;
    if (!is_pp) {
      const uint32_t p = a.I.owner[k];
      const ShapeDev& sh = a.shapes[a.P.type[p]];
      const double rm = sh.r * a.P.f[HOM][p];
      const V3 vert = pview(a, p)[a.I.sub[k] & 0xffffu];
      const DriverDev& dv = a.drv[a.I.partner[k]];
      d = det_none();
      if (dv.kind == 2) {  // ContactLawRShapeDriverFunc (polyhedron/contact.hpp:305-432)
        is_mesh = true;
        d = poly_mesh_detect(a.mesh[dv.mesh], type, a.I.sub[k] & 0xffffu, a.I.sub[k] >> 16, pview(a, p), sh, rm);
      } else if (dv.kind == 0) {
        const V3 nrm = mk(dv.normal[0], dv.normal[1], dv.normal[2]);
        const V3 proj = dot(vert, nrm) * nrm;
        const V3 s2p = -(mk(dv.center_proj[0], dv.center_proj[1], dv.center_proj[2]) - proj);
        const double dd = vnorm(s2p);
        d.dn = dd - rm;
        if (!(d.dn > 0)) {
          d.c = true;
          d.n = s2p / dd;
          d.cp = vert - d.n * (rm + 0.5 * d.dn);
        }
      } else {
        const V3 proj = vert * mk(dv.axis[0], dv.axis[1], dv.axis[2]);
        const V3 dir = mk(dv.center[0], dv.center[1], dv.center[2]) - proj;
        const double dd = vnorm(dir);
        d.dn = dv.radius - (rm + dd);
        if (!(d.dn > 0)) {
          d.c = true;
          d.n = dir / dd;
          d.cp = vert - d.n * (rm + 0.5 * d.dn);
        }
      }
      ri = mk(a.P.f[RX][p], a.P.f[RY][p], a.P.f[RZ][p]);
      hp = &a.pt.drv(a.cpd, a.P.group[p], a.I.partner[k]);  // the pair's parameters (multimat)
      dncut = hp->dncut;
    } else {
      const Roles R = roles(a, k);
      const ShapeDev& si = a.shapes[a.P.type[R.ip]];
      const ShapeDev& sj = a.shapes[a.P.type[R.jp]];
      const double rim = si.r * a.P.f[HOM][R.ip], rjm = sj.r * a.P.f[HOM][R.jp];
      const VView vi = pview(a, R.ip), vj = pview(a, R.jp);
      bool apart = false;
      if (a.screen) {  // FP32 screen: a pair provably apart skips the FP64 detection
        const uint64_t oi = (uint64_t)R.ip * a.MV, oj = (uint64_t)R.jp * a.MV;
        auto wi = [&](int q) { return f3(a.wx[oi + q], a.wy[oi + q], a.wz[oi + q]); };
        auto wj = [&](int q) { return f3(a.wx[oj + q], a.wy[oj + q], a.wz[oj + q]); };
        const float Rf = (float)(rim + rjm) * 1.000001f;
        if (type == DEM_ITYPE_VERTEX_VERTEX) {
          apart = apart_vv(wi(R.sub_i), wj(R.sub_j), Rf);
        } else if (type == DEM_ITYPE_VERTEX_EDGE) {
          apart = apart_ve(wi(R.sub_i), wj(sj.e[2 * R.sub_j]), wj(sj.e[2 * R.sub_j + 1]), Rf);
        } else if (type == DEM_ITYPE_VERTEX_FACE) {
          const int b = sj.fo[R.sub_j], e = sj.fo[R.sub_j + 1];
          apart = apart_vf(wi(R.sub_i), wj(sj.fv[b]), wj(sj.fv[b + 1]), wj(sj.fv[e - 1]), Rf);
        } else {
          apart = apart_ee(wi(si.e[2 * R.sub_i]), wi(si.e[2 * R.sub_i + 1]), wj(sj.e[2 * R.sub_j]),
                           wj(sj.e[2 * R.sub_j + 1]), Rf);
        }
      }
      switch (apart ? ~0u : type) {
        case ~0u:  // no contact: det_none
          break;
        case DEM_ITYPE_VERTEX_VERTEX:
          d = detect_vv(vi[R.sub_i], rim, vj[R.sub_j], rjm);
          break;
        case DEM_ITYPE_VERTEX_EDGE:
          d = detect_ve(vi[R.sub_i], rim, vj[sj.e[2 * R.sub_j]], vj[sj.e[2 * R.sub_j + 1]], rjm);
          break;
        case DEM_ITYPE_VERTEX_FACE:
          d = detect_vf(vi[R.sub_i], rim, vj, sj, R.sub_j, rjm);
          break;
        default:
          d = detect_ee(vi[si.e[2 * R.sub_i]], vi[si.e[2 * R.sub_i + 1]], rim, vj[sj.e[2 * R.sub_j]],
                        vj[sj.e[2 * R.sub_j + 1]], rjm);
      }
      ri = mk(a.P.f[RX][R.ip], a.P.f[RY][R.ip], a.P.f[RZ][R.ip]);
      rj = mk(a.P.f[RX][R.jp], a.P.f[RY][R.jp], a.P.f[RZ][R.jp]);
      hp = &a.pt.pair(a.cp, a.P.group[R.ip], a.P.group[R.jp]);
      dncut = hp->dncut;
    }
    contact = d.c;
    if (a.cohesive) contact = (contact || d.dn <= dncut);
    if (!contact) {
      const V3 z = mk(0, 0, 0);
      if (a.R.live[k]) {  // item.reset(): history and record zeroed once, then skipped by the gathers
        pwrite(a, k, z, z, z, z, z);
        a.R.live[k] = 0;
      }
      a.cs.write(k, 0.0, d.cp, z, z);  // dn = 0, the detector's contact point
    } else if (a.cohesive && d.dn >= 0 && !is_mesh) {
      a.R.live[k] = 1;
      const dem_contact_params& hkp = *hp;
      const double fn_value = (hkp.fc / hkp.dncut) * d.dn - hkp.fc;
      const V3 f = mk(0, 0, 0) + fn_value * d.n;
      const V3 ti = cross(d.cp - ri, f) + mo;
      a.cs.write(k, d.dn, d.cp, f - mk(0, 0, 0), mk(0, 0, 0));  // fn = f - friction, friction reset
      if (!is_pp) {
        pwrite(a, k, mk(0, 0, 0), mo, f, ti, mk(0, 0, 0));
      } else {
        const V3 tj = cross(d.cp - rj, -f) + (-mo);
        if (swap) pwrite(a, k, mk(0, 0, 0), mo, -f, tj, ti);
        else pwrite(a, k, mk(0, 0, 0), mo, f, ti, tj);
      }
    } else {
      heavy = true;
      a.R.live[k] = 1;  // k_phooke writes the record
    }
  }
  const uint32_t pos = warp_append2(heavy, a.cnt + 1);
  const bool idle = heavy && !(d.dn < 0);  // in the Hooke pass without overlap
  const unsigned im = __ballot_sync(0xffffffffu, idle);
  if (im && (threadIdx.x & 31) == __ffs(im) - 1) atomicAdd(a.cnt + 2, (unsigned long long)__popc(im));
  if (heavy) {
    a.L2[pos] = (uint32_t)k;
    a.D[0][pos] = d.dn;
    a.D[1][pos] = d.n.x;
    a.D[2][pos] = d.n.y;
    a.D[3][pos] = d.n.z;
    a.D[4][pos] = d.cp.x;
    a.D[5][pos] = d.cp.y;
    a.D[6][pos] = d.cp.z;
  }
}

// Fast (the fused step): the contact law with the exact rolling-clip shortcut
// (contact_force_core_m, rolling_clip_mur0); the operator path keeps the
// formula as written.
template <bool Fast>
__device__ __forceinline__ void hooke(bool cohesive, double dn, V3 n, double dt, const dem_contact_params& hkp,
                                      double meff, V3& ft, V3 cpos, V3 pos_i, V3 vel_i, V3& f_i, V3& mom_i,
                                      V3 vrot_i, V3 pos_j, V3 vel_j, V3 vrot_j, bool dmt, double reff) {
  if (Fast) {
    MulFP64 mm;
    contact_force_core_m(mm, cohesive, dn, n, dt, hkp, meff, ft, cpos, pos_i, vel_i, f_i, mom_i, vrot_i, pos_j,
                         vel_j, vrot_j, dmt, reff);
  } else {
    contact_force_core(cohesive, dn, n, dt, hkp, meff, ft, cpos, pos_i, vel_i, f_i, mom_i, vrot_i, pos_j, vel_j,
                       vrot_j, dmt, reff);
  }
}

template <bool Fast>
__global__ void __launch_bounds__(PT) k_phooke(PCArgs a) {
  const uint64_t n2 = a.cnt[1];
  if (blockIdx.x == 0 && threadIdx.x == 0) *a.n_active = n2 - a.cnt[2];
  const uint64_t stride = (uint64_t)gridDim.x * PT;
  for (uint64_t w = (uint64_t)blockIdx.x * PT + threadIdx.x; w < n2; w += stride) {
    const uint32_t k = a.L2[w];
    const double dn = a.D[0][w];
    const V3 n = mk(a.D[1][w], a.D[2][w], a.D[3][w]);
    const V3 cpos = mk(a.D[4][w], a.D[5][w], a.D[6][w]);
    const uint32_t meta = a.I.meta[k];
    V3 ft = mk(a.I.ft[0][k], a.I.ft[1][k], a.I.ft[2][k]);
    V3 mo = mk(a.I.mo[0][k], a.I.mo[1][k], a.I.mo[2][k]);
    V3 f = mk(0, 0, 0);
    if (meta_type(meta) > DEM_ITYPE_EDGE_EDGE) {
      const uint32_t p = a.I.owner[k];
      const DriverDev& d = a.drv[a.I.partner[k]];
      const V3 r = ldv(a.P, RX, p), v = ldv(a.P, VX, p), w_ = ldv(a.P, WX, p);
      const double meff = a.P.f[MASS][p];
      if (d.kind == 2) {
        // ContactLawRShapeDriverFunc (polyhedron/contact.hpp:305-432): reff =
        // compute_effective_radius of the two Minkowski radii; types 7-10 apply the
        // law with the particle as i, 11-12 with the mesh as i: the particle takes
        // -f and -moment, and the friction is stored negated
        const double ra = a.P.f[HOM][p] * a.shapes[a.P.type[p]].r, mr = a.mesh[d.mesh].r;
        const double reff = a.dmt ? (ra * mr) / (ra + mr) : 0.0;
        const dem_contact_params& hp = a.pt.drv(a.cpd, a.P.group[p], a.I.partner[k]);
        const V3 dpos = mk(d.center[0], d.center[1], d.center[2]);
        const V3 dvel = mk(d.vel[0], d.vel[1], d.vel[2]), dvrot = mk(d.vrot[0], d.vrot[1], d.vrot[2]);
        if (meta_type(meta) <= DEM_ITYPE_EDGE_MESH_EDGE) {
          hooke<Fast>(a.cohesive, dn, n, a.dt, hp, meff, ft, cpos, r, v, f, mo, w_, dpos, dvel, dvrot, a.dmt, reff);
          pwrite(a, k, ft, mo, f, cross(cpos - r, f) + mo, mk(0, 0, 0));
          a.cs.write(k, dn, cpos, f - ft, ft);
        } else {
          hooke<Fast>(a.cohesive, dn, n, a.dt, hp, meff, ft, cpos, dpos, dvel, f, mo, dvrot, r, v, w_, a.dmt, reff);
          const V3 fp = -f;
          pwrite(a, k, -ft, mo, fp, cross(cpos - r, fp) + (-mo), mk(0, 0, 0));
          a.cs.write(k, dn, cpos, ft - f, -ft);
        }
        continue;
      }
      // DMT: reff = shp.minkowski(h) (polyhedron/contact.hpp:281)
      const double reff = a.dmt ? a.P.f[HOM][p] * a.shapes[a.P.type[p]].r : 0.0;
      hooke<Fast>(a.cohesive, dn, n, a.dt, a.pt.drv(a.cpd, a.P.group[p], a.I.partner[k]), meff, ft, cpos, r, v, f,
                  mo, w_,
                  mk(d.center[0], d.center[1], d.center[2]), mk(d.vel[0], d.vel[1], d.vel[2]),
                  mk(d.vrot[0], d.vrot[1], d.vrot[2]), a.dmt, reff);
      pwrite(a, k, ft, mo, f, cross(cpos - r, f) + mo, mk(0, 0, 0));
      a.cs.write(k, dn, cpos, f - ft, ft);
      continue;
    }
    const Roles R = roles(a, k);
    const V3 r_i = ldv(a.P, RX, R.ip), r_j = ldv(a.P, RX, R.jp);
    const V3 v_i = ldv(a.P, VX, R.ip), v_j = ldv(a.P, VX, R.jp);
    const V3 w_i = ldv(a.P, WX, R.ip), w_j = ldv(a.P, WX, R.jp);
    const double m_i = a.P.f[MASS][R.ip], m_j = a.P.f[MASS][R.jp];
    const double meff = (m_i * m_j) / (m_i + m_j);
    // DMT: reff = compute_effective_mass(rad_i, rad_j) of the Minkowski radii h r (polyhedron/contact.hpp:179-183)
    double reff = 0.0;
    if (a.dmt) {
      const double rad_i = a.P.f[HOM][R.ip] * a.shapes[a.P.type[R.ip]].r;
      const double rad_j = a.P.f[HOM][R.jp] * a.shapes[a.P.type[R.jp]].r;
      reff = (rad_i * rad_j) / (rad_i + rad_j);
    }
    hooke<Fast>(a.cohesive, dn, n, a.dt, a.pt.pair(a.cp, a.P.group[R.ip], a.P.group[R.jp]), meff, ft, cpos, r_i, v_i,
                f, mo, w_i, r_j, v_j, w_j, a.dmt, reff);
    const V3 t_i = cross(cpos - r_i, f) + mo;
    const V3 t_j = cross(cpos - r_j, -f) + (-mo);
    a.cs.write(k, dn, cpos, f - ft, ft);  // the law's particle i (polyhedron/contact.hpp:191-210)
    if ((meta >> 15) & 1u)
      pwrite(a, k, ft, mo, -f, t_j, t_i);
    else
      pwrite(a, k, ft, mo, f, t_i, t_j);
  }
}

PolyArgs make_pargs(dem_ctx* c) {
  PolyArgs a;
  a.P = c->P[c->pcur];
  a.n = c->n;
  a.shapes = (const ShapeDev*)c->shapes_dev;
  a.MV = c->MV;
  a.vx = c->vtx[0];
  a.vy = c->vtx[1];
  a.vz = c->vtx[2];
  a.bx = c->bvtx[0];
  a.by = c->bvtx[1];
  a.bz = c->bvtx[2];
  a.obb = c->pobb;
  a.fx = c->vrf[0];
  a.fy = c->vrf[1];
  a.fz = c->vrf[2];
  a.fbox = c->pfbox;
  a.qb = c->pqb;
  a.wx = c->vwf[0];
  a.wy = c->vwf[1];
  a.wz = c->vwf[2];
  a.rV = c->prm.rcut_inc;
  return a;
}
}  // namespace

int launch_poly_fused_prolog(dem_ctx* c) {
  DEM_CUDA_TRY(c, cudaMemsetAsync(c->d_scalars, 0, sizeof(unsigned long long), c->stream));
  ProfScope ps(c, K_PROLOG, c->n ? 1 : 0);
  if (!c->n) return DEM_OK;
  const PolyArgs a = make_pargs(c);
  const double dt = c->prm.dt;
  const double md = c->prm.rcut_inc * 0.5;
  const auto kern = by_mode(c->mul_mode, k_poly_fused_prolog<0>, k_poly_fused_prolog<1>, k_poly_fused_prolog<2>,
                            k_poly_fused_prolog<3>);
  kern<<<grid_for(c->n, PT), PT, 0, c->stream>>>(a, dt, dt * 0.5, dt * dt * 0.5, md * md, (float)md, c->d_scalars);
  DEM_CUDA_TRY(c, cudaGetLastError());
  return DEM_OK;
}

int launch_vertex_list(dem_ctx* c) {
  c->nvlist = 0;
  if (!c->n) return DEM_OK;
  DEM_CUDA_TRY(c, cudaMemsetAsync(c->vneed, 0, (c->n + 1) * 4, c->stream));
  if (c->ni)
    k_vertex_needs<<<grid_for(c->ni, 256), 256, 0, c->stream>>>(c->I[c->icur], c->ni, c->vneed);
  int rc = launch_bond_needs(c, c->vneed);  // the bonded vertices are read every step
  if (rc) return rc;
  rc = scan_exclusive_u32(c, c->vneed, c->vneed_off, c->n);
  if (rc) return rc;
  k_vertex_compact<<<grid_for(c->n, 256), 256, 0, c->stream>>>(c->vneed, c->vneed_off, c->n, c->vlist);
  uint32_t cnt = 0;
  DEM_CUDA_TRY(c, cudaMemcpyAsync(&cnt, c->vneed_off + c->n, 4, cudaMemcpyDeviceToHost, c->stream));
  DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  c->nvlist = cnt;
  return DEM_OK;
}

int launch_poly_vertices_listed(dem_ctx* c) {
  ProfScope ps(c, K_PROLOG, c->nvlist ? 1 : 0);
  if (!c->nvlist) return DEM_OK;
  const PolyArgs a = make_pargs(c);
  const auto kern = by_mode(c->mul_mode, k_poly_vertices_listed<0>, k_poly_vertices_listed<1>,
                            k_poly_vertices_listed<2>, k_poly_vertices_listed<3>);
  kern<<<grid_for(c->nvlist * (uint64_t)c->MV, PT), PT, 0, c->stream>>>(a, c->vlist, c->nvlist);
  DEM_CUDA_TRY(c, cudaGetLastError());
  return DEM_OK;
}

// vertices (+ displacement flag, or + backup and world OBBs at a rebuild)
int launch_poly_vertices(dem_ctx* c, int mode) {
  if (!c->n) return DEM_OK;
  ProfScope ps(c, K_PROLOG, 1);
  const PolyArgs a = make_pargs(c);
  const double md = c->prm.rcut_inc * 0.5;
  if (mode == 1) {
    DEM_CUDA_TRY(c, cudaMemsetAsync(c->d_scalars, 0, sizeof(unsigned long long), c->stream));
    k_poly_vertices<true, false><<<grid_for(c->n, PT), PT, 0, c->stream>>>(a, md * md, c->d_scalars);
  } else if (mode == 2) {
    k_poly_vertices<false, true><<<grid_for(c->n, PT), PT, 0, c->stream>>>(a, 0.0, nullptr);
  } else {
    k_poly_vertices<false, false><<<grid_for(c->n, PT), PT, 0, c->stream>>>(a, 0.0, nullptr);
  }
  DEM_CUDA_TRY(c, cudaGetLastError());
  return DEM_OK;
}

// Units + SAT; returns the number of units in *nu (host sync).
int launch_poly_units(dem_ctx* c, uint64_t* nu_out, int (*grow_units)(dem_ctx*, uint64_t)) {
  UnitArgs a;
  a.P = c->P[c->pcur];
  a.n = c->n;
  a.g = c->grid;
  a.cell_start = c->cell_start;
  a.cell_of = c->cell_of;
  a.drv = c->drv_dev;
  a.ndrv = c->ndrv;
  a.mesh = c->mesh_dev;
  a.shapes = (const ShapeDev*)c->shapes_dev;
  a.rV = c->prm.rcut_inc;
  const double nd = 2 * c->rad_max + c->prm.rcut_inc;
  a.rcut2 = nd * nd;
  a.xr = c->crel[0];
  a.yr = c->crel[1];
  a.zr = c->crel[2];
  a.rf = c->crel[3];
  for (int d = 0; d < 3; d++) a.csz[d] = (float)c->grid.csz[d];
  a.skin_f = (float)c->prm.rcut_inc;
  a.f32 = c->prm.fp32_broad_phase;
  a.b_first = c->nb ? c->b_own_first : nullptr;
  a.b_cnt = c->nb ? c->b_own_cnt : nullptr;
  a.b_idj = c->nb ? c->B[c->bcur].id_j : nullptr;
  a.urec = c->urec;
  {
    ProfScope ps(c, K_BROAD_COUNT, 1);
    k_unit_count<<<grid_for(c->n, PT), PT, 0, c->stream>>>(a, c->pcnt);
  }
  int rc = scan_exclusive_u32(c, c->pcnt, c->u_off, c->n);
  if (rc) return rc;
  uint32_t nu = 0;
  DEM_CUDA_TRY(c, cudaMemcpyAsync(&nu, c->u_off + c->n, 4, cudaMemcpyDeviceToHost, c->stream));
  DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  if ((rc = grow_units(c, nu))) return rc;
  ProfScope ps(c, K_BROAD_FILL, 2);
  k_unit_fill<<<grid_for(c->n, PT), PT, 0, c->stream>>>(a, c->u_off, c->u_owner, c->u_partner, c->u_pid, c->u_kind);
  if (nu)
    k_unit_sat<<<grid_for(nu, PT), PT, 0, c->stream>>>(nu, c->u_owner, c->u_partner, c->u_kind, c->pobb,
                                                       c->prm.rcut_inc, c->u_pass);
  DEM_CUDA_TRY(c, cudaGetLastError());
  *nu_out = nu;
  return DEM_OK;
}

static FeatArgs make_fargs(dem_ctx* c, uint64_t nu) {
  FeatArgs a;
  a.P = c->P[c->pcur];
  a.shapes = (const ShapeDev*)c->shapes_dev;
  a.drv = c->drv_dev;
  a.mesh = c->mesh_dev;
  a.MV = c->MV;
  a.vx = c->vtx[0];
  a.vy = c->vtx[1];
  a.vz = c->vtx[2];
  a.obb = c->pobb;
  a.rV = c->prm.rcut_inc;
  a.nu = nu;
  a.u_owner = c->u_owner;
  a.u_partner = c->u_partner;
  a.u_pid = c->u_pid;
  a.u_kind = c->u_kind;
  a.pass = c->u_pass;
  a.fcnt = c->f_cnt;
  a.foff = c->f_off;
  a.dst = c->I[1 - c->icur];
  a.old = c->I[c->icur];
  a.old_off = c->own_off[c->icur];
  a.perm = c->perm;
  a.have_old = c->hist_valid ? 1 : 0;
  a.fvx = c->vrf[0];
  a.fvy = c->vrf[1];
  a.fvz = c->vrf[2];
  a.fbox = c->pfbox;
  a.slots = c->u_slots;
  a.slot_off = c->learned_slots ? c->u_slotoff : nullptr;
  a.order = (c->learned_slots && c->prm.learned_sizing >= 2) ? c->u_order : nullptr;
  a.utypes = c->u_types;
  a.bh_oid = c->bh_oid;
  a.bh_pid = c->bh_pid;
  a.bh_sub = c->bh_sub;
  for (int d = 0; d < 3; d++) a.bh_ft[d] = c->bh_ft[d];
  a.nbh = c->nbh;
  return a;
}

int launch_poly_feature_count(dem_ctx* c, uint64_t nu, uint32_t* total) {
  FeatArgs a = make_fargs(c, nu);
  const unsigned blocks = (unsigned)std::min<uint64_t>((nu * 32 + PT - 1) / PT + 1, (uint64_t)c->num_sms * 16);
  const bool mesh = !c->meshes.empty();
  c->t_flat = nu && c->prm.fp32_broad_phase && !c->learned_slots;
  if (c->t_flat) {  // flattened enumeration: prep, scan of the test counts, tests, per-unit counts
    UnitRec* rec = reinterpret_cast<UnitRec*>(c->u_rec);
    {
      ProfScope ps(c, K_BROAD_COUNT, 1);
      k_feat_prep<<<blocks, PT, 0, c->stream>>>(a, rec, c->t_cnt);
    }
    int rc = scan_exclusive_u32(c, c->t_cnt, c->t_off, 6 * nu);
    if (rc) return rc;
    uint32_t nt = 0;
    DEM_CUDA_TRY(c, cudaMemcpyAsync(&nt, c->t_off + 6 * nu, 4, cudaMemcpyDeviceToHost, c->stream));
    DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    const uint64_t words = ((uint64_t)nt + 31) / 32;
    if (words > c->t_keepcap) {
      cudaFree(c->t_keep);
      c->t_keep = nullptr;
      c->t_keepcap = 0;
      const uint64_t cap = words + words / 4 + 1024;
      DEM_CUDA_TRY(c, cudaMalloc(&c->t_keep, cap * 4));
      c->t_keepcap = cap;
    }
    ProfScope ps(c, K_BROAD_COUNT, (nt ? 2 : 1) + (mesh ? 1 : 0));
    if (nt) {
      const unsigned tb = (unsigned)std::min<uint64_t>((words * 32 + PT - 1) / PT, (uint64_t)c->num_sms * 32);
      k_feat_test<<<tb, PT, 0, c->stream>>>(a, rec, c->t_off, nt, c->t_keep);
    }
    k_feat_collect<false><<<blocks, PT, 0, c->stream>>>(a, rec, c->t_off, c->t_keep, c->t_cnt);
    c->t_ntests = nt;
    if (mesh) k_mesh_units<false, true><<<blocks, PT, 0, c->stream>>>(a);
  } else {
    ProfScope ps(c, K_BROAD_COUNT, nu ? (mesh ? 2 : 1) : 0);
    if (nu && c->prm.fp32_broad_phase)
      k_feat_dec<false><<<blocks, PT, 0, c->stream>>>(a);
    else if (nu)
      k_feat<false><<<blocks, PT, 0, c->stream>>>(a);
    if (nu && mesh && c->prm.fp32_broad_phase)
      k_mesh_units<false, true><<<blocks, PT, 0, c->stream>>>(a);
    else if (nu && mesh)
      k_mesh_units<false, false><<<blocks, PT, 0, c->stream>>>(a);
  }
  int rc = scan_exclusive_u32(c, c->f_cnt, c->f_off, nu);
  if (rc) return rc;
  if (c->learned_slots && nu) {  // pairs whose features overflowed the predicted record
    DEM_CUDA_TRY(c, cudaMemsetAsync(c->d_scalars + SC_LEARNED_OVF, 0, sizeof(unsigned long long), c->stream));
    k_learned_overflow<<<grid_for(nu, 256), 256, 0, c->stream>>>(nu, c->f_cnt, c->u_slotoff, c->d_scalars + SC_LEARNED_OVF);
  }
  unsigned long long ovf = 0;
  DEM_CUDA_TRY(c, cudaMemcpyAsync(total, c->f_off + nu, 4, cudaMemcpyDeviceToHost, c->stream));
  if (c->learned_slots)
    DEM_CUDA_TRY(c, cudaMemcpyAsync(&ovf, c->d_scalars + SC_LEARNED_OVF, 8, cudaMemcpyDeviceToHost, c->stream));
  DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  c->learned_overflow = ovf;
  c->nu_last = nu;
  c->labels_valid = c->prm.fp32_broad_phase != 0;  // the FP32-decided count pass writes the labels
  return DEM_OK;
}

int launch_poly_feature_fill(dem_ctx* c, uint64_t nu) {
  FeatArgs a = make_fargs(c, nu);
  const unsigned blocks = (unsigned)std::min<uint64_t>((nu * 32 + PT - 1) / PT + 1, (uint64_t)c->num_sms * 16);
  const bool mesh = !c->meshes.empty();
  ProfScope ps(c, K_BROAD_FILL, mesh ? 4 : 2);
  if (nu && c->t_flat) {
    const UnitRec* rec = reinterpret_cast<const UnitRec*>(c->u_rec);
    if (c->ndrv) k_feat_collect<true><<<blocks, PT, 0, c->stream>>>(a, rec, c->t_off, c->t_keep, nullptr);
    const uint32_t nt = c->t_ntests;
    if (nt) {
      const unsigned tb = (unsigned)std::min<uint64_t>(((uint64_t)nt + PT - 1) / PT, (uint64_t)c->num_sms * 32);
      k_feat_fill_flat<<<tb, PT, 0, c->stream>>>(a, rec, c->t_off, nt, c->t_keep, c->t_cnt);
    }
  }
  else if (nu && c->prm.fp32_broad_phase)
    k_feat_dec<true><<<blocks, PT, 0, c->stream>>>(a);
  else if (nu)
    k_feat<true><<<blocks, PT, 0, c->stream>>>(a);
  if (nu && mesh && c->prm.fp32_broad_phase)
    k_mesh_units<true, true><<<blocks, PT, 0, c->stream>>>(a);
  else if (nu && mesh)
    k_mesh_units<true, false><<<blocks, PT, 0, c->stream>>>(a);
  if (nu && mesh)
    k_mesh_unit_sort<<<grid_for(nu, 128), 128, 0, c->stream>>>(nu, c->u_kind, c->u_partner, c->drv_dev, c->f_off,
                                                              a.dst);
  k_own_from_units<<<grid_for(c->n + 1, 256), 256, 0, c->stream>>>(c->n, c->u_off, c->f_off, c->own_off[1 - c->icur]);
  DEM_CUDA_TRY(c, cudaGetLastError());
  return DEM_OK;
}

int launch_unit_features(dem_ctx* c, uint64_t nu) {
  if (!nu) return DEM_OK;
  k_unit_features<<<grid_for(nu, 128), 128, 0, c->stream>>>(nu, c->P[c->pcur], c->u_owner, c->u_partner, c->u_kind,
                                                             c->u_pass, c->pfbox, (float)c->prm.rcut_inc, c->u_x);
  DEM_CUDA_TRY(c, cudaGetLastError());
  return DEM_OK;
}

// MLP rates -> per-unit feature records (scan) and the bin order of the count pass
int launch_learned_sizing(dem_ctx* c, uint64_t nu) {
  int rc = mlp_rates(c, c->u_x, nu, c->u_rates);
  if (rc) return rc;
  unsigned int* d_bins = reinterpret_cast<unsigned int*>(c->d_scalars + SC_LEARNED_BINS);  // 7 counters, 7 cursors
  DEM_CUDA_TRY(c, cudaMemsetAsync(d_bins, 0, 14 * sizeof(unsigned int), c->stream));
  k_learned_caps<<<grid_for(nu, 256), 256, 0, c->stream>>>(nu, c->P[c->pcur], (const ShapeDev*)c->shapes_dev,
                                                            c->u_owner, c->u_kind, c->u_pass, c->u_rates, c->f_cnt,
                                                            c->u_order, d_bins);
  if ((rc = scan_exclusive_u32(c, c->f_cnt, c->u_slotoff, nu))) return rc;
  unsigned int bins[7];
  uint32_t total = 0;
  DEM_CUDA_TRY(c, cudaMemcpyAsync(bins, d_bins, sizeof(bins), cudaMemcpyDeviceToHost, c->stream));
  DEM_CUDA_TRY(c, cudaMemcpyAsync(&total, c->u_slotoff + nu, 4, cudaMemcpyDeviceToHost, c->stream));
  if ((rc = mlp_check(c))) return rc;  // synchronises the stream
  if (total > c->slot_cap) {
    cudaFree(c->u_slots);
    c->u_slots = nullptr;
    c->slot_cap = 0;
    DEM_CUDA_TRY(c, cudaMalloc(&c->u_slots, ((uint64_t)total + total / 4 + 1024) * sizeof(uint16_t)));
    c->slot_cap = (uint64_t)total + total / 4 + 1024;
  }
  unsigned int cursor[7];
  unsigned int acc = 0;
  for (int b = 0; b < 7; b++) {
    cursor[b] = acc;
    acc += bins[b];
  }
  // the bins were written into u_order by k_learned_caps: copy them out, then sort
  uint32_t* bin_of = c->u_types;  // free until the count pass writes the labels
  DEM_CUDA_TRY(c, cudaMemcpyAsync(bin_of, c->u_order, nu * 4, cudaMemcpyDeviceToDevice, c->stream));
  DEM_CUDA_TRY(c, cudaMemcpyAsync(d_bins + 7, cursor, sizeof(cursor), cudaMemcpyHostToDevice, c->stream));
  k_learned_order<<<grid_for(nu, 256), 256, 0, c->stream>>>(nu, bin_of, d_bins + 7, c->u_order);
  DEM_CUDA_TRY(c, cudaGetLastError());
  c->learned_slots = true;
  c->learned_units = nu;
  return DEM_OK;
}

int launch_harvest(dem_ctx* c, float* x, uint8_t* y, uint64_t capacity, uint64_t* count, uint64_t* available) {
  const uint64_t nu = c->nu_last;
  *count = *available = 0;
  if (!nu) return DEM_OK;
  int rc = launch_unit_features(c, nu);
  if (rc) return rc;
  uint32_t* flag = c->u_slotoff;  // scratch: flags, then positions in u_order
  k_harvest_flags<<<grid_for(nu, 256), 256, 0, c->stream>>>(nu, c->u_kind, c->u_pass, flag);
  if ((rc = scan_exclusive_u32(c, flag, c->u_order, nu))) return rc;
  uint32_t tot = 0;
  DEM_CUDA_TRY(c, cudaMemcpyAsync(&tot, c->u_order + nu, 4, cudaMemcpyDeviceToHost, c->stream));
  k_harvest_write<<<grid_for(nu, 256), 256, 0, c->stream>>>(nu, flag, c->u_order, c->u_x, c->u_types, capacity, x, y);
  DEM_CUDA_TRY(c, cudaGetLastError());
  DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  *available = tot;
  *count = std::min<uint64_t>(tot, capacity);
  return DEM_OK;
}

int launch_contact_poly(dem_ctx* c) {
  DEM_CUDA_TRY(c, cudaMemsetAsync(c->d_scalars + 3, 0, 3 * sizeof(unsigned long long), c->stream));
  ProfScope ps(c, K_CONTACT, 2);
  PCArgs a;
  a.P = c->P[c->pcur];
  a.I = c->I[c->icur];
  a.R = c->R;
  a.ni = c->ni;
  a.shapes = (const ShapeDev*)c->shapes_dev;
  a.drv = c->drv_dev;
  a.MV = c->MV;
  a.vx = c->vtx[0];
  a.vy = c->vtx[1];
  a.vz = c->vtx[2];
  a.wx = c->vwf[0];
  a.wy = c->vwf[1];
  a.wz = c->vwf[2];
  a.cp = c->prm.config;
  a.cpd = c->prm.config_driver;
  a.dt = c->prm.dt;
  a.cohesive = c->prm.law == DEM_LAW_HOOKE_COHESIVE;
  a.dmt = c->prm.law == DEM_LAW_HOOKE_DMT;
  a.screen = c->prm.fused_step && c->prm.fp32_contact_screen && !a.cohesive && !a.dmt && !c->cs.dn;
  a.pt = c->ptable();
  a.cs = c->cs;
  a.mesh = c->mesh_dev;
  a.L2 = c->L2;
  for (int q = 0; q < 7; q++) a.D[q] = c->Dscr[q];
  a.cnt = c->d_scalars + 3;
  a.n_active = c->d_scalars + 1;
  if (c->ni) k_pdetect<<<grid_for(c->ni, PT), PT, 0, c->stream>>>(a);
  if (c->prm.fused_step)
    k_phooke<true><<<(unsigned)c->num_sms * 8u, PT, 0, c->stream>>>(a);
  else
    k_phooke<false><<<(unsigned)c->num_sms * 8u, PT, 0, c->stream>>>(a);
  DEM_CUDA_TRY(c, cudaGetLastError());
  return DEM_OK;
}
}  // namespace dem
