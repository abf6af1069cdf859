// k_step_fused.cu -- the optimised Verlet step: fewer launches, dense FP64 warps.
//
// FP64 on GB300 runs at 2 thread-instructions per clock per SM (1/64 of FP32),
// so the step is bound by the FP64 pipe, not by HBM.  Two consequences drive
// this file, and neither changes a single result bit:
//  * lanes that need no FP64 work must not share a warp with lanes that do:
//    a warp instruction with one active lane costs the FP64 pipe as much as a
//    full one.  The contact law therefore runs in three passes:
//      k_cscreen  one thread per interaction; an FP32 test proves most pairs
//                 apart (history reset, zero record, no FP64 at all); the others
//                 are appended to list L1 with warp-aggregated atomics;
//      k_cdetect  dense over L1: FP64 detection; no contact -> reset; cohesive
//                 attraction without overlap (cheap branch) finished here;
//                 overlapping pairs append (k, dn, n, cp) to list L2;
//      k_chooke   dense over L2: the full Hooke law with friction and rolling.
//  * the divisions by mass and inertia use exact reciprocal-based division
//    (math_exact.cuh) and reset + gravity + gather + force_to_accel + epilog
//    are one kernel, prolog + displacement trigger another.
// Order of summation, operation order and rounding are those of the operator
// kernels (contact_core.cuh, integrate_core.cuh).
#include "contact_core.cuh"
#include "integrate_core.cuh"
#include "mesh_core.cuh"

namespace dem {
namespace {

constexpr int FT = 128;  // threads per block

// All 32 lanes must call it.  Returns the slot of this lane when want is set.
__device__ __forceinline__ uint32_t warp_append(bool want, unsigned long long* counter) {
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

struct CArgs {
  PArrays P;
  IArrays I;
  Records R;
  uint64_t ni;
  const unsigned long long* ni_dev;  // graph step: the count lives on the device
  SysView sv;  // periodic lengths of the owner's system
  const DriverDev* drv;
  const MeshDev* mesh;
  dem_contact_params cp, cpd;
  double dt;
  int cohesive;
  int dmt;        // Hooke_DMT law combination
  ParamTable pt;  // multi-material parameters (pt.pp == nullptr: cp / cpd)
  ContactStateArrays cs;  // analysis (cs.dn == nullptr: off)
  int screen;
  uint32_t* L1;
  uint32_t* L2;
  double* D[7];  // dn, n(3), cp(3) of the L2 entries
  unsigned long long* cnt;  // [0] L1 count (particle pairs), [1] L2 count, [2] driver pairs of L1
  uint64_t l1cap;           // L1 entries: particle pairs from the front, driver pairs from the back
  int int_share;            // k_cfused: Hooke tiles out of 8 run with AllInt (the integer pipe)
  unsigned long long* n_active;
};

// L1 as one list: the particle pairs (front, n1 of them), then the driver pairs
// (stored from the back).  Grouping the two kinds keeps each warp on one
// detection and one law, so neither runs with the other's lanes idle.
__device__ __forceinline__ uint32_t l1_at(const CArgs& a, uint64_t w, uint64_t n1) {
  return w < n1 ? a.L1[w] : a.L1[a.l1cap - 1 - (w - n1)];
}

__device__ __forceinline__ void write_result(const CArgs& a, uint64_t k, V3 ft, V3 mo, V3 f, V3 ti, V3 tj) {
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

// partner position, moved by the periodic lengths of the owner i's system for an image
__device__ __forceinline__ V3 partner_pos(const CArgs& a, uint32_t meta, uint32_t i, uint32_t j) {
  V3 rj = ldv(a.P, RX, j);
  const int sx = meta_shift(meta, 0), sy = meta_shift(meta, 1), sz = meta_shift(meta, 2);
  if (sx | sy | sz) {
    const GridDev& g = a.sv.g[a.sv.of(i)];
    if (sx) rj.x = rj.x + (double)sx * g.L[0];
    if (sy) rj.y = rj.y + (double)sy * g.L[1];
    if (sz) rj.z = rj.z + (double)sz * g.L[2];
  }
  return rj;
}

__global__ void __launch_bounds__(FT) k_cscreen(CArgs a) {
  const uint64_t ni = a.ni_dev ? *a.ni_dev : a.ni;
  const uint64_t stride = (uint64_t)gridDim.x * FT;
  for (uint64_t base = (uint64_t)blockIdx.x * FT; base < ni; base += stride) {
  const uint64_t k = base + threadIdx.x;
  bool want = false, drv = false;
  if (k < ni) {
    const uint32_t meta = a.I.meta[k];
    want = true;
    drv = meta_type(meta) != DEM_ITYPE_VERTEX_VERTEX;
    if (a.screen && meta_type(meta) == DEM_ITYPE_VERTEX_VERTEX) {
      const uint32_t i = a.I.owner[k], j = a.I.partner[k];
      const V3 ri = ldv(a.P, RX, i);
      const V3 rj = partner_pos(a, meta, i, j);
      const double rad_i = a.P.f[RAD][i], rad_j = a.P.f[RAD][j];
      // same proof of separation as the one-pass kernel (k_contact_sphere.cu)
      const float ex = (float)(ri.x - rj.x), ey = (float)(ri.y - rj.y), ez = (float)(ri.z - rj.z);
      const float d2f = ex * ex + ey * ey + ez * ez;
      const double lim =
          rad_i + rad_j + (a.cohesive ? fmax(a.pt.pair(a.cp, a.P.group[i], a.P.group[j]).dncut, 0.0) : 0.0);
      const float limf = (float)lim;
      if (lim > 1e-15 && lim < 1e15 && d2f > limf * limf * 1.0000039f) {
        want = false;
        if (a.R.live[k]) {  // not yet zero: reset history and record once
          const V3 z = mk(0, 0, 0);
          write_result(a, k, z, z, z, z, z);
          a.R.live[k] = 0;
        }
      }
    }
  }
  drv = drv && want;
  const uint32_t pos = warp_append(want && !drv, a.cnt);
  const uint32_t pd = warp_append(drv, a.cnt + 2);
  if (want && !drv) a.L1[pos] = (uint32_t)k;
  if (drv) a.L1[a.l1cap - 1 - pd] = (uint32_t)k;
  }
}

// FP64 detection of interaction k; a pair that does not touch is finished here.
// Returns PAIR_DONE for it, PAIR_HOOKE for an overlapping pair and PAIR_ATTRACT
// for the cohesive attraction before contact; their law is left to the caller
// (hooke_pair, attract_pair) with (dn, n, cpos).
constexpr int PAIR_DONE = 0, PAIR_HOOKE = 1, PAIR_ATTRACT = 2;
__device__ __forceinline__ int detect_pair(const CArgs& a, uint32_t k, double& dn, V3& n, V3& cpos) {
  int kind = PAIR_DONE;
  const uint32_t meta = a.I.meta[k];
  const uint32_t i = a.I.owner[k], j = a.I.partner[k];
  const V3 ri = ldv(a.P, RX, i);
  const double rad_i = a.P.f[RAD][i];
  bool contact;
  bool is_vv = meta_type(meta) == DEM_ITYPE_VERTEX_VERTEX;
  V3 rj = mk(0, 0, 0);
  double dncut;
  if (is_vv) {
    rj = partner_pos(a, meta, i, j);
    const double rad_j = a.P.f[RAD][j];
    const double R = rad_i + rad_j;
    const V3 dist = ri - rj;
    const double dist_norm = vnorm(dist);
    dn = dist_norm - R;
    contact = emu_lt0(dn);  // comparisons of this kernel on the integer pipe (emu64.cuh)
    dncut = a.pt.pair(a.cp, a.P.group[i], a.P.group[j]).dncut;
    if (contact || (a.cohesive && emu_le(dn, dncut)) || a.cs.dn) {  // n and cpos are used only then
      const double inv_dist_norm = 1.0 / dist_norm;
      n = dist * inv_dist_norm;
      cpos = ri - n * (rad_i + 0.5 * dn);
    }
  } else {
    const DriverDev& d = a.drv[j];
    if (d.kind == 2) {  // detect<7|8|9> (contact_sphere.hpp:300-396)
      const DetD q = mesh_detect(a.mesh[d.mesh], meta_type(meta), a.I.sub[k] >> 16, ri, rad_i);
      dn = q.dn;
      contact = q.c;
      n = q.n;
      cpos = q.cp;
    } else if (d.kind == 0) {
      const V3 nrm = mk(d.normal[0], d.normal[1], d.normal[2]);
      const V3 proj = dot(ri, nrm) * nrm;
      const V3 s2p = -(mk(d.center_proj[0], d.center_proj[1], d.center_proj[2]) - proj);
      const double dd = vnorm(s2p);
      dn = dd - rad_i;
      contact = !emu_gt0(dn);
      if (contact) {
        n = s2p / dd;
        cpos = ri - n * (rad_i + 0.5 * dn);
      }
    } else {
      const V3 proj = ri * mk(d.axis[0], d.axis[1], d.axis[2]);
      const V3 dir = mk(d.center[0], d.center[1], d.center[2]) - proj;
      const double dd = vnorm(dir);
      dn = d.radius - (rad_i + dd);
      contact = !emu_gt0(dn);
      if (contact) {
        n = dir / dd;
        cpos = ri - n * (rad_i + 0.5 * dn);
      }
    }
    dncut = a.pt.drv(a.cpd, a.P.group[i], j).dncut;
  }
  if (a.cohesive) contact = (contact || emu_le(dn, dncut));
  if (!contact) {
    a.cs.write(k, 0.0, cpos, mk(0, 0, 0), mk(0, 0, 0));  // item.reset(), dn = 0
    if (a.R.live[k] || a.cs.dn) {
      const V3 z = mk(0, 0, 0);
      write_result(a, k, z, z, z, z, z);
      a.R.live[k] = 0;
    }
  } else if (a.cohesive && emu_ge0(dn)) {
    kind = PAIR_ATTRACT;
  } else {
    kind = PAIR_HOOKE;
  }
  return kind;
}

// cohesive attraction before contact (contact_force.hpp:165-173): f = fn_value n, ft = 0
__device__ __forceinline__ void attract_pair(const CArgs& a, uint32_t k, double dn, V3 n, V3 cpos) {
  const uint32_t meta = a.I.meta[k];
  const uint32_t i = a.I.owner[k], j = a.I.partner[k];
  const bool is_vv = meta_type(meta) == DEM_ITYPE_VERTEX_VERTEX;
  const V3 ri = ldv(a.P, RX, i);
  const V3 mo = mk(a.I.mo[0][k], a.I.mo[1][k], a.I.mo[2][k]);
  const dem_contact_params& hkp =
      is_vv ? a.pt.pair(a.cp, a.P.group[i], a.P.group[j]) : a.pt.drv(a.cpd, a.P.group[i], j);
  const double fn_value = (hkp.fc / hkp.dncut) * dn - hkp.fc;
  const V3 f = mk(0, 0, 0) + fn_value * n;
  const V3 ti = cross(cpos - ri, f) + mo;
  V3 tj = mk(0, 0, 0);
  if (is_vv) tj = cross(cpos - partner_pos(a, meta, i, j), -f) + (-mo);
  write_result(a, k, mk(0, 0, 0), mo, f, ti, tj);
  a.R.live[k] = 1;
  a.cs.write(k, dn, cpos, f - mk(0, 0, 0), mk(0, 0, 0));  // ft = 0 before contact
}

__global__ void __launch_bounds__(FT) k_cdetect(CArgs a) {
  const uint64_t n1 = a.cnt[0], nl = n1 + a.cnt[2];
  const uint64_t stride = (uint64_t)gridDim.x * FT;
  for (uint64_t base = (uint64_t)blockIdx.x * FT; base < nl; base += stride) {
    const uint64_t w = base + threadIdx.x;
    bool heavy = false;
    uint32_t k = 0;
    double dn = 0;
    V3 n = mk(0, 0, 0), cpos = mk(0, 0, 0);
    if (w < nl) {
      k = l1_at(a, w, n1);
      const int kind = detect_pair(a, k, dn, n, cpos);
      if (kind == PAIR_ATTRACT) attract_pair(a, k, dn, n, cpos);
      heavy = kind == PAIR_HOOKE;
    }
    const uint32_t pos = warp_append(heavy, a.cnt + 1);
    if (heavy) {
      a.L2[pos] = k;
      a.D[0][pos] = dn;
      a.D[1][pos] = n.x;
      a.D[2][pos] = n.y;
      a.D[3][pos] = n.z;
      a.D[4][pos] = cpos.x;
      a.D[5][pos] = cpos.y;
      a.D[6][pos] = cpos.z;
    }
  }
}

// The Hooke law of one overlapping pair with the arithmetic policy Pol
// (mul_policy.cuh): MulFP64, MulInt (its multiplies on the integer pipe) or
// AllInt (multiplies and additions there).  An operand outside an integer
// path makes the pair run again on the FP64 pipe from its stored inputs
// (nothing is written before write_result): the same bits in every case.
template <class M>
__device__ __forceinline__ void hooke_run(M& mm, const CArgs& a, uint32_t k, double dn, V3 n, V3 cpos, V3& ft,
                                          V3& mo, V3& f, V3& ti, V3& tj) {
  const uint32_t meta = a.I.meta[k];
  const uint32_t i = a.I.owner[k], j = a.I.partner[k];
  const V3 ri = ldv(a.P, RX, i);
  ft = mk(a.I.ft[0][k], a.I.ft[1][k], a.I.ft[2][k]);
  mo = mk(a.I.mo[0][k], a.I.mo[1][k], a.I.mo[2][k]);
  f = mk(0, 0, 0);
  tj = mk(0, 0, 0);
  const V3 vi = ldv(a.P, VX, i);
  const V3 wi = ldv(a.P, WX, i);
  if (meta_type(meta) == DEM_ITYPE_VERTEX_VERTEX) {
    const V3 rj = partner_pos(a, meta, i, j);
    const V3 vj = ldv(a.P, VX, j), wj = ldv(a.P, WX, j);
    // the pair's damping coefficient, set when the list was built (k_fill); DMT:
    // reff = compute_effective_radius (common_kernels.hpp:99-102)
    double reff = 0.0;
    if (a.dmt) {
      const double rad_i = a.P.f[RAD][i], rad_j = a.P.f[RAD][j];
      reff = mm.mul(rad_i, rad_j) / mm.add(rad_i, rad_j);
    }
    const dem_contact_params& cp = a.pt.pair(a.cp, a.P.group[i], a.P.group[j]);
    contact_force_core_m<M, true>(mm, a.cohesive, dn, n, a.dt, cp, a.I.damp[k], ft, cpos, ri, vi, f, mo, wi, rj,
                                  vj, wj, a.dmt, reff);
    ti = add_m(mm, cross_m(mm, sub_m(mm, cpos, ri), f), mo);
    tj = add_m(mm, cross_m(mm, sub_m(mm, cpos, rj), -f), -mo);
  } else {
    const DriverDev& d = a.drv[j];
    const V3 dpos = mk(d.center[0], d.center[1], d.center[2]);
    const V3 dvel = mk(d.vel[0], d.vel[1], d.vel[2]);
    const V3 dvrot = mk(d.vrot[0], d.vrot[1], d.vrot[2]);
    const dem_contact_params& cpd = a.pt.drv(a.cpd, a.P.group[i], j);
    contact_force_core_m<M, true>(mm, a.cohesive, dn, n, a.dt, cpd, a.I.damp[k], ft, cpos, ri, vi, f, mo, wi, dpos,
                                  dvel, dvrot, a.dmt, a.P.f[RAD][i]);
    ti = add_m(mm, cross_m(mm, sub_m(mm, cpos, ri), f), mo);
  }
}

// The Hooke law of one overlapping pair with the arithmetic policy Pol
// (mul_policy.cuh): MulFP64, MulInt (its multiplies on the integer pipe) or
// AllInt (multiplies and additions there).  An operand outside an integer
// path makes the pair run again on the FP64 pipe from its stored inputs
// (nothing is written before write_result): the same bits in every case.
template <class Pol>
__device__ __forceinline__ void hooke_pair_p(const CArgs& a, uint32_t k, double dn, V3 n, V3 cpos) {
  V3 ft, mo, f, ti, tj;
  Pol mm;
  hooke_run(mm, a, k, dn, n, cpos, ft, mo, f, ti, tj);
  if (mm.failed()) {
    asm volatile("" ::: "memory");
    MulFP64 nm;
    hooke_run(nm, a, k, dn, n, cpos, ft, mo, f, ti, tj);
  }
  write_result(a, k, ft, mo, f, ti, tj);
  a.R.live[k] = 1;
  if (a.cs.dn) a.cs.write(k, dn, cpos, f - ft, ft);
}

// Mode bit 2 (instance 1): the law's multiplies on the integer pipe
template <int Mode>
__device__ __forceinline__ void hooke_pair(const CArgs& a, uint32_t k, double dn, V3 n, V3 cpos) {
  hooke_pair_p<RotMul<Mode>>(a, k, dn, n, cpos);
}

// The Hooke law on the contacts found by k_cdetect.  Mode bit 2 (instance 1):
// its multiplies on the integer pipe (contact_force_core_m); an operand outside
// that fast path makes the pair run again on the FP64 pipe from its stored
// inputs (nothing is written before write_result).
template <int Mode>
__global__ void __launch_bounds__(FT, (Mode ? 4 : 1)) k_chooke(CArgs a) {
  const uint64_t n2 = a.cnt[1];
  if (blockIdx.x == 0 && threadIdx.x == 0) *a.n_active = n2;  // every L2 pair overlaps (dn < 0)
  const uint64_t stride = (uint64_t)gridDim.x * FT;
  for (uint64_t w = (uint64_t)blockIdx.x * FT + threadIdx.x; w < n2; w += stride)
    hooke_pair<Mode>(a, a.L2[w], a.D[0][w], mk(a.D[1][w], a.D[2][w], a.D[3][w]), mk(a.D[4][w], a.D[5][w], a.D[6][w]));
}

// The law of queued pair idx of queue q (0: Hooke, 1: attraction); a share of
// the Hooke tiles runs on the integer pipe, so both pipes work at once.
template <int Mode, bool IntTiles>
__device__ __forceinline__ void run_queued(const CArgs& a, int q, uint32_t idx, const uint32_t* qk,
                                           const double (*qd)[2 * FT], uint32_t& tiles) {
  const V3 n = mk(qd[1][idx], qd[2][idx], qd[3][idx]);
  const V3 cpos = mk(qd[4][idx], qd[5][idx], qd[6][idx]);
  if (q == 0) {
    if (IntTiles && (int)(tiles & 7u) < a.int_share)
      hooke_pair_p<AllInt>(a, qk[idx], qd[0][idx], n, cpos);
    else
      hooke_pair<Mode>(a, qk[idx], qd[0][idx], n, cpos);
    tiles++;
  } else {
    attract_pair(a, qk[idx], qd[0][idx], n, cpos);
  }
}

// Detection and the contact laws in one kernel.  The pairs a block's detection
// finds overlapping (Hooke law) or within the cohesion distance (attraction)
// wait in shared memory, one queue per law, until a full tile of one kind is
// ready; then every thread of the block runs that law on one of them, so the
// FP64 warps stay dense and on one law, while the detection results never go
// through global memory.  The particle pairs of L1 come before its driver
// pairs, so the warps of both stages see one kind of pair at a time.  Each
// pair is computed exactly as by k_cdetect + k_chooke and writes only its own
// records: the same bits.  The overlapping pairs are counted into *n_active
// (zeroed by the launcher).
// IntTiles: the instance with the integer-pipe tiles (int_share > 0); it needs
// more registers, so the FP64-only instance stays the lean one.
template <int Mode, bool IntTiles>
__global__ void __launch_bounds__(FT, (Mode ? 4 : (IntTiles ? 3 : 1))) k_cfused(CArgs a) {
  __shared__ uint32_t q_k[2][2 * FT];
  __shared__ double q_d[2][7][2 * FT];
  __shared__ uint32_t q_n[2], q_tot;
  if (threadIdx.x == 0) {
    q_n[0] = q_n[1] = 0;
    q_tot = 0;
  }
  __syncthreads();
  const uint64_t n1 = a.cnt[0], nl = n1 + a.cnt[2];
  const uint64_t stride = (uint64_t)gridDim.x * FT;
  const int lane = threadIdx.x & 31;
  const uint32_t t = threadIdx.x;
  uint32_t tiles = 0;  // Hooke tiles run by this block (the same count in every thread)
  for (uint64_t base = (uint64_t)blockIdx.x * FT; base < nl; base += stride) {  // the same trips for the block
    const uint64_t w = base + threadIdx.x;
    int kind = PAIR_DONE;
    uint32_t k = 0;
    double dn = 0;
    V3 n = mk(0, 0, 0), cpos = mk(0, 0, 0);
    if (w < nl) {
      k = l1_at(a, w, n1);
      kind = detect_pair(a, k, dn, n, cpos);
    }
#pragma unroll
    for (int q = 0; q < 2; q++) {
      const bool mine = kind == (q == 0 ? PAIR_HOOKE : PAIR_ATTRACT);
      const unsigned mask = __ballot_sync(0xffffffffu, mine);
      uint32_t wb = 0;
      if (lane == 0 && mask) {
        wb = atomicAdd(&q_n[q], (uint32_t)__popc(mask));
        if (q == 0) atomicAdd(&q_tot, (uint32_t)__popc(mask));
      }
      wb = __shfl_sync(0xffffffffu, wb, 0);
      if (mine) {
        const uint32_t pos = wb + (uint32_t)__popc(mask & ((1u << lane) - 1u));  // < 2 FT: at most FT - 1 wait
        q_k[q][pos] = k;
        q_d[q][0][pos] = dn;
        q_d[q][1][pos] = n.x;
        q_d[q][2][pos] = n.y;
        q_d[q][3][pos] = n.z;
        q_d[q][4][pos] = cpos.x;
        q_d[q][5][pos] = cpos.y;
        q_d[q][6][pos] = cpos.z;
      }
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 2; q++) {
      const uint32_t have = q_n[q];
      if (have >= FT) {  // a full tile: one pair per thread
        run_queued<Mode, IntTiles>(a, q, t, q_k[q], q_d[q], tiles);
        __syncthreads();
        const uint32_t rest = have - FT;  // < FT: the waiting pairs move to the front
        if (t < rest) {
          q_k[q][t] = q_k[q][FT + t];
#pragma unroll
          for (int c = 0; c < 7; c++) q_d[q][c][t] = q_d[q][c][FT + t];
        }
        if (t == 0) q_n[q] = rest;
        __syncthreads();
      }
    }
  }
  if (t < q_n[0]) run_queued<Mode, IntTiles>(a, 0, t, q_k[0], q_d[0], tiles);
  if (t < q_n[1]) run_queued<Mode, IntTiles>(a, 1, t, q_k[1], q_d[1], tiles);
  if (t == 0 && q_tot) atomicAdd(a.n_active, (unsigned long long)q_tot);
}

// prolog + displacement trigger.  Every particle gets its translation and, when
// it does not spin, its (exact, integer sign logic) quaternion step here; the
// spinning particles run the full quaternion update in place when most of their
// warp spins, otherwise through prl_list in k_prolog_rotation, so sparse
// spinning particles do not hold whole warps on the FP64 pipe.  The trigger
// depends on positions only.
template <int Mode>
__global__ void __launch_bounds__(256, (Mode ? 3 : 1)) k_fused_prolog(PArrays P, uint64_t n, double delta_t,
                                                                     double half_delta_t, double delta_t2_2,
                                                                     double thr2, unsigned long long* flag,
                                                                     SysView sv, uint32_t* prl_list,
                                                                     unsigned long long* prl_cnt) {
  const uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  bool over = false, need = false;
  if (s < n) {
    need = prolog_cheap<Mode>(P, s, delta_t, half_delta_t, delta_t2_2);
    const double dx = P.f[RX][s] - P.f[BX][s], dy = P.f[RY][s] - P.f[BY][s], dz = P.f[RZ][s] - P.f[BZ][s];
    over = emu_ge_nonneg(dx * dx + dy * dy + dz * dz, thr2);  // >= on the integer pipe
    if (over && sv.nsys > 1) atomicOr(&sv.trig[sv.of(s)], 1u);  // this system's own trigger
  }
  if (__any_sync(0xffffffffu, over) && (threadIdx.x & 31) == 0) atomicOr(flag, 1ull);
  const unsigned busy = __ballot_sync(0xffffffffu, need);
  if (__popc(busy) > 24) {
    if (need) prolog_rotation<Mode>(P, s, delta_t, half_delta_t);
  } else {
    const uint32_t pos = warp_append(need, prl_cnt);
    if (need) prl_list[pos] = (uint32_t)s;
  }
}

// the rotational half of the prolog for the particles listed by k_fused_prolog
template <int Mode>
__global__ void __launch_bounds__(256, (Mode ? 3 : 1)) k_prolog_rotation(PArrays P, const uint32_t* __restrict__ list,
                                                                        const unsigned long long* cnt, double delta_t,
                                                                        double half_delta_t) {
  const uint64_t m = *cnt;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t w = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; w < m; w += stride)
    prolog_rotation<Mode>(P, list[w], delta_t, half_delta_t);
}

// reset_force_moment + gravity_force + contact gather + force_to_accel + epilog.
// The velocity half of the epilog runs here for every particle.  The
// rotational half is exactly zero for a particle without spin and torque
// (rotation_idle); the others run it here when most of their warp needs it,
// otherwise they are appended to rot_list for k_epilog_rotation, so sparse
// rotating particles do not hold whole warps on the FP64 pipe.
// Mode != 0: the integer-pipe multiplies raise register use; at most 80
// registers keep 3 blocks of 256 per SM (measured faster than 2 blocks)
template <int Mode>
__global__ void __launch_bounds__(256, (Mode ? 3 : 1)) k_fused_epilog(PArrays P, Records R, uint64_t n,
                                                                     const uint32_t* __restrict__ own_off,
                                                                     const uint32_t* __restrict__ rev_off,
                                                                     const uint32_t* __restrict__ rev_idx,
                                                                     double gx, double gy, double gz,
                                                                     double half_delta_t, uint32_t* rot_list,
                                                                     unsigned long long* rot_cnt) {
  const uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  bool need = false;
  V3 mom = mk(0.0, 0.0, 0.0);
  if (s < n) {
    const double m = P.f[MASS][s];
    // 0.0 + g_c m is +0 for g_c = +-0 and a finite m (+0 + +-0 = +0): no FP64 work
    const bool mfin = ((emu_bits(m) >> 52) & 0x7ffu) != 0x7ffu;
    V3 f = mk(emu_is_zero(gx) && mfin ? 0.0 : 0.0 + gx * m, emu_is_zero(gy) && mfin ? 0.0 : 0.0 + gy * m,
              emu_is_zero(gz) && mfin ? 0.0 : 0.0 + gz * m);
    // f and mom start at +0 or a nonzero value and, in round to nearest, never
    // become -0 (x + (-x) = +0; -0 needs two -0 operands), so a record whose six
    // components are all +-0 (a listed pair that does not touch) leaves them
    // unchanged bit for bit and its additions are skipped.
    // (a record whose live flag is 0 is zero and is not read)
    // The owned records, then the partner records, in one loop: a particle's
    // owned and partner counts vary a lot (by id order), their sum (its
    // neighbour count) much less, so one loop keeps the warp's FP64 adds on
    // most lanes.  The order of the additions is that of two loops.
    const uint32_t o0 = own_off[s], no = own_off[s + 1] - o0;
    const uint32_t r0 = rev_off[s], nt = no + (rev_off[s + 1] - r0);
    for (uint32_t m = 0; m < nt; m++) {
      const bool own = m < no;
      const uint32_t k = own ? o0 + m : rev_idx[r0 + (m - no)];
      if (!R.live[k]) continue;
      const double* t0 = own ? R.ti[0] : R.tj[0];
      const double* t1 = own ? R.ti[1] : R.tj[1];
      const double* t2 = own ? R.ti[2] : R.tj[2];
      const V3 rf = mk(R.f[0][k], R.f[1][k], R.f[2][k]), rt = mk(t0[k], t1[k], t2[k]);
      if (((emu_bits(rf.x) | emu_bits(rf.y) | emu_bits(rf.z) | emu_bits(rt.x) | emu_bits(rt.y) | emu_bits(rt.z))
           << 1) != 0) {
        const uint64_t flip = own ? 0ull : 0x8000000000000000ull;  // -rf for a partner record (exact)
        f = f + mk(emu_double(emu_bits(rf.x) ^ flip), emu_double(emu_bits(rf.y) ^ flip),
                   emu_double(emu_bits(rf.z) ^ flip));
        mom = mom + rt;
      }
    }
    const double im = P.f[IMASS][s];
    LinMul<Mode> lm;
    V3 acc = mk(div_rn_m(lm, f.x, m, im), div_rn_m(lm, f.y, m, im), div_rn_m(lm, f.z, m, im));
    const V3 vel = mk(P.f[VX][s], P.f[VY][s], P.f[VZ][s]);
    // v + a dt/2: a zero a gives the zero addend of emu_add_zero (integer pipe)
    const bool hok = emu_nonneg_finite(half_delta_t);
    auto vstep = [&](double vc, double ac) {
      if (hok && emu_is_zero(ac)) {
        bool ok;
        const double r = emu_add_zero(vc, emu_sign(ac), ok);
        if (ok) return r;
      }
      return vc + lm.mul(ac, half_delta_t);
    };
    V3 v = mk(vstep(vel.x, acc.x), vstep(vel.y, acc.y), vstep(vel.z, acc.z));
    if (lm.failed()) {
      acc = mk(div_rn(f.x, m, im), div_rn(f.y, m, im), div_rn(f.z, m, im));
      v = mk(vel.x + acc.x * half_delta_t, vel.y + acc.y * half_delta_t, vel.z + acc.z * half_delta_t);
    }
    P.f[FX][s] = acc.x;
    P.f[FY][s] = acc.y;
    P.f[FZ][s] = acc.z;
    P.f[MX][s] = mom.x;
    P.f[MY][s] = mom.y;
    P.f[MZ][s] = mom.z;
    P.f[VX][s] = v.x;
    P.f[VY][s] = v.y;
    P.f[VZ][s] = v.z;
    const V3 vrot = mk(P.f[WX][s], P.f[WY][s], P.f[WZ][s]);
    need = true;
    if (((emu_bits(vrot.x) | emu_bits(vrot.y) | emu_bits(vrot.z) | emu_bits(mom.x) | emu_bits(mom.y) |
          emu_bits(mom.z))) == 0) {
      const Q4 Q = {P.f[QW][s], P.f[QX][s], P.f[QY][s], P.f[QZ][s]};
      const V3 I = mk(P.f[IX][s], P.f[IY][s], P.f[IZ][s]);
      const V3 II = mk(P.f[IIX][s], P.f[IIY][s], P.f[IIZ][s]);
      if (rotation_idle(Q, vrot, mom, I, II)) {
        need = false;
        P.f[AX][s] = 0.0;  // w stays +0
        P.f[AY][s] = 0.0;
        P.f[AZ][s] = 0.0;
      }
    }
  }
  const unsigned busy = __ballot_sync(0xffffffffu, need);
  if (__popc(busy) > 24) {
    if (need) epilog_rotation<Mode>(P, s, half_delta_t, mom);
  } else {
    const uint32_t pos = warp_append(need, rot_cnt);
    if (need) rot_list[pos] = (uint32_t)s;
  }
}

// the rotational half of the epilog for the particles listed by k_fused_epilog
template <int Mode>
__global__ void __launch_bounds__(256, (Mode ? 3 : 1)) k_epilog_rotation(PArrays P, const uint32_t* __restrict__ rot_list,
                                                                        const unsigned long long* rot_cnt,
                                                                        double half_delta_t) {
  const uint64_t cnt = *rot_cnt;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t w = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; w < cnt; w += stride) {
    const uint32_t s = rot_list[w];
    epilog_rotation<Mode>(P, s, half_delta_t, mk(P.f[MX][s], P.f[MY][s], P.f[MZ][s]));
  }
}

CArgs make_cargs(dem_ctx* c) {
  CArgs a;
  a.P = c->P[c->pcur];
  a.I = c->I[c->icur];
  a.R = c->R;
  a.ni = c->ni;
  a.ni_dev = c->capturing ? c->d_ni : nullptr;
  a.sv = c->sysview();
  a.drv = c->drv_dev;
  a.mesh = c->mesh_dev;
  a.cp = c->prm.config;
  a.cpd = c->prm.config_driver;
  a.dt = c->prm.dt;
  a.cohesive = c->prm.law == DEM_LAW_HOOKE_COHESIVE;
  a.dmt = c->prm.law == DEM_LAW_HOOKE_DMT;
  a.pt = c->ptable();
  a.cs = c->cs;
  a.screen = c->prm.fp32_contact_screen && !c->analysis;  // analysis: every pair's state
  a.L1 = c->L1;
  a.L2 = c->L2;
  for (int q = 0; q < 7; q++) a.D[q] = c->Dscr[q];
  a.cnt = c->d_scalars + 3;
  a.l1cap = c->rcap;
  a.int_share = c->tune_int_share;
  a.n_active = c->d_scalars + 1;
  return a;
}
}  // namespace

int launch_fused_prolog(dem_ctx* c) {
  const double delta_t = c->prm.dt;
  const double half_delta_t = delta_t * 0.5;
  const double delta_t2_2 = delta_t * delta_t * 0.5;
  const double max_displ = c->prm.rcut_inc * 0.5;
  DEM_CUDA_TRY(c, cudaMemsetAsync(c->d_scalars, 0, sizeof(unsigned long long), c->stream));
  unsigned long long* prl_cnt = c->d_scalars + SC_ROT_CNT;  // the rotation list is free until the epilog
  DEM_CUDA_TRY(c, cudaMemsetAsync(prl_cnt, 0, sizeof(unsigned long long), c->stream));
  ProfScope ps(c, K_PROLOG, c->n ? 2 : 0);
  const auto kern = by_mode(c->mul_mode, k_fused_prolog<0>, k_fused_prolog<1>, k_fused_prolog<2>, k_fused_prolog<3>);
  const auto krot = by_mode(c->mul_mode, k_prolog_rotation<0>, k_prolog_rotation<1>, k_prolog_rotation<2>,
                            k_prolog_rotation<3>);
  if (c->n) {
    kern<<<grid_for(c->n, c->tune_block), c->tune_block, 0, c->stream>>>(c->P[c->pcur], c->n, delta_t, half_delta_t,
                                                                         delta_t2_2, max_displ * max_displ,
                                                                         c->d_scalars, c->sysview(), c->rot_list,
                                                                         prl_cnt);
    krot<<<(unsigned)c->num_sms * 3, 256, 0, c->stream>>>(c->P[c->pcur], c->rot_list, prl_cnt, delta_t,
                                                            half_delta_t);
  }
  DEM_CUDA_TRY(c, cudaGetLastError());
  return DEM_OK;
}

int launch_contact_compact(dem_ctx* c) {
  DEM_CUDA_TRY(c, cudaMemsetAsync(c->d_scalars + 3, 0, 3 * sizeof(unsigned long long), c->stream));
  const CArgs a = make_cargs(c);
  const unsigned persistent = (unsigned)c->num_sms * (unsigned)c->tune_contact_bps;
  {
    ProfScope ps(c, K_CSCREEN, c->capturing || c->ni ? 1 : 0);
    if (c->capturing)
      k_cscreen<<<persistent, FT, 0, c->stream>>>(a);
    else if (c->ni)
      k_cscreen<<<grid_for(c->ni, FT), FT, 0, c->stream>>>(a);
  }
  if (c->fuse_contact) {  // detection and law in one kernel (k_cfused)
    DEM_CUDA_TRY(c, cudaMemsetAsync(a.n_active, 0, sizeof(unsigned long long), c->stream));
    ProfScope ps(c, K_CONTACT, 1);
    // mode bit 2: the contact law's multiplies on the integer pipe; int_share: a
    // share of its tiles with multiplies and additions there
    const auto kf = (c->mul_mode & 4) ? k_cfused<1, false>
                                      : (c->tune_int_share > 0 ? k_cfused<0, true> : k_cfused<0, false>);
    kf<<<persistent, FT, 0, c->stream>>>(a);
  } else {
    {
      ProfScope ps(c, K_CDETECT, 1);
      k_cdetect<<<persistent, FT, 0, c->stream>>>(a);
    }
    ProfScope ps(c, K_CONTACT, 1);  // the Hooke law on the contacts
    const auto kh = (c->mul_mode & 4) ? k_chooke<1> : k_chooke<0>;  // mode bit 2: the contact law
    kh<<<persistent, FT, 0, c->stream>>>(a);
  }
  DEM_CUDA_TRY(c, cudaGetLastError());
  return DEM_OK;
}

int launch_fused_epilog(dem_ctx* c) {
  ProfScope ps(c, K_EPILOG, c->n ? 2 : 0);
  const auto kern = by_mode(c->mul_mode, k_fused_epilog<0>, k_fused_epilog<1>, k_fused_epilog<2>, k_fused_epilog<3>);
  const auto krot = by_mode(c->mul_mode, k_epilog_rotation<0>, k_epilog_rotation<1>, k_epilog_rotation<2>,
                            k_epilog_rotation<3>);
  unsigned long long* rot_cnt = c->d_scalars + SC_ROT_CNT;
  DEM_CUDA_TRY(c, cudaMemsetAsync(rot_cnt, 0, sizeof(unsigned long long), c->stream));
  if (c->n) {
    kern<<<grid_for(c->n, c->tune_block), c->tune_block, 0, c->stream>>>(
        c->P[c->pcur], c->R, c->n, c->own_off[c->icur], c->rev_off, c->rev_idx, c->prm.gravity[0],
        c->prm.gravity[1], c->prm.gravity[2], c->prm.dt * 0.5, c->rot_list, rot_cnt);
    krot<<<(unsigned)c->num_sms * 3, 256, 0, c->stream>>>(c->P[c->pcur], c->rot_list, rot_cnt, c->prm.dt * 0.5);
  }
  DEM_CUDA_TRY(c, cudaGetLastError());
  return DEM_OK;
}
}  // namespace dem
