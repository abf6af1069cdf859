// k_bond.cu -- fragmentation: inner bonds between polyhedra.
//
// The bonds (InnerBondInteraction, inner_bond_interaction.hpp:28-62) live in
// structure-of-arrays form in bond order (id_i, id_j, sub_i, sub_j), double
// buffered for the compaction at a rebuild; an interface is a run of bonds of
// one particle pair (interface.hpp:27-31).
//  - dem_stick_polyhedra (host, once, stick_polyhedra.cpp:60-360) makes them
//    from the vertices computed on the device;
//  - k_bond_criterion, one thread per interface, right after the prolog:
//    apply_interface_fracture_criterion (apply_interface_fracture_criterion.hpp:
//    35-76) on the previous bond pass, then broken_interface_friction_updater
//    (broken_interface_friction_updater.cpp:52-86) on a broken one, which also
//    raises the rebuild flag (config_fragmentation.msp displ_or_break);
//  - at a rebuild, a stable compaction moves the broken bonds into a table of
//    vertex-vertex history (broke_interaction, inner_bond_interaction.hpp:
//    202-210) that the feature fill searches by key when the old list has no
//    entry, the interfaces are rebuilt (update_interfaces.cpp:48-79), the bonds
//    follow the particle reorder and each slot gets the list of its owned bonds
//    and of the bonds where it is j; the unit enumeration lists nothing between
//    bonded particles (interaction_manager.hpp:114-160);
//  - after the contact gather, k_bond_force (one thread per bond: vertex-vertex
//    detection of the bonded vertices and force_law_core, inner_bond.hpp:
//    112-186, inner_bond_force.hpp:24-70) and k_bond_gather (one thread per
//    particle: owned bonds, then the bonds where it is j, in bond order).
// Operation order is that of the reference (compiled with --fmad=false): the
// results are bit-identical to the CPU restatement.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <unordered_map>
#include <vector>

#include "dem_ctx.cuh"
#include "poly_core.cuh"

namespace dem {
namespace {

constexpr int BT = 256;

struct BondArgs {
  PArrays P;
  BondArrays B;
  uint64_t nb;
  const ShapeDev* shapes;
  int MV;
  const double* vx;
  const double* vy;
  const double* vz;
  const dem_inner_bond_params* ibp;  // ng == 0: ibp[0] for every pair
  int ng;
  double dt;
};

__host__ __device__ __forceinline__ const dem_inner_bond_params& bond_params(const dem_inner_bond_params* ibp, int ng,
                                                                           uint32_t gi, uint32_t gj) {
  return ng == 0 ? ibp[0] : ibp[gi * (uint32_t)ng + gj];
}

// force_law_core (forcefield/inner_bond_force.hpp:24-70)
__device__ __forceinline__ void bond_law(double dn, V3 n, double dn0, double weight, double dt,
                                         const dem_inner_bond_params& p, double meff, double& En, V3& tds,
                                         double& Et, V3& ft, V3 cp, V3 pos_i, V3 vel_i, V3& f_i, V3 vrot_i,
                                         V3 pos_j, V3 vel_j, V3 vrot_j) {
  const double damp = p.damp_rate * 2.0 * sqrt(p.kn * meff);
  const V3 contribution_i = vel_i - cross(cp - pos_i, vrot_i);
  const V3 contribution_j = vel_j - cross(cp - pos_j, vrot_j);
  const V3 vel = contribution_j - contribution_i;
  const double vn = dot(vel, n);
  const double delta = dn - dn0;
  const double kn_w = p.kn * weight;
  const double kt_w = p.kt * weight;
  const double fne = -kn_w * delta;
  const double fnv = damp * vn;
  const double fn = fne + fnv;
  const V3 vfn = fn * n;
  const V3 vt = vel - vn * n;
  const V3 ds = dt * vt;
  tds = tds + ds;
  ft = kt_w * tds;
  f_i = vfn + ft;
  En = static_cast<double>(fne <= 0) * (0.5 * kn_w * delta * delta);
  Et = 0.5 * kt_w * dot(tds, tds);
}

__global__ void __launch_bounds__(BT) k_bond_force(BondArgs a) {
  const uint64_t b = (uint64_t)blockIdx.x * BT + threadIdx.x;
  if (b >= a.nb) return;
  const BondArrays& B = a.B;
  const PArrays& P = a.P;
  const uint32_t i = B.i[b], j = B.j[b], sub = B.sub[b];
  const uint64_t vi = (uint64_t)i * a.MV + (sub & 0xffffu), vj = (uint64_t)j * a.MV + (sub >> 16);
  const double ri = a.shapes[P.type[i]].r * P.f[HOM][i];
  const double rj = a.shapes[P.type[j]].r * P.f[HOM][j];
  const DetD d = detect_vv(mk(a.vx[vi], a.vy[vi], a.vz[vi]), ri, mk(a.vx[vj], a.vy[vj], a.vz[vj]), rj);
  const V3 pos_i = mk(P.f[RX][i], P.f[RY][i], P.f[RZ][i]), pos_j = mk(P.f[RX][j], P.f[RY][j], P.f[RZ][j]);
  const double mi = P.f[MASS][i], mj = P.f[MASS][j];
  const double meff = (mi * mj) / (mi + mj);
  double En = 0.0, Et = 0.0;
  V3 tds = mk(B.tds[0][b], B.tds[1][b], B.tds[2][b]), ft, f;
  bond_law(d.dn, d.n, B.dn0[b], B.weight[b], a.dt, bond_params(a.ibp, a.ng, P.group[i], P.group[j]), meff, En, tds,
           Et, ft, d.cp, pos_i, mk(P.f[VX][i], P.f[VY][i], P.f[VZ][i]), f, mk(P.f[WX][i], P.f[WY][i], P.f[WZ][i]),
           pos_j, mk(P.f[VX][j], P.f[VY][j], P.f[VZ][j]), mk(P.f[WX][j], P.f[WY][j], P.f[WZ][j]));
  const V3 z = mk(0.0, 0.0, 0.0);
  const V3 ti = cross(d.cp - pos_i, f) + z;  // compute_moments with a zero moment
  const V3 tj = cross(d.cp - pos_j, -f) + z;
  const V3 fnv = f - ft;
  const double* src[15] = {&tds.x, &tds.y, &tds.z, &ft.x, &ft.y, &ft.z, &f.x, &f.y, &f.z,
                           &ti.x,  &ti.y,  &ti.z,  &tj.x, &tj.y, &tj.z};
  double* dst[15] = {B.tds[0], B.tds[1], B.tds[2], B.ft[0], B.ft[1], B.ft[2], B.f[0], B.f[1], B.f[2],
                     B.ti[0],  B.ti[1],  B.ti[2],  B.tj[0], B.tj[1], B.tj[2]};
#pragma unroll
  for (int q = 0; q < 15; q++) dst[q][b] = *src[q];
  B.en[b] = En;
  B.et[b] = Et;
  B.dn[b] = d.dn;
  B.fn[0][b] = fnv.x;
  B.fn[1][b] = fnv.y;
  B.fn[2][b] = fnv.z;
}

__global__ void __launch_bounds__(BT) k_bond_gather(PArrays P, BondArrays B, uint64_t n,
                                                    const uint32_t* __restrict__ own_first,
                                                    const uint32_t* __restrict__ own_cnt,
                                                    const uint32_t* __restrict__ rev_off,
                                                    const uint32_t* __restrict__ rev_idx) {
  const uint64_t s = (uint64_t)blockIdx.x * BT + threadIdx.x;
  if (s >= n) return;
  const uint32_t c0 = own_cnt[s], r0 = rev_off[s], r1 = rev_off[s + 1];
  if (c0 == 0 && r0 == r1) return;
  V3 f = mk(P.f[FX][s], P.f[FY][s], P.f[FZ][s]);
  V3 m = mk(P.f[MX][s], P.f[MY][s], P.f[MZ][s]);
  const uint32_t b0 = c0 ? own_first[s] : 0u;
  for (uint32_t k = b0; k < b0 + c0; k++) {
    f = f + mk(B.f[0][k], B.f[1][k], B.f[2][k]);
    m = m + mk(B.ti[0][k], B.ti[1][k], B.ti[2][k]);
  }
  for (uint32_t q = r0; q < r1; q++) {
    const uint32_t k = rev_idx[q];
    f = f + (-mk(B.f[0][k], B.f[1][k], B.f[2][k]));
    m = m + mk(B.tj[0][k], B.tj[1][k], B.tj[2][k]);
  }
  P.f[FX][s] = f.x;
  P.f[FY][s] = f.y;
  P.f[FZ][s] = f.z;
  P.f[MX][s] = m.x;
  P.f[MY][s] = m.y;
  P.f[MZ][s] = m.z;
}

struct CritArgs {
  BondArrays B;
  const uint32_t* iface;
  uint64_t nif;
  const uint32_t* group;
  dem_contact_params cp;  // singlemat contact parameters (mu of the friction updater)
  ParamTable pt;
  unsigned long long* flag;    // rebuild flag
  unsigned long long* broken;  // interfaces broken
};

__global__ void __launch_bounds__(BT) k_bond_criterion(CritArgs a) {
  const uint64_t q = (uint64_t)blockIdx.x * BT + threadIdx.x;
  if (q >= a.nif) return;
  const BondArrays& B = a.B;
  const uint32_t off = a.iface[q], end = a.iface[q + 1];
  double En = 0.0, Et = 0.0, S = 0.0;
  for (uint32_t j = off; j < end; j++) {
    En += B.en[j];
    Et += B.et[j];
    if (B.dn[j] > 0.0) S += vnorm(mk(B.fn[0][j], B.fn[1][j], B.fn[2][j]));
  }
  S /= (double)(end - off);
  const int mode = B.mode[off];
  const double c1 = B.c1[off], c2 = B.c2[off];
  bool brk = false;
  if (mode == DEM_RUPTURE_ENERGY_MIXED) {
    if (En + Et > c1) brk = true;
  } else if (mode == DEM_RUPTURE_ENERGY_SEPARATE) {
    if (En > c1 || Et > c2) brk = true;
  } else if (mode == DEM_RUPTURE_STRESS_ENERGY_SEPARATE) {
    if ((En > c1) && (S > c2)) brk = true;
  }
  if (!brk) return;
  for (uint32_t j = off; j < end; j++) {
    B.unbroken[j] = 0;
    const V3 ftv = mk(B.ft[0][j], B.ft[1][j], B.ft[2][j]);
    const double ft = vnorm(ftv);
    const double mu = a.pt.pair(a.cp, a.group[B.i[j]], a.group[B.j[j]]).mu;
    const double ft_threshold = mu * vnorm(mk(B.fn[0][j], B.fn[1][j], B.fn[2][j]));
    V3 nf = ftv;
    if (ft > ft_threshold && ft > 0) nf = ftv * ft_threshold / ft;
    if (B.dn[j] > 0) nf = mk(0.0, 0.0, 0.0);
    B.ft[0][j] = nf.x;
    B.ft[1][j] = nf.y;
    B.ft[2][j] = nf.z;
  }
  atomicAdd(a.broken, 1ull);
  atomicExch(a.flag, 1ull);
}

// ---- rebuild: compaction, interfaces, new slots, per-slot lists
__global__ void k_bond_keep_flags(const uint8_t* __restrict__ unbroken, uint64_t nb, uint32_t* __restrict__ flag) {
  const uint64_t b = (uint64_t)blockIdx.x * BT + threadIdx.x;
  if (b < nb) flag[b] = unbroken[b] ? 1u : 0u;
}

struct BondHist {
  uint64_t* oid;
  uint64_t* pid;
  uint32_t* sub;
  double* ft[3];
};

__global__ void k_bond_compact(BondArrays S, BondArrays D, uint64_t nb, const uint32_t* __restrict__ pos,
                               BondHist H) {
  const uint64_t b = (uint64_t)blockIdx.x * BT + threadIdx.x;
  if (b >= nb) return;
  if (!S.unbroken[b]) {  // broke_interaction: vertex-vertex pair, friction kept, moment 0
    const uint64_t h = b - pos[b];
    H.oid[h] = S.id_i[b];
    H.pid[h] = S.id_j[b];
    H.sub[h] = S.sub[b];
    for (int d = 0; d < 3; d++) H.ft[d][h] = S.ft[d][b];
    return;
  }
  const uint32_t w = pos[b];
  D.id_i[w] = S.id_i[b];
  D.id_j[w] = S.id_j[b];
  D.i[w] = S.i[b];
  D.j[w] = S.j[b];
  D.sub[w] = S.sub[b];
  D.mode[w] = S.mode[b];
  D.unbroken[w] = 1;
  D.dn0[w] = S.dn0[b];
  D.weight[w] = S.weight[b];
  D.c1[w] = S.c1[b];
  D.c2[w] = S.c2[b];
  D.en[w] = S.en[b];
  D.et[w] = S.et[b];
  D.dn[w] = S.dn[b];
  for (int d = 0; d < 3; d++) {
    D.ft[d][w] = S.ft[d][b];
    D.tds[d][w] = S.tds[d][b];
    D.f[d][w] = S.f[d][b];
    D.ti[d][w] = S.ti[d][b];
    D.tj[d][w] = S.tj[d][b];
    D.fn[d][w] = S.fn[d][b];
  }
}

__global__ void k_iface_flags(const uint64_t* __restrict__ id_i, const uint64_t* __restrict__ id_j, uint64_t nb,
                              uint32_t* __restrict__ flag) {
  const uint64_t b = (uint64_t)blockIdx.x * BT + threadIdx.x;
  if (b < nb) flag[b] = (b == 0 || id_i[b] != id_i[b - 1] || id_j[b] != id_j[b - 1]) ? 1u : 0u;
}

__global__ void k_iface_write(const uint32_t* __restrict__ flag, const uint32_t* __restrict__ pos, uint64_t nb,
                              uint32_t* __restrict__ iface) {
  const uint64_t b = (uint64_t)blockIdx.x * BT + threadIdx.x;
  if (b < nb && flag[b]) iface[pos[b]] = (uint32_t)b;
}

__global__ void k_inv_perm(const uint32_t* __restrict__ perm, uint64_t n, uint32_t* __restrict__ inv) {
  const uint64_t s = (uint64_t)blockIdx.x * BT + threadIdx.x;
  if (s < n) inv[perm[s]] = (uint32_t)s;
}

__global__ void k_bond_remap(uint32_t* __restrict__ bi, uint32_t* __restrict__ bj, uint64_t nb,
                             const uint32_t* __restrict__ inv) {
  const uint64_t b = (uint64_t)blockIdx.x * BT + threadIdx.x;
  if (b >= nb) return;
  bi[b] = inv[bi[b]];
  bj[b] = inv[bj[b]];
}

// owned bonds of a slot: the run of its id_i (bonds are sorted by id_i)
__global__ void k_bond_own(const uint64_t* __restrict__ id_i, const uint32_t* __restrict__ bi, uint64_t nb,
                           uint32_t* __restrict__ first, uint32_t* __restrict__ cnt) {
  const uint64_t b = (uint64_t)blockIdx.x * BT + threadIdx.x;
  if (b >= nb || (b > 0 && id_i[b] == id_i[b - 1])) return;
  uint64_t e = b + 1;
  while (e < nb && id_i[e] == id_i[b]) e++;
  first[bi[b]] = (uint32_t)b;
  cnt[bi[b]] = (uint32_t)(e - b);
}

__global__ void k_bond_rev_count(const uint32_t* __restrict__ bj, uint64_t nb, uint32_t* __restrict__ cnt) {
  const uint64_t b = (uint64_t)blockIdx.x * BT + threadIdx.x;
  if (b < nb) atomicAdd(&cnt[bj[b]], 1u);
}

__global__ void k_bond_rev_fill(const uint32_t* __restrict__ bj, uint64_t nb, uint32_t* __restrict__ cur,
                                uint32_t* __restrict__ idx) {
  const uint64_t b = (uint64_t)blockIdx.x * BT + threadIdx.x;
  if (b < nb) idx[atomicAdd(&cur[bj[b]], 1u)] = (uint32_t)b;
}

// the bonds where a slot is j, in bond order (a few per slot: insertion sort)
__global__ void k_bond_rev_sort(const uint32_t* __restrict__ off, uint64_t n, uint32_t* __restrict__ idx) {
  const uint64_t s = (uint64_t)blockIdx.x * BT + threadIdx.x;
  if (s >= n) return;
  const uint32_t b = off[s], e = off[s + 1];
  for (uint32_t x = b + 1; x < e; x++) {
    const uint32_t v = idx[x];
    uint32_t y = x;
    while (y > b && idx[y - 1] > v) {
      idx[y] = idx[y - 1];
      y--;
    }
    idx[y] = v;
  }
}

__global__ void k_bond_needs(const uint32_t* __restrict__ bi, const uint32_t* __restrict__ bj, uint64_t nb,
                             uint32_t* __restrict__ need) {
  const uint64_t b = (uint64_t)blockIdx.x * BT + threadIdx.x;
  if (b >= nb) return;
  need[bi[b]] = 1u;
  need[bj[b]] = 1u;
}

// ---- memory
// carves aligned arrays out of one allocation
struct Carver {
  char* p;
  size_t used = 0;
  template <class T>
  T* take(uint64_t count) {
    used = (used + 255) & ~size_t(255);
    T* r = reinterpret_cast<T*>(p ? p + used : nullptr);
    used += count * sizeof(T);
    return r;
  }
};

void carve_bonds(Carver& cv, BondArrays& B, uint64_t cap) {
  B.id_i = cv.take<uint64_t>(cap);
  B.id_j = cv.take<uint64_t>(cap);
  B.i = cv.take<uint32_t>(cap);
  B.j = cv.take<uint32_t>(cap);
  B.sub = cv.take<uint32_t>(cap);
  B.mode = cv.take<int32_t>(cap);
  B.unbroken = cv.take<uint8_t>(cap);
  double** d1[9] = {&B.dn0, &B.weight, &B.c1, &B.c2, &B.en, &B.et, &B.dn, nullptr, nullptr};
  for (int k = 0; k < 7; k++) *d1[k] = cv.take<double>(cap);
  for (int d = 0; d < 3; d++) {
    B.ft[d] = cv.take<double>(cap);
    B.tds[d] = cv.take<double>(cap);
    B.f[d] = cv.take<double>(cap);
    B.ti[d] = cv.take<double>(cap);
    B.tj[d] = cv.take<double>(cap);
    B.fn[d] = cv.take<double>(cap);
  }
}

int ensure_bond_cap(dem_ctx* c, uint64_t need) {
  if (need <= c->bcap && c->bblock[0]) return DEM_OK;
  const uint64_t cap = std::max<uint64_t>(need + need / 4, 1024);
  if (cap >= (1ull << 31)) return c->fail(DEM_ERR_INVALID_ARG, "too many bonds");
  DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  Carver probe{nullptr};
  BondArrays tmp{};
  carve_bonds(probe, tmp, cap);
  const size_t one = probe.used + 256;
  void* nb[2] = {nullptr, nullptr};
  for (int k = 0; k < 2; k++) {
    if (cudaMalloc(&nb[k], one) != cudaSuccess) {
      cudaFree(nb[0]);
      return c->fail(DEM_ERR_OOM, "bond arrays: device allocation failed");
    }
  }
  BondArrays nB[2]{};
  for (int k = 0; k < 2; k++) {
    Carver cv{static_cast<char*>(nb[k])};
    carve_bonds(cv, nB[k], cap);
  }
  // keep the current bonds (same layout, the first nb rows of every array)
  if (c->nb && c->bblock[c->bcur]) {
    const BondArrays& S = c->B[c->bcur];
    BondArrays& D = nB[0];
    auto cp = [&](void* d, const void* s, size_t bytes) {
      return cudaMemcpyAsync(d, s, bytes, cudaMemcpyDeviceToDevice, c->stream);
    };
    const uint64_t m = c->nb;
    DEM_CUDA_TRY(c, cp(D.id_i, S.id_i, m * 8));
    DEM_CUDA_TRY(c, cp(D.id_j, S.id_j, m * 8));
    DEM_CUDA_TRY(c, cp(D.i, S.i, m * 4));
    DEM_CUDA_TRY(c, cp(D.j, S.j, m * 4));
    DEM_CUDA_TRY(c, cp(D.sub, S.sub, m * 4));
    DEM_CUDA_TRY(c, cp(D.mode, S.mode, m * 4));
    DEM_CUDA_TRY(c, cp(D.unbroken, S.unbroken, m));
    const double* sd[7] = {S.dn0, S.weight, S.c1, S.c2, S.en, S.et, S.dn};
    double* dd[7] = {D.dn0, D.weight, D.c1, D.c2, D.en, D.et, D.dn};
    for (int k = 0; k < 7; k++) DEM_CUDA_TRY(c, cp(dd[k], sd[k], m * 8));
    for (int d = 0; d < 3; d++) {
      DEM_CUDA_TRY(c, cp(D.ft[d], S.ft[d], m * 8));
      DEM_CUDA_TRY(c, cp(D.tds[d], S.tds[d], m * 8));
      DEM_CUDA_TRY(c, cp(D.f[d], S.f[d], m * 8));
      DEM_CUDA_TRY(c, cp(D.ti[d], S.ti[d], m * 8));
      DEM_CUDA_TRY(c, cp(D.tj[d], S.tj[d], m * 8));
      DEM_CUDA_TRY(c, cp(D.fn[d], S.fn[d], m * 8));
    }
    DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  }
  cudaFree(c->bblock[0]);
  cudaFree(c->bblock[1]);
  c->bblock[0] = nb[0];
  c->bblock[1] = nb[1];
  c->B[0] = nB[0];
  c->B[1] = nB[1];
  c->bcur = 0;
  // scans, interfaces, history table, reverse list
  cudaFree(c->b_scan);
  cudaFree(c->b_iface);
  cudaFree(c->bh_oid);
  cudaFree(c->b_rev_idx);
  c->b_scan = c->b_iface = c->b_rev_idx = nullptr;
  c->bh_oid = nullptr;
  DEM_CUDA_TRY(c, cudaMalloc(&c->b_scan, 2 * (cap + 1) * sizeof(uint32_t)));
  DEM_CUDA_TRY(c, cudaMalloc(&c->b_iface, (cap + 1) * sizeof(uint32_t)));
  DEM_CUDA_TRY(c, cudaMalloc(&c->b_rev_idx, cap * sizeof(uint32_t)));
  Carver hp{nullptr};
  hp.take<uint64_t>(cap);
  hp.take<uint64_t>(cap);
  hp.take<uint32_t>(cap);
  for (int d = 0; d < 3; d++) hp.take<double>(cap);
  void* hb = nullptr;
  DEM_CUDA_TRY(c, cudaMalloc(&hb, hp.used + 256));
  Carver hc{static_cast<char*>(hb)};
  c->bh_oid = hc.take<uint64_t>(cap);
  c->bh_pid = hc.take<uint64_t>(cap);
  c->bh_sub = hc.take<uint32_t>(cap);
  for (int d = 0; d < 3; d++) c->bh_ft[d] = hc.take<double>(cap);
  c->bcap = cap;
  return DEM_OK;
}

int ensure_bond_slots(dem_ctx* c) {
  if (c->n + 1 <= c->bpcap && c->b_own_first) return DEM_OK;
  const uint64_t cap = std::max<uint64_t>(c->pcap, c->n) + 1;
  cudaFree(c->b_own_first);
  c->b_own_first = nullptr;
  void* blk = nullptr;
  DEM_CUDA_TRY(c, cudaMalloc(&blk, 5 * cap * sizeof(uint32_t)));
  uint32_t* u = static_cast<uint32_t*>(blk);
  c->b_own_first = u;
  c->b_own_cnt = u + cap;
  c->b_rev_off = u + 2 * cap;
  c->b_rev_cur = u + 3 * cap;
  c->b_inv = u + 4 * cap;
  c->bpcap = cap;
  return DEM_OK;
}

// interfaces of the current bonds (update_interfaces.cpp:48-79): runs of one
// (id_i, id_j); the reference's scan never compares the last bond with the one
// before it, so a last run of a single bond joins the run before it
int build_interfaces(dem_ctx* c) {
  c->nif = 0;
  if (!c->nb) return DEM_OK;
  const BondArrays& B = c->B[c->bcur];
  uint32_t* flag = c->b_scan;
  uint32_t* pos = c->b_scan + c->bcap + 1;
  k_iface_flags<<<grid_for(c->nb, BT), BT, 0, c->stream>>>(B.id_i, B.id_j, c->nb, flag);
  int rc = scan_exclusive_u32(c, flag, pos, c->nb);
  if (rc) return rc;
  k_iface_write<<<grid_for(c->nb, BT), BT, 0, c->stream>>>(flag, pos, c->nb, c->b_iface);
  uint32_t nif = 0, last = 0;
  DEM_CUDA_TRY(c, cudaMemcpyAsync(&nif, pos + c->nb, 4, cudaMemcpyDeviceToHost, c->stream));
  DEM_CUDA_TRY(c, cudaMemcpyAsync(&last, flag + c->nb - 1, 4, cudaMemcpyDeviceToHost, c->stream));
  DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  if (nif >= 2 && last) nif--;
  const uint32_t end = (uint32_t)c->nb;
  DEM_CUDA_TRY(c, cudaMemcpyAsync(c->b_iface + nif, &end, 4, cudaMemcpyHostToDevice, c->stream));
  DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  c->nif = nif;
  return DEM_OK;
}

// per-slot lists of the current bonds (owned; as j, in bond order)
int build_slot_lists(dem_ctx* c) {
  if (!c->nb) return DEM_OK;
  int rc = ensure_bond_slots(c);
  if (rc) return rc;
  const BondArrays& B = c->B[c->bcur];
  const uint64_t n = c->n;
  DEM_CUDA_TRY(c, cudaMemsetAsync(c->b_own_cnt, 0, n * 4, c->stream));
  DEM_CUDA_TRY(c, cudaMemsetAsync(c->b_rev_cur, 0, (n + 1) * 4, c->stream));
  k_bond_own<<<grid_for(c->nb, BT), BT, 0, c->stream>>>(B.id_i, B.i, c->nb, c->b_own_first, c->b_own_cnt);
  k_bond_rev_count<<<grid_for(c->nb, BT), BT, 0, c->stream>>>(B.j, c->nb, c->b_rev_cur);
  if ((rc = scan_exclusive_u32(c, c->b_rev_cur, c->b_rev_off, n))) return rc;
  DEM_CUDA_TRY(c, cudaMemcpyAsync(c->b_rev_cur, c->b_rev_off, (n + 1) * 4, cudaMemcpyDeviceToDevice, c->stream));
  k_bond_rev_fill<<<grid_for(c->nb, BT), BT, 0, c->stream>>>(B.j, c->nb, c->b_rev_cur, c->b_rev_idx);
  k_bond_rev_sort<<<grid_for(n, BT), BT, 0, c->stream>>>(c->b_rev_off, n, c->b_rev_idx);
  DEM_CUDA_TRY(c, cudaGetLastError());
  return DEM_OK;
}

// ---- host restatement pieces of stick_polyhedra (run once, on the host)
struct HV {
  double x, y, z;
};
inline V3 hv(const double* x, const double* y, const double* z, uint64_t k) { return mk(x[k], y[k], z[k]); }

// shape::compute_face_areas (shape.hpp:674-697)
double host_face_area(const ShapeDev& s, int f) {
  const int b = s.fo[f], e = s.fo[f + 1];
  if (e - b < 3) return 0.0;
  const V3 v0 = mk(s.v[3 * s.fv[b]], s.v[3 * s.fv[b] + 1], s.v[3 * s.fv[b] + 2]);
  double surface = 0;
  for (int j = 1; j < e - b - 1; j++) {
    const int k = j + 1;
    const int vj = s.fv[b + j], vk = s.fv[b + k];
    const V3 v1 = mk(s.v[3 * vj], s.v[3 * vj + 1], s.v[3 * vj + 2]) - v0;
    const V3 v2 = mk(s.v[3 * vk], s.v[3 * vk + 1], s.v[3 * vk + 2]) - v0;
    surface += 0.5 * vnorm(cross(v1, v2));
  }
  return surface;
}

inline V3 stick_normalize(V3 in) {  // stick_polyhedra.cpp:40-43
  const double inv_norm = 1.0 / vnorm(in);
  return in * inv_norm;
}

struct HostBond {
  uint64_t id_i, id_j;
  uint32_t i, j, sub_i, sub_j;
  int32_t mode;
  double dn0, weight, c1, c2;
};

struct StickCtx {
  const std::vector<ShapeDev>* shapes;
  const std::vector<std::vector<double>>* areas;
  const std::vector<uint64_t>* id;
  const std::vector<uint32_t>* type;
  const std::vector<uint32_t>* group;
  const std::vector<double>* hom;
  const double* vx;
  const double* vy;
  const double* vz;
  int MV;
  const dem_inner_bond_params* ibp;
  int ng;
};

// the bonds of the pair (a, b), id_a < id_b (stick_polyhedra.cpp:235-350)
void stick_pair(const StickCtx& k, uint32_t a, uint32_t b, double dn_crit, std::vector<HostBond>& out) {
  const ShapeDev& si = (*k.shapes)[(*k.type)[a]];
  const ShapeDev& sj = (*k.shapes)[(*k.type)[b]];
  const std::vector<double>& ai = (*k.areas)[(*k.type)[a]];
  const std::vector<double>& aj = (*k.areas)[(*k.type)[b]];
  const double hi = (*k.hom)[a], hj = (*k.hom)[b];
  const double ri = si.r * hi, rj = sj.r * hj;
  const uint64_t oa = (uint64_t)a * k.MV, ob = (uint64_t)b * k.MV;
  auto va = [&](int v) { return hv(k.vx, k.vy, k.vz, oa + v); };
  auto vb = [&](int v) { return hv(k.vx, k.vy, k.vz, ob + v); };
  const dem_inner_bond_params& ibp = bond_params(k.ibp, k.ng, (*k.group)[a], (*k.group)[b]);
  std::vector<V3> nj(sj.nf);
  for (int j = 0; j < sj.nf; j++) {
    const int* f = sj.fv + sj.fo[j];
    if (sj.fo[j + 1] - sj.fo[j] < 3) continue;
    nj[j] = stick_normalize(cross(vb(f[1]) - vb(f[0]), vb(f[2]) - vb(f[0])));
  }
  std::vector<HostBond> local;
  bool found = false;
  for (int i = 0; i < si.nf && !found; i++) {
    const int* fi = si.fv + si.fo[i];
    const int size_i = si.fo[i + 1] - si.fo[i];
    if (size_i < 3) continue;
    const V3 ni = stick_normalize(cross(va(fi[1]) - va(fi[0]), va(fi[2]) - va(fi[0])));
    const double area_i = ai[i];
    for (int j = 0; j < sj.nf && !found; j++) {
      const int* fj = sj.fv + sj.fo[j];
      const int size_j = sj.fo[j + 1] - sj.fo[j];
      if (size_j < 3) continue;
      if (size_i != size_j) continue;
      const double surface_ratio = area_i / aj[j];
      if (surface_ratio > 1.01 || surface_ratio < 0.99) continue;
      if (vnorm(cross(ni, nj[j])) > 1.e-10) continue;
      const double area = ai[i] * hi * hi;  // get_face_area(i, h_i)
      HostBond proto{};
      proto.id_i = (*k.id)[a];
      proto.id_j = (*k.id)[b];
      proto.i = a;
      proto.j = b;
      proto.mode = ibp.mode;
      switch (ibp.mode) {
        case DEM_RUPTURE_ENERGY_MIXED: proto.c1 = 2 * area * ibp.crit1; break;
        case DEM_RUPTURE_ENERGY_SEPARATE:
          proto.c1 = 2 * area * ibp.crit1;
          proto.c2 = 2 * area * ibp.crit2;
          break;
        default:
          proto.c1 = 2 * area * ibp.crit1;
          proto.c2 = area * ibp.crit2;
          break;
      }
      found = true;
      for (int ivf = 0; ivf < size_i; ivf++) {
        for (int jvf = 0; jvf < size_j; jvf++) {
          const V3 pi = va(fi[ivf]), pj = vb(fj[jvf]);  // detection_vertex_vertex: dn only
          const double R = ri + rj;
          const double dn = vnorm(pi - pj) - R;
          if (dn <= dn_crit) {
            HostBond bnd = proto;
            bnd.sub_i = (uint32_t)fi[ivf];
            bnd.sub_j = (uint32_t)fj[jvf];
            bnd.dn0 = dn;
            local.push_back(bnd);
            break;
          }
        }
      }
      if (local.size() <= 2) {
        local.clear();
        found = false;
      }
    }
  }
  for (HostBond& bnd : local) bnd.weight = 1. / static_cast<double>(local.size());
  // check_stiked_face (interaction_manager.hpp:225-277)
  if (local.empty()) return;
  if (local.size() <= 2) return;
  const V3 v0 = va(local[0].sub_i), v1 = va(local[1].sub_i), v2 = va(local[2].sub_i);
  const V3 normal = cross(v1 - v0, v2 - v0);
  for (size_t q = 3; q < local.size(); q++)
    if (std::fabs(dot(va(local[q].sub_i) - v0, normal)) > 1.e-10) return;
  out.insert(out.end(), local.begin(), local.end());
}

inline bool host_bond_less(const HostBond& a, const HostBond& b) {
  if (a.id_i != b.id_i) return a.id_i < b.id_i;
  if (a.id_j != b.id_j) return a.id_j < b.id_j;
  if (a.sub_i != b.sub_i) return a.sub_i < b.sub_i;
  return a.sub_j < b.sub_j;
}

// uploads host bonds (bond order) with zero state and records, or the given state
int upload_bonds(dem_ctx* c, const std::vector<HostBond>& hb, const dem_bond_list* state,
                 const std::vector<size_t>* order) {
  const uint64_t m = hb.size();
  int rc = ensure_bond_cap(c, m);
  if (rc) return rc;
  c->bcur = 0;
  c->nb = m;
  c->nbh = 0;
  if (!m) {
    c->nif = 0;
    return DEM_OK;
  }
  // every column gets its own host buffer: the copies are queued on the ctx
  // stream and the buffers live until the stream is synchronised below
  const BondArrays& B = c->B[0];
  std::vector<std::vector<uint64_t>> h64(2, std::vector<uint64_t>(m));
  std::vector<std::vector<uint32_t>> h32(4, std::vector<uint32_t>(m));
  std::vector<int32_t> hmode(m);
  std::vector<uint8_t> hunb(m, 1);
  std::vector<std::vector<double>> hd(12, std::vector<double>(m));
  auto put = [&](void* dst, const void* src, size_t bytes) {
    return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, c->stream);
  };
  const auto at = [&](uint64_t k) { return order ? (*order)[k] : (size_t)k; };
  for (uint64_t k = 0; k < m; k++) {
    const HostBond& b = hb[k];
    h64[0][k] = b.id_i;
    h64[1][k] = b.id_j;
    h32[0][k] = b.i;
    h32[1][k] = b.j;
    h32[2][k] = (b.sub_i & 0xffffu) | ((b.sub_j & 0xffffu) << 16);
    hmode[k] = b.mode;
    hd[0][k] = b.dn0;
    hd[1][k] = b.weight;
    hd[2][k] = b.c1;
    hd[3][k] = b.c2;
    if (state) {
      const size_t r = at(k);
      hunb[k] = state->unbroken[r] ? 1 : 0;
      hd[4][k] = state->en[r];
      hd[5][k] = state->et[r];
      for (int q = 0; q < 3; q++) {
        hd[6 + q][k] = state->tds[3 * r + q];
        hd[9 + q][k] = state->friction[3 * r + q];
      }
    } else {
      for (int q = 4; q < 12; q++) hd[q][k] = 0.0;
    }
  }
  DEM_CUDA_TRY(c, put(B.id_i, h64[0].data(), m * 8));
  DEM_CUDA_TRY(c, put(B.id_j, h64[1].data(), m * 8));
  DEM_CUDA_TRY(c, put(B.i, h32[0].data(), m * 4));
  DEM_CUDA_TRY(c, put(B.j, h32[1].data(), m * 4));
  DEM_CUDA_TRY(c, put(B.sub, h32[2].data(), m * 4));
  DEM_CUDA_TRY(c, put(B.mode, hmode.data(), m * 4));
  DEM_CUDA_TRY(c, put(B.unbroken, hunb.data(), m));
  double* cols[12] = {B.dn0, B.weight, B.c1, B.c2, B.en, B.et, B.tds[0], B.tds[1], B.tds[2],
                      B.ft[0], B.ft[1], B.ft[2]};
  for (int q = 0; q < 12; q++) DEM_CUDA_TRY(c, put(cols[q], hd[q].data(), m * 8));
  for (int q = 0; q < 3; q++) {  // records of the last bond pass start at zero
    DEM_CUDA_TRY(c, cudaMemsetAsync(B.f[q], 0, m * 8, c->stream));
    DEM_CUDA_TRY(c, cudaMemsetAsync(B.ti[q], 0, m * 8, c->stream));
    DEM_CUDA_TRY(c, cudaMemsetAsync(B.tj[q], 0, m * 8, c->stream));
    DEM_CUDA_TRY(c, cudaMemsetAsync(B.fn[q], 0, m * 8, c->stream));
  }
  DEM_CUDA_TRY(c, cudaMemsetAsync(B.dn, 0, m * 8, c->stream));
  DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return build_interfaces(c);
}

int download_ids(dem_ctx* c, std::vector<uint64_t>& id) {
  id.resize(c->n);
  if (c->n)
    DEM_CUDA_TRY(c, cudaMemcpyAsync(id.data(), c->P[c->pcur].id, c->n * 8, cudaMemcpyDeviceToHost, c->stream));
  DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return DEM_OK;
}

}  // namespace

// ------------------------------------------------------------ launchers
void clear_bonds(dem_ctx* c) {
  c->nb = 0;
  c->nif = 0;
  c->nbh = 0;
}

void free_bonds(dem_ctx* c) {
  cudaFree(c->bblock[0]);
  cudaFree(c->bblock[1]);
  cudaFree(c->b_scan);
  cudaFree(c->b_iface);
  cudaFree(c->bh_oid);
  cudaFree(c->b_rev_idx);
  cudaFree(c->b_own_first);
  cudaFree(c->ibp_dev);
  c->bblock[0] = c->bblock[1] = nullptr;
  c->b_scan = c->b_iface = c->b_rev_idx = c->b_own_first = nullptr;
  c->bh_oid = nullptr;
  c->ibp_dev = nullptr;
  c->bcap = c->bpcap = 0;
  clear_bonds(c);
}

// rebuild, before the particle reorder: the broken bonds leave the list for the
// history table (stable compaction); interfaces of the bonds kept
int bonds_before_reorder(dem_ctx* c) {
  c->nbh = 0;
  if (!c->nb) return DEM_OK;
  ProfScope ps(c, K_BOND, 2);
  const BondArrays& S = c->B[c->bcur];
  uint32_t* flag = c->b_scan;
  uint32_t* pos = c->b_scan + c->bcap + 1;
  k_bond_keep_flags<<<grid_for(c->nb, BT), BT, 0, c->stream>>>(S.unbroken, c->nb, flag);
  int rc = scan_exclusive_u32(c, flag, pos, c->nb);
  if (rc) return rc;
  uint32_t keep = 0;
  DEM_CUDA_TRY(c, cudaMemcpyAsync(&keep, pos + c->nb, 4, cudaMemcpyDeviceToHost, c->stream));
  DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  if (keep != c->nb) {
    BondHist H{c->bh_oid, c->bh_pid, c->bh_sub, {c->bh_ft[0], c->bh_ft[1], c->bh_ft[2]}};
    k_bond_compact<<<grid_for(c->nb, BT), BT, 0, c->stream>>>(S, c->B[1 - c->bcur], c->nb, pos, H);
    DEM_CUDA_TRY(c, cudaGetLastError());
    c->bcur = 1 - c->bcur;
    c->nbh = c->nb - keep;
    c->nb = keep;
  }
  return build_interfaces(c);
}

// rebuild, after the particle reorder (perm: new slot -> old slot)
int bonds_after_reorder(dem_ctx* c) {
  if (!c->nb) return DEM_OK;
  int rc = ensure_bond_slots(c);
  if (rc) return rc;
  ProfScope ps(c, K_BOND, 2);
  k_inv_perm<<<grid_for(c->n, BT), BT, 0, c->stream>>>(c->perm, c->n, c->b_inv);
  const BondArrays& B = c->B[c->bcur];
  k_bond_remap<<<grid_for(c->nb, BT), BT, 0, c->stream>>>(B.i, B.j, c->nb, c->b_inv);
  DEM_CUDA_TRY(c, cudaGetLastError());
  return build_slot_lists(c);
}

int launch_bond_needs(dem_ctx* c, uint32_t* need) {
  if (!c->nb) return DEM_OK;
  const BondArrays& B = c->B[c->bcur];
  k_bond_needs<<<grid_for(c->nb, BT), BT, 0, c->stream>>>(B.i, B.j, c->nb, need);
  DEM_CUDA_TRY(c, cudaGetLastError());
  return DEM_OK;
}

int launch_bond_criterion(dem_ctx* c) {
  if (!c->nif) return DEM_OK;
  ProfScope ps(c, K_BOND, 1);
  CritArgs a;
  a.B = c->B[c->bcur];
  a.iface = c->b_iface;
  a.nif = c->nif;
  a.group = c->P[c->pcur].group;
  a.cp = c->prm.config;
  a.pt = c->ptable();
  a.flag = c->d_scalars;
  a.broken = c->d_scalars + SC_BROKEN;
  k_bond_criterion<<<grid_for(c->nif, BT), BT, 0, c->stream>>>(a);
  DEM_CUDA_TRY(c, cudaGetLastError());
  return DEM_OK;
}

int launch_bond_force(dem_ctx* c) {
  if (!c->nb) return DEM_OK;
  if (c->ib_ng < 0) return c->fail(DEM_ERR_STATE, "bonds without inner bond parameters");
  ProfScope ps(c, K_BOND, 2);
  BondArgs a;
  a.P = c->P[c->pcur];
  a.B = c->B[c->bcur];
  a.nb = c->nb;
  a.shapes = (const ShapeDev*)c->shapes_dev;
  a.MV = c->MV;
  a.vx = c->vtx[0];
  a.vy = c->vtx[1];
  a.vz = c->vtx[2];
  a.ibp = c->ibp_dev;
  a.ng = c->ib_ng;
  a.dt = c->prm.dt;
  k_bond_force<<<grid_for(c->nb, BT), BT, 0, c->stream>>>(a);
  k_bond_gather<<<grid_for(c->n, BT), BT, 0, c->stream>>>(c->P[c->pcur], c->B[c->bcur], c->n, c->b_own_first,
                                                          c->b_own_cnt, c->b_rev_off, c->b_rev_idx);
  DEM_CUDA_TRY(c, cudaGetLastError());
  return DEM_OK;
}

}  // namespace dem

using namespace dem;

extern "C" {

int dem_set_inner_bond_params(dem_ctx* c, int ngroups, const dem_inner_bond_params* pairs) {
  if (!c || ngroups < 0 || !pairs) return DEM_ERR_INVALID_ARG;
  const size_t cnt = ngroups == 0 ? 1 : (size_t)ngroups * ngroups;
  for (size_t k = 0; k < cnt; k++)
    if (pairs[k].mode < DEM_RUPTURE_ENERGY_MIXED || pairs[k].mode > DEM_RUPTURE_STRESS_ENERGY_SEPARATE)
      return c->fail(DEM_ERR_INVALID_ARG, "inner bond parameters: unknown rupture mode");
  DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  cudaFree(c->ibp_dev);
  c->ibp_dev = nullptr;
  DEM_CUDA_TRY(c, cudaMalloc(&c->ibp_dev, cnt * sizeof(dem_inner_bond_params)));
  DEM_CUDA_TRY(c, cudaMemcpyAsync(c->ibp_dev, pairs, cnt * sizeof(dem_inner_bond_params), cudaMemcpyHostToDevice,
                                  c->stream));
  DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  c->ibp_host.assign(pairs, pairs + cnt);
  c->ib_ng = ngroups;
  return DEM_OK;
}

int dem_stick_polyhedra(dem_ctx* c, const uint64_t* ids, const double* cluster, uint64_t n, double thr,
                        uint64_t* nbonds) {
  if (!c) return DEM_ERR_INVALID_ARG;
  if (!c->poly) return c->fail(DEM_ERR_STATE, "stick_polyhedra needs polyhedron shapes (dem_set_shapes)");
  if (c->ib_ng < 0) return c->fail(DEM_ERR_STATE, "stick_polyhedra needs inner bond parameters");
  if (n != c->n || (n && (!ids || !cluster)))
    return c->fail(DEM_ERR_INVALID_ARG, "stick_polyhedra: one cluster value per particle");
  if (c->ib_ng > 0) {
    std::vector<uint32_t> g(c->n);
    if (c->n)
      DEM_CUDA_TRY(c, cudaMemcpyAsync(g.data(), c->P[c->pcur].group, c->n * 4, cudaMemcpyDeviceToHost, c->stream));
    DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    for (uint32_t x : g)
      if (x >= (uint32_t)c->ib_ng) return c->fail(DEM_ERR_INVALID_ARG, "a particle group has no inner bond parameters");
  }
  int rc = launch_poly_vertices(c, 0);
  if (rc) return rc;
  const uint64_t np = c->n, nvx = np * (uint64_t)c->MV;
  const PArrays& P = c->P[c->pcur];
  std::vector<uint64_t> id(np);
  std::vector<uint32_t> type(np), group(np);
  std::vector<double> rx(np), ry(np), rz(np), hom(np), vx(nvx), vy(nvx), vz(nvx);
  auto get = [&](void* dst, const void* src, size_t bytes) {
    return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, c->stream);
  };
  if (np) {
    DEM_CUDA_TRY(c, get(id.data(), P.id, np * 8));
    DEM_CUDA_TRY(c, get(type.data(), P.type, np * 4));
    DEM_CUDA_TRY(c, get(group.data(), P.group, np * 4));
    DEM_CUDA_TRY(c, get(rx.data(), P.f[RX], np * 8));
    DEM_CUDA_TRY(c, get(ry.data(), P.f[RY], np * 8));
    DEM_CUDA_TRY(c, get(rz.data(), P.f[RZ], np * 8));
    DEM_CUDA_TRY(c, get(hom.data(), P.f[HOM], np * 8));
    DEM_CUDA_TRY(c, get(vx.data(), c->vtx[0], nvx * 8));
    DEM_CUDA_TRY(c, get(vy.data(), c->vtx[1], nvx * 8));
    DEM_CUDA_TRY(c, get(vz.data(), c->vtx[2], nvx * 8));
  }
  DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  // cluster of every slot, by id
  std::unordered_map<uint64_t, uint32_t> slot_of;
  slot_of.reserve(np * 2);
  for (uint64_t s = 0; s < np; s++) slot_of[id[s]] = (uint32_t)s;
  std::vector<double> cl(np);
  std::vector<uint8_t> seen(np, 0);
  for (uint64_t k = 0; k < n; k++) {
    const auto it = slot_of.find(ids[k]);
    if (it == slot_of.end() || seen[it->second])
      return c->fail(DEM_ERR_INVALID_ARG, "stick_polyhedra: ids must list every particle once");
    seen[it->second] = 1;
    cl[it->second] = cluster[k];
  }
  // shapes and face areas
  std::vector<ShapeDev> shapes(c->nshapes);
  std::memcpy(shapes.data(), c->shapes_host.data(), sizeof(ShapeDev) * c->nshapes);
  std::vector<std::vector<double>> areas(c->nshapes);
  for (int s = 0; s < c->nshapes; s++)
    for (int f = 0; f < shapes[s].nf; f++) areas[s].push_back(host_face_area(shapes[s], f));
  // pairs of one cluster within the neighbour distance (the chunk neighbour list)
  const double nd = 2 * c->rad_max + c->prm.rcut_inc;
  const double rcut2 = nd * nd;
  const double cs = nd > 0 ? nd * 1.001 : 1.0;
  std::unordered_map<uint64_t, std::vector<uint32_t>> cells;
  auto key = [&](int64_t x, int64_t y, int64_t z) {
    return (uint64_t)((x & 0x1fffff) | ((y & 0x1fffff) << 21) | ((z & 0x1fffff) << 42));
  };
  std::vector<int64_t> cc(3 * np);
  for (uint64_t s = 0; s < np; s++) {
    cc[3 * s] = (int64_t)std::floor((rx[s] - c->prm.bounds_lo[0]) / cs);
    cc[3 * s + 1] = (int64_t)std::floor((ry[s] - c->prm.bounds_lo[1]) / cs);
    cc[3 * s + 2] = (int64_t)std::floor((rz[s] - c->prm.bounds_lo[2]) / cs);
    cells[key(cc[3 * s], cc[3 * s + 1], cc[3 * s + 2])].push_back((uint32_t)s);
  }
  StickCtx sk{&shapes, &areas, &id, &type, &group, &hom, vx.data(), vy.data(), vz.data(), c->MV,
              c->ibp_host.data(), c->ib_ng};
  std::vector<HostBond> out;
  for (uint64_t a = 0; a < np; a++)
    for (int dz = -1; dz <= 1; dz++)
      for (int dy = -1; dy <= 1; dy++)
        for (int dx = -1; dx <= 1; dx++) {
          const auto it = cells.find(key(cc[3 * a] + dx, cc[3 * a + 1] + dy, cc[3 * a + 2] + dz));
          if (it == cells.end()) continue;
          for (uint32_t b : it->second) {
            if (b == a || cl[b] != cl[a] || id[a] >= id[b]) continue;
            const double ddx = rx[b] - rx[a], ddy = ry[b] - ry[a], ddz = rz[b] - rz[a];
            if (!(ddx * ddx + ddy * ddy + ddz * ddz < rcut2)) continue;
            stick_pair(sk, (uint32_t)a, b, thr, out);
          }
        }
  std::stable_sort(out.begin(), out.end(), host_bond_less);
  if ((rc = upload_bonds(c, out, nullptr, nullptr))) return rc;
  // the interaction storage now holds the bonds only (update_extra_storage<false>):
  // the contacts' history is dropped and the next build lists around the bonds
  c->have_list = false;
  c->hist_valid = false;
  c->gen++;
  if (nbonds) *nbonds = out.size();
  return DEM_OK;
}

int dem_bond_count(dem_ctx* c, uint64_t* out) {
  if (!c || !out) return DEM_ERR_INVALID_ARG;
  *out = c->nb;
  return DEM_OK;
}

int dem_get_bonds(dem_ctx* c, dem_bond_list* l) {
  if (!c || !l) return DEM_ERR_INVALID_ARG;
  const uint64_t m = c->nb;
  l->count = m;
  if (l->capacity < m) return c->fail(DEM_ERR_INVALID_ARG, "bond list capacity too small");
  if (!m) return DEM_OK;
  const BondArrays& B = c->B[c->bcur];
  DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  auto get = [&](void* dst, const void* src, size_t bytes) { return cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost); };
  if (l->id_i) DEM_CUDA_TRY(c, get(l->id_i, B.id_i, m * 8));
  if (l->id_j) DEM_CUDA_TRY(c, get(l->id_j, B.id_j, m * 8));
  if (l->sub_i || l->sub_j) {
    std::vector<uint32_t> sub(m);
    DEM_CUDA_TRY(c, get(sub.data(), B.sub, m * 4));
    for (uint64_t k = 0; k < m; k++) {
      if (l->sub_i) l->sub_i[k] = sub[k] & 0xffffu;
      if (l->sub_j) l->sub_j[k] = sub[k] >> 16;
    }
  }
  if (l->mode) DEM_CUDA_TRY(c, get(l->mode, B.mode, m * 4));
  if (l->unbroken) DEM_CUDA_TRY(c, get(l->unbroken, B.unbroken, m));
  double* dd[6] = {l->dn0, l->weight, l->crit1, l->crit2, l->en, l->et};
  const double* sd[6] = {B.dn0, B.weight, B.c1, B.c2, B.en, B.et};
  for (int k = 0; k < 6; k++)
    if (dd[k]) DEM_CUDA_TRY(c, get(dd[k], sd[k], m * 8));
  std::vector<double> t(m);
  for (int q = 0; q < 3; q++) {
    if (l->tds) {
      DEM_CUDA_TRY(c, get(t.data(), B.tds[q], m * 8));
      for (uint64_t k = 0; k < m; k++) l->tds[3 * k + q] = t[k];
    }
    if (l->friction) {
      DEM_CUDA_TRY(c, get(t.data(), B.ft[q], m * 8));
      for (uint64_t k = 0; k < m; k++) l->friction[3 * k + q] = t[k];
    }
  }
  return DEM_OK;
}

int dem_get_bond_state(dem_ctx* c, uint64_t capacity, uint64_t* count, double* dn, double* fn, double* ft) {
  if (!c) return DEM_ERR_INVALID_ARG;
  const uint64_t m = c->nb;
  if (count) *count = m;
  if (capacity < m) return c->fail(DEM_ERR_INVALID_ARG, "bond state capacity too small");
  if (!m) return DEM_OK;
  const BondArrays& B = c->B[c->bcur];
  DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  if (dn) DEM_CUDA_TRY(c, cudaMemcpy(dn, B.dn, m * 8, cudaMemcpyDeviceToHost));
  std::vector<double> t(m);
  for (int q = 0; q < 3; q++) {
    if (fn) {
      DEM_CUDA_TRY(c, cudaMemcpy(t.data(), B.fn[q], m * 8, cudaMemcpyDeviceToHost));
      for (uint64_t k = 0; k < m; k++) fn[3 * k + q] = t[k];
    }
    if (ft) {
      DEM_CUDA_TRY(c, cudaMemcpy(t.data(), B.ft[q], m * 8, cudaMemcpyDeviceToHost));
      for (uint64_t k = 0; k < m; k++) ft[3 * k + q] = t[k];
    }
  }
  return DEM_OK;
}

int dem_set_bonds(dem_ctx* c, const dem_bond_list* l) {
  if (!c || !l) return DEM_ERR_INVALID_ARG;
  if (!c->poly) return c->fail(DEM_ERR_STATE, "bonds need polyhedron shapes (dem_set_shapes)");
  const uint64_t m = l->count;
  if (m && (!l->id_i || !l->id_j || !l->sub_i || !l->sub_j || !l->dn0 || !l->weight || !l->mode || !l->crit1 ||
            !l->crit2 || !l->en || !l->et || !l->tds || !l->friction || !l->unbroken))
    return c->fail(DEM_ERR_INVALID_ARG, "set_bonds: every column is required");
  std::vector<uint64_t> id;
  int rc = download_ids(c, id);
  if (rc) return rc;
  std::vector<uint32_t> type(c->n);
  if (c->n)
    DEM_CUDA_TRY(c, cudaMemcpyAsync(type.data(), c->P[c->pcur].type, c->n * 4, cudaMemcpyDeviceToHost, c->stream));
  DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  std::unordered_map<uint64_t, uint32_t> slot_of;
  for (uint64_t s = 0; s < c->n; s++) slot_of[id[s]] = (uint32_t)s;
  const ShapeDev* shapes = reinterpret_cast<const ShapeDev*>(c->shapes_host.data());
  std::vector<HostBond> hb(m);
  for (uint64_t k = 0; k < m; k++) {
    HostBond& b = hb[k];
    const auto a = slot_of.find(l->id_i[k]), z = slot_of.find(l->id_j[k]);
    if (a == slot_of.end() || z == slot_of.end() || l->id_i[k] >= l->id_j[k])
      return c->fail(DEM_ERR_INVALID_ARG, "set_bonds: unknown particle id or id_i >= id_j");
    b.id_i = l->id_i[k];
    b.id_j = l->id_j[k];
    b.i = a->second;
    b.j = z->second;
    b.sub_i = l->sub_i[k];
    b.sub_j = l->sub_j[k];
    if (b.sub_i >= (uint32_t)shapes[type[b.i]].nv || b.sub_j >= (uint32_t)shapes[type[b.j]].nv)
      return c->fail(DEM_ERR_INVALID_ARG, "set_bonds: vertex index out of the shape");
    if (l->mode[k] < DEM_RUPTURE_ENERGY_MIXED || l->mode[k] > DEM_RUPTURE_STRESS_ENERGY_SEPARATE)
      return c->fail(DEM_ERR_INVALID_ARG, "set_bonds: unknown rupture mode");
    b.mode = l->mode[k];
    b.dn0 = l->dn0[k];
    b.weight = l->weight[k];
    b.c1 = l->crit1[k];
    b.c2 = l->crit2[k];
  }
  std::vector<size_t> order(m);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](size_t x, size_t y) { return host_bond_less(hb[x], hb[y]); });
  std::vector<HostBond> sorted(m);
  for (uint64_t k = 0; k < m; k++) sorted[k] = hb[order[k]];
  if ((rc = upload_bonds(c, sorted, l, &order))) return rc;
  c->have_list = false;  // the next build lists around the bonds (history kept)
  c->gen++;
  return DEM_OK;
}

int dem_inner_bond_polyhedron(dem_ctx* c) {
  if (!c) return DEM_ERR_INVALID_ARG;
  if (!c->have_list) return c->fail(DEM_ERR_STATE, "no interaction list: call dem_update_particle_neighbors first");
  return launch_bond_force(c);
}

int dem_apply_interface_fracture_criterion(dem_ctx* c, uint64_t* broken) {
  if (!c) return DEM_ERR_INVALID_ARG;
  unsigned long long before = 0, after = 0;
  DEM_CUDA_TRY(c, cudaMemcpyAsync(&before, c->d_scalars + SC_BROKEN, 8, cudaMemcpyDeviceToHost, c->stream));
  int rc = launch_bond_criterion(c);
  if (rc) return rc;
  DEM_CUDA_TRY(c, cudaMemcpyAsync(&after, c->d_scalars + SC_BROKEN, 8, cudaMemcpyDeviceToHost, c->stream));
  DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  if (broken) *broken = after - before;
  return DEM_OK;
}

int dem_broken_interface_count(dem_ctx* c, uint64_t* out) {
  if (!c || !out) return DEM_ERR_INVALID_ARG;
  unsigned long long v = 0;
  DEM_CUDA_TRY(c, cudaMemcpyAsync(&v, c->d_scalars + SC_BROKEN, 8, cudaMemcpyDeviceToHost, c->stream));
  DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  *out = v;
  return DEM_OK;
}

}  // extern "C"
