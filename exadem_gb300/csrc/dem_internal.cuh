// dem_internal.cuh -- device data layout and shared helpers of the GB300 DEM hot path.
//
// Layout in HBM (all structure-of-arrays):
//   particles: 35 FP64 fields + id (u64) + type/group (u32), double-buffered so
//              the cell reorder at a rebuild is a gather from one copy into the other;
//   interactions: sorted by owner slot, and by InteractionPair key inside one
//              owner; keys (partner slot, partner id, meta), history (6 FP64)
//              and the per-step force record (9 FP64) in separate arrays;
//   cells: counts/starts of the cell grid used by the broad phase.
// All FP64 arithmetic that decides a result keeps the operation order of the
// reference and is compiled with --fmad=false, so the results are bit-identical
// to the CPU restatement of the reference.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/dem_hotpath.h"

namespace dem {

// ---------------------------------------------------------------- fields
enum PField : int {
  RX, RY, RZ, VX, VY, VZ, FX, FY, FZ,
  WX, WY, WZ,   // vrot
  AX, AY, AZ,   // arot
  MX, MY, MZ,   // mom
  QW, QX, QY, QZ,
  IX, IY, IZ,   // inertia
  MASS, RAD, HOM,
  IMASS, IIX, IIY, IIZ,  // RN(1/mass), RN(1/inertia): exact divisions by Markstein's step
  BX, BY, BZ,   // backup positions for the displacement trigger
  NPF
};
constexpr int NUSER = HOM + 1;  // fields exchanged with the caller (rx .. homothety)

struct PArrays {
  double* f[NPF];
  uint64_t* id;
  uint32_t* type;
  uint32_t* group;
};

// interaction meta word: bits 0..7 type, bits 8..13 periodic image shift of
// the partner (2 bits per axis: 0 none, 1 = +L, 2 = -L), bit 14 owner-only
// (partner is a periodic ghost image whose force is discarded), bit 15 swap
// (polyhedra: the contact law's particle i is the partner).
__host__ __device__ inline uint32_t meta_type(uint32_t m) { return m & 0xffu; }
__host__ __device__ inline int meta_shift(uint32_t m, int d) {
  uint32_t s = (m >> (8 + 2 * d)) & 3u;
  return s == 1 ? 1 : (s == 2 ? -1 : 0);
}
__host__ __device__ inline bool meta_owner_only(uint32_t m) { return (m >> 14) & 1u; }
__host__ __device__ inline uint32_t make_meta(uint32_t type, int sx, int sy, int sz, bool owner_only) {
  auto enc = [](int s) -> uint32_t { return s == 1 ? 1u : (s == -1 ? 2u : 0u); };
  return type | (enc(sx) << 8) | (enc(sy) << 10) | (enc(sz) << 12) | ((owner_only ? 1u : 0u) << 14);
}

struct IArrays {
  uint32_t* owner;    // owner particle slot
  uint32_t* partner;  // partner particle slot, or driver index
  uint64_t* pid;      // partner id (particle id, or driver index) -- key
  uint32_t* meta;
  uint32_t* sub;      // owner sub (low 16 bits) | partner sub (high 16 bits); polyhedra
  double* ft[3];      // history: attr::friction
  double* mo[3];      // history: attr::moment
  double* damp;       // spheres: the pair's damping coefficient damp_rate 2 sqrt(kn meff), set at the build
};

struct Records {  // per-interaction force record of the last force pass
  double* f[3];
  double* ti[3];
  double* tj[3];
  // fused sphere step: 0 when the interaction's record and history are known to
  // be zero (written as zeros by the screen or the detection and untouched since),
  // so that the screen need not write them again and the gather need not read
  // them; 1 otherwise.  Every rebuild sets all entries to 1.
  uint8_t* live;
};

// Inner bonds (fragmentation), in bond order (id_i, id_j, sub_i): keys, the
// bonded vertices, parameters fixed at the stick, the bond state
// (InnerBondInteraction, inner_bond_interaction.hpp:28-62) and the record of
// the last bond pass (force, torques, dn and fn = f - friction for the
// fracture criterion).
struct BondArrays {
  uint64_t* id_i;
  uint64_t* id_j;
  uint32_t* i;        // particle slots (remapped at every reorder)
  uint32_t* j;
  uint32_t* sub;      // sub_i (low 16 bits) | sub_j (high 16 bits)
  int32_t* mode;      // rupture mode (DEM_RUPTURE_*)
  uint8_t* unbroken;
  double* dn0;
  double* weight;
  double* c1;
  double* c2;
  double* en;
  double* et;
  double* ft[3];      // attr::friction
  double* tds[3];
  double* f[3];       // record: force on i
  double* ti[3];
  double* tj[3];
  double* dn;
  double* fn[3];
};

// Multi-material contact parameters (multimat_parameters.hpp:38-300,
// contact_force_accessor.hpp:15-23): pp[g_i * ng + g_j] for a particle pair,
// pd[g_i * nd + driver] for a particle and a driver, by the particles' group
// field.  pp == nullptr: the single sets config / config_driver (singlemat).
struct ParamTable {
  const dem_contact_params* pp = nullptr;
  const dem_contact_params* pd = nullptr;
  int ng = 0, nd = 0;
  __host__ __device__ inline const dem_contact_params& pair(const dem_contact_params& single, uint32_t gi,
                                                            uint32_t gj) const {
    return pp ? pp[gi * (uint32_t)ng + gj] : single;
  }
  __host__ __device__ inline const dem_contact_params& drv(const dem_contact_params& single, uint32_t gi,
                                                           uint32_t d) const {
    return pd ? pd[gi * (uint32_t)nd + d] : single;
  }
};

// drivers in device-friendly form (stationary; vrot enters the relative velocity)
struct DriverDev {
  int kind;  // 0 surface, 1 cylinder, 2 mesh
  int mesh;  // kind 2: index into the context's mesh table
  double offset, radius;
  double normal[3], center[3], center_proj[3], axis[3], vel[3], vrot[3];
};

// Mesh driver (RShapeDriver, rshape.hpp:104-420) on the device.  World vertices
// center + quat * v in SoA; edges as vertex pairs; faces as CSR vertex lists.
// A uniform bin grid covers the mesh: bin b lists (kind << 30 | index, kind 0
// vertex, 1 edge, 2 face, sorted) every feature whose Verlet filter can pass
// for a point of b; a point outside the grid passes none.  The bin of a point
// is floor((p - lo) * inv_bs) per axis.
struct MeshDev {
  int nv, ne, nf;
  double r;  // Minkowski radius
  const double* x;
  const double* y;
  const double* z;
  const int* e;   // 2 ne
  const int* fo;  // nf + 1
  const int* fv;  // fo[nf]
  double lo[3];
  double inv_bs;
  int dims[3];
  const uint32_t* boff;   // bins + 1
  const uint32_t* bitem;  // boff[bins]
  // per feature (vertices, edges, faces): a bounding sphere (x, y, z, r) in FP32
  // of its vertex, its segment extended by the bins' skin in the line
  // parameter, or its polygon
  const float4* fsph;
};
struct GridDev {
  int dims[3];
  double lo[3];
  double hi[3];
  double csz[3];
  int periodic[3];
  double L[3];
};

// Systems of a batched context (one system when not batched).  System k owns
// particles [pfirst[k], pfirst[k+1]) (the cell sort keeps particles inside
// their system's range), cells [coff[k], coff[k+1]) of the global cell index
// space, and drivers [drange[k].x, drange[k].x + drange[k].y).  trig[k] is set
// when system k's own displacement trigger fired: a rebuild wraps the periodic
// positions and resets the displacement backups of those systems only, so
// every system keeps the wrap times and trigger steps it has when run alone.
struct SysView {
  const GridDev* g;
  const uint32_t* coff;
  const uint64_t* pfirst;  // nsys + 1 entries
  const int2* drange;
  uint32_t* trig;          // nsys entries: the system's own rebuild trigger fired
  int nsys;
  __device__ __forceinline__ bool triggered(int k) const { return nsys == 1 || trig[k] != 0u; }
  __device__ __forceinline__ int of(uint64_t s) const {
    int lo = 0, hi = nsys - 1;
    while (lo < hi) {  // last k with pfirst[k] <= s
      const int mid = (lo + hi + 1) >> 1;
      if (pfirst[mid] <= s)
        lo = mid;
      else
        hi = mid - 1;
    }
    return lo;
  }
};

// ------------------------------------------------------------- vector math
struct V3 {
  double x, y, z;
};
__host__ __device__ inline V3 mk(double x, double y, double z) { return V3{x, y, z}; }
__host__ __device__ inline V3 operator+(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__host__ __device__ inline V3 operator-(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__host__ __device__ inline V3 operator-(V3 a) { return V3{-a.x, -a.y, -a.z}; }
__host__ __device__ inline V3 operator*(V3 a, double s) { return V3{a.x * s, a.y * s, a.z * s}; }
__host__ __device__ inline V3 operator*(double s, V3 a) { return V3{s * a.x, s * a.y, s * a.z}; }
__host__ __device__ inline V3 operator*(V3 a, V3 b) { return V3{a.x * b.x, a.y * b.y, a.z * b.z}; }
__host__ __device__ inline V3 operator/(V3 a, double s) { return V3{a.x / s, a.y / s, a.z / s}; }
__host__ __device__ inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__host__ __device__ inline V3 cross(V3 a, V3 b) {
  return V3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__host__ __device__ inline double vnorm(V3 a) { return sqrt(dot(a, a)); }

// Per-interaction contact state of the last force pass (ContactState,
// classifier/contact_state.hpp:22-50, written by AnalysisDataPacker,
// classifier_for_all.hpp:55-97): overlap, contact point, normal force f - ft
// and tangential force ft.  dn == nullptr: analysis off, nothing is written.
struct ContactStateArrays {
  double* dn = nullptr;
  double* cp[3] = {nullptr, nullptr, nullptr};
  double* fn[3] = {nullptr, nullptr, nullptr};
  double* ft[3] = {nullptr, nullptr, nullptr};
  __device__ inline void write(uint64_t k, double d, V3 c, V3 n, V3 t) const {
    if (!dn) return;
    dn[k] = d;
    cp[0][k] = c.x;
    cp[1][k] = c.y;
    cp[2][k] = c.z;
    fn[0][k] = n.x;
    fn[1][k] = n.y;
    fn[2][k] = n.z;
    ft[0][k] = t.x;
    ft[1][k] = t.y;
    ft[2][k] = t.z;
  }
};


// ----------------------------------------------------------------- errors
struct Status {
  int code = DEM_OK;
  std::string msg;
};

}  // namespace dem

#define DEM_CUDA_TRY(ctx, call)                                                            \
  do {                                                                                     \
    cudaError_t _e = (call);                                                               \
    if (_e != cudaSuccess) {                                                               \
      return (ctx)->fail(_e == cudaErrorMemoryAllocation ? DEM_ERR_OOM : DEM_ERR_CUDA,     \
                         std::string(#call) + ": " + cudaGetErrorString(_e));              \
    }                                                                                      \
  } while (0)
