/*
 * dem_oracle.cpp -- CPU oracle for the exaDEM per-timestep hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker the GPU library is
 * compared against (tests/, the smoke check and the CPU baseline leg of the
 * benchmark).  Nothing in the product links or calls it.
 *
 * It restates, in plain sequential C++ (OpenMP only over independent items,
 * so results do not depend on the thread count), the arithmetic of the
 * reference CPU path: spheres and polyhedra, surfaces, cylinders and
 * stationary mesh drivers (the mesh candidates brute force over every feature),
 * the Hooke / cohesive / DMT laws, multi-material tables, the contact state
 * and the stress tensor.  Each function cites the reference lines it follows
 * (paths relative to the exaDEM source tree).  Two external libraries
 * of the reference are not vendored and are restated from their mathematics:
 *   - onika (Collab4exaNBody/onika, unpinned HEAD): Vec3d operators
 *     (component-wise), dot/cross/norm, Quaternion*Vec3d rotation,
 *     dot(Quaternion, Vec3d) time derivative and normalize().  The quaternion
 *     formulas follow exaDEM's own quat type, which is the same lineage
 *     (src/shape/include/exaDEM/type/quat.hpp:71-110,233-242).
 *   - exaNBody (Collab4exaNBody/exaNBody, unpinned HEAD): the neighbour search
 *     (all pairs with d2 > 0, d2 < (r_a+r_b+rcut_inc)^2 and d2 < nbh_dist^2,
 *     src/grid/chunk_neighbors_contact.cpp:45-57), periodic ghost images,
 *     PushVec3{First,Second}OrderFunctor (x += v*dt + a*dt^2/2, v += a*dt/2)
 *     and particle_displ_over (|r - r_backup|^2 >= max_displ^2).
 * Parity status: exaDEM as a whole cannot be built here (exaNBody, onika, MPI
 * and yaml-cpp are absent), but its hot-path arithmetic lives in headers that
 * compile on the host against small stand-ins for those libraries
 * (oracle/ref_harness.cpp, oracle/ref_shim/, built by oracle/ref_build.py).
 * The oracle_unit_* entry points at the end of this file run the functions
 * below on rows of inputs; tests/test_oracle_vs_ref.py compares them with
 * exaDEM's own functions bit for bit (contact_force_core for the three laws,
 * compute_moments, the damping and effective mass, the vertex-vertex, -edge,
 * -face and edge-edge filters and detections, OBB intersect / compute_obb /
 * enlarge, shape::get_vertex, the rotation functors of the prolog and epilog,
 * InteractionPair ordering, the Surface and Cylinder drivers), and
 * tests/test_oracle_golden.py repeats it on stored exaDEM outputs.  Still
 * restated without a compiled counterpart: the neighbour search and periodic
 * images (exaNBody), the translation pushes (exaNBody functors), the loops of
 * nbh_sphere / nbh_polyhedron that decide which features are tested (grid and
 * cell machinery), and the Vec3d / Quaternion operators themselves (onika,
 * restated identically in the stand-ins).
 *
 * Canonical summation order (the reference sums with unordered atomics,
 * contact_sphere.hpp:183-196): for each particle, f = g*m, then the
 * contributions of the interactions it owns in InteractionPair order, then
 * those where it is the partner, in InteractionPair order.
 *
 * Build: g++ -O2 -ffp-contract=off -fopenmp (no -ffast-math: the rolling
 * clip below relies on IEEE NaN semantics).
 */
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/dem_hotpath.h"

namespace {

struct V3 {
  double x, y, z;
};
inline V3 operator+(const V3& a, const V3& b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(const V3& a, const V3& b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator-(const V3& a) { return {-a.x, -a.y, -a.z}; }
inline V3 operator*(const V3& a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline V3 operator*(double s, const V3& a) { return {s * a.x, s * a.y, s * a.z}; }
inline V3 operator*(const V3& a, const V3& b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline V3 operator/(const V3& a, double s) { return {a.x / s, a.y / s, a.z / s}; }
inline V3& operator+=(V3& a, const V3& b) { a.x += b.x; a.y += b.y; a.z += b.z; return a; }
inline V3& operator-=(V3& a, const V3& b) { a.x -= b.x; a.y -= b.y; a.z -= b.z; return a; }
inline V3& operator*=(V3& a, double s) { a.x *= s; a.y *= s; a.z *= s; return a; }
inline double dot(const V3& a, const V3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(const V3& a, const V3& b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline double norm(const V3& a) { return std::sqrt(dot(a, a)); }
inline bool is_null(const V3& a) { return a.x == 0.0 && a.y == 0.0 && a.z == 0.0; }

struct Quat {
  double w, x, y, z;
};
// Quaternion * Vec3d rotation (type/quat.hpp:79-89).
inline V3 rotate(const Quat& q, const V3& v) {
  V3 qv = {q.x, q.y, q.z};
  V3 uv = cross(qv, v);
  V3 uuv = cross(qv, uv);
  uv *= (2.0 * q.w);
  uuv *= 2.0;
  return v + uv + uuv;
}
// dot(Q, omega): quaternion time derivative (type/quat.hpp:91-96).
inline Quat qdot(const Quat& q, const V3& om) {
  Quat r;
  r.x = 0.5 * (om.y * q.z - om.z * q.y + om.x * q.w);
  r.y = 0.5 * (om.z * q.x - om.x * q.z + om.y * q.w);
  r.z = 0.5 * (om.x * q.y - om.y * q.x + om.z * q.w);
  r.w = -0.5 * (om.x * q.x + om.y * q.y + om.z * q.z);
  return r;
}
// normalize (type/quat.hpp:233-242).
inline Quat qnormalize(Quat q) {
  double norm2 = q.w * q.w + (q.x * q.x + q.y * q.y + q.z * q.z);
  if (norm2 <= 1e-9) return {1.0, 0.0, 0.0, 0.0};
  double n = std::sqrt(norm2);
  double inv = 1.0 / n;
  return {q.w * inv, q.x * inv, q.y * inv, q.z * inv};
}

struct Surface {
  double offset;
  V3 normal, center, center_proj, vel, vrot;
};
struct Cylinder {
  double radius;
  V3 axis, center, vel, vrot;
};
struct Driver {
  int kind;  // 0 surface, 1 cylinder, 2 mesh
  Surface s;
  Cylinder c;
  int mesh = -1;  // kind 2: index into Oracle::meshes
};

// Mesh driver (RShapeDriver, rshape.hpp:104-420), stationary: world vertices
// center + quat * (1.0 * v) (RShapeDriver::update_vertex), edges as vertex pairs,
// faces as vertex lists, Minkowski radius r; position() = center, zero velocities.
struct MeshO {
  std::vector<V3> w;
  std::vector<int> e;
  std::vector<std::vector<int>> f;
  double r = 0;
  V3 center{};
};

// One interaction = InteractionPair + Interaction data (interaction_pair.hpp:56-71,
// interaction.hpp:44-49).  Sphere pairs: type 0, swap 0, subs 0.
struct Inter {
  uint64_t oid, pid;
  uint16_t type;
  uint8_t swap;
  uint8_t owner_only;  // partner is a periodic ghost image: its force is discarded
  uint32_t osub, psub;
  int32_t oi, pj;      // particle indices (pj = driver index for drivers)
  int8_t sh[3];        // periodic image of the partner: r_j + sh*L
  V3 friction, moment;
};
inline bool key_less(const Inter& a, const Inter& b) {  // InteractionPair::operator< (interaction_pair.hpp:222-249)
  if (a.oid != b.oid) return a.oid < b.oid;
  if (a.pid != b.pid) return a.pid < b.pid;
  if (a.type != b.type) return a.type < b.type;
  if (a.swap != b.swap) return a.swap < b.swap;
  if (a.osub != b.osub) return a.osub < b.osub;
  return a.psub < b.psub;
}
inline bool key_eq(const Inter& a, const Inter& b) {  // interaction_pair.hpp:186-198
  return a.oid == b.oid && a.pid == b.pid && a.osub == b.osub && a.psub == b.psub && a.swap == b.swap &&
         a.type == b.type;
}

struct Rec {  // per-interaction force record
  V3 f, ti, tj;
  int active;
  // contact state (AnalysisDataPacker, classifier_for_all.hpp:55-97): dn (0 when
  // the pair does not touch), contact point, fn = f - friction, ft = friction
  double sdn = 0;
  V3 scp{}, sfn{}, sft{};
};

// InnerBondInteraction (interaction/inner_bond_interaction.hpp:28-62): particle
// indices i (owner, id_i < id_j) and j, bonded vertices, dn0, weight, the
// rupture criterion (rupture_criterion.hpp:35-40) and the bond's state.
struct Bond {
  uint64_t id_i, id_j;
  int32_t i, j;
  uint32_t sub_i, sub_j;
  double dn0 = 0, weight = 1;
  int32_t mode = 0;
  double c1 = 0, c2 = 0;
  V3 friction{}, tds{};
  double en = 0, et = 0;
  uint8_t unbroken = 1;
};
inline bool bond_less(const Bond& a, const Bond& b) {  // InteractionPair order within type 13
  if (a.id_i != b.id_i) return a.id_i < b.id_i;
  if (a.id_j != b.id_j) return a.id_j < b.id_j;
  if (a.sub_i != b.sub_i) return a.sub_i < b.sub_i;
  return a.sub_j < b.sub_j;
}
struct BondRec {  // force record and contact state of the last bond pass
  V3 f{}, ti{}, tj{};
  double dn = 0;
  V3 fn{};
};

struct Oracle {
  dem_params prm;
  // multi-material contact parameters (multimat_parameters.hpp:38-300): mm_pp[g_i * ng + g_j],
  // mm_pd[g_i * nd + driver]; empty: the single sets config / config_driver
  int mm_ng = 0, mm_nd = 0;
  std::vector<dem_contact_params> mm_pp, mm_pd;
  const dem_contact_params& pair_params(size_t i, size_t j) const {
    return mm_pp.empty() ? prm.config : mm_pp[(size_t)group[i] * mm_ng + group[j]];
  }
  const dem_contact_params& driver_params(size_t i, size_t d) const {
    return mm_pp.empty() ? prm.config_driver : mm_pd[(size_t)group[i] * mm_nd + d];
  }
  size_t n = 0;
  std::vector<double> rx, ry, rz, vx, vy, vz, fx, fy, fz, wx, wy, wz, ax, ay, az, mx, my, mz, qw, qx, qy, qz, ix,
      iy, iz, mass, rad, hom, bx, by, bz;
  std::vector<uint64_t> id;
  std::vector<uint32_t> type, group;
  std::vector<Driver> drivers;
  std::vector<Inter> inter;          // global InteractionPair order
  std::vector<size_t> own_off;       // per particle: owned range (particles sorted by id index)
  std::vector<int32_t> own_first;    // per particle index: first owned interaction or -1
  std::vector<int32_t> own_cnt;
  std::vector<size_t> rev_off;       // per particle: partner-side interactions
  std::vector<int32_t> rev_idx;
  std::vector<Rec> rec;
  // polyhedron mode
  bool poly = false;
  std::vector<struct PShape> shapes;
  std::vector<MeshO> meshes;
  std::vector<std::vector<V3>> vtx;   // world vertices per particle
  std::vector<std::vector<V3>> bvtx;  // vertices at the last rebuild (backup_dem)
  uint64_t rebuilds = 0;
  uint64_t n_active = 0;
  // inner bonds (fragmentation), in bond order
  std::vector<Bond> bonds;
  std::vector<BondRec> brec;
  std::vector<size_t> iface;        // interface offsets into bonds (nif + 1)
  std::vector<int32_t> bown_first;  // per particle: first owned bond or -1
  std::vector<int32_t> bown_cnt;
  std::vector<size_t> brev_off;     // per particle: bonds where it is j
  std::vector<int32_t> brev_idx;
  int ib_ng = -1;                   // -1: no inner bond parameters; 0: one set
  std::vector<dem_inner_bond_params> ibp;
  const dem_inner_bond_params& bond_params(size_t i, size_t j) const {
    return ib_ng == 0 ? ibp[0] : ibp[(size_t)group[i] * ib_ng + group[j]];
  }
  std::vector<Inter> broken_hist;   // bonds broken since the last rebuild, as vertex-vertex history
  uint64_t broken_total = 0;
  std::string err;
};

inline double L(const Oracle& o, int d) { return o.prm.bounds_hi[d] - o.prm.bounds_lo[d]; }

V3 pos(const Oracle& o, size_t i) { return {o.rx[i], o.ry[i], o.rz[i]}; }

// Partner position with its periodic ghost image (exaNBody ghost copy r + shift).
V3 partner_pos(const Oracle& o, const Inter& it) {
  V3 r = pos(o, it.pj);
  if (it.sh[0]) r.x = r.x + (double)it.sh[0] * L(o, 0);
  if (it.sh[1]) r.y = r.y + (double)it.sh[1] * L(o, 1);
  if (it.sh[2]) r.z = r.z + (double)it.sh[2] * L(o, 2);
  return r;
}

double nbh_dist(const Oracle& o) {
  double rmax = 0.0;
  for (size_t i = 0; i < o.n; i++) rmax = std::max(rmax, 2 * o.rad[i]);  // dem_rcut_max.cpp:49-66
  return rmax + o.prm.rcut_inc;
}

// ---------------------------------------------------------------- drivers
// Surface::filter / detector (src/driver/include/exaDEM/surface.hpp:320-350)
bool surface_filter(const Surface& s, double rcut, const V3& p) {
  V3 proj = dot(p, s.normal) * s.normal;
  double d = norm(proj - s.center_proj);
  return d <= rcut;
}
bool surface_detect(const Surface& s, double rcut, const V3& p, double& dn, V3& n, V3& cp) {
  V3 proj = dot(p, s.normal) * s.normal;
  V3 s2p = -(s.center_proj - proj);
  double d = norm(s2p);
  dn = d - rcut;
  if (dn > 0) return false;
  n = s2p / d;
  cp = p - n * (rcut + 0.5 * dn);
  return true;
}
// Cylinder::filter / detector (src/driver/include/exaDEM/cylinder.hpp:225-277)
bool cylinder_filter(const Cylinder& c, double rcut, const V3& vi) {
  V3 proj = vi * c.axis;
  V3 dir = proj - c.center;
  double d = norm(dir);
  double dn = c.radius - (d + rcut);
  return dn <= 0;
}
bool cylinder_detect(const Cylinder& c, double rcut, const V3& pi, double& dn, V3& n, V3& cp) {
  V3 proj = pi * c.axis;
  V3 dir = c.center - proj;
  double d = norm(dir);
  dn = c.radius - (rcut + d);
  if (dn > 0) return false;
  n = dir / d;
  cp = pi - n * (rcut + 0.5 * dn);
  return true;
}

// register_surface: the YAML decoder's default centre (surface.hpp:68-84), then
// Surface::initialize (surface.hpp:145-175) for a stationary surface.
Surface surface_from(const dem_surface* s) {
  Surface w{};
  w.offset = s->offset;
  w.normal = {s->normal[0], s->normal[1], s->normal[2]};
  w.vel = {s->vel[0], s->vel[1], s->vel[2]};
  w.vrot = {s->vrot[0], s->vrot[1], s->vrot[2]};
  w.center_proj = w.offset * w.normal;
  if (is_null(w.vrot) && is_null({s->center[0], s->center[1], s->center[2]}))
    w.center = w.offset * w.normal;
  else
    w.center = {s->center[0], s->center[1], s->center[2]};
  // a centre off the plane on the normal's side is replaced (surface.hpp:166-173)
  if (dot(w.center - w.center_proj, w.normal) >= 1e-14) w.center = dot(w.center_proj - w.center, w.normal) * w.normal + w.center_proj;
  return w;
}
// register_cylinder: Cylinder::initialize (cylinder.hpp:94-105) stores axis * center.
Cylinder cylinder_from(const dem_cylinder* c) {
  Cylinder w{};
  w.radius = c->radius;
  w.axis = {c->axis[0], c->axis[1], c->axis[2]};
  w.center = w.axis * V3{c->center[0], c->center[1], c->center[2]};
  w.vel = {c->vel[0], c->vel[1], c->vel[2]};
  w.vrot = {c->vrot[0], c->vrot[1], c->vrot[2]};
  return w;
}

// ---------------------------------------------------------- neighbour build
// Periodic wrap done by move_particles before each rebuild.
void wrap(Oracle& o) {
  for (int d = 0; d < 3; d++) {
    if (!o.prm.periodic[d]) continue;
    double lo = o.prm.bounds_lo[d], hi = o.prm.bounds_hi[d], Ld = hi - lo;
    std::vector<double>& r = d == 0 ? o.rx : (d == 1 ? o.ry : o.rz);
    for (size_t i = 0; i < o.n; i++) {
      double x = r[i];
      if (x < lo) {
        x = x + Ld;
        if (x >= hi) x = lo;
      } else if (x >= hi) {
        x = x - Ld;
        if (x < lo) x = lo;
      }
      r[i] = x;
    }
  }
}

// chunk_neighbors_contact + nbh_sphere (symetric) + classify, with history
// carried over by InteractionPair equality (interaction_manager.hpp:89-112,
// placeholder_interaction.hpp:398-408).
// sphere-mesh candidates and detection (defined with the polyhedron geometry)
void mesh_candidates(const Oracle& o, size_t k, size_t i, const V3& ri, double rad, double skin, std::vector<Inter>& lst);
bool mesh_detect(const Oracle& o, const Inter& it, const V3& ri, double rad, double& dn, V3& n, V3& cp);

int update_neighbors(Oracle& o) {
  wrap(o);
  const double skin = o.prm.rcut_inc;
  const double nd = nbh_dist(o);
  const double rcut2 = nd * nd;
  double cs = std::max(o.prm.cell_size, nd);
  int dims[3];
  double lo[3];
  for (int d = 0; d < 3; d++) {
    lo[d] = o.prm.bounds_lo[d];
    dims[d] = std::max(1, (int)std::floor(L(o, d) / cs));
    if (o.prm.periodic[d] && dims[d] < 3) {
      o.err = "periodic dimension needs at least 3 cells";
      return DEM_ERR_INVALID_ARG;
    }
  }
  double csz[3];
  for (int d = 0; d < 3; d++) csz[d] = o.prm.periodic[d] ? L(o, d) / dims[d] : cs;
  if (!o.prm.periodic[0] || !o.prm.periodic[1] || !o.prm.periodic[2]) {
    // non periodic dims: grid from bounds, particles outside clamped into border cells
    for (int d = 0; d < 3; d++)
      if (!o.prm.periodic[d]) dims[d] = std::max(1, (int)std::ceil(L(o, d) / cs));
  }
  auto cell_of = [&](size_t i, int c[3]) {
    double r[3] = {o.rx[i], o.ry[i], o.rz[i]};
    for (int d = 0; d < 3; d++) {
      long k = (long)std::floor((r[d] - lo[d]) / csz[d]);
      if (k < 0) k = 0;
      if (k >= dims[d]) k = dims[d] - 1;
      c[d] = (int)k;
    }
  };
  size_t ncell = (size_t)dims[0] * dims[1] * dims[2];
  std::vector<size_t> cstart(ncell + 1, 0), cidx(o.n);
  std::vector<int> pc(3 * o.n);
  for (size_t i = 0; i < o.n; i++) {
    cell_of(i, &pc[3 * i]);
    size_t c = (size_t)pc[3 * i] + dims[0] * ((size_t)pc[3 * i + 1] + (size_t)dims[1] * pc[3 * i + 2]);
    cstart[c + 1]++;
  }
  for (size_t c = 0; c < ncell; c++) cstart[c + 1] += cstart[c];
  {
    std::vector<size_t> cur(cstart.begin(), cstart.end() - 1);
    for (size_t i = 0; i < o.n; i++) {
      size_t c = (size_t)pc[3 * i] + dims[0] * ((size_t)pc[3 * i + 1] + (size_t)dims[1] * pc[3 * i + 2]);
      cidx[cur[c]++] = i;
    }
  }

  // per owner candidate lists
  std::vector<std::vector<Inter>> per(o.n);
#pragma omp parallel for schedule(dynamic, 256)
  for (long ii = 0; ii < (long)o.n; ii++) {
    size_t i = (size_t)ii;
    std::vector<Inter>& lst = per[i];
    const V3 ri = pos(o, i);
    // drivers first (nbh_sphere.cu:140-233)
    for (size_t k = 0; k < o.drivers.size(); k++) {
      const Driver& dv = o.drivers[k];
      if (dv.kind == 2) {
        mesh_candidates(o, k, i, ri, o.rad[i], skin, lst);
        continue;
      }
      const double rv = o.rad[i] + skin;
      bool keep = dv.kind == 0 ? surface_filter(dv.s, rv, ri) : cylinder_filter(dv.c, rv, ri);
      if (!keep) continue;
      Inter it{};
      it.oid = o.id[i];
      it.pid = k;
      it.type = dv.kind == 0 ? DEM_ITYPE_VERTEX_SURFACE : DEM_ITYPE_VERTEX_CYLINDER;
      it.oi = (int32_t)i;
      it.pj = (int32_t)k;
      lst.push_back(it);
    }
    // particle pairs over the 27-cell stencil (nbh_sphere.cu:238-263)
    const int* ci = &pc[3 * i];
    for (int dz = -1; dz <= 1; dz++)
      for (int dy = -1; dy <= 1; dy++)
        for (int dx = -1; dx <= 1; dx++) {
          int c[3] = {ci[0] + dx, ci[1] + dy, ci[2] + dz};
          int sh[3] = {0, 0, 0};
          bool skip = false;
          for (int d = 0; d < 3; d++) {
            if (c[d] < 0) {
              if (!o.prm.periodic[d]) { skip = true; break; }
              c[d] += dims[d];
              sh[d] = -1;
            } else if (c[d] >= dims[d]) {
              if (!o.prm.periodic[d]) { skip = true; break; }
              c[d] -= dims[d];
              sh[d] = 1;
            }
          }
          if (skip) continue;
          size_t cc = (size_t)c[0] + dims[0] * ((size_t)c[1] + (size_t)dims[1] * c[2]);
          for (size_t q = cstart[cc]; q < cstart[cc + 1]; q++) {
            size_t j = cidx[q];
            V3 rj = pos(o, j);
            if (sh[0]) rj.x = rj.x + (double)sh[0] * L(o, 0);
            if (sh[1]) rj.y = rj.y + (double)sh[1] * L(o, 1);
            if (sh[2]) rj.z = rj.z + (double)sh[2] * L(o, 2);
            const double ddx = rj.x - ri.x, ddy = rj.y - ri.y, ddz = rj.z - ri.z;
            const double d2 = ddx * ddx + ddy * ddy + ddz * ddz;
            const double rmax = o.rad[i] + o.rad[j] + skin;  // ContactNeighborFilterFunc
            if (!(d2 > 0.0 && d2 < rmax * rmax && d2 < rcut2)) continue;
            const bool ghost = sh[0] || sh[1] || sh[2];
            if (!ghost && o.id[i] >= o.id[j]) continue;
            Inter it{};
            it.oid = o.id[i];
            it.pid = o.id[j];
            it.type = DEM_ITYPE_VERTEX_VERTEX;
            it.oi = (int32_t)i;
            it.pj = (int32_t)j;
            it.owner_only = ghost ? 1 : 0;
            it.sh[0] = (int8_t)sh[0];
            it.sh[1] = (int8_t)sh[1];
            it.sh[2] = (int8_t)sh[2];
            lst.push_back(it);
          }
        }
    std::sort(lst.begin(), lst.end(), key_less);
  }
  // global InteractionPair order = owners by id
  std::vector<size_t> by_id(o.n);
  for (size_t i = 0; i < o.n; i++) by_id[i] = i;
  std::sort(by_id.begin(), by_id.end(), [&](size_t a, size_t b) { return o.id[a] < o.id[b]; });
  std::vector<Inter> fresh;
  size_t tot = 0;
  for (size_t i = 0; i < o.n; i++) tot += per[i].size();
  fresh.reserve(tot);
  for (size_t k = 0; k < o.n; k++) {
    auto& l = per[by_id[k]];
    fresh.insert(fresh.end(), l.begin(), l.end());
  }
  // history carry-over: old list is sorted by key, binary search like update()
#pragma omp parallel for schedule(static)
  for (long k = 0; k < (long)fresh.size(); k++) {
    Inter& it = fresh[k];
    auto lb = std::lower_bound(o.inter.begin(), o.inter.end(), it, key_less);
    if (lb != o.inter.end() && key_eq(*lb, it)) {
      it.friction = lb->friction;
      it.moment = lb->moment;
    }
  }
  o.inter.swap(fresh);
  // owned ranges and partner lists (canonical gather order)
  o.own_first.assign(o.n, -1);
  o.own_cnt.assign(o.n, 0);
  for (size_t k = 0; k < o.inter.size(); k++) {
    const Inter& it = o.inter[k];
    if (o.own_first[it.oi] < 0) o.own_first[it.oi] = (int32_t)k;
    o.own_cnt[it.oi]++;
  }
  o.rev_off.assign(o.n + 1, 0);
  for (const Inter& it : o.inter)
    if (it.type == DEM_ITYPE_VERTEX_VERTEX && !it.owner_only) o.rev_off[it.pj + 1]++;
  for (size_t i = 0; i < o.n; i++) o.rev_off[i + 1] += o.rev_off[i];
  o.rev_idx.assign(o.rev_off[o.n], 0);
  {
    std::vector<size_t> cur(o.rev_off.begin(), o.rev_off.end() - 1);
    for (size_t k = 0; k < o.inter.size(); k++) {  // k ascending = key order
      const Inter& it = o.inter[k];
      if (it.type == DEM_ITYPE_VERTEX_VERTEX && !it.owner_only) o.rev_idx[cur[it.pj]++] = (int32_t)k;
    }
  }
  o.rec.assign(o.inter.size(), Rec{});
  // backup_r
  o.bx = o.rx;
  o.by = o.ry;
  o.bz = o.rz;
  o.rebuilds++;
  return DEM_OK;
}

// ---- detection cores: {contact, dn, n, cp}; no contact returns dn = 0 like contact()
struct Det {
  bool c = false;
  double dn = 0;
  V3 n = {0, 0, 0}, cp = {0, 0, 0};
};
Det detect_vv(const V3& pi, double ri, const V3& pj, double rj) {  // :57-81
  const double R = ri + rj;
  const V3 dist = pi - pj;
  const double dist_norm = norm(dist);
  const double inv_dist_norm = 1.0 / dist_norm;
  const double dn = dist_norm - R;
  const V3 n = dist * inv_dist_norm;
  const V3 cp = pi - n * (ri + 0.5 * dn);
  return {dn < 0, dn, n, cp};
}
// --------------------------------------------------------------- contact law
// contact_force_core<Hooke, None|Cohesive|DMT> (src/forcefield/include/exaDEM/forcefield/contact_force.hpp:146-235)
// with common_kernels.hpp:27-145; dmt: apply_dmt_force (contact_force.hpp:115-127) with the pair's reff.
void contact_force_core(bool cohesive, double dn, const V3& n, double dt, const dem_contact_params& hkp, double meff,
                        V3& ft, const V3& cp, const V3& pos_i, const V3& vel_i, V3& f_i, V3& mom_i,
                        const V3& vrot_i, const V3& pos_j, const V3& vel_j, const V3& vrot_j, bool dmt = false,
                        double reff = 0.0) {
  if (cohesive) {
    if (dn >= 0) {
      const double fn_value = (hkp.fc / hkp.dncut) * dn - hkp.fc;
      f_i += fn_value * n;
      ft = {0, 0, 0};
      return;
    }
  }
  const double damp = hkp.damp_rate * 2.0 * std::sqrt(hkp.kn * meff);  // compute_damp
  // compute_relative_velocity
  const V3 contribution_i = vel_i - cross(cp - pos_i, vrot_i);
  const V3 contribution_j = vel_j - cross(cp - pos_j, vrot_j);
  const V3 vel = contribution_j - contribution_i;
  const double vn = dot(vel, n);
  V3 fn;
  {
    const double fne = -hkp.kn * dn;
    const double fnv = damp * vn;
    double nf = (fnv + fne > 0) ? fnv + fne : 0;  // normal_force
    if (cohesive) {
      const double fn_norm = nf - hkp.fc;
      nf = fn_norm < (-hkp.fc) ? -hkp.fc : fn_norm;
    }
    fn = nf * n;
  }
  {
    const V3 vt = vel - vn * n;
    const V3 ftd = dt * vt;
    ft += hkp.kt * ftd;  // compute_tangential_force
  }
  double threshold_ft;
  if (!cohesive) {
    const double fne = hkp.kn * dn;
    threshold_ft = std::fabs(hkp.mu * fne);
  } else {
    threshold_ft = std::fabs(hkp.mu * (dot(fn, n) + hkp.fc));
  }
  {
    double ft_square = dot(ft, ft);  // fit_tangential_force
    if (ft_square > 0.0 && ft_square > threshold_ft * threshold_ft) ft *= (threshold_ft / std::sqrt(ft_square));
  }
  f_i = fn + ft;
  if (dmt && hkp.gamma > 0.0 && dn < 0.0) {  // attraction -2 pi reff gamma n in contact
    const double F_dmt = 2.0 * 3.14159265358979323846 * reff * hkp.gamma;
    f_i -= F_dmt * n;
  }
  mom_i += hkp.kr * (vrot_j - vrot_i) * dt;
  V3 branch = cp - pos_i;
  double r = (dot(branch, vrot_i)) / (dot(vrot_i, vrot_i));
  branch -= r * vrot_i;
  constexpr double mur = 0;
  double threshold_mom = std::fabs(mur * norm(branch) * norm(fn));
  double mom_square = dot(mom_i, mom_i);
  if (mom_square > 0.0 && mom_square > threshold_mom * threshold_mom)
    mom_i = mom_i * (threshold_mom / std::sqrt(mom_square));
}

// sphere::ContactLawFunc (src/sphere/include/exaDEM/sphere/contact_sphere.hpp:122-203) and
// ContactLawDriverFunc (contact_sphere.hpp:231-297), producing a force record.
void contact_one(Oracle& o, size_t k) {
  Inter& it = o.inter[k];
  Rec& rc = o.rec[k];
  rc = Rec{};
  const bool cohesive = o.prm.law == DEM_LAW_HOOKE_COHESIVE;
  const bool dmt = o.prm.law == DEM_LAW_HOOKE_DMT;
  const double dt = o.prm.dt;
  const size_t i = it.oi;
  const V3 ri = pos(o, i);
  const V3 vrot_i = {o.wx[i], o.wy[i], o.wz[i]};
  if (it.type == DEM_ITYPE_VERTEX_VERTEX) {
    const size_t j = it.pj;
    const V3 rj = partner_pos(o, it);
    const double rad_i = o.rad[i], rad_j = o.rad[j];
    const V3 vrot_j = {o.wx[j], o.wy[j], o.wz[j]};
    // detection_vertex_vertex_core (src/shape/include/exaDEM/shape_detection_core.hpp:57-81)
    const Det det = detect_vv(ri, rad_i, rj, rad_j);
    const double dn = det.dn;
    const V3 n = det.n, cp = det.cp;
    bool contact = det.c;
    const dem_contact_params& cpar = o.pair_params(i, j);  // contact_sphere.hpp:147-152
    if (cohesive) contact = (contact || dn <= cpar.dncut);
    if (contact) {
      const V3 vi = {o.vx[i], o.vy[i], o.vz[i]};
      const V3 vj = {o.vx[j], o.vy[j], o.vz[j]};
      const double m_i = o.mass[i], m_j = o.mass[j];
      V3 f = {0, 0, 0};
      const double meff = (m_i * m_j) / (m_i + m_j);  // compute_effective_mass
      const double reff = dmt ? (rad_i * rad_j) / (rad_i + rad_j) : 0.0;  // compute_effective_radius
      contact_force_core(cohesive, dn, n, dt, cpar, meff, it.friction, cp, ri, vi, f, it.moment, vrot_i, rj, vj,
                         vrot_j, dmt, reff);
      rc.f = f;
      rc.ti = cross(cp - ri, f) + it.moment;       // compute_moments
      rc.tj = cross(cp - rj, -f) + (-it.moment);
      rc.active = dn < 0;
      rc.sdn = dn;
      rc.scp = cp;
      rc.sfn = f - it.friction;
      rc.sft = it.friction;
    } else {
      it.friction = {0, 0, 0};
      it.moment = {0, 0, 0};
      rc.scp = cp;  // item.reset(), dn = 0, the detector's contact point
    }
    return;
  }
  // drivers
  const Driver& dv = o.drivers[it.pj];
  const double rad = o.rad[i];
  double dn = 0;
  V3 n{}, cp{};
  bool contact;
  V3 dpos, dvel, dvrot;
  if (dv.kind == 2) {  // ContactLawRShapeDriverFunc (contact_sphere.hpp:300-396)
    contact = mesh_detect(o, it, ri, rad, dn, n, cp);
    dpos = o.meshes[dv.mesh].center;
    dvel = {0, 0, 0};
    dvrot = {0, 0, 0};
  } else if (dv.kind == 0) {
    contact = surface_detect(dv.s, rad, ri, dn, n, cp);
    dpos = dv.s.center;
    dvel = dv.s.vel;
    dvrot = dv.s.vrot;
  } else {
    contact = cylinder_detect(dv.c, rad, ri, dn, n, cp);
    dpos = dv.c.center;
    dvel = dv.c.vel;
    dvrot = dv.c.vrot;
  }
  const dem_contact_params& cpar = o.driver_params(i, it.pj);  // contact_sphere.hpp:254-257
  if (cohesive) contact = (contact || dn <= cpar.dncut);
  if (contact) {
    const V3 v = {o.vx[i], o.vy[i], o.vz[i]};
    const double meff = o.mass[i];
    V3 f = {0, 0, 0};
    contact_force_core(cohesive, dn, n, dt, cpar, meff, it.friction, cp, ri, v, f, it.moment, vrot_i, dpos, dvel,
                       dvrot, dmt, rad);  // reff = the particle's radius (contact_sphere.hpp:270)
    rc.f = f;
    rc.ti = cross(cp - ri, f) + it.moment;
    rc.active = dn < 0;
    rc.sdn = dn;
    rc.scp = cp;
    rc.sfn = f - it.friction;
    rc.sft = it.friction;
  } else {
    it.friction = {0, 0, 0};
    it.moment = {0, 0, 0};
    if (dv.kind == 2) rc.scp = cp;  // dn = 0, the detector's contact point
  }
}

void contact_one_poly(Oracle& o, size_t k);

void contact_all(Oracle& o) {
  if (o.poly) {
#pragma omp parallel for schedule(static)
    for (long k = 0; k < (long)o.inter.size(); k++) contact_one_poly(o, (size_t)k);
  } else {
#pragma omp parallel for schedule(static)
    for (long k = 0; k < (long)o.inter.size(); k++) contact_one(o, (size_t)k);
  }
  uint64_t na = 0;
  for (const Rec& r : o.rec) na += r.active ? 1 : 0;
  o.n_active = na;
  // deterministic gather: owned contributions (key order) then partner contributions (key order)
#pragma omp parallel for schedule(static)
  for (long ii = 0; ii < (long)o.n; ii++) {
    size_t i = (size_t)ii;
    V3 f = {o.fx[i], o.fy[i], o.fz[i]};
    V3 m = {o.mx[i], o.my[i], o.mz[i]};
    if (o.own_first[i] >= 0) {
      for (int32_t k = o.own_first[i]; k < o.own_first[i] + o.own_cnt[i]; k++) {
        f += o.rec[k].f;
        m += o.rec[k].ti;
      }
    }
    for (size_t q = o.rev_off[i]; q < o.rev_off[i + 1]; q++) {
      const Rec& r = o.rec[o.rev_idx[q]];
      f += -r.f;
      m += r.tj;
    }
    o.fx[i] = f.x;
    o.fy[i] = f.y;
    o.fz[i] = f.z;
    o.mx[i] = m.x;
    o.my[i] = m.y;
    o.mz[i] = m.z;
  }
}

// ------------------------------------------------------------ particle ops
void reset_force_moment(Oracle& o) {  // reset_force_moment.cu:69-70
  std::fill(o.fx.begin(), o.fx.end(), 0.0);
  std::fill(o.fy.begin(), o.fy.end(), 0.0);
  std::fill(o.fz.begin(), o.fz.end(), 0.0);
  std::fill(o.mx.begin(), o.mx.end(), 0.0);
  std::fill(o.my.begin(), o.my.end(), 0.0);
  std::fill(o.mz.begin(), o.mz.end(), 0.0);
}
void gravity_force(Oracle& o) {  // gravity_force.hpp:38-46
  const double* g = o.prm.gravity;
#pragma omp parallel for schedule(static)
  for (long i = 0; i < (long)o.n; i++) {
    o.fx[i] += g[0] * o.mass[i];
    o.fy[i] += g[1] * o.mass[i];
    o.fz[i] += g[2] * o.mass[i];
  }
}
void force_to_accel(Oracle& o) {  // force_to_accel.hpp:26-33
#pragma omp parallel for schedule(static)
  for (long i = 0; i < (long)o.n; i++) {
    o.fx[i] /= o.mass[i];
    o.fy[i] /= o.mass[i];
    o.fz[i] /= o.mass[i];
  }
}
// PushToQuaternionFunctor (push_to_quaternion.hpp:26-38): Q += dot(Q, w) dt, normalize, w += dt/2 a.
inline void push_quaternion(Quat& Q, V3& w, const V3& a, double delta_t, double half_delta_t) {
  const Quat d = qdot(Q, w);
  Q = {Q.w + d.w * delta_t, Q.x + d.x * delta_t, Q.y + d.y * delta_t, Q.z + d.z * delta_t};
  Q = qnormalize(Q);
  w.x += half_delta_t * a.x;
  w.y += half_delta_t * a.y;
  w.z += half_delta_t * a.z;
}
// PushToAngularAccelerationFunctor (angular_acceleration.hpp:27-43): Euler's equations in the body frame.
inline V3 angular_acceleration(const Quat& Q, const V3& mom, const V3& vrot, const V3& I) {
  const Quat Qinv = {Q.w, -Q.x, -Q.y, -Q.z};
  const V3 omega = rotate(Qinv, vrot);
  const V3 M = rotate(Qinv, mom);
  const V3 domega = {(M.x - (I.z - I.y) * omega.y * omega.z) / I.x, (M.y - (I.x - I.z) * omega.z * omega.x) / I.y,
                     (M.z - (I.y - I.x) * omega.x * omega.y) / I.z};
  return rotate(Q, domega);
}
// combined_compute_prolog (combined_compute_prolog.cu:94-116): PushVec3SecondOrder,
// PushVec3FirstOrder, PushToQuaternion (push_to_quaternion.hpp:26-38).
void prolog(Oracle& o) {
  const double delta_t = o.prm.dt;
  const double half_delta_t = delta_t * 0.5;
  const double delta_t2_2 = delta_t * delta_t * 0.5;
#pragma omp parallel for schedule(static)
  for (long i = 0; i < (long)o.n; i++) {
    o.rx[i] += o.vx[i] * delta_t + o.fx[i] * delta_t2_2;
    o.ry[i] += o.vy[i] * delta_t + o.fy[i] * delta_t2_2;
    o.rz[i] += o.vz[i] * delta_t + o.fz[i] * delta_t2_2;
    o.vx[i] += o.fx[i] * half_delta_t;
    o.vy[i] += o.fy[i] * half_delta_t;
    o.vz[i] += o.fz[i] * half_delta_t;
    Quat Q = {o.qw[i], o.qx[i], o.qy[i], o.qz[i]};
    V3 w = {o.wx[i], o.wy[i], o.wz[i]};
    push_quaternion(Q, w, {o.ax[i], o.ay[i], o.az[i]}, delta_t, half_delta_t);
    o.qw[i] = Q.w;
    o.qx[i] = Q.x;
    o.qy[i] = Q.y;
    o.qz[i] = Q.z;
    o.wx[i] = w.x;
    o.wy[i] = w.y;
    o.wz[i] = w.z;
  }
}
// combined_compute_epilog (combined_compute_epilog.cu:94-113) with
// PushToAngularAcceleration (angular_acceleration.hpp:27-43) and PushToAngularVelocity.
void epilog(Oracle& o) {
  const double half_delta_t = o.prm.dt * 0.5;
#pragma omp parallel for schedule(static)
  for (long i = 0; i < (long)o.n; i++) {
    const Quat Q = {o.qw[i], o.qx[i], o.qy[i], o.qz[i]};
    const V3 arot = angular_acceleration(Q, {o.mx[i], o.my[i], o.mz[i]}, {o.wx[i], o.wy[i], o.wz[i]},
                                         {o.ix[i], o.iy[i], o.iz[i]});
    o.ax[i] = arot.x;
    o.ay[i] = arot.y;
    o.az[i] = arot.z;
    o.wx[i] += arot.x * half_delta_t;
    o.wy[i] += arot.y * half_delta_t;
    o.wz[i] += arot.z * half_delta_t;
    o.vx[i] += o.fx[i] * half_delta_t;
    o.vy[i] += o.fy[i] * half_delta_t;
    o.vz[i] += o.fz[i] * half_delta_t;
  }
}
int displ_over(const Oracle& o) {
  const double max_displ = o.prm.rcut_inc * 0.5;
  const double thr2 = max_displ * max_displ;
  int over = 0;
#pragma omp parallel for schedule(static) reduction(| : over)
  for (long i = 0; i < (long)o.n; i++) {
    const double dx = o.rx[i] - o.bx[i], dy = o.ry[i] - o.by[i], dz = o.rz[i] - o.bz[i];
    if (dx * dx + dy * dy + dz * dz >= thr2) over |= 1;
  }
  return over;
}

void bond_force(Oracle& o);
// compute_force with fragmentation (config_fragmentation.msp compute_force):
// gravity, the contact laws, then inner_bond_polyhedron
void compute_force(Oracle& o) {
  gravity_force(o);
  contact_all(o);
  if (o.poly && !o.bonds.empty()) bond_force(o);
}

// Profile: solid fraction of spheres in horizontal slabs (analytic cap volumes).
double sphere_slab_volume(double zc, double r, double a, double b) {
  double lo = std::max(a, zc - r), hi = std::min(b, zc + r);
  if (hi <= lo) return 0.0;
  // integral of pi*(r^2 - (z-zc)^2) dz from lo to hi
  auto F = [&](double z) {
    double u = z - zc;
    return r * r * u - u * u * u / 3.0;
  };
  return M_PI * (F(hi) - F(lo));
}

// ======================================================= polyhedra
// Oriented bounding box (src/shape/include/exaDEM/type/OBB.hpp).
struct OBBr {
  V3 c, e1, e2, e3, ext;
};
struct PShape {
  std::vector<V3> v;
  std::vector<int> e;                  // 2*ne
  std::vector<std::vector<int>> f;     // faces
  double r = 0;                        // Minkowski radius
  std::vector<double> fa;              // face areas (shape::compute_face_areas, shape.hpp:674-697)
  OBBr obb;
  int nv() const { return (int)v.size(); }
  int ne() const { return (int)e.size() / 2; }
  int nf() const { return (int)f.size(); }
  double max_rcut() const {            // shape.hpp:479-489
    double rc = 0;
    for (const V3& x : v) rc = std::max(rc, norm(x) + r);
    return rc;
  }
};

inline void obb_enlarge(OBBr& o, double m) {  // OBB::enlarge
  o.ext.x += m;
  o.ext.y += m;
  o.ext.z += m;
}
// compute_obb (src/shape/include/exaDEM/basic_types.hpp:37-48)
OBBr compute_obb(const OBBr& in, const V3& p, const Quat& q, double h) {
  OBBr o = in;
  o.e1 = rotate(q, o.e1);
  o.e2 = rotate(q, o.e2);
  o.e3 = rotate(q, o.e3);
  o.c = rotate(q, o.c);
  if (h != 1.0) {
    o.ext *= h;
    o.c *= h;
  }
  o.c += p;
  return o;
}
// OBB::intersect, separating axis test with tol = FLT_EPSILON (type/OBB.hpp:90-220)
bool obb_intersect(const OBBr& A, const OBBr& B) {
  const double tol = 1.1920928955078125e-07;
  double ra, rb;
  double Rxx, Rxy, Rxz, Ryx, Ryy, Ryz, Rzx, Rzy, Rzz;
  double Axx, Axy, Axz, Ayx, Ayy, Ayz, Azx, Azy, Azz;
  Rxx = dot(A.e1, B.e1);
  Rxy = dot(A.e1, B.e2);
  Rxz = dot(A.e1, B.e3);
  Axx = std::fabs(Rxx) + tol;
  Axy = std::fabs(Rxy) + tol;
  Axz = std::fabs(Rxz) + tol;
  const V3 tt = A.c - B.c;
  const V3 t = {dot(tt, A.e1), dot(tt, A.e2), dot(tt, A.e3)};
  ra = A.ext.x;
  rb = B.ext.x * Axx + B.ext.y * Axy + B.ext.z * Axz;
  if (std::fabs(t.x) > ra + rb) return false;
  Ryx = dot(A.e2, B.e1);
  Ayx = std::fabs(Ryx) + tol;
  Ryy = dot(A.e2, B.e2);
  Ayy = std::fabs(Ryy) + tol;
  Ryz = dot(A.e2, B.e3);
  Ayz = std::fabs(Ryz) + tol;
  ra = A.ext.y;
  rb = B.ext.x * Ayx + B.ext.y * Ayy + B.ext.z * Ayz;
  if (std::fabs(t.y) > ra + rb) return false;
  Rzx = dot(A.e3, B.e1);
  Azx = std::fabs(Rzx) + tol;
  Rzy = dot(A.e3, B.e2);
  Azy = std::fabs(Rzy) + tol;
  Rzz = dot(A.e3, B.e3);
  Azz = std::fabs(Rzz) + tol;
  ra = A.ext.z;
  rb = B.ext.x * Azx + B.ext.y * Azy + B.ext.z * Azz;
  if (std::fabs(t.z) > ra + rb) return false;
  ra = A.ext.x * Axx + A.ext.y * Ayx + A.ext.z * Azx;
  rb = B.ext.x;
  if (std::fabs(t.x * Rxx + t.y * Ryx + t.z * Rzx) > ra + rb) return false;
  ra = A.ext.x * Axy + A.ext.y * Ayy + A.ext.z * Azy;
  rb = B.ext.y;
  if (std::fabs(t.x * Rxy + t.y * Ryy + t.z * Rzy) > ra + rb) return false;
  ra = A.ext.x * Axz + A.ext.y * Ayz + A.ext.z * Azz;
  rb = B.ext.z;
  if (std::fabs(t.x * Rxz + t.y * Ryz + t.z * Rzz) > ra + rb) return false;
  ra = A.ext.y * Azx + A.ext.z * Ayx;
  rb = B.ext.y * Axz + B.ext.z * Axy;
  if (std::fabs(t.z * Ryx - t.y * Rzx) > ra + rb) return false;
  ra = A.ext.y * Azy + A.ext.z * Ayy;
  rb = B.ext.x * Axz + B.ext.z * Axx;
  if (std::fabs(t.z * Ryy - t.y * Rzy) > ra + rb) return false;
  ra = A.ext.y * Azz + A.ext.z * Ayz;
  rb = B.ext.x * Axy + B.ext.y * Axx;
  if (std::fabs(t.z * Ryz - t.y * Rzz) > ra + rb) return false;
  ra = A.ext.x * Azx + A.ext.z * Axx;
  rb = B.ext.y * Ayz + B.ext.z * Ayy;
  if (std::fabs(t.x * Rzx - t.z * Rxx) > ra + rb) return false;
  ra = A.ext.x * Azy + A.ext.z * Axy;
  rb = B.ext.x * Ayz + B.ext.z * Ayx;
  if (std::fabs(t.x * Rzy - t.z * Rxy) > ra + rb) return false;
  ra = A.ext.x * Azz + A.ext.z * Axz;
  rb = B.ext.x * Ayy + B.ext.y * Ayx;
  if (std::fabs(t.x * Rzz - t.z * Rxz) > ra + rb) return false;
  ra = A.ext.x * Ayx + A.ext.y * Axx;
  rb = B.ext.y * Azz + B.ext.z * Azy;
  if (std::fabs(t.y * Rxx - t.x * Ryx) > ra + rb) return false;
  ra = A.ext.x * Ayy + A.ext.y * Axy;
  rb = B.ext.x * Azz + B.ext.z * Azx;
  if (std::fabs(t.y * Rxy - t.x * Ryy) > ra + rb) return false;
  ra = A.ext.x * Ayz + A.ext.y * Axz;
  rb = B.ext.x * Azy + B.ext.y * Azx;
  if (std::fabs(t.y * Rxz - t.x * Ryz) > ra + rb) return false;
  return true;
}

inline void vnormalize(V3& v) { v = v / norm(v); }  // _normalize (include/exaDEM/normalize.hpp:43-46)

// ---- filters (src/shape/include/exaDEM/shape_detection_core.hpp)
bool filter_vv(double rV, const V3& vi, double ri, const V3& vj, double rj) {  // :43-53
  const double R = ri + rj + rV;
  const V3 dist = vi - vj;
  const double d2 = dot(dist, dist);
  return d2 <= R * R;
}
bool filter_ve(double rV, const V3& vi, double ri, const V3& vf, const V3& vs, double rj) {  // :83-101
  const V3 distfs = vs - vf;
  const V3 distfi = vi - vf;
  const double r = (dot(distfs, distfi)) / (dot(distfs, distfs));
  if (r < -rV || r > 1.0 + rV) return false;
  const V3 dist = distfi - distfs * r;
  const double Rmax = ri + rj + rV;
  return (dot(dist, dist) < (Rmax * Rmax));
}
// point-in-face test shared by the face filter and detection (:246-309, :398-466)
bool vf_core(double lim, const V3& vi, const std::vector<V3>& vaj, const std::vector<int>& face, double& dist_out,
             V3& n_out) {
  const int nf = (int)face.size();
  const V3& va = vaj[face[0]];
  const V3& vb = vaj[face[1]];
  const V3& vc = vaj[face[nf - 1]];
  const V3 v = vi - va;
  V3 v1 = vb - va;
  V3 v2 = vc - va;
  vnormalize(v1);
  V3 n = cross(v1, v2);
  vnormalize(n);
  double dist = dot(n, v);
  if (dist < 0) {
    n = n * (-1);
    dist = -dist;
  }
  dist_out = dist;
  n_out = n;
  if (dist > lim) return false;
  const V3 P = vi - n * dist;
  int ODD = 0;
  v2 = cross(n, v1);
  const double ori1 = dot(P, v1);
  const double ori2 = dot(P, v2);
  for (int iva = 0; iva < nf; ++iva) {
    int ivb = iva + 1;
    if (ivb == nf) ivb = 0;
    const V3& _va = vaj[face[iva]];
    const V3& _vb = vaj[face[ivb]];
    const double pa1 = dot(_va, v1);
    const double pb1 = dot(_vb, v1);
    const double pa2 = dot(_va, v2);
    const double pb2 = dot(_vb, v2);
    if ((pa2 < ori2 && pb2 >= ori2) || (pb2 < ori2 && pa2 >= ori2)) {
      if (pa1 + (ori2 - pa2) / (pb2 - pa2) * (pb1 - pa1) < ori1) ODD = 1 - ODD;
    }
  }
  return ODD == 1;
}
bool filter_vf(double rV, const V3& vi, double ri, const std::vector<V3>& vaj, const std::vector<int>& face,
               double rj) {
  double dist;
  V3 n;
  return vf_core(ri + rj + rV, vi, vaj, face, dist, n);
}
bool filter_ee(double rV, const V3& vfi, const V3& vsi, double ri, const V3& vfj, const V3& vsj, double rj) {  // :468-504
  const double R = ri + rj + rV;
  const V3 Ei = vsi - vfi;
  const V3 Ej = vsj - vfj;
  const V3 v = vfi - vfj;
  const double c = dot(Ei, Ei);
  const double d = dot(Ej, Ej);
  const double e = dot(Ei, Ej);
  double f = (c * d) - (e * e);
  if (std::fabs(f) > 1.0e-12) {
    f = 1.0 / f;
    const double a = dot(Ei, v);
    const double b = dot(Ej, v);
    const double s_ = (e * b - a * d) * f;
    const double t_ = (c * b - e * a) * f;
    if (s_ <= 0.0 || s_ >= 1.0 || t_ <= 0.0 || t_ >= 1.0) return false;
    const V3 pi = vfi + Ei * s_;
    const V3 pj = vfj + Ej * t_;
    const V3 n = pi - pj;
    return (dot(n, n) <= (R * R));
  }
  return false;
}

Det detect_ve(const V3& vi, double ri, const V3& vf, const V3& vs, double rj) {  // :122-148
  const V3 distfs = vs - vf;
  const V3 distfi = vi - vf;
  const double r = (dot(distfs, distfi)) / (dot(distfs, distfs));
  if (r <= 0 || r >= 1.0) return Det{};
  V3 n = distfi - distfs * r;
  const double dn = norm(n) - (ri + rj);
  if (dn > 0) return Det{};
  vnormalize(n);
  const V3 cp = vi - n * (ri + 0.5 * dn);
  return {true, dn, n, cp};
}
Det detect_vf(const V3& vi, double ri, const std::vector<V3>& vaj, const std::vector<int>& face, double rj) {
  double dist;
  V3 n;
  const bool inside = vf_core(ri + rj, vi, vaj, face, dist, n);
  if (dist > (ri + rj)) return Det{};
  const double dn = dist - (ri + rj);
  const V3 cp = vi - n * (ri + 0.5 * dn);
  return {inside, dn, n, cp};
}
Det detect_ee(const V3& vfi, const V3& vsi, double ri, const V3& vfj, const V3& vsj, double rj) {  // :521-566
  const double R = ri + rj;
  const V3 Ei = vsi - vfi;
  const V3 Ej = vsj - vfj;
  const V3 v = vfi - vfj;
  const double c = dot(Ei, Ei);
  const double d = dot(Ej, Ej);
  const double e = dot(Ei, Ej);
  double f = (c * d) - (e * e);
  if (std::fabs(f) > 1.0e-12) {
    f = 1.0 / f;
    const double a = dot(Ei, v);
    const double b = dot(Ej, v);
    const double s_ = (e * b - a * d) * f;
    const double t_ = (c * b - e * a) * f;
    if (s_ <= 0.0 || s_ >= 1.0 || t_ <= 0.0 || t_ >= 1.0) return Det{};
    const V3 pi = vfi + Ei * s_;
    const V3 pj = vfj + Ej * t_;
    V3 n = pi - pj;
    const double dn = norm(n) - R;
    if (dn > 0) return Det{};
    vnormalize(n);
    const V3 cp = pi - n * (ri + 0.5 * dn);
    return {dn <= 0, dn, n, cp};
  }
  return Det{};
}

// world vertices: shape::get_vertex = p + q * (h * v0) (shape.hpp:245-262)
// detection_sphere_driver (sphere/nbh_sphere.hpp:25-86): every vertex, edge and
// face of the mesh whose Verlet filter passes for the sphere (rVerlet = the
// skin), in (type, feature) order; the owner sub is 0, the partner sub the feature
void mesh_candidates(const Oracle& o, size_t k, size_t i, const V3& ri, double rad, double skin,
                     std::vector<Inter>& lst) {
  const MeshO& m = o.meshes[o.drivers[k].mesh];
  auto add = [&](int type, int j) {
    Inter it{};
    it.oid = o.id[i];
    it.pid = k;
    it.type = (uint16_t)type;
    it.psub = (uint32_t)j;
    it.oi = (int32_t)i;
    it.pj = (int32_t)k;
    lst.push_back(it);
  };
  for (int j = 0; j < (int)m.w.size(); j++)
    if (filter_vv(skin, ri, rad, m.w[j], m.r)) add(DEM_ITYPE_VERTEX_MESH_VERTEX, j);
  for (int j = 0; j < (int)m.e.size() / 2; j++)
    if (filter_ve(skin, ri, rad, m.w[m.e[2 * j]], m.w[m.e[2 * j + 1]], m.r)) add(DEM_ITYPE_VERTEX_MESH_EDGE, j);
  for (int j = 0; j < (int)m.f.size(); j++)
    if (filter_vf(skin, ri, rad, m.w, m.f[j], m.r)) add(DEM_ITYPE_VERTEX_MESH_FACE, j);
}

// detect<7|8|9> for spheres (shape_detection_api.hpp:357-386,
// shape_detection_core.hpp:57-220): the sphere as a vertex of radius rad
bool mesh_detect(const Oracle& o, const Inter& it, const V3& ri, double rad, double& dn, V3& n, V3& cp) {
  const MeshO& m = o.meshes[o.drivers[it.pj].mesh];
  const int j = (int)it.psub;
  Det d;
  if (it.type == DEM_ITYPE_VERTEX_MESH_VERTEX)
    d = detect_vv(ri, rad, m.w[j], m.r);
  else if (it.type == DEM_ITYPE_VERTEX_MESH_EDGE)
    d = detect_ve(ri, rad, m.w[m.e[2 * j]], m.w[m.e[2 * j + 1]], m.r);
  else
    d = detect_vf(ri, rad, m.w, m.f[j], m.r);
  dn = d.dn;
  n = d.n;
  cp = d.cp;
  return d.c;
}

// add_driver_interaction for an RShapeDriver (nbh_polyhedron_driver.hpp:61-192):
// every particle-vertex / mesh-feature (7, 8, 9), particle-edge / mesh-edge (10)
// and mesh-vertex / particle-edge or face (11, 12) pair whose Verlet filter
// passes; 11 and 12 only for the mesh vertices whose box (vertex +- Minkowski
// radius) meets the particle's OBB (rotated and translated, homothety not
// applied) enlarged by rVerlet.  The type 9 gate of the reference (face OBB
// against the vertex box) holds whenever the face filter passes.
// Largest distance of a face's vertices from the plane through its first,
// second and last vertex, the plane filter_vertex_face projects on (0 for a
// planar face; the face's extent when that corner is degenerate).
double face_flatness(const std::vector<V3>& w, const std::vector<int>& f) {
  const int nvf = (int)f.size();
  if (nvf <= 3) return 0.0;
  const V3 o = w[f[0]];
  V3 nn = cross(w[f[1]] - o, w[f[nvf - 1]] - o);
  const double len = norm(nn);
  double dmax = 0.0;
  if (len > 0.0) {
    nn = nn / len;
    for (int q = 2; q + 1 < nvf; q++) dmax = std::max(dmax, std::fabs(dot(w[f[q]] - o, nn)));
  } else {
    for (int q = 1; q < nvf; q++) dmax = std::max(dmax, norm(w[f[q]] - o));
  }
  return dmax * (1.0 + 1e-12);
}

// Test switch: 1 = the polyhedron-mesh candidates test every mesh feature (no reach prefilter).
int g_mesh_brute_force = 0;

void poly_mesh_candidates(const Oracle& o, size_t k, size_t a, double rV, std::vector<Inter>& lst) {
  const MeshO& m = o.meshes[o.drivers[k].mesh];
  const PShape& sa = o.shapes[o.type[a]];
  const double ra = sa.r * o.hom[a];
  const std::vector<V3>& va = o.vtx[a];
  auto add = [&](int type, int osub, int psub) {
    Inter it{};
    it.oid = o.id[a];
    it.pid = k;
    it.type = (uint16_t)type;
    it.oi = (int32_t)a;
    it.pj = (int32_t)k;
    it.osub = (uint32_t)osub;
    it.psub = (uint32_t)psub;
    lst.push_back(it);
  };
  const int mnv = (int)m.w.size(), mne = (int)m.e.size() / 2, mnf = (int)m.f.size();
  // features out of the particle's reach pass none of the six filters: its
  // vertices lie within h max|v0| of its centre, its edges extended by rVerlet
  // in their parameter within h max|v0| (1 + 2 rVerlet), every filter range is
  // ra + mr + rVerlet, and a feature lies within its bounding sphere (an edge's
  // extended by rVerlet in its parameter, a face's grown by its flatness, as the
  // face filter projects on a plane); skipping them saves time only
  const V3 c = pos(o, a);
  double vmax = 0.0;
  for (const V3& v : sa.v) vmax = std::max(vmax, norm(v));
  const double reach = o.hom[a] * vmax * (1.0 + 2.0 * rV) + ra + m.r + rV;
  const double slack = 1e-9 * (1.0 + std::fabs(c.x) + std::fabs(c.y) + std::fabs(c.z) + reach);
  std::vector<char> nv_(mnv), ne_(mne), nf_(mnf);
  for (int j = 0; j < mnv; j++) nv_[j] = norm(m.w[j] - c) <= reach + slack;
  for (int j = 0; j < mne; j++) {
    const V3 p0 = m.w[m.e[2 * j]], d = m.w[m.e[2 * j + 1]] - p0;
    ne_[j] = norm(p0 + 0.5 * d - c) <= reach + (0.5 + rV) * norm(d) + slack;
  }
  for (int j = 0; j < mnf; j++) {
    V3 g = {0, 0, 0};
    for (int q : m.f[j]) g = g + m.w[q] * (1.0 / (double)m.f[j].size());
    double rf = 0.0;
    for (int q : m.f[j]) rf = std::max(rf, norm(m.w[q] - g));
    nf_[j] = norm(g - c) <= reach + rf + face_flatness(m.w, m.f[j]) + slack;
  }
  if (g_mesh_brute_force) {
    std::fill(nv_.begin(), nv_.end(), 1);
    std::fill(ne_.begin(), ne_.end(), 1);
    std::fill(nf_.begin(), nf_.end(), 1);
  }
  for (int i = 0; i < sa.nv(); i++) {
    for (int j = 0; j < mnv; j++)
      if (nv_[j] && filter_vv(rV, va[i], ra, m.w[j], m.r)) add(DEM_ITYPE_VERTEX_MESH_VERTEX, i, j);
    for (int j = 0; j < mne; j++)
      if (ne_[j] && filter_ve(rV, va[i], ra, m.w[m.e[2 * j]], m.w[m.e[2 * j + 1]], m.r))
        add(DEM_ITYPE_VERTEX_MESH_EDGE, i, j);
    for (int j = 0; j < mnf; j++)
      if (nf_[j] && filter_vf(rV, va[i], ra, m.w, m.f[j], m.r)) add(DEM_ITYPE_VERTEX_MESH_FACE, i, j);
  }
  for (int e = 0; e < sa.ne(); e++)
    for (int j = 0; j < mne; j++)
      if (ne_[j] && filter_ee(rV, va[sa.e[2 * e]], va[sa.e[2 * e + 1]], ra, m.w[m.e[2 * j]], m.w[m.e[2 * j + 1]], m.r))
        add(DEM_ITYPE_EDGE_MESH_EDGE, e, j);
  OBBr gate = compute_obb(sa.obb, pos(o, a), {o.qw[a], o.qx[a], o.qy[a], o.qz[a]}, 1.0);
  obb_enlarge(gate, rV);
  for (int j = 0; j < mnv; j++) {
    if (!nv_[j]) continue;
    OBBr ov{};
    ov.c = m.w[j];
    ov.e1 = {1, 0, 0};
    ov.e2 = {0, 1, 0};
    ov.e3 = {0, 0, 1};
    obb_enlarge(ov, m.r);
    if (!obb_intersect(ov, gate)) continue;  // obb_v_rshape_j.intersect(obb_i)
    for (int e = 0; e < sa.ne(); e++)
      if (filter_ve(rV, m.w[j], m.r, va[sa.e[2 * e]], va[sa.e[2 * e + 1]], ra)) add(DEM_ITYPE_MESH_VERTEX_EDGE, e, j);
    for (int f = 0; f < sa.nf(); f++)
      if (filter_vf(rV, m.w[j], m.r, va, sa.f[f], ra)) add(DEM_ITYPE_MESH_VERTEX_FACE, f, j);
  }
}

void compute_vertices(Oracle& o) {
  o.vtx.resize(o.n);
#pragma omp parallel for schedule(static)
  for (long ii = 0; ii < (long)o.n; ii++) {
    const size_t i = (size_t)ii;
    const PShape& sh = o.shapes[o.type[i]];
    const V3 p = pos(o, i);
    const Quat q = {o.qw[i], o.qx[i], o.qy[i], o.qz[i]};
    const double h = o.hom[i];
    o.vtx[i].resize(sh.nv());
    for (int k = 0; k < sh.nv(); k++) o.vtx[i][k] = p + rotate(q, h * sh.v[k]);
  }
}

bool bonded_to(const Oracle& o, size_t a, uint64_t id);
void drop_broken_bonds(Oracle& o);

// nbh_polyhedron (src/polyhedron/nbh_polyhedron.cpp:75-384) + add_driver_interaction
// (nbh_polyhedron_driver.hpp:216-238), history by key, canonical order.  With
// bonds: the broken ones become history first; no interaction is listed for a
// bonded pair (nor for a driver whose index is the id of a bonded partner).
int update_neighbors_poly(Oracle& o) {
  for (int d = 0; d < 3; d++)
    if (o.prm.periodic[d]) {
      o.err = "periodic boundaries are not supported for polyhedra";
      return DEM_ERR_UNSUPPORTED;
    }
  if (!o.bonds.empty() || !o.bown_first.empty()) drop_broken_bonds(o);
  compute_vertices(o);
  const double rV = o.prm.rcut_inc;
  const double nd = nbh_dist(o);
  const double rcut2 = nd * nd;
  const double cs = std::max(o.prm.cell_size, nd);
  int dims[3];
  for (int d = 0; d < 3; d++) dims[d] = std::max(1, (int)std::ceil(L(o, d) / cs));
  auto cell_of = [&](size_t i, int c[3]) {
    double r[3] = {o.rx[i], o.ry[i], o.rz[i]};
    for (int d = 0; d < 3; d++) {
      long k = (long)std::floor((r[d] - o.prm.bounds_lo[d]) / cs);
      c[d] = (int)std::min<long>(std::max<long>(k, 0), dims[d] - 1);
    }
  };
  const size_t ncell = (size_t)dims[0] * dims[1] * dims[2];
  std::vector<std::vector<size_t>> cells(ncell);
  std::vector<int> pc(3 * o.n);
  for (size_t i = 0; i < o.n; i++) {
    cell_of(i, &pc[3 * i]);
    cells[(size_t)pc[3 * i] + dims[0] * ((size_t)pc[3 * i + 1] + (size_t)dims[1] * pc[3 * i + 2])].push_back(i);
  }
  std::vector<std::vector<Inter>> per(o.n);
#pragma omp parallel for schedule(dynamic, 64)
  for (long aa = 0; aa < (long)o.n; aa++) {
    const size_t a = (size_t)aa;
    std::vector<Inter>& lst = per[a];
    const PShape& sa = o.shapes[o.type[a]];
    const double ha = o.hom[a];
    const double ra = sa.r * ha;  // minkowski(h)
    // drivers: each vertex against each driver
    for (size_t k = 0; k < o.drivers.size(); k++) {
      const Driver& dv = o.drivers[k];
      if (bonded_to(o, a, (uint64_t)k)) continue;
      if (dv.kind == 2) {
        poly_mesh_candidates(o, k, a, rV, lst);
        continue;
      }
      for (int v = 0; v < sa.nv(); v++) {
        const double rc = rV + ra;
        const bool keep = dv.kind == 0 ? surface_filter(dv.s, rc, o.vtx[a][v]) : cylinder_filter(dv.c, rc, o.vtx[a][v]);
        if (!keep) continue;
        Inter it{};
        it.oid = o.id[a];
        it.pid = k;
        it.type = dv.kind == 0 ? DEM_ITYPE_VERTEX_SURFACE : DEM_ITYPE_VERTEX_CYLINDER;
        it.oi = (int32_t)a;
        it.pj = (int32_t)k;
        it.osub = (uint32_t)v;
        it.psub = 0xffffffffu;  // DRIVER_VERTEX_SUB_IDX = -1
        lst.push_back(it);
      }
    }
    const V3 ra_pos = pos(o, a);
    const int* ca = &pc[3 * a];
    for (int dz = -1; dz <= 1; dz++)
      for (int dy = -1; dy <= 1; dy++)
        for (int dx = -1; dx <= 1; dx++) {
          const int c[3] = {ca[0] + dx, ca[1] + dy, ca[2] + dz};
          if (c[0] < 0 || c[1] < 0 || c[2] < 0 || c[0] >= dims[0] || c[1] >= dims[1] || c[2] >= dims[2]) continue;
          for (size_t b : cells[(size_t)c[0] + dims[0] * ((size_t)c[1] + (size_t)dims[1] * c[2])]) {
            const V3 rb_pos = pos(o, b);
            const double ddx = rb_pos.x - ra_pos.x, ddy = rb_pos.y - ra_pos.y, ddz = rb_pos.z - ra_pos.z;
            const double d2 = ddx * ddx + ddy * ddy + ddz * ddz;
            const double rmax = o.rad[a] + o.rad[b] + rV;
            if (!(d2 > 0.0 && d2 < rmax * rmax && d2 < rcut2)) continue;
            if (o.id[a] >= o.id[b]) continue;
            if (bonded_to(o, a, o.id[b])) continue;
            const PShape& sb = o.shapes[o.type[b]];
            const double hb = o.hom[b];
            const double rb = sb.r * hb;
            OBBr obb_i = compute_obb(sa.obb, ra_pos, {o.qw[a], o.qx[a], o.qy[a], o.qz[a]}, ha);
            OBBr obb_j = compute_obb(sb.obb, rb_pos, {o.qw[b], o.qx[b], o.qy[b], o.qz[b]}, hb);
            obb_enlarge(obb_i, 0.5 * rV);
            obb_enlarge(obb_j, 0.5 * rV);
            if (!obb_intersect(obb_i, obb_j)) continue;
            obb_enlarge(obb_i, 0.5 * rV);
            obb_enlarge(obb_j, 0.5 * rV);
            const std::vector<V3>& va = o.vtx[a];
            const std::vector<V3>& vb = o.vtx[b];
            auto add = [&](int type, int swap, int sub_i, int sub_j) {
              Inter it{};
              it.oid = o.id[a];
              it.pid = o.id[b];
              it.type = (uint16_t)type;
              it.swap = (uint8_t)swap;
              it.oi = (int32_t)a;
              it.pj = (int32_t)b;
              // owner() = swap ? pj_ : pi_ ; pi_.sub = sub_i
              it.osub = (uint32_t)(swap ? sub_j : sub_i);
              it.psub = (uint32_t)(swap ? sub_i : sub_j);
              lst.push_back(it);
            };
            for (int i = 0; i < sa.nv(); i++) {
              OBBr obbvi{};
              obbvi.e1 = {1, 0, 0};
              obbvi.e2 = {0, 1, 0};
              obbvi.e3 = {0, 0, 1};
              obbvi.c = va[i];
              obb_enlarge(obbvi, ra);
              if (obb_intersect(obb_j, obbvi)) {
                for (int j = 0; j < sb.nv(); j++)
                  if (filter_vv(rV, va[i], ra, vb[j], rb)) add(DEM_ITYPE_VERTEX_VERTEX, 0, i, j);
                for (int j = 0; j < sb.ne(); j++)
                  if (filter_ve(rV, va[i], ra, vb[sb.e[2 * j]], vb[sb.e[2 * j + 1]], rb)) add(DEM_ITYPE_VERTEX_EDGE, 0, i, j);
                for (int j = 0; j < sb.nf(); j++)
                  if (filter_vf(rV, va[i], ra, vb, sb.f[j], rb)) add(DEM_ITYPE_VERTEX_FACE, 0, i, j);
              }
            }
            for (int i = 0; i < sa.ne(); i++)
              for (int j = 0; j < sb.ne(); j++)
                if (filter_ee(rV, va[sa.e[2 * i]], va[sa.e[2 * i + 1]], ra, vb[sb.e[2 * j]], vb[sb.e[2 * j + 1]], rb))
                  add(DEM_ITYPE_EDGE_EDGE, 0, i, j);
            for (int j = 0; j < sb.nv(); j++) {
              OBBr obbvj{};
              obbvj.e1 = {1, 0, 0};
              obbvj.e2 = {0, 1, 0};
              obbvj.e3 = {0, 0, 1};
              obbvj.c = vb[j];
              obb_enlarge(obbvj, rb);
              if (obb_intersect(obb_i, obbvj)) {
                for (int i = 0; i < sa.ne(); i++)
                  if (filter_ve(rV, vb[j], rb, va[sa.e[2 * i]], va[sa.e[2 * i + 1]], ra)) add(DEM_ITYPE_VERTEX_EDGE, 1, j, i);
                for (int i = 0; i < sa.nf(); i++)
                  if (filter_vf(rV, vb[j], rb, va, sa.f[i], ra)) add(DEM_ITYPE_VERTEX_FACE, 1, j, i);
              }
            }
          }
        }
    std::sort(lst.begin(), lst.end(), key_less);
  }
  std::vector<size_t> by_id(o.n);
  for (size_t i = 0; i < o.n; i++) by_id[i] = i;
  std::sort(by_id.begin(), by_id.end(), [&](size_t x, size_t y) { return o.id[x] < o.id[y]; });
  std::vector<Inter> fresh;
  for (size_t k = 0; k < o.n; k++) {
    auto& l = per[by_id[k]];
    fresh.insert(fresh.end(), l.begin(), l.end());
  }
#pragma omp parallel for schedule(static)
  for (long k = 0; k < (long)fresh.size(); k++) {
    Inter& it = fresh[k];
    auto lb = std::lower_bound(o.inter.begin(), o.inter.end(), it, key_less);
    if (lb != o.inter.end() && key_eq(*lb, it)) {
      it.friction = lb->friction;
      it.moment = lb->moment;
    } else if (!o.broken_hist.empty()) {
      auto bb = std::lower_bound(o.broken_hist.begin(), o.broken_hist.end(), it, key_less);
      if (bb != o.broken_hist.end() && key_eq(*bb, it)) {
        it.friction = bb->friction;
        it.moment = bb->moment;
      }
    }
  }
  o.broken_hist.clear();
  o.inter.swap(fresh);
  o.own_first.assign(o.n, -1);
  o.own_cnt.assign(o.n, 0);
  for (size_t k = 0; k < o.inter.size(); k++) {
    const Inter& it = o.inter[k];
    if (o.own_first[it.oi] < 0) o.own_first[it.oi] = (int32_t)k;
    o.own_cnt[it.oi]++;
  }
  o.rev_off.assign(o.n + 1, 0);
  for (const Inter& it : o.inter)
    if (it.type <= DEM_ITYPE_EDGE_EDGE) o.rev_off[it.pj + 1]++;
  for (size_t i = 0; i < o.n; i++) o.rev_off[i + 1] += o.rev_off[i];
  o.rev_idx.assign(o.rev_off[o.n], 0);
  {
    std::vector<size_t> cur(o.rev_off.begin(), o.rev_off.end() - 1);
    for (size_t k = 0; k < o.inter.size(); k++)
      if (o.inter[k].type <= DEM_ITYPE_EDGE_EDGE) o.rev_idx[cur[o.inter[k].pj]++] = (int32_t)k;
  }
  o.rec.assign(o.inter.size(), Rec{});
  o.bx = o.rx;
  o.by = o.ry;
  o.bz = o.rz;
  o.bvtx = o.vtx;  // backup_dem: vertices at this rebuild
  o.rebuilds++;
  return DEM_OK;
}

// polyhedron::ContactLawFunc<0..3> (polyhedron/contact.hpp:123-211) and ContactLawDriverFunc
// (:237-303).  The record is written in the owner frame: f on the owner, torque on the
// owner and on the partner (for swap = 1 the contact law's particle i is the partner).
void contact_one_poly(Oracle& o, size_t k) {
  Inter& it = o.inter[k];
  Rec& rc = o.rec[k];
  rc = Rec{};
  const bool cohesive = o.prm.law == DEM_LAW_HOOKE_COHESIVE;
  const bool dmt = o.prm.law == DEM_LAW_HOOKE_DMT;
  const double dt = o.prm.dt;
  if (it.type >= DEM_ITYPE_VERTEX_MESH_VERTEX) {
    // ContactLawRShapeDriverFunc (polyhedron/contact.hpp:305-432): detect<type>,
    // reff = compute_effective_radius of the Minkowski radii; types 7-10 apply the
    // law with the particle as i, 11-12 with the mesh as i (the particle takes -f
    // and -moment, the friction is stored negated)
    const size_t p = it.oi;
    const PShape& sh = o.shapes[o.type[p]];
    const double ra = sh.r * o.hom[p];
    const MeshO& m = o.meshes[o.drivers[it.pj].mesh];
    const std::vector<V3>& va = o.vtx[p];
    const int os = (int)it.osub, ps = (int)it.psub;
    Det d;
    switch (it.type) {
      case DEM_ITYPE_VERTEX_MESH_VERTEX: d = detect_vv(va[os], ra, m.w[ps], m.r); break;
      case DEM_ITYPE_VERTEX_MESH_EDGE: d = detect_ve(va[os], ra, m.w[m.e[2 * ps]], m.w[m.e[2 * ps + 1]], m.r); break;
      case DEM_ITYPE_VERTEX_MESH_FACE: d = detect_vf(va[os], ra, m.w, m.f[ps], m.r); break;
      case DEM_ITYPE_EDGE_MESH_EDGE:
        d = detect_ee(va[sh.e[2 * os]], va[sh.e[2 * os + 1]], ra, m.w[m.e[2 * ps]], m.w[m.e[2 * ps + 1]], m.r);
        break;
      case DEM_ITYPE_MESH_VERTEX_EDGE: d = detect_ve(m.w[ps], m.r, va[sh.e[2 * os]], va[sh.e[2 * os + 1]], ra); break;
      default: d = detect_vf(m.w[ps], m.r, va, sh.f[os], ra);
    }
    const dem_contact_params& cpar = o.driver_params(p, it.pj);
    bool contact = d.c;
    if (cohesive) contact = (contact || d.dn <= cpar.dncut);
    if (contact) {
      const V3 r = pos(o, p);
      const V3 v = {o.vx[p], o.vy[p], o.vz[p]};
      const V3 w = {o.wx[p], o.wy[p], o.wz[p]};
      const double meff = o.mass[p];
      const double reff = dmt ? (ra * m.r) / (ra + m.r) : 0.0;
      const V3 zero = {0, 0, 0};
      V3 f = {0, 0, 0};
      if (it.type <= DEM_ITYPE_EDGE_MESH_EDGE) {
        contact_force_core(cohesive, d.dn, d.n, dt, cpar, meff, it.friction, d.cp, r, v, f, it.moment, w, m.center,
                           zero, zero, dmt, reff);
        rc.f = f;
        rc.ti = cross(d.cp - r, f) + it.moment;
        rc.sfn = f - it.friction;
        rc.sft = it.friction;
      } else {
        contact_force_core(cohesive, d.dn, d.n, dt, cpar, meff, it.friction, d.cp, m.center, zero, f, it.moment,
                           zero, r, v, w, dmt, reff);
        rc.f = -f;
        rc.ti = cross(d.cp - r, -f) + (-it.moment);
        rc.sfn = it.friction - f;
        it.friction = -it.friction;
        rc.sft = it.friction;
      }
      rc.active = d.dn < 0;
      rc.sdn = d.dn;
      rc.scp = d.cp;
    } else {
      it.friction = {0, 0, 0};
      it.moment = {0, 0, 0};
      rc.scp = d.cp;  // dn = 0, the detector's contact point
    }
    return;
  }
  if (it.type >= DEM_ITYPE_VERTEX_CYLINDER) {
    const size_t p = it.oi;
    const PShape& sh = o.shapes[o.type[p]];
    const double h = o.hom[p];
    const V3 r = pos(o, p);
    const Driver& dv = o.drivers[it.pj];
    double dn = 0;
    V3 n{}, cp{};
    bool contact;
    V3 dpos, dvel, dvrot;
    const V3& vert = o.vtx[p][it.osub];
    if (dv.kind == 0) {
      contact = surface_detect(dv.s, sh.r * h, vert, dn, n, cp);
      dpos = dv.s.center;
      dvel = dv.s.vel;
      dvrot = dv.s.vrot;
    } else {
      contact = cylinder_detect(dv.c, sh.r * h, vert, dn, n, cp);
      dpos = dv.c.center;
      dvel = dv.c.vel;
      dvrot = dv.c.vrot;
    }
    const dem_contact_params& cpar = o.driver_params(p, it.pj);
    if (cohesive) contact = (contact || dn <= cpar.dncut);
    if (contact) {
      const V3 v = {o.vx[p], o.vy[p], o.vz[p]};
      const V3 vrot = {o.wx[p], o.wy[p], o.wz[p]};
      const double meff = o.mass[p];
      V3 f = {0, 0, 0};
      contact_force_core(cohesive, dn, n, dt, cpar, meff, it.friction, cp, r, v, f, it.moment, vrot, dpos, dvel, dvrot,
                         dmt, h * sh.r);  // reff = shp.minkowski(h) (polyhedron/contact.hpp:281)
      rc.f = f;
      rc.ti = cross(cp - r, f) + it.moment;
      rc.active = dn < 0;
      rc.sdn = dn;  // polyhedron/contact.hpp:286-303
      rc.scp = cp;
      rc.sfn = f - it.friction;
      rc.sft = it.friction;
    } else {
      it.friction = {0, 0, 0};
      it.moment = {0, 0, 0};
      rc.scp = cp;  // dn = 0; the detector's contact point
    }
    return;
  }
  // particle i of the contact law: pi_ (= owner unless swap)
  const size_t ip = it.swap ? it.pj : it.oi;
  const size_t jp = it.swap ? it.oi : it.pj;
  const dem_contact_params& cpar = o.pair_params(ip, jp);
  const uint32_t sub_i = it.swap ? it.psub : it.osub;
  const uint32_t sub_j = it.swap ? it.osub : it.psub;
  const PShape& shi = o.shapes[o.type[ip]];
  const PShape& shj = o.shapes[o.type[jp]];
  const double ri_m = shi.r * o.hom[ip], rj_m = shj.r * o.hom[jp];
  const std::vector<V3>& vi = o.vtx[ip];
  const std::vector<V3>& vj = o.vtx[jp];
  Det d;
  switch (it.type) {
    case DEM_ITYPE_VERTEX_VERTEX: d = detect_vv(vi[sub_i], ri_m, vj[sub_j], rj_m); break;
    case DEM_ITYPE_VERTEX_EDGE: d = detect_ve(vi[sub_i], ri_m, vj[shj.e[2 * sub_j]], vj[shj.e[2 * sub_j + 1]], rj_m); break;
    case DEM_ITYPE_VERTEX_FACE: d = detect_vf(vi[sub_i], ri_m, vj, shj.f[sub_j], rj_m); break;
    default:
      d = detect_ee(vi[shi.e[2 * sub_i]], vi[shi.e[2 * sub_i + 1]], ri_m, vj[shj.e[2 * sub_j]], vj[shj.e[2 * sub_j + 1]],
                    rj_m);
  }
  bool contact = d.c;
  if (cohesive) contact = (contact || d.dn <= cpar.dncut);
  if (contact) {
    const V3 r_i = pos(o, ip), r_j = pos(o, jp);
    const V3 v_i = {o.vx[ip], o.vy[ip], o.vz[ip]}, v_j = {o.vx[jp], o.vy[jp], o.vz[jp]};
    const V3 w_i = {o.wx[ip], o.wy[ip], o.wz[ip]}, w_j = {o.wx[jp], o.wy[jp], o.wz[jp]};
    const double meff = (o.mass[ip] * o.mass[jp]) / (o.mass[ip] + o.mass[jp]);
    V3 f = {0, 0, 0};
    // reff = compute_effective_mass(rad_i, rad_j) of the Minkowski radii (polyhedron/contact.hpp:179-183)
    const double rad_i = o.hom[ip] * shi.r, rad_j = o.hom[jp] * shj.r;
    const double reff = dmt ? (rad_i * rad_j) / (rad_i + rad_j) : 0.0;
    contact_force_core(cohesive, d.dn, d.n, dt, cpar, meff, it.friction, d.cp, r_i, v_i, f, it.moment, w_i, r_j, v_j,
                       w_j, dmt, reff);
    const V3 t_i = cross(d.cp - r_i, f) + it.moment;
    const V3 t_j = cross(d.cp - r_j, -f) + (-it.moment);
    if (!it.swap) {
      rc.f = f;
      rc.ti = t_i;
      rc.tj = t_j;
    } else {
      rc.f = -f;
      rc.ti = t_j;
      rc.tj = t_i;
    }
    rc.active = d.dn < 0;
    // the state in the contact law's frame (polyhedron/contact.hpp:191-210)
    rc.sdn = d.dn;
    rc.scp = d.cp;
    rc.sfn = f - it.friction;
    rc.sft = it.friction;
  } else {
    it.friction = {0, 0, 0};
    it.moment = {0, 0, 0};
    rc.scp = d.cp;  // item.reset(), dn = 0
  }
}

// vertex_displ_over (src/polyhedron/vertex_displ_over.cu:74-134, backup_dem.hpp:65-110)
int vertex_displ_over(const Oracle& o) {
  const double max_displ = o.prm.rcut_inc * 0.5;
  const double thr2 = max_displ * max_displ;
  int over = 0;
#pragma omp parallel for schedule(static) reduction(| : over)
  for (long ii = 0; ii < (long)o.n; ii++) {
    const size_t i = (size_t)ii;
    for (size_t v = 0; v < o.vtx[i].size(); v++) {
      const V3 dr = o.vtx[i][v] - o.bvtx[i][v];
      if (dot(dr, dr) >= thr2) over |= 1;
    }
  }
  return over;
}


// ------------------------------------------------------------ inner bonds
// shape::compute_face_areas (src/shape/include/exaDEM/shape.hpp:674-697): the
// fan of triangles from the face's first vertex
double face_area(const PShape& sh, const std::vector<int>& f) {
  double surface = 0;
  if (f.size() < 3) return 0;
  const V3& v0 = sh.v[f[0]];
  for (int j = 1; j < (int)f.size() - 1; j++) {
    const int k = j + 1;
    const V3 v1 = sh.v[f[j]] - v0;
    const V3 v2 = sh.v[f[k]] - v0;
    surface += 0.5 * norm(cross(v1, v2));
  }
  return surface;
}
inline V3 stick_normalize(const V3& in) {  // normalize (stick_polyhedra.cpp:40-43)
  const double inv_norm = 1.0 / norm(in);
  return in * inv_norm;
}

// check_stiked_face (interaction_manager.hpp:225-277): the bonded vertices of
// particle i lie in the plane of the first three
bool check_stuck_face(const std::vector<Bond>& local, const std::vector<V3>& va) {
  if (local.empty()) return true;
  if (local.size() <= 2) return false;
  std::vector<V3> v;
  for (const Bond& b : local) v.push_back(va[b.sub_i]);
  const V3 normal = cross(v[1] - v[0], v[2] - v[0]);
  for (size_t j = 3; j < v.size(); j++)
    if (std::fabs(dot(v[j] - v[0], normal)) > 1.e-10) return false;
  return true;
}

// The bonds of the pair (a, b), id_a < id_b (stick_polyhedra.cpp:235-350).
void stick_pair(const Oracle& o, size_t a, size_t b, double dn_crit, std::vector<Bond>& out) {
  const PShape& si = o.shapes[o.type[a]];
  const PShape& sj = o.shapes[o.type[b]];
  const double hi = o.hom[a], hj = o.hom[b];
  const double ri = si.r * hi, rj = sj.r * hj;
  const std::vector<V3>& va = o.vtx[a];
  const std::vector<V3>& vb = o.vtx[b];
  const dem_inner_bond_params& ibp = o.bond_params(a, b);
  const int nfi = si.nf(), nfj = sj.nf();
  std::vector<V3> nj(nfj);
  for (int j = 0; j < nfj; j++) {
    const std::vector<int>& f = sj.f[j];
    if (f.size() < 3) continue;
    nj[j] = stick_normalize(cross(vb[f[1]] - vb[f[0]], vb[f[2]] - vb[f[0]]));
  }
  std::vector<Bond> local;
  bool found = false;
  for (int i = 0; i < nfi && !found; i++) {
    const std::vector<int>& fi = si.f[i];
    if (fi.size() < 3) continue;
    const V3 ni = stick_normalize(cross(va[fi[1]] - va[fi[0]], va[fi[2]] - va[fi[0]]));
    const double area_i = si.fa[i];
    for (int j = 0; j < nfj && !found; j++) {
      const std::vector<int>& fj = sj.f[j];
      if (fj.size() < 3) continue;
      if (fi.size() != fj.size()) continue;
      const double surface_ratio = area_i / sj.fa[j];
      if (surface_ratio > 1.01 || surface_ratio < 0.99) continue;
      if (norm(cross(ni, nj[j])) > 1.e-10) continue;
      const double area = si.fa[i] * hi * hi;  // get_face_area(i, h_i): id_i < id_j
      Bond proto{};
      proto.id_i = o.id[a];
      proto.id_j = o.id[b];
      proto.i = (int32_t)a;
      proto.j = (int32_t)b;
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
      for (size_t ivf = 0; ivf < fi.size(); ivf++) {
        for (size_t jvf = 0; jvf < fj.size(); jvf++) {
          const Det d = detect_vv(va[fi[ivf]], ri, vb[fj[jvf]], rj);
          if (d.dn <= dn_crit) {
            Bond bnd = proto;
            bnd.sub_i = (uint32_t)fi[ivf];
            bnd.sub_j = (uint32_t)fj[jvf];
            bnd.dn0 = d.dn;
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
  for (Bond& bnd : local) bnd.weight = 1. / static_cast<double>(local.size());
  if (check_stuck_face(local, va)) out.insert(out.end(), local.begin(), local.end());
}

// interfaces (update_interfaces.cpp:48-79) and the per-particle bond lists
void bond_lists(Oracle& o) {
  const size_t nb = o.bonds.size();
  o.iface.clear();
  for (size_t k = 0; k < nb; k++)
    if (k == 0 || o.bonds[k].id_i != o.bonds[k - 1].id_i || o.bonds[k].id_j != o.bonds[k - 1].id_j)
      o.iface.push_back(k);
  // the reference's scan never compares the last bond with the one before it:
  // a last interface of one bond joins the interface before it
  if (o.iface.size() >= 2 && o.iface.back() == nb - 1) o.iface.pop_back();
  o.iface.push_back(nb);
  o.bown_first.assign(o.n, -1);
  o.bown_cnt.assign(o.n, 0);
  o.brev_off.assign(o.n + 1, 0);
  for (size_t k = 0; k < nb; k++) {
    const Bond& b = o.bonds[k];
    if (o.bown_first[b.i] < 0) o.bown_first[b.i] = (int32_t)k;
    o.bown_cnt[b.i]++;
    o.brev_off[b.j + 1]++;
  }
  for (size_t i = 0; i < o.n; i++) o.brev_off[i + 1] += o.brev_off[i];
  o.brev_idx.assign(nb, 0);
  std::vector<size_t> cur(o.brev_off.begin(), o.brev_off.end() - 1);
  for (size_t k = 0; k < nb; k++) o.brev_idx[cur[o.bonds[k].j]++] = (int32_t)k;
}

// particle a owns an unbroken bond to the particle of id `id` (the ignore list,
// interaction_manager.hpp:114-160; a driver's partner id is its index)
bool bonded_to(const Oracle& o, size_t a, uint64_t id) {
  if (o.bown_first.size() != o.n || o.bown_first[a] < 0) return false;
  for (int32_t k = o.bown_first[a]; k < o.bown_first[a] + o.bown_cnt[a]; k++)
    if (o.bonds[k].id_j == id && o.bonds[k].unbroken) return true;
  return false;
}

// the broken bonds leave the list as vertex-vertex history (broke_interaction,
// inner_bond_interaction.hpp:202-210), for the rebuild that follows
void drop_broken_bonds(Oracle& o) {
  std::vector<Bond> keep;
  std::vector<BondRec> keep_rec;
  for (size_t k = 0; k < o.bonds.size(); k++) {
    const Bond& b = o.bonds[k];
    if (b.unbroken) {
      keep.push_back(b);
      keep_rec.push_back(k < o.brec.size() ? o.brec[k] : BondRec{});
      continue;
    }
    Inter it{};
    it.oid = b.id_i;
    it.pid = b.id_j;
    it.type = DEM_ITYPE_VERTEX_VERTEX;
    it.swap = 0;
    it.osub = b.sub_i;
    it.psub = b.sub_j;
    it.oi = b.i;
    it.pj = b.j;
    it.friction = b.friction;
    it.moment = {0, 0, 0};
    o.broken_hist.push_back(it);
  }
  o.bonds.swap(keep);
  o.brec.swap(keep_rec);
  std::stable_sort(o.broken_hist.begin(), o.broken_hist.end(), key_less);
  bond_lists(o);
}

// force_law_core (forcefield/inner_bond_force.hpp:24-70)
void bond_law_core(double dn, const V3& n, double dn0, double weight, double dt, const dem_inner_bond_params& p,
                   double meff, double& En, V3& tds, double& Et, V3& ft, const V3& cp, const V3& pos_i,
                   const V3& vel_i, V3& f_i, const V3& vrot_i, const V3& pos_j, const V3& vel_j,
                   const V3& vrot_j) {
  const double damp = p.damp_rate * 2.0 * std::sqrt(p.kn * meff);  // compute_damp
  const V3 contribution_i = vel_i - cross(cp - pos_i, vrot_i);     // compute_relative_velocity
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
  const V3 vt = vel - vn * n;  // compute_tangential_force(dt, vn, n, vel)
  const V3 ds = dt * vt;
  tds += ds;
  ft = kt_w * tds;
  f_i = vfn + ft;
  En = static_cast<double>(fne <= 0) * (0.5 * kn_w * delta * delta);
  Et = 0.5 * kt_w * dot(tds, tds);
}

// inner_bond_law (polyhedron/inner_bond.hpp:112-186): vertex-vertex detection of
// the bonded vertices, force_law_core, compute_moments with a zero moment
void bond_one(Oracle& o, size_t k) {
  Bond& B = o.bonds[k];
  BondRec& r = o.brec[k];
  const size_t i = (size_t)B.i, j = (size_t)B.j;
  const double ri = o.shapes[o.type[i]].r * o.hom[i];
  const double rj = o.shapes[o.type[j]].r * o.hom[j];
  const Det d = detect_vv(o.vtx[i][B.sub_i], ri, o.vtx[j][B.sub_j], rj);
  const V3 pos_i = pos(o, i), pos_j = pos(o, j);
  const double mi = o.mass[i], mj = o.mass[j];
  const double meff = (mi * mj) / (mi + mj);
  V3 f{};
  bond_law_core(d.dn, d.n, B.dn0, B.weight, o.prm.dt, o.bond_params(i, j), meff, B.en, B.tds, B.et, B.friction, d.cp,
                pos_i, {o.vx[i], o.vy[i], o.vz[i]}, f, {o.wx[i], o.wy[i], o.wz[i]}, pos_j,
                {o.vx[j], o.vy[j], o.vz[j]}, {o.wx[j], o.wy[j], o.wz[j]});
  r.f = f;
  r.ti = cross(d.cp - pos_i, f) + V3{0, 0, 0};
  r.tj = cross(d.cp - pos_j, -f) + V3{0, 0, 0};
  r.dn = d.dn;
  r.fn = f - B.friction;
}

// bond pass, then per particle its owned bonds and the bonds where it is j, in bond order
void bond_force(Oracle& o) {
  if (o.brec.size() != o.bonds.size()) o.brec.assign(o.bonds.size(), BondRec{});
#pragma omp parallel for schedule(static)
  for (long k = 0; k < (long)o.bonds.size(); k++) bond_one(o, (size_t)k);
#pragma omp parallel for schedule(static)
  for (long ii = 0; ii < (long)o.n; ii++) {
    const size_t i = (size_t)ii;
    V3 f = {o.fx[i], o.fy[i], o.fz[i]};
    V3 m = {o.mx[i], o.my[i], o.mz[i]};
    if (o.bown_first[i] >= 0)
      for (int32_t k = o.bown_first[i]; k < o.bown_first[i] + o.bown_cnt[i]; k++) {
        f += o.brec[k].f;
        m += o.brec[k].ti;
      }
    for (size_t q = o.brev_off[i]; q < o.brev_off[i + 1]; q++) {
      const BondRec& r = o.brec[o.brev_idx[q]];
      f += -r.f;
      m += r.tj;
    }
    o.fx[i] = f.x;
    o.fy[i] = f.y;
    o.fz[i] = f.z;
    o.mx[i] = m.x;
    o.my[i] = m.y;
    o.mz[i] = m.z;
  }
}

// apply_interface_fracture_criterion (apply_interface_fracture_criterion.hpp:35-76)
// and broken_interface_friction_updater (broken_interface_friction_updater.cpp:
// 52-86), on the state of the last bond pass.  Returns the interfaces broken.
uint64_t fracture(Oracle& o) {
  const long nif = (long)o.iface.size() - 1;
  if (nif <= 0 || o.brec.size() != o.bonds.size()) return 0;
  uint64_t broken = 0;
#pragma omp parallel for schedule(static) reduction(+ : broken)
  for (long q = 0; q < nif; q++) {
    const size_t off = o.iface[q], size = o.iface[q + 1] - off;
    double En = 0.0, Et = 0.0, S = 0.0;
    for (size_t j = off; j < off + size; j++) {
      En += o.bonds[j].en;
      Et += o.bonds[j].et;
      if (o.brec[j].dn > 0.0) S += norm(o.brec[j].fn);
    }
    S /= size;
    const Bond& c = o.bonds[off];
    bool brk = false;
    if (c.mode == DEM_RUPTURE_ENERGY_MIXED) {
      if (En + Et > c.c1) brk = true;
    } else if (c.mode == DEM_RUPTURE_ENERGY_SEPARATE) {
      if (En > c.c1 || Et > c.c2) brk = true;
    } else if (c.mode == DEM_RUPTURE_STRESS_ENERGY_SEPARATE) {
      if ((En > c.c1) && (S > c.c2)) brk = true;
    }
    if (!brk) continue;
    broken++;
    for (size_t j = off; j < off + size; j++) {
      Bond& b = o.bonds[j];
      b.unbroken = 0;
      const V3 ftv = b.friction;
      const double ft = norm(ftv);
      const double mu = o.pair_params((size_t)b.i, (size_t)b.j).mu;
      const double ft_threshold = mu * norm(o.brec[j].fn);
      if (ft > ft_threshold && ft > 0) b.friction = ftv * ft_threshold / ft;
      if (o.brec[j].dn > 0) b.friction = {0, 0, 0};
    }
  }
  o.broken_total += broken;
  return broken;
}
}  // namespace

// ============================================================== C interface
extern "C" {

int oracle_create(const dem_params* p, void** out) {
  if (!p || !out) return DEM_ERR_INVALID_ARG;
  Oracle* o = new Oracle();
  o->prm = *p;
  *out = o;
  return DEM_OK;
}
int oracle_destroy(void* h) {
  delete (Oracle*)h;
  return DEM_OK;
}
// Parameters of a running system.  The contact law parameters (config /
// config_driver slots), dt and gravity are read at every step by the
// operators that use them (contact_force_sphere.cu.in, gravity_force.cu,
// combined_compute_prolog.cu), so they may change between steps with the list
// and its history kept.  A change of domain, skin or cell size needs a new
// grid and is not supported here.
int oracle_set_multimat(void* h, int ng, const dem_contact_params* pairs, int nd, const dem_contact_params* drivers) {
  if (!h || ng < 0 || nd < 0) return DEM_ERR_INVALID_ARG;
  Oracle& o = *(Oracle*)h;
  o.mm_ng = ng;
  o.mm_nd = nd;
  o.mm_pp.assign(pairs, pairs + (size_t)ng * ng);
  o.mm_pd.assign(drivers, drivers + (size_t)ng * nd);
  if (ng == 0) o.mm_pp.clear();
  return DEM_OK;
}
int oracle_set_params(void* h, const dem_params* p) {
  if (!h || !p) return DEM_ERR_INVALID_ARG;
  Oracle& o = *(Oracle*)h;
  if (std::memcmp(p->bounds_lo, o.prm.bounds_lo, sizeof(p->bounds_lo)) ||
      std::memcmp(p->bounds_hi, o.prm.bounds_hi, sizeof(p->bounds_hi)) ||
      std::memcmp(p->periodic, o.prm.periodic, sizeof(p->periodic)) || p->rcut_inc != o.prm.rcut_inc ||
      p->cell_size != o.prm.cell_size)
    return DEM_ERR_UNSUPPORTED;
  o.prm = *p;
  return DEM_OK;
}
int oracle_set_mesh_brute_force(int on) {
  g_mesh_brute_force = on ? 1 : 0;
  return DEM_OK;
}
int oracle_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
  return omp_get_max_threads();
#else
  (void)n;
  return 1;
#endif
}
int oracle_set_particles(void* h, const dem_particles* p) {
  Oracle& o = *(Oracle*)h;
  size_t n = p->n;
  o.n = n;
  auto cp = [n](std::vector<double>& v, const double* s, double dflt) {
    v.assign(n, dflt);
    if (s) std::memcpy(v.data(), s, n * sizeof(double));
  };
  cp(o.rx, p->rx, 0); cp(o.ry, p->ry, 0); cp(o.rz, p->rz, 0);
  cp(o.vx, p->vx, 0); cp(o.vy, p->vy, 0); cp(o.vz, p->vz, 0);
  cp(o.fx, p->fx, 0); cp(o.fy, p->fy, 0); cp(o.fz, p->fz, 0);
  cp(o.wx, p->vrotx, 0); cp(o.wy, p->vroty, 0); cp(o.wz, p->vrotz, 0);
  cp(o.ax, p->arotx, 0); cp(o.ay, p->aroty, 0); cp(o.az, p->arotz, 0);
  cp(o.mx, p->momx, 0); cp(o.my, p->momy, 0); cp(o.mz, p->momz, 0);
  cp(o.qw, p->qw, 1); cp(o.qx, p->qx, 0); cp(o.qy, p->qy, 0); cp(o.qz, p->qz, 0);
  cp(o.ix, p->inertiax, 1); cp(o.iy, p->inertiay, 1); cp(o.iz, p->inertiaz, 1);
  cp(o.mass, p->mass, 1); cp(o.rad, p->radius, 0.5); cp(o.hom, p->homothety, 1);
  o.id.assign(n, 0);
  for (size_t i = 0; i < n; i++) o.id[i] = p->id ? p->id[i] : i;
  o.type.assign(n, 0);
  o.group.assign(n, 0);
  if (p->type) std::memcpy(o.type.data(), p->type, n * 4);
  if (p->group) std::memcpy(o.group.data(), p->group, n * 4);
  o.bx = o.rx;
  o.by = o.ry;
  o.bz = o.rz;
  o.inter.clear();
  o.rec.clear();
  o.own_first.assign(n, -1);
  o.own_cnt.assign(n, 0);
  o.rev_off.assign(n + 1, 0);
  o.rev_idx.clear();
  o.bonds.clear();
  o.brec.clear();
  o.broken_hist.clear();
  o.bown_first.clear();
  o.iface.assign(1, 0);
  return DEM_OK;
}
int oracle_get_particles(void* h, dem_particles* p) {
  Oracle& o = *(Oracle*)h;
  if (p->n < o.n) return DEM_ERR_INVALID_ARG;
  auto cp = [&](double* d, const std::vector<double>& v) {
    if (d) std::memcpy(d, v.data(), o.n * sizeof(double));
  };
  cp(p->rx, o.rx); cp(p->ry, o.ry); cp(p->rz, o.rz);
  cp(p->vx, o.vx); cp(p->vy, o.vy); cp(p->vz, o.vz);
  cp(p->fx, o.fx); cp(p->fy, o.fy); cp(p->fz, o.fz);
  cp(p->vrotx, o.wx); cp(p->vroty, o.wy); cp(p->vrotz, o.wz);
  cp(p->arotx, o.ax); cp(p->aroty, o.ay); cp(p->arotz, o.az);
  cp(p->momx, o.mx); cp(p->momy, o.my); cp(p->momz, o.mz);
  cp(p->qw, o.qw); cp(p->qx, o.qx); cp(p->qy, o.qy); cp(p->qz, o.qz);
  cp(p->inertiax, o.ix); cp(p->inertiay, o.iy); cp(p->inertiaz, o.iz);
  cp(p->mass, o.mass); cp(p->radius, o.rad); cp(p->homothety, o.hom);
  if (p->id) std::memcpy(p->id, o.id.data(), o.n * 8);
  if (p->type) std::memcpy(p->type, o.type.data(), o.n * 4);
  if (p->group) std::memcpy(p->group, o.group.data(), o.n * 4);
  p->n = o.n;
  return DEM_OK;
}
int oracle_register_surface(void* h, const dem_surface* s) {
  Oracle& o = *(Oracle*)h;
  Driver d{};
  d.kind = 0;
  d.s = surface_from(s);
  o.drivers.push_back(d);
  return DEM_OK;
}
int oracle_register_cylinder(void* h, const dem_cylinder* c) {
  Oracle& o = *(Oracle*)h;
  Driver d{};
  d.kind = 1;
  d.c = cylinder_from(c);
  o.drivers.push_back(d);
  return DEM_OK;
}
int oracle_register_mesh(void* h, const dem_mesh* s) {  // register_stl_mesh (register_stl_mesh.cpp:40-147)
  Oracle& o = *(Oracle*)h;
  MeshO m;
  m.r = s->minkowski;
  m.center = {s->center[0], s->center[1], s->center[2]};
  const Quat q = {s->quat[0], s->quat[1], s->quat[2], s->quat[3]};
  for (int k = 0; k < s->nv; k++) {
    const V3 v = {s->vertices[3 * k], s->vertices[3 * k + 1], s->vertices[3 * k + 2]};
    m.w.push_back(m.center + rotate(q, 1.0 * v));  // shape::get_vertex(i, center, 1.0, quat)
  }
  m.e.assign(s->edges, s->edges + 2 * s->ne);
  for (int f = 0; f < s->nf; f++)
    m.f.emplace_back(s->face_vertices + s->face_offsets[f], s->face_vertices + s->face_offsets[f + 1]);
  Driver d{};
  d.kind = 2;
  d.mesh = (int)o.meshes.size();
  o.meshes.push_back(std::move(m));
  o.drivers.push_back(d);
  return DEM_OK;
}
static int rebuild(Oracle& o) { return o.poly ? update_neighbors_poly(o) : update_neighbors(o); }
static int trigger(Oracle& o) {
  if (o.poly) {
    compute_vertices(o);  // compute_fast_vertices / the vertices vertex_displ_over recomputes
    return vertex_displ_over(o);
  }
  return displ_over(o);
}
int oracle_update_neighbors(void* h) { return rebuild(*(Oracle*)h); }
int oracle_displ_over(void* h, int* r) {
  *r = trigger(*(Oracle*)h);
  return DEM_OK;
}
int oracle_compute_vertices(void* h) {
  compute_vertices(*(Oracle*)h);
  return DEM_OK;
}
int oracle_set_shapes(void* h, const dem_shape* shp, int nshapes) {
  Oracle& o = *(Oracle*)h;
  if (!shp || nshapes <= 0) return DEM_ERR_INVALID_ARG;
  o.shapes.clear();
  for (int s = 0; s < nshapes; s++) {
    PShape ps;
    for (int k = 0; k < shp[s].nv; k++)
      ps.v.push_back({shp[s].vertices[3 * k], shp[s].vertices[3 * k + 1], shp[s].vertices[3 * k + 2]});
    ps.e.assign(shp[s].edges, shp[s].edges + 2 * shp[s].ne);
    int off = 0;
    for (int f = 0; f < shp[s].nf; f++) {
      ps.f.emplace_back(shp[s].face_vertices + off, shp[s].face_vertices + off + shp[s].face_sizes[f]);
      off += shp[s].face_sizes[f];
    }
    ps.r = shp[s].radius;
    const dem_shape& d = shp[s];
    ps.obb.c = {d.obb_center[0], d.obb_center[1], d.obb_center[2]};
    ps.obb.e1 = {d.obb_e1[0], d.obb_e1[1], d.obb_e1[2]};
    ps.obb.e2 = {d.obb_e2[0], d.obb_e2[1], d.obb_e2[2]};
    ps.obb.e3 = {d.obb_e3[0], d.obb_e3[1], d.obb_e3[2]};
    ps.obb.ext = {d.obb_extent[0], d.obb_extent[1], d.obb_extent[2]};
    for (const auto& f : ps.f) ps.fa.push_back(face_area(ps, f));
    o.shapes.push_back(ps);
  }
  o.poly = true;
  return DEM_OK;
}
int oracle_reset_force_moment(void* h) {
  reset_force_moment(*(Oracle*)h);
  return DEM_OK;
}
int oracle_gravity_force(void* h) {
  gravity_force(*(Oracle*)h);
  return DEM_OK;
}
int oracle_contact_sphere(void* h) {
  contact_all(*(Oracle*)h);
  return DEM_OK;
}
int oracle_force_to_accel(void* h) {
  force_to_accel(*(Oracle*)h);
  return DEM_OK;
}
int oracle_prolog(void* h) {
  prolog(*(Oracle*)h);
  return DEM_OK;
}
int oracle_epilog(void* h) {
  epilog(*(Oracle*)h);
  return DEM_OK;
}
// first_iteration (main-config.msp:55-65)
int oracle_first_iteration(void* h) {
  Oracle& o = *(Oracle*)h;
  int rc = rebuild(o);
  if (rc) return rc;
  reset_force_moment(o);
  compute_force(o);
  return DEM_OK;
}
// numerical_scheme_verlet (config_numerical_schemes.msp:6-28)
int oracle_step(void* h, int nsteps) {
  Oracle& o = *(Oracle*)h;
  for (int s = 0; s < nsteps; s++) {
    prolog(o);
    // evaluate_particle_displ with fragmentation (config_fragmentation.msp:28-38):
    // vertex displacement, then the interface criterion; either one rebuilds
    int over = trigger(o);
    if (o.poly && !o.bonds.empty() && fracture(o) > 0) over = 1;
    if (over) {
      int rc = rebuild(o);
      if (rc) return rc;
    }
    reset_force_moment(o);
    compute_force(o);
    force_to_accel(o);
    epilog(o);
  }
  return DEM_OK;
}
// ---- inner bonds
int oracle_set_inner_bond_params(void* h, int ng, const dem_inner_bond_params* pairs) {
  Oracle& o = *(Oracle*)h;
  if (ng < 0 || !pairs) return DEM_ERR_INVALID_ARG;
  const size_t cnt = ng == 0 ? 1 : (size_t)ng * ng;
  for (size_t k = 0; k < cnt; k++)
    if (pairs[k].mode < DEM_RUPTURE_ENERGY_MIXED || pairs[k].mode > DEM_RUPTURE_STRESS_ENERGY_SEPARATE)
      return DEM_ERR_INVALID_ARG;
  o.ibp.assign(pairs, pairs + cnt);
  o.ib_ng = ng;
  return DEM_OK;
}
static int index_of_ids(Oracle& o, std::vector<std::pair<uint64_t, int32_t>>& ids) {
  ids.resize(o.n);
  for (size_t i = 0; i < o.n; i++) ids[i] = {o.id[i], (int32_t)i};
  std::sort(ids.begin(), ids.end());
  return DEM_OK;
}
static int32_t find_id(const std::vector<std::pair<uint64_t, int32_t>>& ids, uint64_t id) {
  auto it = std::lower_bound(ids.begin(), ids.end(), std::make_pair(id, (int32_t)-1));
  return (it != ids.end() && it->first == id) ? it->second : -1;
}
// stick_polyhedra: replaces the interaction storage with the bonds (the contacts'
// history is dropped, stick_polyhedra.cpp:116-120 and update_extra_storage<false>)
int oracle_stick_polyhedra(void* h, const uint64_t* ids_in, const double* cluster_in, uint64_t n, double thr,
                           uint64_t* nbonds) {
  Oracle& o = *(Oracle*)h;
  if (!o.poly || o.ib_ng < 0) return DEM_ERR_STATE;
  if (n != o.n || (n && (!ids_in || !cluster_in))) return DEM_ERR_INVALID_ARG;
  std::vector<std::pair<uint64_t, int32_t>> ids;
  index_of_ids(o, ids);
  std::vector<double> cl(o.n);
  std::vector<uint8_t> seen(o.n, 0);
  for (uint64_t k = 0; k < n; k++) {
    const int32_t i = find_id(ids, ids_in[k]);
    if (i < 0 || seen[i]) return DEM_ERR_INVALID_ARG;
    seen[i] = 1;
    cl[i] = cluster_in[k];
  }
  compute_vertices(o);
  const double nd = nbh_dist(o);
  const double rcut2 = nd * nd;
  std::vector<std::vector<Bond>> per(o.n);
#pragma omp parallel for schedule(dynamic, 16)
  for (long aa = 0; aa < (long)o.n; aa++) {
    const size_t a = (size_t)aa;
    for (size_t b = 0; b < o.n; b++) {
      if (b == a || cl[b] != cl[a] || o.id[a] >= o.id[b]) continue;
      const double dx = o.rx[b] - o.rx[a], dy = o.ry[b] - o.ry[a], dz = o.rz[b] - o.rz[a];
      if (!(dx * dx + dy * dy + dz * dz < rcut2)) continue;
      stick_pair(o, a, b, thr, per[a]);
    }
  }
  o.bonds.clear();
  for (auto& v : per) o.bonds.insert(o.bonds.end(), v.begin(), v.end());
  std::stable_sort(o.bonds.begin(), o.bonds.end(), bond_less);
  o.brec.assign(o.bonds.size(), BondRec{});
  o.broken_hist.clear();
  o.inter.clear();
  o.rec.clear();
  o.own_first.assign(o.n, -1);
  o.own_cnt.assign(o.n, 0);
  o.rev_off.assign(o.n + 1, 0);
  o.rev_idx.clear();
  bond_lists(o);
  if (nbonds) *nbonds = o.bonds.size();
  return DEM_OK;
}
int oracle_bond_count(void* h, uint64_t* out) {
  *out = ((Oracle*)h)->bonds.size();
  return DEM_OK;
}
// dem_get_bond_state: dn, fn = f_i - friction, friction of the last bond pass
// (inner_bond.hpp:167-184), in bond order
int oracle_get_bond_state(void* h, uint64_t capacity, uint64_t* count, double* dn, double* fn, double* ft) {
  Oracle& o = *(Oracle*)h;
  const uint64_t m = o.bonds.size();
  if (count) *count = m;
  if (capacity < m) return DEM_ERR_INVALID_ARG;
  for (uint64_t k = 0; k < m; k++) {
    const BondRec r = k < o.brec.size() ? o.brec[k] : BondRec{};
    const Bond& b = o.bonds[k];
    if (dn) dn[k] = r.dn;
    const double n3[3] = {r.fn.x, r.fn.y, r.fn.z}, f3[3] = {b.friction.x, b.friction.y, b.friction.z};
    for (int d = 0; d < 3; d++) {
      if (fn) fn[3 * k + d] = n3[d];
      if (ft) ft[3 * k + d] = f3[d];
    }
  }
  return DEM_OK;
}
int oracle_get_bonds(void* h, dem_bond_list* l) {
  Oracle& o = *(Oracle*)h;
  l->count = o.bonds.size();
  if (l->capacity < o.bonds.size()) return DEM_ERR_INVALID_ARG;
  for (size_t k = 0; k < o.bonds.size(); k++) {
    const Bond& b = o.bonds[k];
    if (l->id_i) l->id_i[k] = b.id_i;
    if (l->id_j) l->id_j[k] = b.id_j;
    if (l->sub_i) l->sub_i[k] = b.sub_i;
    if (l->sub_j) l->sub_j[k] = b.sub_j;
    if (l->dn0) l->dn0[k] = b.dn0;
    if (l->weight) l->weight[k] = b.weight;
    if (l->mode) l->mode[k] = b.mode;
    if (l->crit1) l->crit1[k] = b.c1;
    if (l->crit2) l->crit2[k] = b.c2;
    if (l->en) l->en[k] = b.en;
    if (l->et) l->et[k] = b.et;
    const double t3[3] = {b.tds.x, b.tds.y, b.tds.z}, f3[3] = {b.friction.x, b.friction.y, b.friction.z};
    for (int d = 0; d < 3; d++) {
      if (l->tds) l->tds[3 * k + d] = t3[d];
      if (l->friction) l->friction[3 * k + d] = f3[d];
    }
    if (l->unbroken) l->unbroken[k] = b.unbroken;
  }
  return DEM_OK;
}
// read_dump_particle_fragmentation: the saved bonds, by particle id (the state
// of the last bond pass, dn and fn, starts at zero)
int oracle_set_bonds(void* h, const dem_bond_list* l) {
  Oracle& o = *(Oracle*)h;
  if (!o.poly) return DEM_ERR_STATE;
  std::vector<std::pair<uint64_t, int32_t>> ids;
  index_of_ids(o, ids);
  std::vector<Bond> lst(l->count);
  for (uint64_t k = 0; k < l->count; k++) {
    Bond& b = lst[k];
    b.id_i = l->id_i[k];
    b.id_j = l->id_j[k];
    b.i = find_id(ids, b.id_i);
    b.j = find_id(ids, b.id_j);
    if (b.i < 0 || b.j < 0 || b.id_i >= b.id_j) return DEM_ERR_INVALID_ARG;
    b.sub_i = l->sub_i[k];
    b.sub_j = l->sub_j[k];
    if (b.sub_i >= (uint32_t)o.shapes[o.type[b.i]].nv() || b.sub_j >= (uint32_t)o.shapes[o.type[b.j]].nv())
      return DEM_ERR_INVALID_ARG;
    b.dn0 = l->dn0[k];
    b.weight = l->weight[k];
    b.mode = l->mode[k];
    b.c1 = l->crit1[k];
    b.c2 = l->crit2[k];
    b.en = l->en[k];
    b.et = l->et[k];
    b.tds = {l->tds[3 * k], l->tds[3 * k + 1], l->tds[3 * k + 2]};
    b.friction = {l->friction[3 * k], l->friction[3 * k + 1], l->friction[3 * k + 2]};
    b.unbroken = l->unbroken[k] ? 1 : 0;
  }
  std::stable_sort(lst.begin(), lst.end(), bond_less);
  o.bonds.swap(lst);
  o.brec.assign(o.bonds.size(), BondRec{});
  o.broken_hist.clear();
  bond_lists(o);
  return DEM_OK;
}
int oracle_inner_bond_polyhedron(void* h) {
  Oracle& o = *(Oracle*)h;
  if (o.poly && !o.bonds.empty()) bond_force(o);
  return DEM_OK;
}
int oracle_apply_interface_fracture_criterion(void* h, uint64_t* broken) {
  Oracle& o = *(Oracle*)h;
  const uint64_t b = o.poly ? fracture(o) : 0;
  if (broken) *broken = b;
  return DEM_OK;
}
int oracle_broken_interface_count(void* h, uint64_t* out) {
  *out = ((Oracle*)h)->broken_total;
  return DEM_OK;
}
int oracle_rebuild_count(void* h, uint64_t* out) {
  *out = ((Oracle*)h)->rebuilds;
  return DEM_OK;
}
int oracle_state(void* h, dem_state* s) {  // ReduceSimulationStateFunctor (simulation_state.hpp:48-56)
  Oracle& o = *(Oracle*)h;
  std::memset(s, 0, sizeof(*s));
  for (size_t i = 0; i < o.n; i++) {
    const double m = o.mass[i];
    s->mass += m;
    s->rotation_energy[0] += 0.5 * o.wx[i] * o.wx[i] * m;
    s->rotation_energy[1] += 0.5 * o.wy[i] * o.wy[i] * m;
    s->rotation_energy[2] += 0.5 * o.wz[i] * o.wz[i] * m;
    s->kinetic_energy[0] += 0.5 * o.vx[i] * o.vx[i] * m;
    s->kinetic_energy[1] += 0.5 * o.vy[i] * o.vy[i] * m;
    s->kinetic_energy[2] += 0.5 * o.vz[i] * o.vz[i] * m;
  }
  s->n_particles = o.n;
  s->n_interactions = o.inter.size();
  s->n_active_interactions = o.n_active;
  return DEM_OK;
}
int oracle_interaction_count(void* h, uint64_t* out) {
  *out = ((Oracle*)h)->inter.size();
  return DEM_OK;
}
// read_dump_particle_interaction (src/io/sim_dump_reader_interaction.cpp:56-63): the saved
// list becomes the list the next rebuild carries history from, by key.
int oracle_set_interactions(void* h, const dem_interaction_list* l) {
  Oracle& o = *(Oracle*)h;
  std::vector<int32_t> idx_of;
  std::vector<std::pair<uint64_t, int32_t>> ids(o.n);
  for (size_t i = 0; i < o.n; i++) ids[i] = {o.id[i], (int32_t)i};
  std::sort(ids.begin(), ids.end());
  auto find = [&](uint64_t id) -> int32_t {
    auto it = std::lower_bound(ids.begin(), ids.end(), std::make_pair(id, (int32_t)-1));
    return (it != ids.end() && it->first == id) ? it->second : -1;
  };
  std::vector<Inter> lst(l->count);
  for (uint64_t k = 0; k < l->count; k++) {
    Inter& it = lst[k];
    it = Inter{};
    it.oid = l->owner_id[k];
    it.pid = l->partner_id[k];
    it.type = l->type[k];
    it.swap = l->swap[k];
    it.osub = l->owner_sub[k];
    it.psub = l->partner_sub[k];
    it.oi = find(it.oid);
    if (it.oi < 0) {
      o.err = "set_interactions: owner id is not a particle";
      return DEM_ERR_INVALID_ARG;
    }
    it.friction = {l->friction[3 * k], l->friction[3 * k + 1], l->friction[3 * k + 2]};
    it.moment = {l->moment[3 * k], l->moment[3 * k + 1], l->moment[3 * k + 2]};
  }
  std::stable_sort(lst.begin(), lst.end(), key_less);
  o.inter.swap(lst);
  o.rec.assign(o.inter.size(), Rec{});
  return DEM_OK;
}
int oracle_get_interactions(void* h, dem_interaction_list* l) {
  Oracle& o = *(Oracle*)h;
  l->count = o.inter.size();
  if (l->capacity < o.inter.size()) return DEM_ERR_INVALID_ARG;
  for (size_t k = 0; k < o.inter.size(); k++) {
    const Inter& it = o.inter[k];
    if (l->owner_id) l->owner_id[k] = it.oid;
    if (l->partner_id) l->partner_id[k] = it.pid;
    if (l->type) l->type[k] = it.type;
    if (l->swap) l->swap[k] = it.swap;
    if (l->owner_sub) l->owner_sub[k] = it.osub;
    if (l->partner_sub) l->partner_sub[k] = it.psub;
    if (l->friction) {
      l->friction[3 * k] = it.friction.x;
      l->friction[3 * k + 1] = it.friction.y;
      l->friction[3 * k + 2] = it.friction.z;
    }
    if (l->moment) {
      l->moment[3 * k] = it.moment.x;
      l->moment[3 * k + 1] = it.moment.y;
      l->moment[3 * k + 2] = it.moment.z;
    }
  }
  return DEM_OK;
}
// contact state of the last force pass, in InteractionPair order (polyhedron
// pairs: in the contact law's frame, particle i = pi_)
int oracle_get_contact_state(void* h, dem_contact_state* out) {
  Oracle& o = *(Oracle*)h;
  out->count = o.inter.size();
  if (out->capacity < o.inter.size()) return DEM_ERR_INVALID_ARG;
  for (size_t k = 0; k < o.rec.size() && k < o.inter.size(); k++) {
    const Rec& r = o.rec[k];
    if (out->dn) out->dn[k] = r.sdn;
    const double c3[3] = {r.scp.x, r.scp.y, r.scp.z}, n3[3] = {r.sfn.x, r.sfn.y, r.sfn.z},
                 t3[3] = {r.sft.x, r.sft.y, r.sft.z};
    for (int d = 0; d < 3; d++) {
      if (out->cp) out->cp[3 * k + d] = c3[d];
      if (out->fn) out->fn[3 * k + d] = n3[d];
      if (out->ft) out->ft[3 * k + d] = t3[d];
    }
  }
  return DEM_OK;
}
// stress_tensor (src/interaction/stress_tensor.cu:40-75): per particle, its own
// touching pairs then those where it is the partner, in InteractionPair order;
// m += f c^T row major; total: the sum over the particles in id order.  I.i()
// (pi_: the owner unless swap) takes +(fn + ft), I.j() -(fn + ft).
int oracle_stress_tensor(void* h, double* stress, double* total) {
  Oracle& o = *(Oracle*)h;
  std::vector<double> m(9 * o.n, 0.0);
  auto add = [](double* a, const V3& u, const V3& v) {
    const double uu[3] = {u.x, u.y, u.z}, vv[3] = {v.x, v.y, v.z};
    for (int r = 0; r < 3; r++)
      for (int c = 0; c < 3; c++) a[3 * r + c] = a[3 * r + c] + uu[r] * vv[c];
  };
  for (size_t i = 0; i < o.n; i++) {
    double* a = &m[9 * i];
    const V3 r = pos(o, i);
    if (o.own_first[i] >= 0)
      for (int32_t k = o.own_first[i]; k < o.own_first[i] + o.own_cnt[i]; k++) {
        const Rec& q = o.rec[k];
        const V3 fij = q.sfn + q.sft;
        if (q.sdn < 0.0) add(a, o.inter[k].swap ? -fij : fij, q.scp - r);
      }
    for (size_t p = o.rev_off[i]; p < o.rev_off[i + 1]; p++) {
      const Rec& q = o.rec[o.rev_idx[p]];
      const V3 fij = q.sfn + q.sft;
      if (q.sdn < 0.0) add(a, o.inter[o.rev_idx[p]].swap ? fij : -fij, q.scp - r);
    }
  }
  if (stress) std::copy(m.begin(), m.end(), stress);
  if (total) {
    std::vector<size_t> by_id(o.n);
    for (size_t i = 0; i < o.n; i++) by_id[i] = i;
    std::sort(by_id.begin(), by_id.end(), [&](size_t a, size_t b) { return o.id[a] < o.id[b]; });
    for (int q = 0; q < 9; q++) total[q] = 0.0;
    for (size_t i : by_id)
      for (int q = 0; q < 9; q++) total[q] = total[q] + m[9 * i + q];
  }
  return DEM_OK;
}
int oracle_set_analysis(void*, int) { return DEM_OK; }  // the oracle always keeps the state
int oracle_packing_profile(void* h, int nslabs, double zlo, double zhi, double* out) {
  Oracle& o = *(Oracle*)h;
  if (nslabs <= 0 || !(zhi > zlo)) return DEM_ERR_INVALID_ARG;
  const double dz = (zhi - zlo) / nslabs;
  const double area = L(o, 0) * L(o, 1);
  std::vector<double> vol(nslabs, 0.0);
  for (size_t i = 0; i < o.n; i++) {
    const double zc = o.rz[i], r = o.rad[i];
    int a = (int)std::floor((zc - r - zlo) / dz), b = (int)std::floor((zc + r - zlo) / dz);
    a = std::max(a, 0);
    b = std::min(b, nslabs - 1);
    for (int s = a; s <= b; s++) vol[s] += sphere_slab_volume(zc, r, zlo + s * dz, zlo + (s + 1) * dz);
  }
  for (int s = 0; s < nslabs; s++) out[s] = vol[s] / (area * dz);
  return DEM_OK;
}
// ------------------------------------------------------------ unit entry points
// Per-function entry points over n cases, with the row layouts of
// oracle/ref_harness.cpp (exaDEM's own functions compiled on the host), so the
// restatement above can be compared with exaDEM bit for bit.  Each calls the
// oracle function the step uses.
static inline V3 rv(const double* p) { return {p[0], p[1], p[2]}; }
static inline void wv(double* o, const V3& v) {
  o[0] = v.x;
  o[1] = v.y;
  o[2] = v.z;
}
static inline void wdet(double* o, const Det& d) {
  o[0] = d.c ? 1.0 : 0.0;
  o[1] = d.dn;
  wv(o + 2, d.n);
  wv(o + 5, d.cp);
}
static inline OBBr robb(const double* p) { return OBBr{rv(p), rv(p + 3), rv(p + 6), rv(p + 9), rv(p + 12)}; }
static inline void wobb(double* o, const OBBr& b) {
  wv(o, b.c);
  wv(o + 3, b.e1);
  wv(o + 6, b.e2);
  wv(o + 9, b.e3);
  wv(o + 12, b.ext);
}
// in (35): dn, n[3], dn0, weight, dt, kn, kt, damp_rate, meff, tds[3], cp[3], pos_i[3],
// vel_i[3], vrot_i[3], pos_j[3], vel_j[3], vrot_j[3]
// out (20): En, Et, tds[3], ft[3], f_i[3], torque_i[3], torque_j[3], fn[3] (= f_i - ft)
int oracle_unit_bond_law(long n, const double* in, double* out) {
  for (long c = 0; c < n; c++) {
    const double* p = in + 35 * c;
    double* o = out + 20 * c;
    dem_inner_bond_params prm{};
    prm.kn = p[7];
    prm.kt = p[8];
    prm.damp_rate = p[9];
    double En = 0, Et = 0;
    V3 tds = rv(p + 11), ft{}, f{};
    const V3 cp = rv(p + 14), pos_i = rv(p + 17), pos_j = rv(p + 26);
    bond_law_core(p[0], rv(p + 1), p[4], p[5], p[6], prm, p[10], En, tds, Et, ft, cp, pos_i, rv(p + 20), f,
                  rv(p + 23), pos_j, rv(p + 29), rv(p + 32));
    o[0] = En;
    o[1] = Et;
    wv(o + 2, tds);
    wv(o + 5, ft);
    wv(o + 8, f);
    wv(o + 11, cross(cp - pos_i, f) + V3{0, 0, 0});
    wv(o + 14, cross(cp - pos_j, -f) + V3{0, 0, 0});
    wv(o + 17, f - ft);
  }
  return DEM_OK;
}
// face areas of a shape scaled by h^2 (get_face_area(i, h), shape.hpp:359-362)
int oracle_unit_face_areas(const double* vertices, int nv, const int32_t* face_sizes, const int32_t* face_vertices,
                           int nf, double h, double* out) {
  PShape sh;
  for (int k = 0; k < nv; k++) sh.v.push_back(rv(vertices + 3 * k));
  int off = 0;
  for (int f = 0; f < nf; f++) {
    std::vector<int> fv(face_vertices + off, face_vertices + off + face_sizes[f]);
    off += face_sizes[f];
    out[f] = face_area(sh, fv) * h * h;
  }
  return DEM_OK;
}
int oracle_unit_contact_force_core(int law, long n, const double* in, double* out) {
  for (long c = 0; c < n; c++) {
    const double* p = in + 45 * c;
    double* o = out + 12 * c;
    dem_contact_params hkp{};
    hkp.kn = p[5];
    hkp.kt = p[6];
    hkp.kr = p[7];
    hkp.mu = p[8];
    hkp.damp_rate = p[9];
    hkp.fc = p[10];
    hkp.dncut = p[11];
    hkp.gamma = p[12];
    V3 ft = rv(p + 15), f_i = rv(p + 27), mom_i = rv(p + 30);
    const V3 cp = rv(p + 18), pos_i = rv(p + 21);
    contact_force_core(law == 1, p[0], rv(p + 1), p[4], hkp, p[13], ft, cp, pos_i, rv(p + 24), f_i, mom_i, rv(p + 33),
                       rv(p + 36), rv(p + 39), rv(p + 42), law == 2, p[14]);
    wv(o, f_i);
    wv(o + 3, ft);
    wv(o + 6, mom_i);
    wv(o + 9, cross(cp - pos_i, f_i) + mom_i);  // compute_moments, as in the force records
  }
  return DEM_OK;
}
int oracle_unit_damping(long n, const double* in, double* out) {
  for (long c = 0; c < n; c++) {
    const double* p = in + 5 * c;
    const double meff = (p[2] * p[3]) / (p[2] + p[3]);
    out[2 * c] = meff;
    out[2 * c + 1] = p[0] * 2.0 * std::sqrt(p[1] * meff);
  }
  return DEM_OK;
}
int oracle_unit_detect_vv(long n, const double* in, double* out) {
  for (long c = 0; c < n; c++) {
    const double* p = in + 8 * c;
    wdet(out + 8 * c, detect_vv(rv(p), p[3], rv(p + 4), p[7]));
  }
  return DEM_OK;
}
int oracle_unit_detect_ve(long n, const double* in, double* out) {
  for (long c = 0; c < n; c++) {
    const double* p = in + 11 * c;
    wdet(out + 8 * c, detect_ve(rv(p), p[3], rv(p + 4), rv(p + 7), p[10]));
  }
  return DEM_OK;
}
int oracle_unit_detect_ee(long n, const double* in, double* out) {
  for (long c = 0; c < n; c++) {
    const double* p = in + 14 * c;
    wdet(out + 8 * c, detect_ee(rv(p), rv(p + 3), p[6], rv(p + 7), rv(p + 10), p[13]));
  }
  return DEM_OK;
}
int oracle_unit_filter(int kind, long n, const double* in, double* out) {
  const int k = kind == 0 ? 9 : kind == 1 ? 12 : 15;
  for (long c = 0; c < n; c++) {
    const double* p = in + k * c;
    bool r;
    if (kind == 0)
      r = filter_vv(p[0], rv(p + 1), p[4], rv(p + 5), p[8]);
    else if (kind == 1)
      r = filter_ve(p[0], rv(p + 1), p[4], rv(p + 5), rv(p + 8), p[11]);
    else
      r = filter_ee(p[0], rv(p + 1), rv(p + 4), p[7], rv(p + 8), rv(p + 11), p[14]);
    out[c] = r ? 1.0 : 0.0;
  }
  return DEM_OK;
}
int oracle_unit_world_vertex(long n, const double* in, double* out) {
  for (long c = 0; c < n; c++) {
    const double* p = in + 11 * c;
    const Quat q = {p[3], p[4], p[5], p[6]};
    wv(out + 3 * c, rv(p) + rotate(q, p[7] * rv(p + 8)));  // compute_vertices
  }
  return DEM_OK;
}
// face: the vertex indices of the face; radius: the shape's Minkowski radius (scaled by hj as the list build does)
int oracle_unit_vertex_face(const int32_t* face, int nfv, int nv, double radius, long n, const double* in,
                            double* out) {
  const std::vector<int> f(face, face + nfv);
  std::vector<V3> va(nv);
  for (long c = 0; c < n; c++) {
    const double* p = in + (6 + 3 * nv) * c;
    for (int k = 0; k < nv; k++) va[k] = rv(p + 6 + 3 * k);
    const double rj = radius * p[5];
    double* o = out + 9 * c;
    o[0] = filter_vf(p[0], rv(p + 1), p[4], va, f, rj) ? 1.0 : 0.0;
    wdet(o + 1, detect_vf(rv(p + 1), p[4], va, f, rj));
  }
  return DEM_OK;
}
int oracle_unit_obb_intersect(long n, const double* in, double* out) {
  for (long c = 0; c < n; c++) out[c] = obb_intersect(robb(in + 30 * c), robb(in + 30 * c + 15)) ? 1.0 : 0.0;
  return DEM_OK;
}
int oracle_unit_compute_obb(long n, const double* in, double* out) {
  for (long c = 0; c < n; c++) {
    const double* p = in + 24 * c;
    OBBr b = compute_obb(robb(p), rv(p + 15), Quat{p[18], p[19], p[20], p[21]}, p[22]);
    obb_enlarge(b, p[23]);
    wobb(out + 15 * c, b);
  }
  return DEM_OK;
}
int oracle_unit_push_quaternion(long n, const double* in, double* out) {
  for (long c = 0; c < n; c++) {
    const double* p = in + 11 * c;
    const double delta_t = p[10];
    Quat Q = {p[0], p[1], p[2], p[3]};
    V3 w = rv(p + 4);
    push_quaternion(Q, w, rv(p + 7), delta_t, delta_t * 0.5);
    double* o = out + 7 * c;
    o[0] = Q.w;
    o[1] = Q.x;
    o[2] = Q.y;
    o[3] = Q.z;
    wv(o + 4, w);
  }
  return DEM_OK;
}
int oracle_unit_angular(long n, const double* in, double* out) {
  for (long c = 0; c < n; c++) {
    const double* p = in + 15 * c;
    const double half_delta_t = p[13] * 0.5;
    const V3 arot = angular_acceleration(Quat{p[0], p[1], p[2], p[3]}, rv(p + 4), rv(p + 7), rv(p + 10));
    V3 w = rv(p + 7);
    w.x += arot.x * half_delta_t;
    w.y += arot.y * half_delta_t;
    w.z += arot.z * half_delta_t;
    wv(out + 6 * c, arot);
    wv(out + 6 * c + 3, w);
  }
  return DEM_OK;
}
int oracle_unit_pair_order(long n, const uint64_t* keys, int32_t* out) {
  for (long c = 0; c < n; c++) {
    const uint64_t* k = keys + 12 * c;
    Inter a{}, b{};
    for (Inter* x : {&a, &b}) {
      const uint64_t* q = x == &a ? k : k + 6;
      x->oid = q[0];
      x->pid = q[1];
      x->type = (uint16_t)q[2];
      x->swap = (uint8_t)q[3];
      x->osub = (uint32_t)q[4];
      x->psub = (uint32_t)q[5];
    }
    out[2 * c] = key_less(a, b);
    out[2 * c + 1] = key_eq(a, b);
  }
  return DEM_OK;
}
int oracle_unit_surface(long n, const double* in, double* out) {
  for (long c = 0; c < n; c++) {
    const double* p = in + 11 * c;
    dem_surface ds{};
    ds.offset = p[0];
    for (int d = 0; d < 3; d++) {
      ds.normal[d] = p[1 + d];
      ds.center[d] = p[4 + d];
    }
    const Surface w = surface_from(&ds);
    double* o = out + 13 * c;
    o[0] = surface_filter(w, p[7], rv(p + 8)) ? 1.0 : 0.0;
    double dn = 0;
    V3 nn{}, cp{};
    const bool hit = surface_detect(w, p[7], rv(p + 8), dn, nn, cp);
    o[1] = hit ? 1.0 : 0.0;
    o[2] = dn;
    wv(o + 3, nn);
    wv(o + 6, cp);
    wv(o + 9, w.center);
    o[12] = 0.0;
  }
  return DEM_OK;
}
int oracle_unit_cylinder(long n, const double* in, double* out) {
  for (long c = 0; c < n; c++) {
    const double* p = in + 11 * c;
    dem_cylinder dc{};
    dc.radius = p[0];
    for (int d = 0; d < 3; d++) {
      dc.axis[d] = p[1 + d];
      dc.center[d] = p[4 + d];
    }
    const Cylinder w = cylinder_from(&dc);
    double* o = out + 13 * c;
    o[0] = cylinder_filter(w, p[7], rv(p + 8)) ? 1.0 : 0.0;
    double dn = 0;
    V3 nn{}, cp{};
    const bool hit = cylinder_detect(w, p[7], rv(p + 8), dn, nn, cp);
    o[1] = hit ? 1.0 : 0.0;
    o[2] = dn;
    wv(o + 3, nn);
    wv(o + 6, cp);
    wv(o + 9, w.center);
    o[12] = 0.0;
  }
  return DEM_OK;
}
const char* oracle_last_error(void* h) { return ((Oracle*)h)->err.c_str(); }
}
