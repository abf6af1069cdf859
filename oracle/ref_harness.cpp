/*
 * ref_harness.cpp -- exaDEM's own hot-path functions, compiled on the host.
 *
 * TEST INFRASTRUCTURE ONLY: the checker of the oracle (tests/ and the golden
 * vector generator), never the product.  Built by oracle/ref_build.py into
 * oracle/_ref/libexadem_ref.so from the exaDEM source tree, read in place; the
 * stand-in headers of oracle/ref_shim/ replace onika, exaNBody, MPI, yaml-cpp
 * and tinyexpr (see oracle/ref_shim/README.md for what they restate).
 *
 * Every entry point takes n cases as rows of doubles and writes n rows of
 * results.  The oracle exports the same entry points under the prefix
 * oracle_unit_ (oracle/dem_oracle.cpp), calling its own restatement, so a test
 * can compare the two bit for bit on the same inputs.  Row layouts are given
 * beside each function; a vector takes 3 doubles, a quaternion 4 (w, x, y, z).
 */
#include <cstdint>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include <exaDEM/forcefield/contact_force.hpp>   // contact_force_core, common_kernels
#include <exaDEM/forcefield/inner_bond_force.hpp>  // force_law_core of the inner bonds
#include <exaDEM/shape.hpp>                      // shape, get_vertex, minkowski
#include <exaDEM/shape_detection.hpp>            // filters and detection cores
#include <exaDEM/shape_reader.hpp>               // read_shp
#include <exaDEM/shape/basic_shape/cube.hpp>     // create_cube (add_cube)
#include <exaDEM/basic_types.hpp>                // compute_obb
#include <exaDEM/angular_acceleration.hpp>       // PushToAngularAccelerationFunctor
#include <exaDEM/push_to_quaternion.hpp>         // PushToQuaternionFunctor
#include <exaDEM/angular_velocity.hpp>           // PushToAngularVelocityFunctor
#include <exaDEM/interaction/interaction_pair.hpp>
#include <exaDEM/surface.hpp>
#include <exaDEM/cylinder.hpp>

using exanb::Quaternion;
using exanb::Vec3d;

namespace {
inline Vec3d V(const double* p) { return Vec3d(p[0], p[1], p[2]); }
inline Quaternion Q(const double* p) { return Quaternion{p[0], p[1], p[2], p[3]}; }
inline void put(double* o, const Vec3d& v) {
  o[0] = v.x;
  o[1] = v.y;
  o[2] = v.z;
}
inline void put_contact(double* o, const exaDEM::contact& c) {
  o[0] = c.is_contact ? 1.0 : 0.0;
  o[1] = c.dn;
  put(o + 2, c.normal);
  put(o + 5, c.position);
}
inline vec3r v3r(const double* p) { return vec3r(p[0], p[1], p[2]); }
inline void put_obb(double* o, const OBB& b) {
  const vec3r* parts[5] = {&b.center, &b.e1, &b.e2, &b.e3, &b.extent};
  for (int k = 0; k < 5; k++) {
    o[3 * k] = parts[k]->x;
    o[3 * k + 1] = parts[k]->y;
    o[3 * k + 2] = parts[k]->z;
  }
}
inline OBB get_obb(const double* p) {  // center, e1, e2, e3, extent
  OBB b;
  b.center = v3r(p);
  b.e1 = v3r(p + 3);
  b.e2 = v3r(p + 6);
  b.e3 = v3r(p + 9);
  b.extent = v3r(p + 12);
  return b;
}

std::vector<exaDEM::shape> g_shapes;  // shapes read by ref_read_shp, addressed by index
}  // namespace

extern "C" {

/* contact_force_core<Hooke, None|Cohesive|DMT> (contact_force.hpp:146-235) followed by
 * compute_moments (common_kernels.hpp:136-145) of the new force and moment.
 * law 0 none, 1 cohesive, 2 DMT.
 * in  (45): dn, n[3], dt, kn, kt, kr, mu, damp_rate, fc, dncut, gamma, meff, reff, ft[3], cp[3],
 *           pos_i[3], vel_i[3], f_i[3], mom_i[3], vrot_i[3], pos_j[3], vel_j[3], vrot_j[3]
 * out (12): f_i[3], ft[3], mom_i[3], torque_i[3] */
int ref_unit_contact_force_core(int law, long n, const double* in, double* out) {
  for (long c = 0; c < n; c++) {
    const double* p = in + 45 * c;
    double* o = out + 12 * c;
    exaDEM::ContactParams hkp;
    hkp.kn_ = p[5];
    hkp.kt_ = p[6];
    hkp.kr_ = p[7];
    hkp.mu_ = p[8];
    hkp.damp_rate_ = p[9];
    hkp.fc_ = p[10];
    hkp.dncut_ = p[11];
    hkp.gamma_ = p[12];
    Vec3d ft = V(p + 15), f_i = V(p + 27), mom_i = V(p + 30);
    const Vec3d nrm = V(p + 1), cp = V(p + 18), pos_i = V(p + 21);
    if (law == 0)
      exaDEM::contact_force_core<ContactLawType::Hooke, CohesiveLawType::None>(
          p[0], nrm, p[4], hkp, p[13], p[14], ft, cp, pos_i, V(p + 24), f_i, mom_i, V(p + 33), V(p + 36),
          V(p + 39), V(p + 42));
    else if (law == 1)
      exaDEM::contact_force_core<ContactLawType::Hooke, CohesiveLawType::Cohesive>(
          p[0], nrm, p[4], hkp, p[13], p[14], ft, cp, pos_i, V(p + 24), f_i, mom_i, V(p + 33), V(p + 36),
          V(p + 39), V(p + 42));
    else
      exaDEM::contact_force_core<ContactLawType::Hooke, CohesiveLawType::DMT>(
          p[0], nrm, p[4], hkp, p[13], p[14], ft, cp, pos_i, V(p + 24), f_i, mom_i, V(p + 33), V(p + 36),
          V(p + 39), V(p + 42));
    put(o, f_i);
    put(o + 3, ft);
    put(o + 6, mom_i);
    put(o + 9, exaDEM::compute_moments(cp, pos_i, f_i, mom_i));
  }
  return 0;
}

/* force_law_core (inner_bond_force.hpp:24-70) followed by compute_moments with a zero
 * moment on both particles and fn = f_i - ft (inner_bond.hpp:166-183).
 * in (35): dn, n[3], dn0, weight, dt, kn, kt, damp_rate, meff, tds[3], cp[3], pos_i[3],
 *          vel_i[3], vrot_i[3], pos_j[3], vel_j[3], vrot_j[3]
 * out (20): En, Et, tds[3], ft[3], f_i[3], torque_i[3], torque_j[3], fn[3] */
int ref_unit_bond_law(long n, const double* in, double* out) {
  for (long c = 0; c < n; c++) {
    const double* p = in + 35 * c;
    double* o = out + 20 * c;
    exaDEM::InnerBondParams ibp;
    ibp.kn_ = p[7];
    ibp.kt_ = p[8];
    ibp.damp_rate_ = p[9];
    double En = 0, Et = 0;
    Vec3d tds = V(p + 11), ft, f_i;
    const Vec3d cp = V(p + 14), pos_i = V(p + 17), pos_j = V(p + 26);
    exaDEM::force_law_core(p[0], V(p + 1), p[4], p[5], p[6], ibp, p[10], En, tds, Et, ft, cp, pos_i, V(p + 20),
                           f_i, V(p + 23), pos_j, V(p + 29), V(p + 32));
    o[0] = En;
    o[1] = Et;
    put(o + 2, tds);
    put(o + 5, ft);
    put(o + 8, f_i);
    put(o + 11, exaDEM::compute_moments(cp, pos_i, f_i, Vec3d{}));
    put(o + 14, exaDEM::compute_moments(cp, pos_j, -f_i, Vec3d{}));
    put(o + 17, f_i - ft);
  }
  return 0;
}

/* compute_damp and compute_effective_mass (common_kernels.hpp:27-31,86-90).
 * in (5): damp_rate, kn, mi, mj, unused.  out (2): meff, damp(damp_rate, kn, meff) */
int ref_unit_damping(long n, const double* in, double* out) {
  for (long c = 0; c < n; c++) {
    const double* p = in + 5 * c;
    const double meff = exaDEM::compute_effective_mass(p[2], p[3]);
    out[2 * c] = meff;
    out[2 * c + 1] = exaDEM::compute_damp(p[0], p[1], meff);
  }
  return 0;
}

/* detection_vertex_vertex_core (shape_detection_core.hpp:57-81): sphere-sphere and
 * polyhedron vertex-vertex detection.  in (8): pi[3], ri, pj[3], rj.
 * out (8): contact, dn, normal[3], position[3] */
int ref_unit_detect_vv(long n, const double* in, double* out) {
  for (long c = 0; c < n; c++) {
    const double* p = in + 8 * c;
    put_contact(out + 8 * c, exaDEM::detection_vertex_vertex_core(V(p), p[3], V(p + 4), p[7]));
  }
  return 0;
}

/* detection_vertex_edge_core (:122-148).  in (11): vi[3], ri, vf[3], vs[3], rj.  out (8) */
int ref_unit_detect_ve(long n, const double* in, double* out) {
  for (long c = 0; c < n; c++) {
    const double* p = in + 11 * c;
    put_contact(out + 8 * c, exaDEM::detection_vertex_edge_core(V(p), p[3], V(p + 4), V(p + 7), p[10]));
  }
  return 0;
}

/* detection_edge_edge_core (:521-566).  in (14): vfi[3], vsi[3], ri, vfj[3], vsj[3], rj.  out (8) */
int ref_unit_detect_ee(long n, const double* in, double* out) {
  for (long c = 0; c < n; c++) {
    const double* p = in + 14 * c;
    put_contact(out + 8 * c,
                exaDEM::detection_edge_edge_core(V(p), V(p + 3), p[6], V(p + 7), V(p + 10), p[13]));
  }
  return 0;
}

/* Verlet filters (:43-53, :83-101, :468-504).  kind 0 vertex-vertex
 * in (9): rV, vi[3], ri, vj[3], rj;  kind 1 vertex-edge in (12): rV, vi[3], ri, vf[3], vs[3], rj;
 * kind 2 edge-edge in (15): rV, vfi[3], vsi[3], ri, vfj[3], vsj[3], rj.  out (1): 1 or 0 */
int ref_unit_filter(int kind, long n, const double* in, double* out) {
  const int k = kind == 0 ? 9 : kind == 1 ? 12 : 15;
  for (long c = 0; c < n; c++) {
    const double* p = in + k * c;
    bool r;
    if (kind == 0)
      r = exaDEM::filter_vertex_vertex(p[0], V(p + 1), p[4], V(p + 5), p[8]);
    else if (kind == 1)
      r = exaDEM::filter_vertex_edge_core(p[0], V(p + 1), p[4], V(p + 5), V(p + 8), p[11]);
    else
      r = exaDEM::filter_edge_edge_core(p[0], V(p + 1), V(p + 4), p[7], V(p + 8), V(p + 11), p[14]);
    out[c] = r ? 1.0 : 0.0;
  }
  return 0;
}

/* Reads every shape of a .shp file with read_shp (shape_reader.hpp:36-111), as
 * read_shps does (:121-140), and keeps them; *first is the index of the first,
 * *count how many.  The shapes' arrays are read back with ref_shape_info /
 * ref_shape_arrays. */
int ref_read_shps(const char* path, int* first, int* count) {
  std::ifstream input(path);
  if (!input.is_open()) return -1;
  *first = (int)g_shapes.size();
  *count = 0;
  for (std::string line; std::getline(input, line);) {
    if (line == "<") {
      g_shapes.push_back(exaDEM::read_shp(input, false));
      (*count)++;
    }
  }
  return 0;
}
/* counts (4): nv, ne, nf, size of the face array (faces_[0] = nf, then per face its count and vertices) */
/* basic_shape::create_cube (add_cube): appends the cube to the shapes read so
 * far; *index is its index for ref_shape_info / ref_shape_arrays. */
int ref_create_cube(double length, double minkowski, int* index) {
  g_shapes.push_back(exaDEM::basic_shape::create_cube("cube", length, minkowski));
  *index = (int)g_shapes.size() - 1;
  return 0;
}

int ref_shape_info(int s, int64_t* counts) {
  const exaDEM::shape& sh = g_shapes[s];
  counts[0] = sh.get_number_of_vertices();
  counts[1] = sh.get_number_of_edges();
  counts[2] = sh.get_number_of_faces();
  counts[3] = (int64_t)sh.faces_.size();
  return 0;
}
/* vertices (3 nv), edges (2 ne), faces (counts[3]), scalars (5): radius, volume, I/m[3],
 * obb (15): the shape OBB built by read_shp (build_obb_from_shape), name (64 bytes) */
int ref_shape_arrays(int s, double* vertices, int32_t* edges, int32_t* faces, double* scalars, double* obb,
                     char* name) {
  const exaDEM::shape& sh = g_shapes[s];
  for (int i = 0; i < sh.get_number_of_vertices(); i++) put(vertices + 3 * i, sh.get_vertex(i));
  for (size_t i = 0; i < sh.edges_.size(); i++) edges[i] = sh.edges_[i];
  for (size_t i = 0; i < sh.faces_.size(); i++) faces[i] = sh.faces_[i];
  scalars[0] = sh.radius_;
  scalars[1] = sh.volume_;
  put(scalars + 2, sh.inertia_on_mass_);
  put_obb(obb, sh.obb_);
  std::strncpy(name, sh.name_.c_str(), 63);
  name[63] = 0;
  return 0;
}

/* Derived shape quantities set_fields uses (set_fields.cu:296-300): compute_max_rcut
 * (shape.hpp:479-489), get_volume(h) (:145-148) and get_Im(h) (:163-164).
 * out (5): max_rcut, volume(h), I/m(h)[3] */
int ref_shape_derived(int s, double h, double* out) {
  const exaDEM::shape& sh = g_shapes[s];
  out[0] = sh.compute_max_rcut();
  out[1] = sh.get_volume(h);
  put(out + 2, sh.get_Im(h));
  return 0;
}

/* get_face_area(i, h) (shape.hpp:359-362) of every face, from compute_face_areas
 * (shape.hpp:674-697) run by read_shp.  out (nf) */
int ref_shape_face_areas(int s, double h, double* out) {
  const exaDEM::shape& sh = g_shapes[s];
  for (int f = 0; f < sh.get_number_of_faces(); f++) out[f] = sh.get_face_area(f, h);
  return 0;
}

/* shape::get_vertex (shape.hpp:245-262): p + Q * (h * v0).
 * in (11): p[3], Q[4], h, v0[3] (the shape's vertex is replaced by v0).  out (3) */
int ref_unit_world_vertex(long n, const double* in, double* out) {
  exaDEM::shape sh;
  sh.add_vertex(Vec3d(0, 0, 0));
  for (long c = 0; c < n; c++) {
    const double* p = in + 11 * c;
    sh.vertices_[0] = V(p + 8);
    put(out + 3 * c, sh.get_vertex(0, V(p), p[7], Q(p + 3)));
  }
  return 0;
}

/* Vertex-face filter and detection against face j of shape s
 * (filter_vertex_face :246-309, detection_vertex_face_core :398-466), the shape's
 * Minkowski radius scaled by hj.  in (6 + 3 nv): rV, vi[3], ri, hj, then the world
 * vertices of shape s.  out (9): filter, then the detection's contact, dn, normal, position */
int ref_unit_vertex_face(int s, int j, long n, const double* in, double* out) {
  const exaDEM::shape& sh = g_shapes[s];
  const int nv = sh.get_number_of_vertices();
  std::vector<Vec3d> va(nv);
  for (long c = 0; c < n; c++) {
    const double* p = in + (6 + 3 * nv) * c;
    for (int k = 0; k < nv; k++) va[k] = V(p + 6 + 3 * k);
    double* o = out + 9 * c;
    const double ri = p[4];
    o[0] = exaDEM::filter_vertex_face(p[0], V(p + 1), ri, va, p[5], j, &sh) ? 1.0 : 0.0;
    put_contact(o + 1, exaDEM::detection_vertex_face_core(V(p + 1), ri, va, p[5], j, &sh));
  }
  return 0;
}

/* OBB::intersect (type/OBB.hpp:90-220) of a against b.  in (30): a, b as center, e1, e2, e3, extent.
 * out (1) */
int ref_unit_obb_intersect(long n, const double* in, double* out) {
  for (long c = 0; c < n; c++) {
    const double* p = in + 30 * c;
    OBB a = get_obb(p), b = get_obb(p + 15);
    out[c] = a.intersect(b) ? 1.0 : 0.0;
  }
  return 0;
}

/* compute_obb (basic_types.hpp:37-48) then OBB::enlarge (type/OBB.hpp:66-70).
 * in (24): obb[15], pos[3], Q[4], homothety, enlarge.  out (15) */
int ref_unit_compute_obb(long n, const double* in, double* out) {
  for (long c = 0; c < n; c++) {
    const double* p = in + 24 * c;
    OBB b = exaDEM::compute_obb(get_obb(p), V(p + 15), Q(p + 18), p[22]);
    b.enlarge(p[23]);
    put_obb(out + 15 * c, b);
  }
  return 0;
}

/* Rotation half of combined_compute_prolog: PushToQuaternionFunctor (push_to_quaternion.hpp:26-38).
 * in (11): Q[4], vrot[3], arot[3], dt.  out (7): Q[4], vrot[3] */
int ref_unit_push_quaternion(long n, const double* in, double* out) {
  for (long c = 0; c < n; c++) {
    const double* p = in + 11 * c;
    const double dt = p[10];
    exaDEM::PushToQuaternionFunctor f{dt, 0.5 * dt, 0.5 * dt * dt};
    Quaternion q = Q(p);
    Vec3d vrot = V(p + 4);
    f(q, vrot, V(p + 7));
    double* o = out + 7 * c;
    o[0] = q.w;
    o[1] = q.x;
    o[2] = q.y;
    o[3] = q.z;
    put(o + 4, vrot);
  }
  return 0;
}

/* Rotation half of combined_compute_epilog: PushToAngularAccelerationFunctor
 * (angular_acceleration.hpp:27-43) then PushToAngularVelocityFunctor (angular_velocity.hpp).
 * in (15): Q[4], mom[3], vrot[3], inertia[3], dt, unused.  out (6): arot[3], vrot[3] */
int ref_unit_angular(long n, const double* in, double* out) {
  for (long c = 0; c < n; c++) {
    const double* p = in + 15 * c;
    const double dt = p[13];
    Vec3d arot(0, 0, 0), vrot = V(p + 7);
    exaDEM::PushToAngularAccelerationFunctor{}(Q(p), V(p + 4), vrot, arot, V(p + 10));
    exaDEM::PushToAngularVelocityFunctor{0.5 * dt}(vrot, arot);
    put(out + 6 * c, arot);
    put(out + 6 * c + 3, vrot);
  }
  return 0;
}

/* InteractionPair::operator< and operator== (interaction_pair.hpp:186-249) on keys
 * (owner id, partner id, type, swap, owner sub, partner sub), a against b.
 * keys: 12 u64 per case.  out: 2 per case, (a < b, a == b) */
int ref_unit_pair_order(long n, const uint64_t* keys, int32_t* out) {
  auto make = [](const uint64_t* k) {
    exaDEM::InteractionPair ip{};
    ip.type_ = (uint16_t)k[2];
    ip.swap_ = (uint8_t)k[3];
    exaDEM::ParticleSubLocation own{}, par{};
    own.id_ = k[0];
    own.sub_ = (uint32_t)k[4];
    par.id_ = k[1];
    par.sub_ = (uint32_t)k[5];
    ip.owner() = own;
    ip.partner() = par;
    return ip;
  };
  for (long c = 0; c < n; c++) {
    const exaDEM::InteractionPair a = make(keys + 12 * c), b = make(keys + 12 * c + 6);
    out[2 * c] = a < b;
    out[2 * c + 1] = a == b;
  }
  return 0;
}

/* Surface::initialize (stationary), filter and detector (surface.hpp:145-180,320-350).
 * in (11): offset, normal[3], center[3] (all zero: not given), rcut, p[3].
 * out (13): filter, contact, dn, normal[3], position[3], center[3] (after initialize) */
int ref_unit_surface(long n, const double* in, double* out) {
  exaDEM::Driver_params motion;
  for (long c = 0; c < n; c++) {
    const double* p = in + 11 * c;
    exaDEM::Surface s;
    s.motion_type_ = exaDEM::MotionType::STATIONARY;
    s.fields_.offset_ = p[0];
    s.fields_.normal_ = V(p + 1);
    // the YAML decoder's default centre when none is given and the surface does not spin (surface.hpp:73-84)
    const Vec3d c0 = V(p + 4);
    s.fields_.center_ = (c0 == Vec3d(0, 0, 0)) ? s.fields_.offset_ * s.fields_.normal_ : c0;
    s.initialize(motion);
    double* o = out + 13 * c;
    o[0] = s.filter(p[7], V(p + 8)) ? 1.0 : 0.0;
    auto [hit, dn, nrm, pos] = s.detector(p[7], V(p + 8));
    o[1] = hit ? 1.0 : 0.0;
    o[2] = dn;
    put(o + 3, nrm);
    put(o + 6, pos);
    put(o + 9, s.fields_.center_);
    o[12] = 0.0;
  }
  return 0;
}

/* Cylinder::initialize (stationary), filter and detector (cylinder.hpp:94-105,225-277).
 * in (11): radius, axis[3], center[3], rcut, p[3].  out (13): as ref_unit_surface */
int ref_unit_cylinder(long n, const double* in, double* out) {
  exaDEM::Driver_params motion;
  for (long c = 0; c < n; c++) {
    const double* p = in + 11 * c;
    exaDEM::Cylinder s;
    s.motion_type_ = exaDEM::MotionType::STATIONARY;
    s.fields_.radius_ = p[0];
    s.fields_.axis_ = V(p + 1);
    s.fields_.center_ = V(p + 4);
    s.initialize(motion);
    double* o = out + 13 * c;
    o[0] = s.filter(p[7], V(p + 8)) ? 1.0 : 0.0;
    auto [hit, dn, nrm, pos] = s.detector(p[7], V(p + 8));
    o[1] = hit ? 1.0 : 0.0;
    o[2] = dn;
    put(o + 3, nrm);
    put(o + 6, pos);
    put(o + 9, s.fields_.center_);
    o[12] = 0.0;
  }
  return 0;
}

}  // extern "C"
