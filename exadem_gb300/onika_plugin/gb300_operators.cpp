// gb300_operators.cpp -- onika operator shims that run exaDEM's per-timestep
// hot path on libexadem_gb300 (GB300), registered under exaDEM's own operator
// names so that an unchanged .msp deck uses them.
//
// Build it into a plugin of an exaDEM build (with onika and exaNBody), link it
// with libexadem_gb300.so, and load it after exaDEM's own plugins: the
// factory then resolves these names to the versions below.  Each operator
// keeps the slots of the exaDEM operator it replaces (the file cited beside
// it), passes them to the library's parameters, calls the entry point of
// include/dem_hotpath.h, and writes back to the grid the fields that operator
// writes in exaDEM (gb300_bridge.hpp).  The list of interactions and its
// friction/moment history stay in the library between operators, in exaDEM
// they stay in the grid's extra storage.
#include <onika/scg/operator.h>
#include <onika/scg/operator_factory.h>
#include <onika/scg/operator_slot.h>
#include <exanb/core/domain.h>
#include <exanb/core/grid.h>
#include <exanb/core/make_grid_variant_operator.h>

#include <exaDEM/cylinder.hpp>
#include <exaDEM/forcefield/contact_parameters.hpp>
#include <exaDEM/forcefield/inner_bond_parameters.hpp>
#include <exaDEM/forcefield/multimat_parameters.hpp>
#include <exaDEM/surface.hpp>

#include "gb300_bridge.hpp"

namespace exaDEM {
using namespace exanb;
using gb300::Bridge;

namespace gb300_detail {
inline dem_contact_params to_abi(const ContactParams& c) {
  dem_contact_params p{};
  p.kn = c.kn_;
  p.kt = c.kt_;
  p.kr = c.kr_;
  p.mu = c.mu_;
  p.damp_rate = c.damp_rate_;
  p.fc = c.fc_;
  p.dncut = c.dncut_;
  p.gamma = c.gamma_;
  return p;
}
inline void set_domain(dem_params& p, const Domain& d) {
  const auto b = d.bounds();
  p.bounds_lo[0] = b.bmin.x, p.bounds_lo[1] = b.bmin.y, p.bounds_lo[2] = b.bmin.z;
  p.bounds_hi[0] = b.bmax.x, p.bounds_hi[1] = b.bmax.y, p.bounds_hi[2] = b.bmax.z;
  p.periodic[0] = d.periodic_boundary_x(), p.periodic[1] = d.periodic_boundary_y();
  p.periodic[2] = d.periodic_boundary_z();
  p.cell_size = d.cell_size();
}
// Parameters known so far to this grid's bridge, with `edit` applied, then the context (re)configured.
template <class GridT, class F>
inline Bridge& configured(GridT& grid, F&& edit) {
  Bridge& b = gb300::bridge_for(grid);
  if (!b.have_prm) {
    b.prm.symetric = 1;
    b.prm.gravity[2] = -9.807;  // gravity_force's default
    b.prm.fused_step = 1;
    b.prm.fp32_broad_phase = 1;
    b.prm.fp32_contact_screen = 1;
  }
  dem_params p = b.prm;
  edit(p);
  b.configure(p);
  b.pull(grid);
  return b;
}
// inner_bond_params (multimat_inner_bond.cpp:104-200) as the library's table:
// one group (a default_config) becomes the one set for every pair
inline void set_inner_bond_params(Bridge& b, const MultiMatParamsT<InnerBondParams>& m) {
  const int ng = m.number_of_groups_;
  std::vector<dem_inner_bond_params> t;
  for (int i = 0; i < ng * ng; i++) {
    const InnerBondParams& q = m.multimat_cp_[i];
    dem_inner_bond_params p{};
    p.kn = q.kn_;
    p.kt = q.kt_;
    p.damp_rate = q.damp_rate_;
    p.mode = q.mode_ == RuptureMode::EnergySeparateMode         ? DEM_RUPTURE_ENERGY_SEPARATE
             : q.mode_ == RuptureMode::StressEnergySeparateMode ? DEM_RUPTURE_STRESS_ENERGY_SEPARATE
                                                                : DEM_RUPTURE_ENERGY_MIXED;
    p.crit1 = q.crit1_;
    p.crit2 = q.crit2_;
    t.push_back(p);
  }
  if (t.empty()) gb300::check(DEM_ERR_INVALID_ARG, nullptr, "inner_bond_params: no parameters");
  gb300::check(dem_set_inner_bond_params(b.ctx, ng <= 1 ? 0 : ng, t.data()), b.ctx, "inner_bond_params");
}
}  // namespace gb300_detail

// chunk_neighbors_contact (src/grid/chunk_neighbors_contact.cpp:118-121) and
// classify_interactions (src/interaction/classify_interactions.cpp:140-143): the
// library's neighbour build does both, so these names have nothing left to do.
template <typename GridT>
class GB300NoOp : public OperatorNode {
  ADD_SLOT(GridT, grid, INPUT_OUTPUT, REQUIRED);

 public:
  inline void execute() final {}
};

// nbh_sphere (src/sphere/nbh_sphere.cu:313-316) / nbh_polyhedron (src/polyhedron/nbh_polyhedron.cpp:388-391):
// cell grid, Verlet list with history carry-over, interaction types, classification.
template <typename GridT>
class GB300Neighbors : public OperatorNode {
  ADD_SLOT(GridT, grid, INPUT_OUTPUT, REQUIRED);
  ADD_SLOT(Domain, domain, INPUT, REQUIRED);
  ADD_SLOT(double, rcut_inc, INPUT, REQUIRED, DocString{"Verlet skin"});
  ADD_SLOT(bool, symetric, INPUT, true);

 public:
  inline void execute() final {
    if (!*symetric) gb300::check(DEM_ERR_UNSUPPORTED, nullptr, "nbh: symetric: false");
    Bridge& b = gb300_detail::configured(*grid, [&](dem_params& p) {
      gb300_detail::set_domain(p, *domain);
      p.rcut_inc = *rcut_inc;
    });
    gb300::check(dem_update_particle_neighbors(b.ctx), b.ctx, "nbh");
  }
};

// reset_force_moment (src/numericalscheme/reset_force_moment.cu:75-78)
template <typename GridT>
class GB300ResetForceMoment : public OperatorNode {
  ADD_SLOT(GridT, grid, INPUT_OUTPUT, REQUIRED);

 public:
  inline void execute() final {
    Bridge& b = gb300_detail::configured(*grid, [](dem_params&) {});
    gb300::check(dem_reset_force_moment(b.ctx), b.ctx, "reset_force_moment");
    b.push(*grid, {gb300::FX, gb300::MX});
  }
};

// gravity_force (src/forcefield/gravity_force.cu:90-92)
template <typename GridT>
class GB300Gravity : public OperatorNode {
  ADD_SLOT(GridT, grid, INPUT_OUTPUT, REQUIRED);
  ADD_SLOT(Vec3d, gravity, INPUT, Vec3d(0.0, 0.0, -9.807));

 public:
  inline void execute() final {
    Bridge& b = gb300_detail::configured(*grid, [&](dem_params& p) {
      p.gravity[0] = gravity->x, p.gravity[1] = gravity->y, p.gravity[2] = gravity->z;
    });
    gb300::check(dem_gravity_force(b.ctx), b.ctx, "gravity_force");
    b.push(*grid, {gb300::FX});
  }
};

// contact_sphere / contact_singlemat_sphere_hooke{,_none,_cohesive,_dmt}
// (src/sphere/contact_force_sphere.cu.in:355-358) and contact_polyhedron /
// contact_singlemat_polyhedron_hooke{,_none,_cohesive,_dmt} (contact_force_polyhedron.cu.in).
template <typename GridT, int Law, bool Polyhedra>
class GB300Contact : public OperatorNode {
  ADD_SLOT(GridT, grid, INPUT_OUTPUT, REQUIRED);
  ADD_SLOT(ContactParams, config, INPUT, REQUIRED);
  ADD_SLOT(ContactParams, config_driver, INPUT, OPTIONAL);
  ADD_SLOT(double, dt, INPUT, REQUIRED);
  ADD_SLOT(bool, symetric, INPUT, REQUIRED);

 public:
  inline void execute() final {
    if (!*symetric) gb300::check(DEM_ERR_UNSUPPORTED, nullptr, "contact: symetric: false");
    Bridge& b = gb300_detail::configured(*grid, [&](dem_params& p) {
      p.law = Law;
      p.dt = *dt;
      p.config = gb300_detail::to_abi(*config);
      p.config_driver = gb300_detail::to_abi(config_driver.has_value() ? *config_driver : *config);
    });
    gb300::check(Polyhedra ? dem_contact_polyhedron(b.ctx) : dem_contact_sphere(b.ctx), b.ctx, "contact");
    b.push(*grid, {gb300::FX, gb300::MX});
  }
};
template <class G> using GB300ContactSphereNone = GB300Contact<G, DEM_LAW_HOOKE_NONE, false>;
template <class G> using GB300ContactSphereCohesive = GB300Contact<G, DEM_LAW_HOOKE_COHESIVE, false>;
template <class G> using GB300ContactSphereDMT = GB300Contact<G, DEM_LAW_HOOKE_DMT, false>;
template <class G> using GB300ContactPolyNone = GB300Contact<G, DEM_LAW_HOOKE_NONE, true>;
template <class G> using GB300ContactPolyCohesive = GB300Contact<G, DEM_LAW_HOOKE_COHESIVE, true>;
template <class G> using GB300ContactPolyDMT = GB300Contact<G, DEM_LAW_HOOKE_DMT, true>;

// force_to_accel (src/numericalscheme/force_to_accel.cu:56-58)
template <typename GridT>
class GB300ForceToAccel : public OperatorNode {
  ADD_SLOT(GridT, grid, INPUT_OUTPUT, REQUIRED);

 public:
  inline void execute() final {
    Bridge& b = gb300_detail::configured(*grid, [](dem_params&) {});
    gb300::check(dem_force_to_accel(b.ctx), b.ctx, "force_to_accel");
    b.push(*grid, {gb300::FX});
  }
};

// combined_compute_prolog (src/numericalscheme/combined_compute_prolog.cu:123-126)
template <typename GridT>
class GB300Prolog : public OperatorNode {
  ADD_SLOT(GridT, grid, INPUT_OUTPUT, REQUIRED);
  ADD_SLOT(Domain, domain, INPUT, REQUIRED);
  ADD_SLOT(double, dt, INPUT, REQUIRED);

 public:
  inline void execute() final {
    Bridge& b = gb300_detail::configured(*grid, [&](dem_params& p) {
      gb300_detail::set_domain(p, *domain);
      p.dt = *dt;
    });
    gb300::check(dem_combined_compute_prolog(b.ctx), b.ctx, "combined_compute_prolog");
    b.push(*grid, {gb300::RX, gb300::VX, gb300::QW, gb300::WX});
  }
};

// combined_compute_epilog (src/numericalscheme/combined_compute_epilog.cu:120-123)
template <typename GridT>
class GB300Epilog : public OperatorNode {
  ADD_SLOT(GridT, grid, INPUT_OUTPUT, REQUIRED);
  ADD_SLOT(double, dt, INPUT, REQUIRED);

 public:
  inline void execute() final {
    Bridge& b = gb300_detail::configured(*grid, [&](dem_params& p) { p.dt = *dt; });
    gb300::check(dem_combined_compute_epilog(b.ctx), b.ctx, "combined_compute_epilog");
    b.push(*grid, {gb300::VX, gb300::WX, gb300::AX});
  }
};

// vertex_displ_over (src/polyhedron/vertex_displ_over.cu:146-149): the rotation-aware
// rebuild trigger of polyhedra; particle_displ_over (exaNBody) for spheres.
template <typename GridT, bool Polyhedra>
class GB300DisplOver : public OperatorNode {
  ADD_SLOT(GridT, grid, INPUT, REQUIRED);
  ADD_SLOT(bool, result, OUTPUT);

 public:
  inline void execute() final {
    Bridge& b = gb300_detail::configured(*grid, [](dem_params&) {});
    int over = 0;
    gb300::check(Polyhedra ? dem_vertex_displ_over(b.ctx, &over) : dem_particle_displ_over(b.ctx, &over), b.ctx,
                 "displ_over");
    *result = over != 0;
  }
};
template <class G> using GB300SphereDispl = GB300DisplOver<G, false>;
template <class G> using GB300VertexDispl = GB300DisplOver<G, true>;

// stick_polyhedra (src/polyhedron/stick_polyhedra.cpp:365-369): bonds between the
// touching faces of the particles of one cluster (the grid's cluster field).
template <typename GridT>
class GB300StickPolyhedra : public OperatorNode {
  ADD_SLOT(GridT, grid, INPUT_OUTPUT, REQUIRED);
  ADD_SLOT(double, sticking_threshold, INPUT, REQUIRED);
  ADD_SLOT(MultiMatParamsT<InnerBondParams>, multimat_ibp, INPUT, REQUIRED);

 public:
  inline void execute() final {
    Bridge& b = gb300_detail::configured(*grid, [](dem_params&) {});
    gb300_detail::set_inner_bond_params(b, *multimat_ibp);
    std::vector<uint64_t> ids;
    std::vector<double> cluster;
    auto cells = grid->cells();
    for (size_t c = 0; c < grid->number_of_cells(); c++) {
      if (grid->is_ghost_cell(c)) continue;
      for (size_t p = 0; p < cells[c].size(); p++) {
        ids.push_back(cells[c][field::id][p]);
        cluster.push_back(cells[c][field::cluster][p]);
      }
    }
    uint64_t nb = 0;
    gb300::check(dem_stick_polyhedra(b.ctx, ids.data(), cluster.data(), ids.size(), *sticking_threshold, &nb), b.ctx,
                 "stick_polyhedra");
  }
};

// inner_bond_polyhedron (src/polyhedron/inner_bond_force.cu:138-141)
template <typename GridT>
class GB300InnerBond : public OperatorNode {
  ADD_SLOT(GridT, grid, INPUT_OUTPUT, REQUIRED);
  ADD_SLOT(MultiMatParamsT<InnerBondParams>, multimat_ibp, INPUT, REQUIRED);
  ADD_SLOT(double, dt, INPUT, REQUIRED);

 public:
  inline void execute() final {
    Bridge& b = gb300_detail::configured(*grid, [&](dem_params& p) { p.dt = *dt; });
    gb300_detail::set_inner_bond_params(b, *multimat_ibp);
    gb300::check(dem_inner_bond_polyhedron(b.ctx), b.ctx, "inner_bond_polyhedron");
    b.push(*grid, {gb300::FX, gb300::MX});
  }
};

// apply_interface_fracture_criterion (src/interaction/apply_interface_fracture_criterion.cu:92-95);
// the library applies broken_interface_friction_updater in the same pass.
template <typename GridT>
class GB300FractureCriterion : public OperatorNode {
  ADD_SLOT(GridT, grid, INPUT, REQUIRED);
  ADD_SLOT(bool, result, OUTPUT);
  ADD_SLOT(bool, display, INPUT, false);

 public:
  inline void execute() final {
    Bridge& b = gb300_detail::configured(*grid, [](dem_params&) {});
    uint64_t broken = 0;
    gb300::check(dem_apply_interface_fracture_criterion(b.ctx, &broken), b.ctx, "apply_interface_fracture_criterion");
    if (*display && broken > 0)
      lout << broken << (broken == 1 ? " interface has been broken." : " interfaces have been broken.") << std::endl;
    *result = broken > 0;
  }
};

// register_surface / register_cylinder (src/driver/drivers.hpp:291-320), stationary drivers.
template <typename GridT>
class GB300RegisterSurface : public OperatorNode {
  ADD_SLOT(GridT, grid, INPUT_OUTPUT, REQUIRED);
  ADD_SLOT(SurfaceFields, state, INPUT, REQUIRED);

 public:
  inline void execute() final {
    Bridge& b = gb300_detail::configured(*grid, [](dem_params&) {});
    dem_surface s{};
    s.offset = state->offset_;
    s.normal[0] = state->normal_.x, s.normal[1] = state->normal_.y, s.normal[2] = state->normal_.z;
    s.center[0] = state->center_.x, s.center[1] = state->center_.y, s.center[2] = state->center_.z;
    s.vel[0] = state->vel_.x, s.vel[1] = state->vel_.y, s.vel[2] = state->vel_.z;
    s.vrot[0] = state->vrot_.x, s.vrot[1] = state->vrot_.y, s.vrot[2] = state->vrot_.z;
    gb300::check(dem_register_surface(b.ctx, &s), b.ctx, "register_surface");
  }
};
template <typename GridT>
class GB300RegisterCylinder : public OperatorNode {
  ADD_SLOT(GridT, grid, INPUT_OUTPUT, REQUIRED);
  ADD_SLOT(CylinderFields, state, INPUT, REQUIRED);

 public:
  inline void execute() final {
    Bridge& b = gb300_detail::configured(*grid, [](dem_params&) {});
    dem_cylinder c{};
    c.radius = state->radius_;
    c.axis[0] = state->axis_.x, c.axis[1] = state->axis_.y, c.axis[2] = state->axis_.z;
    c.center[0] = state->center_.x, c.center[1] = state->center_.y, c.center[2] = state->center_.z;
    c.vel[0] = state->vel_.x, c.vel[1] = state->vel_.y, c.vel[2] = state->vel_.z;
    c.vrot[0] = state->vrot_.x, c.vrot[1] = state->vrot_.y, c.vrot[2] = state->vrot_.z;
    gb300::check(dem_register_cylinder(b.ctx, &c), b.ctx, "register_cylinder");
  }
};

// === register factories ===
ONIKA_AUTORUN_INIT(gb300_operators) {
  auto* f = OperatorNodeFactory::instance();
  f->register_factory("chunk_neighbors_contact", make_grid_variant_operator<GB300NoOp>);
  f->register_factory("classify_interactions", make_grid_variant_operator<GB300NoOp>);
  f->register_factory("nbh_sphere", make_grid_variant_operator<GB300Neighbors>);
  f->register_factory("nbh_polyhedron", make_grid_variant_operator<GB300Neighbors>);
  f->register_factory("reset_force_moment", make_grid_variant_operator<GB300ResetForceMoment>);
  f->register_factory("gravity_force", make_grid_variant_operator<GB300Gravity>);
  f->register_factory("contact_sphere", make_grid_variant_operator<GB300ContactSphereNone>);
  f->register_factory("contact_singlemat_sphere_hooke", make_grid_variant_operator<GB300ContactSphereNone>);
  f->register_factory("contact_singlemat_sphere_hooke_none", make_grid_variant_operator<GB300ContactSphereNone>);
  f->register_factory("contact_singlemat_sphere_hooke_cohesive",
                      make_grid_variant_operator<GB300ContactSphereCohesive>);
  f->register_factory("contact_singlemat_sphere_hooke_dmt", make_grid_variant_operator<GB300ContactSphereDMT>);
  f->register_factory("contact_polyhedron", make_grid_variant_operator<GB300ContactPolyNone>);
  f->register_factory("contact_singlemat_polyhedron_hooke", make_grid_variant_operator<GB300ContactPolyNone>);
  f->register_factory("contact_singlemat_polyhedron_hooke_none", make_grid_variant_operator<GB300ContactPolyNone>);
  f->register_factory("contact_singlemat_polyhedron_hooke_cohesive",
                      make_grid_variant_operator<GB300ContactPolyCohesive>);
  f->register_factory("contact_singlemat_polyhedron_hooke_dmt", make_grid_variant_operator<GB300ContactPolyDMT>);
  f->register_factory("force_to_accel", make_grid_variant_operator<GB300ForceToAccel>);
  f->register_factory("combined_compute_prolog", make_grid_variant_operator<GB300Prolog>);
  f->register_factory("combined_compute_epilog", make_grid_variant_operator<GB300Epilog>);
  f->register_factory("particle_displ_over", make_grid_variant_operator<GB300SphereDispl>);
  f->register_factory("vertex_displ_over", make_grid_variant_operator<GB300VertexDispl>);
  f->register_factory("stick_polyhedra", make_grid_variant_operator<GB300StickPolyhedra>);
  f->register_factory("inner_bond_polyhedron", make_grid_variant_operator<GB300InnerBond>);
  f->register_factory("apply_interface_fracture_criterion", make_grid_variant_operator<GB300FractureCriterion>);
  // done by the criterion pass, the neighbour build and the bond list of the library
  f->register_factory("broken_interface_friction_updater", make_grid_variant_operator<GB300NoOp>);
  f->register_factory("update_interfaces", make_grid_variant_operator<GB300NoOp>);
  f->register_factory("update_persistent_interactions", make_grid_variant_operator<GB300NoOp>);
  f->register_factory("register_surface", make_grid_variant_operator<GB300RegisterSurface>);
  f->register_factory("register_cylinder", make_grid_variant_operator<GB300RegisterCylinder>);
}
}  // namespace exaDEM
