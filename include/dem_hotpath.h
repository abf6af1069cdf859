/*
 * dem_hotpath.h -- C ABI of the GB300-native exaDEM per-timestep hot path.
 *
 * Every entry point replaces one exaDEM / exaNBody operator (or a fixed
 * sequence of them) of the default Verlet deck.  The reference interface each
 * one stands in for is cited beside it (paths are relative to the exaDEM
 * source tree).  The library owns its device memory; callers hand in and read
 * back host (or device) arrays through plain pointers and sizes.
 *
 * Conventions
 *   - every function returns an int status: DEM_OK (0) or a DEM_ERR_* code;
 *     dem_last_error() returns a one-line description of the last failure.
 *     (The reference prints and exits through color_log::error, e.g.
 *     src/interaction/include/exaDEM/interaction/placeholder_interaction.hpp:188-193.)
 *   - one dem_ctx is one simulated system (or one batch of systems); a ctx is
 *     not thread-safe; all work is queued on the ctx's own CUDA stream.
 *   - all particle state is FP64 structure-of-arrays, ids are uint64,
 *     type/group are uint32 (include/exaDEM/fields.h:34-54).
 */
#ifndef DEM_HOTPATH_H
#define DEM_HOTPATH_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define DEM_OK 0
#define DEM_ERR_INVALID_ARG 1 /* bad pointer, size or parameter            */
#define DEM_ERR_CUDA 2        /* a CUDA runtime call failed                */
#define DEM_ERR_OOM 3         /* device allocation failed                  */
#define DEM_ERR_UNSUPPORTED 4 /* feature outside the implemented path      */
#define DEM_ERR_OVERFLOW 5    /* a fixed-capacity device buffer overflowed */
#define DEM_ERR_TIMEOUT 6     /* a bounded device wait gave up             */
#define DEM_ERR_STATE 7       /* call order violated (e.g. no particles)   */
#define DEM_ERR_NO_DEVICE 8   /* no CUDA device visible                    */

/* ---- interaction type ids (src/interaction/include/exaDEM/interaction/interaction_enum.hpp:24-57) */
#define DEM_ITYPE_VERTEX_VERTEX 0
#define DEM_ITYPE_VERTEX_EDGE 1
#define DEM_ITYPE_VERTEX_FACE 2
#define DEM_ITYPE_EDGE_EDGE 3
#define DEM_ITYPE_VERTEX_CYLINDER 4
#define DEM_ITYPE_VERTEX_SURFACE 5
#define DEM_ITYPE_VERTEX_MESH_VERTEX 7 /* VertexRshapeDriverVertex */
#define DEM_ITYPE_VERTEX_MESH_EDGE 8   /* VertexRshapeDriverEdge   */
#define DEM_ITYPE_VERTEX_MESH_FACE 9   /* VertexRshapeDriverFace   */
#define DEM_ITYPE_EDGE_MESH_EDGE 10    /* EdgeRshapeDriverEdge     */
#define DEM_ITYPE_MESH_VERTEX_EDGE 11  /* EdgeRshapeDriverVertex: particle edge, mesh vertex */
#define DEM_ITYPE_MESH_VERTEX_FACE 12  /* FaceRshapeDriverVertex: particle face, mesh vertex */

/* ---- contact law parameters -------------------------------------------
 * Mirrors ContactParams {dncut, kn, kt, kr, fc, mu, damp_rate}
 * (src/forcefield/include/exaDEM/forcefield/contact_parameters.hpp:32-41,138-190).
 * dncut == 0 and fc == 0 means "no cohesion".                             */
typedef struct dem_contact_params {
  double kn, kt, kr, mu, damp_rate;
  double fc, dncut;
  double gamma; /* adhesion energy per unit surface of the DMT law (ContactParams::gamma_) */
} dem_contact_params;

/* Contact law variant, as in the operator names contact_singlemat_sphere_hooke_{none,cohesive,dmt}
 * (src/sphere/CMakeLists.txt:63-110, contact_force.hpp:26-98).  DMT adds, in
 * contact and for gamma > 0, the attraction -2 pi reff gamma n to the Hooke
 * force (apply_dmt_force, contact_force.hpp:115-127).                     */
#define DEM_LAW_HOOKE_NONE 0
#define DEM_LAW_HOOKE_COHESIVE 1
#define DEM_LAW_HOOKE_DMT 2

/* ---- simulation / domain parameters ------------------------------------
 * domain: bounds + periodic flags (exaNBody Domain, e.g.
 * example/spheres/rotating-drum/rotating-drum-mini.msp "domain:" block);
 * rcut_inc: Verlet skin (slot rcut_inc, nbh_sphere.cu:48);
 * cell_size: 0 = deduced as max(2*r_max + rcut_inc) (config_globals.msp:35-37,
 * src/field/dem_rcut_max.cpp:49-66).                                       */
typedef struct dem_params {
  double bounds_lo[3];
  double bounds_hi[3];
  int32_t periodic[3];
  double rcut_inc;
  double cell_size;
  double dt;
  double gravity[3];       /* gravity_force slot "gravity" (gravity_force.hpp:38-46) */
  int32_t symetric;        /* nbh_sphere / contact_sphere slot "symetric"; only 1 is supported */
  int32_t law;             /* DEM_LAW_* */
  dem_contact_params config;        /* contact_sphere slot "config"        */
  dem_contact_params config_driver; /* contact_sphere slot "config_driver" */
  /* Split-precision switches (no effect on results):
   * fp32_broad_phase: FP32 cell-relative broad phase with a proven superset bound,
   *                   then an exact FP64 decision in the rounding band;
   *                   polyhedra: FP32 feature tests with error bounds, FP64
   *                   where undecided;
   * fp32_contact_screen: FP32 test that skips the FP64 contact law (spheres)
   *                   or detection (polyhedra, fused step) for pairs that are
   *                   provably apart.                                      */
  int32_t fp32_broad_phase;
  int32_t fp32_contact_screen;
  /* fused_step: dem_step runs the fused kernels (prolog + displacement test,
   * compacted three-pass contact law, gather + force_to_accel + epilog) with
   * exact reciprocal-based divisions.  Same results bit for bit.          */
  int32_t fused_step;
  /* graph_step (with fused_step, spheres): dem_step replays the whole step as
   * one CUDA graph; the neighbour rebuild is a conditional node that the
   * device enables from its displacement trigger, with fixed-capacity
   * interaction buffers (on overflow the call restores its starting state,
   * doubles the capacity and runs again).  Same results bit for bit.       */
  int32_t graph_step;
  /* learned_sizing (polyhedra, with fp32_broad_phase and trained weights,
   * dem_learned.h): 1: the MLP's predicted feature counts size each candidate
   * pair's feature record in the count pass; 2: and the count pass visits the
   * pairs in warp bins by predicted contact type.  A pair whose features
   * overflow its record is enumerated again exactly.  Same results bit for bit. */
  int32_t learned_sizing;
  int32_t reserved[3];
} dem_params;

/* ---- particle state view (host or device pointers) ---------------------
 * Field names follow include/exaDEM/fields.h:34-54 and the implicit exaNBody
 * fields rx..fz, id, type.  f holds forces after compute_force and
 * accelerations after force_to_accel, exactly as in the reference.
 * Pointers that are NULL in dem_get_particles are skipped.                */
typedef struct dem_particles {
  uint64_t n;
  double *rx, *ry, *rz;
  double *vx, *vy, *vz;
  double *fx, *fy, *fz;
  double *vrotx, *vroty, *vrotz; /* angular velocity (field vrot)      */
  double *arotx, *aroty, *arotz; /* angular acceleration (field arot)  */
  double *momx, *momy, *momz;    /* torque (field mom)                 */
  double *qw, *qx, *qy, *qz;     /* orientation (field orient)         */
  double *inertiax, *inertiay, *inertiaz;
  double *mass, *radius, *homothety;
  uint64_t *id;
  uint32_t *type, *group;
} dem_particles;

/* ---- drivers (src/driver/include/exaDEM/surface.hpp:29-44, cylinder.hpp:27-36) */
typedef struct dem_surface {
  double offset;     /* along normal                       */
  double normal[3];  /* unit normal                        */
  double center[3];  /* defaults to offset*normal if vrot==0 (surface.hpp:68-76) */
  double vel[3];
  double vrot[3];
} dem_surface;

typedef struct dem_cylinder {
  double radius;
  double axis[3];    /* component mask, e.g. (1,0,1) for a y-axis drum (cylinder.hpp:255-277) */
  double center[3];  /* stored as axis*center (cylinder.hpp:89-99)          */
  double vel[3];
  double vrot[3];    /* drum angular velocity                               */
} dem_cylinder;

/* Mesh driver: register_stl_mesh / register_rshape (register_stl_mesh.cpp:40-147,
 * rshape.hpp:104-420) with STATIONARY motion and zero velocities.  The shape
 * is given as the reference's shape arrays after the STL conversion and
 * rescale (stl_mesh_to_driver.hpp:26-121): vertices in the mesh frame, edges
 * as vertex pairs, faces as vertex lists (at least 3 each).  World vertices are
 * center + quat * vertex (shape::get_vertex with homothety 1).  Each of nv, ne,
 * nf must be below 65535 (the partner sub of the list is 16 bits).         */
typedef struct dem_mesh {
  int32_t nv, ne, nf;
  const double* vertices;       /* 3 * nv                                  */
  const int32_t* edges;         /* 2 * ne                                  */
  const int32_t* face_offsets;  /* nf + 1, face f = face_vertices[off[f] .. off[f+1]) */
  const int32_t* face_vertices; /* face_offsets[nf]                        */
  double minkowski;             /* Minkowski radius (shape::add_radius)    */
  double center[3];
  double quat[4];               /* w x y z                                 */
} dem_mesh;

/* ---- thermodynamic state (src/io/include/exaDEM/simulation_state.hpp:48-56) */
typedef struct dem_state {
  double kinetic_energy[3];  /* sum 0.5*m*v*v per component            */
  double rotation_energy[3]; /* sum 0.5*m*w*w per component (sic)      */
  double mass;
  uint64_t n_particles;
  uint64_t n_interactions;        /* candidate interactions in the list */
  uint64_t n_active_interactions; /* with dn < 0 at the last force pass */
} dem_state;

/* ---- interaction list readback ------------------------------------------
 * One row per interaction, sorted by InteractionPair::operator<
 * (owner id, partner id, type, swap, owner sub, partner sub)
 * (src/interaction/include/exaDEM/interaction/interaction_pair.hpp:222-249).
 * For driver interactions partner_id is the driver index (in a batched
 * context, the index within the owner's system).  Arrays must hold
 * `capacity` rows; NULL arrays are skipped.                               */
typedef struct dem_interaction_list {
  uint64_t capacity;
  uint64_t count; /* out */
  uint64_t *owner_id, *partner_id;
  uint16_t *type;
  uint8_t *swap;
  uint32_t *owner_sub, *partner_sub;
  double *friction;  /* 3*capacity, xyz interleaved (attr::friction) */
  double *moment;    /* 3*capacity (attr::moment)                    */
} dem_interaction_list;

/* ---- convex sphero-polyhedron shapes --------------------------------------
 * Mirrors exaDEM's shape (src/shape/include/exaDEM/shape.hpp:50-68) and the
 * .shp file layout (example/polyhedra/rotating_drum/octahedron.shp):
 * vertices, edges (vertex pairs), faces (vertex lists), Minkowski radius and
 * the precomputed shape OBB (preCompDone: obb.center/e1/e2/e3/extent, the
 * extent including the radius, shape_prepro.hpp:26-97).  Particle field
 * `type` indexes the shape table.                                          */
typedef struct dem_shape {
  int32_t nv, ne, nf;
  const double* vertices;       /* 3*nv, body frame                   */
  const int32_t* edges;         /* 2*ne                               */
  const int32_t* face_sizes;    /* nf                                 */
  const int32_t* face_vertices; /* sum(face_sizes), in face order     */
  double radius;                /* Minkowski radius                   */
  double obb_center[3], obb_e1[3], obb_e2[3], obb_e3[3], obb_extent[3];
} dem_shape;
#define DEM_MAX_SHAPE_VERTICES 32
#define DEM_MAX_SHAPE_FACE_SIZE 16

typedef struct dem_ctx dem_ctx;

/* ---- lifecycle ----------------------------------------------------------- */
/* Creates a context on the current CUDA device.  No reference counterpart:
 * in exaDEM the operator slots own the data (onika::scg slots).           */
int dem_ctx_create(const dem_params* params, dem_ctx** out);
int dem_ctx_destroy(dem_ctx* ctx);
const char* dem_last_error(const dem_ctx* ctx);
/* The ctx's CUDA stream (cudaStream_t), as the operator's
 * parallel_execution_context() stream (classifier_for_all.hpp:244-255).  */
int dem_ctx_stream(dem_ctx* ctx, void** stream);
int dem_set_params(dem_ctx* ctx, const dem_params* params);
/* Multi-material contact parameters (multimat_contact_params /
 * drivers_contact_params operators, multimat_parameters.hpp:38-300; the
 * contact_multimat_* operator variants).  The parameters of a particle pair
 * are pairs[g_i * ngroups + g_j] and of a particle and driver d
 * drivers[g_i * ndrivers + d], g the particle's group field; the law
 * (dem_params.law) stays global.  pairs must be symmetric; ndrivers must equal
 * the number of registered drivers; every particle group must be < ngroups
 * (checked here and by dem_set_particles).  ngroups = 0 returns to the single
 * sets config / config_driver.  Takes effect at the next step.            */
int dem_set_multimat(dem_ctx* ctx, int ngroups, const dem_contact_params* pairs, int ndrivers,
                     const dem_contact_params* drivers);

/* ---- state binding ------------------------------------------------------ */
/* Replaces the particle set (input_data + set_fields, src/field/set_fields.cu:238-330).
 * on_device != 0: the pointers are device pointers.                      */
int dem_set_particles(dem_ctx* ctx, const dem_particles* p, int on_device);
/* Reads the particle set back (in the library's internal cell order; use id). */
int dem_get_particles(dem_ctx* ctx, dem_particles* out, int on_device);
/* register_surface / register_cylinder (drivers.hpp:291-320).  Stationary
 * motion only; vrot enters the relative velocity (rotating drum).         */
int dem_register_surface(dem_ctx* ctx, const dem_surface* s);
int dem_register_cylinder(dem_ctx* ctx, const dem_cylinder* c);
/* register_stl_mesh.  Spheres: interaction types 7-9, the sphere against a mesh
 * vertex, edge or face (nbh_sphere.hpp:25-86, contact_sphere.hpp:300-396).
 * Polyhedra: types 7-12 (nbh_polyhedron_driver.hpp:61-192,
 * polyhedron/contact.hpp:305-432), owner sub = the particle's vertex, edge or
 * face, partner sub = the mesh's.  The driver index is the registration order,
 * shared with the other drivers.  Polyhedron systems with a mesh need
 * learned_sizing = 0.                                                        */
int dem_register_mesh(dem_ctx* ctx, const dem_mesh* m);

/* ---- batching: many independent systems in one context -------------------
 * No reference counterpart (one exaDEM run is one system).  Each system is a
 * contiguous range of the particles given to dem_set_particles, with its own
 * domain (bounds, periodicity; cell grid of the shared cell size) and its own
 * drivers (a range of the registration order).  Particles of different
 * systems never interact, every system evolves exactly as it would alone, and
 * every kernel of a step covers all systems in one launch.  Spheres only.
 * Ids must be unique over all systems.  Each system rebuilds on its own
 * displacement trigger: a rebuild launch covers all systems, but systems whose
 * trigger did not fire keep their particle slots, positions, backups and
 * interaction list unchanged (the list is copied), so every system evolves
 * bit for bit as it does alone, list included.  The cohesive law is accepted
 * for a single system only.  Call after dem_set_particles (which resets the
 * context to a single system spanning the params' domain) and after the
 * drivers are registered.                                                  */
typedef struct dem_system {
  uint64_t first;         /* first particle of the system                    */
  uint64_t count;         /* number of particles                             */
  double bounds_lo[3], bounds_hi[3];
  int32_t periodic[3];
  int32_t driver_first;   /* drivers [driver_first, driver_first + driver_count) */
  int32_t driver_count;
} dem_system;
#define DEM_MAX_SYSTEMS 65536
#define DEM_MAX_DRIVERS 1024
int dem_set_systems(dem_ctx* ctx, const dem_system* systems, int nsystems);
int dem_system_count(dem_ctx* ctx, int* out);
/* simulation_state of each system: out[k] for system k (nsystems entries).
 * n_interactions / n_active_interactions are those owned by the system.  */
int dem_simulation_state_systems(dem_ctx* ctx, dem_state* out, int nsystems);

/* Switches the context to polyhedron mode (nbh_polyhedron, contact_polyhedron,
 * vertex_displ_over, config_polyhedra.msp:6-34).  Shapes are copied.       */
int dem_set_shapes(dem_ctx* ctx, const dem_shape* shapes, int nshapes);

/* ---- one call per reference operator ------------------------------------ */
/* particle_displ_over (exaNBody; threshold max_displ = rcut_inc/2,
 * config_move_particles.msp:12-15): *result = 1 if some particle moved by
 * >= threshold since the last neighbour update.                          */
int dem_particle_displ_over(dem_ctx* ctx, int* result);
/* update_particle_neighbors for spheres: periodic wrap (move_particles),
 * chunk_neighbors_contact (src/grid/chunk_neighbors_contact.cpp:45-114),
 * nbh_sphere with history carry-over (src/sphere/nbh_sphere.cu:64-309,
 * interaction_manager.hpp:89-112), classify_interactions
 * (src/interaction/classify_interactions.cpp:52-136) and backup_r.      */
int dem_update_particle_neighbors(dem_ctx* ctx);
/* compute_vertices (src/polyhedron/compute_vertices.cu:68-108): world-space
 * vertices v = r + q * (h * v0) of every polyhedron.                      */
int dem_compute_vertices(dem_ctx* ctx);
/* vertex_displ_over (src/polyhedron/vertex_displ_over.cu:74-134, backup_dem.hpp:65-110):
 * *result = 1 if some vertex moved by >= rcut_inc/2 since the last rebuild. */
int dem_vertex_displ_over(dem_ctx* ctx, int* result);
/* contact_polyhedron / contact_singlemat_polyhedron_hooke[_none]
 * (src/polyhedron/contact_force_polyhedron.cu.in:186-215,
 * polyhedron/contact.hpp:123-303): VV, VE, VF, EE and vertex-driver contacts. */
int dem_contact_polyhedron(dem_ctx* ctx);
/* reset_force_moment (src/numericalscheme/reset_force_moment.cu:69-70) */
int dem_reset_force_moment(dem_ctx* ctx);
/* gravity_force (src/forcefield/gravity_force.cu:67-86), g from params */
int dem_gravity_force(dem_ctx* ctx);
/* contact_sphere / contact_singlemat_sphere_hooke_{none,cohesive}
 * (src/sphere/contact_force_sphere.cu.in:133-188, contact_sphere.hpp:122-297).
 * Adds contact forces and torques to f and mom with a deterministic
 * per-particle gather instead of atomics.                                 */
int dem_contact_sphere(dem_ctx* ctx);
/* force_to_accel (src/numericalscheme/include/exaDEM/force_to_accel.hpp:26-33) */
int dem_force_to_accel(dem_ctx* ctx);
/* combined_compute_prolog (src/numericalscheme/combined_compute_prolog.cu:94-116) */
int dem_combined_compute_prolog(dem_ctx* ctx);
/* combined_compute_epilog (src/numericalscheme/combined_compute_epilog.cu:94-113) */
int dem_combined_compute_epilog(dem_ctx* ctx);
/* simulation_state (src/io/simulation_state.cu:121-200) */
int dem_simulation_state(dem_ctx* ctx, dem_state* out);

/* ---- fused sequences ------------------------------------------------------ */
/* first_iteration (data/config/main-config.msp:55-65): init_particles
 * (neighbour build), reset_force_moment, compute_force (gravity + contact).
 * As in the reference deck, force_to_accel is NOT applied here.           */
int dem_first_iteration(dem_ctx* ctx);
/* nsteps iterations of compute_loop with numerical_scheme_verlet
 * (config_numerical_schemes.msp:6-28): prolog, displacement trigger and
 * conditional rebuild, reset, gravity, contact, force_to_accel, epilog.
 * The device decides rebuilds; the host does not synchronise per step.  */
int dem_step(dem_ctx* ctx, int nsteps);
/* Initial interaction capacity of the graph step (graph_step; default twice
 * the current list + 4096).  It only sizes buffers: an overflow is recovered
 * by rerunning the call's steps with twice the capacity.                  */
int dem_set_graph_capacity(dem_ctx* ctx, uint64_t capacity);

/* Autotuner of the fused sphere step (no reference counterpart; exaDEM takes
 * cell_size and rcut_inc from the deck).  It times, on a copy of the state
 * restored after each trial, a forced rebuild and steps_per_trial steps of
 * candidate cell sizes (1, 1.25, 1.5 x (2 r_max + skin)), skins (0.5 to 3 x the
 * current one) and launch shapes, and keeps the one with the lowest
 * t_step + t_rebuild / min(50, (skin/2) / (v_max dt)).  Cell size and launch shapes
 * never change the list or the arithmetic.  The skin is tuned
 *   skin_policy 0: never;
 *   skin_policy 1: only without cohesion and without periodic axes, where a
 *                  pair outside the list is apart and no result bit changes;
 *   skin_policy 2: also with periodic axes (a rebuild wraps positions, so the
 *                  rebuild steps reach the low bits: the run then equals the
 *                  reference run with the chosen skin).  Never with cohesion. */
typedef struct dem_tune_result {
  double rcut_inc;               /* chosen skin (unchanged with cohesion)        */
  double cell_size;              /* chosen cell_size parameter                   */
  int32_t block;                 /* threads per block, fused prolog / epilog     */
  int32_t contact_blocks_per_sm; /* persistent grid of the compacted contact law */
  double ms_per_step;            /* model cost of the choice                     */
  double ms_per_step_before;     /* model cost of the configuration before       */
  int32_t trials;
  float vmax;                    /* fastest particle speed used by the model     */
  int32_t mul_mode;              /* multiply placement, see dem_set_mul_mode     */
  int32_t fused_contact;         /* 1: detection and law of the compacted contact
                                    in one kernel, 0: in two (same bits)         */
  int32_t contact_int_share;     /* see dem_set_contact_int_share                */
} dem_tune_result;
int dem_autotune(dem_ctx* ctx, int steps_per_trial, int skin_policy, dem_tune_result* out);
/* Multiply placement of the fused integration kernels (prolog, epilog).  The
 * FP64 pipe of sm_103a retires ~2 lanes per clock per SM; an IEEE multiply
 * built from integer partial products runs on the otherwise idle integer pipe
 * and returns the same bits.  mode bit 0: rotation multiplies (quaternion
 * rotations and derivative, normalisation, Euler terms) on the integer pipe;
 * bit 1: the other multiplies (Verlet pushes, quotient estimates); bit 2:
 * the sphere contact law's multiplies.  0 = FP64 pipe only.  Results are
 * identical in every mode (0..7).  Default 2; the autotuner picks the fastest
 * for the sphere step.                                                     */
int dem_set_mul_mode(dem_ctx* ctx, int mode);
int dem_get_mul_mode(dem_ctx* ctx, int* mode);
/* Share (0..8, in eighths) of the fused contact kernel's tiles of overlapping
 * pairs whose contact-law multiplies and additions run on the integer pipe
 * (IEEE binary64 round-to-nearest built from integer operations; square roots
 * and divisions stay on the FP64 pipe), so that both pipes work at once.
 * Results are identical for every share.  Default 0.  Measured on GB300 (2 M
 * sphere bed): every share from 2/8 up slows the kernel (2/8: 1.9x), because
 * an emulated addition costs several times an FP64 one; the autotuner leaves
 * it at 0.  No reference counterpart (a placement of the same arithmetic). */
int dem_set_contact_int_share(dem_ctx* ctx, int eighths);
/* Sphere broad phase with fp32_broad_phase (replaces the particle-pair part of
 * nbh_sphere, src/sphere/nbh_sphere.cu:64-309, as the default kernels do):
 * 0 = one thread per owner particle (default); 1 = one warp per cell, the
 * 27-cell neighbourhood's FP32 coordinates, radii and ids staged in shared
 * memory, candidates compacted with warp ballots, drivers tested per particle.
 * The lists are identical in both modes.  Measured on GB300 (2 M sphere bed,
 * about 35 particles per neighbourhood): mode 1 runs the count and fill passes
 * slower, since a warp per cell leaves lanes idle where a thread per owner keeps
 * all 32 busy and L1 already serves the stencil reuse. */
int dem_set_sphere_cell_broad_phase(dem_ctx* ctx, int on);
/* Number of neighbour rebuilds done so far (trigger_move_particles count). */
int dem_rebuild_count(dem_ctx* ctx, uint64_t* out);

/* ---- analysis / parity readback ------------------------------------------ */
int dem_interaction_count(dem_ctx* ctx, uint64_t* out);
int dem_get_interactions(dem_ctx* ctx, dem_interaction_list* out);
/* read_dump_particle_interaction (src/io/sim_dump_reader_interaction.cpp:56-63):
 * restart from a checkpoint.  Installs the friction/moment history of a saved
 * list (rows as dem_get_interactions writes them, count = rows) for the
 * particles currently set, matched by id; the next neighbour build carries it
 * over by InteractionPair key, as a rebuild of a running context does.  To
 * resume a run: dem_set_particles with the saved state (f holding the
 * accelerations of the saved step), dem_set_interactions with the saved list,
 * dem_update_particle_neighbors, then dem_step: the run continues with the
 * same bits as if it had not stopped (no dem_first_iteration, whose forces
 * would replace the saved accelerations).  Call it after dem_set_particles
 * and after registering the drivers.                                       */
int dem_set_interactions(dem_ctx* ctx, const dem_interaction_list* list);
/* Packing-fraction profile: solid volume fraction of the spheres in nslabs
 * equal horizontal slabs between zlo and zhi (no reference counterpart;
 * analytic sphere/slab volumes).  out has nslabs entries.                 */
int dem_packing_profile(dem_ctx* ctx, int nslabs, double zlo, double zhi, double* out);

/* ---- analysis -------------------------------------------------------------
 * Contact state and stress tensor (classifier/contact_state.hpp:22-50,
 * AnalysisDataPacker classifier_for_all.hpp:55-97, stress_tensor.cu:30-160).
 * With dem_set_analysis(ctx, 1) every contact pass writes, per interaction,
 * the overlap dn (0 for a pair that does not touch), the contact point, the
 * normal force f - ft and the tangential force ft; the FP32 separation screen
 * and the skipped zero records are off while it is on, so every pair's state
 * is computed.  A polyhedron pair's state is in its contact law's frame: f is
 * the force on pi_, which is the partner when the pair is swapped
 * (interaction_pair.hpp:70-112, polyhedron/contact.hpp:191-210).          */
typedef struct dem_contact_state {
  uint64_t capacity;  /* entries the caller's arrays hold                      */
  uint64_t count;     /* written: interactions, in dem_get_interactions order  */
  double* dn;         /* count                                                 */
  double* cp;         /* 3 * count, x y z of each contact point                */
  double* fn;         /* 3 * count                                             */
  double* ft;         /* 3 * count                                             */
} dem_contact_state;
int dem_set_analysis(dem_ctx* ctx, int on);
int dem_get_contact_state(dem_ctx* ctx, dem_contact_state* out);
/* stress_tensor: for every touching pair (dn < 0) of the last force pass,
 * fij = fn + ft and cij = cp - r_i add the outer product fij cij^T (row major,
 * m[3 r + c] = fij_r cij_c) to the law's particle i, and -fij (cp - r_j)^T to
 * its particle j (not to a periodic image; drivers: particle i only).  Each particle sums its own pairs, then
 * the pairs where it is the partner, in InteractionPair order (the reference
 * adds with unordered atomics).  stress: 9 n doubles in the particles'
 * internal order (dem_get_particles); total: the 9-component sum over the
 * particles in id order.  Either may be NULL.                             */
int dem_stress_tensor(dem_ctx* ctx, double* stress, double* total);

/* ---- profiling ------------------------------------------------------------
 * Stands in for onika's per-operator timers (profiling: exectime / summary,
 * data/config/config_defaults.msp:30-33).  Kernel launches are always
 * counted; with dem_profile(ctx, 1) each kernel class is also timed with CUDA
 * events on the ctx stream.  dem_kernel_stats fills up to `capacity` rows.  */
typedef struct dem_kernel_stat {
  char name[24];
  uint64_t launches;
  uint64_t timed;   /* number of timed launch groups  */
  double total_ms;  /* summed CUDA-event time          */
} dem_kernel_stat;
int dem_profile(dem_ctx* ctx, int enable);
int dem_kernel_stats(dem_ctx* ctx, dem_kernel_stat* out, int capacity, int* count);
int dem_reset_kernel_stats(dem_ctx* ctx);

/* ---- fragmentation: inner bonds between polyhedra --------------------------
 * A bond ties vertex sub_i of particle id_i to vertex sub_j of particle id_j
 * (id_i < id_j), InnerBondInteraction (interaction/inner_bond_interaction.hpp:
 * 28-62, interaction type 13).  The bonds of one particle pair form an
 * interface (interface/interface.hpp:27-31) that breaks as a whole.  Bonds are
 * kept in (id_i, id_j, sub_i) order.  Every step:
 *   - after the prolog, apply_interface_fracture_criterion (interface/
 *     apply_interface_fracture_criterion.hpp:35-76) on the energies and forces
 *     of the previous force pass, per interface: En = sum en, Et = sum et, S =
 *     (sum of |fn| over the bonds with dn > 0) / size; it breaks when
 *       DEM_RUPTURE_ENERGY_MIXED:          En + Et > crit1,
 *       DEM_RUPTURE_ENERGY_SEPARATE:       En > crit1 or Et > crit2,
 *       DEM_RUPTURE_STRESS_ENERGY_SEPARATE: En > crit1 and S > crit2;
 *     broken_interface_friction_updater (broken_interface_friction_updater.cpp:
 *     52-86) then clips each bond's friction to mu |fn| (mu of the contact
 *     parameters of the two groups), or zeroes it where dn > 0;
 *   - a broken interface forces a neighbour rebuild, where its bonds become
 *     vertex-vertex history (broke_interaction, inner_bond_interaction.hpp:
 *     202-210: friction kept, moment 0, carried by key like any history) and
 *     leave the bond list;
 *   - a rebuild lists no contact between two bonded particles (the ignore list
 *     of interaction_manager.hpp:114-160; as there, a particle that owns a bond
 *     to the particle of id k also lists no interaction with driver k);
 *   - the force pass runs inner_bond_law (polyhedron/inner_bond.hpp:112-186,
 *     forcefield/inner_bond_force.hpp:24-70) on every bond after the contacts;
 *     each particle adds gravity, its contacts (owned, then as partner) and
 *     then its bonds (owned, then as partner), each in list order.
 * The criterion is stored per bond (2 area g, ... as dem_stick_polyhedra
 * computes it); an interface uses the one of its first bond.               */
#define DEM_RUPTURE_ENERGY_MIXED 0
#define DEM_RUPTURE_ENERGY_SEPARATE 1
#define DEM_RUPTURE_STRESS_ENERGY_SEPARATE 2
/* InnerBondParams (forcefield/inner_bond_parameters.hpp:27-35). */
typedef struct dem_inner_bond_params {
  double kn, kt, damp_rate;
  int32_t mode; /* DEM_RUPTURE_*                                            */
  int32_t pad;
  double crit1; /* g (mixed, stress-energy) or gn (separate)                */
  double crit2; /* unused (mixed), gt (separate) or sigma (stress-energy)   */
} dem_inner_bond_params;
/* inner_bond_params (src/forcefield/multimat_inner_bond.cpp:104-200): the
 * table pairs[g_i * ngroups + g_j] by the particles' group field, or with
 * ngroups = 0 the one set pairs[0] for every pair.                        */
int dem_set_inner_bond_params(dem_ctx* ctx, int ngroups, const dem_inner_bond_params* pairs);
/* stick_polyhedra (src/polyhedron/stick_polyhedra.cpp:60-360): bonds between
 * the faces that touch.  cluster[k] is the cluster of particle ids[k] (the
 * cluster field; every particle must be listed).  For each pair of particles of
 * the same cluster with id_i < id_j and centres closer than the neighbour
 * distance, the first face i of particle id_i (file order) and face j of id_j
 * with the same vertex count (>= 3), areas within 1 %, and parallel unit
 * normals (|n_i x n_j| <= 1e-10) bond each vertex of face i to the first
 * vertex of face j closer than sticking_threshold (vertex-vertex dn); a face
 * match with fewer than 3 such vertices is dropped and the search goes on.
 * Weight 1/(bonds of the pair); criterion 2 area g (area of face i scaled by
 * h_i^2; stress-energy: area sigma) from the pair's inner bond parameters;
 * the bond vertices of particle id_i must be coplanar (1e-10).  Replaces
 * the bond list; the contacts of bonded pairs leave the list at the next
 * rebuild (call it before dem_first_iteration).  nbonds: bonds made.      */
int dem_stick_polyhedra(dem_ctx* ctx, const uint64_t* ids, const double* cluster, uint64_t n,
                        double sticking_threshold, uint64_t* nbonds);
/* One row per bond, in bond order (en, et: energies of the last force pass;
 * tds: cumulated tangential displacement; friction = kt weight tds). */
typedef struct dem_bond_list {
  uint64_t capacity; /* rows the caller's arrays hold                         */
  uint64_t count;    /* rows written (get) or given (set)                     */
  uint64_t* id_i;
  uint64_t* id_j;
  uint32_t* sub_i;
  uint32_t* sub_j;
  double* dn0;
  double* weight;
  int32_t* mode;
  double* crit1;
  double* crit2;
  double* en;
  double* et;
  double* tds;      /* 3 per row */
  double* friction; /* 3 per row */
  uint8_t* unbroken;
} dem_bond_list;
int dem_bond_count(dem_ctx* ctx, uint64_t* out);
int dem_get_bonds(dem_ctx* ctx, dem_bond_list* out);
/* read_dump_particle_fragmentation: installs a saved bond list (rows as
 * dem_get_bonds writes them) for the particles currently set, by id.     */
int dem_set_bonds(dem_ctx* ctx, const dem_bond_list* list);
/* Contact state of the inner bonds, as inner_bond_law returns it for the
 * analysis (src/polyhedron/include/exaDEM/polyhedron/inner_bond.hpp:167-184):
 * per bond of the last bond pass, dn, fn = f_i - friction and the friction, in
 * the rows of dem_get_bonds.  capacity: rows the arrays hold (count written to
 * *count); fn and ft hold 3 per row; a null array is skipped.  Zero before the
 * first bond pass.  dump_contact_network adds these to the network. */
int dem_get_bond_state(dem_ctx* ctx, uint64_t capacity, uint64_t* count, double* dn, double* fn, double* ft);
/* Interfaces broken since the context was made (the sum of the
 * apply_interface_fracture_criterion results). */
int dem_broken_interface_count(dem_ctx* ctx, uint64_t* out);
/* The two operators on their own, for callers that schedule the operators
 * themselves (dem_step runs both):
 * inner_bond_polyhedron (src/polyhedron/inner_bond_force.cu:98-134): the bond
 * pass on the current vertices, its forces added after the contact gather;
 * apply_interface_fracture_criterion + broken_interface_friction_updater
 * (apply_interface_fracture_criterion.cu:44-86): broken = interfaces broken
 * now; their bonds leave the list at the next dem_update_particle_neighbors. */
int dem_inner_bond_polyhedron(dem_ctx* ctx);
int dem_apply_interface_fracture_criterion(dem_ctx* ctx, uint64_t* broken);

/* ---- state reduction without any device allocation ---------------------
 * No counterpart in the reference.  For callers that may not call cudaMalloc
 * (their device memory is owned by another allocator, or they must not pay
 * the implicit synchronisation of cudaMalloc/cudaFree): the same sums as
 * dem_simulation_state, over particle arrays already on the device.  The only
 * scratch is a file-scope device array sized for
 * DEM_STATE_NOALLOC_MAX_PARTICLES particles (448 KiB, held by every GPU that
 * loads the library until exit); larger n returns DEM_ERR_INVALID_ARG.
 *   dev:     device pointers vx, vy, vz, vrotx, vroty, vrotz, mass and n
 *            (other fields unused);
 *   dev_out: device array of 7 doubles, written in the order
 *            kinetic_energy x,y,z, rotation_energy x,y,z, mass;
 *   stream:  cudaStream_t (NULL = legacy default stream); asynchronous.
 * Every call looks up the scratch address on the current device; the first
 * call on a device also loads the device code (make it before any stream
 * capture).  A CUDA error pending from the caller's earlier work makes the
 * call return DEM_ERR_CUDA without launching.  Calls share the scratch: calls
 * that overlap on the GPU race. */
#define DEM_STATE_NOALLOC_MAX_PARTICLES 16777216ull
int dem_simulation_state_noalloc(const dem_particles* dev, double* dev_out, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* DEM_HOTPATH_H */
