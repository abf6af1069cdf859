/*
 * dem_workloads.h -- seeded synthetic particle sets for tests and benchmarks.
 *
 * Not part of the reference boundary: exaDEM builds its inputs with deck
 * operators (lattice, rsa_vol_frac through the external rsa_mpi library,
 * set_fields, src/field/set_fields.cu:238-330).  This generator produces the
 * same kind of input -- non-overlapping spheres placed by random sequential
 * addition, with sphere mass rho*4/3*pi*r^3 and inertia 0.4*m*r^2 as in
 * set_fields.cu:320-327 -- from a fixed seed, so that every run of a workload
 * sees identical inputs.
 */
#ifndef DEM_WORKLOADS_H
#define DEM_WORKLOADS_H
#include <stdint.h>

#include "dem_hotpath.h"

#ifdef __cplusplus
extern "C" {
#endif

#define DEM_REGION_BOX 0
#define DEM_REGION_CYLINDER_Y 1 /* drum with its axis along y */

typedef struct dem_rsa_spec {
  uint64_t n;
  double rmin, rmax;      /* radius uniform in [rmin, rmax]                  */
  double density;
  double lo[3], hi[3];    /* placement box                                   */
  int32_t periodic[3];    /* periodic axes: minimum-image overlap test        */
  int32_t grow_axis;      /* -1: fail when full; else extend hi[axis] when a
                             sphere finds no room in max_attempts draws     */
  int32_t region;         /* DEM_REGION_*                                    */
  double cyl_center[2];   /* (x, z) of the drum axis for DEM_REGION_CYLINDER_Y */
  double cyl_radius;
  double vmin, vmax;      /* velocity components uniform in [vmin, vmax]     */
  uint64_t seed;
  uint64_t max_attempts;
  uint64_t id_offset;     /* ids are id_offset + k                           */
  const double* radii;    /* optional: radius of sphere k (overrides rmin/rmax draws) */
} dem_rsa_spec;

/* Fills out->rx..rz, radius, mass, inertia*, vx..vz, qw (=1), id for
 * spec->n spheres.  out arrays must hold n entries (NULL ones are skipped).
 * *placed_hi receives the final hi[grow_axis] (or hi[2]).                  */
int dem_generate_rsa_spheres(const dem_rsa_spec* spec, dem_particles* out, double* placed_hi);

#ifdef __cplusplus
}
#endif
#endif
