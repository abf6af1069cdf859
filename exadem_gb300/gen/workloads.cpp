// workloads.cpp -- seeded random sequential addition (RSA) of spheres.
//
// Host-only input generation for tests and benchmarks (see include/dem_workloads.h).
// Portable across x86-64 and aarch64: mt19937_64 with our own uniform mapping
// (no std::*_distribution, whose algorithms are implementation-defined).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "../../include/dem_workloads.h"

namespace {
struct Rng {
  std::mt19937_64 g;
  explicit Rng(uint64_t s) : g(s) {}
  double u01() { return (double)(g() >> 11) * (1.0 / 9007199254740992.0); }
  double uniform(double a, double b) { return a + (b - a) * u01(); }
};

// Cells of at least `cell` per axis; on periodic axes the cells tile the
// period exactly (floor(L/cell) cells of width L/dims) so the +-1 stencil with
// wrap-around sees every neighbour across the boundary.
struct HashGrid {
  double lo[3], cs[3];
  int dims[3];
  std::vector<int64_t> head;
  std::vector<int64_t> next;
  void init(const double* l, const double* h, double cell, const int32_t* periodic, uint64_t n) {
    for (int d = 0; d < 3; d++) {
      lo[d] = l[d];
      const double Ld = h[d] - l[d];
      if (periodic[d]) {
        dims[d] = std::max(1, (int)std::floor(Ld / cell));
        cs[d] = Ld / dims[d];
      } else {
        dims[d] = std::max(1, (int)std::ceil(Ld / cell));
        cs[d] = cell;
      }
    }
    head.assign((size_t)dims[0] * dims[1] * dims[2], -1);
    next.assign(n, -1);
  }
  int coord(int d, double x) const {
    int k = (int)std::floor((x - lo[d]) / cs[d]);
    return std::min(std::max(k, 0), dims[d] - 1);
  }
  size_t idx(int x, int y, int z) const { return (size_t)x + (size_t)dims[0] * ((size_t)y + (size_t)dims[1] * z); }
};
}  // namespace

extern "C" int dem_generate_rsa_spheres(const dem_rsa_spec* sp, dem_particles* out, double* placed_hi) {
  if (!sp || !out || sp->n == 0 || !(sp->rmax >= sp->rmin) || !(sp->rmin > 0)) return DEM_ERR_INVALID_ARG;
  const uint64_t n = sp->n;
  Rng rng(sp->seed);
  double lo[3], hi[3];
  for (int d = 0; d < 3; d++) {
    lo[d] = sp->lo[d];
    hi[d] = sp->hi[d];
  }
  const int ga = sp->grow_axis;
  // grid big enough for generous growth along the grow axis
  double ghi[3] = {hi[0], hi[1], hi[2]};
  if (ga >= 0) {
    // room for a column at a solid fraction down to 0.05 (the moving-window RSA reaches ~0.29)
    double area = 1.0;
    for (int d = 0; d < 3; d++)
      if (d != ga) area *= hi[d] - lo[d];
    const double vmax = 4.0 / 3.0 * 3.14159265358979 * sp->rmax * sp->rmax * sp->rmax;
    ghi[ga] = hi[ga] + (double)n * vmax / (0.05 * area) + 16 * sp->rmax;
  }
  HashGrid grid;
  grid.init(lo, ghi, 2.0 * sp->rmax, sp->periodic, n);
  std::vector<double> x(n), y(n), z(n), r(n);
  const double L[3] = {hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]};
  const uint64_t max_att = sp->max_attempts ? sp->max_attempts : 64;
  for (uint64_t k = 0; k < n; k++) {
    const double rk = sp->radii ? sp->radii[k] : (sp->rmin == sp->rmax ? sp->rmin : rng.uniform(sp->rmin, sp->rmax));
    uint64_t att = 0;
    for (;;) {
      double p[3];
      bool ok_region = true;
      for (int d = 0; d < 3; d++) {
        if (sp->periodic[d])
          p[d] = rng.uniform(lo[d], hi[d]);
        else if (d == ga)
          // growing domain: draw inside a window of 4*rmax below the fill front
          p[d] = rng.uniform(std::max(lo[d] + rk, hi[d] - 4.0 * sp->rmax), hi[d] - rk);
        else
          p[d] = rng.uniform(lo[d] + rk, hi[d] - rk);
      }
      if (sp->region == DEM_REGION_CYLINDER_Y) {
        const double dx = p[0] - sp->cyl_center[0], dz = p[2] - sp->cyl_center[1];
        const double lim = sp->cyl_radius - rk;
        ok_region = lim > 0 && dx * dx + dz * dz <= lim * lim;
      }
      bool ok = ok_region;
      if (ok) {
        // per axis: the distinct cells within +-1 (wrapped on periodic axes)
        int cand[3][3], nc[3];
        for (int d = 0; d < 3; d++) {
          const int c = grid.coord(d, p[d]);
          nc[d] = 0;
          for (int o = -1; o <= 1; o++) {
            int q = c + o;
            if (q < 0 || q >= grid.dims[d]) {
              if (!sp->periodic[d]) continue;
              q = (q + grid.dims[d]) % grid.dims[d];
            }
            bool dup = false;
            for (int m = 0; m < nc[d]; m++) dup |= cand[d][m] == q;
            if (!dup) cand[d][nc[d]++] = q;
          }
        }
        for (int a = 0; a < nc[2] && ok; a++)
          for (int b = 0; b < nc[1] && ok; b++)
            for (int e = 0; e < nc[0] && ok; e++) {
              for (int64_t j = grid.head[grid.idx(cand[0][e], cand[1][b], cand[2][a])]; j >= 0; j = grid.next[j]) {
                double dd[3] = {p[0] - x[j], p[1] - y[j], p[2] - z[j]};
                for (int d = 0; d < 3; d++)
                  if (sp->periodic[d]) dd[d] -= L[d] * std::round(dd[d] / L[d]);
                const double sr = rk + r[j];
                if (dd[0] * dd[0] + dd[1] * dd[1] + dd[2] * dd[2] < sr * sr) {
                  ok = false;
                  break;
                }
              }
            }
      }
      if (ok) {
        x[k] = p[0];
        y[k] = p[1];
        z[k] = p[2];
        r[k] = rk;
        const size_t ci = grid.idx(grid.coord(0, p[0]), grid.coord(1, p[1]), grid.coord(2, p[2]));
        grid.next[k] = grid.head[ci];
        grid.head[ci] = (int64_t)k;
        break;
      }
      if (++att >= max_att) {
        if (ga < 0) return DEM_ERR_OVERFLOW;
        hi[ga] += 0.25 * sp->rmax;
        if (hi[ga] > ghi[ga]) return DEM_ERR_OVERFLOW;
        att = 0;
      }
    }
  }
  if (placed_hi) *placed_hi = ga >= 0 ? hi[ga] : hi[2];
  const double pi = 4 * std::atan(1);
  for (uint64_t k = 0; k < n; k++) {
    const double rr = r[k];
    const double V = ((4.0) / (3.0)) * pi * rr * rr * rr;  // set_fields.cu:323-327
    const double m = V * sp->density;
    const double inertia = 0.4 * m * rr * rr;
    if (out->rx) out->rx[k] = x[k];
    if (out->ry) out->ry[k] = y[k];
    if (out->rz) out->rz[k] = z[k];
    if (out->radius) out->radius[k] = rr;
    if (out->mass) out->mass[k] = m;
    if (out->inertiax) out->inertiax[k] = inertia;
    if (out->inertiay) out->inertiay[k] = inertia;
    if (out->inertiaz) out->inertiaz[k] = inertia;
    if (out->homothety) out->homothety[k] = 1.0;
    if (out->qw) out->qw[k] = 1.0;
    if (out->id) out->id[k] = sp->id_offset + k;
  }
  // velocities drawn after placement so the positions do not depend on them
  for (uint64_t k = 0; k < n; k++) {
    const double a = rng.uniform(sp->vmin, sp->vmax), b = rng.uniform(sp->vmin, sp->vmax),
                 c = rng.uniform(sp->vmin, sp->vmax);
    if (out->vx) out->vx[k] = a;
    if (out->vy) out->vy[k] = b;
    if (out->vz) out->vz[k] = c;
  }
  out->n = n;
  return DEM_OK;
}
