// gb300_bridge.hpp -- the bridge between an exaNBody grid and a libexadem_gb300
// context, for the onika operator shims of gb300_operators.cpp.
//
// Compiled inside an exaDEM build (onika and exaNBody headers, this repository's
// include/ on the include path, linked with libexadem_gb300.so).  One library
// context per grid object holds the particles and the interaction list with its
// friction/moment history for the whole run, as exaDEM's extra storage does
// between operators.  The grid is its mirror:
// - pull(): the real (non-ghost) cells' particles are gathered into the
//   library's structure-of-arrays layout and uploaded (dem_set_particles) the
//   first time and whenever the grid's particle count changed (particles added
//   or removed by operators outside the hot path);
// - push(): after an operator, the fields it wrote are read back
//   (dem_get_particles) and scattered into the cells by particle id.
// Errors print the library's message and exit, as color_log::error does.
#pragma once

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <unordered_map>
#include <vector>

#include <dem_hotpath.h>

namespace gb300 {

inline void check(int rc, dem_ctx* ctx, const char* op) {
  if (rc == DEM_OK) return;
  std::fprintf(stderr, "[ERROR, %s] %s\n", op, ctx ? dem_last_error(ctx) : "no context");
  std::exit(EXIT_FAILURE);
}

// Fields the bridge moves, in dem_particles order.
enum Field : int {
  RX, RY, RZ, VX, VY, VZ, FX, FY, FZ, WX, WY, WZ, AX, AY, AZ, MX, MY, MZ, QW, QX, QY, QZ, IX, IY, IZ, MASS, RAD, HOM,
  NFIELDS
};

struct Bridge {
  dem_ctx* ctx = nullptr;
  dem_params prm{};
  bool have_prm = false;
  size_t n = 0;                                   // particles in the context
  std::vector<double> f[NFIELDS];
  std::vector<uint64_t> id;
  std::vector<uint32_t> type, group;
  std::unordered_map<uint64_t, std::pair<size_t, size_t>> cell_of_id;  // id -> (cell, index in cell)

  dem_particles view() {
    dem_particles p{};
    p.n = n;
    double** dst[NFIELDS] = {&p.rx, &p.ry, &p.rz, &p.vx, &p.vy, &p.vz, &p.fx, &p.fy, &p.fz,
                             &p.vrotx, &p.vroty, &p.vrotz, &p.arotx, &p.aroty, &p.arotz,
                             &p.momx, &p.momy, &p.momz, &p.qw, &p.qx, &p.qy, &p.qz,
                             &p.inertiax, &p.inertiay, &p.inertiaz, &p.mass, &p.radius, &p.homothety};
    for (int k = 0; k < NFIELDS; k++) *dst[k] = f[k].data();
    p.id = id.data();
    p.type = type.data();
    p.group = group.data();
    return p;
  }

  // Creates the context on first use, or updates its parameters.
  void configure(const dem_params& p) {
    if (!ctx) {
      check(dem_ctx_create(&p, &ctx), nullptr, "gb300");
    } else {
      check(dem_set_params(ctx, &p), ctx, "gb300");
    }
    prm = p;
    have_prm = true;
  }

  template <class GridT>
  size_t real_count(GridT& grid) const {
    size_t total = 0;
    auto cells = grid.cells();
    for (size_t c = 0; c < grid.number_of_cells(); c++)
      if (!grid.is_ghost_cell(c)) total += cells[c].size();
    return total;
  }

  template <class GridT>
  void pull(GridT& grid) {
    if (ctx && real_count(grid) == n && n > 0) return;  // the context already holds these particles
    using namespace exanb;
    auto cells = grid.cells();
    n = real_count(grid);
    for (auto& v : f) v.resize(n);
    id.resize(n);
    type.resize(n);
    group.resize(n);
    cell_of_id.clear();
    size_t k = 0;
    for (size_t c = 0; c < grid.number_of_cells(); c++) {
      if (grid.is_ghost_cell(c)) continue;
      auto& cell = cells[c];
      for (size_t p = 0; p < cell.size(); p++, k++) {
        f[RX][k] = cell[field::rx][p];
        f[RY][k] = cell[field::ry][p];
        f[RZ][k] = cell[field::rz][p];
        f[VX][k] = cell[field::vx][p];
        f[VY][k] = cell[field::vy][p];
        f[VZ][k] = cell[field::vz][p];
        f[FX][k] = cell[field::fx][p];
        f[FY][k] = cell[field::fy][p];
        f[FZ][k] = cell[field::fz][p];
        const auto& w = cell[field::vrot][p];
        const auto& a = cell[field::arot][p];
        const auto& m = cell[field::mom][p];
        const auto& q = cell[field::orient][p];
        const auto& I = cell[field::inertia][p];
        f[WX][k] = w.x, f[WY][k] = w.y, f[WZ][k] = w.z;
        f[AX][k] = a.x, f[AY][k] = a.y, f[AZ][k] = a.z;
        f[MX][k] = m.x, f[MY][k] = m.y, f[MZ][k] = m.z;
        f[QW][k] = q.w, f[QX][k] = q.x, f[QY][k] = q.y, f[QZ][k] = q.z;
        f[IX][k] = I.x, f[IY][k] = I.y, f[IZ][k] = I.z;
        f[MASS][k] = cell[field::mass][p];
        f[RAD][k] = cell[field::radius][p];
        f[HOM][k] = cell[field::homothety][p];
        id[k] = cell[field::id][p];
        type[k] = static_cast<uint32_t>(cell[field::type][p]);
        group[k] = static_cast<uint32_t>(cell[field::group][p]);
        cell_of_id[id[k]] = {c, p};
      }
    }
    dem_particles v = view();
    check(dem_set_particles(ctx, &v, 0), ctx, "gb300 pull");
  }

  // Reads the context's particles back and writes the fields in `which` into the grid.
  template <class GridT>
  void push(GridT& grid, std::initializer_list<int> which) {
    using namespace exanb;
    dem_particles v = view();
    check(dem_get_particles(ctx, &v, 0), ctx, "gb300 push");
    auto cells = grid.cells();
    for (size_t k = 0; k < n; k++) {
      const auto it = cell_of_id.find(id[k]);
      if (it == cell_of_id.end()) continue;
      auto& cell = cells[it->second.first];
      const size_t p = it->second.second;
      for (int fld : which) {
        switch (fld) {
          case RX: cell[field::rx][p] = f[RX][k], cell[field::ry][p] = f[RY][k], cell[field::rz][p] = f[RZ][k]; break;
          case VX: cell[field::vx][p] = f[VX][k], cell[field::vy][p] = f[VY][k], cell[field::vz][p] = f[VZ][k]; break;
          case FX: cell[field::fx][p] = f[FX][k], cell[field::fy][p] = f[FY][k], cell[field::fz][p] = f[FZ][k]; break;
          case WX: cell[field::vrot][p] = {f[WX][k], f[WY][k], f[WZ][k]}; break;
          case AX: cell[field::arot][p] = {f[AX][k], f[AY][k], f[AZ][k]}; break;
          case MX: cell[field::mom][p] = {f[MX][k], f[MY][k], f[MZ][k]}; break;
          case QW: cell[field::orient][p] = {f[QW][k], f[QX][k], f[QY][k], f[QZ][k]}; break;
          default: break;
        }
      }
    }
  }
};

// One bridge per grid object for the life of the process.
template <class GridT>
inline Bridge& bridge_for(GridT& grid) {
  static std::unordered_map<const void*, Bridge> bridges;
  return bridges[static_cast<const void*>(&grid)];
}

}  // namespace gb300
