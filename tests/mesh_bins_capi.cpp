// C entry points over exadem_gb300/csrc/mesh_bins.hpp for tests/test_mesh_bins.py:
// build a mesh's feature bins on the host and list the features of a point's bin.
#include <cstdint>

#include "mesh_bins.hpp"

using dem::meshbins::Input;
using dem::meshbins::Output;

extern "C" {

void* mb_build(int nv, const double* x, const double* y, const double* z, int ne, const int* e, int nf,
               const int* fo, const int* fv, double minkowski, double rad, double skin, int* status) {
  Input in{nv, ne, nf, x, y, z, e, fo, fv, minkowski};
  Output* o = new Output();
  *status = dem::meshbins::build(in, rad, skin, *o);
  return o;
}

// features (kind << 30 | index) listed in the bin of p; returns their count (-1: outside the grid)
int mb_items(void* h, double px, double py, double pz, uint32_t* out, int cap) {
  const Output& o = *(const Output*)h;
  uint64_t b;
  if (!dem::meshbins::bin_of(o, px, py, pz, b)) return -1;
  const uint32_t q0 = o.boff[b], q1 = o.boff[b + 1];
  for (uint32_t q = q0; q < q1 && (int)(q - q0) < cap; q++) out[q - q0] = o.items[q];
  return (int)(q1 - q0);
}

void mb_free(void* h) { delete (Output*)h; }
}
