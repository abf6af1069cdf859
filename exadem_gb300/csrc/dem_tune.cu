// dem_tune.cu -- launch-shape, cell-size and skin autotuner for the fused sphere step.
//
// No reference counterpart: exaDEM takes cell_size and rcut_inc from the deck.
// The tuner only touches values that leave every result bit unchanged:
//  * the cell size and the launch shapes never change the interaction list
//    (the same pairs, the same canonical order) nor any arithmetic;
//  * the skin (rcut_inc) changes which non-touching pairs are listed and when
//    rebuilds happen.  Without cohesion and without periodic axes that changes
//    no force: a pair outside the list is apart, because it was beyond
//    R + skin at the last rebuild and both particles moved less than skin / 2
//    since.  With the cohesive law a pair outside the list can be inside the
//    attraction range: the skin is left alone.  With periodic axes a rebuild
//    wraps positions (x +- L, rounded), so the rebuild steps reach the low bits
//    of the trajectory: skin_policy 2 tunes it anyway (the run then equals the
//    reference run with the chosen skin), skin_policy 1 does not.
// Cost model of a configuration: t_step + t_rebuild / interval, where
// interval = (skin / 2) / (v_max dt) steps is the rebuild period of the
// fastest particle.  t_rebuild and t_step are timed with CUDA events on a
// copy of the state, which is restored after every trial.
#include <algorithm>
#include <cstring>
#include <vector>

#include "dem_ctx.cuh"

namespace dem {
int ext_update_neighbors(dem_ctx* c);
int ext_setup_grid(dem_ctx* c);
int launch_reverse_lists(dem_ctx* c);

namespace {
// max |v| over the particles: non-negative floats order like their bit patterns
__global__ void k_vmax(PArrays P, uint64_t n, unsigned int* out) {
  float m = 0.f;
  for (uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n; s += (uint64_t)gridDim.x * blockDim.x) {
    const double vx = P.f[VX][s], vy = P.f[VY][s], vz = P.f[VZ][s];
    m = fmaxf(m, (float)sqrt(vx * vx + vy * vy + vz * vz));
  }
  for (int o = 16; o; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, __float_as_uint(m));
}

size_t pblock_bytes(const dem_ctx* c) {
  return (NPF * sizeof(double) + sizeof(uint64_t) + 2 * sizeof(uint32_t)) * std::max<uint64_t>(c->pcap, 1);
}

// state of the context that a trial may change, on the device and on the host
struct Saved {
  void* dev = nullptr;
  int pcur, icur;
  uint64_t ni, rebuilds;
  bool have_list, hist_valid;
  dem_params prm;
  int tune_block, tune_contact_bps, mul_mode, int_share;
  bool fuse_contact;
};

int save_state(dem_ctx* c, Saved& s) {
  s.pcur = c->pcur;
  s.icur = c->icur;
  s.ni = c->ni;
  s.rebuilds = c->rebuilds;
  s.have_list = c->have_list;
  s.hist_valid = c->hist_valid;
  s.prm = c->prm;
  s.tune_block = c->tune_block;
  s.tune_contact_bps = c->tune_contact_bps;
  s.mul_mode = c->mul_mode;
  s.int_share = c->tune_int_share;
  s.fuse_contact = c->fuse_contact;
  const size_t bytes = pblock_bytes(c) + (c->n + 1) * 4 + c->ni * 80 + 1024;
  DEM_CUDA_TRY(c, cudaMalloc(&s.dev, bytes));
  char* p = static_cast<char*>(s.dev);
  const IArrays& I = c->I[c->icur];
  auto put = [&](const void* src, size_t b) {
    cudaMemcpyAsync(p, src, b, cudaMemcpyDeviceToDevice, c->stream);
    p += (b + 15) & ~size_t(15);
  };
  put(c->pblock[c->pcur], pblock_bytes(c));
  put(c->own_off[c->icur], (c->n + 1) * 4);
  if (c->ni) {
    put(I.owner, c->ni * 4);
    put(I.partner, c->ni * 4);
    put(I.pid, c->ni * 8);
    put(I.meta, c->ni * 4);
    put(I.sub, c->ni * 4);
    for (int d = 0; d < 3; d++) put(I.ft[d], c->ni * 8);
    for (int d = 0; d < 3; d++) put(I.mo[d], c->ni * 8);
    put(I.damp, c->ni * 8);
  }
  DEM_CUDA_TRY(c, cudaGetLastError());
  return DEM_OK;
}

int restore_state(dem_ctx* c, const Saved& s) {
  c->pcur = s.pcur;
  c->icur = s.icur;
  c->ni = s.ni;
  c->rebuilds = s.rebuilds;
  c->have_list = s.have_list;
  c->hist_valid = s.hist_valid;
  c->tune_block = s.tune_block;
  c->tune_contact_bps = s.tune_contact_bps;
  c->mul_mode = s.mul_mode;
  c->tune_int_share = s.int_share;
  c->fuse_contact = s.fuse_contact;
  if (std::memcmp(&c->prm, &s.prm, sizeof(dem_params))) {
    c->prm = s.prm;
    int rc = ext_setup_grid(c);
    if (rc) return rc;
  }
  int rc = ext_alloc_iarrays(c, c->icur, c->ni);  // a trial may have freed it (capacity only grows)
  if (rc) return rc;
  const char* p = static_cast<const char*>(s.dev);
  IArrays& I = c->I[c->icur];
  auto get = [&](void* dst, size_t b) {
    cudaMemcpyAsync(dst, p, b, cudaMemcpyDeviceToDevice, c->stream);
    p += (b + 15) & ~size_t(15);
  };
  get(c->pblock[c->pcur], pblock_bytes(c));
  get(c->own_off[c->icur], (c->n + 1) * 4);
  if (c->ni) {
    get(I.owner, c->ni * 4);
    get(I.partner, c->ni * 4);
    get(I.pid, c->ni * 8);
    get(I.meta, c->ni * 4);
    get(I.sub, c->ni * 4);
    for (int d = 0; d < 3; d++) get(I.ft[d], c->ni * 8);
    for (int d = 0; d < 3; d++) get(I.mo[d], c->ni * 8);
    get(I.damp, c->ni * 8);
  }
  DEM_CUDA_TRY(c, cudaGetLastError());
  if ((rc = launch_reverse_lists(c))) return rc;
  if ((rc = mark_records_live(c))) return rc;  // the records were not saved
  DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  c->gen++;
  return DEM_OK;
}

struct Timer {
  dem_ctx* c;
  cudaEvent_t a, b;
  explicit Timer(dem_ctx* ctx) : c(ctx) {
    cudaEventCreate(&a);
    cudaEventCreate(&b);
  }
  ~Timer() {
    cudaEventDestroy(a);
    cudaEventDestroy(b);
  }
  void start() { cudaEventRecord(a, c->stream); }
  float stop() {
    cudaEventRecord(b, c->stream);
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    return ms;
  }
};
}  // namespace
}  // namespace dem

using namespace dem;

extern "C" int dem_autotune(dem_ctx* c, int steps_per_trial, int skin_policy, dem_tune_result* out) {
  if (!c || !out || steps_per_trial < 1 || skin_policy < 0 || skin_policy > 2) return DEM_ERR_INVALID_ARG;
  if (c->poly) return c->fail(DEM_ERR_UNSUPPORTED, "the autotuner covers the fused sphere step");
  if (!c->prm.fused_step) return c->fail(DEM_ERR_STATE, "the autotuner tunes the fused step (fused_step = 1)");
  if (!c->n) return c->fail(DEM_ERR_STATE, "no particles");
  int rc;
  if (!c->have_list && (rc = ext_update_neighbors(c))) return rc;
  const bool prof = c->prof_on;
  c->prof_on = false;
  const int graph = c->prm.graph_step;
  c->prm.graph_step = 0;  // trials run the host-launched fused step (same kernels)

  // fastest particle: rebuild period of each skin
  unsigned int* d_v = nullptr;
  DEM_CUDA_TRY(c, cudaMalloc(&d_v, sizeof(unsigned int)));
  DEM_CUDA_TRY(c, cudaMemsetAsync(d_v, 0, sizeof(unsigned int), c->stream));
  k_vmax<<<c->num_sms * 4, 256, 0, c->stream>>>(c->P[c->pcur], c->n, d_v);
  unsigned int vbits = 0;
  DEM_CUDA_TRY(c, cudaMemcpyAsync(&vbits, d_v, sizeof(vbits), cudaMemcpyDeviceToHost, c->stream));
  DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  cudaFree(d_v);
  float vmax;
  std::memcpy(&vmax, &vbits, sizeof(vmax));
  const double dt = c->prm.dt;

  Saved base;
  if ((rc = save_state(c, base))) return rc;
  const double skin0 = c->prm.rcut_inc;
  const double nd0 = 2 * c->rad_max;
  const bool cohesive = c->prm.law == DEM_LAW_HOOKE_COHESIVE;
  bool periodic = false;
  if (c->systems.empty()) {
    for (int d = 0; d < 3; d++) periodic |= c->prm.periodic[d] != 0;
  } else {
    for (const dem_system& q : c->systems)
      for (int d = 0; d < 3; d++) periodic |= q.periodic[d] != 0;
  }
  // skin_policy 1: only where the skin cannot change a bit (no cohesion, no periodic
  // wrap, whose rounding depends on the rebuild step); 2: also with periodic axes
  const bool tune_skin = !cohesive && (skin_policy == 2 || (skin_policy == 1 && !periodic));
  std::vector<double> skins = {skin0};
  if (tune_skin)
    for (double f : {0.5, 1.5, 2.0, 3.0}) skins.push_back(skin0 * f);
  const double cell_factors[] = {1.0, 1.25, 1.5};
  Timer tm(c);
  int trials = 0;

  // one trial: forced rebuild (timed), then steps (timed); the state is restored after
  auto trial = [&](double skin, double cell, int block, int bps, int mode, double* cost) -> int {
    c->prm.rcut_inc = skin;
    c->prm.cell_size = cell;
    c->tune_block = block;
    c->tune_contact_bps = bps;
    c->mul_mode = mode;
    int r = ext_setup_grid(c);
    if (r) return r;
    tm.start();
    if ((r = ext_update_neighbors(c))) return r;
    const float t_reb = tm.stop();
    const uint64_t r0 = c->rebuilds;
    tm.start();
    if ((r = dem_step(c, steps_per_trial))) return r;
    const float t_steps = tm.stop();
    const uint64_t extra = c->rebuilds - r0;
    const double t_step = std::max(0.0, ((double)t_steps - (double)extra * t_reb) / steps_per_trial);
    // rebuild interval of this skin at the fastest particle's speed, at most 50
    // steps: at rest (vmax = 0, the start of a deposition) rebuild cost still counts
    const double interval =
        vmax > 0 ? std::min(50.0, std::max(1.0, 0.5 * skin / ((double)vmax * dt))) : 50.0;
    *cost = t_step + t_reb / interval;
    trials++;
    return restore_state(c, base);
  };

  double best = 1e300, before = 0;
  double best_skin = skin0, best_cell = c->prm.cell_size;
  const int mode0 = c->mul_mode;
  if ((rc = trial(skin0, c->prm.cell_size, c->tune_block, c->tune_contact_bps, mode0, &before))) return rc;
  best = before;
  for (double sk : skins)
    for (double f : cell_factors) {
      const double cell = f * (nd0 + sk);
      double cost;
      if ((rc = trial(sk, cell, c->tune_block, c->tune_contact_bps, mode0, &cost))) return rc;
      if (cost < best) {
        best = cost;
        best_skin = sk;
        best_cell = cell;
      }
    }
  int best_block = c->tune_block, best_bps = c->tune_contact_bps;
  for (int block : {64, 128, 256})
    for (int bps : {4, 8, 16}) {
      double cost;
      if ((rc = trial(best_skin, best_cell, block, bps, mode0, &cost))) return rc;
      if (cost < best) {
        best = cost;
        best_block = block;
        best_bps = bps;
      }
    }
  // multiply placement of the integration kernels (same bits in every mode)
  int best_mode = mode0;
  for (int mode : {0, 1, 2, 3}) {
    if (mode == (mode0 & 3)) continue;
    double cost;
    if ((rc = trial(best_skin, best_cell, best_block, best_bps, mode | (mode0 & 4), &cost))) return rc;
    if (cost < best) {
      best = cost;
      best_mode = mode | (mode0 & 4);
    }
  }
  {  // the contact law's multiplies
    double cost;
    const int mode = best_mode ^ 4;
    if ((rc = trial(best_skin, best_cell, best_block, best_bps, mode, &cost))) return rc;
    if (cost < best) {
      best = cost;
      best_mode = mode;
    }
  }
  bool best_fuse = c->fuse_contact;
  {  // detection and law of the compacted contact in one kernel or in two (same bits)
    double cost;
    c->fuse_contact = !best_fuse;  // the trial restores the saved value after it
    if ((rc = trial(best_skin, best_cell, best_block, best_bps, best_mode, &cost))) return rc;
    if (cost < best) {
      best = cost;
      best_fuse = !best_fuse;
    }
  }
  // (the integer-pipe share of the contact tiles, dem_set_contact_int_share, is not
  // tried: on GB300 its emulated additions made the contact kernel slower at every
  // share measured, 2/8 to 8/8)
  const int best_share = c->tune_int_share;
  cudaFree(base.dev);

  // apply: launch shapes and cell size keep the current list (they take effect at the
  // next rebuild); a new skin rebuilds now (no effect on any result without cohesion)
  c->tune_block = best_block;
  c->tune_contact_bps = best_bps;
  c->mul_mode = best_mode;
  c->fuse_contact = best_fuse;
  c->tune_int_share = best_share;
  const bool skin_changed = best_skin != skin0;
  c->prm.cell_size = best_cell;
  c->prm.rcut_inc = best_skin;
  if ((rc = ext_setup_grid(c))) return rc;
  if (skin_changed && (rc = ext_update_neighbors(c))) return rc;  // the list of the new skin
  c->prm.graph_step = graph;
  c->prof_on = prof;
  c->gen++;
  out->rcut_inc = best_skin;
  out->cell_size = best_cell;
  out->block = best_block;
  out->contact_blocks_per_sm = best_bps;
  out->ms_per_step = best;
  out->ms_per_step_before = before;
  out->trials = trials;
  out->vmax = vmax;
  out->mul_mode = best_mode;
  out->fused_contact = best_fuse ? 1 : 0;
  out->contact_int_share = best_share;
  return DEM_OK;
}
