// dem_graph.cu -- the fused sphere step replayed as one CUDA graph.
//
// One graph replay is one Verlet iteration of the reference deck
// (data/config/main-config.msp compute_loop, numerical_scheme_verlet):
//   memset(trigger); k_fused_prolog (prolog + particle_displ_over)
//   k_set_cond: the trigger enables the conditional node
//   IF trigger: the neighbour rebuild (bin, sort, reorder, count, scan, fill
//               with history carry-over, reverse lists)
//   compacted contact law (screen, detect, Hooke); k_fused_epilog
// so a step needs no host synchronisation: dem_step replays the graph nsteps
// times and reads the device counters once at the end.
//
// A graph fixes its buffers, so inside it the particle and interaction double
// buffers do not alternate: the rebuild writes the new order and the new list
// into buffer 1 and copies them back onto buffer 0.  The interaction buffers
// have a fixed capacity; the count that exceeds it sets an overflow flag and
// leaves an empty list (every later kernel stays in bounds).  On overflow the
// call restores the state saved at its start, doubles the capacity, captures
// again and runs the steps again, so results never depend on the capacity.
#include <cstring>

#include "dem_ctx.cuh"

namespace dem {
int launch_bin_particles(dem_ctx* c);
int launch_reorder_particles(dem_ctx* c);
int launch_count_sphere(dem_ctx* c);
int launch_fill_sphere(dem_ctx* c, uint32_t* new_off, uint64_t total);
int launch_reverse_lists(dem_ctx* c);
int launch_fused_prolog(dem_ctx* c);
int launch_contact_compact(dem_ctx* c);
int launch_fused_epilog(dem_ctx* c);

namespace {
enum : int { GS_NI = 0, GS_OVERFLOW = 1, GS_REBUILDS = 2, GS_CAP = 3 };

__global__ void k_set_cond(cudaGraphConditionalHandle h, const unsigned long long* flag) {
  cudaGraphSetConditional(h, *flag ? 1u : 0u);
}

// size of the new list (exclusive scan total) against the capacity
__global__ void k_graph_total(const uint32_t* __restrict__ off_new, uint64_t n, unsigned long long* gs) {
  const unsigned long long total = off_new[n];
  if (total > gs[GS_CAP]) {
    gs[GS_OVERFLOW] = 1ull;
    gs[GS_NI] = 0ull;
  } else {
    gs[GS_NI] = total;
  }
  gs[GS_REBUILDS] += 1ull;
}

// the new list (buffer 1) onto the current one (buffer 0); empty after an overflow
__global__ void k_graph_copy_list(IArrays dst, IArrays src, const uint32_t* __restrict__ off_src,
                                  uint32_t* __restrict__ off_dst, uint64_t n, const unsigned long long* gs) {
  const bool ovf = gs[GS_OVERFLOW] != 0ull;
  const uint64_t ni = gs[GS_NI];
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t t0 = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (uint64_t s = t0; s <= n; s += stride) off_dst[s] = ovf ? 0u : off_src[s];
  for (uint64_t k = t0; k < ni; k += stride) {
    dst.owner[k] = src.owner[k];
    dst.partner[k] = src.partner[k];
    dst.pid[k] = src.pid[k];
    dst.meta[k] = src.meta[k];
    dst.sub[k] = src.sub[k];
#pragma unroll
    for (int d = 0; d < 3; d++) {
      dst.ft[d][k] = src.ft[d][k];
      dst.mo[d][k] = src.mo[d][k];
    }
    dst.damp[k] = src.damp[k];
  }
}

size_t particle_block_bytes(const dem_ctx* c) {
  return (NPF * sizeof(double) + sizeof(uint64_t) + 2 * sizeof(uint32_t)) * std::max<uint64_t>(c->pcap, 1);
}

// copies ni interactions of list `from` into list `to` (host-driven, outside capture)
int copy_list(dem_ctx* c, IArrays& to, const IArrays& from, uint64_t ni) {
  cudaStream_t st = c->stream;
  if (!ni) return DEM_OK;
  DEM_CUDA_TRY(c, cudaMemcpyAsync(to.owner, from.owner, ni * 4, cudaMemcpyDeviceToDevice, st));
  DEM_CUDA_TRY(c, cudaMemcpyAsync(to.partner, from.partner, ni * 4, cudaMemcpyDeviceToDevice, st));
  DEM_CUDA_TRY(c, cudaMemcpyAsync(to.pid, from.pid, ni * 8, cudaMemcpyDeviceToDevice, st));
  DEM_CUDA_TRY(c, cudaMemcpyAsync(to.meta, from.meta, ni * 4, cudaMemcpyDeviceToDevice, st));
  DEM_CUDA_TRY(c, cudaMemcpyAsync(to.sub, from.sub, ni * 4, cudaMemcpyDeviceToDevice, st));
  for (int d = 0; d < 3; d++) {
    DEM_CUDA_TRY(c, cudaMemcpyAsync(to.ft[d], from.ft[d], ni * 8, cudaMemcpyDeviceToDevice, st));
    DEM_CUDA_TRY(c, cudaMemcpyAsync(to.mo[d], from.mo[d], ni * 8, cudaMemcpyDeviceToDevice, st));
  }
  DEM_CUDA_TRY(c, cudaMemcpyAsync(to.damp, from.damp, ni * 8, cudaMemcpyDeviceToDevice, st));
  return DEM_OK;
}

// grows list b to hold `need` interactions, keeping its first ni entries
int grow_list_keep(dem_ctx* c, int b, uint64_t need, uint64_t keep) {
  if (need <= c->icap[b] && c->I[b].owner) return DEM_OK;
  IArrays old = c->I[b];
  const uint64_t oldcap = c->icap[b];
  c->I[b] = IArrays{};
  c->icap[b] = 0;
  int rc = ext_alloc_iarrays(c, b, need);
  if (rc) return rc;
  if (keep && oldcap) {
    if ((rc = copy_list(c, c->I[b], old, keep))) return rc;
  }
  DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  ext_free_iarrays(old);
  return DEM_OK;
}

// the rebuild as captured inside the conditional node (pcur = icur = 0 throughout)
int rebuild_body(dem_ctx* c) {
  const uint64_t n = c->n;
  int rc;
  if ((rc = launch_bin_particles(c))) return rc;
  if ((rc = launch_reorder_particles(c))) return rc;  // one system: P[0] -> P[1], swapped
  if (c->pcur != 0) {                                   // (several systems reorder in place)
    DEM_CUDA_TRY(c, cudaMemcpyAsync(c->pblock[0], c->pblock[1], particle_block_bytes(c), cudaMemcpyDeviceToDevice,
                                    c->stream));
    c->pcur = 0;
  }
  if ((rc = launch_count_sphere(c))) return rc;
  if ((rc = scan_exclusive_u32(c, c->pcnt, c->own_off[1], n))) return rc;
  k_graph_total<<<1, 1, 0, c->stream>>>(c->own_off[1], n, c->d_gs);
  if ((rc = launch_fill_sphere(c, c->own_off[1], 0))) return rc;  // into I[1], history from I[0]
  k_graph_copy_list<<<(unsigned)c->num_sms * 4u, 256, 0, c->stream>>>(c->I[0], c->I[1], c->own_off[1], c->own_off[0],
                                                                       n, c->d_gs);
  DEM_CUDA_TRY(c, cudaGetLastError());
  if ((rc = launch_reverse_lists(c))) return rc;
  if ((rc = mark_records_live(c))) return rc;  // new list indices: every record is stale
  DEM_CUDA_TRY(c, cudaMemsetAsync(c->trig_dev, 0, c->nsys * sizeof(uint32_t), c->stream));
  return DEM_OK;
}

void destroy_graph(dem_ctx* c) {
  if (c->gexec) cudaGraphExecDestroy(c->gexec);
  if (c->graph) cudaGraphDestroy(c->graph);
  c->gexec = nullptr;
  c->graph = nullptr;
}

int build_graph(dem_ctx* c) {
  destroy_graph(c);
  cudaStream_t st = c->stream;
  int rc;
  // fixed buffers: current particles in P[0], current list in I[0]
  if (c->pcur != 0) {
    DEM_CUDA_TRY(c, cudaMemcpyAsync(c->pblock[0], c->pblock[1], particle_block_bytes(c), cudaMemcpyDeviceToDevice, st));
    c->pcur = 0;
  }
  // the requested capacity, at least the current list (the rebuilt one may overflow it)
  const uint64_t cap = c->gcap ? std::max<uint64_t>(c->gcap, c->ni + 1) : 2 * c->ni + 4096;
  if ((rc = grow_list_keep(c, 0, cap, c->icur == 0 ? c->ni : 0))) return rc;
  if (c->icur != 0) {
    if ((rc = copy_list(c, c->I[0], c->I[1], c->ni))) return rc;
    DEM_CUDA_TRY(c, cudaMemcpyAsync(c->own_off[0], c->own_off[1], (c->n + 1) * 4, cudaMemcpyDeviceToDevice, st));
    c->icur = 0;
  }
  if ((rc = grow_list_keep(c, 1, cap, 0))) return rc;
  if ((rc = ext_alloc_records(c, cap))) return rc;  // records, compaction lists and partner lists
  if ((rc = launch_reverse_lists(c))) return rc;  // the partner lists were reallocated
  c->gcap = std::min(std::min(c->icap[0], c->icap[1]), c->rcap);
  // scan scratch for the largest scan of the step (no allocation inside a capture)
  if ((rc = scan_reserve(c, std::max<uint64_t>(c->ncell, c->n)))) return rc;
  if (!c->d_gs) DEM_CUDA_TRY(c, cudaMalloc(&c->d_gs, 4 * sizeof(unsigned long long)));
  c->d_ni = c->d_gs;
  const unsigned long long gs0[4] = {c->ni, 0ull, 0ull, c->gcap};
  DEM_CUDA_TRY(c, cudaMemcpyAsync(c->d_gs, gs0, sizeof(gs0), cudaMemcpyHostToDevice, st));
  DEM_CUDA_TRY(c, cudaStreamSynchronize(st));

  std::memset(c->graph_launches_per_step, 0, sizeof(c->graph_launches_per_step));
  std::memset(c->graph_launches_per_rebuild, 0, sizeof(c->graph_launches_per_rebuild));
  cudaGraph_t g = nullptr;
  DEM_CUDA_TRY(c, cudaGraphCreate(&g, 0));
  c->graph = g;
  cudaGraphConditionalHandle h;
  DEM_CUDA_TRY(c, cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault));
  c->capturing = true;
  // part 1: prolog + trigger + condition
  cudaGraphNode_t last = nullptr;
  {
    DEM_CUDA_TRY(c, cudaStreamBeginCaptureToGraph(st, g, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    rc = launch_fused_prolog(c);
    if (!rc) {
      k_set_cond<<<1, 1, 0, st>>>(h, c->d_scalars);
      c->graph_launches_per_step[K_PROLOG] += 1;
    }
    cudaStreamCaptureStatus status;
    const cudaGraphNode_t* deps = nullptr;
    size_t ndeps = 0;
    if (!rc && cudaStreamGetCaptureInfo(st, &status, nullptr, nullptr, &deps, nullptr, &ndeps) == cudaSuccess &&
        ndeps == 1)
      last = deps[0];
    cudaGraph_t out = nullptr;
    const cudaError_t e = cudaStreamEndCapture(st, &out);
    if (rc || e != cudaSuccess || !last) {
      c->capturing = false;
      return rc ? rc : c->fail(DEM_ERR_CUDA, "graph capture of the prolog failed");
    }
  }
  // part 2: the conditional rebuild
  cudaGraphNodeParams cp{};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = h;
  cp.conditional.type = cudaGraphCondTypeIf;
  cp.conditional.size = 1;
  cudaGraphNode_t cn = nullptr;
  if (cudaGraphAddNode(&cn, g, &last, nullptr, 1, &cp) != cudaSuccess) {
    c->capturing = false;
    return c->fail(DEM_ERR_CUDA, "conditional graph node not available");
  }
  {
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    DEM_CUDA_TRY(c, cudaStreamBeginCaptureToGraph(st, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    c->capturing_body = true;
    rc = rebuild_body(c);
    c->capturing_body = false;
    cudaGraph_t out = nullptr;
    const cudaError_t e = cudaStreamEndCapture(st, &out);
    if (rc || e != cudaSuccess) {
      c->capturing = false;
      return rc ? rc : c->fail(DEM_ERR_CUDA, "graph capture of the rebuild failed");
    }
  }
  // part 3: contact + epilog after the conditional node
  {
    DEM_CUDA_TRY(c, cudaStreamBeginCaptureToGraph(st, g, &cn, nullptr, 1, cudaStreamCaptureModeThreadLocal));
    rc = launch_contact_compact(c);
    if (!rc) rc = launch_fused_epilog(c);
    cudaGraph_t out = nullptr;
    const cudaError_t e = cudaStreamEndCapture(st, &out);
    c->capturing = false;
    if (rc || e != cudaSuccess) return rc ? rc : c->fail(DEM_ERR_CUDA, "graph capture of the contact step failed");
  }
  DEM_CUDA_TRY(c, cudaGraphInstantiate(&c->gexec, g, 0));
  c->graph_gen = c->gen;
  return DEM_OK;
}

// state needed to run the steps of one call again: particles, list, offsets
int snapshot(dem_ctx* c, bool save) {
  const size_t pb = particle_block_bytes(c);
  const uint64_t ni = c->ni, n = c->n;
  const size_t need = pb + (size_t)ni * 80 + (n + 1) * 4 + 256;
  if (save && need > c->snap_bytes) {
    cudaFree(c->snap);
    c->snap = nullptr;
    c->snap_bytes = 0;
    DEM_CUDA_TRY(c, cudaMalloc(&c->snap, need + need / 4));
    c->snap_bytes = need + need / 4;
  }
  char* p = static_cast<char*>(c->snap);
  const cudaMemcpyKind k = cudaMemcpyDeviceToDevice;
  cudaStream_t st = c->stream;
  auto mv = [&](void* dev, size_t bytes) -> cudaError_t {
    const cudaError_t e = save ? cudaMemcpyAsync(p, dev, bytes, k, st) : cudaMemcpyAsync(dev, p, bytes, k, st);
    p += (bytes + 15) & ~size_t(15);
    return e;
  };
  IArrays& I = c->I[0];
  DEM_CUDA_TRY(c, mv(c->pblock[0], pb));
  DEM_CUDA_TRY(c, mv(c->own_off[0], (n + 1) * 4));
  if (ni) {
    DEM_CUDA_TRY(c, mv(I.owner, ni * 4));
    DEM_CUDA_TRY(c, mv(I.partner, ni * 4));
    DEM_CUDA_TRY(c, mv(I.pid, ni * 8));
    DEM_CUDA_TRY(c, mv(I.meta, ni * 4));
    DEM_CUDA_TRY(c, mv(I.sub, ni * 4));
    for (int d = 0; d < 3; d++) {
      DEM_CUDA_TRY(c, mv(I.ft[d], ni * 8));
      DEM_CUDA_TRY(c, mv(I.mo[d], ni * 8));
    }
    DEM_CUDA_TRY(c, mv(I.damp, ni * 8));
  }
  return DEM_OK;
}
}  // namespace

void free_graph(dem_ctx* c) {
  destroy_graph(c);
  cudaFree(c->d_gs);
  cudaFree(c->snap);
  c->d_gs = c->d_ni = nullptr;
  c->snap = nullptr;
  c->snap_bytes = 0;
}

// dem_step with graph_step: nsteps replays; on an interaction-buffer overflow
// the state is restored, the capacity doubled and the steps run again.
int step_graph(dem_ctx* c, int nsteps) {
  int rc;
  for (int attempt = 0; attempt < 4; attempt++) {
    if (!c->gexec || c->graph_gen != c->gen || c->pcur != 0 || c->icur != 0) {
      if ((rc = build_graph(c))) return rc;
    }
    const uint64_t ni0 = c->ni;
    if ((rc = snapshot(c, true))) return rc;
    unsigned long long gs[4] = {c->ni, 0ull, 0ull, c->gcap};
    DEM_CUDA_TRY(c, cudaMemcpyAsync(c->d_gs, gs, sizeof(gs), cudaMemcpyHostToDevice, c->stream));
    for (int s = 0; s < nsteps; s++) DEM_CUDA_TRY(c, cudaGraphLaunch(c->gexec, c->stream));
    DEM_CUDA_TRY(c, cudaMemcpyAsync(gs, c->d_gs, sizeof(gs), cudaMemcpyDeviceToHost, c->stream));
    DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    if (!gs[GS_OVERFLOW]) {
      c->ni = gs[GS_NI];
      c->rebuilds += gs[GS_REBUILDS];
      for (int k = 0; k < K_NCLASS; k++)
        c->launches[k] += c->graph_launches_per_step[k] * (uint64_t)nsteps +
                          c->graph_launches_per_rebuild[k] * gs[GS_REBUILDS];
      return DEM_OK;
    }
    // overflow: back to the state of the call's start, twice the capacity
    c->ni = ni0;
    if ((rc = snapshot(c, false))) return rc;
    if ((rc = launch_reverse_lists(c))) return rc;
    if ((rc = mark_records_live(c))) return rc;  // the records were not saved
    DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    c->gcap = 2 * c->gcap;
    destroy_graph(c);
  }
  return c->fail(DEM_ERR_OVERFLOW, "interaction buffer kept overflowing in the graph step");
}
}  // namespace dem
