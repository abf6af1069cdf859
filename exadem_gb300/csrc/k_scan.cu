// k_scan.cu -- device-wide exclusive prefix sum of uint32 counts (n -> n+1 offsets).
//
// Three launches: per-tile totals, one-block scan of the tile totals, per-tile
// scan plus tile offset.  A tile is 2048 counts (512 threads x 4); the counts
// are read twice and the offsets written once.
// Integer addition is associative, so the result is deterministic.
#include "dem_ctx.cuh"

namespace dem {
namespace {
constexpr int SCAN_THREADS = 512;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

__device__ inline uint32_t warp_incl_scan(uint32_t v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += t;
  }
  return v;
}

// Block-wide exclusive scan of one value per thread; returns exclusive prefix, sets *total.
// Must be called by all threads of the block (it synchronises).
__device__ inline uint32_t block_excl_scan(uint32_t v, uint32_t* total) {
  constexpr int NW = SCAN_THREADS / 32;
  __shared__ uint32_t warp_tot[NW];
  __shared__ uint32_t s_total;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const uint32_t incl = warp_incl_scan(v);
  if (lane == 31) warp_tot[wid] = incl;
  __syncthreads();
  if (wid == 0) {
    const uint32_t w = lane < NW ? warp_tot[lane] : 0u;
    const uint32_t wi = warp_incl_scan(w);
    if (lane < NW) warp_tot[lane] = wi - w;
    if (lane == NW - 1) s_total = wi;
  }
  __syncthreads();
  const uint32_t res = incl - v + warp_tot[wid];
  if (total) *total = s_total;
  __syncthreads();  // warp_tot / s_total are reused by the next call
  return res;
}

__global__ void k_tile_sums(const uint32_t* __restrict__ in, uint64_t n, uint32_t* __restrict__ tile_sum) {
  const uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE + (uint64_t)threadIdx.x * SCAN_ITEMS;
  uint32_t s = 0;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; k++)
    if (base + k < n) s += in[base + k];
  uint32_t tot;
  block_excl_scan(s, &tot);
  if (threadIdx.x == 0) tile_sum[blockIdx.x] = tot;
}

// One block scans all tile sums in chunks (exclusive), writes the grand total to out_total.
__global__ void k_scan_tiles(uint32_t* __restrict__ tile_sum, uint64_t ntiles, uint32_t* __restrict__ out_total) {
  uint32_t carry = 0;
  for (uint64_t base = 0; base < ntiles; base += SCAN_THREADS) {
    const uint64_t t = base + threadIdx.x;
    uint32_t v = t < ntiles ? tile_sum[t] : 0u;
    uint32_t tot;
    uint32_t ex = block_excl_scan(v, &tot);
    if (t < ntiles) tile_sum[t] = ex + carry;
    carry += tot;
    __syncthreads();
  }
  if (threadIdx.x == 0) *out_total = carry;
}

__global__ void k_scan_apply(const uint32_t* __restrict__ in, uint64_t n, const uint32_t* __restrict__ tile_off,
                             uint32_t* __restrict__ out) {
  const uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE + (uint64_t)threadIdx.x * SCAN_ITEMS;
  uint32_t v[SCAN_ITEMS];
  uint32_t s = 0;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; k++) {
    v[k] = base + k < n ? in[base + k] : 0u;
    s += v[k];
  }
  uint32_t ex = block_excl_scan(s, nullptr) + tile_off[blockIdx.x];
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; k++) {
    if (base + k < n) out[base + k] = ex;
    ex += v[k];
  }
}
}  // namespace

// out has n+1 entries; out[n] = total.  in and out may not alias.
// scratch for scans of up to n elements (called before a graph capture)
int scan_reserve(dem_ctx* c, uint64_t n) {
  const uint64_t ntiles = n == 0 ? 1 : (n + SCAN_TILE - 1) / SCAN_TILE;
  if (ntiles <= c->scan_cap) return DEM_OK;
  if (c->scan_blk) cudaFree(c->scan_blk);
  c->scan_blk = nullptr;
  c->scan_cap = 0;
  DEM_CUDA_TRY(c, cudaMalloc(&c->scan_blk, ntiles * sizeof(uint32_t)));
  c->scan_cap = ntiles;
  return DEM_OK;
}

int scan_exclusive_u32(dem_ctx* c, const uint32_t* in, uint32_t* out, uint64_t n) {
  const uint64_t ntiles = n == 0 ? 1 : (n + SCAN_TILE - 1) / SCAN_TILE;
  if (ntiles > c->scan_cap) {
    if (c->scan_blk) cudaFree(c->scan_blk);
    c->scan_blk = nullptr;
    c->scan_cap = 0;
    DEM_CUDA_TRY(c, cudaMalloc(&c->scan_blk, ntiles * sizeof(uint32_t)));
    c->scan_cap = ntiles;
  }
  ProfScope ps(c, K_SCAN, 3);
  k_tile_sums<<<(unsigned)ntiles, SCAN_THREADS, 0, c->stream>>>(in, n, c->scan_blk);
  k_scan_tiles<<<1, SCAN_THREADS, 0, c->stream>>>(c->scan_blk, ntiles, out + n);
  k_scan_apply<<<(unsigned)ntiles, SCAN_THREADS, 0, c->stream>>>(in, n, c->scan_blk, out);
  DEM_CUDA_TRY(c, cudaGetLastError());
  return DEM_OK;
}
}  // namespace dem
