// k_state_noalloc.cu -- the simulation_state reduction for callers that cannot allocate.
//
// Some callers of this library may not call cudaMalloc: a host framework whose
// own allocator (e.g. a caching pool) already holds the device memory it
// manages, or a code path that must not pay the implicit device
// synchronisation cudaMalloc/cudaFree can cause.  dem_simulation_state needs a
// dem_ctx (which allocates); this entry point computes the same reduction over
// particle arrays the caller already has on the device, and keeps its only
// scratch -- one partial-sum vector per thread block -- in the file-scope
// device array below, sized for DEM_STATE_NOALLOC_MAX_PARTICLES particles.
// Every GPU that loads the library holds this array until the process exits.
//
// Set-up: every call, with the device current, looks up the array's device
// address with cudaGetSymbolAddress (checked).  Looking it up each time keeps
// the address right on every device and after a cudaDeviceReset, which reloads
// the module.  The first call on a device also loads the module's device code,
// so make it before any stream capture on that device.
//
// A CUDA error still pending from earlier work of the caller is not taken as
// this call's: the call then returns DEM_ERR_CUDA without launching anything
// and leaves the error for the caller to read.
//
// Calls share the array and it keeps the last call's contents.  Every partial
// read by a call is first written by the same call, so nothing has to start at
// zero; but two calls whose kernels overlap on the GPU (different streams, no
// ordering between them) race on the array and give wrong results.
#include "dem_ctx.cuh"

namespace {
constexpr int NA_THREADS = 256;
constexpr int NA_ITEMS = 8;
constexpr uint64_t NA_TILE = (uint64_t)NA_THREADS * NA_ITEMS;  // particles per block
constexpr uint64_t NA_MAX_BLOCKS = DEM_STATE_NOALLOC_MAX_PARTICLES / NA_TILE;
static_assert(DEM_STATE_NOALLOC_MAX_PARTICLES % NA_TILE == 0, "tile must divide the maximum");

// 7 partial sums (kinetic xyz, rotation xyz, mass) per block: 448 KiB.
static __device__ __align__(256) double g_state_noalloc_partials[7 * NA_MAX_BLOCKS];

__global__ void k_na_partial(const double* __restrict__ vx, const double* __restrict__ vy,
                             const double* __restrict__ vz, const double* __restrict__ wx,
                             const double* __restrict__ wy, const double* __restrict__ wz,
                             const double* __restrict__ mass, uint64_t n, double* __restrict__ part) {
  __shared__ double sh[7][NA_THREADS];
  double acc[7] = {0, 0, 0, 0, 0, 0, 0};
  const uint64_t base = (uint64_t)blockIdx.x * NA_TILE + threadIdx.x;
#pragma unroll
  for (int k = 0; k < NA_ITEMS; k++) {
    const uint64_t s = base + (uint64_t)k * NA_THREADS;
    if (s < n) {
      const double m = mass[s];
      // ReduceSimulationStateFunctor (src/io/include/exaDEM/simulation_state.hpp:48-56)
      acc[0] += 0.5 * vx[s] * vx[s] * m;
      acc[1] += 0.5 * vy[s] * vy[s] * m;
      acc[2] += 0.5 * vz[s] * vz[s] * m;
      acc[3] += 0.5 * wx[s] * wx[s] * m;
      acc[4] += 0.5 * wy[s] * wy[s] * m;
      acc[5] += 0.5 * wz[s] * wz[s] * m;
      acc[6] += m;
    }
  }
#pragma unroll
  for (int c = 0; c < 7; c++) sh[c][threadIdx.x] = acc[c];
  __syncthreads();
  for (int w = NA_THREADS / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w)
#pragma unroll
      for (int c = 0; c < 7; c++) sh[c][threadIdx.x] += sh[c][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x < 7) part[(uint64_t)blockIdx.x * 7 + threadIdx.x] = sh[threadIdx.x][0];
}

__global__ void k_na_final(const double* __restrict__ part, uint64_t nb, double* __restrict__ out) {
  if (threadIdx.x < 7) {
    double a = 0.0;
    for (uint64_t b = 0; b < nb; b++) a += part[b * 7 + threadIdx.x];
    out[threadIdx.x] = a;
  }
}

// Device address of the scratch array on the current device.
int scratch_for_current_device(double** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return DEM_ERR_NO_DEVICE;
  double* ptr = nullptr;
  if (cudaGetSymbolAddress((void**)&ptr, g_state_noalloc_partials) != cudaSuccess || !ptr) return DEM_ERR_CUDA;
  *out = ptr;
  return DEM_OK;
}
}  // namespace

extern "C" int dem_simulation_state_noalloc(const dem_particles* dev, double* dev_out, void* stream) {
  if (!dev || !dev_out) return DEM_ERR_INVALID_ARG;
  if (dev->n > DEM_STATE_NOALLOC_MAX_PARTICLES) return DEM_ERR_INVALID_ARG;  // beyond the scratch array
  if (!dev->vx || !dev->vy || !dev->vz || !dev->vrotx || !dev->vroty || !dev->vrotz || !dev->mass)
    return DEM_ERR_INVALID_ARG;
  if (cudaPeekAtLastError() != cudaSuccess) return DEM_ERR_CUDA;  // an earlier error of the caller, left pending
  double* part = nullptr;
  int rc = scratch_for_current_device(&part);
  if (rc) return rc;
  const uint64_t n = dev->n;
  const uint64_t nb = (n + NA_TILE - 1) / NA_TILE;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (nb) {
    k_na_partial<<<(unsigned)nb, NA_THREADS, 0, st>>>(dev->vx, dev->vy, dev->vz, dev->vrotx, dev->vroty, dev->vrotz,
                                                      dev->mass, n, part);
  }
  k_na_final<<<1, 32, 0, st>>>(part, nb, dev_out);
  return cudaGetLastError() == cudaSuccess ? DEM_OK : DEM_ERR_CUDA;
}
