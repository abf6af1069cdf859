// k_selftest.cu -- GPU self-test of div_rn (math_exact.cuh) against a / b.
#include "../../include/dem_selftest.h"
#include "dem_ctx.cuh"
#include "math_exact.cuh"

namespace {
__device__ __forceinline__ uint64_t mix(uint64_t x) {  // splitmix64 finaliser
  x += 0x9e3779b97f4a7c15ull;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
  return x ^ (x >> 31);
}
// random double with the given exponent window [e0, e0 + span), random sign and mantissa
__device__ __forceinline__ double draw(uint64_t h, int e0, int span) {
  const uint64_t mant = h & ((1ull << 52) - 1);
  const uint64_t e = (uint64_t)(e0 + (int)((h >> 52) % (uint64_t)span)) & 0x7ffu;
  const uint64_t sign = (h >> 63) & 1u;
  return __longlong_as_double((long long)((sign << 63) | (e << 52) | mant));
}

__global__ void k_div_test(uint64_t n, uint64_t seed, unsigned long long* bad, unsigned long long* fast) {
  unsigned long long nbad = 0, nfast = 0;
  for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t h1 = mix(seed ^ (2 * t)), h2 = mix(seed ^ (2 * t + 1));
    double a, b;
    switch (t % 4) {
      case 0:  // force- and mass-like magnitudes
        a = draw(h1, 1023 - 30, 60);
        b = fabs(draw(h2, 1023 - 20, 40));
        break;
      case 1:  // whole fast-path window
        a = draw(h1, 1023 - 499, 998);
        b = draw(h2, 1023 - 499, 998);
        break;
      case 2:  // b near powers of two (all-ones / all-zeros mantissas)
        a = draw(h1, 1023 - 10, 20);
        b = __longlong_as_double((long long)((uint64_t)(1023 + (h2 % 9) - 4) << 52 |
                                             ((h2 >> 8) & 1 ? ((1ull << 52) - 1 - (h2 >> 60)) : (h2 >> 60))));
        break;
      default:  // outside the window: fallback path
        a = draw(h1, 1, 2045);
        b = draw(h2, 1, 2045);
        break;
    }
    const double y = 1.0 / b;
    const double q1 = dem::div_rn(a, b, y);
    const double q2 = a / b;
    const bool same = __double_as_longlong(q1) == __double_as_longlong(q2) || (q1 != q1 && q2 != q2);
    nbad += same ? 0 : 1;
    nfast += (a != 0.0 && dem::exp_in_safe_range(a) && dem::exp_in_safe_range(b)) ? 1 : 0;
  }
  atomicAdd(bad, nbad);
  atomicAdd(fast, nfast);
}
}  // namespace

extern "C" int dem_selftest_division(uint64_t n, uint64_t seed, uint64_t* mismatches, uint64_t* fast_path_taken) {
  if (!mismatches || !fast_path_taken) return DEM_ERR_INVALID_ARG;
  unsigned long long* d = nullptr;
  if (cudaMalloc(&d, 2 * sizeof(unsigned long long)) != cudaSuccess) return DEM_ERR_CUDA;
  cudaMemset(d, 0, 2 * sizeof(unsigned long long));
  k_div_test<<<1216, 256>>>(n, seed, d, d + 1);
  unsigned long long h[2] = {0, 0};
  const bool ok = cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost) == cudaSuccess;
  cudaFree(d);
  if (!ok || cudaGetLastError() != cudaSuccess) return DEM_ERR_CUDA;
  *mismatches = h[0];
  *fast_path_taken = h[1];
  return DEM_OK;
}
