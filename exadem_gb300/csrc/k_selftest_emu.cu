// k_selftest_emu.cu -- GPU self-tests of the integer-pipe binary64 multiply
// and addition (emu64.cuh) against the hardware multiply and addition and of the rolling-clip shortcut
// (contact_core.cuh) against the formula.
#include "../../include/dem_selftest.h"
#include "contact_core.cuh"
#include "dem_ctx.cuh"
#include "emu64.cuh"

namespace {
__device__ __forceinline__ uint64_t mix(uint64_t x) {  // splitmix64 finaliser
  x += 0x9e3779b97f4a7c15ull;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
  return x ^ (x >> 31);
}

// operand classes as in the host check: typical magnitudes, short
// significands (exact products and ties), the whole normal range, boundary
// exponents, zeros / subnormals, infinities / NaNs, all-ones significands
__device__ double draw(uint64_t h1, uint64_t h2) {
  const uint64_t sign = (h1 & 1) << 63;
  const int cls = (int)((h1 >> 1) % 16);
  uint64_t frac = h2 & 0xfffffffffffffull;
  const uint64_t r = h1 >> 8;
  uint64_t e;
  if (cls < 7) {
    e = 1023 - 60 + (r % 121);
  } else if (cls < 10) {
    const int keep = (int)(r % 12);
    frac &= ~((1ull << (52 - keep)) - 1);
    e = 1023 - 30 + ((r >> 8) % 61);
  } else if (cls < 12) {
    e = 1 + (r % 2046);
  } else if (cls == 12) {
    e = (r & 1) ? 1 + ((r >> 1) % 40) : 2046 - ((r >> 1) % 40);
  } else if (cls == 13) {
    e = 0;
    if (r & 1) frac = 0;
  } else if (cls == 14) {
    e = 2047;
    if (r & 1) frac = 0;
  } else {
    frac = (r & 1) ? 0xfffffffffffffull : 0;
    e = 1023 - 8 + ((r >> 1) % 17);
  }
  return __longlong_as_double((long long)(sign | (e << 52) | frac));
}

__device__ __forceinline__ bool same_bits(double x, double y) {
  return __double_as_longlong(x) == __double_as_longlong(y) || (x != x && y != y);
}

__global__ void k_emu_test(uint64_t n, uint64_t seed, unsigned long long* bad) {
  unsigned long long nbad = 0;
  for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t h = mix(seed ^ (4 * t));
    const double a = draw(h, mix(h ^ 1)), b = draw(mix(h ^ 2), mix(h ^ 3));
    nbad += same_bits(dem::emu_dmul(a, b), __dmul_rn(a, b)) ? 0 : 1;
    nbad += same_bits(dem::emu_mul2(a), __dmul_rn(a, 2.0)) ? 0 : 1;
    nbad += same_bits(dem::emu_mulhalf(a), __dmul_rn(a, 0.5)) ? 0 : 1;
    nbad += same_bits(dem::emu_mulnhalf(a), __dmul_rn(a, -0.5)) ? 0 : 1;
    // sums: the drawn pair, a against its negation and its neighbours, and a
    // gap of 0..70 binades between the operands
    const uint64_t ua = (uint64_t)__double_as_longlong(a), h4 = mix(h ^ 5);
    const uint64_t ea = (ua >> 52) & 0x7ff, gap = h4 % 71;
    const double pairs[4] = {b, -a, __longlong_as_double((long long)((ua ^ 0x8000000000000000ull) + (h4 % 9) - 4)),
                             __longlong_as_double((long long)(((h4 >> 8) & 1) << 63 |
                                                              ((ea > gap ? ea - gap : 1) << 52) |
                                                              (mix(h4) & 0xfffffffffffffull)))};
    for (int q = 0; q < 4; q++) {
      bool fa = false, fs = false;
      const double ga = dem::emu_dadd_nb(a, pairs[q], fa), gs = dem::emu_dsub_nb(a, pairs[q], fs);
      nbad += (fa || same_bits(ga, __dadd_rn(a, pairs[q]))) ? 0 : 1;
      nbad += (fs || same_bits(gs, __dsub_rn(a, pairs[q]))) ? 0 : 1;
    }
  }
  atomicAdd(bad, nbad);
}

// operand for the rolling-clip test: magnitudes around the range bounds of
// rolling_clip_mur0 (2^-200, 2^200, 2^500), typical values, zeros,
// subnormals, infinities and NaNs
__device__ double draw_clip(uint64_t h) {
  const uint64_t sign = (h & 1) << 63;
  const int cls = (int)((h >> 1) % 10);
  const uint64_t frac = (h >> 12) & 0xfffffffffffffull;
  const uint64_t r = h >> 5;
  uint64_t e;
  switch (cls) {
    case 0: case 1: case 2: e = 1023 - 30 + (r % 60); break;   // typical
    case 3: e = 1023 - 203 + (r % 7); break;                    // near 2^-200
    case 4: e = 1023 + 197 + (r % 7); break;                    // near 2^200
    case 5: e = 1023 + 497 + (r % 7); break;                    // near 2^500
    case 6: return __longlong_as_double((long long)sign);        // signed zero
    case 7: e = 0; break;                                       // subnormal
    case 8: e = 1 + (r % 2046); break;                          // any normal
    default: e = 2047; break;                                   // inf / NaN
  }
  return __longlong_as_double((long long)(sign | (e << 52) | frac));
}

__global__ void k_clip_test(uint64_t n, uint64_t seed, unsigned long long* bad, unsigned long long* fast) {
  unsigned long long nbad = 0, nfast = 0;
  for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t h = mix(seed ^ (16 * t));
    double v[12];
    for (int q = 0; q < 12; q++) {
      v[q] = draw_clip(h);
      h = mix(h ^ (uint64_t)(q + 1));
    }
    if ((t & 3) == 0) v[3] = v[4] = v[5] = 0.0;  // no spin: the 0/0 case
    const dem::V3 branch = dem::mk(v[0], v[1], v[2]), vrot = dem::mk(v[3], v[4], v[5]);
    const dem::V3 fn = dem::mk(v[6], v[7], v[8]);
    dem::V3 m1 = dem::mk(v[9], v[10], v[11]), m2 = m1;
    dem::rolling_clip_mur0(branch, vrot, fn, m1);
    {  // the formula of contact_force_core
      dem::V3 b = branch;
      const double r = (dem::dot(b, vrot)) / (dem::dot(vrot, vrot));
      b = b - r * vrot;
      const double mur = 0;
      const double threshold_mom = fabs(mur * dem::vnorm(b) * dem::vnorm(fn));
      const double mom_square = dem::dot(m2, m2);
      if (mom_square > 0.0 && mom_square > threshold_mom * threshold_mom)
        m2 = m2 * (threshold_mom / sqrt(mom_square));
    }
    nbad += (same_bits(m1.x, m2.x) && same_bits(m1.y, m2.y) && same_bits(m1.z, m2.z)) ? 0 : 1;
    nfast += (dem::exp_below(v[0], 200) && dem::exp_below(v[1], 200) && dem::exp_below(v[2], 200) &&
              dem::exp_below(v[6], 500) && dem::exp_below(v[7], 500) && dem::exp_below(v[8], 500) &&
              dem::exp_below(v[3], 200) && dem::exp_below(v[4], 200) && dem::exp_below(v[5], 200) &&
              (dem::exp_at_least(v[3], -200) || dem::exp_at_least(v[4], -200) || dem::exp_at_least(v[5], -200)))
                 ? 1
                 : 0;
  }
  atomicAdd(bad, nbad);
  atomicAdd(fast, nfast);
}

}  // namespace

extern "C" int dem_selftest_emu_mul(uint64_t n, uint64_t seed, uint64_t* mismatches) {
  if (!mismatches) return DEM_ERR_INVALID_ARG;
  unsigned long long* d = nullptr;
  if (cudaMalloc(&d, sizeof(unsigned long long)) != cudaSuccess) return DEM_ERR_CUDA;
  cudaMemset(d, 0, sizeof(unsigned long long));
  k_emu_test<<<1216, 256>>>(n, seed, d);
  unsigned long long h = 0;
  const bool ok = cudaMemcpy(&h, d, sizeof(h), cudaMemcpyDeviceToHost) == cudaSuccess;
  cudaFree(d);
  if (!ok || cudaGetLastError() != cudaSuccess) return DEM_ERR_CUDA;
  *mismatches = h;
  return DEM_OK;
}

extern "C" int dem_selftest_rolling_clip(uint64_t n, uint64_t seed, uint64_t* mismatches, uint64_t* fast_path_taken) {
  if (!mismatches || !fast_path_taken) return DEM_ERR_INVALID_ARG;
  unsigned long long* d = nullptr;
  if (cudaMalloc(&d, 2 * sizeof(unsigned long long)) != cudaSuccess) return DEM_ERR_CUDA;
  cudaMemset(d, 0, 2 * sizeof(unsigned long long));
  k_clip_test<<<1216, 256>>>(n, seed, d, d + 1);
  unsigned long long h[2] = {0, 0};
  const bool ok = cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost) == cudaSuccess;
  cudaFree(d);
  if (!ok || cudaGetLastError() != cudaSuccess) return DEM_ERR_CUDA;
  *mismatches = h[0];
  *fast_path_taken = h[1];
  return DEM_OK;
}
