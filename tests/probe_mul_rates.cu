// probe_mul_rates.cu -- measurement probe (test-only translation unit, not part
// of the library): multiply throughput of the FP64 pipe, of the integer-pipe
// binary64 multiply (emu64.cuh), and of both in the same threads.  Built by
// tests/test_emu64.py into tests/_build/libdem_probe.so.
#include <cstdint>
#include <cuda_runtime.h>

#include "../exadem_gb300/csrc/emu64.cuh"

namespace {
// NN chains multiplied on the FP64 pipe and NE chains on the integer pipe,
// all in the same thread; factors alternate around 1 so values stay normal.
// The factors are kernel arguments, so no part of the emulated product is
// folded at compile time; the branch-free form is the one the integration
// kernels use.
template <int NN, int NE>
__global__ void __launch_bounds__(256) k_rate(int iters, double seed, double c1, double c2, double* out) {
  double xn[NN > 0 ? NN : 1], xe[NE > 0 ? NE : 1];
  const double base = seed + 1e-3 * (double)(threadIdx.x & 31);
#pragma unroll
  for (int k = 0; k < NN; k++) xn[k] = base + k;
#pragma unroll
  for (int k = 0; k < NE; k++) xe[k] = base - k;
  bool bad = false;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int k = 0; k < NN; k++) xn[k] = __dmul_rn(__dmul_rn(xn[k], c1), c2);
#pragma unroll
    for (int k = 0; k < NE; k++) xe[k] = dem::emu_dmul_nb(dem::emu_dmul_nb(xe[k], c1, bad), c2, bad);
  }
  double s = bad ? -1.0 : 0.0;
#pragma unroll
  for (int k = 0; k < NN; k++) s += xn[k];
#pragma unroll
  for (int k = 0; k < NE; k++) s += xe[k];
  out[(uint64_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <int NN, int NE>
int time_rate(int blocks, int iters, double* out, double* gops) {
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const double c1 = 1.0 + 1.0 / 1048576.0, c2 = 1.0 - 1.0 / 2097152.0;
  k_rate<NN, NE><<<blocks, 256>>>(iters / 8, 1.25, c1, c2, out);  // warm-up
  cudaEventRecord(e0);
  k_rate<NN, NE><<<blocks, 256>>>(iters, 1.25, c1, c2, out);
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (cudaGetLastError() != cudaSuccess) return 2;
  const double ops = 2.0 * (NN + NE) * (double)iters * (double)blocks * 256.0;
  *gops = ops / (ms * 1e-3) * 1e-9;
  return 0;
}
}  // namespace

// gops[5]: G multiplies/s for (FP64, integer) chains per thread of (4,0), (0,4), (4,4), (4,2), (2,4).
// Returns 0, 1 (bad argument) or 2 (CUDA error).
extern "C" int dem_probe_mul_rates(int iters, double* gops) {
  if (!gops || iters < 8) return 1;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = sms * 8;
  double* out = nullptr;
  if (cudaMalloc(&out, (size_t)blocks * 256 * sizeof(double)) != cudaSuccess) return 2;
  int st = time_rate<4, 0>(blocks, iters, out, &gops[0]);
  if (st == 0) st = time_rate<0, 4>(blocks, iters, out, &gops[1]);
  if (st == 0) st = time_rate<4, 4>(blocks, iters, out, &gops[2]);
  if (st == 0) st = time_rate<4, 2>(blocks, iters, out, &gops[3]);
  if (st == 0) st = time_rate<2, 4>(blocks, iters, out, &gops[4]);
  cudaFree(out);
  return st;
}
