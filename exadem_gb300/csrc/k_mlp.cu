// k_mlp.cu -- the learned part: a 16 -> 64 -> 64 -> 4 MLP that predicts, for a
// candidate polyhedron pair, its number of vertex-vertex, vertex-edge,
// vertex-face and edge-edge feature contacts.  No reference counterpart.
//
// Arithmetic: BF16 inputs and weights, FP32 accumulation.  Inference (the
// rates a rebuild sizes its records with, dem_mlp_forward) runs on the
// tcgen05 tensor cores with TMEM accumulators, 128 samples per CTA tile
// (k_mlp_infer_tc).  Training keeps warp-level mma.m16n8k16 products: a warp
// owns 16 gathered samples, the FP32 result fragments of one layer are, element
// for element, the A fragments of the next layer's product, and the forward and
// backward chain of a tile stays in registers.
// Weight gradients are split-K reductions over the batch (FP32 FMA, fixed
// order, deterministic), then Adam (FP32 master weights, BF16 copies).
// Loss: Poisson with log link, rate = exp(z), loss = mean(exp(z) - y z).
//
// Parameter vector (FP32 master, DEM_MLP_NPARAM): W1[64][16], b1[64],
// W2[64][64], b2[64], W3[4][64], b3[4]  (y = W x + b, rows = outputs).
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <random>
#include <vector>

#include "../../include/dem_learned.h"
#include "dem_ctx.cuh"

namespace dem {
namespace {
constexpr int NIN = DEM_MLP_IN, NH = DEM_MLP_HID, NOUT = DEM_MLP_OUT;
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + NH * NIN, OFF_W2 = OFF_B1 + NH, OFF_B2 = OFF_W2 + NH * NH,
              OFF_W3 = OFF_B2 + NH, OFF_B3 = OFF_W3 + NOUT * NH, NPARAM = OFF_B3 + NOUT;
static_assert(NPARAM == DEM_MLP_NPARAM, "parameter layout");

// BF16 weights as the kernels read them: W1b[64][16], W2b[64][64], W3b[8][64]
// (rows 4..7 zero), and transposed W2t[64][64] (= W2^T), W3t[64][8].
struct MlpWeights {
  __nv_bfloat16 w1[NH * NIN];
  __nv_bfloat16 w2[NH * NH];
  __nv_bfloat16 w2t[NH * NH];
  __nv_bfloat16 w3[8 * NH];
  __nv_bfloat16 w3t[NH * 8];
  float b1[NH], b2[NH], b3[8];
};

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t*>(&v);
}
__device__ __forceinline__ uint32_t ld_pair(const __nv_bfloat16* p) { return *reinterpret_cast<const uint32_t*>(p); }
__device__ __forceinline__ uint32_t ld_two(const __nv_bfloat16* lo, const __nv_bfloat16* hi) {
  const uint16_t a = *reinterpret_cast<const uint16_t*>(lo), b = *reinterpret_cast<const uint16_t*>(hi);
  return (uint32_t)a | ((uint32_t)b << 16);
}

// D = A (16x16 bf16, row) * B (16x8 bf16, col) + C (16x8 f32)
__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Fragment coordinates (lane = 4 g + t): C/D element e of n-tile j is at row
// g + 8 (e >> 1), column 8 j + 2 t + (e & 1).  A fragment k-step s: a[0] =
// (g, 16s+2t..+1), a[1] = (g+8, 16s+2t..+1), a[2] = (g, 16s+8+2t..+1),
// a[3] = (g+8, 16s+8+2t..+1): n-tiles 2s and 2s+1 of the previous result.
struct Tile64 {
  float c[8][4];  // 16 x 64 result, n-tiles 0..7
};

__device__ __forceinline__ void to_afrag(const Tile64& h, int s, uint32_t (&a)[4]) {
  a[0] = pack_bf16(h.c[2 * s][0], h.c[2 * s][1]);
  a[1] = pack_bf16(h.c[2 * s][2], h.c[2 * s][3]);
  a[2] = pack_bf16(h.c[2 * s + 1][0], h.c[2 * s + 1][1]);
  a[3] = pack_bf16(h.c[2 * s + 1][2], h.c[2 * s + 1][3]);
}

// forward of one 16-sample tile: x (16 x 16 floats, rows r0 .. r0+15) -> h1, h2, z
__device__ __forceinline__ void forward_tile(const MlpWeights& w, const float* __restrict__ X, uint64_t r0,
                                             uint64_t n, int g, int t, uint32_t (&ax)[4], Tile64& h1, Tile64& h2,
                                             float (&z)[4]) {
  auto xv = [&](int row, int col) -> float {
    const uint64_t r = r0 + row;
    return r < n ? X[r * NIN + col] : 0.f;
  };
  ax[0] = pack_bf16(xv(g, 2 * t), xv(g, 2 * t + 1));
  ax[1] = pack_bf16(xv(g + 8, 2 * t), xv(g + 8, 2 * t + 1));
  ax[2] = pack_bf16(xv(g, 2 * t + 8), xv(g, 2 * t + 9));
  ax[3] = pack_bf16(xv(g + 8, 2 * t + 8), xv(g + 8, 2 * t + 9));
#pragma unroll
  for (int j = 0; j < 8; j++) {
    const int o = 8 * j + g;  // output unit of this lane's B column
    float d[4] = {0.f, 0.f, 0.f, 0.f};
    mma16816(d, ax, ld_pair(&w.w1[o * NIN + 2 * t]), ld_pair(&w.w1[o * NIN + 2 * t + 8]));
    const float bl = w.b1[8 * j + 2 * t], bh = w.b1[8 * j + 2 * t + 1];
    h1.c[j][0] = fmaxf(d[0] + bl, 0.f);
    h1.c[j][1] = fmaxf(d[1] + bh, 0.f);
    h1.c[j][2] = fmaxf(d[2] + bl, 0.f);
    h1.c[j][3] = fmaxf(d[3] + bh, 0.f);
  }
  uint32_t a[4][4];
#pragma unroll
  for (int s = 0; s < 4; s++) to_afrag(h1, s, a[s]);
#pragma unroll
  for (int j = 0; j < 8; j++) {
    const int o = 8 * j + g;
    float d[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int s = 0; s < 4; s++)
      mma16816(d, a[s], ld_pair(&w.w2[o * NH + 16 * s + 2 * t]), ld_pair(&w.w2[o * NH + 16 * s + 8 + 2 * t]));
    const float bl = w.b2[8 * j + 2 * t], bh = w.b2[8 * j + 2 * t + 1];
    h2.c[j][0] = fmaxf(d[0] + bl, 0.f);
    h2.c[j][1] = fmaxf(d[1] + bh, 0.f);
    h2.c[j][2] = fmaxf(d[2] + bl, 0.f);
    h2.c[j][3] = fmaxf(d[3] + bh, 0.f);
  }
#pragma unroll
  for (int s = 0; s < 4; s++) to_afrag(h2, s, a[s]);
  float d[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
  for (int s = 0; s < 4; s++)
    mma16816(d, a[s], ld_pair(&w.w3[g * NH + 16 * s + 2 * t]), ld_pair(&w.w3[g * NH + 16 * s + 8 + 2 * t]));
  // columns 2t, 2t+1: outputs 0..3 live on t = 0, 1
  z[0] = d[0] + w.b3[2 * t];
  z[1] = d[1] + w.b3[2 * t + 1];
  z[2] = d[2] + w.b3[2 * t];
  z[3] = d[3] + w.b3[2 * t + 1];
}

// ---- inference on the 5th-generation tensor cores (tcgen05, TMEM accumulators)
// A CTA of 128 threads runs 128 samples per tile: each layer is one
// tcgen05.mma (K = 16 per instruction, so 1 + 4 + 4 instructions) issued by one
// thread, with the operands in shared memory in the canonical K-major layout
// without swizzling (8 x 16-byte core matrices: 128 B each, K-neighbours 128 B
// apart, 8-row groups K/8 x 128 B apart) and the FP32 accumulator in TMEM
// (lane = sample, column = unit).  Completion is signalled by tcgen05.commit on
// an mbarrier; each warp reads its 32 lanes back with tcgen05.ld, adds the bias,
// applies ReLU and writes the BF16 activations as the next layer's A operand.
// Same rounding points as the training pass (BF16 inputs, weights and
// activations, FP32 accumulation and bias).
constexpr int TC_M = 128;
constexpr uint32_t TC_COLS = 128;  // TMEM columns: 0..63 layers 1-2, 64..79 layer 3

struct alignas(1024) TcSmem {
  __nv_bfloat16 x[TC_M * NIN];  // A, layer 1 (K = 16)
  __nv_bfloat16 h[TC_M * NH];   // A, layers 2 and 3 (K = 64)
  __nv_bfloat16 w1[NH * NIN];   // B, layer 1 (N = 64, K = 16)
  __nv_bfloat16 w2[NH * NH];    // B, layer 2 (N = 64, K = 64)
  __nv_bfloat16 w3[16 * NH];    // B, layer 3 (N = 16; rows 4..15 zero)
  float b1[NH], b2[NH], b3[16];
  uint64_t mbar;
  uint32_t tmem;
};

// byte offset of element (row, k) of a K-major matrix with K columns
__device__ __forceinline__ uint32_t kmajor_off(int row, int k, int K) {
  return (uint32_t)((row >> 3) * (K / 8) * 128 + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2);
}
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
// shared-memory matrix descriptor: start, leading (K) byte offset, stride (8-row
// group) byte offset, descriptor version 1, no swizzling
__device__ __forceinline__ uint64_t sm_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
         (1ull << 46);
}
// instruction descriptor, kind::f16: FP32 D, BF16 A and B, both K-major, M = 128
__host__ __device__ constexpr uint32_t tc_idesc(uint32_t n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((n >> 3) << 17) | ((128u >> 4) << 24);
}
__device__ __forceinline__ void tc_mma(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc));
}
__device__ __forceinline__ void tc_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
// waits for phase `ph` of the mbarrier, at most about a second of SM clocks
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t ph) {
  const long long t0 = clock64();
  for (;;) {
    uint32_t done;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(mbar), "r"(ph)
        : "memory");
    if (done) return true;
    if (clock64() - t0 > (1ll << 31)) return false;
  }
}
// 16 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}
// this thread's row of a 64-unit layer: bias, ReLU, BF16 into h (K-major, K = 64)
__device__ __forceinline__ void tc_hidden(TcSmem& S, uint32_t taddr, const float* b, int row) {
  uint8_t* hb = reinterpret_cast<uint8_t*>(S.h);
#pragma unroll
  for (int c0 = 0; c0 < NH; c0 += 16) {
    float v[16];
    tmem_ld16(taddr + (uint32_t)c0, v);
#pragma unroll
    for (int q = 0; q < 16; q += 8) {
      uint4 pk;
      pk.x = pack_bf16(fmaxf(v[q] + b[c0 + q], 0.f), fmaxf(v[q + 1] + b[c0 + q + 1], 0.f));
      pk.y = pack_bf16(fmaxf(v[q + 2] + b[c0 + q + 2], 0.f), fmaxf(v[q + 3] + b[c0 + q + 3], 0.f));
      pk.z = pack_bf16(fmaxf(v[q + 4] + b[c0 + q + 4], 0.f), fmaxf(v[q + 5] + b[c0 + q + 5], 0.f));
      pk.w = pack_bf16(fmaxf(v[q + 6] + b[c0 + q + 6], 0.f), fmaxf(v[q + 7] + b[c0 + q + 7], 0.f));
      *reinterpret_cast<uint4*>(hb + kmajor_off(row, c0 + q, NH)) = pk;
    }
  }
}

__global__ void __launch_bounds__(TC_M, 1) k_mlp_infer_tc(const MlpWeights* __restrict__ wg,
                                                          const float* __restrict__ X, uint64_t n,
                                                          float* __restrict__ rates, uint32_t* __restrict__ err) {
  __shared__ TcSmem S;
  const int tid = threadIdx.x, warp = tid >> 5;
  // weights into the K-major layouts, biases; the mbarrier; TMEM
  for (int i = tid; i < NH * NIN; i += TC_M) {
    const int o = i / NIN, k = i % NIN;
    *reinterpret_cast<__nv_bfloat16*>(reinterpret_cast<uint8_t*>(S.w1) + kmajor_off(o, k, NIN)) = wg->w1[i];
  }
  for (int i = tid; i < NH * NH; i += TC_M) {
    const int o = i / NH, k = i % NH;
    *reinterpret_cast<__nv_bfloat16*>(reinterpret_cast<uint8_t*>(S.w2) + kmajor_off(o, k, NH)) = wg->w2[i];
  }
  for (int i = tid; i < 16 * NH; i += TC_M) {
    const int o = i / NH, k = i % NH;
    *reinterpret_cast<__nv_bfloat16*>(reinterpret_cast<uint8_t*>(S.w3) + kmajor_off(o, k, NH)) =
        o < 8 ? wg->w3[i] : __float2bfloat16_rn(0.f);
  }
  for (int i = tid; i < NH; i += TC_M) {
    S.b1[i] = wg->b1[i];
    S.b2[i] = wg->b2[i];
  }
  if (tid < 16) S.b3[tid] = tid < 8 ? wg->b3[tid] : 0.f;
  const uint32_t mbar = smem_u32(&S.mbar);
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&S.tmem)),
                 "r"(TC_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = S.tmem;
  const uint32_t lane_base = (uint32_t)(warp * 32) << 16;  // this warp's TMEM lanes
  const uint32_t ax = smem_u32(S.x), ah = smem_u32(S.h);
  const uint32_t bw1 = smem_u32(S.w1), bw2 = smem_u32(S.w2), bw3 = smem_u32(S.w3);
  uint32_t ph = 0;
  bool bad = false;
  for (uint64_t r0 = (uint64_t)blockIdx.x * TC_M; r0 < n && !bad; r0 += (uint64_t)gridDim.x * TC_M) {
    // this thread's sample: row tid of the tile
    {
      const uint64_t r = r0 + (uint64_t)tid;
      uint8_t* xb = reinterpret_cast<uint8_t*>(S.x);
#pragma unroll
      for (int q = 0; q < NIN; q += 8) {
        float v[8];
#pragma unroll
        for (int e = 0; e < 8; e++) v[e] = r < n ? X[r * NIN + q + e] : 0.f;
        uint4 pk;
        pk.x = pack_bf16(v[0], v[1]);
        pk.y = pack_bf16(v[2], v[3]);
        pk.z = pack_bf16(v[4], v[5]);
        pk.w = pack_bf16(v[6], v[7]);
        *reinterpret_cast<uint4*>(xb + kmajor_off(tid, q, NIN)) = pk;
      }
    }
    for (int layer = 0; layer < 3; layer++) {
      fence_async_smem();
      tc_fence_before();
      __syncthreads();
      tc_fence_after();
      if (tid == 0) {
        if (layer == 0) {
          tc_mma(tmem, sm_desc(ax, 128, 256), sm_desc(bw1, 128, 256), tc_idesc(64), 0u);
        } else {
#pragma unroll
          for (int s = 0; s < NH / 16; s++)
            tc_mma(tmem + (layer == 2 ? 64u : 0u), sm_desc(ah + 256u * s, 128, 1024),
                   sm_desc((layer == 1 ? bw2 : bw3) + 256u * s, 128, 1024), tc_idesc(layer == 1 ? 64 : 16),
                   s ? 1u : 0u);
        }
        tc_commit(mbar);
      }
      const bool ok = mbar_wait(mbar, ph);
      ph ^= 1u;
      if (__syncthreads_or(!ok)) {
        bad = true;
        break;
      }
      tc_fence_after();
      if (layer < 2) {
        tc_hidden(S, tmem + lane_base, layer == 0 ? S.b1 : S.b2, tid);
      } else {
        float v[16];
        tmem_ld16(tmem + lane_base + 64u, v);
        const uint64_t r = r0 + (uint64_t)tid;
        if (r < n) {
#pragma unroll
          for (int o = 0; o < NOUT; o++) rates[r * NOUT + o] = expf(v[o] + S.b3[o]);
        }
      }
    }
  }
  if (bad && tid == 0) atomicOr(err, 1u);
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_COLS) : "memory");
  }
}

// Training pass over a batch: forward, Poisson loss, backward through the
// activations.  Writes per sample (BF16): x, h1, h2, dh1, dh2 and dz (FP32) for
// the weight gradients, and one loss partial per block.
__global__ void __launch_bounds__(128) k_mlp_fwd_bwd(const MlpWeights* __restrict__ wg, const float* __restrict__ X,
                                                      const uint8_t* __restrict__ Y, const uint32_t* __restrict__ idx,
                                                      uint64_t n, float scale, __nv_bfloat16* __restrict__ xb,
                                                      __nv_bfloat16* __restrict__ h1b, __nv_bfloat16* __restrict__ h2b,
                                                      __nv_bfloat16* __restrict__ dh1b,
                                                      __nv_bfloat16* __restrict__ dh2b, float* __restrict__ dzf,
                                                      double* __restrict__ loss_part) {
  __shared__ MlpWeights w;
  __shared__ float xs[4][16 * NIN];  // the warp's gathered samples
  __shared__ double lsum[4];
  for (int i = threadIdx.x; i < (int)(sizeof(MlpWeights) / 4); i += blockDim.x)
    reinterpret_cast<uint32_t*>(&w)[i] = reinterpret_cast<const uint32_t*>(wg)[i];
  __syncthreads();
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3, wib = threadIdx.x >> 5;
  const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  double loss = 0.0;
  for (uint64_t r0 = warp * 16; r0 < n; r0 += nwarps * 16) {
    // gather the tile's samples (batch row r -> dataset row idx[r])
    for (int e = lane; e < 16 * NIN; e += 32) {
      const uint64_t r = r0 + e / NIN;
      xs[wib][e] = r < n ? X[(uint64_t)idx[r] * NIN + e % NIN] : 0.f;
    }
    __syncwarp();
    uint32_t ax[4];
    Tile64 h1, h2;
    float z[4];
    forward_tile(w, xs[wib], 0, 16, g, t, ax, h1, h2, z);
    // loss and dL/dz on the valid outputs (t < 2), zero elsewhere
    float dz[4];
#pragma unroll
    for (int e = 0; e < 4; e++) {
      const uint64_t r = r0 + g + 8 * (e >> 1);
      const int o = 2 * t + (e & 1);
      dz[e] = 0.f;
      if (t < 2 && r < n) {
        const float y = (float)Y[(uint64_t)idx[r] * NOUT + o];
        const float lam = expf(z[e]);
        loss += (double)(lam - y * z[e]);
        dz[e] = (lam - y) * scale;
        dzf[r * NOUT + o] = dz[e];
      }
    }
    // dh2 = dz W3 (contraction over the 8 padded outputs), masked by h2 > 0
    uint32_t adz[4] = {pack_bf16(dz[0], dz[1]), pack_bf16(dz[2], dz[3]), 0u, 0u};
    Tile64 d2;
#pragma unroll
    for (int j = 0; j < 8; j++) {
      const int hcol = 8 * j + g;  // hidden unit of this lane's B column
      float d[4] = {0.f, 0.f, 0.f, 0.f};
      mma16816(d, adz, ld_pair(&w.w3t[hcol * 8 + 2 * t]), 0u);
#pragma unroll
      for (int e = 0; e < 4; e++) d2.c[j][e] = h2.c[j][e] > 0.f ? d[e] : 0.f;
    }
    // dh1 = dh2 W2, masked by h1 > 0
    uint32_t a[4][4];
#pragma unroll
    for (int s = 0; s < 4; s++) to_afrag(d2, s, a[s]);
    Tile64 d1;
#pragma unroll
    for (int j = 0; j < 8; j++) {
      const int i = 8 * j + g;  // layer-1 unit of this lane's B column
      float d[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
      for (int s = 0; s < 4; s++)
        mma16816(d, a[s], ld_pair(&w.w2t[i * NH + 16 * s + 2 * t]), ld_pair(&w.w2t[i * NH + 16 * s + 8 + 2 * t]));
#pragma unroll
      for (int e = 0; e < 4; e++) d1.c[j][e] = h1.c[j][e] > 0.f ? d[e] : 0.f;
    }
    // store the tile (BF16 as the products saw them)
#pragma unroll
    for (int j = 0; j < 8; j++)
#pragma unroll
      for (int hf = 0; hf < 2; hf++) {
        const uint64_t r = r0 + g + 8 * hf;
        if (r >= n) continue;
        const uint64_t o = r * NH + 8 * j + 2 * t;
        *reinterpret_cast<uint32_t*>(&h1b[o]) = pack_bf16(h1.c[j][2 * hf], h1.c[j][2 * hf + 1]);
        *reinterpret_cast<uint32_t*>(&h2b[o]) = pack_bf16(h2.c[j][2 * hf], h2.c[j][2 * hf + 1]);
        *reinterpret_cast<uint32_t*>(&dh1b[o]) = pack_bf16(d1.c[j][2 * hf], d1.c[j][2 * hf + 1]);
        *reinterpret_cast<uint32_t*>(&dh2b[o]) = pack_bf16(d2.c[j][2 * hf], d2.c[j][2 * hf + 1]);
      }
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const uint64_t r = r0 + g + 8 * (q & 1);
      const int col = 2 * t + 8 * (q >> 1);
      if (r < n) *reinterpret_cast<uint32_t*>(&xb[r * NIN + col]) = ax[q];
    }
    __syncwarp();
  }
  // deterministic loss partial: lanes in order, then warps in order
  for (int o = 16; o; o >>= 1) loss += __shfl_down_sync(0xffffffffu, loss, o);
  if (lane == 0) lsum[wib] = loss;
  __syncthreads();
  if (threadIdx.x == 0) loss_part[blockIdx.x] = lsum[0] + lsum[1] + lsum[2] + lsum[3];
}

// Split-K weight gradients: block b sums rows [b*chunk, (b+1)*chunk) in order.
// dW1 = dh1^T x, dW2 = dh2^T h1, dW3 = dz^T h2, db1 = sum dh1, db2 = sum dh2, db3 = sum dz.
constexpr int GT = 256, GROWS = 32;
__global__ void __launch_bounds__(GT) k_mlp_wgrad(const __nv_bfloat16* __restrict__ xb,
                                                  const __nv_bfloat16* __restrict__ h1b,
                                                  const __nv_bfloat16* __restrict__ h2b,
                                                  const __nv_bfloat16* __restrict__ dh1b,
                                                  const __nv_bfloat16* __restrict__ dh2b,
                                                  const float* __restrict__ dzf, uint64_t n, uint64_t chunk,
                                                  float* __restrict__ part) {
  __shared__ float sx[GROWS][NIN], sh1[GROWS][NH], sh2[GROWS][NH], sd1[GROWS][NH], sd2[GROWS][NH], sdz[GROWS][NOUT];
  const int tid = threadIdx.x;
  // outputs of this thread: dW2 row o2 = tid / 4, columns 16 (tid % 4) .. +16;
  // dW1 row tid / 4, columns 4 (tid % 4) .. +4; dW3 entry tid (o = tid / 64, i = tid % 64);
  // biases: tid < 64 -> db1, 64..127 -> db2, 128..131 -> db3
  const int o2 = tid >> 2, c2 = (tid & 3) * 16, c1 = (tid & 3) * 4;
  float aw2[16], aw1[4], aw3 = 0.f, ab = 0.f;
#pragma unroll
  for (int q = 0; q < 16; q++) aw2[q] = 0.f;
#pragma unroll
  for (int q = 0; q < 4; q++) aw1[q] = 0.f;
  const uint64_t rb = (uint64_t)blockIdx.x * chunk, re = std::min<uint64_t>(n, rb + chunk);
  for (uint64_t r0 = rb; r0 < re; r0 += GROWS) {
    const int nr = (int)std::min<uint64_t>(GROWS, re - r0);
    for (int e = tid; e < GROWS * NH; e += GT) {
      const int rr = e / NH, cc = e % NH;
      const bool ok = rr < nr;
      const uint64_t o = (r0 + rr) * NH + cc;
      sh1[rr][cc] = ok ? __bfloat162float(h1b[o]) : 0.f;
      sh2[rr][cc] = ok ? __bfloat162float(h2b[o]) : 0.f;
      sd1[rr][cc] = ok ? __bfloat162float(dh1b[o]) : 0.f;
      sd2[rr][cc] = ok ? __bfloat162float(dh2b[o]) : 0.f;
    }
    for (int e = tid; e < GROWS * NIN; e += GT) {
      const int rr = e / NIN, cc = e % NIN;
      sx[rr][cc] = rr < nr ? __bfloat162float(xb[(r0 + rr) * NIN + cc]) : 0.f;
    }
    for (int e = tid; e < GROWS * NOUT; e += GT) {
      const int rr = e / NOUT, cc = e % NOUT;
      sdz[rr][cc] = rr < nr ? dzf[(r0 + rr) * NOUT + cc] : 0.f;
    }
    __syncthreads();
    for (int rr = 0; rr < nr; rr++) {
      const float d2 = sd2[rr][o2], d1 = sd1[rr][o2];
#pragma unroll
      for (int q = 0; q < 16; q++) aw2[q] += d2 * sh1[rr][c2 + q];
#pragma unroll
      for (int q = 0; q < 4; q++) aw1[q] += d1 * sx[rr][c1 + q];
      aw3 += sdz[rr][tid >> 6] * sh2[rr][tid & 63];
      if (tid < NH)
        ab += sd1[rr][tid];
      else if (tid < 2 * NH)
        ab += sd2[rr][tid - NH];
      else if (tid < 2 * NH + NOUT)
        ab += sdz[rr][tid - 2 * NH];
    }
    __syncthreads();
  }
  float* p = part + (uint64_t)blockIdx.x * NPARAM;
#pragma unroll
  for (int q = 0; q < 16; q++) p[OFF_W2 + o2 * NH + c2 + q] = aw2[q];
#pragma unroll
  for (int q = 0; q < 4; q++) p[OFF_W1 + o2 * NIN + c1 + q] = aw1[q];
  p[OFF_W3 + tid] = aw3;  // tid = o * 64 + i
  if (tid < NH)
    p[OFF_B1 + tid] = ab;
  else if (tid < 2 * NH)
    p[OFF_B2 + tid - NH] = ab;
  else if (tid < 2 * NH + NOUT)
    p[OFF_B3 + tid - 2 * NH] = ab;
}

// sum of the block partials (in block order) -> gradient; Adam on the FP32 master
__global__ void k_mlp_reduce_adam(const float* __restrict__ part, int nblocks, float* __restrict__ grad,
                                  float* __restrict__ master, float* __restrict__ m, float* __restrict__ v, float lr,
                                  float b1t, float b2t, int do_step) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= NPARAM) return;
  float gsum = 0.f;
  for (int b = 0; b < nblocks; b++) gsum += part[(uint64_t)b * NPARAM + p];
  grad[p] = gsum;
  if (!do_step) return;
  const float beta1 = 0.9f, beta2 = 0.999f, eps = 1e-8f;
  const float mm = beta1 * m[p] + (1.f - beta1) * gsum;
  const float vv = beta2 * v[p] + (1.f - beta2) * gsum * gsum;
  m[p] = mm;
  v[p] = vv;
  master[p] -= lr * (mm / (1.f - b1t)) / (sqrtf(vv / (1.f - b2t)) + eps);
}

// BF16 copies (and transposes) of the master weights
__global__ void k_mlp_pack(const float* __restrict__ master, MlpWeights* __restrict__ w) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < NH * NIN) w->w1[i] = __float2bfloat16_rn(master[OFF_W1 + i]);
  if (i < NH * NH) {
    const int o = i / NH, c = i % NH;
    const __nv_bfloat16 b = __float2bfloat16_rn(master[OFF_W2 + i]);
    w->w2[i] = b;
    w->w2t[c * NH + o] = b;
  }
  if (i < 8 * NH) {
    const int o = i / NH, c = i % NH;
    const __nv_bfloat16 b = o < NOUT ? __float2bfloat16_rn(master[OFF_W3 + o * NH + c]) : __float2bfloat16_rn(0.f);
    w->w3[i] = b;
    w->w3t[c * 8 + o] = b;
  }
  if (i < NH) {
    w->b1[i] = master[OFF_B1 + i];
    w->b2[i] = master[OFF_B2 + i];
  }
  if (i < 8) w->b3[i] = i < NOUT ? master[OFF_B3 + i] : 0.f;
}
}  // namespace

// ---------------------------------------------------------------- host side
struct MlpState {
  float* master = nullptr;  // NPARAM
  float* m = nullptr;
  float* v = nullptr;
  float* grad = nullptr;
  MlpWeights* w = nullptr;
  int64_t step = 0;
  bool ready = false;
  // training scratch
  uint64_t cap = 0;
  __nv_bfloat16 *xb = nullptr, *h1b = nullptr, *h2b = nullptr, *dh1b = nullptr, *dh2b = nullptr;
  float* dzf = nullptr;
  float* part = nullptr;
  double* loss_part = nullptr;
  uint32_t* idx = nullptr;
  uint32_t* err = nullptr;  // k_mlp_infer_tc: an mbarrier wait gave up
};

void mlp_free(dem_ctx* c) {
  MlpState* s = c->mlp;
  if (!s) return;
  for (void* p : {(void*)s->master, (void*)s->m, (void*)s->v, (void*)s->grad, (void*)s->w, (void*)s->xb,
                  (void*)s->h1b, (void*)s->h2b, (void*)s->dh1b, (void*)s->dh2b, (void*)s->dzf, (void*)s->part,
                  (void*)s->loss_part, (void*)s->idx, (void*)s->err})
    cudaFree(p);
  delete s;
  c->mlp = nullptr;
}

static int mlp_alloc(dem_ctx* c) {
  if (c->mlp) return DEM_OK;
  MlpState* s = new MlpState;
  c->mlp = s;
  DEM_CUDA_TRY(c, cudaMalloc(&s->master, NPARAM * 4));
  DEM_CUDA_TRY(c, cudaMalloc(&s->m, NPARAM * 4));
  DEM_CUDA_TRY(c, cudaMalloc(&s->v, NPARAM * 4));
  DEM_CUDA_TRY(c, cudaMalloc(&s->grad, NPARAM * 4));
  DEM_CUDA_TRY(c, cudaMalloc(&s->w, sizeof(MlpWeights)));
  DEM_CUDA_TRY(c, cudaMalloc(&s->err, 4));
  DEM_CUDA_TRY(c, cudaMemsetAsync(s->err, 0, 4, c->stream));
  return DEM_OK;
}

static int mlp_scratch(dem_ctx* c, uint64_t batch) {
  MlpState* s = c->mlp;
  if (batch <= s->cap) return DEM_OK;
  for (void* p : {(void*)s->xb, (void*)s->h1b, (void*)s->h2b, (void*)s->dh1b, (void*)s->dh2b, (void*)s->dzf,
                  (void*)s->part, (void*)s->loss_part})
    cudaFree(p);
  const uint64_t nb = (batch + 255) / 256;
  DEM_CUDA_TRY(c, cudaMalloc(&s->xb, batch * NIN * 2));
  DEM_CUDA_TRY(c, cudaMalloc(&s->h1b, batch * NH * 2));
  DEM_CUDA_TRY(c, cudaMalloc(&s->h2b, batch * NH * 2));
  DEM_CUDA_TRY(c, cudaMalloc(&s->dh1b, batch * NH * 2));
  DEM_CUDA_TRY(c, cudaMalloc(&s->dh2b, batch * NH * 2));
  DEM_CUDA_TRY(c, cudaMalloc(&s->dzf, batch * NOUT * 4));
  DEM_CUDA_TRY(c, cudaMalloc(&s->part, nb * NPARAM * 4));
  DEM_CUDA_TRY(c, cudaMalloc(&s->loss_part, 4096 * 8));
  s->cap = batch;
  return DEM_OK;
}

static int mlp_upload(dem_ctx* c, const float* host) {
  MlpState* s = c->mlp;
  DEM_CUDA_TRY(c, cudaMemcpyAsync(s->master, host, NPARAM * 4, cudaMemcpyHostToDevice, c->stream));
  DEM_CUDA_TRY(c, cudaMemsetAsync(s->m, 0, NPARAM * 4, c->stream));
  DEM_CUDA_TRY(c, cudaMemsetAsync(s->v, 0, NPARAM * 4, c->stream));
  k_mlp_pack<<<(NH * NH + 255) / 256, 256, 0, c->stream>>>(s->master, s->w);
  DEM_CUDA_TRY(c, cudaGetLastError());
  DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  s->step = 0;
  s->ready = true;
  return DEM_OK;
}

bool mlp_ready(const dem_ctx* c) { return c->mlp && c->mlp->ready; }

int mlp_rates(dem_ctx* c, const float* dev_x, uint64_t n, float* dev_rates) {
  if (!c->mlp || !c->mlp->ready) return c->fail(DEM_ERR_STATE, "the MLP has no weights (dem_mlp_init / set_params)");
  if (!n) return DEM_OK;
  // four CTAs of 128 TMEM columns fill an SM's 512
  const unsigned blocks = (unsigned)std::min<uint64_t>((n + TC_M - 1) / TC_M, (uint64_t)c->num_sms * 4);
  k_mlp_infer_tc<<<blocks, TC_M, 0, c->stream>>>(c->mlp->w, dev_x, n, dev_rates, c->mlp->err);
  DEM_CUDA_TRY(c, cudaGetLastError());
  return DEM_OK;
}

// whether a tensor-core pass gave up waiting (reads the flag: synchronises the stream)
int mlp_check(dem_ctx* c) {
  if (!c->mlp) return DEM_OK;
  uint32_t e = 0;
  DEM_CUDA_TRY(c, cudaMemcpyAsync(&e, c->mlp->err, 4, cudaMemcpyDeviceToHost, c->stream));
  DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  if (e) return c->fail(DEM_ERR_CUDA, "tensor-core MLP pass: an mbarrier wait timed out");
  return DEM_OK;
}

// one optimisation pass over batch rows idx[0..bn): gradients into s->grad; Adam when step
static int mlp_batch(dem_ctx* c, const float* x, const uint8_t* y, const uint32_t* idx, uint64_t bn, float lr,
                     bool step, double* loss) {
  MlpState* s = c->mlp;
  int rc = mlp_scratch(c, bn);
  if (rc) return rc;
  const unsigned fb = (unsigned)std::min<uint64_t>((bn + 63) / 64, 4096);
  k_mlp_fwd_bwd<<<fb, 128, 0, c->stream>>>(s->w, x, y, idx, bn, 1.0f / (float)(bn * NOUT), s->xb, s->h1b, s->h2b,
                                            s->dh1b, s->dh2b, s->dzf, s->loss_part);
  const uint64_t chunk = 256;
  const int nb = (int)((bn + chunk - 1) / chunk);
  k_mlp_wgrad<<<nb, GT, 0, c->stream>>>(s->xb, s->h1b, s->h2b, s->dh1b, s->dh2b, s->dzf, bn, chunk, s->part);
  if (step) s->step++;
  const float b1t = (float)std::pow(0.9, (double)std::max<int64_t>(s->step, 1));
  const float b2t = (float)std::pow(0.999, (double)std::max<int64_t>(s->step, 1));
  k_mlp_reduce_adam<<<(NPARAM + 255) / 256, 256, 0, c->stream>>>(s->part, nb, s->grad, s->master, s->m, s->v, lr,
                                                                  b1t, b2t, step ? 1 : 0);
  if (step) k_mlp_pack<<<(NH * NH + 255) / 256, 256, 0, c->stream>>>(s->master, s->w);
  DEM_CUDA_TRY(c, cudaGetLastError());
  if (loss) {
    std::vector<double> lp(fb);
    DEM_CUDA_TRY(c, cudaMemcpyAsync(lp.data(), s->loss_part, fb * 8, cudaMemcpyDeviceToHost, c->stream));
    DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    double a = 0;
    for (double v : lp) a += v;
    *loss = a / (double)(bn * NOUT);
  }
  return DEM_OK;
}
}  // namespace dem

using namespace dem;

extern "C" {

int dem_mlp_harvest(dem_ctx* c, float* dev_x, uint8_t* dev_y, uint64_t capacity, uint64_t* count,
                    uint64_t* available) {
  if (!c || !count || !available || (capacity && (!dev_x || !dev_y))) return DEM_ERR_INVALID_ARG;
  if (!c->poly) return c->fail(DEM_ERR_STATE, "harvest needs a polyhedron context");
  if (!c->labels_valid)
    return c->fail(DEM_ERR_STATE, "no labels: rebuild the neighbour list with fp32_broad_phase first");
  return launch_harvest(c, dev_x, dev_y, capacity, count, available);
}

int dem_learned_stats(dem_ctx* c, uint64_t* units, uint64_t* overflow, uint64_t* record_entries) {
  if (!c || !units || !overflow || !record_entries) return DEM_ERR_INVALID_ARG;
  *units = c->learned_slots ? c->learned_units : 0;
  *overflow = c->learned_slots ? c->learned_overflow : 0;
  *record_entries = 0;
  if (c->learned_slots && c->learned_units) {
    uint32_t tot = 0;
    DEM_CUDA_TRY(c, cudaMemcpyAsync(&tot, c->u_slotoff + c->learned_units, 4, cudaMemcpyDeviceToHost, c->stream));
    DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    *record_entries = tot;
  }
  return DEM_OK;
}

int dem_mlp_init(dem_ctx* c, uint64_t seed, const float* label_means) {
  if (!c) return DEM_ERR_INVALID_ARG;
  int rc = mlp_alloc(c);
  if (rc) return rc;
  // He-uniform weights, zero biases; output biases log(mean label) when given
  std::mt19937_64 g(seed);
  std::vector<float> p(NPARAM, 0.f);
  auto fill = [&](int off, int rows, int cols) {
    const double lim = std::sqrt(6.0 / cols);
    for (int i = 0; i < rows * cols; i++) p[off + i] = (float)((2.0 * ((g() >> 11) * 0x1.0p-53) - 1.0) * lim);
  };
  fill(OFF_W1, NH, NIN);
  fill(OFF_W2, NH, NH);
  fill(OFF_W3, NOUT, NH);
  for (int i = 0; i < NOUT * NH; i++) p[OFF_W3 + i] *= 0.1f;  // start near the label means
  for (int k = 0; k < NOUT; k++) p[OFF_B3 + k] = label_means ? std::log(std::max(label_means[k], 1e-3f)) : 0.f;
  return mlp_upload(c, p.data());
}

int dem_mlp_set_params(dem_ctx* c, const float* host) {
  if (!c || !host) return DEM_ERR_INVALID_ARG;
  int rc = mlp_alloc(c);
  return rc ? rc : mlp_upload(c, host);
}

int dem_mlp_get_params(dem_ctx* c, float* host) {
  if (!c || !host) return DEM_ERR_INVALID_ARG;
  if (!c->mlp || !c->mlp->ready) return c->fail(DEM_ERR_STATE, "the MLP has no weights");
  DEM_CUDA_TRY(c, cudaMemcpyAsync(host, c->mlp->master, NPARAM * 4, cudaMemcpyDeviceToHost, c->stream));
  DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return DEM_OK;
}

int dem_mlp_forward(dem_ctx* c, const float* dev_x, uint64_t n, float* dev_rates) {
  if (!c || (n && (!dev_x || !dev_rates))) return DEM_ERR_INVALID_ARG;
  int rc = mlp_rates(c, dev_x, n, dev_rates);
  if (rc) return rc;
  return mlp_check(c);
}

int dem_mlp_loss_grad(dem_ctx* c, const float* dev_x, const uint8_t* dev_y, uint64_t n, float* host_grad,
                      double* loss) {
  if (!c || !dev_x || !dev_y || !host_grad || !n) return DEM_ERR_INVALID_ARG;
  if (!c->mlp || !c->mlp->ready) return c->fail(DEM_ERR_STATE, "the MLP has no weights");
  MlpState* s = c->mlp;
  std::vector<uint32_t> id(n);
  std::iota(id.begin(), id.end(), 0u);
  uint32_t* d_idx = nullptr;
  DEM_CUDA_TRY(c, cudaMalloc(&d_idx, n * 4));
  DEM_CUDA_TRY(c, cudaMemcpyAsync(d_idx, id.data(), n * 4, cudaMemcpyHostToDevice, c->stream));
  int rc = mlp_batch(c, dev_x, dev_y, d_idx, n, 0.f, false, loss);
  if (!rc) {
    DEM_CUDA_TRY(c, cudaMemcpyAsync(host_grad, s->grad, NPARAM * 4, cudaMemcpyDeviceToHost, c->stream));
    DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  }
  cudaFree(d_idx);
  return rc;
}

int dem_mlp_train(dem_ctx* c, const float* dev_x, const uint8_t* dev_y, uint64_t n, int epochs, uint64_t batch,
                  float lr, uint64_t seed, double* loss_per_epoch) {
  if (!c || !dev_x || !dev_y || !n || epochs < 1 || batch < 16 || batch > (1ull << 24)) return DEM_ERR_INVALID_ARG;
  if (!c->mlp || !c->mlp->ready) return c->fail(DEM_ERR_STATE, "the MLP has no weights (dem_mlp_init)");
  MlpState* s = c->mlp;
  uint32_t* d_idx = nullptr;
  DEM_CUDA_TRY(c, cudaMalloc(&d_idx, n * 4));
  std::vector<uint32_t> perm(n);
  std::mt19937_64 g(seed);
  int rc = DEM_OK;
  for (int e = 0; e < epochs && !rc; e++) {
    std::iota(perm.begin(), perm.end(), 0u);
    std::shuffle(perm.begin(), perm.end(), g);
    DEM_CUDA_TRY(c, cudaMemcpyAsync(d_idx, perm.data(), n * 4, cudaMemcpyHostToDevice, c->stream));
    double acc = 0.0;
    uint64_t seen = 0;
    for (uint64_t b0 = 0; b0 + batch <= n && !rc; b0 += batch) {  // full batches only
      double l = 0.0;
      rc = mlp_batch(c, dev_x, dev_y, d_idx + b0, batch, lr, true, loss_per_epoch ? &l : nullptr);
      acc += l * (double)batch;
      seen += batch;
    }
    if (loss_per_epoch) loss_per_epoch[e] = seen ? acc / (double)seen : 0.0;
  }
  DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  cudaFree(d_idx);
  (void)s;
  return rc;
}
}  // extern "C"
