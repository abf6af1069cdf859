// k_particles.cu -- per-particle operators of the Verlet scheme and the state reductions.
//
//   reset_force_moment   src/numericalscheme/reset_force_moment.cu:69-70
//   gravity_force        src/forcefield/include/exaDEM/forcefield/gravity_force.hpp:38-46
//   force_to_accel       src/numericalscheme/include/exaDEM/force_to_accel.hpp:26-33
//   prolog               src/numericalscheme/combined_compute_prolog.cu:94-116,
//                        push_to_quaternion.hpp:26-38 (x, v/2, q, w/2)
//   epilog               src/numericalscheme/combined_compute_epilog.cu:94-113,
//                        angular_acceleration.hpp:27-43, angular_velocity.hpp:27-33
//   particle_displ_over  exaNBody: any |r - r_backup|^2 >= max_displ^2, max_displ = rcut_inc/2
//   simulation_state     src/io/include/exaDEM/simulation_state.hpp:48-56 (deterministic tree sum)
// Quaternion arithmetic restates onika's Quaternion operators following exaDEM's
// quat type (src/shape/include/exaDEM/type/quat.hpp:79-96,233-242).
#include "integrate_core.cuh"

namespace dem {
namespace {

__global__ void k_reset(PArrays P, uint64_t n) {
  const uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  P.f[FX][s] = 0.0;
  P.f[FY][s] = 0.0;
  P.f[FZ][s] = 0.0;
  P.f[MX][s] = 0.0;
  P.f[MY][s] = 0.0;
  P.f[MZ][s] = 0.0;
}

__global__ void k_gravity(PArrays P, uint64_t n, double gx, double gy, double gz) {
  const uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const double m = P.f[MASS][s];
  P.f[FX][s] = P.f[FX][s] + gx * m;
  P.f[FY][s] = P.f[FY][s] + gy * m;
  P.f[FZ][s] = P.f[FZ][s] + gz * m;
}

__global__ void k_force_to_accel(PArrays P, uint64_t n) {
  const uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const double m = P.f[MASS][s];
  P.f[FX][s] = P.f[FX][s] / m;
  P.f[FY][s] = P.f[FY][s] / m;
  P.f[FZ][s] = P.f[FZ][s] / m;
}

__global__ void k_prolog(PArrays P, uint64_t n, double delta_t, double half_delta_t, double delta_t2_2) {
  const uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  prolog_one(P, s, delta_t, half_delta_t, delta_t2_2);
}

__global__ void k_epilog(PArrays P, uint64_t n, double half_delta_t) {
  const uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const V3 a = mk(P.f[FX][s], P.f[FY][s], P.f[FZ][s]);
  const V3 mom = mk(P.f[MX][s], P.f[MY][s], P.f[MZ][s]);
  epilog_one<false>(P, s, half_delta_t, a, mom);
}

__global__ void k_displ(PArrays P, uint64_t n, double thr2, unsigned long long* flag, SysView sv) {
  const uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  bool over = false;
  if (s < n) {
    const double dx = P.f[RX][s] - P.f[BX][s], dy = P.f[RY][s] - P.f[BY][s], dz = P.f[RZ][s] - P.f[BZ][s];
    over = dx * dx + dy * dy + dz * dz >= thr2;
    if (over && sv.nsys > 1) atomicOr(&sv.trig[sv.of(s)], 1u);  // this system's own trigger
  }
  if (__any_sync(0xffffffffu, over) && (threadIdx.x & 31) == 0) atomicOr(flag, 1ull);
}

// Deterministic two-level reduction: fixed block partition, fixed tree order.
constexpr int RED_THREADS = 256;
__global__ void k_state_partial(PArrays P, uint64_t n, double* __restrict__ part) {
  __shared__ double sh[7][RED_THREADS];
  double acc[7] = {0, 0, 0, 0, 0, 0, 0};
  for (uint64_t s = (uint64_t)blockIdx.x * RED_THREADS + threadIdx.x; s < n; s += (uint64_t)gridDim.x * RED_THREADS) {
    const double m = P.f[MASS][s];
    acc[0] += m;
    acc[1] += 0.5 * P.f[WX][s] * P.f[WX][s] * m;
    acc[2] += 0.5 * P.f[WY][s] * P.f[WY][s] * m;
    acc[3] += 0.5 * P.f[WZ][s] * P.f[WZ][s] * m;
    acc[4] += 0.5 * P.f[VX][s] * P.f[VX][s] * m;
    acc[5] += 0.5 * P.f[VY][s] * P.f[VY][s] * m;
    acc[6] += 0.5 * P.f[VZ][s] * P.f[VZ][s] * m;
  }
#pragma unroll
  for (int k = 0; k < 7; k++) sh[k][threadIdx.x] = acc[k];
  __syncthreads();
  for (int w = RED_THREADS / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w)
#pragma unroll
      for (int k = 0; k < 7; k++) sh[k][threadIdx.x] += sh[k][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x < 7) part[blockIdx.x * 7 + threadIdx.x] = sh[threadIdx.x][0];
}
__global__ void k_state_final(const double* __restrict__ part, int nb, double* __restrict__ out) {
  if (threadIdx.x < 7) {
    double a = 0;
    for (int b = 0; b < nb; b++) a += part[b * 7 + threadIdx.x];
    out[threadIdx.x] = a;
  }
}

// One block per system: the sums of k_state_partial over the system's
// particles, and its interactions (owned by its particles; sorted by owner, so
// the range own_off[first] .. own_off[last + 1]), counting those with a
// non-zero friction or moment history (Interaction::active, interaction.hpp:129-136).
__global__ void k_state_sys(PArrays P, SysView sv, IArrays I, const uint32_t* __restrict__ own_off, int have_list,
                            double* __restrict__ out, unsigned long long* __restrict__ cnt) {
  __shared__ double sh[7][RED_THREADS];
  __shared__ unsigned long long sa[RED_THREADS];
  const int k = blockIdx.x;
  const uint64_t b = sv.pfirst[k], e = sv.pfirst[k + 1];
  double acc[7] = {0, 0, 0, 0, 0, 0, 0};
  for (uint64_t s = b + threadIdx.x; s < e; s += RED_THREADS) {
    const double m = P.f[MASS][s];
    acc[0] += m;
    acc[1] += 0.5 * P.f[WX][s] * P.f[WX][s] * m;
    acc[2] += 0.5 * P.f[WY][s] * P.f[WY][s] * m;
    acc[3] += 0.5 * P.f[WZ][s] * P.f[WZ][s] * m;
    acc[4] += 0.5 * P.f[VX][s] * P.f[VX][s] * m;
    acc[5] += 0.5 * P.f[VY][s] * P.f[VY][s] * m;
    acc[6] += 0.5 * P.f[VZ][s] * P.f[VZ][s] * m;
  }
  unsigned long long act = 0;
  uint64_t ib = 0, ie = 0;
  if (have_list) {
    ib = own_off[b];
    ie = own_off[e];
    for (uint64_t q = ib + threadIdx.x; q < ie; q += RED_THREADS)
      act += (I.ft[0][q] != 0.0 || I.ft[1][q] != 0.0 || I.ft[2][q] != 0.0 || I.mo[0][q] != 0.0 ||
              I.mo[1][q] != 0.0 || I.mo[2][q] != 0.0)
                 ? 1
                 : 0;
  }
#pragma unroll
  for (int q = 0; q < 7; q++) sh[q][threadIdx.x] = acc[q];
  sa[threadIdx.x] = act;
  __syncthreads();
  for (int w = RED_THREADS / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
#pragma unroll
      for (int q = 0; q < 7; q++) sh[q][threadIdx.x] += sh[q][threadIdx.x + w];
      sa[threadIdx.x] += sa[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x < 7) out[k * 7 + threadIdx.x] = sh[threadIdx.x][0];
  if (threadIdx.x == 0) {
    cnt[2 * k] = ie - ib;
    cnt[2 * k + 1] = sa[0];
  }
}

__global__ void k_profile(PArrays P, uint64_t n, int nslabs, double zlo, double dz, double* __restrict__ vol) {
  const uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const double zc = P.f[RZ][s], r = P.f[RAD][s];
  int a = (int)floor((zc - r - zlo) / dz), b = (int)floor((zc + r - zlo) / dz);
  if (a < 0) a = 0;
  if (b > nslabs - 1) b = nslabs - 1;
  for (int k = a; k <= b; k++) {
    const double s0 = zlo + k * dz, s1 = zlo + (k + 1) * dz;
    const double lo = fmax(s0, zc - r), hi = fmin(s1, zc + r);
    if (hi <= lo) continue;
    const double ul = lo - zc, uh = hi - zc;
    const double Fh = r * r * uh - uh * uh * uh / 3.0, Fl = r * r * ul - ul * ul * ul / 3.0;
    atomicAdd(&vol[k], M_PI * (Fh - Fl));
  }
}
__global__ void k_reciprocals(PArrays P, uint64_t n) {
  const uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  P.f[IMASS][s] = 1.0 / P.f[MASS][s];
  P.f[IIX][s] = 1.0 / P.f[IX][s];
  P.f[IIY][s] = 1.0 / P.f[IY][s];
  P.f[IIZ][s] = 1.0 / P.f[IZ][s];
}
}  // namespace

int launch_reciprocals(dem_ctx* c, uint64_t n) {
  if (n) k_reciprocals<<<grid_for(n, 256), 256, 0, c->stream>>>(c->P[0], n);
  DEM_CUDA_TRY(c, cudaGetLastError());
  return DEM_OK;
}

int launch_reset_force_moment(dem_ctx* c) {
  ProfScope ps(c, K_RESET, c->n ? 1 : 0);
  if (c->n) k_reset<<<grid_for(c->n, 256), 256, 0, c->stream>>>(c->P[c->pcur], c->n);
  DEM_CUDA_TRY(c, cudaGetLastError());
  return DEM_OK;
}
int launch_gravity(dem_ctx* c) {
  ProfScope ps(c, K_GRAVITY, c->n ? 1 : 0);
  if (c->n)
    k_gravity<<<grid_for(c->n, 256), 256, 0, c->stream>>>(c->P[c->pcur], c->n, c->prm.gravity[0], c->prm.gravity[1],
                                                            c->prm.gravity[2]);
  DEM_CUDA_TRY(c, cudaGetLastError());
  return DEM_OK;
}
int launch_force_to_accel(dem_ctx* c) {
  ProfScope ps(c, K_F2A, c->n ? 1 : 0);
  if (c->n) k_force_to_accel<<<grid_for(c->n, 256), 256, 0, c->stream>>>(c->P[c->pcur], c->n);
  DEM_CUDA_TRY(c, cudaGetLastError());
  return DEM_OK;
}
int launch_prolog(dem_ctx* c) {
  const double delta_t = c->prm.dt;
  const double half_delta_t = delta_t * 0.5;
  const double delta_t2_2 = delta_t * delta_t * 0.5;
  ProfScope ps(c, K_PROLOG, c->n ? 1 : 0);
  if (c->n)
    k_prolog<<<grid_for(c->n, 128), 128, 0, c->stream>>>(c->P[c->pcur], c->n, delta_t, half_delta_t, delta_t2_2);
  DEM_CUDA_TRY(c, cudaGetLastError());
  return DEM_OK;
}
int launch_epilog(dem_ctx* c) {
  const double half_delta_t = c->prm.dt * 0.5;
  ProfScope ps(c, K_EPILOG, c->n ? 1 : 0);
  if (c->n) k_epilog<<<grid_for(c->n, 128), 128, 0, c->stream>>>(c->P[c->pcur], c->n, half_delta_t);
  DEM_CUDA_TRY(c, cudaGetLastError());
  return DEM_OK;
}
int launch_displ_over(dem_ctx* c) {
  const double max_displ = c->prm.rcut_inc * 0.5;
  DEM_CUDA_TRY(c, cudaMemsetAsync(c->d_scalars, 0, sizeof(unsigned long long), c->stream));
  ProfScope ps(c, K_DISPL, c->n ? 1 : 0);
  if (c->n)
    k_displ<<<grid_for(c->n, 256), 256, 0, c->stream>>>(c->P[c->pcur], c->n, max_displ * max_displ, c->d_scalars,
                                                         c->sysview());
  DEM_CUDA_TRY(c, cudaGetLastError());
  return DEM_OK;
}
int launch_state(dem_ctx* c, dem_state* out) {
  const int nb = 2 * c->num_sms;
  double* part = c->d_red;
  double* fin = c->d_red + 7 * nb;
  ProfScope ps(c, K_STATE, 2);
  k_state_partial<<<nb, RED_THREADS, 0, c->stream>>>(c->P[c->pcur], c->n, part);
  k_state_final<<<1, 32, 0, c->stream>>>(part, nb, fin);
  double h[7];
  DEM_CUDA_TRY(c, cudaMemcpyAsync(h, fin, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
  DEM_CUDA_TRY(c, cudaMemcpyAsync(c->h_scalars, c->d_scalars, 3 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                                  c->stream));
  DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  out->mass = h[0];
  for (int d = 0; d < 3; d++) {
    out->rotation_energy[d] = h[1 + d];
    out->kinetic_energy[d] = h[4 + d];
  }
  out->n_particles = c->n;
  out->n_interactions = c->ni;
  out->n_active_interactions = c->h_scalars[1];
  return DEM_OK;
}
int launch_state_systems(dem_ctx* c, dem_state* out) {
  const int ns = c->nsys;
  double* d_out = nullptr;
  unsigned long long* d_cnt = nullptr;
  DEM_CUDA_TRY(c, cudaMallocAsync(&d_out, (size_t)ns * 7 * sizeof(double), c->stream));
  DEM_CUDA_TRY(c, cudaMallocAsync(&d_cnt, (size_t)ns * 2 * sizeof(unsigned long long), c->stream));
  {
    ProfScope ps(c, K_STATE, 1);
    k_state_sys<<<ns, RED_THREADS, 0, c->stream>>>(c->P[c->pcur], c->sysview(), c->I[c->icur], c->own_off[c->icur],
                                                   (c->have_list && c->ni) ? 1 : 0, d_out, d_cnt);
  }
  std::vector<double> h((size_t)ns * 7);
  std::vector<unsigned long long> hc((size_t)ns * 2);
  DEM_CUDA_TRY(c, cudaMemcpyAsync(h.data(), d_out, h.size() * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  DEM_CUDA_TRY(c, cudaMemcpyAsync(hc.data(), d_cnt, hc.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                                  c->stream));
  DEM_CUDA_TRY(c, cudaFreeAsync(d_out, c->stream));
  DEM_CUDA_TRY(c, cudaFreeAsync(d_cnt, c->stream));
  DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  const std::vector<dem_system>& sys = c->systems;
  for (int k = 0; k < ns; k++) {
    dem_state& o = out[k];
    o.mass = h[k * 7];
    for (int d = 0; d < 3; d++) {
      o.rotation_energy[d] = h[k * 7 + 1 + d];
      o.kinetic_energy[d] = h[k * 7 + 4 + d];
    }
    o.n_particles = sys.empty() ? c->n : sys[k].count;
    o.n_interactions = hc[2 * k];
    o.n_active_interactions = hc[2 * k + 1];
  }
  return DEM_OK;
}

int launch_profile(dem_ctx* c, int nslabs, double zlo, double zhi, double* out) {
  if ((uint64_t)nslabs > c->red_cap) return c->fail(DEM_ERR_INVALID_ARG, "nslabs too large");
  const double dz = (zhi - zlo) / nslabs;
  DEM_CUDA_TRY(c, cudaMemsetAsync(c->d_red, 0, nslabs * sizeof(double), c->stream));
  if (c->n) k_profile<<<grid_for(c->n, 256), 256, 0, c->stream>>>(c->P[c->pcur], c->n, nslabs, zlo, dz, c->d_red);
  DEM_CUDA_TRY(c, cudaMemcpyAsync(out, c->d_red, nslabs * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  DEM_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  const double area = c->grid.L[0] * c->grid.L[1];
  for (int k = 0; k < nslabs; k++) out[k] = out[k] / (area * dz);
  return DEM_OK;
}
}  // namespace dem
