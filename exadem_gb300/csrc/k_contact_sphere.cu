// k_contact_sphere.cu -- Hooke contact law for spheres and the deterministic force gather.
//
// k_contact: one thread per interaction.  Restates sphere::ContactLawFunc and
// ContactLawDriverFunc<Surface|Cylinder> (src/sphere/include/exaDEM/sphere/contact_sphere.hpp:122-297)
// around contact_force_core<Hooke, None|Cohesive>
// (src/forcefield/include/exaDEM/forcefield/contact_force.hpp:146-235,
// common_kernels.hpp:27-145) in the same FP64 operation order.  Instead of the
// reference's FP64 atomicAdd into both particles (contact_sphere.hpp:183-196)
// it writes a force record per interaction: f, the owner torque
// cross(cp - r_i, f) + moment and the partner torque cross(cp - r_j, -f) - moment.
// k_gather: one thread per particle sums, in a fixed order, the records of the
// interactions it owns (InteractionPair order) and then those where it is the
// partner (InteractionPair order).  The result does not depend on scheduling.
//
// Split precision (fp32_contact_screen): a pair whose FP32 distance test
// proves dn > max(0, dncut) (the proof margin covers the FP32 rounding of the
// squared distance) takes the no-contact branch (history reset) without any
// FP64 work; every other pair runs the full FP64 law.
#include "contact_core.cuh"
#include "mesh_core.cuh"

namespace dem {
namespace {

struct ContactArgs {
  PArrays P;
  IArrays I;
  Records R;
  uint64_t ni;
  SysView sv;  // periodic lengths of the owner's system
  const DriverDev* drv;
  const MeshDev* mesh;
  dem_contact_params cp;   // particle-particle
  dem_contact_params cpd;  // particle-driver
  double dt;
  int cohesive;
  int dmt;        // Hooke_DMT law combination
  ParamTable pt;  // multi-material parameters (pt.pp == nullptr: cp / cpd)
  ContactStateArrays cs;  // analysis (cs.dn == nullptr: off)
  int screen;
  unsigned long long* n_active;
};

__global__ void __launch_bounds__(128) k_contact(ContactArgs a) {
  const uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  bool act = false;
  if (k < a.ni) {
    const uint32_t meta = a.I.meta[k];
    const uint32_t type = meta_type(meta);
    const uint32_t i = a.I.owner[k];
    const uint32_t j = a.I.partner[k];
    const V3 ri = ldv(a.P, RX, i);
    V3 ft = mk(a.I.ft[0][k], a.I.ft[1][k], a.I.ft[2][k]);
    V3 mo = mk(a.I.mo[0][k], a.I.mo[1][k], a.I.mo[2][k]);
    V3 f = mk(0, 0, 0), ti = mk(0, 0, 0), tj = mk(0, 0, 0);
    const double rad_i = a.P.f[RAD][i];
    bool contact = false;
    if (type == DEM_ITYPE_VERTEX_VERTEX) {
      V3 rj = ldv(a.P, RX, j);
      const int sx = meta_shift(meta, 0), sy = meta_shift(meta, 1), sz = meta_shift(meta, 2);
      if (sx | sy | sz) {
        const GridDev& g = a.sv.g[a.sv.of(i)];
        if (sx) rj.x = rj.x + (double)sx * g.L[0];
        if (sy) rj.y = rj.y + (double)sy * g.L[1];
        if (sz) rj.z = rj.z + (double)sz * g.L[2];
      }
      const double rad_j = a.P.f[RAD][j];
      const dem_contact_params& cp = a.pt.pair(a.cp, a.P.group[i], a.P.group[j]);  // contact_sphere.hpp:147-152
      bool skip = false;
      if (a.screen) {
        // FP32 proof of separation: |d|^2 computed in FP32 from FP64 differences
        // (relative error < 2^-21 for the sum of squares) against (R + dncut)^2 * (1 + 2^-18).
        const float ex = (float)(ri.x - rj.x), ey = (float)(ri.y - rj.y), ez = (float)(ri.z - rj.z);
        const float d2f = ex * ex + ey * ey + ez * ez;
        const double lim = rad_i + rad_j + (a.cohesive ? fmax(cp.dncut, 0.0) : 0.0);
        const float limf = (float)lim;
        // only where lim^2 is a normal FP32 number, so the relative bound holds
        skip = lim > 1e-15 && lim < 1e15 && d2f > limf * limf * 1.0000039f;
      }
      if (!skip) {
        // detection_vertex_vertex_core (shape_detection_core.hpp:57-81)
        const double R = rad_i + rad_j;
        const V3 dist = ri - rj;
        const double dist_norm = vnorm(dist);
        const double inv_dist_norm = 1.0 / dist_norm;
        const double dn = dist_norm - R;
        const V3 n = dist * inv_dist_norm;
        const V3 cpos = ri - n * (rad_i + 0.5 * dn);
        contact = dn < 0;
        if (a.cohesive) contact = (contact || dn <= cp.dncut);
        if (contact) {
          const V3 vi = ldv(a.P, VX, i), vj = ldv(a.P, VX, j);
          const V3 wi = ldv(a.P, WX, i), wj = ldv(a.P, WX, j);
          const double m_i = a.P.f[MASS][i], m_j = a.P.f[MASS][j];
          const double meff = (m_i * m_j) / (m_i + m_j);
          // reff = compute_effective_radius (common_kernels.hpp:99-102), DMT only
          const double reff = a.dmt ? (rad_i * rad_j) / (rad_i + rad_j) : 0.0;
          contact_force_core(a.cohesive, dn, n, a.dt, cp, meff, ft, cpos, ri, vi, f, mo, wi, rj, vj, wj, a.dmt,
                             reff);
          ti = cross(cpos - ri, f) + mo;
          tj = cross(cpos - rj, -f) + (-mo);
          act = dn < 0;
          a.cs.write(k, dn, cpos, f - ft, ft);  // AnalysisDataPacker: fn = f - friction
        } else {
          a.cs.write(k, 0.0, cpos, mk(0, 0, 0), mk(0, 0, 0));  // item.reset(), dn = 0
        }
      }
    } else {
      const DriverDev& d = a.drv[j];
      double dn;
      V3 n = mk(0, 0, 0), cpos = mk(0, 0, 0), dpos, dvel, dvrot;
      if (d.kind == 2) {
        // ContactLawRShapeDriverFunc (contact_sphere.hpp:300-396): detect<7|8|9>
        const DetD q = mesh_detect(a.mesh[d.mesh], type, a.I.sub[k] >> 16, ri, rad_i);
        dn = q.dn;
        contact = q.c;
        n = q.n;
        cpos = q.cp;
      } else if (d.kind == 0) {
        const V3 nrm = mk(d.normal[0], d.normal[1], d.normal[2]);
        const V3 proj = dot(ri, nrm) * nrm;
        const V3 s2p = -(mk(d.center_proj[0], d.center_proj[1], d.center_proj[2]) - proj);
        const double dd = vnorm(s2p);
        dn = dd - rad_i;
        contact = !(dn > 0);
        if (contact) {
          n = s2p / dd;
          cpos = ri - n * (rad_i + 0.5 * dn);
        }
      } else {
        const V3 proj = ri * mk(d.axis[0], d.axis[1], d.axis[2]);
        const V3 dir = mk(d.center[0], d.center[1], d.center[2]) - proj;
        const double dd = vnorm(dir);
        dn = d.radius - (rad_i + dd);
        contact = !(dn > 0);
        if (contact) {
          n = dir / dd;
          cpos = ri - n * (rad_i + 0.5 * dn);
        }
      }
      dpos = mk(d.center[0], d.center[1], d.center[2]);
      dvel = mk(d.vel[0], d.vel[1], d.vel[2]);
      dvrot = mk(d.vrot[0], d.vrot[1], d.vrot[2]);
      const dem_contact_params& cpd = a.pt.drv(a.cpd, a.P.group[i], j);  // contact_sphere.hpp:254-257
      if (a.cohesive) contact = (contact || dn <= cpd.dncut);
      if (contact) {
        const V3 v = ldv(a.P, VX, i);
        const V3 wi = ldv(a.P, WX, i);
        const double meff = a.P.f[MASS][i];
        contact_force_core(a.cohesive, dn, n, a.dt, cpd, meff, ft, cpos, ri, v, f, mo, wi, dpos, dvel, dvrot, a.dmt,
                           rad_i);  // reff = the particle's radius (contact_sphere.hpp:270)
        ti = cross(cpos - ri, f) + mo;
        act = dn < 0;
        a.cs.write(k, dn, cpos, f - ft, ft);
      } else {
        a.cs.write(k, 0.0, cpos, mk(0, 0, 0), mk(0, 0, 0));
      }
    }
    if (!contact) {
      ft = mk(0, 0, 0);
      mo = mk(0, 0, 0);
    }
    a.I.ft[0][k] = ft.x;
    a.I.ft[1][k] = ft.y;
    a.I.ft[2][k] = ft.z;
    a.I.mo[0][k] = mo.x;
    a.I.mo[1][k] = mo.y;
    a.I.mo[2][k] = mo.z;
    a.R.f[0][k] = f.x;
    a.R.f[1][k] = f.y;
    a.R.f[2][k] = f.z;
    a.R.ti[0][k] = ti.x;
    a.R.ti[1][k] = ti.y;
    a.R.ti[2][k] = ti.z;
    a.R.tj[0][k] = tj.x;
    a.R.tj[1][k] = tj.y;
    a.R.tj[2][k] = tj.z;
  }
  const unsigned ball = __ballot_sync(0xffffffffu, act);
  if ((threadIdx.x & 31) == 0 && ball) atomicAdd(a.n_active, (unsigned long long)__popc(ball));
}

__global__ void k_gather(PArrays P, Records R, uint64_t n, const uint32_t* __restrict__ own_off,
                         const uint32_t* __restrict__ rev_off, const uint32_t* __restrict__ rev_idx) {
  const uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  V3 f = ldv(P, FX, (uint32_t)s);
  V3 m = ldv(P, MX, (uint32_t)s);
  // a record whose live flag is 0 is zero (+0 or -0 components); the sums start
  // at +0 or a nonzero value and never become -0, so skipping it keeps every bit
  for (uint32_t k = own_off[s]; k < own_off[s + 1]; k++) {
    if (!R.live[k]) continue;
    f = f + mk(R.f[0][k], R.f[1][k], R.f[2][k]);
    m = m + mk(R.ti[0][k], R.ti[1][k], R.ti[2][k]);
  }
  for (uint32_t q = rev_off[s]; q < rev_off[s + 1]; q++) {
    const uint32_t k = rev_idx[q];
    if (!R.live[k]) continue;
    f = f + (-mk(R.f[0][k], R.f[1][k], R.f[2][k]));
    m = m + mk(R.tj[0][k], R.tj[1][k], R.tj[2][k]);
  }
  P.f[FX][s] = f.x;
  P.f[FY][s] = f.y;
  P.f[FZ][s] = f.z;
  P.f[MX][s] = m.x;
  P.f[MY][s] = m.y;
  P.f[MZ][s] = m.z;
}
}  // namespace

int launch_contact_sphere(dem_ctx* c) {
  ContactArgs a;
  a.P = c->P[c->pcur];
  a.I = c->I[c->icur];
  a.R = c->R;
  a.ni = c->ni;
  a.sv = c->sysview();
  a.drv = c->drv_dev;
  a.mesh = c->mesh_dev;
  a.cp = c->prm.config;
  a.cpd = c->prm.config_driver;
  a.dt = c->prm.dt;
  a.cohesive = c->prm.law == DEM_LAW_HOOKE_COHESIVE;
  a.dmt = c->prm.law == DEM_LAW_HOOKE_DMT;
  a.pt = c->ptable();
  a.cs = c->cs;
  a.screen = c->prm.fp32_contact_screen && !c->analysis;  // analysis: every pair's state
  a.n_active = c->d_scalars + 1;
  DEM_CUDA_TRY(c, cudaMemsetAsync(c->d_scalars + 1, 0, sizeof(unsigned long long), c->stream));
  ProfScope ps(c, K_CONTACT, c->ni ? 1 : 0);
  if (c->ni) k_contact<<<grid_for(c->ni, 128), 128, 0, c->stream>>>(a);
  DEM_CUDA_TRY(c, cudaGetLastError());
  return mark_records_live(c);  // this kernel writes every record without keeping the flags
}

int launch_gather_forces(dem_ctx* c) {
  ProfScope ps(c, K_GATHER, c->n ? 1 : 0);
  if (c->n)
    k_gather<<<grid_for(c->n, 128), 128, 0, c->stream>>>(c->P[c->pcur], c->R, c->n, c->own_off[c->icur], c->rev_off,
                                                          c->rev_idx);
  DEM_CUDA_TRY(c, cudaGetLastError());
  return DEM_OK;
}
}  // namespace dem
