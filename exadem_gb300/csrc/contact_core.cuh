// contact_core.cuh -- device restatement of contact_force_core shared by the
// contact kernels (plain one-pass and compacted three-pass).
#pragma once
#include "dem_ctx.cuh"

namespace dem {

// contact_force_core (contact_force.hpp:146-235).  f_i must be {0,0,0} on entry.
__device__ __forceinline__ void contact_force_core(bool cohesive, double dn, V3 n, double dt, const dem_contact_params& hkp,
                                          double meff, V3& ft, V3 cpos, V3 pos_i, V3 vel_i, V3& f_i, V3& mom_i,
                                          V3 vrot_i, V3 pos_j, V3 vel_j, V3 vrot_j) {
  if (cohesive) {
    if (dn >= 0) {
      const double fn_value = (hkp.fc / hkp.dncut) * dn - hkp.fc;
      f_i = f_i + fn_value * n;
      ft = mk(0, 0, 0);
      return;
    }
  }
  const double damp = hkp.damp_rate * 2.0 * sqrt(hkp.kn * meff);
  const V3 contribution_i = vel_i - cross(cpos - pos_i, vrot_i);
  const V3 contribution_j = vel_j - cross(cpos - pos_j, vrot_j);
  const V3 vel = contribution_j - contribution_i;
  const double vn = dot(vel, n);
  V3 fn;
  {
    const double fne = -hkp.kn * dn;
    const double fnv = damp * vn;
    double nf = (fnv + fne > 0) ? fnv + fne : 0;
    if (cohesive) {
      const double fn_norm = nf - hkp.fc;
      nf = fn_norm < (-hkp.fc) ? -hkp.fc : fn_norm;
    }
    fn = nf * n;
  }
  {
    const V3 vt = vel - vn * n;
    const V3 ftd = dt * vt;
    ft = ft + hkp.kt * ftd;
  }
  double threshold_ft;
  if (!cohesive) {
    const double fne = hkp.kn * dn;
    threshold_ft = fabs(hkp.mu * fne);
  } else {
    threshold_ft = fabs(hkp.mu * (dot(fn, n) + hkp.fc));
  }
  {
    const double ft_square = dot(ft, ft);
    if (ft_square > 0.0 && ft_square > threshold_ft * threshold_ft) {
      const double s = threshold_ft / sqrt(ft_square);
      ft = ft * s;
    }
  }
  f_i = fn + ft;
  mom_i = mom_i + hkp.kr * (vrot_j - vrot_i) * dt;
  // rolling clip with mur = 0 (contact_force.hpp:225-234): the IEEE NaN of
  // 0/0 when vrot_i == 0 keeps the moment, otherwise the moment is scaled by 0.
  V3 branch = cpos - pos_i;
  const double r = (dot(branch, vrot_i)) / (dot(vrot_i, vrot_i));
  branch = branch - r * vrot_i;
  const double mur = 0;
  const double threshold_mom = fabs(mur * vnorm(branch) * vnorm(fn));
  const double mom_square = dot(mom_i, mom_i);
  if (mom_square > 0.0 && mom_square > threshold_mom * threshold_mom)
    mom_i = mom_i * (threshold_mom / sqrt(mom_square));
}


__device__ __forceinline__ V3 ldv(const PArrays& P, int f0, uint32_t i) {
  return mk(P.f[f0][i], P.f[f0 + 1][i], P.f[f0 + 2][i]);
}

}  // namespace dem
