// contact_core.cuh -- device restatement of contact_force_core shared by the
// contact kernels (plain one-pass and compacted three-pass).
#pragma once
#include "dem_ctx.cuh"
#include "mul_policy.cuh"

namespace dem {

// Rolling clip of contact_force_core with its mur = 0 (contact_force.hpp:225-234):
//   r = (b.w)/(w.w); b' = b - r w; t = |0 * |b'| * |fn||;
//   if (|m|^2 > 0 && |m|^2 > t^2) m = m * (t / |m|)
// t is +0 when |b'| and |fn| are finite and NaN otherwise (0 * inf, NaN).
// Both are finite, with no operation overflowing, when every |b_c| < 2^200,
// every |fn_c| < 2^500, every |w_c| < 2^200 and some |w_c| >= 2^-200: then
// w.w lies in [2^-400, 3 2^400], |r w| <= |b| (1 + 8u) (a projection), and
// every square stays below 2^1024.  So in that range the clip is exactly
// "if (|m|^2 > 0) m = m * (+0)" (the signed zeros of m; m * 0 of an infinite
// component is NaN, as in the formula), without the two norms, the division
// and the square roots.  A spin of exactly zero keeps the moment (0/0 below);
// outside both cases (huge or non-finite values) the formula itself runs.
__device__ __forceinline__ bool exp_below(double x, int e2) {  // |x| < 2^e2, x finite
  return (int)((emu_bits(x) >> 52) & 0x7ffu) < 1023 + e2;
}
__device__ __forceinline__ bool exp_at_least(double x, int e2) {  // |x| >= 2^e2
  return (int)((emu_bits(x) >> 52) & 0x7ffu) >= 1023 + e2;
}
template <class M>
__device__ __forceinline__ void rolling_clip_mur0_m(M& mm, V3 branch, V3 vrot_i, V3 fn, V3& mom_i);
__device__ __forceinline__ void rolling_clip_mur0(V3 branch, V3 vrot_i, V3 fn, V3& mom_i) {
  MulFP64 mm;
  rolling_clip_mur0_m(mm, branch, vrot_i, fn, mom_i);
}
template <class M>
__device__ __forceinline__ void rolling_clip_mur0_m(M& mm, V3 branch, V3 vrot_i, V3 fn, V3& mom_i) {
  // w = +-0: r = (b.w)/(w.w) is (+-0 or NaN)/(+0) = NaN for any b, so t = NaN and
  // the comparison with t^2 is false: the moment is kept as it is
  if (((emu_bits(vrot_i.x) | emu_bits(vrot_i.y) | emu_bits(vrot_i.z)) << 1) == 0) return;
  const bool in_range = exp_below(branch.x, 200) && exp_below(branch.y, 200) && exp_below(branch.z, 200) &&
                        exp_below(fn.x, 500) && exp_below(fn.y, 500) && exp_below(fn.z, 500) &&
                        exp_below(vrot_i.x, 200) && exp_below(vrot_i.y, 200) && exp_below(vrot_i.z, 200) &&
                        (exp_at_least(vrot_i.x, -200) || exp_at_least(vrot_i.y, -200) ||
                         exp_at_least(vrot_i.z, -200));
  const double mom_square = dot_m(mm, mom_i, mom_i);
  if (in_range) {
    if (emu_gt0(mom_square)) mom_i = mk(mm.mul(mom_i.x, 0.0), mm.mul(mom_i.y, 0.0), mm.mul(mom_i.z, 0.0));
    return;
  }
  const double r = (dot(branch, vrot_i)) / (dot(vrot_i, vrot_i));
  branch = branch - r * vrot_i;
  const double mur = 0;
  const double threshold_mom = fabs(mur * vnorm(branch) * vnorm(fn));
  if (mom_square > 0.0 && mom_square > threshold_mom * threshold_mom)
    mom_i = mom_i * (threshold_mom / sqrt(mom_square));
}

template <class M>
__device__ __forceinline__ V3 cross_m(M& mm, V3 a, V3 b) {
  return mk(mm.sub(mm.mul(a.y, b.z), mm.mul(a.z, b.y)), mm.sub(mm.mul(a.z, b.x), mm.mul(a.x, b.z)),
            mm.sub(mm.mul(a.x, b.y), mm.mul(a.y, b.x)));
}
template <class M>
__device__ __forceinline__ double dot_m(M& mm, V3 a, V3 b) {
  return mm.add(mm.add(mm.mul(a.x, b.x), mm.mul(a.y, b.y)), mm.mul(a.z, b.z));
}
template <class M>
__device__ __forceinline__ V3 add_m(M& mm, V3 a, V3 b) {
  return mk(mm.add(a.x, b.x), mm.add(a.y, b.y), mm.add(a.z, b.z));
}
template <class M>
__device__ __forceinline__ V3 sub_m(M& mm, V3 a, V3 b) {
  return mk(mm.sub(a.x, b.x), mm.sub(a.y, b.y), mm.sub(a.z, b.z));
}
template <class M>
__device__ __forceinline__ V3 scale_m(M& mm, double s, V3 a) {
  return mk(mm.mul(s, a.x), mm.mul(s, a.y), mm.mul(s, a.z));
}

// contact_force_core below with its multiplies through mm, in the same
// operation order, and the rolling clip through rolling_clip_mur0 (same
// result); the clip's arithmetic keeps the FP64 pipe.
// With Damp, `meff` carries the pair's damping coefficient damp_rate 2
// sqrt(kn meff) itself, computed with the same operations when the list was
// built (IArrays::damp), instead of the effective mass.
template <class M, bool Damp = false>
__device__ __forceinline__ void contact_force_core_m(M& mm, bool cohesive, double dn, V3 n, double dt,
                                                     const dem_contact_params& hkp, double meff, V3& ft, V3 cpos,
                                                     V3 pos_i, V3 vel_i, V3& f_i, V3& mom_i, V3 vrot_i, V3 pos_j,
                                                     V3 vel_j, V3 vrot_j, bool dmt = false, double reff = 0.0) {
  if (cohesive) {
    if (emu_ge0(dn)) {  // comparisons of this form on the integer pipe (emu64.cuh)
      const double fn_value = mm.sub(mm.mul(hkp.fc / hkp.dncut, dn), hkp.fc);
      f_i = add_m(mm, f_i, scale_m(mm, fn_value, n));
      ft = mk(0, 0, 0);
      return;
    }
  }
  const double damp = Damp ? meff : mm.mul(mm.twice(hkp.damp_rate), sqrt(mm.mul(hkp.kn, meff)));
  const V3 contribution_i = sub_m(mm, vel_i, cross_m(mm, sub_m(mm, cpos, pos_i), vrot_i));
  const V3 contribution_j = sub_m(mm, vel_j, cross_m(mm, sub_m(mm, cpos, pos_j), vrot_j));
  const V3 vel = sub_m(mm, contribution_j, contribution_i);
  const double vn = dot_m(mm, vel, n);
  V3 fn;
  {
    const double fne = mm.mul(-hkp.kn, dn);
    const double fnv = mm.mul(damp, vn);
    const double s = mm.add(fnv, fne);
    double nf = emu_gt0(s) ? s : 0;
    if (cohesive) {
      const double fn_norm = mm.sub(nf, hkp.fc);
      nf = emu_lt(fn_norm, -hkp.fc) ? -hkp.fc : fn_norm;
    }
    fn = scale_m(mm, nf, n);
  }
  {
    const V3 vt = sub_m(mm, vel, scale_m(mm, vn, n));
    const V3 ftd = scale_m(mm, dt, vt);
    ft = add_m(mm, ft, scale_m(mm, hkp.kt, ftd));
  }
  double threshold_ft;
  if (!cohesive) {
    const double fne = mm.mul(hkp.kn, dn);
    threshold_ft = fabs(mm.mul(hkp.mu, fne));
  } else {
    threshold_ft = fabs(mm.mul(hkp.mu, mm.add(dot_m(mm, fn, n), hkp.fc)));
  }
  {
    const double ft_square = dot_m(mm, ft, ft);
    if (emu_gt0(ft_square) && emu_gt_nonneg(ft_square, mm.mul(threshold_ft, threshold_ft))) {
      const double s = threshold_ft / sqrt(ft_square);
      ft = mk(mm.mul(ft.x, s), mm.mul(ft.y, s), mm.mul(ft.z, s));
    }
  }
  f_i = add_m(mm, fn, ft);
  if (dmt && hkp.gamma > 0.0 && emu_lt0(dn)) {
    const double F = mm.mul(mm.mul(2.0 * 3.14159265358979323846, reff), hkp.gamma);
    f_i = sub_m(mm, f_i, scale_m(mm, F, n));
  }
  {
    const V3 d = sub_m(mm, vrot_j, vrot_i);
    mom_i = add_m(mm, mom_i, mk(mm.mul(mm.mul(hkp.kr, d.x), dt), mm.mul(mm.mul(hkp.kr, d.y), dt),
                                mm.mul(mm.mul(hkp.kr, d.z), dt)));
  }
  rolling_clip_mur0_m(mm, sub_m(mm, cpos, pos_i), vrot_i, fn, mom_i);
}

// apply_dmt_force (contact_force.hpp:115-127): in contact (dn < 0) and for
// gamma > 0, f_i -= (2 pi reff gamma) n, the operation order of the reference
__device__ __forceinline__ double dmt_magnitude(double reff, double gamma) {
  return 2.0 * 3.14159265358979323846 * reff * gamma;
}

// contact_force_core (contact_force.hpp:146-235).  f_i must be {0,0,0} on entry.
// dmt: the Hooke_DMT law combination (contact_force.hpp:70-76) with reff the
// effective radius of the pair.
__device__ __forceinline__ void contact_force_core(bool cohesive, double dn, V3 n, double dt, const dem_contact_params& hkp,
                                          double meff, V3& ft, V3 cpos, V3 pos_i, V3 vel_i, V3& f_i, V3& mom_i,
                                          V3 vrot_i, V3 pos_j, V3 vel_j, V3 vrot_j, bool dmt = false,
                                          double reff = 0.0) {
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
  if (dmt && hkp.gamma > 0.0 && dn < 0.0) f_i = f_i - dmt_magnitude(reff, hkp.gamma) * n;
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
