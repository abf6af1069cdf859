// k_selftest_poly.cu -- GPU self-test of the FP32 decisions of the polyhedron
// broad phase (poly_f32.cuh) against the FP64 tests they stand in for
// (poly_core.cuh).  Every case is drawn close to a threshold of its test --
// separating-axis boundaries of the vertex gate, |d| = R, the edge parameter
// bounds, face planes and face edges, near-parallel edges -- at offsets from
// 1e-10 to 1e-1 of the particle size, with world coordinates up to 1e2 times
// the particle size away from the origin.  A decided FP32 result must equal
// the FP64 one.
#include "../../include/dem_selftest.h"
#include "dem_ctx.cuh"
#include "poly_core.cuh"
#include "poly_f32.cuh"

namespace dem {
namespace {
struct Rng {
  uint64_t s;
  __device__ uint64_t next() {  // splitmix64
    uint64_t x = (s += 0x9e3779b97f4a7c15ull);
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
    return x ^ (x >> 31);
  }
  __device__ double uni() { return (double)(next() >> 11) * 0x1.0p-53; }
  __device__ double uni(double a, double b) { return a + (b - a) * uni(); }
  __device__ V3 vec(double s) { return mk(uni(-s, s), uni(-s, s), uni(-s, s)); }
  __device__ V3 unit() {
    for (;;) {
      const V3 v = vec(1.0);
      const double l = vnorm(v);
      if (l > 0.1 && l <= 1.0) return v / l;
    }
  }
  // signed offset of magnitude 10^U(-10, -1) times s
  __device__ double eps(double s) {
    const double m = s * pow(10.0, uni(-10.0, -1.0));
    return (next() & 1) ? m : -m;
  }
};

__device__ void frame(Rng& g, V3& a, V3& b, V3& c) {
  a = g.unit();
  const V3 h = fabs(a.x) < 0.9 ? mk(1, 0, 0) : mk(0, 1, 0);
  b = cross(a, h);
  b = b / vnorm(b);
  c = cross(a, b);
}

__device__ __forceinline__ F3 rel32(V3 v, V3 o) { return f3((float)(v.x - o.x), (float)(v.y - o.y), (float)(v.z - o.z)); }

struct Case {
  int kind;
  int exact;
  int dec;
};

__device__ Case run_case(uint64_t seed, uint64_t t) {
  Rng g{seed * 0x2545f4914f6cdd1dull + t * 0x9e3779b97f4a7c15ull};
  g.next();
  const int kind = (int)(t % 6);
  const double sc = pow(10.0, g.uni(-3.0, 1.0));  // particle size
  const V3 pA = g.vec(100.0 * sc);
  const V3 pB = pA + g.unit() * (g.uni(0.0, 3.0) * sc);
  const F3 dR = rel32(pB, pA);
  const double ra = g.uni(0.0, 0.1) * sc, rb = g.uni(0.0, 0.1) * sc, rV = g.uni(0.0, 0.1) * sc;
  const double R = ra + rb + rV;
  const float Rf = (float)R, rVf = (float)rV;
  auto relB = [&](V3 v) { return rel32(v, pB) + dR; };
  Case out{kind, 0, DEC_UNDECIDED};
  switch (kind) {
    case 0: {  // vertex gate
      OBBd o;
      o.c = pB + g.vec(0.5 * sc);
      frame(g, o.e1, o.e2, o.e3);
      if (g.next() & 1) {  // axes along the world axes up to a rotation of 1e-17 .. 1e-6 (cube covariance OBBs)
        const double tilt = pow(10.0, g.uni(-17.0, -6.0));
        V3 a = mk(1.0, tilt * g.uni(-1.0, 1.0), tilt * g.uni(-1.0, 1.0));
        a = a / vnorm(a);
        V3 b = cross(mk(tilt * g.uni(-1.0, 1.0), tilt * g.uni(-1.0, 1.0), 1.0), a);
        b = b / vnorm(b);
        o.e1 = a;
        o.e2 = b;
        o.e3 = cross(a, b);
      }
      o.ext = mk(g.uni(0.1, 1.0) * sc, g.uni(0.1, 1.0) * sc, g.uni(0.1, 1.0) * sc);
      const double rv = g.uni(0.0, 0.05) * sc;
      // a point near the enlarged box surface (face, edge or corner region)
      double q[3];
      const double ex[3] = {o.ext.x, o.ext.y, o.ext.z};
      const int k = (int)(g.next() % 3);
      for (int l = 0; l < 3; l++) q[l] = g.uni(-1.1, 1.1) * (ex[l] + 2.0 * rv);
      q[k] = ((g.next() & 1) ? 1.0 : -1.0) * (ex[k] + rv * g.uni(0.5, 2.5)) + g.eps(sc);
      if (g.next() & 1) {  // edge / corner region: push a second coordinate out as well
        const int k2 = (k + 1 + (int)(g.next() % 2)) % 3;
        q[k2] = ((g.next() & 1) ? 1.0 : -1.0) * (ex[k2] + rv * g.uni(0.0, 2.0)) + g.eps(sc);
      }
      const V3 p = o.c + o.e1 * q[0] + o.e2 * q[1] + o.e3 * q[2];
      OBBd ov;
      ov.c = p;
      ov.e1 = mk(1, 0, 0);
      ov.e2 = mk(0, 1, 0);
      ov.e3 = mk(0, 0, 1);
      ov.ext = mk(0, 0, 0);
      obb_enlarge(ov, rv);
      out.exact = obb_intersect(o, ov);
      const F3 fp = rel32(p, pA);
      const float S = flen(fp) * 1.001f + (float)rv;
      out.dec = decide_gate(obb_f32(o, pA), fp, (float)rv, S);
      break;
    }
    case 1: {  // vertex - vertex
      const V3 vi = pA + g.vec(sc);
      const V3 vj = vi + g.unit() * (R + g.eps(sc));
      out.exact = filter_vv(rV, vi, ra, vj, rb);
      const F3 a = rel32(vi, pA), b = relB(vj);
      const float S = fmaxf(flen(a), flen(b)) * 1.001f + Rf;
      out.dec = decide_vv(a, b, Rf, S);
      break;
    }
    case 2: {  // vertex - edge
      const V3 vf = pB + g.vec(sc);
      const V3 dir = g.unit();
      const V3 E = dir * (g.uni(0.1, 1.0) * sc);
      const int mode = (int)(g.next() % 3);
      const double r0 = mode == 0 ? -rV + g.eps(1.0) : (mode == 1 ? 1.0 + rV + g.eps(1.0) : g.uni(-0.2, 1.2));
      V3 pa, pb, pc;
      frame(g, pa, pb, pc);
      V3 perp = cross(dir, pa);
      perp = perp / vnorm(perp);
      const double d0 = (g.next() & 1) ? R + g.eps(sc) : g.uni(0.0, 2.0) * R;
      const V3 vi = vf + E * r0 + perp * d0;
      out.exact = filter_ve(rV, vi, ra, vf, vf + E, rb);
      const F3 a = rel32(vi, pA), f = relB(vf), s = relB(vf + E);
      const float S = fmaxf(flen(a), fmaxf(flen(f), flen(s))) * 1.001f + Rf;
      out.dec = decide_ve(a, f, s, Rf, rVf, S);
      break;
    }
    case 3: {  // vertex - face (a convex polygon of 3 to 6 vertices)
      const int nfv = 3 + (int)(g.next() % 4);
      V3 u1, u2, nn;
      frame(g, nn, u1, u2);
      const V3 c = pB + g.vec(0.5 * sc);
      const double rho = g.uni(0.2, 1.0) * sc;
      const double ph = g.uni(0.0, 6.283185307179586);
      ShapeDev sf;
      sf.nv = nfv;
      sf.ne = 0;
      sf.nf = 1;
      sf.fo[0] = 0;
      sf.fo[1] = nfv;
      double vx[6], vy[6], vz[6];
      float fx[6], fy[6], fz[6];
      double px[6], py[6];
      for (int k = 0; k < nfv; k++) {
        const double an = ph + 6.283185307179586 * (k + g.uni(-0.2, 0.2)) / nfv;
        px[k] = rho * cos(an);
        py[k] = rho * sin(an);
        const V3 v = c + u1 * px[k] + u2 * py[k];
        vx[k] = v.x;
        vy[k] = v.y;
        vz[k] = v.z;
        const F3 fv = rel32(v, pB);
        fx[k] = fv.x;
        fy[k] = fv.y;
        fz[k] = fv.z;
        sf.fv[k] = k;
      }
      // in-plane point: near an edge, at the level of a vertex along the test's v2 axis, or anywhere
      const int mode = (int)(g.next() % 3);
      double x, y;
      if (mode == 0) {
        const int k = (int)(g.next() % nfv), k1 = (k + 1) % nfv;
        const double s = g.uni(0.0, 1.0);
        const double ex = px[k1] - px[k], ey = py[k1] - py[k];
        const double el = sqrt(ex * ex + ey * ey);
        const double off = g.eps(sc);
        x = px[k] + s * ex + off * ey / el;
        y = py[k] + s * ey - off * ex / el;
      } else if (mode == 1) {
        // v1 = direction of edge 0 -> 1; shift along v1 from a vertex by a random amount
        const int k = (int)(g.next() % nfv);
        const double ex = px[1] - px[0], ey = py[1] - py[0];
        const double el = sqrt(ex * ex + ey * ey);
        const double w = g.uni(-1.5, 1.5) * rho;
        const double off = g.eps(sc);
        x = px[k] + w * ex / el - off * ey / el;
        y = py[k] + w * ey / el + off * ex / el;
      } else {
        x = g.uni(-1.2, 1.2) * rho;
        y = g.uni(-1.2, 1.2) * rho;
      }
      const double h = (g.next() & 1) ? (R + g.eps(sc)) * ((g.next() & 1) ? 1 : -1) : g.uni(-2.0, 2.0) * R;
      const V3 vi = c + u1 * x + u2 * y + nn * h;
      const VView vv{vx, vy, vz};
      out.exact = filter_vf(rV, vi, ra, vv, sf, 0, rb);
      const FView fv{fx, fy, fz, dR};
      const F3 a = rel32(vi, pA);
      float S = flen(a);
      for (int k = 0; k < nfv; k++) S = fmaxf(S, flen(fv[k]));
      S = S * 1.001f + Rf;
      out.dec = decide_vf(a, fv, sf, 0, Rf, S);
      break;
    }
    case 5: {  // vertex displacement since the last rebuild against max_displ
      const V3 p = pA;
      const double h = g.uni(0.5, 2.0);
      const V3 v0 = g.vec(sc);
      Q4 q = {g.uni(-1, 1), g.uni(-1, 1), g.uni(-1, 1), g.uni(-1, 1)};
      const double qs = (g.next() % 4 == 0 ? g.uni(0.98, 1.02) : 1.0) /
                        sqrt(q.w * q.w + q.x * q.x + q.y * q.y + q.z * q.z);
      q = {q.w * qs, q.x * qs, q.y * qs, q.z * qs};
      // backup orientation: q turned by a small angle about a random axis
      const V3 ax = g.unit();
      const double an = g.uni(0.0, 0.2) * ((g.next() & 1) ? 1.0 : 1e-3);
      const Q4 dq = {cos(0.5 * an), ax.x * sin(0.5 * an), ax.y * sin(0.5 * an), ax.z * sin(0.5 * an)};
      const Q4 qb = {dq.w * q.w - dq.x * q.x - dq.y * q.y - dq.z * q.z, dq.w * q.x + dq.x * q.w + dq.y * q.z - dq.z * q.y,
                     dq.w * q.y - dq.x * q.z + dq.y * q.w + dq.z * q.x, dq.w * q.z + dq.x * q.y - dq.y * q.x + dq.z * q.w};
      const double md = g.uni(0.001, 0.1) * sc;
      // backup centre placing the backup vertex at md (+ a small offset) from the current one
      const V3 v = p + qrotate(q, h * v0);
      const V3 pb = v - qrotate(qb, h * v0) - g.unit() * (md + g.eps(sc));
      const V3 b = pb + qrotate(qb, h * v0);
      const V3 dr = v - b;
      out.exact = dot(dr, dr) >= md * md;
      const float4 qn = make_float4((float)q.w, (float)q.x, (float)q.y, (float)q.z);
      const float4 qbf = make_float4((float)qb.w, (float)qb.x, (float)qb.y, (float)qb.z);
      const float q2 = fmaxf(fmaxf(qn.x * qn.x + qn.y * qn.y + qn.z * qn.z + qn.w * qn.w,
                                   qbf.x * qbf.x + qbf.y * qbf.y + qbf.z * qbf.z + qbf.w * qbf.w),
                             1.f);
      const F3 dp = f3((float)(p.x - pb.x), (float)(p.y - pb.y), (float)(p.z - pb.z));
      const F3 v0h = f3((float)v0.x, (float)v0.y, (float)v0.z) * (float)h;
      out.dec = decide_displ(dp, qn, qbf, v0h, q2, (float)(fabs(p.x) + fabs(p.y) + fabs(p.z)), (float)md);
      break;
    }
    default: {  // edge - edge
      const V3 di = g.unit();
      V3 dj;
      if (g.next() % 4 == 0) {  // near parallel
        V3 p1, p2, p3;
        frame(g, p1, p2, p3);
        dj = di + cross(di, p1) * pow(10.0, g.uni(-9.0, -1.0));
        dj = dj / vnorm(dj);
      } else {
        dj = g.unit();
      }
      const V3 Ei = di * (g.uni(0.1, 1.0) * sc), Ej = dj * (g.uni(0.1, 1.0) * sc);
      auto par = [&]() {
        const int m = (int)(g.next() % 3);
        return m == 0 ? g.eps(1.0) : (m == 1 ? 1.0 + g.eps(1.0) : g.uni(-0.2, 1.2));
      };
      const double s0 = par(), t0 = par();
      V3 nrm = cross(di, dj);
      const double nl = vnorm(nrm);
      if (nl > 1e-6) {
        nrm = nrm / nl;
      } else {
        V3 p1, p2, p3;
        frame(g, p1, p2, p3);
        nrm = cross(di, p1);
        nrm = nrm / vnorm(nrm);
      }
      const double d0 = (g.next() & 1) ? R + g.eps(sc) : g.uni(0.0, 2.0) * R;
      const V3 vfi = pA + g.vec(sc);
      const V3 pi = vfi + Ei * s0;
      const V3 pj = pi - nrm * d0;
      const V3 vfj = pj - Ej * t0;
      out.exact = filter_ee(rV, vfi, vfi + Ei, ra, vfj, vfj + Ej, rb);
      const F3 a0 = rel32(vfi, pA), a1 = rel32(vfi + Ei, pA), b0 = relB(vfj), b1 = relB(vfj + Ej);
      const float S = fmaxf(fmaxf(flen(a0), flen(a1)), fmaxf(flen(b0), flen(b1))) * 1.001f + Rf;
      out.dec = decide_ee(a0, a1, b0, b1, Rf, S);
      break;
    }
  }
  return out;
}

// counters: [kind][0] mismatches, [1] undecided, [2] decided true, [3] exact true
__global__ void k_poly_dec_test(uint64_t n, uint64_t seed, unsigned long long* cnt) {
  __shared__ unsigned long long sc[24];
  if (threadIdx.x < 24) sc[threadIdx.x] = 0;
  __syncthreads();
  for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (uint64_t)gridDim.x * blockDim.x) {
    const Case c = run_case(seed, t);
    if (c.dec != DEC_UNDECIDED && c.dec != c.exact) atomicAdd(&sc[c.kind * 4 + 0], 1ull);
    if (c.dec == DEC_UNDECIDED) atomicAdd(&sc[c.kind * 4 + 1], 1ull);
    if (c.dec == DEC_TRUE) atomicAdd(&sc[c.kind * 4 + 2], 1ull);
    if (c.exact) atomicAdd(&sc[c.kind * 4 + 3], 1ull);
  }
  __syncthreads();
  if (threadIdx.x < 24) atomicAdd(&cnt[threadIdx.x], sc[threadIdx.x]);
}
}  // namespace
}  // namespace dem

extern "C" int dem_selftest_poly_decisions(uint64_t n, uint64_t seed, uint64_t* counts) {
  if (!counts) return DEM_ERR_INVALID_ARG;
  unsigned long long* d = nullptr;
  if (cudaMalloc(&d, 24 * sizeof(unsigned long long)) != cudaSuccess) return DEM_ERR_CUDA;
  cudaMemset(d, 0, 24 * sizeof(unsigned long long));
  dem::k_poly_dec_test<<<608, 128>>>(n, seed, d);
  unsigned long long h[24];
  const bool ok = cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost) == cudaSuccess;
  cudaFree(d);
  if (!ok || cudaGetLastError() != cudaSuccess) return DEM_ERR_CUDA;
  for (int k = 0; k < 24; k++) counts[k] = h[k];
  return DEM_OK;
}
