// Forward-mode derivatives of a calibration path with respect to its primary ray direction d0 (three tangents, one
// per component of d0), and the Jacobian of the KB4 camera ray with respect to the intrinsics (fx, fy, cx, cy,
// k1..k4). They give the image loss's derivative in the intrinsics through everything that moves smoothly with the
// ray: the hit points (plane of the hit triangle), the interpolated shading and emitter normals, every light sample's
// weight (distance, cosines, power-heuristic MIS, the emission profile), the cosine-sampled continuation and the
// emitter hit's MIS weight. What changes in steps (the triangle a ray hits, a shadow ray's outcome, a node's
// radiosity) is held fixed: the edge term of the derivative is not taken.
//
// The values of the path are the estimator's own (bit for bit the forward's); the tangents are separate arithmetic.
#pragma once

#include "vt_device.cuh"

namespace vtk {
using namespace vtd;

// derivative of a 3-vector with respect to d0: c[j] = d vec / d d0_j
struct Tan3 { float3 c[3]; };

__device__ __forceinline__ Tan3 tan_zero() { Tan3 t; t.c[0] = t.c[1] = t.c[2] = f3(0, 0, 0); return t; }
__device__ __forceinline__ Tan3 tan_identity() { Tan3 t; t.c[0] = f3(1, 0, 0); t.c[1] = f3(0, 1, 0); t.c[2] = f3(0, 0, 1); return t; }
// derivative of a . v for a fixed a
__device__ __forceinline__ float3 tan_dot(float3 a, const Tan3& v) { return f3(dot(a, v.c[0]), dot(a, v.c[1]), dot(a, v.c[2])); }
__device__ __forceinline__ float3 mul3(float3 a, float3 b) { return f3(a.x * b.x, a.y * b.y, a.z * b.z); }

// hit of the ray o + t d on the plane with normal N (the hit triangle's): t = N.(v0 - o) / N.d, so
// dt = -N.(do + t dd) / N.d and dx = do + t dd + d dt
__device__ __forceinline__ void tan_plane_hit(const Tan3& Jo, const Tan3& Jd, float3 d, float3 N, float t, Tan3& Jx, float3& dt) {
  const float nd = dot(N, d);
  float dtv[3];
  for (int j = 0; j < 3; j++) {
    const float3 a = Jo.c[j] + Jd.c[j] * t;
    dtv[j] = -dot(N, a) / nd;
    Jx.c[j] = a + d * dtv[j];
  }
  dt = f3(dtv[0], dtv[1], dtv[2]);
}

// normalized barycentric interpolation of the hit triangle's vertex normals, rotated with its instance; returns the
// unit normal and its derivative (the hit moves in the triangle's plane: u = c1 . (x - v0), v = c2 . (x - v0))
__device__ __forceinline__ float3 tan_interp_normal(const Scene& S, const Hit& h, const Surf& s, float time, const Tan3& Jx, Tan3& Jn) {
  const float4* r = S.tris + 4u * h.tri;
  float3 e1 = xyz(__ldg(r + 1)), e2 = xyz(__ldg(r + 2));
  float3 n0 = vnormal(S, s.vi0), n1 = vnormal(S, s.vi1), n2 = vnormal(S, s.vi2);
  if (h.inst != MISS) {
    Rot R;
    float3 p;
    inst_pose(S, h.inst, time, R, p);
    e1 = rmul(R, e1); e2 = rmul(R, e2);
    n0 = rmul(R, n0); n1 = rmul(R, n1); n2 = rmul(R, n2);
  }
  const float3 N = cross(e1, e2);
  const float inv = 1.0f / dot(N, N);
  const float3 c1 = cross(e2, N) * inv, c2 = cross(N, e1) * inv;
  const float3 m = n0 * s.b.x + n1 * s.b.y + n2 * s.b.z;
  const float ml = length(m);
  const float3 mh = m / ml;
  for (int j = 0; j < 3; j++) {
    const float du = dot(c1, Jx.c[j]), dv = dot(c2, Jx.c[j]);
    const float3 dm = (n1 - n0) * du + (n2 - n0) * dv;
    Jn.c[j] = (dm - mh * dot(mh, dm)) / ml;
  }
  return mh;
}

// derivative of the surface's shading normal s.ns: the interpolated normal with the two-sided flips; where the
// estimator replaced it by the geometric normal (grazing view) or the vertex normals are the face's, it is fixed
__device__ __forceinline__ Tan3 tan_shading_normal(const Scene& S, const Hit& h, const Surf& s, float time, const Tan3& Jx) {
  Tan3 Jn = tan_zero();
  if (s.ns.x == s.ng.x && s.ns.y == s.ng.y && s.ns.z == s.ng.z) return Jn;
  const float3 mh = tan_interp_normal(S, h, s, time, Jx, Jn);
  if (dot(mh, s.ns) < 0.0f)
    for (int j = 0; j < 3; j++) Jn.c[j] = -Jn.c[j];
  return Jn;
}

// slope dp/dtheta of the piecewise-linear emission profile on the segment profile() interpolates (0 past the last
// knot)
__device__ __forceinline__ float profile_slope(const Scene& S, float th) {
  const float4 last = __ldg(S.params + S.prof_off + S.prof_n - 1u);
  if (th >= last.x) return 0.0f;
  uint32_t lo = 0, hi = S.prof_n - 1u;
  for (uint32_t it = 0; it < 40u && hi - lo > 1u; it++) {
    const uint32_t m = (lo + hi) >> 1;
    if (__ldg(S.params + S.prof_off + m).x <= th) lo = m; else hi = m;
  }
  const float4 a = __ldg(S.params + S.prof_off + lo), b = __ldg(S.params + S.prof_off + hi);
  const float w = b.x - a.x;
  if (w <= 1e-12f) return 0.0f;
  const float f = (th - a.x) / w;
  return (f > 0.0f && f < 1.0f) || (f == 0.0f) ? (b.y - a.y) / w : 0.0f;
}

// d theta for theta = acos(c) given dc (0 at |c| = 1)
__device__ __forceinline__ float3 tan_acos(float c, float3 dc) {
  const float s2 = 1.0f - c * c;
  return s2 > 0.0f ? dc * (-1.0f / sqrtf(s2)) : f3(0, 0, 0);
}

// one light sample's contribution per unit emitter radiance and albedo, q = prof cosS w / (pi pdfW) with
// pdfW = d2 / (cosE area), pb = cosS / pi, w = nl^2 pdfW^2 / (nl^2 pdfW^2 + pb^2) (gpu/wgsl/shade.wgsl.js:135
// lightEval), and its derivative, for a fixed emitter point lp (normal ln, axis la) seen from x with normal n
__device__ __forceinline__ float3 tan_light(const Scene& S, float3 x, float3 n, float3 lp, float3 ln, float3 la, float area, float fnl, float q,
                                           const Tan3& Jx, const Tan3& Jn) {
  const float3 wi = lp - x;
  const float d2 = dot(wi, wi), dist = sqrtf(d2);
  const float3 w = wi / dist;
  const float cosE = dot(-w, ln), cosS = dot(n, w);
  const float c = clampf(dot(-w, la), -1.0f, 1.0f);
  const float th = acosf(c);
  const float prof = profile(S, th), slope = profile_slope(S, th);
  const float pdfW = d2 / (cosE * area), pb = cosS * INV_PI_F;
  const float A = fnl * fnl * pdfW * pdfW, B = pb * pb, AB = A + B;
  const float wm = A / AB;
  float out[3];
  for (int j = 0; j < 3; j++) {
    const float3 dwi = -Jx.c[j];
    const float dd2 = 2.0f * dot(wi, dwi);
    const float3 dw = (dwi - w * dot(w, dwi)) / dist;
    const float dcosE = -dot(ln, dw);
    const float dcosS = dot(Jn.c[j], w) + dot(n, dw);
    const float dc = -dot(la, dw);
    const float dth = (1.0f - c * c) > 0.0f ? -dc / sqrtf(1.0f - c * c) : 0.0f;
    const float dprof = slope * dth;
    const float dpdf = (dd2 * cosE - d2 * dcosE) / (cosE * cosE * area);
    const float dpb = dcosS * INV_PI_F;
    const float dA = 2.0f * fnl * fnl * pdfW * dpdf, dB = 2.0f * pb * dpb;
    const float dwm = (dA * B - A * dB) / (AB * AB);
    out[j] = (dprof * cosS * wm + prof * dcosS * wm + prof * cosS * dwm) * INV_PI_F / pdfW - q * dpdf / pdfW;
  }
  return f3(out[0], out[1], out[2]);
}

// the orthonormal basis of basis_t / basis_b (the sign s of n.z held) and its derivative along dn
__device__ __forceinline__ void tan_basis(float3 n, float3 dn, float3& dt, float3& db) {
  const float s = n.z >= 0.0f ? 1.0f : -1.0f;
  const float a = -1.0f / (s + n.z), b = n.x * n.y * a;
  const float da = a * a * dn.z;
  const float dbv = dn.x * n.y * a + n.x * dn.y * a + n.x * n.y * da;
  dt = f3(s * (2.0f * n.x * dn.x * a + n.x * n.x * da), s * dbv, -s * dn.x);
  db = f3(dbv, 2.0f * n.y * dn.y * a + n.y * n.y * da, -dn.y);
  (void)b;
}

// the cosine-sampled continuation l = t (r cos phi) + b (r sin phi) + n sqrt(1 - u1) and its derivative
__device__ __forceinline__ Tan3 tan_continue(float3 n, const Tan3& Jn, float r, float cphi, float sphi, float sq) {
  Tan3 Jl;
  for (int j = 0; j < 3; j++) {
    float3 dt, db;
    tan_basis(n, Jn.c[j], dt, db);
    Jl.c[j] = dt * (r * cphi) + db * (r * sphi) + Jn.c[j] * sq;
  }
  return Jl;
}

// the camera sub-sample's ray d0 = normalize(R dc), dc = kb4Unproject(K, u, v) (8 Newton steps on theta), and the
// Jacobian d d0 / d K (three rows, eight columns: fx, fy, cx, cy, k1..k4) at the converged theta: with
// f(theta) = theta (1 + k1 theta^2 + ...) = theta_d, d theta / d theta_d = 1 / f'(theta) and
// d theta / d k_i = -theta^(2i+1) / f'(theta) (gpu/lens.js:25 distortDeriv is f')
__device__ __forceinline__ void kb4_ray_jacobian(const Kb4& L, float u, float v, float3 rx, float3 ry, float3 rz, float J[3][8]) {
  const float yd = (v - L.cy) / L.fy;
  const float xd = (u - L.cx) / L.fx - L.alpha * yd;
  const float thd = sqrtf(xd * xd + yd * yd);
  // d(xd, yd) / d(fx, fy, cx, cy)
  const float dyd[4] = {0.0f, -yd / L.fy, 0.0f, -1.0f / L.fy};
  const float dxd[4] = {-(xd + L.alpha * yd) / L.fx, -L.alpha * dyd[1], -1.0f / L.fx, -L.alpha * dyd[3]};
  float3 dc[8];
  if (thd < 1e-12f) {
    for (int k = 0; k < 4; k++) dc[k] = f3(dxd[k], dyd[k], 0.0f);
    for (int k = 4; k < 8; k++) dc[k] = f3(0, 0, 0);
  } else {
    float th = thd;
    for (int i = 0; i < 8; i++) {
      const float t2 = th * th;
      const float f = th * (1.0f + t2 * (L.k0 + t2 * (L.k1 + t2 * (L.k2 + t2 * L.k3)))) - thd;
      const float fp = 1.0f + t2 * (3.0f * L.k0 + t2 * (5.0f * L.k1 + t2 * (7.0f * L.k2 + t2 * 9.0f * L.k3)));
      th = th - f / fp;
    }
    const float t2 = th * th;
    const float fp = 1.0f + t2 * (3.0f * L.k0 + t2 * (5.0f * L.k1 + t2 * (7.0f * L.k2 + t2 * 9.0f * L.k3)));
    float sn, cs;
    sincosf(th, &sn, &cs);
    const float S_ = sn / thd;
    // dc = (xd S, yd S, cos theta), S = sin theta / theta_d; through (xd, yd) and through theta
    const float dS_dth = cs / thd;
    for (int k = 0; k < 4; k++) {
      const float dthd = (xd * dxd[k] + yd * dyd[k]) / thd;
      const float dth = dthd / fp;
      const float dS = dS_dth * dth - sn * dthd / (thd * thd);
      dc[k] = f3(dxd[k] * S_ + xd * dS, dyd[k] * S_ + yd * dS, -sn * dth);
    }
    float tp = th * t2;
    for (int k = 4; k < 8; k++) {
      const float dth = -tp / fp;
      dc[k] = f3(xd * dS_dth * dth, yd * dS_dth * dth, -sn * dth);
      tp *= t2;
    }
  }
  // d0 = normalize(R dc): the projection off d0 of R ddc
  const float3 dcv = kb4_unproject(L, u, v);
  const float3 w = rx * dcv.x + ry * dcv.y + rz * dcv.z;
  const float wl = length(w);
  const float3 d0 = w / wl;
  for (int k = 0; k < 8; k++) {
    const float3 g = rx * dc[k].x + ry * dc[k].y + rz * dc[k].z;
    const float3 p = (g - d0 * dot(d0, g)) / wl;
    J[0][k] = p.x; J[1][k] = p.y; J[2][k] = p.z;
  }
}

}  // namespace vtk
