// Device building blocks of the sm_103a hot path: sample numbers, the KB4 lens, the twin's BSDF, BVH2 traversal of
// the gpu/bvh.js node layout with the posed-body instance loop, surface records, emitter sampling and the two
// estimators (the twin's shadeHit and the depth-N path tracer). Float32 throughout, like the reference's WGSL.
//
// Data in HBM (all read-only during a launch, a few MB for the configs, so L2-resident):
//   nodes   float4[4 per node]   [c0.lo|ref][c0.hi|count][c1.lo|ref][c1.hi|count]     (gpu/bvh.js:5-11)
//   tris    float4[4 per tri]    v0|i0, e1|i1, e2|i2, (mesh, flags, -, -)              (gpu/scene_gpu.js:351-373)
//   verts   float4[2 per vert]   pos|mesh-or-u, normal|area-or-v                       (gpu/scene_gpu.js:375-393)
//   params  float4[]             mesh table | materials | albedo tables | profile | emitter triangles
//   su      float[24 + 48*24]    scene uniform: emitter, info, 24 instances            (gpu/wgsl/common.wgsl.js:60-77)
//   nstate  float4[4 per node]   node radiosity: E_free|V, Ls1, Ls2, B_dir|vis        (gpu/renderer.js:316-326)
#pragma once

#include <cstdint>

#include "../../include/vtwin.h"

namespace vtd {

constexpr float PI_F = 3.14159265358979f;
constexpr float INV_PI_F = 0.318309886183791f;
constexpr float BIG = 1e30f;
constexpr uint32_t MISS = 0xffffffffu;
constexpr float EPS_OFF = 2e-6f;
constexpr uint32_t STACK = 32;
constexpr uint32_t MAX_VISITS = 2048;
constexpr uint32_t MAX_LEAF = 64;

// debug counters (gpu/renderer.js:447 debugFlags)
enum { DBG_VISITS = 0, DBG_LEAF = 1, DBG_CORRUPT = 6 };

struct Scene {
  const float4* __restrict__ nodes;
  const float4* __restrict__ tris;
  const float4* __restrict__ verts;
  const float4* __restrict__ params;
  const float* __restrict__ su;
  const float4* __restrict__ nstate;
  uint32_t* dbg;
  uint32_t mesh_off, mat_off, alb_off, prof_off, prof_n, emit_off, emit_n;
  const float4* __restrict__ top;   // the static BVH's top levels, staged in shared memory by the traversal lanes
  uint32_t n_top, top_root;
};

// Top levels of the static BVH held in shared memory by the persistent traversal lanes: the first VT_TOP_NODES
// nodes of a breadth-first walk from the static root, each a copy of its 64-byte record whose interior-child
// references into the set are rewritten as TOP_BIT | slot (slot 0 is the root). A traversal started at TOP_BIT
// therefore reads these levels from shared memory and leaves the set through an ordinary global reference; the
// visit order, and so every hit and counter, is that of the global records. Off by default: on the 657k-triangle
// dome (640x480, 16 spp, depth 4) the frame takes 24.4 ms with 32 to 256 staged nodes against 21.9 ms without,
// images identical; the top levels already hit in L1.
#ifndef VT_TOP_NODES
#define VT_TOP_NODES 0
#endif
constexpr uint32_t TOP_NODES = VT_TOP_NODES;
constexpr uint32_t TOP_BIT = 0x80000000u;

// ------------------------------------------------------------------------------------------------ float3 math
__device__ __forceinline__ float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
__device__ __forceinline__ float3 xyz(float4 a) { return make_float3(a.x, a.y, a.z); }
__device__ __forceinline__ float3 operator+(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 operator-(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 operator-(float3 a) { return f3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ float3 operator*(float3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float3 operator*(float s, float3 a) { return f3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float3 operator*(float3 a, float3 b) { return f3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ float3 operator/(float3 a, float s) { return f3(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float3 cross(float3 a, float3 b) { return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
__device__ __forceinline__ float length(float3 a) { return sqrtf(dot(a, a)); }
__device__ __forceinline__ float3 normalize(float3 a) { return a / sqrtf(dot(a, a)); }
__device__ __forceinline__ float maxc(float3 a) { return fmaxf(a.x, fmaxf(a.y, a.z)); }
__device__ __forceinline__ float clampf(float x, float a, float b) { return fminf(fmaxf(x, a), b); }
__device__ __forceinline__ float3 mix3(float3 a, float3 b, float t) { return a * (1.0f - t) + b * t; }
__device__ __forceinline__ float lum(float3 c) { return c.x * 0.2126f + c.y * 0.7152f + c.z * 0.0722f; }
__device__ __forceinline__ uint32_t fu(float f) { return __float_as_uint(f); }

// ------------------------------------------------------------------------------------------------ sample numbers
// gpu/wgsl/common.wgsl.js:94-113: PCG hash, 24-bit uniforms, Kronecker sequences (rounding each product and sum
// separately, so every implementation draws the same numbers)
__device__ __forceinline__ uint32_t pcg(uint32_t v) {
  uint32_t s = v * 747796405u + 2891336453u;
  uint32_t w = ((s >> ((s >> 28u) + 4u)) ^ s) * 277803737u;
  return (w >> 22u) ^ w;
}
__device__ __forceinline__ uint32_t hash3(uint32_t a, uint32_t b, uint32_t c) { return pcg(a ^ pcg(b ^ pcg(c))); }
__device__ __forceinline__ float u01(uint32_t x) { return float(x >> 8u) * (1.0f / 16777216.0f); }
__device__ __forceinline__ float kr(uint32_t i, float a, float shift) {
  float s = __fadd_rn(shift, __fmul_rn(float(i), a));
  return __fsub_rn(s, floorf(s));
}
__device__ __forceinline__ float mixr(float a, float b, float t) { return __fadd_rn(__fmul_rn(a, __fsub_rn(1.0f, t)), __fmul_rn(b, t)); }
constexpr float R2A = 0.7548776662466927f, R2B = 0.5698402909980532f, GOLD = 0.6180339887498949f;
constexpr float KL0 = 0.41421356237f, KL1 = 0.73205080757f, KL2 = 0.23606797750f;
constexpr float KB0 = 0.64575131106f, KB1 = 0.31662479036f, KB2 = 0.60555127546f;

// per-pixel Kronecker shifts (gpu/wgsl/kernels.wgsl.js:34-38); hs kept for the path mode's deeper bounces
struct Seeds { float s[9]; uint32_t hs; };
__device__ __forceinline__ Seeds pixel_seeds(uint32_t x, uint32_t y, uint32_t seed, uint32_t cam) {
  Seeds S;
  S.hs = hash3(x, y, seed * 64u + cam);
#pragma unroll
  for (uint32_t k = 0; k < 9; k++) S.s[k] = u01(pcg(S.hs + k));
  return S;
}
// bounce b >= 2 of the path mode: light dims k = 0..2, BSDF dims k = 3..5
__device__ __forceinline__ float bounce_shift(uint32_t hs, uint32_t b, uint32_t k) { return u01(pcg(hs + 9u + 6u * (b - 2u) + k)); }

// ------------------------------------------------------------------------------------------------ KB4 lens
// theta_d = theta (1 + k1 theta^2 + k2 theta^4 + k3 theta^6 + k4 theta^8); pixel -> unit camera ray by 8 Newton
// steps on theta (gpu/wgsl/lens.wgsl.js:9-30; gpu/lens.js:54)
struct Kb4 { float fx, fy, cx, cy, alpha, k0, k1, k2, k3; };
__device__ __forceinline__ float3 kb4_unproject(const Kb4& L, float u, float v) {
  const float yd = (v - L.cy) / L.fy;
  const float xd = (u - L.cx) / L.fx - L.alpha * yd;
  const float thd = sqrtf(xd * xd + yd * yd);
  if (thd < 1e-20f) return f3(0.0f, 0.0f, 1.0f);
  float th = thd;
#pragma unroll
  for (int i = 0; i < 8; i++) {
    const float t2 = th * th;
    const float f = th * (1.0f + t2 * (L.k0 + t2 * (L.k1 + t2 * (L.k2 + t2 * L.k3)))) - thd;
    const float fp = 1.0f + t2 * (3.0f * L.k0 + t2 * (5.0f * L.k1 + t2 * (7.0f * L.k2 + t2 * 9.0f * L.k3)));
    th = th - f / fp;
  }
  float sn, cs;
  sincosf(th, &sn, &cs);
  const float s = sn / thd;
  return f3(xd * s, yd * s, cs);
}
// camera-frame point -> pixel (gpu/wgsl/lens.wgsl.js:32 kb4Project)
__device__ __forceinline__ float2 kb4_project(const Kb4& L, float3 X) {
  const float rho = sqrtf(X.x * X.x + X.y * X.y);
  if (rho < 1e-30f) return make_float2(L.cx, L.cy);
  const float th = atan2f(rho, X.z);
  const float t2 = th * th;
  const float s = th * (1.0f + t2 * (L.k0 + t2 * (L.k1 + t2 * (L.k2 + t2 * L.k3)))) / rho;
  const float xd = X.x * s, yd = X.y * s;
  return make_float2(L.fx * (xd + L.alpha * yd) + L.cx, L.fy * yd + L.cy);
}

// ------------------------------------------------------------------------------------------------ BSDF
// gpu/bsdf.js:4-18 (the WGSL copy gpu/wgsl/bsdf.wgsl.js:28-155)
struct Mat {
  float3 c; float alpha, ior, metal, fbar;
  float3 hh;
  float4 x;   // coated: tau rgb, alpha_coat
  uint32_t idx;
};
__device__ __forceinline__ Mat load_mat(const Scene& S, uint32_t m) {
  const float4* p = S.params + S.mat_off + 5u * m;
  const float4 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2), e = __ldg(p + 4);
  Mat M;
  M.c = xyz(a); M.alpha = a.w; M.ior = b.x; M.metal = b.y; M.fbar = b.z;
  M.hh = xyz(c); M.x = e; M.idx = m;
  return M;
}
__device__ __forceinline__ float fresnel(float cosi, float eta) {
  const float c = clampf(cosi, 0.0f, 1.0f);
  const float s2 = (1.0f - c * c) / (eta * eta);
  if (s2 >= 1.0f) return 1.0f;
  const float ct = sqrtf(1.0f - s2);
  const float rs = (c - eta * ct) / (c + eta * ct);
  const float rp = (eta * c - ct) / (eta * c + ct);
  return 0.5f * (rs * rs + rp * rp);
}
__device__ __forceinline__ float3 schlick3(float3 f0, float c) {
  const float m = powf(1.0f - clampf(c, 0.0f, 1.0f), 5.0f);   // gpu/wgsl/bsdf.wgsl.js:38: pow(1 - c, 5)
  return f0 + (f3(1.0f, 1.0f, 1.0f) - f0) * m;
}
__device__ __forceinline__ float3 fresnel_rgb(const Mat& M, float c) {
  if (M.metal > 0.5f) return schlick3(M.c, c);
  const float F = fresnel(c, M.ior);
  return f3(F, F, F);
}
__device__ __forceinline__ float ggx_d(float nh, float a) {
  if (nh <= 0.0f) return 0.0f;
  const float a2 = a * a, d = nh * nh * (a2 - 1.0f) + 1.0f;
  return a2 / (PI_F * d * d);
}
__device__ __forceinline__ float ggx_lambda(float c, float a) {
  const float c2 = fmaxf(c * c, 1e-12f);
  return 0.5f * (-1.0f + sqrtf(1.0f + a * a * ((1.0f - c2) / c2)));
}
__device__ __forceinline__ float ggx_g1(float c, float a) { return 1.0f / (1.0f + ggx_lambda(c, a)); }
__device__ __forceinline__ float ggx_g2(float l, float v, float a) { return 1.0f / (1.0f + ggx_lambda(l, a) + ggx_lambda(v, a)); }

__device__ __forceinline__ float3 eval_bsdf(const Mat& M, float3 n, float3 l, float3 v) {
  const float nl = dot(n, l), nv = dot(n, v);
  if (nl <= 0.0f || nv <= 0.0f) return f3(0, 0, 0);
  const float3 h = normalize(l + v);
  const float nh = dot(n, h), vh = fmaxf(0.0f, dot(v, h));
  if (M.metal > 1.5f) {
    const float ac = M.x.w;
    const float coat = ggx_d(nh, ac) * ggx_g2(nl, nv, ac) * fresnel(vh, M.ior) / (4.0f * nl * nv);
    const float t = (1.0f - fresnel(nl, M.ior)) * (1.0f - fresnel(nv, M.ior));
    const float metal = ggx_d(nh, M.alpha) * ggx_g2(nl, nv, M.alpha) / (4.0f * nl * nv);
    const float ex = 1.0f / nl + 1.0f / nv;
    const float3 tp = f3(powf(M.x.x, ex), powf(M.x.y, ex), powf(M.x.z, ex));
    return f3(coat, coat, coat) + tp * schlick3(M.c, vh) * (t * metal);
  }
  const float spec = ggx_d(nh, M.alpha) * ggx_g2(nl, nv, M.alpha) / (4.0f * nl * nv);
  float3 out = fresnel_rgb(M, vh) * spec;
  if (M.metal < 0.5f) {
    const float kd = INV_PI_F * (1.0f - fresnel(nl, M.ior)) * (1.0f - fresnel(nv, M.ior)) / (1.0f - M.fbar);
    out = out + M.c * kd;
  }
  return out;
}
__device__ __forceinline__ float3 basis_t(float3 n) {
  const float s = n.z >= 0.0f ? 1.0f : -1.0f;
  const float a = -1.0f / (s + n.z), b = n.x * n.y * a;
  return f3(1.0f + s * n.x * n.x * a, s * b, -s * n.x);
}
__device__ __forceinline__ float3 basis_b(float3 n) {
  const float s = n.z >= 0.0f ? 1.0f : -1.0f;
  const float a = -1.0f / (s + n.z), b = n.x * n.y * a;
  return f3(b, s + n.y * n.y * a, -n.y);
}
// visible GGX normal (Heitz 2018) for local view ve
__device__ __forceinline__ float3 sample_vndf(float3 ve, float a, float u1, float u2) {
  const float3 vh = normalize(f3(a * ve.x, a * ve.y, ve.z));
  const float lensq = vh.x * vh.x + vh.y * vh.y;
  const float3 T1 = lensq > 0.0f ? f3(-vh.y, vh.x, 0.0f) / sqrtf(lensq) : f3(1.0f, 0.0f, 0.0f);
  const float3 T2 = cross(vh, T1);
  const float r = sqrtf(u1);
  float sp, cp;
  sincosf(2.0f * PI_F * u2, &sp, &cp);
  const float t1 = r * cp;
  float t2 = r * sp;
  const float s = 0.5f * (1.0f + vh.z);
  t2 = (1.0f - s) * sqrtf(fmaxf(0.0f, 1.0f - t1 * t1)) + s * t2;
  const float t3 = sqrtf(fmaxf(0.0f, 1.0f - t1 * t1 - t2 * t2));
  const float3 nh = T1 * t1 + T2 * t2 + vh * t3;
  return normalize(f3(a * nh.x, a * nh.y, fmaxf(1e-7f, nh.z)));
}
__device__ __forceinline__ float spec_prob(const Mat& M, float nv) {
  if (M.metal > 1.5f) {
    const float Fc = fresnel(nv, M.ior);
    return Fc / (Fc + (1.0f - Fc) * (M.c.x + M.c.y + M.c.z) / 3.0f);
  }
  if (M.metal > 0.5f) return 1.0f;
  const float F = fresnel(nv, M.ior);
  const float d = lum(M.c) * (1.0f - F);
  const float s = fmaxf(F, 0.04f);
  return clampf(s / (s + d), 0.05f, 0.95f);
}
__device__ __forceinline__ float pdf_bsdf(const Mat& M, float3 n, float3 v, float3 l) {
  const float nl = dot(n, l), nv = dot(n, v);
  if (nl <= 0.0f || nv <= 0.0f) return 0.0f;
  const float3 h = normalize(l + v);
  const float nh = dot(n, h), vh = dot(v, h);
  const float ps = spec_prob(M, nv);
  if (M.metal > 1.5f) {
    if (vh <= 0.0f) return 0.0f;
    return ps * ggx_g1(nv, M.x.w) * ggx_d(nh, M.x.w) / (4.0f * nv) + (1.0f - ps) * ggx_g1(nv, M.alpha) * ggx_d(nh, M.alpha) / (4.0f * nv);
  }
  const float pdf_spec = vh > 0.0f ? ggx_g1(nv, M.alpha) * ggx_d(nh, M.alpha) / (4.0f * nv) : 0.0f;
  return ps * pdf_spec + (1.0f - ps) * nl * INV_PI_F;
}
// returns the pdf (0: invalid sample) and the direction in l
__device__ __forceinline__ float sample_bsdf(const Mat& M, float3 n, float3 v, float3 u, float3& l) {
  const float nv = dot(n, v);
  if (nv <= 0.0f) return 0.0f;
  const float3 t = basis_t(n), b = basis_b(n);
  const float ps = spec_prob(M, nv);
  if (M.metal > 1.5f || u.x < ps) {
    const float a = (M.metal > 1.5f && u.x < ps) ? M.x.w : M.alpha;
    const float3 hl = sample_vndf(f3(dot(t, v), dot(b, v), nv), a, u.y, u.z);
    const float3 h = t * hl.x + b * hl.y + n * hl.z;
    l = h * (2.0f * dot(v, h)) - v;
  } else {
    const float r = sqrtf(u.y);
    float sp, cp;
    sincosf(2.0f * PI_F * u.z, &sp, &cp);
    l = t * (r * cp) + b * (r * sp) + n * sqrtf(fmaxf(0.0f, 1.0f - u.y));
  }
  if (dot(n, l) <= 0.0f) return 0.0f;
  return pdf_bsdf(M, n, v, l);
}
// directional albedo tables at cosine mu (gpu/wgsl/bsdf.wgsl.js:158-173): part 0 the specular lobe (albedoSpec),
// part 1 the diffuse one (albedoDiff)
__device__ __forceinline__ float3 albedo_part(const Scene& S, uint32_t m, float mu, uint32_t part) {
  const float x = clampf(mu * float(VT_ALBEDO_BINS) - 0.5f, 0.0f, float(VT_ALBEDO_BINS - 1));
  const uint32_t i = uint32_t(floorf(x));
  const uint32_t j = min(uint32_t(VT_ALBEDO_BINS - 1), i + 1u);
  const float f = x - float(i);
  const float4* base = S.params + S.alb_off + m * VT_ALBEDO_BINS * 2u;
  return mix3(xyz(__ldg(base + 2 * i + part)), xyz(__ldg(base + 2 * j + part)), f);
}
// specular + diffuse parts
__device__ __forceinline__ float3 albedo(const Scene& S, uint32_t m, float mu) {
  return albedo_part(S, m, mu, 0u) + albedo_part(S, m, mu, 1u);
}

// ------------------------------------------------------------------------------------------------ instances
__device__ __forceinline__ const float* inst_rec(const Scene& S, uint32_t i) { return S.su + 24 + 48 * i; }
__device__ __forceinline__ float3 ld3(const float* p) { return f3(__ldg(p), __ldg(p + 1), __ldg(p + 2)); }
__device__ __forceinline__ uint32_t ldu(const float* p) { return __float_as_uint(__ldg(p)); }

struct Rot { float3 c0, c1, c2; };  // columns
__device__ __forceinline__ float3 rmul(const Rot& R, float3 v) { return R.c0 * v.x + R.c1 * v.y + R.c2 * v.z; }
__device__ __forceinline__ float3 rtmul(const Rot& R, float3 v) { return f3(dot(v, R.c0), dot(v, R.c1), dot(v, R.c2)); }
__device__ __forceinline__ Rot quat_rot(float4 q) {
  const float x = q.x, y = q.y, z = q.z, w = q.w;
  Rot R;
  R.c0 = f3(1.0f - 2.0f * (y * y + z * z), 2.0f * (x * y + z * w), 2.0f * (x * z - y * w));
  R.c1 = f3(2.0f * (x * y - z * w), 1.0f - 2.0f * (x * x + z * z), 2.0f * (y * z + x * w));
  R.c2 = f3(2.0f * (x * z + y * w), 2.0f * (y * z - x * w), 1.0f - 2.0f * (x * x + y * y));
  return R;
}
// instance pose at ray time (gpu/wgsl/common.wgsl.js:125-143: slerp + lerp when moving)
__device__ __forceinline__ void inst_pose(const Scene& S, uint32_t i, float time, Rot& R, float3& p) {
  const float* I = inst_rec(S, i);
  float4 q0 = make_float4(__ldg(I), __ldg(I + 1), __ldg(I + 2), __ldg(I + 3));
  if (ldu(I + 15) & 1u) {
    float4 b = make_float4(__ldg(I + 4), __ldg(I + 5), __ldg(I + 6), __ldg(I + 7));
    float c = q0.x * b.x + q0.y * b.y + q0.z * b.z + q0.w * b.w;
    if (c < 0.0f) { b = make_float4(-b.x, -b.y, -b.z, -b.w); c = -c; }
    float4 q;
    if (c > 0.9995f) {
      q = make_float4(q0.x * (1.0f - time) + b.x * time, q0.y * (1.0f - time) + b.y * time, q0.z * (1.0f - time) + b.z * time,
                      q0.w * (1.0f - time) + b.w * time);
      const float l = sqrtf(q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w);
      q = make_float4(q.x / l, q.y / l, q.z / l, q.w / l);
    } else {
      const float th = acosf(c), s = sinf(th);
      const float wa = sinf((1.0f - time) * th), wb = sinf(time * th);
      q = make_float4((q0.x * wa + b.x * wb) / s, (q0.y * wa + b.y * wb) / s, (q0.z * wa + b.z * wb) / s, (q0.w * wa + b.w * wb) / s);
    }
    R = quat_rot(q);
    p = mix3(ld3(I + 8), ld3(I + 12), time);
    return;
  }
  R = quat_rot(q0);
  p = ld3(I + 8);
}

// ------------------------------------------------------------------------------------------------ traversal
struct Hit { float t, u, v; uint32_t tri, inst; };

// sign(d) / max(|d|, 1e-20) per component: the correctly rounded reciprocal of the positive denominator with d's sign,
// the same value as the IEEE quotient and fewer instructions
__device__ __forceinline__ float3 safe_inv(float3 d) {
  return f3(copysignf(__frcp_rn(fmaxf(fabsf(d.x), 1e-20f)), d.x), copysignf(__frcp_rn(fmaxf(fabsf(d.y), 1e-20f)), d.y),
            copysignf(__frcp_rn(fmaxf(fabsf(d.z), 1e-20f)), d.z));
}
// entry distance of the ray into [lo, hi] within [tmin, tmax], BIG when missed (gpu/wgsl/trace.wgsl.js:178)
__device__ __forceinline__ float slab(float3 lo, float3 hi, float3 o, float3 inv, float tmin, float tmax) {
  const float3 t0 = (lo - o) * inv, t1 = (hi - o) * inv;
  const float a = fmaxf(fmaxf(fminf(t0.x, t1.x), fminf(t0.y, t1.y)), fmaxf(fminf(t0.z, t1.z), tmin));
  const float b = fminf(fminf(fmaxf(t0.x, t1.x), fmaxf(t0.y, t1.y)), fminf(fmaxf(t0.z, t1.z), tmax));
  return a <= b ? a : BIG;
}
// slab() of a node's two children at once (boxes [a0, a1] and [a2, a3]): each axis's plane distances of both boxes as
// a pair of float32 lanes, every element rounded as slab()'s own subtraction and product (x - y is x + (-y) exactly)
__device__ __forceinline__ void slab_pair(float4 a0, float4 a1, float4 a2, float4 a3, float3 o, float3 inv, float tmin, float tmax,
                                          float& t0, float& t1) {
  const float2 ox = make_float2(-o.x, -o.x), oy = make_float2(-o.y, -o.y), oz = make_float2(-o.z, -o.z);
  const float2 ix = make_float2(inv.x, inv.x), iy = make_float2(inv.y, inv.y), iz = make_float2(inv.z, inv.z);
  const float2 lx = __fmul2_rn(__fadd2_rn(make_float2(a0.x, a2.x), ox), ix), hx = __fmul2_rn(__fadd2_rn(make_float2(a1.x, a3.x), ox), ix);
  const float2 ly = __fmul2_rn(__fadd2_rn(make_float2(a0.y, a2.y), oy), iy), hy = __fmul2_rn(__fadd2_rn(make_float2(a1.y, a3.y), oy), iy);
  const float2 lz = __fmul2_rn(__fadd2_rn(make_float2(a0.z, a2.z), oz), iz), hz = __fmul2_rn(__fadd2_rn(make_float2(a1.z, a3.z), oz), iz);
  const float e0 = fmaxf(fmaxf(fminf(lx.x, hx.x), fminf(ly.x, hy.x)), fmaxf(fminf(lz.x, hz.x), tmin));
  const float f0 = fminf(fminf(fmaxf(lx.x, hx.x), fmaxf(ly.x, hy.x)), fminf(fmaxf(lz.x, hz.x), tmax));
  const float e1 = fmaxf(fmaxf(fminf(lx.y, hx.y), fminf(ly.y, hy.y)), fmaxf(fminf(lz.y, hz.y), tmin));
  const float f1 = fminf(fminf(fmaxf(lx.y, hx.y), fmaxf(ly.y, hy.y)), fminf(fmaxf(lz.y, hz.y), tmax));
  t0 = e0 <= f0 ? e0 : BIG;
  t1 = e1 <= f1 ? e1 : BIG;
}
// Moller-Trumbore on the packed record (gpu/wgsl/trace.wgsl.js:195)
__device__ __forceinline__ bool tri_hit(const Scene& S, uint32_t k, float3 o, float3 d, float tmin, float tmax, float& t, float& u, float& v) {
  const float4* r = S.tris + 4u * k;
  const float3 v0 = xyz(__ldg(r)), e1 = xyz(__ldg(r + 1)), e2 = xyz(__ldg(r + 2));
  const float3 p = cross(d, e2);
  const float det = dot(e1, p);
  if (fabsf(det) < 1e-30f) return false;
  const float inv = 1.0f / det;
  const float3 s = o - v0;
  u = dot(s, p) * inv;
  if (u < 0.0f || u > 1.0f) return false;
  const float3 q = cross(s, e1);
  v = dot(d, q) * inv;
  if (v < 0.0f || u + v > 1.0f) return false;
  t = dot(e2, q) * inv;
  return t > tmin && t < tmax;
}
// Ordered BVH2 descent from `root` with a 32-entry stack of (node, entry t); near child first; leaves tested as
// soon as their box is entered; 2048-visit and 64-triangle caps and the parent-before-child check count into dbg
// (gpu/wgsl/trace.wgsl.js:215-277). Node fetches are four 128-bit read-only loads.
template <bool ANY>
__device__ __forceinline__ bool traverse(const Scene& S, uint32_t root, float3 o, float3 d, float tmin, Hit& best, uint32_t inst) {
  const float3 inv = safe_inv(d);
  uint32_t stN[STACK];
  float stT[STACK];
  uint32_t sp = 0, node = root;
  for (uint32_t visits = 1;; visits++) {
    if (visits > MAX_VISITS) { atomicAdd(S.dbg + DBG_VISITS, 1u); break; }
    const float4* nb = S.nodes + 4u * node;
    const float4 a0 = __ldg(nb), a1 = __ldg(nb + 1), a2 = __ldg(nb + 2), a3 = __ldg(nb + 3);
    float t0 = slab(xyz(a0), xyz(a1), o, inv, tmin, best.t);
    float t1 = slab(xyz(a2), xyz(a3), o, inv, tmin, best.t);
    const uint32_t c0 = fu(a1.w), c1 = fu(a3.w), r0 = fu(a0.w), r1 = fu(a2.w);
#pragma unroll
    for (int c = 0; c < 2; c++) {
      const float tc = c == 0 ? t0 : t1;
      const uint32_t cnt = c == 0 ? c0 : c1, ref = c == 0 ? r0 : r1;
      if (tc < best.t && cnt > 0u) {
        if (cnt > MAX_LEAF) atomicAdd(S.dbg + DBG_LEAF, 1u);
        const uint32_t end = ref + min(cnt, MAX_LEAF);
        for (uint32_t k = ref; k < end; k++) {
          float t, u, v;
          if (tri_hit(S, k, o, d, tmin, best.t, t, u, v)) {
            best.t = t; best.u = u; best.v = v; best.tri = k; best.inst = inst;
            if (ANY) return true;
          }
        }
        if (c == 0) t0 = BIG; else t1 = BIG;
      }
    }
    t0 = t0 < best.t ? t0 : BIG;
    t1 = t1 < best.t ? t1 : BIG;
    if ((t0 < BIG && c0 == 0u && r0 <= node) || (t1 < BIG && c1 == 0u && r1 <= node)) { atomicAdd(S.dbg + DBG_CORRUPT, 1u); break; }
    const bool go0 = t0 < BIG, go1 = t1 < BIG;
    if (go0 && go1) {
      if (t1 < t0) { stN[sp] = r0; stT[sp] = t0; node = r1; }
      else { stN[sp] = r1; stT[sp] = t1; node = r0; }
      sp = min(sp + 1u, STACK - 1u);
    } else if (go0) {
      node = r0;
    } else if (go1) {
      node = r1;
    } else {
      bool found = false;
      while (sp > 0u) {
        sp--;
        if (stT[sp] < best.t) { node = stN[sp]; found = true; break; }
      }
      if (!found) break;
    }
  }
  return false;
}
// does the segment o + t d, t in [t0, t1], pass within r of segment a-b (gpu/wgsl/trace.wgsl.js:280)
__device__ __forceinline__ bool seg_near_capsule(float3 o, float3 d, float t0, float t1, float3 a, float3 b, float r) {
  const float3 p0 = o + d * t0, u = d * (t1 - t0), v = b - a, w = p0 - a;
  const float A = dot(u, u), B = dot(u, v), C = dot(v, v), D = dot(u, w), E = dot(v, w);
  const float den = A * C - B * B;
  float s = 0.0f;
  if (den > 1e-20f * A * C) s = clampf((B * E - C * D) / den, 0.0f, 1.0f);
  float t = C > 1e-30f ? (B * s + E) / C : 0.0f;
  if (t < 0.0f) { t = 0.0f; s = clampf(-D / fmaxf(A, 1e-30f), 0.0f, 1.0f); }
  else if (t > 1.0f) { t = 1.0f; s = clampf((B - D) / fmaxf(A, 1e-30f), 0.0f, 1.0f); }
  const float3 q = (p0 + u * s) - (a + v * t);
  return dot(q, q) <= r * r;
}
// the static BVH (mask 1) and every posed body's BLAS in its own frame at the ray's time (mask 2); skip: bodies
// this ray ignores (gpu/wgsl/trace.wgsl.js:302 traceSceneSkip). The static BVH is visited first, then the
// instances in order, through a single traversal call site (k = -1 is the static BVH).
template <bool ANY>
__device__ __forceinline__ Hit trace_scene(const Scene& S, uint32_t root, float3 o, float3 d, float tmin, float tmax, float time,
                                           uint32_t mask, uint32_t skip) {
  Hit best{tmax, 0.0f, 0.0f, MISS, MISS};
  const int n_inst = (mask & 2u) ? int(min(ldu(S.su + 16), uint32_t(VT_MAX_INST))) : 0;
  const float3 inv = safe_inv(d);
  for (int k = (mask & 1u) ? -1 : 0; k < n_inst; k++) {
    uint32_t r = root, id = MISS;
    float3 ol = o, dl = d;
    if (k >= 0) {
      const float* I = inst_rec(S, uint32_t(k));
      if ((ldu(I + 15) & 2u) || ((skip >> k) & 1u)) continue;
      if (slab(ld3(I + 16), ld3(I + 20), o, inv, tmin, best.t) >= best.t) continue;
      if (!seg_near_capsule(o, d, tmin, fminf(best.t, 1e3f), ld3(I + 32), ld3(I + 36), __ldg(I + 35))) continue;
      Rot R;
      float3 p;
      inst_pose(S, uint32_t(k), time, R, p);
      ol = rtmul(R, o - p);
      dl = rtmul(R, d);
      r = ldu(I + 11);
      id = uint32_t(k);
    }
    if (traverse<ANY>(S, r, ol, dl, tmin, best, id)) return best;
  }
  return best;
}

// ------------------------------------------------------------------------------------------------ resumable trace
// trace_scene split into single node visits, so that a warp of persistent lanes can take a new ray on any lane that
// finishes while the others keep traversing. Per ray the sequence of operations is trace_scene's: the static BVH,
// then each posed body that passes the same culls, each traversed by the same ordered descent; so are the hits.
struct TraceState {
  float3 ol, dl, inv;   // the ray in the current BVH's frame and its inverse direction
  Hit best;
  uint32_t node, sp, visits;
  int k;                // current phase: -1 the static BVH, k >= 0 posed body k
  // trace_step's node in progress: its children's entry distances (BIG once a leaf child is taken) and records (the
  // triangle counts clamped to 16 bits: child 0's low, child 1's high), and the leaf being tested
  float t0, t1;
  uint32_t r0, r1, c01;
  uint32_t lk, lend;    // triangles lk .. lend - 1 of the leaf are left (lk == lend: the next step visits st.node)
};

// set up the first phase at or after `from` that has something to traverse; false when none is left
__device__ __forceinline__ bool trace_phase(const Scene& S, uint32_t root, float3 o, float3 d, float tmin, float time, uint32_t mask,
                                            uint32_t skip, TraceState& st, int from) {
  int k = from;
  if (k < 0) {
    if (mask & 1u) {
      st.k = -1; st.ol = o; st.dl = d; st.inv = safe_inv(d); st.node = root; st.sp = 0; st.visits = 0;
      st.lk = st.lend = 0;
      return true;
    }
    k = 0;
  }
  const int n_inst = (mask & 2u) ? int(min(ldu(S.su + 16), uint32_t(VT_MAX_INST))) : 0;
  // the world-frame inverse direction, once a body gets past its flags (a ray's last phase usually meets none)
  float3 winv;
  bool have_inv = false;
  for (; k < n_inst; k++) {
    const float* I = inst_rec(S, uint32_t(k));
    if ((ldu(I + 15) & 2u) || ((skip >> k) & 1u)) continue;
    if (!have_inv) { winv = safe_inv(d); have_inv = true; }
    if (slab(ld3(I + 16), ld3(I + 20), o, winv, tmin, st.best.t) >= st.best.t) continue;
    if (!seg_near_capsule(o, d, tmin, fminf(st.best.t, 1e3f), ld3(I + 32), ld3(I + 36), __ldg(I + 35))) continue;
    Rot R;
    float3 p;
    inst_pose(S, uint32_t(k), time, R, p);
    st.ol = rtmul(R, o - p);
    st.dl = rtmul(R, d);
    st.inv = safe_inv(st.dl);
    st.node = ldu(I + 11);
    st.sp = 0;
    st.visits = 0;
    st.lk = st.lend = 0;
    st.k = k;
    return true;
  }
  st.k = n_inst;
  return false;
}

// the traversal stack of a lane: its first SH_DEPTH entries in shared memory (entry-major, so a warp's accesses are
// consecutive words), the rest of the 32 in local memory
#ifndef VT_SH_DEPTH
#define VT_SH_DEPTH 16
#endif
constexpr uint32_t SH_DEPTH = VT_SH_DEPTH;
struct LaneStack {
  uint2* sh;           // shared: SH_DEPTH x stride entries of (node, t bits)
  const float4* top = nullptr;   // shared: the staged top levels (4 float4 per slot), when the kernel stages them
  uint32_t lane, stride;
  uint2 deep[STACK - SH_DEPTH];
  __device__ __forceinline__ void set(uint32_t i, uint32_t node, float t) {
    const uint2 v = make_uint2(node, __float_as_uint(t));
    if (i < SH_DEPTH) sh[i * stride + lane] = v; else deep[i - SH_DEPTH] = v;
  }
  __device__ __forceinline__ uint2 get(uint32_t i) const { return i < SH_DEPTH ? sh[i * stride + lane] : deep[i - SH_DEPTH]; }
};

// The current phase's traversal, one unit of traverse's loop per step: a step either visits a node (the child boxes,
// and the first leaf child to test) or tests one triangle of that leaf. The node's children stay in the state until
// its leaves are done; then the same step takes the next node from its interior children or the stack. Per ray the
// sequence of operations is traverse's (child 0's leaf in triangle order, child 1's leaf only if its box is still
// nearer than the best hit, then the push / pop with the updated best), so are the hits; a warp's lanes do not wait
// for the longest leaf loop among them. The 2048-visit and 64-triangle caps and the parent-before-child check count
// into dbg as in traverse. 0 continue, 1 the phase is finished, 2 an any-hit query found its hit.
// the leaf of child c, when its box is nearer than the best hit: its triangles become the ones left, and the child's
// distance BIG (traverse drops a tested leaf child from the push / pop the same way, after its loop)
__device__ __forceinline__ bool leaf_enter(const Scene& S, TraceState& st, uint32_t c) {
  const float tc = c == 0u ? st.t0 : st.t1;
  const uint32_t cnt = (st.c01 >> (16u * c)) & 0xffffu, ref = c == 0u ? st.r0 : st.r1;
  if (!(tc < st.best.t && cnt > 0u)) return false;
  if (cnt > MAX_LEAF) atomicAdd(S.dbg + DBG_LEAF, 1u);
  st.lk = ref;
  st.lend = ref + min(cnt, MAX_LEAF);
  if (c == 0u) st.t0 = BIG; else st.t1 = BIG;
  return true;
}

template <bool ANY>
__device__ __forceinline__ int trace_step(const Scene& S, float tmin, TraceState& st, LaneStack& stk) {
  bool more;
  if (st.lk == st.lend) {
    if (++st.visits > MAX_VISITS) { atomicAdd(S.dbg + DBG_VISITS, 1u); return 1; }
    const uint32_t node = st.node;
#if VT_TOP_NODES
    float4 a0, a1, a2, a3;
    if ((node & TOP_BIT) != 0u) {
      const float4* nb = stk.top + 4u * (node & 0xffffu);
      a0 = nb[0]; a1 = nb[1]; a2 = nb[2]; a3 = nb[3];
    } else {
      const float4* nb = S.nodes + 4u * node;
      a0 = __ldg(nb); a1 = __ldg(nb + 1); a2 = __ldg(nb + 2); a3 = __ldg(nb + 3);
    }
#else
    const float4* nb = S.nodes + 4u * node;
    const float4 a0 = __ldg(nb), a1 = __ldg(nb + 1), a2 = __ldg(nb + 2), a3 = __ldg(nb + 3);
#endif
    slab_pair(a0, a1, a2, a3, st.ol, st.inv, tmin, st.best.t, st.t0, st.t1);
    st.c01 = min(fu(a1.w), 0xffffu) | (min(fu(a3.w), 0xffffu) << 16);
    st.r0 = fu(a0.w); st.r1 = fu(a2.w);
    more = leaf_enter(S, st, 0u) || leaf_enter(S, st, 1u);
  } else {
    const uint32_t k = st.lk++;
    float t, u, v;
    if (tri_hit(S, k, st.ol, st.dl, tmin, st.best.t, t, u, v)) {
      st.best.t = t; st.best.u = u; st.best.v = v; st.best.tri = k; st.best.inst = st.k < 0 ? MISS : uint32_t(st.k);
      if (ANY) return 2;
    }
    // the leaf done: child 1's leaf next (when that was child 0's and child 1's box is still nearer)
    more = st.lk != st.lend || leaf_enter(S, st, 1u);
  }
  if (more) return 0;
  const uint32_t node = st.node;
#if VT_TOP_NODES
  const bool staged = (node & TOP_BIT) != 0u;
#else
  constexpr bool staged = false;
#endif
  const float t0 = st.t0 < st.best.t ? st.t0 : BIG;
  const float t1 = st.t1 < st.best.t ? st.t1 : BIG;
  const uint32_t r0 = st.r0, r1 = st.r1;
  if (!staged && ((t0 < BIG && (st.c01 & 0xffffu) == 0u && r0 <= node) || (t1 < BIG && (st.c01 >> 16) == 0u && r1 <= node))) {
    atomicAdd(S.dbg + DBG_CORRUPT, 1u);
    return 1;
  }
  const bool go0 = t0 < BIG, go1 = t1 < BIG;
  if (go0 && go1) {
    if (t1 < t0) { stk.set(st.sp, r0, t0); st.node = r1; }
    else { stk.set(st.sp, r1, t1); st.node = r0; }
    st.sp = min(st.sp + 1u, STACK - 1u);
  } else if (go0) {
    st.node = r0;
  } else if (go1) {
    st.node = r1;
  } else {
    while (st.sp > 0u) {
      st.sp--;
      const uint2 e = stk.get(st.sp);
      if (__uint_as_float(e.y) < st.best.t) { st.node = e.x; return 0; }
    }
    return 1;
  }
  return 0;
}

// Persistent traversal lanes: every lane keeps one ray in flight, one node visit per loop iteration; once `refill`
// lanes of the warp are idle they take the next queue entries with one atomic. Lanes stay busy until the queue
// drains instead of waiting for the warp's slowest ray (warp-level ray compaction).
template <typename F>
__device__ __forceinline__ bool take_rays(bool& active, bool& exhausted, uint32_t* head, uint32_t n, uint32_t refill, F&& start) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t idle = __ballot_sync(0xffffffffu, !active);
  if (!exhausted && idle && (__popc(idle) >= int(refill) || idle == 0xffffffffu)) {
    const uint32_t leader = __ffs(idle) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(head, uint32_t(__popc(idle)));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (base + uint32_t(__popc(idle)) >= n) exhausted = true;
    if (!active) {
      const uint32_t idx = base + __popc(idle & ((1u << lane) - 1u));
      if (idx < n) start(idx);
    }
  }
  return __any_sync(0xffffffffu, active) || !exhausted;
}

// copy the staged top levels into the block's shared array; returns the root to start static traversals at
__device__ __forceinline__ uint32_t stage_top(const Scene& S, float4* top_sh, uint32_t root) {
#if VT_TOP_NODES
  const uint32_t n = min(S.n_top, TOP_NODES) * 4u;
  for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) top_sh[i] = __ldg(S.top + i);
  __syncthreads();
  return n && root == S.top_root ? TOP_BIT : root;
#else
  (void)S; (void)top_sh;
  return root;
#endif
}

// ------------------------------------------------------------------------------------------------ surfaces
struct Surf { float3 p, ng, ns, b; uint32_t vi0, vi1, vi2, mesh, flags, mat, inst; };

__device__ __forceinline__ float3 vnormal(const Scene& S, uint32_t v) { return xyz(__ldg(S.verts + 2u * v + 1u)); }

// gpu/wgsl/trace.wgsl.js:330 surface: hit point, two-sided geometric and shading normals, mesh, material
__device__ __forceinline__ Surf surface(const Scene& S, const Hit& h, float3 o, float3 d, float time) {
  Surf s;
  const float4* r = S.tris + 4u * h.tri;
  const float4 r0 = __ldg(r), r1 = __ldg(r + 1), r2 = __ldg(r + 2), at = __ldg(r + 3);
  s.vi0 = fu(r0.w); s.vi1 = fu(r1.w); s.vi2 = fu(r2.w);
  s.mesh = fu(at.x); s.flags = fu(at.y);
  s.b = f3(1.0f - h.u - h.v, h.u, h.v);
  float3 ng = normalize(cross(xyz(r1), xyz(r2)));
  float3 ns = normalize(vnormal(S, s.vi0) * s.b.x + vnormal(S, s.vi1) * s.b.y + vnormal(S, s.vi2) * s.b.z);
  if (h.inst != MISS) {
    Rot R;
    float3 p;
    inst_pose(S, h.inst, time, R, p);
    ng = rmul(R, ng);
    ns = rmul(R, ns);
  }
  if (dot(ng, d) > 0.0f) ng = -ng;
  if (dot(ns, ng) < 0.0f) ns = -ns;
  if (dot(ns, -d) < 1e-4f) ns = ng;
  s.ng = ng; s.ns = ns;
  s.mat = fu(__ldg(S.params + S.mesh_off + 2u * s.mesh).w);
  s.inst = h.inst;
  s.p = o + d * h.t;
  return s;
}
__device__ __forceinline__ float3 offset_ray(float3 p, float3 ng, float3 dir) {
  return p + ng * (dot(ng, dir) > 0.0f ? EPS_OFF : -EPS_OFF);
}
// FDM layer lines, h(s) = depth/2 cos(2 pi s / period) with s = p . bd: the tilted normal (gpu/wgsl/bsdf.wgsl.js:176
// layerNormal); the phase is taken first so that the sine's argument stays small in float32
__device__ __forceinline__ float3 layer_normal(float3 n, float3 p, float3 bd, float period, float depth) {
  const float x = dot(p, bd) / period;
  const float ph = x - floorf(x);
  const float dh = -(depth * 0.5f) * (2.0f * PI_F / period) * sinf(2.0f * PI_F * ph);
  const float3 bt = bd - n * dot(bd, n);
  return normalize(n - bt * dh);
}
// gpu/wgsl/shade.wgsl.js:100 shadingNormal
__device__ __forceinline__ float3 shading_normal(const Scene& S, const Surf& s, uint32_t opts) {
  if (!(opts & VT_O_LAYER) || !(s.flags & VT_F_LAYER)) return s.ns;
  const float4 r0 = __ldg(S.params + S.mesh_off + 2u * s.mesh), r1 = __ldg(S.params + S.mesh_off + 2u * s.mesh + 1u);
  float3 n = layer_normal(s.ns, s.p, xyz(r0), r1.y, r1.z);
  if (dot(n, s.ng) <= 0.0f) n = s.ns;
  return n;
}

// ------------------------------------------------------------------------------------------------ emitter
// piecewise-linear p(theta), 0 past the last knot (gpu/wgsl/shade.wgsl.js:12)
__device__ __forceinline__ float profile(const Scene& S, float th) {
  const float4 last = __ldg(S.params + S.prof_off + S.prof_n - 1u);
  if (th >= last.x) return th == last.x ? last.y : 0.0f;
  uint32_t lo = 0, hi = S.prof_n - 1u;
  for (uint32_t it = 0; it < 40u && hi - lo > 1u; it++) {
    const uint32_t m = (lo + hi) >> 1;
    if (__ldg(S.params + S.prof_off + m).x <= th) lo = m; else hi = m;
  }
  const float4 a = __ldg(S.params + S.prof_off + lo), b = __ldg(S.params + S.prof_off + hi);
  const float f = clampf((th - a.x) / fmaxf(b.x - a.x, 1e-12f), 0.0f, 1.0f);
  return a.y * (1.0f - f) + b.y * f;
}
// radiance leaving the emitter (normal n, axis) toward w (gpu/wgsl/shade.wgsl.js:50)
__device__ __forceinline__ float3 emitted(const Scene& S, float3 n, float3 axis, float3 w) {
  if (dot(w, n) <= 0.0f) return f3(0, 0, 0);
  return ld3(S.su) * profile(S, acosf(clampf(dot(w, axis), -1.0f, 1.0f)));
}
// area sample of the emitter by its triangle CDF, posed with the emitter body (gpu/wgsl/shade.wgsl.js:31)
__device__ __forceinline__ void sample_emitter(const Scene& S, float3 u, float time, float3& p, float3& n, float3& axis) {
  uint32_t lo = 0, hi = S.emit_n - 1u;
  for (uint32_t it = 0; it < 40u && lo < hi; it++) {
    const uint32_t m = (lo + hi) >> 1;
    if (__ldg(S.params + S.emit_off + 4u * m).w < u.x) lo = m + 1u; else hi = m;
  }
  const float4* e = S.params + S.emit_off + 4u * lo;
  const float3 v0 = xyz(__ldg(e)), e1 = xyz(__ldg(e + 1)), e2 = xyz(__ldg(e + 2)), nl = xyz(__ldg(e + 3));
  const float su = sqrtf(u.y);
  const float3 pl = v0 + e1 * (su * (1.0f - u.z)) + e2 * (su * u.z);
  Rot R;
  float3 pp;
  inst_pose(S, ldu(S.su + 17), time, R, pp);
  p = rmul(R, pl) + pp;
  n = rmul(R, nl);
  axis = rmul(R, ld3(S.su + 4));
}
__device__ __forceinline__ float3 emitter_axis_at(const Scene& S, float time) {
  Rot R;
  float3 p;
  inst_pose(S, ldu(S.su + 17), time, R, p);
  return rmul(R, ld3(S.su + 4));
}
__device__ __forceinline__ float3 emitter_normal(const Scene& S, const Hit& h, const Surf& s, float time) {
  const float3 n = normalize(vnormal(S, s.vi0) * s.b.x + vnormal(S, s.vi1) * s.b.y + vnormal(S, s.vi2) * s.b.z);
  Rot R;
  float3 p;
  inst_pose(S, h.inst, time, R, p);
  return rmul(R, n);
}

// ------------------------------------------------------------------------------------------------ indirect
// cosine-weighted hemisphere fraction hidden by a thin cylinder (gpu/wgsl/shade.wgsl.js:59). The integral's sines
// come from the angles' tangents instead of sin(): with f = atan(t), sin 2f = 2t / (1 + t^2) and sin^2 f = t^2 /
// (1 + t^2); an end clamped to f0 -+ pi/2 (f0 = atan2(na, np)) has sin 2f = -sin 2f0 = -2 na np / rho^2 and sin^2 f =
// cos^2 f0 = np^2 / rho^2, rho^2 = na^2 + np^2. The same integral to float rounding, four sines fewer per capsule.
__device__ __forceinline__ float capsule_occ(float3 p, float3 n, float3 a, float3 bb, float r) {
  const float3 ab = bb - a;
  const float L = length(ab);
  if (L < 1e-9f || r <= 0.0f) return 0.0f;
  const float3 e = ab / L;
  const float3 ap = p - a;
  const float s0 = dot(ap, e);
  const float3 perp = ap - e * s0;
  const float h = sqrtf(dot(perp, perp) + r * r);
  const float pl = length(perp);
  float3 ep = -perp / fmaxf(pl, 1e-12f);
  if (pl < 1e-12f) ep = normalize(cross(e, basis_t(e)));
  const float np = dot(n, ep), na = dot(n, e);
  const float t1 = (0.0f - s0) / h, t2 = (L - s0) / h;
  float f1 = atanf(t1), f2 = atanf(t2);
  const float f0 = atan2f(na, np);
  const float rho2 = na * na + np * np;
  // sin 2f and sin^2 f of each end, clamped or not
  float s2a = 2.0f * t1 / (1.0f + t1 * t1), sqa = t1 * t1 / (1.0f + t1 * t1);
  float s2b = 2.0f * t2 / (1.0f + t2 * t2), sqb = t2 * t2 / (1.0f + t2 * t2);
  if (f0 - 0.5f * PI_F > f1) {
    f1 = f0 - 0.5f * PI_F;
    s2a = rho2 > 0.0f ? -2.0f * na * np / rho2 : 0.0f;
    sqa = rho2 > 0.0f ? np * np / rho2 : 1.0f;
  }
  if (f0 + 0.5f * PI_F < f2) {
    f2 = f0 + 0.5f * PI_F;
    s2b = rho2 > 0.0f ? -2.0f * na * np / rho2 : 0.0f;
    sqb = rho2 > 0.0f ? np * np / rho2 : 1.0f;
  }
  if (f2 <= f1) return 0.0f;
  const float I = np * (0.5f * (f2 - f1) + 0.25f * (s2b - s2a)) + na * 0.5f * (sqb - sqa);
  return clampf(INV_PI_F * (2.0f * r / h) * I, 0.0f, 1.0f);
}
__device__ __forceinline__ float capsule_vis(const Scene& S, float3 p, float3 n) {
  float v = 1.0f;
  const uint32_t cnt = min(ldu(S.su + 16), uint32_t(VT_MAX_INST));
  for (uint32_t i = 0; i < cnt; i++) {
    const float* I = inst_rec(S, i);
    if (ldu(I + 15) & 2u) continue;
    v = v - capsule_occ(p, n, ld3(I + 24), ld3(I + 28), __ldg(I + 27)) * (1.0f - __ldg(I + 31));
  }
  return clampf(v, 0.0f, 1.0f);
}
// barycentrics renormalised over the triangle's active nodes (gpu/wgsl/shade.wgsl.js:194-209)
__device__ __forceinline__ float3 node_weights(const Scene& S, const Surf& s, uint32_t slot) {
  const float3 w = s.b * f3(__ldg(S.nstate + 4u * s.vi0 + slot).w, __ldg(S.nstate + 4u * s.vi1 + slot).w, __ldg(S.nstate + 4u * s.vi2 + slot).w);
  const float sw = w.x + w.y + w.z;
  return sw <= 1e-6f ? s.b : w / sw;
}
__device__ __forceinline__ float3 node_slot(const Scene& S, const Surf& s, uint32_t slot, uint32_t wslot) {
  const float3 b = node_weights(S, s, wslot);
  return xyz(__ldg(S.nstate + 4u * s.vi0 + slot)) * b.x + xyz(__ldg(S.nstate + 4u * s.vi1 + slot)) * b.y + xyz(__ldg(S.nstate + 4u * s.vi2 + slot)) * b.z;
}

// ------------------------------------------------------------------------------------------------ estimators
// One emitter sample: its contribution before the shadow test, MIS-weighted (power heuristic, nL light samples : 1
// BSDF sample) against BSDF sampling when `mis`, and the shadow segment to test (gpu/wgsl/shade.wgsl.js:135
// lightEval / :160 directLight). Returns false when the sample contributes nothing whatever the visibility.
__device__ __forceinline__ bool light_sample(const Scene& S, const Surf& s, float3 n, const Mat& M, float3 wo, float time, float3 u, bool mis,
                                             float nL, float3& c, float3& so, float3& wi, float& tmax) {
  float3 lp, ln, la;
  sample_emitter(S, u, time, lp, ln, la);
  wi = lp - s.p;
  const float d2 = dot(wi, wi), dist = sqrtf(d2);
  wi = wi / dist;
  c = f3(0, 0, 0);
  so = s.p;
  tmax = 0.0f;
  const float cosE = dot(-wi, ln);
  if (cosE <= 0.0f) return false;
  const float cosS = dot(n, wi);
  if (cosS <= 0.0f || dot(s.ng, wi) <= 0.0f) return false;
  const float3 Le = emitted(S, ln, la, -wi);
  if (maxc(Le) <= 0.0f) return false;
  const float3 f = eval_bsdf(M, n, wi, wo);
  if (maxc(f) <= 0.0f) return false;
  const float pdfW = d2 / (cosE * __ldg(S.su + 3));
  float w = 1.0f;
  if (mis) {
    const float pb = pdf_bsdf(M, n, wo, wi);
    w = nL * nL * pdfW * pdfW / (nL * nL * pdfW * pdfW + pb * pb);
  }
  c = f * Le * (cosS * w / pdfW);
  so = offset_ray(s.p, s.ng, wi);
  tmax = dist - 2e-5f;
  return true;
}

}  // namespace vtd
