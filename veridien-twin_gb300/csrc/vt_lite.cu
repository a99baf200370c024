// The raster camera pass of lite_nodes on sm_103a, around the rasteriser of vt_lite_raster.cu: the vertex stage
// (vsCam / vsShadow) and the fragment stage fused with the MSAA resolve and FINISH (lite_nodes/renderer.js:92-374).
//
// The fragment stage runs once per (pixel, triangle) among the pixel's surviving samples at the pixel centre (a list
// of such fragments is built first, static-surface and posed-body fragments apart, so the shading threads of a warp
// do the same work), with
// perspective-correct attributes of the unclipped triangle (2D-homogeneous barycentrics, Olano and Greer 1997), as
// a raster pipeline's centre interpolation does. The 3x3 shadow-map taps one texel apart share one bilinear
// fraction, so the 16 texels under them are compared once per map.
#include <cuda_fp16.h>

#include "vt_kernels.cuh"
#include "vt_lite.cuh"

using namespace vtd;

namespace vtl {
namespace {

__device__ __forceinline__ float3 v3(const float a[4]) { return f3(a[0], a[1], a[2]); }
__device__ __forceinline__ float len2(float x, float y) { return sqrtf(x * x + y * y); }

struct WorldV { float3 p, n; bool ok; };

// toWorld (lite_nodes/renderer.js:193): static vertices as stored; posed bodies at the view's time, hidden bodies
// and the camera's own skipped bodies dropped
__device__ __forceinline__ WorldV to_world(const Scene& S, const View& V, uint4 a, uint4 b) {
  WorldV w;
  w.p = f3(__uint_as_float(a.x), __uint_as_float(a.y), __uint_as_float(a.z));
  w.n = f3(__uint_as_float(b.x), __uint_as_float(b.y), __uint_as_float(b.z));
  w.ok = true;
  const uint32_t inst = a.w >> 16;
  if (inst == STATIC_INST) return w;
  if (inst >= uint32_t(VT_MAX_INST) || (ldu(inst_rec(S, inst) + 15) & 2u) || ((V.misc[0] >> inst) & 1u)) { w.ok = false; return w; }
  Rot R;
  float3 t;
  inst_pose(S, inst, V.env[3], R, t);
  w.p = rmul(R, w.p) + t;
  w.n = rmul(R, w.n);
  return w;
}

// projectCam (lite_nodes/renderer.js:203): pinhole (mode 1) or KB4 with the cut at thetaCut; a point past the cut
// becomes a point at infinity along its azimuth (w < 0), so clipping at z = 0 extends a crossing triangle outward
__device__ __forceinline__ float4 project_cam(const View& V, float3 p) {
  const float3 d = p - v3(V.pos);
  const float x = dot(d, v3(V.rx)), y = dot(d, v3(V.ry)), z = dot(d, v3(V.rz));
  const float W = V.size[0], H = V.size[1], FAR = V.lb[3];
  if (V.pos[3] > 0.5f) {
    const float nearZ = 1e-3f;
    return make_float4((2.0f * V.lensA[0] * x + (2.0f * (V.lensA[2] + 0.5f) - W) * z) / W,
                       ((H - 2.0f * (V.lensA[3] + 0.5f)) * z - 2.0f * V.lensA[1] * y) / H, (z - nearZ) * FAR / (FAR - nearZ), z);
  }
  const float r = len2(x, y);
  const float th = atan2f(r, z);
  if (th > V.size[2]) {
    const float ex = V.lensA[0] * x / W + 1e-12f, ey = -V.lensA[1] * y / H;
    const float l = len2(ex, ey);
    return make_float4(ex / l, ey / l, -1e-3f, -1e-3f);
  }
  const float t2 = th * th;
  const float thd = th * (1.0f + t2 * (V.lensB[0] + t2 * (V.lensB[1] + t2 * (V.lensB[2] + t2 * V.lensB[3]))));
  const float s = thd / fmaxf(r, 1e-12f);
  const float u = V.lensA[0] * x * s + V.lensA[2] + 0.5f;
  const float vv = V.lensA[1] * y * s + V.lensA[3] + 0.5f;
  return make_float4(2.0f * u / W - 1.0f, 1.0f - 2.0f * vv / H, length(d) / FAR, 1.0f);
}

// smProject (lite_nodes/renderer.js:180): equidistant projection about the emission axis from sector origin k
__device__ __forceinline__ float3 sm_project(const View& V, float3 pw, uint32_t k) {
  const float3 d = pw - v3(V.lo[k]);
  const float x = dot(d, v3(V.lt)), y = dot(d, v3(V.lb)), z = dot(d, v3(V.axisW));
  const float rho = len2(x, y);
  const float th = atan2f(rho, z);
  const float s = th / (V.lt[3] * fmaxf(rho, 1e-12f));
  return f3(x * s, y * s, length(d));
}

__global__ void vertex_cam_kernel(const Scene S, const Geo g, const View V, uint32_t first, uint32_t count, float4* __restrict__ clip) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const uint32_t v = first + i;
  const WorldV w = to_world(S, V, __ldg(g.v + 2 * v), __ldg(g.v + 2 * v + 1));
  clip[v] = w.ok ? project_cam(V, w.p) : make_float4(0.0f, 0.0f, -2.0f, 1.0f);
}

// vsShadow (lite_nodes/renderer.js:241): casters only (no emitter or scope mesh; static or dynamic per the view)
__global__ void vertex_shadow_kernel(const Scene S, const Geo g, const View V, uint32_t first, uint32_t count, float4* __restrict__ clip) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const uint32_t v = first + i;
  const uint4 a = __ldg(g.v + 2 * v);
  const WorldV w = to_world(S, V, a, __ldg(g.v + 2 * v + 1));
  const bool is_static = (a.w >> 16) == STATIC_INST;
  const uint32_t mesh = a.w & 0xffffu;
  const uint32_t flags = fu(__ldg(S.params + S.mesh_off + 2u * mesh + 1u).x);
  bool keep = w.ok && (flags & (VT_F_EMITTER | VT_F_SCOPE)) == 0u;
  if (V.misc[3] == 1u && !is_static) keep = false;
  if (V.misc[3] == 2u && is_static) keep = false;
  for (uint32_t k = 0; k < K_SECT; k++) {
    float4 o = make_float4(0.0f, 0.0f, -2.0f, 1.0f);
    if (keep) {
      const float3 q = sm_project(V, w.p, k);
      if (len2(q.x, q.y) > 1.0f) {
        const float ex = q.x + 1e-12f, ey = q.y;
        const float l = len2(ex, ey);
        o = make_float4(ex / l, ey / l, -1e-3f, -1e-3f);
      } else {
        o = make_float4(q.x, q.y, q.z / V.lb[3], 1.0f);
      }
    }
    clip[size_t(k) * g.n_verts + v] = o;
  }
}

// ---------------------------------------------------------------------------------------------- fragment stage
__device__ __forceinline__ uint32_t sm_less(const uint32_t* m, uint32_t res, uint32_t k, int x, int y, float dref) {
  x = min(max(x, 0), int(res) - 1);
  y = min(max(y, 0), int(res) - 1);
  const uint32_t b = __ldg(m + (size_t(k) * res + y) * res + x);
  return dref < (b == 0xffffffffu ? 1.0f : __uint_as_float(b)) ? 1u : 0u;
}
// smVis (lite_nodes/renderer.js:267): 3x3 taps one texel apart of textureSampleCompareLevel ('less' comparison,
// linear filtering, clamp to edge: the 2x2 texels around a tap compare dref < depth and blend bilinearly), min of
// the static and dynamic maps per tap. The taps share the bilinear fraction of the centre tap (they sit exactly one
// texel apart), so the 4x4 texels under them are compared once per map.
__device__ float sm_vis(const View& V, const ShadeArgs& a, float3 pw, uint32_t k, float bias) {
  const float3 q = sm_project(V, pw, k);
  if (fabsf(q.x) >= 1.0f || fabsf(q.y) >= 1.0f) return 1.0f;
  const float u = 0.5f + 0.5f * q.x, v = 0.5f - 0.5f * q.y;
  const float dref = (q.z - bias) / V.lb[3];
  const float res = float(a.sm_res);
  const float tx = u * res - 0.5f, ty = v * res - 0.5f;
  const float fx0 = floorf(tx), fy0 = floorf(ty);
  const float fx = tx - fx0, fy = ty - fy0;
  const int x0 = int(fx0) - 1, y0 = int(fy0) - 1;
  uint32_t ms = 0, md = 0;
#pragma unroll
  for (int j = 0; j < 4; j++)
#pragma unroll
    for (int i = 0; i < 4; i++) {
      ms |= sm_less(a.sm_static, a.sm_res, k, x0 + i, y0 + j, dref) << (4 * j + i);
      md |= sm_less(a.sm_dyn, a.sm_res, k, x0 + i, y0 + j, dref) << (4 * j + i);
    }
  const float w00 = (1.0f - fx) * (1.0f - fy), w10 = fx * (1.0f - fy), w01 = (1.0f - fx) * fy, w11 = fx * fy;
  float s = 0.0f;
#pragma unroll
  for (int j = 0; j < 3; j++)
#pragma unroll
    for (int i = 0; i < 3; i++) {
      const int b = 4 * j + i;
      const float cs = w00 * float((ms >> b) & 1u) + w10 * float((ms >> (b + 1)) & 1u) + w01 * float((ms >> (b + 4)) & 1u) +
                       w11 * float((ms >> (b + 5)) & 1u);
      const float cd = w00 * float((md >> b) & 1u) + w10 * float((md >> (b + 1)) & 1u) + w01 * float((md >> (b + 4)) & 1u) +
                       w11 * float((md >> (b + 5)) & 1u);
      s = s + fminf(cs, cd);
    }
  return s / 9.0f;
}

// evalBSDF (gpu/bsdf.js:98) for a fixed shading normal and view: the factors that depend only on n . v (the view's
// Fresnel terms and GGX Smith lambdas) are computed once per fragment; each light direction then costs the rest.
// The operations and their order are those of eval_bsdf, so the values are the same.
struct BsdfView {
  float nv, lam_v, lam_v_coat, F_v, Fv_coat_t;
};
__device__ __forceinline__ BsdfView bsdf_view(const Mat& M, float3 n, float3 v) {
  BsdfView b;
  b.nv = dot(n, v);
  b.lam_v = ggx_lambda(b.nv, M.alpha);
  b.lam_v_coat = M.metal > 1.5f ? ggx_lambda(b.nv, M.x.w) : 0.0f;
  b.F_v = fresnel(b.nv, M.ior);
  b.Fv_coat_t = 1.0f - b.F_v;
  return b;
}
__device__ __forceinline__ float3 eval_bsdf_v(const Mat& M, const BsdfView& B, float3 n, float3 l, float3 v) {
  const float nl = dot(n, l), nv = B.nv;
  if (nl <= 0.0f || nv <= 0.0f) return f3(0, 0, 0);
  const float3 h = normalize(l + v);
  const float nh = dot(n, h), vh = fmaxf(0.0f, dot(v, h));
  if (M.metal > 1.5f) {
    const float ac = M.x.w;
    const float coat = ggx_d(nh, ac) * (1.0f / (1.0f + ggx_lambda(nl, ac) + B.lam_v_coat)) * fresnel(vh, M.ior) / (4.0f * nl * nv);
    const float t = (1.0f - fresnel(nl, M.ior)) * B.Fv_coat_t;
    const float metal = ggx_d(nh, M.alpha) * (1.0f / (1.0f + ggx_lambda(nl, M.alpha) + B.lam_v)) / (4.0f * nl * nv);
    const float ex = 1.0f / nl + 1.0f / nv;
    const float3 tp = f3(powf(M.x.x, ex), powf(M.x.y, ex), powf(M.x.z, ex));
    return f3(coat, coat, coat) + tp * schlick3(M.c, vh) * (t * metal);
  }
  const float spec = ggx_d(nh, M.alpha) * (1.0f / (1.0f + ggx_lambda(nl, M.alpha) + B.lam_v)) / (4.0f * nl * nv);
  float3 out = fresnel_rgb(M, vh) * spec;
  if (M.metal < 0.5f) {
    const float kd = INV_PI_F * (1.0f - fresnel(nl, M.ior)) * (1.0f - B.F_v) / (1.0f - M.fbar);
    out = out + M.c * kd;
  }
  return out;
}

// fsCam (lite_nodes/renderer.js:284) for triangle `tri` at the centre of pixel (px, py); radiance x outScale
__device__ float3 fragment(const Scene& S, const Geo& g, const View& V, const ShadeArgs& a, uint32_t tri, uint32_t px, uint32_t py) {
  uint4 va[3], vb[3];
  float4 c[3];
  for (int j = 0; j < 3; j++) {
    const uint32_t vi = __ldg(g.idx + 3u * tri + j);
    va[j] = __ldg(g.v + 2 * vi);
    vb[j] = __ldg(g.v + 2 * vi + 1);
    c[j] = __ldg(a.clip + vi);
  }
  WorldV w[3];
  for (int j = 0; j < 3; j++) w[j] = to_world(S, V, va[j], vb[j]);
  // perspective-correct barycentrics at the pixel centre from the homogeneous pixel coordinates, relative to it
  const float W2 = V.size[0] * 0.5f, H2 = V.size[1] * 0.5f;
  const float sx = float(px) + 0.5f, sy = float(py) + 0.5f;
  float X[3], Y[3];
  for (int j = 0; j < 3; j++) {
    X[j] = (c[j].x + c[j].w) * W2 - sx * c[j].w;
    Y[j] = (c[j].w - c[j].y) * H2 - sy * c[j].w;
  }
  float u0 = X[1] * Y[2] - X[2] * Y[1], u1 = X[2] * Y[0] - X[0] * Y[2], u2 = X[0] * Y[1] - X[1] * Y[0];
  const float su = u0 + u1 + u2;
  if (su != 0.0f) { u0 = u0 / su; u1 = u1 / su; u2 = u2 / su; } else { u0 = u1 = u2 = 1.0f / 3.0f; }
  const float3 p = w[0].p * u0 + w[1].p * u1 + w[2].p * u2;
  const float3 nin = w[0].n * u0 + w[1].n * u1 + w[2].n * u2;
  // node irradiance per vertex (vsCam :226): E x active weight, weight
  const uint32_t slot = ldu(S.su + 18);
  float4 ew = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  const float bw[3] = {u0, u1, u2};
  for (int j = 0; j < 3; j++) {
    const uint32_t ni = vb[j].w;
    if (ni == MISS) continue;
    const float wa = __ldg(S.nstate + 4u * ni + slot).w;
    const float3 e = xyz(__ldg(S.nstate + 4u * ni)) * wa;
    ew.x = ew.x + e.x * bw[j]; ew.y = ew.y + e.y * bw[j]; ew.z = ew.z + e.z * bw[j]; ew.w = ew.w + wa * bw[j];
  }
  const uint32_t bits = va[0].w;
  const uint32_t mesh = bits & 0xffffu, inst = bits >> 16;
  const float4 row0 = __ldg(S.params + S.mesh_off + 2u * mesh);
  const uint32_t flags = fu(__ldg(S.params + S.mesh_off + 2u * mesh + 1u).x);
  const uint32_t mat = fu(row0.w);
  const float3 wo = normalize(v3(V.pos) - p);
  // the derivative of the interpolated position over a planar triangle spans its plane: the face normal
  float3 ng = cross(w[1].p - w[0].p, w[2].p - w[0].p);
  if (dot(ng, ng) < 1e-30f) ng = nin;
  ng = normalize(ng);
  if (dot(ng, wo) < 0.0f) ng = -ng;
  float3 ns = normalize(nin);
  const float3 axis = v3(V.axisW);
  if (flags & VT_F_EMITTER) {
    if (dot(wo, ns) <= 0.0f) return f3(0.0f, 0.0f, 0.0f);
    const float3 Le = ld3(S.su) * profile(S, acosf(clampf(dot(wo, axis), -1.0f, 1.0f)));
    const float sc = V.size[3];
    return f3(fminf(Le.x * sc, 60000.0f), fminf(Le.y * sc, 60000.0f), fminf(Le.z * sc, 60000.0f));
  }
  if (dot(ns, ng) < 0.0f) ns = -ns;
  if (dot(ns, wo) < 1e-4f) ns = ng;
  const Mat M = load_mat(S, mat);   // a textured board's print mask is a 1x1 white texture: the material as loaded
  const bool is_static = inst == STATIC_INST;
  const uint32_t nS = is_static ? V.misc[1] : V.misc[2];
  const BsdfView BV = bsdf_view(M, ns, wo);
  // per-sector sums in registers (the sample's sector is the same for every thread of a warp)
  float3 acc0 = f3(0.0f, 0.0f, 0.0f), acc1 = acc0, acc2 = acc0, acc3 = acc0;
  for (uint32_t j = 0; j < nS; j++) {
    const float4 ea = __ldg(g.es + 2 * j), eb = __ldg(g.es + 2 * j + 1);
    float3 wi = xyz(ea) - p;
    const float d2 = dot(wi, wi);
    wi = wi * (1.0f / sqrtf(d2));
    const float cosE = dot(-wi, xyz(eb));
    if (cosE <= 0.0f) continue;
    const float cosS = dot(ns, wi);
    if (cosS <= 0.0f || dot(ng, wi) <= 0.0f) continue;
    const float pr = profile(S, acosf(clampf(dot(-wi, axis), -1.0f, 1.0f)));
    if (pr <= 0.0f) continue;
    const float3 f = eval_bsdf_v(M, BV, ns, wi, wo);
    const float3 add = f * (pr * cosS * cosE * eb.w / d2);
    const uint32_t k = uint32_t(ea.w);
    if (k == 0u) acc0 = acc0 + add;
    else if (k == 1u) acc1 = acc1 + add;
    else if (k == 2u) acc2 = acc2 + add;
    else acc3 = acc3 + add;
  }
  float3 L = f3(0.0f, 0.0f, 0.0f);
  const float3 off = p + ng * (is_static ? 1.5e-4f : 6e-4f);
  const uint32_t dbg = __float_as_uint(V.axisW[3]);
  float vsum = 0.0f;
#pragma unroll
  for (uint32_t k = 0; k < K_SECT; k++) {
    const float3 ak = k == 0 ? acc0 : k == 1 ? acc1 : k == 2 ? acc2 : acc3;
    float vk = 1.0f;
    if (dbg != 1u) vk = sm_vis(V, a, off, k, is_static ? V.lo[k][3] : 6e-4f);
    vsum = vsum + vk;
    if (maxc(ak) <= 0.0f) continue;
    L = L + ak * vk;
  }
  if (dbg == 2u) return f3(vsum / float(K_SECT), vsum / float(K_SECT), vsum / float(K_SECT));
  L = L * ld3(S.su) / float(nS);
  const float mu = fmaxf(dot(ns, wo), 0.0f);
  const float3 Al = albedo(S, mat, mu);
  if (is_static) {
    float3 E = f3(0.0f, 0.0f, 0.0f);
    if (ew.w > 1e-6f) E = f3(ew.x, ew.y, ew.z) / ew.w;
    E = E * capsule_vis(S, p, ns);
    L = L + E * INV_PI_F * Al;
  } else {
    L = L + v3(V.env) * Al;
  }
  return L * V.size[3];
}

__device__ __forceinline__ float h16(float x) { return __half2float(__float2half_rn(x)); }

// Fragment list: per pixel, each distinct triangle among its 4 samples becomes one fragment, static-surface
// fragments (24 emitter samples, capsule occlusion) appended from the front of the list and posed-body fragments (96
// emitter samples) from the back, so a warp of the shading kernel runs fragments of one kind; sidx[pixel] holds each
// sample's fragment (MISS: empty). Appends are one atomic per warp and kind.
__global__ void __launch_bounds__(256) frag_kernel(const unsigned long long* __restrict__ key, uint32_t W, uint32_t H, uint32_t n_static_tris,
                                                    uint2* __restrict__ frags, uint32_t cap, uint32_t* __restrict__ counts, uint4* __restrict__ sidx) {
  const uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
  const bool live = pix < W * H;
  uint32_t id[4], f[4], ns = 0, nd = 0;
  bool fresh[4];
  for (int s = 0; s < 4; s++) {
    const unsigned long long k = live ? key[size_t(pix) * 4 + s] : EMPTY_KEY;
    id[s] = k == EMPTY_KEY ? MISS : uint32_t(k & 0xffffffffu);
    fresh[s] = id[s] != MISS;
    for (int t = 0; t < s; t++) fresh[s] = fresh[s] && id[t] != id[s];
    if (fresh[s]) { if (id[s] < n_static_tris) ns++; else nd++; }
  }
  // warp-wide exclusive prefix sums of the new fragments of each kind
  const uint32_t lane = threadIdx.x & 31u;
  uint32_t ps = ns, pd = nd;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t a = __shfl_up_sync(0xffffffffu, ps, o), b = __shfl_up_sync(0xffffffffu, pd, o);
    if (lane >= uint32_t(o)) { ps += a; pd += b; }
  }
  const uint32_t ts = __shfl_sync(0xffffffffu, ps, 31), td = __shfl_sync(0xffffffffu, pd, 31);
  uint32_t bs = 0, bd = 0;
  if (lane == 0) { bs = ts ? atomicAdd(counts, ts) : 0; bd = td ? atomicAdd(counts + 1, td) : 0; }
  bs = __shfl_sync(0xffffffffu, bs, 0) + ps - ns;
  bd = __shfl_sync(0xffffffffu, bd, 0) + pd - nd;
  if (!live) return;
  for (int s = 0; s < 4; s++) {
    if (id[s] == MISS) { f[s] = MISS; continue; }
    if (!fresh[s]) {
      for (int t = 0; t < s; t++)
        if (id[t] == id[s]) { f[s] = f[t]; break; }
      continue;
    }
    f[s] = id[s] < n_static_tris ? bs++ : cap - 1u - bd++;
    frags[f[s]] = make_uint2(pix, id[s]);
  }
  sidx[pix] = make_uint4(f[0], f[1], f[2], f[3]);
}

// one thread per fragment: the static fragments, then the posed-body ones; colours stored as half floats (the
// multisample target is rgba16float)
// blocks of 128 an SM holds: 7 caps the registers at 72 (a few spills); measured per 1280x720 view 0.487 ms at
// 6 (80 registers), 0.475 at 7, 0.472-0.477 at 8 (64 registers, 132 B of spills)
#ifndef VT_SHADE_BLOCKS
#define VT_SHADE_BLOCKS 7
#endif
// waves of the grid: fragments cost 24 or 96 emitter samples, so more, shorter blocks balance the SMs. Per 1280x720
// view: 0.477 ms at 1 wave, 0.468 at 2, 0.436 at 4, 0.421 at 8, 0.453 at 16
#ifndef VT_SHADE_WAVES
#define VT_SHADE_WAVES 8
#endif
__global__ void __launch_bounds__(128, VT_SHADE_BLOCKS) shade_frag_kernel(const Scene S, const Geo g, const View V, const ShadeArgs a, const uint2* __restrict__ frags,
                                                         uint32_t cap, const uint32_t* __restrict__ counts, uint2* __restrict__ colors) {
  const uint32_t ns = counts[0], nd = counts[1];
  const uint32_t W = uint32_t(V.size[0]);
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < ns + nd; i += gridDim.x * blockDim.x) {
    const uint32_t fi = i < ns ? i : cap - nd + (i - ns);
    const uint2 fr = frags[fi];
    const float3 c = fragment(S, g, V, a, fr.y, fr.x % W, fr.x / W);
    const __half2 rg = __floats2half2_rn(c.x, c.y), bz = __floats2half2_rn(c.z, 0.0f);
    colors[fi] = make_uint2(*reinterpret_cast<const uint32_t*>(&rg), *reinterpret_cast<const uint32_t*>(&bz));
  }
}

// resolve (average of the 4 samples into rgba16float), then FINISH: x 1 / outScale, the SCOPE circle mask
__global__ void __launch_bounds__(256) resolve_kernel(const View V, const ShadeArgs a, const uint4* __restrict__ sidx, const uint2* __restrict__ colors) {
  const uint32_t W = uint32_t(V.size[0]), H = uint32_t(V.size[1]);
  const uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
  if (pix >= W * H) return;
  const uint4 f = sidx[pix];
  const uint32_t fs[4] = {f.x, f.y, f.z, f.w};
  float3 col[4];
  for (int s = 0; s < 4; s++) {
    col[s] = f3(0.0f, 0.0f, 0.0f);
    if (fs[s] == MISS) continue;
    const uint2 c = colors[fs[s]];
    const float2 rg = __half22float2(*reinterpret_cast<const __half2*>(&c.x));
    col[s] = f3(rg.x, rg.y, __low2float(*reinterpret_cast<const __half2*>(&c.y)));
  }
  float3 r = f3(h16((((col[0].x + col[1].x) + col[2].x) + col[3].x) * 0.25f), h16((((col[0].y + col[1].y) + col[2].y) + col[3].y) * 0.25f),
                h16((((col[0].z + col[1].z) + col[2].z) + col[3].z) * 0.25f));
  r = r * a.inv_scale;
  if (a.circle > 0.0f) {
    const uint32_t px = pix % W, py = pix / W;
    const float qx = float(px) + 0.5f - 0.5f * float(W), qy = float(py) + 0.5f - 0.5f * float(H);
    if (len2(qx, qy) > a.circle) r = f3(0.0f, 0.0f, 0.0f);
  }
  a.out[pix] = make_float4(r.x, r.y, r.z, 1.0f);
}

}  // namespace

void launch_vertex_cam(const Scene& S, const Geo& g, const View& v, uint32_t first, uint32_t count, float4* clip, cudaStream_t st) {
  if (!count) return;
  vertex_cam_kernel<<<(count + 255) / 256, 256, 0, st>>>(S, g, v, first, count, clip);
}
void launch_vertex_shadow(const Scene& S, const Geo& g, const View& v, uint32_t first, uint32_t count, float4* clip, cudaStream_t st) {
  if (!count) return;
  vertex_shadow_kernel<<<(count + 255) / 256, 256, 0, st>>>(S, g, v, first, count, clip);
}
// whole waves: the grid is VT_SHADE_WAVES x the SM count x the blocks of shade_frag_kernel an SM holds, so the last
// wave is not a partial one that leaves a tail (a 1216-block grid with 912 resident took 0.548 ms per view)
void launch_shade(const Scene& S, const Geo& g, const View& v, const ShadeArgs& a, const FragBufs& fb, int sms, cudaStream_t st) {
  static std::atomic<int> occupancy[vtk::MAX_DEVICES];
  const int per_sm = vtk::per_device_value(occupancy, [](int) {
    int per = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, shade_frag_kernel, 128, 0);
    return per;
  });
  const int blocks = sms * per_sm * VT_SHADE_WAVES;
  const uint32_t W = uint32_t(v.size[0]), H = uint32_t(v.size[1]);
  const uint32_t cap = W * H * 4u;
  cudaMemsetAsync(fb.counts, 0, 8, st);
  frag_kernel<<<(W * H + 255) / 256, 256, 0, st>>>(a.key, W, H, g.n_static_tris, fb.frags, cap, fb.counts, fb.sidx);
  shade_frag_kernel<<<blocks, 128, 0, st>>>(S, g, v, a, fb.frags, cap, fb.counts, fb.colors);
  resolve_kernel<<<(W * H + 255) / 256, 256, 0, st>>>(v, a, fb.sidx, fb.colors);
}
}  // namespace vtl
