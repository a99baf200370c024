// The raster camera pass of lite_nodes on sm_103a: vertex stage, a software rasteriser with exact integer edge
// functions and 64-bit depth|triangle keys, and the fragment stage fused with the MSAA resolve (lite_nodes/
// renderer.js:92-374: vsCam, vsShadow, fsCam, FINISH).
//
// Rasterisation (this library's own rules, the ones a 4x MSAA raster pipeline with 'less' depth and no culling
// follows): clip against 0 <= z <= w (the near and far planes) and a guard band |x|, |y| <= 8 w; snap x/w, y/w in
// pixels to 1/256; a sample is covered when all three int64 edge functions are positive, or zero on an edge that
// owns its ties (edge direction dy < 0, or dy = 0 and dx > 0: of two triangles that share an edge exactly one owns
// it); its depth is z/w interpolated linearly in the screen with the covered sample's edge weights, clamped to
// [0, 1], and it is kept when below 1 and below what the sample holds. atomicMin on (depth bits << 32 | triangle)
// keeps the nearest fragment and, on equal depth, the one drawn first, which is what the ordered 'less' test keeps.
// The fragment stage runs once per (pixel, triangle) among the pixel's surviving samples at the pixel centre,
// with perspective-correct attributes of the unclipped triangle (2D-homogeneous barycentrics, Olano and Greer
// 1997), as a raster pipeline's centre interpolation does.
//
// The translation unit is compiled without multiply-add contraction (--fmad=false), so the clip, snap, coverage and
// depth arithmetic is the sequence of IEEE operations that the CPU restatement performs on the same clip
// coordinates: sample keys and shadow maps are bit-identical to it.
#include <cuda_fp16.h>

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

// ---------------------------------------------------------------------------------------------- rasteriser
__device__ __forceinline__ float plane_dist(const float4& v, int p) {
  switch (p) {
    case 0: return v.z;
    case 1: return v.w - v.z;
    case 2: return GUARD * v.w - v.x;
    case 3: return GUARD * v.w + v.x;
    case 4: return GUARD * v.w - v.y;
    default: return GUARD * v.w + v.y;
  }
}
__device__ __forceinline__ bool inside_all(const float4& v) {
  bool in = true;
#pragma unroll
  for (int p = 0; p < 6; p++) in &= plane_dist(v, p) >= 0.0f;
  return in;
}

// Sutherland-Hodgman against the six planes; a crossing point is interpolated from the inside endpoint, so a shared
// edge gives its two triangles the same point. Returns the vertex count (0: nothing left), at most 9.
__device__ int clip_poly(const float4 in[3], float4 out[9]) {
  float4 a[9], b[9];
  a[0] = in[0]; a[1] = in[1]; a[2] = in[2];
  int n = 3;
  for (int p = 0; p < 6; p++) {
    int m = 0;
    for (int i = 0; i < n; i++) {
      const float4 A = a[i], B = a[i + 1 < n ? i + 1 : 0];
      const float da = plane_dist(A, p), db = plane_dist(B, p);
      if (da >= 0.0f && m < 9) b[m++] = A;
      if ((da >= 0.0f) != (db >= 0.0f) && m < 9) {
        const float4 I = da >= 0.0f ? A : B, O = da >= 0.0f ? B : A;
        const float di = da >= 0.0f ? da : db, dq = da >= 0.0f ? db : da;
        const float t = di / (di - dq);
        b[m++] = make_float4(I.x + t * (O.x - I.x), I.y + t * (O.y - I.y), I.z + t * (O.z - I.z), I.w + t * (O.w - I.w));
      }
    }
    n = m;
    if (n < 3) return 0;
    for (int i = 0; i < n; i++) a[i] = b[i];
  }
  for (int i = 0; i < n; i++) out[i] = a[i];
  return n;
}

struct Snap { int x, y; float z; };
// viewport transform and the 1/256-pixel snap; false for a vertex that cannot be projected (w <= 0 or not finite)
__device__ __forceinline__ bool snap(const float4& c, float W2, float H2, Snap& s) {
  if (!(c.w > 0.0f)) return false;
  const float nx = c.x / c.w, ny = c.y / c.w;
  const float X = (nx + 1.0f) * W2, Y = (1.0f - ny) * H2;
  if (!(fabsf(X) < 1e6f) || !(fabsf(Y) < 1e6f)) return false;
  s.x = __float2int_rn(X * 256.0f);
  s.y = __float2int_rn(Y * 256.0f);
  s.z = c.z / c.w;
  return true;
}

__device__ __forceinline__ int floor_div256(int v) { return v >= 0 ? v >> 8 : -((255 - v) >> 8); }

// sample offsets in 1/256 pixel: the 4x MSAA pattern, or the centre
__device__ __forceinline__ void sample_pos(uint32_t samples, uint32_t s, int& ox, int& oy) {
  if (samples == 1u) { ox = 128; oy = 128; return; }
  const int sx[4] = {96, 224, 32, 160}, sy[4] = {32, 96, 160, 224};
  ox = sx[s]; oy = sy[s];
}

struct Edge { long long dx, dy, x0, y0; int bias; };
__device__ __forceinline__ Edge make_edge(const Snap& j, const Snap& k) {
  Edge e;
  e.dx = (long long)k.x - j.x;
  e.dy = (long long)k.y - j.y;
  e.x0 = j.x;
  e.y0 = j.y;
  e.bias = (e.dy < 0 || (e.dy == 0 && e.dx > 0)) ? 0 : -1;
  return e;
}
__device__ __forceinline__ long long edge_at(const Edge& e, long long sx, long long sy) { return e.dx * (sy - e.y0) - e.dy * (sx - e.x0); }

// the samples of pixel rows [py0, py1] x columns [px0, px1] that sub-triangle (a, b, c) covers, thread `lane` of
// `lanes` taking every lanes-th pixel
__device__ void raster_sub(Snap a, Snap b, Snap c, uint32_t id, uint32_t layer, const Target& T, int lane, int lanes) {
  long long A = ((long long)b.x - a.x) * ((long long)c.y - a.y) - ((long long)b.y - a.y) * ((long long)c.x - a.x);
  if (A == 0) return;
  if (A < 0) { const Snap t = b; b = c; c = t; A = -A; }
  const Edge e0 = make_edge(b, c), e1 = make_edge(c, a), e2 = make_edge(a, b);
  const int xmin = min(a.x, min(b.x, c.x)), xmax = max(a.x, max(b.x, c.x));
  const int ymin = min(a.y, min(b.y, c.y)), ymax = max(a.y, max(b.y, c.y));
  const int px0 = max(0, floor_div256(xmin)), px1 = min(int(T.W) - 1, floor_div256(xmax));
  const int py0 = max(0, floor_div256(ymin)), py1 = min(int(T.H) - 1, floor_div256(ymax));
  if (px0 > px1 || py0 > py1) return;
  const int nx = px1 - px0 + 1;
  const int npx = nx * (py1 - py0 + 1);
  const float fA = float(A);
  for (int q = lane; q < npx; q += lanes) {
    const int px = px0 + q % nx, py = py0 + q / nx;
    for (uint32_t s = 0; s < T.samples; s++) {
      int ox, oy;
      sample_pos(T.samples, s, ox, oy);
      const long long sx = (long long)px * 256 + ox, sy = (long long)py * 256 + oy;
      const long long w0 = edge_at(e0, sx, sy), w1 = edge_at(e1, sx, sy), w2 = edge_at(e2, sx, sy);
      if (w0 + e0.bias < 0 || w1 + e1.bias < 0 || w2 + e2.bias < 0) continue;
      const float l1 = float(w1) / fA, l2 = float(w2) / fA;
      float z = a.z + l1 * (b.z - a.z) + l2 * (c.z - a.z);
      z = fminf(z, 1.0f);
      if (!(z > 0.0f)) z = 0.0f;
      if (!(z < 1.0f)) continue;
      if (T.samples == 4u) {
        const unsigned long long key = ((unsigned long long)__float_as_uint(z) << 32) | id;
        unsigned long long* p = T.key + (size_t(py) * T.W + px) * 4u + s;
        if (*p > key) atomicMin(p, key);
      } else {
        uint32_t* p = T.depth + size_t(layer) * T.W * T.H + size_t(py) * T.W + px;
        const uint32_t d = __float_as_uint(z);
        if (*p > d) atomicMin(p, d);
      }
    }
  }
}

// one triangle: clip, snap, then either raster here or (box larger than BIG_PIXELS) leave it to the block path
__device__ __forceinline__ int setup_tri(const float4* clip, const uint32_t* idx, uint32_t n_verts, uint32_t tri, uint32_t layer,
                                         const Target& T, Snap* P) {
  const float4* C = clip + size_t(layer) * n_verts;
  float4 in[3];
  for (int j = 0; j < 3; j++) in[j] = __ldg(C + __ldg(idx + 3u * tri + j));
  float4 poly[9];
  int n;
  if (inside_all(in[0]) && inside_all(in[1]) && inside_all(in[2])) {
    poly[0] = in[0]; poly[1] = in[1]; poly[2] = in[2];
    n = 3;
  } else {
    n = clip_poly(in, poly);
  }
  const float W2 = float(T.W) * 0.5f, H2 = float(T.H) * 0.5f;
  for (int i = 0; i < n; i++)
    if (!snap(poly[i], W2, H2, P[i])) return 0;
  return n;
}

__global__ void raster_kernel(const float4* __restrict__ clip, const uint32_t* __restrict__ idx, uint32_t n_verts, uint32_t t0, uint32_t nt,
                              uint32_t layers, const Target T) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nt * layers) return;
  const uint32_t layer = i / nt, tri = t0 + i % nt;
  Snap P[9];
  const int n = setup_tri(clip, idx, n_verts, tri, layer, T, P);
  if (n < 3) return;
  int xmin = P[0].x, xmax = P[0].x, ymin = P[0].y, ymax = P[0].y;
  for (int k = 1; k < n; k++) { xmin = min(xmin, P[k].x); xmax = max(xmax, P[k].x); ymin = min(ymin, P[k].y); ymax = max(ymax, P[k].y); }
  const long long bw = (long long)min(int(T.W) - 1, floor_div256(xmax)) - max(0, floor_div256(xmin)) + 1;
  const long long bh = (long long)min(int(T.H) - 1, floor_div256(ymax)) - max(0, floor_div256(ymin)) + 1;
  if (bw <= 0 || bh <= 0) return;
  if (bw * bh > (long long)BIG_PIXELS) {
    const uint32_t slot = atomicAdd(T.big, 1u);
    if (slot < T.big_cap) T.big[1 + slot] = tri | (layer << 28);
    return;
  }
  for (int k = 1; k + 1 < n; k++) raster_sub(P[0], P[k], P[k + 1], tri, layer, T, 0, 1);
}

// the queued many-pixel triangles: one block per triangle, the block's threads over its pixels
__global__ void raster_big_kernel(const float4* __restrict__ clip, const uint32_t* __restrict__ idx, uint32_t n_verts, const Target T) {
  const uint32_t count = min(T.big[0], T.big_cap);
  for (uint32_t q = blockIdx.x; q < count; q += gridDim.x) {
    const uint32_t e = T.big[1 + q];
    const uint32_t tri = e & 0x0fffffffu, layer = e >> 28;
    Snap P[9];
    const int n = setup_tri(clip, idx, n_verts, tri, layer, T, P);
    for (int k = 1; k + 1 < n; k++) raster_sub(P[0], P[k], P[k + 1], tri, layer, T, threadIdx.x, blockDim.x);
  }
}

__global__ void fill_kernel(uint32_t* p, size_t n, uint32_t value) {
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) p[i] = value;
}

// ---------------------------------------------------------------------------------------------- fragment stage
__device__ __forceinline__ float sm_texel(const uint32_t* m, uint32_t res, uint32_t k, int x, int y) {
  x = min(max(x, 0), int(res) - 1);
  y = min(max(y, 0), int(res) - 1);
  const uint32_t b = __ldg(m + (size_t(k) * res + y) * res + x);
  return b == 0xffffffffu ? 1.0f : __uint_as_float(b);
}
// textureSampleCompareLevel with a 'less' comparison sampler, linear filtering, clamp to edge: the 2x2 texels
// around the point each compare dref < depth, blended bilinearly
__device__ __forceinline__ float sm_cmp(const uint32_t* m, uint32_t res, uint32_t k, float u, float v, float dref) {
  const float tx = u * float(res) - 0.5f, ty = v * float(res) - 0.5f;
  const float fx0 = floorf(tx), fy0 = floorf(ty);
  const float fx = tx - fx0, fy = ty - fy0;
  const int x0 = int(fx0), y0 = int(fy0);
  const float c00 = dref < sm_texel(m, res, k, x0, y0) ? 1.0f : 0.0f;
  const float c10 = dref < sm_texel(m, res, k, x0 + 1, y0) ? 1.0f : 0.0f;
  const float c01 = dref < sm_texel(m, res, k, x0, y0 + 1) ? 1.0f : 0.0f;
  const float c11 = dref < sm_texel(m, res, k, x0 + 1, y0 + 1) ? 1.0f : 0.0f;
  return (1.0f - fx) * (1.0f - fy) * c00 + fx * (1.0f - fy) * c10 + (1.0f - fx) * fy * c01 + fx * fy * c11;
}
// smVis (lite_nodes/renderer.js:267): 3x3 taps one texel apart, min of the static and dynamic maps per tap
__device__ float sm_vis(const View& V, const ShadeArgs& a, float3 pw, uint32_t k, float bias) {
  const float3 q = sm_project(V, pw, k);
  if (fabsf(q.x) >= 1.0f || fabsf(q.y) >= 1.0f) return 1.0f;
  const float u = 0.5f + 0.5f * q.x, v = 0.5f - 0.5f * q.y;
  const float dref = (q.z - bias) / V.lb[3];
  const float t = 1.0f / float(a.sm_res);
  float s = 0.0f;
  for (int j = -1; j <= 1; j++)
    for (int i = -1; i <= 1; i++) {
      const float ou = u + float(i) * t, ov = v + float(j) * t;
      const float cs = sm_cmp(a.sm_static, a.sm_res, k, ou, ov, dref);
      const float cd = sm_cmp(a.sm_dyn, a.sm_res, k, ou, ov, dref);
      s = s + fminf(cs, cd);
    }
  return s / 9.0f;
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
  float3 acc[K_SECT];
  for (uint32_t k = 0; k < K_SECT; k++) acc[k] = f3(0.0f, 0.0f, 0.0f);
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
    const float3 f = eval_bsdf(M, ns, wi, wo);
    const uint32_t k = min(uint32_t(ea.w), K_SECT - 1u);
    acc[k] = acc[k] + f * (pr * cosS * cosE * eb.w / d2);
  }
  float3 L = f3(0.0f, 0.0f, 0.0f);
  const float3 off = p + ng * (is_static ? 1.5e-4f : 6e-4f);
  const uint32_t dbg = __float_as_uint(V.axisW[3]);
  float vsum = 0.0f;
  for (uint32_t k = 0; k < K_SECT; k++) {
    float vk = 1.0f;
    if (dbg != 1u) vk = sm_vis(V, a, off, k, is_static ? V.lo[k][3] : 6e-4f);
    vsum = vsum + vk;
    if (maxc(acc[k]) <= 0.0f) continue;
    L = L + acc[k] * vk;
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

__global__ void __launch_bounds__(128) shade_kernel(const Scene S, const Geo g, const View V, const ShadeArgs a) {
  const uint32_t W = uint32_t(V.size[0]), H = uint32_t(V.size[1]);
  const uint32_t px = blockIdx.x * 16 + (threadIdx.x & 15), py = blockIdx.y * 8 + (threadIdx.x >> 4);
  if (px >= W || py >= H) return;
  const size_t pix = size_t(py) * W + px;
  unsigned long long k[4];
  for (int s = 0; s < 4; s++) k[s] = a.key[pix * 4 + s];
  float3 col[4];
  uint32_t done = 0;
  for (int s = 0; s < 4; s++) {
    if (done & (1u << s)) continue;
    float3 c = f3(0.0f, 0.0f, 0.0f);
    if (k[s] != EMPTY_KEY) {
      c = fragment(S, g, V, a, uint32_t(k[s] & 0xffffffffu), px, py);
      c = f3(h16(c.x), h16(c.y), h16(c.z));
    }
    for (int t = s; t < 4; t++)
      if (!(done & (1u << t)) && (uint32_t(k[t] & 0xffffffffu) == uint32_t(k[s] & 0xffffffffu)) && ((k[t] == EMPTY_KEY) == (k[s] == EMPTY_KEY))) {
        col[t] = c;
        done |= 1u << t;
      }
  }
  // resolve (average of the samples into rgba16float), then FINISH: x 1 / outScale, the SCOPE circle mask
  float3 r = f3(h16((((col[0].x + col[1].x) + col[2].x) + col[3].x) * 0.25f), h16((((col[0].y + col[1].y) + col[2].y) + col[3].y) * 0.25f),
                h16((((col[0].z + col[1].z) + col[2].z) + col[3].z) * 0.25f));
  r = r * a.inv_scale;
  if (a.circle > 0.0f) {
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
void launch_raster(const float4* clip, const uint32_t* idx, uint32_t n_verts, uint32_t t0, uint32_t nt, uint32_t layers, const Target& T,
                   int blocks_big, cudaStream_t st) {
  cudaMemsetAsync(T.big, 0, 4, st);
  const size_t n = size_t(nt) * layers;
  if (n) raster_kernel<<<uint32_t((n + 127) / 128), 128, 0, st>>>(clip, idx, n_verts, t0, nt, layers, T);
  raster_big_kernel<<<blocks_big, 256, 0, st>>>(clip, idx, n_verts, T);
}
void launch_shade(const Scene& S, const Geo& g, const View& v, const ShadeArgs& a, cudaStream_t st) {
  const uint32_t W = uint32_t(v.size[0]), H = uint32_t(v.size[1]);
  dim3 grid((W + 15) / 16, (H + 7) / 8);
  shade_kernel<<<grid, 128, 0, st>>>(S, g, v, a);
}
void launch_fill(uint32_t* p, size_t n, uint32_t value, cudaStream_t st) {
  fill_kernel<<<1024, 256, 0, st>>>(p, n, value);
}

}  // namespace vtl
