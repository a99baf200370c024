// The rasteriser of the raster camera pass (lite_nodes/renderer.js: the camera pass of vsCam / fsCam with 4x MSAA
// and the sector shadow passes of vsShadow), on sm_103a.
//
// Rules (this library's own, the ones a raster pipeline with 'less' depth and no culling follows): clip against
// 0 <= z <= w (the near and far planes) and a guard band |x|, |y| <= 8 w; snap x/w, y/w in pixels to 1/256; a sample
// is covered when all three int64 edge functions are positive, or zero on an edge that owns its ties (edge direction
// dy < 0, or dy = 0 and dx > 0: of two triangles that share an edge exactly one owns it); its depth is z/w
// interpolated linearly in the screen with the sample's edge weights, clamped to [0, 1], and it is kept when below 1
// and below what the sample holds. atomicMin on (depth bits << 32 | triangle) keeps the nearest fragment and, on
// equal depth, the one drawn first, which is what the ordered 'less' test keeps; a shadow map keeps the depth bits.
//
// Work split: one pass snaps every vertex once (a vertex inside every clip plane, nearly all, keeps its snapped
// point); then one thread per triangle; a triangle of three such vertices needs no clipping. Its box, if at most
// BIG_SAMPLES samples, is rasterised by that thread (edge functions stepped exactly from pixel to pixel), else one
// (triangle, 32 x 32-pixel tile) item per tile of its box is queued and a warp per item rasterises that tile: the
// lanes find the tile's 4 x 4-pixel sub-blocks that the triangle may cover, then take their pixels (tiles that do
// not fit in the queue are rasterised by the triangle's own thread).
//
// The translation unit is compiled without multiply-add contraction (--fmad=false), so the clip, snap, coverage and
// depth arithmetic is the sequence of IEEE operations that the CPU restatement performs on the same clip
// coordinates: sample keys and shadow maps are bit-identical to it.
#include "vt_lite.cuh"

namespace vtl {
namespace {

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
__device__ __noinline__ int clip_poly(const float4 in[3], float4 out[9]) {
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

// pixel box of the snapped points, clamped to the target; false when empty
struct Box { int x0, x1, y0, y1; };
__device__ __forceinline__ bool box_of(const Snap* P, int n, const Target& T, Box& b) {
  int xmin = P[0].x, xmax = P[0].x, ymin = P[0].y, ymax = P[0].y;
  for (int k = 1; k < n; k++) { xmin = min(xmin, P[k].x); xmax = max(xmax, P[k].x); ymin = min(ymin, P[k].y); ymax = max(ymax, P[k].y); }
  b.x0 = max(0, floor_div256(xmin)); b.x1 = min(int(T.W) - 1, floor_div256(xmax));
  b.y0 = max(0, floor_div256(ymin)); b.y1 = min(int(T.H) - 1, floor_div256(ymax));
  return b.x0 <= b.x1 && b.y0 <= b.y1;
}

// the samples that sub-triangle (a, b, c) covers within pixel box `lim`; with lanes = 32 the warp's lanes take a
// 16 x 2 pattern of pixels (lane % 16, lane / 16) stepping by 16 columns and 2 rows, else one thread walks the box.
// Edge functions are stepped exactly in int64 from the pixel origin; sample s adds its constant offset.
template <uint32_t NS>
__device__ void raster_sub_n(Snap a, Snap b, Snap c, uint32_t id, uint32_t layer, const Target& T, const Box& lim, int lane, int lanes) {
  long long A = ((long long)b.x - a.x) * ((long long)c.y - a.y) - ((long long)b.y - a.y) * ((long long)c.x - a.x);
  if (A == 0) return;
  if (A < 0) { const Snap t = b; b = c; c = t; A = -A; }
  const Snap P[3] = {a, b, c};
  Box bx;
  if (!box_of(P, 3, T, bx)) return;
  bx.x0 = max(bx.x0, lim.x0); bx.x1 = min(bx.x1, lim.x1); bx.y0 = max(bx.y0, lim.y0); bx.y1 = min(bx.y1, lim.y1);
  if (bx.x0 > bx.x1 || bx.y0 > bx.y1) return;
  const Edge E[3] = {make_edge(b, c), make_edge(c, a), make_edge(a, b)};
  if (lanes > 1) {
    // a tile of a many-pixel triangle: skip it when one edge excludes every sample position of the box (the edge
    // function is linear, so its largest value over the box is at a corner of the samples' extent)
    const long long sx0 = (long long)bx.x0 * 256 + 32, sx1 = (long long)bx.x1 * 256 + 224;
    const long long sy0 = (long long)bx.y0 * 256 + 32, sy1 = (long long)bx.y1 * 256 + 224;
    for (int k = 0; k < 3; k++) {
      const long long m = max(max(edge_at(E[k], sx0, sy0), edge_at(E[k], sx1, sy0)), max(edge_at(E[k], sx0, sy1), edge_at(E[k], sx1, sy1)));
      if (m + E[k].bias < 0) return;
    }
  }
  const int LX = lanes > 1 ? 16 : 1, LY = lanes > 1 ? 2 : 1;
  const int px0 = bx.x0 + lane % LX, py0 = bx.y0 + lane / LX;   // lanes past the box run no iteration
  // sample offsets in 1/256 pixel: the 4x MSAA pattern (0.375, 0.125), (0.875, 0.375), (0.125, 0.625),
  // (0.625, 0.875), or the centre
  long long off[3][NS];
#pragma unroll
  for (uint32_t s = 0; s < NS; s++) {
    const long long ox = NS == 1u ? 128 : (long long)((0xa020e060u >> (8 * s)) & 0xffu);
    const long long oy = NS == 1u ? 128 : 32 + 64 * (long long)s;
#pragma unroll
    for (int k = 0; k < 3; k++) off[k][s] = E[k].dx * oy - E[k].dy * ox + E[k].bias;
  }
  long long row[3], stepx[3], stepy[3];
  for (int k = 0; k < 3; k++) {
    row[k] = edge_at(E[k], (long long)px0 * 256, (long long)py0 * 256);
    stepx[k] = -E[k].dy * 256 * LX;
    stepy[k] = E[k].dx * 256 * LY;
  }
  const float rA = 1.0f / float(A);
  const float dz1 = b.z - a.z, dz2 = c.z - a.z;
  for (int py = py0; py <= bx.y1; py += LY) {
    long long w[3] = {row[0], row[1], row[2]};
    for (int px = px0; px <= bx.x1; px += LX) {
#pragma unroll
      for (uint32_t s = 0; s < NS; s++) {
        const long long w0 = w[0] + off[0][s], w1 = w[1] + off[1][s], w2 = w[2] + off[2][s];   // edge + tie bias
        if (w0 < 0 || w1 < 0 || w2 < 0) continue;
        const float l1 = float(w1 - E[1].bias) * rA, l2 = float(w2 - E[2].bias) * rA;
        float z = a.z + l1 * dz1 + l2 * dz2;
        z = fminf(z, 1.0f);
        if (!(z > 0.0f)) z = 0.0f;
        if (!(z < 1.0f)) continue;
        if (NS == 4u)
          atomicMin(T.key + (size_t(py) * T.W + px) * 4u + s, ((unsigned long long)__float_as_uint(z) << 32) | id);   // a reduction
        else
          atomicMin(T.depth + size_t(layer) * T.W * T.H + size_t(py) * T.W + px, __float_as_uint(z));
      }
      for (int k = 0; k < 3; k++) w[k] += stepx[k];
    }
    for (int k = 0; k < 3; k++) row[k] += stepy[k];
  }
}

// one sample's test and write (edge values w already include the tie bias)
template <uint32_t NS>
__device__ __forceinline__ void shade_sample(const Snap& a, float dz1, float dz2, float rA, long long w0, long long w1, long long w2, int b1, int b2,
                                             uint32_t id, uint32_t layer, const Target& T, int px, int py, uint32_t s) {
  if (w0 < 0 || w1 < 0 || w2 < 0) return;
  const float l1 = float(w1 - b1) * rA, l2 = float(w2 - b2) * rA;
  float z = a.z + l1 * dz1 + l2 * dz2;
  z = fminf(z, 1.0f);
  if (!(z > 0.0f)) z = 0.0f;
  if (!(z < 1.0f)) return;
  if (NS == 4u)
    atomicMin(T.key + (size_t(py) * T.W + px) * 4u + s, ((unsigned long long)__float_as_uint(z) << 32) | id);   // a reduction
  else
    atomicMin(T.depth + size_t(layer) * T.W * T.H + size_t(py) * T.W + px, __float_as_uint(z));
}

// a tile (box `lim`, at most 32 x 32 pixels) of a many-pixel triangle, by a whole warp: each lane tests two of the
// tile's 4 x 4-pixel sub-blocks against the three edges (the edge functions are linear: their largest value over a
// sub-block's samples is at a corner of the samples' extent), then the warp covers the candidate sub-blocks two at a
// time, one pixel per lane
template <uint32_t NS>
__device__ void raster_tile_n(Snap a, Snap b, Snap c, uint32_t id, uint32_t layer, const Target& T, const Box& lim, int lane) {
  long long A = ((long long)b.x - a.x) * ((long long)c.y - a.y) - ((long long)b.y - a.y) * ((long long)c.x - a.x);
  if (A == 0) return;
  if (A < 0) { const Snap t = b; b = c; c = t; A = -A; }
  const Snap P[3] = {a, b, c};
  Box bx;
  if (!box_of(P, 3, T, bx)) return;
  bx.x0 = max(bx.x0, lim.x0); bx.x1 = min(bx.x1, lim.x1); bx.y0 = max(bx.y0, lim.y0); bx.y1 = min(bx.y1, lim.y1);
  if (bx.x0 > bx.x1 || bx.y0 > bx.y1) return;
  const Edge E[3] = {make_edge(b, c), make_edge(c, a), make_edge(a, b)};
  const int nbx = (bx.x1 - bx.x0) / 4 + 1, nby = (bx.y1 - bx.y0) / 4 + 1;   // at most 8 x 8
  bool cand[2];
#pragma unroll
  for (int h = 0; h < 2; h++) {
    const int q = lane + 32 * h;
    const int qx = q % 8, qy = q / 8;
    bool in = qx < nbx && qy < nby;
    if (in) {
      const int x0 = bx.x0 + 4 * qx, x1 = min(x0 + 3, bx.x1), y0 = bx.y0 + 4 * qy, y1 = min(y0 + 3, bx.y1);
      const long long sx0 = (long long)x0 * 256 + 32, sx1 = (long long)x1 * 256 + 224;
      const long long sy0 = (long long)y0 * 256 + 32, sy1 = (long long)y1 * 256 + 224;
#pragma unroll
      for (int k = 0; k < 3; k++) {
        const long long m = max(max(edge_at(E[k], sx0, sy0), edge_at(E[k], sx1, sy0)), max(edge_at(E[k], sx0, sy1), edge_at(E[k], sx1, sy1)));
        in = in && m + E[k].bias >= 0;
      }
    }
    cand[h] = in;
  }
  unsigned long long mask = (unsigned long long)__ballot_sync(0xffffffffu, cand[0]) | ((unsigned long long)__ballot_sync(0xffffffffu, cand[1]) << 32);
  long long off[3][NS];
#pragma unroll
  for (uint32_t s = 0; s < NS; s++) {
    const long long ox = NS == 1u ? 128 : (long long)((0xa020e060u >> (8 * s)) & 0xffu);
    const long long oy = NS == 1u ? 128 : 32 + 64 * (long long)s;
#pragma unroll
    for (int k = 0; k < 3; k++) off[k][s] = E[k].dx * oy - E[k].dy * ox + E[k].bias;
  }
  const float rA = 1.0f / float(A);
  const float dz1 = b.z - a.z, dz2 = c.z - a.z;
  while (mask) {
    // two candidate sub-blocks: lanes 0-15 the first, 16-31 the second
    const int q0 = __ffsll(mask) - 1;
    mask &= mask - 1;
    const int q1 = mask ? __ffsll(mask) - 1 : -1;
    if (q1 >= 0) mask &= mask - 1;
    const int q = lane < 16 ? q0 : q1;
    if (q < 0) continue;
    const int px = bx.x0 + 4 * (q % 8) + (lane & 3), py = bx.y0 + 4 * (q / 8) + ((lane >> 2) & 3);
    if (px > bx.x1 || py > bx.y1) continue;
    long long w[3];
#pragma unroll
    for (int k = 0; k < 3; k++) w[k] = edge_at(E[k], (long long)px * 256, (long long)py * 256);
#pragma unroll
    for (uint32_t s = 0; s < NS; s++)
      shade_sample<NS>(a, dz1, dz2, rA, w[0] + off[0][s], w[1] + off[1][s], w[2] + off[2][s], E[1].bias, E[2].bias, id, layer, T, px, py, s);
  }
}

__device__ __forceinline__ void raster_sub(Snap a, Snap b, Snap c, uint32_t id, uint32_t layer, const Target& T, const Box& lim, int lane,
                                           int lanes) {
  if (lanes > 1) {
    if (T.samples == 4u) raster_tile_n<4>(a, b, c, id, layer, T, lim, lane);
    else raster_tile_n<1>(a, b, c, id, layer, T, lim, lane);
    return;
  }
  if (T.samples == 4u) raster_sub_n<4>(a, b, c, id, layer, T, lim, 0, 1);
  else raster_sub_n<1>(a, b, c, id, layer, T, lim, 0, 1);
}

__device__ __forceinline__ void load_tri(const float4* clip, const uint32_t* idx, uint32_t n_verts, uint32_t tri, uint32_t layer, float4 in[3]) {
  const float4* C = clip + size_t(layer) * n_verts;
  for (int j = 0; j < 3; j++) in[j] = __ldg(C + __ldg(idx + 3u * tri + j));
}

// a triangle that needs clipping: its polygon snapped into P (returns the count, 0: nothing to draw)
__device__ __noinline__ int setup_clipped(const float4 in[3], const Target& T, Snap P[9]) {
  float4 poly[9];
  const int n = clip_poly(in, poly);
  const float W2 = float(T.W) * 0.5f, H2 = float(T.H) * 0.5f;
  for (int i = 0; i < n; i++)
    if (!snap(poly[i], W2, H2, P[i])) return 0;
  return n;
}

constexpr int TILE = 32;
__device__ __forceinline__ Box everything() { return Box{0, 1 << 30, 0, 1 << 30}; }

// a many-pixel triangle (polygon P of n snapped points, box b): one queued item per 32 x 32 tile of its box; the
// tiles that do not fit in the queue are rasterised here
__device__ void queue_tiles(const Target& T, uint32_t tri, uint32_t layer, const Box& b, const Snap* P, int n) {
  const int tx0 = b.x0 / TILE, tx1 = b.x1 / TILE, ty0 = b.y0 / TILE, ty1 = b.y1 / TILE;
  const uint32_t cnt = uint32_t((tx1 - tx0 + 1) * (ty1 - ty0 + 1));
  const uint32_t slot = atomicAdd(T.big, cnt);
  uint2* items = reinterpret_cast<uint2*>(T.big + 2);
  uint32_t t = 0;
  for (int ty = ty0; ty <= ty1; ty++)
    for (int tx = tx0; tx <= tx1; tx++, t++) {
      if (slot < T.big_cap && t < T.big_cap - slot) {
        items[slot + t] = make_uint2(tri | (layer << 28), uint32_t(tx) | (uint32_t(ty) << 16));
      } else {
        const Box lim{tx * TILE, tx * TILE + TILE - 1, ty * TILE, ty * TILE + TILE - 1};
        for (int k = 1; k + 1 < n; k++) raster_sub(P[0], P[k], P[k + 1], tri, layer, T, lim, 0, 1);
      }
    }
}

// per vertex and layer: the snapped point when the vertex lies inside every clip plane (w = 1), else w = 0 (its
// triangles take the clipping path)
__global__ void snap_kernel(const float4* __restrict__ clip, uint32_t n_verts, uint32_t v0, uint32_t nv, uint32_t layers, const Target T,
                            int4* __restrict__ snaps) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nv * layers) return;
  const size_t v = size_t(i / nv) * n_verts + v0 + i % nv;
  const float4 c = __ldg(clip + v);
  Snap s{0, 0, 0.0f};
  const bool ok = inside_all(c) && snap(c, float(T.W) * 0.5f, float(T.H) * 0.5f, s);
  snaps[v] = make_int4(s.x, s.y, __float_as_int(s.z), ok ? 1 : 0);
}

__device__ __forceinline__ bool load_snaps(const int4* snaps, const uint32_t* idx, uint32_t n_verts, uint32_t tri, uint32_t layer, Snap P[3]) {
  const int4* Sn = snaps + size_t(layer) * n_verts;
  bool ok = true;
  for (int j = 0; j < 3; j++) {
    const int4 r = __ldg(Sn + __ldg(idx + 3u * tri + j));
    P[j] = Snap{r.x, r.y, __int_as_float(r.z)};
    ok = ok && r.w != 0;
  }
  return ok;
}

__global__ void __launch_bounds__(128) raster_kernel(const float4* __restrict__ clip, const int4* __restrict__ snaps,
                                                     const uint32_t* __restrict__ idx, uint32_t n_verts, uint32_t t0, uint32_t nt,
                                                     uint32_t layers, const Target T) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nt * layers) return;
  const uint32_t layer = i / nt, tri = t0 + i % nt;
  {
    Snap P[3];
    if (load_snaps(snaps, idx, n_verts, tri, layer, P)) {
      Box b;
      if (!box_of(P, 3, T, b)) return;
      if ((b.x1 - b.x0 + 1) * (b.y1 - b.y0 + 1) * int(T.samples) > int(BIG_SAMPLES)) { queue_tiles(T, tri, layer, b, P, 3); return; }
      raster_sub(P[0], P[1], P[2], tri, layer, T, everything(), 0, 1);
      return;
    }
  }
  float4 in[3];
  load_tri(clip, idx, n_verts, tri, layer, in);
  if (in[0].z < 0.0f && in[1].z < 0.0f && in[2].z < 0.0f) return;   // wholly behind the near plane (dropped vertices)
  if (inside_all(in[0]) && inside_all(in[1]) && inside_all(in[2])) return;   // inside but not projectable (w = 0)
  Snap P[9];
  const int n = setup_clipped(in, T, P);
  if (n < 3) return;
  Box b;
  if (!box_of(P, n, T, b)) return;
  if ((b.x1 - b.x0 + 1) * (b.y1 - b.y0 + 1) * int(T.samples) > int(BIG_SAMPLES)) { queue_tiles(T, tri, layer, b, P, n); return; }
  for (int k = 1; k + 1 < n; k++) raster_sub(P[0], P[k], P[k + 1], tri, layer, T, everything(), 0, 1);
}

// the queued (triangle, tile) items: one warp per item, lanes over the tile's pixels
__global__ void __launch_bounds__(256) raster_big_kernel(const float4* __restrict__ clip, const int4* __restrict__ snaps,
                                                         const uint32_t* __restrict__ idx, uint32_t n_verts, const Target T) {
  const uint32_t count = min(*(volatile uint32_t*)T.big, T.big_cap);
  const uint2* items = reinterpret_cast<const uint2*>(T.big + 2);
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nwarps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t q = warp; q < count; q += nwarps) {
    const uint2 e = items[q];
    const uint32_t tri = e.x & 0x0fffffffu, layer = e.x >> 28;
    const int tx = int(e.y & 0xffffu), ty = int(e.y >> 16);
    const Box lim{tx * TILE, tx * TILE + TILE - 1, ty * TILE, ty * TILE + TILE - 1};
    Snap P3[3];
    if (load_snaps(snaps, idx, n_verts, tri, layer, P3)) {
      raster_sub(P3[0], P3[1], P3[2], tri, layer, T, lim, int(lane), 32);
      __syncwarp();
      continue;
    }
    float4 in[3];
    load_tri(clip, idx, n_verts, tri, layer, in);
    Snap P[9];
    const int n = setup_clipped(in, T, P);
    for (int k = 1; k + 1 < n; k++) raster_sub(P[0], P[k], P[k + 1], tri, layer, T, lim, int(lane), 32);
    __syncwarp();   // the lanes leave an item together
  }
}

__global__ void fill_kernel(uint32_t* p, size_t n, uint32_t value) {
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) p[i] = value;
}

}  // namespace

void launch_raster(const float4* clip, int4* snaps, const uint32_t* idx, uint32_t n_verts, uint32_t v0, uint32_t nv, uint32_t t0, uint32_t nt,
                   uint32_t layers, const Target& T, int blocks_big, cudaStream_t st) {
  cudaMemsetAsync(T.big, 0, 4, st);
  if (nv) snap_kernel<<<uint32_t((size_t(nv) * layers + 255) / 256), 256, 0, st>>>(clip, n_verts, v0, nv, layers, T, snaps);
  const size_t n = size_t(nt) * layers;
  if (n) raster_kernel<<<uint32_t((n + 127) / 128), 128, 0, st>>>(clip, snaps, idx, n_verts, t0, nt, layers, T);
  raster_big_kernel<<<blocks_big, 256, 0, st>>>(clip, snaps, idx, n_verts, T);
}
void launch_fill(uint32_t* p, size_t n, uint32_t value, cudaStream_t st) {
  fill_kernel<<<1024, 256, 0, st>>>(p, n, value);
}

}  // namespace vtl
