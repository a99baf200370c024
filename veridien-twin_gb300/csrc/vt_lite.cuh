// The raster camera pass of lite_nodes (vt_lite.cu): view uniform, buffers and launchers.
//
// Pipeline per camera view (lite_nodes/renderer.js:844 renderCamera):
//   vertex     one thread per raster vertex: world position (posed bodies at mid-exposure), clip coordinates
//              (KB4 or pinhole camera; equidistant sector projection for the shadow maps, 4 sectors at once)
//   raster     (vt_lite_raster.cu) one thread per triangle: clip against 0 <= z <= w and a guard band |x|, |y| <= 8 w,
//              snap to 1/256 pixel, exact int64 edge functions; every covered sample takes atomicMin(depth bits << 32
//              | triangle) (64-bit keys for the camera's 4 samples, 32-bit depth for a shadow map). Triangles whose
//              box holds more than 256 samples are queued as 32 x 32-pixel tiles that a warp per tile rasterises.
//   shade      a fragment list (each distinct triangle among a pixel's samples, static and posed-body fragments
//              apart), one thread per fragment shading at the pixel centre (the fragment stage, colours rounded to
//              half), then per pixel the average of the samples rounded to half and scaled back (the MSAA resolve
//              into rgba16float and the FINISH pass)
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "vt_device.cuh"

namespace vtl {

constexpr uint32_t K_SECT = 4;          // emitter sectors = shadow maps (lite_nodes/renderer.js:58)
constexpr uint32_t STATIC_INST = 0xffffu;
constexpr uint32_t BIG_SAMPLES = 256;   // a triangle box with more samples goes to the warp-per-tile path
constexpr float GUARD = 8.0f;           // clip-space guard band: |x|, |y| <= GUARD w
constexpr unsigned long long EMPTY_KEY = ~0ull;

// the view uniform (lite_nodes/renderer.js:72-84 ViewU, written by _viewData :766); the same 128 floats are what
// vt_lite_debug(VT_LITE_VIEW) returns
struct View {
  float rx[4], ry[4], rz[4];   // camera axes in the dome frame (x right, y down, z forward)
  float pos[4];                // centre; w = mode (0 kb4, 1 pinhole, 2 shadow)
  float lensA[4];              // fx fy cx cy
  float lensB[4];              // k1..k4
  float size[4];               // w h thetaCut outScale
  uint32_t misc[4];            // skip mask, static samples, dynamic samples, casters (0 all, 1 static, 2 dynamic)
  float env[4];                // environment radiance of posed bodies (rgb), time
  float axisW[4];              // emission axis (world), debug mode
  float lt[4], lb[4];          // shadow frame tangent / bitangent (world); lt.w = thetaMax, lb.w = far
  float lo[K_SECT][4];         // shadow origins (world); w = depth bias for static receivers (m)
  float pad[128 - 64];
};
static_assert(sizeof(View) == 512, "view uniform is 128 words");

struct Geo {
  const uint4* v;              // 2 per vertex: position | mesh + instance << 16, normal | node
  const uint32_t* idx;         // 3 per triangle
  const float4* es;            // 2 per emitter sample (world): position | sector, normal | area
  uint32_t n_verts, n_tris, n_static_verts, n_static_tris;
};

// a raster target: w x h pixels of `samples` (4: MSAA, 64-bit keys; 1: a shadow map layer, 32-bit depth bits)
struct Target {
  uint32_t W, H, samples;
  unsigned long long* key;     // samples == 4
  uint32_t* depth;             // samples == 1: layers of W x H, one per sector
  uint32_t* big;               // [0] count, [1] unused, then (triangle | sector << 28, tile x | tile y << 16) items
  uint32_t big_cap;            // items
};

struct ShadeArgs {
  const unsigned long long* key;
  const float4* clip;
  const uint32_t* sm_static;   // K_SECT x res x res depth bits (all ones: cleared)
  const uint32_t* sm_dyn;
  uint32_t sm_res;
  float inv_scale;             // 1 / outScale (float of the double quotient)
  float circle;                // SCOPE image circle radius in pixels, 0 = none
  uint32_t env_mat;
  float4* out;                 // radiance (w x h)
};

// vertex stage: clip coordinates of vertices [first, first + count) for a camera view (mode 0 / 1) into clip[v]
void launch_vertex_cam(const vtd::Scene& S, const Geo& g, const View& v, uint32_t first, uint32_t count, float4* clip, cudaStream_t st);
// vertex stage of the shadow maps: K_SECT layers of clip coordinates, clip[k * n_verts + v]
void launch_vertex_shadow(const vtd::Scene& S, const Geo& g, const View& v, uint32_t first, uint32_t count, float4* clip, cudaStream_t st);
// raster of triangles [t0, t0 + nt) over clip (n_verts per layer; `layers` sector layers for a shadow target), whose
// vertices are [v0, v0 + nv); snaps: scratch of one int4 per clip entry
void launch_raster(const float4* clip, int4* snaps, const uint32_t* idx, uint32_t n_verts, uint32_t v0, uint32_t nv, uint32_t t0, uint32_t nt,
                   uint32_t layers, const Target& T, int blocks_big, cudaStream_t st);
// the fragment list and its shading (scratch for a w x h view: frags and colors w*h*4 entries, sidx w*h)
struct FragBufs {
  uint2* frags;                // (pixel, triangle): static fragments from the front, posed-body ones from the back
  uint2* colors;               // per fragment: rgb as half floats
  uint4* sidx;                 // per pixel: each sample's fragment, MISS = empty
  uint32_t* counts;            // [0] static, [1] posed-body fragments
};
// fragment list + fragment stage + resolve + finish
void launch_shade(const vtd::Scene& S, const Geo& g, const View& v, const ShadeArgs& a, const FragBufs& fb, int sms, cudaStream_t st);
// clear a 32-bit depth target to all ones
void launch_fill(uint32_t* p, size_t n, uint32_t value, cudaStream_t st);

}  // namespace vtl
