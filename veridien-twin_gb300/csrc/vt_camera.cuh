// Camera sub-samples shared by the wavefront renderer and the calibration kernels: pixel enumeration and the KB4
// camera ray of a (pixel, sub-sample) pair with its sample numbers (gpu/wgsl/kernels.wgsl.js:34-53, 161-213).
#pragma once

#include "vt_kernels.cuh"

namespace vtk {
using namespace vtd;

// pixel id (tiled order, so consecutive paths are neighbouring pixels) -> x, y
__device__ __forceinline__ bool pixel_xy(const CamParams& cp, uint32_t id, uint32_t& x, uint32_t& y) {
  const uint32_t tw = cp.tile_w, th = cp.tile_h;
  const uint32_t tiles_x = (cp.w + tw - 1) / tw;
  const uint32_t tile = id / (tw * th), within = id % (tw * th);
  x = (tile % tiles_x) * tw + within % tw;
  y = (tile / tiles_x) * th + within / tw;
  return x < cp.w && y < cp.h;
}

// the image position (u, v) of sub-sample i of pixel (x, y): the pixel box jittered by the R2 sequence
// (gpu/wgsl/kernels.wgsl.js:177-185)
__device__ __forceinline__ float2 subsample_uv(uint32_t x, uint32_t y, uint32_t i, uint32_t hs) {
  const float u = __fsub_rn(__fadd_rn(float(x), kr(i, R2A, u01(pcg(hs)))), 0.5f);
  const float v = __fsub_rn(__fadd_rn(float(y), kr(i, R2B, u01(pcg(hs + 1u)))), 0.5f);
  return make_float2(u, v);
}

// the camera sub-sample (pixel id, index i): KB4 ray, exposure time and pixel hash (gpu/wgsl/kernels.wgsl.js:35
// pixSeeds, :177-185 camMain sub-samples)
__device__ __forceinline__ bool camera_path(const CamParams& cp, uint32_t id, uint32_t i, float4& o4, float4& d4, uint32_t& hs) {
  uint32_t x, y;
  const bool valid = pixel_xy(cp, id, x, y);
  hs = hash3(x, y, cp.seed * 64u + cp.cam_index);
  float3 d = f3(0, 0, 1);
  float tt = 0.0f;
  if (valid) {
    const float2 uv = subsample_uv(x, y, i, hs);
    const float u = uv.x, v = uv.y;
    tt = mixr(cp.t0, cp.t1, kr(i, GOLD, u01(pcg(hs + 2u))));
    const float3 rx = f3(cp.rx[0], cp.rx[1], cp.rx[2]), ry = f3(cp.ry[0], cp.ry[1], cp.ry[2]), rz = f3(cp.rz[0], cp.rz[1], cp.rz[2]);
    const float3 dc = kb4_unproject(cp.lens, u, v);
    d = normalize(rx * dc.x + ry * dc.y + rz * dc.z);
  }
  o4 = make_float4(cp.pos[0], cp.pos[1], cp.pos[2], tt);
  d4 = make_float4(d.x, d.y, d.z, 0.0f);
  return valid;
}

}  // namespace vtk
