// Camera rendering and ray queries on sm_103a.
//
// render_kernel: one persistent launch per camera. Each warp pulls an 8x4 pixel tile from a device counter (one
// atomic per warp), and each lane renders its pixel's spp sub-samples in order, so a pixel's sum is the same on
// every run (gpu/renderer.js:60-61 "a fixed seed renders a static frame identically"). Per sub-sample: the KB4 ray
// of its stratified sub-pixel position (gpu/wgsl/kernels.wgsl.js:177-185), the static BVH then the posed bodies
// (kernels.wgsl.js:194-198), and the estimator (shadeHit or the depth-N path tracer).
#include "vt_kernels.cuh"

namespace vtk {
using namespace vtd;

__global__ void __launch_bounds__(RENDER_THREADS) render_kernel(const Scene S, const CamParams cp, float4* __restrict__ out,
                                                              uint32_t* __restrict__ work_counter) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t tiles_x = (cp.w + TILE_W - 1) / TILE_W;
  const uint32_t n_tiles = tiles_x * ((cp.h + TILE_H - 1) / TILE_H);
  const float3 rx = f3(cp.rx[0], cp.rx[1], cp.rx[2]), ry = f3(cp.ry[0], cp.ry[1], cp.ry[2]), rz = f3(cp.rz[0], cp.rz[1], cp.rz[2]);
  const float3 pos = f3(cp.pos[0], cp.pos[1], cp.pos[2]);
  const uint32_t spp = cp.spp;
  const uint32_t nl = max(1u, cp.n_light);
  for (;;) {
    uint32_t tile = 0;
    if (lane == 0) tile = atomicAdd(work_counter, 1u);
    tile = __shfl_sync(0xffffffffu, tile, 0);
    if (tile >= n_tiles) break;
    const uint32_t x = (tile % tiles_x) * TILE_W + (lane % TILE_W);
    const uint32_t y = (tile / tiles_x) * TILE_H + (lane / TILE_W);
    if (x >= cp.w || y >= cp.h) continue;
    const Seeds sd = pixel_seeds(x, y, cp.seed, cp.cam_index);
    float3 acc = f3(0, 0, 0);
    uint32_t key = 0;
    for (uint32_t i = 0; i < spp; i++) {
      const float u = __fsub_rn(__fadd_rn(float(x), kr(i, R2A, sd.s[0])), 0.5f);
      const float v = __fsub_rn(__fadd_rn(float(y), kr(i, R2B, sd.s[1])), 0.5f);
      const float tt = mixr(cp.t0, cp.t1, kr(i, GOLD, sd.s[2]));
      const float3 dc = kb4_unproject(cp.lens, u, v);
      const float3 d = normalize(rx * dc.x + ry * dc.y + rz * dc.z);
      const float3 ul = f3(kr(i * nl, KL0, sd.s[3]), kr(i * nl, KL1, sd.s[4]), kr(i * nl, KL2, sd.s[5]));
      const float3 ub = f3(kr(i, KB0, sd.s[6]), kr(i, KB1, sd.s[7]), kr(i, KB2, sd.s[8]));
      Hit h = trace_scene<false>(S, cp.root, pos, d, 0.0f, BIG, tt, 1u, 0u);
      const Hit hd = trace_scene<false>(S, cp.root, pos, d, 0.0f, h.t, tt, 2u, cp.skip);
      if (hd.tri != MISS) h = hd;
      uint32_t gk;
      const float3 c = cp.mode == VT_SHADE_TWIN
                           ? shade_twin(S, cp.root, h, pos, d, tt, ul, ub, cp.options, i * nl, sd, cp.n_light, gk)
                           : shade_path(S, cp.root, h, pos, d, tt, ul, ub, cp.options, i, sd, cp.n_light, cp.max_depth, gk);
      acc = acc + c;
      if (i == 0) key = gk;
      else if ((gk & 0xffffu) != (key & 0xffffu)) key |= 0x40000u;
      key |= gk & 0x30000u;
    }
    const float sc = cp.scale / float(spp);
    out[size_t(y) * cp.w + x] = make_float4(acc.x * sc, acc.y * sc, acc.z * sc, key == 0xfffeu ? 0.0f : 1.0f);
  }
}

int render_blocks_per_sm() {
  int n = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, render_kernel, RENDER_THREADS, 0);
  return n > 0 ? n : 1;
}

void launch_render(const Scene& S, const CamParams& cp, float4* out, uint32_t* work_counter, int blocks, cudaStream_t st) {
  render_kernel<<<blocks, RENDER_THREADS, 0, st>>>(S, cp, out, work_counter);
}

// gpu/wgsl/kernels.wgsl.js:535 traceTest: one ray per thread
__global__ void trace_kernel(const Scene S, const float4* __restrict__ o4, const float4* __restrict__ d4, uint32_t n, uint32_t mask,
                             uint32_t any_hit, uint32_t root, float4* __restrict__ out4, float* __restrict__ out_v) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 o = o4[i], d = d4[i];
  const Hit h = any_hit ? trace_scene<true>(S, root, xyz(o), xyz(d), 0.0f, BIG, o.w, mask, 0u)
                        : trace_scene<false>(S, root, xyz(o), xyz(d), 0.0f, BIG, o.w, mask, 0u);
  out4[i] = make_float4(h.t, __uint_as_float(h.tri), __uint_as_float(h.inst), h.u);
  if (out_v) out_v[i] = h.v;
}

void launch_trace(const Scene& S, const float4* o4, const float4* d4, uint32_t n, uint32_t mask, uint32_t any_hit, uint32_t root,
                  float4* out4, float* out_v, cudaStream_t st) {
  if (!n) return;
  trace_kernel<<<(n + 127) / 128, 128, 0, st>>>(S, o4, d4, n, mask, any_hit, root, out4, out_v);
}

// gpu/renderer.js:1238 visible: occlusion between the camera centre and each point (static BVH from its full root,
// then every posed body at `time`, the camera's own bodies skipped)
__global__ void visible_kernel(const Scene S, float3 c, const float3* __restrict__ pts, uint32_t n, float tol, float time, uint32_t skip,
                               uint8_t* __restrict__ out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float3 v = pts[i] - c;
  const float dist = length(v);
  if (!(dist > tol)) { out[i] = 1; return; }
  const float3 d = v / dist;
  const Hit h = trace_scene<true>(S, 0u, c, d, 0.0f, dist - tol, time, 3u, skip);
  out[i] = h.tri == MISS ? 1 : 0;
}

void launch_visible(const Scene& S, float3 c, const float3* pts, uint32_t n, float tol, float time, uint32_t skip, uint8_t* out,
                    cudaStream_t st) {
  if (!n) return;
  visible_kernel<<<(n + 127) / 128, 128, 0, st>>>(S, c, pts, n, tol, time, skip, out);
}

}  // namespace vtk
