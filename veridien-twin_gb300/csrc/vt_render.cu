// Ray queries on sm_103a: traceTest (gpu/wgsl/kernels.wgsl.js:535) and visible (gpu/renderer.js:1238). Camera
// rendering is the wavefront path tracer in vt_wave.cu.
#include <algorithm>

#include "vt_kernels.cuh"

namespace vtk {
using namespace vtd;

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
