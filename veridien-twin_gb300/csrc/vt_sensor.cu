// Sensor expose stage on sm_103a (gpu/wgsl/sensor.wgsl.js:177 sensorExpose): vertical optics blur of the
// irradiance image, then the per-pixel sensor model of vt_sensor.cuh. One thread per pixel; HBM-bound (16 B read,
// 4 B written per pixel, plus the blur's neighbouring rows from L1/L2).
#include "vt_kernels.cuh"
#include "vt_sensor.cuh"

namespace vtk {

template <typename OUT>
__global__ void sensor_expose_kernel(const SensorParams su, const float4* __restrict__ E, float scale, OUT* __restrict__ raw) {
  const int W = int(su.w[0]), H = int(su.w[1]);
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= W || y >= H) return;
  const float* f = reinterpret_cast<const float*>(su.w);
  const float sg = f[5];
  const int r = min(max(int(ceilf(3.0f * sg + 0.5f)), 0), 12);
  float ex = 0.0f, ey = 0.0f, ez = 0.0f, ws = 0.0f;
  for (int k = -r; k <= r; k++) {
    const int yy = min(max(y + k, 0), H - 1);
    const float w = tapW(k, sg);
    float4 e = __ldg(E + size_t(yy) * W + x);
    if (scale != 1.0f) e = make_float4(__fmul_rn(e.x, scale), __fmul_rn(e.y, scale), __fmul_rn(e.z, scale), e.w);
    ex = __fmaf_rn(w, e.x, ex); ey = __fmaf_rn(w, e.y, ey); ez = __fmaf_rn(w, e.z, ez);
    ws = __fadd_rn(ws, w);
  }
  ex = __fdiv_rn(ex, ws); ey = __fdiv_rn(ey, ws); ez = __fdiv_rn(ez, ws);
  raw[size_t(y) * W + x] = OUT(sensor_dn(su.w, ex, ey, ez, x, y, W, su.w[3]));
}

void launch_sensor_expose(const SensorParams& su, const float4* E, float scale, float* raw, cudaStream_t st) {
  const dim3 b(16, 8), g((su.w[0] + 15) / 16, (su.w[1] + 7) / 8);
  sensor_expose_kernel<float><<<g, b, 0, st>>>(su, E, scale, raw);
}
void launch_sensor_expose_u16(const SensorParams& su, const float4* E, float scale, uint16_t* raw, cudaStream_t st) {
  const dim3 b(16, 8), g((su.w[0] + 15) / 16, (su.w[1] + 7) / 8);
  sensor_expose_kernel<uint16_t><<<g, b, 0, st>>>(su, E, scale, raw);
}

}  // namespace vtk
