// The camera sensor chain after the path tracer, radiance -> raw DN -> 8-bit RGB and YCbCr (gpu/wgsl/sensor.wgsl.js):
//   isp_optics       E = L (pi T / 4 N^2) RI, the horizontal half of the optics blur (pixel-integrated Gaussian)
//   glare_down/blur  veiling glare on a 1/F level: box mean, then a Gaussian over whole rows and columns (zero outside)
//   isp_expose       the vertical half of the blur, the glare mix E' = (1 - k) E + k G, the sensor model (vt_sensor.cuh)
//   demosaic_g       green plane: bilinear, edge-aware (OpenCV EA) or Hamilton-Adams
//   demosaic_rb      red and blue (colour differences or bilinear), black level, white-balance statistics, WB, CCM
//   isp_nr           3x3 bilateral on linear RGB, range sigma from the modelled shot + read noise
//   isp_output       tone curve, unsharp mask on luma, BT.601 full-range YCbCr, 4:2:0 chroma, 8-bit RGB, luma sum
// Each stage is one pass over the frame (a 1920x1200 frame is 2.3 M pixels: every pass is HBM/L2-bound at a few
// microseconds); the statistics are integer sums of per-block partials added by one small kernel, so they do not
// depend on scheduling.
//
// This translation unit is compiled without multiply-add contraction (--fmad=false) and uses the fixed-order
// elementary functions of vt_sensor.cuh, so every value is the one the CPU restatement computes from the same
// sequence of IEEE operations: raw DN, 8-bit RGB, YCbCr planes and statistics are bit-identical to it.
#include <cstring>

#include "vt_isp.cuh"
#include "vt_sensor.cuh"

namespace vtk {

namespace {

struct Su {
  const uint32_t* w;
  __device__ float f(int i) const { return __uint_as_float(w[i]); }
};

__device__ __forceinline__ float vt_powf(float x, float y) {
  if (!(x > 0.0f)) return y == 0.0f ? 1.0f : 0.0f;
  return vt_expf(y * vt_logf(x));
}
__device__ __forceinline__ int clampi(int v, int a, int b) { return v < a ? a : v > b ? b : v; }
__device__ __forceinline__ float clamp01(float v) { return fminf(fmaxf(v, 0.0f), 1.0f); }
__device__ __forceinline__ int gauss_taps(float sg) { return clampi(int(ceilf(3.0f * sg + 0.5f)), 0, 12); }

// 2x2 CFA: codes RGGB, GRBG, GBRG, BGGR; channel 0 R, 1 G, 2 B
__device__ __forceinline__ uint32_t cfa_channel(uint32_t code, uint32_t x, uint32_t y) {
  const uint32_t pats = code == 0 ? 0x2110u : code == 1 ? 0x1201u : code == 2 ? 0x1021u : 0x0112u;
  return (pats >> (4u * ((y & 1u) * 2u + (x & 1u)))) & 0xfu;
}

}  // namespace

// the blur's tap weights depend only on the tap: each block evaluates them once into shared memory
__device__ __forceinline__ void block_taps(float sg, int r, float* taps) {
  const int t = threadIdx.y * blockDim.x + threadIdx.x;
  if (t <= 2 * r) taps[t] = tapW(t - r, sg);
  __syncthreads();
}

__global__ void isp_optics_kernel(const SensorParams P, const float4* __restrict__ L, const float* __restrict__ ri, float4* __restrict__ A) {
  __shared__ float taps[25];
  const Su su{P.w};
  const int W = int(P.w[0]), H = int(P.w[1]);
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
  const float sg = su.f(5);
  const int r = gauss_taps(sg);
  block_taps(sg, r, taps);
  if (x >= W || y >= H) return;
  float ax = 0.0f, ay = 0.0f, az = 0.0f, ws = 0.0f;
  for (int k = -r; k <= r; k++) {
    const int xx = clampi(x + k, 0, W - 1);
    const float w = taps[k + r];
    const float4 l = __ldg(L + size_t(y) * W + xx);
    const float m = __ldg(ri + size_t(y) * W + xx);
    ax = ax + w * l.x * m;
    ay = ay + w * l.y * m;
    az = az + w * l.z * m;
    ws = ws + w;
  }
  const float s = su.f(4) / ws;
  A[size_t(y) * W + x] = make_float4(ax * s, ay * s, az * s, 1.0f);
}

__global__ void glare_down_kernel(const SensorParams P, const float4* __restrict__ L, const float* __restrict__ ri, float4* __restrict__ G) {
  const Su su{P.w};
  const int W = int(P.w[0]), H = int(P.w[1]), F = int(su.f(54));
  const int gw = (W + F - 1) / F, gh = (H + F - 1) / F;
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= gw || y >= gh) return;
  float ax = 0.0f, ay = 0.0f, az = 0.0f, n = 0.0f;
  const int fm = min(F, 32);
  for (int j = 0; j < fm; j++)
    for (int i = 0; i < fm; i++) {
      const int xx = x * F + i, yy = y * F + j;
      if (xx >= W || yy >= H) continue;
      const float4 l = __ldg(L + size_t(yy) * W + xx);
      const float m = __ldg(ri + size_t(yy) * W + xx);
      ax = ax + l.x * m;
      ay = ay + l.y * m;
      az = az + l.z * m;
      n = n + 1.0f;
    }
  const float s = su.f(4) / fmaxf(n, 1.0f);
  G[size_t(y) * gw + x] = make_float4(ax * s, ay * s, az * s, 1.0f);
}

// a Gaussian over the whole row (dir 0) or column (dir 1) of the level, zero outside, normalised on the infinite line
__global__ void glare_blur_kernel(const SensorParams P, const float4* __restrict__ Gin, float4* __restrict__ Gout, int dir) {
  const Su su{P.w};
  const int W = int(P.w[0]), H = int(P.w[1]), F = int(su.f(54));
  const int gw = (W + F - 1) / F, gh = (H + F - 1) / F;
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= gw || y >= gh) return;
  const float sg = fmaxf(su.f(53), 1e-3f);
  const int n = dir == 0 ? gw : gh, c = dir == 0 ? x : y;
  float ax = 0.0f, ay = 0.0f, az = 0.0f;
  for (int k = 0; k < min(n, 256); k++) {
    const float d = float(k - c);
    const float w = vt_expf(-0.5f * d * d / (sg * sg));
    const float4 g = Gin[dir == 0 ? size_t(y) * gw + k : size_t(k) * gw + x];
    ax = ax + w * g.x;
    ay = ay + w * g.y;
    az = az + w * g.z;
  }
  const float s = sg * 2.5066282746f;
  Gout[size_t(y) * gw + x] = make_float4(ax / s, ay / s, az / s, 1.0f);
}

__device__ __forceinline__ float3 glare_at(const Su& su, const float4* __restrict__ G, int x, int y, int W, int H) {
  const float F = su.f(54);
  const int Fi = int(F);
  const int gw = (W + Fi - 1) / Fi, gh = (H + Fi - 1) / Fi;
  const float px = (float(x) + 0.5f) / F - 0.5f, py = (float(y) + 0.5f) / F - 0.5f;
  const float fx0 = floorf(px), fy0 = floorf(py);
  const int x0 = int(fx0), y0 = int(fy0);
  const float fx = px - fx0, fy = py - fy0;
  auto at = [&](int xx, int yy) { const float4 g = G[size_t(clampi(yy, 0, gh - 1)) * gw + clampi(xx, 0, gw - 1)]; return make_float3(g.x, g.y, g.z); };
  const float3 a = at(x0, y0), b = at(x0 + 1, y0), c = at(x0, y0 + 1), d = at(x0 + 1, y0 + 1);
  auto mix = [](float p, float q, float t) { return p * (1.0f - t) + q * t; };
  return make_float3(mix(mix(a.x, b.x, fx), mix(c.x, d.x, fx), fy), mix(mix(a.y, b.y, fx), mix(c.y, d.y, fx), fy),
                     mix(mix(a.z, b.z, fx), mix(c.z, d.z, fx), fy));
}

__global__ void isp_expose_kernel(const SensorParams P, const float4* __restrict__ A, const float4* __restrict__ G, float* __restrict__ raw) {
  __shared__ float taps[25];
  const Su su{P.w};
  const int W = int(P.w[0]), H = int(P.w[1]);
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
  const float sg = su.f(5);
  const int r = gauss_taps(sg);
  block_taps(sg, r, taps);
  if (x >= W || y >= H) return;
  float ex = 0.0f, ey = 0.0f, ez = 0.0f, ws = 0.0f;
  for (int k = -r; k <= r; k++) {
    const int yy = clampi(y + k, 0, H - 1);
    const float w = taps[k + r];
    const float4 e = A[size_t(yy) * W + x];
    ex = ex + w * e.x;
    ey = ey + w * e.y;
    ez = ez + w * e.z;
    ws = ws + w;
  }
  ex = ex / ws; ey = ey / ws; ez = ez / ws;
  const float k = su.f(52);
  if (k > 0.0f) {
    const float3 g = glare_at(su, G, x, y, W, H);
    ex = (1.0f - k) * ex + k * g.x;
    ey = (1.0f - k) * ey + k * g.y;
    ez = (1.0f - k) * ez + k * g.z;
  }
  raw[size_t(y) * W + x] = sensor_dn(P.w, ex, ey, ez, x, y, W, P.w[3]);
}

// raw DN mirrored at the borders (reflect by one, which keeps the CFA phase), then clamped
__device__ __forceinline__ float raw_at(const float* __restrict__ raw, int x, int y, int W, int H) {
  if (x < 0) x = -x;
  if (x >= W) x = 2 * (W - 1) - x;
  if (y < 0) y = -y;
  if (y >= H) y = 2 * (H - 1) - y;
  return raw[size_t(clampi(y, 0, H - 1)) * W + clampi(x, 0, W - 1)];
}

__global__ void demosaic_g_kernel(const SensorParams P, const float* __restrict__ raw, float* __restrict__ gpl) {
  const Su su{P.w};
  const int W = int(P.w[0]), H = int(P.w[1]);
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= W || y >= H) return;
  float g = raw_at(raw, x, y, W, H);
  if (cfa_channel(P.w[2], uint32_t(x), uint32_t(y)) != 1u) {
    const float gl = raw_at(raw, x - 1, y, W, H), gr = raw_at(raw, x + 1, y, W, H);
    const float gu = raw_at(raw, x, y - 1, W, H), gd = raw_at(raw, x, y + 1, W, H);
    const uint32_t mode = P.w[50];
    if (mode == 0) {
      g = 0.25f * (gl + gr + gu + gd);
    } else if (mode == 1) {
      const float dh = fabsf(gl - gr), dv = fabsf(gu - gd);
      g = dh < dv ? 0.5f * (gl + gr) : dv < dh ? 0.5f * (gu + gd) : 0.25f * (gl + gr + gu + gd);
    } else {
      const float c = g;
      const float lh = 2.0f * c - raw_at(raw, x - 2, y, W, H) - raw_at(raw, x + 2, y, W, H);
      const float lv = 2.0f * c - raw_at(raw, x, y - 2, W, H) - raw_at(raw, x, y + 2, W, H);
      const float dh = fabsf(gl - gr) + fabsf(lh), dv = fabsf(gu - gd) + fabsf(lv);
      const float gh = 0.5f * (gl + gr) + 0.25f * lh, gv = 0.5f * (gu + gd) + 0.25f * lv;
      g = dh < dv ? gh : dv < dh ? gv : 0.5f * (gh + gv);
      g = fminf(fmaxf(g, 0.0f), su.f(24));
    }
  }
  gpl[size_t(y) * W + x] = g;
}

// a block's sums of v[0..2] (256 threads) written to out[0..2]
__device__ __forceinline__ void block_sum3(const uint32_t v[3], uint32_t* out) {
  __shared__ uint32_t sm[8][3];
  const int t = threadIdx.y * blockDim.x + threadIdx.x, lane = t & 31, warp = t >> 5;
  uint32_t a[3] = {v[0], v[1], v[2]};
  for (int k = 0; k < 3; k++)
    for (int s = 16; s > 0; s >>= 1) a[k] += __shfl_xor_sync(0xffffffffu, a[k], s);
  if (lane == 0)
    for (int k = 0; k < 3; k++) sm[warp][k] = a[k];
  __syncthreads();
  if (t < 3) {
    uint32_t s = 0;
    for (int w = 0; w < int(blockDim.x * blockDim.y) / 32; w++) s += sm[w][t];
    out[t] = s;
  }
}

__global__ void __launch_bounds__(256) demosaic_rb_kernel(const SensorParams P, const float* __restrict__ raw, const float* __restrict__ gpl,
                                                          float4* __restrict__ B, uint32_t* __restrict__ part) {
  const Su su{P.w};
  const int W = int(P.w[0]), H = int(P.w[1]);
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
  uint32_t q[3] = {0u, 0u, 0u};
  if (x < W && y < H) {
    const uint32_t code = P.w[2], mode = P.w[50];
    const uint32_t own = cfa_channel(code, uint32_t(x), uint32_t(y));
    auto g_at = [&](int xx, int yy) { return gpl[size_t(clampi(yy, 0, H - 1)) * W + clampi(xx, 0, W - 1)]; };
    const float g = g_at(x, y);
    float sr = 0.0f, sb = 0.0f, cr = 0.0f, cb = 0.0f;
    for (int dy = -1; dy <= 1; dy++)
      for (int dx = -1; dx <= 1; dx++) {
        const int xx = clampi(x + dx, 0, W - 1), yy = clampi(y + dy, 0, H - 1);
        const uint32_t ch = cfa_channel(code, uint32_t(xx), uint32_t(yy));
        if (ch == 1u) continue;
        if (ch == own && !(dx == 0 && dy == 0)) continue;
        const float d = raw_at(raw, xx, yy, W, H) - g_at(xx, yy);
        if (ch == 0u) { sr = sr + d; cr = cr + 1.0f; } else { sb = sb + d; cb = cb + 1.0f; }
      }
    float r = g + sr / fmaxf(cr, 1.0f), gg = g, b = g + sb / fmaxf(cb, 1.0f);
    if (mode <= 1u) {
      float s0 = 0.0f, s1 = 0.0f, s2 = 0.0f, c0 = 0.0f, c1 = 0.0f, c2 = 0.0f;
      for (int dy = -1; dy <= 1; dy++)
        for (int dx = -1; dx <= 1; dx++) {
          const int xx = clampi(x + dx, 0, W - 1), yy = clampi(y + dy, 0, H - 1);
          const uint32_t ch = cfa_channel(code, uint32_t(xx), uint32_t(yy));
          if (ch == own && !(dx == 0 && dy == 0)) continue;
          if (ch == 1u && own == 1u && !(dx == 0 && dy == 0)) continue;
          const float v = raw_at(raw, xx, yy, W, H);
          if (ch == 0u) { s0 = s0 + v; c0 = c0 + 1.0f; } else if (ch == 1u) { s1 = s1 + v; c1 = c1 + 1.0f; } else { s2 = s2 + v; c2 = c2 + 1.0f; }
        }
      r = s0 / fmaxf(c0, 1.0f);
      gg = s1 / fmaxf(c1, 1.0f);
      b = s2 / fmaxf(c2, 1.0f);
      if (mode == 1u) gg = g;
    }
    const float black = su.f(25), full = fmaxf(su.f(24) - black, 1.0f);
    float c[3] = {(r - black) / full, (gg - black) / full, (b - black) / full};
    for (int k = 0; k < 3; k++) q[k] = uint32_t(rintf(clamp01(c[k]) * 1023.0f));
    for (int k = 0; k < 3; k++) c[k] = c[k] * su.f(28 + k);
    float o[3];
    for (int k = 0; k < 3; k++) o[k] = su.f(32 + 4 * k) * c[0] + su.f(33 + 4 * k) * c[1] + su.f(34 + 4 * k) * c[2];
    B[size_t(y) * W + x] = make_float4(o[0], o[1], o[2], 1.0f);
  }
  // white-balance statistics: integer sums per block into this block's partial (added up by isp_stats_kernel)
  block_sum3(q, part + 3 * size_t(blockIdx.y * gridDim.x + blockIdx.x));
}

__global__ void isp_nr_kernel(const SensorParams P, const float4* __restrict__ B, float4* __restrict__ A) {
  const Su su{P.w};
  const int W = int(P.w[0]), H = int(P.w[1]);
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= W || y >= H) return;
  const float4 c0 = B[size_t(y) * W + x];
  if (P.w[51] == 0u || su.f(58) <= 0.0f) { A[size_t(y) * W + x] = c0; return; }
  const float Y0 = fmaxf(c0.x * 0.2126f + c0.y * 0.7152f + c0.z * 0.0722f, 0.0f);
  const float fullE = fmaxf(su.f(24) - su.f(25), 1.0f) / fmaxf(su.f(23) * su.f(7), 1e-9f);
  const float sn = sqrtf(Y0 * fullE + su.f(20) * su.f(20)) / fullE;
  const float rs = fmaxf(su.f(59) * sn, 1e-6f), ss = su.f(58);
  float ax = 0.0f, ay = 0.0f, az = 0.0f, ws = 0.0f;
  for (int dy = -1; dy <= 1; dy++)
    for (int dx = -1; dx <= 1; dx++) {
      const float4 c = B[size_t(clampi(y + dy, 0, H - 1)) * W + clampi(x + dx, 0, W - 1)];
      const float dY = (c.x - c0.x) * 0.2126f + (c.y - c0.y) * 0.7152f + (c.z - c0.z) * 0.0722f;
      const float w = vt_expf(-0.5f * float(dx * dx + dy * dy) / (ss * ss) - 0.5f * dY * dY / (rs * rs));
      ax = ax + w * c.x;
      ay = ay + w * c.y;
      az = az + w * c.z;
      ws = ws + w;
    }
  A[size_t(y) * W + x] = make_float4(ax / ws, ay / ws, az / ws, 1.0f);
}

__device__ __forceinline__ float srgb_oetf(float v) { return v <= 0.0031308f ? 12.92f * v : 1.055f * vt_powf(v, 0.41666666666666669f) - 0.055f; }
__device__ __forceinline__ float tone_c(const Su& su, float x) {
  const float m = su.f(44);
  if (m > 2.5f) {
    const float b = su.f(57);
    const float v = clamp01((x - b) / (1.0f - b));
    const float u = srgb_oetf(v);
    const float cc = su.f(56);
    const float a = vt_powf(u, cc);
    return a / fmaxf(a + vt_powf(1.0f - u, cc), 1e-12f);
  }
  const float c = clamp01(x);
  if (m < 0.5f) return srgb_oetf(c);
  if (m < 1.5f) return vt_powf(c, 1.0f / fmaxf(su.f(45), 1e-3f));
  return c;
}
__device__ __forceinline__ float3 toned(const Su& su, const float4* __restrict__ A, int x, int y, int W, int H) {
  const float4 c = A[size_t(clampi(y, 0, H - 1)) * W + clampi(x, 0, W - 1)];
  return make_float3(tone_c(su, c.x), tone_c(su, c.y), tone_c(su, c.z));
}
__device__ __forceinline__ float luma601(float3 c) { return c.x * 0.299f + c.y * 0.587f + c.z * 0.114f; }

// one thread per 2x2 block
__global__ void __launch_bounds__(256) isp_output_kernel(const SensorParams P, const float4* __restrict__ A, uchar4* __restrict__ out,
                                                         uint8_t* __restrict__ yuv, uint32_t* __restrict__ part) {
  const Su su{P.w};
  const int W = int(P.w[0]), H = int(P.w[1]);
  const int gx = blockIdx.x * blockDim.x + threadIdx.x, gy = blockIdx.y * blockDim.y + threadIdx.y;
  const int bx = gx * 2, by = gy * 2;
  uint32_t lsum = 0;
  if (bx < W && by < H) {
    float Ys[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    float cb = 0.0f, cr = 0.0f, nb = 0.0f;
    const float amt = su.f(46);
    const int rad = clampi(int(rintf(su.f(47))), 1, 4);
    const bool c420 = P.w[48] != 0u;
    for (int q = 0; q < 4; q++) {
      const int x = bx + (q & 1), y = by + (q >> 1);
      if (x >= W || y >= H) continue;
      float3 c = toned(su, A, x, y, W, H);
      if (amt > 0.0f) {
        float m = 0.0f, n = 0.0f;
        for (int dy = -rad; dy <= rad; dy++)
          for (int dx = -rad; dx <= rad; dx++) {
            m = m + luma601(toned(su, A, x + dx, y + dy, W, H));
            n = n + 1.0f;
          }
        const float s = amt * (luma601(c) - m / n);
        c = make_float3(c.x + s, c.y + s, c.z + s);
      }
      const float r8 = clamp01(c.x) * 255.0f, g8 = clamp01(c.y) * 255.0f, b8 = clamp01(c.z) * 255.0f;
      Ys[q] = 0.299f * r8 + 0.587f * g8 + 0.114f * b8;
      cb = cb + (128.0f - 0.168736f * r8 - 0.331264f * g8 + 0.5f * b8);
      cr = cr + (128.0f + 0.5f * r8 - 0.418688f * g8 - 0.081312f * b8);
      nb = nb + 1.0f;
      if (!c420) {
        const float y8 = fminf(fmaxf(rintf(Ys[q]), 0.0f), 255.0f);
        out[size_t(y) * W + x] = make_uchar4(uint8_t(rintf(r8)), uint8_t(rintf(g8)), uint8_t(rintf(b8)), 255);
        lsum += uint32_t(y8);
      }
    }
    if (c420) {
      const float Cb = fminf(fmaxf(rintf(cb / nb), 0.0f), 255.0f), Cr = fminf(fmaxf(rintf(cr / nb), 0.0f), 255.0f);
      const int cw = (W + 1) / 2, chh = (H + 1) / 2;
      for (int q = 0; q < 4; q++) {
        const int x = bx + (q & 1), y = by + (q >> 1);
        if (x >= W || y >= H) continue;
        const float y8 = fminf(fmaxf(rintf(Ys[q]), 0.0f), 255.0f);
        const float r = y8 + 1.402f * (Cr - 128.0f);
        const float g = y8 - 0.344136f * (Cb - 128.0f) - 0.714136f * (Cr - 128.0f);
        const float b = y8 + 1.772f * (Cb - 128.0f);
        out[size_t(y) * W + x] = make_uchar4(uint8_t(fminf(fmaxf(rintf(r), 0.0f), 255.0f)), uint8_t(fminf(fmaxf(rintf(g), 0.0f), 255.0f)),
                                             uint8_t(fminf(fmaxf(rintf(b), 0.0f), 255.0f)), 255);
        yuv[size_t(y) * W + x] = uint8_t(y8);
        lsum += uint32_t(y8);
      }
      yuv[size_t(W) * H + size_t(gy) * cw + gx] = uint8_t(Cb);
      yuv[size_t(W) * H + size_t(cw) * chh + size_t(gy) * cw + gx] = uint8_t(Cr);
    }
  }
  const uint32_t v[3] = {lsum, 0u, 0u};
  block_sum3(v, part + 3 * size_t(blockIdx.y * gridDim.x + blockIdx.x));
}

// stats[k] = the sum of the blocks' partials of statistic k (n blocks, 3 words each): one block, fixed order
__global__ void __launch_bounds__(1024) isp_stats_kernel(const uint32_t* __restrict__ part, uint32_t n, int k0, int k1, uint32_t* __restrict__ stats) {
  __shared__ uint32_t sm[32];
  for (int k = k0; k < k1; k++) {
    uint32_t s = 0;
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) s += part[3 * size_t(i) + (k - k0)];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31u) == 0) sm[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
      uint32_t t = 0;
      for (int w = 0; w < int(blockDim.x) / 32; w++) t += sm[w];
      stats[k] = t;
    }
    __syncthreads();
  }
}

static float host_float(uint32_t u) {
  float f;
  std::memcpy(&f, &u, 4);
  return f;
}

void launch_isp(const SensorParams& P, const IspBufs& b, cudaStream_t st) {
  const uint32_t W = P.w[0], H = P.w[1];
  const dim3 blk(32, 8), g((W + 31) / 32, (H + 7) / 8);
  isp_optics_kernel<<<g, blk, 0, st>>>(P, b.L, b.ri, b.A);
  const float k = host_float(P.w[52]);
  if (k > 0.0f) {
    const int F = int(host_float(P.w[54]));
    const int gw = (int(W) + F - 1) / F, gh = (int(H) + F - 1) / F;
    const dim3 gg((gw + 31) / 32, (gh + 7) / 8);
    glare_down_kernel<<<gg, blk, 0, st>>>(P, b.L, b.ri, b.GA);
    glare_blur_kernel<<<gg, blk, 0, st>>>(P, b.GA, b.GB, 0);
    glare_blur_kernel<<<gg, blk, 0, st>>>(P, b.GB, b.GA, 1);
  }
  isp_expose_kernel<<<g, blk, 0, st>>>(P, b.A, b.GA, b.raw);
  demosaic_g_kernel<<<g, blk, 0, st>>>(P, b.raw, b.gpl);
  demosaic_rb_kernel<<<g, blk, 0, st>>>(P, b.raw, b.gpl, b.B, b.part);
  isp_stats_kernel<<<1, 1024, 0, st>>>(b.part, g.x * g.y, 1, 4, b.stats);
  // noise reduction off: the output stage reads the demosaiced image directly (the kernel would copy it)
  const bool nr = P.w[51] != 0u && host_float(P.w[58]) > 0.0f;
  if (nr) isp_nr_kernel<<<g, blk, 0, st>>>(P, b.B, b.A);
  const uint32_t cw = (W + 1) / 2, ch = (H + 1) / 2;
  const dim3 go((cw + 31) / 32, (ch + 7) / 8);
  isp_output_kernel<<<go, blk, 0, st>>>(P, nr ? b.A : b.B, b.out, b.yuv, b.part);
  isp_stats_kernel<<<1, 1024, 0, st>>>(b.part, go.x * go.y, 0, 1, b.stats);
}

// ------------------------------------------------------------------------------------- the raster pass's display
// lite_nodes/renderer.js:369 DISPLAY (the lite renderer's sensor look): scaled luma of every 4th pixel in x and y
// summed for the next frame's exposure; exposure gain, the KB4 cameras' cos-like falloff, veiling glare as the
// previous frame's global mean, white balance, sRGB and S-curve into rgba8. The sums are per-warp reductions added
// once per warp: integer, so independent of the order.
__global__ void __launch_bounds__(256) lite_display_kernel(const LiteDisplay P, const float4* __restrict__ L, uchar4* __restrict__ out,
                                                           uint32_t* __restrict__ stats) {
  const uint32_t x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
  uint32_t sy = 0, cnt = 0;
  if (x < P.W && y < P.H) {
    const float4 l = L[size_t(y) * P.W + x];
    if ((x & 3u) == 0u && (y & 3u) == 0u) {
      const float yl = l.x * 0.2126f + l.y * 0.7152f + l.z * 0.0722f;
      sy = __float2uint_rz(fminf(fmaxf(yl * P.du[3], 0.0f), 65535.0f));
      cnt = 1;
    }
    const float n = fmaxf(float(P.prev[1]), 1.0f);
    const float mean = float(P.prev[0]) / fmaxf(P.du[3], 1e-30f) / n;
    float E[3] = {l.x, l.y, l.z};
    if (P.du[12] > 0.0f) {
      const float qx = (float(x) + 0.5f - P.du[14]) / P.du[12], qy = (float(y) + 0.5f - P.du[15]) / P.du[13];
      const float c = clamp01(sqrtf(qx * qx + qy * qy) / 1.1f);
      const float t = c * c;
      const float f = 1.0f * (1.0f - t) + 0.57f * t;
      for (int k = 0; k < 3; k++) E[k] = E[k] * f;
    }
    const float g = P.du[1], b = P.du[9], sc = P.du[8];
    uint8_t o[3];
    for (int k = 0; k < 3; k++) {
      const float e = (1.0f - g) * E[k] + g * mean;
      const float xv = e * P.du[0] * P.du[4 + k];
      const float v = clamp01((xv - b) / (1.0f - b));
      float t = srgb_oetf(v);
      if (sc > 0.0f) {
        const float a = vt_powf(clamp01(t), sc);
        t = a / (a + vt_powf(clamp01(1.0f - t), sc));
      }
      o[k] = uint8_t(__float2uint_rn(t * 255.0f));
    }
    out[size_t(y) * P.W + x] = make_uchar4(o[0], o[1], o[2], 255);
  }
  sy = __reduce_add_sync(0xffffffffu, sy);
  cnt = __reduce_add_sync(0xffffffffu, cnt);
  if (threadIdx.x == 0 && cnt) {
    atomicAdd(stats, sy);
    atomicAdd(stats + 1, cnt);
  }
}

void launch_lite_display(const LiteDisplay& P, const float4* L, uchar4* out, uint32_t* stats, cudaStream_t st) {
  cudaMemsetAsync(stats, 0, 16, st);
  const dim3 blk(32, 8), g((P.W + 31) / 32, (P.H + 7) / 8);
  lite_display_kernel<<<g, blk, 0, st>>>(P, L, out, stats);
}

}  // namespace vtk
