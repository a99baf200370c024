// The camera sensor chain after the path tracer, radiance -> raw DN -> 8-bit RGB and YCbCr (gpu/wgsl/sensor.wgsl.js),
// in three fused passes over the frame (plus three small ones on the glare level when veiling glare is on):
//   glare_down/blur   veiling glare on a 1/F level: box mean, then a Gaussian over whole rows and columns (zero outside)
//   isp_expose        E = L (pi T / 4 N^2) RI with the pixel-integrated Gaussian optics blur (the horizontal half into
//                     shared rows with the vertical half's halo, then the vertical half), the glare mix
//                     E' = (1 - k) E + k G and the sensor model (vt_sensor.cuh): raw DN
//   isp_demosaic      a raw tile with a 3-pixel halo in shared memory; the green plane (bilinear, edge-aware or
//                     Hamilton-Adams) on the tile and a 1-pixel ring; red and blue (colour differences or bilinear),
//                     black level, white-balance statistics, WB, CCM
//   isp_finish        3x3 bilateral noise reduction on linear RGB (range sigma from the modelled shot + read noise) and
//                     the output stage on each 2x2 block: tone curve, BT.601 full-range YCbCr, 4:2:0 chroma, 8-bit RGB,
//                     luma sum. With sharpening on (an unsharp mask over toned luma, radius up to 4) noise reduction
//                     and output run as two passes (isp_nr, isp_output), since the mask reads the reduced image's
//                     neighbours.
// The statistics are integer sums: each block adds its partial with one atomic per word, exact in any order. The
// exposure pass clears them.
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

// a block's sums of v[0..n-1] added to stats[0..n-1] with one atomic each (integer: exact in any order)
__device__ __forceinline__ void block_add(const uint32_t* v, int n, uint32_t* stats) {
  __shared__ uint32_t sm[8][3];
  const int t = threadIdx.y * blockDim.x + threadIdx.x, lane = t & 31, warp = t >> 5;
  uint32_t a[3] = {v[0], n > 1 ? v[1] : 0u, n > 2 ? v[2] : 0u};
  for (int k = 0; k < n; k++)
    for (int s = 16; s > 0; s >>= 1) a[k] += __shfl_xor_sync(0xffffffffu, a[k], s);
  if (lane == 0)
    for (int k = 0; k < n; k++) sm[warp][k] = a[k];
  __syncthreads();
  if (t < n) {
    uint32_t s = 0;
    for (int w = 0; w < int(blockDim.x * blockDim.y) / 32; w++) s += sm[w][t];
    if (s) atomicAdd(stats + t, s);
  }
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

// the exposure pass's blocks: 32 columns x ty output rows (ty <= EX_MAX; 32 x 8 threads, a thread takes every 8th
// row) and the shared rows they need with the vertical blur's halo (at most 12 taps each side)
constexpr int EX_MAX = 40;
constexpr int EX_ROWS = EX_MAX + 24;

__global__ void __launch_bounds__(256) isp_expose_kernel(const SensorParams P, const float4* __restrict__ L, const float* __restrict__ ri,
                                                         const float4* __restrict__ G, float* __restrict__ raw, uint32_t* __restrict__ stats,
                                                         int ty_rows) {
  __shared__ float taps[25];
  __shared__ float hx[EX_ROWS][32], hy[EX_ROWS][32], hz[EX_ROWS][32];
  const Su su{P.w};
  const int W = int(P.w[0]), H = int(P.w[1]);
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int x = blockIdx.x * 32 + tx, y0 = blockIdx.y * ty_rows;
  if (blockIdx.x == 0 && blockIdx.y == 0 && ty == 0 && tx < 4) stats[tx] = 0u;
  const float sg = su.f(5);
  const int r = gauss_taps(sg);
  block_taps(sg, r, taps);
  // the horizontal half on shared row j = image row clamp(y0 - r + j): the vertical half's tap k of output row y0 + i
  // is row i + k + r, the clamped row y0 + i + k as the separable blur has it
  const int rows = min(ty_rows, H - y0) + 2 * r;
  if (x < W) {
    for (int j = ty; j < rows; j += 8) {
      const int yy = clampi(y0 - r + j, 0, H - 1);
      float ax = 0.0f, ay = 0.0f, az = 0.0f, ws = 0.0f;
      for (int k = -r; k <= r; k++) {
        const int xx = clampi(x + k, 0, W - 1);
        const float w = taps[k + r];
        const float4 l = __ldg(L + size_t(yy) * W + xx);
        const float m = __ldg(ri + size_t(yy) * W + xx);
        ax = ax + w * l.x * m;
        ay = ay + w * l.y * m;
        az = az + w * l.z * m;
        ws = ws + w;
      }
      const float s = su.f(4) / ws;
      hx[j][tx] = ax * s;
      hy[j][tx] = ay * s;
      hz[j][tx] = az * s;
    }
  }
  __syncthreads();
  if (x >= W) return;
  const float kg = su.f(52);
  for (int i = ty; i < ty_rows; i += 8) {
    const int y = y0 + i;
    if (y >= H) break;
    float ex = 0.0f, ey = 0.0f, ez = 0.0f, ws = 0.0f;
    for (int k = -r; k <= r; k++) {
      const float w = taps[k + r];
      const int j = i + k + r;
      ex = ex + w * hx[j][tx];
      ey = ey + w * hy[j][tx];
      ez = ez + w * hz[j][tx];
      ws = ws + w;
    }
    ex = ex / ws; ey = ey / ws; ez = ez / ws;
    if (kg > 0.0f) {
      const float3 g = glare_at(su, G, x, y, W, H);
      ex = (1.0f - kg) * ex + kg * g.x;
      ey = (1.0f - kg) * ey + kg * g.y;
      ez = (1.0f - kg) * ez + kg * g.z;
    }
    raw[size_t(y) * W + x] = sensor_dn(P.w, ex, ey, ez, x, y, W, P.w[3]);
  }
}

// raw DN mirrored at the borders (reflect by one, which keeps the CFA phase), then clamped
__device__ __forceinline__ float raw_at(const float* __restrict__ raw, int x, int y, int W, int H) {
  if (x < 0) x = -x;
  if (x >= W) x = 2 * (W - 1) - x;
  if (y < 0) y = -y;
  if (y >= H) y = 2 * (H - 1) - y;
  return raw[size_t(clampi(y, 0, H - 1)) * W + clampi(x, 0, W - 1)];
}

// the green value at (x, y) of the image, with rw(xx, yy) = raw_at(raw, xx, yy) for |xx - x|, |yy - y| <= 2
template <class Raw>
__device__ __forceinline__ float green_at(const Su& su, uint32_t code, uint32_t mode, Raw&& rw, int x, int y) {
  float g = rw(x, y);
  if (cfa_channel(code, uint32_t(x), uint32_t(y)) != 1u) {
    const float gl = rw(x - 1, y), gr = rw(x + 1, y);
    const float gu = rw(x, y - 1), gd = rw(x, y + 1);
    if (mode == 0) {
      g = 0.25f * (gl + gr + gu + gd);
    } else if (mode == 1) {
      const float dh = fabsf(gl - gr), dv = fabsf(gu - gd);
      g = dh < dv ? 0.5f * (gl + gr) : dv < dh ? 0.5f * (gu + gd) : 0.25f * (gl + gr + gu + gd);
    } else {
      const float c = g;
      const float lh = 2.0f * c - rw(x - 2, y) - rw(x + 2, y);
      const float lv = 2.0f * c - rw(x, y - 2) - rw(x, y + 2);
      const float dh = fabsf(gl - gr) + fabsf(lh), dv = fabsf(gu - gd) + fabsf(lv);
      const float gh = 0.5f * (gl + gr) + 0.25f * lh, gv = 0.5f * (gu + gd) + 0.25f * lv;
      g = dh < dv ? gh : dv < dh ? gv : 0.5f * (gh + gv);
      g = fminf(fmaxf(g, 0.0f), su.f(24));
    }
  }
  return g;
}

// the demosaic pass's tile: 64 pixels x 2 tq rows per block of 32 x 8 threads (tq <= QR_MAX quad rows), one 2x2
// quad per thread and quad row
constexpr int DM_TX = 64, QR_MAX = 16;

// the 2x2 CFA pattern words of cfa_channel: RGGB, GRBG, GBRG, BGGR
constexpr uint32_t CFA_PATS[4] = {0x2110u, 0x1201u, 0x1021u, 0x0112u};
__host__ __device__ constexpr uint32_t pat_channel(uint32_t pats, int x, int y) { return (pats >> (4u * (uint32_t(y & 1) * 2u + uint32_t(x & 1)))) & 0xfu; }

// black level, white-balance statistics (added to q), WB and CCM of one demosaiced pixel
__device__ __forceinline__ float4 rb_finish(const Su& su, float r, float gg, float b, uint32_t q[3]) {
  const float black = su.f(25), full = fmaxf(su.f(24) - black, 1.0f);
  float c[3] = {(r - black) / full, (gg - black) / full, (b - black) / full};
  for (int k = 0; k < 3; k++) q[k] += uint32_t(rintf(clamp01(c[k]) * 1023.0f));
  for (int k = 0; k < 3; k++) c[k] = c[k] * su.f(28 + k);
  float o[3];
  for (int k = 0; k < 3; k++) o[k] = su.f(32 + 4 * k) * c[0] + su.f(33 + 4 * k) * c[1] + su.f(34 + 4 * k) * c[2];
  return make_float4(o[0], o[1], o[2], 1.0f);
}

// red and blue of image pixel (x, y) anywhere in the frame (neighbours clamped): rw / g_at give the raw and green
// values of image pixels within one of it
template <class Raw, class Green>
__device__ __forceinline__ void rb_general(uint32_t code, uint32_t mode, Raw&& rw, Green&& g_at, int x, int y, int W, int H,
                                           float& r, float& gg, float& b) {
  const uint32_t own = cfa_channel(code, uint32_t(x), uint32_t(y));
  const float g = g_at(x, y);
  float sr = 0.0f, sb = 0.0f, cr = 0.0f, cb = 0.0f;
  for (int dy = -1; dy <= 1; dy++)
    for (int dx = -1; dx <= 1; dx++) {
      const int xx = clampi(x + dx, 0, W - 1), yy = clampi(y + dy, 0, H - 1);
      const uint32_t ch = cfa_channel(code, uint32_t(xx), uint32_t(yy));
      if (ch == 1u) continue;
      if (ch == own && !(dx == 0 && dy == 0)) continue;
      const float d = rw(xx, yy) - g_at(xx, yy);
      if (ch == 0u) { sr = sr + d; cr = cr + 1.0f; } else { sb = sb + d; cb = cb + 1.0f; }
    }
  r = g + sr / fmaxf(cr, 1.0f); gg = g; b = g + sb / fmaxf(cb, 1.0f);
  if (mode <= 1u) {
    float s0 = 0.0f, s1 = 0.0f, s2 = 0.0f, c0 = 0.0f, c1 = 0.0f, c2 = 0.0f;
    for (int dy = -1; dy <= 1; dy++)
      for (int dx = -1; dx <= 1; dx++) {
        const int xx = clampi(x + dx, 0, W - 1), yy = clampi(y + dy, 0, H - 1);
        const uint32_t ch = cfa_channel(code, uint32_t(xx), uint32_t(yy));
        if (ch == own && !(dx == 0 && dy == 0)) continue;
        if (ch == 1u && own == 1u && !(dx == 0 && dy == 0)) continue;
        const float v = rw(xx, yy);
        if (ch == 0u) { s0 = s0 + v; c0 = c0 + 1.0f; } else if (ch == 1u) { s1 = s1 + v; c1 = c1 + 1.0f; } else { s2 = s2 + v; c2 = c2 + 1.0f; }
      }
    r = s0 / fmaxf(c0, 1.0f);
    gg = s1 / fmaxf(c1, 1.0f);
    b = s2 / fmaxf(c2, 1.0f);
    if (mode == 1u) gg = g;
  }
}

// rb_general for a pixel whose 3x3 neighbourhood lies inside the frame, at CFA phase (PX, PY) of pattern PATS: the
// same taps in the same order, with every channel test and count known at compile time (counts 1, 2 or 4, so each
// quotient is a product by 1, 1/2 or 1/4, exactly as the division gives it); rw / g_at take offsets from the pixel
template <uint32_t PATS, int PX, int PY, class Raw, class Green>
__device__ __forceinline__ void rb_inner(uint32_t mode, Raw&& rw, Green&& g_at, float& r, float& gg, float& b) {
  constexpr uint32_t own = pat_channel(PATS, PX, PY);
  const float g = g_at(0, 0);
  float sr = 0.0f, sb = 0.0f, cr = 0.0f, cb = 0.0f;
#pragma unroll
  for (int dy = -1; dy <= 1; dy++)
#pragma unroll
    for (int dx = -1; dx <= 1; dx++) {
      const uint32_t ch = pat_channel(PATS, PX + dx, PY + dy);
      if (ch == 1u) continue;
      if (ch == own && !(dx == 0 && dy == 0)) continue;
      const float d = rw(dx, dy) - g_at(dx, dy);
      if (ch == 0u) { sr = sr + d; cr = cr + 1.0f; } else { sb = sb + d; cb = cb + 1.0f; }
    }
  r = g + sr / fmaxf(cr, 1.0f); gg = g; b = g + sb / fmaxf(cb, 1.0f);
  if (mode <= 1u) {
    float s0 = 0.0f, s1 = 0.0f, s2 = 0.0f, c0 = 0.0f, c1 = 0.0f, c2 = 0.0f;
#pragma unroll
    for (int dy = -1; dy <= 1; dy++)
#pragma unroll
      for (int dx = -1; dx <= 1; dx++) {
        const uint32_t ch = pat_channel(PATS, PX + dx, PY + dy);
        if (ch == own && !(dx == 0 && dy == 0)) continue;
        if (ch == 1u && own == 1u && !(dx == 0 && dy == 0)) continue;
        const float v = rw(dx, dy);
        if (ch == 0u) { s0 = s0 + v; c0 = c0 + 1.0f; } else if (ch == 1u) { s1 = s1 + v; c1 = c1 + 1.0f; } else { s2 = s2 + v; c2 = c2 + 1.0f; }
      }
    r = s0 / fmaxf(c0, 1.0f);
    gg = s1 / fmaxf(c1, 1.0f);
    b = s2 / fmaxf(c2, 1.0f);
    if (mode == 1u) gg = g;
  }
}

// CODE: the CFA pattern index as cfa_channel reads the uniform's code (0 RGGB, 1 GRBG, 2 GBRG, 3 and above BGGR)
template <int CODE>
__global__ void __launch_bounds__(256) isp_demosaic_kernel(const SensorParams P, const float* __restrict__ raw, float4* __restrict__ B,
                                                           uint32_t* __restrict__ stats, int tq) {
  constexpr uint32_t PATS = CFA_PATS[CODE];
  // rs[j][i] = raw_at(x0 - 3 + i, y0 - 3 + j); gs[j][i] = the green plane at the image pixel clamp(x0 - 1 + i, y0 - 1 + j)
  __shared__ float rs[2 * QR_MAX + 6][DM_TX + 6];
  __shared__ float gs[2 * QR_MAX + 2][DM_TX + 2];
  const Su su{P.w};
  const int W = int(P.w[0]), H = int(P.w[1]);
  const int x0 = blockIdx.x * DM_TX, y0 = blockIdx.y * 2 * tq;
  const int t = threadIdx.y * 32 + threadIdx.x;
  constexpr int RW = DM_TX + 6, GW = DM_TX + 2;
  for (int e = t; e < (2 * tq + 6) * RW; e += 256) rs[e / RW][e % RW] = raw_at(raw, x0 - 3 + e % RW, y0 - 3 + e / RW, W, H);
  __syncthreads();
  const uint32_t code = P.w[2], mode = P.w[50];
  auto rw = [&](int xx, int yy) { return rs[yy - y0 + 3][xx - x0 + 3]; };
  for (int e = t; e < (2 * tq + 2) * GW; e += 256) {
    const int px = clampi(x0 - 1 + e % GW, 0, W - 1), py = clampi(y0 - 1 + e / GW, 0, H - 1);
    gs[e / GW][e % GW] = green_at(su, code, mode, rw, px, py);
  }
  __syncthreads();
  auto g_at = [&](int xx, int yy) { return gs[yy - y0 + 1][xx - x0 + 1]; };
  uint32_t q[3] = {0u, 0u, 0u};
  for (int qr = int(threadIdx.y); qr < tq; qr += 8) {
  const int qx = x0 + 2 * int(threadIdx.x), qy = y0 + 2 * qr;
  if (qx >= 2 && qx + 3 <= W && qy >= 2 && qy + 3 <= H) {
    // the quad's 4 x 4 neighbourhood lies inside the frame: tile offsets of pixel (qx, qy)
    const int ri = qx - x0 + 3, rj = qy - y0 + 3, gi = qx - x0 + 1, gj = qy - y0 + 1;
    float r, gg, b;
    float4* o = B + size_t(qy) * W + qx;
#define VT_QUAD_PIXEL(PX, PY)                                                                                        \
    {                                                                                                                \
      auto rwq = [&](int dx, int dy) { return rs[rj + PY + dy][ri + PX + dx]; };                                     \
      auto gq = [&](int dx, int dy) { return gs[gj + PY + dy][gi + PX + dx]; };                                      \
      rb_inner<PATS, PX, PY>(mode, rwq, gq, r, gg, b);                                                               \
      o[size_t(PY) * W + PX] = rb_finish(su, r, gg, b, q);                                                           \
    }
    VT_QUAD_PIXEL(0, 0)
    VT_QUAD_PIXEL(1, 0)
    VT_QUAD_PIXEL(0, 1)
    VT_QUAD_PIXEL(1, 1)
#undef VT_QUAD_PIXEL
  } else {
    for (int k = 0; k < 4; k++) {
      const int x = qx + (k & 1), y = qy + (k >> 1);
      if (x >= W || y >= H) continue;
      float r, gg, b;
      rb_general(code, mode, rw, g_at, x, y, W, H, r, gg, b);
      B[size_t(y) * W + x] = rb_finish(su, r, gg, b, q);
    }
  }
  }
  // white-balance statistics R, G, B
  block_add(q, 3, stats + 1);
}

// the noise-reduced pixel (x, y) of the image, with b(xx, yy) = the demosaiced pixel at the clamped (xx, yy)
template <class Fetch>
__device__ __forceinline__ float4 nr_pixel(const Su& su, const uint32_t* w, Fetch&& b, int x, int y) {
  const float4 c0 = b(x, y);
  if (w[51] == 0u || su.f(58) <= 0.0f) return c0;
  const float Y0 = fmaxf(c0.x * 0.2126f + c0.y * 0.7152f + c0.z * 0.0722f, 0.0f);
  const float fullE = fmaxf(su.f(24) - su.f(25), 1.0f) / fmaxf(su.f(23) * su.f(7), 1e-9f);
  const float sn = sqrtf(Y0 * fullE + su.f(20) * su.f(20)) / fullE;
  const float rs = fmaxf(su.f(59) * sn, 1e-6f), ss = su.f(58);
  float ax = 0.0f, ay = 0.0f, az = 0.0f, ws = 0.0f;
  for (int dy = -1; dy <= 1; dy++)
    for (int dx = -1; dx <= 1; dx++) {
      const float4 c = b(x + dx, y + dy);
      const float dY = (c.x - c0.x) * 0.2126f + (c.y - c0.y) * 0.7152f + (c.z - c0.z) * 0.0722f;
      // the centre tap's exponent is exactly zero for a finite pixel (the demosaiced image is finite): weight 1
      const float wt = dx == 0 && dy == 0 ? 1.0f : vt_expf(-0.5f * float(dx * dx + dy * dy) / (ss * ss) - 0.5f * dY * dY / (rs * rs));
      ax = ax + wt * c.x;
      ay = ay + wt * c.y;
      az = az + wt * c.z;
      ws = ws + wt;
    }
  return make_float4(ax / ws, ay / ws, az / ws, 1.0f);
}

__global__ void isp_nr_kernel(const SensorParams P, const float4* __restrict__ B, float4* __restrict__ A) {
  const Su su{P.w};
  const int W = int(P.w[0]), H = int(P.w[1]);
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= W || y >= H) return;
  auto b = [&](int xx, int yy) { return B[size_t(clampi(yy, 0, H - 1)) * W + clampi(xx, 0, W - 1)]; };
  A[size_t(y) * W + x] = nr_pixel(su, P.w, b, x, y);
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
__device__ __forceinline__ float3 toned(const Su& su, float4 c) {
  return make_float3(tone_c(su, c.x), tone_c(su, c.y), tone_c(su, c.z));
}
__device__ __forceinline__ float luma601(float3 c) { return c.x * 0.299f + c.y * 0.587f + c.z * 0.114f; }

// the output stage of the 2x2 block (gx, gy): at(x, y) = the linear pixel at the clamped (x, y) (read at the block's
// pixels, and with SHARPEN at their neighbours within the mask's radius); returns the block's luma sum
template <bool SHARPEN, class Fetch>
__device__ __forceinline__ uint32_t output_block(const Su& su, const uint32_t* w, Fetch&& at, int gx, int gy, int W, int H,
                                                 uchar4* __restrict__ out, uint8_t* __restrict__ yuv) {
  const int bx = gx * 2, by = gy * 2;
  uint32_t lsum = 0;
  float Ys[4] = {0.0f, 0.0f, 0.0f, 0.0f};
  float cb = 0.0f, cr = 0.0f, nb = 0.0f;
  const bool c420 = w[48] != 0u;
  for (int q = 0; q < 4; q++) {
    const int x = bx + (q & 1), y = by + (q >> 1);
    if (x >= W || y >= H) continue;
    float3 c = toned(su, at(x, y));
    if (SHARPEN) {
      const float amt = su.f(46);
      const int rad = clampi(int(rintf(su.f(47))), 1, 4);
      float m = 0.0f, n = 0.0f;
      for (int dy = -rad; dy <= rad; dy++)
        for (int dx = -rad; dx <= rad; dx++) {
          m = m + luma601(toned(su, at(x + dx, y + dy)));
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
  return lsum;
}

// the output stage with sharpening, on the (noise-reduced) image A: one thread per 2x2 block
__global__ void __launch_bounds__(256) isp_output_kernel(const SensorParams P, const float4* __restrict__ A, uchar4* __restrict__ out,
                                                         uint8_t* __restrict__ yuv, uint32_t* __restrict__ stats) {
  const Su su{P.w};
  const int W = int(P.w[0]), H = int(P.w[1]);
  const int gx = blockIdx.x * blockDim.x + threadIdx.x, gy = blockIdx.y * blockDim.y + threadIdx.y;
  uint32_t lsum = 0;
  if (gx * 2 < W && gy * 2 < H) {
    auto at = [&](int xx, int yy) { return A[size_t(clampi(yy, 0, H - 1)) * W + clampi(xx, 0, W - 1)]; };
    lsum = output_block<true>(su, P.w, at, gx, gy, W, H, out, yuv);
  }
  block_add(&lsum, 1, stats);
}

// noise reduction and the output stage without sharpening: one thread per 2x2 block, the block's 64 x 2 tq pixels
// (tq <= QR_MAX quad rows; a thread takes every 8th quad row) of the demosaiced image with a
// 1-pixel ring in shared memory (bs[j][i] = B at the clamped (x0 - 1 + i, y0 - 1 + j))
__global__ void __launch_bounds__(256) isp_finish_kernel(const SensorParams P, const float4* __restrict__ B, uchar4* __restrict__ out,
                                                         uint8_t* __restrict__ yuv, uint32_t* __restrict__ stats, int tq) {
  __shared__ float4 bs[2 * QR_MAX + 2][66];
  const Su su{P.w};
  const int W = int(P.w[0]), H = int(P.w[1]);
  const int x0 = blockIdx.x * 64, y0 = blockIdx.y * 2 * tq;
  const int t = threadIdx.y * 32 + threadIdx.x;
  for (int e = t; e < (2 * tq + 2) * 66; e += 256)
    bs[e / 66][e % 66] = B[size_t(clampi(y0 - 1 + e / 66, 0, H - 1)) * W + clampi(x0 - 1 + e % 66, 0, W - 1)];
  __syncthreads();
  // the ring holds the clamped neighbours of the block's pixels, so the offsets index it directly
  auto b = [&](int xx, int yy) { return bs[yy - y0 + 1][xx - x0 + 1]; };
  auto at = [&](int xx, int yy) { return nr_pixel(su, P.w, b, xx, yy); };
  const int gx = blockIdx.x * 32 + threadIdx.x;
  uint32_t lsum = 0;
  for (int qr = int(threadIdx.y); qr < tq; qr += 8) {
    const int gy = blockIdx.y * tq + qr;
    if (gx * 2 < W && gy * 2 < H) lsum += output_block<false>(su, P.w, at, gx, gy, W, H, out, yuv);
  }
  block_add(&lsum, 1, stats);
}

static float host_float(uint32_t u) {
  float f;
  std::memcpy(&f, &u, 4);
  return f;
}

// block heights: 24 output rows for the exposure pass, 8 quad rows (16 pixel rows) for demosaic and finish. Taller
// blocks with fewer of them (one wave on 1280x720) measured no faster: the passes lose their overlap of one block's
// loads with another's arithmetic.
constexpr int EX_ROWS_PER_BLOCK = 24, QR_PER_BLOCK = 8;

int launch_isp(const SensorParams& P, const IspBufs& b, cudaStream_t st) {
  const uint32_t W = P.w[0], H = P.w[1];
  const dim3 blk(32, 8);
  int launches = 0;
  const float k = host_float(P.w[52]);
  if (k > 0.0f) {
    const int F = int(host_float(P.w[54]));
    const int gw = (int(W) + F - 1) / F, gh = (int(H) + F - 1) / F;
    const dim3 gg((gw + 31) / 32, (gh + 7) / 8);
    glare_down_kernel<<<gg, blk, 0, st>>>(P, b.L, b.ri, b.GA);
    glare_blur_kernel<<<gg, blk, 0, st>>>(P, b.GA, b.GB, 0);
    glare_blur_kernel<<<gg, blk, 0, st>>>(P, b.GB, b.GA, 1);
    launches += 3;
  }
  constexpr int ex_rows = EX_ROWS_PER_BLOCK, dm_q = QR_PER_BLOCK, fn_q = QR_PER_BLOCK;
  isp_expose_kernel<<<dim3((W + 31) / 32, (H + ex_rows - 1) / ex_rows), blk, 0, st>>>(P, b.L, b.ri, b.GA, b.raw, b.stats, ex_rows);
  const uint32_t qrows = (H + 1) / 2;
  const dim3 gd((W + DM_TX - 1) / DM_TX, (qrows + dm_q - 1) / dm_q);
  const uint32_t code = P.w[2];
  if (code == 0u) isp_demosaic_kernel<0><<<gd, blk, 0, st>>>(P, b.raw, b.B, b.stats, dm_q);
  else if (code == 1u) isp_demosaic_kernel<1><<<gd, blk, 0, st>>>(P, b.raw, b.B, b.stats, dm_q);
  else if (code == 2u) isp_demosaic_kernel<2><<<gd, blk, 0, st>>>(P, b.raw, b.B, b.stats, dm_q);
  else isp_demosaic_kernel<3><<<gd, blk, 0, st>>>(P, b.raw, b.B, b.stats, dm_q);
  launches += 2;
  const uint32_t cw = (W + 1) / 2, ch = (H + 1) / 2;
  if (host_float(P.w[46]) > 0.0f) {   // sharpening: the mask reads the reduced image's neighbours
    const dim3 go((cw + 31) / 32, (ch + 7) / 8);
    const bool nr = P.w[51] != 0u && host_float(P.w[58]) > 0.0f;
    if (nr) isp_nr_kernel<<<dim3((W + 31) / 32, (H + 7) / 8), blk, 0, st>>>(P, b.B, b.A);
    isp_output_kernel<<<go, blk, 0, st>>>(P, nr ? b.A : b.B, b.out, b.yuv, b.stats);
    return launches + (nr ? 2 : 1);
  }
  isp_finish_kernel<<<dim3((cw + 31) / 32, (ch + fn_q - 1) / fn_q), blk, 0, st>>>(P, b.B, b.out, b.yuv, b.stats, fn_q);
  return launches + 1;
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
