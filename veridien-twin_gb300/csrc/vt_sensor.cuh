// Per-pixel sensor arithmetic shared by the expose stage and the batched renderer's fused sensor (gpu/wgsl/sensor.wgsl.js
// :143-208): CFA site, Poisson shot noise (sequential inversion up to 64 e-, normal above), Gaussian read noise,
// full-well clip, gain, black level and ADC to raw DN.
//
// The elementary functions below are this project's own fixed-order float32 versions; every multiply-add is an
// explicit fused or separately rounded operation, so raw DN are bit-identical to any implementation that performs
// the same sequence (the CPU restatement does):
//   ln(x):      x = m 2^e with m in [sqrt(1/2), sqrt(2)); ln m = 2 atanh(s), s = (m-1)/(m+1), odd series to s^9
//   exp(x):     Cody-Waite reduction x = n ln2 + r with ln2 split hi/lo, Taylor polynomial of degree 7, times 2^n
//   cos(2 pi u): reduction in turns to [0, 1/8], Taylor series of cos (to x^10) or sin (to x^11) on [0, pi/4]
#pragma once

#include "vt_device.cuh"

namespace vtk {

__device__ __forceinline__ float vt_logf(float x) {
  const uint32_t bits = __float_as_uint(x);
  int e = int((bits >> 23) & 0xffu) - 127;
  float m = __uint_as_float((bits & 0x7fffffu) | 0x3f800000u);
  if (m > 1.41421356f) { m = __fmul_rn(m, 0.5f); e += 1; }
  const float s = __fdiv_rn(__fsub_rn(m, 1.0f), __fadd_rn(m, 1.0f));
  const float s2 = __fmul_rn(s, s);
  float p = __fmaf_rn(s2, 1.0f / 9.0f, 1.0f / 7.0f);
  p = __fmaf_rn(s2, p, 1.0f / 5.0f);
  p = __fmaf_rn(s2, p, 1.0f / 3.0f);
  p = __fmaf_rn(s2, p, 1.0f);
  const float lm = __fmul_rn(__fmul_rn(2.0f, s), p);
  return __fmaf_rn(float(e), 0.693147180559945f, lm);
}
__device__ __forceinline__ float vt_expf(float x) {
  const float n = rintf(__fmul_rn(x, 1.44269504088896f));
  float r = __fmaf_rn(-n, 0.693145751953125f, x);
  r = __fmaf_rn(-n, 1.42860682030941723e-6f, r);
  float p = __fmaf_rn(r, 1.0f / 5040.0f, 1.0f / 720.0f);
  p = __fmaf_rn(r, p, 1.0f / 120.0f);
  p = __fmaf_rn(r, p, 1.0f / 24.0f);
  p = __fmaf_rn(r, p, 1.0f / 6.0f);
  p = __fmaf_rn(r, p, 0.5f);
  p = __fmaf_rn(r, p, 1.0f);
  p = __fmaf_rn(r, p, 1.0f);
  const int ni = int(n);
  if (ni < -126) return 0.0f;
  return __fmul_rn(p, __uint_as_float(uint32_t(ni + 127) << 23));
}
__device__ __forceinline__ float vt_cos2pi(float u) {
  const float t = __fsub_rn(u, floorf(__fadd_rn(u, 0.5f)));
  float a = fabsf(t), sign = 1.0f;
  if (a > 0.25f) { a = __fsub_rn(0.5f, a); sign = -1.0f; }
  float c;
  if (a <= 0.125f) {
    const float x = __fmul_rn(a, 6.28318530717959f), x2 = __fmul_rn(x, x);
    float p = __fmaf_rn(x2, -1.0f / 3628800.0f, 1.0f / 40320.0f);
    p = __fmaf_rn(x2, p, -1.0f / 720.0f);
    p = __fmaf_rn(x2, p, 1.0f / 24.0f);
    p = __fmaf_rn(x2, p, -0.5f);
    c = __fmaf_rn(x2, p, 1.0f);
  } else {
    const float x = __fmul_rn(__fsub_rn(0.25f, a), 6.28318530717959f), x2 = __fmul_rn(x, x);
    float p = __fmaf_rn(x2, -1.0f / 39916800.0f, 1.0f / 362880.0f);
    p = __fmaf_rn(x2, p, -1.0f / 5040.0f);
    p = __fmaf_rn(x2, p, 1.0f / 120.0f);
    p = __fmaf_rn(x2, p, -1.0f / 6.0f);
    c = __fmaf_rn(__fmul_rn(x, x2), p, x);
  }
  return sign * c;
}
__device__ __forceinline__ float uS(uint32_t x) { return __fmul_rn(__fadd_rn(float(x >> 8u), 0.5f), 1.0f / 16777216.0f); }
// erf by Abramowitz-Stegun 7.1.26 (gpu/wgsl/sensor.wgsl.js:57)
__device__ __forceinline__ float erfA(float z) {
  const float t = __fdiv_rn(1.0f, __fadd_rn(1.0f, __fmul_rn(0.3275911f, fabsf(z))));
  float p = __fmaf_rn(1.061405429f, t, -1.453152027f);
  p = __fmaf_rn(p, t, 1.421413741f);
  p = __fmaf_rn(p, t, -0.284496736f);
  p = __fmaf_rn(p, t, 0.254829592f);
  const float y = __fsub_rn(1.0f, __fmul_rn(__fmul_rn(p, t), vt_expf(__fmul_rn(-z, z))));
  return z >= 0.0f ? y : -y;
}
// weight of tap k of a pixel-integrated Gaussian (gpu/wgsl/sensor.wgsl.js:62)
__device__ __forceinline__ float tapW(int k, float sg) {
  if (sg <= 0.0f) return k == 0 ? 1.0f : 0.0f;
  const float s2 = __fmul_rn(sg, 1.41421356f);
  return __fmul_rn(0.5f, __fsub_rn(erfA(__fdiv_rn(__fadd_rn(float(k), 0.5f), s2)), erfA(__fdiv_rn(__fsub_rn(float(k), 0.5f), s2))));
}
__device__ __forceinline__ float gauss(uint32_t h) {
  const float u1 = uS(vtd::pcg(h)), u2 = uS(vtd::pcg(h ^ 0x68bc21ebu));
  return __fmul_rn(__fsqrt_rn(__fmul_rn(-2.0f, vt_logf(u1))), vt_cos2pi(u2));
}
// Poisson(lam): sequential inversion (at most 200 steps) up to 64, normal approximation above
__device__ __forceinline__ float poisson(float lam, uint32_t h) {
  if (lam <= 0.0f) return 0.0f;
  if (lam > 64.0f) return fmaxf(0.0f, floorf(__fadd_rn(__fmaf_rn(__fsqrt_rn(lam), gauss(h), lam), 0.5f)));
  const float u = uS(vtd::pcg(h ^ 0x1b873593u));
  float p = vt_expf(-lam), F = p, k = 0.0f;
  for (int i = 0; i < 200; i++) {
    if (u <= F) break;
    k = __fadd_rn(k, 1.0f);
    p = __fdiv_rn(__fmul_rn(p, lam), k);
    F = __fadd_rn(F, p);
  }
  return k;
}

// raw DN of pixel (x, y) of a W-wide frame from its (blurred, scaled) irradiance; `frame` is the uniform's frame word
__device__ __forceinline__ float sensor_dn(const uint32_t* w, float ex, float ey, float ez, int x, int y, int W, uint32_t frame) {
  const float* f = reinterpret_cast<const float*>(w);
  // 2x2 CFA codes RGGB, GRBG, GBRG, BGGR (0 R, 1 G, 2 B), gpu/wgsl/sensor.wgsl.js:143
  const uint32_t pats = (w[2] & 3u) == 0 ? 0x2110u : (w[2] & 3u) == 1 ? 0x1201u : (w[2] & 3u) == 2 ? 0x1021u : 0x0112u;
  const uint32_t ch = (pats >> (4u * ((uint32_t(y) & 1u) * 2u + (uint32_t(x) & 1u)))) & 0xfu;
  const float* row = f + 8 + 4 * ch;
  const float texp = f[6];
  const float dt = __fmaf_rn(row[2], ez, __fmaf_rn(row[1], ey, __fmul_rn(row[0], ex)));
  const float lam = __fmaf_rn(fmaxf(0.0f, dt), texp, __fmul_rn(f[22], texp));
  const uint32_t h = vtd::pcg((uint32_t(y * W + x) * 0x9E3779B9u) ^ vtd::pcg((frame * 0x85ebca6bu) ^ vtd::pcg(w[26] ^ (w[49] * 0xc2b2ae35u))));
  float e = lam;
  if (f[27] > 0.5f) e = __fmaf_rn(f[20], gauss(h ^ 0x27d4eb2fu), poisson(lam, h));
  e = fminf(e, f[21]);
  const float t = __fmaf_rn(__fmul_rn(e, f[23]), f[7], f[25]);
  const float dn = floorf(__fadd_rn(t, 0.5f));
  return fminf(fmaxf(dn, 0.0f), f[24]);
}

}  // namespace vtk
