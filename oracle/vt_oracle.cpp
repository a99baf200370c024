// ORACLE - test infrastructure only. A CPU restatement of the veridien twin's rendering hot path, used by tests/,
// by __graft_entry__.smoke() and by bench.py's CPU-baseline leg as the checker. Nothing in the product links,
// calls or ships this file.
//
// PARITY UNPINNED: the reference is JavaScript + WGSL. Neither runs on this machine or the GPU machine (no node, no
// WebGPU), and the reference carries no golden vectors for this path (its hot-path tests are not in the tree).
// This restatement is anchored instead on the reference's own stated known answers: brute force checks the BVH
// (gpu/bvh.js:3, :253), the KB4 round trip (gpu/lens.js:43-62), the Gauss-Legendre disc irradiance
// (gpu/shade_ref.js:40-62), fresnelAverage by Simpson (gpu/bsdf.js:34-42), the furnace test and the direct FP64
// linear solve of the radiosity.
//
// Every function cites the reference file:line it restates. Real arithmetic is templated: R = double is the FP64
// oracle (the JS modules' float64 semantics); R = float is the FP32 WGSL-order restatement (also the timed CPU
// baseline). Sample numbers (PCG hashes, Kronecker sequences, sub-pixel positions, shutter times) are generated in
// float32 exactly as the WGSL does in both modes, so the FP64 oracle prices the GPU's own samples.
#include "../include/vtwin.h"

#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <thread>
#include <vector>

namespace orc {

static const double BIGD = 1e30;
static const float BIGF = 1e30f;
static const uint32_t MISS = 0xffffffffu;

static inline float as_f(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }
static inline uint32_t as_u(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }

// ============================================================================================ rng (control/rng.js)

// control/rng.js:4-13 mulberry32
struct Mulberry32 {
  uint32_t a;
  explicit Mulberry32(uint32_t s) : a(s) {}
  double next() {
    a = a + 0x6d2b79f5u;
    uint32_t t = a;
    t = (t ^ (t >> 15)) * (t | 1u);
    t ^= t + (t ^ (t >> 7)) * (t | 61u);
    return double(t ^ (t >> 14)) / 4294967296.0;
  }
};

// ============================================================================================ sampling (WGSL, f32)

// gpu/wgsl/common.wgsl.js:94-100 pcg, hash3, u01
static inline uint32_t pcg(uint32_t v) {
  uint32_t s = v * 747796405u + 2891336453u;
  uint32_t w = ((s >> ((s >> 28u) + 4u)) ^ s) * 277803737u;
  return (w >> 22u) ^ w;
}
static inline uint32_t hash3(uint32_t a, uint32_t b, uint32_t c) { return pcg(a ^ pcg(b ^ pcg(c))); }
static inline float u01(uint32_t x) { return float(x >> 8u) * (1.0f / 16777216.0f); }

// gpu/wgsl/common.wgsl.js:104-113 Kronecker constants and kr(i, a, shift) = fract(shift + f32(i) * a)
static const float R2A = 0.7548776662466927f, R2B = 0.5698402909980532f, GOLD = 0.6180339887498949f;
static const float KL0 = 0.41421356237f, KL1 = 0.73205080757f, KL2 = 0.23606797750f;
static const float KB0 = 0.64575131106f, KB1 = 0.31662479036f, KB2 = 0.60555127546f;
static inline float kr(uint32_t i, float a, float shift) {
  volatile float t = float(i) * a;   // separate roundings (no contraction), as the device code does
  float s = shift + t;
  return s - std::floor(s);
}
static inline float mixf(float a, float b, float t) { volatile float x = a * (1.0f - t); volatile float y = b * t; return x + y; }

// gpu/wgsl/kernels.wgsl.js:34-38 pixSeeds; hs is kept for the deeper-bounce dimensions of the path mode
struct PixSeeds { float s[9]; uint32_t hs; };
static inline PixSeeds pix_seeds(uint32_t x, uint32_t y, uint32_t seed, uint32_t cam) {
  PixSeeds S;
  S.hs = hash3(x, y, seed * 64u + cam);
  for (uint32_t k = 0; k < 9; k++) S.s[k] = u01(pcg(S.hs + k));
  return S;
}
// Path-mode extension (beyond the reference's depth 2): bounce b >= 2 draws its light (k = 0..2) and BSDF (k = 3..5)
// Kronecker shifts from further PCG outputs of the pixel hash.
static inline float bounce_shift(const PixSeeds& S, uint32_t b, uint32_t k) { return u01(pcg(S.hs + 9u + 6u * (b - 2u) + k)); }

// ============================================================================================ vectors

template <typename R> struct V3 {
  R x, y, z;
  V3() : x(0), y(0), z(0) {}
  V3(R a, R b, R c) : x(a), y(b), z(c) {}
  V3 operator+(const V3& o) const { return V3(x + o.x, y + o.y, z + o.z); }
  V3 operator-(const V3& o) const { return V3(x - o.x, y - o.y, z - o.z); }
  V3 operator-() const { return V3(-x, -y, -z); }
  V3 operator*(R s) const { return V3(x * s, y * s, z * s); }
  V3 operator*(const V3& o) const { return V3(x * o.x, y * o.y, z * o.z); }
  V3 operator/(R s) const { return V3(x / s, y / s, z / s); }
  V3 operator/(const V3& o) const { return V3(x / o.x, y / o.y, z / o.z); }
};
template <typename R> static inline R dot(const V3<R>& a, const V3<R>& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <typename R> static inline V3<R> cross(const V3<R>& a, const V3<R>& b) {
  return V3<R>(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
template <typename R> static inline R len(const V3<R>& a) { return std::sqrt(dot(a, a)); }
template <typename R> static inline V3<R> normalize(const V3<R>& a) { return a / len(a); }
template <typename R> static inline R maxc(const V3<R>& a) { return std::max(a.x, std::max(a.y, a.z)); }
template <typename R> static inline R clampR(R x, R a, R b) { return std::min(std::max(x, a), b); }
template <typename R> static inline V3<R> mixv(const V3<R>& a, const V3<R>& b, R t) { return a * (R(1) - t) + b * t; }
template <typename R> static inline V3<R> ld3(const float* p) { return V3<R>(R(p[0]), R(p[1]), R(p[2])); }

// column-major 3x3 (WGSL mat3x3f): c[0..2] columns
template <typename R> struct M3 {
  V3<R> c[3];
  V3<R> mul(const V3<R>& v) const { return c[0] * v.x + c[1] * v.y + c[2] * v.z; }      // M v
  V3<R> tmul(const V3<R>& v) const { return V3<R>(dot(v, c[0]), dot(v, c[1]), dot(v, c[2])); } // v M = M^T v
};

// ============================================================================================ lens (gpu/lens.js)

struct Lens { double fx, fy, cx, cy, alpha, k[4]; };

// gpu/lens.js:19 distort, :25 distortDeriv, :31 undistortTheta, :43 project, :54 unproject (float64)
static inline double distort(const Lens& L, double th) {
  double t2 = th * th;
  return th * (1 + t2 * (L.k[0] + t2 * (L.k[1] + t2 * (L.k[2] + t2 * L.k[3]))));
}
static inline double distort_deriv(const Lens& L, double th) {
  double t2 = th * th;
  return 1 + t2 * (3 * L.k[0] + t2 * (5 * L.k[1] + t2 * (7 * L.k[2] + t2 * 9 * L.k[3])));
}
static inline double undistort_theta(const Lens& L, double thd, int iters = 20) {
  double th = thd;
  for (int i = 0; i < iters; i++) {
    double f = distort(L, th) - thd;
    double step = f / distort_deriv(L, th);
    th -= step;
    if (std::fabs(step) < 1e-15) break;
  }
  return th;
}
static inline void project(const Lens& L, const double X[3], double uv[2]) {
  double x = X[0], y = X[1], z = X[2];
  double rho = std::hypot(x, y);
  if (rho < 1e-300) { uv[0] = L.cx; uv[1] = L.cy; return; }
  double th = std::atan2(rho, z);
  double s = distort(L, th) / rho;
  double xd = x * s, yd = y * s;
  uv[0] = L.fx * (xd + L.alpha * yd) + L.cx;
  uv[1] = L.fy * yd + L.cy;
}
static inline void unproject(const Lens& L, const double uv[2], double out[3]) {
  double yd = (uv[1] - L.cy) / L.fy;
  double xd = (uv[0] - L.cx) / L.fx - L.alpha * yd;
  double thd = std::hypot(xd, yd);
  if (thd < 1e-300) { out[0] = 0; out[1] = 0; out[2] = 1; return; }
  double th = undistort_theta(L, thd);
  double s = std::sin(th) / thd;
  out[0] = xd * s; out[1] = yd * s; out[2] = std::cos(th);
}
// gpu/wgsl/lens.wgsl.js:32 kb4Project in precision R (the FP64 mode is gpu/lens.js:43 project)
template <typename R> static inline void kb4_project(const Lens& L, R x, R y, R z, R uv[2]) {
  if (sizeof(R) == 8) {
    double X[3] = {double(x), double(y), double(z)}, o[2];
    project(L, X, o);
    uv[0] = R(o[0]); uv[1] = R(o[1]);
    return;
  }
  R rho = std::sqrt(x * x + y * y);
  if (rho < R(1e-30)) { uv[0] = R(L.cx); uv[1] = R(L.cy); return; }
  R th = std::atan2(rho, z), t2 = th * th;
  R k0 = R(L.k[0]), k1 = R(L.k[1]), k2 = R(L.k[2]), k3 = R(L.k[3]);
  R s = th * (R(1) + t2 * (k0 + t2 * (k1 + t2 * (k2 + t2 * k3)))) / rho;
  R xd = x * s, yd = y * s;
  uv[0] = R(L.fx) * (xd + R(L.alpha) * yd) + R(L.cx);
  uv[1] = R(L.fy) * yd + R(L.cy);
}
// gpu/wgsl/lens.wgsl.js:9-30 kb4Theta (8 fixed Newton steps) / kb4Unproject, in precision R. The FP64 mode uses
// gpu/lens.js's unproject (20 steps, 1e-15 break).
template <typename R> static inline V3<R> kb4_unproject(const Lens& L, R u, R v) {
  if (sizeof(R) == 8) {
    double uv[2] = {double(u), double(v)}, o[3];
    unproject(L, uv, o);
    return V3<R>(R(o[0]), R(o[1]), R(o[2]));
  }
  R fx = R(L.fx), fy = R(L.fy), cx = R(L.cx), cy = R(L.cy), al = R(L.alpha);
  R k0 = R(L.k[0]), k1 = R(L.k[1]), k2 = R(L.k[2]), k3 = R(L.k[3]);
  R yd = (v - cy) / fy;
  R xd = (u - cx) / fx - al * yd;
  R thd = std::sqrt(xd * xd + yd * yd);
  if (thd < R(1e-20)) return V3<R>(0, 0, 1);
  R th = thd;
  for (int i = 0; i < 8; i++) {
    R t2 = th * th;
    R f = th * (R(1) + t2 * (k0 + t2 * (k1 + t2 * (k2 + t2 * k3)))) - thd;
    R fp = R(1) + t2 * (R(3) * k0 + t2 * (R(5) * k1 + t2 * (R(7) * k2 + t2 * R(9) * k3)));
    th = th - f / fp;
  }
  R s = std::sin(th) / thd;
  return V3<R>(xd * s, yd * s, std::cos(th));
}

// ============================================================================================ bvh (gpu/bvh.js)

struct BVH {
  std::vector<uint32_t> nodes;  // 16 words per node
  std::vector<uint32_t> order;
  uint32_t node_count = 0, max_depth = 1;
  float bmin[3], bmax[3];
};

// gpu/bvh.js:18-161 buildBVH (binned SAH, 16 bins, travCost = triCost = 1), float64 scratch over float32 boxes
static BVH build_bvh(const float* pos, const uint32_t* idx, uint32_t n, int leafSize) {
  const int bins = 16;
  const double travCost = 1.0, triCost = 1.0;
  std::vector<float> tbmin(3 * size_t(n)), tbmax(3 * size_t(n)), cen(3 * size_t(n));
  for (uint32_t t = 0; t < n; t++) {
    size_t a = size_t(idx[3 * t]) * 3, b = size_t(idx[3 * t + 1]) * 3, c = size_t(idx[3 * t + 2]) * 3;
    for (int k = 0; k < 3; k++) {
      double lo = std::min(std::min(double(pos[a + k]), double(pos[b + k])), double(pos[c + k]));
      double hi = std::max(std::max(double(pos[a + k]), double(pos[b + k])), double(pos[c + k]));
      tbmin[3 * t + k] = float(lo); tbmax[3 * t + k] = float(hi); cen[3 * t + k] = float(0.5 * (lo + hi));
    }
  }
  BVH out;
  out.order.resize(n);
  for (uint32_t i = 0; i < n; i++) out.order[i] = i;
  std::vector<uint32_t>& order = out.order;
  std::vector<uint32_t>& nodes = out.nodes;
  auto alloc = [&]() { nodes.resize(nodes.size() + 16, 0); return out.node_count++; };
  std::vector<uint32_t> bCount(bins), rCount(bins);
  std::vector<double> bMin(bins * 3), bMax(bins * 3), rArea(bins);
  struct Bounds { double lo[3], hi[3], clo[3], chi[3]; };
  auto rangeBounds = [&](int64_t s, int64_t e) {
    Bounds B;
    for (int k = 0; k < 3; k++) { B.lo[k] = BIGD; B.hi[k] = -BIGD; B.clo[k] = BIGD; B.chi[k] = -BIGD; }
    for (int64_t i = s; i < e; i++) {
      uint32_t t = order[i];
      for (int k = 0; k < 3; k++) {
        double a = tbmin[3 * t + k], b = tbmax[3 * t + k], c = cen[3 * t + k];
        if (a < B.lo[k]) B.lo[k] = a;
        if (b > B.hi[k]) B.hi[k] = b;
        if (c < B.clo[k]) B.clo[k] = c;
        if (c > B.chi[k]) B.chi[k] = c;
      }
    }
    return B;
  };
  auto area = [](const double* lo, const double* hi) {
    double dx = std::max(0.0, hi[0] - lo[0]), dy = std::max(0.0, hi[1] - lo[1]), dz = std::max(0.0, hi[2] - lo[2]);
    return dx * dy + dy * dz + dz * dx;
  };
  auto binOf = [&](uint32_t t, int ax, double lo, double sc) {
    double b = std::floor((double(cen[3 * t + ax]) - lo) * sc);
    int64_t bi = int64_t(b);
    if (bi >= bins) bi = bins - 1;
    return bi;
  };
  auto split = [&](int64_t s, int64_t e, const Bounds& B) -> int64_t {
    int64_t cnt = e - s;
    if (cnt <= 1) return -1;
    double best = std::numeric_limits<double>::infinity();
    int bestAxis = -1, bestBin = -1;
    double pA = area(B.lo, B.hi);
    for (int ax = 0; ax < 3; ax++) {
      double lo = B.clo[ax], ext = B.chi[ax] - lo;
      if (!(ext > 0)) continue;
      std::fill(bCount.begin(), bCount.end(), 0u);
      std::fill(bMin.begin(), bMin.end(), BIGD);
      std::fill(bMax.begin(), bMax.end(), -BIGD);
      double sc = bins / ext;
      for (int64_t i = s; i < e; i++) {
        uint32_t t = order[i];
        int64_t b = binOf(t, ax, lo, sc);
        bCount[b]++;
        for (int k = 0; k < 3; k++) {
          if (tbmin[3 * t + k] < bMin[3 * b + k]) bMin[3 * b + k] = tbmin[3 * t + k];
          if (tbmax[3 * t + k] > bMax[3 * b + k]) bMax[3 * b + k] = tbmax[3 * t + k];
        }
      }
      double lo3[3] = {BIGD, BIGD, BIGD}, hi3[3] = {-BIGD, -BIGD, -BIGD};
      uint32_t c = 0;
      for (int b = bins - 1; b > 0; b--) {
        c += bCount[b];
        for (int k = 0; k < 3; k++) { lo3[k] = std::min(lo3[k], bMin[3 * b + k]); hi3[k] = std::max(hi3[k], bMax[3 * b + k]); }
        rCount[b] = c; rArea[b] = c ? area(lo3, hi3) : 0;
      }
      for (int k = 0; k < 3; k++) { lo3[k] = BIGD; hi3[k] = -BIGD; }
      c = 0;
      for (int b = 0; b < bins - 1; b++) {
        c += bCount[b];
        for (int k = 0; k < 3; k++) { lo3[k] = std::min(lo3[k], bMin[3 * b + k]); hi3[k] = std::max(hi3[k], bMax[3 * b + k]); }
        if (c == 0 || rCount[b + 1] == 0) continue;
        double cost = travCost + triCost * (double(c) * area(lo3, hi3) + double(rCount[b + 1]) * rArea[b + 1]) / pA;
        if (cost < best) { best = cost; bestAxis = ax; bestBin = b; }
      }
    }
    if (bestAxis < 0) return cnt > int64_t(leafSize) * 4 ? s + (cnt >> 1) : -1;
    if (cnt <= leafSize && best >= triCost * double(cnt)) return -1;
    double lo = B.clo[bestAxis], sc = bins / (B.chi[bestAxis] - lo);
    int64_t i = s, j = e - 1;
    while (i <= j) {
      uint32_t t = order[i];
      int64_t b = binOf(t, bestAxis, lo, sc);
      if (b <= bestBin) i++;
      else { order[i] = order[j]; order[j] = t; j--; }
    }
    if (i == s || i == e) return s + (cnt >> 1);
    return i;
  };
  auto writeChild = [&](uint32_t node, int slot, const double* lo, const double* hi, uint32_t ref, uint32_t count) {
    size_t o = size_t(node) * 16 + slot * 8;
    nodes[o] = as_u(float(lo[0])); nodes[o + 1] = as_u(float(lo[1])); nodes[o + 2] = as_u(float(lo[2])); nodes[o + 3] = ref;
    nodes[o + 4] = as_u(float(hi[0])); nodes[o + 5] = as_u(float(hi[1])); nodes[o + 6] = as_u(float(hi[2])); nodes[o + 7] = count;
  };
  uint32_t root = alloc();
  Bounds R = rangeBounds(0, n);
  struct Item { uint32_t node; int64_t s, e, m; uint32_t d; };
  std::vector<Item> stack;
  int64_t m0 = n ? split(0, n, R) : -1;
  if (n == 0) {
    double far_[3] = {BIGD, BIGD, BIGD};
    writeChild(root, 0, far_, far_, 0, 1); writeChild(root, 1, far_, far_, 0, 1);
  } else if (m0 < 0) {
    uint32_t h = n > 1 ? n >> 1 : n;
    Bounds B0 = rangeBounds(0, h);
    writeChild(root, 0, B0.lo, B0.hi, 0, h);
    if (n > 1) { Bounds B1 = rangeBounds(h, n); writeChild(root, 1, B1.lo, B1.hi, h, n - h); }
    else writeChild(root, 1, R.lo, R.hi, 0, n);
  } else stack.push_back({root, 0, int64_t(n), m0, 1});
  out.max_depth = 1;
  while (!stack.empty()) {
    Item it = stack.back(); stack.pop_back();
    out.max_depth = std::max(out.max_depth, it.d);
    int64_t ranges[2][2] = {{it.s, it.m}, {it.m, it.e}};
    for (int slot = 0; slot < 2; slot++) {
      int64_t a = ranges[slot][0], b = ranges[slot][1];
      Bounds B = rangeBounds(a, b);
      int64_t mm = split(a, b, B);
      if (mm < 0) writeChild(it.node, slot, B.lo, B.hi, uint32_t(a), uint32_t(b - a));
      else {
        uint32_t child = alloc();
        writeChild(it.node, slot, B.lo, B.hi, child, 0);
        stack.push_back({child, a, b, mm, it.d + 1});
      }
    }
  }
  for (int k = 0; k < 3; k++) { out.bmin[k] = float(R.lo[k]); out.bmax[k] = float(R.hi[k]); }
  return out;
}

// gpu/bvh.js:189 intersectTri (float64 over the packed float32 record)
static inline double intersect_tri_js(const float* T, uint32_t k, const double o[3], const double d[3], double tmin,
                                      double tmax, double bary[2]) {
  const float* b = T + size_t(k) * 16;
  double e1x = b[4], e1y = b[5], e1z = b[6], e2x = b[8], e2y = b[9], e2z = b[10];
  double px = d[1] * e2z - d[2] * e2y, py = d[2] * e2x - d[0] * e2z, pz = d[0] * e2y - d[1] * e2x;
  double det = e1x * px + e1y * py + e1z * pz;
  if (std::fabs(det) < 1e-30) return INFINITY;
  double inv = 1 / det;
  double sx = o[0] - b[0], sy = o[1] - b[1], sz = o[2] - b[2];
  double u = (sx * px + sy * py + sz * pz) * inv;
  if (u < 0 || u > 1) return INFINITY;
  double qx = sy * e1z - sz * e1y, qy = sz * e1x - sx * e1z, qz = sx * e1y - sy * e1x;
  double v = (d[0] * qx + d[1] * qy + d[2] * qz) * inv;
  if (v < 0 || u + v > 1) return INFINITY;
  double t = (e2x * qx + e2y * qy + e2z * qz) * inv;
  if (t <= tmin || t >= tmax) return INFINITY;
  bary[0] = u; bary[1] = v;
  return t;
}
// gpu/bvh.js:208 slab
static inline double slab_js(const float* N, const double o[3], const double inv[3], size_t x, double tmin, double tmax) {
  double t0 = tmin, t1 = tmax;
  for (int k = 0; k < 3; k++) {
    double a = (double(N[x + k]) - o[k]) * inv[k], b = (double(N[x + 4 + k]) - o[k]) * inv[k];
    if (a > b) std::swap(a, b);
    if (a > t0) t0 = a;
    if (b < t1) t1 = b;
    if (t0 > t1) return INFINITY;
  }
  return t0;
}
struct HitJS { double t, u, v; int64_t tri; };
// gpu/bvh.js:224-250 traverse (closest or any hit), ordered descent with a stack of node ids
static HitJS traverse_js(const uint32_t* nodesU, const float* T, const double o[3], const double d[3], double tmin,
                         double tmax, bool anyHit, uint32_t root) {
  const float* N = reinterpret_cast<const float*>(nodesU);
  double inv[3] = {1 / d[0], 1 / d[1], 1 / d[2]};
  double bary[2] = {0, 0};
  double best = tmax, bu = 0, bv = 0;
  int64_t tri = -1;
  std::vector<uint32_t> stack;
  stack.push_back(root);
  while (!stack.empty()) {
    uint32_t node = stack.back(); stack.pop_back();
    size_t base = size_t(node) * 16;
    double tc[2] = {slab_js(N, o, inv, base, tmin, best), slab_js(N, o, inv, base + 8, tmin, best)};
    std::pair<double, uint32_t> push[2];
    int np = 0;
    for (int c = 0; c < 2; c++) {
      if (!(tc[c] < best)) continue;
      uint32_t ref = nodesU[base + c * 8 + 3], cnt = nodesU[base + c * 8 + 7];
      if (cnt > 0) {
        for (uint32_t k = ref; k < ref + cnt; k++) {
          double t = intersect_tri_js(T, k, o, d, tmin, best, bary);
          if (t < best) {
            best = t; tri = k; bu = bary[0]; bv = bary[1];
            if (anyHit) return {t, bu, bv, tri};
          }
        }
      } else push[np++] = {tc[c], ref};
    }
    if (np == 2 && push[1].first > push[0].first) std::swap(push[0], push[1]);   // far first (stable sort)
    for (int i = 0; i < np; i++) stack.push_back(push[i].second);
  }
  return {tri >= 0 ? best : INFINITY, bu, bv, tri};
}
// gpu/bvh.js:253 bruteForce
static HitJS brute_force(const float* T, uint32_t count, const double o[3], const double d[3], double tmin, double tmax) {
  double bary[2] = {0, 0}, best = tmax, bu = 0, bv = 0;
  int64_t tri = -1;
  for (uint32_t k = 0; k < count; k++) {
    double t = intersect_tri_js(T, k, o, d, tmin, best, bary);
    if (t < best) { best = t; tri = k; bu = bary[0]; bv = bary[1]; }
  }
  return {tri >= 0 ? best : INFINITY, bu, bv, tri};
}

// ============================================================================================ bsdf (gpu/bsdf.js)

struct Mat {
  int metallic = 0;          // 0 dielectric, 1 conductor, 2 coated conductor
  bool coated = false, emitter = false, has_table = true, textured = false;
  double rho[3] = {0, 0, 0}, f0[3] = {0, 0, 0};
  double roughness = 0.5, alpha = 0.25, ior = 1.5, fbar = 0, fbarComputed = 0;
  double alphaC = 0, tau[3] = {1, 1, 1};
  double ink[3] = {0, 0, 0}, roughInk = 0.4;
  std::vector<double> spec, diff;  // albedo table, 3 per bin
  double hh[3] = {0, 0, 0}, hhSpec[3] = {0, 0, 0};
};

static const double INV_PI_D = 1.0 / M_PI;

// gpu/bsdf.js:25 fresnelDielectric
template <typename R> static inline R fresnel_dielectric(R cosi, R eta) {
  R c = std::min(R(1), std::max(R(0), cosi));
  R s2 = (R(1) - c * c) / (eta * eta);
  if (s2 >= R(1)) return R(1);
  R ct = std::sqrt(R(1) - s2);
  R rs = (c - eta * ct) / (c + eta * ct), rp = (eta * c - ct) / (eta * c + ct);
  return R(0.5) * (rs * rs + rp * rp);
}
// gpu/bsdf.js:35 fresnelAverage (composite Simpson, 4096 intervals)
static double fresnel_average(double eta, int n = 4096) {
  double s = 0;
  for (int i = 0; i <= n; i++) {
    double mu = double(i) / n;
    double w = (i == 0 || i == n) ? 1 : (i % 2 ? 4 : 2);
    s += w * fresnel_dielectric(mu, eta) * mu;
  }
  return 2 * s / (3 * n);
}
template <typename R> static inline R schlick(R f0, R c) {
  R m = std::pow(R(1) - std::min(R(1), std::max(R(0), c)), R(5));
  return f0 + (R(1) - f0) * m;
}
// gpu/bsdf.js:46-59 GGX D, Lambda, G1, G2
template <typename R> static inline R ggx_d(R nh, R a) {
  if (nh <= R(0)) return R(0);
  R a2 = a * a, d = nh * nh * (a2 - R(1)) + R(1);
  return a2 / (R(M_PI) * d * d);
}
template <typename R> static inline R ggx_lambda(R c, R a) {
  R c2 = std::max(c * c, R(1e-12));
  R t2 = (R(1) - c2) / c2;
  return R(0.5) * (R(-1) + std::sqrt(R(1) + a * a * t2));
}
template <typename R> static inline R ggx_g1(R c, R a) { return R(1) / (R(1) + ggx_lambda(c, a)); }
template <typename R> static inline R ggx_g2(R nl, R nv, R a) { return R(1) / (R(1) + ggx_lambda(nl, a) + ggx_lambda(nv, a)); }

// The material record as the WGSL sees it (gpu/wgsl/bsdf.wgsl.js:4-26 Mat / loadMat), in precision R
template <typename R> struct MatR {
  V3<R> c; R alpha, ior, metal, fbar, rough; V3<R> hh, hhSpec; R x[4]; uint32_t idx;
};
template <typename R> static inline R lumR(const V3<R>& c) { return c.x * R(0.2126) + c.y * R(0.7152) + c.z * R(0.0722); }

// gpu/wgsl/bsdf.wgsl.js:43 fresnelRGB, :63 evalBSDF (= gpu/bsdf.js:98)
template <typename R> static inline V3<R> schlick3(const V3<R>& f0, R c) {
  R m = std::pow(R(1) - clampR(c, R(0), R(1)), R(5));
  return f0 + (V3<R>(1, 1, 1) - f0) * m;
}
template <typename R> static inline V3<R> fresnel_rgb(const MatR<R>& M, R c) {
  if (M.metal > R(0.5)) return schlick3(M.c, c);
  R F = fresnel_dielectric(c, M.ior);
  return V3<R>(F, F, F);
}
template <typename R> static inline V3<R> eval_bsdf(const MatR<R>& M, const V3<R>& n, const V3<R>& l, const V3<R>& v) {
  R nl = dot(n, l), nv = dot(n, v);
  if (nl <= R(0) || nv <= R(0)) return V3<R>();
  V3<R> h = normalize(l + v);
  R nh = dot(n, h), vh = std::max(R(0), dot(v, h));
  if (M.metal > R(1.5)) {
    R ac = M.x[3];
    R coat = ggx_d(nh, ac) * ggx_g2(nl, nv, ac) * fresnel_dielectric(vh, M.ior) / (R(4) * nl * nv);
    R t = (R(1) - fresnel_dielectric(nl, M.ior)) * (R(1) - fresnel_dielectric(nv, M.ior));
    R metal = ggx_d(nh, M.alpha) * ggx_g2(nl, nv, M.alpha) / (R(4) * nl * nv);
    R ex = R(1) / nl + R(1) / nv;
    V3<R> tp(std::pow(M.x[0], ex), std::pow(M.x[1], ex), std::pow(M.x[2], ex));
    return V3<R>(coat, coat, coat) + tp * (schlick3(M.c, vh) * (t * metal));
  }
  R spec = ggx_d(nh, M.alpha) * ggx_g2(nl, nv, M.alpha) / (R(4) * nl * nv);
  V3<R> out = fresnel_rgb(M, vh) * spec;
  if (M.metal < R(0.5)) {
    R kd = R(INV_PI_D) * (R(1) - fresnel_dielectric(nl, M.ior)) * (R(1) - fresnel_dielectric(nv, M.ior)) / (R(1) - M.fbar);
    out = out + M.c * kd;
  }
  return out;
}
// gpu/wgsl/common.wgsl.js:146-157 basisT / basisB (Duff et al. 2017)
template <typename R> static inline V3<R> basis_t(const V3<R>& n) {
  R s = n.z >= R(0) ? R(1) : R(-1);
  R a = R(-1) / (s + n.z), b = n.x * n.y * a;
  return V3<R>(R(1) + s * n.x * n.x * a, s * b, -s * n.x);
}
template <typename R> static inline V3<R> basis_b(const V3<R>& n) {
  R s = n.z >= R(0) ? R(1) : R(-1);
  R a = R(-1) / (s + n.z), b = n.x * n.y * a;
  return V3<R>(b, s + n.y * n.y * a, -n.y);
}
// gpu/bsdf.js:131 sampleVNDF (Heitz 2018)
template <typename R> static inline V3<R> sample_vndf(const V3<R>& ve, R a, R u1, R u2) {
  V3<R> vh = normalize(V3<R>(a * ve.x, a * ve.y, ve.z));
  R lensq = vh.x * vh.x + vh.y * vh.y;
  V3<R> T1 = lensq > R(0) ? V3<R>(-vh.y, vh.x, 0) / std::sqrt(lensq) : V3<R>(1, 0, 0);
  V3<R> T2 = cross(vh, T1);
  R r = std::sqrt(u1), phi = R(2) * R(M_PI) * u2;
  R t1 = r * std::cos(phi);
  R t2 = r * std::sin(phi);
  R s = R(0.5) * (R(1) + vh.z);
  t2 = (R(1) - s) * std::sqrt(std::max(R(0), R(1) - t1 * t1)) + s * t2;
  R t3 = std::sqrt(std::max(R(0), R(1) - t1 * t1 - t2 * t2));
  V3<R> nh = T1 * t1 + T2 * t2 + vh * t3;
  return normalize(V3<R>(a * nh.x, a * nh.y, std::max(R(1e-7), nh.z)));
}
// gpu/bsdf.js:147 specProb
template <typename R> static inline R spec_prob(const MatR<R>& M, R nv) {
  if (M.metal > R(1.5)) {
    R Fc = fresnel_dielectric(nv, M.ior);
    return Fc / (Fc + (R(1) - Fc) * (M.c.x + M.c.y + M.c.z) / R(3));
  }
  if (M.metal > R(0.5)) return R(1);
  R F = fresnel_dielectric(nv, M.ior);
  R d = lumR(M.c) * (R(1) - F);
  R s = std::max(F, R(0.04));
  return clampR(s / (s + d), R(0.05), R(0.95));
}
// gpu/bsdf.js:160 pdfBSDF
template <typename R> static inline R pdf_bsdf(const MatR<R>& M, const V3<R>& n, const V3<R>& v, const V3<R>& l) {
  R nl = dot(n, l), nv = dot(n, v);
  if (nl <= R(0) || nv <= R(0)) return R(0);
  V3<R> h = normalize(l + v);
  R nh = dot(n, h), vh = dot(v, h);
  R ps = spec_prob(M, nv);
  if (M.metal > R(1.5)) {
    if (vh <= R(0)) return R(0);
    return ps * ggx_g1(nv, M.x[3]) * ggx_d(nh, M.x[3]) / (R(4) * nv) + (R(1) - ps) * ggx_g1(nv, M.alpha) * ggx_d(nh, M.alpha) / (R(4) * nv);
  }
  R pdfSpec = vh > R(0) ? ggx_g1(nv, M.alpha) * ggx_d(nh, M.alpha) / (R(4) * nv) : R(0);
  return ps * pdfSpec + (R(1) - ps) * nl * R(INV_PI_D);
}
// gpu/bsdf.js:176 sampleBSDF; returns pdf 0 for an invalid sample
template <typename R> static inline R sample_bsdf(const MatR<R>& M, const V3<R>& n, const V3<R>& v, const V3<R>& u, V3<R>& l) {
  R nv = dot(n, v);
  if (nv <= R(0)) return R(0);
  V3<R> t = basis_t(n), b = basis_b(n);
  R ps = spec_prob(M, nv);
  if (M.metal > R(1.5) || u.x < ps) {
    R a = (M.metal > R(1.5)) ? (u.x < ps ? M.x[3] : M.alpha) : M.alpha;
    V3<R> hl = sample_vndf(V3<R>(dot(t, v), dot(b, v), nv), a, u.y, u.z);
    V3<R> h = t * hl.x + b * hl.y + n * hl.z;
    l = h * (R(2) * dot(v, h)) - v;
  } else {
    R r = std::sqrt(u.y), phi = R(2) * R(M_PI) * u.z;
    l = t * (r * std::cos(phi)) + b * (r * std::sin(phi)) + n * std::sqrt(std::max(R(0), R(1) - u.y));
  }
  if (dot(n, l) <= R(0)) return R(0);
  return pdf_bsdf(M, n, v, l);
}
// gpu/bsdf.js:176 sampleBSDF / :98 evalBSDF on the float64 material (for the albedo tables)
static double radinv2(uint32_t i) { double b = 0, f = 0.5; while (i) { if (i & 1) b += f; i >>= 1; f *= 0.5; } return b; }
static MatR<double> mat_r64(const Mat& m) {
  MatR<double> M;
  const double* c = m.metallic ? m.f0 : m.rho;
  M.c = V3<double>(c[0], c[1], c[2]);
  M.alpha = m.alpha; M.ior = m.ior; M.metal = m.metallic; M.fbar = m.fbar; M.rough = m.roughness;
  M.x[0] = m.tau[0]; M.x[1] = m.tau[1]; M.x[2] = m.tau[2]; M.x[3] = m.alphaC; M.idx = 0;
  return M;
}
// gpu/bsdf.js:210 albedoTable (bins = 32, samples = 1024 as gpu/scene_gpu.js:197)
static void albedo_table(Mat& M, int bins, int samples) {
  M.spec.assign(bins * 3, 0); M.diff.assign(bins * 3, 0);
  MatR<double> MR = mat_r64(M);
  V3<double> n(0, 0, 1);
  for (int k = 0; k < bins; k++) {
    double mu = (k + 0.5) / bins;
    V3<double> v(std::sqrt(1 - mu * mu), 0, mu);
    double acc[3] = {0, 0, 0};
    if (M.coated) {
      for (int i = 0; i < samples; i++) {
        V3<double> u((i + 0.5) / samples, radinv2(i), std::fmod(radinv2(i ^ 0x5555), 1.0)), l;
        double pdf = sample_bsdf(MR, n, v, u, l);
        if (!(pdf > 0)) continue;
        V3<double> f = eval_bsdf(MR, n, l, v);
        acc[0] += f.x * l.z / pdf; acc[1] += f.y * l.z / pdf; acc[2] += f.z * l.z / pdf;
      }
      for (int c = 0; c < 3; c++) { M.spec[3 * k + c] = acc[c] / samples; M.diff[3 * k + c] = 0; }
      continue;
    }
    for (int i = 0; i < samples; i++) {
      double u1 = (i + 0.5) / samples, u2 = radinv2(i);
      V3<double> h = sample_vndf(v, M.alpha, u1, u2);
      double vh = dot(v, h);
      V3<double> l = h * (2 * vh) - v;
      if (l.z <= 0) continue;
      double w = ggx_g2(l.z, mu, M.alpha) / ggx_g1(mu, M.alpha);
      V3<double> F = fresnel_rgb(MR, vh);
      acc[0] += F.x * w; acc[1] += F.y * w; acc[2] += F.z * w;
    }
    for (int c = 0; c < 3; c++) {
      M.spec[3 * k + c] = acc[c] / samples;
      M.diff[3 * k + c] = M.metallic ? 0 : M.rho[c] * (1 - fresnel_dielectric(mu, M.ior)) * (1 - M.fbarComputed) / (1 - M.fbar);
    }
  }
  for (int c = 0; c < 3; c++) { M.hh[c] = 0; M.hhSpec[c] = 0; }
  for (int k = 0; k < bins; k++) {
    double mu = (k + 0.5) / bins;
    for (int c = 0; c < 3; c++) {
      M.hh[c] += 2 * mu * (M.spec[3 * k + c] + M.diff[3 * k + c]) / bins;
      M.hhSpec[c] += 2 * mu * M.spec[3 * k + c] / bins;
    }
  }
}
// gpu/bsdf.js:68 prepareMaterial
static Mat prepare_material(const vt_material& m, int albedoSamples) {
  Mat M;
  if (m.coated) {
    double roughness = std::max(double(m.roughness), 0.02), rc = std::max(double(m.coat_roughness), 0.02);
    M.metallic = 2; M.coated = true; M.roughness = roughness; M.alpha = roughness * roughness;
    for (int c = 0; c < 3; c++) { M.f0[c] = m.f0[c]; M.rho[c] = 0; M.tau[c] = m.tau[c]; }
    M.ior = m.coat_ior; M.alphaC = rc * rc; M.fbar = 0; M.fbarComputed = 0;
  } else {
    M.metallic = m.metallic ? 1 : 0;
    double roughness = std::max(double(m.roughness), 0.02);
    M.roughness = roughness; M.alpha = roughness * roughness;
    for (int c = 0; c < 3; c++) { M.rho[c] = M.metallic ? 0 : m.rho[c]; M.f0[c] = M.metallic ? m.f0[c] : 0; }
    M.ior = m.ior;
    M.fbarComputed = M.metallic ? 0 : fresnel_average(M.ior);
    M.fbar = M.metallic ? 0 : (std::isfinite(m.fbar) ? double(m.fbar) : M.fbarComputed);
  }
  M.emitter = m.emitter != 0;
  M.textured = m.textured != 0;
  for (int c = 0; c < 3; c++) M.ink[c] = m.ink_rho[c];
  M.roughInk = m.ink_roughness;
  M.has_table = !m.no_table;
  if (M.has_table) albedo_table(M, VT_ALBEDO_BINS, albedoSamples);
  return M;
}

// ============================================================================================ shade_ref helpers

// gpu/shade_ref.js:5 profile
static double profile_js(double theta, const std::vector<double>& knots, const std::vector<double>& p) {
  size_t n = knots.size();
  if (theta >= knots[n - 1]) return theta == knots[n - 1] ? p[n - 1] : 0;
  size_t lo = 0, hi = n - 1;
  while (hi - lo > 1) { size_t m = (lo + hi) >> 1; if (knots[m] <= theta) lo = m; else hi = m; }
  double f = std::min(1.0, std::max(0.0, (theta - knots[lo]) / std::max(knots[hi] - knots[lo], 1e-12)));
  return p[lo] + (p[hi] - p[lo]) * f;
}
// gpu/shade_ref.js:64 gaussLegendre
static void gauss_legendre(int n, std::vector<double>& x, std::vector<double>& w) {
  x.assign(n, 0); w.assign(n, 0);
  for (int i = 0; i < n; i++) {
    double z = std::cos(M_PI * (i + 0.75) / (n + 0.5)), pp = 0;
    for (int it = 0; it < 100; it++) {
      double p1 = 1, p2 = 0;
      for (int j = 1; j <= n; j++) { double p3 = p2; p2 = p1; p1 = ((2 * j - 1) * z * p2 - (j - 1) * p3) / j; }
      pp = n * (z * p1 - p2) / (z * z - 1);
      double z1 = z; z = z1 - p1 / pp;
      if (std::fabs(z - z1) < 1e-15) break;
    }
    x[i] = -z; w[i] = 2 / ((1 - z * z) * pp * pp);
  }
}
// gpu/shade_ref.js:44 discIrradiance
static double disc_irradiance(const double* x, const double* n, const double* c, const double* m, double a, double L,
                              int nr, int nphi) {
  std::vector<double> gx, gw;
  gauss_legendre(nr, gx, gw);
  double t[3] = {std::fabs(m[0]) < 0.9 ? 1.0 : 0.0, std::fabs(m[0]) < 0.9 ? 0.0 : 1.0, 0};
  double u[3] = {m[1] * t[2] - m[2] * t[1], m[2] * t[0] - m[0] * t[2], m[0] * t[1] - m[1] * t[0]};
  double ul = std::sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
  for (double& q : u) q /= ul;
  double w[3] = {m[1] * u[2] - m[2] * u[1], m[2] * u[0] - m[0] * u[2], m[0] * u[1] - m[1] * u[0]};
  double E = 0;
  for (int i = 0; i < nr; i++) {
    double rho = 0.5 * a * (gx[i] + 1), wr = 0.5 * a * gw[i];
    for (int j = 0; j < nphi; j++) {
      double ph = (2 * M_PI * (j + 0.5)) / nphi;
      double q[3], d[3];
      for (int k = 0; k < 3; k++) { q[k] = c[k] + rho * (std::cos(ph) * u[k] + std::sin(ph) * w[k]); d[k] = q[k] - x[k]; }
      double d2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2], dl = std::sqrt(d2);
      double cosX = (n[0] * d[0] + n[1] * d[1] + n[2] * d[2]) / dl, cosQ = -(m[0] * d[0] + m[1] * d[1] + m[2] * d[2]) / dl;
      if (cosX > 0 && cosQ > 0) E += L * cosX * cosQ / d2 * rho * wr * (2 * M_PI / nphi);
    }
  }
  return E;
}
// gpu/shade_ref.js:21 capsuleOcc (= gpu/wgsl/shade.wgsl.js:59), precision R
template <typename R> static R capsule_occ(const V3<R>& p, const V3<R>& n, const V3<R>& a, const V3<R>& bb, R r) {
  V3<R> ab = bb - a;
  R L = len(ab);
  if (L < R(1e-9) || r <= R(0)) return R(0);
  V3<R> e = ab / L;
  V3<R> ap = p - a;
  R s0 = dot(ap, e);
  V3<R> perp = ap - e * s0;
  R h = std::sqrt(dot(perp, perp) + r * r);
  R pl = len(perp);
  V3<R> ep = -perp / std::max(pl, R(1e-12));
  if (pl < R(1e-12)) ep = normalize(cross(e, basis_t(e)));
  R np = dot(n, ep), na = dot(n, e);
  R f1 = std::atan((R(0) - s0) / h), f2 = std::atan((L - s0) / h);
  R f0 = std::atan2(na, np);
  f1 = std::max(f1, f0 - R(0.5) * R(M_PI));
  f2 = std::min(f2, f0 + R(0.5) * R(M_PI));
  if (f2 <= f1) return R(0);
  R I = np * (R(0.5) * (f2 - f1) + R(0.25) * (std::sin(R(2) * f2) - std::sin(R(2) * f1))) +
        na * R(0.5) * (std::sin(f2) * std::sin(f2) - std::sin(f1) * std::sin(f1));
  return clampR(R(INV_PI_D) * (R(2) * r / h) * I, R(0), R(1));
}

// ============================================================================================ scene (prepareScene)

struct Blas {
  uint32_t root, tri_off, tri_count, kind;
  float bmin[3], bmax[3];
  double cap_a[3], cap_b[3], cap_r, occ_a[3], occ_b[3], occ_r, rho_eff;
  int owner;
};
struct Inst { float w[48]; };   // gpu/wgsl/common.wgsl.js:60-67 Inst: 12 vec4

struct Scene {
  std::vector<uint32_t> nodes, tris, verts;
  std::vector<float> params;     // vec4 array
  uint32_t nodeCount = 0, triCount = 0, vertCount = 0, staticVerts = 0, staticTris = 0, nMesh = 0, nMat = 0;
  uint32_t meshOff, matOff, albOff, profOff, profN, emitOff, emitN;
  std::vector<Blas> blas;
  std::vector<Mat> mats;
  std::vector<vt_mesh> meshes;
  double emitArea = 0, emitAxis[3], emitNormal[3], centroid[3], radius = 0, scopeAhead;
  bool shadowSkipsScope = false;
  int scopeIndex = -1;
  float L0[3];
  std::vector<double> profTheta, profP;
  std::vector<vt_camera_desc> cams;
  // scene uniform
  float sceneU[24 + 48 * VT_MAX_INST];
  std::vector<float> nodeState;   // 16 per static vertex
  double eAvg[3] = {0, 0, 0};
  // instance poses
  struct Pose4 { double q0[4], q1[4], p0[3], p1[3]; bool valid; };
  std::vector<Pose4> inst;
  std::vector<uint32_t> emitOfTri;   // per triangle slot: index in the emitter table, or MISS
  std::vector<float> solvedCaps;     // 8 per body: bounding capsules at the last node update (empty: the current ones)
  std::vector<double> emitTris;      // 14 per emitter triangle (scope frame): v0, e1, e2, n, area, cdf
};

// gpu/scene_gpu.js:504 fitCapsule
static void fit_capsule(const float* P, size_t n, double a[3], double b[3], double& r) {
  if (!n) { for (int k = 0; k < 3; k++) a[k] = b[k] = 0; r = 0; return; }
  double c[3] = {0, 0, 0};
  for (size_t v = 0; v < n; v++) for (int k = 0; k < 3; k++) c[k] += double(P[3 * v + k]) / double(n);
  double C[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  for (size_t v = 0; v < n; v++) {
    double d[3] = {P[3 * v] - c[0], P[3 * v + 1] - c[1], P[3 * v + 2] - c[2]};
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) C[i][j] += d[i] * d[j];
  }
  double ax[3] = {0.3, 0.5, 0.8};
  for (int it = 0; it < 64; it++) {
    double y[3];
    for (int i = 0; i < 3; i++) y[i] = C[i][0] * ax[0] + C[i][1] * ax[1] + C[i][2] * ax[2];
    double l = std::sqrt(y[0] * y[0] + y[1] * y[1] + y[2] * y[2]);
    if (!(l > 0)) break;
    for (int i = 0; i < 3; i++) ax[i] = y[i] / l;
  }
  double smin = INFINITY, smax = -INFINITY;
  r = 0;
  for (size_t v = 0; v < n; v++) {
    double d[3] = {P[3 * v] - c[0], P[3 * v + 1] - c[1], P[3 * v + 2] - c[2]};
    double s = d[0] * ax[0] + d[1] * ax[1] + d[2] * ax[2];
    smin = std::min(smin, s); smax = std::max(smax, s);
    double e0 = d[0] - s * ax[0], e1 = d[1] - s * ax[1], e2 = d[2] - s * ax[2];
    r = std::max(r, std::sqrt(e0 * e0 + e1 * e1 + e2 * e2));
  }
  for (int k = 0; k < 3; k++) { a[k] = c[k] + smin * ax[k]; b[k] = c[k] + smax * ax[k]; }
}

static void pack_tri(std::vector<uint32_t>& tris, uint32_t slot, const float* pos, const uint32_t* I, uint32_t t,
                     uint32_t i0, uint32_t i1, uint32_t i2, uint32_t mesh, uint32_t flags) {
  // gpu/bvh.js:175 packTriangles + gpu/scene_gpu.js:361-365 putAttr (64 B record)
  size_t a = size_t(I[3 * t]) * 3, b = size_t(I[3 * t + 1]) * 3, c = size_t(I[3 * t + 2]) * 3;
  size_t o = size_t(slot) * 16;
  float* T = reinterpret_cast<float*>(tris.data());
  T[o] = pos[a]; T[o + 1] = pos[a + 1]; T[o + 2] = pos[a + 2];
  T[o + 4] = pos[b] - pos[a]; T[o + 5] = pos[b + 1] - pos[a + 1]; T[o + 6] = pos[b + 2] - pos[a + 2];
  T[o + 8] = pos[c] - pos[a]; T[o + 9] = pos[c + 1] - pos[a + 1]; T[o + 10] = pos[c + 2] - pos[a + 2];
  tris[o + 3] = i0; tris[o + 7] = i1; tris[o + 11] = i2; tris[o + 12] = mesh; tris[o + 13] = flags;
}

// gpu/scene_gpu.js:241-472 prepareScene (static part already welded) + gpu/renderer.js:271-331 _buildBuffers params
static Scene* prepare_scene(const vt_scene_desc* sd, int leafSize, int albedoSamples) {
  Scene* S = new Scene();
  S->meshes.assign(sd->meshes, sd->meshes + sd->n_meshes);
  for (uint32_t i = 0; i < sd->n_materials; i++) S->mats.push_back(prepare_material(sd->materials[i], albedoSamples));
  S->nMesh = sd->n_meshes; S->nMat = sd->n_materials;
  S->staticVerts = sd->n_static_verts; S->staticTris = sd->n_static_tris;
  BVH sb = build_bvh(sd->static_P, sd->static_I, sd->n_static_tris, leafSize);
  std::vector<BVH> bb;
  struct EmitTri { double v0[3], e1[3], e2[3], n[3], area, cdf; };
  std::vector<EmitTri> emit;
  std::vector<std::vector<uint32_t>> emitIdx(sd->n_bodies);
  for (uint32_t bi = 0; bi < sd->n_bodies; bi++) {
    const vt_body_desc& B = sd->bodies[bi];
    bb.push_back(build_bvh(B.P, B.I, B.n_tris, leafSize));
    emitIdx[bi].assign(B.n_tris, MISS);
    for (uint32_t t = 0; t < B.n_tris; t++) {
      if (!(sd->meshes[B.tri_mesh[t]].flags & VT_F_EMITTER)) continue;
      emitIdx[bi][t] = uint32_t(emit.size());
      size_t a = size_t(B.I[3 * t]) * 3, b = size_t(B.I[3 * t + 1]) * 3, c = size_t(B.I[3 * t + 2]) * 3;
      EmitTri e;
      for (int k = 0; k < 3; k++) { e.v0[k] = B.P[a + k]; e.e1[k] = double(B.P[b + k]) - e.v0[k]; e.e2[k] = double(B.P[c + k]) - e.v0[k]; }
      double n[3] = {e.e1[1] * e.e2[2] - e.e1[2] * e.e2[1], e.e1[2] * e.e2[0] - e.e1[0] * e.e2[2], e.e1[0] * e.e2[1] - e.e1[1] * e.e2[0]};
      e.area = 0.5 * std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
      double vn[3];
      for (int k = 0; k < 3; k++) vn[k] = double(B.N[a + k]) + double(B.N[b + k]) + double(B.N[c + k]);
      if (n[0] * vn[0] + n[1] * vn[1] + n[2] * vn[2] < 0) for (double& q : n) q = -q;
      double l = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
      if (!(l > 0)) l = 1;
      for (int k = 0; k < 3; k++) e.n[k] = n[k] / l;
      emit.push_back(e);
    }
  }
  uint32_t nodeTotal = sb.node_count, triTotal = sd->n_static_tris;
  S->blas.resize(sd->n_bodies);
  for (uint32_t bi = 0; bi < sd->n_bodies; bi++) {
    Blas& bl = S->blas[bi];
    bl.root = nodeTotal; bl.tri_off = triTotal; bl.tri_count = sd->bodies[bi].n_tris; bl.kind = sd->bodies[bi].kind;
    bl.owner = sd->bodies[bi].owner_camera;
    for (int k = 0; k < 3; k++) { bl.bmin[k] = bb[bi].bmin[k]; bl.bmax[k] = bb[bi].bmax[k]; }
    nodeTotal += bb[bi].node_count; triTotal += sd->bodies[bi].n_tris;
  }
  S->nodeCount = nodeTotal; S->triCount = triTotal;
  S->nodes.assign(size_t(nodeTotal) * 16, 0);
  std::copy(sb.nodes.begin(), sb.nodes.end(), S->nodes.begin());
  for (uint32_t bi = 0; bi < sd->n_bodies; bi++) {   // gpu/bvh.js:164 relocate
    std::vector<uint32_t> u = bb[bi].nodes;
    for (size_t o = 0; o < u.size(); o += 8) u[o + 3] += (u[o + 7] == 0) ? S->blas[bi].root : S->blas[bi].tri_off;
    std::copy(u.begin(), u.end(), S->nodes.begin() + size_t(S->blas[bi].root) * 16);
  }
  S->tris.assign(size_t(triTotal) * 16, 0);
  S->emitOfTri.assign(triTotal, MISS);
  for (uint32_t k = 0; k < sd->n_static_tris; k++) {
    uint32_t t = sb.order[k];
    uint32_t m = sd->static_tri_mesh[t];
    pack_tri(S->tris, k, sd->static_P, sd->static_I, t, sd->static_I[3 * t], sd->static_I[3 * t + 1], sd->static_I[3 * t + 2], m, sd->meshes[m].flags);
  }
  uint32_t vbase = sd->n_static_verts;
  std::vector<uint32_t> vertBase(sd->n_bodies);
  for (uint32_t bi = 0; bi < sd->n_bodies; bi++) {
    const vt_body_desc& B = sd->bodies[bi];
    vertBase[bi] = vbase;
    for (uint32_t k = 0; k < B.n_tris; k++) {
      uint32_t t = bb[bi].order[k];
      uint32_t m = B.tri_mesh[t];
      pack_tri(S->tris, S->blas[bi].tri_off + k, B.P, B.I, t, B.I[3 * t] + vbase, B.I[3 * t + 1] + vbase, B.I[3 * t + 2] + vbase, m, sd->meshes[m].flags);
      S->emitOfTri[S->blas[bi].tri_off + k] = emitIdx[bi][t];
    }
    vbase += B.n_verts;
  }
  S->vertCount = vbase;
  S->verts.assign(size_t(vbase) * 8, 0);
  float* V = reinterpret_cast<float*>(S->verts.data());
  std::vector<double> nodeArea(sd->n_static_verts, 0.0);
  const float* sP = sd->static_P;
  for (uint32_t k = 0; k < sd->n_static_tris; k++) {
    uint32_t a = sd->static_I[3 * k], b = sd->static_I[3 * k + 1], c = sd->static_I[3 * k + 2];
    double ux = double(sP[3 * b]) - sP[3 * a], uy = double(sP[3 * b + 1]) - sP[3 * a + 1], uz = double(sP[3 * b + 2]) - sP[3 * a + 2];
    double vx = double(sP[3 * c]) - sP[3 * a], vy = double(sP[3 * c + 1]) - sP[3 * a + 1], vz = double(sP[3 * c + 2]) - sP[3 * a + 2];
    double cx = uy * vz - uz * vy, cy = uz * vx - ux * vz, cz = ux * vy - uy * vx;
    double ar = 0.5 * std::sqrt(cx * cx + cy * cy + cz * cz) / 3;
    nodeArea[a] += ar; nodeArea[b] += ar; nodeArea[c] += ar;
  }
  for (uint32_t v = 0; v < sd->n_static_verts; v++) {
    float* o = V + size_t(v) * 8;
    o[0] = sP[3 * v]; o[1] = sP[3 * v + 1]; o[2] = sP[3 * v + 2];
    S->verts[size_t(v) * 8 + 3] = sd->static_vert_mesh[v];
    o[4] = sd->static_N[3 * v]; o[5] = sd->static_N[3 * v + 1]; o[6] = sd->static_N[3 * v + 2]; o[7] = float(nodeArea[v]);
  }
  for (uint32_t bi = 0; bi < sd->n_bodies; bi++) {
    const vt_body_desc& B = sd->bodies[bi];
    for (uint32_t v = 0; v < B.n_verts; v++) {
      float* o = V + size_t(vertBase[bi] + v) * 8;
      o[0] = B.P[3 * v]; o[1] = B.P[3 * v + 1]; o[2] = B.P[3 * v + 2]; o[3] = B.UV ? B.UV[2 * v] : 0.0f;
      o[4] = B.N[3 * v]; o[5] = B.N[3 * v + 1]; o[6] = B.N[3 * v + 2]; o[7] = B.UV ? B.UV[2 * v + 1] : 0.0f;
    }
  }
  // emitter (gpu/scene_gpu.js:395-423)
  double emitArea = 0;
  for (auto& e : emit) emitArea += e.area;
  double acc = 0;
  for (auto& e : emit) { acc += e.area; e.cdf = acc / (emitArea != 0 ? emitArea : 1); }
  double meanN[3] = {0, 0, 0};
  for (auto& e : emit) for (int k = 0; k < 3; k++) meanN[k] += e.n[k] * e.area;
  double ml = std::sqrt(meanN[0] * meanN[0] + meanN[1] * meanN[1] + meanN[2] * meanN[2]);
  if (!(ml > 0)) ml = 1;
  for (int k = 0; k < 3; k++) { S->emitNormal[k] = meanN[k] / ml; S->emitAxis[k] = S->emitNormal[k]; }
  if (std::isfinite(sd->axis_deg)) {
    double a = double(sd->axis_deg) * M_PI / 180;
    S->emitAxis[0] = 0; S->emitAxis[1] = std::sin(a); S->emitAxis[2] = std::cos(a);
  }
  S->scopeIndex = -1;
  for (uint32_t bi = 0; bi < sd->n_bodies; bi++) if (sd->bodies[bi].kind == VT_BODY_SCOPE) { S->scopeIndex = int(bi); break; }
  double scopeAhead = -INFINITY;
  if (!emit.empty()) {
    double c[3] = {0, 0, 0};
    for (auto& e : emit) for (int k = 0; k < 3; k++) c[k] += e.v0[k] * e.area;
    for (int k = 0; k < 3; k++) c[k] /= (emitArea != 0 ? emitArea : 1);
    for (uint32_t bi = 0; bi < sd->n_bodies; bi++) {
      if (sd->bodies[bi].kind != VT_BODY_SCOPE) continue;
      const vt_body_desc& B = sd->bodies[bi];
      for (uint32_t v = 0; v < B.n_verts; v++) {
        double d = (B.P[3 * v] - c[0]) * S->emitNormal[0] + (B.P[3 * v + 1] - c[1]) * S->emitNormal[1] + (B.P[3 * v + 2] - c[2]) * S->emitNormal[2];
        scopeAhead = std::max(scopeAhead, d);
      }
    }
  }
  S->scopeAhead = scopeAhead;
  S->shadowSkipsScope = scopeAhead <= 1e-6;
  for (int k = 0; k < 3; k++) S->centroid[k] = 0;
  for (auto& e : emit) for (int k = 0; k < 3; k++) S->centroid[k] += (e.v0[k] + (e.e1[k] + e.e2[k]) / 3) * e.area / (emitArea != 0 ? emitArea : 1);
  double radius = 0;
  for (auto& e : emit) {
    double q[3][3];
    for (int k = 0; k < 3; k++) { q[0][k] = e.v0[k]; q[1][k] = e.v0[k] + e.e1[k]; q[2][k] = e.v0[k] + e.e2[k]; }
    for (int j = 0; j < 3; j++) {
      double dx = q[j][0] - S->centroid[0], dy = q[j][1] - S->centroid[1], dz = q[j][2] - S->centroid[2];
      radius = std::max(radius, std::sqrt(dx * dx + dy * dy + dz * dz));
    }
  }
  S->radius = radius;
  S->emitArea = emitArea;
  for (const auto& e : emit) {
    for (int k = 0; k < 3; k++) S->emitTris.push_back(e.v0[k]);
    for (int k = 0; k < 3; k++) S->emitTris.push_back(e.e1[k]);
    for (int k = 0; k < 3; k++) S->emitTris.push_back(e.e2[k]);
    for (int k = 0; k < 3; k++) S->emitTris.push_back(e.n[k]);
    S->emitTris.push_back(e.area);
    S->emitTris.push_back(e.cdf);
  }
  // capsules, rhoEff (gpu/scene_gpu.js:427-456): overview_only meshes (outside the cavity) are left out of the
  // occlusion capsule and the effective albedo
  for (uint32_t bi = 0; bi < sd->n_bodies; bi++) {
    const vt_body_desc& B = sd->bodies[bi];
    Blas& bl = S->blas[bi];
    fit_capsule(B.P, B.n_verts, bl.cap_a, bl.cap_b, bl.cap_r);
    std::vector<char> used(B.n_verts, 0);
    bool dropped = false;
    for (uint32_t t = 0; t < B.n_tris; t++) {
      if (sd->meshes[B.tri_mesh[t]].overview_only) { dropped = true; continue; }
      used[B.I[3 * t]] = used[B.I[3 * t + 1]] = used[B.I[3 * t + 2]] = 1;
    }
    if (!dropped) {
      for (int k = 0; k < 3; k++) { bl.occ_a[k] = bl.cap_a[k]; bl.occ_b[k] = bl.cap_b[k]; }
      bl.occ_r = bl.cap_r;
    } else {
      std::vector<float> kept;
      for (uint32_t v = 0; v < B.n_verts; v++)
        if (used[v]) { kept.push_back(B.P[3 * v]); kept.push_back(B.P[3 * v + 1]); kept.push_back(B.P[3 * v + 2]); }
      if (kept.empty()) { for (int k = 0; k < 3; k++) bl.occ_a[k] = bl.occ_b[k] = 0; bl.occ_r = 0; }
      else fit_capsule(kept.data(), kept.size() / 3, bl.occ_a, bl.occ_b, bl.occ_r);
    }
    double ar = 0, rho = 0;
    for (uint32_t t = 0; t < B.n_tris; t++) {
      if (dropped && sd->meshes[B.tri_mesh[t]].overview_only) continue;
      size_t a = size_t(B.I[3 * t]) * 3, c = size_t(B.I[3 * t + 1]) * 3, d = size_t(B.I[3 * t + 2]) * 3;
      double ux = double(B.P[c]) - B.P[a], uy = double(B.P[c + 1]) - B.P[a + 1], uz = double(B.P[c + 2]) - B.P[a + 2];
      double vx = double(B.P[d]) - B.P[a], vy = double(B.P[d + 1]) - B.P[a + 1], vz = double(B.P[d + 2]) - B.P[a + 2];
      double cx = uy * vz - uz * vy, cy = uz * vx - ux * vz, cz = ux * vy - uy * vx;
      double A = 0.5 * std::sqrt(cx * cx + cy * cy + cz * cz);
      const Mat& m = S->mats[sd->meshes[B.tri_mesh[t]].mat];
      double hh0 = m.has_table ? m.hh[0] : 0, hh1 = m.has_table ? m.hh[1] : 0, hh2 = m.has_table ? m.hh[2] : 0;
      ar += A; rho += A * (0.2126 * hh0 + 0.7152 * hh1 + 0.0722 * hh2);
    }
    bl.rho_eff = ar != 0 ? rho / ar : 0;
  }
  // params (gpu/renderer.js:273-306)
  uint32_t nMesh = sd->n_meshes, nMat = sd->n_materials;
  uint32_t emitN = std::max<uint32_t>(1, uint32_t(emit.size())), profN = std::max<uint32_t>(2, sd->n_profile);
  S->meshOff = 0; S->matOff = 2 * nMesh; S->albOff = S->matOff + 5 * nMat; S->profOff = S->albOff + nMat * VT_ALBEDO_BINS * 2;
  S->emitOff = S->profOff + profN; S->profN = profN; S->emitN = emitN;
  uint32_t nVec = S->emitOff + 4 * emitN;
  S->params.assign(size_t(nVec) * 4, 0.0f);
  float* P = S->params.data();
  for (uint32_t i = 0; i < nMesh; i++) {
    float* o = P + (S->meshOff + 2 * i) * 4;
    const vt_mesh& m = sd->meshes[i];
    const Mat& mat = S->mats[m.mat];
    (void)mat;
    o[0] = m.build_dir[0]; o[1] = m.build_dir[1]; o[2] = m.build_dir[2]; o[3] = as_f(m.mat);
    o[4] = as_f(m.flags); o[5] = m.layer_period; o[6] = m.layer_depth;
  }
  for (uint32_t i = 0; i < nMat; i++) {
    float* o = P + (S->matOff + 5 * i) * 4;
    const Mat& m = S->mats[i];
    const double* c = m.metallic ? m.f0 : m.rho;
    float vals[8] = {float(c[0]), float(c[1]), float(c[2]), float(m.alpha), float(m.ior), float(m.metallic), float(m.fbar), float(m.roughness)};
    std::memcpy(o, vals, sizeof(vals));
    float v2[8] = {float(m.has_table ? m.hh[0] : 0), float(m.has_table ? m.hh[1] : 0), float(m.has_table ? m.hh[2] : 0), 0,
                   float(m.has_table ? m.hhSpec[0] : 0), float(m.has_table ? m.hhSpec[1] : 0), float(m.has_table ? m.hhSpec[2] : 0), m.emitter ? 1.0f : 0.0f};
    std::memcpy(o + 8, v2, sizeof(v2));
    if (m.coated) { o[16] = float(m.tau[0]); o[17] = float(m.tau[1]); o[18] = float(m.tau[2]); o[19] = float(m.alphaC); }
    else if (m.textured) { o[16] = float(m.ink[0]); o[17] = float(m.ink[1]); o[18] = float(m.ink[2]); o[19] = float(m.roughInk * m.roughInk); }
    if (m.has_table) for (int b = 0; b < VT_ALBEDO_BINS; b++) {
      float* q = P + (S->albOff + (i * VT_ALBEDO_BINS + b) * 2) * 4;
      q[0] = float(m.spec[3 * b]); q[1] = float(m.spec[3 * b + 1]); q[2] = float(m.spec[3 * b + 2]);
      q[4] = float(m.diff[3 * b]); q[5] = float(m.diff[3 * b + 1]); q[6] = float(m.diff[3 * b + 2]);
    }
  }
  for (uint32_t k = 0; k < profN; k++) {
    double th, p;
    if (sd->n_profile) { uint32_t j = std::min(k, sd->n_profile - 1); th = sd->profile_theta[j]; p = sd->profile_p[j]; }
    else { th = k ? M_PI / 2 : 0; p = 1; }
    float* o = P + (S->profOff + k) * 4;
    o[0] = float(th); o[1] = float(p);
  }
  for (size_t k = 0; k < emit.size(); k++) {
    float* o = P + (S->emitOff + 4 * k) * 4;
    const EmitTri& e = emit[k];
    float vals[16] = {float(e.v0[0]), float(e.v0[1]), float(e.v0[2]), float(e.cdf), float(e.e1[0]), float(e.e1[1]), float(e.e1[2]), 0,
                      float(e.e2[0]), float(e.e2[1]), float(e.e2[2]), 0, float(e.n[0]), float(e.n[1]), float(e.n[2]), float(e.area)};
    std::memcpy(o, vals, sizeof(vals));
  }
  for (int k = 0; k < 3; k++) S->L0[k] = sd->L0[k];
  for (uint32_t k = 0; k < sd->n_profile; k++) { S->profTheta.push_back(sd->profile_theta[k]); S->profP.push_back(sd->profile_p[k]); }
  S->cams.assign(sd->cameras, sd->cameras + sd->n_cameras);
  S->nodeState.assign(size_t(sd->n_static_verts) * 16, 0.0f);
  for (uint32_t i = 0; i < sd->n_static_verts; i++) { S->nodeState[16 * i + 3] = 1; S->nodeState[16 * i + 15] = -1; }
  S->inst.assign(sd->n_bodies, Scene::Pose4{});
  return S;
}

// ---------------------------------------------------------------------------------------- poses (renderer.js)

// gpu/renderer.js:70 quatFromMat (column-major 4x4)
static void quat_from_mat(const double* m, double q[4]) {
  double r00 = m[0], r10 = m[1], r20 = m[2], r01 = m[4], r11 = m[5], r21 = m[6], r02 = m[8], r12 = m[9], r22 = m[10];
  double tr = r00 + r11 + r22, x, y, z, w;
  if (tr > 0) { double s = std::sqrt(tr + 1) * 2; w = 0.25 * s; x = (r21 - r12) / s; y = (r02 - r20) / s; z = (r10 - r01) / s; }
  else if (r00 > r11 && r00 > r22) { double s = std::sqrt(1 + r00 - r11 - r22) * 2; w = (r21 - r12) / s; x = 0.25 * s; y = (r01 + r10) / s; z = (r02 + r20) / s; }
  else if (r11 > r22) { double s = std::sqrt(1 + r11 - r00 - r22) * 2; w = (r02 - r20) / s; x = (r01 + r10) / s; y = 0.25 * s; z = (r12 + r21) / s; }
  else { double s = std::sqrt(1 + r22 - r00 - r11) * 2; w = (r10 - r01) / s; x = (r02 + r20) / s; y = (r12 + r21) / s; z = 0.25 * s; }
  double l = std::sqrt(x * x + y * y + z * z + w * w);
  q[0] = x / l; q[1] = y / l; q[2] = z / l; q[3] = w / l;
}
// gpu/renderer.js:81 quatMat, :85 slerpJS
static void quat_mat(const double q[4], double R[3][3]) {
  double x = q[0], y = q[1], z = q[2], w = q[3];
  R[0][0] = 1 - 2 * (y * y + z * z); R[0][1] = 2 * (x * y - z * w); R[0][2] = 2 * (x * z + y * w);
  R[1][0] = 2 * (x * y + z * w); R[1][1] = 1 - 2 * (x * x + z * z); R[1][2] = 2 * (y * z - x * w);
  R[2][0] = 2 * (x * z - y * w); R[2][1] = 2 * (y * z + x * w); R[2][2] = 1 - 2 * (x * x + y * y);
}
static void slerp_js(const double a[4], const double b[4], double t, double out[4]) {
  double c = a[0] * b[0] + a[1] * b[1] + a[2] * b[2] + a[3] * b[3];
  double bb[4] = {b[0], b[1], b[2], b[3]};
  if (c < 0) { for (double& q : bb) q = -q; c = -c; }
  if (c > 0.9995) {
    double r[4], l = 0;
    for (int i = 0; i < 4; i++) { r[i] = a[i] + (bb[i] - a[i]) * t; l += r[i] * r[i]; }
    l = std::sqrt(l);
    for (int i = 0; i < 4; i++) out[i] = r[i] / l;
    return;
  }
  double th = std::acos(c), s = std::sin(th);
  for (int i = 0; i < 4; i++) out[i] = (a[i] * std::sin((1 - t) * th) + bb[i] * std::sin(t * th)) / s;
}
static bool pose_at(const Scene& S, int i, double t, double R[3][3], double p[3]) {
  const Scene::Pose4& I = S.inst[i];
  if (!I.valid) return false;
  double q[4];
  slerp_js(I.q0, I.q1, t, q);
  quat_mat(q, R);
  for (int k = 0; k < 3; k++) p[k] = I.p0[k] + (I.p1[k] - I.p0[k]) * t;
  return true;
}
static void mul_rv(const double R[3][3], const double* v, double* o) {
  for (int i = 0; i < 3; i++) o[i] = R[i][0] * v[0] + R[i][1] * v[1] + R[i][2] * v[2];
}
// gpu/renderer.js:642-705 _writeSceneU (no cut plane; no ports: cavityCapsule keeps the capsule except fixed/board)
static void write_scene_u(Scene& S, uint32_t slot, uint32_t frame) {
  float* f = S.sceneU;
  uint32_t* u = reinterpret_cast<uint32_t*>(f);
  std::fill(f, f + 24 + 48 * VT_MAX_INST, 0.0f);
  f[0] = S.L0[0]; f[1] = S.L0[1]; f[2] = S.L0[2]; f[3] = S.emitArea != 0 ? float(S.emitArea) : 1e-12f;
  f[4] = float(S.emitAxis[0]); f[5] = float(S.emitAxis[1]); f[6] = float(S.emitAxis[2]);
  u[7] = (S.shadowSkipsScope && S.scopeIndex >= 0) ? (1u << S.scopeIndex) : 0u;
  f[8] = float(S.eAvg[0]); f[9] = float(S.eAvg[1]); f[10] = float(S.eAvg[2]); f[11] = 5e-4f;
  f[12] = 0; f[13] = 0; f[14] = 0; f[15] = 1e30f;
  u[16] = uint32_t(S.blas.size()); u[17] = S.scopeIndex < 0 ? 0 : uint32_t(S.scopeIndex); u[18] = slot ? slot : 1; u[19] = frame;
  f[20] = float(S.centroid[0]); f[21] = float(S.centroid[1]); f[22] = float(S.centroid[2]); f[23] = float(S.radius);
  for (size_t i = 0; i < S.blas.size(); i++) {
    size_t o = 24 + 48 * i;
    const Blas& bl = S.blas[i];
    const Scene::Pose4& I = S.inst[i];
    if (!I.valid) { u[o + 15] = 2; u[o + 11] = bl.root; continue; }
    for (int k = 0; k < 4; k++) { f[o + k] = float(I.q0[k]); f[o + 4 + k] = float(I.q1[k]); }
    for (int k = 0; k < 3; k++) { f[o + 8 + k] = float(I.p0[k]); f[o + 12 + k] = float(I.p1[k]); }
    u[o + 11] = bl.root;
    bool moving = false;
    for (int k = 0; k < 4; k++) if (I.q0[k] != I.q1[k]) moving = true;
    for (int k = 0; k < 3; k++) if (I.p0[k] != I.p1[k]) moving = true;
    u[o + 15] = moving ? 1 : 0;
    double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    const double ts5[5] = {0, 0.25, 0.5, 0.75, 1};
    int nts = moving ? 5 : 1;
    for (int ti = 0; ti < nts; ti++) {
      double R[3][3], p[3];
      pose_at(S, int(i), ts5[ti], R, p);
      for (int c = 0; c < 8; c++) {
        double v[3] = {(c & 1) ? bl.bmax[0] : bl.bmin[0], (c & 2) ? bl.bmax[1] : bl.bmin[1], (c & 4) ? bl.bmax[2] : bl.bmin[2]}, w[3];
        mul_rv(R, v, w);
        for (int k = 0; k < 3; k++) { lo[k] = std::min(lo[k], w[k] + p[k]); hi[k] = std::max(hi[k], w[k] + p[k]); }
      }
    }
    double pad = moving ? 1e-3 : 1e-6;
    for (int k = 0; k < 3; k++) { f[o + 16 + k] = float(lo[k] - pad); f[o + 20 + k] = float(hi[k] + pad); }
    double R[3][3], p[3];
    pose_at(S, int(i), 0.5, R, p);
    double ca[3], cb[3], oa[3], ob[3];
    mul_rv(R, bl.occ_a, oa); mul_rv(R, bl.occ_b, ob);
    for (int k = 0; k < 3; k++) { oa[k] += p[k]; ob[k] += p[k]; }
    double cr = (bl.kind == VT_BODY_FIXED || bl.kind == VT_BODY_BOARD) ? 0 : bl.occ_r;
    for (int k = 0; k < 3; k++) { f[o + 24 + k] = float(oa[k]); f[o + 28 + k] = float(ob[k]); }
    f[o + 27] = float(cr); f[o + 31] = float(bl.rho_eff);
    mul_rv(R, bl.cap_a, ca); mul_rv(R, bl.cap_b, cb);
    for (int k = 0; k < 3; k++) { ca[k] += p[k]; cb[k] += p[k]; }
    double motion = 0;
    if (moving) {
      double R0[3][3], p0[3], R1[3][3], p1[3];
      pose_at(S, int(i), 0, R0, p0); pose_at(S, int(i), 1, R1, p1);
      const double* vs[2] = {bl.cap_a, bl.cap_b};
      for (int vi = 0; vi < 2; vi++) for (int qi = 0; qi < 2; qi++) {
        double w[3], m[3];
        mul_rv(qi ? R1 : R0, vs[vi], w);
        mul_rv(R, vs[vi], m);
        for (int k = 0; k < 3; k++) { w[k] += qi ? p1[k] : p0[k]; m[k] += p[k]; }
        motion = std::max(motion, std::sqrt((w[0] - m[0]) * (w[0] - m[0]) + (w[1] - m[1]) * (w[1] - m[1]) + (w[2] - m[2]) * (w[2] - m[2])));
      }
      motion *= 1.5;
    }
    float bc[8] = {float(ca[0]), float(ca[1]), float(ca[2]), float(bl.cap_r * 1.0001 + 1e-6 + motion), float(cb[0]), float(cb[1]), float(cb[2]), 0};
    const bool havePc = S.solvedCaps.size() >= 8 * (i + 1) && !std::isnan(S.solvedCaps[8 * i]);
    for (int k = 0; k < 8; k++) { f[o + 32 + k] = bc[k]; f[o + 40 + k] = havePc ? S.solvedCaps[8 * i + k] : bc[k]; }
  }
}
static void set_poses(Scene& S, const double* T0, const double* T1, uint32_t nb) {
  for (uint32_t i = 0; i < S.blas.size(); i++) {
    Scene::Pose4& I = S.inst[i];
    I.valid = false;
    if (S.blas[i].kind == VT_BODY_FIXED) {
      I.valid = true;
      for (int k = 0; k < 4; k++) I.q0[k] = I.q1[k] = (k == 3);
      for (int k = 0; k < 3; k++) I.p0[k] = I.p1[k] = 0;
      continue;
    }
    if (i >= nb || !T0 || std::isnan(T0[16 * i])) continue;
    const double* A = T0 + 16 * i;
    const double* B = (T1 && !std::isnan(T1[16 * i])) ? T1 + 16 * i : A;
    quat_from_mat(A, I.q0); quat_from_mat(B, I.q1);
    for (int k = 0; k < 3; k++) { I.p0[k] = A[12 + k]; I.p1[k] = B[12 + k]; }
    I.valid = true;
  }
}

// ============================================================================================ tracing (WGSL, R)

template <typename R> struct Hit { R t, u, v; uint32_t tri, inst; };

struct Dbg { uint64_t c[16] = {0}; };

template <typename R> struct Tracer {
  const Scene& S;
  Dbg& dbg;
  uint32_t gRoot = 0;
  const float* N;   // nodes as floats
  const float* T;
  const float* V;
  const float* SU;
  Tracer(const Scene& s, Dbg& d) : S(s), dbg(d) {
    N = reinterpret_cast<const float*>(S.nodes.data());
    T = reinterpret_cast<const float*>(S.tris.data());
    V = reinterpret_cast<const float*>(S.verts.data());
    SU = S.sceneU;
  }
  uint32_t su_u(size_t i) const { return as_u(SU[i]); }
  const float* inst(uint32_t i) const { return SU + 24 + 48 * i; }

  // gpu/wgsl/trace.wgsl.js:178 slab, :188 safeInv
  static R slab(const V3<R>& lo, const V3<R>& hi, const V3<R>& o, const V3<R>& inv, R tmin, R tmax) {
    V3<R> t0 = (lo - o) * inv, t1 = (hi - o) * inv;
    R tnx = std::min(t0.x, t1.x), tny = std::min(t0.y, t1.y), tnz = std::min(t0.z, t1.z);
    R tfx = std::max(t0.x, t1.x), tfy = std::max(t0.y, t1.y), tfz = std::max(t0.z, t1.z);
    R a = std::max(std::max(tnx, tny), std::max(tnz, tmin));
    R b = std::min(std::min(tfx, tfy), std::min(tfz, tmax));
    return a <= b ? a : R(BIGD);
  }
  static V3<R> safe_inv(const V3<R>& d) {
    auto f = [](R x) { R s = x >= R(0) ? R(1) : R(-1); return s / std::max(std::fabs(x), R(1e-20)); };
    return V3<R>(f(d.x), f(d.y), f(d.z));
  }
  // gpu/wgsl/trace.wgsl.js:195 triHit
  bool tri_hit(uint32_t k, const V3<R>& o, const V3<R>& d, R tmin, R tmax, R& t, R& u, R& v) const {
    const float* r = T + size_t(k) * 16;
    V3<R> v0 = ld3<R>(r), e1 = ld3<R>(r + 4), e2 = ld3<R>(r + 8);
    V3<R> p = cross(d, e2);
    R det = dot(e1, p);
    if (std::fabs(det) < R(1e-30)) return false;
    R inv = R(1) / det;
    V3<R> s = o - v0;
    u = dot(s, p) * inv;
    if (u < R(0) || u > R(1)) return false;
    V3<R> q = cross(s, e1);
    v = dot(d, q) * inv;
    if (v < R(0) || u + v > R(1)) return false;
    t = dot(e2, q) * inv;
    if (t <= tmin || t >= tmax) return false;
    return true;
  }
  // gpu/wgsl/trace.wgsl.js:215-277 traverse (32-entry stack, 2048-visit cap, 64-triangle leaf cap)
  bool traverse(uint32_t root, const V3<R>& o, const V3<R>& d, R tmin, Hit<R>& best, bool anyHit, uint32_t instI) const {
    V3<R> inv = safe_inv(d);
    uint32_t stN[32];
    R stT[32];
    uint32_t sp = 0, node = root, visits = 0;
    const uint32_t* NU = S.nodes.data();
    for (;;) {
      visits++;
      if (visits > 2048u) { dbg.c[0]++; break; }
      dbg.c[8]++;   // node fetched (64 B)
      if (!anyHit) dbg.c[11]++;   // ... by a closest-hit query
      const float* a = N + size_t(node) * 16;
      R t0 = slab(ld3<R>(a), ld3<R>(a + 4), o, inv, tmin, best.t);
      R t1 = slab(ld3<R>(a + 8), ld3<R>(a + 12), o, inv, tmin, best.t);
      uint32_t c0 = NU[size_t(node) * 16 + 7], c1 = NU[size_t(node) * 16 + 15];
      uint32_t r0 = NU[size_t(node) * 16 + 3], r1 = NU[size_t(node) * 16 + 11];
      for (int c = 0; c < 2; c++) {
        R tc = c == 0 ? t0 : t1;
        uint32_t cnt = c == 0 ? c0 : c1, ref0 = c == 0 ? r0 : r1;
        if (tc < best.t && cnt > 0) {
          if (cnt > 64u) dbg.c[1]++;
          for (uint32_t k = ref0; k < ref0 + std::min(cnt, 64u); k++) {
            R t, u, v;
            dbg.c[9]++;   // triangle tested (v0, e1, e2: 48 B)
            if (!anyHit) dbg.c[12]++;
            if (tri_hit(k, o, d, tmin, best.t, t, u, v) && t < best.t) {
              best.t = t; best.tri = k; best.u = u; best.v = v; best.inst = instI;
              if (anyHit) return true;
            }
          }
          if (c == 0) t0 = R(BIGD); else t1 = R(BIGD);
        }
      }
      t0 = t0 < best.t ? t0 : R(BIGD);
      t1 = t1 < best.t ? t1 : R(BIGD);
      if ((t0 < R(BIGD) && c0 == 0 && r0 <= node) || (t1 < R(BIGD) && c1 == 0 && r1 <= node)) { dbg.c[6]++; break; }
      bool go0 = t0 < R(BIGD), go1 = t1 < R(BIGD);
      if (go0 && go1) {
        if (t1 < t0) { stN[sp] = r0; stT[sp] = t0; node = r1; }
        else { stN[sp] = r1; stT[sp] = t1; node = r0; }
        sp = std::min(sp + 1u, 31u);
      } else if (go0) node = r0;
      else if (go1) node = r1;
      else {
        bool found = false;
        for (uint32_t pops = 0; pops <= 32; pops++) {
          if (sp == 0) break;
          sp--;
          if (stT[sp] < best.t) { node = stN[sp]; found = true; break; }
        }
        if (!found) break;
      }
    }
    return false;
  }
  // gpu/wgsl/common.wgsl.js:117-143 quatToMat, slerp, instPose
  static M3<R> quat_to_mat(const R q[4]) {
    R x = q[0], y = q[1], z = q[2], w = q[3];
    M3<R> m;
    m.c[0] = V3<R>(R(1) - R(2) * (y * y + z * z), R(2) * (x * y + z * w), R(2) * (x * z - y * w));
    m.c[1] = V3<R>(R(2) * (x * y - z * w), R(1) - R(2) * (x * x + z * z), R(2) * (y * z + x * w));
    m.c[2] = V3<R>(R(2) * (x * z + y * w), R(2) * (y * z - x * w), R(1) - R(2) * (x * x + y * y));
    return m;
  }
  static void slerp(const R a[4], const R b0[4], R t, R out[4]) {
    R b[4] = {b0[0], b0[1], b0[2], b0[3]};
    R c = a[0] * b[0] + a[1] * b[1] + a[2] * b[2] + a[3] * b[3];
    if (c < R(0)) { for (R& q : b) q = -q; c = -c; }
    if (c > R(0.9995)) {
      R r[4], l = 0;
      for (int i = 0; i < 4; i++) { r[i] = a[i] * (R(1) - t) + b[i] * t; l += r[i] * r[i]; }
      l = std::sqrt(l);
      for (int i = 0; i < 4; i++) out[i] = r[i] / l;
      return;
    }
    R th = std::acos(c), s = std::sin(th);
    for (int i = 0; i < 4; i++) out[i] = (a[i] * std::sin((R(1) - t) * th) + b[i] * std::sin(t * th)) / s;
  }
  void inst_pose(uint32_t i, R time, M3<R>& M, V3<R>& p) const {
    const float* I = inst(i);
    R q0[4] = {I[0], I[1], I[2], I[3]};
    if (as_u(I[15]) & 1u) {
      R q1[4] = {I[4], I[5], I[6], I[7]}, q[4];
      slerp(q0, q1, time, q);
      M = quat_to_mat(q);
      p = mixv(ld3<R>(I + 8), ld3<R>(I + 12), time);
      return;
    }
    M = quat_to_mat(q0);
    p = ld3<R>(I + 8);
  }
  // gpu/wgsl/trace.wgsl.js:280 segNearCapsule
  static bool seg_near_capsule(const V3<R>& o, const V3<R>& d, R t0, R t1, const V3<R>& a, const V3<R>& b, R r) {
    V3<R> p0 = o + d * t0, u = d * (t1 - t0), v = b - a, w = p0 - a;
    R A = dot(u, u), B = dot(u, v), C = dot(v, v), D = dot(u, w), E = dot(v, w);
    R den = A * C - B * B;
    R s = 0;
    if (den > R(1e-20) * A * C) s = clampR((B * E - C * D) / den, R(0), R(1));
    R t = C > R(1e-30) ? (B * s + E) / C : R(0);
    if (t < R(0)) { t = 0; s = clampR(-D / std::max(A, R(1e-30)), R(0), R(1)); }
    else if (t > R(1)) { t = 1; s = clampR((B - D) / std::max(A, R(1e-30)), R(0), R(1)); }
    V3<R> q = (p0 + u * s) - (a + v * t);
    return dot(q, q) <= r * r;
  }
  // the hit of a ray on a given triangle's plane (instance `inst` posed at `time`, MISS: static), with no range test
  // on t, u, v: the frozen replay of a path whose hit triangles are fixed (checks of the intrinsics' derivative)
  Hit<R> frozen_hit(uint32_t tri, uint32_t inst, const V3<R>& o, const V3<R>& d, R time) const {
    V3<R> ol = o, dl = d;
    if (inst != MISS) {
      M3<R> M; V3<R> p;
      inst_pose(inst, time, M, p);
      ol = M.tmul(o - p); dl = M.tmul(d);
    }
    const float* r = T + size_t(tri) * 16;
    V3<R> v0 = ld3<R>(r), e1 = ld3<R>(r + 4), e2 = ld3<R>(r + 8);
    V3<R> pv = cross(dl, e2);
    R inv = R(1) / dot(e1, pv);
    V3<R> sv = ol - v0;
    V3<R> qv = cross(sv, e1);
    return Hit<R>{dot(e2, qv) * inv, dot(sv, pv) * inv, dot(dl, qv) * inv, tri, inst};
  }
  // gpu/wgsl/trace.wgsl.js:302 traceSceneSkip
  Hit<R> trace(const V3<R>& o, const V3<R>& d, R tmin, R tmax, R time, bool anyHit, uint32_t mask, uint32_t skip) const {
    Hit<R> best{tmax, 0, 0, MISS, MISS};
    if (mask & 1u) dbg.c[anyHit ? 14 : 13]++;   // rays: closest-hit (13) and any-hit (14) queries
    if (mask & 1u) if (traverse(gRoot, o, d, tmin, best, anyHit, MISS)) return best;
    if (mask & 2u) {
      V3<R> inv = safe_inv(d);
      uint32_t n = std::min<uint32_t>(su_u(16), VT_MAX_INST);
      for (uint32_t i = 0; i < n; i++) {
        const float* I = inst(i);
        if ((as_u(I[15]) & 2u) || ((skip >> i) & 1u)) continue;
        if (slab(ld3<R>(I + 16), ld3<R>(I + 20), o, inv, tmin, best.t) >= best.t) continue;
        if (!seg_near_capsule(o, d, tmin, std::min(best.t, R(1e3)), ld3<R>(I + 32), ld3<R>(I + 36), R(I[35]))) continue;
        M3<R> M; V3<R> p;
        inst_pose(i, time, M, p);
        V3<R> ol = M.tmul(o - p), dl = M.tmul(d);
        if (traverse(as_u(I[11]), ol, dl, tmin, best, anyHit, i)) return best;
      }
    }
    return best;
  }
};

// ============================================================================================ shading (WGSL, R)

template <typename R> struct Surf { V3<R> p, ng, ns, b; uint32_t vi[3], mesh, flags, mat, inst; };

template <typename R> struct Shader {
  Tracer<R>& tr;
  const Scene& S;
  const float* P;     // params
  const float* NS;    // node state
  mutable bool shadowTraced = false;   // a light sample of the current vertex reached its shadow ray
  Shader(Tracer<R>& t) : tr(t), S(t.S), P(t.S.params.data()), NS(t.S.nodeState.data()) {}
  const float* pv(uint32_t i) const { return P + size_t(i) * 4; }
  const float* vert(uint32_t i, int row) const { return tr.V + size_t(i) * 8 + row * 4; }

  // gpu/wgsl/trace.wgsl.js:330 surface
  Surf<R> surface(const Hit<R>& h, const V3<R>& o, const V3<R>& d, R time) const {
    tr.dbg.c[10]++;   // a shaded hit
    Surf<R> s;
    const float* r = tr.T + size_t(h.tri) * 16;
    const uint32_t* ru = S.tris.data() + size_t(h.tri) * 16;
    s.vi[0] = ru[3]; s.vi[1] = ru[7]; s.vi[2] = ru[11];
    s.mesh = ru[12]; s.flags = ru[13];
    s.b = V3<R>(R(1) - h.u - h.v, h.u, h.v);
    V3<R> ng = normalize(cross(ld3<R>(r + 4), ld3<R>(r + 8)));
    V3<R> ns = normalize(ld3<R>(vert(s.vi[0], 1)) * s.b.x + ld3<R>(vert(s.vi[1], 1)) * s.b.y + ld3<R>(vert(s.vi[2], 1)) * s.b.z);
    if (h.inst != MISS) {
      M3<R> M; V3<R> p;
      tr.inst_pose(h.inst, time, M, p);
      ng = M.mul(ng); ns = M.mul(ns);
    }
    if (dot(ng, d) > R(0)) ng = -ng;
    if (dot(ns, ng) < R(0)) ns = -ns;
    if (dot(ns, -d) < R(1e-4)) ns = ng;
    s.ng = ng; s.ns = ns;
    s.mat = as_u(pv(S.meshOff + 2 * s.mesh)[3]);
    s.inst = h.inst;
    s.p = o + d * h.t;
    return s;
  }
  MatR<R> load_mat(uint32_t m) const {
    const float* a = pv(S.matOff + 5 * m);
    MatR<R> M;
    M.c = ld3<R>(a); M.alpha = a[3]; M.ior = a[4]; M.metal = a[5]; M.fbar = a[6]; M.rough = a[7];
    M.hh = ld3<R>(a + 8); M.hhSpec = ld3<R>(a + 12);
    M.x[0] = a[16]; M.x[1] = a[17]; M.x[2] = a[18]; M.x[3] = a[19]; M.idx = m;
    return M;
  }
  // gpu/wgsl/bsdf.wgsl.js:158 albedoSpec / albedoDiff
  V3<R> albedo(uint32_t m, R mu, int which) const {
    R x = clampR(mu * R(VT_ALBEDO_BINS) - R(0.5), R(0), R(VT_ALBEDO_BINS - 1));
    uint32_t i = uint32_t(std::floor(x));
    uint32_t j = std::min<uint32_t>(VT_ALBEDO_BINS - 1, i + 1);
    R f = x - R(i);
    uint32_t base = S.albOff + m * VT_ALBEDO_BINS * 2;
    return mixv(ld3<R>(pv(base + 2 * i + which)), ld3<R>(pv(base + 2 * j + which)), f);
  }
  V3<R> albedo_all(uint32_t m, R mu) const { return albedo(m, mu, 0) + albedo(m, mu, 1); }
  // gpu/wgsl/shade.wgsl.js:12 profile
  R profile(R th) const {
    const float* last = pv(S.profOff + S.profN - 1);
    if (th >= R(last[0])) return th == R(last[0]) ? R(last[1]) : R(0);
    uint32_t lo = 0, hi = S.profN - 1;
    for (uint32_t it = 0; it < 40; it++) {
      if (hi - lo <= 1) break;
      uint32_t m = (lo + hi) / 2;
      if (R(pv(S.profOff + m)[0]) <= th) lo = m; else hi = m;
    }
    const float* a = pv(S.profOff + lo);
    const float* b = pv(S.profOff + hi);
    R f = clampR((th - R(a[0])) / std::max(R(b[0]) - R(a[0]), R(1e-12)), R(0), R(1));
    return R(a[1]) * (R(1) - f) + R(b[1]) * f;
  }
  // gpu/wgsl/shade.wgsl.js:31 sampleEmitter
  void sample_emitter(const V3<R>& u, R time, V3<R>& p, V3<R>& n, V3<R>& axis) const {
    uint32_t lo = 0, hi = S.emitN - 1;
    for (uint32_t it = 0; it < 40; it++) {
      if (lo >= hi) break;
      uint32_t m = (lo + hi) / 2;
      if (R(pv(S.emitOff + 4 * m)[3]) < u.x) lo = m + 1; else hi = m;
    }
    V3<R> v0 = ld3<R>(pv(S.emitOff + 4 * lo)), e1 = ld3<R>(pv(S.emitOff + 4 * lo + 1)), e2 = ld3<R>(pv(S.emitOff + 4 * lo + 2));
    V3<R> nl = ld3<R>(pv(S.emitOff + 4 * lo + 3));
    R su = std::sqrt(u.y);
    V3<R> pl = v0 + e1 * (su * (R(1) - u.z)) + e2 * (su * u.z);
    M3<R> M; V3<R> pp;
    tr.inst_pose(tr.su_u(17), time, M, pp);
    p = M.mul(pl) + pp; n = M.mul(nl); axis = M.mul(ld3<R>(tr.SU + 4));
  }
  // gpu/wgsl/shade.wgsl.js:50 emitted
  V3<R> emitted(const V3<R>& n, const V3<R>& axis, const V3<R>& w) const {
    if (dot(w, n) <= R(0)) return V3<R>();
    return ld3<R>(tr.SU) * profile(std::acos(clampR(dot(w, axis), R(-1), R(1))));
  }
  V3<R> emitter_axis_at(R time) const {
    M3<R> M; V3<R> p;
    tr.inst_pose(tr.su_u(17), time, M, p);
    return M.mul(ld3<R>(tr.SU + 4));
  }
  // gpu/wgsl/shade.wgsl.js:85 capsuleVis
  R capsule_vis(const V3<R>& p, const V3<R>& n) const {
    R v = 1;
    uint32_t cnt = std::min<uint32_t>(tr.su_u(16), VT_MAX_INST);
    for (uint32_t i = 0; i < cnt; i++) {
      const float* I = tr.inst(i);
      if (as_u(I[15]) & 2u) continue;
      R o = capsule_occ(p, n, ld3<R>(I + 24), ld3<R>(I + 28), R(I[27]));
      v = v - o * (R(1) - R(I[31]));
    }
    return clampR(v, R(0), R(1));
  }
  // gpu/wgsl/bsdf.wgsl.js:176 layerNormal: h(s) = depth/2 cos(2 pi s / period), s = p . bd, phase taken first
  static V3<R> layer_normal(const V3<R>& n, const V3<R>& p, const V3<R>& bd, R period, R depth) {
    R x = dot(p, bd) / period;
    R ph = x - std::floor(x);
    R dh = -(depth * R(0.5)) * (R(2) * R(M_PI) / period) * std::sin(R(2) * R(M_PI) * ph);
    V3<R> bt = bd - n * dot(bd, n);
    return normalize(n - bt * dh);
  }
  // gpu/wgsl/shade.wgsl.js:100 shadingNormal
  V3<R> shading_normal(const Surf<R>& s, uint32_t opts) const {
    if (!(opts & VT_O_LAYER) || !(s.flags & VT_F_LAYER)) return s.ns;
    const float* r0 = pv(S.meshOff + 2 * s.mesh);
    const float* r1 = pv(S.meshOff + 2 * s.mesh + 1);
    V3<R> n = layer_normal(s.ns, s.p, ld3<R>(r0), R(r1[1]), R(r1[2]));
    if (dot(n, s.ng) <= R(0)) n = s.ns;
    return n;
  }
  static V3<R> offset_ray(const V3<R>& p, const V3<R>& ng, const V3<R>& dir) {
    R s = dot(ng, dir) > R(0) ? R(1) : R(-1);
    return p + ng * (s * R(2e-6));
  }
  // gpu/wgsl/shade.wgsl.js:160 directLight (cached visibility off: every shadow ray traced)
  V3<R> direct_light(const Surf<R>& s, const V3<R>& n, const MatR<R>& M, const V3<R>& wo, R time, const V3<R>& u, bool mis, R nL) const {
    V3<R> lp, ln, la;
    sample_emitter(u, time, lp, ln, la);
    V3<R> wi = lp - s.p;
    R d2 = dot(wi, wi), dist = std::sqrt(d2);
    wi = wi / dist;
    R cosE = dot(-wi, ln);
    if (cosE <= R(0)) return V3<R>();
    R cosS = dot(n, wi);
    if (cosS <= R(0) || dot(s.ng, wi) <= R(0)) return V3<R>();
    V3<R> Le = emitted(ln, la, -wi);
    if (maxc(Le) <= R(0)) return V3<R>();
    V3<R> f = eval_bsdf(M, n, wi, wo);
    if (maxc(f) <= R(0)) return V3<R>();
    V3<R> o = offset_ray(s.p, s.ng, wi);
    shadowTraced = true;
    Hit<R> sh = tr.trace(o, wi, R(0), dist - R(2e-5), time, true, 3u, tr.su_u(7));
    if (sh.tri != MISS) return V3<R>();
    R pdfW = d2 / (cosE * R(tr.SU[3]));
    R w = 1;
    if (mis) {
      R pb = pdf_bsdf(M, n, wo, wi);
      w = nL * nL * pdfW * pdfW / (nL * nL * pdfW * pdfW + pb * pb);
    }
    return f * Le * (cosS * w / pdfW);
  }
  // gpu/wgsl/shade.wgsl.js:135 lightEval: the sample's contribution before the shadow test and its shadow segment
  bool light_eval(const Surf<R>& s, const V3<R>& n, const MatR<R>& M, const V3<R>& wo, R time, const V3<R>& u, bool mis, R nL,
                  V3<R>& c, V3<R>& o, V3<R>& wi, R& tmax) const {
    V3<R> lp, ln, la;
    sample_emitter(u, time, lp, ln, la);
    wi = lp - s.p;
    R d2 = dot(wi, wi), dist = std::sqrt(d2);
    wi = wi / dist;
    R cosE = dot(-wi, ln);
    if (cosE <= R(0)) return false;
    R cosS = dot(n, wi);
    if (cosS <= R(0) || dot(s.ng, wi) <= R(0)) return false;
    V3<R> Le = emitted(ln, la, -wi);
    if (maxc(Le) <= R(0)) return false;
    V3<R> f = eval_bsdf(M, n, wi, wo);
    if (maxc(f) <= R(0)) return false;
    R pdfW = d2 / (cosE * R(tr.SU[3]));
    R w = 1;
    if (mis) {
      R pb = pdf_bsdf(M, n, wo, wi);
      w = nL * nL * pdfW * pdfW / (nL * nL * pdfW * pdfW + pb * pb);
    }
    c = f * Le * (cosS * w / pdfW);
    o = offset_ray(s.p, s.ng, wi);
    tmax = dist - R(2e-5);
    return true;
  }
  // gpu/wgsl/shade.wgsl.js:194-209 nodeWeights / nodeEfree / nodeLout
  V3<R> node_weights(const uint32_t* vi, const V3<R>& b) const {
    uint32_t slot = tr.su_u(18);
    V3<R> w = b * V3<R>(NS[16 * vi[0] + 4 * slot + 3], NS[16 * vi[1] + 4 * slot + 3], NS[16 * vi[2] + 4 * slot + 3]);
    R sw = w.x + w.y + w.z;
    if (sw <= R(1e-6)) return b;
    return w / sw;
  }
  V3<R> node_efree(const uint32_t* vi, const V3<R>& b0) const {
    V3<R> b = node_weights(vi, b0);
    return ld3<R>(NS + 16 * vi[0]) * b.x + ld3<R>(NS + 16 * vi[1]) * b.y + ld3<R>(NS + 16 * vi[2]) * b.z;
  }
  V3<R> node_lout(const uint32_t* vi, const V3<R>& b0) const {
    uint32_t slot = tr.su_u(18);
    V3<R> b = node_weights(vi, b0);
    return ld3<R>(NS + 16 * vi[0] + 4 * slot) * b.x + ld3<R>(NS + 16 * vi[1] + 4 * slot) * b.y + ld3<R>(NS + 16 * vi[2] + 4 * slot) * b.z;
  }
  V3<R> emitter_normal(const Hit<R>& h, const Surf<R>& s, R time) const {
    V3<R> n = normalize(ld3<R>(vert(s.vi[0], 1)) * s.b.x + ld3<R>(vert(s.vi[1], 1)) * s.b.y + ld3<R>(vert(s.vi[2], 1)) * s.b.z);
    M3<R> M; V3<R> p;
    tr.inst_pose(h.inst, time, M, p);
    return M.mul(n);
  }
  // gpu/wgsl/shade.wgsl.js:224 secondary
  V3<R> secondary(const V3<R>& o, const V3<R>& l, R time, R pdfB, uint32_t opts, R nL) const {
    Hit<R> h = tr.trace(o, l, R(0), R(BIGD), time, false, 3u, 0u);
    if (h.tri == MISS) return V3<R>();
    Surf<R> s = surface(h, o, l, time);
    if (s.flags & VT_F_EMITTER) {
      if (opts & VT_O_NO_MIS) return V3<R>();
      V3<R> nE = emitter_normal(h, s, time);
      R cosE = dot(-l, nE);
      if (cosE <= R(0)) return V3<R>();
      V3<R> Le = emitted(nE, emitter_axis_at(time), -l);
      R pdfL = h.t * h.t / (cosE * R(tr.SU[3]));
      return Le * (pdfB * pdfB / (pdfB * pdfB + nL * nL * pdfL * pdfL));
    }
    if (opts & (VT_O_DIRECT_ONLY | VT_O_NO_INDIRECT)) return V3<R>();
    if (s.flags & VT_F_STATIC) {
      R mu = clampR(dot(s.ns, -l), R(0), R(1));
      return albedo_all(s.mat, mu) * node_lout(s.vi, s.b);
    }
    MatR<R> M2 = load_mat(s.mat);
    return M2.hh * ld3<R>(tr.SU + 8) * R(INV_PI_D);
  }
  // gpu/wgsl/shade.wgsl.js:250 shadeHit (no static-occlusion cache, no board texture: a 1x1 white mask)
  V3<R> shade_hit(const Hit<R>& h, const V3<R>& o, const V3<R>& d, R time, const V3<R>& ul, const V3<R>& ub,
                  uint32_t opts, uint32_t lightIndex, const PixSeeds& Sd, uint32_t nLight, uint32_t& key) const {
    if (h.tri == MISS) { key = 0xfffeu; return V3<R>(); }
    Surf<R> s = surface(h, o, d, time);
    key = s.mesh | ((h.inst == MISS || (s.flags & VT_F_STATIC)) ? 0u : 0x10000u);
    V3<R> wo = -d;
    if (opts & VT_O_NORMALS) return s.ns * R(0.5) + V3<R>(0.5, 0.5, 0.5);
    if (s.flags & VT_F_EMITTER) return emitted(emitter_normal(h, s, time), emitter_axis_at(time), wo);
    MatR<R> M = load_mat(s.mat);
    V3<R> n = shading_normal(s, opts);
    bool isStatic = (s.flags & VT_F_STATIC) != 0;
    bool mis = !isStatic && !(opts & VT_O_NO_MIS);
    uint32_t nl = std::min<uint32_t>(std::max<uint32_t>(nLight, 1u), 16u);
    V3<R> L;
    if (isStatic && (opts & VT_O_SHADOW_CACHE) && (opts & (VT_O_CACHE_WRITE | VT_O_CACHE_READ))) {
      // shade.wgsl.js:270-301, the static-occlusion cache's branch: the static scene and the posed bodies are asked
      // separately, and the shadow key bit marks a body blocking a sample, a penumbra or uneven light samples
      uint32_t nvis = 0, nlit = 0;
      R lmin = R(BIGD), lmax = 0;
      bool dyn = false;
      for (uint32_t j = 0; j < nl; j++) {
        V3<R> uj = j == 0 ? ul : V3<R>(kr(lightIndex + j, KL0, Sd.s[3]), kr(lightIndex + j, KL1, Sd.s[4]), kr(lightIndex + j, KL2, Sd.s[5]));
        V3<R> c, o, wi;
        R tmax;
        if (!light_eval(s, n, M, wo, time, uj, mis, R(nl), c, o, wi, tmax)) continue;
        nlit++;
        if (tr.trace(o, wi, R(0), tmax, time, true, 1u, 0u).tri != MISS) continue;
        if (tr.trace(o, wi, R(0), tmax, time, true, 2u, tr.su_u(7)).tri != MISS) { dyn = true; continue; }
        nvis++;
        L = L + c;
        R y = c.x * R(0.2126) + c.y * R(0.7152) + c.z * R(0.0722);
        lmin = std::min(lmin, y);
        lmax = std::max(lmax, y);
      }
      if (dyn || (nvis > 0 && nvis < nlit) || (nvis > 1 && lmax - lmin > R(0.2) * (lmax + lmin) * R(0.5))) key |= 0x20000u;
    } else {
      shadowTraced = false;
      L = direct_light(s, n, M, wo, time, ul, mis, R(nl));
      for (uint32_t j = 1; j < nl; j++) {
        V3<R> uj(kr(lightIndex + j, KL0, Sd.s[3]), kr(lightIndex + j, KL1, Sd.s[4]), kr(lightIndex + j, KL2, Sd.s[5]));
        L = L + direct_light(s, n, M, wo, time, uj, mis, R(nl));
      }
      if (shadowTraced) key |= 0x20000u;   // shade.wgsl.js:177 (no shadow culling: every sample that gets this far)
    }
    L = L / R(nl);
    if (isStatic) {
      if (!(opts & (VT_O_NO_INDIRECT | VT_O_DIRECT_ONLY))) {
        V3<R> E = node_efree(s.vi, s.b);
        if (!(opts & VT_O_NO_CAPSULE)) E = E * capsule_vis(s.p, n);
        R mu = std::max(dot(n, wo), R(0));
        L = L + E * R(INV_PI_D) * albedo_all(s.mat, mu);
      }
    } else {
      V3<R> l;
      R pdf = sample_bsdf(M, n, wo, ub, l);
      if (pdf > R(0) && dot(s.ng, l) > R(0)) {
        V3<R> thr = eval_bsdf(M, n, l, wo) * (dot(n, l) / pdf);
        L = L + thr * secondary(offset_ray(s.p, s.ng, l), l, time, pdf, opts, R(nl));
      }
    }
    return L;
  }
  // Path mode: unidirectional path tracing to maxDepth vertices. Each vertex: emitter hit (MIS-weighted against the
  // previous BSDF sample, power heuristic nL:1 as shade.wgsl.js:186/235), nL light samples with MIS
  // (directLight), then a BSDF sample (sampleBSDF) continues the path. Bounce 1 uses the reference's own sample
  // numbers (kernels.wgsl.js:50-51); bounce b >= 2 adds pixel-hash shifts (bounce_shift).
  V3<R> radiance_path(const Hit<R>& h0, const V3<R>& o0, const V3<R>& d0, R time, const V3<R>& ul0, const V3<R>& ub0,
                      uint32_t opts, uint32_t i, const PixSeeds& Sd, uint32_t nLight, uint32_t maxDepth, uint32_t& key) const {
    uint32_t nl = std::min<uint32_t>(std::max<uint32_t>(nLight, 1u), 16u);
    V3<R> L, thr(1, 1, 1), o = o0, d = d0;
    Hit<R> h = h0;
    R pdfPrev = 0;
    key = 0xfffeu;
    for (uint32_t b = 1; b <= maxDepth; b++) {
      if (b > 1) h = tr.trace(o, d, R(0), R(BIGD), time, false, 3u, 0u);
      if (h.tri == MISS) break;
      Surf<R> s = surface(h, o, d, time);
      if (b == 1) key = s.mesh | ((h.inst == MISS || (s.flags & VT_F_STATIC)) ? 0u : 0x10000u);
      V3<R> wo = -d;
      if (s.flags & VT_F_EMITTER) {
        V3<R> nE = emitter_normal(h, s, time);
        V3<R> Le = emitted(nE, emitter_axis_at(time), wo);
        if (b == 1 || (opts & VT_O_NO_MIS)) { if (b == 1) L = L + thr * Le; }
        else {
          R cosE = dot(-d, nE);
          if (cosE > R(0)) {
            R pdfL = h.t * h.t / (cosE * R(tr.SU[3]));
            L = L + thr * Le * (pdfPrev * pdfPrev / (pdfPrev * pdfPrev + R(nl) * R(nl) * pdfL * pdfL));
          }
        }
        break;
      }
      MatR<R> M = load_mat(s.mat);
      V3<R> n = shading_normal(s, opts);
      bool mis = !(opts & VT_O_NO_MIS);
      V3<R> ub = ub0;
      V3<R> Ld;
      shadowTraced = false;
      for (uint32_t j = 0; j < nl; j++) {
        V3<R> uj;
        if (b == 1) uj = j == 0 ? ul0 : V3<R>(kr(i * nl + j, KL0, Sd.s[3]), kr(i * nl + j, KL1, Sd.s[4]), kr(i * nl + j, KL2, Sd.s[5]));
        else uj = V3<R>(kr(i * nl + j, KL0, bounce_shift(Sd, b, 0)), kr(i * nl + j, KL1, bounce_shift(Sd, b, 1)), kr(i * nl + j, KL2, bounce_shift(Sd, b, 2)));
        Ld = Ld + direct_light(s, n, M, wo, time, uj, mis, R(nl));
      }
      if (b == 1 && shadowTraced) key |= 0x20000u;
      L = L + thr * (Ld / R(nl));
      if (b == maxDepth) break;
      if (b > 1) ub = V3<R>(kr(i, KB0, bounce_shift(Sd, b, 3)), kr(i, KB1, bounce_shift(Sd, b, 4)), kr(i, KB2, bounce_shift(Sd, b, 5)));
      V3<R> l;
      R pdf = sample_bsdf(M, n, wo, ub, l);
      if (!(pdf > R(0)) || dot(s.ng, l) <= R(0)) break;
      thr = thr * eval_bsdf(M, n, l, wo) * (dot(n, l) / pdf);
      pdfPrev = pdf;
      o = offset_ray(s.p, s.ng, l);
      d = l;
    }
    return L;
  }
};

// gpu/wgsl/kernels.wgsl.js:161-213 camMain / :70 cachedSubSample for one pixel (no caches, no packet traversal):
// sub-samples [i0, i1) with nl light samples each, summed in index order into acc; the key (first-hit mesh, posed
// body 0x10000, shadow traced 0x20000, mesh change among the sub-samples 0x40000) is carried across calls
template <typename R> static void pixel_samples(Tracer<R>& tr, const Shader<R>& sh, const vt_camera_desc& cam, uint32_t camIndex,
                                                const vt_render_req& q, uint32_t x, uint32_t y, uint32_t skip, uint32_t i0, uint32_t i1,
                                                uint32_t lightSamples, V3<R>& acc, uint32_t& key) {
  // the camera uniform is float32 (gpu/renderer.js:888-898 _packCam): lens and axes are priced at those values
  Lens L{double(float(cam.fx)), double(float(cam.fy)), double(float(cam.cx)), double(float(cam.cy)), double(float(cam.alpha)),
         {double(float(cam.k[0])), double(float(cam.k[1])), double(float(cam.k[2])), double(float(cam.k[3]))}};
  const double* T = cam.T_D_C;
  auto col = [&](int a, int b, int c) { return V3<R>(R(float(T[a])), R(float(T[b])), R(float(T[c]))); };
  V3<R> rx = col(0, 4, 8), ry = col(1, 5, 9), rz = col(2, 6, 10), pos = col(3, 7, 11);
  PixSeeds Sd = pix_seeds(x, y, q.seed, camIndex);
  uint32_t nl = std::max(1u, lightSamples);
  for (uint32_t i = i0; i < i1; i++) {
    float uvx = float(x) + kr(i, R2A, Sd.s[0]);
    uvx = uvx - 0.5f;
    float uvy = float(y) + kr(i, R2B, Sd.s[1]);
    uvy = uvy - 0.5f;
    float tt = mixf(q.shutter[0], q.shutter[1], kr(i, GOLD, Sd.s[2]));
    V3<R> dc = kb4_unproject<R>(L, R(uvx), R(uvy));
    V3<R> d = normalize(rx * dc.x + ry * dc.y + rz * dc.z);
    V3<R> ul(kr(i * nl, KL0, Sd.s[3]), kr(i * nl, KL1, Sd.s[4]), kr(i * nl, KL2, Sd.s[5]));
    V3<R> ub(kr(i, KB0, Sd.s[6]), kr(i, KB1, Sd.s[7]), kr(i, KB2, Sd.s[8]));
    Hit<R> h = tr.trace(pos, d, R(0), R(BIGD), R(tt), false, 1u, 0u);
    Hit<R> hd = tr.trace(pos, d, R(0), h.t, R(tt), false, 2u, skip);
    if (hd.tri != MISS) h = hd;
    uint32_t gk;
    V3<R> c = q.mode == VT_SHADE_TWIN ? sh.shade_hit(h, pos, d, R(tt), ul, ub, q.options, i * nl, Sd, lightSamples, gk)
                                      : sh.radiance_path(h, pos, d, R(tt), ul, ub, q.options, i, Sd, lightSamples, std::max(1u, q.max_depth), gk);
    acc = acc + c;
    if (i == 0) key = gk;
    else if ((gk & 0xffffu) != (key & 0xffffu)) key |= 0x40000u;
    key |= (gk & 0x30000u);
  }
}

static uint32_t pass1_spp(const vt_render_req& q) { return std::min(std::max(q.spp, 1u), q.mode == VT_SHADE_TWIN ? 64u : 4096u); }

template <typename R> static void render_pixel(Tracer<R>& tr, const Shader<R>& sh, const vt_camera_desc& cam, uint32_t camIndex,
                                               const vt_render_req& q, uint32_t x, uint32_t y, uint32_t skip, double out[4]) {
  const uint32_t spp = pass1_spp(q);
  V3<R> acc;
  uint32_t key = 0;
  pixel_samples<R>(tr, sh, cam, camIndex, q, x, y, skip, 0, spp, q.light_samples, acc, key);
  R sc = R(q.scale) / R(spp);
  out[0] = double(acc.x * sc); out[1] = double(acc.y * sc); out[2] = double(acc.z * sc);
  out[3] = key == 0xfffeu ? 0.0 : 1.0;
}

// ============================================================================================ calibration
// The differentiable calibration estimator of the CUDA library (its own model: the reference differentiates
// nothing), restated for the CPU: Lambertian vertices (f = rho / pi), nL emitter samples per vertex with the power
// heuristic against cosine sampling, cosine continuation (throughput x rho), the node term rho / pi x H(node) at the
// last vertex, emitter hits MIS-weighted after the first vertex. Parameters: per-material albedo, per-emitter-
// triangle radiance, node irradiance H (planar 3 x n).
struct CalibIn {
  const double* albedo; const double* lamp; const double* H; uint32_t nNodes; const uint32_t* triNode; uint32_t nStatic;
  // frozen replay (checks only): per path in (row, column, sub-sample) order, 4 x (triangle, instance) of its bounces
  // and 4 x 4 light-sample weights (0: occluded); null for the ordinary estimator
  const uint32_t* fzTI = nullptr; const float* fzQ = nullptr;
};
// fti / fq (frozen replay): this path's bounces' triangles and light-sample weights; the rays then meet those
// triangles' planes and a light sample with weight 0 counts as occluded, so that the estimator moves smoothly with
// the camera ray
template <typename R> static V3<R> calib_path(Tracer<R>& tr, const Shader<R>& sh, const CalibIn& C, const V3<R>& pos, const V3<R>& d0, R tt,
                                              uint32_t i, const PixSeeds& Sd, uint32_t nl, uint32_t depth, uint32_t skip,
                                              const uint32_t* fti = nullptr, const float* fq = nullptr) {
  const Scene& S = tr.S;
  V3<R> L, T(1, 1, 1), o = pos, d = d0;
  const R area = R(tr.SU[3]);
  R pbPrev = 0;
  for (uint32_t b = 1; b <= depth; b++) {
    Hit<R> h;
    if (fti) {
      if (fti[2 * (b - 1)] == MISS) break;
      h = tr.frozen_hit(fti[2 * (b - 1)], fti[2 * (b - 1) + 1], o, d, tt);
    } else if (b == 1) {
      h = tr.trace(o, d, R(0), R(BIGD), tt, false, 1u, 0u);
      Hit<R> hd = tr.trace(o, d, R(0), h.t, tt, false, 2u, skip);
      if (hd.tri != MISS) h = hd;
    } else {
      h = tr.trace(o, d, R(0), R(BIGD), tt, false, 3u, 0u);
    }
    if (h.tri == MISS) break;
    Surf<R> s = sh.surface(h, o, d, tt);
    if (s.flags & VT_F_EMITTER) {
      V3<R> nE = sh.emitter_normal(h, s, tt);
      R cosE = dot(-d, nE);
      if (cosE > R(0)) {
        R prof = sh.profile(std::acos(clampR(dot(-d, sh.emitter_axis_at(tt)), R(-1), R(1))));
        R w = 1;
        if (b > 1) {
          R pL = h.t * h.t / (cosE * area);
          w = pbPrev * pbPrev / (pbPrev * pbPrev + R(nl) * R(nl) * pL * pL);
        }
        uint32_t t = S.emitOfTri[h.tri];
        L = L + T * (w * prof * R(C.lamp[t]));
      }
      break;
    }
    const double* alb = C.albedo + 3 * s.mat;
    const V3<R> rho = V3<R>(R(alb[0]), R(alb[1]), R(alb[2]));
    V3<R> n = s.ns, wo = -d;
    R sum = 0;
    for (uint32_t j = 0; j < nl; j++) {
      V3<R> u;
      if (b == 1) u = V3<R>(kr(i * nl + j, KL0, Sd.s[3]), kr(i * nl + j, KL1, Sd.s[4]), kr(i * nl + j, KL2, Sd.s[5]));
      else u = V3<R>(kr(i * nl + j, KL0, bounce_shift(Sd, b, 0)), kr(i * nl + j, KL1, bounce_shift(Sd, b, 1)), kr(i * nl + j, KL2, bounce_shift(Sd, b, 2)));
      // the emitter triangle of the sample (the same CDF search as sample_emitter)
      uint32_t lo = 0, hi = S.emitN - 1;
      for (uint32_t it = 0; it < 40 && lo < hi; it++) {
        uint32_t m = (lo + hi) / 2;
        if (R(sh.pv(S.emitOff + 4 * m)[3]) < u.x) lo = m + 1; else hi = m;
      }
      V3<R> lp, ln, la;
      sh.sample_emitter(u, tt, lp, ln, la);
      V3<R> wi = lp - s.p;
      R d2 = dot(wi, wi), dist = std::sqrt(d2);
      wi = wi / dist;
      R cosE = dot(-wi, ln), cosS = dot(n, wi);
      if (cosE <= R(0) || cosS <= R(0) || dot(s.ng, wi) <= R(0) || dot(n, wo) <= R(0)) continue;
      R prof = sh.profile(std::acos(clampR(dot(-wi, la), R(-1), R(1))));
      if (prof <= R(0)) continue;
      R pdfW = d2 / (cosE * area), pb = cosS * R(INV_PI_D);
      R w = R(nl) * R(nl) * pdfW * pdfW / (R(nl) * R(nl) * pdfW * pdfW + pb * pb);
      bool vis;
      if (fq) vis = fq[4 * (b - 1) + j] != 0.0f;
      else vis = tr.trace(Shader<R>::offset_ray(s.p, s.ng, wi), wi, R(0), dist - R(2e-5), tt, true, 3u, tr.su_u(7)).tri == MISS;
      if (vis) sum = sum + R(C.lamp[lo]) * (prof * cosS * w * R(INV_PI_D) / pdfW);
    }
    V3<R> Tr = T * rho;
    L = L + Tr * (sum / R(nl));
    if (b == depth) {
      if (h.inst == MISS && h.tri < C.nStatic) {
        uint32_t nd = C.triNode[h.tri];
        const V3<R> Hn = V3<R>(R(C.H[nd]), R(C.H[C.nNodes + nd]), R(C.H[2 * C.nNodes + nd]));
        L = L + Tr * Hn * R(INV_PI_D);
      }
      break;
    }
    if (dot(n, wo) <= R(0)) break;
    R u1 = b == 1 ? R(kr(i, KB1, Sd.s[7])) : R(kr(i, KB1, bounce_shift(Sd, b, 4)));
    R u2 = b == 1 ? R(kr(i, KB2, Sd.s[8])) : R(kr(i, KB2, bounce_shift(Sd, b, 5)));
    V3<R> tb = basis_t(n), bb = basis_b(n);
    R r = std::sqrt(u1);
    V3<R> l = tb * (r * std::cos(R(2) * R(M_PI) * u2)) + bb * (r * std::sin(R(2) * R(M_PI) * u2)) + n * std::sqrt(std::max(R(0), R(1) - u1));
    R cl = dot(n, l);
    if (cl <= R(0) || dot(s.ng, l) <= R(0)) break;
    pbPrev = cl * R(INV_PI_D);
    T = Tr;
    o = Shader<R>::offset_ray(s.p, s.ng, l);
    d = l;
  }
  return L;
}

template <typename R> static void calib_pixel(Tracer<R>& tr, const Shader<R>& sh, const CalibIn& C, const vt_camera_desc& cam, uint32_t camIndex,
                                              uint32_t spp, uint32_t nl, uint32_t seed, uint32_t depth, uint32_t x, uint32_t y, uint32_t skip,
                                              double out[3]) {
  Lens L{double(float(cam.fx)), double(float(cam.fy)), double(float(cam.cx)), double(float(cam.cy)), double(float(cam.alpha)),
         {double(float(cam.k[0])), double(float(cam.k[1])), double(float(cam.k[2])), double(float(cam.k[3]))}};
  const double* T = cam.T_D_C;
  auto col = [&](int a, int b, int c) { return V3<R>(R(float(T[a])), R(float(T[b])), R(float(T[c]))); };
  V3<R> rx = col(0, 4, 8), ry = col(1, 5, 9), rz = col(2, 6, 10), pos = col(3, 7, 11);
  PixSeeds Sd = pix_seeds(x, y, seed, camIndex);
  V3<R> acc;
  for (uint32_t i = 0; i < spp; i++) {
    float uvx = float(x) + kr(i, R2A, Sd.s[0]);
    uvx = uvx - 0.5f;
    float uvy = float(y) + kr(i, R2B, Sd.s[1]);
    uvy = uvy - 0.5f;
    float tt = mixf(0.0f, 1.0f, kr(i, GOLD, Sd.s[2]));
    V3<R> dc = kb4_unproject<R>(L, R(uvx), R(uvy));
    V3<R> d = normalize(rx * dc.x + ry * dc.y + rz * dc.z);
    const size_t path = (size_t(y) * cam.width + x) * spp + i;
    acc = acc + calib_path<R>(tr, sh, C, pos, d, R(tt), i, Sd, nl, depth, skip, C.fzTI ? C.fzTI + path * 8 : nullptr,
                              C.fzQ ? C.fzQ + path * 16 : nullptr);
  }
  R sc = R(1) / R(spp);
  out[0] = double(acc.x * sc); out[1] = double(acc.y * sc); out[2] = double(acc.z * sc);
}

// irradiance at each node (centre, normal) from each emitter triangle at unit radiance: stratified points
// (Kronecker, the sampler's triangle warp), cosines, profile, visibility through the BVH
template <typename R> static void direct_transfer(Tracer<R>& tr, const Shader<R>& sh, const float* Cn, const float* Nn, uint32_t n0, uint32_t n1,
                                                  uint32_t samples, double* D) {
  const Scene& S = tr.S;
  const uint32_t nL = S.emitN;
  M3<R> M; V3<R> pp;
  tr.inst_pose(tr.su_u(17), R(0.5), M, pp);
  V3<R> axis = M.mul(ld3<R>(tr.SU + 4));
  for (uint32_t i = n0; i < n1; i++) {
    V3<R> c = ld3<R>(Cn + 3 * i), nn = ld3<R>(Nn + 3 * i);
    V3<R> org = c + nn * R(1e-4);
    for (uint32_t t = 0; t < nL; t++) {
      const float* e = sh.pv(S.emitOff + 4 * t);
      V3<R> v0 = ld3<R>(e), e1 = ld3<R>(e + 4), e2 = ld3<R>(e + 8), nl0 = ld3<R>(e + 12);
      R At = R(0.5) * len(cross(e1, e2));
      V3<R> nl = M.mul(nl0);
      R acc = 0;
      for (uint32_t s = 0; s < samples; s++) {
        R u1 = R(kr(s, R2A, 0.5f)), u2 = R(kr(s, R2B, 0.5f));
        R su = std::sqrt(u1);
        V3<R> lp = M.mul(v0 + e1 * (su * (R(1) - u2)) + e2 * (su * u2)) + pp;
        V3<R> w = lp - org;
        R r2 = dot(w, w), r = std::sqrt(r2);
        w = w / r;
        R ci = dot(nn, w), ct = dot(nl, -w);
        if (ci <= R(0) || ct <= R(0)) continue;
        R prof = sh.profile(std::acos(clampR(dot(-w, axis), R(-1), R(1))));
        if (prof <= R(0)) continue;
        Hit<R> h = tr.trace(org, w, R(0), r - R(2e-5), R(0.5), true, 3u, tr.su_u(7));
        if (h.tri == MISS) acc = acc + prof * ci * ct / r2;
      }
      D[size_t(i) * nL + t] = double(acc * At / R(samples));
    }
  }
}

// ============================================================================================ sensor (f32)
// gpu/wgsl/sensor.wgsl.js:46-208. The elementary functions are this project's own fixed-order float32 versions
// (the same sequence of correctly rounded operations on the device), so raw DN agree bit for bit:
//   ln(x): x = m 2^e, m in [sqrt(1/2), sqrt(2)), ln m = 2 atanh(s), s = (m-1)/(m+1), odd series to s^9;
//   exp(x): Cody-Waite reduction x = n ln2 + r (ln2 split hi/lo), Taylor degree 7, scale by 2^n;
//   cos(2 pi u): reduction in turns to [0, 1/8], Taylor series of cos / sin on [0, pi/4].
static inline float vt_logf(float x) {
  uint32_t bits = as_u(x);
  int e = int((bits >> 23) & 0xffu) - 127;
  float m = as_f((bits & 0x7fffffu) | 0x3f800000u);
  if (m > 1.41421356f) { m = m * 0.5f; e += 1; }
  float s = (m - 1.0f) / (m + 1.0f);
  float s2 = s * s;
  float p = std::fma(s2, 1.0f / 9.0f, 1.0f / 7.0f);
  p = std::fma(s2, p, 1.0f / 5.0f);
  p = std::fma(s2, p, 1.0f / 3.0f);
  p = std::fma(s2, p, 1.0f);
  float lm = 2.0f * s * p;
  return std::fma(float(e), 0.693147180559945f, lm);
}
static inline float vt_expf(float x) {
  float n = std::nearbyint(x * 1.44269504088896f);
  float r = std::fma(-n, 0.693145751953125f, x);
  r = std::fma(-n, 1.42860682030941723e-6f, r);
  float p = std::fma(r, 1.0f / 5040.0f, 1.0f / 720.0f);
  p = std::fma(r, p, 1.0f / 120.0f);
  p = std::fma(r, p, 1.0f / 24.0f);
  p = std::fma(r, p, 1.0f / 6.0f);
  p = std::fma(r, p, 0.5f);
  p = std::fma(r, p, 1.0f);
  p = std::fma(r, p, 1.0f);
  int ni = int(n);
  if (ni < -126) return 0.0f;
  return p * as_f(uint32_t(ni + 127) << 23);
}
static inline float vt_cos2pi(float u) {
  float t = u - std::floor(u + 0.5f);      // [-0.5, 0.5]
  float a = std::fabs(t);
  float sign = 1.0f;
  if (a > 0.25f) { a = 0.5f - a; sign = -1.0f; }
  float c;
  if (a <= 0.125f) {
    float x = a * 6.28318530717959f, x2 = x * x;
    float p = std::fma(x2, -1.0f / 3628800.0f, 1.0f / 40320.0f);
    p = std::fma(x2, p, -1.0f / 720.0f);
    p = std::fma(x2, p, 1.0f / 24.0f);
    p = std::fma(x2, p, -0.5f);
    c = std::fma(x2, p, 1.0f);
  } else {
    float x = (0.25f - a) * 6.28318530717959f, x2 = x * x;
    float p = std::fma(x2, -1.0f / 39916800.0f, 1.0f / 362880.0f);
    p = std::fma(x2, p, -1.0f / 5040.0f);
    p = std::fma(x2, p, 1.0f / 120.0f);
    p = std::fma(x2, p, -1.0f / 6.0f);
    c = std::fma(x * x2, p, x);
  }
  return sign * c;
}
static inline uint32_t pcgS(uint32_t v) { return pcg(v); }
static inline float uS(uint32_t x) { return (float(x >> 8u) + 0.5f) * (1.0f / 16777216.0f); }
static inline float erfA(float z) {   // gpu/wgsl/sensor.wgsl.js:57 (Abramowitz-Stegun 7.1.26)
  float t = 1.0f / (1.0f + 0.3275911f * std::fabs(z));
  float p = std::fma(1.061405429f, t, -1.453152027f);
  p = std::fma(p, t, 1.421413741f);
  p = std::fma(p, t, -0.284496736f);
  p = std::fma(p, t, 0.254829592f);
  float y = 1.0f - p * t * vt_expf(-z * z);
  return z >= 0.0f ? y : -y;
}
static inline float tapW(int k, float sg) {
  if (sg <= 0.0f) return k == 0 ? 1.0f : 0.0f;
  float s2 = sg * 1.41421356f;
  return 0.5f * (erfA((float(k) + 0.5f) / s2) - erfA((float(k) - 0.5f) / s2));
}
static inline int gaussTaps(float sigma) { return std::min(std::max(int(std::ceil(3.0f * sigma + 0.5f)), 0), 12); }
static inline float gauss(uint32_t h) {
  float u1 = uS(pcgS(h)), u2 = uS(pcgS(h ^ 0x68bc21ebu));
  return std::sqrt(-2.0f * vt_logf(u1)) * vt_cos2pi(u2);
}
static inline float poisson(float lam, uint32_t h) {
  if (lam <= 0.0f) return 0.0f;
  if (lam > 64.0f) return std::max(0.0f, std::floor(std::fma(std::sqrt(lam), gauss(h), lam) + 0.5f));
  float u = uS(pcgS(h ^ 0x1b873593u));
  float p = vt_expf(-lam), F = p, k = 0.0f;
  for (int i = 0; i < 200; i++) {
    if (u <= F) break;
    k = k + 1.0f;
    p = p * lam / k;
    F = F + p;
  }
  return k;
}
static void sensor_expose(const uint32_t* su, const float* E4, float* raw) {
  const float* f = reinterpret_cast<const float*>(su);
  int W = int(su[0]), H = int(su[1]);
  uint32_t cfa = su[2], frame = su[3];
  float sg = f[5];
  int r = gaussTaps(sg);
  static const uint32_t pats[4][4] = {{0, 1, 1, 2}, {1, 0, 2, 1}, {1, 2, 0, 1}, {2, 1, 1, 0}};
  for (int y = 0; y < H; y++) for (int x = 0; x < W; x++) {
    float Ex = 0, Ey = 0, Ez = 0, ws = 0;
    for (int k = -r; k <= r; k++) {
      int yy = std::min(std::max(y + k, 0), H - 1);
      float w = tapW(k, sg);
      const float* e = E4 + (size_t(yy) * W + x) * 4;
      Ex = std::fma(w, e[0], Ex); Ey = std::fma(w, e[1], Ey); Ez = std::fma(w, e[2], Ez);
      ws = ws + w;
    }
    Ex = Ex / ws; Ey = Ey / ws; Ez = Ez / ws;
    uint32_t ch = pats[cfa & 3u][(uint32_t(y) & 1u) * 2u + (uint32_t(x) & 1u)];
    const float* row = f + 8 + 4 * ch;
    float texp = f[6];
    float d = std::fma(row[2], Ez, std::fma(row[1], Ey, row[0] * Ex));
    float lam = std::fma(std::max(0.0f, d), texp, f[22] * texp);
    uint32_t h = pcgS((uint32_t(y * W + x) * 0x9E3779B9u) ^ pcgS((frame * 0x85ebca6bu) ^ pcgS(su[26] ^ (su[49] * 0xc2b2ae35u))));
    float e = lam;
    if (f[27] > 0.5f) e = std::fma(f[20], gauss(h ^ 0x27d4eb2fu), poisson(lam, h));
    e = std::min(e, f[21]);
    float t = e * f[23];
    t = std::fma(t, f[7], f[25]);
    float dn = std::floor(t + 0.5f);
    raw[size_t(y) * W + x] = std::min(std::max(dn, 0.0f), f[24]);
  }
}

// ============================================================================================ sensor chain (f32)
// gpu/wgsl/sensor.wgsl.js:67-427 restated per pixel, each multiply and add rounded separately in the order the
// reference's expressions give (the CUDA translation unit is compiled without contraction to match): optics with
// the relative-illumination map and the horizontal blur, veiling glare on a 1/F level, expose, demosaic (three
// modes), white balance + CCM with the AWB sums, bilateral noise reduction, tone curve, unsharp mask, YCbCr 4:2:0.
static inline float vt_powf(float x, float y) {
  if (!(x > 0.0f)) return y == 0.0f ? 1.0f : 0.0f;
  return vt_expf(y * vt_logf(x));
}
static inline int clampi(int v, int a, int b) { return v < a ? a : v > b ? b : v; }
static inline float clamp01(float v) { return std::min(std::max(v, 0.0f), 1.0f); }
static inline uint32_t cfa_ch(uint32_t code, uint32_t x, uint32_t y) {
  static const uint32_t pats[4][4] = {{0, 1, 1, 2}, {1, 0, 2, 1}, {1, 2, 0, 1}, {2, 1, 1, 0}};
  return pats[code & 3u][(y & 1u) * 2u + (x & 1u)];
}
static inline float srgb_oetf(float v) { return v <= 0.0031308f ? 12.92f * v : 1.055f * vt_powf(v, 0.41666666666666669f) - 0.055f; }

struct IspRef {
  const uint32_t* w;
  const float* f;
  int W, H;
  IspRef(const uint32_t* su) : w(su), f(reinterpret_cast<const float*>(su)), W(int(su[0])), H(int(su[1])) {}
  float tone(float x) const {   // sensor.wgsl.js:364 toneC
    float m = f[44];
    if (m > 2.5f) {
      float b = f[57];
      float v = clamp01((x - b) / (1.0f - b));
      float u = srgb_oetf(v);
      float cc = f[56];
      float a = vt_powf(u, cc);
      return a / std::max(a + vt_powf(1.0f - u, cc), 1e-12f);
    }
    float c = clamp01(x);
    if (m < 0.5f) return srgb_oetf(c);
    if (m < 1.5f) return vt_powf(c, 1.0f / std::max(f[45], 1e-3f));
    return c;
  }
};

static void isp_chain(const uint32_t* su, const float* L4, const float* ri, float* raw, uint8_t* rgba, uint8_t* yuv, uint32_t* stats) {
  IspRef I(su);
  const int W = I.W, H = I.H;
  const float* f = I.f;
  const size_t px = size_t(W) * H;
  std::vector<float> A(px * 3), Bv(px * 3), gpl(px);
  // sensorOptics (:67)
  const float sg = f[5];
  const int r = gaussTaps(sg);
  for (int y = 0; y < H; y++)
    for (int x = 0; x < W; x++) {
      float a[3] = {0, 0, 0}, ws = 0;
      for (int k = -r; k <= r; k++) {
        int xx = clampi(x + k, 0, W - 1);
        float w = tapW(k, sg);
        const float* l = L4 + (size_t(y) * W + xx) * 4;
        float m = ri[size_t(y) * W + xx];
        for (int c = 0; c < 3; c++) a[c] = a[c] + w * l[c] * m;
        ws = ws + w;
      }
      float s = f[4] / ws;
      for (int c = 0; c < 3; c++) A[(size_t(y) * W + x) * 3 + c] = a[c] * s;
    }
  // veiling glare (:86-141)
  const float kgl = f[52];
  const int F = int(f[54]);
  const int gw = (W + F - 1) / F, gh = (H + F - 1) / F;
  std::vector<float> GA, GB;
  if (kgl > 0.0f) {
    GA.assign(size_t(gw) * gh * 3, 0.0f);
    GB.assign(size_t(gw) * gh * 3, 0.0f);
    for (int y = 0; y < gh; y++)
      for (int x = 0; x < gw; x++) {
        float a[3] = {0, 0, 0}, n = 0;
        for (int j = 0; j < std::min(F, 32); j++)
          for (int i = 0; i < std::min(F, 32); i++) {
            int xx = x * F + i, yy = y * F + j;
            if (xx >= W || yy >= H) continue;
            const float* l = L4 + (size_t(yy) * W + xx) * 4;
            float m = ri[size_t(yy) * W + xx];
            for (int c = 0; c < 3; c++) a[c] = a[c] + l[c] * m;
            n = n + 1.0f;
          }
        float s = f[4] / std::max(n, 1.0f);
        for (int c = 0; c < 3; c++) GA[(size_t(y) * gw + x) * 3 + c] = a[c] * s;
      }
    const float gs = std::max(f[53], 1e-3f);
    for (int dir = 0; dir < 2; dir++) {
      const std::vector<float>& in = dir == 0 ? GA : GB;
      std::vector<float>& out = dir == 0 ? GB : GA;
      std::vector<float> tmp(in.size());
      for (int y = 0; y < gh; y++)
        for (int x = 0; x < gw; x++) {
          int n = dir == 0 ? gw : gh, c0 = dir == 0 ? x : y;
          float a[3] = {0, 0, 0};
          for (int k = 0; k < std::min(n, 256); k++) {
            float d = float(k - c0);
            float w = vt_expf(-0.5f * d * d / (gs * gs));
            const float* g = &in[(dir == 0 ? size_t(y) * gw + k : size_t(k) * gw + x) * 3];
            for (int c = 0; c < 3; c++) a[c] = a[c] + w * g[c];
          }
          float s = gs * 2.5066282746f;
          for (int c = 0; c < 3; c++) tmp[(size_t(y) * gw + x) * 3 + c] = a[c] / s;
        }
      out = tmp;
    }
  }
  auto glare_at = [&](int x, int y, float g[3]) {
    float Ff = f[54];
    float pxf = (float(x) + 0.5f) / Ff - 0.5f, pyf = (float(y) + 0.5f) / Ff - 0.5f;
    float fx0 = std::floor(pxf), fy0 = std::floor(pyf);
    int x0 = int(fx0), y0 = int(fy0);
    float fx = pxf - fx0, fy = pyf - fy0;
    auto at = [&](int xx, int yy, int c) { return GA[(size_t(clampi(yy, 0, gh - 1)) * gw + clampi(xx, 0, gw - 1)) * 3 + c]; };
    auto mix = [](float p, float q, float t) { return p * (1.0f - t) + q * t; };
    for (int c = 0; c < 3; c++) g[c] = mix(mix(at(x0, y0, c), at(x0 + 1, y0, c), fx), mix(at(x0, y0 + 1, c), at(x0 + 1, y0 + 1, c), fx), fy);
  };
  // sensorExpose (:177)
  for (int y = 0; y < H; y++)
    for (int x = 0; x < W; x++) {
      float e[3] = {0, 0, 0}, ws = 0;
      for (int k = -r; k <= r; k++) {
        int yy = clampi(y + k, 0, H - 1);
        float w = tapW(k, sg);
        for (int c = 0; c < 3; c++) e[c] = e[c] + w * A[(size_t(yy) * W + x) * 3 + c];
        ws = ws + w;
      }
      for (int c = 0; c < 3; c++) e[c] = e[c] / ws;
      if (kgl > 0.0f) {
        float g[3];
        glare_at(x, y, g);
        for (int c = 0; c < 3; c++) e[c] = (1.0f - kgl) * e[c] + kgl * g[c];
      }
      uint32_t ch = cfa_ch(su[2], uint32_t(x), uint32_t(y));
      const float* row = f + 8 + 4 * ch;
      float texp = f[6];
      float d = std::fma(row[2], e[2], std::fma(row[1], e[1], row[0] * e[0]));
      float lam = std::fma(std::max(0.0f, d), texp, f[22] * texp);
      uint32_t h = pcgS((uint32_t(y * W + x) * 0x9E3779B9u) ^ pcgS((su[3] * 0x85ebca6bu) ^ pcgS(su[26] ^ (su[49] * 0xc2b2ae35u))));
      float el = lam;
      if (f[27] > 0.5f) el = std::fma(f[20], gauss(h ^ 0x27d4eb2fu), poisson(lam, h));
      el = std::min(el, f[21]);
      float t = el * f[23];
      t = std::fma(t, f[7], f[25]);
      raw[size_t(y) * W + x] = std::min(std::max(std::floor(t + 0.5f), 0.0f), f[24]);
    }
  auto raw_at = [&](int x, int y) {
    if (x < 0) x = -x;
    if (x >= W) x = 2 * (W - 1) - x;
    if (y < 0) y = -y;
    if (y >= H) y = 2 * (H - 1) - y;
    return raw[size_t(clampi(y, 0, H - 1)) * W + clampi(x, 0, W - 1)];
  };
  // demosaicG (:222)
  const uint32_t mode = su[50];
  for (int y = 0; y < H; y++)
    for (int x = 0; x < W; x++) {
      float g = raw_at(x, y);
      if (cfa_ch(su[2], uint32_t(x), uint32_t(y)) != 1u) {
        float gl = raw_at(x - 1, y), gr = raw_at(x + 1, y), gu = raw_at(x, y - 1), gd = raw_at(x, y + 1);
        if (mode == 0) g = 0.25f * (gl + gr + gu + gd);
        else if (mode == 1) {
          float dh = std::fabs(gl - gr), dv = std::fabs(gu - gd);
          g = dh < dv ? 0.5f * (gl + gr) : dv < dh ? 0.5f * (gu + gd) : 0.25f * (gl + gr + gu + gd);
        } else {
          float c = g;
          float lh = 2.0f * c - raw_at(x - 2, y) - raw_at(x + 2, y);
          float lv = 2.0f * c - raw_at(x, y - 2) - raw_at(x, y + 2);
          float dh = std::fabs(gl - gr) + std::fabs(lh), dv = std::fabs(gu - gd) + std::fabs(lv);
          float gh2 = 0.5f * (gl + gr) + 0.25f * lh, gv = 0.5f * (gu + gd) + 0.25f * lv;
          g = dh < dv ? gh2 : dv < dh ? gv : 0.5f * (gh2 + gv);
          g = std::min(std::max(g, 0.0f), f[24]);
        }
      }
      gpl[size_t(y) * W + x] = g;
    }
  // demosaicRB (:264)
  stats[0] = stats[1] = stats[2] = stats[3] = 0;
  auto g_at = [&](int x, int y) { return gpl[size_t(clampi(y, 0, H - 1)) * W + clampi(x, 0, W - 1)]; };
  for (int y = 0; y < H; y++)
    for (int x = 0; x < W; x++) {
      uint32_t own = cfa_ch(su[2], uint32_t(x), uint32_t(y));
      float g = g_at(x, y);
      float sr = 0, sb = 0, cr = 0, cb = 0;
      for (int dy = -1; dy <= 1; dy++)
        for (int dx = -1; dx <= 1; dx++) {
          int xx = clampi(x + dx, 0, W - 1), yy = clampi(y + dy, 0, H - 1);
          uint32_t ch = cfa_ch(su[2], uint32_t(xx), uint32_t(yy));
          if (ch == 1u) continue;
          if (ch == own && !(dx == 0 && dy == 0)) continue;
          float d = raw_at(xx, yy) - g_at(xx, yy);
          if (ch == 0u) { sr = sr + d; cr = cr + 1.0f; } else { sb = sb + d; cb = cb + 1.0f; }
        }
      float rgb[3] = {g + sr / std::max(cr, 1.0f), g, g + sb / std::max(cb, 1.0f)};
      if (mode <= 1u) {
        float s3[3] = {0, 0, 0}, c3[3] = {0, 0, 0};
        for (int dy = -1; dy <= 1; dy++)
          for (int dx = -1; dx <= 1; dx++) {
            int xx = clampi(x + dx, 0, W - 1), yy = clampi(y + dy, 0, H - 1);
            uint32_t ch = cfa_ch(su[2], uint32_t(xx), uint32_t(yy));
            if (ch == own && !(dx == 0 && dy == 0)) continue;
            if (ch == 1u && own == 1u && !(dx == 0 && dy == 0)) continue;
            s3[ch] = s3[ch] + raw_at(xx, yy);
            c3[ch] = c3[ch] + 1.0f;
          }
        for (int c = 0; c < 3; c++) rgb[c] = s3[c] / std::max(c3[c], 1.0f);
        if (mode == 1u) rgb[1] = g;
      }
      float black = f[25], full = std::max(f[24] - black, 1.0f);
      float c[3];
      for (int k = 0; k < 3; k++) c[k] = (rgb[k] - black) / full;
      for (int k = 0; k < 3; k++) stats[1 + k] += uint32_t(std::nearbyint(clamp01(c[k]) * 1023.0f));
      for (int k = 0; k < 3; k++) c[k] = c[k] * f[28 + k];
      for (int k = 0; k < 3; k++) Bv[(size_t(y) * W + x) * 3 + k] = f[32 + 4 * k] * c[0] + f[33 + 4 * k] * c[1] + f[34 + 4 * k] * c[2];
    }
  // sensorNR (:321) into A
  for (int y = 0; y < H; y++)
    for (int x = 0; x < W; x++) {
      const float* c0 = &Bv[(size_t(y) * W + x) * 3];
      float* o = &A[(size_t(y) * W + x) * 3];
      if (su[51] == 0u || f[58] <= 0.0f) { o[0] = c0[0]; o[1] = c0[1]; o[2] = c0[2]; continue; }
      float Y0 = std::max(c0[0] * 0.2126f + c0[1] * 0.7152f + c0[2] * 0.0722f, 0.0f);
      float fullE = std::max(f[24] - f[25], 1.0f) / std::max(f[23] * f[7], 1e-9f);
      float sn = std::sqrt(Y0 * fullE + f[20] * f[20]) / fullE;
      float rs = std::max(f[59] * sn, 1e-6f), ss = f[58];
      float a[3] = {0, 0, 0}, ws = 0;
      for (int dy = -1; dy <= 1; dy++)
        for (int dx = -1; dx <= 1; dx++) {
          const float* c = &Bv[(size_t(clampi(y + dy, 0, H - 1)) * W + clampi(x + dx, 0, W - 1)) * 3];
          float dY = (c[0] - c0[0]) * 0.2126f + (c[1] - c0[1]) * 0.7152f + (c[2] - c0[2]) * 0.0722f;
          float w = vt_expf(-0.5f * float(dx * dx + dy * dy) / (ss * ss) - 0.5f * dY * dY / (rs * rs));
          for (int k = 0; k < 3; k++) a[k] = a[k] + w * c[k];
          ws = ws + w;
        }
      for (int k = 0; k < 3; k++) o[k] = a[k] / ws;
    }
  // sensorOutput (:387), one 2x2 block at a time
  auto toned = [&](int x, int y, float c[3]) {
    const float* a = &A[(size_t(clampi(y, 0, H - 1)) * W + clampi(x, 0, W - 1)) * 3];
    for (int k = 0; k < 3; k++) c[k] = I.tone(a[k]);
  };
  auto luma = [](const float c[3]) { return c[0] * 0.299f + c[1] * 0.587f + c[2] * 0.114f; };
  const float amt = f[46];
  const int rad = clampi(int(std::nearbyint(f[47])), 1, 4);
  const bool c420 = su[48] != 0u;
  const int cw = (W + 1) / 2, chh = (H + 1) / 2;
  for (int gy = 0; gy < chh; gy++)
    for (int gx = 0; gx < cw; gx++) {
      int bx = 2 * gx, by = 2 * gy;
      float Ys[4] = {0, 0, 0, 0}, cb = 0, cr = 0, nb = 0;
      for (int q = 0; q < 4; q++) {
        int x = bx + (q & 1), y = by + (q >> 1);
        if (x >= W || y >= H) continue;
        float c[3];
        toned(x, y, c);
        if (amt > 0.0f) {
          float m = 0, n = 0;
          for (int dy = -rad; dy <= rad; dy++)
            for (int dx = -rad; dx <= rad; dx++) {
              float t[3];
              toned(x + dx, y + dy, t);
              m = m + luma(t);
              n = n + 1.0f;
            }
          float sh = amt * (luma(c) - m / n);
          for (int k = 0; k < 3; k++) c[k] = c[k] + sh;
        }
        float r8 = clamp01(c[0]) * 255.0f, g8 = clamp01(c[1]) * 255.0f, b8 = clamp01(c[2]) * 255.0f;
        Ys[q] = 0.299f * r8 + 0.587f * g8 + 0.114f * b8;
        cb = cb + (128.0f - 0.168736f * r8 - 0.331264f * g8 + 0.5f * b8);
        cr = cr + (128.0f + 0.5f * r8 - 0.418688f * g8 - 0.081312f * b8);
        nb = nb + 1.0f;
        if (!c420) {
          float y8 = std::min(std::max(std::nearbyint(Ys[q]), 0.0f), 255.0f);
          uint8_t* o = rgba + (size_t(y) * W + x) * 4;
          o[0] = uint8_t(std::nearbyint(r8)); o[1] = uint8_t(std::nearbyint(g8)); o[2] = uint8_t(std::nearbyint(b8)); o[3] = 255;
          stats[0] += uint32_t(y8);
        }
      }
      if (c420) {
        float Cb = std::min(std::max(std::nearbyint(cb / nb), 0.0f), 255.0f), Cr = std::min(std::max(std::nearbyint(cr / nb), 0.0f), 255.0f);
        for (int q = 0; q < 4; q++) {
          int x = bx + (q & 1), y = by + (q >> 1);
          if (x >= W || y >= H) continue;
          float y8 = std::min(std::max(std::nearbyint(Ys[q]), 0.0f), 255.0f);
          float rr = y8 + 1.402f * (Cr - 128.0f);
          float gg = y8 - 0.344136f * (Cb - 128.0f) - 0.714136f * (Cr - 128.0f);
          float bb = y8 + 1.772f * (Cb - 128.0f);
          uint8_t* o = rgba + (size_t(y) * W + x) * 4;
          o[0] = uint8_t(std::min(std::max(std::nearbyint(rr), 0.0f), 255.0f));
          o[1] = uint8_t(std::min(std::max(std::nearbyint(gg), 0.0f), 255.0f));
          o[2] = uint8_t(std::min(std::max(std::nearbyint(bb), 0.0f), 255.0f));
          o[3] = 255;
          yuv[size_t(y) * W + x] = uint8_t(y8);
          stats[0] += uint32_t(y8);
        }
        yuv[px + size_t(gy) * cw + gx] = uint8_t(Cb);
        yuv[px + size_t(cw) * chh + size_t(gy) * cw + gx] = uint8_t(Cr);
      }
    }
}

// gpu/sensor.js:98 relativeIlluminationMap (FP64, lens.js unproject / distort / distortDeriv)
static void ri_map(const vt_camera_desc& c, double q, const double* vdeg, const double* vv, uint32_t nv, float* out) {
  Lens L{c.fx, c.fy, c.cx, c.cy, c.alpha, {c.k[0], c.k[1], c.k[2], c.k[3]}};
  for (uint32_t y = 0; y < c.height; y++)
    for (uint32_t x = 0; x < c.width; x++) {
      double uv[2] = {double(x), double(y)}, r[3];
      unproject(L, uv, r);
      double th = std::acos(std::max(-1.0, std::min(1.0, r[2])));
      double ri = 1.0;
      if (th > 1e-6) ri = std::pow(std::cos(th), q) * std::sin(th) / (distort(L, th) * distort_deriv(L, th));
      double vg = 1.0;
      if (nv) {
        double t0 = vdeg[0] * M_PI / 180.0;
        if (th <= t0) vg = vv[0];
        else {
          vg = vv[nv - 1];
          for (uint32_t i = 1; i < nv; i++) {
            double ti = vdeg[i] * M_PI / 180.0, tp = vdeg[i - 1] * M_PI / 180.0;
            if (th <= ti) { vg = vv[i - 1] + (vv[i] - vv[i - 1]) * (th - tp) / (ti - tp); break; }
          }
        }
      }
      out[size_t(y) * c.width + x] = float(std::max(0.0, ri) * vg);
    }
}

// ============================================================================================ radiosity (FP64)

// Direct FP64 solve of (I - diag(rho) F) B = E (Gaussian elimination with partial pivoting), R right-hand sides.
static void solve_dense(int n, const float* F, const float* rho, const float* E, int R, double* B) {
  std::vector<double> A(size_t(n) * n), X(size_t(n) * R);
  for (int i = 0; i < n; i++) {
    for (int j = 0; j < n; j++) A[size_t(i) * n + j] = (i == j ? 1.0 : 0.0) - double(rho[i]) * double(F[size_t(i) * n + j]);
    for (int r = 0; r < R; r++) X[size_t(i) * R + r] = E[size_t(i) * R + r];
  }
  for (int k = 0; k < n; k++) {
    int p = k;
    for (int i = k + 1; i < n; i++) if (std::fabs(A[size_t(i) * n + k]) > std::fabs(A[size_t(p) * n + k])) p = i;
    if (p != k) {
      for (int j = 0; j < n; j++) std::swap(A[size_t(k) * n + j], A[size_t(p) * n + j]);
      for (int r = 0; r < R; r++) std::swap(X[size_t(k) * R + r], X[size_t(p) * R + r]);
    }
    double piv = A[size_t(k) * n + k];
    for (int i = k + 1; i < n; i++) {
      double m = A[size_t(i) * n + k] / piv;
      if (m == 0) continue;
      for (int j = k; j < n; j++) A[size_t(i) * n + j] -= m * A[size_t(k) * n + j];
      for (int r = 0; r < R; r++) X[size_t(i) * R + r] -= m * X[size_t(k) * R + r];
    }
  }
  for (int i = n - 1; i >= 0; i--) for (int r = 0; r < R; r++) {
    double s = X[size_t(i) * R + r];
    for (int j = i + 1; j < n; j++) s -= A[size_t(i) * n + j] * X[size_t(j) * R + r];
    X[size_t(i) * R + r] = s / A[size_t(i) * n + i];
  }
  std::copy(X.begin(), X.end(), B);
}

// FP64 Jacobi B <- E + rho (F B) to a relative update below tol, for large n: threads over blocks of 8 rows, each
// block streaming the rows of B once (B stays in the caches; the per-row sums over j run in order).
static int jacobi64(int n, const float* F, const float* rho, const float* E, int R, double* B, double tol, int maxIt, int threads) {
  std::vector<double> Bn(size_t(n) * R);
  for (size_t i = 0; i < size_t(n) * R; i++) B[i] = E[i];
  int it = 0;
  const int RB = 8;
  for (; it < maxIt; it++) {
    std::atomic<int> next(0);
    auto work = [&]() {
      std::vector<double> acc(size_t(RB) * R);
      for (;;) {
        const int i0 = next.fetch_add(RB);
        if (i0 >= n) break;
        const int rows = std::min(RB, n - i0);
        std::fill(acc.begin(), acc.end(), 0.0);
        for (int j = 0; j < n; j++) {
          const double* Bj = B + size_t(j) * R;
          for (int k = 0; k < rows; k++) {
            const double f = F[size_t(i0 + k) * n + j];
            if (f == 0) continue;
            double* a = acc.data() + size_t(k) * R;
            for (int r = 0; r < R; r++) a[r] += f * Bj[r];
          }
        }
        for (int k = 0; k < rows; k++)
          for (int r = 0; r < R; r++) Bn[size_t(i0 + k) * R + r] = double(E[size_t(i0 + k) * R + r]) + double(rho[i0 + k]) * acc[size_t(k) * R + r];
      }
    };
    std::vector<std::thread> th;
    for (int t = 0; t < threads; t++) th.emplace_back(work);
    for (auto& x : th) x.join();
    double num = 0, den = 0;
    for (size_t i = 0; i < size_t(n) * R; i++) { double d = Bn[i] - B[i]; num += d * d; den += Bn[i] * Bn[i]; }
    std::copy(Bn.begin(), Bn.end(), B);
    if (std::sqrt(num) <= tol * std::sqrt(den)) { it++; break; }
  }
  return it;
}

// F_ij = A_j max(0, n_i.w) max(0, -n_j.w) / (pi r^2 + A_j), w = (c_j - c_i)/r, rows scaled to sum <= 1 (FP64)
static void form_factors(int n, const float* C, const float* Nn, const float* A, float* F) {
  for (int i = 0; i < n; i++) {
    double s = 0;
    std::vector<double> row(n, 0.0);
    for (int j = 0; j < n; j++) {
      if (i == j) continue;
      double w[3] = {double(C[3 * j]) - C[3 * i], double(C[3 * j + 1]) - C[3 * i + 1], double(C[3 * j + 2]) - C[3 * i + 2]};
      double r2 = w[0] * w[0] + w[1] * w[1] + w[2] * w[2];
      double r = std::sqrt(r2);
      if (!(r > 0)) continue;
      double ci = (Nn[3 * i] * w[0] + Nn[3 * i + 1] * w[1] + Nn[3 * i + 2] * w[2]) / r;
      double cj = -(Nn[3 * j] * w[0] + Nn[3 * j + 1] * w[1] + Nn[3 * j + 2] * w[2]) / r;
      if (ci <= 0 || cj <= 0) continue;
      double f = double(A[j]) * ci * cj / (M_PI * r2 + double(A[j]));
      row[j] = f; s += f;
    }
    double sc = s > 1 ? 1 / s : 1;
    for (int j = 0; j < n; j++) F[size_t(i) * n + j] = float(row[j] * sc);
  }
}

}  // namespace orc

// ============================================================================================ C API (ctypes)

using namespace orc;

// ============================================================================================ node radiosity
// The scene's own node radiosity (gpu/wgsl/kernels.wgsl.js:255-461; gpu/renderer.js:456-851), restated for the CPU:
// the gather table, its escape counts and remap, the smoothing neighbours, the nodes' direct light and the Jacobi
// steps of the separable transport. Precision R for the geometry and transport; the gather directions' sample
// numbers (the spiral radius and angle fraction) in float32, rounded per operation as the CUDA kernels draw them.
template <typename R> struct NodeRad {
  Tracer<R>& tr;
  Shader<R>& sh;
  const Scene& S;
  NodeRad(Tracer<R>& t, Shader<R>& s) : tr(t), sh(s), S(t.S) {}
  V3<R> pos(uint32_t i) const { return ld3<R>(tr.V + 8 * size_t(i)); }
  V3<R> nrm(uint32_t i) const { return normalize(ld3<R>(tr.V + 8 * size_t(i) + 4)); }
  uint32_t mat(uint32_t i) const { return as_u(sh.pv(S.meshOff + 2 * S.verts[8 * size_t(i) + 3])[3]); }
  // gpu/wgsl/kernels.wgsl.js:271 gatherDir
  static V3<R> dir(uint32_t i, uint32_t j, uint32_t K, const V3<R>& n) {
    V3<R> t = basis_t(n), b = basis_b(n);
    float rot = u01(pcg(i * 2654435761u + 17u));
    float rr = std::sqrt((float(j) + 0.5f) / float(K));
    float a = float(j) * 0.6180339887498949f;
    a = a + rot;
    float fr = a - std::floor(a);
    R ph = R(2) * R(M_PI) * R(fr), r = R(rr);
    return normalize(t * (r * std::cos(ph)) + b * (r * std::sin(ph)) + n * std::sqrt(std::max(R(0), R(1) - r * r)));
  }
  // gpu/wgsl/kernels.wgsl.js:284 gatherBuild (one entry)
  uint32_t build(uint32_t i, uint32_t j, uint32_t K) const {
    V3<R> p = pos(i), n = nrm(i), d = dir(i, j, K, n);
    Hit<R> h = tr.trace(p + n * R(2e-6), d, R(0), R(BIGD), R(0.5), false, 1u, 0u);
    if (h.tri == MISS) return MISS;
    V3<R> bb(R(1) - h.u - h.v, h.u, h.v);
    const uint32_t* ru = S.tris.data() + size_t(h.tri) * 16;
    uint32_t v0 = ru[3], v1 = ru[7], v2 = ru[11];
    V3<R> nv = ld3<R>(tr.V + 8 * size_t(v0) + 4) * bb.x + ld3<R>(tr.V + 8 * size_t(v1) + 4) * bb.y + ld3<R>(tr.V + 8 * size_t(v2) + 4) * bb.z;
    if (!(dot(nv, d) < R(0))) return MISS;
    if (bb.x >= bb.y && bb.x >= bb.z) return v0;
    return bb.y >= bb.z ? v1 : v2;
  }
  // gpu/wgsl/kernels.wgsl.js:300 gatherRemap (one entry)
  uint32_t remap(uint32_t i, uint32_t j, uint32_t K, uint32_t v0, const float* misses) const {
    const float half = 0.5f * float(K);
    if (v0 == MISS || misses[v0] <= half) return v0;
    V3<R> p = pos(i), n = nrm(i), d = dir(i, j, K, n);
    Hit<R> h = tr.trace(p + n * R(2e-6), d, R(0), R(BIGD), R(0.5), false, 1u, 0u);
    if (h.tri == MISS) return v0;
    V3<R> bb(R(1) - h.u - h.v, h.u, h.v);
    const uint32_t* ru = S.tris.data() + size_t(h.tri) * 16;
    uint32_t a = ru[3], b = ru[7], c = ru[11], best = v0;
    R bw = -1;
    if (misses[a] <= half && bb.x > bw) { best = a; bw = bb.x; }
    if (misses[b] <= half && bb.y > bw) { best = b; bw = bb.y; }
    if (misses[c] <= half && bb.z > bw) { best = c; bw = bb.z; }
    return best;
  }
  // gpu/wgsl/kernels.wgsl.js:348 nodeDirect (one node): B_dir (3), visibility code, capsule visibility
  bool direct(uint32_t i, uint32_t NS, uint32_t moved, R out[5]) const {
    V3<R> p = pos(i), n = nrm(i);
    if (moved) {
      M3<R> M; V3<R> pp;
      tr.inst_pose(tr.su_u(17), R(0.5), M, pp);
      V3<R> dE = (M.mul(ld3<R>(tr.SU + 20)) + pp) - p;
      R rr = R(tr.SU[23]) + R(1e-3);
      bool near = false;
      for (uint32_t b = 0; b < std::min<uint32_t>(tr.su_u(16), VT_MAX_INST) && !near; b++) {
        if (!((moved >> b) & 1u)) continue;
        const float* I = tr.inst(b);
        near = Tracer<R>::seg_near_capsule(p, dE, R(0), R(1), ld3<R>(I + 32), ld3<R>(I + 36), R(I[35]) + rr) ||
               Tracer<R>::seg_near_capsule(p, dE, R(0), R(1), ld3<R>(I + 40), ld3<R>(I + 44), R(I[43]) + rr);
      }
      if (!near) return false;
    }
    uint32_t m = mat(i);
    uint32_t hs = pcg(i * 2246822519u + 3u);
    float s0 = u01(pcg(hs)), s1 = u01(pcg(hs + 1u)), s2 = u01(pcg(hs + 2u));
    V3<R> B;
    uint32_t nLit = 0, nVis = 0;
    V3<R> o = p + n * R(2e-6);
    for (uint32_t s = 0; s < NS; s++) {
      V3<R> lp, ln, la;
      sh.sample_emitter(V3<R>(kr(s, KL0, s0), kr(s, KL1, s1), kr(s, KL2, s2)), R(0.5), lp, ln, la);
      V3<R> wi = lp - p;
      R d2 = dot(wi, wi), dist = std::sqrt(d2);
      wi = wi / dist;
      R cosE = dot(-wi, ln), cosN = dot(n, wi);
      if (cosE <= R(0) || cosN <= R(0)) continue;
      V3<R> Le = sh.emitted(ln, la, -wi);
      if (maxc(Le) <= R(0)) continue;
      nLit++;
      if (tr.trace(o, wi, R(0), dist - R(2e-5), R(0.5), true, 3u, tr.su_u(7)).tri != MISS) continue;
      nVis++;
      B = B + Le * (cosE * cosN * R(tr.SU[3]) / d2) * sh.albedo_all(m, cosN);
    }
    B = B / R(NS);
    out[0] = B.x; out[1] = B.y; out[2] = B.z;
    out[3] = nLit == 0 ? R(-1) : nVis == nLit ? R(1) : nVis == 0 ? R(0) : R(0.5);
    out[4] = sh.capsule_vis(p, n);
    return true;
  }
  // gpu/wgsl/kernels.wgsl.js:416 jacobiGather (one active node)
  V3<R> gather(uint32_t i, uint32_t K, const uint32_t* gtable, const double* st, uint32_t slotIn) const {
    V3<R> n = nrm(i);
    uint32_t mi = mat(i);
    V3<R> acc;
    for (uint32_t j = 0; j < K; j++) {
      uint32_t h = gtable[size_t(i) * K + j];
      if (h == MISS) continue;
      V3<R> d = dir(i, j, K, n);
      R muIn = std::sqrt(std::max(R(0), R(1) - (R(j) + R(0.5)) / R(K)));
      R muOut = clampR(-dot(d, nrm(h)), R(0), R(1));
      const double* L = st + 16 * size_t(h) + 4 * slotIn;
      acc = acc + sh.albedo_all(mi, muIn) * sh.albedo_all(mat(h), muOut) * V3<R>(R(L[0]), R(L[1]), R(L[2]));
    }
    V3<R> hh = sh.load_mat(mi).hh;
    R sc = R(M_PI) / R(K);
    return V3<R>(acc.x * sc / std::max(hh.x, R(1e-4)), acc.y * sc / std::max(hh.y, R(1e-4)), acc.z * sc / std::max(hh.z, R(1e-4)));
  }
};

template <typename F> static void parallel_for(size_t n, int threads, F&& f) {
  std::atomic<size_t> next(0);
  auto work = [&]() {
    for (;;) {
      size_t k = next.fetch_add(64);
      if (k >= n) break;
      for (size_t q = k; q < std::min(n, k + 64); q++) f(q);
    }
  };
  if (threads <= 1) { work(); return; }
  std::vector<std::thread> th;
  for (int t = 0; t < threads; t++) th.emplace_back(work);
  for (auto& x : th) x.join();
}

// ============================================================================================ raster pass
// lite_nodes/renderer.js restated for the CPU: the raster geometry (sliceTris :443, _buildGeometry :527), the
// emitter samples (:598, posed by setPoses :729), the vertex stage (vsCam / vsShadow :224-265), a rasteriser with
// the rules the library documents (clip 0 <= z <= w and |x|, |y| <= 8 w; 1/256-pixel snap; int64 edge functions,
// ties to the edge with dy < 0 or dy = 0 and dx > 0; screen-linear depth (edge weights times one reciprocal of the
// doubled area) clamped to [0, 1] and kept below 1 and
// below the sample's, ties to the earlier triangle), the fragment stage (fsCam :284, smVis :267) with the MSAA
// resolve through half floats and FINISH (:363), and the display look (DISPLAY :369); the 3x3 shadow taps one texel
// apart share the centre tap's bilinear fraction. Float32 arithmetic in the
// order the kernels use (this file is built with -ffp-contract=off), so raster keys, shadow maps and display bytes
// compare bit for bit, radiance to float rounding.

namespace lite {

struct SV { double p[3], n[3]; };
static bool sv_before(const SV& a, const SV& b) {
  for (int k = 0; k < 2; k++) if (a.p[k] != b.p[k]) return a.p[k] < b.p[k];
  return a.p[2] < b.p[2];
}
static void unit(double* v) {
  double l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  if (l == 0 || std::isnan(l)) l = 1;
  v[0] /= l; v[1] /= l; v[2] /= l;
}
// the point of edge (A, B) on the plane p[ax] = c, computed from the lexicographically smaller endpoint
static SV crossing(const SV& A, const SV& B, int ax, double c) {
  const bool ab = sv_before(A, B);
  const SV& lo = ab ? A : B;
  const SV& hi = ab ? B : A;
  const double f = (c - lo.p[ax]) / (hi.p[ax] - lo.p[ax]);
  SV X;
  for (int k = 0; k < 3; k++) { X.p[k] = lo.p[k] + f * (hi.p[k] - lo.p[k]); X.n[k] = lo.n[k] + f * (hi.n[k] - lo.n[k]); }
  X.p[ax] = c;
  unit(X.n);
  return X;
}
using Tri3 = std::array<SV, 3>;
static void fan_out(const std::vector<SV>& poly, std::vector<Tri3>& out) {
  for (size_t j = 2; j < poly.size(); j++) out.push_back(Tri3{poly[0], poly[j - 1], poly[j]});
}
static std::vector<Tri3> slice(std::vector<Tri3> tris, double h) {
  for (int ax = 0; ax < 3; ax++) {
    std::vector<Tri3> next;
    for (const Tri3& t : tris) {
      double lo = t[0].p[ax], hi = t[0].p[ax];
      for (int j = 1; j < 3; j++) { lo = std::min(lo, t[j].p[ax]); hi = std::max(hi, t[j].p[ax]); }
      const long long first = (long long)std::floor(lo / h) + 1, last = (long long)std::ceil(hi / h) - 1;
      if (last < first) { next.push_back(t); continue; }
      std::vector<SV> poly(t.begin(), t.end());
      bool done = false;
      for (long long k = first; k <= last && !done; k++) {
        const double c = double(k) * h;
        std::vector<SV> below, above;
        for (size_t j = 0; j < poly.size(); j++) {
          const SV& A = poly[j];
          const SV& B = poly[(j + 1) % poly.size()];
          const double sa = A.p[ax] - c, sb = B.p[ax] - c;
          if (sa <= 0) below.push_back(A);
          if (sa >= 0) above.push_back(A);
          if ((sa < 0 && sb > 0) || (sa > 0 && sb < 0)) { SV X = crossing(A, B, ax, c); below.push_back(X); above.push_back(X); }
        }
        if (below.size() >= 3) fan_out(below, next);
        if (above.size() < 3) done = true;
        else poly = above;
      }
      if (!done) fan_out(poly, next);
    }
    tris.swap(next);
  }
  return tris;
}

static void geometry(const Scene& S, double h, double hfix, std::vector<uint32_t>& V, std::vector<uint32_t>& I) {
  V.clear();
  I.clear();
  for (uint32_t i = 0; i < S.staticVerts; i++) {
    const uint32_t* s = S.verts.data() + 8 * size_t(i);
    const uint32_t w[8] = {s[0], s[1], s[2], (s[3] & 0xffffu) | 0xffff0000u, s[4], s[5], s[6], i};
    V.insert(V.end(), w, w + 8);
  }
  for (uint32_t k = 0; k < S.staticTris; k++) {
    const uint32_t* t = S.tris.data() + 16 * size_t(k);
    I.push_back(t[3]); I.push_back(t[7]); I.push_back(t[11]);
  }
  uint32_t next = S.staticVerts;
  for (size_t b = 0; b < S.blas.size(); b++) {
    const Blas& B = S.blas[b];
    std::vector<uint32_t> meshes;
    for (uint32_t k = 0; k < B.tri_count; k++) {
      const uint32_t m = S.tris[16 * size_t(B.tri_off + k) + 12];
      if (m < S.meshes.size() && S.meshes[m].overview_only) continue;   // not drawn by the raster pass
      if (std::find(meshes.begin(), meshes.end(), m) == meshes.end()) meshes.push_back(m);
    }
    for (uint32_t m : meshes) {
      std::vector<Tri3> tris;
      for (uint32_t k = 0; k < B.tri_count; k++) {
        const uint32_t* t = S.tris.data() + 16 * size_t(B.tri_off + k);
        if (t[12] != m) continue;
        Tri3 tr;
        for (int j = 0; j < 3; j++) {
          const uint32_t* v = S.verts.data() + 8 * size_t(t[3 + 4 * j]);
          for (int q = 0; q < 3; q++) { tr[j].p[q] = double(as_f(v[q])); tr[j].n[q] = double(as_f(v[4 + q])); }
        }
        tris.push_back(tr);
      }
      for (const Tri3& t : slice(tris, B.kind == VT_BODY_FIXTURE ? hfix : h))
        for (const SV& v : t) {
          const uint32_t w[8] = {as_u(float(v.p[0])), as_u(float(v.p[1])), as_u(float(v.p[2])), (m & 0xffffu) | (uint32_t(b) << 16),
                                 as_u(float(v.n[0])), as_u(float(v.n[1])), as_u(float(v.n[2])), MISS};
          V.insert(V.end(), w, w + 8);
          I.push_back(next++);
        }
    }
  }
}

// the emitter samples in the world for the scope pose T (column-major 4x4): 8 floats each
static void emitter_world(const Scene& S, uint32_t n, const double* T, std::vector<float>& out, double sectC[4][3]) {
  const double* c = S.centroid;
  const double* nr = S.emitNormal;
  double t[3], up[3] = {0, 0, 0};
  up[std::fabs(nr[0]) < 0.9 ? 0 : 1] = 1;
  t[0] = up[1] * nr[2] - up[2] * nr[1]; t[1] = up[2] * nr[0] - up[0] * nr[2]; t[2] = up[0] * nr[1] - up[1] * nr[0];
  unit(t);
  const double bb[3] = {nr[1] * t[2] - nr[2] * t[1], nr[2] * t[0] - nr[0] * t[2], nr[0] * t[1] - nr[1] * t[0]};
  const double g = 1.22074408460575947536;
  const size_t nt = S.emitTris.size() / 14;
  std::vector<double> P(3 * size_t(n)), N(3 * size_t(n));
  std::vector<int> sect(n);
  for (uint32_t i = 0; i < n; i++) {
    const double u1 = std::fmod(0.5 + i / g, 1.0), u2 = std::fmod(0.5 + i / (g * g), 1.0), u3 = std::fmod(0.5 + i / (g * g * g), 1.0);
    size_t a = 0, z = nt ? nt - 1 : 0;
    while (a < z) { const size_t m = (a + z) / 2; if (S.emitTris[14 * m + 13] < u1) a = m + 1; else z = m; }
    const double* e = S.emitTris.data() + 14 * a;
    const double su = std::sqrt(u2);
    double d[3];
    for (int k = 0; k < 3; k++) {
      P[3 * i + k] = nt ? e[k] + e[3 + k] * su * (1 - u3) + e[6 + k] * su * u3 : 0.0;
      N[3 * i + k] = nt ? e[9 + k] : (k == 2 ? 1.0 : 0.0);
      d[k] = P[3 * i + k] - c[k];
    }
    const double ang = std::atan2(d[0] * bb[0] + d[1] * bb[1] + d[2] * bb[2], d[0] * t[0] + d[1] * t[1] + d[2] * t[2]);
    sect[i] = std::min(3, int(std::floor((ang + M_PI) / (2 * M_PI) * 4)));
  }
  auto W = [&](const double* v, double* o) { for (int i = 0; i < 3; i++) o[i] = T[i] * v[0] + T[4 + i] * v[1] + T[8 + i] * v[2] + T[12 + i]; };
  for (int k = 0; k < 4; k++) {
    double acc[3] = {0, 0, 0};
    int cnt = 0;
    for (uint32_t i = 0; i < n; i++) if (sect[i] == k) { for (int j = 0; j < 3; j++) acc[j] += P[3 * i + j]; cnt++; }
    for (int j = 0; j < 3; j++) sectC[k][j] = cnt ? acc[j] / cnt : c[j];
  }
  out.assign(8 * size_t(n), 0.0f);
  for (uint32_t i = 0; i < n; i++) {
    double w[3];
    W(&P[3 * i], w);
    float* o = out.data() + 8 * size_t(i);
    for (int k = 0; k < 3; k++) {
      o[k] = float(w[k]);
      o[4 + k] = float(T[k] * N[3 * i] + T[4 + k] * N[3 * i + 1] + T[8 + k] * N[3 * i + 2]);
    }
    o[3] = float(sect[i]);
    o[7] = float(S.emitArea);
  }
}

struct View {
  const float* f;
  uint32_t u(int i) const { return as_u(f[i]); }
  V3<float> v3(int i) const { return V3<float>(f[i], f[i + 1], f[i + 2]); }
};
static inline float hyp(float x, float y) { return std::sqrt(x * x + y * y); }

static bool world_of(Tracer<float>& tr, const View& V, const uint32_t* w, V3<float>& p, V3<float>& n) {
  p = V3<float>(as_f(w[0]), as_f(w[1]), as_f(w[2]));
  n = V3<float>(as_f(w[4]), as_f(w[5]), as_f(w[6]));
  const uint32_t inst = w[3] >> 16;
  if (inst == 0xffffu) return true;
  if (inst >= VT_MAX_INST || (tr.su_u(24 + 48 * inst + 15) & 2u) || ((V.u(28) >> inst) & 1u)) return false;
  M3<float> M;
  V3<float> t;
  tr.inst_pose(inst, V.f[35], M, t);
  p = M.mul(p) + t;
  n = M.mul(n);
  return true;
}
static void project_cam(const View& V, const V3<float>& p, float o[4]) {
  const V3<float> d = p - V.v3(12);
  const float x = dot(d, V.v3(0)), y = dot(d, V.v3(4)), z = dot(d, V.v3(8));
  const float W = V.f[24], H = V.f[25], FAR = V.f[47];
  const float fx = V.f[16], fy = V.f[17], cx = V.f[18], cy = V.f[19];
  if (V.f[15] > 0.5f) {
    const float nz = 1e-3f;
    o[0] = (2.0f * fx * x + (2.0f * (cx + 0.5f) - W) * z) / W;
    o[1] = ((H - 2.0f * (cy + 0.5f)) * z - 2.0f * fy * y) / H;
    o[2] = (z - nz) * FAR / (FAR - nz);
    o[3] = z;
    return;
  }
  const float r = hyp(x, y);
  const float th = std::atan2(r, z);
  if (th > V.f[26]) {
    const float ex = fx * x / W + 1e-12f, ey = -fy * y / H;
    const float l = hyp(ex, ey);
    o[0] = ex / l; o[1] = ey / l; o[2] = -1e-3f; o[3] = -1e-3f;
    return;
  }
  const float t2 = th * th;
  const float thd = th * (1.0f + t2 * (V.f[20] + t2 * (V.f[21] + t2 * (V.f[22] + t2 * V.f[23]))));
  const float s = thd / std::max(r, 1e-12f);
  const float u = fx * x * s + cx + 0.5f, v = fy * y * s + cy + 0.5f;
  o[0] = 2.0f * u / W - 1.0f; o[1] = 1.0f - 2.0f * v / H; o[2] = len(d) / FAR; o[3] = 1.0f;
}
static V3<float> sm_project(const View& V, const V3<float>& pw, int k) {
  const V3<float> d = pw - V.v3(48 + 4 * k);
  const float x = dot(d, V.v3(40)), y = dot(d, V.v3(44)), z = dot(d, V.v3(36));
  const float rho = hyp(x, y);
  const float s = std::atan2(rho, z) / (V.f[43] * std::max(rho, 1e-12f));
  return V3<float>(x * s, y * s, len(d));
}

// ------------------------------------------------------------------------------------------- rasteriser
static float pdist(const float* v, int p) {
  const float G = 8.0f;
  switch (p) {
    case 0: return v[2];
    case 1: return v[3] - v[2];
    case 2: return G * v[3] - v[0];
    case 3: return G * v[3] + v[0];
    case 4: return G * v[3] - v[1];
    default: return G * v[3] + v[1];
  }
}
struct Pt { long long x, y; float z; };
// clip + snap: the polygon's snapped vertices (empty: nothing to draw)
static std::vector<Pt> setup(const float* c0, const float* c1, const float* c2, uint32_t W, uint32_t H) {
  std::vector<std::array<float, 4>> poly = {{c0[0], c0[1], c0[2], c0[3]}, {c1[0], c1[1], c1[2], c1[3]}, {c2[0], c2[1], c2[2], c2[3]}};
  bool inside = true;
  for (auto& v : poly) for (int p = 0; p < 6; p++) inside = inside && pdist(v.data(), p) >= 0.0f;
  if (!inside) {
    for (int p = 0; p < 6; p++) {
      std::vector<std::array<float, 4>> out;
      for (size_t i = 0; i < poly.size(); i++) {
        const auto& A = poly[i];
        const auto& B = poly[(i + 1) % poly.size()];
        const float da = pdist(A.data(), p), db = pdist(B.data(), p);
        if (da >= 0.0f && out.size() < 9) out.push_back(A);
        if ((da >= 0.0f) != (db >= 0.0f) && out.size() < 9) {
          const auto& In = da >= 0.0f ? A : B;
          const auto& Out = da >= 0.0f ? B : A;
          const float di = da >= 0.0f ? da : db, dq = da >= 0.0f ? db : da;
          const float t = di / (di - dq);
          out.push_back({In[0] + t * (Out[0] - In[0]), In[1] + t * (Out[1] - In[1]), In[2] + t * (Out[2] - In[2]), In[3] + t * (Out[3] - In[3])});
        }
      }
      poly.swap(out);
      if (poly.size() < 3) return {};
    }
  }
  const float W2 = float(W) * 0.5f, H2 = float(H) * 0.5f;
  std::vector<Pt> P;
  for (auto& v : poly) {
    if (!(v[3] > 0.0f)) return {};
    const float nx = v[0] / v[3], ny = v[1] / v[3];
    const float X = (nx + 1.0f) * W2, Y = (1.0f - ny) * H2;
    if (!(std::fabs(X) < 1e6f) || !(std::fabs(Y) < 1e6f)) return {};
    P.push_back(Pt{(long long)std::lrint(X * 256.0f), (long long)std::lrint(Y * 256.0f), v[2] / v[3]});
  }
  return P;
}
static long long fdiv256(long long v) { return v >= 0 ? v / 256 : -((255 - v) / 256); }

// raster triangles [t0, t0 + nt) of layer `layer` into keys (samples 4: 64-bit keys; 1: depth bits in the high word)
static void raster(const float* clip, const uint32_t* idx, uint32_t t0, uint32_t nt, uint32_t W, uint32_t H, uint32_t samples, uint64_t* keys) {
  static const int SX[4] = {96, 224, 32, 160}, SY[4] = {32, 96, 160, 224};
  for (uint32_t t = t0; t < t0 + nt; t++) {
    const std::vector<Pt> P = setup(clip + 4 * size_t(idx[3 * t]), clip + 4 * size_t(idx[3 * t + 1]), clip + 4 * size_t(idx[3 * t + 2]), W, H);
    for (size_t k = 1; k + 1 < P.size(); k++) {
      Pt a = P[0], b = P[k], c = P[k + 1];
      long long A = (b.x - a.x) * (c.y - a.y) - (b.y - a.y) * (c.x - a.x);
      if (A == 0) continue;
      if (A < 0) { std::swap(b, c); A = -A; }
      const Pt* ends[3][2] = {{&b, &c}, {&c, &a}, {&a, &b}};
      long long dx[3], dy[3], ox[3], oy[3];
      int bias[3];
      for (int e = 0; e < 3; e++) {
        dx[e] = ends[e][1]->x - ends[e][0]->x; dy[e] = ends[e][1]->y - ends[e][0]->y;
        ox[e] = ends[e][0]->x; oy[e] = ends[e][0]->y;
        bias[e] = (dy[e] < 0 || (dy[e] == 0 && dx[e] > 0)) ? 0 : -1;
      }
      const long long x0 = std::max(0LL, fdiv256(std::min(a.x, std::min(b.x, c.x)))), x1 = std::min((long long)W - 1, fdiv256(std::max(a.x, std::max(b.x, c.x))));
      const long long y0 = std::max(0LL, fdiv256(std::min(a.y, std::min(b.y, c.y)))), y1 = std::min((long long)H - 1, fdiv256(std::max(a.y, std::max(b.y, c.y))));
      const float rA = 1.0f / float(A);
      for (long long py = y0; py <= y1; py++)
        for (long long px = x0; px <= x1; px++)
          for (uint32_t s = 0; s < samples; s++) {
            const long long sx = px * 256 + (samples == 1 ? 128 : SX[s]), sy = py * 256 + (samples == 1 ? 128 : SY[s]);
            long long w[3];
            bool in = true;
            for (int e = 0; e < 3; e++) { w[e] = dx[e] * (sy - oy[e]) - dy[e] * (sx - ox[e]); in = in && w[e] + bias[e] >= 0; }
            if (!in) continue;
            const float l1 = float(w[1]) * rA, l2 = float(w[2]) * rA;
            float z = a.z + l1 * (b.z - a.z) + l2 * (c.z - a.z);
            z = std::min(z, 1.0f);
            if (!(z > 0.0f)) z = 0.0f;
            if (!(z < 1.0f)) continue;
            uint64_t key = (uint64_t(as_u(z)) << 32) | (samples == 1 ? 0xffffffffull : uint64_t(t));
            uint64_t& slot = keys[(size_t(py) * W + px) * samples + s];
            if (key < slot) slot = key;
          }
    }
  }
}

// ------------------------------------------------------------------------------------------- fragment stage
static float h16(float x) {
  if (std::isnan(x) || std::isinf(x) || x == 0.0f) return x;
  int ex;
  std::frexp(double(x), &ex);
  const double q = std::fabs(x) < 6.103515625e-05 ? std::ldexp(1.0, -24) : std::ldexp(1.0, ex - 11);
  const double r = std::nearbyint(double(x) / q) * q;
  if (std::fabs(r) > 65504.0) return x > 0 ? INFINITY : -INFINITY;
  return float(r);
}
// depth compare of one texel (clamp to edge; all ones = cleared = depth 1)
static int less_texel(const uint32_t* m, uint32_t res, int k, int x, int y, float dref) {
  x = std::min(std::max(x, 0), int(res) - 1);
  y = std::min(std::max(y, 0), int(res) - 1);
  const uint32_t b = m[(size_t(k) * res + y) * res + x];
  return dref < (b == 0xffffffffu ? 1.0f : as_f(b)) ? 1 : 0;
}
struct Frag {
  Tracer<float>& tr;
  Shader<float>& sh;
  const View& V;
  const uint32_t* Vx;       // raster vertices, 8 words
  const uint32_t* idx;
  const float* clip;
  const float* es;
  const uint32_t *sms, *smd;
  uint32_t res;

  // smVis: 3x3 taps one texel apart, each a bilinear blend of 2x2 depth compares ('less', clamp to edge), min of
  // the static and dynamic maps per tap; the taps share the centre tap's bilinear fraction
  float vis(const V3<float>& pw, int k, float bias) const {
    const V3<float> q = sm_project(V, pw, k);
    if (std::fabs(q.x) >= 1.0f || std::fabs(q.y) >= 1.0f) return 1.0f;
    const float u = 0.5f + 0.5f * q.x, v = 0.5f - 0.5f * q.y, dref = (q.z - bias) / V.f[47];
    const float tx = u * float(res) - 0.5f, ty = v * float(res) - 0.5f;
    const float fx0 = std::floor(tx), fy0 = std::floor(ty), fx = tx - fx0, fy = ty - fy0;
    const int x0 = int(fx0) - 1, y0 = int(fy0) - 1;
    int cs[4][4], cd[4][4];
    for (int j = 0; j < 4; j++)
      for (int i = 0; i < 4; i++) {
        cs[j][i] = less_texel(sms, res, k, x0 + i, y0 + j, dref);
        cd[j][i] = less_texel(smd, res, k, x0 + i, y0 + j, dref);
      }
    const float w00 = (1.0f - fx) * (1.0f - fy), w10 = fx * (1.0f - fy), w01 = (1.0f - fx) * fy, w11 = fx * fy;
    float s = 0.0f;
    for (int j = 0; j < 3; j++)
      for (int i = 0; i < 3; i++) {
        const float a = w00 * float(cs[j][i]) + w10 * float(cs[j][i + 1]) + w01 * float(cs[j + 1][i]) + w11 * float(cs[j + 1][i + 1]);
        const float b = w00 * float(cd[j][i]) + w10 * float(cd[j][i + 1]) + w01 * float(cd[j + 1][i]) + w11 * float(cd[j + 1][i + 1]);
        s = s + std::min(a, b);
      }
    return s / 9.0f;
  }
  V3<float> shade(uint32_t tri, uint32_t px, uint32_t py) const {
    const Scene& S = tr.S;
    V3<float> wp[3], wn[3];
    float X[3], Y[3];
    const float W2 = V.f[24] * 0.5f, H2 = V.f[25] * 0.5f, sx = float(px) + 0.5f, sy = float(py) + 0.5f;
    const uint32_t* vw[3];
    for (int j = 0; j < 3; j++) {
      const uint32_t vi = idx[3 * tri + j];
      vw[j] = Vx + 8 * size_t(vi);
      world_of(tr, V, vw[j], wp[j], wn[j]);
      const float* c = clip + 4 * size_t(vi);
      X[j] = (c[0] + c[3]) * W2 - sx * c[3];
      Y[j] = (c[3] - c[1]) * H2 - sy * c[3];
    }
    float b[3] = {X[1] * Y[2] - X[2] * Y[1], X[2] * Y[0] - X[0] * Y[2], X[0] * Y[1] - X[1] * Y[0]};
    const float sb = b[0] + b[1] + b[2];
    if (sb != 0.0f) for (float& q : b) q = q / sb;
    else for (float& q : b) q = 1.0f / 3.0f;
    const V3<float> p = wp[0] * b[0] + wp[1] * b[1] + wp[2] * b[2];
    const V3<float> nin = wn[0] * b[0] + wn[1] * b[1] + wn[2] * b[2];
    const uint32_t slot = tr.su_u(18);
    float ew[4] = {0, 0, 0, 0};
    for (int j = 0; j < 3; j++) {
      const uint32_t ni = vw[j][7];
      if (ni == MISS) continue;
      const float wa = S.nodeState[16 * size_t(ni) + 4 * slot + 3];
      for (int k = 0; k < 3; k++) ew[k] = ew[k] + S.nodeState[16 * size_t(ni) + k] * wa * b[j];
      ew[3] = ew[3] + wa * b[j];
    }
    const uint32_t mesh = vw[0][3] & 0xffffu, inst = vw[0][3] >> 16;
    const uint32_t flags = as_u(sh.pv(S.meshOff + 2 * mesh + 1)[0]), mat = as_u(sh.pv(S.meshOff + 2 * mesh)[3]);
    const V3<float> wo = normalize(V.v3(12) - p);
    V3<float> ng = cross(wp[1] - wp[0], wp[2] - wp[0]);
    if (dot(ng, ng) < 1e-30f) ng = nin;
    ng = normalize(ng);
    if (dot(ng, wo) < 0.0f) ng = -ng;
    V3<float> ns = normalize(nin);
    const V3<float> axis = V.v3(36);
    const V3<float> L0 = V3<float>(tr.SU[0], tr.SU[1], tr.SU[2]);
    if (flags & VT_F_EMITTER) {
      if (dot(wo, ns) <= 0.0f) return V3<float>();
      const V3<float> Le = L0 * sh.profile(std::acos(clampR(dot(wo, axis), -1.0f, 1.0f)));
      return V3<float>(std::min(Le.x * V.f[27], 60000.0f), std::min(Le.y * V.f[27], 60000.0f), std::min(Le.z * V.f[27], 60000.0f));
    }
    if (dot(ns, ng) < 0.0f) ns = -ns;
    if (dot(ns, wo) < 1e-4f) ns = ng;
    const MatR<float> M = sh.load_mat(mat);
    const bool st = inst == 0xffffu;
    const uint32_t nS = st ? V.u(29) : V.u(30);
    V3<float> acc[4];
    for (uint32_t j = 0; j < nS; j++) {
      const float* ea = es + 8 * size_t(j);
      V3<float> wi = V3<float>(ea[0], ea[1], ea[2]) - p;
      const float d2 = dot(wi, wi);
      wi = wi * (1.0f / std::sqrt(d2));
      const float cosE = dot(-wi, V3<float>(ea[4], ea[5], ea[6]));
      if (cosE <= 0.0f) continue;
      const float cosS = dot(ns, wi);
      if (cosS <= 0.0f || dot(ng, wi) <= 0.0f) continue;
      const float pr = sh.profile(std::acos(clampR(dot(-wi, axis), -1.0f, 1.0f)));
      if (pr <= 0.0f) continue;
      const V3<float> f = eval_bsdf(M, ns, wi, wo);
      const int k = std::min(int(ea[3]), 3);
      acc[k] = acc[k] + f * (pr * cosS * cosE * ea[7] / d2);
    }
    V3<float> L;
    const V3<float> off = p + ng * (st ? 1.5e-4f : 6e-4f);
    const uint32_t dbg = V.u(39);
    float vsum = 0.0f;
    for (int k = 0; k < 4; k++) {
      const float vk = dbg != 1u ? vis(off, k, st ? V.f[51 + 4 * k] : 6e-4f) : 1.0f;
      vsum = vsum + vk;
      if (maxc(acc[k]) <= 0.0f) continue;
      L = L + acc[k] * vk;
    }
    if (dbg == 2u) return V3<float>(vsum / 4.0f, vsum / 4.0f, vsum / 4.0f);
    L = L * L0 / float(nS);
    const float mu = std::max(dot(ns, wo), 0.0f);
    const V3<float> Al = sh.albedo_all(mat, mu);
    if (st) {
      V3<float> E;
      if (ew[3] > 1e-6f) E = V3<float>(ew[0], ew[1], ew[2]) / ew[3];
      E = E * sh.capsule_vis(p, ns);
      L = L + E * float(INV_PI_D) * Al;
    } else {
      L = L + V.v3(32) * Al;
    }
    return L * V.f[27];
  }
};

}  // namespace lite

extern "C" {

void or_mulberry32(uint32_t seed, int n, double* out) { Mulberry32 m(seed); for (int i = 0; i < n; i++) out[i] = m.next(); }
void or_pcg(const uint32_t* in, int n, uint32_t* out) { for (int i = 0; i < n; i++) out[i] = pcg(in[i]); }
void or_kr(const uint32_t* i, const float* a, const float* shift, int n, float* out) { for (int k = 0; k < n; k++) out[k] = kr(i[k], a[k], shift[k]); }

static Lens lens_of(const double* p) { return Lens{p[0], p[1], p[2], p[3], p[4], {p[5], p[6], p[7], p[8]}}; }
void or_unproject(const double* lens, int n, const double* uv, double* out) { Lens L = lens_of(lens); for (int i = 0; i < n; i++) unproject(L, uv + 2 * i, out + 3 * i); }
void or_project(const double* lens, int n, const double* X, double* out) { Lens L = lens_of(lens); for (int i = 0; i < n; i++) project(L, X + 3 * i, out + 2 * i); }
void or_unproject_f32(const double* lens, int n, const float* uv, float* out) {
  Lens L = lens_of(lens);
  for (int i = 0; i < n; i++) { V3<float> r = kb4_unproject<float>(L, uv[2 * i], uv[2 * i + 1]); out[3 * i] = r.x; out[3 * i + 1] = r.y; out[3 * i + 2] = r.z; }
}
void or_distort_deriv(const double* lens, int n, const double* th, double* out) { Lens L = lens_of(lens); for (int i = 0; i < n; i++) out[i] = distort_deriv(L, th[i]); }

// buildBVH: returns node count; nodes_out needs cap*16 words, order_out n words; info = [maxDepth, bmin3, bmax3]
int or_bvh_build(const float* pos, const uint32_t* idx, uint32_t n, int leafSize, uint32_t* nodes_out, int cap, uint32_t* order_out, double* info) {
  BVH b = build_bvh(pos, idx, n, leafSize);
  if (int(b.node_count) > cap) return -int(b.node_count);
  std::copy(b.nodes.begin(), b.nodes.end(), nodes_out);
  std::copy(b.order.begin(), b.order.end(), order_out);
  info[0] = b.max_depth;
  for (int k = 0; k < 3; k++) { info[1 + k] = b.bmin[k]; info[4 + k] = b.bmax[k]; }
  return int(b.node_count);
}
void or_pack_triangles(const float* pos, const uint32_t* idx, const uint32_t* order, uint32_t n, float* T) {
  std::vector<uint32_t> tmp(size_t(n) * 16, 0);
  for (uint32_t k = 0; k < n; k++) pack_tri(tmp, k, pos, idx, order[k], 0, 0, 0, 0, 0);
  for (size_t i = 0; i < tmp.size(); i++) if (i % 4 != 3) T[i] = as_f(tmp[i]); else T[i] = 0;
}
// out per ray: t, u, v, tri (as double)
void or_traverse_js(const uint32_t* nodes, const float* T, int n, const float* o, const float* d, double tmin, double tmax, int anyHit, uint32_t root, double* out) {
  for (int i = 0; i < n; i++) {
    double oo[3] = {o[3 * i], o[3 * i + 1], o[3 * i + 2]}, dd[3] = {d[3 * i], d[3 * i + 1], d[3 * i + 2]};
    HitJS h = traverse_js(nodes, T, oo, dd, tmin, tmax, anyHit != 0, root);
    out[4 * i] = h.t; out[4 * i + 1] = h.u; out[4 * i + 2] = h.v; out[4 * i + 3] = double(h.tri);
  }
}
void or_brute_force(const float* T, uint32_t count, int n, const float* o, const float* d, double tmin, double tmax, double* out) {
  for (int i = 0; i < n; i++) {
    double oo[3] = {o[3 * i], o[3 * i + 1], o[3 * i + 2]}, dd[3] = {d[3 * i], d[3 * i + 1], d[3 * i + 2]};
    HitJS h = brute_force(T, count, oo, dd, tmin, tmax);
    out[4 * i] = h.t; out[4 * i + 1] = h.u; out[4 * i + 2] = h.v; out[4 * i + 3] = double(h.tri);
  }
}

double or_fresnel_average(double eta) { return fresnel_average(eta); }
double or_fresnel_dielectric(double cosi, double eta) { return fresnel_dielectric<double>(cosi, eta); }
double or_disc_irradiance(const double* x, const double* n, const double* c, const double* m, double a, double L, int nr, int nphi) {
  return disc_irradiance(x, n, c, m, a, L, nr, nphi);
}
double or_profile(double th, const double* knots, const double* p, int n) {
  std::vector<double> k(knots, knots + n), pp(p, p + n);
  return profile_js(th, k, pp);
}
double or_capsule_occ(const double* p, const double* n, const double* a, const double* b, double r) {
  return capsule_occ<double>(V3<double>(p[0], p[1], p[2]), V3<double>(n[0], n[1], n[2]), V3<double>(a[0], a[1], a[2]), V3<double>(b[0], b[1], b[2]), r);
}
// material evaluation on host: mat = vt_material; cases n,l,v,u (12 doubles each) -> f rgb, pdf, sampled l, pdf (8)
void or_bsdf_eval(const vt_material* m, int n, const double* cases, double* out) {
  Mat M = prepare_material(*m, 1024);
  MatR<double> MR = mat_r64(M);
  for (int i = 0; i < n; i++) {
    const double* c = cases + 12 * i;
    V3<double> nn(c[0], c[1], c[2]), l(c[3], c[4], c[5]), v(c[6], c[7], c[8]), u(c[9], c[10], c[11]), ls;
    V3<double> f = eval_bsdf(MR, nn, l, v);
    double pdf = pdf_bsdf(MR, nn, v, l);
    double sp = sample_bsdf(MR, nn, v, u, ls);
    double* o = out + 8 * i;
    o[0] = f.x; o[1] = f.y; o[2] = f.z; o[3] = pdf; o[4] = ls.x; o[5] = ls.y; o[6] = ls.z; o[7] = sp;
  }
}
// albedo table of one material: spec (bins*3), diff (bins*3), hh (3), hhSpec (3)
void or_albedo_table(const vt_material* m, int samples, double* out) {
  Mat M = prepare_material(*m, samples);
  for (int i = 0; i < VT_ALBEDO_BINS * 3; i++) { out[i] = M.has_table ? M.spec[i] : 0; out[VT_ALBEDO_BINS * 3 + i] = M.has_table ? M.diff[i] : 0; }
  for (int c = 0; c < 3; c++) { out[VT_ALBEDO_BINS * 6 + c] = M.hh[c]; out[VT_ALBEDO_BINS * 6 + 3 + c] = M.hhSpec[c]; }
}

// -------- scene
void* or_scene_create(const vt_scene_desc* sd, int leafSize, int albedoSamples) { return prepare_scene(sd, leafSize, albedoSamples); }
void or_scene_destroy(void* h) { delete static_cast<Scene*>(h); }
// sizes: nodeCount, triCount, vertCount, paramVec4s, staticVerts, meshOff, matOff, albOff, profOff, profN, emitOff, emitN
void or_scene_sizes(void* h, uint32_t* out) {
  Scene* S = static_cast<Scene*>(h);
  uint32_t v[12] = {S->nodeCount, S->triCount, S->vertCount, uint32_t(S->params.size() / 4), S->staticVerts, S->meshOff,
                    S->matOff, S->albOff, S->profOff, S->profN, S->emitOff, S->emitN};
  std::memcpy(out, v, sizeof(v));
}
void or_scene_arrays(void* h, uint32_t* nodes, uint32_t* tris, uint32_t* verts, float* params) {
  Scene* S = static_cast<Scene*>(h);
  if (nodes) std::copy(S->nodes.begin(), S->nodes.end(), nodes);
  if (tris) std::copy(S->tris.begin(), S->tris.end(), tris);
  if (verts) std::copy(S->verts.begin(), S->verts.end(), verts);
  if (params) std::copy(S->params.begin(), S->params.end(), params);
}
// emitter: area, axis3, normal3, centroid3, radius, shadowSkipsScope, scopeIndex
void or_scene_emitter(void* h, double* out) {
  Scene* S = static_cast<Scene*>(h);
  out[0] = S->emitArea;
  for (int k = 0; k < 3; k++) { out[1 + k] = S->emitAxis[k]; out[4 + k] = S->emitNormal[k]; out[7 + k] = S->centroid[k]; }
  out[10] = S->radius; out[11] = S->shadowSkipsScope; out[12] = S->scopeIndex;
}
// blas i: root, triOff, triCount, bmin3, bmax3, capA3, capB3, capR, rhoEff
void or_scene_blas(void* h, int i, double* out) {
  Scene* S = static_cast<Scene*>(h);
  const Blas& b = S->blas[i];
  out[0] = b.root; out[1] = b.tri_off; out[2] = b.tri_count;
  for (int k = 0; k < 3; k++) { out[3 + k] = b.bmin[k]; out[6 + k] = b.bmax[k]; out[9 + k] = b.cap_a[k]; out[12 + k] = b.cap_b[k]; }
  out[15] = b.cap_r; out[16] = b.rho_eff;
}
void or_scene_set_poses(void* h, const double* T0, const double* T1, uint32_t nb, uint32_t slot, uint32_t frame) {
  Scene* S = static_cast<Scene*>(h);
  set_poses(*S, T0, T1, nb);
  write_scene_u(*S, slot, frame);
}
void or_scene_set_eavg(void* h, const float* e, uint32_t slot, uint32_t frame) {
  Scene* S = static_cast<Scene*>(h);
  for (int k = 0; k < 3; k++) S->eAvg[k] = e[k];
  write_scene_u(*S, slot, frame);
}
void or_scene_uniform(void* h, float* out) { Scene* S = static_cast<Scene*>(h); std::copy(S->sceneU, S->sceneU + 24 + 48 * VT_MAX_INST, out); }
void or_scene_set_node_state(void* h, const float* st, uint32_t slot, uint32_t frame) {
  Scene* S = static_cast<Scene*>(h);
  std::copy(st, st + S->nodeState.size(), S->nodeState.begin());
  write_scene_u(*S, slot, frame);
}
// trace (WGSL semantics, precision by flag): o4, d4 -> t, tri, inst, u, v per ray (double)
void or_trace_wgsl(void* h, int n, const float* o4, const float* d4, uint32_t mask, int anyHit, uint32_t root, int fp64, double* out, uint64_t* dbgOut) {
  Scene* S = static_cast<Scene*>(h);
  Dbg dbg;
  auto run = [&](auto tag) {
    using R = decltype(tag);
    Tracer<R> tr(*S, dbg);
    tr.gRoot = root;
    for (int i = 0; i < n; i++) {
      V3<R> o(o4[4 * i], o4[4 * i + 1], o4[4 * i + 2]), d(d4[4 * i], d4[4 * i + 1], d4[4 * i + 2]);
      Hit<R> hh = tr.trace(o, d, R(0), R(BIGD), R(o4[4 * i + 3]), anyHit != 0, mask, 0u);
      double* q = out + 5 * i;
      q[0] = double(hh.t); q[1] = hh.tri == MISS ? -1.0 : double(hh.tri); q[2] = hh.inst == MISS ? -1.0 : double(hh.inst); q[3] = double(hh.u); q[4] = double(hh.v);
    }
  };
  if (fp64) run(double(0)); else run(float(0));
  if (dbgOut) for (int k = 0; k < 16; k++) dbgOut[k] = dbg.c[k];
}
// gpu/wgsl/kernels.wgsl.js:494-551 lensTest / bsdfTest / capsuleTest / profileTest on the CPU, with the same float4
// input and output slots (kind 0 lens, 1 BSDF, 2 capsule, 3 profile); lens = fx, fy, cx, cy, k1..k4, alpha. fp64 = 0
// is the float32 WGSL-order restatement, 1 the float64 one (gpu/lens.js's 20-step inverse, gpu/bsdf.js).
void or_unit_test(void* h, uint32_t kind, const double* lens, int n, const float* in, float* out, int fp64) {
  Scene* S = static_cast<Scene*>(h);
  Dbg dbg;
  auto run = [&](auto tag) {
    using R = decltype(tag);
    Tracer<R> tr(*S, dbg);
    Shader<R> sh(tr);
    auto v3 = [&](int slot) { const float* p = in + 4 * size_t(slot); return V3<R>(R(p[0]), R(p[1]), R(p[2])); };
    auto put = [&](int slot, R a, R b, R c, R d) {
      float* o = out + 4 * size_t(slot);
      o[0] = float(a); o[1] = float(b); o[2] = float(c); o[3] = float(d);
    };
    for (int i = 0; i < n; i++) {
      if (kind == 0) {
        Lens L{lens[0], lens[1], lens[2], lens[3], lens[8], {lens[4], lens[5], lens[6], lens[7]}};
        if (sizeof(R) == 4) {   // the device's float lens: its parameters rounded to float32 first
          L.fx = float(L.fx); L.fy = float(L.fy); L.cx = float(L.cx); L.cy = float(L.cy); L.alpha = float(L.alpha);
          for (double& k : L.k) k = float(k);
        }
        V3<R> r = kb4_unproject<R>(L, R(in[4 * i]), R(in[4 * i + 1]));
        R uv[2];
        const float* X = in + 4 * size_t(n + i);
        kb4_project<R>(L, R(X[0]), R(X[1]), R(X[2]), uv);
        put(2 * i, r.x, r.y, r.z, R(0));
        put(2 * i + 1, uv[0], uv[1], R(0), R(0));
      } else if (kind == 1) {
        const float mw = in[16 * size_t(i) + 15];
        const uint32_t m = uint32_t(mw);
        if (!(mw >= 0.0f) || m >= S->nMat) {
          const R q = std::numeric_limits<R>::quiet_NaN();
          for (int k = 0; k < 3; k++) put(3 * i + k, q, q, q, q);
          continue;
        }
        V3<R> nn = v3(4 * i), l = v3(4 * i + 1), v = v3(4 * i + 2), u = v3(4 * i + 3), ls;
        MatR<R> M = sh.load_mat(m);
        V3<R> f = eval_bsdf(M, nn, l, v);
        R pdf = pdf_bsdf(M, nn, v, l);
        R sp = sample_bsdf(M, nn, v, u, ls);
        V3<R> a = sh.albedo(m, dot(nn, v), 0);
        V3<R> ln = Shader<R>::layer_normal(nn, l * R(0.1), normalize(v + V3<R>(R(0.3f), R(0.1f), R(0.2f))), R(2e-4f), R(2e-5f));
        put(3 * i, f.x, f.y, f.z, pdf);
        if (sp > R(0)) put(3 * i + 1, ls.x, ls.y, ls.z, sp); else put(3 * i + 1, R(0), R(0), R(0), R(0));
        put(3 * i + 2, a.x, a.y, a.z, ln.x);
      } else if (kind == 2) {
        const float* a = in + 16 * size_t(i) + 8;
        R o = capsule_occ<R>(v3(4 * i), v3(4 * i + 1), V3<R>(R(a[0]), R(a[1]), R(a[2])), v3(4 * i + 3), R(a[3]));
        put(i, o, R(0), R(0), R(0));
      } else {
        put(i, sh.profile(R(in[4 * i])), R(0), R(0), R(0));
      }
    }
  };
  if (fp64) run(double(0)); else run(float(0));
}
// render rows [y0, y1) of a camera; out: w x (y1-y0) x 4 doubles. threads > 1 splits rows.
void or_render(void* h, const vt_render_req* q, uint32_t y0, uint32_t y1, uint32_t x0, uint32_t x1, int fp64, int threads, double* out, uint64_t* dbgOut) {
  Scene* S = static_cast<Scene*>(h);
  const vt_camera_desc& cam = S->cams[q->camera];
  uint32_t skip = 0;
  for (size_t i = 0; i < S->blas.size(); i++) if (S->blas[i].owner == int(q->camera)) skip |= 1u << i;
  const uint32_t w = x1 - x0, extra = std::min(q->refine, 64u);
  // with a refinement pass, pass 1 covers the region grown by one pixel (the 3x3 neighbourhood test)
  const uint32_t gy0 = extra && y0 > 0 ? y0 - 1 : y0, gy1 = extra ? std::min(y1 + 1, cam.height) : y1;
  const uint32_t gx0 = extra && x0 > 0 ? x0 - 1 : x0, gx1 = extra ? std::min(x1 + 1, cam.width) : x1, gw = gx1 - gx0;
  std::vector<double> acc1(extra ? size_t(gy1 - gy0) * gw * 3 : 0);
  std::vector<uint32_t> key1(extra ? size_t(gy1 - gy0) * gw : 0);
  std::vector<Dbg> dbgs(std::max(1, threads));
  auto parallel = [&](uint32_t r0, uint32_t r1, auto&& row) {
    std::atomic<uint32_t> next(r0);
    auto work = [&](int t) {
      for (;;) {
        uint32_t y = next.fetch_add(1);
        if (y >= r1) break;
        row(t, y);
      }
    };
    if (threads <= 1) work(0);
    else {
      std::vector<std::thread> th;
      for (int t = 0; t < threads; t++) th.emplace_back(work, t);
      for (auto& x : th) x.join();
    }
  };
  auto run = [&](auto tag) {
    using R = decltype(tag);
    if (!extra) {
      parallel(y0, y1, [&](int t, uint32_t y) {
        Tracer<R> tr(*S, dbgs[t]);
        tr.gRoot = q->root;
        Shader<R> sh(tr);
        for (uint32_t x = x0; x < x1; x++) render_pixel<R>(tr, sh, cam, q->camera, *q, x, y, skip, out + (size_t(y - y0) * w + (x - x0)) * 4);
      });
      return;
    }
    const uint32_t spp = pass1_spp(*q);
    parallel(gy0, gy1, [&](int t, uint32_t y) {
      Tracer<R> tr(*S, dbgs[t]);
      tr.gRoot = q->root;
      Shader<R> sh(tr);
      for (uint32_t x = gx0; x < gx1; x++) {
        V3<R> a;
        uint32_t k = 0;
        pixel_samples<R>(tr, sh, cam, q->camera, *q, x, y, skip, 0, spp, q->light_samples, a, k);
        const size_t j = size_t(y - gy0) * gw + (x - gx0);
        acc1[3 * j] = double(a.x); acc1[3 * j + 1] = double(a.y); acc1[3 * j + 2] = double(a.z);
        key1[j] = k;
      }
    });
    // gpu/wgsl/kernels.wgsl.js:218-252 camRefine
    std::vector<Dbg> rdbg(std::max(1, threads));
    const uint32_t nl2 = q->refine_light_samples ? q->refine_light_samples : q->light_samples;
    parallel(y0, y1, [&](int t, uint32_t y) {
      Tracer<R> tr(*S, dbgs[t]);
      tr.gRoot = q->root;
      Shader<R> sh(tr);
      for (uint32_t x = x0; x < x1; x++) {
        const size_t j = size_t(y - gy0) * gw + (x - gx0);
        uint32_t k = key1[j];
        bool want = (k & 0x50000u) != 0u || ((k & 0x20000u) != 0u && (q->options & VT_O_REFINE_SHADOW) != 0u);
        for (int dy = -1; dy <= 1 && !want; dy++)
          for (int dx = -1; dx <= 1; dx++) {
            const uint32_t xx = uint32_t(std::min(std::max(int(x) + dx, 0), int(cam.width) - 1));
            const uint32_t yy = uint32_t(std::min(std::max(int(y) + dy, 0), int(cam.height) - 1));
            if ((key1[size_t(yy - gy0) * gw + (xx - gx0)] & 0xffffu) != (k & 0xffffu)) want = true;
          }
        V3<R> a(R(acc1[3 * j]), R(acc1[3 * j + 1]), R(acc1[3 * j + 2]));
        double* o = out + (size_t(y - y0) * w + (x - x0)) * 4;
        if (!want) {
          R sc = R(q->scale) / R(spp);
          o[0] = double(a.x * sc); o[1] = double(a.y * sc); o[2] = double(a.z * sc);
          o[3] = k == 0xfffeu ? 0.0 : 1.0;
          continue;
        }
        rdbg[t].c[2]++;
        if (k & 0x10000u) rdbg[t].c[3]++;
        if (k & 0x20000u) rdbg[t].c[4]++;
        if (k & 0x40000u) rdbg[t].c[5]++;
        pixel_samples<R>(tr, sh, cam, q->camera, *q, x, y, skip, spp, spp + extra, nl2, a, k);
        R sc = R(q->scale) / R(spp + extra);
        o[0] = double(a.x * sc); o[1] = double(a.y * sc); o[2] = double(a.z * sc);
        o[3] = 1.0;
      }
    });
    for (int t = 0; t < std::max(1, threads); t++)
      for (int c = 2; c <= 5; c++) dbgs[t].c[c] += rdbg[t].c[c];
  };
  if (fp64) run(double(0)); else run(float(0));
  if (dbgOut) for (int k = 0; k < 16; k++) { dbgOut[k] = 0; for (auto& d : dbgs) dbgOut[k] += d.c[k]; }
}

// the calibration render with optional frozen path decisions (fz_ti, fz_q: see CalibIn; null for the estimator) and
// optional intrinsics K (fx, fy, cx, cy, k1..k4; null: the scene camera's)
void or_calib_render_frozen(void* h, uint32_t camera, uint32_t spp, uint32_t nl, uint32_t seed, uint32_t depth, const double* albedo,
                            const double* lamp, const double* H, uint32_t nNodes, const uint32_t* triNode, uint32_t y0, uint32_t y1, int fp64,
                            int threads, const uint32_t* fz_ti, const float* fz_q, const double* K, double* out) {
  Scene* S = static_cast<Scene*>(h);
  vt_camera_desc cam = S->cams[camera];
  if (K) { cam.fx = K[0]; cam.fy = K[1]; cam.cx = K[2]; cam.cy = K[3]; for (int k = 0; k < 4; k++) cam.k[k] = K[4 + k]; }
  uint32_t skip = 0;
  for (size_t i = 0; i < S->blas.size(); i++) if (S->blas[i].owner == int(camera)) skip |= 1u << i;
  CalibIn C{albedo, lamp, H, nNodes, triNode, S->staticTris, fz_ti, fz_q};
  const uint32_t w = cam.width;
  std::atomic<uint32_t> next(y0);
  std::vector<Dbg> dbgs(std::max(1, threads));
  auto work = [&](int t) {
    auto run = [&](auto tag) {
      using R = decltype(tag);
      Tracer<R> tr(*S, dbgs[t]);
      Shader<R> sh(tr);
      for (;;) {
        uint32_t y = next.fetch_add(1);
        if (y >= y1) break;
        for (uint32_t x = 0; x < w; x++) calib_pixel<R>(tr, sh, C, cam, camera, spp, nl, seed, depth, x, y, skip, out + (size_t(y - y0) * w + x) * 3);
      }
    };
    if (fp64) run(double(0)); else run(float(0));
  };
  if (threads <= 1) work(0);
  else {
    std::vector<std::thread> th;
    for (int t = 0; t < threads; t++) th.emplace_back(work, t);
    for (auto& x : th) x.join();
  }
}

void or_calib_render(void* h, uint32_t camera, uint32_t spp, uint32_t nl, uint32_t seed, uint32_t depth, const double* albedo,
                     const double* lamp, const double* H, uint32_t nNodes, const uint32_t* triNode, uint32_t y0, uint32_t y1, int fp64,
                     int threads, double* out) {
  or_calib_render_frozen(h, camera, spp, nl, seed, depth, albedo, lamp, H, nNodes, triNode, y0, y1, fp64, threads, nullptr, nullptr, nullptr, out);
}

void or_direct_transfer(void* h, const float* C, const float* N, uint32_t n, uint32_t samples, int fp64, int threads, double* D) {
  Scene* S = static_cast<Scene*>(h);
  std::atomic<uint32_t> next(0);
  std::vector<Dbg> dbgs(std::max(1, threads));
  auto work = [&](int t) {
    auto run = [&](auto tag) {
      using R = decltype(tag);
      Tracer<R> tr(*S, dbgs[t]);
      Shader<R> sh(tr);
      for (;;) {
        uint32_t i = next.fetch_add(16);
        if (i >= n) break;
        direct_transfer<R>(tr, sh, C, N, i, std::min(n, i + 16), samples, D);
      }
    };
    if (fp64) run(double(0)); else run(float(0));
  };
  if (threads <= 1) work(0);
  else {
    std::vector<std::thread> th;
    for (int t = 0; t < threads; t++) th.emplace_back(work, t);
    for (auto& x : th) x.join();
  }
}
uint32_t or_scene_emit_count(void* h) { return static_cast<Scene*>(h)->emitN; }

// dense form factors with visibility through the scene, restated: disk form factor of the centres x the fraction
// of K rays between the two patch discs (half radius, Kronecker sample k on each disc with its own shift, lifted
// 5 mm + a tenth of the half radius) that no surface blocks (the emitter body does not occlude); each unordered
// pair traced once; rows
// scaled to a sum <= 1 in FP64
void or_form_factors_visible(void* h, int n, const float* C, const float* Nn, const float* A, int K, int fp64, int threads, float* F,
                             uint8_t* counts) {
  Scene* S = static_cast<Scene*>(h);
  std::vector<Dbg> dbgs(std::max(1, threads));
  std::atomic<int> next(0);
  auto work = [&](int t) {
    auto run = [&](auto tag) {
      using R = decltype(tag);
      Tracer<R> tr(*S, dbgs[t]);
      auto disc = [&](int i, float u, float v) {
        V3<R> c = ld3<R>(C + 3 * i), nn = ld3<R>(Nn + 3 * i);
        R rh = R(0.5) * std::sqrt(R(A[i]) * R(INV_PI_D)), r = rh * std::sqrt(R(u));
        R ph = R(2) * R(M_PI) * R(v);
        return c + basis_t(nn) * (r * std::cos(ph)) + basis_b(nn) * (r * std::sin(ph)) + nn * (R(5e-3) + R(0.1) * rh);
      };
      for (;;) {
        int i = next.fetch_add(1);
        if (i >= n) break;
        for (int j = i + 1; j < n; j++) {
          float wx = C[3 * j] - C[3 * i], wy = C[3 * j + 1] - C[3 * i + 1], wz = C[3 * j + 2] - C[3 * i + 2];
          bool face = Nn[3 * i] * wx + Nn[3 * i + 1] * wy + Nn[3 * i + 2] * wz > 0.0f && Nn[3 * j] * wx + Nn[3 * j + 1] * wy + Nn[3 * j + 2] * wz < 0.0f;
          int vis = 0;
          if (face) {
            for (int k = 0; k < K; k++) {
              V3<R> a = disc(i, kr(k, R2A, 0.5f), kr(k, R2B, 0.5f)), b = disc(j, kr(k, R2A, 0.25f), kr(k, R2B, 0.75f));
              V3<R> w = b - a;
              R dist = len(w);
              if (!(dist > R(2e-4))) { vis++; continue; }
              Hit<R> hh = tr.trace(a, w / dist, R(0), dist - R(1e-4), R(0.5), true, 3u, tr.su_u(7));
              if (hh.tri == MISS) vis++;
            }
          }
          counts[size_t(i) * n + j] = counts[size_t(j) * n + i] = uint8_t(vis);
        }
      }
    };
    if (fp64) run(double(0)); else run(float(0));
  };
  for (int i = 0; i < n; i++) counts[size_t(i) * n + i] = 0;
  if (threads <= 1) work(0);
  else {
    std::vector<std::thread> th;
    for (int t = 0; t < threads; t++) th.emplace_back(work, t);
    for (auto& x : th) x.join();
  }
  for (int i = 0; i < n; i++) {
    std::vector<double> row(n, 0.0);
    double s = 0;
    for (int j = 0; j < n; j++) {
      if (j == i || !counts[size_t(i) * n + j]) continue;
      double wx = double(C[3 * j]) - C[3 * i], wy = double(C[3 * j + 1]) - C[3 * i + 1], wz = double(C[3 * j + 2]) - C[3 * i + 2];
      double r2 = wx * wx + wy * wy + wz * wz, r = std::sqrt(r2);
      if (!(r > 0)) continue;
      double ci = (Nn[3 * i] * wx + Nn[3 * i + 1] * wy + Nn[3 * i + 2] * wz) / r;
      double cj = -(Nn[3 * j] * wx + Nn[3 * j + 1] * wy + Nn[3 * j + 2] * wz) / r;
      if (ci <= 0 || cj <= 0) continue;
      row[j] = double(A[j]) * ci * cj / (M_PI * r2 + double(A[j])) * (double(counts[size_t(i) * n + j]) / K);
      s += row[j];
    }
    double sc = s > 1.0 ? 1.0 / s : 1.0;
    for (int j = 0; j < n; j++) F[size_t(i) * n + j] = float(row[j] * sc);
  }
}

void or_sensor_expose(const uint32_t* su, const float* E4, float* raw) { sensor_expose(su, E4, raw); }
void or_isp_chain(const uint32_t* su, const float* L4, const float* ri, float* raw, uint8_t* rgba, uint8_t* yuv, uint32_t* stats) {
  isp_chain(su, L4, ri, raw, rgba, yuv, stats);
}
void or_scene_ri_map(void* h, uint32_t camera, double q, const double* vdeg, const double* vv, uint32_t nv, float* out) {
  ri_map(static_cast<Scene*>(h)->cams[camera], q, vdeg, vv, nv, out);
}
void or_vt_logf(const float* x, int n, float* out) { for (int i = 0; i < n; i++) out[i] = vt_logf(x[i]); }
void or_vt_expf(const float* x, int n, float* out) { for (int i = 0; i < n; i++) out[i] = vt_expf(x[i]); }
void or_vt_cos2pi(const float* x, int n, float* out) { for (int i = 0; i < n; i++) out[i] = vt_cos2pi(x[i]); }

void or_solve_dense(int n, const float* F, const float* rho, const float* E, int R, double* B) { solve_dense(n, F, rho, E, R, B); }
int or_jacobi64(int n, const float* F, const float* rho, const float* E, int R, double* B, double tol, int maxIt, int threads) {
  return jacobi64(n, F, rho, E, R, B, tol, maxIt, threads);
}
void or_form_factors(int n, const float* C, const float* Nn, const float* A, float* F) { form_factors(n, C, Nn, A, F); }

// gather table of every static vertex (K rays each): build, escape counts, remap (gpu/renderer.js:456-500)
void or_gather_table(void* h, uint32_t K, int fp64, int threads, uint32_t* gtable, float* misses) {
  Scene* S = static_cast<Scene*>(h);
  const uint32_t n = S->staticVerts;
  auto run = [&](auto tag) {
    using R = decltype(tag);
    Dbg dbg;
    parallel_for(size_t(n) * K, threads, [&](size_t r) {
      Dbg d;
      Tracer<R> tr(*S, d);
      Shader<R> sh(tr);
      NodeRad<R> nr(tr, sh);
      gtable[r] = nr.build(uint32_t(r / K), uint32_t(r % K), K);
    });
    for (uint32_t i = 0; i < n; i++) {
      uint32_t m = 0;
      for (uint32_t j = 0; j < K; j++) m += gtable[size_t(i) * K + j] == MISS;
      misses[i] = float(m);
    }
    parallel_for(size_t(n) * K, threads, [&](size_t r) {
      Dbg d;
      Tracer<R> tr(*S, d);
      Shader<R> sh(tr);
      NodeRad<R> nr(tr, sh);
      gtable[r] = nr.remap(uint32_t(r / K), uint32_t(r % K), K, gtable[r], misses);
    });
  };
  if (fp64) run(double(0)); else run(float(0));
}

// gpu/renderer.js:573 _neighbours by brute force: the nbrK largest Gaussian weights (ties: smaller active index)
// over active nodes within R that face the same way (n.n >= 0.9); out: nA x nbrK x (index, float weight bits)
void or_node_neighbours(void* h, const uint32_t* active, uint32_t nA, uint32_t nbrK, double R, double sg, uint32_t* out) {
  Scene* S = static_cast<Scene*>(h);
  std::fill(out, out + size_t(nA) * nbrK * 2, 0u);
  auto vf = [&](uint32_t i, int w) { return double(as_f(S->verts[8 * size_t(i) + w])); };
  for (uint32_t k = 0; k < nA; k++) {
    if (!(sg > 0)) { out[size_t(k) * nbrK * 2] = k; float one = 1.0f; std::memcpy(&out[size_t(k) * nbrK * 2 + 1], &one, 4); continue; }
    const uint32_t i = active[k];
    std::vector<std::pair<double, uint32_t>> c;
    for (uint32_t m = 0; m < nA; m++) {
      const uint32_t j = active[m];
      double ex = vf(j, 0) - vf(i, 0), ey = vf(j, 1) - vf(i, 1), ez = vf(j, 2) - vf(i, 2), d2 = ex * ex + ey * ey + ez * ez;
      if (d2 > R * R) continue;
      if (vf(i, 4) * vf(j, 4) + vf(i, 5) * vf(j, 5) + vf(i, 6) * vf(j, 6) < 0.9) continue;
      c.push_back({std::exp(-0.5 * d2 / (sg * sg)), m});
    }
    std::sort(c.begin(), c.end(), [](const auto& a, const auto& b) { return a.first > b.first || (a.first == b.first && a.second < b.second); });
    for (size_t q = 0; q < std::min<size_t>(c.size(), nbrK); q++) {
      float w = float(c[q].first);
      out[(size_t(k) * nbrK + q) * 2] = c[q].second;
      std::memcpy(&out[(size_t(k) * nbrK + q) * 2 + 1], &w, 4);
    }
  }
}

// nodeDirect over the active nodes (moved != 0: only those near a moved body); st: n x 16 doubles, in and out
void or_node_direct(void* h, const uint32_t* active, uint32_t nA, uint32_t NS, uint32_t moved, int fp64, int threads, double* st) {
  Scene* S = static_cast<Scene*>(h);
  auto run = [&](auto tag) {
    using R = decltype(tag);
    parallel_for(nA, threads, [&](size_t k) {
      Dbg d;
      Tracer<R> tr(*S, d);
      Shader<R> sh(tr);
      NodeRad<R> nr(tr, sh);
      const uint32_t i = active[k];
      R o[5];
      if (!nr.direct(i, NS, moved, o)) return;
      double* q = st + 16 * size_t(i);
      q[12] = double(o[0]); q[13] = double(o[1]); q[14] = double(o[2]); q[15] = double(o[3]); q[3] = double(o[4]);
    });
  };
  if (fp64) run(double(0)); else run(float(0));
}

// `iters` Jacobi steps from slot slotIn (gather into aux, then update, ping-pong); returns the final slot
uint32_t or_node_jacobi(void* h, const uint32_t* gtable, uint32_t K, const uint32_t* active, uint32_t nA, const uint32_t* nbr, uint32_t nbrK,
                        uint32_t slotIn, uint32_t iters, int fp64, int threads, double* st) {
  Scene* S = static_cast<Scene*>(h);
  std::vector<double> aux(size_t(nA) * 3);
  uint32_t slot = slotIn;
  auto run = [&](auto tag) {
    using R = decltype(tag);
    for (uint32_t it = 0; it < iters; it++) {
      const uint32_t out = slot == 1 ? 2 : 1;
      parallel_for(nA, threads, [&](size_t k) {
        Dbg d;
        Tracer<R> tr(*S, d);
        Shader<R> sh(tr);
        NodeRad<R> nr(tr, sh);
        V3<R> a = nr.gather(active[k], K, gtable, st, slot);
        aux[3 * k] = double(a.x); aux[3 * k + 1] = double(a.y); aux[3 * k + 2] = double(a.z);
      });
      parallel_for(nA, threads, [&](size_t k) {
        Dbg d;
        Tracer<R> tr(*S, d);
        Shader<R> sh(tr);
        NodeRad<R> nr(tr, sh);
        const uint32_t i = active[k];
        V3<R> ef;
        R ws = 0;
        for (uint32_t j = 0; j < nbrK; j++) {
          const uint32_t* e = nbr + (k * nbrK + j) * 2;
          R w = R(as_f(e[1]));
          if (w <= R(0)) break;
          ef = ef + V3<R>(R(aux[3 * e[0]]), R(aux[3 * e[0] + 1]), R(aux[3 * e[0] + 2])) * w;
          ws = ws + w;
        }
        ef = ws > R(0) ? ef / ws : V3<R>(R(aux[3 * k]), R(aux[3 * k + 1]), R(aux[3 * k + 2]));
        double* q = st + 16 * size_t(i);
        V3<R> hh = sh.load_mat(nr.mat(i)).hh;
        R hm[3] = {std::max(hh.x, R(1e-4)), std::max(hh.y, R(1e-4)), std::max(hh.z, R(1e-4))};
        R e3[3] = {ef.x, ef.y, ef.z};
        const R V = R(q[3]);
        for (int c = 0; c < 3; c++) q[4 * out + c] = double((R(q[12 + c]) + e3[c] * V * hm[c]) * R(INV_PI_D) / hm[c]);
        q[4 * out + 3] = 1.0;
        q[0] = double(ef.x); q[1] = double(ef.y); q[2] = double(ef.z);
      });
      slot = out;
    }
  };
  if (fp64) run(double(0)); else run(float(0));
  return slot;
}

void or_scene_set_solved_caps(void* h, const float* caps, uint32_t nb, uint32_t slot, uint32_t frame) {
  Scene* S = static_cast<Scene*>(h);
  S->solvedCaps.assign(caps, caps + 8 * size_t(nb));
  write_scene_u(*S, slot, frame);
}

// ---- raster pass (lite_nodes)
// sizes of the raster geometry: counts = [vertices, triangles]
void or_lite_geometry_size(void* h, double subdiv, double subdiv_fixture, uint32_t* counts) {
  std::vector<uint32_t> V, I;
  lite::geometry(*static_cast<Scene*>(h), subdiv, subdiv_fixture, V, I);
  counts[0] = uint32_t(V.size() / 8);
  counts[1] = uint32_t(I.size() / 3);
}
void or_lite_geometry(void* h, double subdiv, double subdiv_fixture, uint32_t* verts, uint32_t* idx) {
  std::vector<uint32_t> V, I;
  lite::geometry(*static_cast<Scene*>(h), subdiv, subdiv_fixture, V, I);
  std::copy(V.begin(), V.end(), verts);
  std::copy(I.begin(), I.end(), idx);
}
// emitter samples in the world for scope pose T (column-major): 8 floats each; sector origins (4 x 3)
void or_lite_emitter(void* h, uint32_t n, const double* T, float* out, double* sect_c) {
  std::vector<float> es;
  double sc[4][3];
  lite::emitter_world(*static_cast<Scene*>(h), n, T, es, sc);
  std::copy(es.begin(), es.end(), out);
  for (int k = 0; k < 4; k++) for (int j = 0; j < 3; j++) sect_c[3 * k + j] = sc[k][j];
}
// vertex stage: shadow = 0 camera clip coordinates (n x 4); shadow = 1 / 2 the four sector layers (4 x n x 4) of
// the static / dynamic casters (other vertices left as they are in out)
void or_lite_vertex(void* h, const float* view, const uint32_t* verts, uint32_t n, int shadow, float* out) {
  Scene* S = static_cast<Scene*>(h);
  Dbg d;
  Tracer<float> tr(*S, d);
  lite::View V{view};
  for (uint32_t i = 0; i < n; i++) {
    const uint32_t* w = verts + 8 * size_t(i);
    V3<float> p, nn;
    const bool ok = lite::world_of(tr, V, w, p, nn);
    if (!shadow) {
      float* o = out + 4 * size_t(i);
      if (ok) lite::project_cam(V, p, o);
      else { o[0] = 0.0f; o[1] = 0.0f; o[2] = -2.0f; o[3] = 1.0f; }
      continue;
    }
    const bool st = (w[3] >> 16) == 0xffffu;
    if ((shadow == 1) != st) continue;
    const uint32_t flags = as_u(S->params[4 * (S->meshOff + 2 * (w[3] & 0xffffu) + 1)]);
    const bool keep = ok && (flags & (VT_F_EMITTER | VT_F_SCOPE)) == 0u;
    for (int k = 0; k < 4; k++) {
      float* o = out + 4 * (size_t(k) * n + i);
      if (!keep) { o[0] = 0.0f; o[1] = 0.0f; o[2] = -2.0f; o[3] = 1.0f; continue; }
      const V3<float> q = lite::sm_project(V, p, k);
      if (lite::hyp(q.x, q.y) > 1.0f) {
        const float ex = q.x + 1e-12f, ey = q.y, l = lite::hyp(ex, ey);
        o[0] = ex / l; o[1] = ey / l; o[2] = -1e-3f; o[3] = -1e-3f;
      } else {
        o[0] = q.x; o[1] = q.y; o[2] = q.z / view[47]; o[3] = 1.0f;
      }
    }
  }
}
// rasteriser: keys (w x h x samples uint64) start all ones
void or_raster(const float* clip, const uint32_t* idx, uint32_t t0, uint32_t nt, uint32_t W, uint32_t H, uint32_t samples, uint64_t* keys) {
  std::fill(keys, keys + size_t(W) * H * samples, ~0ull);
  lite::raster(clip, idx, t0, nt, W, H, samples, keys);
}
// fragment stage + resolve + finish for rows [y0, y1) from the given keys, clip coordinates and shadow maps
void or_lite_shade(void* h, const float* view, const uint32_t* verts, const uint32_t* idx, const float* clip, const uint64_t* keys,
                   const float* es, const uint32_t* sm_static, const uint32_t* sm_dyn, uint32_t res, float inv_scale, float circle,
                   uint32_t y0, uint32_t y1, int threads, float* out) {
  Scene* S = static_cast<Scene*>(h);
  const uint32_t W = uint32_t(view[24]), H = uint32_t(view[25]);
  y1 = std::min(y1, H);
  parallel_for(y1 > y0 ? y1 - y0 : 0, threads, [&](size_t r) {
    Dbg d;
    Tracer<float> tr(*S, d);
    Shader<float> sh(tr);
    lite::View V{view};
    lite::Frag F{tr, sh, V, verts, idx, clip, es, sm_static, sm_dyn, res};
    const uint32_t py = y0 + uint32_t(r);
    for (uint32_t px = 0; px < W; px++) {
      const uint64_t* k = keys + (size_t(py) * W + px) * 4;
      V3<float> col[4];
      bool done[4] = {false, false, false, false};
      for (int s = 0; s < 4; s++) {
        if (done[s]) continue;
        V3<float> c;
        if (k[s] != ~0ull) {
          c = F.shade(uint32_t(k[s] & 0xffffffffu), px, py);
          c = V3<float>(lite::h16(c.x), lite::h16(c.y), lite::h16(c.z));
        }
        for (int t = s; t < 4; t++)
          if (!done[t] && uint32_t(k[t]) == uint32_t(k[s])) { col[t] = c; done[t] = true; }
      }
      float rgb[3];
      for (int ch = 0; ch < 3; ch++) {
        const float v = ((((ch == 0 ? col[0].x : ch == 1 ? col[0].y : col[0].z) + (ch == 0 ? col[1].x : ch == 1 ? col[1].y : col[1].z)) +
                          (ch == 0 ? col[2].x : ch == 1 ? col[2].y : col[2].z)) + (ch == 0 ? col[3].x : ch == 1 ? col[3].y : col[3].z)) * 0.25f;
        rgb[ch] = lite::h16(v) * inv_scale;
      }
      if (circle > 0.0f) {
        const float qx = float(px) + 0.5f - 0.5f * float(W), qy = float(py) + 0.5f - 0.5f * float(H);
        if (lite::hyp(qx, qy) > circle) rgb[0] = rgb[1] = rgb[2] = 0.0f;
      }
      float* o = out + 4 * (size_t(py) * W + px);
      o[0] = rgb[0]; o[1] = rgb[1]; o[2] = rgb[2]; o[3] = 1.0f;
    }
  });
}
// the display look (DISPLAY): rgba8 and stats (luma sum, count)
void or_lite_display(const float* du, const uint32_t* prev, const float* L4, uint32_t W, uint32_t H, uint8_t* rgba, uint32_t* stats) {
  stats[0] = stats[1] = stats[2] = stats[3] = 0;
  const float n = std::max(float(prev[1]), 1.0f);
  const float mean = float(prev[0]) / std::max(du[3], 1e-30f) / n;
  for (uint32_t y = 0; y < H; y++)
    for (uint32_t x = 0; x < W; x++) {
      const float* l = L4 + 4 * (size_t(y) * W + x);
      if ((x & 3u) == 0u && (y & 3u) == 0u) {
        const float yl = l[0] * 0.2126f + l[1] * 0.7152f + l[2] * 0.0722f;
        stats[0] += uint32_t(std::min(std::max(yl * du[3], 0.0f), 65535.0f));
        stats[1] += 1;
      }
      float E[3] = {l[0], l[1], l[2]};
      if (du[12] > 0.0f) {
        const float qx = (float(x) + 0.5f - du[14]) / du[12], qy = (float(y) + 0.5f - du[15]) / du[13];
        const float c = clamp01(std::sqrt(qx * qx + qy * qy) / 1.1f);
        const float t = c * c;
        const float f = 1.0f * (1.0f - t) + 0.57f * t;
        for (float& e : E) e = e * f;
      }
      uint8_t* o = rgba + 4 * (size_t(y) * W + x);
      for (int k = 0; k < 3; k++) {
        const float e = (1.0f - du[1]) * E[k] + du[1] * mean;
        const float xv = e * du[0] * du[4 + k];
        const float v = clamp01((xv - du[9]) / (1.0f - du[9]));
        float t = srgb_oetf(v);
        if (du[8] > 0.0f) {
          const float a = vt_powf(clamp01(t), du[8]);
          t = a / (a + vt_powf(clamp01(1.0f - t), du[8]));
        }
        o[k] = uint8_t(std::lrint(t * 255.0f));
      }
      o[3] = 255;
    }
}
// load a scene uniform as given (the raster pass's shading reads the poses, the slot and the capsules from it)
void or_scene_load_uniform(void* h, const float* su) {
  Scene* S = static_cast<Scene*>(h);
  std::copy(su, su + 24 + 48 * VT_MAX_INST, S->sceneU);
}

}  // extern "C"

