// Host scene preparation for libvtwin (see vt_host.h). The arrays it writes are the device layout the kernels
// read, and they are the reference's own layouts (gpu/bvh.js:5-11 nodes, gpu/scene_gpu.js:351-393 triangles and
// vertices, gpu/renderer.js:273-306 params), so a scene prepared here and one prepared by the reference match
// word for word.
#include "vt_host.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <limits>
#include <stdexcept>
#include <thread>

namespace vt {

static inline uint32_t fbits(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }
static const double kBig = 1e30;

// ------------------------------------------------------------------------------------------------------ BVH
// Binned SAH over triangle centroids, 16 bins per axis, traversal and intersection cost 1 (gpu/bvh.js:18-161):
// the same split choices (float64 bin bounds over float32 triangle boxes), the same in-place partition of the
// slot order, and the same node numbering (LIFO task order, both children of a node decided before either is
// expanded), so the node array is identical to the reference builder's.
namespace {
struct Box { double lo[3], hi[3], clo[3], chi[3]; };

class SahBuilder {
 public:
  SahBuilder(const float* P, const uint32_t* I, uint32_t n, uint32_t leaf) : n_(n), leaf_(leaf) {
    bmin_.resize(3 * size_t(n)); bmax_.resize(3 * size_t(n)); cen_.resize(3 * size_t(n));
    for (uint32_t t = 0; t < n; t++) {
      const float* a = P + 3 * size_t(I[3 * t]);
      const float* b = P + 3 * size_t(I[3 * t + 1]);
      const float* c = P + 3 * size_t(I[3 * t + 2]);
      for (int k = 0; k < 3; k++) {
        double lo = std::min(std::min(double(a[k]), double(b[k])), double(c[k]));
        double hi = std::max(std::max(double(a[k]), double(b[k])), double(c[k]));
        bmin_[3 * t + k] = float(lo);
        bmax_[3 * t + k] = float(hi);
        cen_[3 * t + k] = float(0.5 * (lo + hi));
      }
    }
    out_.order.resize(n);
    for (uint32_t i = 0; i < n; i++) out_.order[i] = i;
  }

  // The children of a node are decided (bounds, split and partition of their slot ranges) independently of every
  // other node's, so subtrees are decided in parallel on the host's threads; the node numbering is then replayed in
  // the sequential builder's task order (LIFO, both children of a node numbered before either is expanded), which
  // gives the same node array as building one task at a time.
  Bvh run() {
    uint32_t root = new_node();
    Box all = bounds(0, n_);
    if (n_ == 0) {
      double far_[3] = {kBig, kBig, kBig};
      put(root, 0, far_, far_, 0, 1);
      put(root, 1, far_, far_, 0, 1);
    } else {
      int64_t m = choose(0, n_, all);
      if (m < 0) {
        uint32_t h = n_ > 1 ? n_ / 2 : n_;
        Box b0 = bounds(0, h);
        put(root, 0, b0.lo, b0.hi, 0, h);
        if (n_ > 1) { Box b1 = bounds(h, n_); put(root, 1, b1.lo, b1.hi, h, n_ - h); }
        else put(root, 1, all.lo, all.hi, 0, n_);
      } else {
        shapes_.resize(std::max<size_t>(1, n_));
        shapes_[0].s = 0; shapes_[0].e = int64_t(n_); shapes_[0].m = m;
        n_shapes_ = 1;
        threads_left_ = int(std::max(1u, std::thread::hardware_concurrency())) - 1;
        decide(0);
        number(root);
      }
    }
    for (int k = 0; k < 3; k++) { out_.lo[k] = float(all.lo[k]); out_.hi[k] = float(all.hi[k]); }
    return std::move(out_);
  }

 private:
  // an interior node: its range [s, e) split at m, and per child its bounds and either a leaf or an interior child
  struct Shape {
    int64_t s = 0, e = 0, m = 0;
    Box b[2];
    int64_t child[2] = {-1, -1};
  };
  static constexpr int kBins = 16;
  static constexpr int64_t kParallelMin = 8192;   // ranges at least this large are decided on their own thread

  void decide(int64_t si) {
    const int64_t lo[2] = {shapes_[si].s, shapes_[si].m}, hi[2] = {shapes_[si].m, shapes_[si].e};
    auto slot_of = [&](int slot) {
      Shape& S = shapes_[si];
      S.b[slot] = bounds(lo[slot], hi[slot]);
      const int64_t mm = choose(lo[slot], hi[slot], S.b[slot]);
      if (mm >= 0) {
        const int64_t c = n_shapes_.fetch_add(1);
        shapes_[c].s = lo[slot]; shapes_[c].e = hi[slot]; shapes_[c].m = mm;
        S.child[slot] = c;
      }
    };
    const bool split = hi[0] - lo[0] >= kParallelMin && hi[1] - lo[1] >= kParallelMin && take_thread();
    if (split) {
      std::thread t([&] { slot_of(0); if (shapes_[si].child[0] >= 0) decide(shapes_[si].child[0]); });
      slot_of(1);
      if (shapes_[si].child[1] >= 0) decide(shapes_[si].child[1]);
      t.join();
      threads_left_.fetch_add(1);
    } else {
      slot_of(0);
      slot_of(1);
      for (int slot = 0; slot < 2; slot++)
        if (shapes_[si].child[slot] >= 0) decide(shapes_[si].child[slot]);
    }
  }
  bool take_thread() {
    int k = threads_left_.load();
    while (k > 0)
      if (threads_left_.compare_exchange_weak(k, k - 1)) return true;
    return false;
  }
  // node numbers in task order: pop a node, number its interior children (slot 0 then 1), push them
  void number(uint32_t root) {
    struct Item { int64_t shape; uint32_t node, depth; };
    std::vector<Item> stack{{0, root, 1}};
    while (!stack.empty()) {
      const Item it = stack.back();
      stack.pop_back();
      out_.max_depth = std::max(out_.max_depth, it.depth);
      const Shape& S = shapes_[it.shape];
      const int64_t lo[2] = {S.s, S.m}, hi[2] = {S.m, S.e};
      for (int slot = 0; slot < 2; slot++) {
        if (S.child[slot] < 0) {
          put(it.node, slot, S.b[slot].lo, S.b[slot].hi, uint32_t(lo[slot]), uint32_t(hi[slot] - lo[slot]));
        } else {
          const uint32_t child = new_node();
          put(it.node, slot, S.b[slot].lo, S.b[slot].hi, child, 0);
          stack.push_back({S.child[slot], child, it.depth + 1});
        }
      }
    }
  }

  uint32_t new_node() { out_.words.resize(out_.words.size() + VT_NODE_WORDS, 0u); return out_.node_count++; }
  void put(uint32_t node, int slot, const double* lo, const double* hi, uint32_t ref, uint32_t count) {
    uint32_t* w = out_.words.data() + size_t(node) * VT_NODE_WORDS + slot * 8;
    w[0] = fbits(float(lo[0])); w[1] = fbits(float(lo[1])); w[2] = fbits(float(lo[2])); w[3] = ref;
    w[4] = fbits(float(hi[0])); w[5] = fbits(float(hi[1])); w[6] = fbits(float(hi[2])); w[7] = count;
  }
  Box bounds_serial(int64_t s, int64_t e) const {
    Box b;
    for (int k = 0; k < 3; k++) { b.lo[k] = kBig; b.hi[k] = -kBig; b.clo[k] = kBig; b.chi[k] = -kBig; }
    for (int64_t i = s; i < e; i++) {
      const uint32_t t = out_.order[i];
      for (int k = 0; k < 3; k++) {
        double a = bmin_[3 * t + k], z = bmax_[3 * t + k], c = cen_[3 * t + k];
        if (a < b.lo[k]) b.lo[k] = a;
        if (z > b.hi[k]) b.hi[k] = z;
        if (c < b.clo[k]) b.clo[k] = c;
        if (c > b.chi[k]) b.chi[k] = c;
      }
    }
    return b;
  }
  // minima and maxima do not depend on the order they are taken in: large ranges are split over threads
  Box bounds(int64_t s, int64_t e) const {
    const int nt = chunks(e - s);
    if (nt <= 1) return bounds_serial(s, e);
    std::vector<Box> part(nt);
    std::vector<std::thread> th;
    for (int t = 0; t < nt; t++) th.emplace_back([&, t] { part[t] = bounds_serial(s + (e - s) * t / nt, s + (e - s) * (t + 1) / nt); });
    for (auto& x : th) x.join();
    Box b = part[0];
    for (int t = 1; t < nt; t++)
      for (int k = 0; k < 3; k++) {
        b.lo[k] = std::min(b.lo[k], part[t].lo[k]); b.hi[k] = std::max(b.hi[k], part[t].hi[k]);
        b.clo[k] = std::min(b.clo[k], part[t].clo[k]); b.chi[k] = std::max(b.chi[k], part[t].chi[k]);
      }
    return b;
  }
  static int chunks(int64_t n) {
    if (n < 131072) return 1;
    return int(std::max<int64_t>(1, std::min<int64_t>(std::thread::hardware_concurrency(), n / 65536)));
  }
  struct Bins {
    uint32_t count[16];
    double lo[16][3], hi[16][3];
  };
  void bin_range(int64_t s, int64_t e, int ax, double origin, double scale, Bins& B) const {
    for (int b = 0; b < kBins; b++) { B.count[b] = 0; for (int k = 0; k < 3; k++) { B.lo[b][k] = kBig; B.hi[b][k] = -kBig; } }
    for (int64_t i = s; i < e; i++) {
      const uint32_t t = out_.order[i];
      const int64_t b = bin_of(t, ax, origin, scale);
      B.count[b]++;
      for (int k = 0; k < 3; k++) {
        if (bmin_[3 * t + k] < B.lo[b][k]) B.lo[b][k] = bmin_[3 * t + k];
        if (bmax_[3 * t + k] > B.hi[b][k]) B.hi[b][k] = bmax_[3 * t + k];
      }
    }
  }
  static double half_area(const double* lo, const double* hi) {
    double x = std::max(0.0, hi[0] - lo[0]), y = std::max(0.0, hi[1] - lo[1]), z = std::max(0.0, hi[2] - lo[2]);
    return x * y + y * z + z * x;
  }
  int64_t bin_of(uint32_t t, int axis, double origin, double scale) const {
    int64_t b = int64_t(std::floor((double(cen_[3 * t + axis]) - origin) * scale));
    return b >= kBins ? kBins - 1 : b;
  }
  // best split point of [s, e) or -1 for a leaf; partitions the slot order at the chosen plane
  int64_t choose(int64_t s, int64_t e, const Box& B) {
    const int64_t cnt = e - s;
    if (cnt <= 1) return -1;
    double best_cost = std::numeric_limits<double>::infinity();
    int best_axis = -1, best_bin = -1;
    const double parent = half_area(B.lo, B.hi);
    for (int ax = 0; ax < 3; ax++) {
      const double origin = B.clo[ax], extent = B.chi[ax] - origin;
      if (!(extent > 0)) continue;
      const double scale = kBins / extent;
      // counts, minima and maxima per bin: exact whatever the order, so large ranges are binned over threads
      Bins all;
      const int nt = chunks(cnt);
      if (nt <= 1) {
        bin_range(s, e, ax, origin, scale, all);
      } else {
        std::vector<Bins> part(nt);
        std::vector<std::thread> th;
        for (int t = 0; t < nt; t++) th.emplace_back([&, t] { bin_range(s + cnt * t / nt, s + cnt * (t + 1) / nt, ax, origin, scale, part[t]); });
        for (auto& x : th) x.join();
        all = part[0];
        for (int t = 1; t < nt; t++)
          for (int b = 0; b < kBins; b++) {
            all.count[b] += part[t].count[b];
            for (int k = 0; k < 3; k++) { all.lo[b][k] = std::min(all.lo[b][k], part[t].lo[b][k]); all.hi[b][k] = std::max(all.hi[b][k], part[t].hi[b][k]); }
          }
      }
      const uint32_t* count = all.count;
      const double(*blo)[3] = all.lo;
      const double(*bhi)[3] = all.hi;
      uint32_t right_count[kBins];
      double right_area[kBins];
      double lo[3] = {kBig, kBig, kBig}, hi[3] = {-kBig, -kBig, -kBig};
      uint32_t acc = 0;
      for (int b = kBins - 1; b > 0; b--) {
        acc += count[b];
        for (int k = 0; k < 3; k++) { lo[k] = std::min(lo[k], blo[b][k]); hi[k] = std::max(hi[k], bhi[b][k]); }
        right_count[b] = acc;
        right_area[b] = acc ? half_area(lo, hi) : 0.0;
      }
      for (int k = 0; k < 3; k++) { lo[k] = kBig; hi[k] = -kBig; }
      acc = 0;
      for (int b = 0; b < kBins - 1; b++) {
        acc += count[b];
        for (int k = 0; k < 3; k++) { lo[k] = std::min(lo[k], blo[b][k]); hi[k] = std::max(hi[k], bhi[b][k]); }
        if (acc == 0 || right_count[b + 1] == 0) continue;
        const double cost = 1.0 + 1.0 * (double(acc) * half_area(lo, hi) + double(right_count[b + 1]) * right_area[b + 1]) / parent;
        if (cost < best_cost) { best_cost = cost; best_axis = ax; best_bin = b; }
      }
    }
    if (best_axis < 0) return cnt > int64_t(leaf_) * 4 ? s + (cnt >> 1) : -1;
    if (cnt <= int64_t(leaf_) && best_cost >= double(cnt)) return -1;
    const double origin = B.clo[best_axis], scale = kBins / (B.chi[best_axis] - origin);
    int64_t i = s, j = e - 1;
    uint32_t* order = out_.order.data();
    while (i <= j) {
      const uint32_t t = order[i];
      if (bin_of(t, best_axis, origin, scale) <= best_bin) i++;
      else { order[i] = order[j]; order[j] = t; j--; }
    }
    if (i == s || i == e) return s + (cnt >> 1);
    return i;
  }

  uint32_t n_, leaf_;
  std::vector<float> bmin_, bmax_, cen_;
  std::vector<Shape> shapes_;
  std::atomic<int64_t> n_shapes_{0};
  std::atomic<int> threads_left_{0};
  Bvh out_;
};
}  // namespace

Bvh sah_build(const float* P, const uint32_t* I, uint32_t n_tris, uint32_t leaf_size) {
  return SahBuilder(P, I, n_tris, std::max(1u, leaf_size)).run();
}

// ------------------------------------------------------------------------------------------------- materials
// gpu/bsdf.js:25-266 in float64: exact dielectric Fresnel, its cosine-weighted mean by composite Simpson, GGX with
// the height-correlated Smith term, visible-normal sampling (Heitz 2018), and the 32-bin directional-albedo tables.
namespace {
double fresnel(double cosi, double eta) {
  double c = std::min(1.0, std::max(0.0, cosi));
  double s2 = (1 - c * c) / (eta * eta);
  if (s2 >= 1) return 1;
  double ct = std::sqrt(1 - s2);
  double rs = (c - eta * ct) / (c + eta * ct), rp = (eta * c - ct) / (eta * c + ct);
  return 0.5 * (rs * rs + rp * rp);
}
double lambda_ggx(double c, double a) {
  double c2 = std::max(c * c, 1e-12);
  return 0.5 * (-1 + std::sqrt(1 + a * a * (1 - c2) / c2));
}
double g1(double c, double a) { return 1 / (1 + lambda_ggx(c, a)); }
double g2(double l, double v, double a) { return 1 / (1 + lambda_ggx(l, a) + lambda_ggx(v, a)); }
double d_ggx(double nh, double a) {
  if (nh <= 0) return 0;
  double a2 = a * a, d = nh * nh * (a2 - 1) + 1;
  return a2 / (M_PI * d * d);
}
double schlick1(double f0, double c) { return f0 + (1 - f0) * std::pow(1 - std::min(1.0, std::max(0.0, c)), 5.0); }
struct D3 { double x, y, z; };
D3 unit(D3 a) { double l = std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); return {a.x / l, a.y / l, a.z / l}; }
double dot3(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
// visible normal of GGX(a) seen from local direction ve (Heitz 2018)
D3 vndf(D3 ve, double a, double u1, double u2) {
  D3 vh = unit({a * ve.x, a * ve.y, ve.z});
  double lensq = vh.x * vh.x + vh.y * vh.y;
  D3 T1 = lensq > 0 ? D3{-vh.y / std::sqrt(lensq), vh.x / std::sqrt(lensq), 0} : D3{1, 0, 0};
  D3 T2 = {vh.y * T1.z - vh.z * T1.y, vh.z * T1.x - vh.x * T1.z, vh.x * T1.y - vh.y * T1.x};
  double r = std::sqrt(u1), phi = 2 * M_PI * u2;
  double t1 = r * std::cos(phi), t2 = r * std::sin(phi);
  double s = 0.5 * (1 + vh.z);
  t2 = (1 - s) * std::sqrt(std::max(0.0, 1 - t1 * t1)) + s * t2;
  double t3 = std::sqrt(std::max(0.0, 1 - t1 * t1 - t2 * t2));
  D3 nh = {t1 * T1.x + t2 * T2.x + t3 * vh.x, t1 * T1.y + t2 * T2.y + t3 * vh.y, t1 * T1.z + t2 * T2.z + t3 * vh.z};
  return unit({a * nh.x, a * nh.y, std::max(1e-7, nh.z)});
}
double van_der_corput(uint32_t i) { double b = 0, f = 0.5; while (i) { if (i & 1) b += f; i >>= 1; f *= 0.5; } return b; }

// the coated conductor's f(l, v) and sampling pdf at n = +z (gpu/bsdf.js:98-117, :160-173)
void coated_eval(const Material& M, D3 l, D3 v, double f[3], double& pdf) {
  f[0] = f[1] = f[2] = 0; pdf = 0;
  double nl = l.z, nv = v.z;
  if (nl <= 0 || nv <= 0) return;
  D3 h = unit({l.x + v.x, l.y + v.y, l.z + v.z});
  double nh = h.z, vh = std::max(0.0, dot3(v, h));
  double coat = d_ggx(nh, M.alpha_coat) * g2(nl, nv, M.alpha_coat) * fresnel(vh, M.ior) / (4 * nl * nv);
  double t = (1 - fresnel(nl, M.ior)) * (1 - fresnel(nv, M.ior));
  double metal = d_ggx(nh, M.alpha) * g2(nl, nv, M.alpha) / (4 * nl * nv);
  for (int c = 0; c < 3; c++) f[c] = coat + t * std::pow(M.tau[c], 1 / nl + 1 / nv) * metal * schlick1(M.f0[c], vh);
  double Fc = fresnel(nv, M.ior), mf = (M.f0[0] + M.f0[1] + M.f0[2]) / 3;
  double ps = Fc / (Fc + (1 - Fc) * mf);
  double vh2 = dot3(v, h);
  if (!(vh2 > 0)) return;
  pdf = ps * g1(nv, M.alpha_coat) * d_ggx(nh, M.alpha_coat) / (4 * nv) + (1 - ps) * g1(nv, M.alpha) * d_ggx(nh, M.alpha) / (4 * nv);
}

void fill_albedo_table(Material& M, uint32_t samples) {
  const int bins = VT_ALBEDO_BINS;
  for (int k = 0; k < bins; k++) {
    const double mu = (k + 0.5) / bins;
    const D3 v = {std::sqrt(1 - mu * mu), 0, mu};
    double acc[3] = {0, 0, 0};
    if (M.kind == 2) {
      // both lobes specular: the material's own sampler with a stratified lobe choice (gpu/bsdf.js:216-225)
      const double Fc = fresnel(mu, M.ior), mf = (M.f0[0] + M.f0[1] + M.f0[2]) / 3;
      const double ps = Fc / (Fc + (1 - Fc) * mf);
      for (uint32_t i = 0; i < samples; i++) {
        double u0 = (i + 0.5) / samples, u1 = van_der_corput(i), u2 = std::fmod(van_der_corput(i ^ 0x5555u), 1.0);
        // basis around n = +z: t = (1, 0, 0), b = (0, 1, 0) (Duff et al. with n.z = 1)
        D3 hl = vndf(v, u0 < ps ? M.alpha_coat : M.alpha, u1, u2);
        double vh = dot3(v, hl);
        D3 l = {2 * vh * hl.x - v.x, 2 * vh * hl.y - v.y, 2 * vh * hl.z - v.z};
        if (l.z <= 0) continue;
        double f[3], pdf;
        coated_eval(M, l, v, f, pdf);
        if (!(pdf > 0)) continue;
        for (int c = 0; c < 3; c++) acc[c] += f[c] * l.z / pdf;
      }
      for (int c = 0; c < 3; c++) { M.spec[k][c] = acc[c] / samples; M.diff[k][c] = 0; }
      continue;
    }
    for (uint32_t i = 0; i < samples; i++) {
      const double u1 = (i + 0.5) / samples, u2 = van_der_corput(i);
      const D3 h = vndf(v, M.alpha, u1, u2);
      const double vh = dot3(v, h);
      const D3 l = {2 * vh * h.x - v.x, 2 * vh * h.y - v.y, 2 * vh * h.z - v.z};
      if (l.z <= 0) continue;
      const double w = g2(l.z, mu, M.alpha) / g1(mu, M.alpha);
      if (M.kind == 1) for (int c = 0; c < 3; c++) acc[c] += schlick1(M.f0[c], vh) * w;
      else { const double F = fresnel(vh, M.ior); for (int c = 0; c < 3; c++) acc[c] += F * w; }
    }
    for (int c = 0; c < 3; c++) {
      M.spec[k][c] = acc[c] / samples;
      M.diff[k][c] = M.kind == 1 ? 0 : M.rho[c] * (1 - fresnel(mu, M.ior)) * (1 - M.fbar_exact) / (1 - M.fbar);
    }
  }
  for (int c = 0; c < 3; c++) { M.hh[c] = 0; M.hh_spec[c] = 0; }
  for (int k = 0; k < bins; k++) {
    const double mu = (k + 0.5) / bins;
    for (int c = 0; c < 3; c++) {
      M.hh[c] += 2 * mu * (M.spec[k][c] + M.diff[k][c]) / bins;
      M.hh_spec[c] += 2 * mu * M.spec[k][c] / bins;
    }
  }
}
}  // namespace

double fresnel_mean(double eta) {
  const int n = 4096;
  double s = 0;
  for (int i = 0; i <= n; i++) {
    const double mu = double(i) / n;
    const double w = (i == 0 || i == n) ? 1 : (i % 2 ? 4 : 2);
    s += w * fresnel(mu, eta) * mu;
  }
  return 2 * s / (3 * n);
}

Material make_material(const vt_material& m, uint32_t albedo_samples) {
  Material M;
  if (m.coated) {
    const double r = std::max(double(m.roughness), 0.02), rc = std::max(double(m.coat_roughness), 0.02);
    M.kind = 2; M.roughness = r; M.alpha = r * r; M.ior = m.coat_ior; M.alpha_coat = rc * rc;
    for (int c = 0; c < 3; c++) { M.f0[c] = m.f0[c]; M.tau[c] = m.tau[c]; }
  } else {
    M.kind = m.metallic ? 1 : 0;
    const double r = std::max(double(m.roughness), 0.02);
    M.roughness = r; M.alpha = r * r; M.ior = m.ior;
    for (int c = 0; c < 3; c++) { M.rho[c] = M.kind ? 0 : m.rho[c]; M.f0[c] = M.kind ? m.f0[c] : 0; }
    M.fbar_exact = M.kind ? 0 : fresnel_mean(M.ior);
    M.fbar = M.kind ? 0 : (std::isfinite(m.fbar) ? double(m.fbar) : M.fbar_exact);
  }
  M.emitter = m.emitter != 0;
  M.textured = m.textured != 0;
  for (int c = 0; c < 3; c++) M.ink[c] = m.ink_rho[c];
  M.rough_ink = m.ink_roughness;
  M.table = !m.no_table;
  if (M.table) fill_albedo_table(M, albedo_samples);
  return M;
}

// ---------------------------------------------------------------------------------------------- the scene
namespace {
void capsule_fit(const float* P, size_t n, double a[3], double b[3], double& r) {
  // principal axis by power iteration from (0.3, 0.5, 0.8), radius = largest distance from it (scene_gpu.js:504)
  if (!n) { for (int k = 0; k < 3; k++) a[k] = b[k] = 0; r = 0; return; }
  double c[3] = {0, 0, 0};
  for (size_t v = 0; v < n; v++) for (int k = 0; k < 3; k++) c[k] += double(P[3 * v + k]) / double(n);
  double cov[3][3] = {};
  for (size_t v = 0; v < n; v++) {
    const double d[3] = {P[3 * v] - c[0], P[3 * v + 1] - c[1], P[3 * v + 2] - c[2]};
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) cov[i][j] += d[i] * d[j];
  }
  double ax[3] = {0.3, 0.5, 0.8};
  for (int it = 0; it < 64; it++) {
    double y[3];
    for (int i = 0; i < 3; i++) y[i] = cov[i][0] * ax[0] + cov[i][1] * ax[1] + cov[i][2] * ax[2];
    const double l = std::sqrt(y[0] * y[0] + y[1] * y[1] + y[2] * y[2]);
    if (!(l > 0)) break;
    for (int i = 0; i < 3; i++) ax[i] = y[i] / l;
  }
  double smin = INFINITY, smax = -INFINITY;
  r = 0;
  for (size_t v = 0; v < n; v++) {
    const double d[3] = {P[3 * v] - c[0], P[3 * v + 1] - c[1], P[3 * v + 2] - c[2]};
    const double s = d[0] * ax[0] + d[1] * ax[1] + d[2] * ax[2];
    smin = std::min(smin, s); smax = std::max(smax, s);
    const double e[3] = {d[0] - s * ax[0], d[1] - s * ax[1], d[2] - s * ax[2]};
    r = std::max(r, std::sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]));
  }
  for (int k = 0; k < 3; k++) { a[k] = c[k] + smin * ax[k]; b[k] = c[k] + smax * ax[k]; }
}

using Emit = EmitTri;

// one 64-byte triangle record (v0|i0, e1|i1, e2|i2, mesh, flags, -, -)
void tri_record(uint32_t* rec, const float* P, const uint32_t* tri, uint32_t i0, uint32_t i1, uint32_t i2, uint32_t mesh, uint32_t flags) {
  const float* a = P + 3 * size_t(tri[0]);
  const float* b = P + 3 * size_t(tri[1]);
  const float* c = P + 3 * size_t(tri[2]);
  const float v[12] = {a[0], a[1], a[2], 0, b[0] - a[0], b[1] - a[1], b[2] - a[2], 0, c[0] - a[0], c[1] - a[1], c[2] - a[2], 0};
  for (int k = 0; k < 12; k++) rec[k] = fbits(v[k]);
  rec[3] = i0; rec[7] = i1; rec[11] = i2; rec[12] = mesh; rec[13] = flags; rec[14] = 0; rec[15] = 0;
}
}  // namespace

Prepared prepare_scene(const vt_scene_desc& d, uint32_t leaf, uint32_t albedo_samples, const StaticBuilder& build_static) {
  if (!d.meshes || !d.n_meshes || !d.materials || !d.n_materials) throw std::runtime_error("scene: no meshes or materials");
  if (d.n_static_tris && (!d.static_P || !d.static_N || !d.static_I || !d.static_tri_mesh || !d.static_vert_mesh))
    throw std::runtime_error("scene: static arrays missing");
  if (d.n_bodies > VT_MAX_INST) throw std::runtime_error("too many bodies");
  Prepared S;
  S.meshes.assign(d.meshes, d.meshes + d.n_meshes);
  for (uint32_t i = 0; i < d.n_meshes; i++)
    if (d.meshes[i].mat >= d.n_materials) throw std::runtime_error("scene: mesh material out of range");
  for (uint32_t i = 0; i < d.n_static_tris; i++) {
    if (d.static_tri_mesh[i] >= d.n_meshes) throw std::runtime_error("scene: static triangle mesh out of range");
    for (int k = 0; k < 3; k++) if (d.static_I[3 * i + k] >= d.n_static_verts) throw std::runtime_error("scene: static index out of range");
  }
  for (uint32_t b = 0; b < d.n_bodies; b++) {
    const vt_body_desc& B = d.bodies[b];
    if (B.n_tris && (!B.P || !B.N || !B.I || !B.tri_mesh)) throw std::runtime_error("scene: body arrays missing");
    for (uint32_t i = 0; i < B.n_tris; i++) {
      if (B.tri_mesh[i] >= d.n_meshes) throw std::runtime_error("scene: body triangle mesh out of range");
      for (int k = 0; k < 3; k++) if (B.I[3 * i + k] >= B.n_verts) throw std::runtime_error("scene: body index out of range");
    }
  }
  for (uint32_t i = 0; i < d.n_materials; i++) S.mats.push_back(make_material(d.materials[i], albedo_samples));
  S.static_verts = d.n_static_verts;
  S.static_tris = d.n_static_tris;
  S.cams.assign(d.cameras, d.cameras + d.n_cameras);
  for (int k = 0; k < 3; k++) S.L0[k] = d.L0[k];

  Bvh sb = build_static ? build_static(d.static_P, d.n_static_verts, d.static_I, d.n_static_tris, leaf)
                       : sah_build(d.static_P, d.static_I, d.n_static_tris, leaf);
  std::vector<Bvh> bb(d.n_bodies);
  std::vector<Emit> emit;
  std::vector<std::vector<uint32_t>> emit_idx(d.n_bodies);
  for (uint32_t b = 0; b < d.n_bodies; b++) {
    const vt_body_desc& B = d.bodies[b];
    bb[b] = sah_build(B.P, B.I, B.n_tris, leaf);
    emit_idx[b].assign(B.n_tris, 0xffffffffu);
    for (uint32_t t = 0; t < B.n_tris; t++) {
      if (!(d.meshes[B.tri_mesh[t]].flags & VT_F_EMITTER)) continue;
      emit_idx[b][t] = uint32_t(emit.size());
      const float* p0 = B.P + 3 * size_t(B.I[3 * t]);
      const float* p1 = B.P + 3 * size_t(B.I[3 * t + 1]);
      const float* p2 = B.P + 3 * size_t(B.I[3 * t + 2]);
      const float* n0 = B.N + 3 * size_t(B.I[3 * t]);
      const float* n1 = B.N + 3 * size_t(B.I[3 * t + 1]);
      const float* n2 = B.N + 3 * size_t(B.I[3 * t + 2]);
      Emit e;
      for (int k = 0; k < 3; k++) { e.v0[k] = p0[k]; e.e1[k] = double(p1[k]) - e.v0[k]; e.e2[k] = double(p2[k]) - e.v0[k]; }
      double n[3] = {e.e1[1] * e.e2[2] - e.e1[2] * e.e2[1], e.e1[2] * e.e2[0] - e.e1[0] * e.e2[2], e.e1[0] * e.e2[1] - e.e1[1] * e.e2[0]};
      e.area = 0.5 * std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
      double vn[3];
      for (int k = 0; k < 3; k++) vn[k] = double(n0[k]) + double(n1[k]) + double(n2[k]);
      if (n[0] * vn[0] + n[1] * vn[1] + n[2] * vn[2] < 0) for (double& q : n) q = -q;
      double l = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
      if (!(l > 0)) l = 1;
      for (int k = 0; k < 3; k++) e.n[k] = n[k] / l;
      e.cdf = 0;
      emit.push_back(e);
    }
  }
  // combined node and triangle buffers: the static BVH first, then each body's BLAS relocated (gpu/bvh.js:164)
  uint32_t nodes = sb.node_count, tris = d.n_static_tris;
  S.bodies.resize(d.n_bodies);
  for (uint32_t b = 0; b < d.n_bodies; b++) {
    BodyRec& r = S.bodies[b];
    r.root = nodes; r.tri_off = tris; r.tri_count = d.bodies[b].n_tris; r.kind = d.bodies[b].kind; r.owner = d.bodies[b].owner_camera;
    for (int k = 0; k < 3; k++) { r.lo[k] = bb[b].lo[k]; r.hi[k] = bb[b].hi[k]; }
    nodes += bb[b].node_count; tris += d.bodies[b].n_tris;
  }
  S.node_count = nodes; S.tri_count = tris;
  S.nodes.assign(size_t(nodes) * VT_NODE_WORDS, 0u);
  std::copy(sb.words.begin(), sb.words.end(), S.nodes.begin());
  for (uint32_t b = 0; b < d.n_bodies; b++) {
    uint32_t* dst = S.nodes.data() + size_t(S.bodies[b].root) * VT_NODE_WORDS;
    std::copy(bb[b].words.begin(), bb[b].words.end(), dst);
    for (size_t o = 0; o < bb[b].words.size(); o += 8) dst[o + 3] += dst[o + 7] == 0 ? S.bodies[b].root : S.bodies[b].tri_off;
  }
  S.tris.assign(size_t(tris) * 16, 0u);
  S.emit_of_tri.assign(tris, 0xffffffffu);
  for (uint32_t k = 0; k < d.n_static_tris; k++) {
    const uint32_t t = sb.order[k];
    const uint32_t* tri = d.static_I + 3 * size_t(t);
    const uint32_t mesh = d.static_tri_mesh[t];
    tri_record(S.tris.data() + size_t(k) * 16, d.static_P, tri, tri[0], tri[1], tri[2], mesh, d.meshes[mesh].flags);
  }
  std::vector<uint32_t> vbase(d.n_bodies);
  uint32_t vb = d.n_static_verts;
  for (uint32_t b = 0; b < d.n_bodies; b++) {
    const vt_body_desc& B = d.bodies[b];
    vbase[b] = vb;
    for (uint32_t k = 0; k < B.n_tris; k++) {
      const uint32_t t = bb[b].order[k];
      const uint32_t* tri = B.I + 3 * size_t(t);
      const uint32_t mesh = B.tri_mesh[t];
      tri_record(S.tris.data() + size_t(S.bodies[b].tri_off + k) * 16, B.P, tri, tri[0] + vb, tri[1] + vb, tri[2] + vb, mesh, d.meshes[mesh].flags);
      S.emit_of_tri[S.bodies[b].tri_off + k] = emit_idx[b][t];
    }
    vb += B.n_verts;
  }
  // vertices (32 B): static pos|mesh, normal|node area; body pos|u, normal|v
  S.vert_count = vb;
  S.verts.assign(size_t(vb) * 8, 0u);
  std::vector<double> area(d.n_static_verts, 0.0);
  const float* sP = d.static_P;
  for (uint32_t k = 0; k < d.n_static_tris; k++) {
    const uint32_t a = d.static_I[3 * k], b = d.static_I[3 * k + 1], c = d.static_I[3 * k + 2];
    const double u[3] = {double(sP[3 * b]) - sP[3 * a], double(sP[3 * b + 1]) - sP[3 * a + 1], double(sP[3 * b + 2]) - sP[3 * a + 2]};
    const double v[3] = {double(sP[3 * c]) - sP[3 * a], double(sP[3 * c + 1]) - sP[3 * a + 1], double(sP[3 * c + 2]) - sP[3 * a + 2]};
    const double x = u[1] * v[2] - u[2] * v[1], y = u[2] * v[0] - u[0] * v[2], z = u[0] * v[1] - u[1] * v[0];
    const double third = 0.5 * std::sqrt(x * x + y * y + z * z) / 3;
    area[a] += third; area[b] += third; area[c] += third;
  }
  S.node_area.resize(d.n_static_verts);
  for (uint32_t v = 0; v < d.n_static_verts; v++) {
    uint32_t* o = S.verts.data() + size_t(v) * 8;
    o[0] = fbits(sP[3 * v]); o[1] = fbits(sP[3 * v + 1]); o[2] = fbits(sP[3 * v + 2]); o[3] = d.static_vert_mesh[v];
    o[4] = fbits(d.static_N[3 * v]); o[5] = fbits(d.static_N[3 * v + 1]); o[6] = fbits(d.static_N[3 * v + 2]);
    o[7] = fbits(float(area[v]));
    S.node_area[v] = float(area[v]);
  }
  for (uint32_t b = 0; b < d.n_bodies; b++) {
    const vt_body_desc& B = d.bodies[b];
    for (uint32_t v = 0; v < B.n_verts; v++) {
      uint32_t* o = S.verts.data() + size_t(vbase[b] + v) * 8;
      o[0] = fbits(B.P[3 * v]); o[1] = fbits(B.P[3 * v + 1]); o[2] = fbits(B.P[3 * v + 2]); o[3] = fbits(B.UV ? B.UV[2 * v] : 0.0f);
      o[4] = fbits(B.N[3 * v]); o[5] = fbits(B.N[3 * v + 1]); o[6] = fbits(B.N[3 * v + 2]); o[7] = fbits(B.UV ? B.UV[2 * v + 1] : 0.0f);
    }
  }
  // emitter: area CDF over its triangles, mean normal, emission axis, scope-ahead test, centroid and radius
  double total = 0;
  for (const Emit& e : emit) total += e.area;
  const double norm = total != 0 ? total : 1;
  double run = 0;
  for (Emit& e : emit) { run += e.area; e.cdf = run / norm; }
  double mn[3] = {0, 0, 0};
  for (const Emit& e : emit) for (int k = 0; k < 3; k++) mn[k] += e.n[k] * e.area;
  double ml = std::sqrt(mn[0] * mn[0] + mn[1] * mn[1] + mn[2] * mn[2]);
  if (!(ml > 0)) ml = 1;
  for (int k = 0; k < 3; k++) { S.emit_normal[k] = mn[k] / ml; S.emit_axis[k] = S.emit_normal[k]; }
  if (std::isfinite(d.axis_deg)) {
    const double a = double(d.axis_deg) * M_PI / 180;
    S.emit_axis[0] = 0; S.emit_axis[1] = std::sin(a); S.emit_axis[2] = std::cos(a);
  }
  for (uint32_t b = 0; b < d.n_bodies; b++) if (d.bodies[b].kind == VT_BODY_SCOPE) { S.scope_index = int(b); break; }
  double ahead = -INFINITY;
  if (!emit.empty()) {
    double c[3] = {0, 0, 0};
    for (const Emit& e : emit) for (int k = 0; k < 3; k++) c[k] += e.v0[k] * e.area;
    for (int k = 0; k < 3; k++) c[k] /= norm;
    for (uint32_t b = 0; b < d.n_bodies; b++) {
      if (d.bodies[b].kind != VT_BODY_SCOPE) continue;
      const vt_body_desc& B = d.bodies[b];
      for (uint32_t v = 0; v < B.n_verts; v++) {
        const double q = (B.P[3 * v] - c[0]) * S.emit_normal[0] + (B.P[3 * v + 1] - c[1]) * S.emit_normal[1] + (B.P[3 * v + 2] - c[2]) * S.emit_normal[2];
        ahead = std::max(ahead, q);
      }
    }
  }
  S.shadow_skips_scope = ahead <= 1e-6;
  for (const Emit& e : emit) for (int k = 0; k < 3; k++) S.emit_centroid[k] += (e.v0[k] + (e.e1[k] + e.e2[k]) / 3) * e.area / norm;
  for (const Emit& e : emit) {
    for (int j = 0; j < 3; j++) {
      double dx = 0, q2 = 0;
      for (int k = 0; k < 3; k++) {
        const double p = e.v0[k] + (j == 1 ? e.e1[k] : j == 2 ? e.e2[k] : 0.0);
        dx = p - S.emit_centroid[k];
        q2 += dx * dx;
      }
      S.emit_radius = std::max(S.emit_radius, std::sqrt(q2));
    }
  }
  S.emit_area = total;
  S.emit_tris = uint32_t(emit.size());
  S.emitters = emit;
  // body capsules and effective albedo (scene_gpu.js:427-456): the bounding capsule of every vertex; the occlusion
  // capsule and the effective albedo from the triangles of meshes in the cavity (not overview-only)
  for (uint32_t b = 0; b < d.n_bodies; b++) {
    const vt_body_desc& B = d.bodies[b];
    BodyRec& r = S.bodies[b];
    capsule_fit(B.P, B.n_verts, r.cap_a, r.cap_b, r.cap_r);
    std::vector<uint8_t> keep(B.n_verts, 0);
    bool any_drop = false;
    for (uint32_t t = 0; t < B.n_tris; t++) {
      if (d.meshes[B.tri_mesh[t]].overview_only) { any_drop = true; continue; }
      for (int k = 0; k < 3; k++) keep[B.I[3 * t + k]] = 1;
    }
    if (any_drop) {
      std::vector<float> pc;
      for (uint32_t v = 0; v < B.n_verts; v++)
        if (keep[v]) for (int k = 0; k < 3; k++) pc.push_back(B.P[3 * size_t(v) + k]);
      if (pc.empty()) { for (int k = 0; k < 3; k++) { r.occ_a[k] = 0; r.occ_b[k] = 0; } r.occ_r = 0; }
      else capsule_fit(pc.data(), uint32_t(pc.size() / 3), r.occ_a, r.occ_b, r.occ_r);
    } else {
      for (int k = 0; k < 3; k++) { r.occ_a[k] = r.cap_a[k]; r.occ_b[k] = r.cap_b[k]; }
      r.occ_r = r.cap_r;
    }
    double ar = 0, rho = 0;
    for (uint32_t t = 0; t < B.n_tris; t++) {
      if (any_drop && d.meshes[B.tri_mesh[t]].overview_only) continue;
      const float* p0 = B.P + 3 * size_t(B.I[3 * t]);
      const float* p1 = B.P + 3 * size_t(B.I[3 * t + 1]);
      const float* p2 = B.P + 3 * size_t(B.I[3 * t + 2]);
      const double u[3] = {double(p1[0]) - p0[0], double(p1[1]) - p0[1], double(p1[2]) - p0[2]};
      const double v[3] = {double(p2[0]) - p0[0], double(p2[1]) - p0[1], double(p2[2]) - p0[2]};
      const double x = u[1] * v[2] - u[2] * v[1], y = u[2] * v[0] - u[0] * v[2], z = u[0] * v[1] - u[1] * v[0];
      const double A = 0.5 * std::sqrt(x * x + y * y + z * z);
      const Material& m = S.mats[d.meshes[B.tri_mesh[t]].mat];
      const double h0 = m.table ? m.hh[0] : 0, h1 = m.table ? m.hh[1] : 0, h2 = m.table ? m.hh[2] : 0;
      ar += A;
      rho += A * (0.2126 * h0 + 0.7152 * h1 + 0.0722 * h2);
    }
    r.rho_eff = ar != 0 ? rho / ar : 0;
  }
  // params: mesh table | materials (5 vec4) | albedo tables (2 vec4 per bin) | profile knots | emitter triangles
  const uint32_t nMesh = d.n_meshes, nMat = d.n_materials;
  S.emit_n = std::max<uint32_t>(1, uint32_t(emit.size()));
  S.prof_n = std::max<uint32_t>(2, d.n_profile);
  S.mesh_off = 0;
  S.mat_off = 2 * nMesh;
  S.alb_off = S.mat_off + 5 * nMat;
  S.prof_off = S.alb_off + nMat * VT_ALBEDO_BINS * 2;
  S.emit_off = S.prof_off + S.prof_n;
  S.params.assign(size_t(S.emit_off + 4 * S.emit_n) * 4, 0.0f);
  float* P = S.params.data();
  auto u2f = [](uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; };
  for (uint32_t i = 0; i < nMesh; i++) {
    float* o = P + size_t(S.mesh_off + 2 * i) * 4;
    const vt_mesh& m = d.meshes[i];
    o[0] = m.build_dir[0]; o[1] = m.build_dir[1]; o[2] = m.build_dir[2]; o[3] = u2f(m.mat);
    o[4] = u2f(m.flags); o[5] = m.layer_period; o[6] = m.layer_depth; o[7] = 0;
  }
  for (uint32_t i = 0; i < nMat; i++) {
    float* o = P + size_t(S.mat_off + 5 * i) * 4;
    const Material& m = S.mats[i];
    const double* c = m.kind ? m.f0 : m.rho;
    o[0] = float(c[0]); o[1] = float(c[1]); o[2] = float(c[2]); o[3] = float(m.alpha);
    o[4] = float(m.ior); o[5] = float(m.kind); o[6] = float(m.fbar); o[7] = float(m.roughness);
    for (int k = 0; k < 3; k++) { o[8 + k] = m.table ? float(m.hh[k]) : 0.0f; o[12 + k] = m.table ? float(m.hh_spec[k]) : 0.0f; }
    o[15] = m.emitter ? 1.0f : 0.0f;
    if (m.kind == 2) { o[16] = float(m.tau[0]); o[17] = float(m.tau[1]); o[18] = float(m.tau[2]); o[19] = float(m.alpha_coat); }
    else if (m.textured) { o[16] = float(m.ink[0]); o[17] = float(m.ink[1]); o[18] = float(m.ink[2]); o[19] = float(m.rough_ink * m.rough_ink); }
    if (m.table) for (int b = 0; b < VT_ALBEDO_BINS; b++) {
      float* q = P + size_t(S.alb_off + (i * VT_ALBEDO_BINS + b) * 2) * 4;
      for (int k = 0; k < 3; k++) { q[k] = float(m.spec[b][k]); q[4 + k] = float(m.diff[b][k]); }
    }
  }
  for (uint32_t k = 0; k < S.prof_n; k++) {
    float* o = P + size_t(S.prof_off + k) * 4;
    if (d.n_profile) { const uint32_t j = std::min(k, d.n_profile - 1); o[0] = d.profile_theta[j]; o[1] = d.profile_p[j]; }
    else { o[0] = k ? float(M_PI / 2) : 0.0f; o[1] = 1.0f; }
  }
  for (size_t k = 0; k < emit.size(); k++) {
    float* o = P + size_t(S.emit_off + 4 * k) * 4;
    const Emit& e = emit[k];
    const float v[16] = {float(e.v0[0]), float(e.v0[1]), float(e.v0[2]), float(e.cdf), float(e.e1[0]), float(e.e1[1]), float(e.e1[2]), 0,
                         float(e.e2[0]), float(e.e2[1]), float(e.e2[2]), 0, float(e.n[0]), float(e.n[1]), float(e.n[2]), float(e.area)};
    std::memcpy(o, v, sizeof(v));
  }
  return S;
}

// ---------------------------------------------------------------------------------------------- poses
namespace {
void quat_of(const double* m, double q[4]) {  // column-major rotation -> unit quaternion (x, y, z, w)
  const double r00 = m[0], r10 = m[1], r20 = m[2], r01 = m[4], r11 = m[5], r21 = m[6], r02 = m[8], r12 = m[9], r22 = m[10];
  const double tr = r00 + r11 + r22;
  double x, y, z, w;
  if (tr > 0) { const double s = std::sqrt(tr + 1) * 2; w = 0.25 * s; x = (r21 - r12) / s; y = (r02 - r20) / s; z = (r10 - r01) / s; }
  else if (r00 > r11 && r00 > r22) { const double s = std::sqrt(1 + r00 - r11 - r22) * 2; w = (r21 - r12) / s; x = 0.25 * s; y = (r01 + r10) / s; z = (r02 + r20) / s; }
  else if (r11 > r22) { const double s = std::sqrt(1 + r11 - r00 - r22) * 2; w = (r02 - r20) / s; x = (r01 + r10) / s; y = 0.25 * s; z = (r12 + r21) / s; }
  else { const double s = std::sqrt(1 + r22 - r00 - r11) * 2; w = (r10 - r01) / s; x = (r02 + r20) / s; y = (r12 + r21) / s; z = 0.25 * s; }
  const double l = std::sqrt(x * x + y * y + z * z + w * w);
  q[0] = x / l; q[1] = y / l; q[2] = z / l; q[3] = w / l;
}
void mat_of(const double q[4], double R[3][3]) {
  const double x = q[0], y = q[1], z = q[2], w = q[3];
  R[0][0] = 1 - 2 * (y * y + z * z); R[0][1] = 2 * (x * y - z * w); R[0][2] = 2 * (x * z + y * w);
  R[1][0] = 2 * (x * y + z * w); R[1][1] = 1 - 2 * (x * x + z * z); R[1][2] = 2 * (y * z - x * w);
  R[2][0] = 2 * (x * z - y * w); R[2][1] = 2 * (y * z + x * w); R[2][2] = 1 - 2 * (x * x + y * y);
}
void rot(const double R[3][3], const double* v, const double* p, double* o) {
  for (int i = 0; i < 3; i++) o[i] = R[i][0] * v[0] + R[i][1] * v[1] + R[i][2] * v[2] + (p ? p[i] : 0.0);
}
}  // namespace

bool pose_at(const InstPose& I, double t, double R[3][3], double p[3]) {
  if (!I.valid) return false;
  // slerp with the short-arc flip and a normalised lerp above cos 0.9995 (gpu/renderer.js:85)
  double b[4] = {I.q1[0], I.q1[1], I.q1[2], I.q1[3]};
  double c = I.q0[0] * b[0] + I.q0[1] * b[1] + I.q0[2] * b[2] + I.q0[3] * b[3];
  if (c < 0) { for (double& x : b) x = -x; c = -c; }
  double q[4];
  if (c > 0.9995) {
    double l = 0;
    for (int i = 0; i < 4; i++) { q[i] = I.q0[i] + (b[i] - I.q0[i]) * t; l += q[i] * q[i]; }
    l = std::sqrt(l);
    for (double& x : q) x /= l;
  } else {
    const double th = std::acos(c), s = std::sin(th);
    for (int i = 0; i < 4; i++) q[i] = (I.q0[i] * std::sin((1 - t) * th) + b[i] * std::sin(t * th)) / s;
  }
  mat_of(q, R);
  for (int k = 0; k < 3; k++) p[k] = I.p0[k] + (I.p1[k] - I.p0[k]) * t;
  return true;
}

std::vector<InstPose> poses_from(const Prepared& S, const double* T0, const double* T1, uint32_t n) {
  std::vector<InstPose> out(S.bodies.size());
  for (size_t i = 0; i < S.bodies.size(); i++) {
    InstPose& I = out[i];
    if (S.bodies[i].kind == VT_BODY_FIXED) {
      I.valid = true;
      for (int k = 0; k < 4; k++) I.q0[k] = I.q1[k] = k == 3 ? 1 : 0;
      for (int k = 0; k < 3; k++) I.p0[k] = I.p1[k] = 0;
      continue;
    }
    if (i >= n || !T0 || std::isnan(T0[16 * i])) continue;
    const double* A = T0 + 16 * i;
    const double* B = (T1 && !std::isnan(T1[16 * i])) ? T1 + 16 * i : A;
    quat_of(A, I.q0);
    quat_of(B, I.q1);
    for (int k = 0; k < 3; k++) { I.p0[k] = A[12 + k]; I.p1[k] = B[12 + k]; }
    I.valid = true;
  }
  return out;
}

void scene_uniform(const Prepared& S, const std::vector<InstPose>& inst, const float eavg[3], uint32_t slot, uint32_t frame, float* f,
                   const float* pcaps) {
  uint32_t* u = reinterpret_cast<uint32_t*>(f);
  std::fill(f, f + SU_WORDS, 0.0f);
  f[0] = S.L0[0]; f[1] = S.L0[1]; f[2] = S.L0[2]; f[3] = S.emit_area != 0 ? float(S.emit_area) : 1e-12f;
  f[4] = float(S.emit_axis[0]); f[5] = float(S.emit_axis[1]); f[6] = float(S.emit_axis[2]);
  u[7] = (S.shadow_skips_scope && S.scope_index >= 0) ? (1u << S.scope_index) : 0u;
  f[8] = eavg[0]; f[9] = eavg[1]; f[10] = eavg[2]; f[11] = 5e-4f;
  f[15] = 1e30f;
  u[16] = uint32_t(S.bodies.size()); u[17] = S.scope_index < 0 ? 0u : uint32_t(S.scope_index); u[18] = slot ? slot : 1; u[19] = frame;
  f[20] = float(S.emit_centroid[0]); f[21] = float(S.emit_centroid[1]); f[22] = float(S.emit_centroid[2]); f[23] = float(S.emit_radius);
  for (size_t i = 0; i < S.bodies.size(); i++) {
    float* o = f + SU_INST + 48 * i;
    uint32_t* ou = u + SU_INST + 48 * i;
    const BodyRec& bl = S.bodies[i];
    const InstPose& I = inst[i];
    if (!I.valid) { ou[15] = 2; ou[11] = bl.root; continue; }
    for (int k = 0; k < 4; k++) { o[k] = float(I.q0[k]); o[4 + k] = float(I.q1[k]); }
    for (int k = 0; k < 3; k++) { o[8 + k] = float(I.p0[k]); o[12 + k] = float(I.p1[k]); }
    ou[11] = bl.root;
    bool moving = false;
    for (int k = 0; k < 4; k++) moving |= I.q0[k] != I.q1[k];
    for (int k = 0; k < 3; k++) moving |= I.p0[k] != I.p1[k];
    ou[15] = moving ? 1u : 0u;
    // world box swept over the exposure (5 time samples when moving)
    double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    const double times[5] = {0, 0.25, 0.5, 0.75, 1};
    for (int ti = 0; ti < (moving ? 5 : 1); ti++) {
      double R[3][3], p[3];
      pose_at(I, times[ti], R, p);
      for (int c = 0; c < 8; c++) {
        const double v[3] = {(c & 1) ? bl.hi[0] : bl.lo[0], (c & 2) ? bl.hi[1] : bl.lo[1], (c & 4) ? bl.hi[2] : bl.lo[2]};
        double w[3];
        rot(R, v, p, w);
        for (int k = 0; k < 3; k++) { lo[k] = std::min(lo[k], w[k]); hi[k] = std::max(hi[k], w[k]); }
      }
    }
    const double pad = moving ? 1e-3 : 1e-6;
    for (int k = 0; k < 3; k++) { o[16 + k] = float(lo[k] - pad); o[20 + k] = float(hi[k] + pad); }
    double R[3][3], p[3];
    pose_at(I, 0.5, R, p);
    double oa[3], ob[3];
    rot(R, bl.occ_a, p, oa);
    rot(R, bl.occ_b, p, ob);
    const double cr = (bl.kind == VT_BODY_FIXED || bl.kind == VT_BODY_BOARD) ? 0.0 : bl.occ_r;
    for (int k = 0; k < 3; k++) { o[24 + k] = float(oa[k]); o[28 + k] = float(ob[k]); }
    o[27] = float(cr); o[31] = float(bl.rho_eff);
    double ca[3], cb[3];
    rot(R, bl.cap_a, p, ca);
    rot(R, bl.cap_b, p, cb);
    double motion = 0;
    if (moving) {
      double R0[3][3], p0[3], R1[3][3], p1[3];
      pose_at(I, 0, R0, p0);
      pose_at(I, 1, R1, p1);
      for (const double* v : {bl.cap_a, bl.cap_b}) {
        double m[3], w0[3], w1[3];
        rot(R, v, p, m);
        rot(R0, v, p0, w0);
        rot(R1, v, p1, w1);
        for (const double* w : {w0, w1}) {
          const double dx = w[0] - m[0], dy = w[1] - m[1], dz = w[2] - m[2];
          motion = std::max(motion, std::sqrt(dx * dx + dy * dy + dz * dz));
        }
      }
      motion *= 1.5;
    }
    const float bc[8] = {float(ca[0]), float(ca[1]), float(ca[2]), float(bl.cap_r * 1.0001 + 1e-6 + motion), float(cb[0]), float(cb[1]), float(cb[2]), 0};
    const bool have_pc = pcaps && !std::isnan(pcaps[8 * i]);
    for (int k = 0; k < 8; k++) { o[32 + k] = bc[k]; o[40 + k] = have_pc ? pcaps[8 * i + k] : bc[k]; }
  }
}

void relative_illumination(const vt_camera_desc& c, double q, const double* vdeg, const double* vv, uint32_t nv, float* out) {
  const double k[4] = {c.k[0], c.k[1], c.k[2], c.k[3]};
  auto distort = [&](double th) { const double t2 = th * th; return th * (1 + t2 * (k[0] + t2 * (k[1] + t2 * (k[2] + t2 * k[3])))); };
  auto deriv = [&](double th) { const double t2 = th * th; return 1 + t2 * (3 * k[0] + t2 * (5 * k[1] + t2 * (7 * k[2] + t2 * 9 * k[3]))); };
  std::vector<double> vt(nv), vw(nv);
  for (uint32_t i = 0; i < nv; i++) { vt[i] = vdeg[i] * M_PI / 180.0; vw[i] = vv[i]; }
  auto vig = [&](double th) {
    if (!nv) return 1.0;
    if (th <= vt[0]) return vw[0];
    for (uint32_t i = 1; i < nv; i++)
      if (th <= vt[i]) return vw[i - 1] + (vw[i] - vw[i - 1]) * (th - vt[i - 1]) / (vt[i] - vt[i - 1]);
    return vw[nv - 1];
  };
  const uint32_t W = c.width, H = c.height;
  auto rows = [&](uint32_t y0, uint32_t y1) {
    for (uint32_t y = y0; y < y1; y++)
      for (uint32_t x = 0; x < W; x++) {
        // the pixel's unit ray (KB4 inverse, lens.js unproject); only its z is needed
        const double yd = (double(y) - c.cy) / c.fy, xd = (double(x) - c.cx) / c.fx - c.alpha * yd;
        const double thd = std::hypot(xd, yd);
        double z = 1.0;
        if (thd >= 1e-300) {
          double th = thd;
          for (int it = 0; it < 20; it++) {
            const double step = (distort(th) - thd) / deriv(th);
            th -= step;
            if (std::fabs(step) < 1e-15) break;
          }
          z = std::cos(th);
        }
        const double th = std::acos(std::max(-1.0, std::min(1.0, z)));
        double ri = 1.0;
        if (th > 1e-6) ri = std::pow(std::cos(th), q) * std::sin(th) / (distort(th) * deriv(th));
        out[size_t(y) * W + x] = float(std::max(0.0, ri) * vig(th));
      }
  };
  const uint32_t nt = std::max(1u, std::min(std::thread::hardware_concurrency(), (H + 63) / 64));
  std::vector<std::thread> th;
  for (uint32_t t = 0; t < nt; t++) th.emplace_back(rows, H * t / nt, H * (t + 1) / nt);
  for (auto& t : th) t.join();
}

void node_neighbours(const Prepared& S, const std::vector<uint32_t>& active, uint32_t K, double R, double sg, std::vector<uint32_t>& out) {
  const size_t n = active.size();
  out.assign(n * K * 2, 0u);
  if (!(sg > 0)) {
    const float one = 1.0f;
    for (size_t k = 0; k < n; k++) { out[k * K * 2] = uint32_t(k); std::memcpy(&out[k * K * 2 + 1], &one, 4); }
    return;
  }
  auto vf = [&](uint32_t i, int w) { float x; std::memcpy(&x, &S.verts[8 * size_t(i) + w], 4); return double(x); };
  // cells of side R: every node within R of another lies in one of the 27 cells around it
  auto cell = [&](double x) { return int64_t(std::floor(x / R)); };
  auto key = [](int64_t x, int64_t y, int64_t z) {
    return (uint64_t(x + (1 << 20)) << 42) | (uint64_t(y + (1 << 20)) << 21) | uint64_t(z + (1 << 20));
  };
  std::vector<uint64_t> keys(n);
  for (size_t k = 0; k < n; k++) keys[k] = key(cell(vf(active[k], 0)), cell(vf(active[k], 1)), cell(vf(active[k], 2)));
  std::vector<uint32_t> order(n);
  for (size_t k = 0; k < n; k++) order[k] = uint32_t(k);
  std::sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return keys[a] < keys[b] || (keys[a] == keys[b] && a < b); });
  std::vector<uint64_t> sorted(n);
  for (size_t q = 0; q < n; q++) sorted[q] = keys[order[q]];
  // nodes are independent: split them over the host's threads
  auto range = [&](size_t k0, size_t k1) {
    std::vector<double> cw(K);
    std::vector<uint32_t> cm(K);
    for (size_t k = k0; k < k1; k++) {
      const uint32_t i = active[k];
      const double px = vf(i, 0), py = vf(i, 1), pz = vf(i, 2), nx = vf(i, 4), ny = vf(i, 5), nz = vf(i, 6);
      const int64_t cx = cell(px), cy = cell(py), cz = cell(pz);
      uint32_t cnt = 0;
      for (int dx = -1; dx <= 1; dx++)
        for (int dy = -1; dy <= 1; dy++)
          for (int dz = -1; dz <= 1; dz++) {
            const uint64_t kk = key(cx + dx, cy + dy, cz + dz);
            auto lo = std::lower_bound(sorted.begin(), sorted.end(), kk);
            for (size_t q = size_t(lo - sorted.begin()); q < n && sorted[q] == kk; q++) {
              const uint32_t m = order[q], j = active[m];
              const double ex = vf(j, 0) - px, ey = vf(j, 1) - py, ez = vf(j, 2) - pz, d2 = ex * ex + ey * ey + ez * ez;
              if (d2 > R * R) continue;
              if (nx * vf(j, 4) + ny * vf(j, 5) + nz * vf(j, 6) < 0.9) continue;
              const double w = std::exp(-0.5 * d2 / (sg * sg));
              // keep the K largest (descending weight, then ascending index)
              uint32_t pos = cnt < K ? cnt : K;
              while (pos > 0 && (cw[pos - 1] < w || (cw[pos - 1] == w && cm[pos - 1] > m))) pos--;
              if (pos >= K) continue;
              for (uint32_t z = std::min(cnt, K - 1); z > pos; z--) { cw[z] = cw[z - 1]; cm[z] = cm[z - 1]; }
              cw[pos] = w; cm[pos] = m;
              if (cnt < K) cnt++;
            }
          }
      for (uint32_t z = 0; z < cnt; z++) {
        const float wf = float(cw[z]);
        out[(k * K + z) * 2] = cm[z];
        std::memcpy(&out[(k * K + z) * 2 + 1], &wf, 4);
      }
    }
  };
  const size_t nt = std::max<size_t>(1, std::min<size_t>(std::thread::hardware_concurrency(), (n + 4095) / 4096));
  if (nt == 1) { range(0, n); return; }
  std::vector<std::thread> th;
  for (size_t t = 0; t < nt; t++) th.emplace_back(range, n * t / nt, n * (t + 1) / nt);
  for (auto& x : th) x.join();
}

}  // namespace vt
