// Scene preparation on the host, ahead of vt_create: the mesh clean-up of gpu/scene_gpu.js that the reference runs in
// JavaScript at load (weld :68, subdivide :95, benchMesh :146, computeNormals :37). Double precision like the
// JavaScript numbers; the same orders of new vertices and triangles, so the nodes (every static vertex) come out in
// the reference's numbering.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <unordered_map>
#include <vector>

#include "../../include/vtwin.h"

#include "vt_scene_prep.h"

namespace {

struct Buf {
  std::vector<double> P, N;
  std::vector<uint32_t> I;
};

vt_status hand_out(Buf&& b, vt_mesh_out* out) {
  Buf* h = new Buf(std::move(b));
  out->P = h->P.data();
  out->N = h->N.data();
  out->I = h->I.data();
  out->n_verts = uint32_t(h->P.size() / 3);
  out->n_idx = uint32_t(h->I.size());
  out->handle = h;
  return VT_OK;
}

// JavaScript's Math.round: the nearest integer, halves toward +infinity
inline long long js_round(double x) { return (long long)std::floor(x + 0.5); }

// Math.hypot of three numbers as V8 evaluates it: scaled by the largest magnitude, squares summed with Kahan
// compensation, square root times the scale
inline double js_hypot3(double x, double y, double z) {
  const double v[3] = {std::fabs(x), std::fabs(y), std::fabs(z)};
  const double mx = std::max(v[0], std::max(v[1], v[2]));
  if (mx == 0) return 0;
  double sum = 0, comp = 0;
  for (double a : v) {
    const double n = a / mx;
    const double summand = n * n - comp;
    const double pre = sum + summand;
    comp = (pre - sum) - summand;
    sum = pre;
  }
  return std::sqrt(sum) * mx;
}

struct Key6 {
  long long k[6];
  bool operator==(const Key6& o) const { return std::memcmp(k, o.k, sizeof(k)) == 0; }
};
struct Key6Hash {
  size_t operator()(const Key6& a) const {
    uint64_t h = 1469598103934665603ull;
    for (long long v : a.k) { h ^= uint64_t(v); h *= 1099511628211ull; h ^= h >> 29; }
    return size_t(h);
  }
};

}  // namespace

namespace vt {
vt_status mesh_hand_out(std::vector<double>&& P, std::vector<double>&& N, std::vector<uint32_t>&& I, vt_mesh_out* out) {
  Buf b;
  b.P = std::move(P);
  b.N = std::move(N);
  b.I = std::move(I);
  return hand_out(std::move(b), out);
}
}  // namespace vt

extern "C" {

vt_status vt_weld(const float* P, const float* N, uint32_t n_verts, const uint32_t* I, uint32_t n_idx, vt_mesh_out* out) {
  if (!out || (n_verts && (!P || !N)) || (n_idx && !I) || n_idx % 3) return VT_ERR_ARG;
  std::memset(out, 0, sizeof(*out));
  for (uint32_t k = 0; k < n_idx; k++)
    if (I[k] >= n_verts) return VT_ERR_ARG;
  Buf b;
  std::unordered_map<Key6, uint32_t, Key6Hash> map;
  map.reserve(size_t(n_verts) * 2 + 16);
  std::vector<uint32_t> remap(n_verts);
  for (uint32_t v = 0; v < n_verts; v++) {
    Key6 key;
    for (int c = 0; c < 3; c++) {
      key.k[c] = js_round(double(P[3 * size_t(v) + c]) * 1e7);
      key.k[3 + c] = js_round(double(N[3 * size_t(v) + c]) * 1e4);
    }
    auto it = map.find(key);
    if (it == map.end()) {
      const uint32_t id = uint32_t(b.P.size() / 3);
      map.emplace(key, id);
      for (int c = 0; c < 3; c++) { b.P.push_back(double(P[3 * size_t(v) + c])); b.N.push_back(double(N[3 * size_t(v) + c])); }
      remap[v] = id;
    } else {
      remap[v] = it->second;
    }
  }
  b.I.reserve(n_idx);
  for (uint32_t k = 0; k < n_idx; k += 3) {
    const uint32_t a = remap[I[k]], c1 = remap[I[k + 1]], c2 = remap[I[k + 2]];
    if (a == c1 || c1 == c2 || a == c2) continue;   // degenerate after welding
    b.I.push_back(a); b.I.push_back(c1); b.I.push_back(c2);
  }
  return hand_out(std::move(b), out);
}

vt_status vt_subdivide(const double* P, const double* N, uint32_t n_verts, const uint32_t* I, uint32_t n_idx, double h, uint32_t max_passes,
                       vt_mesh_out* out) {
  if (!out || (n_verts && (!P || !N)) || (n_idx && !I) || n_idx % 3 || !(h > 0)) return VT_ERR_ARG;
  std::memset(out, 0, sizeof(*out));
  for (uint32_t k = 0; k < n_idx; k++)
    if (I[k] >= n_verts) return VT_ERR_ARG;
  Buf b;
  b.P.assign(P, P + 3 * size_t(n_verts));
  b.N.assign(N, N + 3 * size_t(n_verts));
  std::vector<uint32_t> tris(I, I + n_idx), next;
  const double h2 = h * h;
  auto len2 = [&](uint32_t a, uint32_t c) {
    const double x = b.P[3 * size_t(a)] - b.P[3 * size_t(c)], y = b.P[3 * size_t(a) + 1] - b.P[3 * size_t(c) + 1],
                 z = b.P[3 * size_t(a) + 2] - b.P[3 * size_t(c) + 2];
    return x * x + y * y + z * z;
  };
  for (uint32_t pass = 0; pass < max_passes; pass++) {
    std::unordered_map<uint64_t, uint32_t> mid;
    bool any = false;
    // one new vertex per split edge, numbered in the order the edges are first met
    auto midpoint = [&](uint32_t a, uint32_t c) {
      const uint64_t key = a < c ? (uint64_t(a) << 32) | c : (uint64_t(c) << 32) | a;
      auto it = mid.find(key);
      if (it != mid.end()) return it->second;
      const uint32_t m = uint32_t(b.P.size() / 3);
      for (int k = 0; k < 3; k++) b.P.push_back(0.5 * (b.P[3 * size_t(a) + k] + b.P[3 * size_t(c) + k]));
      double nx = b.N[3 * size_t(a)] + b.N[3 * size_t(c)], ny = b.N[3 * size_t(a) + 1] + b.N[3 * size_t(c) + 1],
             nz = b.N[3 * size_t(a) + 2] + b.N[3 * size_t(c) + 2];
      const double l = js_hypot3(nx, ny, nz);
      if (l > 1e-6) { nx /= l; ny /= l; nz /= l; } else { nx = b.N[3 * size_t(a)]; ny = b.N[3 * size_t(a) + 1]; nz = b.N[3 * size_t(a) + 2]; }
      b.N.push_back(nx); b.N.push_back(ny); b.N.push_back(nz);
      mid.emplace(key, m);
      return m;
    };
    next.clear();
    next.reserve(tris.size() * 2);
    for (size_t k = 0; k < tris.size(); k += 3) {
      const uint32_t v[3] = {tris[k], tris[k + 1], tris[k + 2]};
      const bool mk[3] = {len2(v[0], v[1]) > h2, len2(v[1], v[2]) > h2, len2(v[2], v[0]) > h2};
      const int cnt = int(mk[0]) + int(mk[1]) + int(mk[2]);
      if (!cnt) { next.insert(next.end(), v, v + 3); continue; }
      any = true;
      if (cnt == 3) {
        const uint32_t a = midpoint(v[0], v[1]), c1 = midpoint(v[1], v[2]), c2 = midpoint(v[2], v[0]);
        const uint32_t t[12] = {v[0], a, c2, a, v[1], c1, c2, c1, v[2], a, c1, c2};
        next.insert(next.end(), t, t + 12);
      } else if (cnt == 1) {
        const int e = mk[0] ? 0 : mk[1] ? 1 : 2;
        const uint32_t p = v[e], q = v[(e + 1) % 3], r = v[(e + 2) % 3], m = midpoint(p, q);
        const uint32_t t[6] = {p, m, r, m, q, r};
        next.insert(next.end(), t, t + 6);
      } else {
        // two split edges: the unsplit one is (A, B); a corner triangle at C and the quad A, B, mBC, mCA cut by its
        // shorter diagonal
        const int e = !mk[0] ? 0 : !mk[1] ? 1 : 2;
        const uint32_t A = v[e], B = v[(e + 1) % 3], Cc = v[(e + 2) % 3];
        const uint32_t mBC = midpoint(B, Cc), mCA = midpoint(Cc, A);
        const uint32_t t0[3] = {mCA, mBC, Cc};
        next.insert(next.end(), t0, t0 + 3);
        if (len2(A, mBC) < len2(B, mCA)) { const uint32_t t[6] = {A, B, mBC, A, mBC, mCA}; next.insert(next.end(), t, t + 6); }
        else { const uint32_t t[6] = {A, B, mCA, B, mBC, mCA}; next.insert(next.end(), t, t + 6); }
      }
    }
    tris.swap(next);
    if (!any) break;
  }
  b.I = std::move(tris);
  return hand_out(std::move(b), out);
}

vt_status vt_bench_mesh(double z, const double extent[4], const double fine[4], double h, vt_mesh_out* out) {
  if (!out || !extent || !fine || !(h > 0)) return VT_ERR_ARG;
  std::memset(out, 0, sizeof(*out));
  Buf b;
  const double ex0 = extent[0], ey0 = extent[1], ex1 = extent[2], ey1 = extent[3];
  const double fx0 = std::max(ex0, fine[0]), fy0 = std::max(ey0, fine[1]), fx1 = std::min(ex1, fine[2]), fy1 = std::min(ey1, fine[3]);
  const double gx = std::ceil((fx1 - fx0) / (h * 0.999)), gy = std::ceil((fy1 - fy0) / (h * 0.999));
  if (!(gx < 1e5) || !(gy < 1e5)) return VT_ERR_ARG;   // a fine grid past 10^5 cells a side: an argument error
  const long nx = std::max(1L, long(gx)), ny = std::max(1L, long(gy));
  auto vert = [&](double x, double y) {
    b.P.push_back(x); b.P.push_back(y); b.P.push_back(z);
    b.N.push_back(0); b.N.push_back(0); b.N.push_back(1);
    return uint32_t(b.P.size() / 3 - 1);
  };
  std::vector<uint32_t> grid(size_t(nx + 1) * (ny + 1));
  for (long j = 0; j <= ny; j++)
    for (long i = 0; i <= nx; i++) grid[size_t(j) * (nx + 1) + i] = vert(fx0 + (fx1 - fx0) * double(i) / double(nx), fy0 + (fy1 - fy0) * double(j) / double(ny));
  for (long j = 0; j < ny; j++)
    for (long i = 0; i < nx; i++) {
      const uint32_t a = grid[size_t(j) * (nx + 1) + i], c = grid[size_t(j) * (nx + 1) + i + 1], d = grid[size_t(j + 1) * (nx + 1) + i],
                     e = grid[size_t(j + 1) * (nx + 1) + i + 1];
      if ((i + j) & 1) { const uint32_t t[6] = {a, c, e, a, e, d}; b.I.insert(b.I.end(), t, t + 6); }
      else { const uint32_t t[6] = {a, c, d, c, e, d}; b.I.insert(b.I.end(), t, t + 6); }
    }
  auto quad = [&](double x0, double y0, double x1, double y1) {
    if (!(x1 > x0 && y1 > y0)) return;
    const uint32_t a = vert(x0, y0), c = vert(x1, y0), d = vert(x0, y1), e = vert(x1, y1);
    const uint32_t t[6] = {a, c, e, a, e, d};
    b.I.insert(b.I.end(), t, t + 6);
  };
  quad(ex0, ey0, ex1, fy0);
  quad(ex0, fy1, ex1, ey1);
  quad(ex0, fy0, fx0, fy1);
  quad(fx1, fy0, ex1, fy1);
  return hand_out(std::move(b), out);
}

vt_status vt_compute_normals(const float* P, uint32_t n_verts, const uint32_t* I, uint32_t n_idx, float* N) {
  if ((n_verts && (!P || !N)) || (n_idx && !I) || n_idx % 3) return VT_ERR_ARG;
  for (uint32_t k = 0; k < n_idx; k++)
    if (I[k] >= n_verts) return VT_ERR_ARG;
  // the JavaScript accumulates double face normals into a Float32Array (rounded after every add)
  std::fill(N, N + 3 * size_t(n_verts), 0.0f);
  for (uint32_t k = 0; k < n_idx; k += 3) {
    const size_t a = 3 * size_t(I[k]), c = 3 * size_t(I[k + 1]), d = 3 * size_t(I[k + 2]);
    const double ux = double(P[c]) - P[a], uy = double(P[c + 1]) - P[a + 1], uz = double(P[c + 2]) - P[a + 2];
    const double vx = double(P[d]) - P[a], vy = double(P[d + 1]) - P[a + 1], vz = double(P[d + 2]) - P[a + 2];
    const double nx = uy * vz - uz * vy, ny = uz * vx - ux * vz, nz = ux * vy - uy * vx;
    for (size_t v : {a, c, d}) {
      N[v] = float(double(N[v]) + nx);
      N[v + 1] = float(double(N[v + 1]) + ny);
      N[v + 2] = float(double(N[v + 2]) + nz);
    }
  }
  for (size_t v = 0; v < 3 * size_t(n_verts); v += 3) {
    double l = js_hypot3(N[v], N[v + 1], N[v + 2]);
    if (!(l != 0)) l = 1;   // `|| 1`
    N[v] = float(double(N[v]) / l); N[v + 1] = float(double(N[v + 1]) / l); N[v + 2] = float(double(N[v + 2]) / l);
  }
  return VT_OK;
}

void vt_mesh_free(vt_mesh_out* m) {
  if (!m) return;
  delete static_cast<Buf*>(m->handle);
  std::memset(m, 0, sizeof(*m));
}

}  // extern "C"
