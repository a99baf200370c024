// Host side of the raster camera pass (lite_nodes/renderer.js): the raster geometry with the posed bodies sliced
// into short triangles, and the emitter's stratified area samples. Both run once per scene, in double precision
// like the reference's JavaScript, and store float32 like its vertex buffer.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <map>
#include <vector>

#include "vt_host.h"

namespace vt {
namespace {

struct SV { double p[3], n[3]; };
using Tri = std::array<SV, 3>;

inline float f32(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }
inline uint32_t bits(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }

// lexicographic order of positions (lite_nodes/renderer.js:449 less)
inline bool less_p(const SV& a, const SV& b) {
  if (a.p[0] != b.p[0]) return a.p[0] < b.p[0];
  if (a.p[1] != b.p[1]) return a.p[1] < b.p[1];
  return a.p[2] < b.p[2];
}
inline void norm3(double v[3]) {
  double l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  if (!(l != 0)) l = 1;
  for (int k = 0; k < 3; k++) v[k] /= l;
}
// the crossing of edge AB with the plane p[ax] = c, from the canonically first endpoint (renderer.js:450 cut)
inline SV cut(const SV& A, const SV& B, int ax, double c) {
  const SV& a = less_p(A, B) ? A : B;
  const SV& b = less_p(A, B) ? B : A;
  const double f = (c - a.p[ax]) / (b.p[ax] - a.p[ax]);
  SV x;
  for (int k = 0; k < 3; k++) x.p[k] = a.p[k] + f * (b.p[k] - a.p[k]);
  x.p[ax] = c;
  for (int k = 0; k < 3; k++) x.n[k] = a.n[k] + f * (b.n[k] - a.n[k]);
  norm3(x.n);
  return x;
}
inline void fan(const std::vector<SV>& poly, std::vector<Tri>& out) {
  for (size_t j = 1; j + 1 < poly.size(); j++) out.push_back({poly[0], poly[j], poly[j + 1]});
}

}  // namespace

void slice_tris(const std::vector<double>& P, const std::vector<double>& N, const std::vector<uint32_t>& I, double h,
                std::vector<double>& P2, std::vector<double>& N2) {
  std::vector<Tri> tris;
  tris.reserve(I.size() / 3);
  for (size_t t = 0; t + 2 < I.size(); t += 3) {
    Tri tri;
    for (int j = 0; j < 3; j++) {
      const size_t v = I[t + j];
      for (int k = 0; k < 3; k++) { tri[j].p[k] = P[3 * v + k]; tri[j].n[k] = N[3 * v + k]; }
    }
    tris.push_back(tri);
  }
  for (int ax = 0; ax < 3; ax++) {
    std::vector<Tri> out;
    out.reserve(tris.size());
    for (const Tri& tri : tris) {
      const double lo = std::min(tri[0].p[ax], std::min(tri[1].p[ax], tri[2].p[ax]));
      const double hi = std::max(tri[0].p[ax], std::max(tri[1].p[ax], tri[2].p[ax]));
      const long long k0 = (long long)std::floor(lo / h) + 1, k1 = (long long)std::ceil(hi / h) - 1;
      if (k1 < k0) { out.push_back(tri); continue; }
      std::vector<SV> poly(tri.begin(), tri.end()), below, above;
      for (long long k = k0; k <= k1 + 1; k++) {
        if (k > k1) { fan(poly, out); break; }
        const double c = double(k) * h;
        below.clear();
        above.clear();
        for (size_t j = 0; j < poly.size(); j++) {
          const SV& A = poly[j];
          const SV& B = poly[(j + 1) % poly.size()];
          const double sa = A.p[ax] - c, sb = B.p[ax] - c;
          if (sa <= 0) below.push_back(A);
          if (sa >= 0) above.push_back(A);
          if ((sa < 0 && sb > 0) || (sa > 0 && sb < 0)) {
            const SV X = cut(A, B, ax, c);
            below.push_back(X);
            above.push_back(X);
          }
        }
        if (below.size() >= 3) fan(below, out);
        if (above.size() < 3) break;
        poly = above;
      }
    }
    tris.swap(out);
  }
  P2.resize(tris.size() * 9);
  N2.resize(tris.size() * 9);
  size_t o = 0;
  for (const Tri& tri : tris)
    for (const SV& v : tri) {
      for (int k = 0; k < 3; k++) { P2[3 * o + k] = v.p[k]; N2[3 * o + k] = v.n[k]; }
      o++;
    }
}

LiteGeom lite_geometry(const Prepared& S, double h, double h_fixture) {
  LiteGeom g;
  g.n_static_verts = S.static_verts;
  g.n_static_tris = S.static_tris;
  // the static part: the packed static vertices (node i = vertex i) and triangles in slot order
  g.v.resize(size_t(S.static_verts) * 8);
  for (uint32_t i = 0; i < S.static_verts; i++) {
    const uint32_t* s = S.verts.data() + size_t(i) * 8;
    uint32_t* o = g.v.data() + size_t(i) * 8;
    o[0] = s[0]; o[1] = s[1]; o[2] = s[2]; o[3] = (s[3] & 0xffffu) | (0xffffu << 16);
    o[4] = s[4]; o[5] = s[5]; o[6] = s[6]; o[7] = i;
  }
  g.idx.reserve(size_t(S.static_tris) * 3);
  for (uint32_t k = 0; k < S.static_tris; k++) {
    const uint32_t* t = S.tris.data() + size_t(k) * 16;
    g.idx.push_back(t[3]); g.idx.push_back(t[7]); g.idx.push_back(t[11]);
  }
  // posed bodies: per body, per mesh in order of first appearance, the body-frame triangles re-indexed and sliced
  uint32_t base = S.static_verts;
  for (size_t bi = 0; bi < S.bodies.size(); bi++) {
    const BodyRec& bl = S.bodies[bi];
    std::vector<uint32_t> mesh_order;
    std::map<uint32_t, std::vector<uint32_t>> by_mesh;
    for (uint32_t k = 0; k < bl.tri_count; k++) {
      const uint32_t* t = S.tris.data() + size_t(bl.tri_off + k) * 16;
      const uint32_t mesh = t[12];
      if (mesh < S.meshes.size() && S.meshes[mesh].overview_only) continue;   // outside the cavity: not drawn
      auto it = by_mesh.find(mesh);
      if (it == by_mesh.end()) { mesh_order.push_back(mesh); it = by_mesh.emplace(mesh, std::vector<uint32_t>()).first; }
      it->second.push_back(t[3]); it->second.push_back(t[7]); it->second.push_back(t[11]);
    }
    for (uint32_t mesh : mesh_order) {
      const std::vector<uint32_t>& gi = by_mesh[mesh];
      std::map<uint32_t, uint32_t> remap;
      std::vector<double> P, N;
      std::vector<uint32_t> I;
      for (uint32_t gv : gi) {
        auto it = remap.find(gv);
        uint32_t l;
        if (it == remap.end()) {
          l = uint32_t(P.size() / 3);
          remap.emplace(gv, l);
          const uint32_t* s = S.verts.data() + size_t(gv) * 8;
          for (int k = 0; k < 3; k++) { P.push_back(double(f32(s[k]))); N.push_back(double(f32(s[4 + k]))); }
        } else {
          l = it->second;
        }
        I.push_back(l);
      }
      std::vector<double> P2, N2;
      slice_tris(P, N, I, bl.kind == VT_BODY_FIXTURE ? h_fixture : h, P2, N2);
      const uint32_t n = uint32_t(P2.size() / 3);
      for (uint32_t v = 0; v < n; v++) {
        g.v.push_back(bits(float(P2[3 * v]))); g.v.push_back(bits(float(P2[3 * v + 1]))); g.v.push_back(bits(float(P2[3 * v + 2])));
        g.v.push_back((mesh & 0xffffu) | (uint32_t(bi) << 16));
        g.v.push_back(bits(float(N2[3 * v]))); g.v.push_back(bits(float(N2[3 * v + 1]))); g.v.push_back(bits(float(N2[3 * v + 2])));
        g.v.push_back(0xffffffffu);
        g.idx.push_back(base + v);
      }
      base += n;
    }
  }
  g.n_verts = uint32_t(g.v.size() / 8);
  g.n_tris = uint32_t(g.idx.size() / 3);
  return g;
}

LiteEmit lite_emitter_samples(const Prepared& S, uint32_t n) {
  LiteEmit e;
  const double* c = S.emit_centroid;
  const double* nrm = S.emit_normal;
  const double ax[3] = {std::fabs(nrm[0]) < 0.9 ? 1.0 : 0.0, std::fabs(nrm[0]) < 0.9 ? 0.0 : 1.0, 0.0};
  double t[3] = {ax[1] * nrm[2] - ax[2] * nrm[1], ax[2] * nrm[0] - ax[0] * nrm[2], ax[0] * nrm[1] - ax[1] * nrm[0]};
  norm3(t);
  const double b[3] = {nrm[1] * t[2] - nrm[2] * t[1], nrm[2] * t[0] - nrm[0] * t[2], nrm[0] * t[1] - nrm[1] * t[0]};
  // a three-dimensional Kronecker sequence (the R3 sequence: g is the real root of g^4 = g + 1)
  const double g = 1.22074408460575947536, a1 = 1 / g, a2 = 1 / (g * g), a3 = 1 / (g * g * g);
  const std::vector<EmitTri>& T = S.emitters;
  for (uint32_t i = 0; i < n; i++) {
    const double u1 = std::fmod(0.5 + a1 * i, 1.0), u2 = std::fmod(0.5 + a2 * i, 1.0), u3 = std::fmod(0.5 + a3 * i, 1.0);
    size_t lo = 0, hi = T.empty() ? 0 : T.size() - 1;
    while (lo < hi) {
      const size_t m = (lo + hi) >> 1;
      if (T[m].cdf < u1) lo = m + 1; else hi = m;
    }
    double p[3] = {0, 0, 0}, nn[3] = {0, 0, 1};
    if (!T.empty()) {
      const EmitTri& E = T[lo];
      const double su = std::sqrt(u2);
      for (int k = 0; k < 3; k++) { p[k] = E.v0[k] + E.e1[k] * su * (1 - u3) + E.e2[k] * su * u3; nn[k] = E.n[k]; }
    }
    const double d[3] = {p[0] - c[0], p[1] - c[1], p[2] - c[2]};
    const double ang = std::atan2(d[0] * b[0] + d[1] * b[1] + d[2] * b[2], d[0] * t[0] + d[1] * t[1] + d[2] * t[2]);
    const uint32_t sect = std::min<uint32_t>(3, uint32_t(std::floor(((ang + M_PI) / (2 * M_PI)) * 4)));
    for (int k = 0; k < 3; k++) { e.p.push_back(p[k]); e.n.push_back(nn[k]); }
    e.sect.push_back(sect);
  }
  for (int k = 0; k < 4; k++) {
    double s[3] = {0, 0, 0};
    uint32_t cnt = 0;
    for (uint32_t i = 0; i < n; i++)
      if (e.sect[i] == uint32_t(k)) { for (int j = 0; j < 3; j++) s[j] += e.p[3 * i + j]; cnt++; }
    for (int j = 0; j < 3; j++) e.sect_c[k][j] = cnt ? s[j] / cnt : c[j];
  }
  return e;
}

}  // namespace vt
