// Host side of libvtwin: scene preparation (the part of gpu/scene_gpu.js:prepareScene after welding), the BVH
// builder of gpu/bvh.js, material preparation with directional-albedo tables (gpu/bsdf.js) and the scene uniform
// written from poses (gpu/renderer.js:620-705). Everything here runs once per scene or once per pose change.
#pragma once

#include <cstdint>
#include <string>
#include <functional>
#include <vector>

#include "../../include/vtwin.h"

namespace vt {

// Scene uniform layout in 32-bit words (gpu/wgsl/common.wgsl.js:60-77 SceneU / Inst): 24 header words, then
// 48 words per instance.
constexpr int SU_WORDS = 24 + 48 * VT_MAX_INST;
constexpr int SU_INST = 24;

struct Bvh {
  std::vector<uint32_t> words;   // 16 per node
  std::vector<uint32_t> order;   // input triangle of each slot
  uint32_t node_count = 0, max_depth = 1;
  float lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
};
Bvh sah_build(const float* P, const uint32_t* I, uint32_t n_tris, uint32_t leaf_size);

struct Material {
  int kind = 0;                  // 0 dielectric, 1 conductor, 2 coated conductor
  bool emitter = false, table = true, textured = false;
  double rho[3] = {0, 0, 0}, f0[3] = {0, 0, 0}, tau[3] = {1, 1, 1}, ink[3] = {0, 0, 0};
  double roughness = 0.5, alpha = 0.25, ior = 1.5, fbar = 0, fbar_exact = 0, alpha_coat = 0, rough_ink = 0.4;
  double spec[VT_ALBEDO_BINS][3] = {}, diff[VT_ALBEDO_BINS][3] = {};
  double hh[3] = {0, 0, 0}, hh_spec[3] = {0, 0, 0};
};
Material make_material(const vt_material& m, uint32_t albedo_samples);
double fresnel_mean(double eta);

struct BodyRec {
  uint32_t root = 0, tri_off = 0, tri_count = 0;
  int32_t kind = 0, owner = -1;
  float lo[3], hi[3];
  double cap_a[3], cap_b[3], cap_r = 0, occ_a[3], occ_b[3], occ_r = 0, rho_eff = 0;
};

// an emitter triangle in its body's frame with its area CDF (gpu/scene_gpu.js emitter.tris)
struct EmitTri { double v0[3], e1[3], e2[3], n[3], area, cdf; };

struct Prepared {
  std::vector<uint32_t> nodes, tris, verts;   // 16, 16, 8 words per item
  std::vector<float> params;                  // vec4 array
  std::vector<float> node_area;
  std::vector<uint32_t> emit_of_tri;          // per triangle slot: index in the emitter table, or ~0
  uint32_t node_count = 0, tri_count = 0, vert_count = 0, static_verts = 0, static_tris = 0;
  uint32_t mesh_off = 0, mat_off = 0, alb_off = 0, prof_off = 0, prof_n = 0, emit_off = 0, emit_n = 0, emit_tris = 0;
  std::vector<BodyRec> bodies;
  std::vector<Material> mats;
  std::vector<vt_mesh> meshes;
  std::vector<vt_camera_desc> cams;
  std::vector<EmitTri> emitters;
  double emit_area = 0, emit_axis[3] = {0, 0, 1}, emit_normal[3] = {0, 0, 1}, emit_centroid[3] = {0, 0, 0}, emit_radius = 0;
  bool shadow_skips_scope = false;
  int scope_index = -1;
  float L0[3] = {1, 1, 1};
};
// builder of the static BVH (positions, vertex count, indices, triangle count, leaf size); sah_build when empty
using StaticBuilder = std::function<Bvh(const float*, uint32_t, const uint32_t*, uint32_t, uint32_t)>;
// gpu/scene_gpu.js:241-472 + gpu/renderer.js:271-306; throws std::runtime_error on bad input
Prepared prepare_scene(const vt_scene_desc& d, uint32_t leaf_size, uint32_t albedo_samples, const StaticBuilder& build_static = {});

struct InstPose { bool valid = false; double q0[4], q1[4], p0[3], p1[3]; };
// gpu/renderer.js:620 setPoses: quaternion + translation per body (T column-major 4x4; NaN hides a body)
std::vector<InstPose> poses_from(const Prepared& S, const double* T0, const double* T1, uint32_t n);
// gpu/renderer.js:642-705 _writeSceneU
// pcaps: 8 floats per body, each body's bounding capsule at the last node-radiosity update (NaN first word or a
// null pointer: its current capsule)
void scene_uniform(const Prepared& S, const std::vector<InstPose>& inst, const float eavg[3], uint32_t slot, uint32_t frame,
                   float* out /* SU_WORDS */, const float* pcaps = nullptr);

// Relative illumination x vignetting per pixel of a KB4 camera (gpu/sensor.js:98 relativeIlluminationMap), FP64:
// RI = cos^q(theta) sin(theta) / (theta_d dtheta_d/dtheta) at the pixel's ray (Newton inverse of the distortion, at
// most 20 steps), times the vignetting table (n knots, theta in degrees, linear between). out: w x h floats.
void relative_illumination(const vt_camera_desc& cam, double pupil_exponent, const double* vig_theta_deg, const double* vig, uint32_t n_vig,
                           float* out);

// Smoothing neighbours of the active nodes (gpu/renderer.js:573 _neighbours): for each active node the nbr_k largest
// Gaussian weights exp(-d^2 / 2 sigma^2) (ties: smaller active index first) over active nodes within `radius` whose
// normals agree (n.n >= 0.9), as (active index, float weight bits) pairs, weight 0 after the last. sigma <= 0: each
// node alone with weight 1.
void node_neighbours(const Prepared& S, const std::vector<uint32_t>& active, uint32_t nbr_k, double radius, double sigma,
                     std::vector<uint32_t>& out);
// gpu/renderer.js:635 _poseAt
bool pose_at(const InstPose& I, double t, double R[3][3], double p[3]);

// ------------------------------------------------------------------------ the raster camera pass (lite_nodes)
// lite_nodes/renderer.js:443 sliceTris: cut a mesh by the planes x = k h, y = k h, z = k h (one axis after the other)
// so no triangle spans more than h along any axis; crossings are computed from canonically ordered endpoints, so
// triangles that share an edge get bit-identical new vertices. In: positions / normals (3 per vertex, double),
// indices; out: an unindexed triangle list (3 vertices per triangle).
void slice_tris(const std::vector<double>& P, const std::vector<double>& N, const std::vector<uint32_t>& I, double h,
                std::vector<double>& P2, std::vector<double>& N2);
// lite_nodes/renderer.js:527 _buildGeometry: the raster vertices (8 words: position | mesh + instance << 16,
// normal | node; the static part is the scene's static vertices, instance 0xffff, node = vertex) and triangles (the
// static triangles in packed order, then every posed body's triangles mesh by mesh, sliced to h (fixtures: h_fixture))
struct LiteGeom {
  std::vector<uint32_t> v;      // 8 words per vertex
  std::vector<uint32_t> idx;    // 3 per triangle
  uint32_t n_static_verts = 0, n_static_tris = 0, n_verts = 0, n_tris = 0;
};
LiteGeom lite_geometry(const Prepared& S, double h, double h_fixture);
// lite_nodes/renderer.js:598 _buildEmitterSamples: n stratified area samples of the emitter (scope frame), each in
// one of 4 sectors about the emitter's centroid, and the sectors' centroids
struct LiteEmit {
  std::vector<double> p, n;     // 3 per sample
  std::vector<uint32_t> sect;
  double sect_c[4][3];
};
LiteEmit lite_emitter_samples(const Prepared& S, uint32_t n);

}  // namespace vt

namespace vtk {
// the static BVH built on the current CUDA device: the same words and order as vt::sah_build. False with err empty
// when the root is itself a leaf (a handful of triangles), with err set on a CUDA failure.
bool gpu_sah_build(const float* P, uint32_t n_verts, const uint32_t* I, uint32_t n, uint32_t leaf, vt::Bvh& out, std::string& err);
}  // namespace vtk
