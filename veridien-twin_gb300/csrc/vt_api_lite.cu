// C ABI of the raster camera pass (include/vtwin.h, "lite_nodes: the raster camera pass"): lite_nodes/renderer.js
// _init (:497), setPoses (:729), _viewData (:766), _shadowPasses (:825), renderCamera (:844), sensor (:892) and
// readback (:940), around the kernels of vt_lite.cu and the display pass of vt_isp.cu.
#include <chrono>

#include "vt_ctx.cuh"

using namespace vtapi;

namespace {

size_t al(size_t b) { return (b + 255) & ~size_t(255); }

vt_lite_opts default_opts() {
  vt_lite_opts o{};
  o.ns_static = 24; o.ns_dyn = 96; o.sm_res = 2048; o.sm_theta_max_deg = 62.0; o.far_m = 1.0;
  o.subdiv_h = 0.003; o.subdiv_fixture = 0.01; o.scope_hfov_deg = 75.0; o.scope_circle_frac = 0.95;
  o.scope_width = 1280; o.scope_height = 720;
  o.scope_view_dir[0] = 0.0; o.scope_view_dir[1] = 0.5; o.scope_view_dir[2] = 0.866;
  return o;
}

void norm3(double v[3]) {
  double l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  if (!(l != 0)) l = 1;
  for (int k = 0; k < 3; k++) v[k] /= l;
}
void cross3(const double a[3], const double b[3], double o[3]) {
  o[0] = a[1] * b[2] - a[2] * b[1]; o[1] = a[2] * b[0] - a[0] * b[2]; o[2] = a[0] * b[1] - a[1] * b[0];
}
void mul_rv(const double R[3][3], const double v[3], double o[3]) {
  for (int i = 0; i < 3; i++) o[i] = R[i][0] * v[0] + R[i][1] * v[1] + R[i][2] * v[2];
}

double out_scale(const vt_ctx* ctx) {
  const float* L0 = ctx->S.L0;
  return 1000.0 / std::max(std::max(double(L0[0]), double(L0[1])), std::max(double(L0[2]), 1e-30));
}

// setPoses (lite_nodes/renderer.js:729): the scope pose moves the emitter samples, the emission frame, the sector
// origins and the SCOPE camera; a changed scope pose makes the static shadow map stale
vt_status lite_poses(vt_ctx* ctx) {
  auto& L = ctx->lite;
  const double* T = ctx->scope_T;
  double R[3][3], P[3];
  for (int i = 0; i < 3; i++) {
    for (int j = 0; j < 3; j++) R[i][j] = T[4 * j + i];
    P[i] = T[12 + i];
  }
  std::vector<double> key(T, T + 16);
  if (key == L.scope_key) return VT_OK;
  L.scope_key = key;
  L.sm_static_dirty = true;
  std::memcpy(L.R, R, sizeof(R));
  std::memcpy(L.P, P, sizeof(P));
  auto W = [&](const double v[3], double o[3]) { mul_rv(R, v, o); for (int k = 0; k < 3; k++) o[k] += P[k]; };
  const uint32_t n = L.o.ns_dyn;
  std::vector<float> es(size_t(n) * 8);
  for (uint32_t i = 0; i < n; i++) {
    double p[3], nn[3];
    W(&L.em.p[3 * i], p);
    mul_rv(R, &L.em.n[3 * i], nn);
    float* o = es.data() + 8 * size_t(i);
    o[0] = float(p[0]); o[1] = float(p[1]); o[2] = float(p[2]); o[3] = float(L.em.sect[i]);
    o[4] = float(nn[0]); o[5] = float(nn[1]); o[6] = float(nn[2]); o[7] = float(ctx->S.emit_area);
  }
  VT_CK(cudaMemcpyAsync(L.es, es.data(), es.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
  VT_CK(cudaStreamSynchronize(ctx->stream));   // the host vector goes out of scope
  double ax[3];
  mul_rv(R, ctx->S.emit_axis, ax);
  norm3(ax);
  const double pick[3] = {std::fabs(ax[0]) < 0.9 ? 1.0 : 0.0, std::fabs(ax[0]) < 0.9 ? 0.0 : 1.0, 0.0};
  double t[3], b[3];
  cross3(pick, ax, t);
  norm3(t);
  cross3(ax, t, b);
  for (int k = 0; k < 3; k++) { L.axisW[k] = float(ax[k]); L.lt[k] = float(t[k]); L.lb[k] = float(b[k]); }
  for (int s = 0; s < 4; s++) {
    double o[3];
    W(L.em.sect_c[s], o);
    for (int k = 0; k < 3; k++) L.lo[s][k] = float(o[k]);
  }
  // the SCOPE camera follows the scope body: view direction, image up = the tilt side (+y of the scope frame)
  double vd[3] = {L.o.scope_view_dir[0], L.o.scope_view_dir[1], L.o.scope_view_dir[2]}, z[3], upK[3];
  mul_rv(R, vd, z);
  norm3(z);
  const double yK[3] = {0, 1, 0};
  mul_rv(R, yK, upK);
  const double d = upK[0] * z[0] + upK[1] * z[1] + upK[2] * z[2];
  double up[3] = {upK[0] - z[0] * d, upK[1] - z[1] * d, upK[2] - z[2] * d};
  norm3(up);
  const double y[3] = {-up[0], -up[1], -up[2]};
  double x[3];
  cross3(y, z, x);
  for (int i = 0; i < 3; i++) { L.scopeR[i][0] = x[i]; L.scopeR[i][1] = y[i]; L.scopeR[i][2] = z[i]; }
  const double oc[3] = {L.o.scope_objective[0], L.o.scope_objective[1], L.o.scope_objective[2]};
  W(oc, L.scope_pos);
  return VT_OK;
}

// _viewData (lite_nodes/renderer.js:766): camera = scene camera, n_cams = SCOPE, ~0u = a shadow view
vtl::View make_view(const vt_ctx* ctx, uint32_t camera, uint32_t casters) {
  const auto& L = ctx->lite;
  vtl::View v;
  std::memset(&v, 0, sizeof(v));
  double R[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}}, pos[3] = {0, 0, 0};
  float mode = 2, fx = 0, fy = 0, cx = 0, cy = 0, D[4] = {0, 0, 0, 0}, W = float(L.o.sm_res), H = float(L.o.sm_res), cut = 1.5f;
  uint32_t skip = 0;
  const uint32_t nc = uint32_t(ctx->S.cams.size());
  if (camera < nc) {
    const vt_camera_desc& c = ctx->S.cams[camera];
    for (int i = 0; i < 3; i++) { for (int j = 0; j < 3; j++) R[i][j] = c.T_D_C[4 * i + j]; pos[i] = c.T_D_C[4 * i + 3]; }
    mode = 0; fx = float(c.fx); fy = float(c.fy); cx = float(c.cx); cy = float(c.cy);
    for (int k = 0; k < 4; k++) D[k] = float(c.k[k]);
    W = float(c.width); H = float(c.height);
    cut = float(std::min(1.45, 1.5 * 0.97));
    skip = skip_mask(ctx, camera);
  } else if (camera == nc) {
    std::memcpy(R, L.scopeR, sizeof(R));
    std::memcpy(pos, L.scope_pos, sizeof(pos));
    const double f = L.o.scope_width / 2.0 / std::tan(L.o.scope_hfov_deg * M_PI / 180.0 / 2.0);
    mode = 1; fx = fy = float(f); cx = float(L.o.scope_width / 2.0); cy = float(L.o.scope_height / 2.0);
    W = float(L.o.scope_width); H = float(L.o.scope_height);
    if (ctx->S.scope_index >= 0) skip = 1u << ctx->S.scope_index;
  }
  for (int k = 0; k < 3; k++) { v.rx[k] = float(R[k][0]); v.ry[k] = float(R[k][1]); v.rz[k] = float(R[k][2]); v.pos[k] = float(pos[k]); }
  v.pos[3] = mode;
  v.lensA[0] = fx; v.lensA[1] = fy; v.lensA[2] = cx; v.lensA[3] = cy;
  for (int k = 0; k < 4; k++) v.lensB[k] = D[k];
  v.size[0] = W; v.size[1] = H; v.size[2] = cut; v.size[3] = float(out_scale(ctx));
  v.misc[0] = skip; v.misc[1] = L.o.ns_static; v.misc[2] = L.o.ns_dyn; v.misc[3] = casters;
  const vt::Material& dm = ctx->S.mats[std::min<size_t>(L.o.env_material, ctx->S.mats.size() - 1)];
  for (int k = 0; k < 3; k++) v.env[k] = float(double(ctx->eavg[k]) * (dm.table ? dm.hh[k] : 0.9) / M_PI);
  v.env[3] = 0.5f;
  for (int k = 0; k < 3; k++) { v.axisW[k] = L.axisW[k]; v.lt[k] = L.lt[k]; v.lb[k] = L.lb[k]; }
  uint32_t dbg = L.o.debug;
  std::memcpy(&v.axisW[3], &dbg, 4);
  v.lt[3] = float(L.o.sm_theta_max_deg * M_PI / 180.0);
  v.lb[3] = float(L.o.far_m);
  for (int s = 0; s < 4; s++) { for (int k = 0; k < 3; k++) v.lo[s][k] = L.lo[s][k]; v.lo[s][3] = 2e-4f; }
  return v;
}

vtl::Geo geo_of(const vt_ctx* ctx) {
  const auto& L = ctx->lite;
  vtl::Geo g;
  g.v = L.v; g.idx = L.idx; g.es = L.es;
  g.n_verts = L.n_verts; g.n_tris = L.n_tris; g.n_static_verts = L.n_static_verts; g.n_static_tris = L.n_static_tris;
  return g;
}

int big_blocks(const vt_ctx* ctx) {
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
  return std::max(1, sms) * 4;
}

// _shadowPasses (lite_nodes/renderer.js:825): which = 1 static casters, 2 dynamic casters; 4 sector layers
vt_status shadow_pass(vt_ctx* ctx, uint32_t which) {
  auto& L = ctx->lite;
  const vtd::Scene S = dev_scene(ctx);
  const vtl::View v = make_view(ctx, ~0u, which);
  const vtl::Geo g = geo_of(ctx);
  uint32_t* map = which == 1 ? L.sm_static : L.sm_dyn;
  const uint32_t v0 = which == 1 ? 0 : L.n_static_verts, nv = which == 1 ? L.n_static_verts : L.n_verts - L.n_static_verts;
  const uint32_t t0 = which == 1 ? 0 : L.n_static_tris, nt = which == 1 ? L.n_static_tris : L.n_tris - L.n_static_tris;
  vtl::launch_fill(map, size_t(vtl::K_SECT) * L.o.sm_res * L.o.sm_res, 0xffffffffu, ctx->stream);
  vtl::launch_vertex_shadow(S, g, v, v0, nv, L.sclip, ctx->stream);
  vtl::Target T{};
  T.W = L.o.sm_res; T.H = L.o.sm_res; T.samples = 1; T.depth = map; T.big = L.big; T.big_cap = L.big_cap;
  vtl::launch_raster(L.sclip, L.ssnap, L.idx, L.n_verts, v0, nv, t0, nt, vtl::K_SECT, T, big_blocks(ctx), ctx->stream);
  VT_CK(cudaGetLastError());
  L.launches += 5;
  return VT_OK;
}

vt_status ensure_cam(vt_ctx* ctx, uint32_t camera) {
  auto& L = ctx->lite;
  auto& C = L.cams[camera];
  const size_t px = size_t(C.W) * C.H;
  if (L.frag_pixels < px) {
    VT_CK(cudaStreamSynchronize(ctx->stream));
    cudaFree(L.frag_mem);
    L.frag_mem = nullptr;
    L.frag_pixels = 0;
    if (cudaMalloc(&L.frag_mem, al(px * 32) * 2 + al(px * 16) + al(16)) != cudaSuccess) {
      cudaGetLastError();
      return fail(ctx, VT_ERR_OOM, "lite: fragment list");
    }
    char* p = static_cast<char*>(L.frag_mem);
    L.fb.frags = reinterpret_cast<uint2*>(p); p += al(px * 32);
    L.fb.colors = reinterpret_cast<uint2*>(p); p += al(px * 32);
    L.fb.sidx = reinterpret_cast<uint4*>(p); p += al(px * 16);
    L.fb.counts = reinterpret_cast<uint32_t*>(p);
    L.frag_pixels = px;
  }
  if (C.mem) return VT_OK;
  const size_t n = size_t(C.W) * C.H;
  const size_t bytes = al(n * 32) + al(n * 16) + al(n * 4) + al(16);
  if (cudaMalloc(&C.mem, bytes) != cudaSuccess) { cudaGetLastError(); C.mem = nullptr; return fail(ctx, VT_ERR_OOM, "lite: camera targets"); }
  char* p = static_cast<char*>(C.mem);
  C.key = reinterpret_cast<unsigned long long*>(p); p += al(n * 32);
  C.rad = reinterpret_cast<float4*>(p); p += al(n * 16);
  C.out = reinterpret_cast<uchar4*>(p); p += al(n * 4);
  C.stats = reinterpret_cast<uint32_t*>(p);
  return VT_OK;
}

float ms_between(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0;
  cudaEventElapsedTime(&ms, a, b);
  return ms;
}

}  // namespace

vt_status vt_lite_create(vt_ctx* ctx, const vt_lite_opts* opts, vt_lite_info* info) {
  if (!ctx) return VT_ERR_ARG;
  if (!ctx->nodes.built) return fail(ctx, VT_ERR_STATE, "lite: build the node radiosity first (vt_nodes_build)");
  const auto t0 = std::chrono::steady_clock::now();
  auto& L = ctx->lite;
  vt_lite_opts o = opts ? *opts : default_opts();
  if (!o.ns_static) o.ns_static = 24;
  if (!o.ns_dyn) o.ns_dyn = 96;
  if (o.ns_static > o.ns_dyn) return fail(ctx, VT_ERR_ARG, "lite: ns_static > ns_dyn (the static samples are the first of the set)");
  if (o.ns_dyn > 4096) return fail(ctx, VT_ERR_ARG, "lite: ns_dyn > 4096");
  if (!o.sm_res) o.sm_res = 2048;
  if (o.sm_res > 8192) return fail(ctx, VT_ERR_ARG, "lite: sm_res > 8192");
  if (!(o.sm_theta_max_deg > 0)) o.sm_theta_max_deg = 62.0;
  if (!(o.far_m > 0)) o.far_m = 1.0;
  if (!(o.subdiv_h > 0)) o.subdiv_h = 0.003;
  if (!(o.subdiv_fixture > 0)) o.subdiv_fixture = 0.01;
  if (!(o.scope_hfov_deg > 0)) o.scope_hfov_deg = 75.0;
  if (!(o.scope_circle_frac > 0)) o.scope_circle_frac = 0.95;
  if (!o.scope_width) o.scope_width = 1280;
  if (!o.scope_height) o.scope_height = 720;
  if (o.scope_view_dir[0] == 0 && o.scope_view_dir[1] == 0 && o.scope_view_dir[2] == 0) {
    o.scope_view_dir[1] = 0.5; o.scope_view_dir[2] = 0.866;
  }
  if (o.debug > 2) return fail(ctx, VT_ERR_ARG, "lite: debug mode 0, 1 or 2");
  vt::LiteGeom gm;
  try {
    gm = vt::lite_geometry(ctx->S, o.subdiv_h, o.subdiv_fixture);
    L.em = vt::lite_emitter_samples(ctx->S, o.ns_dyn);
  } catch (const std::exception& e) {
    return fail(ctx, VT_ERR_ARG, std::string("lite: ") + e.what());
  }
  if (gm.n_tris >= (1u << 28)) return fail(ctx, VT_ERR_ARG, "lite: more than 2^28 raster triangles");
  VT_CK(cudaStreamSynchronize(ctx->stream));
  cudaFree(L.mem);
  L.mem = nullptr;
  for (auto& c : L.cams) cudaFree(c.mem);
  L.cams.clear();
  L.o = o;
  L.n_verts = gm.n_verts; L.n_tris = gm.n_tris; L.n_static_verts = gm.n_static_verts; L.n_static_tris = gm.n_static_tris;
  L.dyn_verts = gm.n_verts - gm.n_static_verts;
  L.big_cap = std::max<uint32_t>(1u << 22, std::min<uint64_t>(uint64_t(gm.n_tris) * vtl::K_SECT * 2, 1u << 26));
  const size_t smb = size_t(vtl::K_SECT) * o.sm_res * o.sm_res * 4;
  const size_t bytes = al(size_t(L.n_verts) * 32) + al(size_t(L.n_tris) * 12) + al(size_t(o.ns_dyn) * 32) + al(size_t(L.n_verts) * 16) +
                       al(size_t(vtl::K_SECT) * L.n_verts * 16) + al((size_t(L.big_cap) + 1) * 8) + 2 * al(smb) +
                       al(size_t(L.n_verts) * 16) + al(size_t(vtl::K_SECT) * L.n_verts * 16);
  if (cudaMalloc(&L.mem, bytes) != cudaSuccess) { cudaGetLastError(); L.mem = nullptr; return fail(ctx, VT_ERR_OOM, "lite: device buffers"); }
  char* p = static_cast<char*>(L.mem);
  L.v = reinterpret_cast<uint4*>(p); p += al(size_t(L.n_verts) * 32);
  L.idx = reinterpret_cast<uint32_t*>(p); p += al(size_t(L.n_tris) * 12);
  L.es = reinterpret_cast<float4*>(p); p += al(size_t(o.ns_dyn) * 32);
  L.clip = reinterpret_cast<float4*>(p); p += al(size_t(L.n_verts) * 16);
  L.sclip = reinterpret_cast<float4*>(p); p += al(size_t(vtl::K_SECT) * L.n_verts * 16);
  L.big = reinterpret_cast<uint32_t*>(p); p += al((size_t(L.big_cap) + 1) * 8);
  L.sm_static = reinterpret_cast<uint32_t*>(p); p += al(smb);
  L.sm_dyn = reinterpret_cast<uint32_t*>(p); p += al(smb);
  L.snap = reinterpret_cast<int4*>(p); p += al(size_t(L.n_verts) * 16);
  L.ssnap = reinterpret_cast<int4*>(p);
  VT_CK(cudaMemcpyAsync(L.v, gm.v.data(), gm.v.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
  VT_CK(cudaMemcpyAsync(L.idx, gm.idx.data(), gm.idx.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
  VT_CK(cudaMemsetAsync(L.sclip, 0, size_t(vtl::K_SECT) * L.n_verts * 16, ctx->stream));
  VT_CK(cudaMemsetAsync(L.clip, 0, size_t(L.n_verts) * 16, ctx->stream));
  const uint32_t nc = uint32_t(ctx->S.cams.size());
  L.cams.resize(nc + 1);
  for (uint32_t c = 0; c < nc; c++) { L.cams[c].W = ctx->S.cams[c].width; L.cams[c].H = ctx->S.cams[c].height; }
  L.cams[nc].W = o.scope_width;
  L.cams[nc].H = o.scope_height;
  for (cudaEvent_t& e : L.ev)
    if (!e) VT_CK(cudaEventCreate(&e));
  L.scope_key.clear();
  L.sm_static_dirty = true;
  L.sm_dyn_version = ~0ull;
  L.last_clip_cam = -1;
  L.ready = true;
  vt_status s = lite_poses(ctx);
  if (s != VT_OK) return s;
  VT_CK(cudaStreamSynchronize(ctx->stream));
  L.build_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return vt_lite_info_get(ctx, info);
}

vt_status vt_lite_geometry(const vt_scene_desc* scene, double subdiv_h, double subdiv_fixture, uint32_t counts[2], uint32_t* verts, uint32_t* idx) {
  if (!scene || !counts || !(subdiv_h > 0) || !(subdiv_fixture > 0)) return VT_ERR_ARG;
  try {
    const vt::Prepared S = vt::prepare_scene(*scene, 4, 16);
    const vt::LiteGeom g = vt::lite_geometry(S, subdiv_h, subdiv_fixture);
    const uint32_t cap_v = counts[0], cap_t = counts[1];
    counts[0] = g.n_verts;
    counts[1] = g.n_tris;
    if (verts && cap_v >= g.n_verts) std::memcpy(verts, g.v.data(), g.v.size() * 4);
    if (idx && cap_t >= g.n_tris) std::memcpy(idx, g.idx.data(), g.idx.size() * 4);
  } catch (const std::exception&) {
    return VT_ERR_ARG;
  }
  return VT_OK;
}

vt_status vt_lite_info_get(vt_ctx* ctx, vt_lite_info* info) {
  if (!ctx) return VT_ERR_ARG;
  if (!info) return VT_OK;
  const auto& L = ctx->lite;
  std::memset(info, 0, sizeof(*info));
  info->raster_tris = L.n_tris; info->static_tris = L.n_static_tris; info->dyn_verts = L.dyn_verts;
  info->n_cameras = uint32_t(L.cams.size());
  info->build_ms = L.build_ms;
  info->shadow_static_ms = L.sm_static_ms; info->shadow_dyn_ms = L.sm_dyn_ms; info->camera_ms = L.cam_ms;
  info->camera_raster_ms = L.raster_ms; info->camera_shade_ms = L.shade_ms;
  info->big_tris = L.big_tris; info->launches = L.launches; info->shadow_big_tiles = L.shadow_big;
  return VT_OK;
}

vt_status vt_lite_render_camera(vt_ctx* ctx, uint32_t camera, float* out_rgba) {
  if (!ctx) return VT_ERR_ARG;
  auto& L = ctx->lite;
  if (!L.ready) return fail(ctx, VT_ERR_STATE, "lite: vt_lite_create first");
  if (camera >= L.cams.size()) return fail(ctx, VT_ERR_UNKNOWN_CAMERA, "unknown camera " + std::to_string(camera));
  // node radiosity for the current poses (lite_nodes/renderer.js:849 _ensureRadiosity)
  if (ctx->nodes.built && ctx->nodes.auto_update) {
    vt_status s = vt_nodes_update(ctx, 0, nullptr);
    if (s != VT_OK) return s;
  }
  vt_status s = lite_poses(ctx);
  if (s != VT_OK) return s;
  if ((s = ensure_cam(ctx, camera)) != VT_OK) return s;
  auto& C = L.cams[camera];
  L.launches = 0;
  const bool do_static = L.sm_static_dirty, do_dyn = L.sm_dyn_version != ctx->nodes.poses_version;
  VT_CK(cudaEventRecord(L.ev[0], ctx->stream));
  if (do_static) { if ((s = shadow_pass(ctx, 1)) != VT_OK) return s; L.sm_static_dirty = false; }
  VT_CK(cudaEventRecord(L.ev[1], ctx->stream));
  if (do_dyn) {
    if ((s = shadow_pass(ctx, 2)) != VT_OK) return s;
    L.sm_dyn_version = ctx->nodes.poses_version;
    VT_CK(cudaMemcpyAsync(&L.shadow_big, L.big, 4, cudaMemcpyDeviceToHost, ctx->stream));
  }
  VT_CK(cudaEventRecord(L.ev[2], ctx->stream));
  // the camera pass: vertices, raster into the 4-sample keys, fragments + resolve + finish
  const vtd::Scene S = dev_scene(ctx);
  const vtl::View v = make_view(ctx, camera, 0);
  const vtl::Geo g = geo_of(ctx);
  vtl::launch_vertex_cam(S, g, v, 0, L.n_verts, L.clip, ctx->stream);
  VT_CK(cudaMemsetAsync(C.key, 0xff, size_t(C.W) * C.H * 32, ctx->stream));
  vtl::Target T{};
  T.W = C.W; T.H = C.H; T.samples = 4; T.key = C.key; T.big = L.big; T.big_cap = L.big_cap;
  vtl::launch_raster(L.clip, L.snap, L.idx, L.n_verts, 0, L.n_verts, 0, L.n_tris, 1, T, big_blocks(ctx), ctx->stream);
  VT_CK(cudaEventRecord(L.ev[4], ctx->stream));
  vtl::ShadeArgs a{};
  a.key = C.key; a.clip = L.clip; a.sm_static = L.sm_static; a.sm_dyn = L.sm_dyn; a.sm_res = L.o.sm_res;
  a.inv_scale = float(1.0 / out_scale(ctx));
  a.circle = camera == uint32_t(ctx->S.cams.size()) ? float(L.o.scope_circle_frac * L.o.scope_width / 2.0) : 0.0f;
  a.env_mat = L.o.env_material;
  a.out = C.rad;
  vtl::launch_shade(S, g, v, a, L.fb, big_blocks(ctx) / 4, ctx->stream);
  VT_CK(cudaGetLastError());
  L.launches += 7;
  VT_CK(cudaEventRecord(L.ev[3], ctx->stream));
  VT_CK(cudaMemcpyAsync(&L.big_tris, L.big, 4, cudaMemcpyDeviceToHost, ctx->stream));
  if (out_rgba) { if ((s = from_device(ctx, out_rgba, C.rad, size_t(C.W) * C.H * 16)) != VT_OK) return s; }
  VT_CK(cudaStreamSynchronize(ctx->stream));
  L.sm_static_ms = do_static ? ms_between(L.ev[0], L.ev[1]) : 0.0;
  L.sm_dyn_ms = do_dyn ? ms_between(L.ev[1], L.ev[2]) : 0.0;
  L.cam_ms = ms_between(L.ev[2], L.ev[3]);
  L.raster_ms = ms_between(L.ev[2], L.ev[4]);
  L.shade_ms = ms_between(L.ev[4], L.ev[3]);
  L.last_clip_cam = int32_t(camera);
  C.rendered = true;
  C.displayed = false;
  ctx->tim.launches += L.launches;
  return VT_OK;
}

vt_status vt_lite_display(vt_ctx* ctx, uint32_t camera, const float du[20], const uint32_t prev[4], uint32_t stats[4]) {
  if (!ctx || !du) return VT_ERR_ARG;
  auto& L = ctx->lite;
  if (!L.ready) return fail(ctx, VT_ERR_STATE, "lite: vt_lite_create first");
  if (camera >= L.cams.size()) return fail(ctx, VT_ERR_UNKNOWN_CAMERA, "unknown camera " + std::to_string(camera));
  auto& C = L.cams[camera];
  if (!C.rendered) return fail(ctx, VT_ERR_STATE, "lite: display before render");
  vtk::LiteDisplay P{};
  std::memcpy(P.du, du, sizeof(P.du));
  if (prev) std::memcpy(P.prev, prev, sizeof(P.prev));
  P.W = C.W; P.H = C.H;
  vtk::launch_lite_display(P, C.rad, C.out, C.stats, ctx->stream);
  VT_CK(cudaGetLastError());
  uint32_t h[4] = {0, 0, 0, 0};
  VT_CK(cudaMemcpyAsync(h, C.stats, 16, cudaMemcpyDeviceToHost, ctx->stream));
  VT_CK(cudaStreamSynchronize(ctx->stream));
  if (stats) std::memcpy(stats, h, 16);
  C.displayed = true;
  ctx->tim.launches += 1;
  return VT_OK;
}

vt_status vt_lite_readback(vt_ctx* ctx, uint32_t camera, int kind, void* dst, size_t bytes) {
  if (!ctx || !dst) return VT_ERR_ARG;
  auto& L = ctx->lite;
  if (!L.ready) return fail(ctx, VT_ERR_STATE, "lite: vt_lite_create first");
  if (camera >= L.cams.size()) return fail(ctx, VT_ERR_UNKNOWN_CAMERA, "unknown camera " + std::to_string(camera));
  auto& C = L.cams[camera];
  const size_t n = size_t(C.W) * C.H;
  if (kind == VT_READ_LINEAR) {
    if (!C.rendered) return fail(ctx, VT_ERR_STATE, "lite: readback before render");
    if (bytes < n * 16) return fail(ctx, VT_ERR_ARG, "lite readback: buffer too small");
    vt_status s = from_device(ctx, dst, C.rad, n * 16);
    if (s != VT_OK) return s;
  } else if (kind == VT_READ_RGBA8 || kind == VT_READ_RGB8) {
    if (!C.displayed) return fail(ctx, VT_ERR_STATE, "lite: 8-bit readback before display");
    const size_t ch = kind == VT_READ_RGBA8 ? 4 : 3;
    if (bytes < n * ch) return fail(ctx, VT_ERR_ARG, "lite readback: buffer too small");
    std::vector<uint8_t> h(n * 4);
    VT_CK(cudaMemcpyAsync(h.data(), C.out, n * 4, cudaMemcpyDeviceToHost, ctx->stream));
    VT_CK(cudaStreamSynchronize(ctx->stream));
    uint8_t* o = static_cast<uint8_t*>(dst);
    if (ch == 4) std::memcpy(o, h.data(), n * 4);
    else for (size_t i = 0; i < n; i++) { o[3 * i] = h[4 * i]; o[3 * i + 1] = h[4 * i + 1]; o[3 * i + 2] = h[4 * i + 2]; }
    return VT_OK;
  } else {
    return fail(ctx, VT_ERR_ARG, "lite readback: linear, rgb8 or rgba8 (the raster pass has no raw or YCbCr planes)");
  }
  VT_CK(cudaStreamSynchronize(ctx->stream));
  return VT_OK;
}

vt_status vt_lite_debug(vt_ctx* ctx, int what, uint32_t camera, void* dst, size_t bytes) {
  if (!ctx || !dst) return VT_ERR_ARG;
  auto& L = ctx->lite;
  if (!L.ready) return fail(ctx, VT_ERR_STATE, "lite: vt_lite_create first");
  if (camera >= L.cams.size()) return fail(ctx, VT_ERR_UNKNOWN_CAMERA, "unknown camera " + std::to_string(camera));
  const void* src = nullptr;
  size_t n = 0;
  switch (what) {
    case VT_LITE_VIEW: {
      if (bytes < sizeof(vtl::View)) return fail(ctx, VT_ERR_ARG, "lite debug: buffer too small");
      vt_status s = lite_poses(ctx);
      if (s != VT_OK) return s;
      const vtl::View v = make_view(ctx, camera, 0);
      std::memcpy(dst, &v, sizeof(v));
      return VT_OK;
    }
    case VT_LITE_CLIP:
      if (L.last_clip_cam != int32_t(camera)) return fail(ctx, VT_ERR_STATE, "lite debug: clip coordinates are those of the last rendered camera");
      src = L.clip; n = size_t(L.n_verts) * 16; break;
    case VT_LITE_KEYS:
      if (!L.cams[camera].rendered) return fail(ctx, VT_ERR_STATE, "lite debug: camera not rendered");
      src = L.cams[camera].key; n = size_t(L.cams[camera].W) * L.cams[camera].H * 32; break;
    case VT_LITE_SM_STATIC: src = L.sm_static; n = size_t(vtl::K_SECT) * L.o.sm_res * L.o.sm_res * 4; break;
    case VT_LITE_SM_DYN: src = L.sm_dyn; n = size_t(vtl::K_SECT) * L.o.sm_res * L.o.sm_res * 4; break;
    case VT_LITE_SM_CLIP: src = L.sclip; n = size_t(vtl::K_SECT) * L.n_verts * 16; break;
    case VT_LITE_GEOM: src = L.v; n = size_t(L.n_verts) * 32; break;
    case VT_LITE_INDEX: src = L.idx; n = size_t(L.n_tris) * 12; break;
    case VT_LITE_EMIT: {
      vt_status s = lite_poses(ctx);   // the samples as the current poses place them
      if (s != VT_OK) return s;
      src = L.es; n = size_t(L.o.ns_dyn) * 32;
      break;
    }
    default: return fail(ctx, VT_ERR_ARG, "lite debug: unknown buffer");
  }
  if (bytes < n) return fail(ctx, VT_ERR_ARG, "lite debug: buffer too small");
  vt_status s = from_device(ctx, dst, src, n);
  if (s != VT_OK) return s;
  VT_CK(cudaStreamSynchronize(ctx->stream));
  return VT_OK;
}

vt_status vt_raster(vt_ctx* ctx, const float* clip, uint32_t n_verts, const uint32_t* idx, uint32_t n_tris, uint32_t width, uint32_t height,
                    uint32_t samples, uint64_t* keys) {
  if (!ctx || !clip || !idx || !keys || !n_verts) return VT_ERR_ARG;
  if (samples != 1 && samples != 4) return fail(ctx, VT_ERR_ARG, "raster: 1 or 4 samples per pixel");
  if (!width || !height || width > 16384 || height > 16384) return fail(ctx, VT_ERR_ARG, "raster: target size 1..16384");
  if (n_tris >= (1u << 28)) return fail(ctx, VT_ERR_ARG, "raster: more than 2^28 triangles");
  if (reject_foreign(ctx, {clip, idx, keys}) != VT_OK) return VT_ERR_ARG;
  // every index in range before anything reaches the device
  std::vector<uint32_t> hidx(size_t(n_tris) * 3);
  if (is_device_ptr(idx)) { VT_CK(cudaMemcpy(hidx.data(), idx, hidx.size() * 4, cudaMemcpyDeviceToHost)); }
  else std::memcpy(hidx.data(), idx, hidx.size() * 4);
  for (uint32_t i : hidx)
    if (i >= n_verts) return fail(ctx, VT_ERR_ARG, "raster: index out of range");
  const size_t nk = size_t(width) * height * 4;
  const uint32_t cap = 1u << 20;
  const size_t bytes = al(size_t(n_verts) * 16) + al(hidx.size() * 4) + al(nk * 8) + al((size_t(cap) + 1) * 8) + al(size_t(n_verts) * 16);
  void* mem = nullptr;
  if (cudaMalloc(&mem, bytes) != cudaSuccess) { cudaGetLastError(); return fail(ctx, VT_ERR_OOM, "raster: device buffers"); }
  char* p = static_cast<char*>(mem);
  float4* dclip = reinterpret_cast<float4*>(p); p += al(size_t(n_verts) * 16);
  uint32_t* didx = reinterpret_cast<uint32_t*>(p); p += al(hidx.size() * 4);
  unsigned long long* dkey = reinterpret_cast<unsigned long long*>(p); p += al(nk * 8);
  uint32_t* dbig = reinterpret_cast<uint32_t*>(p); p += al((size_t(cap) + 1) * 8);
  int4* dsnap = reinterpret_cast<int4*>(p);
  vt_status s = VT_OK;
  auto run = [&]() -> vt_status {
    vt_status r = to_device(ctx, dclip, clip, size_t(n_verts) * 16);
    if (r != VT_OK) return r;
    VT_CK(cudaMemcpyAsync(didx, hidx.data(), hidx.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
    VT_CK(cudaMemsetAsync(dkey, 0xff, nk * 8, ctx->stream));
    vtl::Target T{};
    T.W = width; T.H = height; T.samples = samples; T.big = dbig; T.big_cap = cap;
    if (samples == 4) {
      T.key = dkey;
      vtl::launch_raster(dclip, dsnap, didx, n_verts, 0, n_verts, 0, n_tris, 1, T, big_blocks(ctx), ctx->stream);
    } else {
      // one 32-bit depth layer in the first half of the key buffer, triangles recovered below by a second pass
      T.depth = reinterpret_cast<uint32_t*>(dkey);
      vtl::launch_fill(T.depth, size_t(width) * height, 0xffffffffu, ctx->stream);
      vtl::launch_raster(dclip, dsnap, didx, n_verts, 0, n_verts, 0, n_tris, 1, T, big_blocks(ctx), ctx->stream);
    }
    VT_CK(cudaGetLastError());
    if (samples == 4) {
      r = from_device(ctx, keys, dkey, nk * 8);
      if (r != VT_OK) return r;
    } else {
      std::vector<uint32_t> d(size_t(width) * height);
      VT_CK(cudaMemcpyAsync(d.data(), dkey, d.size() * 4, cudaMemcpyDeviceToHost, ctx->stream));
      VT_CK(cudaStreamSynchronize(ctx->stream));
      std::vector<unsigned long long> h(d.size());
      for (size_t i = 0; i < d.size(); i++) h[i] = d[i] == 0xffffffffu ? ~0ull : (static_cast<unsigned long long>(d[i]) << 32) | 0xffffffffull;
      if (is_device_ptr(keys)) { VT_CK(cudaMemcpy(keys, h.data(), h.size() * 8, cudaMemcpyHostToDevice)); }
      else std::memcpy(keys, h.data(), h.size() * 8);
    }
    VT_CK(cudaStreamSynchronize(ctx->stream));
    return VT_OK;
  };
  s = run();
  cudaStreamSynchronize(ctx->stream);
  cudaFree(mem);
  return s;
}
