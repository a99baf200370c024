// The C ABI of include/vtwin.h: contexts, device-resident scene, poses, rendering, ray queries, sensor and the
// node-radiosity solve. One CUDA stream per context. There is no CPU fallback: without a device every entry
// point that needs one returns VT_ERR_NO_DEVICE.
#include <cuda_runtime.h>

#include <algorithm>
#include <stdexcept>
#include <cmath>
#include <cstring>
#include <exception>
#include <string>
#include <vector>

#include "vt_tc.cuh"

#include "vt_ctx.cuh"

using namespace vtapi;

extern "C" {

const char* vt_last_error(const vt_ctx* ctx) { return ctx ? ctx->err.c_str() : g_static_err; }
void* vt_stream(vt_ctx* ctx) { return ctx ? reinterpret_cast<void*>(ctx->stream) : nullptr; }

uint32_t vt_bvh_capacity(uint32_t n_tris, uint32_t leaf_size) {
  // every node is interior and holds two children, every leaf at least one triangle: at most n_tris - 1 nodes
  (void)leaf_size;
  return std::max<uint32_t>(4, n_tris);
}

vt_status vt_bvh_build(const float* pos, uint32_t n_verts, const uint32_t* idx, uint32_t n_tris, uint32_t leaf_size, uint32_t* nodes_out,
                       uint32_t* order_out, vt_bvh_result* res) {
  if ((n_tris && (!pos || !idx)) || !nodes_out || !res || (n_tris && !order_out)) return VT_ERR_ARG;
  for (uint64_t i = 0; i < uint64_t(n_tris) * 3; i++) if (idx[i] >= n_verts) return VT_ERR_ARG;
  vt::Bvh b = vt::sah_build(pos, idx, n_tris, leaf_size);
  if (b.node_count > vt_bvh_capacity(n_tris, leaf_size)) return VT_ERR_ARG;
  std::copy(b.words.begin(), b.words.end(), nodes_out);
  std::copy(b.order.begin(), b.order.end(), order_out);
  res->node_count = b.node_count;
  res->max_depth = b.max_depth;
  for (int k = 0; k < 3; k++) { res->bmin[k] = b.lo[k]; res->bmax[k] = b.hi[k]; }
  return VT_OK;
}

vt_status vt_bvh_build_device(int32_t device, const float* pos, uint32_t n_verts, const uint32_t* idx, uint32_t n_tris, uint32_t leaf_size,
                              uint32_t* nodes_out, uint32_t* order_out, vt_bvh_result* res) {
  if ((n_tris && (!pos || !idx)) || !nodes_out || !res || (n_tris && !order_out)) return VT_ERR_ARG;
  for (uint64_t i = 0; i < uint64_t(n_tris) * 3; i++) if (idx[i] >= n_verts) return VT_ERR_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev || cudaSetDevice(device) != cudaSuccess) {
    cudaGetLastError();
    return VT_ERR_NO_DEVICE;
  }
  vt::Bvh b;
  std::string err;
  if (!vtk::gpu_sah_build(pos, n_verts, idx, n_tris, leaf_size, b, err)) {
    if (!err.empty()) { g_static_err = "gpu bvh build failed"; return VT_ERR_CUDA; }
    b = vt::sah_build(pos, idx, n_tris, leaf_size);
  }
  if (b.node_count > vt_bvh_capacity(n_tris, leaf_size)) return VT_ERR_ARG;
  std::copy(b.words.begin(), b.words.end(), nodes_out);
  std::copy(b.order.begin(), b.order.end(), order_out);
  res->node_count = b.node_count;
  res->max_depth = b.max_depth;
  for (int k = 0; k < 3; k++) { res->bmin[k] = b.lo[k]; res->bmax[k] = b.hi[k]; }
  return VT_OK;
}

vt_status vt_create(const vt_scene_desc* scene, const vt_options* opts, vt_ctx** out) {
  if (!scene || !out) return VT_ERR_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) { cudaGetLastError(); return VT_ERR_NO_DEVICE; }
  vt_ctx* ctx = new vt_ctx();
  const uint32_t leaf = opts && opts->leaf_size ? opts->leaf_size : 4;
  const uint32_t albs = opts && opts->albedo_samples ? opts->albedo_samples : 1024;
  ctx->device = opts ? opts->device : 0;
  if (cudaSetDevice(ctx->device) != cudaSuccess) { cudaGetLastError(); delete ctx; return VT_ERR_NO_DEVICE; }
  // the static BVH is built on the device (the host builder's tree); a root that is itself a leaf stays on the host
  auto build_static = [](const float* P, uint32_t nv, const uint32_t* I, uint32_t n, uint32_t lf) {
    vt::Bvh b;
    std::string err;
    if (vtk::gpu_sah_build(P, nv, I, n, lf, b, err)) return b;
    if (!err.empty()) throw std::runtime_error(err);
    return vt::sah_build(P, I, n, lf);
  };
  try {
    ctx->S = vt::prepare_scene(*scene, leaf, albs, build_static);
  } catch (const std::exception& e) {
    const std::string m = e.what();
    delete ctx;
    g_static_err = "scene preparation failed";
    if (m.find("gpu bvh build") != std::string::npos) return VT_ERR_CUDA;
    return m.find("too many bodies") != std::string::npos ? VT_ERR_TOO_MANY_BODIES : VT_ERR_ARG;
  }
  auto bail = [&](vt_status s) { vt_destroy(ctx); return s; };
  if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) return bail(VT_ERR_CUDA);
  if (cudaEventCreate(&ctx->ev0) != cudaSuccess || cudaEventCreate(&ctx->ev1) != cudaSuccess || cudaEventCreate(&ctx->ev2) != cudaSuccess ||
      cudaEventCreate(&ctx->ev3) != cudaSuccess)
    return bail(VT_ERR_CUDA);
  for (cudaEvent_t& e : ctx->nev)
    if (cudaEventCreate(&e) != cudaSuccess) return bail(VT_ERR_CUDA);
  const vt::Prepared& S = ctx->S;
  vt_status s;
  if ((s = upload(ctx, &ctx->d_nodes, S.nodes.data(), S.nodes.size() * 4)) != VT_OK) return bail(s);
  {
    const std::vector<uint32_t> top = top_records(S.nodes, 0, vtd::TOP_NODES);
    ctx->n_top = uint32_t(top.size() / VT_NODE_WORDS);
    if (ctx->n_top && (s = upload(ctx, &ctx->d_top, top.data(), top.size() * 4)) != VT_OK) return bail(s);
  }
  if ((s = upload(ctx, &ctx->d_tris, S.tris.data(), S.tris.size() * 4)) != VT_OK) return bail(s);
  if ((s = upload(ctx, &ctx->d_verts, S.verts.data(), S.verts.size() * 4)) != VT_OK) return bail(s);
  if ((s = upload(ctx, &ctx->d_params, S.params.data(), S.params.size() * 4)) != VT_OK) return bail(s);
  // node state: E_free|V = (0,0,0,1), slots 0, B_dir|vis = (0,0,0,-1) (gpu/renderer.js:323-327)
  std::vector<float> st(std::max<size_t>(16, size_t(S.static_verts) * 16), 0.0f);
  for (uint32_t i = 0; i < S.static_verts; i++) { st[16 * i + 3] = 1; st[16 * i + 15] = -1; }
  if ((s = upload(ctx, &ctx->d_nstate, st.data(), st.size() * 4)) != VT_OK) return bail(s);
  if (cudaMalloc(&ctx->d_su, sizeof(ctx->su_host)) != cudaSuccess) return bail(VT_ERR_OOM);
  if (cudaMalloc(&ctx->d_dbg, 64) != cudaSuccess || cudaMemsetAsync(ctx->d_dbg, 0, 64, ctx->stream) != cudaSuccess) return bail(VT_ERR_OOM);
  if (cudaMalloc(&ctx->d_work, 256) != cudaSuccess) return bail(VT_ERR_OOM);
  ctx->cams.resize(S.cams.size());
  for (size_t c = 0; c < S.cams.size(); c++) {
    const size_t px = size_t(S.cams[c].width) * S.cams[c].height;
    if (cudaMalloc(&ctx->cams[c].radiance, std::max<size_t>(px, 1) * 16) != cudaSuccess) return bail(VT_ERR_OOM);
    if (cudaMalloc(&ctx->cams[c].raw, std::max<size_t>(px, 1) * 4) != cudaSuccess) return bail(VT_ERR_OOM);
  }
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
  ctx->wave_blocks = std::max(1, sms) * vtk::wave_blocks_per_sm();
  // no poses yet: bodies of kind 'fixed' at identity, the rest hidden (gpu/renderer.js:259 setPoses({bodies: {}}))
  ctx->inst = vt::poses_from(S, nullptr, nullptr, 0);
  if ((s = write_su(ctx)) != VT_OK) return bail(s);
  if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) return bail(VT_ERR_CUDA);
  *out = ctx;
  return VT_OK;
}

vt_status vt_destroy(vt_ctx* ctx) {
  if (!ctx) return VT_ERR_ARG;
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  for (auto& c : ctx->cams) { cudaFree(c.radiance); cudaFree(c.raw); cudaFree(c.ri); cudaFree(c.isp_mem); cudaFree(c.hcache); cudaFree(c.scache); }
  cudaFree(ctx->d_nodes); cudaFree(ctx->d_top); cudaFree(ctx->d_tris); cudaFree(ctx->d_verts); cudaFree(ctx->d_params); cudaFree(ctx->d_nstate);
  cudaFree(ctx->d_su); cudaFree(ctx->d_dbg); cudaFree(ctx->d_work); cudaFree(ctx->d_scratch); cudaFree(ctx->d_wave); cudaFree(ctx->tc.mem);
  cudaFree(ctx->batch.su); cudaFree(ctx->batch.cull); cudaFree(ctx->batch.ctr); cudaFree(ctx->batch.sensor); cudaFree(ctx->batch.mem);
  cudaFree(ctx->batch.rad); cudaFree(ctx->batch.raw);
  if (ctx->batch.exec) cudaGraphExecDestroy(ctx->batch.exec);
  for (auto& e : ctx->kev) cudaEventDestroy(e);
  cudaFree(ctx->calib.mem);
  cudaFree(ctx->nodes.mem);
  cudaFree(ctx->nodes.table_mem);
  cudaFree(ctx->nodes.direct_mem);
  cudaFree(ctx->calib.records);
  cudaFree(ctx->calib.tan);
  cudaFree(ctx->calib.dec);
  for (float4* p : ctx->calib.image) cudaFree(p);
  for (float4* p : ctx->calib.target) cudaFree(p);
  if (ctx->ev0) cudaEventDestroy(ctx->ev0);
  if (ctx->ev1) cudaEventDestroy(ctx->ev1);
  if (ctx->ev2) cudaEventDestroy(ctx->ev2);
  if (ctx->ev3) cudaEventDestroy(ctx->ev3);
  for (cudaEvent_t e : ctx->nev)
    if (e) cudaEventDestroy(e);
  if (ctx->h_stats) cudaFreeHost(ctx->h_stats);
  cudaFree(ctx->lite.mem);
  cudaFree(ctx->lite.frag_mem);
  for (auto& c : ctx->lite.cams) cudaFree(c.mem);
  for (cudaEvent_t e : ctx->lite.ev)
    if (e) cudaEventDestroy(e);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return VT_OK;
}

vt_status vt_scene_info_get(const vt_ctx* ctx, vt_scene_info* o) {
  if (!ctx || !o) return VT_ERR_ARG;
  const vt::Prepared& S = ctx->S;
  o->node_count = S.node_count; o->tri_count = S.tri_count; o->vert_count = S.vert_count;
  o->param_vec4s = uint32_t(S.params.size() / 4); o->static_verts = S.static_verts; o->static_tris = S.static_tris;
  o->n_bodies = uint32_t(S.bodies.size()); o->n_materials = uint32_t(S.mats.size()); o->n_meshes = uint32_t(S.meshes.size());
  o->emit_tris = S.emit_tris; o->mesh_off = S.mesh_off; o->mat_off = S.mat_off; o->alb_off = S.alb_off; o->prof_off = S.prof_off;
  o->prof_n = S.prof_n; o->emit_off = S.emit_off;
  o->emit_area = float(S.emit_area); o->emit_radius = float(S.emit_radius);
  for (int k = 0; k < 3; k++) { o->emit_axis[k] = float(S.emit_axis[k]); o->emit_normal[k] = float(S.emit_normal[k]); o->emit_centroid[k] = float(S.emit_centroid[k]); }
  o->shadow_skips_scope = S.shadow_skips_scope; o->scope_index = S.scope_index;
  return VT_OK;
}

vt_status vt_scene_export(const vt_ctx* ctx, uint32_t* nodes, uint32_t* tris, uint32_t* verts, float* params) {
  if (!ctx) return VT_ERR_ARG;
  const vt::Prepared& S = ctx->S;
  if (nodes) std::copy(S.nodes.begin(), S.nodes.end(), nodes);
  if (tris) std::copy(S.tris.begin(), S.tris.end(), tris);
  if (verts) std::copy(S.verts.begin(), S.verts.end(), verts);
  if (params) std::copy(S.params.begin(), S.params.end(), params);
  return VT_OK;
}

vt_status vt_blas_info_get(const vt_ctx* ctx, uint32_t body, vt_blas_info* o) {
  if (!ctx || !o || body >= ctx->S.bodies.size()) return VT_ERR_ARG;
  const vt::BodyRec& b = ctx->S.bodies[body];
  o->root = b.root; o->tri_off = b.tri_off; o->tri_count = b.tri_count; o->kind = b.kind;
  for (int k = 0; k < 3; k++) {
    o->bmin[k] = b.lo[k]; o->bmax[k] = b.hi[k]; o->cap_a[k] = float(b.cap_a[k]); o->cap_b[k] = float(b.cap_b[k]);
    o->occ_a[k] = float(b.occ_a[k]); o->occ_b[k] = float(b.occ_b[k]);
  }
  o->cap_r = float(b.cap_r); o->occ_r = float(b.occ_r); o->rho_eff = float(b.rho_eff);
  return VT_OK;
}

vt_status vt_set_poses(vt_ctx* ctx, const double* T0, const double* T1, uint32_t n_bodies) {
  if (!ctx) return VT_ERR_ARG;
  if (n_bodies && !T0) return fail(ctx, VT_ERR_ARG, "poses: T0 is null");
  ctx->inst = vt::poses_from(ctx->S, T0, T1, n_bodies);
  ctx->nodes.poses_version++;
  {
    const int sc = ctx->S.scope_index;
    const bool have = sc >= 0 && uint32_t(sc) < n_bodies && T0 && !std::isnan(T0[16 * size_t(sc)]);
    for (int k = 0; k < 16; k++) ctx->scope_T[k] = have ? T0[16 * size_t(sc) + k] : (k % 5 == 0 ? 1.0 : 0.0);
  }
  return write_su(ctx);
}

vt_status vt_set_eavg(vt_ctx* ctx, const float e[3]) {
  if (!ctx || !e) return VT_ERR_ARG;
  for (int k = 0; k < 3; k++) ctx->eavg[k] = e[k];
  return write_su(ctx);
}

vt_status vt_scene_uniform_get(const vt_ctx* ctx, void* out, size_t bytes) {
  if (!ctx || !out || bytes < sizeof(ctx->su_host)) return VT_ERR_ARG;
  std::memcpy(out, ctx->su_host, sizeof(ctx->su_host));
  return VT_OK;
}

vt_status vt_set_node_state(vt_ctx* ctx, const float* state, uint32_t slot) {
  if (!ctx || !state || slot < 1 || slot > 2) return VT_ERR_ARG;
  vt_status s = to_device(ctx, ctx->d_nstate, state, size_t(ctx->S.static_verts) * 64);
  if (s != VT_OK) return s;
  ctx->slot = slot;
  ctx->nodes.auto_update = false;   // a caller-supplied state stays until vt_converge or vt_nodes_build
  return write_su(ctx);
}

vt_status vt_trace_rays(vt_ctx* ctx, const float* o4, const float* d4, uint32_t n, uint32_t mask, uint32_t any_hit, uint32_t root,
                        float* out4, float* out_v) {
  if (!ctx || (n && (!o4 || !d4 || !out4))) return VT_ERR_ARG;
  if (root >= ctx->S.node_count) return fail(ctx, VT_ERR_ARG, "trace: root out of range");
  if (!n) return VT_OK;
  const size_t b16 = size_t(n) * 16, b4 = size_t(n) * 4;
  vt_status s = ensure_scratch(ctx, 3 * b16 + b4 + 256);
  if (s != VT_OK) return s;
  char* base = static_cast<char*>(ctx->d_scratch);
  float4 *dO = reinterpret_cast<float4*>(base), *dD = reinterpret_cast<float4*>(base + b16), *dOut = reinterpret_cast<float4*>(base + 2 * b16);
  float* dV = reinterpret_cast<float*>(base + 3 * b16);
  if ((s = to_device(ctx, dO, o4, b16)) != VT_OK) return s;
  if ((s = to_device(ctx, dD, d4, b16)) != VT_OK) return s;
  VT_CK(cudaEventRecord(ctx->ev0, ctx->stream));
  vtk::launch_trace(dev_scene(ctx), dO, dD, n, mask, any_hit, root, dOut, dV, ctx->stream);
  VT_CK(cudaGetLastError());
  VT_CK(cudaEventRecord(ctx->ev1, ctx->stream));
  ctx->tim.launches++;
  if ((s = from_device(ctx, out4, dOut, b16)) != VT_OK) return s;
  if (out_v && (s = from_device(ctx, out_v, dV, b4)) != VT_OK) return s;
  VT_CK(cudaStreamSynchronize(ctx->stream));
  float ms = 0;
  cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
  ctx->tim.trace_ms = ms;
  return VT_OK;
}

vt_status vt_visible(vt_ctx* ctx, uint32_t camera, const double* pts, uint32_t n, double tol, double time, uint8_t* out) {
  if (!ctx || (n && (!pts || !out))) return VT_ERR_ARG;
  if (camera >= ctx->S.cams.size()) return fail(ctx, VT_ERR_UNKNOWN_CAMERA, "unknown camera " + std::to_string(camera));
  if (!n) return VT_OK;
  std::vector<float3> p(n);
  for (uint32_t i = 0; i < n; i++) p[i] = make_float3(float(pts[3 * i]), float(pts[3 * i + 1]), float(pts[3 * i + 2]));
  vt_status s = ensure_scratch(ctx, size_t(n) * 12 + n + 256);
  if (s != VT_OK) return s;
  float3* dp = static_cast<float3*>(ctx->d_scratch);
  uint8_t* dout = reinterpret_cast<uint8_t*>(static_cast<char*>(ctx->d_scratch) + size_t(n) * 12);
  VT_CK(cudaMemcpyAsync(dp, p.data(), size_t(n) * 12, cudaMemcpyHostToDevice, ctx->stream));
  const double* T = ctx->S.cams[camera].T_D_C;
  vtk::launch_visible(dev_scene(ctx), make_float3(float(T[3]), float(T[7]), float(T[11])), dp, n, float(tol), float(time),
                      skip_mask(ctx, camera), dout, ctx->stream);
  VT_CK(cudaGetLastError());
  ctx->tim.launches++;
  VT_CK(cudaMemcpyAsync(out, dout, n, cudaMemcpyDeviceToHost, ctx->stream));
  VT_CK(cudaStreamSynchronize(ctx->stream));
  return VT_OK;
}

vt_status vt_project(vt_ctx* ctx, uint32_t camera, const double* pts, uint32_t n, double* uv) {
  if (!ctx || (n && (!pts || !uv))) return VT_ERR_ARG;
  if (camera >= ctx->S.cams.size()) return fail(ctx, VT_ERR_UNKNOWN_CAMERA, "unknown camera " + std::to_string(camera));
  const vt_camera_desc& c = ctx->S.cams[camera];
  const double* T = c.T_D_C;
  for (uint32_t i = 0; i < n; i++) {
    // camera-frame point R^T (p - c), then KB4 in float64 (gpu/lens.js:43 project)
    const double d[3] = {pts[3 * i] - T[3], pts[3 * i + 1] - T[7], pts[3 * i + 2] - T[11]};
    const double x = T[0] * d[0] + T[4] * d[1] + T[8] * d[2];
    const double y = T[1] * d[0] + T[5] * d[1] + T[9] * d[2];
    const double z = T[2] * d[0] + T[6] * d[1] + T[10] * d[2];
    const double rho = std::hypot(x, y);
    if (rho < 1e-300) { uv[2 * i] = c.cx; uv[2 * i + 1] = c.cy; continue; }
    const double th = std::atan2(rho, z), t2 = th * th;
    const double thd = th * (1 + t2 * (c.k[0] + t2 * (c.k[1] + t2 * (c.k[2] + t2 * c.k[3]))));
    const double s = thd / rho, xd = x * s, yd = y * s;
    uv[2 * i] = c.fx * (xd + c.alpha * yd) + c.cx;
    uv[2 * i + 1] = c.fy * yd + c.cy;
  }
  return VT_OK;
}

// one camera's render; sync = false leaves it queued on the context's stream (vt_render_frame)
static vt_status render_impl(vt_ctx* ctx, const vt_render_req* q, float* out_rgba, bool sync) {
  if (!ctx || !q) return VT_ERR_ARG;
  if (q->camera >= ctx->S.cams.size()) return fail(ctx, VT_ERR_UNKNOWN_CAMERA, "unknown camera " + std::to_string(q->camera));
  if (q->root >= ctx->S.node_count) return fail(ctx, VT_ERR_ARG, "render: root out of range");
  if (q->mode != VT_SHADE_TWIN && q->mode != VT_SHADE_PATH) return fail(ctx, VT_ERR_ARG, "render: unknown mode");
  // gpu/renderer.js:976 renderCamera: _ensureRadiosity first (the twin shading reads the node state; path mode does not)
  if (ctx->nodes.built && ctx->nodes.auto_update && q->mode == VT_SHADE_TWIN) {
    vt_status s = vt_nodes_update(ctx, 0, nullptr);
    if (s != VT_OK) return s;
  }
  const vt_camera_desc& c = ctx->S.cams[q->camera];
  vtk::CamParams cp = make_cam(ctx, q->camera, q->spp, q->light_samples, q->seed, q->options, q->mode, q->max_depth, q->root, q->shutter,
                               q->scale);
  cp.refine = std::min(q->refine, 64u);   // kernels.wgsl.js:224 extra = min(expo.w, 64)
  vtk::CamParams cp2 = make_cam(ctx, q->camera, q->spp, q->refine_light_samples ? q->refine_light_samples : q->light_samples, q->seed,
                                q->options, q->mode, q->max_depth, q->root, q->shutter, q->scale);
  cp2.refine = cp.refine;
  if (q->frame != ctx->frame) { ctx->frame = q->frame; vt_status s = write_su(ctx); if (s != VT_OK) return s; }
  // wave of up to 8 M paths (whole sub-sample indices): ~1.4 GB of path state at one light sample
  const uint32_t n_pix = vtk::tiled_pixels(c.width, c.height, cp.tile_w, cp.tile_h);
  const uint32_t per_wave = std::max(1u, std::min(cp.spp, (8u << 20) / std::max(1u, n_pix)));
  const uint32_t paths = per_wave * n_pix;
  const size_t need = vtk::wave_bytes(paths, std::max(cp.n_light, cp2.n_light), n_pix);
  if (ctx->wave_cap < need) {
    VT_CK(cudaStreamSynchronize(ctx->stream));
    cudaFree(ctx->d_wave);
    ctx->d_wave = nullptr;
    ctx->wave_cap = 0;
    if (cudaMalloc(&ctx->d_wave, need) != cudaSuccess) { cudaGetLastError(); return fail(ctx, VT_ERR_OOM, "wavefront state allocation failed"); }
    ctx->wave_cap = need;
  }
  vtk::WaveBufs wb = vtk::wave_carve(ctx->d_wave, paths, std::max(cp.n_light, cp2.n_light), n_pix, ctx->d_work);
  wb.rcount = ctx->d_work + 12;
  if (q->options & (VT_O_CACHE_WRITE | VT_O_CACHE_READ)) {
    // the cache stays valid while what decides a camera ray's static hit holds (its time does not: the static
    // BVH does not move)
    auto& C = ctx->cams[q->camera];
    std::vector<double> key = {double(q->seed), double(q->root), double(cp.tile_w), double(cp.tile_h), double(n_pix), c.fx, c.fy, c.cx, c.cy,
                               c.alpha, c.k[0], c.k[1], c.k[2], c.k[3]};
    key.insert(key.end(), c.T_D_C, c.T_D_C + 16);
    const uint32_t cap = std::max(1u, std::min(cp.spp, 64u) + cp.refine);
    if (key != C.hc_key || cap > C.hc_cap) {
      VT_CK(cudaStreamSynchronize(ctx->stream));
      cudaFree(C.hcache);
      cudaFree(C.scache);
      C.hcache = nullptr;
      C.scache = nullptr;
      C.hc_cap = 0;
      C.hc_key.clear();
      C.sc_key.clear();
      if (cudaMalloc(&C.hcache, size_t(n_pix) * cap * 16) != cudaSuccess) { cudaGetLastError(); C.hcache = nullptr; }
      else {
        VT_CK(cudaMemsetAsync(C.hcache, 0, size_t(n_pix) * cap * 16, ctx->stream));
        C.hc_cap = cap;
        C.hc_stride = n_pix;
        C.hc_key = key;
      }
    }
    if (C.hcache) { wb.hcache = C.hcache; wb.hc_stride = C.hc_stride; wb.hc_cap = C.hc_cap; }
    // the static-occlusion cache (twin shading of static first hits): also keyed on the emitter body's pose over the
    // exposure and both passes' light-sample counts (gpu/renderer.js:952-956)
    if (C.hcache && (q->options & VT_O_SHADOW_CACHE) && q->mode == VT_SHADE_TWIN) {
      std::vector<double> sk = C.hc_key;
      sk.push_back(double(cp.n_light));
      sk.push_back(double(cp2.n_light));
      sk.push_back(double(C.hc_cap));
      const int sc = ctx->S.scope_index;
      if (sc >= 0 && size_t(sc) < ctx->inst.size() && ctx->inst[sc].valid) {
        const vt::InstPose& I = ctx->inst[sc];
        sk.insert(sk.end(), I.q0, I.q0 + 4); sk.insert(sk.end(), I.q1, I.q1 + 4);
        sk.insert(sk.end(), I.p0, I.p0 + 3); sk.insert(sk.end(), I.p1, I.p1 + 3);
      }
      if (!C.scache || sk != C.sc_key) {
        if (!C.scache && cudaMalloc(&C.scache, size_t(C.hc_stride) * C.hc_cap * 4) != cudaSuccess) { cudaGetLastError(); C.scache = nullptr; }
        if (C.scache) VT_CK(cudaMemsetAsync(C.scache, 0, size_t(C.hc_stride) * C.hc_cap * 4, ctx->stream));
        C.sc_key = C.scache ? sk : std::vector<double>();
      }
      if (C.scache) wb.scache = C.scache;
    }
  }
  vtk::KernelTimer timer{ctx->kev.data(), ctx->kkind.data(), int(ctx->kev.size() / 2), 0};
  if (ctx->kprof) wb.stats = reinterpret_cast<unsigned long long*>(ctx->d_work + 16);
  VT_CK(cudaEventRecord(ctx->ev0, ctx->stream));
  vtk::wave_render(dev_scene(ctx), cp, wb, paths, ctx->cams[q->camera].radiance, ctx->wave_blocks, ctx->stream, &ctx->tim.launches,
                   ctx->kprof ? &timer : nullptr, &cp2);
  VT_CK(cudaGetLastError());
  VT_CK(cudaEventRecord(ctx->ev1, ctx->stream));
  ctx->cams[q->camera].rendered = true;
  if (!sync) return VT_OK;
  if (out_rgba) {
    vt_status s = from_device(ctx, out_rgba, ctx->cams[q->camera].radiance, size_t(c.width) * c.height * 16);
    if (s != VT_OK) return s;
  }
  VT_CK(cudaStreamSynchronize(ctx->stream));
  float ms = 0;
  cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
  ctx->tim.render_ms = ms;
  if (ctx->kprof) {
    for (int i = 0; i < timer.n; i++) {
      float k = 0;
      cudaEventElapsedTime(&k, ctx->kev[2 * i], ctx->kev[2 * i + 1]);
      if (ctx->kkind[i] == 0) { ctx->tim.extend_ms += k; ctx->tim.extend_launches++; }
      else if (ctx->kkind[i] == 1) ctx->tim.shade_ms += k;
      else { ctx->tim.shadow_ms += k; ctx->tim.shadow_launches++; }
    }
    unsigned long long st[2];
    VT_CK(cudaMemcpy(st, ctx->d_work + 16, 16, cudaMemcpyDeviceToHost));
    ctx->tim.extend_rays = st[0];
    ctx->tim.shadow_paths = st[1];
  }
  return VT_OK;
}

vt_status vt_render_camera(vt_ctx* ctx, const vt_render_req* q, float* out_rgba) { return render_impl(ctx, q, out_rgba, true); }

vt_status vt_kernel_profile(vt_ctx* ctx, int enable, int reset) {
  if (!ctx) return VT_ERR_ARG;
  if (enable && ctx->kev.empty()) {
    ctx->kev.resize(2 * 3 * 256);
    ctx->kkind.resize(3 * 256);
    for (auto& e : ctx->kev) VT_CK(cudaEventCreate(&e));
  }
  ctx->kprof = enable != 0;
  if (reset) {
    ctx->tim.extend_ms = ctx->tim.shade_ms = ctx->tim.shadow_ms = 0;
    ctx->tim.extend_launches = ctx->tim.shadow_launches = ctx->tim.extend_rays = ctx->tim.shadow_paths = 0;
    VT_CK(cudaMemsetAsync(ctx->d_work + 16, 0, 16, ctx->stream));
    VT_CK(cudaStreamSynchronize(ctx->stream));
  }
  return VT_OK;
}

vt_status vt_readback(vt_ctx* ctx, uint32_t camera, uint32_t kind, void* out, size_t bytes) {
  if (!ctx || !out) return VT_ERR_ARG;
  if (camera >= ctx->S.cams.size()) return fail(ctx, VT_ERR_UNKNOWN_CAMERA, "unknown camera " + std::to_string(camera));
  const size_t px = size_t(ctx->S.cams[camera].width) * ctx->S.cams[camera].height;
  const auto& C = ctx->cams[camera];
  if (kind == VT_READ_LINEAR) {
    if (!C.rendered) return fail(ctx, VT_ERR_STATE, "readback before renderCamera");
    if (bytes < px * 16) return VT_ERR_ARG;
    vt_status s = from_device(ctx, out, C.radiance, px * 16);
    if (s != VT_OK) return s;
  } else if (kind == VT_READ_RAW) {
    if (!C.exposed) return fail(ctx, VT_ERR_STATE, "raw readback before sensor");
    if (bytes < px * 4) return VT_ERR_ARG;
    vt_status s = from_device(ctx, out, C.raw, px * 4);
    if (s != VT_OK) return s;
  } else if (kind == VT_READ_RGBA8 || kind == VT_READ_RGB8 || kind == VT_READ_YUV420) {
    if (!C.processed) return fail(ctx, VT_ERR_STATE, "8-bit readback before vt_sensor_frame");
    const uint32_t W = ctx->S.cams[camera].width, H = ctx->S.cams[camera].height;
    if (kind == VT_READ_RGBA8) {
      if (bytes < px * 4) return VT_ERR_ARG;
      vt_status s = from_device(ctx, out, C.isp.out, px * 4);
      if (s != VT_OK) return s;
    } else if (kind == VT_READ_YUV420) {
      const size_t n = px + 2 * size_t((W + 1) / 2) * ((H + 1) / 2);
      if (bytes < n) return VT_ERR_ARG;
      vt_status s = from_device(ctx, out, C.isp.yuv, n);
      if (s != VT_OK) return s;
    } else {
      if (bytes < px * 3) return VT_ERR_ARG;
      std::vector<uint8_t> rgba(px * 4);
      VT_CK(cudaMemcpyAsync(rgba.data(), C.isp.out, px * 4, cudaMemcpyDeviceToHost, ctx->stream));
      VT_CK(cudaStreamSynchronize(ctx->stream));
      uint8_t* o = static_cast<uint8_t*>(out);
      for (size_t i = 0; i < px; i++) { o[3 * i] = rgba[4 * i]; o[3 * i + 1] = rgba[4 * i + 1]; o[3 * i + 2] = rgba[4 * i + 2]; }
    }
  } else {
    return fail(ctx, VT_ERR_ARG, "readback kind");
  }
  VT_CK(cudaStreamSynchronize(ctx->stream));
  return VT_OK;
}

vt_status vt_sensor_expose(vt_ctx* ctx, const vt_sensor_uniform* su, const float* irradiance, float* raw) {
  if (!ctx || !su || !irradiance || !raw) return VT_ERR_ARG;
  const uint32_t W = su->words[0], H = su->words[1];
  float glare;
  std::memcpy(&glare, &su->words[52], 4);
  if (!W || !H) return fail(ctx, VT_ERR_ARG, "sensor: empty image");
  if (glare != 0.0f) return fail(ctx, VT_ERR_ARG, "sensor: veiling glare is not supported by the expose stage (fraction must be 0)");
  const size_t px = size_t(W) * H;
  vt_status s = reject_foreign(ctx, {irradiance, raw});
  if (s != VT_OK) return s;
  // a device irradiance is read as float4: one that is not 16-byte aligned is copied like a host one
  const bool din = is_device_ptr(irradiance) && aligned16(irradiance), dout = is_device_ptr(raw);
  s = ensure_scratch(ctx, (din ? 0 : px * 16) + (dout ? 0 : px * 4) + 256);
  if (s != VT_OK) return s;
  const float4* dE = reinterpret_cast<const float4*>(irradiance);
  char* base = static_cast<char*>(ctx->d_scratch);
  if (!din) { if ((s = to_device(ctx, base, irradiance, px * 16)) != VT_OK) return s; dE = reinterpret_cast<float4*>(base); base += px * 16; }
  float* dR = dout ? raw : reinterpret_cast<float*>(base);
  vtk::SensorParams sp;
  std::memcpy(sp.w, su->words, sizeof(sp.w));
  VT_CK(cudaEventRecord(ctx->ev0, ctx->stream));
  vtk::launch_sensor_expose(sp, dE, 1.0f, dR, ctx->stream);
  VT_CK(cudaGetLastError());
  VT_CK(cudaEventRecord(ctx->ev1, ctx->stream));
  ctx->tim.launches++;
  if (!dout) VT_CK(cudaMemcpyAsync(raw, dR, px * 4, cudaMemcpyDeviceToHost, ctx->stream));
  VT_CK(cudaStreamSynchronize(ctx->stream));
  float ms = 0;
  cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
  ctx->tim.sensor_ms = ms;
  return VT_OK;
}

vt_status vt_sensor_camera(vt_ctx* ctx, uint32_t camera, const vt_sensor_uniform* su, float optics_scale) {
  if (!ctx || !su) return VT_ERR_ARG;
  if (camera >= ctx->S.cams.size()) return fail(ctx, VT_ERR_UNKNOWN_CAMERA, "unknown camera " + std::to_string(camera));
  auto& C = ctx->cams[camera];
  if (!C.rendered) return fail(ctx, VT_ERR_STATE, "sensor before renderCamera");
  if (su->words[0] != ctx->S.cams[camera].width || su->words[1] != ctx->S.cams[camera].height) return fail(ctx, VT_ERR_ARG, "sensor: size mismatch");
  float glare;
  std::memcpy(&glare, &su->words[52], 4);
  if (glare != 0.0f) return fail(ctx, VT_ERR_ARG, "sensor: veiling glare is not supported by the expose stage (fraction must be 0)");
  vtk::SensorParams sp;
  std::memcpy(sp.w, su->words, sizeof(sp.w));
  VT_CK(cudaEventRecord(ctx->ev0, ctx->stream));
  vtk::launch_sensor_expose(sp, C.radiance, optics_scale, C.raw, ctx->stream);
  VT_CK(cudaGetLastError());
  VT_CK(cudaEventRecord(ctx->ev1, ctx->stream));
  ctx->tim.launches++;
  C.exposed = true;
  VT_CK(cudaStreamSynchronize(ctx->stream));
  float ms = 0;
  cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
  ctx->tim.sensor_ms = ms;
  return VT_OK;
}

static vt_status sensor_impl(vt_ctx* ctx, uint32_t camera, const vt_sensor_uniform* su, uint32_t* stats, bool sync);

vt_status vt_sensor_frame(vt_ctx* ctx, uint32_t camera, const vt_sensor_uniform* su, uint32_t stats[4]) {
  return sensor_impl(ctx, camera, su, stats, true);
}

vt_status vt_render_frame(vt_ctx* ctx, vt_frame_req* f) {
  if (!ctx || !f || !f->cameras || !f->n_cameras) return VT_ERR_ARG;
  for (uint32_t k = 0; k < f->n_cameras; k++)
    if (f->cameras[k] >= ctx->S.cams.size()) return fail(ctx, VT_ERR_UNKNOWN_CAMERA, "unknown camera " + std::to_string(f->cameras[k]));
  if (f->stats && f->sensors) {   // pinned host words for the statistics copies that stay queued until the end
    const size_t need = size_t(f->n_cameras) * 16;
    if (ctx->h_stats_bytes < need) {
      if (ctx->h_stats) cudaFreeHost(ctx->h_stats);
      ctx->h_stats = nullptr;
      ctx->h_stats_bytes = 0;
      if (cudaMallocHost(&ctx->h_stats, need) != cudaSuccess) { cudaGetLastError(); return fail(ctx, VT_ERR_OOM, "frame: pinned statistics"); }
      ctx->h_stats_bytes = need;
    }
  }
  VT_CK(cudaEventRecord(ctx->ev2, ctx->stream));
  for (uint32_t k = 0; k < f->n_cameras; k++) {
    vt_render_req q = f->render;
    q.camera = f->cameras[k];
    vt_status s = render_impl(ctx, &q, nullptr, false);
    if (s != VT_OK) return s;
  }
  if (f->sensors)
    for (uint32_t k = 0; k < f->n_cameras; k++) {
      vt_status s = sensor_impl(ctx, f->cameras[k], &f->sensors[k], f->stats ? static_cast<uint32_t*>(ctx->h_stats) + 4 * k : nullptr, false);
      if (s != VT_OK) return s;
    }
  VT_CK(cudaEventRecord(ctx->ev3, ctx->stream));
  VT_CK(cudaStreamSynchronize(ctx->stream));
  float ms = 0;
  cudaEventElapsedTime(&ms, ctx->ev2, ctx->ev3);
  f->ms = ms;
  if (f->stats && f->sensors) std::memcpy(f->stats, ctx->h_stats, size_t(f->n_cameras) * 16);
  return VT_OK;
}

vt_status vt_set_relative_illumination(vt_ctx* ctx, uint32_t camera, const float* ri, double pupil_exponent, const double* vig_theta_deg,
                                       const double* vig, uint32_t n_vig) {
  if (!ctx) return VT_ERR_ARG;
  if (camera >= ctx->S.cams.size()) return fail(ctx, VT_ERR_UNKNOWN_CAMERA, "unknown camera " + std::to_string(camera));
  if (n_vig && (!vig_theta_deg || !vig)) return fail(ctx, VT_ERR_ARG, "relative illumination: vignetting table is null");
  const vt_camera_desc& c = ctx->S.cams[camera];
  const size_t px = size_t(c.width) * c.height;
  auto& C = ctx->cams[camera];
  if (!C.ri && cudaMalloc(&C.ri, px * 4) != cudaSuccess) { cudaGetLastError(); C.ri = nullptr; return fail(ctx, VT_ERR_OOM, "relative illumination map"); }
  if (ri) return to_device(ctx, C.ri, ri, px * 4);
  std::vector<float> m(px);
  vt::relative_illumination(c, pupil_exponent, vig_theta_deg, vig, n_vig, m.data());
  VT_CK(cudaMemcpyAsync(C.ri, m.data(), px * 4, cudaMemcpyHostToDevice, ctx->stream));
  VT_CK(cudaStreamSynchronize(ctx->stream));
  return VT_OK;
}

vt_status vt_get_relative_illumination(vt_ctx* ctx, uint32_t camera, float* ri) {
  if (!ctx || !ri) return VT_ERR_ARG;
  if (camera >= ctx->S.cams.size()) return fail(ctx, VT_ERR_UNKNOWN_CAMERA, "unknown camera " + std::to_string(camera));
  const auto& C = ctx->cams[camera];
  if (!C.ri) return fail(ctx, VT_ERR_STATE, "no relative illumination map (vt_set_relative_illumination)");
  vt_status s = from_device(ctx, ri, C.ri, size_t(ctx->S.cams[camera].width) * ctx->S.cams[camera].height * 4);
  if (s != VT_OK) return s;
  VT_CK(cudaStreamSynchronize(ctx->stream));
  return VT_OK;
}

// the sensor chain of one camera; sync = false queues it and an asynchronous copy of its statistics into stats_async
static vt_status sensor_impl(vt_ctx* ctx, uint32_t camera, const vt_sensor_uniform* su, uint32_t* stats, bool sync) {
  if (!ctx || !su) return VT_ERR_ARG;
  if (camera >= ctx->S.cams.size()) return fail(ctx, VT_ERR_UNKNOWN_CAMERA, "unknown camera " + std::to_string(camera));
  auto& C = ctx->cams[camera];
  if (!C.rendered) return fail(ctx, VT_ERR_STATE, "sensor before renderCamera");
  const vt_camera_desc& cd = ctx->S.cams[camera];
  const uint32_t W = cd.width, H = cd.height;
  if (su->words[0] != W || su->words[1] != H) return fail(ctx, VT_ERR_ARG, "sensor: size mismatch");
  float F;
  std::memcpy(&F, &su->words[54], 4);
  if (!(F >= 1.0f && F <= 4096.0f)) return fail(ctx, VT_ERR_ARG, "sensor: glare level factor out of range");
  if (!C.ri) {   // gpu/sensor.js defaults: pupil obliquity exponent 1, no vignetting
    const double vt[2] = {0.0, 90.0}, vv[2] = {1.0, 1.0};
    vt_status s = vt_set_relative_illumination(ctx, camera, nullptr, 1.0, vt, vv, 2);
    if (s != VT_OK) return s;
  }
  const size_t Fi = size_t(F), lev = ((W + Fi - 1) / Fi) * ((H + Fi - 1) / Fi);
  if (C.isp_mem && lev > C.isp_lev) {   // a finer glare level than the buffers hold: size them again
    VT_CK(cudaStreamSynchronize(ctx->stream));
    cudaFree(C.isp_mem);
    C.isp_mem = nullptr;
    C.processed = false;
  }
  if (!C.isp_mem) {
    const size_t px = size_t(W) * H;
    auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
    const size_t b4 = al(px * 16), bl = al(std::max<size_t>(lev, 1) * 16), bo = al(px * 4),
                 by = al(px + 2 * size_t((W + 1) / 2) * ((H + 1) / 2)), bs = 256;
    if (cudaMalloc(&C.isp_mem, 2 * b4 + 2 * bl + bo + by + bs) != cudaSuccess) {
      cudaGetLastError();
      C.isp_mem = nullptr;
      return fail(ctx, VT_ERR_OOM, "sensor chain buffers");
    }
    char* p = static_cast<char*>(C.isp_mem);
    C.isp.A = reinterpret_cast<float4*>(p); p += b4;
    C.isp.B = reinterpret_cast<float4*>(p); p += b4;
    C.isp.GA = reinterpret_cast<float4*>(p); p += bl;
    C.isp.GB = reinterpret_cast<float4*>(p); p += bl;
    C.isp.out = reinterpret_cast<uchar4*>(p); p += bo;
    C.isp.yuv = reinterpret_cast<uint8_t*>(p); p += by;
    C.isp.stats = reinterpret_cast<uint32_t*>(p);
    C.isp_lev = std::max<size_t>(lev, 1);
  }
  C.isp.L = C.radiance;
  C.isp.ri = C.ri;
  C.isp.raw = C.raw;
  vtk::SensorParams sp;
  std::memcpy(sp.w, su->words, sizeof(sp.w));
  VT_CK(cudaEventRecord(ctx->ev0, ctx->stream));
  const int isp_launches = vtk::launch_isp(sp, C.isp, ctx->stream);
  VT_CK(cudaGetLastError());
  VT_CK(cudaEventRecord(ctx->ev1, ctx->stream));
  if (!sync) {
    if (stats) VT_CK(cudaMemcpyAsync(stats, C.isp.stats, 16, cudaMemcpyDeviceToHost, ctx->stream));
    ctx->tim.launches += isp_launches;
    C.exposed = C.processed = true;
    return VT_OK;
  }
  uint32_t st[4];
  VT_CK(cudaMemcpyAsync(st, C.isp.stats, 16, cudaMemcpyDeviceToHost, ctx->stream));
  VT_CK(cudaStreamSynchronize(ctx->stream));
  if (stats) std::memcpy(stats, st, 16);
  float ms = 0;
  cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
  ctx->tim.sensor_ms = ms;
  ctx->tim.launches += isp_launches;
  C.exposed = C.processed = true;
  return VT_OK;
}

vt_status vt_form_factors(vt_ctx* ctx, uint32_t n, const float* centres, const float* normals, const float* areas, float* F) {
  if (!ctx || !n || !centres || !normals || !areas || !F) return VT_ERR_ARG;
  const size_t nn = size_t(n) * n * 4;
  vt_status s = reject_foreign(ctx, {F});
  if (s != VT_OK) return s;
  const bool dF = is_device_ptr(F);
  s = ensure_scratch(ctx, size_t(n) * 28 + (dF ? 0 : nn) + 256);
  if (s != VT_OK) return s;
  char* base = static_cast<char*>(ctx->d_scratch);
  float *dC = reinterpret_cast<float*>(base), *dN = dC + 3 * size_t(n), *dA = dN + 3 * size_t(n);
  if ((s = to_device(ctx, dC, centres, size_t(n) * 12)) != VT_OK) return s;
  if ((s = to_device(ctx, dN, normals, size_t(n) * 12)) != VT_OK) return s;
  if ((s = to_device(ctx, dA, areas, size_t(n) * 4)) != VT_OK) return s;
  float* dOut = dF ? F : reinterpret_cast<float*>(base + ((size_t(n) * 28 + 255) / 256) * 256);
  vtk::launch_form_factors(n, dC, dN, dA, dOut, ctx->stream);
  VT_CK(cudaGetLastError());
  ctx->tim.launches++;
  if (!dF) VT_CK(cudaMemcpyAsync(F, dOut, nn, cudaMemcpyDeviceToHost, ctx->stream));
  VT_CK(cudaStreamSynchronize(ctx->stream));
  return VT_OK;
}

vt_status vt_form_factors_visible(vt_ctx* ctx, uint32_t n, const float* centres, const float* normals, const float* areas, uint32_t rays,
                                  float* F) {
  if (!ctx || !n || !centres || !normals || !areas || !F) return VT_ERR_ARG;
  if (n > 65535 || rays < 1 || rays > 255) return fail(ctx, VT_ERR_ARG, "form factors: n <= 65535 and 1..255 rays per pair");
  const size_t nn = size_t(n) * n * 4;
  vt_status s = reject_foreign(ctx, {F});
  if (s != VT_OK) return s;
  const bool dF = is_device_ptr(F);
  const size_t head = (size_t(n) * 28 + 255) / 256 * 256, cnt = head + 256, out = cnt + (size_t(n) * n + 255) / 256 * 256;
  s = ensure_scratch(ctx, out + (dF ? 0 : nn) + 256);
  if (s != VT_OK) return s;
  char* base = static_cast<char*>(ctx->d_scratch);
  float *dC = reinterpret_cast<float*>(base), *dN = dC + 3 * size_t(n), *dA = dN + 3 * size_t(n);
  if ((s = to_device(ctx, dC, centres, size_t(n) * 12)) != VT_OK) return s;
  if ((s = to_device(ctx, dN, normals, size_t(n) * 12)) != VT_OK) return s;
  if ((s = to_device(ctx, dA, areas, size_t(n) * 4)) != VT_OK) return s;
  float* dOut = dF ? F : reinterpret_cast<float*>(base + out);
  VT_CK(cudaEventRecord(ctx->ev0, ctx->stream));
  vtk::launch_form_factors_visible(dev_scene(ctx), n, dC, dN, dA, rays, reinterpret_cast<uint32_t*>(base + head), reinterpret_cast<uint8_t*>(base + cnt),
                                   dOut, ctx->wave_blocks, ctx->stream);
  VT_CK(cudaGetLastError());
  VT_CK(cudaEventRecord(ctx->ev1, ctx->stream));
  ctx->tim.launches += 2;
  if (!dF) VT_CK(cudaMemcpyAsync(F, dOut, nn, cudaMemcpyDeviceToHost, ctx->stream));
  VT_CK(cudaStreamSynchronize(ctx->stream));
  float ms = 0;
  cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
  ctx->tim.trace_ms = ms;
  return VT_OK;
}

vt_status vt_debug_flags(vt_ctx* ctx, uint32_t out[16], int reset) {
  if (!ctx || !out) return VT_ERR_ARG;
  VT_CK(cudaMemcpyAsync(out, ctx->d_dbg, 64, cudaMemcpyDeviceToHost, ctx->stream));
  if (reset) VT_CK(cudaMemsetAsync(ctx->d_dbg, 0, 64, ctx->stream));
  VT_CK(cudaStreamSynchronize(ctx->stream));
  return VT_OK;
}

vt_status vt_wait_check(vt_ctx* ctx, uint64_t cycles, int arrive) {
  if (!ctx || cycles == 0 || cycles > (1ull << 36)) return VT_ERR_ARG;
  uint32_t* err = ctx->d_work + 32;
  VT_CK(cudaMemsetAsync(err, 0, 4, ctx->stream));
  vtk::launch_wait_check(cycles, arrive ? 1u : 0u, err, ctx->stream);
  VT_CK(cudaGetLastError());
  uint32_t e = 0;
  VT_CK(cudaMemcpyAsync(&e, err, 4, cudaMemcpyDeviceToHost, ctx->stream));
  VT_CK(cudaStreamSynchronize(ctx->stream));
  return e ? fail(ctx, VT_ERR_TIMEOUT, "wait check: the barrier phase did not complete within the limit") : VT_OK;
}

vt_status vt_timings_get(const vt_ctx* ctx, vt_timings* out) {
  if (!ctx || !out) return VT_ERR_ARG;
  *out = ctx->tim;
  // the node radiosity's last direct-light and Jacobi calls (events on the context's stream)
  float ms = 0;
  if (ctx->nodes.timed_direct && cudaEventSynchronize(ctx->nev[1]) == cudaSuccess && cudaEventElapsedTime(&ms, ctx->nev[0], ctx->nev[1]) == cudaSuccess)
    out->node_direct_ms = ms;
  if (ctx->nodes.timed_jacobi && cudaEventSynchronize(ctx->nev[3]) == cudaSuccess && cudaEventElapsedTime(&ms, ctx->nev[2], ctx->nev[3]) == cudaSuccess)
    out->node_jacobi_ms = ms;
  out->node_jacobi_steps = ctx->nodes.last_steps;
  return VT_OK;
}

}  // extern "C"

// ------------------------------------------------------------------------------------------------ mixed precision
// Iterative refinement (outer, accurate) around low-precision Jacobi (inner, tensor cores):
//   r = E + rho F B - B            F = F_hi + F_lo and B = B_hi + B_lo in bf16, three tcgen05 products, FP64 epilogue
//   d <- r + rho F_lp d            BF16 or FP8 (per-row / per-column scales) sweeps until the update stalls
//   B <- B + d
// Splits of K are chosen so the grid of 128-row tiles x splits fills whole waves of the SMs.
namespace {
uint32_t choose_splits(uint32_t mtiles, uint32_t ktiles, int sms) {
  uint32_t best = 1;
  double best_eff = 0;
  for (uint32_t s = 1; s <= 8 && s <= ktiles; s++) {
    const double ctas = double(mtiles) * s, waves = std::ceil(ctas / sms);
    const double eff = ctas / (waves * sms);
    if (eff > best_eff + 0.02) { best_eff = eff; best = s; }
  }
  return best;
}
}  // namespace

static vt_status tc_solve(vt_ctx* ctx, vt_solve_req* q) {
  const uint32_t n = q->n, R = q->n_rhs;
  if (n % 16) return fail(ctx, VT_ERR_ARG, "solve: BF16/FP8 need n % 16 == 0");
  const bool fp8 = q->precision == VT_PREC_FP8;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
  const uint32_t mtiles = (n + 127) / 128;
  const uint32_t kt_bf = (n + 63) / 64, kt_q = (n + 127) / 128;
  const uint32_t sp_bf = choose_splits(mtiles, kt_bf, sms), sp_q = choose_splits(mtiles, kt_q, sms);
  const uint32_t sp_max = std::max(sp_bf, sp_q);
  const size_t nn = size_t(n) * n, nr = size_t(n) * R;
  const bool dF = is_device_ptr(q->F);
  // layout of the context's mixed-precision block (each piece 256-byte aligned)
  size_t off = 0;
  auto place = [&](size_t bytes) { const size_t o = off; off += (bytes + 255) / 256 * 256; return o; };
  const size_t o_f32 = dF ? 0 : place(nn * 4), o_hi = place(nn * 2), o_lo = place(nn * 2), o_q = fp8 ? place(nn) : 0;
  const size_t o_rs = place(size_t(n) * 4), o_bhi = place(size_t(64) * n * 2), o_blo = place(size_t(64) * n * 2),
               o_bq = place(size_t(64) * n), o_cs = place(256), o_cm = place(256), o_part = place(size_t(sp_max) * n * 64 * 4),
               o_E = place(nr * 4), o_rho = place(size_t(n) * 4), o_B = place(nr * 4), o_r = place(nr * 4), o_d = place(nr * 4),
               o_d2 = place(nr * 4), o_np = place((nr / 256 + 2) * 16), o_err = place(64);
  auto& T = ctx->tc;
  const bool same_f = q->reuse_f && T.f_src == q->F && T.n == n && T.mem;
  if (T.bytes < off) {
    VT_CK(cudaStreamSynchronize(ctx->stream));
    cudaFree(T.mem);
    T = vt_ctx::Tc{};
    if (cudaMalloc(&T.mem, off) != cudaSuccess) { cudaGetLastError(); return fail(ctx, VT_ERR_OOM, "solve: mixed-precision buffers"); }
    T.bytes = off;
  }
  char* m = static_cast<char*>(T.mem);
  const float* F32 = dF ? q->F : reinterpret_cast<float*>(m + o_f32);
  uint16_t* Fhi = reinterpret_cast<uint16_t*>(m + o_hi);
  uint16_t* Flo = reinterpret_cast<uint16_t*>(m + o_lo);
  uint8_t* Fq = fp8 ? reinterpret_cast<uint8_t*>(m + o_q) : nullptr;
  float* rs = reinterpret_cast<float*>(m + o_rs);
  uint16_t* Bhi = reinterpret_cast<uint16_t*>(m + o_bhi);
  uint16_t* Blo = reinterpret_cast<uint16_t*>(m + o_blo);
  uint8_t* Bq = reinterpret_cast<uint8_t*>(m + o_bq);
  float* cs = reinterpret_cast<float*>(m + o_cs);
  uint32_t* cm = reinterpret_cast<uint32_t*>(m + o_cm);
  float* part = reinterpret_cast<float*>(m + o_part);
  float* E = reinterpret_cast<float*>(m + o_E);
  float* rho = reinterpret_cast<float*>(m + o_rho);
  float* B = reinterpret_cast<float*>(m + o_B);
  float* r = reinterpret_cast<float*>(m + o_r);
  float* d = reinterpret_cast<float*>(m + o_d);
  float* d2 = reinterpret_cast<float*>(m + o_d2);
  double* np = reinterpret_cast<double*>(m + o_np);
  uint32_t* err = reinterpret_cast<uint32_t*>(m + o_err);
  double* norms = reinterpret_cast<double*>(m + o_err + 16);
  vt_status s;
  float conv_ms = 0;
  VT_CK(cudaEventRecord(ctx->ev0, ctx->stream));
  if (!(same_f && T.have_hi_lo && (!fp8 || T.have_q))) {
    if (!dF && (s = to_device(ctx, const_cast<float*>(F32), q->F, nn * 4)) != VT_OK) return s;
    vtk::tc_split_bf16(F32, Fhi, Flo, nn, ctx->stream);
    if (fp8) vtk::tc_quant_rows_fp8(F32, Fq, rs, n, ctx->stream);
    VT_CK(cudaGetLastError());
    T.f_src = q->F; T.n = n; T.have_hi_lo = true; T.have_q = fp8;
  }
  VT_CK(cudaEventRecord(ctx->ev1, ctx->stream));
  VT_CK(cudaEventSynchronize(ctx->ev1));
  cudaEventElapsedTime(&conv_ms, ctx->ev0, ctx->ev1);
  vtk::TcMap mhi, mlo, mq, mbhi, mblo, mbq;
  int code = 0;
  if (!vtk::tc_encode(&mhi, Fhi, n, n, 2, 128, &code) || !vtk::tc_encode(&mlo, Flo, n, n, 2, 128, &code) ||
      !vtk::tc_encode(&mbhi, Bhi, n, 64, 2, 64, &code) || !vtk::tc_encode(&mblo, Blo, n, 64, 2, 64, &code) ||
      (fp8 && (!vtk::tc_encode(&mq, Fq, n, n, 1, 128, &code) || !vtk::tc_encode(&mbq, Bq, n, 64, 1, 64, &code))))
    return fail(ctx, VT_ERR_CUDA, "solve: tensor map encoding failed (" + std::to_string(code) + ")");
  if ((s = to_device(ctx, E, q->E, nr * 4)) != VT_OK) return s;
  if ((s = to_device(ctx, rho, q->rho, size_t(n) * 4)) != VT_OK) return s;
  if (q->warm_start) { if ((s = to_device(ctx, B, q->B, nr * 4)) != VT_OK) return s; }
  else VT_CK(cudaMemcpyAsync(B, E, nr * 4, cudaMemcpyDeviceToDevice, ctx->stream));
  VT_CK(cudaMemsetAsync(err, 0, 64, ctx->stream));
  const uint32_t max_it = q->max_iters ? q->max_iters : 1000;
  const double inner_tol = fp8 ? 2e-3 : 1e-3;
  const uint32_t inner_max = 24;
  uint32_t sweeps = 0, refinements = 0, npart = 0;
  double resid = INFINITY, gemm_ms = 0;
  auto read_norms = [&](double* h) -> vt_status {
    vtk::launch_reduce_partials(np, npart, norms, ctx->stream);
    VT_CK(cudaGetLastError());
    VT_CK(cudaMemcpyAsync(h, norms, 16, cudaMemcpyDeviceToHost, ctx->stream));
    VT_CK(cudaStreamSynchronize(ctx->stream));
    return VT_OK;
  };
  VT_CK(cudaEventRecord(ctx->ev0, ctx->stream));
  double last_rate = 0.0;   // the sweeps' rate of change in the previous correction (the same matrix)
  for (;;) {
    // accurate residual of the current iterate
    vtk::tc_pack_b(vtk::TC_BF16X3, B, n, R, Bhi, Blo, nullptr, nullptr, nullptr, ctx->stream);
    vtk::tc_gemm(vtk::TC_BF16X3, &mhi, &mlo, &mbhi, &mblo, n, sp_bf, (kt_bf + sp_bf - 1) / sp_bf, part, err, ctx->stream);
    vtk::tc_combine_residual(part, sp_bf, n, R, rho, E, B, r, np, &npart, ctx->stream);
    ctx->tim.launches += 3;
    double h[2];
    if ((s = read_norms(h)) != VT_OK) return s;
    refinements++;
    resid = h[1] > 0 ? std::sqrt(h[0] / h[1]) : 0.0;
    if (resid <= q->tol || sweeps >= max_it) break;
    // correction: (I - diag(rho) F_lp) d = r by Jacobi sweeps from d = r, to the accuracy the next residual needs to
    // fall under tol with a margin of 4 (an inexact correction), never finer than the low precision's floor
    const double inner_goal = std::min(0.1, std::max(inner_tol, 0.25 * q->tol / resid));
    VT_CK(cudaMemcpyAsync(d, r, nr * 4, cudaMemcpyDeviceToDevice, ctx->stream));
    // The sweeps' relative change falls geometrically. Each host check costs a stream synchronisation, about as
    // much as a sweep at small n, so the observed rate (from two checked sweeps, or the previous correction's)
    // predicts how many more sweeps reach the goal; they run back to back and one check follows (then one per
    // sweep, should the prediction fall short).
    uint32_t batch = 1, in_batch = 0, k_prev = 0;
    double c_prev = -1.0;
    for (uint32_t k = 0; k < inner_max && sweeps < max_it; k++) {
      if (fp8) {
        vtk::tc_pack_b(vtk::TC_FP8, d, n, R, nullptr, nullptr, Bq, cs, cm, ctx->stream);
        VT_CK(cudaEventRecord(ctx->ev2, ctx->stream));
        vtk::tc_gemm(vtk::TC_FP8, &mq, nullptr, &mbq, nullptr, n, sp_q, (kt_q + sp_q - 1) / sp_q, part, err, ctx->stream);
        VT_CK(cudaEventRecord(ctx->ev3, ctx->stream));
        vtk::tc_combine_sweep(part, sp_q, n, R, rho, r, d, d2, rs, cs, np, &npart, ctx->stream);
      } else {
        vtk::tc_pack_b(vtk::TC_BF16, d, n, R, Bhi, nullptr, nullptr, nullptr, nullptr, ctx->stream);
        VT_CK(cudaEventRecord(ctx->ev2, ctx->stream));
        vtk::tc_gemm(vtk::TC_BF16, &mhi, nullptr, &mbhi, nullptr, n, sp_bf, (kt_bf + sp_bf - 1) / sp_bf, part, err, ctx->stream);
        VT_CK(cudaEventRecord(ctx->ev3, ctx->stream));
        vtk::tc_combine_sweep(part, sp_bf, n, R, rho, r, d, d2, nullptr, nullptr, np, &npart, ctx->stream);
      }
      ctx->tim.launches += 3;
      std::swap(d, d2);
      sweeps++;
      if (++in_batch < batch && k + 1 < inner_max && sweeps < max_it) continue;
      if ((s = read_norms(h)) != VT_OK) return s;
      float gms = 0;
      cudaEventElapsedTime(&gms, ctx->ev2, ctx->ev3);
      gemm_ms += gms * float(in_batch);
      const double c = h[1] > 0 ? std::sqrt(h[0] / h[1]) : 0.0;
      if (!(h[1] > 0) || c <= inner_goal) break;
      batch = 1;
      double rate = 0.0;
      if (c_prev > 0.0 && c < c_prev) rate = std::pow(c / c_prev, 1.0 / double(k + 1 - k_prev));
      else if (c_prev < 0.0) rate = last_rate;   // a later correction's first check: the previous correction's rate
      if (c_prev > 0.0 && rate > 0.0) last_rate = rate;
      if (rate > 0.0 && rate < 0.95) batch = uint32_t(std::min(8.0, std::max(1.0, std::ceil(std::log(inner_goal / c) / std::log(rate)))));
      c_prev = c;
      k_prev = k + 1;
      in_batch = 0;
    }
    vtk::tc_axpy(B, d, nr, ctx->stream);
  }
  VT_CK(cudaEventRecord(ctx->ev1, ctx->stream));
  uint32_t herr = 0;
  VT_CK(cudaMemcpyAsync(&herr, err, 4, cudaMemcpyDeviceToHost, ctx->stream));
  if ((s = from_device(ctx, q->B, B, nr * 4)) != VT_OK) return s;
  VT_CK(cudaStreamSynchronize(ctx->stream));
  float ms = 0;
  cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
  q->iters = sweeps; q->refinements = refinements; q->residual = resid; q->ms = ms;
  q->sweep_ms = sweeps ? gemm_ms / sweeps : 0.0;
  q->convert_ms = conv_ms;
  ctx->tim.solve_ms = ms;
  if (herr) return fail(ctx, VT_ERR_TIMEOUT, "solve: a tensor-core pipeline wait ran out");
  return resid <= q->tol ? VT_OK : VT_ERR_NOT_CONVERGED;
}

// ------------------------------------------------------------------------------------------------ radiosity solve
// Plain FP32: Jacobi sweeps B <- E + rho F B on CUDA cores (the matvec for one right-hand side, the FP32 GEMM
// for several), the relative update checked every `check_every` sweeps. BF16 / FP8: see vt_tc.cu.
vt_status vt_radiosity_solve(vt_ctx* ctx, vt_solve_req* q) {
  if (!ctx || !q || !q->n || !q->n_rhs || !q->F || !q->rho || !q->E || !q->B) return VT_ERR_ARG;
  if (q->n_rhs > 64) return fail(ctx, VT_ERR_ARG, "solve: at most 64 right-hand sides");
  if (q->n_rhs > 1 && (q->n_rhs % 4)) return fail(ctx, VT_ERR_ARG, "solve: several right-hand sides must be a multiple of 4");
  if (reject_foreign(ctx, {q->F, q->rho, q->E, q->B}) != VT_OK) return VT_ERR_ARG;
  if (q->precision == VT_PREC_BF16 || q->precision == VT_PREC_FP8) return tc_solve(ctx, q);
  if (q->precision != VT_PREC_FP32 && q->precision != VT_PREC_FP32_TMA) return fail(ctx, VT_ERR_ARG, "solve: unknown precision");
  if (q->precision == VT_PREC_FP32_TMA && (q->n_rhs != 1 || q->n % 4u))
    return fail(ctx, VT_ERR_ARG, "solve: the bulk-copy matvec takes one right-hand side and n % 4 == 0");
  const uint32_t n = q->n, R = q->n_rhs;
  const size_t nb = size_t(n) * R * 4, nf = size_t(n) * n * 4;
  const bool dF = is_device_ptr(q->F);
  const bool tma = q->precision == VT_PREC_FP32_TMA;
  if (tma && dF && !aligned16(q->F)) return fail(ctx, VT_ERR_ARG, "solve: the bulk-copy matvec needs a 16-byte aligned F");
  const uint32_t max_blocks = std::max<uint32_t>(std::max<uint32_t>((n + 7) / 8, uint32_t((size_t(n) * R / 4 + 255) / 256)),
                                                 tma ? vtk::jacobi_matvec_tma_blocks(n) : 0u) + 8;
  const size_t gemm_work = R > 1 ? vtk::jacobi_gemm_fp32_work(n, R) : 0;
  const size_t need = (dF ? 0 : nf) + 3 * nb + size_t(n) * 4 + size_t(max_blocks) * 16 + gemm_work + 64 + 2048;
  vt_status s = ensure_scratch(ctx, need);
  if (s != VT_OK) return s;
  char* base = static_cast<char*>(ctx->d_scratch);
  auto take = [&](size_t bytes) { char* p = base; base += (bytes + 255) / 256 * 256; return p; };
  const float* Fd = dF ? q->F : reinterpret_cast<float*>(take(nf));
  float* E = reinterpret_cast<float*>(take(nb));
  float* B0 = reinterpret_cast<float*>(take(nb));
  float* B1 = reinterpret_cast<float*>(take(nb));
  float* rho = reinterpret_cast<float*>(take(size_t(n) * 4));
  double* partials = reinterpret_cast<double*>(take(size_t(max_blocks) * 16));
  double* norms = reinterpret_cast<double*>(take(64));
  float* work = gemm_work ? reinterpret_cast<float*>(take(gemm_work)) : nullptr;
  if (!dF && (s = to_device(ctx, const_cast<float*>(Fd), q->F, nf)) != VT_OK) return s;
  if ((s = to_device(ctx, E, q->E, nb)) != VT_OK) return s;
  if ((s = to_device(ctx, rho, q->rho, size_t(n) * 4)) != VT_OK) return s;
  if (q->warm_start) { if ((s = to_device(ctx, B0, q->B, nb)) != VT_OK) return s; }
  else VT_CK(cudaMemcpyAsync(B0, E, nb, cudaMemcpyDeviceToDevice, ctx->stream));
  const uint32_t check = q->check_every ? q->check_every : 8;
  const uint32_t max_it = q->max_iters ? q->max_iters : 1000;
  float* cur = B0;
  float* nxt = B1;
  uint32_t it = 0, np = 0, sweep_n = 0;
  double resid = INFINITY, sweep_sum = 0;
  VT_CK(cudaEventRecord(ctx->ev0, ctx->stream));
  while (it < max_it) {
    const uint32_t k = std::min(check, max_it - it);
    for (uint32_t j = 0; j < k; j++) {
      if (j == 0) VT_CK(cudaEventRecord(ctx->ev2, ctx->stream));
      if (tma) vtk::launch_jacobi_matvec_tma(Fd, rho, E, cur, nxt, n, partials, &np, ctx->stream);
      else if (R == 1) vtk::launch_jacobi_matvec(Fd, rho, E, cur, nxt, n, partials, &np, ctx->stream);
      else vtk::launch_jacobi_gemm_fp32(Fd, rho, E, cur, nxt, n, R, work, partials, &np, ctx->stream);
      if (j == 0) VT_CK(cudaEventRecord(ctx->ev3, ctx->stream));
      std::swap(cur, nxt);
    }
    ctx->tim.launches += k * (work ? 2 : 1) + 1;
    it += k;
    vtk::launch_reduce_partials(partials, np, norms, ctx->stream);
    VT_CK(cudaGetLastError());
    double h[2];
    VT_CK(cudaMemcpyAsync(h, norms, 16, cudaMemcpyDeviceToHost, ctx->stream));
    VT_CK(cudaStreamSynchronize(ctx->stream));
    resid = h[1] > 0 ? std::sqrt(h[0] / h[1]) : 0.0;
    float gms = 0;
    cudaEventElapsedTime(&gms, ctx->ev2, ctx->ev3);
    sweep_sum += gms;
    sweep_n++;
    if (resid <= q->tol) break;
  }
  VT_CK(cudaEventRecord(ctx->ev1, ctx->stream));
  if ((s = from_device(ctx, q->B, cur, nb)) != VT_OK) return s;
  VT_CK(cudaStreamSynchronize(ctx->stream));
  if (tma && vtk::matvec_error(ctx->stream, true)) return fail(ctx, VT_ERR_TIMEOUT, "solve: a bulk copy of F did not complete");
  float ms = 0;
  cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
  q->iters = it; q->refinements = 0; q->residual = resid; q->ms = ms;
  q->sweep_ms = sweep_n ? sweep_sum / sweep_n : 0.0;
  q->convert_ms = 0.0;
  ctx->tim.solve_ms = ms;
  return resid <= q->tol ? VT_OK : VT_ERR_NOT_CONVERGED;
}
