// C ABI of the differentiable calibration (include/vtwin.h vt_calib_*, vt_set_camera_intrinsics, vt_reproj_loss):
// radiosity nodes from the static triangles, the node form factors F and emitter transfer D, the forward render and
// loss, the path-replay backward with the transposed-Jacobi adjoint, and the analytic KB4 reprojection Jacobian.
#include <algorithm>
#include <cstdlib>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "vt_calib.cuh"
#include "vt_ctx.cuh"

using namespace vtapi;

namespace {

constexpr uint32_t kMaxMat = 64, kMaxLamps = 4096, kDefaultIters = 96;

float fl(uint32_t w) { float f; std::memcpy(&f, &w, 4); return f; }

// node i = the static triangle slots [i T / n, (i + 1) T / n): consecutive slots of the SAH order are spatially
// coherent (the BVH's leaves in traversal order), so each node is a small patch of one surface. Centre = area-
// weighted centroid, normal = area-weighted face normal (oriented with the vertex normals), material = the one with
// the largest area.
void build_nodes(const vt::Prepared& S, uint32_t n, vt_ctx::Calib& K) {
  const uint32_t T = S.static_tris;
  K.centres.assign(size_t(n) * 3, 0.0f);
  K.normals.assign(size_t(n) * 3, 0.0f);
  K.areas.assign(n, 0.0f);
  K.node_mat.assign(n, 0u);
  K.tri_node.assign(T, 0u);
  std::vector<double> c(size_t(n) * 3, 0.0), nn(size_t(n) * 3, 0.0), a(n, 0.0);
  std::vector<std::vector<double>> mat_area(n);
  for (uint32_t s = 0; s < T; s++) {
    const uint32_t i = uint32_t((uint64_t(s) * n) / T);
    K.tri_node[s] = i;
    const uint32_t* w = S.tris.data() + size_t(s) * 16;
    const double v0[3] = {fl(w[0]), fl(w[1]), fl(w[2])}, e1[3] = {fl(w[4]), fl(w[5]), fl(w[6])}, e2[3] = {fl(w[8]), fl(w[9]), fl(w[10])};
    double fn[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
    const double ar = 0.5 * std::sqrt(fn[0] * fn[0] + fn[1] * fn[1] + fn[2] * fn[2]);
    double vn[3] = {0, 0, 0};
    for (int k = 0; k < 3; k++) {
      const uint32_t v = w[4 * k + 3];
      const uint32_t* vw = S.verts.data() + size_t(v) * 8;
      for (int q = 0; q < 3; q++) vn[q] += fl(vw[4 + q]);
    }
    if (fn[0] * vn[0] + fn[1] * vn[1] + fn[2] * vn[2] < 0) for (double& x : fn) x = -x;
    for (int q = 0; q < 3; q++) {
      c[3 * i + q] += ar * (v0[q] + (e1[q] + e2[q]) / 3.0);
      nn[3 * i + q] += 0.5 * fn[q];   // |fn| / 2 = area: area-weighted unit normal
    }
    a[i] += ar;
    const uint32_t mat = S.meshes[w[12]].mat;
    if (mat_area[i].size() <= mat) mat_area[i].resize(mat + 1, 0.0);
    mat_area[i][mat] += ar;
  }
  for (uint32_t i = 0; i < n; i++) {
    const double l = std::sqrt(nn[3 * i] * nn[3 * i] + nn[3 * i + 1] * nn[3 * i + 1] + nn[3 * i + 2] * nn[3 * i + 2]);
    for (int q = 0; q < 3; q++) {
      K.centres[3 * i + q] = float(a[i] > 0 ? c[3 * i + q] / a[i] : 0.0);
      K.normals[3 * i + q] = float(l > 0 ? nn[3 * i + q] / l : (q == 2 ? 1.0 : 0.0));
    }
    K.areas[i] = float(a[i]);
    uint32_t best = 0;
    for (uint32_t m = 0; m < mat_area[i].size(); m++) if (mat_area[i][m] > mat_area[i][best]) best = m;
    K.node_mat[i] = best;
  }
}

vt_status alloc_calib(vt_ctx* ctx) {
  auto& K = ctx->calib;
  const size_t n = K.n, L = K.n_lamps;
  K.max_partials = std::max<uint32_t>(4096, 2 * ((K.n + 7) / 8) + 16);
  const size_t bytes[] = {n * n * 4, n * L * 4, n * 12, n * 12, n * 4, size_t(ctx->S.tri_count) * 4, size_t(ctx->S.tri_count) * 4,
                          kMaxMat * 12, L * 4, n * 12, n * 4, n * 12,
                          size_t(K.max_partials) * 8, kMaxMat * 24, L * 8, n * 24, n * 8, n * 8, n * 24, vtk::jacobi_t_work(uint32_t(n)), 64,
                          ctx->S.cams.size() * 64};
  size_t total = 0;
  for (size_t b : bytes) total += (b + 255) / 256 * 256;
  cudaFree(K.mem);
  K.mem = nullptr;
  if (cudaMalloc(&K.mem, total) != cudaSuccess) { cudaGetLastError(); return fail(ctx, VT_ERR_OOM, "calibration allocation failed"); }
  char* p = static_cast<char*>(K.mem);
  size_t k = 0;
  auto take = [&]() { char* r = p; p += (bytes[k++] + 255) / 256 * 256; return r; };
  K.F = reinterpret_cast<float*>(take()); K.D = reinterpret_cast<float*>(take());
  K.C = reinterpret_cast<float*>(take()); K.N = reinterpret_cast<float*>(take()); K.A = reinterpret_cast<float*>(take());
  K.tri_node_d = reinterpret_cast<uint32_t*>(take()); K.emit_of_tri_d = reinterpret_cast<uint32_t*>(take());
  K.albedo = reinterpret_cast<float*>(take()); K.lamp = reinterpret_cast<float*>(take()); K.rho = reinterpret_cast<float*>(take());
  K.DL = reinterpret_cast<float*>(take()); K.H = reinterpret_cast<float*>(take());
  K.partials = reinterpret_cast<double*>(take());
  K.g_alb = reinterpret_cast<double*>(take()); K.g_lamp = reinterpret_cast<double*>(take()); K.g_H = reinterpret_cast<double*>(take());
  K.lam0 = reinterpret_cast<double*>(take()); K.lam1 = reinterpret_cast<double*>(take()); K.lam = reinterpret_cast<double*>(take());
  K.work = reinterpret_cast<double*>(take()); K.loss = reinterpret_cast<double*>(take());
  K.g_K = reinterpret_cast<double*>(take());
  return VT_OK;
}

vtk::CamParams calib_cam(const vt_ctx* ctx, uint32_t cam, uint32_t spp, uint32_t nl, uint32_t seed, uint32_t depth) {
  const float sh[2] = {0.0f, 1.0f};
  vtk::CamParams cp = make_cam(ctx, cam, spp, nl, seed, 0u, VT_SHADE_PATH, depth, 0u, sh, 1.0f);
  cp.n_light = std::min(cp.n_light, vtk::CAL_MAX_NL);
  cp.max_depth = std::min(cp.max_depth, vtk::CAL_MAX_DEPTH);
  return cp;
}

vtk::CalibDev calib_dev(vt_ctx* ctx, uint32_t cam) {
  auto& K = ctx->calib;
  vtk::CalibDev C{};
  C.albedo = K.albedo; C.lamp = K.lamp; C.emit_of_tri = K.emit_of_tri_d; C.tri_node = K.tri_node_d; C.H = K.H;
  C.n_static_tris = K.n_static; C.n_mat = K.n_mat; C.n_lamps = K.n_lamps; C.n_nodes = K.n;
  C.target = K.target[cam]; C.image = K.image[cam]; C.inv_count = K.inv_count;
  C.partials = K.partials; C.g_albedo = K.g_alb; C.g_lamp = K.g_lamp; C.g_H = K.g_H;
  C.g_K = K.g_K + 8 * size_t(cam);
  return C;
}

}  // namespace

extern "C" {

vt_status vt_calib_setup(vt_ctx* ctx, const vt_calib_desc* d, vt_calib_info* info) {
  if (!ctx || !d) return VT_ERR_ARG;
  auto& K = ctx->calib;
  const vt::Prepared& S = ctx->S;
  if (!d->n_nodes || d->n_nodes > S.static_tris) return fail(ctx, VT_ERR_ARG, "calib: n_nodes must be 1..static triangles");
  if (S.emit_tris == 0 || S.emit_tris > kMaxLamps) return fail(ctx, VT_ERR_ARG, "calib: the scene needs 1..4096 emitter triangles");
  if (S.mats.size() > kMaxMat) return fail(ctx, VT_ERR_ARG, "calib: at most 64 materials");
  VT_CK(cudaStreamSynchronize(ctx->stream));
  K.ready = K.have_forward = false;
  K.n = d->n_nodes;
  K.n_lamps = S.emit_tris;
  K.n_mat = uint32_t(S.mats.size());
  K.n_static = S.static_tris;
  build_nodes(S, K.n, K);
  vt_status s = alloc_calib(ctx);
  if (s != VT_OK) return s;
  VT_CK(cudaMemcpyAsync(K.C, K.centres.data(), K.centres.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
  VT_CK(cudaMemcpyAsync(K.N, K.normals.data(), K.normals.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
  VT_CK(cudaMemcpyAsync(K.A, K.areas.data(), K.areas.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
  std::vector<uint32_t> tn(S.tri_count, 0xffffffffu);
  std::copy(K.tri_node.begin(), K.tri_node.end(), tn.begin());
  VT_CK(cudaMemcpyAsync(K.tri_node_d, tn.data(), tn.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
  VT_CK(cudaMemcpyAsync(K.emit_of_tri_d, S.emit_of_tri.data(), S.emit_of_tri.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
  vtk::launch_form_factors(K.n, K.C, K.N, K.A, K.F, ctx->stream);
  vtk::launch_direct_transfer(dev_scene(ctx), K.C, K.N, K.n, K.n_lamps, std::max(1u, d->lamp_samples), K.D, ctx->stream);
  VT_CK(cudaGetLastError());
  K.D_host.resize(size_t(K.n) * K.n_lamps);
  VT_CK(cudaMemcpyAsync(K.D_host.data(), K.D, K.D_host.size() * 4, cudaMemcpyDeviceToHost, ctx->stream));
  K.image.assign(S.cams.size(), nullptr);
  K.target.assign(S.cams.size(), nullptr);
  VT_CK(cudaStreamSynchronize(ctx->stream));
  K.ready = true;
  if (info) { info->n_nodes = K.n; info->n_materials = K.n_mat; info->n_lamps = K.n_lamps; info->n_static_tris = K.n_static; }
  return VT_OK;
}

vt_status vt_calib_export(vt_ctx* ctx, float* centres, float* normals, float* areas, uint32_t* node_mat, uint32_t* tri_node, float* F, float* D) {
  if (!ctx) return VT_ERR_ARG;
  auto& K = ctx->calib;
  if (!K.ready) return fail(ctx, VT_ERR_STATE, "calib: export before setup");
  if (centres) std::copy(K.centres.begin(), K.centres.end(), centres);
  if (normals) std::copy(K.normals.begin(), K.normals.end(), normals);
  if (areas) std::copy(K.areas.begin(), K.areas.end(), areas);
  if (node_mat) std::copy(K.node_mat.begin(), K.node_mat.end(), node_mat);
  if (tri_node) std::copy(K.tri_node.begin(), K.tri_node.end(), tri_node);
  if (D) std::copy(K.D_host.begin(), K.D_host.end(), D);
  if (F) {
    VT_CK(cudaMemcpyAsync(F, K.F, size_t(K.n) * K.n * 4, cudaMemcpyDefault, ctx->stream));
    VT_CK(cudaStreamSynchronize(ctx->stream));
  }
  return VT_OK;
}

vt_status vt_calib_forward(vt_ctx* ctx, const vt_calib_req* q, double* loss) {
  if (!ctx || !q || !q->cameras || !q->n_cameras || !q->albedo || !q->lamp) return VT_ERR_ARG;
  auto& K = ctx->calib;
  const vt::Prepared& S = ctx->S;
  if (!K.ready) return fail(ctx, VT_ERR_STATE, "calib: forward before setup");
  for (uint32_t c = 0; c < q->n_cameras; c++)
    if (q->cameras[c] >= S.cams.size()) return fail(ctx, VT_ERR_UNKNOWN_CAMERA, "unknown camera " + std::to_string(q->cameras[c]));
  // Lambertian materials: the estimator's f = rho / pi is the reference BSDF only for dielectrics of ior 1
  std::vector<float> alb(size_t(K.n_mat) * 3), lamp(K.n_lamps);
  for (uint32_t m = 0; m < K.n_mat; m++) {
    for (int c = 0; c < 3; c++) {
      const double a = q->albedo[3 * m + c];
      if (!(a > 0.0 && a <= 1.0)) return fail(ctx, VT_ERR_ARG, "calib: albedos must be in (0, 1]");
      alb[3 * m + c] = float(a);
    }
  }
  for (uint32_t t = 0; t < K.n_lamps; t++) {
    if (!(q->lamp[t] >= 0.0) || !std::isfinite(q->lamp[t])) return fail(ctx, VT_ERR_ARG, "calib: lamp radiances must be finite and >= 0");
    lamp[t] = float(q->lamp[t]);
  }
  const uint32_t iters = q->jacobi_iters ? q->jacobi_iters : kDefaultIters;
  // node albedo per channel (planar 3 x n)
  std::vector<float> rho(size_t(3) * K.n);
  for (uint32_t c = 0; c < 3; c++) for (uint32_t i = 0; i < K.n; i++) rho[size_t(c) * K.n + i] = alb[3 * K.node_mat[i] + c];
  VT_CK(cudaMemcpyAsync(K.albedo, alb.data(), alb.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
  VT_CK(cudaMemcpyAsync(K.lamp, lamp.data(), lamp.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
  VT_CK(cudaMemcpyAsync(K.rho, rho.data(), rho.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
  // radiosity: B = rho o (D L + F B) per channel, iters sweeps at FP64 accuracy from B = rho o D L; H = F B. FP64
  // accuracy so that the node light carries no rounding that moves with every parameter (central differences of the
  // loss see it). The three channels in one pass over F; the iterates in the adjoint's work array (48 n bytes of its
  // JT splits x n doubles), which the forward does not otherwise use
  vtk::launch_dl(K.D, K.lamp, K.n, K.n_lamps, K.DL, ctx->stream);
  vtk::launch_radiosity64(K.F, K.rho, K.DL, K.n, iters, K.work, K.H, ctx->stream);
  // cameras
  size_t px_total = 0;
  for (uint32_t c = 0; c < q->n_cameras; c++) px_total += size_t(S.cams[q->cameras[c]].width) * S.cams[q->cameras[c]].height;
  K.inv_count = 1.0 / (3.0 * double(px_total));
  size_t off = 0;
  for (uint32_t c = 0; c < q->n_cameras; c++) {
    const uint32_t cam = q->cameras[c];
    const size_t px = size_t(S.cams[cam].width) * S.cams[cam].height;
    if (!K.image[cam]) {
      if (cudaMalloc(&K.image[cam], px * 16) != cudaSuccess || cudaMalloc(&K.target[cam], px * 16) != cudaSuccess) {
        cudaGetLastError();
        return fail(ctx, VT_ERR_OOM, "calib: image allocation failed");
      }
      VT_CK(cudaMemsetAsync(K.target[cam], 0, px * 16, ctx->stream));
    }
    if (q->targets) VT_CK(cudaMemcpyAsync(K.target[cam], q->targets + 4 * off, px * 16, cudaMemcpyDefault, ctx->stream));
    off += px;
  }
  // stored form when every path's record fits in half the free device memory (and replay is not asked for)
  std::vector<vtk::CamParams> cps;
  size_t rec_total = 0;
  K.rec_off.clear();
  for (uint32_t c = 0; c < q->n_cameras; c++) {
    cps.push_back(calib_cam(ctx, q->cameras[c], q->spp, q->light_samples, q->seed, q->max_depth));
    K.rec_off.push_back(rec_total);
    rec_total += size_t(vtk::tiled_pixels(cps[c].w, cps[c].h, cps[c].tile_w, cps[c].tile_h)) * cps[c].spp;
  }
  K.stored = false;
  K.use_dec = false;
  K.want_k = q->intrinsics != 0;
  K.have_k = false;
  uint32_t wave_paths = 0;
  if (!q->replay) {
    size_t fr = 0, tot = 0;
    cudaMemGetInfo(&fr, &tot);
    const size_t rec_bytes = vtk::calib_record_bytes(uint32_t(std::min<size_t>(rec_total, 0xffffffffu)));
    const size_t tan_bytes = K.want_k ? vtk::calib_tan_bytes(uint32_t(std::min<size_t>(rec_total, 0xffffffffu))) : 0;
    wave_paths = uint32_t(std::min<size_t>(8u << 20, rec_total));
    const size_t wave_need = vtk::wave_bytes(wave_paths, cps[0].n_light, 0);
    if (rec_total < 0xffffffffu && rec_bytes + tan_bytes + (ctx->wave_cap >= wave_need ? 0 : wave_need) <= fr / 2) {
      vt_status st = VT_OK;
      if (K.rec_cap < rec_bytes) {
        VT_CK(cudaStreamSynchronize(ctx->stream));
        cudaFree(K.records);
        K.records = nullptr;
        K.rec_cap = 0;
        if (cudaMalloc(&K.records, rec_bytes) != cudaSuccess) { cudaGetLastError(); st = VT_ERR_OOM; }
        else K.rec_cap = rec_bytes;
      }
      if (st == VT_OK && K.tan_cap < tan_bytes) {
        VT_CK(cudaStreamSynchronize(ctx->stream));
        cudaFree(K.tan);
        K.tan = nullptr;
        K.tan_cap = 0;
        if (cudaMalloc(&K.tan, tan_bytes) != cudaSuccess) { cudaGetLastError(); st = VT_ERR_OOM; }
        else K.tan_cap = tan_bytes;
      }
      if (st == VT_OK && ctx->wave_cap < wave_need) {
        VT_CK(cudaStreamSynchronize(ctx->stream));
        cudaFree(ctx->d_wave);
        ctx->d_wave = nullptr;
        ctx->wave_cap = 0;
        if (cudaMalloc(&ctx->d_wave, wave_need) != cudaSuccess) { cudaGetLastError(); st = VT_ERR_OOM; }
        else ctx->wave_cap = wave_need;
      }
      K.stored = st == VT_OK;
    }
  }
  if (!K.stored) {
    // replay form: the paths traced in chunks of sub-samples, one chunk's records (and derivative records) at a time,
    // a chunk sized to a quarter of the free memory (or to replay - 1 sub-samples when the request asks for less)
    size_t fr = 0, tot = 0;
    cudaMemGetInfo(&fr, &tot);
    size_t n_pix_max = 1;
    for (const auto& cp : cps) n_pix_max = std::max<size_t>(n_pix_max, vtk::tiled_pixels(cp.w, cp.h, cp.tile_w, cp.tile_h));
    const size_t per_sub = n_pix_max * (vtk::calib_record_bytes(1) + (K.want_k ? vtk::calib_tan_bytes(1) : 0));
    const uint32_t cap = q->replay >= 2 ? q->replay - 1 : q->spp;
    K.chunk = uint32_t(std::max<size_t>(1, std::min<size_t>({size_t(cap), size_t(q->spp), (fr / 4) / std::max<size_t>(per_sub, 1)})));
    const size_t chunk_paths = n_pix_max * K.chunk;
    K.wave_paths = uint32_t(std::min<size_t>(8u << 20, chunk_paths));
    const size_t rec_bytes = vtk::calib_record_bytes(uint32_t(chunk_paths));
    const size_t tan_bytes = K.want_k ? vtk::calib_tan_bytes(uint32_t(chunk_paths)) : 0;
    const size_t wave_need = vtk::wave_bytes(K.wave_paths, cps[0].n_light, 0);
    auto grow = [&](void*& ptr, size_t& cap_bytes, size_t need) -> bool {
      if (cap_bytes >= need) return true;
      cudaStreamSynchronize(ctx->stream);
      cudaFree(ptr);
      ptr = nullptr;
      cap_bytes = 0;
      if (cudaMalloc(&ptr, need) != cudaSuccess) { cudaGetLastError(); return false; }
      cap_bytes = need;
      return true;
    };
    void* wave = ctx->d_wave;
    size_t wave_cap = ctx->wave_cap;
    const bool ok = grow(K.records, K.rec_cap, rec_bytes) && (!tan_bytes || grow(K.tan, K.tan_cap, tan_bytes)) && grow(wave, wave_cap, wave_need);
    ctx->d_wave = wave;
    ctx->wave_cap = wave_cap;
    if (!ok) return fail(ctx, VT_ERR_OOM, "calib: replay buffers (one chunk of path records and the wave state)");
    // the paths' decisions (24 B each) when they fit in a quarter of what is left; otherwise the backward traces
    // again. VT_CALIB_RETRACE=1 makes it trace again regardless.
    const char* rt = std::getenv("VT_CALIB_RETRACE");
    const size_t dec_bytes = vtk::calib_dec_bytes(uint32_t(std::min<size_t>(rec_total, 0xffffffffu)));
    K.use_dec = false;
    if (!(rt && *rt && *rt != '0') && rec_total < 0xffffffffu) {
      cudaMemGetInfo(&fr, &tot);
      K.use_dec = (K.dec_cap >= dec_bytes || dec_bytes <= fr / 4) && grow(K.dec, K.dec_cap, dec_bytes);
    }
  }
  double total = 0.0;
  off = 0;
  for (uint32_t c = 0; c < q->n_cameras; c++) {
    const uint32_t cam = q->cameras[c];
    const vtk::CamParams& cp = cps[c];
    const vtk::CalibDev C = calib_dev(ctx, cam);
    const int blocks = std::min<int>(ctx->wave_blocks * 2, int(K.max_partials));
    uint32_t nb;
    if (K.stored) {
      const vtk::WaveBufs wb = vtk::wave_carve(ctx->d_wave, wave_paths, cp.n_light, 0, ctx->d_work);
      nb = vtk::calib_wave_forward(dev_scene(ctx), cp, C, wb, wave_paths, static_cast<char*>(K.records) + K.rec_off[c] * vtk::calib_record_bytes(1),
                                   K.want_k ? static_cast<char*>(K.tan) + K.rec_off[c] * vtk::calib_tan_bytes(1) : nullptr,
                                   std::min<int>(ctx->wave_blocks, int(K.max_partials)), ctx->stream);
    } else {
      const vtk::WaveBufs wb = vtk::wave_carve(ctx->d_wave, K.wave_paths, cp.n_light, 0, ctx->d_work);
      const int wblocks = std::min<int>(ctx->wave_blocks, int(K.max_partials));
      nb = 0;
      for (uint32_t i0 = 0; i0 < cp.spp; i0 += K.chunk)
        nb = vtk::calib_wave_chunk(dev_scene(ctx), cp, C, wb, K.wave_paths, K.records, nullptr, i0, std::min(cp.spp, i0 + K.chunk), 0, wblocks,
                                   ctx->stream, K.use_dec ? static_cast<char*>(K.dec) + K.rec_off[c] * vtk::calib_dec_bytes(1) : nullptr,
                                   K.use_dec ? 1 : 0);
    }
    vtk::launch_sum(K.partials, nb, K.loss, ctx->stream);
    VT_CK(cudaGetLastError());
    double l = 0;
    VT_CK(cudaMemcpyAsync(&l, K.loss, 8, cudaMemcpyDeviceToHost, ctx->stream));
    VT_CK(cudaStreamSynchronize(ctx->stream));
    total += l;
    const size_t px = size_t(S.cams[cam].width) * S.cams[cam].height;
    if (q->images) VT_CK(cudaMemcpyAsync(q->images + 4 * off, K.image[cam], px * 16, cudaMemcpyDefault, ctx->stream));
    off += px;
  }
  VT_CK(cudaStreamSynchronize(ctx->stream));
  K.cams.assign(q->cameras, q->cameras + q->n_cameras);
  K.spp = q->spp; K.nl = q->light_samples; K.seed = q->seed; K.depth = q->max_depth; K.iters = iters;
  K.rho_host = rho;
  K.have_forward = true;
  if (loss) *loss = total;
  return VT_OK;
}

vt_status vt_calib_backward(vt_ctx* ctx, double* g_albedo, double* g_lamp) {
  if (!ctx) return VT_ERR_ARG;
  auto& K = ctx->calib;
  if (!K.ready || !K.have_forward) return fail(ctx, VT_ERR_STATE, "calib: backward before forward");
  const size_t n = K.n;
  VT_CK(cudaMemsetAsync(K.g_alb, 0, size_t(K.n_mat) * 24, ctx->stream));
  VT_CK(cudaMemsetAsync(K.g_lamp, 0, size_t(K.n_lamps) * 8, ctx->stream));
  VT_CK(cudaMemsetAsync(K.g_H, 0, n * 24, ctx->stream));
  VT_CK(cudaMemsetAsync(K.g_K, 0, ctx->S.cams.size() * 64, ctx->stream));
  // every camera of the forward: from the kept records, or by tracing each path again
  for (size_t c = 0; c < K.cams.size(); c++) {
    const uint32_t cam = K.cams[c];
    const vtk::CamParams cp = calib_cam(ctx, cam, K.spp, K.nl, K.seed, K.depth);
    if (K.stored)
      vtk::calib_records_backward(cp, calib_dev(ctx, cam), static_cast<char*>(K.records) + K.rec_off[c] * vtk::calib_record_bytes(1),
                                  K.want_k ? static_cast<char*>(K.tan) + K.rec_off[c] * vtk::calib_tan_bytes(1) : nullptr,
                                  ctx->wave_blocks * 2, ctx->stream);
    else {
      const vtk::WaveBufs wb = vtk::wave_carve(ctx->d_wave, K.wave_paths, cp.n_light, 0, ctx->d_work);
      const int wblocks = std::min<int>(ctx->wave_blocks, int(K.max_partials));
      for (uint32_t i0 = 0; i0 < cp.spp; i0 += K.chunk)
        vtk::calib_wave_chunk(dev_scene(ctx), cp, calib_dev(ctx, cam), wb, K.wave_paths, K.records, K.want_k ? K.tan : nullptr, i0,
                              std::min(cp.spp, i0 + K.chunk), K.want_k ? 2 : 1, wblocks, ctx->stream,
                              K.use_dec ? static_cast<char*>(K.dec) + K.rec_off[c] * vtk::calib_dec_bytes(1) : nullptr, K.use_dec ? 2 : 0);
    }
  }
  K.have_k = K.want_k;
  VT_CK(cudaGetLastError());
  // transposed Jacobi: lambda = F^T (g_H + rho o lambda) per channel, from lambda = 0
  for (uint32_t c = 0; c < 3; c++) {
    VT_CK(cudaMemsetAsync(K.lam0, 0, n * 8, ctx->stream));
    double *cur = K.lam0, *nxt = K.lam1;
    for (uint32_t it = 0; it < K.iters; it++) {
      vtk::launch_jacobi_t(K.F, K.g_H + c * n, K.rho + c * n, cur, nxt, uint32_t(n), K.work, ctx->stream);
      std::swap(cur, nxt);
    }
    VT_CK(cudaMemcpyAsync(K.lam + c * n, cur, n * 8, cudaMemcpyDeviceToDevice, ctx->stream));
  }
  VT_CK(cudaGetLastError());
  std::vector<double> ga(size_t(K.n_mat) * 3), gl(K.n_lamps), lam(3 * n);
  std::vector<float> DL(n), H(3 * n);
  VT_CK(cudaMemcpyAsync(ga.data(), K.g_alb, ga.size() * 8, cudaMemcpyDeviceToHost, ctx->stream));
  VT_CK(cudaMemcpyAsync(gl.data(), K.g_lamp, gl.size() * 8, cudaMemcpyDeviceToHost, ctx->stream));
  VT_CK(cudaMemcpyAsync(lam.data(), K.lam, lam.size() * 8, cudaMemcpyDeviceToHost, ctx->stream));
  VT_CK(cudaMemcpyAsync(DL.data(), K.DL, n * 4, cudaMemcpyDeviceToHost, ctx->stream));
  VT_CK(cudaMemcpyAsync(H.data(), K.H, 3 * n * 4, cudaMemcpyDeviceToHost, ctx->stream));
  VT_CK(cudaStreamSynchronize(ctx->stream));
  // the nodes' share: d/d rho_i = lambda_i (D L + H)_i, d/d L_t = sum_i lambda_i rho_i D_it (FP64)
  for (uint32_t c = 0; c < 3; c++) {
    for (size_t i = 0; i < n; i++) {
      const double l = lam[c * n + i];
      if (l == 0.0) continue;
      ga[3 * K.node_mat[i] + c] += l * (double(DL[i]) + double(H[c * n + i]));
      const double lr = l * double(K.rho_host[c * n + i]);
      const float* Drow = K.D_host.data() + i * K.n_lamps;
      for (uint32_t t = 0; t < K.n_lamps; t++) gl[t] += lr * double(Drow[t]);
    }
  }
  if (g_albedo) std::copy(ga.begin(), ga.end(), g_albedo);
  if (g_lamp) std::copy(gl.begin(), gl.end(), g_lamp);
  return VT_OK;
}

vt_status vt_calib_intrinsics_grad(vt_ctx* ctx, double* g_K) {
  if (!ctx || !g_K) return VT_ERR_ARG;
  auto& K = ctx->calib;
  if (!K.have_k) return fail(ctx, VT_ERR_STATE, "calib: no backward of a forward with intrinsics = 1");
  std::vector<double> all(ctx->S.cams.size() * 8);
  VT_CK(cudaMemcpyAsync(all.data(), K.g_K, all.size() * 8, cudaMemcpyDeviceToHost, ctx->stream));
  VT_CK(cudaStreamSynchronize(ctx->stream));
  for (size_t c = 0; c < K.cams.size(); c++) std::copy(all.begin() + 8 * K.cams[c], all.begin() + 8 * K.cams[c] + 8, g_K + 8 * c);
  return VT_OK;
}

vt_status vt_calib_export_paths(vt_ctx* ctx, uint32_t slot, uint32_t* tri_inst, float* q) {
  if (!ctx || !tri_inst || !q) return VT_ERR_ARG;
  auto& K = ctx->calib;
  if (!K.have_forward || !K.stored || !K.want_k) return fail(ctx, VT_ERR_STATE, "calib: export needs a stored forward with intrinsics = 1");
  if (slot >= K.cams.size()) return fail(ctx, VT_ERR_ARG, "calib: camera slot out of range");
  const uint32_t cam = K.cams[slot];
  const vtk::CamParams cp = calib_cam(ctx, cam, K.spp, K.nl, K.seed, K.depth);
  const size_t paths = size_t(cp.w) * cp.h * cp.spp;
  const size_t b_ti = paths * vtk::CAL_MAX_DEPTH * 8, b_q = paths * vtk::CAL_MAX_DEPTH * vtk::CAL_MAX_NL * 4;
  vt_status s = ensure_scratch(ctx, b_ti + b_q + 512);
  if (s != VT_OK) return s;
  char* base = static_cast<char*>(ctx->d_scratch);
  uint32_t* d_ti = reinterpret_cast<uint32_t*>(base);
  float* d_q = reinterpret_cast<float*>(base + (b_ti + 255) / 256 * 256);
  vtk::calib_export_paths(cp, static_cast<char*>(K.records) + K.rec_off[slot] * vtk::calib_record_bytes(1),
                          static_cast<char*>(K.tan) + K.rec_off[slot] * vtk::calib_tan_bytes(1), d_ti, d_q, ctx->stream);
  VT_CK(cudaGetLastError());
  VT_CK(cudaMemcpyAsync(tri_inst, d_ti, b_ti, cudaMemcpyDefault, ctx->stream));
  VT_CK(cudaMemcpyAsync(q, d_q, b_q, cudaMemcpyDefault, ctx->stream));
  VT_CK(cudaStreamSynchronize(ctx->stream));
  return VT_OK;
}

vt_status vt_set_camera_intrinsics(vt_ctx* ctx, uint32_t camera, const double K[8]) {
  if (!ctx || !K) return VT_ERR_ARG;
  if (camera >= ctx->S.cams.size()) return fail(ctx, VT_ERR_UNKNOWN_CAMERA, "unknown camera " + std::to_string(camera));
  for (int k = 0; k < 8; k++) if (!std::isfinite(K[k])) return fail(ctx, VT_ERR_ARG, "intrinsics must be finite");
  if (!(K[0] > 0 && K[1] > 0)) return fail(ctx, VT_ERR_ARG, "focal lengths must be positive");
  vt_camera_desc& c = ctx->S.cams[camera];
  c.fx = K[0]; c.fy = K[1]; c.cx = K[2]; c.cy = K[3];
  for (int k = 0; k < 4; k++) c.k[k] = K[4 + k];
  return VT_OK;
}

vt_status vt_get_camera_intrinsics(const vt_ctx* ctx, uint32_t camera, double K[8]) {
  if (!ctx || !K || camera >= ctx->S.cams.size()) return VT_ERR_ARG;
  const vt_camera_desc& c = ctx->S.cams[camera];
  K[0] = c.fx; K[1] = c.fy; K[2] = c.cx; K[3] = c.cy;
  for (int k = 0; k < 4; k++) K[4 + k] = c.k[k];
  return VT_OK;
}

// gpu/lens.js:43 project: u = fx (xd + alpha yd) + cx, v = fy yd + cy, (xd, yd) = (x, y) theta_d / r,
// theta_d = theta (1 + k1 theta^2 + k2 theta^4 + k3 theta^6 + k4 theta^8). Its Jacobian in (fx, fy, cx, cy, k1..k4):
// du/dfx = xd + alpha yd, dv/dfy = yd, du/dcx = dv/dcy = 1, du/dk_i = fx (x + alpha y) / r theta^(2i+1),
// dv/dk_i = fy y / r theta^(2i+1).
vt_status vt_reproj_loss(vt_ctx* ctx, const uint32_t* cameras, uint32_t n_cameras, const double* pts, uint32_t n_pts, const double* uv_t,
                         double* loss, double* g_K) {
  if (!ctx || !cameras || !n_cameras || (n_pts && (!pts || !uv_t)) || !loss) return VT_ERR_ARG;
  double L = 0.0;
  size_t observed = 0;   // a NaN target: the point is not observed by that camera
  for (size_t i = 0; i < size_t(n_cameras) * n_pts; i++) observed += std::isnan(uv_t[2 * i]) || std::isnan(uv_t[2 * i + 1]) ? 0 : 1;
  const double norm = 1.0 / (2.0 * double(std::max<size_t>(1, observed)));
  for (uint32_t ci = 0; ci < n_cameras; ci++) {
    if (cameras[ci] >= ctx->S.cams.size()) return fail(ctx, VT_ERR_UNKNOWN_CAMERA, "unknown camera " + std::to_string(cameras[ci]));
    const vt_camera_desc& c = ctx->S.cams[cameras[ci]];
    const double* T = c.T_D_C;
    double g[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (uint32_t i = 0; i < n_pts; i++) {
      const double ut = uv_t[(size_t(ci) * n_pts + i) * 2], vt = uv_t[(size_t(ci) * n_pts + i) * 2 + 1];
      if (std::isnan(ut) || std::isnan(vt)) continue;
      const double d[3] = {pts[3 * i] - T[3], pts[3 * i + 1] - T[7], pts[3 * i + 2] - T[11]};
      const double x = T[0] * d[0] + T[4] * d[1] + T[8] * d[2];
      const double y = T[1] * d[0] + T[5] * d[1] + T[9] * d[2];
      const double z = T[2] * d[0] + T[6] * d[1] + T[10] * d[2];
      const double r = std::hypot(x, y);
      double u, v, J[2][8] = {{0}};
      if (r < 1e-300) {
        u = c.cx; v = c.cy;
        J[0][2] = 1; J[1][3] = 1;
      } else {
        const double th = std::atan2(r, z), t2 = th * th;
        const double thd = th * (1 + t2 * (c.k[0] + t2 * (c.k[1] + t2 * (c.k[2] + t2 * c.k[3]))));
        const double s = thd / r, xd = x * s, yd = y * s;
        u = c.fx * (xd + c.alpha * yd) + c.cx;
        v = c.fy * yd + c.cy;
        J[0][0] = xd + c.alpha * yd; J[1][1] = yd; J[0][2] = 1; J[1][3] = 1;
        double tp = th * t2;
        for (int k = 0; k < 4; k++) {
          J[0][4 + k] = c.fx * (x + c.alpha * y) / r * tp;
          J[1][4 + k] = c.fy * y / r * tp;
          tp *= t2;
        }
      }
      const double du = u - ut, dv = v - vt;
      L += (du * du + dv * dv) * norm;
      for (int k = 0; k < 8; k++) g[k] += 2.0 * norm * (du * J[0][k] + dv * J[1][k]);
    }
    if (g_K) std::copy(g, g + 8, g_K + 8 * ci);
  }
  *loss = L;
  return VT_OK;
}

}  // extern "C"
