// C ABI of the batched multi-pose renderer (include/vtwin.h vt_render_batch, vt_batch_autotune): per-pose scene
// uniforms, the (pose, body) cull BVH, wave sizing, the CUDA graph of the launch sequence, and the autotuner.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "vt_batch.cuh"
#include "vt_ctx.cuh"

using namespace vtapi;

namespace {

constexpr uint32_t kMaxItems = VT_BATCH_MAX_POSES * VT_MAX_INST;
constexpr uint32_t kMaxNodes = 2 * kMaxItems;
constexpr uint32_t kDefaultWave = 8u << 20;
constexpr uint32_t kMaxCams = 64;

struct Item { float lo[3], hi[3], a[3], b[3], r; uint32_t pose, body; };

// BVH over the items by median split on the widest centroid axis (leaves of <= 4; children adjacent); the shape
// depends only on the item count, so a CUDA graph stays valid across pose sets with the same visible bodies
void build_cull(std::vector<Item>& items, std::vector<float>& nodes) {
  nodes.clear();
  if (items.empty()) return;
  struct Task { uint32_t node, first, count; };
  nodes.resize(8, 0.0f);
  std::vector<Task> todo{{0, 0, uint32_t(items.size())}};
  auto put = [&](uint32_t n, const float lo[3], const float hi[3], uint32_t ref, uint32_t cnt) {
    float* w = nodes.data() + 8 * n;
    for (int k = 0; k < 3; k++) { w[k] = lo[k]; w[4 + k] = hi[k]; }
    std::memcpy(w + 3, &ref, 4);
    std::memcpy(w + 7, &cnt, 4);
  };
  while (!todo.empty()) {
    const Task t = todo.back();
    todo.pop_back();
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    float clo[3] = {INFINITY, INFINITY, INFINITY}, chi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint32_t i = t.first; i < t.first + t.count; i++) {
      for (int k = 0; k < 3; k++) {
        lo[k] = std::min(lo[k], items[i].lo[k]); hi[k] = std::max(hi[k], items[i].hi[k]);
        const float c = 0.5f * (items[i].lo[k] + items[i].hi[k]);
        clo[k] = std::min(clo[k], c); chi[k] = std::max(chi[k], c);
      }
    }
    if (t.count <= 4) { put(t.node, lo, hi, t.first, t.count); continue; }
    int ax = 0;
    for (int k = 1; k < 3; k++) if (chi[k] - clo[k] > chi[ax] - clo[ax]) ax = k;
    const uint32_t half = t.count / 2;
    std::nth_element(items.begin() + t.first, items.begin() + t.first + half, items.begin() + t.first + t.count,
                     [ax](const Item& x, const Item& y) {
                       const float cx = x.lo[ax] + x.hi[ax], cy = y.lo[ax] + y.hi[ax];
                       return cx < cy || (cx == cy && (x.pose < y.pose || (x.pose == y.pose && x.body < y.body)));
                     });
    const uint32_t left = uint32_t(nodes.size() / 8);
    nodes.resize(nodes.size() + 16, 0.0f);
    put(t.node, lo, hi, left, 0);
    todo.push_back({left + 1, t.first + half, t.count - half});
    todo.push_back({left, t.first, half});
  }
}

// the batch's pose sets -> per-pose uniforms, the mask of bodies whose pose varies, the cull items
vt_status prepare_poses(vt_ctx* ctx, const vt_batch_req* q, std::vector<float>& su, uint32_t& vary, std::vector<Item>& items) {
  const vt::Prepared& S = ctx->S;
  const uint32_t nb = q->n_bodies;
  std::vector<std::vector<vt::InstPose>> P(q->n_poses);
  for (uint32_t k = 0; k < q->n_poses; k++)
    P[k] = vt::poses_from(S, q->poses0 + size_t(k) * nb * 16, q->poses1 ? q->poses1 + size_t(k) * nb * 16 : nullptr, nb);
  vary = 0;
  for (size_t i = 0; i < S.bodies.size(); i++) {
    const vt::InstPose& a = P[0][i];
    for (uint32_t k = 1; k < q->n_poses; k++) {
      const vt::InstPose& b = P[k][i];
      bool same = a.valid == b.valid;
      if (same && a.valid) {
        for (int j = 0; j < 4; j++) same &= a.q0[j] == b.q0[j] && a.q1[j] == b.q1[j];
        for (int j = 0; j < 3; j++) same &= a.p0[j] == b.p0[j] && a.p1[j] == b.p1[j];
      }
      if (!same) { vary |= 1u << i; break; }
    }
  }
  if (S.scope_index >= 0 && ((vary >> S.scope_index) & 1u))
    return fail(ctx, VT_ERR_ARG, "render_batch: the body carrying the emitter must keep one pose across the batch");
  su.assign(size_t(q->n_poses) * vt::SU_WORDS, 0.0f);
  items.clear();
  for (uint32_t k = 0; k < q->n_poses; k++) {
    float* f = su.data() + size_t(k) * vt::SU_WORDS;
    vt::scene_uniform(S, P[k], ctx->eavg, ctx->slot, ctx->frame, f);
    for (size_t i = 0; i < S.bodies.size(); i++) {
      if (!((vary >> i) & 1u)) continue;
      const float* I = f + vt::SU_INST + 48 * i;
      uint32_t flags;
      std::memcpy(&flags, I + 15, 4);
      if (flags & 2u) continue;   // hidden under this pose
      Item it{};
      for (int j = 0; j < 3; j++) { it.lo[j] = I[16 + j]; it.hi[j] = I[20 + j]; it.a[j] = I[32 + j]; it.b[j] = I[36 + j]; }
      it.r = I[35];
      it.pose = k;
      it.body = uint32_t(i);
      items.push_back(it);
    }
  }
  return VT_OK;
}

vt_status ensure(vt_ctx* ctx, void** p, size_t& have, size_t need) {
  if (have >= need) return VT_OK;
  VT_CK(cudaStreamSynchronize(ctx->stream));
  if (ctx->batch.exec) { cudaGraphExecDestroy(ctx->batch.exec); ctx->batch.exec = nullptr; ctx->batch.key.clear(); }
  cudaFree(*p);
  *p = nullptr;
  have = 0;
  if (cudaMalloc(p, need) != cudaSuccess) { cudaGetLastError(); return fail(ctx, VT_ERR_OOM, "batch allocation of " + std::to_string(need) + " bytes failed"); }
  have = need;
  return VT_OK;
}

struct Plan {
  std::vector<vtk::CamParams> cams;
  std::vector<size_t> frame_off;   // first pixel of each camera's frames in the outputs
  size_t total_px = 0;             // pixels of all frames
  uint32_t n_pw = 0, P = 0, cap = 0, waves = 0;
  uint64_t shared_paths = 0, samples = 0;
  bool fused = true;
};

vt_status validate(vt_ctx* ctx, const vt_batch_req* q, uint16_t* raw_out) {
  if (!q || !q->cameras || !q->n_cameras || !q->poses0) return fail(ctx, VT_ERR_ARG, "render_batch: missing cameras or poses");
  if (q->n_poses < 1 || q->n_poses > VT_BATCH_MAX_POSES) return fail(ctx, VT_ERR_ARG, "render_batch: n_poses must be 1..64");
  if (q->n_cameras > kMaxCams) return fail(ctx, VT_ERR_ARG, "render_batch: at most 64 cameras per batch");
  if (q->n_bodies > ctx->S.bodies.size()) return fail(ctx, VT_ERR_TOO_MANY_BODIES, "render_batch: more bodies than the scene has");
  for (uint32_t c = 0; c < q->n_cameras; c++)
    if (q->cameras[c] >= ctx->S.cams.size()) return fail(ctx, VT_ERR_UNKNOWN_CAMERA, "unknown camera " + std::to_string(q->cameras[c]));
  if (raw_out && !q->sensor) return fail(ctx, VT_ERR_ARG, "render_batch: raw frames need sensor uniforms");
  if (q->sensor) {
    for (uint32_t c = 0; c < q->n_cameras; c++) {
      const uint32_t* w = q->sensor[c].words;
      const vt_camera_desc& cd = ctx->S.cams[q->cameras[c]];
      float glare, maxdn;
      std::memcpy(&glare, &w[52], 4);
      std::memcpy(&maxdn, &w[24], 4);
      if (w[0] != cd.width || w[1] != cd.height) return fail(ctx, VT_ERR_ARG, "render_batch: sensor size differs from the camera");
      if (glare != 0.0f) return fail(ctx, VT_ERR_ARG, "sensor: veiling glare is not supported by the expose stage (fraction must be 0)");
      if (!(maxdn <= 65535.0f)) return fail(ctx, VT_ERR_ARG, "render_batch: raw frames are uint16 (ADC depth <= 16 bits)");
    }
  }
  return VT_OK;
}

vt_status plan_batch(vt_ctx* ctx, const vt_batch_req* q, uint32_t wave_paths, uint32_t tw, uint32_t th, uint32_t refill, Plan& pl) {
  pl = Plan{};
  uint32_t n_pix_max = 0;
  for (uint32_t c = 0; c < q->n_cameras; c++) {
    vtk::CamParams cp = make_cam(ctx, q->cameras[c], q->spp, q->light_samples, q->seed, q->options, VT_SHADE_PATH, q->max_depth, 0, q->shutter,
                                 q->scale);
    cp.tile_w = tw;
    cp.tile_h = th;
    if (refill) cp.refill = refill;
    pl.cams.push_back(cp);
    pl.frame_off.push_back(pl.total_px);
    pl.total_px += size_t(q->n_poses) * cp.w * cp.h;
    n_pix_max = std::max(n_pix_max, vtk::tiled_pixels(cp.w, cp.h, tw, th));
    pl.samples += uint64_t(q->n_poses) * cp.w * cp.h * cp.spp;
  }
  const uint32_t spp = pl.cams[0].spp;
  const uint32_t band = std::max<uint32_t>(32, (wave_paths / spp) / 32 * 32);
  pl.n_pw = std::min(band, n_pix_max);
  pl.P = pl.n_pw * spp;
  pl.cap = std::max<uint32_t>(ctx->batch.cap, std::max<uint32_t>(pl.P / 2, 1u << 16));
  for (const auto& cp : pl.cams) {
    const uint32_t n_pix = vtk::tiled_pixels(cp.w, cp.h, tw, th);
    pl.waves += (n_pix + pl.n_pw - 1) / pl.n_pw;
    pl.shared_paths += uint64_t(n_pix) * spp;
  }
  if (q->sensor) {
    for (uint32_t c = 0; c < q->n_cameras; c++) {
      float sg;
      std::memcpy(&sg, &q->sensor[c].words[5], 4);
      if (sg > 0.0f) pl.fused = false;
    }
  }
  return VT_OK;
}

// one batch, enqueued on the context's stream (or captured into a graph)
void enqueue(vt_ctx* ctx, const vt_batch_req* q, const Plan& pl, const vtk::BatchCull& bc, const vtk::BatchWave& bw, bool want_rad, bool want_raw) {
  auto& B = ctx->batch;
  cudaMemsetAsync(B.ctr + 8, 0, 64, ctx->stream);   // status and stats
  vtd::Scene S = dev_scene(ctx);
  S.su = B.su;   // pose 0's uniform: the shared paths see the bodies common to the batch there
  for (size_t c = 0; c < pl.cams.size(); c++) {
    const vtk::CamParams& cp = pl.cams[c];
    vtk::BatchOut out{};
    const bool stage_rad = want_rad || (want_raw && !pl.fused);
    out.radiance = stage_rad ? B.rad + pl.frame_off[c] : nullptr;
    out.raw = want_raw ? B.raw + pl.frame_off[c] : nullptr;
    out.sensor = B.sensor + 64 * c;
    out.frame0 = q->frame0;
    out.optics_scale = q->optics_scale;
    out.fused = pl.fused ? 1 : 0;
    vtk::batch_camera(S, cp, bc, bw, q->n_poses, out, ctx->wave_blocks, ctx->stream, &ctx->tim.launches);
    if (want_raw && !pl.fused) {
      const size_t frame = size_t(cp.w) * cp.h;
      for (uint32_t k = 0; k < q->n_poses; k++) {
        vtk::SensorParams sp;
        std::memcpy(sp.w, q->sensor[c].words, sizeof(sp.w));
        sp.w[3] = q->frame0 + k;
        vtk::launch_sensor_expose_u16(sp, B.rad + pl.frame_off[c] + k * frame, q->optics_scale, B.raw + pl.frame_off[c] + k * frame, ctx->stream);
        ctx->tim.launches++;
      }
    }
  }
}

std::string graph_key(const vt_batch_req* q, const Plan& pl, const vtk::BatchCull& bc, const vt_ctx* ctx, bool want_rad, bool want_raw) {
  std::string k;
  auto put = [&](const void* p, size_t n) { k.append(static_cast<const char*>(p), n); };
  for (const auto& cp : pl.cams) put(&cp, sizeof(cp));
  const uint32_t u[] = {q->n_poses, q->frame0, pl.n_pw, pl.P, pl.cap, bc.n_nodes, bc.vary, uint32_t(want_rad), uint32_t(want_raw), uint32_t(pl.fused),
                        uint32_t(ctx->wave_blocks)};
  put(u, sizeof(u));
  put(&q->optics_scale, 4);
  if (q->sensor) put(q->sensor, sizeof(vt_sensor_uniform) * q->n_cameras);
  const void* ptrs[] = {ctx->batch.mem, ctx->batch.rad, ctx->batch.raw};
  put(ptrs, sizeof(ptrs));
  return k;
}

// run the batch once; ms = device time; on a pair-capacity overflow returns VT_OK with *overflow set
vt_status run_batch(vt_ctx* ctx, const vt_batch_req* q, uint16_t* raw_out, float* rad_out, uint32_t wave_paths, uint32_t tw, uint32_t th,
                    uint32_t refill, bool allow_graph, Plan& pl, double& ms, bool& overflow, bool& replayed, uint32_t& vary, uint64_t& pairs) {
  auto& B = ctx->batch;
  overflow = false;
  replayed = false;
  std::vector<float> su;
  std::vector<Item> items;
  vt_status s = prepare_poses(ctx, q, su, vary, items);
  if (s != VT_OK) return s;
  std::vector<float> nodes;
  build_cull(items, nodes);
  if (!B.su) {
    if (cudaMalloc(&B.su, size_t(VT_BATCH_MAX_POSES) * vt::SU_WORDS * 4) != cudaSuccess ||
        cudaMalloc(&B.cull, size_t(2 * kMaxNodes + 4 * kMaxItems) * 16) != cudaSuccess || cudaMalloc(&B.ctr, 256) != cudaSuccess ||
        cudaMalloc(&B.sensor, size_t(kMaxCams) * 256) != cudaSuccess) {
      cudaGetLastError();
      return fail(ctx, VT_ERR_OOM, "batch allocation failed");
    }
  }
  if ((s = plan_batch(ctx, q, wave_paths, tw, th, refill, pl)) != VT_OK) return s;
  const bool want_raw = raw_out != nullptr, want_rad = rad_out != nullptr;
  size_t need = vtk::batch_wave_bytes(pl.P, pl.n_pw, pl.cap, pl.cams[0].n_light);
  if ((s = ensure(ctx, &B.mem, B.mem_bytes, need)) != VT_OK) return s;
  if (want_rad || (want_raw && !pl.fused)) {
    void* p = B.rad;
    if ((s = ensure(ctx, &p, B.rad_bytes, pl.total_px * 16)) != VT_OK) return s;
    B.rad = static_cast<float4*>(p);
  }
  if (want_raw) {
    void* p = B.raw;
    if ((s = ensure(ctx, &p, B.raw_bytes, pl.total_px * 2)) != VT_OK) return s;
    B.raw = static_cast<uint16_t*>(p);
  }
  // inputs of this batch (outside any graph: the graph reads them from these fixed buffers)
  VT_CK(cudaMemcpyAsync(B.su, su.data(), su.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
  std::vector<float> cull(size_t(2 * kMaxNodes + 4 * kMaxItems) * 4, 0.0f);
  std::copy(nodes.begin(), nodes.end(), cull.begin());
  float* it = cull.data() + size_t(2 * kMaxNodes) * 4;
  for (size_t i = 0; i < items.size(); i++) {
    float* w = it + 16 * i;
    for (int k = 0; k < 3; k++) { w[k] = items[i].lo[k]; w[4 + k] = items[i].hi[k]; w[8 + k] = items[i].a[k]; w[12 + k] = items[i].b[k]; }
    std::memcpy(w + 3, &items[i].pose, 4);
    std::memcpy(w + 7, &items[i].body, 4);
    w[11] = items[i].r;
  }
  VT_CK(cudaMemcpyAsync(B.cull, cull.data(), cull.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
  if (q->sensor) VT_CK(cudaMemcpyAsync(B.sensor, q->sensor, sizeof(vt_sensor_uniform) * q->n_cameras, cudaMemcpyHostToDevice, ctx->stream));
  vtk::BatchCull bc{};
  bc.nodes = B.cull;
  bc.items = B.cull + 2 * kMaxNodes;
  bc.n_nodes = uint32_t(nodes.size() / 8);
  bc.vary = vary;
  bc.su_base = B.su;
  bc.su_stride = vt::SU_WORDS;
  const vtk::BatchWave bw = vtk::batch_carve(B.mem, pl.P, pl.n_pw, pl.cap, pl.cams[0].n_light, B.ctr, B.ctr + 8,
                                             reinterpret_cast<unsigned long long*>(B.ctr + 16));
  VT_CK(cudaEventRecord(ctx->ev0, ctx->stream));
  if (allow_graph && q->use_graph) {
    const std::string key = graph_key(q, pl, bc, ctx, want_rad, want_raw);
    if (!B.exec || key != B.key) {
      if (B.exec) { cudaGraphExecDestroy(B.exec); B.exec = nullptr; }
      B.key.clear();
      cudaGraph_t g = nullptr;
      VT_CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
      const uint64_t l0 = ctx->tim.launches;
      enqueue(ctx, q, pl, bc, bw, want_rad, want_raw);
      B.graph_launches = ctx->tim.launches - l0;
      ctx->tim.launches = l0;
      cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
      if (e != cudaSuccess) return fail(ctx, VT_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
      e = cudaGraphInstantiate(&B.exec, g, 0);
      cudaGraphDestroy(g);
      if (e != cudaSuccess) { B.exec = nullptr; return fail(ctx, VT_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e)); }
      B.key = key;
    } else {
      replayed = true;
    }
    VT_CK(cudaEventRecord(ctx->ev0, ctx->stream));
    VT_CK(cudaGraphLaunch(B.exec, ctx->stream));
    ctx->tim.launches += B.graph_launches;
  } else {
    enqueue(ctx, q, pl, bc, bw, want_rad, want_raw);
  }
  VT_CK(cudaGetLastError());
  VT_CK(cudaEventRecord(ctx->ev1, ctx->stream));
  uint32_t ctr[24];
  VT_CK(cudaMemcpyAsync(ctr, B.ctr, sizeof(ctr), cudaMemcpyDeviceToHost, ctx->stream));
  VT_CK(cudaStreamSynchronize(ctx->stream));
  float fms = 0;
  cudaEventElapsedTime(&fms, ctx->ev0, ctx->ev1);
  ms = fms;
  uint64_t pr;
  std::memcpy(&pr, ctr + 16, 8);
  pairs = pr;
  if (ctr[8] > pl.cap) {
    overflow = true;
    B.cap = uint32_t(std::min<uint64_t>(uint64_t(ctr[8]) * 5 / 4 + 1024, 0xffffffffull));
    return VT_OK;
  }
  if (raw_out) VT_CK(cudaMemcpyAsync(raw_out, B.raw, pl.total_px * 2, cudaMemcpyDefault, ctx->stream));
  if (rad_out) VT_CK(cudaMemcpyAsync(rad_out, B.rad, pl.total_px * 16, cudaMemcpyDefault, ctx->stream));
  VT_CK(cudaStreamSynchronize(ctx->stream));
  return VT_OK;
}

}  // namespace

extern "C" {

vt_status vt_render_batch(vt_ctx* ctx, const vt_batch_req* q, uint16_t* raw_out, float* radiance_out, vt_batch_stats* st) {
  if (!ctx) return VT_ERR_ARG;
  vt_status s = validate(ctx, q, raw_out);
  if (s != VT_OK) return s;
  const uint32_t wave = q->wave_paths ? q->wave_paths : (ctx->batch.wave_paths ? ctx->batch.wave_paths : kDefaultWave);
  const uint32_t tw = ctx->batch.tile_w ? ctx->batch.tile_w : vtk::TILE_W, th = ctx->batch.tile_h ? ctx->batch.tile_h : vtk::TILE_H;
  Plan pl;
  double ms = 0;
  bool overflow = false, replayed = false;
  uint32_t vary = 0, reruns = 0;
  uint64_t pairs = 0;
  for (;;) {
    s = run_batch(ctx, q, raw_out, radiance_out, wave, tw, th, 0, true, pl, ms, overflow, replayed, vary, pairs);
    if (s != VT_OK) return s;
    if (!overflow) break;
    if (++reruns > 3) return fail(ctx, VT_ERR_OOM, "render_batch: pair capacity kept overflowing");
  }
  ctx->tim.render_ms = ms;
  if (st) {
    st->ms = ms;
    st->shared_paths = pl.shared_paths;
    st->pair_paths = pairs;
    st->samples = pl.samples;
    st->waves = pl.waves;
    st->graph_replayed = replayed ? 1u : 0u;
    st->reruns = reruns;
    st->vary_mask = vary;
  }
  return VT_OK;
}

vt_status vt_batch_autotune(vt_ctx* ctx, const vt_batch_req* req, vt_tune_row* table, uint32_t max_rows, uint32_t* n_rows, vt_tune_row* best) {
  if (!ctx) return VT_ERR_ARG;
  vt_status s = validate(ctx, req, nullptr);
  if (s != VT_OK) return s;
  vt_batch_req q = *req;
  q.spp = std::min(std::max(req->spp, 1u), 4u);
  q.n_poses = std::min(req->n_poses, 8u);
  q.sensor = nullptr;
  q.use_graph = 0;
  const uint32_t waves[] = {2u << 20, 4u << 20, 8u << 20, 16u << 20};
  const uint32_t tiles[][2] = {{8, 4}, {16, 2}, {4, 8}, {32, 1}};
  const uint32_t refills[] = {4, 16, 32};
  vt_tune_row top{0, 0, 0, INFINITY, 0};
  uint32_t rows = 0;
  auto trial = [&](uint32_t w, uint32_t tw, uint32_t th, uint32_t rf, Plan& pl) -> vt_status {
    double ms = 0;
    bool overflow = false, replayed = false;
    uint32_t vary = 0;
    uint64_t pairs = 0;
    for (int rep = 0; rep < 4; rep++) {   // warm (and grow the pair capacity), then time
      vt_status st = run_batch(ctx, &q, nullptr, nullptr, w, tw, th, rf, false, pl, ms, overflow, replayed, vary, pairs);
      if (st != VT_OK) return st;
      if (!overflow && rep >= 1) break;
    }
    if (overflow) return VT_OK;
    const vt_tune_row r{w, tw, th, float(ms / (double(pl.shared_paths) / 1e6)), rf};
    if (table && rows < max_rows) table[rows] = r;
    rows++;
    if (r.ms_per_mpath < top.ms_per_mpath) top = r;
    return VT_OK;
  };
  // wave size x pixel tile at the default refill threshold, then the refill threshold at the best of those
  uint32_t prev_pw = 0;
  for (uint32_t w : waves) {
    Plan pl;
    if ((s = plan_batch(ctx, &q, w, vtk::TILE_W, vtk::TILE_H, 0, pl)) != VT_OK) return s;
    if (pl.n_pw == prev_pw) continue;   // the frames already fit a smaller wave: the same plan
    prev_pw = pl.n_pw;
    for (const auto& t : tiles) {
      if ((s = trial(w, t[0], t[1], vtk::REFILL, pl)) != VT_OK) return s;
    }
  }
  if (top.wave_paths) {
    const vt_tune_row base = top;
    for (uint32_t rf : refills) {
      Plan pl;
      if ((s = trial(base.wave_paths, base.tile_w, base.tile_h, rf, pl)) != VT_OK) return s;
    }
  }
  if (n_rows) *n_rows = std::min(rows, max_rows);
  if (top.wave_paths == 0) return fail(ctx, VT_ERR_OOM, "autotune: no candidate ran");
  ctx->batch.wave_paths = top.wave_paths;
  ctx->batch.tile_w = top.tile_w;
  ctx->batch.tile_h = top.tile_h;
  ctx->batch.refill = top.refill;
  if (best) *best = top;
  return VT_OK;
}

}  // extern "C"
