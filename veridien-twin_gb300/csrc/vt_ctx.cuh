// The context behind the C ABI (include/vtwin.h) and the helpers its entry points share (vt_api.cu, vt_api_batch.cu).
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <initializer_list>
#include <string>
#include <vector>

#include "vt_host.h"
#include "vt_kernels.cuh"
#include "vt_isp.cuh"
#include "vt_lite.cuh"
#include "vt_wave.cuh"

struct vt_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev2 = nullptr, ev3 = nullptr;
  cudaEvent_t nev[4] = {nullptr, nullptr, nullptr, nullptr};   // node radiosity: direct light, Jacobi steps
  void* h_stats = nullptr;       // pinned host words for a frame's sensor statistics (vt_render_frame)
  size_t h_stats_bytes = 0;
  std::string err;
  vt::Prepared S;
  std::vector<vt::InstPose> inst;
  float eavg[3] = {0, 0, 0};
  uint32_t slot = 1, frame = 0;
  float su_host[vt::SU_WORDS];
  // device scene
  float4 *d_nodes = nullptr, *d_tris = nullptr, *d_verts = nullptr, *d_params = nullptr, *d_nstate = nullptr;
  float4* d_top = nullptr;      // staged top levels of the static BVH (vtd::TOP_NODES records at most)
  uint32_t n_top = 0;
  float* d_su = nullptr;
  uint32_t* d_dbg = nullptr;
  uint32_t* d_work = nullptr;   // queue counters of the wavefront path tracer
  int wave_blocks = 0;
  void* d_wave = nullptr;       // wavefront path state (grown on demand)
  size_t wave_cap = 0;
  struct Cam {
    float4* radiance = nullptr;
    float* raw = nullptr;
    bool rendered = false, exposed = false;
    // the sensor chain (vt_sensor_frame): relative illumination map and its working buffers, grown on first use
    float* ri = nullptr;
    void* isp_mem = nullptr;
    vtk::IspBufs isp{};
    size_t isp_lev = 0;   // glare-level pixels the buffers hold
    bool processed = false;
    // static first-hit cache (VT_O_CACHE_*): entries, sub-samples held, and the key they were traced under
    float4* hcache = nullptr;
    uint32_t hc_cap = 0, hc_stride = 0;
    std::vector<double> hc_key;
    // static-occlusion cache (VT_O_SHADOW_CACHE), indexed like the first-hit cache, and its key
    uint32_t* scache = nullptr;
    std::vector<double> sc_key;
  };
  std::vector<Cam> cams;
  // scratch for ray queries and the solver (grown on demand)
  void* d_scratch = nullptr;
  size_t scratch_bytes = 0;
  vt_timings tim{};
  // kernel profiling of vt_render_camera: event pairs around the bounce kernels, ray counters at d_work + 64 B
  bool kprof = false;
  std::vector<cudaEvent_t> kev;
  std::vector<uint8_t> kkind;
  // mixed-precision radiosity: converted copies of F and the solver's work buffers
  struct Tc {
    void* mem = nullptr;
    size_t bytes = 0;
    const float* f_src = nullptr;   // F whose copies are held
    uint32_t n = 0, R = 0, prec = 0;
    bool have_hi_lo = false, have_q = false;
  } tc;
  // batched multi-pose rendering: per-pose uniforms, the (pose, body) cull BVH, wave buffers, staging, graph
  struct Batch {
    float* su = nullptr;            // VT_BATCH_MAX_POSES scene uniforms
    float4* cull = nullptr;         // nodes, then items
    uint32_t* ctr = nullptr;        // queue counters [0..7], status [8], stats (u64) at [16]
    uint32_t* sensor = nullptr;     // 64 words per camera
    void* mem = nullptr;            // wave buffers
    size_t mem_bytes = 0;
    float4* rad = nullptr;          // radiance frames (staging)
    size_t rad_bytes = 0;
    uint16_t* raw = nullptr;        // raw frames (staging)
    size_t raw_bytes = 0;
    cudaGraphExec_t exec = nullptr;
    std::string key;
    uint64_t graph_launches = 0;   // kernels in the captured graph
    uint32_t cap = 0;               // pair capacity of a wave
    // tuned configuration (0: defaults); tile and refill also apply to vt_render_camera
    uint32_t wave_paths = 0, tile_w = 0, tile_h = 0, refill = 0;
  } batch;
  // differentiable calibration: radiosity nodes (clusters of static triangles), F, the emitter transfer D, parameters,
  // per-camera images and targets, and the last forward's state for the backward
  struct Calib {
    bool ready = false, have_forward = false;
    uint32_t n = 0, n_lamps = 0, n_mat = 0, n_static = 0;
    std::vector<float> centres, normals, areas, D_host;
    std::vector<uint32_t> node_mat, tri_node;
    void* mem = nullptr;            // device arena
    float *F = nullptr, *D = nullptr, *C = nullptr, *N = nullptr, *A = nullptr;
    uint32_t *tri_node_d = nullptr, *emit_of_tri_d = nullptr;
    float *albedo = nullptr, *lamp = nullptr, *rho = nullptr /* 3 x n */, *DL = nullptr, *H = nullptr /* 3 x n */;
    double *partials = nullptr, *g_alb = nullptr, *g_lamp = nullptr, *g_H = nullptr, *lam0 = nullptr, *lam1 = nullptr,
           *lam = nullptr /* 3 x n */, *work = nullptr, *loss = nullptr;
    uint32_t max_partials = 0;
    std::vector<float4*> image, target;   // per scene camera (device, w x h)
    std::vector<std::vector<float>> albedo_host;
    // path records of the last forward (stored form), per camera of the request, and with the intrinsics' derivative
    // asked for, each path's derivative record in its primary direction
    void* records = nullptr;
    size_t rec_cap = 0;
    void* tan = nullptr;
    size_t tan_cap = 0;
    bool want_k = false, have_k = false;
    double* g_K = nullptr;   // 8 per scene camera
    std::vector<size_t> rec_off;
    bool stored = false;
    // replay form: sub-samples per chunk and the wave size of the tracing; every path's discrete decisions (per
    // camera at rec_off), kept by the forward when they fit so that the backward re-shades without tracing
    uint32_t chunk = 0, wave_paths = 0;
    void* dec = nullptr;
    size_t dec_cap = 0;
    bool use_dec = false;
    // last forward
    std::vector<uint32_t> cams;
    uint32_t spp = 0, nl = 0, seed = 0, depth = 0, iters = 0;
    double inv_count = 0;
    std::vector<float> rho_host, lamp_host;
  } calib;
  // the scene's node radiosity (vt_nodes_*): gather table, active list, neighbours, update bookkeeping
  struct Nodes {
    bool built = false, auto_update = false;
    vt_nodes_opts o{};
    uint32_t n = 0, n_active = 0, n_mat = 0;
    void* mem = nullptr;
    uint32_t* gtable = nullptr;
    float4* aux = nullptr;
    uint32_t* active = nullptr;
    uint2* nbr = nullptr;
    float4* amu = nullptr;
    void* table_mem = nullptr;               // transport table: row offsets, then entries
    void* direct_mem = nullptr;              // the direct light's shadow rays and terms (node_direct_bytes)
    uint32_t* row = nullptr;
    float4* ent = nullptr;
    uint64_t nnz = 0;
    std::vector<uint32_t> active_h;
    std::vector<float> misses;
    uint64_t poses_version = 0;
    int64_t solved_version = -1;
    int64_t pending = 0;
    bool eavg_settled = false;
    std::vector<vt::InstPose> solved_inst;   // poses of the last update
    std::vector<float> solved_caps;          // 8 floats per body: bounding capsules of the last update
    double build_ms = 0, nbr_ms = 0;
    bool timed_direct = false, timed_jacobi = false;
    uint32_t last_steps = 0;
  } nodes;
  // the scope body's poses0 matrix (column-major), kept for the raster pass's emitter samples and SCOPE camera
  double scope_T[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
  // the raster camera pass (vt_lite_*): geometry, emitter samples, shadow maps, per-camera targets
  struct Lite {
    bool ready = false;
    vt_lite_opts o{};
    uint32_t n_verts = 0, n_tris = 0, n_static_verts = 0, n_static_tris = 0, dyn_verts = 0;
    vt::LiteEmit em;
    void* mem = nullptr;                 // geometry, emitter samples, clip buffers, big-triangle queue, shadow maps
    uint4* v = nullptr;
    uint32_t* idx = nullptr;
    float4* es = nullptr;
    float4* clip = nullptr;              // camera pass (n_verts)
    float4* sclip = nullptr;             // shadow passes (K_SECT x n_verts)
    int4 *snap = nullptr, *ssnap = nullptr;   // snapped vertices of the camera pass and of the shadow passes
    uint32_t* big = nullptr;             // 1 + big_cap words
    uint32_t big_cap = 0;
    uint32_t *sm_static = nullptr, *sm_dyn = nullptr;
    bool sm_static_dirty = true;
    uint64_t sm_dyn_version = ~0ull;
    std::vector<double> scope_key;
    double R[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}}, P[3] = {0, 0, 0};   // scope pose of the current state
    float axisW[3] = {0, 0, 1}, lt[3] = {1, 0, 0}, lb[3] = {0, 1, 0}, lo[4][3] = {};
    double scopeR[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}}, scope_pos[3] = {0, 0, 0};
    struct LCam {
      uint32_t W = 0, H = 0;
      void* mem = nullptr;
      unsigned long long* key = nullptr;
      float4* rad = nullptr;
      uchar4* out = nullptr;
      uint32_t* stats = nullptr;
      bool rendered = false, displayed = false;
    };
    std::vector<LCam> cams;              // the scene cameras, then SCOPE
    void* frag_mem = nullptr;            // fragment-list scratch shared by the cameras (grown to the largest view)
    size_t frag_pixels = 0;
    vtl::FragBufs fb{};
    int32_t last_clip_cam = -1;
    double build_ms = 0, sm_static_ms = 0, sm_dyn_ms = 0, cam_ms = 0, raster_ms = 0, shade_ms = 0;
    uint32_t big_tris = 0, launches = 0, shadow_big = 0;
    cudaEvent_t ev[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  } lite;
};

namespace vtapi {

inline const char* g_static_err = "no context";

#define VT_CK(call)                                                                  \
  do {                                                                               \
    cudaError_t e_ = (call);                                                         \
    if (e_ != cudaSuccess) return fail(ctx, VT_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

inline vt_status fail(vt_ctx* ctx, vt_status s, const std::string& m) {
  if (ctx) ctx->err = m;
  return s;
}

// Where a caller's pointer lives, seen from the current device: host memory (pageable, pinned or registered), this
// device's memory (device or managed, allocated against this device), or another device's memory. A kernel on this
// device must not be given the last kind: with peer access off that is an illegal-address fault.
enum PtrKind { PTR_HOST = 0, PTR_DEVICE = 1, PTR_FOREIGN = 2 };

inline PtrKind ptr_kind(const void* p) {
  if (!p) return PTR_HOST;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) { cudaGetLastError(); return PTR_HOST; }
  if (a.type != cudaMemoryTypeDevice && a.type != cudaMemoryTypeManaged) return PTR_HOST;
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) { cudaGetLastError(); return PTR_FOREIGN; }
  return a.device == dev ? PTR_DEVICE : PTR_FOREIGN;
}

inline bool is_device_ptr(const void* p) { return ptr_kind(p) == PTR_DEVICE; }

// VT_ERR_ARG when any of the pointers is another device's memory
inline vt_status reject_foreign(vt_ctx* ctx, std::initializer_list<const void*> ptrs) {
  for (const void* p : ptrs)
    if (ptr_kind(p) == PTR_FOREIGN) return fail(ctx, VT_ERR_ARG, "a buffer lives on another device than the context's");
  return VT_OK;
}

inline bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

template <typename T>
inline vt_status upload(vt_ctx* ctx, T** dst, const void* src, size_t bytes) {
  VT_CK(cudaMalloc(reinterpret_cast<void**>(dst), std::max<size_t>(bytes, 16)));
  if (bytes) VT_CK(cudaMemcpyAsync(*dst, src, bytes, cudaMemcpyHostToDevice, ctx->stream));
  return VT_OK;
}

inline vt_status ensure_scratch(vt_ctx* ctx, size_t bytes) {
  if (ctx->scratch_bytes >= bytes) return VT_OK;
  if (ctx->d_scratch) { VT_CK(cudaStreamSynchronize(ctx->stream)); VT_CK(cudaFree(ctx->d_scratch)); ctx->d_scratch = nullptr; ctx->scratch_bytes = 0; }
  cudaError_t e = cudaMalloc(&ctx->d_scratch, bytes);
  if (e != cudaSuccess) { cudaGetLastError(); return fail(ctx, VT_ERR_OOM, "scratch allocation of " + std::to_string(bytes) + " bytes failed"); }
  ctx->scratch_bytes = bytes;
  return VT_OK;
}

// The staged top levels of the BVH rooted at `root` (the layout of vtd::TOP_NODES): a breadth-first walk assigns
// slots to the first max_n nodes, and each staged record's references to staged children become TOP_BIT | slot.
// Empty when a walked child index is not above its parent's or past the array (the traversal's own check then
// meets it on the global records).
inline std::vector<uint32_t> top_records(const std::vector<uint32_t>& nodes, uint32_t root, uint32_t max_n) {
  const uint32_t count = uint32_t(nodes.size() / VT_NODE_WORDS);
  if (!max_n || root >= count) return {};
  std::vector<uint32_t> order{root}, out;
  std::vector<std::pair<uint32_t, uint32_t>> slot_of;   // (node, slot), few entries
  slot_of.emplace_back(root, 0);
  for (size_t q = 0; q < order.size(); q++) {
    const uint32_t* r = nodes.data() + size_t(order[q]) * VT_NODE_WORDS;
    for (int c = 0; c < 2; c++) {
      const uint32_t ref = r[8 * c + 3], cnt = r[8 * c + 7];
      if (cnt) continue;
      if (ref <= order[q] || ref >= count) return {};
      if (order.size() < max_n) { slot_of.emplace_back(ref, uint32_t(order.size())); order.push_back(ref); }
    }
  }
  for (uint32_t nd : order) {
    const uint32_t* r = nodes.data() + size_t(nd) * VT_NODE_WORDS;
    uint32_t w[VT_NODE_WORDS];
    std::copy(r, r + VT_NODE_WORDS, w);
    for (int c = 0; c < 2; c++) {
      if (w[8 * c + 7]) continue;
      for (const auto& ps : slot_of)
        if (ps.first == w[8 * c + 3]) { w[8 * c + 3] = vtd::TOP_BIT | ps.second; break; }
    }
    out.insert(out.end(), w, w + VT_NODE_WORDS);
  }
  return out;
}

inline vtd::Scene dev_scene(vt_ctx* ctx) {
  vtd::Scene S;
  S.nodes = ctx->d_nodes; S.tris = ctx->d_tris; S.verts = ctx->d_verts; S.params = ctx->d_params;
  S.su = ctx->d_su; S.nstate = ctx->d_nstate; S.dbg = ctx->d_dbg;
  S.mesh_off = ctx->S.mesh_off; S.mat_off = ctx->S.mat_off; S.alb_off = ctx->S.alb_off; S.prof_off = ctx->S.prof_off;
  S.prof_n = ctx->S.prof_n; S.emit_off = ctx->S.emit_off; S.emit_n = ctx->S.emit_n;
  S.top = ctx->d_top; S.n_top = ctx->n_top; S.top_root = 0;
  return S;
}

inline vt_status write_su(vt_ctx* ctx) {
  vt::scene_uniform(ctx->S, ctx->inst, ctx->eavg, ctx->slot, ctx->frame, ctx->su_host,
                    ctx->nodes.solved_caps.empty() ? nullptr : ctx->nodes.solved_caps.data());
  VT_CK(cudaMemcpyAsync(ctx->d_su, ctx->su_host, sizeof(ctx->su_host), cudaMemcpyHostToDevice, ctx->stream));
  return VT_OK;
}

inline uint32_t skip_mask(const vt_ctx* ctx, uint32_t cam) {
  uint32_t m = 0;
  for (size_t i = 0; i < ctx->S.bodies.size(); i++) if (ctx->S.bodies[i].owner == int(cam)) m |= 1u << i;
  return m;
}

// copy `bytes` from a host or device source into device memory `dst`
inline vt_status to_device(vt_ctx* ctx, void* dst, const void* src, size_t bytes) {
  const PtrKind k = ptr_kind(src);
  if (k == PTR_FOREIGN) return fail(ctx, VT_ERR_ARG, "an input buffer lives on another device than the context's");
  VT_CK(cudaMemcpyAsync(dst, src, bytes, k == PTR_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, ctx->stream));
  return VT_OK;
}
inline vt_status from_device(vt_ctx* ctx, void* dst, const void* src, size_t bytes) {
  const PtrKind k = ptr_kind(dst);
  if (k == PTR_FOREIGN) return fail(ctx, VT_ERR_ARG, "an output buffer lives on another device than the context's");
  VT_CK(cudaMemcpyAsync(dst, src, bytes, k == PTR_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, ctx->stream));
  return VT_OK;
}

// launch parameters of one camera dispatch (gpu/renderer.js:888 _packCam)
inline vtk::CamParams make_cam(const vt_ctx* ctx, uint32_t camera, uint32_t spp, uint32_t n_light, uint32_t seed, uint32_t options, uint32_t mode,
                               uint32_t max_depth, uint32_t root, const float shutter[2], float scale) {
  const vt_camera_desc& c = ctx->S.cams[camera];
  vtk::CamParams cp{};
  const double* T = c.T_D_C;
  for (int k = 0; k < 3; k++) {
    cp.rx[k] = float(T[4 * k]); cp.ry[k] = float(T[4 * k + 1]); cp.rz[k] = float(T[4 * k + 2]); cp.pos[k] = float(T[4 * k + 3]);
  }
  cp.lens = {float(c.fx), float(c.fy), float(c.cx), float(c.cy), float(c.alpha), float(c.k[0]), float(c.k[1]), float(c.k[2]), float(c.k[3])};
  cp.w = c.width; cp.h = c.height;
  cp.spp = std::min(std::max(spp, 1u), mode == VT_SHADE_TWIN ? 64u : 4096u);   // kernels.wgsl.js:169 clamps to 64
  cp.seed = seed; cp.cam_index = camera; cp.options = options; cp.skip = skip_mask(ctx, camera);
  cp.n_light = std::min(std::max(n_light, 1u), 16u);   // shade.wgsl.js:270 clamps to 16
  cp.mode = mode;
  cp.max_depth = std::max(1u, std::min(max_depth, 64u));
  cp.root = root;
  cp.t0 = shutter[0]; cp.t1 = shutter[1]; cp.scale = scale;
  cp.tile_w = ctx->batch.tile_w ? ctx->batch.tile_w : vtk::TILE_W;
  cp.tile_h = ctx->batch.tile_h ? ctx->batch.tile_h : vtk::TILE_H;
  cp.refill = ctx->batch.refill ? ctx->batch.refill : vtk::REFILL;
  return cp;
}

}  // namespace vtapi

