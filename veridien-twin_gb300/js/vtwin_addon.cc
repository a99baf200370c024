// Node-API addon over libvtwin's C ABI (include/vtwin.h): the binding the JavaScript TwinRenderer /
// LiteNodesRenderer of renderer.js call in place of the reference's WebGPU code (gpu/renderer.js, lite_nodes/renderer.js).
//
// Conventions: a context is a JS external wrapping the vt_ctx (destroyed by destroy() or by the garbage collector);
// array arguments are TypedArrays (Float32Array, Float64Array, Uint32Array) or ArrayBuffers, read in place; results
// are new TypedArrays or plain objects; a vt_status other than VT_OK (and VT_ERR_NOT_CONVERGED where a solve reports
// it) throws an Error with vt_last_error's text and a `status` property, as the reference throws Error.
// Build: node-gyp with binding.gyp beside this file (links libvtwin.so).
#include <node_api.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "vtwin.h"

namespace {

// ------------------------------------------------------------------------------------------------ helpers
struct Holder { vt_ctx* ctx; };

void finalize_ctx(napi_env, void* data, void*) {
  Holder* h = static_cast<Holder*>(data);
  if (h->ctx) vt_destroy(h->ctx);
  delete h;
}

napi_value undefined(napi_env env) { napi_value u; napi_get_undefined(env, &u); return u; }

bool throw_status(napi_env env, vt_status st, const vt_ctx* ctx) {
  if (st == VT_OK) return false;
  napi_value msg, err, code;
  const std::string text = std::string("vtwin status ") + std::to_string(st) + ": " + vt_last_error(ctx);
  napi_create_string_utf8(env, text.c_str(), NAPI_AUTO_LENGTH, &msg);
  napi_create_error(env, nullptr, msg, &err);
  napi_create_int32(env, st, &code);
  napi_set_named_property(env, err, "status", code);
  napi_throw(env, err);
  return true;
}

bool throw_arg(napi_env env, const char* what) {
  napi_throw_type_error(env, nullptr, what);
  return true;
}

struct Args {
  napi_value v[8];
  size_t n = 8;
  Args(napi_env env, napi_callback_info info) { napi_get_cb_info(env, info, &n, v, nullptr, nullptr); }
};

vt_ctx* ctx_of(napi_env env, napi_value v) {
  void* p = nullptr;
  if (napi_get_value_external(env, v, &p) != napi_ok || !p || !static_cast<Holder*>(p)->ctx) {
    napi_throw_error(env, nullptr, "vtwin: not a live renderer context");
    return nullptr;
  }
  return static_cast<Holder*>(p)->ctx;
}

bool has(napi_env env, napi_value obj, const char* name) {
  bool b = false;
  if (!obj) return false;
  napi_valuetype t;
  if (napi_typeof(env, obj, &t) != napi_ok || t != napi_object) return false;
  napi_has_named_property(env, obj, name, &b);
  if (!b) return false;
  napi_value v;
  napi_get_named_property(env, obj, name, &v);
  napi_typeof(env, v, &t);
  return t != napi_undefined && t != napi_null;
}
napi_value prop(napi_env env, napi_value obj, const char* name) {
  napi_value v = nullptr;
  napi_get_named_property(env, obj, name, &v);
  return v;
}
double num(napi_env env, napi_value obj, const char* name, double def) {
  if (!has(env, obj, name)) return def;
  double d = def;
  napi_get_value_double(env, prop(env, obj, name), &d);
  return d;
}
uint32_t u32(napi_env env, napi_value obj, const char* name, uint32_t def) { return uint32_t(num(env, obj, name, double(def))); }
bool boolean(napi_env env, napi_value obj, const char* name, bool def) {
  if (!has(env, obj, name)) return def;
  bool b = def;
  napi_value v = prop(env, obj, name);
  if (napi_get_value_bool(env, v, &b) != napi_ok) { double d = 0; napi_get_value_double(env, v, &d); b = d != 0; }
  return b;
}
uint32_t u32v(napi_env env, napi_value v) { uint32_t u = 0; napi_get_value_uint32(env, v, &u); return u; }
double f64v(napi_env env, napi_value v) { double d = 0; napi_get_value_double(env, v, &d); return d; }

// the data of a TypedArray, DataView or ArrayBuffer (null for undefined / null); bytes receives its length
void* data_of(napi_env env, napi_value v, size_t* bytes = nullptr) {
  if (bytes) *bytes = 0;
  if (!v) return nullptr;
  napi_valuetype t;
  napi_typeof(env, v, &t);
  if (t == napi_undefined || t == napi_null) return nullptr;
  bool is = false;
  void* data = nullptr;
  napi_is_typedarray(env, v, &is);
  if (is) {
    napi_typedarray_type type;
    size_t len = 0, off = 0;
    napi_value ab;
    napi_get_typedarray_info(env, v, &type, &len, &data, &ab, &off);
    size_t el = 1;
    switch (type) {
      case napi_int16_array: case napi_uint16_array: el = 2; break;
      case napi_int32_array: case napi_uint32_array: case napi_float32_array: el = 4; break;
      case napi_float64_array: case napi_bigint64_array: case napi_biguint64_array: el = 8; break;
      default: el = 1;
    }
    if (bytes) *bytes = len * el;
    return data;
  }
  napi_is_arraybuffer(env, v, &is);
  if (is) {
    size_t len = 0;
    napi_get_arraybuffer_info(env, v, &data, &len);
    if (bytes) *bytes = len;
    return data;
  }
  napi_is_dataview(env, v, &is);
  if (is) {
    size_t len = 0, off = 0;
    napi_value ab;
    napi_get_dataview_info(env, v, &len, &data, &ab, &off);
    if (bytes) *bytes = len;
    return data;
  }
  return nullptr;
}
template <typename T> T* arr(napi_env env, napi_value obj, const char* name, size_t* n = nullptr) {
  size_t b = 0;
  T* p = has(env, obj, name) ? static_cast<T*>(data_of(env, prop(env, obj, name), &b)) : nullptr;
  if (n) *n = b / sizeof(T);
  return p;
}
// a plain JS array of numbers (or a TypedArray) into out[0..k)
void numbers(napi_env env, napi_value obj, const char* name, double* out, uint32_t k) {
  if (!has(env, obj, name)) return;
  napi_value v = prop(env, obj, name);
  bool is = false;
  napi_is_array(env, v, &is);
  if (is) {
    for (uint32_t i = 0; i < k; i++) { napi_value e; napi_get_element(env, v, i, &e); out[i] = f64v(env, e); }
    return;
  }
  size_t b = 0;
  void* p = data_of(env, v, &b);
  napi_typedarray_type type = napi_float64_array;
  bool ta = false;
  napi_is_typedarray(env, v, &ta);
  if (ta) { size_t len, off; napi_value ab; void* d; napi_get_typedarray_info(env, v, &type, &len, &d, &ab, &off); }
  for (uint32_t i = 0; i < k; i++) {
    if (type == napi_float32_array && (i + 1) * 4 <= b) out[i] = static_cast<float*>(p)[i];
    else if (type == napi_float64_array && (i + 1) * 8 <= b) out[i] = static_cast<double*>(p)[i];
    else if (type == napi_uint32_array && (i + 1) * 4 <= b) out[i] = static_cast<uint32_t*>(p)[i];
  }
}
void floats(napi_env env, napi_value obj, const char* name, float* out, uint32_t k) {
  double d[16] = {0};
  for (uint32_t i = 0; i < k && i < 16; i++) d[i] = out[i];
  numbers(env, obj, name, d, k);
  for (uint32_t i = 0; i < k && i < 16; i++) out[i] = float(d[i]);
}
uint32_t length_of(napi_env env, napi_value v) { uint32_t n = 0; napi_get_array_length(env, v, &n); return n; }

napi_value typed(napi_env env, napi_typedarray_type type, size_t count, size_t el, void** data) {
  napi_value ab, out;
  napi_create_arraybuffer(env, count * el, data, &ab);
  napi_create_typedarray(env, type, count, ab, 0, &out);
  return out;
}
napi_value f64_array(napi_env env, const double* v, size_t n) {
  void* d;
  napi_value out = typed(env, napi_float64_array, n, 8, &d);
  std::memcpy(d, v, n * 8);
  return out;
}
napi_value u32_array(napi_env env, const uint32_t* v, size_t n) {
  void* d;
  napi_value out = typed(env, napi_uint32_array, n, 4, &d);
  std::memcpy(d, v, n * 4);
  return out;
}
void set_num(napi_env env, napi_value obj, const char* name, double v) { napi_value x; napi_create_double(env, v, &x); napi_set_named_property(env, obj, name, x); }
napi_value object(napi_env env) { napi_value o; napi_create_object(env, &o); return o; }

// ------------------------------------------------------------------------------------------------ scene
// The scene description (vt_scene_desc) from a JS object built by renderer.js from the welded scene:
// {static: {P, N, I, triMesh, vertMesh}, bodies: [{P, N, I, triMesh, UV?, kind, ownerCamera}], meshes: [{mat, flags,
//  buildDir, layerPeriod, layerDepth, overviewOnly}], materials: [{metallic, coated, emitter, noTable, rho, f0,
//  roughness, ior, fbar, coatIor, coatRoughness, tau, textured, inkRho, inkRoughness}], L0, profileTheta, profileP,
//  axisDeg, cameras: [{width, height, fx, fy, cx, cy, alpha, k, T_D_C}]}
struct SceneDesc {
  vt_scene_desc d{};
  std::vector<vt_body_desc> bodies;
  std::vector<vt_mesh> meshes;
  std::vector<vt_material> mats;
  std::vector<vt_camera_desc> cams;
};

bool scene_desc(napi_env env, napi_value s, SceneDesc& out) {
  vt_scene_desc& d = out.d;
  napi_value st = prop(env, s, "static");
  size_t nP = 0, nI = 0;
  d.static_P = arr<float>(env, st, "P", &nP);
  d.static_N = arr<float>(env, st, "N");
  d.static_I = arr<uint32_t>(env, st, "I", &nI);
  d.static_tri_mesh = arr<uint32_t>(env, st, "triMesh");
  d.static_vert_mesh = arr<uint32_t>(env, st, "vertMesh");
  d.n_static_verts = uint32_t(nP / 3);
  d.n_static_tris = uint32_t(nI / 3);
  if (!d.static_P || !d.static_N || !d.static_I || !d.static_tri_mesh || !d.static_vert_mesh) return !throw_arg(env, "scene.static: P, N, I, triMesh, vertMesh");
  napi_value bl = prop(env, s, "bodies");
  for (uint32_t i = 0, n = has(env, s, "bodies") ? length_of(env, bl) : 0; i < n; i++) {
    napi_value b;
    napi_get_element(env, bl, i, &b);
    vt_body_desc x{};
    size_t bp = 0, bi = 0;
    x.P = arr<float>(env, b, "P", &bp);
    x.N = arr<float>(env, b, "N");
    x.I = arr<uint32_t>(env, b, "I", &bi);
    x.tri_mesh = arr<uint32_t>(env, b, "triMesh");
    x.UV = arr<float>(env, b, "UV");
    x.n_verts = uint32_t(bp / 3);
    x.n_tris = uint32_t(bi / 3);
    x.kind = int32_t(num(env, b, "kind", VT_BODY_FIXTURE));
    x.owner_camera = int32_t(num(env, b, "ownerCamera", -1));
    if (!x.P || !x.N || !x.I || !x.tri_mesh) return !throw_arg(env, "scene.bodies[i]: P, N, I, triMesh");
    out.bodies.push_back(x);
  }
  napi_value ml = prop(env, s, "meshes");
  for (uint32_t i = 0, n = length_of(env, ml); i < n; i++) {
    napi_value m;
    napi_get_element(env, ml, i, &m);
    vt_mesh x{};
    x.mat = u32(env, m, "mat", 0);
    x.flags = u32(env, m, "flags", VT_F_STATIC);
    x.build_dir[2] = 1.0f;
    floats(env, m, "buildDir", x.build_dir, 3);
    x.layer_period = float(num(env, m, "layerPeriod", 0.0));
    x.layer_depth = float(num(env, m, "layerDepth", 0.0));
    x.overview_only = boolean(env, m, "overviewOnly", false) ? 1u : 0u;
    out.meshes.push_back(x);
  }
  napi_value al = prop(env, s, "materials");
  for (uint32_t i = 0, n = length_of(env, al); i < n; i++) {
    napi_value m;
    napi_get_element(env, al, i, &m);
    vt_material x{};
    x.metallic = int32_t(num(env, m, "metallic", 0));
    x.coated = boolean(env, m, "coated", false) ? 1 : 0;
    x.emitter = boolean(env, m, "emitter", false) ? 1 : 0;
    x.no_table = boolean(env, m, "noTable", false) ? 1 : 0;
    x.rho[0] = x.rho[1] = x.rho[2] = 0.5f;
    floats(env, m, "rho", x.rho, 3);
    x.f0[0] = 0.56f; x.f0[1] = 0.57f; x.f0[2] = 0.58f;
    floats(env, m, "f0", x.f0, 3);
    x.roughness = float(num(env, m, "roughness", 0.5));
    x.ior = float(num(env, m, "ior", 1.5));
    x.fbar = float(num(env, m, "fbar", NAN));
    x.coat_ior = float(num(env, m, "coatIor", 1.5));
    x.coat_roughness = float(num(env, m, "coatRoughness", 0.05));
    x.tau[0] = x.tau[1] = x.tau[2] = 1.0f;
    floats(env, m, "tau", x.tau, 3);
    x.textured = boolean(env, m, "textured", false) ? 1 : 0;
    floats(env, m, "inkRho", x.ink_rho, 3);
    x.ink_roughness = float(num(env, m, "inkRoughness", 0.4));
    out.mats.push_back(x);
  }
  d.L0[0] = d.L0[1] = d.L0[2] = 1.0f;
  floats(env, s, "L0", d.L0, 3);
  size_t np = 0;
  d.profile_theta = arr<float>(env, s, "profileTheta", &np);
  d.profile_p = arr<float>(env, s, "profileP");
  d.n_profile = uint32_t(np);
  d.axis_deg = float(num(env, s, "axisDeg", NAN));
  napi_value cl = prop(env, s, "cameras");
  for (uint32_t i = 0, n = has(env, s, "cameras") ? length_of(env, cl) : 0; i < n; i++) {
    napi_value c;
    napi_get_element(env, cl, i, &c);
    vt_camera_desc x{};
    x.width = u32(env, c, "width", 0);
    x.height = u32(env, c, "height", 0);
    x.fx = num(env, c, "fx", 1.0); x.fy = num(env, c, "fy", 1.0); x.cx = num(env, c, "cx", 0.0); x.cy = num(env, c, "cy", 0.0);
    x.alpha = num(env, c, "alpha", 0.0);
    numbers(env, c, "k", x.k, 4);
    numbers(env, c, "T_D_C", x.T_D_C, 16);
    out.cams.push_back(x);
  }
  d.bodies = out.bodies.data(); d.n_bodies = uint32_t(out.bodies.size());
  d.meshes = out.meshes.data(); d.n_meshes = uint32_t(out.meshes.size());
  d.materials = out.mats.data(); d.n_materials = uint32_t(out.mats.size());
  d.cameras = out.cams.data(); d.n_cameras = uint32_t(out.cams.size());
  return true;
}

// create(scene, {leafSize, albedoSamples, device}) -> context (gpu/renderer.js:202 create)
napi_value Create(napi_env env, napi_callback_info info) {
  Args a(env, info);
  SceneDesc sd;
  if (a.n < 1 || !scene_desc(env, a.v[0], sd)) return nullptr;
  vt_options o{};
  napi_value opt = a.n > 1 ? a.v[1] : nullptr;
  o.leaf_size = u32(env, opt, "leafSize", 4);
  o.albedo_samples = u32(env, opt, "albedoSamples", 1024);
  o.device = int32_t(num(env, opt, "device", 0));
  vt_ctx* ctx = nullptr;
  if (throw_status(env, vt_create(&sd.d, &o, &ctx), nullptr)) return nullptr;
  napi_value ext;
  napi_create_external(env, new Holder{ctx}, finalize_ctx, nullptr, &ext);
  return ext;
}

// destroy(ctx) (gpu/renderer.js:1278)
napi_value Destroy(napi_env env, napi_callback_info info) {
  Args a(env, info);
  void* p = nullptr;
  if (a.n >= 1 && napi_get_value_external(env, a.v[0], &p) == napi_ok && p) {
    Holder* h = static_cast<Holder*>(p);
    if (h->ctx) { vt_destroy(h->ctx); h->ctx = nullptr; }
  }
  return undefined(env);
}

// sceneInfo(ctx) -> {nodeCount, triCount, ..., emitArea}
napi_value SceneInfo(napi_env env, napi_callback_info info) {
  Args a(env, info);
  vt_ctx* ctx = ctx_of(env, a.v[0]);
  if (!ctx) return nullptr;
  vt_scene_info s{};
  if (throw_status(env, vt_scene_info_get(ctx, &s), ctx)) return nullptr;
  napi_value o = object(env);
  set_num(env, o, "nodeCount", s.node_count); set_num(env, o, "triCount", s.tri_count); set_num(env, o, "vertCount", s.vert_count);
  set_num(env, o, "staticVerts", s.static_verts); set_num(env, o, "staticTris", s.static_tris); set_num(env, o, "bodies", s.n_bodies);
  set_num(env, o, "materials", s.n_materials); set_num(env, o, "emitTris", s.emit_tris); set_num(env, o, "emitArea", s.emit_area);
  return o;
}

// setPoses(ctx, T0: Float64Array (bodies x 16, NaN hides), T1?: Float64Array) (gpu/renderer.js:620)
napi_value SetPoses(napi_env env, napi_callback_info info) {
  Args a(env, info);
  vt_ctx* ctx = ctx_of(env, a.v[0]);
  if (!ctx) return nullptr;
  size_t b0 = 0, b1 = 0;
  const double* T0 = static_cast<const double*>(data_of(env, a.v[1], &b0));
  const double* T1 = a.n > 2 ? static_cast<const double*>(data_of(env, a.v[2], &b1)) : nullptr;
  if (!T0 || (T1 && b1 != b0)) { throw_arg(env, "setPoses: Float64Array of bodies x 16 (T1 the same size)"); return nullptr; }
  throw_status(env, vt_set_poses(ctx, T0, T1, uint32_t(b0 / 128)), ctx);
  return undefined(env);
}

// setEavg(ctx, [r, g, b]) (gpu/renderer.js:848)
napi_value SetEavg(napi_env env, napi_callback_info info) {
  Args a(env, info);
  vt_ctx* ctx = ctx_of(env, a.v[0]);
  if (!ctx) return nullptr;
  float e[3] = {0, 0, 0};
  napi_value holder = object(env);
  napi_set_named_property(env, holder, "e", a.v[1]);
  floats(env, holder, "e", e, 3);
  throw_status(env, vt_set_eavg(ctx, e), ctx);
  return undefined(env);
}

// the render request of renderCamera's options (gpu/renderer.js:922 _options, :935 _submitCamera)
vt_render_req render_req(napi_env env, napi_value o, uint32_t camera) {
  vt_render_req q{};
  q.camera = camera;
  q.spp = u32(env, o, "spp", 1);
  q.light_samples = u32(env, o, "lightSamples", 4);
  q.seed = u32(env, o, "seed", 0);
  q.options = u32(env, o, "options", 0);
  q.mode = u32(env, o, "mode", VT_SHADE_TWIN);
  q.max_depth = u32(env, o, "maxDepth", 2);
  q.root = u32(env, o, "root", 0);
  q.frame = u32(env, o, "frame", 0);
  q.shutter[0] = 0.0f; q.shutter[1] = 1.0f;
  floats(env, o, "shutter", q.shutter, 2);
  q.scale = float(num(env, o, "scale", 1.0));
  q.refine = u32(env, o, "refine", 0);
  q.refine_light_samples = u32(env, o, "refineLightSamples", 0);
  return q;
}

// renderCamera(ctx, camera, opts, out?: Float32Array w*h*4) (gpu/renderer.js:975)
napi_value RenderCamera(napi_env env, napi_callback_info info) {
  Args a(env, info);
  vt_ctx* ctx = ctx_of(env, a.v[0]);
  if (!ctx) return nullptr;
  const vt_render_req q = render_req(env, a.n > 2 ? a.v[2] : nullptr, u32v(env, a.v[1]));
  float* out = a.n > 3 ? static_cast<float*>(data_of(env, a.v[3])) : nullptr;
  throw_status(env, vt_render_camera(ctx, &q, out), ctx);
  return undefined(env);
}

// renderFrame(ctx, {cameras: Uint32Array, render: opts, sensors?: Uint32Array (cameras x 64 words)}) ->
// {ms, stats: Uint32Array (cameras x 4)} (gpu/renderer.js:986)
napi_value RenderFrame(napi_env env, napi_callback_info info) {
  Args a(env, info);
  vt_ctx* ctx = ctx_of(env, a.v[0]);
  if (!ctx) return nullptr;
  size_t nc = 0, ns = 0;
  const uint32_t* cams = arr<uint32_t>(env, a.v[1], "cameras", &nc);
  const uint32_t* su = arr<uint32_t>(env, a.v[1], "sensors", &ns);
  if (!cams || (su && ns != nc * 64)) { throw_arg(env, "renderFrame: cameras Uint32Array, sensors cameras x 64 words"); return nullptr; }
  vt_frame_req f{};
  f.cameras = cams;
  f.n_cameras = uint32_t(nc);
  f.render = render_req(env, prop(env, a.v[1], "render"), 0);
  f.sensors = reinterpret_cast<const vt_sensor_uniform*>(su);
  std::vector<uint32_t> stats(nc * 4, 0);
  f.stats = stats.data();
  if (throw_status(env, vt_render_frame(ctx, &f), ctx)) return nullptr;
  napi_value o = object(env);
  set_num(env, o, "ms", f.ms);
  napi_set_named_property(env, o, "stats", u32_array(env, stats.data(), stats.size()));
  return o;
}

// readback(ctx, camera, kind (0 linear, 1 raw, 2 rgba8, 3 rgb8, 4 yuv420), bytes) -> ArrayBuffer (gpu/renderer.js:1191)
napi_value Readback(napi_env env, napi_callback_info info) {
  Args a(env, info);
  vt_ctx* ctx = ctx_of(env, a.v[0]);
  if (!ctx) return nullptr;
  const size_t bytes = size_t(f64v(env, a.v[3]));
  void* data = nullptr;
  napi_value ab;
  napi_create_arraybuffer(env, bytes, &data, &ab);
  if (throw_status(env, vt_readback(ctx, u32v(env, a.v[1]), u32v(env, a.v[2]), data, bytes), ctx)) return nullptr;
  return ab;
}

// sensor(ctx, camera, uniform: Uint32Array(64)) -> Uint32Array(4) stats (gpu/renderer.js:1092 sensor; the uniform is
// gpu/sensor.js:158 packSensorUniform's)
napi_value Sensor(napi_env env, napi_callback_info info) {
  Args a(env, info);
  vt_ctx* ctx = ctx_of(env, a.v[0]);
  if (!ctx) return nullptr;
  size_t b = 0;
  const void* su = data_of(env, a.v[2], &b);
  if (!su || b < sizeof(vt_sensor_uniform)) { throw_arg(env, "sensor: the uniform is 64 words"); return nullptr; }
  uint32_t stats[4] = {0, 0, 0, 0};
  if (throw_status(env, vt_sensor_frame(ctx, u32v(env, a.v[1]), static_cast<const vt_sensor_uniform*>(su), stats), ctx)) return nullptr;
  return u32_array(env, stats, 4);
}

// setRelativeIllumination(ctx, camera, pupilExponent, vigThetaDeg: Float64Array, vig: Float64Array)
// (gpu/sensor.js:103 relativeIlluminationMap, computed in the library)
napi_value SetRelativeIllumination(napi_env env, napi_callback_info info) {
  Args a(env, info);
  vt_ctx* ctx = ctx_of(env, a.v[0]);
  if (!ctx) return nullptr;
  size_t bt = 0, bv = 0;
  const double* th = static_cast<const double*>(data_of(env, a.v[3], &bt));
  const double* vg = static_cast<const double*>(data_of(env, a.v[4], &bv));
  throw_status(env, vt_set_relative_illumination(ctx, u32v(env, a.v[1]), nullptr, f64v(env, a.v[2]), th, vg, uint32_t(std::min(bt, bv) / 8)), ctx);
  return undefined(env);
}

// visible(ctx, camera, points: Float64Array n x 3, tol, time) -> Uint8Array (gpu/renderer.js:1238)
napi_value Visible(napi_env env, napi_callback_info info) {
  Args a(env, info);
  vt_ctx* ctx = ctx_of(env, a.v[0]);
  if (!ctx) return nullptr;
  size_t b = 0;
  const double* pts = static_cast<const double*>(data_of(env, a.v[2], &b));
  const size_t n = b / 24;
  void* d;
  napi_value out = typed(env, napi_uint8_array, n, 1, &d);
  if (throw_status(env, vt_visible(ctx, u32v(env, a.v[1]), pts, uint32_t(n), f64v(env, a.v[3]), f64v(env, a.v[4]), static_cast<uint8_t*>(d)), ctx))
    return nullptr;
  return out;
}

// project(ctx, camera, points: Float64Array n x 3) -> Float64Array n x 2 (gpu/renderer.js:1261, gpu/lens.js:43)
napi_value Project(napi_env env, napi_callback_info info) {
  Args a(env, info);
  vt_ctx* ctx = ctx_of(env, a.v[0]);
  if (!ctx) return nullptr;
  size_t b = 0;
  const double* pts = static_cast<const double*>(data_of(env, a.v[2], &b));
  const size_t n = b / 24;
  void* d;
  napi_value out = typed(env, napi_float64_array, n * 2, 8, &d);
  if (throw_status(env, vt_project(ctx, u32v(env, a.v[1]), pts, uint32_t(n), static_cast<double*>(d)), ctx)) return nullptr;
  return out;
}

// traceRays(ctx, o4: Float32Array n x 4, d4, mask, anyHit, root) -> {hits: Float32Array n x 4 (t, tri bits, inst bits,
// u), v: Float32Array} (gpu/wgsl/kernels.wgsl.js:535 traceTest)
napi_value TraceRays(napi_env env, napi_callback_info info) {
  Args a(env, info);
  vt_ctx* ctx = ctx_of(env, a.v[0]);
  if (!ctx) return nullptr;
  size_t b = 0;
  const float* o4 = static_cast<const float*>(data_of(env, a.v[1], &b));
  const float* d4 = static_cast<const float*>(data_of(env, a.v[2]));
  const size_t n = b / 16;
  void *h, *v;
  napi_value hits = typed(env, napi_float32_array, n * 4, 4, &h), vv = typed(env, napi_float32_array, n, 4, &v);
  if (throw_status(env, vt_trace_rays(ctx, o4, d4, uint32_t(n), u32v(env, a.v[3]), u32v(env, a.v[4]), u32v(env, a.v[5]), static_cast<float*>(h),
                                      static_cast<float*>(v)), ctx))
    return nullptr;
  napi_value o = object(env);
  napi_set_named_property(env, o, "hits", hits);
  napi_set_named_property(env, o, "v", vv);
  return o;
}

// unitTest(ctx, kind, tin: Float32Array, lens?: [fx, fy, cx, cy, k1..k4, alpha]) -> Float32Array
// (gpu/wgsl/kernels.wgsl.js:494-551 lensTest / bsdfTest / capsuleTest / profileTest)
napi_value UnitTest(napi_env env, napi_callback_info info) {
  Args a(env, info);
  vt_ctx* ctx = ctx_of(env, a.v[0]);
  if (!ctx) return nullptr;
  vt_unit_req q{};
  q.kind = u32v(env, a.v[1]);
  static const uint32_t slots_in[4] = {2, 4, 4, 1}, slots_out[4] = {2, 3, 1, 1};
  if (q.kind > 3) { throw_arg(env, "unitTest: kind 0..3"); return nullptr; }
  size_t b = 0;
  const float* tin = static_cast<const float*>(data_of(env, a.v[2], &b));
  q.n = uint32_t(b / 16 / slots_in[q.kind]);
  if (a.n > 3) {
    napi_value holder = object(env);
    napi_set_named_property(env, holder, "l", a.v[3]);
    floats(env, holder, "l", q.lens, 9);
  }
  void* d;
  napi_value out = typed(env, napi_float32_array, size_t(q.n) * slots_out[q.kind] * 4, 4, &d);
  if (throw_status(env, vt_unit_test(ctx, &q, tin, static_cast<float*>(d)), ctx)) return nullptr;
  return out;
}

// ------------------------------------------------------------------------------------------------ node radiosity
// nodesBuild(ctx, {gatherK, nodeSamples, nbrK, smoothSigma, smoothRadius, radiosityEvery, itersPerFrame,
// itersInitial, perStepFactors}) -> info (gpu/renderer.js:456 _buildGatherTable)
napi_value NodesBuild(napi_env env, napi_callback_info info) {
  Args a(env, info);
  vt_ctx* ctx = ctx_of(env, a.v[0]);
  if (!ctx) return nullptr;
  napi_value o = a.n > 1 ? a.v[1] : nullptr;
  vt_nodes_opts q{};
  q.gather_k = u32(env, o, "gatherK", 64);
  q.node_samples = u32(env, o, "nodeSamples", 4);
  q.nbr_k = u32(env, o, "nbrK", 16);
  q.smooth_sigma = float(num(env, o, "smoothSigma", 0.003));
  q.smooth_radius = float(num(env, o, "smoothRadius", 0.006));
  q.radiosity_every = u32(env, o, "radiosityEvery", 1);
  q.iters_per_frame = u32(env, o, "itersPerFrame", 4);
  q.iters_initial = u32(env, o, "itersInitial", 96);
  q.per_step_factors = boolean(env, o, "perStepFactors", false) ? 1u : 0u;
  vt_nodes_info s{};
  if (throw_status(env, vt_nodes_build(ctx, &q, &s), ctx)) return nullptr;
  napi_value r = object(env);
  set_num(env, r, "nodes", s.n_nodes); set_num(env, r, "activeNodes", s.n_active); set_num(env, r, "gatherK", s.gather_k);
  set_num(env, r, "nbrK", s.nbr_k); set_num(env, r, "gatherBuildMs", s.build_ms); set_num(env, r, "neighbourMs", s.neighbour_ms);
  set_num(env, r, "tableEntries", double(s.table_entries));
  return r;
}

// nodesUpdate(ctx, force) -> 'none' | 'full' | 'incremental' | 'reused' (gpu/renderer.js:771 _ensureRadiosity)
napi_value NodesUpdate(napi_env env, napi_callback_info info) {
  Args a(env, info);
  vt_ctx* ctx = ctx_of(env, a.v[0]);
  if (!ctx) return nullptr;
  bool force = false;
  if (a.n > 1) napi_get_value_bool(env, a.v[1], &force);
  uint32_t what = 0;
  if (throw_status(env, vt_nodes_update(ctx, force ? 1 : 0, &what), ctx)) return nullptr;
  static const char* names[4] = {"none", "full", "incremental", "reused"};
  napi_value s;
  napi_create_string_utf8(env, names[what & 3u], NAPI_AUTO_LENGTH, &s);
  return s;
}

// converge(ctx, iters) (gpu/renderer.js:804)
napi_value Converge(napi_env env, napi_callback_info info) {
  Args a(env, info);
  vt_ctx* ctx = ctx_of(env, a.v[0]);
  if (!ctx) return nullptr;
  throw_status(env, vt_converge(ctx, u32v(env, a.v[1])), ctx);
  return undefined(env);
}

// nodeSummary(ctx) -> {area, meanIndirect, meanDirect, meanLout, eAvg} (gpu/renderer.js:825)
napi_value NodeSummary(napi_env env, napi_callback_info info) {
  Args a(env, info);
  vt_ctx* ctx = ctx_of(env, a.v[0]);
  if (!ctx) return nullptr;
  double s[13];
  if (throw_status(env, vt_node_summary(ctx, s), ctx)) return nullptr;
  napi_value o = object(env);
  set_num(env, o, "area", s[0]);
  napi_set_named_property(env, o, "meanIndirect", f64_array(env, s + 1, 3));
  napi_set_named_property(env, o, "meanDirect", f64_array(env, s + 4, 3));
  napi_set_named_property(env, o, "meanLout", f64_array(env, s + 7, 3));
  napi_set_named_property(env, o, "eAvg", f64_array(env, s + 10, 3));
  return o;
}

// setNodeState(ctx, state: Float32Array staticVerts x 16, slot) (gpu/renderer.js:316-326)
napi_value SetNodeState(napi_env env, napi_callback_info info) {
  Args a(env, info);
  vt_ctx* ctx = ctx_of(env, a.v[0]);
  if (!ctx) return nullptr;
  throw_status(env, vt_set_node_state(ctx, static_cast<const float*>(data_of(env, a.v[1])), u32v(env, a.v[2])), ctx);
  return undefined(env);
}

// formFactorsVisible(ctx, centres, normals, areas, rays) -> Float32Array n x n (the dense F of the node transport)
napi_value FormFactorsVisible(napi_env env, napi_callback_info info) {
  Args a(env, info);
  vt_ctx* ctx = ctx_of(env, a.v[0]);
  if (!ctx) return nullptr;
  size_t b = 0;
  const float* c = static_cast<const float*>(data_of(env, a.v[1], &b));
  const size_t n = b / 12;
  void* d;
  napi_value out = typed(env, napi_float32_array, n * n, 4, &d);
  if (throw_status(env, vt_form_factors_visible(ctx, uint32_t(n), c, static_cast<const float*>(data_of(env, a.v[2])),
                                                static_cast<const float*>(data_of(env, a.v[3])), u32v(env, a.v[4]), static_cast<float*>(d)), ctx))
    return nullptr;
  return out;
}

// radiositySolve(ctx, {F, rho, E, nRhs, precision, tol, maxIters, checkEvery, reuseF, B?}) -> {B, iters, refinements,
// residual, ms, sweepMs, convertMs, converged} (B = E + diag(rho) F B; FP32, or BF16 / FP8 with FP64-residual refinement)
napi_value RadiositySolve(napi_env env, napi_callback_info info) {
  Args a(env, info);
  vt_ctx* ctx = ctx_of(env, a.v[0]);
  if (!ctx) return nullptr;
  napi_value o = a.v[1];
  size_t nr = 0, ne = 0;
  vt_solve_req q{};
  q.F = arr<float>(env, o, "F");
  q.rho = arr<float>(env, o, "rho", &nr);
  q.E = arr<float>(env, o, "E", &ne);
  q.n = uint32_t(nr);
  q.n_rhs = u32(env, o, "nRhs", 1);
  if (!q.F || !q.rho || !q.E || ne != size_t(q.n) * q.n_rhs) { throw_arg(env, "radiositySolve: F, rho (n), E (n x nRhs)"); return nullptr; }
  void* d;
  napi_value B = typed(env, napi_float32_array, ne, 4, &d);
  const float* B0 = arr<float>(env, o, "B");
  if (B0) { std::memcpy(d, B0, ne * 4); q.warm_start = 1; }
  q.B = static_cast<float*>(d);
  q.precision = u32(env, o, "precision", VT_PREC_FP32);
  q.max_iters = u32(env, o, "maxIters", 1000);
  q.check_every = u32(env, o, "checkEvery", 8);
  q.reuse_f = boolean(env, o, "reuseF", false) ? 1u : 0u;
  q.tol = num(env, o, "tol", 1e-6);
  const vt_status st = vt_radiosity_solve(ctx, &q);
  if (st != VT_ERR_NOT_CONVERGED && throw_status(env, st, ctx)) return nullptr;
  napi_value r = object(env);
  napi_set_named_property(env, r, "B", B);
  set_num(env, r, "iters", q.iters); set_num(env, r, "refinements", q.refinements); set_num(env, r, "residual", q.residual);
  set_num(env, r, "ms", q.ms); set_num(env, r, "sweepMs", q.sweep_ms); set_num(env, r, "convertMs", q.convert_ms);
  napi_value conv;
  napi_get_boolean(env, st == VT_OK, &conv);
  napi_set_named_property(env, r, "converged", conv);
  return r;
}

// ------------------------------------------------------------------------------------------------ batches
vt_batch_req batch_req(napi_env env, napi_value o, std::vector<uint32_t>& cams) {
  vt_batch_req q{};
  size_t nc = 0, np0 = 0;
  const uint32_t* c = arr<uint32_t>(env, o, "cameras", &nc);
  cams.assign(c, c + nc);
  q.cameras = cams.data();
  q.n_cameras = uint32_t(nc);
  q.n_bodies = u32(env, o, "nBodies", 0);
  q.poses0 = arr<double>(env, o, "poses0", &np0);
  q.poses1 = arr<double>(env, o, "poses1");
  q.n_poses = q.n_bodies ? uint32_t(np0 / (16 * size_t(q.n_bodies))) : 0;
  q.spp = u32(env, o, "spp", 1);
  q.light_samples = u32(env, o, "lightSamples", 1);
  q.seed = u32(env, o, "seed", 0);
  q.options = u32(env, o, "options", 0);
  q.max_depth = u32(env, o, "maxDepth", 4);
  q.shutter[0] = 0.0f; q.shutter[1] = 1.0f;
  floats(env, o, "shutter", q.shutter, 2);
  q.scale = float(num(env, o, "scale", 1.0));
  q.sensor = reinterpret_cast<const vt_sensor_uniform*>(arr<uint32_t>(env, o, "sensors"));
  q.frame0 = u32(env, o, "frame0", 0);
  q.optics_scale = float(num(env, o, "opticsScale", 1.0));
  q.use_graph = boolean(env, o, "useGraph", true) ? 1u : 0u;
  q.wave_paths = u32(env, o, "wavePaths", 0);
  return q;
}

// renderBatch(ctx, {cameras, nBodies, poses0, poses1?, spp, lightSamples, seed, options, maxDepth, shutter, scale,
// sensors?, frame0, opticsScale, useGraph, wavePaths}, rawOut?: Uint16Array, radianceOut?: Float32Array) -> stats
// (renderFrame + sensor over a sweep of setPoses)
napi_value RenderBatch(napi_env env, napi_callback_info info) {
  Args a(env, info);
  vt_ctx* ctx = ctx_of(env, a.v[0]);
  if (!ctx) return nullptr;
  std::vector<uint32_t> cams;
  const vt_batch_req q = batch_req(env, a.v[1], cams);
  uint16_t* raw = a.n > 2 ? static_cast<uint16_t*>(data_of(env, a.v[2])) : nullptr;
  float* rad = a.n > 3 ? static_cast<float*>(data_of(env, a.v[3])) : nullptr;
  vt_batch_stats s{};
  if (throw_status(env, vt_render_batch(ctx, &q, raw, rad, &s), ctx)) return nullptr;
  napi_value o = object(env);
  set_num(env, o, "ms", s.ms); set_num(env, o, "sharedPaths", double(s.shared_paths)); set_num(env, o, "pairPaths", double(s.pair_paths));
  set_num(env, o, "samples", double(s.samples)); set_num(env, o, "waves", s.waves); set_num(env, o, "graphReplayed", s.graph_replayed);
  return o;
}

// batchAutotune(ctx, request) -> {wavePaths, tile: [w, h], refill}
napi_value BatchAutotune(napi_env env, napi_callback_info info) {
  Args a(env, info);
  vt_ctx* ctx = ctx_of(env, a.v[0]);
  if (!ctx) return nullptr;
  std::vector<uint32_t> cams;
  const vt_batch_req q = batch_req(env, a.v[1], cams);
  vt_tune_row best{};
  uint32_t rows = 0;
  if (throw_status(env, vt_batch_autotune(ctx, &q, nullptr, 0, &rows, &best), ctx)) return nullptr;
  napi_value o = object(env);
  set_num(env, o, "wavePaths", best.wave_paths);
  const uint32_t tile[2] = {best.tile_w, best.tile_h};
  napi_set_named_property(env, o, "tile", u32_array(env, tile, 2));
  set_num(env, o, "refill", best.refill);
  return o;
}

// ------------------------------------------------------------------------------------------------ calibration
// calibSetup(ctx, {nNodes, lampSamples}) -> {nNodes, nMaterials, nLamps, nStaticTris}
napi_value CalibSetup(napi_env env, napi_callback_info info) {
  Args a(env, info);
  vt_ctx* ctx = ctx_of(env, a.v[0]);
  if (!ctx) return nullptr;
  vt_calib_desc d{u32(env, a.v[1], "nNodes", 4096), u32(env, a.v[1], "lampSamples", 16)};
  vt_calib_info s{};
  if (throw_status(env, vt_calib_setup(ctx, &d, &s), ctx)) return nullptr;
  napi_value o = object(env);
  set_num(env, o, "nNodes", s.n_nodes); set_num(env, o, "nMaterials", s.n_materials); set_num(env, o, "nLamps", s.n_lamps);
  set_num(env, o, "nStaticTris", s.n_static_tris);
  return o;
}

// calibForward(ctx, {cameras, spp, lightSamples, seed, maxDepth, jacobiIters, albedo: Float64Array, lamp: Float64Array,
// targets?: Float32Array, images?: Float32Array, replay, intrinsics}) -> loss
napi_value CalibForward(napi_env env, napi_callback_info info) {
  Args a(env, info);
  vt_ctx* ctx = ctx_of(env, a.v[0]);
  if (!ctx) return nullptr;
  napi_value o = a.v[1];
  size_t nc = 0;
  vt_calib_req q{};
  q.cameras = arr<uint32_t>(env, o, "cameras", &nc);
  q.n_cameras = uint32_t(nc);
  q.spp = u32(env, o, "spp", 32);
  q.light_samples = u32(env, o, "lightSamples", 1);
  q.seed = u32(env, o, "seed", 0);
  q.max_depth = u32(env, o, "maxDepth", 3);
  q.jacobi_iters = u32(env, o, "jacobiIters", 0);
  q.albedo = arr<double>(env, o, "albedo");
  q.lamp = arr<double>(env, o, "lamp");
  q.targets = arr<float>(env, o, "targets");
  q.images = arr<float>(env, o, "images");
  q.replay = boolean(env, o, "replay", false) ? 1u : 0u;
  q.intrinsics = boolean(env, o, "intrinsics", false) ? 1u : 0u;
  double loss = 0.0;
  if (throw_status(env, vt_calib_forward(ctx, &q, &loss), ctx)) return nullptr;
  napi_value r;
  napi_create_double(env, loss, &r);
  return r;
}

// calibBackward(ctx, nMaterials, nLamps, nCameras) -> {gAlbedo, gLamp, gIntrinsics (when the forward asked for it)}
napi_value CalibBackward(napi_env env, napi_callback_info info) {
  Args a(env, info);
  vt_ctx* ctx = ctx_of(env, a.v[0]);
  if (!ctx) return nullptr;
  const uint32_t nm = u32v(env, a.v[1]), nl = u32v(env, a.v[2]), nc = a.n > 3 ? u32v(env, a.v[3]) : 0;
  void *ga, *gl;
  napi_value A = typed(env, napi_float64_array, size_t(nm) * 3, 8, &ga), L = typed(env, napi_float64_array, nl, 8, &gl);
  if (throw_status(env, vt_calib_backward(ctx, static_cast<double*>(ga), static_cast<double*>(gl)), ctx)) return nullptr;
  napi_value o = object(env);
  napi_set_named_property(env, o, "gAlbedo", A);
  napi_set_named_property(env, o, "gLamp", L);
  if (nc) {
    void* gk;
    napi_value K = typed(env, napi_float64_array, size_t(nc) * 8, 8, &gk);
    if (vt_calib_intrinsics_grad(ctx, static_cast<double*>(gk)) == VT_OK) napi_set_named_property(env, o, "gIntrinsics", K);
  }
  return o;
}

// setCameraIntrinsics(ctx, camera, [fx, fy, cx, cy, k1..k4]) / getCameraIntrinsics(ctx, camera) -> Float64Array(8)
napi_value SetCameraIntrinsics(napi_env env, napi_callback_info info) {
  Args a(env, info);
  vt_ctx* ctx = ctx_of(env, a.v[0]);
  if (!ctx) return nullptr;
  double K[8] = {0};
  napi_value holder = object(env);
  napi_set_named_property(env, holder, "k", a.v[2]);
  numbers(env, holder, "k", K, 8);
  throw_status(env, vt_set_camera_intrinsics(ctx, u32v(env, a.v[1]), K), ctx);
  return undefined(env);
}
napi_value GetCameraIntrinsics(napi_env env, napi_callback_info info) {
  Args a(env, info);
  vt_ctx* ctx = ctx_of(env, a.v[0]);
  if (!ctx) return nullptr;
  double K[8];
  if (throw_status(env, vt_get_camera_intrinsics(ctx, u32v(env, a.v[1]), K), ctx)) return nullptr;
  return f64_array(env, K, 8);
}

// reprojLoss(ctx, cameras: Uint32Array, points: Float64Array n x 3, uvTargets: Float64Array cameras x n x 2 (NaN:
// unobserved)) -> {loss, gK: Float64Array cameras x 8} (gpu/lens.js:43 project with its analytic Jacobian)
napi_value ReprojLoss(napi_env env, napi_callback_info info) {
  Args a(env, info);
  vt_ctx* ctx = ctx_of(env, a.v[0]);
  if (!ctx) return nullptr;
  size_t bc = 0, bp = 0;
  const uint32_t* cams = static_cast<const uint32_t*>(data_of(env, a.v[1], &bc));
  const double* pts = static_cast<const double*>(data_of(env, a.v[2], &bp));
  const double* uv = static_cast<const double*>(data_of(env, a.v[3]));
  const uint32_t nc = uint32_t(bc / 4), np = uint32_t(bp / 24);
  void* g;
  napi_value G = typed(env, napi_float64_array, size_t(nc) * 8, 8, &g);
  double loss = 0.0;
  if (throw_status(env, vt_reproj_loss(ctx, cams, nc, pts, np, uv, &loss, static_cast<double*>(g)), ctx)) return nullptr;
  napi_value o = object(env);
  set_num(env, o, "loss", loss);
  napi_set_named_property(env, o, "gK", G);
  return o;
}

// ------------------------------------------------------------------------------------------------ lite_nodes
// liteCreate(ctx, {nsStatic, nsDyn, smRes, scopeWidth, scopeHeight, envMaterial, smThetaMaxDeg, farM, subdivH,
// subdivFixture, scopeHfovDeg, scopeCircleFrac, scopeViewDir, scopeObjective}) -> info (lite_nodes/renderer.js:491)
napi_value LiteCreate(napi_env env, napi_callback_info info) {
  Args a(env, info);
  vt_ctx* ctx = ctx_of(env, a.v[0]);
  if (!ctx) return nullptr;
  napi_value o = a.n > 1 ? a.v[1] : nullptr;
  vt_lite_opts q{};
  q.ns_static = u32(env, o, "nsStatic", 24); q.ns_dyn = u32(env, o, "nsDyn", 96); q.sm_res = u32(env, o, "smRes", 2048);
  q.scope_width = u32(env, o, "scopeWidth", 1280); q.scope_height = u32(env, o, "scopeHeight", 720);
  q.env_material = u32(env, o, "envMaterial", 0); q.debug = u32(env, o, "debug", 0);
  q.sm_theta_max_deg = num(env, o, "smThetaMaxDeg", 62.0); q.far_m = num(env, o, "farM", 1.0);
  q.subdiv_h = num(env, o, "subdivH", 0.003); q.subdiv_fixture = num(env, o, "subdivFixture", 0.01);
  q.scope_hfov_deg = num(env, o, "scopeHfovDeg", 75.0); q.scope_circle_frac = num(env, o, "scopeCircleFrac", 0.95);
  q.scope_view_dir[1] = 0.5; q.scope_view_dir[2] = 0.8660254037844386;
  numbers(env, o, "scopeViewDir", q.scope_view_dir, 3);
  numbers(env, o, "scopeObjective", q.scope_objective, 3);
  vt_lite_info s{};
  if (throw_status(env, vt_lite_create(ctx, &q, &s), ctx)) return nullptr;
  napi_value r = object(env);
  set_num(env, r, "rasterTris", s.raster_tris); set_num(env, r, "staticTris", s.static_tris); set_num(env, r, "cameras", s.n_cameras);
  set_num(env, r, "buildMs", s.build_ms);
  return r;
}

// liteRenderCamera(ctx, camera (SCOPE: the scene's camera count), out?: Float32Array) (lite_nodes/renderer.js:844)
napi_value LiteRenderCamera(napi_env env, napi_callback_info info) {
  Args a(env, info);
  vt_ctx* ctx = ctx_of(env, a.v[0]);
  if (!ctx) return nullptr;
  throw_status(env, vt_lite_render_camera(ctx, u32v(env, a.v[1]), a.n > 2 ? static_cast<float*>(data_of(env, a.v[2])) : nullptr), ctx);
  return undefined(env);
}

// liteDisplay(ctx, camera, du: Float32Array(20), prev: Uint32Array(4)) -> Uint32Array(4) stats (lite_nodes/renderer.js:892
// sensor: the display look and its luma statistics)
napi_value LiteDisplay(napi_env env, napi_callback_info info) {
  Args a(env, info);
  vt_ctx* ctx = ctx_of(env, a.v[0]);
  if (!ctx) return nullptr;
  uint32_t stats[4] = {0, 0, 0, 0};
  if (throw_status(env, vt_lite_display(ctx, u32v(env, a.v[1]), static_cast<const float*>(data_of(env, a.v[2])),
                                        static_cast<const uint32_t*>(data_of(env, a.v[3])), stats), ctx))
    return nullptr;
  return u32_array(env, stats, 4);
}

// liteReadback(ctx, camera, kind, bytes) -> ArrayBuffer (lite_nodes/renderer.js:940)
napi_value LiteReadback(napi_env env, napi_callback_info info) {
  Args a(env, info);
  vt_ctx* ctx = ctx_of(env, a.v[0]);
  if (!ctx) return nullptr;
  const size_t bytes = size_t(f64v(env, a.v[3]));
  void* data = nullptr;
  napi_value ab;
  napi_create_arraybuffer(env, bytes, &data, &ab);
  if (throw_status(env, vt_lite_readback(ctx, u32v(env, a.v[1]), int(u32v(env, a.v[2])), data, bytes), ctx)) return nullptr;
  return ab;
}

// liteInfo(ctx) -> {shadowStaticMs, shadowDynMs, cameraMs, cameraRasterMs, cameraShadeMs} (lite_nodes/renderer.js:981)
napi_value LiteInfo(napi_env env, napi_callback_info info) {
  Args a(env, info);
  vt_ctx* ctx = ctx_of(env, a.v[0]);
  if (!ctx) return nullptr;
  vt_lite_info s{};
  if (throw_status(env, vt_lite_info_get(ctx, &s), ctx)) return nullptr;
  napi_value o = object(env);
  set_num(env, o, "shadowStaticMs", s.shadow_static_ms); set_num(env, o, "shadowDynMs", s.shadow_dyn_ms);
  set_num(env, o, "cameraMs", s.camera_ms); set_num(env, o, "cameraRasterMs", s.camera_raster_ms);
  set_num(env, o, "cameraShadeMs", s.camera_shade_ms);
  return o;
}

// ------------------------------------------------------------------------------------------------ scene preparation
napi_value mesh_result(napi_env env, vt_mesh_out& m) {
  napi_value o = object(env);
  void *P, *N, *I;
  napi_value Pa = typed(env, napi_float64_array, size_t(m.n_verts) * 3, 8, &P), Na = typed(env, napi_float64_array, size_t(m.n_verts) * 3, 8, &N),
             Ia = typed(env, napi_uint32_array, m.n_idx, 4, &I);
  if (m.n_verts) { std::memcpy(P, m.P, size_t(m.n_verts) * 24); std::memcpy(N, m.N, size_t(m.n_verts) * 24); }
  if (m.n_idx) std::memcpy(I, m.I, size_t(m.n_idx) * 4);
  vt_mesh_free(&m);
  napi_set_named_property(env, o, "P", Pa);
  napi_set_named_property(env, o, "N", Na);
  napi_set_named_property(env, o, "I", Ia);
  return o;
}

// weld(P: Float32Array, N: Float32Array, I: Uint32Array, device?) -> {P, N, I} (gpu/scene_gpu.js:68); with a CUDA
// device ordinal the weld runs there (the same result)
napi_value Weld(napi_env env, napi_callback_info info) {
  Args a(env, info);
  size_t bp = 0, bi = 0;
  const float* P = static_cast<const float*>(data_of(env, a.v[0], &bp));
  const float* N = static_cast<const float*>(data_of(env, a.v[1]));
  const uint32_t* I = static_cast<const uint32_t*>(data_of(env, a.v[2], &bi));
  const int device = a.n > 3 ? int(f64v(env, a.v[3])) : -1;
  vt_mesh_out m{};
  const vt_status st = device >= 0 ? vt_weld_device(device, P, N, uint32_t(bp / 12), I, uint32_t(bi / 4), &m)
                                   : vt_weld(P, N, uint32_t(bp / 12), I, uint32_t(bi / 4), &m);
  if (throw_status(env, st, nullptr)) return nullptr;
  return mesh_result(env, m);
}

// subdivide(P: Float64Array, N: Float64Array, I: Uint32Array, h, maxPasses, device?) -> {P, N, I} (gpu/scene_gpu.js:93)
napi_value Subdivide(napi_env env, napi_callback_info info) {
  Args a(env, info);
  size_t bp = 0, bi = 0;
  const double* P = static_cast<const double*>(data_of(env, a.v[0], &bp));
  const double* N = static_cast<const double*>(data_of(env, a.v[1]));
  const uint32_t* I = static_cast<const uint32_t*>(data_of(env, a.v[2], &bi));
  const uint32_t passes = a.n > 4 ? u32v(env, a.v[4]) : 24;
  const int device = a.n > 5 ? int(f64v(env, a.v[5])) : -1;
  vt_mesh_out m{};
  const vt_status st = device >= 0 ? vt_subdivide_device(device, P, N, uint32_t(bp / 24), I, uint32_t(bi / 4), f64v(env, a.v[3]), passes, &m)
                                   : vt_subdivide(P, N, uint32_t(bp / 24), I, uint32_t(bi / 4), f64v(env, a.v[3]), passes, &m);
  if (throw_status(env, st, nullptr)) return nullptr;
  return mesh_result(env, m);
}

// benchMesh(z, extent [[x0, y0], [x1, y1]] as Float64Array(4), fine likewise, h) -> {P, N, I} (gpu/scene_gpu.js:146)
napi_value BenchMesh(napi_env env, napi_callback_info info) {
  Args a(env, info);
  const double* ext = static_cast<const double*>(data_of(env, a.v[1]));
  const double* fine = static_cast<const double*>(data_of(env, a.v[2]));
  vt_mesh_out m{};
  if (throw_status(env, vt_bench_mesh(f64v(env, a.v[0]), ext, fine, f64v(env, a.v[3]), &m), nullptr)) return nullptr;
  return mesh_result(env, m);
}

// computeNormals(P: Float32Array, I: Uint32Array) -> Float32Array (gpu/scene_gpu.js:37)
napi_value ComputeNormals(napi_env env, napi_callback_info info) {
  Args a(env, info);
  size_t bp = 0, bi = 0;
  const float* P = static_cast<const float*>(data_of(env, a.v[0], &bp));
  const uint32_t* I = static_cast<const uint32_t*>(data_of(env, a.v[1], &bi));
  void* d;
  napi_value N = typed(env, napi_float32_array, bp / 4, 4, &d);
  if (throw_status(env, vt_compute_normals(P, uint32_t(bp / 12), I, uint32_t(bi / 4), static_cast<float*>(d)), nullptr)) return nullptr;
  return N;
}

// buildBVH(pos: Float32Array, idx: Uint32Array, {leafSize, device}) -> {nodes: Uint32Array, nodeCount, order,
// maxDepth} (gpu/bvh.js:18 buildBVH: the same node words; device >= 0 builds on that CUDA device)
napi_value BuildBVH(napi_env env, napi_callback_info info) {
  Args a(env, info);
  size_t bp = 0, bi = 0;
  const float* pos = static_cast<const float*>(data_of(env, a.v[0], &bp));
  const uint32_t* idx = static_cast<const uint32_t*>(data_of(env, a.v[1], &bi));
  napi_value o = a.n > 2 ? a.v[2] : nullptr;
  const uint32_t leaf = u32(env, o, "leafSize", 4), n = uint32_t(bi / 12);
  const int device = int(num(env, o, "device", -1));
  std::vector<uint32_t> nodes(size_t(vt_bvh_capacity(n, leaf)) * 16), order(std::max(n, 1u));
  vt_bvh_result r{};
  const vt_status st = device >= 0 ? vt_bvh_build_device(device, pos, uint32_t(bp / 12), idx, n, leaf, nodes.data(), order.data(), &r)
                                   : vt_bvh_build(pos, uint32_t(bp / 12), idx, n, leaf, nodes.data(), order.data(), &r);
  if (throw_status(env, st, nullptr)) return nullptr;
  napi_value out = object(env);
  napi_set_named_property(env, out, "nodes", u32_array(env, nodes.data(), size_t(r.node_count) * 16));
  napi_set_named_property(env, out, "order", u32_array(env, order.data(), n));
  set_num(env, out, "nodeCount", r.node_count);
  set_num(env, out, "maxDepth", r.max_depth);
  return out;
}

// ------------------------------------------------------------------------------------------------ diagnostics
// debugFlags(ctx, reset) -> Uint32Array(16) (gpu/renderer.js:447)
napi_value DebugFlags(napi_env env, napi_callback_info info) {
  Args a(env, info);
  vt_ctx* ctx = ctx_of(env, a.v[0]);
  if (!ctx) return nullptr;
  bool reset = false;
  if (a.n > 1) napi_get_value_bool(env, a.v[1], &reset);
  uint32_t f[16];
  if (throw_status(env, vt_debug_flags(ctx, f, reset ? 1 : 0), ctx)) return nullptr;
  return u32_array(env, f, 16);
}

// timings(ctx) -> {renderMs, sensorMs, solveMs, traceMs, launches, nodeDirectMs, nodeJacobiMs} (gpu/renderer.js:1271)
napi_value Timings(napi_env env, napi_callback_info info) {
  Args a(env, info);
  vt_ctx* ctx = ctx_of(env, a.v[0]);
  if (!ctx) return nullptr;
  vt_timings t{};
  if (throw_status(env, vt_timings_get(ctx, &t), ctx)) return nullptr;
  napi_value o = object(env);
  set_num(env, o, "renderMs", t.render_ms); set_num(env, o, "sensorMs", t.sensor_ms); set_num(env, o, "solveMs", t.solve_ms);
  set_num(env, o, "traceMs", t.trace_ms); set_num(env, o, "launches", double(t.launches));
  set_num(env, o, "nodeDirectMs", t.node_direct_ms); set_num(env, o, "nodeJacobiMs", t.node_jacobi_ms);
  return o;
}

void add(napi_env env, napi_value exports, const char* name, napi_callback cb) {
  napi_value f;
  napi_create_function(env, name, NAPI_AUTO_LENGTH, cb, nullptr, &f);
  napi_set_named_property(env, exports, name, f);
}

}  // namespace

NAPI_MODULE_INIT() {
  add(env, exports, "create", Create);
  add(env, exports, "destroy", Destroy);
  add(env, exports, "sceneInfo", SceneInfo);
  add(env, exports, "setPoses", SetPoses);
  add(env, exports, "setEavg", SetEavg);
  add(env, exports, "renderCamera", RenderCamera);
  add(env, exports, "renderFrame", RenderFrame);
  add(env, exports, "readback", Readback);
  add(env, exports, "sensor", Sensor);
  add(env, exports, "setRelativeIllumination", SetRelativeIllumination);
  add(env, exports, "visible", Visible);
  add(env, exports, "project", Project);
  add(env, exports, "traceRays", TraceRays);
  add(env, exports, "unitTest", UnitTest);
  add(env, exports, "nodesBuild", NodesBuild);
  add(env, exports, "nodesUpdate", NodesUpdate);
  add(env, exports, "converge", Converge);
  add(env, exports, "nodeSummary", NodeSummary);
  add(env, exports, "setNodeState", SetNodeState);
  add(env, exports, "formFactorsVisible", FormFactorsVisible);
  add(env, exports, "radiositySolve", RadiositySolve);
  add(env, exports, "renderBatch", RenderBatch);
  add(env, exports, "batchAutotune", BatchAutotune);
  add(env, exports, "calibSetup", CalibSetup);
  add(env, exports, "calibForward", CalibForward);
  add(env, exports, "calibBackward", CalibBackward);
  add(env, exports, "setCameraIntrinsics", SetCameraIntrinsics);
  add(env, exports, "getCameraIntrinsics", GetCameraIntrinsics);
  add(env, exports, "reprojLoss", ReprojLoss);
  add(env, exports, "liteCreate", LiteCreate);
  add(env, exports, "liteRenderCamera", LiteRenderCamera);
  add(env, exports, "liteDisplay", LiteDisplay);
  add(env, exports, "liteReadback", LiteReadback);
  add(env, exports, "liteInfo", LiteInfo);
  add(env, exports, "weld", Weld);
  add(env, exports, "subdivide", Subdivide);
  add(env, exports, "benchMesh", BenchMesh);
  add(env, exports, "computeNormals", ComputeNormals);
  add(env, exports, "buildBVH", BuildBVH);
  add(env, exports, "debugFlags", DebugFlags);
  add(env, exports, "timings", Timings);
  return exports;
}
