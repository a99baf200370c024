/*
 * vtwin.h - C ABI of the GB300 (sm_103a) rendering hot path of the veridien dome twin.
 *
 * The reference is a WebGPU/JavaScript renderer. Each entry point below replaces one JavaScript interface of it
 * (cited as file:line of the reference project). Rules for every call:
 *   - return a vt_status (no exceptions cross the ABI); vt_last_error(ctx) describes the last failure;
 *   - caller-owned host buffers, library-owned device buffers; a pointer argument documented as "host or device"
 *     is classified by the CUDA runtime (cudaPointerGetAttributes);
 *   - one CUDA stream per context; a context is not thread-safe;
 *   - every device-side loop is bounded: a loop cap that is hit is counted (vt_debug_flags) and a bounded wait that
 *     runs out returns VT_ERR_TIMEOUT, never a hang.
 */
#ifndef VTWIN_H
#define VTWIN_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t vt_status;
enum {
  VT_OK = 0,
  VT_ERR_ARG = 1,            /* bad argument (null pointer, size out of range) */
  VT_ERR_CUDA = 2,           /* a CUDA runtime call failed */
  VT_ERR_OOM = 3,            /* device allocation failed */
  VT_ERR_TIMEOUT = 4,        /* a bounded device wait ran out */
  VT_ERR_STATE = 5,          /* call out of order (e.g. readback before render) */
  VT_ERR_UNKNOWN_CAMERA = 6, /* gpu/renderer.js:857 "unknown camera" */
  VT_ERR_TOO_MANY_BODIES = 7,/* gpu/renderer.js:655 "too many bodies" */
  VT_ERR_NO_DEVICE = 8,      /* no CUDA device: the library has no CPU fallback */
  VT_ERR_NOT_CONVERGED = 9   /* a solve stopped at max_iters above its tolerance (results are still written) */
};

#define VT_MAX_INST 24          /* gpu/wgsl/common.wgsl.js:5 MAX_INST */
#define VT_NODE_WORDS 16        /* gpu/bvh.js:11 NODE_WORDS */
#define VT_ALBEDO_BINS 32       /* gpu/scene_gpu.js:15 ALBEDO_BINS */
#define VT_MISS 0xffffffffu     /* gpu/wgsl/common.wgsl.js:32 MISS */

/* mesh flags, gpu/scene_gpu.js:14 MESH_FLAG */
enum { VT_F_STATIC = 1, VT_F_EMITTER = 2, VT_F_LAYER = 4, VT_F_BOARD = 8, VT_F_INSTRUMENT = 16, VT_F_SCOPE = 32,
       VT_F_BENCH = 64, VT_F_TEXTURED = 128 };

/* camera option bits, gpu/renderer.js:26 OPTION_BITS. VT_O_CACHE_WRITE / VT_O_CACHE_READ (either) turn on the static
 * first-hit cache of the camera (gpu/renderer.js:941-950 hitCache): each sub-sample's closest hit in the static BVH
 * is traced once and kept while the seed, the BVH root, the camera pose and lens and the pixel tiling hold (the
 * library keeps the key and fills empty entries), so later renders trace only the posed bodies for camera rays.
 * Exact: the images are the uncached ones bit for bit. VT_O_SHADOW_CACHE with the first-hit cache, in twin mode,
 * adds the static-occlusion cache (gpu/wgsl/shade.wgsl.js:270-301): per first-hit light sample on a static surface
 * whether the static scene hides it, kept while the emitter body stays where it was (the posed bodies are traced
 * every frame). The radiance is the same; as in the reference, the refinement's shadow key bit then marks pixels
 * where a posed body blocks a sample, penumbrae and uneven light samples instead of every traced shadow ray. */
enum { VT_O_CUT = 1, VT_O_AID = 2, VT_O_NO_INDIRECT = 4, VT_O_DIRECT_ONLY = 8, VT_O_LAYER = 16, VT_O_NO_CAPSULE = 32,
       VT_O_NORMALS = 64, VT_O_NO_MIS = 128, VT_O_SPEC_STATIC = 256, VT_O_PACKET = 512, VT_O_REFINE_SHADOW = 1024,
       VT_O_CACHE_WRITE = 2048, VT_O_CACHE_READ = 4096, VT_O_SHADOW_CACHE = 8192 };

/* body kinds (gpu/scene_gpu.js:218-235 bodyOfPart) */
enum { VT_BODY_INSTRUMENT = 0, VT_BODY_SCOPE = 1, VT_BODY_BOARD = 2, VT_BODY_FIXED = 3, VT_BODY_FIXTURE = 4 };

typedef struct vt_ctx vt_ctx;

/* ---------------------------------------------------------------------------------------------- scene input */

/* One row of the mesh table (gpu/scene_gpu.js:252-255; packed as at gpu/renderer.js:279-285). */
typedef struct {
  uint32_t mat;          /* material index */
  uint32_t flags;        /* VT_F_* */
  float build_dir[3];    /* FDM build direction (layer lines) */
  float layer_period;    /* m, 0 = no layer lines */
  float layer_depth;     /* m */
  uint32_t overview_only;/* 1: scene.json `overview_only` (outside the cavity: left out of its body's occlusion capsule and
                            effective albedo, gpu/scene_gpu.js:427-450, and of the raster pass, lite_nodes/renderer.js:529) */
} vt_mesh;

/* A material as gpu/bsdf.js:68 prepareMaterial receives it (values unwrapped from physics.yaml). */
typedef struct {
  int32_t metallic;       /* 0 dielectric, 1 conductor */
  int32_t coated;         /* 1 coated conductor (metallic 2) */
  int32_t emitter;        /* 1 the emitter material */
  int32_t no_table;       /* 1 no directional-albedo table (the emitter body's own material, scene_gpu.js:323) */
  float rho[3];           /* rho_d (dielectric) */
  float f0[3];            /* conductor / coated-conductor F0 */
  float roughness;        /* clamped to >= 0.02 as prepareMaterial does */
  float ior;              /* dielectric IOR */
  float fbar;             /* NaN: computed by fresnelAverage (gpu/bsdf.js:35) */
  float coat_ior, coat_roughness;
  float tau[3];           /* coat transmittance per normal pass */
  int32_t textured;       /* charuco print: ink values below (the print mask itself is a 1x1 white texture) */
  float ink_rho[3];
  float ink_roughness;
} vt_material;

/* A posed body: one BLAS built in the body frame (gpu/scene_gpu.js:316-349). */
typedef struct {
  const float* P;          /* n_verts x 3 */
  const float* N;          /* n_verts x 3 */
  const uint32_t* I;       /* n_tris x 3, indices into this body's vertices */
  const uint32_t* tri_mesh;/* n_tris mesh ids */
  const float* UV;         /* n_verts x 2, may be NULL */
  uint32_t n_verts, n_tris;
  int32_t kind;            /* VT_BODY_* */
  int32_t owner_camera;    /* camera index whose own rays skip this body (a lens front), -1 none */
} vt_body_desc;

/* A KB4 camera (scene.json cameras[]: lens {model 'kb4', K, D, size}, T_D_C), gpu/lens.js:8 lensParams. */
typedef struct {
  uint32_t width, height;
  double fx, fy, cx, cy, alpha;   /* alpha = K[0][1] / fx */
  double k[4];
  double T_D_C[16];               /* row-major 4x4: camera-to-dome */
} vt_camera_desc;

/* The welded scene (gpu/scene_gpu.js:241 prepareScene input after weld + subdivide of the static meshes). */
typedef struct {
  const float* static_P;          /* n_static_verts x 3; every static vertex is a radiosity node */
  const float* static_N;
  const uint32_t* static_I;       /* n_static_tris x 3 */
  const uint32_t* static_tri_mesh;
  const uint32_t* static_vert_mesh;
  uint32_t n_static_verts, n_static_tris;
  const vt_body_desc* bodies; uint32_t n_bodies;
  const vt_mesh* meshes; uint32_t n_meshes;
  const vt_material* materials; uint32_t n_materials;
  float L0[3];                    /* emitter radiance scale */
  const float* profile_theta;     /* radians, ascending */
  const float* profile_p;
  uint32_t n_profile;
  float axis_deg;                 /* emission axis angle from the scope shaft, NaN: the emitter's mean normal */
  const vt_camera_desc* cameras; uint32_t n_cameras;
} vt_scene_desc;

typedef struct {
  uint32_t leaf_size;    /* BVH leaf size (gpu/renderer.js:51 DEFAULTS.leafSize = 4) */
  uint32_t albedo_samples; /* VNDF samples per albedo-table bin (gpu/scene_gpu.js:197 uses 1024) */
  int32_t device;        /* CUDA device ordinal */
} vt_options;

/* gpu/renderer.js:202 TwinRenderer.create (+ gpu/scene_gpu.js:241 prepareScene without weld/subdivide). */
vt_status vt_create(const vt_scene_desc* scene, const vt_options* opts, vt_ctx** out);
/* gpu/renderer.js:1278 destroy */
vt_status vt_destroy(vt_ctx* ctx);
/* last error message of this context (static text if ctx is NULL) */
const char* vt_last_error(const vt_ctx* ctx);

/* Sizes of the packed scene: nodes (x16 words), triangles (x16 words), vertices (x8 words), params (x4 words),
 * static vertices, bodies. gpu/scene_gpu.js:461-469 (prepareScene's return value). */
typedef struct {
  uint32_t node_count, tri_count, vert_count, param_vec4s, static_verts, static_tris, n_bodies, n_materials,
           n_meshes, emit_tris;
  uint32_t mesh_off, mat_off, alb_off, prof_off, prof_n, emit_off;
  float emit_area, emit_axis[3], emit_normal[3], emit_centroid[3], emit_radius;
  int32_t shadow_skips_scope, scope_index;
} vt_scene_info;
vt_status vt_scene_info_get(const vt_ctx* ctx, vt_scene_info* out);
/* Copy the packed scene arrays to host buffers (any may be NULL): nodes, tris, verts, params. */
vt_status vt_scene_export(const vt_ctx* ctx, uint32_t* nodes, uint32_t* tris, uint32_t* verts, float* params);
/* Per-body BLAS record: root node, first triangle, triangle count, local bounds, capsules, rho_eff. */
typedef struct { uint32_t root, tri_off, tri_count; float bmin[3], bmax[3]; float cap_a[3], cap_b[3], cap_r;
                 float occ_a[3], occ_b[3], occ_r; float rho_eff; int32_t kind; } vt_blas_info;
vt_status vt_blas_info_get(const vt_ctx* ctx, uint32_t body, vt_blas_info* out);

/* --------------------------------------------------------------------------------------------------- poses */

/* gpu/renderer.js:620 setPoses(poses0, poses1). T0/T1: n_bodies column-major 4x4 (doubles), body order of the
 * scene; a NaN in T0[16*i] hides body i (no pose). T1 may be NULL (= T0). Writes the scene uniform
 * (gpu/renderer.js:642 _writeSceneU). */
vt_status vt_set_poses(vt_ctx* ctx, const double* T0, const double* T1, uint32_t n_bodies);
/* Mean dome irradiance eAvg (rgb) read by a posed body's second bounce (gpu/renderer.js:848-850). */
vt_status vt_set_eavg(vt_ctx* ctx, const float eavg[3]);
/* Copy the packed scene uniform (96 + 24 x 192 bytes, gpu/renderer.js:28) to the host. */
vt_status vt_scene_uniform_get(const vt_ctx* ctx, void* out, size_t bytes);

/* Node radiosity state (16 floats per static vertex: E_free|V, Ls slot 1, Ls slot 2, B_dir|vis; gpu/renderer.js
 * :316-326) and the latest slot (scene uniform info.z). state: host or device, n_static_verts x 16 floats. */
vt_status vt_set_node_state(vt_ctx* ctx, const float* state, uint32_t slot);

/* -------------------------------------------------------------------------------------------- ray queries */

/* gpu/wgsl/kernels.wgsl.js:535 traceTest / gpu/wgsl/trace.wgsl.js:297 traceScene: n rays, o4 = (x, y, z, time),
 * d4 = (dx, dy, dz, -); mask 1 static, 2 posed bodies, 3 both; out4 = (t, tri bits, inst bits, u) and out_v = v.
 * Buffers are host or device. root: static BVH root (0 = full). Miss: t = 1e30, tri = inst = VT_MISS. */
vt_status vt_trace_rays(vt_ctx* ctx, const float* o4, const float* d4, uint32_t n, uint32_t mask, uint32_t any_hit,
                        uint32_t root, float* out4, float* out_v);

/* gpu/wgsl/kernels.wgsl.js:494-551 lensTest / bsdfTest / capsuleTest / profileTest: one of the renderer's device
 * functions on n caller cases, in the reference's float4 slots (TestU.la, lb, lc = lens[0..3], lens[4..7],
 * lens[8..11]: (fx, fy, cx, cy), (k1..k4), (alpha, -, -, -)).
 *   VT_UNIT_LENS     in 2n slots: (u, v, -, -) x n, then (x, y, z, -) x n;
 *                    out 2n: (kb4Unproject(u, v), 0), (kb4Project(x, y, z), 0, 0) per case
 *   VT_UNIT_BSDF     in 4n: n, l, v, (u0, u1, u2, material index of the context's scene);
 *                    out 3n: (evalBSDF, pdfBSDF(v -> l)), sampleBSDF (l, pdf) or 0,
 *                    (albedoSpec(material, n.v), layerNormal(n, 0.1 l, normalize(v + (0.3, 0.1, 0.2)), 2e-4, 2e-5).x);
 *                    a material index beyond the scene's gives NaN
 *   VT_UNIT_CAPSULE  in 4n: p, n, (a, r), b; out n: (capsuleOcc, 0, 0, 0)
 *   VT_UNIT_PROFILE  in n: (theta, -, -, -); out n: (p(theta) of the scene's emitter, 0, 0, 0)
 * Buffers are host or device; n <= 2^24. traceTest is vt_trace_rays. */
enum { VT_UNIT_LENS = 0, VT_UNIT_BSDF = 1, VT_UNIT_CAPSULE = 2, VT_UNIT_PROFILE = 3 };
typedef struct {
  uint32_t kind, n;
  float lens[12];
} vt_unit_req;
vt_status vt_unit_test(vt_ctx* ctx, const vt_unit_req* q, const float* in, float* out);

/* gpu/renderer.js:1238 visible(name, pointsD, {tol, time}): occlusion from the camera centre to each point.
 * pts: n x 3 doubles (host); out: n bytes (1 visible). Traced on the device. */
vt_status vt_visible(vt_ctx* ctx, uint32_t camera, const double* pts, uint32_t n, double tol, double time,
                     uint8_t* out);

/* gpu/renderer.js:1261 project(name, pointsD): KB4 projection in float64 (gpu/lens.js:43). uv: n x 2. */
vt_status vt_project(vt_ctx* ctx, uint32_t camera, const double* pts, uint32_t n, double* uv);

/* ----------------------------------------------------------------------------------------------- rendering */

enum { VT_SHADE_TWIN = 0,   /* gpu/wgsl/shade.wgsl.js:250 shadeHit: direct light + node radiosity (depth 2) */
       VT_SHADE_PATH = 1 }; /* unidirectional path tracing to max_depth: NEE + BSDF continuation, power-heuristic MIS */

/* gpu/renderer.js:975 renderCamera(name, {spp, refine, lightSamples, seed, shutter, exactShadows, ...}). */
typedef struct {
  uint32_t camera;         /* camera index */
  uint32_t spp;            /* sub-samples per pixel (1..4096) */
  uint32_t light_samples;  /* emitter samples per sub-sample (1..16) */
  uint32_t seed;
  uint32_t options;        /* VT_O_* */
  uint32_t mode;           /* VT_SHADE_* */
  uint32_t max_depth;      /* path vertices (VT_SHADE_PATH); 2 for VT_SHADE_TWIN */
  uint32_t root;           /* static BVH root (0 = full) */
  uint32_t frame;          /* frame counter (scene uniform info.w) */
  float shutter[2];        /* exposure open/close in [0, 1] between poses0 and poses1 */
  float scale;             /* output scale (gpu/renderer.js:888 _packCam expo.z; 1) */
  uint32_t refine;         /* pass-2 extra sub-samples (0..64) on edge, posed-body and (VT_O_REFINE_SHADOW) shadowed
                              pixels, continuing the same sequences (gpu/wgsl/kernels.wgsl.js:218 camRefine) */
  uint32_t refine_light_samples; /* emitter samples per pass-2 sub-sample (0: light_samples) */
} vt_render_req;

/* Render one camera into its device radiance image (rgba32f, w x h; alpha 0 where every sub-sample missed).
 * out_rgba: NULL (stay on the device) or a host/device buffer of w*h*4 floats receiving a copy. */
vt_status vt_render_camera(vt_ctx* ctx, const vt_render_req* req, float* out_rgba);

/* gpu/renderer.js:1191 readback(name, 'linear'|'raw'|'rgba8'|'rgb8'|'yuv420'): copy a camera's last radiance
 * (rgba32f), raw DN image (f32), 8-bit RGB (4 or 3 bytes per pixel) or YCbCr 4:2:0 planes (Y w x h, then Cb and Cr
 * ceil(w/2) x ceil(h/2), one byte per sample) into a host buffer of `bytes`. The 8-bit kinds need vt_sensor_frame. */
enum { VT_READ_LINEAR = 0, VT_READ_RAW = 1, VT_READ_RGBA8 = 2, VT_READ_RGB8 = 3, VT_READ_YUV420 = 4 };
vt_status vt_readback(vt_ctx* ctx, uint32_t camera, uint32_t kind, void* out, size_t bytes);

/* ------------------------------------------------------------------------------------------------- sensor */

/* The sensor uniform, gpu/sensor.js:158 packSensorUniform (the 256-byte SensU of gpu/wgsl/sensor.wgsl.js:20-32). */
typedef struct { uint32_t words[64]; } vt_sensor_uniform;

/* gpu/wgsl/sensor.wgsl.js:177 sensorExpose: irradiance image (rgba32f, host or device, w x h as the uniform says)
 * -> raw DN (f32, host or device). Vertical optics blur, CFA site, Poisson shot + Gaussian read noise, full well,
 * gain, black level, ADC. Veiling glare is off (fraction must be 0). */
vt_status vt_sensor_expose(vt_ctx* ctx, const vt_sensor_uniform* su, const float* irradiance, float* raw);
/* gpu/renderer.js:1092 sensor(name, opts) for the expose stage: the camera's last radiance (scaled by
 * `optics_scale`, the pi T / (4 N^2) x RI factor, 1 for the configs' unit-radiance sensor) -> its raw DN image. */
vt_status vt_sensor_camera(vt_ctx* ctx, uint32_t camera, const vt_sensor_uniform* su, float optics_scale);

/* gpu/renderer.js:1141 sensor(name, opts) (the passes of :1074 _encodeSensor, gpu/wgsl/sensor.wgsl.js): the whole
 * chain on the camera's last radiance. sensorOptics (E = L pi T / (4 N^2) RI, horizontal optics blur), veiling glare
 * on a 1/F level when its fraction is > 0, sensorExpose (vertical blur, glare mix, raw DN), demosaic (bilinear,
 * edge-aware or Hamilton-Adams), white balance and CCM, noise reduction (3x3 bilateral), sensorOutput (tone curve,
 * unsharp mask, BT.601 YCbCr with 4:2:0 or 4:4:4 chroma, 8-bit RGB). stats (may be NULL): the sum of the 8-bit luma
 * (AE) and the raw channel sums R, G, B of the black-subtracted values x 1023 (AWB), as the reference's stats
 * buffer. The relative illumination map is the one set by vt_set_relative_illumination (else computed with
 * pupil exponent 1 and no vignetting). */
vt_status vt_sensor_frame(vt_ctx* ctx, uint32_t camera, const vt_sensor_uniform* su, uint32_t stats[4]);
/* gpu/sensor.js:98 relativeIlluminationMap: relative illumination x vignetting per pixel of a camera (w x h floats),
 * cos^q(theta) sin(theta) / (theta_d dtheta_d/dtheta) from its KB4 lens in FP64 times the vignetting table (n_vig
 * knots, theta in degrees, linear between), computed when ri is NULL, else copied (host or device). */
vt_status vt_set_relative_illumination(vt_ctx* ctx, uint32_t camera, const float* ri, double pupil_exponent, const double* vig_theta_deg,
                                       const double* vig, uint32_t n_vig);
vt_status vt_get_relative_illumination(vt_ctx* ctx, uint32_t camera, float* ri);

/* gpu/renderer.js:986 renderFrame({cameras, sensor}): every listed camera rendered with `render` (its camera field
 * ignored; in twin mode the node radiosity is brought up to the poses first), then, when `sensors` is set, each
 * camera's sensor chain (vt_sensor_frame) with its uniform; everything queued on the context's stream with one
 * synchronisation at the end. stats (n_cameras x 4, may be NULL) receives each camera's AE / AWB statistics; ms the
 * frame's device time. Radiance, raw and 8-bit images stay on the device for vt_readback. */
typedef struct {
  const uint32_t* cameras;
  uint32_t n_cameras;
  vt_render_req render;
  const vt_sensor_uniform* sensors;   /* n_cameras uniforms, or NULL: no sensor stage */
  uint32_t* stats;
  double ms;                          /* out */
} vt_frame_req;
vt_status vt_render_frame(vt_ctx* ctx, vt_frame_req* frame);

/* -------------------------------------------------------------------------------------- batched rendering */

/* Many cameras x many kinematic poses of one scene in one call: the twin's renderFrame (gpu/renderer.js:986) over
 * a sweep of setPoses (gpu/renderer.js:620), with the sensor's expose stage (gpu/wgsl/sensor.wgsl.js:177) applied
 * to every frame. Frame (camera c, pose q) is identical to vt_set_poses(poses0[q], poses1[q]), vt_render_camera
 * (mode VT_SHADE_PATH, the request's spp / light_samples / seed / max_depth / shutter / scale) and, with a sensor,
 * vt_sensor_camera with the uniform's frame word set to frame0 + q (DN stored as uint16).
 * The common part of the scene is traced once per path for all poses; the (path, pose) pairs that may reach a
 * body whose pose varies across the batch are re-traced under their own pose. The body that carries the emitter
 * must keep one pose across the batch. Launches are captured in a CUDA graph and replayed while the request's
 * shapes repeat (use_graph = 1). */
#define VT_BATCH_MAX_POSES 64
typedef struct {
  const uint32_t* cameras;        /* n_cameras camera indices */
  uint32_t n_cameras;
  uint32_t n_poses;               /* pose sets, 1..VT_BATCH_MAX_POSES */
  uint32_t n_bodies;              /* bodies per pose set (as vt_set_poses) */
  const double* poses0;           /* n_poses x n_bodies x 16: column-major body transforms at exposure open */
  const double* poses1;           /* the same at exposure close, or NULL (= poses0) */
  uint32_t spp;                   /* sub-samples per pixel (1..4096) */
  uint32_t light_samples;         /* 1..16 */
  uint32_t seed;
  uint32_t options;               /* VT_O_* */
  uint32_t max_depth;             /* path vertices (1..64) */
  float shutter[2];
  float scale;                    /* output scale (1) */
  const vt_sensor_uniform* sensor;/* n_cameras uniforms (sizes as the cameras), or NULL: no raw frames */
  uint32_t frame0;                /* pose q exposes sensor frame frame0 + q */
  float optics_scale;             /* as vt_sensor_camera (1 for a unit-radiance sensor) */
  uint32_t use_graph;             /* 1: capture / replay the launch sequence as a CUDA graph */
  uint32_t wave_paths;            /* shared paths per wave (0: the tuned or default size) */
} vt_batch_req;
typedef struct {
  double ms;                      /* device time of the batch */
  uint64_t shared_paths;          /* camera paths traced for all poses at once */
  uint64_t pair_paths;            /* (path, pose) pairs re-traced under their own pose */
  uint64_t samples;               /* camera samples delivered: n_cameras x n_poses x w x h x spp */
  uint32_t waves, graph_replayed, reruns, vary_mask;
} vt_batch_stats;
/* raw_out: NULL, or host/device uint16 frames [camera][pose][h][w] (needs req->sensor); radiance_out: NULL, or
 * host/device rgba32f frames [camera][pose][h][w]. stats may be NULL. */
vt_status vt_render_batch(vt_ctx* ctx, const vt_batch_req* req, uint16_t* raw_out, float* radiance_out, vt_batch_stats* stats);

/* Autotuner of the batched renderer: times each candidate (wave size x pixel tile, then the traversal lanes' refill
 * threshold) on the request cut to min(spp, 4) sub-samples and its first 8 poses, and keeps the fastest in the
 * context for later batches with wave_paths = 0; the refill threshold also applies to vt_render_camera (results do
 * not depend on any of these choices).
 * table (may be NULL): up to max_rows rows of (wave_paths, tile_w, tile_h, ms per million shared paths, refill). */
typedef struct { uint32_t wave_paths, tile_w, tile_h; float ms_per_mpath; uint32_t refill; } vt_tune_row;
vt_status vt_batch_autotune(vt_ctx* ctx, const vt_batch_req* req, vt_tune_row* table, uint32_t max_rows, uint32_t* n_rows,
                            vt_tune_row* best);

/* ------------------------------------------------------------------------------ differentiable calibration */

/* No counterpart in the reference, which differentiates nothing (it has only the analytic dtheta_d/dtheta of
 * gpu/lens.js:25). A forward/backward pair for calibrating the twin from camera images:
 *
 *   image model  per camera sub-sample (the path tracer's KB4 rays and sample numbers), up to max_depth vertices on
 *                Lambertian surfaces: nL emitter samples per vertex (area CDF, power-heuristic MIS), cosine-weighted
 *                continuation, and at the last vertex the node radiosity's light rho/pi x H(node), H = F B;
 *   radiosity    n nodes (clusters of the static triangles), B = rho_node o (D L + F B) per colour channel: D the
 *                direct transfer from each emitter triangle (visibility through the BVH), L the emitter triangles'
 *                radiances, F the node form factors; `jacobi_iters` Jacobi sweeps;
 *   loss         mean over pixels and channels of (I - T)^2 against per-camera target images (FP64 reduction).
 *
 * The backward differentiates every path (path-replay backpropagation: from its record kept by a wavefront forward,
 * or, when the records do not fit, by shading the paths again in chunks of sub-samples through the same wavefront
 * kernels, from each path's hit triangles and shadow outcomes kept by the forward, 24 B per path; with the
 * environment variable VT_CALIB_RETRACE=1, or when those do not fit either, by tracing them again) and solves the
 * transposed radiosity
 * system lambda = F^T (g_H + rho o lambda) for the nodes' share. Parameters: per-material albedo (RGB, all
 * in (0, 1]) and per-emitter-triangle radiance. KB4 intrinsics enter through vt_reproj_loss (analytic Jacobians)
 * and, with `intrinsics` set, through the image term: forward-mode tangents of each path's primary ray chained
 * through the KB4 inverse (vt_calib_intrinsics_grad). The image's dependence through visibility edges (a hit or a
 * shadow outcome that changes with the ray) is not differentiated. */
typedef struct {
  uint32_t n_nodes;       /* radiosity nodes (<= static triangles), e.g. 4096 */
  uint32_t lamp_samples;  /* points per (node, emitter triangle) for D, e.g. 16 */
} vt_calib_desc;
typedef struct { uint32_t n_nodes, n_materials, n_lamps, n_static_tris; } vt_calib_info;
vt_status vt_calib_setup(vt_ctx* ctx, const vt_calib_desc* desc, vt_calib_info* info);
/* The calibration model's node data for checking (any pointer may be NULL): centres, normals (n x 3), areas (n),
 * node materials (n), node of each static triangle slot, F (n x n), D (n x n_lamps). */
vt_status vt_calib_export(vt_ctx* ctx, float* centres, float* normals, float* areas, uint32_t* node_mat, uint32_t* tri_node, float* F,
                          float* D);
typedef struct {
  const uint32_t* cameras;
  uint32_t n_cameras;
  uint32_t spp, light_samples, seed, max_depth;  /* light_samples 1..4, max_depth 1..4 */
  uint32_t jacobi_iters;                          /* radiosity sweeps, forward and adjoint (0: 96) */
  const double* albedo;                           /* n_materials x 3 */
  const double* lamp;                             /* n_lamps */
  const float* targets;                           /* rgba32f target images of the cameras, concatenated; NULL: keep the last */
  float* images;                                  /* optional out: the rendered images, same layout (host or device) */
  uint32_t replay;                                /* 0: the forward keeps each path's record (160 B) when they fit in half
                                                     the free device memory, and replays otherwise; 1: replay: the paths
                                                     are traced in chunks of sub-samples whose records fit a quarter of
                                                     the free memory (the same kernels and images as the stored form),
                                                     keeping their hits and shadow outcomes; the backward shades each
                                                     chunk again from those and differentiates it before the next;
                                                     1 + c: replay in chunks of at most c sub-samples */
  uint32_t intrinsics;                            /* 1: the backward also gives the image loss's derivative in each
                                                     camera's KB4 intrinsics (vt_calib_intrinsics_grad); the stored form
                                                     then keeps a derivative record per path (320 B) beside its record */
} vt_calib_req;
/* Image loss of the request (and the images). Keeps the state the backward replays. */
vt_status vt_calib_forward(vt_ctx* ctx, const vt_calib_req* req, double* loss);
/* Gradient of the last forward's image loss: g_albedo (n_materials x 3), g_lamp (n_lamps). */
vt_status vt_calib_backward(vt_ctx* ctx, double* g_albedo, double* g_lamp);
/* The last backward's derivative of the image loss in the intrinsics (fx, fy, cx, cy, k1..k4) of each camera of the
 * forward, in the request's camera order (n_cameras x 8), when that forward set `intrinsics`. It follows every path's
 * smooth dependence on its primary ray: the hit points, the interpolated normals, the light samples' distances,
 * cosines, MIS weights and emission profile, the cosine-sampled continuations, the emitter hit's MIS weight, chained
 * through the KB4 inverse (gpu/lens.js:25 distortDeriv). Where a path changes in steps (the triangle a ray hits, a
 * shadow ray's outcome, a node's radiosity) the step is not differentiated. No counterpart in the reference. */
vt_status vt_calib_intrinsics_grad(vt_ctx* ctx, double* g_K);
/* For checking the intrinsics' derivative: the discrete decisions of the stored forward's paths of the camera at
 * `slot` of the request (stored form with `intrinsics` = 1), per path in (row, column, sub-sample) order:
 * tri_inst 4 x (triangle, instance) of each bounce (VT_MISS: none), q 4 x 4 light-sample weights of each vertex
 * (0: occluded or no contribution). Host or device buffers. */
vt_status vt_calib_export_paths(vt_ctx* ctx, uint32_t slot, uint32_t* tri_inst, float* q);
/* KB4 intrinsics of a camera: fx, fy, cx, cy, k1..k4 (gpu/lens.js:8 lensParams; skew stays). */
vt_status vt_set_camera_intrinsics(vt_ctx* ctx, uint32_t camera, const double K[8]);
vt_status vt_get_camera_intrinsics(const vt_ctx* ctx, uint32_t camera, double K[8]);
/* Reprojection loss of n_pts dome-frame points in the cameras (gpu/lens.js:43 project, FP64): mean over the observed
 * (camera, point) pairs and both coordinates of (uv - uv_target)^2, uv_target n_cameras x n_pts x 2 (NaN: not
 * observed by that camera); g_K (n_cameras x 8) its gradient with respect to each camera's (fx, fy, cx, cy, k1..k4)
 * by the analytic KB4 Jacobian. */
vt_status vt_reproj_loss(vt_ctx* ctx, const uint32_t* cameras, uint32_t n_cameras, const double* pts, uint32_t n_pts, const double* uv_target,
                         double* loss, double* g_K);

/* -------------------------------------------------------------------------------------- node radiosity */

enum { VT_PREC_FP32 = 0, VT_PREC_BF16 = 1, VT_PREC_FP8 = 2,
       VT_PREC_FP32_TMA = 3 };  /* FP32, one right-hand side, n % 4 == 0: F fed to shared memory by bulk copies */

/* Dense node radiosity B = E + diag(rho) F B (the lite_nodes / TwinRenderer Jacobi, gpu/wgsl/kernels.wgsl.js
 * :416-461 jacobiGather + jacobiUpdate with Lambertian nodes, gpu/renderer.js:729 _submitJacobi, :804 converge).
 * FP32: plain Jacobi sweeps on CUDA cores. BF16 / FP8 (E4M3, per-row scales of F, per-column scales of the iterate):
 * tcgen05 GEMM sweeps with FP32 accumulation solve for a correction, recovered by iterative refinement on an accurate
 * residual r = E + rho F B - B (F and B split into bf16 high and low parts, FP64 epilogue). BF16/FP8 need n % 16 == 0
 * and keep converted copies of F in the context (2 x n^2 x 2 B, plus n^2 B for FP8). `iters` counts low-precision
 * sweeps and `refinements` accurate residuals. */
typedef struct {
  uint32_t n;              /* nodes */
  uint32_t n_rhs;          /* right-hand sides (columns of E and B) */
  const float* F;          /* n x n row-major, host or device */
  const float* rho;        /* n */
  const float* E;          /* n x n_rhs row-major */
  float* B;                /* n x n_rhs row-major out (in: warm start when warm_start = 1) */
  uint32_t precision;      /* VT_PREC_* */
  uint32_t max_iters;      /* total sweeps */
  uint32_t warm_start;
  uint32_t check_every;    /* sweeps between convergence checks (0 = 8) */
  uint32_t reuse_f;        /* 1: F is the matrix of this context's previous BF16/FP8 solve: reuse its converted copies */
  double tol;              /* relative residual ||r|| / ||B|| (Frobenius over all right-hand sides) */
  /* outputs */
  uint32_t iters;          /* sweeps done */
  uint32_t refinements;    /* accurate residuals evaluated */
  double residual;         /* final relative residual (accurate) */
  double ms;               /* device time of the solve (CUDA events) */
  double sweep_ms;         /* mean device time of one GEMM launch of a sweep (BF16/FP8: the tcgen05 kernel) */
  double convert_ms;       /* BF16/FP8: device time of converting F (hi/lo split, FP8 rows; 0 when reused), not in ms */
} vt_solve_req;
vt_status vt_radiosity_solve(vt_ctx* ctx, vt_solve_req* req);

/* Dense form factors of n patches (centres, normals, areas; host or device, float32): the disk approximation
 * F_ij = A_j max(0, n_i.w) max(0, -n_j.w) / (pi r^2 + A_j), F_ii = 0, rows scaled to sum <= 1. F: device or host
 * n x n row-major. Unoccluded (the scene's visibility is not applied). */
vt_status vt_form_factors(vt_ctx* ctx, uint32_t n, const float* centres, const float* normals, const float* areas,
                          float* F);
/* The same with visibility through the context's scene (static BVH and posed bodies at their current poses, the
 * emitter body not occluding): F_ij x V_ij, V_ij the fraction of `rays` (1..255) stratified rays between the two
 * patch discs (half radius, lifted 5 mm + a tenth of it) that nothing blocks, then rows scaled to <= 1; n <= 65535
 * (gpu/wgsl/kernels.wgsl.js:271 gatherDir, dense). */
vt_status vt_form_factors_visible(vt_ctx* ctx, uint32_t n, const float* centres, const float* normals, const float* areas, uint32_t rays,
                                  float* F);

/* One-right-hand-side node radiosity (B = E + diag(rho) F B, plain FP32 Jacobi as vt_radiosity_solve) that allocates
 * no device memory. No counterpart in the reference. For callers that cannot allocate while they run: a per-frame
 * loop with a fixed time budget (cudaMalloc/cudaFree may synchronise the device) or a host that sizes all its device
 * memory up front. F (n x n), rho (n), E (n) and B (n, out) are device pointers the caller owns; scratch is a static
 * device array of VT_STATIC_SOLVE_MAX_N nodes (about 160 KB) that every GPU loading the library holds until exit.
 * n > VT_STATIC_SOLVE_MAX_N or a host pointer returns VT_ERR_ARG. The first call on a device looks up the array's
 * device address. All calls share the array: calls that overlap on the GPU race. stream: a cudaStream_t (NULL =
 * legacy default stream). iters / residual may be NULL. */
#define VT_STATIC_SOLVE_MAX_N 16384
vt_status vt_radiosity_solve_static(const float* F, const float* rho, const float* E, float* B, uint32_t n, uint32_t max_iters,
                                    uint32_t check_every, double tol, void* stream, uint32_t* iters, double* residual);

/* ------------------------------------------------------------------------------- scene node radiosity */
/* The twin's own node radiosity, the producer of the node state the camera shading reads (gpu/renderer.js:456
 * _buildGatherTable, :713 _submitNodeDirect, :730 _submitJacobi, :771 _ensureRadiosity, :804 converge, :825
 * nodeSummary; gpu/wgsl/kernels.wgsl.js:271-461). Nodes are the static vertices. The gather table holds, per node,
 * the nearest node hit by each of K cosine-distributed rays (MISS for an escape or a back face); nodes with at most
 * K/2 escapes are active. Each update computes the direct light of the active nodes (node_samples emitter samples
 * with shadow rays) and Jacobi steps of the separable transport, smoothed over same-facing neighbours. */
typedef struct {
  uint32_t gather_k;        /* gather rays per node (gpu/renderer.js:38, 64; 1..1024) */
  uint32_t node_samples;    /* emitter samples per node per update (4) */
  uint32_t nbr_k;           /* smoothing neighbours kept per node (16; 1..64) */
  float smooth_sigma;       /* Gaussian sigma of the smoothing (m, 0.003; 0: no smoothing) */
  float smooth_radius;      /* neighbours within this distance (m, 0.006) */
  uint32_t radiosity_every; /* update on every n-th pose change (1) */
  uint32_t iters_per_frame; /* Jacobi steps per update (4) */
  uint32_t iters_initial;   /* Jacobi steps of the first solve, 8 at once and the rest spread over updates (96) */
  uint32_t per_step_factors;/* 0: each landing ray's transport factor is evaluated once per build into a table of
                               16 B per ray (a Jacobi gather is then a sparse product); 1: evaluated in every step */
} vt_nodes_opts;
typedef struct {
  uint32_t n_nodes;         /* static vertices */
  uint32_t n_active;
  uint32_t gather_k, nbr_k;
  double build_ms;          /* gather table: build, count, remap (device time) */
  double neighbour_ms;      /* smoothing neighbours (host) */
  uint64_t table_entries;   /* landing rays in the transport table (0: factors evaluated per step) */
} vt_nodes_info;
/* Build the gather table, the active list and the neighbours (static BVH only); node state reset to its initial
 * values. Afterwards renders run vt_nodes_update first (like renderCamera), until vt_set_node_state. opts NULL =
 * defaults. info may be NULL. */
vt_status vt_nodes_build(vt_ctx* ctx, const vt_nodes_opts* opts, vt_nodes_info* info);
/* Direct light at the active nodes at mid-exposure; moved != 0: only nodes whose segment to the emitter passes near
 * a body of the mask, where it is now or where it was at the last full update. */
vt_status vt_nodes_direct(vt_ctx* ctx, uint32_t moved);
/* `iters` Jacobi steps (gather, then update, ping-pong of the Ls slots 1 and 2). */
vt_status vt_nodes_jacobi(vt_ctx* ctx, uint32_t iters);
/* _ensureRadiosity: bring the node radiosity up to the current poses (nothing when they did not change, an
 * incremental update when only bodies other than the emitter moved, else a full one). what (may be NULL): 0 nothing
 * to do, 1 full, 2 incremental, 3 reused (poses set but nothing moved). */
vt_status vt_nodes_update(vt_ctx* ctx, int force, uint32_t* what);
/* converge(iters): the direct light if the poses changed since, then `iters` Jacobi steps, then the node summary
 * (eAvg written to the scene uniform). */
vt_status vt_converge(vt_ctx* ctx, uint32_t iters);
/* nodeSummary: area-weighted means over the active nodes of the indirect irradiance (E_free V), the direct
 * irradiance (B_dir / hh) and Ls x hh; eAvg = indirect + direct, also written to the scene uniform. out: area,
 * mean_indirect[3], mean_direct[3], mean_lout[3], eavg[3]. */
vt_status vt_node_summary(vt_ctx* ctx, double out[13]);
/* Copies of the node radiosity's tables: gtable n_nodes x gather_k, active n_active, nbr n_active x nbr_k x 2 words
 * (active index, float weight bits; weight 0 ends a list), misses n_nodes. Any pointer may be NULL. */
vt_status vt_nodes_export(vt_ctx* ctx, uint32_t* gtable, uint32_t* active, uint32_t* nbr, float* misses);
/* The node state (n_nodes x 16 floats) and its latest slot. */
vt_status vt_get_node_state(vt_ctx* ctx, float* state, uint32_t* slot);

/* The bounded-wait path of the device pipelines (the tcgen05 and bulk-copy ring buffers), exercised on purpose:
 * one block waits on an mbarrier phase for at most `cycles` SM clocks (1 .. 2^36); with arrive = 1 the phase
 * completes and the call returns VT_OK, with arrive = 0 nothing arrives, the wait runs out and the call returns
 * VT_ERR_TIMEOUT with the context still usable. No counterpart in the reference (its device waits are the
 * browser's). */
vt_status vt_wait_check(vt_ctx* ctx, uint64_t cycles, int arrive);

/* ------------------------------------------------------------------- lite_nodes: the raster camera pass */

/* lite_nodes/renderer.js: a raster live renderer that keeps the node radiosity (vt_nodes_*) and replaces the camera
 * path tracing by a rasterised view. Camera view: 4-sample MSAA raster of the static mesh (its vertices are the
 * radiosity nodes) and of the posed bodies sliced to <= subdiv_h (sliceTris :443), per-vertex KB4 projection
 * (SCOPE: a pinhole camera that follows the scope body); per fragment the BSDF over ns_static / ns_dyn stratified
 * emitter samples, soft shadows from 4 sector shadow maps (equidistant about the emission axis, 3x3 taps of 2x2
 * bilinear depth compares, static and dynamic casters in separate maps), node irradiance interpolated per vertex
 * times the capsule occlusion on static surfaces, a uniform environment on posed bodies (SHADER :92-360). The
 * multisample buffer is resolved through half floats and scaled back (FINISH :363). Rasterisation is this
 * library's own: clip against 0 <= z <= w and a guard band, vertices snapped to 1/256 pixel, exact integer edge
 * functions with a tie rule that gives a shared edge's samples to exactly one triangle, 'less' depth with ties to
 * the earlier triangle, shading once per (pixel, triangle) at the pixel centre, as in a 4x MSAA raster pipeline. */
typedef struct {
  uint32_t ns_static, ns_dyn;            /* emitter samples per fragment: static surfaces / posed bodies (24, 96) */
  uint32_t sm_res;                       /* shadow map side (2048) */
  uint32_t scope_width, scope_height;    /* SCOPE image (1280 x 720) */
  uint32_t env_material;                 /* material whose hemispherical albedo sets the posed bodies' environment */
  uint32_t debug;                        /* 0; 1 no shadows; 2 shadow visibility as grey */
  uint32_t reserved;
  double sm_theta_max_deg;               /* shadow map cone half-angle (62) */
  double far_m;                          /* depth range (1.0 m) */
  double subdiv_h, subdiv_fixture;       /* posed-body slicing step, fixtures (0.003, 0.01 m) */
  double scope_hfov_deg, scope_circle_frac;      /* SCOPE pinhole (75 deg, image circle 0.95 of the width) */
  double scope_view_dir[3], scope_objective[3];  /* scope frame: view direction (0, 0.5, 0.866), objective (0, 0, 0) */
} vt_lite_opts;
typedef struct {
  uint32_t raster_tris, static_tris, dyn_verts, n_cameras;   /* n_cameras = scene cameras + SCOPE (the last) */
  double build_ms;
  double shadow_static_ms, shadow_dyn_ms, camera_ms;          /* device ms of the last render's passes */
  double camera_raster_ms, camera_shade_ms;                   /* the camera pass: vertices + raster, fragments */
  uint32_t big_tris, launches;                                /* tiles queued for the many-pixel path by the last
                                                                 camera pass; kernel launches */
  uint32_t shadow_big_tiles, reserved;                        /* tiles queued by the last dynamic shadow pass */
} vt_lite_info;
/* lite_nodes/renderer.js:497 _init (geometry :527, emitter samples :598, cameras :696). Needs vt_nodes_build. */
vt_status vt_lite_create(vt_ctx* ctx, const vt_lite_opts* opts, vt_lite_info* info);
vt_status vt_lite_info_get(vt_ctx* ctx, vt_lite_info* info);
/* The raster geometry alone, on the host (no device needed): counts = [vertices, triangles]; verts (8 words each:
 * position | mesh + instance << 16, normal | node) and idx (3 per triangle) are filled when not NULL and large
 * enough for the counts of a previous call. lite_nodes/renderer.js:527 _buildGeometry with sliceTris (:443). */
vt_status vt_lite_geometry(const vt_scene_desc* scene, double subdiv_h, double subdiv_fixture, uint32_t counts[2], uint32_t* verts, uint32_t* idx);
/* lite_nodes/renderer.js:844 renderCamera: node radiosity brought up to the poses, shadow maps re-rendered when
 * the scope (static casters) or any pose (dynamic casters) changed, then the camera pass into the camera's
 * radiance (w x h rgba32f; out_rgba receives a copy when not NULL). camera: scene camera index, or n_cameras - 1
 * for SCOPE. */
vt_status vt_lite_render_camera(vt_ctx* ctx, uint32_t camera, float* out_rgba);
/* lite_nodes/renderer.js:892 sensor (the DISPLAY pass :369): exposure, relative illumination of the KB4 cameras,
 * global-mean glare, white balance, sRGB + S-curve into rgba8; du = (gain, glare k, 0, scaleY, wb rgb, 0, c, black,
 * 0, 0, fx, fy, cx, cy, 0 x 4); prev: the previous frame's statistics (sum of scaled luma, count); stats: this
 * frame's. */
vt_status vt_lite_display(vt_ctx* ctx, uint32_t camera, const float du[20], const uint32_t prev[4], uint32_t stats[4]);
/* lite_nodes/renderer.js:940 readback('linear' | 'rgb8' | 'rgba8'): VT_READ_LINEAR, VT_READ_RGB8, VT_READ_RGBA8. */
vt_status vt_lite_readback(vt_ctx* ctx, uint32_t camera, int kind, void* dst, size_t bytes);
/* The raster pass's intermediate buffers, for checking each stage on its own (bytes: the buffer's size, or
 * larger). VIEW: the camera's view uniform (128 floats, lite_nodes/renderer.js:766 _viewData layout); CLIP: clip
 * coordinates of every raster vertex for the camera's last pass (float4); KEYS: its 4 samples per pixel (uint64:
 * depth bits << 32 | triangle, all ones = empty); SM_STATIC / SM_DYN: the shadow maps (4 x res x res depth bits,
 * all ones = cleared); SM_CLIP: the last shadow pass's clip coordinates (4 x raster vertices float4); GEOM: raster
 * vertices (8 words: position | mesh + instance << 16, normal | node); INDEX: 3 per triangle; EMIT: the emitter
 * samples in the world (8 floats: position | sector, normal | area). */
enum { VT_LITE_VIEW = 0, VT_LITE_CLIP = 1, VT_LITE_KEYS = 2, VT_LITE_SM_STATIC = 3, VT_LITE_SM_DYN = 4, VT_LITE_SM_CLIP = 5,
       VT_LITE_GEOM = 6, VT_LITE_INDEX = 7, VT_LITE_EMIT = 8 };
vt_status vt_lite_debug(vt_ctx* ctx, int what, uint32_t camera, void* dst, size_t bytes);
/* The rasteriser on its own: triangles (3 indices each) over clip-space vertices (x, y, z, w) into a w x h target
 * of `samples` (4: the MSAA positions (0.375, 0.125), (0.875, 0.375), (0.125, 0.625), (0.625, 0.875); 1: the pixel
 * centre) per pixel; keys: w x h x samples uint64, depth bits << 32 | triangle index, all ones where nothing passed
 * (1 sample: a shadow-map layer, depth only, the triangle bits all ones). Host or device buffers. */
vt_status vt_raster(vt_ctx* ctx, const float* clip, uint32_t n_verts, const uint32_t* idx, uint32_t n_tris, uint32_t width,
                    uint32_t height, uint32_t samples, uint64_t* keys);

/* ------------------------------------------------------------------ scene preparation */

/* The mesh clean-up the reference runs in JavaScript before packing (gpu/scene_gpu.js), for callers that load a
 * scene directory (scene.json + meshes/\*.bin): results are library-owned until vt_mesh_free. Positions and normals
 * are doubles (the JavaScript keeps numbers), indices 3 per triangle. */
typedef struct {
  double* P;           /* n_verts x 3 */
  double* N;           /* n_verts x 3 */
  uint32_t* I;         /* n_idx */
  uint32_t n_verts, n_idx;
  void* handle;
} vt_mesh_out;
/* gpu/scene_gpu.js:68 weld: merge vertices whose positions agree to 1e-7 m and normals to 1e-4 (keys rounded as
 * JavaScript's Math.round does), in order of first appearance; triangles that become degenerate are dropped. */
vt_status vt_weld(const float* P, const float* N, uint32_t n_verts, const uint32_t* I, uint32_t n_idx, vt_mesh_out* out);
/* gpu/scene_gpu.js:95 subdivide: conforming edge bisection, every pass splitting all edges longer than h at their
 * midpoints (one shared vertex per edge, numbered in the order the edges are met) and re-triangulating each
 * triangle by its pattern of split edges, until no edge is longer than h or after max_passes (24). */
vt_status vt_subdivide(const double* P, const double* N, uint32_t n_verts, const uint32_t* I, uint32_t n_idx, double h, uint32_t max_passes,
                       vt_mesh_out* out);
/* The same weld and subdivide on a CUDA device: identical vertices, numbering and triangles, host buffers in and out.
 * First-met numbering becomes a sort of (key, input position) pairs whose runs lead with the first occurrence, and
 * a scan of the leads in input order; the arithmetic is the host's, in doubles without contraction. */
vt_status vt_weld_device(int32_t device, const float* P, const float* N, uint32_t n_verts, const uint32_t* I, uint32_t n_idx, vt_mesh_out* out);
vt_status vt_subdivide_device(int32_t device, const double* P, const double* N, uint32_t n_verts, const uint32_t* I, uint32_t n_idx, double h,
                              uint32_t max_passes, vt_mesh_out* out);
/* gpu/scene_gpu.js:146 benchMesh: a grid of cells <= h over `fine` (x0, y0, x1, y1) within `extent` and four coarse
 * quads out to the extent, at height z, normal +z. */
vt_status vt_bench_mesh(double z, const double extent[4], const double fine[4], double h, vt_mesh_out* out);
/* gpu/scene_gpu.js:37 computeNormals: area-weighted vertex normals for a mesh shipped without them. */
vt_status vt_compute_normals(const float* P, uint32_t n_verts, const uint32_t* I, uint32_t n_idx, float* N);
void vt_mesh_free(vt_mesh_out* mesh);

/* ---------------------------------------------------------------------------------------- bvh (pure) */

/* gpu/bvh.js:18 buildBVH(pos, idx, {leafSize}): binned SAH BVH2 on the host. nodes_out must hold
 * vt_bvh_capacity(n_tris, leaf) * 16 words (= max(4, n_tris) nodes); order_out n_tris. Returns node count etc. */
typedef struct { uint32_t node_count, max_depth; float bmin[3], bmax[3]; } vt_bvh_result;
uint32_t vt_bvh_capacity(uint32_t n_tris, uint32_t leaf_size);
vt_status vt_bvh_build(const float* pos, uint32_t n_verts, const uint32_t* idx, uint32_t n_tris, uint32_t leaf_size,
                       uint32_t* nodes_out, uint32_t* order_out, vt_bvh_result* res);
/* The same build on a CUDA device (gpu/bvh.js:18 buildBVH): identical nodes, order and result, host buffers in and
 * out. vt_create builds the static scene's BVH this way. */
vt_status vt_bvh_build_device(int32_t device, const float* pos, uint32_t n_verts, const uint32_t* idx, uint32_t n_tris,
                              uint32_t leaf_size, uint32_t* nodes_out, uint32_t* order_out, vt_bvh_result* res);

/* -------------------------------------------------------------------------------------------- diagnostics */

/* gpu/renderer.js:447 debugFlags(): loop-cap counters {traversalCap, leafCap, refined, refinedBody,
 * refinedShadow, refinedSubsample, corruptTree, packetCap, ...} (16 words). reset = 1 clears them. */
vt_status vt_debug_flags(vt_ctx* ctx, uint32_t out[16], int reset);
/* gpu/renderer.js:1271 timings(): device ms of the last render, sensor and solve calls, and kernel launches; with
 * kernel profiling on, the summed device ms and launches of the path tracer's traversal and shading kernels and the
 * rays they traced (since profiling was last reset). */
typedef struct {
  double render_ms, sensor_ms, solve_ms, trace_ms;
  uint64_t launches;
  double extend_ms, shade_ms, shadow_ms;           /* closest-hit, shading and any-hit kernels (profiling on) */
  uint64_t extend_launches, shadow_launches;
  uint64_t extend_rays, shadow_paths;              /* rays the closest-hit kernels traced, paths the any-hit kernels served */
  double node_direct_ms, node_jacobi_ms;           /* the node radiosity's last vt_nodes_direct / vt_nodes_jacobi (device) */
  uint32_t node_jacobi_steps, reserved;            /* steps of that vt_nodes_jacobi call */
} vt_timings;
vt_status vt_timings_get(const vt_ctx* ctx, vt_timings* out);
/* Kernel profiling of vt_render_camera: events around each traversal and shading launch (enable 1), and the
 * counters reset (reset 1). Adds a little launch overhead; off by default. */
vt_status vt_kernel_profile(vt_ctx* ctx, int enable, int reset);
/* The context's CUDA stream (cudaStream_t), for callers that order their own device work after ours. */
void* vt_stream(vt_ctx* ctx);

#ifdef __cplusplus
}
#endif
#endif /* VTWIN_H */
