// TwinRenderer / LiteNodesRenderer over libvtwin (the CUDA renderer for one GB300) through the Node-API addon
// (vtwin_addon.cc): the drop-in for gpu/renderer.js and lite_nodes/renderer.js. It keeps their method names, option
// defaults and presets, and sits in the reference's gpu/ directory in place of renderer.js, beside the pure modules
// it reuses (scene_gpu.js: decodeMesh, loadScene, unwrap, MESH_FLAG; sensor.js: sensorParams, packSensorUniform,
// AutoExposure, updateAWB; lens.js: lensParams). Images stay in device memory until readback copies them out.
//
// The WebGPU device is replaced by one CUDA context per renderer; methods that awaited the GPU queue in the reference
// still return promises, and synchronous ones stay synchronous. Errors throw, as the reference's do (unknown camera,
// too many bodies), with the library's message and a `status` property.
import { createRequire } from 'node:module';
import { loadScene, unwrap, MESH_FLAG } from './scene_gpu.js';
import { sensorParams, packSensorUniform, AutoExposure, updateAWB } from './sensor.js';
import { lensParams } from './lens.js';

const require = createRequire(import.meta.url);
const addon = require(process.env.VTWIN_ADDON || './build/Release/vtwin.node');

// gpu/renderer.js:31 DEFAULTS and :58 PRESETS, unchanged
export const DEFAULTS = Object.freeze({
  spp: 1, refine: 6, lightSamples: 4, refineLightSamples: 1, radiosityEvery: 1, nodeSpacing: 0.003, gatherK: 64,
  nodeSamples: 4, itersPerFrame: 4, itersInitial: 96, smoothSigma: 0.003, smoothRadius: 0.006, nbrK: 16, packet: false,
  refineShadows: true, hitCache: true, shadowCache: true, cullShadows: true, layerLines: false, leafSize: 4,
});
export const PRESETS = Object.freeze({
  judge: {},
  balanced: { spp: 1, lightSamples: 2, refine: 2, refineLightSamples: 1, refineShadows: false, radiosityEvery: 2, itersPerFrame: 1 },
  live: { spp: 1, lightSamples: 1, refine: 0, radiosityEvery: 2, itersPerFrame: 1 },
});

// the library's constants (include/vtwin.h)
const O = { LAYER: 16, REFINE_SHADOW: 1024, CACHE_WRITE: 2048, SHADOW_CACHE: 8192 };
const READ = { linear: 0, raw: 1, rgba8: 2, rgb8: 3, yuv420: 4 };
const BODY = { instrument: 0, scope: 1, board: 2, fixed: 3, fixture: 4 };

// ------------------------------------------------------------------ scene preparation (gpu/scene_gpu.js:241, front half)

/** gpu/scene_gpu.js:218 bodyOfPart: mesh name -> {key, kind, emitter?, owner?}. */
function bodyOfPart(scene) {
  const map = {};
  for (const inst of scene.instruments || []) for (const part of inst.parts || []) map[part.mesh] = { key: `${inst.id}/${part.body}`, kind: 'instrument' };
  const sc = scene.scope || {};
  for (const m of sc.mesh_parts || []) map[m] = { key: 'scope', kind: 'scope' };
  if (sc.emitter_mesh) map[sc.emitter_mesh] = { key: 'scope', kind: 'scope', emitter: true };
  for (const b of scene.boards || []) map[b.mesh] = { key: `board/${b.name}`, kind: 'board' };
  for (const m of scene.meshes || []) if (m.owner_camera && !map[m.name]) map[m.name] = { key: `fixed/${m.name}`, kind: 'fixed', owner: m.owner_camera };
  for (const m of scene.meshes || []) {
    if (map[m.name] || !m.dynamic || !m.body) continue;
    const head = m.body.split('/')[0];
    map[m.name] = { key: m.body, kind: m.body === 'scope' ? 'scope' : head === 'board' ? 'board' : 'fixture' };
  }
  return map;
}

/** gpu/scene_gpu.js:170 materialsFromPhysics for one name, as the library's material record. */
function materialOf(name, physics) {
  const m = physics?.materials?.[name] || {};
  const model = unwrap(m.model);
  const textured = m.rho_d_paper != null && m.rho_d_ink != null;
  const fa = unwrap(m.fresnel_avg);
  let out;
  if (model === 'coated_conductor') {
    let tau = [].concat(unwrap(m.coat_transmittance) ?? [1, 1, 1]).map(Number);
    if (tau.length === 1) tau = [tau[0], tau[0], tau[0]];
    out = { metallic: 2, coated: true, f0: unwrap(m.f0) ?? [0.56, 0.57, 0.58], roughness: Number(unwrap(m.roughness) ?? 0.3),
      coatIor: Number(unwrap(m.coat_ior) ?? 1.5), coatRoughness: Number(unwrap(m.coat_roughness) ?? 0.05), tau };
  } else {
    out = { metallic: Number(unwrap(m.metallic) ?? (model === 'conductor' ? 1 : 0)),
      roughness: Number(unwrap(textured ? m.roughness_paper : m.roughness) ?? 0.5), ior: Number(unwrap(m.ior) ?? 1.5),
      rho: unwrap(textured ? m.rho_d_paper : m.rho_d) ?? [0.5, 0.5, 0.5], f0: unwrap(m.f0) ?? [0.56, 0.57, 0.58],
      fbar: fa == null ? NaN : Number(fa) };
  }
  if (textured) Object.assign(out, { textured: true, inkRho: unwrap(m.rho_d_ink).map(Number), inkRoughness: Number(unwrap(m.roughness_ink) ?? 0.4) });
  const ll = m.layer_lines;
  out.layer = ll && unwrap(ll.height_m) ? [Number(unwrap(ll.height_m)), Number(unwrap(ll.depth_m) ?? 0)] : null;
  out.emitter = model === 'emitter';
  out.name = name;
  return out;
}

/** gpu/scene_gpu.js:205 emitterFromPhysics. */
function emitterOf(physics) {
  const em = physics?.materials?.emitter || {};
  let prof = unwrap(em.profile);
  if (typeof prof === 'string') prof = prof.split('.').reduce((o, k) => o?.[k], physics);
  prof = prof || physics?.light?.profile || {};
  const th = unwrap(prof.theta_deg) ?? [0, 90], p = unwrap(prof.p) ?? [1, 1];
  return { L0: (unwrap(em.L0) ?? [1, 1, 1]).map(Number), profileTheta: Float32Array.from(th, (t) => (t * Math.PI) / 180),
    profileP: Float32Array.from(p, Number), axisDeg: Number(unwrap(physics?.scope?.emission_axis?.angle_from_shaft_deg) ?? NaN) };
}

const cat = (T, parts) => { const n = parts.reduce((a, p) => a + p.length, 0); const o = new T(n); let k = 0; for (const p of parts) { o.set(p, k); k += p.length; } return o; };

/**
 * The scene description the library's create takes: static meshes welded and subdivided to the node spacing (the
 * library's weld / subdivide, the reference's arithmetic), the bench, posed bodies by bodyOfPart in the body frame,
 * the mesh table, materials and the emitter from physics, the KB4 cameras. gpu/scene_gpu.js:241-330.
 */
export function prepareDesc(scene, meshData, physics, { nodeSpacing = 0.003, device = -1 } = {}) {
  const bodies = bodyOfPart(scene);
  const benchMat = scene.bench?.material || 'bench_white';
  const matNames = [], matIndex = {};
  for (const n of [...scene.meshes.map((m) => m.material), benchMat]) if (!(n in matIndex)) { matIndex[n] = matNames.length; matNames.push(n); }
  const materials = matNames.map((n) => materialOf(n, physics));
  const meshes = [];
  const addMesh = (name, material, flags, buildDir, overviewOnly = false) => {
    const lay = materials[matIndex[material]].layer;
    meshes.push({ name, mat: matIndex[material], flags, buildDir: buildDir || [0, 0, 1], layerPeriod: lay ? lay[0] : 0, layerDepth: lay ? lay[1] : 0, overviewOnly });
    return meshes.length - 1;
  };
  const sP = [], sN = [], sI = [], sTM = [], sVM = [];
  let nv = 0;
  const fine = [[Infinity, Infinity], [-Infinity, -Infinity]];
  for (const m of scene.meshes) {
    if (m.dynamic || bodies[m.name]) continue;
    const d = meshData[m.name];
    if (!d) throw new Error(`mesh ${m.name} not loaded`);
    const lay = materials[matIndex[m.material]].layer;
    const flags = MESH_FLAG.STATIC | (m.build_dir && lay && lay[1] > 0 ? MESH_FLAG.LAYER : 0);
    const mid = addMesh(m.name, m.material, flags, m.build_dir);
    const w = addon.weld(d.P, d.N, d.I, device);
    const s = addon.subdivide(w.P, w.N, w.I, nodeSpacing, 24, device);
    sP.push(Float32Array.from(s.P)); sN.push(Float32Array.from(s.N));
    sI.push(Uint32Array.from(s.I, (i) => i + nv)); sTM.push(new Uint32Array(s.I.length / 3).fill(mid)); sVM.push(new Uint32Array(s.P.length / 3).fill(mid));
    for (let i = 0; i < s.P.length; i += 3) {
      fine[0][0] = Math.min(fine[0][0], s.P[i]); fine[0][1] = Math.min(fine[0][1], s.P[i + 1]);
      fine[1][0] = Math.max(fine[1][0], s.P[i]); fine[1][1] = Math.max(fine[1][1], s.P[i + 1]);
    }
    nv += s.P.length / 3;
  }
  if (scene.bench) {
    const ext = scene.bench.extent || [[-0.5, -0.5], [0.5, 0.5]];
    const f = Number.isFinite(fine[0][0]) ? fine : ext, mg = 0.006;
    const b = addon.benchMesh(scene.bench.z ?? 0, Float64Array.from(ext.flat()),
      Float64Array.from([f[0][0] - mg, f[0][1] - mg, f[1][0] + mg, f[1][1] + mg]), nodeSpacing);
    const mid = addMesh('bench', benchMat, MESH_FLAG.STATIC | MESH_FLAG.BENCH);
    sP.push(Float32Array.from(b.P)); sN.push(Float32Array.from(b.N));
    sI.push(Uint32Array.from(b.I, (i) => i + nv)); sTM.push(new Uint32Array(b.I.length / 3).fill(mid)); sVM.push(new Uint32Array(b.P.length / 3).fill(mid));
    nv += b.P.length / 3;
  }
  const order = [], byKey = {};
  for (const m of scene.meshes) {
    const b = bodies[m.name];
    if (!b) continue;
    if (!byKey[b.key]) { byKey[b.key] = { key: b.key, kind: b.kind, owner: b.owner, meshes: [] }; order.push(b.key); }
    byKey[b.key].meshes.push(m);
  }
  const camNames = (scene.cameras || []).map((c) => c.name);
  const outBodies = order.map((key) => {
    const body = byKey[key];
    const P = [], N = [], I = [], TM = [], UV = [];
    let off = 0;
    for (const m of body.meshes) {
      const d = meshData[m.name];
      const isEm = !!bodies[m.name].emitter;
      const mat = isEm ? 'emitter' : m.material;
      if (isEm && !(mat in matIndex)) { matIndex[mat] = materials.length; materials.push({ name: 'emitter', metallic: 0, rho: [0.02, 0.02, 0.02], roughness: 0.05, ior: 1.5, emitter: true, noTable: true }); }
      const texd = !isEm && materials[matIndex[m.material]].textured && d.UV;
      const flags = (isEm ? MESH_FLAG.EMITTER : 0) | (body.kind === 'board' ? MESH_FLAG.BOARD : 0) | (texd ? MESH_FLAG.TEXTURED : 0) |
        (body.kind === 'instrument' ? MESH_FLAG.INSTRUMENT : 0) | (body.kind === 'scope' ? MESH_FLAG.SCOPE : 0);
      const mid = addMesh(m.name, mat, flags, m.build_dir, !!m.overview_only);
      P.push(Float32Array.from(d.P)); N.push(Float32Array.from(d.N)); I.push(Uint32Array.from(d.I, (i) => i + off)); UV.push(d.UV || new Float32Array((d.P.length / 3) * 2));
      TM.push(new Uint32Array(d.I.length / 3).fill(mid));
      off += d.P.length / 3;
    }
    return { key, kind: BODY[body.kind], ownerCamera: body.owner ? camNames.indexOf(body.owner) : -1,
      P: cat(Float32Array, P), N: cat(Float32Array, N), I: cat(Uint32Array, I), triMesh: cat(Uint32Array, TM), UV: cat(Float32Array, UV) };
  });
  const cameras = (scene.cameras || []).map((c) => {
    const L = lensParams(c.lens);
    const [w, h] = c.size || c.lens.size;
    return { name: c.name, width: w, height: h, fx: L.fx, fy: L.fy, cx: L.cx, cy: L.cy, alpha: L.alpha, k: L.k,
      T_D_C: Float64Array.from(c.T_D_C.flat()), lens: c.lens };
  });
  for (const m of materials) delete m.layer;
  return {
    static: { P: cat(Float32Array, sP), N: cat(Float32Array, sN), I: cat(Uint32Array, sI), triMesh: cat(Uint32Array, sTM), vertMesh: cat(Uint32Array, sVM) },
    bodies: outBodies, meshes, materials, ...emitterOf(physics), cameras,
  };
}

// ------------------------------------------------------------------ TwinRenderer (gpu/renderer.js:200)

export class TwinRenderer {
  /** gpu/renderer.js:202 create({scene, physics, preset, ...DEFAULTS}): scene = a base URL/path for loadScene, or
   * {scene, meshes} already loaded; prepares the scene, builds the library context and the node radiosity. */
  static async create(opts = {}) {
    const r = new TwinRenderer();
    r.opts = { ...DEFAULTS, ...(PRESETS[opts.preset] || {}), ...opts };
    const loaded = typeof opts.scene === 'string' ? await loadScene(opts.scene) : opts.scene;
    r.scene = loaded.scene;
    r.physics = opts.physics || {};
    r.desc = prepareDesc(loaded.scene, loaded.meshes, r.physics, { nodeSpacing: r.opts.nodeSpacing, device: opts.device ?? 0 });
    r.ctx = addon.create(r.desc, { leafSize: r.opts.leafSize, albedoSamples: 1024, device: opts.device ?? 0 });
    r.cameras = {};
    r.desc.cameras.forEach((c, i) => { r.cameras[c.name] = { index: i, size: [c.width, c.height], lens: c.lens, manual: null, awb: null }; });
    r.bodies = r.desc.bodies.map((b) => ({ key: b.key, kind: b.kind }));
    r.sensorP = sensorParams(r.physics, r.opts.sensor || {});
    for (const cam of Object.values(r.cameras)) cam.ae = new AutoExposure(r.sensorP, { exposureUnits: r.sensorP.exposureUnits0 });
    r.frame = 0;
    r.nodesInfo = addon.nodesBuild(r.ctx, r.opts);          // gpu/renderer.js:456 _buildGatherTable
    r.setPoses({ bodies: {} });
    return r;
  }

  _cam(name) {
    const cam = this.cameras[name];
    if (!cam) throw new Error(`unknown camera ${name}`);  // gpu/renderer.js:857
    return cam;
  }

  /** gpu/renderer.js:620 setPoses(poses0, poses1?): poses.bodies[key] = column-major 4x4; fixed bodies stay put. */
  setPoses(poses0, poses1 = null) {
    const pack = (poses) => {
      const T = new Float64Array(this.bodies.length * 16).fill(NaN);
      const b = poses?.bodies || {};
      this.bodies.forEach((bd, i) => {
        if (bd.kind === BODY.fixed) { for (let k = 0; k < 16; k++) T[16 * i + k] = k % 5 === 0 ? 1 : 0; return; }
        const m = b[bd.key];
        if (m) T.set(m, 16 * i);
        else if (bd.kind === BODY.scope && !(bd.key in b)) for (let k = 0; k < 16; k++) T[16 * i + k] = k % 5 === 0 ? 1 : 0;
      });
      return T;
    };
    addon.setPoses(this.ctx, pack(poses0), poses1 ? pack(poses1) : undefined);
    this.poses0 = poses0; this.poses1 = poses1 || poses0;
  }

  /** gpu/renderer.js:922 _options: the camera option bits of a render. */
  _options(o) {
    const hit = o.hitCache ?? this.opts.hitCache, shadow = o.shadowCache ?? this.opts.shadowCache;
    return ((o.refineShadows ?? this.opts.refineShadows) ? O.REFINE_SHADOW : 0) | (hit ? O.CACHE_WRITE : 0) |
      (hit && shadow && !o.exactShadows ? O.SHADOW_CACHE : 0) | (this.opts.layerLines ? O.LAYER : 0);
  }

  _request(o = {}) {
    return { spp: o.spp ?? this.opts.spp, lightSamples: o.lightSamples ?? this.opts.lightSamples, seed: o.seed ?? 0,
      refine: o.refine ?? this.opts.refine, refineLightSamples: o.refineLightSamples ?? this.opts.refineLightSamples,
      options: this._options(o), mode: 0, maxDepth: 2, shutter: o.shutter ?? [0, 1], frame: this.frame };
  }

  /** gpu/renderer.js:975 renderCamera(name, {spp, refine, lightSamples, seed, shutter, exactShadows}): the camera's
   * radiance stays on the device (readback copies it); the node radiosity follows the poses first. */
  async renderCamera(name, opts = {}) {
    addon.renderCamera(this.ctx, this._cam(name).index, this._request(opts));
  }

  _sensorUniform(name, o = {}) {
    const cam = this._cam(name), [w, h] = cam.size, ex = this.exposureOf(name);
    if (!cam.ri) {  // gpu/sensor.js:103 relativeIlluminationMap, computed by the library from the same parameters
      addon.setRelativeIllumination(this.ctx, cam.index, this.sensorP.pupilExponent,
        Float64Array.from(this.sensorP.vignettingThetaDeg), Float64Array.from(this.sensorP.vignetting));
      cam.ri = true;
    }
    const p = { ...this.sensorP, ...(o.params || {}) };
    if (p.awb && cam.awb && !(o.params && o.params.wb)) p.wb = p.wb.map((g, c) => g * cam.awb[c]);
    if (o.noise === false) p.noise = false;
    return new Uint32Array(packSensorUniform(p, { width: w, height: h, frame: o.frame ?? this.frame, seed: o.seed ?? 0,
      exposure: o.exposure_s ?? ex.time_s, gain: o.gain ?? ex.gain, camIndex: cam.index }));
  }

  /** gpu/renderer.js:1075 _afterSensor: AE and AWB from the frame's statistics. */
  _afterSensor(name, st) {
    const cam = this.cameras[name], [w, h] = cam.size;
    cam.meanLuma = st[0] / (w * h * 255);
    cam.meanRGB = [st[1], st[2], st[3]].map((x) => x / (w * h * 1023));
    if (!cam.manual) cam.ae.update(cam.meanLuma);
    if (this.sensorP.awb) cam.awb = updateAWB(cam.awb, cam.meanRGB, this.sensorP.awbDamping);
  }

  /** gpu/renderer.js:1092 sensor(name, {seed, frame, noise, exposure_s, gain, params}). */
  sensor(name, opts = {}) {
    const st = addon.sensor(this.ctx, this._cam(name).index, this._sensorUniform(name, opts));
    this._afterSensor(name, st);
  }

  /** gpu/renderer.js:986 renderFrame({cameras, sensor}): every camera's render (and sensor chain) in one call. */
  renderFrame(opts = {}) {
    const names = opts.cameras || Object.keys(this.cameras);
    const sensors = opts.sensor ? (() => { const u = new Uint32Array(64 * names.length); names.forEach((n, i) => u.set(this._sensorUniform(n, opts.sensorOpts || {}), 64 * i)); return u; })() : undefined;
    const f = addon.renderFrame(this.ctx, { cameras: Uint32Array.from(names, (n) => this._cam(n).index), render: this._request(opts), sensors });
    if (opts.sensor) names.forEach((n, i) => this._afterSensor(n, f.stats.subarray(4 * i, 4 * i + 4)));
    this.frame++;
    return { ms: f.ms, done: Promise.resolve() };
  }

  /** gpu/renderer.js:1050 exposureOf / :1043 _manualExposure */
  exposureOf(name) {
    const cam = this._cam(name);
    if (cam.manual) return { ...cam.manual, auto: false };
    return { time_s: cam.ae.exposure, gain: cam.ae.gain, gainUnits: cam.ae.gainUnits, units: cam.ae.units, auto: true };
  }
  setExposure(name, e) {
    const cam = this._cam(name);
    cam.manual = e === null || e === 'auto' ? null : typeof e === 'number' ? { time_s: e, gain: 1 } : { time_s: e.time_s ?? e.exposure_s ?? e.time, gain: e.gain ?? 1 };
  }
  sensorInfo() { return { params: this.sensorP }; }

  /** gpu/renderer.js:1191 readback(name, 'linear' | 'raw' | 'rgba8' | 'rgb8' | 'yuv420'). */
  async readback(name, kind = 'rgb8') {
    const cam = this._cam(name), [w, h] = cam.size;
    if (!(kind in READ)) throw new Error(`readback kind ${kind}`);
    const cw = Math.ceil(w / 2), ch = Math.ceil(h / 2);
    const bytes = { linear: w * h * 16, raw: w * h * 4, rgba8: w * h * 4, rgb8: w * h * 3, yuv420: w * h + 2 * cw * ch }[kind];
    const ab = addon.readback(this.ctx, cam.index, READ[kind], bytes);
    if (kind === 'linear' || kind === 'raw') return new Float32Array(ab);
    if (kind === 'yuv420') return { width: w, height: h, y: new Uint8Array(ab, 0, w * h), cb: new Uint8Array(ab, w * h, cw * ch), cr: new Uint8Array(ab, w * h + cw * ch, cw * ch) };
    return new Uint8Array(ab);
  }

  /** gpu/renderer.js:1238 visible(name, pointsD, {tol, time}) -> bool[] */
  visible(name, pointsD, { tol = 2e-4, time = 0.5 } = {}) {
    const v = addon.visible(this.ctx, this._cam(name).index, Float64Array.from(pointsD.flat()), tol, time);
    return Array.from(v, (x) => x !== 0);
  }

  /** gpu/renderer.js:1261 project(name, pointsD) -> [u, v][] (gpu/lens.js:43, FP64) */
  project(name, pointsD) {
    const uv = addon.project(this.ctx, this._cam(name).index, Float64Array.from(pointsD.flat()));
    return Array.from({ length: uv.length / 2 }, (_, i) => [uv[2 * i], uv[2 * i + 1]]);
  }

  /** gpu/renderer.js:804 converge(iters) and :825 nodeSummary() */
  async converge(iters = 200) {
    const n = typeof iters === 'boolean' ? (iters ? 200 : 0) : Number.isFinite(iters) ? iters : 200;
    addon.converge(this.ctx, n);
    return this.nodeSummary();
  }
  async nodeSummary() { return addon.nodeSummary(this.ctx); }

  /** gpu/renderer.js:1271 timings(), :447 debugFlags() */
  timings() { return addon.timings(this.ctx); }
  async debugFlags() {
    const f = addon.debugFlags(this.ctx, false);
    return { traversalCap: f[0], leafCap: f[1], refined: f[2], refinedBody: f[3], refinedShadow: f[4], refinedSubsample: f[5],
      corruptTree: f[6], packetCap: f[7], raw: f };
  }
  async idle() {}
  destroy() { addon.destroy(this.ctx); }

  // ---------------------------------------------------------------- the library's additions
  /** B = E + diag(rho) F B on the dense node transport (FP32, or BF16 / FP8 tcgen05 sweeps with FP64 refinement). */
  radiositySolve(req) { return addon.radiositySolve(this.ctx, req); }
  /** Many cameras x many poses in one call (renderFrame + sensor over a sweep of setPoses). */
  renderBatch(req, rawOut, radianceOut) { return addon.renderBatch(this.ctx, req, rawOut, radianceOut); }
  batchAutotune(req) { return addon.batchAutotune(this.ctx, req); }
}

// ------------------------------------------------------------------ LiteNodesRenderer (lite_nodes/renderer.js:489)

export class LiteNodesRenderer {
  /** lite_nodes/renderer.js:491 create({scene, physics, tracerOpts}): the node radiosity with the live preset, then
   * the raster pass's geometry, emitter samples and shadow maps. */
  static async create(opts = {}) {
    const r = new LiteNodesRenderer();
    r.tr = await TwinRenderer.create({ ...opts, preset: 'live', ...(opts.tracerOpts || {}) });
    r.info = addon.liteCreate(r.tr.ctx, opts.lite || {});
    r.cameras = { ...r.tr.cameras, SCOPE: { index: r.info.cameras - 1, size: [1280, 720] } };
    r.prev = {};
    return r;
  }
  setPoses(poses0, poses1 = null) { this.tr.setPoses(poses0, poses1); }
  /** lite_nodes/renderer.js:844 renderCamera(name) */
  async renderCamera(name) {
    const cam = this.cameras[name];
    if (!cam) throw new Error(`unknown camera ${name}`);
    addon.liteRenderCamera(this.tr.ctx, cam.index);
  }
  /** lite_nodes/renderer.js:892 sensor(name, {gain, exposure_s}): du is the 20-float display uniform the reference
   * builds (AE gain from the previous frame's mean, glare k, scaleY, WB, S-curve c, black, KB4 lens). */
  sensor(name, du) {
    const cam = this.cameras[name];
    const st = addon.liteDisplay(this.tr.ctx, cam.index, Float32Array.from(du), this.prev[name] || new Uint32Array(4));
    this.prev[name] = st;
    return st;
  }
  /** lite_nodes/renderer.js:940 readback(name, 'linear' | 'rgb8' | 'rgba8') */
  async readback(name, kind = 'rgb8') {
    const cam = this.cameras[name], [w, h] = cam.size;
    if (kind === 'raw' || kind === 'yuv420') return null;
    const bytes = { linear: w * h * 16, rgba8: w * h * 4, rgb8: w * h * 3 }[kind];
    const ab = addon.liteReadback(this.tr.ctx, cam.index, READ[kind], bytes);
    return kind === 'linear' ? new Float32Array(ab) : new Uint8Array(ab);
  }
  visible(name, pointsD, o) { return this.tr.visible(name, pointsD, o); }
  async converge(iters = 200) { return this.tr.converge(iters); }
  timings() { return addon.liteInfo(this.tr.ctx); }
  destroy() { this.tr.destroy(); }
}

// ------------------------------------------------------------------ calibration as an autograd-style function

/**
 * The twin's calibration loss over one packed parameter vector x (a Float64Array) = [albedo (nMat x 3), lamp radiances, intrinsics
 * (nCam x 8: fx, fy, cx, cy, k1..k4)]: image loss (mean of (I - T)^2) + wReproj x reprojection loss of the fiducials.
 * forward(x) -> loss; backward() -> d loss / d x (path-replay adjoint and transposed radiosity solve for albedos and
 * lamps; the intrinsics through the fiducials' analytic KB4 Jacobian and, with imageIntrinsics, the image term's
 * derivative along every path's primary ray).
 */
export function calibrationLoss(renderer, cameras, targets, fiducials, uvTargets, { wReproj = 1e-3, spp = 32, maxDepth = 3, imageIntrinsics = false, nNodes = 4096 } = {}) {
  const ctx = renderer.ctx;
  const info = addon.calibSetup(ctx, { nNodes, lampSamples: 16 });
  const cams = Uint32Array.from(cameras, (c) => renderer._cam(c).index);
  const tg = Float32Array.from(targets.flatMap((t) => Array.from(t)));
  const nA = 3 * info.nMaterials, nL = info.nLamps;
  let gK = null;
  return {
    info,
    forward(x) {
      cams.forEach((c, i) => addon.setCameraIntrinsics(ctx, c, x.subarray(nA + nL + 8 * i, nA + nL + 8 * i + 8)));
      const img = addon.calibForward(ctx, { cameras: cams, spp, maxDepth, albedo: x.subarray(0, nA), lamp: x.subarray(nA, nA + nL), targets: tg, intrinsics: imageIntrinsics });
      const rep = addon.reprojLoss(ctx, cams, Float64Array.from(fiducials.flat()), Float64Array.from(uvTargets.flat(2)));
      gK = rep.gK;
      return img + wReproj * rep.loss;
    },
    backward() {
      const g = addon.calibBackward(ctx, info.nMaterials, nL, imageIntrinsics ? cams.length : 0);
      const out = new Float64Array(nA + nL + 8 * cams.length);
      out.set(g.gAlbedo, 0);
      out.set(g.gLamp, nA);
      for (let i = 0; i < gK.length; i++) out[nA + nL + i] = wReproj * gK[i] + (g.gIntrinsics ? g.gIntrinsics[i] : 0);
      return out;
    },
  };
}
