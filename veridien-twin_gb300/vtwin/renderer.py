"""TwinRenderer: the host-side mirror of gpu/renderer.js's TwinRenderer over libvtwin's C ABI.

Same method names and argument meanings as the reference (gpu/renderer.js:3-10): create, setPoses, renderCamera,
renderFrame, sensor, readback, visible, project, timings, debugFlags, destroy; snake_case aliases are provided.
Errors raise VtError (the reference throws Error: unknown camera, too many bodies, ...).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi as A
from ._lib import VtError, check, load
from . import sensor as sensor_mod

# gpu/renderer.js:31 DEFAULTS, except refine: the refinement pass is opt-in here (the reference adds 6 sub-samples on
# edges by default), so that a default render is the plain pass-1 estimator
DEFAULTS = {"spp": 1, "refine": 0, "refineLightSamples": 1, "refineShadows": True, "lightSamples": 4, "leafSize": 4,
            "albedoSamples": 1024, "radiosityEvery": 1, "gatherK": 64, "nodeSamples": 4, "itersPerFrame": 4, "itersInitial": 96,
            "smoothSigma": 0.003, "smoothRadius": 0.006, "nbrK": 16, "nodes": True}
PRESETS = {"judge": {}, "balanced": {"spp": 1, "lightSamples": 2, "refine": 2, "refineLightSamples": 1, "refineShadows": False,
                                     "radiosityEvery": 2, "itersPerFrame": 1},
           "live": {"spp": 1, "lightSamples": 1, "refine": 0, "radiosityEvery": 2, "itersPerFrame": 1}}


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


class TwinRenderer:
    """gpu/renderer.js:200 TwinRenderer (the WebGPU device replaced by one CUDA context)."""

    def __init__(self):
        self._ctx = None

    # ------------------------------------------------------------------------------------------- lifecycle
    @classmethod
    def create(cls, scene: dict, physics: dict | None = None, preset: str | None = None, device: int = 0, **opts):
        """gpu/renderer.js:202 create({scene, physics, preset, ...DEFAULTS}); `scene` is a dict of welded arrays
        (vtwin.dome), physics is accepted for the API's sake (materials already resolved in `scene`)."""
        r = cls()
        r.opts = {**DEFAULTS, **PRESETS.get(preset or "", {}), **opts}
        r.lib = load()
        r.scene = scene
        r._desc = A.SceneDesc(scene)
        o = A.vt_options(leaf_size=int(r.opts["leafSize"]), albedo_samples=int(r.opts["albedoSamples"]), device=device)
        ctx = C.c_void_p()
        st = r.lib.vt_create(r._desc.ref, C.byref(o), C.byref(ctx))
        if st != A.VT_OK:
            raise VtError(st, r.lib.vt_last_error(None).decode())
        r._ctx = ctx
        r.cameras = {c.get("name", f"CAM{i + 1}"): i for i, c in enumerate(scene.get("cameras", []))}
        r.bodies = [b["key"] for b in scene.get("bodies", [])]
        r.frame = 0
        r.sensor_p = sensor_mod.sensor_params((opts or {}).get("sensor"))
        r.nodes_info = None
        r._sens = {}
        if r.opts.get("nodes", True):     # gpu/renderer.js:256: the gather table is part of create
            r.build_nodes()
        r.set_poses({"bodies": {}})
        return r

    # ------------------------------------------------------------------------------------------- node radiosity
    def build_nodes(self, **o):
        """gpu/renderer.js:456 _buildGatherTable: gather table, active nodes, smoothing neighbours. Renders then keep
        the node radiosity up to date with the poses (renderCamera's _ensureRadiosity) until set_node_state."""
        op = {**self.opts, **o}
        q = A.vt_nodes_opts(gather_k=int(op["gatherK"]), node_samples=int(op["nodeSamples"]), nbr_k=int(op["nbrK"]),
                            smooth_sigma=float(op["smoothSigma"]), smooth_radius=float(op["smoothRadius"]),
                            radiosity_every=int(op["radiosityEvery"]), iters_per_frame=int(op["itersPerFrame"]),
                            iters_initial=int(op["itersInitial"]), per_step_factors=int(bool(op.get("perStepFactors", False))))
        info = A.vt_nodes_info()
        check(self.lib.vt_nodes_build(self._ctx, C.byref(q), C.byref(info)), self._ctx)
        self.nodes_info = {"nodes": info.n_nodes, "activeNodes": info.n_active, "gatherK": info.gather_k, "nbrK": info.nbr_k,
                           "gatherBuildMs": info.build_ms, "neighbourMs": info.neighbour_ms, "tableEntries": int(info.table_entries)}
        return self.nodes_info

    def converge(self, iters=200):
        """gpu/renderer.js:804 converge(iters): direct light if the poses changed, `iters` Jacobi steps, node summary
        (eAvg). A boolean means a full solve (True: 200 steps) or none."""
        if isinstance(iters, bool) or not isinstance(iters, (int, float)) or not np.isfinite(iters):
            iters = 0 if iters is False else 200
        check(self.lib.vt_converge(self._ctx, int(iters)), self._ctx)
        return self.nodeSummary()

    def nodeSummary(self) -> dict:
        """gpu/renderer.js:825 nodeSummary(): area-weighted means over the active nodes; refreshes eAvg."""
        out = np.zeros(13)
        check(self.lib.vt_node_summary(self._ctx, _p(out)), self._ctx)
        return {"area": out[0], "meanIndirect": out[1:4], "meanDirect": out[4:7], "meanLout": out[7:10], "eAvg": out[10:13]}

    node_summary = nodeSummary

    def update_nodes(self, force=False) -> str:
        """gpu/renderer.js:771 _ensureRadiosity: 'none', 'full', 'incremental' or 'reused'."""
        w = C.c_uint32(0)
        check(self.lib.vt_nodes_update(self._ctx, int(force), C.byref(w)), self._ctx)
        return ["none", "full", "incremental", "reused"][w.value]

    def node_direct(self, moved=0):
        check(self.lib.vt_nodes_direct(self._ctx, int(moved)), self._ctx)

    def node_jacobi(self, iters):
        check(self.lib.vt_nodes_jacobi(self._ctx, int(iters)), self._ctx)

    def nodes_export(self) -> dict:
        """Copies of the gather table (n x K), the active list, the neighbours (n_active x nbrK x 2) and the escapes."""
        i = self.nodes_info
        n, na, K, nk = i["nodes"], i["activeNodes"], i["gatherK"], i["nbrK"]
        g = np.zeros((n, K), np.uint32)
        act = np.zeros(na, np.uint32)
        nb = np.zeros((na, nk, 2), np.uint32)
        mis = np.zeros(n, np.float32)
        check(self.lib.vt_nodes_export(self._ctx, _p(g), _p(act), _p(nb), _p(mis)), self._ctx)
        return {"gtable": g, "active": act, "nbr": nb, "misses": mis}

    def get_node_state(self):
        """The node state (n_static_verts x 16 float32) and its latest slot."""
        st = np.zeros((len(self.scene["static"]["P"]), 16), np.float32)
        slot = C.c_uint32(0)
        check(self.lib.vt_get_node_state(self._ctx, _p(st), C.byref(slot)), self._ctx)
        return st, slot.value

    def destroy(self):
        if self._ctx is not None:
            self.lib.vt_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass

    def _cam(self, name) -> int:
        if isinstance(name, int):
            if 0 <= name < len(self.cameras):
                return name
        elif name in self.cameras:
            return self.cameras[name]
        raise VtError(A.VT_ERR_UNKNOWN_CAMERA, f"unknown camera {name}")

    # ------------------------------------------------------------------------------------------- scene
    def info(self) -> A.vt_scene_info:
        i = A.vt_scene_info()
        check(self.lib.vt_scene_info_get(self._ctx, C.byref(i)), self._ctx)
        return i

    def export(self) -> dict:
        i = self.info()
        nodes = np.zeros(i.node_count * 16, np.uint32)
        tris = np.zeros(i.tri_count * 16, np.uint32)
        verts = np.zeros(i.vert_count * 8, np.uint32)
        params = np.zeros(i.param_vec4s * 4, np.float32)
        check(self.lib.vt_scene_export(self._ctx, _p(nodes), _p(tris), _p(verts), _p(params)), self._ctx)
        return {"nodes": nodes, "tris": tris, "verts": verts, "params": params}

    def blas(self, body: int) -> A.vt_blas_info:
        b = A.vt_blas_info()
        check(self.lib.vt_blas_info_get(self._ctx, body, C.byref(b)), self._ctx)
        return b

    # ------------------------------------------------------------------------------------------- poses
    def _pose_array(self, poses):
        out = np.full((len(self.bodies), 16), np.nan)
        bodies = (poses or {}).get("bodies", {}) if isinstance(poses, dict) else {}
        for i, key in enumerate(self.bodies):
            T = bodies.get(key)
            if T is not None:
                out[i] = np.asarray(T, np.float64).ravel()
        # bodies the caller never posed: the emitter body stays where it was built (identity), as a scene
        # without a light makes no image; everything else is hidden (gpu/renderer.js:626)
        for i, b in enumerate(self.scene.get("bodies", [])):
            if np.isnan(out[i, 0]) and b["kind"] == "scope" and key_missing(bodies, b["key"]):
                out[i] = np.eye(4).T.ravel()
        return np.ascontiguousarray(out)

    def setPoses(self, poses0, poses1=None):
        """gpu/renderer.js:620 setPoses(poses0, poses1?): poses.bodies[key] = column-major 4x4."""
        T0 = self._pose_array(poses0)
        T1 = self._pose_array(poses1) if poses1 is not None else None
        check(self.lib.vt_set_poses(self._ctx, _p(T0), _p(T1) if T1 is not None else None, len(T0)), self._ctx)

    set_poses = setPoses

    def set_pose_array(self, T0, T1=None):
        T0 = np.ascontiguousarray(T0, np.float64).reshape(-1, 16)
        T1 = None if T1 is None else np.ascontiguousarray(T1, np.float64).reshape(-1, 16)
        check(self.lib.vt_set_poses(self._ctx, _p(T0), _p(T1) if T1 is not None else None, len(T0)), self._ctx)

    def set_eavg(self, e):
        e = np.ascontiguousarray(e, np.float32)
        check(self.lib.vt_set_eavg(self._ctx, _p(e)), self._ctx)

    def scene_uniform(self) -> np.ndarray:
        out = np.zeros(24 + 48 * 24, np.float32)
        check(self.lib.vt_scene_uniform_get(self._ctx, _p(out), out.nbytes), self._ctx)
        return out

    def set_node_state(self, state, slot=1):
        state = np.ascontiguousarray(state, np.float32)
        check(self.lib.vt_set_node_state(self._ctx, _p(state), slot), self._ctx)

    # ------------------------------------------------------------------------------------------- rendering
    def request(self, name, spp=None, lightSamples=None, seed=0, options=0, mode=A.VT_SHADE_TWIN, max_depth=2,
                shutter=(0.0, 1.0), scale=1.0, root=0, frame=None, refine=None, refineLightSamples=None,
                refineShadows=None, hitCache=None, shadowCache=None, exactShadows=False) -> A.vt_render_req:
        """gpu/renderer.js:935 _submitCamera's options: pass 1 (spp sub-samples, lightSamples each) and the refinement
        pass (refine more sub-samples on edges, posed bodies and, with refineShadows, pixels whose shadow rays were
        traced; refineLightSamples each)."""
        opts = int(options)
        if refineShadows if refineShadows is not None else self.opts.get("refineShadows", True):
            opts |= A.OPTION_BITS["REFINE_SHADOW"]
        # gpu/renderer.js:944 the static first-hit cache of the twin's camera feeds (exact; the library keeps its key)
        if int(mode) == A.VT_SHADE_TWIN and (hitCache if hitCache is not None else self.opts.get("hitCache", True)):
            opts |= A.OPTION_BITS["CACHE_WRITE"]
            # :952 the static-occlusion cache, unless exact shadows are asked for
            if (shadowCache if shadowCache is not None else self.opts.get("shadowCache", True)) and not exactShadows:
                opts |= A.OPTION_BITS["SHADOW_CACHE"]
        q = A.vt_render_req(camera=self._cam(name), spp=int(spp if spp is not None else self.opts["spp"]),
                            light_samples=int(lightSamples if lightSamples is not None else self.opts["lightSamples"]),
                            seed=int(seed), options=opts, mode=int(mode), max_depth=int(max_depth), root=int(root),
                            frame=int(self.frame if frame is None else frame),
                            refine=int(refine if refine is not None else self.opts.get("refine", 0)),
                            refine_light_samples=int(refineLightSamples if refineLightSamples is not None
                                                     else self.opts.get("refineLightSamples", 1)))
        q.shutter[:] = [float(shutter[0]), float(shutter[1])]
        q.scale = float(scale)
        return q

    def renderCamera(self, name, out=None, **o):
        """gpu/renderer.js:975 renderCamera(name, {spp, lightSamples, seed, shutter, ...}). Radiance stays on the
        device; `out` (a float32 array of w*h*4, host or device pointer-holder) receives a copy when given."""
        q = self.request(name, **o)
        check(self.lib.vt_render_camera(self._ctx, C.byref(q), _p(out) if isinstance(out, np.ndarray) else out), self._ctx)
        return q

    render_camera = renderCamera

    def renderFrame(self, cameras=None, sensor=False, sensorOpts=None, **o):
        """gpu/renderer.js:986 renderFrame({cameras, sensor}): every listed camera, then its sensor stage, queued as
        one call on the library's stream with one synchronisation (vt_render_frame); AE / AWB then take each camera's
        statistics. Returns the frame's device time in ms under "ms" and, with a sensor, each camera's statistics."""
        names = cameras or list(self.cameras)
        idx = [self._cam(n) for n in names]
        q = self.request(idx[0], **o)
        f = A.vt_frame_req()
        cams = (C.c_uint32 * len(idx))(*idx)
        f.cameras = C.cast(cams, C.POINTER(C.c_uint32))
        f.n_cameras = len(idx)
        f.render = q
        sus, stats = None, None
        if sensor:
            so = sensorOpts or {}
            sus = (A.vt_sensor_uniform * len(idx))(*[self._sensor_uniform(c, **so) for c in idx])
            stats = np.zeros((len(idx), 4), np.uint32)
            f.sensors = C.cast(sus, C.POINTER(A.vt_sensor_uniform))
            f.stats = stats.ctypes.data_as(C.POINTER(C.c_uint32))
        check(self.lib.vt_render_frame(self._ctx, C.byref(f)), self._ctx)
        out = {n: {"linear": n} for n in names}
        if sensor:
            for k, (n, c) in enumerate(zip(names, idx)):
                out[n].update(self._after_sensor(c, stats[k], sus[k]))
        self.frame += 1
        out["ms"] = float(f.ms)
        return out

    render_frame = renderFrame

    def readback(self, name, kind="linear"):
        """gpu/renderer.js:1191 readback(name, 'linear'|'raw'|'rgb8'|'rgba8'|'yuv420') -> a host copy."""
        c = self._cam(name)
        w, h = self.scene["cameras"][c]["size"]
        if kind == "linear":
            out = np.zeros((h, w, 4), np.float32)
            check(self.lib.vt_readback(self._ctx, c, A.VT_READ_LINEAR, _p(out), out.nbytes), self._ctx)
        elif kind == "raw":
            out = np.zeros((h, w), np.float32)
            check(self.lib.vt_readback(self._ctx, c, A.VT_READ_RAW, _p(out), out.nbytes), self._ctx)
        elif kind in ("rgb8", "rgba8"):
            out = np.zeros((h, w, 3 if kind == "rgb8" else 4), np.uint8)
            check(self.lib.vt_readback(self._ctx, c, A.VT_READ_RGB8 if kind == "rgb8" else A.VT_READ_RGBA8, _p(out), out.nbytes), self._ctx)
        elif kind == "yuv420":
            cw, ch = (w + 1) // 2, (h + 1) // 2
            buf = np.zeros(w * h + 2 * cw * ch, np.uint8)
            check(self.lib.vt_readback(self._ctx, c, A.VT_READ_YUV420, _p(buf), buf.nbytes), self._ctx)
            return {"width": w, "height": h, "y": buf[:w * h].reshape(h, w), "cb": buf[w * h:w * h + cw * ch].reshape(ch, cw),
                    "cr": buf[w * h + cw * ch:].reshape(ch, cw)}
        else:
            raise VtError(A.VT_ERR_ARG, f"readback kind {kind} (linear, raw, rgb8, rgba8, yuv420)")
        return out

    def expose(self, name, seed=0, frame=None, noise=True, exposure_s=1.0, gain=1.0, params=None, optics_scale=1.0):
        """The expose stage alone (gpu/wgsl/sensor.wgsl.js:177 sensorExpose with the vertical blur): the camera's last
        radiance x `optics_scale` -> its raw DN image (vt_sensor_camera)."""
        c = self._cam(name)
        w, h = self.scene["cameras"][c]["size"]
        p = {**self.sensor_p, **(params or {})}
        if noise is False:
            p["noise"] = False
        su = A.vt_sensor_uniform()
        su.words[:] = [int(x) for x in sensor_mod.pack_sensor_uniform(
            p, w, h, frame=self.frame if frame is None else frame, seed=seed, exposure=exposure_s, gain=gain, cam_index=c)]
        check(self.lib.vt_sensor_camera(self._ctx, c, C.byref(su), float(optics_scale)), self._ctx)

    def _sensor_state(self, c):
        st = self._sens.get(c)
        if st is None:
            p = self.sensor_p
            st = self._sens[c] = {"ae": sensor_mod.AutoExposure(p, exposure_units=p.get("exposureUnits0", 10)), "awb": None, "manual": None,
                                  "ri": False, "meanLuma": None, "meanRGB": None}
        return st

    def set_exposure(self, name, e):
        """gpu/renderer.js:1042 _manualExposure: a number (seconds), {time_s, gain}, or None / 'auto' for AE."""
        st = self._sensor_state(self._cam(name))
        if e is None or e == "auto":
            st["manual"] = None
        elif isinstance(e, (int, float)):
            st["manual"] = {"time_s": float(e), "gain": 1.0}
        else:
            st["manual"] = {"time_s": float(e.get("time_s", e.get("exposure_s", e.get("time")))), "gain": float(e.get("gain", 1.0))}

    def exposureOf(self, name) -> dict:
        """gpu/renderer.js:1049 exposureOf: the exposure the next sensor() uses (AE or manual)."""
        st = self._sensor_state(self._cam(name))
        if st["manual"]:
            return {**st["manual"], "auto": False}
        ae = st["ae"]
        return {"time_s": ae.exposure, "gain": ae.gain, "gainUnits": ae.gain_units, "units": ae.units, "auto": True}

    exposure_of = exposureOf

    def _sensor_uniform(self, c, seed=0, frame=None, noise=True, exposure_s=None, gain=None, params=None):
        """The camera's sensor uniform for its next frame: AE / manual exposure, AWB gains (gpu/renderer.js:1141);
        the relative-illumination map is set on first use."""
        w, h = self.scene["cameras"][c]["size"]
        st = self._sensor_state(c)
        base = self.sensor_p
        if not st["ri"]:
            vt = np.ascontiguousarray(base["vignettingThetaDeg"], np.float64)
            vv = np.ascontiguousarray(base["vignetting"], np.float64)
            check(self.lib.vt_set_relative_illumination(self._ctx, c, None, float(base["pupilExponent"]), _p(vt), _p(vv), len(vt)), self._ctx)
            st["ri"] = True
        ex = self.exposureOf(c)
        p = {**base, **(params or {})}
        if p.get("awb") and st["awb"] is not None and not (params and "wb" in params):
            p["wb"] = [g * a for g, a in zip(p["wb"], st["awb"])]
        if noise is False:
            p["noise"] = False
        su = A.vt_sensor_uniform()
        su.words[:] = [int(x) for x in sensor_mod.pack_sensor_uniform(
            p, w, h, frame=self.frame if frame is None else frame, seed=seed, exposure=ex["time_s"] if exposure_s is None else exposure_s,
            gain=ex["gain"] if gain is None else gain, cam_index=c)]
        return su

    def _after_sensor(self, c, stats, su):
        """gpu/renderer.js:1117 _afterSensor: this frame's statistics drive the next frame's AE and AWB."""
        w, h = self.scene["cameras"][c]["size"]
        st = self._sensor_state(c)
        st["meanLuma"] = float(stats[0]) / (w * h * 255)
        st["meanRGB"] = [float(x) / (w * h * 1023) for x in stats[1:]]
        if not st["manual"]:
            st["ae"].update(st["meanLuma"])
        if self.sensor_p.get("awb"):
            st["awb"] = sensor_mod.update_awb(st["awb"], st["meanRGB"], self.sensor_p.get("awbDamping", 0.3))
        return {"stats": np.array(stats, np.uint32), "meanLuma": st["meanLuma"], "meanRGB": st["meanRGB"],
                "uniform": np.array(su.words, np.uint32)}

    def sensor(self, name, seed=0, frame=None, noise=True, exposure_s=None, gain=None, params=None):
        """gpu/renderer.js:1141 sensor(name, {seed, frame, noise, exposure_s, gain, params}): the whole chain on the
        camera's last radiance (optics with relative illumination, glare, expose, demosaic, white balance + CCM, noise
        reduction, tone, YCbCr) into its raw, 8-bit RGB and YCbCr images; then the auto exposure and auto white
        balance take this frame's statistics for the next (gpu/renderer.js:1117 _afterSensor)."""
        c = self._cam(name)
        su = self._sensor_uniform(c, seed, frame, noise, exposure_s, gain, params)
        stats = np.zeros(4, np.uint32)
        check(self.lib.vt_sensor_frame(self._ctx, c, C.byref(su), _p(stats)), self._ctx)
        return self._after_sensor(c, stats, su)

    def relative_illumination(self, name):
        c = self._cam(name)
        w, h = self.scene["cameras"][c]["size"]
        out = np.zeros((h, w), np.float32)
        check(self.lib.vt_get_relative_illumination(self._ctx, c, _p(out)), self._ctx)
        return out

    # ------------------------------------------------------------------------------------------- batches
    def _batch_req(self, cameras, poses0, poses1, spp, lightSamples, seed, max_depth, shutter, scale, options, sensor, frame0,
                   optics_scale, use_graph, wave_paths, exposure_s=1.0, gain=1.0):
        cams = [self._cam(c) for c in cameras]
        P0 = np.ascontiguousarray(poses0, np.float64)
        if P0.ndim == 2:
            P0 = P0[None]
        n_poses, n_bodies = P0.shape[0], P0.shape[1]
        P0 = P0.reshape(n_poses, n_bodies, 16)
        P1 = None if poses1 is None else np.ascontiguousarray(poses1, np.float64).reshape(n_poses, n_bodies, 16)
        cam_arr = np.ascontiguousarray(cams, np.uint32)
        q = A.vt_batch_req(cameras=cam_arr.ctypes.data_as(C.POINTER(C.c_uint32)), n_cameras=len(cams), n_poses=n_poses,
                           n_bodies=n_bodies, poses0=P0.ctypes.data_as(C.POINTER(C.c_double)),
                           poses1=P1.ctypes.data_as(C.POINTER(C.c_double)) if P1 is not None else None,
                           spp=int(spp), light_samples=int(lightSamples), seed=int(seed), options=int(options),
                           max_depth=int(max_depth), scale=float(scale), frame0=int(frame0), optics_scale=float(optics_scale),
                           use_graph=int(bool(use_graph)), wave_paths=int(wave_paths))
        q.shutter[:] = [float(shutter[0]), float(shutter[1])]
        keep = [cam_arr, P0, P1]
        if sensor is not None:
            p = {**self.sensor_p, **(sensor if isinstance(sensor, dict) else {})}
            su = (A.vt_sensor_uniform * len(cams))()
            for k, c in enumerate(cams):
                w, h = self.scene["cameras"][c]["size"]
                su[k].words[:] = [int(x) for x in sensor_mod.pack_sensor_uniform(p, w, h, frame=frame0, seed=seed, exposure=exposure_s,
                                                                                  gain=gain, cam_index=c)]
            q.sensor = C.cast(su, C.POINTER(A.vt_sensor_uniform))
            keep.append(su)
        return q, cams, n_poses, keep

    def render_batch(self, cameras, poses0, poses1=None, spp=64, lightSamples=1, seed=0, max_depth=6, shutter=(0.0, 1.0), scale=1.0,
                     options=0, sensor=None, frame0=0, optics_scale=1.0, use_graph=True, wave_paths=0, radiance=False,
                     raw_out=None, radiance_out=None, exposure_s=1.0, gain=1.0):
        """Many cameras x many kinematic poses in one call (renderFrame over a setPoses sweep, gpu/renderer.js:620,986).
        poses0 / poses1: (n_poses, n_bodies, 16) column-major body transforms. sensor: None (radiance only) or sensor
        parameters (dict, or True for the renderer's): raw uint16 frames, pose q exposing frame frame0 + q.
        Returns {"raw": [per camera (n_poses, h, w) uint16], "radiance": [per camera (n_poses, h, w, 4)], "stats": {...}}.
        raw_out / radiance_out: preallocated host arrays or device tensors (anything with data_ptr()) of all frames."""
        q, cams, n_poses, keep = self._batch_req(cameras, poses0, poses1, spp, lightSamples, seed, max_depth, shutter, scale, options,
                                                 None if sensor is None or sensor is False else (sensor if isinstance(sensor, dict) else {}),
                                                 frame0, optics_scale, use_graph, wave_paths, exposure_s, gain)
        sizes = [tuple(self.scene["cameras"][c]["size"]) for c in cams]
        total = sum(n_poses * w * h for w, h in sizes)
        want_raw = q.sensor is not None and bool(q.sensor)
        raw = rad = None
        if want_raw:
            raw = raw_out if raw_out is not None else np.empty(total, np.uint16)
        if radiance or radiance_out is not None:
            rad = radiance_out if radiance_out is not None else np.empty(total * 4, np.float32)
        ptr = lambda a: None if a is None else (C.c_void_p(a.data_ptr()) if hasattr(a, "data_ptr") else _p(a))
        st = A.vt_batch_stats()
        check(self.lib.vt_render_batch(self._ctx, C.byref(q), ptr(raw), ptr(rad), C.byref(st)), self._ctx)
        out = {"stats": {"ms": st.ms, "shared_paths": st.shared_paths, "pair_paths": st.pair_paths, "samples": st.samples,
                         "waves": st.waves, "graph_replayed": bool(st.graph_replayed), "reruns": st.reruns, "vary_mask": st.vary_mask}}
        if raw_out is None and raw is not None:
            out["raw"], o = [], 0
            for w, h in sizes:
                out["raw"].append(raw[o:o + n_poses * w * h].reshape(n_poses, h, w))
                o += n_poses * w * h
        if radiance_out is None and rad is not None:
            out["radiance"], o = [], 0
            for w, h in sizes:
                out["radiance"].append(rad[4 * o:4 * (o + n_poses * w * h)].reshape(n_poses, h, w, 4))
                o += n_poses * w * h
        del keep
        return out

    def autotune_batch(self, cameras, poses0, poses1=None, spp=64, lightSamples=1, seed=0, max_depth=6, **kw):
        """Time the batched renderer's candidate wave sizes and pixel tiles; the fastest is kept for later batches."""
        q, cams, n_poses, keep = self._batch_req(cameras, poses0, poses1, spp, lightSamples, seed, max_depth, (0.0, 1.0), 1.0, 0, None, 0,
                                                 1.0, False, 0)
        rows = (A.vt_tune_row * 64)()
        n = C.c_uint32(0)
        best = A.vt_tune_row()
        check(self.lib.vt_batch_autotune(self._ctx, C.byref(q), rows, 64, C.byref(n), C.byref(best)), self._ctx)
        del keep
        tab = [{"wave_paths": r.wave_paths, "tile": (r.tile_w, r.tile_h), "refill": r.refill, "ms_per_mpath": r.ms_per_mpath}
               for r in rows[:n.value]]
        return {"wave_paths": best.wave_paths, "tile": (best.tile_w, best.tile_h), "refill": best.refill,
                "ms_per_mpath": best.ms_per_mpath}, tab

    # ------------------------------------------------------------------------------------------- calibration
    def calib_setup(self, n_nodes=4096, lamp_samples=16) -> dict:
        """Radiosity nodes (clusters of the static triangles), their form factors F and the emitter transfer D of
        the differentiable calibration model (include/vtwin.h vt_calib_setup)."""
        info = A.vt_calib_info()
        check(self.lib.vt_calib_setup(self._ctx, C.byref(A.vt_calib_desc(n_nodes=int(n_nodes), lamp_samples=int(lamp_samples))),
                                      C.byref(info)), self._ctx)
        self.calib_info = {"n_nodes": info.n_nodes, "n_materials": info.n_materials, "n_lamps": info.n_lamps,
                           "n_static_tris": info.n_static_tris}
        return self.calib_info

    def calib_export(self, with_F=False) -> dict:
        i = self.calib_info
        n, L = i["n_nodes"], i["n_lamps"]
        out = {"centres": np.zeros((n, 3), np.float32), "normals": np.zeros((n, 3), np.float32), "areas": np.zeros(n, np.float32),
               "node_mat": np.zeros(n, np.uint32), "tri_node": np.zeros(i["n_static_tris"], np.uint32), "D": np.zeros((n, L), np.float32)}
        F = np.zeros((n, n), np.float32) if with_F else None
        check(self.lib.vt_calib_export(self._ctx, _p(out["centres"]), _p(out["normals"]), _p(out["areas"]), _p(out["node_mat"]),
                                       _p(out["tri_node"]), _p(F) if F is not None else None, _p(out["D"])), self._ctx)
        if F is not None:
            out["F"] = F
        return out

    def calib_forward(self, cameras, albedo, lamp, spp=32, lightSamples=1, seed=0, max_depth=3, jacobi_iters=0, targets=None,
                      images=True, replay=False, intrinsics=False):
        """Image loss (mean of (I - T)^2 over pixels and channels) of the calibration render; returns (loss, images)
        with images a list of (h, w, 4) float32 arrays per camera (or None). intrinsics: the backward also gives the
        loss's derivative in each camera's KB4 intrinsics (calib_intrinsics_grad). replay: False keeps every path's
        record when they fit; True traces the paths in chunks of sub-samples sized to the free memory, keeping only
        their hits and shadow outcomes, from which the backward shades each chunk again; an integer c >= 1 does the
        same in chunks of at most c sub-samples."""
        cams = [self._cam(c) for c in cameras]
        cam_arr = np.ascontiguousarray(cams, np.uint32)
        alb = np.ascontiguousarray(albedo, np.float64).reshape(-1, 3)
        lam = np.ascontiguousarray(lamp, np.float64).ravel()
        sizes = [tuple(self.scene["cameras"][c]["size"]) for c in cams]
        total = sum(w * h for w, h in sizes)
        tg = None if targets is None else np.ascontiguousarray(
            np.concatenate([np.asarray(t, np.float32).reshape(-1, 4) for t in targets]) if isinstance(targets, (list, tuple)) else targets,
            np.float32)
        img = np.empty((total, 4), np.float32) if images else None
        q = A.vt_calib_req(cameras=cam_arr.ctypes.data_as(C.POINTER(C.c_uint32)), n_cameras=len(cams), spp=int(spp),
                           light_samples=int(lightSamples), seed=int(seed), max_depth=int(max_depth), jacobi_iters=int(jacobi_iters),
                           albedo=alb.ctypes.data_as(C.POINTER(C.c_double)), lamp=lam.ctypes.data_as(C.POINTER(C.c_double)),
                           targets=tg.ctypes.data_as(C.POINTER(C.c_float)) if tg is not None else None,
                           images=img.ctypes.data_as(C.POINTER(C.c_float)) if img is not None else None, replay=0 if replay is False else 1 if replay is True else 1 + int(replay),
                           intrinsics=int(bool(intrinsics)))
        loss = C.c_double(0.0)
        check(self.lib.vt_calib_forward(self._ctx, C.byref(q), C.byref(loss)), self._ctx)
        self._calib_cams = cams
        out = None
        if img is not None:
            out, o = [], 0
            for w, h in sizes:
                out.append(img[o:o + w * h].reshape(h, w, 4))
                o += w * h
        return loss.value, out

    def calib_backward(self):
        """Gradient of the last calib_forward's loss: (d/d albedo (n_materials x 3), d/d lamp (n_lamps))."""
        i = self.calib_info
        ga = np.zeros((i["n_materials"], 3), np.float64)
        gl = np.zeros(i["n_lamps"], np.float64)
        check(self.lib.vt_calib_backward(self._ctx, _p(ga), _p(gl)), self._ctx)
        return ga, gl

    def calib_intrinsics_grad(self):
        """The last calib_backward's image-loss derivative in each forward camera's (fx, fy, cx, cy, k1..k4): an
        (n_cameras, 8) array (the forward must have asked for it with intrinsics=True)."""
        n = len(self._calib_cams) if getattr(self, "_calib_cams", None) else 0
        g = np.zeros((max(n, 1), 8), np.float64)
        check(self.lib.vt_calib_intrinsics_grad(self._ctx, _p(g)), self._ctx)
        return g[:n]

    def calib_export_paths(self, slot, spp):
        """The stored forward's discrete path decisions of the forward's camera `slot` (for checks): triangle and
        instance per bounce (h, w, spp, 4, 2) and light-sample weights per vertex (h, w, spp, 4, 4)."""
        w, h = self.scene["cameras"][self._calib_cams[slot]]["size"]
        ti = np.zeros((h, w, spp, 4, 2), np.uint32)
        q = np.zeros((h, w, spp, 4, 4), np.float32)
        check(self.lib.vt_calib_export_paths(self._ctx, int(slot), _p(ti), _p(q)), self._ctx)
        return ti, q

    def set_intrinsics(self, name, K):
        K = np.ascontiguousarray(K, np.float64)
        check(self.lib.vt_set_camera_intrinsics(self._ctx, self._cam(name), _p(K)), self._ctx)

    def get_intrinsics(self, name):
        K = np.zeros(8, np.float64)
        check(self.lib.vt_get_camera_intrinsics(self._ctx, self._cam(name), _p(K)), self._ctx)
        return K

    def observed(self, name, pts, margin=0.0, max_theta=None):
        """Which dome-frame points a camera observes: in front of it and projecting inside its image (a fiducial
        mask for reproj_loss)."""
        c = self._cam(name)
        cam = self.scene["cameras"][c]
        T = np.asarray(cam["T_D_C"], np.float64).reshape(4, 4)
        P = np.ascontiguousarray(pts, np.float64).reshape(-1, 3)
        Xc = (P - T[:3, 3]) @ T[:3, :3]
        th = np.arctan2(np.hypot(Xc[:, 0], Xc[:, 1]), Xc[:, 2])
        uv = self.project(c, P)
        w, h = cam["size"]
        ok = (uv[:, 0] >= margin) & (uv[:, 0] <= w - 1 - margin) & (uv[:, 1] >= margin) & (uv[:, 1] <= h - 1 - margin) & (Xc[:, 2] > 0)
        if max_theta is not None:
            ok &= th <= max_theta
        return ok

    def reproj_loss(self, cameras, pts, uv_target):
        """Reprojection loss of dome-frame points (NaN targets: not observed) and its analytic gradient in each
        camera's KB4 intrinsics."""
        cams = np.ascontiguousarray([self._cam(c) for c in cameras], np.uint32)
        P = np.ascontiguousarray(pts, np.float64).reshape(-1, 3)
        T = np.ascontiguousarray(uv_target, np.float64).reshape(len(cams), len(P), 2)
        g = np.zeros((len(cams), 8), np.float64)
        loss = C.c_double(0.0)
        check(self.lib.vt_reproj_loss(self._ctx, _p(cams), len(cams), _p(P), len(P), _p(T), C.byref(loss), _p(g)), self._ctx)
        return loss.value, g

    # ------------------------------------------------------------------------------------------- queries
    def trace(self, o4, d4, mask=3, any_hit=False, root=0):
        """gpu/wgsl/kernels.wgsl.js:535 traceTest: rays (o.xyz, time), (d.xyz, -) -> (t, tri, inst, u), v."""
        o4 = np.ascontiguousarray(o4, np.float32).reshape(-1, 4)
        d4 = np.ascontiguousarray(d4, np.float32).reshape(-1, 4)
        out = np.zeros((len(o4), 4), np.float32)
        v = np.zeros(len(o4), np.float32)
        check(self.lib.vt_trace_rays(self._ctx, _p(o4), _p(d4), len(o4), mask, int(any_hit), root, _p(out), _p(v)), self._ctx)
        t = out[:, 0].copy()
        tri = out[:, 1].view(np.uint32).copy()
        inst = out[:, 2].view(np.uint32).copy()
        return t, tri, inst, out[:, 3].copy(), v

    def unit_test(self, kind, tin, lens=None):
        """gpu/wgsl/kernels.wgsl.js:494-551 lensTest / bsdfTest / capsuleTest / profileTest (vt_unit_test): tin is the
        reference's float4 input slots ((n x slots) x 4); returns the output slots. lens: (fx, fy, cx, cy, k1..k4,
        alpha) for VT_UNIT_LENS."""
        slots_in, slots_out = {A.VT_UNIT_LENS: (2, 2), A.VT_UNIT_BSDF: (4, 3), A.VT_UNIT_CAPSULE: (4, 1),
                               A.VT_UNIT_PROFILE: (1, 1)}[kind]
        tin = np.ascontiguousarray(tin, np.float32).reshape(-1, 4)
        if len(tin) % slots_in:
            raise VtError(A.VT_ERR_ARG, f"unit test: {len(tin)} input slots is not a multiple of {slots_in}")
        n = len(tin) // slots_in
        q = A.vt_unit_req(kind=int(kind), n=n)
        if lens is not None:
            q.lens[:9] = [float(x) for x in lens]
        out = np.zeros((n * slots_out, 4), np.float32)
        check(self.lib.vt_unit_test(self._ctx, C.byref(q), _p(tin), _p(out)), self._ctx)
        return out

    def visible(self, name, pointsD, tol=2e-4, time=0.5):
        pts = np.ascontiguousarray(pointsD, np.float64).reshape(-1, 3)
        out = np.zeros(len(pts), np.uint8)
        check(self.lib.vt_visible(self._ctx, self._cam(name), _p(pts), len(pts), tol, time, _p(out)), self._ctx)
        return out.astype(bool)

    def project(self, name, pointsD):
        pts = np.ascontiguousarray(pointsD, np.float64).reshape(-1, 3)
        uv = np.zeros((len(pts), 2), np.float64)
        check(self.lib.vt_project(self._ctx, self._cam(name), _p(pts), len(pts), _p(uv)), self._ctx)
        return uv

    # ------------------------------------------------------------------------------------------- diagnostics
    def debugFlags(self, reset=False) -> dict:
        v = np.zeros(16, np.uint32)
        check(self.lib.vt_debug_flags(self._ctx, _p(v), int(reset)), self._ctx)
        return {"traversalCap": int(v[0]), "leafCap": int(v[1]), "refined": int(v[2]), "refinedBody": int(v[3]),
                "refinedShadow": int(v[4]), "refinedSubsample": int(v[5]), "corruptTree": int(v[6]), "packetCap": int(v[7])}

    debug_flags = debugFlags

    def timings(self) -> dict:
        t = A.vt_timings()
        check(self.lib.vt_timings_get(self._ctx, C.byref(t)), self._ctx)
        return {"render_ms": t.render_ms, "sensor_ms": t.sensor_ms, "solve_ms": t.solve_ms, "trace_ms": t.trace_ms,
                "launches": int(t.launches), "extend_ms": t.extend_ms, "shade_ms": t.shade_ms, "shadow_ms": t.shadow_ms,
                "extend_launches": int(t.extend_launches), "shadow_launches": int(t.shadow_launches),
                "extend_rays": int(t.extend_rays), "shadow_paths": int(t.shadow_paths), "node_direct_ms": t.node_direct_ms,
                "node_jacobi_ms": t.node_jacobi_ms, "node_jacobi_steps": int(t.node_jacobi_steps)}

    def kernel_profile(self, enable=True, reset=True):
        """Events around the path tracer's bounce kernels (timings() then reports their device ms and rays)."""
        check(self.lib.vt_kernel_profile(self._ctx, int(enable), int(reset)), self._ctx)

    # ------------------------------------------------------------------------------------------- radiosity
    def solve_radiosity(self, F, rho, E, precision=A.VT_PREC_FP32, tol=1e-6, max_iters=1000, check_every=8, B0=None, reuse_f=False):
        return solve_radiosity(F, rho, E, precision, tol, max_iters, check_every, B0, ctx=self._ctx, reuse_f=reuse_f)

    def form_factors(self, centres, normals, areas, out=None):
        return form_factors(centres, normals, areas, out, ctx=self._ctx)

    def form_factors_visible(self, centres, normals, areas, rays=64, out=None):
        """Dense node form factors with each pair's visibility through this scene (vt_form_factors_visible): `rays`
        stratified rays per pair. out: a numpy array or a device tensor (data_ptr()) of n x n float32."""
        C_ = np.ascontiguousarray(centres, np.float32)
        n = len(C_)
        N_ = np.ascontiguousarray(normals, np.float32)
        A_ = np.ascontiguousarray(areas, np.float32)
        if out is None:
            out = np.zeros((n, n), np.float32)
        optr = C.c_void_p(out.data_ptr()) if hasattr(out, "data_ptr") else out.ctypes.data_as(C.c_void_p)
        check(self.lib.vt_form_factors_visible(self._ctx, n, _p(C_), _p(N_), _p(A_), int(rays), optr), self._ctx)
        return out


def key_missing(bodies: dict, key: str) -> bool:
    return key not in bodies


class _Ctx:
    """A context without a scene, for the radiosity solve and the form-factor builder."""
    _ctx = None

    @classmethod
    def get(cls):
        if cls._ctx is None:
            lib = load()
            desc = A.vt_scene_desc()
            m = (A.vt_mesh * 1)()
            mt = (A.vt_material * 1)()
            mt[0] = A.material_struct({"rho": [0.5, 0.5, 0.5], "ior": 1.0, "no_table": 1})
            desc.meshes, desc.n_meshes, desc.materials, desc.n_materials = m, 1, mt, 1
            desc.L0[:] = [1, 1, 1]
            cls._keep = (desc, m, mt)
            ctx = C.c_void_p()
            st = lib.vt_create(C.byref(desc), None, C.byref(ctx))
            if st != A.VT_OK:
                raise VtError(st, lib.vt_last_error(None).decode())
            cls._ctx = ctx
        return cls._ctx


def solve_radiosity(F, rho, E, precision=A.VT_PREC_FP32, tol=1e-6, max_iters=1000, check_every=8, B0=None, ctx=None, reuse_f=False):
    """B = E + diag(rho) F B on the device (gpu/renderer.js:804 converge, the lite_nodes Jacobi). F, rho, E are
    numpy arrays (host) or objects exposing an integer device pointer via `.data_ptr()` (device). Returns
    (B, info) with info = {iters, refinements, residual, ms, status}."""
    lib = load()
    ctx = ctx or _Ctx.get()
    n = int(rho.shape[0])
    E2 = E.reshape(n, -1) if hasattr(E, "reshape") else E
    R = int(E2.shape[1])

    def ptr(a):
        if hasattr(a, "data_ptr"):
            return C.cast(C.c_void_p(a.data_ptr()), C.POINTER(C.c_float))
        return np.ascontiguousarray(a, np.float32).ctypes.data_as(C.POINTER(C.c_float))

    keep = [np.ascontiguousarray(x, np.float32) if isinstance(x, np.ndarray) else x for x in (F, rho, E2)]
    B = np.ascontiguousarray(B0, np.float32).copy() if B0 is not None else np.zeros((n, R), np.float32)
    q = A.vt_solve_req(n=n, n_rhs=R, F=ptr(keep[0]), rho=ptr(keep[1]), E=ptr(keep[2]), B=B.ctypes.data_as(C.POINTER(C.c_float)),
                       precision=int(precision), max_iters=int(max_iters), warm_start=int(B0 is not None),
                       check_every=int(check_every), reuse_f=int(bool(reuse_f)), tol=float(tol))
    st = lib.vt_radiosity_solve(ctx, C.byref(q))
    if st not in (A.VT_OK, A.VT_ERR_NOT_CONVERGED):
        check(st, ctx)
    return B, {"iters": q.iters, "refinements": q.refinements, "residual": q.residual, "ms": q.ms, "sweep_ms": q.sweep_ms,
               "convert_ms": q.convert_ms, "status": st}


def solve_radiosity_static(F, rho, E, B, tol=1e-6, max_iters=1000, check_every=8, stream=None):
    """One right-hand side, no device allocation (vt_radiosity_solve_static): F, rho, E, B are device tensors
    (objects with .data_ptr()), B receives the solution. Returns {iters, residual, status}."""
    lib = load()
    n = int(rho.shape[0])
    # the C side cannot check sizes: every buffer is a contiguous float32 CUDA tensor big enough for n nodes (the C
    # side itself refuses host memory and another device's memory)
    for name, t, want in (("F", F, n * n), ("rho", rho, n), ("E", E, n), ("B", B, n)):
        if not hasattr(t, "data_ptr") or str(t.dtype) != "torch.float32" or not t.is_contiguous():
            raise VtError(A.VT_ERR_ARG, f"solve_radiosity_static: {name} must be a contiguous float32 device tensor")
        if t.device.type != "cuda":
            raise VtError(A.VT_ERR_ARG, f"solve_radiosity_static: {name} is not a CUDA tensor")
        if t.numel() < want or (name != "F" and t.numel() != n):
            raise VtError(A.VT_ERR_ARG, f"solve_radiosity_static: {name} holds {t.numel()} values, {want} needed")
    it = C.c_uint32(0)
    res = C.c_double(0.0)
    dp = lambda t: C.c_void_p(t.data_ptr())
    st = lib.vt_radiosity_solve_static(dp(F), dp(rho), dp(E), dp(B), n, int(max_iters), int(check_every), float(tol),
                                       C.c_void_p(stream) if stream else None, C.byref(it), C.byref(res))
    if st not in (A.VT_OK, A.VT_ERR_NOT_CONVERGED):
        raise VtError(st, "vt_radiosity_solve_static failed")
    return {"iters": it.value, "residual": res.value, "status": st}


def form_factors(centres, normals, areas, out=None, ctx=None):
    lib = load()
    ctx = ctx or _Ctx.get()
    C_ = np.ascontiguousarray(centres, np.float32)
    n = len(C_)
    N_ = np.ascontiguousarray(normals, np.float32)
    A_ = np.ascontiguousarray(areas, np.float32)
    if out is None:
        out = np.zeros((n, n), np.float32)
    optr = C.c_void_p(out.data_ptr()) if hasattr(out, "data_ptr") else out.ctypes.data_as(C.c_void_p)
    check(lib.vt_form_factors(ctx, n, _p(C_), _p(N_), _p(A_), optr), ctx)
    return out


def build_bvh(pos, idx, leaf_size=4, device=None) -> dict:
    """gpu/bvh.js:18 buildBVH(pos, idx, {leafSize}) -> {nodes (uint32 words), nodeCount, order, bmin, bmax, maxDepth}.

    device=None builds on the host's threads, an int on that CUDA device (the same tree)."""
    lib = load()
    pos = np.ascontiguousarray(pos, np.float32).ravel()
    idx = np.ascontiguousarray(idx, np.uint32).ravel()
    n = len(idx) // 3
    cap = lib.vt_bvh_capacity(n, leaf_size)
    nodes = np.zeros(cap * 16, np.uint32)
    order = np.zeros(max(1, n), np.uint32)
    res = A.vt_bvh_result()
    if device is None:
        check(lib.vt_bvh_build(_p(pos), len(pos) // 3, _p(idx), n, leaf_size, _p(nodes), _p(order), C.byref(res)))
    else:
        check(lib.vt_bvh_build_device(int(device), _p(pos), len(pos) // 3, _p(idx), n, leaf_size, _p(nodes), _p(order),
                                      C.byref(res)))
    return {"nodes": nodes[: res.node_count * 16].copy(), "nodeCount": res.node_count, "order": order[:n].copy(),
            "bmin": np.array(res.bmin[:]), "bmax": np.array(res.bmax[:]), "maxDepth": res.max_depth}
