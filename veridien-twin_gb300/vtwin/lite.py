"""lite_nodes/renderer.js LiteNodesRenderer: the raster live renderer that keeps the node radiosity of TwinRenderer
and draws the cameras by rasterisation (vt_lite_* of libvtwin: CUDA vertex, raster and fragment kernels).

The tracer behind it is a TwinRenderer with the live preset (lite_nodes/renderer.js:28 NodeTracer); its node
radiosity is kept up to date with the poses by every renderCamera, as the reference's _ensureRadiosity does.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi as A
from ._lib import VtError, check
from .renderer import TwinRenderer, _p

LITE_DEFAULTS = {"nsStatic": 24, "nsDyn": 96, "smRes": 2048, "smThetaMaxDeg": 62.0, "far": 1.0, "subdivH": 0.003,
                 "subdivFixture": 0.01, "scopeHfovDeg": 75.0, "scopeCircleFrac": 0.95, "scopeSize": (1280, 720),
                 "scopeViewDir": (0.0, 0.5, 0.866), "scopeObjective": (0.0, 0.0, 0.0), "envMaterial": None, "debug": 0}


def _unwrap(x):
    return x["value"] if isinstance(x, dict) and "value" in x else x


class LiteNodesRenderer:
    """lite_nodes/renderer.js:489 LiteNodesRenderer."""

    @classmethod
    def create(cls, scene: dict, physics: dict | None = None, device: int = 0, fast: bool = False, tracerOpts: dict | None = None,
               **opts):
        """lite_nodes/renderer.js:491 create({scene, physics, device, tracerOpts}) + _init (:497). `fast`: 32 gather
        rays and no node smoothing (the reference's fast mode also coarsens the node spacing, which is the scene's
        tessellation here)."""
        r = cls()
        r.physics = physics or {}
        fast_o = {"gatherK": 32, "smoothSigma": 0.0} if fast else {}
        r.tr = TwinRenderer.create(scene, physics, preset="live", device=device, **{**fast_o, **(tracerOpts or {})})
        r.lib = r.tr.lib
        r.scene = scene
        o = {**LITE_DEFAULTS, **opts}
        env = o["envMaterial"]
        if env is None:   # the dome's own material (lite_nodes/renderer.js:690), else the first
            names = [m.get("name") for m in scene.get("materials", [])]
            env = names.index("pla_matte_white") if "pla_matte_white" in names else 0
        q = A.vt_lite_opts(ns_static=int(o["nsStatic"]), ns_dyn=int(o["nsDyn"]), sm_res=int(o["smRes"]),
                           sm_theta_max_deg=float(o["smThetaMaxDeg"]), far_m=float(o["far"]), subdiv_h=float(o["subdivH"]),
                           subdiv_fixture=float(o["subdivFixture"]), scope_hfov_deg=float(o["scopeHfovDeg"]),
                           scope_circle_frac=float(o["scopeCircleFrac"]), scope_width=int(o["scopeSize"][0]),
                           scope_height=int(o["scopeSize"][1]), env_material=int(env), debug=int(o["debug"]))
        q.scope_view_dir[:] = [float(x) for x in o["scopeViewDir"]]
        q.scope_objective[:] = [float(x) for x in o["scopeObjective"]]
        info = A.vt_lite_info()
        check(r.lib.vt_lite_create(r.tr._ctx, C.byref(q), C.byref(info)), r.tr._ctx)
        r.o = o
        r.stats = {"rasterTris": info.raster_tris, "staticTris": info.static_tris, "dynVerts": info.dyn_verts, "loadMs": info.build_ms}
        r._names = list(r.tr.cameras) + ["SCOPE"]
        r._disp = {}
        r._ref_exposure = None
        return r

    @property
    def cameras(self):
        """lite_nodes/renderer.js:522: the scene's cameras, then SCOPE."""
        return list(self._names)

    def _cam(self, name) -> int:
        if isinstance(name, int) and 0 <= name < len(self._names):
            return name
        if name in self._names:
            return self._names.index(name)
        raise VtError(A.VT_ERR_UNKNOWN_CAMERA, f"unknown camera {name}")

    def size(self, name):
        c = self._cam(name)
        if c < len(self._names) - 1:
            return tuple(self.scene["cameras"][c]["size"])
        return tuple(int(x) for x in self.o["scopeSize"])

    # ------------------------------------------------------------------------------------------- poses
    def setPoses(self, poses0, poses1=None):
        """lite_nodes/renderer.js:729 setPoses: the tracer's poses; the scope pose moves the emitter samples, the
        shadow frame and the SCOPE camera."""
        self.tr.setPoses(poses0, poses1)

    set_poses = setPoses

    def set_pose_array(self, T0, T1=None):
        self.tr.set_pose_array(T0, T1)

    # ------------------------------------------------------------------------------------------- rendering
    def renderCamera(self, name, out=None, **_):
        """lite_nodes/renderer.js:844 renderCamera(name): scene-referred linear radiance stays on the device (`out`,
        a float32 host array of h x w x 4, receives a copy when given)."""
        check(self.lib.vt_lite_render_camera(self.tr._ctx, self._cam(name), _p(out) if isinstance(out, np.ndarray) else out), self.tr._ctx)

    render_camera = renderCamera

    def _out_scale(self):
        L0 = self.scene["emitter"]["L0"]
        return 1000.0 / max(L0[0], L0[1], L0[2], 1e-30)

    def sensor(self, name, gain=None, exposure_s=None):
        """lite_nodes/renderer.js:892 sensor(name, {gain, exposure_s}): the display look into rgba8, with the auto
        exposure from the previous frame's mean luma (its statistics, read back after the pass)."""
        c = self._cam(name)
        ph = self.physics or {}
        sp, isp = ph.get("sensor", {}) or {}, ph.get("isp", {}) or {}
        sc = _unwrap(isp.get("s_curve_c"))
        sc = 1.39 if sc is None else float(sc)
        b = _unwrap(isp.get("black_offset_linear"))
        b = 0.014 if b is None else float(b)
        k = _unwrap(((sp.get("lens") or {}).get("veiling_glare") or {}).get("fraction"))
        k = 0.0 if k is None else float(k)
        target = _unwrap((sp.get("auto_exposure") or {}).get("target_mean"))
        target = 0.18 if target is None else float(target)
        st = self._disp.setdefault(c, {"meanY": 0.0, "prev": np.zeros(4, np.uint32)})
        L0max = max(self.scene["emitter"]["L0"])
        if gain is None:
            m = st["meanY"] or 0.0
            gain = target / m if m > 0 else 1.0 / (5e-3 * L0max if self._out_scale() > 0 else 1.0)
            if exposure_s is not None and self._ref_exposure:
                gain *= exposure_s / self._ref_exposure
        wb = _unwrap(isp.get("white_balance_gains")) or [1.0, 1.0, 1.0]
        if c < len(self._names) - 1:
            cam = self.scene["cameras"][c]
            lens = [cam["fx"], cam["fy"], cam["cx"], cam["cy"]]
        else:
            lens = [0.0, 0.0, 0.0, 0.0]
        scaleY = 4096.0 / max(1e-30, (st["meanY"] or 5e-3 * L0max) * 4)
        du = np.array([gain, k, 0, scaleY, *wb[:3], 0, sc, b, 0, 0, *lens, 0, 0, 0, 0], np.float32)
        stats = np.zeros(4, np.uint32)
        check(self.lib.vt_lite_display(self.tr._ctx, c, _p(du), _p(st["prev"]), _p(stats)), self.tr._ctx)
        if stats[1]:
            st["meanY"] = (float(stats[0]) / float(stats[1])) / scaleY
        st["prev"] = stats
        return {"stats": stats, "meanY": st["meanY"], "du": du}

    def readback(self, name, kind="rgb8"):
        """lite_nodes/renderer.js:940 readback(name, 'linear' | 'rgb8' | 'rgba8'); 'yuv420' and 'raw' give None
        (the raster pass has no ISP planes)."""
        if kind in ("yuv420", "raw"):
            return None
        c = self._cam(name)
        w, h = self.size(c)
        if kind == "linear":
            out = np.zeros((h, w, 4), np.float32)
            check(self.lib.vt_lite_readback(self.tr._ctx, c, A.VT_READ_LINEAR, _p(out), out.nbytes), self.tr._ctx)
        elif kind in ("rgb8", "rgba8"):
            out = np.zeros((h, w, 3 if kind == "rgb8" else 4), np.uint8)
            check(self.lib.vt_lite_readback(self.tr._ctx, c, A.VT_READ_RGB8 if kind == "rgb8" else A.VT_READ_RGBA8, _p(out), out.nbytes),
                  self.tr._ctx)
        else:
            raise VtError(A.VT_ERR_ARG, f"readback kind {kind} (linear, rgb8, rgba8)")
        return out

    def visible(self, name, pointsD, **o):
        """lite_nodes/renderer.js:960 visible: SCOPE by its pinhole and image circle, the other cameras by the tracer."""
        c = self._cam(name)
        if c < len(self._names) - 1:
            return self.tr.visible(c, pointsD, **o)
        v = self.view(c)
        R = np.array([v[0:3], v[4:7], v[8:11]], np.float64)       # rows: camera axes in the dome frame
        d = np.asarray(pointsD, np.float64).reshape(-1, 3) - np.array(v[12:15], np.float64)
        x, y, z = d @ R[0], d @ R[1], d @ R[2]
        f = v[16]
        frac = self.o["scopeCircleFrac"] * self.o["scopeSize"][0] / 2.0
        with np.errstate(divide="ignore", invalid="ignore"):
            ok = (z > 0) & (np.hypot(f * x / z, f * y / z) < frac)
        return ok

    def converge(self, iters=200):
        """lite_nodes/renderer.js:979 converge: the tracer's full radiosity solve."""
        return self.tr.converge(iters)

    def info(self) -> dict:
        i = A.vt_lite_info()
        check(self.lib.vt_lite_info_get(self.tr._ctx, C.byref(i)), self.tr._ctx)
        return {"rasterTris": i.raster_tris, "staticTris": i.static_tris, "dynVerts": i.dyn_verts, "cameras": i.n_cameras,
                "loadMs": i.build_ms, "shadowStaticMs": i.shadow_static_ms, "shadowDynMs": i.shadow_dyn_ms, "cameraMs": i.camera_ms,
                "cameraRasterMs": i.camera_raster_ms, "cameraShadeMs": i.camera_shade_ms,
                "bigTiles": i.big_tris, "launches": i.launches, "shadowBigTiles": i.shadow_big_tiles}

    def timings(self) -> dict:
        """lite_nodes/renderer.js:982 timings: device ms of the last render's passes, load time, the tracer's."""
        return {"last": self.info(), "load_ms": self.stats["loadMs"], "stats": self.stats, "tracer": self.tr.timings()}

    # ------------------------------------------------------------------------------------------- stage buffers
    def view(self, name) -> np.ndarray:
        """The camera's view uniform (128 float32; misc words as their bits)."""
        out = np.zeros(128, np.float32)
        check(self.lib.vt_lite_debug(self.tr._ctx, A.VT_LITE_VIEW, self._cam(name), _p(out), out.nbytes), self.tr._ctx)
        return out

    def debug_buffer(self, what: int, name=0) -> np.ndarray:
        """A raster-pass buffer (VT_LITE_*) as a numpy array of its natural shape."""
        c = self._cam(name)
        info = self.info()
        nv = self.stats["dynVerts"] + len(self.scene["static"]["P"])
        res = int(self.o["smRes"])
        w, h = self.size(c)
        shapes = {A.VT_LITE_CLIP: ((nv, 4), np.float32), A.VT_LITE_KEYS: ((h, w, 4), np.uint64),
                  A.VT_LITE_SM_STATIC: ((4, res, res), np.uint32), A.VT_LITE_SM_DYN: ((4, res, res), np.uint32),
                  A.VT_LITE_SM_CLIP: ((4, nv, 4), np.float32), A.VT_LITE_GEOM: ((nv, 8), np.uint32),
                  A.VT_LITE_INDEX: ((info["rasterTris"], 3), np.uint32), A.VT_LITE_EMIT: ((int(self.o["nsDyn"]), 8), np.float32)}
        shape, dt = shapes[what]
        out = np.zeros(shape, dt)
        check(self.lib.vt_lite_debug(self.tr._ctx, int(what), c, _p(out), out.nbytes), self.tr._ctx)
        return out

    def destroy(self):
        if getattr(self, "tr", None) is not None:
            self.tr.destroy()
            self.tr = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


def lite_geometry(scene: dict, subdiv=0.003, subdiv_fixture=0.01):
    """The raster geometry on the host (vt_lite_geometry, no device needed): vertices (n x 8 words) and triangles
    (m x 3), as vt_lite_create builds them."""
    from ._lib import load

    lib = load()
    desc = A.SceneDesc(scene)
    cnt = np.zeros(2, np.uint32)
    check(lib.vt_lite_geometry(desc.ref, float(subdiv), float(subdiv_fixture), _p(cnt), None, None), None)
    V = np.zeros((int(cnt[0]), 8), np.uint32)
    I = np.zeros((int(cnt[1]), 3), np.uint32)
    check(lib.vt_lite_geometry(desc.ref, float(subdiv), float(subdiv_fixture), _p(cnt), _p(V), _p(I)), None)
    return V, I


def raster(lib_owner: TwinRenderer, clip, idx, width, height, samples=4) -> np.ndarray:
    """The rasteriser alone (vt_raster): uint64 keys (h x w x samples), depth bits << 32 | triangle."""
    clip = np.ascontiguousarray(clip, np.float32).reshape(-1, 4)
    idx = np.ascontiguousarray(idx, np.uint32).reshape(-1, 3)
    out = np.zeros((height, width, samples), np.uint64)
    check(lib_owner.lib.vt_raster(lib_owner._ctx, _p(clip), len(clip), _p(idx), len(idx), int(width), int(height), int(samples), _p(out)),
          lib_owner._ctx)
    return out
