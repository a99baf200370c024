"""ctypes mirror of include/vtwin.h (the C ABI), and the packing of a scene dict into vt_scene_desc.

Pure data layout: loading no library here.  `SceneDesc(scene)` keeps every numpy array it points at alive for
as long as the descriptor lives.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

VT_OK, VT_ERR_ARG, VT_ERR_CUDA, VT_ERR_OOM, VT_ERR_TIMEOUT, VT_ERR_STATE = 0, 1, 2, 3, 4, 5
VT_ERR_UNKNOWN_CAMERA, VT_ERR_TOO_MANY_BODIES, VT_ERR_NO_DEVICE, VT_ERR_NOT_CONVERGED = 6, 7, 8, 9
VT_SHADE_TWIN, VT_SHADE_PATH = 0, 1
VT_PREC_FP32, VT_PREC_BF16, VT_PREC_FP8, VT_PREC_FP32_TMA = 0, 1, 2, 3
VT_READ_LINEAR, VT_READ_RAW, VT_READ_RGBA8, VT_READ_RGB8, VT_READ_YUV420 = 0, 1, 2, 3, 4
VT_MAX_INST = 24
VT_MISS = 0xFFFFFFFF
BODY_KIND = {"instrument": 0, "scope": 1, "board": 2, "fixed": 3, "fixture": 4}
OPTION_BITS = {"CUT": 1, "AID": 2, "NO_INDIRECT": 4, "DIRECT_ONLY": 8, "LAYER": 16, "NO_CAPSULE": 32, "NORMALS": 64,
               "NO_MIS": 128, "SPEC_STATIC": 256, "PACKET": 512, "REFINE_SHADOW": 1024, "CACHE_WRITE": 2048, "CACHE_READ": 4096,
               "SHADOW_CACHE": 8192}

f32p = C.POINTER(C.c_float)
u32p = C.POINTER(C.c_uint32)
f64p = C.POINTER(C.c_double)


class vt_mesh(C.Structure):
    _fields_ = [("mat", C.c_uint32), ("flags", C.c_uint32), ("build_dir", C.c_float * 3),
                ("layer_period", C.c_float), ("layer_depth", C.c_float), ("overview_only", C.c_uint32)]


class vt_material(C.Structure):
    _fields_ = [("metallic", C.c_int32), ("coated", C.c_int32), ("emitter", C.c_int32), ("no_table", C.c_int32),
                ("rho", C.c_float * 3), ("f0", C.c_float * 3), ("roughness", C.c_float), ("ior", C.c_float),
                ("fbar", C.c_float), ("coat_ior", C.c_float), ("coat_roughness", C.c_float), ("tau", C.c_float * 3),
                ("textured", C.c_int32), ("ink_rho", C.c_float * 3), ("ink_roughness", C.c_float)]


class vt_body_desc(C.Structure):
    _fields_ = [("P", f32p), ("N", f32p), ("I", u32p), ("tri_mesh", u32p), ("UV", f32p),
                ("n_verts", C.c_uint32), ("n_tris", C.c_uint32), ("kind", C.c_int32), ("owner_camera", C.c_int32)]


class vt_camera_desc(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("fx", C.c_double), ("fy", C.c_double),
                ("cx", C.c_double), ("cy", C.c_double), ("alpha", C.c_double), ("k", C.c_double * 4),
                ("T_D_C", C.c_double * 16)]


class vt_scene_desc(C.Structure):
    _fields_ = [("static_P", f32p), ("static_N", f32p), ("static_I", u32p), ("static_tri_mesh", u32p),
                ("static_vert_mesh", u32p), ("n_static_verts", C.c_uint32), ("n_static_tris", C.c_uint32),
                ("bodies", C.POINTER(vt_body_desc)), ("n_bodies", C.c_uint32),
                ("meshes", C.POINTER(vt_mesh)), ("n_meshes", C.c_uint32),
                ("materials", C.POINTER(vt_material)), ("n_materials", C.c_uint32),
                ("L0", C.c_float * 3), ("profile_theta", f32p), ("profile_p", f32p), ("n_profile", C.c_uint32),
                ("axis_deg", C.c_float), ("cameras", C.POINTER(vt_camera_desc)), ("n_cameras", C.c_uint32)]


class vt_options(C.Structure):
    _fields_ = [("leaf_size", C.c_uint32), ("albedo_samples", C.c_uint32), ("device", C.c_int32)]


class vt_scene_info(C.Structure):
    _fields_ = [("node_count", C.c_uint32), ("tri_count", C.c_uint32), ("vert_count", C.c_uint32),
                ("param_vec4s", C.c_uint32), ("static_verts", C.c_uint32), ("static_tris", C.c_uint32),
                ("n_bodies", C.c_uint32), ("n_materials", C.c_uint32), ("n_meshes", C.c_uint32),
                ("emit_tris", C.c_uint32), ("mesh_off", C.c_uint32), ("mat_off", C.c_uint32),
                ("alb_off", C.c_uint32), ("prof_off", C.c_uint32), ("prof_n", C.c_uint32), ("emit_off", C.c_uint32),
                ("emit_area", C.c_float), ("emit_axis", C.c_float * 3), ("emit_normal", C.c_float * 3),
                ("emit_centroid", C.c_float * 3), ("emit_radius", C.c_float), ("shadow_skips_scope", C.c_int32),
                ("scope_index", C.c_int32)]


class vt_blas_info(C.Structure):
    _fields_ = [("root", C.c_uint32), ("tri_off", C.c_uint32), ("tri_count", C.c_uint32), ("bmin", C.c_float * 3),
                ("bmax", C.c_float * 3), ("cap_a", C.c_float * 3), ("cap_b", C.c_float * 3), ("cap_r", C.c_float),
                ("occ_a", C.c_float * 3), ("occ_b", C.c_float * 3), ("occ_r", C.c_float), ("rho_eff", C.c_float),
                ("kind", C.c_int32)]


VT_UNIT_LENS, VT_UNIT_BSDF, VT_UNIT_CAPSULE, VT_UNIT_PROFILE = 0, 1, 2, 3


class vt_unit_req(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("n", C.c_uint32), ("lens", C.c_float * 12)]


class vt_render_req(C.Structure):
    _fields_ = [("camera", C.c_uint32), ("spp", C.c_uint32), ("light_samples", C.c_uint32), ("seed", C.c_uint32),
                ("options", C.c_uint32), ("mode", C.c_uint32), ("max_depth", C.c_uint32), ("root", C.c_uint32),
                ("frame", C.c_uint32), ("shutter", C.c_float * 2), ("scale", C.c_float), ("refine", C.c_uint32),
                ("refine_light_samples", C.c_uint32)]


class vt_sensor_uniform(C.Structure):
    _fields_ = [("words", C.c_uint32 * 64)]


class vt_frame_req(C.Structure):
    _fields_ = [("cameras", C.POINTER(C.c_uint32)), ("n_cameras", C.c_uint32), ("render", vt_render_req),
                ("sensors", C.POINTER(vt_sensor_uniform)), ("stats", C.POINTER(C.c_uint32)), ("ms", C.c_double)]


VT_BATCH_MAX_POSES = 64


class vt_batch_req(C.Structure):
    _fields_ = [("cameras", C.POINTER(C.c_uint32)), ("n_cameras", C.c_uint32), ("n_poses", C.c_uint32),
                ("n_bodies", C.c_uint32), ("poses0", C.POINTER(C.c_double)), ("poses1", C.POINTER(C.c_double)),
                ("spp", C.c_uint32), ("light_samples", C.c_uint32), ("seed", C.c_uint32), ("options", C.c_uint32),
                ("max_depth", C.c_uint32), ("shutter", C.c_float * 2), ("scale", C.c_float),
                ("sensor", C.POINTER(vt_sensor_uniform)), ("frame0", C.c_uint32), ("optics_scale", C.c_float),
                ("use_graph", C.c_uint32), ("wave_paths", C.c_uint32)]


class vt_batch_stats(C.Structure):
    _fields_ = [("ms", C.c_double), ("shared_paths", C.c_uint64), ("pair_paths", C.c_uint64), ("samples", C.c_uint64),
                ("waves", C.c_uint32), ("graph_replayed", C.c_uint32), ("reruns", C.c_uint32), ("vary_mask", C.c_uint32)]


class vt_tune_row(C.Structure):
    _fields_ = [("wave_paths", C.c_uint32), ("tile_w", C.c_uint32), ("tile_h", C.c_uint32), ("ms_per_mpath", C.c_float),
                ("refill", C.c_uint32)]


class vt_calib_desc(C.Structure):
    _fields_ = [("n_nodes", C.c_uint32), ("lamp_samples", C.c_uint32)]


class vt_calib_info(C.Structure):
    _fields_ = [("n_nodes", C.c_uint32), ("n_materials", C.c_uint32), ("n_lamps", C.c_uint32), ("n_static_tris", C.c_uint32)]


class vt_calib_req(C.Structure):
    _fields_ = [("cameras", C.POINTER(C.c_uint32)), ("n_cameras", C.c_uint32), ("spp", C.c_uint32), ("light_samples", C.c_uint32),
                ("seed", C.c_uint32), ("max_depth", C.c_uint32), ("jacobi_iters", C.c_uint32),
                ("albedo", C.POINTER(C.c_double)), ("lamp", C.POINTER(C.c_double)), ("targets", C.POINTER(C.c_float)),
                ("images", C.POINTER(C.c_float)), ("replay", C.c_uint32), ("intrinsics", C.c_uint32)]


class vt_solve_req(C.Structure):
    _fields_ = [("n", C.c_uint32), ("n_rhs", C.c_uint32), ("F", f32p), ("rho", f32p), ("E", f32p), ("B", f32p),
                ("precision", C.c_uint32), ("max_iters", C.c_uint32), ("warm_start", C.c_uint32),
                ("check_every", C.c_uint32), ("reuse_f", C.c_uint32), ("tol", C.c_double), ("iters", C.c_uint32),
                ("refinements", C.c_uint32), ("residual", C.c_double), ("ms", C.c_double), ("sweep_ms", C.c_double),
                ("convert_ms", C.c_double)]


class vt_bvh_result(C.Structure):
    _fields_ = [("node_count", C.c_uint32), ("max_depth", C.c_uint32), ("bmin", C.c_float * 3),
                ("bmax", C.c_float * 3)]


class vt_nodes_opts(C.Structure):
    _fields_ = [("gather_k", C.c_uint32), ("node_samples", C.c_uint32), ("nbr_k", C.c_uint32), ("smooth_sigma", C.c_float),
                ("smooth_radius", C.c_float), ("radiosity_every", C.c_uint32), ("iters_per_frame", C.c_uint32),
                ("iters_initial", C.c_uint32), ("per_step_factors", C.c_uint32)]


class vt_lite_opts(C.Structure):
    _fields_ = [("ns_static", C.c_uint32), ("ns_dyn", C.c_uint32), ("sm_res", C.c_uint32), ("scope_width", C.c_uint32),
                ("scope_height", C.c_uint32), ("env_material", C.c_uint32), ("debug", C.c_uint32), ("reserved", C.c_uint32),
                ("sm_theta_max_deg", C.c_double), ("far_m", C.c_double), ("subdiv_h", C.c_double), ("subdiv_fixture", C.c_double),
                ("scope_hfov_deg", C.c_double), ("scope_circle_frac", C.c_double), ("scope_view_dir", C.c_double * 3),
                ("scope_objective", C.c_double * 3)]


class vt_lite_info(C.Structure):
    _fields_ = [("raster_tris", C.c_uint32), ("static_tris", C.c_uint32), ("dyn_verts", C.c_uint32), ("n_cameras", C.c_uint32),
                ("build_ms", C.c_double), ("shadow_static_ms", C.c_double), ("shadow_dyn_ms", C.c_double), ("camera_ms", C.c_double),
                ("camera_raster_ms", C.c_double), ("camera_shade_ms", C.c_double), ("big_tris", C.c_uint32), ("launches", C.c_uint32),
                ("shadow_big_tiles", C.c_uint32), ("reserved", C.c_uint32)]


class vt_mesh_out(C.Structure):
    _fields_ = [("P", C.POINTER(C.c_double)), ("N", C.POINTER(C.c_double)), ("I", C.POINTER(C.c_uint32)), ("n_verts", C.c_uint32),
                ("n_idx", C.c_uint32), ("handle", C.c_void_p)]


VT_LITE_VIEW, VT_LITE_CLIP, VT_LITE_KEYS, VT_LITE_SM_STATIC, VT_LITE_SM_DYN, VT_LITE_SM_CLIP, VT_LITE_GEOM, VT_LITE_INDEX, VT_LITE_EMIT = range(9)


class vt_nodes_info(C.Structure):
    _fields_ = [("n_nodes", C.c_uint32), ("n_active", C.c_uint32), ("gather_k", C.c_uint32), ("nbr_k", C.c_uint32),
                ("build_ms", C.c_double), ("neighbour_ms", C.c_double), ("table_entries", C.c_uint64)]


class vt_timings(C.Structure):
    _fields_ = [("render_ms", C.c_double), ("sensor_ms", C.c_double), ("solve_ms", C.c_double),
                ("trace_ms", C.c_double), ("launches", C.c_uint64), ("extend_ms", C.c_double), ("shade_ms", C.c_double),
                ("shadow_ms", C.c_double), ("extend_launches", C.c_uint64), ("shadow_launches", C.c_uint64),
                ("extend_rays", C.c_uint64), ("shadow_paths", C.c_uint64), ("node_direct_ms", C.c_double),
                ("node_jacobi_ms", C.c_double), ("node_jacobi_steps", C.c_uint32), ("reserved", C.c_uint32)]


def ptr(a: np.ndarray, ct):
    return a.ctypes.data_as(C.POINTER(ct)) if a is not None else None


def _c(a, dt):
    return np.ascontiguousarray(np.asarray(a, dt))


def material_struct(m: dict) -> vt_material:
    s = vt_material()
    s.metallic = int(m.get("metallic", 0))
    s.coated = int(m.get("coated", 0))
    s.emitter = int(m.get("emitter", 0))
    s.no_table = int(m.get("no_table", 0))
    s.rho[:] = [float(x) for x in m.get("rho", [0.5, 0.5, 0.5])]
    s.f0[:] = [float(x) for x in m.get("f0", [0.56, 0.57, 0.58])]
    s.roughness = float(m.get("roughness", 0.5))
    s.ior = float(m.get("ior", 1.5))
    fb = m.get("fbar", float("nan"))
    s.fbar = float("nan") if fb is None else float(fb)
    s.coat_ior = float(m.get("coat_ior", 1.5))
    s.coat_roughness = float(m.get("coat_roughness", 0.05))
    s.tau[:] = [float(x) for x in m.get("tau", [1.0, 1.0, 1.0])]
    s.textured = int(m.get("textured", 0))
    s.ink_rho[:] = [float(x) for x in m.get("ink_rho", [0.0, 0.0, 0.0])]
    s.ink_roughness = float(m.get("ink_roughness", 0.4))
    return s


class SceneDesc:
    """vt_scene_desc built from a scene dict (see vtwin.dome); `.desc` is the structure, `.ref` its pointer."""

    def __init__(self, scene: dict):
        keep = []
        st = scene["static"]
        P, N = _c(st["P"], np.float32), _c(st["N"], np.float32)
        I, tm, vm = _c(st["I"], np.uint32), _c(st["tri_mesh"], np.uint32), _c(st["vert_mesh"], np.uint32)
        keep += [P, N, I, tm, vm]
        d = vt_scene_desc()
        d.static_P, d.static_N, d.static_I = ptr(P, C.c_float), ptr(N, C.c_float), ptr(I, C.c_uint32)
        d.static_tri_mesh, d.static_vert_mesh = ptr(tm, C.c_uint32), ptr(vm, C.c_uint32)
        d.n_static_verts, d.n_static_tris = len(P), len(I)
        bodies = scene.get("bodies", [])
        barr = (vt_body_desc * max(1, len(bodies)))()
        for i, b in enumerate(bodies):
            bp, bn, bi, btm = _c(b["P"], np.float32), _c(b["N"], np.float32), _c(b["I"], np.uint32), _c(b["tri_mesh"], np.uint32)
            uv = _c(b["UV"], np.float32) if b.get("UV") is not None else None
            keep += [bp, bn, bi, btm, uv]
            barr[i].P, barr[i].N, barr[i].I, barr[i].tri_mesh = ptr(bp, C.c_float), ptr(bn, C.c_float), ptr(bi, C.c_uint32), ptr(btm, C.c_uint32)
            barr[i].UV = ptr(uv, C.c_float) if uv is not None else None
            barr[i].n_verts, barr[i].n_tris = len(bp), len(bi)
            barr[i].kind = BODY_KIND[b["kind"]] if isinstance(b["kind"], str) else int(b["kind"])
            barr[i].owner_camera = int(b.get("owner_camera", -1))
        d.bodies, d.n_bodies = barr, len(bodies)
        meshes = scene["meshes"]
        marr = (vt_mesh * len(meshes))()
        for i, m in enumerate(meshes):
            marr[i].mat, marr[i].flags = int(m["mat"]), int(m["flags"])
            marr[i].build_dir[:] = [float(x) for x in m.get("build_dir", [0, 0, 1])]
            lay = m.get("layer", [0.0, 0.0])
            marr[i].layer_period, marr[i].layer_depth = float(lay[0]), float(lay[1])
            marr[i].overview_only = int(bool(m.get("overview_only", False)))
        d.meshes, d.n_meshes = marr, len(meshes)
        mats = scene["materials"]
        tarr = (vt_material * len(mats))()
        for i, m in enumerate(mats):
            tarr[i] = material_struct(m)
        d.materials, d.n_materials = tarr, len(mats)
        em = scene["emitter"]
        d.L0[:] = [float(x) for x in em["L0"]]
        th, pp = _c(em["theta"], np.float32), _c(em["p"], np.float32)
        keep += [th, pp]
        d.profile_theta, d.profile_p, d.n_profile = ptr(th, C.c_float), ptr(pp, C.c_float), len(th)
        ad = em.get("axis_deg", float("nan"))
        d.axis_deg = float("nan") if ad is None else float(ad)
        cams = scene.get("cameras", [])
        carr = (vt_camera_desc * max(1, len(cams)))()
        for i, c in enumerate(cams):
            carr[i].width, carr[i].height = int(c["size"][0]), int(c["size"][1])
            carr[i].fx, carr[i].fy, carr[i].cx, carr[i].cy = c["fx"], c["fy"], c["cx"], c["cy"]
            carr[i].alpha = c.get("alpha", 0.0)
            carr[i].k[:] = [float(x) for x in c["k"]]
            carr[i].T_D_C[:] = [float(x) for x in np.asarray(c["T_D_C"], float).ravel()]
        d.cameras, d.n_cameras = carr, len(cams)
        self.desc = d
        self._keep = (keep, barr, marr, tarr, carr)
        self.ref = C.byref(self.desc)
        self.scene = scene


def lens_params(cam: dict) -> np.ndarray:
    """gpu/lens.js:8 lensParams flattened: fx, fy, cx, cy, alpha, k1..k4 (float64)."""
    return np.array([cam["fx"], cam["fy"], cam["cx"], cam["cy"], cam.get("alpha", 0.0)] + list(cam["k"]), np.float64)


def identity_poses(n_bodies: int) -> np.ndarray:
    return np.tile(np.eye(4).T.ravel(), (n_bodies, 1)).astype(np.float64)


NAN = math.nan
