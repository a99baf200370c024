"""ORACLE loader - test infrastructure only (tests/, __graft_entry__.smoke(), bench.py's CPU-baseline leg).

ctypes front of oracle/libvtoracle.so, the CPU restatement of the reference's rendering hot path
(see vt_oracle.cpp for what it restates and why its parity is unpinned). Nothing in the product imports this.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "veridien-twin_gb300"))
from vtwin import _abi as A  # noqa: E402  (struct layouts of include/vtwin.h)

LIB = os.path.join(HERE, "libvtoracle.so")
_lib = None


def build(force=False):
    src = os.path.join(HERE, "vt_oracle.cpp")
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(LIB)
        _lib.or_scene_create.restype = C.c_void_p
        _lib.or_scene_create.argtypes = [C.c_void_p, C.c_int, C.c_int]
        for nm in ("or_scene_destroy", "or_scene_sizes", "or_scene_arrays", "or_scene_emitter", "or_scene_blas",
                   "or_scene_set_poses", "or_scene_set_eavg", "or_scene_uniform", "or_scene_set_node_state",
                   "or_trace_wgsl", "or_render", "or_calib_render", "or_direct_transfer", "or_form_factors_visible",
                   "or_lite_geometry_size", "or_lite_geometry", "or_lite_emitter", "or_lite_vertex", "or_raster", "or_lite_shade",
                   "or_lite_display", "or_scene_load_uniform"):
            getattr(_lib, nm).restype = None
        _lib.or_fresnel_average.restype = C.c_double
        _lib.or_fresnel_dielectric.restype = C.c_double
        _lib.or_disc_irradiance.restype = C.c_double
        _lib.or_profile.restype = C.c_double
        _lib.or_capsule_occ.restype = C.c_double
        _lib.or_jacobi64.restype = C.c_int
        _lib.or_bvh_build.restype = C.c_int
        _lib.or_scene_emit_count.restype = C.c_uint32
    return _lib


def _p(a, ct=C.c_double):
    return a.ctypes.data_as(C.POINTER(ct))


def mulberry32(seed, n):
    out = np.zeros(n, np.float64)
    lib().or_mulberry32(C.c_uint32(seed), n, _p(out))
    return out


def unproject(lens, uv):
    uv = np.ascontiguousarray(uv, np.float64).reshape(-1, 2)
    out = np.zeros((len(uv), 3))
    lib().or_unproject(_p(np.ascontiguousarray(lens, np.float64)), len(uv), _p(uv), _p(out))
    return out


def project(lens, X):
    X = np.ascontiguousarray(X, np.float64).reshape(-1, 3)
    out = np.zeros((len(X), 2))
    lib().or_project(_p(np.ascontiguousarray(lens, np.float64)), len(X), _p(X), _p(out))
    return out


def bvh_build(pos, idx, leaf=4):
    pos = np.ascontiguousarray(pos, np.float32).ravel()
    idx = np.ascontiguousarray(idx, np.uint32).ravel()
    n = len(idx) // 3
    cap = max(4, -(-n // max(1, leaf)) * 2) * 4 + 16
    while True:
        nodes = np.zeros(cap * 16, np.uint32)
        order = np.zeros(max(1, n), np.uint32)
        info = np.zeros(7)
        cnt = lib().or_bvh_build(_p(pos, C.c_float), _p(idx, C.c_uint32), C.c_uint32(n), leaf, _p(nodes, C.c_uint32), cap,
                                 _p(order, C.c_uint32), _p(info))
        if cnt >= 0 or -cnt <= cap:
            break
        cap = -cnt   # the node count the build needs (many leaves smaller than `leaf`)
    assert cnt > 0, cnt
    return {"nodes": nodes[: cnt * 16].copy(), "node_count": cnt, "order": order[:n].copy(), "max_depth": int(info[0]),
            "bmin": info[1:4].copy(), "bmax": info[4:7].copy()}


def pack_triangles(pos, idx, order):
    pos = np.ascontiguousarray(pos, np.float32).ravel()
    idx = np.ascontiguousarray(idx, np.uint32).ravel()
    order = np.ascontiguousarray(order, np.uint32)
    T = np.zeros(len(order) * 16, np.float32)
    lib().or_pack_triangles(_p(pos, C.c_float), _p(idx, C.c_uint32), _p(order, C.c_uint32), C.c_uint32(len(order)), _p(T, C.c_float))
    return T


def traverse_js(nodes, T, o, d, tmin=0.0, tmax=np.inf, any_hit=False, root=0):
    """gpu/bvh.js:224 traverse in float64: returns (t, u, v, tri) arrays."""
    o = np.ascontiguousarray(o, np.float32).reshape(-1, 3)
    d = np.ascontiguousarray(d, np.float32).reshape(-1, 3)
    out = np.zeros((len(o), 4))
    lib().or_traverse_js(_p(np.ascontiguousarray(nodes, np.uint32), C.c_uint32), _p(np.ascontiguousarray(T, np.float32), C.c_float),
                         len(o), _p(o, C.c_float), _p(d, C.c_float), C.c_double(tmin), C.c_double(tmax), int(any_hit),
                         C.c_uint32(root), _p(out))
    return out[:, 0], out[:, 1], out[:, 2], out[:, 3].astype(np.int64)


def brute_force(T, count, o, d, tmin=0.0, tmax=np.inf):
    o = np.ascontiguousarray(o, np.float32).reshape(-1, 3)
    d = np.ascontiguousarray(d, np.float32).reshape(-1, 3)
    out = np.zeros((len(o), 4))
    lib().or_brute_force(_p(np.ascontiguousarray(T, np.float32), C.c_float), C.c_uint32(count), len(o), _p(o, C.c_float),
                         _p(d, C.c_float), C.c_double(tmin), C.c_double(tmax), _p(out))
    return out[:, 0], out[:, 1], out[:, 2], out[:, 3].astype(np.int64)


def fresnel_average(eta):
    return lib().or_fresnel_average(C.c_double(eta))


def fresnel_dielectric(cosi, eta):
    """gpu/bsdf.js:25 fresnelDielectric (unpolarised, FP64)."""
    return lib().or_fresnel_dielectric(C.c_double(cosi), C.c_double(eta))


def disc_irradiance(x, n, c, m, a, L, nr=48, nphi=96):
    f = lambda v: _p(np.ascontiguousarray(v, np.float64))
    return lib().or_disc_irradiance(f(x), f(n), f(c), f(m), C.c_double(a), C.c_double(L), nr, nphi)


def profile(theta, knots, p):
    knots = np.ascontiguousarray(knots, np.float64)
    p = np.ascontiguousarray(p, np.float64)
    return lib().or_profile(C.c_double(theta), _p(knots), _p(p), len(knots))


def capsule_occ(p, n, a, b, r):
    f = lambda v: _p(np.ascontiguousarray(v, np.float64))
    return lib().or_capsule_occ(f(p), f(n), f(a), f(b), C.c_double(r))


def bsdf_eval(material: dict, cases):
    m = A.material_struct(material)
    cases = np.ascontiguousarray(cases, np.float64).reshape(-1, 12)
    out = np.zeros((len(cases), 8))
    lib().or_bsdf_eval(C.byref(m), len(cases), _p(cases), _p(out))
    return out


def albedo_table(material: dict, samples=1024):
    m = A.material_struct(material)
    out = np.zeros(32 * 6 + 6)
    lib().or_albedo_table(C.byref(m), samples, _p(out))
    return {"spec": out[:96].reshape(32, 3), "diff": out[96:192].reshape(32, 3), "hh": out[192:195], "hhSpec": out[195:198]}


class Scene:
    """prepareScene restated (gpu/scene_gpu.js:241) + poses (gpu/renderer.js:620) + the estimator."""

    def __init__(self, scene: dict, leaf=4, albedo_samples=1024):
        self.sd = A.SceneDesc(scene)
        self.h = C.c_void_p(lib().or_scene_create(self.sd.ref, leaf, albedo_samples))
        self.scene = scene
        sz = np.zeros(12, np.uint32)
        lib().or_scene_sizes(self.h, _p(sz, C.c_uint32))
        (self.node_count, self.tri_count, self.vert_count, self.param_vec4s, self.static_verts, self.mesh_off,
         self.mat_off, self.alb_off, self.prof_off, self.prof_n, self.emit_off, self.emit_n) = [int(x) for x in sz]
        self.n_bodies = len(scene.get("bodies", []))
        self.slot, self.frame = 1, 0

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.or_scene_destroy(self.h)
            self.h = None

    def arrays(self):
        nodes = np.zeros(self.node_count * 16, np.uint32)
        tris = np.zeros(self.tri_count * 16, np.uint32)
        verts = np.zeros(self.vert_count * 8, np.uint32)
        params = np.zeros(self.param_vec4s * 4, np.float32)
        lib().or_scene_arrays(self.h, _p(nodes, C.c_uint32), _p(tris, C.c_uint32), _p(verts, C.c_uint32), _p(params, C.c_float))
        return {"nodes": nodes, "tris": tris, "verts": verts, "params": params}

    def emitter(self):
        out = np.zeros(13)
        lib().or_scene_emitter(self.h, _p(out))
        return {"area": out[0], "axis": out[1:4], "normal": out[4:7], "centroid": out[7:10], "radius": out[10],
                "shadow_skips_scope": bool(out[11]), "scope_index": int(out[12])}

    def blas(self, i):
        out = np.zeros(17)
        lib().or_scene_blas(self.h, i, _p(out))
        return {"root": int(out[0]), "tri_off": int(out[1]), "tri_count": int(out[2]), "bmin": out[3:6], "bmax": out[6:9],
                "cap_a": out[9:12], "cap_b": out[12:15], "cap_r": out[15], "rho_eff": out[16]}

    def set_poses(self, T0=None, T1=None):
        T0 = A.identity_poses(self.n_bodies) if T0 is None else np.ascontiguousarray(T0, np.float64).reshape(-1, 16)
        T1p = None if T1 is None else _p(np.ascontiguousarray(T1, np.float64).reshape(-1, 16))
        self._T = (T0, T1)
        lib().or_scene_set_poses(self.h, _p(T0), T1p, C.c_uint32(len(T0)), C.c_uint32(self.slot), C.c_uint32(self.frame))

    def set_eavg(self, e):
        e = np.ascontiguousarray(e, np.float32)
        lib().or_scene_set_eavg(self.h, _p(e, C.c_float), C.c_uint32(self.slot), C.c_uint32(self.frame))

    def set_node_state(self, st, slot=1):
        st = np.ascontiguousarray(st, np.float32)
        self.slot = slot
        lib().or_scene_set_node_state(self.h, _p(st, C.c_float), C.c_uint32(slot), C.c_uint32(self.frame))

    def uniform(self):
        out = np.zeros(24 + 48 * 24, np.float32)
        lib().or_scene_uniform(self.h, _p(out, C.c_float))
        return out

    def trace(self, o4, d4, mask=3, any_hit=False, root=0, fp64=True):
        o4 = np.ascontiguousarray(o4, np.float32).reshape(-1, 4)
        d4 = np.ascontiguousarray(d4, np.float32).reshape(-1, 4)
        out = np.zeros((len(o4), 5))
        dbg = np.zeros(16, np.uint64)
        lib().or_trace_wgsl(self.h, len(o4), _p(o4, C.c_float), _p(d4, C.c_float), C.c_uint32(mask), int(any_hit),
                            C.c_uint32(root), int(fp64), _p(out), _p(dbg, C.c_uint64))
        return out, dbg

    def unit_test(self, kind, tin, lens=None, fp64=False):
        """gpu/wgsl/kernels.wgsl.js:494-551 lensTest / bsdfTest / capsuleTest / profileTest restated (kind 0..3), with
        the reference's float4 slots; lens = (fx, fy, cx, cy, k1..k4, alpha). fp64=False: the float32 WGSL order."""
        slots_in, slots_out = {0: (2, 2), 1: (4, 3), 2: (4, 1), 3: (1, 1)}[int(kind)]
        tin = np.ascontiguousarray(tin, np.float32).reshape(-1, 4)
        n = len(tin) // slots_in
        out = np.zeros((n * slots_out, 4), np.float32)
        lz = np.zeros(9) if lens is None else np.ascontiguousarray(lens, np.float64)
        lib().or_unit_test(self.h, C.c_uint32(int(kind)), _p(lz), int(n), _p(tin, C.c_float), _p(out, C.c_float), int(fp64))
        return out

    def render(self, req: "A.vt_render_req", y0=0, y1=None, x0=0, x1=None, fp64=True, threads=1):
        cam = self.scene["cameras"][req.camera]
        W, H = cam["size"]
        y1 = H if y1 is None else y1
        x1 = W if x1 is None else x1
        out = np.zeros((y1 - y0, x1 - x0, 4))
        dbg = np.zeros(16, np.uint64)
        lib().or_render(self.h, C.byref(req), C.c_uint32(y0), C.c_uint32(y1), C.c_uint32(x0), C.c_uint32(x1), int(fp64),
                        int(threads), _p(out), _p(dbg, C.c_uint64))
        return out, dbg

    # ----------------------------------------------------------------------------------------- calibration
    def calib_render(self, camera, albedo, lamp, H, tri_node, spp=4, nl=1, seed=0, depth=3, y0=0, y1=None, fp64=True, threads=1,
                     frozen=None, K=None):
        """The calibration estimator of the CUDA library restated: rows [y0, y1) of a camera's image (h, w, 3).
        frozen = (tri_inst (h, w, spp, 4, 2), q (h, w, spp, 4, 4)): replay every path on the given triangles' planes
        with the given shadow outcomes (q = 0 occluded), so the image moves smoothly with the intrinsics K (fx, fy,
        cx, cy, k1..k4; None: the scene camera's)."""
        cam = self.scene["cameras"][camera]
        W, Hh = cam["size"]
        y1 = Hh if y1 is None else y1
        alb = np.ascontiguousarray(albedo, np.float64).ravel()
        lam = np.ascontiguousarray(lamp, np.float64).ravel()
        Hn = np.ascontiguousarray(H, np.float64).ravel()
        tn = np.ascontiguousarray(tri_node, np.uint32)
        out = np.zeros((y1 - y0, W, 3))
        ti = qq = None
        if frozen is not None:
            ti = np.ascontiguousarray(frozen[0], np.uint32)
            qq = np.ascontiguousarray(frozen[1], np.float32)
        Kd = None if K is None else np.ascontiguousarray(K, np.float64)
        lib().or_calib_render_frozen(self.h, C.c_uint32(camera), C.c_uint32(spp), C.c_uint32(nl), C.c_uint32(seed), C.c_uint32(depth),
                                     _p(alb), _p(lam), _p(Hn), C.c_uint32(len(Hn) // 3), _p(tn, C.c_uint32), C.c_uint32(y0), C.c_uint32(y1),
                                     int(fp64), int(threads), _p(ti, C.c_uint32) if ti is not None else None,
                                     _p(qq, C.c_float) if qq is not None else None, _p(Kd) if Kd is not None else None, _p(out))
        return out

    def direct_transfer(self, centres, normals, samples=16, fp64=True, threads=1):
        """Irradiance at each node from each emitter triangle at unit radiance (n x n_lamps), with visibility."""
        Cn = np.ascontiguousarray(centres, np.float32)
        Nn = np.ascontiguousarray(normals, np.float32)
        n = len(Cn)
        D = np.zeros((n, int(lib().or_scene_emit_count(self.h))))
        lib().or_direct_transfer(self.h, _p(Cn, C.c_float), _p(Nn, C.c_float), C.c_uint32(n), C.c_uint32(samples), int(fp64), int(threads),
                                 _p(D))
        return D

    def ri_map(self, camera, pupil_exponent=1.0, vig_theta_deg=(0.0, 90.0), vig=(1.0, 1.0)):
        """gpu/sensor.js:98 relativeIlluminationMap of a camera (h x w float32, FP64 arithmetic)."""
        W, H = self.scene["cameras"][camera]["size"]
        vt = np.ascontiguousarray(vig_theta_deg, np.float64)
        vv = np.ascontiguousarray(vig, np.float64)
        out = np.zeros((H, W), np.float32)
        lib().or_scene_ri_map(self.h, C.c_uint32(camera), C.c_double(pupil_exponent), _p(vt), _p(vv), C.c_uint32(len(vt)), _p(out, C.c_float))
        return out

    # ------------------------------------------------------------------------------------- node radiosity
    def gather_table(self, K=64, fp64=True, threads=8):
        """The gather table of every static vertex (n x K node ids, MISS = escape) and the escapes per node."""
        n = self.static_verts
        g = np.zeros(n * K, np.uint32)
        m = np.zeros(n, np.float32)
        lib().or_gather_table(self.h, C.c_uint32(K), int(fp64), int(threads), _p(g, C.c_uint32), _p(m, C.c_float))
        return g.reshape(n, K), m

    def node_neighbours(self, active, nbr_k=16, radius=0.006, sigma=0.003):
        """Smoothing neighbours by brute force: (n_active, nbr_k, 2) uint32 (active index, float weight bits)."""
        act = np.ascontiguousarray(active, np.uint32)
        out = np.zeros(len(act) * nbr_k * 2, np.uint32)
        lib().or_node_neighbours(self.h, _p(act, C.c_uint32), C.c_uint32(len(act)), C.c_uint32(nbr_k), C.c_double(radius),
                                 C.c_double(sigma), _p(out, C.c_uint32))
        return out.reshape(len(act), nbr_k, 2)

    def node_direct(self, active, state, node_samples=4, moved=0, fp64=True, threads=8):
        """nodeDirect of the active nodes applied to a copy of `state` (n x 16, float64)."""
        act = np.ascontiguousarray(active, np.uint32)
        st = np.array(state, np.float64).reshape(-1, 16).copy()
        lib().or_node_direct(self.h, _p(act, C.c_uint32), C.c_uint32(len(act)), C.c_uint32(node_samples), C.c_uint32(moved), int(fp64),
                             int(threads), _p(st))
        return st

    def node_jacobi(self, gtable, active, nbr, state, slot, iters, fp64=True, threads=8):
        """`iters` Jacobi steps of the node transport on a copy of `state`; returns (state, final slot)."""
        g = np.ascontiguousarray(gtable, np.uint32)
        act = np.ascontiguousarray(active, np.uint32)
        nb = np.ascontiguousarray(nbr, np.uint32)
        st = np.array(state, np.float64).reshape(-1, 16).copy()
        out = lib().or_node_jacobi(self.h, _p(g, C.c_uint32), C.c_uint32(g.shape[1]), _p(act, C.c_uint32), C.c_uint32(len(act)),
                                   _p(nb, C.c_uint32), C.c_uint32(nb.shape[1]), C.c_uint32(slot), C.c_uint32(iters), int(fp64), int(threads),
                                   _p(st))
        return st, int(out)

    def set_solved_caps(self, caps):
        """Bounding capsules of the last node update (n_bodies x 8), written to the scene uniform."""
        c = np.ascontiguousarray(caps, np.float32)
        lib().or_scene_set_solved_caps(self.h, _p(c, C.c_float), C.c_uint32(len(c) // 8 if c.ndim == 1 else len(c)),
                                       C.c_uint32(self.slot), C.c_uint32(self.frame))

    # ---- raster pass (lite_nodes)
    def lite_geometry(self, subdiv=0.003, subdiv_fixture=0.01):
        """Raster vertices (n x 8 words) and triangles (m x 3) of lite_nodes/renderer.js:527 _buildGeometry."""
        cnt = np.zeros(2, np.uint32)
        lib().or_lite_geometry_size(self.h, C.c_double(subdiv), C.c_double(subdiv_fixture), _p(cnt, C.c_uint32))
        V = np.zeros((int(cnt[0]), 8), np.uint32)
        I = np.zeros((int(cnt[1]), 3), np.uint32)
        lib().or_lite_geometry(self.h, C.c_double(subdiv), C.c_double(subdiv_fixture), _p(V, C.c_uint32), _p(I, C.c_uint32))
        return V, I

    def lite_emitter(self, n, T_scope):
        """The n emitter samples in the world (n x 8 float32) for the scope pose (column-major 4x4) and the four
        sector origins in the scope frame."""
        T = np.ascontiguousarray(T_scope, np.float64).reshape(16)
        out = np.zeros((n, 8), np.float32)
        sc = np.zeros((4, 3))
        lib().or_lite_emitter(self.h, C.c_uint32(n), _p(T), _p(out, C.c_float), _p(sc))
        return out, sc

    def lite_vertex(self, view, verts, shadow=0, base=None):
        """Clip coordinates of the raster vertices for a view (128 float32): camera (n x 4) or, shadow = 1 / 2, the
        static / dynamic casters' four sector layers (4 x n x 4, other vertices taken from `base`)."""
        v = np.ascontiguousarray(view, np.float32)
        V = np.ascontiguousarray(verts, np.uint32)
        n = len(V)
        out = np.zeros((n, 4) if not shadow else (4, n, 4), np.float32) if base is None else np.array(base, np.float32, copy=True)
        lib().or_lite_vertex(self.h, _p(v, C.c_float), _p(V, C.c_uint32), C.c_uint32(n), int(shadow), _p(out, C.c_float))
        return out

    def load_uniform(self, su):
        s = np.ascontiguousarray(su, np.float32)
        lib().or_scene_load_uniform(self.h, _p(s, C.c_float))

    def lite_shade(self, view, verts, idx, clip, keys, es, sm_static, sm_dyn, inv_scale, circle=0.0, y0=0, y1=None, threads=8):
        """Fragment stage + resolve + finish (h x w x 4 float32) from the given per-sample keys, clip coordinates and
        shadow maps."""
        v = np.ascontiguousarray(view, np.float32)
        W, H = int(v[24]), int(v[25])
        out = np.zeros((H, W, 4), np.float32)
        res = int(np.asarray(sm_static).shape[-1])
        lib().or_lite_shade(self.h, _p(v, C.c_float), _p(np.ascontiguousarray(verts, np.uint32), C.c_uint32),
                            _p(np.ascontiguousarray(idx, np.uint32), C.c_uint32), _p(np.ascontiguousarray(clip, np.float32), C.c_float),
                            _p(np.ascontiguousarray(keys, np.uint64), C.c_uint64), _p(np.ascontiguousarray(es, np.float32), C.c_float),
                            _p(np.ascontiguousarray(sm_static, np.uint32), C.c_uint32), _p(np.ascontiguousarray(sm_dyn, np.uint32), C.c_uint32),
                            C.c_uint32(res), C.c_float(inv_scale), C.c_float(circle), C.c_uint32(y0), C.c_uint32(H if y1 is None else y1),
                            int(threads), _p(out, C.c_float))
        return out

    def form_factors_visible(self, centres, normals, areas, rays=16, fp64=True, threads=1):
        """Dense node form factors with visibility through this scene (n x n float32) and the visible-ray counts."""
        Cn = np.ascontiguousarray(centres, np.float32)
        Nn = np.ascontiguousarray(normals, np.float32)
        An = np.ascontiguousarray(areas, np.float32)
        n = len(Cn)
        F = np.zeros((n, n), np.float32)
        cnt = np.zeros((n, n), np.uint8)
        lib().or_form_factors_visible(self.h, n, _p(Cn, C.c_float), _p(Nn, C.c_float), _p(An, C.c_float), int(rays), int(fp64), int(threads),
                                      _p(F, C.c_float), _p(cnt, C.c_uint8))
        return F, cnt


def calib_radiosity(F, D, lamp, albedo, node_mat):
    """The calibration model's node radiosity in FP64: B_c = rho_c o (D L + F B_c) by a direct solve per channel;
    returns H = F B (3 x n) and B."""
    F = np.asarray(F, np.float64)
    n = len(F)
    DL = np.asarray(D, np.float64) @ np.asarray(lamp, np.float64)
    H = np.zeros((3, n))
    B = np.zeros((3, n))
    for c in range(3):
        rho = np.asarray(albedo, np.float64)[np.asarray(node_mat), c]
        B[c] = np.linalg.solve(np.eye(n) - rho[:, None] * F, rho * DL)
        H[c] = F @ B[c]
    return H, B


def sensor_expose(su_words, E4):
    su = np.ascontiguousarray(su_words, np.uint32)
    E4 = np.ascontiguousarray(E4, np.float32)
    W, H = int(su[0]), int(su[1])
    raw = np.zeros((H, W), np.float32)
    lib().or_sensor_expose(_p(su, C.c_uint32), _p(E4, C.c_float), _p(raw, C.c_float))
    return raw


def vt_math(name, x):
    x = np.ascontiguousarray(x, np.float32)
    out = np.zeros_like(x)
    getattr(lib(), "or_vt_" + name)(_p(x, C.c_float), len(x), _p(out, C.c_float))
    return out


def solve_dense(F, rho, E):
    F = np.ascontiguousarray(F, np.float32)
    n = F.shape[0]
    E = np.ascontiguousarray(E, np.float32).reshape(n, -1)
    B = np.zeros(E.shape, np.float64)
    lib().or_solve_dense(n, _p(F, C.c_float), _p(np.ascontiguousarray(rho, np.float32), C.c_float), _p(E, C.c_float),
                         E.shape[1], _p(B))
    return B


def jacobi64(F, rho, E, tol=1e-12, max_it=10000, threads=None):
    F = np.ascontiguousarray(F, np.float32)
    n = F.shape[0]
    E = np.ascontiguousarray(E, np.float32).reshape(n, -1)
    B = np.zeros(E.shape, np.float64)
    it = lib().or_jacobi64(n, _p(F, C.c_float), _p(np.ascontiguousarray(rho, np.float32), C.c_float), _p(E, C.c_float),
                           E.shape[1], _p(B), C.c_double(tol), max_it, threads or os.cpu_count() or 1)
    return B, it


def form_factors(C_, N_, A_):
    C_ = np.ascontiguousarray(C_, np.float32)
    n = len(C_)
    F = np.zeros((n, n), np.float32)
    lib().or_form_factors(n, _p(C_, C.c_float), _p(np.ascontiguousarray(N_, np.float32), C.c_float),
                          _p(np.ascontiguousarray(A_, np.float32), C.c_float), _p(F, C.c_float))
    return F


def isp_chain(su_words, radiance, ri):
    """The sensor chain restated (gpu/wgsl/sensor.wgsl.js:67-427): radiance (h, w, 4) float32, relative illumination
    (h, w) -> raw DN (h, w) float32, 8-bit RGBA (h, w, 4), YCbCr planes (y, cb, cr) and the stats words."""
    su = np.ascontiguousarray(su_words, np.uint32)
    L = np.ascontiguousarray(radiance, np.float32)
    R = np.ascontiguousarray(ri, np.float32)
    W, H = int(su[0]), int(su[1])
    cw, ch = (W + 1) // 2, (H + 1) // 2
    raw = np.zeros((H, W), np.float32)
    rgba = np.zeros((H, W, 4), np.uint8)
    yuv = np.zeros(W * H + 2 * cw * ch, np.uint8)
    st = np.zeros(4, np.uint32)
    lib().or_isp_chain(_p(su, C.c_uint32), _p(L, C.c_float), _p(R, C.c_float), _p(raw, C.c_float), _p(rgba, C.c_uint8), _p(yuv, C.c_uint8),
                       _p(st, C.c_uint32))
    planes = {"y": yuv[:W * H].reshape(H, W), "cb": yuv[W * H:W * H + cw * ch].reshape(ch, cw), "cr": yuv[W * H + cw * ch:].reshape(ch, cw)}
    return raw, rgba, planes, st


def raster(clip, idx, width, height, samples=4, t0=0, nt=None):
    """The rasteriser restated: keys (h x w x samples uint64: depth bits << 32 | triangle; 1 sample: triangle bits
    all ones), all ones where nothing passed."""
    c = np.ascontiguousarray(clip, np.float32).reshape(-1, 4)
    I = np.ascontiguousarray(idx, np.uint32).reshape(-1, 3)
    nt = len(I) - t0 if nt is None else nt
    keys = np.zeros((height, width, samples), np.uint64)
    lib().or_raster(_p(c, C.c_float), _p(I, C.c_uint32), C.c_uint32(t0), C.c_uint32(nt), C.c_uint32(width), C.c_uint32(height),
                    C.c_uint32(samples), _p(keys, C.c_uint64))
    return keys


def lite_display(du, prev, radiance):
    """The raster pass's display look restated (lite_nodes/renderer.js:369): rgba8 (h x w x 4) and stats."""
    L = np.ascontiguousarray(radiance, np.float32)
    H, W = L.shape[:2]
    rgba = np.zeros((H, W, 4), np.uint8)
    st = np.zeros(4, np.uint32)
    lib().or_lite_display(_p(np.ascontiguousarray(du, np.float32), C.c_float), _p(np.ascontiguousarray(prev, np.uint32), C.c_uint32),
                          _p(L, C.c_float), C.c_uint32(W), C.c_uint32(H), _p(rgba, C.c_uint8), _p(st, C.c_uint32))
    return rgba, st



# ---- scene preparation (gpu/scene_gpu.js:37-165), restated in plain Python for small meshes
def _js_round(x):
    return math.floor(x + 0.5)


def _js_hypot3(x, y, z):
    v = [abs(x), abs(y), abs(z)]
    mx = max(v)
    if mx == 0:
        return 0.0
    s = c = 0.0
    for a in v:
        n = a / mx
        summand = n * n - c
        pre = s + summand
        c = (pre - s) - summand
        s = pre
    return math.sqrt(s) * mx


def weld_ref(P, N, I):
    P = np.asarray(P, np.float32).reshape(-1, 3).astype(np.float64)
    N = np.asarray(N, np.float32).reshape(-1, 3).astype(np.float64)
    seen, P2, N2, remap = {}, [], [], []
    for v in range(len(P)):
        k = tuple(_js_round(float(x) * 1e7) for x in P[v]) + tuple(_js_round(float(x) * 1e4) for x in N[v])
        if k not in seen:
            seen[k] = len(P2)
            P2.append(P[v]); N2.append(N[v])
        remap.append(seen[k])
    I2 = []
    for t in np.asarray(I, np.uint32).reshape(-1, 3):
        a, b, c = remap[t[0]], remap[t[1]], remap[t[2]]
        if a == b or b == c or a == c:
            continue
        I2 += [a, b, c]
    return np.array(P2).reshape(-1, 3), np.array(N2).reshape(-1, 3), np.array(I2, np.uint32)


def subdivide_ref(P, N, I, h, max_passes=24):
    P = [list(map(float, p)) for p in np.asarray(P, np.float64).reshape(-1, 3)]
    N = [list(map(float, n)) for n in np.asarray(N, np.float64).reshape(-1, 3)]
    tris = [int(x) for x in np.asarray(I).ravel()]
    h2 = h * h
    len2 = lambda a, b: (P[a][0] - P[b][0]) ** 2 + (P[a][1] - P[b][1]) ** 2 + (P[a][2] - P[b][2]) ** 2
    for _ in range(max_passes):
        mid, anyc = {}, False

        def midpoint(a, b):
            key = (min(a, b), max(a, b))
            if key in mid:
                return mid[key]
            m = len(P)
            P.append([0.5 * (P[a][k] + P[b][k]) for k in range(3)])
            n = [N[a][k] + N[b][k] for k in range(3)]
            l = _js_hypot3(*n)
            N.append([x / l for x in n] if l > 1e-6 else list(N[a]))
            mid[key] = m
            return m

        out = []
        for k in range(0, len(tris), 3):
            v = tris[k:k + 3]
            mk = [len2(v[0], v[1]) > h2, len2(v[1], v[2]) > h2, len2(v[2], v[0]) > h2]
            cnt = sum(mk)
            if not cnt:
                out += v
                continue
            anyc = True
            if cnt == 3:
                a, b, c = midpoint(v[0], v[1]), midpoint(v[1], v[2]), midpoint(v[2], v[0])
                out += [v[0], a, c, a, v[1], b, c, b, v[2], a, b, c]
            elif cnt == 1:
                e = mk.index(True)
                p, q, r = v[e], v[(e + 1) % 3], v[(e + 2) % 3]
                m = midpoint(p, q)
                out += [p, m, r, m, q, r]
            else:
                e = mk.index(False)
                Aa, Bb, Cc = v[e], v[(e + 1) % 3], v[(e + 2) % 3]
                mBC, mCA = midpoint(Bb, Cc), midpoint(Cc, Aa)
                out += [mCA, mBC, Cc]
                out += [Aa, Bb, mBC, Aa, mBC, mCA] if len2(Aa, mBC) < len2(Bb, mCA) else [Aa, Bb, mCA, Bb, mBC, mCA]
        tris = out
        if not anyc:
            break
    return np.array(P), np.array(N), np.array(tris, np.uint32)


def bench_mesh_ref(z, extent, fine, h):
    (ex0, ey0), (ex1, ey1) = extent
    fx0, fy0, fx1, fy1 = max(ex0, fine[0][0]), max(ey0, fine[0][1]), min(ex1, fine[1][0]), min(ey1, fine[1][1])
    nx, ny = max(1, math.ceil((fx1 - fx0) / (h * 0.999))), max(1, math.ceil((fy1 - fy0) / (h * 0.999)))
    P, I = [], []

    def v(x, y):
        P.append([x, y, z])
        return len(P) - 1

    grid = [[v(fx0 + (fx1 - fx0) * i / nx, fy0 + (fy1 - fy0) * j / ny) for i in range(nx + 1)] for j in range(ny + 1)]
    for j in range(ny):
        for i in range(nx):
            a, b, c, d = grid[j][i], grid[j][i + 1], grid[j + 1][i], grid[j + 1][i + 1]
            I += [a, b, d, a, d, c] if (i + j) & 1 else [a, b, c, b, d, c]

    def quad(x0, y0, x1, y1):
        if not (x1 > x0 and y1 > y0):
            return
        a, b, c, d = v(x0, y0), v(x1, y0), v(x0, y1), v(x1, y1)
        I.extend([a, b, d, a, d, c])

    quad(ex0, ey0, ex1, fy0); quad(ex0, fy1, ex1, ey1); quad(ex0, fy0, fx0, fy1); quad(fx1, fy0, ex1, fy1)
    return np.array(P), np.tile([0.0, 0.0, 1.0], (len(P), 1)), np.array(I, np.uint32)


def compute_normals_ref(P, I):
    P = np.asarray(P, np.float32).reshape(-1, 3)
    N = np.zeros_like(P)
    for t in np.asarray(I).reshape(-1, 3):
        a, b, c = (P[i].astype(np.float64) for i in t)
        u, w = b - a, c - a
        n = [u[1] * w[2] - u[2] * w[1], u[2] * w[0] - u[0] * w[2], u[0] * w[1] - u[1] * w[0]]
        for i in t:
            for k in range(3):
                N[i, k] = np.float32(float(N[i, k]) + n[k])
    for i in range(len(N)):
        l = _js_hypot3(float(N[i, 0]), float(N[i, 1]), float(N[i, 2])) or 1.0
        N[i] = [np.float32(float(N[i, k]) / l) for k in range(3)]
    return N
