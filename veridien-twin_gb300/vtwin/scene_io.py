"""Loading a twin scene directory (scene.json + meshes/*.bin) into the scene dict that TwinRenderer.create takes:
the front half of gpu/scene_gpu.js:241 prepareScene (static meshes welded and subdivided to the node spacing, the
bench mesh, bodies by bodyOfPart, the mesh table and its flags, materials and the emitter from physics), with the
mesh clean-up in libvtwin (vt_weld, vt_subdivide, vt_bench_mesh, vt_compute_normals on the host; weld and subdivide
also on a CUDA device, vt_weld_device / vt_subdivide_device, with identical results). The packing, BVHs, capsules and
albedo tables are vt_create's.
"""
from __future__ import annotations

import ctypes as C
import json
import math
import os

import numpy as np

from . import _abi as A
from ._lib import VtError, check, load

MESH_FLAG = {"STATIC": 1, "EMITTER": 2, "LAYER": 4, "BOARD": 8, "INSTRUMENT": 16, "SCOPE": 32, "BENCH": 64, "TEXTURED": 128}


def _unwrap(x):
    return x["value"] if isinstance(x, dict) and "value" in x else x


def _take(out: A.vt_mesh_out):
    lib = load()
    try:
        nv, ni = int(out.n_verts), int(out.n_idx)
        P = np.ctypeslib.as_array(out.P, (nv * 3,)).reshape(nv, 3).copy() if nv else np.zeros((0, 3))
        N = np.ctypeslib.as_array(out.N, (nv * 3,)).reshape(nv, 3).copy() if nv else np.zeros((0, 3))
        I = np.ctypeslib.as_array(out.I, (ni,)).copy() if ni else np.zeros(0, np.uint32)
    finally:
        lib.vt_mesh_free(C.byref(out))
    return P, N, I


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


# ------------------------------------------------------------------------------------------- mesh clean-up
def weld(P, N, I, device=None):
    """gpu/scene_gpu.js:68 weld: vertices merged by position (1e-7 m) and normal (1e-4); float64 out. device: a CUDA
    ordinal to weld on (the same result), None for the host."""
    P = np.ascontiguousarray(P, np.float32).reshape(-1, 3)
    N = np.ascontiguousarray(N, np.float32).reshape(-1, 3)
    I = np.ascontiguousarray(I, np.uint32).ravel()
    out = A.vt_mesh_out()
    if device is None:
        check(load().vt_weld(_p(P), _p(N), len(P), _p(I), len(I), C.byref(out)))
    else:
        check(load().vt_weld_device(int(device), _p(P), _p(N), len(P), _p(I), len(I), C.byref(out)))
    return _take(out)


def subdivide(P, N, I, h, max_passes=24, device=None):
    """gpu/scene_gpu.js:95 subdivide: conforming edge bisection until every edge is <= h. device: a CUDA ordinal to
    subdivide on (the same result), None for the host."""
    P = np.ascontiguousarray(P, np.float64).reshape(-1, 3)
    N = np.ascontiguousarray(N, np.float64).reshape(-1, 3)
    I = np.ascontiguousarray(I, np.uint32).ravel()
    out = A.vt_mesh_out()
    if device is None:
        check(load().vt_subdivide(_p(P), _p(N), len(P), _p(I), len(I), float(h), int(max_passes), C.byref(out)))
    else:
        check(load().vt_subdivide_device(int(device), _p(P), _p(N), len(P), _p(I), len(I), float(h), int(max_passes), C.byref(out)))
    return _take(out)


def bench_mesh(z, extent, fine, h):
    """gpu/scene_gpu.js:146 benchMesh: extent / fine = ((x0, y0), (x1, y1))."""
    e = np.array([extent[0][0], extent[0][1], extent[1][0], extent[1][1]], np.float64)
    f = np.array([fine[0][0], fine[0][1], fine[1][0], fine[1][1]], np.float64)
    out = A.vt_mesh_out()
    check(load().vt_bench_mesh(float(z), _p(e), _p(f), float(h), C.byref(out)))
    return _take(out)


def compute_normals(P, I):
    """gpu/scene_gpu.js:37 computeNormals (float32)."""
    P = np.ascontiguousarray(P, np.float32).reshape(-1, 3)
    I = np.ascontiguousarray(I, np.uint32).ravel()
    N = np.zeros_like(P)
    check(load().vt_compute_normals(_p(P), len(P), _p(I), len(I), _p(N)))
    return N


# ------------------------------------------------------------------------------------------- files
def decode_mesh(meta: dict, buf: bytes) -> dict:
    """gpu/scene_gpu.js:22 decodeMesh: one mesh's .bin by its layout block ([byteOffset, count] per array, a count
    of vertices or of scalars); normals computed when the mesh ships none."""
    lay = meta["layout"]
    nv, nt = int(meta["vertex_count"]), int(meta["triangle_count"])
    vec = lambda c: nv if (c == nv * 3 and nv * 3 != nv) else c
    idx = lambda c: nt * 3 if c == nt else c
    po, pc = lay["positions"]
    io, ic = lay["indices"]
    P = np.frombuffer(buf, np.float32, vec(pc) * 3, po).reshape(-1, 3).copy()
    I = np.frombuffer(buf, np.uint32, idx(ic), io).copy()
    if lay.get("normals"):
        no, nc = lay["normals"]
        N = np.frombuffer(buf, np.float32, vec(nc) * 3, no).reshape(-1, 3).copy()
    else:
        N = compute_normals(P, I)
    UV = None
    if lay.get("uvs"):
        uo, uc = lay["uvs"]
        UV = np.frombuffer(buf, np.float32, (nv if (uc == nv * 2 and nv * 2 != nv) else uc) * 2, uo).reshape(-1, 2).copy()
    return {"P": P, "N": N, "I": I, "UV": UV}


def load_scene_dir(path: str):
    """gpu/scene_gpu.js:52 loadScene: scene.json and every mesh it lists."""
    with open(os.path.join(path, "scene.json")) as f:
        scene = json.load(f)
    meshes = {}
    for m in scene["meshes"]:
        with open(os.path.join(path, m["file"]), "rb") as f:
            meshes[m["name"]] = decode_mesh(m, f.read())
    return scene, meshes


# ------------------------------------------------------------------------------------------- the scene dict
def _body_of_part(scene: dict) -> dict:
    """gpu/scene_gpu.js:218 bodyOfPart: mesh name -> the posed body it belongs to."""
    out = {}
    for inst in scene.get("instruments") or []:
        for part in inst.get("parts") or []:
            out[part["mesh"]] = {"key": f"{inst['id']}/{part['body']}", "kind": "instrument"}
    sc = scene.get("scope") or {}
    for m in sc.get("mesh_parts") or []:
        out[m] = {"key": "scope", "kind": "scope"}
    if sc.get("emitter_mesh"):
        out[sc["emitter_mesh"]] = {"key": "scope", "kind": "scope", "emitter": True}
    for b in scene.get("boards") or []:
        out[b["mesh"]] = {"key": f"board/{b['name']}", "kind": "board"}
    cams = [c["name"] for c in scene.get("cameras") or []]
    for m in scene.get("meshes") or []:
        if m.get("owner_camera") and m["name"] not in out:
            out[m["name"]] = {"key": f"fixed/{m['name']}", "kind": "fixed", "owner": m["owner_camera"]}
    ports = {p["id"] for p in scene.get("ports") or []}
    for m in scene.get("meshes") or []:
        if m["name"] in out or not m.get("dynamic") or not m.get("body"):
            continue
        head = m["body"].split("/")[0]
        out[m["name"]] = {"key": m["body"], "kind": "scope" if m["body"] == "scope" else "board" if head == "board" else "fixture"}
    for v in out.values():
        if "owner" in v:
            v["owner_camera"] = cams.index(v["owner"]) if v["owner"] in cams else -1
    return out


def _material(name: str, physics: dict | None) -> dict:
    """gpu/scene_gpu.js:170 materialsFromPhysics for one name (a missing one is a neutral grey)."""
    m = ((physics or {}).get("materials") or {}).get(name) or {}
    model = _unwrap(m.get("model"))
    textured = m.get("rho_d_paper") is not None and m.get("rho_d_ink") is not None
    fa = _unwrap(m.get("fresnel_avg"))
    if model == "coated_conductor":
        tau = _unwrap(m.get("coat_transmittance"))
        tau = [1.0, 1.0, 1.0] if tau is None else ([float(tau)] * 3 if np.isscalar(tau) else [float(x) for x in tau])
        if len(tau) == 1:
            tau = tau * 3
        out = {"metallic": 2, "coated": 1, "f0": [float(x) for x in (_unwrap(m.get("f0")) or [0.56, 0.57, 0.58])],
               "roughness": float(_unwrap(m.get("roughness")) if m.get("roughness") is not None else 0.3),
               "coat_ior": float(_unwrap(m.get("coat_ior")) or 1.5), "coat_roughness": float(_unwrap(m.get("coat_roughness")) or 0.05),
               "tau": tau}
    else:
        metallic = int(_unwrap(m.get("metallic")) if m.get("metallic") is not None else (1 if model == "conductor" else 0))
        rough = _unwrap(m.get("roughness_paper") if textured else m.get("roughness"))
        rho = _unwrap(m.get("rho_d_paper") if textured else m.get("rho_d"))
        out = {"metallic": metallic, "roughness": float(0.5 if rough is None else rough), "ior": float(_unwrap(m.get("ior")) or 1.5),
               "rho": [float(x) for x in (rho or [0.5, 0.5, 0.5])], "f0": [float(x) for x in (_unwrap(m.get("f0")) or [0.56, 0.57, 0.58])],
               "fbar": float("nan") if fa is None else float(fa)}
    if textured:
        out.update({"textured": 1, "ink_rho": [float(x) for x in _unwrap(m["rho_d_ink"])],
                    "ink_roughness": float(_unwrap(m.get("roughness_ink")) or 0.4)})
    ll = m.get("layer_lines") or {}
    out["layer"] = (float(_unwrap(ll.get("height_m")) or 0.0), float(_unwrap(ll.get("depth_m")) or 0.0)) if _unwrap(ll.get("height_m")) else None
    out["emitter"] = 1 if model == "emitter" else 0
    out["name"] = name
    return out


def _emitter(physics: dict | None) -> dict:
    """gpu/scene_gpu.js:205 emitterFromPhysics."""
    ph = physics or {}
    em = (ph.get("materials") or {}).get("emitter") or {}
    L0 = _unwrap(em.get("L0")) or [1.0, 1.0, 1.0]
    prof = _unwrap(em.get("profile"))
    if isinstance(prof, str):
        node = ph
        for k in prof.split("."):
            node = (node or {}).get(k) if isinstance(node, dict) else None
        prof = node
    prof = prof or (ph.get("light") or {}).get("profile") or {}
    th = _unwrap(prof.get("theta_deg")) or [0.0, 90.0]
    p = _unwrap(prof.get("p")) or [1.0, 1.0]
    ax = _unwrap((((ph.get("scope") or {}).get("emission_axis")) or {}).get("angle_from_shaft_deg"))
    return {"L0": [float(x) for x in L0], "theta": [math.radians(float(t)) for t in th], "p": [float(x) for x in p],
            "axis_deg": float("nan") if ax is None else float(ax)}


def prepare_scene(scene: dict, meshes: dict, physics: dict | None = None, node_spacing: float = 0.003, device: int | None = None) -> dict:
    """gpu/scene_gpu.js:241 prepareScene up to the packing: the scene dict of vtwin.dome's form. device: a CUDA ordinal
    to weld and subdivide on (the same scene), None for the host."""
    bodies = _body_of_part(scene)
    metas = list(scene["meshes"])
    bench_mat = (scene.get("bench") or {}).get("material") or "bench_white"
    mat_names, mat_index = [], {}
    for n in [m["material"] for m in metas] + [bench_mat]:
        if n not in mat_index:
            mat_index[n] = len(mat_names)
            mat_names.append(n)
    materials = [_material(n, physics) for n in mat_names]
    table = []

    def add_mesh(name, material, flags, build_dir=None, overview_only=False):
        mat = materials[mat_index[material]]
        lay = mat.get("layer")
        table.append({"name": name, "mat": mat_index[material], "flags": int(flags), "build_dir": list(build_dir or [0.0, 0.0, 1.0]),
                      "layer": list(lay) if lay else [0.0, 0.0], "overview_only": bool(overview_only)})
        return len(table) - 1

    sP, sN, sI, sTM, sVM = [], [], [], [], []
    nv = 0
    fine = [[math.inf, math.inf], [-math.inf, -math.inf]]
    for m in metas:
        if m.get("dynamic") or m["name"] in bodies:
            continue
        d = meshes.get(m["name"])
        if d is None:
            raise VtError(A.VT_ERR_ARG, f"mesh {m['name']} not loaded")
        mat = materials[mat_index[m["material"]]]
        lay = mat.get("layer")
        flags = MESH_FLAG["STATIC"] | (MESH_FLAG["LAYER"] if m.get("build_dir") and lay and lay[1] > 0 else 0)
        mid = add_mesh(m["name"], m["material"], flags, m.get("build_dir"))
        P, N, I = weld(d["P"], d["N"], d["I"], device=device)
        P, N, I = subdivide(P, N, I, node_spacing, device=device)
        sP.append(P); sN.append(N); sI.append(I.reshape(-1, 3) + nv)
        sTM.append(np.full(len(I) // 3, mid, np.uint32)); sVM.append(np.full(len(P), mid, np.uint32))
        nv += len(P)
        if len(P):
            fine[0][0] = min(fine[0][0], float(P[:, 0].min())); fine[0][1] = min(fine[0][1], float(P[:, 1].min()))
            fine[1][0] = max(fine[1][0], float(P[:, 0].max())); fine[1][1] = max(fine[1][1], float(P[:, 1].max()))
    if scene.get("bench"):
        b = scene["bench"]
        ext = b.get("extent") or [[-0.5, -0.5], [0.5, 0.5]]
        if not math.isfinite(fine[0][0]):
            fine = ext
        mg = 0.006
        fb = [[fine[0][0] - mg, fine[0][1] - mg], [fine[1][0] + mg, fine[1][1] + mg]]
        P, N, I = bench_mesh(b.get("z", 0.0), ext, fb, node_spacing)
        mid = add_mesh("bench", bench_mat, MESH_FLAG["STATIC"] | MESH_FLAG["BENCH"])
        sP.append(P); sN.append(N); sI.append(I.reshape(-1, 3) + nv)
        sTM.append(np.full(len(I) // 3, mid, np.uint32)); sVM.append(np.full(len(P), mid, np.uint32))
        nv += len(P)
    static = {"P": np.concatenate(sP).astype(np.float32), "N": np.concatenate(sN).astype(np.float32),
              "I": np.concatenate(sI).astype(np.uint32), "tri_mesh": np.concatenate(sTM), "vert_mesh": np.concatenate(sVM)}
    # posed bodies in order of first mesh, each a BLAS of its meshes in the body frame
    order, by_key = [], {}
    for m in metas:
        b = bodies.get(m["name"])
        if not b:
            continue
        if b["key"] not in by_key:
            by_key[b["key"]] = {"key": b["key"], "kind": b["kind"], "owner_camera": b.get("owner_camera", -1), "meshes": []}
            order.append(b["key"])
        by_key[b["key"]]["meshes"].append(m)
    out_bodies = []
    for key in order:
        body = by_key[key]
        P, N, I, TM, UV = [], [], [], [], []
        off = 0
        for m in body["meshes"]:
            d = meshes.get(m["name"])
            if d is None:
                raise VtError(A.VT_ERR_ARG, f"mesh {m['name']} not loaded")
            is_em = bool(bodies[m["name"]].get("emitter"))
            mat = "emitter" if is_em else m["material"]
            if is_em and mat not in mat_index:
                mat_index[mat] = len(materials)
                materials.append({"name": "emitter", "metallic": 0, "rho": [0.02, 0.02, 0.02], "roughness": 0.05, "ior": 1.5,
                                  "emitter": 1, "no_table": 1})
            texd = not is_em and materials[mat_index[m["material"]]].get("textured") and d.get("UV") is not None
            flags = ((MESH_FLAG["EMITTER"] if is_em else 0) | (MESH_FLAG["BOARD"] if body["kind"] == "board" else 0) |
                     (MESH_FLAG["TEXTURED"] if texd else 0) | (MESH_FLAG["INSTRUMENT"] if body["kind"] == "instrument" else 0) |
                     (MESH_FLAG["SCOPE"] if body["kind"] == "scope" else 0))
            mid = add_mesh(m["name"], mat, flags, m.get("build_dir"), m.get("overview_only", False))
            P.append(d["P"]); N.append(d["N"]); I.append(d["I"].reshape(-1, 3) + off)
            UV.append(d["UV"] if d.get("UV") is not None else np.zeros((len(d["P"]), 2), np.float32))
            TM.append(np.full(len(d["I"]) // 3, mid, np.uint32))
            off += len(d["P"])
        out_bodies.append({"key": key, "kind": body["kind"], "owner_camera": body["owner_camera"],
                           "P": np.concatenate(P).astype(np.float32), "N": np.concatenate(N).astype(np.float32),
                           "I": np.concatenate(I).astype(np.uint32), "tri_mesh": np.concatenate(TM), "UV": np.concatenate(UV).astype(np.float32)})
    cams = []
    for c in scene.get("cameras") or []:
        K, D = c["lens"]["K"], c["lens"].get("D") or [0.0, 0.0, 0.0, 0.0]
        size = c.get("size") or c["lens"]["size"]
        cams.append({"name": c["name"], "size": [int(size[0]), int(size[1])], "fx": float(K[0][0]), "fy": float(K[1][1]),
                     "cx": float(K[0][2]), "cy": float(K[1][2]), "alpha": float(K[0][1]) / float(K[0][0]), "k": [float(x) for x in D],
                     "T_D_C": np.asarray(c["T_D_C"], np.float64), "theta_fold": float(c.get("theta_fold_rad", 1.5))})
    for m in materials:
        m.pop("layer", None)
    return {"static": static, "bodies": out_bodies, "meshes": table, "materials": materials, "emitter": _emitter(physics),
            "cameras": cams, "scope": scene.get("scope")}


def load_scene(path: str, physics: dict | None = None, node_spacing: float = 0.003, device: int | None = None) -> dict:
    """A scene directory to the scene dict: load_scene_dir + prepare_scene."""
    scene, meshes = load_scene_dir(path)
    return prepare_scene(scene, meshes, physics, node_spacing, device=device)
