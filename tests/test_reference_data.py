"""The oracle and the scene path pinned against data the reference holds (CPU only).

- configs/twin/physics.yaml's derived values (tests/golden/physics_kat.json, read as text by make_golden.py):
  rho_d = albedo / (1 - F(0)) for the materials that state it, with F(0) the oracle's unpolarised Fresnel of their
  ior; the emitter radiance chain Y0 = flux / (683 A_face int p cos dw), L0 = Y0 x chromaticity, with the oracle's
  integral of the tabulated profile; and, on the twin's own scene, the emitter area the scene preparation packs from
  the outlet mesh against area_on_face.
- assets/preview_stats.json: per camera, the share of pixels by surface class, which the reference made with "a CPU
  painter's z-buffer of Lens.project-ed triangles at 1/4 resolution; dynamic parts at scene default_state
  (instruments, scope, cannulas; housings left out)". The same method is restated here: the twin's raw CAD
  triangles (scene.json meshes, decoded by the scene loader; the bench as the scene preparation grids it), posed at
  default_state by the kinematics restatement (tests/twin_kinematics.py), projected through the oracle's KB4 project
  (gpu/lens.js:43), rasterised by the oracle's watertight rasteriser at 320 x 180 with one depth per triangle (the
  largest of its vertices', a painter's order). The reference records neither the depth rule nor how it treats
  triangles past the fold, and its 31 cm shaft triangles, drawn with straight edges, are exactly where those rules
  matter, so the tolerance is the spread of those variants: 1.5 points for the two large classes, 0.6 for the rest.
- the renderer's first hits against the same z-buffer on geometry fine enough that straight edges are exact: the
  oracle's ray-cast classes of the 1/4-resolution pixel centres against a z-buffer of the scene with every mesh
  subdivided to 5 mm; they differ only on class-boundary pixels.

The twin's scene files are the reference's ($VT_REFERENCE, or ../reference beside this repository); without them
those tests skip.
"""
import json
import math
import os

import numpy as np
import pytest

import oracle as O
from conftest import reference_path

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "physics_kat.json")))
HAVE_TWIN = os.path.isfile(reference_path("assets", "scene.json")) and os.path.isfile(reference_path("assets", "preview_stats.json"))
CLASSES = ["interior", "bench", "within_5mm", "other_lens", "port_hardware", "cannulas", "instruments", "scope", "miss"]
# scene.json mesh groups -> the preview statistics' classes
GROUP_CLASS = {"shell": "interior", "hatch": "interior", "lid": "interior", "membrane": "port_hardware", "lens_front": "other_lens",
               "instrument_part": "instruments", "scope": "scope", "board": "board", "trocar": "cannulas"}


def test_rho_d_from_albedo_matches_reference_config():
    """rho_d = albedo / (1 - F0), F0 the normal-incidence Fresnel of the material's ior (physics.yaml: pla_matte_white,
    bench_white, petg_cap): the oracle's Fresnel gives the stated F0 to its 3-4 digits and rho_d to its 3 decimals."""
    assert len(GOLD["rho_d_from_albedo"]) == 3
    for m in GOLD["rho_d_from_albedo"]:
        F0 = O.fresnel_dielectric(1.0, m["ior"])
        assert F0 == pytest.approx(m["F0"], abs=5e-4), m["name"]
        rho = np.array(m["albedo"]) / (1.0 - F0)
        assert np.all(np.abs(rho - np.array(m["rho_d"])) <= 5e-4 + 1e-12), (m["name"], rho)


def test_emitter_radiance_chain_matches_reference_config():
    """L0 = Y0 x chromaticity with Y0 = flux / (683 A_face int p cos dw): with the oracle's integral of the tabulated
    profile, physics.yaml's L0 to its 5 digits."""
    pr, li = GOLD["profile"], GOLD["light"]
    th, pp = np.radians(pr["theta_deg"]), np.array(pr["p"], float)
    x = np.linspace(0.0, math.pi / 2, 8001)
    psa = 2 * math.pi * np.trapezoid(np.array([O.profile(t, th, pp) for t in x]) * np.cos(x) * np.sin(x), x)
    Y0 = li["flux_lm"] / (683.0 * li["area_on_face"] * psa)
    L0 = Y0 * np.array(li["srgb_chromaticity"])
    assert np.all(np.abs(L0 - np.array(li["L0"])) <= 1e-4 * np.array(li["L0"])), L0
    # the face area is the cross-section over cos 30 deg (the tip face's tilt)
    assert li["area_cross_section"] / math.cos(math.radians(30.0)) == pytest.approx(li["area_on_face"], rel=2e-4)


def _twin():
    from vtwin import scene_io

    physics = json.load(open(reference_path("configs", "twin", "physics.json")))
    sj, meshes = scene_io.load_scene_dir(reference_path("assets"))
    sc = scene_io.prepare_scene(sj, meshes, physics)
    return sj, meshes, sc


@pytest.fixture(scope="module")
def twin():
    if not HAVE_TWIN:
        pytest.skip("the twin's scene files are not here")
    return _twin()


def test_twin_emitter_area_matches_area_on_face(twin):
    """The scene preparation packs the outlet mesh (scope_light) as the emitter: its area against physics.yaml's
    area_on_face (4.7930e-5 m^2, 'Monte-Carlo check 4.790e-5')."""
    sj, meshes, sc = twin
    area = O.Scene(sc).emitter()["area"]
    print(f"\nemitter area {area:.5e} m^2, area_on_face {GOLD['light']['area_on_face']:.5e}")
    assert area == pytest.approx(GOLD["light"]["area_on_face"], rel=1.5e-3)


def _posed_triangles(sj, meshes, sc, cam_name, h=None):
    """World triangles of the twin's raw meshes at default_state (housings and the camera's own lens front left out,
    unposed boards hidden) and of the prepared bench; their classes. h: subdivide every mesh to edges <= h."""
    import twin_kinematics as TK
    from vtwin import scene_io

    poses = TK.poses_from_state(sj, sj["default_state"])
    bodies = scene_io._body_of_part(sj)
    Ps, Is, cls = [], [], []
    off = 0
    for m in sj["meshes"]:
        if m.get("overview_only") or m.get("owner_camera") == cam_name:
            continue
        d = meshes[m["name"]]
        P, I = d["P"].astype(np.float64), d["I"].reshape(-1, 3)
        b = bodies.get(m["name"])
        if b is not None and b["kind"] != "fixed":
            if b["key"] not in poses:
                continue
            T = np.asarray(poses[b["key"]]).reshape(4, 4).T
            P = P @ T[:3, :3].T + T[:3, 3]
        if h is not None:
            P, _, I = scene_io.subdivide(P, np.zeros_like(P), I.ravel(), h)
            I = I.reshape(-1, 3)
        Ps.append(P)
        Is.append(I + off)
        cls += [GROUP_CLASS[m["group"]]] * len(I)
        off += len(P)
    st = sc["static"]
    bench = [i for i, t in enumerate(sc["meshes"]) if t["name"] == "bench"][0]
    Ps.append(st["P"].astype(np.float64))
    Is.append(st["I"][st["tri_mesh"] == bench] + off)
    cls += ["bench"] * int(np.sum(st["tri_mesh"] == bench))
    return np.concatenate(Ps), np.concatenate(Is), np.array(cls)


def _zbuffer_classes(cam, P, I, cls, depth="max"):
    """Class of each of the 4 samples of every pixel of a 1/4-resolution z-buffer of the triangles, KB4-projected by
    the oracle (full-resolution lens, quarter pixel i at full-resolution 4 i + 1.5); one depth per triangle (the
    largest of its vertices' distances) or per vertex (interpolated in the image); a triangle with a vertex past the
    lens's fold (or behind the lens) is not drawn."""
    T = np.asarray(cam["T_D_C"], np.float64)
    X = (P - T[:3, 3]) @ T[:3, :3]
    uv = O.project([cam["fx"], cam["fy"], cam["cx"], cam["cy"], cam["alpha"], *cam["k"]], X)
    th = np.arctan2(np.hypot(X[:, 0], X[:, 1]), X[:, 2])
    dist = np.linalg.norm(X, axis=1)
    w, h = cam["size"][0] // 4, cam["size"][1] // 4
    uq, vq = (uv[:, 0] - 1.5) / 4, (uv[:, 1] - 1.5) / 4
    V = I.ravel()
    clip = np.zeros((len(V), 4), np.float32)
    clip[:, 0] = 2 * (uq[V] + 0.5) / w - 1
    clip[:, 1] = 1 - 2 * (vq[V] + 0.5) / h
    clip[:, 2] = (np.repeat(dist[I].max(axis=1), 3) if depth == "max" else dist[V]) / 10.0
    clip[:, 3] = 1.0
    past = np.repeat((th[I] > min(cam["theta_fold"], math.pi / 2)).any(axis=1), 3)
    clip[past] = [0.0, 0.0, -1e-3, -1e-3]
    keys = O.raster(clip, np.arange(len(V), dtype=np.uint32).reshape(-1, 3), w, h, samples=4)
    tri = (keys & np.uint64(0xFFFFFFFF)).astype(np.int64)
    return np.where(tri == 0xFFFFFFFF, "miss", cls[np.minimum(tri, len(cls) - 1)])


@pytest.mark.skipif(not HAVE_TWIN, reason="the twin's scene files are not here")
def test_preview_statistics_match_reference(twin):
    """The reference's per-camera class shares (assets/preview_stats.json) from its own method restated: a 1/4-
    resolution z-buffer of the raw CAD triangles at default_state."""
    sj, meshes, sc = twin
    ref = json.load(open(reference_path("assets", "preview_stats.json")))
    for cam in sc["cameras"]:
        P, I, cls = _posed_triangles(sj, meshes, sc, cam["name"])
        lab = _zbuffer_classes(cam, P, I, cls)
        r = ref[cam["name"]]
        assert r["pixels"] == lab.shape[0] * lab.shape[1]
        line = []
        for k in CLASSES:
            ours, want = 100.0 * np.mean(lab == k), r[k + "_pct"]
            line.append(f"{k} {ours:.3f}/{want:.3f}")
            tol = 1.5 if want > 10.0 else 0.6
            assert abs(ours - want) <= tol, (cam["name"], k, ours, want)
        print(f"\n{cam['name']}: " + "  ".join(line), end="")


@pytest.mark.skipif(not HAVE_TWIN, reason="the twin's scene files are not here")
def test_ray_cast_first_hits_match_fine_zbuffer(twin):
    """The renderer's first hits (the oracle's traversal of the prepared scene: its BVH, the posed instances, the
    camera's own lens skipped) classify the 1/4-resolution pixel centres as a z-buffer of the same surfaces
    subdivided to 5 mm does, but for pixels on class boundaries (where one point sample and four raster samples may
    fall on different sides); on the reference's long CAD triangles the two differ (the shafts), which is why the
    reference's shares are checked with its own method above."""
    import twin_kinematics as TK

    sj, meshes, sc = twin
    S = O.Scene(sc)
    poses = TK.poses_from_state(sj, sj["default_state"])
    T0 = np.full((len(sc["bodies"]), 16), np.nan)
    for i, b in enumerate(sc["bodies"]):
        if b["key"] in poses:
            T0[i] = poses[b["key"]]
        elif b["kind"] == "fixed":
            T0[i] = np.eye(4).ravel()
    S.set_poses(T0)
    cam = sc["cameras"][2]            # the camera that sees every class but within_5mm
    w, h = cam["size"][0] // 4, cam["size"][1] // 4
    ray_cls, _ = ray_cast_classes(lambda o4, d4: S.trace(o4, d4, mask=3, fp64=True)[0], S.arrays()["tris"], sj, sc, cam, w, h)
    P, I, cls = _posed_triangles(sj, meshes, sc, cam["name"], h=0.005)
    zb = _zbuffer_classes(cam, P, I, cls, depth="vertex")
    names = np.array(CLASSES + ["board"])
    idx = np.searchsorted(np.sort(names), zb)            # class index of each sample
    order = np.argsort(names)
    counts = np.stack([(order[idx] == c).sum(axis=2) for c in range(len(names))], axis=2)
    zb_major = names[counts.argmax(axis=2)]              # the majority of a pixel's 4 samples
    bd = np.zeros((h, w), bool)                          # a 4-neighbour of another class
    dx, dy = ray_cls[:, 1:] != ray_cls[:, :-1], ray_cls[1:, :] != ray_cls[:-1, :]
    bd[:, 1:] |= dx
    bd[:, :-1] |= dx
    bd[1:, :] |= dy
    bd[:-1, :] |= dy
    off = (ray_cls != zb_major) & ~bd
    shares = "  ".join(f"{k} {100 * np.mean(ray_cls == k):.3f}/{100 * np.mean(zb_major == k):.3f}" for k in CLASSES)
    print(f"\n{cam['name']} ray cast / fine z-buffer: {shares}; pixels off a boundary that differ: {off.sum()}")
    assert off.sum() <= 0.001 * w * h


def ray_cast_classes(trace, tris, sj, sc, cam, w, h):
    """Class and hit triangle of each 1/4-resolution pixel centre by closest hits (trace(o4, d4) -> rows (t, triangle
    or -1, ...); tris: the packed triangle records), the camera's own lens front and the housings passed through as
    the reference's renderer and statistics skip them."""
    meta = {m["name"]: m for m in sj["meshes"]}
    names = [m["name"] for m in sc["meshes"]]
    tri_mesh = np.asarray(tris).reshape(-1, 16)[:, 12]
    ys, xs = np.mgrid[0:h, 0:w]
    uv = np.stack([4 * xs.ravel() + 1.5, 4 * ys.ravel() + 1.5], 1).astype(np.float64)
    dc = O.unproject([cam["fx"], cam["fy"], cam["cx"], cam["cy"], cam["alpha"], *cam["k"]], uv)
    T = np.asarray(cam["T_D_C"], np.float64)
    d = dc @ T[:3, :3].T
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    n = len(d)
    o = np.tile(T[:3, 3], (n, 1))
    dist = np.zeros(n)
    out_cls = np.full(n, "miss", object)
    out_tri = np.full(n, -1, np.int64)
    todo = np.arange(n)
    for _ in range(6):
        o4 = np.zeros((len(todo), 4), np.float32)
        d4 = np.zeros((len(todo), 4), np.float32)
        o4[:, :3], d4[:, :3] = o[todo], d[todo]
        hit = trace(o4, d4)
        again = []
        for k, i in enumerate(todo):
            t, tri = hit[k, 0], int(hit[k, 1])
            if tri < 0:
                continue
            out_tri[i] = tri
            name = names[tri_mesh[tri]]
            if name == f"lens_front_{cam['name']}" or meta.get(name, {}).get("overview_only"):
                o[i] = o[i] + d[i] * (t + 1e-6)
                dist[i] += t + 1e-6
                again.append(i)
                continue
            dist[i] += t
            out_cls[i] = "within_5mm" if dist[i] < 0.005 else ("bench" if name == "bench" else GROUP_CLASS[meta[name]["group"]])
        todo = np.array(again, int)
        if not len(todo):
            break
    return out_cls.reshape(h, w).astype(str), out_tri.reshape(h, w)
