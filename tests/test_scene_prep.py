"""Scene preparation on the host (gpu/scene_gpu.js:37-165 and the front half of prepareScene :241): vt_weld,
vt_subdivide, vt_bench_mesh and vt_compute_normals against their plain-Python restatement (same vertices, normals
and triangles in the same order, bit for bit), the subdivision's invariants (edges <= h, area and closedness kept,
no cracks), and the scene loader on a scene directory written here. No device needed."""
import json
import math
import os

import numpy as np
import pytest

import oracle as O
from conftest import reference_path
from vtwin import dome
from vtwin import scene_io as S


def _sphere(level=2, r=0.05, seed=0, noise=2e-9):
    V, F = dome.icosphere(level)
    rng = np.random.default_rng(seed)
    P = (V * r).astype(np.float32)
    N = V.astype(np.float32)
    # unwelded copy: every triangle with its own vertices (positions and normals repeated), plus float noise below the
    # weld tolerance on half of the copies
    P3 = P[F.ravel()].copy()
    N3 = N[F.ravel()].copy()
    P3[::2] += rng.uniform(-noise, noise, P3[::2].shape).astype(np.float32)
    return P3, N3, np.arange(len(P3), dtype=np.uint32)


def test_weld_matches_restatement_and_welds():
    P, N, I = _sphere()
    a = S.weld(P, N, I)
    b = O.weld_ref(P, N, I)
    for x, y in zip(a, b):
        assert x.shape == y.shape and np.array_equal(x, y)
    # without the noise (keys can straddle a rounding boundary) the copies weld back to the icosphere
    V, F = dome.icosphere(2)
    c = S.weld(*_sphere(noise=0.0))
    assert len(c[0]) == len(V) and len(c[2]) == 3 * len(F)
    # degenerate triangles (two corners that weld together) are dropped
    P2 = np.concatenate([P, P[:3]]); P2[-1] = P2[-2]
    N2 = np.concatenate([N, N[:3]]); N2[-1] = N2[-2]
    I2 = np.arange(len(P2), dtype=np.uint32)
    assert len(S.weld(P2, N2, I2)[2]) == len(a[2])


def test_subdivide_matches_restatement_and_keeps_the_surface():
    P, N, I = S.weld(*_sphere(level=1, noise=0.0))
    h = 0.012
    a = S.subdivide(P, N, I, h)
    b = O.subdivide_ref(P, N, I, h)
    for x, y in zip(a, b):
        assert x.shape == y.shape and np.array_equal(x, y)
    Pa, Na, Ia = a
    T = Ia.reshape(-1, 3)
    e = np.concatenate([np.linalg.norm(Pa[T[:, i]] - Pa[T[:, (i + 1) % 3]], axis=1) for i in range(3)])
    assert e.max() <= h
    area = lambda Q, Tt: 0.5 * np.linalg.norm(np.cross(Q[Tt[:, 1]] - Q[Tt[:, 0]], Q[Tt[:, 2]] - Q[Tt[:, 0]]), axis=1).sum()
    assert abs(area(Pa, T) - area(P, I.reshape(-1, 3))) < 1e-12
    # conforming: every edge of the closed sphere is shared by exactly two triangles
    edges = {}
    for t in T:
        for i in range(3):
            k = (min(t[i], t[(i + 1) % 3]), max(t[i], t[(i + 1) % 3]))
            edges[k] = edges.get(k, 0) + 1
    assert set(edges.values()) == {2}
    assert np.allclose(np.linalg.norm(Na, axis=1), 1.0, atol=1e-12)


def test_bench_mesh_and_normals_match_restatement():
    ext, fine = ((-0.3, -0.2), (0.25, 0.28)), ((-0.05, -0.04), (0.06, 0.05))
    a = S.bench_mesh(0.004, ext, fine, 0.003)
    b = O.bench_mesh_ref(0.004, ext, fine, 0.003)
    for x, y in zip(a, b):
        assert x.shape == y.shape and np.array_equal(x, y)
    P, _, I = _sphere(level=2)
    P, I = P[: 3 * 60], I[: 3 * 60]
    assert np.array_equal(S.compute_normals(P, I), O.compute_normals_ref(P, I))


def test_scene_directory_loader(tmp_path):
    """A scene directory in the reference's format (scene.json, meshes/*.bin with [byteOffset, count] layouts; a
    static mesh, a bench, a scope body with its emitter mesh, an instrument, a camera's lens front) through
    load_scene: welded and subdivided static nodes, the bench, bodies and flags, cameras."""
    os.makedirs(tmp_path / "meshes")
    metas = []

    def write(name, P, N, I, **kw):
        P, N, I = np.asarray(P, np.float32), np.asarray(N, np.float32), np.asarray(I, np.uint32)
        buf = P.tobytes() + N.tobytes() + I.tobytes()
        (tmp_path / "meshes" / f"{name}.bin").write_bytes(buf)
        metas.append({"name": name, "file": f"meshes/{name}.bin", "vertex_count": len(P), "triangle_count": len(I) // 3,
                      "layout": {"positions": [0, len(P)], "normals": [P.nbytes, len(N)], "indices": [P.nbytes + N.nbytes, len(I) // 3]}, **kw})

    Ps, Ns, Is = _sphere(level=1, r=0.2)
    write("shell", Ps, Ns, Is, material="pla_matte_white", dynamic=False)
    Pc, Nc, Ic = dome.capsule_geometry(radius=0.003, length=0.1)
    write("scope_shaft", Pc, Nc, Ic.ravel(), material="scope_steel", dynamic=True, body="scope")
    Pd, Nd, Id = dome.disk_geometry(0.002)
    write("scope_light", Pd, Nd, Id.ravel(), material="emitter", dynamic=True, body="scope")
    write("L_shaft", Pc, Nc, Ic.ravel(), material="insulation_black", dynamic=True, body="L/shaft")
    write("lens_front_CAM1", Pd, Nd, Id.ravel(), material="lens_glass_black", dynamic=False, owner_camera="CAM1")
    cam = {"name": "CAM1", "size": [64, 48], "lens": {"model": "kb4", "K": [[50.0, 0.0, 31.5], [0.0, 50.0, 23.5], [0.0, 0.0, 1.0]],
                                                     "D": [0.01, 0.0, 0.0, 0.0], "size": [64, 48]},
           "T_D_C": np.eye(4).tolist(), "theta_fold_rad": 1.2}
    scene = {"meshes": metas, "bench": {"z": 0.0, "material": "bench_white", "extent": [[-0.3, -0.3], [0.3, 0.3]]},
             "cameras": [cam], "scope": {"mesh_parts": ["scope_shaft"], "emitter_mesh": "scope_light"},
             "instruments": [{"id": "L", "parts": [{"mesh": "L_shaft", "body": "shaft"}]}]}
    (tmp_path / "scene.json").write_text(json.dumps(scene))
    physics = {"materials": {"pla_matte_white": {"model": "dielectric", "rho_d": [0.8, 0.8, 0.78], "roughness": 0.6, "ior": 1.5},
                             "emitter": {"model": "emitter", "L0": [100.0, 95.0, 90.0], "profile": {"theta_deg": [0, 30, 60], "p": [1, 0.5, 0]}}}}
    sc = S.load_scene(str(tmp_path), physics, node_spacing=0.02)
    names = [m["name"] for m in sc["meshes"]]
    assert names == ["shell", "bench", "scope_shaft", "scope_light", "L_shaft", "lens_front_CAM1"]
    assert [b["key"] for b in sc["bodies"]] == ["scope", "L/shaft", "fixed/lens_front_CAM1"]
    assert [b["kind"] for b in sc["bodies"]] == ["scope", "instrument", "fixed"] and sc["bodies"][2]["owner_camera"] == 0
    fl = {m["name"]: m["flags"] for m in sc["meshes"]}
    assert fl["shell"] == 1 and fl["bench"] == 1 | 64 and fl["scope_light"] == 2 | 32 and fl["L_shaft"] == 16
    st = sc["static"]
    T = st["I"].reshape(-1, 3)[st["tri_mesh"] == 0]        # the shell (the bench's outer quads are coarse by design)
    e = np.concatenate([np.linalg.norm(st["P"][T[:, i]].astype(np.float64) - st["P"][T[:, (i + 1) % 3]], axis=1) for i in range(3)])
    assert e.max() <= 0.02 * (1 + 1e-6)
    assert sc["emitter"]["L0"] == [100.0, 95.0, 90.0] and math.isclose(sc["emitter"]["theta"][1], math.radians(30))
    assert sc["cameras"][0]["fx"] == 50.0 and sc["cameras"][0]["theta_fold"] == 1.2
    # the packed scene (the oracle's prepareScene restatement) accepts it
    Osc = O.Scene(sc)
    assert Osc.static_verts == len(st["P"]) and Osc.n_bodies == 3


@pytest.mark.skipif(not os.path.isdir(reference_path("assets", "meshes")), reason="no twin scene files here")
def test_real_mesh_weld_and_subdivide_match_restatement():
    """One of the twin's own meshes (the smallest static one) through weld + subdivide, native against the
    restatement."""
    scene = json.load(open(reference_path("assets", "scene.json")))
    m = min((x for x in scene["meshes"] if not x.get("dynamic")), key=lambda x: x["triangle_count"])
    d = S.decode_mesh(m, open(reference_path("assets", m["file"]), "rb").read())
    a = S.weld(d["P"], d["N"], d["I"])
    b = O.weld_ref(d["P"], d["N"], d["I"])
    assert all(np.array_equal(x, y) for x, y in zip(a, b))
    sa, sb = S.subdivide(*a, 0.003), O.subdivide_ref(*a, 0.003)
    assert all(np.array_equal(x, y) for x, y in zip(sa, sb))
