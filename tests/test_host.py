"""Host logic of the product on CPU: the C-ABI library loads and exports every symbol include/vtwin.h declares,
its host BVH builder reproduces gpu/bvh.js's node array word for word (checked against the oracle), the sensor
uniform packing follows gpu/sensor.js:158, and without a GPU the library fails loudly (no CPU fallback)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import oracle as O
from conftest import ROOT, has_gpu
from vtwin import _abi as A
from vtwin import _lib, dome
from vtwin import sensor as S
from vtwin.renderer import build_bvh


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "vtwin.h")).read()
    # function declarations: a return type at the start of a line, then the vt_ name and its parameter list
    return sorted(set(re.findall(r"^(?:vt_status|uint32_t|const char\*|void\*|void)\s+(vt_[a-z0-9_]+)\s*\(", text, re.M)))


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    syms = declared_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(lib, s), s
    assert set(syms) == set(_lib.SIGNATURES)


@pytest.mark.parametrize("leaf", [1, 2, 4, 8])
def test_bvh_builder_matches_oracle_on_dome(dome_small, leaf):
    st = dome_small["static"]
    a = build_bvh(st["P"], st["I"], leaf)
    b = O.bvh_build(st["P"], st["I"], leaf)
    assert a["nodeCount"] == b["node_count"] and a["maxDepth"] == b["max_depth"]
    assert np.array_equal(a["nodes"], b["nodes"]) and np.array_equal(a["order"], b["order"])


def test_bvh_builder_matches_oracle_on_random_and_degenerate_meshes():
    rng = np.random.default_rng(11)
    for n in [0, 1, 2, 3, 5, 17, 100, 1000]:
        P = rng.normal(size=(3 * max(n, 1), 3)).astype(np.float32)
        I = np.arange(3 * n, dtype=np.uint32).reshape(-1, 3)
        a, b = build_bvh(P, I), O.bvh_build(P, I)
        assert np.array_equal(a["nodes"], b["nodes"]) and np.array_equal(a["order"], b["order"]), n
    # coincident centroids, axis-aligned slivers, duplicated triangles
    P = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 0], [0, 0, 0], [0, 0, 0]], np.float32)
    for I in (np.tile([[0, 1, 2]], (50, 1)), np.tile([[3, 4, 5]], (9, 1)), np.array([[0, 1, 2], [0, 2, 1]])):
        I = I.astype(np.uint32)
        a, b = build_bvh(P, I), O.bvh_build(P, I)
        assert np.array_equal(a["nodes"], b["nodes"]) and np.array_equal(a["order"], b["order"])


def test_parallel_bvh_build_matches_the_sequential_restatement():
    """Subtrees of at least 8192 triangles are decided on their own threads and the node numbers replayed in task
    order: the node array and slot order equal the sequential builder's (the oracle) on a 166k-triangle dome and on
    a mesh of many coincident centroids (the split-in-half fallback)."""
    import time

    sc = dome.make_dome_scene(seed=1, width=32, height=24, level=7)
    st = sc["static"]
    t0 = time.perf_counter()
    a = build_bvh(st["P"], st["I"], 4)
    t1 = time.perf_counter()
    b = O.bvh_build(st["P"], st["I"], 4)
    t2 = time.perf_counter()
    print(f"\nSAH build of {len(st['I'])} triangles: {1e3 * (t1 - t0):.0f} ms (library) vs {1e3 * (t2 - t1):.0f} ms (sequential restatement)")
    assert a["nodeCount"] == b["node_count"] and a["maxDepth"] == b["max_depth"]
    assert np.array_equal(a["nodes"], b["nodes"]) and np.array_equal(a["order"], b["order"])
    rng = np.random.default_rng(3)
    P = np.repeat(rng.normal(size=(40, 3)).astype(np.float32), 3, axis=0)
    P[::3] += 1e-3
    I = np.tile(np.arange(120, dtype=np.uint32).reshape(-1, 3), (600, 1))
    a, b = build_bvh(P, I), O.bvh_build(P, I)
    assert np.array_equal(a["nodes"], b["nodes"]) and np.array_equal(a["order"], b["order"])


def test_bvh_builder_rejects_bad_indices():
    lib = _lib.load()
    P = np.zeros((3, 3), np.float32)
    I = np.array([[0, 1, 7]], np.uint32)
    nodes = np.zeros(64, np.uint32)
    order = np.zeros(1, np.uint32)
    r = A.vt_bvh_result()
    st = lib.vt_bvh_build(P.ctypes.data_as(C.c_void_p), 3, I.ctypes.data_as(C.c_void_p), 1, 4,
                          nodes.ctypes.data_as(C.c_void_p), order.ctypes.data_as(C.c_void_p), C.byref(r))
    assert st == A.VT_ERR_ARG


def test_sensor_uniform_layout():
    p = S.sensor_params({"cfa": "RGGB", "readNoise": 2.0, "adcBits": 12, "esfSigmaPx": 0.3})
    u = S.pack_sensor_uniform(p, 640, 480, frame=3, seed=7, exposure=0.01, gain=2.0, cam_index=2)
    f = u.view(np.float32)
    assert list(u[:4]) == [640, 480, 0, 3] and u[26] == 7 and u[49] == 2
    assert f[5] == pytest.approx(np.sqrt(0.3 ** 2 - 1 / 12), rel=1e-6)   # optics blur minus the pixel aperture
    assert f[6] == pytest.approx(0.01) and f[7] == 2.0 and f[20] == 2.0 and f[24] == 4095.0 and f[27] == 1.0
    assert f[4] == pytest.approx(np.pi * 0.9 / 16)


def test_scene_descriptor_round_trip(dome_small):
    d = A.SceneDesc(dome_small)
    assert d.desc.n_static_tris == len(dome_small["static"]["I"]) and d.desc.n_bodies == 1
    assert d.desc.n_materials == len(dome_small["materials"]) and d.desc.bodies[0].kind == A.BODY_KIND["scope"]


@pytest.mark.skipif(has_gpu(), reason="checks the no-device path")
def test_no_gpu_fails_loudly(dome_small):
    lib = _lib.load()
    d = A.SceneDesc(dome_small)
    ctx = C.c_void_p()
    assert lib.vt_create(d.ref, None, C.byref(ctx)) == A.VT_ERR_NO_DEVICE
    from vtwin.renderer import TwinRenderer, VtError

    with pytest.raises(VtError):
        TwinRenderer.create(dome_small)


def test_ctypes_mirror_matches_header_layout(tmp_path):
    """Every struct of include/vtwin.h has the size and field offsets that vtwin/_abi.py gives it (compiled with gcc)."""
    import ctypes
    import shutil
    import subprocess

    from vtwin import _abi as A

    if shutil.which("gcc") is None:
        pytest.skip("no gcc")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    names = [n for n in dir(A) if n.startswith("vt_") and isinstance(getattr(A, n), type) and issubclass(getattr(A, n), ctypes.Structure)]
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "vtwin.h"', "int main(void) {"]
    for n in names:
        lines.append(f'  printf("{n} %zu\\n", sizeof({n}));')
        for f in getattr(A, n)._fields_:
            lines.append(f'  printf("{n}.{f[0]} %zu\\n", offsetof({n}, {f[0]}));')
    lines.append("  return 0;\n}")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(root, "include"), str(src), "-o", str(exe)], check=True)
    got = dict(l.split() for l in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines())
    for n in names:
        S = getattr(A, n)
        assert int(got[n]) == ctypes.sizeof(S), n
        for f in S._fields_:
            assert int(got[f"{n}.{f[0]}"]) == getattr(S, f[0]).offset, f"{n}.{f[0]}"


def test_lite_geometry_matches_oracle():
    """The raster pass's geometry (vt_lite_geometry: the static mesh + the posed bodies sliced by sliceTris,
    lite_nodes/renderer.js:443-586) is the CPU restatement's, word for word; no device needed."""
    import oracle as O
    from vtwin import dome
    from vtwin.lite import lite_geometry

    sc = dome.make_scope_scene(seed=2, level=4, n_tools=2, width=64, height=36)
    V, I = lite_geometry(sc, 0.003, 0.01)
    Vo, Io = O.Scene(sc).lite_geometry(0.003, 0.01)
    assert V.shape == Vo.shape and I.shape == Io.shape
    assert np.array_equal(V, Vo) and np.array_equal(I, Io)
    assert len(I) > len(sc["static"]["I"]) + 1000


def test_lite_geometry_slices_fixtures_with_their_own_step():
    """Bodies of kind 'fixture' are sliced with subdiv_fixture (lite_nodes/renderer.js:560), the others with
    subdiv_h; same words as the restatement."""
    import oracle as O
    from vtwin import dome
    from vtwin.lite import lite_geometry

    sc = dome.make_scope_scene(seed=2, level=3, n_tools=2, width=64, height=36)
    sc["bodies"][2] = {**sc["bodies"][2], "kind": "fixture"}
    V, I = lite_geometry(sc, 0.003, 0.01)
    Vo, Io = O.Scene(sc).lite_geometry(0.003, 0.01)
    assert np.array_equal(V, Vo) and np.array_equal(I, Io)
    ns = len(sc["static"]["P"])
    inst = V[ns:, 3] >> 16
    P = V[ns:, :3].view(np.float32)
    tri_inst = inst[I[len(sc["static"]["I"]):, 0] - ns]
    T = I[len(sc["static"]["I"]):] - ns
    ext = lambda m: (P[T[m]].max(axis=1) - P[T[m]].min(axis=1)).max()
    assert ext(tri_inst == 1) <= 0.003 + 1e-7 and 0.003 + 1e-7 < ext(tri_inst == 2) <= 0.01 + 1e-7
