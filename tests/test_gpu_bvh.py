"""The BVH build on the GPU (vt_bvh_build_device, also vt_create's static BVH) against the sequential restatement of
gpu/bvh.js:18-161 in the oracle and the host builder: the same node words, slot order, depth and bounds, bit for
bit, on the dome, random and degenerate meshes, coincident centroids (the split-in-half fallback after a
partition that moved every slot) and signed zeros (the node boxes keep the first slot among equal values)."""
import os
import sys
import time

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "veridien-twin_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle as O  # noqa: E402
from vtwin import dome  # noqa: E402
from vtwin.renderer import build_bvh  # noqa: E402

pytestmark = pytest.mark.gpu


def _same(a, b):
    assert a["nodeCount"] == b["node_count"] and a["maxDepth"] == b["max_depth"]
    assert np.array_equal(a["nodes"], b["nodes"]) and np.array_equal(a["order"], b["order"])
    assert np.array_equal(np.float32(a["bmin"]).view(np.uint32), np.float32(b["bmin"]).view(np.uint32))
    assert np.array_equal(np.float32(a["bmax"]).view(np.uint32), np.float32(b["bmax"]).view(np.uint32))


@pytest.mark.parametrize("leaf", [1, 4, 8])
def test_device_build_matches_oracle_on_dome(leaf):
    st = dome.make_dome_scene(seed=1, width=32, height=24, level=7)["static"]
    _same(build_bvh(st["P"], st["I"], leaf, device=0), O.bvh_build(st["P"], st["I"], leaf))


def test_device_build_matches_oracle_on_random_and_degenerate_meshes():
    rng = np.random.default_rng(11)
    for n in [0, 1, 2, 3, 5, 17, 100, 1000, 20000]:
        P = rng.normal(size=(3 * max(n, 1), 3)).astype(np.float32)
        I = np.arange(3 * n, dtype=np.uint32).reshape(-1, 3)
        for leaf in (1, 4):
            _same(build_bvh(P, I, leaf, device=0), O.bvh_build(P, I, leaf))
    P = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 0], [0, 0, 0], [0, 0, 0]], np.float32)
    for I in (np.tile([[0, 1, 2]], (50, 1)), np.tile([[3, 4, 5]], (9, 1)), np.array([[0, 1, 2], [0, 2, 1]]),
              np.tile([[0, 1, 2]], (30000, 1))):
        I = I.astype(np.uint32)
        _same(build_bvh(P, I, 4, device=0), O.bvh_build(P, I, 4))


def test_device_build_at_task_size_boundaries():
    """Meshes whose root and top ranges sit at the builder's boundaries: one thread (32 slots or fewer), one warp,
    one block (1024-8191), 4096-slot chunks (8192 and more, one of them partial)."""
    rng = np.random.default_rng(21)
    for n in (32, 33, 1023, 1024, 4096, 4097, 8191, 8192, 8193, 12289, 16385):
        P = rng.normal(size=(3 * n, 3)).astype(np.float32)
        I = np.arange(3 * n, dtype=np.uint32).reshape(-1, 3)
        for leaf in (1, 4):
            _same(build_bvh(P, I, leaf, device=0), O.bvh_build(P, I, leaf))


@pytest.mark.parametrize("leaf", [600, 2500])
def test_device_build_large_leaves(leaf):
    """A leaf size large enough that ranges handled by whole blocks (1024-8191 slots) and by chunks (8192 slots and
    more) end as leaves, or split at the median when no split is priced."""
    st = dome.make_dome_scene(seed=1, width=32, height=24, level=6)["static"]
    _same(build_bvh(st["P"], st["I"], leaf, device=0), O.bvh_build(st["P"], st["I"], leaf))
    rng = np.random.default_rng(12)
    P = rng.normal(size=(3 * 40000, 3)).astype(np.float32)
    I = np.arange(3 * 40000, dtype=np.uint32).reshape(-1, 3)
    _same(build_bvh(P, I, leaf, device=0), O.bvh_build(P, I, leaf))


def test_device_build_coincident_centroids_and_signed_zeros():
    rng = np.random.default_rng(3)
    P = np.repeat(rng.normal(size=(40, 3)).astype(np.float32), 3, axis=0)
    P[::3] += 1e-3
    I = np.tile(np.arange(120, dtype=np.uint32).reshape(-1, 3), (600, 1))
    _same(build_bvh(P, I, 4, device=0), O.bvh_build(P, I, 4))
    # a grid whose coordinates are +0 and -0 in random places: box corners at zero keep the first slot's sign
    g = np.stack(np.meshgrid(np.arange(-20, 21), np.arange(-20, 21), indexing="ij"), -1).reshape(-1, 2).astype(np.float32) * 0.05
    P = np.zeros((len(g), 3), np.float32)
    P[:, :2] = g
    P[:, 2] = np.where(rng.random(len(g)) < 0.5, np.float32(-0.0), np.float32(0.0))
    P[:, :2][P[:, :2] == 0] *= np.where(rng.random((P[:, :2] == 0).sum()) < 0.5, -1, 1).astype(np.float32)
    quads = np.array([[i * 41 + j, (i + 1) * 41 + j, i * 41 + j + 1, (i + 1) * 41 + j + 1] for i in range(40) for j in range(40)])
    I = np.concatenate([quads[:, [0, 1, 2]], quads[:, [2, 1, 3]]]).astype(np.uint32)
    I = I[rng.permutation(len(I))]
    assert (np.signbit(P) & (P == 0)).any()
    for leaf in (1, 4):
        _same(build_bvh(P, I, leaf, device=0), O.bvh_build(P, I, leaf))


def test_device_build_matches_host_builder_on_657k_triangles():
    st = dome.make_dome_scene(seed=1, width=32, height=24, level=8)["static"]
    build_bvh(np.eye(3, dtype=np.float32), np.array([[0, 1, 2], [0, 2, 1]], np.uint32), 1, device=0)   # context setup untimed
    t0 = time.perf_counter()
    a = build_bvh(st["P"], st["I"], 4, device=0)
    t1 = time.perf_counter()
    b = build_bvh(st["P"], st["I"], 4)
    t2 = time.perf_counter()
    print(f"\nSAH build of {len(st['I'])} triangles: {1e3 * (t1 - t0):.1f} ms on the GPU (host buffers in and out) vs "
          f"{1e3 * (t2 - t1):.1f} ms on {os.cpu_count()} host threads")
    assert a["nodeCount"] == b["nodeCount"] and a["maxDepth"] == b["maxDepth"]
    assert np.array_equal(a["nodes"], b["nodes"]) and np.array_equal(a["order"], b["order"])
