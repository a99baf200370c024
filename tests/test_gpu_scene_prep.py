"""Weld and subdivide on the device (vt_weld_device, vt_subdivide_device) against the host code (vt_weld, vt_subdivide,
themselves checked against the plain-Python restatement of gpu/scene_gpu.js:68-143 in tests/test_scene_prep.py): the
same vertices, normals and triangles in the same order, bit for bit, on meshes that exercise every path (noise at the
weld tolerance, one long run of identical vertices, degenerate triangles, empty input, long thin triangles that take
the two-split case, a scan over more than 2^20 items, a pass limit)."""
import time

import numpy as np
import pytest

from vtwin import dome
from vtwin import scene_io as S

pytestmark = pytest.mark.gpu


def _unwelded(level, r=0.05, seed=0, noise=2e-9):
    V, F = dome.icosphere(level)
    rng = np.random.default_rng(seed)
    P = (V * r).astype(np.float32)
    N = V.astype(np.float32)
    P3 = P[F.ravel()].copy()
    N3 = N[F.ravel()].copy()
    P3[::2] += rng.uniform(-noise, noise, P3[::2].shape).astype(np.float32)
    return P3, N3, np.arange(len(P3), dtype=np.uint32)


def _same(a, b):
    for x, y in zip(a, b):
        assert x.shape == y.shape and np.array_equal(x, y), (x.shape, y.shape)


@pytest.mark.parametrize("level,noise", [(2, 2e-9), (3, 0.0), (4, 5e-8)])
def test_weld_device_matches_host(level, noise):
    P, N, I = _unwelded(level, noise=noise)
    _same(S.weld(P, N, I, device=0), S.weld(P, N, I))


def test_weld_device_edge_cases():
    # one long run: every vertex the same; every triangle degenerate
    P = np.tile(np.array([[0.1, 0.2, 0.3]], np.float32), (3000, 1))
    N = np.tile(np.array([[0.0, 0.0, 1.0]], np.float32), (3000, 1))
    I = np.arange(3000, dtype=np.uint32)
    a = S.weld(P, N, I, device=0)
    _same(a, S.weld(P, N, I))
    assert len(a[0]) == 1 and len(a[2]) == 0
    # empty
    e = S.weld(np.zeros((0, 3), np.float32), np.zeros((0, 3), np.float32), np.zeros(0, np.uint32), device=0)
    assert len(e[0]) == 0 and len(e[2]) == 0
    # shuffled vertices and a few degenerate triangles
    P, N, I = _unwelded(3, noise=1e-8, seed=4)
    rng = np.random.default_rng(5)
    perm = rng.permutation(len(P)).astype(np.uint32)
    P2, N2 = P[perm], N[perm]
    inv = np.empty_like(perm)
    inv[perm] = np.arange(len(perm), dtype=np.uint32)
    I2 = inv[I]
    I2[:30] = I2[0]
    _same(S.weld(P2, N2, I2, device=0), S.weld(P2, N2, I2))


def test_weld_device_large_scan():
    """more than 2^20 vertices: the scans recurse twice"""
    P, N, I = _unwelded(7, noise=2e-9)
    extra = 1100000 - len(P)
    if extra > 0:
        P = np.concatenate([P, P[:extra]])
        N = np.concatenate([N, N[:extra]])
        I = np.concatenate([I, (np.arange(extra - extra % 3, dtype=np.uint32) + len(I))])
    t0 = time.perf_counter()
    b = S.weld(P, N, I)
    t1 = time.perf_counter()
    a = S.weld(P, N, I, device=0)
    t2 = time.perf_counter()
    print(f"\nweld of {len(P)} vertices: host {1e3 * (t1 - t0):.1f} ms, device (host buffers in and out) {1e3 * (t2 - t1):.1f} ms")
    _same(a, b)


@pytest.mark.parametrize("level,h", [(1, 0.012), (2, 0.004), (3, 0.02)])
def test_subdivide_device_matches_host(level, h):
    P, N, I = S.weld(*_unwelded(level, noise=0.0))
    _same(S.subdivide(P, N, I, h, device=0), S.subdivide(P, N, I, h))


def test_subdivide_device_thin_triangles_and_pass_limit():
    # long thin triangles: most passes split two of their three edges (the quad's shorter diagonal decides)
    rng = np.random.default_rng(9)
    n = 400
    base = rng.uniform(-1, 1, (n, 3))
    P = np.concatenate([base, base + rng.uniform(-0.3, 0.3, (n, 3)), base + rng.uniform(-0.01, 0.01, (n, 3))])
    N = rng.normal(size=P.shape)
    N /= np.linalg.norm(N, axis=1, keepdims=True)
    I = np.stack([np.arange(n), np.arange(n) + n, np.arange(n) + 2 * n], 1).astype(np.uint32).ravel()
    for passes in (1, 3, 24):
        _same(S.subdivide(P, N, I, 0.05, max_passes=passes, device=0), S.subdivide(P, N, I, 0.05, max_passes=passes))
    # opposite normals: the normalised mean is below 1e-6, the first endpoint's normal is kept
    N2 = N.copy()
    N2[n:2 * n] = -N2[:n]
    _same(S.subdivide(P, N2, I, 0.2, device=0), S.subdivide(P, N2, I, 0.2))


def test_subdivide_device_dome_mesh():
    sc = dome.make_dome_scene(seed=1, width=32, height=24, level=6)
    st = sc["static"]
    P = np.asarray(st["P"], np.float64).reshape(-1, 3)
    N = np.asarray(st["N"], np.float64).reshape(-1, 3)
    I = np.asarray(st["I"], np.uint32).ravel()
    t0 = time.perf_counter()
    b = S.subdivide(P, N, I, 0.02)
    t1 = time.perf_counter()
    a = S.subdivide(P, N, I, 0.02, device=0)
    t2 = time.perf_counter()
    print(f"\nsubdivide of {len(I) // 3} triangles into {len(b[2]) // 3}: host {1e3 * (t1 - t0):.1f} ms, device {1e3 * (t2 - t1):.1f} ms")
    _same(a, b)
