"""The camera sensor chain on the GPU (vt_sensor_frame) against its CPU restatement, bit for bit.

The chain (gpu/wgsl/sensor.wgsl.js): optics with the relative-illumination map and the horizontal blur, veiling glare,
expose, demosaic, white balance + CCM, noise reduction, tone, unsharp mask, YCbCr. Both sides perform the same
sequence of separately rounded float32 operations with the project's own fixed-order exp / log, so raw DN, 8-bit RGB,
the YCbCr planes and the AE / AWB statistics must be identical for every parameter set.
"""
import numpy as np
import pytest

import oracle as O
from vtwin import _abi as A
from vtwin import dome
from vtwin.renderer import TwinRenderer

pytestmark = pytest.mark.gpu

VARIANTS = [
    {},   # the defaults: GRBG, bilinear, no noise reduction, sRGB, 4:2:0, no glare
    {"cfa": "RGGB", "demosaic": "edge-aware", "noiseReduction": "bilateral", "tone": "gamma", "sharpenAmount": 0.6,
     "sharpenRadius": 2, "chroma": "4:4:4", "glareFraction": 0.05},
    {"cfa": "BGGR", "demosaic": "hamilton-adams", "tone": "srgb", "sCurveC": 1.4, "blackOffset": 0.02, "blackLevel": 64.0,
     "glareFraction": 0.1, "glareLevel": 8},
    {"cfa": "GBRG", "tone": "linear", "wb": [1.8, 1.0, 1.4], "ccm": [[1.6, -0.4, -0.2], [-0.3, 1.5, -0.2], [0.0, -0.5, 1.5]],
     "noiseReduction": "on", "nrSigmaPx": 0.8, "esfSigmaPx": 1.4},
]


@pytest.fixture(scope="module")
def rendered():
    sc = dome.make_dome_scene(seed=1, width=97, height=63, level=4, with_instruments=2)
    r = TwinRenderer.create(sc)
    T = dome.instrument_poses(n_poses=1, n_tools=2, seed=11)[0]
    r.set_pose_array(np.concatenate([A.identity_poses(1), T]))
    r.renderCamera(0, spp=4, lightSamples=2, seed=1, mode=A.VT_SHADE_PATH, max_depth=3)
    yield sc, r
    r.destroy()


def test_relative_illumination_matches_fp64_restatement(rendered):
    sc, r = rendered
    p = {**r.sensor_p, "vignettingThetaDeg": [0.0, 40.0, 90.0], "vignetting": [1.0, 0.9, 0.6], "pupilExponent": 1.3}
    vt = np.array(p["vignettingThetaDeg"], np.float64)
    vv = np.array(p["vignetting"], np.float64)
    import ctypes as C

    assert r.lib.vt_set_relative_illumination(r._ctx, 0, None, 1.3, vt.ctypes.data_as(C.c_void_p), vv.ctypes.data_as(C.c_void_p), 3) == 0
    got = r.relative_illumination(0)
    want = O.Scene(sc).ri_map(0, 1.3, vt, vv)
    rel = np.abs(got.astype(np.float64) - want) / np.maximum(want, 1e-6)
    print(f"\nrelative illumination: {got.min():.4f}..{got.max():.4f}, max rel diff {rel.max():.2e}")
    assert rel.max() < 1e-6 and got.max() <= 1.0 + 1e-6 and got.min() > 0.0


@pytest.mark.parametrize("k", range(len(VARIANTS)))
def test_chain_bit_exact(rendered, k):
    sc, r = rendered
    L = r.readback(0, "linear")
    out = r.sensor(0, seed=3, frame=7, exposure_s=2e-3, gain=1.5, params=VARIANTS[k])
    ri = r.relative_illumination(0)
    raw = r.readback(0, "raw")
    rgba = r.readback(0, "rgba8")
    rgb = r.readback(0, "rgb8")
    yuv = r.readback(0, "yuv420")
    raw_w, rgba_w, yuv_w, st_w = O.isp_chain(out["uniform"], L, ri)
    print(f"\nvariant {k}: raw mean {raw.mean():.1f} DN, rgb mean {rgba[..., :3].mean():.1f}, stats {out['stats'].tolist()}")
    assert np.array_equal(raw, raw_w), (np.abs(raw - raw_w).max(), (raw != raw_w).sum())
    assert np.array_equal(rgba, rgba_w), ((rgba != rgba_w).sum(),)
    assert np.array_equal(rgb, rgba[..., :3])
    assert np.array_equal(out["stats"], st_w)
    if int(out["uniform"][48]):
        for plane in ("y", "cb", "cr"):
            assert np.array_equal(yuv[plane], yuv_w[plane]), plane
    assert 5 < rgba[..., :3].mean() < 250     # not saturated or black: the comparison means something


@pytest.mark.parametrize("k", [0, 1, 3])
def test_chain_bit_exact_1280x720(k):
    """The frame size the sensor chain is measured at (1280 x 720): every fused tile of the expose, demosaic, noise
    reduction and output passes, the image's ragged right and bottom tiles and the block statistics, bit for bit."""
    sc = dome.make_dome_scene(seed=2, width=1280, height=720, level=4, with_instruments=2)
    r = TwinRenderer.create(sc)
    try:
        T = dome.instrument_poses(n_poses=1, n_tools=2, seed=5)[0]
        r.set_pose_array(np.concatenate([A.identity_poses(1), T]))
        r.renderCamera(0, spp=1, lightSamples=1, seed=2, mode=A.VT_SHADE_PATH, max_depth=2)
        L = r.readback(0, "linear")
        out = r.sensor(0, seed=9, frame=3, exposure_s=2e-3, gain=1.5, params=VARIANTS[k])
        raw_w, rgba_w, yuv_w, st_w = O.isp_chain(out["uniform"], L, r.relative_illumination(0))
        raw, rgba = r.readback(0, "raw"), r.readback(0, "rgba8")
        assert raw.shape == (720, 1280)
        assert np.array_equal(raw, raw_w), (np.abs(raw - raw_w).max(), (raw != raw_w).sum())
        assert np.array_equal(rgba, rgba_w), ((rgba != rgba_w).sum(),)
        assert np.array_equal(out["stats"], st_w)
        if int(out["uniform"][48]):
            yuv = r.readback(0, "yuv420")
            for plane in ("y", "cb", "cr"):
                assert np.array_equal(yuv[plane], yuv_w[plane]), plane
        assert 5 < rgba[..., :3].mean() < 250
    finally:
        r.destroy()


def test_auto_exposure_converges(rendered):
    """AE (gpu/sensor.js:128) moves the exposure toward the target mean luma 0.45 frame by frame; AWB gains stay
    finite and positive."""
    sc, r = rendered
    r._sens.clear()
    lumas, exps = [], []
    for _ in range(12):
        e = r.exposureOf(0)
        out = r.sensor(0, seed=0)
        lumas.append(out["meanLuma"])
        exps.append(e["time_s"])
    print(f"\nAE: luma {np.round(lumas, 3).tolist()}, exposure {exps}")
    assert abs(lumas[-1] - 0.45) < abs(lumas[0] - 0.45) or abs(lumas[-1] - 0.45) < 0.05
    awb = r._sens[0]["awb"]
    assert all(np.isfinite(awb)) and all(g > 0 for g in awb)
    # a manual exposure holds
    r.set_exposure(0, 1e-3)
    assert r.exposureOf(0)["time_s"] == 1e-3 and not r.exposureOf(0)["auto"]


def test_render_frame_matches_per_camera_calls():
    """renderFrame queues every camera's render and sensor chain in one library call (vt_render_frame) with one
    synchronisation; the images, statistics and the AE / AWB state it leaves must equal those of renderCamera +
    sensor called camera by camera (gpu/renderer.js:986)."""
    sc = dome.make_dome_scene(seed=1, width=97, height=63, level=4, with_instruments=2)
    sc["cameras"] = dome.batched_cameras(seed=3, n=3, width=80, height=56)
    T = dome.instrument_poses(n_poses=2, n_tools=2, seed=11)
    a, b = TwinRenderer.create(sc), TwinRenderer.create(sc)
    try:
        for k in range(2):
            for r in (a, b):
                r.set_pose_array(np.concatenate([A.identity_poses(1), T[k]]))
            fr = a.renderFrame(sensor=True, spp=2, lightSamples=2, seed=k)
            names = list(a.cameras)
            for c in names:
                b.renderCamera(c, spp=2, lightSamples=2, seed=k)
            st = {c: b.sensor(c) for c in names}
            b.frame += 1
            assert fr["ms"] > 0 and len(names) == 3
            for c in names:
                assert np.array_equal(a.readback(c, "linear"), b.readback(c, "linear")), (k, c)
                assert np.array_equal(a.readback(c, "rgba8"), b.readback(c, "rgba8")), (k, c)
                assert np.array_equal(fr[c]["stats"], st[c]["stats"]), (k, c)
                assert a.exposureOf(c) == b.exposureOf(c)
                assert a._sens[a._cam(c)]["awb"] == b._sens[b._cam(c)]["awb"]
    finally:
        a.destroy()
        b.destroy()


def test_render_frame_without_sensor():
    """vt_render_frame with no sensor uniforms renders every camera as renderCamera does."""
    sc = dome.make_dome_scene(seed=1, width=97, height=63, level=4, with_instruments=2)
    sc["cameras"] = dome.batched_cameras(seed=3, n=2, width=64, height=40)
    T = dome.instrument_poses(n_poses=1, n_tools=2, seed=11)[0]
    a, b = TwinRenderer.create(sc), TwinRenderer.create(sc)
    try:
        for r in (a, b):
            r.set_pose_array(np.concatenate([A.identity_poses(1), T]))
        fr = a.renderFrame(spp=2, lightSamples=1, seed=5)
        for c in list(b.cameras):
            b.renderCamera(c, spp=2, lightSamples=1, seed=5)
            assert np.array_equal(a.readback(c, "linear"), b.readback(c, "linear"))
        assert fr["ms"] > 0 and "stats" not in fr[list(a.cameras)[0]]
    finally:
        a.destroy()
        b.destroy()
