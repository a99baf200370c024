"""The raster camera pass of lite_nodes (vt_lite_*) against its CPU restatement, stage by stage.

lite_nodes/renderer.js draws the twin's cameras by rasterisation on top of the tracer's node radiosity. Each stage is
checked on its own inputs: the raster geometry and emitter samples bit for bit, the view uniform against a
restatement of _viewData (:766), the vertex stage to float rounding, the rasteriser (sample keys of the camera pass,
the shadow maps) bit for bit from the same clip coordinates, the fragment stage + resolve per pixel to float
rounding from the same keys, clip coordinates and shadow maps, and the display look bit for bit.
"""
import math

import numpy as np
import pytest

import oracle as O
from vtwin import _abi as A
from vtwin import dome
from vtwin.lite import LiteNodesRenderer, raster

pytestmark = pytest.mark.gpu

EMPTY = np.uint64(2**64 - 1)


@pytest.fixture(scope="module")
def lite():
    sc = dome.make_scope_scene(seed=2, level=5, n_tools=3, width=320, height=180)
    r = LiteNodesRenderer.create(sc, smRes=512, scopeSize=(320, 180))
    poses = dome.scope_poses(3, 3, seed=9)
    r.set_pose_array(poses[0])
    for c in r.cameras:
        r.renderCamera(c)
    S = O.Scene(sc)
    yield sc, r, S, poses
    r.destroy()


def _view_restated(sc, r, cam, poses0):
    """lite_nodes/renderer.js:766 _viewData, restated here in numpy (float64 -> float32)."""
    f = np.zeros(128, np.float64)
    u = np.zeros(4, np.uint32)
    T = np.asarray(poses0[0], np.float64).reshape(4, 4).T      # the scope body's pose
    Rs, Ps = T[:3, :3], T[:3, 3]
    o = r.o
    if cam < len(sc["cameras"]):
        c = sc["cameras"][cam]
        M = np.array(c["T_D_C"], np.float64).reshape(4, 4)
        R, pos, mode = M[:3, :3], M[:3, 3], 0
        lens = [c["fx"], c["fy"], c["cx"], c["cy"]]
        D = list(c["k"])
        W, H = c["size"]
        cut = min(1.45, 1.5 * 0.97)
    else:
        z = Rs @ np.array(o["scopeViewDir"], np.float64)
        z /= np.linalg.norm(z)
        upK = Rs @ np.array([0.0, 1.0, 0.0])
        up = upK - z * (upK @ z)
        up /= np.linalg.norm(up)
        y = -up
        x = np.cross(y, z)
        R, pos, mode = np.stack([x, y, z], 1), Rs @ np.array(o["scopeObjective"], np.float64) + Ps, 1
        W, H = o["scopeSize"]
        fx = W / 2 / math.tan(math.radians(o["scopeHfovDeg"]) / 2)
        lens, D, cut = [fx, fx, W / 2, H / 2], [0, 0, 0, 0], 1.5
    f[0:3], f[4:7], f[8:11] = R[:, 0], R[:, 1], R[:, 2]
    f[12:15], f[15] = pos, mode
    f[16:20], f[20:24] = lens, D
    L0 = sc["emitter"]["L0"]
    f[24:28] = [W, H, cut, 1000.0 / max(L0)]
    ax = Rs @ np.array([0.0, math.sin(0.0), math.cos(0.0)])
    ax /= np.linalg.norm(ax)
    t = np.cross([1.0, 0.0, 0.0] if abs(ax[0]) < 0.9 else [0.0, 1.0, 0.0], ax)
    t /= np.linalg.norm(t)
    f[36:39], f[40:43], f[44:47] = ax, t, np.cross(ax, t)
    f[43], f[47] = math.radians(o["smThetaMaxDeg"]), o["far"]
    return f.astype(np.float32)


def test_geometry_and_emitter_samples_match_the_restatement(lite):
    sc, r, S, poses = lite
    V, I = S.lite_geometry(subdiv=0.003, subdiv_fixture=0.01)
    assert np.array_equal(r.debug_buffer(A.VT_LITE_GEOM), V)
    assert np.array_equal(r.debug_buffer(A.VT_LITE_INDEX), I)
    es, _ = S.lite_emitter(96, poses[0][0])
    got = r.debug_buffer(A.VT_LITE_EMIT)
    print(f"\n{len(I)} raster triangles ({r.stats['dynVerts']} posed-body vertices), emitter samples max diff {np.abs(got - es).max():.2e}")
    assert np.abs(got - es).max() <= 1e-7


def test_view_uniform_matches_view_data(lite):
    sc, r, S, poses = lite
    for c in range(len(r.cameras)):
        v = r.view(c)
        want = _view_restated(sc, r, c, poses[0])
        mask = np.ones(128, bool)
        mask[28:36] = False          # misc words (integers) and the environment (eAvg-dependent) checked below
        mask[39] = False
        mask[48:128] = False         # sector origins: checked through the shadow maps
        assert np.allclose(v[mask], want[mask], rtol=1e-6, atol=1e-7), (c, np.abs(v - want)[mask].max())
        misc = v[28:32].view(np.uint32)
        assert misc[1] == 24 and misc[2] == 96 and misc[3] == 0
        assert v[35] == 0.5


def test_vertex_stage_matches_restatement(lite):
    sc, r, S, poses = lite
    V = r.debug_buffer(A.VT_LITE_GEOM)
    S.load_uniform(r.tr.scene_uniform())
    for c in range(len(r.cameras)):
        r.renderCamera(c)
        clip = r.debug_buffer(A.VT_LITE_CLIP, c)
        want = S.lite_vertex(r.view(c), V)
        d = np.abs(clip - want) / np.maximum(np.abs(want), 1.0)
        print(f"\ncamera {r.cameras[c]}: clip max rel diff {d.max():.2e}")
        assert d.max() < 2e-5


def test_rasteriser_keys_and_shadow_maps_bit_exact(lite):
    """Same clip coordinates in, the same sample keys out: nearest triangle, depth bits, coverage, ties."""
    sc, r, S, poses = lite
    I = r.debug_buffer(A.VT_LITE_INDEX)
    for c in range(len(r.cameras)):
        r.renderCamera(c)
        clip = r.debug_buffer(A.VT_LITE_CLIP, c)
        keys = r.debug_buffer(A.VT_LITE_KEYS, c)
        w, h = r.size(c)
        want = O.raster(clip, I, w, h, 4)
        cov = (keys != EMPTY).mean()
        print(f"\ncamera {r.cameras[c]}: {cov:.3f} of the samples covered, {len(np.unique(keys & np.uint64(0xffffffff)))} triangles")
        assert cov > 0.2
        assert np.array_equal(keys, want), (keys != want).sum()
    # shadow maps: the static casters' and the posed bodies' four sector layers
    sclip = r.debug_buffer(A.VT_LITE_SM_CLIP)
    ns = int(r.info()["staticTris"])
    res = 512
    for which, t0, nt in ((A.VT_LITE_SM_STATIC, 0, ns), (A.VT_LITE_SM_DYN, ns, len(I) - ns)):
        sm = r.debug_buffer(which)
        for k in range(4):
            want = O.raster(sclip[k], I, res, res, 1, t0=t0, nt=nt)[..., 0]
            wd = (want >> np.uint64(32)).astype(np.uint32)
            wd[want == EMPTY] = 0xFFFFFFFF
            assert np.array_equal(sm[k], wd), (which, k, (sm[k] != wd).sum())
        print(f"shadow map {which}: {(sm != 0xFFFFFFFF).mean():.3f} of the texels hold a caster")


def test_fragment_stage_matches_restatement(lite):
    """The shading of every (pixel, triangle) at the pixel centre, the resolve through half floats and FINISH."""
    sc, r, S, poses = lite
    V, I = r.debug_buffer(A.VT_LITE_GEOM), r.debug_buffer(A.VT_LITE_INDEX)
    st, slot = r.tr.get_node_state()
    S.set_node_state(st, slot)
    S.load_uniform(r.tr.scene_uniform())
    es = r.debug_buffer(A.VT_LITE_EMIT)
    sms, smd = r.debug_buffer(A.VT_LITE_SM_STATIC), r.debug_buffer(A.VT_LITE_SM_DYN)
    inv = float(1.0 / (1000.0 / max(sc["emitter"]["L0"])))
    for c in range(len(r.cameras)):
        out = np.zeros((r.size(c)[1], r.size(c)[0], 4), np.float32)
        r.renderCamera(c, out=out)
        circle = 0.95 * 320 / 2 if r.cameras[c] == "SCOPE" else 0.0
        want = S.lite_shade(r.view(c), V, I, r.debug_buffer(A.VT_LITE_CLIP, c), r.debug_buffer(A.VT_LITE_KEYS, c), es, sms, smd, inv,
                            circle=circle)
        g, w = out[..., :3].astype(np.float64), want[..., :3].astype(np.float64)
        rel = np.abs(g - w) / np.maximum(np.abs(w), 1e-3 * max(w.max(), 1e-30))
        print(f"\ncamera {r.cameras[c]}: mean radiance {g.mean():.4g}, within 1e-3: {(rel <= 1e-3).mean():.5f}, "
              f"median {np.median(rel):.1e}, max {rel.max():.2e}")
        assert g.max() > 0
        assert (rel <= 1e-3).mean() > 0.999 and np.median(rel) < 1e-5
        if circle:
            yy, xx = np.mgrid[0:180, 0:320]
            outside = np.hypot(xx + 0.5 - 160, yy + 0.5 - 90) > circle
            assert (out[outside][:, :3] == 0).all()


def test_display_bit_exact_and_auto_exposure(lite):
    sc, r, S, poses = lite
    c = 0
    r.renderCamera(c)
    L = r.readback(c, "linear")
    prev = r._disp.get(c, {}).get("prev", np.zeros(4, np.uint32)).copy()
    out = r.sensor(c)
    rgba = r.readback(c, "rgba8")
    want, st = O.lite_display(out["du"], prev, L)
    assert np.array_equal(rgba, want), (rgba != want).sum()
    assert np.array_equal(out["stats"], st)
    assert np.array_equal(r.readback(c, "rgb8"), rgba[..., :3])
    assert r.readback(c, "yuv420") is None and r.readback(c, "raw") is None
    # auto exposure: the mean luma settles near the target
    for _ in range(4):
        out = r.sensor(c)
    m = r.readback(c, "rgb8").mean()
    print(f"\ndisplay mean {m:.1f}, meanY {out['meanY']:.4g}")
    assert 20 < m < 235


def test_shadow_maps_follow_the_poses(lite):
    """The static casters' map is re-rendered only when the scope moves, the posed bodies' map when any pose
    changes (lite_nodes/renderer.js:849-851)."""
    sc, r, S, poses = lite
    r.renderCamera(0)
    i = r.info()
    assert i["shadowStaticMs"] == 0.0 and i["shadowDynMs"] == 0.0
    p = poses[0].copy()
    p[1:] = poses[1][1:]                        # tools move, the scope stays
    r.set_pose_array(p)
    r.renderCamera(0)
    i = r.info()
    assert i["shadowStaticMs"] == 0.0 and i["shadowDynMs"] > 0.0
    r.set_pose_array(poses[1])                  # the scope moves
    r.renderCamera(0)
    i = r.info()
    assert i["shadowStaticMs"] > 0.0 and i["shadowDynMs"] > 0.0
    print(f"\nlast pass: {i}")
    r.set_pose_array(poses[0])
    r.renderCamera(0)


def test_scope_visibility_and_unknown_camera(lite):
    sc, r, S, poses = lite
    v = r.view("SCOPE")
    pos, z = v[12:15].astype(np.float64), v[8:11].astype(np.float64)
    pts = np.array([pos + 0.05 * z, pos - 0.05 * z, pos + 0.05 * z + 0.2 * v[0:3].astype(np.float64)])
    assert r.visible("SCOPE", pts).tolist() == [True, False, False]
    from vtwin._lib import VtError

    with pytest.raises(VtError):
        r.renderCamera("NOPE")


def test_raster_entry_point_matches_restatement():
    """vt_raster on random triangles, some crossing w = 0, the near and far planes and the guard band."""
    from vtwin.renderer import TwinRenderer

    rng = np.random.default_rng(4)
    n = 400
    clip = np.concatenate([rng.uniform(-1.5, 1.5, (3 * n, 2)), rng.uniform(-0.2, 1.2, (3 * n, 1)), rng.uniform(-0.3, 1.5, (3 * n, 1))],
                          1).astype(np.float32)
    clip[::7, :2] *= 30.0
    idx = np.arange(3 * n, dtype=np.uint32).reshape(n, 3)
    sc = dome.make_dome_scene(seed=1, width=32, height=24, level=2)
    tr = TwinRenderer.create(sc, nodes=False)
    try:
        for W, H, s in ((97, 61, 4), (64, 64, 1)):
            got = raster(tr, clip, idx, W, H, s)
            want = O.raster(clip, idx, W, H, s)
            assert np.array_equal(got, want), (W, H, s, (got != want).sum())
            assert (got != EMPTY).mean() > 0.3
    finally:
        tr.destroy()


def test_parity_after_the_scope_moves(lite):
    """A second pose with the scope moved: emitter samples, sector origins and both shadow maps re-made; keys and
    maps bit-exact again, fragments within tolerance (also for SCOPE, whose camera follows the scope)."""
    sc, r, S, poses = lite
    r.set_pose_array(poses[2])
    es, _ = S.lite_emitter(96, poses[2][0])
    assert np.abs(r.debug_buffer(A.VT_LITE_EMIT) - es).max() <= 1e-7
    V, I = r.debug_buffer(A.VT_LITE_GEOM), r.debug_buffer(A.VT_LITE_INDEX)
    for c in (0, len(r.cameras) - 1):
        w, h = r.size(c)
        out = np.zeros((h, w, 4), np.float32)
        r.renderCamera(c, out=out)
        clip, keys = r.debug_buffer(A.VT_LITE_CLIP, c), r.debug_buffer(A.VT_LITE_KEYS, c)
        assert np.array_equal(keys, O.raster(clip, I, w, h, 4))
        st, slot = r.tr.get_node_state()
        S.set_node_state(st, slot)
        S.load_uniform(r.tr.scene_uniform())
        sms, smd = r.debug_buffer(A.VT_LITE_SM_STATIC), r.debug_buffer(A.VT_LITE_SM_DYN)
        circle = 0.95 * w / 2 if r.cameras[c] == "SCOPE" else 0.0
        want = S.lite_shade(r.view(c), V, I, clip, keys, r.debug_buffer(A.VT_LITE_EMIT), sms, smd,
                            float(1.0 / (1000.0 / max(sc["emitter"]["L0"]))), circle=circle)
        g, wv = out[..., :3].astype(np.float64), want[..., :3].astype(np.float64)
        rel = np.abs(g - wv) / np.maximum(np.abs(wv), 1e-3 * max(wv.max(), 1e-30))
        print(f"\nmoved scope, camera {r.cameras[c]}: within 1e-3 {(rel <= 1e-3).mean():.5f}")
        assert (rel <= 1e-3).mean() > 0.999
    sclip = r.debug_buffer(A.VT_LITE_SM_CLIP)
    ns = int(r.info()["staticTris"])
    sm = r.debug_buffer(A.VT_LITE_SM_STATIC)
    want = O.raster(sclip[1], I, 512, 512, 1, t0=0, nt=ns)[..., 0]
    wd = (want >> np.uint64(32)).astype(np.uint32)
    wd[want == EMPTY] = 0xFFFFFFFF
    assert np.array_equal(sm[1], wd)
    r.set_pose_array(poses[0])
    for c in r.cameras:
        r.renderCamera(c)


def test_debug_modes_no_shadows_and_visibility():
    """debug 1 renders without shadow maps (every sector visible), debug 2 writes the mean sector visibility as
    grey (lite_nodes/renderer.js:330-336)."""
    sc = dome.make_scope_scene(seed=3, level=4, n_tools=2, width=160, height=90)
    T = dome.scope_poses(1, 2, seed=4)[0]
    imgs = {}
    for dbg in (0, 1, 2):
        r = LiteNodesRenderer.create(sc, smRes=256, scopeSize=(160, 90), debug=dbg)
        try:
            r.set_pose_array(T)
            out = np.zeros((90, 160, 4), np.float32)
            r.renderCamera(0, out=out)
            imgs[dbg] = out[..., :3]
        finally:
            r.destroy()
    assert imgs[1].mean() >= imgs[0].mean()                        # no shadows: at least as bright
    vis = imgs[2]
    scale = 1000.0 / max(sc["emitter"]["L0"])
    assert np.isfinite(vis).all() and 0.0 <= vis.min() and vis.max() <= 1.0 / scale * 1.001
    assert vis.max() > 0
