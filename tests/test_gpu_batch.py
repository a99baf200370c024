"""Batched multi-pose rendering against rendering each pose on its own (vt_render_batch vs vt_set_poses +
vt_render_camera + vt_sensor_camera): radiance and raw DN must be bit-identical for every camera and pose."""
import numpy as np
import pytest

from vtwin import _abi as A
from vtwin import dome
from vtwin import sensor as sensor_mod
from vtwin._lib import VtError
from vtwin.renderer import TwinRenderer

pytestmark = pytest.mark.gpu

W, H = 96, 64


@pytest.fixture(scope="module")
def rig():
    # thicker tools than the 6 mm instruments so that many (path, pose) pairs diverge at this small size
    sc = dome.make_dome_scene(seed=1, width=W, height=H, level=3, with_instruments=6, tool_radius=0.04)
    sc["cameras"] = dome.batched_cameras(seed=3, n=2, width=W, height=H)
    r = TwinRenderer.create(sc)
    yield r, sc
    r.destroy()


def poses(n, seed=11):
    return dome.batch_pose_array(dome.instrument_poses(n_poses=n, n_tools=6, seed=seed))


def per_pose(r, cams, P, spp, depth, seed, sensor=None, frame0=0):
    rad, raw = [], []
    for c in cams:
        rc, wc = [], []
        for q in range(len(P)):
            r.set_pose_array(P[q])
            r.renderCamera(c, spp=spp, lightSamples=1, seed=seed, mode=A.VT_SHADE_PATH, max_depth=depth)
            rc.append(r.readback(c, "linear").reshape(H, W, 4))
            if sensor is not None:
                r.expose(c, seed=seed, frame=frame0 + q, params=sensor)
                wc.append(r.readback(c, "raw").reshape(H, W))
        rad.append(np.stack(rc))
        raw.append(np.stack(wc) if wc else None)
    return rad, raw


def test_batch_equals_per_pose(rig):
    r, _ = rig
    P = poses(5)
    sens = sensor_mod.unit_radiance_sensor()
    out = r.render_batch([0, 1], P, spp=4, max_depth=4, seed=7, sensor=sens, frame0=3, radiance=True, use_graph=False)
    st = out["stats"]
    print("\nstats", st)
    assert st["vary_mask"] == 0b1111110            # the six tools vary, the lamps do not
    assert 0 < st["pair_paths"] < 5 * st["shared_paths"]
    rad, raw = per_pose(r, [0, 1], P, 4, 4, 7, sensor=sens, frame0=3)
    for c in range(2):
        np.testing.assert_array_equal(out["radiance"][c], rad[c])
        np.testing.assert_array_equal(out["raw"][c].astype(np.float32), raw[c])
    # the poses differ from one another where the tools are, so the shared paths alone would not pass
    assert not np.array_equal(rad[0][0], rad[0][1])


def test_graph_replay_and_new_poses(rig):
    r, _ = rig
    sens = sensor_mod.unit_radiance_sensor()
    a = r.render_batch([1, 0], poses(4, seed=21), spp=3, max_depth=3, seed=2, sensor=sens, radiance=True, use_graph=True)
    b = r.render_batch([1, 0], poses(4, seed=21), spp=3, max_depth=3, seed=2, sensor=sens, radiance=True, use_graph=True)
    assert b["stats"]["graph_replayed"]
    for c in range(2):
        np.testing.assert_array_equal(a["radiance"][c], b["radiance"][c])
        np.testing.assert_array_equal(a["raw"][c], b["raw"][c])
    # a new pose set with the same visible bodies replays the same graph with the new uniforms and cull tree
    P = poses(4, seed=99)
    c = r.render_batch([1, 0], P, spp=3, max_depth=3, seed=2, sensor=sens, radiance=True, use_graph=True)
    assert c["stats"]["graph_replayed"]
    rad, raw = per_pose(r, [1, 0], P, 3, 3, 2, sensor=sens)
    for k in range(2):
        np.testing.assert_array_equal(c["radiance"][k], rad[k])
        np.testing.assert_array_equal(c["raw"][k].astype(np.float32), raw[k])


def test_wave_and_tile_do_not_change_results(rig):
    r, _ = rig
    P = poses(3, seed=5)
    ref = r.render_batch([0], P, spp=4, max_depth=3, seed=1, radiance=True, use_graph=False)["radiance"][0]
    small = r.render_batch([0], P, spp=4, max_depth=3, seed=1, radiance=True, use_graph=False, wave_paths=4096)
    assert small["stats"]["waves"] > 1
    np.testing.assert_array_equal(small["radiance"][0], ref)
    best, table = r.autotune_batch([0], P, spp=4, max_depth=3, seed=1)
    print("\nautotune", best, len(table))
    assert len(table) >= 4 and best["wave_paths"] > 0   # waves larger than the frames repeat a plan and are skipped
    tuned = r.render_batch([0], P, spp=4, max_depth=3, seed=1, radiance=True, use_graph=False)["radiance"][0]
    np.testing.assert_array_equal(tuned, ref)


def test_hidden_tools_single_pose_and_blurred_sensor(rig):
    r, _ = rig
    P = poses(3, seed=8)
    P[1, 3, :] = np.nan                     # tool 2 hidden in pose 1
    sens = {**sensor_mod.unit_radiance_sensor(), "esfSigmaPx": 0.7}   # optics blur: sensor runs after the frames
    out = r.render_batch([0], P, spp=2, max_depth=3, seed=4, sensor=sens, radiance=True, use_graph=False)
    rad, raw = per_pose(r, [0], P, 2, 3, 4, sensor=sens)
    np.testing.assert_array_equal(out["radiance"][0], rad[0])
    np.testing.assert_array_equal(out["raw"][0].astype(np.float32), raw[0])
    one = r.render_batch([0], P[:1], spp=2, max_depth=3, seed=4, radiance=True, use_graph=False)
    assert one["stats"]["vary_mask"] == 0 and one["stats"]["pair_paths"] == 0
    np.testing.assert_array_equal(one["radiance"][0][0], rad[0][0])


def test_batch_errors(rig):
    r, _ = rig
    P = poses(2)
    moved = P.copy()
    moved[1, 0, 12] = 0.5                   # the lamps (emitter body) move in pose 1
    with pytest.raises(VtError):
        r.render_batch([0], moved, spp=1, max_depth=2)
    with pytest.raises(VtError):
        r.render_batch([0], poses(A.VT_BATCH_MAX_POSES + 1), spp=1, max_depth=2)
    with pytest.raises(VtError):
        r.render_batch([5], P, spp=1, max_depth=2)
