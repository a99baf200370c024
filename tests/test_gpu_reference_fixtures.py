"""The GPU's first hits on the twin's own scene (its CAD meshes prepared by the scene loader, posed at the scene's
default_state) against the oracle's FP64 traversal of the same rays: the 1/4-resolution pixel centres of the three
tracking cameras, whose class shares tests/test_reference_data.py ties to the reference's preview statistics. Needs
the twin's scene files ($VT_REFERENCE, or ../reference beside this repository); skips without them."""
import numpy as np
import pytest

import oracle as O
from test_reference_data import CLASSES, HAVE_TWIN, _twin, ray_cast_classes

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not HAVE_TWIN, reason="the twin's scene files are not here")]


def test_gpu_first_hits_match_oracle_on_twin_scene():
    import twin_kinematics as TK
    from vtwin.renderer import TwinRenderer

    sj, meshes, sc = _twin()
    poses = TK.poses_from_state(sj, sj["default_state"])
    T0 = np.full((len(sc["bodies"]), 16), np.nan)
    for i, b in enumerate(sc["bodies"]):
        if b["key"] in poses:
            T0[i] = poses[b["key"]]
        elif b["kind"] == "fixed":
            T0[i] = np.eye(4).ravel()
    r = TwinRenderer.create(sc, nodes=False)
    r.set_pose_array(T0)
    S = O.Scene(sc)
    S.set_poses(T0)
    tris = S.arrays()["tris"]

    def gpu_trace(o4, d4):
        t, tri, inst, u, v = r.trace(o4, d4, mask=3)
        return np.stack([t, np.where(tri == 0xFFFFFFFF, -1, tri.astype(np.int64))], 1)

    for cam in sc["cameras"]:
        w, h = cam["size"][0] // 4, cam["size"][1] // 4
        g_cls, g_tri = ray_cast_classes(gpu_trace, tris, sj, sc, cam, w, h)
        o_cls, o_tri = ray_cast_classes(lambda o4, d4: S.trace(o4, d4, mask=3, fp64=True)[0], tris, sj, sc, cam, w, h)
        same_tri = np.mean(g_tri == o_tri)
        same_cls = np.mean(g_cls == o_cls)
        shares = "  ".join(f"{k} {100 * np.mean(g_cls == k):.3f}" for k in CLASSES)
        print(f"\n{cam['name']}: identical hit triangles {same_tri:.5f}, identical classes {same_cls:.5f}; GPU shares {shares}")
        assert same_tri >= 0.999 and same_cls >= 0.9995
    r.destroy()
