"""Test helper: the twin's state -> body poses (control/kinematics.js:226-251 posesFromState, with forward :106-118,
shaftRotation :101, scopeForward :143-151, cannulaT :255-257), restated to pose the twin's own scene at its
default_state for the checks against the reference's preview statistics. The library takes poses as matrices, as
the reference's renderer does (gpu/renderer.js:620 setPoses); kinematics are the control plane's, so this lives with
the tests.

Conventions (control/kinematics.js:1-18): frame D in metres; port frame P = scene.ports[].R_D_P; shaft frame
R_D_S = R_D_P Ry(yaw) Rx(pitch) Rz(roll); the jaw hinge at pivot + insertion z_S; jaw a = shaft Rx(-jaw/2), jaw b =
shaft Rx(+jaw/2) about the hinge; the scope's lens point at pivot + insertion z_K through its port (C); a cannula in
a port turns with the yaw and pitch of the tool in it, at the pivot. Poses are column-major 4x4 (p_D = T p_body).
"""
import numpy as np


def rot_x(a):
    c, s = np.cos(a), np.sin(a)
    return np.array([[1, 0, 0], [0, c, -s], [0, s, c]])


def rot_y(a):
    c, s = np.cos(a), np.sin(a)
    return np.array([[c, 0, s], [0, 1, 0], [-s, 0, c]])


def rot_z(a):
    c, s = np.cos(a), np.sin(a)
    return np.array([[c, -s, 0], [s, c, 0], [0, 0, 1]])


def make_T(R, t):
    """Column-major 4x4 (16 values) of rotation R and translation t."""
    M = np.eye(4)
    M[:3, :3] = R
    M[:3, 3] = t
    return M.T.ravel().copy()


def _port(scene, pid):
    p = next(q for q in scene["ports"] if q["id"] == pid)
    return np.array(p["pivot"], float), np.array(p["R_D_P"], float), p.get("cannula_body")


def _shaft_rotation(R_D_P, q):
    return R_D_P @ rot_y(q["yaw"]) @ rot_x(q["pitch"]) @ rot_z(q.get("roll", 0.0))


def poses_from_state(scene, state):
    """{body key: column-major 4x4} for the instruments (shaft, jaws), their cannulas, the scope and its cannula;
    boards without a pose are left out (hidden)."""
    bodies = {}
    for ins in scene.get("instruments") or []:
        q = next((s for s in state["instruments"] if s["id"] == ins["id"]), None)
        if q is None:
            continue
        pivot, R_D_P, cannula = _port(scene, ins["port"])
        R = _shaft_rotation(R_D_P, q)
        hinge = pivot + R[:, 2] * q["insertion"]
        h = np.array(ins.get("hinge_in_S") or [0.0, 0.0, 0.0])
        bodies[f"{ins['id']}/shaft"] = make_T(R, hinge - R @ h)
        bodies[f"{ins['id']}/jaw_a"] = make_T(R @ rot_x(-q["jaw"] / 2), hinge)
        bodies[f"{ins['id']}/jaw_b"] = make_T(R @ rot_x(q["jaw"] / 2), hinge)
        if cannula:
            bodies[cannula] = make_T(R_D_P @ rot_y(q["yaw"]) @ rot_x(q["pitch"]), pivot)
    sc, qs = scene.get("scope"), state.get("scope")
    if sc and qs:
        pivot, R_D_P, cannula = _port(scene, sc.get("port", "C"))
        R = _shaft_rotation(R_D_P, qs)
        bodies["scope"] = make_T(R, pivot + R[:, 2] * qs["insertion"])
        if cannula:
            bodies[cannula] = make_T(R_D_P @ rot_y(qs["yaw"]) @ rot_x(qs["pitch"]), pivot)
    return bodies
