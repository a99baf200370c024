"""Differentiable calibration: the forward render against the FP64 oracle, the emitter transfer D against the
oracle, the path-replay + transposed-Jacobi gradient against central finite differences (h = 1e-4 relative) on the
GPU and against the FP64 oracle's finite differences, and the analytic KB4 reprojection Jacobian."""
import numpy as np
import pytest

import oracle as O
from vtwin import _abi as A
from vtwin import dome
from vtwin.renderer import TwinRenderer

pytestmark = pytest.mark.gpu

W, H = 96, 60


@pytest.fixture(scope="module")
def rig():
    sc = dome.make_dome_scene(seed=1, width=W, height=H, level=3)
    # the tracking cameras' poses and distortion, at the C0 camera's field of view (fx = 300 at 640 px): at this small
    # size the configs' fx would put the image edge past 90 degrees, where 8 float32 Newton steps of the KB4 inverse
    # (gpu/wgsl/lens.wgsl.js:24) and the FP64 oracle's part ways
    # a third camera at 320 x 200 for the FP64 check: with more samples the few sub-samples whose shadow decision
    # flips between float32 and float64 weigh less in the gradient. Its drawn distortion turns back (d theta_d /
    # d theta < 0) inside the image, where the KB4 inverse has no solution and Newton's steps diverge differently in
    # float32 and float64, so it takes the second camera's distortion.
    sc["cameras"] = dome.batched_cameras(seed=3, n=2, width=W, height=H) + dome.batched_cameras(seed=3, n=3, width=320, height=200)[2:]
    sc["cameras"][2]["k"] = list(sc["cameras"][1]["k"])
    for cam in sc["cameras"]:
        cam["fx"] = cam["fy"] = 300.0 * cam["size"][0] / 640.0
    r = TwinRenderer.create(sc)
    info = r.calib_setup(n_nodes=384, lamp_samples=8)
    truth_alb = np.array([m["rho"] for m in sc["materials"]], np.float64)
    truth_alb = np.clip(truth_alb, 0.05, 1.0)
    truth_lamp = np.full(info["n_lamps"], 50.0)
    rng = np.random.default_rng(7)
    truth_lamp *= 1.0 + 0.2 * (rng.random(info["n_lamps"]) - 0.5)
    _, targets = r.calib_forward([0, 1, 2], truth_alb, truth_lamp, spp=4, max_depth=3)
    yield r, sc, info, truth_alb, truth_lamp, targets
    r.destroy()


def f32(x):
    return np.asarray(x, np.float32).astype(np.float64)


def test_forward_matches_fp64_oracle(rig):
    r, sc, info, alb, lamp, _ = rig
    alb, lamp = f32(alb), f32(lamp)
    _, imgs = r.calib_forward([0, 1], alb, lamp, spp=4, max_depth=3)
    ex = r.calib_export(with_F=True)
    Hn, _ = O.calib_radiosity(ex["F"], ex["D"], lamp, alb, ex["node_mat"])
    S = O.Scene(sc)
    S.set_poses()
    for c in range(2):
        ref = S.calib_render(c, alb, lamp, Hn, ex["tri_node"], spp=4, depth=3, fp64=True, threads=8)
        got = imgs[c][..., :3].astype(np.float64)
        rel = np.abs(got - ref) / np.maximum(np.abs(ref), 1e-3 * np.abs(ref).max())
        print(f"\ncamera {c}: median rel {np.median(rel):.2e}, within 1e-4 {np.mean(rel <= 1e-4):.4f}, mean {got.mean():.5f} vs {ref.mean():.5f}")
        assert np.median(rel) <= 1e-5
        assert np.mean(rel <= 1e-4) >= 0.97
        assert abs(got.mean() - ref.mean()) <= 1e-4 * ref.mean()


def test_direct_transfer_matches_oracle(rig):
    r, sc, info, *_ = rig
    ex = r.calib_export()
    S = O.Scene(sc)
    S.set_poses()
    D = S.direct_transfer(ex["centres"], ex["normals"], samples=8, fp64=True, threads=8)
    rel = np.abs(ex["D"] - D) / max(D.max(), 1e-30)
    print(f"\nD: max |diff| / max D {rel.max():.2e}, entries {D.size}, nonzero {np.count_nonzero(D)}")
    assert np.count_nonzero(D) > 0.2 * D.size
    assert np.mean(rel <= 1e-5) >= 0.99
    assert abs(ex["D"].sum() - D.sum()) <= 1e-3 * D.sum()


def fd_grad(r, params, which, idx, targets, h=1e-4, **kw):
    """Central differences of the image loss in parameter (which, idx), FP64 loss reduction, with the denominator
    taken from the float32-rounded parameters the device sees."""
    alb, lamp = params
    vals = []
    for s in (+1, -1):
        a, l = alb.copy(), lamp.copy()
        if which == "albedo":
            a.flat[idx] = np.float32(a.flat[idx] * (1 + s * h))
            x = a.flat[idx]
        else:
            l[idx] = np.float32(l[idx] * (1 + s * h))
            x = l[idx]
        loss, _ = r.calib_forward([0, 1], a, l, targets=targets[:2], images=False, **kw)
        vals.append((loss, x))
    return (vals[0][0] - vals[1][0]) / (vals[0][1] - vals[1][1])


def test_adjoint_matches_central_differences(rig):
    """Central differences of the GPU's own loss (FP32 render, FP64 node radiosity and loss reduction). Every albedo
    reaches every pixel through the node radiosity, so each perturbation re-rounds every float32 pixel: the noise of a
    difference is ~1e-6 / h of the derivative's scale. h = 3e-3 balances it against the truncation error (the loss is
    a low-degree polynomial in each parameter); the FP64 check below uses h = 1e-4."""
    r, sc, info, t_alb, t_lamp, targets = rig
    rng = np.random.default_rng(3)
    alb = f32(np.clip(t_alb * (1 + 0.1 * (2 * rng.random(t_alb.shape) - 1)), 0.01, 1.0))
    lamp = f32(t_lamp * (1 + 0.1 * (2 * rng.random(t_lamp.shape) - 1)))
    kw = dict(spp=4, max_depth=3)
    r.calib_forward([0, 1], alb, lamp, targets=targets[:2], images=False, **kw)
    ga, gl = r.calib_backward()
    for name, g, ids in (("albedo", ga.ravel(), range(24)), ("lamp", gl, np.linspace(0, info["n_lamps"] - 1, 12).astype(int))):
        G = np.array([g[i] for i in ids])
        FD = np.array([fd_grad(r, (alb, lamp), name, int(i), targets, h=3e-3, **kw) for i in ids])
        vec = np.linalg.norm(G - FD) / np.linalg.norm(FD)
        comp = np.max(np.abs(G - FD) / np.maximum(np.abs(FD), 1e-2 * np.abs(FD).max()))
        print(f"\n{name}: {len(ids)} entries, vector relative error {vec:.2e}, worst entry {comp:.2e}")
        assert vec <= 1e-3 and comp <= 5e-3


def test_adjoint_matches_fp64_oracle_fd(rig):
    """The FP64 CPU reference gradient: central differences of the oracle's FP64 image loss (FP64 radiosity solve,
    FP64 estimator) on a 320 x 200 camera, against the GPU adjoint of the same loss."""
    r, sc, info, t_alb, t_lamp, targets = rig
    alb = f32(np.clip(t_alb * 1.07, 0.01, 1.0))
    lamp = f32(t_lamp * 0.93)
    kw = dict(spp=4, max_depth=3)
    r.calib_forward([2], alb, lamp, targets=[targets[2]], images=False, **kw)
    ga, gl = r.calib_backward()
    ex = r.calib_export(with_F=True)
    S = O.Scene(sc)
    S.set_poses()
    T2 = targets[2][..., :3].astype(np.float64)

    def loss64(a, l):
        Hn, _ = O.calib_radiosity(ex["F"], ex["D"], l, a, ex["node_mat"])
        img = S.calib_render(2, a, l, Hn, ex["tri_node"], spp=4, depth=3, fp64=True, threads=16)
        return np.mean((img - T2) ** 2)

    h = 1e-4
    cases = [("albedo", (m, m % 3)) for m in range(8)] + [("lamp", t) for t in (0, 5, 31, 60, 77, 95)]
    G, FD = [], []
    for which, idx in cases:
        a, l = alb.copy(), lamp.copy()
        if which == "albedo":
            x = a[idx]
            a[idx] = x * (1 + h); lp = loss64(a, l)
            a[idx] = x * (1 - h); lm = loss64(a, l)
            fd, g = (lp - lm) / (2 * h * x), ga[idx]
        else:
            x = l[idx]
            l[idx] = x * (1 + h); lp = loss64(a, l)
            l[idx] = x * (1 - h); lm = loss64(a, l)
            fd, g = (lp - lm) / (2 * h * x), gl[idx]
        err = abs(g - fd) / max(abs(fd), 1e-12)
        print(f"\n{which} {idx}: adjoint {g:.6e} FP64 FD {fd:.6e} rel {err:.1e}")
        G.append(g)
        FD.append(fd)
        assert err <= 3e-3
    G, FD = np.array(G), np.array(FD)
    # per group (albedo, lamp): the gradient vector's relative error (the float32 estimator and the FP64 oracle take
    # different shadow decisions on ~2% of sub-samples, which moves single small entries by ~1e-3)
    for sl in (slice(0, 8), slice(8, None)):
        vec = np.linalg.norm(G[sl] - FD[sl]) / np.linalg.norm(FD[sl])
        print(f"vector relative error {vec:.2e}")
        assert vec <= 1e-3


def test_image_intrinsics_gradient_matches_frozen_fp64_fd(rig):
    """The image loss's derivative in a camera's KB4 intrinsics (fx, fy, cx, cy, k1..k4) against FP64 central
    differences of the FP64 oracle's estimator replayed with the GPU's own discrete decisions frozen: every path's
    hit triangles and shadow outcomes are the GPU forward's (vt_calib_export_paths), so the oracle's image moves
    smoothly with K and its differences measure exactly the derivative the adjoint computes (the interior term; a ray
    crossing an edge is a step that is not differentiated). The steps are 1e-6 and 5e-7 relative (taken exactly
    between float32 lens values, as the device holds them): the frozen estimator keeps threshold tests of its own (a
    grazing view switching to the geometric normal, the emitter's cosine cut-off at its silhouette), and steps of
    1e-4 or 1e-5 (0.016 or 0.0016 px for cx) cross them on a handful of the 256k paths; at 1e-6 and 5e-7 none is
    crossed and the two agree. Then the same derivative from the replay form, and, for information, the ordinary FP64
    differences at 1e-4, which also see the edges."""
    r, sc, info, t_alb, t_lamp, targets = rig
    alb, lamp = f32(np.clip(t_alb * 1.03, 0.01, 1.0)), f32(t_lamp * 0.97)
    K_true = r.get_intrinsics(2)
    K0 = f32(K_true * np.array([1.02, 0.985, 1.0, 1.0, 1.1, 0.9, 1.2, 0.8]) + np.array([0, 0, 2.0, -1.5, 0.004, -0.003, 0, 0]))
    r.set_intrinsics(2, K0)
    kw = dict(spp=4, max_depth=3)
    try:
        loss_g, imgs = r.calib_forward([2], alb, lamp, targets=[targets[2]], intrinsics=True, **kw)
        r.calib_backward()
        gK = r.calib_intrinsics_grad()[0]
        frozen = r.calib_export_paths(0, spp=4)
        r.calib_forward([2], alb, lamp, targets=[targets[2]], images=False, intrinsics=True, replay=1, **kw)
        r.calib_backward()
        gK_replay = r.calib_intrinsics_grad()[0]
    finally:
        r.set_intrinsics(2, K_true)
    ex = r.calib_export(with_F=True)
    Hn, _ = O.calib_radiosity(ex["F"], ex["D"], lamp, alb, ex["node_mat"])
    S = O.Scene(sc)
    S.set_poses()
    T2 = targets[2][..., :3].astype(np.float64)

    def loss64(K, fz):
        img = S.calib_render(2, alb, lamp, Hn, ex["tri_node"], spp=4, depth=3, fp64=True, threads=16, frozen=fz, K=K)
        return np.mean((img - T2) ** 2)

    base = loss64(K0, frozen)

    def central(k, rel, fz):
        h = rel * max(abs(K0[k]), 1e-2)
        Kp, Km = K0.copy(), K0.copy()
        Kp[k], Km[k] = np.float32(K0[k] + h), np.float32(K0[k] - h)   # the device's float32 lens, steps taken exactly
        return (loss64(Kp, fz) - loss64(Km, fz)) / (Kp[k] - Km[k])

    FD = np.array([central(k, 1e-6, frozen) for k in range(8)])
    FD6 = np.array([central(k, 5e-7, frozen) for k in range(8)])
    FD_plain = np.array([central(k, 1e-4, None) for k in range(8)])
    names = ["fx", "fy", "cx", "cy", "k1", "k2", "k3", "k4"]
    for k in range(8):
        print(f"\n{names[k]}: adjoint {gK[k]: .6e}  frozen FP64 FD {FD[k]: .6e} ({FD6[k]: .6e})  replay form {gK_replay[k]: .6e}  "
              f"ordinary FD {FD_plain[k]: .6e}", end="")
    vec = np.linalg.norm(gK - FD) / np.linalg.norm(FD)
    steps = np.linalg.norm(FD6 - FD) / np.linalg.norm(FD)
    worst = np.max(np.abs(gK - FD) / np.abs(FD))
    vec_replay = np.linalg.norm(gK_replay - gK) / np.linalg.norm(gK)
    vec_plain = np.linalg.norm(gK - FD_plain) / np.linalg.norm(FD_plain)
    print(f"\nloss GPU {loss_g:.6e} / frozen FP64 {base:.6e}; vector relative error {vec:.2e} against the frozen FP64 "
          f"differences (worst entry {worst:.1e}; steps 1e-6 and 5e-7 agree to {steps:.1e}), {vec_replay:.1e} between the stored and "
          f"replay forms, {vec_plain:.2e} against the ordinary differences (edges included)")
    assert abs(base - loss_g) <= 1e-4 * loss_g
    assert steps <= 1e-4
    assert vec <= 1e-3 and worst <= 1e-2
    assert vec_replay <= 1e-4


def test_reprojection_jacobian(rig):
    r, sc, *_ = rig
    rng = np.random.default_rng(11)
    pts = dome.fib_hemisphere(200, 3.9)[0]
    K0 = [r.get_intrinsics(c) for c in (0, 1)]
    uv_t = np.zeros((2, 200, 2))
    for c in (0, 1):
        Kt = K0[c] * (1 + 0.01 * (rng.random(8) - 0.5))
        r.set_intrinsics(c, Kt)
        uv_t[c] = r.project(c, pts)
        r.set_intrinsics(c, K0[c])
    uv_t[0, ::3] = np.nan                   # unobserved pairs are skipped
    loss, g = r.reproj_loss([0, 1], pts, uv_t)
    assert loss > 0
    for c in (0, 1):
        for k in range(8):
            h = 1e-6 * max(1.0, abs(K0[c][k]))
            Kp, Km = K0[c].copy(), K0[c].copy()
            Kp[k] += h
            Km[k] -= h
            r.set_intrinsics(c, Kp)
            lp, _ = r.reproj_loss([0, 1], pts, uv_t)
            r.set_intrinsics(c, Km)
            lm, _ = r.reproj_loss([0, 1], pts, uv_t)
            r.set_intrinsics(c, K0[c])
            fd = (lp - lm) / (2 * h)
            assert abs(g[c, k] - fd) <= 1e-5 * max(abs(fd), 1e-3 * np.abs(g).max()), (c, k, g[c, k], fd)


def test_descent_recovers_parameters(rig):
    """A few Adam steps on albedo and lamp radiance from a 10% perturbation reduce the image loss by 10x."""
    r, sc, info, t_alb, t_lamp, targets = rig
    rng = np.random.default_rng(5)
    alb = np.clip(t_alb * (1 + 0.1 * (2 * rng.random(t_alb.shape) - 1)), 0.01, 1.0)
    lamp = t_lamp * (1 + 0.1 * (2 * rng.random(t_lamp.shape) - 1))
    x = np.concatenate([alb.ravel(), lamp / 50.0])
    m = np.zeros_like(x)
    v = np.zeros_like(x)
    first = None
    for it in range(1, 61):
        a = np.clip(x[:alb.size].reshape(alb.shape), 0.01, 1.0)
        l = np.maximum(x[alb.size:] * 50.0, 0.0)
        loss, _ = r.calib_forward([0, 1], a, l, targets=targets[:2], images=False, spp=4, max_depth=3)
        first = loss if first is None else first
        ga, gl = r.calib_backward()
        g = np.concatenate([ga.ravel(), gl * 50.0])
        m = 0.9 * m + 0.1 * g
        v = 0.999 * v + 0.001 * g * g
        x = x - 0.01 * (m / (1 - 0.9 ** it)) / (np.sqrt(v / (1 - 0.999 ** it)) + 1e-12)
    print(f"\nloss {first:.3e} -> {loss:.3e}")
    assert loss < 0.1 * first


def test_calibration_function_with_torch(rig):
    """The packed forward/backward pair as a torch.autograd.Function: Adam on albedo, lamp radiance and the KB4
    intrinsics (image loss + fiducial reprojection loss) from a 10% perturbation."""
    torch = pytest.importorskip("torch")
    from vtwin.calibrate import Calibration

    class CalibrationFunction(torch.autograd.Function):
        """Test adapter: the packed forward/backward pair as a torch.autograd.Function, so that a torch optimiser
        can drive it (loss = CalibrationFunction.apply(x, calibration), x float64)."""

        @staticmethod
        def forward(ctx, x, calib):
            ctx.calib = calib
            return torch.tensor(calib.forward(x.detach().cpu().numpy()), dtype=torch.float64)

        @staticmethod
        def backward(ctx, grad):
            return grad * torch.from_numpy(ctx.calib.backward()), None

    r, sc, info, t_alb, t_lamp, targets = rig
    pts = dome.fib_hemisphere(200, 3.9)[0]
    K_true = np.stack([r.get_intrinsics(c) for c in (0, 1)])
    uv_t = np.stack([np.where(r.observed(c, pts, margin=2.0)[:, None], r.project(c, pts), np.nan) for c in (0, 1)])
    cal = Calibration(r, [0, 1], targets[:2], fiducials=pts, uv_targets=uv_t, w_reproj=1e-3, spp=4, max_depth=3)
    x_true = cal.pack(t_alb, t_lamp, K_true)
    rng = np.random.default_rng(9)
    x0 = x_true * (1 + 0.1 * (2 * rng.random(x_true.shape) - 1))
    x0[:3 * info["n_materials"]] = np.clip(x0[:3 * info["n_materials"]], 0.01, 1.0)
    scale = np.maximum(np.abs(x_true), 1e-3)
    z = torch.tensor(x0 / scale, dtype=torch.float64, requires_grad=True)
    opt = torch.optim.Adam([z], lr=3e-3)
    first = None
    for it in range(80):
        opt.zero_grad()
        x = z * torch.from_numpy(scale)
        x = torch.cat([x[:3 * info["n_materials"]].clamp(0.01, 1.0), x[3 * info["n_materials"]:]])
        loss = CalibrationFunction.apply(x, cal)
        loss.backward()
        opt.step()
        first = float(loss.detach()) if first is None else first
    err_K = np.abs(z.detach().numpy()[-16:] * scale[-16:] - x_true[-16:]) / np.abs(x_true[-16:]).clip(1e-3)
    print(f"\nloss {first:.3e} -> {float(loss.detach()):.3e}; intrinsics max rel error {err_K.max():.2e} (start 1e-1)")
    assert float(loss.detach()) < 0.05 * first


@pytest.mark.parametrize("replay,retrace", [(True, False), (1, False), (3, False), (True, True), (3, True)])
def test_stored_and_replayed_paths_agree(rig, replay, retrace, monkeypatch):
    """The forward that keeps every path's record and the replay form, which traces the paths again in chunks of
    sub-samples (all 4 at once, 4 chunks of 1, chunks of 3 and 1) through the same wavefront kernels: the images and
    the loss are identical bit for bit (the per-pixel sums carry across chunks in sub-sample order), the gradients
    agree to the order of their FP64 accumulation. The replay backward re-shades from the forward's recorded hits
    and shadow outcomes, or (retrace, VT_CALIB_RETRACE=1) traces every path again."""
    if retrace:
        monkeypatch.setenv("VT_CALIB_RETRACE", "1")
    r, sc, info, t_alb, t_lamp, targets = rig
    alb = f32(np.clip(t_alb * 1.05, 0.01, 1.0))
    lamp = f32(t_lamp * 0.95)
    kw = dict(spp=4, max_depth=3, targets=targets[:2])
    l_s, im_s = r.calib_forward([0, 1], alb, lamp, replay=False, **kw)
    ga_s, gl_s = r.calib_backward()
    l_r, im_r = r.calib_forward([0, 1], alb, lamp, replay=replay, **kw)
    ga_r, gl_r = r.calib_backward()
    same = np.mean([np.mean(a == b) for a, b in zip(im_s, im_r)])
    print(f"\nstored vs replayed ({replay}): identical pixels {same:.5f}, loss {l_s:.12e} vs {l_r:.12e}")
    assert all(np.array_equal(a, b) for a, b in zip(im_s, im_r))
    assert l_s == l_r
    np.testing.assert_allclose(ga_s, ga_r, rtol=1e-9, atol=1e-12 * np.abs(ga_r).max())
    np.testing.assert_allclose(gl_s, gl_r, rtol=1e-9, atol=1e-12 * np.abs(gl_r).max())


def test_replayed_decisions_with_posed_bodies(monkeypatch):
    """The replay backward's recorded decisions on a scene with posed instrument bodies: an extension ray that met a
    body meets the recorded triangle again in the body's frame at the path's time.
    - Without the intrinsics' term, the stored form, the replay form from recorded decisions and the replay form
      tracing again give identical images and losses, and albedo and lamp gradients that agree to the order of
      their FP64 accumulation.
    - With it, the stored forward shades with the derivative-record kernel and the replay forward with the plain
      one, whose rays can differ in their last bits. The three forms' gradients, intrinsics included, then agree to
      1e-6."""
    sc = dome.make_dome_scene(seed=4, width=96, height=64, level=3, with_instruments=2)
    sc["cameras"] = dome.batched_cameras(seed=3, n=2, width=96, height=64)
    for cam in sc["cameras"]:
        cam["fx"] = cam["fy"] = 300.0 * cam["size"][0] / 640.0
    r = TwinRenderer.create(sc)
    try:
        T = dome.instrument_poses(n_poses=1, n_tools=2, seed=2)[0]
        r.set_pose_array(np.concatenate([A.identity_poses(1), T]))
        info = r.calib_setup(n_nodes=128, lamp_samples=4)
        alb = np.clip(np.array([m["rho"] for m in sc["materials"]], np.float64), 0.05, 1.0)
        lamp = np.full(info["n_lamps"], 50.0)
        kw = dict(spp=3, max_depth=3)
        _, tg = r.calib_forward([0, 1], alb, lamp, **kw)

        def run(intrinsics):
            out = {}
            for name, rp, rt in (("stored", False, "0"), ("decisions", True, "0"), ("retrace", 2, "1")):
                monkeypatch.setenv("VT_CALIB_RETRACE", rt)
                l, im = r.calib_forward([0, 1], f32(alb * 0.9), f32(lamp), targets=tg, replay=rp, intrinsics=intrinsics, **kw)
                ga, gl = r.calib_backward()
                out[name] = (l, im, ga, gl, r.calib_intrinsics_grad() if intrinsics else None)
            return out

        out = run(False)
        l_s, im_s, ga_s, gl_s, _ = out["stored"]
        assert np.abs(ga_s).max() > 0
        for name in ("decisions", "retrace"):
            l, im, ga, gl, _ = out[name]
            assert l == l_s and all(np.array_equal(a, b) for a, b in zip(im, im_s)), name
            np.testing.assert_allclose(ga, ga_s, rtol=1e-9, atol=1e-12 * np.abs(ga_s).max())
            np.testing.assert_allclose(gl, gl_s, rtol=1e-9, atol=1e-12 * np.abs(gl_s).max())
        out = run(True)
        ref = out["stored"]
        assert np.abs(ref[4]).max() > 0
        for name in ("decisions", "retrace"):
            errs = [np.linalg.norm(out[name][k] - ref[k]) / np.linalg.norm(ref[k]) for k in (2, 3, 4)]
            print(f"\nposed bodies, {name} vs stored with the intrinsics' term: albedo {errs[0]:.1e}, lamps {errs[1]:.1e}, "
                  f"intrinsics {errs[2]:.1e}")
            assert max(errs) < 1e-6, (name, errs)
    finally:
        monkeypatch.delenv("VT_CALIB_RETRACE", raising=False)
        r.destroy()
