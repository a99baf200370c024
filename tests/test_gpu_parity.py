"""The CUDA path against the oracle, through the C ABI (GB300).

Bit-exact: the packed scene (nodes, triangles, vertices, params, scene uniform), raw sensor DN.
Hit identity: primary-ray triangle ids against gpu/bvh.js's float64 traversal; any mismatch must be a t-tie
(two triangles within |dt| <= 1e-6 m, a shared edge) or a ray grazing an edge - counted and reported.
Float32 tolerance: radiance per pixel against the FP64 estimator with the GPU's own sample numbers
(tolerance 1e-4 relative per pixel for the bulk; whole-sample visibility flips at shadow and silhouette edges are
counted and bounded), radiosity against a direct FP64 solve.
"""
import numpy as np
import pytest

import oracle as O
from vtwin import _abi as A
from vtwin import dome
from vtwin import sensor as S
from vtwin.renderer import TwinRenderer, solve_radiosity, form_factors

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def inst_scene():
    return dome.make_dome_scene(seed=1, width=160, height=120, with_instruments=3)


@pytest.fixture(scope="module")
def inst_poses(inst_scene):
    T = dome.instrument_poses(n_poses=1, n_tools=3, seed=11)[0]
    return np.concatenate([A.identity_poses(1), T])


def test_scene_packing_bit_exact(inst_scene, inst_poses):
    r = TwinRenderer.create(inst_scene)
    ref = O.Scene(inst_scene)
    a, b = r.export(), ref.arrays()
    for k in ("nodes", "tris", "verts"):
        assert np.array_equal(a[k], b[k]), k
    assert np.array_equal(a["params"].view(np.uint32), b["params"].view(np.uint32))
    r.set_pose_array(inst_poses)
    ref.set_poses(inst_poses)
    assert np.array_equal(r.scene_uniform().view(np.uint32), ref.uniform().view(np.uint32))
    # a moving exposure (poses0 != poses1): swept boxes, padded capsules
    T1 = inst_poses.copy()
    T1[1:, 12:15] += 0.01
    r.set_pose_array(inst_poses, T1)
    ref.set_poses(inst_poses, T1)
    assert np.array_equal(r.scene_uniform().view(np.uint32), ref.uniform().view(np.uint32))
    r.destroy()


def _camera_rays(cam, step=1):
    """Primary rays through pixel centres, built on the host in float64 (gpu/lens.js:54) then rounded."""
    W, H = cam["size"]
    xs, ys = np.meshgrid(np.arange(0, W, step), np.arange(0, H, step))
    uv = np.stack([xs.ravel(), ys.ravel()], 1).astype(np.float64)
    rays = O.unproject(A.lens_params(cam), uv)
    T = np.asarray(cam["T_D_C"])
    d = rays @ T[:3, :3].T
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    o = np.tile(T[:3, 3], (len(d), 1))
    return o.astype(np.float32), d.astype(np.float32)


def test_primary_hit_ids_match_reference_traversal(dome_c0):
    r = TwinRenderer.create(dome_c0)
    ref = O.Scene(dome_c0)
    arr = ref.arrays()
    o, d = _camera_rays(dome_c0["cameras"][0])       # 640 x 480 = 307,200 primary rays
    o4 = np.concatenate([o, np.full((len(o), 1), 0.5, np.float32)], 1)
    d4 = np.concatenate([d, np.zeros((len(d), 1), np.float32)], 1)
    t, tri, inst, u, v = r.trace(o4, d4, mask=1)
    tj, uj, vj, kj = O.traverse_js(arr["nodes"], arr["tris"].view(np.float32), o, d)
    gpu = np.where(tri == A.VT_MISS, -1, tri.astype(np.int64))
    same = gpu == kj
    hit = kj >= 0
    tie = ~same & hit & (gpu >= 0) & (np.abs(t.astype(np.float64) - tj) <= 1e-6)
    other = ~same & ~tie
    print(f"\nprimary rays {len(o)}: identical ids {same.sum()}, t-ties {tie.sum()}, other {other.sum()}")
    assert same.mean() > 0.9995
    # whatever is not identical is a tie, or an edge ray where float32 and float64 disagree about the edge
    assert other.sum() <= max(5, int(2e-5 * len(o)))
    ok = same & hit
    assert np.abs(t[ok] - tj[ok]).max() <= 1e-5 * max(1.0, tj[ok].max())
    r.destroy()


def test_random_rays_with_posed_bodies(inst_scene, inst_poses):
    r = TwinRenderer.create(inst_scene)
    r.set_pose_array(inst_poses)
    ref = O.Scene(inst_scene)
    ref.set_poses(inst_poses)
    rng = np.random.default_rng(2)
    n = 20000
    # half the rays aimed at points on the instruments' axes (posed capsules, r = 6 mm), half scattered
    T = inst_poses[1:].reshape(-1, 4, 4).transpose(0, 2, 1)            # row-major body-to-dome
    k = rng.integers(0, len(T), n // 2)
    s = rng.uniform(0.0, 0.25, n // 2)
    on_axis = T[k, :3, 3] + T[k, :3, 2] * s[:, None] + rng.normal(0, 0.003, (n // 2, 3))
    tgt = np.concatenate([on_axis, rng.uniform([-3, -3, 0], [3, 3, 3], (n // 2, 3))])
    org = rng.uniform([-2.5, -2.5, 0.2], [2.5, 2.5, 3.0], (n, 3))
    d = tgt - org
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    o4 = np.concatenate([org, rng.uniform(0, 1, (n, 1))], 1).astype(np.float32)
    d4 = np.concatenate([d, np.zeros((n, 1))], 1).astype(np.float32)
    for any_hit in (False, True):
        t, tri, inst, _, _ = r.trace(o4, d4, mask=3, any_hit=any_hit)
        out, dbg = ref.trace(o4, d4, mask=3, any_hit=any_hit, fp64=False)
        k = np.where(tri == A.VT_MISS, -1, tri.astype(np.int64))
        kr = out[:, 1].astype(np.int64)
        if any_hit:
            assert ((k >= 0) == (kr >= 0)).mean() > 0.9999
        else:
            agree = (k == kr) | (np.abs(t - out[:, 0]) <= 1e-5)
            print(f"\nrandom rays {n}: id agreement {(k == kr).mean():.6f}; hits on posed bodies {(inst != A.VT_MISS).sum()}")
            assert agree.mean() > 0.9999 and (inst != A.VT_MISS).sum() > 500
    flags = r.debugFlags(reset=True)
    assert flags["traversalCap"] == 0 and flags["corruptTree"] == 0 and flags["leafCap"] == 0
    r.destroy()


def _render_pair(scene, poses, mode, depth, spp, nl, node_state=None, eavg=None, options=0):
    r = TwinRenderer.create(scene)
    ref = O.Scene(scene)
    r.set_pose_array(poses)
    ref.set_poses(poses)
    if node_state is not None:
        r.set_node_state(node_state, 1)
        ref.set_node_state(node_state, 1)
    if eavg is not None:
        r.set_eavg(eavg)
        ref.set_eavg(eavg)
    W, H = scene["cameras"][0]["size"]
    out = np.zeros((H, W, 4), np.float32)
    q = r.renderCamera(0, out=out, spp=spp, lightSamples=nl, seed=3, mode=mode, max_depth=depth, options=options)
    img64, _ = ref.render(q, fp64=True, threads=8)
    again = np.zeros_like(out)
    r.renderCamera(0, out=again, spp=spp, lightSamples=nl, seed=3, mode=mode, max_depth=depth, options=options)
    assert np.array_equal(out, again)      # a fixed seed renders identically (gpu/renderer.js:60-61)
    flags = r.debugFlags()
    r.destroy()
    return out, img64


def _radiance_stats(gpu, ref):
    """Per-pixel relative error (largest channel); over the pixels outside 1e-4 (whole sub-samples whose shadow or
    silhouette decision flips between float32 and float64) the mean signed error and its standard error, so that a
    bias hiding among them would show: flips that are rounding go both ways and average to zero."""
    g, f = gpu[..., :3].astype(np.float64), ref[..., :3]
    den = np.maximum(np.abs(f).max(-1), 1e-3 * max(1e-12, np.abs(f).max()))
    rel = np.abs(g - f).max(-1) / den
    out = rel > 1e-4
    signed = ((g - f).sum(-1) / (3.0 * den))[out]
    return {"within_1e-4": float((rel <= 1e-4).mean()), "median": float(np.median(rel)), "p99": float(np.quantile(rel, 0.99)),
            "mean_rel": float(abs(g.mean() / f.mean() - 1)), "alpha_same": float((gpu[..., 3] == ref[..., 3]).mean()),
            "outside": int(out.sum()), "outside_signed_mean": float(signed.mean()) if out.any() else 0.0,
            "outside_signed_sem": float(signed.std() / np.sqrt(max(1, out.sum()))) if out.any() else 0.0}


def _assert_unbiased(s):
    # the flipped pixels' signed errors average to zero within 4 standard errors
    assert abs(s["outside_signed_mean"]) <= 4.0 * s["outside_signed_sem"] + 1e-4, s


def test_twin_radiance_matches_fp64_oracle(inst_scene, inst_poses):
    n_nodes = len(inst_scene["static"]["P"])
    rng = np.random.default_rng(4)
    st = np.zeros((n_nodes, 16), np.float32)
    st[:, 0:3] = rng.uniform(0.5, 2.0, (n_nodes, 3))     # E_free
    st[:, 3] = 1.0
    st[:, 4:7] = rng.uniform(0.05, 0.3, (n_nodes, 3))    # Ls slot 1
    st[:, 7] = 1.0
    st[:, 15] = -1.0
    gpu, ref = _render_pair(inst_scene, inst_poses, A.VT_SHADE_TWIN, 2, 4, 2, node_state=st, eavg=[1.0, 1.1, 0.9])
    s = _radiance_stats(gpu, ref)
    print("\ntwin radiance vs FP64:", s)
    assert s["median"] < 1e-5 and s["within_1e-4"] > 0.97 and s["mean_rel"] < 1e-3 and s["alpha_same"] == 1.0
    _assert_unbiased(s)


def test_path_radiance_matches_fp64_oracle(dome_small):
    gpu, ref = _render_pair(dome_small, A.identity_poses(1), A.VT_SHADE_PATH, 4, 4, 1)
    s = _radiance_stats(gpu, ref)
    print("\npath (depth 4) radiance vs FP64:", s)
    assert s["median"] < 1e-5 and s["within_1e-4"] > 0.9 and s["mean_rel"] < 2e-3 and s["alpha_same"] == 1.0
    _assert_unbiased(s)


def test_refinement_pass(inst_scene, inst_poses):
    """gpu/wgsl/kernels.wgsl.js:218 camRefine: every pixel is bit-exactly its spp render or its spp + refine render
    (the same sub-samples summed in the same order); the refined set and the image agree with the FP64 oracle."""
    r = TwinRenderer.create(inst_scene)
    ref = O.Scene(inst_scene)
    r.set_pose_array(inst_poses)
    ref.set_poses(inst_poses)
    W, H = inst_scene["cameras"][0]["size"]

    def render(refineShadows=False, **o):
        out = np.zeros((H, W, 4), np.float32)
        q = r.renderCamera(0, out=out, lightSamples=2, seed=3, refineShadows=refineShadows, **o)
        return out, q

    a, _ = render(spp=2)
    b, _ = render(spp=5)
    r.debugFlags(reset=True)
    c, q = render(spp=2, refine=3, refineLightSamples=2)
    f = r.debugFlags(reset=True)
    # the first twin render brought the node radiosity up to the poses: the oracle shades with the same node state
    st, slot = r.get_node_state()
    ref.set_node_state(st, slot)
    ref.set_eavg(r.scene_uniform()[8:11])
    same_a = np.all(c == a, -1)
    same_b = np.all(c[..., :3] == b[..., :3], -1) & (c[..., 3] == 1.0)
    assert np.all(same_a | same_b)
    assert int((same_b & ~same_a).sum()) <= f["refined"] <= int(same_b.sum())
    assert 0 < f["refined"] < W * H and f["refinedBody"] > 0
    img64, dbg = ref.render(q, fp64=True, threads=8)
    s = _radiance_stats(c, img64)
    print("\nrefinement: gpu refined", f, "oracle refined", dbg[2:6], s)
    assert abs(f["refined"] - int(dbg[2])) <= 0.01 * int(dbg[2]) + 4
    assert s["median"] < 1e-5 and s["within_1e-4"] > 0.95 and s["mean_rel"] < 1e-3
    # one light sample per refinement sub-sample (the reference's default): the same pixels refined
    d, _ = render(spp=2, refine=3, refineLightSamples=1)
    g = r.debugFlags(reset=True)
    assert g["refined"] == f["refined"] and np.all(np.isfinite(d))
    known_plain = same_a & ~same_b
    assert np.all(d[known_plain] == a[known_plain])
    # shadow-traced pixels too
    render(spp=2, refine=3, refineLightSamples=1, refineShadows=True)
    assert r.debugFlags(reset=True)["refined"] > f["refined"]
    r.destroy()


def test_static_first_hit_cache_is_exact(inst_scene, inst_poses):
    """gpu/renderer.js:941-956 hitCache and shadowCache: a twin camera's static first hits and their static occlusion
    are traced once and kept; renders that read them (the instruments moved in between) equal renders without the
    caches bit for bit (refinement included, with the refinement's shadow criterion off: the caches change which
    pixels it picks, as they do in the reference)."""
    r = TwinRenderer.create(inst_scene)
    W, H = inst_scene["cameras"][0]["size"]
    T = dome.instrument_poses(n_poses=3, n_tools=3, seed=5)

    def render(cache):
        out = np.zeros((H, W, 4), np.float32)
        r.renderCamera(0, out=out, spp=2, lightSamples=2, seed=3, refine=2, refineShadows=False, hitCache=cache)
        return out

    for k in range(3):                     # k = 0 fills the cache, k = 1, 2 read it
        # one pose change per k (a pose change also brings the node radiosity along, so both renders follow it)
        r.set_pose_array(np.concatenate([A.identity_poses(1), T[k]]))
        a = render(True)
        b = render(False)
        assert np.array_equal(a, b), (k, (a != b).sum())
    # a new seed changes the key: the cache is traced again, and still exact
    r.set_pose_array(np.concatenate([A.identity_poses(1), T[0]]))
    a = np.zeros((H, W, 4), np.float32)
    b = np.zeros_like(a)
    r.renderCamera(0, out=a, spp=2, lightSamples=2, seed=4, hitCache=True)
    r.renderCamera(0, out=b, spp=2, lightSamples=2, seed=4, hitCache=False)
    assert np.array_equal(a, b)
    r.destroy()


def test_shadow_cache_refinement_matches_oracle(inst_scene, inst_poses):
    """With the static-occlusion cache the refinement's shadow criterion is the reference's cached one (a posed body
    blocks a sample, a penumbra, light samples more than 20 % apart): the refined pixels and the image against the
    FP64 oracle restating that branch, on the frame that fills the caches and on one that reads them."""
    r = TwinRenderer.create(inst_scene)
    ref = O.Scene(inst_scene)
    W, H = inst_scene["cameras"][0]["size"]
    T = dome.instrument_poses(n_poses=2, n_tools=3, seed=5)
    for k in range(2):
        P = np.concatenate([A.identity_poses(1), T[k]])
        r.set_pose_array(P)
        ref.set_poses(P)
        r.debugFlags(reset=True)
        out = np.zeros((H, W, 4), np.float32)
        q = r.renderCamera(0, out=out, spp=2, lightSamples=3, seed=3, refine=3, refineLightSamples=3, refineShadows=True)
        f = r.debugFlags(reset=True)
        assert q.options & A.OPTION_BITS["SHADOW_CACHE"]
        st, slot = r.get_node_state()
        ref.set_node_state(st, slot)
        ref.set_eavg(r.scene_uniform()[8:11])
        img64, dbg = ref.render(q, fp64=True, threads=8)
        s = _radiance_stats(out, img64)
        print(f"\nshadow cache, frame {k}: refined gpu {f['refined']} (shadow {f['refinedShadow']}) oracle {int(dbg[2])} ({int(dbg[4])}); {s}")
        assert abs(f["refined"] - int(dbg[2])) <= 0.01 * int(dbg[2]) + 6
        assert s["median"] < 1e-5 and s["within_1e-4"] > 0.95
    r.destroy()


def test_sensor_expose_bit_exact():
    W, H = 320, 240
    rng = np.random.default_rng(8)
    E = np.zeros((H, W, 4), np.float32)
    E[..., :3] = rng.gamma(2.0, 8.0, (H, W, 3)).astype(np.float32)
    E[: H // 4] *= 20.0
    for p, seed in ((S.unit_radiance_sensor(), 5), (S.sensor_params({"cfa": "GRBG", "esfSigmaPx": 0.7, "fullWell": 150.0}), 6)):
        su = S.pack_sensor_uniform(p, W, H, seed=seed, frame=2, cam_index=1, exposure=1.0 if p["conversionGain"] == 1.0 else 3e-7)
        ref = O.sensor_expose(su, E)
        r = TwinRenderer.create(dome.make_dome_scene(seed=1, width=32, height=24, level=1))
        sw = A.vt_sensor_uniform()
        sw.words[:] = [int(x) for x in su]
        raw = np.zeros((H, W), np.float32)
        import ctypes as C
        st = r.lib.vt_sensor_expose(r._ctx, C.byref(sw), E.ctypes.data_as(C.c_void_p), raw.ctypes.data_as(C.c_void_p))
        assert st == 0
        assert np.array_equal(raw, ref), (np.abs(raw - ref).max(), (raw != ref).sum())
        r.destroy()


def test_radiosity_fp32_matches_direct_fp64_solve():
    P = dome.dome_patches(1024, seed=2)
    F = O.form_factors(P["centres"], P["normals"], P["areas"])
    Fg = form_factors(P["centres"], P["normals"], P["areas"])
    assert np.abs(Fg - F).max() <= 1e-6 * max(1e-30, F.max()) + 1e-12
    for R in (1, 8):
        E = dome.radiosity_rhs(1024, P["lamps"], R)
        Bd = O.solve_dense(F, P["rho"], E)
        B, info = solve_radiosity(F, P["rho"], E, tol=1e-6, max_iters=2000)
        err = np.linalg.norm(B - Bd) / np.linalg.norm(Bd)
        print(f"\nradiosity FP32 R={R}: iters {info['iters']} residual {info['residual']:.2e} rel err vs FP64 {err:.2e}")
        assert info["status"] == 0 and err < 1e-5
    # the bulk-copy (TMA) fed matvec: one right-hand side, n % 4 == 0
    E = dome.radiosity_rhs(1024, P["lamps"], 1)
    Bd = O.solve_dense(F, P["rho"], E)
    B, info = solve_radiosity(F, P["rho"], E, precision=A.VT_PREC_FP32_TMA, tol=1e-6, max_iters=2000)
    err = np.linalg.norm(B - Bd) / np.linalg.norm(Bd)
    print(f"radiosity FP32 (bulk-copy matvec): iters {info['iters']} rel err vs FP64 {err:.2e}")
    assert info["status"] == 0 and err < 1e-5
    from vtwin._lib import VtError
    with pytest.raises(VtError):
        solve_radiosity(F, P["rho"], dome.radiosity_rhs(1024, P["lamps"], 8), precision=A.VT_PREC_FP32_TMA)


def test_errors_are_reported(dome_small):
    r = TwinRenderer.create(dome_small)
    from vtwin._lib import VtError
    with pytest.raises(VtError) as e:
        r.renderCamera(5)
    assert e.value.status == A.VT_ERR_UNKNOWN_CAMERA
    with pytest.raises(VtError) as e:
        r.readback(0, "raw")
    assert e.value.status == A.VT_ERR_STATE
    r.destroy()


def test_visible_and_project(dome_small):
    r = TwinRenderer.create(dome_small)
    cam = dome_small["cameras"][0]
    rng = np.random.default_rng(9)
    pts = np.concatenate([rng.uniform([-1, -0.4, 0.9], [1, 0.4, 0.9], (200, 3)),       # table top: visible
                          rng.uniform([-0.9, -0.3, 0.1], [0.9, 0.3, 0.8], (200, 3))])   # inside the table: hidden
    vis = r.visible(0, pts, tol=2e-4)
    assert vis[:200].mean() > 0.95 and vis[200:].sum() == 0
    uv = r.project(0, pts)
    T = np.asarray(cam["T_D_C"])
    Xc = (pts - T[:3, 3]) @ T[:3, :3]
    assert np.abs(uv - O.project(A.lens_params(cam), Xc)).max() < 1e-9
    r.destroy()
