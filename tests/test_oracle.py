"""The oracle pinned against the reference's known answers (CPU only).

Golden vectors from the reference's own configuration (tests/golden/physics_kat.json, made by make_golden.py),
and the known-answer methods the reference's source states: brute force checks the BVH (gpu/bvh.js:3),
the KB4 round trip (gpu/lens.js:43-62), the Gauss-Legendre disc irradiance (gpu/shade_ref.js:40-62), the
furnace (tools/gpu_bench.py:7), reciprocity, and the direct FP64 solve of the radiosity.
"""
import json
import math
import os

import numpy as np
import pytest

import oracle as O
from vtwin import dome

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "physics_kat.json")))


def test_fresnel_average_matches_reference_config():
    # physics.yaml lists fresnel_avg "derived from ior" for 12 materials, rounded to 4 decimals
    for p in GOLD["fresnel_avg"]:
        assert round(O.fresnel_average(p["ior"]), 4) == pytest.approx(p["fresnel_avg"], abs=1e-12), p


def test_profile_projected_solid_angle_matches_reference_config():
    pr = GOLD["profile"]
    th, pp = np.radians(pr["theta_deg"]), np.array(pr["p"], float)
    x = np.linspace(0.0, math.pi / 2, 4001)
    y = np.array([O.profile(t, th, pp) for t in x])
    psa = 2 * math.pi * np.trapezoid(y * np.cos(x) * np.sin(x), x)
    assert psa == pytest.approx(pr["projected_solid_angle"], abs=2e-6)
    # p = 0 past the last knot, p(last) exactly at it (gpu/shade_ref.js:7)
    assert O.profile(th[-1] + 1e-9, th, pp) == 0.0 and O.profile(th[-1], th, pp) == pp[-1]


def test_mulberry32_two_restatements_agree():
    a = O.mulberry32(12345, 1000)
    g = dome.mulberry32(12345)
    b = np.array([g() for _ in range(1000)])
    assert np.array_equal(a, b)
    assert (a >= 0).all() and (a < 1).all() and abs(a.mean() - 0.5) < 0.03


def test_kb4_round_trip():
    lens = np.array([300.0, 301.0, 319.5, 239.5, 0.001, 0.05, -0.01, 0.002, -0.0003])
    rng = np.random.default_rng(0)
    uv = np.stack([rng.uniform(-0.5, 639.5, 500), rng.uniform(-0.5, 479.5, 500)], 1)
    rays = O.unproject(lens, uv)
    assert np.allclose(np.linalg.norm(rays, axis=1), 1.0, atol=1e-12)
    back = O.project(lens, rays * 2.5)
    assert np.abs(back - uv).max() < 1e-9
    # the principal point maps to the optical axis
    assert np.allclose(O.unproject(lens, [[319.5, 239.5]]), [[0, 0, 1]])


def test_disc_irradiance_on_axis_closed_form():
    # a point on the axis of a Lambertian disc (radius a, distance d), normal facing it: E = pi L a^2 / (a^2 + d^2)
    for a, d in [(0.1, 0.5), (0.3, 0.2), (1.0, 1.0)]:
        E = O.disc_irradiance([0, 0, 0], [0, 0, 1], [0, 0, d], [0, 0, -1], a, 2.0)
        assert E == pytest.approx(math.pi * 2.0 * a * a / (a * a + d * d), rel=1e-9)


def _cylinder_occ_quadrature(p, n, a, b, r, m=20000):
    # the thin-cylinder integral the closed form evaluates: (1/pi) int (2r/h) cos(phi) max(0, n.omega(phi)) dphi
    ab = np.subtract(b, a)
    L = np.linalg.norm(ab)
    e = ab / L
    ap = np.subtract(p, a)
    s0 = ap @ e
    perp = ap - s0 * e
    h = math.sqrt(perp @ perp + r * r)
    ep = -perp / max(np.linalg.norm(perp), 1e-12)
    f1, f2 = math.atan(-s0 / h), math.atan((L - s0) / h)
    phi = np.linspace(f1, f2, m)
    om = np.cos(phi)[:, None] * ep + np.sin(phi)[:, None] * e
    g = np.cos(phi) * np.maximum(0.0, om @ n)
    return min(1.0, max(0.0, (2 * r / h) * np.trapezoid(g, phi) / math.pi))


def test_capsule_occlusion_matches_quadrature():
    rng = np.random.default_rng(3)
    for _ in range(40):
        p = rng.normal(size=3) * 0.05
        n = rng.normal(size=3)
        n /= np.linalg.norm(n)
        a, b = rng.normal(size=3) * 0.1, rng.normal(size=3) * 0.1
        r = rng.uniform(0.001, 0.01)
        assert O.capsule_occ(p, n, a, b, r) == pytest.approx(_cylinder_occ_quadrature(p, n, a, b, r), abs=2e-5)


def test_bsdf_reciprocity_and_sampling_pdf():
    mats = [dome.lambertian("l", [0.6, 0.4, 0.2]),
            {**dome.lambertian("d", [0.6, 0.4, 0.2]), "ior": 1.5, "roughness": 0.3},
            {**dome.lambertian("m", [0, 0, 0]), "metallic": 1, "f0": [0.9, 0.6, 0.3], "roughness": 0.4},
            {**dome.lambertian("c", [0, 0, 0]), "coated": 1, "f0": [0.56, 0.57, 0.58], "roughness": 0.3,
             "coat_ior": 1.5, "coat_roughness": 0.1, "tau": [0.9, 0.8, 0.7]}]
    rng = np.random.default_rng(5)
    for m in mats:
        cases = []
        for _ in range(200):
            n = np.array([0, 0, 1.0])
            l, v = rng.normal(size=3), rng.normal(size=3)
            l[2], v[2] = abs(l[2]), abs(v[2])
            cases.append(np.concatenate([n, l / np.linalg.norm(l), v / np.linalg.norm(v), rng.uniform(size=3)]))
        cases = np.array(cases)
        f_lv = O.bsdf_eval(m, cases)
        swapped = cases.copy()
        swapped[:, 3:6], swapped[:, 6:9] = cases[:, 6:9], cases[:, 3:6]
        f_vl = O.bsdf_eval(m, swapped)
        assert np.allclose(f_lv[:, :3], f_vl[:, :3], rtol=1e-10, atol=1e-14)  # reciprocity
        # a sampled direction's pdf is pdfBSDF at that direction
        ok = f_lv[:, 7] > 0
        again = cases[ok].copy()
        again[:, 3:6] = f_lv[ok, 4:7]
        assert np.allclose(O.bsdf_eval(m, again)[:, 3], f_lv[ok, 7], rtol=1e-9)


def test_albedo_table_furnace():
    # Lambertian with ior 1: spec = 0, diffuse = rho in every bin, hemispherical albedo = rho (no energy lost)
    t = O.albedo_table(dome.lambertian("l", [0.3, 0.5, 0.7]))
    assert np.abs(t["spec"]).max() < 1e-15
    assert np.allclose(t["diff"], [0.3, 0.5, 0.7]) and np.allclose(t["hh"], [0.3, 0.5, 0.7])
    # a white conductor never creates energy, and near normal incidence at low roughness keeps almost all of it
    c = O.albedo_table({**dome.lambertian("m", [0, 0, 0]), "metallic": 1, "f0": [1, 1, 1], "roughness": 0.1})
    assert c["spec"].max() <= 1.0 + 1e-9 and c["spec"][-1].min() > 0.98


def test_bvh_traverse_equals_brute_force(dome_small):
    st = dome_small["static"]
    b = O.bvh_build(st["P"], st["I"])
    T = O.pack_triangles(st["P"], st["I"], b["order"])
    rng = np.random.default_rng(7)
    n = 3000
    o = rng.uniform([-3, -3, 0.05], [3, 3, 3.5], (n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    t1, _, _, k1 = O.traverse_js(b["nodes"], T, o, d)
    t2, _, _, k2 = O.brute_force(T, len(st["I"]), o, d)
    same = k1 == k2
    # a tie is two triangles at the same t (shared edges): brute force keeps the first in slot order
    assert (same | (np.abs(t1 - t2) <= 1e-9)).all()
    assert np.array_equal(t1, t2)
    # any-hit finds a hit exactly when closest-hit does
    ta, _, _, ka = O.traverse_js(b["nodes"], T, o, d, any_hit=True)
    assert np.array_equal(ka >= 0, k1 >= 0)


def test_bvh_structure(dome_small):
    st = dome_small["static"]
    b = O.bvh_build(st["P"], st["I"])
    W = b["nodes"].reshape(-1, 16)
    F = W.view(np.float32)
    seen = np.zeros(len(st["I"]), int)
    for i, w in enumerate(W):
        for c in (0, 1):
            ref, cnt = w[8 * c + 3], w[8 * c + 7]
            if cnt == 0:
                assert ref > i  # children after the parent (gpu/wgsl/trace.wgsl.js:99)
            else:
                seen[ref:ref + cnt] += 1
                lo, hi = F[i, 8 * c:8 * c + 3], F[i, 8 * c + 4:8 * c + 7]
                tri = st["P"][st["I"][b["order"][ref:ref + cnt]]].reshape(-1, 3)
                assert (tri >= lo).all() and (tri <= hi).all()
    assert (seen == 1).all()  # every triangle in exactly one leaf
    assert sorted(b["order"]) == list(range(len(st["I"])))


def test_bvh_edge_cases():
    P = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], np.float32)
    one = O.bvh_build(P, np.array([[0, 1, 2]], np.uint32))
    W = one["nodes"].reshape(-1, 16)
    assert one["node_count"] == 1 and W[0, 7] == 1 and W[0, 15] == 1   # a single triangle: both children the same leaf
    zero = O.bvh_build(np.zeros((0, 3), np.float32), np.zeros((0, 3), np.uint32))
    assert zero["node_count"] == 1 and zero["nodes"].view(np.float32)[0] == np.float32(1e30)
    # many triangles with one centroid: split in the middle when too big for a leaf (gpu/bvh.js:101-104)
    I = np.tile(np.array([[0, 1, 2]], np.uint32), (40, 1))
    same = O.bvh_build(P, I)
    W = same["nodes"].reshape(-1, 16)
    assert same["node_count"] > 1 and (W[:, [7, 15]] <= 16).all()


def test_sensor_math_accuracy():
    x = np.linspace(1e-7, 1.0, 20001, dtype=np.float32)
    assert np.max(np.abs(O.vt_math("logf", x) - np.log(x.astype(np.float64))) / np.maximum(1e-30, np.abs(np.log(x.astype(np.float64))))) < 2e-6
    y = np.linspace(-80.0, 0.0, 20001, dtype=np.float32)
    assert np.max(np.abs(O.vt_math("expf", y) - np.exp(y.astype(np.float64))) / np.exp(y.astype(np.float64))) < 1e-6
    u = np.linspace(0.0, 1.0, 20001, dtype=np.float32)
    assert np.max(np.abs(O.vt_math("cos2pi", u) - np.cos(2 * np.pi * u.astype(np.float64)))) < 1e-6


def test_sensor_expose_statistics():
    from vtwin import sensor as S

    W, H = 256, 256
    p = S.unit_radiance_sensor()
    su = S.pack_sensor_uniform(p, W, H, seed=9)
    E = np.zeros((H, W, 4), np.float32)
    E[..., :3] = 25.0  # 100 e- per pixel: the normal branch; and a dim half in the inversion branch
    E[H // 2:, :, :3] = 2.5
    raw = O.sensor_expose(su, E)
    hi, lo = raw[: H // 2], raw[H // 2:]
    assert abs(hi.mean() - 100.0) < 0.5 and abs(hi.var() - (100.0 + 4.0)) < 6.0
    assert abs(lo.mean() - 10.0) < 0.2 and abs(lo.var() - (10.0 + 4.0)) < 1.2
    assert np.array_equal(raw, O.sensor_expose(su, E))   # deterministic per seed / frame / camera
    su2 = S.pack_sensor_uniform(p, W, H, seed=10)
    assert not np.array_equal(raw, O.sensor_expose(su2, E))


def test_radiosity_direct_and_jacobi_agree():
    P = dome.dome_patches(300, seed=2)
    F = O.form_factors(P["centres"], P["normals"], P["areas"])
    assert (F >= 0).all() and F.sum(1).max() <= 1 + 1e-6 and np.all(np.diag(F) == 0)
    E = dome.radiosity_rhs(300, P["lamps"], 4)
    Bd = O.solve_dense(F, P["rho"], E)
    Bj, it = O.jacobi64(F, P["rho"], E, tol=1e-13, max_it=5000, threads=2)
    assert np.abs(Bj - Bd).max() / np.abs(Bd).max() < 1e-11
    # the solution satisfies B = E + rho F B
    r = E + P["rho"][:, None] * (F.astype(np.float64) @ Bd) - Bd
    assert np.abs(r).max() < 1e-9 * np.abs(Bd).max()


def test_form_factor_reciprocity_before_scaling():
    P = dome.dome_patches(200, seed=4)
    F = O.form_factors(P["centres"], P["normals"], P["areas"]).astype(np.float64)
    s = F.sum(1)
    unscaled = np.where(s[:, None] > 1, F * s[:, None], F)   # undo the row scaling
    A = P["areas"].astype(np.float64)
    lhs, rhs = A[:, None] * unscaled, (A[:, None] * unscaled).T
    # the disk approximation is reciprocal up to its A_j in the denominator
    big = lhs > 1e-6
    assert np.median(np.abs(lhs[big] - rhs[big]) / lhs[big]) < 0.05


def test_calibration_estimator_is_linear_in_emission():
    """The calibration estimator is linear in the emitter radiances jointly with the node irradiance H (and exactly
    so when both double), and polynomial in the albedos: the FP64 restatement checked on a 24 x 16 view."""
    sc = dome.make_dome_scene(seed=1, width=24, height=16, level=2)
    S = O.Scene(sc)
    S.set_poses()
    n_static = len(sc["static"]["I"])
    n_nodes = 64
    tri_node = (np.arange(n_static, dtype=np.uint64) * n_nodes // n_static).astype(np.uint32)
    alb = np.clip(np.array([m["rho"] for m in sc["materials"]], np.float64), 0.05, 1.0)
    lamp = np.full(S.emit_n, 50.0)
    rng = np.random.default_rng(1)
    Hn = rng.random((3, n_nodes)) * 5.0
    a = S.calib_render(0, alb, lamp, Hn, tri_node, spp=2, depth=3)
    b = S.calib_render(0, alb, 2 * lamp, 2 * Hn, tri_node, spp=2, depth=3)
    assert a.max() > 0 and np.array_equal(b, 2 * a)
    # emission and node light add: I(L, H) = I(L, 0) + I(0, H)
    c = S.calib_render(0, alb, lamp, 0 * Hn, tri_node, spp=2, depth=3)
    d = S.calib_render(0, alb, 0 * lamp, Hn, tri_node, spp=2, depth=3)
    np.testing.assert_allclose(a, c + d, rtol=1e-12, atol=1e-12)
    # depth 1 sees no albedo of its own vertex beyond the first factor: doubling every albedo at most doubles
    e = S.calib_render(0, np.minimum(alb * 2, 1.0), lamp, 0 * Hn, tri_node, spp=2, depth=1)
    f = S.calib_render(0, alb, lamp, 0 * Hn, tri_node, spp=2, depth=1)
    assert np.all(e <= 2 * f + 1e-12)


def _refine_req(spp, nl, refine, refine_nl, options=0):
    from vtwin import _abi as A

    q = A.vt_render_req(camera=0, spp=spp, light_samples=nl, seed=3, options=options, mode=A.VT_SHADE_TWIN, max_depth=2,
                        root=0, frame=0, refine=refine, refine_light_samples=refine_nl)
    q.shutter[:] = [0.0, 1.0]
    q.scale = 1.0
    return q


def test_refinement_pass_continues_the_sub_sample_sequences():
    """gpu/wgsl/kernels.wgsl.js:218 camRefine restated: a refined pixel is its (spp + refine)-sample value, exactly
    (the same sub-samples summed in the same order), every other pixel its spp-sample value; refined pixels are edges
    in the 3x3 neighbourhood, posed bodies and (VT_O_REFINE_SHADOW) pixels whose shadow rays were traced."""
    from vtwin import _abi as A

    sc = dome.make_dome_scene(seed=1, width=40, height=30, level=2, with_instruments=2)
    S = O.Scene(sc)
    T = dome.instrument_poses(n_poses=1, n_tools=2, seed=11)[0]
    S.set_poses(np.concatenate([A.identity_poses(1), T]))
    a, _ = S.render(_refine_req(2, 2, 0, 0), threads=8)
    b, _ = S.render(_refine_req(5, 2, 0, 0), threads=8)
    c, dbg = S.render(_refine_req(2, 2, 3, 2), threads=8)
    same_a = np.all(c == a, -1)
    same_b = np.all(c[..., :3] == b[..., :3], -1) & (c[..., 3] == 1.0)
    assert np.all(same_a | same_b)
    refined = int(dbg[2])
    assert int((same_b & ~same_a).sum()) <= refined <= int(same_b.sum())
    assert 0 < refined < c.shape[0] * c.shape[1]
    assert dbg[3] > 0                      # posed bodies in view
    # a region renders as the same pixels of the whole image (the neighbourhood test reads one pixel beyond it)
    part, _ = S.render(_refine_req(2, 2, 3, 2), y0=7, y1=19, x0=5, x1=31, threads=4)
    assert np.array_equal(part, c[7:19, 5:31])
    # shadow-traced pixels join the refinement with VT_O_REFINE_SHADOW
    d, dbg2 = S.render(_refine_req(2, 2, 3, 2, options=A.OPTION_BITS["REFINE_SHADOW"]), threads=8)
    assert dbg2[2] > dbg[2] and dbg2[4] > 0


def test_node_transport_reduces_to_the_linear_system():
    """With Lambertian nodes (A(mu) = rho = hh) and no smoothing, the Jacobi steps of the separable node transport
    (gpu/wgsl/kernels.wgsl.js:416-461) converge to M = B_dir + diag(rho V) F M, M = pi rho Ls the exitance and
    F_ih = #{j : gtable[i, j] = h} / K over the active nodes: the restatement checked against a direct solve."""
    sc = dome.make_dome_scene(seed=1, width=32, height=24, level=3)
    S = O.Scene(sc)
    S.set_poses()
    K = 32
    g, mis = S.gather_table(K)
    act = np.nonzero(mis <= K / 2)[0].astype(np.uint32)
    assert 0 < len(act) < S.static_verts
    # every entry is MISS or a node; after the remap no entry names an inactive node that has an active alternative
    assert np.all((g == 0xFFFFFFFF) | (g < S.static_verts))
    nb = S.node_neighbours(act, nbr_k=4, sigma=0.0)
    assert np.array_equal(nb[:, 0, 0], np.arange(len(act))) and np.all(nb[:, 1:, 1] == 0)
    st = np.zeros((S.static_verts, 16))
    st[:, 3] = 1.0
    st[:, 15] = -1.0
    st = S.node_direct(act, st)
    assert np.all(st[act, 12:15] >= 0) and st[act, 12:15].max() > 0
    out, slot = S.node_jacobi(g, act, nb, st, 1, 200)
    # the linear system over the active nodes (entries on inactive nodes read their zero source)
    pos = {int(i): k for k, i in enumerate(act)}
    n = len(act)
    F = np.zeros((n, n))
    for k, i in enumerate(act):
        for h in g[i]:
            if int(h) in pos:
                F[k, pos[int(h)]] += 1.0 / K
    # the albedo tables and hh hold rho in float32
    rho = np.array([sc["materials"][sc["meshes"][m]["mat"]]["rho"] for m in sc["static"]["vert_mesh"][act]], np.float32).astype(np.float64)
    V = st[act, 3]
    for c in range(3):
        M = np.linalg.solve(np.eye(n) - (rho[:, c] * V)[:, None] * F, st[act, 12 + c])
        got = np.pi * rho[:, c] * out[act, 4 * slot + c]
        np.testing.assert_allclose(got, M, rtol=1e-9, atol=1e-12 * M.max())


def test_sensor_chain_known_answers():
    """The restated sensor chain (gpu/wgsl/sensor.wgsl.js) on inputs with closed-form outputs: a flat grey field with
    noise off, no blur, unit relative illumination and a linear tone curve gives raw DN = round(M E t g + black) per
    CFA site, the same value in every demosaiced channel, 8-bit RGB = round(255 (DN - black) / (max - black)), and
    4:2:0 chroma 128 with Y from BT.601."""
    from vtwin import sensor as S

    W, H = 12, 8
    L = np.zeros((H, W, 4), np.float32)
    L[..., :3] = 0.8
    ri = np.ones((H, W), np.float32)
    for demosaic in ("bilinear", "edge-aware", "hamilton"):
        p = S.sensor_params({"noise": False, "esfSigmaPx": 0.0, "esfIncludesAperture": False, "tone": "linear", "demosaic": demosaic,
                             "responseMatrix": [[1000.0, 0, 0], [0, 1000.0, 0], [0, 0, 1000.0]], "blackLevel": 64.0,
                             "conversionGain": 1.0, "fullWell": 1e9, "cfa": "RGGB"})
        su = S.pack_sensor_uniform(p, W, H, exposure=5.0, gain=1.0)
        raw, rgba, yuv, st = O.isp_chain(su, L, ri)
        E = np.float32(0.8) * np.float32(np.pi * 0.9 / 16)
        want_dn = np.floor(np.float32(1000.0) * E * np.float32(5.0) + np.float32(64.0) + np.float32(0.5))
        assert np.all(raw == want_dn), (raw[0, :4], want_dn)
        c8 = np.round((want_dn - 64.0) / (4095.0 - 64.0) * 255.0)
        assert np.all(rgba[..., :3] == c8) and np.all(rgba[..., 3] == 255)
        assert np.all(yuv["cb"] == 128) and np.all(yuv["cr"] == 128)
        assert np.all(yuv["y"] == np.round(0.299 * c8 + 0.587 * c8 + 0.114 * c8))
        assert st[0] == yuv["y"].astype(np.int64).sum() and st[1] == st[2] == st[3] == W * H * round((want_dn - 64.0) / 4031.0 * 1023)
    # 4:4:4 and an sRGB tone: the 8-bit value is the sRGB OETF of the normalised DN
    p = S.sensor_params({"noise": False, "esfSigmaPx": 0.0, "esfIncludesAperture": False, "chroma": "4:4:4", "conversionGain": 1.0,
                         "responseMatrix": [[1000.0, 0, 0], [0, 1000.0, 0], [0, 0, 1000.0]], "fullWell": 1e9})
    su = S.pack_sensor_uniform(p, W, H, exposure=5.0, gain=1.0)
    raw, rgba, yuv, st = O.isp_chain(su, L, ri)
    v = (raw[0, 0] - 0.0) / 4095.0
    want = round(255 * (1.055 * v ** (1 / 2.4) - 0.055))
    assert np.all(np.abs(rgba[..., :3].astype(int) - want) <= 1)


def test_relative_illumination_pinhole_closed_form():
    """gpu/sensor.js:98 relativeIlluminationMap with k = 0 (theta_d = theta): RI = cos^q(theta) sin(theta) / theta."""
    sc = dome.make_dome_scene(seed=1, width=48, height=32, level=1)
    sc["cameras"][0]["k"] = [0.0, 0.0, 0.0, 0.0]
    S = O.Scene(sc)
    lens = S.scene["cameras"][0]
    q = 1.5
    ri = S.ri_map(0, q, (0.0, 90.0), (1.0, 1.0))
    from vtwin import _abi as A

    p = A.lens_params(lens)
    fx, fy, cx, cy, alpha, k = p[0], p[1], p[2], p[3], p[4], p[5:9]
    ys, xs = np.mgrid[0:32, 0:48].astype(np.float64)
    yd = (ys - cy) / fy
    xd = (xs - cx) / fx - alpha * yd
    th = np.hypot(xd, yd)
    want = np.where(th > 1e-6, np.cos(th) ** q * np.sin(th) / np.maximum(th, 1e-300), 1.0)
    np.testing.assert_allclose(ri, want.astype(np.float32), rtol=2e-7)


# ------------------------------------------------------------------------------------------ raster pass (lite_nodes)
def _grid_mesh(nx, ny, z=0.5, jitter=0.0, seed=0):
    """A (nx x ny)-cell grid of clip-space triangles covering [-0.9, 0.9]^2 with shared (jittered) vertices."""
    rng = np.random.default_rng(seed)
    xs, ys = np.linspace(-0.9, 0.9, nx + 1), np.linspace(-0.9, 0.9, ny + 1)
    P = np.array([[x, y] for y in ys for x in xs])
    inner = (np.abs(P[:, 0]) < 0.89) & (np.abs(P[:, 1]) < 0.89)
    P[inner] += rng.uniform(-jitter, jitter, (inner.sum(), 2))
    clip = np.concatenate([P, np.full((len(P), 1), z), np.ones((len(P), 1))], 1).astype(np.float32)
    idx = []
    for j in range(ny):
        for i in range(nx):
            a, b, c, d = j * (nx + 1) + i, j * (nx + 1) + i + 1, (j + 1) * (nx + 1) + i + 1, (j + 1) * (nx + 1) + i
            idx += [(a, b, c), (a, c, d)] if (i + j) % 2 else [(a, b, d), (b, c, d)]
    return clip, np.array(idx, np.uint32)


def test_raster_is_watertight_and_covers_each_sample_once():
    """Shared edges of a jittered grid: every sample inside the grid is covered by exactly one triangle (no cracks, no
    double hits), counted by drawing each triangle alone."""
    clip, idx = _grid_mesh(9, 7, jitter=0.08, seed=3)
    W, H = 61, 47
    cover = np.zeros((H, W, 4), np.int32)
    for t in range(len(idx)):
        k = O.raster(clip, idx, W, H, 4, t0=t, nt=1)
        cover += (k != np.uint64(2**64 - 1)).astype(np.int32)
    # samples well inside the grid's outline
    ys, xs = np.mgrid[0:H, 0:W]
    offs = np.array([[0.375, 0.125], [0.875, 0.375], [0.125, 0.625], [0.625, 0.875]])
    inside = np.ones((H, W, 4), bool)
    for s in range(4):
        nx = 2 * (xs + offs[s, 0]) / W - 1
        ny = 1 - 2 * (ys + offs[s, 1]) / H
        inside[..., s] = (np.abs(nx) < 0.88) & (np.abs(ny) < 0.88)
    assert cover[inside].min() == 1 and cover[inside].max() == 1, np.unique(cover[inside], return_counts=True)
    # and drawn together every such sample holds one of the triangles
    k = O.raster(clip, idx, W, H, 4)
    assert (k[inside] != np.uint64(2**64 - 1)).all()


def test_raster_depth_order_ties_and_clipping():
    """'less' depth: the nearer triangle wins wherever both cover; on equal depth the one drawn first; samples
    beyond the far plane, behind the near plane or at depth 1 stay empty; a triangle crossing w = 0 keeps its
    visible part."""
    quad = lambda z, w=1.0: np.array([[-w, -w, z, w], [w, -w, z, w], [w, w, z, w], [-w, w, z, w]], np.float32)
    I2 = np.array([[0, 1, 2], [0, 2, 3], [4, 5, 6], [4, 6, 7]], np.uint32)
    E = np.uint64(2**64 - 1)
    k = O.raster(np.concatenate([quad(0.6), quad(0.3)]), I2, 16, 12, 4)
    assert set(np.unique(k & np.uint64(0xffffffff)).tolist()) <= {2, 3}
    k = O.raster(np.concatenate([quad(0.4), quad(0.4)]), I2, 16, 12, 4)
    assert set(np.unique(k & np.uint64(0xffffffff)).tolist()) <= {0, 1}
    for z in (1.0, 1.2, -0.1):
        assert (O.raster(quad(z), I2[:2], 16, 12, 4) == E).all(), z
    # one vertex behind the camera (w < 0): the visible part is drawn, nothing from the part behind
    clip = np.array([[-0.5, -0.5, 0.5, 1.0], [0.5, -0.5, 0.5, 1.0], [0.0, 0.2, -0.5, -0.5]], np.float32)
    k = O.raster(clip, np.array([[0, 1, 2]], np.uint32), 32, 32, 4)
    assert (k != E).sum() > 100
    d = np.frombuffer(((k[k != E] >> np.uint64(32)).astype(np.uint32)).tobytes(), np.float32)
    assert d.min() >= 0.0 and d.max() < 1.0


def test_slice_tris_bounds_area_and_shared_vertices():
    """sliceTris (lite_nodes/renderer.js:443): every piece spans at most h per axis, the area is kept, and the cut
    points shared by neighbouring pieces are bit-identical (each sliced capsule stays closed: no edge is used by an
    odd number of triangles)."""
    sc = dome.make_scope_scene(level=3, n_tools=1, width=64, height=36)
    S = O.Scene(sc)
    V, I = S.lite_geometry(subdiv=0.003, subdiv_fixture=0.01)
    ns = len(sc["static"]["P"])
    dyn = V[ns:]
    P = dyn[:, :3].view(np.float32).astype(np.float64)
    tris = I[len(sc["static"]["I"]):] - ns
    ext = P[tris].max(axis=1) - P[tris].min(axis=1)
    assert ext.max() <= 0.003 + 1e-7, ext.max()   # float32 positions: a few ulps at 0.2 m
    area = lambda p, t: 0.5 * np.linalg.norm(np.cross(p[t[:, 1]] - p[t[:, 0]], p[t[:, 2]] - p[t[:, 0]]), axis=1).sum()
    b = sc["bodies"][1]
    assert abs(area(P, tris[(dyn[tris[:, 0], 3] >> 16) == 1]) - area(b["P"].astype(np.float64), b["I"])) < 1e-4 * area(b["P"].astype(np.float64), b["I"])
    # closed surface after slicing: undirected edges keyed by the vertices' exact bits
    tool = tris[(dyn[tris[:, 0], 3] >> 16) == 1]
    key = {tuple(dyn[v, :3]) for v in tool.ravel()}
    ids = {k: i for i, k in enumerate(sorted(key))}
    e = {}
    for t in tool:
        a, bb, c = (ids[tuple(dyn[v, :3])] for v in t)
        for u, w in ((a, bb), (bb, c), (c, a)):
            if u != w:
                e[(min(u, w), max(u, w))] = e.get((min(u, w), max(u, w)), 0) + 1
    counts = np.array(list(e.values()))
    # no open edge (a crack would leave an edge used once; collinear cut points make some edges shared 4 or 6 times)
    assert (counts % 2 == 0).all(), np.unique(counts, return_counts=True)


def test_lite_emitter_samples_are_stratified_and_posed():
    """The 96 outlet samples (lite_nodes/renderer.js:598): on the emitter, balanced over the 4 sectors, and moved
    rigidly by the scope pose."""
    sc = dome.make_scope_scene(level=3, n_tools=0, width=64, height=36)
    S = O.Scene(sc)
    es0, sc0 = S.lite_emitter(96, np.eye(4).T.ravel())
    assert np.allclose(es0[:, 2], 0.0, atol=1e-7) and (np.hypot(es0[:, 0], es0[:, 1]) <= 0.004 + 1e-6).all()
    cnt = np.bincount(es0[:, 3].astype(int), minlength=4)
    assert cnt.min() >= 20, cnt
    T = dome.scope_poses(1, 0, seed=5)[0, 0].reshape(4, 4).T
    es1, _ = S.lite_emitter(96, T.T.ravel())
    want = (T[:3, :3] @ es0[:, :3].astype(np.float64).T).T + T[:3, 3]
    assert np.abs(es1[:, :3] - want).max() < 1e-6
    assert np.array_equal(es1[:, 3], es0[:, 3]) and np.allclose(es1[:, 7], es0[:, 7])


def test_unit_kernel_restatements_agree_across_precisions():
    """The restated unit kernels (gpu/wgsl/kernels.wgsl.js:494-551): the float32 WGSL-order forms against the float64
    ones on random cases: KB4 unproject / project (8 fixed Newton steps against gpu/lens.js's 20), the capsule
    occlusion, the emission profile at and between its knots, and the BSDF on all material kinds, where float32 is
    within 1e-5 of float64 on nearly every case (the rest are grazing angles that float32 itself rounds away)."""
    from vtwin import dome

    sc = dome.make_dome_scene(seed=1, width=64, height=48, level=2)
    sc["materials"].append({**dome.lambertian("coated", [0.0, 0.0, 0.0]), "metallic": 1, "coated": 1, "f0": [0.95, 0.64, 0.54],
                            "roughness": 0.4, "ior": 1.5, "coat_ior": 1.5, "coat_roughness": 0.08, "tau": [0.9, 0.7, 0.5]})
    sc["emitter"]["theta"] = [0.0, 0.5, 1.0]
    sc["emitter"]["p"] = [1.0, 0.6, 0.1]
    S = O.Scene(sc)
    rng = np.random.default_rng(1)
    n = 4000
    lens = [300.0, 300.0, 319.5, 239.5, 0.05, -0.01, 0.002, -0.0003, 0.0]
    tin = np.zeros((2 * n, 4), np.float32)
    tin[:n, 0], tin[:n, 1] = rng.uniform(0, 640, n), rng.uniform(0, 480, n)
    tin[n:, :3] = rng.normal(size=(n, 3))
    tin[n:, 2] = np.abs(tin[n:, 2]) + 0.5
    a, b = S.unit_test(0, tin, lens=lens), S.unit_test(0, tin, lens=lens, fp64=True)
    assert np.abs(a[0::2, :3] - b[0::2, :3]).max() <= 1e-5 and np.abs(a[1::2, :2] - b[1::2, :2]).max() <= 1e-3
    tb = np.zeros((2 * n, 4), np.float32)
    tb[n:, :3] = b[0::2, :3]
    back = S.unit_test(0, tb, lens=lens, fp64=True)[1::2, :2]
    assert np.abs(back - tin[:n, :2]).max() <= 1e-3                 # project(unproject(uv)) = uv
    pt = np.zeros((6, 4), np.float32)
    pt[:, 0] = [0.0, 0.25, 0.5, 0.75, 1.0, 1.5]
    assert np.allclose(S.unit_test(3, pt, fp64=True)[:, 0], [1.0, 0.8, 0.6, 0.35, 0.1, 0.0], atol=1e-6)
    tc = np.zeros((4 * n, 4), np.float32)
    tc[0::4, :3] = rng.uniform(-0.1, 0.1, (n, 3))
    tc[1::4, :3] = rng.normal(size=(n, 3))
    tc[1::4, :3] /= np.linalg.norm(tc[1::4, :3], axis=1, keepdims=True)
    tc[2::4, :3], tc[2::4, 3], tc[3::4, :3] = [0.0, 0.0, -0.1], 0.01, [0.0, 0.0, 0.1]
    c32, c64 = S.unit_test(2, tc)[:, 0], S.unit_test(2, tc, fp64=True)[:, 0]
    assert np.abs(c32 - c64).max() <= 1e-5 and np.mean(c64 > 0) > 0.5
    nm = len(sc["materials"])
    tv = np.zeros((4 * n, 4), np.float32)
    for k in range(3):
        w = rng.normal(size=(n, 3))
        tv[k::4, :3] = w / np.linalg.norm(w, axis=1, keepdims=True)
    tv[1::4, :3] *= np.sign(np.sum(tv[1::4, :3] * tv[0::4, :3], 1))[:, None]
    tv[2::4, :3] *= np.sign(np.sum(tv[2::4, :3] * tv[0::4, :3], 1))[:, None]
    tv[3::4, :3] = rng.random((n, 3))
    tv[3::4, 3] = rng.integers(0, nm, n)
    f32, f64 = S.unit_test(1, tv)[0::3], S.unit_test(1, tv, fp64=True)[0::3]
    rel = np.abs(f32[:, :3] - f64[:, :3]).max(1) / np.maximum(np.abs(f64[:, :3]).max(1), 1e-3)
    assert np.mean(rel <= 1e-5) >= 0.99
