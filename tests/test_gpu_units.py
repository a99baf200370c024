"""The reference's GPU unit kernels (gpu/wgsl/kernels.wgsl.js:494-551 lensTest, bsdfTest, capsuleTest, profileTest)
run through vt_unit_test on the device, against the oracle's float32 WGSL-order restatement of the same functions
and against its float64 form.

Cases are random and seeded: pixels over the whole image and points across the field of view for the KB4 lens (the
synthetic dome's camera and the twin's CAM1 lens), and for the BSDF every material kind the scene can hold: the
dielectric with ior 1 (the configs' Lambertian), rough and smooth dielectrics, a conductor and a coated conductor.
The bar: the float32 device functions agree with the float32 restatement to 1e-5 relative on 99% of cases (the two
sides round sin, cos, atan2 and pow differently and the device contracts multiply-adds, so not every case is
bit-exact; the count of bit-exact cases is printed); where float32 itself is ill-conditioned (grazing angles, a
peaked lobe's D(h) near n.h = 1, the phase of the layer lines) the device is as close to float64 as the float32
restatement is; a sampled direction may change lobe only where the lobe choice u0 < specProb sits within float
rounding of its threshold.
"""
import json
import os

import numpy as np
import pytest

import oracle as O
from vtwin import _abi as A
from vtwin import dome

pytestmark = pytest.mark.gpu

C0_LENS = [300.0, 300.0, 319.5, 239.5, 0.05, -0.01, 0.002, -0.0003, 0.0]
# the twin's CAM1 lens (its scene's KB4 calibration: K and D)
CAM1_LENS = [745.386252, 747.207117, 633.927484, 380.042876, -0.012300643, -0.016677738, 0.035329677, -0.033581606, 0.0]


def unit(v):
    return v / np.linalg.norm(v, axis=-1, keepdims=True)


@pytest.fixture(scope="module")
def rig():
    from vtwin.renderer import TwinRenderer

    sc = dome.make_dome_scene(seed=1, width=64, height=48, level=2)
    m = sc["materials"]
    rough = {**dome.lambertian("rough_dielectric", [0.6, 0.4, 0.3]), "ior": 1.5, "roughness": 0.55}
    smooth = {**dome.lambertian("smooth_dielectric", [0.2, 0.5, 0.7]), "ior": 1.6, "roughness": 0.12}
    metal = {**dome.lambertian("conductor", [0.0, 0.0, 0.0]), "metallic": 1, "f0": [0.56, 0.57, 0.58], "roughness": 0.35,
             "ior": 1.5}
    coated = {**dome.lambertian("coated", [0.0, 0.0, 0.0]), "metallic": 1, "coated": 1, "f0": [0.95, 0.64, 0.54],
              "roughness": 0.4, "ior": 1.5, "coat_ior": 1.5, "coat_roughness": 0.08, "tau": [0.9, 0.7, 0.5]}
    first_extra = len(m)
    m.extend([rough, smooth, metal, coated])
    # the emission profile of the reference's own light (configs/twin/physics.yaml light.profile, via the golden file)
    kat = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "physics_kat.json")))
    sc["emitter"]["theta"] = [float(np.radians(t)) for t in kat["profile"]["theta_deg"]]
    sc["emitter"]["p"] = [float(p) for p in kat["profile"]["p"]]
    r = TwinRenderer.create(sc, nodes=False)
    ref = O.Scene(sc)
    yield r, ref, sc, first_extra
    r.destroy()


def rel_err(a, b, floor):
    return np.abs(a - b) / np.maximum(np.abs(b), floor)


@pytest.mark.parametrize("lens", [C0_LENS, CAM1_LENS], ids=["c0", "cam1"])
def test_lens_kernel(rig, lens):
    r, ref, _, _ = rig
    rng = np.random.default_rng(3)
    n = 20000
    lens32 = [float(np.float32(x)) for x in lens]
    W, H = 2.0 * lens32[2] + 1.0, 2.0 * lens32[3] + 1.0
    uv = np.stack([rng.uniform(0, W, n), rng.uniform(0, H, n)], 1)
    th = rng.uniform(0.0, 1.0, n)                         # up to 57 degrees off axis, inside both fields of view
    ph = rng.uniform(0.0, 2 * np.pi, n)
    X = np.stack([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)], 1) * rng.uniform(0.05, 5.0, n)[:, None]
    tin = np.zeros((2 * n, 4), np.float32)
    tin[:n, :2] = uv
    tin[n:, :3] = X
    g = r.unit_test(A.VT_UNIT_LENS, tin, lens=lens32)
    c32 = ref.unit_test(0, tin, lens=lens32, fp64=False)
    c64 = ref.unit_test(0, tin, lens=lens32, fp64=True)
    ray_g, ray_c, ray_d = g[0::2, :3], c32[0::2, :3], c64[0::2, :3]
    uv_g, uv_c, uv_d = g[1::2, :2], c32[1::2, :2], c64[1::2, :2]
    e_ray = np.abs(ray_g - ray_c).max()
    e_ray64 = np.abs(ray_g - ray_d).max()
    e_uv = np.abs(uv_g - uv_c).max()
    e_uv64 = np.abs(uv_g - uv_d).max()
    exact = np.mean(np.all(g == c32, axis=1))
    # the round trip through the device functions: project(unproject(uv)) = uv
    back = r.unit_test(A.VT_UNIT_LENS, np.concatenate([np.zeros((n, 4), np.float32), np.pad(ray_g, ((0, 0), (0, 1)))]), lens=lens32)
    e_rt = np.abs(back[1::2, :2] - uv.astype(np.float32)).max()
    print(f"\nlens {lens[0]:.0f}: ray vs f32 {e_ray:.1e}, vs f64 {e_ray64:.1e}; uv vs f32 {e_uv:.1e} px, vs f64 {e_uv64:.1e} px; "
          f"bit-exact slots {exact:.4f}; round trip {e_rt:.1e} px")
    assert e_ray <= 1e-6 and e_ray64 <= 1e-5
    assert e_uv <= 1e-3 and e_uv64 <= 2e-3
    assert e_rt <= 2e-3


def bsdf_cases(n, n_mat, seed):
    rng = np.random.default_rng(seed)
    nn = unit(rng.normal(size=(n, 3)))
    def around(k, neg_frac):
        w = unit(rng.normal(size=(n, 3)))
        s = np.sign(np.sum(w * nn, 1))
        flip = rng.random(n) < neg_frac
        return w * np.where(flip, -s, s)[:, None]
    v = around(0, 0.05)
    l = around(1, 0.05)
    u = rng.random((n, 3))
    mat = rng.integers(0, n_mat, n)
    tin = np.zeros((4 * n, 4), np.float32)
    tin[0::4, :3], tin[1::4, :3], tin[2::4, :3], tin[3::4, :3] = nn, l, v, u
    tin[3::4, 3] = mat
    return tin, mat


def test_bsdf_kernel(rig):
    r, ref, sc, first_extra = rig
    n_mat = len(sc["materials"])
    n = 40000
    tin, mat = bsdf_cases(n, n_mat, seed=5)
    g = r.unit_test(A.VT_UNIT_BSDF, tin)
    c32 = ref.unit_test(1, tin, fp64=False)
    c64 = ref.unit_test(1, tin, fp64=True)
    kinds = {"lambertian": mat < first_extra, "dielectric": (mat == first_extra) | (mat == first_extra + 1),
             "conductor": mat == first_extra + 2, "coated": mat == first_extra + 3}

    def err(a, b):   # per case: f (relative to the largest channel) and pdf (relative)
        sc_ = np.maximum(np.abs(b[:, :3]).max(1), 1e-3)
        return np.maximum(np.abs(a[:, :3] - b[:, :3]).max(1) / sc_, np.abs(a[:, 3] - b[:, 3]) / np.maximum(np.abs(b[:, 3]), 1e-3))

    f_g, f_c, f_d = g[0::3], c32[0::3], c64[0::3]
    e32 = err(f_g, f_c)               # the device against the float32 restatement
    e64 = err(f_g, f_d)               # the device against float64
    cond = err(f_c, f_d)              # how far float32 arithmetic itself is from float64 on each case
    # sampled directions: the lobe choice u0 < specProb and the validity test n.l > 0 may go either way within float
    # rounding; where both sides took the same lobe, the directions and their pdfs are compared (a peaked lobe's pdf
    # at its own sample, D(h) with n.h near 1, magnifies float rounding: judged against the float32 restatement's
    # own distance from float64)
    s_g, s_c, s_d = g[1::3], c32[1::3], c64[1::3]
    valid = (s_g[:, 3] > 0) & (s_c[:, 3] > 0) & (s_d[:, 3] > 0)
    same_lobe = valid & (np.abs(s_g[:, :3] - s_c[:, :3]).max(1) < 1e-3) & (np.abs(s_c[:, :3] - s_d[:, :3]).max(1) < 1e-3)
    lobe_flips = np.mean(valid & ~same_lobe)
    validity_flips = np.mean((s_g[:, 3] > 0) != (s_c[:, 3] > 0))
    e_dir = np.abs(s_g[same_lobe, :3] - s_c[same_lobe, :3]).max(1)
    e_spdf64 = rel_err(s_g[same_lobe, 3], s_d[same_lobe, 3], 1e-3)
    c_spdf = rel_err(s_c[same_lobe, 3], s_d[same_lobe, 3], 1e-3)
    x_g, x_c, x_d = g[2::3], c32[2::3], c64[2::3]
    e_alb = rel_err(x_g[:, :3], x_c[:, :3], 1e-4).max()
    e_alb64 = rel_err(x_g[:, :3], x_d[:, :3], 1e-4).max()
    # layerNormal takes fract(p.bd / period) of a value near 500, so float32 itself keeps about 4 digits of the phase
    e_ln64 = np.abs(x_g[:, 3] - x_d[:, 3])
    c_ln = np.abs(x_c[:, 3] - x_d[:, 3])
    exact = np.mean(np.all(g == c32, axis=1))
    q = lambda a, p=0.999: float(np.quantile(a, p))
    for name, sel in kinds.items():
        print(f"\n{name:11s}: {sel.sum():6d} cases, vs f32 q99 {q(e32[sel], 0.99):.1e} max {e32[sel].max():.1e}; vs f64 q99.9 "
              f"{q(e64[sel]):.1e} (the f32 restatement {q(cond[sel]):.1e})", end="")
    worse = np.mean(e64 > np.maximum(4 * cond, 1e-5))
    print(f"\nfurther from f64 than 4x the f32 restatement: {worse:.1e} of cases")
    print(f"samples: lobe flips {lobe_flips:.1e}, validity flips {validity_flips:.1e}, direction vs f32 {e_dir.max():.1e}, "
          f"pdf vs f64 q99.9 {q(e_spdf64):.1e} (f32 restatement {q(c_spdf):.1e}); albedoSpec {e_alb:.1e} (f64 {e_alb64:.1e}); "
          f"layerNormal.x vs f64 q99.9 {q(e_ln64):.1e} (f32 restatement {q(c_ln):.1e}); bit-exact slots {exact:.4f}")
    for name, sel in kinds.items():
        assert sel.sum() > 1000
        # the device functions agree with the float32 restatement to 1e-5 on 99% of the cases of every kind
        assert q(e32[sel], 0.99) <= 1e-5, name
        # and are as close to float64 as the float32 restatement itself is
        assert q(e64[sel]) <= 2 * q(cond[sel]) + 1e-5, name
    assert worse <= 1e-3
    assert lobe_flips <= 1e-3 and validity_flips <= 1e-3
    assert e_dir.max() <= 1e-4 and q(e_dir) <= 1e-5
    assert q(e_spdf64) <= 2 * q(c_spdf) + 1e-5
    assert e_alb <= 1e-6 and e_alb64 <= 1e-6
    assert q(e_ln64) <= 2 * q(c_ln) + 1e-6
    # a material index beyond the scene's gives NaN, as a bad index must not read past the material table
    bad = tin[:8].copy()
    bad[3, 3] = n_mat + 3
    assert np.isnan(r.unit_test(A.VT_UNIT_BSDF, bad)[:3]).all()


def test_capsule_kernel(rig):
    r, ref, _, _ = rig
    rng = np.random.default_rng(7)
    n = 20000
    a = rng.uniform(-0.2, 0.2, (n, 3))
    b = a + unit(rng.normal(size=(n, 3))) * rng.uniform(0.02, 0.3, n)[:, None]
    rad = rng.uniform(0.002, 0.02, n)
    p = a + (b - a) * rng.uniform(-0.5, 1.5, n)[:, None] + unit(rng.normal(size=(n, 3))) * rng.uniform(0.01, 0.2, n)[:, None]
    nrm = unit(rng.normal(size=(n, 3)))
    tin = np.zeros((4 * n, 4), np.float32)
    tin[0::4, :3], tin[1::4, :3], tin[2::4, :3], tin[2::4, 3], tin[3::4, :3] = p, nrm, a, rad, b
    g = r.unit_test(A.VT_UNIT_CAPSULE, tin)[:, 0]
    c32 = ref.unit_test(2, tin, fp64=False)[:, 0]
    c64 = ref.unit_test(2, tin, fp64=True)[:, 0]
    e32, e64 = np.abs(g - c32).max(), np.abs(g - c64).max()
    print(f"\ncapsule: {np.mean(g > 0):.3f} occluding, max occlusion {g.max():.3f}; |gpu - f32| {e32:.1e}, |gpu - f64| {e64:.1e}")
    assert np.mean(g > 0) > 0.3
    assert e32 <= 1e-5 and e64 <= 1e-5


def test_profile_kernel(rig):
    r, ref, sc, _ = rig
    knots = np.array(sc["emitter"]["theta"], np.float32)
    rng = np.random.default_rng(9)
    th = np.concatenate([rng.uniform(0, float(knots[-1]) * 1.2, 5000), knots, knots[-1:] + 1e-3, [0.0, np.pi]]).astype(np.float32)
    tin = np.zeros((len(th), 4), np.float32)
    tin[:, 0] = th
    g = r.unit_test(A.VT_UNIT_PROFILE, tin)[:, 0]
    c32 = ref.unit_test(3, tin, fp64=False)[:, 0]
    c64 = ref.unit_test(3, tin, fp64=True)[:, 0]
    # the tabulated profile at its own knots, and 0 past the last one (gpu/wgsl/shade.wgsl.js:15)
    p_knots = np.array(sc["emitter"]["p"], np.float32)
    e_knots = np.abs(g[5000:5000 + len(knots)] - p_knots).max()
    print(f"\nprofile: {len(knots)} knots; |gpu - f32| {np.abs(g - c32).max():.1e}, |gpu - f64| {np.abs(g - c64).max():.1e}, "
          f"at the knots {e_knots:.1e}")
    assert np.abs(g - c32).max() <= 1e-6 and np.abs(g - c64).max() <= 1e-6
    assert e_knots <= 1e-6
    assert g[5000 + len(knots)] == 0.0
