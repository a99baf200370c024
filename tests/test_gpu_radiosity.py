"""Mixed-precision node radiosity (tcgen05 BF16 / FP8 sweeps + iterative refinement) against a direct FP64 solve.

The bar: at most 1e-4 relative error against FP64, for one and for many right-hand sides.
"""
import numpy as np
import pytest

import oracle as O
from vtwin import _abi as A
from vtwin import dome
from vtwin.renderer import form_factors, solve_radiosity

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def system():
    n = 1024
    P = dome.dome_patches(n, seed=2)
    F = form_factors(P["centres"], P["normals"], P["areas"])
    return n, P, F


@pytest.mark.parametrize("prec", [A.VT_PREC_BF16, A.VT_PREC_FP8])
@pytest.mark.parametrize("R", [64, 8])
def test_mixed_precision_matches_fp64(system, prec, R):
    n, P, F = system
    E = dome.radiosity_rhs(n, P["lamps"], R, seed=5)
    Bd = O.solve_dense(F, P["rho"], E)
    B, info = solve_radiosity(F, P["rho"], E, precision=prec, tol=1e-6, max_iters=400)
    err = np.linalg.norm(B - Bd) / np.linalg.norm(Bd)
    col = np.max(np.linalg.norm(B - Bd, axis=0) / np.linalg.norm(Bd, axis=0))
    print(f"\nprecision {prec} R={R}: sweeps {info['iters']} refinements {info['refinements']} residual {info['residual']:.2e} "
          f"rel err {err:.2e} (worst column {col:.2e})")
    assert info["status"] == A.VT_OK
    assert err <= 1e-4 and col <= 1e-4


def test_reuse_of_converted_f(system):
    n, P, F = system
    E = dome.radiosity_rhs(n, P["lamps"], 16, seed=7)
    from vtwin.renderer import TwinRenderer
    r = TwinRenderer.create(dome.make_dome_scene(seed=1, width=32, height=24, level=1))
    B1, i1 = r.solve_radiosity(F, P["rho"], E, precision=A.VT_PREC_BF16, tol=1e-6)
    B2, i2 = r.solve_radiosity(F, P["rho"], E, precision=A.VT_PREC_BF16, tol=1e-6, reuse_f=True)
    assert np.array_equal(B1, B2) and i1["iters"] == i2["iters"]
    r.destroy()


def test_form_factors_with_visibility_match_oracle():
    """Dense F with each pair's visibility traced through the dome scene (the table occludes floor-to-floor and
    floor-to-dome pairs) against the FP64 restatement: the visible-ray counts agree on nearly every pair (shadow
    decisions at grazing rays may flip between float32 and float64), rows sum to <= 1, and F is below the
    unoccluded F."""
    from vtwin.renderer import TwinRenderer

    sc = dome.make_dome_scene(seed=1, width=32, height=24, level=5)
    r = TwinRenderer.create(sc)
    r.set_pose_array(A.identity_poses(1))
    n, K = 384, 16
    P = dome.dome_patches(n, seed=2)
    F = r.form_factors_visible(P["centres"], P["normals"], P["areas"], rays=K)
    S = O.Scene(sc)
    S.set_poses()
    F64, cnt = S.form_factors_visible(P["centres"], P["normals"], P["areas"], rays=K, fp64=True, threads=16)
    F0 = form_factors(P["centres"], P["normals"], P["areas"])
    facing = F0 > 0
    occluded = np.mean(cnt[facing] < K)
    row = np.abs(F - F64).sum(axis=1) / np.maximum(F64.sum(axis=1), 1e-30)
    whole = np.abs(F - F64).sum() / F64.sum()
    print(f"\nvisibility: {occluded:.3f} of facing pairs partly occluded; relative L1 difference {whole:.2e} overall, "
          f"rows within 1e-2: {np.mean(row <= 1e-2):.4f}, worst row {row.max():.2e}")
    assert occluded > 0.01
    # a ray that flips between float32 and float64 moves one entry by 1/K (and its row's scale)
    assert whole <= 1e-3 and np.mean(row <= 1e-2) >= 0.98
    assert np.all(F.sum(axis=1) <= 1 + 1e-5)
    assert np.all(F.sum(axis=1) <= F0.sum(axis=1) * (1 + 1e-5) + 1e-7)   # occlusion only takes light away
    r.destroy()


def test_offset_device_f_matches_aligned(system):
    """A device F that is an offset view (rows not 16-byte aligned) gives the same FP32 solution as an aligned F,
    for one right-hand side (the matvec) and for several (the GEMM sweep); the bulk-copy matvec refuses it."""
    torch = pytest.importorskip("torch")
    from vtwin.renderer import VtError

    n, P, F = system
    Fa = torch.from_numpy(F).cuda()
    store = torch.empty(n * n + 1, dtype=torch.float32, device="cuda")
    Fo = store[1:].view(n, n)
    Fo.copy_(Fa)
    assert Fo.data_ptr() % 16 == 4
    for R in (1, 8):
        E = dome.radiosity_rhs(n, P["lamps"], R, seed=3)
        Ba, ia = solve_radiosity(Fa, P["rho"], E, tol=1e-6, max_iters=400)
        Bo, io = solve_radiosity(Fo, P["rho"], E, tol=1e-6, max_iters=400)
        assert ia["status"] == A.VT_OK and io["status"] == A.VT_OK and ia["iters"] == io["iters"]
        assert np.linalg.norm(Bo - Ba) / np.linalg.norm(Ba) <= 1e-6
    E = dome.radiosity_rhs(n, P["lamps"], 1, seed=3)
    with pytest.raises(VtError):
        solve_radiosity(Fo, P["rho"], E, precision=A.VT_PREC_FP32_TMA, tol=1e-6, max_iters=50)


@pytest.mark.parametrize("case", ["c1", "c2_shaped"])
def test_configured_solves_match_fp64(case):
    """The configurations' systems gated in the suite, against the oracle's FP64 Jacobi (to 1e-12): C1 (N = 4096, one
    right-hand side, dense F with visibility through the dome, 64 rays per pair) for FP32, BF16 and FP8; and a
    C2-shaped system (N = 8192, 64 right-hand sides: random masks over the 96 lamp nodes, intensities U[10, 100]; F with
    4 rays per pair, as the C2 bench builds it) for FP32, BF16 and FP8, on 8 of the columns. The bar: 1e-4 relative
    error against FP64 (the configurations' target), each column."""
    torch = pytest.importorskip("torch")
    from vtwin.renderer import TwinRenderer

    n, R, rays = (4096, 1, 64) if case == "c1" else (8192, 64, 4)
    precs = (A.VT_PREC_FP32, A.VT_PREC_BF16, A.VT_PREC_FP8)
    scene_r = TwinRenderer.create(dome.make_dome_scene(seed=1, width=32, height=24, level=5), nodes=False)
    scene_r.set_pose_array(A.identity_poses(1))
    P = dome.dome_patches(n, seed=2)
    F = torch.empty((n, n), dtype=torch.float32, device="cuda")
    scene_r.form_factors_visible(P["centres"], P["normals"], P["areas"], rays=rays, out=F)
    E = dome.radiosity_rhs(n, P["lamps"], R, seed=5)
    Fh = F.cpu().numpy()
    pick = np.unique(np.linspace(0, R - 1, min(8, R)).astype(int))
    B64, _ = O.jacobi64(Fh, P["rho"], np.ascontiguousarray(E[:, pick]), tol=1e-12, max_it=600, threads=16)
    for prec in precs:
        B, info = solve_radiosity(F, P["rho"], E, precision=prec, tol=1e-6 if case == "c1" else 1e-5, max_iters=400)
        col = np.linalg.norm(B[:, pick] - B64, axis=0) / np.linalg.norm(B64, axis=0)
        print(f"\n{case} precision {prec}: {info['iters']} sweeps, {info['refinements']} residuals, {info['ms']:.2f} ms; "
              f"worst column {col.max():.2e} against FP64")
        assert info["status"] == A.VT_OK
        assert col.max() <= 1e-4
    scene_r.destroy()
