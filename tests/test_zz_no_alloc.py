"""The allocation-free radiosity entry point (vt_radiosity_solve_static) against the allocating one.

Callers that cannot allocate device memory while they run (a frame loop with a fixed time budget, a host that sizes
all device memory up front) call vt_radiosity_solve_static with their own device buffers; its scratch is a static
device array inside the library. Two calls in a row with different right-hand sides must each reproduce
vt_radiosity_solve (the second call must not see the first call's iterates). This file is collected last so that a
run stopping at its first failure has run every other test already.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_static_solve_matches_allocating_solve_twice():
    torch = pytest.importorskip("torch")
    from vtwin import _abi as A
    from vtwin import dome
    from vtwin.renderer import VtError, form_factors, solve_radiosity, solve_radiosity_static

    n = 2048
    P = dome.dome_patches(n, seed=2)
    F = torch.empty((n, n), dtype=torch.float32, device="cuda")
    form_factors(P["centres"], P["normals"], P["areas"], out=F)
    rho = torch.from_numpy(P["rho"]).cuda()
    E1 = dome.radiosity_rhs(n, P["lamps"], 1)
    E2 = np.zeros_like(E1)
    E2[P["lamps"][::2], 0] = 80.0                      # a different right-hand side for the second call
    for E in (E1, E2):
        B_ref, info_ref = solve_radiosity(F, P["rho"], E, tol=1e-6, max_iters=500)
        Ed = torch.from_numpy(np.ascontiguousarray(E[:, 0])).cuda()
        B = torch.full((n,), float("nan"), dtype=torch.float32, device="cuda")
        info = solve_radiosity_static(F, rho, Ed, B, tol=1e-6, max_iters=500)
        torch.cuda.synchronize()
        got = B.cpu().numpy()
        assert info["status"] == A.VT_OK and info["iters"] == info_ref["iters"]
        err = np.linalg.norm(got - B_ref[:, 0]) / np.linalg.norm(B_ref[:, 0])
        assert err <= 1e-6, err
    # F as an offset view (rows not 16-byte aligned): the same solution as the aligned F
    Fo_store = torch.empty(n * n + 1, dtype=torch.float32, device="cuda")
    Fo = Fo_store[1:].view(n, n)
    Fo.copy_(F)
    assert Fo.data_ptr() % 16 == 4
    B_ref, info_ref = solve_radiosity(F, P["rho"], E1, tol=1e-6, max_iters=500)
    Ed = torch.from_numpy(np.ascontiguousarray(E1[:, 0])).cuda()
    B = torch.full((n,), float("nan"), dtype=torch.float32, device="cuda")
    info = solve_radiosity_static(Fo, rho, Ed, B, tol=1e-6, max_iters=500)
    torch.cuda.synchronize()
    assert info["status"] == A.VT_OK and info["iters"] == info_ref["iters"]
    err = np.linalg.norm(B.cpu().numpy() - B_ref[:, 0]) / np.linalg.norm(B_ref[:, 0])
    assert err <= 1e-6, err
    # sizes beyond the static maximum are refused by the C side itself, not truncated
    import ctypes as C

    from vtwin.renderer import load

    lib = load()
    big = 16385
    buf = torch.zeros((big,), dtype=torch.float32, device="cuda")
    p = C.c_void_p(buf.data_ptr())
    st = lib.vt_radiosity_solve_static(p, p, p, p, big, 10, 8, 1e-6, None, None, None)
    assert st == A.VT_ERR_ARG
    # a host pointer is refused (the entry point takes device buffers only)
    h = np.zeros(16, np.float32)
    hp = h.ctypes.data_as(C.c_void_p)
    assert lib.vt_radiosity_solve_static(hp, p, p, p, 4, 10, 8, 1e-6, None, None, None) == A.VT_ERR_ARG
    # and so are wrong-sized tensors, before anything reaches the C side
    with pytest.raises(VtError):
        solve_radiosity_static(buf[:8], rho, Ed, B)
