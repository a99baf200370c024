"""Failure detection without a GPU fault: a device wait that nothing completes runs out, the kernel returns, the host
reads VT_ERR_TIMEOUT, and the context keeps working (the pipelines' bounded mbarrier waits, vt_wait_check)."""
import time

import numpy as np
import pytest

from vtwin import _abi as A
from vtwin import dome
from vtwin.renderer import TwinRenderer

pytestmark = pytest.mark.gpu


def test_bounded_wait_times_out_and_the_context_survives():
    sc = dome.make_dome_scene(seed=1, width=48, height=32, level=2)
    r = TwinRenderer.create(sc)
    assert r.lib.vt_wait_check(r._ctx, 2_000_000, 1) == A.VT_OK          # the phase completes: no timeout
    t0 = time.perf_counter()
    st = r.lib.vt_wait_check(r._ctx, 2_000_000, 0)                        # nothing arrives: ~1 ms of waiting
    dt = time.perf_counter() - t0
    assert st == A.VT_ERR_TIMEOUT and dt < 2.0
    assert b"did not complete" in r.lib.vt_last_error(r._ctx)
    # the context is still usable: a render and another completed wait
    out = np.zeros((32, 48, 4), np.float32)
    r.renderCamera(0, out=out, spp=2, lightSamples=1, seed=0, mode=A.VT_SHADE_PATH, max_depth=2)
    assert np.all(np.isfinite(out)) and out[..., :3].max() > 0
    assert r.lib.vt_wait_check(r._ctx, 2_000_000, 1) == A.VT_OK
    assert r.lib.vt_wait_check(r._ctx, 0, 1) == A.VT_ERR_ARG
    r.destroy()
