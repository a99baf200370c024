import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "veridien-twin_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))


# A checkout of the reference project, for the CPU tests that read its own files (scene meshes, configuration):
# $VT_REFERENCE, else a sibling directory named `reference` beside this repository. Tests that need it skip without it.
REFERENCE = os.environ.get("VT_REFERENCE") or os.path.join(os.path.dirname(ROOT), "reference")


def reference_path(*parts) -> str:
    return os.path.join(REFERENCE, *parts)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def has_gpu() -> bool:
    try:
        import ctypes

        cudart = None
        for name in ("libcudart.so", "libcudart.so.13", "libcudart.so.12"):
            try:
                cudart = ctypes.CDLL(name)
                break
            except OSError:
                continue
        if cudart is None:
            return False
        n = ctypes.c_int(0)
        return cudart.cudaGetDeviceCount(ctypes.byref(n)) == 0 and n.value > 0
    except Exception:
        return False


@pytest.fixture(scope="session")
def dome_small():
    from vtwin import dome

    return dome.make_dome_scene(seed=1, width=160, height=120)


@pytest.fixture(scope="session")
def dome_c0():
    from vtwin import dome

    return dome.make_dome_scene(seed=1)
