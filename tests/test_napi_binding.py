"""The Node-API drop-in (veridien-twin_gb300/js): the addon compiles against the Node-API declarations, every library
function it calls is exported by libvtwin.so, and renderer.js calls only functions the addon registers and imports only
names the reference's own gpu/ modules export. Node is not installed here, so nothing JavaScript runs."""
import os
import re
import shutil
import subprocess

import pytest

from conftest import ROOT, reference_path

JS = os.path.join(ROOT, "veridien-twin_gb300", "js")
ADDON = os.path.join(JS, "vtwin_addon.cc")
RENDERER = os.path.join(JS, "renderer.js")
LIB = os.path.join(ROOT, "veridien-twin_gb300", "vtwin", "libvtwin.so")


def _read(p):
    with open(p) as f:
        return f.read()


def _registered():
    return set(re.findall(r'add\(env, exports, "(\w+)", \w+\)', _read(ADDON)))


@pytest.mark.skipif(shutil.which("g++") is None, reason="g++ absent")
def test_addon_compiles_against_node_api():
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-Wall", "-Wextra", "-Wno-unused-parameter", "-Werror",
                        "-I", os.path.join(ROOT, "tests", "napi"), "-I", os.path.join(ROOT, "include"), ADDON],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_addon_calls_only_exported_library_functions():
    if not os.path.exists(LIB):
        pytest.skip("libvtwin.so not built")
    called = set(re.findall(r"\b(vt_[a-z0-9_]+)\(", _read(ADDON)))
    header = set(re.findall(r"\b(vt_[a-z0-9_]+)\(", _read(os.path.join(ROOT, "include", "vtwin.h"))))
    called &= header  # the library's entry points (not local helpers named vt_*)
    assert len(called) > 40
    nm = shutil.which("nm")
    if nm is None:
        pytest.skip("nm absent")
    out = subprocess.run([nm, "-D", "--defined-only", LIB], capture_output=True, text=True, check=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if ln.strip()}
    assert not called - exported, sorted(called - exported)


def test_renderer_js_uses_registered_addon_functions():
    used = set(re.findall(r"\baddon\.(\w+)\(", _read(RENDERER)))
    reg = _registered()
    assert len(reg) >= 40
    assert used and not used - reg, sorted(used - reg)


def test_renderer_js_keeps_reference_defaults_and_presets():
    src = _read(RENDERER)
    for key, val in {"spp": "1", "refine": "6", "lightSamples": "4", "refineLightSamples": "1", "radiosityEvery": "1",
                     "nodeSpacing": "0.003", "gatherK": "64", "nodeSamples": "4", "itersPerFrame": "4",
                     "itersInitial": "96", "smoothSigma": "0.003", "smoothRadius": "0.006", "nbrK": "16",
                     "leafSize": "4"}.items():
        assert re.search(rf"\b{key}: {re.escape(val)}\b", src), key
    for preset in ("judge", "balanced", "live"):
        assert re.search(rf"\b{preset}: \{{", src), preset
    for method in ("renderCamera", "renderFrame", "sensor", "readback", "visible", "project", "setPoses", "converge",
                   "nodeSummary", "exposureOf", "setExposure", "timings", "debugFlags", "destroy"):
        assert re.search(rf"^  (async |static async )?{method}\(", src, re.M), method


def test_renderer_js_imports_exist_in_reference_modules():
    gpu = reference_path("gpu")
    if not os.path.isdir(gpu):
        pytest.skip("reference checkout absent")
    src = _read(RENDERER)
    for names, mod in re.findall(r"import \{([^}]*)\} from '\./(\w+\.js)'", src):
        exports = set(re.findall(r"^export (?:async )?(?:function|const|class) (\w+)", _read(os.path.join(gpu, mod)), re.M))
        for n in (x.strip() for x in names.split(",")):
            assert n in exports, (mod, n)
