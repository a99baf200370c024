"""Build libvtwin.so (sm_103a) in-tree: one nvcc process per translation unit in parallel, then one link.

python -m vtwin.build [--force]   (from veridien-twin_gb300/), or vtwin.build.build() from Python.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(ROOT, "csrc")
OBJ = os.path.join(ROOT, "_build")
LIB = os.path.join(PKG, "libvtwin.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code: no FMA contraction (aarch64 gcc contracts a*b+c by default), so the host scene preparation gives the
# same bits on x86 and Arm
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fno-fast-math", "-Xcompiler", "-ffp-contract=off",
          "--expt-relaxed-constexpr"]


# per-file flags: the sensor chain, the rasteriser, the BVH builder and the scene preparation are compiled without multiply-add
# contraction, so their arithmetic is the sequence of separately rounded operations that the CPU code performs
EXTRA = {"vt_isp.cu": ["--fmad=false"], "vt_lite_raster.cu": ["--fmad=false"], "vt_bvh_gpu.cu": ["--fmad=false"], "vt_scene_gpu.cu": ["--fmad=false"],
         # the raster pass's shading: WGSL's own f32 precision (division 2.5 ulp, inverseSqrt 2 ulp), not IEEE division
         "vt_lite.cu": ["--use_fast_math"]}


def nvcc() -> str:
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: libvtwin.so cannot be built")


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _newest_dep():
    return max(os.path.getmtime(os.path.join(CSRC, f)) for f in os.listdir(CSRC)) if os.listdir(CSRC) else 0


def needs_build() -> bool:
    if not os.path.exists(LIB):
        return True
    inc = os.path.join(ROOT, "..", "include", "vtwin.h")
    return os.path.getmtime(LIB) < max(_newest_dep(), os.path.getmtime(inc))


def _compile(src: str, verbose_ptxas: bool) -> str:
    out = os.path.join(OBJ, src + ".o")
    cmd = [nvcc(), *ARCH, *COMMON, *EXTRA.get(src, []), "-c", os.path.join(CSRC, src), "-o", out]
    if verbose_ptxas and src.endswith(".cu"):
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}")
    if verbose_ptxas and r.stderr:
        sys.stderr.write(r.stderr)
    return out


def build(force: bool = False, verbose_ptxas: bool = False) -> str:
    if not force and not needs_build():
        return LIB
    os.makedirs(OBJ, exist_ok=True)
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose_ptxas), srcs))
    tmp = LIB + ".tmp"
    r = subprocess.run([nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lpthread"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv))
