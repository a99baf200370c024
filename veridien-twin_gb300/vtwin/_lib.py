"""Loads libvtwin.so (built in-tree by vtwin.build). There is no CPU fallback: if the library is missing this
raises, and every GPU entry point of the library returns VT_ERR_NO_DEVICE without a CUDA device."""
from __future__ import annotations

import ctypes as C
import os

from . import _abi as A

PKG = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(PKG, "libvtwin.so")

# every entry point of include/vtwin.h with its ctypes signature
SIGNATURES = {
    "vt_create": (C.c_int32, [C.POINTER(A.vt_scene_desc), C.POINTER(A.vt_options), C.POINTER(C.c_void_p)]),
    "vt_destroy": (C.c_int32, [C.c_void_p]),
    "vt_last_error": (C.c_char_p, [C.c_void_p]),
    "vt_scene_info_get": (C.c_int32, [C.c_void_p, C.POINTER(A.vt_scene_info)]),
    "vt_scene_export": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "vt_blas_info_get": (C.c_int32, [C.c_void_p, C.c_uint32, C.POINTER(A.vt_blas_info)]),
    "vt_set_poses": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32]),
    "vt_set_eavg": (C.c_int32, [C.c_void_p, C.c_void_p]),
    "vt_scene_uniform_get": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "vt_set_node_state": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_uint32]),
    "vt_trace_rays": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32,
                                  C.c_void_p, C.c_void_p]),
    "vt_unit_test": (C.c_int32, [C.c_void_p, C.POINTER(A.vt_unit_req), C.c_void_p, C.c_void_p]),
    "vt_visible": (C.c_int32, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_double, C.c_double, C.c_void_p]),
    "vt_project": (C.c_int32, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_void_p]),
    "vt_render_camera": (C.c_int32, [C.c_void_p, C.POINTER(A.vt_render_req), C.c_void_p]),
    "vt_readback": (C.c_int32, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p, C.c_size_t]),
    "vt_sensor_expose": (C.c_int32, [C.c_void_p, C.POINTER(A.vt_sensor_uniform), C.c_void_p, C.c_void_p]),
    "vt_sensor_camera": (C.c_int32, [C.c_void_p, C.c_uint32, C.POINTER(A.vt_sensor_uniform), C.c_float]),
    "vt_sensor_frame": (C.c_int32, [C.c_void_p, C.c_uint32, C.POINTER(A.vt_sensor_uniform), C.c_void_p]),
    "vt_render_frame": (C.c_int32, [C.c_void_p, C.POINTER(A.vt_frame_req)]),
    "vt_weld": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.POINTER(A.vt_mesh_out)]),
    "vt_subdivide": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_double, C.c_uint32, C.POINTER(A.vt_mesh_out)]),
    "vt_weld_device": (C.c_int32, [C.c_int32, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.POINTER(A.vt_mesh_out)]),
    "vt_subdivide_device": (C.c_int32, [C.c_int32, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_double, C.c_uint32,
                                        C.POINTER(A.vt_mesh_out)]),
    "vt_bench_mesh": (C.c_int32, [C.c_double, C.c_void_p, C.c_void_p, C.c_double, C.POINTER(A.vt_mesh_out)]),
    "vt_compute_normals": (C.c_int32, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_void_p]),
    "vt_mesh_free": (None, [C.POINTER(A.vt_mesh_out)]),
    "vt_lite_create": (C.c_int32, [C.c_void_p, C.POINTER(A.vt_lite_opts), C.POINTER(A.vt_lite_info)]),
    "vt_lite_info_get": (C.c_int32, [C.c_void_p, C.POINTER(A.vt_lite_info)]),
    "vt_lite_geometry": (C.c_int32, [C.POINTER(A.vt_scene_desc), C.c_double, C.c_double, C.c_void_p, C.c_void_p, C.c_void_p]),
    "vt_lite_render_camera": (C.c_int32, [C.c_void_p, C.c_uint32, C.c_void_p]),
    "vt_lite_display": (C.c_int32, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p]),
    "vt_lite_readback": (C.c_int32, [C.c_void_p, C.c_uint32, C.c_int, C.c_void_p, C.c_size_t]),
    "vt_lite_debug": (C.c_int32, [C.c_void_p, C.c_int, C.c_uint32, C.c_void_p, C.c_size_t]),
    "vt_raster": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32,
                              C.c_void_p]),
    "vt_set_relative_illumination": (C.c_int32, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_double, C.c_void_p, C.c_void_p, C.c_uint32]),
    "vt_get_relative_illumination": (C.c_int32, [C.c_void_p, C.c_uint32, C.c_void_p]),
    "vt_calib_setup": (C.c_int32, [C.c_void_p, C.POINTER(A.vt_calib_desc), C.POINTER(A.vt_calib_info)]),
    "vt_calib_export": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "vt_calib_forward": (C.c_int32, [C.c_void_p, C.POINTER(A.vt_calib_req), C.POINTER(C.c_double)]),
    "vt_calib_backward": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "vt_calib_intrinsics_grad": (C.c_int32, [C.c_void_p, C.c_void_p]),
    "vt_calib_export_paths": (C.c_int32, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p]),
    "vt_set_camera_intrinsics": (C.c_int32, [C.c_void_p, C.c_uint32, C.c_void_p]),
    "vt_get_camera_intrinsics": (C.c_int32, [C.c_void_p, C.c_uint32, C.c_void_p]),
    "vt_reproj_loss": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_void_p, C.POINTER(C.c_double),
                                   C.c_void_p]),
    "vt_kernel_profile": (C.c_int32, [C.c_void_p, C.c_int32, C.c_int32]),
    "vt_render_batch": (C.c_int32, [C.c_void_p, C.POINTER(A.vt_batch_req), C.c_void_p, C.c_void_p, C.POINTER(A.vt_batch_stats)]),
    "vt_batch_autotune": (C.c_int32, [C.c_void_p, C.POINTER(A.vt_batch_req), C.POINTER(A.vt_tune_row), C.c_uint32,
                                      C.POINTER(C.c_uint32), C.POINTER(A.vt_tune_row)]),
    "vt_radiosity_solve": (C.c_int32, [C.c_void_p, C.POINTER(A.vt_solve_req)]),
    "vt_form_factors": (C.c_int32, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "vt_form_factors_visible": (C.c_int32, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p]),
    "vt_nodes_build": (C.c_int32, [C.c_void_p, C.POINTER(A.vt_nodes_opts), C.POINTER(A.vt_nodes_info)]),
    "vt_nodes_direct": (C.c_int32, [C.c_void_p, C.c_uint32]),
    "vt_nodes_jacobi": (C.c_int32, [C.c_void_p, C.c_uint32]),
    "vt_nodes_update": (C.c_int32, [C.c_void_p, C.c_int, C.POINTER(C.c_uint32)]),
    "vt_converge": (C.c_int32, [C.c_void_p, C.c_uint32]),
    "vt_node_summary": (C.c_int32, [C.c_void_p, C.c_void_p]),
    "vt_nodes_export": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "vt_get_node_state": (C.c_int32, [C.c_void_p, C.c_void_p, C.POINTER(C.c_uint32)]),
    "vt_radiosity_solve_static": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32,
                                              C.c_double, C.c_void_p, C.POINTER(C.c_uint32), C.POINTER(C.c_double)]),
    "vt_bvh_capacity": (C.c_uint32, [C.c_uint32, C.c_uint32]),
    "vt_bvh_build": (C.c_int32, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p,
                                 C.POINTER(A.vt_bvh_result)]),
    "vt_bvh_build_device": (C.c_int32, [C.c_int32, C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p,
                                        C.c_void_p, C.POINTER(A.vt_bvh_result)]),
    "vt_debug_flags": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_int]),
    "vt_timings_get": (C.c_int32, [C.c_void_p, C.POINTER(A.vt_timings)]),
    "vt_stream": (C.c_void_p, [C.c_void_p]),
    "vt_wait_check": (C.c_int32, [C.c_void_p, C.c_uint64, C.c_int]),
}

_lib = None


class VtError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"vtwin status {status}: {msg}")
        self.status = status


def load(build_if_missing: bool = True):
    """The loaded library. Builds it first when missing (needs nvcc); raises if it cannot be loaded."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB):
        if not build_if_missing:
            raise RuntimeError(f"{LIB} is not built: run `python -c 'import __graft_entry__ as g; g.build()'`")
        from . import build
        build.build()
    lib = C.CDLL(LIB)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def check(status: int, ctx=None):
    if status != A.VT_OK:
        msg = load().vt_last_error(ctx).decode(errors="replace") if ctx is not None else ""
        raise VtError(status, msg)
