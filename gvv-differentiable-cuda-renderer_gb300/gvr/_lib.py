"""ctypes binding of libgvr.so (include/gvr.h).  There is no fallback: if the
library is missing or fails to load, every call raises."""
from __future__ import annotations

import ctypes
import os

from . import native_build as _build

P = ctypes.c_void_p
I32 = ctypes.c_int32

OK = 0
STATUS = {0: "GVR_OK", -1: "GVR_ERR_INVALID_ARGUMENT", -2: "GVR_ERR_CUDA", -3: "GVR_ERR_OUT_OF_MEMORY",
          -4: "GVR_ERR_WORKSPACE", -5: "GVR_ERR_UNSUPPORTED"}
# the reference's modes, then texturedBilinear, uv and phong (include/gvr.h)
ALBEDO = {"vertexColor": 0, "textured": 1, "normal": 2, "lighting": 3, "foregroundMask": 4, "texturedBilinear": 5,
          "uv": 6}
SHADING = {"shaded": 0, "shadeless": 1, "phong": 2}


class GvrTopology(ctypes.Structure):
    _fields_ = [("faces", P), ("texture_coordinates", P), ("num_faces", I32), ("num_vertices", I32)]


class GvrAttrs(ctypes.Structure):
    _fields_ = [("num_cameras", I32), ("render_resolution_u", I32), ("render_resolution_v", I32),
                ("albedo_mode", I32), ("shading_mode", I32), ("image_filter_size", I32),
                ("texture_filter_size", I32), ("compute_normal_map", I32)]


class GvrForwardArgs(ctypes.Structure):
    _fields_ = [("batch", I32), ("texture_height", I32), ("texture_width", I32),
                ("vertex_pos", P), ("vertex_color", P), ("texture", P), ("sh_coeff", P), ("target_image", P),
                ("extrinsics", P), ("intrinsics", P),
                ("barycentric", P), ("face", P), ("render", P), ("vertex_normal", P), ("target_image_out", P),
                ("normal_map", P), ("workspace", P), ("workspace_bytes", ctypes.c_size_t)]


class GvrBackwardArgs(ctypes.Structure):
    _fields_ = [("batch", I32), ("texture_height", I32), ("texture_width", I32),
                ("render_grad", P), ("vertex_pos", P), ("vertex_color", P), ("texture", P), ("sh_coeff", P),
                ("target_image", P), ("vertex_normal", P), ("barycentric", P), ("face", P), ("target_grad", P),
                ("extrinsics", P), ("intrinsics", P),
                ("vertex_pos_grad", P), ("vertex_color_grad", P), ("texture_grad", P), ("sh_coeff_grad", P),
                ("workspace", P), ("workspace_bytes", ctypes.c_size_t), ("flags", I32)]


BACKWARD_ALBEDO_POSITION = 1  # GVR_BACKWARD_ALBEDO_POSITION


class GvrJob(ctypes.Structure):
    _fields_ = [("handle", P), ("forward", GvrForwardArgs), ("tile_width", I32), ("big_tiles", I32)]


PLAN_AUTOTUNE = 1
PLAN_PERSISTENT = 2
PLAN_LANES = 16


class GvrKernelTime(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * 48), ("launches", ctypes.c_longlong), ("total_ms", ctypes.c_double)]


# Every symbol include/gvr.h declares.
EXPORTS = ("gvr_create", "gvr_destroy", "gvr_forward", "gvr_backward", "gvr_forward_workspace_size",
           "gvr_backward_workspace_size", "gvr_last_error", "gvr_abi_version", "gvr_debug_rays",
           "gvr_profile_enable", "gvr_profile_read", "gvr_launch_count", "gvr_probe_reductions", "gvr_backward_noalloc",
           "gvr_plan_create", "gvr_plan_forward", "gvr_plan_forward_graph", "gvr_plan_tile_config",
           "gvr_plan_bind_backward", "gvr_plan_backward", "gvr_plan_backward_graph", "gvr_plan_destroy", "gvr_image_gradient", "gvr_image_gaussian3x3",
           # include/gvr_nn.h
           "gvr_gemm_bf16", "gvr_tc_error", "gvr_tc_wait_probe", "gvr_im2col_3x3s2", "gvr_col2im_3x3s2", "gvr_nn_last_error")

NOALLOC_SCRATCH_BYTES = 32 << 20  # GVR_NOALLOC_SCRATCH_BYTES

_lib = None


def load(build_if_missing: bool = True):
    """Load libgvr.so (building it first when it is absent)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB_PATH
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(f"libgvr.so not built ({path}); run gvr.build()")
        _build.build()
    L = ctypes.CDLL(path)
    L.gvr_create.argtypes = [ctypes.POINTER(GvrTopology), ctypes.POINTER(GvrAttrs), ctypes.POINTER(P)]
    L.gvr_create.restype = ctypes.c_int
    L.gvr_destroy.argtypes = [P]
    L.gvr_destroy.restype = None
    L.gvr_forward.argtypes = [P, ctypes.POINTER(GvrForwardArgs), P]
    L.gvr_forward.restype = ctypes.c_int
    L.gvr_backward.argtypes = [P, ctypes.POINTER(GvrBackwardArgs), P]
    L.gvr_backward.restype = ctypes.c_int
    L.gvr_forward_workspace_size.argtypes = [P, I32, I32, I32]
    L.gvr_forward_workspace_size.restype = ctypes.c_size_t
    L.gvr_backward_workspace_size.argtypes = [P, I32, I32, I32]
    L.gvr_backward_workspace_size.restype = ctypes.c_size_t
    L.gvr_last_error.argtypes = []
    L.gvr_last_error.restype = ctypes.c_char_p
    L.gvr_abi_version.restype = ctypes.c_int
    L.gvr_debug_rays.argtypes = [P, I32, P, P, P, P]
    L.gvr_debug_rays.restype = ctypes.c_int
    L.gvr_profile_enable.argtypes = [ctypes.c_int]
    L.gvr_profile_enable.restype = ctypes.c_int
    L.gvr_profile_read.argtypes = [ctypes.POINTER(GvrKernelTime), ctypes.c_int]
    L.gvr_profile_read.restype = ctypes.c_int
    L.gvr_launch_count.argtypes = []
    L.gvr_launch_count.restype = ctypes.c_longlong
    L.gvr_probe_reductions.argtypes = [P, ctypes.c_longlong, ctypes.c_int, ctypes.c_int, ctypes.c_int, P]
    L.gvr_probe_reductions.restype = ctypes.c_int
    L.gvr_backward_noalloc.argtypes = [P, ctypes.POINTER(GvrBackwardArgs), P]
    L.gvr_backward_noalloc.restype = ctypes.c_int
    L.gvr_plan_create.argtypes = [ctypes.POINTER(GvrJob), I32, I32, ctypes.POINTER(P)]
    L.gvr_plan_create.restype = ctypes.c_int
    L.gvr_plan_forward.argtypes = [P, P]
    L.gvr_plan_forward.restype = ctypes.c_int
    L.gvr_plan_forward_graph.argtypes = [P, P]
    L.gvr_plan_forward_graph.restype = ctypes.c_int
    I32P = ctypes.POINTER(I32)
    L.gvr_plan_tile_config.argtypes = [P, I32, I32P, I32P, I32P]
    L.gvr_plan_tile_config.restype = ctypes.c_int
    L.gvr_plan_bind_backward.argtypes = [P, ctypes.POINTER(GvrBackwardArgs), I32]
    L.gvr_plan_bind_backward.restype = ctypes.c_int
    L.gvr_plan_backward.argtypes = [P, P]
    L.gvr_plan_backward.restype = ctypes.c_int
    L.gvr_plan_backward_graph.argtypes = [P, P]
    L.gvr_plan_backward_graph.restype = ctypes.c_int
    L.gvr_plan_destroy.argtypes = [P]
    L.gvr_plan_destroy.restype = None
    L.gvr_image_gradient.argtypes = [P, P, P, I32, I32, I32, P]
    L.gvr_image_gradient.restype = ctypes.c_int
    L.gvr_image_gaussian3x3.argtypes = [P, P, I32, I32, I32, P]
    L.gvr_image_gaussian3x3.restype = ctypes.c_int
    _lib = L
    return L


def profile_read():
    """{kernel name: (launches, total_ms)} since the last profile_enable()."""
    L = load()
    n = L.gvr_profile_read(None, 0)
    arr = (GvrKernelTime * max(n, 1))()
    n = L.gvr_profile_read(arr, n)
    return {arr[i].name.decode(): (int(arr[i].launches), float(arr[i].total_ms)) for i in range(n)}


class GvrError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


def check(status: int):
    if status != OK:
        raise GvrError(status, load().gvr_last_error().decode("utf-8", "replace"))
