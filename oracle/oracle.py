"""ctypes wrapper around oracle/gvr_oracle.c -- the CPU restatement of the
reference renderer (cpp/src/Renderer/CUDABasedRasterization.cu:23-408 and
CUDABasedRasterizationGrad.cu:114-617).  Test infrastructure only: tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg call it as the checker.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "liboracle.so")

ALBEDO = {"vertexColor": 0, "textured": 1, "normal": 2, "lighting": 3, "foregroundMask": 4, "texturedBilinear": 5,
          "uv": 6}
SHADING = {"shaded": 0, "shadeless": 1, "phong": 2}


class _Scene(ctypes.Structure):
    _fields_ = [
        ("N", ctypes.c_int), ("F", ctypes.c_int), ("C", ctypes.c_int), ("W", ctypes.c_int),
        ("H", ctypes.c_int), ("Ht", ctypes.c_int), ("Wt", ctypes.c_int),
        ("albedo_mode", ctypes.c_int), ("shading_mode", ctypes.c_int), ("image_filter_size", ctypes.c_int),
        ("faces", ctypes.c_void_p), ("uvs", ctypes.c_void_p), ("verts", ctypes.c_void_p),
        ("colors", ctypes.c_void_p), ("texture", ctypes.c_void_p), ("sh", ctypes.c_void_p),
        ("extr", ctypes.c_void_p), ("intr", ctypes.c_void_p), ("rays", ctypes.c_void_p),
    ]


def build(force: bool = False) -> str:
    """Compile liboracle.so with the committed Makefile (gcc, OpenMP)."""
    src = os.path.join(_HERE, "gvr_oracle.c")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE, "-B", "liboracle.so"], check=True)
    return _LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        P = ctypes.c_void_p
        L.orc_forward.argtypes = [ctypes.POINTER(_Scene), P, P, P, P, P, P, P]
        L.orc_forward.restype = None
        L.orc_backward.argtypes = [ctypes.POINTER(_Scene), P, P, P, P, P, P, P, P, P, P]
        L.orc_backward.restype = None
        L.orc_backward_ex.argtypes = [ctypes.POINTER(_Scene), P, P, P, P, P, P, P, P, P, P, ctypes.c_int]
        L.orc_backward_ex.restype = None
        L.orc_rays.argtypes = [ctypes.POINTER(_Scene), P]
        L.orc_project.argtypes = [ctypes.POINTER(_Scene), ctypes.c_int, P, P]
        L.orc_camera.argtypes = [P, P, P, P]
        L.orc_render_fp64.argtypes = [ctypes.POINTER(_Scene), P, P, P, P]
        L.orc_render_fp64.restype = None
        L.orc_render_fp64_ex.argtypes = [ctypes.POINTER(_Scene), P, P, P, P, P, P]
        L.orc_render_fp64_ex.restype = None
        L.orc_uv_face_map.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_int, P, P]
        L.orc_uv_face_map.restype = None
        L.orc_normal_map_from.argtypes = [P, P, P, P, ctypes.c_int, ctypes.c_int, P]
        L.orc_normal_map_from.restype = None
        L.orc_normal_map.argtypes = [ctypes.POINTER(_Scene), P]
        L.orc_normal_map.restype = None
        L.orc_max_ties.restype = ctypes.c_int
        L.orc_num_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _ptr(a):
    return None if a is None else a.ctypes.data


class OracleScene:
    """One batch element of a scene, held as contiguous numpy arrays."""

    def __init__(self, faces, uvs, verts, colors, texture, sh, extr, intr, width, height,
                 albedo_mode="vertexColor", shading_mode="shaded", image_filter_size=1, rays=None):
        self.faces = np.ascontiguousarray(faces, dtype=np.int32).reshape(-1, 3)
        self.uvs = _f32(uvs).reshape(-1, 6)
        self.verts = _f32(verts).reshape(-1, 3)
        self.colors = _f32(colors).reshape(-1, 3)
        self.texture = _f32(texture)
        self.sh = _f32(sh).reshape(-1, 27)
        self.extr = _f32(extr).reshape(-1, 12)
        self.intr = _f32(intr).reshape(-1, 9)
        self.rays = None if rays is None else _f32(rays)
        self.W, self.H = int(width), int(height)
        self.albedo_mode, self.shading_mode = albedo_mode, shading_mode
        self.image_filter_size = int(image_filter_size)
        self.N, self.F, self.C = self.verts.shape[0], self.faces.shape[0], self.extr.shape[0]
        self.Ht, self.Wt = self.texture.shape[0], self.texture.shape[1]

    def _struct(self):
        s = _Scene()
        s.N, s.F, s.C, s.W, s.H, s.Ht, s.Wt = self.N, self.F, self.C, self.W, self.H, self.Ht, self.Wt
        s.albedo_mode = ALBEDO[self.albedo_mode]
        s.shading_mode = SHADING[self.shading_mode]
        s.image_filter_size = self.image_filter_size
        s.faces, s.uvs, s.verts = _ptr(self.faces), _ptr(self.uvs), _ptr(self.verts)
        s.colors, s.texture, s.sh = _ptr(self.colors), _ptr(self.texture), _ptr(self.sh)
        s.extr, s.intr, s.rays = _ptr(self.extr), _ptr(self.intr), _ptr(self.rays)
        return s

    def forward(self):
        C, H, W, N = self.C, self.H, self.W, self.N
        T = lib().orc_max_ties()
        out = dict(
            face=np.empty((C, H, W), np.int32), bary=np.empty((C, H, W, 2), np.float32),
            render=np.empty((C, H, W, 3), np.float64), vertex_normal=np.empty((C, N, 3), np.float32),
            depth=np.empty((C, H, W), np.int32), ties=np.empty((C, H, W), np.int32),
            tie_faces=np.empty((C, H, W, T), np.int32))
        s = self._struct()
        lib().orc_forward(ctypes.byref(s), _ptr(out["face"]), _ptr(out["bary"]), _ptr(out["render"]),
                          _ptr(out["vertex_normal"]), _ptr(out["depth"]), _ptr(out["ties"]),
                          _ptr(out["tie_faces"]))
        return out

    def backward(self, face, bary, vertex_normal, grad_render, target, grad_target, flags=0):
        """flags & 1: also the vertex colour's change through the barycentrics
        (the GVR_BACKWARD_ALBEDO_POSITION option)."""
        N, C = self.N, self.C
        face = np.ascontiguousarray(face, np.int32)
        bary, vertex_normal = _f32(bary), _f32(vertex_normal)
        grad_render, target, grad_target = _f32(grad_render), _f32(target), _f32(grad_target)
        out = dict(vertex_pos_grad=np.empty((N, 3)), vertex_color_grad=np.empty((N, 3)),
                   texture_grad=np.empty((self.Ht, self.Wt, 3)), sh_coeff_grad=np.empty((C, 27)))
        s = self._struct()
        lib().orc_backward_ex(ctypes.byref(s), _ptr(face), _ptr(bary), _ptr(vertex_normal), _ptr(grad_render),
                              _ptr(target), _ptr(grad_target), _ptr(out["vertex_pos_grad"]),
                              _ptr(out["vertex_color_grad"]), _ptr(out["texture_grad"]), _ptr(out["sh_coeff_grad"]),
                              int(flags))
        return out

    def render_fp64(self, face, verts_d=None, colors_d=None, sh_d=None):
        """FP64 render at fixed visibility `face` [C,H,W]; returns (render, flags).
        `verts_d` [N,3], `colors_d` [N,3] and `sh_d` [C,27] optionally give
        FP64 values in place of the scene's FP32 arrays.  flags per pixel:
        1 normal flipped toward the camera, 2 grazing face, 4 interpolated
        normal within 0.01 of perpendicular to the ray (a small input change
        can flip it) -- pixels where finite differences are not meaningful."""
        face = np.ascontiguousarray(face, np.int32)
        dbl = lambda a: None if a is None else np.ascontiguousarray(a, np.float64).reshape(-1)
        vd, cd, sd = dbl(verts_d), dbl(colors_d), dbl(sh_d)
        out = np.empty((self.C, self.H, self.W, 3), np.float64)
        flags = np.empty((self.C, self.H, self.W), np.int32)
        s = self._struct()
        lib().orc_render_fp64_ex(ctypes.byref(s), _ptr(vd), _ptr(cd), _ptr(sd), _ptr(face), _ptr(out), _ptr(flags))
        return out, flags

    def with_(self, **kw):
        """Copy of this scene with some arrays replaced (finite differences)."""
        o = OracleScene.__new__(OracleScene)
        o.__dict__.update(self.__dict__)
        for k, v in kw.items():
            setattr(o, k, v if k in ("albedo_mode", "shading_mode") else _f32(v).reshape(getattr(self, k).shape))
        return o

    def rays_fp32(self):
        out = np.empty((self.C, self.H, self.W, 3), np.float32)
        s = self._struct()
        lib().orc_rays(ctypes.byref(s), _ptr(out))
        return out

    def normal_map(self):
        """[Ht, Wt, 3] texture-space normal map of the normal-map mode (FP32)."""
        out = np.empty((self.Ht, self.Wt, 3), np.float32)
        s = self._struct()
        lib().orc_normal_map(ctypes.byref(s), _ptr(out))
        return out

    def project(self, c):
        proj = np.empty((self.N, 3), np.float32)
        bbox = np.empty((self.F, 4), np.int32)
        s = self._struct()
        lib().orc_project(ctypes.byref(s), int(c), _ptr(proj), _ptr(bbox))
        return proj, bbox


def camera_inverse(extr12, intr9):
    """FP32 (invE, invP) of one camera, as CUDABasedRasterization.cu:23-67 computes them."""
    e, k = _f32(extr12).reshape(12), _f32(intr9).reshape(9)
    invE, invP = np.empty(16, np.float32), np.empty(16, np.float32)
    lib().orc_camera(_ptr(e), _ptr(k), _ptr(invE), _ptr(invP))
    return invE.reshape(4, 4), invP.reshape(4, 4)


def uv_face_map(uvs, Ht, Wt):
    """(owner [Ht,Wt] int32, -1 = uncovered; abc [Ht,Wt,3]) of the normal-map
    mode's texture-space raster (CUDABasedRasterization.cpp:241-294)."""
    uvs = _f32(uvs).reshape(-1)
    F = uvs.size // 6
    owner = np.empty((Ht, Wt), np.int32)
    abc = np.empty((Ht, Wt, 3), np.float32)
    lib().orc_uv_face_map(_ptr(uvs), F, int(Ht), int(Wt), _ptr(owner), _ptr(abc))
    return owner, abc


def normal_map_from(faces, vertex_normal, owner, abc):
    """renderNormalMapDevice (CUDABasedRasterization.cu:415-445) for a face map."""
    faces = np.ascontiguousarray(faces, np.int32).reshape(-1)
    vn = _f32(vertex_normal).reshape(-1)
    owner = np.ascontiguousarray(owner, np.int32)
    abc = _f32(abc)
    Ht, Wt = owner.shape
    out = np.empty((Ht, Wt, 3), np.float32)
    lib().orc_normal_map_from(_ptr(faces), _ptr(vn), _ptr(owner), _ptr(abc), int(Ht), int(Wt), _ptr(out))
    return out


def num_threads() -> int:
    return int(lib().orc_num_threads())
