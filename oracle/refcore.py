"""Runs the reference's own CUDA kernels on the GPU (test infrastructure only).

Build recipe (build_fatbins, only where the reference sources are present):
  nvcc -fatbin for sm_103a of cpp/src/Renderer/CUDABasedRasterization.cu and
  CUDABasedRasterizationGrad.cu, once with nvcc's default flags and once with
  -fmad=false, plus the one compile shim the CUDA 13 toolkit needs
  (-DclockRate=l2CacheSize: cudaDeviceProp::clockRate, read only by a
  device-selection helper of the vendored cutil headers, no longer exists).
  Outputs go to oracle/_ref/ (git-ignored; device code only, so the same
  files load on any host architecture).  layout_probe.cu is compiled against
  the reference headers to record the byte layout of its kernel parameter
  structs in oracle/_ref/layout.json.
The harness (refcore/refcore.cu, our code) is compiled on every machine by
build_harness() into oracle/_ref/librefcore.so.
"""
from __future__ import annotations

import ctypes
import json
import os
import shutil
import subprocess

import numpy as np

from .refsrc import reference_path

_HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(_HERE, "_ref")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FATBINS = {"fwd": "CUDABasedRasterization.cu", "bwd": "CUDABasedRasterizationGrad.cu"}


def _nvcc():
    return shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"


def _fatbin(kind, fmad):
    return os.path.join(REF_DIR, f"ref_{kind}{'' if fmad else '_nofma'}.fatbin")


def build_fatbins():
    """Compile the reference kernels (needs the reference sources)."""
    src = reference_path("cpp", "src")
    if not os.path.isdir(src):
        return False
    os.makedirs(REF_DIR, exist_ok=True)
    inc = ["-I", reference_path("cpp", "thirdParty", "Shared", "cutil", "inc"), "-I",
           os.path.join(src, "Utils"), "-I", os.path.join(src, "Renderer")]
    for kind, fname in FATBINS.items():
        for fmad in (True, False):
            out = _fatbin(kind, fmad)
            cmd = [_nvcc(), "-fatbin", *ARCH, "-DclockRate=l2CacheSize", *inc, "-o", out,
                   os.path.join(src, "Renderer", fname)]
            if not fmad:
                cmd.insert(2, "-fmad=false")
            subprocess.run(cmd, check=True, capture_output=True)
    probe = os.path.join(REF_DIR, "layout_probe")
    subprocess.run([_nvcc(), "-DclockRate=l2CacheSize", *inc, "-o", probe,
                    os.path.join(_HERE, "refcore", "layout_probe.cu")], check=True, capture_output=True)
    layout = subprocess.run([probe], check=True, capture_output=True, text=True).stdout
    with open(os.path.join(REF_DIR, "layout.json"), "w") as fh:
        fh.write(layout)
    os.remove(probe)
    return True


def build_harness():
    os.makedirs(REF_DIR, exist_ok=True)
    out = os.path.join(REF_DIR, "librefcore.so")
    src = os.path.join(_HERE, "refcore", "refcore.cu")
    if os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(src):
        return out
    cuda_lib = os.path.join(os.path.dirname(os.path.dirname(_nvcc())), "lib64")
    subprocess.run([_nvcc(), *ARCH, "-O2", "-std=c++17", "-Xcompiler", "-fPIC", "-shared", "-o", out, src,
                    "-L", os.path.join(cuda_lib, "stubs"), "-lcuda"], check=True, capture_output=True)
    return out


def build_layout_lib():
    """The harness's struct-layout table alone (no CUDA driver needed to load it)."""
    os.makedirs(REF_DIR, exist_ok=True)
    out = os.path.join(REF_DIR, "librefcore_layout.so")
    src = os.path.join(_HERE, "refcore", "refcore.cu")
    if os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(src):
        return out
    subprocess.run([_nvcc(), *ARCH, "-DREFCORE_LAYOUT_ONLY", "-std=c++17", "-Xcompiler", "-fPIC", "-shared", "-o",
                    out, src], check=True, capture_output=True)
    return out


def harness_layout():
    """{"fwd": {field: offset}, "bwd": {...}} of the harness's struct replicas."""
    L = ctypes.CDLL(build_layout_lib())
    L.refcore_layout.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_char_p), ctypes.POINTER(ctypes.c_longlong),
                                 ctypes.c_int]
    out = {}
    for which, key in ((0, "fwd"), (1, "bwd")):
        names = (ctypes.c_char_p * 64)()
        offs = (ctypes.c_longlong * 64)()
        n = L.refcore_layout(which, names, offs, 64)
        out[key] = {names[i].decode(): int(offs[i]) for i in range(n)}
    return out


UVMAP_LIB = os.path.join(REF_DIR, "libref_uvmap.so")


def build_uvmap_ref():
    """Host library around the reference's rayTriangleIntersectHost: g++ on
    cpp/src/Renderer/CUDABasedRasterization.cpp (unchanged, plus the same
    clockRate shim) and refcore/uvmap_ref.cpp.  Only where the reference
    sources are present; needs no GPU."""
    src = reference_path("cpp", "src")
    if not os.path.isdir(src):
        return False
    os.makedirs(REF_DIR, exist_ok=True)
    cuda = os.path.dirname(os.path.dirname(_nvcc()))
    inc = ["-I", os.path.join(cuda, "include"), "-I",
           reference_path("cpp", "thirdParty", "Shared", "cutil", "inc"), "-I", os.path.join(src, "Utils"),
           "-I", os.path.join(src, "Renderer")]
    subprocess.run(["g++", "-O2", "-fPIC", "-fopenmp", "-w", "-shared", "-DclockRate=l2CacheSize", *inc, "-o",
                    UVMAP_LIB, os.path.join(src, "Renderer", "CUDABasedRasterization.cpp"),
                    os.path.join(_HERE, "refcore", "uvmap_ref.cpp"), "-L", os.path.join(cuda, "lib64"), "-lcudart"],
                   check=True, capture_output=True)
    return True


def uv_face_map_reference(uvs, Ht, Wt):
    """(owner, abc) from the reference's own host test (see build_uvmap_ref)."""
    L = ctypes.CDLL(UVMAP_LIB)
    P = ctypes.c_void_p
    L.refuv_face_map.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_int, P, P]
    L.refuv_face_map.restype = None
    uvs = np.ascontiguousarray(uvs, np.float32).reshape(-1)
    owner = np.empty((Ht, Wt), np.int32)
    abc = np.empty((Ht, Wt, 3), np.float32)
    L.refuv_face_map(uvs.ctypes.data, uvs.size // 6, int(Ht), int(Wt), owner.ctypes.data, abc.ctypes.data)
    return owner, abc


def build_if_possible():
    for step in (build_fatbins, build_harness, build_layout_lib, build_uvmap_ref):
        try:
            step()
        except (subprocess.CalledProcessError, OSError):
            pass


def available():
    return all(os.path.exists(p) for p in (_fatbin("fwd", True), _fatbin("bwd", True), _fatbin("fwd", False),
                                           _fatbin("bwd", False), os.path.join(REF_DIR, "layout.json")))


class Refcore:
    """The reference kernels of one build (fmad=True: nvcc defaults; False: -fmad=false)."""

    def __init__(self, fmad=False):
        lib_path = build_harness()
        L = ctypes.CDLL(lib_path)
        P = ctypes.c_void_p
        I = ctypes.c_int
        L.refcore_open.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(P)]
        L.refcore_error.restype = ctypes.c_char_p
        L.refcore_close.argtypes = [P]
        L.refcore_forward.argtypes = [P, P, P] + [I] * 9 + [P] * 10 + [P]
        L.refcore_backward.argtypes = [P, P, P] + [I] * 11 + [P] * 16 + [P]
        L.refcore_layout.argtypes = [I, ctypes.POINTER(ctypes.c_char_p), ctypes.POINTER(ctypes.c_longlong), I]
        L.refcore_normal_map.argtypes = [P, P, I, I, I, I, P, P, P]
        self.L = L
        self._check_layout()
        h = P()
        rc = L.refcore_open(_fatbin("fwd", fmad).encode(), _fatbin("bwd", fmad).encode(), ctypes.byref(h))
        if rc != 0:
            raise RuntimeError("refcore_open: " + L.refcore_error().decode())
        self.h = h

    def _check_layout(self):
        ref = json.load(open(os.path.join(REF_DIR, "layout.json")))
        if harness_layout() != ref:
            raise RuntimeError("parameter struct layout differs from the reference header")

    def close(self):
        if getattr(self, "h", None):
            self.L.refcore_close(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def forward(self, s, b=0, albedo=None, shading=None):
        """One batch element of scene dict `s` (numpy) through the reference
        forward kernels.  Returns numpy face, bary, render, vertex_normal, ms."""
        import torch
        dev = torch.device("cuda", torch.cuda.current_device())
        albedo = albedo or s["albedo_mode"]
        shading = shading or s["shading_mode"]
        if albedo == "foregroundMask":
            shading = "shadeless"      # CudaRenderer.cpp:72-76
        A = {"vertexColor": 0, "textured": 1, "normal": 2, "lighting": 3, "foregroundMask": 4}[albedo]
        S = {"shaded": 0, "shadeless": 1}[shading]
        t = {k: torch.from_numpy(np.ascontiguousarray(s[k][b])).to(dev)
             for k in ("vertex_pos", "vertex_color", "texture", "sh_coeff", "extrinsics", "intrinsics")}
        C, H, W, N = s["num_views"], s["height"], s["width"], s["num_vertices"]
        faces = np.ascontiguousarray(s["faces"], np.int32)
        uvs = np.ascontiguousarray(s["uvs"], np.float32)
        F = faces.shape[0]
        Ht, Wt = t["texture"].shape[0], t["texture"].shape[1]
        face = torch.empty((C, H, W), dtype=torch.int32, device=dev)
        bary = torch.empty((C, H, W, 2), device=dev)
        img = torch.empty((C, H, W, 3), device=dev)
        vn = torch.empty((C, N, 3), device=dev)
        ms = ctypes.c_float()
        p = lambda x: ctypes.c_void_p(x.data_ptr())
        rc = self.L.refcore_forward(self.h, faces.ctypes.data, uvs.ctypes.data, N, F, C, W, H, A, S, Ht, Wt,
                                    p(t["vertex_pos"]), p(t["vertex_color"]), p(t["texture"]), p(t["sh_coeff"]),
                                    p(t["extrinsics"]), p(t["intrinsics"]), p(face), p(bary), p(img), p(vn),
                                    ctypes.byref(ms))
        if rc != 0:
            raise RuntimeError("refcore_forward: " + self.L.refcore_error().decode())
        return dict(face=face.cpu().numpy(), bary=bary.cpu().numpy(), render=img.cpu().numpy(),
                    vertex_normal=vn.cpu().numpy(), ms=ms.value)

    def normal_map(self, faces, num_vertices, owner, abc, vertex_normal):
        """renderNormalMapDevice of the reference on a face map (owner, abc)
        and one view's vertex normals [N,3]; returns [Ht,Wt,3]."""
        import torch
        dev = torch.device("cuda", torch.cuda.current_device())
        faces = np.ascontiguousarray(faces, np.int32).reshape(-1)
        Ht, Wt = owner.shape
        # the reference's float4 (face, a, b, c) per texel; uncovered = (0, 0, 0, 0)
        ids = np.zeros((Ht, Wt, 4), np.float32)
        ids[..., 0] = np.where(owner >= 0, owner, 0).astype(np.float32)
        ids[..., 1:] = abc
        vn = torch.from_numpy(np.ascontiguousarray(vertex_normal, np.float32)).to(dev)
        out = torch.empty((Ht, Wt, 3), device=dev)
        rc = self.L.refcore_normal_map(self.h, faces.ctypes.data, faces.size // 3, int(num_vertices), Ht, Wt,
                                       ids.ctypes.data, ctypes.c_void_p(vn.data_ptr()),
                                       ctypes.c_void_p(out.data_ptr()))
        if rc != 0:
            raise RuntimeError("refcore_normal_map: " + self.L.refcore_error().decode())
        return out.cpu().numpy()

    def backward(self, s, fwd, b=0, albedo=None, shading=None, image_filter_size=1, with_target=False):
        """Reference gradients for the forward outputs `fwd` of the same scene."""
        import torch
        dev = torch.device("cuda", torch.cuda.current_device())
        albedo = albedo or s["albedo_mode"]
        shading = shading or s["shading_mode"]
        if albedo == "foregroundMask":
            shading = "shadeless"
        A = {"vertexColor": 0, "textured": 1, "foregroundMask": 4}[albedo]
        S = {"shaded": 0, "shadeless": 1}[shading]
        t = {k: torch.from_numpy(np.ascontiguousarray(s[k][b])).to(dev)
             for k in ("vertex_pos", "vertex_color", "texture", "sh_coeff", "extrinsics", "intrinsics",
                       "grad_render", "target_image", "grad_target")}
        if not with_target:
            t["grad_target"] = torch.zeros_like(t["grad_target"])
        C, H, W, N = s["num_views"], s["height"], s["width"], s["num_vertices"]
        faces = np.ascontiguousarray(s["faces"], np.int32)
        uvs = np.ascontiguousarray(s["uvs"], np.float32)
        F = faces.shape[0]
        Ht, Wt = t["texture"].shape[0], t["texture"].shape[1]
        face = torch.from_numpy(fwd["face"]).to(dev)
        bary = torch.from_numpy(fwd["bary"]).to(dev)
        vn = torch.from_numpy(fwd["vertex_normal"]).to(dev)
        gp = torch.empty((N, 3), device=dev)
        gc = torch.empty((N, 3), device=dev)
        gt = torch.empty((Ht, Wt, 3), device=dev)
        gs = torch.empty((C, 27), device=dev)
        ms = ctypes.c_float()
        p = lambda x: ctypes.c_void_p(x.data_ptr())
        rc = self.L.refcore_backward(self.h, faces.ctypes.data, uvs.ctypes.data, N, F, C, W, H, A, S,
                                     image_filter_size, 1, Ht, Wt, p(t["grad_render"]), p(t["grad_target"]),
                                     p(t["vertex_pos"]), p(t["vertex_color"]), p(t["texture"]), p(t["sh_coeff"]),
                                     p(vn), p(bary), p(face), p(t["target_image"]), p(t["extrinsics"]),
                                     p(t["intrinsics"]), p(gp), p(gc), p(gt), p(gs), ctypes.byref(ms))
        if rc != 0:
            raise RuntimeError("refcore_backward: " + self.L.refcore_error().decode())
        return dict(vertex_pos_grad=gp.cpu().numpy(), vertex_color_grad=gc.cpu().numpy(),
                    texture_grad=gt.cpu().numpy(), sh_coeff_grad=gs.cpu().numpy(), ms=ms.value)
