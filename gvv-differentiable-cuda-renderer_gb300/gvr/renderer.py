"""PyTorch host side of the renderer: the reference's `CudaRendererGpu`
operator surface (python/CudaRenderer.py:30-215) over the C ABI.

  RendererHandle       owns one GvrHandle (topology + attrs), like the TF op
                       kernel object that owns its CUDABasedRasterization.
  render_forward/...   raw calls: device tensors in, device tensors out.
  RenderFunction       torch.autograd.Function: forward = CudaRendererGpu,
                       backward = CudaRendererGradGpu with the wrapper's
                       zero-gradient rules (python/CudaRenderer.py:170-215).
  CudaRendererGpu      same constructor kwargs and getters as the reference.
"""
from __future__ import annotations

import collections
import ctypes
import hashlib

import numpy as np
import torch

from . import _lib

__all__ = ["RendererHandle", "RenderFunction", "CudaRendererGpu", "get_handle", "render_forward", "render_backward"]


def _ptr(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def _stream(device):
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)


class RendererHandle:
    """One GvrHandle: topology, vertex->face adjacency and render attrs."""

    def __init__(self, faces, texture_coordinates, num_vertices, num_cameras, width, height,
                 albedo_mode="textured", shading_mode="shaded", image_filter_size=1, texture_filter_size=1,
                 compute_normal_map=False, device=None):
        L = _lib.load()
        if albedo_mode not in _lib.ALBEDO:
            raise ValueError(f"INVALID ALBEDO MODE: {albedo_mode!r}")
        if shading_mode not in _lib.SHADING:
            raise ValueError(f"INVALID SHADING MODE: {shading_mode!r}")
        self.faces = np.ascontiguousarray(np.asarray(faces, dtype=np.int32).reshape(-1))
        if self.faces.size % 3:
            raise ValueError("No triangular faces!")
        tc = np.asarray(texture_coordinates if texture_coordinates is not None else [], dtype=np.float32).reshape(-1)
        if tc.size and tc.size != 2 * self.faces.size:
            raise ValueError("Texture coordinates have wrong dimensionality!")
        self.uvs = np.ascontiguousarray(tc) if tc.size else None
        self.N, self.F = int(num_vertices), self.faces.size // 3
        self.C, self.W, self.H = int(num_cameras), int(width), int(height)
        self.albedo_mode = albedo_mode
        self.shading_mode = "shadeless" if albedo_mode == "foregroundMask" else shading_mode
        self.image_filter_size, self.texture_filter_size = int(image_filter_size), int(texture_filter_size)
        self.compute_normal_map = bool(compute_normal_map)
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        topo = _lib.GvrTopology(self.faces.ctypes.data, None if self.uvs is None else self.uvs.ctypes.data,
                                self.F, self.N)
        attrs = _lib.GvrAttrs(self.C, self.W, self.H, _lib.ALBEDO[albedo_mode], _lib.SHADING[shading_mode],
                              self.image_filter_size, self.texture_filter_size, int(self.compute_normal_map))
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _lib.check(L.gvr_create(ctypes.byref(topo), ctypes.byref(attrs), ctypes.byref(h)))
        self._h = h
        self._L = L

    @property
    def ptr(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._L.gvr_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def forward_workspace_size(self, batch, texture_height=0, texture_width=0):
        return int(self._L.gvr_forward_workspace_size(self._h, batch, texture_height, texture_width))

    def backward_workspace_size(self, batch):
        return int(self._L.gvr_backward_workspace_size(self._h, batch, 0, 0))

    def debug_rays(self, extrinsics, intrinsics):
        B = extrinsics.shape[0]
        out = torch.empty((B, self.C, self.H, self.W, 3), dtype=torch.float32, device=self.device)
        _lib.check(self._L.gvr_debug_rays(self._h, B, _ptr(extrinsics), _ptr(intrinsics), _ptr(out),
                                          _stream(self.device)))
        return out


_HANDLES: "collections.OrderedDict[tuple, RendererHandle]" = collections.OrderedDict()
_MAX_HANDLES = 32


def get_handle(faces, texture_coordinates, num_vertices, num_cameras, width, height, albedo_mode="textured",
               shading_mode="shaded", image_filter_size=1, texture_filter_size=1, compute_normal_map=False,
               device=None) -> RendererHandle:
    """Cached RendererHandle for this topology + attr set (the reference builds
    its renderer once per op node; here once per distinct attr set)."""
    f = np.ascontiguousarray(np.asarray(faces, dtype=np.int32).reshape(-1))
    t = np.ascontiguousarray(np.asarray(texture_coordinates if texture_coordinates is not None else [],
                                        dtype=np.float32).reshape(-1))
    dev = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
    key = (hashlib.sha1(f.tobytes()).hexdigest(), hashlib.sha1(t.tobytes()).hexdigest(), f.size, t.size,
           int(num_vertices), int(num_cameras), int(width), int(height), albedo_mode, shading_mode,
           int(image_filter_size), int(texture_filter_size), bool(compute_normal_map), str(dev))
    h = _HANDLES.get(key)
    if h is None:
        h = RendererHandle(f, t, num_vertices, num_cameras, width, height, albedo_mode, shading_mode,
                           image_filter_size, texture_filter_size, compute_normal_map, dev)
        _HANDLES[key] = h
        while len(_HANDLES) > _MAX_HANDLES:
            _HANDLES.popitem(last=False)
    else:
        _HANDLES.move_to_end(key)
    return h


def _as_f32(x, device, shape=None):
    if x is None:
        return None
    if not torch.is_tensor(x):
        x = torch.as_tensor(np.asarray(x, dtype=np.float32))
    x = x.to(device=device, dtype=torch.float32)
    if shape is not None:
        x = x.reshape(shape)
    return x.contiguous()


def render_forward(h: RendererHandle, vertex_pos, vertex_color, texture, sh_coeff, extrinsics, intrinsics,
                   target_image=None, copy_target=False):
    """Forward render of every view of every batch element.
    Returns (barycentric, face, render, vertex_normal, target_image_out, normal_map)."""
    dev = h.device
    B = vertex_pos.shape[0]
    vp = _as_f32(vertex_pos, dev, (B, h.N, 3))
    vc = _as_f32(vertex_color, dev, (B, h.N, 3)) if vertex_color is not None else None
    tex = _as_f32(texture, dev) if texture is not None else torch.zeros((B, 1, 1, 3), device=dev)
    if tex.dim() != 4 or tex.shape[0] != B or tex.shape[3] != 3:
        raise ValueError("texture must be [B, Ht, Wt, 3] with the vertex batch size")
    sh = _as_f32(sh_coeff, dev, (B, h.C, 27))
    ex = _as_f32(extrinsics, dev, (B, h.C, 12))
    ix = _as_f32(intrinsics, dev, (B, h.C, 9))
    tgt = _as_f32(target_image, dev, (B, h.C, h.H, h.W, 3)) if target_image is not None else None
    Ht, Wt = tex.shape[1], tex.shape[2]
    bary = torch.empty((B, h.C, h.H, h.W, 2), dtype=torch.float32, device=dev)
    face = torch.empty((B, h.C, h.H, h.W), dtype=torch.int32, device=dev)
    img = torch.empty((B, h.C, h.H, h.W, 3), dtype=torch.float32, device=dev)
    vnorm = torch.empty((B, h.C, h.N, 3), dtype=torch.float32, device=dev)
    tout = torch.empty_like(tgt) if (copy_target and tgt is not None) else None
    # written by the forward with compute_normal_map; zeros otherwise (the
    # reference leaves that output unwritten)
    nmap = (torch.empty if h.compute_normal_map else torch.zeros)((B, Ht, Wt, 3), dtype=torch.float32, device=dev)
    ws_bytes = h.forward_workspace_size(B, Ht, Wt)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=dev)
    args = _lib.GvrForwardArgs(B, Ht, Wt, _ptr(vp), _ptr(vc), _ptr(tex), _ptr(sh), _ptr(tgt), _ptr(ex), _ptr(ix),
                               _ptr(bary), _ptr(face), _ptr(img), _ptr(vnorm), _ptr(tout),
                               _ptr(nmap) if h.compute_normal_map else None, _ptr(ws), ws_bytes)
    _lib.check(h._L.gvr_forward(h.ptr, ctypes.byref(args), _stream(dev)))
    return bary, face, img, vnorm, (tout if tout is not None else tgt), nmap


def render_backward(h: RendererHandle, grad_render, vertex_pos, vertex_color, texture, sh_coeff, target_image,
                    vertex_normal, barycentric, face, grad_target, extrinsics, intrinsics, flags=0):
    """Gradients (vertex_pos, vertex_color, texture, sh_coeff) of CudaRendererGradGpu.
    flags: GVR_BACKWARD_* options (_lib.BACKWARD_ALBEDO_POSITION); 0 = the reference's gradient."""
    dev = h.device
    B = vertex_pos.shape[0]
    Ht, Wt = texture.shape[1], texture.shape[2]
    gp = torch.empty((B, h.N, 3), dtype=torch.float32, device=dev)
    gc = torch.empty((B, h.N, 3), dtype=torch.float32, device=dev)
    gt = torch.empty((B, Ht, Wt, 3), dtype=torch.float32, device=dev)
    gs = torch.empty((B, h.C, 27), dtype=torch.float32, device=dev)
    if grad_render is None:
        grad_render = torch.zeros((B, h.C, h.H, h.W, 3), dtype=torch.float32, device=dev)
    grad_render = grad_render.contiguous().float()
    if grad_target is not None:
        grad_target = grad_target.contiguous().float()
        if target_image is None:
            raise ValueError("grad of target_image_out needs target_image")
    ws_bytes = h.backward_workspace_size(B)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=dev)
    args = _lib.GvrBackwardArgs(B, Ht, Wt, _ptr(grad_render), _ptr(vertex_pos), _ptr(vertex_color), _ptr(texture),
                                _ptr(sh_coeff), _ptr(target_image), _ptr(vertex_normal), _ptr(barycentric),
                                _ptr(face), _ptr(grad_target), _ptr(extrinsics), _ptr(intrinsics),
                                _ptr(gp), _ptr(gc), _ptr(gt), _ptr(gs), _ptr(ws), ws_bytes, int(flags))
    _lib.check(h._L.gvr_backward(h.ptr, ctypes.byref(args), _stream(dev)))
    return gp, gc, gt, gs


class RenderFunction(torch.autograd.Function):
    """Differentiable render.  Outputs: barycentric, face (int32, not
    differentiable), render, vertex_normal, target_image_out, normal_map.
    Gradients reach vertex_pos, vertex_color, texture and sh_coeff; target,
    extrinsics and intrinsics get none (python/CudaRenderer.py:215)."""

    @staticmethod
    def forward(ctx, h, vertex_pos, vertex_color, texture, sh_coeff, target_image, extrinsics, intrinsics,
                backward_flags=0):
        bary, face, img, vnorm, tout, nmap = render_forward(h, vertex_pos, vertex_color, texture, sh_coeff,
                                                            extrinsics, intrinsics, target_image, copy_target=True)
        ctx.h = h
        ctx.backward_flags = backward_flags
        # only the face ids are kept for the backward, which recomputes the
        # barycentrics from them (no per-pixel intermediates kept)
        ctx.save_for_backward(vertex_pos, vertex_color, texture, sh_coeff, target_image, extrinsics, intrinsics,
                              face, vnorm)
        ctx.mark_non_differentiable(face, bary, vnorm, nmap)
        return bary, face, img, vnorm, tout, nmap

    @staticmethod
    def backward(ctx, g_bary, g_face, g_render, g_vnorm, g_target, g_nmap):
        vp, vc, tex, sh, tgt, ex, ix, face, vnorm = ctx.saved_tensors
        h = ctx.h
        gp, gc, gt, gs = render_backward(h, g_render, vp, vc, tex, sh, tgt, vnorm, None, face, g_target, ex, ix,
                                         ctx.backward_flags)
        return None, gp, gc, gt, gs, None, None, None, None


class CudaRendererGpu:
    """The reference's python/CudaRenderer.py:30-164 operator, on torch tensors.
    Inputs may be torch tensors (CUDA or CPU), numpy arrays or lists; they are
    moved to the current CUDA device as float32.  Outputs are torch tensors."""

    def __init__(self,
                 faces_attr=(),
                 texCoords_attr=(),
                 numberOfVertices_attr=-1,
                 numberOfCameras_attr=-1,
                 renderResolutionU_attr=-1,
                 renderResolutionV_attr=-1,
                 albedoMode_attr='textured',
                 shadingMode_attr='shaded',
                 image_filter_size_attr=1,
                 texture_filter_size_attr=1,
                 compute_normal_map_attr=False,
                 vertexPos_input=None,
                 vertexColor_input=None,
                 texture_input=None,
                 shCoeff_input=None,
                 targetImage_input=None,
                 extrinsics_input=(),
                 intrinsics_input=(),
                 nodeName='CudaRenderer'):
        self.faces_attr = faces_attr
        self.texCoords_attr = texCoords_attr
        self.numberOfVertices_attr = numberOfVertices_attr
        self.numberOfCameras_attr = numberOfCameras_attr
        self.renderResolutionU_attr = renderResolutionU_attr
        self.renderResolutionV_attr = renderResolutionV_attr
        self.albedoMode_attr = albedoMode_attr
        self.shadingMode_attr = shadingMode_attr
        self.image_filter_size_attr = image_filter_size_attr
        self.texture_filter_size_attr = texture_filter_size_attr
        self.compute_normal_map_attr = compute_normal_map_attr
        self.nodeName = nodeName

        self.handle = get_handle(faces_attr, texCoords_attr, numberOfVertices_attr, numberOfCameras_attr,
                                 renderResolutionU_attr, renderResolutionV_attr, albedoMode_attr, shadingMode_attr,
                                 image_filter_size_attr, texture_filter_size_attr, compute_normal_map_attr)
        h = self.handle
        dev = h.device
        vp = _as_f32(vertexPos_input, dev)
        B = vp.shape[0]
        vp = vp.reshape(B, h.N, 3)
        vc = _as_f32(vertexColor_input, dev, (B, h.N, 3)) if vertexColor_input is not None else torch.zeros_like(vp)
        tex = _as_f32(texture_input, dev) if texture_input is not None else torch.zeros((B, 1, 1, 3), device=dev)
        sh = _as_f32(shCoeff_input, dev, (B, h.C, 27))
        tgt = (_as_f32(targetImage_input, dev, (B, h.C, h.H, h.W, 3)) if targetImage_input is not None
               else torch.zeros((B, h.C, h.H, h.W, 3), device=dev))
        ex = _as_f32(extrinsics_input, dev, (B, h.C, 12))
        ix = _as_f32(intrinsics_input, dev, (B, h.C, 9))
        self.vertexPos_input, self.vertexColor_input, self.texture_input = vp, vc, tex
        self.shCoeff_input, self.targetImage_input = sh, tgt
        self.extrinsics_input, self.intrinsics_input = ex, ix
        self.cudaRendererOperator = RenderFunction.apply(h, vp, vc, tex, sh, tgt, ex, ix)

    def getBaryCentricBufferTF(self):
        return self.cudaRendererOperator[0]

    def getFaceBufferTF(self):
        return self.cudaRendererOperator[1]

    def getRenderBufferTF(self):
        return self.cudaRendererOperator[2]

    def getVertexNormalTF(self):
        return self.cudaRendererOperator[3]

    def getTargetBufferTF(self):
        return self.cudaRendererOperator[4]

    def getNormalMap(self):
        if self.compute_normal_map_attr:
            return self.cudaRendererOperator[5].reshape(self.texture_input.shape)
        print('Requesting normal map but computation was not enabled!')
        return None

    def getModelMaskTF(self):
        """[B, C, H, W, 3] float mask of covered pixels (python/CudaRenderer.py:134-140)."""
        face = self.cudaRendererOperator[1]
        return (face >= 0).unsqueeze(-1).expand(*face.shape, 3).float()

    # torch-style names
    barycentric = property(getBaryCentricBufferTF)
    face = property(getFaceBufferTF)
    render = property(getRenderBufferTF)
    vertex_normal = property(getVertexNormalTF)
    target = property(getTargetBufferTF)
