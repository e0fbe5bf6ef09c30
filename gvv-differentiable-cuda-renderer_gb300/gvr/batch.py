"""Batched forward and backward of many meshes through one plan (gvr_plan_* in include/gvr.h).

The reference renders one mesh per op call and loops over the batch on the
host (cpp/src/TensorflowOperators/CudaRenderer/CudaRenderer.cpp:309).  A
BatchPlan binds many jobs -- each a RendererHandle (mesh, views, resolution,
modes) with its own inputs -- once, and renders them all with one launch per
pipeline stage and one persistent raster kernel, optionally replayed as a
captured CUDA graph.  Each job's outputs equal render_forward's bit for bit.
The backward (cpp/src/TensorflowOperators/CudaRenderer/CudaRendererGrad.cpp:259
loops the same way) is batched likewise: bind one backward call per job,
then one launch per stage and per pixel-kernel variant.
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib
from .renderer import RendererHandle, _as_f32


def _ptr(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


class BatchPlan:
    """jobs: list of dicts with keys handle (RendererHandle), vertex_pos
    [B,N,3], vertex_color [B,N,3] (vertexColor mode), texture [B,Ht,Wt,3]
    (textured mode), sh_coeff [B,C,27], extrinsics [B,C,12], intrinsics
    [B,C,9], and optionally tile_width (8/16/32) and big_tiles (1..16) to fix
    the bin/tile configuration.  Inputs are copied to contiguous float32
    device tensors owned by the plan; update them in place (plan.inputs[j])
    between calls.  Outputs live in plan.outputs[j]."""

    def __init__(self, jobs, autotune=False, persistent=False):
        if not jobs:
            raise ValueError("a plan needs at least one job")
        self._L = _lib.load()
        self.inputs, self.outputs, self.handles = [], [], []
        arr = (_lib.GvrJob * len(jobs))()
        for j, job in enumerate(jobs):
            h: RendererHandle = job["handle"]
            dev = h.device
            B = int(job["vertex_pos"].shape[0])
            vp = _as_f32(job["vertex_pos"], dev, (B, h.N, 3))
            vc = _as_f32(job.get("vertex_color"), dev, (B, h.N, 3)) if job.get("vertex_color") is not None else None
            tex = _as_f32(job.get("texture"), dev) if job.get("texture") is not None else None
            sh = _as_f32(job["sh_coeff"], dev, (B, h.C, 27))
            ex = _as_f32(job["extrinsics"], dev, (B, h.C, 12))
            ix = _as_f32(job["intrinsics"], dev, (B, h.C, 9))
            Ht, Wt = (int(tex.shape[1]), int(tex.shape[2])) if tex is not None else (1, 1)
            out = dict(barycentric=torch.empty((B, h.C, h.H, h.W, 2), device=dev),
                       face=torch.empty((B, h.C, h.H, h.W), dtype=torch.int32, device=dev),
                       render=torch.empty((B, h.C, h.H, h.W, 3), device=dev),
                       vertex_normal=torch.empty((B, h.C, h.N, 3), device=dev))
            inp = dict(vertex_pos=vp, vertex_color=vc, texture=tex, sh_coeff=sh, extrinsics=ex, intrinsics=ix)
            arr[j].handle = h.ptr
            arr[j].forward = _lib.GvrForwardArgs(B, Ht, Wt, _ptr(vp), _ptr(vc), _ptr(tex), _ptr(sh), None, _ptr(ex),
                                                 _ptr(ix), _ptr(out["barycentric"]), _ptr(out["face"]),
                                                 _ptr(out["render"]), _ptr(out["vertex_normal"]), None, None, None, 0)
            arr[j].tile_width = int(job.get("tile_width", 0))
            arr[j].big_tiles = int(job.get("big_tiles", 0))
            self.inputs.append(inp)
            self.outputs.append(out)
            self.handles.append(h)
        self.device = self.handles[0].device
        self._jobs = arr
        plan = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            flags = (_lib.PLAN_AUTOTUNE if autotune else 0) | (_lib.PLAN_PERSISTENT if persistent else 0)
            _lib.check(self._L.gvr_plan_create(arr, len(jobs), flags, ctypes.byref(plan)))
        self._plan = plan

    def forward(self, stream=None, graph=False):
        """Renders every job on `stream` (default: torch's current stream).
        graph=True captures the plan into a CUDA graph on the first call and
        replays it afterwards (needs a non-default stream)."""
        st = stream if stream is not None else torch.cuda.current_stream(self.device)
        s = ctypes.c_void_p(st.cuda_stream)
        fn = self._L.gvr_plan_forward_graph if graph else self._L.gvr_plan_forward
        _lib.check(fn(self._plan, s))
        return self.outputs

    def forward_per_call(self, stream=None):
        """The same jobs through gvr_forward one by one (one launch chain per
        job, default tiles) into the same outputs: the per-mesh loop the
        plan replaces."""
        st = stream if stream is not None else torch.cuda.current_stream(self.device)
        s = ctypes.c_void_p(st.cuda_stream)
        if not hasattr(self, "_ws"):
            need = max(int(self._L.gvr_forward_workspace_size(self.handles[j].ptr, self._jobs[j].forward.batch,
                                                              self._jobs[j].forward.texture_height,
                                                              self._jobs[j].forward.texture_width))
                       for j in range(len(self.handles)))
            self._ws = torch.empty(need, dtype=torch.uint8, device=self.device)
        for j, h in enumerate(self.handles):
            args = _lib.GvrForwardArgs.from_buffer_copy(self._jobs[j].forward)
            args.workspace = ctypes.c_void_p(self._ws.data_ptr())
            args.workspace_bytes = self._ws.numel()
            _lib.check(self._L.gvr_forward(h.ptr, ctypes.byref(args), s))
        return self.outputs

    def bind_backward(self, grad_render, grad_target=None, target_image=None, flags=0):
        """Binds one backward call per job: grad_render[j] [B,C,H,W,3] (the
        upstream gradient of job j's render), optionally grad_target[j] and
        target_image[j] (the model-to-data term; None entries leave it out)
        and the GVR_BACKWARD_* flags.  Uses the plan's inputs and the
        forward's outputs (face ids, vertex normals).  Gradients land in
        self.grads[j] (vertex_pos, vertex_color, texture, sh_coeff); update
        self.grad_inputs[j] in place between calls."""
        J = len(self.handles)
        gt = grad_target if grad_target is not None else [None] * J
        ti = target_image if target_image is not None else [None] * J
        arr = (_lib.GvrBackwardArgs * J)()
        self.grad_inputs, self.grads = [], []
        for j, h in enumerate(self.handles):
            inp, out = self.inputs[j], self.outputs[j]
            dev = h.device
            B = int(inp["vertex_pos"].shape[0])
            tex = inp["texture"]
            Ht, Wt = (int(tex.shape[1]), int(tex.shape[2])) if tex is not None else (1, 1)
            g = dict(grad_render=_as_f32(grad_render[j], dev, (B, h.C, h.H, h.W, 3)),
                     grad_target=_as_f32(gt[j], dev, (B, h.C, h.H, h.W, 3)) if gt[j] is not None else None,
                     target_image=_as_f32(ti[j], dev, (B, h.C, h.H, h.W, 3)) if ti[j] is not None else None)
            o = dict(vertex_pos=torch.empty((B, h.N, 3), device=dev), vertex_color=torch.empty((B, h.N, 3), device=dev),
                     texture=torch.empty((B, Ht, Wt, 3), device=dev), sh_coeff=torch.empty((B, h.C, 27), device=dev))
            arr[j] = _lib.GvrBackwardArgs(B, Ht, Wt, _ptr(g["grad_render"]), _ptr(inp["vertex_pos"]),
                                          _ptr(inp["vertex_color"]), _ptr(tex), _ptr(inp["sh_coeff"]),
                                          _ptr(g["target_image"]), _ptr(out["vertex_normal"]), _ptr(out["barycentric"]),
                                          _ptr(out["face"]), _ptr(g["grad_target"]), _ptr(inp["extrinsics"]),
                                          _ptr(inp["intrinsics"]), _ptr(o["vertex_pos"]), _ptr(o["vertex_color"]),
                                          _ptr(o["texture"]), _ptr(o["sh_coeff"]), None, 0, int(flags))
            self.grad_inputs.append(g)
            self.grads.append(o)
        self._bwd_args = arr
        with torch.cuda.device(self.device):
            _lib.check(self._L.gvr_plan_bind_backward(self._plan, arr, J))

    def backward(self, stream=None, graph=False):
        """Gradients of every bound job on `stream`; graph=True captures the
        batched backward into a CUDA graph on the first call and replays it
        afterwards (needs a non-default stream)."""
        st = stream if stream is not None else torch.cuda.current_stream(self.device)
        s = ctypes.c_void_p(st.cuda_stream)
        fn = self._L.gvr_plan_backward_graph if graph else self._L.gvr_plan_backward
        _lib.check(fn(self._plan, s))
        return self.grads

    def backward_per_call(self, stream=None):
        """The bound backward calls through gvr_backward one by one (the
        reference's per-element loop), into the same gradient buffers."""
        st = stream if stream is not None else torch.cuda.current_stream(self.device)
        s = ctypes.c_void_p(st.cuda_stream)
        if not hasattr(self, "_bws"):
            need = max(int(self._L.gvr_backward_workspace_size(h.ptr, self._bwd_args[j].batch, 0, 0))
                       for j, h in enumerate(self.handles))
            self._bws = torch.empty(max(need, 256), dtype=torch.uint8, device=self.device)
        for j, h in enumerate(self.handles):
            args = _lib.GvrBackwardArgs.from_buffer_copy(self._bwd_args[j])
            args.workspace = ctypes.c_void_p(self._bws.data_ptr())
            args.workspace_bytes = self._bws.numel()
            _lib.check(self._L.gvr_backward(h.ptr, ctypes.byref(args), s))
        return self.grads

    def tile_config(self, j):
        w, h, b = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        _lib.check(self._L.gvr_plan_tile_config(self._plan, j, ctypes.byref(w), ctypes.byref(h), ctypes.byref(b)))
        return w.value, h.value, b.value

    def close(self):
        if getattr(self, "_plan", None) is not None and self._plan.value:
            self._L.gvr_plan_destroy(self._plan)
            self._plan = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
