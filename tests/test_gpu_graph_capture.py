"""The call pair gvr_forward + gvr_backward captured into a CUDA graph and
replayed.  Every kernel of a call is a programmatic dependent launch, so the
captured graph holds programmatic edges; its replay must give the outputs
of the eager calls (face ids, barycentrics, render and SH gradient bit for
bit; the atomically accumulated gradients to FP32 summation order)."""
import ctypes

import numpy as np
import pytest

from helpers import rel_norm, small_scene

pytestmark = pytest.mark.gpu


def test_call_pair_replays_from_a_cuda_graph():
    import torch
    from gvr import _lib, renderer
    dev = torch.device("cuda", 0)
    s = small_scene(num_faces=1280, views=2, size=64, albedo="textured", shading="shaded", tex=16, seed=3)
    h = renderer.get_handle(s["faces"], s["uvs"], s["num_vertices"], s["num_views"], s["width"], s["height"],
                            s["albedo_mode"], s["shading_mode"], device=dev)
    t = {k: torch.from_numpy(np.ascontiguousarray(s[k])).to(dev)
         for k in ("vertex_pos", "vertex_color", "texture", "sh_coeff", "extrinsics", "intrinsics", "grad_render")}
    B, C, H, W, N = 1, h.C, h.H, h.W, h.N
    Ht, Wt = t["texture"].shape[1], t["texture"].shape[2]
    out = dict(bary=torch.empty((B, C, H, W, 2), device=dev), face=torch.empty((B, C, H, W), dtype=torch.int32, device=dev),
               render=torch.empty((B, C, H, W, 3), device=dev), vnorm=torch.empty((B, C, N, 3), device=dev),
               gpos=torch.empty((B, N, 3), device=dev), gcol=torch.empty((B, N, 3), device=dev),
               gtex=torch.empty((B, Ht, Wt, 3), device=dev), gsh=torch.empty((B, C, 27), device=dev))
    # caller-owned scratch: nothing is allocated while the stream is captured
    fws = torch.empty(h.forward_workspace_size(B, Ht, Wt), dtype=torch.uint8, device=dev)
    bws = torch.empty(h.backward_workspace_size(B), dtype=torch.uint8, device=dev)
    p = lambda x: ctypes.c_void_p(x.data_ptr())
    fa = _lib.GvrForwardArgs(B, Ht, Wt, p(t["vertex_pos"]), p(t["vertex_color"]), p(t["texture"]), p(t["sh_coeff"]),
                             None, p(t["extrinsics"]), p(t["intrinsics"]), p(out["bary"]), p(out["face"]),
                             p(out["render"]), p(out["vnorm"]), None, None, p(fws), fws.numel())
    ba = _lib.GvrBackwardArgs(B, Ht, Wt, p(t["grad_render"]), p(t["vertex_pos"]), p(t["vertex_color"]),
                              p(t["texture"]), p(t["sh_coeff"]), None, p(out["vnorm"]), p(out["bary"]),
                              p(out["face"]), None, p(t["extrinsics"]), p(t["intrinsics"]), p(out["gpos"]),
                              p(out["gcol"]), p(out["gtex"]), p(out["gsh"]), p(bws), bws.numel())
    L = h._L

    def call():
        sp = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
        _lib.check(L.gvr_forward(h.ptr, ctypes.byref(fa), sp))
        _lib.check(L.gvr_backward(h.ptr, ctypes.byref(ba), sp))

    side = torch.cuda.Stream(dev)
    with torch.cuda.stream(side):
        call()
    side.synchronize()
    ref = {k: v.clone() for k, v in out.items()}
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=side):
        call()
    for _ in range(2):
        for v in out.values():
            v.zero_()
        torch.cuda.synchronize()
        graph.replay()
        torch.cuda.synchronize()
        for k in ("bary", "face", "render", "vnorm", "gsh"):
            assert torch.equal(out[k], ref[k]), k
        for k in ("gpos", "gcol", "gtex"):
            a, b = out[k].cpu().numpy(), ref[k].cpu().numpy()
            assert rel_norm(a, b) <= 1e-6 if np.any(b) else np.all(a == 0), k
