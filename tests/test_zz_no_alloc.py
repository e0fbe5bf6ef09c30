"""gvr_backward_noalloc: the backward pass for callers that must not allocate
device memory (a host that fixes the GPU memory budget up front, or a
real-time path where an allocation would synchronise the device).  Its
scratch lives in a fixed array inside the library, so it is compared here,
through the C ABI, with gvr_backward on the same inputs, on two calls in a
row (the array keeps the previous call's contents), at the gradient
tolerance of the other parity tests (||a - b|| <= 1e-4 ||b||).

The file is named to be collected last.
"""
import ctypes

import numpy as np
import pytest

from helpers import rel_norm, small_scene

pytestmark = pytest.mark.gpu

GRAD_TOL = 1e-4


def _setup(albedo, shading, batch=1):
    import torch
    from gvr import renderer
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    s = small_scene(num_faces=1280, views=2, size=64, albedo=albedo, shading=shading, tex=16, seed=41, batch=batch)
    rng = np.random.default_rng(41)
    s["target_image"] = rng.uniform(0, 1, s["target_image"].shape).astype(np.float32)
    s["grad_target"] = rng.normal(0, 1, s["grad_target"].shape).astype(np.float32)
    h = renderer.get_handle(s["faces"], s["uvs"], s["num_vertices"], s["num_views"], s["width"], s["height"],
                            albedo, shading, device=dev)
    t = {k: torch.from_numpy(np.ascontiguousarray(s[k])).to(dev)
         for k in ("vertex_pos", "vertex_color", "texture", "sh_coeff", "extrinsics", "intrinsics", "target_image",
                   "grad_render", "grad_target")}
    bary, face, _, vn, _, _ = renderer.render_forward(h, t["vertex_pos"], t["vertex_color"], t["texture"],
                                                      t["sh_coeff"], t["extrinsics"], t["intrinsics"])
    return h, t, bary, face, vn


def _call(h, t, bary, face, vn, entry, workspace=None, target=True):
    import torch
    from gvr import _lib
    dev = t["vertex_pos"].device
    B, N = t["vertex_pos"].shape[0], h.N
    Ht, Wt = t["texture"].shape[1], t["texture"].shape[2]
    outs = [torch.full((B, N, 3), float("nan"), device=dev), torch.full((B, N, 3), float("nan"), device=dev),
            torch.full((B, Ht, Wt, 3), float("nan"), device=dev), torch.full((B, h.C, 27), float("nan"), device=dev)]
    p = lambda x: None if x is None else ctypes.c_void_p(x.data_ptr())
    args = _lib.GvrBackwardArgs(B, Ht, Wt, p(t["grad_render"]), p(t["vertex_pos"]), p(t["vertex_color"]),
                                p(t["texture"]), p(t["sh_coeff"]), p(t["target_image"]), p(vn), p(bary), p(face),
                                p(t["grad_target"]) if target else None, p(t["extrinsics"]), p(t["intrinsics"]),
                                *[p(o) for o in outs], p(workspace), 0 if workspace is None else workspace.numel())
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.check(entry(h.ptr, ctypes.byref(args), stream))
    torch.cuda.synchronize()
    return [o.cpu().numpy() for o in outs]


def _same(got, ref):
    for a, b in zip(got, ref):
        assert np.isfinite(a).all()
        if np.all(b == 0):
            assert np.all(a == 0)
        else:
            assert rel_norm(a, b) <= GRAD_TOL


# (albedo, shading, batch, target gradient): every part of the scratch is
# written by at least one case (per-face accumulators and SH partials in
# the shaded modes, face records in all), and "normal" needs none at all
CASES = [("vertexColor", "shaded", 1, True), ("textured", "shaded", 1, False), ("vertexColor", "shaded", 2, False),
         ("textured", "shadeless", 2, True), ("foregroundMask", "shaded", 1, True), ("normal", "shaded", 1, False)]


def _reference(case):
    import torch
    albedo, shading, batch, target = case
    h, t, bary, face, vn = _setup(albedo, shading, batch)
    ws = torch.empty(max(h.backward_workspace_size(batch), 256), dtype=torch.uint8, device=t["vertex_pos"].device)
    return (h, t, bary, face, vn), _call(h, t, bary, face, vn, h._L.gvr_backward, ws, target)


@pytest.mark.parametrize("case", CASES, ids=["-".join(map(str, c)) for c in CASES])
def test_noalloc_backward_matches_backward(case):
    (h, t, bary, face, vn), ref = _reference(case)
    for _ in range(2):  # the second call starts from the first call's scratch contents
        _same(_call(h, t, bary, face, vn, h._L.gvr_backward_noalloc, target=case[3]), ref)


def test_noalloc_calls_of_different_shapes_in_a_row():
    """Each call starts from whatever the previous call, of another mode or
    batch size, left in the shared array; results must not depend on it."""
    runs = [(_reference(c), c[3]) for c in CASES]
    for _ in range(2):
        for ((h, t, bary, face, vn), ref), target in runs:
            _same(_call(h, t, bary, face, vn, h._L.gvr_backward_noalloc, target=target), ref)


def test_noalloc_rejects_calls_beyond_its_scratch():
    from gvr import _lib
    import torch
    rng = np.random.default_rng(0)
    N, F = 200_000, 400_000                      # scratch for one element: ~80 MB > 32 MiB
    faces = rng.integers(0, N, size=(F, 3)).astype(np.int32)
    from gvr.renderer import RendererHandle
    h = RendererHandle(faces, None, N, 8, 1024, 1024, "vertexColor", "shaded",
                       device=torch.device("cuda", 0))
    assert h.backward_workspace_size(1) > _lib.NOALLOC_SCRATCH_BYTES
    args = _lib.GvrBackwardArgs()
    args.batch, args.texture_height, args.texture_width = 1, 1, 1
    rc = h._L.gvr_backward_noalloc(h.ptr, ctypes.byref(args), None)   # refused before anything runs
    assert rc == -4
    assert "fixed scratch array" in h._L.gvr_last_error().decode()
    h.close()
