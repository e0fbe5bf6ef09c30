"""GPU parity: the CUDA path (through the C ABI) against the CPU oracle on the
same seeded inputs.

Bars (written out per test):
  * face ids, barycentrics, vertex normals: bit-exact.  The oracle is given
    the device's per-pixel FP32 ray directions (gvr_debug_rays), because the
    reference normalises rays with the device rsqrtf, which a CPU cannot
    reproduce bit-for-bit; every other FP32 operation is restated exactly.
    Pixels whose minimal quantised depth is shared by several faces (the
    reference resolves them by a write race) must hold the smallest id.
  * render: max |gpu - oracle| <= 1e-5 * max |oracle| (FP64 oracle).
  * gradients: ||gpu - oracle||_2 <= 1e-4 * ||oracle||_2 per output (FP64 oracle).
"""
import numpy as np
import pytest

from helpers import oracle_scene, rel_max, rel_norm, small_scene

pytestmark = pytest.mark.gpu

IMG_TOL = 1e-5
GRAD_TOL = 1e-4


def _dev():
    import torch
    return torch.device("cuda", 0)


def _tensors(s):
    import torch
    return {k: torch.from_numpy(np.ascontiguousarray(s[k])).to(_dev())
            for k in ("vertex_pos", "vertex_color", "texture", "sh_coeff", "extrinsics", "intrinsics", "target_image",
                      "grad_render", "grad_target")}


def _handle(s, albedo=None, shading=None, image_filter_size=1):
    from gvr import renderer
    return renderer.get_handle(s["faces"], s["uvs"], s["num_vertices"], s["num_views"], s["width"], s["height"],
                               albedo or s["albedo_mode"], shading or s["shading_mode"], image_filter_size,
                               device=_dev())


def run_gpu(s, albedo=None, shading=None, with_target=False, image_filter_size=1, flags=0):
    import torch
    from gvr import renderer
    h = _handle(s, albedo, shading, image_filter_size)
    t = _tensors(s)
    bary, face, img, vn, _, _ = renderer.render_forward(h, t["vertex_pos"], t["vertex_color"], t["texture"],
                                                        t["sh_coeff"], t["extrinsics"], t["intrinsics"])
    g = renderer.render_backward(h, t["grad_render"], t["vertex_pos"], t["vertex_color"], t["texture"],
                                 t["sh_coeff"], t["target_image"], vn, bary, face,
                                 t["grad_target"] if with_target else None, t["extrinsics"], t["intrinsics"],
                                 flags)
    rays = h.debug_rays(t["extrinsics"], t["intrinsics"])
    torch.cuda.synchronize()
    cpu = lambda x: x.cpu().numpy()
    return dict(bary=cpu(bary), face=cpu(face), render=cpu(img), vertex_normal=cpu(vn), rays=cpu(rays),
                vertex_pos_grad=cpu(g[0]), vertex_color_grad=cpu(g[1]), texture_grad=cpu(g[2]),
                sh_coeff_grad=cpu(g[3]))


def check_batch(s, gpu, albedo=None, shading=None, with_target=False, image_filter_size=1, grads=True, flags=0):
    B = s["vertex_pos"].shape[0]
    for b in range(B):
        o = oracle_scene(s, b, rays=gpu["rays"][b], albedo=albedo, shading=shading,
                         image_filter_size=image_filter_size)
        ref = o.forward()
        # visibility: bit-exact, ties resolved to the smallest face id
        assert np.array_equal(gpu["face"][b], ref["face"]), \
            f"batch {b}: {(gpu['face'][b] != ref['face']).sum()} face-id mismatches"
        assert np.array_equal(gpu["bary"][b].view(np.uint32), ref["bary"].view(np.uint32))
        assert np.array_equal(gpu["vertex_normal"][b].view(np.uint32), ref["vertex_normal"].view(np.uint32))
        assert rel_max(gpu["render"][b], ref["render"]) <= IMG_TOL
        if not grads:
            continue
        gt = s["grad_target"][b] if with_target else np.zeros_like(s["grad_target"][b])
        g = o.backward(ref["face"], ref["bary"], ref["vertex_normal"], s["grad_render"][b], s["target_image"][b], gt,
                       flags=flags)
        for k in ("vertex_pos_grad", "vertex_color_grad", "texture_grad", "sh_coeff_grad"):
            if np.all(g[k] == 0):
                assert np.all(gpu[k][b] == 0), k
            else:
                assert rel_norm(gpu[k][b], g[k]) <= GRAD_TOL, (k, rel_norm(gpu[k][b], g[k]))


MODES = [(a, sh) for a in ("vertexColor", "textured", "normal", "lighting", "foregroundMask")
         for sh in ("shaded", "shadeless")]
# modes without reference counterpart (include/gvr.h), pinned by the oracle's restatement
MODES += [("texturedBilinear", "shaded"), ("texturedBilinear", "shadeless"), ("uv", "shaded"),
          ("vertexColor", "phong"), ("textured", "phong"), ("texturedBilinear", "phong"), ("normal", "phong")]


@pytest.mark.parametrize("albedo,shading", MODES)
def test_modes_small_batch(albedo, shading):
    s = small_scene(num_faces=1280, views=2, size=64, albedo=albedo, shading=shading, tex=16, seed=11, batch=2)
    s["vertex_pos"][1] *= np.float32(1.1)          # batch elements differ
    s["sh_coeff"][1] = s["sh_coeff"][1][::-1].copy()
    gpu = run_gpu(s)
    check_batch(s, gpu)


@pytest.mark.parametrize("shading", ["shaded", "shadeless"])
def test_albedo_position_option(shading):
    """GVR_BACKWARD_ALBEDO_POSITION (no reference counterpart): the position
    gradient also carries the vertex colour's change through the
    barycentrics; GPU against the oracle's restatement of the same option."""
    s = small_scene(num_faces=1280, views=2, size=64, albedo="vertexColor", shading=shading, seed=21, batch=2)
    gpu = run_gpu(s, flags=1)
    check_batch(s, gpu, flags=1)
    base = run_gpu(s)
    assert not np.allclose(base["vertex_pos_grad"], gpu["vertex_pos_grad"])
    assert rel_norm(gpu["vertex_color_grad"], base["vertex_color_grad"]) <= 1e-6   # float atomics reorder sums


def test_target_image_term():
    s = small_scene(num_faces=1280, views=2, size=64, albedo="vertexColor", seed=5)
    rng = np.random.default_rng(5)
    s["target_image"] = rng.uniform(0, 1, s["target_image"].shape).astype(np.float32)
    s["grad_target"] = rng.normal(0, 1, s["grad_target"].shape).astype(np.float32)
    for k in (1, 2):
        gpu = run_gpu(s, with_target=True, image_filter_size=k)
        check_batch(s, gpu, with_target=True, image_filter_size=k)


def test_odd_resolution_and_borders():
    s = small_scene(num_faces=720, views=3, size=64, seed=2)
    from gvr import scenes
    # 53 x 37, camera close enough that the mesh crosses every border
    s = scenes.scene(720, 3, 53, 37, "vertexColor", "shaded", tex_size=4, seed=2)
    s["extrinsics"][..., [3, 7, 11]] *= np.float32(0.55)
    gpu = run_gpu(s)
    check_batch(s, gpu)
    assert (gpu["face"][0][:, 0] >= 0).any() and (gpu["face"][0][0] >= 0).any()


def test_mesh_behind_camera_and_straddling():
    from gvr import scenes
    s = scenes.scene(320, 2, 48, 48, "vertexColor", "shaded", seed=4)
    s["extrinsics"][0, 0, 11] = -3000.0           # view 0: whole mesh behind the camera
    s["extrinsics"][0, 1, 11] = 500.0             # view 1: camera inside the sphere
    gpu = run_gpu(s)
    check_batch(s, gpu, grads=True)
    assert np.all(gpu["face"][0][0] == -1)


def test_duplicate_faces_tie_to_min_id():
    from gvr import scenes
    s = scenes.scene(320, 1, 48, 48, "vertexColor", "shaded", seed=6)
    F0 = s["faces"].shape[0]
    s["faces"] = np.concatenate([s["faces"][40:], s["faces"][:80]]).astype(np.int32)  # 40 faces appear twice
    s["uvs"] = np.concatenate([s["uvs"][40:], s["uvs"][:80]]).astype(np.float32)
    gpu = run_gpu(s)
    o = oracle_scene(s, 0, rays=gpu["rays"][0])
    ref = o.forward()
    tie = ref["ties"] > 1
    assert tie.any()
    assert np.array_equal(gpu["face"][0], ref["face"])
    assert np.all(gpu["face"][0][tie] < F0 - 40)   # the lower copy of the duplicated face
    check_batch(s, gpu)


def test_single_view_vertex_color_workload():
    """2,562 V / 5,120 F displaced icosphere, vertex colours, shaded, 256x256."""
    from gvr import scenes
    s = scenes.single_view_vertex_color(seed=0)
    gpu = run_gpu(s)
    check_batch(s, gpu)


def test_multiview_textured_workload():
    """Full size: 35,002 V / 70,000 F, 1024^2 texture, 8 views at 1024x1024."""
    from gvr import scenes
    s = scenes.multiview_textured(seed=0)
    gpu = run_gpu(s)
    check_batch(s, gpu)


@pytest.mark.parametrize("views", [3, 33])
def test_views_rendered_together_equal_views_rendered_alone(views):
    """Three 1024x1024 views in one call hold 12,288 tiles, which the tile
    scan splits over two blocks (the second partly filled); 33 views hold
    135,168 tiles, scanned by the single-block scan.  Each view must come out
    bit for bit as when rendered alone (4,096 tiles, one block)."""
    import torch
    from gvr import renderer, scenes
    s = scenes.scene(5120, views, 1024, 1024, "textured", "shaded", tex_size=64, seed=6)
    t = _tensors(s)
    h = _handle(s)
    together = renderer.render_forward(h, t["vertex_pos"], t["vertex_color"], t["texture"], t["sh_coeff"],
                                       t["extrinsics"], t["intrinsics"])[:3]
    h1 = renderer.get_handle(s["faces"], s["uvs"], s["num_vertices"], 1, 1024, 1024, "textured", "shaded",
                             device=_dev())
    for c in sorted({0, views // 2, views - 1}):
        alone = renderer.render_forward(h1, t["vertex_pos"], t["vertex_color"], t["texture"],
                                        t["sh_coeff"][:, c:c + 1].contiguous(),
                                        t["extrinsics"][:, c:c + 1].contiguous(),
                                        t["intrinsics"][:, c:c + 1].contiguous())[:3]
        torch.cuda.synchronize()
        for a, b in zip(together, alone):
            assert torch.equal(a[:, c:c + 1], b), c


def test_forward_is_deterministic_and_workspace_paths_agree():
    import ctypes
    import torch
    from gvr import _lib, renderer
    s = small_scene(num_faces=1280, views=2, size=64, albedo="textured", seed=8)
    h = _handle(s)
    t = _tensors(s)
    outs = []
    for use_ws in (True, False, True):
        B = 1
        bary = torch.empty((B, h.C, h.H, h.W, 2), device=_dev())
        face = torch.empty((B, h.C, h.H, h.W), dtype=torch.int32, device=_dev())
        img = torch.empty((B, h.C, h.H, h.W, 3), device=_dev())
        vn = torch.empty((B, h.C, h.N, 3), device=_dev())
        n = h.forward_workspace_size(B)
        ws = torch.empty(n, dtype=torch.uint8, device=_dev()) if use_ws else None
        p = lambda x: None if x is None else ctypes.c_void_p(x.data_ptr())
        args = _lib.GvrForwardArgs(B, t["texture"].shape[1], t["texture"].shape[2], p(t["vertex_pos"]),
                                   p(t["vertex_color"]), p(t["texture"]), p(t["sh_coeff"]), None, p(t["extrinsics"]),
                                   p(t["intrinsics"]), p(bary), p(face), p(img), p(vn), None, None, p(ws),
                                   n if use_ws else 0)
        _lib.check(h._L.gvr_forward(h.ptr, ctypes.byref(args), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))
        torch.cuda.synchronize()
        outs.append([x.cpu().numpy() for x in (bary, face, img, vn)])
    for a, b in zip(outs[0], outs[1]):
        assert np.array_equal(a, b)
    for a, b in zip(outs[0], outs[2]):
        assert np.array_equal(a, b)
    # a workspace one byte short is refused
    small = torch.empty(h.forward_workspace_size(1) - 256, dtype=torch.uint8, device=_dev())
    args.workspace, args.workspace_bytes = ctypes.c_void_p(small.data_ptr()), small.numel()
    assert h._L.gvr_forward(h.ptr, ctypes.byref(args), None) == -4


@pytest.mark.parametrize("albedo", ["textured", "vertexColor"])
def test_backward_reads_the_barycentric_input(albedo):
    """The backward takes the barycentrics from its input, as the reference's
    grad does (CUDABasedRasterizationGrad.cu:210-211): given perturbed
    barycentrics it follows the oracle given the same ones.  Without the
    input it recomputes them from the face ids and equals the call given the
    forward's own (float atomics only reorder sums)."""
    import torch
    from gvr import renderer
    s = small_scene(num_faces=1280, views=2, size=64, albedo=albedo, shading="shaded", tex=16, seed=31)
    h = _handle(s)
    t = _tensors(s)
    bary, face, img, vn, _, _ = renderer.render_forward(h, t["vertex_pos"], t["vertex_color"], t["texture"],
                                                        t["sh_coeff"], t["extrinsics"], t["intrinsics"])
    rng = np.random.default_rng(31)
    noise = torch.from_numpy(rng.uniform(-0.02, 0.02, tuple(bary.shape)).astype(np.float32)).to(_dev())
    pert = (bary + noise * (face >= 0).unsqueeze(-1)).contiguous()

    def grads(b):
        g = renderer.render_backward(h, t["grad_render"], t["vertex_pos"], t["vertex_color"], t["texture"],
                                     t["sh_coeff"], t["target_image"], vn, b, face, None, t["extrinsics"],
                                     t["intrinsics"])
        torch.cuda.synchronize()
        return [x.cpu().numpy()[0] for x in g]

    keys = ("vertex_pos_grad", "vertex_color_grad", "texture_grad", "sh_coeff_grad")
    rays = h.debug_rays(t["extrinsics"], t["intrinsics"]).cpu().numpy()[0]
    o = oracle_scene(s, 0, rays=rays)
    g_orc = o.backward(face.cpu().numpy()[0], pert.cpu().numpy()[0], vn.cpu().numpy()[0], s["grad_render"][0],
                       s["target_image"][0], np.zeros_like(s["grad_target"][0]))
    for k, x in zip(keys, grads(pert)):
        if np.all(g_orc[k] == 0):
            assert np.all(x == 0), k
        else:
            assert rel_norm(x, g_orc[k]) <= GRAD_TOL, (k, rel_norm(x, g_orc[k]))
    for k, x, y in zip(keys, grads(None), grads(bary)):
        assert rel_norm(x, y) <= 1e-6 if np.any(y) else np.all(x == 0), k
