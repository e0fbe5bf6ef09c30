"""The reference's Python operator surface (python/CudaRenderer.py) on the GPU:
constructor kwargs, getters, autograd, the zero-gradient rules, and headless
versions of the reference's three recovery demos
(python/test_gradients_{SphericalHarmonics,VertexColor,Texture}.py) with
numeric assertions in place of image windows."""
import numpy as np
import pytest

from helpers import small_scene

pytestmark = pytest.mark.gpu


def _renderer(s, **kw):
    import torch
    from gvr import CudaRendererGpu
    dev = torch.device("cuda", 0)
    args = dict(faces_attr=s["faces"].reshape(-1).tolist(), texCoords_attr=s["uvs"].reshape(-1).tolist(),
                numberOfVertices_attr=s["num_vertices"], numberOfCameras_attr=s["num_views"],
                renderResolutionU_attr=s["width"], renderResolutionV_attr=s["height"],
                albedoMode_attr=s["albedo_mode"], shadingMode_attr=s["shading_mode"], image_filter_size_attr=1,
                texture_filter_size_attr=1,
                vertexPos_input=torch.from_numpy(s["vertex_pos"]).to(dev),
                vertexColor_input=torch.from_numpy(s["vertex_color"]).to(dev),
                texture_input=torch.from_numpy(s["texture"]).to(dev),
                shCoeff_input=torch.from_numpy(s["sh_coeff"]).to(dev),
                targetImage_input=torch.from_numpy(s["target_image"]).to(dev),
                extrinsics_input=s["extrinsics"].reshape(s["extrinsics"].shape[0], -1).tolist(),
                intrinsics_input=s["intrinsics"].reshape(s["intrinsics"].shape[0], -1).tolist(),
                nodeName="test")
    args.update(kw)
    return CudaRendererGpu(**args)


def test_getters_shapes_and_dtypes():
    import torch
    s = small_scene(views=2, size=48, batch=2)
    r = _renderer(s)
    B, C, H, W, N = 2, 2, 48, 48, s["num_vertices"]
    assert r.getBaryCentricBufferTF().shape == (B, C, H, W, 2)
    assert r.getFaceBufferTF().shape == (B, C, H, W) and r.getFaceBufferTF().dtype == torch.int32
    assert r.getRenderBufferTF().shape == (B, C, H, W, 3)
    assert r.getTargetBufferTF().shape == (B, C, H, W, 3)
    assert r.getVertexNormalTF().shape == (B, C, N, 3)
    m = r.getModelMaskTF()
    assert m.shape == (B, C, H, W, 3) and m.dtype == torch.float32
    assert torch.equal(m[..., 0] > 0, r.getFaceBufferTF() >= 0)
    assert r.getNormalMap() is None


def test_target_image_out_is_a_copy_of_target_image():
    """Output 4 of the forward op is target_image copied device to device
    (cpp/src/TensorflowOperators/CudaRenderer/CudaRenderer.cpp:286): equal
    bytes, in a buffer of its own, for every batch element and view."""
    import torch
    from gvr import renderer
    s = small_scene(views=2, size=48, batch=2)
    rng = np.random.default_rng(3)
    s["target_image"] = rng.uniform(-2, 2, s["target_image"].shape).astype(np.float32)
    s["target_image"][0, 1, 5, 7] = [np.nan, np.inf, -0.0]          # bytes, not values, are copied
    dev = torch.device("cuda", 0)
    h = renderer.get_handle(s["faces"], s["uvs"], s["num_vertices"], s["num_views"], s["width"], s["height"],
                            s["albedo_mode"], s["shading_mode"], device=dev)
    t = {k: torch.from_numpy(np.ascontiguousarray(s[k])).to(dev)
         for k in ("vertex_pos", "vertex_color", "texture", "sh_coeff", "extrinsics", "intrinsics", "target_image")}
    out = renderer.render_forward(h, t["vertex_pos"], t["vertex_color"], t["texture"], t["sh_coeff"],
                                  t["extrinsics"], t["intrinsics"], target_image=t["target_image"], copy_target=True)
    torch.cuda.synchronize()
    tout = out[4]
    assert tout.data_ptr() != t["target_image"].data_ptr()
    assert np.array_equal(tout.cpu().numpy().view(np.uint32), s["target_image"].view(np.uint32))
    # through the operator surface, too
    r = _renderer(s)
    assert np.array_equal(r.getTargetBufferTF().cpu().numpy().view(np.uint32), s["target_image"].view(np.uint32))


def test_autograd_matches_raw_backward():
    import torch
    from gvr import renderer
    s = small_scene(views=2, size=48, albedo="vertexColor")
    dev = torch.device("cuda", 0)
    vp = torch.from_numpy(s["vertex_pos"]).to(dev).requires_grad_()
    vc = torch.from_numpy(s["vertex_color"]).to(dev).requires_grad_()
    sh = torch.from_numpy(s["sh_coeff"]).to(dev).requires_grad_()
    tex = torch.from_numpy(s["texture"]).to(dev).requires_grad_()
    r = _renderer(s, vertexPos_input=vp, vertexColor_input=vc, shCoeff_input=sh, texture_input=tex)
    G = torch.from_numpy(s["grad_render"]).to(dev)
    (r.getRenderBufferTF() * G).sum().backward()
    h = r.handle
    gp, gc, gt, gs = renderer.render_backward(h, G, vp.detach(), vc.detach(), tex.detach(), sh.detach(),
                                              r.targetImage_input, r.getVertexNormalTF(), None,
                                              r.getFaceBufferTF(), None, r.extrinsics_input, r.intrinsics_input)
    torch.testing.assert_close(vp.grad, gp, rtol=1e-5, atol=1e-6)
    torch.testing.assert_close(vc.grad, gc, rtol=1e-5, atol=1e-6)
    torch.testing.assert_close(sh.grad, gs, rtol=1e-5, atol=1e-6)
    assert torch.all(tex.grad == 0)


@pytest.mark.parametrize("mode", ["normal", "lighting"])
def test_zero_gradient_modes(mode):
    import torch
    s = small_scene(views=1, size=32, albedo=mode)
    dev = torch.device("cuda", 0)
    vp = torch.from_numpy(s["vertex_pos"]).to(dev).requires_grad_()
    sh = torch.from_numpy(s["sh_coeff"]).to(dev).requires_grad_()
    r = _renderer(s, vertexPos_input=vp, shCoeff_input=sh)
    r.getRenderBufferTF().sum().backward()
    assert torch.all(vp.grad == 0) and torch.all(sh.grad == 0)


def test_invalid_mode_raises():
    s = small_scene(views=1, size=16)
    with pytest.raises(ValueError):
        _renderer(s, albedoMode_attr="phong?")


def _fit(s, param, make_kwargs, steps, lr, opt="adam"):
    import torch
    dev = torch.device("cuda", 0)
    target = _renderer(s).getRenderBufferTF().detach()
    losses = []
    optim = torch.optim.Adam([param], lr=lr) if opt == "adam" else torch.optim.SGD([param], lr=lr)
    for _ in range(steps):
        optim.zero_grad()
        img = _renderer(s, **make_kwargs(param)).getRenderBufferTF()
        loss = ((img - target) ** 2).sum()
        loss.backward()
        optim.step()
        losses.append(loss.item())
    return losses


def test_sh_recovery():
    """python/test_gradients_SphericalHarmonics.py: start from SH + U[0, 0.5), Adam."""
    import torch
    s = small_scene(num_faces=1280, views=1, size=64, albedo="vertexColor", seed=1)
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(1)
    sh0 = torch.from_numpy(s["sh_coeff"] + rng.uniform(0, 0.5, s["sh_coeff"].shape).astype(np.float32)).to(dev)
    sh0.requires_grad_()
    losses = _fit(s, sh0, lambda p: dict(shCoeff_input=p), steps=60, lr=0.02)
    assert losses[-1] < 0.05 * losses[0]
    assert all(b <= a * 1.05 for a, b in zip(losses, losses[1:]))


def test_vertex_color_recovery():
    """python/test_gradients_VertexColor.py: start from zeros."""
    import torch
    s = small_scene(num_faces=1280, views=2, size=64, albedo="vertexColor", seed=2)
    dev = torch.device("cuda", 0)
    vc0 = torch.zeros_like(torch.from_numpy(s["vertex_color"])).to(dev).requires_grad_()
    losses = _fit(s, vc0, lambda p: dict(vertexColor_input=p), steps=80, lr=0.05)
    assert losses[-1] < 0.05 * losses[0]


def test_texture_recovery():
    """python/test_gradients_Texture.py: textured + shadeless, start from an all-ones texture."""
    import torch
    s = small_scene(num_faces=1280, views=2, size=64, albedo="textured", shading="shadeless", tex=16, seed=3)
    dev = torch.device("cuda", 0)
    t0 = torch.ones_like(torch.from_numpy(s["texture"])).to(dev).requires_grad_()
    losses = _fit(s, t0, lambda p: dict(texture_input=p), steps=40, lr=0.05)
    assert losses[-1] < 0.02 * losses[0]
