"""Normal-map mode (compute_normal_map) on the GPU, through the C ABI.

The reference (CUDABasedRasterization.cpp:241-294 and .cu:415-445) writes
the texture-space normal map and leaves the frame cleared.  The GPU result
must equal the oracle bit for bit (FP32 arithmetic in the reference's order,
no contraction), the vertex normals must equal the normal render's, and the
reference's own renderNormalMapDevice (-fmad=false build), fed the oracle's
face map, must give the same texels.
"""
import numpy as np
import pytest

from helpers import oracle_scene, small_scene

pytestmark = pytest.mark.gpu


def _render(s, compute_normal_map):
    import torch
    from gvr import renderer
    dev = torch.device("cuda", 0)
    h = renderer.get_handle(s["faces"], s["uvs"], s["num_vertices"], s["num_views"], s["width"], s["height"],
                            s["albedo_mode"], s["shading_mode"], compute_normal_map=compute_normal_map, device=dev)
    t = {k: torch.from_numpy(np.ascontiguousarray(s[k])).to(dev)
         for k in ("vertex_pos", "vertex_color", "texture", "sh_coeff", "extrinsics", "intrinsics")}
    out = renderer.render_forward(h, t["vertex_pos"], t["vertex_color"], t["texture"], t["sh_coeff"],
                                  t["extrinsics"], t["intrinsics"])
    torch.cuda.synchronize()
    return [None if o is None else o.cpu().numpy() for o in out]


@pytest.mark.parametrize("faces,tex,batch", [(1280, 64, 1), (5120, 96, 2), (20000, 256, 1)])
def test_normal_map_matches_oracle(faces, tex, batch):
    s = small_scene(num_faces=faces, views=2, size=32, albedo="textured", tex=tex, seed=faces, batch=batch)
    bary, face, img, vn, _, nmap = _render(s, True)
    assert np.all(face == -1) and np.all(bary == 0)
    assert np.all(img[..., 0] == 0) and np.all(img[..., 1] == 1) and np.all(img[..., 2] == 0)
    assert nmap.shape == (batch, tex, tex, 3)
    _, _, _, vn_plain, _, _ = _render(s, False)
    assert np.array_equal(vn.view(np.uint32), vn_plain.view(np.uint32))
    for b in range(batch):
        ref = oracle_scene(s, b).normal_map()
        assert np.array_equal(nmap[b].view(np.uint32), ref.view(np.uint32))


def test_normal_map_rectangular_texture_and_overlapping_uvs():
    s = small_scene(num_faces=720, views=1, size=16, albedo="vertexColor", tex=8, seed=5)
    rng = np.random.default_rng(5)
    s["uvs"] = rng.uniform(-0.1, 1.1, s["uvs"].shape).astype(np.float32)   # overlapping UV triangles
    s["texture"] = np.zeros((1, 45, 70, 3), np.float32)
    _, _, _, _, _, nmap = _render(s, True)
    ref = oracle_scene(s).normal_map()
    assert np.array_equal(nmap[0].view(np.uint32), ref.view(np.uint32))


def test_normal_map_reference_kernel():
    from oracle import refcore
    from oracle.oracle import uv_face_map
    if not refcore.available():
        pytest.skip("reference kernels not built")
    s = small_scene(num_faces=5120, views=1, size=16, albedo="textured", tex=128, seed=9)
    _, _, _, vn, _, nmap = _render(s, True)
    owner, abc = uv_face_map(s["uvs"], 128, 128)
    ref = refcore.Refcore(fmad=False)
    try:
        got = ref.normal_map(s["faces"], s["num_vertices"], owner, abc, vn[0, 0])
    finally:
        ref.close()
    assert np.array_equal(nmap[0].view(np.uint32), got.view(np.uint32))
