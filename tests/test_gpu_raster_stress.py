"""Adversarial visibility cases for the raster's skip tests: random triangle
soups that intersect each other, grazing triangles, sub-pixel and
screen-filling triangles (the per-view big list), triangles crossing the
camera plane and coplanar duplicates.  Face ids, barycentrics and vertex
normals must match the oracle bit for bit (ties: smallest face id)."""
import numpy as np
import pytest

from gvr import scenes
from test_gpu_parity import check_batch, run_gpu

pytestmark = pytest.mark.gpu


def soup(seed, n_faces, size=96, spread=600.0, tri_scale=80.0, views=2, near=False):
    rng = np.random.default_rng(seed)
    centres = rng.normal(0, spread, (n_faces, 3))
    verts = (centres[:, None, :] + rng.normal(0, tri_scale, (n_faces, 3, 3))).reshape(-1, 3)
    if near:  # some triangles reach behind the camera plane (camera ~3 m away)
        verts[: 3 * (n_faces // 4)] *= 2.5
    faces = np.arange(3 * n_faces, dtype=np.int32).reshape(-1, 3)
    N = verts.shape[0]
    s = scenes.scene(320, views, size, size, "vertexColor", "shaded", tex_size=8, seed=seed)
    s["faces"] = faces
    s["uvs"] = rng.uniform(0, 1, (n_faces, 6)).astype(np.float32)
    s["num_vertices"] = N
    s["vertex_pos"] = verts[None].astype(np.float32)
    s["vertex_color"] = rng.uniform(0, 1, (1, N, 3)).astype(np.float32)
    return s


@pytest.mark.parametrize("seed", range(4))
def test_random_soup(seed):
    s = soup(seed, 400)
    check_batch(s, run_gpu(s))


def test_big_triangles_and_subpixel_triangles():
    rng = np.random.default_rng(7)
    big = soup(1, 12, tri_scale=900.0)          # boxes spanning many tiles
    tiny = soup(2, 600, tri_scale=2.0)          # sub-pixel triangles
    s = big
    off = big["num_vertices"]
    s["faces"] = np.concatenate([big["faces"], tiny["faces"] + off]).astype(np.int32)
    s["uvs"] = np.concatenate([big["uvs"], tiny["uvs"]]).astype(np.float32)
    s["vertex_pos"] = np.concatenate([big["vertex_pos"], tiny["vertex_pos"]], axis=1)
    s["vertex_color"] = np.concatenate([big["vertex_color"], tiny["vertex_color"]], axis=1)
    s["num_vertices"] = s["vertex_pos"].shape[1]
    check_batch(s, run_gpu(s))


def test_triangles_crossing_the_camera_plane():
    s = soup(3, 300, near=True)
    check_batch(s, run_gpu(s))


def test_grazing_triangles():
    # triangles almost parallel to the view rays of camera 0
    rng = np.random.default_rng(5)
    n = 300
    c = rng.normal(0, 400, (n, 3))
    d = np.stack([np.zeros(n), np.zeros(n), np.ones(n)], 1)      # roughly along the view axis
    side = rng.normal(0, 1, (n, 3))
    side -= (side * d).sum(1, keepdims=True) * d
    side /= np.linalg.norm(side, axis=1, keepdims=True)
    tilt = rng.normal(0, 1e-3, (n, 1)) * side
    v0 = c
    v1 = c + 300 * (d + tilt)
    v2 = c + 60 * side + rng.normal(0, 0.05, (n, 3))
    s = soup(4, n)
    s["vertex_pos"] = np.stack([v0, v1, v2], 1).reshape(1, -1, 3).astype(np.float32)
    check_batch(s, run_gpu(s))


def test_coplanar_duplicates_and_shared_edges():
    s = scenes.scene(720, 2, 80, 80, "vertexColor", "shaded", seed=9, sigma_mm=0.0)
    F0 = s["faces"].shape[0]
    s["faces"] = np.concatenate([s["faces"], s["faces"][::-1]]).astype(np.int32)
    s["uvs"] = np.concatenate([s["uvs"], s["uvs"][::-1]]).astype(np.float32)
    gpu = run_gpu(s)
    check_batch(s, gpu)
    assert np.all(gpu["face"][gpu["face"] >= 0] < F0)


def test_long_slivers_across_warp_blocks():
    """Long thin triangles at random angles: their boxes meet many 8x4 warp
    blocks that the triangles themselves miss (the walk's ballot drops those
    by a corner test), over a sphere that fills the frame behind them."""
    rng = np.random.default_rng(11)
    back = scenes.scene(720, 2, 96, 96, "vertexColor", "shaded", seed=11)
    n = 300
    c = rng.normal(0, 500, (n, 3))
    d = rng.normal(0, 1, (n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    w = rng.normal(0, 1, (n, 3))
    w -= (w * d).sum(1, keepdims=True) * d
    w /= np.linalg.norm(w, axis=1, keepdims=True)
    width = rng.uniform(0.5, 8.0, (n, 1))
    sl = np.stack([c - 700 * d, c + 700 * d, c + width * w], 1).reshape(-1, 3)
    N0, F0 = back["num_vertices"], back["faces"].shape[0]
    s = back
    s["faces"] = np.concatenate([back["faces"], np.arange(3 * n, dtype=np.int32).reshape(-1, 3) + N0]).astype(np.int32)
    s["uvs"] = np.concatenate([back["uvs"], rng.uniform(0, 1, (n, 6))]).astype(np.float32)
    s["vertex_pos"] = np.concatenate([back["vertex_pos"], sl[None].astype(np.float32)], axis=1)
    s["vertex_color"] = np.concatenate([back["vertex_color"], rng.uniform(0, 1, (1, 3 * n, 3)).astype(np.float32)],
                                       axis=1)
    s["num_vertices"] = s["vertex_pos"].shape[1]
    gpu = run_gpu(s)
    check_batch(s, gpu)
    assert (gpu["face"] >= F0).any()   # some sliver is visible


def test_stacked_coplanar_layers_overflow_the_register_candidates():
    """Ten copies of every face: each covered pixel has ten candidates of
    equal depth, more than a pixel keeps in registers, so the resolve takes
    the slow path over the tile's staged entries; ties go to the smallest
    face id."""
    s = scenes.scene(720, 2, 64, 64, "vertexColor", "shaded", seed=12)
    F0 = s["faces"].shape[0]
    s["faces"] = np.concatenate([s["faces"]] * 10).astype(np.int32)
    s["uvs"] = np.concatenate([s["uvs"]] * 10).astype(np.float32)
    gpu = run_gpu(s)
    check_batch(s, gpu)
    assert np.all(gpu["face"][gpu["face"] >= 0] < F0)


def test_dense_tiles_go_through_shared_memory_in_chunks():
    """A 40,000-face sphere at 48x48: a 16x16 tile holds thousands of face
    entries, staged and walked 256 at a time (and, with three stacked
    copies, resolved by the slow path over the bins)."""
    s = scenes.scene(40000, 1, 48, 48, "vertexColor", "shaded", seed=13)
    check_batch(s, run_gpu(s), grads=False)
    F0 = s["faces"].shape[0]
    s["faces"] = np.concatenate([s["faces"]] * 3).astype(np.int32)
    s["uvs"] = np.concatenate([s["uvs"]] * 3).astype(np.float32)
    gpu = run_gpu(s)
    check_batch(s, gpu, grads=False)
    assert np.all(gpu["face"][gpu["face"] >= 0] < F0)
