"""The synthetic workloads (gvr.scenes) that stand in for the reference's
demo scenes: exact face counts, closed meshes, UV ranges, camera geometry
and the uneven batch, all on the host."""
import numpy as np
import pytest

from gvr import scenes


@pytest.mark.parametrize("F", [20, 5120, 70000])
def test_sphere_mesh_has_exact_face_count_and_is_closed(F):
    v, f = scenes.sphere_mesh(F)
    assert f.shape == (F, 3)
    assert v.shape[0] == F // 2 + 2                       # Euler: V - E + F = 2 with E = 3F/2
    assert np.allclose(np.linalg.norm(v, axis=1), 1.0, atol=1e-6)
    e = np.sort(np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]]), axis=1)
    _, counts = np.unique(e, axis=0, return_counts=True)
    assert np.all(counts == 2)                             # every edge shared by exactly two faces
    n = np.cross(v[f[:, 1]] - v[f[:, 0]], v[f[:, 2]] - v[f[:, 0]])
    assert np.all((n * v[f].mean(1)).sum(1) > 0)          # consistently outward


def test_sphere_mesh_rejects_odd_counts():
    with pytest.raises(ValueError):
        scenes.sphere_mesh(101)


def test_spherical_uvs_unwrap_the_seam():
    v, f = scenes.sphere_mesh(5120)
    uv = scenes.spherical_uvs(v, f).reshape(-1, 3, 2)
    assert uv[..., 1].min() >= 0.0 and uv[..., 1].max() <= 1.0
    assert uv[..., 0].min() >= 0.0 and uv[..., 0].max() <= 1.5
    away = np.abs(v[f][:, :, 1]).max(1) < 0.98              # u is ill-defined at the poles
    assert (uv[away, :, 0].max(1) - uv[away, :, 0].min(1)).max() < 0.5   # no face spans the seam


def test_ring_cameras_look_at_the_origin():
    E = scenes.ring_cameras(8, 3000.0, 15.0, np.random.default_rng(0)).reshape(-1, 3, 4).astype(np.float64)
    for e in E:
        R, t = e[:, :3], e[:, 3]
        assert np.allclose(R @ R.T, np.eye(3), atol=1e-5)
        centre = -R.T @ t
        assert abs(np.linalg.norm(centre) - 3000.0) < 1e-2
        assert np.allclose(R @ np.zeros(3) + t, [0, 0, 3000.0], atol=1e-2)   # origin straight ahead
    K = scenes.intrinsics(1024, 1024).reshape(3, 3)
    assert abs(K[0, 0] - 512.0 / np.tan(np.radians(20.0))) < 1e-3 and K[0, 2] == 512.0


def test_workloads_have_the_configured_sizes():
    s0 = scenes.single_view_vertex_color(seed=0)
    assert s0["faces"].shape[0] == 5120 and s0["num_vertices"] == 2562 and s0["width"] == 256
    s1 = scenes.multiview_textured(seed=0, width=64, tex_size=16)
    assert s1["faces"].shape[0] == 70000 and s1["num_vertices"] == 35002 and s1["num_views"] == 8
    assert s1["vertex_pos"].dtype == np.float32 and s1["grad_render"].shape == (1, 8, 64, 64, 3)


def test_uneven_batch_spans_the_configured_ranges():
    specs = scenes.uneven_batch(seed=0, num_meshes=64)
    assert len(specs) >= 64
    F = np.array([s["faces"].shape[0] for s in specs])
    assert F.min() >= 1000 and F.max() <= 200000 and np.all(F % 2 == 0)
    assert {s["width"] for s in specs} <= {256, 512, 1024}
    assert all(1 <= s["num_views"] <= 8 for s in specs)
