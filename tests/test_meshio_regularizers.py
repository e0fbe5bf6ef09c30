"""Scene files (gvr.meshio) and mesh regularisers (gvr.regularizers), CPU only.

The readers are checked on files written here in the formats of the
reference's scenes (and on the reference's own fixtures when they are
present); the sparse regularisers against a dense restatement of the
reference's formulas (python/utils/LaplacianLoss.py:9-33,
IsometryLoss.py:11-70) on a small mesh.
"""
import os
import struct
import zlib

import numpy as np
import pytest

from oracle.refsrc import reference_data

REF_DATA = reference_data()


def _write_png_filtered(path, img8, filters):
    """PNG with the given filter type per row (PNG specification, 6.3)."""
    H, W, C = img8.shape
    prev = np.zeros(W * C, np.int32)
    rows = []
    for y in range(H):
        cur = img8[y].reshape(-1).astype(np.int32)
        f = filters[y % len(filters)]
        left = np.concatenate([np.zeros(C, np.int32), cur[:-C]])
        upleft = np.concatenate([np.zeros(C, np.int32), prev[:-C]])
        if f == 0:
            enc = cur
        elif f == 1:
            enc = cur - left
        elif f == 2:
            enc = cur - prev
        elif f == 3:
            enc = cur - ((left + prev) >> 1)
        else:
            p = left + prev - upleft
            pa, pb, pc = np.abs(p - left), np.abs(p - prev), np.abs(p - upleft)
            pred = np.where((pa <= pb) & (pa <= pc), left, np.where(pb <= pc, prev, upleft))
            enc = cur - pred
        rows.append(bytes([f]) + (enc & 255).astype(np.uint8).tobytes())
        prev = cur

    def chunk(kind, body):
        return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body) & 0xFFFFFFFF)

    with open(path, "wb") as fh:
        fh.write(b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", W, H, 8, {3: 2, 4: 6}[C], 0, 0, 0)) +
                 chunk(b"IDAT", zlib.compress(b"".join(rows))) + chunk(b"IEND", b""))


def test_png_filters_and_round_trip(tmp_path):
    from gvr import meshio
    rng = np.random.default_rng(0)
    img8 = rng.integers(0, 256, (9, 7, 3), dtype=np.uint8)
    p = str(tmp_path / "f.png")
    _write_png_filtered(p, img8, [0, 1, 2, 3, 4])
    assert np.array_equal(np.round(meshio.read_png(p) * 255).astype(np.uint8), img8)
    q = str(tmp_path / "w.png")
    meshio.write_png(q, img8 / 255.0)
    assert np.array_equal(np.round(meshio.read_png(q) * 255).astype(np.uint8), img8)


def test_obj_mtl_segmentation(tmp_path):
    from gvr import meshio
    (tmp_path / "m.mtl").write_text("newmtl a\nKd 0.8 0.8 0.8\nmap_Kd tex.png\n")
    meshio.write_png(str(tmp_path / "tex.png"), np.full((4, 5, 3), 0.5))
    (tmp_path / "segmentation.txt").write_text("13\n9\n0\n15\n")
    (tmp_path / "m.obj").write_text(
        "mtllib ./m.mtl\n"
        "v 0 0 0 1 0 0\nv 1 0 0 0 1 0\nv 1 1 0 0 0 1\nv 0 1 0 0.5 0.5 0.5\n"
        "vt 0.0 0.0\nvt 1.0 0.0\nvt 1.0 1.0\nvt 0.0 1.0\n"
        "f 1/1/1 2/2/2 3/3/3\nf 1/1 3/3 4/4\nf 1/1 2/2 3/3 4/4\n")
    m = meshio.read_obj(str(tmp_path / "m.obj"))
    assert m.num_vertices == 4 and m.num_faces == 3          # the quad keeps its first three corners
    assert np.array_equal(m.faces, [[0, 1, 2], [0, 2, 3], [0, 1, 2]])
    assert np.allclose(m.colors[1], [0, 1, 0])
    assert np.allclose(m.uvs[:6], [0, 0, 1, 0, 1, 1])
    assert m.texture.shape == (4, 5, 3) and np.allclose(m.texture, 128 / 255)
    assert np.array_equal(m.labels, [13, 9, 0, 15])
    assert np.allclose(m.weights, [400, 2, 1, 5])
    t = meshio.read_obj(str(tmp_path / "m.obj"), triangulate=True)
    assert t.num_faces == 4 and np.array_equal(t.faces[3], [0, 2, 3])


def test_calibration_rescales_intrinsics(tmp_path):
    from gvr import meshio
    (tmp_path / "c.calibration").write_text(
        "Skeletool Camera Calibration File V1.0\n"
        "name 0\n  sensor 10 10\n  size 1024 512\n  animated 0\n"
        "  intrinsic 700 0 500 0 0 710 260 0 0 0 1 0 0 0 0 1\n"
        "  extrinsic 1 0 0 10 0 1 0 20 0 0 1 3000 0 0 0 1\n  radial 0\n"
        "name 1\n  sensor 10 10\n  size 256 256\n  animated 0\n"
        "  intrinsic 300 0 128 0 0 300 128 0 0 0 1 0 0 0 0 1\n"
        "  extrinsic 0 0 -1 0 0 1 0 0 1 0 0 2500 0 0 0 1\n")
    ex, K = meshio.read_calibration(str(tmp_path / "c.calibration"), 512, 512)
    assert ex.shape == (2, 12) and K.shape == (2, 9)
    assert np.allclose(ex[0], [1, 0, 0, 10, 0, 1, 0, 20, 0, 0, 1, 3000])
    assert np.allclose(K[0], [350, 0, 250, 0, 710, 260, 0, 0, 1])
    assert np.allclose(K[1], [600, 0, 256, 0, 600, 256, 0, 0, 1])


@pytest.mark.skipif(not os.path.isdir(REF_DATA), reason="reference scene files not present")
def test_reference_scene_files():
    from gvr import meshio
    m = meshio.read_obj(os.path.join(REF_DATA, "cone.obj"), load_texture=False)
    assert m.num_vertices == 5 and m.num_faces == 6
    ex, K = meshio.read_calibration(os.path.join(REF_DATA, "cameras.calibration"), 512, 512)
    assert ex.shape == (1, 12) and abs(K[0, 0] - 752.6881 / 2) < 1e-3


def _dense_reference(faces, N, w, verts, rest):
    A = np.zeros((N, N))
    for a, b, c in faces:
        for i, j in ((a, b), (a, c), (b, a), (b, c), (c, a), (c, b)):
            A[i, j] = 1
    deg = A.sum(1)
    E = deg.sum()
    L = -A + np.diag(deg)
    rw = np.array([sum((w[i] + w[j]) / 2 for j in np.nonzero(A[i])[0]) / deg[i] for i in range(N)])
    lap = 0.0
    iso = 0.0
    for b in range(verts.shape[0]):
        d = (verts[b] - rest) / 1000.0
        lap += ((L @ d) ** 2).sum(1) @ rw
        lr = np.linalg.norm(rest[:, None] - rest[None], axis=2) * A
        lb = np.linalg.norm(verts[b][:, None] - verts[b][None], axis=2) * A
        iso += ((lr - lb) ** 2).sum()
    B = verts.shape[0]
    return lap / (B * E), iso / (B * E)


def test_regularizers_match_dense_restatement():
    import torch
    from gvr import regularizers, scenes
    v, f, _ = scenes.displaced_sphere(80, 1000.0, 20.0, np.random.default_rng(1))
    N = v.shape[0]
    rng = np.random.default_rng(2)
    w = rng.choice([1.0, 2.0, 5.0, 400.0], N)
    verts = v[None] + rng.normal(0, 15, (2, N, 3))
    edges = regularizers.MeshEdges(f, N, w)
    vt = torch.tensor(verts, dtype=torch.float64)
    rt = torch.tensor(v, dtype=torch.float64)
    lap = regularizers.laplacian_loss(edges, vt, rt)
    iso = regularizers.isometry_loss(edges, vt, rt)
    ref_lap, ref_iso = _dense_reference(f, N, w, verts.astype(np.float64), v.astype(np.float64))
    assert abs(float(lap) - ref_lap) <= 1e-6 * abs(ref_lap)
    assert abs(float(iso) - ref_iso) <= 1e-6 * abs(ref_iso)
    vt.requires_grad_(True)
    (regularizers.laplacian_loss(edges, vt, rt) + regularizers.isometry_loss(edges, vt, rt)).backward()
    assert torch.isfinite(vt.grad).all()
