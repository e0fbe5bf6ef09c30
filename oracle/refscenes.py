"""The reference's own demo scenes as arrays (test infrastructure only).

build() reads the reference's fixture files in place, where its checkout is
present, and writes one oracle/_ref/scene_<name>.npz per scene.  Like the
compiled reference kernels beside it, that file is a build output kept out
of the repository; the GPU tests load it and skip when it is absent.

  magdalena  python/data/magdalena.obj (10,115 faces, per-face-corner texture
             coordinates, per-vertex colours), its textureMap.png (RGB / 255,
             python/utils/OBJReader.py:208-212), cameras.calibration at
             1024 x 1024 (one camera, intrinsics rescaled as
             python/utils/CameraReader.py:41-46 does), the ground-truth vertex
             positions of data/test_mesh_tensor.getGTMesh (5,118 x 3, mm) and
             the SH coefficients of data/test_SH_tensor.getSHCoeff -- the scene
             of python/test_gradients_{Texture,VertexColor,SphericalHarmonics}.py:31-54.
  cone       python/data/cone.obj with its own vertex positions and colours,
             the same camera and SH -- the scene of python/test_render.py:21-42.

The two data/*.py files are read as text (their number lists), not imported.
"""
from __future__ import annotations

import os
import re
import sys

import numpy as np

from .refsrc import reference_data

_HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(_HERE, "_ref")
RESOLUTION = 1024


def scene_path(name: str) -> str:
    return os.path.join(REF_DIR, f"scene_{name}.npz")


def _numbers_in_array_literal(path: str) -> np.ndarray:
    """The numbers inside the first `np.array([...])` of a Python file."""
    text = open(path).read()
    m = re.search(r"np\.array\(\s*\[(.*?)\]\s*\)", text, re.S)
    if not m:
        raise ValueError(f"{path}: no array literal")
    return np.array([float(x) for x in m.group(1).replace("\n", " ").split(",") if x.strip()], np.float64)


def _meshio():
    pkg = os.path.join(os.path.dirname(_HERE), "gvv-differentiable-cuda-renderer_gb300")
    if pkg not in sys.path:
        sys.path.insert(0, pkg)
    from gvr import meshio
    return meshio


def _scene(obj_name: str, positions=None):
    meshio = _meshio()
    mesh = meshio.read_obj(reference_data(obj_name), load_texture=True, load_segmentation=False)
    texture = mesh.texture if mesh.texture is not None else np.ones((1, 1, 3), np.float32)
    extr, intr = meshio.read_calibration(reference_data("cameras.calibration"), RESOLUTION, RESOLUTION)
    sh = _numbers_in_array_literal(reference_data("test_SH_tensor.py")).astype(np.float32)
    verts = mesh.vertices if positions is None else positions.reshape(mesh.num_vertices, 3).astype(np.float32)
    return dict(faces=mesh.faces.astype(np.int32), uvs=mesh.uvs.astype(np.float32), vertex_pos=verts,
                vertex_color=mesh.colors.astype(np.float32), texture=np.ascontiguousarray(texture, np.float32),
                sh_coeff=np.tile(sh.reshape(1, 27), (extr.shape[0], 1)), extrinsics=extr, intrinsics=intr,
                size=np.array([RESOLUTION, RESOLUTION], np.int32))


def build() -> bool:
    """Writes the scene files; False where the reference checkout is absent."""
    if not os.path.exists(reference_data("magdalena.obj")):
        return False
    os.makedirs(REF_DIR, exist_ok=True)
    gt = _numbers_in_array_literal(reference_data("test_mesh_tensor.py"))
    scenes = {"magdalena": _scene("magdalena.obj", gt), "cone": _scene("cone.obj")}
    for name, arrays in scenes.items():
        np.savez_compressed(scene_path(name), **arrays)
    return True


def load(name: str):
    """dict of one scene (numpy), or None when it was not built."""
    p = scene_path(name)
    if not os.path.exists(p):
        return None
    z = np.load(p)
    return {k: z[k] for k in z.files}
