"""Generates tests/golden/uvmap/*.npz: texture-space face maps of the
normal-map mode computed with the reference's own host ray/triangle test
(rayTriangleIntersectHost, compiled from the reference source by
oracle/refcore.py build_uvmap_ref; needs no GPU).

  python tests/golden/make_golden_uvmap.py   # needs the reference sources

Each fixture holds the per-corner UVs, the texture size and, per texel, the
face the reference's loop leaves there (-1 = none) and its (a, b, c).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
for p in (os.path.join(REPO, "gvv-differentiable-cuda-renderer_gb300"), REPO):
    if p not in sys.path:
        sys.path.insert(0, p)


def odd_uvs(seed=3, count=400):
    """Overlapping, degenerate, tiny and out-of-range UV triangles."""
    rng = np.random.default_rng(seed)
    uv = rng.uniform(-0.2, 1.2, (count, 6)).astype(np.float32)
    uv[:20, 2:4] = uv[:20, 0:2]                                   # two equal corners
    uv[20:40, 2:4] = uv[20:40, 0:2] + np.float32(2e-4)            # far below one texel
    uv[20:40, 4:6] = uv[20:40, 0:2] + np.float32([3e-4, -1e-4])
    uv[40:60, 1::2] = uv[40:60, 1:2]                              # collinear (same v)
    return uv


def main():
    from gvr import scenes
    from oracle import refcore

    if not refcore.build_uvmap_ref():
        raise SystemExit("reference sources not found")
    out_dir = os.path.join(HERE, "uvmap")
    os.makedirs(out_dir, exist_ok=True)
    sphere = scenes.scene(5120, 1, 16, 16, "textured", tex_size=8, seed=0)["uvs"]
    cases = [("sphere_64x64", sphere, 64, 64), ("sphere_96x160", sphere, 96, 160), ("odd_97x61", odd_uvs(), 97, 61)]
    for name, uvs, Ht, Wt in cases:
        owner, abc = refcore.uv_face_map_reference(uvs, Ht, Wt)
        np.savez_compressed(os.path.join(out_dir, name + ".npz"), uvs=np.asarray(uvs, np.float32), owner=owner,
                            abc=abc, size=np.array([Ht, Wt], np.int32))
        print(name, "covered", float((owner >= 0).mean()))


if __name__ == "__main__":
    main()
