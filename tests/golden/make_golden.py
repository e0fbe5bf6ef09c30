"""Generates the golden fixtures in this directory by running the reference's
own kernels (compiled from its sources, oracle/refcore.py) on a GPU.

  python tests/golden/make_golden.py [name ...]   # needs a GPU and oracle/_ref; names: only those cases

Each fixture holds the seeded inputs of one small scene, the per-pixel FP32
ray directions the device computes (a CPU cannot reproduce the device rsqrtf
bit for bit), and the reference's outputs: face ids, barycentrics, render,
vertex normals (-fmad=false build) and its gradients.  The *_interior
cases zero the upstream gradients off the pixels where the reference's FP32
position gradient is well conditioned (tests/helpers.py interior_mask).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
for p in (os.path.join(REPO, "gvv-differentiable-cuda-renderer_gb300"), REPO, os.path.join(REPO, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)

CASES = [
    # name, faces, views, size, albedo, shading, texture, seed, with target term
    ("vc_shaded", 1280, 2, 64, "vertexColor", "shaded", 8, 31, True),
    ("tex_shaded", 1280, 2, 64, "textured", "shaded", 16, 32, False),
    ("tex_shadeless", 720, 2, 48, "textured", "shadeless", 16, 33, True),
    ("fg_mask", 720, 1, 48, "foregroundMask", "shaded", 8, 34, True),
    ("normal", 720, 1, 48, "normal", "shaded", 8, 35, False),
    ("lighting", 720, 1, 48, "lighting", "shadeless", 8, 36, False),
]
# the same kind of scenes with the upstream gradients zeroed off the interior
# pixels (tests/helpers.py interior_mask): there the reference's FP32 position
# gradient is well conditioned, and the oracle must match it to 1e-4
INTERIOR_CASES = [
    ("vc_shaded_interior", 1280, 2, 64, "vertexColor", "shaded", 8, 41, True),
    ("tex_shaded_interior", 1280, 2, 64, "textured", "shaded", 16, 42, False),
    ("tex_shadeless_interior", 720, 2, 48, "textured", "shadeless", 16, 43, True),
]


def main():
    import torch
    from gvr import renderer, scenes
    from oracle import refcore

    from helpers import interior_mask, oracle_scene
    ref = refcore.Refcore(fmad=False)
    dev = torch.device("cuda", 0)
    only = set(sys.argv[1:])
    for name, F, C, size, albedo, shading, tex, seed, target in CASES + INTERIOR_CASES:
        if only and name not in only:
            continue
        s = scenes.scene(F, C, size, size, albedo, shading, tex_size=tex, seed=seed)
        rng = np.random.default_rng(seed)
        if target:
            s["target_image"] = rng.uniform(0, 1, s["target_image"].shape).astype(np.float32)
            s["grad_target"] = rng.normal(0, 1, s["grad_target"].shape).astype(np.float32)
        h = renderer.get_handle(s["faces"], s["uvs"], s["num_vertices"], C, size, size, albedo, shading, device=dev)
        rays = h.debug_rays(torch.from_numpy(s["extrinsics"]).to(dev), torch.from_numpy(s["intrinsics"]).to(dev))
        fwd = ref.forward(s)
        interior = name.endswith("_interior")
        if interior:
            r = rays.cpu().numpy()
            ties = oracle_scene(s, 0, rays=r[0]).forward()["ties"]
            mask = interior_mask(s, 0, fwd, r[0], ties)
            s["grad_render"] = s["grad_render"] * mask[None, ..., None]
            s["grad_target"] = s["grad_target"] * mask[None, ..., None]
        out = dict(faces=s["faces"], uvs=s["uvs"], vertex_pos=s["vertex_pos"][0], vertex_color=s["vertex_color"][0],
                   texture=s["texture"][0], sh_coeff=s["sh_coeff"][0], extrinsics=s["extrinsics"][0],
                   intrinsics=s["intrinsics"][0], target_image=s["target_image"][0],
                   grad_render=s["grad_render"][0], grad_target=s["grad_target"][0] if target else
                   np.zeros_like(s["grad_target"][0]), rays=rays.cpu().numpy()[0],
                   ref_face=fwd["face"], ref_bary=fwd["bary"], ref_render=fwd["render"],
                   ref_vertex_normal=fwd["vertex_normal"],
                   meta=np.array([size, size, C], np.int32), modes=np.array([albedo, shading]),
                   interior=np.array(interior))
        if albedo in ("vertexColor", "textured", "foregroundMask"):
            g = ref.backward(s, fwd, with_target=target)
            for k in ("vertex_pos_grad", "vertex_color_grad", "texture_grad", "sh_coeff_grad"):
                out["ref_" + k] = g[k]
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
        print(name, "covered", float((fwd["face"] >= 0).mean()))


if __name__ == "__main__":
    main()
