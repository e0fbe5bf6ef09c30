"""Batched forward plans (gvr_plan_*): many meshes of uneven size, views,
resolutions and modes in one launch per stage plus one persistent raster.

Every job's face ids, barycentrics, render and vertex normals must equal
gvr_forward on the same inputs bit for bit, under every bin/tile
configuration, with the autotuner, and when the plan is replayed as a CUDA
graph after its inputs changed in place.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KEYS = ("barycentric", "face", "render", "vertex_normal")


def _jobs(seed=7, meshes=6, faces=(400, 6000), res=(48, 64, 96), tex=32):
    from gvr import scenes
    return scenes.uneven_batch(seed=seed, num_meshes=meshes, faces_range=faces, max_views=4, resolutions=res,
                               tex_size=tex)


def _plan_jobs(specs, dev, **extra):
    from gvr import renderer
    out = []
    for s in specs:
        h = renderer.get_handle(s["faces"], s["uvs"], s["num_vertices"], s["num_views"], s["width"], s["height"],
                                s["albedo_mode"], s["shading_mode"], device=dev)
        j = dict(handle=h, vertex_pos=s["vertex_pos"], vertex_color=s["vertex_color"], texture=s["texture"],
                 sh_coeff=s["sh_coeff"], extrinsics=s["extrinsics"], intrinsics=s["intrinsics"])
        j.update(extra)
        out.append(j)
    return out


def _single(job):
    import torch
    from gvr import renderer
    inp = {k: v for k, v in job.items() if k not in ("handle", "tile_width", "big_tiles")}
    bary, face, img, vn, _, _ = renderer.render_forward(job["handle"], inp["vertex_pos"], inp["vertex_color"],
                                                        inp["texture"], inp["sh_coeff"], inp["extrinsics"],
                                                        inp["intrinsics"])
    torch.cuda.synchronize()
    return dict(barycentric=bary.cpu().numpy(), face=face.cpu().numpy(), render=img.cpu().numpy(),
                vertex_normal=vn.cpu().numpy())


def _same(a, b):
    return np.array_equal(np.asarray(a).view(np.uint32), np.asarray(b).view(np.uint32))


def _check(plan, jobs):
    import torch
    torch.cuda.synchronize()
    for j, job in enumerate(jobs):
        ref = _single(job)
        got = plan.outputs[j]
        for k in KEYS:
            assert _same(got[k].cpu().numpy(), ref[k]), (j, k)


@pytest.mark.parametrize("tile_width,big_tiles", [(16, 16), (32, 4), (8, 16), (16, 1)])
def test_plan_matches_single_calls(tile_width, big_tiles):
    import torch
    from gvr.batch import BatchPlan
    dev = torch.device("cuda", 0)
    jobs = _plan_jobs(_jobs(), dev, tile_width=tile_width, big_tiles=big_tiles)
    plan = BatchPlan(jobs)
    assert all(plan.tile_config(j) == (tile_width, 256 // tile_width, big_tiles) for j in range(len(jobs)))
    plan.forward()
    _check(plan, jobs)
    plan.close()


def test_plan_autotune_and_graph_replay():
    import torch
    from gvr.batch import BatchPlan
    dev = torch.device("cuda", 0)
    specs = _jobs(seed=11, meshes=5)
    jobs = _plan_jobs(specs, dev)
    plan = BatchPlan(jobs, autotune=True)
    for j in range(len(jobs)):
        w, h, b = plan.tile_config(j)
        assert w in (8, 16, 32) and w * h == 256 and b in (4, 16)
    stream = torch.cuda.Stream(dev)
    with torch.cuda.stream(stream):
        plan.forward(stream=stream, graph=True)
    stream.synchronize()
    _check(plan, [dict(j, **{"vertex_pos": plan.inputs[i]["vertex_pos"]}) for i, j in enumerate(jobs)])
    # move every mesh and replay the captured graph: outputs follow the new inputs
    for i, inp in enumerate(plan.inputs):
        inp["vertex_pos"].mul_(1.05)
        inp["sh_coeff"].add_(0.1)
    with torch.cuda.stream(stream):
        plan.forward(stream=stream, graph=True)
    stream.synchronize()
    moved = [dict(j, vertex_pos=plan.inputs[i]["vertex_pos"], sh_coeff=plan.inputs[i]["sh_coeff"])
             for i, j in enumerate(jobs)]
    _check(plan, moved)
    plan.close()


def test_plan_batch_of_two_and_one_view_jobs():
    import torch
    from gvr import scenes
    from gvr.batch import BatchPlan
    dev = torch.device("cuda", 0)
    a = scenes.scene(1280, 3, 40, 40, "textured", tex_size=16, seed=3, batch=2)
    b = scenes.scene(720, 1, 72, 72, "vertexColor", seed=4)
    jobs = _plan_jobs([a, b], dev)
    plan = BatchPlan(jobs)
    plan.forward()
    _check(plan, jobs)
    plan.close()


def test_plan_refuses_normal_map_handles_and_bad_tiles():
    import ctypes
    import torch
    from gvr import _lib, renderer, scenes
    from gvr.batch import BatchPlan
    dev = torch.device("cuda", 0)
    s = scenes.scene(720, 1, 32, 32, "textured", tex_size=8, seed=5)
    h = renderer.get_handle(s["faces"], s["uvs"], s["num_vertices"], 1, 32, 32, "textured", "shaded",
                            compute_normal_map=True, device=dev)
    job = dict(handle=h, vertex_pos=s["vertex_pos"], texture=s["texture"], sh_coeff=s["sh_coeff"],
               extrinsics=s["extrinsics"], intrinsics=s["intrinsics"])
    with pytest.raises(_lib.GvrError) as e:
        BatchPlan([job])
    assert e.value.status == -5
    job = _plan_jobs([s], dev, tile_width=12)[0]
    with pytest.raises(_lib.GvrError) as e:
        BatchPlan([job])
    assert e.value.status == -1
    L = _lib.load()
    assert L.gvr_plan_create(None, 0, 0, ctypes.byref(ctypes.c_void_p())) == -1


def test_full_uneven_workload_against_single_calls_and_oracle():
    """The whole uneven workload of the batched bench (64 displaced spheres,
    1k..200k faces, 1..8 views at 256/512/1024^2, mixed modes, 512^2
    textures), autotuned and replayed as a CUDA graph: every job equals
    gvr_forward bit for bit, and sampled (job, view) pairs -- the densest
    mesh at its lowest resolution, the largest at its highest, the smallest,
    and three drawn at random -- equal the FP64 oracle (face ids,
    barycentrics, vertex normals bit-exact; render 1e-5) given the device's
    rays."""
    import torch
    from gvr import scenes
    from gvr.batch import BatchPlan
    from helpers import oracle_scene, rel_max
    dev = torch.device("cuda", 0)
    specs = scenes.uneven_batch(seed=0, num_meshes=64)
    jobs = _plan_jobs(specs, dev)
    plan = BatchPlan(jobs, autotune=True)
    stream = torch.cuda.Stream(dev)
    with torch.cuda.stream(stream):
        plan.forward(stream=stream, graph=True)
        plan.forward(stream=stream, graph=True)   # a replay writes the same bits
    stream.synchronize()
    _check(plan, jobs)
    F = [s["faces"].shape[0] for s in specs]
    R = [s["width"] for s in specs]
    big = max(F)
    picks = {min((j for j in range(len(specs)) if F[j] == big), key=lambda j: R[j]),
             max((j for j in range(len(specs)) if F[j] == big), key=lambda j: R[j]),
             min(range(len(specs)), key=lambda j: F[j])}
    rng = np.random.default_rng(5)
    picks |= set(int(x) for x in rng.choice(len(specs), size=3, replace=False))
    for j in sorted(picks):
        s, out, h = specs[j], plan.outputs[j], plan.handles[j]
        c = int(rng.integers(0, s["num_views"]))
        rays = h.debug_rays(plan.inputs[j]["extrinsics"], plan.inputs[j]["intrinsics"]).cpu().numpy()[0]
        one = dict(s, num_views=1, sh_coeff=s["sh_coeff"][:, c:c + 1], extrinsics=s["extrinsics"][:, c:c + 1],
                   intrinsics=s["intrinsics"][:, c:c + 1])
        ref = oracle_scene(one, 0, rays=rays[c:c + 1]).forward()
        face = out["face"].cpu().numpy()[0, c]
        assert np.array_equal(face, ref["face"][0]), (j, c, int((face != ref["face"][0]).sum()))
        assert _same(out["barycentric"].cpu().numpy()[0, c], ref["bary"][0]), (j, c)
        assert _same(out["vertex_normal"].cpu().numpy()[0, c], ref["vertex_normal"][0]), (j, c)
        assert rel_max(out["render"].cpu().numpy()[0, c], ref["render"][0]) <= 1e-5, (j, c)
    plan.close()
