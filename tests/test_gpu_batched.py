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


@pytest.mark.parametrize("persistent", [False, True], ids=["lanes", "persistent"])
@pytest.mark.parametrize("tile_width,big_tiles", [(16, 16), (32, 4), (8, 16), (16, 1)])
def test_plan_matches_single_calls(tile_width, big_tiles, persistent):
    import torch
    from gvr.batch import BatchPlan
    dev = torch.device("cuda", 0)
    jobs = _plan_jobs(_jobs(), dev, tile_width=tile_width, big_tiles=big_tiles)
    plan = BatchPlan(jobs, persistent=persistent)
    assert all(plan.tile_config(j) == (tile_width, 256 // tile_width, big_tiles) for j in range(len(jobs)))
    plan.forward()
    _check(plan, jobs)
    plan.close()


@pytest.mark.parametrize("persistent", [False, True], ids=["lanes", "persistent"])
def test_plan_autotune_and_graph_replay(persistent):
    import torch
    from gvr.batch import BatchPlan
    dev = torch.device("cuda", 0)
    specs = _jobs(seed=11, meshes=5)
    jobs = _plan_jobs(specs, dev)
    plan = BatchPlan(jobs, autotune=True, persistent=persistent)
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


# ---------------------------------------------------------------------------- batched backward

GRAD_KEYS = ("vertex_pos", "vertex_color", "texture", "sh_coeff")


def _grads_per_call(plan, j):
    """render_backward of job j on the plan's buffers (the reference's per-element call)."""
    import torch
    from gvr import renderer
    inp, out, g = plan.inputs[j], plan.outputs[j], plan.grad_inputs[j]
    h = plan.handles[j]
    tex = inp["texture"] if inp["texture"] is not None else torch.zeros((inp["vertex_pos"].shape[0], 1, 1, 3),
                                                                      device=h.device)
    vc = inp["vertex_color"] if inp["vertex_color"] is not None else torch.zeros_like(inp["vertex_pos"])
    r = renderer.render_backward(h, g["grad_render"], inp["vertex_pos"], vc, tex, inp["sh_coeff"], g["target_image"],
                                 out["vertex_normal"], out["barycentric"], out["face"], g["grad_target"],
                                 inp["extrinsics"], inp["intrinsics"])
    torch.cuda.synchronize()
    return dict(zip(GRAD_KEYS, (x.cpu().numpy() for x in r)))


def _check_grads(plan, jobs, rng=None, oracle_sample=0):
    """Every job: the batched gradients equal the per-call backward up to the
    order of FP32 atomic sums (||a - b|| <= 1e-6 ||b||; SH bit for bit);
    `oracle_sample` jobs also against the FP64 oracle at the parity bar."""
    import torch
    from helpers import oracle_scene, rel_norm
    torch.cuda.synchronize()
    for j in range(len(jobs)):
        ref = _grads_per_call(plan, j)
        got = {k: plan.grads[j][k].cpu().numpy() for k in GRAD_KEYS}
        assert _same(got["sh_coeff"], ref["sh_coeff"]), (j, "sh_coeff")
        for k in GRAD_KEYS:
            if np.all(ref[k] == 0):
                assert np.all(got[k] == 0), (j, k)
            else:
                assert rel_norm(got[k], ref[k]) <= 1e-6, (j, k, rel_norm(got[k], ref[k]))
    if oracle_sample and rng is not None:
        for j in rng.choice(len(jobs), size=min(oracle_sample, len(jobs)), replace=False):
            s = jobs[int(j)]["spec"]
            out, g = plan.outputs[j], plan.grad_inputs[j]
            rays = plan.handles[j].debug_rays(plan.inputs[j]["extrinsics"], plan.inputs[j]["intrinsics"]).cpu().numpy()
            o = oracle_scene(s, 0, rays=rays[0])
            gt = g["grad_target"].cpu().numpy()[0] if g["grad_target"] is not None else \
                np.zeros(g["grad_render"].shape[1:], np.float32)
            tgt = g["target_image"].cpu().numpy()[0] if g["target_image"] is not None else np.zeros_like(gt)
            orc = o.backward(out["face"].cpu().numpy()[0], out["barycentric"].cpu().numpy()[0],
                             out["vertex_normal"].cpu().numpy()[0], g["grad_render"].cpu().numpy()[0], tgt, gt)
            for k in GRAD_KEYS:
                mine, theirs = plan.grads[j][k].cpu().numpy()[0], orc[k + "_grad"]
                if np.all(theirs == 0):
                    assert np.all(mine == 0), (int(j), k)
                else:
                    assert rel_norm(mine, theirs) <= 1e-4, (int(j), k, rel_norm(mine, theirs))


def _bind_random_backward(plan, specs, rng, target_every=3):
    grads, targets, images = [], [], []
    for j, s in enumerate(specs):
        shape = (1, s["num_views"], s["height"], s["width"], 3)
        grads.append(rng.normal(0, 1, shape).astype(np.float32))
        with_t = j % target_every == 1
        targets.append(rng.normal(0, 1, shape).astype(np.float32) if with_t else None)
        images.append(rng.uniform(0, 1, shape).astype(np.float32) if with_t else None)
    plan.bind_backward(grads, targets, images)


def test_plan_backward_matches_single_calls_and_oracle():
    """Mixed modes (every albedo x shading mode of the reference, with and
    without the model-to-data term) through one batched backward."""
    import torch
    from gvr.batch import BatchPlan
    dev = torch.device("cuda", 0)
    specs = _jobs(seed=13, meshes=8)
    jobs = _plan_jobs(specs, dev)
    for j, s in zip(jobs, specs):
        j["spec"] = s
    plan = BatchPlan([{k: v for k, v in j.items() if k != "spec"} for j in jobs])
    plan.forward()
    rng = np.random.default_rng(13)
    _bind_random_backward(plan, specs, rng)
    plan.backward()
    _check_grads(plan, jobs, rng, oracle_sample=4)
    plan.close()


def test_plan_backward_graph_replay_follows_new_gradients():
    import torch
    from gvr.batch import BatchPlan
    dev = torch.device("cuda", 0)
    specs = _jobs(seed=17, meshes=5)
    jobs = _plan_jobs(specs, dev)
    plan = BatchPlan(jobs)
    stream = torch.cuda.Stream(dev)
    rng = np.random.default_rng(17)
    with torch.cuda.stream(stream):
        plan.forward(stream=stream, graph=True)
        _bind_random_backward(plan, specs, rng)
        plan.backward(stream=stream, graph=True)
    stream.synchronize()
    _check_grads(plan, jobs)
    for g in plan.grad_inputs:                       # new upstream gradients, same buffers
        g["grad_render"].mul_(-0.5).add_(0.25)
    with torch.cuda.stream(stream):
        plan.backward(stream=stream, graph=True)
    stream.synchronize()
    _check_grads(plan, jobs)
    plan.close()


def test_plan_backward_refuses_a_wrong_job_count():
    import ctypes
    import torch
    from gvr import _lib
    from gvr.batch import BatchPlan
    dev = torch.device("cuda", 0)
    plan = BatchPlan(_plan_jobs(_jobs(seed=3, meshes=2), dev))
    L = _lib.load()
    assert L.gvr_plan_bind_backward(plan._plan, (_lib.GvrBackwardArgs * 1)(), 1) == -1
    assert L.gvr_plan_backward(plan._plan, None) == -1          # nothing bound
    plan.close()


def test_full_uneven_workload_backward():
    """The batched bench's whole uneven workload, forward and backward through
    the plan's graphs: every job's gradients equal the per-call backward,
    four sampled jobs equal the FP64 oracle."""
    import torch
    from gvr import scenes
    from gvr.batch import BatchPlan
    dev = torch.device("cuda", 0)
    specs = scenes.uneven_batch(seed=0, num_meshes=64)
    jobs = _plan_jobs(specs, dev)
    for j, s in zip(jobs, specs):
        j["spec"] = s
    plan = BatchPlan([{k: v for k, v in j.items() if k != "spec"} for j in jobs], autotune=True)
    stream = torch.cuda.Stream(dev)
    rng = np.random.default_rng(29)
    with torch.cuda.stream(stream):
        plan.forward(stream=stream, graph=True)
        _bind_random_backward(plan, specs, rng, target_every=7)
        plan.backward(stream=stream, graph=True)
    stream.synchronize()
    _check_grads(plan, jobs, rng, oracle_sample=4)
    plan.close()
