"""The reference's own kernels (compiled from its sources for sm_103a,
oracle/refcore.py) against the new kernels and the oracle, on the GPU.

Visibility is compared with the reference built with -fmad=false, whose
FP32 expression sequence the new kernels reproduce: face ids must be equal
on every pixel whose minimal quantised depth is unique; where several faces
share it the reference's choice (a write race) must be one of them and ours
the smallest.  Barycentrics and vertex normals must be bit-identical.  The
nvcc-default reference build (FMA contraction) is reported, not asserted.
Reference gradients are FP32 with atomics; they are checked against the
FP64 oracle at the tolerance FP32 accumulation allows.
"""
import numpy as np
import pytest

from helpers import interior_mask, oracle_scene, rel_max, rel_norm, small_scene
from test_gpu_parity import check_batch, run_gpu

pytestmark = pytest.mark.gpu

refcore = pytest.importorskip("oracle.refcore")
if not refcore.available():
    pytest.skip("reference kernels not built (oracle/_ref missing)", allow_module_level=True)


@pytest.fixture(scope="module")
def ref_nofma():
    return refcore.Refcore(fmad=False)


@pytest.fixture(scope="module")
def ref_default():
    return refcore.Refcore(fmad=True)


def compare_visibility(s, ours, ref, tag="", b=0):
    o = oracle_scene(s, b, rays=ours["rays"][b])
    orc = o.forward()
    uniq = orc["ties"] <= 1
    f_ref, f_ours = ref["face"], ours["face"][b]
    assert np.array_equal(f_ref[uniq], f_ours[uniq]), f"{tag}: {(f_ref[uniq] != f_ours[uniq]).sum()} unique-depth mismatches"
    tie = ~uniq
    if tie.any():
        assert np.all(np.any(orc["tie_faces"][tie] == f_ref[tie][:, None], axis=1) | (orc["ties"][tie] > orc["tie_faces"].shape[-1]))
        assert np.array_equal(f_ours[tie], orc["face"][tie])
    same = f_ref == f_ours
    assert np.array_equal(ref["bary"][same].view(np.uint32), ours["bary"][b][same].view(np.uint32))
    assert np.array_equal(ref["vertex_normal"].view(np.uint32), ours["vertex_normal"][b].view(np.uint32))
    assert rel_max(ours["render"][b][same], ref["render"][same]) <= 1e-5
    return orc, int(tie.sum())


def _time_ours(s, reps=20):
    """Mean ms of one render_forward + render_backward call pair on the
    scene (CUDA events around `reps` calls after 3 warm-up calls)."""
    import torch
    from gvr import renderer
    from test_gpu_parity import _handle, _tensors
    h, t = _handle(s, None, None, 1), _tensors(s)

    def once():
        bary, face, img, vn, _, _ = renderer.render_forward(h, t["vertex_pos"], t["vertex_color"], t["texture"],
                                                            t["sh_coeff"], t["extrinsics"], t["intrinsics"])
        renderer.render_backward(h, t["grad_render"], t["vertex_pos"], t["vertex_color"], t["texture"], t["sh_coeff"],
                                 t["target_image"], vn, bary, face, None, t["extrinsics"], t["intrinsics"], 0)
    for _ in range(3):
        once()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        once()
    e1.record()
    e1.synchronize()
    return e0.elapsed_time(e1) / reps


MODES = [("vertexColor", "shaded"), ("textured", "shaded"), ("textured", "shadeless"), ("normal", "shaded"),
         ("lighting", "shadeless"), ("foregroundMask", "shaded")]


@pytest.mark.parametrize("albedo,shading", MODES)
def test_forward_matches_reference_kernels(ref_nofma, albedo, shading):
    s = small_scene(num_faces=1280, views=2, size=64, albedo=albedo, shading=shading, tex=16, seed=21)
    ours = run_gpu(s)
    ref = ref_nofma.forward(s)
    compare_visibility(s, ours, ref, albedo)


def test_workloads_match_reference_kernels(ref_nofma, ref_default):
    from gvr import scenes
    for s in (scenes.single_view_vertex_color(seed=0), scenes.multiview_textured(seed=0)):
        ours = run_gpu(s)
        ref = ref_nofma.forward(s)
        _, ties = compare_visibility(s, ours, ref, "workload")
        d = ref_default.forward(s)
        mism = (d["face"] != ours["face"][0]).mean()
        g = ref_default.backward(s, d)
        print(f"\n{s['num_views']}x{s['width']}^2, F={s['faces'].shape[0]}: tie pixels {ties}, "
              f"default-build (FMA) face mismatch rate {mism:.2e}, reference kernels: forward "
              f"{d['ms']:.2f} ms, backward {g['ms']:.2f} ms (default build), forward {ref['ms']:.2f} ms (-fmad=false); "
              f"this build through renderer.render_forward/backward: {_time_ours(s):.3f} ms fwd+bwd")
        assert mism < 0.01


@pytest.mark.parametrize("albedo,shading", [("vertexColor", "shaded"), ("textured", "shaded"),
                                            ("textured", "shadeless"), ("foregroundMask", "shaded")])
def test_reference_gradients_vs_oracle(ref_nofma, albedo, shading):
    s = small_scene(num_faces=1280, views=2, size=64, albedo=albedo, shading=shading, tex=16, seed=22)
    rng = np.random.default_rng(22)
    s["target_image"] = rng.uniform(0, 1, s["target_image"].shape).astype(np.float32)
    s["grad_target"] = rng.normal(0, 1, s["grad_target"].shape).astype(np.float32)
    fwd = ref_nofma.forward(s)
    g_ref = ref_nofma.backward(s, fwd, with_target=True)
    o = oracle_scene(s, 0)
    g_orc = o.backward(fwd["face"], fwd["bary"], fwd["vertex_normal"], s["grad_render"][0], s["target_image"][0],
                       s["grad_target"][0])
    for k in ("vertex_color_grad", "texture_grad", "sh_coeff_grad"):
        if np.all(g_orc[k] == 0):
            assert np.all(g_ref[k] == 0), k
        else:
            assert rel_norm(g_ref[k], g_orc[k]) < 1e-4, (k, rel_norm(g_ref[k], g_orc[k]))
    # FP32 Jacobians near grazing incidence: a looser bound for positions
    assert rel_norm(g_ref["vertex_pos_grad"], g_orc["vertex_pos_grad"]) < 2e-2


# ---------------------------------------------------------------------------- position gradient, pinned

def _pin_position_gradient(ref, s, with_target, b=0):
    """The reference kernels, the FP64 oracle and this build's backward on
    the same pixels (upstream gradients zeroed off the interior mask)."""
    ours = run_gpu(s)
    o = oracle_scene(s, b, rays=ours["rays"][b])
    orc = o.forward()
    fwd = ref.forward(s, b)
    mask = interior_mask(s, b, fwd, ours["rays"][b], orc["ties"])
    assert mask.sum() > 0.3 * (fwd["face"] >= 0).sum(), (mask.sum(), (fwd["face"] >= 0).sum())
    m = dict(s)
    m["grad_render"] = s["grad_render"] * mask[None, ..., None]
    m["grad_target"] = s["grad_target"] * mask[None, ..., None]
    g_ref = ref.backward(m, fwd, b, with_target=with_target)
    gt = m["grad_target"][b] if with_target else np.zeros_like(m["grad_target"][b])
    g_orc = o.backward(fwd["face"], fwd["bary"], fwd["vertex_normal"], m["grad_render"][b], m["target_image"][b], gt)
    g_ours = run_gpu(m, with_target=with_target)
    e_ref = rel_norm(g_ref["vertex_pos_grad"], g_orc["vertex_pos_grad"])
    e_ours = rel_norm(g_ours["vertex_pos_grad"][b], g_orc["vertex_pos_grad"])
    print(f"\ninterior pixels {mask.mean():.3f}: vertex_pos_grad rel err reference kernels {e_ref:.2e}, "
          f"this build {e_ours:.2e} (vs the FP64 oracle)")
    return e_ref, e_ours


PIN_CASES = [("vertexColor", "shaded", False), ("textured", "shaded", False), ("vertexColor", "shaded", True),
             ("textured", "shadeless", True)]


@pytest.mark.parametrize("albedo,shading,target", PIN_CASES)
def test_position_gradient_pinned_to_reference_kernels(ref_nofma, albedo, shading, target):
    """vertex_pos_grad of the reference's own kernels equals the FP64 oracle
    to 1e-4 on the interior pixels (and so does this build's): the shading
    term (dJBCDVerpos, RendererUtil.h:670-861), the model-to-data term
    (CUDABasedRasterizationGrad.cu:531-555) and the normal-adjacency term
    (:559-615).  The all-pixel comparison of
    test_reference_gradients_vs_oracle keeps its looser bound."""
    s = small_scene(num_faces=1280, views=2, size=64, albedo=albedo, shading=shading, tex=16, seed=23)
    rng = np.random.default_rng(23)
    s["target_image"] = rng.uniform(0, 1, s["target_image"].shape).astype(np.float32)
    s["grad_target"] = rng.normal(0, 1, s["grad_target"].shape).astype(np.float32)
    e_ref, e_ours = _pin_position_gradient(ref_nofma, s, target)
    assert e_ref <= 1e-4 and e_ours <= 1e-4, (e_ref, e_ours)


def test_position_gradient_pinned_on_single_view_workload(ref_nofma):
    """The same pin on the 2,562 V / 5,120 F vertex-colour workload at 256^2."""
    from gvr import scenes
    s = scenes.single_view_vertex_color(seed=0)
    e_ref, e_ours = _pin_position_gradient(ref_nofma, s, False)
    assert e_ref <= 1e-4 and e_ours <= 1e-4, (e_ref, e_ours)


# ---------------------------------------------------------------------------- the reference's own scenes

def _fixture_scene(name, albedo, shading, batch, seed):
    """A scene of oracle/refscenes.py (the reference's demo data) as a scene
    dict.  Batch element 0 holds the demo's inputs; later elements perturb
    the SH coefficients by U[0, 0.5), the starting point of
    python/test_gradients_SphericalHarmonics.py:87."""
    from oracle import refscenes
    sc = refscenes.load(name)
    if sc is None:
        pytest.skip(f"scene {name} not built (oracle/_ref/scene_{name}.npz; needs the reference's data files)")
    C, (H, W) = sc["extrinsics"].shape[0], (int(x) for x in sc["size"])
    rng = np.random.default_rng(seed)
    rep = lambda a: np.repeat(np.asarray(a, np.float32)[None], batch, axis=0)
    sh = rep(sc["sh_coeff"])
    sh[1:] += rng.uniform(0, 0.5, sh[1:].shape).astype(np.float32)
    return dict(faces=sc["faces"], uvs=sc["uvs"], num_vertices=sc["vertex_pos"].shape[0], num_views=C, width=W,
                height=H, albedo_mode=albedo, shading_mode=shading, vertex_pos=rep(sc["vertex_pos"]),
                vertex_color=rep(sc["vertex_color"]), texture=rep(sc["texture"]), sh_coeff=sh,
                extrinsics=rep(sc["extrinsics"]), intrinsics=rep(sc["intrinsics"]),
                target_image=rng.uniform(0, 1, (batch, C, H, W, 3)).astype(np.float32),
                grad_render=rng.normal(0, 1, (batch, C, H, W, 3)).astype(np.float32),
                grad_target=rng.normal(0, 1, (batch, C, H, W, 3)).astype(np.float32))


# (scene, albedo, shading, batch): the demos' render modes and batch sizes,
# python/test_gradients_Texture.py:61-125 (textured, shadeless, 1),
# test_gradients_VertexColor.py:32-120 and test_gradients_SphericalHarmonics.py:31-121
# (vertexColor, shaded, 3), test_render.py:21-66 (cone, vertexColor, shaded, 2)
FIXTURE_CASES = [("magdalena", "textured", "shadeless", 1), ("magdalena", "vertexColor", "shaded", 3),
                 ("magdalena", "textured", "shaded", 1), ("cone", "vertexColor", "shaded", 2)]


@pytest.mark.parametrize("name,albedo,shading,batch", FIXTURE_CASES)
def test_reference_fixture_scenes(ref_nofma, name, albedo, shading, batch):
    """The reference's own scenes (real camera, open mesh, per-face-corner
    UV seams) through gvr_forward / gvr_backward against the reference's
    kernels (-fmad=false) and the FP64 oracle, with the bars of the other
    parity tests: face ids on unique-depth pixels, barycentrics and vertex
    normals bit-exact, render 1e-5; gradients 1e-4 against the oracle
    (ours: all four; the reference's: colour, texture and SH, and positions
    on the interior pixels)."""
    s = _fixture_scene(name, albedo, shading, batch, seed=51)
    ours = run_gpu(s)
    for b in range(batch):
        ref = ref_nofma.forward(s, b)
        assert (ref["face"] >= 0).mean() > 0.01
        compare_visibility(s, ours, ref, f"{name}[{b}]", b=b)
    check_batch(s, ours)
    fwd = ref_nofma.forward(s, 0)
    g_ref = ref_nofma.backward(s, fwd, 0)
    o = oracle_scene(s, 0)
    g_orc = o.backward(fwd["face"], fwd["bary"], fwd["vertex_normal"], s["grad_render"][0], s["target_image"][0],
                       np.zeros_like(s["grad_target"][0]))
    for k in ("vertex_color_grad", "texture_grad", "sh_coeff_grad"):
        if np.all(g_orc[k] == 0):
            assert np.all(g_ref[k] == 0), k
        else:
            assert rel_norm(g_ref[k], g_orc[k]) < 1e-4, (k, rel_norm(g_ref[k], g_orc[k]))
    if shading == "shaded":
        e_ref, e_ours = _pin_position_gradient(ref_nofma, s, False)
        assert e_ref <= 1e-4 and e_ours <= 1e-4, (e_ref, e_ours)
