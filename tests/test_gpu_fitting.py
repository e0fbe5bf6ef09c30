"""Analysis-by-synthesis fitting (gvr.fitting) on the GPU.

The photometric-loss gradient w.r.t. the model parameters -- the renderer's
backward kernels chained with torch through the linear model, pose and SH --
is checked against FP64 central differences (h = 1e-4) of the same loss
computed with the oracle's FP64 render at the GPU's visibility, over the
pixels whose normal the renderer does not flip toward the camera: there the
reference's position gradient chains the lighting Jacobian of the flipped
normal with the Jacobian of the unflipped normalisation
(CUDABasedRasterizationGrad.cu:231-240, :458-470), so it is not the loss's
derivative.  Shape and pose are checked twice: with the reference's
gradient and constant colours (it leaves out the colour's change through
the barycentrics, :489), and with per-vertex colours and the
GVR_BACKWARD_ALBEDO_POSITION option that adds that term.  Tolerance: 1e-3
relative (norm over the checked coordinates).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FD_H = 1e-4
FD_TOL = 1e-3


def _setup(constant_albedo=None, seed=0):
    import torch
    from gvr.fitting import Fitter, MorphableModel, make_targets
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    model = MorphableModel(num_vertices=2562, seed=seed, device=dev, constant_albedo=constant_albedo)
    fitter = Fitter(model, num_views=2, size=128)
    gt, target = make_targets(fitter, np.random.default_rng(seed))
    return model, fitter, gt, target


def _oracle_render(model, fitter, face, theta):
    from gvr.fitting import PARAM_SLICES
    from oracle.oracle import OracleScene
    C, S = fitter.C, fitter.size
    o = OracleScene(model.faces, model.uvs, model.mean.cpu().numpy(), model.albedo_mean.cpu().numpy(),
                    np.zeros((1, 1, 3), np.float32), np.zeros((C, 27), np.float32), fitter.extr.cpu().numpy(),
                    fitter.intr.cpu().numpy(), S, S, "vertexColor", "shaded")
    sh = np.tile(np.asarray(theta, np.float64)[PARAM_SLICES["sh"]], (C, 1))
    return o.render_fp64(face, verts_d=model.vertices_fp64(theta), colors_d=model.colors_fp64(theta), sh_d=sh)


def _check_fd(model, fitter, theta, target, idx):
    """Relative error of the GPU gradient of the photometric loss over the
    pixels whose normal is not flipped and whose view ray is not grazing
    (there the function is too curved for a 1e-4 central difference),
    against central differences."""
    import torch
    p = torch.tensor(theta[None], device=model.device, requires_grad=True)
    img, face = fitter.render(p, with_face=True)
    face = face[0].cpu().numpy()
    _, flags = _oracle_render(model, fitter, face, theta)
    keep = (flags == 0)[..., None].astype(np.float64)   # neither flipped nor grazing (|cos| < 0.002)
    mask = torch.from_numpy(keep.astype(np.float32)).to(model.device)[None]
    per = fitter.loss(img * mask, target * mask)
    g, = torch.autograd.grad(per.sum(), p)
    g = g[0].double().cpu().numpy()
    tgt = target[0].double().cpu().numpy()

    def loss(t):
        r, _ = _oracle_render(model, fitter, face, t)
        return float(np.mean(((r - tgt) * keep) ** 2))

    fd = []
    for k in idx:
        tp, tm = theta.astype(np.float64).copy(), theta.astype(np.float64).copy()
        tp[k] += FD_H
        tm[k] -= FD_H
        fd.append((loss(tp) - loss(tm)) / (2 * FD_H))
    fd = np.array(fd)
    err = np.linalg.norm(g[idx] - fd) / np.linalg.norm(fd)
    return err, g[idx], fd


def test_fit_gradient_sh_and_albedo_match_fd():
    model, fitter, gt, target = _setup(seed=1)
    theta = gt[0].copy()
    theta[166:193] += 0.05
    theta[80:160] += np.random.default_rng(2).normal(0, 0.5, 80).astype(np.float32)
    idx = list(range(166, 193)) + list(range(80, 160, 10))
    err, g, fd = _check_fd(model, fitter, theta, target, idx)
    assert err <= FD_TOL, (err, g, fd)


def _shape_pose_theta(gt, seed):
    theta = gt[0].copy()
    theta[0:80] += np.random.default_rng(seed).normal(0, 0.3, 80).astype(np.float32)
    theta[160:163] += np.float32([0.01, 0.02, -0.01])
    theta[163:166] += np.float32([3.0, -2.0, 1.0])
    return theta


def test_fit_gradient_shape_and_pose_match_fd_reference_gradient():
    """The reference's gradient (no albedo term) with constant colours."""
    import torch
    from gvr.fitting import Fitter
    model, _, gt, _ = _setup(constant_albedo=0.5, seed=3)
    fitter = Fitter(model, num_views=2, size=128, albedo_position=False)
    theta = _shape_pose_theta(gt, 4)
    theta[80:160] = 0.0  # constant albedo: the reference's position gradient is the loss's derivative
    with torch.no_grad():
        target = fitter.render(torch.from_numpy(gt).to(model.device))
    idx = list(range(0, 80, 10)) + list(range(160, 166))
    err, g, fd = _check_fd(model, fitter, theta, target, idx)
    assert err <= FD_TOL, (err, g, fd)


def test_fit_gradient_shape_and_pose_match_fd_with_albedo_term():
    """Per-vertex colours with GVR_BACKWARD_ALBEDO_POSITION: the position
    gradient includes the colour's change through the barycentrics."""
    model, fitter, gt, target = _setup(seed=6)
    theta = _shape_pose_theta(gt, 7)
    idx = list(range(0, 80, 10)) + list(range(160, 166))
    err, g, fd = _check_fd(model, fitter, theta, target, idx)
    assert err <= FD_TOL, (err, g, fd)


def test_fit_recovers_lighting():
    """From the true geometry, pose and albedo with the mean lighting, 150
    Adam steps on the SH coefficients alone (every other step size zero,
    no decay) cut the photometric RMSE to under a fifth, steadily, and the
    fit records the RMSE and GPU time of every step.  (With geometry and
    albedo free as well, they drift to absorb the wrong shading and the
    RMSE stalls near 0.04: the lighting is identified only with the rest
    held.)"""
    model, fitter, gt, target = _setup(seed=5)
    init = gt.copy()
    init[:, 166:193] = 0.0
    init[:, [166, 175, 184]] = 0.85
    frozen = dict(shape=0.0, albedo=0.0, rot=0.0, trans=0.0)
    res = fitter.fit(target, init, steps=150, goal=0.001, lr=frozen, decay=1.0)
    r = res.rmse[:, 0]
    assert r[0] > 0.03
    assert r[-1] < r[0] / 5, r[::10]
    assert np.allclose(res.params[0, :166], gt[0, :166])
    assert np.all(r[10::10] <= r[:-10:10] * 1.05), r[::10]   # no divergence
    assert res.step_ms.shape == (151,) and np.all(np.diff(res.step_ms) >= 0)


def _outline_mismatch(fitter, params, target):
    """Fraction of pixels that only one of render and target covers."""
    import torch
    bg = torch.tensor([0.0, 1.0, 0.0], device=target.device)
    with torch.no_grad():
        _, face = fitter.render(torch.from_numpy(params).to(target.device), with_face=True)
    return ((face >= 0) ^ ((target - bg).abs().amax(-1) > 0)).float().mean().item()


def test_fit_silhouette_term_pulls_outline():
    """From the true pose, albedo and lighting with the mean shape, the
    silhouette term (distance field to the target's outline handed to the
    renderer as its target image, so the model-to-data gradient moves the
    render's outline pixels) shrinks the outline mismatch to under half
    within 100 steps, and below what the photometric fit alone leaves."""
    from gvr.fitting import Fitter
    model, plain, gt, target = _setup(seed=8)
    init = gt.copy()
    init[:, 0:80] = 0.0
    sil = Fitter(model, num_views=2, size=128, silhouette=0.1)
    lr = dict(shape=0.1, rot=0.02, trans=4.0)
    before = _outline_mismatch(plain, init, target)
    after_sil = _outline_mismatch(plain, sil.fit(target, init, steps=100, lr=lr, decay=0.2).params, target)
    after_plain = _outline_mismatch(plain, plain.fit(target, init, steps=100, lr=lr, decay=0.2).params, target)
    assert before > 0.005, before
    assert after_sil < 0.5 * before, (before, after_sil)
    assert after_sil < after_plain, (after_sil, after_plain)
