"""Analysis-by-synthesis fitting with the differentiable renderer.

A linear morphable model -- a displaced-sphere mean (mm) plus shape and
albedo bases -- posed by a rigid transform and lit by 27 SH coefficients is
rendered (vertexColor albedo, SH-shaded) into several views and fitted to
target images by Adam on the photometric L2 loss.  The forward and backward
are the renderer's own kernels through RenderFunction; the linear model,
pose and loss are plain torch.

Parameter vector per fit, in this order (PARAM_SLICES): 80 shape and 80
albedo coefficients, pose (rotation vector in radians, translation in mm),
27 SH coefficients shared by all views.
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib, renderer, scenes

N_SHAPE, N_ALBEDO, N_POSE, N_SH = 80, 80, 6, 27
PARAM_SLICES = {"shape": slice(0, 80), "albedo": slice(80, 160), "pose": slice(160, 166), "sh": slice(166, 193)}
N_PARAMS = 193


def smooth_fields(unit, count, sigma, rng, waves=8, freq=2.0):
    """`count` random smooth vector fields on the sphere points `unit` [N, 3]:
    each coordinate a sum of `waves` plane waves cos(w.u + phi) with
    w ~ N(0, freq^2 I), scaled so that every field's values have RMS `sigma`
    (marginally ~N(0, sigma^2) per vertex).  Returns [count, N * 3]."""
    N = unit.shape[0]
    out = np.empty((count, N * 3), np.float64)
    for k in range(count):
        w = rng.normal(0.0, freq, size=(3, waves, 3))
        phi = rng.uniform(0.0, 2.0 * np.pi, size=(3, waves))
        amp = rng.normal(0.0, 1.0, size=(3, waves))
        f = np.einsum("dj,ndj->nd", amp, np.cos(np.einsum("djc,nc->ndj", w, unit) + phi[None]))
        f *= sigma / np.sqrt(np.mean(f * f))
        out[k] = f.reshape(-1)
    return out


class MorphableModel:
    """Mean: a sphere of radius 1000 mm (num_vertices = F/2 + 2) displaced
    along its normals by a smooth field of RMS 20 mm (per-vertex noise of that
    size would make a golf ball whose shading changes chaotically with the
    slightest shift, which no photometric fit can follow); plus `n_shape` shape
    bases (mm) and `n_albedo` albedo bases: smooth random fields whose values
    are N(0, shape_sigma_mm^2) and N(0, albedo_sigma^2) per vertex and
    coordinate (smooth rather than independent per vertex, so that a
    combination of 80 of them is a shape, not per-vertex noise).  Mean albedo
    0.5 plus a smooth field of RMS 0.12, clipped to [0.05, 0.95] (or
    `constant_albedo`)."""

    def __init__(self, num_vertices=28000, n_shape=N_SHAPE, n_albedo=N_ALBEDO, shape_sigma_mm=10.0,
                 albedo_sigma=0.01, seed=0, device=None, constant_albedo=None):
        rng = np.random.default_rng(seed)
        F = 2 * num_vertices - 4
        unit, faces = scenes.sphere_mesh(F)
        faces = faces.astype(np.int32)
        # the mean: the sphere displaced along its normals by a smooth field of RMS 20 mm
        disp = smooth_fields(unit, 1, 20.0, rng)[0].reshape(-1, 3)[:, 0]
        disp *= 20.0 / np.sqrt(np.mean(disp * disp))
        verts = (unit * (1000.0 + disp)[:, None]).astype(np.float32)
        self.faces = faces
        self.uvs = scenes.spherical_uvs(unit, faces)
        self.N, self.F = verts.shape[0], faces.shape[0]
        dev = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        self.device = dev
        f32 = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.float32)).to(dev)
        self.mean = f32(verts)
        self.shape_basis = f32(smooth_fields(unit, n_shape, shape_sigma_mm, rng))
        if constant_albedo is None:
            self.albedo_mean = f32(np.clip(0.5 + smooth_fields(unit, 1, 0.12, rng)[0].reshape(self.N, 3), 0.05, 0.95))
        else:
            self.albedo_mean = torch.full((self.N, 3), float(constant_albedo), device=dev)
        self.albedo_basis = f32(smooth_fields(unit, n_albedo, albedo_sigma, rng))

    def vertices(self, params):
        """[B, N, 3] posed vertices (mm)."""
        B = params.shape[0]
        alpha = params[:, PARAM_SLICES["shape"]]
        pose = params[:, PARAM_SLICES["pose"]]
        v = self.mean.unsqueeze(0) + (alpha @ self.shape_basis).view(B, self.N, 3)
        R = rotation_matrix(pose[:, :3])
        return torch.einsum("bij,bnj->bni", R, v) + pose[:, None, 3:6]

    def colors(self, params):
        B = params.shape[0]
        beta = params[:, PARAM_SLICES["albedo"]]
        return self.albedo_mean.unsqueeze(0) + (beta @ self.albedo_basis).view(B, self.N, 3)

    def vertices_fp64(self, params):
        """FP64 numpy [N, 3] for one parameter vector (finite differences)."""
        p = np.asarray(params, np.float64)
        v = self.mean.double().cpu().numpy() + (p[PARAM_SLICES["shape"]] @ self.shape_basis.double().cpu().numpy()
                                                ).reshape(self.N, 3)
        R = rotation_matrix(torch.from_numpy(p[None, 160:163])).numpy()[0]
        return v @ R.T + p[163:166]

    def colors_fp64(self, params):
        p = np.asarray(params, np.float64)
        return self.albedo_mean.double().cpu().numpy() + (p[PARAM_SLICES["albedo"]] @
                                                          self.albedo_basis.double().cpu().numpy()).reshape(self.N, 3)


def rotation_matrix(rvec):
    """Rodrigues: [B, 3] rotation vectors -> [B, 3, 3] (differentiable, also at 0)."""
    theta2 = (rvec * rvec).sum(-1, keepdim=True)
    theta = torch.sqrt(theta2 + 1e-30)
    small = theta2 < 1e-12
    # sin(t)/t and (1 - cos t)/t^2 with their series near 0
    a = torch.where(small, 1.0 - theta2 / 6.0, torch.sin(theta) / theta)
    b = torch.where(small, 0.5 - theta2 / 24.0, (1.0 - torch.cos(theta)) / torch.clamp(theta2, min=1e-30))
    x, y, z = rvec[:, 0:1], rvec[:, 1:2], rvec[:, 2:3]
    zero = torch.zeros_like(x)
    K = torch.cat([zero, -z, y, z, zero, -x, -y, x, zero], dim=1).view(-1, 3, 3)
    eye = torch.eye(3, dtype=rvec.dtype, device=rvec.device).expand_as(K)
    return eye + a[..., None] * K + b[..., None] * (K @ K)


def fit_cameras(num_views=4, size=512, distance_mm=3000.0):
    """Views on a ring around the model (yaw 0, 360/n, ...), no pitch, 40 deg FOV."""
    extr = scenes.ring_cameras(num_views, distance_mm, 0.0, None)
    intr = np.stack([scenes.intrinsics(size, size)] * num_views)
    return extr, intr


def sample_params(rng, batch=1):
    """Ground-truth parameters: shape and albedo coefficients N(0, 1), yaw
    U[-45, 45] deg (no other rotation, no translation), SH band 0 U[0.5, 1.2]
    per channel and the other coefficients N(0, 0.1^2)."""
    p = np.zeros((batch, N_PARAMS), np.float32)
    p[:, PARAM_SLICES["shape"]] = rng.normal(0.0, 1.0, (batch, N_SHAPE))
    p[:, PARAM_SLICES["albedo"]] = rng.normal(0.0, 1.0, (batch, N_ALBEDO))
    p[:, 161] = np.radians(rng.uniform(-45.0, 45.0, batch))
    sh = rng.normal(0.0, 0.1, (batch, N_SH))
    sh[:, [0, 9, 18]] = rng.uniform(0.5, 1.2, (batch, 3))
    p[:, PARAM_SLICES["sh"]] = sh
    return p


def mean_params(batch=1):
    """The plain fit's start: zero coefficients and pose, SH band 0 at 0.85."""
    p = np.zeros((batch, N_PARAMS), np.float32)
    p[:, [166, 175, 184]] = 0.85
    return p


@dataclass
class FitResult:
    params: np.ndarray                 # [B, 193] final parameters
    rmse: np.ndarray                   # [steps + 1, B] RMSE before each update (last row: final)
    step_ms: np.ndarray                # [steps + 1] GPU time from the start to each RMSE evaluation
    steps_to_goal: list = field(default_factory=list)   # per element: first step with RMSE <= goal, or None
    gpu_ms_to_goal: list = field(default_factory=list)  # per element: GPU ms to that step, or None
    gpu_ms: float = 0.0


class Fitter:
    """Renders a MorphableModel into `num_views` views and fits parameters."""

    # Adam step sizes per parameter group (coefficient units, rad / mm, SH),
    # tuned with the silhouette term on 4 views at 512^2.  LR refines a
    # start near the solution (a proposal); LR_FROM_MEAN, twice as large,
    # suits the plain fit from the mean: over 1,000 held-out draws the plain
    # fit reaches RMSE <= 0.01 in 38 with LR_FROM_MEAN and in none with LR,
    # while fits from the learned proposal reach it in 259 with LR and in
    # 123 with LR_FROM_MEAN.
    LR = {"shape": 0.1, "albedo": 0.15, "rot": 0.02, "trans": 4.0, "sh": 0.03}
    LR_FROM_MEAN = {"shape": 0.2, "albedo": 0.3, "rot": 0.04, "trans": 8.0, "sh": 0.06}
    SILHOUETTE = 0.03   # weight of the silhouette term in the tuned setting

    def __init__(self, model: MorphableModel, num_views=4, size=512, albedo_position=True, model_to_data=False,
                 image_filter_size=1, silhouette=0.0, contour_radius=48):
        """albedo_position: the renderer's backward also moves vertices by
        the change of their interpolated colour (GVR_BACKWARD_ALBEDO_POSITION);
        without it the position gradient is the reference's, which leaves
        that term out and so is not the loss's derivative for per-vertex
        colours.

        model_to_data: the fit's residual compares the render with the
        target as the renderer passes it through (target_image_out), so the
        residual's gradient also reaches the vertices through the target
        image's own gradient at each covered pixel, estimated over an
        image_filter_size window (the reference's model-to-data term,
        CUDABasedRasterizationGrad.cu:531-555): a surface point is pulled
        toward where the target looks like its render, which moves
        silhouettes that the shading gradient alone cannot.

        silhouette > 0: adds silhouette * sum over the render's outline
        pixels of contour_field(target outline) (the distance, in pixels up
        to contour_radius, from the target's outline pixels), per pixel of
        the image.  The field is handed to the renderer as its
        target image, so the same model-to-data term turns the field's
        gradient at each outline pixel into a vertex gradient: the render's
        outline is pulled onto the target's from inside and outside (the
        photometric gradient has no visibility term and cannot move an
        outline)."""
        self.model = model
        self.C, self.size = num_views, size
        self.backward_flags = _lib.BACKWARD_ALBEDO_POSITION if albedo_position else 0
        self.model_to_data = model_to_data
        self.silhouette = float(silhouette)
        self.contour_radius = int(contour_radius)
        if model_to_data and silhouette > 0:
            raise ValueError("model_to_data and silhouette both use the renderer's target image")
        dev = model.device
        self.handle = renderer.get_handle(model.faces, model.uvs, model.N, num_views, size, size, "vertexColor",
                                          "shaded", image_filter_size=image_filter_size, device=dev)
        extr, intr = fit_cameras(num_views, size)
        self.extr = torch.from_numpy(extr).to(dev)
        self.intr = torch.from_numpy(intr).to(dev)
        self._tex = torch.zeros((1, 1, 1, 3), device=dev)

    def render(self, params, with_face=False, target=None):
        """[B, C, H, W, 3] renders of a [B, 193] parameter tensor
        (differentiable), then the face ids if `with_face`, then, if a
        `target` [B, C, H, W, 3] is given, the target as passed through the
        renderer (equal to it; its gradient reaches the vertices through the
        model-to-data term)."""
        B = params.shape[0]
        dev = self.model.device
        V = self.model.vertices(params)
        col = self.model.colors(params)
        sh = params[:, PARAM_SLICES["sh"]].unsqueeze(1).expand(B, self.C, N_SH).contiguous()
        if target is None:
            tgt = torch.zeros((B, self.C, self.size, self.size, 3), device=dev)
        else:
            tgt = target.expand(B, self.C, self.size, self.size, 3).contiguous()
        bary, face, img, vn, tout, _ = renderer.RenderFunction.apply(
            self.handle, V.contiguous(), col.contiguous(), self._tex.expand(B, 1, 1, 3).contiguous(), sh, tgt,
            self.extr.expand(B, self.C, 12).contiguous(), self.intr.expand(B, self.C, 9).contiguous(),
            self.backward_flags)
        out = (img,) + ((face,) if with_face else ()) + ((tout,) if target is not None else ())
        return out if len(out) > 1 else img

    @staticmethod
    def loss(img, target):
        """Photometric L2: mean squared error over every pixel and channel, per batch element."""
        return ((img - target) ** 2).flatten(1).mean(1)

    def fit(self, target, init, steps=200, goal=0.01, fallback=None, lr=None, decay=0.5, objective="interior",
            betas=(0.9, 0.99)):
        """Adam on the photometric L2 loss from `init` [B, 193], step sizes
        decaying geometrically to `decay` times their start over `steps`.
        objective="interior" descends the loss over the pixels that are
        foreground in both the render and the target, one pixel in from
        either silhouette: shading cannot reduce the residual of a pixel
        that only one image covers, and the renderer's gradient is not the
        derivative on the flipped-normal pixels at the silhouette;
        "rendered" uses every pixel the render covers (with model_to_data,
        those the target does not cover pull the silhouette in); "all"
        uses every pixel.  The RMSE recorded (and compared with `goal`) is
        always over every pixel.  Records every element's RMSE per step and
        the GPU time (CUDA events, read back once at the end) to the first
        step at or below `goal`.  `fallback` = (step, threshold, params): at
        `step`, elements whose RMSE exceeds `threshold` restart from `params`
        with fresh Adam state (counting on from the steps already spent)."""
        lr = dict(self.LR, **(lr or {}))
        dev = self.model.device
        p = torch.tensor(np.asarray(init, np.float32), device=dev, requires_grad=True)
        B = p.shape[0]
        scale = torch.ones(N_PARAMS, device=dev)
        groups = {"shape": PARAM_SLICES["shape"], "albedo": PARAM_SLICES["albedo"], "rot": slice(160, 163),
                  "trans": slice(163, 166), "sh": PARAM_SLICES["sh"]}
        for g, sl in groups.items():
            scale[sl] = lr[g]
        # Adam with per-coordinate step sizes (bias-corrected moments)
        m = torch.zeros_like(p)
        v = torch.zeros_like(p)
        (b1, b2), eps = betas, 1e-8
        t_count = torch.zeros(B, 1, device=dev)
        hist = torch.empty((steps + 1, B), device=dev)
        events = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 2)]
        bg = torch.tensor([0.0, 1.0, 0.0], device=dev)
        target_fg = (target - bg).abs().amax(-1) > 0        # the background is exactly (0, 1, 0)
        events[0].record()
        if self.silhouette > 0:
            field = torch.zeros_like(target)
            field[..., 0] = contour_field(target_fg, self.contour_radius)
        for k in range(steps + 1):
            if self.model_to_data:
                img, face, ref = self.render(p, with_face=True, target=target)
            elif self.silhouette > 0:
                img, face, dist = self.render(p, with_face=True, target=field)
                ref = target
            else:
                img, face = self.render(p, with_face=True)
                ref = target
            per = self.loss(img, target)
            rmse = torch.sqrt(per.detach())
            hist[k] = rmse
            events[k + 1].record()
            if k == steps:
                break
            if objective in ("interior", "rendered"):
                keep = interior_mask((face >= 0) & target_fg) if objective == "interior" else (face >= 0).float()
                obj = (((img - ref) ** 2) * keep[..., None]).flatten(1).sum(1) / img[0].numel()
            else:
                obj = self.loss(img, ref)
            if self.silhouette > 0:
                edge = silhouette_pixels(face >= 0)
                obj = obj + self.silhouette * (dist[..., 0] * edge).flatten(1).sum(1) / img[0].numel()
            g, = torch.autograd.grad(obj.sum(), p)
            if fallback is not None and k == fallback[0]:
                bad = rmse > fallback[1]
                if bool(bad.any()):
                    with torch.no_grad():
                        fb = torch.as_tensor(np.asarray(fallback[2], np.float32), device=dev)
                        p[bad] = fb[bad]
                        g[bad] = 0  # the restarted elements take no step from the old point
                        m[bad] = 0
                        v[bad] = 0
                        t_count[bad] = 0
            with torch.no_grad():
                t_count += 1
                m.mul_(b1).add_(g, alpha=1 - b1)
                v.mul_(b2).addcmul_(g, g, value=1 - b2)
                mh = m / (1 - b1 ** t_count)
                vh = v / (1 - b2 ** t_count)
                p -= (scale * decay ** (k / max(steps, 1))) * mh / (vh.sqrt() + eps)
        events[-1].synchronize()
        rm = hist.cpu().numpy()
        ms = np.array([events[0].elapsed_time(e) for e in events[1:]])
        res = FitResult(params=p.detach().cpu().numpy(), rmse=rm, step_ms=ms, gpu_ms=float(ms[-1]))
        for i in range(B):
            hit = np.nonzero(rm[:, i] <= goal)[0]
            res.steps_to_goal.append(int(hit[0]) if hit.size else None)
            res.gpu_ms_to_goal.append(float(ms[hit[0]]) if hit.size else None)
        return res


def interior_mask(fg):
    """[B, C, H, W] bool -> float mask eroded by one pixel (3x3)."""
    B, C, H, W = fg.shape
    outside = (~fg).float().view(B * C, 1, H, W)
    grown = torch.nn.functional.max_pool2d(outside, 3, stride=1, padding=1)
    return (1.0 - grown).view(B, C, H, W)


def contour_field(fg, radius):
    """[B, C, H, W] bool -> float field that is 0 on the outline pixels of
    `fg` (foreground pixels with a background pixel among their 8
    neighbours) and grows by one per pixel away from them on either side:
    d - 1 inside and d outside, d the chessboard distance (pixels, capped at
    `radius`) to the nearest pixel of the other side.  Its minimum is one
    pixel wide and sits exactly on the outline pixels, so the model-to-data
    gradient (a centred difference) of a render outline pixel that already
    lies on the target's outline is zero, while farther pixels feel the
    same pull at any distance.  (A field that is zero on both sides of the
    outline pushes such pixels back and forth by half a pixel.)  Computed
    by `radius` 3x3 dilations of each side."""
    B, C, H, W = fg.shape
    dist = []
    for side in (fg, ~fg):
        x = (~side).float().view(B * C, 1, H, W)     # the other side, grown one pixel per pass
        d = torch.zeros_like(x)
        for _ in range(radius):
            d += 1.0 - x
            x = torch.nn.functional.max_pool2d(x, 3, stride=1, padding=1)
        dist.append(d.view(B, C, H, W))
    return torch.where(fg, dist[0] - 1.0, dist[1])


def silhouette_pixels(fg):
    """[B, C, H, W] bool -> float mask of the foreground pixels with a
    background pixel among their 8 neighbours."""
    B, C, H, W = fg.shape
    bgn = torch.nn.functional.max_pool2d((~fg).float().view(B * C, 1, H, W), 3, stride=1, padding=1)
    return (fg.float().view(B * C, 1, H, W) * bgn).view(B, C, H, W)


def make_targets(fitter: Fitter, rng, batch=1):
    """Ground-truth parameters and their renders [B, C, H, W, 3]."""
    gt = sample_params(rng, batch)
    with torch.no_grad():
        img = fitter.render(torch.from_numpy(gt).to(fitter.model.device))
    return gt, img.detach()
