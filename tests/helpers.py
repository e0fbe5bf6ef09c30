"""Shared test helpers: small seeded scenes and comparison metrics."""
from __future__ import annotations

import numpy as np

from gvr import scenes


def small_scene(num_faces=1280, views=2, size=64, albedo="vertexColor", shading="shaded", tex=16, seed=0,
                batch=1, sigma=20.0, pitch=15.0):
    s = scenes.scene(num_faces, views, size, size, albedo, shading, tex_size=tex, sigma_mm=sigma,
                     pitch_range_deg=pitch, seed=seed, batch=batch)
    return s


def oracle_scene(s, b=0, rays=None, albedo=None, shading=None, image_filter_size=1):
    from oracle.oracle import OracleScene
    return OracleScene(s["faces"], s["uvs"], s["vertex_pos"][b], s["vertex_color"][b], s["texture"][b],
                       s["sh_coeff"][b], s["extrinsics"][b], s["intrinsics"][b], s["width"], s["height"],
                       albedo or s["albedo_mode"], shading or s["shading_mode"], image_filter_size, rays=rays)


def rel_norm(a, b):
    """||a - b|| / ||b|| (FP64)."""
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / nb if nb > 0 else np.linalg.norm(a)


def rel_max(a, b):
    """max |a - b| / max |b| (FP64)."""
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    mb = np.abs(b).max() if b.size else 0.0
    return np.abs(a - b).max() / mb if mb > 0 else np.abs(a).max() if a.size else 0.0


def interior_mask(s, b, fwd, rays, ties, cos_min=0.1):
    """Pixels where the reference's FP32 position gradient is well
    conditioned: covered, one face at the minimal depth, the face seen at
    |cos(ray, face normal)| >= cos_min, and the interpolated normal facing
    the camera at least 0.02 away from the flip decision (on flipped pixels
    the reference chains the flipped normal's lighting Jacobian with the
    unflipped normalisation, CUDABasedRasterizationGrad.cu:231-240, 458-470)."""
    face, bary, vn = fwd["face"], fwd["bary"].astype(np.float64), fwd["vertex_normal"].astype(np.float64)
    V = s["vertex_pos"][b].astype(np.float64)
    covered = face >= 0
    idx = s["faces"][np.where(covered, face, 0)]                      # [C,H,W,3]
    v0, v1, v2 = V[idx[..., 0]], V[idx[..., 1]], V[idx[..., 2]]
    Nf = np.cross(v1 - v0, v2 - v0)
    d = rays.astype(np.float64)
    d /= np.linalg.norm(d, axis=-1, keepdims=True)
    cos = np.abs((d * Nf).sum(-1)) / np.maximum(np.linalg.norm(Nf, axis=-1), 1e-300)
    c = np.arange(face.shape[0])[:, None, None]
    a0, a1 = bary[..., 0:1], bary[..., 1:2]
    n = a0 * vn[c, idx[..., 0]] + a1 * vn[c, idx[..., 1]] + (1.0 - a0 - a1) * vn[c, idx[..., 2]]
    nd = (n * d).sum(-1) / np.maximum(np.linalg.norm(n, axis=-1), 1e-300)
    return covered & (ties <= 1) & (cos >= cos_min) & (nd <= -0.02)
