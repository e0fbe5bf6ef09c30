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
