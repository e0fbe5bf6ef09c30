"""Seeded synthetic scenes for the renderer's workloads.

All lengths are millimetres.  The reference's ray/triangle test divides
positions by 1000 and rejects a triangle when |dot(dir, N)| < 1e-7 with the
un-normalised cross product N (cpp/src/Utils/RendererUtil.h:29-47), so a
unit-radius mesh of thousands of faces renders nothing; its own fixture
scenes are in millimetres (python/data/cameras.calibration places the camera
3.3 m away).  A similarity transform leaves the images unchanged, so every
workload here is the unit-scale description scaled by 1000.

Camera convention (as cpp/src/Utils/CameraUtil.h:141-186 uses it): the
extrinsics are the world->camera [R|t] (3x4, row-major), camera z looks
forward, image v grows downwards, intrinsics are the 3x3 K (row-major).
"""
from __future__ import annotations

import functools
import math

import numpy as np

# ----------------------------------------------------------------------------- meshes


def _icosahedron():
    t = (1.0 + 5 ** 0.5) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t],
                  [0, 1, -t], [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4],
                  [11, 10, 2], [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8],
                  [3, 8, 9], [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], np.int64)
    n = np.cross(v[f[:, 1]] - v[f[:, 0]], v[f[:, 2]] - v[f[:, 0]])
    flip = (n * v[f].sum(1)).sum(1) < 0
    f[flip] = f[flip][:, ::-1]
    return v, f


@functools.lru_cache(maxsize=16)
def geodesic_sphere(freq: int):
    """Frequency-`freq` geodesic icosphere on the unit sphere: 10 f^2 + 2
    vertices, 20 f^2 faces, outward counter-clockwise winding."""
    iv, ifc = _icosahedron()
    pts, tris = [], []
    base = 0
    for a, b, c in ifc:
        A, B, C = iv[a], iv[b], iv[c]
        idx = {}
        for i in range(freq + 1):
            for j in range(freq + 1 - i):
                idx[(i, j)] = base + len(idx)
                pts.append(A + (B - A) * (i / freq) + (C - A) * (j / freq))
        for i in range(freq):
            for j in range(freq - i):
                tris.append((idx[(i, j)], idx[(i + 1, j)], idx[(i, j + 1)]))
                if i + j <= freq - 2:
                    tris.append((idx[(i + 1, j)], idx[(i + 1, j + 1)], idx[(i, j + 1)]))
        base += len(idx)
    pts = np.array(pts)
    pts /= np.linalg.norm(pts, axis=1, keepdims=True)
    key = np.round(pts * 1e9).astype(np.int64)
    _, first, inv = np.unique(key, axis=0, return_index=True, return_inverse=True)
    order = np.argsort(first)                      # keep first-seen order
    remap = np.empty_like(order)
    remap[order] = np.arange(order.size)
    verts = pts[first[order]]
    faces = remap[inv.reshape(-1)][np.array(tris)]
    assert verts.shape[0] == 10 * freq * freq + 2 and faces.shape[0] == 20 * freq * freq
    return verts, faces


def _split_edges(verts, faces, nsplit):
    """Split `nsplit` longest edges (pairwise face-disjoint, ties broken by
    vertex ids) at their midpoints projected back onto the unit sphere.
    Each split adds one vertex and two faces."""
    if nsplit == 0:
        return verts, faces
    F = faces.shape[0]
    e = np.concatenate([faces[:, [0, 1]], faces[:, [1, 2]], faces[:, [2, 0]]])
    fid = np.tile(np.arange(F), 3)
    lo, hi = np.minimum(e[:, 0], e[:, 1]), np.maximum(e[:, 0], e[:, 1])
    length = np.linalg.norm(verts[lo] - verts[hi], axis=1)
    order = np.lexsort((hi, lo, -np.round(length, 12)))
    used = np.zeros(F, bool)
    chosen = {}
    owner = {}
    for k in order:
        key = (int(lo[k]), int(hi[k]))
        owner.setdefault(key, []).append(int(fid[k]))
    seen = set()
    for k in order:
        key = (int(lo[k]), int(hi[k]))
        if key in seen:
            continue
        seen.add(key)
        fs = owner[key]
        if len(fs) != 2 or used[fs].any():
            continue
        used[fs] = True
        chosen[key] = fs
        if len(chosen) == nsplit:
            break
    assert len(chosen) == nsplit, "not enough disjoint edges to split"
    new_verts = [verts]
    faces = faces.copy()
    extra = []
    nv = verts.shape[0]
    for (a, b), fs in chosen.items():
        m = verts[a] + verts[b]
        new_verts.append((m / np.linalg.norm(m))[None])
        for f in fs:
            tri = list(faces[f])
            k = [i for i in range(3) if {tri[i], tri[(i + 1) % 3]} == {a, b}][0]
            p, q, r = tri[k], tri[(k + 1) % 3], tri[(k + 2) % 3]
            faces[f] = (p, nv, r)
            extra.append((nv, q, r))
        nv += 1
    return np.concatenate(new_verts), np.concatenate([faces, np.array(extra, faces.dtype)])


@functools.lru_cache(maxsize=16)
def sphere_mesh(num_faces: int):
    """Closed genus-0 unit-sphere mesh with exactly `num_faces` faces (even):
    a geodesic sphere of frequency floor(sqrt(F/20)) plus longest-edge splits.
    35,002 V / 70,000 F is frequency 59 (34,812 V / 69,620 F) + 190 splits."""
    if num_faces % 2 or num_faces < 20:
        raise ValueError("a closed triangle mesh needs an even face count >= 20")
    freq = max(1, int(math.isqrt(num_faces // 20)))
    v, f = geodesic_sphere(freq)
    v, f = _split_edges(v, f, (num_faces - f.shape[0]) // 2)
    return v, f


def displaced_sphere(num_faces, radius_mm=1000.0, sigma_mm=20.0, rng=None):
    """Sphere mesh displaced along its normals by N(0, sigma^2) (mm)."""
    rng = np.random.default_rng(0) if rng is None else rng
    v, f = sphere_mesh(num_faces)
    r = radius_mm + rng.normal(0.0, sigma_mm, size=v.shape[0])
    return (v * r[:, None]).astype(np.float32), f.astype(np.int32), v


def spherical_uvs(unit_verts, faces):
    """Per-face-corner spherical (u, v) in [0, 1] with the seam unwrapped:
    a face that straddles the u seam gets u + 1 on its low corners (the
    renderer clamps texture coordinates to the texture)."""
    x, y, z = unit_verts[:, 0], unit_verts[:, 1], unit_verts[:, 2]
    u = 0.5 + np.arctan2(x, z) / (2 * np.pi)
    v = 0.5 + np.arcsin(np.clip(y, -1, 1)) / np.pi
    fu, fv = u[faces], v[faces]
    seam = (fu.max(1) - fu.min(1)) > 0.5
    fu[seam] = np.where(fu[seam] < 0.5, fu[seam] + 1.0, fu[seam])
    return np.stack([fu, fv], axis=2).reshape(-1, 6).astype(np.float32)


# ----------------------------------------------------------------------------- cameras


def look_at_extrinsics(center):
    """World->camera [R|t] for a camera at `center` looking at the origin,
    image v downwards (world y is up)."""
    c = np.asarray(center, np.float64)
    z = -c / np.linalg.norm(c)
    up = np.array([0.0, 1.0, 0.0])
    x = np.cross(z, up)
    x /= np.linalg.norm(x)
    y = np.cross(z, x)
    R = np.stack([x, y, z])
    t = -R @ c
    return np.concatenate([R, t[:, None]], axis=1).astype(np.float32).reshape(12)


def intrinsics(width, height, fov_deg=40.0):
    f = (width / 2.0) / math.tan(math.radians(fov_deg / 2.0))
    return np.array([f, 0, width / 2.0, 0, f, height / 2.0, 0, 0, 1], np.float32)


def ring_cameras(n, distance_mm=3000.0, pitch_range_deg=15.0, rng=None, yaw0_deg=0.0):
    rng = np.random.default_rng(0) if rng is None else rng
    ext = []
    for k in range(n):
        yaw = math.radians(yaw0_deg + 360.0 * k / n)
        pitch = math.radians(rng.uniform(-pitch_range_deg, pitch_range_deg)) if pitch_range_deg else 0.0
        cen = distance_mm * np.array([math.sin(yaw) * math.cos(pitch), math.sin(pitch),
                                      -math.cos(yaw) * math.cos(pitch)])
        ext.append(look_at_extrinsics(cen))
    return np.stack(ext)


def sh_coefficients(num_views, rng, band0=0.8, sigma=0.1):
    sh = rng.normal(0.0, sigma, size=(num_views, 27))
    sh[:, [0, 9, 18]] = band0
    return sh.astype(np.float32)


# ----------------------------------------------------------------------------- workloads


def scene(num_faces, num_views, width, height, albedo_mode, shading_mode="shaded", tex_size=1,
          sigma_mm=20.0, pitch_range_deg=15.0, seed=0, batch=1):
    """One renderer workload as a dict of float32/int32 numpy arrays with a
    leading batch dimension on the per-call inputs."""
    rng = np.random.default_rng(seed)
    verts, faces, unit = displaced_sphere(num_faces, 1000.0, sigma_mm, rng)
    uvs = spherical_uvs(unit, faces)
    N = verts.shape[0]
    out = dict(faces=faces, uvs=uvs, num_vertices=N, num_views=num_views, width=width, height=height,
               albedo_mode=albedo_mode, shading_mode=shading_mode)
    out["vertex_pos"] = np.stack([verts] * batch)
    out["vertex_color"] = rng.uniform(0, 1, size=(batch, N, 3)).astype(np.float32)
    out["texture"] = rng.uniform(0, 1, size=(batch, tex_size, tex_size, 3)).astype(np.float32)
    out["sh_coeff"] = np.stack([sh_coefficients(num_views, rng) for _ in range(batch)])
    cams = ring_cameras(num_views, 3000.0, pitch_range_deg, rng)
    out["extrinsics"] = np.stack([cams] * batch)
    out["intrinsics"] = np.stack([np.stack([intrinsics(width, height)] * num_views)] * batch)
    out["target_image"] = np.zeros((batch, num_views, height, width, 3), np.float32)
    out["grad_render"] = rng.normal(0, 1, size=(batch, num_views, height, width, 3)).astype(np.float32)
    out["grad_target"] = np.zeros((batch, num_views, height, width, 3), np.float32)
    return out


ALBEDO_MODES = ("vertexColor", "textured", "normal", "lighting", "foregroundMask")
SHADING_MODES = ("shaded", "shadeless")


def uneven_batch(seed=0, num_meshes=64, faces_range=(1000, 200000), max_views=8, resolutions=(256, 512, 1024),
                 tex_size=512, sigma_mm=20.0):
    """Batched uneven workload: `num_meshes` displaced spheres with face
    counts log-uniform in `faces_range` (rounded to even), 1..max_views ring
    views each, every view's resolution drawn from `resolutions`, albedo and
    shading modes drawn from the reference's 5 x 2 set, textures
    tex_size^2 U[0, 1].  The reference op renders all its cameras at one
    resolution, so the views of a mesh that share a resolution form one job.
    Returns a list of job dicts in scene()'s layout (batch 1) with the mesh
    index under "mesh"."""
    rng = np.random.default_rng(seed)
    lo, hi = math.log(faces_range[0]), math.log(faces_range[1])
    jobs = []
    for m in range(num_meshes):
        F = max(20, int(round(math.exp(rng.uniform(lo, hi)) / 2.0)) * 2)
        views = int(rng.integers(1, max_views + 1))
        res = rng.choice(np.asarray(resolutions), size=views)
        albedo = ALBEDO_MODES[int(rng.integers(0, len(ALBEDO_MODES)))]
        shading = SHADING_MODES[int(rng.integers(0, len(SHADING_MODES)))]
        verts, faces, unit = displaced_sphere(F, 1000.0, sigma_mm, rng)
        uvs = spherical_uvs(unit, faces)
        N = verts.shape[0]
        colors = rng.uniform(0, 1, size=(1, N, 3)).astype(np.float32)
        texture = rng.uniform(0, 1, size=(1, tex_size, tex_size, 3)).astype(np.float32)
        cams = ring_cameras(views, 3000.0, 15.0, rng, yaw0_deg=float(rng.uniform(0, 360)))
        sh = sh_coefficients(views, rng)
        for r in sorted(set(int(x) for x in res)):
            sel = np.nonzero(res == r)[0]
            C = len(sel)
            jobs.append(dict(mesh=m, faces=faces, uvs=uvs, num_vertices=N, num_views=C, width=r, height=r,
                             albedo_mode=albedo, shading_mode=shading, vertex_pos=verts[None], vertex_color=colors,
                             texture=texture, sh_coeff=sh[sel][None], extrinsics=cams[sel][None],
                             intrinsics=np.stack([intrinsics(r, r)] * C)[None]))
    return jobs


def single_view_vertex_color(seed=0):
    """Plain fwd+bwd: 2,562 V / 5,120 F displaced icosphere (sigma 20 mm),
    vertex colours, SH-shaded, one 256x256 view 3 m away, 40 deg FOV."""
    return scene(5120, 1, 256, 256, "vertexColor", "shaded", tex_size=1, sigma_mm=20.0,
                 pitch_range_deg=0.0, seed=seed)


def multiview_textured(seed=0, width=1024, tex_size=1024, num_views=8):
    """Textured multi-view SH render: 35,002 V / 70,000 F (sigma 30 mm),
    1024^2 texture, 8 ring views 45 deg apart with pitch U[-15, 15] deg,
    1024x1024."""
    return scene(70000, num_views, width, width, "textured", "shaded", tex_size=tex_size, sigma_mm=30.0,
                 pitch_range_deg=15.0, seed=seed)
