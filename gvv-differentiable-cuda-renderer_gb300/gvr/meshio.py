"""Mesh, camera and image files in the formats of the reference's scenes.

* OBJ with per-vertex colours (`v x y z r g b`), texture coordinates
  (`vt u v`), faces `f v/t[/n] ...` (1-based) and `mtllib` -> the renderer's
  topology attrs: faces [F, 3], per-face-corner UVs [F * 6], vertex
  positions and colours (python/utils/OBJReader.py:41-108 reads the same
  fields).  Polygons keep their first three corners, as there; triangulate=True
  fans them instead.  A missing texture index gives UV (0, 0).
* MTL `map_Kd` -> the texture as float RGB in [0, 1] (:214-228).
* Skeletool `.calibration` -> extrinsics [C, 12] (the first three rows of the
  4x4 `extrinsic`) and intrinsics [C, 9] (the 3x3 of the 4x4 `intrinsic`)
  with focal lengths and principal point rescaled from each camera's `size`
  to the render resolution (python/utils/CameraReader.py:20-46).
* `segmentation.txt` vertex labels -> per-vertex weights (OBJReader.py:232-283)
  for the mesh regularisers.
* PNG (8-bit grey, RGB, RGBA; non-interlaced) read and write, with zlib.
"""
from __future__ import annotations

import os
import struct
import zlib
from dataclasses import dataclass, field

import numpy as np


@dataclass
class Mesh:
    vertices: np.ndarray                 # [N, 3] float32
    colors: np.ndarray                   # [N, 3] float32 (ones if the file has none)
    faces: np.ndarray                    # [F, 3] int32, 0-based
    uvs: np.ndarray                      # [F * 6] float32 per-face-corner (u, v)
    texture: np.ndarray | None = None    # [Ht, Wt, 3] float32 in [0, 1]
    texture_path: str | None = None
    labels: np.ndarray | None = None     # [N] int32 segmentation labels
    weights: np.ndarray | None = None    # [N] float32 vertex weights
    extra: dict = field(default_factory=dict)

    @property
    def num_vertices(self):
        return int(self.vertices.shape[0])

    @property
    def num_faces(self):
        return int(self.faces.shape[0])

    def neighbours(self):
        """Per-vertex neighbour lists in first-seen order (face order, corner
        order), each neighbour once: (start [N+1], index [sum of degrees])."""
        N = self.num_vertices
        seen = [dict() for _ in range(N)]
        for a, b, c in self.faces.tolist():
            for v, others in ((a, (b, c)), (b, (a, c)), (c, (a, b))):
                for o in others:
                    seen[v].setdefault(o, None)
        start = np.zeros(N + 1, np.int64)
        for v in range(N):
            start[v + 1] = start[v] + len(seen[v])
        index = np.fromiter((o for v in range(N) for o in seen[v]), dtype=np.int64, count=int(start[-1]))
        return start, index


def read_obj(path, triangulate=False, load_texture=True, load_segmentation=True):
    verts, cols, vts, faces, ftex = [], [], [], [], []
    mtl = None
    with open(path) as fh:
        for line in fh:
            t = line.split()
            if not t:
                continue
            if t[0] == "v":
                verts.append([float(x) for x in t[1:4]])
                cols.append([float(x) for x in t[4:7]] if len(t) >= 7 else [1.0, 1.0, 1.0])
            elif t[0] == "vt":
                vts.append([float(t[1]), float(t[2])])
            elif t[0] == "f":
                corners = [c.split("/") for c in t[1:]]
                vi = [int(c[0]) - 1 for c in corners]
                ti = [int(c[1]) - 1 if len(c) > 1 and c[1] else -1 for c in corners]
                tris = [(0, k, k + 1) for k in range(1, len(vi) - 1)] if triangulate else [(0, 1, 2)]
                for i, j, k in tris:
                    faces.append([vi[i], vi[j], vi[k]])
                    ftex.append([ti[i], ti[j], ti[k]])
            elif t[0] == "mtllib":
                mtl = " ".join(t[1:])
    vertices = np.asarray(verts, np.float32).reshape(-1, 3)
    faces_a = np.asarray(faces, np.int32).reshape(-1, 3)
    ft = np.asarray(ftex, np.int64).reshape(-1, 3)
    vt = np.asarray(vts, np.float32).reshape(-1, 2)
    uv = np.zeros((faces_a.shape[0], 3, 2), np.float32)
    ok = ft >= 0
    if vt.shape[0]:
        uv[ok] = vt[ft[ok]]
    mesh = Mesh(vertices, np.asarray(cols, np.float32).reshape(-1, 3), faces_a, uv.reshape(-1))
    folder = os.path.dirname(os.path.abspath(path))
    if mtl and load_texture:
        mtl_path = os.path.join(folder, mtl[2:] if mtl.startswith("./") else mtl)
        if os.path.exists(mtl_path):
            tex = read_mtl_texture(mtl_path)
            if tex is not None:
                mesh.texture_path = tex
                mesh.texture = read_png(tex)[..., :3]
    seg = os.path.join(folder, "segmentation.txt")
    if load_segmentation and os.path.exists(seg):
        mesh.labels, mesh.weights = read_segmentation(seg)
    return mesh


def read_mtl_texture(path):
    """Path of the `map_Kd` image of an MTL file (the last one), or None."""
    tex = None
    with open(path) as fh:
        for line in fh:
            t = line.split()
            if len(t) > 1 and t[0] == "map_Kd":
                tex = os.path.join(os.path.dirname(os.path.abspath(path)), " ".join(t[1:]))
    return tex


# label -> regulariser weight (OBJReader.py:250-281: skin, accessories and face
# regions are weighted up so that they deform less)
_LABEL_WEIGHTS = {2: 400.0, 13: 400.0, 9: 2.0}
for _l in (14, 15, 16, 17, 18, 19, 1, 3, 4):
    _LABEL_WEIGHTS[_l] = 5.0


def read_segmentation(path):
    labels = []
    with open(path) as fh:
        for line in fh:
            t = line.split()
            if t:
                labels.append(int(t[0]))
    labels = np.asarray(labels, np.int32)
    weights = np.asarray([_LABEL_WEIGHTS.get(int(l), 1.0) for l in labels], np.float32)
    return labels, weights


def read_calibration(path, render_u, render_v):
    """(extrinsics [C, 12], intrinsics [C, 9]) float32 of a Skeletool
    calibration file, intrinsics rescaled to render_u x render_v."""
    ex, K, size = [], [], []
    with open(path) as fh:
        for line in fh:
            t = line.split()
            if not t:
                continue
            if t[0] == "intrinsic":
                m = [float(x) for x in t[1:17]]
                K.append([m[0], m[1], m[2], m[4], m[5], m[6], m[8], m[9], m[10]])
            elif t[0] == "extrinsic":
                ex.append([float(x) for x in t[1:13]])
            elif t[0] == "size":
                size.append((float(t[1]), float(t[2])))
    C = len(ex)
    if len(K) != C or len(size) != C:
        raise ValueError(f"{path}: {C} extrinsic, {len(K)} intrinsic and {len(size)} size entries")
    K = np.asarray(K, np.float64).reshape(C, 3, 3)
    for c, (su, sv) in enumerate(size):
        K[c, 0, 0] = K[c, 0, 0] / su * render_u
        K[c, 1, 1] = K[c, 1, 1] / sv * render_v
        K[c, 0, 2] = K[c, 0, 2] / su * render_u
        K[c, 1, 2] = K[c, 1, 2] / sv * render_v
    return np.asarray(ex, np.float32).reshape(C, 12), K.reshape(C, 9).astype(np.float32)


# ----------------------------------------------------------------------------- PNG


def _paeth(a, b, c):
    p = a.astype(np.int32) + b - c
    pa, pb, pc = np.abs(p - a), np.abs(p - b), np.abs(p - c)
    return np.where((pa <= pb) & (pa <= pc), a, np.where(pb <= pc, b, c))


def read_png(path):
    """[H, W, C] float32 in [0, 1] of an 8-bit non-interlaced PNG (C = 1, 3, 4)."""
    data = open(path, "rb").read()
    if data[:8] != b"\x89PNG\r\n\x1a\n":
        raise ValueError(f"{path}: not a PNG file")
    pos, idat, hdr = 8, [], None
    while pos < len(data):
        n, kind = struct.unpack(">I4s", data[pos:pos + 8])
        chunk = data[pos + 8:pos + 8 + n]
        pos += 12 + n
        if kind == b"IHDR":
            hdr = struct.unpack(">IIBBBBB", chunk)
        elif kind == b"IDAT":
            idat.append(chunk)
        elif kind == b"IEND":
            break
    W, H, depth, ctype, _, _, interlace = hdr
    ch = {0: 1, 2: 3, 4: 2, 6: 4}.get(ctype)
    if depth != 8 or ch is None or interlace:
        raise ValueError(f"{path}: only 8-bit grey/RGB/RGBA non-interlaced PNG is supported")
    raw = np.frombuffer(zlib.decompress(b"".join(idat)), np.uint8).reshape(H, 1 + W * ch)
    out = np.zeros((H, W * ch), np.uint8)
    prev = np.zeros(W * ch, np.uint8)
    for y in range(H):
        f, row = raw[y, 0], raw[y, 1:].astype(np.int32)
        if f == 0:
            cur = row
        elif f == 2:
            cur = row + prev
        elif f == 1:  # Sub: running sum along each channel
            cur = np.cumsum(row.reshape(W, ch), axis=0).reshape(-1)
        else:
            cur = np.zeros(W * ch, np.int32)
            for x in range(W * ch):  # left-dependent filters run per byte
                a = cur[x - ch] if x >= ch else 0
                b = int(prev[x])
                c = int(prev[x - ch]) if x >= ch else 0
                if f == 1:
                    cur[x] = (row[x] + a) & 255
                elif f == 3:
                    cur[x] = (row[x] + ((a + b) >> 1)) & 255
                else:
                    cur[x] = (row[x] + int(_paeth(np.int32(a), np.int32(b), np.int32(c)))) & 255
        out[y] = (cur & 255).astype(np.uint8)
        prev = out[y]
    img = out.reshape(H, W, ch).astype(np.float32) / 255.0
    if ch == 1:
        img = np.repeat(img, 3, axis=2)
    elif ch == 2:
        img = np.concatenate([np.repeat(img[..., :1], 3, axis=2), img[..., 1:]], axis=2)
    return img


def write_png(path, img):
    """Writes [H, W, 3 or 4] values in [0, 1] (clipped) as an 8-bit PNG."""
    a = np.clip(np.asarray(img, np.float64) * 255.0 + 0.5, 0, 255).astype(np.uint8)
    if a.ndim == 2:
        a = np.repeat(a[..., None], 3, axis=2)
    H, W, C = a.shape
    ctype = {3: 2, 4: 6}[C]
    raw = b"".join(b"\x00" + a[y].tobytes() for y in range(H))

    def chunk(kind, body):
        return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body) & 0xFFFFFFFF)

    with open(path, "wb") as fh:
        fh.write(b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", W, H, 8, ctype, 0, 0, 0)) +
                 chunk(b"IDAT", zlib.compress(raw, 6)) + chunk(b"IEND", b""))
