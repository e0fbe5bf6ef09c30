"""Mesh regularisers of the reference's fitting scripts as sparse torch losses.

The reference builds dense N x N adjacency, Laplacian and weight matrices
(python/utils/OBJReader.py:110-212) and evaluates

* the Laplacian loss (python/utils/LaplacianLoss.py:9-33):
    sum_b sum_i rowWeight_i * |(L (V_b - V_rest) / 1000)_i|^2 / (B * E)
  with L = D - A (graph Laplacian of the mesh edges) and rowWeight_i the
  mean over i's neighbours j of (w_i + w_j) / 2 for vertex weights w;
* the isometry loss (python/utils/IsometryLoss.py:11-70):
    sum_b sum_{(i, j) adjacent, both orders} (|v_i - v_j|_rest - |v_i - v_j|_b)^2 / (B * E)
where E counts the directed neighbour pairs (each undirected edge twice).
Here both use the edge list (O(E) memory and work instead of O(N^2)), so
they run on meshes of any size, on the GPU or the CPU, and differentiate
with autograd.
"""
from __future__ import annotations

import numpy as np
import torch


class MeshEdges:
    """Directed neighbour pairs (i, j) of a triangle mesh (each undirected
    edge in both orders), degrees, and optional vertex weights."""

    def __init__(self, faces, num_vertices, weights=None, device=None):
        f = np.asarray(faces, np.int64).reshape(-1, 3)
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 0]], f[:, [0, 2]], f[:, [2, 0]], f[:, [1, 2]], f[:, [2, 1]]])
        e = e[e[:, 0] != e[:, 1]]
        e = np.unique(e, axis=0)
        self.N = int(num_vertices)
        self.E = int(e.shape[0])
        deg = np.bincount(e[:, 0], minlength=self.N).astype(np.float32)
        dev = torch.device(device) if device is not None else torch.device("cpu")
        self.i = torch.from_numpy(e[:, 0]).to(dev)
        self.j = torch.from_numpy(e[:, 1]).to(dev)
        self.deg = torch.from_numpy(deg).to(dev)
        w = np.ones(self.N, np.float32) if weights is None else np.asarray(weights, np.float32)
        # row weight: mean over the neighbours j of (w_i + w_j) / 2
        rw = np.zeros(self.N, np.float64)
        np.add.at(rw, e[:, 0], (w[e[:, 0]] + w[e[:, 1]]) / 2.0)
        rw = np.where(deg > 0, rw / np.maximum(deg, 1.0), 0.0)
        self.row_weight = torch.from_numpy(rw.astype(np.float32)).to(dev)

    def laplacian(self, x):
        """(D - A) x for x [..., N, 3]."""
        out = x * self.deg[:, None]
        return out.index_add(-2, self.i, -x.index_select(-2, self.j))


def laplacian_loss(edges: MeshEdges, verts, rest):
    """verts [B, N, 3], rest [N, 3] or [B, N, 3] (mm)."""
    B = verts.shape[0]
    d = (verts - rest) / 1000.0
    lap = edges.laplacian(d)
    inner = (lap * lap).sum(-1)                               # [B, N]
    return (inner * edges.row_weight).sum() / (B * edges.E)


def isometry_loss(edges: MeshEdges, verts, rest):
    """verts [B, N, 3], rest [N, 3] (mm)."""
    B = verts.shape[0]
    def lengths(v):
        return (v.index_select(-2, edges.i) - v.index_select(-2, edges.j)).norm(dim=-1)
    diff = lengths(rest) - lengths(verts)
    return (diff * diff).sum() / (B * edges.E)
