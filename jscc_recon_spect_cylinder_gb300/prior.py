"""Neighbour tables of the relative-difference prior on the reference's polar image grid.

The grid is z-major, and within a z layer ring after ring of possibly different lengths
(the layout compton_sparse_ops.py:59-92 infers from ``coor_polar_full``). Edges of a voxel:

* its two angular neighbours in the same ring (periodic);
* in each adjacent ring, the voxel nearest in angle (both directions are added, so rings of
  different lengths still give a symmetric table); with ``diagonal`` also that voxel's two
  angular neighbours (the 8-neighbourhood on a uniform grid);
* the voxel at the same (ring, angle) slot in the adjacent z layers.

The default (no diagonals) is the polar 4-neighbourhood: ring +-1 angular step plus the
nearest angle in the adjacent rings. Weights: ``"index"`` gives face edges 1 and diagonal
edges 1/sqrt(2) (index space, independent of the polar voxel sizes);
``"distance"`` gives 1 / |c_j - c_k| in 1/mm. The table is neighbour-major
``[K, V]`` (jscc_rdp_prior's layout), -1 / 0 padded.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import torch

from . import compton_sparse_ops as cso


@dataclass
class NeighbourTable:
    nbr: torch.Tensor     # [K, V] int32, -1 = padding
    weight: torch.Tensor  # [K, V] float32

    @property
    def n_vox(self) -> int:
        return self.nbr.size(1)

    @property
    def n_nbr(self) -> int:
        return self.nbr.size(0)

    def to(self, device) -> "NeighbourTable":
        return NeighbourTable(self.nbr.to(device).contiguous(), self.weight.to(device).contiguous())


def polar_neighbour_edges(coor_full, diagonal=False):
    """Undirected edges ``(j, k, diagonal_flag)`` of the polar grid, j < k, no duplicates."""
    c = np.asarray(torch.as_tensor(coor_full, dtype=torch.float32).cpu().numpy(), dtype=np.float64)
    layout = cso._infer_polar_layout(torch.as_tensor(coor_full, dtype=torch.float32).cpu())
    n_z, n_layer = int(layout["fine_z_num"]), int(layout["fine_layer_num"])
    lengths = [int(v) for v in layout["ring_lengths"]]
    starts = np.concatenate(([0], np.cumsum(lengths)[:-1])).astype(np.int64)
    ang = np.arctan2(c[:n_layer, 1], c[:n_layer, 0])
    edges = {}

    def add(a, b, diag):
        a, b = np.asarray(a, np.int64).ravel(), np.asarray(b, np.int64).ravel()
        for u, v in zip(a.tolist(), b.tolist()):
            if u == v:
                continue
            key = (u, v) if u < v else (v, u)
            # a pair reached both as a face and as a diagonal edge keeps the face weight
            edges[key] = edges.get(key, True) and diag

    def ring_idx(r, t):
        return starts[r] + np.mod(t, lengths[r])

    def nearest(r_from, r_to):
        """For each voxel of ring r_from, the slot of ring r_to nearest in angle."""
        a_from = ang[starts[r_from]:starts[r_from] + lengths[r_from]]
        a_to = ang[starts[r_to]:starts[r_to] + lengths[r_to]]
        diff = np.angle(np.exp(1j * (a_from[:, None] - a_to[None, :])))
        return np.argmin(np.abs(diff), axis=1)

    for r, L in enumerate(lengths):
        t = np.arange(L)
        if L >= 2:
            add(ring_idx(r, t), ring_idx(r, t + 1), False)
        for r2 in (r - 1, r + 1):
            if not 0 <= r2 < len(lengths):
                continue
            t2 = nearest(r, r2)
            add(ring_idx(r, t), ring_idx(r2, t2), False)
            if diagonal and lengths[r2] >= 2:
                add(ring_idx(r, t), ring_idx(r2, t2 + 1), True)
                add(ring_idx(r, t), ring_idx(r2, t2 - 1), True)
    in_layer = list(edges.items())
    out = []
    for z in range(n_z):
        off = z * n_layer
        out.extend(((u + off, v + off), d) for (u, v), d in in_layer)
        if z + 1 < n_z:
            j = np.arange(n_layer) + off
            out.extend(((int(u), int(u + n_layer)), False) for u in j)
    return out


def polar_neighbours(coor_full, diagonal=False, weights="index", device="cpu") -> NeighbourTable:
    """The symmetric neighbour table of ``coor_full`` ([V, 3]) for jscc_rdp_prior."""
    if weights not in ("index", "distance"):
        raise ValueError(f"weights must be 'index' or 'distance', got {weights!r}")
    coor = torch.as_tensor(coor_full, dtype=torch.float32).cpu()
    V = coor.size(0)
    edges = polar_neighbour_edges(coor, diagonal=diagonal)
    if not edges:
        return NeighbourTable(torch.full((0, V), -1, dtype=torch.int32, device=device),
                              torch.zeros((0, V), dtype=torch.float32, device=device))
    uv = np.array([e[0] for e in edges], dtype=np.int64)
    diag = np.array([e[1] for e in edges], dtype=bool)
    if weights == "index":
        w = np.where(diag, 1.0 / np.sqrt(2.0), 1.0)
    else:
        c = coor.numpy().astype(np.float64)
        w = 1.0 / np.maximum(np.linalg.norm(c[uv[:, 0]] - c[uv[:, 1]], axis=1), 1e-9)
    src = np.concatenate((uv[:, 0], uv[:, 1]))
    dst = np.concatenate((uv[:, 1], uv[:, 0]))
    ww = np.concatenate((w, w))
    order = np.lexsort((dst, src))
    src, dst, ww = src[order], dst[order], ww[order]
    deg = np.bincount(src, minlength=V)
    K = int(deg.max())
    slot = np.arange(src.size) - np.repeat(np.cumsum(deg) - deg, deg)
    nbr = np.full((K, V), -1, dtype=np.int32)
    wt = np.zeros((K, V), dtype=np.float32)
    nbr[slot, src] = dst
    wt[slot, src] = ww
    return NeighbourTable(torch.from_numpy(nbr).to(device), torch.from_numpy(wt).to(device))
