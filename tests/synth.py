"""Synthetic surface grids for the tests (seeded numpy)."""

from __future__ import annotations

import numpy as np


def box_surfaces(n_boxes: int, resolution: int, seed: int) -> np.ndarray:
    """Voxels on the faces of `n_boxes` random axis-aligned boxes in [0,1)^3 (side lengths
    U[0.1, 0.5] per axis, min corner U[0, 1 - side]) voxelised at `resolution`^3, unique."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n_boxes):
        side = rng.uniform(0.1, 0.5, 3)
        lo = rng.uniform(0.0, 1.0 - side)
        a = np.floor(lo * resolution).astype(np.int64)
        b = np.floor((lo + side) * resolution).astype(np.int64)
        for axis in range(3):
            u, v = [ax for ax in range(3) if ax != axis]
            gu, gv = np.meshgrid(np.arange(a[u], b[u] + 1), np.arange(a[v], b[v] + 1), indexing="ij")
            for face in (a[axis], b[axis]):
                pts = np.empty((gu.size, 3), dtype=np.int64)
                pts[:, axis] = face
                pts[:, u] = gu.ravel()
                pts[:, v] = gv.ravel()
                out.append(pts)
    ijk = np.unique(np.concatenate(out, 0), axis=0)
    return ijk.astype(np.int32)
