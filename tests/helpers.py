"""Shared helpers of the test-suite: synthetic grids and dense reference convolutions.

Dense convention of the reference tests (tests/unit/test_conv.py:94,109): features are
written to [C, Z, Y, X] (= write_to_dense_xyzc(...).squeeze(0).permute(3,2,1,0)), so conv3d's
D axis is ijk axis 2 and weight dim K0 acts on ijk axis 2.
"""

from __future__ import annotations

import numpy as np
import torch


def dense_ijk(dims, mn=(0, 0, 0)) -> np.ndarray:
    ax = [np.arange(d) + m for d, m in zip(dims, mn)]
    g = np.stack(np.meshgrid(*ax, indexing="ij"), -1).reshape(-1, 3)
    return g.astype(np.int32)


def random_sparse_ijk(n: int, extent: int, seed: int, lo: int = 0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    idx = rng.choice(extent**3, size=min(n, extent**3), replace=False)
    ijk = np.stack([idx // (extent * extent), (idx // extent) % extent, idx % extent], 1) + lo
    return ijk.astype(np.int32)


def to_dense_czyx(ijk: np.ndarray, feats: np.ndarray, mn, size) -> torch.Tensor:
    """[C, Z, Y, X] float64 tensor with feats written at ijk - mn."""
    C = feats.shape[1]
    out = np.zeros((size[0], size[1], size[2], C), dtype=np.float64)
    rel = ijk.astype(np.int64) - np.asarray(mn, dtype=np.int64)
    ok = np.all((rel >= 0) & (rel < np.asarray(size)), 1)
    out[rel[ok, 0], rel[ok, 1], rel[ok, 2]] = feats[ok]
    return torch.from_numpy(out).permute(3, 2, 1, 0).contiguous()


def dense_at(dense_czyx: torch.Tensor, ijk: np.ndarray, mn=(0, 0, 0)):
    """Rows of dense [C, Z, Y, X] at voxel coordinates ijk (returns values, in-range mask)."""
    C, Z, Y, X = dense_czyx.shape
    rel = ijk.astype(np.int64) - np.asarray(mn, dtype=np.int64)
    size = np.array([X, Y, Z])
    ok = np.all((rel >= 0) & (rel < size), 1)
    vals = np.zeros((ijk.shape[0], C), dtype=np.float64)
    d = dense_czyx.detach().numpy()
    vals[ok] = d[:, rel[ok, 2], rel[ok, 1], rel[ok, 0]].T
    return vals, ok


def kernel_start(k: int) -> int:
    """floor(-k/2 + 1): first kernel offset of the reference's map (ConvolutionKernelMap.cu:66-68)."""
    return int(np.floor(-k / 2.0 + 1.0))


def dense_conv_reference(ijk_in, feats, weight, stride, box_mn, box_size):
    """F.conv3d over the dense box with the padding that makes output index == target ijk.

    Output position o of conv3d(padding p, stride s) reads input o*s - p + j, j in [0,k);
    the sparse map reads t*s + floor(-k/2+1) + j, so p = -floor(-k/2+1) per axis (D<->k0)."""
    w = torch.as_tensor(weight, dtype=torch.float64)
    k0, k1, k2 = w.shape[2:]
    s = stride
    pad = [-kernel_start(k0), -kernel_start(k1), -kernel_start(k2)]
    x = to_dense_czyx(ijk_in, feats, box_mn, box_size)
    # the box origin must sit on the stride lattice for output index == target ijk
    return torch.nn.functional.conv3d(x[None], w, padding=pad, stride=(s[0], s[1], s[2]))[0]


# ------------------------------------------------------------------ golden fixtures ------
import glob as _glob
import os as _os

GOLDEN_DIR = _os.path.join(_os.path.dirname(_os.path.abspath(__file__)), "golden")


def golden_cases(prefix: str = "sparse_"):
    return sorted(_os.path.basename(p)[:-4] for p in _glob.glob(_os.path.join(GOLDEN_DIR, prefix + "*.npz")))


def load_golden(name: str) -> dict:
    with np.load(_os.path.join(GOLDEN_DIR, name + ".npz")) as z:
        return {k: z[k] for k in z.files}


def rows_by_coord(ijk: np.ndarray) -> dict:
    return {tuple(r): i for i, r in enumerate(ijk.tolist())}


def kmap_to_coords(kmap: np.ndarray, src_ijk: np.ndarray) -> np.ndarray:
    """[T, K, 3] source coordinates of a kernel map (INT32_MIN where absent)."""
    out = np.full(kmap.shape + (3,), np.iinfo(np.int32).min, dtype=np.int32)
    v = kmap >= 0
    out[v] = src_ijk[kmap[v]]
    return out
