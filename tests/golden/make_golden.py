"""Generates the golden fixtures of tests/golden/*.npz (run: python tests/golden/make_golden.py).

The expected values come from torch's dense float64 convolutions (F.conv3d /
F.conv_transpose3d), an implementation independent of this repository, evaluated on a
dense box that holds the sparse features.  Expected neighbour relations are stated in
coordinate form (target coordinate, offset) -> source coordinate by a pure-Python loop over
the reference's kernel-map definition (ConvolutionKernelMap.cu:60-102), so the fixtures do
not depend on any voxel index order.  Target voxel sets follow BuildGridForConv.cu:66-124.
"""

from __future__ import annotations

import math
import os

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))


def kstart(k):
    return int(math.floor(-k / 2.0 + 1.0))


def target_set(ijk, ks, st):
    if tuple(st) == (1, 1, 1) or tuple(st) == tuple(ks):
        return sorted({(x // st[0], y // st[1], z // st[2]) for x, y, z in ijk.tolist()})
    out = set()
    rng = [range(0, k) if k % 2 == 0 else range(-(k - 1) // 2, (k - 1) // 2 + 1) for k in ks]
    for x, y, z in ijk.tolist():
        for di in rng[0]:
            for dj in rng[1]:
                for dk in rng[2]:
                    dx, dy, dz = x + dk, y + dj, z + di
                    if math.fmod(dx, st[2]) or math.fmod(dy, st[1]) or math.fmod(dz, st[0]):
                        continue
                    out.add((int(dx / st[2]), int(dy / st[1]), int(dz / st[0])))
    return sorted(out)


def neighbours(src_set, tgt, ks, st):
    """[T, K, 3] source coordinate per (target, offset), with 'absent' rows = INT32_MIN."""
    s0 = [kstart(k) for k in ks]
    K = ks[0] * ks[1] * ks[2]
    out = np.full((len(tgt), K, 3), np.iinfo(np.int32).min, dtype=np.int32)
    for i, (tx, ty, tz) in enumerate(tgt):
        k = 0
        for kz in range(s0[2], s0[2] + ks[2]):
            for ky in range(s0[1], s0[1] + ks[1]):
                for kx in range(s0[0], s0[0] + ks[0]):
                    c = (tx * st[2] + kz, ty * st[1] + ky, tz * st[0] + kx)
                    if c in src_set:
                        out[i, k] = c
                    k += 1
    return out


def dense_forward(ijk, x, w, ks, st, tgt, shift=12):
    sax = [st[2], st[1], st[0]]
    kax = [ks[2], ks[1], ks[0]]
    t = np.array(tgt, dtype=np.int64).reshape(-1, 3)
    size = [int(max(t[:, a].max() + shift // sax[a], 0)) * sax[a] + kax[a] + 2 for a in range(3)]
    size = [max(sz, int(ijk[:, a].max()) + shift + 2) for a, sz in enumerate(size)]
    d = torch.zeros(size + [x.shape[1]], dtype=torch.float64)
    d[tuple(torch.from_numpy(ijk[:, a].astype(np.int64) + shift) for a in range(3))] = torch.from_numpy(x)
    pad = [-kstart(k) for k in ks]
    y = torch.nn.functional.conv3d(d.permute(3, 2, 1, 0)[None], torch.from_numpy(w), padding=pad, stride=tuple(st))[0]
    tp = [torch.from_numpy(t[:, a] + shift // sax[a]) for a in range(3)]
    return y[:, tp[2], tp[1], tp[0]].T.numpy()


def case(name, n, extent, cin, cout, ks, st, seed, lo=0):
    rng = np.random.default_rng(seed)
    idx = rng.choice(extent**3, size=n, replace=False)
    ijk = (np.stack([idx // extent**2, (idx // extent) % extent, idx % extent], 1) + lo).astype(np.int32)
    x = rng.standard_normal((n, cin))
    w = rng.standard_normal((cout, cin) + tuple(ks)) / math.sqrt(cin * np.prod(ks))
    tgt = target_set(ijk, ks, st)
    expected = dense_forward(ijk, x, w, ks, st, tgt)
    nb = neighbours({tuple(r) for r in ijk.tolist()}, tgt, ks, st)
    np.savez_compressed(
        os.path.join(HERE, name + ".npz"),
        ijk=ijk,
        features=x,
        weights=w,
        kernel_size=np.array(ks),
        stride=np.array(st),
        target_ijk=np.array(tgt, dtype=np.int32).reshape(-1, 3),
        expected=expected,
        neighbours=nb,
    )
    print(name, ijk.shape[0], "->", len(tgt))


def transposed_case(name, extent, cin, cout, k, seed):
    """Stride-1 transposed conv on a dense box (test_conv.py:579-675), features on the target."""
    rng = np.random.default_rng(seed)
    g = np.stack(np.meshgrid(*[np.arange(extent)] * 3, indexing="ij"), -1).reshape(-1, 3).astype(np.int32)
    x = rng.standard_normal((g.shape[0], cin))
    w = rng.standard_normal((cin, cout, k, k, k)) / math.sqrt(cin * k**3)
    d = torch.zeros((extent, extent, extent, cin), dtype=torch.float64)
    d[tuple(torch.from_numpy(g[:, a].astype(np.int64)) for a in range(3))] = torch.from_numpy(x)
    y = torch.nn.functional.conv_transpose3d(d.permute(3, 2, 1, 0)[None], torch.from_numpy(w), stride=1, padding=-kstart(k))[0]
    y = y[:, :extent, :extent, :extent]
    gi = [torch.from_numpy(g[:, a].astype(np.int64)) for a in range(3)]
    expected = y[:, gi[2], gi[1], gi[0]].T.numpy()
    np.savez_compressed(
        os.path.join(HERE, name + ".npz"), ijk=g, features=x, weights=w, kernel_size=np.array([k] * 3),
        stride=np.array([1, 1, 1]), target_ijk=g, expected=expected,
    )
    print(name, g.shape[0])


def transposed_strided_case(name, n, extent, cin, cout, ks, st, seed, lo=0, shift=12):
    """Strided transposed conv (the decoder side of a UNet: coarse features onto the fine grid
    whose forward map defines the pairs).  Features live on the coarse target set of
    (ijk, ks, st); the expected output on the fine voxels is torch's dense conv_transpose3d, the
    adjoint of the dense conv3d whose restriction the sparse forward is."""
    rng = np.random.default_rng(seed)
    idx = rng.choice(extent**3, size=n, replace=False)
    ijk = (np.stack([idx // extent**2, (idx // extent) % extent, idx % extent], 1) + lo).astype(np.int32)
    tgt = np.array(target_set(ijk, ks, st), dtype=np.int64).reshape(-1, 3)
    x = rng.standard_normal((tgt.shape[0], cin))
    w = rng.standard_normal((cin, cout) + tuple(ks)) / math.sqrt(cin * np.prod(ks))
    sax = [st[2], st[1], st[0]]
    kax = [ks[2], ks[1], ks[0]]
    osz = [int(tgt[:, a].max()) + shift // sax[a] + 2 + kax[a] for a in range(3)]
    d = torch.zeros(osz + [cin], dtype=torch.float64)
    d[tuple(torch.from_numpy(tgt[:, a] + shift // sax[a]) for a in range(3))] = torch.from_numpy(x)
    pad = [-kstart(k) for k in ks]
    y = torch.nn.functional.conv_transpose3d(d.permute(3, 2, 1, 0)[None], torch.from_numpy(w), stride=tuple(st),
                                             padding=pad)[0]
    fi = [torch.from_numpy(ijk[:, a].astype(np.int64) + shift) for a in range(3)]
    assert all(int(fi[a].max()) < y.shape[3 - a] for a in range(3))
    expected = y[:, fi[2], fi[1], fi[0]].T.numpy()
    np.savez_compressed(
        os.path.join(HERE, name + ".npz"), ijk=ijk, features=x, weights=w, kernel_size=np.array(ks),
        stride=np.array(st), target_ijk=tgt.astype(np.int32), expected=expected,
    )
    print(name, ijk.shape[0], "<-", tgt.shape[0])


if __name__ == "__main__":
    case("sparse_k3_s1_c16", 2000, 24, 16, 16, (3, 3, 3), (1, 1, 1), seed=0)
    case("sparse_k3_s2_c8", 1500, 20, 8, 12, (3, 3, 3), (2, 2, 2), seed=1)
    case("sparse_k2_s2_c8", 1500, 20, 8, 8, (2, 2, 2), (2, 2, 2), seed=2)
    case("sparse_aniso_c4", 800, 16, 4, 8, (5, 3, 1), (1, 3, 2), seed=3, lo=-7)
    case("sparse_k5_s2_neg", 600, 14, 4, 4, (5, 5, 5), (2, 2, 2), seed=4, lo=-6)
    transposed_case("dense_transposed_k3", 8, 4, 8, 3, seed=5)
    transposed_case("dense_transposed_k4", 8, 4, 8, 4, seed=6)
    case("sparse_k2_s1_c8", 1500, 18, 8, 8, (2, 2, 2), (1, 1, 1), seed=7)
    case("sparse_k4_s2_c4", 900, 16, 4, 6, (4, 4, 4), (2, 2, 2), seed=8, lo=-5)
    case("sparse_k3_s3_c4", 1200, 18, 4, 4, (3, 3, 3), (3, 3, 3), seed=9, lo=-4)
    transposed_strided_case("strided_transposed_k2_s2", 1200, 16, 8, 4, (2, 2, 2), (2, 2, 2), seed=10, lo=-3)
    transposed_strided_case("strided_transposed_k3_s2", 900, 14, 4, 6, (3, 3, 3), (2, 2, 2), seed=11)
    transposed_strided_case("strided_transposed_aniso", 700, 14, 4, 4, (3, 2, 1), (1, 2, 3), seed=12, lo=-2)
