"""Pins the CPU oracle (no GPU).

The reference holds no golden vectors for raw map integers; its conv tests pin semantics by
equivalence with torch's dense convolutions (tests/unit/test_conv.py:73-131,361-675).  Those
equivalences are re-hosted here against the oracle: map + gather-scatter must equal
F.conv3d / F.conv_transpose3d on dense and random-sparse boxes, for the kernel sizes,
strides and anisotropic shapes the reference tests use, forward and backward.  The voxel
index order is checked against an independent pure-Python statement of NanoVDB's order.
"""

import itertools

import numpy as np
import pytest
import torch

from oracle import oracle as orc
from tests.helpers import dense_at, dense_conv_reference, dense_ijk, kernel_start, random_sparse_ijk, to_dense_czyx


def nanovdb_order_py(c):
    x, y, z = (int(v) for v in c)
    root = tuple(((v & 0xFFFFFFFF) >> 12) for v in (x, y, z))
    up = (((x & 4095) >> 7), ((y & 4095) >> 7), ((z & 4095) >> 7))
    lo = (((x & 127) >> 3), ((y & 127) >> 3), ((z & 127) >> 3))
    lf = ((x & 7), (y & 7), (z & 7))
    return root + up + lo + lf


@pytest.mark.parametrize("lo,extent,n", [(0, 40, 3000), (-20, 40, 3000), (4090, 12, 900), (-4100, 20, 2000)])
def test_grid_order_matches_definition(lo, extent, n):
    ijk = random_sparse_ijk(n, extent, seed=extent + n, lo=lo)
    dup = np.concatenate([ijk, ijk[::7]], 0)  # duplicates collapse
    out, off = orc.grid_from_ijk(dup, np.array([0, dup.shape[0]]))
    expect = sorted({tuple(r) for r in ijk.tolist()}, key=nanovdb_order_py)
    assert off.tolist() == [0, len(expect)]
    assert [tuple(r) for r in out.tolist()] == expect


def test_grid_batches_keep_offsets():
    a = random_sparse_ijk(500, 16, 1)
    b = random_sparse_ijk(10, 16, 2) + 100
    empty = np.zeros((0, 3), np.int32)
    ijk = np.concatenate([a, empty, b, a[:5]], 0)
    off = np.array([0, 500, 500, 510, 515])
    out, ooff = orc.grid_from_ijk(ijk, off)
    assert ooff.tolist() == [0, 500, 500, 510, 515]
    for bi, part in enumerate([a, empty, b, a[:5]]):
        s, e = ooff[bi], ooff[bi + 1]
        assert sorted(map(tuple, out[s:e].tolist())) == sorted(map(tuple, part.tolist()))


def kmap_by_definition(src, tgt, ks, st):
    """Pure-Python restatement of ConvolutionKernelMap.cu:60-102 on one grid."""
    pos = {tuple(r): i for i, r in enumerate(src.tolist())}
    s0 = [kernel_start(k) for k in ks]
    out = []
    for t in tgt.tolist():
        sx, sy, sz = t[0] * st[2], t[1] * st[1], t[2] * st[0]
        row = []
        for kz in range(s0[2], s0[2] + ks[2]):
            for ky in range(s0[1], s0[1] + ks[1]):
                for kx in range(s0[0], s0[0] + ks[0]):
                    row.append(pos.get((sx + kz, sy + ky, sz + kx), -1))
        out.append(row)
    return np.array(out, dtype=np.int32).reshape(len(out), -1)


@pytest.mark.parametrize("ks,st", [((3, 3, 3), (1, 1, 1)), ((2, 2, 2), (2, 2, 2)), ((4, 1, 4), (1, 2, 1)), ((5, 3, 1), (1, 3, 2))])
def test_kernel_map_matches_definition(ks, st):
    ijk = random_sparse_ijk(700, 14, seed=sum(ks) + sum(st), lo=-3)
    src, soff = orc.grid_from_ijk(ijk, np.array([0, ijk.shape[0]]))
    tgt, toff = orc.conv_grid(src, soff, ks, st) if st != (1, 1, 1) else (src, soff)
    got = orc.kernel_map(src, soff, tgt, toff, ks, st)
    assert np.array_equal(got, kmap_by_definition(src, tgt, ks, st))


def conv_grid_by_definition(ijk, ks, st):
    coarse = st == (1, 1, 1) or tuple(st) == tuple(ks)
    out = set()
    for x, y, z in ijk.tolist():
        if coarse:
            out.add((x // st[0], y // st[1], z // st[2]))
            continue
        rng = [range(0, k) if k % 2 == 0 else range(-(k - 1) // 2, (k - 1) // 2 + 1) for k in ks]
        for di in rng[0]:
            for dj in rng[1]:
                for dk in rng[2]:
                    dx, dy, dz = x + dk, y + dj, z + di
                    if int(np.fmod(dx, st[2])) or int(np.fmod(dy, st[1])) or int(np.fmod(dz, st[0])):
                        continue
                    out.add((int(dx / st[2]), int(dy / st[1]), int(dz / st[0])))
    return out


@pytest.mark.parametrize("ks,st", [((3, 3, 3), (2, 2, 2)), ((2, 2, 2), (2, 2, 2)), ((5, 5, 5), (2, 2, 2)), ((3, 1, 2), (1, 3, 2)), ((2, 4, 2), (2, 4, 2))])
def test_conv_grid_matches_definition(ks, st):
    ijk = random_sparse_ijk(400, 12, seed=7, lo=-5)
    out, off = orc.conv_grid(ijk, np.array([0, ijk.shape[0]]), ks, st)
    assert set(map(tuple, out.tolist())) == conv_grid_by_definition(ijk, ks, st)


# ----------------------------------------------------------------- dense equivalence -----
def _sparse_case(dense: bool, extent: int, seed: int):
    ijk = dense_ijk((extent,) * 3) if dense else random_sparse_ijk(int(0.35 * extent**3), extent, seed)
    src, soff = orc.grid_from_ijk(ijk, np.array([0, ijk.shape[0]]))
    return src, soff


@pytest.mark.parametrize(
    "dense,ks,st",
    [(True, k, s) for k, s in itertools.product([2, 3, 4, 5, 6], [1, 2, 4])]
    + [(False, k, s) for k, s in [(3, 1), (2, 2), (3, 2), (5, 1)]]
    + [(True, ks, st) for ks, st in itertools.product([(3, 3, 3), (1, 3, 1), (4, 1, 4), (5, 3, 1)], [(1, 1, 1), (2, 2, 2), (1, 3, 2)])],
)
def test_oracle_forward_backward_vs_dense_conv3d(dense, ks, st):
    ks = (ks,) * 3 if isinstance(ks, int) else tuple(ks)
    st = (st,) * 3 if isinstance(st, int) else tuple(st)
    if ks == (1, 1, 1) and st == (1, 1, 1):
        pytest.skip("1x1 conv has no kernel map")
    extent = 12
    src, soff = _sparse_case(dense, extent, seed=sum(ks) * 10 + sum(st))
    tgt, toff = (src, soff) if st == (1, 1, 1) else orc.conv_grid(src, soff, ks, st)
    kmap = orc.kernel_map(src, soff, tgt, toff, ks, st)
    rng = np.random.default_rng(3)
    x = rng.standard_normal((src.shape[0], 4))
    w = rng.standard_normal((5, 4) + ks)
    out = orc.conv_forward_f64(x, w, kmap)
    # the dense box is shifted by 12 per axis (a multiple of every stride used) so that
    # targets at negative coordinates (e.g. k=5, s=2) land inside it: target t -> t + 12/s
    shift = 12
    sax = [st[2], st[1], st[0]]  # stride acting on ijk axis 0, 1, 2
    kax = [ks[2], ks[1], ks[0]]
    size = [int(tgt[:, a].max() + shift // sax[a]) * sax[a] + kax[a] + 2 for a in range(3)]
    size = [max(sz, extent + shift + 2) for sz in size]
    xt = torch.from_numpy(x).requires_grad_(True)
    wt = torch.from_numpy(w).requires_grad_(True)
    dense_in = torch.zeros((size[0], size[1], size[2], 4), dtype=torch.float64)
    sidx = tuple(torch.from_numpy(src[:, a] + shift).long() for a in range(3))
    dense_in = dense_in.index_put(sidx, xt)
    pad = [-kernel_start(k) for k in ks]
    ref = torch.nn.functional.conv3d(dense_in.permute(3, 2, 1, 0)[None], wt, padding=pad, stride=st)[0]
    tpos = [torch.from_numpy(tgt[:, a] + shift // sax[a]).long() for a in range(3)]
    ref_rows = ref[:, tpos[2], tpos[1], tpos[0]].T
    np.testing.assert_allclose(out, ref_rows.detach().numpy(), rtol=1e-10, atol=1e-10)
    # backward
    dy = rng.standard_normal(out.shape)
    ref_rows.backward(torch.from_numpy(dy))
    dx, dw = orc.conv_backward_f64(x, w, kmap, dy)
    np.testing.assert_allclose(dx, xt.grad.numpy(), rtol=1e-9, atol=1e-9)
    np.testing.assert_allclose(dw, wt.grad.numpy(), rtol=1e-9, atol=1e-9)


@pytest.mark.parametrize("k", [2, 3, 4, 5, 6])
def test_oracle_transposed_vs_conv_transpose3d(k):
    """test_torch_transposed_sparse_conv (test_conv.py:579-675): stride 1 on a dense box."""
    extent = 10
    src, soff = _sparse_case(True, extent, 0)
    kmap = orc.kernel_map(src, soff, src, soff, (k,) * 3, (1,) * 3)
    rng = np.random.default_rng(k)
    x = rng.standard_normal((src.shape[0], 4))  # features on the target grid (== source here)
    w = rng.standard_normal((4, 6, k, k, k))  # (Cin, Cout, K0, K1, K2)
    out = orc.conv_forward_f64(x, w, kmap, transposed=True, n_src=src.shape[0])
    xt = torch.from_numpy(x).requires_grad_(True)
    wt = torch.from_numpy(w).requires_grad_(True)
    dense_in = torch.zeros((extent, extent, extent, 4), dtype=torch.float64)
    dense_in = dense_in.index_put((torch.from_numpy(src[:, 0]).long(), torch.from_numpy(src[:, 1]).long(), torch.from_numpy(src[:, 2]).long()), xt)
    p = -kernel_start(k)
    ref = torch.nn.functional.conv_transpose3d(dense_in.permute(3, 2, 1, 0)[None], wt, stride=1, padding=p)[0]
    ref = ref[:, :extent, :extent, :extent]
    idx = (slice(None), torch.from_numpy(src[:, 2]).long(), torch.from_numpy(src[:, 1]).long(), torch.from_numpy(src[:, 0]).long())
    ref_rows = ref[idx].T
    np.testing.assert_allclose(out, ref_rows.detach().numpy(), rtol=1e-10, atol=1e-10)
    dy = rng.standard_normal(out.shape)
    ref_rows.backward(torch.from_numpy(dy))
    dx, dw = orc.conv_backward_f64(x, w, kmap, dy, transposed=True, n_src=src.shape[0])
    np.testing.assert_allclose(dx, xt.grad.numpy(), rtol=1e-9, atol=1e-9)
    np.testing.assert_allclose(dw, wt.grad.numpy(), rtol=1e-9, atol=1e-9)


@pytest.mark.parametrize("st,middle", [((1, 1, 1), True), ((1, 1, 1), False), ((2, 2, 2), False)])
def test_reference_cpu_path_matches_f64(st, middle):
    """The timed CPU baseline (gather -> torch.mm -> scatter, float32) equals the FP64 sums."""
    src, soff = _sparse_case(False, 20, 5)
    tgt, toff = (src, soff) if st == (1, 1, 1) else orc.conv_grid(src, soff, (3, 3, 3), st)
    kmap = orc.kernel_map(src, soff, tgt, toff, (3, 3, 3), st)
    nbmap, nbsizes = orc.neighbour_map(kmap)
    rng = np.random.default_rng(0)
    x = rng.standard_normal((src.shape[0], 16)).astype(np.float32)
    w = (rng.standard_normal((16, 16, 3, 3, 3)) / np.sqrt(27 * 16)).astype(np.float32)
    got = orc.gs_forward(torch.from_numpy(x), torch.from_numpy(w), nbmap, nbsizes, tgt.shape[0], middle=middle)
    ref = orc.conv_forward_f64(x, w, kmap)
    np.testing.assert_allclose(got.numpy(), ref, rtol=1e-4, atol=1e-5)


def test_neighbour_map_order():
    src, soff = _sparse_case(False, 10, 9)
    kmap = orc.kernel_map(src, soff, src, soff, (3, 3, 3), (1, 1, 1))
    nbmap, nbsizes = orc.neighbour_map(kmap)
    assert nbsizes.sum() == (kmap >= 0).sum() == nbmap.shape[0]
    # ordered by (offset, out) as torch.nonzero(kmap.t() != -1)
    k_of = np.repeat(np.arange(kmap.shape[1]), nbsizes)
    key = k_of.astype(np.int64) * (1 << 32) + nbmap[:, 1]
    assert np.all(np.diff(key) > 0)
    assert np.array_equal(kmap[nbmap[:, 1], k_of], nbmap[:, 0])
