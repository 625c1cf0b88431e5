"""The feature-wise layers of fvdb.nn and FillFromGrid / GridBatch.inject_from.

* Every activation, Linear and Dropout layer equals the torch layer on the [N, C] features, with
  grid and kernel map passed through (reference: fvdb/nn/modules.py:529-620).
* inject_from copies rows of the source grid's voxels that the destination holds, grid by grid in
  index space, and fills the rest with default_value (or keeps dst): checked against a host
  dictionary of (grid, i, j, k) -> row; gradients reach the injected rows only.
* FillFromGrid is inject_from onto the other VDBTensor's grid, keeping its kernel map.
"""

import numpy as np
import pytest
import torch

from tests.helpers import random_sparse_ijk

pytestmark = pytest.mark.gpu


def _batch(fvdb, dev, sizes, extent, seed):
    parts = [torch.from_numpy(random_sparse_ijk(n, extent, seed + i)).to(dev) for i, n in enumerate(sizes)]
    return fvdb.GridBatch.from_ijk(fvdb.JaggedTensor(parts))


@pytest.mark.parametrize("name,args", [("ReLU", ()), ("LeakyReLU", (0.1,)), ("ELU", (0.7,)), ("CELU", (1.3,)),
                                       ("GELU", ()), ("SELU", ()), ("SiLU", ()), ("Tanh", ()), ("Sigmoid", ()),
                                       ("Linear", (16, 8)), ("Dropout", (0.3,))])
def test_feature_layers_equal_torch(cuda_device, name, args):
    import fvdb
    import fvdb.nn as fvnn

    grid = _batch(fvdb, cuda_device, [500, 900], 16, 5)
    x = torch.randn(grid.total_voxels, 16, device=cuda_device)
    kmap, _ = grid.sparse_conv_kernel_map(3, 1)
    t = fvnn.VDBTensor(grid, grid.jagged_like(x), kmap)
    ours = getattr(fvnn, name)(*args).to(cuda_device).eval()
    ref = getattr(torch.nn, name)(*args).to(cuda_device).eval()
    ref.load_state_dict(ours.state_dict())
    out = ours(t)
    assert out.grid.is_same(grid) and out.kmap is kmap
    assert torch.equal(out.data.jdata, ref(x))
    with pytest.raises(TypeError):
        ours(x)


def _rows(grid):
    ijk = grid.ijk.jdata.cpu().numpy()
    b = grid.jidx.cpu().numpy() if hasattr(grid, "jidx") else None
    off = grid.joffsets.cpu().numpy()
    bidx = np.repeat(np.arange(len(off) - 1), np.diff(off)) if b is None else b.astype(np.int64)
    return {(int(bi), *map(int, c)): r for r, (bi, c) in enumerate(zip(bidx, ijk))}


def test_inject_from_matches_host_lookup(cuda_device):
    import fvdb

    src = _batch(fvdb, cuda_device, [3000, 0, 1500], 20, 11)
    dst = _batch(fvdb, cuda_device, [2500, 700, 1800], 20, 11 + 50)  # overlapping, not equal
    g = torch.Generator().manual_seed(3)
    x = torch.randn(src.total_voxels, 5, generator=g).to(cuda_device).requires_grad_(True)
    out = dst.inject_from(src, src.jagged_like(x), default_value=-7.0)
    srows = _rows(src)
    expect = np.full((dst.total_voxels, 5), -7.0, np.float32)
    xn = x.detach().cpu().numpy()
    hit = []
    for key, r in _rows(dst).items():
        if key in srows:
            expect[r] = xn[srows[key]]
            hit.append(srows[key])
    assert hit, "the grids should overlap"
    assert np.array_equal(out.jdata.detach().cpu().numpy(), expect)
    out.jdata.sum().backward()
    gexp = np.zeros(src.total_voxels)
    gexp[hit] = 1
    assert np.array_equal(x.grad[:, 0].cpu().numpy(), gexp)
    # into an existing destination: rows without a source voxel keep their values
    d0 = torch.randn(dst.total_voxels, 5, generator=g).to(cuda_device)
    out2 = dst.inject_from(src, src.jagged_like(x.detach()), dst.jagged_like(d0.clone()))
    miss = torch.ones(dst.total_voxels, dtype=torch.bool)
    for key, r in _rows(dst).items():
        if key in srows:
            miss[r] = False
    miss = miss.to(cuda_device)
    assert torch.equal(out2.jdata[miss], d0[miss])
    assert torch.equal(out2.jdata[~miss], out.jdata.detach()[~miss])
    with pytest.raises(ValueError):
        dst.inject_from(src, src.jagged_like(x.detach()), dst.jagged_like(torch.zeros(dst.total_voxels, 4,
                                                                                        device=cuda_device)))


def test_fill_from_grid(cuda_device):
    import fvdb
    import fvdb.nn as fvnn

    a = _batch(fvdb, cuda_device, [1200], 14, 21)
    b = _batch(fvdb, cuda_device, [1500], 14, 22)
    x = torch.randn(a.total_voxels, 3, device=cuda_device)
    kb, _ = b.sparse_conv_kernel_map(3, 1)
    other = fvnn.VDBTensor(b, b.jagged_like(torch.zeros(b.total_voxels, 3, device=cuda_device)), kb)
    layer = fvnn.FillFromGrid(default_value=2.5)
    out = layer(fvnn.VDBTensor(a, a.jagged_like(x)), other)
    assert out.grid.is_same(b) and out.kmap is kb
    assert torch.equal(out.data.jdata, b.inject_from(a, a.jagged_like(x), default_value=2.5).jdata)
    out_g = layer(fvnn.VDBTensor(a, a.jagged_like(x)), b)
    assert out_g.kmap is None and torch.equal(out_g.data.jdata, out.data.jdata)
    same = fvnn.VDBTensor(a, a.jagged_like(x))
    assert layer(same) is same


def test_vdbtensor_arithmetic_keeps_grid_and_map(cuda_device):
    import fvdb
    import fvdb.nn as fvnn

    grid = _batch(fvdb, cuda_device, [600, 400], 12, 31)
    kmap, _ = grid.sparse_conv_kernel_map(3, 1)
    a0 = torch.rand(grid.total_voxels, 4, device=cuda_device) + 0.5
    b0 = torch.rand(grid.total_voxels, 4, device=cuda_device) + 0.5
    a = fvnn.VDBTensor(grid, grid.jagged_like(a0.clone()), kmap)
    b = fvnn.VDBTensor(grid, grid.jagged_like(b0.clone()))
    for got, want in [(a + b, a0 + b0), (a - b, a0 - b0), (a * b, a0 * b0), (a / b, a0 / b0), (a ** 2, a0 ** 2),
                      (2.0 * a, 2.0 * a0), (-a, -a0), (a // b, a0 // b0), (a % b, a0 % b0), (a > b, a0 > b0),
                      (a.sqrt(), a0.sqrt()), ((a - 1).abs(), (a0 - 1).abs()), (a.floor(), a0.floor())]:
        assert got.grid.is_same(grid) and got.kmap is kmap
        assert torch.equal(got.jdata, want)
    c = a.clone()
    c += b
    c *= 3
    assert torch.equal(c.jdata, (a0 + b0) * 3) and torch.equal(a.jdata, a0)
    other = _batch(fvdb, cuda_device, [10], 12, 99)
    with pytest.raises(ValueError):
        a + fvnn.VDBTensor(other, other.jagged_like(torch.zeros(other.total_voxels, 4, device=cuda_device)))
    g0 = a[1]
    assert g0.grid.total_voxels == grid.num_voxels_at(1) and torch.equal(g0.jdata, a0[grid.cum_voxels_at(1):])
    assert a.to(torch.float64).dtype == torch.float64 and a.detach().requires_grad is False


def test_vdbtensor_from_dense_round_trip(cuda_device):
    import fvdb.nn as fvnn

    dense = torch.randn(2, 5, 6, 7, 3, device=cuda_device)
    t = fvnn.vdbtensor_from_dense(dense, ijk_min=[-2, 1, 4])
    assert t.grid_count == 2 and t.total_voxels == 2 * 5 * 6 * 7
    assert torch.equal(t.grid.ijk.jdata.min(0).values.cpu(), torch.tensor([-2, 1, 4], dtype=torch.int32))
    assert torch.equal(t.to_dense(), dense)


def test_jcat_grids_and_vdbtensors(cuda_device):
    import fvdb
    import fvdb.nn as fvnn

    a = _batch(fvdb, cuda_device, [300, 500], 12, 41)
    b = _batch(fvdb, cuda_device, [700], 12, 43)
    ab = fvdb.jcat([a, b])
    assert ab.grid_count == 3 and ab.total_voxels == a.total_voxels + b.total_voxels
    assert torch.equal(ab.ijk.jdata, torch.cat([a.ijk.jdata, b.ijk.jdata]))
    xa = torch.randn(a.total_voxels, 4, device=cuda_device)
    xb = torch.randn(b.total_voxels, 4, device=cuda_device)
    t = fvdb.jcat([fvnn.VDBTensor(a, a.jagged_like(xa)), fvnn.VDBTensor(b, b.jagged_like(xb))])
    assert t.grid.grid_count == 3 and torch.equal(t.jdata, torch.cat([xa, xb]))
    kmap, _ = a.sparse_conv_kernel_map(3, 1)
    skip = fvnn.VDBTensor(a, a.jagged_like(xa), kmap)
    up = fvnn.VDBTensor(a, a.jagged_like(xa * 2))
    cat = fvdb.jcat([up, skip], dim=1)
    assert cat.grid.is_same(a) and cat.jdata.shape == (a.total_voxels, 8)
    assert torch.equal(cat.jdata, torch.cat([xa * 2, xa], 1))
    with pytest.raises(ValueError):
        fvdb.jcat([up, skip], dim=0)
    with pytest.raises(ValueError):
        fvdb.jcat([a, b], dim=1)
