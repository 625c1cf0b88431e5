"""GPU parity of pooling and nearest upsampling (fvdb.nn.MaxPool / AvgPool / UpsamplingNearest)
against the oracle: grids (coarsened / subdivided) bit-exact, FP32 and FP64 values and gradients
bit-exact where the reference is deterministic (non-overlapping windows), BF16 within 1e-2 of
the oracle on the same rounded inputs, overlapping windows within 1e-6 (FP32; summation order)."""

import numpy as np
import pytest
import torch

from oracle import oracle as orc
from tests.helpers import random_sparse_ijk

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def fvdb(cuda_device):
    import fvdb as m

    return m


def _grid(fvdb, dev, seeds=(1, 2), n=3000, extent=24):
    parts = [random_sparse_ijk(n, extent, s, lo=-10 * s) for s in seeds]
    ijk = np.concatenate(parts)
    off = np.cumsum([0] + [p.shape[0] for p in parts])
    jt = fvdb.JaggedTensor.from_data_and_offsets(torch.from_numpy(ijk).to(dev), torch.from_numpy(off).to(dev))
    g = fvdb.GridBatch.from_ijk(jt)
    return g, g.ijk.jdata.cpu().numpy(), g.joffsets.cpu().numpy()


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
@pytest.mark.parametrize("mode", ["max", "avg"])
@pytest.mark.parametrize("pool,stride", [(2, 0), ((2, 3, 1), 0), (3, 4), (2, (2, 3, 2))])
def test_pool_bit_exact(fvdb, cuda_device, dtype, mode, pool, stride):
    g, ijk, off = _grid(fvdb, cuda_device)
    x = torch.randn(g.total_voxels, 5, dtype=dtype, generator=torch.Generator().manual_seed(3))
    xd = x.to(cuda_device).requires_grad_(True)
    fn = g.max_pool if mode == "max" else g.avg_pool
    y, cg = fn(pool, fvdb.JaggedTensor.from_data_and_offsets(xd, g.joffsets), stride=stride)
    st = stride if stride else pool
    c_o, coff_o = orc.coarsened_grid(ijk, off, st)
    c = cg.ijk.jdata.cpu().numpy()
    assert np.array_equal(c, c_o) and np.array_equal(cg.joffsets.cpu().numpy(), coff_o)
    ref = orc.pool_forward(ijk, off, c, coff_o, x.numpy(), pool, stride, mode)
    assert np.array_equal(y.jdata.detach().cpu().numpy(), ref)
    dy = torch.randn(y.jdata.shape, dtype=dtype, generator=torch.Generator().manual_seed(4))
    y.jdata.backward(dy.to(cuda_device))
    ref_dx = orc.pool_backward(ijk, off, c, coff_o, x.numpy(), dy.numpy(), pool, stride, mode)
    assert np.array_equal(xd.grad.cpu().numpy(), ref_dx)


def test_overlapping_windows_and_user_coarse_grid(fvdb, cuda_device):
    g, ijk, off = _grid(fvdb, cuda_device)
    cg = g.coarsened_grid(2)  # stride 2 with a 3-wide window: windows overlap
    x = torch.randn(g.total_voxels, 4, generator=torch.Generator().manual_seed(5))
    xd = x.to(cuda_device).requires_grad_(True)
    y, out_grid = g.avg_pool(3, fvdb.JaggedTensor.from_data_and_offsets(xd, g.joffsets), stride=2, coarse_grid=cg)
    assert out_grid.is_same(cg)
    c, coff = cg.ijk.jdata.cpu().numpy(), cg.joffsets.cpu().numpy()
    ref = orc.pool_forward(ijk, off, c, coff, x.numpy(), 3, 2, "avg")
    assert np.array_equal(y.jdata.detach().cpu().numpy(), ref)
    dy = torch.randn(y.jdata.shape, generator=torch.Generator().manual_seed(6))
    y.jdata.backward(dy.to(cuda_device))
    ref_dx = orc.pool_backward(ijk, off, c, coff, x.numpy(), dy.numpy(), 3, 2, "avg")
    np.testing.assert_allclose(xd.grad.cpu().numpy(), ref_dx, rtol=1e-6, atol=1e-6)


def test_bf16_pool_and_modules(fvdb, cuda_device):
    g, ijk, off = _grid(fvdb, cuda_device)
    x = torch.randn(g.total_voxels, 8, generator=torch.Generator().manual_seed(7)).bfloat16()
    vt = fvdb.nn.VDBTensor(g, g.jagged_like(x.to(cuda_device)))
    out = fvdb.nn.MaxPool(2)(vt)
    c, coff = out.grid.ijk.jdata.cpu().numpy(), out.grid.joffsets.cpu().numpy()
    ref = orc.pool_forward(ijk, off, c, coff, x.float().numpy(), 2, 0, "max")
    assert np.array_equal(out.data.jdata.float().cpu().numpy(), ref)  # max of bf16 values is exact
    avg = fvdb.nn.AvgPool(2)(vt)
    ref_a = orc.pool_forward(ijk, off, c, coff, x.float().numpy(), 2, 0, "avg")
    np.testing.assert_allclose(avg.data.jdata.float().cpu().numpy(), ref_a, rtol=1e-2, atol=1e-2)
    # coarse transform as the reference: size 2w, origin o + w/2
    assert torch.allclose(out.grid.voxel_sizes[0], g.voxel_sizes[0] * 2)
    assert torch.allclose(out.grid.origins[0], g.origins[0] + 0.5 * g.voxel_sizes[0])


def test_maxpool_module_zeroes_empty_windows(fvdb, cuda_device):
    src = fvdb.GridBatch.from_ijk(torch.tensor([[0, 0, 0], [1, 1, 1]], dtype=torch.int32, device=cuda_device))
    coarse = fvdb.GridBatch.from_ijk(torch.tensor([[0, 0, 0], [5, 5, 5]], dtype=torch.int32, device=cuda_device))
    vt = fvdb.nn.VDBTensor(src, src.jagged_like(torch.tensor([[1.0], [-3.0]], device=cuda_device)))
    raw, _ = src.max_pool(2, vt.data, coarse_grid=coarse)
    assert torch.isinf(raw.jdata[1]).all() and raw.jdata[1, 0] < 0
    out = fvdb.nn.MaxPool(2)(vt, coarse)
    assert out.data.jdata[:, 0].tolist() == [1.0, 0.0]


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
@pytest.mark.parametrize("factor,masked", [(2, False), ((1, 2, 3), True)])
def test_upsample_bit_exact(fvdb, cuda_device, dtype, factor, masked):
    g, ijk, off = _grid(fvdb, cuda_device, n=800, extent=16)
    mask = None
    if masked:
        mask = torch.rand(g.total_voxels, generator=torch.Generator().manual_seed(8)) < 0.6
    x = torch.randn(g.total_voxels, 3, dtype=dtype, generator=torch.Generator().manual_seed(9))
    xd = x.to(cuda_device).requires_grad_(True)
    y, fg = g.subdivide(factor, fvdb.JaggedTensor.from_data_and_offsets(xd, g.joffsets),
                        mask=None if mask is None else mask.to(cuda_device))
    f_o, foff_o = orc.subdivided_grid(ijk, off, factor, None if mask is None else mask.numpy())
    f = fg.ijk.jdata.cpu().numpy()
    assert np.array_equal(f, f_o) and np.array_equal(fg.joffsets.cpu().numpy(), foff_o)
    assert np.array_equal(y.jdata.detach().cpu().numpy(), orc.upsample_forward(ijk, off, f, foff_o, x.numpy(), factor))
    dy = torch.randn(y.jdata.shape, dtype=dtype, generator=torch.Generator().manual_seed(10))
    y.jdata.backward(dy.to(cuda_device))
    assert np.array_equal(xd.grad.cpu().numpy(), orc.upsample_backward(ijk, off, f, foff_o, dy.numpy(), factor))
    # fine transform as the reference: size w/f, origin o - (f-1) w / (2f)
    fv = torch.tensor(orc._vec3(factor), dtype=torch.float64)
    vs, org = g.voxel_sizes[0].cpu().double(), g.origins[0].cpu().double()
    assert torch.allclose(fg.voxel_sizes[0].cpu().double(), vs / fv)
    assert torch.allclose(fg.origins[0].cpu().double(), org - (fv - 1) * vs / fv * 0.5)


def test_upsample_module_onto_user_grid(fvdb, cuda_device):
    coarse = fvdb.GridBatch.from_ijk(torch.tensor([[0, 0, 0]], dtype=torch.int32, device=cuda_device))
    fine = fvdb.GridBatch.from_ijk(torch.tensor([[1, 1, 1], [4, 4, 4]], dtype=torch.int32, device=cuda_device))
    vt = fvdb.nn.VDBTensor(coarse, coarse.jagged_like(torch.tensor([[2.5, -1.0]], device=cuda_device)))
    out = fvdb.nn.UpsamplingNearest(2)(vt, ref_fine_data=fine)
    assert out.grid.is_same(fine)
    # (1,1,1) has parent (0,0,0); (4,4,4) has none and reads zero
    assert out.data.jdata.cpu().tolist() == [[2.5, -1.0], [0.0, 0.0]]
