"""GridBatch.sparse_conv_halo: the reference's stride-1 3x3x3 halo-tiled convolution API
(tests/unit/test_conv.py:133-200 set-up: 100 random points per grid at voxel size 0.05, batch 1
and 4, FP32), computed by the leaf-halo kernels with no kernel map.  Forward and both gradients
against the FP64 oracle (the reference's gather-scatter convolution), agreement with
sparse_conv_3d over the grid's stride-1 3^3 map up to summation order, dense blocks that cross
leaf boundaries at negative coordinates, FP64 / BF16 data, an empty grid, and the reference's
error types."""

import numpy as np
import pytest
import torch

from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


@pytest.mark.parametrize("cin,cout,batch", [(8, 8, 1), (64, 128, 4), (128, 64, 4), (8, 64, 4)])
def test_halo_matches_oracle_forward_and_backward(cuda_device, cin, cout, batch):
    import fvdb

    torch.manual_seed(0)
    pts = [torch.randn((100, 3), device=cuda_device) for _ in range(batch)]
    grid = fvdb.GridBatch.from_points(fvdb.JaggedTensor(pts), voxel_sizes=0.05, origins=[0.0] * 3)
    feats = grid.jagged_like(torch.randn((grid.total_voxels, cin), device=cuda_device))
    w = torch.randn(cout, cin, 3, 3, 3, device=cuda_device)
    feats.jdata.requires_grad_(True)
    w.requires_grad_(True)
    out = grid.sparse_conv_halo(feats, w, 8)
    dy = torch.randn_like(out.jdata)
    out.jdata.backward(dy)
    ijk = grid.ijk.jdata.cpu().numpy()
    off = grid.joffsets.cpu().numpy()
    kmap = orc.kernel_map(ijk, off, ijk, off, 3, 1)
    x64, w64, dy64 = (t.detach().double().cpu().numpy() for t in (feats.jdata, w, dy))
    ref = orc.conv_forward_f64(x64, w64, kmap)
    dx, dw = orc.conv_backward_f64(x64, w64, kmap, dy64)
    assert rel_l2(out.jdata.detach().double().cpu().numpy(), ref) < 1e-5
    assert rel_l2(feats.jdata.grad.double().cpu().numpy(), dx) < 1e-5
    assert rel_l2(w.grad.double().cpu().numpy(), dw) < 1e-5
    # the kernel-map path on the same grid: the same sums in another order
    pack, _ = grid.sparse_conv_kernel_map(3, 1)
    torch.testing.assert_close(pack.sparse_conv_3d(feats.jdata.detach(), w.detach()).jdata, out.jdata.detach(),
                               rtol=1e-5, atol=1e-5)


def _block_grid(fvdb, device, seed, batch=2, extent=20, keep=0.7):
    """Dense-ish blocks around the origin (leaves full and partly full, halos across leaf
    boundaries and negative coordinates), a different hole pattern per grid."""
    g = torch.Generator().manual_seed(seed)
    r = torch.arange(-extent // 2, extent - extent // 2, dtype=torch.int32)
    cube = torch.stack(torch.meshgrid(r, r, r, indexing="ij"), -1).reshape(-1, 3)
    parts = [cube[torch.rand(cube.shape[0], generator=g) < keep] + 3 * b for b in range(batch)]
    return fvdb.GridBatch.from_ijk(fvdb.JaggedTensor([p.to(device) for p in parts]))


@pytest.mark.parametrize("dtype,tol", [(torch.float32, 1e-5), (torch.float64, 1e-12)])
@pytest.mark.parametrize("cin,cout", [(16, 16), (3, 40), (64, 32)])
def test_halo_dense_blocks(cuda_device, dtype, tol, cin, cout):
    import fvdb

    grid = _block_grid(fvdb, cuda_device, seed=cin + cout)
    g = torch.Generator().manual_seed(5)
    x = torch.randn((grid.total_voxels, cin), generator=g, dtype=dtype)
    w = torch.randn((cout, cin, 3, 3, 3), generator=g, dtype=dtype)
    xd, wd = x.to(cuda_device).requires_grad_(True), w.to(cuda_device).requires_grad_(True)
    out = grid.sparse_conv_halo(grid.jagged_like(xd), wd)
    dy = torch.randn(out.jdata.shape, generator=g, dtype=dtype)
    out.jdata.backward(dy.to(cuda_device))
    ijk = grid.ijk.jdata.cpu().numpy()
    off = grid.joffsets.cpu().numpy()
    kmap = orc.kernel_map(ijk, off, ijk, off, 3, 1)
    x64, w64, dy64 = x.double().numpy(), w.double().numpy(), dy.double().numpy()
    ref = orc.conv_forward_f64(x64, w64, kmap)
    dx, dw = orc.conv_backward_f64(x64, w64, kmap, dy64)
    assert rel_l2(out.jdata.detach().double().cpu().numpy(), ref) < tol
    assert rel_l2(xd.grad.double().cpu().numpy(), dx) < tol
    assert rel_l2(wd.grad.double().cpu().numpy(), dw) < tol
    # the weight gradient is deterministic (fixed-order reduction)
    dw_first = wd.grad.clone()
    wd.grad = None
    out2 = grid.sparse_conv_halo(grid.jagged_like(xd), wd)
    out2.jdata.backward(dy.to(cuda_device))
    assert torch.equal(out2.jdata.detach(), out.jdata.detach())
    assert torch.equal(wd.grad, dw_first)


def test_halo_bf16(cuda_device):
    import fvdb

    grid = _block_grid(fvdb, cuda_device, seed=11)
    g = torch.Generator().manual_seed(6)
    x = torch.randn((grid.total_voxels, 32), generator=g).bfloat16()
    w = (torch.randn((32, 32, 3, 3, 3), generator=g) * 0.1).bfloat16()
    xd, wd = x.to(cuda_device).requires_grad_(True), w.to(cuda_device).requires_grad_(True)
    out = grid.sparse_conv_halo(grid.jagged_like(xd), wd)
    assert out.jdata.dtype == torch.bfloat16
    dy = torch.randn(out.jdata.shape, generator=g).bfloat16()
    out.jdata.backward(dy.to(cuda_device))
    ijk, off = grid.ijk.jdata.cpu().numpy(), grid.joffsets.cpu().numpy()
    kmap = orc.kernel_map(ijk, off, ijk, off, 3, 1)
    x64, w64, dy64 = x.double().numpy(), w.double().numpy(), dy.double().numpy()
    ref = orc.conv_forward_f64(x64, w64, kmap)
    dx, dw = orc.conv_backward_f64(x64, w64, kmap, dy64)
    # FP32 accumulation of BF16 products, one BF16 rounding of the result (2^-8 relative)
    assert rel_l2(out.jdata.detach().double().cpu().numpy(), ref) < 8e-3
    assert rel_l2(xd.grad.double().cpu().numpy(), dx) < 8e-3
    assert rel_l2(wd.grad.double().cpu().numpy(), dw) < 8e-3


def test_halo_deterministic_and_empty(cuda_device):
    import fvdb

    grid = _block_grid(fvdb, cuda_device, seed=3, batch=3)
    x = torch.randn((grid.total_voxels, 24), device=cuda_device, requires_grad=True)
    w = torch.randn((8, 24, 3, 3, 3), device=cuda_device, requires_grad=True)
    grads = []
    for _ in range(2):
        w.grad = None
        x.grad = None
        out = grid.sparse_conv_halo(grid.jagged_like(x), w)
        out.jdata.backward(torch.ones_like(out.jdata))
        grads.append((out.jdata.detach().clone(), x.grad.clone(), w.grad.clone()))
    for a, b in zip(*grads):
        assert torch.equal(a, b)
    empty = fvdb.GridBatch.from_ijk(fvdb.JaggedTensor([torch.zeros((0, 3), dtype=torch.int32, device=cuda_device)]))
    xe = torch.zeros((0, 8), device=cuda_device, requires_grad=True)
    we = torch.randn((4, 8, 3, 3, 3), device=cuda_device, requires_grad=True)
    oe = empty.sparse_conv_halo(empty.jagged_like(xe), we)
    assert oe.jdata.shape == (0, 4)
    oe.jdata.sum().backward()
    assert torch.equal(we.grad, torch.zeros_like(we))


def test_halo_error_types(cuda_device):
    import fvdb

    torch.manual_seed(1)
    grid = fvdb.GridBatch.from_points(fvdb.JaggedTensor([torch.randn((100, 3), device=cuda_device)]),
                                      voxel_sizes=0.05, origins=[0.0] * 3)
    f = grid.jagged_like(torch.randn((grid.total_voxels, 8), device=cuda_device))
    with pytest.raises(NotImplementedError):
        grid.sparse_conv_halo(f, torch.randn(8, 8, 5, 5, 5, device=cuda_device))
    with pytest.raises(ValueError):
        grid.sparse_conv_halo(f, torch.randn(8, 16, 3, 3, 3, device=cuda_device))
    with pytest.raises(ValueError):
        grid.sparse_conv_halo(f, torch.randn(8, 8, 3, 3, device=cuda_device))
    with pytest.raises(TypeError):
        grid.sparse_conv_halo(grid.jagged_like(torch.ones((grid.total_voxels, 8), device=cuda_device,
                                                          dtype=torch.int32)), torch.randn(8, 8, 3, 3, 3, device=cuda_device))
    with pytest.raises(ValueError):
        grid.sparse_conv_halo(fvdb.JaggedTensor([torch.randn((grid.total_voxels + 1, 8), device=cuda_device)]),
                              torch.randn(8, 8, 3, 3, 3, device=cuda_device))
