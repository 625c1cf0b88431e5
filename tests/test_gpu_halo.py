"""GridBatch.sparse_conv_halo: the reference's stride-1 3x3x3 halo-tiled convolution API
(tests/unit/test_conv.py:133-200 set-up: 100 random points per grid at voxel size 0.05, batch 1
and 4, FP32).  Forward and both gradients against the FP64 oracle (the reference's gather-scatter
convolution), the same integers as sparse_conv_3d over the grid's stride-1 3^3 map, and the
reference's error types."""

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
    # the same result as the kernel-map path on the same grid
    pack, _ = grid.sparse_conv_kernel_map(3, 1)
    assert torch.equal(pack.sparse_conv_3d(feats.jdata.detach(), w.detach()).jdata, out.jdata.detach())


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
