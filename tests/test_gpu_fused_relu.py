"""Convolution with ReLU fused into the epilogue: values and gradients identical to
torch.relu applied to the unfused convolution (rounding to the output type keeps signs, and the
backward masks with the same positions), on the tensor-core path (BF16, unplanned and over a
tile plan, FP8) and the CUDA-core path (FP32); nn.Sequential fuses SparseConv3d + ReLU."""

import numpy as np
import pytest
import torch

from tests.helpers import random_sparse_ijk

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def case(cuda_device):
    import fvdb

    grid = fvdb.GridBatch.from_ijk(torch.from_numpy(random_sparse_ijk(6000, 28, 31)).to(cuda_device))
    pack, _ = grid.sparse_conv_kernel_map(3, 1)
    return fvdb, grid, pack


@pytest.mark.parametrize("dtype,cin,cout", [(torch.bfloat16, 32, 64), (torch.bfloat16, 64, 64), (torch.float32, 16, 24)])
def test_fused_relu_equals_relu_of_conv(cuda_device, case, dtype, cin, cout):
    fvdb, grid, pack = case
    g = torch.Generator().manual_seed(cin + cout)
    x0 = torch.randn(grid.total_voxels, cin, generator=g).to(cuda_device, dtype)
    w0 = (torch.randn(cout, cin, 3, 3, 3, generator=g) * 0.1).to(cuda_device, dtype)
    b0 = torch.randn(cout, generator=g).to(cuda_device, dtype)
    dy = torch.randn(grid.total_voxels, cout, generator=g).to(cuda_device, dtype)
    for rep in range(2):  # the second pass runs over a tile plan where the shape takes one
        outs = []
        for fused in (True, False):
            x, w, b = (t.clone().requires_grad_(True) for t in (x0, w0, b0))
            if fused:
                y = pack._conv_with_bias(x, w, b, False, None, relu=True).jdata
            else:
                y = torch.relu(pack._conv_with_bias(x, w, b, False, None).jdata)
            y.backward(dy)
            outs.append((y.detach(), x.grad, w.grad, b.grad))
        torch.cuda.synchronize()
        fvdb._lib.load().check_device_errors(cuda_device)
        for a, r in zip(outs[0], outs[1]):
            assert torch.equal(a, r)
        assert (outs[0][0] >= 0).all() and (outs[0][0] == 0).any()


def test_fused_relu_fp8(cuda_device, case):
    fvdb, grid, pack = case
    g = torch.Generator().manual_seed(5)
    x = torch.randn(grid.total_voxels, 64, generator=g).to(cuda_device, torch.bfloat16)
    w = (torch.randn(64, 64, 3, 3, 3, generator=g) * 0.05).to(cuda_device, torch.bfloat16)
    with torch.no_grad():
        for _ in range(2):
            a = pack._conv_with_bias(x, w, None, False, "fp8", relu=True).jdata
            r = torch.relu(pack._conv_with_bias(x, w, None, False, "fp8").jdata)
            assert torch.equal(a, r)


def test_sequential_fuses_conv_relu(cuda_device, case):
    fvdb, grid, _ = case
    torch.manual_seed(3)
    c1 = fvdb.nn.SparseConv3d(32, 64, 3).to(cuda_device, torch.bfloat16)
    c2 = fvdb.nn.SparseConv3d(64, 32, 3).to(cuda_device, torch.bfloat16)
    seq = fvdb.nn.Sequential(c1, fvdb.nn.ReLU(), c2)
    x = torch.randn(grid.total_voxels, 32, device=cuda_device).bfloat16()
    vt = fvdb.nn.VDBTensor(grid, grid.jagged_like(x))
    y = seq(vt).data.jdata
    h = c1(vt)
    ref = c2(fvdb.nn.VDBTensor(h.grid, h.grid.jagged_like(torch.relu(h.data.jdata)), h.kmap)).data.jdata
    assert torch.equal(y, ref)
