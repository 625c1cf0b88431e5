"""Bias added in the contraction's epilogue (nn.SparseConv3d with bias=True): forward against the
FP64 oracle plus bias, gradients of features and weights identical to the bias-free layer's, the
bias gradient equal to the column sum of dy, rows without any active offset equal to the bias,
and the FP32 CUDA-core path (bias added after the contraction)."""

import numpy as np
import pytest
import torch

from oracle import oracle as orc
from tests.helpers import random_sparse_ijk

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def _oracle_forward(grid, x, w, b):
    ijk = grid.ijk.jdata.cpu().numpy()
    off = grid.joffsets.cpu().numpy()
    kmap = orc.kernel_map(ijk, off, ijk, off, 3, 1)
    y = orc.conv_forward_f64(x.detach().double().cpu().numpy(), w.detach().double().cpu().numpy(), kmap)
    return y + b.detach().double().cpu().numpy()[None, :]


@pytest.mark.parametrize("dtype,tol", [(torch.bfloat16, 1e-2), (torch.float32, 1e-5), (torch.float64, 1e-12)])
def test_module_bias(cuda_device, dtype, tol):
    import fvdb

    grid = fvdb.GridBatch.from_ijk(torch.from_numpy(random_sparse_ijk(6000, 30, 21)).to(cuda_device))
    torch.manual_seed(5)
    conv = fvdb.nn.SparseConv3d(32, 64, 3, bias=True).to(cuda_device, dtype)
    plain = fvdb.nn.SparseConv3d(32, 64, 3, bias=False).to(cuda_device, dtype)
    with torch.no_grad():
        conv.bias.uniform_(-1.0, 1.0)
        plain.weight.copy_(conv.weight)
    x = torch.randn(grid.total_voxels, 32, device=cuda_device, dtype=dtype).requires_grad_(True)
    x2 = x.detach().clone().requires_grad_(True)
    y = conv(fvdb.nn.VDBTensor(grid, grid.jagged_like(x))).data.jdata
    y2 = plain(fvdb.nn.VDBTensor(grid, grid.jagged_like(x2))).data.jdata
    dy = torch.randn_like(y)
    y.backward(dy)
    y2.backward(dy)
    torch.cuda.synchronize()
    fvdb._lib.load().check_device_errors(cuda_device)
    assert rel_l2(y.detach().double().cpu().numpy(), _oracle_forward(grid, x, conv.weight, conv.bias)) <= tol
    assert torch.equal(x.grad, x2.grad)
    assert torch.equal(conv.weight.grad, plain.weight.grad)
    db = dy.double().sum(0)
    assert conv.bias.grad.dtype == dtype
    assert rel_l2(conv.bias.grad.double().cpu().numpy(), db.cpu().numpy()) <= tol


def test_output_dtype_follows_promotion(cuda_device):
    """precision='bf16' on an FP32 module: the output is FP32, as the reference's conv(x) + bias
    (the bias is then added after the BF16 contraction instead of in its epilogue)."""
    import fvdb

    grid = fvdb.GridBatch.from_ijk(torch.from_numpy(random_sparse_ijk(3000, 24, 9)).to(cuda_device))
    torch.manual_seed(2)
    conv = fvdb.nn.SparseConv3d(32, 64, 3, bias=True).to(cuda_device)
    conv.precision = "bf16"
    x = torch.randn(grid.total_voxels, 32, device=cuda_device)
    y = conv(fvdb.nn.VDBTensor(grid, grid.jagged_like(x))).data.jdata
    assert y.dtype == torch.float32
    ref = _oracle_forward(grid, x.bfloat16().float(), conv.weight.bfloat16().float(), conv.bias)
    assert rel_l2(y.detach().double().cpu().numpy(), ref) <= 1e-2


def test_bias_alone_where_no_offset_is_active(cuda_device):
    import fvdb

    src = fvdb.GridBatch.from_ijk(torch.from_numpy(random_sparse_ijk(3000, 24, 4)).to(cuda_device))
    tgt = fvdb.GridBatch.from_ijk(torch.from_numpy(random_sparse_ijk(2000, 24, 5, lo=1000)).to(cuda_device))
    pack, _ = src.sparse_conv_kernel_map(3, 1, target_grid=tgt)
    x = torch.randn(src.total_voxels, 32, device=cuda_device).bfloat16()
    w = torch.randn(64, 32, 3, 3, 3, device=cuda_device).bfloat16()
    b = torch.randn(64, device=cuda_device).bfloat16()  # same dtype: fused into the epilogue
    y = pack._conv_with_bias(x, w, b, False).jdata
    torch.cuda.synchronize()
    assert y.shape == (tgt.total_voxels, 64) and y.dtype == torch.bfloat16
    assert torch.equal(y, b[None, :].expand_as(y))
    b32 = b.float()  # promotes: added after the contraction, FP32 output
    y32 = pack._conv_with_bias(x, w, b32, False).jdata
    assert y32.dtype == torch.float32 and torch.equal(y32, b32[None, :].expand_as(y32))
