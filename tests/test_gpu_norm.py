"""Normalisation layers of the sparse path and the inference fusion of a batch norm into the
convolution before it.

* nn.GroupNorm normalises each (grid, group) over its voxels and channels: equal, within FP32
  rounding, to torch.nn.GroupNorm run grid by grid (the reference's per-grid loop,
  fvdb/nn/modules.py:408-432), gradients included; an empty grid in the batch is skipped.
* nn.BatchNorm is torch.nn.BatchNorm1d on the [N, C] feature matrix.
* Under no_grad, nn.Sequential runs SparseConv3d -> BatchNorm (eval) [-> ReLU] as one
  convolution with the batch norm's affine map in the epilogue (out_scale): within one output
  rounding of the three layers run one by one (FP32 1e-5 relative L2, BF16 1e-2), and the
  folded form is inference-only.
"""

import pytest
import torch

from tests.helpers import random_sparse_ijk

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = a.detach().double(), b.detach().double()
    return float((a - b).norm() / b.norm().clamp(min=1e-30))


def _batch(fvdb, dev, sizes, extent=24, seed=3):
    parts = [torch.from_numpy(random_sparse_ijk(n, extent, seed + i)).to(dev) if n else
             torch.zeros((0, 3), dtype=torch.int32, device=dev) for i, n in enumerate(sizes)]
    return fvdb.GridBatch.from_ijk(fvdb.JaggedTensor(parts))


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_group_norm_equals_per_grid_loop(cuda_device, dtype):
    import fvdb
    import fvdb.nn as fvnn

    grid = _batch(fvdb, cuda_device, [900, 0, 2500, 40])
    g = torch.Generator().manual_seed(1)
    C, G = 24, 6
    x0 = (torch.randn(grid.total_voxels, C, generator=g, dtype=dtype) * 3 + 1).to(cuda_device)
    dy = torch.randn(grid.total_voxels, C, generator=g, dtype=dtype).to(cuda_device)
    ours = fvnn.GroupNorm(G, C).to(cuda_device, dtype)
    with torch.no_grad():
        ours.weight.copy_(torch.rand(C, generator=g, dtype=dtype) + 0.5)
        ours.bias.copy_(torch.randn(C, generator=g, dtype=dtype))
    ref = torch.nn.GroupNorm(G, C).to(cuda_device, dtype)
    ref.load_state_dict(ours.state_dict())

    x = x0.clone().requires_grad_(True)
    y = ours(fvnn.VDBTensor(grid, grid.jagged_like(x))).data.jdata
    y.backward(dy)

    xr = x0.clone().requires_grad_(True)
    off = grid.joffsets.tolist()
    outs = []
    for b in range(grid.grid_count):
        f = xr[off[b]:off[b + 1]]
        if f.shape[0]:
            outs.append(ref(f.t().reshape(1, C, -1)).reshape(C, -1).t())
    yr = torch.cat(outs)
    yr.backward(dy)
    tol = 1e-5 if dtype == torch.float32 else 1e-12
    assert rel(y, yr) <= tol
    assert rel(x.grad, xr.grad) <= tol * 10
    assert rel(ours.weight.grad, ref.weight.grad) <= tol * 10
    assert rel(ours.bias.grad, ref.bias.grad) <= tol * 10


def test_batch_norm_is_batchnorm1d_on_features(cuda_device):
    import fvdb
    import fvdb.nn as fvnn

    grid = _batch(fvdb, cuda_device, [700, 300])
    x = torch.randn(grid.total_voxels, 16, device=cuda_device)
    ours, ref = fvnn.BatchNorm(16).to(cuda_device), torch.nn.BatchNorm1d(16).to(cuda_device)
    for train in (True, False):
        ours.train(train), ref.train(train)
        assert torch.equal(ours(fvnn.VDBTensor(grid, grid.jagged_like(x))).data.jdata, ref(x))
    with pytest.raises(ValueError):
        ours(fvnn.VDBTensor(grid, grid.jagged_like(x[:, :8])))


def _stack(fvnn, cin, cout, dev, dtype, relu, bias, ks=3, stride=1):
    conv = fvnn.SparseConv3d(cin, cout, ks, stride, bias=bias)
    bn = fvnn.BatchNorm(cout)
    g = torch.Generator().manual_seed(cin * 3 + cout)
    with torch.no_grad():
        bn.running_mean.copy_(torch.randn(cout, generator=g) * 0.2)
        bn.running_var.copy_(torch.rand(cout, generator=g) + 0.3)
        bn.weight.copy_(torch.rand(cout, generator=g) + 0.5)
        bn.bias.copy_(torch.randn(cout, generator=g) * 0.1)
    mods = [conv, bn] + ([fvnn.ReLU()] if relu else [])
    return fvnn.Sequential(*mods).to(dev, dtype).eval()


@pytest.mark.parametrize("dtype,cin,cout,relu,bias,ks,stride", [
    (torch.float32, 16, 32, True, True, 3, 1),
    (torch.float32, 8, 24, False, False, 3, 1),
    (torch.bfloat16, 32, 64, True, True, 3, 1),
    (torch.bfloat16, 64, 64, False, True, 3, 1),
    (torch.bfloat16, 32, 64, True, False, 2, 2),
    (torch.float32, 16, 16, True, True, 1, 1),
])
def test_sequential_folds_eval_batch_norm(cuda_device, dtype, cin, cout, relu, bias, ks, stride):
    import fvdb
    import fvdb.nn as fvnn

    grid = _batch(fvdb, cuda_device, [3000, 1200])
    seq = _stack(fvnn, cin, cout, cuda_device, dtype, relu, bias, ks, stride)
    x = fvnn.VDBTensor(grid, grid.jagged_like(torch.randn(grid.total_voxels, cin, device=cuda_device, dtype=dtype)))
    seen = []
    conv = seq[0]
    orig = conv.forward

    def spy(*a, **k):
        seen.append(k.get("out_affine") is not None)
        return orig(*a, **k)

    conv.forward = spy
    with torch.no_grad():
        for _ in range(2):  # the second pass reuses the map (row order / derived weights)
            fused = seq(x)
            unfused = x
            for m in seq:
                unfused = nn_forward(m, unfused)
            assert torch.equal(fused.grid.ijk.jdata, unfused.grid.ijk.jdata)
            assert fused.data.jdata.dtype == unfused.data.jdata.dtype == dtype
            assert rel(fused.data.jdata, unfused.data.jdata) <= (1e-5 if dtype == torch.float32 else 1e-2)
            if relu:
                assert (fused.data.jdata >= 0).all()
    torch.cuda.synchronize()
    fvdb._lib.load().check_device_errors(cuda_device)
    assert seen and all(seen)


def nn_forward(m, x):
    """One layer on its own (no fusion)."""
    return type(m).forward(m, x)


def test_folded_batch_norm_is_inference_only(cuda_device):
    import fvdb
    import fvdb.nn as fvnn

    grid = _batch(fvdb, cuda_device, [800])
    seq = _stack(fvnn, 8, 16, cuda_device, torch.float32, True, True)
    x = fvnn.VDBTensor(grid, grid.jagged_like(torch.randn(grid.total_voxels, 8, device=cuda_device)))
    # with autograd on, the layers run one by one (gradients flow through the batch norm)
    y = seq(x).data.jdata
    y.sum().backward()
    assert seq[0].weight.grad is not None and seq[1].weight.grad is not None
    with pytest.raises(RuntimeError):
        seq[0](x, out_affine=seq[1].folded_affine())
    # a training-mode batch norm normalises with batch statistics: no folding
    seq[1].train()
    assert seq[1].folded_affine() is None
