"""Training-path parity: tensor-core weight gradient, FP64 central finite differences through a
conv -> ReLU -> conv stack, the reference's autograd gradient (oracle restatement of
SparseConvolutionKernelMap backward), and activation recomputation."""

import math

import numpy as np
import pytest
import torch

from oracle import oracle as orc
from tests.helpers import random_sparse_ijk

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def _grid(fvdb, dev, n, extent, seed):
    return fvdb.GridBatch.from_ijk(torch.from_numpy(random_sparse_ijk(n, extent, seed)).to(dev))


@pytest.mark.parametrize("cin,cout,ks,st,transposed", [(64, 64, 3, 1, False), (32, 64, 3, 1, False),
                                                        (128, 128, 3, 1, False), (64, 256, 2, 2, False),
                                                        (64, 128, 2, 2, True)])
def test_tensor_core_wgrad_bf16(cuda_device, cin, cout, ks, st, transposed):
    """BF16 weight gradient on tcgen05 (FP32 partials, FP64 cross-CTA sum): rel-L2 <= 1e-2 vs
    the FP64 oracle on the same bf16-rounded operands."""
    import fvdb

    grid = _grid(fvdb, cuda_device, 9000, 32, cin + cout)
    pack, tgt = grid.sparse_conv_kernel_map(ks, st)
    src = grid.ijk.jdata.cpu().numpy()
    t = tgt.ijk.jdata.cpu().numpy()
    kmap = orc.kernel_map(src, np.array([0, src.shape[0]]), t, np.array([0, t.shape[0]]), ks, st)
    g = torch.Generator().manual_seed(cin * 3 + cout)
    n_in = tgt.total_voxels if transposed else grid.total_voxels
    n_out = grid.total_voxels if transposed else tgt.total_voxels
    x = torch.randn(n_in, cin, generator=g).bfloat16()
    w = (torch.randn(((cin, cout) if transposed else (cout, cin)) + (ks,) * 3, generator=g) / math.sqrt(cin * ks**3)).bfloat16()
    dy = torch.randn(n_out, cout, generator=g).bfloat16()
    xt = x.to(cuda_device)
    wt = w.to(cuda_device).requires_grad_(True)
    f = pack.sparse_transpose_conv_3d if transposed else pack.sparse_conv_3d
    y = f(xt, wt).jdata
    y.backward(dy.to(cuda_device))
    torch.cuda.synchronize()
    fvdb._lib.load().check_device_errors(cuda_device)
    _, dw = orc.conv_backward_f64(x.double().numpy(), w.double().numpy(), kmap, dy.double().numpy(),
                                  transposed=transposed, n_src=grid.total_voxels)
    assert wt.grad.shape == wt.shape
    assert rel_l2(wt.grad.double().cpu().numpy(), dw) <= 1e-2


def _stack(fvdb, dev, dtype, seed=0, recompute=False):
    torch.manual_seed(seed)
    c1 = fvdb.nn.SparseConv3d(64, 64, 3, bias=False).to(dev, dtype)
    c2 = fvdb.nn.SparseConv3d(64, 64, 3, bias=False).to(dev, dtype)
    layers = [c1, fvdb.nn.ReLU(), c2]
    net = fvdb.nn.RecomputeSequential(*layers) if recompute else fvdb.nn.Sequential(*layers)
    return net, c1, c2


def test_finite_differences_fp64_and_bf16_gradients(cuda_device):
    """conv3^3(64->64) -> ReLU -> conv3^3(64->64) on a box-surface grid: analytic FP64 gradients
    of L = <y, dy> against FP64 central differences (eps = 1e-4) on 64 random features and 64
    random second-layer weights (error <= 1e-5 of max(|g|, 1e-3) each), then the BF16
    gradients against the FP64 ones (rel-L2 <= 1e-2)."""
    import fvdb

    from tests.synth import box_surfaces

    grid = fvdb.GridBatch.from_ijk(torch.from_numpy(box_surfaces(8, 64, 200)).to(cuda_device))
    net, c1, c2 = _stack(fvdb, cuda_device, torch.float64)
    x = torch.randn(grid.total_voxels, 64, dtype=torch.float64, device=cuda_device, generator=None)
    dy = torch.randn(grid.total_voxels, 64, dtype=torch.float64, device=cuda_device)

    def loss(xx):
        return (net(fvdb.nn.VDBTensor(grid, grid.jagged_like(xx))).data.jdata * dy).sum()

    xg = x.clone().requires_grad_(True)
    loss(xg).backward()
    gx, gw1 = xg.grad.clone(), c1.weight.grad.clone()
    rng = np.random.default_rng(0)
    eps = 1e-4
    with torch.no_grad():
        for _ in range(64):
            i, j = int(rng.integers(grid.total_voxels)), int(rng.integers(64))
            xp, xm = x.clone(), x.clone()
            xp[i, j] += eps
            xm[i, j] -= eps
            fd = (loss(xp) - loss(xm)).item() / (2 * eps)
            an = gx[i, j].item()
            assert abs(fd - an) <= 1e-5 * max(abs(an), 1e-3) + 1e-7
        # Weights: the second layer's (the loss is linear in them through the whole stack).  A
        # first-layer weight moves ~all pre-activations of one channel, so about one ReLU kink is
        # crossed per 1e-4 perturbation and central differences are not valid there; the
        # first-layer gradient is checked exactly against the reference gradient instead
        # (test_gradient_matches_reference_autograd).
        gw2 = c2.weight.grad.clone()
        wdat = c2.weight.data  # (Do, Di, K0, K1, K2) view of (K2, K1, K0, Di, Do) storage
        for _ in range(64):
            e = tuple(int(v) for v in np.unravel_index(int(rng.integers(wdat.numel())), tuple(wdat.shape)))
            old = wdat[e].item()
            wdat[e] = old + eps
            lp = loss(x).item()
            wdat[e] = old - eps
            lm = loss(x).item()
            wdat[e] = old
            fd = (lp - lm) / (2 * eps)
            an = gw2[e].item()
            assert abs(fd - an) <= 1e-5 * max(abs(an), 1e-3) + 1e-7
    # BF16 stack with the same weights
    net16, d1, d2 = _stack(fvdb, cuda_device, torch.bfloat16)
    with torch.no_grad():
        d1.weight.copy_(c1.weight)
        d2.weight.copy_(c2.weight)
    x16 = x.bfloat16().requires_grad_(True)
    y16 = net16(fvdb.nn.VDBTensor(grid, grid.jagged_like(x16))).data.jdata
    (y16.float() * dy.float()).sum().backward()
    # (a) against FP64 end to end.  BF16 rounding of the first layer's output flips the ReLU mask
    #     of the ~0.2 % of pre-activations within rounding distance of zero, and each flip drops or
    #     adds a whole gradient term: ~4 % rel-L2 on dx and dW1 (the same 3.9 % comes out of a CPU
    #     emulation of BF16 storage with the FP64 oracle), so the bound here is 6e-2.
    assert rel_l2(y16.detach().double().cpu().numpy(), net(fvdb.nn.VDBTensor(grid, grid.jagged_like(x))).data.jdata.detach().cpu().numpy()) <= 1e-2
    assert rel_l2(x16.grad.double().cpu().numpy(), gx.cpu().numpy()) <= 6e-2
    assert rel_l2(d1.weight.grad.double().cpu().numpy(), gw1.cpu().numpy()) <= 6e-2
    # (b) against FP64 arithmetic on the same BF16-rounded operands and activations (same masks):
    #     what the BF16 kernels add beyond BF16 storage must stay within 1e-2.
    bf = lambda t: t.bfloat16().double()
    pack, _ = grid.sparse_conv_kernel_map(3, 1)
    xq = x16.detach().double().requires_grad_(True)
    w1q = d1.weight.detach().double().requires_grad_(True)
    w2q = d2.weight.detach().double()
    pre = pack.sparse_conv_3d(xq, w1q).jdata
    y1 = bf(pre.detach())
    h = torch.relu(y1).requires_grad_(True)
    dh = torch.autograd.grad(pack.sparse_conv_3d(h, w2q).jdata, h, bf(dy))[0]
    dh = bf(dh) * (y1 > 0)
    dxq, dw1q = torch.autograd.grad(pre, (xq, w1q), dh)
    assert rel_l2(x16.grad.double().cpu().numpy(), bf(dxq).cpu().numpy()) <= 1e-2
    assert rel_l2(d1.weight.grad.double().cpu().numpy(), bf(dw1q).cpu().numpy()) <= 1e-2


def test_gradient_matches_reference_autograd(cuda_device):
    """One conv layer: GPU FP64 gradients equal the reference's gather-scatter backward
    (restated by the oracle) to 1e-12."""
    import fvdb

    grid = _grid(fvdb, cuda_device, 4000, 20, 5)
    pack, _ = grid.sparse_conv_kernel_map(3, 1)
    src = grid.ijk.jdata.cpu().numpy()
    kmap = orc.kernel_map(src, np.array([0, src.shape[0]]), src, np.array([0, src.shape[0]]), 3, 1)
    x = torch.randn(grid.total_voxels, 16, dtype=torch.float64)
    w = torch.randn(24, 16, 3, 3, 3, dtype=torch.float64)
    dy = torch.randn(grid.total_voxels, 24, dtype=torch.float64)
    xt, wt = x.to(cuda_device).requires_grad_(True), w.to(cuda_device).requires_grad_(True)
    pack.sparse_conv_3d(xt, wt).jdata.backward(dy.to(cuda_device))
    dx, dw = orc.conv_backward_f64(x.numpy(), w.numpy(), kmap, dy.numpy())
    assert rel_l2(xt.grad.cpu().numpy(), dx) < 1e-12
    assert rel_l2(wt.grad.cpu().numpy(), dw) < 1e-12


def test_recompute_matches_and_saves_memory(cuda_device):
    """RecomputeSequential: identical gradients, fewer bytes held between forward and backward."""
    import fvdb

    grid = _grid(fvdb, cuda_device, 60000, 64, 3)
    grads = []
    held = []
    for recompute in (False, True):
        net, c1, c2 = _stack(fvdb, cuda_device, torch.bfloat16, seed=1, recompute=recompute)
        deep = fvdb.nn.RecomputeSequential(*[net] * 4) if recompute else fvdb.nn.Sequential(*[net] * 4)
        x = torch.randn(grid.total_voxels, 64, device=cuda_device, generator=None).bfloat16()
        torch.manual_seed(9)
        x = torch.randn(grid.total_voxels, 64, device=cuda_device).bfloat16().requires_grad_(True)
        v = fvdb.nn.VDBTensor(grid, grid.jagged_like(x))
        # warm the kernel map cache so both runs hold the same maps
        out0 = net(v)
        torch.cuda.synchronize()
        base = torch.cuda.memory_allocated()
        out = deep(fvdb.nn.VDBTensor(grid, grid.jagged_like(x), out0.kmap))
        torch.cuda.synchronize()
        held.append(torch.cuda.memory_allocated() - base)
        out.data.jdata.float().sum().backward()
        grads.append((x.grad.float().cpu(), c1.weight.grad.float().cpu()))
        del out, out0, v
    assert torch.allclose(grads[0][0], grads[1][0], rtol=1e-2, atol=1e-2)
    assert torch.allclose(grads[0][1], grads[1][1], rtol=1e-2, atol=1e-2)
    assert held[1] < held[0]


def test_single_layer_bf16_forward_backward_within_1e2_of_fp64(cuda_device):
    """One SparseConv3d (3^3, 64->64) in BF16 -- forward, data gradient and weight gradient on
    tcgen05 -- against FP64 on the unrounded inputs: rel-L2 <= 1e-2 for y, dx and dW (the BF16
    rounding of inputs, weights and outputs is the whole error; no ReLU mask can flip)."""
    import fvdb

    from tests.synth import box_surfaces

    grid = fvdb.GridBatch.from_ijk(torch.from_numpy(box_surfaces(8, 96, 300)).to(cuda_device))
    pack, _ = grid.sparse_conv_kernel_map(3, 1)
    g = torch.Generator().manual_seed(301)
    x0 = torch.randn(grid.total_voxels, 64, generator=g, dtype=torch.float64)
    w0 = torch.randn(64, 64, 3, 3, 3, generator=g, dtype=torch.float64) * math.sqrt(2.0 / (27 * 64))
    dy = torch.randn(grid.total_voxels, 64, generator=g, dtype=torch.float64)
    res = {}
    for dtype in (torch.bfloat16, torch.float64):
        x = x0.to(cuda_device, dtype).requires_grad_(True)
        w = w0.to(cuda_device, dtype).requires_grad_(True)
        y = pack.sparse_conv_3d(x, w).jdata
        y.backward(dy.to(cuda_device, dtype))
        res[dtype] = (y.detach().double().cpu().numpy(), x.grad.double().cpu().numpy(), w.grad.double().cpu().numpy())
    torch.cuda.synchronize()
    fvdb._lib.load().check_device_errors(cuda_device)
    for got, ref in zip(res[torch.bfloat16], res[torch.float64]):
        assert rel_l2(got, ref) <= 1e-2
