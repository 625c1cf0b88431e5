"""FP8-E4M3 forward (tcgen05 kind::f8f6f4) parity.

Two checks per case:
  * kernel exactness -- against the FP64 oracle evaluated on the *dequantised* operands
    (e4m3(x/s_x)*s_x and e4m3(s_x W/s_w)*s_w); the only differences left are FP32
    accumulation order and the BF16 output rounding: rel-L2 <= 5e-3, max <= 1e-2 of scale;
  * quantisation error -- against the FP64 oracle on the original BF16 inputs, the bound a
    user sees: rel-L2 <= 8e-2 (E4M3 keeps 3 mantissa bits; ~5 % expected).
"""

import math

import numpy as np
import pytest
import torch

from oracle import oracle as orc
from tests.helpers import random_sparse_ijk

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def _q(t: torch.Tensor) -> torch.Tensor:
    return t.to(torch.float8_e4m3fn).to(torch.float64)


@pytest.mark.parametrize("cin,cout,ks,st,transposed", [(128, 256, 3, 1, False), (32, 64, 3, 1, False),
                                                        (256, 128, 2, 2, True), (64, 96, 2, 2, False)])
def test_fp8_forward(cuda_device, cin, cout, ks, st, transposed):
    import fvdb

    ijk = random_sparse_ijk(8000, 32, cin + cout)
    grid = fvdb.GridBatch.from_ijk(torch.from_numpy(ijk).to(cuda_device))
    pack, tgt = grid.sparse_conv_kernel_map(ks, st)
    src = grid.ijk.jdata.cpu().numpy()
    t = tgt.ijk.jdata.cpu().numpy()
    kmap = orc.kernel_map(src, np.array([0, src.shape[0]]), t, np.array([0, t.shape[0]]), ks, st)
    g = torch.Generator().manual_seed(cin)
    n_in = tgt.total_voxels if transposed else grid.total_voxels
    x = torch.randn(n_in, cin, generator=g).bfloat16()
    wshape = ((cin, cout) if transposed else (cout, cin)) + (ks,) * 3
    w = (torch.randn(wshape, generator=g) * math.sqrt(2.0 / (cin * ks**3))).bfloat16()
    C = fvdb._lib.load()
    y, s_x, s_w = C.conv_forward_fp8(x.to(cuda_device), w.to(cuda_device), pack._impl, transposed)
    torch.cuda.synchronize()
    C.check_device_errors(cuda_device)
    got = y.double().cpu().numpy()
    s_x, s_w = s_x.double().cpu(), s_w.double().cpu()
    # dequantised operands, replaying the kernel's arithmetic (x * (1/s_x) in FP32, RN-even to E4M3)
    inv = (1.0 / s_x.float()).double()
    xq = _q((x.float() * inv.float()).float()) * s_x
    wk = (w.permute(4, 3, 2, 0, 1) if transposed else w.permute(4, 3, 2, 1, 0)).reshape(-1, cin, cout).float()
    wf = wk * s_x.float().view(1, cin, 1)
    wq = _q(wf / s_w.float().view(1, 1, cout)) * s_w.view(1, 1, cout)
    kshape = (ks,) * 3
    wq5 = wq.reshape(kshape[2], kshape[1], kshape[0], cin, cout)
    wq5 = (wq5.permute(3, 4, 2, 1, 0) if transposed else wq5.permute(4, 3, 2, 1, 0)).numpy()
    # folding s_x into W: conv(xq / s_x * s_x, W) == conv(e4m3(x/s_x), e4m3(s_x W / s_w) s_w)
    x_unscaled = (xq / s_x).numpy()
    ref_q = orc.conv_forward_f64(x_unscaled, wq5, kmap, transposed=transposed, n_src=grid.total_voxels)
    assert rel_l2(got, ref_q) <= 5e-3
    assert np.abs(got - ref_q).max() <= 1e-2 * np.abs(ref_q).max()
    ref = orc.conv_forward_f64(x.double().numpy(), w.double().numpy(), kmap, transposed=transposed, n_src=grid.total_voxels)
    assert rel_l2(got, ref) <= 8e-2


def test_fp8_through_module_is_forward_only(cuda_device):
    import fvdb

    grid = fvdb.GridBatch.from_ijk(torch.from_numpy(random_sparse_ijk(3000, 24, 1)).to(cuda_device))
    conv = fvdb.nn.SparseConv3d(32, 64, 3, bias=False).to(cuda_device)
    conv.precision = "fp8"
    x = torch.randn(grid.total_voxels, 32, device=cuda_device)
    with torch.no_grad():
        y = conv(fvdb.nn.VDBTensor(grid, grid.jagged_like(x)))
    assert y.data.jdata.dtype == torch.bfloat16 and y.data.jdata.shape == (grid.total_voxels, 64)
    with pytest.raises(RuntimeError):
        conv(fvdb.nn.VDBTensor(grid, grid.jagged_like(x.requires_grad_(True))))
