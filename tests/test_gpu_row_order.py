"""Row order of the contractions: kernel-map rows sorted by occupancy mask so that a 128-row tile's
rows share their offsets (fvgb_kmap_row_order), and the forward kernels over that order
(fvgb_conv_fwd_tc_rows, fvgb_conv_fwd_simt_rows).

* The order is an integer structure: a permutation of the rows (padding -1), masks descending
  and stable among equal masks, per-tile masks equal to the OR of each ordered tile's row masks.
* The map in that order (sorted_map) holds the map's rows in that order, -1 rows for padding.
* A kernel over the order computes every output row with the same units in the same order as
  the kernel over the index order, so the outputs are bitwise equal (BF16 and FP8 tensor cores,
  FP32 and FP64 CUDA cores), and within the stated tolerance of the FP64 oracle.
"""

import ctypes

import numpy as np
import pytest
import torch

from oracle import oracle as orc
from tests.helpers import random_sparse_ijk

pytestmark = pytest.mark.gpu

P = lambda t: ctypes.c_void_p(t.data_ptr())


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def _case(dev, n_vox, extent, seed, ks=3, stride=1):
    import fvdb

    grid = fvdb.GridBatch.from_ijk(torch.from_numpy(random_sparse_ijk(n_vox, extent, seed)).to(dev))
    pack, tgt = grid.sparse_conv_kernel_map(ks, stride)
    return grid, tgt, pack


def _row_order(lib, kmap, n, K, dev):
    tiles = (n + 127) // 128
    rows = torch.empty(tiles * 128, dtype=torch.int32, device=dev)
    tmask = torch.zeros(tiles, dtype=torch.int32, device=dev)
    smap = torch.empty(tiles * 128, K, dtype=torch.int32, device=dev)
    wsb = ctypes.c_size_t(0)
    assert lib.fvgb_kmap_row_order_workspace(ctypes.c_int64(n), K, ctypes.byref(wsb)) == 0
    ws = torch.empty(wsb.value, dtype=torch.uint8, device=dev)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert lib.fvgb_kmap_row_order(P(kmap), ctypes.c_int64(n), K, ctypes.c_int64(kmap.stride(0)), P(rows), P(tmask),
                                   P(smap), P(ws), ctypes.c_size_t(ws.numel()), stream) == 0
    torch.cuda.synchronize()
    return rows, tmask, smap


@pytest.mark.parametrize("n_vox,extent,ks,stride", [(9000, 30, 3, 1), (5000, 20, 2, 2), (300, 12, 3, 1), (20000, 64, 3, 1)])
def test_row_order_is_a_sorted_permutation(cuda_device, n_vox, extent, ks, stride):
    from fvdb import _lib

    lib = _lib.cdll()
    _, tgt, pack = _case(cuda_device, n_vox, extent, 7, ks, stride)
    kmap = pack._impl.kmap()
    n, K = tgt.total_voxels, kmap.shape[1]
    rows, tmask, smap = _row_order(lib, kmap, n, K, cuda_device)
    r = rows.cpu().numpy()
    assert np.array_equal(np.sort(r[:n]), np.arange(n)) and np.all(r[n:] == -1)
    km = kmap[:n].cpu().numpy()
    mask = ((km >= 0).astype(np.int64) << np.arange(K, dtype=np.int64)).sum(1)
    ref = np.argsort(-mask, kind="stable")  # descending masks, equal masks in index order
    assert np.array_equal(r[:n], ref)
    sm = np.zeros(len(r), np.int64)
    sm[:n] = mask[r[:n]]
    tor = np.bitwise_or.reduce(sm.reshape(-1, 128), axis=1)
    assert np.array_equal(tmask.cpu().numpy().astype(np.int64) & ((1 << K) - 1), tor)
    sm_np = smap.cpu().numpy()
    assert np.array_equal(sm_np[:n], km[r[:n]]) and np.all(sm_np[n:] == -1)


@pytest.mark.parametrize("cin,cout,precision", [(32, 64, 2), (64, 64, 2), (128, 256, 2), (64, 128, 4), (32, 32, 4)])
def test_tensor_core_rows_equals_index_order(cuda_device, cin, cout, precision):
    """fvgb_conv_fwd_tc_rows over the row order == fvgb_conv_fwd_tc_epilogue over the index
    order, bitwise (BF16 = 2, E4M3 = 4), with bias and ReLU; BF16 within 5e-3 of FP64."""
    from fvdb import _lib

    lib = _lib.cdll()
    src, tgt, pack = _case(cuda_device, 9000, 28, cin + cout)
    kmap = pack._impl.kmap()
    tm = pack._impl.tile_mask(False)
    n_in, n_out, K = src.total_voxels, tgt.total_voxels, kmap.shape[1]
    rows, rmask, smap = _row_order(lib, kmap, n_out, K, cuda_device)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    g = torch.Generator().manual_seed(cin * 7 + cout)
    if precision == 2:
        x = torch.randn(n_in, cin, generator=g).bfloat16().to(cuda_device)
        wkio = (torch.randn(K, cin, cout, generator=g) * 0.05).bfloat16().to(cuda_device)
    else:
        x = torch.randn(n_in, cin, generator=g).clamp(-4, 4).to(cuda_device).to(torch.float8_e4m3fn).view(torch.uint8)
        wkio = (torch.randn(K, cin, cout, generator=g) * 0.5).to(cuda_device).to(torch.float8_e4m3fn).view(torch.uint8)
    bias = torch.randn(cout, generator=g).to(cuda_device)
    scale = (torch.rand(cout, generator=g) + 0.5).to(cuda_device)
    wb = ctypes.c_size_t(0)
    assert lib.fvgb_tc_weight_bytes(precision, ctypes.c_int64(K), cin, cout, ctypes.byref(wb)) == 0
    packed = torch.empty(wb.value, dtype=torch.uint8, device=cuda_device)
    assert lib.fvgb_tc_pack_weights(precision, P(wkio), ctypes.c_int64(K), cin, cout, ctypes.c_int64(cin * cout),
                                    ctypes.c_int64(cout), ctypes.c_int64(1), P(packed), wb, stream) == 0
    err = torch.zeros(1, dtype=torch.int32, device=cuda_device)
    y1 = torch.empty(n_out, cout, device=cuda_device, dtype=torch.bfloat16)
    y2 = torch.empty_like(y1)
    sc = P(scale) if precision == 4 else None
    for relu in (0, 1):
        assert lib.fvgb_conv_fwd_tc_rows(precision, P(x), ctypes.c_int64(n_in), cin, ctypes.c_int64(cin), P(smap),
                                         ctypes.c_int64(n_out), K, P(rows), P(rmask), P(packed), cout, P(y1),
                                         ctypes.c_int64(cout), sc, P(bias), relu, P(err), stream) == 0
        assert lib.fvgb_conv_fwd_tc_epilogue(precision, P(x), ctypes.c_int64(n_in), cin, ctypes.c_int64(cin),
                                             P(kmap), ctypes.c_int64(n_out), K, P(tm) if tm is not None else None, P(packed), cout, P(y2),
                                             ctypes.c_int64(cout), sc, P(bias), relu, P(err), stream) == 0
        torch.cuda.synchronize()
        assert int(err.item()) == 0
        assert torch.equal(y1, y2)
    if precision == 2:
        km = kmap[:n_out].cpu().numpy()
        w5 = wkio.double().cpu().numpy().reshape(3, 3, 3, cin, cout).transpose(4, 3, 2, 1, 0)
        ref = np.maximum(orc.conv_forward_f64(x.double().cpu().numpy(), w5, km) + bias.double().cpu().numpy()[None], 0)
        assert rel_l2(y1.double().cpu().numpy(), ref) <= 5e-3


@pytest.mark.parametrize("dtype,code", [(torch.float32, 0), (torch.float64, 1)])
def test_simt_rows_equals_index_order(cuda_device, dtype, code):
    from fvdb import _lib

    lib = _lib.cdll()
    src, tgt, pack = _case(cuda_device, 7000, 26, 3)
    kmap = pack._impl.kmap()
    n_in, n_out, K = src.total_voxels, tgt.total_voxels, kmap.shape[1]
    rows, _, smap = _row_order(lib, kmap, n_out, K, cuda_device)
    g = torch.Generator().manual_seed(11)
    cin, cout = 24, 40
    x = torch.randn(n_in, cin, generator=g, dtype=dtype).to(cuda_device)
    w = torch.randn(K, cin, cout, generator=g, dtype=dtype).to(cuda_device)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    y1 = torch.empty(n_out, cout, device=cuda_device, dtype=dtype)
    y2 = torch.empty_like(y1)
    args = lambda m: (code, P(x), ctypes.c_int64(n_in), cin, ctypes.c_int64(cin), P(m), ctypes.c_int64(n_out),
                      K, ctypes.c_int64(K))
    assert lib.fvgb_conv_fwd_simt_rows(*args(smap), P(rows), P(w), ctypes.c_int64(cin * cout), ctypes.c_int64(cout),
                                       ctypes.c_int64(1), P(y1), cout, ctypes.c_int64(cout), 0, stream) == 0
    assert lib.fvgb_conv_fwd_simt(*args(kmap), P(w), ctypes.c_int64(cin * cout), ctypes.c_int64(cout),
                                  ctypes.c_int64(1), P(y2), cout, ctypes.c_int64(cout), 0, stream) == 0
    torch.cuda.synchronize()
    assert torch.equal(y1, y2)
    km = kmap[:n_out].cpu().numpy()
    w5 = w.double().cpu().numpy().reshape(3, 3, 3, cin, cout).transpose(4, 3, 2, 1, 0)
    ref = orc.conv_forward_f64(x.double().cpu().numpy(), w5, km)
    assert rel_l2(y1.double().cpu().numpy(), ref) <= (1e-6 if dtype == torch.float32 else 1e-13)
