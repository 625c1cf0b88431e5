"""The tile plan of the planned tensor-core convolution, and the convolution over it.

* The plan is an integer structure: decoding it (each tile's phases, their distinct source-row
  lists and the 16-bit local map) must give back the kernel map bit for bit, every phase must
  fit the staging buffer, and the tile's group mask must mark exactly the groups with a valid
  entry.
* Multi-phase tiles are forced with a lattice target grid (voxels three apart over a dense
  source box): every output row then reads 27 source rows no other row of its tile reads, so a
  tile's 3456 distinct rows are split into many phases.
* The planned convolution is checked against the FP64 oracle (tolerances written in each test)
  and, through the C ABI, against the unplanned kernel on the same map: both issue the same MMAs
  in the same order, so their outputs are bitwise equal.
"""

import ctypes
import math

import numpy as np
import pytest
import torch

from oracle import oracle as orc
from tests.helpers import dense_ijk, random_sparse_ijk

pytestmark = pytest.mark.gpu

HDR_WORDS = 68
STAGE_BYTES = 40 * 1024


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def plan_params(row_bytes):
    pack = 128 // row_bytes if row_bytes < 128 else 1
    cap = (STAGE_BYTES // (row_bytes + 16)) & ~31
    return pack, cap


def decode_plan(plan: np.ndarray, n_rows: int, K: int, row_bytes: int):
    """Kernel map rebuilt from the plan; also checks the per-phase invariants."""
    T = (n_rows + 127) // 128
    pack, cap = plan_params(row_bytes)
    G = (K + pack - 1) // pack
    lsz = T * 128 * K * 2
    lmap = plan[:lsz].view(np.uint16).reshape(T, 128, K)
    hdr = plan[lsz : lsz + T * HDR_WORDS * 4].view(np.int32).reshape(T, HDR_WORDS)
    src = plan[lsz + T * HDR_WORDS * 4 : lsz + T * HDR_WORDS * 4 + T * 128 * K * 4].view(np.int32).reshape(T, 128 * K)
    recon = np.full((T * 128, K), -1, dtype=np.int64)
    phases = []
    for t in range(T):
        gmask, nph = int(hdr[t, 0]) & 0xFFFFFFFF, int(hdr[t, 1])
        base, gb = 0, 0
        for p in range(nph):
            ge, cnt = int(hdr[t, 4 + 2 * p]), int(hdr[t, 5 + 2 * p])
            assert 0 <= cnt <= cap and gb <= ge <= G
            lst = src[t, base : base + cnt]
            assert np.unique(lst).size == cnt, "a phase lists a row twice"
            for k in range(gb * pack, min(K, ge * pack)):
                loc = lmap[t, :, k].astype(np.int64)
                ok = loc != 0xFFFF
                assert (loc[ok] < cnt).all()
                recon[t * 128 + np.nonzero(ok)[0], k] = lst[loc[ok]]
            base += cnt
            gb = ge
        assert gb == G
        phases.append(nph)
        rows = recon[t * 128 : t * 128 + 128]
        for g in range(G):
            active = bool((rows[:, g * pack : min(K, (g + 1) * pack)] >= 0).any())
            assert bool((gmask >> g) & 1) == active
    return recon[:n_rows], phases


def _lattice_case(dev, n=24, step=3):
    import fvdb

    src = fvdb.GridBatch.from_ijk(torch.from_numpy(dense_ijk((n, n, n))).to(dev))
    lat = dense_ijk((n // step,) * 3) * step + 1
    tgt = fvdb.GridBatch.from_ijk(torch.from_numpy(lat.astype(np.int32)).to(dev))
    pack, _ = src.sparse_conv_kernel_map(3, 1, target_grid=tgt)
    return src, tgt, pack


def _sparse_case(dev, n_vox, extent, seed):
    import fvdb

    grid = fvdb.GridBatch.from_ijk(torch.from_numpy(random_sparse_ijk(n_vox, extent, seed)).to(dev))
    pack, _ = grid.sparse_conv_kernel_map(3, 1)
    return grid, grid, pack


@pytest.mark.parametrize("row_bytes", [32, 64, 128, 192, 256])
@pytest.mark.parametrize("case", ["sparse", "lattice"])
def test_plan_rebuilds_kernel_map(cuda_device, row_bytes, case):
    if case == "sparse":
        src, tgt, pack = _sparse_case(cuda_device, 9000, 30, row_bytes)
    else:
        src, tgt, pack = _lattice_case(cuda_device)
    kmap = pack._impl.kmap()[: tgt.total_voxels].cpu().numpy()
    plan = pack._impl.tile_plan(False, row_bytes)
    torch.cuda.synchronize()
    recon, phases = decode_plan(plan.cpu().numpy(), tgt.total_voxels, kmap.shape[1], row_bytes)
    assert np.array_equal(recon, kmap)
    if case == "lattice":
        assert min(phases) > 1  # 27 private source rows per output row overflow every staging buffer
    # the transposed map's plan (data gradient) as well
    kt = pack._impl.kmap_t()[: src.total_voxels].cpu().numpy()
    recon_t, _ = decode_plan(pack._impl.tile_plan(True, row_bytes).cpu().numpy(), src.total_voxels, kt.shape[1], row_bytes)
    assert np.array_equal(recon_t, kt)


@pytest.mark.parametrize("cin,cout", [(16, 32), (32, 64), (64, 64), (96, 128), (128, 64)])
def test_planned_forward_multi_phase_bf16(cuda_device, cin, cout):
    """Lattice target (every tile split into phases): BF16 forward vs the FP64 oracle on the
    same bf16-rounded inputs, max error <= 1e-2 of the output scale and rel-L2 <= 5e-3."""
    import fvdb

    src, tgt, pack = _lattice_case(cuda_device)
    s = src.ijk.jdata.cpu().numpy()
    t = tgt.ijk.jdata.cpu().numpy()
    kmap = orc.kernel_map(s, np.array([0, s.shape[0]]), t, np.array([0, t.shape[0]]), 3, 1)
    g = torch.Generator().manual_seed(cin + cout)
    x = torch.randn(src.total_voxels, cin, generator=g).bfloat16()
    w = (torch.randn(cout, cin, 3, 3, 3, generator=g) * math.sqrt(2.0 / (27 * cin))).bfloat16()
    # the first contraction on the map runs in index order, the second over the map's (then
    # built) row order: both issue the same MMAs per row in the same order, so they agree bit for
    # bit; the planned kernel over this map is checked through the C ABI below
    y0 = pack.sparse_conv_3d(x.to(cuda_device), w.to(cuda_device)).jdata
    y = pack.sparse_conv_3d(x.to(cuda_device), w.to(cuda_device)).jdata
    torch.cuda.synchronize()
    fvdb._lib.load().check_device_errors(cuda_device)
    assert torch.equal(y0, y)
    if cin * 2 < 128:
        assert pack._impl.tile_plan(False, cin * 2) is not None
    ref = orc.conv_forward_f64(x.double().numpy(), w.double().numpy(), kmap)
    got = y.double().cpu().numpy()
    assert np.abs(got - ref).max() <= 1e-2 * np.abs(ref).max()
    assert rel_l2(got, ref) <= 5e-3


def test_planned_dgrad_multi_phase_bf16(cuda_device):
    """Data gradient over the transposed map, first in index order then over its row order (bitwise
    equal), lattice case: rel-L2 <= 1e-2 vs FP64."""
    src, tgt, pack = _lattice_case(cuda_device)
    s = src.ijk.jdata.cpu().numpy()
    t = tgt.ijk.jdata.cpu().numpy()
    kmap = orc.kernel_map(s, np.array([0, s.shape[0]]), t, np.array([0, t.shape[0]]), 3, 1)
    g = torch.Generator().manual_seed(3)
    x = torch.randn(src.total_voxels, 32, generator=g).bfloat16()
    w = (torch.randn(32, 32, 3, 3, 3, generator=g) * 0.05).bfloat16()
    dy = torch.randn(tgt.total_voxels, 32, generator=g).bfloat16()
    grads = []
    for _ in range(2):  # the second backward runs over the transposed map's row order
        xt = x.to(cuda_device).requires_grad_(True)
        y = pack.sparse_conv_3d(xt, w.to(cuda_device)).jdata
        y.backward(dy.to(cuda_device))
        grads.append(xt.grad)
    assert torch.equal(grads[0], grads[1])
    dx, _ = orc.conv_backward_f64(x.double().numpy(), w.double().numpy(), kmap, dy.double().numpy())
    assert rel_l2(grads[1].double().cpu().numpy(), dx) <= 1e-2


def test_planned_fp8_multi_phase(cuda_device):
    """FP8-E4M3 on the lattice map, index order then row order (bitwise equal): within the E4M3
    bound of the FP64 oracle (rel-L2 <= 8e-2)."""
    import fvdb

    src, tgt, pack = _lattice_case(cuda_device)
    s = src.ijk.jdata.cpu().numpy()
    t = tgt.ijk.jdata.cpu().numpy()
    kmap = orc.kernel_map(s, np.array([0, s.shape[0]]), t, np.array([0, t.shape[0]]), 3, 1)
    g = torch.Generator().manual_seed(8)
    x = torch.randn(src.total_voxels, 64, generator=g).bfloat16()
    w = (torch.randn(64, 64, 3, 3, 3, generator=g) * math.sqrt(2.0 / (27 * 64))).bfloat16()
    C = fvdb._lib.load()
    y0, _, _ = C.conv_forward_fp8(x.to(cuda_device), w.to(cuda_device), pack._impl, False)
    y, _, _ = C.conv_forward_fp8(x.to(cuda_device), w.to(cuda_device), pack._impl, False)  # over the row order
    torch.cuda.synchronize()
    assert torch.equal(y0, y)
    C.check_device_errors(cuda_device)
    ref = orc.conv_forward_f64(x.double().numpy(), w.double().numpy(), kmap)
    assert rel_l2(y.double().cpu().numpy(), ref) <= 8e-2


@pytest.mark.parametrize("case,cin,cout", [("sparse", 32, 64), ("lattice", 64, 32), ("sparse", 96, 128),
                                           ("lattice", 16, 32), ("lattice", 32, 64), ("lattice", 128, 64)])
def test_planned_through_c_abi_equals_unplanned(cuda_device, case, cin, cout):
    """fvgb_tc_plan_build + fvgb_conv_fwd_tc_planned with raw pointers: bitwise equal to
    fvgb_conv_fwd_tc_bias on the same map, weights and bias, and within 5e-3 rel-L2 of FP64."""
    from fvdb import _lib

    lib = _lib.cdll()
    if case == "sparse":
        src, tgt, pack = _sparse_case(cuda_device, 7000, 28, cin)
    else:
        src, tgt, pack = _lattice_case(cuda_device)
    kmap = pack._impl.kmap()
    n_in, n_out, K = src.total_voxels, tgt.total_voxels, kmap.shape[1]
    P = lambda t: ctypes.c_void_p(t.data_ptr())
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert lib.fvgb_tc_plan_supported(2, K, cin, cout) == 0
    nb = ctypes.c_size_t(0)
    assert lib.fvgb_tc_plan_bytes(ctypes.c_int64(n_out), K, cin * 2, ctypes.byref(nb)) == 0
    plan = torch.empty(nb.value, dtype=torch.uint8, device=cuda_device)
    assert lib.fvgb_tc_plan_build(P(kmap), ctypes.c_int64(n_out), K, cin * 2, P(plan), nb, stream) == 0
    x = torch.randn(n_in, cin, device=cuda_device).bfloat16()
    wkio = (torch.randn(K, cin, cout, device=cuda_device) * 0.05).bfloat16()
    bias = torch.randn(cout, device=cuda_device)
    wb = ctypes.c_size_t(0)
    assert lib.fvgb_tc_weight_bytes(2, ctypes.c_int64(K), cin, cout, ctypes.byref(wb)) == 0
    packed = torch.empty(wb.value, dtype=torch.uint8, device=cuda_device)
    assert lib.fvgb_tc_pack_weights(2, P(wkio), ctypes.c_int64(K), cin, cout, ctypes.c_int64(cin * cout),
                                    ctypes.c_int64(cout), ctypes.c_int64(1), P(packed), wb, stream) == 0
    err = torch.zeros(1, dtype=torch.int32, device=cuda_device)
    y1 = torch.empty(n_out, cout, device=cuda_device, dtype=torch.bfloat16)
    y2 = torch.empty_like(y1)
    assert lib.fvgb_conv_fwd_tc_planned(2, P(x), ctypes.c_int64(n_in), cin, ctypes.c_int64(cin), P(plan),
                                        ctypes.c_int64(n_out), K, P(packed), cout, P(y1), ctypes.c_int64(cout),
                                        None, P(bias), 0, P(err), stream) == 0
    assert lib.fvgb_conv_fwd_tc_bias(2, P(x), ctypes.c_int64(n_in), cin, ctypes.c_int64(cin), P(kmap),
                                     ctypes.c_int64(n_out), K, None, P(packed), cout, P(y2), ctypes.c_int64(cout),
                                     None, P(bias), P(err), stream) == 0
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    assert torch.equal(y1, y2)
    km = kmap[:n_out].cpu().numpy()
    w5 = wkio.double().cpu().numpy().reshape(3, 3, 3, cin, cout).transpose(4, 3, 2, 1, 0)
    ref = orc.conv_forward_f64(x.double().cpu().numpy(), w5, km) + bias.double().cpu().numpy()[None, :]
    assert rel_l2(y1.double().cpu().numpy(), ref) <= 5e-3
    # shapes the planned kernel does not take are rejected before any launch
    assert lib.fvgb_tc_plan_supported(2, K, cin, 256) == 1
    assert lib.fvgb_tc_plan_supported(2, 125, cin, cout) == 1
