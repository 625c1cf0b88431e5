"""GPU parity of the contractions (FP32 plain form, FP64 form, 16-bit features) against the
oracle, the golden fixtures and torch dense convolutions, plus the reference's error-input
contract (tests/unit/test_conv.py:677-716)."""

import math

import numpy as np
import pytest
import torch

from oracle import oracle as orc
from tests.helpers import golden_cases, kernel_start, load_golden, random_sparse_ijk, rows_by_coord

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def fvdb(cuda_device):
    import fvdb as m

    return m


def rel_max(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def test_config1_plain_fp32(fvdb, cuda_device):
    """20,000 unique voxels uniform in [0,64)^3, C 16->16, 3x3x3, stride 1, FP32, no bias:
    kernel map bit-exact; output within 1e-5 relative of the reference CPU path."""
    g = torch.Generator().manual_seed(0)
    idx = torch.randperm(64**3, generator=g)[:20000]
    ijk = torch.stack([idx // 4096, (idx // 64) % 64, idx % 64], 1).to(torch.int32)
    x = torch.randn(20000, 16, generator=g)
    w = torch.randn(16, 16, 3, 3, 3, generator=g) * math.sqrt(1.0 / (27 * 16))
    grid = fvdb.GridBatch.from_ijk(ijk.to(cuda_device))
    pack, tgt = grid.sparse_conv_kernel_map(3, 1)
    pack.build_gather_scatter()
    o_ijk, o_off = orc.grid_from_ijk(ijk.numpy(), np.array([0, 20000]))
    perm = [rows_by_coord(ijk.numpy())[tuple(r)] for r in o_ijk.tolist()]
    xs = x[perm]
    out = pack.sparse_conv_3d(xs.to(cuda_device), w.to(cuda_device), fvdb.ConvPackBackend.GATHER_SCATTER).jdata
    kmap = orc.kernel_map(o_ijk, o_off, o_ijk, o_off, 3, 1)
    assert np.array_equal(pack.out_in_map[:20000].cpu().numpy(), kmap)
    nbmap, nbsizes = orc.neighbour_map(kmap)
    ref_cpu = orc.gs_forward(xs, w, nbmap, nbsizes, 20000, middle=True).numpy()
    got = out.cpu().numpy()
    assert rel_max(got, ref_cpu) < 1e-5
    assert rel_max(got, orc.conv_forward_f64(xs.numpy(), w.numpy(), kmap)) < 1e-5


@pytest.mark.parametrize("name", golden_cases("sparse_"))
@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_golden_forward(fvdb, cuda_device, name, dtype):
    g = load_golden(name)
    ks, st = tuple(g["kernel_size"].tolist()), tuple(g["stride"].tolist())
    grid = fvdb.GridBatch.from_ijk(torch.from_numpy(g["ijk"]).to(cuda_device))
    pack, tgt = grid.sparse_conv_kernel_map(ks, st)
    perm = [rows_by_coord(g["ijk"])[tuple(r)] for r in grid.ijk.jdata.cpu().numpy().tolist()]
    x = torch.from_numpy(g["features"][perm]).to(cuda_device, dtype)
    w = torch.from_numpy(g["weights"]).to(cuda_device, dtype)
    out = pack.sparse_conv_3d(x, w).jdata.double().cpu().numpy()
    order = [rows_by_coord(tgt.ijk.jdata.cpu().numpy())[tuple(r)] for r in g["target_ijk"].tolist()]
    tol = 1e-12 if dtype == torch.float64 else 1e-5
    assert rel_max(out[order], g["expected"]) < tol


@pytest.mark.parametrize("name", golden_cases("dense_transposed"))
def test_golden_transposed(fvdb, cuda_device, name):
    g = load_golden(name)
    ks = tuple(g["kernel_size"].tolist())
    grid = fvdb.GridBatch.from_ijk(torch.from_numpy(g["ijk"]).to(cuda_device))
    pack, tgt = grid.sparse_conv_kernel_map(ks, 1)
    perm = [rows_by_coord(g["ijk"])[tuple(r)] for r in grid.ijk.jdata.cpu().numpy().tolist()]
    x = torch.from_numpy(g["features"][perm]).to(cuda_device)
    w = torch.from_numpy(g["weights"]).to(cuda_device)
    out = pack.sparse_transpose_conv_3d(x, w).jdata.cpu().numpy()
    assert rel_max(out, g["expected"][perm]) < 1e-12


@pytest.mark.parametrize("name", golden_cases("strided_transposed"))
@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_golden_strided_transposed(fvdb, cuda_device, name, dtype):
    """Coarse features onto the fine grid (sparse_transpose_conv_3d over the fine -> coarse map)
    against torch's dense conv_transpose3d."""
    g = load_golden(name)
    ks, st = tuple(g["kernel_size"].tolist()), tuple(g["stride"].tolist())
    grid = fvdb.GridBatch.from_ijk(torch.from_numpy(g["ijk"]).to(cuda_device))
    pack, tgt = grid.sparse_conv_kernel_map(ks, st)
    t_rows = rows_by_coord(g["target_ijk"])
    xt = g["features"][[t_rows[tuple(r)] for r in tgt.ijk.jdata.cpu().numpy().tolist()]]
    x = torch.from_numpy(xt).to(cuda_device, dtype)
    w = torch.from_numpy(g["weights"]).to(cuda_device, dtype)
    out = pack.sparse_transpose_conv_3d(x, w).jdata.double().cpu().numpy()
    perm = [rows_by_coord(g["ijk"])[tuple(r)] for r in grid.ijk.jdata.cpu().numpy().tolist()]
    tol = 1e-12 if dtype == torch.float64 else 1e-5
    assert rel_max(out, g["expected"][perm]) < tol


CASES = [((3, 3, 3), (1, 1, 1), 16, 32), ((2, 2, 2), (2, 2, 2), 32, 16), ((3, 3, 3), (2, 2, 2), 8, 24),
         ((5, 3, 1), (1, 3, 2), 4, 8), ((3, 3, 3), (1, 1, 1), 70, 130)]


@pytest.mark.parametrize("ks,st,cin,cout", CASES)
@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
@pytest.mark.parametrize("transposed", [False, True])
def test_forward_backward_vs_oracle(fvdb, cuda_device, ks, st, cin, cout, dtype, transposed):
    parts = [random_sparse_ijk(2500, 20, 41, lo=-4), random_sparse_ijk(900, 14, 42, lo=30)]
    ijk = np.concatenate(parts, 0)
    off = np.array([0, 2500, 3400])
    jt = fvdb.JaggedTensor.from_data_and_offsets(torch.from_numpy(ijk).to(cuda_device), torch.from_numpy(off).to(cuda_device))
    grid = fvdb.GridBatch.from_ijk(jt)
    pack, tgt = grid.sparse_conv_kernel_map(ks, st)
    src, soff = orc.grid_from_ijk(ijk, off)
    t_ijk, toff = (src, soff) if st == (1, 1, 1) else orc.conv_grid(src, soff, ks, st)
    kmap = orc.kernel_map(src, soff, t_ijk, toff, ks, st)
    rng = np.random.default_rng(7)
    n_in = t_ijk.shape[0] if transposed else src.shape[0]
    x = rng.standard_normal((n_in, cin))
    w = rng.standard_normal(((cin, cout) if transposed else (cout, cin)) + ks) / math.sqrt(cin * np.prod(ks))
    xt = torch.from_numpy(x).to(cuda_device, dtype).requires_grad_(True)
    wt = torch.from_numpy(w).to(cuda_device, dtype).requires_grad_(True)
    if transposed:
        y = pack.sparse_transpose_conv_3d(xt, wt).jdata
    else:
        y = pack.sparse_conv_3d(xt, wt).jdata
    ref = orc.conv_forward_f64(x, w, kmap, transposed=transposed, n_src=src.shape[0])
    tol = 1e-12 if dtype == torch.float64 else 2e-5
    assert rel_max(y.detach().double().cpu().numpy(), ref) < tol
    dy = rng.standard_normal(ref.shape)
    y.backward(torch.from_numpy(dy).to(cuda_device, dtype))
    dx, dw = orc.conv_backward_f64(x, w, kmap, dy, transposed=transposed, n_src=src.shape[0])
    assert rel_max(xt.grad.double().cpu().numpy(), dx) < tol
    assert rel_max(wt.grad.double().cpu().numpy(), dw) < tol
    assert wt.grad.shape == wt.shape


@pytest.mark.parametrize("k", [2, 3, 4, 5, 6])
@pytest.mark.parametrize("stride", [1, 2, 4])
def test_dense_box_vs_conv3d(fvdb, cuda_device, k, stride):
    """test_torch_sparse_conv (test_conv.py:361-461) re-hosted: from_dense box vs F.conv3d."""
    n = 16
    grid = fvdb.GridBatch.from_dense(1, (n, n, n), device=cuda_device)
    torch.manual_seed(0)
    x = torch.randn(grid.total_voxels, 4, dtype=torch.float64, device=cuda_device)
    w = torch.randn(8, 4, k, k, k, dtype=torch.float64, device=cuda_device)
    pack, tgt = grid.sparse_conv_kernel_map(k, stride)
    out = pack.sparse_conv_3d(x, w).jdata
    dense = grid.write_to_dense_xyzc(x).squeeze(0).permute(3, 2, 1, 0)
    p = -kernel_start(k)
    shift = 4  # targets at -1 (k=5, s=2): evaluate on a box shifted by a multiple of the stride
    dpad = torch.nn.functional.pad(dense, (shift, k + stride, shift, k + stride, shift, k + stride))
    ref = torch.nn.functional.conv3d(dpad[None], w, padding=p, stride=stride)[0]
    t = tgt.ijk.jdata.long() + shift // stride
    ref_rows = ref[:, t[:, 2], t[:, 1], t[:, 0]].T
    assert torch.allclose(out, ref_rows, rtol=1e-12, atol=1e-12)


def test_bf16_features_within_tolerance(fvdb, cuda_device):
    grid = fvdb.GridBatch.from_ijk(torch.from_numpy(random_sparse_ijk(20000, 48, 3)).to(cuda_device))
    pack, _ = grid.sparse_conv_kernel_map(3, 1)
    torch.manual_seed(1)
    x = torch.randn(grid.total_voxels, 32, device=cuda_device)
    w = torch.randn(64, 32, 3, 3, 3, device=cuda_device) * math.sqrt(2.0 / (27 * 32))
    y = pack.sparse_conv_3d(x.bfloat16(), w.bfloat16()).jdata
    assert y.dtype == torch.bfloat16
    src = grid.ijk.jdata.cpu().numpy()
    kmap = orc.kernel_map(src, np.array([0, src.shape[0]]), src, np.array([0, src.shape[0]]), 3, 1)
    ref = orc.conv_forward_f64(x.bfloat16().double().cpu().numpy(), w.bfloat16().double().cpu().numpy(), kmap)
    assert rel_l2(y.double().cpu().numpy(), ref) < 1e-2


def test_module_forward_backward_and_kmap_cache(fvdb, cuda_device):
    grid = fvdb.GridBatch.from_ijk(torch.from_numpy(random_sparse_ijk(3000, 20, 8)).to(cuda_device))
    conv1 = fvdb.nn.SparseConv3d(8, 16, 3).to(cuda_device)
    conv2 = fvdb.nn.SparseConv3d(16, 8, 3).to(cuda_device)
    x = torch.randn(grid.total_voxels, 8, device=cuda_device, requires_grad=True)
    v = fvdb.nn.VDBTensor(grid, grid.jagged_like(x))
    h = conv1(v)
    assert h.kmap is not None and h.grid.is_same(grid)
    y = conv2(fvdb.nn.ReLU()(h))
    assert y.kmap is h.kmap  # the stride-1 map is reused, not rebuilt
    y.data.jdata.sum().backward()
    assert x.grad is not None and conv1.weight.grad is not None and conv1.bias.grad is not None
    down = fvdb.nn.SparseConv3d(8, 8, 2, stride=2).to(cuda_device)(v)
    assert down.grid.total_voxels < grid.total_voxels and down.kmap is None
    up = fvdb.nn.SparseConv3d(8, 8, 2, stride=2, transposed=True).to(cuda_device)(down, out_grid=grid)
    assert up.grid.is_same(grid) and up.data.jdata.shape == (grid.total_voxels, 8)


@pytest.mark.parametrize("transposed", [False, True])
def test_error_inputs(fvdb, cuda_device, transposed):
    """test_error_inputs (test_conv.py:677-716): bad shapes raise ValueError."""
    torch.manual_seed(0)
    grid = fvdb.GridBatch.from_points(torch.randn(1000, 3, device=cuda_device), voxel_sizes=0.025, origins=[0.0, 0.0, 0.0])
    n = grid.total_voxels

    def do(feats, kernels):
        pack, _ = grid.sparse_conv_kernel_map(kernels.shape[-1], 1)
        pack.build_gather_scatter()
        f = pack.sparse_transpose_conv_3d if transposed else pack.sparse_conv_3d
        return f(feats, kernels)

    with pytest.raises(ValueError):
        do(torch.randn(n, device=cuda_device), torch.rand(8, 0, 5, 5, 5, device=cuda_device))
    with pytest.raises(ValueError):
        do(torch.randn(n, 5, device=cuda_device), torch.rand(8, 4, 5, 5, 5, device=cuda_device))
    with pytest.raises(ValueError):
        do(torch.randn(n + 7, 4, device=cuda_device), torch.rand(8, 4, 5, 5, 5, device=cuda_device))
    with pytest.raises(TypeError):
        do(torch.randint(0, 3, (n, 4), device=cuda_device), torch.rand(4, 4, 5, 5, 5, device=cuda_device))


def test_empty_target_gives_empty_output(fvdb, cuda_device):
    """test_basic_ops.py:1695-1711: an empty target grid gives an empty output with the channel count."""
    grid = fvdb.GridBatch.from_ijk(torch.from_numpy(random_sparse_ijk(100, 8, 0)).to(cuda_device))
    empty = fvdb.GridBatch.from_ijk(torch.zeros((0, 3), dtype=torch.int32, device=cuda_device))
    pack, _ = grid.sparse_conv_kernel_map(3, 1, empty)
    out = pack.sparse_conv_3d(torch.randn(grid.total_voxels, 4, device=cuda_device), torch.randn(6, 4, 3, 3, 3, device=cuda_device))
    assert out.jdata.shape == (0, 6)


# ----------------------------------------------------------------- tensor cores (BF16) ---
def _bf16_case(fvdb, dev, n, extent, seed, ks=(3, 3, 3), st=(1, 1, 1)):
    ijk = random_sparse_ijk(n, extent, seed)
    grid = fvdb.GridBatch.from_ijk(torch.from_numpy(ijk).to(dev))
    pack, tgt = grid.sparse_conv_kernel_map(ks, st)
    src = grid.ijk.jdata.cpu().numpy()
    t = tgt.ijk.jdata.cpu().numpy()
    kmap = orc.kernel_map(src, np.array([0, src.shape[0]]), t, np.array([0, t.shape[0]]), ks, st)
    return grid, pack, tgt, kmap


@pytest.mark.parametrize(
    "cin,cout,ks,st",
    [(16, 16, (3, 3, 3), (1, 1, 1)), (32, 64, (3, 3, 3), (1, 1, 1)), (64, 64, (3, 3, 3), (1, 1, 1)),
     (96, 48, (3, 3, 3), (1, 1, 1)), (128, 256, (3, 3, 3), (1, 1, 1)), (256, 128, (2, 2, 2), (2, 2, 2)),
     (64, 200, (2, 2, 2), (2, 2, 2)), (32, 32, (5, 5, 5), (1, 1, 1)), (48, 80, (3, 1, 3), (1, 1, 1))],
)
def test_tensor_core_forward_bf16(fvdb, cuda_device, cin, cout, ks, st):
    """tcgen05 forward vs the FP64 oracle on bf16-rounded inputs (tolerances written here:
    max error <= 1e-2 of the output scale and rel-L2 <= 5e-3; bf16 output rounding is 2^-9)."""
    grid, pack, tgt, kmap = _bf16_case(fvdb, cuda_device, 7000, 30, cin + cout, ks=ks, st=st)
    g = torch.Generator().manual_seed(cin * 7 + cout)
    x = torch.randn(grid.total_voxels, cin, generator=g).bfloat16()
    w = (torch.randn((cout, cin) + ks, generator=g) * math.sqrt(2.0 / (cin * np.prod(ks)))).bfloat16()
    y = pack.sparse_conv_3d(x.to(cuda_device), w.to(cuda_device)).jdata
    torch.cuda.synchronize()
    fvdb._lib.load().check_device_errors(cuda_device)
    ref = orc.conv_forward_f64(x.double().numpy(), w.double().numpy(), kmap)
    got = y.double().cpu().numpy()
    assert np.abs(got - ref).max() <= 1e-2 * np.abs(ref).max()
    assert rel_l2(got, ref) <= 5e-3


def test_tensor_core_training_bf16(fvdb, cuda_device):
    """BF16 forward (tcgen05), dgrad (tcgen05 over the transposed map), wgrad (FP32 partials +
    FP64 reduction) against the FP64 oracle: rel-L2 <= 1e-2 each."""
    grid, pack, tgt, kmap = _bf16_case(fvdb, cuda_device, 9000, 32, 5)
    g = torch.Generator().manual_seed(5)
    x = torch.randn(grid.total_voxels, 64, generator=g).bfloat16()
    w = (torch.randn(64, 64, 3, 3, 3, generator=g) * math.sqrt(2.0 / (64 * 27))).bfloat16()
    dy = torch.randn(grid.total_voxels, 64, generator=g).bfloat16()
    xt = x.to(cuda_device).requires_grad_(True)
    wt = w.to(cuda_device).requires_grad_(True)
    y = pack.sparse_conv_3d(xt, wt).jdata
    y.backward(dy.to(cuda_device))
    ref = orc.conv_forward_f64(x.double().numpy(), w.double().numpy(), kmap)
    dx, dw = orc.conv_backward_f64(x.double().numpy(), w.double().numpy(), kmap, dy.double().numpy())
    assert rel_l2(y.detach().double().cpu().numpy(), ref) <= 1e-2
    assert rel_l2(xt.grad.double().cpu().numpy(), dx) <= 1e-2
    assert rel_l2(wt.grad.double().cpu().numpy(), dw) <= 1e-2


def test_tensor_core_transposed_bf16(fvdb, cuda_device):
    grid, pack, tgt, kmap = _bf16_case(fvdb, cuda_device, 6000, 28, 9, ks=(2, 2, 2), st=(2, 2, 2))
    g = torch.Generator().manual_seed(9)
    x = torch.randn(tgt.total_voxels, 128, generator=g).bfloat16()
    w = (torch.randn(128, 64, 2, 2, 2, generator=g) * math.sqrt(2.0 / (128 * 8))).bfloat16()
    y = pack.sparse_transpose_conv_3d(x.to(cuda_device), w.to(cuda_device)).jdata
    ref = orc.conv_forward_f64(x.double().numpy(), w.double().numpy(), kmap, transposed=True, n_src=grid.total_voxels)
    assert rel_l2(y.double().cpu().numpy(), ref) <= 5e-3


def test_tensor_core_through_c_abi(fvdb, cuda_device):
    """fvgb_tc_pack_weights + fvgb_conv_fwd_tc called with raw pointers."""
    import ctypes

    from fvdb import _lib

    lib = _lib.cdll()
    grid, pack, tgt, kmap = _bf16_case(fvdb, cuda_device, 4000, 24, 77)
    n, cin, cout, K = grid.total_voxels, 32, 64, 27
    x = torch.randn(n, cin, device=cuda_device).bfloat16()
    wkio = (torch.randn(K, cin, cout, device=cuda_device) * 0.05).bfloat16()
    npad = (n + 127) // 128 * 128  # the reference's out_in_map layout: rows padded to 128 with -1
    m = torch.full((npad, K), -1, dtype=torch.int32)
    m[:n] = torch.from_numpy(kmap)
    m = m.to(cuda_device)
    nbytes = ctypes.c_size_t(0)
    assert lib.fvgb_tc_weight_bytes(2, ctypes.c_int64(K), cin, cout, ctypes.byref(nbytes)) == 0
    packed = torch.empty(nbytes.value, dtype=torch.uint8, device=cuda_device)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert lib.fvgb_tc_pack_weights(2, ctypes.c_void_p(wkio.data_ptr()), ctypes.c_int64(K), cin, cout,
                                    ctypes.c_int64(cin * cout), ctypes.c_int64(cout), ctypes.c_int64(1),
                                    ctypes.c_void_p(packed.data_ptr()), nbytes, stream) == 0
    y = torch.empty(n, cout, device=cuda_device, dtype=torch.bfloat16)
    err = torch.zeros(1, dtype=torch.int32, device=cuda_device)
    rc = lib.fvgb_conv_fwd_tc(2, ctypes.c_void_p(x.data_ptr()), ctypes.c_int64(n), cin, ctypes.c_int64(cin),
                              ctypes.c_void_p(m.data_ptr()), ctypes.c_int64(n), K, None,
                              ctypes.c_void_p(packed.data_ptr()), cout, ctypes.c_void_p(y.data_ptr()),
                              ctypes.c_int64(cout), None, ctypes.c_void_p(err.data_ptr()), stream)
    assert rc == 0
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    w5 = wkio.double().cpu().numpy().reshape(3, 3, 3, cin, cout).transpose(4, 3, 2, 1, 0)
    ref = orc.conv_forward_f64(x.double().cpu().numpy(), w5, kmap)
    assert rel_l2(y.double().cpu().numpy(), ref) <= 5e-3
    # channel counts the kernel does not take are rejected before launch
    assert lib.fvgb_conv_fwd_tc(2, ctypes.c_void_p(x.data_ptr()), ctypes.c_int64(n), 24, ctypes.c_int64(24),
                                ctypes.c_void_p(m.data_ptr()), ctypes.c_int64(n), K, None,
                                ctypes.c_void_p(packed.data_ptr()), cout, ctypes.c_void_p(y.data_ptr()),
                                ctypes.c_int64(cout), None, ctypes.c_void_p(err.data_ptr()), stream) == 1


@pytest.mark.parametrize("dtype", [torch.bfloat16, torch.float32])
def test_weight_cache_follows_in_place_updates(cuda_device, dtype):
    """The host caches the [K, Cin, Cout] layout and the packed tensor-core image per weight
    tensor (storage + version): an in-place update of the weights (an optimizer step) must give
    the new result, and a new weight tensor at a reused address must not see the old image."""
    import fvdb

    torch.manual_seed(5)
    grid = fvdb.GridBatch.from_ijk(torch.from_numpy(random_sparse_ijk(5000, 24, 4)).to(cuda_device))
    pack, _ = grid.sparse_conv_kernel_map(3, 1)
    x = torch.randn(grid.total_voxels, 32, device=cuda_device, dtype=dtype)
    w = torch.randn(64, 32, 3, 3, 3, device=cuda_device, dtype=dtype) * 0.1
    y0 = pack.sparse_conv_3d(x, w).jdata.clone()
    with torch.no_grad():
        w.mul_(-2.0)  # in place: same storage, new version
    y1 = pack.sparse_conv_3d(x, w).jdata
    torch.testing.assert_close(y1.float(), (-2.0 * y0.float()), rtol=2e-2 if dtype == torch.bfloat16 else 1e-5,
                               atol=2e-2 if dtype == torch.bfloat16 else 1e-5)
    # a fresh computation on a copy (no cache entry) agrees exactly with the cached path
    y2 = pack.sparse_conv_3d(x, w.clone()).jdata
    assert torch.equal(y1, y2)
    # free the weights and allocate new ones of the same shape (likely the same address)
    del w
    w3 = torch.randn(64, 32, 3, 3, 3, device=cuda_device, dtype=dtype) * 0.1
    y3 = pack.sparse_conv_3d(x, w3).jdata
    y4 = pack.sparse_conv_3d(x, w3.clone()).jdata
    assert torch.equal(y3, y4)
