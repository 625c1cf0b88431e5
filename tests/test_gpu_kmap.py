"""GPU parity of the integer path: grid index order, conv_grid, kernel map, transposed map,
gather-scatter neighbour map -- all bit-exact against the oracle."""

import ctypes

import numpy as np
import pytest
import torch

from oracle import oracle as orc
from tests.helpers import golden_cases, kmap_to_coords, load_golden, random_sparse_ijk, rows_by_coord

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def fvdb(cuda_device):
    import fvdb as m

    return m


def _grid(fvdb, parts, dev):
    ijk = np.concatenate(parts, 0) if parts else np.zeros((0, 3), np.int32)
    off = np.cumsum([0] + [p.shape[0] for p in parts])
    jt = fvdb.JaggedTensor.from_data_and_offsets(torch.from_numpy(ijk).to(dev), torch.from_numpy(off).to(dev))
    return fvdb.GridBatch.from_ijk(jt), ijk, off


@pytest.mark.parametrize(
    "parts",
    [
        [random_sparse_ijk(5000, 40, 0)],
        [random_sparse_ijk(3000, 40, 1, lo=-20), random_sparse_ijk(2000, 30, 2, lo=4080)],
        [random_sparse_ijk(100, 8, 3), np.zeros((0, 3), np.int32), random_sparse_ijk(700, 20, 4, lo=-9000)],
    ],
)
def test_grid_order_bit_exact(fvdb, cuda_device, parts):
    parts = [np.concatenate([p, p[::5]], 0) if p.shape[0] else p for p in parts]  # with duplicates
    grid, ijk, off = _grid(fvdb, parts, cuda_device)
    o_ijk, o_off = orc.grid_from_ijk(ijk, off)
    assert grid.joffsets.cpu().tolist() == o_off.tolist()
    assert np.array_equal(grid.ijk.jdata.cpu().numpy(), o_ijk)
    assert np.array_equal(grid.jidx.cpu().numpy(), np.repeat(np.arange(len(parts)), np.diff(o_off)).astype(np.int32))


KS_ST = [
    ((3, 3, 3), (1, 1, 1)),
    ((2, 2, 2), (2, 2, 2)),
    ((3, 3, 3), (2, 2, 2)),
    ((5, 5, 5), (1, 1, 1)),
    ((4, 4, 4), (1, 1, 1)),
    ((5, 3, 1), (1, 3, 2)),
    ((4, 1, 4), (1, 2, 1)),
    ((7, 7, 7), (4, 4, 4)),
    ((3, 3, 3), (8, 8, 8)),  # window of source leaves too large to stage: hash path
]


@pytest.mark.parametrize("ks,st", KS_ST)
def test_kernel_map_bit_exact(fvdb, cuda_device, ks, st):
    parts = [random_sparse_ijk(4000, 36, 11, lo=-10), random_sparse_ijk(1500, 24, 12, lo=500)]
    grid, ijk, off = _grid(fvdb, parts, cuda_device)
    pack, tgt_grid = grid.sparse_conv_kernel_map(ks, st)
    pack.build_implicit_gemm(sorted=False, training=True)
    src, soff = orc.grid_from_ijk(ijk, off)
    tgt, toff = (src, soff) if st == (1, 1, 1) else orc.conv_grid(src, soff, ks, st)
    assert np.array_equal(tgt_grid.ijk.jdata.cpu().numpy(), tgt)
    assert tgt_grid.joffsets.cpu().tolist() == toff.tolist()
    o_kmap = orc.kernel_map(src, soff, tgt, toff, ks, st)
    kmap = pack.out_in_map.cpu().numpy()
    npad = (tgt.shape[0] + 127) // 128 * 128
    assert kmap.shape == (npad, o_kmap.shape[1])
    assert np.array_equal(kmap[: tgt.shape[0]], o_kmap)
    assert (kmap[tgt.shape[0] :] == -1).all()
    kmap_t = pack.out_in_map_bwd.cpu().numpy()
    assert np.array_equal(kmap_t[: src.shape[0]], orc.transpose_map(o_kmap, src.shape[0]))
    assert (kmap_t[src.shape[0] :] == -1).all()


@pytest.mark.parametrize("ks,st", [((3, 3, 3), (1, 1, 1)), ((2, 2, 2), (2, 2, 2))])
def test_neighbour_map_bit_exact(fvdb, cuda_device, ks, st):
    grid, ijk, off = _grid(fvdb, [random_sparse_ijk(6000, 32, 21)], cuda_device)
    pack, tgt_grid = grid.sparse_conv_kernel_map(ks, st)
    pack.build_gather_scatter()
    src, soff = orc.grid_from_ijk(ijk, off)
    tgt, toff = (src, soff) if st == (1, 1, 1) else orc.conv_grid(src, soff, ks, st)
    nbmap, nbsizes = orc.neighbour_map(orc.kernel_map(src, soff, tgt, toff, ks, st))
    assert np.array_equal(pack.neighborhood_map.cpu().numpy(), nbmap)
    assert np.array_equal(pack.neighborhood_sizes.cpu().numpy(), nbsizes)


def test_sorted_implicit_gemm_tensors(fvdb, cuda_device):
    grid, ijk, off = _grid(fvdb, [random_sparse_ijk(3000, 24, 5)], cuda_device)
    pack, _ = grid.sparse_conv_kernel_map(3, 1)
    pack.build_implicit_gemm(sorted=True, split_mask_num=1, training=True, split_mask_num_bwd=3)
    m = pack.out_in_map.cpu().numpy()
    sm = pack.sorted_mask.cpu().numpy()
    loc = pack.reorder_loc.cpu().numpy()
    n = grid.total_voxels
    bits = ((m >= 0) * (1 << np.arange(27))).sum(1)
    bits[n:] = 0
    # sort ties are not stable by contract: compare as a permutation giving equal sorted masks
    assert np.array_equal(np.sort(loc[0]), np.arange(m.shape[0]))
    assert np.array_equal(bits[loc[0]], sm[0])
    assert np.all(np.diff(sm[0].astype(np.int64)) <= 0)
    assert np.array_equal(pack.reorder_out_in_map.cpu().numpy(), m[loc[0]])


@pytest.mark.parametrize("name", golden_cases("sparse_"))
def test_golden_neighbours_through_api(fvdb, cuda_device, name):
    g = load_golden(name)
    ks, st = tuple(g["kernel_size"].tolist()), tuple(g["stride"].tolist())
    grid = fvdb.GridBatch.from_ijk(torch.from_numpy(g["ijk"]).to(cuda_device))
    pack, tgt = grid.sparse_conv_kernel_map(ks, st)
    pack.build_implicit_gemm()
    tijk = tgt.ijk.jdata.cpu().numpy()
    assert set(map(tuple, tijk.tolist())) == set(map(tuple, g["target_ijk"].tolist()))
    order = [rows_by_coord(tijk)[tuple(r)] for r in g["target_ijk"].tolist()]
    kmap = pack.out_in_map[: tgt.total_voxels].cpu().numpy()
    assert np.array_equal(kmap_to_coords(kmap, grid.ijk.jdata.cpu().numpy())[order], g["neighbours"])


def test_kmap_through_c_abi(fvdb, cuda_device):
    """fvgb_kmap_build called directly with raw device pointers (no torch types)."""
    from fvdb import _lib

    lib = _lib.cdll()
    grid, ijk, off = _grid(fvdb, [random_sparse_ijk(5000, 30, 31)], cuda_device)
    impl = grid._impl

    class Grid(ctypes.Structure):
        _fields_ = [
            ("num_grids", ctypes.c_int32), ("reserved", ctypes.c_int32), ("num_voxels", ctypes.c_int64),
            ("num_leaves", ctypes.c_int64), ("hash_capacity", ctypes.c_int64), ("voxel_offsets", ctypes.c_void_p),
            ("ijk", ctypes.c_void_p), ("leaves", ctypes.c_void_p), ("hash_slots", ctypes.c_void_p),
        ]

    g = Grid(impl.grid_count, 0, impl.total_voxels, impl.total_leaf_nodes, impl.hash.numel(),
             impl.joffsets.data_ptr(), impl.ijk.data_ptr(), impl.leaves.data_ptr(), impl.hash.data_ptr())
    K = 27
    kmap = torch.full((impl.total_voxels, K), -7, dtype=torch.int32, device=cuda_device)
    sizes = torch.zeros(K, dtype=torch.int32, device=cuda_device)
    ks = (ctypes.c_int32 * 3)(3, 3, 3)
    st = (ctypes.c_int32 * 3)(1, 1, 1)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    n_tiles = (impl.total_voxels + 127) // 128
    tmask = torch.zeros(n_tiles, dtype=torch.int32, device=cuda_device)
    rc = lib.fvgb_kmap_build(ctypes.byref(g), ctypes.byref(g), ks, st, ctypes.c_void_p(kmap.data_ptr()),
                             ctypes.c_int64(K), ctypes.c_void_p(sizes.data_ptr()), ctypes.c_void_p(tmask.data_ptr()),
                             stream)
    assert rc == 0
    torch.cuda.synchronize()
    src, soff = orc.grid_from_ijk(ijk, off)
    o = orc.kernel_map(src, soff, src, soff, (3, 3, 3), (1, 1, 1))
    assert np.array_equal(kmap.cpu().numpy(), o)
    assert np.array_equal(sizes.cpu().numpy(), (o >= 0).sum(0))
    # per-128-row-tile occupancy masks, computed in the same pass
    bits = ((o >= 0).astype(np.int64) << np.arange(K)).sum(1)
    pad = np.zeros(n_tiles * 128, dtype=np.int64)
    pad[: bits.size] = bits
    expect = np.bitwise_or.reduce(pad.reshape(n_tiles, 128), axis=1)
    assert np.array_equal(tmask.cpu().numpy().astype(np.int64) & 0xFFFFFFFF, expect)
    # bad arguments are rejected before any launch
    assert lib.fvgb_kmap_build(ctypes.byref(g), ctypes.byref(g), ks, st, ctypes.c_void_p(kmap.data_ptr()),
                               ctypes.c_int64(5), None, None, stream) == 1


def test_from_points_and_empty(fvdb, cuda_device):
    pts = torch.rand(5000, 3, generator=torch.Generator().manual_seed(0)) * 2 - 0.5
    grid = fvdb.GridBatch.from_points(pts.to(cuda_device), voxel_sizes=1 / 64, origins=0.0)
    ijk = torch.floor(pts * 64 + 0.5).to(torch.int32).numpy()
    o_ijk, _ = orc.grid_from_ijk(ijk, np.array([0, ijk.shape[0]]))
    assert np.array_equal(grid.ijk.jdata.cpu().numpy(), o_ijk)
    empty = fvdb.GridBatch.from_ijk(torch.zeros((0, 3), dtype=torch.int32, device=cuda_device))
    assert empty.total_voxels == 0
    pack, tgt = empty.sparse_conv_kernel_map(3, 1)
    pack.build_implicit_gemm()
    assert pack.out_in_map.shape[0] == 0


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32, torch.float16])
def test_from_points_rounds_in_point_precision(fvdb, cuda_device, dtype):
    """Points on and a few ulps next to half-voxel boundaries, two grids with their own voxel
    sizes and origins: the voxels are bit-exact vs the oracle's voxelisation in the points'
    own precision (double for FP64, float for FP32 / FP16), as BuildGridFromPoints.cu:27-43."""
    from tests.test_points_oracle import boundary_points

    w, o = [0.1, 0.05], [0.0, 0.37]
    parts = [boundary_points(3000, w[b], o[b], 11 + b) for b in range(2)]
    pts64 = np.concatenate(parts)
    pts = torch.from_numpy(pts64).to(dtype)
    vals = pts.double().numpy()  # the exact values the device sees
    joff = np.array([0, parts[0].shape[0], pts64.shape[0]])
    vs = np.array([[w[0]] * 3, [w[1]] * 3])
    org = np.array([[o[0]] * 3, [o[1]] * 3])
    prec = "f64" if dtype == torch.float64 else "f32"
    o_pts = orc.points_to_ijk(vals, joff, vs, org, prec)
    o_ijk, o_off = orc.grid_from_ijk(o_pts, joff)
    jt = fvdb.JaggedTensor.from_data_and_offsets(pts.to(cuda_device), torch.from_numpy(joff).to(cuda_device))
    grid = fvdb.GridBatch.from_points(jt, voxel_sizes=torch.from_numpy(vs), origins=torch.from_numpy(org))
    assert np.array_equal(grid.ijk.jdata.cpu().numpy(), o_ijk)
    assert np.array_equal(grid.joffsets.cpu().numpy(), o_off)
    if dtype == torch.float64:
        # the float rule places some of these points in other voxels
        f_pts = orc.points_to_ijk(vals.astype(np.float32).astype(np.float64), joff, vs, org, "f32")
        assert (f_pts != o_pts).any()


def test_coordinate_range_is_checked(fvdb, cuda_device):
    bad = torch.tensor([[0, 0, 0], [1 << 21, 0, 0]], dtype=torch.int32, device=cuda_device)
    with pytest.raises(ValueError):
        fvdb.GridBatch.from_ijk(bad)
