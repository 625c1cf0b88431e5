"""fvgb_ijk_sort_unique_in_box: sorting only the order-key bits that can differ inside known
coordinate bounds gives exactly the full sort's voxels and offsets; a coordinate outside the
bounds is reported as FVGB_ERANGE."""

import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

FVGB_ERANGE = 3


def _sort(lib, ijk, joff, box):
    n, B = ijk.shape[0], joff.numel() - 1
    wb = ctypes.c_size_t(0)
    assert lib.fvgb_ijk_sort_unique_workspace(ctypes.c_int64(n), ctypes.c_int32(B), ctypes.byref(wb)) == 0
    ws = torch.empty(wb.value, dtype=torch.uint8, device=ijk.device)
    out = torch.empty_like(ijk)
    ooff = torch.empty(B + 1, dtype=torch.int64, device=ijk.device)
    err = torch.zeros(1, dtype=torch.int32, device=ijk.device)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    P = lambda t: ctypes.c_void_p(t.data_ptr())
    if box is None:
        rc = lib.fvgb_ijk_sort_unique(P(ijk), P(joff), ctypes.c_int32(B), ctypes.c_int64(n), P(out), P(ooff), P(err),
                                      P(ws), wb, stream)
    else:
        lo, hi = (ctypes.c_int32 * 3)(*box[0]), (ctypes.c_int32 * 3)(*box[1])
        rc = lib.fvgb_ijk_sort_unique_in_box(P(ijk), P(joff), ctypes.c_int32(B), ctypes.c_int64(n), lo, hi, P(out),
                                             P(ooff), P(err), P(ws), wb, stream)
    assert rc == 0
    torch.cuda.synchronize()
    m = int(ooff[-1].item())
    return out[:m].cpu(), ooff.cpu(), int(err.item())


@pytest.mark.parametrize("lo,hi", [((0, 0, 0), (127, 127, 127)), ((-300, 1000, -5000), (500, 1040, -4000)),
                                   ((7, -9, 4095), (7, 9, 4100)), ((-2**20, 0, 0), (2**20 - 1, 3, 5)),
                                   ((3, 3, 3), (3, 3, 3))])
def test_bounded_sort_equals_full_sort(cuda_device, lo, hi):
    from fvdb import _lib

    lib = _lib.cdll()
    rng = np.random.default_rng(abs(hash((lo, hi))) % 2**32)
    n = 60000
    ijk = np.stack([rng.integers(lo[a], hi[a] + 1, n) for a in range(3)], 1).astype(np.int32)
    ijk_d = torch.from_numpy(ijk).to(cuda_device)
    joff = torch.tensor([0, n // 3, n], dtype=torch.int64, device=cuda_device)
    full = _sort(lib, ijk_d, joff, None)
    boxed = _sort(lib, ijk_d, joff, (lo, hi))
    assert full[2] == 0 and boxed[2] == 0
    assert torch.equal(full[0], boxed[0])
    assert torch.equal(full[1], boxed[1])


def test_coordinate_outside_box_is_reported(cuda_device):
    from fvdb import _lib

    lib = _lib.cdll()
    ijk = torch.tensor([[0, 0, 0], [5, 5, 5], [9, 2, 2]], dtype=torch.int32, device=cuda_device)
    joff = torch.tensor([0, 3], dtype=torch.int64, device=cuda_device)
    assert _sort(lib, ijk, joff, ((0, 0, 0), (8, 8, 8)))[2] == FVGB_ERANGE
    assert _sort(lib, ijk, joff, ((0, 0, 0), (9, 8, 8)))[2] == 0


def test_large_grid_build_sorts_within_measured_bounds(cuda_device):
    """Inputs of >= 2^18 points are sorted over the key bits their measured bounding box allows;
    the voxels and offsets equal the oracle's NanoVDB order (coordinates crossing zero and a
    root-tile boundary)."""
    import fvdb
    from oracle import oracle as orc

    rng = np.random.default_rng(11)
    n = 300_000
    ijk = np.stack([rng.integers(-700, 300, n), rng.integers(4000, 4400, n), rng.integers(-90, 90, n)],
                   1).astype(np.int32)
    off = np.array([0, 120_000, n], dtype=np.int64)
    jt = fvdb.JaggedTensor.from_data_and_offsets(torch.from_numpy(ijk).to(cuda_device),
                                                 torch.from_numpy(off).to(cuda_device))
    grid = fvdb.GridBatch.from_ijk(jt)
    ref, ref_off = orc.grid_from_ijk(ijk, off)
    assert np.array_equal(grid.ijk.jdata.cpu().numpy(), ref)
    assert np.array_equal(grid.joffsets.cpu().numpy(), ref_off)


@pytest.mark.parametrize("factor", [(2, 2, 2), (4, 4, 4), (8, 8, 8), (2, 4, 1), (1, 8, 2)])
def test_coarse_grid_by_leaves_equals_voxel_sort(cuda_device, factor):
    """conv_grid(k = s) and coarsened_grid for power-of-two factors are built leaf by leaf
    (fvgb_coarse_grid_build): exactly the voxels, order and offsets of the oracle's coarse grid
    (floor(ijk / s) sorted voxel by voxel), for several grids, negative coordinates and sparse and
    dense regions, and a working leaf table (ijk_to_index of every coarse voxel is its index)."""
    import fvdb

    from oracle import oracle as orc
    from tests.helpers import random_sparse_ijk

    parts = [random_sparse_ijk(6000, 48, 11, lo=-70), random_sparse_ijk(300, 9, 12, lo=5),
             random_sparse_ijk(9000, 200, 13, lo=-1000)]
    dense = np.stack(np.meshgrid(*[np.arange(-20, 20)] * 3, indexing="ij"), -1).reshape(-1, 3).astype(np.int32)
    parts.append(dense)
    grid = fvdb.GridBatch.from_ijk(fvdb.JaggedTensor([torch.from_numpy(p).to(cuda_device) for p in parts]))
    ijk = grid.ijk.jdata.cpu().numpy()
    off = grid.joffsets.cpu().numpy()
    c_ijk, c_off = orc.conv_grid(ijk, off, factor, factor)
    for coarse in (grid.conv_grid(factor, factor), grid.coarsened_grid(factor)):
        assert np.array_equal(coarse.ijk.jdata.cpu().numpy(), c_ijk)
        assert np.array_equal(coarse.joffsets.cpu().numpy(), c_off)
        idx = coarse.ijk_to_index(coarse.ijk, cumulative=True).jdata.cpu().numpy()
        assert np.array_equal(idx, np.arange(c_ijk.shape[0]))
