"""fvgb_conv_wgrad_simt_noalloc: the weight gradient for callers that cannot allocate device
memory when they call it (plugins in runtimes that plan all device memory ahead of time,
serving code that must not risk an allocation synchronising the device or failing
mid-request).  It keeps its partials in a fixed 4 MiB device array of the library instead of
a caller workspace.

Checked through the C ABI against the allocating entry point fvgb_conv_wgrad_simt, on two
calls in a row (the shared array keeps the previous call's contents, which must not leak into
the next result).  This file is collected last so that a run stopping at the first failure
has already run every other test.
"""

import ctypes

import numpy as np
import pytest
import torch

from tests.helpers import random_sparse_ijk

pytestmark = pytest.mark.gpu

F32, F64 = 0, 1
OK, ENOSPACE = 0, 6


def _case(dev, n_vox, cin, cout, dtype, seed):
    import fvdb

    grid = fvdb.GridBatch.from_ijk(torch.from_numpy(random_sparse_ijk(n_vox, 40, seed)).to(dev))
    pack, _ = grid.sparse_conv_kernel_map(3, 1)
    pack.build_implicit_gemm()
    kmap = pack.out_in_map
    g = torch.Generator().manual_seed(seed)
    x = torch.randn(grid.total_voxels, cin, generator=g, dtype=dtype).to(dev)
    dy = torch.randn(grid.total_voxels, cout, generator=g, dtype=dtype).to(dev)
    return grid.total_voxels, kmap, x, dy


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


# (64, 64) FP32: one row chunk's partials take 27*64*64*4 = 442 KB, so the 4 MiB array holds 9
# chunks against the 47 that the allocating entry point plans for 12k voxels; the no-alloc
# entry point then re-plans with longer row chunks.
@pytest.mark.parametrize("dtype,code,cin,cout", [(torch.float32, F32, 16, 32), (torch.float64, F64, 24, 8),
                                                 (torch.float32, F32, 64, 64)])
def test_noalloc_matches_allocating_entry_point(cuda_device, dtype, code, cin, cout):
    from fvdb import _lib

    lib = _lib.cdll()
    n, kmap, x, dy = _case(cuda_device, 12000, cin, cout, dtype, seed=cin + cout)
    K = kmap.shape[1]
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    need = ctypes.c_size_t(0)
    assert lib.fvgb_wgrad_workspace(code, ctypes.c_int64(n), K, cin, cout, ctypes.byref(need)) == OK
    ws = torch.empty(need.value, dtype=torch.uint8, device=cuda_device)
    ref = torch.empty(K, cin, cout, dtype=dtype, device=cuda_device)
    assert lib.fvgb_conv_wgrad_simt(code, _p(x), ctypes.c_int64(n), cin, ctypes.c_int64(cin), _p(kmap),
                                    ctypes.c_int64(n), K, ctypes.c_int64(K), _p(dy), cout, ctypes.c_int64(cout),
                                    _p(ref), _p(ws), need, stream) == OK
    tol = 2e-5 if dtype == torch.float32 else 1e-12
    outs = []
    for _ in range(2):  # two calls in a row share the scratch array
        dw = torch.full((K, cin, cout), float("nan"), dtype=dtype, device=cuda_device)
        rc = lib.fvgb_conv_wgrad_simt_noalloc(code, _p(x), ctypes.c_int64(n), cin, ctypes.c_int64(cin), _p(kmap),
                                              ctypes.c_int64(n), K, ctypes.c_int64(K), _p(dy), cout,
                                              ctypes.c_int64(cout), _p(dw), stream)
        assert rc == OK
        outs.append(dw)
    torch.cuda.synchronize()
    r = ref.double().cpu().numpy()
    for dw in outs:
        d = dw.double().cpu().numpy()
        assert np.isfinite(d).all()
        assert np.abs(d - r).max() <= tol * max(np.abs(r).max(), 1e-30)


def test_noalloc_rejects_sizes_beyond_its_scratch(cuda_device):
    from fvdb import _lib

    lib = _lib.cdll()
    lib.fvgb_last_error.restype = ctypes.c_char_p
    n, kmap, x, dy = _case(cuda_device, 2000, 8, 8, torch.float32, seed=3)
    dw = torch.empty(1, device=cuda_device)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    # 27 * 256 * 256 fp32 partials (7 MiB) do not fit the 4 MiB array: rejected before any launch
    rc = lib.fvgb_conv_wgrad_simt_noalloc(F32, _p(x), ctypes.c_int64(n), 256, ctypes.c_int64(256), _p(kmap),
                                          ctypes.c_int64(n), 27, ctypes.c_int64(27), _p(dy), 256,
                                          ctypes.c_int64(256), _p(dw), stream)
    assert rc == ENOSPACE
    assert b"4 MiB" in lib.fvgb_last_error()
    # sizes whose product overflows 64 bits are rejected too, not wrapped into a small size
    big = 1 << 30
    rc = lib.fvgb_conv_wgrad_simt_noalloc(F32, _p(x), ctypes.c_int64(n), big, ctypes.c_int64(big), _p(kmap),
                                          ctypes.c_int64(n), 27, ctypes.c_int64(27), _p(dy), big,
                                          ctypes.c_int64(big), _p(dw), stream)
    assert rc == ENOSPACE
