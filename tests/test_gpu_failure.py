"""Failure detection without a GPU fault: the bounded in-kernel wait that every tensor-core
kernel uses gives up on a phase nothing completes and reports FVGB_ETIMEOUT through the device
error word; the context stays usable afterwards."""

import ctypes

import numpy as np
import pytest
import torch

from tests.helpers import random_sparse_ijk

pytestmark = pytest.mark.gpu

FVGB_ETIMEOUT = 5


def test_bounded_wait_reports_timeout_and_context_survives(cuda_device):
    import fvdb
    from fvdb import _lib

    lib = _lib.cdll()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    err = torch.zeros(1, dtype=torch.int32, device=cuda_device)
    budget = ctypes.c_int64(1 << 22)  # ~2 ms of SM cycles
    # nothing arrives on the barrier: the wait runs out
    assert lib.fvgb_selftest_wait_timeout(ctypes.c_void_p(err.data_ptr()), budget, 0, stream) == 0
    torch.cuda.synchronize()
    assert int(err.item()) == FVGB_ETIMEOUT
    # positive control: the phase completes before the wait
    err.zero_()
    assert lib.fvgb_selftest_wait_timeout(ctypes.c_void_p(err.data_ptr()), budget, 1, stream) == 0
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    # the context is still usable: a tensor-core convolution runs and reports no error
    grid = fvdb.GridBatch.from_ijk(torch.from_numpy(random_sparse_ijk(5000, 24, 3)).to(cuda_device))
    pack, _ = grid.sparse_conv_kernel_map(3, 1)
    x = torch.randn(grid.total_voxels, 32, device=cuda_device).bfloat16()
    w = (torch.randn(64, 32, 3, 3, 3, device=cuda_device) * 0.05).bfloat16()
    y = pack.sparse_conv_3d(x, w).jdata
    torch.cuda.synchronize()
    fvdb._lib.load().check_device_errors(cuda_device)
    assert y.shape == (grid.total_voxels, 64) and bool(torch.isfinite(y.float()).all())


def test_measurement_probes_run(cuda_device):
    """The FFMA and row-gather probes launch, finish without a timeout and report their work."""
    import ctypes

    from fvdb import _lib

    lib = _lib.cdll()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    out = torch.zeros(2, device=cuda_device)
    flops = ctypes.c_double(0.0)
    assert lib.fvgb_ffma_probe(ctypes.c_void_p(out.data_ptr()), ctypes.c_int64(64), 1, ctypes.byref(flops), stream) == 0
    torch.cuda.synchronize()
    assert flops.value > 0
    n = 4096
    x = torch.zeros(n, 64, device=cuda_device, dtype=torch.bfloat16)
    rows = torch.randint(0, n, (1024,), device=cuda_device, dtype=torch.int32)
    err = torch.zeros(1, device=cuda_device, dtype=torch.int32)
    nbytes = ctypes.c_int64(0)
    for mode in range(5):
        assert lib.fvgb_row_gather_probe(mode, ctypes.c_void_p(x.data_ptr()), ctypes.c_int64(n),
                                         ctypes.c_void_p(rows.data_ptr()), rows.numel(), 8,
                                         ctypes.c_void_p(err.data_ptr()), ctypes.byref(nbytes), stream) == 0
        torch.cuda.synchronize()
        assert int(err.item()) == 0 and nbytes.value > 0
    # argument checks: unknown mode, too few row indices
    assert lib.fvgb_row_gather_probe(5, ctypes.c_void_p(x.data_ptr()), ctypes.c_int64(n), ctypes.c_void_p(rows.data_ptr()),
                                     rows.numel(), 8, ctypes.c_void_p(err.data_ptr()), ctypes.byref(nbytes), stream) == 1
    assert lib.fvgb_row_gather_probe(3, ctypes.c_void_p(x.data_ptr()), ctypes.c_int64(n), ctypes.c_void_p(rows.data_ptr()),
                                     64, 8, ctypes.c_void_p(err.data_ptr()), ctypes.byref(nbytes), stream) == 1
