"""Argument checks of the C ABI's newer entry points, run without a GPU: each rejects bad
arguments with FVGB_EINVAL (1) or FVGB_ETYPE (2) before any device work, and the host-only size
queries answer (the reference maps these statuses to ValueError / TypeError)."""

import ctypes
import os

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(ROOT, "fvdb-core_gb300", "fvdb", "_lib", "libfvdb_gb300.so")
EINVAL, ETYPE = 1, 2
BF16, E4M3, F32 = 2, 4, 0
I64, I32, SZ = ctypes.c_int64, ctypes.c_int32, ctypes.c_size_t
P = ctypes.c_void_p(64)  # a non-null pointer that is never dereferenced: every call below fails first


@pytest.fixture(scope="module")
def lib():
    return ctypes.CDLL(LIB)


def test_tc_weight_bytes_is_a_host_query(lib):
    n = SZ(0)
    assert lib.fvgb_tc_weight_bytes(I32(BF16), I64(27), I32(32), I32(64), ctypes.byref(n)) == 0
    assert n.value >= 27 * 32 * 64 * 2
    assert lib.fvgb_tc_weight_bytes(I32(E4M3), I64(27), I32(128), I32(256), ctypes.byref(n)) == 0
    assert n.value >= 27 * 128 * 256
    assert lib.fvgb_tc_weight_bytes(I32(F32), I64(27), I32(32), I32(64), ctypes.byref(n)) == ETYPE
    assert lib.fvgb_tc_weight_bytes(I32(BF16), I64(0), I32(32), I32(64), ctypes.byref(n)) == EINVAL
    assert lib.fvgb_tc_weight_bytes(I32(BF16), I64(27), I32(32), I32(64), None) == EINVAL


def test_row_order_and_coarse_workspace_checks(lib):
    n = SZ(0)
    assert lib.fvgb_kmap_row_order_workspace(I64(-1), I32(27), ctypes.byref(n)) == EINVAL
    assert lib.fvgb_kmap_row_order_workspace(I64(100), I32(33), ctypes.byref(n)) == EINVAL
    assert lib.fvgb_kmap_row_order_workspace(I64(100), I32(0), ctypes.byref(n)) == EINVAL
    assert lib.fvgb_kmap_row_order_workspace(I64(1 << 31), I32(27), ctypes.byref(n)) == EINVAL
    assert lib.fvgb_coarse_grid_workspace(I64(-1), ctypes.byref(n)) == EINVAL
    assert lib.fvgb_coarse_grid_workspace(I64(10), None) == EINVAL
    assert lib.fvgb_coarse_grid_build(None, None, None, None, None, None, None, None, SZ(0), None) == EINVAL


def test_row_order_contraction_checks(lib):
    # fvgb_conv_fwd_tc_rows: element type first, then shapes
    args = lambda dtype, c_in, c_out, ldx: (I32(dtype), P, I64(10), I32(c_in), I64(ldx), P, I64(10), I32(27), P, P, P,
                                            I32(c_out), P, I64(c_out), None, None, I32(0), P, None)
    assert lib.fvgb_conv_fwd_tc_rows(*args(F32, 32, 64, 32)) == ETYPE
    assert lib.fvgb_conv_fwd_tc_rows(*args(BF16, 0, 64, 32)) == EINVAL
    assert lib.fvgb_conv_fwd_tc_rows(*args(BF16, 24, 64, 24)) == EINVAL  # 48-byte rows do not tile 128 bytes
    assert lib.fvgb_conv_fwd_tc_rows(*args(BF16, 32, 64, 16)) == EINVAL  # row stride below the row
    # fvgb_conv_fwd_simt_rows
    assert lib.fvgb_conv_fwd_simt_rows(I32(F32), P, I64(10), I32(8), I64(8), P, I64(10), I32(27), I64(26), P, P,
                                       I64(64), I64(8), I64(1), P, I32(8), I64(8), I32(0), None) == EINVAL


def test_halo_checks(lib):
    n = SZ(0)
    assert lib.fvgb_halo_conv(I32(F32), None, P, I64(8), I32(8), P, I32(8), I32(0), P, I64(8), None) == EINVAL
    assert lib.fvgb_halo_wgrad_workspace(I32(F32), None, I32(8), I32(8), ctypes.byref(n)) == EINVAL
    assert lib.fvgb_halo_wgrad(I32(F32), None, P, I64(8), I32(8), P, I64(8), I32(8), P, P, SZ(1 << 20), None) == EINVAL


def test_probe_checks(lib):
    bytes_ = I64(0)
    flops = ctypes.c_double(0)
    assert lib.fvgb_row_gather_probe(I32(7), P, I64(100), P, I32(128), I32(1), P, ctypes.byref(bytes_), None) == EINVAL
    assert lib.fvgb_row_gather_probe(I32(0), P, I64(100), P, I32(64), I32(1), P, ctypes.byref(bytes_), None) == EINVAL
    assert lib.fvgb_ffma_probe(None, I64(10), I32(1), ctypes.byref(flops), None) == EINVAL
    assert lib.fvgb_ffma_probe(P, I64(10), I32(65), ctypes.byref(flops), None) == EINVAL
