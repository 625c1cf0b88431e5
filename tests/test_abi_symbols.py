"""The C ABI library loads and exports every entry point that include/fvdb_gb300.h declares
(no device work: nothing here needs a GPU)."""

import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "fvdb_gb300.h")
LIB = os.path.join(ROOT, "fvdb-core_gb300", "fvdb", "_lib", "libfvdb_gb300.so")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(fvgb_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert "fvgb_kmap_build" in syms and "fvgb_conv_fwd_simt" in syms
    assert len(syms) >= 15


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(LIB)
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, f"symbols declared but not exported: {missing}"


def test_host_only_entry_points():
    lib = ctypes.CDLL(LIB)
    lib.fvgb_version.restype = ctypes.c_char_p
    assert b"sm_103a" in lib.fvgb_version()
    n = ctypes.c_size_t(0)
    assert lib.fvgb_ijk_sort_unique_workspace(ctypes.c_int64(1000), ctypes.c_int32(2), ctypes.byref(n)) == 0
    assert n.value > 1000 * 8
    # argument validation happens before any device work
    assert lib.fvgb_ijk_sort_unique_workspace(ctypes.c_int64(-1), ctypes.c_int32(1), ctypes.byref(n)) == 1
    assert lib.fvgb_kmap_masks(None, ctypes.c_int64(10), ctypes.c_int32(40), ctypes.c_int64(40), None, None, None) == 1


def test_selftest_wait_rejects_bad_arguments_without_a_gpu():
    """Argument checks of fvgb_selftest_wait_timeout return FVGB_EINVAL before any device work."""
    lib = ctypes.CDLL(LIB)
    assert lib.fvgb_selftest_wait_timeout(None, ctypes.c_int64(100), 0, None) == 1
    assert lib.fvgb_selftest_wait_timeout(ctypes.c_void_p(16), ctypes.c_int64(0), 0, None) == 1
    assert lib.fvgb_selftest_wait_timeout(ctypes.c_void_p(16), ctypes.c_int64(1 << 40), 0, None) == 1
