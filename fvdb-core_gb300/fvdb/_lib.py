"""Loader of the native parts.  There is no fallback: if the CUDA library or the host
extension is missing, importing fvdb fails with an ImportError that says how to build."""

from __future__ import annotations

import ctypes
import glob
import importlib.machinery
import importlib.util
import os

import torch  # noqa: F401  (the extension needs libtorch loaded first)

from ._build import EXT_NAME, LIB_DIR, LIB_NAME

_C = None
_CDLL = None


def _missing(what: str) -> ImportError:
    return ImportError(
        f"fvdb_gb300 native {what} is not built in {LIB_DIR}. Build it with "
        "`python -c 'import __graft_entry__ as g; g.build()'` (or `python -m fvdb._build`)."
    )


def load():
    """Load libfvdb_gb300.so and the host extension (once)."""
    global _C, _CDLL
    if _C is not None:
        return _C
    lib = os.path.join(LIB_DIR, LIB_NAME)
    if not os.path.exists(lib):
        raise _missing("CUDA library " + LIB_NAME)
    _CDLL = ctypes.CDLL(lib, mode=ctypes.RTLD_GLOBAL)
    cands = sorted(glob.glob(os.path.join(LIB_DIR, "ext", EXT_NAME + "*.so")))
    if not cands:
        raise _missing("host extension " + EXT_NAME)
    loader = importlib.machinery.ExtensionFileLoader(EXT_NAME, cands[0])
    spec = importlib.util.spec_from_file_location(EXT_NAME, cands[0], loader=loader)
    mod = importlib.util.module_from_spec(spec)
    loader.exec_module(mod)
    _C = mod
    return _C


def cdll() -> ctypes.CDLL:
    """The C ABI library itself (for callers that bind it directly, e.g. via ctypes)."""
    load()
    return _CDLL
