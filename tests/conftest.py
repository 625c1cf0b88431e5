import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG_PARENT = os.path.join(ROOT, "fvdb-core_gb300")
for p in (ROOT, PKG_PARENT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _ensure_built():
    import importlib.util

    def load(name, path):
        spec = importlib.util.spec_from_file_location(name, path)
        m = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(m)
        return m

    load("_t_oracle_build", os.path.join(ROOT, "oracle", "build.py")).build()
    lib = os.path.join(PKG_PARENT, "fvdb", "_lib", "libfvdb_gb300.so")
    ext_dir = os.path.join(PKG_PARENT, "fvdb", "_lib", "ext")
    have_ext = os.path.isdir(ext_dir) and any(f.endswith(".so") for f in os.listdir(ext_dir))
    if not (os.path.exists(lib) and have_ext):
        load("_t_fvdb_build", os.path.join(PKG_PARENT, "fvdb", "_build.py")).build()


_ensure_built()


@pytest.fixture(scope="session")
def cuda_device():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda", 0)
