"""In-tree build of the native parts of fvdb_gb300.

Two shared objects are produced next to this file, in ``_lib/``:

* ``libfvdb_gb300.so`` -- the CUDA kernels behind the C ABI of ``include/fvdb_gb300.h``,
  compiled by nvcc for sm_103a only (one ``-gencode``), translation units in parallel;
* ``fvdb_gb300_C*.so`` -- the C++ PyTorch extension (host objects + autograd bodies),
  built with ``torch.utils.cpp_extension`` and linked against the library above.

Nothing is installed into site-packages.  ``build()`` is idempotent: units whose sources
did not change are not recompiled.
"""

from __future__ import annotations

import concurrent.futures
import hashlib
import os
import shutil
import subprocess
import sys

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
ROOT_DIR = os.path.dirname(os.path.dirname(PKG_DIR))
CSRC = os.path.join(os.path.dirname(PKG_DIR), "csrc")
INCLUDE = os.path.join(ROOT_DIR, "include")
LIB_DIR = os.path.join(PKG_DIR, "_lib")
LIB_NAME = "libfvdb_gb300.so"
EXT_NAME = "fvdb_gb300_C"

CUDA_UNITS = ["abi.cu", "grid.cu", "kmap.cu", "conv_simt.cu", "conv_fwd_tc.cu", "conv_fwd_plan.cu", "conv_tc.cu", "pool.cu",
              "halo.cu", "probe.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


def _nvcc() -> str:
    home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    cand = os.path.join(home, "bin", "nvcc")
    return cand if os.path.exists(cand) else (shutil.which("nvcc") or "nvcc")


def _digest(paths: list[str], extra: str = "") -> str:
    h = hashlib.sha256(extra.encode())
    for p in paths:
        with open(p, "rb") as f:
            h.update(f.read())
    return h.hexdigest()[:16]


def _headers() -> list[str]:
    hs = [os.path.join(INCLUDE, "fvdb_gb300.h")]
    hs += sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cuh"))
    return hs


def _compile_unit(unit: str, obj_dir: str) -> str:
    src = os.path.join(CSRC, unit)
    obj = os.path.join(obj_dir, unit.replace(".cu", ".o"))
    stamp = obj + ".stamp"
    key = _digest([src] + _headers(), " ".join(ARCH + NVCC_FLAGS))
    if os.path.exists(obj) and os.path.exists(stamp) and open(stamp).read() == key:
        return obj
    cmd = [_nvcc(), *ARCH, *NVCC_FLAGS, "-I", INCLUDE, "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {unit}:\n{r.stdout}\n{r.stderr}")
    with open(stamp, "w") as f:
        f.write(key)
    return obj


def build_cuda_library(verbose: bool = False) -> str:
    """Compile every CUDA unit for sm_103a and link libfvdb_gb300.so (in-tree)."""
    obj_dir = os.path.join(LIB_DIR, "obj")
    os.makedirs(obj_dir, exist_ok=True)
    units = [u for u in CUDA_UNITS if os.path.exists(os.path.join(CSRC, u))]
    with concurrent.futures.ThreadPoolExecutor(max_workers=max(1, min(len(units), os.cpu_count() or 4))) as ex:
        objs = list(ex.map(lambda u: _compile_unit(u, obj_dir), units))
    out = os.path.join(LIB_DIR, LIB_NAME)
    key = _digest(objs)
    stamp = out + ".stamp"
    if not (os.path.exists(out) and os.path.exists(stamp) and open(stamp).read() == key):
        cmd = [_nvcc(), *ARCH, "-shared", "-cudart", "shared", "-o", out, *objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link of {LIB_NAME} failed:\n{r.stdout}\n{r.stderr}")
        with open(stamp, "w") as f:
            f.write(key)
    if verbose:
        print(f"[fvdb_gb300] built {out}")
    return out


def build_extension(verbose: bool = False):
    """Build (or reuse) the C++ host extension; returns the loaded module."""
    from torch.utils import cpp_extension

    ext_dir = os.path.join(LIB_DIR, "ext")
    os.makedirs(ext_dir, exist_ok=True)
    src = os.path.join(CSRC, "host", "ext.cpp")
    mod = cpp_extension.load(
        name=EXT_NAME,
        sources=[src],
        extra_cflags=["-O2", "-std=c++17", f"-I{INCLUDE}"],
        extra_ldflags=[f"-L{LIB_DIR}", "-lfvdb_gb300", f"-Wl,-rpath,{LIB_DIR}"],
        build_directory=ext_dir,
        with_cuda=True,
        verbose=verbose,
    )
    return mod


def build(verbose: bool = False):
    """Build everything native in the package; returns the host extension module."""
    build_cuda_library(verbose)
    return build_extension(verbose)


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
