"""Builds the CPU oracle (test infrastructure only) into oracle/_build/.

The reference's own CPU path cannot be compiled here from its sources: it needs NanoVDB,
CUTLASS and the rest of fvdb-core's CMake-fetched dependencies, none of which are in the
source tree.  So there is no oracle/_ref build; the oracle is the C restatement in
fvdb_oracle.c plus oracle.py.
"""

from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libfvdb_oracle.so")


def build() -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    src = os.path.join(HERE, "fvdb_oracle.c")
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(src):
        return LIB
    cmd = ["gcc", "-O2", "-std=c11", "-shared", "-fPIC", src, "-o", LIB, "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return LIB


if __name__ == "__main__":
    print(build())
