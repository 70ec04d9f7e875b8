"""Build recipe for the CPU oracle (test infrastructure only).

Compiles ``oracle/galax_oracle.cpp`` with the host C++ compiler into
``oracle/_build/libgalax_oracle.so``. The reference (GalacticDynamics/galax) is
pure Python on JAX and has no native sources, so there is no ``oracle/_ref``
build: the oracle is a restatement, pinned against the reference's golden
values (``tests/golden/``).
"""

from __future__ import annotations

import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "galax_oracle.cpp"
OUT_DIR = HERE / "_build"
LIB = OUT_DIR / "libgalax_oracle.so"


def build(force: bool = False) -> Path:
    OUT_DIR.mkdir(exist_ok=True)
    if LIB.exists() and not force and LIB.stat().st_mtime >= SRC.stat().st_mtime:
        return LIB
    cxx = os.environ.get("CXX", "g++")
    tmp = LIB.with_suffix(f".so.tmp{os.getpid()}")
    cmd = [cxx, "-O2", "-std=c++17", "-fopenmp", "-shared", "-fPIC", "-o", str(tmp), str(SRC)]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
