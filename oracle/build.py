"""Build the oracle (test infrastructure only) into oracle/_build/.

    python oracle/build.py

-ffp-contract=off keeps every multiply and add separately rounded, so the
oracle gives the same floats on x86-64 and aarch64.
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build"
LIB = OUT / "libhy_oracle.so"
SRC = [HERE / "hy_oracle.cc", HERE / "synth.cc"]


def build(force: bool = False) -> Path:
    deps = SRC + [HERE / "hy_oracle.h", Path(__file__)]
    if not force and LIB.exists() and all(d.stat().st_mtime <= LIB.stat().st_mtime for d in deps):
        return LIB
    OUT.mkdir(exist_ok=True)
    cxx = os.environ.get("CXX") or shutil.which("g++") or "g++"
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           "-o", str(tmp), *map(str, SRC), "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{' '.join(cmd)}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
