"""Build libhydrant_gb300.so in-tree for sm_103a.

Every translation unit is compiled in parallel, then linked with nvcc.
Device code is compiled with -fmad=false and IEEE division / square root
so the march rounds exactly like the reference's CPU backend; host code
with -ffp-contract=off for the same reason.
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libhydrant_gb300.so"

SOURCES = ["hy_api.cc", "hy_volume.cu", "hy_render.cu", "hy_batch.cu", "hy_page.cu", "hy_diff.cu",
           "hy_synth.cc", "hy_store_io.cc"]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = [
    "-O3",
    "-std=c++17",
    "-lineinfo",
    "-fmad=false",
    "-prec-div=true",
    "-prec-sqrt=true",
    "-ftz=false",
    "-Xcompiler",
    "-fPIC,-O2,-ffp-contract=off,-fno-strict-aliasing",
]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def extra_flags() -> list[str]:
    """Macro settings for tuning builds (e.g. "-DHY_DIFF_MIN_BLOCKS=6"), from
    HYDRANT_GB300_NVCC_DEFINES; only -D options are taken."""
    return [f for f in os.environ.get("HYDRANT_GB300_NVCC_DEFINES", "").split() if f.startswith("-D")]


def _compile(src: str, verbose: bool) -> Path:
    obj = BUILD / (Path(src).stem + ".o")
    cmd = [nvcc(), *ARCH, *NVCC_COMMON, *extra_flags(), "-c", str(CSRC / src), "-o", str(obj)]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile {src} failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose and r.stderr:
        sys.stderr.write(r.stderr)
    return obj


def _stale(sources: list[Path], target: Path) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    deps = list(sources) + list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh"))
    deps += list((PKG.parent / "include").glob("*.h*")) + [Path(__file__)]
    return any(p.exists() and p.stat().st_mtime > t for p in deps)


def build(force: bool = False, verbose: bool = False) -> Path:
    srcs = [CSRC / s for s in SOURCES]
    stamp = BUILD / "defines.txt"
    defines = " ".join(extra_flags())
    same_defines = (stamp.read_text() if stamp.exists() else "") == defines
    if not force and same_defines and not _stale(srcs, LIB):
        return LIB
    BUILD.mkdir(exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    stamp.write_text(defines)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIB)
