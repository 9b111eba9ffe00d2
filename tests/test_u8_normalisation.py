"""The kernels normalise u8 voxels as fma(u, hi, u * lo) with hi + lo = 1/255
in two floats (hydrant_gb300/csrc/hy_shade.cuh, u8_norm) instead of the
reference's u / 255.f (texture_3d.hpp:78-86).  This checks, with the C
library's correctly rounded fmaf and IEEE single precision, that the two agree
bit for bit on all 256 inputs; the CUDA intrinsics compute the same IEEE
operations."""

import shutil
import subprocess

import pytest

SRC = r"""
#include <math.h>
#include <stdio.h>
int main(void) {
    volatile float hi = 1.0f / 255.0f;
    volatile float lo = (float)(1.0 / 255.0 - (double)hi);
    int bad = 0;
    for (unsigned u = 0; u < 256; ++u) {
        volatile float x = (float)u;
        volatile float ref = x / 255.0f;
        volatile float t = x * lo;
        volatile float q = fmaf(x, hi, t);
        if (q != ref) ++bad;
    }
    printf("%d\n", bad);
    return 0;
}
"""


def test_two_word_reciprocal_is_exact(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    (tmp_path / "u8.c").write_text(SRC)
    exe = tmp_path / "u8"
    r = subprocess.run([cc, "-O0", "-ffp-contract=off", str(tmp_path / "u8.c"), "-o", str(exe),
                        "-lm"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=30)
    assert out.stdout.strip() == "0"
