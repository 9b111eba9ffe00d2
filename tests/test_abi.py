"""The C ABI library loads without a GPU and exports every declared symbol."""

import ctypes as C
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
HEADERS = sorted((ROOT / "include").glob("*.h"))


def declared_functions():
    names = []
    for h in HEADERS:
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"^[A-Za-z_][\w \*]*?\b(hy_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_headers_declare_functions():
    names = declared_functions()
    assert "hy_render" in names and "hy_shade_pass" in names and "hy_volume_upload" in names
    assert len(names) >= 20


def test_library_exports_every_declared_symbol(built_lib):
    missing = [n for n in declared_functions() if not hasattr(built_lib, n)]
    assert not missing, f"not exported: {missing}"


def test_struct_sizes_match_reference_layouts(built_lib):
    from hydrant_gb300 import _abi

    # film pixel layouts of the reference (shader.hpp:26-34 etc.)
    assert C.sizeof(_abi.HyView) == 80
    assert C.sizeof(_abi.HyShaderParams) == 4 * (2 + 4 + 3 + 3 + 2 + 16 + 3 + 3 + 3 + 1)


def test_ctx_create_without_gpu_fails_cleanly(built_lib):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    rc = built_lib.hy_ctx_create(0, C.byref(h))
    assert rc != 0 and not h.value


def test_null_arguments_rejected(built_lib):
    from hydrant_gb300 import _abi

    assert built_lib.hy_render(None, None, None, None, 1, 1, None, None, None) == _abi.HY_ERR_INVALID
    assert built_lib.hy_tf_set(None, None, 0) == _abi.HY_ERR_INVALID
    assert built_lib.hy_volume_upload(None, None) == _abi.HY_ERR_INVALID
    assert built_lib.hy_camera_orbit(None, None, 60.0, None) == _abi.HY_ERR_INVALID


def test_python_structs_match_the_header(tmp_path):
    """Every struct the ctypes binding mirrors has the header's size and field
    offsets (a small C program compiled against include/hydrant_gb300.h
    prints them)."""
    import shutil
    import subprocess

    from hydrant_gb300 import _abi

    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    pairs = {"hy_view": _abi.HyView, "hy_camera": _abi.HyCamera,
             "hy_shader_params": _abi.HyShaderParams, "hy_volume_desc": _abi.HyVolumeDesc,
             "hy_volume_info": _abi.HyVolumeInfo, "hy_batch_view": _abi.HyBatchView,
             "hy_batch_config": _abi.HyBatchConfig, "hy_pager_desc": _abi.HyPagerDesc,
             "hy_pager_stats": _abi.HyPagerStats, "hy_diff_params": _abi.HyDiffParams,
             "hy_render_stats": _abi.HyRenderStats}
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "hydrant_gb300.h"',
             "int main(void) {"]
    for cname, py in pairs.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    inc = Path(__file__).resolve().parent.parent / "include"
    subprocess.run([cc, "-std=c99", "-I", str(inc), str(src), "-o", str(exe)], check=True)
    got = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    seen = {}
    for line in got:
        if line:
            c, f, v = line.split()
            seen[(c, f)] = int(v)
    for cname, py in pairs.items():
        assert seen[(cname, "size")] == C.sizeof(py), cname
        for fname, _ in py._fields_:
            assert seen[(cname, fname)] == getattr(py, fname).offset, f"{cname}.{fname}"
