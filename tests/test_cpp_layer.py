"""The C++ layer (include/hydrant_gb300_renderer.hpp, hydrant_gb300_json.hpp).

CPU: the JSON reader / config parsing checks compile and pass, and the
renderer driver compiles against the header and the library.  GPU: the
driver renders a saved dataset from a JSON configuration through
RendererFactory / IRenderer, and its images equal those of the same calls
made through the Python binding of the C ABI.
"""

import json
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
LIBDIR = ROOT / "hydrant_gb300"


def _compile(src: str, out: Path) -> Path:
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    if not (LIBDIR / "libhydrant_gb300.so").exists():
        pytest.skip("library not built")
    cmd = [gxx, "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", f"-I{ROOT / 'include'}",
           str(ROOT / "tests" / "cpp" / src), "-o", str(out), f"-L{LIBDIR}", "-lhydrant_gb300",
           f"-Wl,-rpath,{LIBDIR}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def test_json_and_config_checks(tmp_path):
    exe = _compile("json_check.cc", tmp_path / "json_check")
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr


def test_renderer_driver_compiles(tmp_path):
    _compile("shim_render.cc", tmp_path / "shim_render")


@pytest.mark.gpu
@pytest.mark.parametrize("renderer,params", [
    ("Volume", {"mode": "Default", "density": 0.5, "sample_rate": 0.5, "mem_limit_mb": 4,
                "transfer_fn": {"values": [[0, 0, 0, 0], [1, 0, 0, 1], [1, 0.5, 0, 1],
                                           [1, 1, 0, 1], [0, 1, 0, 1], [0, 1, 1, 1],
                                           [0, 0, 1, 1], [1, 0, 1, 1], [0, 0, 0, 0]]}}),
    ("Isosurface", {"mode": "Color", "isovalue": 0.5, "mem_limit_mb": 4}),
    ("Blocks", {"mode": "Volume", "density": 0.05}),
    ("Paging", {"mem_limit_mb": 4}),
])
def test_renderer_factory_renders_like_the_c_abi(ctx, tmp_path, renderer, params):
    torch = pytest.importorskip("torch")
    import hydrant_gb300 as hy
    from hydrant_gb300 import _abi

    vox = hy.synth_tubes_u8(1, (96, 96, 96), 12)
    vol = hy.Volume(ctx, vox, 16, 1)
    store = hy.Store.from_volume(vol)
    store.build_coarse(2)
    ds = tmp_path / "ds"
    store.save(ds)
    W, H = 80, 64
    cfg = {"camera": {"orbit": {"arm": [30, 40, 2.2]}},
           "render": {"resolution": [W, H], "renderer": renderer, "params": params}}
    (tmp_path / "cfg.json").write_text(json.dumps(cfg))
    exe = _compile("shim_render.cc", tmp_path / "shim_render")
    r = subprocess.run([str(exe), str(ds), str(tmp_path / "cfg.json"), str(tmp_path / "out")],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    got = {k: np.fromfile(tmp_path / f"out.{k}.rgba", np.uint8).reshape(H, W, 4)
           for k in ("offline", "realtime", "updated", "loop_dynamic", "loop_lossless")}
    # the realtime session through IRenderLoop: every callback in order, and
    # the last frame (back at the configured camera) as the single frames
    for q in ("dynamic", "lossless"):
        assert (f"loop {q} post_loop=1 post_frame=3 frames=3 after_frame=3 after_loop=1"
                in r.stdout), r.stdout
    assert np.array_equal(got["loop_dynamic"], got["realtime"])
    assert np.array_equal(got["loop_lossless"], got["offline"])

    # the same frames through the Python binding
    cam = hy.camera_orbit((30, 40, 2.2))
    shader = renderer
    kw = dict(shader=shader, sample_rate=params.get("sample_rate", 1.0),
              density=params.get("density", 1.0 if renderer != "Blocks" else 1e-2),
              isovalue=params.get("isovalue", 0.5))
    kw["mode"] = params.get("mode", "Default")
    if renderer == "Volume":
        ctx.set_transfer_fn(np.array(params["transfer_fn"]["values"], np.float32))
    slots_off = min(4 * 2**20 // store.info.slot_bytes, 4096)
    slots_rt = 4 * 2**20 // store.info.slot_bytes

    def frame(mode, slots, clear=(0, 0, 0)):
        p = hy.shader_params(clear_color=clear, **kw)
        pg = hy.Pager(ctx, store, slots, mode)
        try:
            out = torch.zeros(W * H * 4, dtype=torch.uint8, device="cuda")
            if renderer == "Isosurface":
                hy.iso_lighting(pg.volume, cam, p)
            if renderer == "Blocks":
                view = hy.camera_view(pg.volume, cam)
                return hy.render(ctx, pg.volume, p, view, W, H).rgba
            pg.render(p, cam, W, H, out.data_ptr())
            ctx.synchronize()
            return out.cpu().numpy().reshape(H, W, 4)
        finally:
            pg.close()

    try:
        assert np.array_equal(got["realtime"], frame(_abi.PAGER_REALTIME, slots_rt))
        if renderer == "Paging":  # the reference's offline Paging frame is not rendered
            assert not got["offline"].any() and not got["updated"].any()
            assert (got["realtime"][..., 1] > 0).any()
            return
        assert np.array_equal(got["offline"], frame(_abi.PAGER_LOSSLESS, slots_off))
        upd = frame(_abi.PAGER_LOSSLESS, slots_off, clear=(0.25, 0.5, 1.0))
        assert np.array_equal(got["updated"], upd)
        assert (got["offline"][..., 3] > 0).any()
    finally:
        store.close()
        vol.close()
