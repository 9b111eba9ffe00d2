"""Committed golden vectors (tests/golden/golden.npz, made by make_golden.py).

CPU: the oracle reproduces them bit for bit.
GPU: the CUDA path (through the C ABI) matches them within the parity bar.
"""

from pathlib import Path

import numpy as np
import pytest

from tests.golden import make_golden as mg

GOLDEN = np.load(Path(__file__).resolve().parent / "golden" / "golden.npz")


@pytest.mark.parametrize("case", mg.CASES, ids=[c[0] for c in mg.CASES])
def test_oracle_reproduces_golden(case):
    name = case[0]
    _, view, r = mg.render_case(case)
    np.testing.assert_array_equal(view, GOLDEN[f"{name}/view"])
    np.testing.assert_array_equal(r["rgba"], GOLDEN[f"{name}/rgba"])
    np.testing.assert_array_equal(r["v"], GOLDEN[f"{name}/v"])
    np.testing.assert_array_equal(r["aux"], GOLDEN[f"{name}/aux"])
    assert r["samples"] == int(GOLDEN[f"{name}/samples"][0])


@pytest.mark.gpu
@pytest.mark.parametrize("case", mg.CASES, ids=[c[0] for c in mg.CASES])
def test_gpu_matches_golden(ctx, case):
    import hydrant_gb300 as hy

    name, kind, n, bs, pad, params, arm, W, H = case
    vol = hy.Volume(ctx, mg.volume(kind, n), bs, pad)
    try:
        ctx.set_transfer_fn(mg.TF9)
        v = GOLDEN[f"{name}/view"]
        view = hy._abi.HyView()
        view.trans = (hy._abi.f16)(*v[:16])
        view.ctg_fovy_2 = float(v[16])
        view.ray_o = (hy._abi.f3)(*v[17:20])
        p = hy.shader_params(count_samples=True, **{k: val for k, val in params.items()})
        if p.shader == hy._abi.SHADER_ISOSURFACE:
            hy.iso_lighting(vol, hy.camera_orbit(arm), p)
        # with aux output, and without it (the Volume shader's lean march)
        for want_aux in (True, False):
            r = hy.render(ctx, vol, p, view, W, H, want_v=True, want_aux=want_aux)
            d8 = np.abs(r.rgba.astype(int) - GOLDEN[f"{name}/rgba"].astype(int)).max()
            assert d8 <= 1, f"aux={want_aux}: {d8} LSB"
            gv = GOLDEN[f"{name}/v"]
            assert np.abs(r.v - gv).max() <= 1e-4, f"aux={want_aux}"
            assert r.samples == int(GOLDEN[f"{name}/samples"][0]), f"aux={want_aux}"
    finally:
        vol.close()
