"""Seeded random parity sweep: shader, mode, dtype, volume shape, brick size,
apron, sample rate, density, isovalue, camera, resolution and per-brick
compositing drawn at random, each GPU image compared with the oracle's.

The Volume, Blocks and Paging paths must match bit for bit (images, floats
and sample counts); the Isosurface path within the parity bar (its powf /
pow shading may differ in the last bit).  Every kernel instantiation the
draws reach is covered, so an arithmetic change that rounds differently in
one of them (a contracted multiply-add, a reordered sum) shows up here.
"""

import numpy as np
import pytest

import hydrant_gb300 as hy
from tests._harness import Case, assert_parity, camera

pytestmark = pytest.mark.gpu

N_CASES = 40
SEED = 20261203


def _draw(rng):
    shader = str(rng.choice(["Volume", "Volume", "Volume", "Isosurface", "Blocks", "Paging"]))
    kw = dict(shader=shader)
    if shader == "Volume":
        kw["mode"] = str(rng.choice(["Default", "Default", "Partition", "Paging"]))
        if kw["mode"] == "Partition":
            kw["rank"] = float(rng.uniform(0, 1))
        kw["density"] = float(rng.choice([1e-2, 0.3, 1.0]))
    elif shader == "Isosurface":
        kw["mode"] = str(rng.choice(["Color", "Normal", "Position"]))
        kw["isovalue"] = float(rng.uniform(0.1, 0.9))
    elif shader == "Blocks":
        kw["mode"] = str(rng.choice(["Volume", "Solid"]))
        kw["density"] = float(rng.choice([1e-2, 0.3]))
    kw["sample_rate"] = float(rng.choice([0.25, 0.5, 1.0, 2.0]))
    if shader != "Paging" and rng.random() < 0.3:
        kw["composite"] = True
    dtype = "f32" if rng.random() < 0.25 else "u8"
    dims = tuple(int(x) for x in rng.integers(20, 72, 3))
    bs = int(rng.choice([8, 16, 32, 64]))
    pad = int(rng.choice([0, 1, 1, 2]))
    if rng.random() < 0.15:  # a camera inside the volume
        cam = camera("ptu", a=tuple(rng.uniform(-0.3, 0.3, 3)),
                     target=tuple(rng.uniform(-1, 1, 3)))
    else:
        cam = camera(a=(float(rng.uniform(-180, 180)), float(rng.uniform(-80, 80)),
                        float(rng.uniform(1.3, 3.0))))
    W, H = (int(x) for x in rng.integers(8, 81, 2))
    return kw, dtype, dims, bs, pad, cam, W, H


def _volume(rng, dtype, dims):
    seed = int(rng.integers(0, 1 << 16))
    if dtype == "f32":
        return hy.synth_blobs_f32(seed, dims, 10)
    if rng.random() < 0.5:
        return hy.synth_tubes_u8(seed, dims, 8)
    return hy.synth_blobs_u8(seed, dims, 10)


@pytest.mark.parametrize("case", range(N_CASES))
def test_random_parity(ctx, case):
    rng = np.random.default_rng([SEED, case])
    kw, dtype, dims, bs, pad, cam, W, H = _draw(rng)
    c = Case(ctx, _volume(rng, dtype, dims), bs, pad)
    try:
        what = f"case {case}: {kw} {dtype} {dims} bs{bs} pad{pad} {W}x{H}"
        g, r, _, _ = c.render_both(cam, W, H, **kw)
        stats = assert_parity(g, r, what=what)
        if kw["shader"] != "Isosurface":
            assert stats["max_lsb"] == 0 and stats["max_abs"] == 0.0, f"{what}: {stats}"
    finally:
        c.close()
