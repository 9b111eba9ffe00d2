"""The CPU side of the measurement builds its inputs without the product
library: the oracle's synthetic-volume generators and shader-parameter
builder must give the product's bytes exactly (CPU only: both generators and
the parameter structures are host code)."""

import ctypes as C

import numpy as np
import pytest

import hydrant_gb300 as hy
from oracle import oracle as orc


@pytest.mark.parametrize("gen,dims,count,seed", [
    ("blobs_u8", (40, 33, 27), 12, 0),
    ("blobs_u8", (64, 64, 64), 64, 3),
    ("blobs_f32", (30, 31, 29), 24, 4),
    ("tubes_u8", (48, 40, 56), 10, 2),
    ("tubes_u8", (64, 64, 64), 40, 1),
])
def test_oracle_generators_match_the_product(built_lib, gen, dims, count, seed):
    ours = {"blobs_u8": hy.synth_blobs_u8, "blobs_f32": hy.synth_blobs_f32,
            "tubes_u8": hy.synth_tubes_u8}[gen](seed, dims, count, 3)
    theirs = {"blobs_u8": orc.synth_blobs_u8, "blobs_f32": orc.synth_blobs_f32,
              "tubes_u8": orc.synth_tubes_u8}[gen](seed, dims, count, 5)
    assert ours.dtype == theirs.dtype and ours.shape == theirs.shape
    assert np.array_equal(ours.view(np.uint8), theirs.view(np.uint8))


@pytest.mark.parametrize("kw", [
    dict(),
    dict(shader="Volume", mode="Default", sample_rate=0.25, density=1e-2),
    dict(shader="Volume", mode="Partition", rank=0.3, composite=True, srgb=True),
    dict(shader="Blocks", mode="Solid", density=0.5, clear_color=(0.1, 0.2, 0.3)),
    dict(shader="Isosurface", mode="Normal", isovalue=0.25, surface_color=(0.5, 0.6, 0.7),
         count_samples=True, max_steps=77),
    dict(shader="Paging", lowest_blkcnt=12),
])
def test_oracle_params_match_the_product(kw):
    a = hy.shader_params(**kw)
    b = orc.shader_params(**kw)
    assert C.sizeof(a) == C.sizeof(b)
    assert C.string_at(C.addressof(a), C.sizeof(a)) == C.string_at(C.addressof(b), C.sizeof(b))
