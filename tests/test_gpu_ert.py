"""Opt-in early ray termination (hy_shader_params.early_termination).

The reference marches every ray to its exit (volume_shader.cu:43-79; its
opacity_threshold is commented out at volume_shader.cu:36).  With the opt-in
the lean march stops a warp once every ray in it has v.a >= t.  At
t = 1 - 2^-16 what the skipped samples would add stays below 1.5e-5 per
channel, so the images stay within the parity bar of the non-terminating
oracle (<= 1 LSB, <= 1e-4) while the march takes fewer samples on a volume
whose rays become opaque.  The reference's adaptive step (16 voxels once
v.a > 0.93) already makes the tail of an opaque ray cheap, so the samples
saved are a modest fraction (about 10 % on the dense tubes here).
"""

import numpy as np
import pytest

import hydrant_gb300 as hy
from hydrant_gb300 import workloads as wl
from oracle import oracle as orc
from tests._harness import Case, assert_parity, camera, view_array

pytestmark = pytest.mark.gpu

T = 1.0 - 2.0 ** -16


@pytest.fixture(scope="module")
def dense(ctx):
    c = Case(ctx, hy.synth_tubes_u8(1, (128, 128, 128), 40), 32, 1)
    yield c
    c.close()


def _oracle(case, p, view, W, H):
    return orc.render(case.ov, case.tf, orc.params_from(p), view_array(view), W, H)


def test_terminated_rays_stay_within_the_bar(dense):
    cam = camera(a=(30, 20, 2.0))
    W = H = 96
    view = hy.camera_view(dense.vol, cam)
    full = hy.shader_params(shader="Volume", sample_rate=0.5, density=1.0, count_samples=True)
    ert = hy.shader_params(shader="Volume", sample_rate=0.5, density=1.0, count_samples=True,
                           early_termination=T)
    r = _oracle(dense, full, view, W, H)
    g = hy.render(dense.ctx, dense.vol, ert, view, W, H, want_v=True)
    assert_parity(g, r, check_aux=False, check_samples=False, what="ert")
    assert (r["v"][..., 3] >= T).mean() > 0.2, "the case must have opaque rays"
    # rays past v.a = 0.93 already take 16-voxel steps, so what termination
    # leaves out is the tail of those strides (and only once a whole warp
    # is opaque): fewer samples, not a large fraction
    assert g.samples < r["samples"], (g.samples, r["samples"])


@pytest.mark.parametrize("gather", [True, False], ids=["gathers", "loads"])
def test_batch_terminates_too(ctx, dense, gather):
    views, refs, total = [], [], 0
    rng = wl.SplitMix64(41)
    full = hy.shader_params(shader="Volume", sample_rate=0.5, density=1.0)
    for W, H in ((64, 64), (96, 48), (33, 71)):
        cam = camera(a=(rng.uniform(-180, 180), rng.uniform(-50, 50), 2.0))
        v = hy.camera_view(dense.vol, cam)
        views.append((v, W, H))
        r = _oracle(dense, full, v, W, H)
        refs.append(r["rgba"])
        total += r["samples"]
    p = hy.shader_params(shader="Volume", sample_rate=0.5, density=1.0, early_termination=T)
    dense.vol.set_gather_sampling(gather)
    try:
        b = hy.Batch(ctx, dense.vol, p, views)
    finally:
        dense.vol.set_gather_sampling(True)
    try:
        b.set_counting(True)
        got = b.render()
        assert ctx.stats().samples < total
        for g, ref in zip(got, refs):
            assert np.abs(g.astype(int) - ref.astype(int)).max() <= 1
    finally:
        b.close()


def test_ignored_where_the_full_march_is_needed(dense):
    """Per-brick compositing and the Partition / Paging tints march every ray
    to its exit: the sample counts equal the oracle's."""
    cam = camera(a=(30, 20, 2.0))
    view = hy.camera_view(dense.vol, cam)
    for kw in (dict(composite=True), dict(mode="Partition", rank=0.5)):
        p = hy.shader_params(shader="Volume", sample_rate=0.5, density=1.0, count_samples=True,
                             early_termination=T, **kw)
        g = hy.render(dense.ctx, dense.vol, p, view, 48, 48, want_v=True)
        r = _oracle(dense, p, view, 48, 48)
        assert_parity(g, r, check_aux=False, what=f"ert ignored {kw}")


def test_out_of_range_threshold_is_refused(dense):
    view = hy.camera_view(dense.vol, camera())
    for t in (-0.5, 1.5, float("nan")):
        with pytest.raises(hy.HydrantError):
            hy.render(dense.ctx, dense.vol, hy.shader_params(shader="Volume", early_termination=t),
                      view, 8, 8)
