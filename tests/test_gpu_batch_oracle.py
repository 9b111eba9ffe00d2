"""The batched kernels against the oracle, view by view.

The batch tests elsewhere compare the batch with the per-view GPU path; here
the persistent batch kernels themselves (the lean Volume march the benchmark
times, and per-brick compositing) face the oracle directly, on a downsized
multi-view workload: a 256^3 u8 volume of 64 Gaussian blobs in 64^3 bricks
with a 1-voxel apron (the compile-time brick edge P = 66 of the benchmark),
eight cameras on a seeded sphere at resolutions from 64^2 to 512^2, 1-voxel
steps, density 1e-2 and 0.5 (rays that get opaque take the adaptive steps).

Bar: RGBA8 within 1 LSB per channel (the Volume march is bit-exact in
practice, so the test also records the exact-pixel fraction) and the batch's
brick sample count equal to the oracle's sum over the views.
"""

import numpy as np
import pytest

import hydrant_gb300 as hy
from hydrant_gb300 import workloads as wl
from oracle import oracle as orc
from tests._harness import LSB_TOL, view_array

pytestmark = pytest.mark.gpu

RES = (64, 128, 256, 512)


@pytest.fixture(scope="module")
def c3_small(ctx):
    w = wl.multiview_c3(n=256, nviews=8, resolutions=RES)
    vox = w.voxels()
    vol = hy.Volume(ctx, vox, w.block_size, w.padding)
    ov = orc.OracleVolume(vox, w.block_size, w.padding)
    ctx.set_transfer_fn(w.tf)
    views = [(hy.camera_view(vol, wl.make_camera(v.camera)), v.width, v.height) for v in w.views]
    yield w, vol, ov, views
    vol.close()


def _oracle_views(w, ov, params, views):
    imgs, samples = [], 0
    op = orc.params_from(params)
    for view, W, H in views:
        r = orc.render(ov, w.tf, op, view_array(view), W, H, want_v=False, want_aux=False)
        imgs.append(r["rgba"])
        samples += r["samples"]
    return imgs, samples


def _compare(got, ref, what):
    exact = 0
    total = 0
    for i, (g, r) in enumerate(zip(got, ref)):
        d = np.abs(g.astype(np.int32) - r.astype(np.int32))
        assert d.max() <= LSB_TOL, f"{what}: view {i} max {d.max()} LSB"
        exact += int((d.max(axis=-1) == 0).sum())
        total += d.shape[0] * d.shape[1]
    return exact / total


@pytest.mark.parametrize("gather", [True, False], ids=["gathers", "loads"])
@pytest.mark.parametrize("kw", [
    dict(shader="Volume", mode="Default", sample_rate=0.25, density=1e-2),
    dict(shader="Volume", mode="Default", sample_rate=0.25, density=0.5),
    dict(shader="Volume", mode="Default", sample_rate=0.25, density=0.5, composite=True),
], ids=["lean", "lean_dense", "composite"])
def test_batch_matches_oracle(ctx, c3_small, kw, gather):
    """The lean march samples the bricks by texture gathers (the default for
    u8 bricks with an apron) or by loads; a batch takes the volume's setting
    when it is created."""
    w, vol, ov, views = c3_small
    assert vol.gather_sampling
    p = hy.shader_params(**kw)
    ref, ref_samples = _oracle_views(w, ov, p, views)
    vol.set_gather_sampling(gather)
    try:
        b = hy.Batch(ctx, vol, p, views)
    finally:
        vol.set_gather_sampling(True)
    try:
        b.set_counting(True)
        for cfg in [(8, 1, 4, 0, 1), (16, 2, 8, 0, 0), (8, 1, 4, 0, 1, 2)]:
            b.set_config(*cfg)
            got = b.render()
            assert ctx.stats().samples == ref_samples, cfg
            frac = _compare(got, ref, f"batch {kw} {cfg}")
            if not kw.get("composite"):
                assert frac == 1.0, f"{kw}: {frac:.6f} of the pixels bit-exact"
    finally:
        b.close()



def test_gather_sampling_where_it_applies(ctx):
    """Gather textures are built for u8 volumes with an apron and a brick
    column that fits a gather texture (P^2 rows: P = 202 does not); f32,
    apron-less and too-tall bricks sample by loads, and render as the oracle
    does.  Switching it off and on is honoured."""
    u8 = hy.Volume(ctx, hy.synth_blobs_u8(1, (70, 40, 50), 6), 16, 1)
    f32 = hy.Volume(ctx, hy.synth_blobs_f32(1, (40, 40, 40), 6), 16, 1)
    bare = hy.Volume(ctx, hy.synth_blobs_u8(1, (40, 40, 40), 6), 16, 0)
    big_vox = hy.synth_blobs_u8(2, (210, 60, 50), 6)
    big = hy.Volume(ctx, big_vox, 200, 1)
    try:
        assert u8.gather_sampling
        assert not f32.gather_sampling and not bare.gather_sampling and not big.gather_sampling
        ctx.set_transfer_fn(wl.TF9)
        ov = orc.OracleVolume(big_vox, 200, 1)
        p = hy.shader_params(shader="Volume", density=0.5, sample_rate=0.5)
        cam = wl.make_camera(wl.Camera("orbit", (30.0, 20.0, 2.4)))
        view = hy.camera_view(big, cam)
        b = hy.Batch(ctx, big, p, [(view, 40, 30)])
        try:
            got = b.render()[0]
        finally:
            b.close()
        ref = orc.render(ov, wl.TF9, orc.params_from(p), view_array(view), 40, 30)["rgba"]
        assert np.abs(got.astype(int) - ref.astype(int)).max() <= LSB_TOL
        u8.set_gather_sampling(False)
        assert not u8.gather_sampling
        u8.set_gather_sampling(True)
        assert u8.gather_sampling
    finally:
        for v in (u8, f32, bare, big):
            v.close()
