"""Batched multi-view rendering: identical images to the per-view path."""

import numpy as np
import pytest

import hydrant_gb300 as hy
from hydrant_gb300 import workloads as wl
from tests._harness import camera

pytestmark = pytest.mark.gpu

SIZES = [(64, 64), (37, 23), (128, 96), (16, 16), (96, 128), (1, 1), (200, 33)]


def _views(vol, sizes, seed=11):
    rng = wl.SplitMix64(seed)
    out, cams = [], []
    for W, H in sizes:
        arm = (rng.uniform(-180, 180), rng.uniform(-60, 60), rng.uniform(1.8, 3.0))
        cam = camera(a=arm)
        cams.append(cam)
        out.append((hy.camera_view(vol, cam), W, H))
    return out, cams


def _per_view(ctx, vol, kw, views, cams):
    imgs, samples = [], 0
    for (v, W, H), cam in zip(views, cams):
        p = hy.shader_params(count_samples=True, **kw)
        if p.shader == hy._abi.SHADER_ISOSURFACE:
            hy.iso_lighting(vol, cam, p)
        r = hy.render(ctx, vol, p, v, W, H)
        imgs.append(r.rgba)
        samples += r.samples
    return imgs, samples


def _lighting(vol, cams, kw):
    out = []
    for cam in cams:
        p = hy.shader_params(**kw)
        hy.iso_lighting(vol, cam, p)
        out.append((list(p.eye_pos), list(p.light_pos)))
    return out


@pytest.fixture(scope="module")
def tubes(ctx):
    vol = hy.Volume(ctx, hy.synth_tubes_u8(1, (128, 128, 128), 12), 32, 1)
    ctx.set_transfer_fn(wl.TF9)
    yield vol
    vol.close()


@pytest.mark.parametrize("kw", [
    dict(shader="Volume", density=0.5, sample_rate=0.5),
    dict(shader="Isosurface", mode="Color", isovalue=0.5),
    dict(shader="Blocks", mode="Volume", density=1e-2),
    dict(shader="Volume", density=0.5, composite=True),
    dict(shader="Isosurface", mode="Normal", composite=True),
    dict(shader="Paging"),
])
def test_batch_equals_per_view(ctx, tubes, kw):
    views, cams = _views(tubes, SIZES)
    ref, ref_samples = _per_view(ctx, tubes, kw, views, cams)
    p = hy.shader_params(**kw)
    light = None
    if p.shader == hy._abi.SHADER_ISOSURFACE:
        light = _lighting(tubes, cams, kw)
        hy.iso_lighting(tubes, cams[0], p)  # to_world of the volume
    b = hy.Batch(ctx, tubes, p, views, light)
    try:
        b.set_counting(True)
        for cfg in [(8, 1, 4, 0, 1), (4, 2, 2, 0, 0), (16, 4, 8, 0, 1), (32, 3, 1, 0, 0),
                    (8, 2, 4, 2, 1), (4, 1, 8, 0, 0),
                    (8, 2, 8, 2, 1), (4, 1, 6, 0, 1), (8, 1, 4, 0, 1, 2)]:
            b.set_config(*cfg)
            got = b.render()
            assert ctx.stats().samples == ref_samples
            for i, (g, r) in enumerate(zip(got, ref)):
                assert np.array_equal(g, r), f"view {i} differs with config {cfg}"
    finally:
        b.close()


def test_batch_autotune_and_graph_replay(ctx, tubes):
    torch = pytest.importorskip("torch")
    views, cams = _views(tubes, SIZES * 3, seed=5)
    kw = dict(shader="Volume", density=0.3, sample_rate=0.5)
    ref, _ = _per_view(ctx, tubes, kw, views, cams)
    b = hy.Batch(ctx, tubes, hy.shader_params(**kw), views)
    try:
        out = torch.empty(b.nbytes, dtype=torch.uint8, device="cuda")
        cfg = b.autotune(out.data_ptr(), reps=1)
        assert cfg.tile_w in (4, 8, 16) and cfg.grab in (1, 2, 4)
        for _ in range(3):  # graph replays
            out.zero_()
            b.render_device(out.data_ptr())
            ctx.synchronize()
            got = b.split(out.cpu().numpy())
            for g, r in zip(got, ref):
                assert np.array_equal(g, r)
    finally:
        b.close()


def test_batch_rejects_bad_input(ctx, tubes):
    with pytest.raises(hy.HydrantError):
        hy.Batch(ctx, tubes, hy.shader_params(shader="Volume"), [])
    views, _ = _views(tubes, [(8, 8)])
    b = hy.Batch(ctx, tubes, hy.shader_params(shader="Volume"), views)
    try:
        with pytest.raises(hy.HydrantError):
            b.set_config(tile_w=5)
    finally:
        b.close()


@pytest.fixture(scope="module")
def blobs_bs64(ctx):
    # 64^3 bricks + 1-voxel apron: the compile-time brick edge (P = 66) kernels
    vol = hy.Volume(ctx, hy.synth_blobs_u8(3, (150, 130, 140), 20), 64, 1)
    ctx.set_transfer_fn(wl.TF9)
    yield vol
    vol.close()


@pytest.mark.parametrize("mode", ["Default", "Partition", "Paging"])
def test_batch_equals_per_view_p66(ctx, blobs_bs64, mode):
    """Default mode runs the lean march (no theta / phi), the others the full
    one; both must give the per-view images and samples exactly."""
    kw = dict(shader="Volume", mode=mode, density=0.05, sample_rate=0.25, rank=0.3)
    views, cams = _views(blobs_bs64, SIZES, seed=17)
    ref, ref_samples = _per_view(ctx, blobs_bs64, kw, views, cams)
    b = hy.Batch(ctx, blobs_bs64, hy.shader_params(**kw), views)
    try:
        b.set_counting(True)
        for cfg in [(8, 1, 4, 0, 1), (8, 1, 8, 0, 0), (16, 2, 4, 0, 1), (8, 1, 4, 0, 1, 2)]:
            b.set_config(*cfg)
            got = b.render()
            assert ctx.stats().samples == ref_samples
            for i, (g, r) in enumerate(zip(got, ref)):
                assert np.array_equal(g, r), f"view {i} differs with config {cfg}"
    finally:
        b.close()


def test_batch_follows_the_transfer_function(ctx, tubes):
    """A batch renders with the context's current transfer function, also
    after hy_tf_set grew the table (a new device allocation) or shrank it."""
    torch = pytest.importorskip("torch")
    views, cams = _views(tubes, SIZES[:4], seed=23)
    kw = dict(shader="Volume", density=0.5, sample_rate=0.5)
    ctx.set_transfer_fn(wl.TF9)
    b = hy.Batch(ctx, tubes, hy.shader_params(**kw), views)
    try:
        out = torch.empty(b.nbytes, dtype=torch.uint8, device="cuda")
        rng = np.random.default_rng(4)
        for n in (300, 5, 9):  # larger than any earlier table, then smaller
            tf = rng.uniform(0, 1, (n, 4)).astype(np.float32)
            tf[0] = 0
            ctx.set_transfer_fn(tf)
            ref, _ = _per_view(ctx, tubes, kw, views, cams)
            b.render_device(out.data_ptr())
            ctx.synchronize()
            for g, r in zip(b.split(out.cpu().numpy()), ref):
                assert np.array_equal(g, r), f"{n} knots"
    finally:
        ctx.set_transfer_fn(wl.TF9)
        b.close()


def test_batch_renders_into_pinned_host_memory(ctx, tubes):
    """A pinned, mapped host buffer is written by the kernel directly (no
    staging copy): the bytes equal those rendered into pageable host memory
    and into device memory, and a second render into the same buffer (the
    graph replayed) again equals them."""
    torch = pytest.importorskip("torch")
    views, cams = _views(tubes, SIZES)
    p = hy.shader_params(shader="Volume", density=0.5, sample_rate=0.5)
    b = hy.Batch(ctx, tubes, p, views)
    try:
        pageable = np.concatenate([g.reshape(-1) for g in b.render()])
        dev = torch.empty(b.nbytes, dtype=torch.uint8, device="cuda:0")
        b.render_device(dev.data_ptr())
        torch.cuda.synchronize()
        pinned = torch.zeros(b.nbytes, dtype=torch.uint8, pin_memory=True)
        for _ in range(2):
            pinned.zero_()
            ctx.check(hy.lib().hy_batch_render(b.handle, hy._abi.C.c_void_p(pinned.data_ptr())))
            assert np.array_equal(pinned.numpy(), pageable)
        assert np.array_equal(dev.cpu().numpy(), pageable)
        assert pageable.any()
    finally:
        b.close()


def test_batch_takes_new_cameras_without_a_new_batch(ctx, tubes):
    """hy_batch_update_views: new ViewArgs and lighting for the same sizes are
    rendered by the same batch (its captured graph replayed), equal to the
    per-view path for the new cameras; an update that changes a size is
    refused."""
    torch = pytest.importorskip("torch")
    sizes = SIZES[:5]
    kw = dict(shader="Isosurface", mode="Color", isovalue=0.5)
    views_a, cams_a = _views(tubes, sizes, seed=3)
    views_b, cams_b = _views(tubes, sizes, seed=4)
    p = hy.shader_params(**kw)
    hy.iso_lighting(tubes, cams_a[0], p)
    b = hy.Batch(ctx, tubes, p, views_a, _lighting(tubes, cams_a, kw))
    try:
        out = torch.empty(b.nbytes, dtype=torch.uint8, device="cuda")
        for views, cams in ((views_b, cams_b), (views_a, cams_a), (views_b, cams_b)):
            ref, _ = _per_view(ctx, tubes, kw, views, cams)
            b.update_views(views, _lighting(tubes, cams, kw))
            out.zero_()
            b.render_device(out.data_ptr())
            ctx.synchronize()
            for g, r in zip(b.split(out.cpu().numpy()), ref):
                assert np.array_equal(g, r)
        bad = b.view_array(views_a)
        bad[1].width = bad[1].width + 1
        with pytest.raises(hy.HydrantError):
            b.update_views(bad)
        assert b.view_bytes > 0
    finally:
        b.close()
