"""hy_render_views_noalloc: the entry point that allocates nothing.

It exists for callers that may not allocate device memory while they render
(a host application that owns the GPU memory budget, a frame loop that cannot
pay for cudaMalloc/cudaFree mid-frame); its scratch is a fixed static device
array.  The test calls it through the C ABI twice in a row and compares both
results with the existing batched entry point on the same views.  This file
is collected last so that a run stopping at the first failure has already run
every other test; it also passes on its own in a fresh process.
"""

import ctypes as C

import numpy as np
import pytest

import hydrant_gb300 as hy
from hydrant_gb300 import _abi
from hydrant_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

SIZES = [(96, 64), (37, 23), (128, 128), (1, 1), (64, 100)]


def _setup(ctx, shader):
    vol = hy.Volume(ctx, hy.synth_tubes_u8(1, (96, 96, 96), 10), 32, 1)
    ctx.set_transfer_fn(wl.TF9)
    rng = wl.SplitMix64(17)
    views, arr_views, light = [], (_abi.HyBatchView * len(SIZES))(), []
    p = hy.shader_params(shader=shader, density=0.4, sample_rate=0.5, isovalue=0.5)
    off = 0
    for i, (W, H) in enumerate(SIZES):
        arm = (rng.uniform(-180, 180), rng.uniform(-50, 50), rng.uniform(1.9, 2.8))
        cam = hy.camera_orbit(arm)
        v = hy.camera_view(vol, cam)
        q = hy.shader_params(shader=shader)
        hy.iso_lighting(vol, cam, q)
        if i == 0:
            hy.iso_lighting(vol, cam, p)
        views.append((v, W, H))
        light.append((list(q.eye_pos), list(q.light_pos)))
        arr_views[i].view = v
        arr_views[i].width = W
        arr_views[i].height = H
        arr_views[i].rgba_offset = off
        arr_views[i].eye_pos = q.eye_pos
        arr_views[i].light_pos = q.light_pos
        off += W * H * 4
    return vol, p, views, light, arr_views, off


@pytest.mark.parametrize("shader", ["Volume", "Isosurface"])
def test_noalloc_matches_batch_entry_point(ctx, shader):
    torch = pytest.importorskip("torch")
    vol, p, views, light, arr, nbytes = _setup(ctx, shader)
    try:
        b = hy.Batch(ctx, vol, p, views, light if shader == "Isosurface" else None)
        ref = torch.zeros(nbytes, dtype=torch.uint8, device="cuda")
        b.render_device(ref.data_ptr())
        ctx.synchronize()
        expect = ref.cpu().numpy()
        b.close()
        for attempt in range(2):  # two calls in a row share the static scratch
            out = torch.full((nbytes,), 7, dtype=torch.uint8, device="cuda")
            rc = hy.lib().hy_render_views_noalloc(
                ctx.handle, vol.handle, C.byref(p), arr, len(SIZES), C.c_void_p(out.data_ptr()))
            ctx.check(rc)
            ctx.synchronize()
            got = out.cpu().numpy()
            d = np.abs(got.astype(np.int32) - expect.astype(np.int32))
            assert d.max() <= 1, f"call {attempt}: max diff {d.max()} LSB"
            assert np.array_equal(got, expect)
    finally:
        vol.close()


def test_noalloc_rejects_more_views_than_the_scratch_holds(ctx):
    vol, p, views, light, arr, nbytes = _setup(ctx, "Volume")
    try:
        big = (_abi.HyBatchView * 257)()
        for i in range(257):
            big[i] = arr[0]
        rc = hy.lib().hy_render_views_noalloc(ctx.handle, vol.handle, C.byref(p), big, 257,
                                              C.c_void_p(1 << 20))
        assert rc == _abi.HY_ERR_INVALID
        assert b"256" in hy.lib().hy_last_error(ctx.handle)
    finally:
        vol.close()


def _batch_views(views, offsets):
    arr = (_abi.HyBatchView * len(views))()
    for i, ((v, W, H), off) in enumerate(zip(views, offsets)):
        arr[i].view = v
        arr[i].width = W
        arr[i].height = H
        arr[i].rgba_offset = off
    return arr


def test_noalloc_matches_oracle(ctx):
    """The entry point runs the lean batch march the benchmark times: its
    images face the oracle directly (a 128^3 blob volume in 64^3 bricks with
    an apron, four cameras on a seeded sphere), twice in a row."""
    torch = pytest.importorskip("torch")
    from oracle import oracle as orc
    from tests._harness import view_array

    w = wl.multiview_c3(n=128, nviews=4, resolutions=(48, 96, 160))
    vox = w.voxels()
    vol = hy.Volume(ctx, vox, w.block_size, w.padding)
    ov = orc.OracleVolume(vox, w.block_size, w.padding)
    try:
        ctx.set_transfer_fn(w.tf)
        p = hy.shader_params(**w.params)
        views = [(hy.camera_view(vol, wl.make_camera(v.camera)), v.width, v.height)
                 for v in w.views]
        offsets = np.cumsum([0] + [W * H * 4 for _, W, H in views]).tolist()
        arr = _batch_views(views, offsets[:-1])
        refs = [orc.render(ov, w.tf, orc.params_from(p), view_array(v), W, H, want_v=False,
                           want_aux=False)["rgba"] for v, W, H in views]
        for attempt in range(2):
            out = torch.full((offsets[-1],), 3, dtype=torch.uint8, device="cuda")
            ctx.check(hy.lib().hy_render_views_noalloc(ctx.handle, vol.handle, C.byref(p), arr,
                                                       len(views), C.c_void_p(out.data_ptr())))
            ctx.synchronize()
            flat = out.cpu().numpy()
            for i, ((_, W, H), ref) in enumerate(zip(views, refs)):
                got = flat[offsets[i]:offsets[i] + W * H * 4].reshape(H, W, 4)
                d = np.abs(got.astype(np.int32) - ref.astype(np.int32)).max()
                assert d <= 1, f"call {attempt}, view {i}: {d} LSB"
    finally:
        vol.close()


def test_noalloc_at_the_view_limit(ctx):
    """256 views -- the most the static scratch holds, filling every
    descriptor slot and the largest shared-memory table of view starts --
    render as the batched entry point renders them."""
    torch = pytest.importorskip("torch")
    vol = hy.Volume(ctx, hy.synth_blobs_u8(6, (64, 64, 64), 8), 32, 1)
    try:
        ctx.set_transfer_fn(wl.TF9)
        rng = wl.SplitMix64(29)
        p = hy.shader_params(shader="Volume", density=0.5, sample_rate=0.5)
        views = []
        for i in range(256):
            arm = (rng.uniform(-180, 180), rng.uniform(-60, 60), rng.uniform(1.8, 2.6))
            views.append((hy.camera_view(vol, hy.camera_orbit(arm)), 8 + i % 5, 8 + i % 3))
        offsets = np.cumsum([0] + [W * H * 4 for _, W, H in views]).tolist()
        b = hy.Batch(ctx, vol, p, views)
        ref = torch.zeros(b.nbytes, dtype=torch.uint8, device="cuda")
        b.render_device(ref.data_ptr())
        ctx.synchronize()
        expect = ref.cpu().numpy()
        b.close()
        arr = _batch_views(views, offsets[:-1])
        for attempt in range(2):
            out = torch.full((offsets[-1],), 5, dtype=torch.uint8, device="cuda")
            ctx.check(hy.lib().hy_render_views_noalloc(ctx.handle, vol.handle, C.byref(p), arr,
                                                       256, C.c_void_p(out.data_ptr())))
            ctx.synchronize()
            assert np.array_equal(out.cpu().numpy(), expect), f"call {attempt}"
        assert expect.any()
    finally:
        vol.close()


def test_noalloc_refuses_a_capturing_stream(ctx):
    """The view descriptors are copied from the call's stack, so a captured
    copy would replay from a dead address: on a stream that is capturing the
    entry point returns HY_ERR_STATE and enqueues nothing (the capture is
    opened and closed through the driver API, relaxed mode, and the empty
    graph destroyed)."""
    cuda = C.CDLL("libcuda.so.1")
    vol, p, views, light, arr, nbytes = _setup(ctx, "Volume")
    try:
        ctx.synchronize()
        stream = C.c_void_p(ctx.stream)
        assert cuda.cuStreamBeginCapture_v2(stream, 2) == 0  # CU_STREAM_CAPTURE_MODE_RELAXED
        rc = hy.lib().hy_render_views_noalloc(ctx.handle, vol.handle, C.byref(p), arr, len(SIZES),
                                              C.c_void_p(1 << 20))
        graph = C.c_void_p()
        end = cuda.cuStreamEndCapture(stream, C.byref(graph))
        if graph.value:
            cuda.cuGraphDestroy(graph)
        assert end == 0
        assert rc == _abi.HY_ERR_STATE
        assert b"capturing" in hy.lib().hy_last_error(ctx.handle)
    finally:
        vol.close()
