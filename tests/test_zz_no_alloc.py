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
