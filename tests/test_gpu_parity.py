"""GPU parity: the CUDA path (through the C ABI) against the oracle.

Bar: <= 1 LSB per 8-bit RGBA channel, <= 1e-4 max abs on the
pre-quantisation floats, and the same number of brick samples (which pins
every skip / adaptive-step / termination decision of every ray).
"""

import numpy as np
import pytest

import hydrant_gb300 as hy
from hydrant_gb300 import workloads as wl
from oracle import oracle as orc
from tests._harness import Case, assert_parity, camera, view_array

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def blobs64(ctx):
    c = Case(ctx, hy.synth_blobs_u8(0, (64, 64, 64), 12), 64, 1)
    yield c
    c.close()


@pytest.fixture(scope="module")
def tubes128(ctx):
    c = Case(ctx, hy.synth_tubes_u8(1, (128, 128, 128), 12), 32, 1)
    yield c
    c.close()


@pytest.fixture(scope="module")
def c0(ctx):
    w = wl.volume_c0()
    c = Case(ctx, w.voxels(), w.block_size, w.padding, w.tf)
    yield c, w
    c.close()


def test_volume_c0_full(c0):
    c, w = c0
    v = w.views[0]
    g, r, _, _ = c.render_both(wl.make_camera(v.camera), v.width, v.height, **w.params)
    s = assert_parity(g, r, what="config 0")
    assert r["samples"] > 1_000_000
    print("config0", s)


@pytest.mark.parametrize("density", [1.0, 1e-2, 0.3])
def test_volume_density(blobs64, density):
    g, r, _, _ = blobs64.render_both(camera(), 96, 80, shader="Volume", sample_rate=0.25,
                                     density=density)
    assert_parity(g, r, what=f"density {density}")


@pytest.mark.parametrize("sample_rate", [1.0, 0.5, 2.0])
def test_volume_sample_rate(blobs64, sample_rate):
    g, r, _, _ = blobs64.render_both(camera(a=(10, 30, 2.0)), 64, 64, shader="Volume",
                                     sample_rate=sample_rate, density=1.0)
    assert_parity(g, r, what=f"sample_rate {sample_rate}")


@pytest.mark.parametrize("mode", ["Partition", "Paging"])
def test_volume_modes(blobs64, mode):
    g, r, _, _ = blobs64.render_both(camera(), 64, 48, shader="Volume", mode=mode,
                                     sample_rate=0.5, density=1.0, rank=0.25)
    assert_parity(g, r, what=mode)


def test_volume_multibrick(tubes128):
    g, r, _, _ = tubes128.render_both(camera(a=(40, 20, 2.5)), 128, 128, shader="Volume",
                                      sample_rate=0.5, density=0.5)
    assert_parity(g, r, what="multi-brick volume")


@pytest.mark.parametrize("mode", ["Volume", "Solid"])
def test_blocks(tubes128, mode):
    g, r, _, _ = tubes128.render_both(camera(), 128, 96, shader="Blocks", mode=mode,
                                      density=1e-2)
    assert_parity(g, r, what=f"blocks {mode}")


@pytest.mark.parametrize("mode", ["Color", "Normal", "Position"])
def test_isosurface(tubes128, mode):
    g, r, _, _ = tubes128.render_both(camera(a=(30, 50, 2.4)), 128, 128, shader="Isosurface",
                                      mode=mode, isovalue=0.5)
    assert_parity(g, r, what=f"iso {mode}")


@pytest.mark.parametrize("shader,mode", [("Volume", 0), ("Blocks", "Volume"), ("Blocks", "Solid"),
                                         ("Isosurface", "Color")])
def test_composite_per_brick(tubes128, shader, mode):
    kw = dict(shader=shader, mode=mode, composite=True, density=0.5 if shader == "Volume" else 1e-2,
              sample_rate=0.5)
    g, r, _, _ = tubes128.render_both(camera(a=(-35, 25, 2.3)), 96, 96, **kw)
    assert_parity(g, r, what=f"composite {shader}")


def test_volume_composite_srgb(tubes128):
    g, r, _, _ = tubes128.render_both(camera(), 64, 64, shader="Volume", composite=True, srgb=True,
                                      density=0.5)
    assert_parity(g, r, what="composite srgb")


def test_f32_volume(ctx):
    c = Case(ctx, hy.synth_blobs_f32(4, (48, 48, 48), 16), 16, 1)
    try:
        g, r, _, _ = c.render_both(camera(), 80, 64, shader="Volume", sample_rate=1.0, density=1.0)
        assert_parity(g, r, what="f32 volume")
        # isovalues of every sign: the crossing test compares against sign(0 - iso)
        for iso in (0.3, 0.0, -0.2):
            g, r, _, _ = c.render_both(camera(), 64, 64, shader="Isosurface", isovalue=iso)
            assert_parity(g, r, what=f"f32 iso {iso}")
    finally:
        c.close()


@pytest.mark.parametrize("dtype", ["u8", "f32"])
def test_unpadded_volume(ctx, dtype):
    """No apron: every sample goes through the wrapping, clamping sampler
    (a tap past the brick face wraps to the opposite face, as the reference's
    Wrap address mode does), in every shader."""
    vox = (hy.synth_tubes_u8(2, (48, 40, 56), 10) if dtype == "u8"
           else hy.synth_blobs_f32(5, (48, 40, 56), 14))
    c = Case(ctx, vox, 16, 0)
    try:
        for kw in (dict(shader="Volume", sample_rate=1.0, density=1.0),
                   dict(shader="Volume", sample_rate=0.5, density=0.3, composite=True),
                   dict(shader="Isosurface", isovalue=0.4),
                   dict(shader="Isosurface", isovalue=0.4, composite=True),
                   dict(shader="Blocks", mode="Volume", density=0.5)):
            g, r, _, _ = c.render_both(camera(a=(35, 20, 2.1)), 72, 56, **kw)
            assert_parity(g, r, what=f"unpadded {dtype} {kw}")
    finally:
        c.close()


@pytest.mark.parametrize("wh", [(1, 1), (37, 23), (17, 9), (300, 7)])
def test_ragged_resolutions(blobs64, wh):
    g, r, _, _ = blobs64.render_both(camera(), wh[0], wh[1], shader="Volume", density=1.0)
    assert_parity(g, r, what=f"{wh}")


def test_camera_inside_volume(tubes128):
    cam = camera("ptu", a=(0.1, -0.2, 0.15), target=(1.0, 0.3, -0.4))
    for shader in ("Volume", "Isosurface", "Blocks"):
        g, r, _, _ = tubes128.render_both(cam, 64, 64, shader=shader, density=0.2, sample_rate=0.5)
        assert_parity(g, r, what=f"inside {shader}")


def test_empty_volume_clear_colour(ctx):
    c = Case(ctx, np.zeros((40, 40, 40), np.uint8), 16, 1)
    try:
        g, r, _, _ = c.render_both(camera(), 32, 32, shader="Volume", clear_color=(0.2, 0.4, 0.6))
        assert_parity(g, r, what="empty")
        assert g.samples == 0
        assert np.all(g.rgba[..., :3] == [51, 102, 153]) and np.all(g.rgba[..., 3] == 0)
    finally:
        c.close()


def test_axis_aligned_rays(blobs64):
    # a camera on the z axis gives direction components of exactly 0 near the centre
    cam = camera("ptu", a=(0.0, 0.0, 2.0))
    g, r, _, _ = blobs64.render_both(cam, 33, 33, shader="Volume", density=1.0)
    assert_parity(g, r, what="axis aligned")


def test_camera_helpers_match_oracle(blobs64):
    for arm in [(25, 65, 2.2), (-120, 10, 3.0), (0, 0, 1.5)]:
        cam = camera(a=arm)
        o = orc.camera_orbit(arm)
        got = np.array(list(cam.position) + list(cam.target) + list(cam.up) + [cam.ctg_fovy_2])
        np.testing.assert_allclose(got, o, rtol=1e-6, atol=1e-6)
        v = view_array(hy.camera_view(blobs64.vol, cam))
        ov = orc.camera_view(blobs64.ov, o)
        np.testing.assert_allclose(v, ov, rtol=1e-5, atol=1e-6)


def _film_dtype(shader):
    return 48 if shader in ("Blocks", "Paging") else 64


@pytest.mark.parametrize("shader", ["Volume", "Blocks", "Isosurface", "Paging"])
def test_pass_level_film(tubes128, shader):
    """hy_shade_pass RAY_EMIT / PIXEL / FETCH on a reference-layout film."""
    torch = pytest.importorskip("torch")
    W, H = 48, 40
    cam = camera(a=(15, 35, 2.2))
    p = hy.shader_params(shader=shader, density=0.4, sample_rate=0.5)
    if shader == "Isosurface":
        hy.iso_lighting(tubes128.vol, cam, p)
    view = hy.camera_view(tubes128.vol, cam)
    fb = _film_dtype(shader)
    film = torch.zeros(H * W * fb, dtype=torch.uint8, device="cuda")
    dst = torch.zeros(H * W * 32, dtype=torch.uint8, device="cuda")
    ctx = tubes128.ctx
    hy.shade_pass(ctx, tubes128.vol, p, hy._abi.PASS_RAY_EMIT, view, film.data_ptr(), W, H)
    ctx.synchronize()
    ref = orc.render(tubes128.ov, tubes128.tf, orc.params_from(p), view_array(view), W, H,
                     want_film=True)
    got = film.cpu().numpy().reshape(H, W, fb)
    assert np.array_equal(got, ref["film"]), "emit film differs from the oracle"
    hy.shade_pass(ctx, tubes128.vol, p, hy._abi.PASS_PIXEL, None, film.data_ptr(), W, H,
                  dst.data_ptr(), clear_rgb=(0, 0, 0))
    ctx.synchronize()
    rgb = dst.cpu().numpy()[: H * W * 3].reshape(H, W, 3)
    assert np.array_equal(rgb, ref["rgba"][..., :3])
    if shader != "Blocks":
        hy.shade_pass(ctx, tubes128.vol, p, hy._abi.PASS_FETCH, None, film.data_ptr(), W, H,
                      dst.data_ptr())
        ctx.synchronize()
        fetched = dst.cpu().numpy()
        if shader == "Paging":  # uchar3 saturate(v)
            f = fetched[: H * W * 3].reshape(H, W, 3)
            sat = np.clip(ref["v"][..., :3] * np.float32(255), 0, 255).astype(np.uint8)
            np.testing.assert_array_equal(f, sat)
        elif shader == "Volume":
            f = fetched.view(np.float32)[: H * W * 8].reshape(H, W, 8)
            np.testing.assert_array_equal(f[..., 0:4], ref["aux"])       # theta, phi
            np.testing.assert_array_equal(f[..., 4:8], ref["v"])         # val
        else:
            f = fetched[: H * W * 8].reshape(H, W, 8)
            np.testing.assert_array_equal(f[..., :3], ref["rgba"][..., :3])
            depth = f[..., 4:8].copy().view(np.float32)[..., 0]
            np.testing.assert_array_equal(depth, ref["aux"][..., 0])


def test_tubes_c1_isosurface_full(ctx):
    w = wl.tubes_c1()
    c = Case(ctx, w.voxels(), w.block_size, w.padding)
    try:
        v = w.views[0]
        g, r, _, _ = c.render_both(wl.make_camera(v.camera), v.width, v.height, **w.params)
        assert_parity(g, r, what="config 1 isosurface")
        for mode in ("Volume", "Solid"):
            g, r, _, _ = c.render_both(wl.make_camera(v.camera), v.width, v.height,
                                       shader="Blocks", mode=mode, density=1e-2, composite=True)
            assert_parity(g, r, what=f"config 1 blocks {mode}")
    finally:
        c.close()


def test_paging_shader(tubes128, blobs64):
    """The paging debug view: one colour per brick entered, every brick of a
    resident volume is a fine one (green)."""
    for c, cam in ((tubes128, camera(a=(20, 30, 2.2))), (blobs64, camera())):
        g, r, _, _ = c.render_both(cam, 80, 64, shader="Paging")
        assert_parity(g, r, what="paging shader")
        assert g.rgba[..., 1].any() and not g.rgba[..., 0].any()
    with pytest.raises(hy.HydrantError):
        p = hy.shader_params(shader="Paging", composite=True)
        hy.render(tubes128.ctx, tubes128.vol, p, hy.camera_view(tubes128.vol, camera()), 8, 8)


def test_second_upload_is_rejected(ctx):
    vox = hy.synth_blobs_u8(0, (32, 32, 32), 4)
    vol = hy.Volume(ctx, vox, 16, 1)
    try:
        rc = hy.lib().hy_volume_upload(vol.handle, vox.ctypes.data_as(hy._abi.C.c_void_p))
        assert rc == hy._abi.HY_ERR_STATE
        # the volume still renders
        ctx.set_transfer_fn(wl.TF9)
        r = hy.render(ctx, vol, hy.shader_params(shader="Volume"), hy.camera_view(vol, camera()),
                      16, 16)
        assert r.rgba.shape == (16, 16, 4)
    finally:
        vol.close()


def test_resolution_limits(tubes128):
    """Sizes the launch grid cannot cover are refused before any launch; the
    context stays usable."""
    c = tubes128
    p = hy.shader_params(shader="Volume", sample_rate=0.25)
    view = hy.camera_view(c.vol, camera())
    # (host buffers stay small: the C side refuses these before any copy)
    for w, h in ((0, 8), (8, 0), (1, 65535 * 8 + 1)):
        with pytest.raises(hy.HydrantError):
            hy.render(c.ctx, c.vol, p, view, w, h)
    r = hy.render(c.ctx, c.vol, p, view, 8, 8)
    assert r.rgba.shape == (8, 8, 4)


def test_no_transfer_function_needed(ctx):
    """The Isosurface and Blocks shaders read no transfer function: a context
    that never set one renders them exactly as one that did (nothing is
    staged from an empty knot array); the Volume shader is refused there."""
    vox = hy.synth_tubes_u8(1, (64, 64, 64), 8)
    bare = hy.Context(0)
    vol_bare = hy.Volume(bare, vox, 32, 1)
    vol = hy.Volume(ctx, vox, 32, 1)
    try:
        for kw in (dict(shader="Isosurface", isovalue=0.5),
                   dict(shader="Isosurface", isovalue=0.5, composite=True),
                   dict(shader="Blocks", mode="Volume", density=0.5)):
            p = hy.shader_params(**kw)
            if kw["shader"] == "Isosurface":
                hy.iso_lighting(vol, camera(), p)
            a = hy.render(bare, vol_bare, p, hy.camera_view(vol_bare, camera()), 48, 40)
            b = hy.render(ctx, vol, p, hy.camera_view(vol, camera()), 48, 40)
            assert np.array_equal(a.rgba, b.rgba), kw
            assert a.rgba[..., 3].any(), kw
        with pytest.raises(hy.HydrantError):
            hy.render(bare, vol_bare, hy.shader_params(shader="Volume"),
                      hy.camera_view(vol_bare, camera()), 8, 8)
    finally:
        vol.close()
        vol_bare.close()
        bare.close()


def test_misaligned_device_buffers_are_refused(ctx, tubes128):
    """uchar4 / float4 outputs need 4- / 16-byte aligned device buffers; an
    entry point refuses a misaligned one before anything else.  Each call
    below also lacks its volume or parameters, so even without the check it
    would stop before launching anything."""
    torch = pytest.importorskip("torch")
    buf = torch.empty(1 << 16, dtype=torch.uint8, device="cuda:0")
    base = buf.data_ptr()
    lib, Cv = hy.lib(), hy._abi.C.c_void_p
    p = hy.shader_params(shader="Volume")
    view = hy.camera_view(tubes128.vol, camera())
    cases = [
        lambda: lib.hy_render_device(ctx.handle, None, hy._abi.C.byref(p), hy._abi.C.byref(view),
                                     8, 8, Cv(base + 2), None, None),
        lambda: lib.hy_render_device(ctx.handle, None, hy._abi.C.byref(p), hy._abi.C.byref(view),
                                     8, 8, Cv(base), Cv(base + 4096 + 8), None),
        lambda: lib.hy_shade_pass(ctx.handle, None, hy._abi.C.byref(p), hy._abi.PASS_RAY_EMIT,
                                  hy._abi.C.byref(view), Cv(base + 4), 8, 8, None, None),
        lambda: lib.hy_diff_forward(ctx.handle, None, Cv(base), Cv(base), hy._abi.C.byref(view), 1,
                                    8, 8, Cv(base + 4), Cv(base), Cv(base)),
    ]
    for call in cases:
        with pytest.raises(hy.HydrantError, match="misaligned"):
            ctx.check(call())
    # the context is intact
    r = hy.render(ctx, tubes128.vol, p, view, 8, 8)
    assert r.rgba.shape == (8, 8, 4)


def test_render_into_pinned_host_memory(tubes128):
    """hy_render writes pinned, mapped host buffers directly: RGBA, float and
    aux images equal those rendered into pageable host memory."""
    torch = pytest.importorskip("torch")
    c = tubes128
    p = hy.shader_params(shader="Volume", sample_rate=0.5, density=0.5)
    view = hy.camera_view(c.vol, camera())
    W, H = 40, 24
    ref = hy.render(c.ctx, c.vol, p, view, W, H, want_v=True, want_aux=True)
    rgba = torch.zeros(H * W * 4, dtype=torch.uint8, pin_memory=True)
    v = torch.zeros(H * W * 4, dtype=torch.float32, pin_memory=True)
    aux = torch.zeros(H * W * 4, dtype=torch.float32, pin_memory=True)
    Cv = hy._abi.C.c_void_p
    for pointers in ((rgba, v, aux), (rgba, None, None)):
        c.ctx.check(hy.lib().hy_render(c.ctx.handle, c.vol.handle, hy._abi.C.byref(p),
                                       hy._abi.C.byref(view), W, H,
                                       *[Cv(t.data_ptr()) if t is not None else None
                                         for t in pointers]))
        assert np.array_equal(rgba.numpy().reshape(H, W, 4), ref.rgba)
    assert np.array_equal(v.numpy().reshape(H, W, 4), ref.v)
    assert np.array_equal(aux.numpy().reshape(H, W, 4), ref.aux)
