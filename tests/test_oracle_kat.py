"""Known-answer tests that pin the oracle (CPU only).

The reference has no tests and no golden vectors, and its path cannot be
built here, so the oracle is pinned by (a) a second, pure-Python float32
restatement on tiny volumes (tests/pyref.py) that must agree bit for bit,
and (b) analytic cases: empty and constant volumes, the last-knot lookup,
threshold and quantisation boundaries, the chebyshev transform against
brute force, and the isosurface prev_value quirk.
"""

import numpy as np
import pytest

from oracle import oracle as orc
from tests import pyref

F = np.float32

TF9 = [[0, 0, 0, 0], [1, 0, 0, 1], [1, 0.5, 0, 1], [1, 1, 0, 1], [0, 1, 0, 1], [0, 1, 1, 1],
       [0, 0, 1, 1], [1, 0, 1, 1], [0, 0, 0, 0]]


def params(**kw):
    p = orc.OrcParams()
    p.shader = kw.get("shader", 0)
    p.mode = kw.get("mode", 0)
    p.sample_rate = kw.get("sample_rate", 1.0)
    p.max_steps = kw.get("max_steps", 4000000)
    p.density = kw.get("density", 1.0)
    p.isovalue = kw.get("isovalue", 0.5)
    for i in range(3):
        p.surface_color[i] = 1.0
        p.clear_color[i] = kw.get("clear_color", (0, 0, 0))[i]
    p.composite = kw.get("composite", 0)
    p.srgb = kw.get("srgb", 0)
    p.count_samples = 1
    return p


def blob_volume(n=16, seed=0):
    rng = np.random.default_rng(seed)
    z, y, x = np.meshgrid(*(np.arange(n) + 0.5,) * 3, indexing="ij")
    v = np.zeros((n, n, n))
    for _ in range(4):
        c = rng.uniform(0.2, 0.8, 3) * n
        s = rng.uniform(0.1, 0.25) * n
        v += rng.uniform(60, 255) * np.exp(-((x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2) / (2 * s * s))
    return np.clip(np.round(v), 0, 255).astype(np.uint8)


@pytest.mark.parametrize("bs,pad,sr,density", [(16, 1, 1.0, 1.0), (8, 1, 0.5, 0.7), (8, 2, 0.25, 1.0)])
def test_oracle_matches_python_restatement(bs, pad, sr, density):
    vox = blob_volume(16, seed=bs + pad)
    ov = orc.OracleVolume(vox, bs, pad)
    pv = pyref.Vol(vox, bs, pad)
    cam = orc.camera_orbit((25, 65, 2.2))
    view = orc.camera_view(ov, cam)
    W, H = 12, 10
    r = orc.render(ov, TF9, params(sample_rate=sr, density=density), view, W, H, nthreads=2)
    total = 0
    for y in range(H):
        for x in range(W):
            v, theta, phi, n = pyref.volume_pixel(pv, TF9, view, x, y, W, H, F(sr), F(density))
            total += n
            np.testing.assert_array_equal(r["v"][y, x], np.array(v, np.float32))
            np.testing.assert_array_equal(r["aux"][y, x], np.array(theta + [phi], np.float32))
    assert r["samples"] == total and total > 0


def test_thumbnails_match_brute_force():
    rng = np.random.default_rng(7)
    vox = np.zeros((40, 36, 44), np.uint8)
    for _ in range(5):
        z, y, x = rng.integers(0, 36, 3)
        vox[z, y, x] = rng.integers(1, 255)
    ov = orc.OracleVolume(vox, 8, 1)
    pv = pyref.Vol(vox, 8, 1)
    cheb, mean = ov.thumbnails()
    for (bx, by, bz), d in pv.cheb.items():
        assert cheb[bz, by, bx] == d
    # mean: normalised core voxels
    gz, gy, gx = cheb.shape
    for bz in range(gz):
        for by in range(gy):
            for bx in range(gx):
                zs = np.clip(np.arange(8) + bz * 8, 0, 39)
                ys = np.clip(np.arange(8) + by * 8, 0, 35)
                xs = np.clip(np.arange(8) + bx * 8, 0, 43)
                core = vox[np.ix_(zs, ys, xs)].astype(np.float64)
                assert mean[bz, by, bx] == np.float32(core.sum() / 255.0 / 512.0)


def test_bricks_replicate_edges():
    vox = np.arange(6 * 5 * 4, dtype=np.uint8).reshape(6, 5, 4)
    ov = orc.OracleVolume(vox, 4, 1)
    b = ov.brick(0)  # brick (0,0,0), padded 6^3
    assert b.shape == (6, 6, 6)
    np.testing.assert_array_equal(b[1:5, 1:5, 1:5], vox[0:4, 0:4, 0:4] / np.float32(255))
    np.testing.assert_array_equal(b[0], b[1])  # z apron clamped at the border
    np.testing.assert_array_equal(b[5, 1:5, 1:5], vox[4, 0:4, 0:4] / np.float32(255))


def test_empty_volume_is_clear_colour():
    vox = np.zeros((16, 16, 16), np.uint8)
    ov = orc.OracleVolume(vox, 8, 1)
    view = orc.camera_view(ov, orc.camera_orbit((25, 65, 2.2)))
    r = orc.render(ov, TF9, params(clear_color=(0.2, 0.4, 1.0)), view, 16, 16)
    assert r["samples"] == 0
    assert np.all(r["rgba"][..., :3] == [51, 102, 255]) and np.all(r["rgba"][..., 3] == 0)


def test_constant_volume_analytic():
    # s = 1 everywhere -> the last knot; every sample adds the same alpha, so
    # v.rgb = c * v.a and v.a = 1 - (1 - a)^k for an integer k
    vox = np.full((16, 16, 16), 255, np.uint8)
    c = (0.25, 0.5, 0.75)
    alpha = 0.05
    tf = [[0, 0, 0, 0], [0, 0, 0, 0], [c[0], c[1], c[2], alpha]]
    ov = orc.OracleVolume(vox, 16, 1)
    view = orc.camera_view(ov, orc.camera_orbit((30, 40, 2.2)))
    r = orc.render(ov, tf, params(sample_rate=1.0), view, 24, 24)
    v = r["v"]
    hit = v[..., 3] > 0
    assert hit.sum() > 100
    for i in range(3):
        np.testing.assert_allclose(v[..., i][hit], c[i] * v[..., 3][hit], rtol=1e-5, atol=1e-6)
    k = np.log1p(-v[..., 3][hit].astype(np.float64)) / np.log1p(-alpha)
    assert np.abs(k - np.round(k)).max() < 1e-3


def test_adaptive_step_thresholds_are_double_comparisons():
    # float x > 0.93 (double)  <=>  x >= 0.93f ; same for 0.85 -- the kernels rely on it
    for t in (0.93, 0.85):
        lo = np.float32(t) - np.float32(1e-3)
        xs = np.arange(lo, np.float32(t) + np.float32(1e-3), dtype=np.float32)
        xs = np.concatenate([xs, np.nextafter(np.float32(t), np.float32(0)).reshape(1),
                             np.float32(t).reshape(1)])
        assert np.array_equal(xs.astype(np.float64) > t, xs >= np.float32(t))


def test_saturate_truncates():
    vox = np.full((8, 8, 8), 255, np.uint8)
    ov = orc.OracleVolume(vox, 8, 1)
    view = orc.camera_view(ov, orc.camera_orbit((0, 0, 2.5)))
    # one sample-worth of colour 0.999 at alpha 1 -> 254 (0.999*255 = 254.7, truncated)
    tf = [[0.999, 0.999, 0.999, 1.0]]
    r = orc.render(ov, tf, params(sample_rate=0.25), view, 4, 4)
    centre = r["rgba"][2, 2]
    assert tuple(centre) == (254, 254, 254, 255)


def test_miss_rays_keep_clear_colour():
    vox = blob_volume(16)
    ov = orc.OracleVolume(vox, 16, 1)
    # camera looking away from the volume
    cam = orc.camera_ptu((0, 0, 3.0), (0, 0, 6.0))
    view = orc.camera_view(ov, cam)
    r = orc.render(ov, TF9, params(clear_color=(0, 1, 0)), view, 8, 8)
    assert r["samples"] == 0 and np.all(r["rgba"][..., 1] == 255)


def test_skip_counts_match_python_restatement():
    # one non-empty brick in a corner: rays cross empty bricks with chebyshev skips
    vox = np.zeros((32, 32, 32), np.uint8)
    vox[26:30, 26:30, 26:30] = 200
    ov = orc.OracleVolume(vox, 8, 1)
    pv = pyref.Vol(vox, 8, 1)
    cheb, _ = ov.thumbnails()
    assert cheb.max() >= 3
    view = orc.camera_view(ov, orc.camera_orbit((-30, -20, 2.0)))
    W = H = 10
    r = orc.render(ov, TF9, params(sample_rate=0.5), view, W, H, nthreads=1)
    total = 0
    for y in range(H):
        for x in range(W):
            v, th, ph, n = pyref.volume_pixel(pv, TF9, view, x, y, W, H, F(0.5))
            total += n
            np.testing.assert_array_equal(r["v"][y, x], np.array(v, np.float32))
    assert r["samples"] == total


def test_isosurface_prev_value_quirk():
    # prev_value is never updated (isosurface_shader.cu:58), so the first sample
    # with sign(value - iso) != sign(0 - iso) is a hit -- including value == iso
    vox = np.full((16, 16, 16), 128, np.uint8)
    ov = orc.OracleVolume(vox, 16, 1)
    cam = orc.camera_orbit((20, 30, 2.2))
    view = orc.camera_view(ov, cam)
    p = params(shader=2, mode=2, isovalue=float(np.float32(128) / np.float32(255)))
    orc.iso_lighting(ov, cam, p)
    r = orc.render(ov, TF9, p, view, 8, 8)
    hit = np.isfinite(r["aux"][..., 0])
    assert hit.sum() > 10
    # every hit took exactly one march sample plus 6 gradient samples
    assert r["samples"] == 7 * hit.sum()


def test_composite_single_brick_equals_single_pass_box():
    # with one brick the per-brick segment is the whole box: composite == single pass
    vox = blob_volume(16)
    ov = orc.OracleVolume(vox, 16, 1)
    view = orc.camera_view(ov, orc.camera_orbit((25, 65, 2.2)))
    a = orc.render(ov, TF9, params(), view, 16, 16)
    b = orc.render(ov, TF9, params(composite=1), view, 16, 16)
    np.testing.assert_array_equal(a["v"], b["v"])
    assert a["samples"] == b["samples"]


def test_thread_count_does_not_change_result():
    vox = blob_volume(16)
    ov = orc.OracleVolume(vox, 8, 1)
    view = orc.camera_view(ov, orc.camera_orbit((25, 65, 2.2)))
    a = orc.render(ov, TF9, params(), view, 20, 17, nthreads=1)
    b = orc.render(ov, TF9, params(), view, 20, 17, nthreads=5)
    np.testing.assert_array_equal(a["v"], b["v"])
    np.testing.assert_array_equal(a["rgba"], b["rgba"])


def test_rows_subset_equals_full_render():
    vox = blob_volume(16)
    ov = orc.OracleVolume(vox, 8, 1)
    view = orc.camera_view(ov, orc.camera_orbit((25, 65, 2.2)))
    full = orc.render(ov, TF9, params(), view, 16, 16)
    part = orc.render(ov, TF9, params(), view, 16, 16, rows=(5, 9))
    np.testing.assert_array_equal(full["v"][5:9], part["v"][5:9])


def test_fp64_gradient_matches_central_differences():
    """The oracle's FP64 analytic gradient of the differentiable march (TF
    knots and voxels) against central finite differences, eps 1e-3."""
    n, W, H = 16, 12, 12
    rng = np.random.default_rng(11)
    z, y, x = np.meshgrid(*(np.arange(n) + 0.5,) * 3, indexing="ij")
    vol = np.zeros((n, n, n))
    for _ in range(3):
        c = rng.uniform(0.3, 0.7, 3) * n
        s = rng.uniform(0.15, 0.3) * n
        vol += rng.uniform(0.3, 0.7) * np.exp(-((x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2) / (2 * s * s))
    vol = np.clip(vol, 0, 1)
    ov = orc.OracleVolume(vol.astype(np.float32), n, 1)
    views = np.stack([orc.camera_view(ov, orc.camera_orbit(a)) for a in [(20, 30, 2.2), (-70, -10, 2.4)]])
    ntf = 8
    tf_true = rng.uniform(0, 1, (ntf, 4))
    tf_true[0] = 0
    tf = np.full((ntf, 4), 0.5)
    _, target, _, _ = orc.diff_loss_grad64(vol * 0.9, tf_true, views, W, H, grad=False)
    _, _, dv, dt = orc.diff_loss_grad64(vol, tf, views, W, H, target)
    eps = 1e-3

    def loss(v, t):
        return orc.diff_loss_grad64(v, t, views, W, H, target, grad=False)[0]

    for i in range(ntf):
        for c in range(4):
            tp, tm = tf.copy(), tf.copy()
            tp[i, c] += eps
            tm[i, c] -= eps
            fd = (loss(vol, tp) - loss(vol, tm)) / (2 * eps)
            assert abs(fd - dt[i, c]) <= 1e-3 * max(abs(fd), 1e-2 * np.abs(dt).max()), (i, c, fd, dt[i, c])
    for f in np.argsort(np.abs(dv).ravel())[-8:]:
        vp, vm = vol.copy().ravel(), vol.copy().ravel()
        vp[f] += eps
        vm[f] -= eps
        fd = (loss(vp.reshape(vol.shape), tf) - loss(vm.reshape(vol.shape), tf)) / (2 * eps)
        g = dv.ravel()[f]
        assert abs(fd - g) <= 1e-3 * max(abs(fd), 1e-2 * np.abs(dv).max()), (f, fd, g)


@pytest.mark.parametrize("dims,bs,level", [((16, 16, 16), 8, 1), ((21, 18, 13), 8, 2),
                                          ((33, 17, 9), 4, 2)])
def test_coarse_level_is_rounded_box_mean(dims, bs, level):
    rng = np.random.default_rng(7)
    vox = rng.integers(0, 256, dims[::-1]).astype(np.uint8)
    ov = orc.OracleVolume(vox, bs, 1)
    ov.build_coarse(level)
    s = 1 << level
    cd = [-(-d // s) for d in dims]  # x, y, z
    ref = np.zeros(cd[::-1], np.int64)
    for Z in range(cd[2]):
        for Y in range(cd[1]):
            for X in range(cd[0]):
                blk = vox[Z * s:(Z + 1) * s, Y * s:(Y + 1) * s, X * s:(X + 1) * s].astype(np.int64)
                ref[Z, Y, X] = (blk.sum() + blk.size // 2) // blk.size
    cg = [-(-c // bs) for c in cd]
    P = bs + 2
    for cb in range(cg[0] * cg[1] * cg[2]):
        bx, by, bz = cb % cg[0], (cb // cg[0]) % cg[1], cb // (cg[0] * cg[1])
        idx = [np.clip(np.arange(P) + b * bs - 1, 0, c - 1) for b, c in zip((bx, by, bz), cd)]
        want = ref[np.ix_(idx[2], idx[1], idx[0])].astype(np.float32) / F(255)
        np.testing.assert_array_equal(ov.coarse_brick(cb), want)
    assert ov.lowest_blkcnt == ov.grid[0] * ov.grid[1] * ov.grid[2]


def test_coarse_fallback_of_constant_volume_equals_fine_render():
    # trilinear filtering of a constant is that constant at either level (up
    # to the rounding of x*(1-a) + x*a), so a frame with every brick absent
    # renders what the fine level does, with the same samples
    vox = np.full((32, 32, 32), 200, np.uint8)
    ov = orc.OracleVolume(vox, 8, 1)
    view = orc.camera_view(ov, orc.camera_orbit((30, 40, 2.2)))
    p = params(sample_rate=0.5, density=0.3)
    fine = orc.render(ov, TF9, p, view, 24, 24)
    ov.build_coarse(2)
    nb = ov.grid[0] * ov.grid[1] * ov.grid[2]
    ov.set_present(np.zeros(nb, np.uint8))
    p.lowest_blkcnt = ov.lowest_blkcnt
    coarse = orc.render(ov, TF9, p, view, 24, 24)
    assert coarse["samples"] == fine["samples"] > 0
    np.testing.assert_allclose(coarse["v"], fine["v"], rtol=0, atol=1e-6)
    # Paging mode: all samples from the coarse level are red
    p.mode = 2
    red = orc.render(ov, TF9, p, view, 24, 24)["v"]
    hit = red[..., 3] > 0
    assert hit.any() and not red[..., 1][hit].any() and (red[..., 0][hit] > 0).all()


def test_paging_shader_one_colour_per_brick():
    # a constant volume: every brick non-empty and resident (registry ids >= 0
    # = lowest_blkcnt), so each brick a ray enters adds green 0.5 once:
    # v.w = 1 - 0.5^k after k bricks, v.g = v.w, red and blue stay 0; the
    # ray stops once v.w > 0.95 (k = 5)
    vox = np.full((64, 64, 64), 100, np.uint8)
    ov = orc.OracleVolume(vox, 8, 1)
    view = orc.camera_view(ov, orc.camera_orbit((30, 40, 2.2)))
    p = params(shader=3)
    r = orc.render(ov, TF9, p, view, 32, 32)
    v = r["v"].astype(np.float64)
    hit = v[..., 3] > 0
    assert hit.sum() > 100
    assert not v[..., 0].any() and not v[..., 2].any()
    np.testing.assert_array_equal(v[..., 1], v[..., 3])
    allowed = {1 - 0.5 ** k for k in range(1, 6)}
    assert set(np.unique(v[..., 3][hit]).tolist()) <= allowed
    assert (v[..., 3] == 1 - 0.5 ** 5).any()
    # with a coarse level, absent bricks are red 0.2
    ov.build_coarse(1)
    ov.set_present(np.zeros(ov.grid[0] * ov.grid[1] * ov.grid[2], np.uint8))
    p.lowest_blkcnt = ov.lowest_blkcnt
    red = orc.render(ov, TF9, p, view, 32, 32)["v"]
    hit = red[..., 3] > 0
    assert hit.any() and not red[..., 1][hit].any()
    np.testing.assert_array_equal(red[..., 0], red[..., 3])
