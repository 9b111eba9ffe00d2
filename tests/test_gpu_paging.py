"""Out-of-core path: brick store, visible-brick culling, lossless and realtime pagers.

Culling must give exactly the oracle's visible set and distances; the
lossless pager must reproduce the oracle replaying the same batches with
emit + march passes (holes included); the realtime pager must follow the
reference's replacement policy, simulated here on the host with the oracle's
culling, and render what the oracle renders with that resident set.
"""

import ctypes as C

import numpy as np
import pytest

import hydrant_gb300 as hy
from hydrant_gb300 import _abi
from hydrant_gb300 import workloads as wl
from oracle import oracle as orc
from tests._harness import view_array

pytestmark = pytest.mark.gpu


def cam10(c):
    return np.array(list(c.position) + list(c.target) + list(c.up) + [c.ctg_fovy_2], np.float32)


def write_to(v, clear=(0, 0, 0)):
    out = np.zeros(v.shape[:-1] + (4,), np.uint8)
    sat = lambda x: np.clip(x.astype(np.float32) * np.float32(255), 0, 255).astype(np.uint8)
    hit = v[..., 3] != 0
    for c in range(4):
        out[..., c] = np.where(hit, sat(v[..., c]), clear[c] if c < 3 else 0)
    return out


@pytest.fixture(scope="module")
def tubes(ctx):
    vox = hy.synth_tubes_u8(1, (128, 128, 128), 14)
    vol = hy.Volume(ctx, vox, 16, 1)
    ov = orc.OracleVolume(vox, 16, 1)
    ctx.set_transfer_fn(wl.TF9)
    store = hy.Store.from_volume(vol)
    yield vol, ov, store
    store.close()
    vol.close()


CAMS = [("orbit", (25, 65, 2.2)), ("orbit", (-110, 20, 1.8)), ("orbit", (60, -40, 3.0)),
        ("ptu", (0.2, 0.1, 0.3))]


@pytest.mark.parametrize("cam", CAMS)
@pytest.mark.parametrize("limit", [-1, 7, 60])
def test_cull_matches_oracle(tubes, cam, limit):
    vol, ov, _ = tubes
    c = wl.make_camera(wl.Camera(cam[0], cam[1]))
    view = hy.camera_view(vol, c)
    ids, d2 = hy.cull(vol, view, limit)
    oids, od2 = orc.cull(ov, view_array(view), limit)
    assert np.array_equal(ids, oids)
    assert np.array_equal(d2, od2)
    if limit < 0:
        assert len(ids) > 0


def test_store_holds_the_bricks(tubes):
    vol, ov, store = tubes
    cheb, mean = store.thumbnails()
    ocheb, omean = ov.thumbnails()
    assert np.array_equal(cheb, ocheb.ravel()) and np.array_equal(mean, omean.ravel())
    for b in [0, 7, 100, 511]:
        got = store.brick(b).astype(np.float32) / np.float32(255)
        if cheb[b] == 0:
            np.testing.assert_array_equal(got, ov.brick(b))
        else:
            assert not got.any()


def _oracle_lossless(ov, tf, op, c10, v20, W, H, B):
    ids, _ = orc.cull(ov, v20)
    order = orc.lossless_order(ov, c10, ids)
    batches = [order[i:i + B] for i in range(0, len(order), B)] or [order[:0]]
    film = None
    samples = 0
    for k, batch in enumerate(batches):
        ov.set_present(orc.present_mask(ov, batch))
        if k == 0:
            r = orc.render(ov, tf, op, v20, W, H, want_film=True)
            film = r["film"]
            samples += r["samples"]
        else:
            samples += orc.march_film(ov, tf, op, film, W, H)
    ov.set_present(np.ones(ov.grid[0] * ov.grid[1] * ov.grid[2], np.uint8))
    fb = film.shape[-1] // 4
    v = film.view(np.float32).reshape(H, W, fb)[..., 8:12]
    return write_to(v), len(batches), samples


@pytest.mark.parametrize("shader", ["Volume", "Isosurface", "Blocks"])
@pytest.mark.parametrize("slots", [25, 1000])
def test_lossless_pager_matches_oracle(ctx, tubes, shader, slots):
    torch = pytest.importorskip("torch")
    vol, ov, store = tubes
    pg = hy.Pager(ctx, store, slots, _abi.PAGER_LOSSLESS)
    try:
        W, H = 72, 56
        for cam in CAMS[:3]:
            c = wl.make_camera(wl.Camera(cam[0], cam[1]))
            p = hy.shader_params(shader=shader, density=0.4, sample_rate=0.5, isovalue=0.5,
                                 count_samples=True)
            if shader == "Isosurface":
                hy.iso_lighting(vol, c, p)
            out = torch.zeros(W * H * 4, dtype=torch.uint8, device="cuda")
            pg.render(p, c, W, H, out.data_ptr())
            ctx.synchronize()
            got = out.cpu().numpy().reshape(H, W, 4)
            view = view_array(hy.camera_view(vol, c))
            ref, nb, ref_samples = _oracle_lossless(ov, wl.TF9, orc.params_from(p), cam10(c), view,
                                                    W, H, slots)
            d = np.abs(got.astype(int) - ref.astype(int))
            assert d.max() <= 1, f"{shader} {cam}: {d.max()} LSB"
            # the frame's samples, summed over its passes, as in the batch replay
            assert ctx.stats().samples == ref_samples, f"{shader} {cam}: samples"
        st = pg.stats()
        if slots == 25:
            assert st["passes"] > st["frames"]  # several batches per frame
        assert st["uploads"] > 0
    finally:
        pg.close()


@pytest.mark.parametrize("policy", ["reference", "lru"])
@pytest.mark.parametrize("budget", [0, 9])
def test_realtime_pager_follows_its_policy(ctx, tubes, budget, policy):
    """A host replay of the replacement policy with the oracle's cull gives
    the pager's resident set frame by frame: the reference's redundant-set
    swap (highest brick index evicted first) or LRU (the brick visible least
    recently, ties by index); each frame equals the oracle given that set."""
    torch = pytest.importorskip("torch")
    vol, ov, store = tubes
    slots = 40
    ev = _abi.EVICT_REFERENCE if policy == "reference" else _abi.EVICT_LRU
    pg = hy.Pager(ctx, store, slots, _abi.PAGER_REALTIME, budget, ev)
    page, owner, next_free, stamp = {}, {}, 0, {}
    try:
        W, H = 64, 48
        for f in range(6):
            c = wl.make_camera(wl.Camera("orbit", (25 + 25 * f, 40, 2.2)))
            p = hy.shader_params(shader="Volume", density=0.4, sample_rate=0.5)
            out = torch.zeros(W * H * 4, dtype=torch.uint8, device="cuda")
            pg.render(p, c, W, H, out.data_ptr())
            ctx.synchronize()
            # host simulation of the replacement policy with the oracle's cull
            view = view_array(hy.camera_view(vol, c))
            ids, d2 = orc.cull(ov, view, slots)
            req = set(ids.tolist())
            for b in orc.cull(ov, view, -1)[0].tolist():  # visible resident: used now
                if b in page:
                    stamp[b] = f
            missing = sorted((float(d), int(b)) for b, d in zip(ids, d2) if int(b) not in page)
            if policy == "reference":
                redundant = sorted(b for b in page if b not in req)
            else:  # least recently visible at the end, ties: lowest index at the end
                redundant = sorted((b for b in page if b not in req),
                                   key=lambda b: (-stamp[b], -b))
            n = 0
            for _, b in missing:
                if budget and n >= budget:
                    break
                if next_free < slots:
                    slot = next_free
                    next_free += 1
                elif redundant:
                    old = redundant.pop()
                    slot = page.pop(old)
                else:
                    break
                page[b] = slot
                owner[slot] = b
                stamp[b] = f
                n += 1
            mask = orc.present_mask(ov, list(page))
            assert np.array_equal(pg.present(), mask), f"frame {f}: resident sets differ"
            ov.set_present(mask)
            ref = orc.render(ov, wl.TF9, orc.params_from(p), view, W, H)["rgba"]
            got = out.cpu().numpy().reshape(H, W, 4)
            assert np.abs(got.astype(int) - ref.astype(int)).max() <= 1, f"frame {f}"
        st = pg.stats()
        assert st["evictions"] > 0 and st["hits"] > 0
    finally:
        ov.set_present(np.ones(ov.grid[0] * ov.grid[1] * ov.grid[2], np.uint8))
        pg.close()


def test_noise_store(ctx):
    store = hy.Store.noise(ctx, (128, 128, 64), 32, 1, seed=2, cell_voxels=32.0, occupancy=0.15)
    try:
        info = store.info
        assert tuple(info.grid) == (4, 4, 2)
        cheb, mean = store.thumbnails()
        occ = []
        for b in range(info.nbricks):
            br = store.brick(b)
            core = br[1:33, 1:33, 1:33]
            assert (cheb[b] == 0) == bool(br.any())
            assert mean[b] == np.float32(core.astype(np.float64).sum() / 255.0 / 32 ** 3)
            occ.append((core > 0).mean())
        assert 0.08 < float(np.mean(occ)) < 0.25
    finally:
        store.close()


@pytest.fixture(scope="module")
def tubes_coarse(ctx):
    # 130^3 with 16^3 bricks: a ragged last brick; level 2 -> 33^3 coarse voxels,
    # 3^3 coarse bricks, each covering 4^3 fine bricks
    vox = hy.synth_tubes_u8(3, (130, 130, 130), 14)
    vol = hy.Volume(ctx, vox, 16, 1)
    ov = orc.OracleVolume(vox, 16, 1)
    ov.build_coarse(2)
    store = hy.Store.from_volume(vol)
    store.build_coarse(2)
    yield vol, ov, store
    store.close()
    vol.close()


def test_coarse_level_matches_oracle(tubes_coarse):
    _, ov, store = tubes_coarse
    g = store.coarse_grid
    assert g == (3, 3, 3)
    for cb in range(g[0] * g[1] * g[2]):
        got = store.coarse_brick(cb).astype(np.float32) / np.float32(255)
        np.testing.assert_array_equal(got, ov.coarse_brick(cb), err_msg=f"coarse brick {cb}")
    assert ov.lowest_blkcnt == 9 ** 3


@pytest.mark.parametrize("shader,mode", [("Volume", "Default"), ("Volume", "Paging"),
                                         ("Paging", "Default")])
def test_realtime_coarse_fallback_matches_oracle(ctx, tubes_coarse, shader, mode):
    """Absent bricks sample the coarse level instead of stopping the ray; the
    Paging mode colours coarse samples red and fine ones green."""
    torch = pytest.importorskip("torch")
    vol, ov, store = tubes_coarse
    ctx.set_transfer_fn(wl.TF9)
    pg = hy.Pager(ctx, store, 30, _abi.PAGER_REALTIME, 8)
    try:
        W, H = 64, 48
        nb = ov.grid[0] * ov.grid[1] * ov.grid[2]
        saw_fallback = False
        for f in range(5):
            c = wl.make_camera(wl.Camera("orbit", (20 + 30 * f, 35, 2.2)))
            p = hy.shader_params(shader=shader, mode=mode, density=0.4, sample_rate=0.5,
                                 count_samples=True)
            out = torch.zeros(W * H * 4, dtype=torch.uint8, device="cuda")
            pg.render(p, c, W, H, out.data_ptr())
            ctx.synchronize()
            st = pg.stats()
            saw_fallback |= st["fallback"] > 0
            ov.set_present(pg.present())
            op = orc.params_from(p)
            op.lowest_blkcnt = ov.lowest_blkcnt
            view = view_array(hy.camera_view(vol, c))
            ref = orc.render(ov, wl.TF9, op, view, W, H)
            got = out.cpu().numpy().reshape(H, W, 4)
            d = np.abs(got.astype(int) - ref["rgba"].astype(int))
            assert d.max() <= 1, f"frame {f}: {d.max()} LSB"
            if "Paging" in (shader, mode) and st["fallback"] > 0:
                assert (got[..., 0] > 0).any() and (got[..., 1] > 0).any()
        assert saw_fallback
    finally:
        ov.set_present(np.ones(nb, np.uint8))
        pg.close()


def test_store_save_open_round_trip(ctx, tubes_coarse, tmp_path):
    torch = pytest.importorskip("torch")
    vol, ov, store = tubes_coarse
    store.save(tmp_path / "ds")
    meta = (tmp_path / "ds" / "package_meta.json").read_text()
    assert '"sample_levels"' in meta and '"chebyshev"' in meta
    again = hy.Store.open(ctx, tmp_path / "ds")
    try:
        a, b = store.info, again.info
        assert tuple(a.grid) == tuple(b.grid) and a.nonempty == b.nonempty
        ca, ma = store.thumbnails()
        cb, mb = again.thumbnails()
        assert np.array_equal(ca, cb) and np.array_equal(ma, mb)
        for i in range(a.nbricks):
            assert np.array_equal(store.brick(i), again.brick(i))
        assert again.coarse_grid == store.coarse_grid
        for i in range(int(np.prod(store.coarse_grid))):
            assert np.array_equal(store.coarse_brick(i), again.coarse_brick(i))
        # the same frames from either store
        ctx.set_transfer_fn(wl.TF9)
        imgs = []
        for st in (store, again):
            pg = hy.Pager(ctx, st, 30, _abi.PAGER_REALTIME, 8)
            out = torch.zeros(48 * 40 * 4, dtype=torch.uint8, device="cuda")
            p = hy.shader_params(shader="Volume", density=0.4, sample_rate=0.5)
            pg.render(p, wl.make_camera(wl.Camera("orbit", (30, 30, 2.2))), 48, 40, out.data_ptr())
            ctx.synchronize()
            imgs.append(out.cpu().numpy())
            pg.close()
        assert np.array_equal(imgs[0], imgs[1])
    finally:
        again.close()


def test_store_open_rejects_damaged_dataset(ctx, tubes, tmp_path):
    _, _, store = tubes
    store.save(tmp_path / "ds")
    bricks = tmp_path / "ds" / "level0.bricks"
    data = bricks.read_bytes()
    bricks.write_bytes(data[:-1])
    with pytest.raises(hy.HydrantError):
        hy.Store.open(ctx, tmp_path / "ds")
    (tmp_path / "ds" / "package_meta.json").write_text('{"format": "something-else"}')
    with pytest.raises(hy.HydrantError):
        hy.Store.open(ctx, tmp_path / "ds")


@pytest.mark.parametrize("dtype", ["u8", "f32"])
def test_ingest_raw_equals_device_bricking(ctx, tmp_path, dtype):
    if dtype == "u8":
        vox = hy.synth_tubes_u8(5, (70, 45, 38), 9)
    else:
        vox = hy.synth_blobs_f32(6, (70, 45, 38), 8)
        vox[vox < 0.2] = 0.0  # some empty bricks
    raw = tmp_path / "vol.raw"
    vox.tofile(raw)
    vol = hy.Volume(ctx, vox, 16, 1)
    ref = hy.Store.from_volume(vol)
    got = hy.Store.ingest_raw(ctx, raw, (70, 45, 38), 16, 1,
                              _abi.DTYPE_U8 if dtype == "u8" else _abi.DTYPE_F32)
    try:
        assert got.info.nonempty == ref.info.nonempty > 0
        c0, m0 = ref.thumbnails()
        c1, m1 = got.thumbnails()
        assert np.array_equal(c0, c1)
        if dtype == "u8":
            assert np.array_equal(m0, m1)
        else:
            np.testing.assert_allclose(m1, m0, rtol=1e-6, atol=1e-7)
        npd = np.uint8 if dtype == "u8" else np.float32
        for b in range(got.info.nbricks):
            assert np.array_equal(ref.brick(b, npd), got.brick(b, npd)), f"brick {b}"
    finally:
        got.close()
        ref.close()
        vol.close()
    with pytest.raises(hy.HydrantError):
        hy.Store.ingest_raw(ctx, raw, (70, 45, 39), 16, 1)


def test_coarse_level_of_f32_store_matches_oracle(ctx):
    """f32 coarse voxels are the mean of their cube in double, rounded once."""
    vox = hy.synth_blobs_f32(8, (40, 36, 30), 6)
    vol = hy.Volume(ctx, vox, 8, 1)
    ov = orc.OracleVolume(vox, 8, 1)
    ov.build_coarse(1)
    store = hy.Store.from_volume(vol)
    try:
        store.build_coarse(1)
        g = store.coarse_grid
        assert g == (3, 3, 2)
        for cb in range(g[0] * g[1] * g[2]):
            np.testing.assert_array_equal(store.coarse_brick(cb, np.float32), ov.coarse_brick(cb),
                                          err_msg=f"coarse brick {cb}")
    finally:
        store.close()
        vol.close()


def test_realtime_pager_on_f32_store_matches_oracle(ctx):
    """An f32 dataset through the realtime pager with a coarse level and a
    cache too small for the view: resident bricks fine, the rest coarse."""
    torch = pytest.importorskip("torch")
    vox = hy.synth_blobs_f32(9, (64, 64, 64), 10)
    vol = hy.Volume(ctx, vox, 16, 1)
    ov = orc.OracleVolume(vox, 16, 1)
    ov.build_coarse(1)
    store = hy.Store.from_volume(vol)
    store.build_coarse(1)
    ctx.set_transfer_fn(wl.TF9)
    pg = hy.Pager(ctx, store, 12, _abi.PAGER_REALTIME, 5)
    nb = ov.grid[0] * ov.grid[1] * ov.grid[2]
    try:
        W, H = 56, 48
        for f in range(3):
            c = wl.make_camera(wl.Camera("orbit", (10 + 40 * f, 25, 2.0)))
            p = hy.shader_params(shader="Volume", density=0.5, sample_rate=0.5)
            out = torch.zeros(W * H * 4, dtype=torch.uint8, device="cuda")
            pg.render(p, c, W, H, out.data_ptr())
            ctx.synchronize()
            ov.set_present(pg.present())
            op = orc.params_from(p)
            op.lowest_blkcnt = ov.lowest_blkcnt
            ref = orc.render(ov, wl.TF9, op, view_array(hy.camera_view(vol, c)), W, H)["rgba"]
            got = out.cpu().numpy().reshape(H, W, 4)
            assert np.abs(got.astype(int) - ref.astype(int)).max() <= 1, f"frame {f}"
        assert pg.stats()["fallback"] > 0
    finally:
        ov.set_present(np.ones(nb, np.uint8))
        pg.close()
        store.close()
        vol.close()


def _three_clusters():
    """64^3 u8 volume in 8^3 bricks (apron 1): three clusters of 2x2x2
    non-empty bricks, A at bricks (0..1, 6..7, 6..7) (the highest brick
    indices), B at (0..1, 0..1, 0..1), C at (6..7, 0..1, 6..7); the values
    stay two voxels inside each cluster, so no neighbouring brick's apron
    sees them.  Returns the voxels and, per cluster, a camera (fovy 10) that
    sees that cluster alone."""
    n, bs = 64, 8
    vox = np.zeros((n, n, n), np.uint8)
    cams = {}
    for name, (cx, cy, cz) in {"A": (0, 6, 6), "B": (0, 0, 0), "C": (6, 0, 6)}.items():
        x0, y0, z0 = cx * bs, cy * bs, cz * bs
        vox[z0 + 2:z0 + 14, y0 + 2:y0 + 14, x0 + 2:x0 + 14] = 200
        c = (np.array([cx + 1, cy + 1, cz + 1]) / 8.0 - 0.5)
        cams[name] = (tuple(4.0 * c), tuple(c))
    return vox, cams


@pytest.mark.parametrize("policy", ["lru", "reference"])
def test_lru_keeps_a_revisited_brick(ctx, policy):
    """Frames see A, B, A, C, A with room for two clusters.  At C the cache
    must evict: LRU drops B (last seen two frames earlier), so the return to
    A hits every brick; the reference's policy drops A (the highest brick
    indices), so the return to A misses all eight."""
    torch = pytest.importorskip("torch")
    vox, cams = _three_clusters()
    vol = hy.Volume(ctx, vox, 8, 1)
    store = hy.Store.from_volume(vol)
    ov = orc.OracleVolume(vox, 8, 1)
    ev = _abi.EVICT_LRU if policy == "lru" else _abi.EVICT_REFERENCE
    pg = hy.Pager(ctx, store, 16, _abi.PAGER_REALTIME, 0, ev)
    try:
        ctx.set_transfer_fn(wl.TF9)
        p = hy.shader_params(shader="Volume", density=0.5, sample_rate=0.5)
        out = torch.zeros(32 * 32 * 4, dtype=torch.uint8, device="cuda")
        sets = {}
        for name, (pos, tgt) in cams.items():
            cam = hy.camera_ptu(pos, tgt, (0.0, 1.0, 0.0), 10.0)
            sets[name] = set(orc.cull(ov, view_array(hy.camera_view(vol, cam)), -1)[0].tolist())
            assert len(sets[name]) == 8, name
        misses = []
        for name in "ABACA":
            pos, tgt = cams[name]
            before = pg.stats()["misses"]
            pg.render(p, hy.camera_ptu(pos, tgt, (0.0, 1.0, 0.0), 10.0), 32, 32, out.data_ptr())
            ctx.synchronize()
            misses.append(pg.stats()["misses"] - before)
            if len(misses) == 4:  # after C
                present = set(np.nonzero(pg.present())[0].tolist())
                kept = "A" if policy == "lru" else "B"
                assert present == sets[kept] | sets["C"], policy
        assert misses[:4] == [8, 8, 0, 8]
        assert misses[4] == (0 if policy == "lru" else 8)
        assert pg.stats()["evictions"] == (8 if policy == "lru" else 16)
    finally:
        pg.close()
        store.close()
        vol.close()


def test_cache_size_from_the_camera_path(ctx):
    """hy_pager_tune_slots: the most bricks any camera of the path sees (8
    per cluster here) plus 10 %, capped by the byte budget."""
    vox, cams = _three_clusters()
    vol = hy.Volume(ctx, vox, 8, 1)
    store = hy.Store.from_volume(vol)
    try:
        path = [hy.camera_ptu(pos, tgt, (0.0, 1.0, 0.0), 10.0) for pos, tgt in cams.values()]
        slot = store.info.slot_bytes
        assert hy.Pager.tune_slots(ctx, store, path, 1 << 30) == (9, 8)
        assert hy.Pager.tune_slots(ctx, store, path, 3 * slot + 5) == (3, 8)
        wide = [hy.camera_orbit((30.0, 20.0, 2.5))]
        slots, most = hy.Pager.tune_slots(ctx, store, wide, 1 << 30)
        assert most == 24 and slots == 24  # never more than the store holds
        with pytest.raises(hy.HydrantError):
            hy.Pager.tune_slots(ctx, store, path, slot - 1)
    finally:
        store.close()
        vol.close()


@pytest.mark.parametrize("policy", ["lru", "reference"])
def test_prefetch_during_the_previous_frame(ctx, tubes, policy):
    """hy_pager_prefetch after every frame moves the next camera's bricks on
    the copy stream: each frame still equals the oracle given the resident
    set the pager reports (arrived bricks in, spare slots out), the render
    path misses fewer bricks than without prefetching, and frames stay
    right when the prediction is wrong (the path turns back)."""
    torch = pytest.importorskip("torch")
    vol, ov, store = tubes
    slots = 60
    ev = _abi.EVICT_LRU if policy == "lru" else _abi.EVICT_REFERENCE
    W, H = 48, 40
    p = hy.shader_params(shader="Volume", density=0.4, sample_rate=0.5)
    arms = [(20 + 12 * f, 35, 2.2) for f in range(8)] + [(80, 35, 2.2), (10, 35, 2.2)]

    def run(prefetch):
        pg = hy.Pager(ctx, store, slots, _abi.PAGER_REALTIME, 0, ev)
        out = torch.zeros(W * H * 4, dtype=torch.uint8, device="cuda")
        try:
            for f, arm in enumerate(arms):
                cam = hy.camera_orbit(arm)
                pg.render(p, cam, W, H, out.data_ptr())
                if prefetch and f + 1 < len(arms):
                    # the path's next camera, except a wrong guess near the end
                    guess = arms[f + 1] if f < 7 else (arm[0] + 12, 35, 2.2)
                    pg.prefetch(hy.camera_orbit(guess))
                ctx.synchronize()
                mask = pg.present()
                ov.set_present(mask)
                view = view_array(hy.camera_view(vol, cam))
                ref = orc.render(ov, wl.TF9, orc.params_from(p), view, W, H)["rgba"]
                got = out.cpu().numpy().reshape(H, W, 4)
                d = np.abs(got.astype(int) - ref.astype(int)).max()
                assert d <= 1, f"prefetch={prefetch} frame {f}: {d} LSB"
            return pg.stats()
        finally:
            ov.set_present(np.ones(ov.grid[0] * ov.grid[1] * ov.grid[2], np.uint8))
            pg.close()

    plain = run(False)
    pre = run(True)
    assert plain["prefetched"] == 0 and pre["prefetched"] > 0
    assert pre["misses"] < plain["misses"], (pre["misses"], plain["misses"])


def test_out_of_core_orbit_at_quarter_scale_matches_oracle(ctx):
    """The out-of-core configuration at a quarter of its edge: a
    1024x1024x512 noise volume (3 octaves, 64-voxel cells, 15 % occupancy)
    in 64^3 bricks with the level-3 coarse fallback, a realtime LRU cache of
    a third of the visible bricks, 512^2 frames along the orbit (+3 degrees
    per frame), density 5e-3.  The oracle holds the same volume (assembled
    from the store's bricks, its own bricking, thumbnails and coarse level
    must equal the store's) and renders every 8th row of the frames with the
    pager's resident set."""
    torch = pytest.importorskip("torch")
    dim, bs = (1024, 1024, 512), 64
    store = hy.Store.noise(ctx, dim, bs, 1, seed=2, cell_voxels=64.0, occupancy=0.15)
    try:
        store.build_coarse(3)
        info = store.info
        gx, gy, gz = info.grid
        raw = np.zeros((dim[2], dim[1], dim[0]), np.uint8)
        for b in range(info.nbricks):
            x, y, z = b % gx, (b // gx) % gy, b // (gx * gy)
            raw[z * bs:(z + 1) * bs, y * bs:(y + 1) * bs, x * bs:(x + 1) * bs] = \
                store.brick(b)[1:bs + 1, 1:bs + 1, 1:bs + 1]
        ov = orc.OracleVolume(raw, bs, 1)
        ov.build_coarse(3)
        del raw
        cheb, mean = store.thumbnails()
        ocheb, omean = ov.thumbnails()
        assert np.array_equal(cheb.reshape(-1), ocheb.reshape(-1))
        cg = store.coarse_grid
        for cb in range(0, cg[0] * cg[1] * cg[2], 7):
            got = store.coarse_brick(cb).astype(np.float32) / np.float32(255)
            np.testing.assert_array_equal(got, ov.coarse_brick(cb))
        ctx.set_transfer_fn(wl.TF9)
        res = 512
        path = [hy.camera_orbit((3.0 * f, 30.0, 2.2)) for f in range(6)]
        _, most = hy.Pager.tune_slots(ctx, store, path, 1 << 40)
        slots = max(16, most // 3)
        pg = hy.Pager(ctx, store, slots, _abi.PAGER_REALTIME, 0, _abi.EVICT_LRU)
        # the same cache in gather textures renders the same frames
        pgt = hy.Pager(ctx, store, slots, _abi.PAGER_REALTIME, 0, _abi.EVICT_LRU,
                       _abi.PAGER_GATHERS)
        p = hy.shader_params(shader="Volume", sample_rate=0.25, density=5e-3)
        out = torch.zeros(res * res * 4, dtype=torch.uint8, device="cuda")
        outt = torch.zeros(res * res * 4, dtype=torch.uint8, device="cuda")
        try:
            vol = pg.volume
            for f, cam in enumerate(path):
                pg.render(p, cam, res, res, out.data_ptr())
                pgt.render(p, cam, res, res, outt.data_ptr())
                if f + 1 < len(path):
                    pg.prefetch(path[f + 1])
                    pgt.prefetch(path[f + 1])
                ctx.synchronize()
                st = pg.stats()
                assert torch.equal(out, outt), f"frame {f}: gather cache differs"
                assert np.array_equal(pg.present(), pgt.present())
                stt = pgt.stats()
                assert (st["uploads"], st["evictions"], st["fallback"]) == \
                    (stt["uploads"], stt["evictions"], stt["fallback"])
                if f in (0, len(path) - 1):
                    assert st["fallback"] > 0  # the coarse level is in use
                    ov.set_present(pg.present())
                    op = orc.params_from(p)
                    op.lowest_blkcnt = ov.lowest_blkcnt
                    view = view_array(hy.camera_view(vol, cam))
                    ref = orc.render_row_step(ov, wl.TF9, op, view, res, res, 4, 8)["rgba"]
                    got = out.cpu().numpy().reshape(res, res, 4)
                    d = np.abs(got[4::8].astype(int) - ref[4::8].astype(int)).max()
                    assert d <= 1, f"frame {f}: {d} LSB"
                    assert got[4::8, :, 3].any()
        finally:
            ov.set_present(np.ones(gx * gy * gz, np.uint8))
            pg.close()
            pgt.close()
    finally:
        store.close()


@pytest.mark.parametrize("shader,mode", [("Volume", "Default"), ("Paging", "Default"),
                                         ("Blocks", "Volume")])
def test_gather_cache_matches_oracle(ctx, tubes_coarse, shader, mode):
    """A realtime cache held in gather textures (HY_PAGER_GATHERS): the
    frames, resident sets and counts equal the pool cache's along a path
    with evictions and the coarse fallback, and the oracle's given that
    resident set; the march samples fine and coarse bricks (each entry's own
    mapping) through the textures."""
    torch = pytest.importorskip("torch")
    vol, ov, store = tubes_coarse
    ctx.set_transfer_fn(wl.TF9)
    pl = hy.Pager(ctx, store, 30, _abi.PAGER_REALTIME, 8)
    pt = hy.Pager(ctx, store, 30, _abi.PAGER_REALTIME, 8, _abi.EVICT_LRU, _abi.PAGER_GATHERS)
    nb = ov.grid[0] * ov.grid[1] * ov.grid[2]
    try:
        W, H = 64, 48
        saw_fallback = False
        for f in range(6):
            c = wl.make_camera(wl.Camera("orbit", (20 + 30 * f, 35, 2.2)))
            p = hy.shader_params(shader=shader, mode=mode, density=0.4, sample_rate=0.5,
                                 count_samples=True)
            a = torch.zeros(W * H * 4, dtype=torch.uint8, device="cuda")
            b = torch.zeros(W * H * 4, dtype=torch.uint8, device="cuda")
            pl.render(p, c, W, H, a.data_ptr())
            sl = ctx.stats()
            pt.render(p, c, W, H, b.data_ptr())
            st = ctx.stats()
            ctx.synchronize()
            assert torch.equal(a, b), f"frame {f}"
            assert sl.samples == st.samples
            assert np.array_equal(pl.present(), pt.present())
            s1, s2 = pl.stats(), pt.stats()
            for k in ("uploads", "evictions", "hits", "misses", "fallback"):
                assert s1[k] == s2[k], k
            saw_fallback |= s2["fallback"] > 0
            ov.set_present(pt.present())
            op = orc.params_from(p)
            op.lowest_blkcnt = ov.lowest_blkcnt
            ref = orc.render(ov, wl.TF9, op, view_array(hy.camera_view(vol, c)), W, H)
            d = np.abs(b.cpu().numpy().reshape(H, W, 4).astype(int) - ref["rgba"].astype(int))
            assert d.max() <= 1, f"frame {f}: {d.max()} LSB"
        assert saw_fallback
    finally:
        ov.set_present(np.ones(nb, np.uint8))
        pl.close()
        pt.close()


def test_gather_cache_rejects_what_it_cannot_serve(ctx, tubes):
    """A cache in gather textures serves the lean Volume march and the
    shaders that read no voxels; the Isosurface shader, the Volume shader's
    other modes and compositing, film passes, batches on its volume and a
    lossless pager in textures are refused (HY_ERR_UNSUPPORTED) before any
    launch."""
    torch = pytest.importorskip("torch")
    vol, ov, store = tubes
    ctx.set_transfer_fn(wl.TF9)
    with pytest.raises(hy.HydrantError) as e:
        hy.Pager(ctx, store, 50, _abi.PAGER_LOSSLESS, 0, _abi.EVICT_LRU, _abi.PAGER_GATHERS)
    assert e.value.code == _abi.HY_ERR_UNSUPPORTED
    pg = hy.Pager(ctx, store, 200, _abi.PAGER_REALTIME, 0, _abi.EVICT_LRU, _abi.PAGER_GATHERS)
    try:
        cam = wl.make_camera(wl.Camera("orbit", (25, 65, 2.2)))
        out = torch.zeros(32 * 32 * 4, dtype=torch.uint8, device="cuda")
        for kw in (dict(shader="Isosurface", isovalue=0.5), dict(shader="Volume", mode="Paging"),
                   dict(shader="Volume", composite=True)):
            p = hy.shader_params(**kw)
            if kw["shader"] == "Isosurface":
                hy.iso_lighting(pg.volume, cam, p)
            with pytest.raises(hy.HydrantError) as e:
                pg.render(p, cam, 32, 32, out.data_ptr())
            assert e.value.code == _abi.HY_ERR_UNSUPPORTED
        p = hy.shader_params(shader="Volume", density=0.4)
        pg.render(p, cam, 32, 32, out.data_ptr())  # the lean march serves it
        view = hy.camera_view(pg.volume, cam)
        with pytest.raises(hy.HydrantError) as e:
            hy.Batch(ctx, pg.volume, p, [(view, 32, 32)])
        assert e.value.code == _abi.HY_ERR_UNSUPPORTED
        film = torch.zeros(32 * 32 * 64, dtype=torch.uint8, device="cuda")
        with pytest.raises(hy.HydrantError) as e:
            hy.shade_pass(ctx, pg.volume, p, _abi.PASS_RAY_EMIT, view, film.data_ptr(), 32, 32)
        assert e.value.code == _abi.HY_ERR_UNSUPPORTED
        arr = (_abi.HyBatchView * 1)()
        arr[0].view = view
        arr[0].width = arr[0].height = 32
        rc = hy.lib().hy_render_views_noalloc(ctx.handle, pg.volume.handle, C.byref(p), arr, 1,
                                              C.c_void_p(out.data_ptr()))
        assert rc == _abi.HY_ERR_UNSUPPORTED
        # the shaders that read no voxels are served
        pg.render(hy.shader_params(shader="Blocks", mode="Solid"), cam, 32, 32, out.data_ptr())
        ctx.synchronize()
    finally:
        pg.close()
