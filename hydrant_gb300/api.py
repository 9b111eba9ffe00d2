"""Python handles over the C ABI: context, volume, camera, render calls."""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Optional, Sequence

import numpy as np

from . import _abi
from ._abi import (
    HyBatchConfig,
    HyBatchView,
    HyCamera,
    HyRenderStats,
    HyShaderParams,
    HyView,
    HyVolumeDesc,
    HyVolumeInfo,
    check,
    lib,
)

SHADERS = {"Volume": _abi.SHADER_VOLUME, "Blocks": _abi.SHADER_BLOCKS,
           "Isosurface": _abi.SHADER_ISOSURFACE, "Paging": _abi.SHADER_PAGING}
MODES = {
    _abi.SHADER_VOLUME: {"Default": 0, "Partition": 1, "Paging": 2},
    _abi.SHADER_BLOCKS: {"Volume": 0, "Solid": 1},
    _abi.SHADER_ISOSURFACE: {"Color": 0, "Normal": 1, "Position": 2},
    _abi.SHADER_PAGING: {"Default": 0},
}


def _ptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class Context:
    """One device, one stream (hy_ctx)."""

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        check(lib().hy_ctx_create(device, C.byref(h)))
        self.handle = h
        self.device = device

    def close(self) -> None:
        if self.handle:
            lib().hy_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):  # pragma: no cover - interpreter shutdown order varies
        try:
            self.close()
        except Exception:
            pass

    def check(self, rc: int) -> None:
        check(rc, self.handle)

    @property
    def stream(self) -> int:
        return int(lib().hy_ctx_stream(self.handle) or 0)

    def synchronize(self) -> None:
        self.check(lib().hy_ctx_synchronize(self.handle))

    def set_transfer_fn(self, knots) -> None:
        k = np.ascontiguousarray(np.asarray(knots, dtype=np.float32).reshape(-1, 4))
        self.check(lib().hy_tf_set(self.handle, _ptr(k), k.shape[0]))

    def stats(self) -> HyRenderStats:
        s = HyRenderStats()
        self.check(lib().hy_render_stats_get(self.handle, C.byref(s)))
        return s


class Volume:
    """A bricked volume resident on the device (hy_volume)."""

    def __init__(self, ctx: Context, voxels: np.ndarray, block_size: int, padding: int = 1):
        if voxels.ndim != 3:
            raise ValueError("voxels must be a (z, y, x) array")
        if voxels.dtype == np.uint8:
            dtype = _abi.DTYPE_U8
        elif voxels.dtype == np.float32:
            dtype = _abi.DTYPE_F32
        else:
            raise ValueError("voxels must be uint8 or float32")
        self.ctx = ctx
        nz, ny, nx = voxels.shape
        desc = HyVolumeDesc((nx, ny, nz), block_size, padding, dtype)
        h = C.c_void_p()
        ctx.check(lib().hy_volume_create(ctx.handle, C.byref(desc), C.byref(h)))
        self.handle = h
        self.desc = desc
        vox = np.ascontiguousarray(voxels)
        ctx.check(lib().hy_volume_upload(self.handle, _ptr(vox)))

    def close(self) -> None:
        if self.handle:
            lib().hy_volume_destroy(self.handle)
            self.handle = None

    @property
    def info(self) -> HyVolumeInfo:
        i = HyVolumeInfo()
        self.ctx.check(lib().hy_volume_get_info(self.handle, C.byref(i)))
        return i

    def set_gather_sampling(self, on: bool) -> None:
        """Volume march over u8 bricks with an apron: two texture gathers per
        sample (on, the default) or eight loads (off); same images."""
        self.ctx.check(lib().hy_volume_set_gather_sampling(self.handle, int(bool(on))))

    @property
    def gather_sampling(self) -> bool:
        """Whether renders of this volume use the gathers."""
        v = C.c_int32()
        self.ctx.check(lib().hy_volume_gather_sampling(self.handle, C.byref(v)))
        return bool(v.value)

    def thumbnails(self):
        i = self.info
        n = i.nbricks
        cheb = np.zeros(n, np.int32)
        mean = np.zeros(n, np.float32)
        self.ctx.check(lib().hy_volume_thumbnails(self.handle, _ptr(cheb), _ptr(mean)))
        shape = (i.grid[2], i.grid[1], i.grid[0])
        return cheb.reshape(shape), mean.reshape(shape)


def camera_orbit(arm: Sequence[float], center=(0.0, 0.0, 0.0), fovy: float = 60.0) -> HyCamera:
    cam = HyCamera()
    a = (C.c_float * 3)(*arm)
    c = (C.c_float * 3)(*center)
    check(lib().hy_camera_orbit(C.cast(a, C.c_void_p), C.cast(c, C.c_void_p), fovy, C.byref(cam)))
    return cam


def camera_ptu(position, target=(0.0, 0.0, 0.0), up=(0.0, 1.0, 0.0), fovy: float = 60.0) -> HyCamera:
    cam = HyCamera()
    p, t, u = ((C.c_float * 3)(*v) for v in (position, target, up))
    check(
        lib().hy_camera_ptu(
            C.cast(p, C.c_void_p), C.cast(t, C.c_void_p), C.cast(u, C.c_void_p), fovy, C.byref(cam)
        )
    )
    return cam


def camera_view(vol: Volume, cam: HyCamera) -> HyView:
    v = HyView()
    check(lib().hy_camera_view(vol.handle, C.byref(cam), C.byref(v)))
    return v


def shader_params(
    shader="Volume",
    mode=0,
    sample_rate: float = 1.0,
    max_steps: int = 4000000,
    density: float = 1.0,
    isovalue: float = 0.5,
    surface_color=(1.0, 1.0, 1.0),
    clear_color=(0.0, 0.0, 0.0),
    rank: float = 0.0,
    lowest_blkcnt: int = 0,
    composite: bool = False,
    srgb: bool = False,
    count_samples: bool = False,
    early_termination: float = 0.0,
) -> HyShaderParams:
    p = HyShaderParams()
    p.shader = SHADERS[shader] if isinstance(shader, str) else int(shader)
    p.mode = MODES[p.shader][mode] if isinstance(mode, str) else int(mode)
    p.sample_rate = sample_rate
    p.max_steps = max_steps
    p.density = density
    p.isovalue = isovalue
    p.surface_color = (C.c_float * 3)(*surface_color)
    p.clear_color = (C.c_float * 3)(*clear_color)
    p.rank = rank
    p.lowest_blkcnt = lowest_blkcnt
    p.composite = int(bool(composite))
    p.srgb = int(bool(srgb))
    p.count_samples = int(bool(count_samples))
    p.early_termination = early_termination
    return p


def iso_lighting(vol: Volume, cam: HyCamera, params: HyShaderParams) -> HyShaderParams:
    check(lib().hy_iso_lighting(vol.handle, C.byref(cam), C.byref(params)))
    return params


@dataclass
class RenderResult:
    rgba: np.ndarray
    v: Optional[np.ndarray] = None
    aux: Optional[np.ndarray] = None
    samples: int = -1
    ms: float = 0.0


def render(
    ctx: Context,
    vol: Volume,
    params: HyShaderParams,
    view: HyView,
    width: int,
    height: int,
    want_v: bool = False,
    want_aux: bool = False,
) -> RenderResult:
    """hy_render: host buffers in and out."""
    rgba = np.empty((height, width, 4), np.uint8)
    v = np.empty((height, width, 4), np.float32) if want_v else None
    aux = np.empty((height, width, 4), np.float32) if want_aux else None
    ctx.check(
        lib().hy_render(
            ctx.handle, vol.handle, C.byref(params), C.byref(view), width, height,
            _ptr(rgba), _ptr(v), _ptr(aux),
        )
    )
    st = ctx.stats()
    return RenderResult(rgba, v, aux, int(st.samples), float(st.ms))


def render_device(ctx: Context, vol: Volume, params: HyShaderParams, view: HyView, width: int,
                  height: int, rgba_ptr: int, v_ptr: int = 0, aux_ptr: int = 0) -> None:
    """hy_render_device: device pointers, asynchronous on the context stream."""
    ctx.check(
        lib().hy_render_device(
            ctx.handle, vol.handle, C.byref(params), C.byref(view), width, height,
            C.c_void_p(rgba_ptr), C.c_void_p(v_ptr or None), C.c_void_p(aux_ptr or None),
        )
    )


def shade_pass(ctx: Context, vol: Volume, params: HyShaderParams, pass_: int, view: Optional[HyView],
               film_ptr: int, width: int, height: int, dst_ptr: int = 0, clear_rgb=None) -> None:
    """hy_shade_pass: one reference-layout pass over a device film."""
    clear = None
    if clear_rgb is not None:
        clear = (C.c_uint8 * 3)(*clear_rgb)
    ctx.check(
        lib().hy_shade_pass(
            ctx.handle, vol.handle, C.byref(params), pass_,
            C.byref(view) if view is not None else None,
            C.c_void_p(film_ptr), width, height, C.c_void_p(dst_ptr or None),
            C.cast(clear, C.c_void_p) if clear is not None else None,
        )
    )


def synth_blobs_u8(seed: int, dim, nblobs: int, nthreads: int = 0) -> np.ndarray:
    nx, ny, nz = dim
    out = np.empty((nz, ny, nx), np.uint8)
    d = (C.c_int32 * 3)(nx, ny, nz)
    rc = lib().hy_synth_blobs_u8(seed, C.cast(d, C.c_void_p), nblobs, _ptr(out), nthreads)
    check(rc)
    return out


def synth_blobs_f32(seed: int, dim, nblobs: int, nthreads: int = 0) -> np.ndarray:
    nx, ny, nz = dim
    out = np.empty((nz, ny, nx), np.float32)
    d = (C.c_int32 * 3)(nx, ny, nz)
    check(lib().hy_synth_blobs_f32(seed, C.cast(d, C.c_void_p), nblobs, _ptr(out), nthreads))
    return out


def synth_tubes_u8(seed: int, dim, ntubes: int, nthreads: int = 0) -> np.ndarray:
    nx, ny, nz = dim
    out = np.empty((nz, ny, nx), np.uint8)
    d = (C.c_int32 * 3)(nx, ny, nz)
    check(lib().hy_synth_tubes_u8(seed, C.cast(d, C.c_void_p), ntubes, _ptr(out), nthreads))
    return out


class Batch:
    """Many views in one persistent launch replayed from a CUDA graph (hy_batch)."""

    def __init__(self, ctx: Context, vol: Volume, params: HyShaderParams, views, lighting=None):
        """views: list of (HyView, width, height); lighting: optional list of
        (eye_pos, light_pos) per view for the Isosurface shader."""
        self.ctx = ctx
        n = len(views)
        arr = (HyBatchView * n)()
        off = 0
        self.offsets = []
        self.sizes = []
        for i, (v, W, H) in enumerate(views):
            arr[i].view = v
            arr[i].width = W
            arr[i].height = H
            arr[i].rgba_offset = off
            if lighting is not None:
                arr[i].eye_pos = (C.c_float * 3)(*lighting[i][0])
                arr[i].light_pos = (C.c_float * 3)(*lighting[i][1])
            self.offsets.append(off)
            self.sizes.append((W, H))
            off += W * H * 4
        h = C.c_void_p()
        ctx.check(lib().hy_batch_create(ctx.handle, vol.handle, C.byref(params), arr, n, C.byref(h)))
        self.handle = h
        nb = C.c_int64()
        ctx.check(lib().hy_batch_output_bytes(self.handle, C.byref(nb)))
        self.nbytes = int(nb.value)
        ctx.check(lib().hy_batch_view_bytes(self.handle, C.byref(nb)))
        self.view_bytes = int(nb.value)

    def view_array(self, views, lighting=None):
        """hy_batch_view array of (HyView, W, H) views at this batch's offsets."""
        n = len(views)
        arr = (HyBatchView * n)()
        for i, (v, W, H) in enumerate(views):
            arr[i].view = v
            arr[i].width = W
            arr[i].height = H
            arr[i].rgba_offset = self.offsets[i]
            if lighting is not None:
                arr[i].eye_pos = (C.c_float * 3)(*lighting[i][0])
                arr[i].light_pos = (C.c_float * 3)(*lighting[i][1])
        return arr

    def update_views(self, views, lighting=None) -> None:
        """New cameras (same sizes) for the following renders."""
        arr = views if isinstance(views, C.Array) else self.view_array(views, lighting)
        self.ctx.check(lib().hy_batch_update_views(self.handle, arr, len(arr)))

    def close(self) -> None:
        if self.handle:
            lib().hy_batch_destroy(self.handle)
            self.handle = None

    @property
    def config(self) -> HyBatchConfig:
        c = HyBatchConfig()
        self.ctx.check(lib().hy_batch_get_config(self.handle, C.byref(c)))
        return c

    def set_config(self, tile_w=8, grab=1, block_warps=4, blocks_per_sm=0, block_queue=1,
                   steps_per_iter=1) -> None:
        c = HyBatchConfig(tile_w, grab, block_warps, blocks_per_sm, block_queue, steps_per_iter)
        self.ctx.check(lib().hy_batch_set_config(self.handle, C.byref(c)))

    def set_counting(self, on: bool) -> None:
        self.ctx.check(lib().hy_batch_set_counting(self.handle, int(bool(on))))

    def render_device(self, rgba_ptr: int) -> None:
        self.ctx.check(lib().hy_batch_render_device(self.handle, C.c_void_p(rgba_ptr)))

    def render(self) -> list:
        out = np.empty(self.nbytes, np.uint8)
        self.ctx.check(lib().hy_batch_render(self.handle, _ptr(out)))
        return self.split(out)

    def split(self, flat: np.ndarray) -> list:
        return [flat[o:o + W * H * 4].reshape(H, W, 4) for o, (W, H) in zip(self.offsets, self.sizes)]

    def autotune(self, rgba_ptr: int, reps: int = 3) -> HyBatchConfig:
        c = HyBatchConfig()
        self.ctx.check(lib().hy_batch_autotune(self.handle, C.c_void_p(rgba_ptr), reps, C.byref(c)))
        return c


def cull(vol, view: HyView, limit: int = -1, rect=None):
    """hy_cull: visible non-empty bricks (ids in index order, squared distances)."""
    n = vol.info.nbricks
    ids = np.zeros(n, np.int32)
    d2 = np.zeros(n, np.float32)
    k = C.c_int32()
    r = None if rect is None else np.ascontiguousarray(rect, np.float32)
    vol.ctx.check(lib().hy_cull(vol.handle, C.byref(view), _ptr(r), limit, _ptr(ids), _ptr(d2),
                                C.byref(k)))
    return ids[: k.value].copy(), d2[: k.value].copy()


class Store:
    """Pinned host brick store (hy_store)."""

    def __init__(self, ctx: Context, handle):
        self.ctx = ctx
        self.handle = handle

    @classmethod
    def from_volume(cls, vol: Volume) -> "Store":
        h = C.c_void_p()
        vol.ctx.check(lib().hy_store_from_volume(vol.handle, C.byref(h)))
        return cls(vol.ctx, h)

    @classmethod
    def noise(cls, ctx: Context, dim, block_size: int, padding: int, seed: int,
              cell_voxels: float, occupancy: float) -> "Store":
        desc = HyVolumeDesc(tuple(dim), block_size, padding, _abi.DTYPE_U8)
        h = C.c_void_p()
        ctx.check(lib().hy_store_create_noise(ctx.handle, C.byref(desc), seed, cell_voxels,
                                              occupancy, C.byref(h)))
        return cls(ctx, h)

    @classmethod
    def open(cls, ctx: Context, path) -> "Store":
        """Read a dataset directory written by save() (package_meta.json + bricks)."""
        h = C.c_void_p()
        ctx.check(lib().hy_store_open(ctx.handle, str(path).encode(), C.byref(h)))
        return cls(ctx, h)

    @classmethod
    def ingest_raw(cls, ctx: Context, path, dim, block_size: int, padding: int = 1,
                   dtype: int = _abi.DTYPE_U8) -> "Store":
        """Brick a raw volume file (x fastest) on the host."""
        desc = HyVolumeDesc(tuple(dim), block_size, padding, dtype)
        h = C.c_void_p()
        ctx.check(lib().hy_store_ingest_raw(ctx.handle, str(path).encode(), C.byref(desc),
                                            C.byref(h)))
        return cls(ctx, h)

    def save(self, path) -> None:
        self.ctx.check(lib().hy_store_save(self.handle, str(path).encode()))

    def close(self) -> None:
        if self.handle:
            lib().hy_store_destroy(self.handle)
            self.handle = None

    @property
    def info(self) -> HyVolumeInfo:
        i = HyVolumeInfo()
        self.ctx.check(lib().hy_store_get_info(self.handle, C.byref(i)))
        return i

    def thumbnails(self):
        i = self.info
        cheb = np.zeros(i.nbricks, np.int32)
        mean = np.zeros(i.nbricks, np.float32)
        self.ctx.check(lib().hy_store_thumbnails(self.handle, _ptr(cheb), _ptr(mean)))
        return cheb, mean

    def brick(self, b: int, dtype=np.uint8) -> np.ndarray:
        P = self.info.padded
        out = np.zeros(P ** 3, dtype)
        self.ctx.check(lib().hy_store_brick(self.handle, b, _ptr(out)))
        return out.reshape(P, P, P)

    def build_coarse(self, level: int) -> None:
        """Coarse level (2**level box filter) for the realtime pager's fallback."""
        self.ctx.check(lib().hy_store_build_coarse(self.handle, level))

    @property
    def coarse_grid(self):
        g = (C.c_int32 * 3)()
        self.ctx.check(lib().hy_store_coarse_grid(self.handle, g))
        return (g[0], g[1], g[2])

    def coarse_brick(self, b: int, dtype=np.uint8) -> np.ndarray:
        P = self.info.padded
        out = np.zeros(P ** 3, dtype)
        self.ctx.check(lib().hy_store_coarse_brick(self.handle, b, _ptr(out)))
        return out.reshape(P, P, P)


class _PagedVolume:
    """Non-owning view of a pager's volume, usable wherever a Volume is."""

    def __init__(self, ctx, handle):
        self.ctx = ctx
        self.handle = handle

    @property
    def info(self) -> HyVolumeInfo:
        i = HyVolumeInfo()
        self.ctx.check(lib().hy_volume_get_info(self.handle, C.byref(i)))
        return i


class Pager:
    """Brick cache kept filled from a Store (hy_pager)."""

    @staticmethod
    def tune_slots(ctx: Context, store: "Store", cams, budget_bytes: int):
        """hy_pager_tune_slots: (slots, most visible bricks) for a camera path."""
        arr = (HyCamera * len(cams))(*cams)
        slots, most = C.c_int32(), C.c_int32()
        ctx.check(lib().hy_pager_tune_slots(ctx.handle, store.handle, arr, len(cams),
                                            int(budget_bytes), C.byref(slots), C.byref(most)))
        return int(slots.value), int(most.value)

    def __init__(self, ctx: Context, store: Store, slots: int, mode: int = _abi.PAGER_REALTIME,
                 max_uploads_per_frame: int = 0, eviction: int = _abi.EVICT_LRU,
                 sampler: int = _abi.PAGER_LOADS):
        self.ctx = ctx
        d = _abi.HyPagerDesc(slots, mode, max_uploads_per_frame, eviction, sampler)
        h = C.c_void_p()
        ctx.check(lib().hy_pager_create(ctx.handle, store.handle, C.byref(d), C.byref(h)))
        self.handle = h
        vh = C.c_void_p()
        ctx.check(lib().hy_pager_volume(self.handle, C.byref(vh)))
        self.volume = _PagedVolume(ctx, vh)

    def close(self) -> None:
        if self.handle:
            lib().hy_pager_destroy(self.handle)
            self.handle = None

    def render(self, params: HyShaderParams, cam: HyCamera, width: int, height: int,
               rgba_ptr: int) -> None:
        self.ctx.check(lib().hy_pager_render(self.handle, C.byref(params), C.byref(cam), width,
                                             height, C.c_void_p(rgba_ptr)))

    def prefetch(self, next_cam: HyCamera) -> None:
        """hy_pager_prefetch: move the next camera's bricks during this frame."""
        self.ctx.check(lib().hy_pager_prefetch(self.handle, C.byref(next_cam)))

    def stats(self) -> dict:
        s = _abi.HyPagerStats()
        self.ctx.check(lib().hy_pager_stats_get(self.handle, C.byref(s)))
        return {n: int(getattr(s, n)) for n, _ in _abi.HyPagerStats._fields_}

    def present(self) -> np.ndarray:
        n = self.volume.info.nbricks
        m = np.zeros(n, np.uint8)
        self.ctx.check(lib().hy_pager_present(self.handle, _ptr(m)))
        return m
