"""ctypes view of include/hydrant_gb300.h and include/hydrant_gb300_synth.h.

The shared library is built in-tree (hydrant_gb300/build.py).  Loading fails
loudly when it is missing: there is no CPU fallback for the rendering path.
"""

from __future__ import annotations

import ctypes as C
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libhydrant_gb300.so"

HY_OK = 0
HY_ERR_INVALID = -1
HY_ERR_CUDA = -2
HY_ERR_OOM = -3
HY_ERR_TIMEOUT = -4
HY_ERR_UNSUPPORTED = -5
HY_ERR_STATE = -6

SHADER_VOLUME, SHADER_BLOCKS, SHADER_ISOSURFACE, SHADER_PAGING = 0, 1, 2, 3
VOLUME_DEFAULT, VOLUME_PARTITION, VOLUME_PAGING = 0, 1, 2
BLOCKS_VOLUME, BLOCKS_SOLID = 0, 1
ISO_COLOR, ISO_NORMAL, ISO_POSITION = 0, 1, 2
PASS_RAY_EMIT, PASS_RAY_MARCH, PASS_PIXEL, PASS_FETCH = 0, 1, 2, 3
DTYPE_U8, DTYPE_F32 = 0, 1

f3 = C.c_float * 3
f16 = C.c_float * 16
i3 = C.c_int32 * 3


class HyView(C.Structure):
    _fields_ = [("trans", f16), ("ctg_fovy_2", C.c_float), ("ray_o", f3)]


class HyCamera(C.Structure):
    _fields_ = [("position", f3), ("target", f3), ("up", f3), ("ctg_fovy_2", C.c_float)]


class HyShaderParams(C.Structure):
    _fields_ = [
        ("shader", C.c_int32),
        ("mode", C.c_int32),
        ("sample_rate", C.c_float),
        ("max_steps", C.c_int32),
        ("density", C.c_float),
        ("isovalue", C.c_float),
        ("surface_color", f3),
        ("clear_color", f3),
        ("rank", C.c_float),
        ("lowest_blkcnt", C.c_int32),
        ("to_world", f16),
        ("eye_pos", f3),
        ("light_pos", f3),
        ("composite", C.c_int32),
        ("srgb", C.c_int32),
        ("count_samples", C.c_int32),
        ("early_termination", C.c_float),
    ]


class HyVolumeDesc(C.Structure):
    _fields_ = [("dim", i3), ("block_size", C.c_int32), ("padding", C.c_int32), ("dtype", C.c_int32)]


class HyVolumeInfo(C.Structure):
    _fields_ = [
        ("grid", i3),
        ("nbricks", C.c_int32),
        ("nonempty", C.c_int32),
        ("resident", C.c_int32),
        ("padded", C.c_int32),
        ("slot_bytes", C.c_int64),
        ("pool_bytes", C.c_int64),
        ("bbox_max", f3),
    ]


class HyBatchView(C.Structure):
    _fields_ = [
        ("view", HyView),
        ("width", C.c_int32),
        ("height", C.c_int32),
        ("rgba_offset", C.c_int64),
        ("eye_pos", f3),
        ("light_pos", f3),
    ]


class HyBatchConfig(C.Structure):
    _fields_ = [
        ("tile_w", C.c_int32),
        ("grab", C.c_int32),
        ("block_warps", C.c_int32),
        ("blocks_per_sm", C.c_int32),
        ("block_queue", C.c_int32),
        ("steps_per_iter", C.c_int32),
    ]


PAGER_LOSSLESS, PAGER_REALTIME = 0, 1
EVICT_LRU = 0
EVICT_REFERENCE = 1
PAGER_LOADS, PAGER_GATHERS = 0, 1


class HyPagerDesc(C.Structure):
    _fields_ = [("slots", C.c_int32), ("mode", C.c_int32), ("max_uploads_per_frame", C.c_int32),
                ("eviction", C.c_int32), ("sampler", C.c_int32)]


class HyPagerStats(C.Structure):
    _fields_ = [(n, C.c_int64) for n in ("frames", "passes", "uploads", "upload_bytes", "hits",
                                         "misses", "evictions", "visible", "fallback",
                                         "prefetched")]


class HyDiffParams(C.Structure):
    _fields_ = [
        ("n", C.c_int32),
        ("sample_rate", C.c_float),
        ("max_steps", C.c_int32),
        ("density", C.c_float),
        ("ntf", C.c_int32),
        ("ckpt_k", C.c_int32),
    ]


class HyRenderStats(C.Structure):
    _fields_ = [("samples", C.c_int64), ("pixels", C.c_int64), ("ms", C.c_float)]


P = C.c_void_p
_PROTOS = {
    "hy_ctx_create": (C.c_int, [C.c_int, C.POINTER(P)]),
    "hy_ctx_destroy": (C.c_int, [P]),
    "hy_last_error": (C.c_char_p, [P]),
    "hy_ctx_synchronize": (C.c_int, [P]),
    "hy_ctx_stream": (P, [P]),
    "hy_render_stats_get": (C.c_int, [P, C.POINTER(HyRenderStats)]),
    "hy_tf_set": (C.c_int, [P, P, C.c_int32]),
    "hy_volume_create": (C.c_int, [P, C.POINTER(HyVolumeDesc), C.POINTER(P)]),
    "hy_volume_destroy": (C.c_int, [P]),
    "hy_volume_upload": (C.c_int, [P, P]),
    "hy_volume_get_info": (C.c_int, [P, C.POINTER(HyVolumeInfo)]),
    "hy_volume_thumbnails": (C.c_int, [P, P, P]),
    "hy_volume_set_gather_sampling": (C.c_int, [P, C.c_int32]),
    "hy_volume_gather_sampling": (C.c_int, [P, C.POINTER(C.c_int32)]),
    "hy_camera_orbit": (C.c_int, [P, P, C.c_float, C.POINTER(HyCamera)]),
    "hy_camera_ptu": (C.c_int, [P, P, P, C.c_float, C.POINTER(HyCamera)]),
    "hy_camera_view": (C.c_int, [P, C.POINTER(HyCamera), C.POINTER(HyView)]),
    "hy_iso_lighting": (C.c_int, [P, C.POINTER(HyCamera), C.POINTER(HyShaderParams)]),
    "hy_render": (
        C.c_int,
        [P, P, C.POINTER(HyShaderParams), C.POINTER(HyView), C.c_int32, C.c_int32, P, P, P],
    ),
    "hy_render_device": (
        C.c_int,
        [P, P, C.POINTER(HyShaderParams), C.POINTER(HyView), C.c_int32, C.c_int32, P, P, P],
    ),
    "hy_shade_pass": (
        C.c_int,
        [P, P, C.POINTER(HyShaderParams), C.c_int32, C.POINTER(HyView), P, C.c_int32, C.c_int32, P, P],
    ),
    "hy_batch_create": (
        C.c_int,
        [P, P, C.POINTER(HyShaderParams), C.POINTER(HyBatchView), C.c_int32, C.POINTER(P)],
    ),
    "hy_batch_destroy": (C.c_int, [P]),
    "hy_batch_output_bytes": (C.c_int, [P, C.POINTER(C.c_int64)]),
    "hy_batch_set_config": (C.c_int, [P, C.POINTER(HyBatchConfig)]),
    "hy_batch_get_config": (C.c_int, [P, C.POINTER(HyBatchConfig)]),
    "hy_batch_set_counting": (C.c_int, [P, C.c_int32]),
    "hy_batch_update_views": (C.c_int, [P, P, C.c_int32]),
    "hy_batch_view_bytes": (C.c_int, [P, C.POINTER(C.c_int64)]),
    "hy_batch_render_device": (C.c_int, [P, P]),
    "hy_batch_render": (C.c_int, [P, P]),
    "hy_batch_autotune": (C.c_int, [P, P, C.c_int32, C.POINTER(HyBatchConfig)]),
    "hy_render_views_noalloc": (
        C.c_int,
        [P, P, C.POINTER(HyShaderParams), C.POINTER(HyBatchView), C.c_int32, P],
    ),
    "hy_store_from_volume": (C.c_int, [P, C.POINTER(P)]),
    "hy_store_create_noise": (
        C.c_int, [P, C.POINTER(HyVolumeDesc), C.c_uint64, C.c_float, C.c_float, C.POINTER(P)]),
    "hy_store_destroy": (C.c_int, [P]),
    "hy_store_get_info": (C.c_int, [P, C.POINTER(HyVolumeInfo)]),
    "hy_store_thumbnails": (C.c_int, [P, P, P]),
    "hy_store_brick": (C.c_int, [P, C.c_int32, P]),
    "hy_store_build_coarse": (C.c_int, [P, C.c_int32]),
    "hy_store_coarse_grid": (C.c_int, [P, P]),
    "hy_store_coarse_brick": (C.c_int, [P, C.c_int32, P]),
    "hy_store_save": (C.c_int, [P, C.c_char_p]),
    "hy_store_open": (C.c_int, [P, C.c_char_p, C.POINTER(P)]),
    "hy_store_ingest_raw": (C.c_int, [P, C.c_char_p, C.POINTER(HyVolumeDesc), C.POINTER(P)]),
    "hy_cull": (C.c_int, [P, C.POINTER(HyView), P, C.c_int32, P, P, C.POINTER(C.c_int32)]),
    "hy_pager_create": (C.c_int, [P, P, C.POINTER(HyPagerDesc), C.POINTER(P)]),
    "hy_pager_tune_slots": (C.c_int, [P, P, P, C.c_int32, C.c_int64, C.POINTER(C.c_int32),
                                     C.POINTER(C.c_int32)]),
    "hy_pager_prefetch": (C.c_int, [P, C.POINTER(HyCamera)]),
    "hy_pager_destroy": (C.c_int, [P]),
    "hy_pager_volume": (C.c_int, [P, C.POINTER(P)]),
    "hy_pager_stats_get": (C.c_int, [P, C.POINTER(HyPagerStats)]),
    "hy_pager_present": (C.c_int, [P, P]),
    "hy_pager_render_host": (
        C.c_int, [P, C.POINTER(HyShaderParams), C.POINTER(HyCamera), C.c_int32, C.c_int32, P]),
    "hy_pager_render": (
        C.c_int, [P, C.POINTER(HyShaderParams), C.POINTER(HyCamera), C.c_int32, C.c_int32, P]),
    "hy_diff_ckpt_bytes": (
        C.c_int, [C.POINTER(HyDiffParams), C.c_int32, C.c_int32, C.c_int32, C.POINTER(C.c_int64)]),
    "hy_diff_forward": (
        C.c_int,
        [P, C.POINTER(HyDiffParams), P, P, C.POINTER(HyView), C.c_int32, C.c_int32, C.c_int32, P,
         P, P]),
    "hy_diff_backward": (
        C.c_int,
        [P, C.POINTER(HyDiffParams), P, P, C.POINTER(HyView), C.c_int32, C.c_int32, C.c_int32, P,
         P, P, P, P]),
    "hy_synth_blobs_u8": (C.c_int, [C.c_uint64, P, C.c_int32, P, C.c_int32]),
    "hy_synth_blobs_f32": (C.c_int, [C.c_uint64, P, C.c_int32, P, C.c_int32]),
    "hy_synth_tubes_u8": (C.c_int, [C.c_uint64, P, C.c_int32, P, C.c_int32]),
}

_lib = None


def lib() -> C.CDLL:
    """Load libhydrant_gb300.so, or raise if it has not been built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with hydrant_gb300.build.build() "
                "(there is no CPU fallback for the rendering path)"
            )
        l = C.CDLL(str(LIB_PATH))
        for name, (res, args) in _PROTOS.items():
            fn = getattr(l, name)
            fn.restype = res
            fn.argtypes = args
        _lib = l
    return _lib


class HydrantError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"hydrant_gb300 error {code}: {msg}")
        self.code = code


def check(rc: int, ctx=None) -> None:
    if rc != HY_OK:
        msg = ""
        if ctx is not None:
            raw = lib().hy_last_error(ctx)
            msg = raw.decode() if raw else ""
        raise HydrantError(rc, msg)
