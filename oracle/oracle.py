"""ctypes wrapper of the oracle -- TEST INFRASTRUCTURE ONLY.

The oracle is a CPU restatement of Hydrant's CPU shading backend
(hy_oracle.cc).  Only tests/, __graft_entry__.smoke() and bench.py's CPU
baseline / reference arm load it, as the checker or as the timed CPU
baseline.  PARITY UNPINNED: no reference build and no reference golden
vectors exist for this path; see hy_oracle.h.
"""

from __future__ import annotations

import ctypes as C
from pathlib import Path
from typing import Optional

import numpy as np

from . import build as _build  # type: ignore[attr-defined]

f3 = C.c_float * 3
f16 = C.c_float * 16


class OrcParams(C.Structure):
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
        ("early_termination", C.c_float),  # ignored: the oracle marches every ray to its exit
    ]


P = C.c_void_p
_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        path = _build.build()
        l = C.CDLL(str(path))
        protos = {
            "orc_volume_create": (P, [P, C.c_int32, C.c_int32, C.c_int32, P]),
            "orc_volume_free": (None, [P]),
            "orc_volume_grid": (None, [P, P, P]),
            "orc_volume_thumbnails": (None, [P, P, P]),
            "orc_volume_set_present": (None, [P, P]),
            "orc_volume_brick": (None, [P, C.c_int32, P]),
            "orc_volume_build_coarse": (C.c_int, [P, C.c_int32]),
            "orc_volume_lowest_blkcnt": (C.c_int32, [P]),
            "orc_volume_coarse_brick": (None, [P, C.c_int32, P]),
            "orc_camera_orbit": (None, [P, P, C.c_float, P]),
            "orc_camera_ptu": (None, [P, P, P, C.c_float, P]),
            "orc_camera_view": (None, [P, P, P]),
            "orc_iso_lighting": (None, [P, P, C.POINTER(OrcParams)]),
            "orc_render": (C.c_int64, [P, P, C.c_int32, C.POINTER(OrcParams), P, C.c_int32, C.c_int32,
                                       C.c_int32, P, P, P, P]),
            "orc_render_rows": (C.c_int64, [P, P, C.c_int32, C.POINTER(OrcParams), P, C.c_int32,
                                            C.c_int32, C.c_int32, C.c_int32, C.c_int32, P, P, P, P]),
            "orc_march_film": (C.c_int64, [P, P, C.c_int32, C.POINTER(OrcParams), C.c_int32,
                                           C.c_int32, C.c_int32, P]),
            "orc_cull": (C.c_int32, [P, P, P, C.c_int32, P, P]),
            "orc_lossless_order": (None, [P, P, P, C.c_int32, P]),
            "orc_render_row_step": (C.c_int64, [P, P, C.c_int32, C.POINTER(OrcParams), P,
                                                C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                                C.c_int32, C.c_int32, P, P]),
            "orc_synth_blobs_u8": (C.c_int, [C.c_uint64, P, C.c_int32, P, C.c_int32]),
            "orc_synth_blobs_f32": (C.c_int, [C.c_uint64, P, C.c_int32, P, C.c_int32]),
            "orc_synth_tubes_u8": (C.c_int, [C.c_uint64, P, C.c_int32, P, C.c_int32]),
        }
        for name, (res, args) in protos.items():
            fn = getattr(l, name)
            fn.restype = res
            fn.argtypes = args
        _lib = l
    return _lib


def _p(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


SHADERS = {"Volume": 0, "Blocks": 1, "Isosurface": 2, "Paging": 3}
MODES = {0: {"Default": 0, "Partition": 1, "Paging": 2}, 1: {"Volume": 0, "Solid": 1},
         2: {"Color": 0, "Normal": 1, "Position": 2}, 3: {"Default": 0}}


def shader_params(shader="Volume", mode=0, sample_rate=1.0, max_steps=4000000, density=1.0,
                  isovalue=0.5, surface_color=(1.0, 1.0, 1.0), clear_color=(0.0, 0.0, 0.0),
                  rank=0.0, lowest_blkcnt=0, composite=False, srgb=False,
                  count_samples=False, early_termination=0.0) -> OrcParams:
    """Shader parameters by name, with the product's defaults (the CPU side
    of the measurement builds them without loading the product library;
    tests/test_oracle_synth.py holds the bytes equal)."""
    p = OrcParams()
    p.shader = SHADERS[shader] if isinstance(shader, str) else int(shader)
    p.mode = MODES[p.shader][mode] if isinstance(mode, str) else int(mode)
    p.sample_rate = sample_rate
    p.max_steps = max_steps
    p.density = density
    p.isovalue = isovalue
    p.surface_color = f3(*surface_color)
    p.clear_color = f3(*clear_color)
    p.rank = rank
    p.lowest_blkcnt = lowest_blkcnt
    p.composite = int(bool(composite))
    p.srgb = int(bool(srgb))
    p.count_samples = int(bool(count_samples))
    p.early_termination = early_termination
    return p


def _synth(fn, dtype, seed, dim, count, nthreads):
    nx, ny, nz = dim
    out = np.empty((nz, ny, nx), dtype)
    d = (C.c_int32 * 3)(nx, ny, nz)
    if fn(seed, C.cast(d, P), count, _p(out), nthreads) != 0:
        raise ValueError("bad synthetic volume arguments")
    return out


def synth_blobs_u8(seed, dim, count, nthreads=0):
    return _synth(lib().orc_synth_blobs_u8, np.uint8, seed, dim, count, nthreads)


def synth_blobs_f32(seed, dim, count, nthreads=0):
    return _synth(lib().orc_synth_blobs_f32, np.float32, seed, dim, count, nthreads)


def synth_tubes_u8(seed, dim, count, nthreads=0):
    return _synth(lib().orc_synth_tubes_u8, np.uint8, seed, dim, count, nthreads)


def workload_voxels(w, nthreads=0):
    """Voxels of a workload description (generator, seed, dims, count)."""
    fn = {"blobs_u8": synth_blobs_u8, "tubes_u8": synth_tubes_u8,
          "blobs_f32": synth_blobs_f32}[w.generator]
    return fn(w.seed, w.dim, w.count, nthreads)


def params_from(struct) -> OrcParams:
    """Copy a layout-identical ctypes parameter structure into OrcParams."""
    p = OrcParams()
    C.memmove(C.byref(p), C.byref(struct), C.sizeof(OrcParams))
    return p


class OracleVolume:
    def __init__(self, voxels: np.ndarray, block_size: int, padding: int = 1):
        vox = np.ascontiguousarray(voxels)
        dtype = {np.dtype(np.uint8): 0, np.dtype(np.float32): 1}[vox.dtype]
        nz, ny, nx = vox.shape
        dim = (C.c_int32 * 3)(nx, ny, nz)
        self.h = lib().orc_volume_create(C.cast(dim, P), block_size, padding, dtype, _p(vox))
        if not self.h:
            raise RuntimeError("orc_volume_create failed")
        self.block_size = block_size
        self.padding = padding
        g = (C.c_int32 * 3)()
        ne = C.c_int32()
        lib().orc_volume_grid(self.h, C.cast(g, P), C.byref(ne))
        self.grid = (g[0], g[1], g[2])
        self.nonempty = ne.value

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_volume_free(self.h)
            self.h = None

    def thumbnails(self):
        n = self.grid[0] * self.grid[1] * self.grid[2]
        cheb = np.zeros(n, np.int32)
        mean = np.zeros(n, np.float32)
        lib().orc_volume_thumbnails(self.h, _p(cheb), _p(mean))
        shape = (self.grid[2], self.grid[1], self.grid[0])
        return cheb.reshape(shape), mean.reshape(shape)

    def brick(self, i: int) -> np.ndarray:
        P_ = self.block_size + 2 * self.padding
        out = np.zeros(P_ ** 3, np.float32)
        lib().orc_volume_brick(self.h, i, _p(out))
        return out.reshape(P_, P_, P_)

    def set_present(self, mask: np.ndarray) -> None:
        m = np.ascontiguousarray(mask.astype(np.uint8).ravel())
        lib().orc_volume_set_present(self.h, _p(m))

    def build_coarse(self, level: int) -> None:
        """Coarse sample level: absent bricks then sample it (realtime paging)."""
        if lib().orc_volume_build_coarse(self.h, level) != 0:
            raise ValueError("block_size must be a multiple of 2**level")
        self.coarse_level = level

    @property
    def lowest_blkcnt(self) -> int:
        return int(lib().orc_volume_lowest_blkcnt(self.h))

    def coarse_brick(self, i: int) -> np.ndarray:
        P_ = self.block_size + 2 * self.padding
        out = np.zeros(P_ ** 3, np.float32)
        lib().orc_volume_coarse_brick(self.h, i, _p(out))
        return out.reshape(P_, P_, P_)


def camera_orbit(arm, center=(0.0, 0.0, 0.0), fovy=60.0) -> np.ndarray:
    out = np.zeros(10, np.float32)
    a = np.asarray(arm, np.float32)
    c = np.asarray(center, np.float32)
    lib().orc_camera_orbit(_p(a), _p(c), fovy, _p(out))
    return out


def camera_ptu(pos, target=(0.0, 0.0, 0.0), up=(0.0, 1.0, 0.0), fovy=60.0) -> np.ndarray:
    out = np.zeros(10, np.float32)
    arrs = [np.asarray(v, np.float32) for v in (pos, target, up)]
    lib().orc_camera_ptu(_p(arrs[0]), _p(arrs[1]), _p(arrs[2]), fovy, _p(out))
    return out


def camera_view(vol: OracleVolume, cam: np.ndarray) -> np.ndarray:
    out = np.zeros(20, np.float32)
    c = np.ascontiguousarray(cam, np.float32)
    lib().orc_camera_view(vol.h, _p(c), _p(out))
    return out


def iso_lighting(vol: OracleVolume, cam: np.ndarray, params: OrcParams) -> OrcParams:
    c = np.ascontiguousarray(cam, np.float32)
    lib().orc_iso_lighting(vol.h, _p(c), C.byref(params))
    return params


def render(vol: OracleVolume, tf, params: OrcParams, view: np.ndarray, width: int, height: int,
           nthreads: int = 0, want_v=True, want_aux=True, want_film=False, rows=None):
    tfa = np.ascontiguousarray(np.asarray(tf, np.float32).reshape(-1, 4))
    v = np.zeros((height, width, 4), np.float32) if want_v else None
    rgba = np.zeros((height, width, 4), np.uint8)
    aux = np.zeros((height, width, 4), np.float32) if want_aux else None
    fb = 48 if params.shader in (1, 3) else 64  # StdVec4Pixel films: Blocks, Paging
    film = np.zeros((height, width, fb), np.uint8) if want_film else None
    view = np.ascontiguousarray(view, np.float32)
    if rows is None:
        n = lib().orc_render(vol.h, _p(tfa), tfa.shape[0], C.byref(params), _p(view), width, height,
                             nthreads, _p(v), _p(rgba), _p(aux), _p(film))
    else:
        n = lib().orc_render_rows(vol.h, _p(tfa), tfa.shape[0], C.byref(params), _p(view), width,
                                  height, rows[0], rows[1], nthreads, _p(v), _p(rgba), _p(aux),
                                  _p(film))
    return dict(v=v, rgba=rgba, aux=aux, film=film, samples=int(n))


def render_row_step(vol: OracleVolume, tf, params: OrcParams, view: np.ndarray, width: int,
                    height: int, y0: int, ystep: int, nthreads: int = 0, want_v=False):
    """Rows y0, y0 + ystep, ... of one view (a bounded sample spread over
    the image); the full-size outputs hold those rows."""
    tfa = np.ascontiguousarray(np.asarray(tf, np.float32).reshape(-1, 4))
    v = np.zeros((height, width, 4), np.float32) if want_v else None
    rgba = np.zeros((height, width, 4), np.uint8)
    view = np.ascontiguousarray(view, np.float32)
    n = lib().orc_render_row_step(vol.h, _p(tfa), tfa.shape[0], C.byref(params), _p(view), width,
                                  height, y0, height, ystep, nthreads, _p(v), _p(rgba))
    if n < 0:
        raise ValueError("orc_render_row_step: bad arguments")
    return dict(v=v, rgba=rgba, samples=int(n))


def march_film(vol: OracleVolume, tf, params: OrcParams, film: np.ndarray, width: int, height: int,
               nthreads: int = 0) -> int:
    tfa = np.ascontiguousarray(np.asarray(tf, np.float32).reshape(-1, 4))
    return int(lib().orc_march_film(vol.h, _p(tfa), tfa.shape[0], C.byref(params), width, height,
                                    nthreads, _p(film)))


def cull(vol: OracleVolume, view: np.ndarray, limit: int = -1, rect=None):
    """OctreeCuller::cull restated: (ids in index order, squared distances)."""
    n = vol.grid[0] * vol.grid[1] * vol.grid[2]
    ids = np.zeros(n, np.int32)
    d2 = np.zeros(n, np.float32)
    v = np.ascontiguousarray(view, np.float32)
    r = None if rect is None else np.ascontiguousarray(rect, np.float32)
    k = lib().orc_cull(vol.h, _p(v), _p(r), limit, _p(ids), _p(d2))
    return ids[:k].copy(), d2[:k].copy()


def lossless_order(vol: OracleVolume, cam: np.ndarray, ids: np.ndarray) -> np.ndarray:
    ids = np.ascontiguousarray(ids, np.int32)
    out = np.zeros_like(ids)
    c = np.ascontiguousarray(cam, np.float32)
    lib().orc_lossless_order(vol.h, _p(c), _p(ids), len(ids), _p(out))
    return out


def present_mask(vol: OracleVolume, ids) -> np.ndarray:
    m = np.zeros(vol.grid[0] * vol.grid[1] * vol.grid[2], np.uint8)
    m[np.asarray(ids, np.int64)] = 1
    return m


def _diff_protos():
    l = lib()
    if not hasattr(l, "_diff_ready"):
        l.orc_diff_forward.restype = None
        l.orc_diff_forward.argtypes = [P, C.c_int32, P, C.c_int32, C.c_float, C.c_int32, C.c_float,
                                       P, C.c_int32, C.c_int32, C.c_int32, C.c_int32, P]
        l.orc_diff_loss_grad64.restype = C.c_double
        l.orc_diff_loss_grad64.argtypes = [P, C.c_int32, P, C.c_int32, C.c_float, C.c_int32,
                                           C.c_float, P, C.c_int32, C.c_int32, C.c_int32, P, P, P, P]
        l._diff_ready = True
    return l


def diff_forward(vol: np.ndarray, tf, views: np.ndarray, W: int, H: int, sample_rate=1.0,
                 max_steps=4000000, density=1.0, nthreads=0) -> np.ndarray:
    """FP32 differentiable-mode forward (reference float operations)."""
    v = np.ascontiguousarray(vol, np.float32)
    t = np.ascontiguousarray(np.asarray(tf, np.float32).reshape(-1, 4))
    vw = np.ascontiguousarray(views, np.float32).reshape(-1, 20)
    out = np.zeros((vw.shape[0], H, W, 4), np.float32)
    _diff_protos().orc_diff_forward(_p(v), v.shape[0], _p(t), t.shape[0], sample_rate, max_steps,
                                    density, _p(vw), vw.shape[0], W, H, nthreads or 8, _p(out))
    return out


def diff_loss_grad64(vol: np.ndarray, tf, views: np.ndarray, W: int, H: int, target=None,
                     sample_rate=1.0, max_steps=4000000, density=1.0, grad=True):
    """FP64 forward, L2 loss against `target` and its analytic gradient."""
    v = np.ascontiguousarray(vol, np.float64)
    t = np.ascontiguousarray(np.asarray(tf, np.float64).reshape(-1, 4))
    vw = np.ascontiguousarray(views, np.float32).reshape(-1, 20)
    tg = None if target is None else np.ascontiguousarray(target, np.float64)
    img = np.zeros((vw.shape[0], H, W, 4), np.float64)
    dv = np.zeros_like(v) if grad else None
    dt = np.zeros_like(t) if grad else None
    loss = _diff_protos().orc_diff_loss_grad64(_p(v), v.shape[0], _p(t), t.shape[0], sample_rate,
                                               max_steps, density, _p(vw), vw.shape[0], W, H,
                                               _p(tg), _p(img), _p(dv), _p(dt))
    return loss, img, dv, dt
