"""Autotuned launch shapes of the batched renderer, persisted as JSON.

The cache maps (GPU name, library build, batch signature) to the
hy_batch_config that hy_batch_autotune found fastest.  Signature: shader,
mode, composite, brick edge, volume dims and the sorted view resolutions.
The build is a hash of the loaded library, so a rebuilt kernel is tuned
afresh rather than given a shape measured on its predecessor.
"""

from __future__ import annotations

import hashlib
import json
import os
from pathlib import Path

DEFAULT_PATH = Path(os.environ.get("HYDRANT_GB300_TUNE_CACHE",
                                   Path(__file__).resolve().parent / "autotune_cache.json"))


_BUILD_ID = None


def build_id() -> str:
    """First 12 hex digits of the SHA-1 of libhydrant_gb300.so."""
    global _BUILD_ID
    if _BUILD_ID is None:
        from . import _abi

        try:
            _BUILD_ID = hashlib.sha1(Path(_abi.LIB_PATH).read_bytes()).hexdigest()[:12]
        except OSError:
            _BUILD_ID = "unbuilt"
    return _BUILD_ID


def signature(gpu_name: str, params, vol_desc, sizes) -> str:
    dims = "x".join(str(d) for d in vol_desc.dim)
    res = ",".join(f"{w}x{h}" for w, h in sorted(sizes))
    return (f"{gpu_name}|lib{build_id()}|shader{params.shader}|mode{params.mode}|"
            f"comp{params.composite}|bs{vol_desc.block_size}p{vol_desc.padding}|{dims}|{res}")


def load(path: Path = DEFAULT_PATH) -> dict:
    try:
        return json.loads(Path(path).read_text())
    except (OSError, ValueError):
        return {}


def tuned_config(batch, key: str, rgba_ptr: int, reps: int = 2, path: Path = DEFAULT_PATH,
                 retune: bool = False) -> dict:
    """Apply the cached config for `key`, or autotune and store it."""
    cache = load(path)
    if not retune and key in cache:
        c = cache[key]
        batch.set_config(c["tile_w"], c["grab"], c["block_warps"], c.get("blocks_per_sm", 0),
                         c.get("block_queue", 1), c.get("steps_per_iter", 1))
        return dict(c, source="cache")
    best = batch.autotune(rgba_ptr, reps)
    c = {"tile_w": best.tile_w, "grab": best.grab, "block_warps": best.block_warps,
         "blocks_per_sm": best.blocks_per_sm, "block_queue": best.block_queue,
         "steps_per_iter": max(1, best.steps_per_iter)}
    cache[key] = c
    try:
        Path(path).write_text(json.dumps(cache, indent=1, sort_keys=True))
    except OSError:
        pass
    return dict(c, source="autotune")
