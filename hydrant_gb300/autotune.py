"""Autotuned launch shapes of the batched renderer, persisted as JSON.

The cache maps (GPU name, batch signature) to the hy_batch_config that
hy_batch_autotune found fastest.  Signature: shader, mode, composite, brick
edge, volume dims and the sorted view resolutions.
"""

from __future__ import annotations

import json
import os
from pathlib import Path

DEFAULT_PATH = Path(os.environ.get("HYDRANT_GB300_TUNE_CACHE",
                                   Path(__file__).resolve().parent / "autotune_cache.json"))


def signature(gpu_name: str, params, vol_desc, sizes) -> str:
    dims = "x".join(str(d) for d in vol_desc.dim)
    res = ",".join(f"{w}x{h}" for w, h in sorted(sizes))
    return (f"{gpu_name}|shader{params.shader}|mode{params.mode}|comp{params.composite}|"
            f"bs{vol_desc.block_size}p{vol_desc.padding}|{dims}|{res}")


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
                         c.get("block_queue", 1))
        return dict(c, source="cache")
    best = batch.autotune(rgba_ptr, reps)
    c = {"tile_w": best.tile_w, "grab": best.grab, "block_warps": best.block_warps,
         "blocks_per_sm": best.blocks_per_sm, "block_queue": best.block_queue}
    cache[key] = c
    try:
        Path(path).write_text(json.dumps(cache, indent=1, sort_keys=True))
    except OSError:
        pass
    return dict(c, source="autotune")
