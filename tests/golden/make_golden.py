"""Generate tests/golden/golden.npz with the oracle (test infrastructure).

    python tests/golden/make_golden.py

Volumes are built with integer arithmetic only (no libm), so they are the
same on every platform.  Each case stores the oracle's RGBA8 image, its
pre-quantisation floats, the aux channel and the brick-sample count.
The reference itself ships no golden vectors for this path; these pin the
oracle (and, through the GPU test, the kernels) against regressions.
"""

from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

OUT = Path(__file__).resolve().parent / "golden.npz"

TF9 = [[0, 0, 0, 0], [1, 0, 0, 1], [1, 0.5, 0, 1], [1, 1, 0, 1], [0, 1, 0, 1], [0, 1, 1, 1],
       [0, 0, 1, 1], [1, 0, 1, 1], [0, 0, 0, 0]]


def int_blobs(n: int) -> np.ndarray:
    """u8 volume from integer quadratic falloffs around 5 fixed centres."""
    z, y, x = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    acc = np.zeros((n, n, n), np.int64)
    centres = [(n * 3 // 10, n * 4 // 10, n // 2, n // 4, 250), (n * 6 // 10, n // 2, n * 4 // 10, n // 5, 180),
               (n // 2, n * 7 // 10, n * 6 // 10, n // 6, 220), (n * 7 // 10, n * 3 // 10, n * 3 // 10, n // 7, 140),
               (n // 3, n * 2 // 3, n // 3, n // 8, 255)]
    for cx, cy, cz, r, peak in centres:
        d2 = (x - cx) ** 2 + (y - cy) ** 2 + (z - cz) ** 2
        acc += np.maximum(0, peak * (r * r - d2) // (r * r))
    return np.clip(acc, 0, 255).astype(np.uint8)


def int_rods(n: int) -> np.ndarray:
    """u8 volume of axis-aligned and diagonal rods over a hashed background."""
    z, y, x = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    bg = ((x * 73856093) ^ (y * 19349663) ^ (z * 83492791)) % 31
    v = bg.astype(np.int64)
    rod = ((x - n // 3) ** 2 + (y - n // 2) ** 2 <= (n // 10) ** 2)
    rod |= ((y - n // 4) ** 2 + (z - n // 2) ** 2 <= (n // 12) ** 2)
    rod |= ((x - z) ** 2 + (y - 2 * n // 3) ** 2 <= (n // 9) ** 2)
    v = np.where(rod, 180 + (x + 2 * y + 3 * z) % 60, v)
    return np.clip(v, 0, 255).astype(np.uint8)


CASES = [
    # name, volume fn, n, block, pad, params, camera arm, W, H
    ("volume_blobs", "blobs", 32, 16, 1, dict(shader=0, sample_rate=0.5, density=1.0), (25, 65, 2.2), 40, 32),
    ("volume_blobs_d01", "blobs", 32, 32, 1, dict(shader=0, sample_rate=0.25, density=0.1), (-40, 20, 2.0), 32, 32),
    ("volume_rods_composite", "rods", 48, 16, 1, dict(shader=0, sample_rate=0.5, density=0.5, composite=1), (30, 40, 2.4), 32, 32),
    ("iso_rods_color", "rods", 48, 16, 1, dict(shader=2, mode=0, isovalue=0.5), (30, 40, 2.4), 32, 32),
    ("iso_rods_normal", "rods", 48, 16, 2, dict(shader=2, mode=1, isovalue=0.6), (-60, 10, 2.2), 32, 32),
    ("blocks_rods_volume", "rods", 48, 16, 1, dict(shader=1, mode=0, density=0.01), (30, 40, 2.4), 32, 32),
    ("blocks_rods_solid", "rods", 48, 16, 1, dict(shader=1, mode=1), (30, 40, 2.4), 32, 32),
]


def volume(kind: str, n: int) -> np.ndarray:
    return int_blobs(n) if kind == "blobs" else int_rods(n)


def oracle_params(orc, d: dict):
    p = orc.OrcParams()
    p.shader = d.get("shader", 0)
    p.mode = d.get("mode", 0)
    p.sample_rate = d.get("sample_rate", 1.0)
    p.max_steps = 4000000
    p.density = d.get("density", 1.0)
    p.isovalue = d.get("isovalue", 0.5)
    for i in range(3):
        p.surface_color[i] = 1.0
    p.composite = d.get("composite", 0)
    p.count_samples = 1
    return p


def render_case(case):
    from oracle import oracle as orc

    name, kind, n, bs, pad, params, arm, W, H = case
    vox = volume(kind, n)
    ov = orc.OracleVolume(vox, bs, pad)
    cam = orc.camera_orbit(arm)
    view = orc.camera_view(ov, cam)
    p = oracle_params(orc, params)
    if p.shader == 2:
        orc.iso_lighting(ov, cam, p)
    r = orc.render(ov, TF9, p, view, W, H, nthreads=2)
    return vox, view, r


def main():
    data = {}
    for case in CASES:
        name = case[0]
        _, view, r = render_case(case)
        data[f"{name}/view"] = view
        data[f"{name}/rgba"] = r["rgba"]
        data[f"{name}/v"] = r["v"]
        data[f"{name}/aux"] = r["aux"]
        data[f"{name}/samples"] = np.array([r["samples"]], np.int64)
    np.savez_compressed(OUT, **data)
    print(OUT, OUT.stat().st_size, "bytes")


if __name__ == "__main__":
    main()
