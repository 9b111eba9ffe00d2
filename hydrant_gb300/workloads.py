"""Seeded synthetic workloads with the shapes of the benchmark configurations.

No dataset from the reference is available (the Aneurism volume of its
README is not shipped), so every workload is a seeded procedural volume
generated by libhydrant_gb300 (include/hydrant_gb300_synth.h) plus a camera
set and renderer parameters.  Random draws use splitmix64 so they are the
same on every platform.
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import List, Tuple

# 9 evenly spaced RGBA knots of the Volume configuration (README.md:21-50)
TF9 = [
    [0, 0, 0, 0],
    [1, 0, 0, 1],
    [1, 0.5, 0, 1],
    [1, 1, 0, 1],
    [0, 1, 0, 1],
    [0, 1, 1, 1],
    [0, 0, 1, 1],
    [1, 0, 1, 1],
    [0, 0, 0, 0],
]


class SplitMix64:
    def __init__(self, seed: int):
        self.s = seed & 0xFFFFFFFFFFFFFFFF

    def next(self) -> int:
        self.s = (self.s + 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF
        z = self.s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & 0xFFFFFFFFFFFFFFFF
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & 0xFFFFFFFFFFFFFFFF
        return z ^ (z >> 31)

    def uniform(self, lo: float = 0.0, hi: float = 1.0) -> float:
        return lo + (hi - lo) * ((self.next() >> 11) * (1.0 / 9007199254740992.0))

    def choice(self, seq):
        return seq[min(len(seq) - 1, int(self.uniform() * len(seq)))]


@dataclass
class Camera:
    kind: str  # "orbit" or "ptu"
    a: Tuple[float, float, float]  # arm, or position
    target: Tuple[float, float, float] = (0.0, 0.0, 0.0)
    up: Tuple[float, float, float] = (0.0, 1.0, 0.0)
    fovy: float = 60.0


@dataclass
class View:
    camera: Camera
    width: int
    height: int


@dataclass
class Workload:
    name: str
    dim: Tuple[int, int, int]  # x, y, z
    generator: str  # "blobs_u8" | "tubes_u8" | "blobs_f32"
    seed: int
    count: int  # blobs or tubes
    block_size: int
    padding: int
    views: List[View]
    params: dict = field(default_factory=dict)
    tf: list = field(default_factory=lambda: TF9)

    def voxels(self, nthreads: int = 0):
        from . import api

        fn = {"blobs_u8": api.synth_blobs_u8, "tubes_u8": api.synth_tubes_u8,
              "blobs_f32": api.synth_blobs_f32}[self.generator]
        return fn(self.seed, self.dim, self.count, nthreads)


def volume_c0(scale: int = 1) -> Workload:
    """Plain Volume: 128^3 u8, 12 blobs, one brick, 512^2, orbit [25,65,2.2]."""
    n = 128 // scale
    res = 512 // scale
    return Workload(
        name=f"volume_c0_{n}cube_{res}px",
        dim=(n, n, n), generator="blobs_u8", seed=0, count=12, block_size=n, padding=1,
        views=[View(Camera("orbit", (25.0, 65.0, 2.2)), res, res)],
        params=dict(shader="Volume", mode="Default", sample_rate=0.25, density=1e-2),
    )


def tubes_c1(n: int = 512, block_size: int = 64, res: int = 1024) -> Workload:
    """Isosurface + Blocks: 512^3 u8 tubes in 64^3 bricks, 1024^2."""
    return Workload(
        name=f"tubes_c1_{n}cube_{res}px",
        dim=(n, n, n), generator="tubes_u8", seed=1, count=40, block_size=block_size, padding=1,
        views=[View(Camera("orbit", (25.0, 65.0, 2.2)), res, res)],
        params=dict(shader="Isosurface", mode="Color", sample_rate=1.0, isovalue=0.5),
    )


def sphere_cameras(seed: int, count: int, resolutions, distance: float = 2.2) -> List[View]:
    """Cameras on a sphere around the volume, |dir . up| < 0.99, looking at the centre."""
    rng = SplitMix64(seed)
    views = []
    while len(views) < count:
        z = rng.uniform(-1.0, 1.0)
        phi = rng.uniform(0.0, 2.0 * math.pi)
        r = math.sqrt(max(0.0, 1.0 - z * z))
        d = (r * math.cos(phi), z, r * math.sin(phi))  # y is up
        if abs(d[1]) >= 0.99:
            continue
        res = rng.choice(resolutions)
        pos = tuple(distance * c for c in d)
        views.append(View(Camera("ptu", pos), res, res))
    return views


def multiview_c3(n: int = 1024, nviews: int = 64, resolutions=(256, 512, 1024, 2048)) -> Workload:
    """Batched multi-view: 1024^3 u8, 64 blobs, 64^3 bricks, 64 cameras."""
    return Workload(
        name=f"multiview_c3_{n}cube_{nviews}views",
        dim=(n, n, n), generator="blobs_u8", seed=3, count=64, block_size=64, padding=1,
        views=sphere_cameras(3, nviews, list(resolutions)),
        params=dict(shader="Volume", mode="Default", sample_rate=0.25, density=1e-2),
    )


def make_camera(c: Camera):
    from . import api

    if c.kind == "orbit":
        return api.camera_orbit(c.a, c.target, c.fovy)
    return api.camera_ptu(c.a, c.target, c.up, c.fovy)
