"""Differentiable rendering harness: torch.autograd over hy_diff_forward /
hy_diff_backward (ctypes), and the transfer-function / density fit.

This is a test and fitting harness around the C ABI; the rendering and the
adjoint run in libhydrant_gb300's kernels.  Work is ordered between torch's
current stream and the library's stream with stream waits.
"""

from __future__ import annotations

import ctypes as C
import math
import time
from dataclasses import dataclass, field
from typing import List

import numpy as np
import torch

from . import _abi
from .api import Context, camera_orbit
from .workloads import SplitMix64


def _view_struct(trans, ctg, ray_o) -> _abi.HyView:
    v = _abi.HyView()
    v.trans = (_abi.f16)(*trans)
    v.ctg_fovy_2 = ctg
    v.ray_o = (_abi.f3)(*ray_o)
    return v


class DiffRenderer:
    """One set of views at one resolution over an n^3 f32 volume."""

    def __init__(self, ctx: Context, n: int, views: List[_abi.HyView], width: int, height: int,
                 ntf: int, sample_rate: float = 1.0, density: float = 1.0, ckpt_k: int = 16,
                 max_steps: int = 4000000):
        self.ctx = ctx
        self.p = _abi.HyDiffParams(n, sample_rate, max_steps, density, ntf, ckpt_k)
        self.nviews = len(views)
        self.views = (_abi.HyView * self.nviews)(*views)
        self.W, self.H = width, height
        nb = C.c_int64()
        _abi.check(_abi.lib().hy_diff_ckpt_bytes(C.byref(self.p), width, height, self.nviews,
                                                 C.byref(nb)))
        dev = torch.device("cuda", ctx.device)
        self.ckpt = torch.empty(int(nb.value) // 4, dtype=torch.float32, device=dev)
        self.nsteps = torch.empty(self.nviews * height * width, dtype=torch.int32, device=dev)
        self.stream = torch.cuda.ExternalStream(ctx.stream, device=dev)

    def _enter(self):
        self.stream.wait_stream(torch.cuda.current_stream())

    def _leave(self):
        torch.cuda.current_stream().wait_stream(self.stream)

    def forward(self, vol: torch.Tensor, tf: torch.Tensor, keep: bool = True) -> torch.Tensor:
        img = torch.empty(self.nviews, self.H, self.W, 4, dtype=torch.float32, device=vol.device)
        self._enter()
        self.ctx.check(_abi.lib().hy_diff_forward(
            self.ctx.handle, C.byref(self.p), C.c_void_p(vol.data_ptr()),
            C.c_void_p(tf.data_ptr()), self.views, self.nviews, self.W, self.H,
            C.c_void_p(img.data_ptr()), C.c_void_p(self.ckpt.data_ptr() if keep else None),
            C.c_void_p(self.nsteps.data_ptr() if keep else None)))
        self._leave()
        return img

    def backward(self, vol, tf, dimg):
        dvol = torch.zeros_like(vol)
        dtf = torch.zeros_like(tf)
        self._enter()
        self.ctx.check(_abi.lib().hy_diff_backward(
            self.ctx.handle, C.byref(self.p), C.c_void_p(vol.data_ptr()),
            C.c_void_p(tf.data_ptr()), self.views, self.nviews, self.W, self.H,
            C.c_void_p(dimg.data_ptr()), C.c_void_p(self.ckpt.data_ptr()),
            C.c_void_p(self.nsteps.data_ptr()), C.c_void_p(dvol.data_ptr()),
            C.c_void_p(dtf.data_ptr())))
        self._leave()
        return dvol, dtf


class RenderFn(torch.autograd.Function):
    """image = render(volume, transfer function); gradients through the adjoint kernel."""

    @staticmethod
    def forward(ctx, vol, tf, renderer: DiffRenderer):
        vol = vol.contiguous()
        tf = tf.contiguous()
        img = renderer.forward(vol, tf, keep=True)
        ctx.save_for_backward(vol, tf)
        ctx.renderer = renderer
        return img

    @staticmethod
    def backward(ctx, g):
        vol, tf = ctx.saved_tensors
        dvol, dtf = ctx.renderer.backward(vol, tf, g.contiguous())
        return dvol, dtf, None


def render(vol, tf, renderer: DiffRenderer):
    return RenderFn.apply(vol, tf, renderer)


def orbit_views(ctx_volume, seed: int, count: int, distance: float = 2.2):
    """Seeded orbit cameras (azimuth, elevation) -> ViewArgs for the volume."""
    import hydrant_gb300 as hy

    rng = SplitMix64(seed)
    out = []
    for _ in range(count):
        arm = (rng.uniform(-180, 180), rng.uniform(-60, 60), distance)
        out.append(hy.camera_view(ctx_volume, camera_orbit(arm)))
    return out


def seeded_tf(seed: int, n: int) -> np.ndarray:
    rng = SplitMix64(seed)
    k = np.zeros((n, 4), np.float32)
    for i in range(n):
        k[i] = [rng.uniform(), rng.uniform(), rng.uniform(), rng.uniform(0.0, 1.0)]
    k[0] = 0.0  # empty space stays transparent
    return k


@dataclass
class FitResult:
    losses: List[float] = field(default_factory=list)
    fwd_ms_per_view: float = 0.0
    fwd_adj_ms_per_view: float = 0.0
    iter_ms: List[float] = field(default_factory=list)
    steps: int = 0


def fit(ctx: Context, target_vol: np.ndarray, init_vol: np.ndarray, views, W: int, H: int,
        true_tf: np.ndarray, init_tf: np.ndarray, steps: int = 200, lr_tf: float = 5e-3,
        lr_vol: float = 2e-2, sample_rate: float = 1.0, density: float = 1.0,
        ckpt_k: int = 16, warmup: int = 3) -> FitResult:
    """Adam on (transfer function, volume) against images of the targets.

    Learning rates: on the 256^3, 16 x 512^2 fit, lr_tf 5e-3 / lr_vol 2e-2
    took the loss from 0.211 to 0.0088 in 200 steps; a faster transfer
    function (2e-2 / 1e-2) reached 0.051 by step 25 and then settled at
    0.086 with the rays nearly transparent.

    The first `warmup` iterations (one-off library and allocator set-up) are
    left out of the forward + adjoint timing."""
    dev = torch.device("cuda", ctx.device)
    n = target_vol.shape[0]
    r = DiffRenderer(ctx, n, views, W, H, true_tf.shape[0], sample_rate, density, ckpt_k)
    with torch.no_grad():
        target = r.forward(torch.from_numpy(target_vol).to(dev),
                           torch.from_numpy(true_tf).to(dev), keep=False).clone()
    vol = torch.from_numpy(init_vol).to(dev).requires_grad_(True)
    tf = torch.from_numpy(init_tf).to(dev).requires_grad_(True)
    opt = torch.optim.Adam([{"params": [tf], "lr": lr_tf}, {"params": [vol], "lr": lr_vol}])
    res = FitResult()
    nv = len(views)
    # forward-only timing
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(3):
        r.forward(vol.detach(), tf.detach(), keep=False)
    torch.cuda.synchronize()
    res.fwd_ms_per_view = (time.perf_counter() - t0) / 3 / nv * 1e3
    t_fb = 0.0
    for it in range(warmup + steps):
        opt.zero_grad(set_to_none=True)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        img = render(vol, tf, r)
        loss = ((img - target) ** 2).mean()
        loss.backward()
        torch.cuda.synchronize()
        dt = time.perf_counter() - t1
        if it >= warmup:
            t_fb += dt
            res.iter_ms.append(dt * 1e3)
        opt.step()
        with torch.no_grad():
            vol.clamp_(0.0, 1.0)
            tf.clamp_(0.0, 1.0)
        res.losses.append(float(loss.item()))
    res.steps = steps
    res.fwd_adj_ms_per_view = t_fb / max(1, steps) / nv * 1e3
    return res
