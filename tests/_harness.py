"""Shared helpers: render one case on the GPU (through the C ABI) and with the oracle."""

from __future__ import annotations

import numpy as np

import hydrant_gb300 as hy
from hydrant_gb300 import workloads as wl
from oracle import oracle as orc

LSB_TOL = 1        # per 8-bit channel
FLOAT_TOL = 1e-4   # max abs on pre-quantisation floats


def view_array(view) -> np.ndarray:
    return np.array(list(view.trans) + [view.ctg_fovy_2] + list(view.ray_o), np.float32)


def camera(kind="orbit", a=(25.0, 65.0, 2.2), target=(0.0, 0.0, 0.0), up=(0.0, 1.0, 0.0), fovy=60.0):
    return wl.make_camera(wl.Camera(kind, tuple(a), tuple(target), tuple(up), fovy))


class Case:
    """A volume resident on both sides (GPU and oracle)."""

    def __init__(self, ctx, vox, block_size, padding=1, tf=wl.TF9):
        self.ctx = ctx
        self.vox = vox
        self.vol = hy.Volume(ctx, vox, block_size, padding)
        self.ov = orc.OracleVolume(vox, block_size, padding)
        self.tf = tf
        ctx.set_transfer_fn(tf)

    def close(self):
        self.vol.close()

    def render_both(self, cam, W, H, nthreads=0, **kw):
        """GPU and oracle images of one view.  The GPU renders twice: with the
        aux output (theta / phi or depth) and without it.  Without aux the
        Volume shader in Default mode takes the lean march (the instantiation
        the benchmark times), so both kernel instantiations face the oracle;
        the lean one is checked here (images, floats, sample count) and the
        full one is returned for the caller's own checks.  Where the lean
        march samples by texture gathers (u8 bricks with an apron), it also
        renders with the loads and both must agree bit for bit."""
        p = hy.shader_params(count_samples=True, **kw)
        if p.shader == hy._abi.SHADER_ISOSURFACE:
            hy.iso_lighting(self.vol, cam, p)
        view = hy.camera_view(self.vol, cam)
        self.ctx.set_transfer_fn(self.tf)
        g = hy.render(self.ctx, self.vol, p, view, W, H, want_v=True, want_aux=True)
        lean = hy.render(self.ctx, self.vol, p, view, W, H, want_v=True, want_aux=False)
        r = orc.render(self.ov, self.tf, orc.params_from(p), view_array(view), W, H, nthreads=nthreads)
        assert_parity(lean, r, check_aux=False, what=f"no-aux render {kw}")
        assert np.array_equal(lean.rgba, g.rgba) and np.array_equal(lean.v, g.v), \
            f"no-aux render differs from the aux render {kw}"
        if self.vol.gather_sampling:
            self.vol.set_gather_sampling(False)
            try:
                loads = hy.render(self.ctx, self.vol, p, view, W, H, want_v=True, want_aux=False)
            finally:
                self.vol.set_gather_sampling(True)
            assert np.array_equal(loads.rgba, lean.rgba) and np.array_equal(loads.v, lean.v), \
                f"lean march: loads and gathers differ {kw}"
            assert loads.samples == lean.samples
        return g, r, p, view


def assert_parity(g, r, check_aux=True, check_samples=True, what=""):
    d8 = np.abs(g.rgba.astype(np.int32) - r["rgba"].astype(np.int32))
    assert d8.max() <= LSB_TOL, f"{what}: max {d8.max()} LSB at {np.unravel_index(d8.argmax(), d8.shape)}"
    fin = np.isfinite(r["v"])
    assert np.array_equal(fin, np.isfinite(g.v)), f"{what}: non-finite pattern differs"
    dv = np.abs(np.where(fin, g.v, 0) - np.where(fin, r["v"], 0))
    assert dv.max() <= FLOAT_TOL, f"{what}: max abs {dv.max()} at {np.unravel_index(dv.argmax(), dv.shape)}"
    if check_aux:
        fa = np.isfinite(r["aux"])
        assert np.array_equal(fa, np.isfinite(g.aux)), f"{what}: aux non-finite pattern differs"
        da = np.abs(np.where(fa, g.aux, 0) - np.where(fa, r["aux"], 0))
        rel = da / np.maximum(1.0, np.abs(np.where(fa, r["aux"], 0)))
        assert rel.max() <= FLOAT_TOL, f"{what}: aux max rel {rel.max()}"
    if check_samples:
        assert g.samples == r["samples"], f"{what}: samples {g.samples} != {r['samples']}"
    return dict(max_lsb=int(d8.max()), max_abs=float(dv.max()),
                exact_frac=float((d8.max(axis=-1) == 0).mean()))
