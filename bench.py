#!/usr/bin/env python3
"""Benchmark of the ray-marching path (one JSON line on rank 0).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload multiview|volume|tubes]

Default workload: the batched multi-view configuration -- a 1024^3 u8
Gaussian-blob volume in 64^3 bricks, 64 cameras on a seeded orbit sphere at
resolutions drawn from {256^2, 512^2, 1024^2, 2048^2}, Volume shader, the
9-knot transfer function, 1-voxel steps, density 1e-2.  One step renders all
64 views.  Metric: Gsamples/s (brick trilinear samples per second); views/s
is reported beside it.

--impl ours       the GB300 path: all views of a step in one persistent
                  launch replayed from a CUDA graph (hy_batch); the plain
                  per-view path (one hy_render_device launch per view) is
                  timed beside it.  `e2e` goes through hy_batch_render with a
                  host output buffer (device -> host images inside the timing).
--impl reference  the reference's own CPU multi-thread backend for this path
                  (restated in oracle/, the reference cannot be built here)
                  on all host threads, on a bounded sample of the workload.

Multi-GPU: every rank renders the full batch (replicas, weak scaling); the
timed region is bracketed by a barrier and the max over ranks is reported.
"""

from __future__ import annotations

import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

BYTES_PER_SAMPLE = 8  # 2x2x2 u8 trilinear footprint per brick sample


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["multiview", "volume", "tubes", "paging", "diff"],
                    default="multiview")
    ap.add_argument("--frames", type=int, default=120, help="paging workload: orbit frames")
    ap.add_argument("--paging-scale", type=int, default=1,
                    help="paging workload: divide the volume and image edges by this")
    ap.add_argument("--views", type=int, default=64)
    ap.add_argument("--res", type=int, default=0,
                    help="keep only the views of this resolution (profiling a small case)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--sampler", choices=["gather", "loads"], default="gather",
                    help="Volume march over u8 bricks: texture gathers or loads")
    ap.add_argument("--diff-views", type=int, default=16,
                    help="diff workload: views of the fit (16; fewer for a small profiling case)")
    ap.add_argument("--ckpt-k", type=int, default=32,
                    help="diff workload: checkpoint interval of the differentiable march")
    ap.add_argument("--no-extra", action="store_true",
                    help="leave out the compositing and differentiable legs (profiling)")
    ap.add_argument("--coarse-level", type=int, default=3,
                    help="paging: coarse fallback level (box filter 2**L; 0 = none)")
    ap.add_argument("--pager", choices=["realtime", "lossless"], default="realtime",
                    help="paging: the realtime cache or lossless batches (offline frames)")
    ap.add_argument("--lossless-batch", type=int, default=4096,
                    help="paging, lossless: bricks per batch (the reference caps it at 4096)")
    ap.add_argument("--cache-gib", type=float, default=8.0,
                    help="paging workload: device brick cache of the realtime pager")
    ap.add_argument("--no-tune-cache", action="store_true",
                    help="paging: a cache of the whole --cache-gib (no sizing to the orbit)")
    ap.add_argument("--eviction", choices=["lru", "reference"], default="lru",
                    help="paging, realtime: least recently visible, or the reference's order")
    ap.add_argument("--prefetch", action="store_true",
                    help="paging, realtime: move the next orbit camera's bricks on the copy "
                         "stream while each frame renders (hy_pager_prefetch)")
    ap.add_argument("--pager-sampler", choices=["gathers", "loads"], default="gathers",
                    help="paging, realtime: the cache in gather textures (the Volume march "
                         "samples by texture gathers) or in a device pool (loads)")
    ap.add_argument("--max-uploads", type=int, default=0,
                    help="paging: brick uploads per frame (0 = every missing brick)")
    ap.add_argument("--launch-shape", default="",
                    help="fixed batch launch shape tile_w,grab,block_warps,blocks_per_sm,"
                         "block_queue[,steps_per_iter] (implies --no-autotune)")
    ap.add_argument("--no-autotune", action="store_true",
                    help="use the default batch launch shape (profiling)")
    ap.add_argument("--cpu-row-step", type=int, default=128,
                    help="CPU sample: every this many-th pixel row of every view")
    ap.add_argument("--shader", choices=["Volume", "Blocks", "Isosurface"], default="",
                    help="tubes / volume / multiview: render with this shader instead")
    ap.add_argument("--mode", default="",
                    help="with --shader: its mode (Volume: Default / Partition / Paging; "
                         "Blocks: Volume / Solid; Isosurface: Color / Normal / Position)")
    ap.add_argument("--composite", action="store_true",
                    help="per-brick partial images composited front to back (sort-last)")
    ap.add_argument("--sample-rate", type=float, default=0.0,
                    help="override the workload's sample rate (step = du / 4 / rate)")
    ap.add_argument("--density", type=float, default=None,
                    help="override the workload's density")
    return ap.parse_args()


def workload(args):
    return with_overrides(args, base_workload(args))


def workloads_module():
    """hydrant_gb300/workloads.py (seeds, shapes, cameras, parameters) loaded
    on its own: the CPU side of the measurement reads the workload
    descriptions without importing the product package or its library."""
    import importlib.util

    name = "_hy_workload_defs"
    if name not in sys.modules:
        spec = importlib.util.spec_from_file_location(name, ROOT / "hydrant_gb300" / "workloads.py")
        mod = importlib.util.module_from_spec(spec)
        sys.modules[name] = mod
        spec.loader.exec_module(mod)
    return sys.modules[name]


def base_workload(args):
    wl = workloads_module()

    if args.workload == "volume":
        return wl.volume_c0()
    if args.workload == "tubes":
        return wl.tubes_c1()
    w = wl.multiview_c3(nviews=args.views)
    if args.res:
        w.views = [v for v in w.views if v.width == args.res] or w.views[:1]
        w.views = w.views[: max(1, args.views)]
        # the cameras of the set that render at this resolution
        w.name = f"multiview_c3_{w.dim[0]}cube_{len(w.views)}views_at_{args.res}px"
    return w


def with_overrides(args, w):
    """The configuration's other shader / mode / compositing variants on the
    same volume and cameras (e.g. the tubes with Blocks.Volume and per-brick
    sort-last compositing), named in the workload."""
    tags = []
    if args.shader:
        w.params["shader"] = args.shader
        w.params.pop("mode", None)
        tags.append(args.shader)
    if args.mode:
        w.params["mode"] = args.mode
        tags.append(args.mode)
    if args.composite:
        w.params["composite"] = True
        tags.append("composite")
    if args.sample_rate > 0:
        w.params["sample_rate"] = args.sample_rate
        tags.append(f"rate{args.sample_rate:g}")
    if args.density is not None:
        w.params["density"] = args.density
        tags.append(f"density{args.density:g}")
    if tags:
        w.name = "_".join([w.name] + tags)
    return w


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(values, device="cpu"):
    """Element-wise maximum of a list of floats over all ranks (the job's
    time is its slowest rank's); the values themselves at one rank."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return [float(v) for v in values]
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t.tolist()]


def aggregate_gsamples(samples_per_rank_step, world_size, steps, seconds):
    """Whole-job throughput: every rank renders its own replica of the batch
    (replicas only: no data exchange), so the job processes world_size times
    one rank's samples in the slowest rank's time."""
    return samples_per_rank_step * world_size * steps / seconds / 1e9


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_per_sample(block_queue: int, what: str = "dram_bytes_per_sample",
                       sampler: str = "gather"):
    """A per-sample figure of the batch kernel (DRAM bytes, warp instructions)
    from the committed ncu summary (one capture of 4 views of the same volume;
    both grow with the samples processed, so they scale to a full launch by
    samples)."""
    p = ROOT / "profiles" / "batch_kernel_multiview.txt"
    if not p.exists():
        return None
    tag = f"{what}[sampler={sampler},block_queue={block_queue}]:"
    for line in p.read_text().splitlines():
        if line.startswith(tag):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


def issue_roofline(inst_per_sample, samples, launch_s, clocks, device):
    """The bound the march works against besides L1 latency: warp
    instructions per second (the profiled instructions per sample x samples
    / launch time) against the peak of one instruction per cycle on each of
    the SMs' 4 schedulers at the median SM clock sampled during the timed
    region."""
    if not inst_per_sample or not clocks or not clocks.get("sm_mhz"):
        return None
    import torch

    sms = torch.cuda.get_device_properties(device).multi_processor_count
    peak = sms * 4 * clocks["sm_mhz"] * 1e6 / 1e9
    achieved = inst_per_sample * samples / launch_s / 1e9
    return {"achieved": achieved, "peak": peak, "unit": "G warp instructions/s",
            "frac": achieved / peak, "warp_instructions_per_sample": inst_per_sample,
            "note": "peak = SMs x 4 schedulers x median SM clock"}


class Clocks:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in Path(self.path).read_text().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 9:
                rows.append(f)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(rows)}


def build_all():
    import __graft_entry__

    __graft_entry__.build()


def cpu_model() -> str:
    """The host CPU as /proc/cpuinfo or lscpu name it (architecture first)."""
    import platform
    import subprocess

    name = ""
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "hardware")):
                name = line.split(":", 1)[1].strip()
                break
    except OSError:
        pass
    if not name:
        try:
            out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
            for line in out.splitlines():
                if line.startswith("Model name:"):
                    name = line.split(":", 1)[1].strip()
                    break
        except (OSError, subprocess.SubprocessError):
            pass
    return f"{platform.machine()} {name}".strip()


def workload_config(w, ov):
    """The workload as both arms name it: the volume, bricking, views and
    shader parameters, and the input size against L2 (the brick pool of the
    non-empty bricks, 256-byte aligned slots)."""
    P = w.block_size + 2 * w.padding
    slot = (P ** 3 * (1 if w.generator.endswith("u8") else 4) + 255) // 256 * 256
    pool = ov.nonempty * slot
    return {
        "workload": w.name, "volume": list(w.dim), "block_size": w.block_size,
        "padding": w.padding, "views": len(w.views),
        "pixels_per_step": sum(v.width * v.height for v in w.views),
        "params": {k: v for k, v in w.params.items()},
        "l2": ("inputs larger than L2 (brick pool %.2f GB)" % (pool / 1e9)) if pool >= 256 * 2**20
              else ("L2 flushed between timed steps (brick pool %.1f MB)" % (pool / 1e6)),
    }


def cpu_views(w, ov, views=None):
    """Per view of the workload: (oracle view array, oracle parameters, W, H).
    `views`: the product's view arrays, so the oracle renders exactly the
    rays the GPU rendered (parity); without them the oracle computes the
    cameras itself (the reference arm loads nothing else)."""
    from oracle import oracle as orc

    out = []
    for i, v in enumerate(w.views):
        c = v.camera
        cam = (orc.camera_orbit(c.a, c.target, c.fovy) if c.kind == "orbit"
               else orc.camera_ptu(c.a, c.target, c.up, c.fovy))
        p = orc.shader_params(**w.params)
        if p.shader == 2:
            orc.iso_lighting(ov, cam, p)
        va = views[i] if views is not None else orc.camera_view(ov, cam)
        out.append((va, p, v.width, v.height))
    return out


def sample_rows(H, row_step):
    y0 = min(row_step // 2, H // 2)
    return y0, len(range(y0, H, row_step))


def cpu_step(w, ov, cviews, row_step, nthreads, want_v=False, only=None):
    """One step of the CPU sample: pixel rows row_step/2, row_step/2 +
    row_step, ... of every view (1/row_step of the workload's rays, spread
    over all views and over each image)."""
    from oracle import oracle as orc

    samples, imgs = 0, []
    for i, (va, p, W, H) in enumerate(cviews):
        if only is not None and i not in only:
            imgs.append(None)
            continue
        y0, _ = sample_rows(H, row_step)
        r = orc.render_row_step(ov, w.tf, p, va, W, H, y0, row_step, nthreads, want_v=want_v)
        samples += r["samples"]
        imgs.append(r)
    return samples, imgs


def sample_desc(w, row_step, samples):
    rays = 0
    for v in w.views:
        rays += v.width * sample_rows(v.height, row_step)[1]
    return (f"every {row_step}th pixel row of all {len(w.views)} views ({rays} rays, "
            f"1/{row_step} of the step's rays), {samples} samples per step")


def main_reference(args):
    """The reference's CPU multi-thread backend (cpu_shading.cc:9-90 over the
    shared shaders, restated in oracle/) on every host thread, on a bounded
    sample of the same workload: 1/row_step of every view's pixel rows.
    Loads the oracle only: voxels, cameras and parameters come from the
    oracle's own host code."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    from oracle import build as ob
    from oracle import oracle as orc

    ob.build()
    w = workload(args)
    nthreads = os.cpu_count() or 1
    vox = orc.workload_voxels(w, nthreads)
    ov = orc.OracleVolume(vox, w.block_size, w.padding)
    cviews = cpu_views(w, ov)
    step = max(1, args.cpu_row_step)
    for _ in range(args.warmup):
        cpu_step(w, ov, cviews, step, nthreads)
    tot_s, tot_t = 0, 0.0
    for _ in range(args.steps):
        t = time.perf_counter()
        s, _ = cpu_step(w, ov, cviews, step, nthreads)
        tot_t += time.perf_counter() - t
        tot_s += s
    value = tot_s / tot_t / 1e9
    sample = sample_desc(w, step, tot_s // max(1, args.steps))
    out = {
        "impl": "reference",
        "metric": "Gsamples/s",
        "value": value,
        "unit": "Gsamples/s",
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": tot_t / args.steps * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic",
        "config": workload_config(w, ov),
        "cpu_baseline": {"value": value, "unit": "Gsamples/s", "cores": nthreads, "kind": "port",
                         "sample": sample, "cpu": cpu_model()},
        "e2e": {"value": value, "unit": "Gsamples/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)
    return 0


def composite_leg(hy, ctx, vol, w, views, lighting, stream, flush, args):
    """All views of the step with per-brick sort-last compositing (every
    non-empty brick a ray crosses is its own segment, composited front to
    back with volume.cc:267-280): batched (one persistent launch from a CUDA
    graph) and plain (one launch per view), CUDA events on the library's
    stream."""
    import torch

    kw = dict(w.params)
    kw["composite"] = True
    p = hy.shader_params(**kw)
    batch = hy.Batch(ctx, vol, p, views, lighting)
    try:
        out = torch.empty(batch.nbytes, dtype=torch.uint8, device=f"cuda:{ctx.device}")
        batch.set_counting(True)
        batch.render_device(out.data_ptr())
        samples = ctx.stats().samples
        batch.set_counting(False)
        for _ in range(args.warmup):
            batch.render_device(out.data_ptr())
        evs = _timed_steps(torch, stream, args.steps, lambda: batch.render_device(out.data_ptr()),
                           flush)
        ctx.synchronize()
        tb = sum(a.elapsed_time(b) for a, b in evs) / 1e3 / args.steps

        def plain_step():
            for (view, W, H), off in zip(views, batch.offsets):
                hy.render_device(ctx, vol, p, view, W, H, out.data_ptr() + off)

        for _ in range(args.warmup):
            plain_step()
        evs = _timed_steps(torch, stream, args.steps, plain_step, flush)
        ctx.synchronize()
        tp = sum(a.elapsed_time(b) for a, b in evs) / 1e3 / args.steps
    finally:
        batch.close()
    return {"value": samples / tb / 1e9, "unit": "Gsamples/s", "samples_per_step": samples,
            "ms_per_step": tb * 1e3, "views_per_s": len(views) / tb,
            "plain": {"value": samples / tp / 1e9, "unit": "Gsamples/s", "ms_per_step": tp * 1e3,
                      "views_per_s": len(views) / tp},
            "batched_over_plain": tp / tb,
            "path": "per-brick segments composited front to back; batched = one persistent "
                    "launch per step from a CUDA graph, plain = one launch per view"}


def ert_leg(hy, ctx, dev, reps=5):
    """Early ray termination (opt-in) where rays do become opaque: the
    512^3 tubes volume (64^3 bricks, apron 1) with the Volume shader at
    density 1, 1-voxel steps, one 1024^2 view (orbit 25, 65, 2.2); the lean
    per-view march with and without termination at v.a >= 1 - 2^-16, CUDA
    events on the library's stream, and the image differences between the
    two (the full march is the oracle's, bit for bit)."""
    import numpy as np
    import torch

    from hydrant_gb300 import workloads as wl

    w = wl.tubes_c1()
    vol = hy.Volume(ctx, hy.synth_tubes_u8(w.seed, w.dim, w.count), w.block_size, w.padding)
    try:
        ctx.set_transfer_fn(w.tf)
        cam = wl.make_camera(w.views[0].camera)
        view = hy.camera_view(vol, cam)
        W = H = w.views[0].width
        t = 1.0 - 2.0 ** -16
        out = {}
        stream = torch.cuda.ExternalStream(ctx.stream)
        imgs = {}
        for name, et in (("full", 0.0), ("terminated", t)):
            p = hy.shader_params(shader="Volume", sample_rate=0.25, density=1.0,
                                 early_termination=et, count_samples=True)
            r = hy.render(ctx, vol, p, view, W, H, want_v=True)
            imgs[name] = r
            p.count_samples = 0
            buf = torch.empty(W * H * 4, dtype=torch.uint8, device=dev)
            for _ in range(2):
                hy.render_device(ctx, vol, p, view, W, H, buf.data_ptr())
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(reps):
                hy.render_device(ctx, vol, p, view, W, H, buf.data_ptr())
            e1.record(stream)
            e1.synchronize()
            ms = e0.elapsed_time(e1) / reps
            out[name] = {"ms_per_view": ms, "samples": r.samples,
                         "gsamples_per_s": r.samples / ms / 1e6}
        full, term = imgs["full"], imgs["terminated"]
        out["threshold"] = t
        out["speedup"] = out["full"]["ms_per_view"] / out["terminated"]["ms_per_view"]
        out["full_march_gsamples_per_s"] = out["full"]["samples"] / out["terminated"]["ms_per_view"] / 1e6
        out["max_lsb_vs_full"] = int(np.abs(full.rgba.astype(int) - term.rgba.astype(int)).max())
        out["max_abs_vs_full"] = float(np.abs(full.v - term.v).max())
        out["opaque_ray_fraction"] = float((full.v[..., 3] >= t).mean())
        out["config"] = {"workload": f"{w.name}_Volume_density1", "sampler": "gathers"
                         if vol.gather_sampling else "loads"}
        return out
    finally:
        vol.close()


def configs_leg(hy, ctx, dev, reps=5, row_step=16):
    """The plain-Volume and the tubes configurations at their stated sizes,
    one view each (per-view fused kernel; the L2 written over between timed
    launches, CUDA events on the library's stream), each image checked
    against the oracle: the whole 512^2 frame for the plain Volume
    configuration, every 16th row for the 1024^2 tubes variants (max LSB of
    RGBA8, max abs of the floats, equal sample counts)."""
    import numpy as np
    import torch

    from hydrant_gb300 import workloads as wl
    from oracle import oracle as orc

    stream = torch.cuda.ExternalStream(ctx.stream)
    flush = torch.empty(512 * 2**20, dtype=torch.uint8, device=dev)
    out = {}

    def one(name, w, vol, ov, kw, rows):
        cam = wl.make_camera(w.views[0].camera)
        view = hy.camera_view(vol, cam)
        W = H = w.views[0].width
        p = hy.shader_params(count_samples=True, **kw)
        if p.shader == hy._abi.SHADER_ISOSURFACE:
            hy.iso_lighting(vol, cam, p)
        g = hy.render(ctx, vol, p, view, W, H, want_v=True)
        y0 = 0 if rows == 1 else rows // 2
        r = orc.render_row_step(ov, w.tf, orc.params_from(p), view_array(view), W, H, y0, rows,
                                want_v=True)
        q = hy.shader_params(**kw)
        if q.shader == hy._abi.SHADER_ISOSURFACE:
            hy.iso_lighting(vol, cam, q)
        buf = torch.empty(W * H * 4, dtype=torch.uint8, device=dev)
        evs = _timed_steps(torch, stream, reps,
                           lambda: hy.render_device(ctx, vol, q, view, W, H, buf.data_ptr()),
                           flush)
        ctx.synchronize()
        ms = sum(a.elapsed_time(b) for a, b in evs) / reps
        gs = g.samples
        # the sample count of the GPU image on the checked rows
        lsb = int(np.abs(g.rgba[y0::rows].astype(int) - r["rgba"][y0::rows].astype(int)).max())
        fab = float(np.abs(g.v[y0::rows].astype(np.float64) - r["v"][y0::rows]).max())
        out[name] = {"ms_per_view": ms, "samples": gs, "gsamples_per_s": gs / ms / 1e6,
                     "resolution": W, "parity_vs_oracle": {
                         "rows": "all" if rows == 1 else f"every {rows}th row",
                         "max_lsb": lsb, "max_abs": fab,
                         "samples_equal": (gs == r["samples"]) if rows == 1 else None}}

    w0 = wl.volume_c0()
    vox = hy.synth_blobs_u8(w0.seed, w0.dim, w0.count)
    vol = hy.Volume(ctx, vox, w0.block_size, w0.padding)
    try:
        ctx.set_transfer_fn(w0.tf)
        one(w0.name + "_Volume", w0, vol, orc.OracleVolume(vox, w0.block_size, w0.padding),
            w0.params, 1)
    finally:
        vol.close()
    w1 = wl.tubes_c1()
    vox = hy.synth_tubes_u8(w1.seed, w1.dim, w1.count)
    vol = hy.Volume(ctx, vox, w1.block_size, w1.padding)
    ov = orc.OracleVolume(vox, w1.block_size, w1.padding)
    try:
        ctx.set_transfer_fn(w1.tf)
        one(w1.name + "_Isosurface_Color", w1, vol, ov, w1.params, row_step)
        for mode in ("Volume", "Solid"):
            one(f"{w1.name}_Blocks_{mode}_composite", w1, vol, ov,
                dict(shader="Blocks", mode=mode, density=1e-2, composite=True), row_step)
    finally:
        vol.close()
    return out


def view_array(view):
    """A product view (hy_view) as the oracle's 20 floats."""
    import numpy as np

    return np.array(list(view.trans) + [view.ctg_fovy_2] + list(view.ray_o), np.float32)


def sampled_parity(hy, ctx, vol, w, ov, views, params, cviews, imgs, batch, flat, step, nth):
    """The timed batch kernel's images against the oracle on the CPU
    sample's rows of every view (max LSB of RGBA8), and the pre-quantisation
    floats of the largest view (the per-view lean kernel with a float
    output, same march) against the oracle's on those rows."""
    import numpy as np

    lsb = 0
    rows = 0
    for i, (img, r) in enumerate(zip(batch.split(flat), imgs)):
        H = img.shape[0]
        y0, _ = sample_rows(H, step)
        d = np.abs(img[y0::step].astype(np.int32) - r["rgba"][y0::step].astype(np.int32))
        lsb = max(lsb, int(d.max()))
        rows += d.shape[0]
    big = max(range(len(views)), key=lambda i: views[i][1] * views[i][2])
    v, W, H = views[big]
    _, fl = cpu_step(w, ov, cviews, step, nth, want_v=True, only={big})
    g = hy.render(ctx, vol, params[big], v, W, H, want_v=True)
    y0, _ = sample_rows(H, step)
    fab = float(np.abs(g.v[y0::step].astype(np.float64) - fl[big]["v"][y0::step]).max())
    return {"rows": f"{rows} sampled rows over all {len(views)} views (batch kernel, RGBA8); "
                    f"floats on the {W}x{H} view", "max_lsb": lsb, "max_abs": fab,
            "bar": "<= 1 LSB, <= 1e-4"}


def _timed_steps(torch, stream, steps, fn, flush=None):
    """Run `steps` calls of fn, each bracketed by CUDA events on `stream`;
    a flush buffer (if any) is written between steps outside the events."""
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(steps)]
    for k in range(steps):
        if flush is not None:
            with torch.cuda.stream(stream):
                flush.fill_(k & 0xFF)
        evs[k][0].record(stream)
        fn()
        evs[k][1].record(stream)
    return evs


def main_ours(args):
    import numpy as np
    import torch

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    build_all()
    import hydrant_gb300 as hy
    from hydrant_gb300 import autotune
    from hydrant_gb300 import workloads as wl

    dev = f"cuda:{local}"
    w = workload(args)
    t0 = time.perf_counter()
    vox = {"blobs_u8": hy.synth_blobs_u8, "tubes_u8": hy.synth_tubes_u8,
           "blobs_f32": hy.synth_blobs_f32}[w.generator](w.seed, w.dim, w.count)
    t_gen = time.perf_counter() - t0
    ctx = hy.Context(local)
    t0 = time.perf_counter()
    vol = hy.Volume(ctx, vox, w.block_size, w.padding)
    t_up = time.perf_counter() - t0
    ctx.set_transfer_fn(w.tf)
    vol.set_gather_sampling(args.sampler == "gather")
    info = vol.info

    views, params, lighting, bufs = [], [], [], []
    for v in w.views:
        cam = wl.make_camera(v.camera)
        p = hy.shader_params(**w.params)
        if p.shader == hy._abi.SHADER_ISOSURFACE:
            hy.iso_lighting(vol, cam, p)
        views.append((hy.camera_view(vol, cam), v.width, v.height))
        params.append(p)
        lighting.append((list(p.eye_pos), list(p.light_pos)))
        bufs.append(torch.empty(v.height * v.width * 4, dtype=torch.uint8, device=dev))
    npix = sum(W * H for _, W, H in views)
    stream = torch.cuda.ExternalStream(ctx.stream)
    # L2 is 129 MB: when the brick pool is smaller, a 512 MB buffer is written
    # between timed steps (outside the timed events) so every step starts cold.
    flush = None
    if info.pool_bytes < 256 * 2**20:
        flush = torch.empty(512 * 2**20, dtype=torch.uint8, device=dev)

    # ---- plain per-view path: one fused launch per view -------------------
    samples = 0
    for (view, W, H), p, b in zip(views, params, bufs):
        p.count_samples = 1
        hy.render_device(ctx, vol, p, view, W, H, b.data_ptr())
        samples += ctx.stats().samples
        p.count_samples = 0

    def plain_step():
        for (view, W, H), p, b in zip(views, params, bufs):
            hy.render_device(ctx, vol, p, view, W, H, b.data_ptr())

    for _ in range(args.warmup):
        plain_step()
    ctx.synchronize()
    evs = _timed_steps(torch, stream, args.steps, plain_step, flush)
    ctx.synchronize()
    t_plain = sum(a.elapsed_time(b) for a, b in evs) / 1e3

    # ---- the reference's pass structure per view: the emit pass marches
    # into a film in HBM (64 B/px for the Volume shader), the pixel pass
    # writes the RGB8 image (raycaster.hpp:32-123) -- pass-level ABI --------
    t_passes = None
    if not args.composite:
        max_px = max(W * H for _, W, H in views)
        film = torch.empty(max_px * 64, dtype=torch.uint8, device=dev)
        rgb = torch.empty(max_px * 3, dtype=torch.uint8, device=dev)

        def passes_step():
            for (view, W, H), p in zip(views, params):
                hy.shade_pass(ctx, vol, p, hy._abi.PASS_RAY_EMIT, view, film.data_ptr(), W, H)
                hy.shade_pass(ctx, vol, p, hy._abi.PASS_PIXEL, None, film.data_ptr(), W, H,
                              rgb.data_ptr())

        for _ in range(args.warmup):
            passes_step()
        ctx.synchronize()
        evs = _timed_steps(torch, stream, args.steps, passes_step, flush)
        ctx.synchronize()
        t_passes = sum(a.elapsed_time(b) for a, b in evs) / 1e3
        del film, rgb

    # ---- batched path: one persistent launch per step, graph replay -------
    batch = hy.Batch(ctx, vol, params[0], views, lighting)
    out = torch.empty(batch.nbytes, dtype=torch.uint8, device=dev)
    key = autotune.signature(torch.cuda.get_device_name(local), params[0], vol.desc,
                             [(W, H) for _, W, H in views])
    if args.launch_shape:
        batch.set_config(*[int(x) for x in args.launch_shape.split(",")])
    if args.no_autotune or args.launch_shape:
        c = batch.config
        tuned = {"tile_w": c.tile_w, "grab": c.grab, "block_warps": c.block_warps,
                 "blocks_per_sm": c.blocks_per_sm, "block_queue": c.block_queue,
                 "steps_per_iter": max(1, c.steps_per_iter),
                 "source": "fixed" if args.launch_shape else "default"}
    else:
        tuned = autotune.tuned_config(batch, key, out.data_ptr(), reps=1)
    batch.set_counting(True)
    batch.render_device(out.data_ptr())
    samples_b = ctx.stats().samples
    batch.set_counting(False)
    # the batch reproduces the per-view images exactly
    ref = np.concatenate([b.cpu().numpy() for b in bufs])
    same = bool(np.array_equal(out.cpu().numpy()[: ref.size], ref))

    for _ in range(args.warmup):
        batch.render_device(out.data_ptr())
    ctx.synchronize()
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    clocks = Clocks(local)
    clocks.start()
    evs = _timed_steps(torch, stream, args.steps, lambda: batch.render_device(out.data_ptr()), flush)
    ctx.synchronize()
    torch.cuda.synchronize()
    ck = clocks.stop()
    step_ms = [a.elapsed_time(b) for a, b in evs]
    t = sum(step_ms) / 1e3
    if ws > 1:
        t, t_plain = max_over_ranks([t, t_plain], dev)
        if t_passes is not None:
            (t_passes,) = max_over_ranks([t_passes], dev)
        torch.distributed.barrier()

    # ---- e2e: a frame loop through the host entry points.  Every step
    # carries new cameras (the step's 64 cameras turned by 0.5 degrees about
    # the vertical axis from the previous step's) from host memory into the
    # batch (hy_batch_update_views: the descriptors are copied to the device
    # on the stream) and renders into a pinned host buffer (hy_batch_render:
    # the images cross the host link as the kernel writes them).
    host_t = torch.empty(batch.nbytes, dtype=torch.uint8, pin_memory=True)
    host = host_t.numpy()
    base_cams = [wl.make_camera(v.camera) for v in w.views]

    def turned_views(k):
        a = math.radians(0.5 * k)
        ca, sa = math.cos(a), math.sin(a)
        out = []
        for cam, (_, W, H) in zip(base_cams, views):
            x, y, z = cam.position
            c = hy.camera_ptu((ca * x + sa * z, y, -sa * x + ca * z), tuple(cam.target),
                              tuple(cam.up))
            out.append((hy.camera_view(vol, c), W, H))
        return batch.view_array(out)

    nwarm_e2e = max(1, args.warmup // 2)
    frames = [turned_views(k + 1) for k in range(nwarm_e2e + args.steps)]
    e2e_samples = 0
    batch.set_counting(True)
    for arr in frames[nwarm_e2e:]:
        batch.update_views(arr)
        batch.render_device(out.data_ptr())
        e2e_samples += ctx.stats().samples
    batch.set_counting(False)
    for arr in frames[:nwarm_e2e]:
        batch.update_views(arr)
        batch.render()
    ctx.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    lib_ = hy.lib()
    te = time.perf_counter()
    for arr in frames[nwarm_e2e:]:
        ctx.check(lib_.hy_batch_update_views(batch.handle, arr, len(arr)))
        ctx.check(lib_.hy_batch_render(batch.handle, host.ctypes.data_as(ctypes.c_void_p)))
    ctx.synchronize()
    t_e2e = time.perf_counter() - te
    if ws > 1:
        (t_e2e,) = max_over_ranks([t_e2e], dev)
    # back to the step's own cameras: `out` holds their images for the
    # parity check against the oracle
    batch.update_views(batch.view_array(views))
    batch.render_device(out.data_ptr())
    ctx.synchronize()

    # ---- the configuration's compositing variant and the differentiable
    # configuration, each at its stated size (rank 0 of a 1-GPU run) -------
    composite = diff = ert = others = paging = None
    if ws == 1 and not args.no_extra:
        if not args.composite:
            composite = composite_leg(hy, ctx, vol, w, views, lighting, stream, flush, args)
        diff = diff_leg(hy, ctx, dev)
        ert = ert_leg(hy, ctx, dev)
        others = configs_leg(hy, ctx, dev)
        pargs = argparse.Namespace(**vars(args))
        pargs.warmup = 3
        paging = paging_leg(pargs, hy, ctx, local)
        ctx.set_transfer_fn(w.tf)

    value = aggregate_gsamples(samples, ws, args.steps, t)
    plain_value = aggregate_gsamples(samples, ws, args.steps, t_plain)
    e2e = e2e_samples * ws / t_e2e / 1e9
    hbm, peak_kind = measured_peaks()
    mean_launch_s = t / args.steps  # one batch kernel per step
    achieved = samples * BYTES_PER_SAMPLE / mean_launch_s / 1e9
    # the profiled per-sample figures hold for the Volume shader on the blob
    # volume they were captured on, not for the other workloads
    tps = ipsm = None
    overridden = (args.shader or args.mode or args.composite or args.sample_rate > 0
                  or args.density is not None)
    if args.workload == "multiview" and not overridden:
        smp = "gather" if vol.gather_sampling else "loads"
        tps = profile_per_sample(int(tuned.get("block_queue", 1)), sampler=smp)
        ipsm = profile_per_sample(int(tuned.get("block_queue", 1)),
                                  "warp_instructions_per_sample", sampler=smp)
    if rank == 0:
        from oracle import oracle as orc

        cpu = None
        parity = None
        nth = os.cpu_count() or 1
        ov = orc.OracleVolume(vox, w.block_size, w.padding)
        if not args.no_cpu_baseline:
            step = max(1, args.cpu_row_step)
            cviews = cpu_views(w, ov, [view_array(v) for v, _, _ in views])
            t0 = time.perf_counter()
            s, imgs = cpu_step(w, ov, cviews, step, nth)
            dt = time.perf_counter() - t0
            cpu = {"value": s / dt / 1e9, "unit": "Gsamples/s", "cores": nth, "kind": "port",
                   "sample": sample_desc(w, step, s) + f", {dt:.2f} s", "cpu": cpu_model()}
            parity = sampled_parity(hy, ctx, vol, w, ov, views, params, cviews, imgs, batch,
                                    out.cpu().numpy(), step, nth)
        out_json = {
            "metric": "Gsamples/s",
            "value": value,
            "unit": "Gsamples/s",
            "n_gpus": ws,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": t / args.steps * 1e3,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f32",
            "data": "synthetic",
            "config": workload_config(w, ov),
            "samples_per_step": samples,
            "path": "batched: one persistent launch per step from a CUDA graph",
            "sampler": ("two texture gathers per sample (u8 bricks in gather textures)"
                        if vol.gather_sampling else "eight loads per sample from the brick pool"),
            "launch_shape": tuned,
            "views_per_s": len(views) * ws * args.steps / t,
            "plain": {"value": plain_value, "unit": "Gsamples/s",
                      "views_per_s": len(views) * ws * args.steps / t_plain,
                      "ms_per_step": t_plain / args.steps * 1e3,
                      "path": "one fused hy_render_device launch per view"},
            "batched_over_plain": t_plain / t,
            "passes": None if t_passes is None else {
                "value": aggregate_gsamples(samples, ws, args.steps, t_passes),
                "unit": "Gsamples/s", "views_per_s": len(views) * ws * args.steps / t_passes,
                "ms_per_step": t_passes / args.steps * 1e3,
                "path": "per view: emit pass (march into a 64 B/px film) + pixel pass, "
                        "the reference's pass structure through hy_shade_pass"},
            "batched_over_passes": None if t_passes is None else t_passes / t,
            "batch_matches_plain": same and samples_b == samples,
            "e2e": {"value": e2e, "unit": "Gsamples/s",
                    "h2d_bytes_per_step": batch.view_bytes,
                    "d2h_bytes_per_step": batch.nbytes,
                    "samples": e2e_samples,
                    "views_per_s": len(views) * ws * args.steps / t_e2e,
                    "path": "per step: the step's new cameras through hy_batch_update_views "
                            "(view descriptors host -> device on the stream), then "
                            "hy_batch_render into a pinned, mapped host buffer (the kernel "
                            "writes the pixels across the host link while it marches); "
                            "host wall clock around the loop"},
            "roofline": {
                "bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                "frac": achieved / hbm, "peak_kind": peak_kind,
                "traffic": (tps * samples) if tps else None,
                "note": "8 B/sample algorithmic footprint; the march is bound by L1 latency and instruction issue, not HBM",
            },
            "issue_roofline": issue_roofline(ipsm, samples, mean_launch_s, ck, local),
            "cpu_baseline": cpu,
            "parity_vs_oracle": parity,
            "gpu_launches": args.steps,
            "clocks": ck,
            "setup_s": {"generate": t_gen, "upload_and_brick": t_up},
            "composite": composite,
            "diff": diff,
            "early_termination": ert,
            "other_configs": others,
            "paging": paging,
        }
        print(json.dumps(out_json), flush=True)
    batch.close()
    vol.close()
    ctx.close()
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


def main_paging(args):
    """Out-of-core configuration: 4096x4096x2048 u8 procedural value noise
    (3 octaves, 256-voxel cells, 15% occupancy) in 64^3 bricks held in a
    pinned host store; an 8 GiB device brick cache (realtime pager) renders a
    120-frame orbit (azimuth +3 deg/frame) at 2048^2, density 5e-3.  With
    --coarse-level L the store's 2^L box-filtered level stays resident and
    bricks not (yet) in the cache are drawn from it."""
    import torch

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    build_all()
    import hydrant_gb300 as hy

    ctx = hy.Context(local)
    outj = paging_leg(args, hy, ctx, local, with_clocks=True)
    print(json.dumps(outj), flush=True)
    ctx.close()
    return 0


def paging_leg(args, hy, ctx, local, with_clocks=False):
    """The out-of-core frames (main_paging's workload); returns its JSON line."""
    import torch

    from hydrant_gb300 import _abi
    from hydrant_gb300 import workloads as wl

    sc = max(1, args.paging_scale)
    dim = (4096 // sc, 4096 // sc, 2048 // sc)
    res = 2048 // sc
    ctx.set_transfer_fn(wl.TF9)
    t0 = time.perf_counter()
    store = hy.Store.noise(ctx, dim, 64, 1, seed=2, cell_voxels=256.0 / sc, occupancy=0.15)
    t_store = time.perf_counter() - t0
    t1 = time.perf_counter()
    if args.coarse_level > 0:
        store.build_coarse(args.coarse_level)
    t_coarse = time.perf_counter() - t1
    si = store.info
    if args.pager == "lossless":
        slots = args.lossless_batch
        pg = hy.Pager(ctx, store, slots, _abi.PAGER_LOSSLESS)
    else:
        budget = int(args.cache_gib * 2**30)
        frames_ = max(1, args.frames)
        path = [hy.camera_orbit((3.0 * f, 30.0, 2.2)) for f in range(frames_)]
        if args.no_tune_cache:
            slots, most = int(budget // si.slot_bytes), None
        else:
            # the cache sized to the orbit (the most visible bricks + 10 %),
            # within the --cache-gib budget
            slots, most = hy.Pager.tune_slots(ctx, store, path, budget)
        ev = _abi.EVICT_REFERENCE if args.eviction == "reference" else _abi.EVICT_LRU
        smp = _abi.PAGER_GATHERS if args.pager_sampler == "gathers" else _abi.PAGER_LOADS
        pg = hy.Pager(ctx, store, slots, _abi.PAGER_REALTIME, args.max_uploads, ev, smp)
    p = hy.shader_params(shader="Volume", sample_rate=0.25, density=5e-3)
    pc = hy.shader_params(shader="Volume", sample_rate=0.25, density=5e-3, count_samples=True)
    out = torch.empty(res * res * 4, dtype=torch.uint8, device=f"cuda:{local}")
    stream = torch.cuda.ExternalStream(ctx.stream)
    frames = max(1, args.frames)
    # warm-up frames on a different arc so the timed orbit starts cold
    for f in range(args.warmup):
        pg.render(p, hy.camera_orbit((-90.0 - 3 * f, 30.0, 2.2)), res, res, out.data_ptr())
    ctx.synchronize()
    st0 = pg.stats()
    clocks = Clocks(local) if with_clocks else None
    if clocks:
        clocks.start()
    fallback = 0
    tw = time.perf_counter()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    prefetch = args.prefetch and args.pager == "realtime"
    for f in range(frames):
        pg.render(p, hy.camera_orbit((3.0 * f, 30.0, 2.2)), res, res, out.data_ptr())
        if prefetch:  # the orbit's next camera, moved in while this frame renders
            pg.prefetch(hy.camera_orbit((3.0 * (f + 1), 30.0, 2.2)))
        fallback += pg.stats()["fallback"]
    ev1.record(stream)
    ctx.synchronize()
    wall = time.perf_counter() - tw
    ck = clocks.stop() if clocks else None
    gpu_s = ev0.elapsed_time(ev1) / 1e3
    st = pg.stats()
    d = {k: st[k] - st0[k] for k in st}
    # samples: a second, untimed pass over the same orbit with counting on
    # (reading the counter synchronises every frame).  With the coarse level
    # every visible brick is sampled, so the count does not depend on what
    # the cache holds; without it the second pass starts from a warmer cache.
    samples = 0
    last_pass_ms = 0.0
    for f in range(frames):
        pg.render(pc, hy.camera_orbit((3.0 * f, 30.0, 2.2)), res, res, out.data_ptr())
        st_f = ctx.stats()
        samples += st_f.samples
        last_pass_ms += st_f.ms
    lookups = d["hits"] + d["misses"]
    outj = {
        "metric": "frames/s", "value": frames / wall, "unit": "frames/s", "n_gpus": 1,
        "steps": frames, "warmup": args.warmup, "ms_per_step": wall / frames * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": f"paging_{dim[0]}x{dim[1]}x{dim[2]}_{res}px", "block_size": 64,
                   "pager": args.pager,
                   "cache_gib": args.cache_gib if args.pager == "realtime" else None,
                   "cache_slots": slots, "store_bricks": si.nonempty,
                   "cache_tuned": None if args.pager != "realtime" or args.no_tune_cache else {
                       "slots": slots, "gib": slots * si.slot_bytes / 2**30,
                       "most_visible_bricks": most, "budget_gib": args.cache_gib,
                       "rule": "most visible bricks over the orbit + 10 %, within the budget"},
                   "eviction": args.eviction if args.pager == "realtime" else None,
                   "cache_sampler": args.pager_sampler if args.pager == "realtime" else None,
                   "store_gb": si.pool_bytes / 1e9, "store_build_s": t_store,
                   "coarse_level": args.coarse_level, "coarse_build_s": t_coarse,
                   "max_uploads_per_frame": args.max_uploads},
        "gsamples_per_s": samples / wall / 1e9,
        "samples_per_frame": samples / frames,
        "gpu_s": gpu_s, "wall_s": wall,
        "cache_hit_rate": (d["hits"] / lookups) if lookups else None,
        "uploads_per_frame": d["uploads"] / frames,
        "prefetched_per_frame": d["prefetched"] / frames,
        "prefetch": bool(prefetch),
        "passes_per_frame": d["passes"] / frames,
        "last_pass_ms_per_frame": last_pass_ms / frames,
        "upload_gb_per_s": d["upload_bytes"] / wall / 1e9,
        "evictions": d["evictions"], "visible_last_frame": st["visible"],
        "coarse_bricks_per_frame": fallback / frames,
        "clocks": ck,
    }
    pg.close()
    store.close()
    return outj


DIFF_CONFIG = dict(n=256, res=512, views=16, knots=32, ckpt_k=32, blobs=24)


def diff_leg(hy, ctx, dev, reps=5, fd_params=4, ckpt_k=None):
    """The differentiable configuration at its stated size: 256^3 f32 blob
    density (seed 4 truth, seed 5 estimate), 32-knot TF, 16 views of 512^2
    on a seeded orbit, checkpoints every 32 steps.  Times (CUDA events on the
    library's stream, every launch on that stream) the forward without and
    with checkpoints and the adjoint, per view; and checks the adjoint's
    gradient of the L2 image loss against central finite differences
    (eps 1e-3, loss in float64) on the largest knot and voxel gradients and
    along a random direction over all knots."""
    import numpy as np
    import torch

    from hydrant_gb300 import fit

    c = DIFF_CONFIG
    n, res, nv, ntf = c["n"], c["res"], c["views"], c["knots"]
    K = ckpt_k or c["ckpt_k"]
    vt = hy.synth_blobs_f32(4, (n, n, n), c["blobs"])
    vi = hy.synth_blobs_f32(5, (n, n, n), c["blobs"])
    holder = hy.Volume(ctx, vt, n, 1)
    views = fit.orbit_views(holder, 4, nv)
    holder.close()
    tft = fit.seeded_tf(4, ntf)
    r = fit.DiffRenderer(ctx, n, views, res, res, ntf, ckpt_k=K)
    out = {}
    with torch.cuda.stream(r.stream):
        target = r.forward(torch.from_numpy(vt).to(dev), torch.from_numpy(tft).to(dev),
                           keep=False).clone()
        vol = torch.from_numpy(vi).to(dev)
        # a non-uniform TF (the fit starts from uniform grey, where the image
        # does not depend on the voxels at all)
        tf = torch.from_numpy(np.clip(tft * 0.8 + 0.1, 0, 1).astype(np.float32)).to(dev)

        def timed(fn):
            for _ in range(2):
                fn()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(r.stream)
            for _ in range(reps):
                fn()
            e1.record(r.stream)
            e1.synchronize()
            return e0.elapsed_time(e1) / reps / nv

        img = r.forward(vol, tf, keep=True)
        g = (2.0 / img.numel()) * (img - target)
        fwd = timed(lambda: r.forward(vol, tf, keep=False))
        fwd_k = timed(lambda: r.forward(vol, tf, keep=True))
        bwd = timed(lambda: r.backward(vol, tf, g))
        r.forward(vol, tf, keep=True)
        dvol, dtf = r.backward(vol, tf, g)

        def loss64(v, t):
            im = r.forward(v, t, keep=False)
            return float(((im.double() - target.double()) ** 2).mean())

        eps = 1e-3
        checks = []
        gt = dtf.reshape(-1)
        for idx in torch.topk(gt.abs(), fd_params).indices.tolist():
            tp, tm = tf.clone(), tf.clone()
            tp.view(-1)[idx] += eps
            tm.view(-1)[idx] -= eps
            fd = (loss64(vol, tp) - loss64(vol, tm)) / (2 * eps)
            checks.append(("knot", idx, float(gt[idx]), fd))
        gv = dvol.reshape(-1)
        for idx in torch.topk(gv.abs(), fd_params).indices.tolist():
            vp, vm = vol.clone(), vol.clone()
            vp.view(-1)[idx] += eps
            vm.view(-1)[idx] -= eps
            fd = (loss64(vp, tf) - loss64(vm, tf)) / (2 * eps)
            checks.append(("voxel", idx, float(gv[idx]), fd))
        gen = torch.Generator(device="cpu").manual_seed(7)
        d = torch.randn(tf.shape, generator=gen).to(dev)
        fd = (loss64(vol, tf + eps * d) - loss64(vol, tf - eps * d)) / (2 * eps)
        checks.append(("knot direction", -1, float((dtf * d).sum()), fd))
    torch.cuda.synchronize()
    rel = [abs(a - f) / max(abs(f), 1e-30) for _, _, a, f in checks]
    l2 = math.sqrt(sum((a - f) ** 2 for _, _, a, f in checks) /
                   max(sum(f ** 2 for _, _, _, f in checks), 1e-300))
    out.update({
        "config": {"workload": f"diff_{n}cube_{nv}x{res}px_{ntf}knots_K{K}", "volume": [n, n, n],
                   "dtype": "f32", "views": nv, "resolution": res, "knots": ntf, "ckpt_k": K},
        "forward_ms_per_view": fwd,
        "forward_ckpt_ms_per_view": fwd_k,
        "adjoint_ms_per_view": bwd,
        "fwd_adjoint_ms_per_view": fwd_k + bwd,
        "fwd_adjoint_over_forward": (fwd_k + bwd) / fwd,
        "fwd_adjoint_over_forward_ckpt": (fwd_k + bwd) / fwd_k,
        "fd_check": {"eps": eps, "loss": "mean squared image error (float64)",
                     "max_rel_err": max(rel), "l2_rel_err": l2,
                     "cases": [{"param": k, "index": i, "adjoint": a, "fd": f,
                                "rel_err": e} for (k, i, a, f), e in zip(checks, rel)]},
        "timing": "CUDA events on the library stream, mean of %d launches after 2 warm-up" % reps,
    })
    r.ckpt = None
    return out


def main_diff(args):
    """Differentiable fit: 256^3 f32 blob density (seed 4 truth, seed 5 init),
    32-knot RGBA TF (seeded truth, uniform grey init), 16 views of 512^2 on a
    seeded orbit, L2 image loss, checkpoints every --ckpt-k (32) steps, Adam
    for --frames iterations (default 200 here); the kernel timings and the
    finite-difference check of diff_leg beside it."""
    import numpy as np
    import torch

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    build_all()
    import hydrant_gb300 as hy
    from hydrant_gb300 import fit

    n, res, nviews, ntf = 256, 512, args.diff_views, 32
    steps = args.frames if args.frames != 120 else 200
    ctx = hy.Context(local)
    vt = hy.synth_blobs_f32(4, (n, n, n), 24)
    vi = hy.synth_blobs_f32(5, (n, n, n), 24)
    holder = hy.Volume(ctx, vt, n, 1)
    views = fit.orbit_views(holder, 4, nviews)
    holder.close()
    tft = fit.seeded_tf(4, ntf)
    tfi = np.full((ntf, 4), 0.5, np.float32)
    t0 = time.perf_counter()
    warm = max(3, args.warmup)
    K = args.ckpt_k
    res_fit = fit.fit(ctx, vt, vi, views, res, res, tft, tfi, steps=steps, ckpt_k=K, warmup=warm)
    wall = time.perf_counter() - t0
    kernels = None if args.no_extra else diff_leg(hy, ctx, f"cuda:{local}", ckpt_k=K)
    out = {
        "metric": "fwd+adjoint ms/view", "value": res_fit.fwd_adj_ms_per_view, "unit": "ms/view",
        "n_gpus": 1, "steps": steps, "warmup": warm, "higher_is_better": False, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": f"diff_fit_{n}cube_{nviews}x{res}px_{ntf}knots", "ckpt_k": K},
        "forward_ms_per_view": res_fit.fwd_ms_per_view,
        "adjoint_over_forward": res_fit.fwd_adj_ms_per_view / res_fit.fwd_ms_per_view,
        "iteration_ms_median": float(np.median(res_fit.iter_ms)),
        "loss_first": res_fit.losses[0], "loss_last": res_fit.losses[-1],
        "loss_curve": res_fit.losses[:: max(1, steps // 20)],
        "wall_s": wall,
        "kernels": kernels,
    }
    print(json.dumps(out), flush=True)
    ctx.close()
    return 0


def main():
    args = parse_args()
    if args.impl == "reference":
        return main_reference(args)
    if args.workload == "paging":
        return main_paging(args)
    if args.workload == "diff":
        return main_diff(args)
    return main_ours(args)


if __name__ == "__main__":
    sys.exit(main())
