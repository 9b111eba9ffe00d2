"""hydrant_gb300: GB300-native ray-marching path of Hydrant.

C ABI in include/hydrant_gb300.h over hand-written sm_103a kernels
(hydrant_gb300/csrc).  This package is the ctypes harness used by the
tests, the benchmark and the renderer-interface mirror.
"""

from ._abi import HydrantError, lib  # noqa: F401
from .api import (  # noqa: F401
    Batch,
    Context,
    RenderResult,
    Volume,
    Pager,
    Store,
    camera_orbit,
    camera_ptu,
    camera_view,
    cull,
    iso_lighting,
    render,
    render_device,
    shade_pass,
    shader_params,
    synth_blobs_f32,
    synth_blobs_u8,
    synth_tubes_u8,
)
from . import workloads  # noqa: F401
