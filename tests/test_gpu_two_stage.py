"""The two-kernel RAY frame (RC_TRACE_FUSED=0: a primary kernel that queues
the hit pixels, then a shadow kernel over the queue) gives the float32
oracle's records bit for bit, like the default one-kernel frame (each shadow
ray traced where its primary hit was found) that the other tests check: camera
frames in both orders, and a 1080p caller-ray frame from host buffers equal to
the camera frame. The switch is read once per process, so the checks run in a
child process."""

from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

_CHECKS = """
import sys
sys.path.insert(0, {root!r})
sys.path.insert(0, {tests!r})
import numpy as np
import oracle
from raycer_gb300 import _native as N
from raycer_gb300.tracer import RAY_DTYPE, CudaTracer, TracerState, camera_record
from helpers import camera_floats, small_heightfield, small_room

for which in ("room", "heightfield"):
    for order in (N.RC_ORDER_REFERENCE, N.RC_ORDER_NEAREST):
        sc = small_room() if which == "room" else small_heightfield()
        sc.settings["tracer"] = "ray"
        # lights under which both scenes have shadowed pixels
        sc.light_direction = (-0.3, -1.0, -0.2) if which == "room" else (-1.0, -0.25, -0.2)
        with CudaTracer(0) as t:
            t.initializeBuffers(sc)
            t.set_traversal_order(order)
            t.initializeImageBuffers(sc.width, sc.height)
            t.run(TracerState(scene=sc, filmWidth=sc.width, filmHeight=sc.height, pixelCount=sc.width * sc.height))
            gpu = t.read_cast().view(np.int32).reshape(-1, 4)
            st = t.stats()
        assert st["stage_ms"][1] > 0.0, "the shadow kernel did not run as its own launch"
        L = -np.array(sc.light_direction, np.float32)
        ref, _ = oracle.Oracle(sc).raycast32(camera_floats(camera_record(sc)), sc.width, sc.width * sc.height, L,
                                             order=order)
        assert np.array_equal(gpu, ref), (which, order, int((gpu != ref).any(axis=1).sum()))
        assert (ref[:, 2] >= 0).any(), "no occluded pixel"

sc = small_heightfield(width=1920, height=1080)
sc.settings["tracer"] = "ray"
n = sc.width * sc.height
with CudaTracer(0) as t:
    t.initializeBuffers(sc)
    t.initializeImageBuffers(sc.width, sc.height)
    t.run(TracerState(scene=sc, filmWidth=sc.width, filmHeight=sc.height, pixelCount=n))
    frame = t.read_cast()
    rays = oracle.camera_rays32(camera_floats(camera_record(sc)), sc.width, n)
    out = t.cast_with_shadow(np.ascontiguousarray(rays).view(RAY_DTYPE).reshape(-1))
    stats = t.stats()
assert np.array_equal(out, frame)
assert stats["rays_traced"] == n + int((frame["prim"] >= 0).sum())
print("two-stage ok")
"""


def test_two_kernel_frame_matches_oracle():
    tests = Path(__file__).resolve().parent
    root = str(tests.parent)
    env = dict(os.environ, RC_TRACE_FUSED="0")
    out = subprocess.run([sys.executable, "-c", _CHECKS.format(root=root, tests=str(tests))], env=env,
                         capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stdout[-2000:] + out.stderr[-4000:]
    assert "two-stage ok" in out.stdout


def test_one_kernel_frame_has_no_second_stage():
    """The default frame is one launch: the second stage's time is 0 and the
    rays traced count the shadow rays all the same."""
    import numpy as np

    from raycer_gb300.tracer import CudaTracer, TracerState

    from helpers import small_heightfield

    sc = small_heightfield()
    sc.settings["tracer"] = "ray"
    n = sc.width * sc.height
    with CudaTracer(0) as t:
        t.initializeBuffers(sc)
        t.initializeImageBuffers(sc.width, sc.height)
        t.run(TracerState(scene=sc, filmWidth=sc.width, filmHeight=sc.height, pixelCount=n))
        frame = t.read_cast()
        st = t.stats()
    assert st["stage_ms"][1] == 0.0
    assert st["rays_traced"] == n + int((frame["prim"] >= 0).sum())
    assert int((frame["prim"] >= 0).sum()) > 0
