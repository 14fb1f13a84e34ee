"""The stackless reference-order walk (RC_STACKLESS=1: the rope records,
no traversal stack) gives the float32 oracle's results bit for bit: RAY
frames in both orders (their shadow rays walk it) and reference-order
rc_cast queries, closest and any hit. The switch is read once per process,
so the checks run in a child process."""

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
from raycer_gb300.tracer import CudaTracer, TracerState, camera_record
from helpers import camera_floats, small_heightfield, small_room

for which in ("room", "heightfield"):
    for order in (N.RC_ORDER_REFERENCE, N.RC_ORDER_NEAREST):
        sc = small_room() if which == "room" else small_heightfield()
        sc.settings["tracer"] = "ray"
        if which == "room":
            sc.light_direction = (-0.3, -1.0, -0.2)
        with CudaTracer(0) as t:
            t.initializeBuffers(sc)
            t.set_traversal_order(order)
            t.initializeImageBuffers(sc.width, sc.height)
            t.run(TracerState(scene=sc, filmWidth=sc.width, filmHeight=sc.height, pixelCount=sc.width * sc.height))
            gpu = t.read_cast().view(np.int32).reshape(-1, 4)
        L = -np.array(sc.light_direction, np.float32)
        ref, _ = oracle.Oracle(sc).raycast32(camera_floats(camera_record(sc)), sc.width, sc.width * sc.height, L,
                                             order=order)
        assert np.array_equal(gpu, ref), (which, order, int((gpu != ref).any(axis=1).sum()))

sc = small_room(clutter=1000)
rng = np.random.default_rng(5)
n = 100_000
rays = np.zeros(n, dtype=[("origin", "<f4", 3), ("t_min", "<f4"), ("direction", "<f4", 3), ("t_max", "<f4")])
rays["origin"] = rng.uniform(-0.95, 0.95, size=(n, 3))
d = rng.normal(size=(n, 3))
rays["direction"] = d / np.linalg.norm(d, axis=1, keepdims=True)
rays["t_max"] = np.where(rng.uniform(size=n) < 0.5, np.float32(3.0e38), rng.uniform(0.1, 2.0, size=n))
orc = oracle.Oracle(sc)
with CudaTracer(0) as t:
    t.initializeBuffers(sc)
    for any_hit in (False, True):
        hits = t.cast(rays, any_hit=any_hit, order=N.RC_ORDER_REFERENCE)
        prim, tt, u, v, _ = orc.cast32(rays, any_hit=any_hit, order=N.RC_ORDER_REFERENCE)
        assert np.array_equal(hits["prim"], prim) and np.array_equal(hits["t"], tt), any_hit
        assert np.array_equal(hits["u"], u) and np.array_equal(hits["v"], v), any_hit
print("stackless ok")
"""


def test_stackless_reference_order_matches_oracle():
    tests = Path(__file__).resolve().parent
    root = str(tests.parent)
    env = dict(os.environ, RC_STACKLESS="1")
    out = subprocess.run([sys.executable, "-c", _CHECKS.format(root=root, tests=str(tests))], env=env,
                         capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stdout[-2000:] + out.stderr[-4000:]
    assert "stackless ok" in out.stdout
