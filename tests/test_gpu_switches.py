"""The tuning switches (environment variables, read once per process) change
how the work runs, never its results: for each one a child process renders
the same PATH films, RAY frame records, caller-ray records and tone-mapped
image as the default process, bit for bit."""

from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TESTS = Path(__file__).resolve().parent

_OUTPUTS = """
import numpy as np
import oracle
from raycer_gb300 import scenes
from raycer_gb300.tracer import RAY_DTYPE, CudaTracer, TracerState, camera_record
from helpers import camera_floats, small_heightfield, small_room


def outputs():
    out = {}
    room = small_room(width=64, height=48)
    room.settings.update(multi_sample_count_sqrt=2, path_sample_count=1, max_path_length=6)
    hf = scenes.heightfield_path_scene(width=160, height=90, nx=96, nz=48)
    for name, sc in (("room", room), ("hf", hf)):
        n = sc.width * sc.height
        with CudaTracer(0) as t:
            t.initializeBuffers(sc, seed=6)
            t.initializeImageBuffers(sc.width, sc.height)
            t.run(TracerState(scene=sc, filmWidth=sc.width, filmHeight=sc.height, pixelCount=n))
            out[name + "_film"] = t.read_film().copy()
            out[name + "_image"] = t.downloadImage().copy()
    sc = small_heightfield(width=160, height=90)
    sc.settings["tracer"] = "ray"
    sc.light_direction = (-1.0, -0.25, -0.2)
    n = sc.width * sc.height
    with CudaTracer(0) as t:
        t.initializeBuffers(sc)
        t.initializeImageBuffers(sc.width, sc.height)
        t.run(TracerState(scene=sc, filmWidth=sc.width, filmHeight=sc.height, pixelCount=n))
        out["ray_frame"] = t.read_cast().view(np.int32).reshape(-1, 4).copy()
        rays = oracle.camera_rays32(camera_floats(camera_record(sc)), sc.width, n)
        out["caller_rays"] = t.cast_with_shadow(np.ascontiguousarray(rays).view(RAY_DTYPE).reshape(-1)).view(
            np.int32).reshape(-1, 4).copy()
    return out
"""

_CHILD = """
import sys
sys.path.insert(0, {root!r})
sys.path.insert(0, {tests!r})
import numpy as np
exec(compile({outputs!r}, "outputs", "exec"))
np.savez({path!r}, **outputs())
print("written")
"""

SWITCHES = {
    "extend_refill": {"RC_EXTEND_REFILL": "1"},
    "binary_tree": {"RC_WIDE_BVH": "0"},
    "two_kernel_segments": {"RC_EXTEND_SHADE": "0"},
    "no_packets": {"RC_TRACE_PACKETS": "0"},
    "camera_packets_only": {"RC_TRACE_PACKETS": "1"},
    "two_kernel_frame": {"RC_TRACE_FUSED": "0"},
    "copies": {"RC_CAST_COPY": "1", "RC_RESOLVE_COPY": "1"},
}


@pytest.fixture(scope="module")
def default_outputs():
    ns: dict = {}
    sys.path.insert(0, str(TESTS))
    exec(compile(_OUTPUTS, "outputs", "exec"), ns)
    return ns["outputs"]()


@pytest.mark.parametrize("switch", sorted(SWITCHES))
def test_switch_keeps_results(switch, default_outputs, tmp_path):
    path = str(tmp_path / "out.npz")
    env = dict(os.environ, **SWITCHES[switch])
    code = _CHILD.format(root=str(TESTS.parent), tests=str(TESTS), outputs=_OUTPUTS, path=path)
    res = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stdout[-2000:] + res.stderr[-4000:]
    got = np.load(path)
    for key, ref in default_outputs.items():
        assert np.array_equal(got[key], ref, equal_nan=True), f"{switch}: {key} differs"
    assert default_outputs["ray_frame"][:, 2].max() >= 0  # occluded pixels present
