"""Uncounted nearest-first PATH passes over the 4-wide BVH of a single-level
scene run extend and shade as one kernel per segment (k_extend_shade, plain
and radiance-cache passes); RC_EXTEND_SHADE=0 keeps the two kernels. Both give
the same films bit for bit, and the float32 oracle's where it models the
frame: Russian roulette, the sky extension, dielectric materials and cache
lookups included (a two-level frame rides along: it takes the two kernels
in both processes). The switch is read once per process, so the two-kernel
films are rendered in a child process."""

from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

import oracle
from raycer_gb300 import scenes
from raycer_gb300.tracer import CudaTracer, TracerState, camera_record

from helpers import camera_floats, small_room

pytestmark = pytest.mark.gpu

TESTS = Path(__file__).resolve().parent

# The frames both processes render: (name, kind, scene, seed). "flat":
# a single-level scene; "instanced": the two-level form of a scene; "cache":
# the first frame of a fresh radiance cache (its lookups use the initial
# weights, so the film does not depend on the order of training samples).
_FRAMES = """
import numpy as np
from raycer_gb300 import scenes
from raycer_gb300.nrc import RadianceCache
from raycer_gb300.tracer import CudaTracer, TracerState
from helpers import small_room


def frames():
    room = small_room(width=48, height=36)
    room.settings.update(multi_sample_count_sqrt=2, path_sample_count=1, max_path_length=8,
                         russian_roulette_depth=3)
    sky = scenes.heightfield_blobs_scene(instances=6, blob_level=2, hf_nx=64, hf_nz=32, width=64, height=36)
    sky.settings.update(max_path_length=6)
    two_level = scenes.heightfield_blobs_instanced(instances=6, blob_level=2, hf_nx=64, hf_nz=32, width=64,
                                                   height=36, dielectric_fraction=0.5)
    two_level.settings.update(max_path_length=8)
    glass = two_level.flatten()
    box = scenes.heightfield_blobs_scene(instances=6, blob_level=2, hf_nx=64, hf_nz=32, width=96, height=54,
                                         enclosed=True)
    return [("room_rr", "flat", room, 3), ("sky", "flat", sky, 4), ("glass", "flat", glass, 5),
            ("glass_two_level", "instanced", two_level, 6), ("cache_box", "cache", box, 7)]


def render(kind, sc, seed):
    with CudaTracer(0) as t:
        if kind == "instanced":
            t.initializeInstanced(sc, seed=seed)
        else:
            t.initializeBuffers(sc, seed=seed)
        t.initializeImageBuffers(sc.width, sc.height)
        cache = RadianceCache(t) if kind == "cache" else None
        t.run(TracerState(scene=sc, filmWidth=sc.width, filmHeight=sc.height, pixelCount=sc.width * sc.height))
        if cache is not None:
            assert cache.stats()["lookups"] > 0
        return t.read_film().copy()
"""

_CHILD = """
import sys
sys.path.insert(0, {root!r})
sys.path.insert(0, {tests!r})
import numpy as np
exec(compile({frames!r}, "frames", "exec"))
out = {{name: render(kind, sc, seed) for name, kind, sc, seed in frames()}}
np.savez({path!r}, **out)
print("two-kernel films written")
"""


def _frames_module():
    ns: dict = {}
    sys.path.insert(0, str(TESTS))
    exec(compile(_FRAMES, "frames", "exec"), ns)
    return ns


def test_one_kernel_and_two_kernel_films_are_identical(tmp_path):
    path = str(tmp_path / "two_kernel.npz")
    env = dict(os.environ, RC_EXTEND_SHADE="0")
    code = _CHILD.format(root=str(TESTS.parent), tests=str(TESTS), frames=_FRAMES, path=path)
    res = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stdout[-2000:] + res.stderr[-4000:]
    two = np.load(path)
    ns = _frames_module()
    for name, kind, sc, seed in ns["frames"]():
        one = ns["render"](kind, sc, seed)
        assert np.array_equal(one, two[name]), f"{name}: {(one != two[name]).any(axis=1).sum()} pixels differ"
        assert one[:, :3].max() > 0.0, name


def test_roulette_film_matches_oracle():
    """Russian roulette from segment 3 (depth 8) through the one-kernel
    segments equals the float32 oracle's film bit for bit."""
    sc = small_room(width=48, height=36)
    sc.settings.update(multi_sample_count_sqrt=2, path_sample_count=1, max_path_length=8, russian_roulette_depth=3,
                       sampler="cmj")
    n = sc.width * sc.height
    with CudaTracer(0) as t:
        t.initializeBuffers(sc, seed=9)
        t.initializeImageBuffers(sc.width, sc.height)
        t.run(TracerState(scene=sc, filmWidth=sc.width, filmHeight=sc.height, pixelCount=n))
        film = t.read_film()
        cam = camera_floats(camera_record(sc))
    ref, _ = oracle.Oracle(sc).render_path32(cam, sc.width, n, 2, 1, 4, (0.5, 0.5), 1e-5, 8, 3, 1, 9, 0)
    assert np.array_equal(film, ref), f"{(film != ref).any(axis=1).sum()} pixels differ"
