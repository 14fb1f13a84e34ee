"""The CPU baseline / reference arm of bench.py runs the reference's
algorithm on its own: the float64 port builds its own BVH (its restatement
of FlatBVH::build) and camera, and no part of the product library is loaded
(the product must not be the thing the reference arm measures)."""

from __future__ import annotations

import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent

PROBE = r"""
import sys
sys.path.insert(0, {root!r})
import bench, oracle
from raycer_gb300 import _native, scenes
oracle.ref_available = lambda fast=False: False      # the port, as on a host without the reference's sources
sc = scenes.heightfield_scene(nx=64, nz=32, width=96, height=54)
res = bench.cpu_raycast(sc, 1, 0, None)
assert res["kind"] == "port" and res["rays_per_frame"] > sc.width * sc.height, res
assert _native._lib is None, "the product library was loaded"
maps = open("/proc/self/maps").read()
assert "libraycer_gb300" not in maps, "libraycer_gb300.so is mapped"
print("ok", res["rays_per_frame"])
"""


def test_cpu_arm_never_loads_the_product_library():
    res = subprocess.run([sys.executable, "-c", PROBE.format(root=str(ROOT))], capture_output=True, text=True,
                         timeout=300)
    assert res.returncode == 0 and res.stdout.startswith("ok"), res.stdout + res.stderr


BATCH_PROBE = r"""
import sys
sys.path.insert(0, {root!r})
import bench
from raycer_gb300 import _native, scenes
scs = scenes.batch_scenes(seed=3, count=4, n_max=2e3, resolutions=(64,), spps=(1, 4))
res = bench.batch_cpu_baseline(scs, stride=2, pixels_per_scene=256)
assert res["kind"] == "port" and res["value"] > 0 and res["rays"] >= 2 * 256, res
sizes = sorted(sc.triangle_count for sc in scs)
assert "%d, %d tris" % (sizes[1], sizes[3]) in res["sample"], res["sample"]
assert _native._lib is None, "the product library was loaded"
print("ok", res["value"])
"""


def test_batch_cpu_baseline_samples_the_batch_by_size_with_the_port():
    res = subprocess.run([sys.executable, "-c", BATCH_PROBE.format(root=str(ROOT))], capture_output=True, text=True,
                         timeout=300)
    assert res.returncode == 0 and res.stdout.startswith("ok"), res.stdout + res.stderr
