"""Full-size parity on the GPU.

* 1920x1080 ray casting on the 1,045,506-triangle heightfield: every pixel's
  primary and shadow result equals the float32 oracle bit for bit (both
  traversal orders); at the reference's strided pixels the primary ids equal
  the reference's float64 ids except documented edge ties, t within 1e-5
  relative, and shadow occlusion within the grazing-ray budget.
* 320x240, 16 spp, depth 4 path tracing of the room: the film equals the
  float32 oracle bit for bit, and the image matches the reference's renders
  statistically.
* Traversal counters equal the oracle's (they feed the roofline's byte count).
"""

from __future__ import annotations

import numpy as np
import pytest

import oracle
from raycer_gb300 import _native as N
from raycer_gb300 import scenes
from raycer_gb300.tracer import CudaTracer, TracerState, camera_record

from helpers import camera_floats
from test_golden_pins import _load, check_statistics, classify_edge_ties

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def heightfield():
    sc = scenes.heightfield_scene()
    t = CudaTracer(0)
    t.initializeBuffers(sc)
    t.initializeImageBuffers(sc.width, sc.height)
    nodes, order = t.get_bvh()
    orc = oracle.Oracle(sc, prebuilt=(nodes, order))
    yield sc, t, orc
    t.close()


@pytest.mark.parametrize("order", [N.RC_ORDER_NEAREST, N.RC_ORDER_REFERENCE])
def test_heightfield_frame_bit_exact_and_counters(heightfield, order):
    sc, t, orc = heightfield
    t.set_traversal_order(order)
    t.set_counting(True)
    st = TracerState(scene=sc, filmWidth=sc.width, filmHeight=sc.height, pixelCount=sc.width * sc.height)
    t.run(st)
    stats = t.stats()
    t.set_counting(False)
    gpu = t.read_cast().view(np.int32).reshape(-1, 4)
    cam = camera_floats(camera_record(sc))
    L = -np.array(sc.light_direction, np.float32)
    ref, cnt = orc.raycast32(cam, sc.width, sc.width * sc.height, L, order=order)
    diff = (gpu != ref).any(axis=1)
    assert not diff.any(), f"{diff.sum()} pixels differ"
    assert stats["rays_traced"] == cnt[0]
    assert stats["node_visits"] == cnt[1]
    assert stats["tri_tests"] == cnt[2]


@pytest.mark.parametrize("light", ["config", "low"])
@pytest.mark.parametrize("order", [N.RC_ORDER_NEAREST, N.RC_ORDER_REFERENCE])
def test_heightfield_timed_frame_bit_exact(heightfield, order, light):
    """The frame the benchmark times: uncounted, so one kernel traces each
    8x4 tile's primary rays warp-wide and then every hit pixel's shadow ray
    (k_raycast_primary, packet + fused form). Every pixel's 16-byte record of
    the 1920x1080 frame equals the float32 oracle's, in both traversal
    orders, under the scene's light and under a low light whose shadow rays
    meet the hills (reference: intersectBVH intersections.cl:98-148,
    FlatBVH::intersect FlatBVH.cpp:22-75)."""
    import dataclasses

    sc, t, orc = heightfield
    lit = sc if light == "config" else dataclasses.replace(sc, light_direction=(-1.0, -0.25, -0.2))
    t._set_lights(lit)
    try:
        t.set_traversal_order(order)
        t.set_counting(False)
        st = TracerState(scene=sc, filmWidth=sc.width, filmHeight=sc.height, pixelCount=sc.width * sc.height)
        t.run(st)
        stats = t.stats()
        gpu = t.read_cast().view(np.int32).reshape(-1, 4)
    finally:
        t._set_lights(sc)
    # one kernel: the shadow stage has no launch of its own
    assert stats["stage_ms"][1] == 0.0 and stats["stage_ms"][0] > 0.0
    cam = camera_floats(camera_record(sc))
    L = -np.array(lit.light_direction, np.float32)
    ref, cnt = orc.raycast32(cam, sc.width, sc.width * sc.height, L, order=order)
    diff = (gpu != ref).any(axis=1)
    assert not diff.any(), f"{diff.sum()} pixels differ"
    assert stats["rays_traced"] == cnt[0]
    occluded = int((ref[:, 2] >= 0).sum())
    if light == "low":
        assert occluded > 100_000, occluded


def test_heightfield_vs_reference_fp64(heightfield):
    sc, t, orc = heightfield
    g = _load("heightfield.npz")
    t.set_traversal_order(N.RC_ORDER_NEAREST)
    st = TracerState(scene=sc, filmWidth=sc.width, filmHeight=sc.height, pixelCount=sc.width * sc.height)
    t.run(st)
    cast = t.read_cast()[g["hit_pixels"]]
    rays = oracle.camera_rays32(camera_floats(camera_record(sc)), sc.width, sc.width * sc.height)[g["hit_pixels"]]
    # barycentrics of the device's hits (same float32 arithmetic as the oracle)
    _, _, u, v, _ = orc.cast32(rays, order=1)
    bad = classify_edge_ties(orc, rays, cast["prim"], cast["t"], u, v, g["hit_prim"], g["hit_t"])
    assert not bad, f"{len(bad)} id mismatches are not edge ties"
    same = (cast["prim"] == g["hit_prim"]) & (cast["prim"] >= 0)
    rel = np.abs(cast["t"][same].astype(np.float64) - g["hit_t"][same]) / g["hit_t"][same]
    assert rel.max() <= 1e-5
    occ = (cast["flags"] & 4) != 0
    both = (cast["prim"] >= 0) & (g["hit_prim"] >= 0)
    flips = int(((occ != g["occluded"]) & both).sum())
    assert flips <= max(3, int(1e-3 * both.sum())), flips


def test_room_full_film_bit_exact_and_statistics():
    sc = scenes.room_scene()
    g = _load("room.npz")
    with CudaTracer(0) as t:
        t.initializeBuffers(sc, seed=3)
        t.initializeImageBuffers(sc.width, sc.height)
        st = TracerState(scene=sc, filmWidth=sc.width, filmHeight=sc.height, pixelCount=sc.width * sc.height)
        t.run(st)
        film = t.read_film()
        lin = t.read_linear()
    cam = camera_floats(camera_record(sc))
    orc = oracle.Oracle(sc)
    ref, _ = orc.render_path32(cam, sc.width, sc.width * sc.height, 4, 1, 4, (0.5, 0.5), 1e-5, 4, 0, 1, 3, 0)
    assert np.array_equal(film, ref)
    assert np.array_equal(lin[:, :3], (ref[:, :3] / ref[:, 3:4]).astype(np.float32))
    check_statistics(lin[:, :3].astype(np.float64), g)
