"""GPU ray queries vs the float32 oracle (bit-exact) — closest and any hit,
both traversal orders, the RAY frame (primary + shadow) and the generic cast."""

from __future__ import annotations

import numpy as np
import pytest

import oracle
from raycer_gb300 import _native as N
from raycer_gb300 import scenes
from raycer_gb300.tracer import CudaTracer, TracerState, camera_record

from helpers import camera_floats, small_heightfield, small_room

pytestmark = pytest.mark.gpu


def _frame(sc, order):
    with CudaTracer(0) as t:
        t.initializeBuffers(sc)
        t.set_traversal_order(order)
        t.initializeImageBuffers(sc.width, sc.height)
        st = TracerState(scene=sc, filmWidth=sc.width, filmHeight=sc.height, pixelCount=sc.width * sc.height)
        t.run(st)
        assert st.pixelsProcessed == sc.width * sc.height
        return t.read_cast().view(np.int32).reshape(-1, 4), camera_floats(camera_record(sc))


@pytest.mark.parametrize("order", [N.RC_ORDER_REFERENCE, N.RC_ORDER_NEAREST])
@pytest.mark.parametrize("which", ["room", "heightfield", "heightfield_low_light"])
def test_raycast_frame_bit_exact(which, order):
    sc = small_room() if which == "room" else small_heightfield()
    sc.settings["tracer"] = "ray"
    if which == "room":
        sc.light_direction = (-0.3, -1.0, -0.2)
    elif which == "heightfield_low_light":
        sc.light_direction = (-1.0, -0.25, -0.2)  # the hills shadow the valleys
    gpu, cam = _frame(sc, order)
    orc = oracle.Oracle(sc)
    L = -np.array(sc.light_direction, np.float32)
    ref, _ = orc.raycast32(cam, sc.width, sc.width * sc.height, L, order=order)
    assert np.array_equal(gpu, ref), f"{(gpu != ref).any(axis=1).sum()} pixels differ"
    if which != "heightfield":
        assert (ref[:, 2] >= 0).any(), "no occluded pixel"


@pytest.mark.parametrize("any_hit", [False, True])
@pytest.mark.parametrize("order", [N.RC_ORDER_REFERENCE, N.RC_ORDER_NEAREST])
def test_cast_random_rays_bit_exact(any_hit, order):
    sc = small_room(clutter=1000)
    rng = np.random.default_rng(5)
    n = 200_000
    rays = np.zeros(n, dtype=[("origin", "<f4", 3), ("t_min", "<f4"), ("direction", "<f4", 3), ("t_max", "<f4")])
    rays["origin"] = rng.uniform(-0.95, 0.95, size=(n, 3))
    d = rng.normal(size=(n, 3))
    rays["direction"] = d / np.linalg.norm(d, axis=1, keepdims=True)
    rays["t_min"] = 0.0
    rays["t_max"] = np.where(rng.uniform(size=n) < 0.5, np.float32(3.0e38), rng.uniform(0.1, 2.0, size=n))
    with CudaTracer(0) as t:
        t.initializeBuffers(sc)
        hits = t.cast(rays, any_hit=any_hit, order=order)
    orc = oracle.Oracle(sc)
    prim, tt, u, v, _ = orc.cast32(rays, any_hit=any_hit, order=order)
    assert np.array_equal(hits["prim"], prim)
    assert np.array_equal(hits["t"], tt)
    assert np.array_equal(hits["u"], u)
    assert np.array_equal(hits["v"], v)


@pytest.mark.parametrize("copy", [False, True])
def test_cast_with_shadow_host_buffers_equal_frame(copy, monkeypatch):
    """2,073,600 caller rays from host buffers: traced in place where the
    device reaches host memory, else (and with RC_CAST_COPY=1) through the
    chunked copy path (4 chunks on three streams); the results equal the RAY
    frame's either way."""
    from raycer_gb300.tracer import RAY_DTYPE, TracerState

    if copy:
        monkeypatch.setenv("RC_CAST_COPY", "1")
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


def _edge_rays():
    """Rays at the slab and triangle tests' edge cases: axis-aligned
    directions (two zero components: infinite inverse components of both
    signs, including -0.0), one zero component, origins on the room's wall
    planes and inside the walls, rays lying in a wall's plane (det = 0),
    directions aimed at triangle vertices, empty and reversed t windows,
    and NaN components."""
    rng = np.random.default_rng(11)
    rays = []
    axes = np.eye(3, dtype=np.float32)
    for s in (1.0, -1.0):
        for a in range(3):
            d = s * axes[a]
            for _ in range(400):
                o = rng.uniform(-0.9, 0.9, 3).astype(np.float32)
                rays.append((o, d, 0.0, 3.0e38))
            dz = d.copy()
            dz[dz == 0] = -0.0  # zero components of the other sign
            for _ in range(100):
                rays.append((rng.uniform(-0.9, 0.9, 3).astype(np.float32), dz, 0.0, 3.0e38))
    for _ in range(600):  # one zero component
        d = rng.normal(size=3).astype(np.float32)
        d[rng.integers(0, 3)] = 0.0
        rays.append((rng.uniform(-0.9, 0.9, 3).astype(np.float32), d / np.linalg.norm(d), 0.0, 3.0e38))
    for _ in range(600):  # origins on the wall planes x, y, z = -1 / +1
        o = rng.uniform(-0.9, 0.9, 3).astype(np.float32)
        o[rng.integers(0, 3)] = np.float32(rng.choice([-1.0, 1.0]))
        d = rng.normal(size=3).astype(np.float32)
        rays.append((o, d / np.linalg.norm(d), 0.0, 3.0e38))
    for _ in range(300):  # in the plane of the floor (y = -1) and of the back wall (z = -1)
        o = np.array([rng.uniform(-0.9, 0.9), -1.0, rng.uniform(-0.9, 0.9)], np.float32)
        d = np.array([rng.normal(), 0.0, rng.normal()], np.float32)
        rays.append((o, d / np.linalg.norm(d), 0.0, 3.0e38))
        o = np.array([rng.uniform(-0.9, 0.9), rng.uniform(-0.9, 0.9), -1.0], np.float32)
        d = np.array([rng.normal(), rng.normal(), 0.0], np.float32)
        rays.append((o, d / np.linalg.norm(d), 0.0, 3.0e38))
    corners = np.array([[-1, -1, -1], [1, -1, -1], [-1, 1, -1], [1, 1, -1], [-1, -1, 1], [1, -1, 1]], np.float32)
    for c in corners:  # at wall corners (triangle vertices)
        for _ in range(50):
            o = rng.uniform(-0.5, 0.5, 3).astype(np.float32)
            d = c - o
            rays.append((o, d / np.linalg.norm(d), 0.0, 3.0e38))
    for _ in range(200):  # empty / reversed windows
        d = rng.normal(size=3).astype(np.float32)
        t0 = np.float32(rng.uniform(0.0, 2.0))
        rays.append((rng.uniform(-0.9, 0.9, 3).astype(np.float32), d / np.linalg.norm(d), t0, t0 * np.float32(0.5)))
    nan = np.float32(np.nan)
    for o, d in (((nan, 0, 0), (0, 0, -1)), ((0, 0, 0), (nan, 0, -1)), ((0, 0, 0), (nan, nan, nan))):
        rays.append((np.array(o, np.float32), np.array(d, np.float32), 0.0, 3.0e38))
    out = np.zeros(len(rays), dtype=[("origin", "<f4", 3), ("t_min", "<f4"), ("direction", "<f4", 3),
                                     ("t_max", "<f4")])
    for i, (o, d, t0, t1) in enumerate(rays):
        out[i] = (o, t0, d, t1)
    return out


@pytest.mark.parametrize("any_hit", [False, True])
@pytest.mark.parametrize("order", [N.RC_ORDER_REFERENCE, N.RC_ORDER_NEAREST])
def test_cast_edge_rays_bit_exact(any_hit, order):
    sc = small_room(clutter=500)
    rays = _edge_rays()
    with CudaTracer(0) as t:
        t.initializeBuffers(sc)
        hits = t.cast(rays, any_hit=any_hit, order=order)
    prim, tt, u, v, _ = oracle.Oracle(sc).cast32(rays, any_hit=any_hit, order=order)
    assert (prim >= 0).mean() > 0.5
    assert np.array_equal(hits["prim"], prim), int((hits["prim"] != prim).sum())
    same_t = (hits["t"] == tt) | (np.isnan(hits["t"]) & np.isnan(tt))
    assert same_t.all()
    for g, r in ((hits["u"], u), (hits["v"], v)):
        assert ((g == r) | (np.isnan(g) & np.isnan(r))).all()


@pytest.mark.parametrize("order", [N.RC_ORDER_REFERENCE, N.RC_ORDER_NEAREST])
@pytest.mark.parametrize("shape", [(157, 61, 0, None), (7, 5, 0, None), (300, 3, 0, None), (157, 61, 1000, 3001)])
def test_raycast_frame_odd_shapes(shape, order):
    """One-kernel RAY frames at shapes the 8x4 tiling does not divide: partial
    tiles along both edges (157x61), a frame narrower than a tile (7x5) and
    one shorter than a tile (300x3; the camera needs two rows at least), both
    walked pixel by pixel, and a pixel sub-range of a frame (start 1000, 3001
    pixels), bit-exact against the oracle."""
    width, height, start, count = shape
    count = width * height if count is None else count
    sc = small_heightfield(width=width, height=height)
    sc.settings["tracer"] = "ray"
    sc.light_direction = (-1.0, -0.25, -0.2)  # a low light: the hills shadow the valleys
    with CudaTracer(0) as t:
        t.initializeBuffers(sc)
        t.set_traversal_order(order)
        t.initializeImageBuffers(sc.width, sc.height)
        st = TracerState(scene=sc, filmWidth=sc.width, filmHeight=sc.height, pixelStartOffset=start, pixelCount=count)
        t.run(st)
        assert st.pixelsProcessed == count
        gpu = t.read_cast().view(np.int32).reshape(-1, 4)[:count]
    L = -np.array(sc.light_direction, np.float32)
    ref, _ = oracle.Oracle(sc).raycast32(camera_floats(camera_record(sc)), sc.width, count, L, order=order,
                                         pixel_start=start)
    assert np.array_equal(gpu, ref), f"{(gpu != ref).any(axis=1).sum()} of {count} pixels differ"
    assert (ref[:, 0] >= 0).any()
    if count > 1000:
        assert (ref[:, 2] >= 0).any()  # occluded pixels


def test_cast_with_shadow_ray_lists():
    """Caller ray lists that are not a whole image (a partial frame in pixel
    order, and the whole frame's rays shuffled) go through the one-kernel
    frame walked ray by ray; each ray's record equals the camera frame's
    record of its pixel."""
    from raycer_gb300.tracer import RAY_DTYPE

    sc = small_heightfield(width=160, height=90)
    sc.settings["tracer"] = "ray"
    sc.light_direction = (-1.0, -0.25, -0.2)  # a low light: the hills shadow the valleys
    n = sc.width * sc.height
    with CudaTracer(0) as t:
        t.initializeBuffers(sc)
        t.initializeImageBuffers(sc.width, sc.height)
        t.run(TracerState(scene=sc, filmWidth=sc.width, filmHeight=sc.height, pixelCount=n))
        frame = t.read_cast().copy()
        rays = np.ascontiguousarray(oracle.camera_rays32(camera_floats(camera_record(sc)), sc.width, n))
        rays = rays.view(RAY_DTYPE).reshape(-1)
        part = 5 * sc.width + 17
        out = t.cast_with_shadow(np.ascontiguousarray(rays[:part]))
        assert np.array_equal(out, frame[:part])
        perm = np.random.default_rng(4).permutation(n)
        out = t.cast_with_shadow(np.ascontiguousarray(rays[perm]))
        assert np.array_equal(out, frame[perm])
    assert (frame["prim"] >= 0).any() and (frame["occluder"] >= 0).any()


@pytest.mark.parametrize("light", [(sx * 0.4, sy * 1.0, sz * 0.3) for sx in (1, -1) for sy in (1, -1) for sz in (1, -1)]
                         + [(0.0, -1.0, 0.3), (-0.5, 0.0, -0.2)])
def test_raycast_frame_light_octants(light):
    """The one-kernel frame's shadow walk is compiled per sign octant of the
    light's direction (box tests with the near and far planes known); every
    octant, and lights with a zero component (the general walk), give the
    oracle's records bit for bit, in both orders."""
    sc = small_heightfield(width=160, height=90)
    sc.settings["tracer"] = "ray"
    sc.light_direction = light
    L = -np.array(sc.light_direction, np.float32)
    cam = camera_floats(camera_record(sc))
    with CudaTracer(0) as t:
        t.initializeBuffers(sc)
        t.initializeImageBuffers(sc.width, sc.height)
        orc = oracle.Oracle(sc, prebuilt=t.get_bvh())
        for order in (N.RC_ORDER_NEAREST, N.RC_ORDER_REFERENCE):
            t.set_traversal_order(order)
            t.run(TracerState(scene=sc, filmWidth=sc.width, filmHeight=sc.height, pixelCount=sc.width * sc.height))
            gpu = t.read_cast().view(np.int32).reshape(-1, 4)
            ref, _ = orc.raycast32(cam, sc.width, sc.width * sc.height, L, order=order)
            assert np.array_equal(gpu, ref), f"{(gpu != ref).any(axis=1).sum()} pixels differ"
