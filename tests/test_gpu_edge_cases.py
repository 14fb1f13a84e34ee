"""Edge cases of the ray-query and render entry points on the GPU, against the
float32 oracle: empty batches, an empty scene, the smallest scenes (one
triangle, where the BVH root is a leaf; a root leaf of three triangles; five
triangles under one inner node), and ray counts that are not a multiple of
the 32-ray work unit."""

from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import oracle
from raycer_gb300 import _native as N
from raycer_gb300 import scenes
from raycer_gb300.tracer import RAY_DTYPE, CudaTracer, TracerState, camera_record

from helpers import camera_floats

pytestmark = pytest.mark.gpu

# Triangle 0 is an emissive panel (so a one-triangle scene still lights a
# PATH film); then a large grey triangle behind everything and three small
# grey ones in front of it, which shadow it under the light below.
_TRIS = [
    ([-0.4, 0.5, -0.6, 0.4, 0.5, -0.6, 0.0, 0.9, -0.7], 1),
    ([-2.0, -1.2, -1.5, 2.0, -1.2, -1.5, 0.0, 1.6, -1.6], 0),
    ([-0.9, -0.6, -0.3, -0.4, -0.6, -0.3, -0.6, -0.1, -0.4], 0),
    ([0.4, -0.6, -0.2, 0.9, -0.6, -0.2, 0.6, -0.1, -0.3], 0),
    ([0.0, -0.9, 0.0, 0.3, -0.9, 0.1, 0.1, -0.5, 0.0], 0),
]


def tiny_scene(k: int, width: int = 48, height: int = 32, tracer: str = "path") -> scenes.SceneDesc:
    v = np.array([t for t, _ in _TRIS[:k]], np.float64).astype(np.float32).astype(np.float64)
    mats = [scenes.Material(diffuse=(0.7, 0.7, 0.7)),
            scenes.Material(diffuse=(0.0, 0.0, 0.0), emittance=(4.0, 4.0, 4.0), is_emissive=True)]
    return scenes.SceneDesc(name=f"tiny({k})", vertices=v,
                            material_index=np.array([m for _, m in _TRIS[:k]], np.uint32), materials=mats,
                            camera=scenes.CameraDesc(position=(0.0, 0.0, 3.0), fov=60.0), width=width,
                            height=height, light_direction=(-0.3, -0.6, -1.0),
                            settings={"tracer": tracer, "max_path_length": 4})


def test_empty_batches_are_no_ops():
    """n = 0 returns RC_OK from every cast entry point without reading or
    writing a buffer (null pointers are accepted for an empty batch)."""
    sc = tiny_scene(3, tracer="ray")
    lib = N.lib()
    with CudaTracer(0) as t:
        t.initializeBuffers(sc)
        h = t.handle
        assert lib.rc_cast(h, None, 0, 0, N.RC_ORDER_NEAREST, None) == N.RC_OK
        assert lib.rc_cast_device(h, None, 0, 1, N.RC_ORDER_REFERENCE, None) == N.RC_OK
        assert lib.rc_cast_with_shadow(h, None, 0, N.RC_ORDER_NEAREST, None) == N.RC_OK
        assert lib.rc_cast_with_shadow_device_noalloc(h, None, 0, N.RC_ORDER_NEAREST, None) == N.RC_OK
        assert t.cast_with_shadow(np.zeros(0, RAY_DTYPE)).shape == (0,)
        assert t.cast(np.zeros(0, RAY_DTYPE)).shape == (0,)
        # a negative count is an error in every form
        assert lib.rc_cast(h, None, -1, 0, N.RC_ORDER_NEAREST, None) == N.RC_INVALID_ARG
        assert lib.rc_cast_with_shadow(h, None, -1, N.RC_ORDER_NEAREST, None) == N.RC_INVALID_ARG
        assert lib.rc_cast_with_shadow_device_noalloc(h, None, -1, N.RC_ORDER_NEAREST, None) == N.RC_INVALID_ARG
        # the handle still traces afterwards
        rays = np.zeros(1, RAY_DTYPE)
        rays["origin"] = (0.0, 0.0, 3.0)
        rays["direction"] = (0.0, 0.0, -1.0)
        rays["t_max"] = np.float32(3.0e38)
        assert t.cast(rays)["prim"][0] >= 0


def test_empty_scene_is_rejected():
    """A scene without triangles is an argument error (the reference's CL
    scene requires triangles, CLScene.cpp:196-201), and the handle keeps
    working for the next upload."""
    lib = N.lib()
    mats = (N.rc_material * 1)()
    with CudaTracer(0) as t:
        v = np.zeros(9, np.float64)
        idx = np.zeros(1, np.uint32)
        st = lib.rc_upload_scene(t.handle, v.ctypes.data_as(C.POINTER(C.c_double)),
                                 idx.ctypes.data_as(C.POINTER(C.c_uint32)), 0, mats, 1, 4)
        assert st == N.RC_INVALID_ARG
        assert b"empty" in lib.rc_last_error(t.handle)
        assert lib.rc_render(t.handle, 0, 1, None, None) == N.RC_NOT_READY
        t.initializeBuffers(tiny_scene(1))
        assert t.cast(np.zeros(1, RAY_DTYPE)).shape == (1,)


@pytest.mark.parametrize("k", [1, 3, 5])
@pytest.mark.parametrize("order", [N.RC_ORDER_REFERENCE, N.RC_ORDER_NEAREST])
def test_tiny_scene_raycast_frame(k, order):
    """RAY frames of 1, 3 and 5 triangles (a leaf root, a root leaf of
    three, one inner node) equal the oracle's records bit for bit."""
    sc = tiny_scene(k, tracer="ray")
    n = sc.width * sc.height
    with CudaTracer(0) as t:
        t.initializeBuffers(sc)
        t.set_traversal_order(order)
        t.initializeImageBuffers(sc.width, sc.height)
        st = TracerState(scene=sc, filmWidth=sc.width, filmHeight=sc.height, pixelCount=n)
        t.run(st)
        assert st.pixelsProcessed == n
        gpu = t.read_cast().view(np.int32).reshape(-1, 4)
        cam = camera_floats(camera_record(sc))
    ref, _ = oracle.Oracle(sc).raycast32(cam, sc.width, n, -np.array(sc.light_direction, np.float32), order=order)
    assert np.array_equal(gpu, ref), f"{(gpu != ref).any(axis=1).sum()} pixels differ"
    assert (ref[:, 0] >= 0).any() and (ref[:, 0] < 0).any()  # hits and misses
    if k == 5:
        assert (ref[:, 2] >= 0).any()  # the small triangles shadow the large one


@pytest.mark.parametrize("k", [1, 3, 5])
def test_tiny_scene_path_film(k):
    """PATH films of the same scenes equal the float32 oracle's bit for bit
    (4x4 CMJ samples per pixel, depth 4)."""
    sc = tiny_scene(k)
    sc.settings.update(multi_sample_count_sqrt=4, path_sample_count=1, sampler="cmj")
    n = sc.width * sc.height
    with CudaTracer(0) as t:
        t.initializeBuffers(sc, seed=5)
        t.initializeImageBuffers(sc.width, sc.height)
        t.run(TracerState(scene=sc, filmWidth=sc.width, filmHeight=sc.height, pixelCount=n))
        film = t.read_film()
        cam = camera_floats(camera_record(sc))
    ref, _ = oracle.Oracle(sc).render_path32(cam, sc.width, n, 4, 1, 4, (0.5, 0.5), 1e-5, 4, 0, 1, 5, 0)
    assert np.array_equal(film, ref), f"{(film != ref).any(axis=1).sum()} pixels differ"
    assert film[:, :3].max() > 0.0


@pytest.mark.parametrize("n", [1, 31, 33, 1000, 4097])
def test_ragged_ray_counts(n):
    """Ray counts around the 32-ray work unit and the 8x4 tile: rc_cast
    (closest and any hit) equals the oracle's cast and rc_cast_with_shadow
    equals the RAY frame's records of the same pixels."""
    sc = tiny_scene(5, width=80, height=60, tracer="ray")
    pixels = sc.width * sc.height
    cam = camera_floats(camera_record(sc))
    sel = np.random.default_rng(n).choice(pixels, size=n, replace=False)
    rays = np.ascontiguousarray(oracle.camera_rays32(cam, sc.width, pixels)[sel])
    with CudaTracer(0) as t:
        t.initializeBuffers(sc)
        t.initializeImageBuffers(sc.width, sc.height)
        t.run(TracerState(scene=sc, filmWidth=sc.width, filmHeight=sc.height, pixelCount=pixels))
        frame = t.read_cast().copy()
        out = t.cast_with_shadow(rays.view(RAY_DTYPE).reshape(-1))
        hits = {a: t.cast(rays.view(RAY_DTYPE).reshape(-1), any_hit=a) for a in (False, True)}
    assert np.array_equal(out, frame[sel])
    orc = oracle.Oracle(sc)
    for a, hit in hits.items():
        prim, tt, u, v, _ = orc.cast32(rays, any_hit=a, order=N.RC_ORDER_NEAREST)
        assert np.array_equal(hit["prim"], prim) and np.array_equal(hit["t"], tt)
        assert np.array_equal(hit["u"], u) and np.array_equal(hit["v"], v)
