"""Host-side semantics of the C ABI on the GPU: call order errors, the
TracerState pixel-range contract, progressive accumulation, cancellation,
prebuilt BVH uploads, device-pointer casts."""

from __future__ import annotations

import ctypes as C
import threading

import numpy as np
import pytest

import oracle
from raycer_gb300 import _native as N
from raycer_gb300 import scenes
from raycer_gb300.tracer import CudaTracer, RaycerError, TracerState, camera_record, Film, Tracer, TracerType

from helpers import camera_floats, small_room

pytestmark = pytest.mark.gpu


def test_call_order_errors():
    with CudaTracer(0) as t:
        st = TracerState(scene=small_room(), filmWidth=64, filmHeight=48, pixelCount=64 * 48)
        with pytest.raises(RaycerError) as e:
            t.run(st)
        assert e.value.status == N.RC_NOT_READY
        assert N.lib().rc_render(t.handle, 0, 10, None, None) == N.RC_NOT_READY
        assert N.lib().rc_clear(t.handle) == N.RC_NOT_READY


def test_invalid_prebuilt_bvh_is_rejected():
    sc = small_room()
    with CudaTracer(0) as t:
        t.initializeBuffers(sc)
        nodes, order = t.get_bvh()
        bad = nodes.copy()
        bad["right_offset"][0] = nodes.shape[0] + 5
        with pytest.raises(RaycerError) as e:
            t.initializeBuffers(sc, prebuilt=(bad, order))
        assert e.value.status == N.RC_INVALID_ARG
        dup = order.copy()
        dup[1] = dup[0]
        with pytest.raises(RaycerError):
            t.initializeBuffers(sc, prebuilt=(nodes, dup))


def test_prebuilt_upload_renders_identically():
    sc = small_room()
    with CudaTracer(0) as a, CudaTracer(0) as b:
        a.initializeBuffers(sc, seed=5)
        nodes, order = a.get_bvh()
        b.initializeBuffers(sc, seed=5, prebuilt=(nodes, order))
        for t in (a, b):
            t.initializeImageBuffers(sc.width, sc.height)
            t.run(TracerState(scene=sc, filmWidth=sc.width, filmHeight=sc.height, pixelCount=sc.width * sc.height))
        assert np.array_equal(a.read_film(), b.read_film())


def test_pixel_range_contract():
    """rc_render(start, count) renders pixels start..start+count-1 of the image
    into film pixels 0..count-1 (Tracer.cpp:77-90 indexes the film by the
    range-relative pixel index)."""
    sc = small_room()
    W, H = sc.width, sc.height
    with CudaTracer(0) as t:
        t.initializeBuffers(sc, seed=9)
        t.initializeImageBuffers(W, H)
        full = TracerState(scene=sc, filmWidth=W, filmHeight=H, pixelCount=W * H)
        t.run(full)
        whole = t.read_film().copy()
        t.clear()
        start, count = 700, 1000
        part = TracerState(scene=sc, filmWidth=W, filmHeight=H, pixelStartOffset=start, pixelCount=count)
        t.run(part)
        assert part.pixelsProcessed == count
        f = t.read_film()
        assert np.array_equal(f[:count], whole[start:start + count])
        assert np.all(f[count:] == 0)


def test_progressive_accumulation_and_clear():
    sc = small_room(width=48, height=36)
    cam = camera_floats(camera_record(sc))
    orc = oracle.Oracle(sc)
    with CudaTracer(0) as t:
        t.initializeBuffers(sc, seed=21)
        t.initializeImageBuffers(sc.width, sc.height)
        st = TracerState(scene=sc, filmWidth=sc.width, filmHeight=sc.height, pixelCount=sc.width * sc.height)
        t.run(st)
        t.run(st)
        two = t.read_film()
        ref, _ = orc.render_path32(cam, sc.width, sc.width * sc.height, 4, 1, 4, (0.5, 0.5), 1e-5, 4, 0, 1, 21, 0)
        ref, _ = orc.render_path32(cam, sc.width, sc.width * sc.height, 4, 1, 4, (0.5, 0.5), 1e-5, 4, 0, 1, 21, 1,
                                   film=ref)
        assert np.array_equal(two, ref)
        t.clear()
        assert np.all(t.read_film() == 0)
        t.run(st)
        one, _ = orc.render_path32(cam, sc.width, sc.width * sc.height, 4, 1, 4, (0.5, 0.5), 1e-5, 4, 0, 1, 21, 0)
        assert np.array_equal(t.read_film(), one)


def test_cancel_flag_before_render():
    sc = small_room()
    with CudaTracer(0) as t:
        t.initializeBuffers(sc)
        t.initializeImageBuffers(sc.width, sc.height)
        ev = threading.Event()
        ev.set()
        with pytest.raises(RaycerError) as e:
            t.run(TracerState(scene=sc, filmWidth=sc.width, filmHeight=sc.height, pixelCount=sc.width * sc.height),
                  ev)
        assert e.value.status == N.RC_CANCELLED


def test_cast_device_pointers_with_torch():
    torch = pytest.importorskip("torch")
    sc = small_room(clutter=500)
    rng = np.random.default_rng(2)
    n = 10000
    rays = np.zeros((n, 8), np.float32)
    rays[:, 0:3] = rng.uniform(-0.9, 0.9, size=(n, 3))
    d = rng.normal(size=(n, 3))
    rays[:, 4:7] = d / np.linalg.norm(d, axis=1, keepdims=True)
    rays[:, 7] = 3.0e38
    with CudaTracer(0) as t:
        t.initializeBuffers(sc)
        dr = torch.from_numpy(rays).cuda()
        dh = torch.empty((n, 4), dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        st = N.lib().rc_cast_device(t.handle, C.c_void_p(dr.data_ptr()), n, 0, 1, C.c_void_p(dh.data_ptr()))
        assert st == N.RC_OK
        hits = t.cast(rays.view(np.dtype([("origin", "<f4", 3), ("t_min", "<f4"), ("direction", "<f4", 3),
                                          ("t_max", "<f4")])).reshape(-1))
        assert np.array_equal(dh.cpu().numpy()[:, 0], hits["prim"])
        bad = N.lib().rc_cast_device(t.handle, C.c_void_p(dr.data_ptr() + 4), n - 1, 0, 1, C.c_void_p(dh.data_ptr()))
        assert bad == N.RC_INVALID_ARG


def test_tracer_adapter_accumulates_into_film():
    """Tracer.getTracer(PATH).run adds weighted samples to state.film, and the
    film's tone-mapped image comes from the device Reinhard resolve."""
    sc = small_room(width=48, height=36)
    film = Film(sc.width, sc.height)
    st = TracerState(scene=sc, film=film, filmWidth=sc.width, filmHeight=sc.height, pixelCount=sc.width * sc.height)
    tr = Tracer.getTracer(TracerType.PATH)
    tr.run(st)
    tr.run(st)
    assert st.pixelsProcessed == sc.width * sc.height
    assert np.allclose(film.pixels[:, 3], 2 * 16)
    img = film.generateToneMappedImage(sc, tr.cuda)
    assert img.shape == (sc.width * sc.height, 4) and np.all(img[:, 3] == 1.0)
    assert 0.0 <= img[:, :3].min() and img[:, :3].max() <= 1.0
