"""Progress, cancellation and the time budget of rc_render on the GPU, and the
bounded waits of the tensor-core lookup kernel.

The reference's Tracer::run advances pixelsProcessed while it renders and
stops when `interrupted` is raised from another thread (Tracer.cpp:76-112,
ConsoleRunner.cpp:126-142). Every failure here is made on the host: a flag a
second thread raises, a budget the kernels read, a wait limit of zero polls.
No kernel is made to fault or hang; each stop ends with the kernels draining
on their own and the handle still usable."""

from __future__ import annotations

import threading
import time

import numpy as np
import pytest

from raycer_gb300 import _native as N
from raycer_gb300 import scenes
from raycer_gb300.nrc import RadianceCache
from raycer_gb300.tracer import CudaTracer, Interrupted, RaycerError, TracerState

from helpers import nrc_init_params, nrc_queries

pytestmark = pytest.mark.gpu

# PATH passes hold 4,194,304 path slots: at 64 samples per pixel, 65,536 pixels.
PASS_PIXELS = (1 << 22) // 64


def _untouched(rec: np.ndarray) -> np.ndarray:
    """Records rc_clear zeroed that no kernel wrote (a written miss has
    prim -1; a written hit has t > 0)."""
    v = rec.view(np.int32).reshape(-1, 4)
    return (v == 0).all(axis=1)


@pytest.fixture(scope="module")
def heightfield():
    sc = scenes.heightfield_scene()
    sc.settings["tracer"] = "ray"
    t = CudaTracer(0)
    t.initializeBuffers(sc)
    t.initializeImageBuffers(sc.width, sc.height)
    st = TracerState(scene=sc, filmWidth=sc.width, filmHeight=sc.height, pixelCount=sc.width * sc.height)
    t.run(st)
    full = t.read_cast().copy()
    yield sc, t, full
    t.close()


@pytest.mark.parametrize("counting", [False, True])
@pytest.mark.parametrize("budget_ms", [0.0, 0.05])
def test_ray_frame_time_budget(heightfield, budget_ms, counting):
    """A RAY frame whose budget runs out returns RC_TIMEOUT; the pixels it
    reports finished are exactly the records it wrote, and each of those
    equals the full frame's record (one-kernel and counted two-kernel
    forms)."""
    sc, t, full = heightfield
    n = sc.width * sc.height
    t.set_counting(counting)
    t.clear()
    t.set_time_budget(budget_ms)
    st = TracerState(scene=sc, filmWidth=sc.width, filmHeight=sc.height, pixelCount=n)
    try:
        with pytest.raises(RaycerError) as e:
            t.run(st)
        assert e.value.status == N.RC_TIMEOUT
        rec = t.read_cast()
    finally:
        t.set_time_budget(None)
        t.set_counting(False)
    written = ~_untouched(rec)
    assert st.pixelsProcessed == int(written.sum())
    assert st.pixelsProcessed < n
    assert np.array_equal(rec[written], full[written])
    # the handle renders whole frames again
    t.run(st)
    assert st.pixelsProcessed == n
    assert np.array_equal(t.read_cast(), full)


@pytest.fixture(scope="module")
def long_path_render():
    """The room at 1920x1080 with 8x8 CMJ samples per pixel, depth 4: 32
    passes of 65,536 pixels, a few hundred milliseconds in all."""
    sc = scenes.room_scene(width=1920, height=1080)
    sc.settings["multi_sample_count_sqrt"] = 8
    t = CudaTracer(0)
    t.initializeBuffers(sc, seed=11)
    t.initializeImageBuffers(sc.width, sc.height)
    yield sc, t
    t.close()


def test_path_progress_advances_and_cancel_from_another_thread(long_path_render):
    sc, t = long_path_render
    n = sc.width * sc.height
    st = TracerState(scene=sc, filmWidth=sc.width, filmHeight=sc.height, pixelCount=n)
    flag = Interrupted()
    seen = []
    stop = threading.Event()

    def poll():
        # what ConsoleRunner's main thread does, every 0.2 ms instead of 100 ms
        while not stop.is_set():
            v = st.pixelsProcessed
            if not seen or v != seen[-1]:
                seen.append(v)
            if v >= 3 * PASS_PIXELS:
                flag.set()
            time.sleep(0.0002)

    t.clear()
    watcher = threading.Thread(target=poll)
    watcher.start()
    t0 = time.perf_counter()
    try:
        with pytest.raises(RaycerError) as e:
            t.run(st, flag)
    finally:
        stop.set()
        watcher.join()
    elapsed = time.perf_counter() - t0
    assert e.value.status == N.RC_CANCELLED
    done = st.pixelsProcessed
    # whole passes only, fewer than all of them
    assert 3 * PASS_PIXELS <= done < n and done % PASS_PIXELS == 0, done
    mid = [v for v in seen if 0 < v < n]
    assert len(mid) >= 2, seen
    assert all(b > a for a, b in zip(seen, seen[1:])), seen
    film = t.read_film()
    assert (film[:done, 3] > 0).all() and (film[done:, 3] == 0).all()

    # an uninterrupted render of the same frame takes longer and finishes
    flag.clear()
    t.clear()
    t1 = time.perf_counter()
    t.run(st, flag)
    assert st.pixelsProcessed == n
    assert time.perf_counter() - t1 > elapsed
    assert (t.read_film()[:, 3] > 0).all()


def test_threading_event_cancels_a_running_render(long_path_render):
    """A plain threading.Event works as the interrupted flag (checked by a
    watcher thread every millisecond)."""
    sc, t = long_path_render
    n = sc.width * sc.height
    st = TracerState(scene=sc, filmWidth=sc.width, filmHeight=sc.height, pixelCount=n)
    ev = threading.Event()
    timer = threading.Timer(0.03, ev.set)
    t.clear()
    timer.start()
    try:
        with pytest.raises(RaycerError) as e:
            t.run(st, ev)
    finally:
        timer.cancel()
    assert e.value.status == N.RC_CANCELLED
    assert st.pixelsProcessed < n and st.pixelsProcessed % PASS_PIXELS == 0


@pytest.mark.parametrize("budget_ms", [0.0, 40.0])
def test_path_time_budget(long_path_render, budget_ms):
    sc, t = long_path_render
    n = sc.width * sc.height
    st = TracerState(scene=sc, filmWidth=sc.width, filmHeight=sc.height, pixelCount=n)
    t.clear()
    t.set_time_budget(budget_ms)
    try:
        with pytest.raises(RaycerError) as e:
            t.run(st)
    finally:
        t.set_time_budget(None)
    assert e.value.status == N.RC_TIMEOUT
    done = st.pixelsProcessed
    assert done < n and done % PASS_PIXELS == 0
    if budget_ms == 0.0:
        assert done == 0
    film = t.read_film()
    assert (film[:done, 3] > 0).all() and (film[done:, 3] == 0).all()


def test_tensor_core_wait_gives_up_and_the_handle_recovers():
    """tc_wait_polls < 0: every bounded mbarrier wait of the tcgen05 lookup
    kernel gives up at once. The kernel sets its error bit, lets the MMAs it
    issued finish, frees its TMEM and returns; the call reports
    RC_DEVICE_ERROR. A cache configured with the default limit on the same
    handle then computes the lookups of the warp-level kernel."""
    w = nrc_init_params(seed=9)
    lo, hi = (-10.0, -2.0, -5.0), (10.0, 3.0, 5.0)
    q = nrc_queries(5000, seed=12, lo=lo, hi=hi)
    with CudaTracer(0) as t:
        c = RadianceCache(t, box_min=lo, box_max=hi, lookup_kernel=N.RC_NRC_TCGEN05, tc_wait_polls=-1)
        c.params = w
        with pytest.raises(RaycerError) as e:
            c.infer(q)
        assert e.value.status == N.RC_DEVICE_ERROR
        c2 = RadianceCache(t, box_min=lo, box_max=hi, lookup_kernel=N.RC_NRC_TCGEN05)
        c2.params = w
        got = c2.infer(q).astype(np.float64)
        ref_cache = RadianceCache(t, box_min=lo, box_max=hi, lookup_kernel=N.RC_NRC_MMA_SYNC)
        ref_cache.params = w
        ref = ref_cache.infer(q).astype(np.float64)
    rel = np.abs(got - ref) / np.abs(ref)
    assert np.quantile(rel, 0.99) < 1e-3 and rel.max() < 2e-2


def test_stopped_cache_render_leaves_the_cache_untouched():
    """A radiance-cache render whose budget runs out at once: the pass's later
    kernels (lookups, training targets, the optimizer) find the stop bit and
    do nothing, so the weights are those before the call, bit for bit, and
    the film is empty; the next render trains as usual."""
    sc = scenes.heightfield_blobs_scene(instances=12, blob_level=3, hf_nx=96, hf_nz=48, width=128, height=72,
                                        enclosed=True)
    n = sc.width * sc.height
    with CudaTracer(0) as t:
        t.initializeBuffers(sc, seed=2)
        t.initializeImageBuffers(sc.width, sc.height)
        st = TracerState(scene=sc, filmWidth=sc.width, filmHeight=sc.height, pixelCount=n)
        cache = RadianceCache(t, seed=5)
        for _ in range(3):
            t.run(st)
        before = cache.params.copy()
        t.clear()
        t.set_time_budget(0.0)
        try:
            with pytest.raises(RaycerError) as e:
                t.run(st)
        finally:
            t.set_time_budget(None)
        assert e.value.status == N.RC_TIMEOUT
        assert np.array_equal(cache.params, before)
        assert (t.read_film()[:, 3] == 0).all()
        t.run(st)
        assert not np.array_equal(cache.params, before)
        assert (t.read_film()[:, 3] > 0).all()
