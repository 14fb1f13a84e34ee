"""GPU path tracer vs the float32 oracle (bit-exact film)."""

from __future__ import annotations

import numpy as np
import pytest

import oracle
from raycer_gb300.tracer import CudaTracer, TracerState, camera_record

from helpers import camera_floats, small_room

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("ms,P,depth,sampler", [(1, 1, 4, 4), (2, 1, 4, 4), (3, 2, 5, 4), (2, 1, 3, 1)])
def test_film_bit_exact(ms, P, depth, sampler):
    sc = small_room(width=48, height=36)
    sc.settings.update(multi_sample_count_sqrt=ms, path_sample_count=P, max_path_length=depth,
                       sampler={4: "cmj", 1: "random"}[sampler])
    with CudaTracer(0) as t:
        t.initializeBuffers(sc, seed=11)
        t.initializeImageBuffers(sc.width, sc.height)
        st = TracerState(scene=sc, filmWidth=sc.width, filmHeight=sc.height, pixelCount=sc.width * sc.height)
        t.run(st)
        film = t.read_film()
        cam = camera_floats(camera_record(sc))
    orc = oracle.Oracle(sc)
    ref, _ = orc.render_path32(cam, sc.width, sc.width * sc.height, ms, P, sampler, (0.5, 0.5), 1e-5, depth, 0, 1,
                               11, 0)
    assert np.array_equal(film, ref), f"{(film != ref).any(axis=1).sum()} pixels differ"


@pytest.mark.parametrize("filt,ftype", [("tent", 1), ("bell", 2), ("gaussian", 3), ("mitchell", 4), ("lanczos", 5)])
@pytest.mark.parametrize("ms,sampler", [(2, 4), (3, 1)])
def test_film_bit_exact_filters(filt, ftype, ms, sampler):
    sc = small_room(width=40, height=30)
    sc.settings.update(multi_sample_count_sqrt=ms, path_sample_count=1, max_path_length=4, filter=filt,
                       sampler={4: "cmj", 1: "random"}[sampler])
    with CudaTracer(0) as t:
        t.initializeBuffers(sc, seed=12)
        t.initializeImageBuffers(sc.width, sc.height)
        st = TracerState(scene=sc, filmWidth=sc.width, filmHeight=sc.height, pixelCount=sc.width * sc.height)
        t.run(st)
        film = t.read_film()
        cam = camera_floats(camera_record(sc))
    orc = oracle.Oracle(sc)
    ref, _ = orc.render_path32(cam, sc.width, sc.width * sc.height, ms, 1, sampler, (0.5, 0.5), 1e-5, 4, 0, 1,
                               12, 0, filter_type=ftype)
    assert np.array_equal(film, ref), f"{(film != ref).any(axis=1).sum()} pixels differ"
    if ftype in (4, 5):
        assert (film[:, 3] != film[0, 3]).any()  # weights vary with the sample offsets


@pytest.mark.parametrize("size", ["small", "1080p"])
def test_heightfield_path_frame_bit_exact(size):
    """The path-tracing workload on the 1,045,506-triangle heightfield (an
    emissive panel above it, one camera ray per pixel, depth 4): every film
    pixel equals the float32 oracle's, at 1080p the exact frame the bench
    times (Tracer::run Tracer.cpp:58, PathTracer::traceRecursive
    PathTracer.cpp:25-75)."""
    from raycer_gb300 import scenes

    if size == "small":
        sc = scenes.heightfield_path_scene(width=160, height=90, nx=96, nz=48)
    else:
        sc = scenes.heightfield_path_scene()
    n = sc.width * sc.height
    with CudaTracer(0) as t:
        t.initializeBuffers(sc, seed=1)
        t.initializeImageBuffers(sc.width, sc.height)
        st = TracerState(scene=sc, filmWidth=sc.width, filmHeight=sc.height, pixelCount=n)
        t.run(st)
        assert st.pixelsProcessed == n
        film = t.read_film()
        cam = camera_floats(camera_record(sc))
        nodes, order = t.get_bvh()
    orc = oracle.Oracle(sc, prebuilt=(nodes, order))
    ref, _ = orc.render_path32(cam, sc.width, n, 1, 1, 4, (0.5, 0.5), 1e-5, 4, 0, 1, 1, 0)
    assert np.array_equal(film, ref), f"{(film != ref).any(axis=1).sum()} pixels differ"
    assert (film[:, :3] > 0).any(axis=1).mean() > 0.3   # the panel lights most of the frame
