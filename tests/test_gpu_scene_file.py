"""Scene files on the GPU: a loaded scene renders exactly like the uploaded
one and reports the same BVH; a damaged file leaves the current scene alone."""

from __future__ import annotations

import numpy as np
import pytest

from raycer_gb300 import _native as N
from raycer_gb300.tracer import CudaTracer, RaycerError, TracerState, write_scene_file

from helpers import small_room

pytestmark = pytest.mark.gpu


def render(t, sc):
    t.initializeImageBuffers(sc.width, sc.height)
    t.clear()
    t.run(TracerState(scene=sc, filmWidth=sc.width, filmHeight=sc.height, pixelCount=sc.width * sc.height))
    return t.read_film()


def test_saved_and_written_files_render_identically(tmp_path):
    sc = small_room(width=48, height=36)
    sc.settings.update(multi_sample_count_sqrt=2, max_path_length=4)
    with CudaTracer(0) as a:
        a.initializeBuffers(sc, seed=5)
        film = render(a, sc)
        nodes, order = a.get_bvh()
        a.save_scene(tmp_path / "saved.rcgb")
    write_scene_file(sc, tmp_path / "written.rcgb")
    for name in ("saved.rcgb", "written.rcgb"):
        with CudaTracer(0) as b:
            b.load_scene(tmp_path / name, sc, seed=5)
            assert np.array_equal(render(b, sc), film), name
            n2, o2 = b.get_bvh()
            assert np.array_equal(n2, nodes) and np.array_equal(o2, order)


def test_cache_argument_and_damaged_file(tmp_path):
    sc = small_room(width=32, height=24)
    cache = tmp_path / "room.rcgb"
    with CudaTracer(0) as t:
        t.initializeBuffers(sc, seed=2, cache=cache)   # builds, uploads, writes
        assert cache.exists()
        first = render(t, sc)
    with CudaTracer(0) as t:
        t.initializeBuffers(sc, seed=2, cache=cache)   # loads
        assert np.array_equal(render(t, sc), first)
        raw = bytearray(cache.read_bytes())
        raw[200] ^= 1
        bad = tmp_path / "bad.rcgb"
        bad.write_bytes(bytes(raw))
        with pytest.raises(RaycerError) as e:
            t.load_scene(bad, sc)
        assert e.value.status == N.RC_IO and "checksum" in str(e.value)
        assert np.array_equal(render(t, sc), first)    # the loaded scene is still there


def test_instanced_scene_files(tmp_path):
    """Two-level scenes through scene files: the file saved from a handle and
    the host-written one load into scenes that render and cast exactly like
    the uploaded one (the same mesh BVHs; the top level rebuilt the same)."""
    import oracle
    from raycer_gb300 import scenes
    from raycer_gb300.tracer import RAY_DTYPE, camera_record

    from helpers import camera_floats

    sc = scenes.heightfield_blobs_instanced(instances=8, blob_level=2, hf_nx=32, hf_nz=16, width=48, height=27,
                                            seed=5)
    sc.settings.update(max_path_length=5)
    n = sc.width * sc.height
    rays = np.ascontiguousarray(oracle.camera_rays32(camera_floats(camera_record(sc)), sc.width, n))
    rays = rays.view(RAY_DTYPE).reshape(-1)
    with CudaTracer(0) as a:
        a.initializeInstanced(sc, seed=4)
        film = render(a, sc)
        hits = a.cast(rays)
        a.save_scene(tmp_path / "saved.rcgb")
    assert (hits["prim"] >= 0).mean() > 0.1, (hits["prim"] >= 0).mean()
    write_scene_file(sc, tmp_path / "written.rcgb")
    for name in ("saved.rcgb", "written.rcgb"):
        with CudaTracer(0) as b:
            b.load_scene(tmp_path / name, sc, seed=4)
            assert np.array_equal(render(b, sc), film), name
            assert np.array_equal(b.cast(rays), hits), name
