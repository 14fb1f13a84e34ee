"""Instanced scenes and dielectrics on the GPU: closest hits of the
two-level traversal against the reference's Instance traversal (committed
fixture), renders against the flattened scene, dielectric films bit-exact
against the float32 twin."""

from __future__ import annotations

import numpy as np
import pytest

import oracle
from raycer_gb300 import scenes
from raycer_gb300.tracer import RAY_DTYPE, CudaTracer, TracerState, camera_record

from helpers import camera_floats, small_room
from test_instancing import FIX, PARAMS, flat_to_mesh

pytestmark = pytest.mark.gpu


def test_hits_match_reference_instances():
    sc = scenes.heightfield_blobs_instanced(**PARAMS)
    rays = np.ascontiguousarray(FIX["rays"]).view(RAY_DTYPE).reshape(-1)
    with CudaTracer(0) as t:
        t.initializeInstanced(sc)
        hits = t.cast(rays)
    mesh, local = flat_to_mesh(sc, hits["prim"].astype(np.int64))
    same = (mesh == FIX["mesh"]) & (local == FIX["local"])
    assert same.mean() > 0.995, same.mean()
    hit = same & (hits["prim"] >= 0)
    np.testing.assert_allclose(hits["t"][hit], FIX["t"][hit], rtol=2e-5)


def test_instanced_render_matches_flattened():
    sc = scenes.heightfield_blobs_instanced(**PARAMS)
    sc.settings.update(max_path_length=6)
    flat = sc.flatten()
    means = []
    for s, inst in ((sc, True), (flat, False)):
        with CudaTracer(0) as t:
            if inst:
                t.initializeInstanced(s, seed=4)
            else:
                t.initializeBuffers(s, seed=4)
            t.initializeImageBuffers(s.width, s.height)
            st = TracerState(scene=s, filmWidth=s.width, filmHeight=s.height, pixelCount=s.width * s.height)
            for _ in range(32):
                t.run(st)
            f = t.read_film()
            means.append(f[:, :3] / f[:, 3:4])
    a, b = means
    assert abs(a.mean() - b.mean()) < 0.01 * b.mean()
    # An instance transforms its mesh's shading frame (Instance.cpp:98-99), the
    # flattened triangle builds its own: same distribution, other directions
    # for the same random numbers, so compare 10x10-block means.
    h, w = sc.height, sc.width
    ba = a.mean(axis=1).reshape(h // 10, 10, w // 10, 10).mean(axis=(1, 3))
    bb = b.mean(axis=1).reshape(h // 10, 10, w // 10, 10).mean(axis=(1, 3))
    rel = np.sqrt(np.mean((ba - bb) ** 2)) / bb.mean()
    assert rel < 0.05, rel


def test_instanced_ray_frames():
    """RAY frames of a two-level scene: the primary records are rc_cast's
    closest hits of the same camera rays (the same two-level traversal,
    flattened primitive numbering), the shadow stage's occlusion agrees with
    the flattened scene's RAY frame, and the caller-ray path through host
    buffers returns the frame's records."""
    sc = scenes.heightfield_blobs_instanced(**PARAMS)
    sc.settings["tracer"] = "ray"
    sc.light_direction = (-1.0, -0.35, -0.2)  # low light: long shadows over the blobs
    n = sc.width * sc.height
    rays = np.ascontiguousarray(oracle.camera_rays32(camera_floats(camera_record(sc)), sc.width, n))
    rays = rays.view(RAY_DTYPE).reshape(-1)
    with CudaTracer(0) as t:
        t.initializeInstanced(sc)
        t.initializeImageBuffers(sc.width, sc.height)
        t.run(TracerState(scene=sc, filmWidth=sc.width, filmHeight=sc.height, pixelCount=n))
        frame = t.read_cast()
        hits = t.cast(rays)
        out = t.cast_with_shadow(rays)
    assert np.array_equal(frame["prim"], hits["prim"])
    assert np.array_equal(frame["t"][hits["prim"] >= 0], hits["t"][hits["prim"] >= 0])
    assert np.array_equal(out, frame)
    hit = frame["prim"] >= 0
    assert hit.mean() > 0.5
    # every hit pixel cast its shadow ray; misses did not
    assert np.array_equal((frame["flags"] & 2) != 0, hit)
    assert np.all(frame["occluder"][hit & ((frame["flags"] & 4) == 0)] == -1)
    assert np.all(frame["occluder"][(frame["flags"] & 4) != 0] >= 0)

    flat = sc.flatten()
    flat.settings["tracer"] = "ray"
    with CudaTracer(0) as t:
        t.initializeBuffers(flat)
        t.initializeImageBuffers(flat.width, flat.height)
        t.run(TracerState(scene=flat, filmWidth=flat.width, filmHeight=flat.height, pixelCount=n))
        ref = t.read_cast()
    both = hit & (ref["prim"] >= 0)
    assert both.mean() > 0.99 * hit.mean()
    occ_i = (frame["flags"][both] & 4) != 0
    occ_f = (ref["flags"][both] & 4) != 0
    assert 0.1 < occ_f.mean() < 0.9, occ_f.mean()
    assert (occ_i == occ_f).mean() > 0.99, (occ_i == occ_f).mean()


@pytest.mark.parametrize("ms", [1, 2])
def test_dielectric_film_bit_exact(ms):
    sc = small_room(width=40, height=30)
    # make a third of the clutter glass
    mats = list(sc.materials)
    rng = np.random.default_rng(3)
    for i in range(1, len(mats)):
        if not mats[i].is_emissive and rng.random() < 0.35:
            m = mats[i]
            mats[i] = scenes.Material(diffuse=m.diffuse, dielectric=True, ior=float(np.float32(1.3 + 0.4 * rng.random())))
    sc.materials = mats
    sc.settings.update(multi_sample_count_sqrt=ms, max_path_length=6)
    assert any(m.dielectric for m in mats)
    with CudaTracer(0) as t:
        t.initializeBuffers(sc, seed=8)
        t.initializeImageBuffers(sc.width, sc.height)
        t.run(TracerState(scene=sc, filmWidth=sc.width, filmHeight=sc.height, pixelCount=sc.width * sc.height))
        film = t.read_film()
        cam = camera_floats(camera_record(sc))
    orc = oracle.Oracle(sc)
    ref, _ = orc.render_path32(cam, sc.width, sc.width * sc.height, ms, 1, 4, (0.5, 0.5), 1e-5, 6, 0, 1, 8, 0)
    assert np.array_equal(film, ref), f"{(film != ref).any(axis=1).sum()} pixels differ"


def test_cache_renders_instanced_dielectric_scene():
    from raycer_gb300.nrc import RadianceCache
    sc = scenes.heightfield_blobs_instanced(**PARAMS, dielectric_fraction=0.3)
    with CudaTracer(0) as t:
        t.initializeInstanced(sc, seed=2)
        t.initializeImageBuffers(sc.width, sc.height)
        c = RadianceCache(t)
        st = TracerState(scene=sc, filmWidth=sc.width, filmHeight=sc.height, pixelCount=sc.width * sc.height)
        for _ in range(8):
            t.run(st)
        film = t.read_film()
        stats = c.stats()
    assert np.isfinite(film).all() and film[:, :3].mean() > 0.05
    assert stats["lookups"] > 0 and stats["training_samples"] > 0 and np.isfinite(stats["last_loss"])
