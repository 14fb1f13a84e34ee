"""GPU linear-BVH builder: valid trees for regular and degenerate inputs,
the same closest hits as the reference's SAH tree (except equal-distance
ties) and identical occlusion; equal films up to ties."""

from __future__ import annotations

import numpy as np
import pytest

from raycer_gb300 import _native as N
from raycer_gb300 import scenes
from raycer_gb300.tracer import CudaTracer, TracerState, camera_record

import oracle
from helpers import camera_floats, small_heightfield, small_room

pytestmark = pytest.mark.gpu


def check_tree(sc, nodes, order, leaf_max):
    n = sc.triangle_count
    assert sorted(order.tolist()) == list(range(n))
    v = sc.vertices.astype(np.float32).reshape(-1, 3, 3)
    assert nodes[0]["start_offset"] == 0 and nodes[0]["primitive_count"] == n
    for i, nd in enumerate(nodes):
        lo, hi = nd["aabb_min"], nd["aabb_max"]
        if nd["right_offset"] == 0:
            assert 1 <= nd["primitive_count"] <= leaf_max
            tri = v[order[nd["start_offset"]:nd["start_offset"] + nd["primitive_count"]]].reshape(-1, 3)
            assert np.all(tri >= lo.astype(np.float32)) and np.all(tri <= hi.astype(np.float32))
        else:
            for c in (i + 1, i + nd["right_offset"]):
                assert np.all(nodes[c]["aabb_min"] >= lo) and np.all(nodes[c]["aabb_max"] <= hi)


def upload(t, sc, builder):
    assert t._lib.rc_set_bvh_builder(t._h, builder) == N.RC_OK
    t.initializeBuffers(sc, seed=3)


def degenerate(kind, n=2000, seed=0):
    rng = np.random.default_rng(seed)
    if kind == "same":       # every triangle identical: all Morton codes equal
        tri = np.tile(np.array([[0, 0, 0, 1, 0, 0, 0, 1, 0]], np.float64), (n, 1))
    elif kind == "line":     # centroids on a line
        x = rng.random(n) * 10
        tri = np.stack([x, 0 * x, 0 * x, x + 0.1, 0 * x, 0 * x, x, 0.1 + 0 * x, 0 * x], 1)
    else:                    # random
        c = rng.random((n, 3)) * 4 - 2
        tri = np.concatenate([c + rng.normal(size=(n, 3)) * 0.05 for _ in range(3)], 1)
    sc = small_room(width=32, height=24, clutter=0)
    return scenes.SceneDesc(name=kind, vertices=tri, material_index=np.zeros(n, np.uint32),
                            materials=sc.materials[:1], camera=sc.camera, width=32, height=24,
                            light_direction=None, max_leaf_size=4, settings=dict(sc.settings))


@pytest.mark.parametrize("kind", ["room", "heightfield", "same", "line", "random", "one", "three", "five"])
def test_tree_is_valid(kind):
    if kind == "room":
        sc = small_room()
    elif kind == "heightfield":
        sc = small_heightfield()
    elif kind in ("one", "three", "five"):
        sc = degenerate("random", n={"one": 1, "three": 3, "five": 5}[kind])
    else:
        sc = degenerate(kind)
    with CudaTracer(0) as t:
        upload(t, sc, N.RC_BUILDER_GPU_LBVH)
        nodes, order = t.get_bvh()
        st = t.stats()
    check_tree(sc, nodes, order, sc.max_leaf_size)
    assert 1 <= st["bvh_depth"] <= 64


def test_hits_match_sah_tree():
    sc = small_heightfield(width=320, height=180)
    cam = camera_floats(camera_record(sc))
    rays = oracle.camera_rays32(cam, sc.width, sc.width * sc.height)
    res = {}
    for b in (N.RC_BUILDER_REFERENCE_SAH, N.RC_BUILDER_GPU_LBVH):
        with CudaTracer(0) as t:
            upload(t, sc, b)
            t.initializeImageBuffers(sc.width, sc.height)
            res[b] = (t.cast(rays), t.cast_with_shadow(rays), t.stats()["build_ms"])
    a, b = res[N.RC_BUILDER_REFERENCE_SAH][0], res[N.RC_BUILDER_GPU_LBVH][0]
    same = a["prim"] == b["prim"]
    # a different primitive only at an equal distance (a tie on a shared edge)
    assert np.all(a["t"][~same] == b["t"][~same])
    assert same.mean() > 0.999
    sa, sb = res[N.RC_BUILDER_REFERENCE_SAH][1], res[N.RC_BUILDER_GPU_LBVH][1]
    hit = (sa["prim"] >= 0) & (sb["prim"] >= 0)
    agree = (sa["occluder"] >= 0) == (sb["occluder"] >= 0)
    assert agree[hit & same].all()


def test_films_match_up_to_ties():
    sc = small_room(width=64, height=48)
    sc.settings.update(multi_sample_count_sqrt=2, max_path_length=4)
    films = []
    for b in (N.RC_BUILDER_REFERENCE_SAH, N.RC_BUILDER_GPU_LBVH):
        with CudaTracer(0) as t:
            upload(t, sc, b)
            t.initializeImageBuffers(sc.width, sc.height)
            t.run(TracerState(scene=sc, filmWidth=sc.width, filmHeight=sc.height, pixelCount=sc.width * sc.height))
            films.append(t.read_film())
    differ = (films[0] != films[1]).any(axis=1)
    assert differ.mean() < 0.01, differ.mean()
