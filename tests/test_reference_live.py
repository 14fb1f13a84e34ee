"""Live checks against the reference's own code (oracle/_ref), where it was
compiled from its sources: BVH builds on random and degenerate triangle sets,
float64 queries, Triangle::initialize frames."""

from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import oracle
from raycer_gb300 import scenes

from test_golden_pins import product_bvh

pytestmark = pytest.mark.skipif(not oracle.ref_available(), reason="reference build (oracle/_ref) not present")


def soup(n, seed, spread=1.0, size=0.1):
    rng = np.random.default_rng(seed)
    c = rng.uniform(-spread, spread, size=(n, 1, 3))
    v = (c + rng.normal(scale=size, size=(n, 3, 3))).reshape(n, 9)
    return v.astype(np.float32).astype(np.float64)


def make(v, leaf):
    return scenes.SceneDesc("soup", v, np.zeros(v.shape[0], np.uint32), [scenes.Material(diffuse=(0.5, 0.5, 0.5))],
                            scenes.CameraDesc(position=(0, 0, 5), fov=60), 64, 48, max_leaf_size=leaf)


CASES = {
    "single": soup(1, 1),
    "root_leaf": soup(4, 2),
    "five": soup(5, 3),
    "random_2k": soup(2000, 4),
    "clustered": np.concatenate([soup(500, 5, spread=0.01), soup(500, 6, spread=3.0)]),
    "duplicates": np.repeat(soup(3, 7), 40, axis=0),          # equal centroids: half-split fallback
    "coplanar": (lambda v: (v.__setitem__((slice(None), slice(1, 9, 3)), 0.0), v)[1])(soup(300, 8)),
    "collinear": (lambda v: (v.__setitem__((slice(None), [1, 2, 4, 5, 7, 8]), v[:, [1, 2, 4, 5, 7, 8]] * 1e-3),
                             v)[1])(soup(300, 9)),
}


@pytest.mark.parametrize("leaf", [1, 2, 4, 5, 15])
@pytest.mark.parametrize("case", sorted(CASES))
def test_bvh_equals_reference(case, leaf):
    v = CASES[case]
    sc = make(v, leaf)
    ref_nodes, ref_order = oracle.RefScene(sc).bvh()
    pn, po, _ = product_bvh(sc)
    assert np.array_equal(pn, ref_nodes)
    assert np.array_equal(po, ref_order)
    on, oo = oracle.Oracle(sc).bvh()
    assert np.array_equal(on, ref_nodes) and np.array_equal(oo, ref_order)


@pytest.mark.parametrize("case", ["random_2k", "clustered", "duplicates"])
def test_fp64_queries_equal_reference(case):
    sc = make(CASES[case], 4)
    ref = oracle.RefScene(sc)
    orc = oracle.Oracle(sc)
    rng = np.random.default_rng(11)
    n = 20000
    o = rng.uniform(-3, 3, size=(n, 3))
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r6 = np.concatenate([o, d], axis=1)
    for shadow in (False, True):
        p1, t1 = ref.intersect(r6, shadow=shadow)
        p2, t2, _, _ = orc.intersect64(r6, shadow=shadow)
        assert np.array_equal(p1, p2)
        assert np.array_equal(t1, t2)


def test_triangle_frames_equal_reference():
    sc = make(CASES["random_2k"], 4)
    ref = oracle.RefScene(sc)
    fr = oracle.Oracle(sc).frames()
    for i in range(0, sc.triangle_count, 37):
        assert np.array_equal(fr[i], ref.frame(i))


def test_room_path_trace_ray_count_matches_port():
    """The reference's Tracer::run and the float64 port issue the same number of
    BVH queries in expectation (same estimator, same depth rule)."""
    sc = scenes.room_scene(width=64, height=48)
    ref = oracle.RefScene(sc)
    ref.set_general(1, 4, 1, 2)
    _, _, rays_ref, _ = ref.render(64, 48)
    orc = oracle.Oracle(sc)
    cam64 = oracle.cam64_from_state(ref.camera_state(64, 48))
    _, rays_port, _ = orc.render_path64(cam64, 64, 64 * 48, 4, 1, 2, seed=5)
    assert abs(rays_port - rays_ref) < 0.03 * rays_ref
