"""Traversal parity on degenerate geometry, for the smallest and largest leaf
sizes (1 and 15 triangles, the reference's maxLeafSize range here): a soup
of duplicated triangles (equal centroids: the builder's half-split
fallback; every hit is a tie between identical triangles, decided by the
tie rule), coplanar triangles (many equal distances), long thin slivers
(determinants near zero), and a cluster of tiny triangles beside large
ones. Closest-hit and any-hit casts, RAY frames and PATH films all equal the
float32 oracle's bit for bit, in both traversal orders."""

from __future__ import annotations

import numpy as np
import pytest

import oracle
from raycer_gb300 import _native as N
from raycer_gb300 import scenes
from raycer_gb300.tracer import RAY_DTYPE, CudaTracer, TracerState, camera_record

from helpers import camera_floats

pytestmark = pytest.mark.gpu


def _soup(n, seed, spread=1.0, size=0.1):
    rng = np.random.default_rng(seed)
    c = rng.uniform(-spread, spread, size=(n, 1, 3))
    v = (c + rng.normal(scale=size, size=(n, 3, 3))).reshape(n, 9)
    return v


def _coplanar():
    v = _soup(600, 8)
    v[:, 2::3] = -0.5          # every vertex on the plane z = -0.5
    return v


def _slivers():
    # long thin triangles: the third vertex 1e-2 of the edge length off the
    # midpoint of the other two (determinants near zero)
    rng = np.random.default_rng(9)
    a = rng.uniform(-1.0, 1.0, size=(600, 3))
    b = a + rng.normal(scale=0.3, size=(600, 3))
    off = rng.normal(size=(600, 3))
    off /= np.linalg.norm(off, axis=1, keepdims=True)
    c = 0.5 * (a + b) + 1e-2 * np.linalg.norm(b - a, axis=1, keepdims=True) * off
    return np.concatenate([a, b, c], axis=1)


CASES = {
    "duplicates": lambda: np.repeat(_soup(24, 7, size=0.3), 20, axis=0),
    "coplanar": _coplanar,
    "slivers": _slivers,
    "clustered": lambda: np.concatenate([_soup(800, 5, spread=0.02, size=0.01), _soup(400, 6, spread=1.5)]),
}


def scene(case: str, leaf: int, width=64, height=48) -> scenes.SceneDesc:
    v = CASES[case]().astype(np.float32).astype(np.float64)
    n = v.shape[0]
    mats = [scenes.Material(diffuse=(0.6, 0.6, 0.6)),
            scenes.Material(diffuse=(0.0, 0.0, 0.0), emittance=(3.0, 3.0, 3.0), is_emissive=True)]
    midx = (np.arange(n) % 7 == 0).astype(np.uint32)   # every 7th triangle emits
    return scenes.SceneDesc(f"{case}/{leaf}", v, midx, mats, scenes.CameraDesc(position=(0.0, 0.0, 4.0), fov=50.0),
                            width, height, light_direction=(-0.4, -1.0, -0.6), max_leaf_size=leaf,
                            settings={"tracer": "ray", "max_path_length": 4})


def _rays(n, seed):
    rng = np.random.default_rng(seed)
    r = np.zeros(n, RAY_DTYPE)
    r["origin"] = rng.uniform(-2.0, 2.0, size=(n, 3))
    d = rng.normal(size=(n, 3))
    r["direction"] = d / np.linalg.norm(d, axis=1, keepdims=True)
    r["t_max"] = np.float32(3.0e38)
    # a quarter aimed exactly along -z at the coplanar sheet and the clusters
    k = n // 4
    r["origin"][:k] = np.column_stack([rng.uniform(-1.0, 1.0, k), rng.uniform(-1.0, 1.0, k), np.full(k, 3.0)])
    r["direction"][:k] = (0.0, 0.0, -1.0)
    return r


@pytest.mark.parametrize("order", [N.RC_ORDER_REFERENCE, N.RC_ORDER_NEAREST])
@pytest.mark.parametrize("leaf", [1, 15])
@pytest.mark.parametrize("case", sorted(CASES))
def test_casts_and_frames(case, leaf, order):
    sc = scene(case, leaf)
    rays = _rays(20_000, leaf + 31 * order)
    n = sc.width * sc.height
    with CudaTracer(0) as t:
        t.initializeBuffers(sc)
        t.set_traversal_order(order)
        hits = {a: t.cast(rays, any_hit=a, order=order) for a in (False, True)}
        t.initializeImageBuffers(sc.width, sc.height)
        t.run(TracerState(scene=sc, filmWidth=sc.width, filmHeight=sc.height, pixelCount=n))
        frame = t.read_cast().view(np.int32).reshape(-1, 4)
        cam = camera_floats(camera_record(sc))
    orc = oracle.Oracle(sc)
    r8 = np.ascontiguousarray(rays).view(np.float32).reshape(-1, 8)
    for a, h in hits.items():
        prim, tt, u, v, _ = orc.cast32(r8, any_hit=a, order=order)
        assert np.array_equal(h["prim"], prim), (a, int((h["prim"] != prim).sum()))
        assert np.array_equal(h["t"], tt) and np.array_equal(h["u"], u) and np.array_equal(h["v"], v)
    assert (hits[False]["prim"] >= 0).sum() > 100
    ref, _ = orc.raycast32(cam, sc.width, n, -np.array(sc.light_direction, np.float32), order=order)
    assert np.array_equal(frame, ref), f"{(frame != ref).any(axis=1).sum()} pixels differ"


@pytest.mark.parametrize("leaf", [1, 15])
@pytest.mark.parametrize("case", ["duplicates", "clustered"])
def test_path_films(case, leaf):
    """PATH films through the 4-wide tree collapsed from these trees equal
    the float32 oracle's (2x2 CMJ samples per pixel, depth 4)."""
    sc = scene(case, leaf)
    sc.settings.update(tracer="path", multi_sample_count_sqrt=2, path_sample_count=1, sampler="cmj")
    n = sc.width * sc.height
    with CudaTracer(0) as t:
        t.initializeBuffers(sc, seed=4)
        t.initializeImageBuffers(sc.width, sc.height)
        t.run(TracerState(scene=sc, filmWidth=sc.width, filmHeight=sc.height, pixelCount=n))
        film = t.read_film()
        cam = camera_floats(camera_record(sc))
    ref, _ = oracle.Oracle(sc).render_path32(cam, sc.width, n, 2, 1, 4, (0.5, 0.5), 1e-5, 4, 0, 1, 4, 0)
    assert np.array_equal(film, ref), f"{(film != ref).any(axis=1).sum()} pixels differ"
    assert film[:, :3].max() > 0.0
