"""Batched path tracing: every scene's film equals rendering that scene alone
(bit for bit, frame after frame, after autotuning), with Russian roulette on
and off; Russian roulette leaves the image mean unbiased."""

from __future__ import annotations

import numpy as np
import pytest

from raycer_gb300 import scenes
from raycer_gb300.batch import Batch
from raycer_gb300.tracer import CudaTracer, TracerState, general_record

pytestmark = pytest.mark.gpu


def small_batch():
    specs = [(11, 300, 64, 48, 1, 8, 3), (12, 3000, 96, 64, 2, 8, 3), (13, 20000, 80, 60, 4, 8, 0),
             (14, 150000, 128, 96, 2, 6, 3), (15, 1200, 40, 30, 8, 4, 0)]
    return [scenes.room_with_extra(s, n, w, h, ms, depth, rr) for s, n, w, h, ms, depth, rr in specs]


def render_alone(sc, seed, frames):
    with CudaTracer(0) as t:
        t.initializeBuffers(sc, seed=seed)
        t.initializeImageBuffers(sc.width, sc.height)
        st = TracerState(scene=sc, filmWidth=sc.width, filmHeight=sc.height, pixelCount=sc.width * sc.height)
        films = []
        for _ in range(frames):
            t.run(st)
            films.append(t.read_film().copy())
        return films


def test_batch_equals_single_scene_renders():
    scs = small_batch()
    with Batch(0) as b:
        for i, sc in enumerate(scs):
            assert b.add_scene(sc, seed=100 + i) == i
        tuning = b.autotune(budget_ms=500.0)
        assert all(x in (64, 128, 256) for x in tuning["extend_block"])
        done1 = b.render()
        films1 = [b.read_film(i).copy() for i in range(len(scs))]
        stats = b.stats()
        b.render()
        films2 = [b.read_film(i).copy() for i in range(len(scs))]
    assert stats["passes"] >= 1 and stats["graph_nodes"] > stats["passes"]
    assert stats["rays_traced"] > 0 and stats["last_ms"] > 0
    assert np.all(done1 > 0) and np.all(done1 <= stats["last_ms"] + 1e-3)
    for i, sc in enumerate(scs):
        alone = render_alone(sc, 100 + i, 2)
        assert np.array_equal(films1[i], alone[0]), f"scene {i} frame 0"
        assert np.array_equal(films2[i], alone[1]), f"scene {i} frame 1"


def test_russian_roulette_is_unbiased():
    base = scenes.room_with_extra(21, 2000, 96, 72, 4, 8, 0)
    rr = scenes.room_with_extra(21, 2000, 96, 72, 4, 8, 3)
    means = {}
    for name, sc in (("off", base), ("on", rr)):
        with CudaTracer(0) as t:
            t.initializeBuffers(sc, seed=5)
            t.initializeImageBuffers(sc.width, sc.height)
            st = TracerState(scene=sc, filmWidth=sc.width, filmHeight=sc.height, pixelCount=sc.width * sc.height)
            frames = []
            for k in range(8):
                t.set_general(general_record(sc, seed=1000 * (name == "on") + k + 1))   # independent streams
                t.clear()
                t.run(st)
                lin = t.read_linear()[:, :3].astype(np.float64)
                frames.append(lin.mean(axis=0))
            means[name] = np.array(frames)          # 8 independent 16-spp frame means
    d = means["on"].mean(axis=0) - means["off"].mean(axis=0)
    se = np.sqrt(means["on"].var(axis=0, ddof=1) / 8 + means["off"].var(axis=0, ddof=1) / 8)
    assert np.all(np.abs(d) < 4.0 * se + 1e-6), (d, se)
