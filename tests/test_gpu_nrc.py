"""Radiance cache on the GPU: encoding, inference, gradients and Adam vs the
CPU oracle (oracle/nrc64.cpp); training; the cache inside PATH renders."""

from __future__ import annotations

import numpy as np
import pytest

import oracle
from raycer_gb300 import _native as N
from raycer_gb300 import scenes
from raycer_gb300.nrc import GroundTruth, RadianceCache, unpack_layers
from raycer_gb300.tracer import CudaTracer, TracerState, general_record

from helpers import nrc_box, nrc_init_params, nrc_queries, nrc_smooth_targets

pytestmark = pytest.mark.gpu

LO, HI = (-10.0, -2.0, -5.0), (10.0, 3.0, 5.0)
BOX = nrc_box(LO, HI)


@pytest.fixture(scope="module")
def cache():
    t = CudaTracer(0)
    c = RadianceCache(t, box_min=LO, box_max=HI, seed=1)
    yield c
    t.close()


def test_encoding_matches_oracle(cache):
    q = nrc_queries(1000, seed=1, lo=LO, hi=HI)
    gpu = cache.encode(q)
    ref = oracle.nrc_features(q, BOX)
    # BF16 rounding (2^-9 relative) + the float32 phase of the 2^11 pi terms
    assert np.all(np.abs(gpu - ref) <= np.abs(ref) * 2.0 ** -8 + 1.5e-3)
    assert np.all(gpu[:, 102] == 1.0) and np.all(gpu[:, 103:] == 0.0)
    # the float sin / cos are accurate to a few float ulps: BF16 rounding of
    # the float64 values agrees except next to a rounding boundary
    emu = oracle.nrc_features(q, BOX, emulate=True)
    assert np.mean(gpu == emu) > 0.999, np.mean(gpu == emu)


def test_inference_matches_oracle(cache):
    w = nrc_init_params(seed=5)
    cache.params = w
    q = nrc_queries(5003, seed=2, lo=LO, hi=HI)  # not a multiple of the 16-query tile
    gpu = cache.infer(q).astype(np.float64)
    emu = oracle.nrc_forward(w, q, BOX, emulate=True)
    pure = oracle.nrc_forward(w, q, BOX)
    rel_e = np.abs(gpu - emu) / np.abs(emu)
    rel_p = np.abs(gpu - pure) / np.abs(pure)
    # same rounding points as the oracle's BF16 emulation: float32 vs float64 sums only
    assert np.quantile(rel_e, 0.99) < 2e-3 and rel_e.max() < 2e-2, (np.quantile(rel_e, 0.99), rel_e.max())
    # against the float64 network: BF16 weights and activations
    assert np.median(rel_p) < 2e-2 and rel_p.max() < 0.2, (np.median(rel_p), rel_p.max())


@pytest.mark.parametrize("n", [16, 4100, 16384])
def test_gradient_matches_oracle(cache, n):
    w = nrc_init_params(seed=6)
    cache.params = w
    q = nrc_queries(n, seed=3, lo=LO, hi=HI)
    t = nrc_smooth_targets(q)
    g, loss = cache.gradient(q, t)
    ge, le = oracle.nrc_gradient(w, q, t, BOX, emulate=True)
    gp, lp = oracle.nrc_gradient(w, q, t, BOX)
    assert abs(loss - le) <= 2e-3 * le + 1e-7
    assert abs(loss - lp) <= 0.05 * lp
    assert np.all(g[20480 + 3 * 64:] == 0.0)
    for layer, (a, b, c) in enumerate(zip(unpack_layers(g.astype(np.float64)), unpack_layers(ge), unpack_layers(gp))):
        a, b, c = a[:3] if layer == 4 else a, b[:3] if layer == 4 else b, c[:3] if layer == 4 else c
        err_e = np.linalg.norm(a - b) / np.linalg.norm(b)
        cos_p = float(np.sum(a * c) / (np.linalg.norm(a) * np.linalg.norm(c)))
        assert err_e < 1e-2, (layer, err_e)
        assert cos_p > 0.98, (layer, cos_p)


def test_adam_steps_match_oracle(cache):
    w = nrc_init_params(seed=7)
    cache.params = w
    q = nrc_queries(4096, seed=4, lo=LO, hi=HI)
    t = nrc_smooth_targets(q)
    ge, _ = oracle.nrc_gradient(w, q, t, BOX, emulate=True)
    cache.train(q, t, steps=1)
    w1 = cache.params
    z = np.zeros_like(w)
    exp1, m1, v1 = oracle.nrc_adam(w, z, z, ge.astype(np.float32), 1)
    d = np.abs(w1 - exp1)
    big = np.abs(ge) > 1e-3 * np.abs(ge).max()
    # the first step moves every weight by -lr * sign(g): agreement wherever
    # the gradient is not at the rounding level
    assert np.mean(d[big] < 1e-5) > 0.995
    assert np.all(np.abs(w1 - w) <= 1e-2 * (1 + 1e-3) + 1e-6)
    assert np.all(w1[20480 + 3 * 64:] == 0.0)


def test_training_reduces_loss(cache):
    cache.params = nrc_init_params(seed=8)
    q = nrc_queries(16384, seed=5, lo=LO, hi=HI)
    t = nrc_smooth_targets(q)
    losses = cache.train(q, t, steps=300)
    assert np.all(np.isfinite(losses))
    assert losses[-1] < 0.1 * losses[0], (losses[0], losses[-1])
    qh = nrc_queries(4096, seed=6, lo=LO, hi=HI)
    pred = cache.infer(qh)
    th = nrc_smooth_targets(qh)
    assert np.median(np.abs(pred - th) / th) < 0.1


# ---------------------------------------------------------------------------
# The cache inside PATH renders.


def nrc_scene(width=128, height=72, enclosed=False):
    return scenes.heightfield_blobs_scene(instances=12, blob_level=3, hf_nx=96, hf_nz=48, width=width,
                                          height=height, enclosed=enclosed)


def render_film(sc, seed, frames=1, cache_cfg=None, read_cache=None):
    with CudaTracer(0) as t:
        t.initializeBuffers(sc, seed=seed)
        t.initializeImageBuffers(sc.width, sc.height)
        c = RadianceCache(t, **cache_cfg) if cache_cfg is not None else None
        st = TracerState(scene=sc, filmWidth=sc.width, filmHeight=sc.height, pixelCount=sc.width * sc.height)
        for _ in range(frames):
            t.run(st)
        film = t.read_film()
        extra = read_cache(c) if (read_cache and c) else None
    return film, extra


def test_render_without_termination_equals_plain():
    sc = nrc_scene()
    plain, _ = render_film(sc, seed=3, frames=2)
    # lookups never happen (segment 99) and 1 slot in 16 records a training path
    late, _ = render_film(sc, seed=3, frames=2, cache_cfg=dict(terminate_segment=99, train_steps=2))
    # every slot is a training path
    full, _ = render_film(sc, seed=3, frames=2, cache_cfg=dict(train_stride=1, train_steps=1))
    assert np.array_equal(plain, late)
    assert np.array_equal(plain, full)


def test_sky_radiance_reaches_the_film():
    sc = nrc_scene(64, 36)
    lit, _ = render_film(sc, seed=2)
    sc.settings["miss_radiance"] = None
    dark, _ = render_film(sc, seed=2)
    assert lit[:, :3].mean() > 0.05
    assert np.all(dark[:, :3] == 0.0)  # no emitters: the reference's miss returns black


def test_training_targets_are_path_radiance():
    """With every slot a training path, vertex 0's target is that pixel's plain
    path value (the film at 1 sample per pixel)."""
    sc = nrc_scene()
    film, samples = render_film(sc, seed=4, cache_cfg=dict(train_stride=1, train_steps=0,
                                                            sample_vertices=N.RC_NRC_ALL_VERTICES),
                                read_cache=lambda c: c.samples())
    vi, gi = RadianceCache.sample_tags(samples)
    assert samples.shape[0] > film.shape[0] // 2
    v0 = vi == 0
    tgt = samples[v0, 12:15].astype(np.float64)
    ref = film[gi[v0], :3].astype(np.float64)
    np.testing.assert_allclose(tgt, ref, rtol=2e-5, atol=1e-7)
    # queries lie on surfaces with unit directions and normals
    np.testing.assert_allclose(np.linalg.norm(samples[:, 3:6], axis=1), 1.0, atol=1e-5)
    np.testing.assert_allclose(np.linalg.norm(samples[:, 6:9], axis=1), 1.0, atol=1e-4)
    assert np.all((samples[:, 9:12] >= 0.1 - 1e-6) & (samples[:, 9:12] <= 0.9 + 1e-6))
    # at most max_path_length vertices per path, each counted once
    assert vi.max() < sc.settings["max_path_length"]
    assert len(set(zip(vi.tolist(), gi.tolist()))) == samples.shape[0]


def test_lookup_vertex_samples_are_the_lookup_vertex_targets():
    """RC_NRC_LOOKUP_VERTEX (the default): a training path's only sample is
    its vertex at terminate_segment, whose suffix has the depth budget of a
    lookup there; on the same paths it equals the every-vertex run's sample
    of that vertex, record for record."""
    sc = nrc_scene()
    runs = {}
    for mode in (N.RC_NRC_ALL_VERTICES, N.RC_NRC_LOOKUP_VERTEX):
        _, samples = render_film(sc, seed=4, cache_cfg=dict(train_stride=1, train_steps=0, sample_vertices=mode),
                                 read_cache=lambda c: c.samples())
        runs[mode] = samples
    vi, gi = RadianceCache.sample_tags(runs[N.RC_NRC_LOOKUP_VERTEX])
    assert vi.size > 100 and np.all(vi == 2)
    va, ga = RadianceCache.sample_tags(runs[N.RC_NRC_ALL_VERTICES])
    at2 = runs[N.RC_NRC_ALL_VERTICES][va == 2]
    key = lambda a: np.lexsort((RadianceCache.sample_tags(a)[1],))
    lv = runs[N.RC_NRC_LOOKUP_VERTEX]
    assert np.array_equal(lv[key(lv)], at2[key(at2)])


def zero_cache_params() -> np.ndarray:
    """Weights whose output is exp(-30) ~ 0 everywhere: one hidden unit carries
    the constant input through the ReLU layers and the output layer scales
    it by -30. A tracer with this cache ends its paths at the lookup with no
    estimate of the rest: the method without the network."""
    w = np.zeros(20992, np.float32)
    w[0 * 128 + 102] = 1.0           # W1[0][102]: the constant feature
    for off in (8192, 12288, 16384):  # W2..W4[0][0]
        w[off] = 1.0
    for c in range(3):               # W5[c][0]
        w[20480 + c * 64] = -30.0
    return w


@pytest.mark.parametrize("lighting", ["enclosed", "sky"])
def test_trained_cache_gain(lighting):
    """At equal frames, against a float64 high-spp ground truth: the trained
    cache's image is far closer than the same tracer's with a zero cache
    (paths cut at the lookup) and than with an untrained cache, and not
    worse than plain path tracing beyond noise. Closed box: the default
    training (the lookup vertex's samples). Sky-lit, where few paths live to
    the lookup vertex and a 128x72 film gives it a few dozen samples per
    frame: every vertex's samples."""
    sc = nrc_scene(enclosed=lighting == "enclosed")
    mode = N.RC_NRC_LOOKUP_VERTEX if lighting == "enclosed" else N.RC_NRC_ALL_VERTICES
    with CudaTracer(0) as t:
        t.initializeBuffers(sc, seed=9)
        t.initializeImageBuffers(sc.width, sc.height)
        st = TracerState(scene=sc, filmWidth=sc.width, filmHeight=sc.height, pixelCount=sc.width * sc.height)
        gt = GroundTruth(t)
        for _ in range(512):
            t.run(st)
            gt.add_film(clear_film=True)
        # the renders below restart the frame counter: a different seed keeps
        # their samples independent of the ground truth's
        t.set_general(general_record(sc, seed=10))

        def rmse_after(frames, params=None, **cfg):
            t.clear()
            c = RadianceCache(t, **cfg)
            if params is not None:
                c.params = params
            for _ in range(frames):
                t.run(st)
            r = gt.rmse()
            c.set_enabled(False)
            return r

        frames = 128
        zero = rmse_after(frames, params=zero_cache_params(), train_steps=0, sample_vertices=mode)
        untrained = rmse_after(frames, train_steps=0, seed=3, sample_vertices=mode)
        trained = rmse_after(frames, seed=3, sample_vertices=mode)
        t.clear()
        for _ in range(frames):
            t.run(st)
        plain = gt.rmse()
    print(f"{lighting}: rmse after {frames} frames: trained cache {trained:.4f}, untrained {untrained:.4f}, "
          f"zero cache {zero:.4f}, plain {plain:.4f}")
    assert trained < 0.5 * zero
    assert trained < untrained
    assert trained < 1.15 * plain


@pytest.mark.parametrize("n", [128, 1000, 20000])
def test_tcgen05_lookups_match_mma_sync(n):
    """The tcgen05 / TMEM lookup kernel against the warp-level mma.sync one
    (same BF16 operands, FP32 sums in another order) and the oracle."""
    w = nrc_init_params(seed=9)
    q = nrc_queries(n, seed=12, lo=LO, hi=HI)
    outs = []
    for kind in (0, 1):
        with CudaTracer(0) as t:
            c = RadianceCache(t, box_min=LO, box_max=HI, lookup_kernel=kind)
            c.params = w
            outs.append(c.infer(q).astype(np.float64))
    rel = np.abs(outs[1] - outs[0]) / np.abs(outs[0])
    assert np.quantile(rel, 0.99) < 1e-3 and rel.max() < 2e-2, (np.quantile(rel, 0.99), rel.max())
    emu = oracle.nrc_forward(w, q, BOX, emulate=True)
    rel_e = np.abs(outs[1] - emu) / np.abs(emu)
    assert np.quantile(rel_e, 0.99) < 2e-3, np.quantile(rel_e, 0.99)


def test_tcgen05_lookups_in_renders():
    sc = nrc_scene()
    films = []
    for kind in (0, 1):
        film, _ = render_film(sc, seed=5, frames=3, cache_cfg=dict(lookup_kernel=kind))
        films.append(film[:, :3] / film[:, 3:4])
    # the first frame's lookups come from the same untrained weights and the
    # training sees the same samples: the images agree to rounding
    np.testing.assert_allclose(films[1].mean(), films[0].mean(), rtol=1e-3)
