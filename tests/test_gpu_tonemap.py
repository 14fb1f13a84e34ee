"""Device Reinhard + gamma resolve vs the reference's ReinhardToneMapper
(golden outputs) and the float64 oracle, on identical linear input."""

from __future__ import annotations

import numpy as np
import pytest

import oracle
from raycer_gb300 import _native as N
from raycer_gb300.tracer import CudaTracer

from test_golden_pins import _load

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("key,gamma,clamp,ag", [(0.18, 2.2, 1, 1), (0.5, 1.8, 1, 1), (0.18, 2.2, 0, 1),
                                                (0.18, 2.2, 1, 0)])
def test_reinhard_matches_reference(key, gamma, clamp, ag):
    import ctypes as C
    g = _load("tonemap.npz")
    lin = g["linear"]
    with CudaTracer(0) as t:
        tm = N.rc_tonemapper()
        N.lib().rc_tonemapper_defaults(C.byref(tm))
        tm.key, tm.gamma, tm.should_clamp, tm.apply_gamma = key, gamma, clamp, ag
        assert N.lib().rc_set_tonemapper(t.handle, C.byref(tm)) == N.RC_OK
        out = t.tonemap_film(lin)
    ref = g[f"out_{key}_{gamma}_{clamp}_{ag}"]
    # Summation order of the log-luminance differs (per-thread in the
    # reference); fastPow's 2^-20 high-word steps bound the effect.
    scale = max(1.0, float(np.nanmax(np.abs(ref))))
    assert np.array_equal(np.isnan(out), np.isnan(ref))
    assert np.nanmax(np.abs(out - ref)) <= 4e-6 * scale
    o64 = oracle.tonemap64(lin, key, gamma, bool(clamp), bool(ag))
    assert np.nanmax(np.abs(out - o64)) <= 4e-6 * scale
    assert np.all(out[:, 3] == 1.0)


@pytest.mark.parametrize("pinned", [False, True])
def test_resolve_in_place_equals_copied_image(pinned):
    """rc_resolve maps the film straight into the caller's buffer where the
    device reaches it (here: any memory on a Grace host, or page-locked
    memory); the image equals rc_tonemap_film's, which copies through device
    buffers, bit for bit. A buffer that is not 16-byte aligned takes the
    copy and gives the same image."""
    import ctypes as C

    import torch

    from raycer_gb300.tracer import TracerState

    from helpers import small_room

    sc = small_room(width=96, height=64)
    n = sc.width * sc.height
    with CudaTracer(0) as t:
        t.initializeBuffers(sc, seed=2)
        t.initializeImageBuffers(sc.width, sc.height)
        t.run(TracerState(scene=sc, filmWidth=sc.width, filmHeight=sc.height, pixelCount=n))
        ref = t.tonemap_film(t.read_film())
        if pinned:
            buf = torch.empty((n, 4), dtype=torch.float32, pin_memory=True)
            assert N.lib().rc_resolve(t.handle, C.c_void_p(buf.data_ptr())) == N.RC_OK
            img = buf.numpy()
        else:
            img = t.downloadImage().reshape(n, 4)
        raw = np.zeros(n * 4 + 1, np.float32)          # one float off the 16-byte grid
        assert N.lib().rc_resolve(t.handle, C.c_void_p(raw.ctypes.data + 4)) == N.RC_OK
    assert np.array_equal(img, ref)
    assert np.array_equal(raw[1:].reshape(n, 4), ref)
    assert np.isfinite(ref).all() and ref[:, :3].max() > 0.0
