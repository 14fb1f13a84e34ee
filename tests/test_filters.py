"""Film reconstruction filters (Rendering/Filters/*.cpp): the float64 port
equals the reference's own filters, the float32 twin of the device is within
float rounding of them, and its exp() is accurate. CPU only."""

from __future__ import annotations

import numpy as np
import pytest

import oracle

NAMES = {0: "box", 1: "tent", 2: "bell", 3: "gaussian", 4: "mitchell", 5: "lanczos"}
REF_RADIUS = {0: 0.5, 1: 1.0, 2: 1.5, 3: 7.43384 / 2.0, 4: 2.0, 5: 2.0}


def offsets(r: float) -> np.ndarray:
    rng = np.random.default_rng(1)
    x = np.concatenate([np.linspace(-1.1 * r, 1.1 * r, 2001), rng.uniform(-r, r, 4000),
                        [0.0, -r, r, 0.5, -0.5, 1.0, -1.0, 1.5, -1.5, 2.0, -2.0]])
    return x


@pytest.mark.parametrize("ftype", sorted(NAMES))
def test_port_equals_reference(ftype):
    if not oracle.ref_available():
        pytest.skip("reference library not built here")
    x = offsets(REF_RADIUS[ftype])
    ref, rr = oracle.ref_filter_weight(ftype, x)
    port, rp = oracle.filter_weight64(ftype, x)
    assert rr == rp == pytest.approx(REF_RADIUS[ftype], abs=0)
    np.testing.assert_array_equal(port, ref)


@pytest.mark.parametrize("ftype", sorted(NAMES))
def test_device_twin_within_float_rounding(ftype):
    r = REF_RADIUS[ftype]
    x = offsets(r).astype(np.float32)
    w32, r32 = oracle.filter_weight32(ftype, x)
    w64, r64 = oracle.filter_weight64(ftype, x.astype(np.float64))
    assert r32 == np.float32(r64)
    peak = np.abs(w64).max()
    # float32 evaluation: a few ulp of the peak weight
    np.testing.assert_allclose(w32, w64, rtol=2e-6, atol=2e-6 * peak)


def test_filter_exp_accuracy():
    t = np.linspace(-7.0, 0.0, 100001).astype(np.float32)
    e = oracle.filter_exp32(t).astype(np.float64)
    ref = np.exp(t.astype(np.float64))
    assert np.max(np.abs(e - ref) / ref) < 4e-7
