"""The radiance-cache oracle (oracle/nrc64.cpp) checked against itself:
finite differences pin its analytic gradient, the encoding obeys its
definition, and the BF16-emulating variant stays close to pure float64.
CPU only."""

from __future__ import annotations

import numpy as np
import pytest

import oracle
from tests.helpers import nrc_box, nrc_init_params, nrc_queries, nrc_smooth_targets

BOX = nrc_box()


def test_features_follow_definition():
    q = nrc_queries(64, seed=3)
    f = oracle.nrc_features(q, BOX)
    lo, inv = BOX
    u = (q[:, :3].astype(np.float64) - lo) * inv
    for a in range(3):
        for k in range(12):
            np.testing.assert_allclose(f[:, a * 24 + 2 * k], np.sin(np.pi * 2.0 ** k * u[:, a]), atol=1e-9)
            np.testing.assert_allclose(f[:, a * 24 + 2 * k + 1], np.cos(np.pi * 2.0 ** k * u[:, a]), atol=1e-9)
    ud = 0.5 * (q[:, 3:6].astype(np.float64) + 1.0)
    for a in range(3):
        for k in range(4):
            np.testing.assert_allclose(f[:, 72 + a * 8 + 2 * k], np.sin(np.pi * 2.0 ** k * ud[:, a]), atol=1e-12)
    np.testing.assert_array_equal(f[:, 96:102], q[:, 6:12].astype(np.float64))
    assert np.all(f[:, 102] == 1.0)
    assert np.all(f[:, 103:] == 0.0)
    fe = oracle.nrc_features(q, BOX, emulate=True)
    # BF16 keeps 8 significant bits (|x - bf16(x)| <= 2^-9 |x|); the float32
    # position scaling moves the phase of the 2^11 pi term by up to ~8e-4.
    assert np.all(np.abs(fe - f) <= np.abs(f) * 2.0 ** -8 + 1e-3)


def test_gradient_matches_finite_differences():
    q = nrc_queries(48, seed=5)
    t = nrc_smooth_targets(q)
    w = nrc_init_params(seed=2)
    g, loss = oracle.nrc_gradient(w, q, t, BOX)
    assert np.isfinite(loss) and loss > 0
    assert np.all(g[20480 + 3 * 64:] == 0.0)
    p0 = oracle.nrc_forward(w, q, BOX)
    rng = np.random.default_rng(7)
    idx = np.concatenate([rng.integers(0, 8192, 8), rng.integers(8192, 20480, 12), rng.integers(20480, 20672, 8)])
    h = 1e-4
    l0 = oracle.nrc_loss(w, q, t, BOX, den_pred=p0)
    checked = 0
    for i in idx:
        wp = w.copy()
        wm = w.copy()
        wp[i] += h
        wm[i] -= h
        # the loss's denominator is held at the unperturbed prediction
        lp = oracle.nrc_loss(wp, q, t, BOX, den_pred=p0)
        lm = oracle.nrc_loss(wm, q, t, BOX, den_pred=p0)
        up = (lp - l0) / (float(wp[i]) - float(w[i]))
        dn = (l0 - lm) / (float(w[i]) - float(wm[i]))
        if abs(up - dn) > 0.05 * max(abs(up), abs(dn)) + 1e-6:
            continue  # a ReLU kink inside [w - h, w + h]: the derivative is one-sided there
        fd = (lp - lm) / (float(wp[i]) - float(wm[i]))
        assert abs(fd - g[i]) <= 1e-3 * abs(g[i]) + 1e-7, (int(i), fd, g[i])
        checked += 1
    assert checked >= 0.8 * idx.size


def test_emulated_gradient_close_to_float64():
    q = nrc_queries(2048, seed=11)
    t = nrc_smooth_targets(q)
    w = nrc_init_params(seed=3)
    g64, l64 = oracle.nrc_gradient(w, q, t, BOX)
    gbf, lbf = oracle.nrc_gradient(w, q, t, BOX, emulate=True)
    assert abs(lbf - l64) <= 0.05 * l64
    cos = float(np.dot(g64, gbf) / (np.linalg.norm(g64) * np.linalg.norm(gbf)))
    assert cos > 0.99


def test_first_adam_step_is_signed_learning_rate():
    w = nrc_init_params(seed=4)
    g = np.random.default_rng(1).normal(size=w.size).astype(np.float32)
    g[20480 + 3 * 64:] = 0.0
    z = np.zeros_like(w)
    w1, m1, v1 = oracle.nrc_adam(w, z, z, g, 1, lr=1e-2)
    # |g| / (|g| + eps) differs from 1 by eps / |g|
    np.testing.assert_allclose(w - w1, 1e-2 * np.sign(g), rtol=1e-3, atol=1e-7)
    assert np.all(w1[20480 + 3 * 64:] == w[20480 + 3 * 64:])
