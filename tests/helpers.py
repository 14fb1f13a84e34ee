"""Shared helpers of the test suite."""

from __future__ import annotations

import numpy as np

from raycer_gb300 import scenes


def camera_floats(cam) -> np.ndarray:
    """rc_camera record -> 18 float32 (the oracle's camera layout)."""
    return np.array(list(cam.position) + list(cam.forward) + list(cam.right) + list(cam.up) +
                    list(cam.image_plane_center) + [cam.aspect_ratio, cam.image_plane_width, cam.image_plane_height],
                    np.float32)


def small_heightfield(width=160, height=90):
    return scenes.heightfield_scene(nx=96, nz=48, width=width, height=height)


def small_room(width=64, height=48, clutter=300):
    return scenes.room_scene(clutter=clutter, width=width, height=height)


def nrc_queries(n: int, seed: int = 0, lo=(-10.0, -2.0, -5.0), hi=(10.0, 3.0, 5.0)) -> np.ndarray:
    """Random cache queries (n, 12): position in the box, unit direction and
    normal, albedo U(0.1, 0.9)."""
    rng = np.random.default_rng(seed)
    lo = np.asarray(lo, np.float64)
    hi = np.asarray(hi, np.float64)
    pos = lo + (hi - lo) * rng.random((n, 3))
    w = rng.normal(size=(n, 3))
    w /= np.linalg.norm(w, axis=1, keepdims=True)
    nrm = rng.normal(size=(n, 3))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    rho = 0.1 + 0.8 * rng.random((n, 3))
    return np.concatenate([pos, w, nrm, rho], axis=1).astype(np.float32)


def nrc_box(lo=(-10.0, -2.0, -5.0), hi=(10.0, 3.0, 5.0)):
    """(lo, inv) of an encoding box, as the kernels compute them (float32)."""
    lo = np.asarray(lo, np.float64)
    hi = np.asarray(hi, np.float64)
    return lo.astype(np.float32), (1.0 / (hi - lo)).astype(np.float32)


def nrc_init_params(seed: int = 1) -> np.ndarray:
    """He-uniform weights in the packed layout (padding rows of the output layer zero)."""
    rng = np.random.default_rng(seed)
    w = np.zeros(20992, np.float32)
    for off, rows, cols in ((0, 64, 128), (8192, 64, 64), (12288, 64, 64), (16384, 64, 64), (20480, 3, 64)):
        lim = np.sqrt(6.0 / cols)
        w[off:off + rows * cols] = rng.uniform(-lim, lim, rows * cols).astype(np.float32)
    return w


def nrc_smooth_targets(q: np.ndarray) -> np.ndarray:
    """A smooth positive radiance field over queries (for training tests)."""
    x, y, z = q[:, 0], q[:, 1], q[:, 2]
    nz = q[:, 8]
    r = 0.6 + 0.3 * np.sin(0.5 * x) * np.cos(0.7 * z) + 0.1 * nz
    g = 0.5 + 0.2 * np.cos(0.3 * x + 0.2 * y)
    b = 0.4 + 0.25 * np.sin(0.4 * z) * q[:, 9]
    return np.stack([r, g, b], axis=1).astype(np.float32)
