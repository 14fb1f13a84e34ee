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
