"""Batched path tracing over the C ABI (rc_batch_*): many independent scenes of
uneven size rendered as one CUDA-graph launch per frame."""

from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .scenes import SceneDesc
from .tracer import RaycerError, camera_record, general_record, materials_array, tonemapper_record


class Batch:
    def __init__(self, device: int = 0):
        self._lib = N.lib()
        self._h = C.c_void_p()
        st = self._lib.rc_batch_create(C.byref(self._h), int(device))
        if st != N.RC_OK:
            raise RaycerError(st, "rc_batch_create failed")
        self.scenes: list[SceneDesc] = []

    def _check(self, st: int, what: str) -> None:
        if st != N.RC_OK:
            msg = self._lib.rc_batch_last_error(self._h)
            raise RaycerError(st, f"{what}: {msg.decode() if msg else ''}")

    def close(self) -> None:
        if self._h:
            self._lib.rc_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_scene(self, scene: SceneDesc, seed: int = 1) -> int:
        v = np.ascontiguousarray(scene.vertices, np.float64)
        m = np.ascontiguousarray(scene.material_index, np.uint32)
        mats = materials_array(scene.materials)
        cam = camera_record(scene)
        g = general_record(scene, seed)
        idx = C.c_int32(-1)
        self._check(self._lib.rc_batch_add_scene(self._h, C.c_void_p(v.ctypes.data), C.c_void_p(m.ctypes.data),
                                                 v.shape[0], mats, len(scene.materials), int(scene.max_leaf_size),
                                                 C.byref(cam), C.byref(g), scene.width, scene.height, C.byref(idx)),
                    "add_scene")
        self.scenes.append(scene)
        return idx.value

    def autotune(self, budget_ms: float = 2000.0) -> dict:
        self._check(self._lib.rc_batch_autotune(self._h, float(budget_ms)), "autotune")
        return self.tuning()

    def tuning(self) -> dict:
        t = N.rc_batch_tuning()
        self._check(self._lib.rc_batch_get_tuning(self._h, C.byref(t)), "tuning")
        return {k: list(getattr(t, k)) for k, _ in N.rc_batch_tuning._fields_}

    def render(self) -> np.ndarray:
        """One frame of every scene; returns each scene's completion time (ms from the launch's start)."""
        done = np.zeros(len(self.scenes), np.float64)
        self._check(self._lib.rc_batch_render(self._h, C.c_void_p(done.ctypes.data)), "render")
        return done

    def clear(self) -> None:
        self._check(self._lib.rc_batch_clear(self._h), "clear")

    def read_film(self, i: int) -> np.ndarray:
        sc = self.scenes[i]
        out = np.empty((sc.width * sc.height, 4), np.float32)
        self._check(self._lib.rc_batch_read_film(self._h, int(i), C.c_void_p(out.ctypes.data)), "read_film")
        return out

    def resolve(self, i: int) -> np.ndarray:
        sc = self.scenes[i]
        out = np.empty((sc.width * sc.height, 4), np.float32)
        tm = tonemapper_record(sc)
        self._check(self._lib.rc_batch_resolve(self._h, int(i), C.byref(tm), C.c_void_p(out.ctypes.data)),
                    "resolve")
        return out.reshape(sc.height, sc.width, 4)

    def stats(self) -> dict:
        s = N.rc_batch_stats()
        self._check(self._lib.rc_batch_get_stats(self._h, C.byref(s)), "stats")
        return {k: getattr(s, k) for k, _ in N.rc_batch_stats._fields_}
