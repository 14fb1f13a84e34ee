"""Neural radiance cache and float64 ground-truth helpers over the C ABI.

``RadianceCache`` drives the rc_nrc_* entry points of a ``CudaTracer``:
configuration, weights, host-batch inference / gradients / Adam steps (what
the gradient and training tests call) and the statistics of the cache work
inside PATH renders. ``GroundTruth`` accumulates films in float64 on the
device (rc_film_accumulate_f64) and measures a film's display-space RMSE
against it (rc_film_rmse_f64).

A query is 12 floats: position, direction (unit, toward where the path came
from), normal, diffuse albedo.
"""

from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .tracer import CudaTracer, RaycerError

PARAMS = N.RC_NRC_PARAMS
QUERY_FLOATS = N.RC_NRC_QUERY_FLOATS
INPUTS = N.RC_NRC_INPUTS
# Offsets of the packed [out][in] weight matrices.
LAYERS = ((0, 64, 128), (8192, 64, 64), (12288, 64, 64), (16384, 64, 64), (20480, 8, 64))


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def unpack_layers(params: np.ndarray) -> list[np.ndarray]:
    """The five [out][in] weight matrices of a packed parameter vector."""
    return [params[o:o + r * c].reshape(r, c) for o, r, c in LAYERS]


class RadianceCache:
    def __init__(self, tracer: CudaTracer, **config):
        self.tracer = tracer
        self._lib = tracer._lib
        self._h = tracer._h
        cfg = N.rc_nrc_config()
        self._lib.rc_nrc_defaults(C.byref(cfg))
        for k, v in config.items():
            if k in ("box_min", "box_max"):
                getattr(cfg, k)[:] = [float(x) for x in v]
            elif not hasattr(cfg, k):
                raise KeyError(f"unknown radiance-cache setting {k!r}")
            else:
                setattr(cfg, k, v)
        self.config = cfg
        self._check(self._lib.rc_nrc_configure(self._h, C.byref(cfg)), "nrc_configure")

    def _check(self, st: int, what: str) -> None:
        if st != N.RC_OK:
            msg = self._lib.rc_last_error(self._h)
            raise RaycerError(st, f"{what}: {msg.decode() if msg else ''}")

    def set_enabled(self, enabled: bool) -> None:
        self._check(self._lib.rc_nrc_set_enabled(self._h, int(bool(enabled))), "nrc_set_enabled")

    @property
    def params(self) -> np.ndarray:
        out = np.empty(PARAMS, np.float32)
        self._check(self._lib.rc_nrc_get_params(self._h, _ptr(out), PARAMS), "nrc_get_params")
        return out

    @params.setter
    def params(self, value: np.ndarray) -> None:
        v = np.ascontiguousarray(value, np.float32)
        self._check(self._lib.rc_nrc_set_params(self._h, _ptr(v), v.size), "nrc_set_params")

    @staticmethod
    def _queries(q: np.ndarray) -> np.ndarray:
        q = np.ascontiguousarray(q, np.float32)
        if q.ndim != 2 or q.shape[1] != QUERY_FLOATS:
            raise ValueError("queries must be (n, 12)")
        return q

    def infer(self, queries: np.ndarray) -> np.ndarray:
        q = self._queries(queries)
        out = np.empty((q.shape[0], 3), np.float32)
        self._check(self._lib.rc_nrc_infer(self._h, _ptr(q), q.shape[0], _ptr(out)), "nrc_infer")
        return out

    def encode(self, queries: np.ndarray) -> np.ndarray:
        q = self._queries(queries)
        out = np.empty((q.shape[0], INPUTS), np.float32)
        self._check(self._lib.rc_nrc_encode(self._h, _ptr(q), q.shape[0], _ptr(out)), "nrc_encode")
        return out

    def gradient(self, queries: np.ndarray, targets: np.ndarray) -> tuple[np.ndarray, float]:
        q = self._queries(queries)
        t = np.ascontiguousarray(targets, np.float32).reshape(-1, 3)
        g = np.empty(PARAMS, np.float32)
        loss = np.zeros(1, np.float32)
        self._check(self._lib.rc_nrc_gradient(self._h, _ptr(q), _ptr(t), q.shape[0], _ptr(g), _ptr(loss)),
                    "nrc_gradient")
        return g, float(loss[0])

    def train(self, queries: np.ndarray, targets: np.ndarray, steps: int = 1) -> np.ndarray:
        q = self._queries(queries)
        t = np.ascontiguousarray(targets, np.float32).reshape(-1, 3)
        losses = np.empty(int(steps), np.float32)
        self._check(self._lib.rc_nrc_train(self._h, _ptr(q), _ptr(t), q.shape[0], int(steps), _ptr(losses)),
                    "nrc_train")
        return losses

    def samples(self, capacity: int | None = None) -> np.ndarray:
        """Training samples of the last render pass: (n, 16) = query, target rgb,
        tag (as float32 bits: vertex index << 24 | training-path index)."""
        count = C.c_int64(0)
        self._check(self._lib.rc_nrc_read_samples(self._h, None, 0, C.byref(count)), "nrc_read_samples")
        n = count.value if capacity is None else min(int(capacity), count.value)
        out = np.empty((n, 16), np.float32)
        if n:
            self._check(self._lib.rc_nrc_read_samples(self._h, _ptr(out), n, C.byref(count)), "nrc_read_samples")
        return out

    @staticmethod
    def sample_tags(samples: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
        """(vertex index, training-path index) of each sample."""
        bits = np.ascontiguousarray(samples[:, 15]).view(np.uint32)
        return (bits >> 24).astype(np.int64), (bits & 0xFFFFFF).astype(np.int64)

    def stats(self) -> dict:
        s = N.rc_nrc_stats()
        self._check(self._lib.rc_nrc_get_stats(self._h, C.byref(s)), "nrc_get_stats")
        return {k: getattr(s, k) for k, _ in N.rc_nrc_stats._fields_ if k != "reserved"}


class GroundTruth:
    """A float64 film on the device: sum of the tracer's films (r, g, b, weight)."""

    def __init__(self, tracer: CudaTracer):
        import torch  # device memory only

        self.tracer = tracer
        self.pixels = tracer.imageWidth * tracer.imageHeight
        self.buf = torch.zeros((self.pixels, 4), dtype=torch.float64, device="cuda")
        self.frames = 0

    def add_film(self, clear_film: bool = True) -> None:
        t = self.tracer
        t._check(t._lib.rc_film_accumulate_f64(t._h, C.c_void_p(self.buf.data_ptr()), int(bool(clear_film))),
                 "film_accumulate_f64")
        self.frames += 1

    def rmse(self) -> float:
        """Display-space RMSE of the tracer's current film against this truth."""
        t = self.tracer
        out = C.c_double(0.0)
        t._check(t._lib.rc_film_rmse_f64(t._h, C.c_void_p(self.buf.data_ptr()), C.byref(out)), "film_rmse_f64")
        return float(out.value)

    def numpy(self) -> np.ndarray:
        return self.buf.cpu().numpy()
