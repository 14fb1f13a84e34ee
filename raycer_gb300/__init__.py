"""raycer_gb300 — GB300 (sm_103a) path-tracing / ray-casting hot path of raycer.

The compute runs in hand-written CUDA kernels behind the C ABI of
``include/raycer_gb300.h`` (library ``raycer_gb300/lib/libraycer_gb300.so``).
This package is the Python host side: scene generators, the ctypes binding,
and a mirror of the reference's Tracer / CLTracer / Film / TracerState API.
"""

from .scenes import SceneDesc, Material, CameraDesc, room_scene, heightfield_scene  # noqa: F401

__all__ = ["SceneDesc", "Material", "CameraDesc", "room_scene", "heightfield_scene", "CudaTracer", "Film",
           "TracerState", "Tracer", "TracerType", "RaycerError"]


def __getattr__(name):
    # The tracer API loads the native library on first use (fails loudly if absent).
    if name in ("CudaTracer", "Film", "TracerState", "Tracer", "TracerType", "RaycerError"):
        from . import tracer
        return getattr(tracer, name)
    raise AttributeError(name)
