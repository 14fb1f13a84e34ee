"""CPU oracle for the raycer hot path — test infrastructure only.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg use this package, and only as the checker / the timed CPU baseline; the
product (``raycer_gb300``) never imports it.

Two libraries:
* ``oracle/lib/liboracle.so`` (built from oracle/*.cpp, everywhere):
  ``Oracle64`` — float64 restatement of the reference's CPU path;
  ``Oracle32`` — float32 twin of the device kernels (bit-exact checker).
* ``oracle/_ref/libraycer_ref.so`` — the reference's own code compiled from its
  sources (oracle/Makefile.ref); available only where those sources are.
  ``RefScene`` drives it.
"""

from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ORACLE_LIB = HERE / "lib" / "liboracle.so"
REF_LIB = HERE / "_ref" / "libraycer_ref.so"
REF_FAST_LIB = HERE / "_ref" / "libraycer_ref_fast.so"

P = C.c_void_p
i32, i64, u32, u64, f32, f64 = C.c_int32, C.c_int64, C.c_uint32, C.c_uint64, C.c_float, C.c_double


def _ptr(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)


def _setup(lib: C.CDLL, protos: dict) -> C.CDLL:
    for name, (res, args) in protos.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


_ORACLE_PROTOS = {
    "or_scene_set_ior": (None, [P, P, i32]),
    "or32_filter_weight": (None, [C.c_int, i64, P, P, P]),
    "or64_filter_weight": (None, [C.c_int, i64, P, P, P]),
    "or32_filter_exp": (None, [i64, P, P]),
    "or_nrc_features": (None, [P, i64, P, P, C.c_int, P]),
    "or_nrc_forward": (None, [P, P, i64, P, P, C.c_int, P]),
    "or_nrc_loss": (f64, [P, P, P, i64, P, P, C.c_int, P]),
    "or_nrc_gradient": (f64, [P, P, P, i64, P, P, C.c_int, P]),
    "or_nrc_adam": (None, [P, P, P, P, i64, f32, f32, f32, f32]),
    "or_scene_new": (P, [P, P, i64, P, P, P, i32, u32, C.c_int]),
    "or_scene_set_bvh": (None, [P, i64, P, P, P, P, P]),
    "or_scene_free": (None, [P]),
    "or_bvh_node_count": (i64, [P]),
    "or_bvh_nodes": (None, [P, P, P, P, P, P]),
    "or_frames": (None, [P, P]),
    "or64_intersect": (None, [P, i64, P, C.c_int, P, P, P, P, C.c_int]),
    "or64_tri": (C.c_int, [P, i64, P, C.POINTER(f64), C.POINTER(f64), C.POINTER(f64)]),
    "or64_raycast": (f64, [P, P, u64, u64, u64, P, f64, P, P, P, C.c_int, C.POINTER(u64)]),
    "or64_render_path": (f64, [P, P, u64, u64, u64, u64, u64, u64, C.c_int, f64, f64, f64, u32, C.c_int, P,
                               C.POINTER(u64), C.c_int]),
    "or64_tonemap": (None, [i64, P, f64, f64, C.c_int, C.c_int, P]),
    "or64_fastpow": (f64, [f64, f64]),
    "or32_cast": (None, [P, i64, P, C.c_int, C.c_int, P, P, P, P, P, C.c_int]),
    "or32_raycast": (None, [P, P, u64, u64, u64, P, f32, C.c_int, P, P, C.c_int]),
    "or32_camera_rays": (None, [P, u64, u64, u64, P]),
    "or32_render_path": (None, [P, P, u64, u64, u64, C.c_int, C.c_int, C.c_int, f32, f32, f32, C.c_int, C.c_int,
                                C.c_int, u64, u32, P, P, C.c_int, C.c_int]),
    "or32_sincos_turn": (None, [i64, P, P, P]),
    "or64_cmj": (None, [u64, u64, u64, u64, f64, f64, P]),
    "or32_cmj_permute": (u64, [u64, u64, u64]),
}

_REF_PROTOS = {
    "ref_scene_new": (P, []),
    "ref_scene_free": (None, [P]),
    "ref_scene_add_triangles": (None, [P, i64, P, P, u64]),
    "ref_scene_add_material": (None, [P, u64, P, P, C.c_int, C.c_int]),
    "ref_scene_add_directional_light": (None, [P, P, P, f64]),
    "ref_scene_set_ambient": (None, [P, P, f64]),
    "ref_scene_set_camera": (None, [P, P, f64, f64, f64, f64]),
    "ref_scene_set_general": (None, [P, C.c_int, u64, u64, u64, C.c_int, C.c_int, f64]),
    "ref_scene_set_tonemapper": (None, [P, C.c_int, C.c_int, C.c_int, f64, f64]),
    "ref_scene_initialize": (C.c_int, [P, u64]),
    "ref_last_error": (C.c_char_p, [P]),
    "ref_bvh_node_count": (i64, [P]),
    "ref_bvh_nodes": (None, [P, P, P, P, P]),
    "ref_bvh_ordered_ids": (None, [P, P]),
    "ref_triangle_frame": (None, [P, i64, P]),
    "ref_camera_state": (None, [P, u64, u64, P]),
    "ref_camera_rays": (None, [P, i64, P, P]),
    "ref_intersect": (None, [P, i64, P, C.c_int, u64, P, P, C.c_int]),
    "ref_render": (C.c_int, [P, u64, u64, C.c_int, P, P, C.POINTER(u64), C.POINTER(f64)]),
    "ref_tonemap_reinhard": (None, [i64, P, f64, f64, C.c_int, C.c_int, P]),
    "ref_fastpow": (f64, [f64, f64]),
    "ref_value_noise": (None, [u32, i64, P, u64, f64, f64, P]),
    "ref_cmj_pattern": (None, [u64, u64, u32, P, P]),
    "ref_filter_weight": (None, [C.c_int, i64, P, P, P]),
    "ref_scene_add_instanced_mesh": (None, [P, i64, P, P, u64, u64, i64, P, u64]),
}

_oracle = None
_ref = {}


def oracle_lib() -> C.CDLL:
    global _oracle
    if _oracle is None:
        if not ORACLE_LIB.exists():
            raise ImportError(f"oracle library missing at {ORACLE_LIB}; run the build")
        _oracle = _setup(C.CDLL(str(ORACLE_LIB), mode=os.RTLD_NOW | os.RTLD_LOCAL), _ORACLE_PROTOS)
    return _oracle


def ref_available(fast: bool = False) -> bool:
    return (REF_FAST_LIB if fast else REF_LIB).exists()


def ref_lib(fast: bool = False) -> C.CDLL:
    key = "fast" if fast else "par"
    if key not in _ref:
        path = REF_FAST_LIB if fast else REF_LIB
        if not path.exists():
            raise ImportError(f"reference build missing at {path}")
        _ref[key] = _setup(C.CDLL(str(path), mode=os.RTLD_NOW | os.RTLD_LOCAL), _REF_PROTOS)
    return _ref[key]


NODE_DTYPE = np.dtype([("aabb_min", "<f8", 3), ("aabb_max", "<f8", 3), ("right_offset", "<i8"),
                       ("start_offset", "<u8"), ("primitive_count", "<u8")])


def _mat_arrays(materials):
    m = len(materials)
    diffuse = np.array([mm.diffuse for mm in materials], np.float32).reshape(m, 3)
    emit = np.array([mm.emittance for mm in materials], np.float32).reshape(m, 3)
    flags = np.array([(1 if mm.is_emissive else 0) | (2 if mm.non_shadowing else 0) | (4 if mm.invert_normal else 0)
                      | (8 if getattr(mm, "dielectric", False) else 0) for mm in materials], np.int32)
    return diffuse, emit, flags


class Oracle:
    """float64 restatement + float32 twin over one scene (see module docstring)."""

    def __init__(self, scene, build: bool = True, prebuilt=None):
        self.lib = oracle_lib()
        self.scene = scene
        v = np.ascontiguousarray(scene.vertices, np.float64)
        m = np.ascontiguousarray(scene.material_index, np.uint32)
        d, e, f = _mat_arrays(scene.materials)
        self._keep = (v, m, d, e, f)
        self.h = self.lib.or_scene_new(_ptr(v), _ptr(m), v.shape[0], _ptr(d), _ptr(e), _ptr(f), len(scene.materials),
                                       int(scene.max_leaf_size), 1 if (build and prebuilt is None) else 0)
        ior = np.array([float(getattr(mm, "ior", 0.0)) for mm in scene.materials], np.float32)
        self.lib.or_scene_set_ior(self.h, _ptr(ior), len(scene.materials))
        if prebuilt is not None:
            self.set_bvh(*prebuilt)

    def close(self):
        if self.h:
            self.lib.or_scene_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_bvh(self, nodes: np.ndarray, order: np.ndarray) -> None:
        nodes = np.ascontiguousarray(nodes, NODE_DTYPE)
        aabb = np.ascontiguousarray(np.concatenate([nodes["aabb_min"], nodes["aabb_max"]], axis=1))
        right = np.ascontiguousarray(nodes["right_offset"])
        start = np.ascontiguousarray(nodes["start_offset"])
        count = np.ascontiguousarray(nodes["primitive_count"])
        order = np.ascontiguousarray(order, np.uint64)
        self.lib.or_scene_set_bvh(self.h, nodes.shape[0], _ptr(aabb), _ptr(right), _ptr(start), _ptr(count),
                                  _ptr(order))

    def bvh(self) -> tuple[np.ndarray, np.ndarray]:
        n = self.lib.or_bvh_node_count(self.h)
        aabb = np.empty((n, 6), np.float64)
        right = np.empty(n, np.int64)
        start = np.empty(n, np.uint64)
        count = np.empty(n, np.uint64)
        order = np.empty(self.scene.triangle_count, np.uint64)
        self.lib.or_bvh_nodes(self.h, _ptr(aabb), _ptr(right), _ptr(start), _ptr(count), _ptr(order))
        nodes = np.empty(n, NODE_DTYPE)
        nodes["aabb_min"] = aabb[:, :3]
        nodes["aabb_max"] = aabb[:, 3:]
        nodes["right_offset"] = right
        nodes["start_offset"] = start
        nodes["primitive_count"] = count
        return nodes, order

    def frames(self) -> np.ndarray:
        out = np.empty((self.scene.triangle_count, 9), np.float64)
        self.lib.or_frames(self.h, _ptr(out))
        return out

    # float64 restatement
    def intersect64(self, rays6: np.ndarray, shadow: bool = False, threads: int = 0):
        r = np.ascontiguousarray(rays6, np.float64).reshape(-1, 6)
        n = r.shape[0]
        prim = np.empty(n, np.int64)
        t = np.empty(n, np.float64)
        u = np.empty(n, np.float64)
        v = np.empty(n, np.float64)
        self.lib.or64_intersect(self.h, n, _ptr(r), int(shadow), _ptr(prim), _ptr(t), _ptr(u), _ptr(v), threads)
        return prim, t, u, v

    def tri64(self, caller: int, ray6) -> tuple[bool, float, float, float]:
        r = np.ascontiguousarray(ray6, np.float64)
        t, u, v = f64(), f64(), f64()
        ok = self.lib.or64_tri(self.h, int(caller), _ptr(r), C.byref(t), C.byref(u), C.byref(v))
        return bool(ok), t.value, u.value, v.value

    def raycast64(self, cam64: np.ndarray, width: int, count: int, dir_to_light, offset: float = 1e-5,
                  threads: int = 0, pixel_start: int = 0):
        cam = np.ascontiguousarray(cam64, np.float64)
        prim = np.empty(count, np.int64)
        t = np.empty(count, np.float64)
        occ = np.empty(count, np.int64)
        L = None if dir_to_light is None else np.ascontiguousarray(dir_to_light, np.float64)
        rays = u64(0)
        sec = self.lib.or64_raycast(self.h, _ptr(cam), width, pixel_start, count,
                                    None if L is None else _ptr(L), offset, _ptr(prim), _ptr(t), _ptr(occ),
                                    threads, C.byref(rays))
        return prim, t, occ, rays.value, sec

    def render_path64(self, cam64: np.ndarray, width: int, count: int, max_path_length: int, path_samples: int,
                      ms_sqrt: int, sampler: int = 4, radius=(0.5, 0.5), offset: float = 1e-5, seed: int = 1,
                      threads: int = 0, pixel_start: int = 0, filter_type: int = 0):
        cam = np.ascontiguousarray(cam64, np.float64)
        film = np.zeros((count, 4), np.float64)
        rays = u64(0)
        sec = self.lib.or64_render_path(self.h, _ptr(cam), width, pixel_start, count, max_path_length, path_samples,
                                        ms_sqrt, sampler, radius[0], radius[1], offset, seed, threads, _ptr(film),
                                        C.byref(rays), int(filter_type))
        return film, rays.value, sec

    # float32 twin of the device
    def cast32(self, rays: np.ndarray, any_hit: bool = False, order: int = 1, threads: int = 0):
        r = np.ascontiguousarray(rays).view(np.float32).reshape(-1, 8)
        n = r.shape[0]
        prim = np.empty(n, np.int32)
        t = np.empty(n, np.float32)
        u = np.empty(n, np.float32)
        v = np.empty(n, np.float32)
        cnt = np.zeros(4, np.uint64)
        self.lib.or32_cast(self.h, n, _ptr(r), int(any_hit), int(order), _ptr(prim), _ptr(t), _ptr(u), _ptr(v),
                           _ptr(cnt), threads)
        return prim, t, u, v, cnt

    def raycast32(self, cam: np.ndarray, width: int, count: int, dir_to_light, offset: float = 1e-5, order: int = 1,
                  threads: int = 0, pixel_start: int = 0):
        c = np.ascontiguousarray(cam, np.float32)
        out = np.empty((count, 4), np.int32)
        cnt = np.zeros(4, np.uint64)
        L = None if dir_to_light is None else np.ascontiguousarray(dir_to_light, np.float32)
        self.lib.or32_raycast(self.h, _ptr(c), width, pixel_start, count, None if L is None else _ptr(L), offset,
                              int(order), _ptr(out), _ptr(cnt), threads)
        return out, cnt

    def render_path32(self, cam: np.ndarray, width: int, count: int, n: int, P: int, sampler: int, radius,
                      offset: float, max_path_length: int, rr_depth: int, order: int, seed: int, frame: int,
                      film: np.ndarray | None = None, threads: int = 0, pixel_start: int = 0,
                      filter_type: int = 0):
        c = np.ascontiguousarray(cam, np.float32)
        f = np.zeros((count, 4), np.float32) if film is None else np.ascontiguousarray(film, np.float32).copy()
        cnt = np.zeros(4, np.uint64)
        self.lib.or32_render_path(self.h, _ptr(c), width, pixel_start, count, n, P, sampler, radius[0], radius[1],
                                  offset, max_path_length, rr_depth, order, seed, frame, _ptr(f), _ptr(cnt), threads,
                                  int(filter_type))
        return f, cnt


def camera_rays32(cam: np.ndarray, width: int, count: int, pixel_start: int = 0) -> np.ndarray:
    """Primary rays of the float32 camera (rc_ray layout, 8 floats each)."""
    c = np.ascontiguousarray(cam, np.float32)
    out = np.empty((count, 8), np.float32)
    oracle_lib().or32_camera_rays(_ptr(c), width, pixel_start, count, _ptr(out))
    return out


def tonemap64(linear_rgba: np.ndarray, key=0.18, gamma=2.2, clamp=True, apply_gamma=True) -> np.ndarray:
    lin = np.ascontiguousarray(linear_rgba, np.float32).reshape(-1, 4)
    out = np.empty_like(lin)
    oracle_lib().or64_tonemap(lin.shape[0], _ptr(lin), key, gamma, int(clamp), int(apply_gamma), _ptr(out))
    return out


class RefScene:
    """The reference's own Scene, built through oracle/_ref (where available)."""

    def __init__(self, scene, fast: bool = False, init: bool = True):
        self.lib = ref_lib(fast)
        self.scene = scene
        self.h = self.lib.ref_scene_new()
        for i, m in enumerate(scene.materials):
            d = np.array(m.diffuse, np.float64)
            e = np.array(m.emittance, np.float64)
            self.lib.ref_scene_add_material(self.h, i + 1, _ptr(d), _ptr(e), int(m.is_emissive),
                                            int(m.non_shadowing))
        if hasattr(scene, "meshes"):
            self._add_instanced(scene)
        else:
            v = np.ascontiguousarray(scene.vertices, np.float64)
            mids = np.ascontiguousarray(scene.material_index.astype(np.uint64) + 1)
            self.lib.ref_scene_add_triangles(self.h, v.shape[0], _ptr(v), _ptr(mids), 1)
        c = scene.camera
        pos = np.array(c.position, np.float64)
        self.lib.ref_scene_set_camera(self.h, _ptr(pos), c.pitch, c.yaw, c.roll, c.fov)
        if scene.light_direction is not None:
            d = np.array(scene.light_direction, np.float64)
            col = np.ones(3, np.float64)
            self.lib.ref_scene_add_directional_light(self.h, _ptr(d), _ptr(col), 1.0)
        if init:
            self.initialize()

    # Instanced scenes: mesh m's triangle j has id MESH_ID * m + 1 + j.
    MESH_ID = 10_000_000

    def _add_instanced(self, scene):
        for m, (v, mi) in enumerate(scene.meshes):
            ks = [k for k, d in enumerate(scene.instances) if d.mesh == m]
            if not ks:
                continue
            srt = np.array([[*scene.instances[k].scale, *scene.instances[k].rotate, *scene.instances[k].translate]
                            for k in ks], np.float64)
            v = np.ascontiguousarray(v, np.float64)
            mids = np.ascontiguousarray(np.asarray(mi).astype(np.uint64) + 1)
            self.lib.ref_scene_add_instanced_mesh(self.h, v.shape[0], _ptr(v), _ptr(mids), self.MESH_ID * m + 1,
                                                  900_000_000 + m, len(ks), _ptr(srt), 950_000_000 + 10_000 * m)

    def initialize(self):
        if self.lib.ref_scene_initialize(self.h, int(self.scene.max_leaf_size)) != 0:
            raise RuntimeError(self.lib.ref_last_error(self.h).decode())

    def close(self):
        if self.h:
            self.lib.ref_scene_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_general(self, tracer: int, max_path_length: int, path_samples: int, ms_sqrt: int, sampler: int = 4,
                    filt: int = 0, offset: float = 1e-5):
        self.lib.ref_scene_set_general(self.h, tracer, max_path_length, path_samples, ms_sqrt, sampler, filt, offset)

    def set_tonemapper(self, typ: int = 3, apply_gamma=True, clamp=True, gamma=2.2, key=0.18):
        self.lib.ref_scene_set_tonemapper(self.h, typ, int(apply_gamma), int(clamp), gamma, key)

    def bvh(self):
        n = self.lib.ref_bvh_node_count(self.h)
        aabb = np.empty((n, 6), np.float64)
        right = np.empty(n, np.int64)
        start = np.empty(n, np.uint64)
        count = np.empty(n, np.uint64)
        ids = np.empty(self.scene.triangle_count, np.uint64)
        self.lib.ref_bvh_nodes(self.h, _ptr(aabb), _ptr(right), _ptr(start), _ptr(count))
        self.lib.ref_bvh_ordered_ids(self.h, _ptr(ids))
        nodes = np.empty(n, NODE_DTYPE)
        nodes["aabb_min"] = aabb[:, :3]
        nodes["aabb_max"] = aabb[:, 3:]
        nodes["right_offset"] = right
        nodes["start_offset"] = start
        nodes["primitive_count"] = count
        return nodes, ids - 1

    def camera_state(self, width: int, height: int) -> np.ndarray:
        out = np.empty(19, np.float64)
        self.lib.ref_camera_state(self.h, width, height, _ptr(out))
        return out

    def intersect(self, rays6: np.ndarray, shadow: bool = False, threads: int = 0):
        r = np.ascontiguousarray(rays6, np.float64).reshape(-1, 6)
        n = r.shape[0]
        prim = np.empty(n, np.int64)
        t = np.empty(n, np.float64)
        self.lib.ref_intersect(self.h, n, _ptr(r), int(shadow), 1, _ptr(prim), _ptr(t), threads)
        return prim, t

    def render(self, width: int, height: int, threads: int = 0):
        lin = np.empty((width * height, 4), np.float32)
        tm = np.empty((width * height, 4), np.float32)
        rays = u64(0)
        sec = f64(0)
        if self.lib.ref_render(self.h, width, height, threads, _ptr(lin), _ptr(tm), C.byref(rays), C.byref(sec)):
            raise RuntimeError(self.lib.ref_last_error(self.h).decode())
        return lin, tm, rays.value, sec.value

    def frame(self, i: int) -> np.ndarray:
        out = np.empty(9, np.float64)
        self.lib.ref_triangle_frame(self.h, i, _ptr(out))
        return out


def camera_state64(position, pitch: float, yaw: float, roll: float, fov: float, width: int,
                   height: int) -> np.ndarray:
    """The perspective camera's float64 state after a non-interactive
    Camera::update (Camera.cpp:48-284) and Camera::setImagePlaneSize
    (Camera.cpp:29-34), in the layout of ``RefScene.camera_state``: position,
    forward, right, up, image-plane centre (3 each), aspect = height / width,
    width - 1, height - 1, image-plane distance.

    forward = EulerAngle::getDirection (EulerAngle.cpp:77-87) of the pitch
    clamped to [-89, 89] and both angles wrapped into [-180, 180]
    (EulerAngle::clampPitch / normalize); right, up = ONB::fromNormal
    (ONB.cpp:32-39) with Vector3::ALMOST_UP (Vector3.cpp:15); the image-plane
    centre uses the direction of the angles before clamping, at distance
    0.5 / tan(fov / 2), fov horizontal in [1, 180] degrees. Roll is unused by
    the basis, as in the reference."""
    import math

    d2r = math.pi / 180.0

    def unit(a):
        n = math.sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2])
        return (a[0] / n, a[1] / n, a[2] / n)

    def cross(a, b):
        return (a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0])

    def direction(p, y):
        return unit((-math.sin(y * d2r) * math.cos(p * d2r), math.sin(p * d2r), -math.cos(y * d2r) * math.cos(p * d2r)))

    def wrap(a):
        while abs(a) > 180.0:
            a += -360.0 if a > 0.0 else 360.0
        return a

    pos = tuple(float(x) for x in position)
    fwd0 = direction(float(pitch), float(yaw))
    p = wrap(min(89.0, max(-89.0, float(pitch))))
    y = wrap(float(yaw))
    f = max(1.0, min(float(fov), 180.0))
    ipd = 0.5 / math.tan((f / 2.0) * d2r)
    w = direction(p, y)
    u = unit(cross(w, (0.0001, 1.0, 0.0001)))
    v = unit(cross(u, w))
    centre = tuple(pos[k] + fwd0[k] * ipd for k in range(3))
    return np.array([*pos, *w, *u, *v, *centre, float(height) / float(width), float(width - 1), float(height - 1),
                     ipd], np.float64)


def camera64_of(scene) -> np.ndarray:
    """``raycast64`` camera input of a scene description (float64 throughout)."""
    c = scene.camera
    return cam64_from_state(camera_state64(c.position, c.pitch, c.yaw, c.roll, c.fov, scene.width, scene.height))


def cam64_from_state(state19: np.ndarray) -> np.ndarray:
    """Camera64 input (pos, right, up, centre, aspect, ipw, iph) from the reference camera state."""
    s = np.asarray(state19, np.float64)
    return np.concatenate([s[0:3], s[6:9], s[9:12], s[12:15], s[15:18]])


# ---------------------------------------------------------------------------
# Radiance-cache network (oracle/nrc64.cpp). `box` = (lo[3], inv[3]).

def _box(box):
    lo = np.ascontiguousarray(box[0], np.float32)
    inv = np.ascontiguousarray(box[1], np.float32)
    return lo, inv


def nrc_features(queries: np.ndarray, box, emulate: bool = False) -> np.ndarray:
    q = np.ascontiguousarray(queries, np.float32)
    lo, inv = _box(box)
    out = np.empty((q.shape[0], 128), np.float64)
    oracle_lib().or_nrc_features(_ptr(q), q.shape[0], _ptr(lo), _ptr(inv), int(emulate), _ptr(out))
    return out


def nrc_forward(params: np.ndarray, queries: np.ndarray, box, emulate: bool = False) -> np.ndarray:
    w = np.ascontiguousarray(params, np.float32)
    q = np.ascontiguousarray(queries, np.float32)
    lo, inv = _box(box)
    out = np.empty((q.shape[0], 3), np.float64)
    oracle_lib().or_nrc_forward(_ptr(w), _ptr(q), q.shape[0], _ptr(lo), _ptr(inv), int(emulate), _ptr(out))
    return out


def nrc_loss(params, queries, targets, box, emulate: bool = False, den_pred=None) -> float:
    w = np.ascontiguousarray(params, np.float32)
    q = np.ascontiguousarray(queries, np.float32)
    t = np.ascontiguousarray(targets, np.float32)
    lo, inv = _box(box)
    d = None if den_pred is None else np.ascontiguousarray(den_pred, np.float64)
    return oracle_lib().or_nrc_loss(_ptr(w), _ptr(q), _ptr(t), q.shape[0], _ptr(lo), _ptr(inv), int(emulate),
                                    None if d is None else _ptr(d))


def nrc_gradient(params, queries, targets, box, emulate: bool = False) -> tuple[np.ndarray, float]:
    w = np.ascontiguousarray(params, np.float32)
    q = np.ascontiguousarray(queries, np.float32)
    t = np.ascontiguousarray(targets, np.float32)
    lo, inv = _box(box)
    g = np.empty(w.size, np.float64)
    loss = oracle_lib().or_nrc_gradient(_ptr(w), _ptr(q), _ptr(t), q.shape[0], _ptr(lo), _ptr(inv), int(emulate),
                                        _ptr(g))
    return g, loss


def nrc_adam(master, m, v, grad, t: int, lr=1e-2, b1=0.9, b2=0.99, eps=1e-8):
    """One float32 Adam step; returns (master, m, v) updated copies."""
    w = np.array(master, np.float32)
    mm = np.array(m, np.float32)
    vv = np.array(v, np.float32)
    g = np.ascontiguousarray(grad, np.float32)
    oracle_lib().or_nrc_adam(_ptr(w), _ptr(mm), _ptr(vv), _ptr(g), int(t), lr, b1, b2, eps)
    return w, mm, vv


# ---------------------------------------------------------------------------
# Film filters: one axis's weight at offsets x.

def filter_weight32(filter_type: int, x) -> tuple[np.ndarray, float]:
    xs = np.ascontiguousarray(x, np.float32)
    out = np.empty_like(xs)
    r = f32(0)
    oracle_lib().or32_filter_weight(int(filter_type), xs.size, _ptr(xs), _ptr(out), C.byref(r))
    return out, r.value


def filter_weight64(filter_type: int, x) -> tuple[np.ndarray, float]:
    xs = np.ascontiguousarray(x, np.float64)
    out = np.empty_like(xs)
    r = f64(0)
    oracle_lib().or64_filter_weight(int(filter_type), xs.size, _ptr(xs), _ptr(out), C.byref(r))
    return out, r.value


def filter_exp32(t) -> np.ndarray:
    ts = np.ascontiguousarray(t, np.float32)
    out = np.empty_like(ts)
    oracle_lib().or32_filter_exp(ts.size, _ptr(ts), _ptr(out))
    return out


def ref_filter_weight(filter_type: int, x) -> tuple[np.ndarray, float]:
    """The reference's own Filter::getWeightX (needs oracle/_ref)."""
    xs = np.ascontiguousarray(x, np.float64)
    out = np.empty_like(xs)
    r = f64(0)
    ref_lib().ref_filter_weight(int(filter_type), xs.size, _ptr(xs), _ptr(out), C.byref(r))
    return out, r.value
