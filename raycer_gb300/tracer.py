"""Python host mirror of the reference's tracer interface over the C ABI.

* ``CudaTracer`` has the method shape of the reference's OpenCL tracer
  (src/OpenCL/CLTracer.h:23-41): initializeKernels / releaseKernels,
  initializeImageBuffers / releaseImageBuffers, initializeBuffers /
  releaseBuffers, run, downloadImage, clear. Errors raise RuntimeError, as
  CLManager::checkError does (src/OpenCL/CLManager.cpp:73-101).
* ``TracerState`` mirrors src/Raytracing/Tracers/TracerState.h:13-26.
* ``Film`` mirrors src/Rendering/Film.h:23-52 (per-pixel sum of weighted
  colours and sum of weights; generateToneMappedImage).
* ``Tracer.getTracer(TracerType)`` mirrors Tracer::getTracer
  (Tracer.h:32-38); its ``run(state, interrupted)`` renders on the GPU and
  adds the weighted samples to ``state.film`` like the CPU tracer does.

Scenes are ``raycer_gb300.scenes.SceneDesc`` records (triangles, materials,
camera, settings): the parts of the reference's Scene the hot path reads.
"""

from __future__ import annotations

import ctypes as C
import threading
from enum import IntEnum

import numpy as np

from . import _native as N
from .scenes import SceneDesc


class TracerType(IntEnum):
    RAY = N.RC_TRACER_RAY
    PATH = N.RC_TRACER_PATH


class RaycerError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{message} ({N.STATUS_NAMES.get(status, status)})")
        self.status = status


CAST_DTYPE = np.dtype([("prim", "<i4"), ("t", "<f4"), ("occluder", "<i4"), ("flags", "<i4")])
HIT_DTYPE = np.dtype([("prim", "<i4"), ("t", "<f4"), ("u", "<f4"), ("v", "<f4")])
RAY_DTYPE = np.dtype([("origin", "<f4", 3), ("t_min", "<f4"), ("direction", "<f4", 3), ("t_max", "<f4")])
NODE_DTYPE = np.dtype([("aabb_min", "<f8", 3), ("aabb_max", "<f8", 3), ("right_offset", "<i8"),
                       ("start_offset", "<u8"), ("primitive_count", "<u8")])


def _ptr(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)


def materials_array(mats) -> C.Array:
    arr = (N.rc_material * len(mats))()
    for i, m in enumerate(mats):
        arr[i].diffuse[:] = [float(x) for x in m.diffuse]
        arr[i].emittance[:] = [float(x) for x in m.emittance]
        arr[i].is_emissive = int(m.is_emissive)
        arr[i].non_shadowing = int(m.non_shadowing)
        arr[i].invert_normal = int(m.invert_normal)
        arr[i].dielectric = int(getattr(m, "dielectric", False))
        arr[i].ior = float(getattr(m, "ior", 0.0)) if arr[i].dielectric else 0.0
    return arr


def camera_record(desc: SceneDesc, width: int | None = None, height: int | None = None) -> N.rc_camera:
    cam = N.rc_camera()
    c = desc.camera
    pos = (C.c_double * 3)(*c.position)
    st = N.lib().rc_camera_from_euler(pos, c.pitch, c.yaw, c.roll, c.fov, width or desc.width,
                                       height or desc.height, C.byref(cam))
    if st != N.RC_OK:
        raise RaycerError(st, "rc_camera_from_euler failed")
    return cam


FILTERS = {"box": N.RC_FILTER_BOX, "tent": N.RC_FILTER_TENT, "bell": N.RC_FILTER_BELL,
           "gaussian": N.RC_FILTER_GAUSSIAN, "mitchell": N.RC_FILTER_MITCHELL, "lanczos": N.RC_FILTER_LANCZOS_SINC}


def general_record(desc: SceneDesc, seed: int = 1) -> N.rc_general:
    s = desc.settings
    g = N.rc_general()
    tracer = TracerType.PATH if s.get("tracer", "path") == "path" else TracerType.RAY
    N.lib().rc_general_defaults(C.byref(g), int(tracer))
    if "max_path_length" in s:
        g.max_path_length = int(s["max_path_length"])
    g.path_sample_count = int(s.get("path_sample_count", 1))
    g.multi_sample_count_sqrt = int(s.get("multi_sample_count_sqrt", 1))
    g.multi_sampler_type = {"cmj": N.RC_SAMPLER_CMJ, "random": N.RC_SAMPLER_RANDOM,
                            "center": N.RC_SAMPLER_CENTER}[s.get("sampler", "cmj")]
    g.russian_roulette_depth = int(s.get("russian_roulette_depth", 0))
    # the scene descriptions of this package default to the box filter; the
    # C records' default (rc_general_defaults) is the reference's MITCHELL
    g.filter_type = FILTERS[s.get("filter", "box")]
    if "filter_radius" in s:
        g.filter_radius[:] = [float(x) for x in s["filter_radius"]]
    if s.get("miss_radiance") is not None:
        # GPU extension: escaping paths see a uniform sky of this radiance
        g.flags |= N.RC_GENERAL_SKY
        g.background[:] = [float(x) for x in s["miss_radiance"]]
    g.seed = int(seed)
    return g


def tonemapper_record(desc: SceneDesc) -> N.rc_tonemapper:
    t = N.rc_tonemapper()
    N.lib().rc_tonemapper_defaults(C.byref(t))
    s = desc.settings
    if s.get("tonemap", "reinhard") == "passthrough":
        t.type = N.RC_TONEMAP_PASSTHROUGH
    t.key = float(s.get("key", 0.18))
    t.gamma = float(s.get("gamma", 2.2))
    return t


class TracerState:
    """TracerState (TracerState.h:13-26). ``pixelsProcessed`` is a 64-bit
    word that a running render advances, so another thread can watch it as
    ConsoleRunner's main thread does (ConsoleRunner.cpp:126-142)."""

    def __init__(self, scene: SceneDesc | None = None, film: "Film | None" = None, filmWidth: int = 0,
                 filmHeight: int = 0, pixelStartOffset: int = 0, pixelCount: int = 0, pixelsProcessed: int = 0):
        self.scene = scene
        self.film = film
        self.filmWidth = filmWidth
        self.filmHeight = filmHeight
        self.pixelStartOffset = pixelStartOffset
        self.pixelCount = pixelCount
        self._processed = C.c_uint64(int(pixelsProcessed))

    @property
    def pixelsProcessed(self) -> int:
        return int(self._processed.value)

    @pixelsProcessed.setter
    def pixelsProcessed(self, value: int) -> None:
        self._processed.value = int(value)


class Interrupted:
    """The ``interrupted`` flag of Tracer::run (std::atomic<bool>&,
    Tracer.h:28): ``set()`` from any thread stops a running render at its
    kernels' next work-queue check (the render then raises RaycerError with
    status RC_CANCELLED). A ``threading.Event`` works too, through a watcher
    thread that polls it every millisecond."""

    def __init__(self) -> None:
        self._word = C.c_int32(0)

    def set(self) -> None:
        self._word.value = 1

    def clear(self) -> None:
        self._word.value = 0

    def is_set(self) -> bool:
        return bool(self._word.value)


class Film:
    """Film (Film.h:23-52): per-pixel sum of weighted colours and of weights."""

    def __init__(self, width: int = 0, height: int = 0):
        self.width = 0
        self.height = 0
        self.pixels = np.zeros((0, 4), np.float64)
        self.toneMappedImage = np.zeros((0, 4), np.float32)
        if width and height:
            self.resize(width, height)

    def resize(self, width: int, height: int = 1) -> None:
        self.width, self.height = int(width), int(height)
        self.pixels = np.zeros((self.width * self.height, 4), np.float64)
        self.toneMappedImage = np.zeros((self.width * self.height, 4), np.float32)

    def clear(self) -> None:
        self.pixels[:] = 0.0

    def addSample(self, index: int, color, filterWeight: float) -> None:
        self.pixels[index, :3] += np.asarray(color, np.float64)[:3] * filterWeight
        self.pixels[index, 3] += filterWeight

    def generateToneMappedImage(self, scene: SceneDesc, tracer: "CudaTracer") -> np.ndarray:
        """Film::generateToneMappedImage (Film.cpp:61-69), on the GPU."""
        tracer._set_tonemapper(scene)
        self.toneMappedImage = tracer.tonemap_film(self.pixels.astype(np.float32))
        return self.toneMappedImage

    def getToneMappedImage(self) -> np.ndarray:
        return self.toneMappedImage


def _instanced_arrays(scene):
    """rc_mesh / rc_instance arrays of a two-level scene (scenes.InstancedScene)
    and the numpy arrays they point into (keep them alive during the call)."""
    meshes = (N.rc_mesh * len(scene.meshes))()
    keep = []
    for i, (v, m) in enumerate(scene.meshes):
        v = np.ascontiguousarray(v, np.float64)
        m = np.ascontiguousarray(m, np.uint32)
        keep += [v, m]
        meshes[i].vertices = v.ctypes.data
        meshes[i].material_index = m.ctypes.data
        meshes[i].triangle_count = v.shape[0]
    insts = (N.rc_instance * len(scene.instances))()
    for i, d in enumerate(scene.instances):
        insts[i].mesh = int(d.mesh)
        insts[i].material = int(d.material)
        insts[i].scale[:] = [float(x) for x in d.scale]
        insts[i].rotate[:] = [float(x) for x in d.rotate]
        insts[i].translate[:] = [float(x) for x in d.translate]
    return meshes, insts, keep


def write_scene_file(scene, path) -> None:
    """Host-only: builds the scene's BVH(s) and device records and writes a
    scene file (a SceneDesc, or a two-level scenes.InstancedScene)."""
    err = C.create_string_buffer(512)
    if hasattr(scene, "instances"):
        meshes, insts, keep = _instanced_arrays(scene)
        mats = materials_array(scene.materials)
        st = N.lib().rc_write_instanced_scene_file(meshes, len(scene.meshes), insts, len(scene.instances), mats,
                                                    len(scene.materials), int(scene.max_leaf_size),
                                                    str(path).encode(), err, 512)
        del keep
        if st != N.RC_OK:
            raise RaycerError(st, f"write_scene_file: {err.value.decode()}")
        return
    v = np.ascontiguousarray(scene.vertices, np.float64)
    m = np.ascontiguousarray(scene.material_index, np.uint32)
    mats = materials_array(scene.materials)
    st = N.lib().rc_write_scene_file(_ptr(v), _ptr(m), v.shape[0], mats, len(scene.materials),
                                      int(scene.max_leaf_size), str(path).encode(), err, 512)
    if st != N.RC_OK:
        raise RaycerError(st, f"write_scene_file: {err.value.decode()}")


def inspect_scene_file(path) -> dict:
    """Validates a scene file (host only) and returns its counts and bounds."""
    info = N.rc_scene_file_info()
    err = C.create_string_buffer(512)
    st = N.lib().rc_inspect_scene_file(str(path).encode(), C.byref(info), err, 512)
    if st != N.RC_OK:
        raise RaycerError(st, err.value.decode())
    return {"triangles": info.triangles, "materials": info.materials, "bvh_nodes": info.bvh_nodes,
            "bvh_depth": info.bvh_depth, "bounds": list(info.bounds), "meshes": info.meshes,
            "instances": info.instances}


class CudaTracer:
    """GPU tracer with the method shape of CLTracer (CLTracer.h:23-41)."""

    def __init__(self, device: int = 0):
        self._lib = N.lib()
        self._h = C.c_void_p()
        st = self._lib.rc_create(C.byref(self._h), int(device))
        if st != N.RC_OK:
            raise RaycerError(st, "rc_create failed")
        self.imageWidth = 0
        self.imageHeight = 0
        self._scene: SceneDesc | None = None
        self._seed = 1

    # -- helpers --------------------------------------------------------
    def _check(self, st: int, what: str) -> None:
        if st != N.RC_OK:
            msg = self._lib.rc_last_error(self._h)
            raise RaycerError(st, f"{what}: {msg.decode() if msg else ''}")

    def close(self) -> None:
        if self._h:
            self._lib.rc_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- CLTracer shape -------------------------------------------------
    def initializeKernels(self) -> None:
        """The kernels are compiled into the library; nothing to build at run time."""

    def releaseKernels(self) -> None:
        """Kernels live as long as the library."""

    def initializeImageBuffers(self, width: int, height: int, imageTextureId: int = 0) -> None:
        """CLTracer::initializeImageBuffers (CLTracer.cpp:100-163); the GL texture id is ignored
        (headless device buffer)."""
        del imageTextureId
        self._check(self._lib.rc_resize(self._h, int(width), int(height)), "initializeImageBuffers")
        self.imageWidth, self.imageHeight = int(width), int(height)

    def releaseImageBuffers(self) -> None:
        """Film buffers are released with the handle or replaced by the next resize."""

    def initializeBuffers(self, scene: SceneDesc, seed: int = 1, prebuilt=None, cache=None) -> None:
        """CLTracer::initializeBuffers + CLScene::readSceneFull (CLTracer.cpp:173, CLScene.cpp:72).
        cache: a scene file path; loaded when it holds a scene of this size, else
        written after the upload."""
        if cache is not None and prebuilt is None:
            import os
            if os.path.exists(cache):
                try:
                    info = inspect_scene_file(cache)
                except RaycerError:
                    info = None
                if info and info["triangles"] == scene.triangle_count and info["materials"] == len(scene.materials):
                    self.load_scene(cache, scene, seed)
                    return
            self.initializeBuffers(scene, seed)
            self.save_scene(cache)
            return
        v = np.ascontiguousarray(scene.vertices, np.float64)
        m = np.ascontiguousarray(scene.material_index, np.uint32)
        mats = materials_array(scene.materials)
        if prebuilt is None:
            st = self._lib.rc_upload_scene(self._h, _ptr(v), _ptr(m), v.shape[0], mats, len(scene.materials),
                                           int(scene.max_leaf_size))
        else:
            nodes, order = prebuilt
            nodes = np.ascontiguousarray(nodes, NODE_DTYPE)
            order = np.ascontiguousarray(order, np.uint64)
            st = self._lib.rc_upload_scene_prebuilt(self._h, _ptr(v), _ptr(m), v.shape[0], mats,
                                                    len(scene.materials), _ptr(nodes), nodes.shape[0], _ptr(order))
        self._check(st, "initializeBuffers")
        self._scene = scene
        self._seed = seed
        self._set_general(scene)
        self._set_tonemapper(scene)
        self._set_lights(scene)

    def initializeInstanced(self, scene, seed: int = 1) -> None:
        """Uploads a two-level scene (scenes.InstancedScene) with rc_upload_instanced."""
        meshes, insts, keep = _instanced_arrays(scene)
        mats = materials_array(scene.materials)
        self._check(self._lib.rc_upload_instanced(self._h, meshes, len(scene.meshes), insts, len(scene.instances),
                                                  mats, len(scene.materials), int(scene.max_leaf_size)),
                    "upload_instanced")
        del keep
        self._scene = scene
        self._seed = seed
        self._set_general(scene)
        self._set_tonemapper(scene)
        self._set_lights(scene)

    def save_scene(self, path) -> None:
        """Writes the uploaded scene as a binary scene + BVH file."""
        self._check(self._lib.rc_save_scene(self._h, str(path).encode()), "save_scene")

    def load_scene(self, path, scene: SceneDesc, seed: int = 1) -> None:
        """Loads a scene file; `scene` supplies the camera and render settings."""
        self._check(self._lib.rc_load_scene(self._h, str(path).encode()), "load_scene")
        self._scene = scene
        self._seed = seed
        self._set_general(scene)
        self._set_tonemapper(scene)
        self._set_lights(scene)

    def releaseBuffers(self) -> None:
        self._check(self._lib.rc_release_scene(self._h), "releaseBuffers")
        self._scene = None

    def run(self, state: TracerState, interrupted: "Interrupted | threading.Event | None" = None) -> None:
        """CLTracer::run (CLTracer.cpp:262-305): camera upload, then the
        render. ``state.pixelsProcessed`` advances while it runs; setting
        ``interrupted`` from another thread stops it (RC_CANCELLED)."""
        scene = state.scene or self._scene
        self.set_camera(camera_record(scene, state.filmWidth or self.imageWidth,
                                      state.filmHeight or self.imageHeight))
        count = state.pixelCount or self.imageWidth * self.imageHeight
        watcher = None
        if interrupted is None:
            flag = None
        elif isinstance(interrupted, Interrupted):
            flag = C.byref(interrupted._word)
        else:
            word = C.c_int32(1 if interrupted.is_set() else 0)
            flag = C.byref(word)
            finished = threading.Event()

            def watch():
                while not finished.is_set():
                    if interrupted.wait(0.001):
                        word.value = 1
                        return

            watcher = threading.Thread(target=watch, daemon=True)
            watcher.start()
        try:
            st = self._lib.rc_render(self._h, int(state.pixelStartOffset), int(count), flag,
                                     C.byref(state._processed))
        finally:
            if watcher is not None:
                finished.set()
                watcher.join()
        self._check(st, "run")

    def set_time_budget(self, milliseconds: float | None) -> None:
        """Time budget of later renders (rc_set_time_budget); None removes it."""
        self._check(self._lib.rc_set_time_budget(self._h, -1.0 if milliseconds is None else float(milliseconds)),
                    "set_time_budget")

    def downloadImage(self) -> np.ndarray:
        """Tone-mapped image (CLTracer::downloadImage, CLTracer.cpp:307): (height, width, 4) float32."""
        out = np.empty((self.imageWidth * self.imageHeight, 4), np.float32)
        self._check(self._lib.rc_resolve(self._h, _ptr(out)), "downloadImage")
        return out.reshape(self.imageHeight, self.imageWidth, 4)

    def clear(self) -> None:
        self._check(self._lib.rc_clear(self._h), "clear")

    # -- records ----------------------------------------------------------
    def set_camera(self, cam: N.rc_camera) -> None:
        self._check(self._lib.rc_set_camera(self._h, C.byref(cam)), "set_camera")

    def set_general(self, g: N.rc_general) -> None:
        self._check(self._lib.rc_set_general(self._h, C.byref(g)), "set_general")

    def _set_general(self, scene: SceneDesc) -> None:
        self.set_general(general_record(scene, self._seed))

    def _set_tonemapper(self, scene: SceneDesc) -> None:
        t = tonemapper_record(scene)
        self._check(self._lib.rc_set_tonemapper(self._h, C.byref(t)), "set_tonemapper")

    def _set_lights(self, scene: SceneDesc) -> None:
        if scene.light_direction is None:
            self._check(self._lib.rc_set_directional_lights(self._h, None, 0), "set_lights")
            return
        lights = (N.rc_directional_light * 1)()
        lights[0].direction[:] = [float(x) for x in scene.light_direction]
        lights[0].color[:] = [1.0, 1.0, 1.0]
        lights[0].intensity = 1.0
        self._check(self._lib.rc_set_directional_lights(self._h, lights, 1), "set_lights")

    def set_traversal_order(self, order: int) -> None:
        self._check(self._lib.rc_set_traversal_order(self._h, int(order)), "set_traversal_order")

    def set_counting(self, enable: bool) -> None:
        self._check(self._lib.rc_set_counting(self._h, int(bool(enable))), "set_counting")

    # -- read-back and queries -------------------------------------------
    def read_cast(self) -> np.ndarray:
        out = np.empty(self.imageWidth * self.imageHeight, CAST_DTYPE)
        self._check(self._lib.rc_read_cast(self._h, _ptr(out)), "read_cast")
        return out

    def read_linear(self) -> np.ndarray:
        out = np.empty((self.imageWidth * self.imageHeight, 4), np.float32)
        self._check(self._lib.rc_read_linear(self._h, _ptr(out)), "read_linear")
        return out

    def read_film(self) -> np.ndarray:
        out = np.empty((self.imageWidth * self.imageHeight, 4), np.float32)
        self._check(self._lib.rc_read_film(self._h, _ptr(out)), "read_film")
        return out

    def tonemap_film(self, film_rgbw: np.ndarray) -> np.ndarray:
        f = np.ascontiguousarray(film_rgbw, np.float32).reshape(-1, 4)
        out = np.empty_like(f)
        self._check(self._lib.rc_tonemap_film(self._h, _ptr(f), f.shape[0], _ptr(out)), "tonemap_film")
        return out

    def cast(self, rays: np.ndarray, any_hit: bool = False, order: int = N.RC_ORDER_NEAREST) -> np.ndarray:
        r = np.ascontiguousarray(rays, RAY_DTYPE)
        out = np.empty(r.shape[0], HIT_DTYPE)
        self._check(self._lib.rc_cast(self._h, _ptr(r), r.shape[0], int(any_hit), int(order), _ptr(out)), "cast")
        return out

    def cast_with_shadow(self, rays: np.ndarray, order: int = N.RC_ORDER_NEAREST) -> np.ndarray:
        r = np.ascontiguousarray(rays, RAY_DTYPE)
        out = np.empty(r.shape[0], CAST_DTYPE)
        self._check(self._lib.rc_cast_with_shadow(self._h, _ptr(r), r.shape[0], int(order), _ptr(out)),
                    "cast_with_shadow")
        return out

    def get_bvh(self) -> tuple[np.ndarray, np.ndarray]:
        count = C.c_int64(0)
        self._check(self._lib.rc_get_bvh(self._h, None, 0, C.byref(count), None, 0), "get_bvh")
        nodes = np.empty(count.value, NODE_DTYPE)
        n = self._scene.triangle_count if self._scene else 0
        order = np.empty(n, np.uint64)
        self._check(self._lib.rc_get_bvh(self._h, _ptr(nodes), nodes.shape[0], C.byref(count), _ptr(order), n),
                    "get_bvh")
        return nodes, order

    def stats(self) -> dict:
        s = N.rc_stats()
        self._check(self._lib.rc_get_stats(self._h, C.byref(s)), "stats")
        out = {}
        for k, _ in N.rc_stats._fields_:
            v = getattr(s, k)
            out[k] = list(v) if isinstance(v, C.Array) else v
        return out

    def sync(self) -> None:
        self._check(self._lib.rc_sync(self._h), "sync")

    @property
    def handle(self) -> C.c_void_p:
        return self._h


class _GpuTracerAdapter:
    """Tracer-compatible adapter: run(state, interrupted) renders the state's pixel range on the GPU and
    adds the weighted samples to state.film (Tracer::run, Tracer.cpp:58-113)."""

    def __init__(self, tracer_type: TracerType, device: int = 0):
        self.type = tracer_type
        self.device = device
        self.cuda: CudaTracer | None = None

    def run(self, state: TracerState, interrupted: "threading.Event | None" = None) -> None:
        scene = state.scene
        if self.cuda is None:
            self.cuda = CudaTracer(self.device)
        t = self.cuda
        if t._scene is not scene:
            t.initializeBuffers(scene)
        if (t.imageWidth, t.imageHeight) != (state.filmWidth, state.filmHeight):
            t.initializeImageBuffers(state.filmWidth, state.filmHeight)
        # a new random stream per call, like the CPU tracer's continuing generators
        self.runs = getattr(self, "runs", 0) + 1
        g = general_record(scene, seed=self.runs)
        g.tracer_type = int(self.type)
        t.set_general(g)
        t.clear()
        t.run(state, interrupted)
        if self.type == TracerType.PATH:
            film = t.read_film()[: state.pixelCount]
            state.film.pixels[: state.pixelCount] += film.astype(np.float64)


class Tracer:
    @staticmethod
    def getTracer(tracer_type: TracerType, device: int = 0) -> _GpuTracerAdapter:
        """Tracer::getTracer (Tracer.cpp:24-32)."""
        if tracer_type not in (TracerType.RAY, TracerType.PATH):
            raise RuntimeError("Invalid tracer type")
        return _GpuTracerAdapter(TracerType(tracer_type), device)
