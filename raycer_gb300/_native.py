"""ctypes binding of the C ABI in include/raycer_gb300.h.

Loads the in-tree ``raycer_gb300/lib/libraycer_gb300.so``. There is no CPU
fallback: if the library is missing, importing this module raises, and every
call that reaches the GPU fails with the CUDA error the library reports.
"""

from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "lib" / "libraycer_gb300.so"

RC_OK = 0
RC_INVALID_ARG = 1
RC_OOM = 2
RC_CUDA = 3
RC_CANCELLED = 4
RC_TIMEOUT = 5
RC_NOT_READY = 6
RC_UNSUPPORTED = 7
RC_DEVICE_ERROR = 8
RC_IO = 9

STATUS_NAMES = {
    RC_OK: "RC_OK", RC_INVALID_ARG: "RC_INVALID_ARG", RC_OOM: "RC_OOM", RC_CUDA: "RC_CUDA",
    RC_CANCELLED: "RC_CANCELLED", RC_TIMEOUT: "RC_TIMEOUT", RC_NOT_READY: "RC_NOT_READY",
    RC_UNSUPPORTED: "RC_UNSUPPORTED", RC_DEVICE_ERROR: "RC_DEVICE_ERROR", RC_IO: "RC_IO",
}

RC_TRACER_RAY = 0
RC_TRACER_PATH = 1
RC_SAMPLER_CENTER = 0
RC_SAMPLER_RANDOM = 1
RC_SAMPLER_CMJ = 4
RC_FILTER_BOX = 0
RC_FILTER_TENT = 1
RC_FILTER_BELL = 2
RC_FILTER_GAUSSIAN = 3
RC_FILTER_MITCHELL = 4
RC_FILTER_LANCZOS_SINC = 5
RC_TONEMAP_PASSTHROUGH = 0
RC_TONEMAP_REINHARD = 3
RC_ORDER_REFERENCE = 0
RC_ORDER_NEAREST = 1


class rc_material(C.Structure):
    _fields_ = [("diffuse", C.c_float * 3), ("emittance", C.c_float * 3), ("is_emissive", C.c_int32),
                ("non_shadowing", C.c_int32), ("invert_normal", C.c_int32), ("dielectric", C.c_int32),
                ("ior", C.c_float)]


class rc_camera(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("forward", C.c_float * 3), ("right", C.c_float * 3),
                ("up", C.c_float * 3), ("image_plane_center", C.c_float * 3), ("aspect_ratio", C.c_float),
                ("image_plane_width", C.c_float), ("image_plane_height", C.c_float)]


class rc_general(C.Structure):
    _fields_ = [("tracer_type", C.c_int32), ("max_path_length", C.c_int32), ("path_sample_count", C.c_int32),
                ("multi_sample_count_sqrt", C.c_int32), ("multi_sampler_type", C.c_int32),
                ("filter_type", C.c_int32), ("filter_radius", C.c_float * 2), ("ray_start_offset", C.c_float),
                ("background", C.c_float * 3), ("russian_roulette_depth", C.c_int32), ("flags", C.c_int32),
                ("seed", C.c_uint64)]


class rc_tonemapper(C.Structure):
    _fields_ = [("type", C.c_int32), ("apply_gamma", C.c_int32), ("should_clamp", C.c_int32),
                ("reserved", C.c_int32), ("gamma", C.c_double), ("key", C.c_double)]


class rc_directional_light(C.Structure):
    _fields_ = [("direction", C.c_float * 3), ("color", C.c_float * 3), ("intensity", C.c_float)]


class rc_bvh_node(C.Structure):
    _fields_ = [("aabb_min", C.c_double * 3), ("aabb_max", C.c_double * 3), ("right_offset", C.c_int64),
                ("start_offset", C.c_uint64), ("primitive_count", C.c_uint64)]


class rc_ray(C.Structure):
    _fields_ = [("origin", C.c_float * 3), ("t_min", C.c_float), ("direction", C.c_float * 3),
                ("t_max", C.c_float)]


class rc_hit(C.Structure):
    _fields_ = [("prim", C.c_int32), ("t", C.c_float), ("u", C.c_float), ("v", C.c_float)]


class rc_cast_pixel(C.Structure):
    _fields_ = [("prim", C.c_int32), ("t", C.c_float), ("occluder", C.c_int32), ("flags", C.c_int32)]


class rc_stats(C.Structure):
    _fields_ = [("rays_traced", C.c_uint64), ("node_visits", C.c_uint64), ("tri_tests", C.c_uint64),
                ("last_ms", C.c_double), ("bvh_inner_nodes", C.c_uint64), ("bvh_depth", C.c_uint64),
                ("device_bytes", C.c_uint64), ("stage_rays", C.c_uint64 * 2), ("stage_nodes", C.c_uint64 * 2),
                ("stage_tris", C.c_uint64 * 2), ("stage_ms", C.c_double * 2), ("build_ms", C.c_double)]


class rc_batch_stats(C.Structure):
    _fields_ = [("rays_traced", C.c_uint64), ("paths", C.c_uint64), ("last_ms", C.c_double), ("passes", C.c_int32),
                ("scenes", C.c_int32), ("graph_nodes", C.c_int32), ("reserved", C.c_int32)]


class rc_batch_tuning(C.Structure):
    _fields_ = [("bucket_min_triangles", C.c_uint32 * 4), ("slots", C.c_uint32 * 4), ("extend_block", C.c_int32 * 4),
                ("shade_block", C.c_int32 * 4), ("measured_paths_per_ms", C.c_double * 4)]


class rc_nrc_config(C.Structure):
    _fields_ = [("enabled", C.c_int32), ("terminate_segment", C.c_int32), ("train_stride", C.c_int32),
                ("train_steps", C.c_int32), ("train_batch", C.c_int32), ("min_suffix", C.c_int32),
                ("learning_rate", C.c_float), ("beta1", C.c_float), ("beta2", C.c_float), ("epsilon", C.c_float),
                ("box_min", C.c_float * 3), ("box_max", C.c_float * 3), ("seed", C.c_uint64),
                ("lookup_kernel", C.c_int32), ("tc_wait_polls", C.c_int32), ("sample_vertices", C.c_int32),
                ("reserved", C.c_int32)]


class rc_nrc_stats(C.Structure):
    _fields_ = [("lookups", C.c_uint64), ("training_samples", C.c_uint64), ("steps", C.c_uint64),
                ("last_loss", C.c_float), ("reserved", C.c_float), ("train_ms", C.c_double)]


class rc_mesh(C.Structure):
    _fields_ = [("vertices", C.c_void_p), ("material_index", C.c_void_p), ("triangle_count", C.c_int64)]


class rc_instance(C.Structure):
    _fields_ = [("mesh", C.c_int32), ("material", C.c_int32), ("scale", C.c_double * 3), ("rotate", C.c_double * 3),
                ("translate", C.c_double * 3)]


class rc_scene_file_info(C.Structure):
    _fields_ = [("triangles", C.c_uint64), ("materials", C.c_uint64), ("bvh_nodes", C.c_uint64),
                ("bvh_depth", C.c_uint64), ("bounds", C.c_double * 6), ("meshes", C.c_uint64),
                ("instances", C.c_uint64)]


RC_GENERAL_SKY = 1
RC_BUILDER_REFERENCE_SAH = 0
RC_BUILDER_GPU_LBVH = 1
RC_NRC_MMA_SYNC = 0
RC_NRC_TCGEN05 = 1
RC_NRC_ALL_VERTICES = 0
RC_NRC_LOOKUP_VERTEX = 1
RC_NRC_PARAMS = 20992
RC_NRC_QUERY_FLOATS = 12
RC_NRC_INPUTS = 128

P = C.c_void_p
i32, i64, u32, u64 = C.c_int32, C.c_int64, C.c_uint32, C.c_uint64

# name -> (restype, argtypes); every symbol the header declares.
PROTOTYPES = {
    "rc_create": (i32, [C.POINTER(P), C.c_int]),
    "rc_destroy": (None, [P]),
    "rc_last_error": (C.c_char_p, [P]),
    "rc_version": (C.c_char_p, []),
    "rc_upload_scene": (i32, [P, P, P, i64, P, i32, u32]),
    "rc_upload_scene_prebuilt": (i32, [P, P, P, i64, P, i32, P, i64, P]),
    "rc_get_bvh": (i32, [P, P, i64, C.POINTER(i64), P, i64]),
    "rc_build_bvh": (i32, [P, i64, u32, P, i64, C.POINTER(i64), P, C.POINTER(u32)]),
    "rc_release_scene": (i32, [P]),
    "rc_set_camera": (i32, [P, C.POINTER(rc_camera)]),
    "rc_set_general": (i32, [P, C.POINTER(rc_general)]),
    "rc_set_tonemapper": (i32, [P, C.POINTER(rc_tonemapper)]),
    "rc_set_directional_lights": (i32, [P, P, i32]),
    "rc_camera_from_euler": (i32, [P, C.c_double, C.c_double, C.c_double, C.c_double, u64, u64,
                                   C.POINTER(rc_camera)]),
    "rc_general_defaults": (None, [C.POINTER(rc_general), i32]),
    "rc_tonemapper_defaults": (None, [C.POINTER(rc_tonemapper)]),
    "rc_resize": (i32, [P, u64, u64]),
    "rc_clear": (i32, [P]),
    "rc_render": (i32, [P, u64, u64, P, C.POINTER(u64)]),
    "rc_set_time_budget": (i32, [P, C.c_double]),
    "rc_resolve": (i32, [P, P]),
    "rc_read_linear": (i32, [P, P]),
    "rc_read_film": (i32, [P, P]),
    "rc_read_cast": (i32, [P, P]),
    "rc_tonemap_film": (i32, [P, P, u64, P]),
    "rc_cast": (i32, [P, P, i64, i32, i32, P]),
    "rc_cast_device": (i32, [P, P, i64, i32, i32, P]),
    "rc_cast_with_shadow": (i32, [P, P, i64, i32, P]),
    "rc_cast_with_shadow_device_noalloc": (i32, [P, P, i64, i32, P]),
    "rc_batch_create": (i32, [C.POINTER(P), C.c_int]),
    "rc_batch_destroy": (None, [P]),
    "rc_batch_last_error": (C.c_char_p, [P]),
    "rc_batch_add_scene": (i32, [P, P, P, i64, P, i32, u32, C.POINTER(rc_camera), C.POINTER(rc_general), u64, u64,
                                 C.POINTER(i32)]),
    "rc_batch_autotune": (i32, [P, C.c_double]),
    "rc_batch_get_tuning": (i32, [P, C.POINTER(rc_batch_tuning)]),
    "rc_batch_render": (i32, [P, P]),
    "rc_batch_clear": (i32, [P]),
    "rc_batch_read_film": (i32, [P, i32, P]),
    "rc_batch_resolve": (i32, [P, i32, C.POINTER(rc_tonemapper), P]),
    "rc_batch_get_stats": (i32, [P, C.POINTER(rc_batch_stats)]),
    "rc_set_traversal_order": (i32, [P, i32]),
    "rc_set_counting": (i32, [P, i32]),
    "rc_get_stats": (i32, [P, C.POINTER(rc_stats)]),
    "rc_stream": (P, [P]),
    "rc_sync": (i32, [P]),
    "rc_nrc_defaults": (i32, [C.POINTER(rc_nrc_config)]),
    "rc_nrc_configure": (i32, [P, C.POINTER(rc_nrc_config)]),
    "rc_nrc_set_enabled": (i32, [P, i32]),
    "rc_nrc_get_params": (i32, [P, P, i64]),
    "rc_nrc_set_params": (i32, [P, P, i64]),
    "rc_nrc_infer": (i32, [P, P, i64, P]),
    "rc_nrc_encode": (i32, [P, P, i64, P]),
    "rc_nrc_gradient": (i32, [P, P, P, i64, P, P]),
    "rc_nrc_train": (i32, [P, P, P, i64, i32, P]),
    "rc_nrc_read_samples": (i32, [P, P, i64, C.POINTER(i64)]),
    "rc_nrc_get_stats": (i32, [P, C.POINTER(rc_nrc_stats)]),
    "rc_film_accumulate_f64": (i32, [P, P, i32]),
    "rc_set_bvh_builder": (i32, [P, i32]),
    "rc_upload_instanced": (i32, [P, C.POINTER(rc_mesh), i32, C.POINTER(rc_instance), i64, P, i32, u32]),
    "rc_save_scene": (i32, [P, C.c_char_p]),
    "rc_load_scene": (i32, [P, C.c_char_p]),
    "rc_write_scene_file": (i32, [P, P, i64, P, i32, u32, C.c_char_p, C.c_char_p, i64]),
    "rc_inspect_scene_file": (i32, [C.c_char_p, C.POINTER(rc_scene_file_info), C.c_char_p, i64]),
    "rc_write_instanced_scene_file": (i32, [P, i32, P, i64, P, i32, u32, C.c_char_p, C.c_char_p, i64]),
    "rc_film_rmse_f64": (i32, [P, P, C.POINTER(C.c_double)]),
}


def load(path: Path | None = None) -> C.CDLL:
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise ImportError(
            f"raycer_gb300 native library not found at {p}; build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'` (there is no CPU fallback)")
    lib = C.CDLL(str(p), mode=os.RTLD_NOW | os.RTLD_LOCAL)
    for name, (res, args) in PROTOTYPES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


_lib: C.CDLL | None = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        _lib = load()
    return _lib
