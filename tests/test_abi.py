"""The C ABI library loads, exports every entry point include/*.h declares,
and its host-only entry points behave as documented (no GPU needed)."""

from __future__ import annotations

import ctypes as C
import re
import shutil
from pathlib import Path

import numpy as np
import pytest

from raycer_gb300 import _native as N

INCLUDE = Path(__file__).resolve().parent.parent / "include"


def declared_symbols():
    names = set()
    for h in INCLUDE.glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names.update(re.findall(r"^\s*(?:rc_status|void\s*\*?|const\s+char\s*\*)\s*(rc_\w+)\s*\(", text, flags=re.M))
    return sorted(names)


def test_header_declares_the_entry_points():
    names = declared_symbols()
    assert len(names) >= 30
    assert {"rc_create", "rc_destroy", "rc_upload_scene", "rc_render", "rc_resolve", "rc_cast"} <= set(names)


def test_library_exports_every_declared_symbol():
    lib = N.lib()
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_every_declared_symbol():
    assert set(declared_symbols()) == set(N.PROTOTYPES)


def test_version():
    assert b"sm_103a" in N.lib().rc_version()


def test_null_handle_is_rejected():
    lib = N.lib()
    assert lib.rc_render(None, 0, 1, None, None) == N.RC_INVALID_ARG
    assert lib.rc_clear(None) == N.RC_INVALID_ARG
    assert lib.rc_resize(None, 4, 4) == N.RC_INVALID_ARG
    assert lib.rc_cast(None, None, 1, 0, 0, None) == N.RC_INVALID_ARG
    assert lib.rc_resolve(None, None) == N.RC_INVALID_ARG
    assert lib.rc_sync(None) == N.RC_INVALID_ARG
    assert lib.rc_last_error(None) == b"null handle"
    lib.rc_destroy(None)


def test_defaults_follow_the_reference():
    g = N.rc_general()
    N.lib().rc_general_defaults(C.byref(g), N.RC_TRACER_PATH)
    # Scene::General (Scene.h:89-108)
    assert (g.max_path_length, g.path_sample_count, g.multi_sample_count_sqrt) == (3, 1, 1)
    assert g.multi_sampler_type == N.RC_SAMPLER_CMJ
    assert abs(g.ray_start_offset - 1e-5) < 1e-12
    assert tuple(g.filter_radius) == (0.5, 0.5)
    t = N.rc_tonemapper()
    N.lib().rc_tonemapper_defaults(C.byref(t))
    assert (t.apply_gamma, t.should_clamp, t.gamma, t.key) == (1, 1, 2.2, 0.18)


def test_build_bvh_argument_checks():
    lib = N.lib()
    v = np.zeros((2, 9))
    v[0, 3] = v[1, 4] = 1.0
    v[:, 8] = 1.0
    cnt = C.c_int64(0)
    p = C.c_void_p(v.ctypes.data)
    assert lib.rc_build_bvh(p, 0, 4, None, 0, C.byref(cnt), None, None) == N.RC_INVALID_ARG
    assert lib.rc_build_bvh(p, 2, 0, None, 0, C.byref(cnt), None, None) == N.RC_UNSUPPORTED
    assert lib.rc_build_bvh(p, 2, 16, None, 0, C.byref(cnt), None, None) == N.RC_UNSUPPORTED
    assert lib.rc_build_bvh(p, 2, 4, None, 0, C.byref(cnt), None, None) == N.RC_OK and cnt.value == 1
    bad = v.copy()
    bad[1, 2] = np.nan
    assert lib.rc_build_bvh(C.c_void_p(bad.ctypes.data), 2, 4, None, 0, C.byref(cnt), None, None) == N.RC_INVALID_ARG
    small = np.empty(0, dtype=np.uint8)
    assert lib.rc_build_bvh(p, 2, 1, C.c_void_p(small.ctypes.data), 0, C.byref(cnt), None, None) == N.RC_INVALID_ARG


def test_camera_argument_checks():
    cam = N.rc_camera()
    pos = (C.c_double * 3)(0, 0, 0)
    assert N.lib().rc_camera_from_euler(pos, 0, 0, 0, 45, 1, 10, C.byref(cam)) == N.RC_INVALID_ARG
    assert N.lib().rc_camera_from_euler(pos, 0, 0, 0, 45, 2, 2, C.byref(cam)) == N.RC_OK
    assert cam.image_plane_width == 1.0 and cam.aspect_ratio == 1.0


@pytest.mark.skipif(shutil.which("nvidia-smi") is not None, reason="a GPU is present")
def test_create_without_gpu_fails_cleanly():
    h = C.c_void_p()
    st = N.lib().rc_create(C.byref(h), 0)
    assert st in (N.RC_CUDA, N.RC_OOM)
    assert not h.value
