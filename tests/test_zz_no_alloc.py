"""The allocation-free entry point (rc_cast_with_shadow_device_noalloc).

It serves callers that cannot allocate device memory while they trace (an
application whose GPU memory is owned by its own pool allocator, a per-frame
callback that cannot take cudaMalloc's implicit synchronisation). Its results
and statistics must equal the allocating entry point's, call after call,
although every call reuses the same static scratch array: in both traversal
orders, with and without a light, counted (the two-kernel form, which fills
the static shadow queue) and uncounted, and with the two-kernel form forced
for uncounted frames too (RC_TRACE_FUSED=0, read once per process, so that
case runs in a child process). Collected last on purpose."""

from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

import oracle
from raycer_gb300 import _native as N
from raycer_gb300.tracer import CAST_DTYPE, RAY_DTYPE, CudaTracer, camera_record

from helpers import camera_floats, small_heightfield, small_room

pytestmark = pytest.mark.gpu

MAX_RAYS = 1 << 20
# statistics both entry points report for the same rays (times excluded)
STAT_KEYS = ("rays_traced", "node_visits", "tri_tests", "stage_rays", "stage_nodes", "stage_tris")


def _compare(order: int, light: bool, counting: bool) -> None:
    import torch

    sc = small_room(width=640, height=360, clutter=1500)
    sc.light_direction = (-0.3, -1.0, -0.2) if light else None
    cam = camera_floats(camera_record(sc))
    n = sc.width * sc.height
    rays = oracle.camera_rays32(cam, sc.width, n).view(RAY_DTYPE).reshape(-1)
    with CudaTracer(0) as t:
        t.initializeBuffers(sc)
        t.set_counting(counting)
        expected = t.cast_with_shadow(rays, order=order)
        want = t.stats()
        assert (expected["prim"] >= 0).any()
        if light:
            assert ((expected["flags"] & 4) != 0).any()
        else:
            assert not (expected["flags"] & 2).any()
        d_rays = torch.from_numpy(rays.view(np.float32).reshape(n, 8)).cuda()
        for call in range(2):
            d_out = torch.full((n, 4), -7, dtype=torch.int32, device="cuda")
            torch.cuda.synchronize()
            st = N.lib().rc_cast_with_shadow_device_noalloc(t.handle, C.c_void_p(d_rays.data_ptr()), n, order,
                                                            C.c_void_p(d_out.data_ptr()))
            assert st == N.RC_OK, N.lib().rc_last_error(t.handle)
            got = d_out.cpu().numpy().view(CAST_DTYPE).reshape(-1)
            assert np.array_equal(got, expected), f"call {call}: {(got != expected).sum()} records differ"
            have = t.stats()
            for k in STAT_KEYS:
                assert have[k] == want[k], (call, k, have[k], want[k])
            assert have["rays_traced"] == n + int((expected["flags"] & 2).astype(bool).sum())
            if counting:
                assert have["node_visits"] > 0 and have["tri_tests"] > 0


@pytest.mark.parametrize("counting", [False, True])
@pytest.mark.parametrize("light", [True, False])
@pytest.mark.parametrize("order", [N.RC_ORDER_NEAREST, N.RC_ORDER_REFERENCE])
def test_noalloc_matches_allocating_entry_point_twice(order, light, counting):
    pytest.importorskip("torch")
    _compare(order, light, counting)


@pytest.mark.parametrize("order", [N.RC_ORDER_NEAREST, N.RC_ORDER_REFERENCE])
def test_noalloc_two_kernel_form_matches(order):
    """RC_TRACE_FUSED=0: uncounted frames also run the primary and shadow
    kernels with the shadow queue in the static array."""
    pytest.importorskip("torch")
    here = Path(__file__).resolve().parent
    code = (f"import sys; sys.path[:0] = [{str(here)!r}, {str(here.parent)!r}]\n"
            f"import test_zz_no_alloc as m; m._compare({int(order)}, True, False); print('ok')\n")
    env = dict(os.environ, RC_TRACE_FUSED="0")
    res = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=600)
    assert res.returncode == 0 and "ok" in res.stdout, res.stdout[-2000:] + res.stderr[-4000:]


def test_noalloc_rejects_batches_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    sc = small_heightfield()
    with CudaTracer(0) as t:
        t.initializeBuffers(sc)
        d = torch.zeros((16, 8), dtype=torch.float32, device="cuda")
        st = N.lib().rc_cast_with_shadow_device_noalloc(t.handle, C.c_void_p(d.data_ptr()), MAX_RAYS + 1,
                                                        N.RC_ORDER_NEAREST, C.c_void_p(d.data_ptr()))
        assert st == N.RC_INVALID_ARG
        assert b"1048576" in N.lib().rc_last_error(t.handle)
