"""The allocation-free entry point (rc_cast_with_shadow_device_noalloc).

It serves callers that cannot allocate device memory while they trace (an
application whose GPU memory is owned by its own pool allocator, a per-frame
callback that cannot take cudaMalloc's implicit synchronisation). Its results
must equal the allocating entry point's, call after call, although every call
reuses the same static scratch array. Collected last on purpose."""

from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import oracle
from raycer_gb300 import _native as N
from raycer_gb300.tracer import CAST_DTYPE, RAY_DTYPE, CudaTracer, camera_record

from helpers import camera_floats, small_heightfield, small_room

pytestmark = pytest.mark.gpu

MAX_RAYS = 1 << 20


def test_noalloc_matches_allocating_entry_point_twice():
    torch = pytest.importorskip("torch")
    sc = small_room(width=640, height=360, clutter=1500)
    sc.light_direction = (-0.3, -1.0, -0.2)
    cam = camera_floats(camera_record(sc))
    n = sc.width * sc.height
    rays = oracle.camera_rays32(cam, sc.width, n).view(RAY_DTYPE).reshape(-1)
    with CudaTracer(0) as t:
        t.initializeBuffers(sc)
        expected = t.cast_with_shadow(rays, order=N.RC_ORDER_NEAREST)
        assert (expected["prim"] >= 0).any() and ((expected["flags"] & 4) != 0).any()
        d_rays = torch.from_numpy(rays.view(np.float32).reshape(n, 8)).cuda()
        for call in range(2):
            d_out = torch.full((n, 4), -7, dtype=torch.int32, device="cuda")
            torch.cuda.synchronize()
            st = N.lib().rc_cast_with_shadow_device_noalloc(t.handle, C.c_void_p(d_rays.data_ptr()), n,
                                                            N.RC_ORDER_NEAREST, C.c_void_p(d_out.data_ptr()))
            assert st == N.RC_OK, N.lib().rc_last_error(t.handle)
            got = d_out.cpu().numpy().view(CAST_DTYPE).reshape(-1)
            assert np.array_equal(got, expected), f"call {call}: {(got != expected).sum()} records differ"
            assert t.stats()["rays_traced"] == n + int((expected["flags"] & 2).astype(bool).sum())


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
