"""CPU checks of the oracle and of the product's host code against the golden
fixtures the reference itself produced (tests/golden/make_golden.py)."""

from __future__ import annotations

import ctypes as C
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

import oracle
from raycer_gb300 import _native as N
from raycer_gb300 import scenes

GOLDEN = Path(__file__).resolve().parent / "golden"
META = json.loads((GOLDEN / "golden.json").read_text())


def _load(name):
    return np.load(GOLDEN / name)


def product_bvh(sc):
    lib = N.lib()
    v = np.ascontiguousarray(sc.vertices, np.float64)
    cnt, depth = C.c_int64(0), C.c_uint32(0)
    st = lib.rc_build_bvh(C.c_void_p(v.ctypes.data), v.shape[0], sc.max_leaf_size, None, 0, C.byref(cnt), None,
                          C.byref(depth))
    assert st == N.RC_OK
    nodes = np.empty(cnt.value, oracle.NODE_DTYPE)
    order = np.empty(v.shape[0], np.uint64)
    st = lib.rc_build_bvh(C.c_void_p(v.ctypes.data), v.shape[0], sc.max_leaf_size, C.c_void_p(nodes.ctypes.data),
                          cnt.value, C.byref(cnt), C.c_void_p(order.ctypes.data), C.byref(depth))
    assert st == N.RC_OK
    return nodes, order, depth.value


def digest(nodes, order):
    return {"node_count": int(nodes.shape[0]),
            "nodes_sha256": hashlib.sha256(np.ascontiguousarray(nodes, oracle.NODE_DTYPE).tobytes()).hexdigest(),
            "order_sha256": hashlib.sha256(np.ascontiguousarray(order, np.uint64).tobytes()).hexdigest()}


# -- BVH -----------------------------------------------------------------------

def test_room_bvh_matches_reference():
    g = _load("room.npz")
    sc = scenes.room_scene()
    pn, po, _ = product_bvh(sc)
    assert np.array_equal(pn, g["nodes"]) and np.array_equal(po, g["order"])
    on, oo = oracle.Oracle(sc).bvh()
    assert np.array_equal(on, g["nodes"]) and np.array_equal(oo, g["order"])
    assert digest(pn, po) == META["room_bvh"]


def test_small_heightfield_bvh_matches_reference():
    g = _load("heightfield_small.npz")
    sc = scenes.heightfield_scene(nx=64, nz=32, width=160, height=90)
    pn, po, _ = product_bvh(sc)
    assert np.array_equal(pn, g["nodes"]) and np.array_equal(po, g["order"])


def test_full_heightfield_bvh_digest_matches_reference():
    """1,045,506 triangles: the product's parallel builder and the oracle's serial
    restatement both reproduce the reference's node array and primitive order."""
    sc = scenes.heightfield_scene()
    assert sc.triangle_count == META["heightfield_triangles"] == 2 * 1023 * 511
    pn, po, depth = product_bvh(sc)
    assert digest(pn, po) == META["heightfield_bvh"]
    assert depth <= 64
    on, oo = oracle.Oracle(sc).bvh()
    assert digest(on, oo) == META["heightfield_bvh"]


# -- camera, noise, fastPow, CMJ ----------------------------------------------

def test_camera_from_euler_matches_reference():
    g = _load("camera_poses.npz")
    for pose, state in zip(g["poses"], g["states"]):
        cam = N.rc_camera()
        pos = (C.c_double * 3)(*pose[0:3])
        st = N.lib().rc_camera_from_euler(pos, pose[3], pose[4], pose[5], pose[6], int(pose[7]), int(pose[8]),
                                           C.byref(cam))
        assert st == N.RC_OK
        mine = np.array(list(cam.position) + list(cam.forward) + list(cam.right) + list(cam.up) +
                        list(cam.image_plane_center) + [cam.aspect_ratio, cam.image_plane_width,
                                                        cam.image_plane_height], np.float32)
        assert np.array_equal(mine, state[:18].astype(np.float32))


def test_oracle_camera_state64_matches_reference():
    """The oracle's float64 camera (what the CPU baseline renders through,
    without the product library) agrees with the reference's Camera state to
    a few units in the last place (libm and operation order)."""
    g = _load("camera_poses.npz")
    for pose, state in zip(g["poses"], g["states"]):
        mine = oracle.camera_state64(pose[0:3], pose[3], pose[4], pose[5], pose[6], int(pose[7]), int(pose[8]))
        assert mine.shape == state.shape
        assert np.all(np.abs(mine - state) <= 4 * np.spacing(np.maximum(np.abs(state), 1.0))), pose


def test_value_noise_matches_reference():
    g = _load("math.npz")
    p = g["noise_points"]
    assert np.array_equal(scenes.fbm_noise(2, 6, 2.0, 0.5, p[:, 0], p[:, 1], p[:, 2]), g["fbm_seed2"])
    assert np.array_equal(scenes.value_noise(11, p[:, 0], p[:, 1], p[:, 2]), g["noise_seed11"])


def test_fastpow_matches_reference():
    g = _load("math.npz")
    lib = oracle.oracle_lib()
    for inv, key in [(1.0 / 2.2, "fastpow_inv22"), (1.0 / 1.8, "fastpow_inv18")]:
        mine = np.array([lib.or64_fastpow(float(x), inv) for x in g["fastpow_x"]])
        assert np.array_equal(mine, g[key])


def test_cmj_matches_reference():
    g = _load("math.npz")
    lib = oracle.oracle_lib()
    for i, (n, perm) in enumerate(zip(g["cmj_n"], g["cmj_perm"])):
        out = g[f"cmj_out_{i}"].reshape(-1, 2)
        jit = g[f"cmj_jit_{i}"].reshape(-1, 2)
        n = int(n)
        perm = int(perm)
        buf = np.empty(2)
        for y in range(n):
            for x in range(n):
                k = y * n + x
                lib.or64_cmj(x, y, n, perm, jit[k, 0], jit[k, 1], C.c_void_p(buf.ctypes.data))
                assert np.array_equal(buf, out[k])
                # the device's 64-bit permute() reproduces the reference's strata
                sy = lib.or32_cmj_permute(y, n, (perm * 0x02E5BE93) & (2**64 - 1))
                sx = lib.or32_cmj_permute(x, n, (perm * 0x68BC21EB) & (2**64 - 1))
                assert int(np.rint((out[k, 0] * n - x) * n - jit[k, 0])) == sy
                assert int(np.rint((out[k, 1] * n - y) * n - jit[k, 1])) == sx


# -- tone mapping --------------------------------------------------------------

@pytest.mark.parametrize("key,gamma,clamp,ag", [(0.18, 2.2, 1, 1), (0.5, 1.8, 1, 1), (0.18, 2.2, 0, 1),
                                                (0.18, 2.2, 1, 0)])
def test_tonemap_oracle_matches_reference(key, gamma, clamp, ag):
    g = _load("tonemap.npz")
    out = oracle.tonemap64(g["linear"], key, gamma, bool(clamp), bool(ag))
    ref = g[f"out_{key}_{gamma}_{clamp}_{ag}"]
    # The reference sums log-luminance per OpenMP thread; the serial sum can move
    # a value across one step of fastPow's high-word quantisation (2^-20).
    assert np.nanmax(np.abs(out - ref)) <= 4e-6 * max(1.0, float(np.nanmax(np.abs(ref))))
    assert np.array_equal(np.isnan(out), np.isnan(ref))


# -- float64 hits ---------------------------------------------------------------

def _rays_at(state, width, height, pix):
    cam = state[:18].astype(np.float32)
    allr = oracle.camera_rays32(cam, width, width * height)
    return allr[pix]


def test_room_hits_fp64_bit_exact():
    g = _load("room.npz")
    sc = scenes.room_scene()
    rays = _rays_at(g["camera_state"], sc.width, sc.height, g["hit_pixels"])
    r6 = np.concatenate([rays[:, 0:3], rays[:, 4:7]], axis=1).astype(np.float64)
    prim, t, _, _ = oracle.Oracle(sc).intersect64(r6)
    assert np.array_equal(prim.astype(np.int32), g["hit_prim"])
    assert np.array_equal(t.astype(np.float32), g["hit_t"])


@pytest.fixture(scope="module")
def heightfield_oracle():
    sc = scenes.heightfield_scene()
    nodes, order, _ = product_bvh(sc)   # equal to the reference's (digest test above)
    return sc, oracle.Oracle(sc, prebuilt=(nodes, order))


def test_heightfield_hits_fp64_bit_exact(heightfield_oracle):
    sc, orc = heightfield_oracle
    g = _load("heightfield.npz")
    rays = _rays_at(g["camera_state"], sc.width, sc.height, g["hit_pixels"])
    r6 = np.concatenate([rays[:, 0:3], rays[:, 4:7]], axis=1).astype(np.float64)
    prim, t, _, _ = orc.intersect64(r6)
    assert np.array_equal(prim.astype(np.int32), g["hit_prim"])
    assert np.array_equal(t.astype(np.float32), g["hit_t"])


def classify_edge_ties(orc, rays8, prim, t, u, v, ref_prim, ref_t):
    """Returns the indices of id mismatches that are NOT edge ties.

    Edge tie (documented parity rule): the ray crosses the surface next to a
    triangle edge, so float32 and float64 rounding pick different sides of it.
    Both results are hits at the same distance (|t32 - t64| <= 1e-5 t64), and
    the float32 hit or the float64 hit lies within 1e-4 (barycentric) of an edge
    of its triangle. When one side misses, the other side's hit must lie within
    1e-4 of an edge (a silhouette edge)."""
    bad = []
    for i in np.nonzero(prim != ref_prim)[0]:
        r6 = np.concatenate([rays8[i, 0:3], rays8[i, 4:7]]).astype(np.float64)
        a, b = int(prim[i]), int(ref_prim[i])
        near32 = a >= 0 and min(u[i], v[i], 1.0 - u[i] - v[i]) < 1e-4
        if b >= 0:
            ok, tb, ub, vb = orc.tri64(b, r6)
            near64 = ok and min(ub, vb, 1.0 - ub - vb) < 1e-4
        else:
            near64 = False
        if a >= 0 and b >= 0:
            same_t = abs(float(t[i]) - float(ref_t[i])) <= 1e-5 * float(ref_t[i])
            if not (same_t and (near32 or near64)):
                bad.append(i)
        elif not (near32 or near64):
            bad.append(i)
    return bad


def test_fp32_twin_vs_reference_ids_edge_ties(heightfield_oracle):
    sc, orc = heightfield_oracle
    g = _load("heightfield.npz")
    rays = _rays_at(g["camera_state"], sc.width, sc.height, g["hit_pixels"])
    prim, t, u, v, _ = orc.cast32(rays, order=1)
    ref_prim, ref_t = g["hit_prim"], g["hit_t"]
    bad = classify_edge_ties(orc, rays, prim, t, u, v, ref_prim, ref_t)
    assert not bad, f"{len(bad)} id mismatches are not edge ties"
    same = (prim == ref_prim) & (prim >= 0)
    rel = np.abs(t[same].astype(np.float64) - ref_t[same]) / ref_t[same]
    assert rel.max() <= 1e-5


def test_fp32_twin_shadow_occlusion_vs_reference(heightfield_oracle):
    sc, orc = heightfield_oracle
    g = _load("heightfield.npz")
    cam = g["camera_state"][:18].astype(np.float32)
    L = -np.array(sc.light_direction, np.float32)
    out, _ = orc.raycast32(cam, sc.width, sc.width * sc.height, L, order=1)
    out = out[g["hit_pixels"]]
    occ = (out[:, 3] & 4) != 0
    both_hit = (out[:, 0] >= 0) & (g["hit_prim"] >= 0)
    mism = (occ != g["occluded"]) & both_hit
    # shadow origins differ by float32 rounding of the hit point; only grazing
    # shadow rays may flip.
    assert mism.sum() <= max(3, int(1e-3 * both_hit.sum())), f"{mism.sum()} occlusion flips"


# -- path tracing statistics -------------------------------------------------------

def image_z_scores(img, g):
    """z-scores of one render (H*W x 3 linear) against the reference's K renders:
    per channel for the image mean, and per 8x8 block. One render's spread is
    the reference renders' spread (same estimator, same sample count), so
    var(diff) = var_one * (1 + 1/K), estimated with K-1 dof. Returns the image
    z (3), the block z of blocks with spread, and the count of blocks the
    reference rendered identically K times but this render did not."""
    K = int(g["pt_runs"])
    H, W, B = 240, 320, 8
    im = img.reshape(H, W, 3)
    d = im.mean(axis=(0, 1)) - g["pt_mean"]
    z = d / np.sqrt(g["pt_mean_var"] * (1.0 + 1.0 / K))
    blocks = im.reshape(H // B, B, W // B, B, 3).mean(axis=(1, 3))
    bd = blocks - g["pt_block_mean"]
    var = g["pt_block_var"] * (1.0 + 1.0 / K)
    const = var == 0.0
    const_diff = int(np.sum(np.abs(bd[const]) > 1e-5 * np.maximum(1.0, np.abs(g["pt_block_mean"][const]))))
    return z, bd[~const] / np.sqrt(var[~const]), const_diff


def check_statistics(img, g):
    """Monte Carlo parity of a path-traced image with the reference's.

    * image mean per channel within 3 sigma (the bar for bias);
    * per 8x8 block: the estimator is heavy-tailed and skewed (rare paths that
      reach the emitter), so the block z are judged by robust statistics —
      median in [-0.45, 0.15] (unbiased renders give about -0.2 from the skew),
      1.4826 * MAD in [0.7, 1.2], and fewer than 3.5 % beyond |z| = 3."""
    z, bz, const_diff = image_z_scores(img, g)
    assert np.all(np.abs(z) < 3.0), z
    med = float(np.median(bz))
    mad = 1.4826 * float(np.median(np.abs(bz - med)))
    assert -0.45 <= med <= 0.15, med
    assert 0.7 <= mad <= 1.2, mad
    assert np.mean(np.abs(bz) > 3.0) < 0.035, np.mean(np.abs(bz) > 3.0)
    assert const_diff <= 12, const_diff


def test_fp32_twin_path_tracer_matches_reference_statistically():
    g = _load("room.npz")
    sc = scenes.room_scene()
    orc = oracle.Oracle(sc)
    cam = g["camera_state"][:18].astype(np.float32)
    film, _ = orc.render_path32(cam, sc.width, sc.width * sc.height, 4, 1, 4, (0.5, 0.5), 1e-5, 4, 0, 1, 3, 0)
    img = (film[:, :3] / film[:, 3:4]).astype(np.float64)
    check_statistics(img, g)


def test_fp64_port_path_tracer_matches_reference_statistically():
    g = _load("room.npz")
    sc = scenes.room_scene()
    orc = oracle.Oracle(sc)
    s = g["camera_state"]
    cam64 = oracle.cam64_from_state(s)
    film, rays, _ = orc.render_path64(cam64, sc.width, sc.width * sc.height, 4, 1, 4, seed=17)
    img = film[:, :3] / film[:, 3:4]
    check_statistics(img, g)
    # the port's BVH query count matches the reference's within noise
    ref_rays = g["pt_rays_per_run"].astype(np.float64)
    assert abs(rays - ref_rays.mean()) < 6 * ref_rays.std() + 0.002 * ref_rays.mean()
