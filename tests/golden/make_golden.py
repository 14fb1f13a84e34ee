"""Generates the golden fixtures in tests/golden/ from the reference itself.

Run where the reference's sources are present (it needs oracle/_ref, built by
oracle/Makefile.ref from the reference's own code):

    python tests/golden/make_golden.py

Every array here is an output of the reference's C++ (Scene::initialize /
FlatBVH::build, Camera::update, FlatBVH::intersect, Raytracer shadow rays,
Tracer::run + PathTracer + Film, ReinhardToneMapper, ValueNoise,
MathUtils::fastPow, CMJSampler) on seeded synthetic inputs; the tests compare
the oracle and the device against them where the reference is not available.
"""

from __future__ import annotations

import ctypes as C
import hashlib
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
from raycer_gb300 import scenes  # noqa: E402

OUT = Path(__file__).resolve().parent


def ptr(a):
    return C.c_void_p(a.ctypes.data)


def bvh_digest(nodes: np.ndarray, order: np.ndarray) -> dict:
    nodes = np.ascontiguousarray(nodes, oracle.NODE_DTYPE)
    order = np.ascontiguousarray(order, np.uint64)
    return {
        "node_count": int(nodes.shape[0]),
        "nodes_sha256": hashlib.sha256(nodes.tobytes()).hexdigest(),
        "order_sha256": hashlib.sha256(order.tobytes()).hexdigest(),
    }


def camera_ray_set(cam_state: np.ndarray, width: int, height: int, stride: int):
    """float32 primary rays (the device's camera formula) at a strided pixel set."""
    cam = np.concatenate([cam_state[:18]]).astype(np.float32)
    ys, xs = np.meshgrid(np.arange(0, height, stride), np.arange(0, width, stride), indexing="ij")
    pix = (ys * width + xs).ravel().astype(np.int64)
    allr = oracle.camera_rays32(cam, width, width * height)
    return pix, allr[pix]


def main() -> None:
    lib = oracle.ref_lib()
    meta = {}

    # -- room: BVH, camera, primary hits, path-traced image statistics -----
    room = scenes.room_scene()
    ref = oracle.RefScene(room)
    nodes, order = ref.bvh()
    cs_room = ref.camera_state(room.width, room.height)
    pix, rays = camera_ray_set(cs_room, room.width, room.height, 2)
    r6 = np.concatenate([rays[:, 0:3], rays[:, 4:7]], axis=1).astype(np.float64)
    prim, t = ref.intersect(r6)
    meta["room_bvh"] = bvh_digest(nodes, order)

    # Path tracing at the 320x240 workload settings: 4x4 CMJ samples, box
    # filter, one path per sample, maxPathLength 4, Reinhard key 0.18, gamma 2.2.
    # K independent renders; per 8x8 block (and for the whole image) the mean
    # over renders and the variance of one render's block mean across renders.
    ref.set_general(1, 4, 1, 4, sampler=4, filt=0, offset=1e-5)
    ref.set_tonemapper(3, True, True, 2.2, 0.18)
    K = 16
    H, W, B = room.height, room.width, 8
    block_runs = []
    image_runs = []
    rays_per_run = []
    for _ in range(K):
        lin, tm, nrays, _sec = ref.render(room.width, room.height, threads=0)
        img = lin[:, :3].astype(np.float64).reshape(H, W, 3)
        block_runs.append(img.reshape(H // B, B, W // B, B, 3).mean(axis=(1, 3)))
        image_runs.append(img.mean(axis=(0, 1)))
        rays_per_run.append(nrays)
    block_runs = np.stack(block_runs)
    image_runs = np.stack(image_runs)
    np.savez_compressed(
        OUT / "room.npz",
        nodes=nodes, order=order, camera_state=cs_room,
        hit_pixels=pix, hit_prim=prim.astype(np.int32), hit_t=t.astype(np.float32),
        pt_runs=np.int32(K),
        pt_block_mean=block_runs.mean(axis=0), pt_block_var=block_runs.var(axis=0, ddof=1),
        pt_mean=image_runs.mean(axis=0), pt_mean_var=image_runs.var(axis=0, ddof=1),
        pt_rays_per_run=np.array(rays_per_run, np.uint64),
        pt_tonemapped_last=tm.reshape(H, W, 4)[..., :3].astype(np.float16),
    )

    # -- heightfield (1,045,506 triangles): BVH digest, camera, hits, shadows --
    hf = scenes.heightfield_scene()
    refh = oracle.RefScene(hf)
    hn, ho = refh.bvh()
    meta["heightfield_bvh"] = bvh_digest(hn, ho)
    meta["heightfield_triangles"] = hf.triangle_count
    cs_hf = refh.camera_state(hf.width, hf.height)
    pix, rays = camera_ray_set(cs_hf, hf.width, hf.height, 8)
    r6 = np.concatenate([rays[:, 0:3], rays[:, 4:7]], axis=1).astype(np.float64)
    prim, t = refh.intersect(r6)
    # The reference's own shadow query from its float64 hit position
    # (Raytracer::calculateShadowAmount: origin = p + L * rayStartOffset).
    L = -np.array(hf.light_direction, np.float64)
    hitm = prim >= 0
    pos = r6[:, 0:3] + t[:, None] * r6[:, 3:6]
    srays = np.concatenate([pos + L[None, :] * 1e-5, np.broadcast_to(L, pos.shape)], axis=1)
    sprim, _ = refh.intersect(srays, shadow=True)
    occluded = hitm & (sprim >= 0)
    np.savez_compressed(
        OUT / "heightfield.npz",
        camera_state=cs_hf, hit_pixels=pix, hit_prim=prim.astype(np.int32), hit_t=t.astype(np.float32),
        occluded=occluded,
    )
    # small heightfield: full node arrays
    hs = scenes.heightfield_scene(nx=64, nz=32, width=160, height=90)
    refs = oracle.RefScene(hs)
    sn, so = refs.bvh()
    np.savez_compressed(OUT / "heightfield_small.npz", nodes=sn, order=so,
                        camera_state=refs.camera_state(hs.width, hs.height))

    # -- camera poses --------------------------------------------------------
    poses = []
    states = []
    rng = np.random.default_rng(3)
    for _ in range(32):
        pos = rng.uniform(-10, 10, 3)
        pitch, yaw, roll = rng.uniform(-120, 120), rng.uniform(-400, 400), 0.0
        fov = rng.uniform(10, 170)
        w, h = int(rng.integers(2, 4000)), int(rng.integers(2, 3000))
        sc = scenes.SceneDesc("pose", np.zeros((1, 9)), np.zeros(1, np.uint32), [scenes.Material()],
                              scenes.CameraDesc(tuple(pos), pitch, yaw, roll, fov), w, h)
        rs = oracle.RefScene(sc, init=False)
        states.append(rs.camera_state(w, h))
        poses.append([*pos, pitch, yaw, roll, fov, w, h])
    np.savez_compressed(OUT / "camera_poses.npz", poses=np.array(poses), states=np.array(states))

    # -- tone mapping ----------------------------------------------------------
    rng = np.random.default_rng(4)
    n = 4096
    lin = np.zeros((n, 4), np.float32)
    lin[:, :3] = rng.exponential(0.3, size=(n, 3)).astype(np.float32)
    lin[::97, :3] = 0.0                      # black pixels: 0/0 luminance scale
    lin[5::101, :3] *= 40.0                  # very bright pixels
    lin[:, 3] = 1.0
    outs = {}
    for key, gamma, clamp, ag in [(0.18, 2.2, 1, 1), (0.5, 1.8, 1, 1), (0.18, 2.2, 0, 1), (0.18, 2.2, 1, 0)]:
        o = np.empty_like(lin)
        lib.ref_tonemap_reinhard(n, ptr(lin), key, gamma, clamp, ag, ptr(o))
        outs[f"out_{key}_{gamma}_{clamp}_{ag}"] = o
    np.savez_compressed(OUT / "tonemap.npz", linear=lin, **outs)

    # -- value noise, fastPow, CMJ ---------------------------------------------
    rng = np.random.default_rng(5)
    pts = rng.uniform(-40, 40, size=(3000, 3))
    pts[:1500, 1] = 0.0
    fbm = np.empty(3000)
    n3 = np.empty(3000)
    lib.ref_value_noise(2, 3000, ptr(np.ascontiguousarray(pts)), 6, 2.0, 0.5, ptr(fbm))
    lib.ref_value_noise(11, 3000, ptr(np.ascontiguousarray(pts)), 0, 2.0, 0.5, ptr(n3))
    xs = np.concatenate([np.linspace(0, 1, 1001), rng.uniform(0, 50, 500), [0.0, 1e-300, 1e-12]])
    fp = np.array([lib.ref_fastpow(float(x), 1.0 / 2.2) for x in xs])
    fp2 = np.array([lib.ref_fastpow(float(x), 1.0 / 1.8) for x in xs])
    cmj = []
    for (nn, perm, seed) in [(4, 0, 1), (4, 12345678901234567, 2), (3, 987654321, 3), (8, 2**63 + 5, 4),
                             (5, 42, 5)]:
        out = np.empty(nn * nn * 2)
        jit = np.empty(nn * nn * 2)
        lib.ref_cmj_pattern(nn, perm, seed, ptr(out), ptr(jit))
        cmj.append((nn, perm, out, jit))
    np.savez_compressed(
        OUT / "math.npz", noise_points=pts, fbm_seed2=fbm, noise_seed11=n3, fastpow_x=xs, fastpow_inv22=fp,
        fastpow_inv18=fp2,
        cmj_n=np.array([c[0] for c in cmj]), cmj_perm=np.array([c[1] for c in cmj], np.uint64),
        **{f"cmj_out_{i}": c[2] for i, c in enumerate(cmj)}, **{f"cmj_jit_{i}": c[3] for i, c in enumerate(cmj)},
    )

    (OUT / "golden.json").write_text(json.dumps(meta, indent=1, sort_keys=True) + "\n")
    print("golden fixtures written:", sorted(p.name for p in OUT.iterdir()))


INSTANCED = dict(instances=24, blob_level=3, hf_nx=128, hf_nz=64, width=160, height=90, seed=4)


def instanced_golden() -> None:
    """The reference's own Instance / PrimitiveGroup traversal (Instance.cpp,
    PrimitiveGroup.cpp) on a small heightfield + blob-instances scene: mesh
    and mesh-local triangle of every camera ray's closest hit, and its
    distance. The scene is regenerated from its seeds by the tests."""
    sc = scenes.heightfield_blobs_instanced(**INSTANCED)
    ref = oracle.RefScene(sc)
    state = ref.camera_state(sc.width, sc.height)
    pix, rays = camera_ray_set(state, sc.width, sc.height, 1)
    r32 = np.ascontiguousarray(rays).view(np.float32).reshape(-1, 8)
    rays6 = np.concatenate([r32[:, 0:3], r32[:, 4:7]], axis=1).astype(np.float64)
    prim, t = ref.intersect(rays6)
    mesh = np.where(prim >= 0, prim // oracle.RefScene.MESH_ID, -1)
    local = np.where(prim >= 0, prim % oracle.RefScene.MESH_ID, -1)
    np.savez_compressed(OUT / "instanced.npz", camera_state=state, rays=r32, mesh=mesh.astype(np.int32),
                        local=local.astype(np.int32), t=t)
    print("instanced fixture written:", int((prim >= 0).sum()), "hits of", prim.size)


if __name__ == "__main__":
    if sys.argv[1:] == ["instanced"]:
        instanced_golden()
    else:
        main()
        instanced_golden()
