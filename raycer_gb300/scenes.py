"""Seeded synthetic scenes for the benchmark workloads.

No public dataset is involved: every scene is generated from a seed. Vertex
coordinates are computed in float64 and rounded to float32 (the workloads are
specified in float32), so the reference's float64 code and the device see the
same triangles.

* ``room_scene`` — 320x240 path-tracing workload: an axis-aligned room
  [-1,1]^3 (5 walls, 10 triangles, inward-facing), an emissive 0.5x0.5 ceiling
  quad 1e-3 below the ceiling (2 triangles, radiance 15), and 2,000 random
  clutter triangles (centres U[-0.8,0.8]^3, vertices at uniform unit
  directions scaled by U(0.05,0.2), diffuse albedo U(0.2,0.8)^3). Camera at
  (0,0,3.5) looking down -z, 45 degree horizontal field of view.
* ``heightfield_scene`` — 1920x1080 ray-casting workload: a 1024x512-vertex
  grid over x in [-10,10], z in [-5,5] (2*1023*511 = 1,045,506 triangles),
  height 1.5 * fBm(6 octaves, lacunarity 2, gain 0.5) of the reference's value
  noise with seed 2 (ValueNoise::getNoise / getFbmNoise,
  src/Utils/ValueNoise.cpp:26-97), one directional light toward
  normalize(0.3,1,0.2), camera at (0,4,12) aimed at the origin.

Random draws for the room come from Python's ``random.Random`` (Mersenne
Twister, documented as reproducible for a given seed). The value noise
restates the reference: each lattice corner seeds a std::mt19937 with
``uint32(seed*16381 + x*17389 + y*18313 + z*19423)`` and takes its first
``uniform_real_distribution<double>(0,1)`` draw, i.e. libstdc++'s
generate_canonical<double, 53> over two 32-bit outputs; the needed outputs of
a freshly seeded generator are computed directly (vectorised), which gives the
same numbers as seeding a generator per corner.
"""

from __future__ import annotations

import math
import random
from dataclasses import dataclass, field

import numpy as np

# ---------------------------------------------------------------------------
# Scene description (plain arrays; what rc_upload_scene consumes).


@dataclass
class Material:
    diffuse: tuple = (0.0, 0.0, 0.0)
    emittance: tuple = (0.0, 0.0, 0.0)
    is_emissive: bool = False
    non_shadowing: bool = False
    invert_normal: bool = False
    dielectric: bool = False   # GPU extension: smooth dielectric (Fresnel, refraction)
    ior: float = 0.0


@dataclass
class CameraDesc:
    position: tuple = (0.0, 0.0, 0.0)
    pitch: float = 0.0
    yaw: float = 0.0
    roll: float = 0.0
    fov: float = 75.0


@dataclass
class SceneDesc:
    name: str
    vertices: np.ndarray          # (n, 9) float64, float32-exact values
    material_index: np.ndarray    # (n,) uint32
    materials: list               # [Material]
    camera: CameraDesc
    width: int
    height: int
    light_direction: tuple | None = None   # DirectionalLight.direction (travel direction)
    max_leaf_size: int = 4
    settings: dict = field(default_factory=dict)

    @property
    def triangle_count(self) -> int:
        return int(self.vertices.shape[0])


def _f32(a: np.ndarray) -> np.ndarray:
    return np.asarray(a, dtype=np.float64).astype(np.float32).astype(np.float64)


# ---------------------------------------------------------------------------
# Room (path tracing).


def _quad(p0, u, v):
    p0, u, v = map(np.asarray, (p0, u, v))
    a, b, c, d = p0, p0 + u, p0 + u + v, p0 + v
    return [np.concatenate([a, b, c]), np.concatenate([a, c, d])]


def room_scene(seed: int = 1, clutter: int = 2000, width: int = 320, height: int = 240) -> SceneDesc:
    rng = random.Random(seed)
    tris = []
    mats = [
        Material(diffuse=(0.75, 0.75, 0.75)),
        Material(diffuse=(0.75, 0.25, 0.25)),
        Material(diffuse=(0.25, 0.75, 0.25)),
        Material(diffuse=(0.0, 0.0, 0.0), emittance=(15.0, 15.0, 15.0), is_emissive=True),
    ]
    midx = []
    # Walls: (p0, u, v) with u x v pointing into the room.
    walls = [
        ((-1, -1, -1), (0, 0, 2), (2, 0, 0), 0),   # floor, +y
        ((-1, 1, -1), (2, 0, 0), (0, 0, 2), 0),    # ceiling, -y
        ((-1, -1, -1), (2, 0, 0), (0, 2, 0), 0),   # back, +z
        ((-1, -1, -1), (0, 2, 0), (0, 0, 2), 1),   # left, +x
        ((1, -1, -1), (0, 0, 2), (0, 2, 0), 2),    # right, -x
    ]
    for p0, u, v, m in walls:
        for t in _quad(np.array(p0, float), np.array(u, float), np.array(v, float)):
            tris.append(t)
            midx.append(m)
    for t in _quad(np.array([-0.25, 1.0 - 1e-3, -0.25]), np.array([0.5, 0.0, 0.0]), np.array([0.0, 0.0, 0.5])):
        tris.append(t)
        midx.append(3)
    for _ in range(clutter):
        c = np.array([rng.uniform(-0.8, 0.8) for _ in range(3)])
        verts = []
        for _k in range(3):
            z = rng.uniform(-1.0, 1.0)
            phi = rng.uniform(0.0, 2.0 * math.pi)
            r = math.sqrt(max(0.0, 1.0 - z * z))
            d = np.array([r * math.cos(phi), r * math.sin(phi), z])
            s = rng.uniform(0.05, 0.2)
            verts.append(c + d * s)
        albedo = tuple(float(np.float32(rng.uniform(0.2, 0.8))) for _ in range(3))
        mats.append(Material(diffuse=albedo))
        tris.append(np.concatenate(verts))
        midx.append(len(mats) - 1)
    v = _f32(np.array(tris))
    return SceneDesc(
        name=f"room(seed={seed}, clutter={clutter})",
        vertices=v,
        material_index=np.array(midx, dtype=np.uint32),
        materials=mats,
        camera=CameraDesc(position=(0.0, 0.0, 3.5), pitch=0.0, yaw=0.0, roll=0.0, fov=45.0),
        width=width,
        height=height,
        light_direction=None,
        max_leaf_size=4,
        settings=dict(tracer="path", max_path_length=4, multi_sample_count_sqrt=4, path_sample_count=1,
                      sampler="cmj", filter="box", tonemap="reinhard", key=0.18, gamma=2.2),
    )


# ---------------------------------------------------------------------------
# Value noise (src/Utils/ValueNoise.cpp restated, vectorised).

_MT_MULT = np.uint64(1812433253)
_MASK32 = np.uint64(0xFFFFFFFF)


def _mt19937_first_two(seeds: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """First two outputs of std::mt19937(seed) for an array of uint32 seeds."""
    s = seeds.astype(np.uint64)
    need = {0, 1, 2, 397, 398}
    state = {0: s}
    prev = s
    for i in range(1, 399):
        prev = (_MT_MULT * (prev ^ (prev >> np.uint64(30))) + np.uint64(i)) & _MASK32
        if i in need:
            state[i] = prev
    upper = np.uint64(0x80000000)
    lower = np.uint64(0x7FFFFFFF)
    mag = np.uint64(0x9908B0DF)
    outs = []
    for k in (0, 1):
        y = (state[k] & upper) | (state[k + 1] & lower)
        x = state[k + 397] ^ (y >> np.uint64(1)) ^ np.where((y & np.uint64(1)) != 0, mag, np.uint64(0))
        x = x ^ (x >> np.uint64(11))
        x = x ^ ((x << np.uint64(7)) & np.uint64(0x9D2C5680))
        x = x ^ ((x << np.uint64(15)) & np.uint64(0xEFC60000))
        x = x ^ (x >> np.uint64(18))
        outs.append(x & _MASK32)
    return outs[0], outs[1]


def _canonical(seeds: np.ndarray) -> np.ndarray:
    """uniform_real_distribution<double>(0, 1) first draw of mt19937(seed)."""
    o0, o1 = _mt19937_first_two(seeds)
    r = (o0.astype(np.float64) + o1.astype(np.float64) * 4294967296.0) / 18446744073709551616.0
    return np.where(r >= 1.0, np.nextafter(1.0, 0.0), r)


def _hash(seed: int, x: np.ndarray, y: np.ndarray, z: np.ndarray) -> np.ndarray:
    # ValueNoise::getHashcode: uint32((seed*16381) + x*17389 + y*18313 + z*19423)
    h = (np.int64(seed) * 16381) + x * 17389 + y * 18313 + z * 19423
    return (h & 0xFFFFFFFF).astype(np.uint64)


def value_noise(seed: int, x: np.ndarray, y: np.ndarray, z: np.ndarray) -> np.ndarray:
    """ValueNoise(seed).getNoise(x, y, z) for arrays of points."""
    x = np.asarray(x, np.float64)
    y = np.asarray(y, np.float64)
    z = np.asarray(z, np.float64)
    ix = np.floor(x).astype(np.int64)
    iy = np.floor(y).astype(np.int64)
    iz = np.floor(z).astype(np.int64)
    tx = x - ix
    ty = y - iy
    tz = z - iz
    txi = 1.0 - tx
    tyi = 1.0 - ty
    tzi = 1.0 - tz
    corners = {}
    keys = []
    for dx in (0, 1):
        for dy in (0, 1):
            for dz in (0, 1):
                keys.append(_hash(seed, ix + dx, iy + dy, iz + dz))
    allk = np.concatenate(keys)
    uniq, inv = np.unique(allk, return_inverse=True)
    vals = _canonical(uniq)[inv].reshape(8, -1)
    i = 0
    for dx in (0, 1):
        for dy in (0, 1):
            for dz in (0, 1):
                corners[(dx, dy, dz)] = vals[i]
                i += 1
    c00 = corners[0, 0, 0] * txi + corners[1, 0, 0] * tx
    c01 = corners[0, 0, 1] * txi + corners[1, 0, 1] * tx
    c10 = corners[0, 1, 0] * txi + corners[1, 1, 0] * tx
    c11 = corners[0, 1, 1] * txi + corners[1, 1, 1] * tx
    c0 = c00 * tyi + c10 * ty
    c1 = c01 * tyi + c11 * ty
    c = c0 * tzi + c1 * tz
    return np.maximum(0.0, np.minimum(c, 1.0))


def fbm_noise(seed: int, octaves: int, lacunarity: float, persistence: float, x, y, z) -> np.ndarray:
    """ValueNoise::getFbmNoise (ValueNoise.cpp:78-92)."""
    x = np.asarray(x, np.float64)
    y = np.asarray(y, np.float64)
    z = np.asarray(z, np.float64)
    result = np.zeros_like(x)
    frequency = 1.0
    amplitude = 1.0
    for _ in range(octaves):
        result = result + value_noise(seed, x * frequency, y * frequency, z * frequency) * amplitude
        frequency *= lacunarity
        amplitude *= persistence
    return result


# ---------------------------------------------------------------------------
# Heightfield (ray casting).


def heightfield_scene(seed: int = 2, nx: int = 1024, nz: int = 512, width: int = 1920, height: int = 1080,
                      extent=(-10.0, 10.0, -5.0, 5.0), amplitude: float = 1.5) -> SceneDesc:
    x0, x1, z0, z1 = extent
    xs = x0 + (x1 - x0) * np.arange(nx, dtype=np.float64) / (nx - 1)
    zs = z0 + (z1 - z0) * np.arange(nz, dtype=np.float64) / (nz - 1)
    X, Z = np.meshgrid(xs, zs, indexing="xy")          # (nz, nx)
    Y = amplitude * fbm_noise(seed, 6, 2.0, 0.5, X.ravel(), np.zeros(X.size), Z.ravel()).reshape(X.shape)
    P = np.stack([X, Y, Z], axis=-1)                     # (nz, nx, 3)
    a = P[:-1, :-1]   # (j, i)
    b = P[:-1, 1:]    # (j, i+1)
    c = P[1:, :-1]    # (j+1, i)
    d = P[1:, 1:]     # (j+1, i+1)
    # Two triangles per cell, upward geometric normals: (a, c, b) and (b, c, d).
    t1 = np.concatenate([a, c, b], axis=-1).reshape(-1, 9)
    t2 = np.concatenate([b, c, d], axis=-1).reshape(-1, 9)
    tris = np.stack([t1, t2], axis=1).reshape(-1, 9)
    v = _f32(tris)
    pitch = -math.degrees(math.atan(4.0 / 12.0))
    ld = np.array([0.3, 1.0, 0.2])
    ld = ld / np.linalg.norm(ld)
    return SceneDesc(
        name=f"heightfield(seed={seed}, {nx}x{nz} vertices)",
        vertices=v,
        material_index=np.zeros(v.shape[0], dtype=np.uint32),
        materials=[Material(diffuse=(0.8, 0.8, 0.8))],
        camera=CameraDesc(position=(0.0, 4.0, 12.0), pitch=pitch, yaw=0.0, roll=0.0, fov=45.0),
        width=width,
        height=height,
        light_direction=tuple(float(c) for c in -ld),
        max_leaf_size=4,
        settings=dict(tracer="ray"),
    )


def heightfield_path_scene(width: int = 1920, height: int = 1080, max_path_length: int = 4,
                           panel_height: float = 30.0, panel_half: float = 400.0, radiance: float = 1.0,
                           **kw) -> SceneDesc:
    """The 1,045,506-triangle heightfield path traced with the reference's
    estimator. The heightfield has no emitter and PathTracer::traceRecursive
    collects emission only (PathTracer.cpp:25-75; its directional light does
    nothing there), so a large emissive quad of `radiance` faces down from
    `panel_height` over the terrain (2 triangles): paths that leave the
    terrain upwards end on it, as under an overcast sky. One camera ray per
    pixel (multiSampleCountSqrt 1: the pixel centre, Tracer.cpp:119-123),
    `max_path_length` segments, box filter."""
    sc = heightfield_scene(width=width, height=height, **kw)
    y, r = float(panel_height), float(panel_half)
    # winding (v1 - v0) x (v2 - v0) = -y: the panel faces the terrain
    panel = np.array([[-r, y, -r, r, y, -r, r, y, r],
                      [-r, y, -r, r, y, r, -r, y, r]], np.float64)
    sc.vertices = np.concatenate([sc.vertices, _f32(panel)])
    sc.materials = list(sc.materials) + [Material(emittance=(radiance, radiance, radiance), is_emissive=True)]
    sc.material_index = np.concatenate([sc.material_index, np.full(2, len(sc.materials) - 1, np.uint32)])
    sc.name = sc.name + " + emissive sky panel"
    sc.settings = dict(tracer="path", max_path_length=int(max_path_length), multi_sample_count_sqrt=1,
                       path_sample_count=1, filter="box")
    return sc


# ---------------------------------------------------------------------------
# Batch of rooms (batched path tracing).


def room_with_extra(seed: int, extra: int, width: int, height: int, ms_sqrt: int, max_path_length: int = 8,
                    rr_depth: int = 3, palette: int = 256) -> SceneDesc:
    """The 320x240 workload's room (seed `seed`) plus `extra` random triangles
    drawn like its clutter (centres U[-0.8,0.8]^3, vertices at uniform unit
    directions scaled by U(0.05,0.2)); the extra triangles take their albedo
    U(0.2,0.8)^3 from a palette of `palette` materials. numpy PCG64 stream of
    uniform doubles only."""
    base = room_scene(seed=seed, width=width, height=height)
    rng = np.random.Generator(np.random.PCG64(seed))
    if extra > 0:
        c = -0.8 + 1.6 * rng.random((extra, 1, 3))
        z = -1.0 + 2.0 * rng.random((extra, 3))
        phi = 2.0 * math.pi * rng.random((extra, 3))
        r = np.sqrt(np.maximum(0.0, 1.0 - z * z))
        d = np.stack([r * np.cos(phi), r * np.sin(phi), z], axis=-1)
        sc = 0.05 + 0.15 * rng.random((extra, 3, 1))
        v = _f32((c + d * sc).reshape(extra, 9))
        albedo = (0.2 + 0.6 * rng.random((palette, 3))).astype(np.float32).astype(np.float64)
        first = len(base.materials)
        mats = base.materials + [Material(diffuse=tuple(float(x) for x in a)) for a in albedo]
        midx = first + (rng.random(extra) * palette).astype(np.uint32).clip(0, palette - 1)
        base.vertices = np.concatenate([base.vertices, v])
        base.material_index = np.concatenate([base.material_index, midx.astype(np.uint32)])
        base.materials = mats
    base.name = f"room(seed={seed})+{extra} tris {width}x{height} {ms_sqrt * ms_sqrt} spp"
    base.settings.update(multi_sample_count_sqrt=ms_sqrt, max_path_length=max_path_length,
                         russian_roulette_depth=rr_depth)
    return base


def batch_scenes(seed: int = 3, count: int = 64, n_min: float = 1e3, n_max: float = 2e6,
                 resolutions=(256, 512, 768, 1024), spps=(1, 4, 16, 64)) -> list:
    """The batched workload: `count` rooms, each with N log-uniform in
    [n_min, n_max] extra random triangles, square film size uniform over
    `resolutions`, samples per pixel uniform over `spps` (as n x n CMJ film
    samples), maximum path length 8 with Russian roulette from segment 3."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for i in range(count):
        u = rng.random(3)
        n = int(round(math.exp(math.log(n_min) + u[0] * (math.log(n_max) - math.log(n_min)))))
        res = resolutions[min(int(u[1] * len(resolutions)), len(resolutions) - 1)]
        spp = spps[min(int(u[2] * len(spps)), len(spps) - 1)]
        ms = int(round(math.sqrt(spp)))
        out.append(room_with_extra(seed * 1000 + i, n, res, res, ms))
    return out


# ---------------------------------------------------------------------------
# Heightfield + instanced blobs (radiance-cache workload).


def icosphere(level: int) -> np.ndarray:
    """Unit icosphere triangles (20 * 4^level, each 9 floats, outward winding)."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
             (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
             (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
             (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    v = np.array(verts, np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    tris = v[np.array(faces)]                        # (F, 3, 3)
    for _ in range(level):
        a, b, c = tris[:, 0], tris[:, 1], tris[:, 2]
        ab = a + b
        bc = b + c
        ca = c + a
        ab /= np.linalg.norm(ab, axis=1, keepdims=True)
        bc /= np.linalg.norm(bc, axis=1, keepdims=True)
        ca /= np.linalg.norm(ca, axis=1, keepdims=True)
        tris = np.concatenate([np.stack([a, ab, ca], 1), np.stack([ab, b, bc], 1), np.stack([ca, bc, c], 1),
                               np.stack([ab, bc, ca], 1)])
    return tris.reshape(-1, 9)


def blob_mesh(seed: int = 5, level: int = 5, amplitude: float = 0.35) -> np.ndarray:
    """A random blob: an icosphere (20 * 4^level triangles; level 5 = 20,480)
    whose vertices move radially by a 3-octave value-noise field."""
    tris = icosphere(level).reshape(-1, 3)
    n = fbm_noise(seed, 3, 2.0, 0.5, tris[:, 0] * 1.7 + 11.0, tris[:, 1] * 1.7 + 13.0, tris[:, 2] * 1.7 + 17.0)
    r = 1.0 + amplitude * (n / 1.75 - 0.5)
    return (tris * r[:, None]).reshape(-1, 9)


def _random_rotations(rng, count):
    u1, u2, u3 = rng.random(count), rng.random(count), rng.random(count)
    # uniform unit quaternions (Shoemake)
    a = np.sqrt(1 - u1)
    b = np.sqrt(u1)
    w, x = a * np.sin(2 * math.pi * u2), a * np.cos(2 * math.pi * u2)
    y, z = b * np.sin(2 * math.pi * u3), b * np.cos(2 * math.pi * u3)
    R = np.empty((count, 3, 3))
    R[:, 0, 0] = 1 - 2 * (y * y + z * z)
    R[:, 0, 1] = 2 * (x * y - z * w)
    R[:, 0, 2] = 2 * (x * z + y * w)
    R[:, 1, 0] = 2 * (x * y + z * w)
    R[:, 1, 1] = 1 - 2 * (x * x + z * z)
    R[:, 1, 2] = 2 * (y * z - x * w)
    R[:, 2, 0] = 2 * (x * z - y * w)
    R[:, 2, 1] = 2 * (y * z + x * w)
    R[:, 2, 2] = 1 - 2 * (x * x + y * y)
    return R


def _enclosing_box(panel, panel_radiance):
    """The closed box around the heightfield scenes (x -14..14, y -1..8, z
    -8..14, inward-facing walls of albedo 0.75) and an emissive panel
    (width x depth, centred) facing down just under the ceiling: triangles
    (12 + 2, float32-exact) with material indices 0 (walls) and 1 (panel),
    and those two materials."""
    x0, x1, y0, y1, z0, z1 = -14.0, 14.0, -1.0, 8.0, -8.0, 14.0
    # (p0, u, v) with u x v pointing into the box, as room_scene's walls
    dx, dy, dz = x1 - x0, y1 - y0, z1 - z0
    walls = np.concatenate([
        _quad((x0, y0, z0), (0, 0, dz), (dx, 0, 0)),   # floor, +y
        _quad((x0, y1, z0), (dx, 0, 0), (0, 0, dz)),   # ceiling, -y
        _quad((x0, y0, z0), (dx, 0, 0), (0, dy, 0)),   # back, +z
        _quad((x0, y0, z1), (0, dy, 0), (dx, 0, 0)),   # front (behind the camera), -z
        _quad((x0, y0, z0), (0, dy, 0), (0, 0, dz)),   # left, +x
        _quad((x1, y0, z0), (0, 0, dz), (0, dy, 0)),   # right, -x
    ])
    pw, pd = float(panel[0]), float(panel[1])
    quad = np.array(_quad((-0.5 * pw, y1 - 0.01, -0.5 * pd), (pw, 0, 0), (0, 0, pd)))  # facing down, -y
    le = float(panel_radiance)
    mats = [Material(diffuse=(0.75, 0.75, 0.75)),
            Material(diffuse=(0.0, 0.0, 0.0), emittance=(le, le, le), is_emissive=True)]
    verts = np.concatenate([_f32(walls), _f32(quad)])
    midx = np.concatenate([np.zeros(walls.shape[0], np.uint32), np.ones(quad.shape[0], np.uint32)])
    return (verts, midx), mats


def heightfield_blobs_scene(instances: int = 200, blob_level: int = 5, seed: int = 4, hf_nx: int = 1024,
                            hf_nz: int = 512, width: int = 1920, height: int = 1080,
                            sky=(1.0, 1.0, 1.0), enclosed: bool = False, panel=(20.0, 11.0),
                            panel_radiance: float = 3.0) -> SceneDesc:
    """The radiance-cache workload: the 1,045,506-triangle heightfield (value
    noise seed 2) plus `instances` copies of one 20,480-triangle random blob at
    uniform random positions over the terrain, uniform random rotations,
    scale U(0.25, 0.6) and albedo U(0.1, 0.9)^3, flattened to world-space
    triangles. Lit by a uniform sky: a path that escapes returns `sky`.

    enclosed=True: the same geometry inside a closed box (x -14..14, y -1..8,
    z -8..14, inward-facing walls of albedo 0.75, the camera inside) lit by an
    emissive `panel` (width x depth, centred; 20 x 11 by default, a third of
    the ceiling) of radiance `panel_radiance` (3) just under the ceiling, and
    no sky: every path runs to the depth limit unless it reaches the panel."""
    hf = heightfield_scene(seed=2, nx=hf_nx, nz=hf_nz, width=width, height=height)
    blob = blob_mesh(seed=seed, level=blob_level).reshape(-1, 3, 3)
    rng = np.random.Generator(np.random.PCG64(seed))
    R = _random_rotations(rng, instances)
    px = -9.0 + 18.0 * rng.random(instances)
    pz = -4.5 + 9.0 * rng.random(instances)
    scale = 0.25 + 0.35 * rng.random(instances)
    albedo = (0.1 + 0.8 * rng.random((instances, 3))).astype(np.float32).astype(np.float64)
    # terrain height under each instance, from the vertex grid
    g = hf.vertices.reshape(hf_nz - 1, hf_nx - 1, 2, 9)[:, :, 0, 0:3]   # first vertex of each cell's first tri
    ix = np.clip(((px + 10.0) / 20.0 * (hf_nx - 1)).astype(int), 0, hf_nx - 2)
    iz = np.clip(((pz + 5.0) / 10.0 * (hf_nz - 1)).astype(int), 0, hf_nz - 2)
    py = g[iz, ix, 1] + scale * 0.6
    world = np.einsum("kij,tvj->ktvi", R, blob) * scale[:, None, None, None]
    world += np.stack([px, py, pz], axis=1)[:, None, None, :]
    bv = _f32(world.reshape(-1, 9))
    mats = [Material(diffuse=(0.6, 0.6, 0.6))] + [Material(diffuse=tuple(float(c) for c in a)) for a in albedo]
    midx = np.concatenate([np.zeros(hf.triangle_count, np.uint32),
                           np.repeat(np.arange(1, instances + 1, dtype=np.uint32), blob.shape[0])])
    verts = np.concatenate([hf.vertices, bv])
    name = f"heightfield + {instances} blobs x {blob.shape[0]} tris"
    if enclosed:
        (bv, bm), box_mats = _enclosing_box(panel, panel_radiance)
        first = len(mats)
        mats = mats + box_mats
        verts = np.concatenate([verts, bv])
        midx = np.concatenate([midx, bm + np.uint32(first)])
        name += ", enclosed, emissive panel"
    return SceneDesc(
        name=name,
        vertices=verts,
        material_index=midx,
        materials=mats,
        camera=hf.camera,
        width=width,
        height=height,
        light_direction=None,
        max_leaf_size=4,
        settings=dict(tracer="path", max_path_length=12, multi_sample_count_sqrt=1, path_sample_count=1,
                      sampler="cmj", miss_radiance=None if enclosed else tuple(sky)),
    )


# ---------------------------------------------------------------------------
# Instanced (two-level) scenes.


@dataclass
class InstanceDesc:
    """Instance (Instance.h:33-44): a placed copy of a mesh."""
    mesh: int
    material: int = -1                  # changePrimitive material, or -1: the mesh's own
    scale: tuple = (1.0, 1.0, 1.0)
    rotate: tuple = (0.0, 0.0, 0.0)     # pitch, yaw, roll in degrees (rotateXYZ)
    translate: tuple = (0.0, 0.0, 0.0)


@dataclass
class InstancedScene:
    name: str
    meshes: list                        # [(vertices (n, 9) float64, material_index (n,) uint32)]
    instances: list                     # [InstanceDesc]
    materials: list                     # [Material]
    camera: CameraDesc
    width: int
    height: int
    light_direction: tuple | None = None
    max_leaf_size: int = 4
    settings: dict = field(default_factory=dict)

    @property
    def triangle_count(self) -> int:
        """Triangles of the flattened scene."""
        return int(sum(self.meshes[i.mesh][0].shape[0] for i in self.instances))

    def flatten(self) -> SceneDesc:
        """The same scene as world-space triangles, instance by instance
        (the flattened primitive numbering of rc_upload_instanced)."""
        verts, mats = [], []
        for inst in self.instances:
            v, m = self.meshes[inst.mesh]
            M = instance_matrix(v, inst)
            p = v.reshape(-1, 3) @ M[:3, :3].T + M[:3, 3]
            verts.append(p.reshape(-1, 9))
            mats.append(np.full(v.shape[0], inst.material, np.uint32) if inst.material >= 0 else m)
        return SceneDesc(name=self.name + " (flattened)", vertices=np.concatenate(verts),
                         material_index=np.concatenate(mats).astype(np.uint32), materials=self.materials,
                         camera=self.camera, width=self.width, height=self.height,
                         light_direction=self.light_direction, max_leaf_size=self.max_leaf_size,
                         settings=dict(self.settings))


def _rot(axis: int, deg: float) -> np.ndarray:
    a = math.radians(deg)
    s, c = math.sin(a), math.cos(a)
    r = np.eye(4)
    i, j = [(1, 2), (0, 2), (0, 1)][axis]
    r[i, i] = c
    r[j, j] = c
    if axis == 1:   # rotateY: m[0][2] = s, m[2][0] = -s
        r[i, j], r[j, i] = s, -s
    else:           # rotateX / rotateZ: m[i][j] = -s, m[j][i] = s
        r[i, j], r[j, i] = -s, s
    return r


def instance_matrix(mesh_vertices: np.ndarray, inst: InstanceDesc) -> np.ndarray:
    """T(c + translate) * R_x R_y R_z * S(scale) * T(-c), c = the mesh box centre
    (Instance::initialize, Instance.cpp:17-32)."""
    p = mesh_vertices.reshape(-1, 3)
    c = (p.min(axis=0) + p.max(axis=0)) * 0.5
    t1 = np.eye(4)
    t1[:3, 3] = -c
    t2 = np.eye(4)
    t2[:3, 3] = c + np.asarray(inst.translate, np.float64)
    s = np.diag([*inst.scale, 1.0])
    r = _rot(0, inst.rotate[0]) @ _rot(1, inst.rotate[1]) @ _rot(2, inst.rotate[2])
    return t2 @ r @ s @ t1


def heightfield_blobs_instanced(instances: int = 200, blob_level: int = 5, seed: int = 4, hf_nx: int = 1024,
                                hf_nz: int = 512, width: int = 1920, height: int = 1080, sky=(1.0, 1.0, 1.0),
                                dielectric_fraction: float = 0.0, hf_seed: int = 2,
                                enclosed: bool = False, panel=(20.0, 11.0),
                                panel_radiance: float = 3.0) -> InstancedScene:
    """The heightfield (an identity instance of its own mesh) plus `instances`
    placed copies of one random blob: uniform positions over the terrain,
    Euler rotations U(0, 360)^3, uniform scale U(0.25, 0.6), each copy its
    own material (albedo U(0.1, 0.9)^3; a fraction of them dielectric with
    IOR U(1.3, 1.7)). Lit by a uniform sky, or (enclosed=True) by
    heightfield_blobs_scene's closed box and emissive ceiling panel, a third
    mesh with an identity instance."""
    hf = heightfield_scene(seed=hf_seed, nx=hf_nx, nz=hf_nz, width=width, height=height)
    blob = blob_mesh(seed=seed, level=blob_level)
    rng = np.random.Generator(np.random.PCG64(seed))
    px = -9.0 + 18.0 * rng.random(instances)
    pz = -4.5 + 9.0 * rng.random(instances)
    scale = 0.25 + 0.35 * rng.random(instances)
    rot = 360.0 * rng.random((instances, 3))
    albedo = (0.1 + 0.8 * rng.random((instances, 3))).astype(np.float32).astype(np.float64)
    glass = rng.random(instances) < dielectric_fraction
    ior = 1.3 + 0.4 * rng.random(instances)
    g = hf.vertices.reshape(hf_nz - 1, hf_nx - 1, 2, 9)[:, :, 0, 0:3]
    ix = np.clip(((px + 10.0) / 20.0 * (hf_nx - 1)).astype(int), 0, hf_nx - 2)
    iz = np.clip(((pz + 5.0) / 10.0 * (hf_nz - 1)).astype(int), 0, hf_nz - 2)
    py = g[iz, ix, 1] + scale * 0.6
    bp = blob.reshape(-1, 3)
    c = (bp.min(axis=0) + bp.max(axis=0)) * 0.5
    mats = [Material(diffuse=(0.6, 0.6, 0.6))]
    insts = [InstanceDesc(mesh=0)]
    for k in range(instances):
        mats.append(Material(diffuse=tuple(float(x) for x in albedo[k]), dielectric=bool(glass[k]),
                             ior=float(np.float32(ior[k])) if glass[k] else 0.0))
        insts.append(InstanceDesc(mesh=1, material=k + 1, scale=(float(scale[k]),) * 3,
                                  rotate=tuple(float(x) for x in rot[k]),
                                  translate=(float(px[k] - c[0]), float(py[k] - c[1]), float(pz[k] - c[2]))))
    meshes = [(hf.vertices, hf.material_index), (blob, np.zeros(blob.shape[0], np.uint32))]
    name = f"heightfield + {instances} blob instances"
    if enclosed:
        box, box_mats = _enclosing_box(panel, panel_radiance)
        first = len(mats)
        mats = mats + box_mats
        meshes.append((box[0], box[1] + np.uint32(first)))
        insts.append(InstanceDesc(mesh=2))
        name += ", enclosed, emissive panel"
    return InstancedScene(
        name=name, meshes=meshes, instances=insts, materials=mats, camera=hf.camera, width=width, height=height,
        light_direction=None, max_leaf_size=4,
        settings=dict(tracer="path", max_path_length=12, multi_sample_count_sqrt=1, path_sample_count=1,
                      sampler="cmj", miss_radiance=None if enclosed else tuple(sky)))
