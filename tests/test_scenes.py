"""Synthetic workload generators: sizes, float32 exactness, orientation, determinism."""

from __future__ import annotations

import numpy as np

from raycer_gb300 import scenes


def _normals(v):
    e1 = v[:, 3:6] - v[:, 0:3]
    e2 = v[:, 6:9] - v[:, 0:3]
    return np.cross(e1, e2)


def test_room_layout():
    s = scenes.room_scene()
    assert s.triangle_count == 10 + 2 + 2000
    assert np.array_equal(s.vertices, s.vertices.astype(np.float32).astype(np.float64))
    n = _normals(s.vertices[:12])
    inward = [(0, 1), (1, -1), (2, 1), (0, 1), (1, -1)]  # axis, sign per wall (2 tris each)
    for w, (axis, sign) in enumerate([(1, 1), (1, -1), (2, 1), (0, 1), (0, -1)]):
        for k in range(2):
            assert np.sign(n[2 * w + k, axis]) == sign
    assert np.all(n[10:12, 1] < 0)                     # emitter faces down
    assert s.materials[3].is_emissive and s.materials[3].emittance == (15.0, 15.0, 15.0)
    c = s.vertices[12:].reshape(-1, 3, 3).mean(axis=1)
    assert np.all(np.abs(c) < 1.0)
    alb = np.array([m.diffuse for m in s.materials[4:]])
    assert alb.min() >= 0.2 and alb.max() <= 0.8


def test_room_is_deterministic():
    a, b = scenes.room_scene(seed=1), scenes.room_scene(seed=1)
    assert np.array_equal(a.vertices, b.vertices)
    assert not np.array_equal(a.vertices, scenes.room_scene(seed=2).vertices)


def test_heightfield_layout():
    s = scenes.heightfield_scene(nx=64, nz=32)
    assert s.triangle_count == 2 * 63 * 31
    assert np.all(_normals(s.vertices)[:, 1] > 0)      # upward-facing
    x = s.vertices[:, 0::3]
    z = s.vertices[:, 2::3]
    assert x.min() == -10.0 and x.max() == 10.0 and z.min() == -5.0 and z.max() == 5.0
    y = s.vertices[:, 1::3]
    assert 0.0 <= y.min() and y.max() <= 1.5 * (1 + 0.5 + 0.25 + 0.125 + 0.0625 + 0.03125)
    ld = np.array(s.light_direction)
    assert np.allclose(-ld, np.array([0.3, 1.0, 0.2]) / np.linalg.norm([0.3, 1.0, 0.2]))


def test_enclosed_box_in_both_scene_forms():
    """The closed box and its ceiling panel: 12 wall triangles facing inward
    and 2 emissive panel triangles facing down, the same in the flat
    radiance-cache scene and as the identity-instanced third mesh of the
    combined-run scene."""
    import numpy as np

    from raycer_gb300 import scenes

    flat = scenes.heightfield_blobs_scene(instances=2, blob_level=1, hf_nx=8, hf_nz=4, enclosed=True)
    inst = scenes.heightfield_blobs_instanced(instances=2, blob_level=1, hf_nx=8, hf_nz=4, enclosed=True)
    for sc in (flat, inst.flatten()):
        v = sc.vertices[-14:].reshape(-1, 3, 3)
        mats = [sc.materials[i] for i in sc.material_index[-14:]]
        assert [m.is_emissive for m in mats] == [False] * 12 + [True] * 2
        n = np.cross(v[:, 1] - v[:, 0], v[:, 2] - v[:, 0])
        centre = v.mean(axis=1)
        inward = np.einsum("ij,ij->i", n[:12], np.array([0.0, 3.5, 3.0]) - centre[:12])
        assert (inward > 0).all()
        assert (n[12:, 1] < 0).all()          # the panel faces the floor
        assert sc.settings["miss_radiance"] is None
    assert inst.instances[-1].mesh == 2 and inst.instances[-1].material == -1
