"""Instanced scenes on the CPU: this package's flattening of an instanced
scene applies the reference's Instance transform, checked against the
reference's own Instance / PrimitiveGroup traversal (live where the
reference is built, and through the committed fixture everywhere)."""

from __future__ import annotations

import numpy as np
import pytest

import oracle
from raycer_gb300 import scenes

FIX = np.load(__import__("pathlib").Path(__file__).parent / "golden" / "instanced.npz")
PARAMS = dict(instances=24, blob_level=3, hf_nx=128, hf_nz=64, width=160, height=90, seed=4)


def flat_to_mesh(sc, prim):
    """Flattened primitive index -> (mesh, mesh-local triangle)."""
    counts = np.array([sc.meshes[d.mesh][0].shape[0] for d in sc.instances])
    base = np.concatenate([[0], np.cumsum(counts)])
    k = np.searchsorted(base, prim, side="right") - 1
    mesh = np.array([sc.instances[i].mesh for i in range(len(sc.instances))])[np.clip(k, 0, len(counts) - 1)]
    local = prim - base[np.clip(k, 0, len(counts) - 1)]
    return np.where(prim >= 0, mesh, -1), np.where(prim >= 0, local, -1)


def test_instance_matrix_composition():
    v = np.array([[0.0, 0, 0, 2, 0, 0, 0, 2, 0]])  # box centre (1, 1, 0)
    M = scenes.instance_matrix(v, scenes.InstanceDesc(mesh=0, scale=(2.0, 2.0, 2.0), rotate=(0.0, 90.0, 0.0),
                                                      translate=(0.0, 0.0, 5.0)))
    # the centre goes to centre + translate; rotateY(90) maps +x to -z
    np.testing.assert_allclose(M @ [1, 1, 0, 1], [1, 1, 5, 1], atol=1e-12)
    np.testing.assert_allclose(M[:3, :3] @ [1, 0, 0], [0, 0, -2], atol=1e-12)


def test_flattening_matches_fixture():
    sc = scenes.heightfield_blobs_instanced(**PARAMS)
    flat = sc.flatten()
    orc = oracle.Oracle(flat)
    r32 = FIX["rays"]
    rays6 = np.concatenate([r32[:, 0:3], r32[:, 4:7]], axis=1).astype(np.float64)
    prim, t, _, _ = orc.intersect64(rays6)
    mesh, local = flat_to_mesh(sc, prim)
    same = (mesh == FIX["mesh"]) & (local == FIX["local"])
    assert same.mean() > 0.999, same.mean()
    hit = same & (prim >= 0)
    # the instance path normalises the object-space direction and recomputes
    # the world distance (Instance.cpp:65-100): equal to a few float ulps
    np.testing.assert_allclose(t[hit], FIX["t"][hit], rtol=1e-6)


def test_fixture_is_the_reference():
    if not oracle.ref_available():
        pytest.skip("reference library not built here")
    sc = scenes.heightfield_blobs_instanced(**PARAMS)
    ref = oracle.RefScene(sc)
    r32 = FIX["rays"]
    rays6 = np.concatenate([r32[:, 0:3], r32[:, 4:7]], axis=1).astype(np.float64)
    prim, t = ref.intersect(rays6)
    assert np.array_equal(np.where(prim >= 0, prim // oracle.RefScene.MESH_ID, -1), FIX["mesh"])
    np.testing.assert_array_equal(t, FIX["t"])
