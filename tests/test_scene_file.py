"""Binary scene + BVH files (host side, no GPU): what is written is what the
upload would build, and damaged files are refused with a clear error."""

from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from raycer_gb300 import _native as N
from raycer_gb300.tracer import RaycerError, inspect_scene_file, write_scene_file

from helpers import small_heightfield, small_room


def build_bvh(sc):
    v = np.ascontiguousarray(sc.vertices, np.float64)
    count = C.c_int64(0)
    lib = N.lib()
    assert lib.rc_build_bvh(v.ctypes.data_as(C.c_void_p), v.shape[0], sc.max_leaf_size, None, 0, C.byref(count),
                            None, None) == N.RC_OK
    return count.value


@pytest.mark.parametrize("make", [small_room, small_heightfield])
def test_write_and_inspect(tmp_path, make):
    sc = make()
    path = tmp_path / "scene.rcgb"
    write_scene_file(sc, path)
    info = inspect_scene_file(path)
    assert info["triangles"] == sc.triangle_count
    assert info["materials"] == len(sc.materials)
    assert info["bvh_nodes"] == build_bvh(sc)
    v = sc.vertices.reshape(-1, 3)
    np.testing.assert_allclose(info["bounds"][:3], v.min(axis=0))
    np.testing.assert_allclose(info["bounds"][3:], v.max(axis=0))
    assert 1 <= info["bvh_depth"] <= 64
    expect = 128 + info["bvh_nodes"] * 72 + sc.triangle_count * (4 + 48 + 48) + len(sc.materials) * 32
    assert path.stat().st_size == expect


def test_damaged_files_are_refused(tmp_path):
    sc = small_room(clutter=100)
    path = tmp_path / "scene.rcgb"
    write_scene_file(sc, path)
    raw = bytearray(path.read_bytes())

    def refused(data: bytes, words: str):
        bad = tmp_path / "bad.rcgb"
        bad.write_bytes(data)
        with pytest.raises(RaycerError) as e:
            inspect_scene_file(bad)
        assert e.value.status == N.RC_IO
        assert words in str(e.value)

    flipped = bytearray(raw)
    flipped[128 + 500] ^= 0x40
    refused(bytes(flipped), "checksum")
    refused(bytes(raw[:-10]), "truncated")
    refused(bytes(raw) + b"x", "trailing")
    magic = bytearray(raw)
    magic[0:8] = b"NOTSCENE"
    refused(bytes(magic), "magic")
    counts = bytearray(raw)
    counts[16:24] = (10**12).to_bytes(8, "little")
    refused(bytes(counts), "out of range")
    with pytest.raises(RaycerError):
        inspect_scene_file(tmp_path / "missing.rcgb")


def test_instanced_scene_file(tmp_path):
    """Two-level scenes (version 2): one BVH per mesh, the instances, the
    scene box; a damaged payload is refused like a single-level one."""
    from raycer_gb300 import scenes

    sc = scenes.heightfield_blobs_instanced(instances=6, blob_level=2, hf_nx=32, hf_nz=16, width=32, height=18, seed=3)
    path = tmp_path / "inst.rcgb"
    write_scene_file(sc, path)
    info = inspect_scene_file(path)
    tris = sum(v.shape[0] for v, _ in sc.meshes)
    assert info["meshes"] == len(sc.meshes) and info["instances"] == len(sc.instances)
    assert info["triangles"] == tris and info["materials"] == len(sc.materials)
    assert 1 <= info["bvh_depth"] <= 64
    # the scene box holds every flattened vertex
    flat = sc.flatten().vertices.reshape(-1, 3)
    assert np.all(flat.min(axis=0) >= np.array(info["bounds"][:3]) - 1e-6)
    assert np.all(flat.max(axis=0) <= np.array(info["bounds"][3:]) + 1e-6)
    expect = (128 + len(sc.meshes) * 24 + info["bvh_nodes"] * 72 + tris * (4 + 48 + 48) + len(sc.materials) * 32 +
              len(sc.instances) * 80)
    assert path.stat().st_size == expect
    raw = bytearray(path.read_bytes())
    raw[-40] ^= 0x10  # inside the instance records
    bad = tmp_path / "bad.rcgb"
    bad.write_bytes(bytes(raw))
    with pytest.raises(RaycerError) as e:
        inspect_scene_file(bad)
    assert e.value.status == N.RC_IO and "checksum" in str(e.value)


def test_single_level_file_reports_no_instances(tmp_path):
    path = tmp_path / "room.rcgb"
    write_scene_file(small_room(clutter=50), path)
    info = inspect_scene_file(path)
    assert info["meshes"] == 0 and info["instances"] == 0
