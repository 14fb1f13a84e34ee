"""The rope records of the stackless walk (wide_bvh.cpp build_ropes), checked
on the host: for 300 random binary trees and 20 random box-hit patterns each,
walking the records (hit inner box: next record; hit leaf: its triangles;
then, or on a miss: the record after the subtree) visits the same leaves in
the same order as the reference's stack walk (left child first), and every
tree gets exactly two records per inner node. The GPU walk over the same
records is checked against the oracle in tests/test_gpu_stackless.py."""

from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
CSRC = ROOT / "raycer_gb300" / "csrc"


def _cuda_home() -> Path | None:
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    home = Path(nvcc).resolve().parent.parent
    return home if (home / "include" / "cuda_runtime.h").exists() else None


@pytest.mark.skipif(shutil.which("g++") is None or _cuda_home() is None, reason="no C++ compiler or CUDA headers")
def test_rope_walk_visits_the_stack_walks_leaves(tmp_path):
    cuda = _cuda_home()
    exe = tmp_path / "rope_records_check"
    lib = cuda / "lib64"
    subprocess.run(["g++", "-std=c++17", "-O1", f"-I{cuda / 'include'}", f"-I{CSRC}", f"-I{ROOT / 'include'}",
                    str(Path(__file__).with_name("rope_records_check.cpp")), "-o", str(exe), f"-L{lib}",
                    f"-Wl,-rpath,{lib}", "-lcudart"], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "ropes ok" in out.stdout
