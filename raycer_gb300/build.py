"""Builds the native parts in-tree.

* ``raycer_gb300/lib/libraycer_gb300.so`` — the product: CUDA kernels for
  sm_103a plus the host C++ behind the C ABI of ``include/raycer_gb300.h``.
* ``oracle/lib/liboracle.so`` — the CPU oracle (test infrastructure; only the
  tests and bench.py's CPU baseline load it).
* ``oracle/_ref/*.so`` — the reference's own hot path compiled from its
  sources, only where those sources are present.

Translation units are compiled in parallel; objects go to ``_build/``.
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "raycer_gb300"
CSRC = PKG / "csrc"
BUILD = ROOT / "_build"
LIB = PKG / "lib" / "libraycer_gb300.so"
ORACLE_LIB = ROOT / "oracle" / "lib" / "liboracle.so"
# The reference checkout whose hot path oracle/_ref is compiled from:
# $RAYCER_REFERENCE_DIR, else a directory named "reference" beside the
# repository. Where it is absent (e.g. on a machine with only this
# repository) the oracle runs on its own restatement.
REFERENCE_SRC = Path(os.environ.get("RAYCER_REFERENCE_DIR") or (ROOT.parent / "reference"))

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["trace.cu", "pathtrace.cu", "tonemap.cu", "noalloc.cu", "nrc.cu", "nrc_tc.cu", "gpu_build.cu"]
CPP_SOURCES = ["tracer_host.cpp", "render_path.cpp", "bvh_build.cpp", "batch.cpp", "nrc_host.cpp", "scene_file.cpp", "gpu_build_host.cpp", "instancing.cpp", "wide_bvh.cpp"]
ORACLE_SOURCES = ["oracle64.cpp", "oracle32.cpp", "oracle_api.cpp", "nrc64.cpp"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA extension cannot be built")


def _cuda_home(nvcc: str) -> Path:
    return Path(nvcc).resolve().parent.parent


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"command failed ({res.returncode}): {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build_product(verbose: bool = False) -> Path:
    nvcc = _nvcc()
    cuda = _cuda_home(nvcc)
    BUILD.mkdir(exist_ok=True)
    LIB.parent.mkdir(parents=True, exist_ok=True)
    headers = sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + [ROOT / "include" / "raycer_gb300.h"]
    jobs = []
    objs = []
    for src in CU_SOURCES:
        obj = BUILD / (src + ".o")
        objs.append(obj)
        if _stale(obj, [CSRC / src] + headers):
            jobs.append([nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                         "-c", str(CSRC / src), "-o", str(obj)])
    for src in CPP_SOURCES:
        obj = BUILD / (src + ".o")
        objs.append(obj)
        if _stale(obj, [CSRC / src] + headers):
            # -ffp-contract=off: the BVH builder and the float64 shading frames
            # must round exactly like the reference (aarch64 g++ fuses by default).
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-Wall",
                         "-Wno-unknown-pragmas",
                         f"-I{cuda / 'include'}", "-c", str(CSRC / src), "-o", str(obj)])
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(_run, jobs))
    if jobs or _stale(LIB, objs):
        _run([nvcc, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-Xcompiler", "-fopenmp", "-lgomp"])
    if verbose:
        print(f"built {LIB}")
    return LIB


def build_oracle(verbose: bool = False) -> Path:
    osrc = ROOT / "oracle"
    ORACLE_LIB.parent.mkdir(parents=True, exist_ok=True)
    deps = [osrc / s for s in ORACLE_SOURCES] + sorted(osrc.glob("*.h"))
    if _stale(ORACLE_LIB, deps):
        # -ffp-contract=off: the oracle's float arithmetic is exactly what is
        # written (fmaf where the device fuses, nothing else fused).
        _run(["g++", "-O2", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
              "-shared", "-o", str(ORACLE_LIB), *[str(osrc / s) for s in ORACLE_SOURCES]])
    if verbose:
        print(f"built {ORACLE_LIB}")
    return ORACLE_LIB


def build_reference(verbose: bool = False) -> bool:
    """Compiles the reference's hot path into oracle/_ref (only where its sources are)."""
    if not (REFERENCE_SRC / "src").is_dir():
        return False
    jobs = str(os.cpu_count() or 4)
    _run(["make", "-s", "-f", str(ROOT / "oracle" / "Makefile.ref"), "-C", str(ROOT), f"-j{jobs}",
          f"REF={REFERENCE_SRC}"])
    if verbose:
        print("built oracle/_ref")
    return True


def build_all(verbose: bool = False) -> None:
    with ThreadPoolExecutor(max_workers=2) as ex:
        f1 = ex.submit(build_product, verbose)
        f2 = ex.submit(build_oracle, verbose)
        f1.result()
        f2.result()
    build_reference(verbose)


if __name__ == "__main__":
    build_all(verbose=True)
    sys.exit(0)
