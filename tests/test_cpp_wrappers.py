"""The C++ wrappers compile: CudaTracer.hpp on its own, and RaycerAdapter.hpp
against the reference's own headers (where the reference's sources are)."""

from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import pytest

from raycer_gb300 import build

ROOT = Path(__file__).resolve().parent.parent
CPP = ROOT / "raycer_gb300" / "cpp"


@pytest.mark.skipif(shutil.which("g++") is None, reason="no C++ compiler")
def test_cuda_tracer_header_compiles(tmp_path):
    src = tmp_path / "use.cpp"
    src.write_text('#include "CudaTracer.hpp"\nint main() { raycer_gb300::SceneArrays a; (void)a; return 0; }\n')
    subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-Wall", "-Werror", f"-I{CPP}", str(src)], check=True)


@pytest.mark.skipif(not (build.REFERENCE_SRC / "src").is_dir(), reason="reference sources not present")
def test_raycer_adapter_compiles_against_reference_headers(tmp_path):
    src = tmp_path / "adapter.cpp"
    src.write_text('#include "stdafx.h"\n#include "RaycerAdapter.hpp"\n'
                   'void use(Raycer::Scene& s, Raycer::TracerState& st, std::atomic<bool>& i) {\n'
                   '  raycer_gb300::RaycerCudaTracer t(0); t.initializeKernels(); t.initializeImageBuffers(4, 4, 0);\n'
                   '  t.initializeBuffers(s); t.run(st, i); Raycer::Image img = t.downloadImage(); (void)img; }\n')
    ref = build.REFERENCE_SRC
    subprocess.run(["g++", "-std=c++17", "-fsyntax-only", f"-I{ROOT / 'oracle' / 'refshim'}", "-isystem",
                    str(ref / "include"), f"-I{ref / 'src'}", f"-I{CPP}", str(src)], check=True)
