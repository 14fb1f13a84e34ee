"""The C++ wrapper (raycer_gb300/cpp/CudaTracer.hpp) compiled and run: a
second thread polls TracerStateArrays::pixelsProcessed while run() renders,
as ConsoleRunner's main thread polls the reference's TracerState every
100 ms (ConsoleRunner.cpp:126-142), then raises `interrupted`; run() throws
std::runtime_error like any failed call (CLManager::checkError style). A
render without interruption then reports every pixel processed."""

from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import pytest

from raycer_gb300 import _native as N

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent

PROGRAM = r"""
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <random>
#include <stdexcept>
#include <thread>
#include <vector>

#include "CudaTracer.hpp"

using namespace raycer_gb300;

int main()
{
    SceneArrays scene;
    std::mt19937 rng(5);
    std::uniform_real_distribution<double> u(-1.0, 1.0);
    const int n = 3000;
    for (int i = 0; i < n; ++i)
    {
        const double c[3] = { u(rng), u(rng), u(rng) - 2.0 };
        for (int v = 0; v < 3; ++v)
            for (int k = 0; k < 3; ++k)
                scene.vertices.push_back(c[k] + 0.15 * u(rng));
        scene.materialIndex.push_back(0);
    }
    rc_material m{};
    m.diffuse[0] = m.diffuse[1] = m.diffuse[2] = 0.7f;
    scene.materials.push_back(m);
    rc_general_defaults(&scene.general, RC_TRACER_PATH);
    scene.general.filter_type = RC_FILTER_BOX;
    scene.general.multi_sample_count_sqrt = 8;
    scene.general.max_path_length = 4;
    scene.general.flags = RC_GENERAL_SKY;
    scene.general.background[0] = scene.general.background[1] = scene.general.background[2] = 1.0f;
    rc_tonemapper_defaults(&scene.tonemapper);

    CudaTracer tracer(0);
    tracer.initializeKernels();
    const uint64_t w = 1920, h = 1080;
    tracer.initializeImageBuffers(w, h);
    tracer.initializeBuffers(scene);

    TracerStateArrays state;
    const double pos[3] = { 0.0, 0.0, 1.5 };
    if (rc_camera_from_euler(pos, 0.0, 0.0, 0.0, 60.0, w, h, &state.camera) != RC_OK)
        return 2;
    state.filmWidth = w;
    state.filmHeight = h;
    state.pixelCount = w * h;

    std::atomic<bool> interrupted{ false };
    std::atomic<bool> done{ false };
    std::vector<uint64_t> seen;
    std::thread poller([&] {
        while (!done.load())
        {
            const uint64_t v = state.pixelsProcessed.load();
            if (seen.empty() || seen.back() != v)
                seen.push_back(v);
            if (v >= 2 * 65536)
                interrupted.store(true);
            std::this_thread::sleep_for(std::chrono::microseconds(200));
        }
    });
    bool threw = false;
    std::string message;
    try
    {
        tracer.run(state, interrupted);
    }
    catch (const std::runtime_error& e)
    {
        threw = true;
        message = e.what();
    }
    done.store(true);
    poller.join();
    const uint64_t stopped = state.pixelsProcessed.load();
    size_t mid = 0;
    for (uint64_t v : seen)
        mid += (v > 0 && v < w * h) ? 1 : 0;
    std::printf("threw=%d stopped=%llu mid=%zu message=%s\n", int(threw), (unsigned long long)stopped, mid,
                message.c_str());
    if (!threw || message.find("cancelled") == std::string::npos || stopped == 0 || stopped >= w * h ||
        stopped % 65536 != 0 || mid < 1)
        return 3;

    interrupted.store(false);
    tracer.clear();
    tracer.run(state, interrupted);
    std::printf("full=%llu\n", (unsigned long long)state.pixelsProcessed.load());
    if (state.pixelsProcessed.load() != w * h)
        return 4;
    std::vector<float> img = tracer.downloadImage();
    double sum = 0.0;
    for (size_t i = 0; i < img.size(); i += 4)
        sum += img[i];
    if (!(sum > 0.0) || !std::isfinite(sum))
        return 5;
    std::printf("OK\n");
    return 0;
}
"""


@pytest.mark.skipif(shutil.which("g++") is None, reason="no C++ compiler")
def test_cuda_tracer_wrapper_progress_and_interrupt(tmp_path):
    lib = N.LIB_PATH
    assert lib.exists()
    src = tmp_path / "wrapper_run.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "wrapper_run"
    subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", f"-I{ROOT / 'raycer_gb300' / 'cpp'}", str(src), "-o",
                    str(exe), f"-L{lib.parent}", "-lraycer_gb300", f"-Wl,-rpath,{lib.parent}", "-pthread"],
                   check=True)
    res = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0 and "OK" in res.stdout, (res.returncode, res.stdout, res.stderr)
