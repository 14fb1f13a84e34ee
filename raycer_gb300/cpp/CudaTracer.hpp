// C++ host wrapper over the C ABI (include/raycer_gb300.h) with the method
// shape of the reference's OpenCL tracer (src/OpenCL/CLTracer.h:23-41):
// initializeKernels / releaseKernels, initializeImageBuffers /
// releaseImageBuffers, initializeBuffers / releaseBuffers, run,
// downloadImage, clear. A failed call throws std::runtime_error with the
// library's message, as CLManager::checkError does
// (src/OpenCL/CLManager.cpp:73-101).
//
// Scenes are passed as plain arrays (SceneArrays); RaycerAdapter.hpp builds
// them from the reference's Raycer::Scene. Header-only; link with
// libraycer_gb300.so.
#pragma once

#include <atomic>
#include <chrono>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "../../include/raycer_gb300.h"

namespace raycer_gb300
{

// The parts of a triangle scene the hot path reads.
struct SceneArrays
{
    std::vector<double> vertices;          // n * 9: v0, v1, v2 per triangle
    std::vector<uint32_t> materialIndex;   // n
    std::vector<rc_material> materials;
    uint32_t maxLeafSize = 4;
    // Optional prebuilt BVH in the reference's FlatBVHNode form (CLScene copies
    // the node array verbatim, CLScene.cpp:224-237); empty = build here.
    std::vector<rc_bvh_node> nodes;
    std::vector<uint64_t> orderedIndex;
    rc_general general{};
    rc_tonemapper tonemapper{};
    std::vector<rc_directional_light> lights;
};

// TracerState (src/Raytracing/Tracers/TracerState.h:13-26) without the
// Scene/Film pointers: the camera record travels with it.
struct TracerStateArrays
{
    rc_camera camera{};
    uint64_t filmWidth = 0;
    uint64_t filmHeight = 0;
    uint64_t pixelStartOffset = 0;
    uint64_t pixelCount = 0;
    std::atomic<uint64_t> pixelsProcessed{ 0 };
};

class CudaTracer
{
public:
    explicit CudaTracer(int device = 0)
    {
        check(rc_create(&handle, device), "Could not create the CUDA tracer");
    }

    ~CudaTracer()
    {
        rc_destroy(handle);
    }

    CudaTracer(const CudaTracer&) = delete;
    CudaTracer& operator=(const CudaTracer&) = delete;

    // The kernels are compiled into the library (no run-time program build).
    void initializeKernels() {}
    void releaseKernels() {}

    // CLTracer::initializeImageBuffers (CLTracer.cpp:100-163); there is no GL
    // interop, the image lives in device memory and is downloaded on demand.
    void initializeImageBuffers(uint64_t width, uint64_t height, uint64_t imageTextureId = 0)
    {
        (void)imageTextureId;
        check(rc_resize(handle, width, height), "Could not create image buffers");
        imageWidth = width;
        imageHeight = height;
    }

    void releaseImageBuffers() {}

    // CLTracer::initializeBuffers + CLScene::readSceneFull (CLTracer.cpp:173,
    // CLScene.cpp:72-240).
    void initializeBuffers(const SceneArrays& scene)
    {
        const int64_t n = int64_t(scene.materialIndex.size());
        if (scene.nodes.empty())
            check(rc_upload_scene(handle, scene.vertices.data(), scene.materialIndex.data(), n, scene.materials.data(),
                                  int32_t(scene.materials.size()), scene.maxLeafSize),
                  "Could not upload the scene");
        else
            check(rc_upload_scene_prebuilt(handle, scene.vertices.data(), scene.materialIndex.data(), n,
                                           scene.materials.data(), int32_t(scene.materials.size()), scene.nodes.data(),
                                           int64_t(scene.nodes.size()), scene.orderedIndex.data()),
                  "Could not upload the scene");
        check(rc_set_general(handle, &scene.general), "Could not set the general settings");
        check(rc_set_tonemapper(handle, &scene.tonemapper), "Could not set the tone mapper");
        check(rc_set_directional_lights(handle, scene.lights.data(), int32_t(scene.lights.size())),
              "Could not set the lights");
    }

    void releaseBuffers()
    {
        check(rc_release_scene(handle), "Could not release the scene buffers");
    }

    // CLTracer::run (CLTracer.cpp:262-305) with Tracer::run's progress and
    // interruption contract (Tracer.cpp:76-112): `progress` (by default the
    // state's pixelsProcessed) advances while the kernels run, so another
    // thread can poll it as ConsoleRunner does every 100 ms
    // (ConsoleRunner.cpp:126-142); setting `interrupted` from another thread
    // stops the render at its kernels' next work-queue check, and run throws
    // like any failed call. A watcher thread turns the std::atomic<bool> into
    // the library's 32-bit cancel word (checked every half millisecond).
    void run(TracerStateArrays& state, std::atomic<bool>& interrupted, std::atomic<uint64_t>* progress = nullptr)
    {
        static_assert(sizeof(std::atomic<uint64_t>) == sizeof(uint64_t) && std::atomic<uint64_t>::is_always_lock_free,
                      "the library stores progress into the atomic's object representation");
        static_assert(sizeof(std::atomic<int32_t>) == sizeof(int32_t) && std::atomic<int32_t>::is_always_lock_free,
                      "the library reads the cancel word through the atomic's object representation");
        check(rc_set_camera(handle, &state.camera), "Could not set the camera");
        if (!progress)
            progress = &state.pixelsProcessed;
        std::atomic<int32_t> cancel{ interrupted.load() ? 1 : 0 };
        std::atomic<bool> finished{ false };
        std::thread watcher([&] {
            while (!finished.load(std::memory_order_acquire))
            {
                if (interrupted.load())
                {
                    cancel.store(1);
                    return;
                }
                std::this_thread::sleep_for(std::chrono::microseconds(500));
            }
        });
        const uint64_t count = state.pixelCount ? state.pixelCount : imageWidth * imageHeight;
        const rc_status st = rc_render(handle, state.pixelStartOffset, count,
                                       reinterpret_cast<const volatile int32_t*>(&cancel),
                                       reinterpret_cast<uint64_t*>(progress));
        finished.store(true, std::memory_order_release);
        watcher.join();
        check(st, "Could not run the tracer");
    }

    // Time budget of later renders (rc_set_time_budget; negative: none).
    void setTimeBudget(double milliseconds)
    {
        check(rc_set_time_budget(handle, milliseconds), "Could not set the time budget");
    }

    // CLTracer::downloadImage (CLTracer.cpp:307-323): tone-mapped RGBA floats.
    std::vector<float> downloadImage()
    {
        std::vector<float> data(size_t(imageWidth * imageHeight * 4));
        check(rc_resolve(handle, data.data()), "Could not read the output image");
        return data;
    }

    void clear()
    {
        check(rc_clear(handle), "Could not clear the film");
    }

    rc_tracer* native() { return handle; }

private:
    void check(rc_status status, const char* message)
    {
        if (status != RC_OK)
            throw std::runtime_error(std::string(message) + " (" + std::to_string(int(status)) +
                                     "): " + rc_last_error(handle));
    }

    rc_tracer* handle = nullptr;
    uint64_t imageWidth = 0;
    uint64_t imageHeight = 0;
};

}  // namespace raycer_gb300
