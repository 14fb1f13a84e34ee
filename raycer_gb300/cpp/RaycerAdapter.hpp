// Drop-in for the reference's OpenCL tracer inside the reference's own code
// base: include this header in raycer (it uses raycer's Scene, TracerState and
// Image types) and use raycer_gb300::RaycerCudaTracer where
// src/Runners/ConsoleRunner.cpp:78-101 and
// src/Runners/WindowRunnerStates/DefaultState.cpp:34-43, 104-123, 270-288 use
// CLTracer — same method names and arguments (src/OpenCL/CLTracer.h:23-41).
//
// Scene flattening follows CLScene::readSceneFull (src/OpenCL/CLScene.cpp:
// 72-240): the root BVH must hold only triangles; materials are indexed by
// their position in scene.materials (findMaterialIndex, CLScene.cpp:40-52);
// the already built root BVH (scene.rootBVH.bvh.flatNodes and
// orderedPrimitives) is uploaded as it is.
#pragma once

#include <algorithm>
#include <stdexcept>
#include <unordered_map>

#include "CudaTracer.hpp"

#include "Raytracing/Primitives/Triangle.h"
#include "Raytracing/Scene.h"
#include "Raytracing/Tracers/TracerState.h"
#include "Rendering/Image.h"

namespace raycer_gb300
{

inline uint64_t findMaterialIndex(const std::vector<Raycer::Material>& materials, uint64_t materialId)
{
    auto it = std::find_if(materials.begin(), materials.end(),
                           [materialId](const Raycer::Material& m) { return m.id == materialId; });
    if (it == materials.end())
        throw std::runtime_error("Could not find CUDA material index for material id " + std::to_string(materialId));
    return uint64_t(it - materials.begin());
}

inline SceneArrays sceneArraysFrom(const Raycer::Scene& scene)
{
    SceneArrays a;
    const auto& tris = scene.primitives.triangles;
    std::unordered_map<const Raycer::Primitive*, uint64_t> callerIndex;
    for (size_t i = 0; i < tris.size(); ++i)
        callerIndex[&tris[i]] = i;

    for (const Raycer::Primitive* p : scene.rootBVH.bvh.orderedPrimitives)
        if (dynamic_cast<const Raycer::Triangle*>(p) == nullptr || !callerIndex.count(p))
            throw std::runtime_error("When using CUDA, the root BVH must only contain triangles");

    a.vertices.resize(tris.size() * 9);
    a.materialIndex.resize(tris.size());
    for (size_t i = 0; i < tris.size(); ++i)
    {
        for (int k = 0; k < 3; ++k)
        {
            a.vertices[i * 9 + size_t(k) * 3 + 0] = tris[i].vertices[k].x;
            a.vertices[i * 9 + size_t(k) * 3 + 1] = tris[i].vertices[k].y;
            a.vertices[i * 9 + size_t(k) * 3 + 2] = tris[i].vertices[k].z;
        }
        a.materialIndex[i] = uint32_t(findMaterialIndex(scene.materials, tris[i].materialId));
    }
    for (const Raycer::Material& m : scene.materials)
    {
        rc_material r{};
        r.diffuse[0] = float(m.diffuseReflectance.r);
        r.diffuse[1] = float(m.diffuseReflectance.g);
        r.diffuse[2] = float(m.diffuseReflectance.b);
        r.emittance[0] = float(m.emittance.r);
        r.emittance[1] = float(m.emittance.g);
        r.emittance[2] = float(m.emittance.b);
        r.is_emissive = m.isEmissive;
        r.non_shadowing = m.nonShadowing;
        r.invert_normal = m.invertNormal;
        a.materials.push_back(r);
    }
    for (const Raycer::FlatBVHNode& n : scene.rootBVH.bvh.flatNodes)
    {
        rc_bvh_node r{};
        Raycer::Vector3 mn = n.aabb.getMin(), mx = n.aabb.getMax();
        r.aabb_min[0] = mn.x; r.aabb_min[1] = mn.y; r.aabb_min[2] = mn.z;
        r.aabb_max[0] = mx.x; r.aabb_max[1] = mx.y; r.aabb_max[2] = mx.z;
        r.right_offset = n.rightOffset;
        r.start_offset = n.startOffset;
        r.primitive_count = n.primitiveCount;
        a.nodes.push_back(r);
    }
    for (const Raycer::Primitive* p : scene.rootBVH.bvh.orderedPrimitives)
        a.orderedIndex.push_back(callerIndex.at(p));

    const Raycer::Scene::General& g = scene.general;
    rc_general_defaults(&a.general, g.tracerType == Raycer::TracerType::RAY ? RC_TRACER_RAY : RC_TRACER_PATH);
    a.general.max_path_length = int32_t(g.maxPathLength);
    a.general.path_sample_count = int32_t(g.pathSampleCount);
    a.general.multi_sample_count_sqrt = int32_t(g.multiSampleCountSqrt);
    a.general.multi_sampler_type = int32_t(g.multiSamplerType);
    a.general.filter_type = int32_t(g.multiSamplerFilterType);  // same enum order (Filter.h:10)
    a.general.ray_start_offset = float(g.rayStartOffset);
    a.general.background[0] = float(g.backgroundColor.r);
    a.general.background[1] = float(g.backgroundColor.g);
    a.general.background[2] = float(g.backgroundColor.b);

    rc_tonemapper_defaults(&a.tonemapper);
    a.tonemapper.type = int32_t(scene.toneMapper.type);
    a.tonemapper.apply_gamma = scene.toneMapper.applyGamma;
    a.tonemapper.should_clamp = scene.toneMapper.shouldClamp;
    a.tonemapper.gamma = scene.toneMapper.gamma;
    a.tonemapper.key = scene.toneMapper.key;

    for (const Raycer::DirectionalLight& l : scene.lights.directionalLights)
    {
        rc_directional_light r{};
        r.direction[0] = float(l.direction.x);
        r.direction[1] = float(l.direction.y);
        r.direction[2] = float(l.direction.z);
        r.color[0] = float(l.color.r);
        r.color[1] = float(l.color.g);
        r.color[2] = float(l.color.b);
        r.intensity = float(l.intensity);
        a.lights.push_back(r);
    }
    return a;
}

// Camera::update's perspective basis for a width x height film.
inline rc_camera cameraFrom(const Raycer::Scene& scene, uint64_t width, uint64_t height)
{
    const Raycer::Camera& c = scene.camera;
    double pos[3] = { c.position.x, c.position.y, c.position.z };
    rc_camera cam{};
    if (rc_camera_from_euler(pos, c.orientation.pitch, c.orientation.yaw, c.orientation.roll, c.fov, width, height,
                             &cam) != RC_OK)
        throw std::runtime_error("Invalid camera or film size");
    return cam;
}

// CLTracer's interface over raycer's own types.
class RaycerCudaTracer
{
public:
    explicit RaycerCudaTracer(int device = 0) : tracer(device) {}

    void initializeKernels() { tracer.initializeKernels(); }
    void releaseKernels() { tracer.releaseKernels(); }

    void initializeImageBuffers(uint64_t width, uint64_t height, uint64_t imageTextureId)
    {
        tracer.initializeImageBuffers(width, height, imageTextureId);
        imageWidth = width;
        imageHeight = height;
    }

    void releaseImageBuffers() { tracer.releaseImageBuffers(); }

    void initializeBuffers(const Raycer::Scene& scene) { tracer.initializeBuffers(sceneArraysFrom(scene)); }

    void releaseBuffers() { tracer.releaseBuffers(); }

    void run(Raycer::TracerState& state, std::atomic<bool>& interrupted)
    {
        TracerStateArrays s;
        s.camera = cameraFrom(*state.scene, state.filmWidth, state.filmHeight);
        s.filmWidth = state.filmWidth;
        s.filmHeight = state.filmHeight;
        s.pixelStartOffset = state.pixelStartOffset;
        s.pixelCount = state.pixelCount;
        // the render advances the reference's own counter while it runs
        tracer.run(s, interrupted, &state.pixelsProcessed);
    }

    Raycer::Image downloadImage()
    {
        std::vector<float> data = tracer.downloadImage();
        return Raycer::Image(imageWidth, imageHeight, data.data());
    }

    void clear() { tracer.clear(); }

private:
    CudaTracer tracer;
    uint64_t imageWidth = 0;
    uint64_t imageHeight = 0;
};

}  // namespace raycer_gb300
