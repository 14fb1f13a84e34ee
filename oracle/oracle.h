// Test infrastructure only: NOT part of the product. Only the tests,
// __graft_entry__.smoke() and bench.py's CPU-baseline leg load the oracle.
//
// CPU oracle for the raycer hot path, two layers:
//   oracle64.cpp  float64 restatement of the reference's CPU code path
//                 (FlatBVH::build / intersect, Triangle::intersect,
//                 AABB::intersects, Camera::getRay, Tracer::run +
//                 PathTracer, Film, ReinhardToneMapper). Pinned against the
//                 reference itself (oracle/_ref) by golden fixtures.
//   oracle32.cpp  float32 twin of the device kernels: the reference's
//                 OpenCL kernels (intersections.cl, camera.cl, sampler.cl,
//                 pathtrace.cl) with the exact operation order the CUDA code
//                 uses (fused where the device fuses), so device results can
//                 be checked bit for bit.
// Compiled with -ffp-contract=off: nothing is fused unless written as fma.
#pragma once

#include <cstdint>
#include <vector>

namespace oracle
{

struct Node64
{
    double bmin[3];
    double bmax[3];
    int64_t rightOffset;
    uint64_t start;
    uint64_t count;
};

struct Material
{
    float diffuse[3];
    float emittance[3];
    int32_t flags;  // bit0 emissive, bit1 nonShadowing, bit2 invertNormal, bit3 dielectric
    float ior = 0.0f;
};

struct Scene64
{
    // caller order
    std::vector<double> v;         // n * 9
    std::vector<uint32_t> mat;     // n
    std::vector<Material> mats;
    // BVH (reference form) and primitive order
    std::vector<Node64> nodes;
    std::vector<uint64_t> order;   // order[slot] = caller index
    // Triangle::initialize results per caller triangle (normal, tangent, bitangent)
    std::vector<double> frame;     // n * 9
    uint32_t maxLeafSize = 4;
};

// float32 layout of the same scene (CLScene::readSceneFull, CLScene.cpp:72-240).
struct Scene32
{
    const Scene64* src = nullptr;
    std::vector<float> nodeBox;    // per node: min xyz, max xyz
    std::vector<float> tri;        // per slot: v0 xyz, e1 xyz, e2 xyz
    std::vector<uint32_t> meta;    // per slot: material index | nonShadowing << 31
    std::vector<int32_t> caller;   // per slot: caller index
    std::vector<float> shade;      // per slot: normal, tangent, bitangent (9 floats)
};

void build_bvh(Scene64& s);  // FlatBVH::build restated
void compute_frames(Scene64& s);
void make_scene32(const Scene64& s, Scene32& out);

}  // namespace oracle
