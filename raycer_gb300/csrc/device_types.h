// Device data layout of the scene and of the per-frame records (HBM).
//
// Scene (uploaded once, read by every traversal):
//   DevNode  64 B per INNER node of the flat BVH, both child boxes inline
//            (the 2-wide node of Aila & Laine 2009). One 64-B fetch tests two
//            children; leaves are not stored as nodes — a child link < 0 is
//            ~((start << 4) | count) into the triangle arrays.
//            1M triangles, leaf <= 4: ~264k inner nodes = 17 MB.
//   DevTri   48 B per triangle in BVH order (the order of the reference's
//            FlatBVH::orderedPrimitives): v0, e1 = v1 - v0, e2 = v2 - v0 in
//            float32 (the same float subtraction intersectTriangle performs,
//            intersections.cl:37-38), material index + nonShadowing bit, and
//            the caller's triangle index. 1M triangles = 48 MB.
//   DevShade 48 B per triangle in BVH order: geometric normal, tangent,
//            bitangent (Triangle::initialize, Triangle.cpp:18-47, float64 on
//            the host, cast like CLScene.cpp:214-216); read once per hit.
//   DevMat   32 B per material.
//   DevNode4 128 B per node of the 4-wide BVH collapsed from the DevNode tree
//            (same leaves, same triangle order): the four children's boxes as
//            one float4 per bound (child k in component k), their links, and
//            the number of children. Read by the path tracer's uncounted
//            nearest-first extend kernel (traverse_wide); the binary tree
//            serves every other query.
// Everything is 16-B aligned and fetched with 128-bit loads.
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#include <cuda_runtime.h>
#else
#include <vector_types.h>
#endif

namespace rcx
{

struct __align__(16) DevNode
{
    float4 xy0;  // child 0: lo.x, hi.x, lo.y, hi.y
    float4 xy1;  // child 1: lo.x, hi.x, lo.y, hi.y
    float4 z01;  // child 0 lo.z, hi.z; child 1 lo.z, hi.z
    int4 link;   // child 0 (left), child 1 (right), reserved, reserved
};

// One child box of the binary tree in the reference's preorder (the
// stackless walk, traverse_stackless): a box that is hit leads to the next
// record (its first child) if it is an inner node's, else its leaf's
// triangles are tested; then, or on a miss, the walk jumps to `miss`, the
// first record after the box's subtree (= the record count after the last).
struct __align__(32) DevRope
{
    float4 a;    // lo.x, lo.y, lo.z, hi.x
    float hi_y;
    float hi_z;
    int link;    // >= 0: inner node (its children follow); < 0: leaf code ~((start << 4) | count)
    int miss;
};

struct __align__(16) DevNode4
{
    float4 lox, hix, loy, hiy, loz, hiz;  // child k's box in component k
    int4 link;   // child k: >= 0 DevNode4 index, < 0 leaf code ~((start << 4) | count)
    int4 meta;   // x: number of children (2..4); y, z, w: 0
};

struct __align__(16) DevTri
{
    float4 a;  // v0.x v0.y v0.z e1.x
    float4 b;  // e1.y e1.z e2.x e2.y
    float4 c;  // e2.z, meta (as bits), caller index (as bits), 0
};

struct __align__(16) DevShade
{
    float4 n;   // normal xyz, unused
    float4 t;   // tangent xyz, unused
    float4 bt;  // bitangent xyz, unused
};

struct __align__(16) DevMat
{
    float4 diffuse;    // rgb, unused
    float4 emittance;  // rgb, flags as bits (bit0 emissive, bit1 nonShadowing, bit2 invertNormal)
};

// meta word of DevTri.c.y
constexpr uint32_t kMetaMaterialMask = 0x00ffffffu;
constexpr uint32_t kMetaNonShadowing = 0x80000000u;

constexpr uint32_t kMatEmissive = 1u;
constexpr uint32_t kMatNonShadowing = 2u;
constexpr uint32_t kMatInvertNormal = 4u;
constexpr uint32_t kMatDielectric = 8u;  // DevMat.diffuse.w = index of refraction

constexpr int kLeafCountBits = 4;
constexpr int kMaxStack = 64;

// One placed copy of a mesh (two-level scenes): world -> object rows
// (object = A world + b; r_i = (A_i0, A_i1, A_i2, b_i)), the mesh's BVH
// root link (into the pooled node / triangle arrays), a material that
// replaces the triangles' own (or -1), and the first flattened primitive
// index of this instance (prim = primBase + the triangle's mesh-local index).
struct __align__(16) DevInstance
{
    float4 r0, r1, r2;
    int rootLink;
    int material;
    int primBase;
    int identity;  // 1: A = I, b = 0 (no transform needed)
};

// Progress and stop word of one render (rc_render): pinned host memory mapped
// into the device's address space, so the persistent kernels read the
// caller's cancel request and publish their progress while they run. Both
// fields cross the host link, so only one watching warp of each kernel
// touches them, about every 2 microseconds.
struct RenderMonitor
{
    volatile int cancel;                 // host -> device: non-zero = stop taking work
    int pad;
    volatile unsigned long long pixels;  // device -> host: pixels finished so far
};

constexpr unsigned long long kNoBudget = ~0ull;

// Device scene handed to every kernel by value. Two-level scenes
// (numInstances > 0) keep every mesh's BVH in `nodes` / `tris` / `shade`
// (links already offset into the pools) and a top-level BVH over the
// instances in `tlas` (leaf links index `instances`).
struct DevScene
{
    const DevNode* nodes;
    const DevTri* tris;
    const DevShade* shade;
    const DevMat* mats;
    int rootLink;  // >= 0: inner node 0; < 0: the root is a leaf (~leaf code)
    int numTris;
    int numMats;
    int pad;
    const DevNode* tlas;
    const DevInstance* instances;
    int tlasRoot;
    int numInstances;  // 0: single-level scene
    const DevNode4* wide;  // 4-wide BVH of a single-level scene, or null
    int wideRoot;          // >= 0: DevNode4 0; < 0: the root is a leaf
    int ropeCount;         // records in `ropes`
    const DevRope* ropes;  // the stackless walk's records of a single-level scene, or null
    RenderMonitor* monitor = nullptr;          // rc_render with a cancel flag or progress counter, else null
    unsigned long long budgetNs = kNoBudget;   // rc_render's time budget (kNoBudget: none)
};

// Float32 camera record used by the kernels (same fields as rc_camera).
struct DevCamera
{
    float pos[3];
    float fwd[3];
    float right[3];
    float up[3];
    float center[3];
    float aspect;
    float ipw;
    float iph;
};

}  // namespace rcx
