// Scene upload through the GPU BVH builder (gpu_build.cu): the vertices go
// to the device once, the hierarchy, boxes and triangle records are built
// there, and the host only derives the reference-form flat BVH (for
// rc_get_bvh and scene files) from the finished device nodes.

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstring>
#include <string>
#include <vector>

#include "gpu_build.h"
#include "host_internal.h"

using namespace rcx;

namespace
{

rc_status fail(rc_tracer* h, rc_status s, const std::string& msg)
{
    h->err = msg;
    return s;
}

// Device buffer released at scope exit.
struct DevBuf
{
    void* p = nullptr;
    ~DevBuf()
    {
        if (p)
            cudaFree(p);
    }
    cudaError_t alloc(size_t bytes) { return cudaMalloc(&p, bytes > 0 ? bytes : 1); }
};

// Reference-form flat BVH (preorder, left = i + 1, right = i + rightOffset)
// of the device nodes: boxes as the nodes store them (float, widened).
void flat_from_device(const std::vector<DevNode>& dn, const std::vector<int2>& range, int32_t rootLink, int64_t n,
                      std::vector<BuildNode>& flat)
{
    struct Item
    {
        int32_t link;
        float box[6];  // lo xyz, hi xyz
        int64_t patch;  // flat index whose rightOffset this right child sets, or -1
    };
    flat.clear();
    flat.reserve(dn.size() * 2 + 1);
    std::vector<Item> stack;
    Item root{ rootLink, {}, -1 };
    if (rootLink >= 0)
    {
        const DevNode& d = dn[0];
        root.box[0] = std::min(d.xy0.x, d.xy1.x);
        root.box[3] = std::max(d.xy0.y, d.xy1.y);
        root.box[1] = std::min(d.xy0.z, d.xy1.z);
        root.box[4] = std::max(d.xy0.w, d.xy1.w);
        root.box[2] = std::min(d.z01.x, d.z01.z);
        root.box[5] = std::max(d.z01.y, d.z01.w);
    }
    stack.push_back(root);
    (void)n;
    while (!stack.empty())
    {
        Item it = stack.back();
        stack.pop_back();
        const int64_t idx = int64_t(flat.size());
        if (it.patch >= 0)
            flat[size_t(it.patch)].rightOffset = idx - it.patch;
        BuildNode b{};
        for (int k = 0; k < 3; ++k)
        {
            b.bmin[k] = double(it.box[k]);
            b.bmax[k] = double(it.box[3 + k]);
        }
        if (it.link < 0)
        {
            const uint32_t code = uint32_t(~it.link);
            b.rightOffset = 0;
            b.start = code >> kLeafCountBits;
            b.count = code & ((1u << kLeafCountBits) - 1u);
            flat.push_back(b);
            continue;
        }
        const DevNode& d = dn[size_t(it.link)];
        b.start = uint64_t(range[size_t(it.link)].x);
        b.count = uint64_t(range[size_t(it.link)].y);
        b.rightOffset = 0;  // set when the right child is emitted
        flat.push_back(b);
        Item l{ d.link.x, { d.xy0.x, d.xy0.z, d.z01.x, d.xy0.y, d.xy0.w, d.z01.y }, -1 };
        Item r{ d.link.y, { d.xy1.x, d.xy1.z, d.z01.z, d.xy1.y, d.xy1.w, d.z01.w }, idx };
        stack.push_back(r);
        stack.push_back(l);
    }
}

#define GB_TRY(expr, what)                                                                              \
    do                                                                                                  \
    {                                                                                                   \
        cudaError_t e_ = (expr);                                                                        \
        if (e_ != cudaSuccess)                                                                          \
        {                                                                                               \
            cudaGetLastError();                                                                         \
            return fail(h, e_ == cudaErrorMemoryAllocation ? RC_OOM : RC_CUDA,                          \
                        std::string("gpu build: ") + (what) + ": " + cudaGetErrorString(e_));            \
        }                                                                                               \
    } while (0)

}  // namespace

namespace rcx
{

rc_status upload_gpu_built(rc_tracer* h, const double* v, const uint32_t* matIdx, int64_t n, const rc_material* mats,
                           int32_t matCount, uint32_t maxLeafSize)
{
    const auto t0 = std::chrono::steady_clock::now();
    const size_t N = size_t(n);
    std::vector<DevMat> dm(static_cast<size_t>(matCount));
    {
        HostScene tmp;
        // materials only (no triangles): reuse the host construction
        build_host_scene(v, matIdx, 0, mats, matCount, {}, {}, 0, tmp);
        dm = std::move(tmp.mats);
    }
    DevBuf dV, dIdx, dM, dScratch;
    GB_TRY(dV.alloc(N * 9 * sizeof(double)), "allocate vertices");
    GB_TRY(dIdx.alloc(N * sizeof(uint32_t)), "allocate material indices");
    GB_TRY(dM.alloc(dm.size() * sizeof(DevMat)), "allocate materials");
    GB_TRY(dScratch.alloc(gpu_build_scratch_bytes(n)), "allocate scratch");
    GB_TRY(cudaMemcpyAsync(dV.p, v, N * 9 * sizeof(double), cudaMemcpyHostToDevice, h->stream), "upload vertices");
    GB_TRY(cudaMemcpyAsync(dIdx.p, matIdx, N * sizeof(uint32_t), cudaMemcpyHostToDevice, h->stream),
           "upload material indices");
    GB_TRY(cudaMemcpyAsync(dM.p, dm.data(), dm.size() * sizeof(DevMat), cudaMemcpyHostToDevice, h->stream),
           "upload materials");

    GpuBuildInput in;
    in.vertices = static_cast<const double*>(dV.p);
    in.matIdx = static_cast<const uint32_t*>(dIdx.p);
    in.mats = static_cast<const DevMat*>(dM.p);
    in.n = n;
    in.leafMax = int(maxLeafSize);
    GB_TRY(gpu_build_hierarchy(in, dScratch.p, h->stream), "hierarchy");
    uint32_t counts[3] = { 0, 0, 0 };
    GB_TRY(cudaMemcpyAsync(counts, gpu_build_counts(dScratch.p, n), sizeof(counts), cudaMemcpyDeviceToHost,
                           h->stream),
           "read node count");
    GB_TRY(cudaStreamSynchronize(h->stream), "hierarchy");
    const uint64_t kept = n > 1 ? uint64_t(counts[0]) + uint64_t(counts[1]) : 0;
    // levels of flat nodes on the longest path: internal levels + the leaf
    const uint32_t depth = n > 1 ? counts[2] + 1 : 1;
    if (depth > uint32_t(kMaxStack))
        return fail(h, RC_UNSUPPORTED, "gpu build: BVH depth " + std::to_string(depth) +
                                           " exceeds the traversal stack; use the SAH builder");

    release_scene_data(h);
    DevNode* dNodes = nullptr;
    DevTri* dTris = nullptr;
    DevShade* dShade = nullptr;
    DevMat* dMats = nullptr;
    DevBuf dRange, dOrder;
    const size_t nodeCount = size_t(std::max<uint64_t>(kept, 1));
    cudaError_t e = cudaMalloc(&dNodes, nodeCount * sizeof(DevNode));
    if (e == cudaSuccess)
        e = cudaMalloc(&dTris, N * sizeof(DevTri));
    if (e == cudaSuccess)
        e = cudaMalloc(&dShade, N * sizeof(DevShade));
    if (e == cudaSuccess)
        e = cudaMalloc(&dMats, dm.size() * sizeof(DevMat));
    if (e == cudaSuccess)
        e = dRange.alloc(nodeCount * sizeof(int2));
    if (e == cudaSuccess)
        e = dOrder.alloc(N * sizeof(uint32_t));
    if (e != cudaSuccess)
    {
        cudaGetLastError();
        cudaFree(dNodes);
        cudaFree(dTris);
        cudaFree(dShade);
        cudaFree(dMats);
        return fail(h, RC_OOM, std::string("gpu build: allocate scene: ") + cudaGetErrorString(e));
    }
    h->dNodes = dNodes;
    h->dTris = dTris;
    h->dShade = dShade;
    h->dMats = dMats;
    h->innerCount = nodeCount;
    h->nTris = n;
    h->nMats = matCount;
    h->deviceBytes += nodeCount * sizeof(DevNode) + N * (sizeof(DevTri) + sizeof(DevShade)) + dm.size() * sizeof(DevMat);
    GB_TRY(cudaMemsetAsync(dNodes, 0, nodeCount * sizeof(DevNode), h->stream), "clear nodes");
    GB_TRY(gpu_build_emit(in, dScratch.p, dNodes, static_cast<int2*>(dRange.p), dTris, dShade,
                          static_cast<uint32_t*>(dOrder.p), h->stream),
           "emit");
    GB_TRY(cudaMemcpyAsync(dMats, dm.data(), dm.size() * sizeof(DevMat), cudaMemcpyHostToDevice, h->stream),
           "upload materials");

    std::vector<DevNode> hn(nodeCount);
    std::vector<int2> hr(nodeCount);
    std::vector<uint32_t> order(N);
    GB_TRY(cudaMemcpyAsync(hn.data(), dNodes, nodeCount * sizeof(DevNode), cudaMemcpyDeviceToHost, h->stream),
           "read nodes");
    GB_TRY(cudaMemcpyAsync(hr.data(), dRange.p, nodeCount * sizeof(int2), cudaMemcpyDeviceToHost, h->stream),
           "read node ranges");
    GB_TRY(cudaMemcpyAsync(order.data(), dOrder.p, N * sizeof(uint32_t), cudaMemcpyDeviceToHost, h->stream),
           "read order");
    GB_TRY(cudaStreamSynchronize(h->stream), "emit");

    const int32_t rootLink = kept > 0 ? 0 : ~int32_t((0u << kLeafCountBits) | uint32_t(n));
    std::vector<BuildNode> flat;
    flat_from_device(hn, hr, rootLink, n, flat);
    if (rootLink < 0)
    {
        // a single leaf: its box from the float vertices
        for (int k = 0; k < 3; ++k)
        {
            flat[0].bmin[k] = double(float(v[k]));
            flat[0].bmax[k] = double(float(v[k]));
        }
        for (int64_t i = 0; i < n * 3; ++i)
            for (int k = 0; k < 3; ++k)
            {
                const double c = double(float(v[size_t(i) * 3 + size_t(k)]));
                flat[0].bmin[k] = std::min(flat[0].bmin[k], c);
                flat[0].bmax[k] = std::max(flat[0].bmax[k], c);
            }
    }
    uint32_t flatDepth = 0;
    std::string err;
    if (!validate_flat_bvh(flat, uint64_t(n), flatDepth, err))
    {
        release_scene_data(h);
        return fail(h, RC_DEVICE_ERROR, "gpu build: produced an invalid BVH: " + err);
    }
    h->rootLink = rootLink;
    h->bvhDepth = flatDepth;
    for (int k = 0; k < 3; ++k)
    {
        h->bounds[k] = flat[0].bmin[k];
        h->bounds[3 + k] = flat[0].bmax[k];
    }
    h->bvhInner = kept;
    h->hostNodes = std::move(flat);
    h->hostOrder = std::move(order);
    h->sceneReady = true;
    h->stats.build_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return RC_OK;
}

}  // namespace rcx
