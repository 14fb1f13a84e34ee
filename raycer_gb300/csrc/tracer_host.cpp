// Host side of the C ABI (include/raycer_gb300.h): handle lifetime, scene
// upload and flattening to the device layout, per-frame records, film and
// render orchestration. Mirrors the reference's CLTracer / CLScene host code
// (src/OpenCL/CLTracer.cpp, src/OpenCL/CLScene.cpp) with CUDA underneath.

#include <cuda_runtime.h>
#include <sys/mman.h>
#include <unistd.h>

#include <algorithm>
#include <cstdlib>
#include <chrono>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <limits>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "../../include/raycer_gb300.h"
#include "bvh_build.h"
#include "device_types.h"
#include "host_internal.h"
#include "kernels.h"

using namespace rcx;

namespace
{

const char* kVersion = "raycer_gb300 0.1 (sm_103a)";

rc_status fail(rc_tracer* h, rc_status s, const std::string& msg)
{
    if (h)
        h->err = msg;
    return s;
}

rc_status cuda_fail(rc_tracer* h, cudaError_t e, const char* what)
{
    std::string msg = std::string(what) + ": " + cudaGetErrorString(e);
    if (e == cudaErrorMemoryAllocation)
        return fail(h, RC_OOM, msg);
    return fail(h, RC_CUDA, msg);
}

#define RC_CUDA_TRY(h, expr, what)                 \
    do                                             \
    {                                              \
        cudaError_t e_ = (expr);                   \
        if (e_ != cudaSuccess)                     \
            return cuda_fail((h), e_, (what));     \
    } while (0)

template <typename T>
rc_status dev_alloc(rc_tracer* h, T** ptr, size_t count, const char* what)
{
    *ptr = nullptr;
    if (count == 0)
        count = 1;
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(ptr), count * sizeof(T));
    if (e != cudaSuccess)
    {
        cudaGetLastError();
        return cuda_fail(h, e, what);
    }
    h->deviceBytes += count * sizeof(T);
    return RC_OK;
}

template <typename T>
void dev_free(rc_tracer* h, T** ptr, size_t count)
{
    if (*ptr)
    {
        cudaFree(*ptr);
        h->deviceBytes -= std::max<size_t>(count, 1) * sizeof(T);
        *ptr = nullptr;
    }
}

// Grow-only device scratch buffer.
rc_status ensure_bytes(rc_tracer* h, void** ptr, size_t* cap, size_t bytes, const char* what)
{
    if (*cap >= bytes && *ptr)
        return RC_OK;
    if (*ptr)
    {
        cudaFree(*ptr);
        h->deviceBytes -= *cap;
        *ptr = nullptr;
        *cap = 0;
    }
    cudaError_t e = cudaMalloc(ptr, bytes);
    if (e != cudaSuccess)
    {
        cudaGetLastError();
        return cuda_fail(h, e, what);
    }
    *cap = bytes;
    h->deviceBytes += bytes;
    return RC_OK;
}

void release_scene(rc_tracer* h)
{
    dev_free(h, &h->dNodes, h->innerCount);
    dev_free(h, &h->dTris, size_t(h->nTris));
    dev_free(h, &h->dShade, size_t(h->nTris));
    dev_free(h, &h->dMats, size_t(h->nMats));
    dev_free(h, &h->dTlas, h->tlasCount);
    dev_free(h, &h->dInstances, size_t(h->nInstances));
    dev_free(h, &h->dWide, h->wideCount);
    h->wideCount = 0;
    h->wideRoot = 0;
    h->wideTried = false;
    dev_free(h, &h->dRopes, h->ropeCount);
    h->ropeCount = 0;
    h->ropesTried = false;
    h->tlasCount = 0;
    h->nInstances = 0;
    h->tlasRoot = 0;
    h->sceneReady = false;
    h->nTris = 0;
    h->nMats = 0;
    h->innerCount = 0;
    h->hostNodes.clear();
    h->hostOrder.clear();
    h->instMeshes.clear();
    h->instDescs.clear();
}

void release_film(rc_tracer* h)
{
    dev_free(h, &h->dFilm, size_t(h->filmPixels));
    dev_free(h, &h->dCast, size_t(h->filmPixels));
    dev_free(h, &h->dQueue, size_t(h->filmPixels) * 2);
    h->filmPixels = 0;
    h->width = 0;
    h->height = 0;
}

struct Vec3d
{
    double x, y, z;
};
Vec3d sub(Vec3d a, Vec3d b) { return { a.x - b.x, a.y - b.y, a.z - b.z }; }
Vec3d cross(Vec3d a, Vec3d b) { return { a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x }; }
// Vector3::normalized (Vector3.cpp:162 + operator/ :57): v * (1 / length).
Vec3d normalized(Vec3d v)
{
    double len = std::sqrt(v.x * v.x + v.y * v.y + v.z * v.z);
    double inv = 1.0 / len;
    return { v.x * inv, v.y * inv, v.z * inv };
}

// Validates a reference-form flat BVH (preorder, left = i + 1,
// right = i + rightOffset, leaf <=> rightOffset == 0) over n primitives.
bool validate_flat(const std::vector<BuildNode>& nodes, uint64_t n, uint32_t& depth, std::string& err)
{
    struct Item
    {
        uint64_t idx, end, start, count;
        uint32_t depth;
    };
    if (nodes.empty())
    {
        err = "BVH has no nodes";
        return false;
    }
    if (nodes[0].start != 0 || nodes[0].count != n)
    {
        err = "BVH root does not cover all triangles";
        return false;
    }
    std::vector<Item> stack;
    stack.push_back({ 0, nodes.size(), 0, n, 1 });
    uint64_t visited = 0;
    depth = 0;
    while (!stack.empty())
    {
        Item it = stack.back();
        stack.pop_back();
        if (it.idx >= it.end || it.idx >= nodes.size())
        {
            err = "BVH node index out of range";
            return false;
        }
        const BuildNode& nd = nodes[it.idx];
        if (nd.start != it.start || nd.count != it.count)
        {
            err = "BVH node range does not match its parent's split";
            return false;
        }
        visited++;
        depth = std::max(depth, it.depth);
        if (nd.rightOffset == 0)
        {
            if (it.idx + 1 != it.end)
            {
                err = "BVH leaf is not the last node of its subtree";
                return false;
            }
            if (nd.count == 0 || nd.count > 15)
            {
                err = "BVH leaf primitive count must be in 1..15";
                return false;
            }
            continue;
        }
        if (nd.rightOffset < 2 || it.idx + uint64_t(nd.rightOffset) >= it.end)
        {
            err = "BVH rightOffset out of range";
            return false;
        }
        uint64_t r = it.idx + uint64_t(nd.rightOffset);
        const BuildNode& ln = nodes[it.idx + 1];
        const BuildNode& rn = nodes[r];
        if (ln.start != nd.start || rn.start != ln.start + ln.count || ln.count + rn.count != nd.count ||
            ln.count == 0 || rn.count == 0)
        {
            err = "BVH children do not partition the parent's range";
            return false;
        }
        stack.push_back({ r, it.end, rn.start, rn.count, it.depth + 1 });
        stack.push_back({ it.idx + 1, r, ln.start, ln.count, it.depth + 1 });
    }
    if (visited != nodes.size())
    {
        err = "BVH node array has unreachable nodes";
        return false;
    }
    return true;
}

}  // namespace

namespace rcx
{

// Device nodes from a validated reference-form flat BVH: inner nodes get
// compact indices in preorder, leaves fold into their parents' links.
void device_nodes(const std::vector<BuildNode>& nodes, std::vector<DevNode>& dn, int32_t& rootLink, uint64_t& inner)
{
    std::vector<int32_t> innerIndex(nodes.size(), -1);
    int32_t count = 0;
    for (size_t i = 0; i < nodes.size(); ++i)
        if (nodes[i].rightOffset != 0)
            innerIndex[i] = count++;
    auto link = [&](size_t i) -> int32_t {
        if (nodes[i].rightOffset != 0)
            return innerIndex[i];
        return ~int32_t((nodes[i].start << kLeafCountBits) | nodes[i].count);
    };
    dn.assign(size_t(std::max(count, 1)), DevNode{});
    for (size_t i = 0; i < nodes.size(); ++i)
    {
        if (nodes[i].rightOffset == 0)
            continue;
        size_t l = i + 1, r = i + size_t(nodes[i].rightOffset);
        DevNode& d = dn[size_t(innerIndex[i])];
        // double -> float with round-to-nearest, as CLScene::readVector3 does.
        const BuildNode& L = nodes[l];
        const BuildNode& R = nodes[r];
        d.xy0 = make_float4(float(L.bmin[0]), float(L.bmax[0]), float(L.bmin[1]), float(L.bmax[1]));
        d.xy1 = make_float4(float(R.bmin[0]), float(R.bmax[0]), float(R.bmin[1]), float(R.bmax[1]));
        d.z01 = make_float4(float(L.bmin[2]), float(L.bmax[2]), float(R.bmin[2]), float(R.bmax[2]));
        d.link = make_int4(link(l), link(r), 0, 0);
    }
    rootLink = nodes[0].rightOffset != 0 ? 0 : link(0);
    inner = uint64_t(count);
}

// Triangle, shading and material records of a scene in BVH order.
void build_host_scene(const double* v, const uint32_t* matIdx, int64_t n, const rc_material* mats, int32_t matCount,
                      std::vector<BuildNode>&& nodes, std::vector<uint32_t>&& order, uint32_t depth, HostScene& hs)
{
    std::vector<DevTri>& dt = hs.tris;
    std::vector<DevShade>& ds = hs.shade;
    dt.resize(static_cast<size_t>(n));
    ds.resize(static_cast<size_t>(n));
    for (int64_t s = 0; s < n; ++s)
    {
        uint32_t p = order[size_t(s)];
        const double* t = v + size_t(p) * 9;
        float f[9];
        for (int k = 0; k < 9; ++k)
            f[k] = float(t[k]);
        float e1[3] = { f[3] - f[0], f[4] - f[1], f[5] - f[2] };
        float e2[3] = { f[6] - f[0], f[7] - f[1], f[8] - f[2] };
        uint32_t m = matIdx[p];
        uint32_t meta = m | (mats[m].non_shadowing ? kMetaNonShadowing : 0u);
        DevTri& d = dt[size_t(s)];
        d.a = make_float4(f[0], f[1], f[2], e1[0]);
        d.b = make_float4(e1[1], e1[2], e2[0], e2[1]);
        float metaf, idxf;
        int32_t idx = int32_t(p);
        std::memcpy(&metaf, &meta, 4);
        std::memcpy(&idxf, &idx, 4);
        d.c = make_float4(e2[2], metaf, idxf, 0.0f);

        // Triangle::initialize (Triangle.cpp:18-47) with zero texcoords:
        // normal = normalize(e1 x e2); tangent = normalize(normal x ALMOST_UP);
        // bitangent = normalize(tangent x normal), all float64.
        Vec3d a{ t[0], t[1], t[2] }, b{ t[3], t[4], t[5] }, c{ t[6], t[7], t[8] };
        Vec3d nrm = normalized(cross(sub(b, a), sub(c, a)));
        Vec3d tan = normalized(cross(nrm, Vec3d{ 0.0001, 1.0, 0.0001 }));
        Vec3d bit = normalized(cross(tan, nrm));
        DevShade& sh = ds[size_t(s)];
        sh.n = make_float4(float(nrm.x), float(nrm.y), float(nrm.z), 0.0f);
        sh.t = make_float4(float(tan.x), float(tan.y), float(tan.z), 0.0f);
        sh.bt = make_float4(float(bit.x), float(bit.y), float(bit.z), 0.0f);
    }

    hs.mats.resize(static_cast<size_t>(matCount));
    for (int32_t i = 0; i < matCount; ++i)
    {
        const rc_material& m = mats[i];
        uint32_t flags = (m.is_emissive ? kMatEmissive : 0u) | (m.non_shadowing ? kMatNonShadowing : 0u) |
                         (m.invert_normal ? kMatInvertNormal : 0u) | (m.dielectric ? kMatDielectric : 0u);
        float ff;
        std::memcpy(&ff, &flags, 4);
        hs.mats[size_t(i)].diffuse =
            make_float4(m.diffuse[0], m.diffuse[1], m.diffuse[2], m.dielectric ? m.ior : 0.0f);
        hs.mats[size_t(i)].emittance = make_float4(m.emittance[0], m.emittance[1], m.emittance[2], ff);
    }
    hs.depth = depth;
    hs.flat = std::move(nodes);
    hs.order = std::move(order);
}

// Uploads a host scene (its flat BVH already validated, depth within the stack).
rc_status upload_host_scene(rc_tracer* h, HostScene&& hs)
{
    if (hs.depth > uint32_t(kMaxStack))
        return fail(h, RC_UNSUPPORTED, "BVH depth " + std::to_string(hs.depth) + " exceeds the traversal stack (" +
                                           std::to_string(kMaxStack) + ")");
    std::vector<DevNode> dn;
    int32_t rootLink = 0;
    uint64_t inner = 0;
    device_nodes(hs.flat, dn, rootLink, inner);

    release_scene(h);
    rc_status s;
    if ((s = dev_alloc(h, &h->dNodes, dn.size(), "allocate BVH nodes")) != RC_OK ||
        (s = dev_alloc(h, &h->dTris, hs.tris.size(), "allocate triangles")) != RC_OK ||
        (s = dev_alloc(h, &h->dShade, hs.shade.size(), "allocate shading records")) != RC_OK ||
        (s = dev_alloc(h, &h->dMats, hs.mats.size(), "allocate materials")) != RC_OK)
    {
        release_scene(h);
        return s;
    }
    h->innerCount = dn.size();
    h->nTris = int64_t(hs.tris.size());
    h->nMats = int32_t(hs.mats.size());
    RC_CUDA_TRY(h, cudaMemcpy(h->dNodes, dn.data(), dn.size() * sizeof(DevNode), cudaMemcpyHostToDevice),
                "upload BVH nodes");
    RC_CUDA_TRY(h, cudaMemcpy(h->dTris, hs.tris.data(), hs.tris.size() * sizeof(DevTri), cudaMemcpyHostToDevice),
                "upload triangles");
    RC_CUDA_TRY(h, cudaMemcpy(h->dShade, hs.shade.data(), hs.shade.size() * sizeof(DevShade), cudaMemcpyHostToDevice),
                "upload shading records");
    RC_CUDA_TRY(h, cudaMemcpy(h->dMats, hs.mats.data(), hs.mats.size() * sizeof(DevMat), cudaMemcpyHostToDevice),
                "upload materials");

    h->rootLink = rootLink;
    h->bvhDepth = hs.depth;
    h->bvhInner = inner;
    for (int k = 0; k < 3; ++k)
    {
        h->bounds[k] = hs.flat[0].bmin[k];
        h->bounds[3 + k] = hs.flat[0].bmax[k];
    }
    h->hostNodes = std::move(hs.flat);
    h->hostOrder = std::move(hs.order);
    h->sceneReady = true;
    return RC_OK;
}

void release_scene_data(rc_tracer* h) { release_scene(h); }

bool validate_flat_bvh(const std::vector<BuildNode>& nodes, uint64_t n, uint32_t& depth, std::string& err)
{
    return validate_flat(nodes, n, depth, err);
}

// Flattens the reference-form BVH to the device layout and uploads it.
rc_status upload_common(rc_tracer* h, const double* v, const uint32_t* matIdx, int64_t n, const rc_material* mats,
                        int32_t matCount, std::vector<BuildNode>&& nodes, std::vector<uint32_t>&& order,
                        uint32_t depth)
{
    if (depth > uint32_t(kMaxStack))
        return fail(h, RC_UNSUPPORTED, "BVH depth " + std::to_string(depth) + " exceeds the traversal stack (" +
                                           std::to_string(kMaxStack) + ")");
    HostScene hs;
    build_host_scene(v, matIdx, n, mats, matCount, std::move(nodes), std::move(order), depth, hs);
    return upload_host_scene(h, std::move(hs));
}

}  // namespace rcx

namespace
{

rc_status check_scene_args(rc_tracer* h, const double* v, const uint32_t* matIdx, int64_t n, const rc_material* mats,
                           int32_t matCount)
{
    if (!h)
        return RC_INVALID_ARG;
    if (!v || !matIdx || !mats || n <= 0 || matCount <= 0)
        return fail(h, RC_INVALID_ARG, "upload: null array or empty scene");
    if (n > (int64_t(1) << 27))
        return fail(h, RC_UNSUPPORTED, "upload: more than 2^27 triangles");
    if (matCount > int32_t(kMetaMaterialMask))
        return fail(h, RC_UNSUPPORTED, "upload: too many materials");
    for (int64_t i = 0; i < n; ++i)
        if (matIdx[i] >= uint32_t(matCount))
            return fail(h, RC_INVALID_ARG, "upload: material index out of range at triangle " + std::to_string(i));
    for (int64_t i = 0; i < n * 9; ++i)
        if (!std::isfinite(v[i]))
            return fail(h, RC_INVALID_ARG, "upload: non-finite vertex coordinate");
    for (int32_t i = 0; i < matCount; ++i)
        if ((mats[i].dielectric != 0 && mats[i].dielectric != 1) ||
            (mats[i].dielectric && !(mats[i].ior > 0.0f && std::isfinite(mats[i].ior))))
            return fail(h, RC_INVALID_ARG, "upload: rc_material.dielectric must be 0 or 1 with ior > 0");
    return RC_OK;
}

DevScene dev_scene(const rc_tracer* h)
{
    DevScene s{};
    s.nodes = h->dNodes;
    s.tris = h->dTris;
    s.shade = h->dShade;
    s.mats = h->dMats;
    s.rootLink = h->rootLink;
    s.numTris = int(h->nTris);
    s.numMats = int(h->nMats);
    s.pad = 0;
    s.tlas = h->dTlas;
    s.instances = h->dInstances;
    s.tlasRoot = h->tlasRoot;
    s.numInstances = int(h->nInstances);
    s.wide = h->dWide;
    s.wideRoot = h->wideRoot;
    s.ropes = h->dRopes;
    s.ropeCount = int(h->ropeCount);
    return s;
}

DevCamera dev_camera(const rc_camera& c)
{
    DevCamera d;
    for (int k = 0; k < 3; ++k)
    {
        d.pos[k] = c.position[k];
        d.fwd[k] = c.forward[k];
        d.right[k] = c.right[k];
        d.up[k] = c.up[k];
        d.center[k] = c.image_plane_center[k];
    }
    d.aspect = c.aspect_ratio;
    d.ipw = c.image_plane_width;
    d.iph = c.image_plane_height;
    return d;
}

LaunchInfo launch_info(const rc_tracer* h)
{
    LaunchInfo li;
    li.stream = h->stream;
    li.numSMs = h->numSMs;
    li.counting = h->counting;
    return li;
}

rc_status begin_launch(rc_tracer* h)
{
    RC_CUDA_TRY(h, cudaMemsetAsync(h->dCtl, 0, sizeof(DevControl), h->stream), "reset control block");
    RC_CUDA_TRY(h, cudaEventRecord(h->ev0, h->stream), "record start event");
    return RC_OK;
}

rc_status end_launch(rc_tracer* h, const char* what, bool twoStage, RenderWatch* watch = nullptr)
{
    RC_CUDA_TRY(h, cudaEventRecord(h->ev1, h->stream), "record end event");
    {
        // before the read-back below: a copy into pageable memory returns
        // only once the kernels are done
        rc_status ws = wait_render(h, watch, h->ev1);
        if (ws != RC_OK)
            return ws;
    }
    DevControl ctl;
    RC_CUDA_TRY(h, cudaMemcpyAsync(&ctl, h->dCtl, sizeof(ctl), cudaMemcpyDeviceToHost, h->stream),
                "read control block");
    RC_CUDA_TRY(h, cudaStreamSynchronize(h->stream), what);
    float ms = 0.0f, ms0 = 0.0f;
    cudaEventElapsedTime(&ms, h->ev0, h->ev1);
    h->stats.last_ms = double(ms);
    if (twoStage)
    {
        cudaEventElapsedTime(&ms0, h->ev0, h->evMid);
        h->stats.stage_ms[0] = double(ms0);
        h->stats.stage_ms[1] = double(ms - ms0);
    }
    else
    {
        h->stats.stage_ms[0] = double(ms);
        h->stats.stage_ms[1] = 0.0;
    }
    for (int k = 0; k < 2; ++k)
    {
        h->stats.stage_rays[k] = ctl.stats[3 * k + 0];
        h->stats.stage_nodes[k] = ctl.stats[3 * k + 1];
        h->stats.stage_tris[k] = ctl.stats[3 * k + 2];
    }
    h->stats.rays_traced = ctl.stats[0] + ctl.stats[3];
    h->stats.node_visits = ctl.stats[1] + ctl.stats[4];
    h->stats.tri_tests = ctl.stats[2] + ctl.stats[5];
    // pixels finished: those whose primary ray was traced (a queued shadow
    // ray is always traced by the end of the call)
    if (watch && watch->pixels)
        __atomic_store_n(watch->pixels, uint64_t(ctl.stats[0]), __ATOMIC_RELAXED);
    return render_outcome(h, ctl.error, what);
}

}  // namespace

// ---------------------------------------------------------------------------

extern "C" {

const char* rc_version(void) { return kVersion; }

rc_status rc_create(rc_tracer** out, int device)
{
    if (!out)
        return RC_INVALID_ARG;
    *out = nullptr;
    rc_tracer* h = new (std::nothrow) rc_tracer();
    if (!h)
        return RC_OOM;
    h->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess)
        e = cudaDeviceGetAttribute(&h->numSMs, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess)
        e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess)
        e = cudaEventCreate(&h->ev0);
    if (e == cudaSuccess)
        e = cudaEventCreate(&h->ev1);
    if (e == cudaSuccess)
        e = cudaEventCreate(&h->evMid);
    if (e == cudaSuccess)
        e = cudaMalloc(reinterpret_cast<void**>(&h->dCtl), sizeof(DevControl));
    if (e == cudaSuccess)
        e = cudaHostAlloc(reinterpret_cast<void**>(&h->monHost), sizeof(RenderMonitor), cudaHostAllocMapped);
    if (e == cudaSuccess)
    {
        h->monHost->cancel = 0;
        h->monHost->pixels = 0;
        e = cudaHostGetDevicePointer(reinterpret_cast<void**>(&h->monDev), h->monHost, 0);
    }
    if (e != cudaSuccess)
    {
        cudaGetLastError();
        rc_status s = (e == cudaErrorMemoryAllocation) ? RC_OOM : RC_CUDA;
        rc_destroy(h);
        return s;
    }
    h->deviceBytes += sizeof(DevControl);
    rc_general_defaults(&h->general, RC_TRACER_PATH);
    rc_tonemapper_defaults(&h->tonemapper);
    *out = h;
    return RC_OK;
}

void rc_destroy(rc_tracer* h)
{
    if (!h)
        return;
    cudaSetDevice(h->device);
    if (h->stream)
        cudaStreamSynchronize(h->stream);
    release_scene(h);
    release_film(h);
    release_render_buffers(h);
    nrc_release(h);
    if (h->dRmse)
        cudaFree(h->dRmse);
    if (h->dTmpA)
        cudaFree(h->dTmpA);
    if (h->dTmpB)
        cudaFree(h->dTmpB);
    if (h->dCtl)
        cudaFree(h->dCtl);
    if (h->monHost)
        cudaFreeHost(h->monHost);
    if (h->ev0)
        cudaEventDestroy(h->ev0);
    if (h->ev1)
        cudaEventDestroy(h->ev1);
    if (h->evMid)
        cudaEventDestroy(h->evMid);
    for (cudaEvent_t e : h->evPool)
        cudaEventDestroy(e);
    for (cudaEvent_t e : h->evChunk)
        cudaEventDestroy(e);
    if (h->dCtlChunks)
        cudaFree(h->dCtlChunks);
    if (h->copyIn)
        cudaStreamDestroy(h->copyIn);
    if (h->copyOut)
        cudaStreamDestroy(h->copyOut);
    if (h->stream)
        cudaStreamDestroy(h->stream);
    delete h;
}

const char* rc_last_error(const rc_tracer* h)
{
    return h ? h->err.c_str() : "null handle";
}

rc_status rc_upload_scene(rc_tracer* h, const double* vertices, const uint32_t* material_index, int64_t n,
                          const rc_material* materials, int32_t material_count, uint32_t max_leaf_size)
{
    rc_status s = check_scene_args(h, vertices, material_index, n, materials, material_count);
    if (s != RC_OK)
        return s;
    if (max_leaf_size < 1 || max_leaf_size > 15)
        return fail(h, RC_UNSUPPORTED, "upload: max_leaf_size must be in 1..15");
    cudaSetDevice(h->device);
    if (h->builder == RC_BUILDER_GPU_LBVH)
        return upload_gpu_built(h, vertices, material_index, n, materials, material_count, max_leaf_size);
    const auto t0 = std::chrono::steady_clock::now();
    BuildResult br;
    std::string err;
    if (!buildFlatBVH(vertices, n, max_leaf_size, 0, br, err))
        return fail(h, RC_INVALID_ARG, err);
    s = upload_common(h, vertices, material_index, n, materials, material_count, std::move(br.nodes),
                      std::move(br.order), br.depth);
    h->stats.build_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return s;
}

rc_status rc_set_bvh_builder(rc_tracer* h, int32_t builder)
{
    if (!h)
        return RC_INVALID_ARG;
    if (builder != RC_BUILDER_REFERENCE_SAH && builder != RC_BUILDER_GPU_LBVH)
        return fail(h, RC_INVALID_ARG, "set_bvh_builder: unknown builder");
    h->builder = builder;
    return RC_OK;
}

rc_status rc_upload_scene_prebuilt(rc_tracer* h, const double* vertices, const uint32_t* material_index, int64_t n,
                                   const rc_material* materials, int32_t material_count, const rc_bvh_node* nodes,
                                   int64_t node_count, const uint64_t* ordered_index)
{
    rc_status s = check_scene_args(h, vertices, material_index, n, materials, material_count);
    if (s != RC_OK)
        return s;
    if (!nodes || node_count <= 0 || !ordered_index)
        return fail(h, RC_INVALID_ARG, "upload: null BVH arrays");
    cudaSetDevice(h->device);
    std::vector<uint32_t> order(static_cast<size_t>(n));
    std::vector<char> seen(size_t(n), 0);
    for (int64_t i = 0; i < n; ++i)
    {
        uint64_t p = ordered_index[i];
        if (p >= uint64_t(n) || seen[size_t(p)])
            return fail(h, RC_INVALID_ARG, "upload: ordered_index is not a permutation of the triangles");
        seen[size_t(p)] = 1;
        order[size_t(i)] = uint32_t(p);
    }
    std::vector<BuildNode> bn(static_cast<size_t>(node_count));
    for (int64_t i = 0; i < node_count; ++i)
    {
        for (int k = 0; k < 3; ++k)
        {
            bn[size_t(i)].bmin[k] = nodes[i].aabb_min[k];
            bn[size_t(i)].bmax[k] = nodes[i].aabb_max[k];
        }
        bn[size_t(i)].rightOffset = nodes[i].right_offset;
        bn[size_t(i)].start = nodes[i].start_offset;
        bn[size_t(i)].count = nodes[i].primitive_count;
    }
    uint32_t depth = 0;
    std::string err;
    if (!validate_flat(bn, uint64_t(n), depth, err))
        return fail(h, RC_INVALID_ARG, "upload: " + err);
    return upload_common(h, vertices, material_index, n, materials, material_count, std::move(bn), std::move(order),
                         depth);
}

rc_status rc_get_bvh(const rc_tracer* hc, rc_bvh_node* nodes, int64_t node_capacity, int64_t* node_count,
                     uint64_t* ordered_index, int64_t index_capacity)
{
    rc_tracer* h = const_cast<rc_tracer*>(hc);
    if (!h)
        return RC_INVALID_ARG;
    if (!h->sceneReady)
        return fail(h, RC_NOT_READY, "get_bvh: no scene uploaded");
    if (h->nInstances > 0)
        return fail(h, RC_UNSUPPORTED, "get_bvh: an instanced scene has one BVH per mesh and one over instances");
    if (node_count)
        *node_count = int64_t(h->hostNodes.size());
    if (nodes)
    {
        if (node_capacity < int64_t(h->hostNodes.size()))
            return fail(h, RC_INVALID_ARG, "get_bvh: node buffer too small");
        for (size_t i = 0; i < h->hostNodes.size(); ++i)
        {
            const BuildNode& b = h->hostNodes[i];
            for (int k = 0; k < 3; ++k)
            {
                nodes[i].aabb_min[k] = b.bmin[k];
                nodes[i].aabb_max[k] = b.bmax[k];
            }
            nodes[i].right_offset = b.rightOffset;
            nodes[i].start_offset = b.start;
            nodes[i].primitive_count = b.count;
        }
    }
    if (ordered_index)
    {
        if (index_capacity < int64_t(h->hostOrder.size()))
            return fail(h, RC_INVALID_ARG, "get_bvh: index buffer too small");
        for (size_t i = 0; i < h->hostOrder.size(); ++i)
            ordered_index[i] = h->hostOrder[i];
    }
    return RC_OK;
}

rc_status rc_build_bvh(const double* vertices, int64_t n, uint32_t max_leaf_size, rc_bvh_node* nodes,
                       int64_t node_capacity, int64_t* node_count, uint64_t* ordered_index, uint32_t* depth)
{
    if (!vertices || n <= 0)
        return RC_INVALID_ARG;
    if (max_leaf_size < 1 || max_leaf_size > 15)
        return RC_UNSUPPORTED;
    BuildResult br;
    std::string err;
    if (!buildFlatBVH(vertices, n, max_leaf_size, 0, br, err))
        return RC_INVALID_ARG;
    if (node_count)
        *node_count = int64_t(br.nodes.size());
    if (depth)
        *depth = br.depth;
    if (!nodes)
        return RC_OK;
    if (node_capacity < int64_t(br.nodes.size()))
        return RC_INVALID_ARG;
    for (size_t i = 0; i < br.nodes.size(); ++i)
    {
        const BuildNode& b = br.nodes[i];
        for (int k = 0; k < 3; ++k)
        {
            nodes[i].aabb_min[k] = b.bmin[k];
            nodes[i].aabb_max[k] = b.bmax[k];
        }
        nodes[i].right_offset = b.rightOffset;
        nodes[i].start_offset = b.start;
        nodes[i].primitive_count = b.count;
    }
    if (ordered_index)
        for (size_t i = 0; i < br.order.size(); ++i)
            ordered_index[i] = br.order[i];
    return RC_OK;
}

rc_status rc_release_scene(rc_tracer* h)
{
    if (!h)
        return RC_INVALID_ARG;
    cudaSetDevice(h->device);
    cudaStreamSynchronize(h->stream);
    release_scene(h);
    return RC_OK;
}

rc_status rc_set_camera(rc_tracer* h, const rc_camera* camera)
{
    if (!h)
        return RC_INVALID_ARG;
    if (!camera)
        return fail(h, RC_INVALID_ARG, "set_camera: null record");
    if (!(camera->image_plane_width > 0.0f) || !(camera->image_plane_height > 0.0f))
        return fail(h, RC_INVALID_ARG, "set_camera: image plane width/height must be > 0 (film of at least 2x2)");
    h->camera = *camera;
    h->cameraSet = true;
    return RC_OK;
}

rc_status rc_set_general(rc_tracer* h, const rc_general* g)
{
    if (!h)
        return RC_INVALID_ARG;
    if (!g)
        return fail(h, RC_INVALID_ARG, "set_general: null record");
    if (g->tracer_type != RC_TRACER_RAY && g->tracer_type != RC_TRACER_PATH)
        return fail(h, RC_INVALID_ARG, "set_general: invalid tracer type");
    if (g->max_path_length < 0 || g->path_sample_count < 1 || g->multi_sample_count_sqrt < 1 ||
        g->multi_sample_count_sqrt > 64 || g->path_sample_count > 65536 || g->max_path_length > 1024)
        return fail(h, RC_INVALID_ARG, "set_general: sample counts / path length out of range");
    if (g->multi_sampler_type != RC_SAMPLER_CMJ && g->multi_sampler_type != RC_SAMPLER_RANDOM &&
        g->multi_sampler_type != RC_SAMPLER_CENTER)
        return fail(h, RC_UNSUPPORTED, "set_general: multi sampler must be CENTER, RANDOM or CMJ");
    if (g->filter_type < RC_FILTER_BOX || g->filter_type > RC_FILTER_LANCZOS_SINC)
        return fail(h, RC_INVALID_ARG, "set_general: unknown filter type");
    if (g->filter_type == RC_FILTER_BOX && (!(g->filter_radius[0] > 0.0f) || !(g->filter_radius[1] > 0.0f)))
        return fail(h, RC_INVALID_ARG, "set_general: box filter radius must be > 0");
    if (g->russian_roulette_depth < 0 || (g->flags & ~int32_t(RC_GENERAL_SKY)) != 0)
        return fail(h, RC_INVALID_ARG, "set_general: invalid russian_roulette_depth / flags");
    h->general = *g;
    return RC_OK;
}

rc_status rc_set_tonemapper(rc_tracer* h, const rc_tonemapper* t)
{
    if (!h)
        return RC_INVALID_ARG;
    if (!t)
        return fail(h, RC_INVALID_ARG, "set_tonemapper: null record");
    if (t->type != RC_TONEMAP_REINHARD && t->type != RC_TONEMAP_PASSTHROUGH)
        return fail(h, RC_UNSUPPORTED, "set_tonemapper: only PASSTHROUGH and REINHARD are supported");
    if (t->type == RC_TONEMAP_REINHARD && !(t->gamma > 0.0))
        return fail(h, RC_INVALID_ARG, "set_tonemapper: gamma must be > 0");
    if (t->reserved != 0)
        return fail(h, RC_INVALID_ARG, "set_tonemapper: reserved must be 0");
    h->tonemapper = *t;
    return RC_OK;
}

rc_status rc_set_directional_lights(rc_tracer* h, const rc_directional_light* lights, int32_t count)
{
    if (!h)
        return RC_INVALID_ARG;
    if (count < 0 || (count > 0 && !lights))
        return fail(h, RC_INVALID_ARG, "set_directional_lights: bad array");
    if (count > 1)
        return fail(h, RC_UNSUPPORTED, "set_directional_lights: at most one directional light");
    h->lights.assign(lights, lights + count);
    return RC_OK;
}

void rc_general_defaults(rc_general* g, int32_t tracer_type)
{
    if (!g)
        return;
    std::memset(g, 0, sizeof(*g));
    // Scene::General defaults (Scene.h:89-108).
    g->tracer_type = tracer_type;
    g->max_path_length = 3;
    g->path_sample_count = 1;
    g->multi_sample_count_sqrt = 1;
    g->multi_sampler_type = RC_SAMPLER_CMJ;
    g->filter_type = RC_FILTER_MITCHELL;
    g->filter_radius[0] = 0.5f;
    g->filter_radius[1] = 0.5f;
    g->ray_start_offset = 0.00001f;
    g->russian_roulette_depth = 0;
    g->seed = 1;
}

void rc_tonemapper_defaults(rc_tonemapper* t)
{
    if (!t)
        return;
    // Scene::ToneMapper defaults (Scene.h:135-145) with REINHARD.
    t->type = RC_TONEMAP_REINHARD;
    t->apply_gamma = 1;
    t->should_clamp = 1;
    t->reserved = 0;
    t->gamma = 2.2;
    t->key = 0.18;
}

rc_status rc_camera_from_euler(const double position[3], double pitch, double yaw, double roll, double fov,
                               uint64_t width, uint64_t height, rc_camera* out)
{
    if (!position || !out || width < 2 || height < 2)
        return RC_INVALID_ARG;
    const double d2r = M_PI / 180.0;  // MathUtils::degToRad (MathUtils.cpp:36-39)
    auto direction = [&](double p, double y) {
        // EulerAngle::getDirection (EulerAngle.cpp:77-87)
        Vec3d r{ -std::sin(y * d2r) * std::cos(p * d2r), std::sin(p * d2r), -std::cos(y * d2r) * std::cos(p * d2r) };
        return normalized(r);
    };
    // ONB::fromNormal (ONB.cpp:32-39) with Vector3::ALMOST_UP (Vector3.cpp:15).
    auto onb = [&](Vec3d w, Vec3d& u, Vec3d& v) {
        u = normalized(cross(w, Vec3d{ 0.0001, 1.0, 0.0001 }));
        v = normalized(cross(u, w));
    };
    (void)roll;
    // Camera::update (Camera.cpp:48-284), non-interactive: forward for the
    // image-plane centre comes from the orientation before clampPitch /
    // normalize; the stored basis from the orientation after them.
    Vec3d fwd0 = direction(pitch, yaw);
    double p = std::min(89.0, std::max(-89.0, pitch));
    auto wrap = [](double a) {
        while (std::abs(a) > 180.0)
            a += (a > 0.0) ? -360.0 : 360.0;
        return a;
    };
    p = wrap(p);
    double y = wrap(yaw);
    double f = std::max(1.0, std::min(fov, 180.0));
    double ipd = 0.5 / std::tan((f / 2.0) * d2r);
    Vec3d w = direction(p, y), u, v;
    onb(w, u, v);
    Vec3d pos{ position[0], position[1], position[2] };
    Vec3d centre{ pos.x + fwd0.x * ipd, pos.y + fwd0.y * ipd, pos.z + fwd0.z * ipd };
    const Vec3d* src[5] = { &pos, &w, &u, &v, &centre };
    float* dst[5] = { out->position, out->forward, out->right, out->up, out->image_plane_center };
    for (int i = 0; i < 5; ++i)
    {
        dst[i][0] = float(src[i]->x);
        dst[i][1] = float(src[i]->y);
        dst[i][2] = float(src[i]->z);
    }
    // Camera::setImagePlaneSize (Camera.cpp:29-34)
    out->image_plane_width = float(double(width - 1));
    out->image_plane_height = float(double(height - 1));
    out->aspect_ratio = float(double(height) / double(width));
    return RC_OK;
}

rc_status rc_resize(rc_tracer* h, uint64_t width, uint64_t height)
{
    if (!h)
        return RC_INVALID_ARG;
    if (width == 0 || height == 0 || width * height > (uint64_t(1) << 31))
        return fail(h, RC_INVALID_ARG, "resize: film must have 1 .. 2^31 pixels");
    cudaSetDevice(h->device);
    cudaStreamSynchronize(h->stream);
    release_film(h);
    uint64_t px = width * height;
    rc_status s;
    if ((s = dev_alloc(h, &h->dFilm, size_t(px), "allocate film")) != RC_OK ||
        (s = dev_alloc(h, &h->dCast, size_t(px), "allocate cast buffer")) != RC_OK ||
        (s = dev_alloc(h, &h->dQueue, size_t(px) * 2, "allocate shadow queue")) != RC_OK)
    {
        release_film(h);
        return s;
    }
    h->width = width;
    h->height = height;
    h->filmPixels = px;
    return rc_clear(h);
}

rc_status rc_clear(rc_tracer* h)
{
    if (!h)
        return RC_INVALID_ARG;
    if (!h->dFilm)
        return fail(h, RC_NOT_READY, "clear: no film (call rc_resize)");
    cudaSetDevice(h->device);
    h->frameIndex = 0;
    RC_CUDA_TRY(h, cudaMemsetAsync(h->dFilm, 0, size_t(h->filmPixels) * sizeof(float4), h->stream), "clear film");
    RC_CUDA_TRY(h, cudaMemsetAsync(h->dCast, 0, size_t(h->filmPixels) * sizeof(rc_cast_pixel), h->stream),
                "clear cast buffer");
    RC_CUDA_TRY(h, cudaStreamSynchronize(h->stream), "clear");
    return RC_OK;
}

rc_status rc_render(rc_tracer* h, uint64_t pixel_start, uint64_t pixel_count, const volatile int32_t* cancel,
                    uint64_t* pixels_processed)
{
    if (!h)
        return RC_INVALID_ARG;
    if (!h->sceneReady)
        return fail(h, RC_NOT_READY, "render: no scene uploaded");
    if (!h->dFilm)
        return fail(h, RC_NOT_READY, "render: no film (call rc_resize)");
    if (!h->cameraSet)
        return fail(h, RC_NOT_READY, "render: no camera set");
    if (pixel_count == 0 || pixel_count > h->filmPixels)
        return fail(h, RC_INVALID_ARG, "render: pixel_count must be in 1..film pixels");
    if (pixel_start + pixel_count < pixel_start)
        return fail(h, RC_INVALID_ARG, "render: pixel range overflows");
    cudaSetDevice(h->device);
    if (pixels_processed)
        __atomic_store_n(pixels_processed, uint64_t(0), __ATOMIC_RELAXED);
    if (cancel && *cancel)
        return fail(h, RC_CANCELLED, "render: cancelled");

    // The previous render on this handle has finished (every call blocks
    // until its kernels are done), so nothing reads the monitor now.
    RenderWatch watch;
    watch.cancel = cancel;
    watch.pixels = pixels_processed;
    watch.budgetNs = h->budgetNs;
    if (cancel || pixels_processed)
    {
        h->monHost->cancel = 0;
        h->monHost->pixels = 0;
        watch.dev = h->monDev;
    }
    rc_status s;
    if (h->general.tracer_type == RC_TRACER_RAY)
        s = render_raycast(h, pixel_start, pixel_count, nullptr, &watch);
    else
        s = render_path(h, pixel_start, pixel_count, &watch);
    if (s == RC_OK && pixels_processed)
        __atomic_store_n(pixels_processed, pixel_count, __ATOMIC_RELAXED);
    return s;
}

rc_status rc_set_time_budget(rc_tracer* h, double milliseconds)
{
    if (!h)
        return RC_INVALID_ARG;
    if (std::isnan(milliseconds))
        return fail(h, RC_INVALID_ARG, "set_time_budget: NaN");
    if (milliseconds < 0.0)
        h->budgetNs = kNoBudget;
    else if (milliseconds >= 1.0e12)
        return fail(h, RC_INVALID_ARG, "set_time_budget: budget above 1e12 ms");
    else
        h->budgetNs = static_cast<unsigned long long>(milliseconds * 1.0e6);
    return RC_OK;
}

rc_status rc_read_cast(rc_tracer* h, rc_cast_pixel* out)
{
    if (!h)
        return RC_INVALID_ARG;
    if (!h->dCast || !out)
        return fail(h, RC_NOT_READY, "read_cast: no film or null output");
    cudaSetDevice(h->device);
    RC_CUDA_TRY(h,
                cudaMemcpyAsync(out, h->dCast, size_t(h->filmPixels) * sizeof(rc_cast_pixel), cudaMemcpyDeviceToHost,
                                h->stream),
                "download cast buffer");
    RC_CUDA_TRY(h, cudaStreamSynchronize(h->stream), "read_cast");
    return RC_OK;
}

rc_status rc_cast_device(rc_tracer* h, const rc_ray* d_rays, int64_t n, int32_t any_hit, int32_t order,
                         rc_hit* d_hits)
{
    if (!h)
        return RC_INVALID_ARG;
    if (!h->sceneReady)
        return fail(h, RC_NOT_READY, "cast: no scene uploaded");
    if (n < 0 || n > (int64_t(1) << 31) - 64 || (n > 0 && (!d_rays || !d_hits)))
        return fail(h, RC_INVALID_ARG, "cast: bad ray count or null buffer");
    if ((reinterpret_cast<uintptr_t>(d_rays) | reinterpret_cast<uintptr_t>(d_hits)) & 15u)
        return fail(h, RC_INVALID_ARG, "cast: ray and hit buffers must be 16-byte aligned");
    if (order != RC_ORDER_REFERENCE && order != RC_ORDER_NEAREST)
        return fail(h, RC_INVALID_ARG, "cast: invalid traversal order");
    cudaSetDevice(h->device);
    rc_status s = stackless_walk() ? ensure_ropes(h) : RC_OK;
    if (s != RC_OK)
        return s;
    s = begin_launch(h);
    if (s != RC_OK)
        return s;
    RC_CUDA_TRY(h, launch_cast(launch_info(h), dev_scene(h), d_rays, n, any_hit, order, d_hits, h->dCtl),
                "launch cast kernel");
    return end_launch(h, "cast", false);
}

rc_status rc_cast(rc_tracer* h, const rc_ray* rays, int64_t n, int32_t any_hit, int32_t order, rc_hit* hits)
{
    if (!h)
        return RC_INVALID_ARG;
    if (n < 0 || (n > 0 && (!rays || !hits)))
        return fail(h, RC_INVALID_ARG, "cast: bad ray count or null buffer");
    if (n == 0)
        return RC_OK;
    cudaSetDevice(h->device);
    rc_status s;
    if ((s = ensure_bytes(h, &h->dTmpA, &h->capTmpA, size_t(n) * sizeof(rc_ray), "allocate ray buffer")) != RC_OK ||
        (s = ensure_bytes(h, &h->dTmpB, &h->capTmpB, size_t(n) * sizeof(rc_hit), "allocate hit buffer")) != RC_OK)
        return s;
    RC_CUDA_TRY(h, cudaMemcpyAsync(h->dTmpA, rays, size_t(n) * sizeof(rc_ray), cudaMemcpyHostToDevice, h->stream),
                "upload rays");
    s = rc_cast_device(h, static_cast<const rc_ray*>(h->dTmpA), n, any_hit, order, static_cast<rc_hit*>(h->dTmpB));
    if (s != RC_OK)
        return s;
    RC_CUDA_TRY(h, cudaMemcpyAsync(hits, h->dTmpB, size_t(n) * sizeof(rc_hit), cudaMemcpyDeviceToHost, h->stream),
                "download hits");
    RC_CUDA_TRY(h, cudaStreamSynchronize(h->stream), "cast");
    return RC_OK;
}

rc_status rc_cast_with_shadow(rc_tracer* h, const rc_ray* rays, int64_t n, int32_t order, rc_cast_pixel* out)
{
    if (!h)
        return RC_INVALID_ARG;
    if (!h->sceneReady)
        return fail(h, RC_NOT_READY, "cast_with_shadow: no scene uploaded");
    if (n < 0 || n > (int64_t(1) << 31) - 64 || (n > 0 && (!rays || !out)))
        return fail(h, RC_INVALID_ARG, "cast_with_shadow: bad ray count or null buffer");
    if (order != RC_ORDER_REFERENCE && order != RC_ORDER_NEAREST)
        return fail(h, RC_INVALID_ARG, "cast_with_shadow: invalid traversal order");
    if (n == 0)
        return RC_OK;  // an empty batch, as in rc_cast
    cudaSetDevice(h->device);
    rc_status s = stackless_walk() ? ensure_ropes(h) : RC_OK;
    if (s != RC_OK)
        return s;
    // In place when the device can reach both host buffers (16-byte aligned):
    // the kernels read the rays and write the results over the host link, so
    // no separate copy has to wait for the persistent kernels.
    // (RC_CAST_COPY=1 in the environment forces the copy path.)
    const char* forceCopy = std::getenv("RC_CAST_COPY");
    if (!(forceCopy && forceCopy[0] == '1'))
    {
        void* vr = device_view(h, rays, size_t(n) * sizeof(rc_ray));
        void* vo = vr ? device_view(h, out, size_t(n) * sizeof(rc_cast_pixel)) : nullptr;
        if (vr && vo && ((reinterpret_cast<uintptr_t>(vr) | reinterpret_cast<uintptr_t>(vo)) & 15u) == 0)
        {
            // shadow queue (8 B per entry) + the shadow rays' origins (16 B, device
            // memory): the shadow kernel then reads nothing over the host link
            const size_t queueBytes = (size_t(n) * 2 * sizeof(int) + 15) & ~size_t(15);
            if ((s = ensure_bytes(h, &h->dTmpB, &h->capTmpB, queueBytes + size_t(n) * sizeof(float4),
                                  "allocate shadow queue")) != RC_OK)
                return s;
            s = raycast_into(h, static_cast<const rc_ray*>(vr), 0, uint64_t(n), order, static_cast<rc_cast_pixel*>(vo),
                             static_cast<int*>(h->dTmpB),
                             reinterpret_cast<float4*>(static_cast<char*>(h->dTmpB) + queueBytes));
            h->stats.stage_ms[0] = h->stats.stage_ms[1] = 0.0;
            return s;
        }
    }
    // Chunks of at least 2^RC_CAST_MIN_CHUNK_LOG2 rays: chunk i's upload,
    // chunk i-1's kernels and chunk i-2's download run at the same time on
    // three streams.
#ifndef RC_CAST_MIN_CHUNK_LOG2
#define RC_CAST_MIN_CHUNK_LOG2 19
#endif
    constexpr int64_t kMinChunk = int64_t(1) << RC_CAST_MIN_CHUNK_LOG2;
    constexpr int kMaxChunks = 8;
    const int chunks = int(std::max<int64_t>(1, std::min<int64_t>(kMaxChunks, n / kMinChunk)));
    const int64_t per = (n + chunks - 1) / chunks;
    size_t rayBytes = size_t(n) * sizeof(rc_ray);
    size_t outBytes = size_t(n) * (sizeof(rc_cast_pixel) + 2 * sizeof(int));
    if ((s = ensure_bytes(h, &h->dTmpA, &h->capTmpA, rayBytes, "allocate ray buffer")) != RC_OK ||
        (s = ensure_bytes(h, &h->dTmpB, &h->capTmpB, outBytes, "allocate output buffer")) != RC_OK ||
        (s = ensure_bytes(h, &h->dCtlChunks, &h->capCtlChunks, size_t(kMaxChunks) * sizeof(DevControl),
                          "allocate control blocks")) != RC_OK)
        return s;
    if (!h->copyIn)
        RC_CUDA_TRY(h, cudaStreamCreateWithFlags(&h->copyIn, cudaStreamNonBlocking), "create copy stream");
    if (!h->copyOut)
        RC_CUDA_TRY(h, cudaStreamCreateWithFlags(&h->copyOut, cudaStreamNonBlocking), "create copy stream");
    while (h->evChunk.size() < size_t(2 * kMaxChunks + 1))
    {
        cudaEvent_t e;
        RC_CUDA_TRY(h, cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "create event");
        h->evChunk.push_back(e);
    }
    const rc_ray* dRays = static_cast<const rc_ray*>(h->dTmpA);
    rc_cast_pixel* dOut = static_cast<rc_cast_pixel*>(h->dTmpB);
    int* dQueue = reinterpret_cast<int*>(dOut + n);
    DevControl* ctl = static_cast<DevControl*>(h->dCtlChunks);
    float3 L = make_float3(0.0f, 0.0f, 0.0f);
    const int castShadow = h->lights.empty() ? 0 : 1;
    if (castShadow)
        L = make_float3(-h->lights[0].direction[0], -h->lights[0].direction[1], -h->lights[0].direction[2]);
    const DevCamera cam = dev_camera(h->camera);
    const DevScene sc = dev_scene(h);
    LaunchInfo li = launch_info(h);

    // the previous call's downloads must be done before this call's kernels
    // rewrite the output buffer
    RC_CUDA_TRY(h, cudaEventRecord(h->evChunk[2 * kMaxChunks], h->copyOut), "record event");
    RC_CUDA_TRY(h, cudaStreamWaitEvent(h->stream, h->evChunk[2 * kMaxChunks], 0), "order streams");
    RC_CUDA_TRY(h, cudaMemsetAsync(ctl, 0, size_t(chunks) * sizeof(DevControl), h->stream), "reset control blocks");
    RC_CUDA_TRY(h, cudaEventRecord(h->ev0, h->stream), "record start event");
    RC_CUDA_TRY(h, cudaStreamWaitEvent(h->copyIn, h->ev0, 0), "order streams");
    for (int c = 0; c < chunks; ++c)
    {
        const int64_t off = c * per;
        const int64_t cnt = std::min<int64_t>(per, n - off);
        if (cnt <= 0)
            break;
        RC_CUDA_TRY(h, cudaMemcpyAsync(const_cast<rc_ray*>(dRays) + off, rays + off, size_t(cnt) * sizeof(rc_ray),
                                       cudaMemcpyHostToDevice, h->copyIn),
                    "upload rays");
        RC_CUDA_TRY(h, cudaEventRecord(h->evChunk[2 * c], h->copyIn), "record event");
        RC_CUDA_TRY(h, cudaStreamWaitEvent(h->stream, h->evChunk[2 * c], 0), "order streams");
        RC_CUDA_TRY(h,
                    launch_raycast(li, sc, cam, dRays + off, 0, cnt, 1, order, castShadow, L,
                                   h->general.ray_start_offset, dOut + off, dQueue, ctl + c, nullptr),
                    "launch ray-cast kernels");
        RC_CUDA_TRY(h, cudaEventRecord(h->evChunk[2 * c + 1], h->stream), "record event");
        RC_CUDA_TRY(h, cudaStreamWaitEvent(h->copyOut, h->evChunk[2 * c + 1], 0), "order streams");
        RC_CUDA_TRY(h, cudaMemcpyAsync(out + off, dOut + off, size_t(cnt) * sizeof(rc_cast_pixel),
                                       cudaMemcpyDeviceToHost, h->copyOut),
                    "download results");
    }
    RC_CUDA_TRY(h, cudaEventRecord(h->ev1, h->copyOut), "record end event");
    std::vector<DevControl> ctls(static_cast<size_t>(chunks));
    RC_CUDA_TRY(h, cudaMemcpyAsync(ctls.data(), ctl, size_t(chunks) * sizeof(DevControl), cudaMemcpyDeviceToHost,
                                   h->stream),
                "read control blocks");
    RC_CUDA_TRY(h, cudaStreamSynchronize(h->stream), "cast_with_shadow");
    RC_CUDA_TRY(h, cudaStreamSynchronize(h->copyOut), "cast_with_shadow");
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, h->ev0, h->ev1);
    const double buildMs = h->stats.build_ms;
    h->stats = rc_stats{};
    h->stats.build_ms = buildMs;
    h->stats.last_ms = double(ms);
    int err = 0;
    for (const DevControl& c : ctls)
    {
        for (int k = 0; k < 2; ++k)
        {
            h->stats.stage_rays[k] += c.stats[3 * k + 0];
            h->stats.stage_nodes[k] += c.stats[3 * k + 1];
            h->stats.stage_tris[k] += c.stats[3 * k + 2];
        }
        err |= c.error;
    }
    h->stats.rays_traced = h->stats.stage_rays[0] + h->stats.stage_rays[1];
    h->stats.node_visits = h->stats.stage_nodes[0] + h->stats.stage_nodes[1];
    h->stats.tri_tests = h->stats.stage_tris[0] + h->stats.stage_tris[1];
    if (err & 1)
        return fail(h, RC_DEVICE_ERROR, "cast_with_shadow: traversal stack overflow");
    return RC_OK;
}

rc_status rc_set_traversal_order(rc_tracer* h, int32_t order)
{
    if (!h)
        return RC_INVALID_ARG;
    if (order != RC_ORDER_REFERENCE && order != RC_ORDER_NEAREST)
        return fail(h, RC_INVALID_ARG, "set_traversal_order: invalid order");
    h->order = order;
    return RC_OK;
}

rc_status rc_set_counting(rc_tracer* h, int32_t enable)
{
    if (!h)
        return RC_INVALID_ARG;
    h->counting = enable ? 1 : 0;
    return RC_OK;
}

rc_status rc_get_stats(const rc_tracer* h, rc_stats* out)
{
    if (!h || !out)
        return RC_INVALID_ARG;
    *out = h->stats;
    out->bvh_inner_nodes = h->bvhInner;
    out->bvh_depth = h->bvhDepth;
    out->device_bytes = h->deviceBytes;
    return RC_OK;
}

void* rc_stream(rc_tracer* h) { return h ? static_cast<void*>(h->stream) : nullptr; }

rc_status rc_sync(rc_tracer* h)
{
    if (!h)
        return RC_INVALID_ARG;
    cudaSetDevice(h->device);
    RC_CUDA_TRY(h, cudaStreamSynchronize(h->stream), "sync");
    return RC_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Render helpers shared with the path tracer (host_internal.h).

namespace rcx
{

namespace
{
// Whether every page of [p, p + bytes) is resident (mincore). A kernel that
// writes or reads pageable memory whose pages are not populated yet takes a
// fault per page on the device side (milliseconds for a fresh 33 MB image);
// such buffers go through a copy instead.
bool host_resident(const void* p, size_t bytes)
{
    static const size_t page = [] {
        const long v = sysconf(_SC_PAGESIZE);
        return v > 0 ? size_t(v) : size_t(4096);
    }();
    const uintptr_t a = reinterpret_cast<uintptr_t>(p) & ~uintptr_t(page - 1);
    const uintptr_t e = reinterpret_cast<uintptr_t>(p) + bytes;
    const size_t pages = (e - a + page - 1) / page;
    std::vector<unsigned char> vec(pages);
    if (mincore(reinterpret_cast<void*>(a), pages * page, vec.data()) != 0)
        return false;
    for (unsigned char c : vec)
        if (!(c & 1))
            return false;
    return true;
}
}  // namespace

// Device address of a caller's host buffer of `bytes` bytes when kernels may
// access it in place: page-locked memory mapped into the device's address
// space, or pageable memory whose pages are all resident on a device that
// reads pageable memory coherently (Grace-class hosts). nullptr otherwise.
void* device_view(rc_tracer* h, const void* p, size_t bytes)
{
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess)
    {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type == cudaMemoryTypeHost && a.devicePointer && a.device == h->device)
        return a.devicePointer;
    if (a.type == cudaMemoryTypeManaged || (a.type == cudaMemoryTypeDevice && a.device == h->device))
        return const_cast<void*>(p);
    int pageable = 0;
    if (a.type == cudaMemoryTypeUnregistered &&
        cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccessUsesHostPageTables, h->device) ==
            cudaSuccess &&
        pageable && host_resident(p, bytes))
        return const_cast<void*>(p);
    cudaGetLastError();
    return nullptr;
}

rc_status wait_render(rc_tracer* h, RenderWatch* w, cudaEvent_t done)
{
    if (!w || (!w->cancel && !w->pixels))
        return RC_OK;
    bool raised = false;
    while (true)
    {
        const cudaError_t q = cudaEventQuery(done);
        if (!raised && w->cancel && *w->cancel)
        {
            h->monHost->cancel = 1;
            raised = true;
        }
        if (w->pixels)
        {
            const uint64_t p = h->monHost->pixels;
            if (p > w->seen)
            {
                w->seen = p;
                __atomic_store_n(w->pixels, p, __ATOMIC_RELAXED);
            }
        }
        if (q == cudaSuccess)
            return RC_OK;
        if (q != cudaErrorNotReady)
            return cuda_fail(h, q, "render");
        std::this_thread::yield();
    }
}

rc_status render_outcome(rc_tracer* h, int error, const char* what)
{
    if (error & kErrStack)
        return fail(h, RC_DEVICE_ERROR, std::string(what) + ": traversal stack overflow");
    if (error & kErrCancelled)
        return fail(h, RC_CANCELLED, std::string(what) + ": cancelled");
    if (error & kErrBudget)
        return fail(h, RC_TIMEOUT, std::string(what) + ": the time budget of " +
                                       std::to_string(double(h->budgetNs) / 1.0e6) + " ms ran out");
    return RC_OK;
}

rc_status raycast_into(rc_tracer* h, const rc_ray* dRays, uint64_t pixelStart, uint64_t count, int order,
                       rc_cast_pixel* dOut, int* dQueue, float4* dOrigins, RenderWatch* watch)
{
    float3 L = make_float3(0.0f, 0.0f, 0.0f);
    int castShadow = h->lights.empty() ? 0 : 1;
    if (castShadow)
    {
        // directionToLight = -light.direction (Raytracer.cpp:499, lighting.cl:92)
        L = make_float3(-h->lights[0].direction[0], -h->lights[0].direction[1], -h->lights[0].direction[2]);
    }
    DevCamera cam = dev_camera(h->camera);
    int64_t width = int64_t(h->width ? h->width : 1);
    rc_status s = stackless_walk() ? ensure_ropes(h) : RC_OK;
    if (s != RC_OK)
        return s;
    s = begin_launch(h);
    if (s != RC_OK)
        return s;
    int kernels = 0;
    DevScene sc = dev_scene(h);
    if (watch)
    {
        sc.monitor = watch->dev;
        sc.budgetNs = watch->budgetNs;
    }
    RC_CUDA_TRY(h,
                launch_raycast(launch_info(h), sc, cam, dRays, pixelStart, int64_t(count), width, order, castShadow,
                               L, h->general.ray_start_offset, dOut, dQueue, h->dCtl, h->evMid, dOrigins, &kernels),
                "launch ray-cast kernels");
    return end_launch(h, "ray cast", kernels == 2, watch);
}

rc_status render_raycast(rc_tracer* h, uint64_t pixelStart, uint64_t count, const rc_ray* dRays, RenderWatch* watch)
{
    return raycast_into(h, dRays, pixelStart, count, h->order, h->dCast, h->dQueue, nullptr, watch);
}

}  // namespace rcx
