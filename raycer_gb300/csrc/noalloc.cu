// rc_cast_with_shadow_device_noalloc: the primary + shadow ray query of
// rc_cast_with_shadow on caller device buffers, with no device allocation.
//
// Some callers cannot allocate device memory at the moment they trace: a
// host application whose GPU memory is owned by its own pool allocator (a
// render engine, a training framework) has no budget for a cudaMalloc behind
// its back, and a per-frame callback cannot afford cudaMalloc's implicit
// device synchronisation. This entry point keeps the only memory it needs
// besides the caller's inputs and outputs — the control block (work
// counters, statistics, error flag) and the shadow-ray queue — in the
// file-scope array below, which exists once per GPU in every process that
// loads the library and lives until the process exits.

#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "host_internal.h"
#include "kernels.h"

namespace
{

// At most this many rays per call (the queue holds a (pixel, triangle) pair
// per ray): 1,048,576 rays, 8 MiB of queue + one 256-B control block.
constexpr int64_t kNoAllocMaxRays = int64_t(1) << 20;
constexpr size_t kControlBytes = 256;
constexpr size_t kScratchBytes = kControlBytes + size_t(kNoAllocMaxRays) * 2 * sizeof(int);

static_assert(sizeof(rcx::DevControl) <= kControlBytes, "control block does not fit its slot");

static __device__ __align__(256) unsigned char g_noallocScratch[kScratchBytes];

// Device address of g_noallocScratch per device. In host code the array's
// name is only a host-side stand-in, so the address is fetched with
// cudaGetSymbolAddress once per device, with that device current.
constexpr int kMaxDevices = 64;
std::mutex g_scratchMutex;
void* g_scratchAddress[kMaxDevices] = {};

cudaError_t scratch_address(int device, void** out)
{
    if (device < 0 || device >= kMaxDevices)
        return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_scratchMutex);
    if (!g_scratchAddress[device])
    {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noallocScratch);
        if (e != cudaSuccess)
            return e;
        g_scratchAddress[device] = p;
    }
    *out = g_scratchAddress[device];
    return cudaSuccess;
}

rc_status fail(rc_tracer* h, rc_status s, const std::string& msg)
{
    h->err = msg;
    return s;
}

}  // namespace

extern "C" rc_status rc_cast_with_shadow_device_noalloc(rc_tracer* h, const rc_ray* d_rays, int64_t n, int32_t order,
                                                        rc_cast_pixel* d_out)
{
    if (!h)
        return RC_INVALID_ARG;
    if (!h->sceneReady)
        return fail(h, RC_NOT_READY, "cast_with_shadow_device_noalloc: no scene uploaded");
    if (h->nInstances > 0)
        return fail(h, RC_UNSUPPORTED, "cast_with_shadow_device_noalloc: instanced scenes are traced by rc_cast "
                                       "and PATH renders only");
    if (n < 0 || (n > 0 && (!d_rays || !d_out)))
        return fail(h, RC_INVALID_ARG, "cast_with_shadow_device_noalloc: bad ray count or null buffer");
    if (n > kNoAllocMaxRays)
        return fail(h, RC_INVALID_ARG,
                    "cast_with_shadow_device_noalloc: " + std::to_string(n) + " rays exceed the static scratch "
                    "maximum of " + std::to_string(kNoAllocMaxRays) + " rays per call; split the batch");
    if ((reinterpret_cast<uintptr_t>(d_rays) | reinterpret_cast<uintptr_t>(d_out)) & 15u)
        return fail(h, RC_INVALID_ARG, "cast_with_shadow_device_noalloc: buffers must be 16-byte aligned");
    if (order != RC_ORDER_REFERENCE && order != RC_ORDER_NEAREST)
        return fail(h, RC_INVALID_ARG, "cast_with_shadow_device_noalloc: invalid traversal order");
    if (n == 0)
        return RC_OK;  // an empty batch, as in rc_cast

    cudaError_t e = cudaSetDevice(h->device);
    void* scratch = nullptr;
    if (e == cudaSuccess)
        e = scratch_address(h->device, &scratch);
    if (e != cudaSuccess)
        return fail(h, RC_CUDA, std::string("cast_with_shadow_device_noalloc: scratch set-up: ") +
                                    cudaGetErrorString(e));
    auto* ctl = static_cast<rcx::DevControl*>(scratch);
    int* queue = reinterpret_cast<int*>(static_cast<unsigned char*>(scratch) + kControlBytes);

    float3 L = make_float3(0.0f, 0.0f, 0.0f);
    int castShadow = h->lights.empty() ? 0 : 1;
    if (castShadow)
        L = make_float3(-h->lights[0].direction[0], -h->lights[0].direction[1], -h->lights[0].direction[2]);

    rcx::DevScene sc{};
    sc.nodes = h->dNodes;
    sc.tris = h->dTris;
    sc.shade = h->dShade;
    sc.mats = h->dMats;
    sc.rootLink = h->rootLink;
    sc.numTris = int(h->nTris);
    sc.numMats = int(h->nMats);
    sc.pad = 0;
    sc.ropes = h->dRopes;  // built by an earlier call, if any (nothing is allocated here)
    sc.ropeCount = int(h->ropeCount);
    rcx::DevCamera cam{};
    rcx::LaunchInfo li;
    li.stream = h->stream;
    li.numSMs = h->numSMs;
    li.counting = h->counting;  // counted frames: the two-kernel form, same scratch

    // The array keeps the previous call's contents: the counters must start at zero.
    e = cudaMemsetAsync(ctl, 0, sizeof(rcx::DevControl), h->stream);
    if (e == cudaSuccess)
        e = rcx::launch_raycast(li, sc, cam, d_rays, 0, n, 1, order, castShadow, L, h->general.ray_start_offset,
                                d_out, queue, ctl, nullptr);
    rcx::DevControl result;
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(&result, ctl, sizeof(result), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess)
        return fail(h, RC_CUDA, std::string("cast_with_shadow_device_noalloc: ") + cudaGetErrorString(e));
    // This call's statistics only, as rc_cast_with_shadow keeps them (the
    // scene's build time stays); no events are recorded, so the times are 0.
    const double buildMs = h->stats.build_ms;
    h->stats = rc_stats{};
    h->stats.build_ms = buildMs;
    for (int k = 0; k < 2; ++k)
    {
        h->stats.stage_rays[k] = result.stats[3 * k + 0];
        h->stats.stage_nodes[k] = result.stats[3 * k + 1];
        h->stats.stage_tris[k] = result.stats[3 * k + 2];
    }
    h->stats.rays_traced = result.stats[0] + result.stats[3];
    h->stats.node_visits = result.stats[1] + result.stats[4];
    h->stats.tri_tests = result.stats[2] + result.stats[5];
    if (result.error & rcx::kErrStack)
        return fail(h, RC_DEVICE_ERROR, "cast_with_shadow_device_noalloc: traversal stack overflow");
    return RC_OK;
}
