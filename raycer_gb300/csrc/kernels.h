// Host-callable launchers of the device kernels (defined in the .cu files).
// All launches go to the given stream; none synchronises.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>

#include "../../include/raycer_gb300.h"
#include "device_types.h"

namespace rcx
{

// Small device-side control block shared by the kernels of one handle.
struct DevControl
{
    unsigned int head[8];          // work-queue heads / queue counts
    unsigned long long stats[8];   // per stage s: [3s] rays, [3s+1] node fetches, [3s+2] triangle tests
    int error;                     // bit0: traversal stack overflow; bit1: radiance-cache wait ran out;
                                   // bit2: cancelled; bit3: time budget ran out (kErr* below)
    int pad[3];
    unsigned long long t0;         // %globaltimer at the render's first work-queue check (time budget)
    unsigned long long progress;   // PATH renders: pixels whose samples the film has taken (monitored renders)
};

constexpr int kErrStack = 1;
constexpr int kErrCancelled = 4;
constexpr int kErrBudget = 8;
constexpr int kErrStop = kErrCancelled | kErrBudget;

struct LaunchInfo
{
    cudaStream_t stream;
    int numSMs;
    int counting;  // count node / triangle tests
};

// Resident blocks per SM of a persistent kernel, cached per device (the
// query belongs to the current device's context); launchers multiply it by
// the launching handle's SM count on every launch. Safe to call from
// several host threads.
constexpr int kMaxOccupancyDevices = 64;
struct OccupancyCache
{
    std::atomic<int> perSM[kMaxOccupancyDevices];
};

// One-time per-device set-up (a kernel's function attributes belong to the
// current device's context): runs `f` until it succeeds once on each device.
struct DeviceOnce
{
    std::atomic<int> done[kMaxOccupancyDevices];
};

template <typename F>
cudaError_t once_per_device(DeviceOnce& once, F&& f)
{
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxOccupancyDevices)
        return f();
    if (once.done[dev].load(std::memory_order_acquire))
        return cudaSuccess;
    const cudaError_t e = f();
    if (e == cudaSuccess)
        once.done[dev].store(1, std::memory_order_release);
    return e;
}

template <typename K>
int blocks_per_sm(K kernel, int block, size_t smem, OccupancyCache& cache)
{
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxOccupancyDevices)
        dev = -1;
    if (dev >= 0)
    {
        const int v = cache.perSM[dev].load(std::memory_order_relaxed);
        if (v > 0)
            return v;
    }
    int perSM = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, kernel, block, smem) != cudaSuccess || perSM < 1)
    {
        cudaGetLastError();
        return 1;
    }
    if (dev >= 0)
        cache.perSM[dev].store(perSM, std::memory_order_relaxed);
    return perSM;
}

// Whether uncounted reference-order queries (RAY-frame shadow rays, rc_cast
// in RC_ORDER_REFERENCE) take the stackless walk (traverse_stackless) where
// the scene has rope records (DevScene::ropes; the host builds them on first
// use while this is on).
bool stackless_walk();

// Generic ray queries (rc_ray -> rc_hit).
cudaError_t launch_cast(const LaunchInfo& li, const DevScene& sc, const rc_ray* rays, int64_t n, int anyHit,
                        int order, rc_hit* hits, DevControl* ctl);

// Ray-cast frame: primary closest hit per pixel + shadow any-hit per hit.
// Primary rays come from the camera (rays == nullptr) or from `rays`
// (one per pixel, caller order). Writes out[0..count); shadowQueue needs
// 2 * `count` ints (pixel, hit slot). ctl->head[0], head[1], head[2] must be zero on entry.
// Uncounted frames with a light run as one kernel by default (each shadow
// ray traced where its primary hit was found; no queue); counted frames and
// RC_TRACE_FUSED=0 run the primary and the shadow kernel, with `between`
// recorded between them. *kernels (optional) receives the number of kernels
// launched (0 for an empty frame).
cudaError_t launch_raycast(const LaunchInfo& li, const DevScene& sc, const DevCamera& cam, const rc_ray* rays,
                           uint64_t pixelStart, int64_t count, int64_t width, int order, int castShadow,
                           float3 dirToLight, float rayStartOffset, rc_cast_pixel* out, int* shadowQueue,
                           DevControl* ctl, cudaEvent_t between, float4* shadowOrigins = nullptr,
                           int* kernels = nullptr);
// shadowOrigins (optional, device memory, one float4 per queue entry): in
// the two-kernel form the primary kernel stores each hit pixel's shadow-ray
// origin there (and, in a two-level scene, the hit's instance in w), so the
// shadow kernel reads neither the caller's rays nor the records again: for
// rays and records in host memory, that is the host-link traffic of a
// second pass.

}  // namespace rcx
