// Cancel, time budget and progress of a render, on the device side.
//
// The reference's Tracer::run checks `interrupted` per pixel and advances
// TracerState::pixelsProcessed every 100 pixels (Tracer.cpp:76-112), while
// the main thread polls it every 100 ms (ConsoleRunner.cpp:126-142). Here the
// persistent kernels take their work in items of 32 rays or path slots from
// an atomic queue head. In a monitored render (rc_render with a cancel flag,
// a progress counter or a time budget) one warp of each such kernel, the
// last of block 0, takes no work and watches instead (watch_queue): every
// ~2 us its lane 0
//   * reads the host-mapped cancel word and checks the time budget (measured
//     from the render's first check, %globaltimer);
//   * publishes the pixels finished so far in the host-mapped monitor (PATH
//     renders: the pixels whose samples the film has taken; one-kernel RAY
//     frames: a lower bound from the queue head; the call's exact count is
//     read from the kernels' statistics at the end).
// On a stop it records the reason in DevControl::error and pushes the queue
// head past any item count, so every warp's next fetch ends its loop: the
// items already taken finish, nothing else starts. Kernels that follow in
// the same render find the stop bit at their start and return. The working
// warps' loops carry no poll, and nothing waits on the host, so a stop can
// never hang a kernel.
#pragma once

#include "kernels.h"

namespace rcx
{

constexpr unsigned kHeadPastEnd = 0x7fffffffu;     // above any queue or item count

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ bool monitored(const RenderMonitor* mon, unsigned long long budgetNs)
{
    return mon != nullptr || budgetNs != kNoBudget;
}

// Stop bit of an earlier kernel (or warp) of the render.
__device__ __forceinline__ bool render_stopped(const DevControl* ctl)
{
    return (*reinterpret_cast<const volatile int*>(&ctl->error) & kErrStop) != 0;
}

// What a poll writes into the monitor's pixel count.
constexpr unsigned long long kPublishNone = ~0ull;            // nothing (two-kernel RAY frames)
constexpr unsigned long long kPublishProgress = ~0ull - 1ull;  // DevControl::progress (PATH renders)
constexpr unsigned long long kPublishEstimate = ~0ull - 2ull;  // a lower bound from the queue head (RAY frames)

// One poll by the watch warp's lane 0, for the queue whose head is `head`.
// mayStop = false only publishes. Returns the stop reason (kErrCancelled /
// kErrBudget) or 0.
static __device__ __noinline__ int poll_render(RenderMonitor* mon, unsigned long long budgetNs, DevControl* ctl,
                                               unsigned* head, bool mayStop, unsigned long long publish)
{
    int why = 0;
    if (mayStop && budgetNs != kNoBudget)
    {
        const unsigned long long now = global_ns();
        unsigned long long t0 = atomicCAS(&ctl->t0, 0ull, now);
        if (t0 == 0ull)
            t0 = now;
        if (now - t0 >= budgetNs)
            why = kErrBudget;
    }
    if (mon)
    {
        if (mayStop && mon->cancel)
            why = kErrCancelled;
        if (publish != kPublishNone)
        {
            // a plain store: stores of two warps may land in either order, so
            // the host keeps the largest value it has read
            mon->pixels = publish == kPublishProgress
                              ? *reinterpret_cast<const volatile unsigned long long*>(&ctl->progress)
                              : publish;
            __threadfence_system();
        }
    }
    if (why)
    {
        atomicOr(&ctl->error, why);
        atomicMax(head, kHeadPastEnd);
    }
    return why;
}

// The watch warp of a monitored persistent kernel (the last warp of block
// 0): it takes no work; its lane 0 polls the cancel word and the time budget
// and publishes progress, sleeping ~2 us between polls, until the queue head
// had reached `items` at a poll (every item taken), a stop, or kWatchPolls
// polls (then it just stops watching). The other warps' work loop carries no poll at all.
// publish: kPublishNone, kPublishProgress, or kPublishEstimate (the pixels of
// the items taken before those the other warps may hold, at most `pixels`).
constexpr unsigned kWatchPolls = 1u << 24;

static __device__ __forceinline__ void watch_queue(RenderMonitor* mon, unsigned long long budgetNs, DevControl* ctl,
                                         unsigned* head, unsigned long long items, unsigned long long publish,
                                         unsigned long long pixels)
{
    if ((threadIdx.x & 31u) != 0u)
        return;
    const unsigned long long workers = static_cast<unsigned long long>(gridDim.x) * (blockDim.x >> 5) - 1ull;
    for (unsigned i = 0; i < kWatchPolls; ++i)
    {
        const unsigned long long h = *reinterpret_cast<const volatile unsigned*>(head);
        unsigned long long pub = publish;
        if (publish == kPublishEstimate)
        {
            const unsigned long long item = h >> 5;
            pub = item > workers ? (item - workers) * 32ull : 0ull;
            pub = pub < pixels ? pub : pixels;
        }
        // polled once before the head is looked at: a kernel whose items
        // were all taken at once is still checked (a budget of 0 stops it)
        if (poll_render(mon, budgetNs, ctl, head, true, pub) || h >= items)
            return;
        __nanosleep(2000);
    }
}

// Whether this warp is the watch warp of a monitored kernel.
__device__ __forceinline__ bool is_watch_warp(const RenderMonitor* mon, unsigned long long budgetNs)
{
    return monitored(mon, budgetNs) && blockIdx.x == 0 && (threadIdx.x >> 5) == (blockDim.x >> 5) - 1u;
}

}  // namespace rcx
