// Cancel, time budget and progress of a render, on the device side.
//
// The reference's Tracer::run checks `interrupted` per pixel and advances
// TracerState::pixelsProcessed every 100 pixels (Tracer.cpp:76-112), while
// the main thread polls it every 100 ms (ConsoleRunner.cpp:126-142). Here the
// persistent kernels take their work in items of 32 rays or path slots from
// an atomic queue head; a monitored render (rc_render with a cancel flag, a
// progress counter or a time budget) makes lane 0 of the warp that took
// every 256th item:
//   * read the host-mapped cancel word and check the time budget (measured
//     from the render's first check, %globaltimer);
//   * publish the pixels finished so far in the host-mapped monitor (PATH
//     renders: the pixels whose samples the film has taken; one-kernel RAY
//     frames: a lower bound from the queue head; the call's exact count is
//     read from the kernels' statistics at the end).
// A warp that sees a stop records the reason in DevControl::error and pushes
// the queue head past any item count, so every warp's next fetch ends its
// loop: the items already taken finish, nothing else starts. Kernels that
// follow in the same render find the stop bit at their start and return.
// Nothing waits here, so a stop can never hang a kernel.
#pragma once

#include "kernels.h"

namespace rcx
{

constexpr unsigned kPollItemsLog2 = 8;             // check every 256th work item
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

// Lane 0 of the warp that took a work item of the queue whose head is
// `head`. mayStop = false only publishes. Returns the stop reason
// (kErrCancelled / kErrBudget) or 0.
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

// Whole warp, after its fetch of `base` (a multiple of 32) from `head`:
// true when the warp must stop taking work. `publish` as poll_render's, or
// for a one-kernel RAY frame kPublishEstimate: the pixels of the items
// before the ones in flight (every warp of the grid holds at most one item,
// so when item k is taken at least k - warps items are finished), at most
// `pixels`.
constexpr unsigned long long kPublishEstimate = ~0ull - 2ull;

__device__ __forceinline__ bool warp_poll(RenderMonitor* mon, unsigned long long budgetNs, DevControl* ctl,
                                          unsigned* head, unsigned base, bool mayStop, unsigned long long publish,
                                          unsigned long long pixels = 0)
{
    if (!monitored(mon, budgetNs) || ((base >> 5) & ((1u << kPollItemsLog2) - 1u)) != 0u)
        return false;
    int why = 0;
    if ((threadIdx.x & 31u) == 0u)
    {
        if (publish == kPublishEstimate)
        {
            const unsigned long long warps = static_cast<unsigned long long>(gridDim.x) * (blockDim.x >> 5);
            const unsigned long long item = base >> 5;
            publish = item > warps ? (item - warps) * 32ull : 0ull;
            publish = publish < pixels ? publish : pixels;
        }
        why = poll_render(mon, budgetNs, ctl, head, mayStop, publish);
    }
    return __shfl_sync(0xffffffffu, why, 0) != 0;
}

// warp_poll for a fetch of `n` entries (1..32) at `base` that need not be a
// multiple of 32: polls where the range starts a 256-item block or crosses
// into one.
__device__ __forceinline__ bool warp_poll_range(RenderMonitor* mon, unsigned long long budgetNs, DevControl* ctl,
                                                unsigned* head, unsigned base, unsigned n, bool mayStop,
                                                unsigned long long publish)
{
    constexpr unsigned kShift = kPollItemsLog2 + 5;
    if (!monitored(mon, budgetNs) ||
        ((base & ((1u << kShift) - 1u)) != 0u && (base >> kShift) == ((base + n - 1u) >> kShift)))
        return false;
    int why = 0;
    if ((threadIdx.x & 31u) == 0u)
        why = poll_render(mon, budgetNs, ctl, head, mayStop, publish);
    return __shfl_sync(0xffffffffu, why, 0) != 0;
}

}  // namespace rcx
